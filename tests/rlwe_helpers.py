"""RLWE key generation, encryption and decryption for tests (numpy).

Restates, with this repository's own seeded generator in place of
shell-encryption's ChaCha PRNG and samplers (not in this image), the pieces
the reference's packing tests build their inputs from:
  SampleSecretKey / EncryptRlwe / Decrypt (crypto/encryption.cc:99-330),
  LwestoRlweTest::EncryptKeySwitchingKey and ::ExtractLwes
  (crypto/lwes_to_rlwe_test.cc:69-134).
Only the algebra matters to the properties checked (a packed ciphertext
decrypts to the packed messages), not the sampler bytes.
"""
import numpy as np


def dtype_of(bits):
    return np.uint32 if bits == 32 else np.uint64


def wmask(bits):
    return np.uint64((1 << bits) - 1) if bits < 64 else np.uint64(~0 & ((1 << 64) - 1))


def qmask(log_q, bits):
    return (1 << log_q) - 1 if log_q < bits else (1 << bits) - 1


def negacyclic(u, v, bits):
    """u * v in Z_{2^bits}[X]/(X^d + 1) (schoolbook, numpy wrap-around)."""
    u = np.asarray(u).astype(np.uint64)
    v = np.asarray(v).astype(np.uint64)
    d = u.shape[0]
    acc = np.zeros(d, dtype=np.uint64)
    with np.errstate(over="ignore"):
        for a in np.nonzero(u)[0]:
            x = u[a]
            acc[a:] += x * v[:d - a]
            acc[:a] -= x * v[d - a:]
    return (acc & wmask(bits)).astype(dtype_of(bits))


def automorph(p, power, bits):
    """Polynomial::Automorph (crypto/polynomial.cc:429-456)."""
    p = np.asarray(p).astype(np.uint64)
    d = p.shape[0]
    out = np.zeros(d, dtype=np.uint64)
    idx = (np.arange(d, dtype=np.int64) * power) % (2 * d)
    with np.errstate(over="ignore"):
        pos = idx < d
        out[idx[pos]] += p[pos]
        out[idx[~pos] - d] -= p[~pos]
    return (out & wmask(bits)).astype(dtype_of(bits))


class Rlwe:
    """One key and the key-switching keys of the packing (X -> X^5 and
    X -> X^{2d-1})."""

    def __init__(self, d, bits, log_q, log_digit, num_digits, seed,
                 ksk_noise=2):
        self.d, self.bits, self.log_q = d, bits, log_q
        self.ksk_noise = ksk_noise
        self.log_digit, self.num_digits = log_digit, num_digits
        self.rng = np.random.default_rng(seed)
        self.dt = dtype_of(bits)
        self.mask = qmask(log_q, bits)
        s = self.rng.integers(-1, 2, d)
        self.s = (s.astype(np.int64).astype(np.uint64) & wmask(bits)).astype(self.dt)
        self.w_g, self.y_g = self.key_switching_key(automorph(self.s, 5, bits))
        self.w_h, self.y_h = self.key_switching_key(
            automorph(self.s, 2 * d - 1, bits))

    def uniform(self, *shape):
        x = self.rng.integers(0, self.mask, size=shape, dtype=np.uint64,
                              endpoint=True)
        return x.astype(self.dt)

    def small(self, bound):
        e = self.rng.integers(-bound, bound + 1, self.d).astype(np.int64)
        return (e.astype(np.uint64) & np.uint64(self.mask)).astype(self.dt)

    def key_switching_key(self, s_target):
        """LwestoRlweTest::EncryptKeySwitchingKey: y_i = -w_i s + e +
        s_target * 2^(i*log_digit + offset)."""
        k, d = self.num_digits, self.d
        offset = max(0, self.log_q - k * self.log_digit)
        w = self.uniform(k, d)
        y = np.zeros((k, d), dtype=self.dt)
        with np.errstate(over="ignore"):
            for i in range(k):
                ws = negacyclic(w[i], self.s, self.bits).astype(np.uint64)
                tgt = (s_target.astype(np.uint64)
                       << np.uint64(i * self.log_digit + offset)) & wmask(self.bits)
                e = self.small(self.ksk_noise).astype(np.uint64)
                y[i] = ((np.uint64(0) - ws + e + tgt) & wmask(self.bits)).astype(self.dt)
        return w, y

    def encrypt(self, m, t):
        """EncryptRlwe: b = e - a s + round(m q / t) mod q."""
        a = self.uniform(self.d)
        e = np.rint(self.rng.normal(0.0, np.sqrt(8.0), self.d)).astype(np.int64)
        q = 1 << self.log_q
        scaled = np.array([(int(x) * q + t // 2) // t for x in m], dtype=object)
        with np.errstate(over="ignore"):
            as_ = negacyclic(a, self.s, self.bits).astype(np.uint64)
            b = (e.astype(np.uint64) - as_
                 + np.array([int(x) & ((1 << 64) - 1) for x in scaled],
                            dtype=np.uint64)) & np.uint64(self.mask)
        return a, b.astype(self.dt)

    def extract_lwes(self, a, b):
        """LwestoRlweTest::ExtractLwes: a_k[j] = a[k-j] (j <= k), -a[d+k-j]."""
        d = self.d
        k = np.arange(d)[:, None]
        j = np.arange(d)[None, :]
        src = np.where(j <= k, k - j, d + k - j)
        a64 = a.astype(np.uint64)[src]
        with np.errstate(over="ignore"):
            a_is = np.where(j <= k, a64, np.uint64(0) - a64) & wmask(self.bits)
        return a_is.astype(self.dt), b.copy()

    def decrypt(self, a, b, t):
        """Decrypt: round((b + a s mod q) * t / q) mod t."""
        with np.errstate(over="ignore"):
            noisy = (b.astype(np.uint64)
                     + negacyclic(a, self.s, self.bits).astype(np.uint64)) \
                & np.uint64(self.mask)
        q = 1 << self.log_q
        return np.array([((int(v) * t + q // 2) // q) % t for v in noisy])
