"""CPU restatement of the PirServer file image (test infrastructure).

Follows PirServer::SaveToFile and PirServer::LoadFromBuffer
(crypto/pir/server/pir_server.cc:434-588 and 590-780) and their bit packers
BitPackSigned / BitUnpackSigned / BitPackCoefficients /
BitUnpackCoefficients (pir_server.cc:310-431): little-endian fields; the DB
matrix as its raw (or condensed u64) words; the pack matrix as signed
entries of pack_log_digit + bit_width(d - 1) bits; a_tilde_agg, t_vec_h and
second_dim_a as log_modulus-bit coefficients (raw words when log_modulus is
the coefficient width). Bits are packed least-significant first.

Only tests use this module: it writes images that the GPU loader must read
and reads images that the GPU saver writes.
"""
import struct

import numpy as np


def _bits_of(values, num_bits):
    v = np.asarray(values, dtype=np.uint64)
    shifts = np.arange(num_bits, dtype=np.uint64)
    return ((v[:, None] >> shifts[None, :]) & np.uint64(1)).astype(np.uint8)


def bitpack(values, num_bits):
    """BitPackSigned / BitPackCoefficients below the word width."""
    if len(values) == 0 or num_bits <= 0:
        return b""
    mask = np.uint64((1 << num_bits) - 1) if num_bits < 64 else np.uint64((1 << 64) - 1)
    v = np.asarray(values).astype(np.int64).view(np.uint64) & mask
    return np.packbits(_bits_of(v, num_bits).reshape(-1),
                       bitorder="little").tobytes()


def bitunpack(data, n, num_bits, signed):
    if n == 0 or num_bits <= 0:
        return np.zeros(n, dtype=np.int64 if signed else np.uint64)
    bits = np.unpackbits(np.frombuffer(data, dtype=np.uint8),
                         bitorder="little")[:n * num_bits].reshape(n, num_bits)
    weights = (np.uint64(1) << np.arange(num_bits, dtype=np.uint64))
    v = (bits.astype(np.uint64) * weights[None, :]).sum(axis=1,
                                                        dtype=np.uint64)
    if signed and num_bits < 64:
        neg = (v >> np.uint64(num_bits - 1)) & np.uint64(1)
        v = v | (neg * np.uint64(~((1 << num_bits) - 1) & ((1 << 64) - 1)))
        return v.view(np.int64)
    return v


def _coeffs(poly, log_modulus, coeff_bits):
    poly = np.asarray(poly)
    if log_modulus >= coeff_bits:
        return poly.astype({32: np.uint32, 64: np.uint64}[coeff_bits]).tobytes()
    return bitpack(poly.astype(np.uint64), log_modulus)


def save_image(d, coeff_bits, log_modulus, pack_log_digit, db, pack, a_tilde,
               t_vec_h, second_dim_a, t, l, db_orig_cols=None,
               db_condensed=False, pack_condensed=False):
    """Bytes of PirServer::SaveToFile for combined material."""
    out = bytearray()
    rows, cols = db.shape
    es = db.dtype.itemsize
    phys = cols * es // 8 if db_condensed else cols
    orig = cols if db_orig_cols is None else db_orig_cols
    out += struct.pack("<iiBi", rows, phys, 1 if db_condensed else 0, orig)
    if db_condensed:
        words = np.ascontiguousarray(db).view(np.uint64)
        out += struct.pack("<Q", words.size) + words.tobytes()
    else:
        out += struct.pack("<Q", db.size) + np.ascontiguousarray(db).tobytes()
    prow, pcol = pack.shape
    pes = pack.dtype.itemsize
    pphys = pcol * pes // 8 if pack_condensed else pcol
    bits = pack_log_digit + int(d - 1).bit_length()
    out += struct.pack("<iiiBii", prow, pcol, pphys, 1 if pack_condensed else 0,
                       pcol, bits)
    packed = bitpack(pack.reshape(-1), bits)
    out += struct.pack("<Q", len(packed)) + packed
    out += struct.pack("<i", log_modulus)
    k = t_vec_h.shape[0] // (l * t)
    out += struct.pack("<i", l)
    for s in range(l):
        out += struct.pack("<i", t)
        for i in range(t):
            a = a_tilde[s * t + i]
            pa = _coeffs(a, log_modulus, coeff_bits)
            out += struct.pack("<QQ", d, len(pa)) + pa
            out += struct.pack("<Q", k)
            for j in range(k):
                pt = _coeffs(t_vec_h[(s * t + i) * k + j], log_modulus, coeff_bits)
                out += struct.pack("<QQ", d, len(pt)) + pt
    out += struct.pack("<Q", second_dim_a.shape[0])
    for poly in second_dim_a:
        pp = _coeffs(poly, log_modulus, coeff_bits)
        out += struct.pack("<QQ", d, len(pp)) + pp
    return bytes(out)


class _Reader:
    def __init__(self, buf):
        self.buf, self.off = buf, 0

    def take(self, fmt):
        v = struct.unpack_from(fmt, self.buf, self.off)
        self.off += struct.calcsize(fmt)
        return v

    def raw(self, n):
        b = self.buf[self.off:self.off + n]
        self.off += n
        return b


def load_image(buf, db_dtype, mat_dtype, coeff_bits):
    """PirServer::LoadFromBuffer: the combined material of an image."""
    r = _Reader(buf)
    rows, phys, condensed, orig = r.take("<iiBi")
    (n,) = r.take("<Q")
    if condensed:
        words = np.frombuffer(r.raw(8 * n), dtype=np.uint64)
        db = words.view(db_dtype).reshape(rows, -1)
    else:
        db = np.frombuffer(r.raw(np.dtype(db_dtype).itemsize * n),
                           dtype=db_dtype).reshape(rows, -1)
    prow, pcol, pphys, pcond, porig, bits = r.take("<iiiBii")
    (plen,) = r.take("<Q")
    pack = bitunpack(r.raw(plen), prow * pcol, bits, True).astype(
        mat_dtype).reshape(prow, pcol)
    (log_q,) = r.take("<i")
    cdt = {32: np.uint32, 64: np.uint64}[coeff_bits]

    def poly():
        length, plen = r.take("<QQ")
        data = r.raw(plen)
        if log_q >= coeff_bits:
            return np.frombuffer(data, dtype=cdt)[:length].copy()
        return bitunpack(data, length, log_q, False).astype(cdt)
    (shards,) = r.take("<i")
    a_tilde, t_vec_h = [], []
    for _ in range(shards):
        (slices,) = r.take("<i")
        for _ in range(slices):
            a_tilde.append(poly())
            (k,) = r.take("<Q")
            t_vec_h.extend(poly() for _ in range(k))
    (nsd,) = r.take("<Q")
    sda = [poly() for _ in range(nsd)]
    d = len(a_tilde[0]) if a_tilde else 0
    return {"db": db, "db_orig_cols": orig, "db_condensed": bool(condensed),
            "pack": pack, "pack_condensed": bool(pcond), "pack_bits": bits,
            "log_modulus": log_q, "a_tilde_agg": np.array(a_tilde, dtype=cdt),
            "t_vec_h": np.array(t_vec_h, dtype=cdt),
            "second_dim_a": np.array(sda, dtype=cdt).reshape(-1, d)}
