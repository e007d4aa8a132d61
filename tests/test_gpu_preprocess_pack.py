"""GPU PreprocessMatrixPack against the oracle, and the packing property at
full ring degree.

* Parity: a_tilde_agg, t_vec_h and the matrix (every element type the
  reference instantiates, crypto/lwes_to_rlwe.cc:533-575) equal the oracle's
  exact restatement for several slices at once, d = 64 and 256, and for one
  slice at d = 2048 (the radix-16 reduction chains).
* d = 2048 / 4096 (the C2 / C3 ring degrees): LWE ciphertexts extracted
  from one RLWE encryption, the GPU's matrix and t_vec_h, then
  FinalizeMatrixPack(b + P y_g) decrypts to the messages
  (PackWithMatrixEndToEndWorks, crypto/lwes_to_rlwe_test.cc:364-467, at the
  sizes the oracle cannot run). With q = 2^32 and the 19 x 2 pack gadget the
  key-switching noise of d packed ciphertexts (about 2^30) exceeds any
  message scale, so that case uses noiseless key-switching keys (the algebra
  is still exact end to end); a 8 x 4 gadget runs with noisy keys.
"""
import numpy as np
import pytest

from inspire_gb300 import pir
from oracle import pyoracle as orc
from tests.rlwe_helpers import Rlwe, dtype_of, qmask

pytestmark = pytest.mark.gpu


def _random_case(d, bits, log_q, k, slices, seed, extra_cols=5):
    rng = np.random.default_rng(seed)
    mask = qmask(log_q, bits)
    dt = dtype_of(bits)
    hint = rng.integers(0, mask, (slices * d, d + extra_cols), dtype=np.uint64,
                        endpoint=True).astype(dt)
    pack_a = rng.integers(0, mask, (2 * k, d), dtype=np.uint64,
                          endpoint=True).astype(dt)
    return hint, pack_a


@pytest.mark.parametrize("d,bits,log_q,log_digit,k", [
    (64, 32, 27, 4, 5), (64, 32, 32, 4, 6), (64, 64, 45, 4, 10),
    (64, 64, 64, 4, 14), (256, 32, 32, 19, 2), (256, 64, 52, 19, 2),
    (256, 32, 29, 8, 3)])
def test_matches_oracle(d, bits, log_q, log_digit, k):
    slices = 3
    hint, pack_a = _random_case(d, bits, log_q, k, slices, 7 * d + log_q)
    a_gpu, m_gpu, th_gpu = pir.PreprocessMatrixPack(hint, pack_a, log_q,
                                                    log_digit, k)
    for s in range(slices):
        ref = orc.preprocess_matrix_pack(hint[s * d:(s + 1) * d, :d],
                                         pack_a[:k], pack_a[k:], bits, log_q,
                                         log_digit, k)
        assert np.array_equal(a_gpu[s], ref["a_tilde_agg"]), s
        assert np.array_equal(th_gpu[s], ref["t_vec_h"]), s
        want = ref["matrix"].astype(dtype_of(bits))
        assert np.array_equal(m_gpu[s * d:(s + 1) * d], want), s


@pytest.mark.parametrize("bits,log_q", [(32, 32), (64, 52)])
def test_radix16_chains_match_oracle_at_d2048(bits, log_q):
    # d = 2048: the reduction chains run on the radix-16 register
    # transforms, one thread group per prime (the oracle's chain is O(d^3)
    # and takes seconds here; 4096 is left to the decryption tests below).
    d, k, log_digit = 2048, 2, 19
    hint, pack_a = _random_case(d, bits, log_q, k, 1, 2048 + log_q)
    a_gpu, m_gpu, th_gpu = pir.PreprocessMatrixPack(hint, pack_a, log_q,
                                                    log_digit, k)
    ref = orc.preprocess_matrix_pack(hint[:, :d], pack_a[:k], pack_a[k:], bits,
                                     log_q, log_digit, k)
    assert np.array_equal(a_gpu[0], ref["a_tilde_agg"])
    assert np.array_equal(th_gpu[0], ref["t_vec_h"])
    assert np.array_equal(m_gpu, ref["matrix"].astype(dtype_of(bits)))


@pytest.mark.parametrize("mat", [np.int16, np.int32])
def test_narrow_matrix_types(mat):
    d, bits, log_q, k = 64, 32, 27, 5
    hint, pack_a = _random_case(d, bits, log_q, k, 2, 99)
    _, wide, _ = pir.PreprocessMatrixPack(hint, pack_a, log_q, 4, k)
    _, narrow, _ = pir.PreprocessMatrixPack(hint, pack_a, log_q, 4, k,
                                            mat_dtype=mat)
    assert np.array_equal(narrow, wide.astype(mat))


@pytest.mark.parametrize("d,bits,log_q,log_digit,k,noise", [
    (2048, 32, 32, 19, 2, 0), (4096, 32, 32, 19, 2, 0), (4096, 32, 32, 8, 4, 2),
    (2048, 64, 52, 19, 2, 2), (4096, 64, 52, 19, 2, 2), (8192, 32, 32, 19, 2, 0)])
def test_packed_ciphertext_decrypts_at_full_degree(d, bits, log_q, log_digit,
                                                   k, noise):
    t = 16
    r = Rlwe(d, bits, log_q, log_digit, k, seed=d + log_q + log_digit,
             ksk_noise=noise)
    m = r.rng.integers(0, t, d)
    a, b = r.encrypt(m, t)
    a_is, b_is = r.extract_lwes(a, b)
    pack_a = np.concatenate([r.w_g, r.w_h])
    a_tilde, mat, t_vec_h = pir.PreprocessMatrixPack(a_is, pack_a, log_q,
                                                     log_digit, k)
    # b_agg_partial = P . y_g mod 2^w (matrix entries sign-extended).
    p64 = mat.astype(np.int64).view(np.uint64) if mat.dtype != np.uint64 else mat
    with np.errstate(over="ignore"):
        partial = (p64 @ r.y_g.reshape(-1).astype(np.uint64))
    partial = partial.astype(dtype_of(bits))
    prm = orc.make_params(
        coeff_bits=bits, log_degree=int(np.log2(d)), log_modulus=log_q,
        log_modulus1_after_switch=log_q, log_modulus2_after_switch=log_q,
        pack_log_digit=log_digit, pack_num_digits=k, eval_log_digit=log_digit,
        eval_num_digits=k, num_entries=d, interpolation_degree=1,
        entry_size_multiple=1)
    b_agg = orc.finalize_matrix_pack(prm, b_is, partial, r.y_h, t_vec_h[0])
    assert list(r.decrypt(a_tilde[0], b_agg, t)) == list(m)


def test_rejects_bad_arguments():
    hint = np.zeros((64, 64), np.uint32)
    pack_a = np.zeros((4, 64), np.uint32)
    with pytest.raises(pir.InspireError, match="log_digit and num_digits"):
        pir.PreprocessMatrixPack(hint, pack_a, 32, 0, 2)
    with pytest.raises(pir.InspireError, match="size mismatch"):
        pir.PreprocessMatrixPack(hint, pack_a[:3], 32, 4, 2, slices=1)
