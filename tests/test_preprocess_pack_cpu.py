"""The oracle's PreprocessMatrixPack / Pack restatement, pinned by the
reference's own packing tests (crypto/lwes_to_rlwe_test.cc:149-520):

* PackEndToEndWorks / ...WithApproximateGadgetDecompWorks (149-256, 258-362):
  LWE ciphertexts extracted from one RLWE encryption, PreprocessPack, Pack,
  and the packed RLWE ciphertext decrypts to the messages;
* PackWithMatrixEndToEndWorks (364-467): the matrix route
  FinalizeMatrixPack(b + P y_g) equals the automorphism route, and decrypts;
* PreprocessMatrixNormBounded (470-520): entries below 4 sqrt(d) 2^log_digit.

d = 64, log_digit = 4 and the reference's log_q sets. Keys and ciphertexts
come from the numpy restatement in rlwe_helpers (own seeded generator).
"""
import numpy as np
import pytest

from oracle import pyoracle as orc
from tests.rlwe_helpers import Rlwe, dtype_of, qmask

D = 64
T = 8
LOG_QS = [(32, 27), (32, 29), (32, 32), (64, 45), (64, 54), (64, 64)]


def _setup(bits, log_q, num_digits, seed):
    r = Rlwe(D, bits, log_q, 4, num_digits, seed)
    m = r.rng.integers(0, T, D)
    a, b = r.encrypt(m, T)
    a_is, b_is = r.extract_lwes(a, b)
    return r, m, a_is, b_is


@pytest.mark.parametrize("bits,log_q", LOG_QS)
@pytest.mark.parametrize("approx", [False, True])
def test_pack_end_to_end_decrypts(bits, log_q, approx):
    k = 4 if approx else (log_q + 3) // 4
    r, m, a_is, b_is = _setup(bits, log_q, k, 100 + log_q + approx)
    pre = orc.preprocess_matrix_pack(a_is, r.w_g, r.w_h, bits, log_q, 4, k,
                                     with_matrix=False)
    b_agg = orc.pack(b_is, r.y_g, r.y_h, pre, bits, log_q, 4, k)
    assert list(r.decrypt(pre["a_tilde_agg"], b_agg, T)) == list(m)


def _narrow(matrix, kind):
    return matrix.astype(kind)


def _params(bits, log_q, k):
    return orc.make_params(
        coeff_bits=bits, log_degree=6, log_modulus=log_q,
        log_modulus1_after_switch=log_q, log_modulus2_after_switch=log_q,
        pack_log_digit=4, pack_num_digits=k, eval_log_digit=4,
        eval_num_digits=k, num_entries=D, interpolation_degree=1,
        entry_size_multiple=1)


@pytest.mark.parametrize("bits,log_q", LOG_QS)
def test_matrix_route_equals_automorphism_route(bits, log_q):
    k = (log_q + 3) // 4 - 2
    r, m, a_is, b_is = _setup(bits, log_q, k, 200 + log_q)
    pre = orc.preprocess_matrix_pack(a_is, r.w_g, r.w_h, bits, log_q, 4, k)
    b_direct = orc.pack(b_is, r.y_g, r.y_h, pre, bits, log_q, 4, k)
    mat = _narrow(pre["matrix"], dtype_of(bits))
    partial = orc.matrix_multiply(mat, r.y_g.reshape(-1), bits)
    prm = _params(bits, log_q, k)
    b_matrix = orc.finalize_matrix_pack(prm, b_is, partial, r.y_h,
                                        pre["t_vec_h"])
    assert np.array_equal(b_matrix, b_direct)
    assert list(r.decrypt(pre["a_tilde_agg"], b_matrix, T)) == list(m)


@pytest.mark.parametrize("bits,log_q", [(32, 27), (64, 45)])
@pytest.mark.parametrize("kind", [np.int16, np.int32])
def test_matrix_route_with_narrow_entries(bits, log_q, kind):
    # PackWithMatrixEndToEndWithDifferentMatCoeffTypeWorks (522-...): the
    # matrix narrowed to int16 / int32 still gives the same b_agg.
    k = (log_q + 3) // 4 - 2
    r, m, a_is, b_is = _setup(bits, log_q, k, 300 + log_q)
    pre = orc.preprocess_matrix_pack(a_is, r.w_g, r.w_h, bits, log_q, 4, k)
    b_direct = orc.pack(b_is, r.y_g, r.y_h, pre, bits, log_q, 4, k)
    partial = orc.matrix_multiply(_narrow(pre["matrix"], kind),
                                  r.y_g.reshape(-1), bits)
    prm = _params(bits, log_q, k)
    b_matrix = orc.finalize_matrix_pack(prm, b_is, partial, r.y_h,
                                        pre["t_vec_h"])
    assert np.array_equal(b_matrix, b_direct)


@pytest.mark.parametrize("bits,log_q", LOG_QS)
def test_matrix_entries_bounded(bits, log_q):
    # PreprocessMatrixNormBounded, on uniform a-vectors. The reference stores
    # an entry v >= 2^(log_q-1) as v - 2^log_q of the full-width word, so for
    # log_q below the word width a negative entry keeps a -2^log_q offset
    # (a multiple of 2^log_q: the product mod 2^log_q is unchanged); the
    # bound holds for the entries reduced to centred residues mod 2^log_q.
    k = (log_q + 3) // 4
    r = np.random.default_rng(400 + log_q)
    mask = qmask(log_q, bits)
    a_is = r.integers(0, mask, (D, D), dtype=np.uint64, endpoint=False)
    w = r.integers(0, mask, (2, k, D), dtype=np.uint64, endpoint=False)
    dt = dtype_of(bits)
    pre = orc.preprocess_matrix_pack(a_is.astype(dt), w[0].astype(dt),
                                     w[1].astype(dt), bits, log_q, 4, k)
    mat = pre["matrix"]
    if log_q == bits:   # stored as the two's complement of the word
        assert np.abs(mat).max() < 4 * np.sqrt(D) * 16
        return
    q = 1 << log_q
    centred = ((mat % q) + q // 2) % q - q // 2
    assert np.abs(centred).max() < 4 * np.sqrt(D) * 16
    if log_q < bits:
        off = mat - centred
        assert np.all((off == 0) | (off == -q))


def test_fp64_mode_matches_exact_at_reference_size():
    # The reference computes every inner product with its FP64 FFT; at
    # d = 64 and these digit widths the FFT is exact, so both modes agree.
    k = 5
    r, m, a_is, b_is = _setup(32, 29, k, 501)
    ex = orc.preprocess_matrix_pack(a_is, r.w_g, r.w_h, 32, 29, 4, k)
    fp = orc.preprocess_matrix_pack(a_is, r.w_g, r.w_h, 32, 29, 4, k,
                                    mode=orc.MODE_FP64)
    for key in ("a_tilde_agg", "t_vec_h", "t_vec_g", "t_vec_gh", "matrix"):
        assert np.array_equal(ex[key], fp[key]), key
