"""The algorithmic work counts behind the bench line's roofline.

The limb GEMM's limb-ops count the base-256 digit products the exact plan
computes: a DB entry has two digits, a pack entry four, a request word four
(Z_2^32) or eight (Z_2^64), and a digit pair (i, j) is computed only when
its weight 2^(8 (i + j)) is below the bits the answer reads (2^32, 2^64, or
2^56 for a Z_2^64 server with q <= 2^56). The GEMV's bytes are both
matrices, the request words and the output words.
"""
import pytest

from inspire_gb300 import profiling


def pairs(matrix_digits, request_digits, width_bits):
    return sum(1 for i in range(matrix_digits) for j in range(request_digits)
               if 8 * (i + j) < width_bits)


@pytest.mark.parametrize("coeff_bits,log_q,db_pairs,pack_pairs", [
    (32, None, 7, 10), (64, None, 15, 26), (64, 64, 15, 26), (64, 56, 13, 22),
    (64, 52, 13, 22)])
def test_limb_ops_count_the_digit_pairs_below_the_answer_width(coeff_bits, log_q,
                                                               db_pairs, pack_pairs):
    request_digits = coeff_bits // 8
    width = coeff_bits if log_q is None or log_q > 56 or coeff_bits == 32 else 56
    assert pairs(2, request_digits, width) == db_pairs
    assert pairs(4, request_digits, width) == pack_pairs
    r, c, k, b = 3, 5, 7, 11
    assert profiling.limb_ops(r, c, k, b, coeff_bits, log_q) == \
        2 * (db_pairs * r * c + pack_pairs * r * k) * b


def test_headline_counts():
    # n = 2^20, d = 4096, t = 8: R = 32768, C = 131072, K = 8192, B = 256.
    R, C, K, B = 32768, 131072, 8192, 256
    assert profiling.limb_ops(R, C, K, B) == 16_767_552_323_584
    assert profiling.limb_ops(R, C, K, B, 64, 56) == pytest.approx(3.161e13, rel=1e-3)
    assert profiling.limb_ops(R, C, K, B, 64, 64) == pytest.approx(3.656e13, rel=1e-3)
    # The plain single-request GEMV: u16 DB, i32 pack, u32 words.
    assert profiling.plain_bytes(R, C, K) == 9_664_364_544
    # C1: n = 4096, d = 2048, t = 2 over Z_2^64 (u64 words).
    assert profiling.plain_bytes(4096, 2048, 4096, word=8) == 83_968_000
