"""The reference's FP64 FFT against the exact product, in the oracle.

At d <= 2048 (and at every d for FinalizeMatrixPack's two-polynomial inner
product) the reference's FP64 path rounds to the exact integer, which is what
its own tests assert (crypto/polynomial_test.cc:399-608). Inside
ExternalProduct at d = 4096 its chunk bound log2(6) + 12 + 2*19 = 52.58 is too
close to 53 and a few percent of the output coefficients come out off by a
small multiple of 2^(19*j) (crypto/external_product.cc:100-102). The GPU path
computes the exact integer; this test records how far the FP64 path is from
it, so the difference is measured rather than hidden.
"""
import numpy as np
import pytest

from oracle import pyoracle as orc


def _params(cb, lq, logd, nd=3):
    return orc.make_params(
        coeff_bits=cb, log_degree=logd, log_modulus=lq,
        log_modulus1_after_switch=lq, log_modulus2_after_switch=lq,
        pack_log_digit=19, pack_num_digits=2, eval_log_digit=19,
        eval_num_digits=nd, num_entries=2 << logd, interpolation_degree=2,
        entry_size_multiple=1)


def _ext(cb, lq, logd, seed):
    d = 1 << logd
    rng = np.random.default_rng(seed)
    cdt = np.uint32 if cb == 32 else np.uint64
    hi = (1 << lq) - 1
    ct_a = rng.integers(0, hi, size=d, dtype=cdt, endpoint=True)
    ct_b = rng.integers(0, hi, size=d, dtype=cdt, endpoint=True)
    rgsw = rng.integers(0, hi, size=(12, d), dtype=cdt, endpoint=True)
    prm = _params(cb, lq, logd)
    exact = orc.external_product(prm, ct_a, ct_b, rgsw, orc.MODE_EXACT)
    fp64 = orc.external_product(prm, ct_a, ct_b, rgsw, orc.MODE_FP64)
    return exact, fp64


@pytest.mark.parametrize("cb,lq", [(32, 32), (64, 52)])
def test_external_product_fp64_is_exact_at_d2048(cb, lq):
    exact, fp64 = _ext(cb, lq, 11, seed=1)
    assert np.array_equal(exact[0], fp64[0])
    assert np.array_equal(exact[1], fp64[1])


@pytest.mark.parametrize("cb,lq", [(32, 32), (64, 52)])
def test_external_product_fp64_error_at_d4096_is_small_multiples(cb, lq):
    exact, fp64 = _ext(cb, lq, 12, seed=2)
    mod = 1 << cb
    bad = 0
    for e, f in zip(exact, fp64):
        diff = (f.astype(object) - e.astype(object)) % mod
        for x in diff[diff != 0]:
            bad += 1
            x = int(x)
            x = x if x < mod // 2 else x - mod
            # Each rounding slip is +-1 in one chunk pair, weighted
            # 2^(19 j): in balanced base 2^19 every digit stays small.
            digits = []
            for _ in range((cb + 18) // 19 + 1):
                r = x % (1 << 19)
                r = r - (1 << 19) if r >= (1 << 18) else r
                digits.append(r)
                x = (x - r) >> 19
            assert x in (0, -1) and max(abs(v) for v in digits) <= 4, digits
    rate = bad / (2 * len(exact[0]))
    print("d=4096 ExternalProduct: %d of %d coefficients differ (%.2f%%)"
          % (bad, 2 * len(exact[0]), 100 * rate))
    assert rate < 0.25


def test_finalize_fp64_is_exact_at_d8192():
    d = 8192
    rng = np.random.default_rng(3)
    prm = _params(64, 56, 13)
    b = rng.integers(0, 1 << 56, size=d, dtype=np.uint64)
    bp = rng.integers(0, 1 << 56, size=d, dtype=np.uint64)
    yh = rng.integers(0, 1 << 56, size=(2, d), dtype=np.uint64)
    th = rng.integers(-(1 << 18), 1 << 18, size=(2, d)).astype(np.uint64)
    exact = orc.finalize_matrix_pack(prm, b, bp, yh, th, orc.MODE_EXACT)
    fp64 = orc.finalize_matrix_pack(prm, b, bp, yh, th, orc.MODE_FP64)
    assert np.array_equal(exact, fp64)
