"""Pins the CPU oracle against the reference's own known-answer tests.

Each case cites the reference test it restates. The reference ships no golden
vector files; these known answers and the FFT == exact-product assertions on
std::mt19937_64(12345) inputs are the fixed points its test-suite holds.
"""
import numpy as np
import pytest

from oracle import pyoracle as orc
from tests.refrng import MT19937_64

U32MAX = 0xFFFFFFFF


def negacyclic(u, v, bits):
    """Independent schoolbook negacyclic product mod 2^bits (numpy, wraps)."""
    u = np.asarray(u, dtype=np.uint64)
    v = np.asarray(v, dtype=np.uint64)
    d = u.shape[0]
    acc = np.zeros(d, dtype=np.uint64)
    with np.errstate(over="ignore"):
        for a in range(d):
            if u[a] == 0:
                continue
            acc[a:] += u[a] * v[:d - a]
            acc[:a] -= u[a] * v[d - a:]
    if bits == 32:
        return (acc & np.uint64(U32MAX)).astype(np.uint32)
    return acc


def test_mt19937_64_standard_value():
    # C++ [rand.predef]: the 10000th output of a default-constructed
    # mt19937_64 is 9981545732273789042.
    g = MT19937_64()
    for _ in range(9999):
        g()
    assert g() == 9981545732273789042


@pytest.mark.parametrize("dt,kind", [(np.uint8, "u8"), (np.uint16, "u16"),
                                     (np.uint32, "u32"), (np.uint64, "u64"),
                                     (np.int16, "i16"), (np.int32, "i32")])
@pytest.mark.parametrize("coeff_bits", [32, 64])
def test_matrix_multiply_valid(dt, kind, coeff_bits):
    # crypto/matrix_test.cc:81-88 (MatrixTest.MultiplyValid): [17, 39].
    m = np.array([[1, 2], [3, 4]], dtype=dt)
    out = orc.matrix_multiply(m, [5, 6], coeff_bits)
    assert out.tolist() == [17, 39]


def test_condensed_u16_known_answer():
    # crypto/matrix_test.cc:90-111: entries [1,2,3,4] repeated, vec = 1 -> 80.
    m = np.tile(np.array([1, 2, 3, 4], dtype=np.uint16), (2, 8))
    v = np.ones(32, dtype=np.uint64)
    assert orc.condensed_multiply(m, v).tolist() == [80, 80]
    assert orc.matrix_multiply(m, v, 64).tolist() == [80, 80]


def test_condensed_i32_known_answer():
    # crypto/matrix_test.cc:113-134: entries [-1, 2] repeated -> 16.
    m = np.tile(np.array([-1, 2], dtype=np.int32), (2, 16))
    v = np.ones(32, dtype=np.uint64)
    assert orc.condensed_multiply(m, v).tolist() == [16, 16]
    assert orc.matrix_multiply(m, v, 64).tolist() == [16, 16]


@pytest.mark.parametrize("cols,expect", [(64, 288), (1024, 4608)])
def test_condensed_u8_known_answer(cols, expect):
    # crypto/matrix_test.cc:136-183: entries 1..8 repeated.
    m = np.tile(np.arange(1, 9, dtype=np.uint8), (2, cols // 8))
    v = np.ones(cols, dtype=np.uint64)
    assert orc.condensed_multiply(m, v).tolist() == [expect, expect]


def test_condensed_rejects_ragged_columns():
    # crypto/matrix.cc:269-272.
    m = np.ones((2, 20), dtype=np.uint16)
    with pytest.raises(orc.OracleError, match="multiple of 4 \\* Lanes"):
        orc.condensed_multiply(m, np.ones(20, dtype=np.uint64))


def test_automorph_known_answer():
    # crypto/polynomial_test.cc:103-115.
    out = orc.automorph([1, 2, 3, 4], 32, 3)
    assert out.tolist() == [1, 4, U32MAX - 2, 2]


@pytest.mark.parametrize("power", [-1, 2, 8, 9])
def test_automorph_invalid_power(power):
    # crypto/polynomial_test.cc:117-140.
    with pytest.raises(orc.OracleError,
                       match="non-negative odd integer"):
        orc.automorph([1, 2, 3, 4], 32, power)


def test_gadget_inv_known_answers():
    # crypto/polynomial_test.cc:187-203.
    p = [0x12345678, 0xFFFFFFFF, 0, 1]
    g = orc.gadget_inv(p, 32, 0, 8, 4)
    assert g.tolist() == [[0x78, 0xFF, 0, 1], [0x56, 0xFF, 0, 0],
                          [0x34, 0xFF, 0, 0], [0x12, 0xFF, 0, 0]]
    g2 = orc.gadget_inv(p, 32, 0, 16, 3)
    assert g2.tolist() == [[0x5678, 0xFFFF, 0, 1], [0x1234, 0xFFFF, 0, 0],
                           [0, 0, 0, 0]]


def test_approximate_gadget_inv_known_answer():
    # crypto/polynomial_test.cc:205-214.
    p = [0x12345678, 0xFFFFFFFF, 0, 1, 0x80000000, 0x7FFFFFFF, 0, 0]
    g = orc.gadget_inv(p, 32, 0, 8, 2)
    assert g.tolist() == [[0x34, 0, 0, 0, 0, 0, 0, 0],
                          [0x12, 0, 0, 0, 0x80, 0x80, 0, 0]]


def test_signed_gadget_inv_known_answer():
    # crypto/polynomial_test.cc:216-236.
    p = [0x12345698, 0xFFFFFFFF, 0, 1]
    g = orc.gadget_inv(p, 32, 0, 8, 4, signed=True)
    assert g.tolist() == [[0xFFFFFF98, 0xFFFFFFFF, 0, 1], [0x57, 0, 0, 0],
                          [0x34, 0, 0, 0], [0x12, 0, 0, 0]]
    recon = np.zeros(4, dtype=np.uint64)
    for i in range(4):
        recon += g[i].astype(np.uint64) << np.uint64(8 * i)
    assert (recon & np.uint64(U32MAX)).tolist() == p


def test_approximate_signed_gadget_inv_known_answer():
    # crypto/polynomial_test.cc:238-246.
    g = orc.gadget_inv([0x12345678, 0x129B9856, 0, 1], 32, 0, 8, 2,
                       signed=True)
    assert g.tolist() == [[0x34, 0xFFFFFF9C, 0, 0], [0x12, 0x13, 0, 0]]


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("ld,nd", [(0, 4), (-1, 4), (7, 0), (7, -1)])
def test_gadget_inv_invalid_params(signed, ld, nd):
    # crypto/polynomial_test.cc:248-275.
    with pytest.raises(orc.OracleError, match="must be positive"):
        orc.gadget_inv([1, 2, 3, 4], 32, 0, ld, nd, signed=signed)


@pytest.mark.parametrize("mode", [orc.MODE_EXACT, orc.MODE_FP64])
def test_mult_fft_degree4_u32(mode):
    # crypto/polynomial_test.cc:399-408.
    u = [1, 2, 3, 4]
    v = [5, 6, 7, 8]
    got = orc.inner_product(u, v, 32, mode=mode)
    assert got.tolist() == negacyclic(u, v, 32).tolist()


@pytest.mark.parametrize("mode", [orc.MODE_EXACT, orc.MODE_FP64])
def test_mult_fft_degree16_u64(mode):
    # crypto/polynomial_test.cc:410-425.
    m = (1 << 64) - 1
    c1 = [(0x123456789ABCDEF * (i + 1)) & m for i in range(16)]
    c2 = [(0xFEDCBA987654321 * (16 - i)) & m for i in range(16)]
    got = orc.inner_product(c1, c2, 64, mode=mode)
    assert got.tolist() == negacyclic(c1, c2, 64).tolist()


@pytest.mark.parametrize("mode", [orc.MODE_EXACT, orc.MODE_FP64])
def test_mult_fft_degree1024_u64(mode):
    # crypto/polynomial_test.cc:427-442.
    c1 = [i * 1000000000 for i in range(1024)]
    c2 = [(1024 - i) * 1000000000 for i in range(1024)]
    got = orc.inner_product(c1, c2, 64, mode=mode)
    assert got.tolist() == negacyclic(c1, c2, 64).tolist()


def test_mult_fft_random_mt19937():
    # crypto/polynomial_test.cc:444-491: std::mt19937_64(12345), full-range
    # uniform draws, degrees 128..2048, u32 then u64 at each degree.
    g = MT19937_64(12345)
    for degree in (128, 256, 512, 1024, 2048):
        c1 = [g() & U32MAX for _ in range(degree)]
        c2 = [g() & U32MAX for _ in range(degree)]
        want = negacyclic(c1, c2, 32)
        for mode in (orc.MODE_EXACT, orc.MODE_FP64):
            assert np.array_equal(orc.inner_product(c1, c2, 32, mode=mode),
                                  want)
        c1 = [g() for _ in range(degree)]
        c2 = [g() for _ in range(degree)]
        want = negacyclic(c1, c2, 64)
        for mode in (orc.MODE_EXACT, orc.MODE_FP64):
            assert np.array_equal(orc.inner_product(c1, c2, 64, mode=mode),
                                  want)


def test_mult_fft_explicit_bits_mt19937():
    # crypto/polynomial_test.cc:493-528.
    g = MT19937_64(12345)
    for degree in (128, 256, 512, 1024, 2048):
        this_bits = g() % 31 + 1
        that_bits = g() % 31 + 1
        tm = (1 << this_bits) - 1
        am = (1 << that_bits) - 1
        c1, c2 = [], []
        for _ in range(degree):
            c1.append(g() & U32MAX & tm)
            c2.append(g() & U32MAX & am)
        want = negacyclic(c1, c2, 32)
        for chunk in (12, 16, 20):
            for mode in (orc.MODE_EXACT, orc.MODE_FP64):
                got = orc.inner_product(c1, c2, 32, this_bits, that_bits,
                                        chunk, mode=mode)
                assert np.array_equal(got, want), (degree, chunk, mode)


def test_inner_product_fft_small():
    # crypto/polynomial_test.cc:530-548.
    u = [[1, 2, 3, 4], [2, 3, 4, 5]]
    v = [[5, 6, 7, 8], [1, 1, 1, 1]]
    want = (negacyclic(u[0], v[0], 32).astype(np.uint64) +
            negacyclic(u[1], v[1], 32)) & U32MAX
    for mode in (orc.MODE_EXACT, orc.MODE_FP64):
        assert orc.inner_product(u, v, 32, mode=mode).tolist() == want.tolist()


def test_inner_product_fft_random_mt19937():
    # crypto/polynomial_test.cc:550-608, including the boundary chunk size.
    g = MT19937_64(12345)
    for degree in (128, 512, 2048):
        for k in (1, 5, 10):
            this_bits = g() % 31 + 1
            that_bits = g() % 31 + 1
            tm = (1 << this_bits) - 1
            am = (1 << that_bits) - 1
            u, v = [], []
            want = np.zeros(degree, dtype=np.uint64)
            for _ in range(k):
                c1, c2 = [], []
                for _ in range(degree):
                    c1.append(g() & U32MAX & tm)
                    c2.append(g() & U32MAX & am)
                want = (want + negacyclic(c1, c2, 32)) & np.uint64(U32MAX)
                u.append(c1)
                v.append(c2)
            chunks = [12, 16, 20]
            boundary = int((53.0 - np.log2(k) - np.log2(degree)) / 2.0)
            if boundary > 0:
                chunks.append(boundary)
            for chunk in chunks:
                if np.log2(k) + np.log2(degree) + 2.0 * chunk > 53.0:
                    continue
                for mode in (orc.MODE_EXACT, orc.MODE_FP64):
                    got = orc.inner_product(u, v, 32, this_bits, that_bits,
                                            chunk, mode=mode)
                    assert np.array_equal(got, want.astype(np.uint32)), (
                        degree, k, chunk, mode)


def test_inner_product_precision_guard():
    # crypto/polynomial_fft.cc:93-96.
    u = np.ones((4, 1024), dtype=np.uint32)
    with pytest.raises(orc.OracleError, match="precision overflow"):
        orc.inner_product(u, u, 32, chunk_bits=21)


def test_rescale_rounds_half_up():
    # crypto/polynomial.cc:287-304: round(c * 2^new / 2^cur).
    c = np.array([0, 1, 2, 3, (1 << 20) - 1, 1 << 19, (1 << 19) - 1],
                 dtype=np.uint32)
    got = orc.rescale(c, 32, 20, 1)
    want = [(x * 2 + (1 << 19)) // (1 << 20) for x in c.tolist()]
    assert got.tolist() == want


# --------------------------------------------------------- Interpolate ----
def _evaluate(P, power, d, p):
    """sum_i P_i * X^(i*power) in Z_p[X]/(X^d+1)
    (crypto/db_row_interpolation_test.cc:36-82)."""
    out = np.zeros(d, dtype=np.int64)
    for i, poly in enumerate(P):
        k = (i * power) % (2 * d)
        sign = 1
        if k >= d:
            sign, k = -1, k - d
        rot = np.concatenate([-poly[d - k:], poly[:d - k]]) if k else poly
        out = (out + sign * rot.astype(np.int64)) % p
    return out


@pytest.mark.parametrize("dtype", [np.uint16, np.uint32])
@pytest.mark.parametrize("d,t,p", [(32, 16, 1031), (64, 32, 2031),
                                   (128, 64, 65535)])
def test_oracle_interpolate_reference_property(dtype, d, t, p):
    # crypto/db_row_interpolation_test.cc:91-142: evaluating random P_i at
    # w^j = X^(j*2d/t) and interpolating returns the P_i.
    rng = np.random.default_rng(d * t)
    P = rng.integers(0, p, size=(t, d)).astype(np.int64)
    evals = np.concatenate([_evaluate(P, j * 2 * d // t, d, p)
                            for j in range(t)]).astype(dtype)
    got = orc.interpolate(evals, d, t, p)
    assert np.array_equal(got.reshape(t, d), P.astype(dtype))


def test_oracle_interpolate_invalid_arguments():
    # crypto/db_row_interpolation_test.cc:144-190.
    row = (np.arange(32 * 16) % 1031).astype(np.uint16)
    orc.interpolate(row, 32, 16, 1031)
    with pytest.raises(orc.OracleError, match="ring_degree must be a power"):
        orc.interpolate(np.zeros(31 * 16, np.uint16), 31, 16, 1031)
    with pytest.raises(orc.OracleError,
                       match="interpolation_degree must be a power"):
        orc.interpolate(np.zeros(32 * 15, np.uint16), 32, 15, 1031)
    with pytest.raises(orc.OracleError, match="less than or equal to 2"):
        orc.interpolate(np.zeros(32 * 128, np.uint16), 32, 128, 1031)
    with pytest.raises(orc.OracleError, match="plaintext_modulus must be odd"):
        orc.interpolate(row, 32, 16, 1030)
