"""GPU DB interpolation (PreprocessingServer::InterpolateAndTranspose and
Interpolate) against the CPU oracle and the reference's property test.

crypto/db_row_interpolation_test.cc:91-142 evaluates random polynomials P_i
at w^j = X^(j*2d/t) and checks that Interpolate returns the P_i; its
InvalidArguments test (:144-190) fixes the error messages.
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def evaluate(P, power, d, p):
    """sum_i P_i * X^(i*power) in Z_p[X]/(X^d+1)."""
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
                                   (128, 64, 65535), (4096, 8, 65535),
                                   (8192, 2, 65535)])
def test_interpolate_inverts_evaluation(dtype, d, t, p):
    rng = np.random.default_rng(d + t)
    P = rng.integers(0, p, size=(t, d)).astype(np.int64)
    evals = np.concatenate([evaluate(P, j * 2 * d // t, d, p)
                            for j in range(t)]).astype(dtype)
    got = pir.Interpolate(evals, d, t, p)
    assert np.array_equal(got.reshape(t, d), P.astype(dtype))
    assert np.array_equal(got, orc.interpolate(evals, d, t, p))


def test_interpolate_invalid_arguments():
    d, t, p = 32, 16, 1031
    row = (np.arange(d * t) % p).astype(np.uint16)
    pir.Interpolate(row, d, t, p)
    with pytest.raises(pir.InspireError,
                       match="Length of evals must be ring_degree"):
        pir.Interpolate(row[:-1], d, t, p)
    with pytest.raises(pir.InspireError, match="ring_degree must be a power"):
        pir.Interpolate(np.zeros((d - 1) * t, np.uint16), d - 1, t, p)
    with pytest.raises(pir.InspireError,
                       match="interpolation_degree must be a power"):
        pir.Interpolate(np.zeros(d * (t - 1), np.uint16), d, t - 1, p)
    with pytest.raises(pir.InspireError, match="less than or equal to 2"):
        pir.Interpolate(np.zeros(32 * 128, np.uint16), 32, 128, p)
    with pytest.raises(pir.InspireError, match="plaintext_modulus must be odd"):
        pir.Interpolate(row, d, t, p - 1)


def oracle_db(raw, n, d, t, l, p, cols):
    """The combined DB matrix from the oracle's Interpolate, group by group
    (preprocessing_server.h:68-95, 174-209)."""
    rec = raw.reshape(n, l, d)
    out = np.zeros((l * t * d, cols), dtype=raw.dtype)
    for k in range(l):
        for i in range(n // t):
            row = np.ascontiguousarray(rec[i * t:(i + 1) * t, k, :]).reshape(-1)
            interp = orc.interpolate(row, d, t, p) if t > 1 else row
            out[k * t * d:(k + 1) * t * d, i] = interp
    return out


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32])
@pytest.mark.parametrize("n,d,t,l,pad", [
    (64, 32, 4, 2, 32),       # padded columns (u64-coefficient layout)
    (100, 64, 8, 1, 0),       # n/t = 12 groups, last tile ragged
    (96, 16, 32, 1, 0),       # t = 2d: one position per class
    (50, 32, 1, 3, 0),        # t = 1: transposition only
    (256, 512, 2, 2, 0),      # register form (s = 2d/t >= 32)
    (640, 128, 4, 2, 32),     # register form, padded columns
    (560, 256, 8, 1, 0),      # register form, 70 groups: a ragged last tile
    (1600, 256, 8, 1, 8),     # 16-byte row stores, 8 groups in the last tile
    (1608, 256, 8, 2, 7),     # 16-byte row stores, odd last tile (9 groups)
    (1024, 128, 2, 1, 8),     # t = 2, 16-byte row stores
])
def test_interpolate_db_matches_oracle(dtype, n, d, t, l, pad):
    p = 255 if dtype == np.uint8 else 65535
    rng = np.random.default_rng(n + d + t + l)
    hi = 256 if dtype == np.uint8 else 65536
    raw = rng.integers(0, hi, size=n * l * d).astype(dtype)
    cols = n // t + pad
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=64,
                                   log_q=52, plaintext_modulus=p)
    got = pir.interpolate_db(raw, params, out_cols=cols)
    assert np.array_equal(got, oracle_db(raw, n, d, t, l, p, cols))


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_interpolate_db_streaming_many_tiles_per_block(dtype):
    # 8197 groups x 2 class blocks: more tiles than SMs, so every block of
    # the streaming kernel walks several tiles through its double-buffered
    # input stage; the last tile holds 5 groups.
    n, d, t, l = 8 * 8197, 256, 8, 1
    p = 255 if dtype == np.uint8 else 65535
    hi = 256 if dtype == np.uint8 else 65536
    raw = np.random.default_rng(17).integers(0, hi, size=n * l * d).astype(dtype)
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=64,
                                   log_q=52, plaintext_modulus=p)
    got = pir.interpolate_db(raw, params, out_cols=n // t)
    assert np.array_equal(got, oracle_db(raw, n, d, t, l, p, n // t))


def test_interpolate_db_device_call_and_size_check():
    import ctypes
    import torch
    n, d, t, l, p = 512, 256, 8, 1, 65535
    raw = np.random.default_rng(3).integers(0, 65535, size=n * l * d,
                                            dtype=np.uint16)
    params = synthetic.make_params(d=d, n=n, t=t, l=l, plaintext_modulus=p)
    want = pir.interpolate_db(raw, params)
    t_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    t_out = torch.zeros((l * t * d, n // t), dtype=torch.int16, device="cuda")
    lib = pir._lib.load()
    err = pir._errbuf()
    rc = lib.inspire_interpolate_db(
        16, ctypes.c_void_p(t_raw.data_ptr()), raw.size, n, d, t, l, p,
        ctypes.c_void_p(t_out.data_ptr()), n // t, 1,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), err, len(err))
    assert rc == 0, err.value
    torch.cuda.synchronize()
    assert np.array_equal(t_out.cpu().numpy().view(np.uint16), want)
    with pytest.raises(pir.InspireError, match="Invalid raw database size"):
        pir.interpolate_db(raw[:-1], params)
