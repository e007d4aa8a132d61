"""ComputeHintMatrix on the GPU against the reference's own definition
(crypto/hint_computation_test.cc:36-176: the naive negacyclic-matrix
product, mod 2^w) and the oracle's exact inner products at larger sizes."""
import numpy as np
import pytest

from inspire_gb300 import build, pir
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def naive_hint(db, a):
    """NaiveComputeHintMatrix: out[i][j] = sum_b sum_k db[i][b*d+k] * M_b[k][j]
    with M_b[k][j] = a_b[k-j] (k >= j) else -a_b[d+k-j], mod 2^w."""
    rows = db.shape[0]
    n, d = a.shape
    w = a.dtype.itemsize * 8
    mod = 1 << w
    out = np.zeros((rows, d), dtype=object)
    for b in range(n):
        M = np.empty((d, d), dtype=object)
        for k in range(d):
            for j in range(d):
                M[k][j] = int(a[b][k - j]) if k >= j else (-int(a[b][d + k - j])) % mod
        blk = db[:, b * d:(b + 1) * d].astype(object)
        out = (out + blk.dot(M)) % mod
    return out.astype(a.dtype)


@pytest.mark.parametrize("sdt,tdt", [(np.uint16, np.uint32),
                                     (np.uint16, np.uint64),
                                     (np.uint32, np.uint64)])
def test_hint_matches_reference_definition(sdt, tdt):
    rng = np.random.default_rng(7)
    for log_d in range(1, 5):
        d = 1 << log_d
        for n in (1, 2, 4):
            for rows in (1, 2, d, d + 5):
                db = rng.integers(0, np.iinfo(sdt).max, size=(rows, d * n),
                                  dtype=sdt, endpoint=True)
                a = rng.integers(0, np.iinfo(tdt).max, size=(n, d), dtype=tdt,
                                 endpoint=True)
                got = pir.ComputeHintMatrix(db, a)
                assert np.array_equal(got, naive_hint(db, a)), (d, n, rows)


@pytest.mark.parametrize("d,n,rows,tdt", [(4096, 4, 40, np.uint32),
                                          (2048, 8, 33, np.uint64),
                                          (8192, 2, 17, np.uint32)])
def test_hint_matches_exact_inner_products(d, n, rows, tdt):
    rng = np.random.default_rng(d + n)
    db = rng.integers(0, 65535, size=(rows, d * n), dtype=np.uint16)
    a = rng.integers(0, np.iinfo(tdt).max, size=(n, d), dtype=tdt, endpoint=True)
    got = pir.ComputeHintMatrix(db, a)
    cb = 8 * a.dtype.itemsize
    vinv = np.concatenate([a[:, :1], (-a[:, :0:-1].astype(object)) % (1 << cb)],
                          axis=1).astype(tdt)
    for i in (0, rows - 1):
        u = db[i].reshape(n, d).astype(tdt)
        chunk = min(20, int((53.0 - np.log2(n) - np.log2(d)) / 2.0))
        want = orc.inner_product(u, vinv, cb, 16, cb, chunk)
        assert np.array_equal(got[i], want), i


def test_hint_invalid_parameters():
    a = np.zeros((1, 4), dtype=np.uint32)
    with pytest.raises(pir.InspireError, match="Database matrix cannot be empty"):
        pir.ComputeHintMatrix(np.zeros((0, 4), np.uint16), a)
    with pytest.raises(pir.InspireError, match="a_components cannot be empty"):
        pir.ComputeHintMatrix(np.zeros((2, 4), np.uint16),
                              np.zeros((0, 4), np.uint32))
    with pytest.raises(pir.InspireError,
                       match="Database columns must match d \\* n"):
        pir.ComputeHintMatrix(np.zeros((2, 3), np.uint16), a)


def test_hint_device_pointers_match_host_call():
    import ctypes
    import torch
    rng = np.random.default_rng(11)
    d, n, rows = 256, 3, 20
    db = rng.integers(0, 65535, size=(rows, d * n), dtype=np.uint16)
    a = rng.integers(0, 1 << 32, size=(n, d), dtype=np.uint64).astype(np.uint32)
    want = pir.ComputeHintMatrix(db, a)
    t_db = torch.from_numpy(db.view(np.int16)).cuda()
    t_a = torch.from_numpy(a.view(np.int32)).cuda()
    t_out = torch.zeros((rows, d), dtype=torch.int32, device="cuda")
    err = pir._errbuf()
    rc = pir._lib.load().inspire_compute_hint_matrix(
        1, 32, ctypes.c_void_p(t_db.data_ptr()), rows, d * n,
        ctypes.c_void_p(t_a.data_ptr()), n, d, ctypes.c_void_p(t_out.data_ptr()),
        1, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), err,
        len(err))
    assert rc == 0, err.value
    torch.cuda.synchronize()
    assert np.array_equal(t_out.cpu().numpy().view(np.uint32), want)
