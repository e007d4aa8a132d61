"""The allocation-free InnerProductFft entry point.

inspire_inner_product_noalloc exists for callers that cannot call cudaMalloc
(a host runtime that owns the device memory budget, a request path that must
not block on an allocation): they hand in device buffers for the operands and
the result, and the NTT scratch is a fixed array inside the library. This
file checks it through the C ABI against the allocating entry point
inspire_inner_product and against the CPU oracle's exact InnerProductFft,
bit for bit, on two calls in a row (the second call must not see the first
call's scratch), checks that a call leaves the device's free memory as it
was, and that sizes beyond its fixed scratch are refused. It is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

from inspire_gb300 import _lib, build, pir
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu

CASES = [
    # (coeff_bits, n, d, u_bits, v_bits, chunk_bits, u_signed)
    (32, 6, 4096, 19, 32, 19, False),   # ExternalProduct operands
    (32, 2, 4096, 19, 32, 20, True),    # FinalizeMatrixPack operands
    (64, 2, 2048, 19, 52, 20, True),
    (64, 8, 1024, 64, 64, 20, False),   # full-width 64-bit operands
    (32, 1, 4, 8, 8, 4, True),          # the smallest degrees, one poly
    (64, 1, 32, 64, 64, 16, False),
    (32, 8, 4096, 32, 32, 19, False),   # the largest n and d together
]


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def _call(lib, torch, cb, u, v, n, d, ub, vb, chunk, signed, stream):
    view = np.int32 if cb == 32 else np.int64
    du = torch.from_numpy(u.view(view)).cuda()
    dv = torch.from_numpy(v.view(view)).cuda()
    dout = torch.full((d,), -1, dtype=torch.int32 if cb == 32 else torch.int64,
                      device="cuda")
    err = ctypes.create_string_buffer(512)
    rc = lib.inspire_inner_product_noalloc(
        cb, du.data_ptr(), dv.data_ptr(), n, d, ub, vb, chunk, int(signed),
        dout.data_ptr(), stream, err, len(err))
    assert rc == 0, err.value
    torch.cuda.synchronize()
    return dout.cpu().numpy().view(np.uint32 if cb == 32 else np.uint64)


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_allocating_entry_point(lib, case):
    torch = pytest.importorskip("torch")
    cb, n, d, ub, vb, chunk, signed = case
    cdt = np.uint32 if cb == 32 else np.uint64
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rng = np.random.default_rng(1000 * call + n + d + cb)
        u = rng.integers(0, np.iinfo(cdt).max, size=(n, d), dtype=cdt,
                         endpoint=True)
        v = rng.integers(0, np.iinfo(cdt).max, size=(n, d), dtype=cdt,
                         endpoint=True)
        want = pir.inner_product(u, v, cb, ub, vb, chunk, u_signed=signed)
        got = _call(lib, torch, cb, u, v, n, d, ub, vb, chunk, signed, stream)
        assert np.array_equal(got, want), (case, call)
        exact = orc.inner_product(u, v, cb, ub, vb, chunk, u_signed=signed,
                                  mode=orc.MODE_EXACT)
        assert np.array_equal(got, exact), (case, call)


def test_noalloc_call_leaves_free_memory_unchanged(lib):
    torch = pytest.importorskip("torch")
    cb, n, d, ub, vb, chunk, signed = CASES[0]
    rng = np.random.default_rng(5)
    u = rng.integers(0, 1 << 32, size=(n, d), dtype=np.uint64).astype(np.uint32)
    v = rng.integers(0, 1 << 32, size=(n, d), dtype=np.uint64).astype(np.uint32)
    du = torch.from_numpy(u.view(np.int32)).cuda()
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    dout = torch.empty((d,), dtype=torch.int32, device="cuda")
    err = ctypes.create_string_buffer(512)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = lib.inspire_inner_product_noalloc(
            cb, du.data_ptr(), dv.data_ptr(), n, d, ub, vb, chunk,
            int(signed), dout.data_ptr(), stream, err, len(err))
        assert rc == 0, err.value
        torch.cuda.synchronize()
    call()  # the first call on a device looks up the scratch address
    free_before, _ = torch.cuda.mem_get_info()
    call()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    err = ctypes.create_string_buffer(512)
    for n, d in ((9, 1024), (2, 8192)):
        rc = lib.inspire_inner_product_noalloc(32, None, None, n, d, 19, 32,
                                               18, 0, None, None, err,
                                               len(err))
        assert rc == pir.INVALID_ARGUMENT
        assert b"at most 8 polynomials of degree at most 4096" in err.value
