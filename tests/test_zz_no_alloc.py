"""The allocation-free InnerProductFft entry point.

inspire_inner_product_noalloc exists for callers that cannot call cudaMalloc
(a host runtime that owns the device memory budget, a request path that must
not block on an allocation): they hand in device buffers for the operands and
the result, and the NTT scratch is a fixed array inside the library. This
file checks it through the C ABI against the allocating entry point
inspire_inner_product, bit for bit, on two calls in a row (the second call
must not see the first call's scratch), and checks that sizes beyond its
fixed scratch are refused. It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from inspire_gb300 import _lib, build, pir

pytestmark = pytest.mark.gpu

CASES = [
    # (coeff_bits, n, d, u_bits, v_bits, chunk_bits, u_signed)
    (32, 6, 4096, 19, 32, 19, False),   # ExternalProduct operands
    (32, 2, 4096, 19, 32, 20, True),    # FinalizeMatrixPack operands
    (64, 2, 2048, 19, 52, 20, True),
    (64, 8, 1024, 64, 64, 20, False),   # full-width 64-bit operands
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


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    err = ctypes.create_string_buffer(512)
    for n, d in ((9, 1024), (2, 8192)):
        rc = lib.inspire_inner_product_noalloc(32, None, None, n, d, 19, 32,
                                               18, 0, None, None, err,
                                               len(err))
        assert rc == pir.INVALID_ARGUMENT
        assert b"at most 8 polynomials of degree at most 4096" in err.value
