"""CPU-side checks of the C ABI library: it loads without a GPU and exports
every function that include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

from inspire_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(inspire_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "inspire_pir_server_create" in names
    assert "inspire_pir_process_response" in names
    assert len(names) >= 10


def test_library_exports_every_declared_function(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_signatures_cover_header(lib):
    # Every declared function has a ctypes signature in the Python mirror.
    for name in declared_functions():
        assert name in _lib.SIGNATURES, name


def test_null_server_is_rejected_without_gpu(lib):
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_pir_process_batch(None, 1, None, 0, None, 0, None, 0,
                                       None, 0, err, len(err))
    assert rc == 3
    assert b"server is null" in err.value


def test_inner_product_rejects_empty_without_gpu(lib):
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_inner_product(32, None, None, 0, 32, 32, 32, 20, 0, None,
                                   err, len(err))
    assert rc == 3
    assert b"cannot be empty" in err.value


@pytest.mark.parametrize("coeff_bits,n,d,u_bits,v_bits,chunk_bits,message", [
    (16, 1, 64, 8, 8, 8, b"coeff_bits must be 32 or 64."),
    (32, 1, 48, 8, 8, 8, b"Polynomial lengths or context mismatch."),
    (32, 1, 1, 8, 8, 8, b"Polynomial lengths or context mismatch."),
    (32, 1, 64, 0, 8, 8, b"Invalid bits or chunk_bits."),
    (32, 1, 64, 8, -1, 8, b"Invalid bits or chunk_bits."),
    (64, 1, 64, 8, 8, 64, b"Invalid bits or chunk_bits."),
    # log2(n) + log2(d) + 2 chunk_bits > 53 (polynomial_fft.cc:93-96).
    (32, 8, 4096, 19, 32, 20, b"Potential precision overflow in accumulation."),
])
def test_inner_product_argument_checks_without_gpu(lib, coeff_bits, n, d, u_bits,
                                                   v_bits, chunk_bits, message):
    """InnerProductFft's checks (crypto/polynomial_fft.cc:68-96) come before
    any device work, with the reference's messages."""
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_inner_product(coeff_bits, None, None, n, d, u_bits, v_bits,
                                   chunk_bits, 0, None, err, len(err))
    assert rc == 3
    assert message in err.value


@pytest.mark.parametrize("n,d,t,p,message", [
    (64 * 4 - 1, 64, 4, 65537, b"Length of evals must be ring_degree * interpolation_degree."),
    (48 * 4, 48, 4, 65537, b"ring_degree must be a power of two."),
    (64 * 3, 64, 3, 65537, b"interpolation_degree must be a power of two."),
    (16 * 64, 16, 64, 65537,
     b"interpolation_degree must be less than or equal to 2 * ring_degree."),
    (64 * 4, 64, 4, 65536, b"plaintext_modulus must be odd."),
])
def test_interpolate_argument_checks_without_gpu(lib, n, d, t, p, message):
    """Interpolate's checks (crypto/db_row_interpolation.cc:115-143) come
    before any device work, with the reference's messages."""
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_interpolate(16, None, n, d, t, p, None, err, len(err))
    assert rc == 3
    assert message in err.value


@pytest.mark.parametrize("rows,cols,n,d,message", [
    (0, 128, 2, 64, b"Database matrix cannot be empty."),
    (4, 128, 0, 64, b"a_components cannot be empty."),
    (4, 100, 2, 64, b"Database columns must match d * n where d is the polynomial "
                    b"length and n is the number of polynomials."),
])
def test_hint_matrix_argument_checks_without_gpu(lib, rows, cols, n, d, message):
    """ComputeHintMatrix's checks, in the reference's order
    (crypto/hint_computation.cc:81-97), before any device work."""
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_compute_hint_matrix(1, 32, None, rows, cols, None, n, d, None,  # u16 DB
                                         0, None, err, len(err))
    assert rc == 3
    assert message in err.value


@pytest.mark.parametrize("coeff_bits,mat_kind,log_q,log_digit,digits,d,slices,a_count,message", [
    # PreprocessMatrixPack's inner product of the gadget vector
    # (crypto/lwes_to_rlwe.cc:62-68): 2 * num_digits a-polynomials.
    (32, 5, 32, 8, 4, 64, 1, 7, b"InnerProduct: size mismatch or empty"),
    (48, 5, 32, 8, 4, 64, 1, 8, b"coeff_bits must be 32 or 64."),
    (32, 5, 32, 0, 4, 64, 1, 8, b"log_digit and num_digits must be positive."),
    (32, 5, 40, 8, 4, 64, 1, 8, b"log_modulus must be in (0, coeff_bits]."),
    (32, 5, 32, 8, 4, 48, 1, 8, b"polynomial length must be a power of two"),
    (32, 5, 32, 8, 4, 64, 0, 8, b"slices must be positive."),
])
def test_preprocess_matrix_pack_argument_checks_without_gpu(
        lib, coeff_bits, mat_kind, log_q, log_digit, digits, d, slices, a_count, message):
    err = ctypes.create_string_buffer(256)
    rc = lib.inspire_preprocess_matrix_pack(coeff_bits, mat_kind, log_q, log_digit, digits,
                                            d, slices, None, d, None, a_count, None, None,
                                            None, 0, None, err, len(err))
    assert rc == 3
    assert message in err.value
