"""Loads libinspire_gb300.so and declares the C ABI (include/inspire_pir.h).

There is no fallback: if the library is missing, loading fails loudly.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libinspire_gb300.so")

_lib = None

# name -> (argtypes, restype)
_vp, _i32, _i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
_cp, _sz = ctypes.c_char_p, ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)

SIGNATURES = {
    "inspire_pir_server_create": (
        [_vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp,
         _i64, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_destroy": ([_vp], None),
    "inspire_pir_server_load": ([_vp, _vp, _sz, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_load_file": ([_vp, _cp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_save": ([_vp, _vp, _sz, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_load_preprocessed": (
        [_vp, _vp, _sz, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_load_preprocessed_dir": (
        [_vp, _cp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_save_preprocessed": (
        [_vp, _vp, _sz, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_save_preprocessed_dir": ([_vp, _cp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_save_file": ([_vp, _cp, _cp, _sz], ctypes.c_int),
    "inspire_pir_process_response": (
        [_vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_process_batch": (
        [_vp, _i32, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i32, _cp, _sz],
        ctypes.c_int),
    "inspire_pir_process_batch_device": (
        [_vp, _i32, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i32, _vp, _cp,
         _sz], ctypes.c_int),
    "inspire_vpir_process_batch": (
        [_vp, _i32, _vp, _i64, _vp, _i64, _i32, _vp, _i32, _cp, _sz],
        ctypes.c_int),
    "inspire_pir_products_device": (
        [_vp, _i32, _vp, _vp, _vp, _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_pack_batch_device": (
        [_vp, _i32, _vp, _i64, _vp, _i64, _vp, _i32, _vp, _cp, _sz],
        ctypes.c_int),
    "inspire_pir_external_product_device": (
        [_vp, _i32, _vp, _vp, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_autotune": ([_vp, _i32, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_tune_engines": ([_vp, _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_engine_table": ([_vp, _i32, _vp, _vp, _vp, _vp, _vp], _i32),
    "inspire_pir_tensor_products_device": (
        [_vp, _i32, _vp, _vp, _vp, _i32, _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_graph_begin": ([_vp, _cp, _sz], ctypes.c_int),
    "inspire_graph_end": ([_vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_graph_launch": ([_vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_graph_destroy": ([_vp], None),
    "inspire_pir_server_check": ([_vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_set_tensor_planes": ([_vp, _i32, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_device_bytes": ([_vp], _i64),
    "inspire_serving_create": (
        [_vp, _i32, _i32, _i32, _i32, _i32, _i64, _i32, _vp, _cp, _sz],
        ctypes.c_int),
    "inspire_serving_create_loopback": (
        [_i32, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _cp, _sz],
        ctypes.c_int),
    "inspire_serving_destroy": ([_vp], None),
    "inspire_serving_acquire": (
        [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_serving_submit": ([_vp, _i64, _i64, _cp, _sz], ctypes.c_int),
    "inspire_serving_wait": ([_vp, _i64, _i32, _cp, _sz], ctypes.c_int),
    "inspire_serving_release": ([_vp, _i64], ctypes.c_int),
    "inspire_serving_get_stats": ([_vp, _vp], ctypes.c_int),
    "inspire_serving_reset_stats": ([_vp], ctypes.c_int),
    "inspire_serving_queue_info": ([_vp, _i32, _vp, _vp, _vp], ctypes.c_int),
    "inspire_pir_workspace_bytes": ([_vp, _i32], ctypes.c_int64),
    "inspire_pir_workspace_create": ([_vp, _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_workspace_destroy": ([_vp], None),
    "inspire_pir_workspace_host_buffers": ([_vp, _vp, _vp, _vp, _vp],
                                           ctypes.c_int),
    "inspire_pir_workspace_submit": ([_vp, _i32, _i32, _cp, _sz], ctypes.c_int),
    "inspire_pir_workspace_poll": ([_vp], ctypes.c_int),
    "inspire_pir_workspace_wait": ([_vp, _cp, _sz], ctypes.c_int),
    "inspire_pir_server_shape": ([_vp, _i64p, _i64p, _i64p], ctypes.c_int),
    "inspire_pir_server_timings": ([_vp, _dp, _dp, _dp], ctypes.c_int),
    "inspire_matrix_multiply": (
        [_i32, _i32, _vp, _i64, _i64, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_inner_product": (
        [_i32, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _cp, _sz],
        ctypes.c_int),
    "inspire_external_product": (
        [_vp, _vp, _vp, _vp, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_inner_product_noalloc": (
        [_i32, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _cp,
         _sz], ctypes.c_int),
    "inspire_compute_hint_matrix": (
        [_i32, _i32, _vp, _i64, _i64, _vp, _i32, _i32, _vp, _i32, _vp, _cp,
         _sz], ctypes.c_int),
    "inspire_interpolate_db": (
        [_i32, _vp, _i64, _i64, _i32, _i32, _i32, ctypes.c_uint32, _vp, _i64,
         _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_interpolate": (
        [_i32, _vp, _i64, _i32, _i32, ctypes.c_uint32, _vp, _cp, _sz],
        ctypes.c_int),
    "inspire_finalize_matrix_pack": (
        [_vp, _vp, _vp, _vp, _vp, _vp, _cp, _sz], ctypes.c_int),
    "inspire_client_create_requests": (
        [_vp, _vp, _vp, _i64, _vp, _i32, ctypes.c_uint64, _i32, _vp, _vp, _vp,
         _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_client_process_responses": (
        [_vp, _vp, _vp, _i32, _vp, _i32, _vp, _cp, _sz], ctypes.c_int),
    "inspire_preprocess_matrix_pack": (
        [_i32, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _i64, _vp, _i64, _vp,
         _vp, _vp, _i32, _vp, _cp, _sz], ctypes.c_int),
}


class LibraryMissing(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Returns the loaded library, raising LibraryMissing if not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise LibraryMissing(
            "%s is not built; run `python -c \"import __graft_entry__ as g; "
            "g.build()\"` (the CUDA library has no CPU fallback)" % path)
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib
