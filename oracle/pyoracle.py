"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
leg import this module, and only as the checker or the timed CPU baseline.
The product path (inspire_gb300/) never imports it.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

MODE_EXACT = 0
MODE_FP64 = 1

# Matrix element kinds (match pir_oracle.h).
KIND = {"u8": 0, "u16": 1, "u32": 2, "u64": 3, "i16": 4, "i32": 5}
KIND_DTYPE = {0: np.uint8, 1: np.uint16, 2: np.uint32, 3: np.uint64,
              4: np.int16, 5: np.int32}


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("oracle status %d: %s" % (code, msg))
        self.code = code
        self.msg = msg


class OrcParams(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int32) for name in (
        "coeff_bits", "log_degree", "log_modulus", "log_modulus1_after_switch",
        "log_modulus2_after_switch", "pack_log_digit", "pack_num_digits",
        "eval_log_digit", "eval_num_digits", "num_entries",
        "interpolation_degree", "entry_size_multiple")]


_lib = None
_timing_lib = None


def lib():
    """The checker build of the oracle."""
    global _lib
    if _lib is None:
        _lib = _load(build_oracle.build())
    return _lib


TIMING_FALLBACK = None  # why the checker build stands in for the timing one


def _timing_build_runs(path):
    """Runs a small staged request through the timing build in a child
    process: a build whose target flags the host cannot execute traps
    there, not in the caller."""
    import subprocess
    import sys
    code = ("import numpy as np, ctypes\n"
            "from oracle import pyoracle as o\n"
            "lb = o._load(%r)\n"
            "d = 64\n"
            "p = o.make_params(coeff_bits=64, log_degree=6, log_modulus=52,"
            " log_modulus1_after_switch=24, log_modulus2_after_switch=18,"
            " pack_log_digit=19, pack_num_digits=2, eval_log_digit=19,"
            " eval_num_digits=3, num_entries=256, interpolation_degree=2,"
            " entry_size_multiple=1)\n"
            "r = np.random.default_rng(1)\n"
            "u = lambda *s: r.integers(0, 1 << 52, size=s, dtype=np.uint64)\n"
            "db = r.integers(0, 65535, size=(2 * d, 128), dtype=np.uint16)\n"
            "pk = r.integers(-1000, 1000, size=(2 * d, 2 * d), dtype=np.int32)\n"
            "for c in (0, 1):\n"
            "    o.process_response_staged(p, db, pk, u(2, d), u(4, d),"
            " u(6, d), u(128), u(6, d), u(4, d), threads=2, condensed_db=c,"
            " library=lb)\n"
            "p.coeff_bits, p.log_modulus = 32, 32\n"
            "w = lambda *s: u(*s).astype(np.uint32)\n"
            "o.process_response_staged(p, db, pk, w(2, d), w(4, d), w(6, d),"
            " w(128), w(6, d), w(4, d), threads=2, library=lb)\n" % path)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root,
                       capture_output=True, text=True, timeout=300)
    return r.returncode == 0, (r.stderr.strip().splitlines() or [""])[-1]


def timing_lib():
    """The timing build (same source, host-tuned flags): the CPU baseline.
    If that build cannot run on this host, the checker build is timed
    instead and TIMING_FALLBACK says why."""
    global _timing_lib, TIMING_FALLBACK
    if _timing_lib is None:
        path = build_oracle.build_timing()
        ok, why = _timing_build_runs(path)
        if ok:
            _timing_lib = _load(path)
        else:
            TIMING_FALLBACK = "timing build failed its self-check (%s)" % why
            _timing_lib = lib()
    return _timing_lib


def timing_build_string():
    """The compiler flags of the library timing_lib() returns."""
    timing_lib()
    if TIMING_FALLBACK:
        return ("g++ -O3 -ffp-contract=off (no target flags: %s)"
                % TIMING_FALLBACK)
    return build_oracle.timing_build_string()


def _load(path):
    """Loads one build of the oracle and sets its signatures."""
    lb = ctypes.CDLL(path)
    vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    cp, sz = ctypes.c_char_p, ctypes.c_size_t
    pp = ctypes.POINTER(OrcParams)
    sigs = {
        "orc_matrix_multiply": [ci, ci, vp, i64, i64, vp, vp, cp, sz],
        "orc_condensed_multiply": [ci, vp, i64, i64, vp, vp, ci, cp, sz],
        "orc_inner_product": [ci, ci, vp, vp, ci, ci, ci, ci, ci, ci, vp,
                              cp, sz],
        "orc_gadget_inv": [ci, vp, ci, ci, ci, ci, vp, cp, sz],
        "orc_signed_gadget_inv": [ci, vp, ci, ci, ci, ci, vp, cp, sz],
        "orc_rescale": [ci, vp, ci, ci, ci, vp],
        "orc_automorph": [ci, vp, ci, ci, vp, cp, sz],
        "orc_finalize_matrix_pack": [pp, ci, vp, vp, vp, vp, vp, cp, sz],
        "orc_external_product": [pp, ci, vp, vp, vp, vp, vp, cp, sz],
        "orc_process_response": [pp, ci, ci, vp, i64, ci, vp, i64, vp, vp,
                                 vp, vp, i64, vp, i64, vp, i64, vp, cp,
                                 sz],
        "orc_process_response_staged": [pp, ci, ci, vp, i64, ci, vp, i64,
                                        vp, vp, vp, vp, i64, vp, i64, vp,
                                        i64, vp, ci, ci, vp, cp, sz],
        "orc_interpolate": [ci, vp, ci, ci, ctypes.c_uint32, vp, cp, sz],
        "orc_preprocess_matrix_pack": [ci, ci, ci, ci, ci, ci, vp, vp, vp,
                                       vp, vp, vp, vp, vp, cp, sz],
        "orc_pack": [ci, ci, ci, ci, ci, ci, vp, vp, vp, vp, vp, vp, vp,
                     cp, sz],
    }
    for name, args in sigs.items():
        fn = getattr(lb, name)
        fn.argtypes = args
        fn.restype = ci
    return lb


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _call(fn, *args):
    err = ctypes.create_string_buffer(512)
    rc = fn(*args, err, len(err))
    if rc != 0:
        raise OracleError(rc, err.value.decode(errors="replace"))


def _cdt(coeff_bits):
    return np.uint32 if coeff_bits == 32 else np.uint64


def matrix_multiply(mat, vec, coeff_bits):
    """Matrix::Multiply<CoeffType> (crypto/matrix.h:167-195)."""
    mat = np.ascontiguousarray(mat)
    kind = {np.dtype(v): k for k, v in KIND_DTYPE.items()}[mat.dtype]
    vec = np.ascontiguousarray(vec, dtype=_cdt(coeff_bits))
    rows, cols = mat.shape
    if vec.shape[0] != cols:
        raise OracleError(3, "Vector size must match the number of matrix "
                             "columns.")
    out = np.zeros(rows, dtype=_cdt(coeff_bits))
    _call(lib().orc_matrix_multiply, kind, coeff_bits, _ptr(mat), rows, cols,
          _ptr(vec), _ptr(out))
    return out


def condensed_multiply(mat, vec, lanes=8):
    """CondensedMultiply<uint8/uint16/int32> (crypto/matrix.cc:261-462)."""
    mat = np.ascontiguousarray(mat)
    kind = {np.dtype(v): k for k, v in KIND_DTYPE.items()}[mat.dtype]
    vec = np.ascontiguousarray(vec, dtype=np.uint64)
    rows, cols = mat.shape
    out = np.zeros(rows, dtype=np.uint64)
    _call(lib().orc_condensed_multiply, kind, _ptr(mat), rows, cols, _ptr(vec),
          _ptr(out), lanes)
    return out


def inner_product(u, v, coeff_bits, u_bits=None, v_bits=None, chunk_bits=20,
                  u_signed=False, mode=MODE_EXACT):
    """Polynomial::InnerProductFft (crypto/polynomial_fft.cc:68-197)."""
    dt = _cdt(coeff_bits)
    u = np.ascontiguousarray(u, dtype=dt)
    v = np.ascontiguousarray(v, dtype=dt)
    if u.ndim == 1:
        u = u[None]
        v = v[None]
    n, d = u.shape
    out = np.zeros(d, dtype=dt)
    _call(lib().orc_inner_product, coeff_bits, mode, _ptr(u), _ptr(v), n, d,
          u_bits or coeff_bits, v_bits or coeff_bits, chunk_bits,
          int(u_signed), _ptr(out))
    return out


def gadget_inv(p, coeff_bits, log_modulus, log_digit, num_digits,
               signed=False):
    dt = _cdt(coeff_bits)
    p = np.ascontiguousarray(p, dtype=dt)
    out = np.zeros((max(num_digits, 0), p.shape[0]), dtype=dt)
    fn = lib().orc_signed_gadget_inv if signed else lib().orc_gadget_inv
    _call(fn, coeff_bits, _ptr(p), p.shape[0], log_modulus, log_digit,
          num_digits, _ptr(out))
    return out


def rescale(p, coeff_bits, log_cur, log_new):
    dt = _cdt(coeff_bits)
    p = np.ascontiguousarray(p, dtype=dt)
    out = np.zeros_like(p)
    lib().orc_rescale(coeff_bits, _ptr(p), p.shape[0], log_cur, log_new,
                      _ptr(out))
    return out


def automorph(p, coeff_bits, power):
    dt = _cdt(coeff_bits)
    p = np.ascontiguousarray(p, dtype=dt)
    out = np.zeros_like(p)
    _call(lib().orc_automorph, coeff_bits, _ptr(p), p.shape[0], power,
          _ptr(out))
    return out


def preprocess_matrix_pack(a_is, w_vec_g, w_vec_h, coeff_bits, log_modulus,
                           log_digit, num_digits, mode=MODE_EXACT,
                           with_matrix=True):
    """PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:163-446) for one slice.

    Returns a dict: a_tilde_agg (d), t_vec_h (k x d), t_vec_g / t_vec_gh
    ((d/2-1) x k x d digit polynomials) and, with with_matrix, the
    d x (k*d) matrix as centred int64 entries."""
    dt = _cdt(coeff_bits)
    a_is = np.ascontiguousarray(a_is, dtype=dt)
    d = a_is.shape[0]
    k = num_digits
    w_vec_g = np.ascontiguousarray(w_vec_g, dtype=dt).reshape(k, d)
    w_vec_h = np.ascontiguousarray(w_vec_h, dtype=dt).reshape(k, d)
    a_tilde = np.zeros(d, dtype=dt)
    t_h = np.zeros((k, d), dtype=dt)
    t_g = np.zeros((d // 2 - 1, k, d), dtype=dt)
    t_gh = np.zeros((d // 2 - 1, k, d), dtype=dt)
    mat = np.zeros((d, k * d), dtype=np.int64) if with_matrix else None
    _call(lib().orc_preprocess_matrix_pack, coeff_bits, mode, log_modulus,
          log_digit, num_digits, d, _ptr(a_is), _ptr(w_vec_g), _ptr(w_vec_h),
          _ptr(a_tilde), _ptr(mat) if with_matrix else None, _ptr(t_h),
          _ptr(t_g), _ptr(t_gh))
    return {"a_tilde_agg": a_tilde, "t_vec_h": t_h, "t_vec_g": t_g,
            "t_vec_gh": t_gh, "matrix": mat}


def pack(b, y_vec_g, y_vec_h, pre, coeff_bits, log_modulus, log_digit,
         num_digits, mode=MODE_EXACT):
    """Pack (crypto/lwes_to_rlwe.cc:356-412): b_agg by automorphisms."""
    dt = _cdt(coeff_bits)
    b = np.ascontiguousarray(b, dtype=dt)
    d = b.shape[0]
    y_vec_g = np.ascontiguousarray(y_vec_g, dtype=dt)
    y_vec_h = np.ascontiguousarray(y_vec_h, dtype=dt)
    out = np.zeros(d, dtype=dt)
    _call(lib().orc_pack, coeff_bits, mode, log_modulus, log_digit,
          num_digits, d, _ptr(b), _ptr(y_vec_g), _ptr(y_vec_h),
          _ptr(np.ascontiguousarray(pre["t_vec_g"], dtype=dt)),
          _ptr(np.ascontiguousarray(pre["t_vec_gh"], dtype=dt)),
          _ptr(np.ascontiguousarray(pre["t_vec_h"], dtype=dt)), _ptr(out))
    return out


def make_params(**kw):
    p = OrcParams()
    for name, _ in OrcParams._fields_:
        setattr(p, name, int(kw[name]))
    return p


def finalize_matrix_pack(prm, b, b_agg_partial, y_vec_h, t_vec_h,
                         mode=MODE_EXACT):
    dt = _cdt(prm.coeff_bits)
    arrs = [np.ascontiguousarray(x, dtype=dt)
            for x in (b, b_agg_partial, y_vec_h, t_vec_h)]
    out = np.zeros(1 << prm.log_degree, dtype=dt)
    _call(lib().orc_finalize_matrix_pack, ctypes.byref(prm), mode,
          *[_ptr(a) for a in arrs], _ptr(out))
    return out


def external_product(prm, ct_a, ct_b, rgsw, mode=MODE_EXACT):
    dt = _cdt(prm.coeff_bits)
    ct_a = np.ascontiguousarray(ct_a, dtype=dt)
    ct_b = np.ascontiguousarray(ct_b, dtype=dt)
    rgsw = np.ascontiguousarray(rgsw, dtype=dt)
    d = 1 << prm.log_degree
    oa = np.zeros(d, dtype=dt)
    ob = np.zeros(d, dtype=dt)
    _call(lib().orc_external_product, ctypes.byref(prm), mode, _ptr(ct_a),
          _ptr(ct_b), _ptr(rgsw), _ptr(oa), _ptr(ob))
    return oa, ob


def process_response(prm, db, pack, a_tilde_agg, t_vec_h, second_dim_a,
                     first_dim, second_dim, packing_key, mode=MODE_EXACT):
    """PirServer::ProcessResponse (crypto/pir/server/pir_server.cc:154-306).

    db / pack are the combined (vertically concatenated) matrices; the
    polynomial arguments are 2-D arrays of shape (count, d). Returns an array
    of shape (l, 2, d): per shard the rescaled (a, b).
    """
    dt = _cdt(prm.coeff_bits)
    d = 1 << prm.log_degree
    kinds = {np.dtype(v): k for k, v in KIND_DTYPE.items()}
    db = np.ascontiguousarray(db)
    pack = np.ascontiguousarray(pack)
    a_tilde_agg = np.ascontiguousarray(a_tilde_agg, dtype=dt)
    t_vec_h = np.ascontiguousarray(t_vec_h, dtype=dt)
    if second_dim_a is None or np.size(second_dim_a) == 0:
        second_dim_a = np.zeros((0, d), dtype=dt)
    second_dim_a = np.ascontiguousarray(second_dim_a, dtype=dt)
    first_dim = np.ascontiguousarray(first_dim, dtype=dt)
    second_dim = np.ascontiguousarray(second_dim, dtype=dt).reshape(-1, d)
    packing_key = np.ascontiguousarray(packing_key, dtype=dt).reshape(-1, d)
    out = np.zeros((prm.entry_size_multiple, 2, d), dtype=dt)
    _call(lib().orc_process_response, ctypes.byref(prm), mode,
          kinds[db.dtype], _ptr(db), db.shape[1], kinds[pack.dtype],
          _ptr(pack), pack.shape[1], _ptr(a_tilde_agg), _ptr(t_vec_h),
          _ptr(second_dim_a), _ptr(first_dim), first_dim.shape[0],
          _ptr(second_dim), second_dim.shape[0], _ptr(packing_key),
          packing_key.shape[0], _ptr(out))
    return out


def process_response_staged(prm, db, pack, a_tilde_agg, t_vec_h,
                            second_dim_a, first_dim, second_dim, packing_key,
                            mode=MODE_FP64, threads=1, condensed_db=False,
                            library=None):
    """process_response with the reference's stage timers (pir_server.cc:
    214-285). Returns (response, {"db_mult_ms", "packing_ms",
    "poly_eval_ms"}). library: timing_lib() (default) or lib()."""
    dt = _cdt(prm.coeff_bits)
    d = 1 << prm.log_degree
    kinds = {np.dtype(v): k for k, v in KIND_DTYPE.items()}
    db = np.ascontiguousarray(db)
    pack = np.ascontiguousarray(pack)
    a_tilde_agg = np.ascontiguousarray(a_tilde_agg, dtype=dt)
    t_vec_h = np.ascontiguousarray(t_vec_h, dtype=dt)
    if second_dim_a is None or np.size(second_dim_a) == 0:
        second_dim_a = np.zeros((0, d), dtype=dt)
    second_dim_a = np.ascontiguousarray(second_dim_a, dtype=dt)
    first_dim = np.ascontiguousarray(first_dim, dtype=dt)
    second_dim = np.ascontiguousarray(second_dim, dtype=dt).reshape(-1, d)
    packing_key = np.ascontiguousarray(packing_key, dtype=dt).reshape(-1, d)
    out = np.zeros((prm.entry_size_multiple, 2, d), dtype=dt)
    stages = np.zeros(3, dtype=np.float64)
    lb = library or timing_lib()
    _call(lb.orc_process_response_staged, ctypes.byref(prm), mode,
          kinds[db.dtype], _ptr(db), db.shape[1], kinds[pack.dtype],
          _ptr(pack), pack.shape[1], _ptr(a_tilde_agg), _ptr(t_vec_h),
          _ptr(second_dim_a), _ptr(first_dim), first_dim.shape[0],
          _ptr(second_dim), second_dim.shape[0], _ptr(packing_key),
          packing_key.shape[0], _ptr(out), int(threads), int(condensed_db),
          _ptr(stages))
    return out, {"db_mult_ms": float(stages[0]),
                 "packing_ms": float(stages[1]),
                 "poly_eval_ms": float(stages[2])}


def interpolate(db_row, d, t, plaintext_modulus):
    db_row = np.ascontiguousarray(db_row)
    bits = db_row.dtype.itemsize * 8
    out = np.zeros_like(db_row)
    _call(lib().orc_interpolate, bits, _ptr(db_row), d, t, plaintext_modulus,
          _ptr(out))
    return out
