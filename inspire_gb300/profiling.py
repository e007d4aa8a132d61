"""Live kernel timing and roofline arithmetic for the benchmark.

The dominant kernel of an answer is the stage-1 product (DB * q1 + P * y_g):
the fused GEMV for the plain engine, the 8-bit-limb tensor-core GEMM for the
batched engine. It is timed alone here with CUDA events recorded on the
stream it is launched on.

Algorithmic work per request (rows R = l*t*d, DB columns C, pack columns K):
  bytes (plain)  = 2*R*C (u16 DB) + 4*R*K (i32 pack) + 4*(C + K) + 4*R
  limb-ops (tensor, Z_2^32) = 2*(7*R*C + 10*R*K)
    (DB: low byte x 4 query limbs + high byte x 3; pack: 4+3+2+1 byte pairs,
     only pairs whose weight 2^(8(i+j)) is below 2^32 contribute);
  limb-ops (tensor, Z_2^64) = 2*(15*R*C + 26*R*K)
    (8 query limbs: DB 8+7, pack 8+7+6+5 byte pairs below 2^64).
"""
import ctypes
import json
import os

import numpy as np

from . import _lib, pir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def plain_bytes(rows, db_cols, pack_cols, db_elem=2, pack_elem=4, word=4):
    return (rows * db_cols * db_elem + rows * pack_cols * pack_elem +
            (db_cols + pack_cols) * word + rows * word)


def limb_ops(rows, db_cols, pack_cols, batch, coeff_bits=32, log_q=None):
    """Digit products of the exact limb plan: base-256 digit pairs whose
    weight falls below the bits the answer reads (2^32; 2^64, or 2^56 when
    log_q <= 56, over Z_2^64), times 2 R C B (DB) and 2 R K B (pack)."""
    if coeff_bits == 32:
        db_pairs, pk_pairs = 7, 10
    elif log_q is not None and log_q <= 56:
        db_pairs, pk_pairs = 13, 22
    else:
        db_pairs, pk_pairs = 15, 26
    return 2.0 * (db_pairs * rows * db_cols + pk_pairs * rows * pack_cols) * batch


# DRAM traffic per unit of work from one ncu capture of a smaller case of the
# same kernel, scaled by the units a full launch processes (both kernels
# stream their matrices once, so traffic grows in proportion):
#  * limb GEMM, n=2^18 d=2048 t=8 B=256 (ncu --set full, one launch):
#    dram read 2.998676 GB + write 0.113170 GB over R (C + 2K) =
#    16384 * 40960 row-column units;
#  * limb GEMM over Z_2^64, same shape: read 3.490142 GB + write
#    0.163364 GB;
#  * fused GEMV, n=2^18 d=4096 t=8 (ncu --set full, one launch): read
#    3.221 GB + write 2.9 MB against 3.222 GB of algorithmic bytes.
LIMB_TRAFFIC_PER_UNIT = (2.998676e9 + 0.113170e9) / (16384 * 40960)
LIMB64_TRAFFIC_PER_UNIT = (3.490142e9 + 0.163364e9) / (16384 * 40960)
GEMV_TRAFFIC_PER_ALG_BYTE = (3.221e9 + 2.9e6) / 3.222e9


def launches_per_step(engine, t):
    # products: the fused GEMV, or the tensor engine's query-digit split,
    # pack-key digit split and limb GEMM; then NTT(y_h) + finalize
    # + NTT(rgsw) + (t-1) external products + rescale
    products = 3 if engine == pir.ENGINE_TENSOR else 1
    return products + 2 + (1 + (t - 1) if t > 1 else 0) + 1


def kernel_times(srv, engine, batch, t_fd, t_sd, t_pk, t_out, stream, n1,
                 nsd, npk, reps=5):
    import torch
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)
    rows = srv.rows
    dev = t_fd.device
    cb = srv.params.rlwe.coeff_bits
    word = cb // 8
    out = torch.empty((batch, rows),
                      dtype=torch.int32 if cb == 32 else torch.int64, device=dev)
    sptr = stream.cuda_stream

    def run(b, eng):
        rc = lib.inspire_pir_products_device(srv._h, b, t_fd.data_ptr(),
                                             t_pk.data_ptr(), out.data_ptr(),
                                             eng, sptr, err, len(err))
        if rc:
            raise pir.InspireError(rc, err.value.decode())

    def time_it(b, eng):
        for _ in range(2):
            run(b, eng)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run(b, eng)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    hbm, tfl, kind = peaks()
    ms_plain = time_it(1, pir.ENGINE_PLAIN)
    pb = plain_bytes(rows, srv.db_cols, srv.pack_cols, word=word)
    plain_gbs = pb / (ms_plain / 1e3) / 1e9
    kernels = {"fused_gemv_b1": {"ms": ms_plain, "bytes": pb,
                                 "gbs": plain_gbs,
                                 "frac_hbm": plain_gbs / hbm}}
    if engine == pir.ENGINE_TENSOR:
        ms_t = time_it(batch, engine)
        ops = limb_ops(rows, srv.db_cols, srv.pack_cols, batch, cb,
                       srv.params.rlwe.log_modulus)
        ach = ops / (ms_t / 1e3) / 1e12
        kernels["limb_gemm_b%d" % batch] = {"ms": ms_t, "limb_ops": ops,
                                            "tflops": ach,
                                            "frac_tensor": ach / tfl}
        units = rows * (srv.db_cols + 2 * srv.pack_cols)
        per_unit = LIMB_TRAFFIC_PER_UNIT if cb == 32 else LIMB64_TRAFFIC_PER_UNIT
        roof = {"bound": "tensor", "achieved": ach, "peak": tfl,
                "unit": "TFLOP/s", "frac": ach / tfl,
                "traffic": per_unit * units,
                "traffic_source": "ncu small case scaled by R*(C+2K)",
                "kernel": "limb_gemm", "peak_kind": kind + " bf16 dense"}
    else:
        roof = {"bound": "hbm", "achieved": plain_gbs, "peak": hbm,
                "unit": "GB/s", "frac": plain_gbs / hbm,
                "traffic": GEMV_TRAFFIC_PER_ALG_BYTE * pb,
                "traffic_source": "ncu small case scaled by algorithmic bytes",
                "kernel": "fused_gemv", "peak_kind": kind + " copy"}
    return {"roofline": roof, "kernels": kernels,
            "launches_per_step": launches_per_step(engine,
                                                   srv.params.interpolation_degree)}
