"""Runs one sized PIR answer workload for profiling (ncu captures).

  python -m inspire_gb300.profile_case --n 262144 --d 4096 --t 8 \
      --engine plain --batch 1 --reps 3 [--stage products|answer]
      [--form planes|raw|planes-narrow|raw-narrow --split K]

The server material is seeded synthetic data of the given shape; the chosen
stage runs `reps` times on one stream and the process exits 0 on success.
"""
import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 18)
    ap.add_argument("--d", type=int, default=4096)
    ap.add_argument("--t", type=int, default=8)
    ap.add_argument("--coeff-bits", type=int, default=32)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--engine", default="plain", choices=["plain", "tensor"])
    ap.add_argument("--stage", default="products",
                    choices=["products", "answer"])
    ap.add_argument("--form", default="tuned",
                    choices=["tuned", "planes", "raw", "planes-narrow",
                             "raw-narrow"],
                    help="tensor engine products: the DB form and request "
                         "tile (tuned: the engine's own choice)")
    ap.add_argument("--split", type=int, default=0,
                    help="split-K factor of a forced form (0: heuristic)")
    args = ap.parse_args()

    import ctypes

    import torch

    from inspire_gb300 import _lib, build, pir, synthetic
    build.build()
    params = synthetic.make_params(d=args.d, n=args.n, t=args.t,
                                   coeff_bits=args.coeff_bits)
    rows = args.t * args.d
    cols = args.n // args.t
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, 5)
    k = params.pack_gadget.num_digits
    bound = int(4 * np.sqrt(args.d) * (1 << params.pack_gadget.log_digit))
    pack = synthetic.parallel_integers((rows, k * args.d), -bound + 1, bound,
                                       np.int32, 6)
    mat = synthetic.make_material(
        synthetic.make_params(d=args.d, n=args.d * args.t, t=args.t,
                              coeff_bits=args.coeff_bits), seed=7)
    srv = pir.PirServer.CreateCombined(params, db, pack, mat.a_tilde_agg,
                                       mat.t_vec_h, mat.second_dim_a)
    fd, sd, pk = synthetic.make_requests(params, args.batch, seed=8)
    dev = torch.device("cuda", 0)
    view = np.int32 if args.coeff_bits == 32 else np.int64
    t_fd = torch.from_numpy(fd.view(view)).to(dev)
    t_sd = torch.from_numpy(sd.view(view)).to(dev)
    t_pk = torch.from_numpy(pk.view(view)).to(dev)
    t_out = torch.empty((args.batch, max(rows, 2 * args.d)), dtype=torch.int64,
                        device=dev)
    stream = torch.cuda.Stream(device=dev)
    eng = pir.ENGINE_TENSOR if args.engine == "tensor" else pir.ENGINE_PLAIN
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)
    t0 = time.perf_counter()
    for _ in range(args.reps):
        if args.stage == "products" and args.engine == "tensor" and \
                args.form != "tuned":
            form = {"planes": pir.FORM_PLANES, "raw": pir.FORM_RAW,
                    "planes-narrow": pir.FORM_PLANES | pir.FORM_NARROW,
                    "raw-narrow": pir.FORM_RAW | pir.FORM_NARROW}[args.form]
            srv.tensor_products_device(args.batch, t_fd.data_ptr(),
                                       t_pk.data_ptr(), t_out.data_ptr(), form,
                                       args.split, stream.cuda_stream)
        elif args.stage == "products":
            rc = lib.inspire_pir_products_device(
                srv._h, args.batch, t_fd.data_ptr(), t_pk.data_ptr(),
                t_out.data_ptr(), eng, stream.cuda_stream, err, len(err))
            if rc:
                raise SystemExit(err.value.decode())
        else:
            srv.process_device(args.batch, t_fd.data_ptr(), fd.shape[1],
                               t_sd.data_ptr(), sd.shape[1], t_pk.data_ptr(),
                               pk.shape[1], t_out.data_ptr(), eng,
                               stream.cuda_stream)
    stream.synchronize()
    print("profile_case: %d x %s/%s n=%d d=%d t=%d batch=%d in %.3f s" % (
        args.reps, args.stage, args.engine, args.n, args.d, args.t,
        args.batch, time.perf_counter() - t0))


if __name__ == "__main__":
    main()
