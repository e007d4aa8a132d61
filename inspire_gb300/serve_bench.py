"""Serving benchmark: continuous batching over several device-resident DBs.

Workload (two databases, uniform random plaintext from a seed):
  * DB A: n = 262144 records, ring degree d = 8192, interpolation degree
    t = 2, entry_size_multiple l in {1, 2, 4} (three servers, one per l:
    DB matrices 16384*l x 131072 u16);
  * DB B: n = 2^20, d = 4096, t = 8, l = 1 (32768 x 131072 u16).
Each query goes to DB A or DB B with equal probability (l uniform for A) and
to a uniformly random record (a seeded request from a pool per server).
Queries arrive open-loop with exponential inter-arrival times (Poisson) at
fractions of the measured peak rate. The peak is measured closed-loop: each
server answers full batches back to back, and the peak of the mix is the
weighted harmonic mean of the per-server rates.

Every served response is compared with the answer to the same request
computed alone (one synchronous call per request): the responses must be
bit-identical. The reference answers one request per ProcessResponse call
(crypto/pir/server/pir_server.cc:154-306) and has no serving loop; the
metric is p50/p99 latency and achieved queries/s at each load.

Run: python -m inspire_gb300.serve_bench [--seconds S] [--loads 0.1,0.5,1]
"""
import argparse
import json
import math
import threading
import time

import numpy as np

from . import build, pir, serving, synthetic

SERVERS = (  # name, n, d, t, l, share of the traffic
    ("A_l1", 262144, 8192, 2, 1, 1.0 / 6),
    ("A_l2", 262144, 8192, 2, 2, 1.0 / 6),
    ("A_l4", 262144, 8192, 2, 4, 1.0 / 6),
    ("B", 1 << 20, 4096, 8, 1, 0.5),
)


def make_server(n, d, t, l, seed):
    """A PirServer over seeded uniform material of the given shape."""
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=32)
    rows, cols = l * t * d, n // t
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, seed)
    k = params.pack_gadget.num_digits
    bound = int(4 * math.sqrt(d) * (1 << params.pack_gadget.log_digit))
    pack = synthetic.parallel_integers((rows, k * d), -bound + 1, bound,
                                       np.int32, seed + 1)
    small = synthetic.make_material(
        synthetic.make_params(d=d, n=d * t, t=t, l=l, coeff_bits=32),
        seed=seed + 2)
    srv = pir.PirServer.CreateCombined(params, db, pack, small.a_tilde_agg,
                                       small.t_vec_h, small.second_dim_a)
    return params, srv


def closed_loop_rate(srv, fd, sd, pk, batch, reps=3):
    """Queries/s of back-to-back full batches through the host-buffer call."""
    b = min(batch, fd.shape[0])
    idx = np.arange(batch) % fd.shape[0]
    f, s, p = fd[idx][:b], sd[idx][:b], pk[idx][:b]
    srv.process_arrays(f, s, p, pir.ENGINE_TENSOR)
    t0 = time.perf_counter()
    for _ in range(reps):
        srv.process_arrays(f, s, p, pir.ENGINE_TENSOR)
    return reps * b / (time.perf_counter() - t0)


def run_load(eng, pools, names, weights, rate, seconds, rng):
    """Open-loop Poisson arrivals at `rate` queries/s for `seconds`."""
    n = max(50, int(rate * seconds))
    gaps = rng.exponential(1.0 / rate, size=n)
    which = rng.choice(len(names), size=n, p=weights)
    picks = [int(rng.integers(0, pools[names[w]][0].shape[0])) for w in which]
    futs = []
    t_start = time.perf_counter()
    t_next = t_start
    for i in range(n):
        t_next += gaps[i]
        while True:
            now = time.perf_counter()
            if now >= t_next:
                break
            if t_next - now > 2e-4:
                time.sleep(min(t_next - now - 1e-4, 0.01))
        fd, sd, pk, _ = pools[names[which[i]]]
        j = picks[i]
        futs.append((names[which[i]], j, eng.submit(names[which[i]], fd[j],
                                                   sd[j], pk[j])))
    t_sub = time.perf_counter() - t_start
    results = [(name, j, f.result(timeout=300)) for name, j, f in futs]
    t_all = time.perf_counter() - t_start
    return n, t_sub, t_all, results


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=3.0)
    ap.add_argument("--loads", default="0.1,0.25,0.5,0.75,1.0,1.5",
                    help="offered loads as fractions of the closed-loop peak; "
                         "above 1 the loop saturates")
    ap.add_argument("--pool", type=int, default=64)
    ap.add_argument("--max-batch", type=int, default=256)
    ap.add_argument("--hbm-budget-gb", type=float, default=48.0)
    ap.add_argument("--max-workspaces", type=int, default=1,
                    help="batches in flight per server at most")
    ap.add_argument("--max-wait-us", type=int, default=0,
                    help="batching window of the serving loop")
    ap.add_argument("--plain-max-batch", type=int, default=None,
                    help="largest batch answered by the plain engine "
                         "(default: each server's tuned crossover)")
    ap.add_argument("--small", action="store_true",
                    help="shrunk shapes (n / 16) for a quick functional run")
    args = ap.parse_args(argv)
    build.build()

    servers, pools = {}, {}
    names, weights = [], []
    for i, (name, n, d, t, l, w) in enumerate(SERVERS):
        if args.small:
            n //= 16
        params, srv = make_server(n, d, t, l, seed=1000 + 10 * i)
        srv.autotune(args.max_batch)
        fd, sd, pk = synthetic.make_requests(params, args.pool, seed=2000 + i)
        alone = np.stack([srv.process_arrays(fd[j:j + 1], sd[j:j + 1],
                                             pk[j:j + 1])[0]
                          for j in range(args.pool)])
        servers[name] = srv
        pools[name] = (fd, sd, pk, alone)
        names.append(name)
        weights.append(w)
    weights = np.array(weights) / sum(weights)

    per_rate = {name: closed_loop_rate(servers[name], *pools[name][:3],
                                       args.max_batch) for name in names}
    peak = 1.0 / sum(w / per_rate[nm] for nm, w in zip(names, weights))

    rng = np.random.default_rng(7)
    loads = []
    with serving.ServingEngine(servers, max_batch=args.max_batch,
                               hbm_budget=int(args.hbm_budget_gb * (1 << 30)),
                               max_workspaces=args.max_workspaces,
                               plain_max_batch=args.plain_max_batch,
                               max_wait_us=args.max_wait_us) as eng:
        for frac in [float(x) for x in args.loads.split(",")]:
            eng.reset_stats()
            n, t_sub, t_all, results = run_load(
                eng, pools, names, weights, frac * peak, args.seconds, rng)
            mismatches = sum(
                0 if np.array_equal(r, pools[name][3][j]) else 1
                for name, j, r in results)
            st = eng.stats()
            loads.append({
                "load": frac, "offered_qps": frac * peak,
                "achieved_qps": n / t_all, "requests": n,
                "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                "mean_batch": st["mean_batch"],
                "max_inflight": st["max_inflight"],
                "batches": st["batches"],
                "tensor_batches": st["tensor_batches"],
                "submit_s": t_sub,
                "mismatches": mismatches})
        ws = {nm: eng.queue_info(nm) for nm in names}
        crossovers = dict(eng.crossovers)
    line = {
        "metric": "serving p50/p99 latency and queries/s, open-loop Poisson "
                  "arrivals over two device-resident DBs, bit-exact",
        "unit": "queries/s",
        "config": {"workload": "serve_A_n262144_d8192_t2_l124_B_n2^20_d4096_t8"
                               + ("_small" if args.small else ""),
                   "servers": [dict(zip(("name", "n", "d", "t", "l", "share"),
                                        s)) for s in SERVERS],
                   "max_batch": args.max_batch,
                   "max_wait_us": args.max_wait_us,
                   "plain_max_batch": args.plain_max_batch,
                   "tuned_crossovers": crossovers,
                   "hbm_budget_gb": args.hbm_budget_gb,
                   "max_workspaces": args.max_workspaces,
                   "workspaces": ws},
        "peak_qps": peak,
        "per_server_peak_qps": per_rate,
        "loads": loads,
        "bit_exact": all(x["mismatches"] == 0 for x in loads),
        "data": "synthetic (seeded uniform DBs, pack matrices, requests)",
    }
    print(json.dumps(line))
    return line


if __name__ == "__main__":
    main()
