"""Benchmark of the ReinsPIRe online answer on GB300.

Workload: n = 2^20 records, ring degree d = 4096, entry_size_multiple l = 1,
interpolation degree t = 8, CoeffType u32 (q = 2^32): the DB matrix is
t*d x n/t = 32768 x 131072 u16 (8 GiB), the packing matrix 32768 x 8192 i32
(1 GiB). A step answers one batch of B seeded requests (default B = 256) with
the batched tensor-core engine (8-bit limbs on tcgen05); the plain
single-query engine (fused CUDA-core GEMV) is timed beside it. Every response
of both engines is the same integer vector (checked before timing).

Prints one JSON line (rank 0). `value` is queries/s with the requests already
resident in GPU memory; `e2e` is the same metric through the host-buffer C ABI
call (H2D of the requests and D2H of the responses inside the timed region).
`--impl reference` times the reference algorithm's CPU restatement (the
oracle, FP64 FFT path) on all host cores instead.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_ENTRIES = 1 << 20
DEGREE = 4096
INTERP = 8
COEFF_BITS = 32   # --coeff-bits 64 answers over Z_2^64 with q = 2^56
LOG_Q = 32


def word_tag():
    return "u%d" % COEFF_BITS


def ring_tag():
    return "Z_2^32" if COEFF_BITS == 32 else "Z_2^64, q=2^%d" % LOG_Q


def metric_name():
    """The headline metric, printed identically by both arms."""
    return "queries/s (online answer, n=2^20 d=4096 t=8, %s)" % ring_tag()


def workload_name():
    return "pir_answer_n2^20_d4096_t8_l1_" + word_tag() + \
        ("" if COEFF_BITS == 32 else "_q2^%d" % LOG_Q)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region
    (one nvidia-smi process in its own loop mode, a sample every 25 ms)."""
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, interval_ms=25):
        self.index = index
        self.interval_ms = interval_ms
        self.samples = []
        self._proc = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            # nvidia-smi prints its first sample once it has attached.
            time.sleep(0.3)
        except OSError:
            self._proc = None
        return self

    def __exit__(self, *a):
        if self._proc is None:
            return
        time.sleep(2 * self.interval_ms / 1000.0)
        self._proc.terminate()
        try:
            out, _ = self._proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self._proc.kill()
            out, _ = self._proc.communicate()
        for ln in out.splitlines():
            if ln.strip():
                self.samples.append([x.strip() for x in ln.split(",")])

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def replica_time(ms, dist, device):
    """The job's time for a step: the slowest replica's (max over ranks).
    Replicas share nothing on the data path; this is the only collective."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def make_workload(seed=2026, batch=256):
    from inspire_gb300 import synthetic
    params = synthetic.make_params(d=DEGREE, n=N_ENTRIES, t=INTERP,
                                   coeff_bits=COEFF_BITS, log_q=LOG_Q)
    rows = INTERP * DEGREE
    cols = N_ENTRIES // INTERP
    # Uniform already-interpolated DB values in [0, p) (p = 65535).
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, seed)
    k = params.pack_gadget.num_digits
    bound = int(4 * np.sqrt(DEGREE) * (1 << params.pack_gadget.log_digit))
    pack = synthetic.parallel_integers((rows, k * DEGREE), -bound + 1, bound,
                                       np.int32, seed + 7)
    mat = synthetic.make_material(
        synthetic.make_params(d=DEGREE, n=DEGREE * INTERP, t=INTERP,
                              coeff_bits=COEFF_BITS, log_q=LOG_Q), seed=seed + 1)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=seed + 2)
    return params, db, pack, mat.a_tilde_agg, mat.t_vec_h, mat.second_dim_a, \
        fd, sd, pk


def cpu_reference_profile(params, db, pack, a_tilde, t_vec_h, sda, fd, sd,
                          pk, reps=2):
    """The reference algorithm (the oracle's timing build, FP64 FFT path) on
    one host core, one request at a time as the single-threaded reference
    runs it: mean latency and the reference's stage split (DB mult, packing,
    poly-eval; pir_server.cc:214-285, printed by pir_metrics_tool.cc:435-447).
    """
    from oracle import pyoracle as orc
    op = oracle_params(params)
    condensed = params.rlwe.coeff_bits == 64
    lat, stages = [], []
    for i in range(reps):
        t0 = time.perf_counter()
        _, st = orc.process_response_staged(
            op, db, pack, a_tilde, t_vec_h, sda, fd[i % fd.shape[0]],
            sd[i % fd.shape[0]], pk[i % fd.shape[0]], mode=orc.MODE_FP64,
            threads=1, condensed_db=condensed)
        lat.append((time.perf_counter() - t0) * 1000.0)
        stages.append(st)
    mean = {k: statistics.mean(s[k] for s in stages) for k in stages[0]}
    return {"single_core_ms": statistics.mean(lat),
            "stages_ms": mean,
            "build": orc.timing_build_string(),
            "db_product": "condensed u64 words (matrix.cc:261-318)"
                          if condensed else
                          "scalar u32 loop (matrix.h:183-194; the reference "
                          "condenses the DB only for u64 CoeffType, "
                          "preprocessing_server.h:127-153)"}


def cpu_reference_throughput(params, db, pack, a_tilde, t_vec_h, sda, fd, sd,
                             pk, threads, requests):
    """`requests` full requests, one per host thread at a time on `threads`
    threads (the reference has no threads of its own: independent requests
    per core). Returns (seconds, requests done)."""
    from oracle import pyoracle as orc
    op = oracle_params(params)
    condensed = params.rlwe.coeff_bits == 64
    nxt = [0]
    lock = threading.Lock()

    def work():
        while True:
            with lock:
                i = nxt[0]
                if i >= requests:
                    return
                nxt[0] += 1
            j = i % fd.shape[0]
            orc.process_response_staged(op, db, pack, a_tilde, t_vec_h, sda,
                                        fd[j], sd[j], pk[j],
                                        mode=orc.MODE_FP64, threads=1,
                                        condensed_db=condensed)
    ts = [threading.Thread(target=work) for _ in range(threads)]
    t0 = time.perf_counter()
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return time.perf_counter() - t0, requests


def run_reference(args):
    """The reference algorithm (the oracle's timing build, FP64 FFT path) on
    all host cores: each step answers one request per host thread."""
    threads = os.cpu_count() or 1
    params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk = make_workload(
        batch=max(64, threads))
    prof = cpu_reference_profile(params, db, pack, a_tilde, t_vec_h, sda, fd,
                                 sd, pk, reps=2)

    def one_step():
        return cpu_reference_throughput(params, db, pack, a_tilde, t_vec_h,
                                        sda, fd, sd, pk, threads, threads)[0]

    for _ in range(args.warmup):
        one_step()
    times = [one_step() for _ in range(args.steps)]
    total = sum(times)
    qps = threads * args.steps / total
    line = {
        "impl": "reference",
        "metric": metric_name(),
        "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": word_tag(),
        "data": "synthetic (seeded uniform DB, pack matrix, queries)",
        "config": {"workload": workload_name(),
                   "n": N_ENTRIES, "d": DEGREE, "t": INTERP, "l": 1,
                   "requests_per_step": threads},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads,
                         "kind": "port",
                         "sample": "%d full requests per step, one per host "
                                   "thread (oracle timing build, FP64 FFT "
                                   "path)" % threads,
                         "single_core_ms": prof["single_core_ms"],
                         "stages_ms": prof["stages_ms"],
                         "build": prof["build"],
                         "db_product": prof["db_product"]},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def oracle_params(params):
    from oracle import pyoracle as orc
    r = params.rlwe
    return orc.make_params(
        coeff_bits=r.coeff_bits, log_degree=r.degree.bit_length() - 1,
        log_modulus=r.log_modulus,
        log_modulus1_after_switch=r.log_modulus1_after_switch,
        log_modulus2_after_switch=r.log_modulus2_after_switch,
        pack_log_digit=params.pack_gadget.log_digit,
        pack_num_digits=params.pack_gadget.num_digits,
        eval_log_digit=params.eval_gadget.log_digit,
        eval_num_digits=params.eval_gadget.num_digits,
        num_entries=params.num_entries,
        interpolation_degree=params.interpolation_degree,
        entry_size_multiple=params.entry_size_multiple)


def oracle_check(params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk, got,
                 picks):
    """Compares responses `picks` of `got` (B, l, 2, d) with the oracle's
    exact-product answer on the same bytes, one host thread per response."""
    from oracle import pyoracle as orc
    op = oracle_params(params)
    bad = []
    errs = []

    def one(i):
        try:
            want = orc.process_response(op, db, pack, a_tilde, t_vec_h, sda,
                                        fd[i], sd[i], pk[i],
                                        mode=orc.MODE_EXACT)
            if not np.array_equal(got[i].reshape(want.shape), want):
                bad.append(i)
        except Exception as e:  # reported below, never swallowed
            errs.append("%d: %s" % (i, e))
    t0 = time.perf_counter()
    ts = [threading.Thread(target=one, args=(i,)) for i in picks]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if errs:
        raise SystemExit("oracle check failed: %s" % "; ".join(errs))
    return {"responses": list(picks), "mismatches": sorted(bad),
            "oracle": "exact-product oracle (ORC_MODE_EXACT)",
            "seconds": round(time.perf_counter() - t0, 2)}


def cpu_baseline_sample(params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk,
                        budget_s=20.0):
    """The reference algorithm on the host cores, bounded: two requests on
    one core (latency and stage split), then one request per host thread
    for the rest of the budget."""
    prof = cpu_reference_profile(params, db, pack, a_tilde, t_vec_h, sda, fd,
                                 sd, pk, reps=2)
    threads = os.cpu_count() or 1
    left = budget_s - 2 * prof["single_core_ms"] / 1000.0
    per_req = prof["single_core_ms"] / 1000.0
    requests = max(threads, int(threads * max(left, per_req) / (2 * per_req)))
    requests = (requests + threads - 1) // threads * threads
    el, done = cpu_reference_throughput(params, db, pack, a_tilde, t_vec_h,
                                        sda, fd, sd, pk, threads, requests)
    return {"value": done / el, "unit": "queries/s", "cores": threads,
            "kind": "port",
            "sample": "%d full requests in %.1f s, one per host thread on %d "
                      "threads (oracle timing build, FP64 FFT path)"
                      % (done, el, threads),
            "single_core_ms": prof["single_core_ms"],
            "stages_ms": prof["stages_ms"], "build": prof["build"],
            "db_product": prof["db_product"]}


def run_pack_workload(args):
    """The packing micro-workload: 256 instances of packing d = 2048 LWE
    ciphertexts into one RLWE ciphertext (t = 1: DB and pack products, then
    FinalizeMatrixPack; pir_packing_metrics_tool.cc:226-283) followed by one
    ExternalProduct (eval gadget 19 x 3) of each packed ciphertext with its
    own RGSW ciphertext, replayed as one CUDA graph per step."""
    import torch
    from inspire_gb300 import build, pir, synthetic
    build.build()
    d, B = 2048, args.batch
    params = synthetic.make_params(d=d, n=2048, t=1, coeff_bits=COEFF_BITS)
    mat = synthetic.make_material(params, seed=31)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    fd, _, pk = synthetic.make_requests(params, B, seed=32)
    ne = params.eval_gadget.num_digits
    rgsw = synthetic.parallel_integers((B, 2 * ne, 2, d), 0, 1 << 32,
                                       np.uint64, 33).astype(np.uint32)
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(np.int32)).to(dev)
    t_pk = torch.from_numpy(pk.view(np.int32)).to(dev)
    t_rg = torch.from_numpy(rgsw.view(np.int32)).to(dev)
    packed = torch.zeros((B, 1, 2, d), dtype=torch.int32, device=dev)
    ext = torch.zeros((B, 2, d), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    engine = pir.ENGINE_TENSOR

    def step(eng):
        srv.pack_device(B, t_fd.data_ptr(), fd.shape[1], t_pk.data_ptr(),
                        pk.shape[1], packed.data_ptr(), eng, sp)
        srv.external_product_device(B, packed.data_ptr(), t_rg.data_ptr(),
                                    ext.data_ptr(), sp)
    try:
        step(engine)
    except pir.InspireError:
        engine = pir.ENGINE_PLAIN
        step(engine)
    stream.synchronize()
    ref = ext.clone()
    step(pir.ENGINE_PLAIN)
    stream.synchronize()
    if not torch.equal(ref, ext):
        raise SystemExit("engine outputs differ")
    step(engine)
    stream.synchronize()
    with pir.Graph(sp) as g:
        step(engine)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / args.steps
    with ClockSampler(0) as clk:
        ms_graph = timed(lambda: g.launch(sp))
    ms_eager = timed(lambda: step(engine))
    srv.check()
    line = {
        "metric": "packed RLWE ciphertexts/s (d=2048 LWEs -> 1 RLWE, "
                  "pack 19x2, + ExternalProduct 19x3), bit-exact",
        "value": B / (ms_graph / 1000.0), "unit": "instances/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded uniform pack matrix, keys, RGSW)",
        "config": {"workload": "pack_d2048_b%d_graph" % B, "d": d,
                   "instances": B, "engine": "tensor" if engine else "plain",
                   "l2": "working set fits L2 (40 MiB of matrices)"},
        "eager_ms_per_step": ms_eager,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def run_interpolate_workload(args):
    """Offline DB interpolation + transposition (PreprocessingServer's
    InterpolateAndTranspose) of an n = 2^20, d = 4096, t = 8, l = 1 u16 DB
    (8 GiB in, 8 GiB out), device-resident, against the HBM roofline."""
    import torch
    from inspire_gb300 import _lib, build, pir, synthetic
    build.build()
    n, d, t, l, p = args.entries, DEGREE, INTERP, 1, 65535
    raw = synthetic.parallel_integers((n * l * d,), 0, p, np.uint16, 41)
    dev = torch.device("cuda", 0)
    t_raw = torch.from_numpy(raw.view(np.int16)).to(dev)
    t_out = torch.empty((l * t * d, n // t), dtype=torch.int16, device=dev)
    stream = torch.cuda.Stream(device=dev)
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)

    def step():
        rc = lib.inspire_interpolate_db(
            16, ctypes.c_void_p(t_raw.data_ptr()), raw.size, n, d, t, l, p,
            ctypes.c_void_p(t_out.data_ptr()), n // t, 1,
            ctypes.c_void_p(stream.cuda_stream), err, len(err))
        if rc:
            raise SystemExit(err.value)
    for _ in range(args.warmup):
        step()
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    moved = 2 * raw.nbytes
    hbm, _, peak_kind = peaks()
    gbs = moved / (ms / 1000.0) / 1e9

    # Bit-exact check of the timed output: the first, middle and last DB
    # columns (one group of t records each) against the oracle's Interpolate.
    from oracle import pyoracle as orc
    groups = raw.reshape(n // t, t * d)
    picks = sorted({0, (n // t) // 2, n // t - 1})
    t0 = time.perf_counter()
    bad = [i for i in picks
           if not np.array_equal(t_out[:, i].cpu().numpy().view(np.uint16),
                                 orc.interpolate(groups[i], d, t, p))]
    if bad:
        raise SystemExit("interpolated DB columns %s differ from the oracle"
                         % bad)
    ocheck = {"columns": picks, "mismatches": bad,
              "oracle": "Interpolate restated on the host",
              "seconds": round(time.perf_counter() - t0, 2)}
    n_txt = ("2^%d" % (n.bit_length() - 1)) if n & (n - 1) == 0 else str(n)
    line = {
        "metric": "DB interpolation + transposition GB/s (n=%s, d=%d, "
                  "t=%d, u16 records), bit-exact" % (n_txt, d, t),
        "value": gbs, "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u16",
        "data": "synthetic (seeded uniform records in [0, p))",
        "config": {"workload": "interpolate_n%d_d%d_t%d_l1_u16" % (n, d, t),
                   "records_per_s": n / (ms / 1000.0),
                   "l2": "inputs larger than L2 (%.0f GiB)"
                         % (raw.nbytes / 2**30)},
        "oracle_check": ocheck,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm,
                     "unit": "GB/s", "frac": gbs / hbm, "traffic": None,
                     "peak_kind": peak_kind},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        from oracle import pyoracle as orc
        groups = raw.reshape(n // t, t * d)
        threads = os.cpu_count() or 1
        done = [0]
        lock = threading.Lock()
        deadline = time.perf_counter() + 10.0

        def work(i):
            j = i
            while time.perf_counter() < deadline:
                orc.interpolate(groups[j % groups.shape[0]], d, t, p)
                with lock:
                    done[0] += 1
                j += threads
        t0 = time.perf_counter()
        ts = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
        for th in ts:
            th.start()
        for th in ts:
            th.join()
        el = time.perf_counter() - t0
        cpu_gbs = done[0] * t * d * 2 * 2 / el / 1e9
        line["cpu_baseline"] = {
            "value": cpu_gbs, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "%d groups of t records in %.1f s on %d host threads "
                      "(oracle Interpolate, transposition not included)"
                      % (done[0], el, threads)}
    print(json.dumps(line))


def run_hint_workload(args):
    """Offline hint matrix (ComputeHintMatrix) of the n = 2^20, d = 4096,
    t = 8 DB: 32768 x 131072 u16 entries against 32 a-components of 4096
    u32 coefficients -> 32768 x 4096 u32, device-resident."""
    import torch
    from inspire_gb300 import _lib, build, synthetic
    build.build()
    rows, d = INTERP * DEGREE, DEGREE
    cols = args.entries // INTERP
    n = cols // d
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, 51)
    a = synthetic.parallel_integers((n, d), 0, 1 << 32, np.uint64, 52).astype(np.uint32)
    dev = torch.device("cuda", 0)
    t_db = torch.from_numpy(db.view(np.int16)).to(dev)
    t_a = torch.from_numpy(a.view(np.int32)).to(dev)
    t_out = torch.empty((rows, d), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)

    def step():
        rc = lib.inspire_compute_hint_matrix(
            1, 32, ctypes.c_void_p(t_db.data_ptr()), rows, cols,
            ctypes.c_void_p(t_a.data_ptr()), n, d,
            ctypes.c_void_p(t_out.data_ptr()), 1,
            ctypes.c_void_p(stream.cuda_stream), err, len(err))
        if rc:
            raise SystemExit(err.value)
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            step()
    ms = (time.perf_counter() - t0) * 1000 / args.steps

    # Exact check of the timed output: the first, middle and last hint rows
    # against the oracle's exact negacyclic inner product of the DB row's n
    # polynomials with the reversed-negated a-components.
    from oracle import pyoracle as orc
    vinv = np.concatenate([a[:, :1], (0 - a[:, :0:-1].astype(np.uint64))
                           .astype(np.uint32)], axis=1)
    chunk = min(20, int((53.0 - np.log2(n) - np.log2(d)) / 2.0))
    picks = sorted({0, rows // 2, rows - 1})
    t0 = time.perf_counter()
    bad = [i for i in picks
           if not np.array_equal(
               t_out[i].cpu().numpy().view(np.uint32),
               orc.inner_product(db[i].reshape(n, d).astype(np.uint32), vinv,
                                 32, 16, 32, chunk))]
    if bad:
        raise SystemExit("hint rows %s differ from the oracle" % bad)
    ocheck = {"rows": picks, "mismatches": bad,
              "oracle": "exact inner product restated on the host",
              "seconds": round(time.perf_counter() - t0, 2)}
    line = {
        "metric": "hint matrix rows/s (ComputeHintMatrix, %d x %d u16 DB, "
                  "%d a-components, d=%d, Z_2^32), exact" % (rows, cols, n, d),
        "value": rows / (ms / 1000.0), "unit": "rows/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded uniform DB and "
                                "a-components)",
        "config": {"workload": "hint_n%d_d4096_t8_u32" % args.entries,
                   "rows": rows,
                   "cols": cols, "a_components": n,
                   "ntts_per_step": rows * (n + 1) * 3,
                   "timing": "host clock around synchronous calls"},
        "oracle_check": ocheck,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        done = 0
        while time.perf_counter() - t0 < 10.0:
            orc.inner_product(db[done].reshape(n, d).astype(np.uint32), vinv,
                              32, 16, 32, chunk)
            done += 1
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": done / el, "unit": "rows/s", "cores": 1, "kind": "port",
            "sample": "%d rows in %.1f s on one host thread (oracle exact "
                      "inner product per row)" % (done, el)}
    print(json.dumps(line))


def run_preprocess_workload(args):
    """Offline PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:163-446, per
    slice as PreprocessingServer calls it, preprocessing_server.h:248-271)
    for the n = 2^20, d = 4096, t = 8 packing material: 8 slices of d LWE
    a-vectors (the hint rows) against a k = 2 pack key -> a_tilde_agg, the
    32768 x 8192 int32 pack matrix and t_vec_h. `value`: the device-pointer
    call (inputs and outputs in HBM; its scratch allocations included),
    CUDA events; `e2e`: the host-buffer call (hint in, matrix out).
    Exactness is checked against the oracle by the tests at d = 64 / 256 /
    2048 and by decryption at 4096; here the timing only."""
    import torch
    from inspire_gb300 import _lib, build, pir
    build.build()
    d, slices, k, log_q, log_digit = DEGREE, INTERP, 2, 32, 19
    rng = np.random.default_rng(61)
    hint = rng.integers(0, 1 << 32, size=(slices * d, d), dtype=np.uint64
                        ).astype(np.uint32)
    pack_a = rng.integers(0, 1 << 32, size=(2 * k, d), dtype=np.uint64
                          ).astype(np.uint32)
    dev = torch.device("cuda", 0)
    t_hint = torch.from_numpy(hint.view(np.int32)).to(dev)
    t_pa = torch.from_numpy(pack_a.view(np.int32)).to(dev)
    t_a = torch.empty((slices, d), dtype=torch.int32, device=dev)
    t_m = torch.empty((slices * d, k * d), dtype=torch.int32, device=dev)
    t_th = torch.empty((slices, k, d), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    lib = _lib.load()
    err = ctypes.create_string_buffer(256)

    def step():
        rc = lib.inspire_preprocess_matrix_pack(
            32, 5, log_q, log_digit, k, d, slices,
            ctypes.c_void_p(t_hint.data_ptr()), d,
            ctypes.c_void_p(t_pa.data_ptr()), 2 * k,
            ctypes.c_void_p(t_a.data_ptr()), ctypes.c_void_p(t_m.data_ptr()),
            ctypes.c_void_p(t_th.data_ptr()), 1,
            ctypes.c_void_p(stream.cuda_stream), err, len(err))
        if rc:
            raise SystemExit(err.value)
    for _ in range(args.warmup):
        step()
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # The same through the host-buffer call.
    pir.PreprocessMatrixPack(hint, pack_a, log_q, log_digit, k,
                             mat_dtype=np.int32)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a_h, m_h, th_h = pir.PreprocessMatrixPack(hint, pack_a, log_q,
                                                  log_digit, k,
                                                  mat_dtype=np.int32)
    ms_e2e = (time.perf_counter() - t0) * 1000 / args.steps
    same = (np.array_equal(a_h, t_a.cpu().numpy().view(np.uint32)) and
            np.array_equal(m_h, t_m.cpu().numpy()) and
            np.array_equal(th_h, t_th.cpu().numpy().view(np.uint32)))
    if not same:
        raise SystemExit("device and host-buffer PreprocessMatrixPack differ")
    line = {
        "metric": "PreprocessMatrixPack slices/s (d=%d, k=%d, Z_2^32, int32 "
                  "matrix)" % (d, k),
        "value": slices / (ms / 1000.0), "unit": "slices/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded uniform hint rows and "
                                "pack key)",
        "config": {"workload": "preprocess_d%d_slices%d_k%d_u32"
                               % (d, slices, k),
                   "matrix": [slices * d, k * d]},
        "e2e": {"value": slices / (ms_e2e / 1000.0), "unit": "slices/s",
                "h2d_bytes_per_step": int(hint.nbytes + pack_a.nbytes),
                "d2h_bytes_per_step": int(m_h.nbytes + a_h.nbytes +
                                          th_h.nbytes)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


SINGLE_CONFIGS = {
    # The reference metrics tool's shapes for a single request.
    "c2": dict(n=65536, d=2048, t=4, l=1, coeff_bits=32, log_q=32),
    "c1": dict(n=4096, d=2048, t=2, l=1, coeff_bits=64, log_q=52),
}


def run_single_workload(args):
    """Single-request latency of the plain engine on the small shapes: c2
    (n = 65536, d = 2048, t = 4, Z_2^32; DB 8192 x 16384 u16 + pack 8192 x
    4096 i32) or c1 (n = 4096, d = 2048, t = 2, Z_2^64 with q = 2^52). One
    request per step with L2 flushed (a 256 MB write) before each, each step
    timed alone with CUDA events: device-resident requests (`value`), the
    same calls replayed from a CUDA graph, the host-buffer C ABI (`e2e`), the
    fused GEMV alone against the HBM roofline, and the oracle on one host
    core (the reference is single-threaded)."""
    import torch
    from inspire_gb300 import build, pir, profiling, synthetic
    cfg = SINGLE_CONFIGS[args.config]
    build.build()
    n, d, t, l, cb = cfg["n"], cfg["d"], cfg["t"], cfg["l"], cfg["coeff_bits"]
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=cb,
                                   log_q=cfg["log_q"])
    mat = synthetic.make_material(params, seed=71)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack, mat.a_tilde_agg,
                                       mat.t_vec_h, mat.second_dim_a)
    nreq = 16
    fd, sd, pk = synthetic.make_requests(params, nreq, seed=72)
    iv = np.int32 if cb == 32 else np.int64
    tdt = torch.int32 if cb == 32 else torch.int64
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(iv)).to(dev)
    t_sd = torch.from_numpy(sd.view(iv)).to(dev)
    t_pk = torch.from_numpy(pk.view(iv)).to(dev)
    t_out = torch.empty((nreq, l, 2, d), dtype=tdt, device=dev)
    t_prod = torch.empty((nreq, srv.rows), dtype=tdt, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    lib = __import__("inspire_gb300._lib", fromlist=["load"]).load()
    err = ctypes.create_string_buffer(256)
    n1, nsd, npk = fd.shape[1], sd.shape[1], pk.shape[1]
    esz = np.dtype(params.coeff_dtype).itemsize

    def answer(i):
        srv.process_device(1, t_fd.data_ptr() + i * n1 * esz, n1,
                           t_sd.data_ptr() + i * nsd * d * esz, nsd,
                           t_pk.data_ptr() + i * npk * d * esz, npk,
                           t_out.data_ptr() + i * l * 2 * d * esz,
                           pir.ENGINE_PLAIN, sptr)

    def products(i):
        rc = lib.inspire_pir_products_device(
            srv._h, 1, t_fd.data_ptr() + i * n1 * esz,
            t_pk.data_ptr() + i * npk * d * esz,
            t_prod.data_ptr() + i * srv.rows * esz, pir.ENGINE_PLAIN, sptr,
            err, len(err))
        if rc:
            raise SystemExit(err.value)

    def per_step(fn, steps, warm, label="timed_request"):
        for i in range(warm):
            fn(i % nreq)
        stream.synchronize()
        times = []
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            # NVTX range: a profiler's launch list can keep only the request.
            torch.cuda.nvtx.range_push(label)
            e0.record(stream)
            fn(i % nreq)
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        return times

    # Parity of the timed path against the oracle on the first request.
    from oracle import pyoracle as orc
    r = params.rlwe
    op = orc.make_params(
        coeff_bits=cb, log_degree=d.bit_length() - 1, log_modulus=r.log_modulus,
        log_modulus1_after_switch=r.log_modulus1_after_switch,
        log_modulus2_after_switch=r.log_modulus2_after_switch,
        pack_log_digit=params.pack_gadget.log_digit,
        pack_num_digits=params.pack_gadget.num_digits,
        eval_log_digit=params.eval_gadget.log_digit,
        eval_num_digits=params.eval_gadget.num_digits, num_entries=n,
        interpolation_degree=t, entry_size_multiple=l)
    answer(0)
    stream.synchronize()
    want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                mat.t_vec_h, mat.second_dim_a, fd[0], sd[0], pk[0])
    got = t_out[0].cpu().numpy().view(params.coeff_dtype)
    if not np.array_equal(got.reshape(want.shape), want):
        raise SystemExit("single-request response differs from the oracle")

    hbm, _, peak_kind = peaks()
    with ClockSampler(0) as clk:
        t_ans = per_step(answer, args.steps, args.warmup)
    t_prod_ms = per_step(products, args.steps, args.warmup, "timed_products")

    # The same answer replayed from a CUDA graph (one launch per request).
    graphs = []
    for i in range(nreq):
        with pir.Graph(sptr) as g:
            answer(i)
        graphs.append(g)
    t_graph = per_step(lambda i: graphs[i].launch(sptr), args.steps, args.warmup,
                       "timed_graph")

    # End to end through the host-buffer C ABI (pinned host memory).
    h_fd = torch.from_numpy(fd.view(iv)).pin_memory().numpy().view(params.coeff_dtype)
    h_sd = torch.from_numpy(sd.view(iv)).pin_memory().numpy().view(params.coeff_dtype)
    h_pk = torch.from_numpy(pk.view(iv)).pin_memory().numpy().view(params.coeff_dtype)
    h_out = torch.empty((nreq, l, 2, d), dtype=tdt).pin_memory().numpy()

    def e2e(i):
        rc = lib.inspire_pir_process_batch(
            srv._h, 1, h_fd[i].ctypes.data, n1, h_sd[i].ctypes.data, nsd,
            h_pk[i].ctypes.data, npk, h_out[i].ctypes.data, pir.ENGINE_PLAIN,
            err, len(err))
        if rc:
            raise SystemExit(err.value)
    for i in range(args.warmup):
        e2e(i % nreq)
    t_e2e = []
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        e2e(i % nreq)
        t_e2e.append((time.perf_counter() - t0) * 1000.0)

    ms = statistics.mean(t_ans)
    ms_prod = statistics.mean(t_prod_ms)
    rows = srv.rows
    alg = profiling.plain_bytes(rows, srv.db_cols, srv.pack_cols, word=esz)
    gbs = alg / (ms_prod / 1000.0) / 1e9

    def pct(v, q):
        s = sorted(v)
        return s[min(len(s) - 1, int(q * len(s)))]
    tag = "u%d" % cb
    line = {
        "metric": "queries/s (single request, plain engine, n=%d d=%d t=%d, "
                  "Z_2^%d q=2^%d)" % (n, d, t, cb, cfg["log_q"]),
        "value": 1000.0 / ms, "unit": "queries/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": tag, "data": "synthetic (seeded uniform DB, pack matrix, "
                              "requests)",
        "config": {"workload": "pir_single_n%d_d%d_t%d_l%d_%s" % (n, d, t, l, tag),
                   "n": n, "d": d, "t": t, "l": l, "batch": 1,
                   "engine": "plain", "db_matrix": list(mat.db.shape),
                   "pack_matrix": list(mat.pack.shape),
                   "l2": "flushed before every request (256 MB write)"},
        "latency_ms": {"mean": ms, "p50": pct(t_ans, 0.5), "p99": pct(t_ans, 0.99)},
        "graph": {"queries_per_s": 1000.0 / statistics.mean(t_graph),
                  "latency_ms_p50": pct(t_graph, 0.5)},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": gbs / hbm,
                     "traffic": profiling.GEMV_TRAFFIC_PER_ALG_BYTE * alg,
                     "traffic_source": "ncu small case scaled by algorithmic bytes",
                     "kernel": "fused_gemv", "ms": ms_prod, "bytes": alg,
                     "peak_kind": peak_kind + " copy"},
        "clocks": clk.summary(),
        "gpu_launches": profiling.launches_per_step(pir.ENGINE_PLAIN, t) * args.steps,
        "e2e": {"value": 1000.0 / statistics.mean(t_e2e), "unit": "queries/s",
                "latency_ms_p50": pct(t_e2e, 0.5),
                "h2d_bytes_per_step": int(h_fd[0].nbytes + h_sd[0].nbytes +
                                          h_pk[0].nbytes),
                "d2h_bytes_per_step": int(h_out[0].nbytes)},
    }
    if not args.no_cpu_baseline:
        done, t0 = 0, time.perf_counter()
        stages = []
        while time.perf_counter() - t0 < 10.0:
            _, st = orc.process_response_staged(
                op, mat.db, mat.pack, mat.a_tilde_agg, mat.t_vec_h,
                mat.second_dim_a, fd[done % nreq], sd[done % nreq],
                pk[done % nreq], mode=orc.MODE_FP64, threads=1,
                condensed_db=cb == 64)
            stages.append(st)
            done += 1
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {
            "value": done / el, "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": "%d requests in %.1f s on one host thread (oracle timing "
                      "build, FP64 FFT path, as the single-threaded reference)"
                      % (done, el),
            "single_core_ms": 1000.0 * el / done,
            "stages_ms": {k: statistics.mean(x[k] for x in stages)
                          for k in stages[0]},
            "build": orc.timing_build_string()}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=10)
    ap.add_argument("--entries", type=int, default=N_ENTRIES,
                    help="records of the interpolate / hint workloads")
    ap.add_argument("--workload", default="answer",
                    choices=["answer", "pack", "interpolate", "hint", "single",
                             "preprocess"],
                    help="answer: the online answer (default); pack: the "
                         "packing micro-workload; interpolate: the offline "
                         "DB interpolation; hint: the offline hint matrix; "
                         "preprocess: the offline PreprocessMatrixPack; "
                         "single: one request at a time on the small shapes "
                         "(--config c2 or c1)")
    ap.add_argument("--config", default="c2", choices=sorted(SINGLE_CONFIGS),
                    help="shape of the single workload")
    ap.add_argument("--coeff-bits", type=int, default=32, choices=[32, 64],
                    help="answer workload: CoeffType u32 (q = 2^32) or u64 "
                         "(q = 2^56, the reference's real parameters)")
    args = ap.parse_args()
    global COEFF_BITS, LOG_Q
    COEFF_BITS = args.coeff_bits
    LOG_Q = 32 if COEFF_BITS == 32 else 56
    if args.workload == "pack" and args.impl == "ours":
        run_pack_workload(args)
        return
    if args.workload == "interpolate" and args.impl == "ours":
        run_interpolate_workload(args)
        return
    if args.workload == "hint" and args.impl == "ours":
        run_hint_workload(args)
        return
    if args.workload == "preprocess" and args.impl == "ours":
        run_preprocess_workload(args)
        return
    if args.workload == "single" and args.impl == "ours":
        run_single_workload(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from inspire_gb300 import build, pir
    build.build()

    params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk = make_workload(
        batch=args.batch)
    srv = pir.PirServer.CreateCombined(params, db, pack, a_tilde, t_vec_h, sda)
    B = args.batch
    d = DEGREE
    n1 = fd.shape[1]
    cdt = params.coeff_dtype
    iv = np.int32 if COEFF_BITS == 32 else np.int64
    tdt = torch.int32 if COEFF_BITS == 32 else torch.int64
    l = 1

    # Device-resident requests and responses.
    dev = torch.device("cuda", local)
    t_fd = torch.from_numpy(fd.view(iv)).to(dev)
    t_sd = torch.from_numpy(sd.view(iv)).to(dev)
    t_pk = torch.from_numpy(pk.view(iv)).to(dev)
    t_out = torch.empty((B, l, 2, d), dtype=tdt, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    engine = pir.ENGINE_TENSOR
    try:
        srv.process_device(1, t_fd.data_ptr(), n1, t_sd.data_ptr(), sd.shape[1],
                           t_pk.data_ptr(), pk.shape[1], t_out.data_ptr(),
                           engine, sptr)
        stream.synchronize()
    except pir.InspireError:
        engine = pir.ENGINE_PLAIN

    # The engine autotuner: plain vs tensor (every DB form, request tile
    # and split-K factor) at batch sizes up to B; the timed step then runs
    # the tensor engine in the configuration tuned for B.
    tuned = None
    if engine == pir.ENGINE_TENSOR:
        crossover = srv.tune_engines(B)
        table = srv.engine_table()
        row = [r for r in table if r["batch"] == B][0]
        tuned = {"form": row["form"], "split_k": row["split"],
                 "product_ms": row["tensor_ms"], "crossover": crossover,
                 "engine_table": table}

    # Parity of the two engines on the first requests.
    check = min(B, 8)
    got_plain = srv.process_arrays(fd[:check], sd[:check], pk[:check],
                                   pir.ENGINE_PLAIN)
    got_eng = srv.process_arrays(fd[:check], sd[:check], pk[:check], engine)
    if not np.array_equal(got_plain, got_eng):
        raise SystemExit("engine responses differ")

    def step(bsz, eng):
        srv.process_device(bsz, t_fd.data_ptr(), n1, t_sd.data_ptr(),
                           sd.shape[1], t_pk.data_ptr(), pk.shape[1],
                           t_out.data_ptr(), eng, sptr)

    def timed(fn, steps, warm, label):
        for _ in range(warm):
            fn()
        stream.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        # An NVTX range around the timed launches, so that a profiler's
        # launch list can keep only them (ncu --nvtx --nvtx-include).
        torch.cuda.nvtx.range_push(label)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        e1.synchronize()
        torch.cuda.synchronize()
        ms = replica_time(e0.elapsed_time(e1), dist, dev)
        return ms / steps

    hbm, tflops, peak_kind = peaks()
    with ClockSampler(local) as clk:
        ms_step = timed(lambda: step(B, engine), args.steps, args.warmup,
                        "timed_step")
    # The responses of the last timed step, checked against the oracle once
    # every timed leg has run.
    timed_out = t_out.cpu().numpy().view(cdt)
    # Plain single-query engine beside it (B = 1 per step).
    ms_plain = timed(lambda: step(1, pir.ENGINE_PLAIN), args.plain_steps,
                     args.warmup, "timed_plain")
    # Kernel-only timing of the dominant kernel for the roofline.
    from inspire_gb300 import profiling
    kern = profiling.kernel_times(srv, engine, B, t_fd, t_sd, t_pk, t_out,
                                  stream, n1, sd.shape[1], pk.shape[1])

    # e2e through the host-buffer C ABI (pinned host memory).
    h_fd = torch.from_numpy(fd.view(iv)).pin_memory().numpy().view(cdt)
    h_sd = torch.from_numpy(sd.view(iv)).pin_memory().numpy().view(cdt)
    h_pk = torch.from_numpy(pk.view(iv)).pin_memory().numpy().view(cdt)
    h_out = torch.empty((B, l, 2, d), dtype=tdt).pin_memory().numpy()
    lib = __import__("inspire_gb300._lib", fromlist=["load"]).load()
    err = ctypes.create_string_buffer(256)

    def e2e_step():
        rc = lib.inspire_pir_process_batch(
            srv._h, B, h_fd.ctypes.data, n1, h_sd.ctypes.data, sd.shape[1],
            h_pk.ctypes.data, pk.shape[1], h_out.ctypes.data, engine, err,
            len(err))
        if rc:
            raise SystemExit(err.value)
    for _ in range(args.warmup):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(max(3, args.steps // 2)):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / max(3, args.steps // 2)

    # The same host-buffer path through the asynchronous workspace C ABI
    # with two batches in flight: each step's copies (in pinned staging,
    # written once beforehand like the buffers above) overlap the other
    # batch's GPU work.
    def make_ws():
        h = ctypes.c_void_p()
        rc = lib.inspire_pir_workspace_create(srv._h, B, ctypes.byref(h), err,
                                              len(err))
        if rc:
            raise SystemExit(err.value)
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        lib.inspire_pir_workspace_host_buffers(h, *[ctypes.byref(x) for x in ptrs])
        row = srv.db_cols * np.dtype(cdt).itemsize
        dst = (ctypes.c_uint8 * (B * row)).from_address(ptrs[0].value)
        buf = np.frombuffer(dst, dtype=cdt).reshape(B, srv.db_cols)
        buf[:, :n1] = fd
        buf[:, n1:] = 0
        ctypes.memmove(ptrs[1].value, sd.ctypes.data, sd.nbytes)
        ctypes.memmove(ptrs[2].value, pk.ctypes.data, pk.nbytes)
        return h
    wss = [make_ws(), make_ws()]

    def submit(h):
        if lib.inspire_pir_workspace_submit(h, B, engine, err, len(err)):
            raise SystemExit(err.value)

    def wait(h):
        if lib.inspire_pir_workspace_wait(h, err, len(err)):
            raise SystemExit(err.value)
    for h in wss:
        submit(h)
    for h in wss:
        wait(h)
    pipe_steps = max(4, args.steps)
    t0 = time.perf_counter()
    submit(wss[0])
    for i in range(1, pipe_steps):
        submit(wss[i % 2])
        wait(wss[(i - 1) % 2])
    wait(wss[(pipe_steps - 1) % 2])
    pipe_s = (time.perf_counter() - t0) / pipe_steps
    for h in wss:
        lib.inspire_pir_workspace_destroy(h)

    # Bit-exact check of the timed batch: first, middle and last response
    # against the oracle's exact product (a run that fails exits non-zero).
    picks = sorted({0, B // 2, B - 1})
    ocheck = oracle_check(params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk,
                          timed_out, picks)
    if ocheck["mismatches"]:
        raise SystemExit("timed responses %s differ from the oracle"
                         % ocheck["mismatches"])

    rows, cols = db.shape
    db_bytes = db.nbytes + pack.nbytes
    qps = world * B / (ms_step / 1000.0)
    plain_qps = 1000.0 / ms_plain
    line = {
        "metric": metric_name(),
        "comparison": "batched tensor-core engine (value) vs plain "
                      "single-query engine (plain), responses bit-exact",
        "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": word_tag(), "data": "synthetic (seeded uniform DB, pack matrix, "
                                     "queries)",
        "config": {"workload": workload_name(),
                   "n": N_ENTRIES, "d": DEGREE, "t": INTERP, "l": 1,
                   "batch": B, "engine": "tensor" if engine else "plain",
                   "db_matrix": [rows, cols], "pack_matrix": list(pack.shape),
                   "l2": "inputs larger than L2 (9 GiB matrices per step)",
                   "parallelism": "replicas" if world > 1 else "single",
                   "autotune": tuned},
        "plain": {"queries_per_s": plain_qps, "ms_per_query": ms_plain,
                  "db_gbs": db_bytes / (ms_plain / 1000.0) / 1e9},
        "db_gbs": db_bytes * (1 if engine else B) / (ms_step / 1000.0) / 1e9,
        "speedup_vs_plain": qps / world / plain_qps,
        "roofline": kern["roofline"],
        "kernels": kern["kernels"],
        "peak_kind": peak_kind,
        "clocks": clk.summary(),
        "gpu_launches": kern["launches_per_step"] * args.steps,
        "oracle_check": ocheck,
        "e2e": {"value": world * B / e2e_s, "unit": "queries/s",
                "h2d_bytes_per_step": int(h_fd.nbytes + h_sd.nbytes +
                                          h_pk.nbytes),
                "d2h_bytes_per_step": int(h_out.nbytes)},
        "e2e_pipelined": {"value": world * B / pipe_s, "unit": "queries/s",
                          "workspaces_in_flight": 2,
                          "h2d_bytes_per_step": int(h_fd.nbytes + h_sd.nbytes +
                                                    h_pk.nbytes),
                          "d2h_bytes_per_step": int(h_out.nbytes)},
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(
            params, db, pack, a_tilde, t_vec_h, sda, fd, sd, pk)
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
