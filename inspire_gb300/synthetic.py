"""Seeded synthetic server material and requests with the reference's shapes.

The large workloads (n up to 2^20) cannot run the reference's offline
preprocessing here, so the DB matrix is drawn as already-interpolated values
uniform in [0, p), the packing matrix as signed entries with the reference's
norm bound |x| < 4*sqrt(d)*2^pack_log_digit (crypto/lwes_to_rlwe.cc:203-223,
crypto/lwes_to_rlwe_test.cc:470-526), t_vec_h as signed pack digits and every
ciphertext / key polynomial uniform mod q. All draws come from one seed.
"""
import math
from dataclasses import dataclass

import numpy as np

from .pir import (GadgetParams, PirParams, PirRequest, RlweParams)


def parallel_integers(shape, low, high, dtype, seed, threads=None):
    """Uniform integers in [low, high) filled by several threads (the numpy
    generators release the GIL), one independent stream per slice."""
    import os
    import threading
    out = np.empty(int(np.prod(shape)), dtype=dtype)
    threads = threads or min(32, os.cpu_count() or 1)
    seqs = np.random.SeedSequence(seed).spawn(threads)
    n = out.shape[0]
    step = (n + threads - 1) // threads

    def fill(i):
        lo, hi = i * step, min(n, (i + 1) * step)
        if lo < hi:
            g = np.random.default_rng(seqs[i])
            out[lo:hi] = g.integers(low, high, size=hi - lo, dtype=dtype)

    ts = [threading.Thread(target=fill, args=(i,)) for i in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return out.reshape(shape)


def make_params(d, n, t, l=1, coeff_bits=32, log_q=None, log_p=16,
                plaintext_modulus=65535, pack=(19, 2), evalg=(19, 3),
                log_q1=None, log_q2=None):
    """PirParams with the reference metrics-tool conventions
    (crypto/pir/benchmarking/pir_metrics_tool.cc:79-114)."""
    if log_q is None:
        log_q = coeff_bits
    log_d = d.bit_length() - 1
    if log_q1 is None:
        log_q1 = min(log_q, log_p + log_d + 2)
    if log_q2 is None:
        log_q2 = min(log_q, log_p + 2)
    rlwe = RlweParams(degree=d, log_modulus=log_q,
                      log_modulus1_after_switch=log_q1,
                      log_modulus2_after_switch=log_q2, variance=40,
                      coeff_bits=coeff_bits)
    return PirParams(rlwe=rlwe, plaintext_modulus=plaintext_modulus,
                     pack_gadget=GadgetParams(*pack),
                     eval_gadget=GadgetParams(*evalg), num_entries=n,
                     interpolation_degree=t, entry_size_multiple=l)


@dataclass
class Material:
    db: np.ndarray          # (l*t*d, db_cols) DbDataType
    pack: np.ndarray        # (l*t*d, k*d) MatCoeffType
    a_tilde_agg: np.ndarray  # (l*t, d)
    t_vec_h: np.ndarray     # (l*t*k, d)
    second_dim_a: np.ndarray  # (2*ne, d) or (0, d)


def _uniform_mod(rng, shape, log_q, dtype):
    hi = np.iinfo(dtype).max if log_q >= 8 * np.dtype(dtype).itemsize \
        else (1 << log_q) - 1
    return rng.integers(0, hi, size=shape, dtype=dtype, endpoint=True)


def make_material(params: PirParams, seed=1, db_dtype=np.uint16,
                  mat_dtype=np.int32, db_cols=None, pad_to=1):
    rng = np.random.default_rng(seed)
    r = params.rlwe
    d, t, l = r.degree, params.interpolation_degree, params.entry_size_multiple
    k = params.pack_gadget.num_digits
    ne = params.eval_gadget.num_digits
    cdt = params.coeff_dtype
    rows = l * t * d
    if db_cols is None:
        db_cols = params.InterpolatedRows()
        db_cols = (db_cols + pad_to - 1) // pad_to * pad_to
    pmax = min(params.plaintext_modulus, np.iinfo(db_dtype).max + 1)
    db = rng.integers(0, pmax, size=(rows, db_cols), dtype=db_dtype)
    bound = int(4 * math.sqrt(d) * (1 << params.pack_gadget.log_digit))
    info = np.iinfo(mat_dtype)
    if info.min < 0:
        bound = min(bound, info.max)
        pack = rng.integers(-bound + 1, bound, size=(rows, k * d),
                            dtype=mat_dtype)
    else:
        pack = _uniform_mod(rng, (rows, k * d), r.log_modulus, mat_dtype)
    a_tilde = _uniform_mod(rng, (l * t, d), r.log_modulus, cdt)
    half = 1 << (params.pack_gadget.log_digit - 1)
    th = rng.integers(-half, half, size=(l * t * k, d), dtype=np.int64)
    t_vec_h = th.astype(cdt)  # two's complement, as SignedGadgetInv stores
    if t > 1:
        sda = _uniform_mod(rng, (2 * ne, d), r.log_modulus, cdt)
    else:
        sda = np.zeros((0, d), dtype=cdt)
    return Material(db, pack, a_tilde, t_vec_h, sda)


def make_requests(params: PirParams, batch, seed=2, first_dim_len=None,
                  full_range=False):
    """Stacked request arrays (B, n1), (B, 2ne, d), (B, 2k, d)."""
    rng = np.random.default_rng(seed)
    r = params.rlwe
    d = r.degree
    cdt = params.coeff_dtype
    k = params.pack_gadget.num_digits
    ne = params.eval_gadget.num_digits
    log_q = r.coeff_bits if full_range else r.log_modulus
    n1 = first_dim_len or params.InterpolatedRows()
    fd = _uniform_mod(rng, (batch, n1), log_q, cdt)
    nsd = 2 * ne if params.interpolation_degree > 1 else 0
    sd = _uniform_mod(rng, (batch, nsd, d), log_q, cdt)
    pk = _uniform_mod(rng, (batch, 2 * k, d), log_q, cdt)
    return fd, sd, pk


def as_requests(fd, sd, pk):
    return [PirRequest(fd[i], sd[i], pk[i]) for i in range(fd.shape[0])]
