"""Writes the golden fixtures of fixtures.CASES (seeded inputs and the
oracle's exact outputs) as .npz files beside this script.

  python tests/golden/make_golden.py

The oracle is the CPU restatement in oracle/; its FP64 mode follows the
reference's FFT rounding, and each fixture records whether that mode gives
the same outputs as the exact one on its inputs (`fp64_equal`).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from inspire_gb300 import synthetic  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402
from tests.golden import fixtures  # noqa: E402


def answers(params, mat, fd, sd, pk, mode):
    op = fixtures.oracle_params(params)
    return np.stack([
        orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                             mat.t_vec_h, mat.second_dim_a, fd[i], sd[i],
                             pk[i], mode=mode)
        for i in range(fd.shape[0])])


def make_answer(case):
    params = fixtures.pir_params(case)
    mat = synthetic.make_material(params, seed=case["seed"])
    fd, sd, pk = synthetic.make_requests(params, case["batch"],
                                         seed=case["seed"] + 100,
                                         full_range=True)
    exact = answers(params, mat, fd, sd, pk, orc.MODE_EXACT)
    fp64 = answers(params, mat, fd, sd, pk, orc.MODE_FP64)
    case = dict(case, fp64_equal=bool(np.array_equal(exact, fp64)))
    return case, dict(db=mat.db, pack=mat.pack, a_tilde_agg=mat.a_tilde_agg,
                      t_vec_h=mat.t_vec_h, second_dim_a=mat.second_dim_a,
                      first_dim=fd, second_dim=sd, packing_key=pk,
                      responses=exact)


def make_interpolate(case):
    dt = np.dtype(case["dtype"])
    d, t, p = case["d"], case["t"], case["p"]
    rng = np.random.default_rng(case["seed"])
    evals = rng.integers(0, p, size=t * d).astype(dt)
    return case, dict(evals=evals, out=orc.interpolate(evals, d, t, p))


def make_inner_product(case):
    cb = case["coeff_bits"]
    dt = np.uint32 if cb == 32 else np.uint64
    rng = np.random.default_rng(case["seed"])
    shape = (case["n"], case["d"])
    u = rng.integers(0, np.iinfo(dt).max, size=shape, dtype=dt, endpoint=True)
    v = rng.integers(0, np.iinfo(dt).max, size=shape, dtype=dt, endpoint=True)
    kw = dict(u_bits=case["u_bits"], v_bits=case["v_bits"],
              chunk_bits=case["chunk_bits"], u_signed=case["u_signed"])
    exact = orc.inner_product(u, v, cb, mode=orc.MODE_EXACT, **kw)
    fp64 = orc.inner_product(u, v, cb, mode=orc.MODE_FP64, **kw)
    case = dict(case, fp64_equal=bool(np.array_equal(exact, fp64)))
    return case, dict(u=u, v=v, out=exact)


MAKERS = {"answer": make_answer, "interpolate": make_interpolate,
          "inner_product": make_inner_product}


def main():
    for name, case in fixtures.CASES.items():
        case, arrays = MAKERS[case["kind"]](dict(case))
        fixtures.save(name, case, arrays)
        size = os.path.getsize(fixtures.path(name))
        print("%-36s %7d bytes  fp64_equal=%s"
              % (name, size, case.get("fp64_equal", "-")))


if __name__ == "__main__":
    main()
