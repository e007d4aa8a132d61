"""Golden fixtures of the answer path, frozen as .npz files beside this
module and written by make_golden.py.

Each fixture holds seeded inputs and the oracle's exact outputs:
  * answer_*: PirServer::ProcessResponse
    (crypto/pir/server/pir_server.cc:154-306) on combined matrices, for a
    batch of requests (first-dimension words over the full coefficient
    range, so out-of-range words are covered);
  * interpolate_*: Interpolate (crypto/db_row_interpolation.cc:115-228);
  * inner_product_*: InnerProductFft (crypto/polynomial_fft.cc:68-197) with
    the reference's chunk rule.
Where the reference's FP64 FFT rounds every product exactly on these inputs
the fixture records it (`fp64_equal`), so the exact outputs are also the
reference algorithm's outputs there. The fixtures pin the oracle against
regressions (tests/test_golden_cpu.py) and give the GPU path fixed answers
that do not depend on the oracle at run time (tests/test_gpu_golden.py).
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# name -> how the case is made. `params` are synthetic.make_params keywords.
CASES = {
    "answer_u32_d64_t4_n1024": dict(
        kind="answer", params=dict(d=64, n=1024, t=4, coeff_bits=32),
        seed=11, batch=3, tensor=True),
    "answer_u64_q52_d32_t2_l2_n256": dict(
        kind="answer",
        params=dict(d=32, n=256, t=2, l=2, coeff_bits=64, log_q=52),
        seed=12, batch=2, tensor=False),
    "answer_u32_d64_t1_n128": dict(
        kind="answer", params=dict(d=64, n=128, t=1, coeff_bits=32),
        seed=13, batch=2, tensor=False),
    "answer_u32_d32_t8_n512": dict(
        kind="answer", params=dict(d=32, n=512, t=8, coeff_bits=32),
        seed=14, batch=2, tensor=False),
    "interpolate_u16_d32_t8_p65535": dict(
        kind="interpolate", d=32, t=8, p=65535, dtype="uint16", seed=15),
    "interpolate_u32_d64_t4_p1031": dict(
        kind="interpolate", d=64, t=4, p=1031, dtype="uint32", seed=16),
    "inner_product_u32_n3_d64": dict(
        kind="inner_product", coeff_bits=32, n=3, d=64, u_bits=19,
        v_bits=32, chunk_bits=20, u_signed=False, seed=17),
    "inner_product_u64_n2_d32_signed": dict(
        kind="inner_product", coeff_bits=64, n=2, d=32, u_bits=19,
        v_bits=52, chunk_bits=20, u_signed=True, seed=18),
}


def path(name):
    return os.path.join(HERE, name + ".npz")


def load(name):
    """The fixture's arrays and its case description."""
    with np.load(path(name)) as z:
        arrays = {k: z[k] for k in z.files if k != "case"}
        case = json.loads(str(z["case"]))
    return case, arrays


def save(name, case, arrays):
    np.savez_compressed(path(name), case=np.array(json.dumps(case)), **arrays)


def pir_params(case):
    from inspire_gb300 import synthetic
    return synthetic.make_params(**case["params"])


def oracle_params(params):
    """The oracle's parameter struct for a PirParams."""
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
