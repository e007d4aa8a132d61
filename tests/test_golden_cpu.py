"""The oracle against the committed golden fixtures (tests/golden): the
fixtures' inputs are what their seeds make, and the oracle still gives
their frozen outputs (PirServer::ProcessResponse, pir_server.cc:154-306;
Interpolate, db_row_interpolation.cc:115-228; InnerProductFft,
polynomial_fft.cc:68-197)."""
import numpy as np
import pytest

from inspire_gb300 import synthetic
from oracle import pyoracle as orc
from tests.golden import fixtures


@pytest.mark.parametrize("name", sorted(fixtures.CASES))
def test_fixture_matches_its_case(name):
    case, a = fixtures.load(name)
    want = fixtures.CASES[name]
    assert {k: case[k] for k in want} == want
    if case["kind"] == "answer":
        params = fixtures.pir_params(case)
        mat = synthetic.make_material(params, seed=case["seed"])
        fd, sd, pk = synthetic.make_requests(params, case["batch"],
                                             seed=case["seed"] + 100,
                                             full_range=True)
        for k, v in (("db", mat.db), ("pack", mat.pack),
                     ("a_tilde_agg", mat.a_tilde_agg),
                     ("t_vec_h", mat.t_vec_h),
                     ("second_dim_a", mat.second_dim_a), ("first_dim", fd),
                     ("second_dim", sd), ("packing_key", pk)):
            assert np.array_equal(a[k], v), k


@pytest.mark.parametrize("name", sorted(fixtures.CASES))
def test_oracle_reproduces_fixture(name):
    case, a = fixtures.load(name)
    if case["kind"] == "answer":
        op = fixtures.oracle_params(fixtures.pir_params(case))
        for i in range(a["first_dim"].shape[0]):
            for mode in (orc.MODE_EXACT, orc.MODE_FP64):
                if mode == orc.MODE_FP64 and not case["fp64_equal"]:
                    continue
                got = orc.process_response(
                    op, a["db"], a["pack"], a["a_tilde_agg"], a["t_vec_h"],
                    a["second_dim_a"], a["first_dim"][i], a["second_dim"][i],
                    a["packing_key"][i], mode=mode)
                assert np.array_equal(got, a["responses"][i]), (i, mode)
    elif case["kind"] == "interpolate":
        got = orc.interpolate(a["evals"], case["d"], case["t"], case["p"])
        assert np.array_equal(got, a["out"])
    else:
        for mode in (orc.MODE_EXACT, orc.MODE_FP64):
            got = orc.inner_product(a["u"], a["v"], case["coeff_bits"],
                                    u_bits=case["u_bits"],
                                    v_bits=case["v_bits"],
                                    chunk_bits=case["chunk_bits"],
                                    u_signed=case["u_signed"], mode=mode)
            assert np.array_equal(got, a["out"]), mode
