"""The CUDA path against the committed golden fixtures (tests/golden):
fixed inputs and outputs, so this needs neither the oracle nor the fixture
generator at run time. Answers through the plain engine and, where the DB
has whole 256-row tiles, the tensor engine (PirServer::ProcessResponse,
pir_server.cc:154-306); Interpolate (db_row_interpolation.cc:115-228);
InnerProductFft (polynomial_fft.cc:68-197)."""
import numpy as np
import pytest

from inspire_gb300 import build, pir
from tests.golden import fixtures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


ANSWERS = sorted(n for n, c in fixtures.CASES.items() if c["kind"] == "answer")
OTHERS = sorted(n for n, c in fixtures.CASES.items() if c["kind"] != "answer")


@pytest.mark.parametrize("name", ANSWERS)
def test_answers_match_fixture(name):
    case, a = fixtures.load(name)
    params = fixtures.pir_params(case)
    srv = pir.PirServer.CreateCombined(params, a["db"], a["pack"],
                                       a["a_tilde_agg"], a["t_vec_h"],
                                       a["second_dim_a"])
    engines = [pir.ENGINE_PLAIN] + ([pir.ENGINE_TENSOR] if case["tensor"] else [])
    for engine in engines:
        got = srv.process_arrays(a["first_dim"], a["second_dim"],
                                 a["packing_key"], engine)
        srv.check()
        assert np.array_equal(got.reshape(a["responses"].shape),
                              a["responses"]), engine


@pytest.mark.parametrize("name", OTHERS)
def test_kernels_match_fixture(name):
    case, a = fixtures.load(name)
    if case["kind"] == "interpolate":
        got = pir.Interpolate(a["evals"], case["d"], case["t"], case["p"])
    else:
        got = pir.inner_product(a["u"], a["v"], case["coeff_bits"],
                                u_bits=case["u_bits"], v_bits=case["v_bits"],
                                chunk_bits=case["chunk_bits"],
                                u_signed=case["u_signed"])
    assert np.array_equal(got, a["out"])
