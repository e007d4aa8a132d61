"""The vPIR server answer (crypto/vpir/server/vpir_server.cc:102-195) on the
GPU against the oracle's GEMV and FinalizeMatrixPack, both finalize modes."""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def _oparams(params):
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
        num_entries=params.num_entries, interpolation_degree=1,
        entry_size_multiple=params.entry_size_multiple)


def oracle_vpir(params, mat, fd, pk, local):
    cb = params.rlwe.coeff_bits
    d, k, ell = params.rlwe.degree, params.pack_gadget.num_digits, \
        params.entry_size_multiple
    lq = params.rlwe.log_modulus
    bprime = orc.matrix_multiply(mat.db, fd, cb)
    partial = orc.matrix_multiply(mat.pack, pk[:k].reshape(-1), cb)
    out = []
    for s in range(ell):
        b1, b2 = bprime[s * d:(s + 1) * d], partial[s * d:(s + 1) * d]
        if local:
            v = (b1.astype(object) + b2.astype(object)) % (1 << lq)
            out.append(np.array(v, dtype=params.coeff_dtype))
        else:
            out.append(orc.finalize_matrix_pack(_oparams(params), b1, b2,
                                                pk[k:],
                                                mat.t_vec_h[s * k:(s + 1) * k]))
    return np.stack(out)


@pytest.mark.parametrize("local", [True, False])
@pytest.mark.parametrize("cb,log_q,engine", [(32, 32, pir.ENGINE_PLAIN),
                                             (32, 32, pir.ENGINE_TENSOR),
                                             (64, 52, pir.ENGINE_PLAIN)])
def test_vpir_answer_matches_oracle(local, cb, log_q, engine):
    d, ell, n = 256, 3, 2048
    params = synthetic.make_params(d=d, n=n, t=1, l=ell, coeff_bits=cb,
                                   log_q=log_q)
    mat = synthetic.make_material(params, seed=ell + cb)
    srv = pir.VpirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        local_finalize=local)
    fd, _, pk = synthetic.make_requests(params, 4, seed=cb + 1)
    k = params.pack_gadget.num_digits
    if local:
        pk = pk[:, :k]
    got = srv.process_arrays(fd, pk, engine)
    for i in (0, 3):
        want = oracle_vpir(params, mat, fd[i], pk[i], local)
        assert np.array_equal(got[i], want), i
    # The request form.
    req = pir.VpirRequest([fd[1][j * d:(j + 1) * d] for j in range(n // d)],
                          list(pk[1]))
    assert np.array_equal(srv.ProcessResponse(req).b_responses, got[1])


def test_vpir_validation_messages():
    params = synthetic.make_params(d=128, n=1024, t=1, l=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=1)
    srv = pir.VpirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        local_finalize=True)
    fd, _, pk = synthetic.make_requests(params, 1)
    with pytest.raises(pir.InspireError, match="Packing key must contain 2 "):
        srv.process_arrays(fd, pk)            # 4 polys, local wants 2
    with pytest.raises(pir.InspireError,
                       match="must match DB matrix columns"):
        srv.process_arrays(fd[:, :-1], pk[:, :2])
