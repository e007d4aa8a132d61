"""The batched tensor-core engine (8-bit limbs on tcgen05) against the plain
engine and the CPU oracle. Both engines must give identical responses.

The adversarial cases fill every byte with 255 (DB entries 0xFFFF, pack
entries -1, query words 0xFFFFFFFF): each fp32 accumulator element then
reaches the largest partial sum the limb plan allows (64 * 2 * 255^2), so an
inexact accumulation or decode would show up as a mismatch.
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def oparams(params):
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


def _server(params, mat):
    return pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        mat.second_dim_a)


@pytest.mark.parametrize("d,n,t,batch", [
    (128, 8192, 2, 1),       # R = 256, C = 4096
    (128, 8192, 2, 64),      # one full request tile
    (128, 8192, 2, 65),      # a ragged second tile
    (256, 16000, 4, 7),      # C = 4000: columns padded to a multiple of 64
    (1024, 32768, 4, 130),   # three request tiles
])
def test_tensor_matches_plain_and_oracle(d, n, t, batch):
    params = synthetic.make_params(d=d, n=n, t=t, coeff_bits=32)
    mat = synthetic.make_material(params, seed=d + batch)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=batch,
                                         full_range=True)
    got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    got_p = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(got_t, got_p)
    op = oparams(params)
    for i in sorted({0, batch - 1}):
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i],
                                    sd[i], pk[i])
        assert np.array_equal(got_t[i], want)


@pytest.mark.parametrize("mat_dtype", [np.int32, np.int16])
def test_tensor_all_ones_bytes(mat_dtype):
    params = synthetic.make_params(d=128, n=2 * 8192, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=3, mat_dtype=mat_dtype)
    mat.db[:] = 0xFFFF
    mat.pack[:] = -1
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, 64, seed=4, full_range=True)
    fd[:] = 0xFFFFFFFF
    pk[:] = 0xFFFFFFFF
    got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    got_p = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(got_t, got_p)
    want = orc.process_response(oparams(params), mat.db, mat.pack,
                                mat.a_tilde_agg, mat.t_vec_h,
                                mat.second_dim_a, fd[0], sd[0], pk[0])
    assert np.array_equal(got_t[0], want)


def test_tensor_engine_repeated_batches_reuse_buffers():
    # A large batch followed by smaller ones: the request byte planes are
    # reused, stale rows must not leak into the smaller batches.
    params = synthetic.make_params(d=128, n=8192, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=9)
    srv = _server(params, mat)
    for batch in (100, 3, 64, 1):
        fd, sd, pk = synthetic.make_requests(params, batch, seed=batch + 50)
        assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR),
                              srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN))


def test_tensor_engine_unavailable_for_u64():
    params = synthetic.make_params(d=128, n=8192, t=2, coeff_bits=64, log_q=52)
    mat = synthetic.make_material(params, seed=1, pad_to=32)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, 1)
    with pytest.raises(pir.InspireError, match="tensor engine unavailable"):
        srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
