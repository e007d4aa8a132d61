"""The external-product, request-NTT and finalize kernels with the
register-resident radix-16 NTT (d = 2048, 4096, 8192) against each other,
the radix-4 kernels and the CPU oracle (crypto/external_product.cc:35-114
inside EvalPoly, crypto/pir/server/pir_server.cc:128-150,
crypto/lwes_to_rlwe.cc:448-479): once shards x requests fill the GPU the
answer takes one block per shard and request over all primes; smaller
batches take one block per prime with two transforms side by side (d <= 4096)
or the radix-4 kernels (d = 8192). Every response of a large batch must equal
the same requests answered eight at a time.
"""
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
        num_entries=params.num_entries,
        interpolation_degree=params.interpolation_degree,
        entry_size_multiple=params.entry_size_multiple)


@pytest.mark.parametrize("d,coeff_bits,log_q,t,l,batch", [
    (4096, 32, 32, 4, 1, 160),
    (4096, 32, 32, 8, 2, 80),
    (4096, 64, 56, 4, 1, 160),
    (2048, 32, 32, 4, 1, 320),
    (2048, 64, 52, 2, 2, 160),
    (2048, 32, 32, 4, 1, 160),   # below two per SM: the per-prime kernel
    (8192, 32, 32, 2, 1, 160),
    (8192, 32, 32, 2, 2, 80),
    (8192, 64, 56, 2, 1, 152),
])
def test_radix16_external_product_matches_small_batches_and_oracle(
        d, coeff_bits, log_q, t, l, batch):
    params = synthetic.make_params(d=d, n=t * 2048, t=t, l=l,
                                   coeff_bits=coeff_bits, log_q=log_q)
    mat = synthetic.make_material(params, seed=t + l)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack, mat.a_tilde_agg,
                                       mat.t_vec_h, mat.second_dim_a)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=batch + t,
                                         full_range=True)
    big = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    small = np.concatenate([
        srv.process_arrays(fd[i:i + 8], sd[i:i + 8], pk[i:i + 8], pir.ENGINE_PLAIN)
        for i in range(0, batch, 8)])
    assert np.array_equal(big, small)
    op = _oparams(params)
    for i in (0, batch - 1):
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i], sd[i],
                                    pk[i])
        assert np.array_equal(big[i], want), i
