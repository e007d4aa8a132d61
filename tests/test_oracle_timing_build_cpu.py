"""The timing build of the oracle (the CPU baseline) gives the checker's
bytes: the staged ProcessResponse with the reference's stage timers, and the
condensed-word DB product the reference runs for a u64 CoeffType
(crypto/matrix.cc:261-318, 376-462; preprocessing_server.h:127-153), equal
the checker build's plain ProcessResponse on the same inputs.
"""
import numpy as np
import pytest

from inspire_gb300 import synthetic
from oracle import pyoracle as orc


def _op(params):
    r = params.rlwe
    return orc.make_params(
        coeff_bits=r.coeff_bits, log_degree=r.degree.bit_length() - 1,
        log_modulus=r.log_modulus,
        log_modulus1_after_switch=r.log_modulus1_after_switch,
        log_modulus2_after_switch=r.log_modulus2_after_switch,
        pack_log_digit=19, pack_num_digits=2, eval_log_digit=19,
        eval_num_digits=3, num_entries=params.num_entries,
        interpolation_degree=params.interpolation_degree,
        entry_size_multiple=params.entry_size_multiple)


@pytest.mark.parametrize("cb,log_q,db_dtype,condensed,threads", [
    (32, 32, np.uint16, False, 1),
    (64, 52, np.uint16, True, 1),
    (64, 52, np.uint16, True, 3),
    (64, 52, np.uint8, True, 2),
    (64, 52, np.uint16, False, 1),
])
@pytest.mark.parametrize("mode", [orc.MODE_FP64, orc.MODE_EXACT])
def test_staged_timing_build_equals_checker(cb, log_q, db_dtype, condensed,
                                            threads, mode):
    params = synthetic.make_params(d=256, n=4096, t=4, l=2, coeff_bits=cb,
                                   log_q=log_q)
    mat = synthetic.make_material(params, seed=cb + threads, db_dtype=db_dtype,
                                  pad_to=64)
    fd, sd, pk = synthetic.make_requests(params, 1, seed=3, full_range=True)
    op = _op(params)
    want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                mat.t_vec_h, mat.second_dim_a, fd[0], sd[0],
                                pk[0], mode=mode)
    for library in (orc.timing_lib(), orc.lib()):
        got, stages = orc.process_response_staged(
            op, mat.db, mat.pack, mat.a_tilde_agg, mat.t_vec_h,
            mat.second_dim_a, fd[0], sd[0], pk[0], mode=mode, threads=threads,
            condensed_db=condensed, library=library)
        assert np.array_equal(got, want)
        assert set(stages) == {"db_mult_ms", "packing_ms", "poly_eval_ms"}
        assert all(v >= 0 for v in stages.values())
