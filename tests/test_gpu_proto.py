"""PirPreprocessedData in protobuf form straight to and from the GPU server
(crypto/pir/server/pir_preprocessed_data.h:52-267).

Files written by the oracle's wire-format restatement (itself checked
against the protobuf runtime in test_proto_format_cpu.py) load into a server
that answers as the oracle does on the same material; saving a loaded server
gives back the same bytes, as one message and in the directory form; bad
inputs give the reference's messages.
"""
import numpy as np
import pytest

from inspire_gb300 import pir, synthetic
from oracle import proto_format as pf
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu

CASES = [
    # (coeff_bits, log_q, d, n, t, l, pad, mat dtype, DB condensed, mat condensed)
    (32, 32, 256, 4 * 512, 4, 2, 1, np.int32, False, True),
    (64, 52, 128, 2 * 1000, 2, 1, 32, np.int32, True, True),
    (64, 52, 64, 2 * 256, 2, 2, 32, np.int16, True, False),
]


def _oparams(p, mat):
    return orc.make_params(
        coeff_bits=p.rlwe.coeff_bits, log_degree=p.rlwe.degree.bit_length() - 1,
        log_modulus=p.rlwe.log_modulus,
        log_modulus1_after_switch=p.rlwe.log_modulus1_after_switch,
        log_modulus2_after_switch=p.rlwe.log_modulus2_after_switch,
        pack_log_digit=p.pack_gadget.log_digit,
        pack_num_digits=p.pack_gadget.num_digits,
        eval_log_digit=p.eval_gadget.log_digit,
        eval_num_digits=p.eval_gadget.num_digits, num_entries=p.num_entries,
        interpolation_degree=p.interpolation_degree,
        entry_size_multiple=p.entry_size_multiple)


def _case(case, seed=1):
    cb, lq, d, n, t, l, pad, mdt, dcond, mcond = case
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=cb, log_q=lq,
                                   pack=(19, 2) if mdt == np.int32 else (13, 2))
    mat = synthetic.make_material(params, seed=seed, pad_to=pad, mat_dtype=mdt)
    k = params.pack_gadget.num_digits
    dbs = [mat.db[s * t * d:(s + 1) * t * d] for s in range(l)]
    outs = [[(mat.a_tilde_agg[s * t + i], mat.pack[(s * t + i) * d:(s * t + i + 1) * d],
              mat.t_vec_h[(s * t + i) * k:(s * t + i + 1) * k]) for i in range(t)]
            for s in range(l)]
    return params, mat, dbs, outs


@pytest.mark.parametrize("case", CASES)
def test_loaded_server_answers_and_saves_the_same_bytes(case, tmp_path):
    cb, lq, d, n, t, l, pad, mdt, dcond, mcond = case
    params, mat, dbs, outs = _case(case)
    buf = pf.preprocessed_data(dbs, dcond, outs, mcond,
                               mat.second_dim_a if t > 1 else None, lq)
    srv = pir.PirServer.FromPirPreprocessedData(params, buf, np.uint16, mdt)
    fd, sd, pk = synthetic.make_requests(params, 3, seed=5)
    got = srv.process_arrays(fd, sd, pk)
    op = _oparams(params, mdt)
    for i in range(3):
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i],
                                    sd[i], pk[i])
        assert np.array_equal(got[i], want), i
    assert srv.SerializePirPreprocessedData() == buf
    # The directory form: metadata.bin + shard_<i>.bin.
    srv.SavePirPreprocessedDataToDirectory(tmp_path)
    assert (tmp_path / "metadata.bin").read_bytes() == pf.metadata_message(
        mat.second_dim_a if t > 1 else None, lq)
    for s in range(l):
        assert (tmp_path / ("shard_%d.bin" % s)).read_bytes() == pf.shard_message(
            dbs[s], dcond, outs[s], mcond, lq)
    again = pir.PirServer.FromPirPreprocessedDataDirectory(params, tmp_path,
                                                           np.uint16, mdt)
    assert np.array_equal(again.process_arrays(fd, sd, pk), got)


def test_created_server_serializes_as_the_reference_would():
    # A server made by Create from u32 material: plain DB, condensed int32
    # matrices (BuildPreprocessMatrix condenses int32).
    case = CASES[0]
    params, mat, dbs, outs = _case(case, seed=3)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack, mat.a_tilde_agg,
                                       mat.t_vec_h, mat.second_dim_a)
    assert srv.SerializePirPreprocessedData() == pf.preprocessed_data(
        dbs, False, outs, True, mat.second_dim_a, case[1])


def test_bad_messages():
    case = CASES[0]
    params, mat, dbs, outs = _case(case)
    buf = pf.preprocessed_data(dbs, False, outs, True, mat.second_dim_a, 32)
    with pytest.raises(pir.InspireError, match="Failed to parse"):
        pir.PirServer.FromPirPreprocessedData(params, buf[:len(buf) // 3])
    bad_poly = pf._bytes_field(1, b"\x01\x02")
    short = pf.preprocessed_data(dbs, False, outs, True, None, 32) + \
        pf._bytes_field(3, bad_poly)
    with pytest.raises(pir.InspireError, match="Unexpected serialized size"):
        pir.PirServer.FromPirPreprocessedData(params, short)
    # A condensed flag on a matrix that carries plain data.
    m = pf._bytes_field(1, np.zeros(8, np.uint16).tobytes()) + pf._int_field(3, 1) + \
        pf._int_field(4, 8) + pf._int_field(5, 1) + pf._int_field(6, 8)
    with pytest.raises(pir.InspireError, match="Condensed matrix cannot have normal data"):
        pir.PirServer.FromPirPreprocessedData(params, pf._bytes_field(1, m))
