"""PirServer file images on the GPU: LoadFromBuffer / LoadFromFile /
SaveToFile (crypto/pir/server/pir_server.cc:434-791).

Images come from the oracle's restatement of the writer
(oracle/image_format.py); a loaded server must answer exactly as the oracle
does on the material the reference's loader reconstructs
(pir_server_test.cc:527-679 checks that a loaded server answers like the
original), and saving a loaded server must give back the same bytes.
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import image_format as img
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


CASES = [
    # (coeff_bits, log_q, d, n, t, l, pad, mat dtype, condensed DB)
    (32, 32, 256, 4 * 512, 4, 2, 1, np.int32, False),
    (64, 52, 128, 2 * 1000, 2, 1, 32, np.int32, True),
    (64, 52, 64, 2 * 256, 2, 2, 32, np.int16, True),
]


def _image(case, seed=1):
    cb, lq, d, n, t, l, pad, mdt, cond = case
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=cb, log_q=lq,
                                   pack=(19, 2) if mdt == np.int32 else (13, 2))
    mat = synthetic.make_material(params, seed=seed, pad_to=pad, mat_dtype=mdt)
    buf = img.save_image(d, cb, lq, params.pack_gadget.log_digit, mat.db,
                         mat.pack, mat.a_tilde_agg, mat.t_vec_h,
                         mat.second_dim_a, t=t, l=l, db_orig_cols=n // t,
                         db_condensed=cond, pack_condensed=True)
    return params, mat, buf


@pytest.mark.parametrize("case", CASES)
def test_loaded_server_answers_like_the_oracle(case):
    params, mat, buf = _image(case)
    srv = pir.PirServer.LoadFromBuffer(params, buf, np.uint16, case[7])
    loaded = img.load_image(buf, np.uint16, case[7], case[0])
    fd, sd, pk = synthetic.make_requests(params, 3, seed=5)
    got = srv.process_arrays(fd, sd, pk)
    op = oparams(params)
    for i in range(3):
        want = orc.process_response(op, loaded["db"], loaded["pack"],
                                    loaded["a_tilde_agg"], loaded["t_vec_h"],
                                    loaded["second_dim_a"], fd[i], sd[i], pk[i])
        assert np.array_equal(got[i], want), i


@pytest.mark.parametrize("case", CASES)
def test_save_of_a_loaded_server_gives_the_same_bytes(case, tmp_path):
    params, _, buf = _image(case, seed=2)
    srv = pir.PirServer.LoadFromBuffer(params, buf, np.uint16, case[7])
    assert srv.SaveToBuffer() == buf
    path = tmp_path / "server.img"
    srv.SaveToFile(path)
    assert path.read_bytes() == buf
    again = pir.PirServer.LoadFromFile(params, path, np.uint16, case[7])
    fd, sd, pk = synthetic.make_requests(params, 2, seed=6)
    assert np.array_equal(again.process_arrays(fd, sd, pk),
                          srv.process_arrays(fd, sd, pk))


def test_saved_image_of_a_created_server_reads_back():
    params = synthetic.make_params(d=128, n=2 * 512, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=9)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    got = img.load_image(srv.SaveToBuffer(), np.uint16, np.int32, 32)
    assert np.array_equal(got["db"], mat.db)
    assert np.array_equal(got["pack"], mat.pack)
    assert np.array_equal(got["a_tilde_agg"], mat.a_tilde_agg)
    assert np.array_equal(got["t_vec_h"], mat.t_vec_h)
    assert np.array_equal(got["second_dim_a"], mat.second_dim_a)
    assert got["pack_bits"] == 19 + 7


def test_truncated_image_and_missing_file():
    params, _, buf = _image(CASES[0])
    with pytest.raises(pir.InspireError, match="Error reading from buffer"):
        pir.PirServer.LoadFromBuffer(params, buf[:len(buf) // 2])
    with pytest.raises(pir.InspireError, match="Failed to read file"):
        pir.PirServer.LoadFromFile(params, "/nonexistent/server.img")
