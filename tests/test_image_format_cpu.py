"""The oracle's restatement of the PirServer file image, on the CPU.

Bit order and field layout follow crypto/pir/server/pir_server.cc:310-780;
the round trip below is the property the reference's save/load test checks
(pir_server_test.cc:527-679: a loaded server answers like the original).
"""
import numpy as np

from oracle import image_format as img
from inspire_gb300 import synthetic


def test_bitpack_known_bytes():
    # -1 and 2 in 3 bits, least-significant bit first: 111 010 -> 0x17.
    assert img.bitpack(np.array([-1, 2]), 3) == bytes([0x17])
    got = img.bitunpack(bytes([0x17]), 2, 3, signed=True)
    assert got.tolist() == [-1, 2]
    assert img.bitunpack(bytes([0x17]), 2, 3, signed=False).tolist() == [7, 2]


def test_bitpack_round_trip_random():
    rng = np.random.default_rng(1)
    for bits in (1, 7, 19, 31, 33, 52, 63):
        lo = -(1 << (bits - 1))
        v = rng.integers(lo, -lo, size=257)
        assert np.array_equal(img.bitunpack(img.bitpack(v, bits), 257, bits,
                                            True), v)


def test_image_round_trip_u32_and_u64():
    for cb, log_q, pad in ((32, 32, 1), (64, 52, 32)):
        params = synthetic.make_params(d=64, n=2 * 1000, t=2, l=2,
                                       coeff_bits=cb, log_q=log_q)
        mat = synthetic.make_material(params, seed=cb, pad_to=pad)
        buf = img.save_image(64, cb, log_q, 19, mat.db, mat.pack,
                             mat.a_tilde_agg, mat.t_vec_h, mat.second_dim_a,
                             t=2, l=2, db_orig_cols=1000,
                             db_condensed=(cb == 64), pack_condensed=True)
        got = img.load_image(buf, np.uint16, np.int32, cb)
        assert np.array_equal(got["db"], mat.db)
        assert np.array_equal(got["pack"], mat.pack)
        assert got["db_orig_cols"] == 1000
        mask = (1 << log_q) - 1
        for key in ("a_tilde_agg", "t_vec_h", "second_dim_a"):
            want = getattr(mat, key).astype(np.uint64) & np.uint64(mask)
            assert np.array_equal(got[key].astype(np.uint64), want), key
