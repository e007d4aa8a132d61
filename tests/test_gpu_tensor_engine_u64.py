"""The tensor-core engine over Z_2^64: request words split into eight
balanced base-256 digit planes (32 requests per tile), pack entries into
four digits whose sum is the signed entry itself, the 64-bit epilogue.
Checked against the plain engine, exact integer products mod 2^64 and the
CPU oracle (crypto/pir/server/pir_server.cc:154-306 with CoeffType =
uint64_t).

The extreme cases drive every digit to the ends of its range so that the
fp32 partial sums of one accumulation unit reach about +-2^22, and pick
int32 pack entries at -2^31 and 2^31 - 1, whose top digit is -128 or 128.
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


def _check(params, mat, fd, sd, pk, picks):
    srv = _server(params, mat)
    got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    got_p = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert got_t.dtype == np.uint64
    assert np.array_equal(got_t, got_p)
    op = oparams(params)
    for i in picks:
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i],
                                    sd[i], pk[i])
        assert np.array_equal(got_t[i], want), i
    srv.check()
    return srv


@pytest.mark.parametrize("d,n,t,batch,log_q,mdt", [
    (128, 8192, 2, 1, 64, np.int32),       # R = 256, one request
    (128, 8192, 2, 32, 64, np.int32),      # one full request tile
    (128, 8192, 2, 33, 52, np.int32),      # a ragged second tile, q = 2^52
    (256, 16000, 4, 7, 56, np.int16),      # C = 4000 padded; int16 pack
    (1024, 32768, 4, 70, 64, np.int32),    # three request tiles
    (2048, 2 * 4096, 2, 5, 56, np.int32),  # R = 4096
])
def test_u64_tensor_matches_plain_and_oracle(d, n, t, batch, log_q, mdt):
    params = synthetic.make_params(d=d, n=n, t=t, coeff_bits=64, log_q=log_q,
                                   pack=(19, 2) if mdt == np.int32 else (13, 2))
    mat = synthetic.make_material(params, seed=d + batch, mat_dtype=mdt)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=batch,
                                         full_range=True)
    _check(params, mat, fd, sd, pk, sorted({0, batch - 1}))


def _from_digits(digits):
    """The u64 word whose balanced base-256 digits are `digits` (low first)."""
    return sum(int(d) << (8 * i) for i, d in enumerate(digits)) % (1 << 64)


@pytest.mark.parametrize("log_q", [64, 56])
@pytest.mark.parametrize("pattern", ["alternating", "random_extremes"])
def test_u64_tensor_extreme_digits(pattern, log_q):
    # log_q = 56: the engine computes seven weight blocks (the products
    # mod 2^56 that FinalizeMatrixPack reads), with the same extremes.
    params = synthetic.make_params(d=128, n=2 * 16384, t=2, coeff_bits=64,
                                   log_q=log_q)
    mat = synthetic.make_material(params, seed=13, mat_dtype=np.int32)
    rng = np.random.default_rng(14)
    fd, sd, pk = synthetic.make_requests(params, 32, seed=15, full_range=True)
    if pattern == "alternating":
        mat.db[:] = 65408                       # x0 = -128, x1 = 128
        mat.pack[:] = np.int32(-2**31)          # digits 0, 0, 0, -128
        fd[:] = _from_digits([127, -128] * 4)
        pk[:] = _from_digits([-128, 127] * 4)
    else:
        mat.db[:] = rng.choice(np.array([65408, 127, 0, 65535], np.uint16),
                               size=mat.db.shape)
        # int32 entries with extreme digits, and both ends of the range
        # (2^31 - 1 has the digits -1, 0, 0, 128).
        ends = [_from_digits(rng.choice([-128, 127], size=4)) for _ in range(254)]
        ends = np.array(ends, dtype=np.uint64).astype(np.uint32).view(np.int32)
        vals = np.concatenate([ends, np.array([-2**31, 2**31 - 1], np.int32)])
        mat.pack[:] = rng.choice(vals, size=mat.pack.shape)
        words = np.array([_from_digits(rng.choice([-128, 127], size=8))
                          for _ in range(256)], dtype=np.uint64)
        fd[:] = rng.choice(words, size=fd.shape)
        pk[:] = rng.choice(words, size=pk.shape)
    _check(params, mat, fd, sd, pk, [0, 17, 31])


def test_u64_tensor_products_match_exact_integer_gemm():
    # Stage 1 alone against numpy's integer products, which wrap mod 2^64.
    import torch
    params = synthetic.make_params(d=128, n=2 * 4096, t=2, coeff_bits=64)
    mat = synthetic.make_material(params, seed=17, mat_dtype=np.int32)
    batch = 45
    fd, sd, pk = synthetic.make_requests(params, batch, seed=18, full_range=True)
    srv = _server(params, mat)
    rows = mat.db.shape[0]
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(np.int64)).to(dev)
    t_pk = torch.from_numpy(pk.view(np.int64)).to(dev)
    out = torch.zeros((batch, rows), dtype=torch.int64, device=dev)
    lib = pir._lib.load()
    err = pir._errbuf()
    rc = lib.inspire_pir_products_device(
        srv._h, batch, t_fd.data_ptr(), t_pk.data_ptr(), out.data_ptr(),
        pir.ENGINE_TENSOR, None, err, len(err))
    assert rc == 0, err.value
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint64)
    k = params.pack_gadget.num_digits
    yg = pk[:, :k].reshape(batch, -1)
    db = mat.db.astype(np.uint64)
    pack = mat.pack.astype(np.int64).view(np.uint64)
    with np.errstate(over="ignore"):
        for q in (0, 31, 32, 44):
            want = db @ fd[q] + pack @ yg[q]
            assert np.array_equal(got[q], want), q


def test_u64_split_k_and_buffer_reuse():
    params = synthetic.make_params(d=256, n=4 * 16384, t=4, coeff_bits=64,
                                   log_q=56)
    mat = synthetic.make_material(params, seed=21)
    srv = _server(params, mat)
    split, ms = srv.autotune(100)
    assert split >= 1 and ms > 0
    for batch in (100, 3, 32, 1):
        fd, sd, pk = synthetic.make_requests(params, batch, seed=batch + 22,
                                             full_range=True)
        assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR),
                              srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN))
    srv.check()


@pytest.mark.parametrize("log_q", [56, 52])
def test_u64_tensor_products_mod_2_56_when_q_is_at_most_2_56(log_q):
    # With q <= 2^56 the answer reads the stage-1 words mod 2^56 only, and
    # the tensor engine skips the digit position of weight 2^56: its words
    # equal the plain engine's mod 2^56; the forms API still computes all
    # eight positions (exact mod 2^64).
    import torch
    params = synthetic.make_params(d=128, n=2 * 4096, t=2, coeff_bits=64,
                                   log_q=log_q)
    mat = synthetic.make_material(params, seed=19, mat_dtype=np.int32)
    batch = 40
    fd, sd, pk = synthetic.make_requests(params, batch, seed=20, full_range=True)
    srv = _server(params, mat)
    rows = mat.db.shape[0]
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(np.int64)).to(dev)
    t_pk = torch.from_numpy(pk.view(np.int64)).to(dev)
    lib = pir._lib.load()
    err = pir._errbuf()

    def products(engine):
        out = torch.zeros((batch, rows), dtype=torch.int64, device=dev)
        rc = lib.inspire_pir_products_device(
            srv._h, batch, t_fd.data_ptr(), t_pk.data_ptr(), out.data_ptr(),
            engine, None, err, len(err))
        assert rc == 0, err.value
        torch.cuda.synchronize()
        return out.cpu().numpy().view(np.uint64)
    plain = products(pir.ENGINE_PLAIN)
    tensor = products(pir.ENGINE_TENSOR)
    low = np.uint64((1 << 56) - 1)
    assert np.array_equal(tensor & low, plain & low)
    out = torch.zeros((batch, rows), dtype=torch.int64, device=dev)
    srv.tensor_products_device(batch, t_fd.data_ptr(), t_pk.data_ptr(),
                               out.data_ptr(), pir.FORM_PLANES)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), plain)
    srv.check()
