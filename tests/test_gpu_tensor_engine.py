"""The batched tensor-core engine (8-bit digits on tcgen05) against the plain
engine, exact integer products and the CPU oracle. Both engines must give
identical responses.

The adversarial cases pick operands whose balanced base-256 digits are all
at the ends of their range (-128, 127 and, for DB digits, 128), so the fp32
partial sums of an exact accumulation unit reach about +-2^22, the largest
the digit plan allows: an inexact accumulation or decode would show up as a
mismatch.
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
    (256, 16000, 4, 7),      # C = 4000: columns padded to a multiple of 128
    (1024, 32768, 4, 130),   # three request tiles
    (8192, 2 * 4096, 2, 3),  # the largest ring degree (R = 16384)
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


def _from_digits(digits):
    """The u32 word whose balanced base-256 digits are `digits` (low first)."""
    return sum(int(d) << (8 * i) for i, d in enumerate(digits)) % (1 << 32)


@pytest.mark.parametrize("pattern", ["alternating", "random_extremes"])
def test_tensor_extreme_signed_digits(pattern):
    # The engine splits query and pack words into balanced digits in
    # [-128, 127] and DB entries as x - 2^15 into x0 in [-128, 127],
    # x1 in [-128, 128]. These inputs drive the per-unit fp32 partial sums to
    # their extremes, about +-2^22, with both signs.
    params = synthetic.make_params(d=128, n=2 * 16384, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=13, mat_dtype=np.int32)
    rng = np.random.default_rng(14)
    fd, sd, pk = synthetic.make_requests(params, 64, seed=15, full_range=True)
    if pattern == "alternating":
        mat.db[:] = 65408                       # x0 = -128, x1 = 128
        mat.pack[:] = np.array([_from_digits([-128, 127, -128, 127])],
                               dtype=np.uint32).view(np.int32)[0]
        fd[:] = _from_digits([127, -128, 127, -128])
        pk[:] = _from_digits([127, -128, 127, -128])
    else:
        # DB values whose digit pairs are extreme: (-128, 128), (127, -128),
        # (0, -128), (-1, 128).
        mat.db[:] = rng.choice(np.array([65408, 127, 0, 65535], np.uint16),
                               size=mat.db.shape)
        words = np.array([_from_digits(rng.choice([-128, 127], size=4))
                          for _ in range(256)], dtype=np.uint32)
        mat.pack[:] = rng.choice(words, size=mat.pack.shape).view(np.int32)
        fd[:] = rng.choice(words, size=fd.shape)
        pk[:] = rng.choice(words, size=pk.shape)
    srv = _server(params, mat)
    got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    got_p = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(got_t, got_p)
    want = orc.process_response(oparams(params), mat.db, mat.pack,
                                mat.a_tilde_agg, mat.t_vec_h,
                                mat.second_dim_a, fd[5], sd[5], pk[5])
    assert np.array_equal(got_t[5], want)


def test_tensor_products_match_exact_integer_gemm():
    # Stage 1 alone against numpy's exact integer products mod 2^32.
    import torch
    params = synthetic.make_params(d=128, n=2 * 4096, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=17, mat_dtype=np.int32)
    fd, sd, pk = synthetic.make_requests(params, 70, seed=18, full_range=True)
    srv = _server(params, mat)
    rows = mat.db.shape[0]
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(np.int32)).to(dev)
    t_pk = torch.from_numpy(pk.view(np.int32)).to(dev)
    out = torch.zeros((70, rows), dtype=torch.int32, device=dev)
    lib = pir._lib.load()
    err = pir._errbuf()
    rc = lib.inspire_pir_products_device(
        srv._h, 70, t_fd.data_ptr(), t_pk.data_ptr(), out.data_ptr(),
        pir.ENGINE_TENSOR, None, err, len(err))
    assert rc == 0, err.value
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    k = params.pack_gadget.num_digits
    yg = pk[:, :k].reshape(70, -1).astype(np.uint64)
    db = mat.db.astype(np.uint64)
    pack = mat.pack.astype(np.int64).astype(np.uint64)
    m = np.uint64(0xFFFFFFFF)
    for q in (0, 33, 69):
        want = ((db @ (fd[q].astype(np.uint64) & m)) & m) + \
               ((pack @ yg[q]) & m)
        assert np.array_equal(got[q], (want & m).astype(np.uint32)), q


@pytest.mark.parametrize("batch", [128, 192, 256])
def test_tensor_request_tile_counts(batch):
    # 2, 3 and 4 request tiles per row pair; each tile's CTA issues its own
    # TMA loads of the DB / pack tiles (no multicast).
    params = synthetic.make_params(d=128, n=2 * 8192, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=batch)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=batch + 1,
                                         full_range=True)
    got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    got_p = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(got_t, got_p)
    srv.check()


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


def test_autotuned_split_keeps_responses_identical():
    params = synthetic.make_params(d=256, n=4 * 16384, t=4, coeff_bits=32)
    mat = synthetic.make_material(params, seed=21)
    srv = _server(params, mat)
    split, ms = srv.autotune(100)
    assert split >= 1 and ms > 0
    fd, sd, pk = synthetic.make_requests(params, 100, seed=22, full_range=True)
    assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR),
                          srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN))


def test_tensor_engine_unavailable_for_full_width_pack_words():
    # Over Z_2^64 the engine takes int16 / int32 pack matrices (four digits
    # whose sum is the entry); full u64 words would need eight.
    params = synthetic.make_params(d=128, n=8192, t=2, coeff_bits=64, log_q=52)
    mat = synthetic.make_material(params, seed=1, pad_to=32, mat_dtype=np.uint64)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, 1)
    with pytest.raises(pir.InspireError, match="tensor engine unavailable"):
        srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    with pytest.raises(pir.InspireError, match="tensor engine unavailable"):
        srv.autotune(8)
