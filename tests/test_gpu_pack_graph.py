"""The packing step of a batch, the batched ExternalProduct and CUDA-graph
replay of the device entry points, against the CPU oracle.

The packing step follows the packing benchmark's server loop
(crypto/pir/benchmarking/pir_packing_metrics_tool.cc:226-283): products, then
FinalizeMatrixPack per shard (crypto/lwes_to_rlwe.cc:448-479) with no
EvalPoly and no modulus switch.
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


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


def _dev(x):
    dt = {4: np.int32, 8: np.int64}[x.dtype.itemsize]
    return torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()


def _host(t, cdt):
    return t.cpu().numpy().view(cdt)


def oracle_pack(params, mat, fd, pk):
    """(l*t, 2, d) packed ciphertexts of one request, from the oracle."""
    op = oparams(params)
    cb = params.rlwe.coeff_bits
    d, k = params.rlwe.degree, params.pack_gadget.num_digits
    cdt = params.coeff_dtype
    q1 = np.zeros(mat.db.shape[1], dtype=cdt)
    q1[:fd.shape[0]] = fd
    bprime = orc.matrix_multiply(mat.db, q1, cb)
    partial = orc.matrix_multiply(mat.pack, pk[:k].reshape(-1), cb)
    shards = mat.db.shape[0] // d
    out = np.zeros((shards, 2, d), dtype=cdt)
    for s in range(shards):
        out[s, 0] = mat.a_tilde_agg[s]
        out[s, 1] = orc.finalize_matrix_pack(
            op, bprime[s * d:(s + 1) * d], partial[s * d:(s + 1) * d],
            pk[k:], mat.t_vec_h[s * k:(s + 1) * k])
    return out


def _server(params, mat):
    return pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        mat.second_dim_a)


@pytest.mark.parametrize("engine", [pir.ENGINE_PLAIN, pir.ENGINE_TENSOR])
@pytest.mark.parametrize("d,n,t,l,batch", [
    (2048, 2048, 1, 1, 3),    # the packing benchmark's shape (t = 1)
    (256, 4096, 2, 2, 5),     # several shards per request
])
def test_pack_batch_matches_oracle(engine, d, n, t, l, batch):
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=32)
    mat = synthetic.make_material(params, seed=d + batch)
    srv = _server(params, mat)
    fd, _, pk = synthetic.make_requests(params, batch, seed=batch)
    out = torch.zeros((batch, l * t, 2, d), dtype=torch.int32, device="cuda")
    t_fd, t_pk = _dev(fd), _dev(pk)
    stream = torch.cuda.current_stream().cuda_stream
    try:
        srv.pack_device(batch, t_fd.data_ptr(), fd.shape[1], t_pk.data_ptr(),
                        pk.shape[1], out.data_ptr(), engine, stream)
    except pir.InspireError as e:
        assert engine == pir.ENGINE_TENSOR and e.code == pir.FAILED_PRECONDITION
        pytest.skip("tensor engine needs rows % 256 == 0")
    torch.cuda.synchronize()
    got = _host(out, np.uint32)
    for i in sorted({0, batch - 1}):
        assert np.array_equal(got[i], oracle_pack(params, mat, fd[i], pk[i])), i


@pytest.mark.parametrize("cb,log_q,d,batch", [
    (32, 32, 2048, 4), (32, 32, 4096, 4), (64, 52, 2048, 4),
    # Enough ciphertexts for the radix-16 block-per-ciphertext kernel (one
    # per SM, two at d = 2048).
    (32, 32, 2048, 320), (64, 52, 4096, 160), (32, 32, 8192, 152)])
def test_external_product_batch_matches_oracle(cb, log_q, d, batch):
    params = synthetic.make_params(d=d, n=2 * d, t=2, coeff_bits=cb,
                                   log_q=log_q)
    mat = synthetic.make_material(params, seed=3, pad_to=32 if cb == 64 else 1)
    srv = _server(params, mat)
    ne = params.eval_gadget.num_digits
    cdt = params.coeff_dtype
    rng = np.random.default_rng(d + cb)
    hi = (1 << log_q) - 1
    ct = rng.integers(0, hi, size=(batch, 2, d), dtype=cdt, endpoint=True)
    rgsw = rng.integers(0, hi, size=(batch, 2 * ne, 2, d), dtype=cdt,
                        endpoint=True)
    t_ct, t_rg = _dev(ct), _dev(rgsw)
    out = torch.zeros_like(t_ct)
    srv.external_product_device(batch, t_ct.data_ptr(), t_rg.data_ptr(),
                                out.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = _host(out, cdt)
    op = oparams(params)
    for i in sorted({0, 1, 2, batch - 1}):
        wa, wb = orc.external_product(op, ct[i, 0], ct[i, 1],
                                      rgsw[i].reshape(-1, d))
        assert np.array_equal(got[i, 0], wa), i
        assert np.array_equal(got[i, 1], wb), i
    # The batched call equals the single-ciphertext component call.
    a1, b1 = pir.external_product(params, ct[1, 0], ct[1, 1],
                                  rgsw[1].reshape(-1, d))
    assert np.array_equal(got[1, 0], a1) and np.array_equal(got[1, 1], b1)


@pytest.mark.parametrize("engine", [pir.ENGINE_PLAIN, pir.ENGINE_TENSOR])
def test_graph_replay_of_answer_matches_direct_calls(engine):
    params = synthetic.make_params(d=256, n=4 * 8192, t=4, coeff_bits=32)
    mat = synthetic.make_material(params, seed=5)
    srv = _server(params, mat)
    batch = 9
    fd, sd, pk = synthetic.make_requests(params, batch, seed=6)
    t_fd, t_sd, t_pk = _dev(fd), _dev(sd), _dev(pk)
    out = torch.zeros((batch, 1, 2, 256), dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    def call():
        srv.process_device(batch, t_fd.data_ptr(), fd.shape[1],
                           t_sd.data_ptr(), sd.shape[1], t_pk.data_ptr(),
                           pk.shape[1], out.data_ptr(), engine, sp)

    call()                       # allocates the workspace outside the capture
    stream.synchronize()
    with pir.Graph(sp) as g:
        call()
    # Replays read whatever the bound buffers hold at launch time.
    for seed in (7, 8):
        fd2, sd2, pk2 = synthetic.make_requests(params, batch, seed=seed)
        t_fd.copy_(_dev(fd2))
        t_sd.copy_(_dev(sd2))
        t_pk.copy_(_dev(pk2))
        torch.cuda.synchronize()
        out.zero_()
        torch.cuda.synchronize()
        g.launch(sp)
        stream.synchronize()
        srv.check()
        want = srv.process_arrays(fd2, sd2, pk2, pir.ENGINE_PLAIN)
        assert np.array_equal(_host(out, np.uint32), want)


def test_graph_of_pack_then_external_product():
    # The packing micro-workload shape: t = 1, d = 2048, pack 19 x 2, then
    # one ExternalProduct (eval 19 x 3) of each packed ciphertext.
    d = 2048
    params = synthetic.make_params(d=d, n=2048, t=1, coeff_bits=32)
    mat = synthetic.make_material(params, seed=11)
    srv = _server(params, mat)
    batch = 6
    ne = params.eval_gadget.num_digits
    fd, _, pk = synthetic.make_requests(params, batch, seed=12)
    rng = np.random.default_rng(13)
    rgsw = rng.integers(0, 1 << 32, size=(batch, 2 * ne, 2, d),
                        dtype=np.uint64).astype(np.uint32)
    t_fd, t_pk, t_rg = _dev(fd), _dev(pk), _dev(rgsw)
    packed = torch.zeros((batch, 1, 2, d), dtype=torch.int32, device="cuda")
    ext = torch.zeros((batch, 2, d), dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    def step():
        srv.pack_device(batch, t_fd.data_ptr(), fd.shape[1], t_pk.data_ptr(),
                        pk.shape[1], packed.data_ptr(), pir.ENGINE_PLAIN, sp)
        srv.external_product_device(batch, packed.data_ptr(), t_rg.data_ptr(),
                                    ext.data_ptr(), sp)

    step()
    stream.synchronize()
    with pir.Graph(sp) as g:
        step()
    ext.zero_()
    torch.cuda.synchronize()
    g.launch(sp)
    stream.synchronize()
    got_p = _host(packed, np.uint32)
    got_e = _host(ext, np.uint32)
    op = oparams(params)
    for i in (0, batch - 1):
        want = oracle_pack(params, mat, fd[i], pk[i])
        assert np.array_equal(got_p[i], want)
        wa, wb = orc.external_product(op, want[0, 0], want[0, 1],
                                      rgsw[i].reshape(-1, d))
        assert np.array_equal(got_e[i, 0], wa)
        assert np.array_equal(got_e[i, 1], wb)


def test_graph_begin_rejects_default_stream():
    with pytest.raises(pir.InspireError, match="created stream"):
        with pir.Graph(0):
            pass
