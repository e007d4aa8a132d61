"""Bit-exact parity with the oracle at the full sizes of the benchmarked
workloads (PirServer::ProcessResponse, crypto/pir/server/pir_server.cc:154-306).

The smaller parity tests cover every code path at shapes the oracle finishes
in milliseconds; these run the kernels in the configurations that are timed:

* n = 2^20, d = 4096, t = 8 over Z_2^32 (DB 32768 x 131072 u16, pack matrix
  32768 x 8192 i32): the tensor engine at B = 1, 8, 64 and 256 with the
  split-K factor its autotuner picks for that batch (atomic split-K sums,
  K-slice-major grid, 131072 DB columns), and the plain engine at B = 1;
* n = 65536, d = 2048, t = 4 over Z_2^32 (the single-request shape);
* the packing micro-workload: 256 instances of d = 2048 packing
  (FinalizeMatrixPack, crypto/lwes_to_rlwe.cc:448-479) followed by one
  ExternalProduct each (crypto/external_product.cc:35-114);
* n = 2^18, d = 8192, t = 2, l = 4 over Z_2^32 (DB 65536 x 131072 u16).

Each compares the first, a middle and the last response of a batch with the
oracle's exact product on the same bytes; the oracle requests run on several
host threads.
"""
import gc
import math
import threading

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


def big_material(params, seed):
    """Seeded material of the benchmark's shapes: DB values uniform in
    [0, p), pack entries with the reference's bound, the small
    polynomial parts from make_material."""
    d = params.rlwe.degree
    t, l = params.interpolation_degree, params.entry_size_multiple
    k = params.pack_gadget.num_digits
    rows, cols = l * t * d, params.InterpolatedRows()
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, seed)
    bound = int(4 * math.sqrt(d) * (1 << params.pack_gadget.log_digit))
    pack = synthetic.parallel_integers((rows, k * d), -bound + 1, bound,
                                       np.int32, seed + 1)
    small = synthetic.make_material(
        synthetic.make_params(d=d, n=d * t, t=t, l=l,
                              coeff_bits=params.rlwe.coeff_bits,
                              log_q=params.rlwe.log_modulus), seed=seed + 2)
    return synthetic.Material(db, pack, small.a_tilde_agg, small.t_vec_h,
                              small.second_dim_a)


def server(params, mat):
    return pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        mat.second_dim_a)


def check_with_oracle(params, mat, fd, sd, pk, got, picks):
    """Oracle responses for `picks`, one host thread each; returns the
    indices whose GPU response differs."""
    op = oparams(params)
    bad, errs = [], []

    def one(i):
        try:
            want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                        mat.t_vec_h, mat.second_dim_a, fd[i],
                                        sd[i], pk[i])
            if not np.array_equal(got[i].reshape(want.shape), want):
                bad.append(i)
        except Exception as e:
            errs.append(e)
    ts = [threading.Thread(target=one, args=(i,)) for i in picks]
    for th in ts:
        th.start()
    for th in ts:
        th.join()
    if errs:
        raise errs[0]
    return sorted(bad)


@pytest.fixture(scope="module")
def headline():
    params = synthetic.make_params(d=4096, n=1 << 20, t=8, coeff_bits=32)
    mat = big_material(params, 2026)
    srv = server(params, mat)
    yield params, mat, srv
    del srv
    gc.collect()


@pytest.mark.parametrize("batch", [1, 8, 64, 256])
def test_headline_tensor_engine_matches_oracle(headline, batch):
    params, mat, srv = headline
    split, _ = srv.autotune(batch)
    assert split >= 1
    fd, sd, pk = synthetic.make_requests(params, batch, seed=100 + batch,
                                         full_range=True)
    got = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
    srv.check()
    picks = sorted({0, batch // 2, batch - 1})
    assert check_with_oracle(params, mat, fd, sd, pk, got, picks) == []


def test_headline_plain_engine_matches_oracle(headline):
    params, mat, srv = headline
    fd, sd, pk = synthetic.make_requests(params, 2, seed=99)
    got = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert check_with_oracle(params, mat, fd, sd, pk, got, [0, 1]) == []
    # Both engines on the same requests.
    assert np.array_equal(got, srv.process_arrays(fd, sd, pk,
                                                  pir.ENGINE_TENSOR))


@pytest.mark.parametrize("engine,batch", [(pir.ENGINE_PLAIN, 1),
                                          (pir.ENGINE_PLAIN, 4),
                                          (pir.ENGINE_TENSOR, 16)])
def test_single_request_shape_matches_oracle(engine, batch):
    params = synthetic.make_params(d=2048, n=65536, t=4, coeff_bits=32)
    mat = synthetic.make_material(params, seed=71)
    srv = server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=72 + batch)
    got = srv.process_arrays(fd, sd, pk, engine)
    picks = sorted({0, batch // 2, batch - 1})
    assert check_with_oracle(params, mat, fd, sd, pk, got, picks) == []


@pytest.mark.parametrize("engine", [pir.ENGINE_PLAIN, pir.ENGINE_TENSOR])
def test_packing_workload_256_instances_matches_oracle(engine):
    d, batch = 2048, 256
    params = synthetic.make_params(d=d, n=2048, t=1, coeff_bits=32)
    mat = synthetic.make_material(params, seed=31)
    srv = server(params, mat)
    fd, _, pk = synthetic.make_requests(params, batch, seed=32)
    ne, k = params.eval_gadget.num_digits, params.pack_gadget.num_digits
    rgsw = synthetic.parallel_integers((batch, 2 * ne, 2, d), 0, 1 << 32,
                                       np.uint64, 33).astype(np.uint32)
    dev = torch.device("cuda", 0)
    t_fd = torch.from_numpy(fd.view(np.int32)).to(dev)
    t_pk = torch.from_numpy(pk.view(np.int32)).to(dev)
    t_rg = torch.from_numpy(rgsw.view(np.int32)).to(dev)
    packed = torch.zeros((batch, 1, 2, d), dtype=torch.int32, device=dev)
    ext = torch.zeros((batch, 2, d), dtype=torch.int32, device=dev)
    sp = torch.cuda.current_stream().cuda_stream
    srv.pack_device(batch, t_fd.data_ptr(), fd.shape[1], t_pk.data_ptr(),
                    pk.shape[1], packed.data_ptr(), engine, sp)
    srv.external_product_device(batch, packed.data_ptr(), t_rg.data_ptr(),
                                ext.data_ptr(), sp)
    torch.cuda.synchronize()
    got_pack = packed.cpu().numpy().view(np.uint32)
    got_ext = ext.cpu().numpy().view(np.uint32)
    op = oparams(params)
    q1 = np.zeros((batch, mat.db.shape[1]), dtype=np.uint32)
    q1[:, :fd.shape[1]] = fd
    for i in (0, batch // 2, batch - 1):
        bprime = orc.matrix_multiply(mat.db, q1[i], 32)
        partial = orc.matrix_multiply(mat.pack, pk[i, :k].reshape(-1), 32)
        b = orc.finalize_matrix_pack(op, bprime, partial, pk[i, k:],
                                     mat.t_vec_h[:k])
        assert np.array_equal(got_pack[i, 0, 0], mat.a_tilde_agg[0]), i
        assert np.array_equal(got_pack[i, 0, 1], b), i
        wa, wb = orc.external_product(op, mat.a_tilde_agg[0], b,
                                      rgsw[i].reshape(-1, d))
        assert np.array_equal(got_ext[i, 0], wa), i
        assert np.array_equal(got_ext[i, 1], wb), i


def test_largest_ring_degree_four_shards_matches_oracle():
    params = synthetic.make_params(d=8192, n=1 << 18, t=2, l=4, coeff_bits=32)
    mat = big_material(params, 2718)
    srv = server(params, mat)
    try:
        fd, sd, pk = synthetic.make_requests(params, 8, seed=5,
                                             full_range=True)
        got_t = srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR)
        srv.check()
        assert check_with_oracle(params, mat, fd, sd, pk, got_t,
                                 [0, 7]) == []
        got_p = srv.process_arrays(fd[:1], sd[:1], pk[:1], pir.ENGINE_PLAIN)
        assert np.array_equal(got_p[0], got_t[0])
    finally:
        del srv
        gc.collect()
