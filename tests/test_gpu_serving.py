"""The continuous-batching request loop: every response must be identical
whether its request was answered alone or batched with requests for several
databases of different shapes, while other batches were on the GPU."""
import threading

import numpy as np
import pytest

from inspire_gb300 import build, pir, serving, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def _db(d, n, t, l, seed, pad_to=1):
    params = synthetic.make_params(d=d, n=n, t=t, l=l, coeff_bits=32)
    mat = synthetic.make_material(params, seed=seed, pad_to=pad_to)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    return params, mat, srv


def test_mixed_batching_matches_alone():
    # Two databases of uneven shape: (d=256, t=2, l=2) and (d=128, t=4, l=1).
    pa, ma, sa = _db(256, 8192, 2, 2, seed=1)
    pb, mb, sb = _db(128, 16384, 4, 1, seed=2)
    reqs = {"A": synthetic.make_requests(pa, 40, seed=3),
            "B": synthetic.make_requests(pb, 40, seed=4)}
    # Alone: one request at a time through the synchronous call.
    alone = {name: [(sa if name == "A" else sb).process_arrays(
        fd[i:i + 1], sd[i:i + 1], pk[i:i + 1])[0] for i in range(fd.shape[0])]
        for name, (fd, sd, pk) in reqs.items()}
    # In the mix: two client threads submit interleaved requests for both
    # databases while earlier batches are in flight.
    # A 2 ms batching window groups the two clients' requests per database.
    with serving.ServingEngine({"A": sa, "B": sb}, max_batch=16,
                               max_workspaces=3, plain_max_batch=2,
                               max_wait_us=2000, hbm_budget=1 << 30) as eng:
        assert eng.queue_info("A")["workspaces"] == 3
        futs = {"A": [None] * 40, "B": [None] * 40}

        def client(name):
            fd, sd, pk = reqs[name]
            for i in range(fd.shape[0]):
                futs[name][i] = eng.submit(name, fd[i], sd[i], pk[i])

        ths = [threading.Thread(target=client, args=(n,)) for n in ("A", "B")]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        mixed = {n: [f.result(timeout=120) for f in futs[n]] for n in futs}
        stats = eng.stats()
    for name in ("A", "B"):
        for i in range(40):
            assert np.array_equal(mixed[name][i], alone[name][i]), (name, i)
    assert stats["requests"] == 80
    assert stats["mean_batch"] > 1.0            # requests were batched
    # One response of each database against the oracle.
    for name, params, mat in (("A", pa, ma), ("B", pb, mb)):
        fd, sd, pk = reqs[name]
        r = params.rlwe
        op = orc.make_params(
            coeff_bits=32, log_degree=r.degree.bit_length() - 1,
            log_modulus=r.log_modulus,
            log_modulus1_after_switch=r.log_modulus1_after_switch,
            log_modulus2_after_switch=r.log_modulus2_after_switch,
            pack_log_digit=19, pack_num_digits=2, eval_log_digit=19,
            eval_num_digits=3, num_entries=params.num_entries,
            interpolation_degree=params.interpolation_degree,
            entry_size_multiple=params.entry_size_multiple)
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[7],
                                    sd[7], pk[7])
        assert np.array_equal(mixed[name][7], want)


def test_full_batches_use_the_tensor_engine():
    pa, _, sa = _db(256, 32768, 2, 1, seed=5)
    fd, sd, pk = synthetic.make_requests(pa, 96, seed=6)
    want = sa.process_arrays(fd, sd, pk)
    with serving.ServingEngine({"A": sa}, max_batch=32, max_workspaces=3,
                               plain_max_batch=4, max_wait_us=3000) as eng:
        futs = [eng.submit("A", fd[i], sd[i], pk[i]) for i in range(96)]
        got = np.stack([f.result(timeout=120) for f in futs])
        stats = eng.stats()
    assert np.array_equal(got, want)
    assert stats["tensor_batches"] >= 1
    assert stats["requests"] == 96


def test_u64_server_in_the_mix_uses_the_tensor_engine():
    # A Z_2^64 server (q = 2^56, int32 pack matrix: eight request digit
    # planes on the tensor cores) beside a Z_2^32 one.
    pa, _, sa = _db(256, 32768, 2, 1, seed=11)
    p64 = synthetic.make_params(d=256, n=16384, t=2, coeff_bits=64, log_q=56)
    m64 = synthetic.make_material(p64, seed=12)
    s64 = pir.PirServer.CreateCombined(p64, m64.db, m64.pack, m64.a_tilde_agg,
                                       m64.t_vec_h, m64.second_dim_a)
    reqs = {"A": synthetic.make_requests(pa, 64, seed=13),
            "W": synthetic.make_requests(p64, 64, seed=14)}
    want = {"A": sa.process_arrays(*reqs["A"]), "W": s64.process_arrays(*reqs["W"])}
    with serving.ServingEngine({"A": sa, "W": s64}, max_batch=32, max_workspaces=2,
                               plain_max_batch=4, max_wait_us=3000) as eng:
        futs = {n: [eng.submit(n, r[0][i], r[1][i], r[2][i]) for i in range(64)]
                for n, r in reqs.items()}
        got = {n: np.stack([f.result(timeout=120) for f in fs]) for n, fs in futs.items()}
        stats = eng.stats()
    for n in ("A", "W"):
        assert got[n].dtype == want[n].dtype
        assert np.array_equal(got[n], want[n]), n
    assert stats["tensor_batches"] >= 1


def test_short_first_dimension_and_errors_in_the_mix():
    pa, ma, sa = _db(128, 2 * 4000, 2, 1, seed=8, pad_to=256)
    assert sa.db_cols == 4096
    fd, sd, pk = synthetic.make_requests(pa, 6, seed=9)
    alone = sa.process_arrays(fd, sd, pk)
    with serving.ServingEngine({"A": sa}, max_batch=4, max_workspaces=2) as eng:
        futs = [eng.submit("A", fd[i], sd[i], pk[i]) for i in range(6)]
        with pytest.raises(pir.InspireError, match="First dimension query size"):
            eng.submit("A", fd[0][:10], sd[0], pk[0])
        for i, f in enumerate(futs):
            assert np.array_equal(f.result(timeout=120), alone[i])


def test_hbm_budget_limits_workspaces():
    pa, _, sa = _db(128, 8192, 2, 1, seed=10)
    lib = pir._lib.load()
    per = lib.inspire_pir_workspace_bytes(sa._h, 64)
    with serving.ServingEngine({"A": sa, "B": sa}, max_batch=64,
                               hbm_budget=2 * per + per // 2,
                               max_workspaces=4) as eng:
        assert eng.queue_info("A")["workspaces"] == 1
        assert eng.queue_info("A")["workspace_bytes"] == per
    with serving.ServingEngine({"A": sa}, max_batch=64, hbm_budget=10 * per,
                               max_workspaces=4) as eng:
        assert eng.queue_info("A")["workspaces"] == 4


def test_workspace_bytes_scale_with_batch():
    pa, _, sa = _db(128, 8192, 2, 1, seed=7)
    lib = pir._lib.load()
    b1 = lib.inspire_pir_workspace_bytes(sa._h, 1)
    b64 = lib.inspire_pir_workspace_bytes(sa._h, 64)
    assert 0 < b1 < b64
