"""Scheduling logic of the continuous-batching loop, on the CPU.

A fake workspace stands in for the GPU one: it "answers" a batch with a
deterministic function of each request and finishes after a delay, so the
test can check batching, per-database FIFO order, HBM admission (in-flight
slot counts), result routing and error propagation without a GPU.
"""
import threading
import time
from types import SimpleNamespace

import numpy as np
import pytest

from inspire_gb300 import pir, serving, synthetic


class FakeWorkspace:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, db, max_batch):
        self.db = db
        self.items = []
        self.t_ready = 0.0
        self.fail = False

    def submit(self, items, engine):
        if any(int(it.first_dim[0]) == 999 for it in items):
            raise pir.InspireError(pir.INVALID_ARGUMENT, "bad request")
        self.items = items
        self.engine = engine
        self.t_ready = time.perf_counter() + 0.01
        with FakeWorkspace.lock:
            FakeWorkspace.live += 1
            FakeWorkspace.peak = max(FakeWorkspace.peak, FakeWorkspace.live)

    def done(self):
        return time.perf_counter() >= self.t_ready

    def finish(self):
        with FakeWorkspace.lock:
            FakeWorkspace.live -= 1
        items, self.items = self.items, []
        l, d = self.db.l, self.db.d
        return items, [np.full((l, 2, d), int(it.first_dim[0]) * 7 + len(self.db.name),
                               dtype=np.uint32) for it in items]

    def close(self):
        pass


def fake_server(d=32, t=2, l=1, db_cols=64):
    params = synthetic.make_params(d=d, n=db_cols * t, t=t, l=l, coeff_bits=32)
    return SimpleNamespace(params=params, db_cols=db_cols, _h=None)


def engine(**kw):
    servers = {"A": fake_server(l=2), "BB": fake_server(d=64, t=4)}
    return serving.ServingEngine(servers, workspace_factory=FakeWorkspace,
                                 workspace_bytes=lambda s, b: 1 << 20, **kw)


def _req(db, i):
    fd = np.array([i] + [0] * 9, dtype=np.uint32)
    sd = np.zeros((db.nsd, db.d), dtype=np.uint32)
    pk = np.zeros((db.npk, db.d), dtype=np.uint32)
    return fd, sd, pk


def test_results_route_to_their_requests():
    FakeWorkspace.peak = 0
    with engine(max_batch=8, hbm_budget=6 << 20, max_workspaces=3) as eng:
        futs = []
        for i in range(50):
            name = "A" if i % 3 else "BB"
            futs.append((name, i, eng.submit(name, *_req(eng.dbs[name], i))))
        for name, i, f in futs:
            got = f.result(timeout=10)
            db = eng.dbs[name]
            assert got.shape == (db.l, 2, db.d)
            assert int(got[0, 0, 0]) == i * 7 + len(name)
        st = eng.stats()
    assert st["requests"] == 50
    assert max(b for _, b, _ in eng.batches) <= 8


def test_hbm_budget_limits_inflight_slots():
    # 2 MiB budget split over 2 databases at 1 MiB per workspace: 1 slot each.
    FakeWorkspace.peak = 0
    with engine(max_batch=4, hbm_budget=2 << 20, max_workspaces=3) as eng:
        assert all(len(db.free) == 1 for db in eng.dbs.values())
        futs = [eng.submit("A", *_req(eng.dbs["A"], i)) for i in range(20)]
        for f in futs:
            f.result(timeout=10)
    assert FakeWorkspace.peak <= 2


def test_requests_queued_while_busy_are_batched():
    with engine(max_batch=16, hbm_budget=1 << 20, max_workspaces=1) as eng:
        futs = [eng.submit("A", *_req(eng.dbs["A"], i)) for i in range(40)]
        for f in futs:
            f.result(timeout=10)
        sizes = [b for n, b, _ in eng.batches if n == "A"]
    assert sum(sizes) == 40
    assert max(sizes) > 1


def test_small_batches_use_plain_engine_large_tensor():
    with engine(max_batch=32, hbm_budget=1 << 20, max_workspaces=1,
                plain_max_batch=2) as eng:
        f = eng.submit("A", *_req(eng.dbs["A"], 1))
        f.result(timeout=10)
        futs = [eng.submit("A", *_req(eng.dbs["A"], i)) for i in range(30)]
        for f in futs:
            f.result(timeout=10)
    engines = [e for _, b, e in eng.batches]
    assert engines[0] == pir.ENGINE_PLAIN
    assert pir.ENGINE_TENSOR in engines


def test_failed_batch_sets_exceptions_and_loop_survives():
    with engine(max_batch=4, hbm_budget=1 << 20, max_workspaces=1) as eng:
        bad = eng.submit("A", *_req(eng.dbs["A"], 999))
        with pytest.raises(pir.InspireError):
            bad.result(timeout=10)
        ok = eng.submit("A", *_req(eng.dbs["A"], 5))
        assert int(ok.result(timeout=10)[0, 0, 0]) == 5 * 7 + 1


def test_first_dimension_longer_than_db_is_rejected():
    with engine() as eng:
        db = eng.dbs["A"]
        fd = np.zeros(db.server.db_cols + 1, dtype=np.uint32)
        with pytest.raises(pir.InspireError, match="First dimension query size"):
            eng.submit("A", fd, *_req(db, 0)[1:])
