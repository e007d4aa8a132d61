"""Continuous-batching request loop over GPU-resident PIR servers.

Requests for several databases (servers of different shapes: ring degree,
interpolation degree, entry size multiple l) arrive on any thread via
submit(); a scheduler thread groups the pending requests of each database
into batches and launches them on free workspaces (inspire_pir_workspace_*:
device buffers + a CUDA stream + pinned staging). A database has several
workspaces, so a batch is admitted as soon as a workspace frees up, while
earlier batches are still on the GPU: their work overlaps on the device. The
number of workspaces is set by an HBM budget (workspace bytes come from the
library). Small batches run on the plain engine, larger ones on the
tensor-core engine; both give identical responses.

The reference serves one request per ProcessResponse call on one thread
(crypto/pir/server/pir_server.cc:154-306); the loop keeps that call's
semantics per request (same response bytes) and adds batching.
"""
import ctypes
import threading
import time
from collections import deque
from concurrent.futures import Future

import numpy as np

from . import _lib, pir


class _Workspace:
    """One in-flight batch slot of a database (wraps inspire_pir_workspace)."""

    def __init__(self, db, max_batch):
        lib = _lib.load()
        self.db = db
        self.max_batch = max_batch
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = lib.inspire_pir_workspace_create(db.server._h, max_batch,
                                              ctypes.byref(h), err, len(err))
        if rc:
            raise pir.InspireError(rc, err.value.decode())
        self.h = h
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        lib.inspire_pir_workspace_host_buffers(h, *[ctypes.byref(p) for p in ptrs])
        cdt = db.server.params.coeff_dtype
        d = db.d
        shapes = [(max_batch, db.server.db_cols), (max_batch, db.nsd, d),
                  (max_batch, db.npk, d), (max_batch, db.l, 2, d)]
        self.host = []
        for p, shp in zip(ptrs, shapes):
            n = int(np.prod(shp))
            buf = (ctypes.c_uint8 * (n * np.dtype(cdt).itemsize)).from_address(
                p.value) if n else None
            arr = (np.frombuffer(buf, dtype=cdt).reshape(shp) if n
                   else np.zeros(shp, dtype=cdt))
            self.host.append(arr)
        self.items = []
        self.t_launch = 0.0

    def submit(self, items, engine):
        lib = _lib.load()
        fd, sd, pk, _ = self.host
        for i, it in enumerate(items):
            n1 = it.first_dim.shape[0]
            fd[i, :n1] = it.first_dim
            fd[i, n1:] = 0
            if self.db.nsd:
                sd[i] = it.second_dim
            pk[i] = it.packing_key
        err = ctypes.create_string_buffer(512)
        rc = lib.inspire_pir_workspace_submit(self.h, len(items), engine, err,
                                              len(err))
        if rc:
            raise pir.InspireError(rc, err.value.decode())
        self.items = items
        self.t_launch = time.perf_counter()

    def done(self):
        return _lib.load().inspire_pir_workspace_poll(self.h) != 0

    def finish(self):
        lib = _lib.load()
        err = ctypes.create_string_buffer(512)
        rc = lib.inspire_pir_workspace_wait(self.h, err, len(err))
        items, self.items = self.items, []
        if rc:
            return items, pir.InspireError(rc, err.value.decode())
        resp = self.host[3]
        return items, [resp[i].copy() for i in range(len(items))]

    def close(self):
        if self.h:
            _lib.load().inspire_pir_workspace_destroy(self.h)
            self.h = None


class _Item:
    __slots__ = ("db", "first_dim", "second_dim", "packing_key", "future",
                 "t_submit", "t_done")

    def __init__(self, db, fd, sd, pk):
        self.db = db
        self.first_dim = fd
        self.second_dim = sd
        self.packing_key = pk
        self.future = Future()
        self.t_submit = time.perf_counter()
        self.t_done = None


class _Database:
    def __init__(self, name, server):
        self.name = name
        self.server = server
        self.workspace_bytes = 0
        p = server.params
        self.d = p.rlwe.degree
        self.l = p.entry_size_multiple
        self.nsd = (2 * p.eval_gadget.num_digits
                    if p.interpolation_degree > 1 else 0)
        self.npk = 2 * p.pack_gadget.num_digits
        self.pending = deque()
        self.free = []
        self.inflight = []


class ServingEngine:
    """Continuous batching over one or more PirServer instances.

    servers: {name: PirServer}. max_batch: requests per batch. hbm_budget:
    device bytes the workspaces of all databases may take (split evenly);
    each database gets between 1 and max_workspaces of them. plain_max_batch:
    batches up to this size use the plain engine, larger ones the tensor
    engine when the server has it.
    """

    def __init__(self, servers, max_batch=256, hbm_budget=8 << 30,
                 max_workspaces=3, plain_max_batch=4, workspace_factory=None,
                 workspace_bytes=None):
        self.max_batch = max_batch
        self.plain_max_batch = plain_max_batch
        self.dbs = {n: _Database(n, s) for n, s in servers.items()}
        factory = workspace_factory or _Workspace
        if workspace_bytes is None:
            lib = _lib.load()

            def workspace_bytes(server, b):
                return lib.inspire_pir_workspace_bytes(server._h, b)
        share = hbm_budget // max(1, len(self.dbs))
        for db in self.dbs.values():
            per = workspace_bytes(db.server, max_batch)
            # HBM admission: as many in-flight batch slots as the budget holds.
            n = int(max(1, min(max_workspaces, share // max(per, 1))))
            db.free = [factory(db, max_batch) for _ in range(n)]
            db.workspace_bytes = per
        self._cv = threading.Condition()
        self._stop = False
        self._thread = None
        self.latencies = []
        self.batches = []          # (db name, batch size, engine)
        self.max_inflight = 0
        self._tensor_ok = {n: True for n in self.dbs}

    # -- public ----------------------------------------------------------
    def start(self):
        self._stop = False
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()
        return self

    def stop(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        if self._thread:
            self._thread.join()
        for db in self.dbs.values():
            for ws in db.free + [w for w in db.inflight]:
                ws.close()

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    def submit(self, db_name, first_dim, second_dim, packing_key):
        """Queues one request; returns a Future resolving to (l, 2, d)."""
        db = self.dbs[db_name]
        cdt = db.server.params.coeff_dtype
        it = _Item(db, np.asarray(first_dim, dtype=cdt),
                   np.asarray(second_dim, dtype=cdt).reshape(db.nsd, db.d),
                   np.asarray(packing_key, dtype=cdt).reshape(db.npk, db.d))
        if it.first_dim.shape[0] > db.server.db_cols:
            raise pir.InspireError(
                pir.INVALID_ARGUMENT,
                "First dimension query size (%d) is invalid for DB columns "
                "(%d)." % (it.first_dim.shape[0], db.server.db_cols))
        with self._cv:
            db.pending.append(it)
            self._cv.notify()
        return it.future

    def stats(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"requests": len(self.latencies),
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "batches": len(self.batches),
                "mean_batch": (float(np.mean([b for _, b, _ in self.batches]))
                               if self.batches else 0.0),
                "max_inflight": self.max_inflight}

    # -- scheduler -------------------------------------------------------
    def _engine_for(self, db, n):
        if n > self.plain_max_batch and self._tensor_ok[db.name]:
            return pir.ENGINE_TENSOR
        return pir.ENGINE_PLAIN

    def _loop(self):
        while True:
            progressed = False
            # Retire finished batches (their workspaces become free slots).
            for db in self.dbs.values():
                still = []
                for ws in db.inflight:
                    if ws.done():
                        items, res = ws.finish()
                        t = time.perf_counter()
                        for k, it in enumerate(items):
                            it.t_done = t
                            if isinstance(res, Exception):
                                it.future.set_exception(res)
                            else:
                                it.future.set_result(res[k])
                                self.latencies.append(t - it.t_submit)
                        db.free.append(ws)
                        progressed = True
                    else:
                        still.append(ws)
                db.inflight = still
            # Admit pending requests into free workspaces.
            with self._cv:
                if self._stop and not any(d.pending or d.inflight
                                          for d in self.dbs.values()):
                    return
                launch = []
                for db in self.dbs.values():
                    while db.pending and db.free:
                        n = min(len(db.pending), self.max_batch)
                        items = [db.pending.popleft() for _ in range(n)]
                        launch.append((db, db.free.pop(), items))
            for db, ws, items in launch:
                eng = self._engine_for(db, len(items))
                try:
                    ws.submit(items, eng)
                except pir.InspireError as e:
                    if eng == pir.ENGINE_TENSOR and e.code == pir.FAILED_PRECONDITION:
                        self._tensor_ok[db.name] = False
                        eng = pir.ENGINE_PLAIN
                        ws.submit(items, eng)
                    else:
                        for it in items:
                            it.future.set_exception(e)
                        db.free.append(ws)
                        continue
                db.inflight.append(ws)
                self.batches.append((db.name, len(items), eng))
                progressed = True
            inflight = sum(len(d.inflight) for d in self.dbs.values())
            self.max_inflight = max(self.max_inflight, inflight)
            if not progressed:
                with self._cv:
                    if inflight:
                        self._cv.wait(timeout=0.0002)
                    elif not self._stop and not any(d.pending for d in self.dbs.values()):
                        self._cv.wait(timeout=0.05)
