"""Continuous batching over GPU-resident PIR servers (Python facade).

The request loop itself is native (inspire_gb300/csrc/serving.cu, the
inspire_serving_* C ABI): every server is a queue with a ring of request
slots in pinned host memory, and one scheduler thread batches submitted
slots onto in-flight workspaces as soon as one frees up, so batches of all
servers overlap on the GPU. The number of workspaces per server comes from
an HBM budget; small batches use the plain engine, larger ones the tensor
engine. Every response is identical to the one PirServer::ProcessResponse
gives for the same request (crypto/pir/server/pir_server.cc:154-306).

This module adds Futures: submit() copies a request into a slot and returns
a Future resolving to the (l, 2, d) response; a completion thread waits for
the tickets and copies the responses out.
"""
import ctypes
import threading
from collections import deque
from concurrent.futures import Future

import numpy as np

from . import _lib, pir


class _Queue:
    def __init__(self, name, index, d, l, nsd, npk, db_cols, dtype,
                 min_first_dim):
        self.name = name
        self.index = index
        self.d, self.l, self.nsd, self.npk = d, l, nsd, npk
        self.db_cols = db_cols
        self.dtype = np.dtype(dtype)
        self.min_first_dim = min_first_dim
        self.views = {}      # slot address -> numpy views of the slot

    def slot_views(self, ptrs):
        key = ptrs[0]
        v = self.views.get(key)
        if v is None:
            shapes = [(self.db_cols,), (self.nsd, self.d), (self.npk, self.d),
                      (self.l, 2, self.d)]
            v = []
            for p, shp in zip(ptrs, shapes):
                n = int(np.prod(shp))
                if n == 0:
                    v.append(np.zeros(shp, dtype=self.dtype))
                    continue
                buf = (ctypes.c_char * (n * self.dtype.itemsize)).from_address(p)
                v.append(np.frombuffer(buf, dtype=self.dtype).reshape(shp))
            self.views[key] = v
        return v


class ServingEngine:
    """Continuous batching over one or more PirServer instances.

    servers: {name: PirServer}. max_batch: requests per batch. hbm_budget:
    device bytes the workspaces of all servers may take (split evenly);
    each server gets between 1 and max_workspaces of them. The default, one
    batch in flight per server, keeps each database to one scan at a time:
    concurrent scans of the same matrices only share its HBM bandwidth, so
    requests that arrive meanwhile wait and join the next batch instead
    (measured on the four-server mix: half the p50 and p99 latency of three
    in flight per server, at the same or higher throughput). plain_max_batch:
    None (default) lets each server's engine autotuner pick the engine per
    batch size (inspire_pir_tune_engines runs once per server here, up to
    max_batch); a number instead sends batches up to that size to the plain
    engine and larger ones to the tensor engine when the server has it.
    max_wait_us: batching window (a partial
    batch waits until its oldest request has waited this long; 0 launches as
    soon as a workspace is free). ring_slots: request slots per server
    (default 4 * max_batch).
    """

    def __init__(self, servers, max_batch=256, hbm_budget=8 << 30,
                 max_workspaces=1, plain_max_batch=None, max_wait_us=0,
                 ring_slots=None, _loopback=None):
        self._lib = _lib.load()
        self.max_batch = max_batch
        self.crossovers = {}
        if plain_max_batch is None:
            if _loopback is None:
                for n, srv in servers.items():
                    self.crossovers[n] = srv.tune_engines(max_batch)
            plain_max_batch = -1
        ring_slots = ring_slots or 4 * max_batch
        err = pir._errbuf()
        h = ctypes.c_void_p()
        self.queues = {}
        if _loopback is None:
            names = list(servers)
            arr = (ctypes.c_void_p * len(names))(
                *[servers[n]._h.value for n in names])
            rc = self._lib.inspire_serving_create(
                arr, len(names), max_batch, plain_max_batch, max_wait_us,
                ring_slots, int(hbm_budget), max_workspaces, ctypes.byref(h),
                err, len(err))
            pir._check(rc, err)
            for i, n in enumerate(names):
                s = servers[n]
                p = s.params
                self.queues[n] = _Queue(
                    n, i, p.rlwe.degree, p.entry_size_multiple,
                    2 * p.eval_gadget.num_digits if p.interpolation_degree > 1 else 0,
                    2 * p.pack_gadget.num_digits, s.db_cols, p.coeff_dtype,
                    p.InterpolatedRows())
        else:
            names, words, workspaces, delay_us = _loopback
            w = (ctypes.c_int64 * (4 * len(names)))(*[x for q in words for x in q])
            rc = self._lib.inspire_serving_create_loopback(
                len(names), w, workspaces, delay_us, max_batch,
                plain_max_batch, max_wait_us, ring_slots, ctypes.byref(h), err,
                len(err))
            pir._check(rc, err)
            for i, (n, q) in enumerate(zip(names, words)):
                # Loopback slots: flat u32 words (d = 1 polynomial rows).
                self.queues[n] = _Queue(n, i, 1, q[3] // 2, q[1], q[2], q[0],
                                        np.uint32, 1)
        self._h = h
        self._pending = deque()
        self._cv = threading.Condition()
        self._stop = False
        self._thread = None

    @classmethod
    def loopback(cls, queues, workspaces=2, delay_us=200, **kw):
        """An engine over the host-only loopback device: queues is
        {name: (first_dim_words, second_dim_words, packing_key_words,
        response_words)}; see inspire_serving_create_loopback."""
        names = list(queues)
        return cls(None, _loopback=(names, [tuple(queues[n]) for n in names],
                                    workspaces, delay_us), **kw)

    # -- public ----------------------------------------------------------
    def start(self):
        self._stop = False
        self._thread = threading.Thread(target=self._complete, daemon=True)
        self._thread.start()
        return self

    def stop(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        if self._thread:
            self._thread.join()
            self._thread = None
        if self._h:
            self._lib.inspire_serving_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    def submit(self, name, first_dim, second_dim, packing_key):
        """Queues one request; returns a Future resolving to (l, 2, d)."""
        q = self.queues[name]
        fd = np.asarray(first_dim, dtype=q.dtype).reshape(-1)
        err = pir._errbuf()
        ticket = ctypes.c_int64()
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        if fd.shape[0] > q.db_cols or fd.shape[0] < q.min_first_dim:
            raise pir.InspireError(
                pir.INVALID_ARGUMENT,
                "First dimension query size (%d) is invalid for DB columns "
                "(%d)." % (fd.shape[0], q.db_cols))
        rc = self._lib.inspire_serving_acquire(
            self._h, q.index, 60000, ctypes.byref(ticket),
            *[ctypes.byref(p) for p in ptrs], err, len(err))
        pir._check(rc, err)
        v = q.slot_views([p.value for p in ptrs])
        v[0][:fd.shape[0]] = fd
        if q.nsd:
            v[1][...] = np.asarray(second_dim, dtype=q.dtype).reshape(q.nsd, q.d)
        v[2][...] = np.asarray(packing_key, dtype=q.dtype).reshape(q.npk, q.d)
        fut = Future()
        rc = self._lib.inspire_serving_submit(self._h, ticket.value,
                                              fd.shape[0], err, len(err))
        if rc:
            self._lib.inspire_serving_release(self._h, ticket.value)
            pir._check(rc, err)
        with self._cv:
            self._pending.append((ticket.value, v[3], fut))
            self._cv.notify()
        return fut

    def stats(self):
        s = _Stats()
        self._lib.inspire_serving_get_stats(self._h, ctypes.byref(s))
        return {"requests": s.requests, "failed": s.failed,
                "batches": s.batches, "tensor_batches": s.tensor_batches,
                "mean_batch": s.mean_batch, "p50_ms": s.p50_ms,
                "p99_ms": s.p99_ms, "max_ms": s.max_ms,
                "max_inflight": s.max_inflight}

    def reset_stats(self):
        self._lib.inspire_serving_reset_stats(self._h)

    def queue_info(self, name):
        ws, b, slots = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        self._lib.inspire_serving_queue_info(
            self._h, self.queues[name].index, ctypes.byref(ws),
            ctypes.byref(b), ctypes.byref(slots))
        return {"workspaces": ws.value, "workspace_bytes": b.value,
                "ring_slots": slots.value}

    # -- completion ------------------------------------------------------
    def _complete(self):
        err = pir._errbuf()
        while True:
            with self._cv:
                while not self._pending and not self._stop:
                    self._cv.wait()
                if not self._pending:
                    return
                ticket, resp, fut = self._pending.popleft()
            while True:
                rc = self._lib.inspire_serving_wait(self._h, ticket, 1000, err,
                                                    len(err))
                if rc != pir.DEADLINE_EXCEEDED:
                    break
            if rc == 0:
                fut.set_result(resp.copy())
            else:
                fut.set_exception(pir.InspireError(rc, err.value.decode()))
            self._lib.inspire_serving_release(self._h, ticket)


class _Stats(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("batches", ctypes.c_int64),
                ("tensor_batches", ctypes.c_int64),
                ("mean_batch", ctypes.c_double), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("max_inflight", ctypes.c_int32), ("reserved", ctypes.c_int32)]
