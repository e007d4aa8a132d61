"""The native continuous-batching scheduler on the CPU.

The engine runs over its host-only loopback device (response word k of a
request is first_dim[0] * 7 + queue + k, ready a set delay after the batch
launches), so batching, ring order, admission, result routing and error
propagation are checked without a GPU.
"""
import threading

import numpy as np
import pytest

from inspire_gb300 import _lib, pir, serving

QUEUES = {"A": (16, 4, 4, 8), "BB": (32, 0, 8, 4)}


@pytest.fixture(scope="module", autouse=True)
def lib():
    try:
        return _lib.load()
    except _lib.LibraryMissing:
        pytest.skip("library not built")


def _req(eng, name, i):
    q = eng.queues[name]
    fd = np.zeros(q.db_cols, dtype=np.uint32)
    fd[0] = i
    sd = np.zeros((q.nsd, q.d), dtype=np.uint32)
    pk = np.zeros((q.npk, q.d), dtype=np.uint32)
    return fd, sd, pk


def _want(eng, name, i):
    q = eng.queues[name]
    k = np.arange(q.l * 2 * q.d, dtype=np.uint64)
    return ((i * 7 + q.index + k) % (1 << 32)).astype(np.uint32).reshape(
        q.l, 2, q.d)


def test_results_route_to_their_requests():
    with serving.ServingEngine.loopback(QUEUES, workspaces=3, delay_us=300,
                                        max_batch=8) as eng:
        futs = []
        for i in range(200):
            name = "A" if i % 3 else "BB"
            futs.append((name, i, eng.submit(name, *_req(eng, name, i))))
        for name, i, f in futs:
            assert np.array_equal(f.result(timeout=30), _want(eng, name, i))
        st = eng.stats()
    assert st["requests"] == 200 and st["failed"] == 0
    assert st["mean_batch"] <= 8


def test_requests_queued_while_busy_are_batched():
    with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=1,
                                        delay_us=5000, max_batch=16) as eng:
        futs = [eng.submit("A", *_req(eng, "A", i)) for i in range(64)]
        for i, f in enumerate(futs):
            assert np.array_equal(f.result(timeout=30), _want(eng, "A", i))
        st = eng.stats()
    assert st["batches"] < 64
    assert st["mean_batch"] > 1.5
    assert st["max_inflight"] == 1


def test_batching_window_groups_light_traffic():
    # Requests trickle in one by one with a free workspace each time: with
    # no window every request is its own batch, with a window they group.
    import time
    for window, expect_grouped in ((0, False), (30000, True)):
        with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=4,
                                            delay_us=50, max_batch=64,
                                            max_wait_us=window) as eng:
            futs = []
            for i in range(20):
                futs.append(eng.submit("A", *_req(eng, "A", i)))
                time.sleep(0.001)
            for i, f in enumerate(futs):
                assert np.array_equal(f.result(timeout=30), _want(eng, "A", i))
            st = eng.stats()
        assert (st["mean_batch"] > 2) == expect_grouped, (window, st)


def test_workspaces_overlap():
    with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=3,
                                        delay_us=20000, max_batch=2) as eng:
        futs = [eng.submit("A", *_req(eng, "A", i)) for i in range(12)]
        for f in futs:
            f.result(timeout=30)
        assert eng.stats()["max_inflight"] >= 2


def test_small_batches_use_plain_engine_large_tensor():
    with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=1,
                                        delay_us=3000, max_batch=32,
                                        plain_max_batch=2) as eng:
        eng.submit("A", *_req(eng, "A", 1)).result(timeout=30)
        assert eng.stats()["tensor_batches"] == 0
        futs = [eng.submit("A", *_req(eng, "A", i)) for i in range(40)]
        for f in futs:
            f.result(timeout=30)
        assert eng.stats()["tensor_batches"] >= 1


def test_default_engine_choice_is_the_servers_crossover():
    # plain_max_batch=None: each queue's device picks the engine per batch
    # size (the loopback device's crossover is 5 requests).
    with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=1,
                                        delay_us=3000, max_batch=32) as eng:
        for i in range(3):
            eng.submit("A", *_req(eng, "A", i)).result(timeout=30)
        assert eng.stats()["tensor_batches"] == 0
        futs = [eng.submit("A", *_req(eng, "A", i)) for i in range(40)]
        for i, f in enumerate(futs):
            assert np.array_equal(f.result(timeout=30), _want(eng, "A", i))
        assert eng.stats()["tensor_batches"] >= 1


def test_failed_batch_sets_exceptions_and_loop_survives():
    with serving.ServingEngine.loopback({"A": (4, 0, 2, 2)}, workspaces=1,
                                        delay_us=100, max_batch=4) as eng:
        bad = eng.submit("A", *_req(eng, "A", 0xDEAD))
        with pytest.raises(pir.InspireError, match="rejected"):
            bad.result(timeout=30)
        ok = eng.submit("A", *_req(eng, "A", 5))
        assert np.array_equal(ok.result(timeout=30), _want(eng, "A", 5))
        assert eng.stats()["failed"] >= 1


def test_first_dimension_longer_than_db_is_rejected():
    with serving.ServingEngine.loopback(QUEUES) as eng:
        fd, sd, pk = _req(eng, "A", 1)
        with pytest.raises(pir.InspireError, match="First dimension query size"):
            eng.submit("A", np.zeros(17, np.uint32), sd, pk)


def test_short_first_dimension_is_zero_padded():
    # A slot reused after a full-length request must not leak its old words.
    with serving.ServingEngine.loopback({"A": (8, 0, 2, 2)}, workspaces=1,
                                        delay_us=100, max_batch=1,
                                        ring_slots=1) as eng:
        fd, sd, pk = _req(eng, "A", 3)
        fd[:] = 9
        eng.submit("A", fd, sd, pk).result(timeout=30)
        eng.submit("A", fd[:2], sd, pk).result(timeout=30)
        q = eng.queues["A"]
        slot = next(iter(q.views.values()))
        assert list(slot[0][2:]) == [0] * 6


def test_many_client_threads():
    with serving.ServingEngine.loopback(QUEUES, workspaces=2, delay_us=200,
                                        max_batch=16, ring_slots=64) as eng:
        errors = []

        def client(name, base):
            try:
                fs = [(i, eng.submit(name, *_req(eng, name, i)))
                      for i in range(base, base + 150)]
                for i, f in fs:
                    assert np.array_equal(f.result(timeout=60),
                                          _want(eng, name, i))
            except Exception as e:  # surfaced below
                errors.append(e)

        ths = [threading.Thread(target=client, args=(n, b))
               for n, b in (("A", 0), ("BB", 1000), ("A", 2000), ("BB", 3000))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        assert not errors, errors
        assert eng.stats()["requests"] == 600


def test_bad_ticket_and_arguments(lib):
    err = pir._errbuf()
    import ctypes
    h = ctypes.c_void_p()
    words = (ctypes.c_int64 * 4)(4, 0, 2, 2)
    rc = lib.inspire_serving_create_loopback(1, words, 1, 0, 8, 2, 0, 4,
                                             ctypes.byref(h), err, len(err))
    assert rc == pir.INVALID_ARGUMENT       # ring_slots < max_batch
    rc = lib.inspire_serving_create_loopback(1, words, 1, 0, 8, 2, 0, 8,
                                             ctypes.byref(h), err, len(err))
    assert rc == 0
    try:
        assert lib.inspire_serving_submit(h, 12345, 1, err, len(err)) == \
            pir.INVALID_ARGUMENT
        assert lib.inspire_serving_wait(h, 12345, 1, err, len(err)) == \
            pir.INVALID_ARGUMENT
        t = ctypes.c_int64()
        p = [ctypes.c_void_p() for _ in range(4)]
        assert lib.inspire_serving_acquire(h, 3, 10, ctypes.byref(t),
                                           *[ctypes.byref(x) for x in p],
                                           err, len(err)) == pir.INVALID_ARGUMENT
        assert lib.inspire_serving_acquire(h, 0, 10, ctypes.byref(t),
                                           *[ctypes.byref(x) for x in p],
                                           err, len(err)) == 0
        # Not submitted yet: waiting is refused, releasing is allowed.
        assert lib.inspire_serving_wait(h, t.value, 1, err, len(err)) == \
            pir.FAILED_PRECONDITION
        assert lib.inspire_serving_release(h, t.value) == 0
    finally:
        lib.inspire_serving_destroy(h)


def _loopback(lib, words, workspaces=2, delay_us=0, max_batch=4,
              plain_max_batch=1, max_wait_us=0, ring_slots=8):
    import ctypes
    err = pir._errbuf()
    h = ctypes.c_void_p()
    w = (ctypes.c_int64 * len(words))(*words)
    rc = lib.inspire_serving_create_loopback(
        len(words) // 4, w, workspaces, delay_us, max_batch, plain_max_batch,
        max_wait_us, ring_slots, ctypes.byref(h), err, len(err))
    assert rc == 0, err.value
    return h


def _acquire(lib, h, q, timeout_ms):
    """(status, ticket, [first_dim, second_dim, packing_key, response])."""
    import ctypes
    err = pir._errbuf()
    t = ctypes.c_int64()
    p = [ctypes.c_void_p() for _ in range(4)]
    rc = lib.inspire_serving_acquire(h, q, timeout_ms, ctypes.byref(t),
                                     *[ctypes.byref(x) for x in p], err, len(err))
    return rc, t.value, [x.value for x in p]


def _submit(lib, h, ticket, fd_ptr, word0, n_words):
    import ctypes
    fd = (ctypes.c_uint32 * n_words).from_address(fd_ptr)
    fd[0] = word0
    err = pir._errbuf()
    return lib.inspire_serving_submit(h, ticket, 1, err, len(err))


def test_full_ring_refuses_acquire_after_its_timeout(lib):
    """inspire_serving_acquire blocks up to its timeout for a free slot and
    then answers RESOURCE_EXHAUSTED; releasing the oldest slot frees one."""
    import time
    h = _loopback(lib, [4, 0, 2, 2], max_batch=4, ring_slots=4)
    try:
        tickets = []
        for _ in range(4):
            rc, t, _ = _acquire(lib, h, 0, 100)
            assert rc == 0
            tickets.append(t)
        t0 = time.monotonic()
        rc, _, _ = _acquire(lib, h, 0, 50)
        assert rc == pir.RESOURCE_EXHAUSTED
        assert time.monotonic() - t0 >= 0.04
        assert lib.inspire_serving_release(h, tickets[0]) == 0
        rc, t, _ = _acquire(lib, h, 0, 100)
        assert rc == 0
        for t in tickets[1:] + [t]:
            assert lib.inspire_serving_release(h, t) == 0
    finally:
        lib.inspire_serving_destroy(h)


def test_wait_reports_a_request_still_in_flight(lib):
    """inspire_serving_wait answers DEADLINE_EXCEEDED while the batch runs
    and the response once it is done; a running request cannot be
    released."""
    import ctypes
    err = pir._errbuf()
    h = _loopback(lib, [4, 0, 2, 3], delay_us=300_000)
    try:
        rc, t, p = _acquire(lib, h, 0, 100)
        assert rc == 0
        assert _submit(lib, h, t, p[0], 11, 4) == 0
        assert lib.inspire_serving_wait(h, t, 1, err, len(err)) == pir.DEADLINE_EXCEEDED
        assert b"in flight" in err.value
        assert lib.inspire_serving_release(h, t) == pir.FAILED_PRECONDITION
        assert lib.inspire_serving_wait(h, t, 5000, err, len(err)) == 0
        resp = (ctypes.c_uint32 * 3).from_address(p[3])
        assert list(resp) == [11 * 7 + k for k in range(3)]
        assert lib.inspire_serving_release(h, t) == 0
    finally:
        lib.inspire_serving_destroy(h)


def test_stats_count_completed_and_failed_requests_and_reset(lib):
    """get_stats: completed and failed requests, batches, mean batch size,
    latency percentiles in order, the largest number of batches in flight;
    reset_stats clears them."""
    import ctypes
    err = pir._errbuf()
    h = _loopback(lib, [4, 0, 2, 2], workspaces=2, delay_us=2000, max_batch=4,
                  ring_slots=16)
    try:
        tickets = []
        for i in range(10):
            rc, t, p = _acquire(lib, h, 0, 1000)
            assert rc == 0
            assert _submit(lib, h, t, p[0], 0xDEAD if i == 9 else i + 1, 4) == 0
            tickets.append(t)
        codes = [lib.inspire_serving_wait(h, t, 5000, err, len(err)) for t in tickets]
        for t in tickets:
            assert lib.inspire_serving_release(h, t) == 0
        st = serving._Stats()
        assert lib.inspire_serving_get_stats(h, ctypes.byref(st)) == 0
        n_failed = sum(c != 0 for c in codes)
        assert codes[9] == pir.INVALID_ARGUMENT and n_failed >= 1
        assert st.failed == n_failed
        assert st.requests == 10 - n_failed
        assert st.batches >= 3 and st.mean_batch == pytest.approx(10 / st.batches)
        assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms
        assert 1 <= st.max_inflight <= 2
        assert lib.inspire_serving_reset_stats(h) == 0
        assert lib.inspire_serving_get_stats(h, ctypes.byref(st)) == 0
        assert (st.requests, st.failed, st.batches, st.max_inflight) == (0, 0, 0, 0)
        assert st.p50_ms == st.max_ms == 0.0
    finally:
        lib.inspire_serving_destroy(h)


def test_queue_info(lib):
    import ctypes
    h = _loopback(lib, [4, 0, 2, 2, 8, 2, 2, 4], workspaces=3, ring_slots=12)
    try:
        ws, nbytes, slots = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        for q in (0, 1):
            assert lib.inspire_serving_queue_info(h, q, ctypes.byref(ws), ctypes.byref(nbytes),
                                                  ctypes.byref(slots)) == 0
            assert (ws.value, slots.value) == (3, 12)
        assert lib.inspire_serving_queue_info(h, 2, ctypes.byref(ws), ctypes.byref(nbytes),
                                              ctypes.byref(slots)) == pir.INVALID_ARGUMENT
    finally:
        lib.inspire_serving_destroy(h)
