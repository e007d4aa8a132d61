"""The engine autotuner (inspire_pir_tune_engines) and INSPIRE_ENGINE_AUTO.

The tuner times the plain engine and every form and split-K factor of the
tensor engine at batch sizes up to max_batch and keeps the crossover; AUTO
then sends each batch to the engine that was faster at that size. Checked:
AUTO answers bit-exactly as the fixed engines do (which the other tests
check against the oracle), and at batch sizes 1, 4, 8 and 64 the AUTO call
is never slower than the faster fixed engine beyond timing noise.
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


@pytest.fixture(scope="module")
def tuned():
    # n = 2^19, d = 2048, t = 8: DB 16384 x 65536 u16 (2 GiB) + pack 256 MiB.
    params = synthetic.make_params(d=2048, n=1 << 19, t=8, coeff_bits=32)
    rows, cols = 8 * 2048, (1 << 19) // 8
    db = synthetic.parallel_integers((rows, cols), 0, 65535, np.uint16, 11)
    pack = synthetic.parallel_integers((rows, 2 * 2048), -(1 << 24), 1 << 24,
                                       np.int32, 12)
    small = synthetic.make_material(
        synthetic.make_params(d=2048, n=2048 * 8, t=8, coeff_bits=32), seed=13)
    srv = pir.PirServer.CreateCombined(params, db, pack, small.a_tilde_agg,
                                       small.t_vec_h, small.second_dim_a)
    crossover = srv.tune_engines(64)
    return params, srv, crossover


def _time_products(srv, batch, engine, t_fd, t_pk, out, reps=5):
    import ctypes
    lib = pir._lib.load()
    err = pir._errbuf()
    stream = torch.cuda.current_stream()

    def run():
        rc = lib.inspire_pir_products_device(
            srv._h, batch, ctypes.c_void_p(t_fd.data_ptr()),
            ctypes.c_void_p(t_pk.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            engine, ctypes.c_void_p(stream.cuda_stream), err, len(err))
        pir._check(rc, err)
    run()
    best = None
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return best, out[:batch].clone()


def test_crossover_is_a_tested_batch_size(tuned):
    _, _, crossover = tuned
    assert crossover in (1, 2, 3, 4, 5, 6, 7, 8, 16, 32, 64, 0x7fffffff)


@pytest.mark.parametrize("batch", [1, 4, 8, 64])
def test_auto_engine_never_loses_to_either_fixed_engine(tuned, batch):
    params, srv, _ = tuned
    fd, _, pk = synthetic.make_requests(params, batch, seed=batch)
    t_fd = torch.from_numpy(fd.view(np.int32)).cuda()
    t_pk = torch.from_numpy(pk.view(np.int32)).cuda()
    out = torch.empty((batch, srv.rows), dtype=torch.int32, device="cuda")
    ms_plain, r_plain = _time_products(srv, batch, pir.ENGINE_PLAIN, t_fd,
                                       t_pk, out)
    ms_tensor, r_tensor = _time_products(srv, batch, pir.ENGINE_TENSOR, t_fd,
                                         t_pk, out)
    ms_auto, r_auto = _time_products(srv, batch, pir.ENGINE_AUTO, t_fd, t_pk,
                                     out)
    srv.check()
    assert torch.equal(r_plain, r_tensor) and torch.equal(r_auto, r_plain)
    # 10 % + 20 us of timing noise.
    assert ms_auto <= 1.10 * min(ms_plain, ms_tensor) + 0.02, \
        (batch, ms_auto, ms_plain, ms_tensor)


def test_auto_engine_answers_like_the_oracle_path(tuned):
    params, srv, _ = tuned
    fd, sd, pk = synthetic.make_requests(params, 6, seed=77)
    got_auto = srv.process_arrays(fd, sd, pk, pir.ENGINE_AUTO)
    got_plain = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(got_auto, got_plain)
