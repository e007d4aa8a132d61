"""The forms of the tensor engine's product: the DB as resident fp16 digit
planes, or read as stored (u16) and split into digits in shared memory by
the kernel's converter warpgroup, each with full (64-request) or narrow
(16-request) tiles; over Z_2^64 the planes with 32-request tiles only. All
must give the plain engine's
stage-1 words (b' + b_agg_partial, pir_server.cc:215-254) bit for
bit, for every split-K factor, ragged batches, column counts that are not a
multiple of the 128-column accumulation unit, both word sizes, and DB
entries at the ends of their range (0 and 0xFFFF, whose digits are the
extremes of the digit plan).
"""
import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def _server(params, mat):
    return pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                        mat.a_tilde_agg, mat.t_vec_h,
                                        mat.second_dim_a)


def _products(srv, params, fd, pk, engine=None, form=None, split=0):
    cb = params.rlwe.coeff_bits
    iv = np.int32 if cb == 32 else np.int64
    tdt = torch.int32 if cb == 32 else torch.int64
    b = fd.shape[0]
    q1 = np.zeros((b, srv.db_cols), dtype=params.coeff_dtype)
    q1[:, :fd.shape[1]] = fd
    t_q1 = torch.from_numpy(q1.view(iv)).cuda()
    t_pk = torch.from_numpy(np.ascontiguousarray(pk).view(iv)).cuda()
    out = torch.full((b, srv.rows), -1, dtype=tdt, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    if form is None:
        err = pir._errbuf()
        rc = pir._lib.load().inspire_pir_products_device(
            srv._h, b, t_q1.data_ptr(), t_pk.data_ptr(), out.data_ptr(), engine,
            stream, err, len(err))
        pir._check(rc, err)
    else:
        srv.tensor_products_device(b, t_q1.data_ptr(), t_pk.data_ptr(),
                                   out.data_ptr(), form, split, stream)
    torch.cuda.synchronize()
    srv.check()
    return out.cpu().numpy().view(params.coeff_dtype)


@pytest.mark.parametrize("cb,d,n,t,batch", [
    (32, 128, 8192, 2, 1),       # R = 256, C = 4096
    (32, 128, 8192, 2, 65),      # a ragged second request tile
    (32, 256, 16000, 4, 7),      # C = 4000: the last unit reads past the end
    (32, 1024, 32768, 4, 130),   # three request tiles
])
def test_raw_form_equals_planes_and_plain(cb, d, n, t, batch):
    params = synthetic.make_params(d=d, n=n, t=t, coeff_bits=cb,
                                   log_q=32 if cb == 32 else 56)
    mat = synthetic.make_material(params, seed=d + batch + cb)
    srv = _server(params, mat)
    fd, _, pk = synthetic.make_requests(params, batch, seed=batch,
                                        full_range=True)
    k = params.pack_gadget.num_digits
    plain = _products(srv, params, fd, pk, engine=pir.ENGINE_PLAIN)
    planes = _products(srv, params, fd, pk, form=pir.FORM_PLANES)
    raw = _products(srv, params, fd, pk, form=pir.FORM_RAW)
    assert np.array_equal(planes, plain)
    assert np.array_equal(raw, plain)
    for form in (pir.FORM_PLANES | pir.FORM_NARROW,
                 pir.FORM_RAW | pir.FORM_NARROW):
        got = _products(srv, params, fd, pk, form=form)
        assert np.array_equal(got, plain), form
    for split in (1, 2, 3):
        for form in (pir.FORM_RAW, pir.FORM_RAW | pir.FORM_NARROW):
            got = _products(srv, params, fd, pk, form=form, split=split)
            assert np.array_equal(got, plain), (form, split)
    # Exact integer products mod 2^w on a few requests.
    m = np.uint64((1 << cb) - 1) if cb == 32 else None
    db = mat.db.astype(np.uint64)
    pkm = mat.pack.astype(np.int64).astype(np.uint64)
    for q in sorted({0, batch - 1}):
        x = fd[q].astype(np.uint64)
        y = pk[q, :k].reshape(-1).astype(np.uint64)
        with np.errstate(over="ignore"):
            want = db[:, :x.shape[0]] @ x + pkm @ y
        if m is not None:
            want &= m
        assert np.array_equal(raw[q].astype(np.uint64), want), q


@pytest.mark.parametrize("db_value", [0, 0xFFFF, 0x7F80, 0x8080])
def test_raw_form_extreme_entries(db_value):
    params = synthetic.make_params(d=128, n=2 * 8192, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=3)
    mat.db[:] = db_value
    mat.db[::3, ::5] = 0xFFFF - db_value
    srv = _server(params, mat)
    fd, _, pk = synthetic.make_requests(params, 64, seed=4, full_range=True)
    fd[:8] = 0xFFFFFFFF
    fd[8:16] = 0x80808080
    plain = _products(srv, params, fd, pk, engine=pir.ENGINE_PLAIN)
    raw = _products(srv, params, fd, pk, form=pir.FORM_RAW)
    assert np.array_equal(raw, plain)
    narrow = _products(srv, params, fd, pk,
                       form=pir.FORM_RAW | pir.FORM_NARROW)
    assert np.array_equal(narrow, plain)


def test_z64_engine_keeps_planes_and_full_tiles():
    # Over Z_2^64 the tensor engine runs its resident planes with 32-request
    # tiles only; the other forms are refused, and AUTO / TENSOR answer as
    # the plain engine does.
    params = synthetic.make_params(d=256, n=8192, t=2, coeff_bits=64,
                                   log_q=56)
    mat = synthetic.make_material(params, seed=33)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, 33, seed=34, full_range=True)
    plain = _products(srv, params, fd, pk, engine=pir.ENGINE_PLAIN)
    assert np.array_equal(_products(srv, params, fd, pk,
                                    form=pir.FORM_PLANES), plain)
    for form in (pir.FORM_RAW, pir.FORM_PLANES | pir.FORM_NARROW,
                 pir.FORM_RAW | pir.FORM_NARROW):
        with pytest.raises(pir.InspireError) as e:
            _products(srv, params, fd, pk, form=form)
        assert e.value.code == pir.FAILED_PRECONDITION
    srv.tune_engines(64)
    assert all(r["form"] == "planes" for r in srv.engine_table())
    want = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_AUTO),
                          want)


def test_raw_form_unavailable_when_rows_are_not_16_byte_multiples():
    # 4004 columns: rows of 8008 bytes cannot be a TMA tensor; the planes
    # form still runs and the raw form is refused.
    params = synthetic.make_params(d=128, n=2 * 4004, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=5)
    srv = _server(params, mat)
    fd, _, pk = synthetic.make_requests(params, 3, seed=6)
    plain = _products(srv, params, fd, pk, engine=pir.ENGINE_PLAIN)
    assert np.array_equal(_products(srv, params, fd, pk,
                                    form=pir.FORM_PLANES), plain)
    with pytest.raises(pir.InspireError) as e:
        _products(srv, params, fd, pk, form=pir.FORM_RAW)
    assert e.value.code == pir.FAILED_PRECONDITION


def test_dropping_resident_planes_keeps_answers_and_frees_memory():
    params = synthetic.make_params(d=256, n=2 * 16384, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=9)
    srv = _server(params, mat)
    fd, sd, pk = synthetic.make_requests(params, 20, seed=10, full_range=True)
    want = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    with_planes = srv.device_bytes()
    srv.set_tensor_planes(False)
    # The DB planes were 2 x the u16 DB.
    assert with_planes - srv.device_bytes() == 2 * mat.db.nbytes
    assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_TENSOR),
                          want)
    srv.tune_engines(32)
    assert np.array_equal(srv.process_arrays(fd, sd, pk, pir.ENGINE_AUTO),
                          want)
    assert all(r["form"].startswith("raw") for r in srv.engine_table())
    with pytest.raises(pir.InspireError) as e:
        _products(srv, params, fd, pk, form=pir.FORM_PLANES)
    assert e.value.code == pir.FAILED_PRECONDITION
    srv.set_tensor_planes(True)
    assert srv.device_bytes() == with_planes
    assert np.array_equal(_products(srv, params, fd, pk, form=pir.FORM_PLANES),
                          _products(srv, params, fd, pk,
                                    engine=pir.ENGINE_PLAIN))
