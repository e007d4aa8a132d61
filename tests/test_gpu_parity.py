"""Parity of the CUDA path with the CPU oracle, through the C ABI.

Integer results must be bit-exact. Cases follow the reference's own tests:
crypto/matrix_test.cc, crypto/polynomial_test.cc, crypto/encryption_test.cc
(ExternalProduct), crypto/lwes_to_rlwe_test.cc (FinalizeMatrixPack) and the
nine PirServer type configurations of crypto/pir/server/pir_server_test.cc
(d=32, n=1024, p=257, 2-bit gadget digits), plus the metrics-tool shapes.
"""
import zlib

import numpy as np
import pytest

from inspire_gb300 import build, pir, synthetic
from oracle import pyoracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def oparams(params, coeff_bits=None):
    r = params.rlwe
    return orc.make_params(
        coeff_bits=coeff_bits or r.coeff_bits,
        log_degree=r.degree.bit_length() - 1, log_modulus=r.log_modulus,
        log_modulus1_after_switch=r.log_modulus1_after_switch,
        log_modulus2_after_switch=r.log_modulus2_after_switch,
        pack_log_digit=params.pack_gadget.log_digit,
        pack_num_digits=params.pack_gadget.num_digits,
        eval_log_digit=params.eval_gadget.log_digit,
        eval_num_digits=params.eval_gadget.num_digits,
        num_entries=params.num_entries,
        interpolation_degree=params.interpolation_degree,
        entry_size_multiple=params.entry_size_multiple)


# ---------------------------------------------------------------- GEMV ----
@pytest.mark.parametrize("dt", [np.uint8, np.uint16, np.uint32, np.uint64,
                                np.int16, np.int32])
@pytest.mark.parametrize("coeff_bits", [32, 64])
@pytest.mark.parametrize("shape", [(2, 2), (7, 64), (65, 1000), (300, 4096)])
def test_matrix_multiply(dt, coeff_bits, shape):
    rng = np.random.default_rng(zlib.crc32(repr((str(dt), coeff_bits, shape)).encode()))
    info = np.iinfo(dt)
    m = rng.integers(info.min, info.max, size=shape, dtype=dt, endpoint=True)
    cdt = np.uint32 if coeff_bits == 32 else np.uint64
    v = rng.integers(0, np.iinfo(cdt).max, size=shape[1], dtype=cdt,
                     endpoint=True)
    assert np.array_equal(pir.matrix_multiply(m, v, coeff_bits),
                          orc.matrix_multiply(m, v, coeff_bits))


def test_matrix_multiply_known_answers():
    # crypto/matrix_test.cc:81-134.
    m = np.array([[1, 2], [3, 4]], dtype=np.uint16)
    assert pir.matrix_multiply(m, [5, 6], 32).tolist() == [17, 39]
    m = np.tile(np.array([1, 2, 3, 4], dtype=np.uint16), (2, 8))
    assert pir.matrix_multiply(m, np.ones(32), 64).tolist() == [80, 80]
    m = np.tile(np.array([-1, 2], dtype=np.int32), (2, 16))
    assert pir.matrix_multiply(m, np.ones(32), 64).tolist() == [16, 16]


def test_matrix_multiply_size_mismatch():
    with pytest.raises(pir.InspireError, match="Vector size must match"):
        pir.matrix_multiply(np.ones((2, 3), np.uint16), [1, 2], 32)


# ------------------------------------------------------- inner product ----
@pytest.mark.parametrize("coeff_bits", [32, 64])
@pytest.mark.parametrize("d", [4, 32, 1024, 2048, 4096, 8192])
@pytest.mark.parametrize("n", [1, 2, 6])
def test_inner_product_full_range(coeff_bits, d, n):
    rng = np.random.default_rng(d * 7 + n + coeff_bits)
    cdt = np.uint32 if coeff_bits == 32 else np.uint64
    u = rng.integers(0, np.iinfo(cdt).max, size=(n, d), dtype=cdt, endpoint=True)
    v = rng.integers(0, np.iinfo(cdt).max, size=(n, d), dtype=cdt, endpoint=True)
    chunk = min(20, int((53.0 - np.log2(n) - np.log2(d)) / 2.0))
    want = orc.inner_product(u, v, coeff_bits, chunk_bits=chunk)
    got = pir.inner_product(u, v, coeff_bits, chunk_bits=chunk)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("coeff_bits", [32, 64])
def test_inner_product_signed_digits(coeff_bits):
    # FinalizeMatrixPack's operand shape: signed 19-bit digits x log_q bits.
    rng = np.random.default_rng(5)
    cdt = np.uint32 if coeff_bits == 32 else np.uint64
    d = 2048
    u = rng.integers(-(1 << 18), 1 << 18, size=(2, d)).astype(cdt)
    v = rng.integers(0, np.iinfo(cdt).max, size=(2, d), dtype=cdt, endpoint=True)
    lq = 32 if coeff_bits == 32 else 52
    want = orc.inner_product(u, v, coeff_bits, 19, lq, 20, u_signed=True)
    got = pir.inner_product(u, v, coeff_bits, 19, lq, 20, u_signed=True)
    assert np.array_equal(got, want)


def test_inner_product_reference_random_cases():
    # crypto/polynomial_test.cc:550-608 shapes (varying bits and chunks).
    rng = np.random.default_rng(12345)
    for degree in (128, 512, 2048):
        for k in (1, 5, 10):
            tb, ab = int(rng.integers(1, 32)), int(rng.integers(1, 32))
            u = rng.integers(0, 1 << tb, size=(k, degree), dtype=np.uint32)
            v = rng.integers(0, 1 << ab, size=(k, degree), dtype=np.uint32)
            for chunk in (12, 16, 20):
                if np.log2(k) + np.log2(degree) + 2 * chunk > 53:
                    continue
                want = orc.inner_product(u, v, 32, tb, ab, chunk)
                got = pir.inner_product(u, v, 32, tb, ab, chunk)
                assert np.array_equal(got, want), (degree, k, chunk)


def test_inner_product_precision_guard():
    u = np.ones((4, 1024), dtype=np.uint32)
    with pytest.raises(pir.InspireError, match="precision overflow"):
        pir.inner_product(u, u, 32, chunk_bits=21)


# ------------------------------------------------ external product etc ----
EXT_CASES = [
    # (coeff_bits, log_q, d, ld, nd)
    (32, 32, 2048, 19, 3),
    (32, 32, 4096, 19, 3),
    (32, 30, 32, 2, 14),
    (64, 52, 2048, 19, 3),
    (64, 56, 8192, 19, 3),
    (64, 64, 32, 2, 31),
    (64, 62, 32, 2, 30),
]


@pytest.mark.parametrize("case", EXT_CASES)
def test_external_product(case):
    cb, lq, d, ld, nd = case
    params = synthetic.make_params(d=d, n=2 * d, t=2, coeff_bits=cb, log_q=lq,
                                   evalg=(ld, nd), pack=(ld, nd))
    rng = np.random.default_rng(cb + lq + d)
    cdt = params.coeff_dtype
    full = np.iinfo(cdt).max
    ct_a = rng.integers(0, full, size=d, dtype=cdt, endpoint=True)
    ct_b = rng.integers(0, full, size=d, dtype=cdt, endpoint=True)
    rgsw = rng.integers(0, full, size=(4 * nd, d), dtype=cdt, endpoint=True)
    want = orc.external_product(oparams(params), ct_a, ct_b, rgsw)
    got = pir.external_product(params, ct_a, ct_b, rgsw)
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1], want[1])


FIN_CASES = [(32, 32, 2048, 19, 2), (32, 32, 4096, 19, 2), (64, 52, 2048, 19, 2),
             (64, 56, 2048, 19, 2), (64, 56, 8192, 19, 2), (32, 30, 32, 2, 14),
             (64, 64, 32, 2, 31)]


@pytest.mark.parametrize("case", FIN_CASES)
def test_finalize_matrix_pack(case):
    cb, lq, d, ld, nd = case
    params = synthetic.make_params(d=d, n=2 * d, t=2, coeff_bits=cb, log_q=lq,
                                   pack=(ld, nd))
    rng = np.random.default_rng(d + nd)
    cdt = params.coeff_dtype
    full = np.iinfo(cdt).max
    b = rng.integers(0, full, size=d, dtype=cdt, endpoint=True)
    bp = rng.integers(0, full, size=d, dtype=cdt, endpoint=True)
    yh = rng.integers(0, full, size=(nd, d), dtype=cdt, endpoint=True)
    th = rng.integers(-(1 << (ld - 1)), 1 << (ld - 1), size=(nd, d)).astype(cdt)
    want = orc.finalize_matrix_pack(oparams(params), b, bp, yh, th)
    got = pir.finalize_matrix_pack(params, b, bp, yh, th)
    assert np.array_equal(got, want)


# ---------------------------------------------------------- PirServer -----
def _server_case(params, db_dtype, mat_dtype, seed, batch=1, pad_to=1,
                 first_dim_len=None, full_range=False, engine=0):
    mat = synthetic.make_material(params, seed=seed, db_dtype=db_dtype,
                                  mat_dtype=mat_dtype, pad_to=pad_to)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    fd, sd, pk = synthetic.make_requests(params, batch, seed=seed + 1,
                                         first_dim_len=first_dim_len,
                                         full_range=full_range)
    got = srv.process_arrays(fd, sd, pk, engine)
    op = oparams(params)
    for i in range(batch):
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i],
                                    sd[i], pk[i])
        assert np.array_equal(got[i], want), i
    return srv


# crypto/pir/server/pir_server_test.cc:55-143: (coeff, q, q1, q2, t, mat).
REF_TYPES = [
    ("Uint32Mod0", 32, 32, 31, 30, 32, np.int16),
    ("Uint32Mod30", 32, 30, 29, 28, 32, np.int16),
    ("Uint64Mod0", 64, 64, 61, 60, 32, np.int16),
    ("Uint64Mod62", 64, 62, 61, 60, 32, np.int32),
    ("Uint64Mod62ModSwitch", 64, 62, 28, 20, 32, np.int32),
    ("Uint32Mod0Interp1", 32, 32, 31, 30, 1, np.int16),
    ("Uint32Mod30Interp1", 32, 30, 29, 28, 1, np.int16),
    ("Uint64Mod0Interp1", 64, 64, 61, 60, 1, np.int16),
    ("Uint64Mod62Interp1", 64, 62, 61, 60, 1, np.int32),
]


@pytest.mark.parametrize("case", REF_TYPES, ids=[c[0] for c in REF_TYPES])
def test_server_reference_type_configs(case):
    _, cb, lq, lq1, lq2, t, mat = case
    nd = (lq + 1) // 2 - 1
    params = synthetic.make_params(d=32, n=1024, t=t, coeff_bits=cb, log_q=lq,
                                   log_q1=lq1, log_q2=lq2,
                                   plaintext_modulus=257, pack=(2, nd),
                                   evalg=(2, nd))
    _server_case(params, np.uint16, mat, seed=11, batch=3,
                 pad_to=32 if cb == 64 else 1)


def test_server_entry_size_multiple_3():
    # pir_server_test.cc:277-341: entry_size_multiple = 3.
    params = synthetic.make_params(d=32, n=1024, t=32, l=3, coeff_bits=64,
                                   log_q=62, log_q1=61, log_q2=60,
                                   plaintext_modulus=257, pack=(2, 30),
                                   evalg=(2, 30))
    _server_case(params, np.uint16, np.int32, seed=21, batch=2, pad_to=32)


def test_server_rows_not_multiple_of_d():
    # pir_server_test.cc:354-412: n/t not a multiple of d, short first dim.
    params = synthetic.make_params(d=32, n=1000, t=8, coeff_bits=32,
                                   log_q=32, plaintext_modulus=257,
                                   pack=(2, 15), evalg=(2, 15), log_q1=31,
                                   log_q2=30)
    _server_case(params, np.uint16, np.int16, seed=31, batch=2)


def test_server_metrics_tool_default_shape():
    # The pir_metrics_tool default parameter set at n=4096, d=2048, t=2:
    # u64 coefficients, q = 2^52, pack 19x2, eval 19x3, DB padded to 32.
    params = synthetic.make_params(d=2048, n=4096, t=2, coeff_bits=64,
                                   log_q=52)
    _server_case(params, np.uint16, np.int32, seed=41, batch=2, pad_to=32)


def test_server_u32_t4_shape():
    # Z_{2^32}, d=2048, t=4 (the n=65536 configuration at n=16384).
    params = synthetic.make_params(d=2048, n=16384, t=4, coeff_bits=32)
    _server_case(params, np.uint16, np.int32, seed=51, batch=2)


def test_server_u32_d4096_t8_small():
    params = synthetic.make_params(d=4096, n=8 * 8192, t=8, coeff_bits=32)
    _server_case(params, np.uint16, np.int32, seed=61, batch=1)


def test_server_u8_db_and_full_range_requests():
    params = synthetic.make_params(d=256, n=4096, t=4, coeff_bits=32,
                                   plaintext_modulus=255)
    _server_case(params, np.uint8, np.int32, seed=71, batch=2,
                 full_range=True)


def test_server_odd_columns_generic_path():
    # 1000/8 = 125 DB columns: rows are not 16-byte aligned.
    params = synthetic.make_params(d=64, n=1000, t=8, coeff_bits=64,
                                   log_q=52)
    _server_case(params, np.uint16, np.int32, seed=81, batch=1)


def test_server_short_first_dimension_is_zero_padded():
    params = synthetic.make_params(d=64, n=1024, t=2, coeff_bits=32)
    _server_case(params, np.uint16, np.int32, seed=91, batch=1, pad_to=96)


@pytest.mark.parametrize("d,n,t", [(4096, 2 * 4096, 2), (8192, 2 * 1024, 2),
                                   (2048, 4 * 2048, 4)])
def test_batch_shapes_of_the_polynomial_stage(d, n, t):
    # Large batches run the NTT kernels in their throughput shape (d/16
    # threads per block, or 1024 at d = 8192), single requests in the latency
    # shape (d/4 threads): both must give the oracle's bytes.
    params = synthetic.make_params(d=d, n=n, t=t, coeff_bits=32)
    mat = synthetic.make_material(params, seed=d + t)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    batch = 64
    fd, sd, pk = synthetic.make_requests(params, batch, seed=d + 1,
                                         full_range=True)
    got = srv.process_arrays(fd, sd, pk)
    for i in (0, 37, 63):
        one = srv.process_arrays(fd[i:i + 1], sd[i:i + 1], pk[i:i + 1])[0]
        assert np.array_equal(got[i], one), i
    op = oparams(params)
    for i in (0, 63):
        want = orc.process_response(op, mat.db, mat.pack, mat.a_tilde_agg,
                                    mat.t_vec_h, mat.second_dim_a, fd[i],
                                    sd[i], pk[i])
        assert np.array_equal(got[i], want), i


@pytest.mark.parametrize("engine", [pir.ENGINE_PLAIN, pir.ENGINE_TENSOR])
def test_device_call_short_first_dimension(engine):
    # Device-pointer call with n/t < DB columns: the padding is zeroed on the
    # device, the response equals the host call's.
    import torch
    params = synthetic.make_params(d=128, n=2 * 4000, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=5, pad_to=256)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    fd, sd, pk = synthetic.make_requests(params, 5, seed=6)
    assert fd.shape[1] == 4000 and mat.db.shape[1] == 4096
    want = srv.process_arrays(fd, sd, pk, pir.ENGINE_PLAIN)
    dev = torch.device("cuda", 0)
    t_fd, t_sd, t_pk = (torch.from_numpy(x.view(np.int32)).to(dev)
                        for x in (fd, sd, pk))
    out = torch.zeros((5, 1, 2, 128), dtype=torch.int32, device=dev)
    srv.process_device(5, t_fd.data_ptr(), 4000, t_sd.data_ptr(), sd.shape[1],
                       t_pk.data_ptr(), pk.shape[1], out.data_ptr(), engine,
                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want)


def test_server_request_validation():
    params = synthetic.make_params(d=64, n=1024, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=3)
    srv = pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                       mat.a_tilde_agg, mat.t_vec_h,
                                       mat.second_dim_a)
    fd, sd, pk = synthetic.make_requests(params, 1)
    with pytest.raises(pir.InspireError, match="Packing key must contain"):
        srv.process_arrays(fd, sd, pk[:, :3])
    with pytest.raises(pir.InspireError, match="First dimension query size"):
        srv.process_arrays(fd[:, :10], sd, pk)
    with pytest.raises(pir.InspireError,
                       match="second_dimension_query size mismatch"):
        srv.process_arrays(fd, sd[:, :4], pk)


def test_server_create_validation():
    params = synthetic.make_params(d=64, n=1024, t=2, coeff_bits=32)
    mat = synthetic.make_material(params, seed=3)
    with pytest.raises(pir.InspireError, match="td rows"):
        pir.PirServer.CreateCombined(params, mat.db[:10], mat.pack,
                                     mat.a_tilde_agg, mat.t_vec_h,
                                     mat.second_dim_a)
    with pytest.raises(pir.InspireError, match="second_dim_query_a"):
        pir.PirServer.CreateCombined(params, mat.db, mat.pack,
                                     mat.a_tilde_agg, mat.t_vec_h,
                                     mat.second_dim_a[:2])
