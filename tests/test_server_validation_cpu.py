"""Server creation's and the loaders' argument checks through the C ABI, on
the CPU.

PirParams::Create (crypto/pir/pir_params.cc:29-68), PirServer::Create's
shape checks (crypto/pir/server/pir_server.cc:58-95), LoadFromBuffer's
truncation errors and the PirPreprocessedData parse and structure checks run
before any device work, so their status codes and the reference's message
texts are checked here without a GPU. Valid inputs on a machine without a
GPU fail with an error (no host fallback).
"""
import dataclasses

import numpy as np
import pytest

from inspire_gb300 import _lib, build, pir, synthetic


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()
    return _lib.load()


@pytest.fixture(scope="module")
def material():
    params = synthetic.make_params(d=64, n=1024, t=2, coeff_bits=32)
    return params, synthetic.make_material(params, seed=3)


def create(params, mat, **override):
    args = dict(db=mat.db, pack=mat.pack, a_tilde_agg=mat.a_tilde_agg,
                t_vec_h=mat.t_vec_h, second_dim_a=mat.second_dim_a)
    args.update(override)
    return pir.PirServer.CreateCombined(params, **args)


@pytest.mark.parametrize("change,message", [
    (dict(num_entries=0), "num_entries must be strictly positive."),
    (dict(num_entries=-4), "num_entries must be strictly positive."),
    (dict(entry_size_multiple=0), "entry_size_multiple must be strictly positive."),
    (dict(interpolation_degree=3), "interpolation_degree must be a power of two."),
    (dict(interpolation_degree=0), "interpolation_degree must be a power of two."),
    (dict(num_entries=1025),
     "interpolation_degree (2) must divide num_entries (1025)."),
    (dict(interpolation_degree=256),
     "interpolation_degree (256) must be less than or equal to 2 * ring "
     "degree (128)."),
])
def test_pir_params_checks(material, change, message):
    params, mat = material
    bad = dataclasses.replace(params, **change)
    with pytest.raises(pir.InspireError) as e:
        create(bad, mat)
    assert e.value.code == pir.INVALID_ARGUMENT
    assert message in str(e.value)


def test_server_shape_checks(material):
    params, mat = material
    cases = [
        (dict(db=mat.db[:10]), "DB matrix must have td rows."),
        (dict(db=np.ascontiguousarray(mat.db[:, :100])),
         "DB matrix must have at least N/t columns."),
        (dict(a_tilde_agg=mat.a_tilde_agg[:1]), "Preprocessed outputs must be of length t."),
        (dict(pack=mat.pack[:10]),
         "Packing multiplication resulted in incorrect vector size."),
        (dict(second_dim_a=mat.second_dim_a[:2]),
         "second_dim_query_a must have length 2 * PolyEvalGadgetParams().num_digits."),
    ]
    for override, message in cases:
        with pytest.raises(pir.InspireError) as e:
            create(params, mat, **override)
        assert e.value.code == pir.INVALID_ARGUMENT, override.keys()
        assert message in str(e.value)


def test_valid_server_without_a_gpu_fails_loudly(material):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    params, mat = material
    with pytest.raises(pir.InspireError) as e:
        create(params, mat)
    assert e.value.code == pir.INTERNAL


def test_truncated_image_is_rejected(material):
    """LoadFromBuffer (pir_server.cc:590-780): a buffer that ends inside the
    DB matrix's header or data is an InternalError, before any device
    work."""
    import struct
    params, _ = material
    header = struct.pack("<iiBiQ", 4, 8, 0, 8, 32)  # 4 x 8 u16: 64 bytes
    for buf in (b"\x01\x02\x03", header, header + b"\x00" * 10,
                struct.pack("<iiBiQ", 4, 8, 0, 8, 31) + b"\x00" * 62):
        with pytest.raises(pir.InspireError) as e:
            pir.PirServer.LoadFromBuffer(params, buf)
        assert e.value.code == pir.INTERNAL
        assert "Error reading from buffer" in str(e.value)


def test_malformed_preprocessed_data_is_rejected(material):
    """DeserializePirPreprocessedData and PirServer::Create's structure
    checks on a proto::PirPreprocessedData (pir_preprocessed_data.h:160-172,
    pir_server.cc:58-95), before any device work."""
    from oracle import proto_format as pf
    params, _ = material
    d, log_q, k = params.rlwe.degree, params.rlwe.log_modulus, params.pack_gadget.num_digits
    rng = np.random.default_rng(5)
    db = rng.integers(0, 1 << 16, size=(2 * d, 8), dtype=np.uint16)

    def slice_out():
        mat = rng.integers(-5, 5, size=(d, 16)).astype(np.int32)
        return (rng.integers(0, 1 << 20, size=d), mat,
                [rng.integers(0, 1 << 20, size=d) for _ in range(k)])

    sda = [rng.integers(0, 1 << 20, size=d) for _ in range(2 * params.eval_gadget.num_digits)]
    cases = [
        (b"\xff" * 8, "Failed to parse PirPreprocessedData from file."),
        (pf.preprocessed_data([db], False, [], False, sda, log_q),
         "preprocessed_outputs size mismatch."),
        (pf.preprocessed_data([db, db], False, [[slice_out(), slice_out()]] * 2, False,
                              sda, log_q), "db_matrices size mismatch."),
        (pf.preprocessed_data([db], False, [[slice_out()]], False, sda, log_q),
         "Preprocessed outputs must be of length t."),
    ]
    for data, message in cases:
        with pytest.raises(pir.InspireError) as e:
            pir.PirServer.FromPirPreprocessedData(params, data)
        assert e.value.code == pir.INVALID_ARGUMENT, message
        assert message in str(e.value)
