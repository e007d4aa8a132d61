"""The oracle's protobuf restatement of PirPreprocessedData against the
protobuf runtime itself.

The message types of crypto/proto/pir_server.proto and rlwe.proto are built
at run time from descriptors (no protoc here), with explicit field presence
as edition 2024 gives them; messages filled the way
SerializePirPreprocessedData fills them (pir_preprocessed_data.h:52-94)
must serialize to the oracle's bytes, and the runtime must parse the
oracle's bytes back to the same fields.
"""
import numpy as np
import pytest

from oracle import proto_format as pf
from oracle.image_format import bitpack

pb = pytest.importorskip("google.protobuf")
from google.protobuf import descriptor_pb2, descriptor_pool  # noqa: E402
from google.protobuf import message_factory  # noqa: E402


def _types():
    fd = descriptor_pb2.FileDescriptorProto(name="pir_server_test.proto",
                                            package="t", syntax="proto2")
    F = descriptor_pb2.FieldDescriptorProto

    def msg(name, fields, nested=(), oneofs=()):
        m = fd.message_type.add(name=name) if isinstance(name, str) else name
        for o in oneofs:
            m.oneof_decl.add(name=o)
        for (fname, num, typ, label, tname, oneof) in fields:
            f = m.field.add(name=fname, number=num, type=typ, label=label)
            if tname:
                f.type_name = tname
            if oneof is not None:
                f.oneof_index = oneof
        return m
    opt, rep = F.LABEL_OPTIONAL, F.LABEL_REPEATED
    msg("Polynomial", [("encoded_coeffs", 1, F.TYPE_BYTES, opt, None, None)])
    msg("Matrix", [("data", 1, F.TYPE_BYTES, opt, None, 0),
                   ("condensed_data", 2, F.TYPE_BYTES, opt, None, 0),
                   ("rows", 3, F.TYPE_INT32, opt, None, None),
                   ("cols", 4, F.TYPE_INT32, opt, None, None),
                   ("is_condensed", 5, F.TYPE_BOOL, opt, None, None),
                   ("original_cols", 6, F.TYPE_INT32, opt, None, None)],
        oneofs=("matrix_data",))
    msg("PreprocessMatrixPackOutput", [
        ("a_tilde_agg", 1, F.TYPE_MESSAGE, opt, ".t.Polynomial", None),
        ("matrix", 2, F.TYPE_MESSAGE, opt, ".t.Matrix", None),
        ("t_vec_h", 3, F.TYPE_MESSAGE, rep, ".t.Polynomial", None)])
    data = msg("PirPreprocessedData", [
        ("db_matrices", 1, F.TYPE_MESSAGE, rep, ".t.Matrix", None),
        ("preprocessed_outputs", 2, F.TYPE_MESSAGE, rep,
         ".t.PirPreprocessedData.ShardPreprocessedOutputs", None),
        ("second_dim_a", 3, F.TYPE_MESSAGE, rep, ".t.Polynomial", None)])
    nested = data.nested_type.add(name="ShardPreprocessedOutputs")
    f = nested.field.add(name="outputs", number=1, type=F.TYPE_MESSAGE,
                         label=rep)
    f.type_name = ".t.PreprocessMatrixPackOutput"
    msg("PirPreprocessedShard", [
        ("db_matrix", 1, F.TYPE_MESSAGE, opt, ".t.Matrix", None),
        ("outputs", 2, F.TYPE_MESSAGE, rep, ".t.PreprocessMatrixPackOutput", None)])
    msg("PirPreprocessedMetadata", [
        ("second_dim_a", 1, F.TYPE_MESSAGE, rep, ".t.Polynomial", None)])
    pool = descriptor_pool.DescriptorPool()
    pool.Add(fd)
    return {n: message_factory.GetMessageClass(pool.FindMessageTypeByName("t." + n))
            for n in ("Polynomial", "Matrix", "PreprocessMatrixPackOutput",
                      "PirPreprocessedData", "PirPreprocessedShard",
                      "PirPreprocessedMetadata")}


T = _types()


def _fill_matrix(m, arr, condensed):
    arr = np.ascontiguousarray(arr)
    rows, cols = arr.shape
    m.rows = rows
    m.cols = cols * arr.dtype.itemsize // 8 if condensed else cols
    m.is_condensed = condensed
    m.original_cols = cols
    if arr.size:
        if condensed:
            m.condensed_data = arr.tobytes()
        else:
            m.data = arr.tobytes()


def _material(seed, d=16, t=2, l=2, k=2, log_q=29, cdt=np.uint32, mdt=np.int32):
    rng = np.random.default_rng(seed)
    dbs = [rng.integers(0, 65535, (t * d, 32), dtype=np.uint16) for _ in range(l)]
    outs = [[(rng.integers(0, 1 << log_q, d, dtype=np.uint64).astype(cdt),
              rng.integers(-2**20, 2**20, (d, k * d)).astype(mdt),
              rng.integers(0, 1 << log_q, (k, d), dtype=np.uint64).astype(cdt))
             for _ in range(t)] for _ in range(l)]
    sda = rng.integers(0, 1 << log_q, (6, d), dtype=np.uint64).astype(cdt)
    return dbs, outs, sda


def _poly(p, coeffs, log_q):
    p.encoded_coeffs = bitpack(np.asarray(coeffs).astype(np.uint64), log_q)


@pytest.mark.parametrize("log_q,db_cond,mat_cond", [(29, False, True),
                                                    (32, True, True),
                                                    (27, True, False)])
def test_preprocessed_data_bytes_match_protobuf(log_q, db_cond, mat_cond):
    dbs, outs, sda = _material(log_q, log_q=log_q)
    msg = T["PirPreprocessedData"]()
    for m in dbs:
        _fill_matrix(msg.db_matrices.add(), m, db_cond)
    for shard in outs:
        so = msg.preprocessed_outputs.add()
        for a, mat, th in shard:
            o = so.outputs.add()
            _poly(o.a_tilde_agg, a, log_q)
            _fill_matrix(o.matrix, mat, mat_cond)
            for p in th:
                _poly(o.t_vec_h.add(), p, log_q)
    for p in sda:
        _poly(msg.second_dim_a.add(), p, log_q)
    want = msg.SerializeToString()
    got = pf.preprocessed_data(dbs, db_cond, outs, mat_cond, sda, log_q)
    assert got == want
    back = T["PirPreprocessedData"]()
    back.ParseFromString(got)
    assert back == msg


def test_shard_and_metadata_bytes_match_protobuf():
    dbs, outs, sda = _material(3)
    shard = T["PirPreprocessedShard"]()
    _fill_matrix(shard.db_matrix, dbs[0], True)
    for a, mat, th in outs[0]:
        o = shard.outputs.add()
        _poly(o.a_tilde_agg, a, 29)
        _fill_matrix(o.matrix, mat, True)
        for p in th:
            _poly(o.t_vec_h.add(), p, 29)
    assert pf.shard_message(dbs[0], True, outs[0], True, 29) == shard.SerializeToString()
    meta = T["PirPreprocessedMetadata"]()
    for p in sda:
        _poly(meta.second_dim_a.add(), p, 29)
    assert pf.metadata_message(sda, 29) == meta.SerializeToString()


def test_decoder_reads_fields_back():
    d, log_q = 16, 29
    p = np.arange(d, dtype=np.uint32) * 12345
    msg = pf.polynomial(p, log_q)
    assert np.array_equal(pf.decode_polynomial(msg, d, log_q, np.uint32), p)
    m = pf.matrix(np.ones((2, 8), np.int32), True)
    f = dict(pf.fields(m))
    assert f[3] == 2 and f[4] == 4 and f[5] == 1 and f[6] == 8 and len(f[2]) == 64
