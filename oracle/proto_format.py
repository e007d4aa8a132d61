"""Protobuf form of PirPreprocessedData (test infrastructure).

Restates the messages of crypto/proto/pir_server.proto and rlwe.proto
(Polynomial, Matrix, PreprocessMatrixPackOutput, PirPreprocessedData with its
ShardPreprocessedOutputs, PirPreprocessedShard, PirPreprocessedMetadata) as
SerializePirPreprocessedData / SavePirPreprocessedDataToDirectory fill them
(crypto/pir/server/pir_preprocessed_data.h:52-201): Matrix::ToProto sets
rows, cols (u64 words per row when condensed), is_condensed and
original_cols and the data or condensed_data bytes (crypto/matrix.cc:478-496);
Polynomial::ToProto packs log_modulus bits per coefficient, least significant
first (crypto/polynomial.cc:562-590). Encoded in protobuf wire format, fields
in number order, every set scalar written (explicit presence).

Only tests use this module: it writes the files the GPU loader must read and
checks the bytes the GPU saver writes.
"""
import numpy as np

from oracle.image_format import bitpack, bitunpack


def _varint(v):
    v &= (1 << 64) - 1
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def _bytes_field(num, b):
    return _varint(num << 3 | 2) + _varint(len(b)) + bytes(b)


def _int_field(num, v):
    return _varint(num << 3) + _varint(v)


def polynomial(coeffs, log_q):
    """Polynomial message of one polynomial (CoeffType words)."""
    return _bytes_field(1, bitpack(np.asarray(coeffs).astype(np.uint64), log_q))


def matrix(arr, condensed, original_cols=None):
    """Matrix message of a 2-D array (the condensed form has the same bytes,
    counted in u64 words per row)."""
    arr = np.ascontiguousarray(arr)
    rows, cols = arr.shape
    data = arr.tobytes()
    phys = cols * arr.dtype.itemsize // 8 if condensed else cols
    out = b""
    if data:
        out += _bytes_field(2 if condensed else 1, data)
    out += _int_field(3, rows) + _int_field(4, phys) + _int_field(5, 1 if condensed else 0)
    out += _int_field(6, cols if original_cols is None else original_cols)
    return out


def pack_output(a_tilde, mat, mat_condensed, t_vec_h, log_q):
    """PreprocessMatrixPackOutput message."""
    out = _bytes_field(1, polynomial(a_tilde, log_q))
    out += _bytes_field(2, matrix(mat, mat_condensed))
    for th in t_vec_h:
        out += _bytes_field(3, polynomial(th, log_q))
    return out


def preprocessed_data(db_matrices, db_condensed, outputs, mat_condensed,
                      second_dim_a, log_q, db_original_cols=None):
    """PirPreprocessedData: outputs[shard][slice] = (a_tilde, matrix, t_vec_h)."""
    out = b""
    for m in db_matrices:
        out += _bytes_field(1, matrix(m, db_condensed, db_original_cols))
    for shard in outputs:
        inner = b"".join(_bytes_field(1, pack_output(a, m, mat_condensed, th, log_q))
                         for a, m, th in shard)
        out += _bytes_field(2, inner)
    for p in (second_dim_a if second_dim_a is not None else []):
        out += _bytes_field(3, polynomial(p, log_q))
    return out


def shard_message(db, db_condensed, shard_outputs, mat_condensed, log_q,
                  db_original_cols=None):
    """PirPreprocessedShard (one shard_<i>.bin)."""
    out = _bytes_field(1, matrix(db, db_condensed, db_original_cols))
    for a, m, th in shard_outputs:
        out += _bytes_field(2, pack_output(a, m, mat_condensed, th, log_q))
    return out


def metadata_message(second_dim_a, log_q):
    """PirPreprocessedMetadata (metadata.bin)."""
    return b"".join(_bytes_field(1, polynomial(p, log_q))
                    for p in (second_dim_a if second_dim_a is not None else []))


def fields(buf):
    """Top-level fields of a message: list of (number, value), value an int
    for varints and bytes for length-delimited fields."""
    out, off = [], 0
    buf = bytes(buf)

    def varint():
        nonlocal off
        v, sh = 0, 0
        while True:
            b = buf[off]
            off += 1
            v |= (b & 0x7F) << sh
            sh += 7
            if not b & 0x80:
                return v
    while off < len(buf):
        key = varint()
        num, wt = key >> 3, key & 7
        if wt == 0:
            out.append((num, varint()))
        elif wt == 2:
            n = varint()
            out.append((num, buf[off:off + n]))
            off += n
        else:
            raise ValueError("unexpected wire type %d" % wt)
    return out


def decode_polynomial(msg, d, log_q, dtype):
    enc = dict(fields(msg)).get(1, b"")
    return bitunpack(enc, d, log_q, False).astype(dtype)
