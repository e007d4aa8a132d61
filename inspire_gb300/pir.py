"""Python mirror of the reference PirServer API over the GB300 C ABI.

Names, argument meaning and error behaviour follow the reference
(google/InsPIRe):
  PirParams / RlweParams / GadgetParams   crypto/pir/pir_params.h:36-105,
                                          crypto/encryption.h:30-98
  PirRequest / PirResponse                crypto/pir/pir_params.h:196-216
  PreprocessMatrixPackOutput              crypto/lwes_to_rlwe.h:42-47
  PirPreprocessedData                     crypto/pir/server/pir_preprocessed_data.h
  PirServer::Create / ProcessResponse     crypto/pir/server/pir_server.h:45-72
Errors raise InspireError carrying the absl status code and the reference's
message. Every call runs the CUDA library; there is no CPU path.
"""
import ctypes
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib

INVALID_ARGUMENT = 3
DEADLINE_EXCEEDED = 4
RESOURCE_EXHAUSTED = 8
FAILED_PRECONDITION = 9
INTERNAL = 13

ENGINE_PLAIN = 0
ENGINE_TENSOR = 1
ENGINE_AUTO = 2   # per batch size, the server's tuned crossover
# Layouts of the tensor engine's DB operand (inspire_pir_tensor_products_device).
FORM_PLANES = 0   # resident fp16 digit planes
FORM_RAW = 1      # the u16 DB as stored, split into digits in shared memory
FORM_NARROW = 2   # or-ed in: 16 requests per tile instead of 64 (32 at u64)

KINDS = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1,
         np.dtype(np.uint32): 2, np.dtype(np.uint64): 3,
         np.dtype(np.int16): 4, np.dtype(np.int32): 5}


class InspireError(RuntimeError):
    """A non-OK status from the library (absl::Status equivalent)."""

    def __init__(self, code, message):
        super().__init__("status %d: %s" % (code, message))
        self.code = code
        self.message = message


def _check(rc, err):
    if rc != 0:
        raise InspireError(rc, err.value.decode(errors="replace"))


def _errbuf():
    return ctypes.create_string_buffer(1024)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


@dataclass(frozen=True)
class GadgetParams:
    log_digit: int
    num_digits: int


@dataclass(frozen=True)
class RlweParams:
    """RlweParams<CoeffType>: ring degree, log2 of q, q1, q2 (0 bits = 2^w)."""
    degree: int
    log_modulus: int
    log_modulus1_after_switch: int
    log_modulus2_after_switch: int
    variance: int = 0
    coeff_bits: int = 64

    def Degree(self):
        return self.degree

    def LogModulus(self):
        return self.log_modulus

    def LogModulus1AfterSwitch(self):
        return self.log_modulus1_after_switch

    def LogModulus2AfterSwitch(self):
        return self.log_modulus2_after_switch


@dataclass(frozen=True)
class PirParams:
    rlwe: RlweParams
    plaintext_modulus: int
    pack_gadget: GadgetParams
    eval_gadget: GadgetParams
    num_entries: int
    interpolation_degree: int
    entry_size_multiple: int = 1

    def RlweParameters(self):
        return self.rlwe

    def PlaintextModulus(self):
        return self.plaintext_modulus

    def PackGadgetParams(self):
        return self.pack_gadget

    def PolyEvalGadgetParams(self):
        return self.eval_gadget

    def NumEntries(self):
        return self.num_entries

    def InterpolationDegree(self):
        return self.interpolation_degree

    def EntrySizeMultiple(self):
        return self.entry_size_multiple

    def InterpolatedRows(self):
        return self.num_entries // self.interpolation_degree

    def NumFirstDimSamples(self):
        d = self.rlwe.degree
        return (self.InterpolatedRows() + d - 1) // d

    def PaddedCols(self):
        return self.NumFirstDimSamples() * self.rlwe.degree

    @property
    def coeff_dtype(self):
        return np.uint32 if self.rlwe.coeff_bits == 32 else np.uint64


@dataclass
class PreprocessMatrixPackOutput:
    a_tilde_agg: np.ndarray          # (d,)
    matrix: np.ndarray               # (d, k*d) MatCoeffType
    t_vec_h: np.ndarray              # (k, d)


@dataclass
class PirPreprocessedData:
    db_matrices: List[np.ndarray]                       # l x (t*d, cols)
    preprocessed_outputs: List[List[PreprocessMatrixPackOutput]]  # l x t
    second_dim_a: Optional[np.ndarray] = None           # (2*ne, d)


@dataclass
class PirRequest:
    first_dimension_query: np.ndarray                  # (n_first,)
    second_dimension_query: np.ndarray                 # (2*ne, d)
    packing_key: np.ndarray                            # (2*k, d)


@dataclass
class PirResponse:
    ciphertexts: np.ndarray                            # (l, 2, d): (a, b)


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "coeff_bits", "db_kind", "mat_kind", "log_degree", "log_modulus",
        "log_modulus1_after_switch", "log_modulus2_after_switch",
        "pack_log_digit", "pack_num_digits", "eval_log_digit",
        "eval_num_digits", "num_entries", "interpolation_degree",
        "entry_size_multiple")] + [("plaintext_modulus", ctypes.c_uint64)]


def c_params(params: PirParams, db_dtype=np.uint16, mat_dtype=np.int32):
    r = params.rlwe
    d = r.degree
    log_d = d.bit_length() - 1
    p = Params()
    p.coeff_bits = r.coeff_bits
    p.db_kind = KINDS[np.dtype(db_dtype)]
    p.mat_kind = KINDS[np.dtype(mat_dtype)]
    p.log_degree = log_d
    p.log_modulus = r.log_modulus
    p.log_modulus1_after_switch = r.log_modulus1_after_switch
    p.log_modulus2_after_switch = r.log_modulus2_after_switch
    p.pack_log_digit = params.pack_gadget.log_digit
    p.pack_num_digits = params.pack_gadget.num_digits
    p.eval_log_digit = params.eval_gadget.log_digit
    p.eval_num_digits = params.eval_gadget.num_digits
    p.num_entries = params.num_entries
    p.interpolation_degree = params.interpolation_degree
    p.entry_size_multiple = params.entry_size_multiple
    p.plaintext_modulus = params.plaintext_modulus
    return p


class PirServer:
    """GPU-resident PirServer<DbDataType, CoeffType, MatCoeffType>."""

    def __init__(self, handle, params, rows, db_cols, pack_cols):
        self._h = handle
        self.params = params
        self.rows = rows
        self.db_cols = db_cols
        self.pack_cols = pack_cols

    @staticmethod
    def Create(params: PirParams, data: PirPreprocessedData):
        """PirServer::Create (crypto/pir/server/pir_server.cc:54-124)."""
        t = params.interpolation_degree
        l = params.entry_size_multiple
        if len(data.db_matrices) != l:
            raise InspireError(INVALID_ARGUMENT, "db_matrices size mismatch.")
        if len(data.preprocessed_outputs) != l:
            raise InspireError(INVALID_ARGUMENT,
                               "preprocessed_outputs size mismatch.")
        for outs in data.preprocessed_outputs:
            if len(outs) != t:
                raise InspireError(INVALID_ARGUMENT,
                                   "Preprocessed outputs must be of length t.")
        db_cols = data.db_matrices[0].shape[1]
        for m in data.db_matrices:
            if m.shape[1] != db_cols:
                raise InspireError(
                    INVALID_ARGUMENT,
                    "All DB matrices must have the same number of columns.")
        # VerticalConcatenate (crypto/matrix.cc:162-206).
        db = np.ascontiguousarray(np.concatenate(data.db_matrices, axis=0))
        pack = np.ascontiguousarray(np.concatenate(
            [o.matrix for outs in data.preprocessed_outputs for o in outs],
            axis=0))
        cdt = params.coeff_dtype
        a_tilde = np.ascontiguousarray(np.stack(
            [o.a_tilde_agg for outs in data.preprocessed_outputs for o in outs]
        ).astype(cdt, copy=False))
        t_vec_h = np.ascontiguousarray(np.concatenate(
            [np.asarray(o.t_vec_h) for outs in data.preprocessed_outputs
             for o in outs]).astype(cdt, copy=False))
        return PirServer.CreateCombined(params, db, pack, a_tilde, t_vec_h,
                                        data.second_dim_a)

    @staticmethod
    def CreateCombined(params, db, pack, a_tilde_agg, t_vec_h, second_dim_a):
        """Create from the already-combined matrices (the server's own
        layout after VerticalConcatenate)."""
        lib = _lib.load()
        cdt = params.coeff_dtype
        d = params.rlwe.degree
        db = np.ascontiguousarray(db)
        pack = np.ascontiguousarray(pack)
        a_tilde_agg = np.ascontiguousarray(a_tilde_agg, dtype=cdt).reshape(-1, d)
        t_vec_h = np.ascontiguousarray(t_vec_h, dtype=cdt).reshape(-1, d)
        if second_dim_a is None:
            second_dim_a = np.zeros((0, d), dtype=cdt)
        second_dim_a = np.ascontiguousarray(second_dim_a, dtype=cdt).reshape(-1, d)
        prm = c_params(params, db.dtype, pack.dtype)
        h = ctypes.c_void_p()
        err = _errbuf()
        rc = lib.inspire_pir_server_create(
            ctypes.byref(prm), _ptr(db), db.shape[0], db.shape[1], _ptr(pack),
            pack.shape[0], pack.shape[1], _ptr(a_tilde_agg),
            a_tilde_agg.shape[0], _ptr(t_vec_h), t_vec_h.shape[0],
            _ptr(second_dim_a), second_dim_a.shape[0], ctypes.byref(h), err,
            len(err))
        _check(rc, err)
        return PirServer(h, params, db.shape[0], db.shape[1], pack.shape[1])

    @staticmethod
    def _from_handle(h, params):
        rows, dcols, pcols = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.load().inspire_pir_server_shape(h, ctypes.byref(rows),
                                             ctypes.byref(dcols),
                                             ctypes.byref(pcols))
        return PirServer(h, params, rows.value, dcols.value, pcols.value)

    @staticmethod
    def LoadFromBuffer(params, buffer, db_dtype=np.uint16, mat_dtype=np.int32):
        """PirServer::LoadFromBuffer (crypto/pir/server/pir_server.cc:590-780)
        into GPU memory; the template types come as numpy dtypes."""
        buf = np.frombuffer(bytes(buffer), dtype=np.uint8) \
            if not isinstance(buffer, np.ndarray) else buffer
        prm = c_params(params, db_dtype, mat_dtype)
        h = ctypes.c_void_p()
        err = _errbuf()
        rc = _lib.load().inspire_pir_server_load(
            ctypes.byref(prm), _ptr(buf), buf.size, ctypes.byref(h), err,
            len(err))
        _check(rc, err)
        return PirServer._from_handle(h, params)

    @staticmethod
    def LoadFromFile(params, path, db_dtype=np.uint16, mat_dtype=np.int32):
        """PirServer::LoadFromFile (pir_server.cc:782-791)."""
        prm = c_params(params, db_dtype, mat_dtype)
        h = ctypes.c_void_p()
        err = _errbuf()
        rc = _lib.load().inspire_pir_server_load_file(
            ctypes.byref(prm), str(path).encode(), ctypes.byref(h), err,
            len(err))
        _check(rc, err)
        return PirServer._from_handle(h, params)

    def SaveToBuffer(self):
        """The SaveToFile image (pir_server.cc:434-588) as bytes."""
        lib = _lib.load()
        err = _errbuf()
        size = ctypes.c_size_t()
        _check(lib.inspire_pir_server_save(self._h, None, 0, ctypes.byref(size),
                                           err, len(err)), err)
        out = np.empty(size.value, dtype=np.uint8)
        _check(lib.inspire_pir_server_save(self._h, _ptr(out), out.size,
                                           ctypes.byref(size), err, len(err)),
               err)
        return out.tobytes()

    def SaveToFile(self, path):
        """PirServer::SaveToFile (pir_server.cc:434-588)."""
        err = _errbuf()
        _check(_lib.load().inspire_pir_server_save_file(
            self._h, str(path).encode(), err, len(err)), err)

    @staticmethod
    def FromPirPreprocessedData(params, data, db_dtype=np.uint16,
                                mat_dtype=np.int32):
        """A serialized proto::PirPreprocessedData (what
        LoadPirPreprocessedDataFromFile reads,
        crypto/pir/server/pir_preprocessed_data.h:96-139) straight into a
        GPU server (DeserializePirPreprocessedData + PirServer::Create)."""
        buf = np.frombuffer(bytes(data), dtype=np.uint8)
        prm = c_params(params, db_dtype, mat_dtype)
        h = ctypes.c_void_p()
        err = _errbuf()
        rc = _lib.load().inspire_pir_server_load_preprocessed(
            ctypes.byref(prm), _ptr(buf), buf.size, ctypes.byref(h), err,
            len(err))
        _check(rc, err)
        return PirServer._from_handle(h, params)

    @staticmethod
    def FromPirPreprocessedDataFile(params, path, db_dtype=np.uint16,
                                    mat_dtype=np.int32):
        with open(path, "rb") as f:
            return PirServer.FromPirPreprocessedData(params, f.read(),
                                                     db_dtype, mat_dtype)

    @staticmethod
    def FromPirPreprocessedDataDirectory(params, path, db_dtype=np.uint16,
                                         mat_dtype=np.int32):
        """LoadPirPreprocessedDataFromDirectory (metadata.bin +
        shard_<i>.bin, pir_preprocessed_data.h:203-267) into a GPU server."""
        prm = c_params(params, db_dtype, mat_dtype)
        h = ctypes.c_void_p()
        err = _errbuf()
        rc = _lib.load().inspire_pir_server_load_preprocessed_dir(
            ctypes.byref(prm), str(path).encode(), ctypes.byref(h), err,
            len(err))
        _check(rc, err)
        return PirServer._from_handle(h, params)

    def SerializePirPreprocessedData(self):
        """SerializePirPreprocessedData(...).SerializeAsString() of the
        server's material."""
        lib = _lib.load()
        err = _errbuf()
        size = ctypes.c_size_t()
        _check(lib.inspire_pir_server_save_preprocessed(
            self._h, None, 0, ctypes.byref(size), err, len(err)), err)
        out = np.empty(size.value, dtype=np.uint8)
        _check(lib.inspire_pir_server_save_preprocessed(
            self._h, _ptr(out), out.size, ctypes.byref(size), err, len(err)),
            err)
        return out.tobytes()

    def SavePirPreprocessedDataToFile(self, path):
        with open(path, "wb") as f:
            f.write(self.SerializePirPreprocessedData())

    def SavePirPreprocessedDataToDirectory(self, path):
        """SavePirPreprocessedDataToDirectory (pir_preprocessed_data.h:141-201);
        the directory must exist."""
        err = _errbuf()
        _check(_lib.load().inspire_pir_server_save_preprocessed_dir(
            self._h, str(path).encode(), err, len(err)), err)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().inspire_pir_server_destroy(h)
            self._h = None

    def ProcessResponse(self, request: PirRequest) -> PirResponse:
        """PirServer::ProcessResponse (pir_server.cc:154-306)."""
        return self.ProcessBatch([request])[0]

    def ProcessBatch(self, requests, engine=ENGINE_PLAIN):
        """Answers several requests of equal shape in one pass."""
        cdt = self.params.coeff_dtype
        d = self.params.rlwe.degree
        fd = np.ascontiguousarray(np.stack(
            [np.asarray(r.first_dimension_query, dtype=cdt) for r in requests]))
        sd = np.ascontiguousarray(np.stack(
            [np.asarray(r.second_dimension_query, dtype=cdt).reshape(-1, d)
             for r in requests]))
        pk = np.ascontiguousarray(np.stack(
            [np.asarray(r.packing_key, dtype=cdt).reshape(-1, d)
             for r in requests]))
        out = self.process_arrays(fd, sd, pk, engine)
        return [PirResponse(ciphertexts=o) for o in out]

    def process_arrays(self, first_dim, second_dim, packing_key,
                       engine=ENGINE_PLAIN):
        """Stacked host arrays: (B, n1), (B, 2ne, d), (B, 2k, d) ->
        responses (B, l, 2, d)."""
        lib = _lib.load()
        cdt = self.params.coeff_dtype
        d = self.params.rlwe.degree
        l = self.params.entry_size_multiple
        first_dim = np.ascontiguousarray(first_dim, dtype=cdt)
        second_dim = np.ascontiguousarray(second_dim, dtype=cdt)
        packing_key = np.ascontiguousarray(packing_key, dtype=cdt)
        b = first_dim.shape[0]
        out = np.empty((b, l, 2, d), dtype=cdt)
        err = _errbuf()
        rc = lib.inspire_pir_process_batch(
            self._h, b, _ptr(first_dim), first_dim.shape[1], _ptr(second_dim),
            second_dim.shape[1] if second_dim.ndim == 3 else 0,
            _ptr(packing_key), packing_key.shape[1], _ptr(out), engine, err,
            len(err))
        _check(rc, err)
        return out

    def process_device(self, batch, first_dim_ptr, first_dim_len,
                       second_dim_ptr, second_dim_count, packing_key_ptr,
                       packing_key_count, responses_ptr, engine=ENGINE_PLAIN,
                       stream=0):
        """Device-resident batch: raw CUDA device pointers, async on stream."""
        lib = _lib.load()
        err = _errbuf()
        rc = lib.inspire_pir_process_batch_device(
            self._h, batch, ctypes.c_void_p(first_dim_ptr), first_dim_len,
            ctypes.c_void_p(second_dim_ptr), second_dim_count,
            ctypes.c_void_p(packing_key_ptr), packing_key_count,
            ctypes.c_void_p(responses_ptr), engine, ctypes.c_void_p(stream),
            err, len(err))
        _check(rc, err)

    def pack_device(self, batch, first_dim_ptr, first_dim_len,
                    packing_key_ptr, packing_key_count, out_ptr,
                    engine=ENGINE_PLAIN, stream=0):
        """Packing step of a device batch (products + FinalizeMatrixPack per
        shard, no EvalPoly or modulus switch): out is batch x l*t x 2 x d."""
        err = _errbuf()
        rc = _lib.load().inspire_pir_pack_batch_device(
            self._h, batch, ctypes.c_void_p(first_dim_ptr), first_dim_len,
            ctypes.c_void_p(packing_key_ptr), packing_key_count,
            ctypes.c_void_p(out_ptr), engine, ctypes.c_void_p(stream), err,
            len(err))
        _check(rc, err)

    def external_product_device(self, batch, ct_ptr, rgsw_ptr, out_ptr,
                                stream=0):
        """ExternalProduct of `batch` ciphertexts (batch x 2 x d) with their
        own RGSW ciphertexts (batch x 2ne x 2 x d) under the eval gadget."""
        err = _errbuf()
        rc = _lib.load().inspire_pir_external_product_device(
            self._h, batch, ctypes.c_void_p(ct_ptr), ctypes.c_void_p(rgsw_ptr),
            ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream), err, len(err))
        _check(rc, err)

    def tensor_products_device(self, batch, first_dim_ptr, packing_key_ptr,
                               out_ptr, form, split=0, stream=0):
        """Stage 1 (DB * q1 + P * y_g) of a device batch on the tensor engine
        in a given form (FORM_PLANES / FORM_RAW); split > 0 forces the
        split-K factor. first_dim holds db_cols words per request."""
        err = _errbuf()
        _check(_lib.load().inspire_pir_tensor_products_device(
            self._h, batch, ctypes.c_void_p(first_dim_ptr),
            ctypes.c_void_p(packing_key_ptr), ctypes.c_void_p(out_ptr), form,
            split, ctypes.c_void_p(stream), err, len(err)), err)

    def set_tensor_planes(self, keep):
        """Keep (True, the default) or drop the DB's resident fp16 digit
        planes of the tensor engine; without them the engine reads the u16
        DB as stored. Clears the tuned choices."""
        err = _errbuf()
        _check(_lib.load().inspire_pir_server_set_tensor_planes(
            self._h, 1 if keep else 0, err, len(err)), err)

    def device_bytes(self):
        """Resident device bytes: DB, pack matrix and digit planes."""
        return _lib.load().inspire_pir_server_device_bytes(self._h)

    def tune_engines(self, max_batch):
        """Times both engines at batch sizes up to max_batch and keeps the
        crossover for ENGINE_AUTO; returns it (0x7fffffff: never)."""
        err = _errbuf()
        c = ctypes.c_int32()
        _check(_lib.load().inspire_pir_tune_engines(self._h, max_batch,
                                                    ctypes.byref(c), err,
                                                    len(err)), err)
        return c.value

    def engine_table(self):
        """The last tune_engines measurements: a list of dicts (batch,
        plain_ms, tensor_ms, form, split)."""
        lib = _lib.load()
        n = lib.inspire_pir_engine_table(self._h, 0, None, None, None, None,
                                         None)
        if n <= 0:
            return []
        b = (ctypes.c_int32 * n)()
        pm = (ctypes.c_float * n)()
        tm = (ctypes.c_float * n)()
        f = (ctypes.c_int32 * n)()
        sp = (ctypes.c_int32 * n)()
        lib.inspire_pir_engine_table(self._h, n, b, pm, tm, f, sp)
        names = {FORM_PLANES: "planes", FORM_RAW: "raw"}
        return [{"batch": b[i], "plain_ms": pm[i], "tensor_ms": tm[i],
                 "form": names[f[i] & 1] + ("+narrow" if f[i] & FORM_NARROW
                                            else ""),
                 "split": sp[i]} for i in range(n)]

    def autotune(self, batch):
        """Tunes the tensor engine's split-K factor for this batch size;
        returns (factor, product ms)."""
        err = _errbuf()
        k, ms = ctypes.c_int32(), ctypes.c_float()
        _check(_lib.load().inspire_pir_autotune(self._h, batch, ctypes.byref(k),
                                                ctypes.byref(ms), err, len(err)),
               err)
        return k.value, ms.value

    def check(self):
        """Raises if a tensor-engine launch recorded a pipeline timeout."""
        err = _errbuf()
        _check(_lib.load().inspire_pir_server_check(self._h, err, len(err)),
               err)

    def _timings(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _lib.load().inspire_pir_server_timings(self._h, ctypes.byref(a),
                                               ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def GetDbMultiplyTime(self):
        """Accumulated DB product time in milliseconds."""
        return self._timings()[0]

    def GetPackingTime(self):
        return self._timings()[1]

    def GetPolyEvalTime(self):
        return self._timings()[2]


class Graph:
    """A CUDA graph of device entry points (inspire_graph_*).

        with Graph(stream) as g:       # records, does not run
            srv.process_device(..., stream=stream)
        g.launch(stream)               # replays as one launch

    Make each recorded call once before capturing, with the same batch
    sizes (that allocates the workspaces); a replay must not overlap other
    calls on the same server.
    """

    def __init__(self, stream):
        self.stream = stream
        self._g = None

    def __enter__(self):
        err = _errbuf()
        _check(_lib.load().inspire_graph_begin(ctypes.c_void_p(self.stream),
                                               err, len(err)), err)
        return self

    def __exit__(self, exc_type, exc, tb):
        err = _errbuf()
        g = ctypes.c_void_p()
        rc = _lib.load().inspire_graph_end(ctypes.c_void_p(self.stream),
                                           ctypes.byref(g), err, len(err))
        if exc_type is None:
            _check(rc, err)
            self._g = g
        elif g.value:
            _lib.load().inspire_graph_destroy(g)
        return False

    def launch(self, stream=None):
        err = _errbuf()
        s = self.stream if stream is None else stream
        _check(_lib.load().inspire_graph_launch(self._g, ctypes.c_void_p(s),
                                                err, len(err)), err)

    def __del__(self):
        if getattr(self, "_g", None) is not None and _lib._lib is not None:
            _lib._lib.inspire_graph_destroy(self._g)
            self._g = None


# ---------------------------------------------------------------------------
# Component entry points (reference functions one by one).
# ---------------------------------------------------------------------------
def matrix_multiply(mat, vec, coeff_bits):
    """Matrix<T>::Multiply<CoeffType> (crypto/matrix.h:167-195)."""
    lib = _lib.load()
    mat = np.ascontiguousarray(mat)
    cdt = np.uint32 if coeff_bits == 32 else np.uint64
    vec = np.ascontiguousarray(vec, dtype=cdt)
    if vec.shape[0] != mat.shape[1]:
        raise InspireError(INVALID_ARGUMENT,
                           "Vector size must match the number of matrix "
                           "columns.")
    out = np.zeros(mat.shape[0], dtype=cdt)
    err = _errbuf()
    rc = lib.inspire_matrix_multiply(KINDS[mat.dtype], coeff_bits, _ptr(mat),
                                     mat.shape[0], mat.shape[1], _ptr(vec),
                                     _ptr(out), err, len(err))
    _check(rc, err)
    return out


def inner_product(u, v, coeff_bits, u_bits=None, v_bits=None, chunk_bits=20,
                  u_signed=False):
    """Polynomial<T>::InnerProductFft (crypto/polynomial_fft.cc:68-197)."""
    lib = _lib.load()
    cdt = np.uint32 if coeff_bits == 32 else np.uint64
    u = np.ascontiguousarray(u, dtype=cdt)
    v = np.ascontiguousarray(v, dtype=cdt)
    if u.ndim == 1:
        u, v = u[None], v[None]
    n, d = u.shape
    out = np.zeros(d, dtype=cdt)
    err = _errbuf()
    rc = lib.inspire_inner_product(coeff_bits, _ptr(u), _ptr(v), n, d,
                                   u_bits or coeff_bits, v_bits or coeff_bits,
                                   chunk_bits, int(u_signed), _ptr(out), err,
                                   len(err))
    _check(rc, err)
    return out


def external_product(params: PirParams, ct_a, ct_b, rgsw):
    """ExternalProduct (crypto/external_product.cc:35-114)."""
    lib = _lib.load()
    cdt = params.coeff_dtype
    prm = c_params(params)
    ct_a = np.ascontiguousarray(ct_a, dtype=cdt)
    ct_b = np.ascontiguousarray(ct_b, dtype=cdt)
    rgsw = np.ascontiguousarray(rgsw, dtype=cdt)
    oa = np.zeros_like(ct_a)
    ob = np.zeros_like(ct_b)
    err = _errbuf()
    rc = lib.inspire_external_product(ctypes.byref(prm), _ptr(ct_a),
                                      _ptr(ct_b), _ptr(rgsw), _ptr(oa),
                                      _ptr(ob), err, len(err))
    _check(rc, err)
    return oa, ob


def finalize_matrix_pack(params: PirParams, b, b_agg_partial, y_vec_h,
                         t_vec_h):
    """FinalizeMatrixPack (crypto/lwes_to_rlwe.cc:448-479): the b part."""
    lib = _lib.load()
    cdt = params.coeff_dtype
    prm = c_params(params)
    arrs = [np.ascontiguousarray(x, dtype=cdt)
            for x in (b, b_agg_partial, y_vec_h, t_vec_h)]
    out = np.zeros(params.rlwe.degree, dtype=cdt)
    err = _errbuf()
    rc = lib.inspire_finalize_matrix_pack(ctypes.byref(prm),
                                          *[_ptr(a) for a in arrs], _ptr(out),
                                          err, len(err))
    _check(rc, err)
    return out


_VALUE_BITS = {np.dtype(np.uint8): 8, np.dtype(np.uint16): 16,
               np.dtype(np.uint32): 32}


def Interpolate(db_row, ring_degree, interpolation_degree, plaintext_modulus):
    """Interpolate (crypto/db_row_interpolation.h): t*d evaluations -> the
    t coefficient polynomials, on the GPU."""
    row = np.ascontiguousarray(db_row)
    bits = _VALUE_BITS.get(row.dtype)
    if bits is None:
        raise InspireError(INVALID_ARGUMENT, "value_bits must be 8, 16 or 32.")
    out = np.zeros_like(row)
    err = _errbuf()
    rc = _lib.load().inspire_interpolate(bits, _ptr(row), row.size, ring_degree,
                                         interpolation_degree,
                                         plaintext_modulus, _ptr(out), err,
                                         len(err))
    _check(rc, err)
    return out


def interpolate_db(db_raw, params: PirParams, out_cols=None):
    """PreprocessingServer's interpolation + transposition of every shard
    (crypto/pir/server/preprocessing_server.h:68-95, 174-209) on the GPU:
    the raw DB (num_entries records of l*d values, record-major) -> the
    combined DB matrix (l*t*d, out_cols), zero-padded past n/t columns."""
    raw = np.ascontiguousarray(db_raw).reshape(-1)
    bits = _VALUE_BITS.get(raw.dtype)
    if bits is None:
        raise InspireError(INVALID_ARGUMENT, "value_bits must be 8, 16 or 32.")
    d = params.rlwe.degree
    t = params.interpolation_degree
    l = params.entry_size_multiple
    n = params.num_entries
    cols = out_cols if out_cols is not None else n // t
    out = np.empty((l * t * d, cols), dtype=raw.dtype)
    err = _errbuf()
    rc = _lib.load().inspire_interpolate_db(
        bits, _ptr(raw), raw.size, n, d, t, l, params.plaintext_modulus,
        _ptr(out), cols, 0, None, err, len(err))
    _check(rc, err)
    return out


@dataclass
class VpirRequest:
    """VpirRequest (crypto/vpir/vpir_params.h:161-164)."""
    first_dimension_query: List[np.ndarray]   # N/d polynomials
    packing_key: List[np.ndarray]             # k (local finalize) or 2k


@dataclass
class VpirResponse:
    b_responses: np.ndarray                   # (ell, d)


class VpirServer:
    """VpirServer's online answer (crypto/vpir/server/vpir_server.cc:102-195)
    on the GPU: a server with interpolation degree 1 and ell shards whose
    response is the b polynomial of each shard."""

    def __init__(self, server: PirServer, local_finalize=False):
        if server.params.interpolation_degree != 1:
            raise InspireError(FAILED_PRECONDITION,
                               "a vPIR server has interpolation_degree 1.")
        self.server = server
        self.local_finalize = local_finalize

    @staticmethod
    def CreateCombined(params, db, pack, a_tilde_agg, t_vec_h,
                       local_finalize=False):
        d = params.rlwe.degree
        srv = PirServer.CreateCombined(params, db, pack, a_tilde_agg, t_vec_h,
                                       np.zeros((0, d), params.coeff_dtype))
        return VpirServer(srv, local_finalize)

    def process_arrays(self, first_dim, packing_key, engine=ENGINE_PLAIN):
        """(B, N) first dimensions and (B, K, d) packing keys -> (B, ell, d)."""
        p = self.server.params
        cdt = p.coeff_dtype
        d = p.rlwe.degree
        fd = np.ascontiguousarray(first_dim, dtype=cdt)
        pk = np.ascontiguousarray(packing_key, dtype=cdt)
        b = fd.shape[0]
        out = np.zeros((b, p.entry_size_multiple, d), dtype=cdt)
        err = _errbuf()
        rc = _lib.load().inspire_vpir_process_batch(
            self.server._h, b, _ptr(fd), fd.shape[1], _ptr(pk),
            pk.shape[1] if pk.ndim == 3 else 0,
            1 if self.local_finalize else 0, _ptr(out), engine, err, len(err))
        _check(rc, err)
        return out

    def ProcessResponse(self, request: VpirRequest) -> VpirResponse:
        fd = np.concatenate([np.asarray(x) for x in
                             request.first_dimension_query])[None, :]
        pk = np.stack([np.asarray(x) for x in request.packing_key])[None]
        return VpirResponse(self.process_arrays(fd, pk)[0])


def PreprocessMatrixPack(hint, pack_a, log_modulus, log_digit, num_digits,
                         mat_dtype=None, slices=None):
    """PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:414-446) on the GPU for
    every slice of a hint matrix, as PreprocessingServer does
    (crypto/pir/server/preprocessing_server.h:248-271).

    hint: (slices*d, >= d) u32/u64 (slice i's LWE a-vectors are rows
    i*d .. i*d+d-1, columns 0..d-1); pack_a: (2*num_digits, d), w_vec_g then
    w_vec_h. Returns (a_tilde_agg (slices, d), matrix (slices*d,
    num_digits*d) of mat_dtype (default: the coefficient type; int16 or
    int32 also), t_vec_h (slices, num_digits, d))."""
    h = np.ascontiguousarray(hint)
    pa = np.ascontiguousarray(pack_a)
    if h.dtype not in (np.dtype(np.uint32), np.dtype(np.uint64)) or h.ndim != 2:
        raise InspireError(INVALID_ARGUMENT, "hint must be a 2-D u32/u64 matrix.")
    pa = pa.astype(h.dtype, copy=False)
    if pa.ndim != 2:
        raise InspireError(INVALID_ARGUMENT, "pack_a must be (count, d).")
    count, d = pa.shape
    if slices is None:
        slices = h.shape[0] // d if d else 0
    mdt = np.dtype(mat_dtype) if mat_dtype is not None else h.dtype
    kind = {np.dtype(np.uint32): 2, np.dtype(np.uint64): 3,
            np.dtype(np.int16): 4, np.dtype(np.int32): 5}.get(mdt, -1)
    a_tilde = np.zeros((max(slices, 0), d), dtype=h.dtype)
    mat = np.zeros((max(slices, 0) * d, max(num_digits, 0) * d), dtype=mdt)
    t_h = np.zeros((max(slices, 0), max(num_digits, 0), d), dtype=h.dtype)
    err = _errbuf()
    rc = _lib.load().inspire_preprocess_matrix_pack(
        h.dtype.itemsize * 8, kind, log_modulus, log_digit, num_digits, d,
        slices, _ptr(h), h.shape[1], _ptr(pa), count, _ptr(a_tilde),
        _ptr(mat), _ptr(t_h), 0,
        None, err, len(err))
    _check(rc, err)
    return a_tilde, mat, t_h


class PreprocessingServer:
    """PreprocessingServer (crypto/pir/server/preprocessing_server.h:62-273)
    with every stage on the GPU: interpolation and transposition, the hint
    matrix, PreprocessMatrixPack per slice. The a-components come in as an
    array (the reference draws them from a ChaCha PRNG seeded by prng_seed,
    which this build does not have): NumFirstDimSamples first-dimension
    ones, 2*eval_num_digits second-dimension ones when t > 1, then
    2*pack_num_digits packing ones, each a polynomial of d words."""

    def __init__(self, params: PirParams, a_components):
        self.params = params
        self.a_components = np.ascontiguousarray(a_components,
                                                 dtype=params.coeff_dtype)
        p = params
        self.ns = p.NumFirstDimSamples()
        self.ne = 2 * p.eval_gadget.num_digits if p.interpolation_degree > 1 else 0
        self.np_ = 2 * p.pack_gadget.num_digits
        if self.a_components.shape != (self.ns + self.ne + self.np_,
                                       p.rlwe.degree):
            raise InspireError(INVALID_ARGUMENT,
                               "a_components must hold the first-dimension, "
                               "second-dimension and packing a-components.")

    @staticmethod
    def Create(params: PirParams, a_components):
        return PreprocessingServer(params, a_components)

    def Preprocess(self, db_raw, db_dtype=np.uint16, mat_dtype=np.int32):
        """PreprocessingServer::Preprocess: raw DB (num_entries records of
        entry_size_multiple*d values) -> PirPreprocessedData."""
        p = self.params
        d, t, l = p.rlwe.degree, p.interpolation_degree, p.entry_size_multiple
        raw = np.ascontiguousarray(db_raw, dtype=db_dtype)
        if raw.size != p.num_entries * d * l:
            raise InspireError(INVALID_ARGUMENT, "Invalid raw database size.")
        padded = p.PaddedCols()
        db_all = interpolate_db(raw, p, out_cols=padded)
        first = self.a_components[:self.ns]
        second = self.a_components[self.ns:self.ns + self.ne]
        pack_a = self.a_components[self.ns + self.ne:]
        cols = p.InterpolatedRows()
        if p.rlwe.coeff_bits == 64 and np.dtype(db_dtype).itemsize <= 2:
            # Condensed u64 DB rows (preprocessing_server.h:125-153).
            simd = 64 if np.dtype(db_dtype).itemsize == 1 else 32
            cols = (cols + simd - 1) // simd * simd
        mats, outs = [], []
        k = p.pack_gadget.num_digits
        for s in range(l):
            shard = db_all[s * t * d:(s + 1) * t * d]
            hint = ComputeHintMatrix(shard, first)
            a_t, mat, t_h = PreprocessMatrixPack(
                hint, pack_a, p.rlwe.log_modulus, p.pack_gadget.log_digit, k,
                mat_dtype=mat_dtype)
            outs.append([PreprocessMatrixPackOutput(a_t[i], mat[i * d:(i + 1) * d],
                                                    t_h[i]) for i in range(t)])
            m = np.zeros((t * d, cols), dtype=db_dtype)
            w = min(cols, padded)
            m[:, :w] = shard[:, :w]
            mats.append(m)
        return PirPreprocessedData(mats, outs, second if self.ne else None)


class PirClient:
    """PirClient (crypto/pir/client/pir_client.h) on the GPU, batched: one
    ternary secret key per client, requests for a batch of indices at once,
    responses decrypted at once. The errors come from a reproducible
    counter-based hash, not a cryptographic generator: for load generation
    and tests. variance: the RLWE error variance (the reference's metrics
    tools use 40, pir_metrics_tool.cc:79-87)."""

    def __init__(self, params: PirParams, a_components, secret_keys,
                 variance=40):
        self.params = params
        self.a_components = np.ascontiguousarray(a_components,
                                                 dtype=params.coeff_dtype)
        self.secret_keys = np.ascontiguousarray(secret_keys, dtype=np.int8)
        self.variance = variance
        self._seed = 0

    @staticmethod
    def Create(params: PirParams, a_components, clients=1, seed=0,
               variance=40):
        rng = np.random.default_rng(seed)
        keys = rng.integers(-1, 2, (clients, params.rlwe.degree), dtype=np.int8)
        c = PirClient(params, a_components, keys, variance)
        c._seed = int(rng.integers(0, 2**63))
        return c

    def CreateRequests(self, indices, seed=None):
        """Requests of clients 0..len(indices)-1 for their indices:
        (first_dim (B, n/t), second_dim (B, 2ne, d), packing_key (B, 2k, d))."""
        p = self.params
        idx = np.ascontiguousarray(indices, dtype=np.int64).reshape(-1)
        b = idx.size
        if b > self.secret_keys.shape[0]:
            raise InspireError(INVALID_ARGUMENT, "more indices than clients.")
        d = p.rlwe.degree
        ne = p.eval_gadget.num_digits if p.interpolation_degree > 1 else 0
        k = p.pack_gadget.num_digits
        cdt = p.coeff_dtype
        fd = np.zeros((b, p.InterpolatedRows()), dtype=cdt)
        sd = np.zeros((b, 2 * ne, d), dtype=cdt)
        pk = np.zeros((b, 2 * k, d), dtype=cdt)
        if seed is None:
            self._seed += 1
            seed = self._seed
        prm = c_params(p)
        err = _errbuf()
        rc = _lib.load().inspire_client_create_requests(
            ctypes.byref(prm), _ptr(self.secret_keys), _ptr(self.a_components),
            self.a_components.shape[0], _ptr(idx), b, seed, self.variance,
            _ptr(fd), _ptr(sd), _ptr(pk), 0, None, err, len(err))
        _check(rc, err)
        return fd, sd, pk

    def CreateRequest(self, index):
        fd, sd, pk = self.CreateRequests([index])
        return PirRequest(fd[0], sd[0], pk[0])

    def ProcessResponses(self, responses):
        """(B, l, 2, d) ciphertexts -> (B, l*d) plaintexts."""
        p = self.params
        r = np.ascontiguousarray(responses, dtype=p.coeff_dtype)
        b = r.shape[0]
        d, l = p.rlwe.degree, p.entry_size_multiple
        out = np.zeros((b, l * d), dtype=p.coeff_dtype)
        prm = c_params(p)
        err = _errbuf()
        rc = _lib.load().inspire_client_process_responses(
            ctypes.byref(prm), _ptr(self.secret_keys), _ptr(r), b, _ptr(out), 0,
            None, err, len(err))
        _check(rc, err)
        return out

    def ProcessResponse(self, response: PirResponse):
        return self.ProcessResponses(np.asarray(response.ciphertexts)[None])[0]


def ComputeHintMatrix(database, a_components):
    """ComputeHintMatrix (crypto/hint_computation.cc:78-160) on the GPU:
    database (rows, n*d) of u8/u16/u32, a_components (n, d) of u32/u64 ->
    (rows, d) in the a-components' type."""
    db = np.ascontiguousarray(database)
    a = np.ascontiguousarray(a_components)
    kind = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1,
            np.dtype(np.uint32): 2}.get(db.dtype)
    if kind is None or a.dtype not in (np.dtype(np.uint32), np.dtype(np.uint64)):
        raise InspireError(INVALID_ARGUMENT,
                           "database must be u8/u16/u32, a_components u32/u64.")
    rows = db.shape[0] if db.ndim == 2 else 0
    cols = db.shape[1] if db.ndim == 2 else 0
    n, d = (a.shape if a.ndim == 2 and a.size else (0, 0))
    out = np.zeros((rows, d), dtype=a.dtype)
    err = _errbuf()
    rc = _lib.load().inspire_compute_hint_matrix(
        kind, a.dtype.itemsize * 8, _ptr(db), rows, cols, _ptr(a), n, d,
        _ptr(out), 0, None, err, len(err))
    _check(rc, err)
    return out
