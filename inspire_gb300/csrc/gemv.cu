// Plain (single- or few-query) fused GEMV over Z_{2^w}: the online DB product
// and the LWE-to-RLWE packing product of one request in one pass.
//
// Reference: Matrix<T>::Multiply (crypto/matrix.h:167-195) and the condensed
// Highway kernels CondensedMultiply<uint16_t/int32_t/uint8_t>
// (crypto/matrix.cc:261-462), called from PirServer::ProcessResponse
// (crypto/pir/server/pir_server.cc:215-248). Both products share their rows
// (l*t*d of them), and FinalizeMatrixPack only ever uses their sum
// (crypto/lwes_to_rlwe.cc:463-469), so the two matrices are streamed by the
// same CTA and summed into one accumulator per row.
//
// Design (HBM-bound): each CTA owns RB consecutive rows; every thread streams
// 16-byte vectors of RB rows at a time (ld.global.cs: the DB is read once per
// query, so it must not evict the query vectors, which stay L2-resident and
// are reused by every CTA). The query chunk is loaded once per iteration and
// reused for the RB rows and, when NQ > 1, each DB vector is reused for NQ
// queries. Warp shuffles, then shared memory, reduce the per-thread partial
// sums. Arithmetic wraps mod 2^w exactly like the reference's CoeffType.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <type_traits>

#include "internal.h"

namespace inspire {

int elem_size(int kind) {
  switch (kind) {
    case kU8: return 1;
    case kU16: return 2;
    case kU32: return 4;
    case kU64: return 8;
    case kI16: return 2;
    case kI32: return 4;
    default: return 0;
  }
}

namespace {

constexpr int kGemvDevices = 64;

struct NoMat {};

template <typename E>
struct Elem {
  static constexpr int kPerVec = 16 / sizeof(E);
};
template <>
struct Elem<NoMat> {
  static constexpr int kPerVec = 1;
};

// Streaming 16-byte load (evict-first): the matrices are touched once.
__device__ __forceinline__ uint4 ld_stream(const void* p) {
  return __ldcs(reinterpret_cast<const uint4*>(p));
}

// Loads N consecutive query words with the widest aligned vector loads.
template <typename T, int N>
__device__ __forceinline__ void load_query(const T* p, T (&v)[N]) {
  constexpr int kBytes = N * static_cast<int>(sizeof(T));
  if constexpr (kBytes % 16 == 0) {
#pragma unroll
    for (int k = 0; k < kBytes / 16; ++k)
      reinterpret_cast<uint4*>(v)[k] = __ldg(reinterpret_cast<const uint4*>(p) + k);
  } else if constexpr (kBytes == 8) {
    *reinterpret_cast<uint2*>(v) = __ldg(reinterpret_cast<const uint2*>(p));
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = __ldg(p + i);
  }
}

// Multiply-accumulate of one 16-byte matrix vector with the matching query
// elements. Signed matrix entries convert to T by sign extension, matching
// static_cast<OutputType>(m) in the reference.
template <typename T, typename E>
__device__ __forceinline__ T mac_vec(T acc, const uint4& w, const T* q) {
  alignas(16) E e[16 / sizeof(E)];
  *reinterpret_cast<uint4*>(e) = w;
#pragma unroll
  for (int i = 0; i < 16 / static_cast<int>(sizeof(E)); ++i) {
    acc += static_cast<T>(e[i]) * q[i];
  }
  return acc;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The RB row vectors at column c.
template <typename E, int RB>
__device__ __forceinline__ void load_rows(uint4 (&w)[RB], const E* m, int64_t cols,
                                          int64_t row0, int64_t rows, int64_t c) {
#pragma unroll
  for (int r = 0; r < RB; ++r) {
    const int64_t row = row0 + r;
    w[r] = row < rows ? ld_stream(m + row * cols + c) : make_uint4(0, 0, 0, 0);
  }
}

// One matrix segment: rows x cols of E, query rows of T. PF (a launch of one
// wave, a few iterations per thread): the next iteration's matrix vectors
// are loaded before this one's products, so a thread keeps two iterations'
// loads in flight instead of waiting out one round trip per iteration.
template <typename T, typename E, int RB, int NQ, int NT, bool PF>
__device__ __forceinline__ void segment(T (&acc)[RB][NQ], const E* m,
                                        int64_t cols, const T* q,
                                        int64_t q_stride, int64_t row0,
                                        int64_t rows) {
  constexpr int EPV = 16 / sizeof(E);  // matrix elements per 16-byte vector
  const int64_t nvec = cols / EPV;
  auto products = [&](const uint4 (&w)[RB], int64_t c) {
#pragma unroll
    for (int qi = 0; qi < NQ; ++qi) {
      alignas(16) T qv[EPV];
      load_query<T, EPV>(q + qi * q_stride + c, qv);
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r][qi] = mac_vec<T, E>(acc[r][qi], w[r], qv);
    }
  };
  if constexpr (PF) {
    int64_t v = threadIdx.x;
    if (v >= nvec) return;
    uint4 w[RB];
    load_rows<E, RB>(w, m, cols, row0, rows, v * EPV);
    for (;;) {
      uint4 cur[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) cur[r] = w[r];
      const int64_t c = v * EPV;
      v += NT;
      const bool more = v < nvec;
      if (more) load_rows<E, RB>(w, m, cols, row0, rows, v * EPV);
      products(cur, c);
      if (!more) break;
    }
  } else {
    for (int64_t v = threadIdx.x; v < nvec; v += NT) {
      uint4 w[RB];
      load_rows<E, RB>(w, m, cols, row0, rows, v * EPV);
      products(w, v * EPV);
    }
  }
}

// PF kernels (128 threads) are built for at least seven resident blocks per
// SM (72 registers a thread at most), so that a launch of up to 7 x 152
// blocks runs in one wave.
template <typename T, typename DbT, typename MatT, int RB, int NQ, int NT,
          bool PF = false>
__global__ void __launch_bounds__(NT, PF ? 896 / NT : 1)
fused_gemv_kernel(const DbT* __restrict__ db, int64_t db_cols,
                  const T* __restrict__ q1, int64_t q1_stride,
                  const MatT* __restrict__ pk, int64_t pk_cols,
                  const T* __restrict__ yg, int64_t yg_stride,
                  T* __restrict__ out, int64_t out_stride, int64_t rows) {
  T acc[RB][NQ];
#pragma unroll
  for (int r = 0; r < RB; ++r)
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[r][q] = 0;
  const int64_t row0 = static_cast<int64_t>(blockIdx.x) * RB;

  if (db_cols > 0)
    segment<T, DbT, RB, NQ, NT, PF>(acc, db, db_cols, q1, q1_stride, row0, rows);
  if constexpr (!std::is_same<MatT, NoMat>::value) {
    if (pk_cols > 0)
      segment<T, MatT, RB, NQ, NT, PF>(acc, pk, pk_cols, yg, yg_stride, row0, rows);
  }

  __shared__ T partial[NT / 32][RB * NQ];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < RB; ++r)
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      T s = warp_sum(acc[r][q]);
      if (lane == 0) partial[warp][r * NQ + q] = s;
    }
  __syncthreads();
  if (threadIdx.x < RB * NQ) {
    T s = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += partial[w][threadIdx.x];
    const int r = threadIdx.x / NQ;
    const int q = threadIdx.x % NQ;
    const int64_t row = row0 + r;
    if (row < rows) out[q * out_stride + row] = s;
  }
}

// Generic fallback for shapes whose rows are not 16-byte aligned: one warp
// per row, element-wise loads, run-time element kinds.
template <typename T>
__device__ __forceinline__ T load_as(const void* base, int kind, int64_t i) {
  switch (kind) {
    case kU8: return static_cast<T>(static_cast<const uint8_t*>(base)[i]);
    case kU16: return static_cast<T>(static_cast<const uint16_t*>(base)[i]);
    case kU32: return static_cast<T>(static_cast<const uint32_t*>(base)[i]);
    case kU64: return static_cast<T>(static_cast<const uint64_t*>(base)[i]);
    case kI16: return static_cast<T>(static_cast<const int16_t*>(base)[i]);
    default: return static_cast<T>(static_cast<const int32_t*>(base)[i]);
  }
}

template <typename T>
__global__ void generic_gemv_kernel(int db_kind, const void* db,
                                    int64_t db_cols, const T* q1,
                                    int64_t q1_stride, int pk_kind,
                                    const void* pk, int64_t pk_cols,
                                    const T* yg, int64_t yg_stride, T* out,
                                    int64_t out_stride, int64_t rows, int nq) {
  const int64_t row = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) +
                      (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  for (int q = 0; q < nq; ++q) {
    T acc = 0;
    for (int64_t c = lane; c < db_cols; c += 32) {
      acc += load_as<T>(db, db_kind, row * db_cols + c) * q1[q * q1_stride + c];
    }
    for (int64_t c = lane; c < pk_cols; c += 32) {
      acc += load_as<T>(pk, pk_kind, row * pk_cols + c) * yg[q * yg_stride + c];
    }
    acc = warp_sum(acc);
    if (lane == 0) out[q * out_stride + row] = acc;
  }
}

constexpr int kThreads = 256;

// Blocks of `kernel` (nt threads, no dynamic shared memory) that the current
// device holds at once; 0 if the runtime cannot say.
template <typename K>
int64_t resident_blocks(K kernel, int nt) {
  int dev = 0, per_sm = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, 0) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    return 0;
  }
  return static_cast<int64_t>(per_sm) * sms;
}

// resident_blocks, computed once per device and call site (`cache`).
template <typename K>
int64_t resident_cached(std::atomic<int64_t> (&cache)[kGemvDevices], K kernel, int nt) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kGemvDevices) {
    return resident_blocks(kernel, nt);
  }
  int64_t v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    v = resident_blocks(kernel, nt);
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

template <typename T, typename DbT, typename MatT, int RB, int NQ, int NT, bool PF>
cudaError_t launch_rows(int64_t blocks, const void* db, int64_t db_cols, const void* q1,
                        int64_t q1_stride, const void* pk, int64_t pk_cols,
                        const void* yg, int64_t yg_stride, void* out,
                        int64_t out_stride, int64_t rows, cudaStream_t stream) {
  fused_gemv_kernel<T, DbT, MatT, RB, NQ, NT, PF>
      <<<static_cast<unsigned>(blocks), NT, 0, stream>>>(
          static_cast<const DbT*>(db), db_cols, static_cast<const T*>(q1),
          q1_stride, static_cast<const MatT*>(pk), pk_cols,
          static_cast<const T*>(yg), yg_stride, static_cast<T*>(out),
          out_stride, rows);
  return cudaGetLastError();
}

template <typename T, typename DbT, typename MatT, int NQ>
cudaError_t launch_typed(const void* db, int64_t db_cols, const void* q1,
                         int64_t q1_stride, const void* pk, int64_t pk_cols,
                         const void* yg, int64_t yg_stride, void* out,
                         int64_t out_stride, int64_t rows,
                         cudaStream_t stream) {
  if constexpr (NQ == 1) {
    if (rows < 16384 && rows > 4 * 1216) {
      // Mid-size matrices (e.g. 8192 rows) take 2 rows per block, which
      // evens out the last of their waves: 0.84 instead of 0.78 of the copy
      // peak at 8192 x 16384 u16 + 8192 x 4096 i32.
      return launch_rows<T, DbT, MatT, 2, 1, kThreads, false>(
          (rows + 1) / 2, db, db_cols, q1, q1_stride, pk, pk_cols, yg, yg_stride, out,
          out_stride, rows, stream);
    }
    const int64_t blocks = (rows + 3) / 4;
    if (rows <= 4 * 1216) {
      // Small matrices: 4-row blocks. When 256-thread blocks would not all
      // fit on the device at once (at 64 registers a thread, four per SM)
      // but 128-thread ones would, the launch takes 128-thread blocks with
      // prefetching segments: one wave instead of a second, partly filled
      // one (4096 x 2048 u16 + 4096 x 4096 i32 over Z_2^64: 1.68 waves of
      // 256-thread blocks).
      static std::atomic<int64_t> fit256[kGemvDevices];
      static std::atomic<int64_t> fit128[kGemvDevices];
      if (blocks > resident_cached(fit256, fused_gemv_kernel<T, DbT, MatT, 4, 1, kThreads>,
                                   kThreads) &&
          blocks <= resident_cached(fit128, fused_gemv_kernel<T, DbT, MatT, 4, 1, 128, true>,
                                    128)) {
        return launch_rows<T, DbT, MatT, 4, 1, 128, true>(
            blocks, db, db_cols, q1, q1_stride, pk, pk_cols, yg, yg_stride, out, out_stride,
            rows, stream);
      }
    }
    return launch_rows<T, DbT, MatT, 4, 1, kThreads, false>(
        blocks, db, db_cols, q1, q1_stride, pk, pk_cols, yg, yg_stride, out, out_stride, rows,
        stream);
  } else {
    constexpr int RB = NQ >= 4 ? 2 : 4;
    return launch_rows<T, DbT, MatT, RB, NQ, kThreads, false>(
        (rows + RB - 1) / RB, db, db_cols, q1, q1_stride, pk, pk_cols, yg, yg_stride, out,
        out_stride, rows, stream);
  }
}

template <typename T, typename DbT, typename MatT>
cudaError_t launch_nq(int nq, const void* db, int64_t db_cols, const void* q1,
                      int64_t q1_stride, const void* pk, int64_t pk_cols,
                      const void* yg, int64_t yg_stride, void* out,
                      int64_t out_stride, int64_t rows, cudaStream_t stream) {
  // Split the batch into groups of 4, 2 and 1 queries.
  int done = 0;
  cudaError_t e = cudaSuccess;
  auto off_q = [&](const void* p, int64_t stride, int q) -> const void* {
    return p == nullptr ? nullptr
                        : static_cast<const char*>(p) + q * stride * sizeof(T);
  };
  while (done < nq && e == cudaSuccess) {
    const int left = nq - done;
    void* o = static_cast<char*>(out) + done * out_stride * sizeof(T);
    const void* a = off_q(q1, q1_stride, done);
    const void* b = off_q(yg, yg_stride, done);
    if (left >= 4) {
      e = launch_typed<T, DbT, MatT, 4>(db, db_cols, a, q1_stride, pk, pk_cols, b,
                                        yg_stride, o, out_stride, rows, stream);
      done += 4;
    } else if (left >= 2) {
      e = launch_typed<T, DbT, MatT, 2>(db, db_cols, a, q1_stride, pk, pk_cols, b,
                                        yg_stride, o, out_stride, rows, stream);
      done += 2;
    } else {
      e = launch_typed<T, DbT, MatT, 1>(db, db_cols, a, q1_stride, pk, pk_cols, b,
                                        yg_stride, o, out_stride, rows, stream);
      done += 1;
    }
  }
  return e;
}

template <typename T, typename DbT>
cudaError_t dispatch_pk(int pk_kind, const void* db, int64_t db_cols,
                        const void* q1, int64_t q1_stride, const void* pk,
                        int64_t pk_cols, const void* yg, int64_t yg_stride,
                        void* out, int64_t out_stride, int64_t rows, int nq,
                        cudaStream_t stream) {
  if (pk == nullptr || pk_cols == 0)
    return launch_nq<T, DbT, NoMat>(nq, db, db_cols, q1, q1_stride, nullptr, 0,
                                    nullptr, 0, out, out_stride, rows, stream);
  switch (pk_kind) {
    case kI16:
      return launch_nq<T, DbT, int16_t>(nq, db, db_cols, q1, q1_stride, pk, pk_cols,
                                        yg, yg_stride, out, out_stride, rows, stream);
    case kI32:
      return launch_nq<T, DbT, int32_t>(nq, db, db_cols, q1, q1_stride, pk, pk_cols,
                                        yg, yg_stride, out, out_stride, rows, stream);
    case kU32:
      return launch_nq<T, DbT, uint32_t>(nq, db, db_cols, q1, q1_stride, pk, pk_cols,
                                         yg, yg_stride, out, out_stride, rows, stream);
    case kU64:
      return launch_nq<T, DbT, uint64_t>(nq, db, db_cols, q1, q1_stride, pk, pk_cols,
                                         yg, yg_stride, out, out_stride, rows, stream);
    default:
      return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t dispatch_db(int db_kind, const void* db, int64_t db_cols,
                        const void* q1, int64_t q1_stride, int pk_kind,
                        const void* pk, int64_t pk_cols, const void* yg,
                        int64_t yg_stride, void* out, int64_t out_stride,
                        int64_t rows, int nq, cudaStream_t stream) {
  const bool with_pk = pk != nullptr && pk_cols > 0;
  switch (db_kind) {
    case kU8:
      return dispatch_pk<T, uint8_t>(pk_kind, db, db_cols, q1, q1_stride, pk, pk_cols,
                                     yg, yg_stride, out, out_stride, rows, nq, stream);
    case kU16:
      return dispatch_pk<T, uint16_t>(pk_kind, db, db_cols, q1, q1_stride, pk, pk_cols,
                                      yg, yg_stride, out, out_stride, rows, nq, stream);
    default:
      break;
  }
  // Remaining element kinds are only used as single matrices
  // (Matrix::Multiply on a u32/u64/i16/i32 matrix).
  if (with_pk) return cudaErrorInvalidValue;
  switch (db_kind) {
    case kU32:
      return launch_nq<T, uint32_t, NoMat>(nq, db, db_cols, q1, q1_stride, nullptr, 0,
                                           nullptr, 0, out, out_stride, rows, stream);
    case kU64:
      return launch_nq<T, uint64_t, NoMat>(nq, db, db_cols, q1, q1_stride, nullptr, 0,
                                           nullptr, 0, out, out_stride, rows, stream);
    case kI16:
      return launch_nq<T, int16_t, NoMat>(nq, db, db_cols, q1, q1_stride, nullptr, 0,
                                          nullptr, 0, out, out_stride, rows, stream);
    case kI32:
      return launch_nq<T, int32_t, NoMat>(nq, db, db_cols, q1, q1_stride, nullptr, 0,
                                          nullptr, 0, out, out_stride, rows, stream);
    default:
      return cudaErrorInvalidValue;
  }
}

bool aligned16(const void* p) {
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

}  // namespace

cudaError_t launch_fused_gemv(int coeff_bits, int db_kind, const void* db,
                              int64_t db_cols, const void* q1,
                              int64_t q1_stride, int pk_kind, const void* pk,
                              int64_t pk_cols, const void* yg,
                              int64_t yg_stride, void* out, int64_t out_stride,
                              int64_t rows, int nq, cudaStream_t stream) {
  if (rows <= 0 || nq <= 0) return cudaSuccess;
  const int wsz = coeff_bits / 8;
  const int dbs = elem_size(db_kind);
  const int pks = pk != nullptr && pk_cols > 0 ? elem_size(pk_kind) : 16;
  // The vector kernel needs 16-byte aligned rows, columns that fill whole
  // 16-byte vectors of both the matrix and the query, and aligned query rows.
  auto vec_ok = [&](const void* m, int64_t cols, int es, const void* q,
                    int64_t qs) {
    if (m == nullptr || cols == 0) return true;
    if (es == 0) return false;
    return aligned16(m) && aligned16(q) && (cols * es) % 16 == 0 &&
           (qs * wsz) % 16 == 0;
  };
  const bool fast = vec_ok(db, db_cols, dbs, q1, q1_stride) &&
                    vec_ok(pk, pk_cols, pks, yg, yg_stride);
  if (fast) {
    if (coeff_bits == 32)
      return dispatch_db<uint32_t>(db_kind, db, db_cols, q1, q1_stride, pk_kind, pk,
                                   pk_cols, yg, yg_stride, out, out_stride, rows, nq,
                                   stream);
    return dispatch_db<uint64_t>(db_kind, db, db_cols, q1, q1_stride, pk_kind, pk,
                                 pk_cols, yg, yg_stride, out, out_stride, rows, nq,
                                 stream);
  }
  const int threads = 256;
  const int64_t blocks = (rows + threads / 32 - 1) / (threads / 32);
  if (coeff_bits == 32) {
    generic_gemv_kernel<uint32_t><<<static_cast<unsigned>(blocks), threads, 0, stream>>>(
        db_kind, db, db_cols, static_cast<const uint32_t*>(q1), q1_stride, pk_kind, pk,
        pk_cols, static_cast<const uint32_t*>(yg), yg_stride,
        static_cast<uint32_t*>(out), out_stride, rows, nq);
  } else {
    generic_gemv_kernel<uint64_t><<<static_cast<unsigned>(blocks), threads, 0, stream>>>(
        db_kind, db, db_cols, static_cast<const uint64_t*>(q1), q1_stride, pk_kind, pk,
        pk_cols, static_cast<const uint64_t*>(yg), yg_stride,
        static_cast<uint64_t*>(out), out_stride, rows, nq);
  }
  return cudaGetLastError();
}

}  // namespace inspire
