// Kernels of the polynomial stage of the online answer: the negacyclic
// products of FinalizeMatrixPack and of the EvalPoly external products, all
// as exact multi-prime NTTs, plus the Rescale epilogue.
//
// Reference: FinalizeMatrixPack (crypto/lwes_to_rlwe.cc:448-479),
// ExternalProduct (crypto/external_product.cc:35-114), EvalPoly and the
// modulus switch (crypto/pir/server/pir_server.cc:128-150, 283-297),
// Polynomial::{LowBits,GadgetInv,Rescale} (crypto/polynomial.cc:287-374).
#pragma once
#include <cstdint>

#include "arith.cuh"
#include "ntt.cuh"
#include "ntt16.cuh"

namespace inspire {

constexpr int kPolyThreads = 512;
constexpr int kMaxPer = 16;  // d / kPolyThreads for d <= 8192

// Kernels templated on ITERS (quads per thread per NTT double stage, so
// blockDim.x = d / (4 * ITERS)) keep PolyPer<ITERS> coefficients per thread;
// ITERS == 0 is the generic form (any block size, up to kMaxPer each).
// ITERS == 4 is the throughput shape of d <= 4096 (d/16 <= 256 threads,
// three blocks per SM); 1 and 2 run up to 1024 threads per block.
template <int ITERS>
struct PolyShape {
  static constexpr int kPer = ITERS == 0 ? kMaxPer : 4 * ITERS;
  static constexpr int kMaxThreads =
      ITERS == 4 ? 256 : ((ITERS == 1 || ITERS == 2) ? 1024 : kPolyThreads);
  static constexpr int kMinBlocks = ITERS == 4 ? 3 : 1;
};

template <typename T>
struct Bits {
  static constexpr int value = 8 * sizeof(T);
};

template <typename T>
__device__ __forceinline__ T low_bits(T x, int amount) {
  return amount >= Bits<T>::value ? x : (x & ((T{1} << amount) - 1));
}

template <typename T>
__device__ __forceinline__ T shr_or_zero(T x, int amount) {
  return amount >= Bits<T>::value ? T{0} : (x >> amount);
}

// Polynomial::Rescale: round(c * 2^lnew / 2^lcur) of the full word.
template <typename T>
__device__ __forceinline__ T rescale_word(T c, int lcur, int lnew) {
  if (lnew >= lcur) {
    const int s = lnew - lcur;
    return s >= Bits<T>::value ? T{0} : static_cast<T>(c << s);
  }
  const int s = lcur - lnew;
  if (s >= Bits<T>::value) return c >> (Bits<T>::value - 1);
  return (c >> s) + ((c >> (s - 1)) & T{1});
}

template <typename T>
__device__ __forceinline__ uint32_t to_residue(T x, uint32_t p) {
  if constexpr (sizeof(T) == 4) {
    return reduce_u32(x, p);
  } else {
    return reduce_u64(x, p);
  }
}

// Gadget digit `dg` of a LowBits'd coefficient (Polynomial::GadgetInv with
// the rounding shift when log_modulus > digits * log_digit).
template <typename T>
__device__ __forceinline__ T gadget_digit(T c, int log_modulus, int log_digit,
                                          int num_digits, int dg) {
  const int to_shift = log_modulus - num_digits * log_digit;
  T cur = c;
  if (to_shift > 0) {
    cur = (c >> to_shift) + ((c >> (to_shift - 1)) & T{1});
  }
  const int sh = dg * log_digit;
  cur = sh >= Bits<T>::value ? T{0} : (cur >> sh);
  return low_bits(cur, log_digit);
}

// Forward NTT of CoeffType polynomials (masked to the bits the reference's
// chunk rule reads). grid.x = npoly * r, grid.y = batch.
template <typename T, int ITERS = 0>
__global__ void __launch_bounds__(PolyShape<ITERS>::kMaxThreads, PolyShape<ITERS>::kMinBlocks)
ntt_coeffs_kernel(const T* __restrict__ src, int64_t src_qstride,
                  int64_t src_off, int npoly, T mask, uint32_t* __restrict__ dst,
                  int64_t poly_stride, NttCtx c) {
  extern __shared__ uint32_t smem[];
  const int d = 1 << c.logd;
  const int poly = blockIdx.x / c.r;
  const int pi = blockIdx.x % c.r;
  const int q = blockIdx.y;
  const uint32_t p = c.p[pi];
  const T* in = src + q * src_qstride + src_off + poly * poly_stride;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    smem[j] = to_residue<T>(in[j] & mask, p);
  }
  ntt_forward_t<ITERS>(smem, c, pi);
  uint32_t* out = dst + ((static_cast<int64_t>(q) * npoly + poly) * c.r + pi) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) out[j] = smem[j];
}

// ntt_coeffs_kernel for d = 2^LOGD with the radix-16 transform of ntt16.cuh,
// one block per polynomial over all primes (the input is read once).
// grid = (npoly, batch), d / 16 threads, needs c.tables16.
template <typename T, int LOGD>
__global__ void __launch_bounds__(Ntt16<LOGD>::kThreads, 512 / Ntt16<LOGD>::kThreads)
ntt_coeffs16_kernel(const T* __restrict__ src, int64_t src_qstride,
                    int64_t src_off, int npoly, T mask, uint32_t* __restrict__ dst,
                    int64_t poly_stride, NttCtx c) {
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  __shared__ uint32_t xs[d];
  const int tid = threadIdx.x;
  const int poly = blockIdx.x;
  const int q = blockIdx.y;
  const T* in = src + q * src_qstride + src_off + poly * poly_stride;
  T v[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = in[tid + NT * k] & mask;
  for (int pi = 0; pi < c.r; ++pi) {
    const uint32_t p = c.p[pi];
    uint32_t x[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = to_residue<T>(v[k], p);
    ntt16_forward<LOGD>(x, xs, c.tables16 + static_cast<size_t>(pi) * 4 * d, p, tid);
    uint4* out = reinterpret_cast<uint4*>(
        dst + ((static_cast<int64_t>(q) * npoly + poly) * c.r + pi) * d + 16 * tid);
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      out[w] = make_uint4(x[4 * w], x[4 * w + 1], x[4 * w + 2], x[4 * w + 3]);
    }
  }
}

// Forward NTT of signed 64-bit polynomials (host-prepared operands).
// Internal linkage: the header is shared by several translation units.
static __global__ void __launch_bounds__(kPolyThreads)
ntt_signed_kernel(const int64_t* __restrict__ src, int npoly,
                  uint32_t* __restrict__ dst, NttCtx c) {
  extern __shared__ uint32_t smem[];
  const int d = 1 << c.logd;
  const int poly = blockIdx.x / c.r;
  const int pi = blockIdx.x % c.r;
  const int64_t p = c.p[pi];
  const int64_t* in = src + static_cast<int64_t>(poly) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    int64_t v = in[j] % p;
    if (v < 0) v += p;
    smem[j] = static_cast<uint32_t>(v);
  }
  ntt_forward(smem, c, pi);
  uint32_t* out = dst + (static_cast<int64_t>(poly) * c.r + pi) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) out[j] = smem[j];
}

// sum_i U_i . V_i per prime, inverse NTT, CRT. One block; used by the
// InnerProductFft component entry point. U: [n][r][d], V: [n][r][d].
template <typename T>
__global__ void __launch_bounds__(kPolyThreads)
inner_product_finish_kernel(const uint32_t* __restrict__ U,
                            const uint32_t* __restrict__ V, int n,
                            T* __restrict__ out, NttCtx c) {
  extern __shared__ uint32_t smem[];  // [r][d]
  const int d = 1 << c.logd;
  for (int pi = 0; pi < c.r; ++pi) {
    const uint32_t p = c.p[pi];
    uint32_t* a = smem + static_cast<int64_t>(pi) * d;
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      uint32_t s = 0;
      for (int i = 0; i < n; ++i) {
        const int64_t off = (static_cast<int64_t>(i) * c.r + pi) * d + j;
        s = add_mod(s, mont_mul(U[off], V[off], p, c.pinv[pi]), p);
      }
      a[j] = s;
    }
    ntt_inverse(a, c, pi);
  }
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) {
        x[pi] = shoup_mul(smem[static_cast<int64_t>(pi) * d + j], c.scale[pi],
                          c.scale_s[pi], c.p[pi]);
      }
    }
    out[j] = crt_reconstruct<T>(x, c);
  }
}

// FinalizeMatrixPack for every (request, shard, slice):
//   b_agg = LowBits(LowBits(gemv) + sum_j t_h[j] (*) y_h[j], log_q)
// gemv already holds b' + b_agg_partial (optionally split in two vectors).
// grid.x = l * t slices, grid.y = batch. Th: [l*t][k][r][d] (Montgomery-free
// plain residues), Yh: [batch][k][r][d].
template <typename T, int ITERS = 0>
__global__ void __launch_bounds__(PolyShape<ITERS>::kMaxThreads, PolyShape<ITERS>::kMinBlocks)
finalize_kernel(const uint32_t* __restrict__ Th, const uint32_t* __restrict__ Yh,
                int k, const T* __restrict__ gemv, const T* __restrict__ gemv2,
                int64_t gemv_qstride, T* __restrict__ packed_b,
                int log_q, NttCtx c) {
  extern __shared__ uint32_t smem[];  // [r][d]
  const int d = 1 << c.logd;
  const int s = blockIdx.x;
  const int q = blockIdx.y;
  for (int pi = 0; pi < c.r; ++pi) {
    const uint32_t p = c.p[pi];
    uint32_t* a = smem + static_cast<int64_t>(pi) * d;
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      uint32_t acc = 0;
      for (int i = 0; i < k; ++i) {
        const uint32_t th = Th[((static_cast<int64_t>(s) * k + i) * c.r + pi) * d + j];
        const uint32_t yh = Yh[((static_cast<int64_t>(q) * k + i) * c.r + pi) * d + j];
        acc = add_mod(acc, mont_mul(th, yh, p, c.pinv[pi]), p);
      }
      a[j] = acc;
    }
    ntt_inverse_t<ITERS>(a, c, pi);
  }
  const int64_t base = q * gemv_qstride + static_cast<int64_t>(s) * d;
  T* outp = packed_b + (static_cast<int64_t>(q) * gridDim.x + s) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) {
        x[pi] = shoup_mul(smem[static_cast<int64_t>(pi) * d + j], c.scale[pi],
                          c.scale_s[pi], c.p[pi]);
      }
    }
    const T inner = crt_reconstruct<T>(x, c);
    T g = gemv[base + j];
    if (gemv2 != nullptr) g += gemv2[base + j];
    outp[j] = low_bits<T>(static_cast<T>(low_bits<T>(g, log_q) + inner), log_q);
  }
}

// finalize_kernel for d = 2^LOGD with the radix-16 inverse of ntt16.cuh: the
// products are taken in the slot layout the inverse starts from (16
// consecutive slots per thread, 16-byte loads), each prime's scaled result is
// kept in shared memory at the positions its thread reads back for the CRT.
// grid = (l * t, batch), d / 16 threads, (1 + r) * d words of shared memory,
// needs c.tables16.
template <typename T, int LOGD>
__global__ void __launch_bounds__(Ntt16<LOGD>::kThreads, 512 / Ntt16<LOGD>::kThreads)
finalize16_kernel(const uint32_t* __restrict__ Th, const uint32_t* __restrict__ Yh,
                  int k, const T* __restrict__ gemv, const T* __restrict__ gemv2,
                  int64_t gemv_qstride, T* __restrict__ packed_b, int log_q,
                  NttCtx c) {
  extern __shared__ uint32_t smem[];  // exchange buffer, then [r][d] results
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  uint32_t* xs = smem;
  uint32_t* res = smem + d;
  const int tid = threadIdx.x;
  const int s = blockIdx.x;
  const int q = blockIdx.y;
  for (int pi = 0; pi < c.r; ++pi) {
    const uint32_t p = c.p[pi];
    const uint32_t pinv = c.pinv[pi];
    uint32_t acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = 0;
    for (int i = 0; i < k; ++i) {
      const uint4* th = reinterpret_cast<const uint4*>(
          Th + ((static_cast<int64_t>(s) * k + i) * c.r + pi) * d + 16 * tid);
      const uint4* yh = reinterpret_cast<const uint4*>(
          Yh + ((static_cast<int64_t>(q) * k + i) * c.r + pi) * d + 16 * tid);
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint4 a = __ldg(th + w), b = __ldg(yh + w);
        acc[4 * w] = add_mod(acc[4 * w], mont_mul(a.x, b.x, p, pinv), p);
        acc[4 * w + 1] = add_mod(acc[4 * w + 1], mont_mul(a.y, b.y, p, pinv), p);
        acc[4 * w + 2] = add_mod(acc[4 * w + 2], mont_mul(a.z, b.z, p, pinv), p);
        acc[4 * w + 3] = add_mod(acc[4 * w + 3], mont_mul(a.w, b.w, p, pinv), p);
      }
    }
    ntt16_inverse<LOGD>(acc, xs, c.tables16 + static_cast<size_t>(pi) * 4 * d, p, tid);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      res[pi * d + tid + NT * j] = shoup_mul(acc[j], c.scale[pi], c.scale_s[pi], p);
    }
  }
  const int64_t base = q * gemv_qstride + static_cast<int64_t>(s) * d;
  T* outp = packed_b + (static_cast<int64_t>(q) * gridDim.x + s) * d;
  for (int jj = 0; jj < 16; ++jj) {
    const int j = tid + NT * jj;
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) x[pi] = res[pi * d + j];
    }
    const T inner = crt_reconstruct<T>(x, c);
    T g = gemv[base + j];
    if (gemv2 != nullptr) g += gemv2[base + j];
    outp[j] = low_bits<T>(static_cast<T>(low_bits<T>(g, log_q) + inner), log_q);
  }
}

// finalize16_kernel for launches with fewer blocks than SMs: NGR groups of
// d / 16 threads, group g taking primes g, g + NGR, ... side by side, each
// with its prime's inverse tables copied to shared memory and the compact
// inverse (a block runs once per SM: global twiddle reads would each wait on
// L2 and the unrolled code on instruction fetch); then the whole block does
// the CRT. grid = (l * t, batch), shared memory (3 NGR + r) * d words, needs
// c.tables16.
template <typename T, int LOGD, int NGR = 2>
__global__ void __launch_bounds__(NGR * Ntt16<LOGD>::kThreads, 1)
finalize16_pair_kernel(const uint32_t* __restrict__ Th, const uint32_t* __restrict__ Yh,
                       int k, const T* __restrict__ gemv, const T* __restrict__ gemv2,
                       int64_t gemv_qstride, T* __restrict__ packed_b, int log_q,
                       NttCtx c) {
  extern __shared__ uint32_t smem[];
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  const int tid = threadIdx.x;
  const int grp = tid / NT;
  const int lt = tid & (NT - 1);
  const int bar = 1 + grp;
  uint32_t* xs = smem + grp * d;
  uint32_t* itab = smem + NGR * d + grp * 2 * d;  // IW | IW shoup of the prime
  uint32_t* res = smem + 3 * NGR * d;             // [r][d] scaled residues
  const int s = blockIdx.x;
  const int q = blockIdx.y;
  for (int pi = grp; pi < c.r; pi += NGR) {
    const uint32_t p = c.p[pi];
    const uint32_t pinv = c.pinv[pi];
    const uint4* g16 = reinterpret_cast<const uint4*>(
        c.tables16 + static_cast<size_t>(pi) * 4 * d + 2 * d);
    uint4* s16 = reinterpret_cast<uint4*>(itab);
#pragma unroll
    for (int i = 0; i < 2 * d / 4 / NT; ++i) {
      s16[lt + i * NT] = __ldg(g16 + lt + i * NT);
    }
    uint32_t acc[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j] = 0;
    for (int i = 0; i < k; ++i) {
      const uint4* th = reinterpret_cast<const uint4*>(
          Th + ((static_cast<int64_t>(s) * k + i) * c.r + pi) * d + 16 * lt);
      const uint4* yh = reinterpret_cast<const uint4*>(
          Yh + ((static_cast<int64_t>(q) * k + i) * c.r + pi) * d + 16 * lt);
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const uint4 a = __ldg(th + w), b = __ldg(yh + w);
        acc[4 * w] = add_mod(acc[4 * w], mont_mul(a.x, b.x, p, pinv), p);
        acc[4 * w + 1] = add_mod(acc[4 * w + 1], mont_mul(a.y, b.y, p, pinv), p);
        acc[4 * w + 2] = add_mod(acc[4 * w + 2], mont_mul(a.z, b.z, p, pinv), p);
        acc[4 * w + 3] = add_mod(acc[4 * w + 3], mont_mul(a.w, b.w, p, pinv), p);
      }
    }
    ntt16_sync<LOGD>(bar);  // the group's copy of the tables is complete
    ntt16_inverse_tw<LOGD, true, true>(acc, xs, itab, itab + d, p, lt, bar);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      res[pi * d + lt + NT * j] = shoup_mul(acc[j], c.scale[pi], c.scale_s[pi], p);
    }
  }
  __syncthreads();
  const int64_t base = q * gemv_qstride + static_cast<int64_t>(s) * d;
  T* outp = packed_b + (static_cast<int64_t>(q) * gridDim.x + s) * d;
#pragma unroll 4
  for (int j = tid; j < d; j += NGR * NT) {
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) x[pi] = res[pi * d + j];
    }
    const T inner = crt_reconstruct<T>(x, c);
    T g = gemv[base + j];
    if (gemv2 != nullptr) g += gemv2[base + j];
    outp[j] = low_bits<T>(static_cast<T>(low_bits<T>(g, log_q) + inner), log_q);
  }
}

// The packed ciphertexts as (a_tilde_agg, b_agg) pairs:
// out[q][s] = (a[s], b[q][s]). grid = (shards, batch).
template <typename T>
__global__ void __launch_bounds__(kPolyThreads)
pack_out_kernel(const T* __restrict__ a, const T* __restrict__ b, int d,
                T* __restrict__ out) {
  const int s = blockIdx.x;
  const int64_t qs = static_cast<int64_t>(blockIdx.y) * gridDim.x + s;
  const T* as = a + static_cast<int64_t>(s) * d;
  const T* bs = b + qs * d;
  T* o = out + qs * 2 * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    o[j] = as[j];
    o[d + j] = bs[j];
  }
}

// ComputeHintMatrix (crypto/hint_computation.cc:78-160) per (DB row,
// prime): sum over the n column blocks of NTT(row block) . V_k, then the
// inverse NTT. V: [n][r][d] transforms of the inverted a-components
// (v_k[0] = a_k[0], v_k[j] = -a_k[d-j]); out: [rows][r][d] residues.
// grid = (r, rows).
template <typename S, int ITERS = 0>
__global__ void __launch_bounds__(PolyShape<ITERS>::kMaxThreads, PolyShape<ITERS>::kMinBlocks)
hint_rows_kernel(const S* __restrict__ db, int64_t cols, int n,
                 const uint32_t* __restrict__ V, uint32_t* __restrict__ out,
                 NttCtx c) {
  extern __shared__ uint32_t smem[];
  const int d = 1 << c.logd;
  const int pi = blockIdx.x;
  const int64_t row = blockIdx.y;
  const uint32_t p = c.p[pi];
  const uint32_t pinv = c.pinv[pi];
  constexpr int kPer = PolyShape<ITERS>::kPer;
  uint32_t acc[kPer];
#pragma unroll
  for (int m = 0; m < kPer; ++m) acc[m] = 0;
  const S* src = db + row * cols;
  for (int k = 0; k < n; ++k) {
    __syncthreads();
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      smem[j] = reduce_u32(static_cast<uint32_t>(src[static_cast<int64_t>(k) * d + j]), p);
    }
    ntt_forward_t<ITERS>(smem, c, pi);
    const uint32_t* vk = V + (static_cast<int64_t>(k) * c.r + pi) * d;
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
      const int j = threadIdx.x + m * blockDim.x;
      if (j < d) acc[m] = add_mod(acc[m], mont_mul(smem[j], __ldg(vk + j), p, pinv), p);
    }
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < kPer; ++m) {
    const int j = threadIdx.x + m * blockDim.x;
    if (j < d) smem[j] = acc[m];
  }
  ntt_inverse_t<ITERS>(smem, c, pi);
  uint32_t* o = out + (row * c.r + pi) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    o[j] = shoup_mul(smem[j], c.scale[pi], c.scale_s[pi], p);
  }
}

// hint_rows_kernel for d = 2^LOGD with the radix-16 register transforms of
// ntt16.cuh: one block per (prime, DB row), d / 16 threads; a thread reads
// coefficients tid + (d/16) q of each row block (coalesced), the forward
// transform leaves it slots 16 tid + q (in [0, 2p), straight into the
// Montgomery products with 16-byte loads of V), and the inverse starts from
// the accumulators. Same residues as hint_rows_kernel. grid = (r, rows),
// d words of shared memory, needs c.tables16.
template <typename S, int LOGD>
__global__ void __launch_bounds__(Ntt16<LOGD>::kThreads, 512 / Ntt16<LOGD>::kThreads)
hint_rows16_kernel(const S* __restrict__ db, int64_t cols, int n,
                   const uint32_t* __restrict__ V, uint32_t* __restrict__ out,
                   NttCtx c) {
  extern __shared__ uint32_t smem[];
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  constexpr bool kCompact = true;  // the unrolled form spills at d = 4096
  const int pi = blockIdx.x;
  const int64_t row = blockIdx.y;
  const int tid = threadIdx.x;
  const uint32_t p = c.p[pi];
  const uint32_t pinv = c.pinv[pi];
  const uint32_t* tab16 = c.tables16 + static_cast<size_t>(pi) * 4 * d;
  uint32_t acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0;
  const S* src = db + row * cols;
  for (int k = 0; k < n; ++k) {
    uint32_t x[16];
    const S* rk = src + static_cast<int64_t>(k) * d + tid;  // + NT q: immediates
#pragma unroll
    for (int q = 0; q < 16; ++q) x[q] = reduce_u32(static_cast<uint32_t>(rk[NT * q]), p);
    ntt16_forward<LOGD, false, kCompact, true>(x, smem, tab16, p, tid);
    const uint4* vk = reinterpret_cast<const uint4*>(
        V + (static_cast<int64_t>(k) * c.r + pi) * d + 16 * tid);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const uint4 w = __ldg(vk + v);
      const uint32_t wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[4 * v + i] = add_mod(acc[4 * v + i], mont_mul(x[4 * v + i], wv[i], p, pinv), p);
      }
    }
  }
  ntt16_inverse<LOGD, false, kCompact>(acc, smem, tab16, p, tid);
  uint32_t* o = out + (row * c.r + pi) * d + tid;
#pragma unroll
  for (int q = 0; q < 16; ++q) o[NT * q] = shoup_mul(acc[q], c.scale[pi], c.scale_s[pi], p);
}

// CRT of the hint residues: out[row][j] = the integer mod 2^w.
template <typename T>
__global__ void hint_crt_kernel(const uint32_t* __restrict__ res, int64_t rows, int d,
                                T* __restrict__ out, NttCtx c) {
  const int64_t total = rows * d;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t row = i / d;
    const int j = static_cast<int>(i % d);
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) x[pi] = res[(row * c.r + pi) * d + j];
    }
    out[i] = crt_reconstruct<T>(x, c);
  }
}

struct ExtArgs {
  int log_q;         // LowBits width and GadgetInv log_modulus
  int log_digit;
  int num_digits;    // eval gadget digits (ne)
  int live_digits;   // digits that can be non-zero; the rest are identically 0
  uint64_t umask;    // bits of a digit the chunk rule reads
};

// Gadget digits at or above the coefficient's width are always zero (e.g.
// digit 2 of a 19 x 3 gadget over 32-bit coefficients): their products are
// zero and are skipped.
inline int LiveDigits(int log_q, int log_digit, int num_digits) {
  if (log_q - num_digits * log_digit > 0) return num_digits;
  const int live = (log_q + log_digit - 1) / log_digit;
  return live < num_digits ? live : num_digits;
}

// Reads the Horner state of one coefficient: either the packed ciphertext
// itself (first step) or CRT(previous product residues) + packed ciphertext.
template <typename T>
__device__ __forceinline__ void horner_state(
    bool first, const uint32_t* __restrict__ resid_in, int64_t resid_base, int d,
    int j, const T* __restrict__ ca, const T* __restrict__ cb, const NttCtx& c,
    T& ra, T& rb) {
  if (first) {
    ra = ca[j];
    rb = cb[j];
    return;
  }
  uint32_t xa[kMaxPrimes] = {0, 0, 0, 0, 0};
  uint32_t xb[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int pi = 0; pi < kMaxPrimes; ++pi) {
    if (pi < c.r) {
      const int64_t o = resid_base + static_cast<int64_t>(pi) * 2 * d + j;
      xa[pi] = resid_in[o];
      xb[pi] = resid_in[o + d];
    }
  }
  ra = crt_reconstruct<T>(xa, c) + (ca != nullptr ? ca[j] : T{0});
  rb = crt_reconstruct<T>(xb, c) + (cb != nullptr ? cb[j] : T{0});
}

// One external product per (request, shard) and prime:
//   digits of LowBits(state) -> NTT -> MAC with the RGSW NTTs -> INTT.
// Writes scaled residues of (a', b') to resid_out[q][shard][prime][2][d].
// grid = (r, l, batch). RGSWa: [2ne][r][d] (server; rgswa_qstride = 0) or
// [batch][2ne][r][d] (rgswa_qstride = 2ne*r*d), RGSWb: [batch][2ne][r][d]. coeff_a/coeff_b select the packed
// ciphertext added to the previous product (or the initial state).
template <typename T, int ITERS = 0>
__global__ void __launch_bounds__(PolyShape<ITERS>::kMaxThreads, PolyShape<ITERS>::kMinBlocks)
ext_step_kernel(bool first, const uint32_t* __restrict__ resid_in,
                uint32_t* __restrict__ resid_out,
                const T* __restrict__ coeff_a, int64_t coeff_a_q_stride,
                int64_t coeff_a_shard_stride,
                const T* __restrict__ coeff_b, int64_t coeff_b_q_stride,
                int64_t coeff_b_shard_stride,
                const uint32_t* __restrict__ RGSWa, int64_t rgswa_qstride,
                const uint32_t* __restrict__ RGSWb, ExtArgs e, NttCtx c) {
  extern __shared__ uint32_t smem[];
  const int d = 1 << c.logd;
  const int pi = blockIdx.x;
  const int shard = blockIdx.y;
  const int q = blockIdx.z;
  const int l = gridDim.y;
  const uint32_t p = c.p[pi];
  const uint32_t pinv = c.pinv[pi];
  T* sa = reinterpret_cast<T*>(smem + d);
  T* sb = sa + d;

  const T* ca = coeff_a + q * coeff_a_q_stride + shard * coeff_a_shard_stride;
  const T* cb = coeff_b + q * coeff_b_q_stride + shard * coeff_b_shard_stride;
  const int64_t rbase = (static_cast<int64_t>(q) * l + shard) * c.r * 2 * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    T ra, rb;
    horner_state<T>(first, resid_in, rbase, d, j, ca, cb, c, ra, rb);
    sa[j] = low_bits<T>(ra, e.log_q);
    sb[j] = low_bits<T>(rb, e.log_q);
  }
  constexpr int kPer = PolyShape<ITERS>::kPer;
  uint32_t acc_a[kPer], acc_b[kPer];
#pragma unroll
  for (int m = 0; m < kPer; ++m) acc_a[m] = acc_b[m] = 0;

  const int ng = 2 * e.num_digits;
  for (int g = 0; g < ng; ++g) {
    const T* src = g < e.num_digits ? sa : sb;
    const int dg = g < e.num_digits ? g : g - e.num_digits;
    if (dg >= e.live_digits) continue;
    __syncthreads();
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      const T dig = gadget_digit<T>(src[j], e.log_q, e.log_digit, e.num_digits, dg);
      smem[j] = to_residue<T>(dig & static_cast<T>(e.umask), p);
    }
    ntt_forward_t<ITERS>(smem, c, pi);
    const uint32_t* wa =
        RGSWa + q * rgswa_qstride + (static_cast<int64_t>(g) * c.r + pi) * d;
    const uint32_t* wb =
        RGSWb + ((static_cast<int64_t>(q) * ng + g) * c.r + pi) * d;
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
      const int j = threadIdx.x + m * blockDim.x;
      if (j < d) {
        const uint32_t x = smem[j];
        acc_a[m] = add_mod(acc_a[m], mont_mul(x, __ldg(wa + j), p, pinv), p);
        acc_b[m] = add_mod(acc_b[m], mont_mul(x, __ldg(wb + j), p, pinv), p);
      }
    }
  }
  uint32_t* out = resid_out + rbase + static_cast<int64_t>(pi) * 2 * d;
  for (int half = 0; half < 2; ++half) {
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
      const int j = threadIdx.x + m * blockDim.x;
      if (j < d) smem[j] = half == 0 ? acc_a[m] : acc_b[m];
    }
    ntt_inverse_t<ITERS>(smem, c, pi);
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      out[half * d + j] = shoup_mul(smem[j], c.scale[pi], c.scale_s[pi], p);
    }
  }
}

// The external product of ext_step_kernel for d = 2^LOGD, one block per
// (shard, request) over all primes: the Horner state is reconstructed once
// (not once per prime), every NTT runs in registers with the radix-16
// passes of ntt16.cuh, the RGSW products are taken in the layout the forward
// transform leaves (16 consecutive slots per thread, 16-byte loads) and the
// inverse starts from the accumulators without a trip through shared
// memory. Same residues as ext_step_kernel. grid = (l, batch), d / 16 threads,
// needs c.tables16.
template <typename T, int LOGD>
__global__ void __launch_bounds__(Ntt16<LOGD>::kThreads, 512 / Ntt16<LOGD>::kThreads)
ext_step16_kernel(bool first, const uint32_t* __restrict__ resid_in,
                  uint32_t* __restrict__ resid_out,
                  const T* __restrict__ coeff_a, int64_t coeff_a_q_stride,
                  int64_t coeff_a_shard_stride,
                  const T* __restrict__ coeff_b, int64_t coeff_b_q_stride,
                  int64_t coeff_b_shard_stride,
                  const uint32_t* __restrict__ RGSWa, int64_t rgswa_qstride,
                  const uint32_t* __restrict__ RGSWb, ExtArgs e, NttCtx c) {
  extern __shared__ uint32_t smem[];
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  uint32_t* xs = smem;                           // exchange buffer
  T* sa = reinterpret_cast<T*>(smem + d);        // LowBits of the state
  T* sb = sa + d;
  const int tid = threadIdx.x;
  const int shard = blockIdx.x;
  const int q = blockIdx.y;
  const int l = gridDim.x;
  const T* ca = coeff_a + q * coeff_a_q_stride + shard * coeff_a_shard_stride;
  const T* cb = coeff_b + q * coeff_b_q_stride + shard * coeff_b_shard_stride;
  const int64_t rbase = (static_cast<int64_t>(q) * l + shard) * c.r * 2 * d;
  for (int j = tid; j < d; j += NT) {
    T ra, rb;
    horner_state<T>(first, resid_in, rbase, d, j, ca, cb, c, ra, rb);
    sa[j] = low_bits<T>(ra, e.log_q);
    sb[j] = low_bits<T>(rb, e.log_q);
  }
  // Each thread reads back only the words it wrote: no barrier needed.
  const int ng = 2 * e.num_digits;
  for (int pi = 0; pi < c.r; ++pi) {
    const uint32_t p = c.p[pi];
    const uint32_t pinv = c.pinv[pi];
    const uint32_t* tab16 = c.tables16 + static_cast<size_t>(pi) * 4 * d;
    uint32_t acc_a[16], acc_b[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc_a[k] = acc_b[k] = 0;
    for (int g = 0; g < ng; ++g) {
      const T* src = g < e.num_digits ? sa : sb;
      const int dg = g < e.num_digits ? g : g - e.num_digits;
      if (dg >= e.live_digits) continue;
      uint32_t x[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const T dig = gadget_digit<T>(src[tid + NT * k], e.log_q, e.log_digit,
                                      e.num_digits, dg);
        x[k] = to_residue<T>(dig & static_cast<T>(e.umask), p);
      }
      ntt16_forward<LOGD, false, LOGD != 12, true>(x, xs, tab16, p, tid);
      const uint4* wa = reinterpret_cast<const uint4*>(
          RGSWa + q * rgswa_qstride + (static_cast<int64_t>(g) * c.r + pi) * d + 16 * tid);
      const uint4* wb = reinterpret_cast<const uint4*>(
          RGSWb + ((static_cast<int64_t>(q) * ng + g) * c.r + pi) * d + 16 * tid);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const uint4 va = __ldg(wa + v), vb = __ldg(wb + v);
        const uint32_t ra[4] = {va.x, va.y, va.z, va.w};
        const uint32_t rb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int k = 4 * v + i;
          acc_a[k] = add_mod(acc_a[k], mont_mul(x[k], ra[i], p, pinv), p);
          acc_b[k] = add_mod(acc_b[k], mont_mul(x[k], rb[i], p, pinv), p);
        }
      }
    }
    uint32_t* out = resid_out + rbase + static_cast<int64_t>(pi) * 2 * d;
    ntt16_inverse<LOGD, false, LOGD != 12>(acc_a, xs, tab16, p, tid);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      out[tid + NT * k] = shoup_mul(acc_a[k], c.scale[pi], c.scale_s[pi], p);
    }
    ntt16_inverse<LOGD, false, LOGD != 12>(acc_b, xs, tab16, p, tid);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      out[d + tid + NT * k] = shoup_mul(acc_b[k], c.scale[pi], c.scale_s[pi], p);
    }
  }
}

// The external product for d = 2^LOGD when a launch has fewer requests
// than SMs: one block per (prime, shard, request) as ext_step_kernel, NGR
// groups of d / 16 threads that run the radix-16 transforms side by side
// (NGR = 2, or 4 at d = 2048 for the fewest blocks). The live digits of a
// and b are dealt to the groups in turn; each group keeps its partial
// products for both outputs, the partials meet in shared memory, group 0
// sums and inverts a' and group 1 b'. Each block runs once per SM, so the
// compact transforms (one pass body for all passes) keep the code small.
// Same residues as ext_step_kernel. grid = (r, l, batch), shared memory
// 2 NGR d words + 2 d CoeffType words, needs c.tables16.
template <typename T, int LOGD, int NGR>
__global__ void __launch_bounds__(NGR * Ntt16<LOGD>::kThreads, 1)
ext_step16_pair_kernel(bool first, const uint32_t* __restrict__ resid_in,
                       uint32_t* __restrict__ resid_out,
                       const T* __restrict__ coeff_a, int64_t coeff_a_q_stride,
                       int64_t coeff_a_shard_stride,
                       const T* __restrict__ coeff_b, int64_t coeff_b_q_stride,
                       int64_t coeff_b_shard_stride,
                       const uint32_t* __restrict__ RGSWa, int64_t rgswa_qstride,
                       const uint32_t* __restrict__ RGSWb, ExtArgs e, NttCtx c) {
  extern __shared__ uint32_t smem[];
  constexpr int d = Ntt16<LOGD>::kD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  const int tid = threadIdx.x;
  const int grp = tid / NT;
  const int lt = tid & (NT - 1);
  const int bar = 1 + grp;
  // Per group: [partial a' | partial b'], the first half doubling as the
  // group's exchange buffer while it transforms.
  uint32_t* region = smem + grp * 2 * d;
  T* st = reinterpret_cast<T*>(smem + NGR * 2 * d);  // LowBits of a, then of b
  const int pi = blockIdx.x;
  const uint32_t* tab16 = c.tables16 + static_cast<size_t>(pi) * 4 * d;
  const int shard = blockIdx.y;
  const int q = blockIdx.z;
  const int l = gridDim.y;
  const T* ca = coeff_a + q * coeff_a_q_stride + shard * coeff_a_shard_stride;
  const T* cb = coeff_b + q * coeff_b_q_stride + shard * coeff_b_shard_stride;
  const int64_t rbase = (static_cast<int64_t>(q) * l + shard) * c.r * 2 * d;
#pragma unroll 2
  for (int j = tid; j < d; j += NGR * NT) {
    T ra, rb;
    horner_state<T>(first, resid_in, rbase, d, j, ca, cb, c, ra, rb);
    st[j] = low_bits<T>(ra, e.log_q);
    st[d + j] = low_bits<T>(rb, e.log_q);
  }
  __syncthreads();
  const uint32_t p = c.p[pi];
  const uint32_t pinv = c.pinv[pi];
  const int ng = 2 * e.num_digits;
  const int n_live = 2 * e.live_digits;  // transforms: digits of a, then of b
  uint32_t acc_a[16], acc_b[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) acc_a[k] = acc_b[k] = 0;
  for (int ti = grp; ti < n_live; ti += NGR) {
    const int poly = ti < e.live_digits ? 0 : 1;
    const int dg = ti - poly * e.live_digits;
    const int g = poly * e.num_digits + dg;
    const T* src = st + poly * d;
    uint32_t x[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const T dig = gadget_digit<T>(src[lt + NT * k], e.log_q, e.log_digit,
                                    e.num_digits, dg);
      x[k] = to_residue<T>(dig & static_cast<T>(e.umask), p);
    }
    ntt16_forward<LOGD, false, true, true>(x, region, tab16, p, lt, bar);
    const uint4* wa = reinterpret_cast<const uint4*>(
        RGSWa + q * rgswa_qstride + (static_cast<int64_t>(g) * c.r + pi) * d + 16 * lt);
    const uint4* wb = reinterpret_cast<const uint4*>(
        RGSWb + ((static_cast<int64_t>(q) * ng + g) * c.r + pi) * d + 16 * lt);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const uint4 va = __ldg(wa + v), vb = __ldg(wb + v);
      const uint32_t ra[4] = {va.x, va.y, va.z, va.w};
      const uint32_t rb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k = 4 * v + i;
        acc_a[k] = add_mod(acc_a[k], mont_mul(x[k], ra[i], p, pinv), p);
        acc_b[k] = add_mod(acc_b[k], mont_mul(x[k], rb[i], p, pinv), p);
      }
    }
  }
  // The partials meet: every group leaves both in its region (its exchange
  // buffer is free since its last transform); group 0 sums a', group 1 b'.
  ntt16_store_slots<LOGD>(acc_a, region, lt);
  ntt16_store_slots<LOGD>(acc_b, region + d, lt);
  __syncthreads();
  uint32_t sum[16];
  if (grp < 2) {
#pragma unroll
    for (int k = 0; k < 16; ++k) sum[k] = 0;
    for (int o = 0; o < NGR; ++o) {
      uint32_t part[16];
      ntt16_load_slots<LOGD>(part, smem + o * 2 * d + grp * d, lt);
#pragma unroll
      for (int k = 0; k < 16; ++k) sum[k] = add_mod(sum[k], part[k], p);
    }
  }
  __syncthreads();
  if (grp < 2) {
    ntt16_inverse<LOGD, false, true>(sum, region, tab16, p, lt, bar);
    uint32_t* out = resid_out + rbase + static_cast<int64_t>(pi) * 2 * d + grp * d;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      out[lt + NT * k] = shoup_mul(sum[k], c.scale[pi], c.scale_s[pi], p);
    }
  }
}

// Final Horner addition (or the single packed ciphertext when t == 1) and
// the modulus switch of a to q1 and b to q2. grid = (l, batch).
// With rescale == false it only reconstructs (component entry point).
template <typename T>
__global__ void __launch_bounds__(kPolyThreads)
finish_kernel(bool from_resid, const uint32_t* __restrict__ resid,
              const T* __restrict__ coeff_a, int64_t coeff_a_shard_stride,
              const T* __restrict__ coeff_b, int64_t coeff_b_q_stride,
              int64_t coeff_b_shard_stride, bool rescale, int log_q, int log_q1,
              int log_q2, T* __restrict__ out, NttCtx c) {
  const int d = 1 << c.logd;
  const int shard = blockIdx.x;
  const int q = blockIdx.y;
  const int l = gridDim.x;
  const T* ca = coeff_a == nullptr ? nullptr : coeff_a + shard * coeff_a_shard_stride;
  const T* cb = coeff_b == nullptr
                    ? nullptr
                    : coeff_b + q * coeff_b_q_stride + shard * coeff_b_shard_stride;
  const int64_t rbase = (static_cast<int64_t>(q) * l + shard) * c.r * 2 * d;
  T* oa = out + (static_cast<int64_t>(q) * l + shard) * 2 * d;
  T* ob = oa + d;
#pragma unroll 4
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    T ra, rb;
    horner_state<T>(!from_resid, resid, rbase, d, j, ca, cb, c, ra, rb);
    if (rescale) {
      ra = rescale_word<T>(ra, log_q, log_q1);
      rb = rescale_word<T>(rb, log_q, log_q2);
    }
    oa[j] = ra;
    ob[j] = rb;
  }
}

}  // namespace inspire
