// Block-level negacyclic NTT over one 31-bit prime and the Garner CRT that
// turns r residues back into an integer mod 2^w.
//
// Forward: Cooley-Tukey with the psi-twisted twiddles merged in (natural
// order in, bit-reversed order out); inverse: Gentleman-Sande (bit-reversed
// in, natural out). Pointwise products in between therefore never need a
// permutation. One polynomial of length d lives in shared memory and every
// thread of the block takes d/2/blockDim butterflies per stage.
#pragma once
#include <cstdint>

#include "arith.cuh"

namespace inspire {

struct NttCtx {
  int logd;
  int r;  // primes in use
  uint32_t p[kMaxPrimes];
  uint32_t pinv[kMaxPrimes];
  uint32_t half[kMaxPrimes];
  uint32_t scale[kMaxPrimes];    // d^-1 * 2^32 mod p: undoes INTT growth and
  uint32_t scale_s[kMaxPrimes];  // the 2^-32 of the Montgomery pointwise step
  uint32_t garner[kMaxPrimes][kMaxPrimes];  // [j][i] = p_j^-1 * 2^32 mod p_i
  uint64_t pm[kMaxPrimes];                  // prod_{j<i} p_j mod 2^64
  const uint32_t* tables;  // [prime][4][d]: psi_rev, shoup, ipsi_rev, shoup
};

#ifdef __CUDACC__
__device__ __forceinline__ void ntt_forward(uint32_t* a, const NttCtx& c,
                                            int pi) {
  const int d = 1 << c.logd;
  const uint32_t p = c.p[pi];
  const uint32_t* tw = c.tables + static_cast<size_t>(pi) * 4 * d;
  const uint32_t* tws = tw + d;
  __syncthreads();
  for (int lt = c.logd - 1, m = 1; lt >= 0; --lt, m <<= 1) {
    const int t = 1 << lt;
    for (int b = threadIdx.x; b < d / 2; b += blockDim.x) {
      const int i = b >> lt;
      const int j = (i << (lt + 1)) | (b & (t - 1));
      const uint32_t u = a[j];
      const uint32_t v = shoup_mul(a[j + t], __ldg(tw + m + i),
                                   __ldg(tws + m + i), p);
      a[j] = add_mod(u, v, p);
      a[j + t] = sub_mod(u, v, p);
    }
    __syncthreads();
  }
}

// Inverse transform without the final 1/d scaling (folded into `scale`).
__device__ __forceinline__ void ntt_inverse(uint32_t* a, const NttCtx& c,
                                            int pi) {
  const int d = 1 << c.logd;
  const uint32_t p = c.p[pi];
  const uint32_t* itw = c.tables + static_cast<size_t>(pi) * 4 * d + 2 * d;
  const uint32_t* itws = itw + d;
  __syncthreads();
  for (int lt = 0, h = d >> 1; h >= 1; ++lt, h >>= 1) {
    const int t = 1 << lt;
    for (int b = threadIdx.x; b < d / 2; b += blockDim.x) {
      const int i = b >> lt;
      const int j = (i << (lt + 1)) | (b & (t - 1));
      const uint32_t u = a[j];
      const uint32_t v = a[j + t];
      a[j] = add_mod(u, v, p);
      a[j + t] = shoup_mul(sub_mod(u, v, p), __ldg(itw + h + i),
                           __ldg(itws + h + i), p);
    }
    __syncthreads();
  }
}

// Garner reconstruction: x[i] < p_i -> the integer in
// [-(p_{r-1}-1)/2 * P', (p_{r-1}+1)/2 * P') (P' = product of the other
// primes) congruent to x, reduced mod 2^w.
template <typename T>
__device__ __forceinline__ T crt_reconstruct(const uint32_t (&x)[kMaxPrimes],
                                             const NttCtx& c) {
  uint32_t a[kMaxPrimes];
  a[0] = x[0];
#pragma unroll
  for (int i = 1; i < kMaxPrimes; ++i) {
    if (i < c.r) {
      const uint32_t p = c.p[i];
      uint32_t v = x[i];
#pragma unroll
      for (int j = 0; j < kMaxPrimes; ++j) {
        if (j < i) {
          const uint32_t aj = a[j] >= p ? a[j] - p : a[j];
          v = sub_mod(v, aj, p);
          v = mont_mul(v, c.garner[j][i], p, c.pinv[i]);
        }
      }
      a[i] = v;
    }
  }
  T acc = 0;
#pragma unroll
  for (int i = 0; i < kMaxPrimes; ++i) {
    if (i < c.r - 1) {
      acc += static_cast<T>(a[i]) * static_cast<T>(c.pm[i]);
    } else if (i == c.r - 1) {
      const uint32_t top = a[i];
      if (top > c.half[i]) {
        acc -= static_cast<T>(c.p[i] - top) * static_cast<T>(c.pm[i]);
      } else {
        acc += static_cast<T>(top) * static_cast<T>(c.pm[i]);
      }
    }
  }
  return acc;
}
#endif

}  // namespace inspire
