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
  // The same tables permuted for the radix-16 transform of ntt16.cuh
  // ([prime][4][d]); null unless d = 4096.
  const uint32_t* tables16;
};

#ifdef __CUDACC__
// Forward transform. Two Cooley-Tukey stages at a time: the quad
// (x0, x1, x2, x3) = a[j], a[j+t/2], a[j+t], a[j+3t/2] takes stage (m, t)
// with twiddle W[m+i] on (x0,x2),(x1,x3), then stage (2m, t/2) with W[2m+2i]
// on (x0,x1) and W[2m+2i+1] on (x2,x3). An odd last stage runs radix-2.
__device__ __forceinline__ void ntt_forward(uint32_t* a, const NttCtx& c,
                                            int pi) {
  const int d = 1 << c.logd;
  const uint32_t p = c.p[pi];
  const uint32_t* tw = c.tables + static_cast<size_t>(pi) * 4 * d;
  const uint32_t* tws = tw + d;
  __syncthreads();
  int lt = c.logd - 1;  // log2 of the current half-size t
  int m = 1;
  for (; lt >= 1; lt -= 2, m <<= 2) {
    const int t = 1 << lt;
    const int lh = lt - 1;  // log2(t/2)
    for (int b = threadIdx.x; b < d / 4; b += blockDim.x) {
      const int i = b >> lh;
      const int j = (i << (lt + 1)) | (b & ((t >> 1) - 1));
      const uint32_t w1 = __ldg(tw + m + i), w1s = __ldg(tws + m + i);
      const uint32_t w2 = __ldg(tw + 2 * m + 2 * i), w2s = __ldg(tws + 2 * m + 2 * i);
      const uint32_t w3 = __ldg(tw + 2 * m + 2 * i + 1),
                     w3s = __ldg(tws + 2 * m + 2 * i + 1);
      uint32_t x0 = a[j], x1 = a[j + (t >> 1)], x2 = a[j + t],
               x3 = a[j + t + (t >> 1)];
      uint32_t v = shoup_mul(x2, w1, w1s, p);
      x2 = sub_mod(x0, v, p);
      x0 = add_mod(x0, v, p);
      v = shoup_mul(x3, w1, w1s, p);
      x3 = sub_mod(x1, v, p);
      x1 = add_mod(x1, v, p);
      v = shoup_mul(x1, w2, w2s, p);
      a[j + (t >> 1)] = sub_mod(x0, v, p);
      a[j] = add_mod(x0, v, p);
      v = shoup_mul(x3, w3, w3s, p);
      a[j + t + (t >> 1)] = sub_mod(x2, v, p);
      a[j + t] = add_mod(x2, v, p);
    }
    __syncthreads();
  }
  if (lt == 0) {  // one radix-2 stage left (t = 1)
    for (int b = threadIdx.x; b < d / 2; b += blockDim.x) {
      const int j = b << 1;
      const uint32_t u = a[j];
      const uint32_t v = shoup_mul(a[j + 1], __ldg(tw + m + b), __ldg(tws + m + b), p);
      a[j] = add_mod(u, v, p);
      a[j + 1] = sub_mod(u, v, p);
    }
    __syncthreads();
  }
}

// Inverse transform without the final 1/d scaling (folded into `scale`).
// Two Gentleman-Sande stages at a time: stage (h, t) on (x0,x1),(x2,x3) with
// IW[h+2i], IW[h+2i+1], then stage (h/2, 2t) on (x0,x2),(x1,x3) with
// IW[h/2+i], for the quad a[j], a[j+t], a[j+2t], a[j+3t].
__device__ __forceinline__ void ntt_inverse(uint32_t* a, const NttCtx& c,
                                            int pi) {
  const int d = 1 << c.logd;
  const uint32_t p = c.p[pi];
  const uint32_t* itw = c.tables + static_cast<size_t>(pi) * 4 * d + 2 * d;
  const uint32_t* itws = itw + d;
  __syncthreads();
  int lt = 0;
  int h = d >> 1;
  for (; lt + 1 < c.logd; lt += 2, h >>= 2) {
    const int t = 1 << lt;
    for (int b = threadIdx.x; b < d / 4; b += blockDim.x) {
      const int i = b >> lt;                    // block of size 4t
      const int j = (i << (lt + 2)) | (b & (t - 1));
      const uint32_t wa = __ldg(itw + h + 2 * i), was = __ldg(itws + h + 2 * i);
      const uint32_t wb = __ldg(itw + h + 2 * i + 1),
                     wbs = __ldg(itws + h + 2 * i + 1);
      const uint32_t wc = __ldg(itw + (h >> 1) + i), wcs = __ldg(itws + (h >> 1) + i);
      const uint32_t x0 = a[j], x1 = a[j + t], x2 = a[j + 2 * t], x3 = a[j + 3 * t];
      const uint32_t y0 = add_mod(x0, x1, p);
      const uint32_t y1 = shoup_mul(sub_mod(x0, x1, p), wa, was, p);
      const uint32_t y2 = add_mod(x2, x3, p);
      const uint32_t y3 = shoup_mul(sub_mod(x2, x3, p), wb, wbs, p);
      a[j] = add_mod(y0, y2, p);
      a[j + 2 * t] = shoup_mul(sub_mod(y0, y2, p), wc, wcs, p);
      a[j + t] = add_mod(y1, y3, p);
      a[j + 3 * t] = shoup_mul(sub_mod(y1, y3, p), wc, wcs, p);
    }
    __syncthreads();
  }
  if (lt < c.logd) {  // one radix-2 stage left (h = 1, t = d/2)
    const int t = 1 << lt;
    for (int b = threadIdx.x; b < d / 2; b += blockDim.x) {
      const uint32_t u = a[b];
      const uint32_t v = a[b + t];
      a[b] = add_mod(u, v, p);
      a[b + t] = shoup_mul(sub_mod(u, v, p), __ldg(itw + 1), __ldg(itws + 1), p);
    }
    __syncthreads();
  }
}

// The same transforms with ITERS quads per thread per double stage known at
// compile time (blockDim.x * 4 * ITERS == d): every quad's operands and
// twiddles are loaded before any butterfly, so the loads of a stage overlap
// instead of one quad's latency following another's. ITERS == 0 falls back
// to the loops above (any d and block size).
template <int ITERS>
__device__ __forceinline__ void ntt_forward_t(uint32_t* a, const NttCtx& c,
                                              int pi) {
  if constexpr (ITERS == 0) {
    ntt_forward(a, c, pi);
  } else {
    const uint32_t p = c.p[pi];
    const int d = 1 << c.logd;
    const uint32_t* tw = c.tables + static_cast<size_t>(pi) * 4 * d;
    const uint32_t* tws = tw + d;
    __syncthreads();
    int lt = c.logd - 1;
    int m = 1;
    for (; lt >= 1; lt -= 2, m <<= 2) {
      const int t = 1 << lt;
      const int lh = lt - 1;
      uint32_t x[ITERS][4], w[ITERS][6];
      int jj[ITERS];
#pragma unroll
      for (int it = 0; it < ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        const int i = b >> lh;
        const int j = (i << (lt + 1)) | (b & ((t >> 1) - 1));
        jj[it] = j;
        w[it][0] = __ldg(tw + m + i);
        w[it][1] = __ldg(tws + m + i);
        w[it][2] = __ldg(tw + 2 * m + 2 * i);
        w[it][3] = __ldg(tws + 2 * m + 2 * i);
        w[it][4] = __ldg(tw + 2 * m + 2 * i + 1);
        w[it][5] = __ldg(tws + 2 * m + 2 * i + 1);
        x[it][0] = a[j];
        x[it][1] = a[j + (t >> 1)];
        x[it][2] = a[j + t];
        x[it][3] = a[j + t + (t >> 1)];
      }
#pragma unroll
      for (int it = 0; it < ITERS; ++it) {
        uint32_t x0 = x[it][0], x1 = x[it][1], x2 = x[it][2], x3 = x[it][3];
        uint32_t v = shoup_mul(x2, w[it][0], w[it][1], p);
        x2 = sub_mod(x0, v, p);
        x0 = add_mod(x0, v, p);
        v = shoup_mul(x3, w[it][0], w[it][1], p);
        x3 = sub_mod(x1, v, p);
        x1 = add_mod(x1, v, p);
        const int j = jj[it];
        v = shoup_mul(x1, w[it][2], w[it][3], p);
        a[j + (t >> 1)] = sub_mod(x0, v, p);
        a[j] = add_mod(x0, v, p);
        v = shoup_mul(x3, w[it][4], w[it][5], p);
        a[j + t + (t >> 1)] = sub_mod(x2, v, p);
        a[j + t] = add_mod(x2, v, p);
      }
      __syncthreads();
    }
    if (lt == 0) {  // one radix-2 stage left (t = 1)
      uint32_t u[2 * ITERS], v[2 * ITERS], w[2 * ITERS], ws[2 * ITERS];
#pragma unroll
      for (int it = 0; it < 2 * ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        u[it] = a[2 * b];
        v[it] = a[2 * b + 1];
        w[it] = __ldg(tw + m + b);
        ws[it] = __ldg(tws + m + b);
      }
#pragma unroll
      for (int it = 0; it < 2 * ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        const uint32_t y = shoup_mul(v[it], w[it], ws[it], p);
        a[2 * b] = add_mod(u[it], y, p);
        a[2 * b + 1] = sub_mod(u[it], y, p);
      }
      __syncthreads();
    }
  }
}

template <int ITERS>
__device__ __forceinline__ void ntt_inverse_t(uint32_t* a, const NttCtx& c,
                                              int pi) {
  if constexpr (ITERS == 0) {
    ntt_inverse(a, c, pi);
  } else {
    const uint32_t p = c.p[pi];
    const int d = 1 << c.logd;
    const uint32_t* itw = c.tables + static_cast<size_t>(pi) * 4 * d + 2 * d;
    const uint32_t* itws = itw + d;
    __syncthreads();
    int lt = 0;
    int h = d >> 1;
    for (; lt + 1 < c.logd; lt += 2, h >>= 2) {
      const int t = 1 << lt;
      uint32_t x[ITERS][4], w[ITERS][6];
      int jj[ITERS];
#pragma unroll
      for (int it = 0; it < ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        const int i = b >> lt;
        const int j = (i << (lt + 2)) | (b & (t - 1));
        jj[it] = j;
        w[it][0] = __ldg(itw + h + 2 * i);
        w[it][1] = __ldg(itws + h + 2 * i);
        w[it][2] = __ldg(itw + h + 2 * i + 1);
        w[it][3] = __ldg(itws + h + 2 * i + 1);
        w[it][4] = __ldg(itw + (h >> 1) + i);
        w[it][5] = __ldg(itws + (h >> 1) + i);
        x[it][0] = a[j];
        x[it][1] = a[j + t];
        x[it][2] = a[j + 2 * t];
        x[it][3] = a[j + 3 * t];
      }
#pragma unroll
      for (int it = 0; it < ITERS; ++it) {
        const uint32_t y0 = add_mod(x[it][0], x[it][1], p);
        const uint32_t y1 =
            shoup_mul(sub_mod(x[it][0], x[it][1], p), w[it][0], w[it][1], p);
        const uint32_t y2 = add_mod(x[it][2], x[it][3], p);
        const uint32_t y3 =
            shoup_mul(sub_mod(x[it][2], x[it][3], p), w[it][2], w[it][3], p);
        const int j = jj[it];
        a[j] = add_mod(y0, y2, p);
        a[j + 2 * t] = shoup_mul(sub_mod(y0, y2, p), w[it][4], w[it][5], p);
        a[j + t] = add_mod(y1, y3, p);
        a[j + 3 * t] = shoup_mul(sub_mod(y1, y3, p), w[it][4], w[it][5], p);
      }
      __syncthreads();
    }
    if (lt < c.logd) {  // one radix-2 stage left (h = 1, t = d/2)
      const int t = 1 << lt;
      const uint32_t w = __ldg(itw + 1), ws = __ldg(itws + 1);
      uint32_t u[2 * ITERS], v[2 * ITERS];
#pragma unroll
      for (int it = 0; it < 2 * ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        u[it] = a[b];
        v[it] = a[b + t];
      }
#pragma unroll
      for (int it = 0; it < 2 * ITERS; ++it) {
        const int b = threadIdx.x + it * blockDim.x;
        a[b] = add_mod(u[it], v[it], p);
        a[b + t] = shoup_mul(sub_mod(u[it], v[it], p), w, ws, p);
      }
      __syncthreads();
    }
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
