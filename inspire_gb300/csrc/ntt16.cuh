// Register-resident negacyclic NTT for d = 4096 with 256 threads: three
// radix-16 passes of four stages each, 16 coefficients per thread, two
// exchanges through shared memory in between.
//
// The transform is the one of ntt.cuh (Cooley-Tukey forward with the
// psi-twisted twiddles, natural order in and bit-reversed order out;
// Gentleman-Sande inverse), so both give the same residues. Only the
// grouping of the stages differs. Stage (m groups, distance t = d / 2m) takes
// the pair (e, e + t) of group i = e / 2t with twiddle W[m + i]. Pass P
// (P = 0, 1, 2) runs the stages m = 16^P * 2^s (s = 0..3) on the 16
// coefficients e_k = 2 g t0 + o + k t0 / 8 of one thread, t0 = d / (2 * 16^P),
// g = the thread's group, o = its offset:
//   P = 0: e_k = tid + 256 k         (g = 0,        o = tid)
//   P = 1: e_k = 256 g + o + 16 k    (g = tid / 16, o = tid % 16)
//   P = 2: e_k = 16 tid + k          (g = tid,      o = 0)
// Within a pass, stage s pairs k with k + 8 / 2^s and takes the twiddle
// W[16^P 2^s + g 2^s + (k >> (4 - s))].
//
// Twiddles are read from a permuted copy of the tables (built on the host):
// pass P, stage s, sub-block x, group g at 16^P - 1 + 16^P (2^s - 1) + x 16^P
// + g, so the 32 threads of a warp read consecutive words (pass 2), two
// words (pass 1) or one word (pass 0).
//
// Shared memory holds coefficient e at e ^ swz(e >> 5), swz(r) = (r & 15) |
// ((r >> 3) & 1) << 4, which keeps all three access patterns free of bank
// conflicts (pass 0 reads whole rows; pass 1 two half rows 8 rows apart;
// pass 2 two coefficients of each of 16 consecutive rows).
#pragma once
#include <cstdint>

#include "arith.cuh"

namespace inspire {

constexpr int kNtt16LogD = 12;
constexpr int kNtt16D = 1 << kNtt16LogD;
constexpr int kNtt16Threads = 256;

// Position of twiddle W[m + g] (stage with m = 16^P 2^s groups) in the
// permuted table. Host and device.
__host__ __device__ __forceinline__ int ntt16_twiddle_slot(int pass, int s, int x,
                                                           int g) {
  const int m0 = 1 << (4 * pass);
  return m0 - 1 + m0 * ((1 << s) - 1) + x * m0 + g;
}

#ifdef __CUDACC__
__device__ __forceinline__ int ntt16_pos(int e) {
  const int r = e >> 5;
  return e ^ ((r & 15) | (((r >> 3) & 1) << 4));
}

__device__ __forceinline__ int ntt16_elem(int pass, int tid, int k) {
  return pass == 0 ? tid + 256 * k
                   : (pass == 1 ? 256 * (tid >> 4) + (tid & 15) + 16 * k : 16 * tid + k);
}

// Barrier of the 256 threads running one transform: the whole block
// (bar == 0) or named barrier `bar` when several groups of 256 threads run
// transforms of their own.
__device__ __forceinline__ void ntt16_sync(int bar) {
  if (bar == 0) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(kNtt16Threads) : "memory");
  }
}

__device__ __forceinline__ int ntt16_group(int pass, int tid) {
  return pass == 0 ? 0 : (pass == 1 ? tid >> 4 : tid);
}

// A twiddle word: read-only global memory (kSmem = false) or a copy of the
// tables in shared memory.
template <bool kSmem>
__device__ __forceinline__ uint32_t ntt16_tw(const uint32_t* t, int i) {
  if constexpr (kSmem) {
    return t[i];
  } else {
    return __ldg(t + i);
  }
}

// Four forward stages of pass P on the thread's 16 coefficients.
// tw = permuted W, tws = its Shoup constants.
template <int P, bool kSmem = false>
__device__ __forceinline__ void ntt16_fwd_pass(uint32_t (&x)[16],
                                               const uint32_t* __restrict__ tw,
                                               const uint32_t* __restrict__ tws,
                                               uint32_t p, int tid) {
  const int g = ntt16_group(P, tid);
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int half = 8 >> s;
    uint32_t w[8], ws[8];
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
      const int slot = ntt16_twiddle_slot(P, s, b, g);
      w[b] = ntt16_tw<kSmem>(tw, slot);
      ws[b] = ntt16_tw<kSmem>(tws, slot);
    }
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const int k = b * 2 * half + i;
        const uint32_t v = shoup_mul(x[k + half], w[b], ws[b], p);
        x[k + half] = sub_mod(x[k], v, p);
        x[k] = add_mod(x[k], v, p);
      }
    }
  }
}

// Four inverse stages of pass P (stage s = 3 down to 0).
template <int P, bool kSmem = false>
__device__ __forceinline__ void ntt16_inv_pass(uint32_t (&x)[16],
                                               const uint32_t* __restrict__ itw,
                                               const uint32_t* __restrict__ itws,
                                               uint32_t p, int tid) {
  const int g = ntt16_group(P, tid);
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int half = 8 >> s;
    uint32_t w[8], ws[8];
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
      const int slot = ntt16_twiddle_slot(P, s, b, g);
      w[b] = ntt16_tw<kSmem>(itw, slot);
      ws[b] = ntt16_tw<kSmem>(itws, slot);
    }
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const int k = b * 2 * half + i;
        const uint32_t u = x[k], v = x[k + half];
        x[k] = add_mod(u, v, p);
        x[k + half] = shoup_mul(sub_mod(u, v, p), w[b], ws[b], p);
      }
    }
  }
}

template <int P>
__device__ __forceinline__ void ntt16_store(const uint32_t (&x)[16], uint32_t* xs,
                                            int tid) {
#pragma unroll
  for (int k = 0; k < 16; ++k) xs[ntt16_pos(ntt16_elem(P, tid, k))] = x[k];
}

template <int P>
__device__ __forceinline__ void ntt16_load(uint32_t (&x)[16], const uint32_t* xs,
                                           int tid) {
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = xs[ntt16_pos(ntt16_elem(P, tid, k))];
}

// Forward transform. In: x[k] = coefficient tid + 256 k. Out: x[k] = NTT
// slot 16 tid + k (the bit-reversed output array of ntt_forward). `xs` is a
// 4096-word shared buffer, free again when this returns. tab16 = the
// prime's permuted tables [W | W shoup | IW | IW shoup], 4096 words each.
// tid in [0, 256) within the group that synchronises on `bar`. kSmem: the
// tables were copied to shared memory (tab16 points there).
template <bool kSmem = false>
__device__ __forceinline__ void ntt16_forward(uint32_t (&x)[16], uint32_t* xs,
                                              const uint32_t* __restrict__ tab16,
                                              uint32_t p, int tid, int bar = 0) {
  const uint32_t* tw = tab16;
  const uint32_t* tws = tab16 + kNtt16D;
  ntt16_fwd_pass<0, kSmem>(x, tw, tws, p, tid);
  ntt16_store<0>(x, xs, tid);
  ntt16_sync(bar);
  ntt16_load<1>(x, xs, tid);
  ntt16_fwd_pass<1, kSmem>(x, tw, tws, p, tid);
  ntt16_store<1>(x, xs, tid);  // the same words this thread read
  ntt16_sync(bar);
  ntt16_load<2>(x, xs, tid);
  ntt16_fwd_pass<2, kSmem>(x, tw, tws, p, tid);
  ntt16_sync(bar);
}

// Inverse transform without the 1/d scaling. In: x[k] = slot 16 tid + k.
// Out: x[k] = coefficient tid + 256 k. itw / itws: the permuted inverse
// twiddles and their Shoup constants.
template <bool kSmem = false>
__device__ __forceinline__ void ntt16_inverse_tw(uint32_t (&x)[16], uint32_t* xs,
                                                 const uint32_t* __restrict__ itw,
                                                 const uint32_t* __restrict__ itws,
                                                 uint32_t p, int tid, int bar = 0) {
  ntt16_inv_pass<2, kSmem>(x, itw, itws, p, tid);
  ntt16_store<2>(x, xs, tid);
  ntt16_sync(bar);
  ntt16_load<1>(x, xs, tid);
  ntt16_inv_pass<1, kSmem>(x, itw, itws, p, tid);
  ntt16_store<1>(x, xs, tid);
  ntt16_sync(bar);
  ntt16_load<0>(x, xs, tid);
  ntt16_inv_pass<0, kSmem>(x, itw, itws, p, tid);
  ntt16_sync(bar);
}

// Compact forms: one pass body serves all three passes, the pass index a
// run-time value (coefficients e_k = base + stride * k, twiddle slots
// 16^P - 1 + 16^P (2^s - 1 + x) + g). A third of the code of the unrolled
// transforms, for launches whose blocks each run once per SM, where the
// fetch of the unrolled code, not the arithmetic, sets the time.
__device__ __forceinline__ void ntt16_pass_geometry(int pass, int tid, int& base,
                                                    int& stride, int& g) {
  base = pass == 0 ? tid : (pass == 1 ? 256 * (tid >> 4) + (tid & 15) : 16 * tid);
  stride = pass == 0 ? 256 : (pass == 1 ? 16 : 1);
  g = pass == 0 ? 0 : (pass == 1 ? tid >> 4 : tid);
}

template <bool kSmem, bool kInverse>
__device__ __forceinline__ void ntt16_pass_rt(uint32_t (&x)[16],
                                              const uint32_t* __restrict__ tw,
                                              const uint32_t* __restrict__ tws,
                                              uint32_t p, int pass, int g) {
  const int m0 = 1 << (4 * pass);
  const int base = m0 - 1 + g;
#pragma unroll
  for (int si = 0; si < 4; ++si) {
    const int s = kInverse ? 3 - si : si;
    const int half = 8 >> s;
    uint32_t w[8], ws[8];
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
      const int slot = base + m0 * ((1 << s) - 1 + b);
      w[b] = ntt16_tw<kSmem>(tw, slot);
      ws[b] = ntt16_tw<kSmem>(tws, slot);
    }
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const int k = b * 2 * half + i;
        if (kInverse) {
          const uint32_t u = x[k], v = x[k + half];
          x[k] = add_mod(u, v, p);
          x[k + half] = shoup_mul(sub_mod(u, v, p), w[b], ws[b], p);
        } else {
          const uint32_t v = shoup_mul(x[k + half], w[b], ws[b], p);
          x[k + half] = sub_mod(x[k], v, p);
          x[k] = add_mod(x[k], v, p);
        }
      }
    }
  }
}

template <bool kSmem = false>
__device__ __forceinline__ void ntt16_forward_compact(uint32_t (&x)[16], uint32_t* xs,
                                                      const uint32_t* __restrict__ tab16,
                                                      uint32_t p, int tid, int bar = 0) {
#pragma unroll 1
  for (int pass = 0; pass < 3; ++pass) {
    int base, stride, g;
    ntt16_pass_geometry(pass, tid, base, stride, g);
    if (pass > 0) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = xs[ntt16_pos(base + stride * k)];
    }
    ntt16_pass_rt<kSmem, false>(x, tab16, tab16 + kNtt16D, p, pass, g);
    if (pass < 2) {
#pragma unroll
      for (int k = 0; k < 16; ++k) xs[ntt16_pos(base + stride * k)] = x[k];
    }
    ntt16_sync(bar);
  }
}

template <bool kSmem = false>
__device__ __forceinline__ void ntt16_inverse_compact(uint32_t (&x)[16], uint32_t* xs,
                                                      const uint32_t* __restrict__ itw,
                                                      const uint32_t* __restrict__ itws,
                                                      uint32_t p, int tid, int bar = 0) {
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    const int pass = 2 - i;
    int base, stride, g;
    ntt16_pass_geometry(pass, tid, base, stride, g);
    if (i > 0) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = xs[ntt16_pos(base + stride * k)];
    }
    ntt16_pass_rt<kSmem, true>(x, itw, itws, p, pass, g);
    if (i < 2) {
#pragma unroll
      for (int k = 0; k < 16; ++k) xs[ntt16_pos(base + stride * k)] = x[k];
    }
    ntt16_sync(bar);
  }
}

// The inverse with the prime's whole table block [W | W shoup | IW | IW shoup].
template <bool kSmem = false>
__device__ __forceinline__ void ntt16_inverse(uint32_t (&x)[16], uint32_t* xs,
                                              const uint32_t* __restrict__ tab16,
                                              uint32_t p, int tid, int bar = 0) {
  ntt16_inverse_tw<kSmem>(x, xs, tab16 + 2 * kNtt16D, tab16 + 3 * kNtt16D, p, tid, bar);
}
#endif

}  // namespace inspire
