// Register-resident negacyclic NTT for d = 2^LOGD (LOGD = 11, 12, 13) with
// d / 16 threads: passes of up to four stages on 16 coefficients per
// thread, exchanges through shared memory in between.
//
// The transform is the one of ntt.cuh (Cooley-Tukey forward with the
// psi-twisted twiddles, natural order in and bit-reversed order out;
// Gentleman-Sande inverse), so both give the same residues. Only the
// grouping of the stages differs. Stage j (m = 2^j groups, distance
// t = d / 2m) takes the pair (e, e + t) of group i = e / 2t with twiddle
// W[m + i]. A pass is a window of four stages sp .. sp + 3, of which the
// first `skip` are left out: (0, 0), (4, 0), (8, 0), ... and, when LOGD is
// not a multiple of 4, a last window (LOGD - 4, 4 - LOGD % 4). With
// m0 = 2^sp and t0 = d / (2 m0), a thread holds the 16 coefficients
// e_k = 2 g t0 + o + k t0 / 8 of group g = tid / (t0 / 8) and offset
// o = tid % (t0 / 8). The first pass reads e_k = tid + (d / 16) k (natural
// order, coalesced), the last one e_k = 16 tid + k. Stage s of a window
// pairs k with k + 8 / 2^s and takes W[m0 2^s + g 2^s + (k >> (4 - s))].
//
// Twiddles are read from a permuted copy of the tables (built on the host):
// window w, stage s, sub-block x, group g at base_w + m0 (2^s - 2^skip) +
// x m0 + g, so the threads of a warp read one word, a few words or
// consecutive words.
//
// Shared memory holds coefficient e at e ^ swz(e >> 5), with a swz per size
// that keeps every pass's access pattern free of bank conflicts (the
// patterns and the swz were checked exhaustively on the host).
#pragma once
#include <cstdint>

#include "arith.cuh"

namespace inspire {

constexpr int kNtt16MinLogD = 11;
constexpr int kNtt16MaxLogD = 13;

template <int LOGD>
struct Ntt16 {
  static_assert(LOGD >= kNtt16MinLogD && LOGD <= kNtt16MaxLogD, "ring degree");
  static constexpr int kD = 1 << LOGD;
  static constexpr int kThreads = kD / 16;
  static constexpr int kPasses = (LOGD + 3) / 4;
  __host__ __device__ static constexpr int Start(int w) {
    return (w < kPasses - 1 || LOGD % 4 == 0) ? 4 * w : LOGD - 4;
  }
  __host__ __device__ static constexpr int Skip(int w) {
    return (w == kPasses - 1 && LOGD % 4 != 0) ? 4 - LOGD % 4 : 0;
  }
  // First slot of window w: the full windows before it hold 15 m0 each.
  __host__ __device__ static constexpr int Base(int w) {
    int b = 0;
    for (int i = 0; i < w; ++i) b += 15 << (4 * i);
    return b;
  }
  // Slot of W[m0 2^s + g 2^s + x] (window w, stage s) in the permuted table.
  __host__ __device__ static constexpr int Slot(int w, int s, int x, int g) {
    return Base(w) + (1 << Start(w)) * ((1 << s) - (1 << Skip(w))) +
           x * (1 << Start(w)) + g;
  }
};

#ifdef __CUDACC__
template <int LOGD>
__device__ __forceinline__ int ntt16_pos(int e) {
  const int r = e >> 5;
  if constexpr (LOGD == 11) {
    return e ^ ((r & 7) | ((((r >> 3) ^ (r >> 2)) & 1) << 3) | (((r >> 3) & 1) << 4));
  } else if constexpr (LOGD == 12) {
    return e ^ ((r & 15) | (((r >> 3) & 1) << 4));
  } else {
    return e ^ ((r & 15) ^ ((r & 15) << 1));
  }
}

// Geometry of window w for thread tid: coefficient e_k = base + stride * k,
// group g.
template <int LOGD>
__device__ __forceinline__ void ntt16_geometry(int w, int tid, int& base, int& stride,
                                               int& g) {
  const int m0 = 1 << Ntt16<LOGD>::Start(w);
  const int t0 = Ntt16<LOGD>::kD / (2 * m0);
  stride = t0 / 8;
  g = tid / stride;
  base = 2 * g * t0 + tid % stride;
}

// Barrier of the threads running one transform: the whole block (bar == 0)
// or named barrier `bar` when several groups of threads run transforms of
// their own.
template <int LOGD>
__device__ __forceinline__ void ntt16_sync(int bar) {
  if (bar == 0) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(Ntt16<LOGD>::kThreads) : "memory");
  }
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

// The stages of window w on the thread's 16 coefficients, forward (Cooley-
// Tukey, stages skip .. 3) or inverse (Gentleman-Sande, 3 .. skip). With a
// compile-time window every index folds; the compact transforms pass a
// run-time one and the same instructions serve every window.
//
// Values stay in [0, 2p) between butterflies (2p < 2^32 for the 31-bit
// primes): each butterfly brings its two inputs to [0, p) with one unsigned
// min each, forms u + v and u - v + p in [0, 2p) without a compare, and the
// twiddle product is Shoup's without its correction (Harvey, "Faster
// arithmetic for number-theoretic transforms", 2014, with the reductions
// moved to the inputs since 4p does not fit 32 bits). ntt16_forward and
// ntt16_inverse_tw reduce to [0, p) at the end unless asked not to.
template <int LOGD, bool kSmem, bool kInverse>
__device__ __forceinline__ void ntt16_window(uint32_t (&x)[16],
                                             const uint32_t* __restrict__ tw,
                                             const uint32_t* __restrict__ tws,
                                             uint32_t p, int w, int g) {
  const int m0 = 1 << Ntt16<LOGD>::Start(w);
  const int skip = Ntt16<LOGD>::Skip(w);
  const int base = Ntt16<LOGD>::Base(w) + g - m0 * (1 << skip);
#pragma unroll
  for (int si = 0; si < 4; ++si) {
    const int s = kInverse ? 3 - si : si;
    if (s < skip) continue;
    const int half = 8 >> s;
    uint32_t wv[8], wsv[8];
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
      const int slot = base + m0 * ((1 << s) + b);
      wv[b] = ntt16_tw<kSmem>(tw, slot);
      wsv[b] = ntt16_tw<kSmem>(tws, slot);
    }
#pragma unroll
    for (int b = 0; b < (1 << s); ++b) {
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const int k = b * 2 * half + i;
        if (kInverse) {
          const uint32_t u = umin32(x[k], x[k] - p);
          const uint32_t v = umin32(x[k + half], x[k + half] - p);
          x[k] = u + v;
          x[k + half] = shoup_mul_lazy(u + p - v, wv[b], wsv[b], p);
        } else {
          const uint32_t u = umin32(x[k], x[k] - p);
          uint32_t v = shoup_mul_lazy(x[k + half], wv[b], wsv[b], p);
          v = umin32(v, v - p);
          x[k] = u + v;
          x[k + half] = u + p - v;
        }
      }
    }
  }
}

template <int LOGD>
__device__ __forceinline__ void ntt16_store(const uint32_t (&x)[16], uint32_t* xs, int w,
                                            int tid) {
  int base, stride, g;
  ntt16_geometry<LOGD>(w, tid, base, stride, g);
#pragma unroll
  for (int k = 0; k < 16; ++k) xs[ntt16_pos<LOGD>(base + stride * k)] = x[k];
}

template <int LOGD>
__device__ __forceinline__ void ntt16_load(uint32_t (&x)[16], const uint32_t* xs, int w,
                                           int tid) {
  int base, stride, g;
  ntt16_geometry<LOGD>(w, tid, base, stride, g);
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = xs[ntt16_pos<LOGD>(base + stride * k)];
}

// Forward transform. In: x[k] = coefficient tid + (d / 16) k, any value
// below 2p. Out: x[k] = NTT slot 16 tid + k in [0, p) (the bit-reversed
// output array of ntt_forward). `xs`
// is a d-word shared buffer, free again when this returns. tab16 = the
// prime's permuted tables [W | W shoup | IW | IW shoup], d words each. tid
// in [0, d / 16) within the group that synchronises on `bar`. kSmem: the
// tables were copied to shared memory (tab16 points there). kCompact: one
// window body for all windows (a third of the code, for launches whose
// blocks each run once per SM, where fetching unrolled code sets the time).
// kLazyOut: the slots are left in [0, 2p), for a caller that only passes
// them to mont_mul with a reduced second operand (a b < 2 p^2 < 2^32 p).
template <int LOGD, bool kSmem = false, bool kCompact = false, bool kLazyOut = false>
__device__ __forceinline__ void ntt16_forward(uint32_t (&x)[16], uint32_t* xs,
                                              const uint32_t* __restrict__ tab16,
                                              uint32_t p, int tid, int bar = 0) {
  using N = Ntt16<LOGD>;
  const uint32_t* tw = tab16;
  const uint32_t* tws = tab16 + N::kD;
  if constexpr (kCompact) {
#pragma unroll 1
    for (int w = 0; w < N::kPasses; ++w) {
      int base, stride, g;
      ntt16_geometry<LOGD>(w, tid, base, stride, g);
      if (w > 0) ntt16_load<LOGD>(x, xs, w, tid);
      ntt16_window<LOGD, kSmem, false>(x, tw, tws, p, w, g);
      if (w < N::kPasses - 1) ntt16_store<LOGD>(x, xs, w, tid);
      ntt16_sync<LOGD>(bar);
    }
  } else {
#pragma unroll
    for (int w = 0; w < N::kPasses; ++w) {
      int base, stride, g;
      ntt16_geometry<LOGD>(w, tid, base, stride, g);
      if (w > 0) ntt16_load<LOGD>(x, xs, w, tid);
      ntt16_window<LOGD, kSmem, false>(x, tw, tws, p, w, g);
      // The store goes to the words this thread read (no barrier between).
      if (w < N::kPasses - 1) ntt16_store<LOGD>(x, xs, w, tid);
      ntt16_sync<LOGD>(bar);
    }
  }
  if constexpr (!kLazyOut) {
    // [0, 2p) -> [0, p).
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = umin32(x[k], x[k] - p);
  }
}

// Inverse transform without the 1/d scaling. In: x[k] = slot 16 tid + k,
// any value below 2p. Out: x[k] = coefficient tid + (d / 16) k in [0, p).
// itw / itws: the permuted
// inverse twiddles and their Shoup constants.
template <int LOGD, bool kSmem = false, bool kCompact = false>
__device__ __forceinline__ void ntt16_inverse_tw(uint32_t (&x)[16], uint32_t* xs,
                                                 const uint32_t* __restrict__ itw,
                                                 const uint32_t* __restrict__ itws,
                                                 uint32_t p, int tid, int bar = 0) {
  using N = Ntt16<LOGD>;
  if constexpr (kCompact) {
#pragma unroll 1
    for (int w = N::kPasses - 1; w >= 0; --w) {
      int base, stride, g;
      ntt16_geometry<LOGD>(w, tid, base, stride, g);
      if (w < N::kPasses - 1) ntt16_load<LOGD>(x, xs, w, tid);
      ntt16_window<LOGD, kSmem, true>(x, itw, itws, p, w, g);
      if (w > 0) ntt16_store<LOGD>(x, xs, w, tid);
      ntt16_sync<LOGD>(bar);
    }
  } else {
#pragma unroll
    for (int w = N::kPasses - 1; w >= 0; --w) {
      int base, stride, g;
      ntt16_geometry<LOGD>(w, tid, base, stride, g);
      if (w < N::kPasses - 1) ntt16_load<LOGD>(x, xs, w, tid);
      ntt16_window<LOGD, kSmem, true>(x, itw, itws, p, w, g);
      if (w > 0) ntt16_store<LOGD>(x, xs, w, tid);
      ntt16_sync<LOGD>(bar);
    }
  }
  // [0, 2p) -> [0, p).
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = umin32(x[k], x[k] - p);
}

// The inverse with the prime's whole table block [W | W shoup | IW | IW shoup].
template <int LOGD, bool kSmem = false, bool kCompact = false>
__device__ __forceinline__ void ntt16_inverse(uint32_t (&x)[16], uint32_t* xs,
                                              const uint32_t* __restrict__ tab16,
                                              uint32_t p, int tid, int bar = 0) {
  ntt16_inverse_tw<LOGD, kSmem, kCompact>(x, xs, tab16 + 2 * Ntt16<LOGD>::kD,
                                          tab16 + 3 * Ntt16<LOGD>::kD, p, tid, bar);
}

// The slot layout the forward transform leaves (x[k] = slot 16 tid + k) in
// and out of the d-word buffer `xs`, conflict-free.
template <int LOGD>
__device__ __forceinline__ void ntt16_store_slots(const uint32_t (&x)[16], uint32_t* xs,
                                                  int tid) {
  ntt16_store<LOGD>(x, xs, Ntt16<LOGD>::kPasses - 1, tid);
}

template <int LOGD>
__device__ __forceinline__ void ntt16_load_slots(uint32_t (&x)[16], const uint32_t* xs,
                                                 int tid) {
  ntt16_load<LOGD>(x, xs, Ntt16<LOGD>::kPasses - 1, tid);
}
#endif

}  // namespace inspire
