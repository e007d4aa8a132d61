// Offline DB interpolation on the GPU: PreprocessingServer's
// InterpolateAndTranspose for every shard.
//
// Reference: PreprocessingServer::Preprocess / InterpolateAndTranspose
// (crypto/pir/server/preprocessing_server.h:68-95, 174-209) and Interpolate
// (crypto/db_row_interpolation.cc:115-228). Records i*t .. i*t+t-1 (shard k:
// the k-th d values of each record) are the evaluations of a degree < t
// polynomial over Z_p[X]/(X^d+1) at the powers of w = X^(2d/t); Interpolate
// inverts that DFT (bit-reversed Cooley-Tukey over polynomials, where
// multiplying by a power of w is a negacyclic rotation) and scales by
// t^-1 mod p. The result is transposed into the DB matrix: row
// k*t*d + j*d + c, column i.
//
// Structure. Multiplying by w^q = X^(q*s), s = 2d/t, moves coefficient c to
// c + q*s (negated on wrap-around), so the coefficient positions split into
// s independent classes {c0 + m*s : m < t/2}. A block takes a tile of G
// consecutive groups x R consecutive classes: coalesced loads (R consecutive
// positions of one record), the transform of each (group, class) in shared
// memory by one thread, and coalesced stores (G consecutive columns of one
// DB row). Every value is read and written once: HBM-bound.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/inspire_pir.h"

namespace inspire {
namespace {

constexpr int kTileValues = 16384;  // u32 values of one block's tile
constexpr int kThreads = 512;

struct InterpArgs {
  int d, t, logt, s, half;  // s = 2d/t classes, half = t/2 positions each
  int l;
  int64_t groups;           // n / t
  uint32_t p, tinv;
  uint32_t lazy_off;        // multiple of p >= t * max record value (LAZY)
  int G, R;                 // tile: groups x classes
  int64_t out_cols;
};

__device__ __forceinline__ int bitrev(int x, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r = (r << 1) | ((x >> b) & 1);
  return r;
}

// tile layout: [g][poly][m][class], the group stride padded by one word so
// that the column-major stores read shared memory without bank conflicts.
template <typename V>
__global__ void __launch_bounds__(kThreads)
interpolate_kernel(const V* __restrict__ raw, InterpArgs a, V* __restrict__ out) {
  extern __shared__ uint32_t tile[];
  const int per_group = a.t * a.half * a.R;
  const int gstride = per_group + 1;
  uint32_t* scratch = tile + a.G * gstride;  // t/2 words per subproblem slot
  const int64_t g0 = static_cast<int64_t>(blockIdx.x) * a.G;
  const int c_start = blockIdx.y * a.R;
  const int k = blockIdx.z;
  const int64_t left = a.groups - g0;
  const int G = left < a.G ? static_cast<int>(left) : a.G;
  const int R = min(a.R, a.s - c_start);

  // Load: c0 fastest (R consecutive positions of one record).
  const int64_t rec_stride = static_cast<int64_t>(a.l) * a.d;
  const int n_load = G * a.t * a.half * R;
  for (int idx = threadIdx.x; idx < n_load; idx += blockDim.x) {
    const int c0 = idx % R;
    const int m = (idx / R) % a.half;
    const int r = (idx / (R * a.half)) % a.t;
    const int g = idx / (R * a.half * a.t);
    const int64_t rec = (g0 + g) * a.t + r;
    const uint32_t v = static_cast<uint32_t>(
        raw[rec * rec_stride + static_cast<int64_t>(k) * a.d + c_start + c0 +
            static_cast<int64_t>(m) * a.s]);
    tile[g * gstride + (bitrev(r, a.logt) * a.half + m) * a.R + c0] = v % a.p;
  }
  __syncthreads();

  // Transform: one thread per (group, class).
  const int two_d = 2 * a.d;
  for (int sub = threadIdx.x; sub < G * R; sub += blockDim.x) {
    const int g = sub / R, c0 = sub % R;
    uint32_t* base = tile + g * gstride + c0;
    uint32_t* tmp = scratch + threadIdx.x * a.half;
    for (int len = 2; len <= a.t; len <<= 1) {
      const int h = len >> 1;
      const int step = (two_d - two_d / len) % two_d;
      for (int i = 0; i < a.t; i += len) {
        int w = 0;
        for (int j = 0; j < h; ++j) {
          uint32_t* pa = base + (i + j) * a.half * a.R;
          uint32_t* pb = base + (i + j + h) * a.half * a.R;
          for (int m = 0; m < a.half; ++m) tmp[m] = pb[m * a.R];
          // X^w * b: position c0 + m*s takes b at m - q (mod t/2), negated
          // when the rotation wraps (and once more when w >= d).
          const bool neg_all = w >= a.d;
          const int q = (w - (neg_all ? a.d : 0)) / a.s;
          for (int m = 0; m < a.half; ++m) {
            const bool wrap = m < q;
            const int src = wrap ? m - q + a.half : m - q;
            uint32_t v = tmp[src];
            if ((wrap != neg_all) && v != 0) v = a.p - v;
            // u, v < p, so u + v and u + p - v are below 2p (< 2^33).
            const uint64_t u = pa[m * a.R];
            const uint64_t sum = u + v, dif = u + a.p - v;
            pa[m * a.R] = static_cast<uint32_t>(sum >= a.p ? sum - a.p : sum);
            pb[m * a.R] = static_cast<uint32_t>(dif >= a.p ? dif - a.p : dif);
          }
          w = (w + step) % two_d;
        }
      }
    }
    for (int r = 0; r < a.t; ++r) {
      for (int m = 0; m < a.half; ++m) {
        uint32_t* x = base + (r * a.half + m) * a.R;
        *x = static_cast<uint32_t>((static_cast<uint64_t>(*x) * a.tinv) % a.p);
      }
    }
  }
  __syncthreads();

  // Store: g fastest (G consecutive columns of one DB row).
  const int n_store = G * a.t * a.half * R;
  for (int idx = threadIdx.x; idx < n_store; idx += blockDim.x) {
    const int g = idx % G;
    const int c0 = (idx / G) % R;
    const int m = (idx / (G * R)) % a.half;
    const int r = idx / (G * R * a.half);
    const int64_t row = static_cast<int64_t>(k) * a.t * a.d +
                        static_cast<int64_t>(r) * a.d + c_start + c0 +
                        static_cast<int64_t>(m) * a.s;
    out[row * a.out_cols + g0 + g] =
        static_cast<V>(tile[g * gstride + (r * a.half + m) * a.R + c0]);
  }
}

// Fast form for t in {2, 4, 8} and s = 2d/t >= 32: one thread owns one
// (group, class) subproblem of t x t/2 values in registers, so the
// transform is a fixed sequence of register butterflies (the rotations by
// powers of w are compile-time permutations of the class's positions).
// Loads are coalesced over 32
// consecutive classes; results pass through shared memory once so that the
// stores run over kFastG consecutive groups (DB columns).
constexpr int kFastR = 32;   // classes per block (one warp's lanes)
// Groups per block (kG: the stores run over kG consecutive columns) and
// groups in flight (kGW warps per block). 8- and 16-bit values take 32
// groups (64-byte row pieces; an 80 KB tile of 16-bit values at t = 8, two
// blocks per SM, as the registers of the t = 8 transform allow); wider
// values 16, which keeps the tile within a block's limit.
template <typename V>
struct FastShape {
  static constexpr int kG = sizeof(V) <= 2 ? 32 : 16;
  static constexpr int kGW = 8;
  // Tile row pitch in values: padded against bank conflicts; for 16-bit
  // values 40 (80-byte rows), so that eight neighbouring groups read as one
  // 16-byte vector.
  static constexpr int kRow = kG + (sizeof(V) == 2 ? 8 : 1);
};

// Modular helpers; SMALL: p < 2^31, so sums and Shoup remainders fit in 32
// bits.
template <bool SMALL>
__device__ __forceinline__ uint32_t add_p(uint32_t a, uint32_t b, uint32_t p) {
  if constexpr (SMALL) {
    const uint32_t s = a + b;
    return s >= p ? s - p : s;
  } else {
    const uint64_t s = static_cast<uint64_t>(a) + b;
    return static_cast<uint32_t>(s >= p ? s - p : s);
  }
}
__device__ __forceinline__ uint32_t sub_p(uint32_t a, uint32_t b, uint32_t p) {
  return a >= b ? a - b : static_cast<uint32_t>(static_cast<uint64_t>(a) + p - b);
}

// Constants of the reductions by p, computed on the host.
struct ModConsts {
  uint64_t barrett;   // floor(2^64 / p): x mod p for 32-bit x
  uint64_t tinv_s64;  // floor(tinv * 2^64 / p)
  uint32_t tinv_s32;  // floor(tinv * 2^32 / p) (p < 2^31)
};

// x mod p for any 32-bit x (Barrett: the quotient estimate is at most one
// short).
__device__ __forceinline__ uint32_t reduce_p(uint32_t x, uint32_t p, uint64_t barrett) {
  const uint64_t q = __umul64hi(static_cast<uint64_t>(x), barrett);
  uint64_t r = x - q * p;
  return static_cast<uint32_t>(r >= p ? r - p : r);
}

// x * tinv mod p for x < p (Shoup).
template <bool SMALL>
__device__ __forceinline__ uint32_t scale_p(uint32_t x, uint32_t tinv, uint32_t p,
                                            const ModConsts& mc) {
  if constexpr (SMALL) {
    const uint32_t q = __umulhi(x, mc.tinv_s32);
    const uint32_t r = x * tinv - q * p;
    return r >= p ? r - p : r;
  } else {
    const uint64_t q = __umul64hi(static_cast<uint64_t>(x), mc.tinv_s64);
    const uint64_t r = static_cast<uint64_t>(x) * tinv - q * p;
    return static_cast<uint32_t>(r >= p ? r - p : r);
  }
}

// r with its low `bits` bits reversed (bits <= 3), a constant expression for
// a constant r, so that register arrays indexed by it stay in registers.
__host__ __device__ constexpr int bit_reverse(int r, int bits) {
  return bits == 1 ? r
         : bits == 2 ? ((r & 1) << 1) | ((r >> 1) & 1)
                     : ((r & 1) << 2) | (r & 2) | ((r >> 2) & 1);
}

// The t x t/2 values of subproblem (group grp, class c) in bit-reversed
// record order, as they are stored (no reduction).
template <typename V, int T>
__device__ __forceinline__ void lazy_load(uint32_t (&x)[T][T / 2], const V* __restrict__ raw,
                                          int64_t grp, int64_t rec_stride, int k, int c,
                                          const InterpArgs& a) {
  constexpr int LOGT = T == 2 ? 1 : (T == 4 ? 2 : 3);
#pragma unroll
  for (int r = 0; r < T; ++r) {
    const V* src = raw + (grp * T + r) * rec_stride + static_cast<int64_t>(k) * a.d + c;
#pragma unroll
    for (int m = 0; m < T / 2; ++m) {
      x[bit_reverse(r, LOGT)][m] = static_cast<uint32_t>(src[m * a.s]);
    }
  }
}

// One butterfly stage (pairs LEN/2 apart within blocks of LEN) of the lazy
// transform, then the next: every bound is a template constant, so the
// subproblem's registers are indexed by constants only.
template <int T, int LEN>
__device__ __forceinline__ void lazy_stage(uint32_t (&x)[T][T / 2]) {
  constexpr int H = T / 2;
  constexpr int h = LEN / 2;
#pragma unroll
  for (int i = 0; i < T; i += LEN) {
#pragma unroll
    for (int j = 0; j < h; ++j) {
      // w^j = X^(j (2d - 2d/LEN)): in units of s a rotation by wu classes
      // mod T, negating all when it reaches d (H units).
      const int wu = (j * (T - T / LEN)) % T;
      const bool neg_all = wu >= H;
      const int q = neg_all ? wu - H : wu;
      int32_t v[H];
#pragma unroll
      for (int m = 0; m < H; ++m) {
        const bool wrap = m < q;
        const int32_t b = static_cast<int32_t>(x[i + j + h][wrap ? m - q + H : m - q]);
        v[m] = (wrap != neg_all) ? -b : b;
      }
#pragma unroll
      for (int m = 0; m < H; ++m) {
        const int32_t u = static_cast<int32_t>(x[i + j][m]);
        x[i + j][m] = static_cast<uint32_t>(u + v[m]);
        x[i + j + h][m] = static_cast<uint32_t>(u - v[m]);
      }
    }
  }
  if constexpr (2 * LEN <= T) lazy_stage<T, 2 * LEN>(x);
}

// The lazy transform of one (group, class) subproblem x (t x t/2 values
// of at most max(V) each, bit-reversed record order): butterflies on signed
// integers, (u, b) -> (u + v, u - v) with v = +-b, the rotation's
// permutation and sign fixed at compile time; |x| <= t * max(V) after
// log2(t) stages. One reduction at the end, (x + lazy_off) * t^-1 mod p
// (Shoup, valid for any 32-bit operand), left in x.
template <int T>
__device__ __forceinline__ void lazy_transform(uint32_t (&x)[T][T / 2], const InterpArgs& a,
                                               const ModConsts& mc) {
  lazy_stage<T, 2>(x);
#pragma unroll
  for (int r = 0; r < T; ++r) {
#pragma unroll
    for (int m = 0; m < T / 2; ++m) {
      const uint32_t y = x[r][m] + a.lazy_off;  // in [0, 2 lazy_off)
      const uint32_t qq = __umulhi(y, mc.tinv_s32);
      uint32_t rr = y * a.tinv - qq * a.p;
      x[r][m] = rr >= a.p ? rr - a.p : rr;
    }
  }
}

// Writes the transformed subproblems of groups gi (xa) and gi + 1 (xb, when
// hb) of class c0 to the block's tile; 16-bit values of the two groups go as
// one 32-bit word (gi even, even row pitch).
template <typename V, int T>
__device__ __forceinline__ void lazy_tile_store(const uint32_t (&xa)[T][T / 2],
                                                const uint32_t (&xb)[T][T / 2], bool hb,
                                                int gi, int c0, V* tile) {
  constexpr int H = T / 2;
  constexpr int kRow = FastShape<V>::kRow;
#pragma unroll
  for (int r = 0; r < T; ++r) {
#pragma unroll
    for (int m = 0; m < H; ++m) {
      V* dst = tile + ((r * H + m) * kFastR + c0) * kRow + gi;
      if constexpr (sizeof(V) == 2) {
        if (hb) {
          *reinterpret_cast<uint32_t*>(dst) = xa[r][m] | (xb[r][m] << 16);
        } else {
          dst[0] = static_cast<V>(xa[r][m]);
        }
      } else {
        dst[0] = static_cast<V>(xa[r][m]);
        if (hb) dst[1] = static_cast<V>(xb[r][m]);
      }
    }
  }
}

// LAZY: the transform runs on signed 32-bit integers without any reduction:
// every butterfly is an addition and a subtraction of values whose rotation
// by a power of w only permutes and negates them, so after log2(t) stages
// |x| <= t * max(V) (< 2^20 for 8- and 16-bit records). One reduction at the
// end, (x + lazy_off) * t^-1 mod p with lazy_off a multiple of p at least
// that bound (Shoup, valid for any 32-bit operand), gives the same residue
// as reducing after every step. Used when 2 * lazy_off < 2^32 and p < 2^31.
template <typename V, int T, bool SMALL, bool LAZY = false>
__global__ void __launch_bounds__(kFastR * FastShape<V>::kGW)
interpolate_fast_kernel(const V* __restrict__ raw, InterpArgs a, ModConsts mc,
                        V* __restrict__ out) {
  constexpr int H = T / 2;
  constexpr int LOGT = T == 2 ? 1 : (T == 4 ? 2 : 3);
  constexpr int kFastG = FastShape<V>::kG;
  constexpr int kFastGW = FastShape<V>::kGW;
  // [T*H rows][kFastR classes][kFastG + 1 groups] (dynamic shared memory)
  extern __shared__ __align__(16) unsigned char tile_raw[];
  V* tile = reinterpret_cast<V*>(tile_raw);
  constexpr int kRow = FastShape<V>::kRow;
  const int c0 = threadIdx.x % kFastR;
  const int gw = threadIdx.x / kFastR;
  // Class blocks fastest: blocks running together read neighbouring 64-byte
  // pieces of the same records.
  const int64_t g_base = static_cast<int64_t>(blockIdx.y) * kFastG;
  const int c_start = blockIdx.x * kFastR;
  const int k = blockIdx.z;
  const int64_t rec_stride = static_cast<int64_t>(a.l) * a.d;
  const uint32_t p = a.p;
  if constexpr (LAZY) {
    // Two neighbouring groups per pass: both groups' 2 t (t/2) loads are
    // issued before either is transformed (twice the bytes in flight per
    // warp), and their results share 32-bit tile words.
    for (int gi = 2 * gw; gi < kFastG; gi += 2 * kFastGW) {
      const bool ha = g_base + gi < a.groups;
      const bool hb = g_base + gi + 1 < a.groups;
      if (!ha) break;
      uint32_t xa[T][H], xb[T][H];
      lazy_load<V, T>(xa, raw, g_base + gi, rec_stride, k, c_start + c0, a);
      if (hb) lazy_load<V, T>(xb, raw, g_base + gi + 1, rec_stride, k, c_start + c0, a);
      lazy_transform<T>(xa, a, mc);
      if (hb) lazy_transform<T>(xb, a, mc);
      lazy_tile_store<V, T>(xa, xb, hb, gi, c0, tile);
    }
  } else {
  for (int gi = gw; gi < kFastG; gi += kFastGW) {
    const int64_t grp = g_base + gi;
    if (grp >= a.groups) break;
    uint32_t x[T][H];
    // Load in bit-reversed polynomial order.
#pragma unroll
    for (int r = 0; r < T; ++r) {
      int rb = 0;
#pragma unroll
      for (int b = 0; b < LOGT; ++b) rb |= ((r >> b) & 1) << (LOGT - 1 - b);
      const V* src = raw + (grp * T + r) * rec_stride + static_cast<int64_t>(k) * a.d +
                     c_start + c0;
#pragma unroll
      for (int m = 0; m < H; ++m) {
        x[rb][m] = reduce_p(static_cast<uint32_t>(src[m * a.s]), p, mc.barrett);
      }
    }

    // Butterflies: len = 2 .. T; pair (i + j, i + j + h) with w^j.
#pragma unroll
    for (int len = 2; len <= T; len <<= 1) {
      const int h = len / 2;
#pragma unroll
      for (int i = 0; i < T; i += len) {
#pragma unroll
        for (int j = 0; j < h; ++j) {
          // w^j = X^(j * (2d - 2d/len)); in units of s (2d = T*s, d = H*s)
          // a rotation by wu = j*(T - T/len) mod T, negating all when the
          // exponent reaches d, then a shift of q classes within [0, H).
          const int wu = (j * (T - T / len)) % T;
          const bool neg_all = wu >= H;
          const int q = neg_all ? wu - H : wu;
          uint32_t v[H];
#pragma unroll
          for (int m = 0; m < H; ++m) {
            const bool wrap = m < q;
            const int src = wrap ? m - q + H : m - q;
            const uint32_t b = x[i + j + h][src];
            v[m] = ((wrap != neg_all) && b != 0) ? p - b : b;
          }
#pragma unroll
          for (int m = 0; m < H; ++m) {
            const uint32_t u = x[i + j][m];
            x[i + j][m] = add_p<SMALL>(u, v[m], p);
            x[i + j + h][m] = sub_p(u, v[m], p);
          }
        }
      }
    }
    // Scale by t^-1 mod p.
#pragma unroll
    for (int r = 0; r < T; ++r) {
#pragma unroll
      for (int m = 0; m < H; ++m) {
        tile[((r * H + m) * kFastR + c0) * kRow + gi] =
            static_cast<V>(scale_p<SMALL>(x[r][m], a.tinv, p, mc));
      }
    }
  }
  }
  __syncthreads();
  // Stores: kFastG consecutive columns of each DB row.
  const int64_t left = a.groups - g_base;
  const int G = left < kFastG ? static_cast<int>(left) : kFastG;
  if constexpr (sizeof(V) == 2) {
    if ((a.out_cols & 7) == 0 && G == kFastG &&
        (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
      // Eight neighbouring groups per 16-byte store: four lanes write one
      // DB row's 64 bytes, a warp eight rows per instruction (row pitch a
      // multiple of 8 values, g_base a multiple of 32). Thread i writes
      // chunk i % 4 of class (i / 4) % 32, tile rows i / 128 + 2 j.
      constexpr int kChunks = kFastG / 8;
      constexpr int kThreads = kFastR * kFastGW;
      constexpr int kRmStep = kThreads / (kChunks * kFastR);
      constexpr int kIters = T * H / kRmStep;
      static_assert(kThreads % (kChunks * kFastR) == 0 && (T * H) % kRmStep == 0,
                    "16-byte store mapping");
      const int q = threadIdx.x % kChunks;
      const int c = (threadIdx.x / kChunks) % kFastR;
      const int rm0 = threadIdx.x / (kChunks * kFastR);
      const int64_t ds = static_cast<int64_t>(a.d) * a.out_cols;
      const int64_t ss = static_cast<int64_t>(a.s) * a.out_cols;
      V* dst = out + (static_cast<int64_t>(k) * T * a.d + c_start + c) * a.out_cols + g_base +
               8 * q;
      const V* src = tile + c * kRow + 8 * q;
#pragma unroll
      for (int j = 0; j < kIters; ++j) {
        const int rm = rm0 + kRmStep * j;
        const int r = rm / H, m = rm % H;
        const uint4 v = *reinterpret_cast<const uint4*>(src + rm * kFastR * kRow);
        *reinterpret_cast<uint4*>(dst + r * ds + m * ss) = v;
      }
      return;
    }
    if ((a.out_cols & 1) == 0 && G == kFastG &&
        (reinterpret_cast<uintptr_t>(out) & 3) == 0) {
      // Two neighbouring groups per 32-bit store (even row pitch, g_base a
      // multiple of 32: every store is 4-byte aligned).
      constexpr int kPairs = kFastG / 2;
      for (int idx = threadIdx.x; idx < T * H * kFastR * kPairs; idx += blockDim.x) {
        const int gp = idx % kPairs;
        const int c = (idx / kPairs) % kFastR;
        const int rm = idx / (kPairs * kFastR);
        const int r = rm / H, m = rm % H;
        const int64_t row = static_cast<int64_t>(k) * T * a.d +
                            static_cast<int64_t>(r) * a.d + c_start + c +
                            static_cast<int64_t>(m) * a.s;
        const uint32_t v =
            *reinterpret_cast<const uint32_t*>(tile + (rm * kFastR + c) * kRow + 2 * gp);
        *reinterpret_cast<uint32_t*>(out + row * a.out_cols + g_base + 2 * gp) = v;
      }
      return;
    }
  }
  for (int idx = threadIdx.x; idx < T * H * kFastR * kFastG; idx += blockDim.x) {
    const int g = idx % kFastG;
    const int c = (idx / kFastG) % kFastR;
    const int rm = idx / (kFastG * kFastR);
    if (g >= G) continue;
    const int r = rm / H, m = rm % H;
    const int64_t row = static_cast<int64_t>(k) * T * a.d + static_cast<int64_t>(r) * a.d +
                        c_start + c + static_cast<int64_t>(m) * a.s;
    out[row * a.out_cols + g_base + g] = tile[(rm * kFastR + c) * kRow + g];
  }
}

// t == 1: the transposition alone (Interpolate returns the row unchanged).
template <typename V>
__global__ void transpose_kernel(const V* __restrict__ raw, int d, int l,
                                 int64_t n, int64_t out_cols, V* __restrict__ out) {
  __shared__ V tile[32][33];
  const int64_t rows = static_cast<int64_t>(l) * d;  // per record
  const int64_t c_in = static_cast<int64_t>(blockIdx.x) * 32;  // records
  const int64_t r_in = static_cast<int64_t>(blockIdx.y) * 32;  // values
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t rec = c_in + y, val = r_in + threadIdx.x;
    if (rec < n && val < rows) tile[y][threadIdx.x] = raw[rec * rows + val];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t val = r_in + y, rec = c_in + threadIdx.x;
    if (rec < n && val < rows) out[val * out_cols + rec] = tile[threadIdx.x][y];
  }
}

int Fail(char* err, size_t err_len, int code, const std::string& msg) {
  if (err != nullptr && err_len > 0) std::snprintf(err, err_len, "%s", msg.c_str());
  return code;
}

bool Pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

int64_t ModInverse(int64_t a, int64_t m) {
  int64_t t = 0, nt = 1, r = m, nr = a;
  while (nr != 0) {
    const int64_t q = r / nr;
    int64_t tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  if (r > 1) return -1;
  return t < 0 ? t + m : t;
}

// Validation in the reference's order (db_row_interpolation.cc:122-142).
int Check(int d, int t, uint32_t p, char* err, size_t err_len) {
  if (!Pow2(d)) return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT, "ring_degree must be a power of two.");
  if (!Pow2(t)) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                "interpolation_degree must be a power of two.");
  }
  if (t > 2 * d) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                "interpolation_degree must be less than or equal to 2 * ring_degree.");
  }
  if (t > 1 && p % 2 == 0) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT, "plaintext_modulus must be odd.");
  }
  return INSPIRE_OK;
}

template <typename V>
int Run(const V* raw, int64_t n, int d, int t, int l, uint32_t p, V* out,
        int64_t out_cols, cudaStream_t st, char* err, size_t err_len) {
  const int64_t groups = n / t;
  const int64_t rows = static_cast<int64_t>(l) * t * d;
  cudaError_t e = cudaSuccess;
  if (out_cols > groups) {
    e = cudaMemset2DAsync(out + groups, out_cols * sizeof(V), 0,
                          (out_cols - groups) * sizeof(V), rows, st);
  }
  if (e == cudaSuccess && groups > 0 && t == 1) {
    dim3 grid(static_cast<unsigned>((groups + 31) / 32),
              static_cast<unsigned>((static_cast<int64_t>(l) * d + 31) / 32));
    transpose_kernel<V><<<grid, dim3(32, 8), 0, st>>>(raw, d, l, groups, out_cols, out);
    e = cudaGetLastError();
  } else if (e == cudaSuccess && groups > 0) {
    InterpArgs a{};
    a.d = d;
    a.t = t;
    a.logt = 0;
    while ((1 << a.logt) < t) ++a.logt;
    a.s = 2 * d / t;
    a.half = t / 2;
    a.l = l;
    a.groups = groups;
    a.p = p;
    const int64_t inv = ModInverse(t % p, p);
    if (inv < 0) {
      return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                  "a is not invertible modulo m (not coprime).");
    }
    a.tinv = static_cast<uint32_t>(inv);
    a.out_cols = out_cols;
    if ((t == 2 || t == 4 || t == 8) && a.s >= kFastR && a.s % kFastR == 0) {
      ModConsts mc;
      mc.barrett = static_cast<uint64_t>((static_cast<unsigned __int128>(1) << 64) / p);
      mc.tinv_s64 = static_cast<uint64_t>((static_cast<unsigned __int128>(a.tinv) << 64) / p);
      mc.tinv_s32 = static_cast<uint32_t>((static_cast<uint64_t>(a.tinv) << 32) / p);
      const bool small = p < (1u << 31);
      // The lazy transform: t * max(record value) bounds every intermediate.
      const uint64_t vmax = sizeof(V) >= 4 ? 0xffffffffull : (1ull << (8 * sizeof(V))) - 1;
      const uint64_t bound = static_cast<uint64_t>(t) * std::max<uint64_t>(vmax, p);
      const uint64_t off = (bound + p - 1) / p * p;
      const bool lazy = sizeof(V) <= 2 && small && 2 * off < (1ull << 31);
      a.lazy_off = static_cast<uint32_t>(lazy ? off : 0);
      constexpr int kFastG = FastShape<V>::kG;
      dim3 grid(static_cast<unsigned>(a.s / kFastR),
                static_cast<unsigned>((groups + kFastG - 1) / kFastG), static_cast<unsigned>(l));
      const int threads = kFastR * FastShape<V>::kGW;
      const size_t smem =
          static_cast<size_t>(t) * (t / 2) * kFastR * FastShape<V>::kRow * sizeof(V);
      auto launch = [&](auto kernel) {
        cudaError_t r = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (r == cudaSuccess) {
          kernel<<<grid, threads, smem, st>>>(raw, a, mc, out);
          r = cudaGetLastError();
        }
        return r;
      };
      if (t == 2) {
        e = lazy    ? launch(interpolate_fast_kernel<V, 2, true, true>)
            : small ? launch(interpolate_fast_kernel<V, 2, true>)
                    : launch(interpolate_fast_kernel<V, 2, false>);
      } else if (t == 4) {
        e = lazy    ? launch(interpolate_fast_kernel<V, 4, true, true>)
            : small ? launch(interpolate_fast_kernel<V, 4, true>)
                    : launch(interpolate_fast_kernel<V, 4, false>);
      } else {
        e = lazy    ? launch(interpolate_fast_kernel<V, 8, true, true>)
            : small ? launch(interpolate_fast_kernel<V, 8, true>)
                    : launch(interpolate_fast_kernel<V, 8, false>);
      }
      if (e != cudaSuccess) {
        return Fail(err, err_len, INSPIRE_INTERNAL,
                    std::string("interpolate: ") + cudaGetErrorString(e));
      }
      return INSPIRE_OK;
    }
    const int sub = t * a.half;  // values of one (group, class)
    a.R = std::min(a.s, 32);
    a.G = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(16, kTileValues / (sub * a.R))));
    if (static_cast<int64_t>(a.G) * sub * a.R > kTileValues) {
      a.R = std::max(1, kTileValues / (a.G * sub));
    }
    // Widen the class tile while the block stays within its budget.
    while (a.R * 2 <= a.s && static_cast<int64_t>(a.G) * sub * a.R * 2 <= kTileValues &&
           a.G * a.R * 2 <= 8 * kThreads) {
      a.R *= 2;
    }
    a.out_cols = out_cols;
    const int threads = std::min(kThreads, a.G * a.R);
    const size_t smem = (static_cast<size_t>(a.G) * (sub * a.R + 1) +
                         static_cast<size_t>(threads) * a.half) * 4;
    e = cudaFuncSetAttribute(interpolate_kernel<V>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    if (e == cudaSuccess) {
      dim3 grid(static_cast<unsigned>((groups + a.G - 1) / a.G),
                static_cast<unsigned>((a.s + a.R - 1) / a.R), static_cast<unsigned>(l));
      interpolate_kernel<V><<<grid, threads, smem, st>>>(raw, a, out);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) {
    return Fail(err, err_len, INSPIRE_INTERNAL,
                std::string("interpolate: ") + cudaGetErrorString(e));
  }
  return INSPIRE_OK;
}

template <typename V>
int RunHost(const void* raw, int64_t n, int d, int t, int l, uint32_t p, void* out,
            int64_t out_cols, char* err, size_t err_len) {
  const size_t in_bytes = static_cast<size_t>(n) * l * d * sizeof(V);
  const size_t out_bytes = static_cast<size_t>(l) * t * d * out_cols * sizeof(V);
  void *din = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&din, in_bytes > 0 ? in_bytes : 1);
  if (e == cudaSuccess) e = cudaMalloc(&dout, out_bytes > 0 ? out_bytes : 1);
  if (e == cudaSuccess && in_bytes) e = cudaMemcpy(din, raw, in_bytes, cudaMemcpyHostToDevice);
  int rc = INSPIRE_OK;
  if (e == cudaSuccess) {
    rc = Run<V>(static_cast<const V*>(din), n, d, t, l, p, static_cast<V*>(dout), out_cols,
                nullptr, err, err_len);
    if (rc == INSPIRE_OK) e = cudaDeviceSynchronize();
    if (rc == INSPIRE_OK && e == cudaSuccess && out_bytes) {
      e = cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost);
    }
  }
  if (din) cudaFree(din);
  if (dout) cudaFree(dout);
  if (rc == INSPIRE_OK && e != cudaSuccess) {
    rc = Fail(err, err_len, INSPIRE_INTERNAL, std::string("interpolate: ") + cudaGetErrorString(e));
  }
  return rc;
}

}  // namespace
}  // namespace inspire

extern "C" {

int inspire_interpolate_db(int32_t value_bits, const void* db_raw, int64_t db_raw_len,
                           int64_t num_entries, int32_t ring_degree,
                           int32_t interpolation_degree, int32_t entry_size_multiple,
                           uint32_t plaintext_modulus, void* out, int64_t out_cols,
                           int32_t on_device, void* stream, char* err, size_t err_len) {
  using namespace inspire;
  const int d = ring_degree, t = interpolation_degree, l = entry_size_multiple;
  if (db_raw == nullptr || out == nullptr || num_entries < 0 || l <= 0) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                "db_raw/out must be set, num_entries >= 0, entry_size_multiple > 0.");
  }
  if (db_raw_len != num_entries * d * l) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT, "Invalid raw database size.");
  }
  int rc = Check(d, t, plaintext_modulus, err, err_len);
  if (rc != INSPIRE_OK) return rc;
  if (out_cols < num_entries / t) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                "out_cols must be at least num_entries / interpolation_degree.");
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (value_bits) {
    case 8:
      return on_device ? Run<uint8_t>(static_cast<const uint8_t*>(db_raw), num_entries, d, t,
                                      l, plaintext_modulus, static_cast<uint8_t*>(out),
                                      out_cols, st, err, err_len)
                       : RunHost<uint8_t>(db_raw, num_entries, d, t, l, plaintext_modulus,
                                          out, out_cols, err, err_len);
    case 16:
      return on_device ? Run<uint16_t>(static_cast<const uint16_t*>(db_raw), num_entries, d,
                                       t, l, plaintext_modulus, static_cast<uint16_t*>(out),
                                       out_cols, st, err, err_len)
                       : RunHost<uint16_t>(db_raw, num_entries, d, t, l, plaintext_modulus,
                                           out, out_cols, err, err_len);
    case 32:
      return on_device ? Run<uint32_t>(static_cast<const uint32_t*>(db_raw), num_entries, d,
                                       t, l, plaintext_modulus, static_cast<uint32_t*>(out),
                                       out_cols, st, err, err_len)
                       : RunHost<uint32_t>(db_raw, num_entries, d, t, l, plaintext_modulus,
                                           out, out_cols, err, err_len);
    default:
      return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT, "value_bits must be 8, 16 or 32.");
  }
}

int inspire_interpolate(int32_t value_bits, const void* db_row, int64_t db_row_len,
                        int32_t ring_degree, int32_t interpolation_degree,
                        uint32_t plaintext_modulus, void* out, char* err, size_t err_len) {
  using namespace inspire;
  if (db_row_len != static_cast<int64_t>(ring_degree) * interpolation_degree) {
    return Fail(err, err_len, INSPIRE_INVALID_ARGUMENT,
                "Length of evals must be ring_degree * interpolation_degree.");
  }
  const int rc = Check(ring_degree, interpolation_degree, plaintext_modulus, err, err_len);
  if (rc != INSPIRE_OK) return rc;
  // One group of t records of one shard; the DB matrix of one column is the
  // interpolated row itself (t*d rows x 1 column).
  return inspire_interpolate_db(value_bits, db_row, db_row_len, interpolation_degree,
                                ring_degree, interpolation_degree, 1, plaintext_modulus,
                                out, 1, 0, nullptr, err, err_len);
}

}  // extern "C"
