// Kernels of PreprocessMatrixPack (offline packing preprocessing), all
// exact in Z_{2^w}.
//
// Reference: PreprocessPack, BuildPreprocessMatrix, EvaluateNttInPlace
// (crypto/lwes_to_rlwe.cc:88-119, 136-227, 229-353, 414-446).
//
// Two kinds of work:
//  * evaluations P(X^{2m}) of polynomials P(Z) = sum_i c[i] Z^i whose
//    coefficients are ring elements (a_hat_agg and the matrix blocks): a
//    radix-2 decimation-in-frequency transform whose twiddles are monomials,
//    so every butterfly is an add, a subtract and a signed rotation of whole
//    polynomials, one stage per launch over all (pair, coefficient) cells;
//  * the reduction chains of PreprocessPack: a sequential run of d/2 - 1
//    gadget decompositions and inner products with automorphed key parts,
//    one block per chain, the products as exact multi-prime NTTs in shared
//    memory (an automorphism is a permutation of NTT slots).
#pragma once
#include <cstdint>
#include <type_traits>

#include "ntt.cuh"
#include "ntt16.cuh"

namespace inspire {

template <typename T>
__device__ __forceinline__ T pp_low(T x, int bits) {
  return bits >= static_cast<int>(8 * sizeof(T)) ? x
                                                  : (x & ((T{1} << bits) - 1));
}

__device__ __forceinline__ int pp_bitrev(int x, int bits) {
  return static_cast<int>(__brev(static_cast<unsigned>(x)) >> (32 - bits));
}

// Coefficient x of X^e * p (0 <= e < d), p read through `get`.
template <typename T, typename G>
__device__ __forceinline__ T pp_rot_read(G get, int d, int e, int x) {
  return x >= e ? get(x - e) : static_cast<T>(T{0} - get(x - e + d));
}

// Steps 1-2 of PreprocessPack for every slice, transposed: out[s][m][j] =
// LowBits(LowBits(v, log_q) >> log d, log_q) with v = a_j[0] (m = 0) or
// -a_j[d - m], a_j = row j of the slice's block of the hint matrix.
// grid = (ceil(d/32) j tiles, ceil(d/32) m tiles, slices), block = (32, 8).
template <typename T>
__global__ void pp_atilde_kernel(const T* __restrict__ hint, int64_t stride, int d,
                                 int log_d, int log_q, T* __restrict__ out) {
  __shared__ T tile[32][33];
  const int s = blockIdx.z;
  const int j0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
  for (int jj = threadIdx.y; jj < 32; jj += 8) {
    const int j = j0 + jj, m = m0 + threadIdx.x;
    T v = 0;
    if (j < d && m < d) {
      const T a = hint[(static_cast<int64_t>(s) * d + j) * stride + (m == 0 ? 0 : d - m)];
      v = m == 0 ? a : static_cast<T>(T{0} - a);
      v = pp_low<T>(static_cast<T>(pp_low<T>(v, log_q) >> log_d), log_q);
    }
    tile[jj][threadIdx.x] = v;
  }
  __syncthreads();
  for (int mm = threadIdx.y; mm < 32; mm += 8) {
    const int m = m0 + mm, j = j0 + threadIdx.x;
    if (j < d && m < d) {
      out[(static_cast<int64_t>(s) * d + m) * d + j] = tile[threadIdx.x][mm];
    }
  }
}

// One radix-2 decimation-in-frequency stage of E[m] = sum_i c[i] X^{2im}
// (d polynomials of length d per slice; natural order in, bit-reversed order
// out once all log d stages ran). For blocks of 2h polynomials and j < h:
//   c'[b+j] = c[b+j] + c[b+j+h],  c'[b+j+h] = X^{j d / h} (c[b+j] - c[b+j+h]).
// With rot_in, input polynomial i is X^i * src[i]. One thread per (pair,
// coefficient); grid = (ceil(d/2 * d / blockDim), slices).
template <typename T>
__global__ void pp_dif_stage_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                    int d, int log_d, int log_h, int rot_in) {
  const int64_t cells = static_cast<int64_t>(d / 2) * d;
  const int64_t cell = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (cell >= cells) return;
  const int64_t base = static_cast<int64_t>(blockIdx.y) * d * d;
  const int pr = static_cast<int>(cell >> log_d);
  const int r = static_cast<int>(cell & (d - 1));
  const int h = 1 << log_h;
  const int j = pr & (h - 1);
  const int i0 = ((pr >> log_h) << (log_h + 1)) + j;
  const int i1 = i0 + h;
  const int e = j << (log_d - log_h);  // j d / h < d
  const T* p0 = src + base + static_cast<int64_t>(i0) * d;
  const T* p1 = src + base + static_cast<int64_t>(i1) * d;
  auto load = [&](const T* p, int i, int x) -> T {
    if (!rot_in) return p[x];
    return pp_rot_read<T>([&](int y) { return p[y]; }, d, i, x);
  };
  const T u = load(p0, i0, r), v = load(p1, i1, r);
  dst[base + static_cast<int64_t>(i0) * d + r] = static_cast<T>(u + v);
  const int rr = r >= e ? r - e : r - e + d;
  const T du = static_cast<T>(load(p0, i0, rr) - load(p1, i1, rr));
  dst[base + static_cast<int64_t>(i1) * d + r] = r >= e ? du : static_cast<T>(T{0} - du);
}

// Polynomial i of a matrix block before its transform: digit polynomial l of
// t_vec_g[j] (src_of[i] = 2j) or t_vec_gh[j] (2j + 1), zero for -1
// (BuildPreprocessMatrix, lwes_to_rlwe.cc:154-172). grid = (ceil(d*d/256), slices).
template <typename T>
__global__ void pp_block_input_kernel(const T* __restrict__ tg, const T* __restrict__ tgh,
                                      const int* __restrict__ src_of, int d, int log_d,
                                      int k, int l, int64_t chain_stride,
                                      T* __restrict__ out) {
  const int64_t cell = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (cell >= static_cast<int64_t>(d) * d) return;
  const int s = blockIdx.y;
  const int i = static_cast<int>(cell >> log_d), r = static_cast<int>(cell & (d - 1));
  const int src = __ldg(src_of + i);
  T v = 0;
  if (src >= 0) {
    const T* chain = (src & 1) ? tgh : tg;
    v = chain[s * chain_stride + (static_cast<int64_t>(src >> 1) * k + l) * d + r];
  }
  out[static_cast<int64_t>(s) * d * d + cell] = v;
}

// Column c of block l of the matrix is X^c E[c], E[c] the transform's slot
// bitrev(c); entry (r, l d + c) is that coefficient, shifted down by 2^log_q
// when at or above 2^(log_q - 1) (log_q below the word width), narrowed to
// the matrix element type M. 32 x 32 tiles through shared memory.
// grid = (ceil(d/32) c tiles, ceil(d/32) r tiles, slices), block = (32, 8).
template <typename T, typename M>
__global__ void pp_matrix_kernel(const T* __restrict__ ev, int d, int log_d, int log_q,
                                 int k, int l, M* __restrict__ out) {
  __shared__ T tile[32][33];
  constexpr int kW = 8 * sizeof(T);
  const T threshold = log_q >= kW ? (T{1} << (kW - 1)) : (T{1} << (log_q - 1));
  const int s = blockIdx.z;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int cc = threadIdx.y; cc < 32; cc += 8) {
    const int c = c0 + cc, r = r0 + threadIdx.x;
    T v = 0;
    if (c < d && r < d) {
      const T* e = ev + (static_cast<int64_t>(s) * d + pp_bitrev(c, log_d)) * d;
      v = pp_rot_read<T>([&](int y) { return e[y]; }, d, c, r);
      if (v >= threshold && log_q < kW) v = static_cast<T>(v - (T{1} << log_q));
    }
    tile[cc][threadIdx.x] = v;
  }
  __syncthreads();
  for (int rr = threadIdx.y; rr < 32; rr += 8) {
    const int r = r0 + rr, c = c0 + threadIdx.x;
    if (c < d && r < d) {
      out[(static_cast<int64_t>(s) * d + r) * (static_cast<int64_t>(k) * d) +
          static_cast<int64_t>(l) * d + c] = static_cast<M>(tile[threadIdx.x][rr]);
    }
  }
}

struct ChainArgs {
  int d, log_d, log_q, log_digit, k;
  int64_t chain_stride;   // elements per slice of t_vec_g / t_vec_gh
  const int* hat_row;     // [d]: transform slot holding a_hat_agg[k]
  const int* pow5;        // [d/2]: 5^i mod 2d
  const uint32_t* Wg;     // [k][r][d] NTT of w_vec_g (plain residues)
  const uint32_t* Wh;     // [k][r][d] NTT of w_vec_h
};

__device__ __forceinline__ uint32_t pp_signed_residue(int64_t x, uint32_t p) {
  const int64_t m = x % static_cast<int64_t>(p);
  return static_cast<uint32_t>(m < 0 ? m + p : m);
}

// Polynomial::SignedGadgetInv of LowBits(x, log_q) (polynomial.cc:376-427):
// digit l, a signed value, goes to out[l * stride] as a two's complement word.
template <typename T>
__device__ __forceinline__ void pp_signed_digits(T x, int log_q, int log_digit, int k,
                                                 T* out, int64_t stride) {
  constexpr int kW = 8 * sizeof(T);
  const int lq = log_q == 0 ? kW : log_q;
  T cur = pp_low<T>(x, log_q);
  const int to_shift = lq - k * log_digit;
  if (to_shift > 0) {
    // (cur + 2^(to_shift-1)) >> to_shift without losing the carry.
    const T half = T{1} << (to_shift - 1);
    const T sum = static_cast<T>(cur + half);
    const T carry = sum < cur ? T{1} : T{0};
    cur = static_cast<T>((sum >> to_shift) |
                         (to_shift < kW ? (carry << (kW - to_shift)) : T{0}));
  }
  const T mask = (T{1} << log_digit) - 1;
  const T half = T{1} << (log_digit - 1);
  for (int l = 0; l < k; ++l) {
    const T lower = cur & mask;
    if (lower >= half) {
      out[l * stride] = static_cast<T>(lower - (T{1} << log_digit));
      cur = static_cast<T>((cur >> log_digit) + 1);
    } else {
      out[l * stride] = lower;
      cur = cur >> log_digit;
    }
  }
}

// One link of a chain, in shared memory: digits of LowBits(cur) (written to
// digits[l][d]), their NTTs times the key part transforms read through the
// automorphism X -> X^power, inverse NTT, CRT; cur <- add[] + the product.
// blockDim.x * 4 * ITERS == d.
template <typename T, int ITERS>
__device__ __forceinline__ void pp_link(T* cur, uint32_t* scratch, uint32_t* acc,
                                        const ChainArgs& a, const NttCtx& c, int power,
                                        const uint32_t* W, T* digits, const T* add) {
  using S = typename std::make_signed<T>::type;
  constexpr int kPer = 4 * ITERS;
  const int d = a.d;
  // Digits, kPer coefficients per thread, kept in global memory: the matrix
  // needs them later and every NTT below re-reads one digit plane.
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int r = threadIdx.x + q * blockDim.x;
    pp_signed_digits<T>(cur[r], a.log_q, a.log_digit, a.k, digits + r, d);
  }
  // Slot sl of a transform holds its value at psi^(2 brv(sl) + 1); under
  // X -> X^power that is the key part's value at psi^(power (2 brv(sl) + 1)).
  int src[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int sl = threadIdx.x + q * blockDim.x;
    const int e = static_cast<int>(
        (static_cast<int64_t>(power) * (2 * pp_bitrev(sl, a.log_d) + 1)) % (2 * d));
    src[q] = pp_bitrev((e - 1) >> 1, a.log_d);
  }
  for (int i = threadIdx.x; i < c.r * d; i += blockDim.x) acc[i] = 0;
  __syncthreads();
  for (int l = 0; l < a.k; ++l) {
    for (int pi = 0; pi < c.r; ++pi) {
      const uint32_t p = c.p[pi];
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        const int r = threadIdx.x + q * blockDim.x;
        scratch[r] = pp_signed_residue(
            static_cast<int64_t>(static_cast<S>(digits[static_cast<int64_t>(l) * d + r])), p);
      }
      ntt_forward_t<ITERS>(scratch, c, pi);
      const uint32_t* w = W + (static_cast<int64_t>(l) * c.r + pi) * d;
      uint32_t* ap = acc + static_cast<int64_t>(pi) * d;
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        const int sl = threadIdx.x + q * blockDim.x;
        ap[sl] = add_mod(ap[sl], mont_mul(scratch[sl], __ldg(w + src[q]), p, c.pinv[pi]), p);
      }
      __syncthreads();  // scratch is rewritten next
    }
  }
  for (int pi = 0; pi < c.r; ++pi) ntt_inverse_t<ITERS>(acc + static_cast<int64_t>(pi) * d, c, pi);
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int r = threadIdx.x + q * blockDim.x;
    uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      if (pi < c.r) {
        x[pi] = shoup_mul(acc[static_cast<int64_t>(pi) * d + r], c.scale[pi],
                          c.scale_s[pi], c.p[pi]);
      }
    }
    cur[r] = static_cast<T>(add[r] + crt_reconstruct<T>(x, c));
  }
  __syncthreads();
}

// The two reduction chains of PreprocessPack (lwes_to_rlwe.cc:310-344) for
// every slice: blockIdx.x = 0 runs t_g over a_hat_agg[i], powers 5^i;
// blockIdx.x = 1 runs t_gh over a_hat_agg[d/2 + i], powers (2d-1) 5^i; both
// for i = d/2 - 2 .. 0, writing the digit polynomials t_vec_g[i] /
// t_vec_gh[i] ([slice][i][l][d]) and the final t to fin[slice][chain][d].
// grid = (2, slices), block = d / (4 ITERS).
template <typename T, int ITERS>
__global__ void __launch_bounds__(1024)
pp_chain_kernel(const T* __restrict__ ev, ChainArgs a, NttCtx c, T* __restrict__ tg,
                T* __restrict__ tgh, T* __restrict__ fin) {
  extern __shared__ __align__(16) unsigned char pp_smem[];
  const int d = a.d;
  T* cur = reinterpret_cast<T*>(pp_smem);
  uint32_t* scratch = reinterpret_cast<uint32_t*>(cur + d);
  uint32_t* acc = scratch + d;
  const int chain = blockIdx.x, s = blockIdx.y;
  const T* evs = ev + static_cast<int64_t>(s) * d * d;
  const T* start = evs + static_cast<int64_t>(__ldg(a.hat_row + (chain == 0 ? d / 2 - 1 : d - 1))) * d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) cur[r] = start[r];
  __syncthreads();
  T* out = (chain == 0 ? tg : tgh) + s * a.chain_stride;
  for (int i = d / 2 - 2; i >= 0; --i) {
    const int p5 = __ldg(a.pow5 + i);
    const int power = chain == 0
                          ? p5
                          : static_cast<int>((static_cast<int64_t>(p5) * (2 * d - 1)) % (2 * d));
    const T* add = evs + static_cast<int64_t>(__ldg(a.hat_row + (chain == 0 ? i : d / 2 + i))) * d;
    pp_link<T, ITERS>(cur, scratch, acc, a, c, power, a.Wg,
                      out + static_cast<int64_t>(i) * a.k * d, add);
  }
  T* f = fin + (static_cast<int64_t>(s) * 2 + chain) * d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) f[r] = cur[r];
}

// The tail of PreprocessPack (lwes_to_rlwe.cc:346-353): t_vec_h = the digits
// of LowBits(t_gh), a_tilde_agg = LowBits(t_g + <t_vec_h, w_vec_h>).
// grid = slices, block = d / (4 ITERS).
template <typename T, int ITERS>
__global__ void __launch_bounds__(1024)
pp_tail_kernel(const T* __restrict__ fin, ChainArgs a, NttCtx c, T* __restrict__ t_vec_h,
               T* __restrict__ a_tilde) {
  extern __shared__ __align__(16) unsigned char pp_smem[];
  const int d = a.d;
  T* cur = reinterpret_cast<T*>(pp_smem);
  uint32_t* scratch = reinterpret_cast<uint32_t*>(cur + d);
  uint32_t* acc = scratch + d;
  const int s = blockIdx.x;
  const T* tgf = fin + static_cast<int64_t>(s) * 2 * d;
  const T* tghf = tgf + d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) cur[r] = tghf[r];
  __syncthreads();
  pp_link<T, ITERS>(cur, scratch, acc, a, c, 1, a.Wh,
                    t_vec_h + static_cast<int64_t>(s) * a.k * d, tgf);
  for (int r = threadIdx.x; r < d; r += blockDim.x) {
    a_tilde[static_cast<int64_t>(s) * d + r] = pp_low<T>(cur[r], a.log_q);
  }
}

// pp_link with the radix-16 register transforms of ntt16.cuh (d = 2^LOGD,
// LOGD = 11..13), for a block of G groups of d/16 threads: group g takes
// primes g, g + G, ..., each group's transforms synchronising on named
// barrier g + 1, so the k forward transforms and the inverse of G primes run
// side by side; the residues meet in shared memory (res, natural
// coefficient order) for the CRT. xs: G exchange buffers of d words; dig:
// the k digit planes of `cur` (k d words of T). The link is a chain of
// dependent steps, so the digit planes go to shared memory for the
// transforms (and out to `digits` for the matrix, not read back), and
// `add` is loaded while other groups finish. Signed digits are below p in
// magnitude, so their residues need no division. Same words as pp_link.
template <typename T, int LOGD, int G>
__device__ __forceinline__ void pp_link16(T* cur, uint32_t* res, uint32_t* xs, T* dig,
                                          const ChainArgs& a, const NttCtx& c, int power,
                                          const uint32_t* W, T* digits, const T* add) {
  using S = typename std::make_signed<T>::type;
  constexpr int d = 1 << LOGD;
  constexpr int NT = Ntt16<LOGD>::kThreads;
  constexpr int kPerThread = (d + G * NT - 1) / (G * NT);
  // The compact transforms (one pass body: fewer registers beside the
  // digit and accumulator arrays, less code for a block that runs alone).
  constexpr bool kCompact = true;
  const int g = threadIdx.x / NT;
  const int lt = threadIdx.x % NT;
  // The digit planes, in shared memory and out for the matrix.
  for (int r = threadIdx.x; r < d; r += G * NT) {
    pp_signed_digits<T>(cur[r], a.log_q, a.log_digit, a.k, dig + r, d);
    for (int l = 0; l < a.k; ++l) digits[static_cast<int64_t>(l) * d + r] = dig[l * d + r];
  }
  __syncthreads();
  uint32_t* x_buf = xs + g * d;
  for (int pi = g; pi < c.r; pi += G) {
    const uint32_t p = c.p[pi];
    const uint32_t pinv = c.pinv[pi];
    const uint32_t* tab16 = c.tables16 + static_cast<size_t>(pi) * 4 * d;
    uint32_t acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0;
    for (int l = 0; l < a.k; ++l) {
      uint32_t x[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        // Digit l of coefficient lt + NT q; |digit| <= 2^(log_digit - 1) < p.
        const S v = static_cast<S>(dig[l * d + lt + NT * q]);
        x[q] = v < 0 ? static_cast<uint32_t>(static_cast<int64_t>(v) + p)
                     : static_cast<uint32_t>(v);
      }
      ntt16_forward<LOGD, false, kCompact, true>(x, x_buf, tab16, p, lt, g + 1);
      // Slot 16 lt + q times the key part read through X -> X^power
      // (pp_link's permutation).
      const uint32_t* w = W + (static_cast<int64_t>(l) * c.r + pi) * d;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int sl = 16 * lt + q;
        const int e = static_cast<int>(
            (static_cast<int64_t>(power) * (2 * pp_bitrev(sl, LOGD) + 1)) & (2 * d - 1));
        const int src = pp_bitrev((e - 1) >> 1, LOGD);
        acc[q] = add_mod(acc[q], mont_mul(x[q], __ldg(w + src), p, pinv), p);
      }
    }
    ntt16_inverse<LOGD, false, kCompact>(acc, x_buf, tab16, p, lt, g + 1);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      res[static_cast<int64_t>(pi) * d + lt + NT * q] =
          shoup_mul(acc[q], c.scale[pi], c.scale_s[pi], p);
    }
  }
  T add_r[kPerThread];
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const int r = threadIdx.x + j * G * NT;
    add_r[j] = r < d ? add[r] : T{0};
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const int r = threadIdx.x + j * G * NT;
    if (r < d) {
      uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
      for (int pi = 0; pi < kMaxPrimes; ++pi) {
        if (pi < c.r) x[pi] = res[static_cast<int64_t>(pi) * d + r];
      }
      cur[r] = static_cast<T>(add_r[j] + crt_reconstruct<T>(x, c));
    }
  }
  __syncthreads();
}

// pp_chain_kernel with pp_link16: grid = (2, slices), block = G d/16
// threads, shared memory (1 + k) d words of T + (r + G) d words (needs
// c.tables16).
template <typename T, int LOGD, int G>
__global__ void __launch_bounds__(G * Ntt16<LOGD>::kThreads, 1)
pp_chain16_kernel(const T* __restrict__ ev, ChainArgs a, NttCtx c, T* __restrict__ tg,
                  T* __restrict__ tgh, T* __restrict__ fin) {
  extern __shared__ __align__(16) unsigned char pp_smem[];
  constexpr int d = 1 << LOGD;
  T* cur = reinterpret_cast<T*>(pp_smem);
  uint32_t* res = reinterpret_cast<uint32_t*>(cur + d);
  uint32_t* xs = res + static_cast<int64_t>(c.r) * d;
  T* dig = reinterpret_cast<T*>(xs + G * d);
  const int chain = blockIdx.x, s = blockIdx.y;
  const T* evs = ev + static_cast<int64_t>(s) * d * d;
  const T* start = evs + static_cast<int64_t>(__ldg(a.hat_row + (chain == 0 ? d / 2 - 1 : d - 1))) * d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) cur[r] = start[r];
  __syncthreads();
  T* out = (chain == 0 ? tg : tgh) + s * a.chain_stride;
  for (int i = d / 2 - 2; i >= 0; --i) {
    const int p5 = __ldg(a.pow5 + i);
    const int power = chain == 0
                          ? p5
                          : static_cast<int>((static_cast<int64_t>(p5) * (2 * d - 1)) % (2 * d));
    const T* add = evs + static_cast<int64_t>(__ldg(a.hat_row + (chain == 0 ? i : d / 2 + i))) * d;
    pp_link16<T, LOGD, G>(cur, res, xs, dig, a, c, power, a.Wg,
                          out + static_cast<int64_t>(i) * a.k * d, add);
  }
  T* f = fin + (static_cast<int64_t>(s) * 2 + chain) * d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) f[r] = cur[r];
}

// pp_tail_kernel with pp_link16. grid = slices, block = G d/16 threads.
template <typename T, int LOGD, int G>
__global__ void __launch_bounds__(G * Ntt16<LOGD>::kThreads, 1)
pp_tail16_kernel(const T* __restrict__ fin, ChainArgs a, NttCtx c, T* __restrict__ t_vec_h,
                 T* __restrict__ a_tilde) {
  extern __shared__ __align__(16) unsigned char pp_smem[];
  constexpr int d = 1 << LOGD;
  T* cur = reinterpret_cast<T*>(pp_smem);
  uint32_t* res = reinterpret_cast<uint32_t*>(cur + d);
  uint32_t* xs = res + static_cast<int64_t>(c.r) * d;
  T* dig = reinterpret_cast<T*>(xs + G * d);
  const int s = blockIdx.x;
  const T* tgf = fin + static_cast<int64_t>(s) * 2 * d;
  const T* tghf = tgf + d;
  for (int r = threadIdx.x; r < d; r += blockDim.x) cur[r] = tghf[r];
  __syncthreads();
  pp_link16<T, LOGD, G>(cur, res, xs, dig, a, c, 1, a.Wh,
                        t_vec_h + static_cast<int64_t>(s) * a.k * d, tgf);
  for (int r = threadIdx.x; r < d; r += blockDim.x) {
    a_tilde[static_cast<int64_t>(s) * d + r] = pp_low<T>(cur[r], a.log_q);
  }
}

}  // namespace inspire
