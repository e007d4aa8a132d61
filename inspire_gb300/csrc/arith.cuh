// Word-size modular arithmetic for the exact negacyclic products.
//
// The reference multiplies polynomials with an FP64 FFT over 2d points and
// rounds (crypto/polynomial_fft.cc:68-197). On the GPU the same integer
// result is produced exactly with a negacyclic NTT over a few 31-bit primes
// p = c * 2^16 + 1 (so a primitive 2d-th root of unity exists for d <= 2^15)
// followed by a Garner CRT reconstruction mod 2^w. All arithmetic is 32-bit:
//   * Shoup multiplication by precomputed constants (twiddles, scalings),
//   * signed Montgomery multiplication for variable x variable products.
#pragma once
#include <cstdint>

namespace inspire {

constexpr int kMaxPrimes = 5;
constexpr int kLogMaxDegree = 15;

// Per-prime constants. `pinv` is p^-1 mod 2^32 (Montgomery, R = 2^32).
struct PrimeConst {
  uint32_t p;
  uint32_t pinv;
  uint32_t r2;          // R^2 mod p
  uint32_t half;        // (p - 1) / 2
};

__host__ __device__ __forceinline__ uint32_t add_mod(uint32_t a, uint32_t b,
                                                     uint32_t p) {
  uint32_t r = a + b;  // a, b < p < 2^31: no wrap
  return r >= p ? r - p : r;
}

__host__ __device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b,
                                                     uint32_t p) {
  return a >= b ? a - b : a + p - b;
}

#ifdef __CUDACC__
// Shoup: a * w mod p for a < 2^32 and a constant w < p with
// ws = floor(w * 2^32 / p). Result in [0, p).
__device__ __forceinline__ uint32_t shoup_mul(uint32_t a, uint32_t w,
                                              uint32_t ws, uint32_t p) {
  uint32_t q = __umulhi(a, ws);
  uint32_t r = a * w - q * p;  // in [0, 2p)
  return r >= p ? r - p : r;
}

// Signed Montgomery: a * b * 2^-32 mod p for a, b < p. Result in [0, p).
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b,
                                             uint32_t p, uint32_t pinv) {
  uint32_t lo = a * b;
  uint32_t hi = __umulhi(a, b);
  uint32_t m = lo * pinv;
  uint32_t mp = __umulhi(m, p);
  // (a*b - m*p) / 2^32 = hi - mp, exact; in (-p, p).
  int32_t r = static_cast<int32_t>(hi - mp);
  return r < 0 ? static_cast<uint32_t>(r + static_cast<int32_t>(p))
               : static_cast<uint32_t>(r);
}

// min(a, b) of unsigned words: with b = a - k (mod 2^32) it is a - k when
// a >= k and a otherwise (the wrapped difference is the larger), the
// conditional subtraction in two instructions.
__device__ __forceinline__ uint32_t umin32(uint32_t a, uint32_t b) { return min(a, b); }

__device__ __forceinline__ uint32_t reduce_u32(uint32_t x, uint32_t p) {
  // x < 2^32 < 3p for p > 2^31 / 1.5
  if (x >= p) x -= p;
  if (x >= p) x -= p;
  return x;
}

// Shoup without the final correction: a * w mod p in [0, 2p) for any
// 32-bit a and a constant w < p with ws = floor(w * 2^32 / p).
__device__ __forceinline__ uint32_t shoup_mul_lazy(uint32_t a, uint32_t w,
                                                   uint32_t ws, uint32_t p) {
  return a * w - __umulhi(a, ws) * p;
}

__device__ __forceinline__ uint32_t reduce_u64(uint64_t x, uint32_t p) {
  return static_cast<uint32_t>(x % p);
}
#endif

}  // namespace inspire
