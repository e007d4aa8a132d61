// Kernels of a batched PIR client (query generation and response
// decryption) for load generation and end-to-end tests.
//
// Reference: PirClient::CreateRequest / CreateFirstDimensionQuery /
// CreateSecondDimensionQuery / CreatePackingKey / ProcessResponse
// (crypto/pir/client/pir_client.cc:61-272) over GenerateRlweSamples,
// EncryptFromRlweSample, EncryptGadgetCiphertextFromRlweSamples,
// EncryptRgswCiphertextFromRlweSamples and DecryptAfterModulusSwitch
// (crypto/encryption.cc:150-518).
//
// Every RLWE sample is b = e - a s mod q for a public a-component a (the same
// ones the server preprocessed) and the client's ternary key s; a s is an
// exact multi-prime NTT product. The error e is a centred binomial of the
// parameters' variance drawn from a counter-based hash (the SplitMix64
// finaliser) of (seed, client, row, coefficient): reproducible and fast, NOT
// a cryptographic generator; the reference's clients use ChaCha.
#pragma once
#include <cstdint>

#include "ntt.cuh"

namespace inspire {

// SplitMix64 finaliser (Steele, Lea, Flood 2014).
__device__ __forceinline__ uint64_t cl_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Centred binomial of variance var: popcount of 2 var bits minus popcount of
// 2 var further bits.
__device__ __forceinline__ int cl_error(uint64_t seed, uint64_t ctr, int var) {
  const int n = 2 * var;
  int acc = 0, taken = 0, word = 0;
  uint64_t bits = 0;
  int left = 0;
  while (taken < 2 * n) {
    if (left == 0) {
      bits = cl_mix(seed ^ cl_mix((ctr << 6) + word++));
      left = 64;
    }
    const int take = min(left, (taken < n ? n : 2 * n) - taken);
    const uint64_t m = take >= 64 ? ~0ull : ((1ull << take) - 1);
    const int c = __popcll(bits & m);
    acc += taken < n ? c : -c;
    bits = take >= 64 ? 0 : (bits >> take);
    left -= take;
    taken += take;
  }
  return acc;
}

struct ClientArgs {
  int d, log_d, log_q, k_pack, ne, ns;   // ns first-dimension samples
  int t;                                 // interpolation degree
  int64_t fd_len;                        // first-dimension query words
  int pack_log_digit, eval_log_digit;
  int var;
  uint64_t seed;
  uint64_t plaintext_modulus;
  const int8_t* keys;                    // [batch][d] ternary secret keys
  const int64_t* index;                  // [batch]
};

template <typename T>
__device__ __forceinline__ T cl_qmask(int log_q) {
  return log_q >= static_cast<int>(8 * sizeof(T)) ? ~T{0} : ((T{1} << log_q) - 1);
}

// Coefficient j of X^e * s (0 <= e < 2d) for a ternary s, as a word.
template <typename T>
__device__ __forceinline__ T cl_shift_key(const int8_t* s, int d, int e, int j) {
  bool neg = e >= d;
  if (neg) e -= d;
  int i = j - e;
  if (i < 0) {
    i += d;
    neg = !neg;
  }
  const int v = neg ? -s[i] : s[i];
  return static_cast<T>(static_cast<int64_t>(v));
}

// Coefficient j of s(X^p) (Polynomial::Automorph) for odd p: the i with
// i p = j (or j + d, negated) mod 2d; pinv = p^-1 mod 2d.
template <typename T>
__device__ __forceinline__ T cl_aut_key(const int8_t* s, int d, int pinv, int j) {
  const int e = static_cast<int>((static_cast<int64_t>(j) * pinv) % (2 * d));
  const int v = e < d ? s[e] : -s[e - d];
  return static_cast<T>(static_cast<int64_t>(v));
}

// Forward NTTs of the ternary keys: out[b][pi][d]. grid = (r, batch).
template <int ITERS>
__global__ void __launch_bounds__(1024)
cl_key_ntt_kernel(const int8_t* __restrict__ keys, NttCtx c, uint32_t* __restrict__ out) {
  extern __shared__ uint32_t cl_smem[];
  const int d = 1 << c.logd;
  const int pi = blockIdx.x, b = blockIdx.y;
  const uint32_t p = c.p[pi];
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    const int v = keys[static_cast<int64_t>(b) * d + j];
    cl_smem[j] = v >= 0 ? static_cast<uint32_t>(v) : p - static_cast<uint32_t>(-v);
  }
  ntt_forward_t<ITERS>(cl_smem, c, pi);
  uint32_t* o = out + (static_cast<int64_t>(b) * c.r + pi) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) o[j] = cl_smem[j];
}

// a s for one a (T words) and one key transform: leaves the r residue
// vectors of the product in sm (r * d words), read back by cl_crt.
template <typename T, int ITERS>
__device__ __forceinline__ void cl_times_key(const T* a, const uint32_t* s_hat, uint32_t* sm,
                                             const NttCtx& c, int d) {
  for (int pi = 0; pi < c.r; ++pi) {
    uint32_t* x = sm + static_cast<int64_t>(pi) * d;
    const uint32_t p = c.p[pi];
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      if constexpr (sizeof(T) == 4) {
        x[j] = reduce_u32(a[j], p);
      } else {
        x[j] = reduce_u64(a[j], p);
      }
    }
    ntt_forward_t<ITERS>(x, c, pi);
    const uint32_t* sh = s_hat + static_cast<int64_t>(pi) * d;
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      x[j] = mont_mul(x[j], __ldg(sh + j), p, c.pinv[pi]);
    }
    ntt_inverse_t<ITERS>(x, c, pi);
  }
}

template <typename T>
__device__ __forceinline__ T cl_crt(const uint32_t* sm, const NttCtx& c, int d, int j) {
  uint32_t x[kMaxPrimes] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int pi = 0; pi < kMaxPrimes; ++pi) {
    if (pi < c.r) {
      x[pi] = shoup_mul(sm[static_cast<int64_t>(pi) * d + j], c.scale[pi], c.scale_s[pi],
                        c.p[pi]);
    }
  }
  return crt_reconstruct<T>(x, c);
}

// One request row per block: rows [0, ns) are the first-dimension samples
// (Enc(one-hot)), then 2 ne second-dimension gadget rows (u: m s, v: m, the
// monomial X^{(2d/t) col}), then 2 k packing-key rows (gadget encryptions of
// s(X^5) and s(X^{2d-1})). grid = (rows, batch). Outputs:
// fd[b][fd_len], sd[b][2 ne][d], pk[b][2 k][d].
template <typename T, int ITERS>
__global__ void __launch_bounds__(1024)
cl_request_kernel(const T* __restrict__ a_rows, const uint32_t* __restrict__ s_hat,
                  ClientArgs a, NttCtx c, T* __restrict__ fd, T* __restrict__ sd,
                  T* __restrict__ pk) {
  extern __shared__ uint32_t cl_smem[];
  const int d = a.d;
  const int row = blockIdx.x, b = blockIdx.y;
  const int rows = gridDim.x;
  cl_times_key<T, ITERS>(a_rows + static_cast<int64_t>(row) * d,
                         s_hat + static_cast<int64_t>(b) * c.r * d, cl_smem, c, d);
  const T qm = cl_qmask<T>(a.log_q);
  constexpr int kW = 8 * sizeof(T);
  const int8_t* s = a.keys + static_cast<int64_t>(b) * d;
  const int64_t index = a.index[b];
  const int row_index = static_cast<int>(index / a.t);
  const int col_index = static_cast<int>(index % a.t);
  const int shift = (2 * d / a.t) * col_index;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    const T as = cl_crt<T>(cl_smem, c, d, j);
    const uint64_t ctr = (static_cast<uint64_t>(b) * rows + row) * d + j;
    const int e = cl_error(a.seed, ctr, a.var);
    T v = static_cast<T>(static_cast<T>(static_cast<int64_t>(e)) - as) & qm;
    if (row < a.ns) {
      // EncryptFromRlweSample of the one-hot message: + round(m q / p).
      if (row == row_index / d && j == row_index % d) {
        const unsigned __int128 q = static_cast<unsigned __int128>(1) << a.log_q;
        const unsigned __int128 p = a.plaintext_modulus;
        v = static_cast<T>(v + static_cast<T>((q + p / 2) / p)) & qm;
      }
      const int64_t pos = static_cast<int64_t>(row) * d + j;
      if (pos < a.fd_len) fd[static_cast<int64_t>(b) * a.fd_len + pos] = v;
      continue;
    }
    int g = row - a.ns;
    T target;
    int digit, log_digit, nd;
    T* out;
    if (g < 2 * a.ne) {
      nd = a.ne;
      log_digit = a.eval_log_digit;
      digit = g < a.ne ? g : g - a.ne;
      // The monomial: X^shift, or -X^(shift - d) written as q - 1.
      if (g < a.ne) {
        target = cl_shift_key<T>(s, d, shift, j);
      } else {
        const bool neg = shift >= d;
        const int at = neg ? shift - d : shift;
        target = j == at ? (neg ? static_cast<T>(qm) : T{1}) : T{0};
      }
      out = sd + (static_cast<int64_t>(b) * 2 * a.ne + g) * d;
    } else {
      g -= 2 * a.ne;
      nd = a.k_pack;
      log_digit = a.pack_log_digit;
      digit = g < a.k_pack ? g : g - a.k_pack;
      // s(X^5) or s(X^{2d-1}); inverses of 5 and 2d-1 mod 2d.
      int pinv = 2 * d - 1;
      if (g < a.k_pack) {
        // 5^-1 mod 2d by Newton iteration (2d is a power of two).
        uint32_t x = 5;
        for (int it = 0; it < 5; ++it) x *= 2 - 5 * x;
        pinv = static_cast<int>(x & static_cast<uint32_t>(2 * d - 1));
      }
      target = cl_aut_key<T>(s, d, pinv, j);
      out = pk + (static_cast<int64_t>(b) * 2 * a.k_pack + g) * d;
    }
    // EncryptGadgetCiphertextFromRlweSamples: y = b + (target << (i l + off)).
    const int off = max(0, a.log_q - nd * log_digit);
    const int sh = digit * log_digit + off;
    if (sh < kW) v = static_cast<T>(v + static_cast<T>(target << sh)) & qm;
    out[j] = v;
  }
}

// DecryptAfterModulusSwitch per (client, shard): a s mod q1, rescaled to
// q2, + b mod q2, then round(x p / q2) mod p. grid = (l, batch).
template <typename T, int ITERS>
__global__ void __launch_bounds__(1024)
cl_decrypt_kernel(const T* __restrict__ resp, const uint32_t* __restrict__ s_hat, int l,
                  int log_q1, int log_q2, uint64_t plaintext_modulus, NttCtx c,
                  T* __restrict__ out) {
  extern __shared__ uint32_t cl_smem[];
  const int d = 1 << c.logd;
  const int k = blockIdx.x, b = blockIdx.y;
  const T* ct = resp + (static_cast<int64_t>(b) * l + k) * 2 * d;
  cl_times_key<T, ITERS>(ct, s_hat + static_cast<int64_t>(b) * c.r * d, cl_smem, c, d);
  const T m1 = cl_qmask<T>(log_q1), m2 = cl_qmask<T>(log_q2);
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    T as = cl_crt<T>(cl_smem, c, d, j) & m1;
    as = rescale_word<T>(as, log_q1, log_q2);
    const T v = static_cast<T>(ct[d + j] + as) & m2;
    const unsigned __int128 q2 = static_cast<unsigned __int128>(1) << log_q2;
    const unsigned __int128 p = plaintext_modulus;
    out[(static_cast<int64_t>(b) * l + k) * d + j] =
        static_cast<T>(((static_cast<unsigned __int128>(v) * p + q2 / 2) / q2) % p);
  }
}

}  // namespace inspire
