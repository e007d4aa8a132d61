// InnerProductFft for callers that cannot allocate GPU memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// host runtime that owns the device memory budget (a JNI or Go service whose
// allocator is the only one allowed to reserve device memory), code that
// must not allocate on its request path because allocation can block on
// other streams, and code that works from a fixed pre-reserved footprint.
// inspire_inner_product_noalloc serves them: the caller passes device
// buffers for its inputs and output, and the NTT scratch (twiddle tables and
// the transformed operands) lives in one file-scope __device__ array of a
// fixed size, g_noalloc_scratch (1.6 MB, resident on every GPU that loads the
// library until the process exits). Nothing here calls cudaMalloc,
// cudaFree or an allocating library routine.
//
// The computation is the same exact negacyclic inner product as
// inspire_inner_product (Polynomial<T>::InnerProductFft,
// crypto/polynomial_fft.cc:68-197 in the reference), limited to
// n <= kNoAllocMaxPolys polynomials of degree d <= kNoAllocMaxDegree.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/inspire_pir.h"
#include "arith.cuh"
#include "ntt.cuh"
#include "poly_kernels.cuh"

namespace inspire {
namespace {

constexpr int kNoAllocMaxPolys = 8;
constexpr int kNoAllocLogMaxDegree = 12;
constexpr int kNoAllocMaxDegree = 1 << kNoAllocLogMaxDegree;  // 4096
constexpr size_t kTableWords =
    static_cast<size_t>(kMaxPrimes) * 4 * kNoAllocMaxDegree;
constexpr size_t kOperandWords =
    static_cast<size_t>(kNoAllocMaxPolys) * kMaxPrimes * kNoAllocMaxDegree;
constexpr size_t kScratchWords = kTableWords + 2 * kOperandWords;  // 1.6 MB
constexpr int kMaxDevices = 64;

// The shared scratch: [tables | transformed u | transformed v]. Every call
// rewrites every word it later reads (tables for its degree, the d words of
// each (polynomial, prime) transform), so nothing needs clearing between
// calls. Calls that overlap on the GPU share this array and race.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

constexpr uint32_t kNoAllocPrimes[kMaxPrimes] = {
    2147352577u, 2146959361u, 2146041857u, 2145976321u, 2144796673u};

uint64_t pow_mod(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return r;
}

uint32_t generator_of(uint32_t p) {
  uint64_t n = p - 1;
  uint64_t f[16];
  int nf = 0;
  for (uint64_t x = 2; x * x <= n; ++x) {
    if (n % x == 0) {
      f[nf++] = x;
      while (n % x == 0) n /= x;
    }
  }
  if (n > 1) f[nf++] = n;
  for (uint64_t g = 2;; ++g) {
    bool ok = true;
    for (int i = 0; i < nf && ok; ++i) ok = pow_mod(g, (p - 1) / f[i], p) != 1;
    if (ok) return static_cast<uint32_t>(g);
  }
}

uint32_t shoup_of(uint32_t w, uint32_t p) {
  return static_cast<uint32_t>((static_cast<uint64_t>(w) << 32) / p);
}

// Twiddle tables of every prime for degree 2^logd, written into the scratch.
struct RootSet {
  uint32_t p[kMaxPrimes];
  uint32_t psi[kMaxPrimes];
  uint32_t psi_inv[kMaxPrimes];
};

__global__ void noalloc_tables_kernel(uint32_t* __restrict__ tables, int logd,
                                      RootSet roots) {
  const int d = 1 << logd;
  const int pi = blockIdx.y;
  const uint64_t p = roots.p[pi];
  uint32_t* tab = tables + static_cast<size_t>(pi) * 4 * d;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d;
       i += gridDim.x * blockDim.x) {
    int br = 0;
    for (int b = 0; b < logd; ++b) br = (br << 1) | ((i >> b) & 1);
    uint64_t w = 1, iw = 1, base = roots.psi[pi], ibase = roots.psi_inv[pi];
    for (int e = br; e; e >>= 1) {
      if (e & 1) {
        w = w * base % p;
        iw = iw * ibase % p;
      }
      base = base * base % p;
      ibase = ibase * ibase % p;
    }
    tab[i] = static_cast<uint32_t>(w);
    tab[d + i] = static_cast<uint32_t>((w << 32) / p);
    tab[2 * d + i] = static_cast<uint32_t>(iw);
    tab[3 * d + i] = static_cast<uint32_t>((iw << 32) / p);
  }
}

// Forward NTT of u rebuilt from its chunks exactly as the reference's
// InnerProductFft reads it (signed top chunk when asked). grid = n * r.
template <typename T>
__global__ void __launch_bounds__(kPolyThreads)
noalloc_ntt_u_kernel(const T* __restrict__ u, int chunk_bits, int u_chunks,
                     int u_bits, int is_signed, uint32_t* __restrict__ dst,
                     NttCtx c) {
  extern __shared__ uint32_t smem[];
  const int d = 1 << c.logd;
  const int poly = blockIdx.x / c.r;
  const int pi = blockIdx.x % c.r;
  const int64_t p = c.p[pi];
  const T* in = u + static_cast<int64_t>(poly) * d;
  const uint64_t mask = (1ull << chunk_bits) - 1;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    const uint64_t x = static_cast<uint64_t>(in[j]);
    uint64_t acc = 0;
    for (int ch = 0; ch < u_chunks; ++ch) {
      const uint64_t chunk = (x >> (chunk_bits * ch)) & mask;
      int64_t v = static_cast<int64_t>(chunk);
      if (is_signed && ch == u_chunks - 1) {
        const int shift = 64 - (u_bits - chunk_bits * ch);
        v = static_cast<int64_t>(chunk << shift) >> shift;
      }
      acc += static_cast<uint64_t>(v) << (chunk_bits * ch);
    }
    uint32_t r;
    if (is_signed) {
      int64_t s = static_cast<int64_t>(acc) % p;
      r = static_cast<uint32_t>(s < 0 ? s + p : s);
    } else {
      r = static_cast<uint32_t>(acc % static_cast<uint64_t>(p));
    }
    smem[j] = r;
  }
  ntt_forward(smem, c, pi);
  uint32_t* out = dst + (static_cast<int64_t>(poly) * c.r + pi) * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) out[j] = smem[j];
}

// Host-side constants of one degree: the primes' 2d-th roots and the
// NttCtx fields that do not depend on the call (prime count and table
// address are set per call).
struct DegreeConsts {
  RootSet roots;
  NttCtx ctx;
};

// Computed once per degree (at most 13 degrees), so that a call costs only
// its kernel launches; the generators are found once for all degrees.
const DegreeConsts& ConstsFor(int logd) {
  static std::once_flag gen_once;
  static uint32_t generators[kMaxPrimes];
  std::call_once(gen_once, [] {
    for (int i = 0; i < kMaxPrimes; ++i) {
      generators[i] = generator_of(kNoAllocPrimes[i]);
    }
  });
  static std::once_flag once[kNoAllocLogMaxDegree + 1];
  static DegreeConsts table[kNoAllocLogMaxDegree + 1];
  std::call_once(once[logd], [logd] {
    const uint64_t d = 1ull << logd;
    DegreeConsts& k = table[logd];
    NttCtx& c = k.ctx;
    c.logd = logd;
    for (int i = 0; i < kMaxPrimes; ++i) {
      const uint32_t p = kNoAllocPrimes[i];
      const uint64_t psi = pow_mod(generators[i], (p - 1) / (2 * d), p);
      k.roots.p[i] = p;
      k.roots.psi[i] = static_cast<uint32_t>(psi);
      k.roots.psi_inv[i] = static_cast<uint32_t>(pow_mod(psi, p - 2, p));
      c.p[i] = p;
      uint32_t x = p;
      for (int j = 0; j < 5; ++j) x *= 2 - p * x;
      c.pinv[i] = x;
      c.half[i] = (p - 1) / 2;
      const uint64_t r32 = (1ull << 32) % p;
      c.scale[i] = static_cast<uint32_t>(pow_mod(d, p - 2, p) * r32 % p);
      c.scale_s[i] = shoup_of(c.scale[i], p);
      uint64_t prod = 1;
      for (int j = 0; j < i; ++j) prod *= kNoAllocPrimes[j];
      c.pm[i] = prod;
      for (int j = 0; j < kMaxPrimes; ++j) {
        c.garner[j][i] = j == i ? 0
                                : static_cast<uint32_t>(
                                      pow_mod(kNoAllocPrimes[j] % p, p - 2, p) *
                                      r32 % p);
      }
    }
  });
  return table[logd];
}

struct Status {
  int code = INSPIRE_OK;
  std::string msg;
};

Status Fail(int code, std::string msg) { return Status{code, std::move(msg)}; }

// Device address of g_noalloc_scratch for the current device, looked up
// once per device (host code may not use the symbol itself as a pointer).
Status ScratchAddress(uint32_t** out) {
  static std::mutex mu;
  static uint32_t* cached[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return Fail(INSPIRE_INTERNAL, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) {
    return Fail(INSPIRE_INTERNAL, "device ordinal out of range");
  }
  std::lock_guard<std::mutex> lock(mu);
  if (cached[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      return Fail(INSPIRE_INTERNAL,
                  std::string("cudaGetSymbolAddress(scratch): ") +
                      cudaGetErrorString(e));
    }
    cached[dev] = static_cast<uint32_t*>(p);
  }
  *out = cached[dev];
  return Status{};
}

template <typename T>
Status Run(const void* u, const void* v, int n, int d, int logd, int u_bits,
           int chunk_bits, int u_chunks, int v_chunks, int is_signed, int r,
           void* out, cudaStream_t st) {
  uint32_t* scratch = nullptr;
  Status s = ScratchAddress(&scratch);
  if (s.code != INSPIRE_OK) return s;
  uint32_t* tables = scratch;
  uint32_t* U = scratch + kTableWords;
  uint32_t* V = U + kOperandWords;

  const DegreeConsts& k = ConstsFor(logd);
  NttCtx c = k.ctx;
  c.r = r;
  const RootSet roots = k.roots;
  c.tables = tables;

  const int coeff_bits = 8 * static_cast<int>(sizeof(T));
  const int vb = std::min(v_chunks * chunk_bits, coeff_bits);
  const uint64_t vmask = vb >= 64 ? ~0ull : ((1ull << vb) - 1);
  const size_t smem_fin = static_cast<size_t>(r) * d * 4;
  cudaError_t e = cudaFuncSetAttribute(
      inner_product_finish_kernel<T>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_fin));
  if (e != cudaSuccess) return Fail(INSPIRE_INTERNAL, cudaGetErrorString(e));

  noalloc_tables_kernel<<<dim3(8, r), 512, 0, st>>>(tables, logd, roots);
  noalloc_ntt_u_kernel<T><<<n * r, kPolyThreads, d * 4, st>>>(
      static_cast<const T*>(u), chunk_bits, u_chunks, u_bits, is_signed, U, c);
  ntt_coeffs_kernel<T><<<dim3(n * r, 1), kPolyThreads, d * 4, st>>>(
      static_cast<const T*>(v), 0, 0, n, static_cast<T>(vmask), V, d, c);
  inner_product_finish_kernel<T><<<1, kPolyThreads, smem_fin, st>>>(
      U, V, n, static_cast<T*>(out), c);
  e = cudaGetLastError();
  if (e != cudaSuccess) return Fail(INSPIRE_INTERNAL, cudaGetErrorString(e));
  return Status{};
}

}  // namespace
}  // namespace inspire

extern "C" int inspire_inner_product_noalloc(
    int32_t coeff_bits, const void* u, const void* v, int32_t n, int32_t d,
    int32_t u_bits, int32_t v_bits, int32_t chunk_bits, int32_t u_is_signed,
    void* out, void* stream, char* err, size_t err_len) {
  using namespace inspire;
  auto report = [&](const Status& s) {
    if (err != nullptr && err_len > 0) {
      std::snprintf(err, err_len, "%s", s.msg.c_str());
    }
    return s.code;
  };
  if (coeff_bits != 32 && coeff_bits != 64) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT, "coeff_bits must be 32 or 64."));
  }
  if (n <= 0) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT,
                       "Polynomial vectors cannot be empty."));
  }
  int logd = 0;
  while (logd < 31 && (1 << logd) < d) ++logd;
  if (d < 2 || (1 << logd) != d) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT,
                       "Polynomial lengths or context mismatch."));
  }
  if (n > kNoAllocMaxPolys || d > kNoAllocMaxDegree) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT,
                       "inspire_inner_product_noalloc supports at most 8 "
                       "polynomials of degree at most 4096 (its scratch is a "
                       "fixed 1.6 MB device array)."));
  }
  if (u_bits <= 0 || v_bits <= 0 || chunk_bits <= 0 || chunk_bits > 63) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT, "Invalid bits or chunk_bits."));
  }
  if (std::log2(n) + std::log2(d) + 2.0 * chunk_bits > 53.0) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT,
                       "Potential precision overflow in accumulation."));
  }
  // The reference's chunk rule (crypto/polynomial_fft.cc:98-107).
  const int max_chunks = (coeff_bits + chunk_bits - 1) / chunk_bits;
  const int uc = std::min((u_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  const int vc = std::min((v_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  // Primes for the exact range of |sum| (signed centred CRT).
  const double bound = std::min(uc * chunk_bits, 64) +
                       std::min(vc * chunk_bits, coeff_bits) +
                       std::log2(static_cast<double>(n) * d);
  int r = 0;
  for (int k = 1; k <= kMaxPrimes && r == 0; ++k) {
    double have = std::log2((kNoAllocPrimes[k - 1] - 1) / 2.0);
    for (int j = 0; j < k - 1; ++j) have += std::log2(kNoAllocPrimes[j]);
    if (bound < have - 0.01) r = std::max(k, 2);
  }
  if (r == 0) {
    return report(Fail(INSPIRE_INVALID_ARGUMENT,
                       "Negacyclic product exceeds the supported exact range."));
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  Status s = coeff_bits == 32
                 ? Run<uint32_t>(u, v, n, d, logd, u_bits, chunk_bits, uc, vc,
                                 u_is_signed, r, out, st)
                 : Run<uint64_t>(u, v, n, d, logd, u_bits, chunk_bits, uc, vc,
                                 u_is_signed, r, out, st);
  return report(s);
}
