// The PirServer drop-in: server material resident in GPU memory and the
// C ABI declared in include/inspire_pir.h.
//
// Reference: PirServer<Db,Coeff,Mat>::{Create,ProcessResponse,EvalPoly}
// (crypto/pir/server/pir_server.cc:54-306). The online answer is
//   1. b' + b_agg_partial = DB * q1 + P * y_g  (fused GEMV or limb GEMM)
//   2. FinalizeMatrixPack per (shard, slice)   (exact NTT inner products)
//   3. EvalPoly: t-1 external products per shard (exact NTTs)
//   4. Rescale a to q1 and b to q2.
// Every integer result is the exact value the reference's FP64 FFT rounds to
// whenever that rounding is exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/inspire_pir.h"
#include "arith.cuh"
#include "internal.h"
#include "limb_gemm.h"
#include "ntt.cuh"
#include "poly_kernels.cuh"
#include "preprocess_kernels.cuh"
#include "client_kernels.cuh"
#include "server_api.h"

namespace inspire {
namespace {

// ---------------------------------------------------------------------------
// Status plumbing.
// ---------------------------------------------------------------------------
struct Status {
  int code = INSPIRE_OK;
  std::string msg;
  bool ok() const { return code == INSPIRE_OK; }
};

Status Err(int code, std::string msg) { return Status{code, std::move(msg)}; }

int Report(const Status& s, char* err, size_t err_len) {
  if (err != nullptr && err_len > 0) {
    std::snprintf(err, err_len, "%s", s.ok() ? "" : s.msg.c_str());
  }
  return s.code;
}

Status Cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status{};
  return Err(INSPIRE_INTERNAL,
             std::string(what) + ": " + cudaGetErrorString(e));
}

#define RETURN_IF_ERROR(expr)     \
  do {                            \
    Status _s = (expr);           \
    if (!_s.ok()) return _s;      \
  } while (0)

// ---------------------------------------------------------------------------
// Primes and NTT tables.
// ---------------------------------------------------------------------------
constexpr uint32_t kPrimes[kMaxPrimes] = {2147352577u, 2146959361u,
                                          2146041857u, 2145976321u,
                                          2144796673u};

uint64_t PowMod(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return r;
}

uint32_t Generator(uint32_t p) {
  std::vector<uint64_t> factors;
  uint64_t n = p - 1;
  for (uint64_t f = 2; f * f <= n; ++f) {
    if (n % f == 0) {
      factors.push_back(f);
      while (n % f == 0) n /= f;
    }
  }
  if (n > 1) factors.push_back(n);
  for (uint64_t g = 2;; ++g) {
    bool ok = true;
    for (uint64_t f : factors) {
      if (PowMod(g, (p - 1) / f, p) == 1) {
        ok = false;
        break;
      }
    }
    if (ok) return static_cast<uint32_t>(g);
  }
}

uint32_t InvMod2_32(uint32_t p) {  // p odd
  uint32_t x = p;  // correct to 3 bits
  for (int i = 0; i < 5; ++i) x *= 2 - p * x;
  return x;
}

uint32_t Shoup(uint32_t w, uint32_t p) {
  return static_cast<uint32_t>((static_cast<uint64_t>(w) << 32) / p);
}

int BitRev(int x, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r = (r << 1) | ((x >> b) & 1);
  return r;
}

// One prime's tables [W | W shoup | IW | IW shoup] in the window order of
// the radix-16 transforms.
template <int LOGD>
void Permute16(const uint32_t* tab, uint32_t* t16) {
  using N = Ntt16<LOGD>;
  for (int w = 0; w < N::kPasses; ++w) {
    const int m0 = 1 << N::Start(w);
    for (int st = N::Skip(w); st < 4; ++st) {
      for (int x = 0; x < (1 << st); ++x) {
        for (int g = 0; g < m0; ++g) {
          const int slot = N::Slot(w, st, x, g);
          const int idx = (m0 << st) + (g << st) + x;
          for (int part = 0; part < 4; ++part) {
            t16[part * N::kD + slot] = tab[part * N::kD + idx];
          }
        }
      }
    }
  }
}

// Device tables for one ring degree, all primes.
class NttTables {
 public:
  static Status Create(int logd, std::unique_ptr<NttTables>* out) {
    if (logd < 1 || logd > kLogMaxDegree) {
      return Err(INSPIRE_INVALID_ARGUMENT, "Invalid log_d.");
    }
    std::unique_ptr<NttTables> t(new NttTables());
    t->logd_ = logd;
    const int d = 1 << logd;
    std::vector<uint32_t> host(static_cast<size_t>(kMaxPrimes) * 4 * d);
    for (int pi = 0; pi < kMaxPrimes; ++pi) {
      const uint32_t p = kPrimes[pi];
      const uint64_t psi = PowMod(Generator(p), (p - 1) / (2ull * d), p);
      const uint64_t psi_inv = PowMod(psi, p - 2, p);
      if (PowMod(psi, d, p) != p - 1) {
        return Err(INSPIRE_INTERNAL, "NTT root of unity check failed.");
      }
      uint32_t* tab = host.data() + static_cast<size_t>(pi) * 4 * d;
      for (int i = 0; i < d; ++i) {
        const int br = BitRev(i, logd);
        const uint32_t w = static_cast<uint32_t>(PowMod(psi, br, p));
        const uint32_t iw = static_cast<uint32_t>(PowMod(psi_inv, br, p));
        tab[i] = w;
        tab[d + i] = Shoup(w, p);
        tab[2 * d + i] = iw;
        tab[3 * d + i] = Shoup(iw, p);
      }
    }
    if (logd >= kNtt16MinLogD && logd <= kNtt16MaxLogD) {
      // The radix-16 order of ntt16.cuh, appended after the plain tables:
      // W[m0 2^s + g 2^s + x] of window w at Ntt16<logd>::Slot(w, s, x, g).
      const size_t plain = host.size();
      host.resize(2 * plain, 0);
      for (int pi = 0; pi < kMaxPrimes; ++pi) {
        const uint32_t* tab = host.data() + static_cast<size_t>(pi) * 4 * d;
        uint32_t* t16 = host.data() + plain + static_cast<size_t>(pi) * 4 * d;
        if (logd == 11) {
          Permute16<11>(tab, t16);
        } else if (logd == 12) {
          Permute16<12>(tab, t16);
        } else {
          Permute16<13>(tab, t16);
        }
      }
      t->has16_ = true;
    }
    RETURN_IF_ERROR(Cuda(cudaMalloc(&t->dev_, host.size() * 4), "cudaMalloc"));
    RETURN_IF_ERROR(Cuda(cudaMemcpy(t->dev_, host.data(), host.size() * 4,
                                    cudaMemcpyHostToDevice),
                         "cudaMemcpy"));
    *out = std::move(t);
    return Status{};
  }
  ~NttTables() {
    if (dev_) cudaFree(dev_);
  }

  NttCtx Ctx(int r) const {
    NttCtx c{};
    c.logd = logd_;
    c.r = r;
    const uint64_t d = 1ull << logd_;
    for (int i = 0; i < kMaxPrimes; ++i) {
      const uint32_t p = kPrimes[i];
      c.p[i] = p;
      c.pinv[i] = InvMod2_32(p);
      c.half[i] = (p - 1) / 2;
      const uint64_t dinv = PowMod(d, p - 2, p);
      const uint64_t r32 = (1ull << 32) % p;
      c.scale[i] = static_cast<uint32_t>(dinv * r32 % p);
      c.scale_s[i] = Shoup(c.scale[i], p);
      uint64_t prod = 1;
      for (int j = 0; j < i; ++j) prod *= kPrimes[j];
      c.pm[i] = prod;
      for (int j = 0; j < kMaxPrimes; ++j) {
        const uint64_t inv = PowMod(kPrimes[j] % p, p - 2, p);
        c.garner[j][i] = j == i ? 0 : static_cast<uint32_t>(inv * r32 % p);
      }
    }
    c.tables = dev_;
    c.tables16 = has16_ ? dev_ + static_cast<size_t>(kMaxPrimes) * 4 * d : nullptr;
    return c;
  }

 private:
  NttTables() = default;
  int logd_ = 0;
  bool has16_ = false;
  uint32_t* dev_ = nullptr;
};

// Smallest number of primes whose signed CRT range holds |x| < 2^bits.
Status PrimesFor(double bits, int* r) {
  for (int n = 1; n <= kMaxPrimes; ++n) {
    double have = std::log2((kPrimes[n - 1] - 1) / 2.0);
    for (int j = 0; j < n - 1; ++j) have += std::log2(kPrimes[j]);
    if (bits < have - 0.01) {
      *r = std::max(n, 2);
      return Status{};
    }
  }
  return Err(INSPIRE_INVALID_ARGUMENT,
             "Negacyclic product exceeds the supported exact range.");
}

// ---------------------------------------------------------------------------
// The reference's InnerProductFft chunk rule (polynomial_fft.cc:90-107) and
// the chunk size its callers pick (lwes_to_rlwe.cc:60-74,
// external_product.cc:100-102).
// ---------------------------------------------------------------------------
struct ChunkRule {
  int chunk_bits = 0;
  int u_chunks = 0;
  int v_chunks = 0;
};

int ChunkFor(int num_polys, int d) {
  const int max_allowed =
      static_cast<int>((53.0 - std::log2(num_polys) - std::log2(d)) / 2.0);
  return std::min(20, max_allowed);
}

Status MakeRule(int coeff_bits, int n, int d, int u_bits, int v_bits,
                int chunk_bits, ChunkRule* rule) {
  if (u_bits <= 0 || v_bits <= 0 || chunk_bits <= 0 || chunk_bits > 63) {
    return Err(INSPIRE_INVALID_ARGUMENT, "Invalid bits or chunk_bits.");
  }
  if (std::log2(n) + std::log2(d) + 2.0 * chunk_bits > 53.0) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "Potential precision overflow in accumulation.");
  }
  const int max_chunks = (coeff_bits + chunk_bits - 1) / chunk_bits;
  rule->chunk_bits = chunk_bits;
  rule->u_chunks = std::min((u_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  rule->v_chunks = std::min((v_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  return Status{};
}

uint64_t MaskBits(int bits, int coeff_bits) {
  const int b = std::min(bits, coeff_bits);
  return b >= 64 ? ~0ull : ((1ull << b) - 1);
}

// u rebuilt from its chunks, as the FFT path reads it (with the signed top
// chunk), as a two's complement 64-bit value.
int64_t RebuildU(uint64_t x, const ChunkRule& r, int u_bits, bool is_signed) {
  const uint64_t mask = (1ull << r.chunk_bits) - 1;
  uint64_t acc = 0;
  for (int c = 0; c < r.u_chunks; ++c) {
    const uint64_t chunk = (x >> (r.chunk_bits * c)) & mask;
    int64_t v = static_cast<int64_t>(chunk);
    if (is_signed && c == r.u_chunks - 1) {
      const int bits_in_chunk = u_bits - r.chunk_bits * c;
      const int shift = 64 - bits_in_chunk;
      v = static_cast<int64_t>(chunk << shift) >> shift;
    }
    acc += static_cast<uint64_t>(v) << (r.chunk_bits * c);
  }
  return static_cast<int64_t>(acc);
}

double BoundBits(int n, int d, double u_bits, double v_bits) {
  return u_bits + v_bits + std::log2(static_cast<double>(n) * d);
}

size_t Words(int coeff_bits) { return coeff_bits / 8; }

// ---------------------------------------------------------------------------
// RAII device buffer.
// ---------------------------------------------------------------------------
class DevBuf {
 public:
  DevBuf() = default;
  ~DevBuf() { Free(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  Status Alloc(size_t bytes) {
    Free();
    if (bytes == 0) return Status{};
    cudaError_t e = cudaMalloc(&ptr_, bytes);
    if (e != cudaSuccess) {
      ptr_ = nullptr;
      return Err(INSPIRE_RESOURCE_EXHAUSTED,
                 std::string("GPU allocation of ") + std::to_string(bytes) +
                     " bytes failed: " + cudaGetErrorString(e));
    }
    bytes_ = bytes;
    return Status{};
  }
  Status Upload(const void* host, size_t bytes) {
    RETURN_IF_ERROR(Alloc(bytes));
    if (bytes == 0) return Status{};
    return Cuda(cudaMemcpy(ptr_, host, bytes, cudaMemcpyHostToDevice),
                "cudaMemcpy H2D");
  }
  void Free() {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
  }
  // Moves another buffer's allocation into this one.
  void Take(DevBuf* other) {
    Free();
    ptr_ = other->ptr_;
    bytes_ = other->bytes_;
    other->ptr_ = nullptr;
    other->bytes_ = 0;
  }
  template <typename P = void>
  P* get() const {
    return static_cast<P*>(ptr_);
  }
  size_t bytes() const { return bytes_; }

 private:
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

template <typename K>
Status SetSmem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return Status{};
  return Cuda(cudaFuncSetAttribute(kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(bytes)),
              "cudaFuncSetAttribute");
}

}  // namespace
}  // namespace inspire

// ---------------------------------------------------------------------------
// The server object and its per-batch workspaces.
// ---------------------------------------------------------------------------
namespace inspire {

// Everything one in-flight batch needs: device buffers, the tensor engine's
// request byte planes, a stream, timing events and pinned host staging. A
// server answers synchronous calls with its own workspace; callers that want
// several batches in flight (the serving loop) create more.
struct Workspace {
  int cap = 0;
  DevBuf q1, pkey, sdim, gemv, yh, rgswb, packed, resid0, resid1, resp;
  DevBuf rgswa;  // per-request RGSW a-parts (batched ExternalProduct only)
  std::unique_ptr<LimbScratch> limb;
  cudaStream_t stream = nullptr;
  // Second stream for the host-buffer call: the copy of the second
  // dimension (read only by the polynomial stage) overlaps the products.
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_go = nullptr, sdim_ready = nullptr;
  // The answer forks the request polynomials' transforms onto copy_stream
  // (fork) and joins them back before the polynomial stage (side_done).
  cudaEvent_t fork = nullptr, side_done = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t done = nullptr;
  void* host[4] = {nullptr, nullptr, nullptr, nullptr};  // fd, sd, pk, resp
  int pending_engine = -1;
  ~Workspace() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (done) cudaEventDestroy(done);
    if (copy_go) cudaEventDestroy(copy_go);
    if (sdim_ready) cudaEventDestroy(sdim_ready);
    if (fork) cudaEventDestroy(fork);
    if (side_done) cudaEventDestroy(side_done);
    if (stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    for (auto& h : host)
      if (h) cudaFreeHost(h);
  }
};

}  // namespace inspire

struct inspire_pir_server {
  inspire_pir_params prm{};
  int d = 0, t = 0, l = 0, k = 0, ne = 0;
  int64_t rows = 0, db_cols = 0, pack_cols = 0;
  int interpolated_rows = 0;
  inspire::Status deferred;  // error the reference reports per request
  inspire::Status eval_rule;  // chunk rule of the eval-gadget inner product
  int sms = 152;               // streaming multiprocessors of the device
  std::vector<uint8_t> t_vec_h_raw, second_dim_a_raw;  // host copies
  // SaveToFile header fields (from the loaded image, or the defaults the
  // reference's Preprocess produces: a condensed DB for u64 coefficients).
  bool db_condensed = false, pack_condensed = false;
  int32_t db_orig_cols = 0, pack_bits = 0;
  bool orig_from_file = false;  // db_orig_cols read from an image or proto

  inspire::DevBuf db, pack, a_tilde, th_ntt, rgswa_ntt;
  std::unique_ptr<inspire::NttTables> tables;
  inspire::NttCtx ctx_f{}, ctx_e{};
  uint64_t vmask_f = 0, vmask_e = 0, umask_e = 0;
  std::unique_ptr<inspire::LimbGemm> limb;

  std::unique_ptr<inspire::Workspace> ws0;  // for the synchronous calls
  std::mutex mu;                           // guards ws0 and the timers
  double t_db = 0, t_pack = 0, t_eval = 0;
  // INSPIRE_ENGINE_AUTO: batches of at least `crossover` requests go to the
  // tensor engine (set by inspire_pir_tune_engines; until then a default).
  std::atomic<int32_t> crossover{-1};
  // The last engine tuning: per tested batch size the plain and tensor
  // product times and the tensor engine's chosen form and split-K factor.
  struct TuneRow {
    int32_t batch, form, split;
    float plain_ms, tensor_ms;
  };
  std::vector<TuneRow> tune_table;
};

struct inspire_graph {
  cudaGraphExec_t exec = nullptr;
};

struct inspire_pir_workspace {
  inspire_pir_server* server = nullptr;
  inspire::Workspace ws;
};

namespace inspire {
namespace {

// d/16 coefficients per thread at most (kMaxPer), smaller CTAs otherwise so
// that batches fill the SMs without a wave tail.
inline int PolyThreads(int d) { return d <= 16 * 256 ? 256 : kPolyThreads; }

// Block shape of an NTT kernel launch of `ctas` blocks. Throughput shape
// while the launch has at least one block per SM: d/16 threads for
// 512 <= d <= 4096 (16 coefficients each, three blocks per SM), 1024 threads
// for d = 8192. Latency shape for smaller launches: d/4 threads (up to 1024),
// which shortens the chain of the few blocks of a small batch. iters = quads
// per thread per NTT double stage (0: the generic loops).
struct PolyLaunch {
  int nt;
  int iters;
};
PolyLaunch PolyShapeFor(int d, int64_t ctas, int sms) {
  int nt;
  if (ctas < sms) {
    nt = std::min(1024, std::max(1, d / 4));
  } else if (d >= 512 && d <= 4096) {
    nt = d / 16;
  } else if (d == 8192) {
    nt = 1024;
  } else {
    nt = PolyThreads(d);
  }
  const int q = d / 4;
  const int it = q % nt == 0 ? q / nt : 0;
  if (it == 1 || it == 2 || it == 4) return PolyLaunch{nt, it};
  return PolyLaunch{PolyThreads(d), 0};
}

// Runs the statement with constexpr int LG = log2(d) for the ring degrees of
// the radix-16 transforms (ntt16.cuh).
#define INSPIRE_NTT16_DISPATCH(logd, ...) \
  switch (logd) {                         \
    case 11: {                            \
      constexpr int LG = 11;              \
      __VA_ARGS__;                        \
    } break;                              \
    case 12: {                            \
      constexpr int LG = 12;              \
      __VA_ARGS__;                        \
    } break;                              \
    default: {                            \
      constexpr int LG = 13;              \
      __VA_ARGS__;                        \
    } break;                              \
  }

// The same for the two-group kernels (d / 8 threads), d <= 4096.
#define INSPIRE_NTT16_PAIR_DISPATCH(logd, ...) \
  switch (logd) {                              \
    case 11: {                                 \
      constexpr int LG = 11;                   \
      __VA_ARGS__;                             \
    } break;                                   \
    default: {                                 \
      constexpr int LG = 12;                   \
      __VA_ARGS__;                             \
    } break;                                   \
  }

#define INSPIRE_ITERS_DISPATCH(iters, ...)  \
  switch (iters) {                          \
    case 1: {                               \
      constexpr int IT = 1;                 \
      __VA_ARGS__;                          \
    } break;                                \
    case 2: {                               \
      constexpr int IT = 2;                 \
      __VA_ARGS__;                          \
    } break;                                \
    case 4: {                               \
      constexpr int IT = 4;                 \
      __VA_ARGS__;                          \
    } break;                                \
    default: {                              \
      constexpr int IT = 0;                 \
      __VA_ARGS__;                          \
    } break;                                \
  }

// Forward NTTs of npoly CoeffType polynomials per request (stride
// poly_stride words, masked), batch requests src_qstride words apart.
template <typename T>
Status NttCoeffs(const inspire_pir_server* s, const T* src, int64_t src_qstride,
                 int64_t src_off, int npoly, T mask, uint32_t* dst,
                 int64_t poly_stride, const NttCtx& c, int batch, cudaStream_t st) {
  const int d = s->d;
  if (c.tables16 != nullptr && static_cast<int64_t>(npoly) * batch >= s->sms) {
    INSPIRE_NTT16_DISPATCH(
        c.logd, ntt_coeffs16_kernel<T, LG><<<dim3(npoly, batch), Ntt16<LG>::kThreads, 0, st>>>(
                    src, src_qstride, src_off, npoly, mask, dst, poly_stride, c));
    return Cuda(cudaGetLastError(), "forward NTT");
  }
  const PolyLaunch pl = PolyShapeFor(d, static_cast<int64_t>(npoly) * c.r * batch, s->sms);
  dim3 grid(npoly * c.r, batch);
  INSPIRE_ITERS_DISPATCH(pl.iters, ntt_coeffs_kernel<T, IT><<<grid, pl.nt, d * 4, st>>>(
                                       src, src_qstride, src_off, npoly, mask, dst,
                                       poly_stride, c));
  return Cuda(cudaGetLastError(), "forward NTT");
}

// Shared memory of ext_step16_pair_kernel with NGR transform groups: a
// 2 d-word region per group plus the state.
template <typename T, int LG, int NGR>
constexpr size_t PairExtSmem() {
  return static_cast<size_t>(NGR) * 2 * Ntt16<LG>::kD * 4 + 2ull * Ntt16<LG>::kD * sizeof(T);
}

// Launches ext_step16_pair_kernel with NGR groups: four at d = 2048 when the
// launch has fewer blocks than SMs (each Horner step then waits on one
// transform per group instead of two), else two.
template <typename T, int LG, typename... A>
Status LaunchPairExt(int64_t blocks, int sms, dim3 grid, cudaStream_t st, A... args) {
  if (LG == 11 && blocks < sms) {
    constexpr int NGR = LG == 11 ? 4 : 2;
    const size_t smem = PairExtSmem<T, LG, NGR>();
    RETURN_IF_ERROR(SetSmem(ext_step16_pair_kernel<T, LG, NGR>, smem));
    ext_step16_pair_kernel<T, LG, NGR><<<grid, NGR * Ntt16<LG>::kThreads, smem, st>>>(args...);
  } else {
    const size_t smem = PairExtSmem<T, LG, 2>();
    RETURN_IF_ERROR(SetSmem(ext_step16_pair_kernel<T, LG, 2>, smem));
    ext_step16_pair_kernel<T, LG, 2><<<grid, 2 * Ntt16<LG>::kThreads, smem, st>>>(args...);
  }
  return Cuda(cudaGetLastError(), "external product");
}

// Launches finalize16_pair_kernel with three transform groups at d = 2048
// when there are three primes or more (each group inverts one of the first
// three primes; at most 114 KB of shared memory), else with two groups,
// which take the primes in turns.
template <typename T, int LG>
Status LaunchPairFinalize(const NttCtx& c, dim3 grid, cudaStream_t st, const uint32_t* th,
                          const uint32_t* yh, int k, const T* gemv, int64_t rows,
                          T* packed, int log_q) {
  constexpr int d = Ntt16<LG>::kD;
  if constexpr (LG <= 11) {
    if (c.r >= 3) {
      const size_t smem = static_cast<size_t>(9 + c.r) * d * 4;
      RETURN_IF_ERROR(SetSmem(finalize16_pair_kernel<T, LG, 3>, smem));
      finalize16_pair_kernel<T, LG, 3><<<grid, 3 * Ntt16<LG>::kThreads, smem, st>>>(
          th, yh, k, gemv, nullptr, rows, packed, log_q, c);
      return Cuda(cudaGetLastError(), "finalize");
    }
  }
  const size_t smem = static_cast<size_t>(6 + c.r) * d * 4;
  RETURN_IF_ERROR(SetSmem(finalize16_pair_kernel<T, LG, 2>, smem));
  finalize16_pair_kernel<T, LG, 2><<<grid, 2 * Ntt16<LG>::kThreads, smem, st>>>(
      th, yh, k, gemv, nullptr, rows, packed, log_q, c);
  return Cuda(cudaGetLastError(), "finalize");
}

// Blocks (one per shard and request) from which the external product takes
// one block per request over all primes rather than one per prime: a block
// per SM at d >= 4096; at d = 2048 (128-thread blocks) two per SM, below
// which the per-prime blocks keep more warps busy.
inline int64_t Ext16Min(const inspire_pir_server* s, int d) {
  return static_cast<int64_t>(s->sms) * std::max(1, 4096 / d);
}

// FinalizeMatrixPack for every shard of every request of a batch
// (lwes_to_rlwe.cc:448-479): w->packed[q][shard] = b_agg.
// y_h = packing_key[k..2k): forward NTT over the finalize primes.
template <typename T>
Status YhTransform(inspire_pir_server* s, Workspace* w, int batch, const T* pkey,
                   cudaStream_t st) {
  const int d = s->d, k = s->k;
  return NttCoeffs<T>(s, pkey, static_cast<int64_t>(2 * k) * d,
                      static_cast<int64_t>(k) * d, k, static_cast<T>(s->vmask_f),
                      w->yh.get<uint32_t>(), d, s->ctx_f, batch, st);
}

// The RGSW b parts of the second dimension: forward NTT over the eval
// primes.
template <typename T>
Status RgswTransform(inspire_pir_server* s, Workspace* w, int batch, const T* sdim,
                     cudaStream_t st) {
  const int d = s->d, ne = s->ne;
  return NttCoeffs<T>(s, sdim, static_cast<int64_t>(2 * ne) * d, 0, 2 * ne,
                      static_cast<T>(s->vmask_e), w->rgswb.get<uint32_t>(), d, s->ctx_e,
                      batch, st);
}

// yh_done: the y_h transform is already in w->yh (enqueued on another
// stream that `st` has joined).
template <typename T>
Status FinalizeStage(inspire_pir_server* s, Workspace* w, int batch,
                     const T* pkey, const T* gemv, cudaStream_t st,
                     bool yh_done = false) {
  const int d = s->d, t = s->t, l = s->l, k = s->k;
  const int log_q = s->prm.log_modulus;
  if (!yh_done) RETURN_IF_ERROR(YhTransform<T>(s, w, batch, pkey, st));
  if (s->ctx_f.tables16 != nullptr && static_cast<int64_t>(l) * t * batch >= s->sms) {
    const NttCtx& c = s->ctx_f;
    const size_t smem = static_cast<size_t>(c.r + 1) * d * 4;
    INSPIRE_NTT16_DISPATCH(
        c.logd, RETURN_IF_ERROR(SetSmem(finalize16_kernel<T, LG>, smem));
        finalize16_kernel<T, LG><<<dim3(l * t, batch), Ntt16<LG>::kThreads, smem, st>>>(
            s->th_ntt.get<uint32_t>(), w->yh.get<uint32_t>(), k, gemv, nullptr, s->rows,
            w->packed.get<T>(), log_q, c));
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "finalize"));
  } else if (s->ctx_f.tables16 != nullptr && d <= 4096) {
    // Several transform groups per block.
    const NttCtx& c = s->ctx_f;
    INSPIRE_NTT16_PAIR_DISPATCH(
        c.logd, RETURN_IF_ERROR((LaunchPairFinalize<T, LG>(
                    c, dim3(l * t, batch), st, s->th_ntt.get<uint32_t>(),
                    w->yh.get<uint32_t>(), k, gemv, s->rows, w->packed.get<T>(), log_q))));
  } else {
    const NttCtx& c = s->ctx_f;
    const size_t smem = static_cast<size_t>(c.r) * d * 4;
    const PolyLaunch pl = PolyShapeFor(d, static_cast<int64_t>(l) * t * batch, s->sms);
    dim3 grid(l * t, batch);
    INSPIRE_ITERS_DISPATCH(
        pl.iters, RETURN_IF_ERROR(SetSmem(finalize_kernel<T, IT>, smem));
        finalize_kernel<T, IT><<<grid, pl.nt, smem, st>>>(
            s->th_ntt.get<uint32_t>(), w->yh.get<uint32_t>(), k, gemv, nullptr, s->rows,
            w->packed.get<T>(), log_q, c));
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "finalize"));
  }
  return Status{};
}

// transforms_done: YhTransform and RgswTransform are already enqueued on a
// stream that `st` has joined.
template <typename T>
Status RunPolyStage(inspire_pir_server* s, Workspace* w, int batch,
                    const T* pkey, const T* sdim, const T* gemv, T* resp,
                    cudaStream_t st, bool timed, bool transforms_done = false) {
  const int d = s->d, t = s->t, l = s->l, ne = s->ne;
  const int log_q = s->prm.log_modulus;
  const int nt = PolyThreads(d);
  RETURN_IF_ERROR(FinalizeStage<T>(s, w, batch, pkey, gemv, st, transforms_done));
  if (timed) cudaEventRecord(w->ev[2], st);
  const T* a_tilde = s->a_tilde.get<T>();
  const T* packed = w->packed.get<T>();
  const int64_t a_stride = static_cast<int64_t>(t) * d;        // per shard
  const int64_t b_qstride = static_cast<int64_t>(l) * t * d;   // per request
  uint32_t* resid[2] = {w->resid0.get<uint32_t>(), w->resid1.get<uint32_t>()};
  if (t > 1) {
    const NttCtx& c = s->ctx_e;
    if (!transforms_done) RETURN_IF_ERROR(RgswTransform<T>(s, w, batch, sdim, st));
    ExtArgs e{log_q, s->prm.eval_log_digit, ne,
              LiveDigits(log_q, s->prm.eval_log_digit, ne), s->umask_e};
    const size_t smem = static_cast<size_t>(d) * 4 + 2ull * d * sizeof(T);
    if (c.tables16 != nullptr && static_cast<int64_t>(l) * batch >= Ext16Min(s, d)) {
      // Enough requests to fill the GPU with one block per (shard, request).
      INSPIRE_NTT16_DISPATCH(
          c.logd, RETURN_IF_ERROR(SetSmem(ext_step16_kernel<T, LG>, smem));
          for (int i = t - 2; i >= 0; --i) {
            const bool first = i == t - 2;
            ext_step16_kernel<T, LG><<<dim3(l, batch), Ntt16<LG>::kThreads, smem, st>>>(
                first, first ? nullptr : resid[(i + 1) & 1], resid[i & 1],
                a_tilde + static_cast<int64_t>(i + 1) * d, 0, a_stride,
                packed + static_cast<int64_t>(i + 1) * d, b_qstride, a_stride,
                s->rgswa_ntt.get<uint32_t>(), 0, w->rgswb.get<uint32_t>(), e, c);
            RETURN_IF_ERROR(Cuda(cudaGetLastError(), "external product"));
          });
    } else if (c.tables16 != nullptr && d <= 4096) {
      // Few requests: one block per prime, transforms side by side.
      const int64_t blocks = static_cast<int64_t>(c.r) * l * batch;
      INSPIRE_NTT16_PAIR_DISPATCH(
          c.logd, for (int i = t - 2; i >= 0; --i) {
            const bool first = i == t - 2;
            RETURN_IF_ERROR((LaunchPairExt<T, LG>(
                blocks, s->sms, dim3(c.r, l, batch), st, first,
                first ? nullptr : static_cast<const uint32_t*>(resid[(i + 1) & 1]),
                resid[i & 1], a_tilde + static_cast<int64_t>(i + 1) * d, int64_t{0}, a_stride,
                packed + static_cast<int64_t>(i + 1) * d, b_qstride, a_stride,
                static_cast<const uint32_t*>(s->rgswa_ntt.get<uint32_t>()), int64_t{0},
                static_cast<const uint32_t*>(w->rgswb.get<uint32_t>()), e, c)));
          });
    } else {
      const PolyLaunch pl = PolyShapeFor(d, static_cast<int64_t>(c.r) * l * batch, s->sms);
      dim3 grid(c.r, l, batch);
      INSPIRE_ITERS_DISPATCH(
          pl.iters, RETURN_IF_ERROR(SetSmem(ext_step_kernel<T, IT>, smem));
          for (int i = t - 2; i >= 0; --i) {
            const bool first = i == t - 2;
            ext_step_kernel<T, IT><<<grid, pl.nt, smem, st>>>(
                first, first ? nullptr : resid[(i + 1) & 1], resid[i & 1],
                a_tilde + static_cast<int64_t>(i + 1) * d, 0, a_stride,
                packed + static_cast<int64_t>(i + 1) * d, b_qstride, a_stride,
                s->rgswa_ntt.get<uint32_t>(), 0, w->rgswb.get<uint32_t>(), e, c);
            RETURN_IF_ERROR(Cuda(cudaGetLastError(), "external product"));
          });
    }
  }
  {
    // The widest block: it shortens each block's chain of dependent loads
    // (one block per request runs once per SM at any batch size here).
    dim3 grid(l, batch);
    const int fin_nt = kPolyThreads;
    finish_kernel<T><<<grid, fin_nt, 0, st>>>(
        t > 1, resid[0], a_tilde, a_stride, packed, b_qstride, a_stride, true,
        log_q, s->prm.log_modulus1_after_switch,
        s->prm.log_modulus2_after_switch, resp, t > 1 ? s->ctx_e : s->ctx_f);
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "rescale"));
  }
  return Status{};
}

int64_t WorkspaceBytes(const inspire_pir_server* s, int batch) {
  const int64_t w = Words(s->prm.coeff_bits);
  const int64_t d = s->d;
  const int64_t B = batch;
  int64_t b = B * s->db_cols * w + B * 2 * s->k * d * w +
              B * std::max(1, 2 * s->ne) * d * w + B * s->rows * w +
              B * s->k * s->ctx_f.r * d * 4 +
              B * std::max(1, 2 * s->ne) * s->ctx_e.r * d * 4 +
              B * s->l * s->t * d * w + 2 * B * s->l * s->ctx_e.r * 2 * d * 4 +
              B * s->l * 2 * d * w;
  if (s->limb) b += s->limb->ScratchBytes(batch);
  return b;
}

Status EnsureWorkspace(inspire_pir_server* s, Workspace* ws, int batch) {
  if (batch <= ws->cap) return Status{};
  const size_t w = Words(s->prm.coeff_bits);
  const size_t d = s->d;
  const size_t B = batch;
  RETURN_IF_ERROR(ws->q1.Alloc(B * s->db_cols * w));
  RETURN_IF_ERROR(ws->pkey.Alloc(B * 2 * s->k * d * w));
  RETURN_IF_ERROR(ws->sdim.Alloc(B * std::max(1, 2 * s->ne) * d * w));
  RETURN_IF_ERROR(ws->gemv.Alloc(B * s->rows * w));
  RETURN_IF_ERROR(ws->yh.Alloc(B * s->k * s->ctx_f.r * d * 4));
  RETURN_IF_ERROR(ws->rgswb.Alloc(B * std::max(1, 2 * s->ne) * s->ctx_e.r * d * 4));
  RETURN_IF_ERROR(ws->packed.Alloc(B * s->l * s->t * d * w));
  RETURN_IF_ERROR(ws->resid0.Alloc(B * s->l * s->ctx_e.r * 2 * d * 4));
  RETURN_IF_ERROR(ws->resid1.Alloc(B * s->l * s->ctx_e.r * 2 * d * 4));
  RETURN_IF_ERROR(ws->resp.Alloc(B * s->l * 2 * d * w));
  if (s->limb && !ws->limb) ws->limb = s->limb->NewScratch();
  ws->cap = batch;
  return Status{};
}

Status InitWorkspace(Workspace* ws) {
  RETURN_IF_ERROR(Cuda(cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking),
                       "cudaStreamCreate"));
  for (auto& e : ws->ev) RETURN_IF_ERROR(Cuda(cudaEventCreate(&e), "cudaEventCreate"));
  RETURN_IF_ERROR(Cuda(cudaStreamCreateWithFlags(&ws->copy_stream, cudaStreamNonBlocking),
                       "cudaStreamCreate"));
  RETURN_IF_ERROR(Cuda(cudaEventCreateWithFlags(&ws->copy_go, cudaEventDisableTiming),
                       "cudaEventCreate"));
  RETURN_IF_ERROR(Cuda(cudaEventCreateWithFlags(&ws->sdim_ready, cudaEventDisableTiming),
                       "cudaEventCreate"));
  RETURN_IF_ERROR(Cuda(cudaEventCreateWithFlags(&ws->fork, cudaEventDisableTiming),
                       "cudaEventCreate"));
  RETURN_IF_ERROR(Cuda(cudaEventCreateWithFlags(&ws->side_done, cudaEventDisableTiming),
                       "cudaEventCreate"));
  return Cuda(cudaEventCreateWithFlags(&ws->done, cudaEventDisableTiming),
              "cudaEventCreate");
}

// Validation shared by every ProcessResponse flavour
// (pir_server.cc:160-205 plus the product size checks at :231-254).
Status ValidateRequest(const inspire_pir_server* s, int64_t first_dim_len,
                       int64_t second_dim_count, int64_t packing_key_count) {
  if (packing_key_count != 2 * s->k) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "Packing key must contain 2 * num_digits polynomials.");
  }
  if (first_dim_len < s->interpolated_rows || first_dim_len > s->db_cols) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "First dimension query size (" + std::to_string(first_dim_len) +
                   ") is invalid for DB columns (" +
                   std::to_string(s->db_cols) + ").");
  }
  if (s->t > 1 && second_dim_count != 2 * s->ne) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "second_dimension_query size mismatch. Must be 2 * num_digits.");
  }
  if (s->pack_cols != static_cast<int64_t>(s->k) * s->d) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "Vector size must match the number of matrix columns.");
  }
  return s->deferred;
}

// Batches from this size on use the tensor engine under INSPIRE_ENGINE_AUTO
// until inspire_pir_tune_engines has measured the crossover: the plain
// engine streams the matrices once per group of up to 4 requests, the
// tensor engine once per batch.
constexpr int32_t kDefaultCrossover = 5;

}  // namespace

int ResolveEngine(const inspire_pir_server* s, int engine, int batch) {
  if (engine != INSPIRE_ENGINE_AUTO) return engine;
  if (!s->limb) return INSPIRE_ENGINE_PLAIN;
  const int32_t c = s->crossover.load();
  return batch >= (c >= 0 ? c : kDefaultCrossover) ? INSPIRE_ENGINE_TENSOR
                                                   : INSPIRE_ENGINE_PLAIN;
}

namespace {

// Stage 1: out[q] = DB * q1[q] + P * y_g[q] for the whole batch, exact in
// the bits the answer reads: every caller takes the words mod 2^log_q
// (FinalizeMatrixPack and vPIR's local finalize apply LowBits first,
// lwes_to_rlwe.cc:464-469), so the tensor engine may skip digit positions
// at or above log_q.
Status Products(inspire_pir_server* s, Workspace* ws, int batch,
                const void* q1, const void* pkey, void* out, int engine,
                cudaStream_t st, int64_t pk_stride = -1) {
  const int cb = s->prm.coeff_bits;
  // Words between consecutive requests' packing keys (2k polynomials).
  if (pk_stride < 0) pk_stride = static_cast<int64_t>(2 * s->k) * s->d;
  if (engine == INSPIRE_ENGINE_TENSOR) {
    if (!s->limb) {
      return Err(INSPIRE_FAILED_PRECONDITION,
                 "tensor engine unavailable for these parameters");
    }
    if (!ws->limb) ws->limb = s->limb->NewScratch();
    return Cuda(s->limb->Run(batch, q1, s->db_cols, pkey, pk_stride, out,
                             ws->limb.get(), st, s->prm.log_modulus),
                "limb gemm");
  }
  if (engine != INSPIRE_ENGINE_PLAIN) {
    return Err(INSPIRE_INVALID_ARGUMENT, "unknown engine.");
  }
  return Cuda(launch_fused_gemv(cb, s->prm.db_kind, s->db.get(), s->db_cols, q1,
                                s->db_cols, s->prm.mat_kind, s->pack.get(),
                                s->pack_cols, pkey, pk_stride, out,
                                s->rows, s->rows, batch, st),
              "fused gemv");
}

// LowBits of the stage-1 words: vPIR's local finalize (b' + b_agg_partial
// reduced mod 2^log_q).
template <typename T>
__global__ void low_bits_kernel(const T* __restrict__ in, int64_t n, int log_q,
                                T* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    out[i] = low_bits<T>(in[i], log_q);
  }
}

// VpirServer::ProcessResponse (crypto/vpir/server/vpir_server.cc:102-195) on
// the device: DB and pack products, then per shard either LowBits(b' +
// b_agg_partial) (LocalFinalize) or FinalizeMatrixPack's b. out: batch x
// rows words (rows = ell * d).
Status VpirOnDevice(inspire_pir_server* s, Workspace* w, int batch, const void* q1,
                    const void* pkey, int64_t pk_stride, bool local, void* out,
                    int engine, cudaStream_t st) {
  RETURN_IF_ERROR(Products(s, w, batch, q1, pkey, w->gemv.get(), engine, st, pk_stride));
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    const int64_t n = static_cast<int64_t>(batch) * s->rows;
    if (local) {
      const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 152 * 8));
      low_bits_kernel<T><<<blocks, 256, 0, st>>>(w->gemv.get<T>(), n, s->prm.log_modulus,
                                                 static_cast<T*>(out));
      return Cuda(cudaGetLastError(), "local finalize");
    }
    // FinalizeStage reads y_h at offset k*d of each request's key.
    RETURN_IF_ERROR(FinalizeStage<T>(s, w, batch, static_cast<const T*>(pkey),
                                     w->gemv.get<T>(), st));
    return Cuda(cudaMemcpyAsync(out, w->packed.get(), n * sizeof(T),
                                cudaMemcpyDeviceToDevice, st),
                "finalize output");
  };
  return s->prm.coeff_bits == 32 ? run(uint32_t{}) : run(uint64_t{});
}

// The device part of a batch: products, polynomial stage, rescale.
Status AnswerOnDevice(inspire_pir_server* s, Workspace* w, int batch,
                      const void* q1, const void* pkey, const void* sdim,
                      void* resp, int engine, cudaStream_t st, bool timed,
                      cudaEvent_t sdim_ready = nullptr) {
  const int cb = s->prm.coeff_bits;
  // The request polynomials' transforms (y_h for FinalizeMatrixPack, the
  // RGSW b parts for EvalPoly) do not depend on the products: they run on
  // the workspace's second stream while the products stream the matrices,
  // after the copies already queued there (the host-buffer call copies the
  // second dimension on it), and join back before the polynomial stage.
  RETURN_IF_ERROR(Cuda(cudaEventRecord(w->fork, st), "record fork"));
  RETURN_IF_ERROR(Cuda(cudaStreamWaitEvent(w->copy_stream, w->fork, 0), "wait fork"));
  if (sdim_ready != nullptr) {
    RETURN_IF_ERROR(
        Cuda(cudaStreamWaitEvent(w->copy_stream, sdim_ready, 0), "wait second_dim"));
  }
  if (cb == 32) {
    RETURN_IF_ERROR(YhTransform<uint32_t>(s, w, batch, static_cast<const uint32_t*>(pkey),
                                          w->copy_stream));
    if (s->t > 1) {
      RETURN_IF_ERROR(RgswTransform<uint32_t>(
          s, w, batch, static_cast<const uint32_t*>(sdim), w->copy_stream));
    }
  } else {
    RETURN_IF_ERROR(YhTransform<uint64_t>(s, w, batch, static_cast<const uint64_t*>(pkey),
                                          w->copy_stream));
    if (s->t > 1) {
      RETURN_IF_ERROR(RgswTransform<uint64_t>(
          s, w, batch, static_cast<const uint64_t*>(sdim), w->copy_stream));
    }
  }
  RETURN_IF_ERROR(Cuda(cudaEventRecord(w->side_done, w->copy_stream), "record join"));
  if (timed) cudaEventRecord(w->ev[0], st);
  RETURN_IF_ERROR(Products(s, w, batch, q1, pkey, w->gemv.get(), engine, st));
  if (timed) cudaEventRecord(w->ev[1], st);
  RETURN_IF_ERROR(Cuda(cudaStreamWaitEvent(st, w->side_done, 0), "wait join"));
  if (cb == 32) {
    RETURN_IF_ERROR(RunPolyStage<uint32_t>(
        s, w, batch, static_cast<const uint32_t*>(pkey),
        static_cast<const uint32_t*>(sdim), w->gemv.get<uint32_t>(),
        static_cast<uint32_t*>(resp), st, timed, true));
  } else {
    RETURN_IF_ERROR(RunPolyStage<uint64_t>(
        s, w, batch, static_cast<const uint64_t*>(pkey),
        static_cast<const uint64_t*>(sdim), w->gemv.get<uint64_t>(),
        static_cast<uint64_t*>(resp), st, timed, true));
  }
  if (timed) cudaEventRecord(w->ev[3], st);
  return Status{};
}

// Zero-padded first dimension of a device-resident batch
// (pir_server.cc:221-227): the products read db_cols words per request, so
// short requests are copied into the workspace and padded there.
Status DeviceFirstDim(inspire_pir_server* s, Workspace* ws, int batch,
                      const void** first_dim, int64_t first_dim_len,
                      cudaStream_t st) {
  if (first_dim_len >= s->db_cols) return Status{};
  const size_t w = Words(s->prm.coeff_bits);
  RETURN_IF_ERROR(Cuda(cudaMemcpy2DAsync(ws->q1.get(), s->db_cols * w, *first_dim,
                                         first_dim_len * w, first_dim_len * w,
                                         batch, cudaMemcpyDeviceToDevice, st),
                       "copy first_dim"));
  RETURN_IF_ERROR(Cuda(
      cudaMemset2DAsync(static_cast<char*>(ws->q1.get()) + first_dim_len * w,
                        s->db_cols * w, 0, (s->db_cols - first_dim_len) * w,
                        batch, st),
      "pad first_dim"));
  *first_dim = ws->q1.get();
  return Status{};
}

// The packing tool's server step for a batch: products, then
// FinalizeMatrixPack of every shard, written as (a_tilde_agg, b_agg) pairs;
// no EvalPoly, no modulus switch.
Status PackOnDevice(inspire_pir_server* s, Workspace* w, int batch,
                    const void* q1, const void* pkey, void* out, int engine,
                    cudaStream_t st) {
  RETURN_IF_ERROR(Products(s, w, batch, q1, pkey, w->gemv.get(), engine, st));
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    RETURN_IF_ERROR(FinalizeStage<T>(s, w, batch, static_cast<const T*>(pkey),
                                     w->gemv.get<T>(), st));
    pack_out_kernel<T><<<dim3(s->l * s->t, batch), PolyThreads(s->d), 0, st>>>(
        s->a_tilde.get<T>(), w->packed.get<T>(), s->d, static_cast<T*>(out));
    return Cuda(cudaGetLastError(), "pack output");
  };
  return s->prm.coeff_bits == 32 ? run(uint32_t{}) : run(uint64_t{});
}

// ExternalProduct (external_product.cc:35-114) of `batch` independent
// ciphertexts, each with its own RGSW ciphertext, with the server's eval
// gadget and NTT tables. ct: [batch][2][d] (a, b); rgsw: [batch][2ne][2][d]
// (u[0..ne) then v[0..ne), each an (a, b) pair); out: [batch][2][d].
Status ExternalOnDevice(inspire_pir_server* s, Workspace* w, int batch,
                        const void* ct, const void* rgsw, void* out,
                        cudaStream_t st) {
  RETURN_IF_ERROR(s->eval_rule);
  const int d = s->d, ne = s->ne, ng = 2 * s->ne;
  const NttCtx& c = s->ctx_e;
  const size_t need = static_cast<size_t>(batch) * ng * c.r * d * 4;
  if (w->rgswa.bytes() < need) RETURN_IF_ERROR(w->rgswa.Alloc(need));
  const int nt = PolyThreads(d);
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    const T* rg = static_cast<const T*>(rgsw);
    const int64_t qs = static_cast<int64_t>(2 * ng) * d;
    RETURN_IF_ERROR(NttCoeffs<T>(s, rg, qs, 0, ng, static_cast<T>(s->vmask_e),
                                 w->rgswa.get<uint32_t>(), 2 * d, c, batch, st));
    RETURN_IF_ERROR(NttCoeffs<T>(s, rg, qs, d, ng, static_cast<T>(s->vmask_e),
                                 w->rgswb.get<uint32_t>(), 2 * d, c, batch, st));
    ExtArgs e{s->prm.log_modulus, s->prm.eval_log_digit, ne,
              LiveDigits(s->prm.log_modulus, s->prm.eval_log_digit, ne),
              s->umask_e};
    const size_t smem = static_cast<size_t>(d) * 4 + 2ull * d * sizeof(T);
    const T* cta = static_cast<const T*>(ct);
    const int64_t rq = static_cast<int64_t>(ng) * c.r * d;  // RGSW a per request
    if (c.tables16 != nullptr && batch >= Ext16Min(s, d)) {
      // The radix-16 kernels as in RunPolyStage: one block per ciphertext.
      INSPIRE_NTT16_DISPATCH(
          c.logd, RETURN_IF_ERROR(SetSmem(ext_step16_kernel<T, LG>, smem));
          ext_step16_kernel<T, LG><<<dim3(1, batch), Ntt16<LG>::kThreads, smem, st>>>(
              true, nullptr, w->resid0.get<uint32_t>(), cta, 2 * d, 0, cta + d, 2 * d, 0,
              w->rgswa.get<uint32_t>(), rq, w->rgswb.get<uint32_t>(), e, c));
    } else if (c.tables16 != nullptr && d <= 4096) {
      INSPIRE_NTT16_PAIR_DISPATCH(
          c.logd, RETURN_IF_ERROR((LaunchPairExt<T, LG>(
                      static_cast<int64_t>(c.r) * batch, s->sms, dim3(c.r, 1, batch), st,
                      true, static_cast<const uint32_t*>(nullptr), w->resid0.get<uint32_t>(),
                      cta, int64_t{2} * d, int64_t{0}, cta + d, int64_t{2} * d, int64_t{0},
                      static_cast<const uint32_t*>(w->rgswa.get<uint32_t>()), rq,
                      static_cast<const uint32_t*>(w->rgswb.get<uint32_t>()), e, c))));
    } else {
      const PolyLaunch pl = PolyShapeFor(d, static_cast<int64_t>(c.r) * batch, s->sms);
      INSPIRE_ITERS_DISPATCH(
          pl.iters, RETURN_IF_ERROR(SetSmem(ext_step_kernel<T, IT>, smem));
          ext_step_kernel<T, IT><<<dim3(c.r, 1, batch), pl.nt, smem, st>>>(
              true, nullptr, w->resid0.get<uint32_t>(), cta, 2 * d, 0, cta + d, 2 * d, 0,
              w->rgswa.get<uint32_t>(), rq, w->rgswb.get<uint32_t>(), e, c));
    }
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "external product"));
    finish_kernel<T><<<dim3(1, batch), nt, 0, st>>>(
        true, w->resid0.get<uint32_t>(), nullptr, 0, nullptr, 0, 0, false, 0, 0,
        0, static_cast<T*>(out), c);
    return Cuda(cudaGetLastError(), "external product output");
  };
  return s->prm.coeff_bits == 32 ? run(uint32_t{}) : run(uint64_t{});
}

Status ProcessHostBatch(inspire_pir_server* s, int batch, const void* first_dim,
                        int64_t first_dim_len, const void* second_dim,
                        int64_t second_dim_count, const void* packing_key,
                        int64_t packing_key_count, void* responses,
                        int engine) {
  if (batch <= 0) return Err(INSPIRE_INVALID_ARGUMENT, "batch must be positive.");
  RETURN_IF_ERROR(ValidateRequest(s, first_dim_len, second_dim_count,
                                  packing_key_count));
  std::lock_guard<std::mutex> lock(s->mu);
  Workspace* ws = s->ws0.get();
  RETURN_IF_ERROR(EnsureWorkspace(s, ws, batch));
  const size_t w = Words(s->prm.coeff_bits);
  const size_t d = s->d;
  cudaStream_t st = ws->stream;
  // Zero-padded first dimension (pir_server.cc:221-227).
  RETURN_IF_ERROR(Cuda(cudaMemcpy2DAsync(ws->q1.get(), s->db_cols * w, first_dim,
                                         first_dim_len * w, first_dim_len * w,
                                         batch, cudaMemcpyHostToDevice, st),
                       "copy first_dim"));
  if (first_dim_len < s->db_cols) {
    RETURN_IF_ERROR(Cuda(
        cudaMemset2DAsync(static_cast<char*>(ws->q1.get()) + first_dim_len * w,
                          s->db_cols * w, 0, (s->db_cols - first_dim_len) * w,
                          batch, st),
        "pad first_dim"));
  }
  RETURN_IF_ERROR(Cuda(cudaMemcpyAsync(ws->pkey.get(), packing_key,
                                       batch * packing_key_count * d * w,
                                       cudaMemcpyHostToDevice, st),
                       "copy packing_key"));
  cudaEvent_t sdim_ready = nullptr;
  if (s->t > 1) {
    // On the copy stream, after everything already queued on the workspace
    // stream (an earlier batch may still read sdim); the polynomial stage
    // waits for it, the products do not.
    RETURN_IF_ERROR(Cuda(cudaEventRecord(ws->copy_go, st), "record"));
    RETURN_IF_ERROR(Cuda(cudaStreamWaitEvent(ws->copy_stream, ws->copy_go, 0), "wait"));
    RETURN_IF_ERROR(Cuda(cudaMemcpyAsync(ws->sdim.get(), second_dim,
                                         batch * second_dim_count * d * w,
                                         cudaMemcpyHostToDevice, ws->copy_stream),
                         "copy second_dim"));
    RETURN_IF_ERROR(Cuda(cudaEventRecord(ws->sdim_ready, ws->copy_stream), "record"));
    sdim_ready = ws->sdim_ready;
  }
  RETURN_IF_ERROR(AnswerOnDevice(s, ws, batch, ws->q1.get(), ws->pkey.get(),
                                 ws->sdim.get(), ws->resp.get(), engine, st, true,
                                 sdim_ready));
  const size_t out_bytes = static_cast<size_t>(batch) * s->l * 2 * d * w;
  RETURN_IF_ERROR(Cuda(cudaMemcpyAsync(responses, ws->resp.get(), out_bytes,
                                       cudaMemcpyDeviceToHost, st),
                       "copy response"));
  RETURN_IF_ERROR(Cuda(cudaStreamSynchronize(st), "answer"));
  if (engine == INSPIRE_ENGINE_TENSOR && s->limb && s->limb->CheckError() != 0) {
    return Err(INSPIRE_INTERNAL, "tensor engine pipeline timed out");
  }
  float ms_db = 0, ms_pack = 0, ms_eval = 0;
  cudaEventElapsedTime(&ms_db, ws->ev[0], ws->ev[1]);
  cudaEventElapsedTime(&ms_pack, ws->ev[1], ws->ev[2]);
  cudaEventElapsedTime(&ms_eval, ws->ev[2], ws->ev[3]);
  s->t_db += ms_db;
  s->t_pack += ms_pack;
  s->t_eval += ms_eval;
  return Status{};
}

// Server-constant transforms: t_vec_h (signed digits, the chunk rule's
// operand) and second_dim_a (the RGSW a polynomials).
template <typename T>
Status PrepareConstants(inspire_pir_server* s, const T* t_vec_h,
                        const T* second_dim_a, const ChunkRule& rule_f,
                        const ChunkRule& rule_e) {
  const int d = s->d;
  const int64_t nth = static_cast<int64_t>(s->l) * s->t * s->k;
  {
    std::vector<int64_t> th(nth * d);
    for (int64_t i = 0; i < nth * d; ++i) {
      th[i] = RebuildU(static_cast<uint64_t>(t_vec_h[i]), rule_f,
                       s->prm.pack_log_digit, true);
    }
    DevBuf tmp;
    RETURN_IF_ERROR(tmp.Upload(th.data(), th.size() * 8));
    RETURN_IF_ERROR(s->th_ntt.Alloc(nth * s->ctx_f.r * d * 4));
    ntt_signed_kernel<<<static_cast<unsigned>(nth * s->ctx_f.r), kPolyThreads,
                        d * 4>>>(tmp.get<int64_t>(), static_cast<int>(nth),
                                 s->th_ntt.get<uint32_t>(), s->ctx_f);
    RETURN_IF_ERROR(Cuda(cudaDeviceSynchronize(), "t_vec_h transform"));
  }
  if (s->t > 1) {
    const int ng = 2 * s->ne;
    DevBuf tmp;
    RETURN_IF_ERROR(tmp.Upload(second_dim_a, static_cast<size_t>(ng) * d * sizeof(T)));
    RETURN_IF_ERROR(s->rgswa_ntt.Alloc(static_cast<size_t>(ng) * s->ctx_e.r * d * 4));
    dim3 grid(ng * s->ctx_e.r, 1);
    ntt_coeffs_kernel<T><<<grid, kPolyThreads, d * 4>>>(
        tmp.get<T>(), 0, 0, ng, static_cast<T>(s->vmask_e),
        s->rgswa_ntt.get<uint32_t>(), d, s->ctx_e);
    RETURN_IF_ERROR(Cuda(cudaDeviceSynchronize(), "second_dim_a transform"));
  }
  (void)rule_e;
  return Status{};
}

Status CreateServer(const inspire_pir_params* prm, const void* db,
                    int64_t db_rows, int64_t db_cols, const void* pack,
                    int64_t pack_rows, int64_t pack_cols,
                    const void* a_tilde_agg, int64_t a_count,
                    const void* t_vec_h, int64_t th_count,
                    const void* second_dim_a, int64_t sda_count,
                    std::unique_ptr<inspire_pir_server>* out,
                    DevBuf* db_dev = nullptr, DevBuf* pack_dev = nullptr) {
  if (prm == nullptr) return Err(INSPIRE_INVALID_ARGUMENT, "params is null.");
  if (prm->coeff_bits != 32 && prm->coeff_bits != 64) {
    return Err(INSPIRE_INVALID_ARGUMENT, "coeff_bits must be 32 or 64.");
  }
  if (prm->db_kind != INSPIRE_U8 && prm->db_kind != INSPIRE_U16) {
    return Err(INSPIRE_INVALID_ARGUMENT, "DbDataType must be uint8_t or uint16_t.");
  }
  if (prm->mat_kind != INSPIRE_I16 && prm->mat_kind != INSPIRE_I32 &&
      prm->mat_kind != (prm->coeff_bits == 32 ? INSPIRE_U32 : INSPIRE_U64)) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "MatCoeffType must be int16_t, int32_t or CoeffType.");
  }
  if (prm->log_degree < 5 || prm->log_degree > 13) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "ring degree must be between 32 and 8192.");
  }
  // PirParams::Create validation (crypto/pir/pir_params.cc:29-68).
  const int t = prm->interpolation_degree;
  const int d = 1 << prm->log_degree;
  if (prm->num_entries <= 0) {
    return Err(INSPIRE_INVALID_ARGUMENT, "num_entries must be strictly positive.");
  }
  if (prm->entry_size_multiple <= 0) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "entry_size_multiple must be strictly positive.");
  }
  if (t <= 0 || (t & (t - 1)) != 0) {
    return Err(INSPIRE_INVALID_ARGUMENT, "interpolation_degree must be a power of two.");
  }
  if (prm->num_entries % t != 0) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "interpolation_degree (" + std::to_string(t) +
                   ") must divide num_entries (" +
                   std::to_string(prm->num_entries) + ").");
  }
  if (t > 2 * d) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "interpolation_degree (" + std::to_string(t) +
                   ") must be less than or equal to 2 * ring degree (" +
                   std::to_string(2 * d) + ").");
  }
  if (prm->log_modulus <= 0 || prm->log_modulus > prm->coeff_bits) {
    return Err(INSPIRE_INVALID_ARGUMENT, "log_modulus out of range.");
  }
  if (prm->pack_num_digits <= 0 || prm->pack_log_digit <= 0 ||
      prm->eval_num_digits <= 0 || prm->eval_log_digit <= 0) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "log_digit and num_digits must be positive.");
  }
  const int l = prm->entry_size_multiple;
  // PirServer::Create shape checks (pir_server.cc:58-95).
  if (db_rows != static_cast<int64_t>(l) * t * d) {
    return Err(INSPIRE_INVALID_ARGUMENT, "DB matrix must have td rows.");
  }
  if (db_cols < prm->num_entries / t) {
    return Err(INSPIRE_INVALID_ARGUMENT, "DB matrix must have at least N/t columns.");
  }
  if (a_count != static_cast<int64_t>(l) * t) {
    return Err(INSPIRE_INVALID_ARGUMENT, "Preprocessed outputs must be of length t.");
  }
  if (th_count != static_cast<int64_t>(l) * t * prm->pack_num_digits) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "t_vec_h must hold pack_num_digits polynomials per slice.");
  }
  if (pack_rows != db_rows) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "Packing multiplication resulted in incorrect vector size.");
  }
  if (t > 1 && sda_count != 2 * prm->eval_num_digits) {
    return Err(INSPIRE_INVALID_ARGUMENT,
               "second_dim_query_a must have length 2 * "
               "PolyEvalGadgetParams().num_digits.");
  }
  int dev = 0;
  RETURN_IF_ERROR(Cuda(cudaGetDevice(&dev), "cudaGetDevice"));

  std::unique_ptr<inspire_pir_server> s(new inspire_pir_server());
  s->prm = *prm;
  s->d = d;
  s->t = t;
  s->l = l;
  s->k = prm->pack_num_digits;
  s->ne = prm->eval_num_digits;
  s->rows = db_rows;
  s->db_cols = db_cols;
  s->pack_cols = pack_cols;
  s->interpolated_rows = prm->num_entries / t;
  s->db_orig_cols = static_cast<int32_t>(std::min<int64_t>(db_cols, s->interpolated_rows));
  s->db_condensed = prm->coeff_bits == 64;
  // BuildPreprocessMatrix condenses int32 matrices only (lwes_to_rlwe.cc:221-226).
  s->pack_condensed = prm->mat_kind == INSPIRE_I32;

  // Chunk rules of the two inner products and the prime counts that make
  // the NTT route exact for every operand those rules admit.
  const int cb = prm->coeff_bits;
  ChunkRule rf, re;
  Status sf = MakeRule(cb, s->k, d, prm->pack_log_digit, prm->log_modulus,
                       ChunkFor(s->k, d), &rf);
  Status se = MakeRule(cb, 2 * s->ne, d, prm->eval_log_digit, prm->log_modulus,
                       ChunkFor(2 * s->ne, d), &re);
  if (!sf.ok()) s->deferred = sf;
  if (t > 1 && !se.ok() && s->deferred.ok()) s->deferred = se;
  s->eval_rule = se;
  int r_f = 3, r_e = 3;
  if (sf.ok()) {
    s->vmask_f = MaskBits(rf.v_chunks * rf.chunk_bits, cb);
    RETURN_IF_ERROR(PrimesFor(
        BoundBits(s->k, d, std::min(rf.u_chunks * rf.chunk_bits, 64),
                  std::min(rf.v_chunks * rf.chunk_bits, cb)),
        &r_f));
  }
  if (se.ok()) {
    s->vmask_e = MaskBits(re.v_chunks * re.chunk_bits, cb);
    s->umask_e = MaskBits(re.u_chunks * re.chunk_bits, cb);
    RETURN_IF_ERROR(PrimesFor(
        BoundBits(2 * s->ne, d,
                  std::min({prm->eval_log_digit, re.u_chunks * re.chunk_bits, cb}),
                  std::min(re.v_chunks * re.chunk_bits, cb)),
        &r_e));
  }
  RETURN_IF_ERROR(NttTables::Create(prm->log_degree, &s->tables));
  {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
      cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
    }
  }
  s->ctx_f = s->tables->Ctx(r_f);
  s->ctx_e = s->tables->Ctx(r_e);

  const size_t w = Words(cb);
  const size_t db_bytes = static_cast<size_t>(db_rows) * db_cols * elem_size(prm->db_kind);
  const size_t pack_bytes =
      static_cast<size_t>(pack_rows) * pack_cols * elem_size(prm->mat_kind);
  if (db_dev != nullptr && pack_dev != nullptr) {
    // Matrices already in GPU memory (the image loader) move in.
    if (db_dev->bytes() < db_bytes || pack_dev->bytes() < pack_bytes) {
      return Err(INSPIRE_INTERNAL, "device matrices smaller than their shapes.");
    }
    s->db.Take(db_dev);
    s->pack.Take(pack_dev);
  } else {
    RETURN_IF_ERROR(s->db.Upload(db, db_bytes));
    RETURN_IF_ERROR(s->pack.Upload(pack, pack_bytes));
  }
  // Raw copies of the small polynomial material, for SaveToFile images.
  s->t_vec_h_raw.assign(static_cast<const uint8_t*>(t_vec_h),
                        static_cast<const uint8_t*>(t_vec_h) + th_count * d * w);
  if (sda_count > 0) {
    s->second_dim_a_raw.assign(static_cast<const uint8_t*>(second_dim_a),
                               static_cast<const uint8_t*>(second_dim_a) +
                                   sda_count * d * w);
  }
  RETURN_IF_ERROR(s->a_tilde.Upload(a_tilde_agg, static_cast<size_t>(a_count) * d * w));
  if (sf.ok() && (t == 1 || se.ok())) {
    if (cb == 32) {
      RETURN_IF_ERROR(PrepareConstants<uint32_t>(
          s.get(), static_cast<const uint32_t*>(t_vec_h),
          static_cast<const uint32_t*>(second_dim_a), rf, re));
    } else {
      RETURN_IF_ERROR(PrepareConstants<uint64_t>(
          s.get(), static_cast<const uint64_t*>(t_vec_h),
          static_cast<const uint64_t*>(second_dim_a), rf, re));
    }
  }
  s->ws0.reset(new Workspace());
  RETURN_IF_ERROR(InitWorkspace(s->ws0.get()));
  // The tensor-core engine when the shapes allow it.
  LimbGemm::Create(cb, prm->db_kind, s->db.get(), db_rows, db_cols,
                   prm->mat_kind, s->pack.get(), pack_cols, true, &s->limb);
  *out = std::move(s);
  return Status{};
}

// ---------------------------------------------------------------------------
// The PirServer file image: PirServer::SaveToFile / LoadFromBuffer
// (crypto/pir/server/pir_server.cc:434-588, 590-780). Little-endian fields;
// the DB as its raw (or condensed u64) words; the pack matrix as signed
// entries of pack_log_digit + bit_width(d - 1) bits and the polynomials as
// log_modulus-bit coefficients, least-significant bit first
// (BitPackSigned / BitPackCoefficients, pir_server.cc:310-431). The two
// large sections go straight between the image and GPU memory; the pack
// matrix is bit-packed and unpacked by kernels.
// ---------------------------------------------------------------------------
// Entry i of `bits` bits starts at bit i * bits (sign-extended).
template <typename M>
__global__ void bit_unpack_signed_kernel(const uint8_t* __restrict__ packed,
                                         int64_t packed_len, int64_t n, int bits,
                                         M* __restrict__ out) {
  const uint64_t mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t bit = static_cast<uint64_t>(i) * bits;
    const int64_t byte0 = static_cast<int64_t>(bit >> 3);
    const int shift = static_cast<int>(bit & 7);
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      if (byte0 + b < packed_len) lo |= static_cast<uint64_t>(packed[byte0 + b]) << (8 * b);
    }
    if (byte0 + 8 < packed_len) hi = packed[byte0 + 8];
    uint64_t v = (lo >> shift) | (shift ? (hi << (64 - shift)) : 0);
    v &= mask;
    if (bits < 64 && ((v >> (bits - 1)) & 1)) v |= ~mask;
    out[i] = static_cast<M>(static_cast<int64_t>(v));
  }
}

// Output word w (bits 64w .. 64w+63) gathers the entries overlapping it.
template <typename M>
__global__ void bit_pack_kernel(const M* __restrict__ in, int64_t n, int bits,
                                int64_t words, uint64_t* __restrict__ out) {
  const uint64_t mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
  for (int64_t w = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       w < words; w += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t bit0 = w * 64;
    const int64_t e0 = bit0 / bits;
    const int64_t e1 = min(n, (bit0 + 64 + bits - 1) / bits);
    uint64_t acc = 0;
    for (int64_t e = e0; e < e1; ++e) {
      const uint64_t v =
          static_cast<uint64_t>(static_cast<int64_t>(in[e])) & mask;
      const int64_t start = e * bits - bit0;
      if (start >= 0) {
        if (start < 64) acc |= v << start;
      } else if (-start < 64) {
        acc |= v >> (-start);
      }
    }
    out[w] = acc;
  }
}

struct ImageReader {
  const uint8_t* p;
  size_t size, off = 0;
  bool ok = true;
  template <typename V>
  V get() {
    V v{};
    if (off + sizeof(V) > size) {
      ok = false;
      return v;
    }
    std::memcpy(&v, p + off, sizeof(V));
    off += sizeof(V);
    return v;
  }
  const uint8_t* take(size_t n) {
    if (!ok || off + n > size) {
      ok = false;
      return nullptr;
    }
    const uint8_t* q = p + off;
    off += n;
    return q;
  }
};

// BitUnpackCoefficients (below the coefficient width; raw words otherwise).
void UnpackCoeffs(const uint8_t* data, size_t packed_len, uint64_t n, int bits,
                  int coeff_bits, std::vector<uint8_t>* out) {
  const size_t w = coeff_bits / 8;
  const size_t at = out->size();
  out->resize(at + n * w, 0);
  uint8_t* dst = out->data() + at;
  if (bits >= coeff_bits) {
    std::memcpy(dst, data, std::min<size_t>(packed_len, n * w));
    return;
  }
  uint64_t bit = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t v = 0;
    for (int b = 0; b < bits; ++b, ++bit) {
      const size_t byte = bit >> 3;
      if (byte < packed_len && ((data[byte] >> (bit & 7)) & 1)) v |= uint64_t{1} << b;
    }
    std::memcpy(dst + i * w, &v, w);  // little-endian low bytes
  }
}

std::vector<uint8_t> PackCoeffs(const uint8_t* src, uint64_t n, int bits, int coeff_bits) {
  const size_t w = coeff_bits / 8;
  if (bits >= coeff_bits) return std::vector<uint8_t>(src, src + n * w);
  std::vector<uint8_t> out((n * bits + 7) / 8, 0);
  uint64_t bit = 0;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t v = 0;
    std::memcpy(&v, src + i * w, w);
    for (int b = 0; b < bits; ++b, ++bit) {
      if ((v >> b) & 1) out[bit >> 3] |= static_cast<uint8_t>(1u << (bit & 7));
    }
  }
  return out;
}

Status LoadImage(const inspire_pir_params* prm, const uint8_t* buf, size_t size,
                 std::unique_ptr<inspire_pir_server>* out) {
  if (prm == nullptr || buf == nullptr) {
    return Err(INSPIRE_INTERNAL, "Failed to read buffer");
  }
  const Status bad = Err(INSPIRE_INTERNAL, "Error reading from buffer");
  ImageReader r{buf, size};
  const int cb = prm->coeff_bits;
  // 1. The DB matrix.
  const int32_t db_rows = r.get<int32_t>();
  const int32_t db_phys = r.get<int32_t>();
  const uint8_t db_cond = r.get<uint8_t>();
  const int32_t db_orig = r.get<int32_t>();
  const uint64_t db_n = r.get<uint64_t>();
  const size_t es = elem_size(prm->db_kind);
  const size_t db_bytes = db_n * (db_cond ? 8 : es);
  const int64_t db_cols = db_cond ? static_cast<int64_t>(db_phys) * 8 / es : db_phys;
  const uint8_t* db_src = r.take(db_bytes);
  if (!r.ok || static_cast<size_t>(db_rows) * db_cols * es != db_bytes) return bad;
  DevBuf db;
  RETURN_IF_ERROR(db.Alloc(db_bytes));
  RETURN_IF_ERROR(Cuda(cudaMemcpy(db.get(), db_src, db_bytes, cudaMemcpyHostToDevice),
                       "DB upload"));
  // 2. The pack matrix, bit-unpacked on the GPU.
  const int32_t prow = r.get<int32_t>();
  const int32_t pcol = r.get<int32_t>();
  const int32_t pphys = r.get<int32_t>();
  const uint8_t pcond = r.get<uint8_t>();
  const int32_t porig = r.get<int32_t>();
  const int32_t pbits = r.get<int32_t>();
  const uint64_t plen = r.get<uint64_t>();
  const uint8_t* psrc = r.take(plen);
  const int64_t pn = static_cast<int64_t>(prow) * pcol;
  if (!r.ok || pbits <= 0 || pbits > 64 || (pn * pbits + 7) / 8 > static_cast<int64_t>(plen)) {
    return bad;
  }
  (void)pphys;
  (void)porig;
  DevBuf packed, pack;
  RETURN_IF_ERROR(packed.Upload(psrc, plen));
  RETURN_IF_ERROR(pack.Alloc(pn * elem_size(prm->mat_kind)));
  if (pn > 0) {
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((pn + 255) / 256, 152 * 32));
    switch (prm->mat_kind) {
      case INSPIRE_I16:
        bit_unpack_signed_kernel<int16_t><<<blocks, 256>>>(packed.get<uint8_t>(), plen, pn,
                                                           pbits, pack.get<int16_t>());
        break;
      case INSPIRE_I32:
        bit_unpack_signed_kernel<int32_t><<<blocks, 256>>>(packed.get<uint8_t>(), plen, pn,
                                                           pbits, pack.get<int32_t>());
        break;
      case INSPIRE_U32:
        bit_unpack_signed_kernel<uint32_t><<<blocks, 256>>>(packed.get<uint8_t>(), plen, pn,
                                                            pbits, pack.get<uint32_t>());
        break;
      default:
        bit_unpack_signed_kernel<uint64_t><<<blocks, 256>>>(packed.get<uint8_t>(), plen, pn,
                                                            pbits, pack.get<uint64_t>());
    }
    RETURN_IF_ERROR(Cuda(cudaDeviceSynchronize(), "pack matrix unpack"));
  }
  packed.Free();
  // 3. Per shard and slice: a_tilde_agg and t_vec_h.
  const int32_t log_q = r.get<int32_t>();
  const int32_t shards = r.get<int32_t>();
  std::vector<uint8_t> a_tilde, t_vec_h, sda;
  int64_t a_count = 0, th_count = 0, sda_count = 0;
  auto poly = [&](std::vector<uint8_t>* dst) {
    const uint64_t len = r.get<uint64_t>();
    const uint64_t plen2 = r.get<uint64_t>();
    const uint8_t* data = r.take(plen2);
    if (r.ok) UnpackCoeffs(data, plen2, len, log_q, cb, dst);
  };
  for (int32_t k = 0; k < shards && r.ok; ++k) {
    const int32_t slices = r.get<int32_t>();
    for (int32_t i = 0; i < slices && r.ok; ++i) {
      poly(&a_tilde);
      ++a_count;
      const uint64_t tn = r.get<uint64_t>();
      for (uint64_t j = 0; j < tn && r.ok; ++j) {
        poly(&t_vec_h);
        ++th_count;
      }
    }
  }
  // 4. second_dim_a.
  const uint64_t nsd = r.get<uint64_t>();
  for (uint64_t j = 0; j < nsd && r.ok; ++j) {
    poly(&sda);
    ++sda_count;
  }
  if (!r.ok) return bad;
  RETURN_IF_ERROR(CreateServer(prm, db.get(), db_rows, db_cols, pack.get(), prow, pcol,
                               a_tilde.data(), a_count, t_vec_h.data(), th_count,
                               sda.data(), sda_count, out, &db, &pack));
  (*out)->db_condensed = db_cond != 0;
  (*out)->pack_condensed = pcond != 0;
  (*out)->db_orig_cols = db_orig;
  (*out)->orig_from_file = true;
  (*out)->pack_bits = pbits;
  return Status{};
}

// Writes the image into dst (or only counts its bytes when dst is null).
struct ImageWriter {
  uint8_t* dst;
  size_t cap, off = 0;
  void put(const void* p, size_t n) {
    if (dst != nullptr && off + n <= cap) std::memcpy(dst + off, p, n);
    off += n;
  }
  template <typename V>
  void val(V v) {
    put(&v, sizeof(V));
  }
};

Status SaveImage(inspire_pir_server* s, uint8_t* dst, size_t cap, size_t* size) {
  ImageWriter w{dst, cap};
  const int cb = s->prm.coeff_bits;
  const size_t cw = cb / 8;
  const int d = s->d;
  const size_t es = elem_size(s->prm.db_kind);
  const bool dcond = s->db_condensed && (s->db_cols * es) % 8 == 0;
  // 1. DB.
  w.val<int32_t>(static_cast<int32_t>(s->rows));
  w.val<int32_t>(static_cast<int32_t>(dcond ? s->db_cols * es / 8 : s->db_cols));
  w.val<uint8_t>(dcond ? 1 : 0);
  w.val<int32_t>(s->db_orig_cols);
  const size_t db_bytes = static_cast<size_t>(s->rows) * s->db_cols * es;
  w.val<uint64_t>(dcond ? db_bytes / 8 : static_cast<uint64_t>(s->rows) * s->db_cols);
  if (dst != nullptr && w.off + db_bytes <= cap && db_bytes > 0) {
    RETURN_IF_ERROR(Cuda(cudaMemcpy(dst + w.off, s->db.get(), db_bytes,
                                    cudaMemcpyDeviceToHost),
                         "DB download"));
  }
  w.off += db_bytes;
  // 2. Pack matrix, bit-packed on the GPU.
  const size_t ms = elem_size(s->prm.mat_kind);
  const bool pcond = s->pack_condensed && (s->pack_cols * ms) % 8 == 0;
  int bits = s->pack_bits;
  if (bits <= 0) {
    int bw = 0;
    while ((1 << bw) < d) ++bw;  // bit_width(d - 1) for a power of two d
    bits = s->prm.pack_log_digit + bw;
  }
  w.val<int32_t>(static_cast<int32_t>(s->rows));
  w.val<int32_t>(static_cast<int32_t>(s->pack_cols));
  w.val<int32_t>(static_cast<int32_t>(pcond ? s->pack_cols * ms / 8 : s->pack_cols));
  w.val<uint8_t>(pcond ? 1 : 0);
  w.val<int32_t>(static_cast<int32_t>(s->pack_cols));
  w.val<int32_t>(bits);
  const int64_t pn = s->rows * s->pack_cols;
  const uint64_t plen = (static_cast<uint64_t>(pn) * bits + 7) / 8;
  w.val<uint64_t>(plen);
  if (dst != nullptr && w.off + plen <= cap && plen > 0) {
    const int64_t words = static_cast<int64_t>((plen + 7) / 8);
    DevBuf packed;
    RETURN_IF_ERROR(packed.Alloc(words * 8));
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((words + 255) / 256, 152 * 32));
    switch (s->prm.mat_kind) {
      case INSPIRE_I16:
        bit_pack_kernel<int16_t><<<blocks, 256>>>(s->pack.get<int16_t>(), pn, bits, words,
                                                  packed.get<uint64_t>());
        break;
      case INSPIRE_I32:
        bit_pack_kernel<int32_t><<<blocks, 256>>>(s->pack.get<int32_t>(), pn, bits, words,
                                                  packed.get<uint64_t>());
        break;
      case INSPIRE_U32:
        bit_pack_kernel<int32_t><<<blocks, 256>>>(s->pack.get<int32_t>(), pn, bits, words,
                                                  packed.get<uint64_t>());
        break;
      default:
        bit_pack_kernel<int64_t><<<blocks, 256>>>(s->pack.get<int64_t>(), pn, bits, words,
                                                  packed.get<uint64_t>());
    }
    RETURN_IF_ERROR(Cuda(cudaMemcpy(dst + w.off, packed.get(), plen, cudaMemcpyDeviceToHost),
                         "pack matrix download"));
  }
  w.off += plen;
  // 3. a_tilde_agg and t_vec_h per shard and slice.
  const int log_q = s->prm.log_modulus;
  w.val<int32_t>(log_q);
  w.val<int32_t>(s->l);
  std::vector<uint8_t> a_host(static_cast<size_t>(s->l) * s->t * d * cw);
  RETURN_IF_ERROR(Cuda(cudaMemcpy(a_host.data(), s->a_tilde.get(), a_host.size(),
                                  cudaMemcpyDeviceToHost),
                       "a_tilde download"));
  auto poly = [&](const uint8_t* src) {
    const std::vector<uint8_t> b = PackCoeffs(src, d, log_q, cb);
    w.val<uint64_t>(d);
    w.val<uint64_t>(b.size());
    w.put(b.data(), b.size());
  };
  for (int k = 0; k < s->l; ++k) {
    w.val<int32_t>(s->t);
    for (int i = 0; i < s->t; ++i) {
      const size_t slice = static_cast<size_t>(k) * s->t + i;
      poly(a_host.data() + slice * d * cw);
      w.val<uint64_t>(s->k);
      for (int j = 0; j < s->k; ++j) {
        poly(s->t_vec_h_raw.data() + (slice * s->k + j) * d * cw);
      }
    }
  }
  // 4. second_dim_a.
  const uint64_t nsd = s->second_dim_a_raw.size() / (d * cw);
  w.val<uint64_t>(nsd);
  for (uint64_t j = 0; j < nsd; ++j) poly(s->second_dim_a_raw.data() + j * d * cw);
  *size = w.off;
  if (dst != nullptr && w.off > cap) {
    return Err(INSPIRE_RESOURCE_EXHAUSTED, "image buffer too small.");
  }
  return Status{};
}

// ---------------------------------------------------------------------------
// PirPreprocessedData as protobuf messages (crypto/proto/pir_server.proto,
// crypto/proto/rlwe.proto), the way SerializePirPreprocessedData /
// DeserializePirPreprocessedData and the per-shard directory form write and
// read them (crypto/pir/server/pir_preprocessed_data.h:52-267), through
// Matrix::ToProto / FromProto (crypto/matrix.cc:478-520) and
// Polynomial::ToProto / CreateFromProto (crypto/polynomial.cc:208-252,
// 562-590). Protobuf wire format: each field is a varint key
// (number << 3 | wire type) followed by a varint (type 0) or by a varint
// length and that many bytes (type 2); a writer emits fields in number order
// and, with the explicit presence of these messages, every scalar it set.
// The matrices' bytes go to the GPU straight from the parsed buffer.
// ---------------------------------------------------------------------------
struct PbSpan {
  const uint8_t* p = nullptr;
  size_t n = 0;
};

struct PbReader {
  const uint8_t* p;
  size_t n;
  size_t off = 0;
  bool ok = true;
  bool Varint(uint64_t* v) {
    uint64_t x = 0;
    for (int sh = 0; sh < 64; sh += 7) {
      if (off >= n) break;
      const uint8_t b = p[off++];
      x |= static_cast<uint64_t>(b & 0x7F) << sh;
      if ((b & 0x80) == 0) {
        *v = x;
        return true;
      }
    }
    ok = false;
    return false;
  }
  // The next field; false at the end of the message or on malformed input
  // (then ok is false). Fixed-width fields are skipped.
  bool Next(int* num, uint64_t* v, PbSpan* bytes) {
    if (!ok || off >= n) return false;
    uint64_t key = 0;
    if (!Varint(&key)) return false;
    *num = static_cast<int>(key >> 3);
    switch (key & 7) {
      case 0:
        return Varint(v);
      case 1:
      case 5: {
        const size_t w = (key & 7) == 1 ? 8 : 4;
        if (n - off < w) break;
        off += w;
        *num = -1;
        return true;
      }
      case 2: {
        uint64_t len = 0;
        if (!Varint(&len) || len > n - off) break;
        bytes->p = p + off;
        bytes->n = len;
        off += len;
        return true;
      }
      default:
        break;
    }
    ok = false;
    return false;
  }
};

struct PbMatrix {
  PbSpan bytes;
  bool has_data = false, has_condensed = false, is_condensed = false;
  int64_t rows = 0, cols = 0, orig = 0;
};

Status PbBad(const char* what) { return Err(INSPIRE_INVALID_ARGUMENT, what); }

// Matrix::FromProto's checks, and the element columns of the matrix.
Status ParseMatrix(PbSpan m, size_t es, PbMatrix* out, int64_t* elem_cols) {
  PbReader r{m.p, m.n};
  int num = 0;
  uint64_t v = 0;
  PbSpan b;
  while (r.Next(&num, &v, &b)) {
    switch (num) {
      case 1: out->bytes = b; out->has_data = true; out->has_condensed = false; break;
      case 2: out->bytes = b; out->has_condensed = true; out->has_data = false; break;
      case 3: out->rows = static_cast<int32_t>(v); break;
      case 4: out->cols = static_cast<int32_t>(v); break;
      case 5: out->is_condensed = v != 0; break;
      case 6: out->orig = static_cast<int32_t>(v); break;
      default: break;
    }
  }
  if (!r.ok) return PbBad("Failed to parse PirPreprocessedData.");
  if (out->is_condensed && out->has_data) {
    return PbBad("Condensed matrix cannot have normal data set.");
  }
  if (!out->is_condensed && out->has_condensed) {
    return PbBad("Normal matrix cannot have condensed data set.");
  }
  if (out->bytes.n % (out->is_condensed ? 8 : es) != 0) {
    return PbBad(out->is_condensed ? "Invalid serialized condensed_data size."
                                   : "Invalid serialized data size.");
  }
  *elem_cols = out->is_condensed ? out->cols * 8 / static_cast<int64_t>(es) : out->cols;
  if (static_cast<size_t>(out->rows) * *elem_cols * es != out->bytes.n) {
    return PbBad("Invalid serialized data size.");
  }
  return Status{};
}

// Polynomial::CreateFromProto: d coefficients of log_q bits, appended to out
// as CoeffType words.
Status ParsePoly(PbSpan m, int d, int log_q, int cb, std::vector<uint8_t>* out) {
  PbReader r{m.p, m.n};
  int num = 0;
  uint64_t v = 0;
  PbSpan b, enc;
  while (r.Next(&num, &v, &b)) {
    if (num == 1) enc = b;
  }
  if (!r.ok) return PbBad("Failed to parse PirPreprocessedData.");
  if (log_q <= 0 || log_q > cb) return PbBad("Invalid log_modulus.");
  if (enc.n == 0) return PbBad("Empty serialized polynomial.");
  if (enc.n != (static_cast<size_t>(d) * log_q + 7) / 8) {
    return PbBad("Unexpected serialized size.");
  }
  UnpackCoeffs(enc.p, enc.n, d, log_q, cb, out);
  return Status{};
}

// The material of one shard as it comes out of the messages.
struct PbShard {
  PbMatrix db;
  int64_t db_cols = 0;
  std::vector<PbMatrix> packs;
  std::vector<int64_t> pack_cols;
};

// PreprocessMatrixPackOutput: a_tilde_agg (1), matrix (2), t_vec_h (3).
Status ParseOutput(PbSpan m, const inspire_pir_params* prm, PbShard* sh,
                   std::vector<uint8_t>* a_tilde, std::vector<uint8_t>* t_vec_h,
                   int64_t* th_count) {
  const int d = 1 << prm->log_degree;
  PbReader r{m.p, m.n};
  int num = 0;
  uint64_t v = 0;
  PbSpan b;
  bool have_a = false, have_m = false;
  while (r.Next(&num, &v, &b)) {
    if (num == 1) {
      RETURN_IF_ERROR(ParsePoly(b, d, prm->log_modulus, prm->coeff_bits, a_tilde));
      have_a = true;
    } else if (num == 2) {
      sh->packs.emplace_back();
      sh->pack_cols.push_back(0);
      RETURN_IF_ERROR(ParseMatrix(b, elem_size(prm->mat_kind), &sh->packs.back(),
                                  &sh->pack_cols.back()));
      have_m = true;
    } else if (num == 3) {
      RETURN_IF_ERROR(ParsePoly(b, d, prm->log_modulus, prm->coeff_bits, t_vec_h));
      ++*th_count;
    }
  }
  if (!r.ok) return PbBad("Failed to parse PirPreprocessedData.");
  if (!have_a) return PbBad("Empty serialized polynomial.");
  if (!have_m) return PbBad("Preprocessed output without a matrix.");
  return Status{};
}

// Builds the server from parsed shards: the matrices are copied into one
// device buffer each (vertical concatenation), the polynomials go through
// CreateServer.
Status ServerFromShards(const inspire_pir_params* prm, std::vector<PbShard>& shards,
                        const std::vector<uint8_t>& a_tilde, int64_t a_count,
                        const std::vector<uint8_t>& t_vec_h, int64_t th_count,
                        const std::vector<uint8_t>& sda, int64_t sda_count,
                        std::unique_ptr<inspire_pir_server>* out) {
  if (prm == nullptr) return PbBad("params is null.");
  const int l = prm->entry_size_multiple;
  const int t = prm->interpolation_degree;
  if (static_cast<int>(shards.size()) != l) return PbBad("db_matrices size mismatch.");
  const size_t es = elem_size(prm->db_kind), ms = elem_size(prm->mat_kind);
  int64_t db_rows = 0, pack_rows = 0;
  const int64_t db_cols = shards.empty() ? 0 : shards[0].db_cols;
  const int64_t pack_cols = shards.empty() || shards[0].packs.empty() ? 0 : shards[0].pack_cols[0];
  for (auto& sh : shards) {
    if (sh.db_cols != db_cols) {
      return PbBad("All DB matrices must have the same number of columns.");
    }
    if (static_cast<int>(sh.packs.size()) != t) {
      return PbBad("Preprocessed outputs must be of length t.");
    }
    db_rows += sh.db.rows;
    for (size_t i = 0; i < sh.packs.size(); ++i) {
      if (sh.pack_cols[i] != pack_cols) {
        return PbBad("All pack matrices must have the same number of columns.");
      }
      pack_rows += sh.packs[i].rows;
    }
  }
  DevBuf db, pack;
  RETURN_IF_ERROR(db.Alloc(static_cast<size_t>(db_rows) * db_cols * es));
  RETURN_IF_ERROR(pack.Alloc(static_cast<size_t>(pack_rows) * pack_cols * ms));
  size_t db_off = 0, pack_off = 0;
  for (auto& sh : shards) {
    if (sh.db.bytes.n > 0) {
      RETURN_IF_ERROR(Cuda(cudaMemcpy(db.get<uint8_t>() + db_off, sh.db.bytes.p, sh.db.bytes.n,
                                      cudaMemcpyHostToDevice),
                           "DB upload"));
    }
    db_off += sh.db.bytes.n;
    for (auto& pm : sh.packs) {
      if (pm.bytes.n > 0) {
        RETURN_IF_ERROR(Cuda(cudaMemcpy(pack.get<uint8_t>() + pack_off, pm.bytes.p, pm.bytes.n,
                                        cudaMemcpyHostToDevice),
                             "pack matrix upload"));
      }
      pack_off += pm.bytes.n;
    }
  }
  RETURN_IF_ERROR(CreateServer(prm, db.get(), db_rows, db_cols, pack.get(), pack_rows,
                               pack_cols, a_tilde.data(), a_count, t_vec_h.data(), th_count,
                               sda.data(), sda_count, out, &db, &pack));
  if (!shards.empty()) {
    (*out)->db_condensed = shards[0].db.is_condensed;
    (*out)->db_orig_cols = static_cast<int32_t>(shards[0].db.orig);
    (*out)->orig_from_file = true;
    (*out)->pack_condensed = !shards[0].packs.empty() && shards[0].packs[0].is_condensed;
  }
  return Status{};
}

// DeserializePirPreprocessedData + PirServer::Create from one serialized
// proto::PirPreprocessedData.
Status LoadPreprocessed(const inspire_pir_params* prm, const uint8_t* buf, size_t size,
                        std::unique_ptr<inspire_pir_server>* out) {
  if (prm == nullptr || (buf == nullptr && size > 0)) {
    return PbBad("Failed to parse PirPreprocessedData from file.");
  }
  const int d = 1 << prm->log_degree;
  std::vector<PbShard> shards;
  std::vector<uint8_t> a_tilde, t_vec_h, sda;
  int64_t a_count = 0, th_count = 0, sda_count = 0;
  size_t db_seen = 0, out_seen = 0;
  PbReader r{buf, size};
  int num = 0;
  uint64_t v = 0;
  PbSpan b;
  while (r.Next(&num, &v, &b)) {
    if (num == 1) {  // db_matrices
      if (shards.size() <= db_seen) shards.resize(db_seen + 1);
      RETURN_IF_ERROR(ParseMatrix(b, elem_size(prm->db_kind), &shards[db_seen].db,
                                  &shards[db_seen].db_cols));
      ++db_seen;
    } else if (num == 2) {  // preprocessed_outputs: ShardPreprocessedOutputs
      if (shards.size() <= out_seen) shards.resize(out_seen + 1);
      PbReader rs{b.p, b.n};
      int n2 = 0;
      uint64_t v2 = 0;
      PbSpan o;
      while (rs.Next(&n2, &v2, &o)) {
        if (n2 == 1) {
          RETURN_IF_ERROR(ParseOutput(o, prm, &shards[out_seen], &a_tilde, &t_vec_h, &th_count));
          ++a_count;
        }
      }
      if (!rs.ok) return PbBad("Failed to parse PirPreprocessedData from file.");
      ++out_seen;
    } else if (num == 3) {  // second_dim_a
      RETURN_IF_ERROR(ParsePoly(b, d, prm->log_modulus, prm->coeff_bits, &sda));
      ++sda_count;
    }
  }
  if (!r.ok) return PbBad("Failed to parse PirPreprocessedData from file.");
  if (db_seen != out_seen) return PbBad("preprocessed_outputs size mismatch.");
  return ServerFromShards(prm, shards, a_tilde, a_count, t_vec_h, th_count, sda, sda_count,
                          out);
}

// --- writer ---
void PbPutVarint(std::vector<uint8_t>* o, uint64_t v) {
  while (v >= 0x80) {
    o->push_back(static_cast<uint8_t>(v | 0x80));
    v >>= 7;
  }
  o->push_back(static_cast<uint8_t>(v));
}
void PbPutBytes(std::vector<uint8_t>* o, int num, const uint8_t* p, size_t n) {
  PbPutVarint(o, static_cast<uint64_t>(num) << 3 | 2);
  PbPutVarint(o, n);
  o->insert(o->end(), p, p + n);
}
void PbPutInt(std::vector<uint8_t>* o, int num, int64_t v) {
  PbPutVarint(o, static_cast<uint64_t>(num) << 3);
  PbPutVarint(o, static_cast<uint64_t>(v));  // int32 fields: sign-extended
}

// Matrix::ToProto of rows x elem_cols elements at dev (device).
Status PutMatrix(std::vector<uint8_t>* o, int num, const uint8_t* dev, int64_t rows,
                 int64_t elem_cols, size_t es, bool condensed, int64_t orig) {
  std::vector<uint8_t> m;
  const size_t bytes = static_cast<size_t>(rows) * elem_cols * es;
  std::vector<uint8_t> host(bytes);
  if (bytes > 0) {
    RETURN_IF_ERROR(Cuda(cudaMemcpy(host.data(), dev, bytes, cudaMemcpyDeviceToHost),
                         "matrix download"));
    PbPutBytes(&m, condensed ? 2 : 1, host.data(), bytes);
  }
  PbPutInt(&m, 3, rows);
  PbPutInt(&m, 4, condensed ? elem_cols * static_cast<int64_t>(es) / 8 : elem_cols);
  PbPutInt(&m, 5, condensed ? 1 : 0);
  PbPutInt(&m, 6, orig);
  PbPutBytes(o, num, m.data(), m.size());
  return Status{};
}

// Polynomial::ToProto (log_q bits per coefficient) as field `num`.
void PutPoly(std::vector<uint8_t>* o, int num, const uint8_t* words, int d, int log_q, int cb) {
  const std::vector<uint8_t> enc = PackCoeffs(words, d, log_q, cb);
  std::vector<uint8_t> m;
  PbPutBytes(&m, 1, enc.data(), enc.size());
  PbPutBytes(o, num, m.data(), m.size());
}

// One shard's messages: its DB matrix (field db_num) and its outputs
// (field out_num, each a PreprocessMatrixPackOutput).
Status PutShard(inspire_pir_server* s, int k, const std::vector<uint8_t>& a_host,
                std::vector<uint8_t>* db_part, int db_num, std::vector<uint8_t>* out_part,
                int out_num) {
  const int d = s->d, t = s->t, cb = s->prm.coeff_bits;
  const size_t cw = cb / 8;
  const size_t es = elem_size(s->prm.db_kind), ms = elem_size(s->prm.mat_kind);
  const int64_t shard_rows = static_cast<int64_t>(t) * d;
  const bool dcond = s->db_condensed && (s->db_cols * es) % 8 == 0;
  RETURN_IF_ERROR(PutMatrix(db_part, db_num,
                            s->db.get<uint8_t>() + static_cast<size_t>(k) * shard_rows * s->db_cols * es,
                            shard_rows, s->db_cols, es, dcond,
                            s->orig_from_file ? s->db_orig_cols : s->db_cols));
  const bool pcond = s->pack_condensed && (s->pack_cols * ms) % 8 == 0;
  for (int i = 0; i < t; ++i) {
    const size_t slice = static_cast<size_t>(k) * t + i;
    std::vector<uint8_t> m;
    PutPoly(&m, 1, a_host.data() + slice * d * cw, d, s->prm.log_modulus, cb);
    RETURN_IF_ERROR(PutMatrix(&m, 2,
                              s->pack.get<uint8_t>() + slice * d * s->pack_cols * ms, d,
                              s->pack_cols, ms, pcond, s->pack_cols));
    for (int j = 0; j < s->k; ++j) {
      PutPoly(&m, 3, s->t_vec_h_raw.data() + (slice * s->k + j) * d * cw, d,
              s->prm.log_modulus, cb);
    }
    PbPutBytes(out_part, out_num, m.data(), m.size());
  }
  return Status{};
}

Status SavePreprocessed(inspire_pir_server* s, std::vector<uint8_t>* out) {
  const int d = s->d, cb = s->prm.coeff_bits;
  const size_t cw = cb / 8;
  std::vector<uint8_t> a_host(static_cast<size_t>(s->l) * s->t * d * cw);
  RETURN_IF_ERROR(Cuda(cudaMemcpy(a_host.data(), s->a_tilde.get(), a_host.size(),
                                  cudaMemcpyDeviceToHost),
                       "a_tilde download"));
  std::vector<uint8_t> dbs, outs;
  for (int k = 0; k < s->l; ++k) {
    std::vector<uint8_t> shard_outs;
    RETURN_IF_ERROR(PutShard(s, k, a_host, &dbs, 1, &shard_outs, 1));
    PbPutBytes(&outs, 2, shard_outs.data(), shard_outs.size());
  }
  out->clear();
  out->insert(out->end(), dbs.begin(), dbs.end());
  out->insert(out->end(), outs.begin(), outs.end());
  const size_t nsd = s->second_dim_a_raw.size() / (d * cw);
  for (size_t j = 0; j < nsd; ++j) {
    PutPoly(out, 3, s->second_dim_a_raw.data() + j * d * cw, d, s->prm.log_modulus, cb);
  }
  return Status{};
}

Status ReadWholeFile(const std::string& path, std::vector<uint8_t>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (f == nullptr) return Err(INSPIRE_INTERNAL, "Failed to read file: " + path);
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  Status st;
  if (len < 0) {
    st = Err(INSPIRE_INTERNAL, "Failed to read file: " + path);
  } else {
    out->resize(static_cast<size_t>(len));
    if (len > 0 && std::fread(out->data(), 1, len, f) != static_cast<size_t>(len)) {
      st = Err(INSPIRE_INTERNAL, "Failed to read file: " + path);
    }
  }
  std::fclose(f);
  return st;
}

Status WriteWholeFile(const std::string& path, const std::vector<uint8_t>& data) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (f == nullptr) return Err(INSPIRE_INTERNAL, "Failed to open file for writing: " + path);
  Status st;
  if (!data.empty() && std::fwrite(data.data(), 1, data.size(), f) != data.size()) {
    st = Err(INSPIRE_INTERNAL, "Error writing to file: " + path);
  }
  std::fclose(f);
  return st;
}

}  // namespace

// ---------------------------------------------------------------------------
// Interface for the native serving loop (server_api.h).
// ---------------------------------------------------------------------------
ServerGeometry GetGeometry(const inspire_pir_server* s) {
  ServerGeometry g;
  g.db_cols = s->db_cols;
  g.interpolated_rows = s->interpolated_rows;
  g.d = s->d;
  g.l = s->l;
  g.nsd = s->t > 1 ? 2 * s->ne : 0;
  g.npk = 2 * s->k;
  g.word_bytes = static_cast<int>(Words(s->prm.coeff_bits));
  g.tensor = s->limb != nullptr;
  return g;
}

int64_t BatchWorkspaceBytes(const inspire_pir_server* s, int max_batch) {
  return WorkspaceBytes(s, max_batch);
}

int NewBatchWorkspace(inspire_pir_server* s, int max_batch, Workspace** out,
                      std::string* err) {
  *out = nullptr;
  std::unique_ptr<Workspace> w(new Workspace());
  Status st = InitWorkspace(w.get());
  if (st.ok()) st = EnsureWorkspace(s, w.get(), max_batch);
  if (st.ok() && w->limb) {
    st = Cuda(s->limb->Reserve(w->limb.get(), max_batch), "tensor engine scratch");
  }
  if (!st.ok()) {
    *err = st.msg;
    return st.code;
  }
  *out = w.release();
  return INSPIRE_OK;
}

void DeleteBatchWorkspace(Workspace* w) {
  if (w == nullptr) return;
  cudaStreamSynchronize(w->stream);
  delete w;
}

int ValidateFirstDim(const inspire_pir_server* s, int64_t first_dim_len,
                     std::string* err) {
  Status st = ValidateRequest(s, first_dim_len, 2 * s->ne, 2 * s->k);
  if (!st.ok()) *err = st.msg;
  return st.code;
}

int LaunchBatch(inspire_pir_server* s, Workspace* w, const RequestSegment* segs,
                int nseg, int engine, std::string* err) {
  const size_t cw = Words(s->prm.coeff_bits);
  const size_t d = s->d;
  const size_t fd = s->db_cols * cw, sd = 2 * s->ne * d * cw,
               pk = 2 * s->k * d * cw, rs = 2 * s->l * d * cw;
  const cudaStream_t st = w->stream;
  int batch = 0;
  Status status;
  auto copy = [&](void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    if (status.ok() && bytes > 0) {
      status = Cuda(cudaMemcpyAsync(dst, src, bytes, kind, st), "request copy");
    }
  };
  for (int i = 0; i < nseg; ++i) {
    const size_t n = segs[i].count;
    copy(w->q1.get<char>() + batch * fd, segs[i].first_dim, n * fd,
         cudaMemcpyHostToDevice);
    if (s->t > 1) {
      copy(w->sdim.get<char>() + batch * sd, segs[i].second_dim, n * sd,
           cudaMemcpyHostToDevice);
    }
    copy(w->pkey.get<char>() + batch * pk, segs[i].packing_key, n * pk,
         cudaMemcpyHostToDevice);
    batch += segs[i].count;
  }
  if (status.ok() && (batch <= 0 || batch > w->cap)) {
    status = Err(INSPIRE_INVALID_ARGUMENT, "batch exceeds the workspace capacity.");
  }
  engine = ResolveEngine(s, engine, batch);
  if (status.ok()) {
    status = AnswerOnDevice(s, w, batch, w->q1.get(), w->pkey.get(), w->sdim.get(),
                            w->resp.get(), engine, st, false);
  }
  int off = 0;
  for (int i = 0; i < nseg; ++i) {
    copy(segs[i].responses, w->resp.get<char>() + off * rs, segs[i].count * rs,
         cudaMemcpyDeviceToHost);
    off += segs[i].count;
  }
  if (status.ok()) status = Cuda(cudaEventRecord(w->done, st), "cudaEventRecord");
  if (!status.ok()) *err = status.msg;
  return status.code;
}

int QueryBatch(Workspace* w) {
  const cudaError_t e = cudaEventQuery(w->done);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return -1;
}

int FinishBatch(inspire_pir_server* s, Workspace* w, int engine, std::string* err) {
  Status st = Cuda(cudaEventSynchronize(w->done), "answer");
  if (st.ok() && engine != INSPIRE_ENGINE_PLAIN && s->limb &&
      s->limb->CheckError() != 0) {
    st = Err(INSPIRE_INTERNAL, "tensor engine pipeline timed out");
  }
  if (!st.ok()) *err = st.msg;
  return st.code;
}

}  // namespace inspire

// ---------------------------------------------------------------------------
// C ABI.
// ---------------------------------------------------------------------------
using inspire::Err;
using inspire::Report;
using inspire::Status;

extern "C" {

int inspire_pir_server_create(const inspire_pir_params* params, const void* db,
                              int64_t db_rows, int64_t db_cols,
                              const void* pack, int64_t pack_rows,
                              int64_t pack_cols, const void* a_tilde_agg,
                              int64_t a_tilde_agg_count, const void* t_vec_h,
                              int64_t t_vec_h_count, const void* second_dim_a,
                              int64_t second_dim_a_count,
                              inspire_pir_server** out, char* err,
                              size_t err_len) {
  if (out == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "out is null."), err, err_len);
  }
  *out = nullptr;
  std::unique_ptr<inspire_pir_server> s;
  Status st = inspire::CreateServer(params, db, db_rows, db_cols, pack,
                                    pack_rows, pack_cols, a_tilde_agg,
                                    a_tilde_agg_count, t_vec_h, t_vec_h_count,
                                    second_dim_a, second_dim_a_count, &s);
  if (st.ok()) *out = s.release();
  return Report(st, err, err_len);
}

void inspire_pir_server_destroy(inspire_pir_server* server) { delete server; }

int inspire_pir_server_load(const inspire_pir_params* params, const void* buffer,
                            size_t size, inspire_pir_server** out, char* err,
                            size_t err_len) {
  using namespace inspire;
  if (out == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "out is null."), err, err_len);
  }
  *out = nullptr;
  std::unique_ptr<inspire_pir_server> s;
  Status st = LoadImage(params, static_cast<const uint8_t*>(buffer), size, &s);
  if (st.ok()) *out = s.release();
  return Report(st, err, err_len);
}

int inspire_pir_server_load_file(const inspire_pir_params* params, const char* path,
                                 inspire_pir_server** out, char* err,
                                 size_t err_len) {
  using namespace inspire;
  if (out == nullptr || path == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "out and path must be set."), err,
                  err_len);
  }
  *out = nullptr;
  // LoadFromFile (pir_server.cc:782-791): the whole file into (pinned)
  // host memory, then LoadFromBuffer.
  FILE* f = std::fopen(path, "rb");
  if (f == nullptr) return Report(Err(INSPIRE_INTERNAL, "Failed to read file."), err, err_len);
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  void* host = nullptr;
  Status st;
  if (len < 0 || cudaMallocHost(&host, len > 0 ? len : 1) != cudaSuccess) {
    st = Err(INSPIRE_INTERNAL, "Failed to read file.");
  } else if (len > 0 && std::fread(host, 1, len, f) != static_cast<size_t>(len)) {
    st = Err(INSPIRE_INTERNAL, "Failed to read file.");
  }
  std::fclose(f);
  std::unique_ptr<inspire_pir_server> s;
  if (st.ok()) st = LoadImage(params, static_cast<const uint8_t*>(host), len, &s);
  if (host) cudaFreeHost(host);
  if (st.ok()) *out = s.release();
  return Report(st, err, err_len);
}

int inspire_pir_server_load_preprocessed(const inspire_pir_params* params,
                                         const void* buffer, size_t size,
                                         inspire_pir_server** out, char* err,
                                         size_t err_len) {
  using namespace inspire;
  if (out == nullptr) return Report(Err(INSPIRE_INVALID_ARGUMENT, "out is null."), err, err_len);
  *out = nullptr;
  std::unique_ptr<inspire_pir_server> s;
  Status st = LoadPreprocessed(params, static_cast<const uint8_t*>(buffer), size, &s);
  if (st.ok()) *out = s.release();
  return Report(st, err, err_len);
}

int inspire_pir_server_load_preprocessed_dir(const inspire_pir_params* params,
                                             const char* dir, inspire_pir_server** out,
                                             char* err, size_t err_len) {
  using namespace inspire;
  if (out == nullptr || dir == nullptr || params == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "params, dir and out must be set."), err,
                  err_len);
  }
  *out = nullptr;
  // LoadPirPreprocessedDataFromDirectory (pir_preprocessed_data.h:203-267):
  // metadata.bin (second_dim_a), then shard_<i>.bin per shard.
  const std::string base(dir);
  const int d = 1 << params->log_degree;
  std::vector<uint8_t> meta;
  Status st = ReadWholeFile(base + "/metadata.bin", &meta);
  std::vector<uint8_t> sda;
  int64_t sda_count = 0;
  if (st.ok()) {
    PbReader r{meta.data(), meta.size()};
    int num = 0;
    uint64_t v = 0;
    PbSpan b;
    while (st.ok() && r.Next(&num, &v, &b)) {
      if (num == 1) {
        st = ParsePoly(b, d, params->log_modulus, params->coeff_bits, &sda);
        ++sda_count;
      }
    }
    if (st.ok() && !r.ok) {
      st = Err(INSPIRE_INVALID_ARGUMENT, "Failed to parse PirPreprocessedMetadata.");
    }
  }
  const int l = params->entry_size_multiple;
  std::vector<std::vector<uint8_t>> files(l > 0 ? l : 0);
  std::vector<PbShard> shards(files.size());
  std::vector<uint8_t> a_tilde, t_vec_h;
  int64_t a_count = 0, th_count = 0;
  for (int i = 0; st.ok() && i < l; ++i) {
    st = ReadWholeFile(base + "/shard_" + std::to_string(i) + ".bin", &files[i]);
    if (!st.ok()) break;
    PbReader r{files[i].data(), files[i].size()};
    int num = 0;
    uint64_t v = 0;
    PbSpan b;
    bool have_db = false;
    while (st.ok() && r.Next(&num, &v, &b)) {
      if (num == 1) {
        st = ParseMatrix(b, elem_size(params->db_kind), &shards[i].db, &shards[i].db_cols);
        have_db = true;
      } else if (num == 2) {
        st = ParseOutput(b, params, &shards[i], &a_tilde, &t_vec_h, &th_count);
        ++a_count;
      }
    }
    if (st.ok() && (!r.ok || !have_db)) {
      st = Err(INSPIRE_INVALID_ARGUMENT,
               "Failed to parse PirPreprocessedShard " + std::to_string(i));
    }
  }
  std::unique_ptr<inspire_pir_server> s;
  if (st.ok()) {
    st = ServerFromShards(params, shards, a_tilde, a_count, t_vec_h, th_count, sda, sda_count,
                          &s);
  }
  if (st.ok()) *out = s.release();
  return Report(st, err, err_len);
}

int inspire_pir_server_save_preprocessed(inspire_pir_server* server, void* buffer,
                                         size_t capacity, size_t* size, char* err,
                                         size_t err_len) {
  using namespace inspire;
  if (server == nullptr || size == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server and size must be set."), err,
                  err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  std::vector<uint8_t> bytes;
  Status st = SavePreprocessed(server, &bytes);
  if (st.ok()) {
    *size = bytes.size();
    if (buffer != nullptr) {
      if (capacity < bytes.size()) {
        st = Err(INSPIRE_RESOURCE_EXHAUSTED, "buffer too small.");
      } else {
        std::memcpy(buffer, bytes.data(), bytes.size());
      }
    }
  }
  return Report(st, err, err_len);
}

int inspire_pir_server_save_preprocessed_dir(inspire_pir_server* server, const char* dir,
                                             char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || dir == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server and dir must be set."), err, err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  // SavePirPreprocessedDataToDirectory (pir_preprocessed_data.h:141-201).
  const std::string base(dir);
  const int d = server->d, cb = server->prm.coeff_bits;
  const size_t cw = cb / 8;
  std::vector<uint8_t> meta;
  const size_t nsd = server->second_dim_a_raw.size() / (d * cw);
  for (size_t j = 0; j < nsd; ++j) {
    PutPoly(&meta, 1, server->second_dim_a_raw.data() + j * d * cw, d,
            server->prm.log_modulus, cb);
  }
  Status st = WriteWholeFile(base + "/metadata.bin", meta);
  std::vector<uint8_t> a_host(static_cast<size_t>(server->l) * server->t * d * cw);
  if (st.ok()) {
    st = Cuda(cudaMemcpy(a_host.data(), server->a_tilde.get(), a_host.size(),
                         cudaMemcpyDeviceToHost),
              "a_tilde download");
  }
  for (int k = 0; st.ok() && k < server->l; ++k) {
    std::vector<uint8_t> shard;
    std::vector<uint8_t> outs;
    st = PutShard(server, k, a_host, &shard, 1, &outs, 2);
    if (st.ok()) {
      shard.insert(shard.end(), outs.begin(), outs.end());
      st = WriteWholeFile(base + "/shard_" + std::to_string(k) + ".bin", shard);
    }
  }
  return Report(st, err, err_len);
}

int inspire_pir_server_save(inspire_pir_server* server, void* buffer,
                            size_t capacity, size_t* size, char* err,
                            size_t err_len) {
  using namespace inspire;
  if (server == nullptr || size == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server and size must be set."), err,
                  err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  return Report(SaveImage(server, static_cast<uint8_t*>(buffer), capacity, size), err,
                err_len);
}

int inspire_pir_server_save_file(inspire_pir_server* server, const char* path,
                                 char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || path == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server and path must be set."), err,
                  err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  size_t size = 0;
  Status st = SaveImage(server, nullptr, 0, &size);
  void* host = nullptr;
  if (st.ok() && cudaMallocHost(&host, size > 0 ? size : 1) != cudaSuccess) {
    st = Err(INSPIRE_RESOURCE_EXHAUSTED, "pinned staging allocation failed.");
  }
  if (st.ok()) st = SaveImage(server, static_cast<uint8_t*>(host), size, &size);
  if (st.ok()) {
    FILE* f = std::fopen(path, "wb");
    if (f == nullptr) {
      st = Err(INSPIRE_INTERNAL, std::string("Failed to open file for writing: ") + path);
    } else {
      if (std::fwrite(host, 1, size, f) != size) {
        st = Err(INSPIRE_INTERNAL, std::string("Error writing to file: ") + path);
      }
      std::fclose(f);
    }
  }
  if (host) cudaFreeHost(host);
  return Report(st, err, err_len);
}

int inspire_pir_process_response(inspire_pir_server* server,
                                 const void* first_dim, int64_t first_dim_len,
                                 const void* second_dim,
                                 int64_t second_dim_count,
                                 const void* packing_key,
                                 int64_t packing_key_count, void* response,
                                 char* err, size_t err_len) {
  return inspire_pir_process_batch(server, 1, first_dim, first_dim_len,
                                   second_dim, second_dim_count, packing_key,
                                   packing_key_count, response,
                                   INSPIRE_ENGINE_PLAIN, err, err_len);
}

int inspire_pir_process_batch(inspire_pir_server* server, int32_t batch,
                              const void* first_dim, int64_t first_dim_len,
                              const void* second_dim, int64_t second_dim_count,
                              const void* packing_key,
                              int64_t packing_key_count, void* responses,
                              int32_t engine, char* err, size_t err_len) {
  if (server == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null."), err, err_len);
  }
  engine = inspire::ResolveEngine(server, engine, batch);
  return Report(inspire::ProcessHostBatch(server, batch, first_dim,
                                          first_dim_len, second_dim,
                                          second_dim_count, packing_key,
                                          packing_key_count, responses, engine),
                err, err_len);
}

int inspire_pir_process_batch_device(inspire_pir_server* server,
                                     int32_t batch, const void* first_dim,
                                     int64_t first_dim_len,
                                     const void* second_dim,
                                     int64_t second_dim_count,
                                     const void* packing_key,
                                     int64_t packing_key_count,
                                     void* responses, int32_t engine,
                                     void* stream, char* err, size_t err_len) {
  if (server == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null."), err, err_len);
  }
  if (batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "batch must be positive."), err,
                  err_len);
  }
  engine = inspire::ResolveEngine(server, engine, batch);
  Status st = inspire::ValidateRequest(server, first_dim_len, second_dim_count,
                                       packing_key_count);
  if (!st.ok()) return Report(st, err, err_len);
  std::lock_guard<std::mutex> lock(server->mu);
  inspire::Workspace* ws = server->ws0.get();
  st = inspire::EnsureWorkspace(server, ws, batch);
  if (!st.ok()) return Report(st, err, err_len);
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  st = inspire::DeviceFirstDim(server, ws, batch, &first_dim, first_dim_len, cs);
  if (st.ok()) {
    st = inspire::AnswerOnDevice(server, ws, batch, first_dim, packing_key,
                                 second_dim, responses, engine, cs, false);
  }
  return Report(st, err, err_len);
}

int inspire_pir_pack_batch_device(inspire_pir_server* server, int32_t batch,
                                  const void* first_dim, int64_t first_dim_len,
                                  const void* packing_key,
                                  int64_t packing_key_count, void* out,
                                  int32_t engine, void* stream, char* err,
                                  size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null or batch <= 0."),
                  err, err_len);
  }
  engine = ResolveEngine(server, engine, batch);
  Status st = ValidateRequest(server, first_dim_len, 2 * server->ne,
                              packing_key_count);
  if (!st.ok()) return Report(st, err, err_len);
  std::lock_guard<std::mutex> lock(server->mu);
  Workspace* ws = server->ws0.get();
  st = EnsureWorkspace(server, ws, batch);
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  if (st.ok()) st = DeviceFirstDim(server, ws, batch, &first_dim, first_dim_len, cs);
  if (st.ok()) st = PackOnDevice(server, ws, batch, first_dim, packing_key, out, engine, cs);
  return Report(st, err, err_len);
}

int inspire_pir_external_product_device(inspire_pir_server* server,
                                        int32_t batch, const void* ct,
                                        const void* rgsw, void* out,
                                        void* stream, char* err,
                                        size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0 || ct == nullptr || rgsw == nullptr ||
      out == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "server, ct, rgsw and out must be set and batch positive."),
                  err, err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  Workspace* ws = server->ws0.get();
  Status st = EnsureWorkspace(server, ws, batch);
  if (st.ok()) {
    st = ExternalOnDevice(server, ws, batch, ct, rgsw, out,
                          static_cast<cudaStream_t>(stream));
  }
  return Report(st, err, err_len);
}

int inspire_graph_begin(void* stream, char* err, size_t err_len) {
  using namespace inspire;
  if (stream == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "graph capture needs a created stream, not the legacy "
                      "default stream."),
                  err, err_len);
  }
  return Report(Cuda(cudaStreamBeginCapture(static_cast<cudaStream_t>(stream),
                                            cudaStreamCaptureModeThreadLocal),
                     "cudaStreamBeginCapture"),
                err, err_len);
}

int inspire_graph_end(void* stream, inspire_graph** out, char* err,
                      size_t err_len) {
  using namespace inspire;
  if (stream == nullptr || out == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "stream and out must be set."),
                  err, err_len);
  }
  *out = nullptr;
  cudaGraph_t graph = nullptr;
  Status st = Cuda(cudaStreamEndCapture(static_cast<cudaStream_t>(stream), &graph),
                   "cudaStreamEndCapture (a call inside the capture failed or "
                   "allocated)");
  cudaGraphExec_t exec = nullptr;
  if (st.ok()) st = Cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
  if (graph) cudaGraphDestroy(graph);
  if (!st.ok()) return Report(st, err, err_len);
  *out = new inspire_graph{exec};
  return INSPIRE_OK;
}

int inspire_graph_launch(inspire_graph* graph, void* stream, char* err,
                         size_t err_len) {
  using namespace inspire;
  if (graph == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "graph is null."), err, err_len);
  }
  return Report(Cuda(cudaGraphLaunch(graph->exec, static_cast<cudaStream_t>(stream)),
                     "cudaGraphLaunch"),
                err, err_len);
}

void inspire_graph_destroy(inspire_graph* graph) {
  if (graph == nullptr) return;
  if (graph->exec) cudaGraphExecDestroy(graph->exec);
  delete graph;
}

int inspire_pir_autotune(inspire_pir_server* server, int32_t batch,
                         int32_t* split, float* ms, char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null or batch <= 0."),
                  err, err_len);
  }
  if (!server->limb) {
    return Report(Err(INSPIRE_FAILED_PRECONDITION,
                      "tensor engine unavailable for these parameters"),
                  err, err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  Workspace* ws = server->ws0.get();
  Status st = EnsureWorkspace(server, ws, batch);
  if (st.ok() && !ws->limb) ws->limb = server->limb->NewScratch();
  if (st.ok()) {
    // The workspace's request buffers are timed as they are: the kernels'
    // work does not depend on the operand values.
    st = Cuda(cudaMemsetAsync(ws->q1.get(), 0, ws->q1.bytes(), ws->stream), "memset");
  }
  int chosen = 0, form = 0;
  float best = 0;
  if (st.ok()) {
    st = Cuda(server->limb->Tune(batch, ws->q1.get(), server->db_cols, ws->pkey.get(),
                                 static_cast<int64_t>(2 * server->k) * server->d,
                                 ws->gemv.get(), ws->limb.get(), ws->stream,
                                 server->prm.log_modulus, &chosen, &form, &best),
              "autotune");
  }
  if (st.ok()) {
    if (split) *split = chosen;
    if (ms) *ms = best;
  }
  return Report(st, err, err_len);
}

int inspire_pir_tune_engines(inspire_pir_server* server, int32_t max_batch,
                             int32_t* crossover, char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || max_batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null or max_batch <= 0."),
                  err, err_len);
  }
  constexpr int32_t kNever = 0x7fffffff;
  if (!server->limb) {
    server->crossover.store(kNever);
    if (crossover) *crossover = kNever;
    return INSPIRE_OK;
  }
  std::lock_guard<std::mutex> lock(server->mu);
  Workspace* ws = server->ws0.get();
  Status st = EnsureWorkspace(server, ws, max_batch);
  if (st.ok() && !ws->limb) ws->limb = server->limb->NewScratch();
  if (st.ok()) {
    st = Cuda(cudaMemsetAsync(ws->q1.get(), 0, ws->q1.bytes(), ws->stream), "memset");
  }
  // Every size up to 8 (the plain engine's cost steps every 4 requests),
  // then powers of two, then max_batch.
  std::vector<int> sizes;
  for (int b = 1; b <= std::min(8, max_batch); ++b) sizes.push_back(b);
  for (int b = 16; b < max_batch; b *= 2) sizes.push_back(b);
  if (max_batch > 8) sizes.push_back(max_batch);
  std::vector<float> plain_ms(sizes.size()), tensor_ms(sizes.size());
  std::vector<int> forms(sizes.size()), splits(sizes.size());
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (st.ok()) st = Cuda(cudaEventCreate(&e0), "event");
  if (st.ok()) st = Cuda(cudaEventCreate(&e1), "event");
  const int64_t pk_stride = static_cast<int64_t>(2 * server->k) * server->d;
  for (size_t i = 0; i < sizes.size() && st.ok(); ++i) {
    const int b = sizes[i];
    // The plain engine: one launch to warm up, the mean of three.
    st = Products(server, ws, b, ws->q1.get(), ws->pkey.get(), ws->gemv.get(),
                  INSPIRE_ENGINE_PLAIN, ws->stream);
    if (st.ok()) st = Cuda(cudaEventRecord(e0, ws->stream), "event");
    for (int r = 0; r < 3 && st.ok(); ++r) {
      st = Products(server, ws, b, ws->q1.get(), ws->pkey.get(), ws->gemv.get(),
                    INSPIRE_ENGINE_PLAIN, ws->stream);
    }
    if (st.ok()) st = Cuda(cudaEventRecord(e1, ws->stream), "event");
    if (st.ok()) st = Cuda(cudaEventSynchronize(e1), "event");
    float ms = 0;
    if (st.ok()) st = Cuda(cudaEventElapsedTime(&ms, e0, e1), "event");
    plain_ms[i] = ms / 3;
    // The tensor engine at its tuned form and split-K factor.
    int split = 0, form = 0;
    float best = 0;
    if (st.ok()) {
      st = Cuda(server->limb->Tune(b, ws->q1.get(), server->db_cols, ws->pkey.get(),
                                   pk_stride, ws->gemv.get(), ws->limb.get(),
                                   ws->stream, server->prm.log_modulus, &split, &form,
                                   &best),
                "autotune");
    }
    tensor_ms[i] = best;
    forms[i] = form;
    splits[i] = split;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (!st.ok()) return Report(st, err, err_len);
  // The smallest tested size from which the tensor engine wins at every
  // larger tested size.
  int32_t c = kNever;
  for (size_t i = sizes.size(); i-- > 0;) {
    if (tensor_ms[i] < plain_ms[i]) {
      c = sizes[i];
    } else {
      break;
    }
  }
  server->crossover.store(c);
  server->tune_table.clear();
  for (size_t i = 0; i < sizes.size(); ++i) {
    server->tune_table.push_back(
        {sizes[i], forms[i], splits[i], plain_ms[i], tensor_ms[i]});
  }
  if (crossover) *crossover = c;
  return INSPIRE_OK;
}

int32_t inspire_pir_engine_table(inspire_pir_server* server, int32_t cap,
                                 int32_t* batch, float* plain_ms, float* tensor_ms,
                                 int32_t* form, int32_t* split) {
  if (server == nullptr) return -1;
  std::lock_guard<std::mutex> lock(server->mu);
  const int32_t n = static_cast<int32_t>(server->tune_table.size());
  for (int32_t i = 0; i < n && i < cap; ++i) {
    const auto& r = server->tune_table[i];
    if (batch) batch[i] = r.batch;
    if (plain_ms) plain_ms[i] = r.plain_ms;
    if (tensor_ms) tensor_ms[i] = r.tensor_ms;
    if (form) form[i] = r.form;
    if (split) split[i] = r.split;
  }
  return n;
}

int inspire_pir_server_set_tensor_planes(inspire_pir_server* server, int32_t keep,
                                         char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null."), err, err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  Status st = Cuda(cudaDeviceSynchronize(), "synchronize");
  if (!st.ok()) return Report(st, err, err_len);
  const bool had = server->limb != nullptr;
  if (server->ws0) server->ws0->limb.reset();
  server->limb.reset();
  server->crossover.store(-1);
  server->tune_table.clear();
  LimbGemm::Create(server->prm.coeff_bits, server->prm.db_kind, server->db.get(),
                   server->rows, server->db_cols, server->prm.mat_kind, server->pack.get(),
                   server->pack_cols, keep != 0, &server->limb);
  if (had && !server->limb) {
    return Report(Err(INSPIRE_INTERNAL, "tensor engine could not be re-created"), err,
                  err_len);
  }
  return INSPIRE_OK;
}

int64_t inspire_pir_server_device_bytes(const inspire_pir_server* server) {
  if (server == nullptr) return -1;
  return static_cast<int64_t>(server->db.bytes() + server->pack.bytes()) +
         (server->limb ? server->limb->ResidentBytes() : 0);
}

int inspire_pir_server_check(inspire_pir_server* server, char* err,
                             size_t err_len) {
  using namespace inspire;
  if (server == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null."), err, err_len);
  }
  if (server->limb && server->limb->CheckError() != 0) {
    return Report(Err(INSPIRE_INTERNAL, "tensor engine pipeline timed out"), err,
                  err_len);
  }
  return INSPIRE_OK;
}

int inspire_vpir_process_batch(inspire_pir_server* server, int32_t batch,
                               const void* first_dim, int64_t first_dim_len,
                               const void* packing_key, int64_t packing_key_count,
                               int32_t local_finalize, void* b_responses,
                               int32_t engine, char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null or batch <= 0."),
                  err, err_len);
  }
  inspire_pir_server* s = server;
  engine = ResolveEngine(s, engine, batch);
  const int expected = local_finalize ? s->k : 2 * s->k;
  if (packing_key_count != expected) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "Packing key must contain " + std::to_string(expected) +
                          " polynomials."),
                  err, err_len);
  }
  if (first_dim_len != s->db_cols) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "Flattened first dimension query must match DB matrix "
                      "columns (N)."),
                  err, err_len);
  }
  if (s->t != 1) {
    return Report(Err(INSPIRE_FAILED_PRECONDITION,
                      "a vPIR server has interpolation_degree 1."),
                  err, err_len);
  }
  Status st = s->deferred;
  if (!st.ok()) return Report(st, err, err_len);
  std::lock_guard<std::mutex> lock(s->mu);
  Workspace* ws = s->ws0.get();
  st = EnsureWorkspace(s, ws, batch);
  const size_t w = Words(s->prm.coeff_bits);
  const size_t d = s->d;
  const cudaStream_t cs = ws->stream;
  const size_t pk_bytes = static_cast<size_t>(batch) * expected * d * w;
  if (st.ok()) {
    st = Cuda(cudaMemcpyAsync(ws->q1.get(), first_dim, static_cast<size_t>(batch) * s->db_cols * w,
                              cudaMemcpyHostToDevice, cs),
              "copy first_dim");
  }
  if (st.ok()) {
    st = Cuda(cudaMemcpyAsync(ws->pkey.get(), packing_key, pk_bytes, cudaMemcpyHostToDevice, cs),
              "copy packing_key");
  }
  if (st.ok()) {
    st = VpirOnDevice(s, ws, batch, ws->q1.get(), ws->pkey.get(),
                      static_cast<int64_t>(expected) * s->d, local_finalize != 0,
                      ws->resp.get(), engine, cs);
  }
  const size_t out_bytes = static_cast<size_t>(batch) * s->rows * w;
  if (st.ok()) {
    st = Cuda(cudaMemcpyAsync(b_responses, ws->resp.get(), out_bytes, cudaMemcpyDeviceToHost, cs),
              "copy response");
  }
  if (st.ok()) st = Cuda(cudaStreamSynchronize(cs), "vpir answer");
  if (st.ok() && engine == INSPIRE_ENGINE_TENSOR && s->limb && s->limb->CheckError() != 0) {
    st = Err(INSPIRE_INTERNAL, "tensor engine pipeline timed out");
  }
  return Report(st, err, err_len);
}

int inspire_pir_products_device(inspire_pir_server* server, int32_t batch,
                                const void* first_dim, const void* packing_key,
                                void* out, int32_t engine, void* stream,
                                char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "server is null or batch <= 0."),
                  err, err_len);
  }
  engine = ResolveEngine(server, engine, batch);
  std::lock_guard<std::mutex> lock(server->mu);
  Status st = Products(server, server->ws0.get(), batch, first_dim, packing_key,
                       out, engine, static_cast<cudaStream_t>(stream));
  return Report(st, err, err_len);
}

int inspire_pir_tensor_products_device(inspire_pir_server* server, int32_t batch,
                                       const void* first_dim, const void* packing_key,
                                       void* out, int32_t form, int32_t split,
                                       void* stream, char* err, size_t err_len) {
  using namespace inspire;
  if (server == nullptr || batch <= 0 || form < 0 || form > (kFormRaw | kFormNarrow)) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "server is null, batch <= 0 or unknown form."),
                  err, err_len);
  }
  if (!server->limb) {
    return Report(Err(INSPIRE_FAILED_PRECONDITION,
                      "tensor engine unavailable for these parameters"),
                  err, err_len);
  }
  std::lock_guard<std::mutex> lock(server->mu);
  Workspace* ws = server->ws0.get();
  if (!ws->limb) ws->limb = server->limb->NewScratch();
  const cudaError_t e = server->limb->RunForm(
      batch, first_dim, server->db_cols, packing_key,
      static_cast<int64_t>(2 * server->k) * server->d, out, ws->limb.get(),
      static_cast<cudaStream_t>(stream), form, split, /*out_bits=*/0);
  if (e == cudaErrorNotSupported) {
    return Report(Err(INSPIRE_FAILED_PRECONDITION,
                      "this form of the tensor engine is not available on this server"),
                  err, err_len);
  }
  return Report(Cuda(e, "limb gemm"), err, err_len);
}

int64_t inspire_pir_workspace_bytes(const inspire_pir_server* server,
                                    int32_t max_batch) {
  if (server == nullptr || max_batch <= 0) return -1;
  return inspire::WorkspaceBytes(server, max_batch);
}

int inspire_pir_workspace_create(inspire_pir_server* server, int32_t max_batch,
                                 inspire_pir_workspace** out, char* err,
                                 size_t err_len) {
  using namespace inspire;
  if (server == nullptr || out == nullptr || max_batch <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "server/out must be set and max_batch positive."),
                  err, err_len);
  }
  *out = nullptr;
  std::unique_ptr<inspire_pir_workspace> w(new inspire_pir_workspace());
  w->server = server;
  Status st = InitWorkspace(&w->ws);
  if (st.ok()) st = EnsureWorkspace(server, &w->ws, max_batch);
  const size_t cw = Words(server->prm.coeff_bits);
  const size_t d = server->d;
  const size_t sizes[4] = {
      static_cast<size_t>(max_batch) * server->db_cols * cw,
      static_cast<size_t>(max_batch) * std::max(1, 2 * server->ne) * d * cw,
      static_cast<size_t>(max_batch) * 2 * server->k * d * cw,
      static_cast<size_t>(max_batch) * server->l * 2 * d * cw};
  for (int i = 0; i < 4 && st.ok(); ++i) {
    st = Cuda(cudaMallocHost(&w->ws.host[i], sizes[i]), "cudaMallocHost");
    if (st.ok()) std::memset(w->ws.host[i], 0, sizes[i]);
  }
  if (st.ok()) *out = w.release();
  return Report(st, err, err_len);
}

void inspire_pir_workspace_destroy(inspire_pir_workspace* ws) {
  if (ws != nullptr) cudaStreamSynchronize(ws->ws.stream);
  delete ws;
}

int inspire_pir_workspace_host_buffers(inspire_pir_workspace* ws,
                                       void** first_dim, void** second_dim,
                                       void** packing_key, void** responses) {
  if (ws == nullptr) return INSPIRE_INVALID_ARGUMENT;
  if (first_dim) *first_dim = ws->ws.host[0];
  if (second_dim) *second_dim = ws->ws.host[1];
  if (packing_key) *packing_key = ws->ws.host[2];
  if (responses) *responses = ws->ws.host[3];
  return INSPIRE_OK;
}

int inspire_pir_workspace_submit(inspire_pir_workspace* ws, int32_t batch,
                                 int32_t engine, char* err, size_t err_len) {
  using namespace inspire;
  if (ws == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "workspace is null."), err, err_len);
  }
  inspire_pir_server* s = ws->server;
  Workspace* w = &ws->ws;
  if (batch <= 0 || batch > w->cap) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "batch must be between 1 and the workspace capacity."),
                  err, err_len);
  }
  engine = ResolveEngine(s, engine, batch);
  Status st = s->deferred;
  const size_t cw = Words(s->prm.coeff_bits);
  const size_t d = s->d;
  const cudaStream_t sm = w->stream;
  const size_t nfd = static_cast<size_t>(batch) * s->db_cols * cw;
  const size_t nsd = static_cast<size_t>(batch) * 2 * s->ne * d * cw;
  const size_t npk = static_cast<size_t>(batch) * 2 * s->k * d * cw;
  if (st.ok()) st = Cuda(cudaMemcpyAsync(w->q1.get(), w->host[0], nfd,
                                         cudaMemcpyHostToDevice, sm), "copy");
  if (st.ok() && s->t > 1) {
    st = Cuda(cudaMemcpyAsync(w->sdim.get(), w->host[1], nsd, cudaMemcpyHostToDevice,
                              sm), "copy");
  }
  if (st.ok()) st = Cuda(cudaMemcpyAsync(w->pkey.get(), w->host[2], npk,
                                         cudaMemcpyHostToDevice, sm), "copy");
  if (st.ok()) {
    st = AnswerOnDevice(s, w, batch, w->q1.get(), w->pkey.get(), w->sdim.get(),
                        w->resp.get(), engine, sm, false);
  }
  if (st.ok()) {
    st = Cuda(cudaMemcpyAsync(w->host[3], w->resp.get(),
                              static_cast<size_t>(batch) * s->l * 2 * d * cw,
                              cudaMemcpyDeviceToHost, sm),
              "copy");
  }
  if (st.ok()) st = Cuda(cudaEventRecord(w->done, sm), "cudaEventRecord");
  if (st.ok()) w->pending_engine = engine;
  return Report(st, err, err_len);
}

int inspire_pir_workspace_poll(inspire_pir_workspace* ws) {
  if (ws == nullptr) return -INSPIRE_INVALID_ARGUMENT;
  const cudaError_t e = cudaEventQuery(ws->ws.done);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return -INSPIRE_INTERNAL;
}

int inspire_pir_workspace_wait(inspire_pir_workspace* ws, char* err,
                               size_t err_len) {
  using namespace inspire;
  if (ws == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "workspace is null."), err, err_len);
  }
  Status st = Cuda(cudaEventSynchronize(ws->ws.done), "answer");
  if (st.ok() && ws->ws.pending_engine == INSPIRE_ENGINE_TENSOR &&
      ws->server->limb && ws->server->limb->CheckError() != 0) {
    st = Err(INSPIRE_INTERNAL, "tensor engine pipeline timed out");
  }
  return Report(st, err, err_len);
}

int inspire_pir_server_shape(const inspire_pir_server* server, int64_t* rows,
                             int64_t* db_cols, int64_t* pack_cols) {
  if (server == nullptr) return INSPIRE_INVALID_ARGUMENT;
  if (rows) *rows = server->rows;
  if (db_cols) *db_cols = server->db_cols;
  if (pack_cols) *pack_cols = server->pack_cols;
  return INSPIRE_OK;
}

int inspire_pir_server_timings(const inspire_pir_server* server,
                               double* db_mult_ms, double* packing_ms,
                               double* poly_eval_ms) {
  if (server == nullptr) return INSPIRE_INVALID_ARGUMENT;
  if (db_mult_ms) *db_mult_ms = server->t_db;
  if (packing_ms) *packing_ms = server->t_pack;
  if (poly_eval_ms) *poly_eval_ms = server->t_eval;
  return INSPIRE_OK;
}

int inspire_matrix_multiply(int32_t mat_kind, int32_t coeff_bits,
                            const void* mat, int64_t rows, int64_t cols,
                            const void* vec, void* out, char* err,
                            size_t err_len) {
  using namespace inspire;
  if ((coeff_bits != 32 && coeff_bits != 64) || elem_size(mat_kind) == 0 ||
      rows < 0 || cols < 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "invalid matrix arguments."),
                  err, err_len);
  }
  const size_t w = coeff_bits / 8;
  DevBuf dm, dv, dout;
  Status st = dm.Upload(mat, static_cast<size_t>(rows) * cols * elem_size(mat_kind));
  if (st.ok()) st = dv.Upload(vec, static_cast<size_t>(cols) * w);
  if (st.ok()) st = dout.Alloc(static_cast<size_t>(rows) * w);
  if (st.ok() && rows > 0) {
    st = Cuda(launch_fused_gemv(coeff_bits, mat_kind, dm.get(), cols, dv.get(), cols,
                                INSPIRE_I32, nullptr, 0, nullptr, 0, dout.get(), rows,
                                rows, 1, nullptr),
              "gemv");
    if (st.ok()) st = Cuda(cudaDeviceSynchronize(), "gemv");
    if (st.ok()) {
      st = Cuda(cudaMemcpy(out, dout.get(), rows * w, cudaMemcpyDeviceToHost),
                "copy out");
    }
  }
  return Report(st, err, err_len);
}

int inspire_inner_product(int32_t coeff_bits, const void* u, const void* v,
                          int32_t n, int32_t d, int32_t u_bits, int32_t v_bits,
                          int32_t chunk_bits, int32_t u_is_signed, void* out,
                          char* err, size_t err_len) {
  using namespace inspire;
  if (n <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "Polynomial vectors cannot be empty."),
                  err, err_len);
  }
  if (coeff_bits != 32 && coeff_bits != 64) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "coeff_bits must be 32 or 64."),
                  err, err_len);
  }
  int logd = 0;
  while ((1 << logd) < d) ++logd;
  if (d < 2 || (1 << logd) != d || logd > 13) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "Polynomial lengths or context mismatch."),
                  err, err_len);
  }
  ChunkRule rule;
  Status st = MakeRule(coeff_bits, n, d, u_bits, v_bits, chunk_bits, &rule);
  if (!st.ok()) return Report(st, err, err_len);
  const int ub = std::min(rule.u_chunks * rule.chunk_bits, 64);
  const int vb = std::min(rule.v_chunks * rule.chunk_bits, coeff_bits);
  int r = 0;
  st = PrimesFor(BoundBits(n, d, ub, vb), &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(logd, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  NttCtx c = tabs->Ctx(r);
  const size_t total = static_cast<size_t>(n) * d;
  const size_t w = coeff_bits / 8;
  DevBuf du, dv, dU, dV, dout;
  // u as the chunk rule rebuilds it (signed when asked); v masked.
  std::vector<int64_t> ue(total);
  for (size_t i = 0; i < total; ++i) {
    const uint64_t x = coeff_bits == 32
                           ? static_cast<const uint32_t*>(u)[i]
                           : static_cast<const uint64_t*>(u)[i];
    ue[i] = RebuildU(x, rule, u_bits, u_is_signed != 0);
  }
  const uint64_t vmask = MaskBits(rule.v_chunks * rule.chunk_bits, coeff_bits);
  const bool u_fits_signed = u_is_signed != 0 || ub < 64;
  if (st.ok()) st = dU.Alloc(total * r * 4);
  if (st.ok()) st = dV.Alloc(total * r * 4);
  if (st.ok()) st = dv.Upload(v, total * w);
  if (st.ok()) st = dout.Alloc(d * w);
  if (st.ok()) {
    if (u_fits_signed) {
      st = du.Upload(ue.data(), total * 8);
      if (st.ok()) {
        ntt_signed_kernel<<<n * r, kPolyThreads, d * 4>>>(du.get<int64_t>(), n,
                                                         dU.get<uint32_t>(), c);
      }
    } else if (coeff_bits == 64) {
      st = du.Upload(ue.data(), total * 8);  // full-width unsigned u
      if (st.ok()) {
        ntt_coeffs_kernel<uint64_t><<<dim3(n * r, 1), kPolyThreads, d * 4>>>(
            du.get<uint64_t>(), 0, 0, n, ~0ull, dU.get<uint32_t>(), d, c);
      }
    }
  }
  if (st.ok()) {
    if (coeff_bits == 32) {
      ntt_coeffs_kernel<uint32_t><<<dim3(n * r, 1), kPolyThreads, d * 4>>>(
          dv.get<uint32_t>(), 0, 0, n, static_cast<uint32_t>(vmask),
          dV.get<uint32_t>(), d, c);
      st = SetSmem(inner_product_finish_kernel<uint32_t>, static_cast<size_t>(r) * d * 4);
      if (st.ok())
        inner_product_finish_kernel<uint32_t><<<1, kPolyThreads, r * d * 4>>>(
            dU.get<uint32_t>(), dV.get<uint32_t>(), n, dout.get<uint32_t>(), c);
    } else {
      ntt_coeffs_kernel<uint64_t><<<dim3(n * r, 1), kPolyThreads, d * 4>>>(
          dv.get<uint64_t>(), 0, 0, n, vmask, dV.get<uint32_t>(), d, c);
      st = SetSmem(inner_product_finish_kernel<uint64_t>, static_cast<size_t>(r) * d * 4);
      if (st.ok())
        inner_product_finish_kernel<uint64_t><<<1, kPolyThreads, r * d * 4>>>(
            dU.get<uint32_t>(), dV.get<uint32_t>(), n, dout.get<uint64_t>(), c);
    }
  }
  if (st.ok()) st = Cuda(cudaDeviceSynchronize(), "inner product");
  if (st.ok()) {
    st = Cuda(cudaMemcpy(out, dout.get(), d * w, cudaMemcpyDeviceToHost), "copy out");
  }
  return Report(st, err, err_len);
}

int inspire_compute_hint_matrix(int32_t db_kind, int32_t coeff_bits, const void* db,
                                int64_t rows, int64_t cols, const void* a_components,
                                int32_t n, int32_t d, void* out, int32_t on_device,
                                void* stream, char* err, size_t err_len) {
  using namespace inspire;
  // Checks in the reference's order (hint_computation.cc:81-97).
  if (rows <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "Database matrix cannot be empty."), err,
                  err_len);
  }
  if (n <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "a_components cannot be empty."), err,
                  err_len);
  }
  if (cols != static_cast<int64_t>(d) * n) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT,
                      "Database columns must match d * n where d is the polynomial "
                      "length and n is the number of polynomials."),
                  err, err_len);
  }
  if (coeff_bits != 32 && coeff_bits != 64) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "coeff_bits must be 32 or 64."), err,
                  err_len);
  }
  if (db_kind != INSPIRE_U8 && db_kind != INSPIRE_U16 && db_kind != INSPIRE_U32) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "database type must be u8, u16 or u32."),
                  err, err_len);
  }
  int logd = 0;
  while ((1 << logd) < d) ++logd;
  if (d < 2 || (1 << logd) != d || logd > 13) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "polynomial length must be a power of two "
                                                "between 2 and 8192."),
                  err, err_len);
  }
  const int s_bits = 8 * elem_size(db_kind);
  int r = 0;
  Status st = PrimesFor(BoundBits(n, d, s_bits, coeff_bits), &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(logd, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  NttCtx c = tabs->Ctx(r);
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) {
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const size_t w = coeff_bits / 8;
  const size_t es = elem_size(db_kind);
  // The a-components on the host (a device copy comes back first: they are
  // n * d words).
  std::vector<uint8_t> a_host(static_cast<size_t>(n) * d * w);
  if (on_device) {
    st = Cuda(cudaMemcpy(a_host.data(), a_components, a_host.size(), cudaMemcpyDeviceToHost),
              "a-components download");
    if (!st.ok()) return Report(st, err, err_len);
  } else {
    std::memcpy(a_host.data(), a_components, a_host.size());
  }
  // v_k[0] = a_k[0], v_k[j] = -a_k[d - j] (hint_computation.cc:110-119).
  std::vector<uint8_t> vinv(static_cast<size_t>(n) * d * w);
  for (int k = 0; k < n; ++k) {
    for (int j = 0; j < d; ++j) {
      const int src = j == 0 ? 0 : d - j;
      const uint8_t* a = a_host.data() + (static_cast<size_t>(k) * d + src) * w;
      uint8_t* v = vinv.data() + (static_cast<size_t>(k) * d + j) * w;
      if (w == 4) {
        uint32_t x;
        std::memcpy(&x, a, 4);
        x = j == 0 ? x : 0u - x;
        std::memcpy(v, &x, 4);
      } else {
        uint64_t x;
        std::memcpy(&x, a, 8);
        x = j == 0 ? x : 0ull - x;
        std::memcpy(v, &x, 8);
      }
    }
  }
  const cudaStream_t cs = on_device ? static_cast<cudaStream_t>(stream) : nullptr;
  DevBuf dv, dV, dres, ddb, dout;
  st = dv.Upload(vinv.data(), vinv.size());
  if (st.ok()) st = dV.Alloc(static_cast<size_t>(n) * r * d * 4);
  if (st.ok()) st = dres.Alloc(static_cast<size_t>(rows) * r * d * 4);
  const void* db_dev = db;
  void* out_dev = out;
  if (st.ok() && !on_device) {
    st = ddb.Upload(db, static_cast<size_t>(rows) * cols * es);
    if (st.ok()) st = dout.Alloc(static_cast<size_t>(rows) * d * w);
    db_dev = ddb.get();
    out_dev = dout.get();
  }
  if (st.ok()) {
    auto run = [&](auto ttag, auto stag) -> Status {
      using T = decltype(ttag);
      using S = decltype(stag);
      ntt_coeffs_kernel<T><<<dim3(n * r, 1), PolyThreads(d), d * 4, cs>>>(
          dv.get<T>(), 0, 0, n, static_cast<T>(~0ull), dV.get<uint32_t>(), d, c);
      RETURN_IF_ERROR(Cuda(cudaGetLastError(), "a-component transforms"));
      const dim3 grid(r, static_cast<unsigned>(rows));
      if (c.tables16 != nullptr) {
        // d = 2048..8192: the radix-16 register transforms.
        INSPIRE_NTT16_DISPATCH(
            c.logd, RETURN_IF_ERROR(SetSmem(hint_rows16_kernel<S, LG>, d * 4));
            hint_rows16_kernel<S, LG><<<grid, Ntt16<LG>::kThreads, d * 4, cs>>>(
                static_cast<const S*>(db_dev), cols, n, dV.get<uint32_t>(),
                dres.get<uint32_t>(), c));
      } else {
        const PolyLaunch pl = PolyShapeFor(d, static_cast<int64_t>(r) * rows, sms);
        INSPIRE_ITERS_DISPATCH(
            pl.iters, RETURN_IF_ERROR(SetSmem(hint_rows_kernel<S, IT>, d * 4));
            hint_rows_kernel<S, IT><<<grid, pl.nt, d * 4, cs>>>(
                static_cast<const S*>(db_dev), cols, n, dV.get<uint32_t>(),
                dres.get<uint32_t>(), c));
      }
      RETURN_IF_ERROR(Cuda(cudaGetLastError(), "hint rows"));
      const int64_t total = rows * static_cast<int64_t>(d);
      const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 8));
      hint_crt_kernel<T><<<blocks, 256, 0, cs>>>(dres.get<uint32_t>(), rows, d,
                                                  static_cast<T*>(out_dev), c);
      return Cuda(cudaGetLastError(), "hint CRT");
    };
    if (coeff_bits == 32) {
      st = db_kind == INSPIRE_U8    ? run(uint32_t{}, uint8_t{})
           : db_kind == INSPIRE_U16 ? run(uint32_t{}, uint16_t{})
                                    : run(uint32_t{}, uint32_t{});
    } else {
      st = db_kind == INSPIRE_U8    ? run(uint64_t{}, uint8_t{})
           : db_kind == INSPIRE_U16 ? run(uint64_t{}, uint16_t{})
                                    : run(uint64_t{}, uint32_t{});
    }
  }
  // The temporaries are freed on return: wait for the work that uses them.
  if (st.ok()) st = Cuda(on_device ? cudaStreamSynchronize(cs) : cudaDeviceSynchronize(), "hint");
  if (st.ok() && !on_device) {
    st = Cuda(cudaMemcpy(out, dout.get(), static_cast<size_t>(rows) * d * w,
                         cudaMemcpyDeviceToHost),
              "copy out");
  }
  return Report(st, err, err_len);
}

int inspire_external_product(const inspire_pir_params* params,
                             const void* ct_a, const void* ct_b,
                             const void* rgsw, void* out_a, void* out_b,
                             char* err, size_t err_len) {
  using namespace inspire;
  // A one-request, one-shard server-less run of the EvalPoly step kernel.
  if (params == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "params is null."), err, err_len);
  }
  const int cb = params->coeff_bits;
  const int d = 1 << params->log_degree;
  const int ne = params->eval_num_digits;
  if (ne <= 0 || params->eval_log_digit <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "rgsw_ct sizes must match num_digits."),
                  err, err_len);
  }
  ChunkRule re;
  Status st = MakeRule(cb, 2 * ne, d, params->eval_log_digit, params->log_modulus,
                       ChunkFor(2 * ne, d), &re);
  if (!st.ok()) return Report(st, err, err_len);
  int r = 0;
  st = PrimesFor(BoundBits(2 * ne, d,
                           std::min({params->eval_log_digit,
                                     re.u_chunks * re.chunk_bits, cb}),
                           std::min(re.v_chunks * re.chunk_bits, cb)),
                 &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(params->log_degree, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  NttCtx c = tabs->Ctx(r);
  const size_t w = cb / 8;
  const int ng = 2 * ne;
  // Split the interleaved (a, b) RGSW layout into a-parts and b-parts.
  std::vector<unsigned char> ra(static_cast<size_t>(ng) * d * w),
      rb(static_cast<size_t>(ng) * d * w);
  const unsigned char* src = static_cast<const unsigned char*>(rgsw);
  for (int g = 0; g < ng; ++g) {
    std::memcpy(ra.data() + static_cast<size_t>(g) * d * w,
                src + static_cast<size_t>(2 * g) * d * w, d * w);
    std::memcpy(rb.data() + static_cast<size_t>(g) * d * w,
                src + static_cast<size_t>(2 * g + 1) * d * w, d * w);
  }
  DevBuf dra, drb, dA, dB, dca, dcb, dres, dout;
  st = dra.Upload(ra.data(), ra.size());
  if (st.ok()) st = drb.Upload(rb.data(), rb.size());
  if (st.ok()) st = dA.Alloc(static_cast<size_t>(ng) * r * d * 4);
  if (st.ok()) st = dB.Alloc(static_cast<size_t>(ng) * r * d * 4);
  if (st.ok()) st = dca.Upload(ct_a, d * w);
  if (st.ok()) st = dcb.Upload(ct_b, d * w);
  if (st.ok()) st = dres.Alloc(static_cast<size_t>(r) * 2 * d * 4);
  if (st.ok()) st = dout.Alloc(2 * d * w);
  const uint64_t vmask = MaskBits(re.v_chunks * re.chunk_bits, cb);
  ExtArgs e{params->log_modulus, params->eval_log_digit, ne,
            LiveDigits(params->log_modulus, params->eval_log_digit, ne),
            MaskBits(re.u_chunks * re.chunk_bits, cb)};
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    ntt_coeffs_kernel<T><<<dim3(ng * r, 1), kPolyThreads, d * 4>>>(
        dra.get<T>(), 0, 0, ng, static_cast<T>(vmask), dA.get<uint32_t>(), d, c);
    ntt_coeffs_kernel<T><<<dim3(ng * r, 1), kPolyThreads, d * 4>>>(
        drb.get<T>(), 0, 0, ng, static_cast<T>(vmask), dB.get<uint32_t>(), d, c);
    const size_t smem = static_cast<size_t>(d) * 4 + 2ull * d * sizeof(T);
    RETURN_IF_ERROR(SetSmem(ext_step_kernel<T>, smem));
    ext_step_kernel<T><<<dim3(r, 1, 1), kPolyThreads, smem>>>(
        true, nullptr, dres.get<uint32_t>(), dca.get<T>(), 0, 0, dcb.get<T>(), 0, 0,
        dA.get<uint32_t>(), 0, dB.get<uint32_t>(), e, c);
    finish_kernel<T><<<dim3(1, 1), kPolyThreads>>>(
        true, dres.get<uint32_t>(), nullptr, 0, nullptr, 0, 0, false, 0, 0, 0,
        dout.get<T>(), c);
    return Cuda(cudaDeviceSynchronize(), "external product");
  };
  if (st.ok()) st = cb == 32 ? run(uint32_t{}) : run(uint64_t{});
  if (st.ok()) st = Cuda(cudaMemcpy(out_a, dout.get(), d * w, cudaMemcpyDeviceToHost), "copy");
  if (st.ok())
    st = Cuda(cudaMemcpy(out_b, dout.get<char>() + d * w, d * w, cudaMemcpyDeviceToHost),
              "copy");
  return Report(st, err, err_len);
}

int inspire_preprocess_matrix_pack(int32_t coeff_bits, int32_t mat_kind,
                                   int32_t log_modulus, int32_t log_digit,
                                   int32_t num_digits, int32_t d, int32_t slices,
                                   const void* hint, int64_t hint_stride,
                                   const void* pack_a, int64_t pack_a_count,
                                   void* a_tilde_agg, void* matrix, void* t_vec_h,
                                   int32_t on_device, void* stream, char* err,
                                   size_t err_len) {
  using namespace inspire;
  auto fail = [&](const char* m) { return Report(Err(INSPIRE_INVALID_ARGUMENT, m), err, err_len); };
  if (coeff_bits != 32 && coeff_bits != 64) return fail("coeff_bits must be 32 or 64.");
  const int coeff_kind = coeff_bits == 32 ? INSPIRE_U32 : INSPIRE_U64;
  if (mat_kind != coeff_kind && mat_kind != INSPIRE_I16 && mat_kind != INSPIRE_I32) {
    return fail("matrix type must be the coefficient type, i16 or i32.");
  }
  if (log_digit <= 0 || num_digits <= 0) {
    return fail("log_digit and num_digits must be positive.");
  }
  if (pack_a_count != 2ll * num_digits) {
    return fail("InnerProduct: size mismatch or empty");
  }
  if (num_digits > 64 || log_digit >= coeff_bits) {
    return fail("gadget larger than the coefficient width.");
  }
  if (log_modulus <= 0 || log_modulus > coeff_bits) {
    return fail("log_modulus must be in (0, coeff_bits].");
  }
  int logd = 0;
  while ((1 << logd) < d) ++logd;
  if (d < 4 || (1 << logd) != d || logd > 13) {
    return fail("polynomial length must be a power of two between 4 and 8192.");
  }
  if (slices <= 0) return fail("slices must be positive.");
  if (hint_stride < d) return fail("hint rows must hold d coefficients.");
  if (hint == nullptr || pack_a == nullptr || a_tilde_agg == nullptr ||
      matrix == nullptr || t_vec_h == nullptr) {
    return fail("null buffer.");
  }
  const int k = num_digits;
  int r = 0;
  Status st = PrimesFor(BoundBits(k, d, log_digit, coeff_bits), &r);
  if (!st.ok()) return Report(st, err, err_len);
  const int iters = d > 4096 ? 2 : 1;
  const int threads = d / (4 * iters);
  const size_t w = coeff_bits / 8;
  const size_t chain_smem = d * w + static_cast<size_t>(d) * 4 * (1 + r);
  if (chain_smem > 227 * 1024) return fail("ring degree and gadget too large.");
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(logd, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  const NttCtx c = tabs->Ctx(r);
  const cudaStream_t cs = on_device ? static_cast<cudaStream_t>(stream) : nullptr;
  const size_t mw = elem_size(mat_kind);
  const size_t dd = static_cast<size_t>(d) * d;
  const int64_t chain_stride = static_cast<int64_t>(d / 2 - 1) * k * d;

  // Index tables: a_hat_agg[k] sits in transform slot bitrev((power_k - 1)/2);
  // 5^i mod 2d; matrix block input i <- t_vec_g[j] (2j) / t_vec_gh[j] (2j+1).
  std::vector<int> hat(d), pow5(d / 2), src_of(d, -1);
  {
    int64_t p5 = 1;
    for (int i = 0; i < d / 2; ++i) {
      pow5[i] = static_cast<int>(p5);
      p5 = p5 * 5 % (2 * d);
    }
    for (int kk = 0; kk < d; ++kk) {
      const int64_t power = kk < d / 2 ? pow5[kk]
                                      : static_cast<int64_t>(pow5[kk - d / 2]) * (2 * d - 1) % (2 * d);
      hat[kk] = BitRev(static_cast<int>((power - 1) / 2), logd);
    }
    for (int j = 0; j <= d / 2 - 2; ++j) {
      const int64_t pg = pow5[j];
      const int64_t pgh = pg * (2 * d - 1) % (2 * d);
      src_of[(pg - 1) / 2] = 2 * j;
      src_of[(pgh - 1) / 2] = 2 * j + 1;
    }
  }
  DevBuf dhat, dpow, dsrc, dhint, dpa, dW, dev0, dev1, dtg, dtgh, dfin;
  DevBuf da, dm, dth;
  st = dhat.Upload(hat.data(), hat.size() * 4);
  if (st.ok()) st = dpow.Upload(pow5.data(), pow5.size() * 4);
  if (st.ok()) st = dsrc.Upload(src_of.data(), src_of.size() * 4);
  const void* hint_dev = hint;
  const void* pa_dev = pack_a;
  void* a_out = a_tilde_agg;
  void* m_out = matrix;
  void* th_out = t_vec_h;
  if (st.ok() && !on_device) {
    st = dhint.Upload(hint, static_cast<size_t>(slices) * d * hint_stride * w);
    if (st.ok()) st = dpa.Upload(pack_a, static_cast<size_t>(2 * k) * d * w);
    if (st.ok()) st = da.Alloc(static_cast<size_t>(slices) * d * w);
    if (st.ok()) st = dm.Alloc(static_cast<size_t>(slices) * d * k * d * mw);
    if (st.ok()) st = dth.Alloc(static_cast<size_t>(slices) * k * d * w);
    hint_dev = dhint.get();
    pa_dev = dpa.get();
    a_out = da.get();
    m_out = dm.get();
    th_out = dth.get();
  }
  if (st.ok()) st = dW.Alloc(static_cast<size_t>(2 * k) * r * d * 4);
  if (st.ok()) st = dev0.Alloc(slices * dd * w);
  if (st.ok()) st = dev1.Alloc(slices * dd * w);
  if (st.ok()) st = dtg.Alloc(static_cast<size_t>(slices) * chain_stride * w);
  if (st.ok()) st = dtgh.Alloc(static_cast<size_t>(slices) * chain_stride * w);
  if (st.ok()) st = dfin.Alloc(static_cast<size_t>(slices) * 2 * d * w);

  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    // The transform of every key part (w_vec_g then w_vec_h), plain residues.
    ntt_coeffs_kernel<T><<<dim3(2 * k * r, 1), PolyThreads(d), d * 4, cs>>>(
        static_cast<const T*>(pa_dev), 0, 0, 2 * k, static_cast<T>(~0ull),
        dW.get<uint32_t>(), d, c);
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "key part transforms"));
    // Polynomial transform of d x d words per slice, log d DIF stages from
    // `in` (rotated on input when rot) ping-ponging through dev0/dev1;
    // returns the buffer holding the result.
    auto transform = [&](DevBuf* in, bool rot) -> DevBuf* {
      DevBuf* src = in;
      DevBuf* dst = in == &dev0 ? &dev1 : &dev0;
      const int64_t cells = static_cast<int64_t>(d / 2) * d;
      const dim3 grid(static_cast<unsigned>((cells + 255) / 256), slices);
      for (int lh = logd - 1; lh >= 0; --lh) {
        pp_dif_stage_kernel<T><<<grid, 256, 0, cs>>>(src->get<T>(), dst->get<T>(), d, logd,
                                                      lh, rot && lh == logd - 1 ? 1 : 0);
        std::swap(src, dst);
      }
      return src;
    };
    const dim3 tgrid((d + 31) / 32, (d + 31) / 32, slices);
    pp_atilde_kernel<T><<<tgrid, dim3(32, 8), 0, cs>>>(static_cast<const T*>(hint_dev),
                                                       hint_stride, d, logd, log_modulus,
                                                       dev0.get<T>());
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "a_tilde"));
    DevBuf* ev = transform(&dev0, true);
    RETURN_IF_ERROR(Cuda(cudaGetLastError(), "a_hat_agg transform"));
    ChainArgs ca;
    ca.d = d;
    ca.log_d = logd;
    ca.log_q = log_modulus;
    ca.log_digit = log_digit;
    ca.k = k;
    ca.chain_stride = chain_stride;
    ca.hat_row = dhat.get<int>();
    ca.pow5 = dpow.get<int>();
    ca.Wg = dW.get<uint32_t>();
    ca.Wh = dW.get<uint32_t>() + static_cast<size_t>(k) * r * d;
    auto chains = [&](auto itag) -> Status {
      constexpr int IT = decltype(itag)::value;
      RETURN_IF_ERROR(SetSmem(pp_chain_kernel<T, IT>, chain_smem));
      RETURN_IF_ERROR(SetSmem(pp_tail_kernel<T, IT>, chain_smem));
      pp_chain_kernel<T, IT><<<dim3(2, slices), threads, chain_smem, cs>>>(
          ev->get<T>(), ca, c, dtg.get<T>(), dtgh.get<T>(), dfin.get<T>());
      RETURN_IF_ERROR(Cuda(cudaGetLastError(), "reduction chains"));
      pp_tail_kernel<T, IT><<<slices, threads, chain_smem, cs>>>(
          dfin.get<T>(), ca, c, static_cast<T*>(th_out), static_cast<T*>(a_out));
      return Cuda(cudaGetLastError(), "a_tilde_agg");
    };
    // The radix-16 register transforms (d = 2048..8192): G groups of d/16
    // threads, one prime each at a time, at most 768 threads (85 registers
    // a thread).
    auto chains16 = [&](auto ltag, auto gtag) -> Status {
      constexpr int LG = decltype(ltag)::value;
      constexpr int GR = decltype(gtag)::value;
      const size_t smem16 = (1 + k) * d * w + static_cast<size_t>(d) * 4 * (r + GR);
      RETURN_IF_ERROR(SetSmem(pp_chain16_kernel<T, LG, GR>, smem16));
      RETURN_IF_ERROR(SetSmem(pp_tail16_kernel<T, LG, GR>, smem16));
      constexpr int nt = GR * Ntt16<LG>::kThreads;
      pp_chain16_kernel<T, LG, GR><<<dim3(2, slices), nt, smem16, cs>>>(
          ev->get<T>(), ca, c, dtg.get<T>(), dtgh.get<T>(), dfin.get<T>());
      RETURN_IF_ERROR(Cuda(cudaGetLastError(), "reduction chains"));
      pp_tail16_kernel<T, LG, GR><<<slices, nt, smem16, cs>>>(
          dfin.get<T>(), ca, c, static_cast<T*>(th_out), static_cast<T*>(a_out));
      return Cuda(cudaGetLastError(), "a_tilde_agg");
    };
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I3 = std::integral_constant<int, 3>;
    using I4 = std::integral_constant<int, 4>;
    using I5 = std::integral_constant<int, 5>;
    const int groups16 = logd == 11 ? std::min(r, 5) : logd == 12 ? std::min(r, 3) : 1;
    const bool fits16 =
        (1 + k) * d * w + static_cast<size_t>(d) * 4 * (r + groups16) <= 227 * 1024;
    if (c.tables16 != nullptr && fits16 && logd == 11) {
      if (groups16 == 2) RETURN_IF_ERROR(chains16(std::integral_constant<int, 11>{}, I2{}));
      if (groups16 == 3) RETURN_IF_ERROR(chains16(std::integral_constant<int, 11>{}, I3{}));
      if (groups16 == 4) RETURN_IF_ERROR(chains16(std::integral_constant<int, 11>{}, I4{}));
      if (groups16 == 5) RETURN_IF_ERROR(chains16(std::integral_constant<int, 11>{}, I5{}));
    } else if (c.tables16 != nullptr && fits16 && logd == 12) {
      if (groups16 == 2) RETURN_IF_ERROR(chains16(std::integral_constant<int, 12>{}, I2{}));
      if (groups16 == 3) RETURN_IF_ERROR(chains16(std::integral_constant<int, 12>{}, I3{}));
    } else if (c.tables16 != nullptr && fits16 && logd == 13) {
      RETURN_IF_ERROR(chains16(std::integral_constant<int, 13>{}, I1{}));
    } else if (iters == 2) {
      RETURN_IF_ERROR(chains(std::integral_constant<int, 2>{}));
    } else {
      RETURN_IF_ERROR(chains(std::integral_constant<int, 1>{}));
    }
    // BuildPreprocessMatrix, one d x d block per digit plane l.
    for (int l = 0; l < k; ++l) {
      const int64_t cells = static_cast<int64_t>(d) * d;
      pp_block_input_kernel<T><<<dim3(static_cast<unsigned>((cells + 255) / 256), slices), 256,
                                 0, cs>>>(dtg.get<T>(), dtgh.get<T>(), dsrc.get<int>(), d, logd,
                                          k, l, chain_stride, dev0.get<T>());
      DevBuf* mev = transform(&dev0, false);
      switch (mat_kind) {
        case INSPIRE_I16:
          pp_matrix_kernel<T, int16_t><<<tgrid, dim3(32, 8), 0, cs>>>(
              mev->get<T>(), d, logd, log_modulus, k, l, static_cast<int16_t*>(m_out));
          break;
        case INSPIRE_I32:
          pp_matrix_kernel<T, int32_t><<<tgrid, dim3(32, 8), 0, cs>>>(
              mev->get<T>(), d, logd, log_modulus, k, l, static_cast<int32_t*>(m_out));
          break;
        default:
          pp_matrix_kernel<T, T><<<tgrid, dim3(32, 8), 0, cs>>>(
              mev->get<T>(), d, logd, log_modulus, k, l, static_cast<T*>(m_out));
      }
      RETURN_IF_ERROR(Cuda(cudaGetLastError(), "matrix block"));
    }
    return Status{};
  };
  if (st.ok()) st = coeff_bits == 32 ? run(uint32_t{}) : run(uint64_t{});
  if (st.ok()) st = Cuda(cs == nullptr ? cudaDeviceSynchronize() : cudaStreamSynchronize(cs),
                         "PreprocessMatrixPack");
  if (st.ok() && !on_device) {
    st = Cuda(cudaMemcpy(a_tilde_agg, da.get(), da.bytes(), cudaMemcpyDeviceToHost), "copy");
    if (st.ok()) st = Cuda(cudaMemcpy(matrix, dm.get(), dm.bytes(), cudaMemcpyDeviceToHost), "copy");
    if (st.ok()) st = Cuda(cudaMemcpy(t_vec_h, dth.get(), dth.bytes(), cudaMemcpyDeviceToHost), "copy");
  }
  return Report(st, err, err_len);
}

int inspire_client_create_requests(const inspire_pir_params* params,
                                   const int8_t* secret_keys, const void* a_components,
                                   int64_t a_count, const int64_t* indices, int32_t batch,
                                   uint64_t seed, int32_t variance, void* first_dim,
                                   void* second_dim, void* packing_key, int32_t on_device,
                                   void* stream, char* err, size_t err_len) {
  using namespace inspire;
  auto fail = [&](const char* m) { return Report(Err(INSPIRE_INVALID_ARGUMENT, m), err, err_len); };
  if (params == nullptr) return fail("params is null.");
  const int cb = params->coeff_bits;
  if (cb != 32 && cb != 64) return fail("coeff_bits must be 32 or 64.");
  const int logd = params->log_degree;
  if (logd < 2 || logd > 13) return fail("log_degree must be in [2, 13].");
  const int d = 1 << logd;
  const int t = params->interpolation_degree;
  const int n = params->num_entries;
  if (t <= 0 || n <= 0 || n % t != 0) return fail("num_entries must be a multiple of t.");
  if (batch <= 0) return fail("batch must be positive.");
  if (params->plaintext_modulus == 0) return fail("Plaintext modulus must be positive.");
  const int64_t fd_len = n / t;
  const int ns = static_cast<int>((fd_len + d - 1) / d);
  const int ne = t > 1 ? params->eval_num_digits : 0;
  const int kp = params->pack_num_digits;
  const int64_t rows = ns + 2ll * ne + 2ll * kp;
  if (a_count != rows) {
    return fail("a_components must hold the first-dimension, second-dimension and "
                "packing a-components in that order.");
  }
  std::vector<int64_t> idx(batch);
  if (on_device) {
    Status s0 = Cuda(cudaMemcpy(idx.data(), indices, batch * 8, cudaMemcpyDeviceToHost), "copy");
    if (!s0.ok()) return Report(s0, err, err_len);
  } else {
    std::memcpy(idx.data(), indices, batch * 8);
  }
  for (int64_t x : idx) {
    if (x < 0 || x >= n) {
      return Report(Err(INSPIRE_INVALID_ARGUMENT, "Index out of bounds."), err, err_len);
    }
  }
  int r = 0;
  Status st = PrimesFor(BoundBits(1, d, cb, 2), &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(logd, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  const NttCtx c = tabs->Ctx(r);
  const cudaStream_t cs = on_device ? static_cast<cudaStream_t>(stream) : nullptr;
  const size_t w = cb / 8;
  DevBuf dkeys, da, didx, dshat, dfd, dsd, dpk;
  const int8_t* keys = secret_keys;
  const void* a_dev = a_components;
  void* fd_out = first_dim;
  void* sd_out = second_dim;
  void* pk_out = packing_key;
  if (!on_device) {
    st = dkeys.Upload(secret_keys, static_cast<size_t>(batch) * d);
    if (st.ok()) st = da.Upload(a_components, rows * d * w);
    if (st.ok()) st = didx.Upload(idx.data(), batch * 8);
    if (st.ok()) st = dfd.Alloc(static_cast<size_t>(batch) * fd_len * w);
    if (st.ok() && ne > 0) st = dsd.Alloc(static_cast<size_t>(batch) * 2 * ne * d * w);
    if (st.ok()) st = dpk.Alloc(static_cast<size_t>(batch) * 2 * kp * d * w);
    keys = dkeys.get<int8_t>();
    a_dev = da.get();
    fd_out = dfd.get();
    sd_out = dsd.get();
    pk_out = dpk.get();
  }
  if (st.ok()) st = dshat.Alloc(static_cast<size_t>(batch) * r * d * 4);
  ClientArgs ca;
  ca.d = d;
  ca.log_d = logd;
  ca.log_q = params->log_modulus;
  ca.k_pack = kp;
  ca.ne = ne;
  ca.ns = ns;
  ca.t = t;
  ca.fd_len = fd_len;
  ca.pack_log_digit = params->pack_log_digit;
  ca.eval_log_digit = params->eval_log_digit;
  ca.var = variance;
  ca.seed = seed;
  ca.plaintext_modulus = params->plaintext_modulus;
  ca.keys = keys;
  ca.index = on_device ? indices : didx.get<int64_t>();
  const int iters = d > 4096 ? 2 : 1;
  const int threads = d / (4 * iters);
  const size_t smem = static_cast<size_t>(r) * d * 4;
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    auto go = [&](auto itag) -> Status {
      constexpr int IT = decltype(itag)::value;
      RETURN_IF_ERROR(SetSmem(cl_key_ntt_kernel<IT>, d * 4));
      RETURN_IF_ERROR(SetSmem(cl_request_kernel<T, IT>, smem));
      cl_key_ntt_kernel<IT><<<dim3(r, batch), threads, d * 4, cs>>>(keys, c,
                                                                     dshat.get<uint32_t>());
      cl_request_kernel<T, IT><<<dim3(static_cast<unsigned>(rows), batch), threads, smem, cs>>>(
          static_cast<const T*>(a_dev), dshat.get<uint32_t>(), ca, c, static_cast<T*>(fd_out),
          static_cast<T*>(sd_out), static_cast<T*>(pk_out));
      return Cuda(cudaGetLastError(), "client requests");
    };
    return iters == 2 ? go(std::integral_constant<int, 2>{}) : go(std::integral_constant<int, 1>{});
  };
  if (st.ok()) st = cb == 32 ? run(uint32_t{}) : run(uint64_t{});
  if (st.ok()) st = Cuda(cs == nullptr ? cudaDeviceSynchronize() : cudaStreamSynchronize(cs),
                         "client requests");
  if (st.ok() && !on_device) {
    st = Cuda(cudaMemcpy(first_dim, dfd.get(), dfd.bytes(), cudaMemcpyDeviceToHost), "copy");
    if (st.ok() && ne > 0) {
      st = Cuda(cudaMemcpy(second_dim, dsd.get(), dsd.bytes(), cudaMemcpyDeviceToHost), "copy");
    }
    if (st.ok()) st = Cuda(cudaMemcpy(packing_key, dpk.get(), dpk.bytes(), cudaMemcpyDeviceToHost), "copy");
  }
  return Report(st, err, err_len);
}

int inspire_client_process_responses(const inspire_pir_params* params,
                                     const int8_t* secret_keys, const void* responses,
                                     int32_t batch, void* out, int32_t on_device, void* stream,
                                     char* err, size_t err_len) {
  using namespace inspire;
  auto fail = [&](const char* m) { return Report(Err(INSPIRE_INVALID_ARGUMENT, m), err, err_len); };
  if (params == nullptr) return fail("params is null.");
  const int cb = params->coeff_bits;
  if (cb != 32 && cb != 64) return fail("coeff_bits must be 32 or 64.");
  const int logd = params->log_degree;
  if (logd < 2 || logd > 13) return fail("log_degree must be in [2, 13].");
  if (params->plaintext_modulus == 0) return fail("Plaintext modulus must be positive.");
  if (batch <= 0) return fail("batch must be positive.");
  const int d = 1 << logd;
  const int l = params->entry_size_multiple;
  if (l <= 0) return fail("entry_size_multiple must be positive.");
  int r = 0;
  Status st = PrimesFor(BoundBits(1, d, cb, 2), &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(logd, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  const NttCtx c = tabs->Ctx(r);
  const cudaStream_t cs = on_device ? static_cast<cudaStream_t>(stream) : nullptr;
  const size_t w = cb / 8;
  DevBuf dkeys, dresp, dout, dshat;
  const int8_t* keys = secret_keys;
  const void* resp = responses;
  void* o = out;
  if (!on_device) {
    st = dkeys.Upload(secret_keys, static_cast<size_t>(batch) * d);
    if (st.ok()) st = dresp.Upload(responses, static_cast<size_t>(batch) * l * 2 * d * w);
    if (st.ok()) st = dout.Alloc(static_cast<size_t>(batch) * l * d * w);
    keys = dkeys.get<int8_t>();
    resp = dresp.get();
    o = dout.get();
  }
  if (st.ok()) st = dshat.Alloc(static_cast<size_t>(batch) * r * d * 4);
  const int iters = d > 4096 ? 2 : 1;
  const int threads = d / (4 * iters);
  const size_t smem = static_cast<size_t>(r) * d * 4;
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    auto go = [&](auto itag) -> Status {
      constexpr int IT = decltype(itag)::value;
      RETURN_IF_ERROR(SetSmem(cl_key_ntt_kernel<IT>, d * 4));
      RETURN_IF_ERROR(SetSmem(cl_decrypt_kernel<T, IT>, smem));
      cl_key_ntt_kernel<IT><<<dim3(r, batch), threads, d * 4, cs>>>(keys, c,
                                                                     dshat.get<uint32_t>());
      cl_decrypt_kernel<T, IT><<<dim3(l, batch), threads, smem, cs>>>(
          static_cast<const T*>(resp), dshat.get<uint32_t>(), l,
          params->log_modulus1_after_switch, params->log_modulus2_after_switch,
          params->plaintext_modulus, c, static_cast<T*>(o));
      return Cuda(cudaGetLastError(), "client decryption");
    };
    return iters == 2 ? go(std::integral_constant<int, 2>{}) : go(std::integral_constant<int, 1>{});
  };
  if (st.ok()) st = cb == 32 ? run(uint32_t{}) : run(uint64_t{});
  if (st.ok()) st = Cuda(cs == nullptr ? cudaDeviceSynchronize() : cudaStreamSynchronize(cs),
                         "client decryption");
  if (st.ok() && !on_device) {
    st = Cuda(cudaMemcpy(out, dout.get(), dout.bytes(), cudaMemcpyDeviceToHost), "copy");
  }
  return Report(st, err, err_len);
}

int inspire_finalize_matrix_pack(const inspire_pir_params* params,
                                 const void* b, const void* b_agg_partial,
                                 const void* y_vec_h, const void* t_vec_h,
                                 void* out_b, char* err, size_t err_len) {
  using namespace inspire;
  if (params == nullptr) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "params is null."), err, err_len);
  }
  const int cb = params->coeff_bits;
  const int d = 1 << params->log_degree;
  const int k = params->pack_num_digits;
  if (k <= 0) {
    return Report(Err(INSPIRE_INVALID_ARGUMENT, "InnerProduct: size mismatch or empty"),
                  err, err_len);
  }
  ChunkRule rf;
  Status st = MakeRule(cb, k, d, params->pack_log_digit, params->log_modulus,
                       ChunkFor(k, d), &rf);
  if (!st.ok()) return Report(st, err, err_len);
  int r = 0;
  st = PrimesFor(BoundBits(k, d, std::min(rf.u_chunks * rf.chunk_bits, 64),
                           std::min(rf.v_chunks * rf.chunk_bits, cb)),
                 &r);
  if (!st.ok()) return Report(st, err, err_len);
  std::unique_ptr<NttTables> tabs;
  st = NttTables::Create(params->log_degree, &tabs);
  if (!st.ok()) return Report(st, err, err_len);
  NttCtx c = tabs->Ctx(r);
  const size_t w = cb / 8;
  std::vector<int64_t> th(static_cast<size_t>(k) * d);
  for (size_t i = 0; i < th.size(); ++i) {
    const uint64_t x = cb == 32 ? static_cast<const uint32_t*>(t_vec_h)[i]
                                : static_cast<const uint64_t*>(t_vec_h)[i];
    th[i] = RebuildU(x, rf, params->pack_log_digit, true);
  }
  DevBuf dth, dTh, dy, dYh, db1, db2, dout;
  st = dth.Upload(th.data(), th.size() * 8);
  if (st.ok()) st = dTh.Alloc(static_cast<size_t>(k) * r * d * 4);
  if (st.ok()) st = dy.Upload(y_vec_h, static_cast<size_t>(k) * d * w);
  if (st.ok()) st = dYh.Alloc(static_cast<size_t>(k) * r * d * 4);
  if (st.ok()) st = db1.Upload(b, d * w);
  if (st.ok()) st = db2.Upload(b_agg_partial, d * w);
  if (st.ok()) st = dout.Alloc(d * w);
  const uint64_t vmask = MaskBits(rf.v_chunks * rf.chunk_bits, cb);
  auto run = [&](auto tag) -> Status {
    using T = decltype(tag);
    ntt_signed_kernel<<<k * r, kPolyThreads, d * 4>>>(dth.get<int64_t>(), k,
                                                      dTh.get<uint32_t>(), c);
    ntt_coeffs_kernel<T><<<dim3(k * r, 1), kPolyThreads, d * 4>>>(
        dy.get<T>(), 0, 0, k, static_cast<T>(vmask), dYh.get<uint32_t>(), d, c);
    const size_t smem = static_cast<size_t>(r) * d * 4;
    RETURN_IF_ERROR(SetSmem(finalize_kernel<T>, smem));
    finalize_kernel<T><<<dim3(1, 1), kPolyThreads, smem>>>(
        dTh.get<uint32_t>(), dYh.get<uint32_t>(), k, db1.get<T>(), db2.get<T>(), 0,
        dout.get<T>(), params->log_modulus, c);
    return Cuda(cudaDeviceSynchronize(), "finalize");
  };
  if (st.ok()) st = cb == 32 ? run(uint32_t{}) : run(uint64_t{});
  if (st.ok()) st = Cuda(cudaMemcpy(out_b, dout.get(), d * w, cudaMemcpyDeviceToHost), "copy");
  return Report(st, err, err_len);
}

}  // extern "C"
