// CPU oracle for the ReinsPIRe online answer path -- TEST INFRASTRUCTURE ONLY.
//
// A dependency-free C++17 restatement of the reference server algorithm
// (google/InsPIRe). Each function names the reference file:line it follows.
// The product (inspire_gb300/) never links or loads this file; it is used by
// tests/, the smoke check and bench.py's CPU-baseline leg as the checker.
//
// Build: oracle/build_oracle.py (g++ -O3 -std=c++17 -ffp-contract=off, no
// target-specific flags, so x86_64 and aarch64 builds round identically).
#include "pir_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <chrono>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

using u128 = unsigned __int128;

constexpr int kInvalidArgument = 3;
constexpr int kFailedPrecondition = 9;
constexpr int kInternal = 13;

struct Status {
  int code = 0;
  std::string msg;
  bool ok() const { return code == 0; }
};

Status Error(int code, std::string msg) { return Status{code, std::move(msg)}; }

int Report(const Status& s, char* err, size_t err_len) {
  if (!s.ok() && err != nullptr && err_len > 0) {
    std::snprintf(err, err_len, "%s", s.msg.c_str());
  }
  return s.code;
}

template <typename T>
constexpr int kBits = 8 * sizeof(T);

// ---------------------------------------------------------------------------
// Coefficient helpers: crypto/polynomial.cc:254-338.
// ---------------------------------------------------------------------------
template <typename T>
T LowBitsOf(T x, int amount) {  // Polynomial::LowBits, polynomial.cc:323-338
  if (amount >= kBits<T>) return x;
  return x & ((T{1} << amount) - 1);
}

template <typename T>
T RightShiftOf(T x, int amount) {  // Polynomial::RightShift, :306-321
  if (amount >= kBits<T>) return 0;
  return x >> amount;
}

// Polynomial::Rescale, polynomial.cc:287-304: round(c * 2^new / 2^cur) in
// 128-bit arithmetic on the full CoeffType value.
template <typename T>
T RescaleOf(T c, int log_cur, int log_new) {
  u128 cur = static_cast<u128>(T{1}) << log_cur;
  u128 nw = static_cast<u128>(T{1}) << log_new;
  return static_cast<T>((static_cast<u128>(c) * nw + cur / 2) / cur);
}

// Polynomial::GadgetInv, polynomial.cc:340-374. out holds num_digits polys.
template <typename T>
Status GadgetInv(const T* p, int d, int log_modulus, int log_digit,
                 int num_digits, T* out) {
  if (log_digit <= 0 || num_digits <= 0) {
    return Error(kInvalidArgument,
                 "log_digit and num_digits must be positive.");
  }
  if (log_modulus == 0) log_modulus = kBits<T>;
  const int to_shift = log_modulus - num_digits * log_digit;
  for (int j = 0; j < d; ++j) {
    T cur = p[j];
    if (to_shift > 0) {
      const T round_val = T{1} << (to_shift - 1);
      cur = static_cast<T>((static_cast<u128>(cur) + round_val) >> to_shift);
    }
    for (int i = 0; i < num_digits; ++i) {
      out[static_cast<size_t>(i) * d + j] = LowBitsOf(cur, log_digit);
      cur = RightShiftOf(cur, log_digit);
    }
  }
  return Status{};
}

// Polynomial::SignedGadgetInv, polynomial.cc:376-427.
template <typename T>
Status SignedGadgetInv(const T* p, int d, int log_modulus, int log_digit,
                       int num_digits, T* out) {
  if (log_digit <= 0 || num_digits <= 0) {
    return Error(kInvalidArgument,
                 "log_digit and num_digits must be positive.");
  }
  if (log_modulus == 0) log_modulus = kBits<T>;
  using S = std::make_signed_t<T>;
  const int to_shift = log_modulus - num_digits * log_digit;
  std::vector<T> cur(p, p + d);
  if (to_shift > 0) {
    const T round_val = T{1} << (to_shift - 1);
    for (int j = 0; j < d; ++j) {
      cur[j] = static_cast<T>((static_cast<u128>(cur[j]) + round_val) >>
                              to_shift);
    }
  }
  const T mask = (T{1} << log_digit) - 1;
  const T half = T{1} << (log_digit - 1);
  for (int i = 0; i < num_digits; ++i) {
    for (int j = 0; j < d; ++j) {
      const T lower = cur[j] & mask;
      T digit;
      if (lower >= half) {
        digit = static_cast<T>(static_cast<S>(lower) -
                               static_cast<S>(T{1} << log_digit));
        cur[j] = (cur[j] >> log_digit) + 1;
      } else {
        digit = lower;
        cur[j] = cur[j] >> log_digit;
      }
      out[static_cast<size_t>(i) * d + j] = digit;
    }
  }
  return Status{};
}

// Polynomial::Automorph, polynomial.cc:429-456.
template <typename T>
Status Automorph(const T* p, int d, int power, T* out) {
  if (power < 0 || power % 2 == 0 || power >= 2 * d) {
    return Error(kInvalidArgument,
                 "Automorphism power must be a non-negative odd integer less "
                 "than 2*N.");
  }
  std::fill(out, out + d, T{0});
  for (int i = 0; i < d; ++i) {
    int index = static_cast<int>((static_cast<int64_t>(i) * power) % (2 * d));
    if (index >= d) {
      out[index - d] -= p[i];
    } else {
      out[index] += p[i];
    }
  }
  return Status{};
}

// ---------------------------------------------------------------------------
// Matrix::Multiply, crypto/matrix.h:167-195 (scalar path) and the condensed
// Highway kernels, crypto/matrix.cc:261-462.
// ---------------------------------------------------------------------------
template <typename Out, typename M>
void ScalarMultiply(const M* m, int64_t rows, int64_t cols, const Out* v,
                    Out* out, int64_t row_begin, int64_t row_end) {
  for (int64_t i = row_begin; i < row_end; ++i) {
    Out acc = 0;
    const M* row = m + i * cols;
    for (int64_t j = 0; j < cols; ++j) {
      acc += static_cast<Out>(row[j]) * v[j];
    }
    out[i] = acc;
  }
}

template <typename Out, typename M>
void ScalarMultiplyThreaded(const M* m, int64_t rows, int64_t cols,
                            const Out* v, Out* out, int threads) {
  if (threads <= 1 || rows < 2 * threads) {
    ScalarMultiply(m, rows, cols, v, out, 0, rows);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (rows + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk;
    const int64_t e = std::min(rows, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=] { ScalarMultiply(m, rows, cols, v, out, b, e); });
  }
  for (auto& th : pool) th.join();
}

template <typename M>
Status MatrixMultiplyTyped(int coeff_bits, const M* m, int64_t rows,
                           int64_t cols, const void* v, void* out,
                           int threads) {
  if (coeff_bits == 32) {
    ScalarMultiplyThreaded(m, rows, cols, static_cast<const uint32_t*>(v),
                           static_cast<uint32_t*>(out), threads);
  } else if (coeff_bits == 64) {
    ScalarMultiplyThreaded(m, rows, cols, static_cast<const uint64_t*>(v),
                           static_cast<uint64_t*>(out), threads);
  } else {
    return Error(kInvalidArgument, "coeff_bits must be 32 or 64.");
  }
  return Status{};
}

Status MatrixMultiply(int kind, int coeff_bits, const void* m, int64_t rows,
                      int64_t cols, const void* v, void* out, int threads) {
  switch (kind) {
    case ORC_U8:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const uint8_t*>(m),
                                 rows, cols, v, out, threads);
    case ORC_U16:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const uint16_t*>(m),
                                 rows, cols, v, out, threads);
    case ORC_U32:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const uint32_t*>(m),
                                 rows, cols, v, out, threads);
    case ORC_U64:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const uint64_t*>(m),
                                 rows, cols, v, out, threads);
    case ORC_I16:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const int16_t*>(m),
                                 rows, cols, v, out, threads);
    case ORC_I32:
      return MatrixMultiplyTyped(coeff_bits, static_cast<const int32_t*>(m),
                                 rows, cols, v, out, threads);
    default:
      return Error(kInvalidArgument, "unknown matrix element kind.");
  }
}

// The condensed kernels keep `lanes` u64 accumulators; lane l of block b
// reads the packed word at column-word b*lanes+l and the de-interleaved vector
// entries that the Highway LoadInterleaved{2,4} / rearrangement produce
// (matrix.cc:283-291, 341-348, 399-407), then reduces the lanes.
Status CondensedMultiply(int kind, const void* mat, int64_t rows, int64_t cols,
                         const uint64_t* v, uint64_t* out, int lanes) {
  int per_word = 0;
  int field_bits = 0;
  switch (kind) {
    case ORC_U8: per_word = 8; field_bits = 8; break;
    case ORC_U16: per_word = 4; field_bits = 16; break;
    case ORC_I32: per_word = 2; field_bits = 32; break;
    default:
      return Error(kFailedPrecondition,
                   "CondensedMultiply is only supported for uint8_t, uint16_t, "
                   "and int32_t matrices.");
  }
  if (lanes <= 0 || cols % (static_cast<int64_t>(per_word) * lanes) != 0) {
    return Error(kInvalidArgument,
                 "Original columns must be a multiple of " +
                     std::to_string(per_word) + " * Lanes.");
  }
  const uint64_t* words = static_cast<const uint64_t*>(mat);
  const int64_t words_per_row = cols / per_word;
  const int64_t blocks = cols / (static_cast<int64_t>(per_word) * lanes);
  std::vector<uint64_t> acc(lanes);
  for (int64_t i = 0; i < rows; ++i) {
    std::fill(acc.begin(), acc.end(), 0);
    for (int64_t b = 0; b < blocks; ++b) {
      for (int l = 0; l < lanes; ++l) {
        const uint64_t w = words[i * words_per_row + b * lanes + l];
        const int64_t col0 = (b * lanes + l) * per_word;
        for (int k = 0; k < per_word; ++k) {
          uint64_t field;
          if (kind == ORC_I32) {
            // Sign-extending 32-bit fields (matrix.cc:357-364).
            const int64_t s = static_cast<int64_t>(w);
            field = static_cast<uint64_t>(
                k == 0 ? ((s << 32) >> 32) : (s >> 32));
          } else {
            const uint64_t mask = (uint64_t{1} << field_bits) - 1;
            field = (w >> (k * field_bits)) & mask;
          }
          acc[l] += field * v[col0 + k];
        }
      }
    }
    uint64_t sum = 0;
    for (int l = 0; l < lanes; ++l) sum += acc[l];
    out[i] = sum;
  }
  return Status{};
}

// The condensed DB product as the reference server runs it for a u64
// CoeffType (the DB is condensed only then, preprocessing_server.h:127-153):
// Highway's CondensedMultiply<uint16_t> (matrix.cc:261-318) or <uint8_t>
// (matrix.cc:376-462) de-interleaves the vector once into one array per
// field of a packed word, then sums field_k(word) * V_k[word] over a row's
// words in u64 lanes. Here the lanes are the compiler's: the loop over a
// row's words is a plain reduction that -O3 vectorises (mod-2^64 sums are
// associative, so the lane split does not change the result).
template <int kFields>
void CondensedRows(const uint64_t* words, int64_t wpr, const uint64_t* vt,
                   uint64_t* out, int64_t row_begin, int64_t row_end) {
  constexpr int kFieldBits = 64 / kFields;
  constexpr uint64_t kMask = (uint64_t{1} << kFieldBits) - 1;
  for (int64_t i = row_begin; i < row_end; ++i) {
    const uint64_t* row = words + i * wpr;
    uint64_t acc = 0;
    for (int64_t j = 0; j < wpr; ++j) {
      const uint64_t w = row[j];
      uint64_t s = 0;
      for (int k = 0; k < kFields; ++k) {
        s += ((w >> (k * kFieldBits)) & kMask) * vt[k * wpr + j];
      }
      acc += s;
    }
    out[i] = acc;
  }
}

// Condensed product of a u8 / u16 DB with a u64 vector on `threads` threads;
// false when the shape does not condense (the caller then uses the scalar
// product, as the reference does for uncondensed matrices).
bool CondensedDbProduct(int kind, const void* mat, int64_t rows, int64_t cols,
                        const uint64_t* v, uint64_t* out, int threads) {
  const int fields = kind == ORC_U16 ? 4 : kind == ORC_U8 ? 8 : 0;
  if (fields == 0 || cols % fields != 0) return false;
  const int64_t wpr = cols / fields;
  std::vector<uint64_t> vt(static_cast<size_t>(cols));
  for (int64_t j = 0; j < wpr; ++j) {
    for (int k = 0; k < fields; ++k) vt[k * wpr + j] = v[j * fields + k];
  }
  const uint64_t* words = static_cast<const uint64_t*>(mat);
  auto run = [&](int64_t b, int64_t e) {
    if (fields == 4) {
      CondensedRows<4>(words, wpr, vt.data(), out, b, e);
    } else {
      CondensedRows<8>(words, wpr, vt.data(), out, b, e);
    }
  };
  if (threads <= 1 || rows < 2 * threads) {
    run(0, rows);
    return true;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (rows + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk;
    const int64_t e = std::min(rows, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=] { run(b, e); });
  }
  for (auto& th : pool) th.join();
  return true;
}

// ---------------------------------------------------------------------------
// FP64 FFT: crypto/fft.h:50-151 (FftPlan<double,1>, ComputeFftInternal).
// ---------------------------------------------------------------------------
struct Fft64Plan {
  size_t n = 0;
  std::vector<size_t> bit_rev;
  std::vector<std::complex<double>> tw_fwd, tw_bwd;

  explicit Fft64Plan(size_t size) : n(size) {
    bit_rev.resize(n);
    size_t log_n = 0;
    while ((size_t{1} << log_n) < n) ++log_n;
    for (size_t i = 0; i < n; ++i) {
      size_t r = 0;
      for (size_t b = 0; b < log_n; ++b) {
        if (i & (size_t{1} << b)) r |= size_t{1} << (log_n - 1 - b);
      }
      bit_rev[i] = r;
    }
    tw_fwd.resize(n / 2);
    tw_bwd.resize(n / 2);
    const double pi = std::acos(-1.0);
    for (size_t i = 0; i < n / 2; ++i) {
      const double angle = -2.0 * pi * i / n;
      tw_fwd[i] = std::complex<double>(std::cos(angle), std::sin(angle));
      tw_bwd[i] = std::complex<double>(std::cos(-angle), std::sin(-angle));
    }
  }

  // Radix-2 decimation in time with a bit-reversed load, unnormalised.
  void Run(const std::complex<double>* in, std::complex<double>* out,
           const std::vector<std::complex<double>>& tw) const {
    for (size_t i = 0; i < n; ++i) out[bit_rev[i]] = in[i];
    for (size_t len = 2; len <= n; len <<= 1) {
      const size_t half = len >> 1;
      const size_t step = n / len;
      for (size_t i = 0; i < n; i += len) {
        for (size_t j = 0; j < half; ++j) {
          const std::complex<double> a = out[i + j];
          const std::complex<double> b = out[i + j + half] * tw[j * step];
          out[i + j] = a + b;
          out[i + j + half] = a - b;
        }
      }
    }
  }
};

struct ChunkRule {
  int chunk_bits;
  int u_chunks;
  int v_chunks;
};

template <typename T>
Status MakeChunkRule(int n, int d, int u_bits, int v_bits, int chunk_bits,
                     ChunkRule* rule) {
  if (u_bits <= 0 || v_bits <= 0 || chunk_bits <= 0 || chunk_bits > 63) {
    return Error(kInvalidArgument, "Invalid bits or chunk_bits.");
  }
  if (std::log2(n) + std::log2(d) + 2.0 * chunk_bits > 53.0) {
    return Error(kInvalidArgument,
                 "Potential precision overflow in accumulation.");
  }
  const int max_chunks = (kBits<T> + chunk_bits - 1) / chunk_bits;
  rule->chunk_bits = chunk_bits;
  rule->u_chunks = std::min((u_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  rule->v_chunks = std::min((v_bits + chunk_bits - 1) / chunk_bits, max_chunks);
  return Status{};
}

// The value of chunk c of x as InnerProductFft forms it
// (polynomial_fft.cc:120-133, 141-147).
template <typename T>
int64_t ChunkValue(T x, int c, int chunk_bits, bool is_signed_last,
                   int total_bits) {
  const uint64_t mask = (uint64_t{1} << chunk_bits) - 1;
  const uint64_t chunk = (static_cast<uint64_t>(x) >> (chunk_bits * c)) & mask;
  if (is_signed_last) {
    const int bits_in_chunk = total_bits - chunk_bits * c;
    const int shift = 64 - bits_in_chunk;
    return static_cast<int64_t>(chunk << shift) >> shift;
  }
  return static_cast<int64_t>(chunk);
}

// InnerProductFft, polynomial_fft.cc:68-197, FP64 path.
template <typename T>
Status InnerProductFp64(const T* u, const T* v, int n, int d, int u_bits,
                        int v_bits, int chunk_bits, bool u_signed, T* out) {
  ChunkRule rule;
  Status s = MakeChunkRule<T>(n, d, u_bits, v_bits, chunk_bits, &rule);
  if (!s.ok()) return s;
  const int len2 = 2 * d;
  Fft64Plan plan(len2);
  const int uc = rule.u_chunks, vc = rule.v_chunks;
  std::vector<std::vector<std::complex<double>>> accum(
      uc * vc, std::vector<std::complex<double>>(len2, {0.0, 0.0}));
  std::vector<std::vector<std::complex<double>>> uf(
      uc, std::vector<std::complex<double>>(len2));
  std::vector<std::vector<std::complex<double>>> vf(
      vc, std::vector<std::complex<double>>(len2));
  std::vector<std::complex<double>> in(len2), tmp(len2);
  for (int i = 0; i < n; ++i) {
    const T* ui = u + static_cast<size_t>(i) * d;
    const T* vi = v + static_cast<size_t>(i) * d;
    for (int c = 0; c < uc; ++c) {
      for (int j = 0; j < len2; ++j) {
        double val = 0.0;
        if (j < d) {
          val = static_cast<double>(ChunkValue(
              ui[j], c, chunk_bits, u_signed && c == uc - 1, u_bits));
        }
        in[j] = std::complex<double>(val, 0.0);
      }
      plan.Run(in.data(), tmp.data(), plan.tw_fwd);
      uf[c] = tmp;
    }
    for (int c = 0; c < vc; ++c) {
      for (int j = 0; j < len2; ++j) {
        in[j] = std::complex<double>(
            j < d ? static_cast<double>(
                        ChunkValue(vi[j], c, chunk_bits, false, v_bits))
                  : 0.0,
            0.0);
      }
      plan.Run(in.data(), tmp.data(), plan.tw_fwd);
      vf[c] = tmp;
    }
    for (int a = 0; a < uc; ++a) {
      for (int b = 0; b < vc; ++b) {
        if (chunk_bits * (a + b) >= kBits<T>) continue;
        auto& acc = accum[a * vc + b];
        for (int j = 0; j < len2; ++j) acc[j] += uf[a][j] * vf[b][j];
      }
    }
  }
  std::fill(out, out + d, T{0});
  for (int a = 0; a < uc; ++a) {
    for (int b = 0; b < vc; ++b) {
      const int shift = chunk_bits * (a + b);
      if (shift >= kBits<T>) continue;
      plan.Run(accum[a * vc + b].data(), tmp.data(), plan.tw_bwd);
      for (int j = 0; j < len2; ++j) {
        const double val_double = tmp[j].real() / len2;
        const int64_t val64 = static_cast<int64_t>(std::round(val_double));
        const T val = static_cast<T>(static_cast<uint64_t>(val64));
        if (j < d) {
          out[j] += static_cast<T>(val << shift);
        } else {
          out[j - d] -= static_cast<T>(val << shift);
        }
      }
    }
  }
  return Status{};
}

// The exact integer value of InnerProductFft: sum_i u_eff_i (*) v_eff_i in
// Z_{2^w}[X]/(X^d+1), where u_eff / v_eff are the operands rebuilt from the
// same chunks the FFT path transforms. Pairs of chunks whose shift reaches
// 8*sizeof(T) contribute multiples of 2^w, so skipping them changes nothing.
template <typename T>
Status InnerProductExact(const T* u, const T* v, int n, int d, int u_bits,
                         int v_bits, int chunk_bits, bool u_signed, T* out) {
  ChunkRule rule;
  Status s = MakeChunkRule<T>(n, d, u_bits, v_bits, chunk_bits, &rule);
  if (!s.ok()) return s;
  std::vector<uint64_t> acc(d, 0), ue(d), ve(d);
  for (int i = 0; i < n; ++i) {
    const T* ui = u + static_cast<size_t>(i) * d;
    const T* vi = v + static_cast<size_t>(i) * d;
    for (int j = 0; j < d; ++j) {
      uint64_t x = 0;
      for (int c = 0; c < rule.u_chunks; ++c) {
        const int64_t cv = ChunkValue(ui[j], c, chunk_bits,
                                      u_signed && c == rule.u_chunks - 1,
                                      u_bits);
        x += static_cast<uint64_t>(cv) << (chunk_bits * c);
      }
      ue[j] = x;
      uint64_t y = 0;
      for (int c = 0; c < rule.v_chunks; ++c) {
        y += static_cast<uint64_t>(
                 ChunkValue(vi[j], c, chunk_bits, false, v_bits))
             << (chunk_bits * c);
      }
      ve[j] = y;
    }
    // Negacyclic schoolbook product, wrapping mod 2^64.
    for (int a = 0; a < d; ++a) {
      const uint64_t x = ue[a];
      if (x == 0) continue;
      for (int b = 0; b < d - a; ++b) acc[a + b] += x * ve[b];
      for (int b = d - a; b < d; ++b) acc[a + b - d] -= x * ve[b];
    }
  }
  for (int j = 0; j < d; ++j) out[j] = static_cast<T>(acc[j]);
  return Status{};
}

template <typename T>
Status InnerProduct(int mode, const T* u, const T* v, int n, int d, int u_bits,
                    int v_bits, int chunk_bits, bool u_signed, T* out) {
  if (n <= 0) {
    return Error(kInvalidArgument, "Polynomial vectors cannot be empty.");
  }
  if (mode == ORC_MODE_FP64) {
    return InnerProductFp64(u, v, n, d, u_bits, v_bits, chunk_bits, u_signed,
                            out);
  }
  return InnerProductExact(u, v, n, d, u_bits, v_bits, chunk_bits, u_signed,
                           out);
}

// Chunk size chosen by the InnerProduct wrapper (lwes_to_rlwe.cc:60-74) and
// by ExternalProduct (external_product.cc:100-102).
int ChunkFor(int num_polys, int d) {
  const int max_allowed =
      static_cast<int>((53.0 - std::log2(num_polys) - std::log2(d)) / 2.0);
  return std::min(20, max_allowed);
}

// ---------------------------------------------------------------------------
// FinalizeMatrixPack, crypto/lwes_to_rlwe.cc:448-479.
// ---------------------------------------------------------------------------
template <typename T>
Status FinalizeMatrixPack(const orc_params& p, int mode, const T* b,
                          const T* b_agg_partial, const T* y_vec_h,
                          const T* t_vec_h, T* out_b) {
  const int d = 1 << p.log_degree;
  const int k = p.pack_num_digits;
  std::vector<T> agg(d);
  for (int m = 0; m < d; ++m) {
    agg[m] = LowBitsOf<T>(static_cast<T>(b[m] + b_agg_partial[m]),
                          p.log_modulus);
  }
  std::vector<T> inner(d);
  Status s = InnerProduct<T>(mode, t_vec_h, y_vec_h, k, d, p.pack_log_digit,
                             p.log_modulus, ChunkFor(k, d), true,
                             inner.data());
  if (!s.ok()) return s;
  for (int m = 0; m < d; ++m) {
    out_b[m] = LowBitsOf<T>(static_cast<T>(agg[m] + inner[m]), p.log_modulus);
  }
  return Status{};
}

// ---------------------------------------------------------------------------
// ExternalProduct, crypto/external_product.cc:35-114. rgsw layout:
// u[i].a, u[i].b for i < nd, then v[i].a, v[i].b.
// ---------------------------------------------------------------------------
template <typename T>
Status ExternalProduct(const orc_params& p, int mode, const T* ct_a,
                       const T* ct_b, const T* rgsw, T* out_a, T* out_b) {
  const int d = 1 << p.log_degree;
  const int nd = p.eval_num_digits;
  const int log_q = p.log_modulus;
  std::vector<T> a_mod(d), b_mod(d);
  for (int j = 0; j < d; ++j) {
    a_mod[j] = LowBitsOf(ct_a[j], log_q);
    b_mod[j] = LowBitsOf(ct_b[j], log_q);
  }
  // Joined operand lists: [g^-1(a) ; g^-1(b)] against [u.a ; v.a] and
  // [u.b ; v.b].
  std::vector<T> digits(static_cast<size_t>(2) * nd * d);
  Status s = GadgetInv<T>(a_mod.data(), d, p.log_modulus, p.eval_log_digit, nd,
                          digits.data());
  if (!s.ok()) return s;
  s = GadgetInv<T>(b_mod.data(), d, p.log_modulus, p.eval_log_digit, nd,
                   digits.data() + static_cast<size_t>(nd) * d);
  if (!s.ok()) return s;
  std::vector<T> va(static_cast<size_t>(2) * nd * d),
      vb(static_cast<size_t>(2) * nd * d);
  for (int i = 0; i < 2 * nd; ++i) {
    const T* pa = rgsw + static_cast<size_t>(2 * i) * d;
    const T* pb = pa + d;
    std::copy(pa, pa + d, va.begin() + static_cast<size_t>(i) * d);
    std::copy(pb, pb + d, vb.begin() + static_cast<size_t>(i) * d);
  }
  const int chunk = ChunkFor(2 * nd, d);
  s = InnerProduct<T>(mode, digits.data(), va.data(), 2 * nd, d,
                      p.eval_log_digit, log_q, chunk, false, out_a);
  if (!s.ok()) return s;
  return InnerProduct<T>(mode, digits.data(), vb.data(), 2 * nd, d,
                         p.eval_log_digit, log_q, chunk, false, out_b);
}

// ---------------------------------------------------------------------------
// PirServer::ProcessResponse, crypto/pir/server/pir_server.cc:154-306,
// including EvalPoly (:128-150).
// ---------------------------------------------------------------------------
template <typename T>
Status ProcessResponse(const orc_params& p, int mode, int db_kind,
                       const void* db, int64_t db_cols, int pack_kind,
                       const void* pack, int64_t pack_cols,
                       const T* a_tilde_agg, const T* t_vec_h,
                       const T* second_dim_a, const T* first_dim,
                       int64_t first_dim_len, const T* second_dim,
                       int64_t second_dim_count, const T* packing_key,
                       int64_t packing_key_count, T* out, int threads,
                       double* stage_ms = nullptr, bool condensed_db = false) {
  using Clock = std::chrono::steady_clock;
  auto ms_since = [](Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0)
        .count();
  };
  double db_ms = 0, pack_ms = 0, eval_ms = 0;
  const int d = 1 << p.log_degree;
  const int t = p.interpolation_degree;
  const int l = p.entry_size_multiple;
  const int kd = p.pack_num_digits;
  const int ne = p.eval_num_digits;
  const int64_t rows = static_cast<int64_t>(l) * t * d;

  if (packing_key_count != 2 * kd) {
    return Error(kInvalidArgument,
                 "Packing key must contain 2 * num_digits polynomials.");
  }
  const T* y_vec_g = packing_key;
  const T* y_vec_h = packing_key + static_cast<size_t>(kd) * d;
  const int64_t interpolated_rows = p.num_entries / t;
  if (first_dim_len < interpolated_rows || first_dim_len > db_cols) {
    return Error(kInvalidArgument,
                 "First dimension query size (" +
                     std::to_string(first_dim_len) +
                     ") is invalid for DB columns (" +
                     std::to_string(db_cols) + ").");
  }
  if (t > 1 && second_dim_count != 2 * ne) {
    return Error(kInvalidArgument,
                 "second_dimension_query size mismatch. Must be 2 * "
                 "num_digits.");
  }
  if (p.log_degree < 0 || p.log_degree > 30) {
    return Error(kInvalidArgument, "Invalid log_d.");
  }
  // RGSW ciphertext: u[i] = (second_dim_a[i], q2[i]), v[i] likewise
  // (pir_server.cc:189-205).
  std::vector<T> rgsw;
  if (t > 1) {
    rgsw.resize(static_cast<size_t>(4) * ne * d);
    for (int i = 0; i < 2 * ne; ++i) {
      std::copy(second_dim_a + static_cast<size_t>(i) * d,
                second_dim_a + static_cast<size_t>(i + 1) * d,
                rgsw.begin() + static_cast<size_t>(2 * i) * d);
      std::copy(second_dim + static_cast<size_t>(i) * d,
                second_dim + static_cast<size_t>(i + 1) * d,
                rgsw.begin() + static_cast<size_t>(2 * i + 1) * d);
    }
  }
  // Stage 1: the DB product with the zero-padded first dimension
  // (timed as the reference's db_mult_time_, pir_server.cc:214-229).
  const auto t_db = Clock::now();
  std::vector<T> q1(db_cols, 0);
  std::copy(first_dim, first_dim + first_dim_len, q1.begin());
  std::vector<T> b_prime(rows);
  Status s;
  bool condensed = false;
  if (condensed_db && kBits<T> == 64) {
    condensed = CondensedDbProduct(
        db_kind, db, rows, db_cols, reinterpret_cast<const uint64_t*>(q1.data()),
        reinterpret_cast<uint64_t*>(b_prime.data()), threads);
  }
  if (!condensed) {
    s = MatrixMultiply(db_kind, kBits<T>, db, rows, db_cols, q1.data(),
                       b_prime.data(), threads);
    if (!s.ok()) return s;
  }
  db_ms = ms_since(t_db);
  // Stage 2: the packing product with the flattened y_vec_g (packing_time_
  // starts here, pir_server.cc:237).
  const auto t_pack = Clock::now();
  if (pack_cols != static_cast<int64_t>(kd) * d) {
    return Error(kInvalidArgument,
                 "Vector size must match the number of matrix columns.");
  }
  std::vector<T> b_agg_partial(rows);
  s = MatrixMultiply(pack_kind, kBits<T>, pack, rows, pack_cols, y_vec_g,
                     b_agg_partial.data(), threads);
  if (!s.ok()) return s;

  std::vector<T> packed_b(static_cast<size_t>(t) * d);
  std::vector<T> res_a(d), res_b(d), prod_a(d), prod_b(d);
  for (int k = 0; k < l; ++k) {
    for (int i = 0; i < t; ++i) {
      const size_t off = (static_cast<size_t>(k) * t + i) * d;
      s = FinalizeMatrixPack<T>(
          p, mode, b_prime.data() + off, b_agg_partial.data() + off, y_vec_h,
          t_vec_h + (static_cast<size_t>(k) * t + i) * kd * d,
          packed_b.data() + static_cast<size_t>(i) * d);
      if (!s.ok()) return s;
    }
    // The reference adds (now - start_pack) once per shard
    // (pir_server.cc:276), so for l > 1 its packing time counts the earlier
    // shards again; the same sum is kept here.
    pack_ms += ms_since(t_pack);
    const auto t_eval = Clock::now();
    // EvalPoly: Horner from the last coefficient, no LowBits between steps.
    const T* a_slice = a_tilde_agg + static_cast<size_t>(k) * t * d;
    std::copy(a_slice + static_cast<size_t>(t - 1) * d,
              a_slice + static_cast<size_t>(t) * d, res_a.begin());
    std::copy(packed_b.begin() + static_cast<size_t>(t - 1) * d,
              packed_b.begin() + static_cast<size_t>(t) * d, res_b.begin());
    for (int i = t - 2; i >= 0; --i) {
      s = ExternalProduct<T>(p, mode, res_a.data(), res_b.data(), rgsw.data(),
                             prod_a.data(), prod_b.data());
      if (!s.ok()) return s;
      for (int j = 0; j < d; ++j) {
        res_a[j] = prod_a[j] + a_slice[static_cast<size_t>(i) * d + j];
        res_b[j] = prod_b[j] + packed_b[static_cast<size_t>(i) * d + j];
      }
    }
    eval_ms += ms_since(t_eval);
    T* oa = out + static_cast<size_t>(2 * k) * d;
    T* ob = oa + d;
    for (int j = 0; j < d; ++j) {
      oa[j] = RescaleOf(res_a[j], p.log_modulus, p.log_modulus1_after_switch);
      ob[j] = RescaleOf(res_b[j], p.log_modulus, p.log_modulus2_after_switch);
    }
  }
  if (stage_ms != nullptr) {
    stage_ms[0] = db_ms;
    stage_ms[1] = pack_ms;
    stage_ms[2] = eval_ms;
  }
  return Status{};
}

// ---------------------------------------------------------------------------
// Interpolate, crypto/db_row_interpolation.cc:115-228.
// ---------------------------------------------------------------------------
// Multiply by X^power in Z_p[X]/(X^d+1) (db_row_interpolation.cc:44-75).
std::vector<uint32_t> XPowerTimes(const std::vector<uint32_t>& poly, int power,
                                  uint32_t p) {
  const int d = static_cast<int>(poly.size());
  power %= 2 * d;
  if (power < 0) power += 2 * d;
  bool negate_all = false;
  if (power >= d) {
    negate_all = true;
    power -= d;
  }
  std::vector<uint32_t> r(d);
  for (int i = 0; i < d; ++i) {
    bool neg = negate_all;
    uint32_t val;
    if (i < power) {
      val = poly[d - power + i];
      neg = !neg;
    } else {
      val = poly[i - power];
    }
    r[i] = (neg && val != 0) ? p - val : val;
  }
  return r;
}

// Extended Euclid modular inverse (db_row_interpolation.cc:82-111).
bool ModInverse(int64_t a, int64_t m, int64_t* inv) {
  int64_t t = 0, nt = 1, r = m, nr = a;
  while (nr != 0) {
    const int64_t q = r / nr;
    const int64_t tt = t - q * nt;
    t = nt;
    nt = tt;
    const int64_t rr = r - q * nr;
    r = nr;
    nr = rr;
  }
  if (r > 1) return false;
  if (t < 0) t += m;
  *inv = t;
  return true;
}

template <typename V>
Status Interpolate(const V* row, int d, int t, uint32_t pmod, V* out) {
  auto pow2 = [](unsigned x) { return x != 0 && (x & (x - 1)) == 0; };
  if (!pow2(static_cast<unsigned>(d))) {
    return Error(kInvalidArgument, "ring_degree must be a power of two.");
  }
  if (!pow2(static_cast<unsigned>(t))) {
    return Error(kInvalidArgument,
                 "interpolation_degree must be a power of two.");
  }
  if (t > 2 * d) {
    return Error(kInvalidArgument,
                 "interpolation_degree must be less than or equal to 2 * "
                 "ring_degree.");
  }
  const size_t total = static_cast<size_t>(d) * t;
  if (t == 1) {
    std::copy(row, row + total, out);
    return Status{};
  }
  if (pmod % 2 == 0) {
    return Error(kInvalidArgument, "plaintext_modulus must be odd.");
  }
  int log_t = 0;
  while ((1 << log_t) < t) ++log_t;
  auto bitrev = [](int n, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r = (r << 1) | ((n >> b) & 1);
    return r;
  };
  std::vector<std::vector<uint32_t>> polys(t, std::vector<uint32_t>(d));
  for (int i = 0; i < t; ++i) {
    auto& dst = polys[bitrev(i, log_t)];
    for (int j = 0; j < d; ++j) {
      dst[j] = static_cast<uint32_t>(row[static_cast<size_t>(i) * d + j]) %
               pmod;
    }
  }
  for (int len = 2; len <= t; len <<= 1) {
    const int half = len / 2;
    const int step = (2 * d - 2 * d / len) % (2 * d);
    for (int i = 0; i < t; i += len) {
      int w = 0;
      for (int j = 0; j < half; ++j) {
        const auto& u = polys[i + j];
        const auto v = XPowerTimes(polys[i + j + half], w, pmod);
        std::vector<uint32_t> s(d), df(d);
        for (int c = 0; c < d; ++c) {
          s[c] = static_cast<uint32_t>((static_cast<uint64_t>(u[c]) + v[c]) %
                                       pmod);
          df[c] = static_cast<uint32_t>(
              (static_cast<uint64_t>(u[c]) + pmod - v[c]) % pmod);
        }
        polys[i + j] = std::move(s);
        polys[i + j + half] = std::move(df);
        w = (w + step) % (2 * d);
      }
    }
  }
  int64_t tinv = 0;
  if (!ModInverse(static_cast<int64_t>(t % pmod), pmod, &tinv)) {
    return Error(kInvalidArgument,
                 "a is not invertible modulo m (not coprime).");
  }
  for (int i = 0; i < t; ++i) {
    for (int j = 0; j < d; ++j) {
      out[static_cast<size_t>(i) * d + j] = static_cast<V>(
          (static_cast<uint64_t>(polys[i][j]) * static_cast<uint64_t>(tinv)) %
          pmod);
    }
  }
  return Status{};
}

// ---------------------------------------------------------------------------
// PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:163-446): PreprocessPack,
// then BuildPreprocessMatrix; and Pack (lwes_to_rlwe.cc:356-412), the
// automorphism route the matrix replaces.
// ---------------------------------------------------------------------------
// 5^k mod 2d (ComputePower, lwes_to_rlwe.cc:77-83).
int PowerOf5(int k, int two_d) {
  int64_t r = 1;
  for (int i = 0; i < k; ++i) r = (r * 5) % two_d;
  return static_cast<int>(r);
}

// p * X^e in Z_{2^w}[X]/(X^d + 1), 0 <= e < 2d.
template <typename T>
void TimesXPower(const T* p, int d, int e, T* out) {
  const bool flip = e >= d;
  if (flip) e -= d;
  for (int i = 0; i < d; ++i) {
    T v = i < e ? static_cast<T>(T{0} - p[d - e + i]) : p[i - e];
    out[i] = flip ? static_cast<T>(T{0} - v) : v;
  }
}

// The values P(X^{2m}), m < d, of P(Z) = sum_i c[i] Z^i whose coefficients
// c[i] are ring elements (what EvaluateNttInPlace computes,
// lwes_to_rlwe.cc:88-119), by direct summation: out[m] = sum_i c[i] X^{2im}.
template <typename T>
void EvaluateAtEvenPowers(const std::vector<T>& c, int d, std::vector<T>* out) {
  out->assign(static_cast<size_t>(d) * d, T{0});
  std::vector<T> tmp(d);
  for (int m = 0; m < d; ++m) {
    T* o = out->data() + static_cast<size_t>(m) * d;
    for (int i = 0; i < d; ++i) {
      const int e = static_cast<int>((2ll * i * m) % (2 * d));
      TimesXPower(c.data() + static_cast<size_t>(i) * d, d, e, tmp.data());
      for (int r = 0; r < d; ++r) o[r] += tmp[r];
    }
  }
}

// Odd power of slot k of the packing order: 5^k for k < d/2, (2d-1) 5^{k-d/2}
// after (lwes_to_rlwe.cc:297-308).
int SlotPower(int k, int d) {
  if (k < d / 2) return PowerOf5(k, 2 * d);
  return static_cast<int>((static_cast<int64_t>(PowerOf5(k - d / 2, 2 * d)) *
                           (2 * d - 1)) % (2 * d));
}

// sum_l digits[l] (*) Automorph(w[l], power) as the InnerProduct wrapper
// computes it (a_bits = log_digit, b_bits = log_q, signed digits).
template <typename T>
Status AutInner(int mode, const T* digits, const T* w, int k, int d, int power,
                int log_digit, int log_q, T* out) {
  std::vector<T> aut(static_cast<size_t>(k) * d);
  for (int l = 0; l < k; ++l) {
    Status s = Automorph<T>(w + static_cast<size_t>(l) * d, d, power,
                            aut.data() + static_cast<size_t>(l) * d);
    if (!s.ok()) return s;
  }
  return InnerProduct<T>(mode, digits, aut.data(), k, d, log_digit, log_q,
                         ChunkFor(k, d), true, out);
}

// PreprocessPack (lwes_to_rlwe.cc:229-353). a_is: d rows of d words; w_g,
// w_h: k = num_digits polynomials. t_vec_g / t_vec_gh: (d/2 - 1) x k x d.
template <typename T>
Status PreprocessPack(int mode, int log_q, int log_digit, int k, int d,
                      const T* a_is, const T* w_g, const T* w_h, T* a_tilde_agg,
                      T* t_vec_g, T* t_vec_gh, T* t_vec_h) {
  int log2_d = 0;
  while ((1 << log2_d) < d) ++log2_d;
  const size_t dd = static_cast<size_t>(d) * d;
  // 1-2) a_tilde_j = LowBits(RightShift(LowBits(sum_m a_j[m] X^{-m}), log d)).
  std::vector<T> a_tilde(dd);
  for (int j = 0; j < d; ++j) {
    const T* a = a_is + static_cast<size_t>(j) * d;
    T* o = a_tilde.data() + static_cast<size_t>(j) * d;
    for (int m = 0; m < d; ++m) {
      const T v = m == 0 ? a[0] : static_cast<T>(T{0} - a[d - m]);
      o[m] = LowBitsOf<T>(static_cast<T>(LowBitsOf<T>(v, log_q) >> log2_d), log_q);
    }
  }
  // 3) P_m = X^m sum_j a_tilde_j[m] X^j, evaluated at Z = X^{2i}; slot order.
  std::vector<T> pk(dd), col(d), prime;
  for (int m = 0; m < d; ++m) {
    for (int j = 0; j < d; ++j) col[j] = a_tilde[static_cast<size_t>(j) * d + m];
    TimesXPower(col.data(), d, m, pk.data() + static_cast<size_t>(m) * d);
  }
  EvaluateAtEvenPowers(pk, d, &prime);
  auto hat = [&](int kk) {
    return prime.data() + static_cast<size_t>((SlotPower(kk, d) - 1) / 2) * d;
  };
  // 4) The two reduction chains.
  std::vector<T> tg(hat(d / 2 - 1), hat(d / 2 - 1) + d);
  std::vector<T> tgh(hat(d - 1), hat(d - 1) + d);
  std::vector<T> low(d), inner(d);
  for (int i = d / 2 - 2; i >= 0; --i) {
    const int pg = PowerOf5(i, 2 * d);
    const int pgh = static_cast<int>((static_cast<int64_t>(pg) * (2 * d - 1)) % (2 * d));
    T* dg = t_vec_g + static_cast<size_t>(i) * k * d;
    for (int r = 0; r < d; ++r) low[r] = LowBitsOf<T>(tg[r], log_q);
    Status s = SignedGadgetInv<T>(low.data(), d, log_q, log_digit, k, dg);
    if (!s.ok()) return s;
    s = AutInner<T>(mode, dg, w_g, k, d, pg, log_digit, log_q, inner.data());
    if (!s.ok()) return s;
    const T* ag = hat(i);
    for (int r = 0; r < d; ++r) tg[r] = static_cast<T>(ag[r] + inner[r]);

    T* dgh = t_vec_gh + static_cast<size_t>(i) * k * d;
    for (int r = 0; r < d; ++r) low[r] = LowBitsOf<T>(tgh[r], log_q);
    s = SignedGadgetInv<T>(low.data(), d, log_q, log_digit, k, dgh);
    if (!s.ok()) return s;
    s = AutInner<T>(mode, dgh, w_g, k, d, pgh, log_digit, log_q, inner.data());
    if (!s.ok()) return s;
    const T* agh = hat(d / 2 + i);
    for (int r = 0; r < d; ++r) tgh[r] = static_cast<T>(agh[r] + inner[r]);
  }
  for (int r = 0; r < d; ++r) low[r] = LowBitsOf<T>(tgh[r], log_q);
  Status s = SignedGadgetInv<T>(low.data(), d, log_q, log_digit, k, t_vec_h);
  if (!s.ok()) return s;
  s = InnerProduct<T>(mode, t_vec_h, w_h, k, d, log_digit, log_q, ChunkFor(k, d),
                      true, inner.data());
  if (!s.ok()) return s;
  for (int r = 0; r < d; ++r) {
    a_tilde_agg[r] = LowBitsOf<T>(static_cast<T>(tg[r] + inner[r]), log_q);
  }
  return Status{};
}

// BuildPreprocessMatrix (lwes_to_rlwe.cc:136-227): d x (k d) entries,
// centred mod 2^log_q, as signed 64-bit values (the caller narrows them to
// the matrix element type).
template <typename T>
void BuildPreprocessMatrix(int log_q, int k, int d, const T* t_vec_g,
                           const T* t_vec_gh, int64_t* matrix) {
  const size_t dd = static_cast<size_t>(d) * d;
  std::vector<T> t(dd), ev, colp(d);
  const int w = kBits<T>;
  const T threshold = (log_q == 0 || log_q >= w) ? (T{1} << (w - 1))
                                                : (T{1} << (log_q - 1));
  for (int l = 0; l < k; ++l) {
    std::fill(t.begin(), t.end(), T{0});
    for (int j = 0; j <= d / 2 - 2; ++j) {
      const int pg = PowerOf5(j, 2 * d);
      const int pgh = static_cast<int>((static_cast<int64_t>(pg) * (2 * d - 1)) % (2 * d));
      const T* src_g = t_vec_g + (static_cast<size_t>(j) * k + l) * d;
      const T* src_gh = t_vec_gh + (static_cast<size_t>(j) * k + l) * d;
      std::copy(src_g, src_g + d, t.data() + static_cast<size_t>((pg - 1) / 2) * d);
      std::copy(src_gh, src_gh + d, t.data() + static_cast<size_t>((pgh - 1) / 2) * d);
    }
    EvaluateAtEvenPowers(t, d, &ev);
    for (int c = 0; c < d; ++c) {
      TimesXPower(ev.data() + static_cast<size_t>(c) * d, d, c, colp.data());
      for (int r = 0; r < d; ++r) {
        T v = colp[r];
        if (v >= threshold && log_q < w) v = static_cast<T>(v - (T{1} << log_q));
        using S = std::make_signed_t<T>;
        matrix[static_cast<size_t>(r) * k * d + static_cast<size_t>(l) * d + c] =
            static_cast<int64_t>(static_cast<S>(v));
      }
    }
  }
}

// Pack (lwes_to_rlwe.cc:356-412): the b part of the packed ciphertext.
template <typename T>
Status Pack(int mode, int log_q, int log_digit, int k, int d, const T* b,
            const T* y_g, const T* y_h, const T* t_vec_g, const T* t_vec_gh,
            const T* t_vec_h, T* b_agg) {
  std::vector<T> acc(d), inner(d);
  for (int r = 0; r < d; ++r) acc[r] = LowBitsOf<T>(b[r], log_q);
  for (int j = 0; j <= d / 2 - 2; ++j) {
    const int pg = PowerOf5(j, 2 * d);
    const int pgh = static_cast<int>((static_cast<int64_t>(pg) * (2 * d - 1)) % (2 * d));
    Status s = AutInner<T>(mode, t_vec_g + static_cast<size_t>(j) * k * d, y_g, k,
                           d, pg, log_digit, log_q, inner.data());
    if (!s.ok()) return s;
    for (int r = 0; r < d; ++r) acc[r] = LowBitsOf<T>(static_cast<T>(acc[r] + inner[r]), log_q);
    s = AutInner<T>(mode, t_vec_gh + static_cast<size_t>(j) * k * d, y_g, k, d,
                    pgh, log_digit, log_q, inner.data());
    if (!s.ok()) return s;
    for (int r = 0; r < d; ++r) acc[r] = LowBitsOf<T>(static_cast<T>(acc[r] + inner[r]), log_q);
  }
  Status s = InnerProduct<T>(mode, t_vec_h, y_h, k, d, log_digit, log_q,
                             ChunkFor(k, d), true, inner.data());
  if (!s.ok()) return s;
  for (int r = 0; r < d; ++r) {
    b_agg[r] = LowBitsOf<T>(static_cast<T>(acc[r] + inner[r]), log_q);
  }
  return Status{};
}

}  // namespace

// ---------------------------------------------------------------------------
// C entry points.
// ---------------------------------------------------------------------------
extern "C" {

int orc_matrix_multiply(int mat_kind, int coeff_bits, const void* mat,
                        int64_t rows, int64_t cols, const void* v, void* out,
                        char* err, size_t err_len) {
  return Report(MatrixMultiply(mat_kind, coeff_bits, mat, rows, cols, v, out, 1),
                err, err_len);
}

int orc_condensed_multiply(int mat_kind, const void* mat, int64_t rows,
                           int64_t cols, const uint64_t* v, uint64_t* out,
                           int lanes, char* err, size_t err_len) {
  return Report(CondensedMultiply(mat_kind, mat, rows, cols, v, out, lanes),
                err, err_len);
}

int orc_inner_product(int coeff_bits, int mode, const void* u, const void* v,
                      int n, int d, int u_bits, int v_bits, int chunk_bits,
                      int u_is_signed, void* out, char* err, size_t err_len) {
  Status s;
  if (coeff_bits == 32) {
    s = InnerProduct<uint32_t>(mode, static_cast<const uint32_t*>(u),
                               static_cast<const uint32_t*>(v), n, d, u_bits,
                               v_bits, chunk_bits, u_is_signed != 0,
                               static_cast<uint32_t*>(out));
  } else {
    s = InnerProduct<uint64_t>(mode, static_cast<const uint64_t*>(u),
                               static_cast<const uint64_t*>(v), n, d, u_bits,
                               v_bits, chunk_bits, u_is_signed != 0,
                               static_cast<uint64_t*>(out));
  }
  return Report(s, err, err_len);
}

int orc_gadget_inv(int coeff_bits, const void* p, int d, int log_modulus,
                   int log_digit, int num_digits, void* out, char* err,
                   size_t err_len) {
  Status s = coeff_bits == 32
                 ? GadgetInv<uint32_t>(static_cast<const uint32_t*>(p), d,
                                       log_modulus, log_digit, num_digits,
                                       static_cast<uint32_t*>(out))
                 : GadgetInv<uint64_t>(static_cast<const uint64_t*>(p), d,
                                       log_modulus, log_digit, num_digits,
                                       static_cast<uint64_t*>(out));
  return Report(s, err, err_len);
}

int orc_signed_gadget_inv(int coeff_bits, const void* p, int d,
                          int log_modulus, int log_digit, int num_digits,
                          void* out, char* err, size_t err_len) {
  Status s = coeff_bits == 32
                 ? SignedGadgetInv<uint32_t>(static_cast<const uint32_t*>(p),
                                             d, log_modulus, log_digit,
                                             num_digits,
                                             static_cast<uint32_t*>(out))
                 : SignedGadgetInv<uint64_t>(static_cast<const uint64_t*>(p),
                                             d, log_modulus, log_digit,
                                             num_digits,
                                             static_cast<uint64_t*>(out));
  return Report(s, err, err_len);
}

int orc_rescale(int coeff_bits, const void* p, int d, int log_cur, int log_new,
                void* out) {
  for (int j = 0; j < d; ++j) {
    if (coeff_bits == 32) {
      static_cast<uint32_t*>(out)[j] = RescaleOf<uint32_t>(
          static_cast<const uint32_t*>(p)[j], log_cur, log_new);
    } else {
      static_cast<uint64_t*>(out)[j] = RescaleOf<uint64_t>(
          static_cast<const uint64_t*>(p)[j], log_cur, log_new);
    }
  }
  return 0;
}

int orc_automorph(int coeff_bits, const void* p, int d, int power, void* out,
                  char* err, size_t err_len) {
  Status s = coeff_bits == 32
                 ? Automorph<uint32_t>(static_cast<const uint32_t*>(p), d,
                                       power, static_cast<uint32_t*>(out))
                 : Automorph<uint64_t>(static_cast<const uint64_t*>(p), d,
                                       power, static_cast<uint64_t*>(out));
  return Report(s, err, err_len);
}

int orc_finalize_matrix_pack(const orc_params* prm, int mode, const void* b,
                             const void* b_agg_partial, const void* y_vec_h,
                             const void* t_vec_h, void* out_b, char* err,
                             size_t err_len) {
  Status s;
  if (prm->coeff_bits == 32) {
    s = FinalizeMatrixPack<uint32_t>(
        *prm, mode, static_cast<const uint32_t*>(b),
        static_cast<const uint32_t*>(b_agg_partial),
        static_cast<const uint32_t*>(y_vec_h),
        static_cast<const uint32_t*>(t_vec_h), static_cast<uint32_t*>(out_b));
  } else {
    s = FinalizeMatrixPack<uint64_t>(
        *prm, mode, static_cast<const uint64_t*>(b),
        static_cast<const uint64_t*>(b_agg_partial),
        static_cast<const uint64_t*>(y_vec_h),
        static_cast<const uint64_t*>(t_vec_h), static_cast<uint64_t*>(out_b));
  }
  return Report(s, err, err_len);
}

int orc_external_product(const orc_params* prm, int mode, const void* ct_a,
                         const void* ct_b, const void* rgsw, void* out_a,
                         void* out_b, char* err, size_t err_len) {
  Status s;
  if (prm->coeff_bits == 32) {
    s = ExternalProduct<uint32_t>(
        *prm, mode, static_cast<const uint32_t*>(ct_a),
        static_cast<const uint32_t*>(ct_b), static_cast<const uint32_t*>(rgsw),
        static_cast<uint32_t*>(out_a), static_cast<uint32_t*>(out_b));
  } else {
    s = ExternalProduct<uint64_t>(
        *prm, mode, static_cast<const uint64_t*>(ct_a),
        static_cast<const uint64_t*>(ct_b), static_cast<const uint64_t*>(rgsw),
        static_cast<uint64_t*>(out_a), static_cast<uint64_t*>(out_b));
  }
  return Report(s, err, err_len);
}

int orc_process_response_staged(
    const orc_params* prm, int mode, int db_kind, const void* db,
    int64_t db_cols, int pack_kind, const void* pack, int64_t pack_cols,
    const void* a_tilde_agg, const void* t_vec_h, const void* second_dim_a,
    const void* first_dim, int64_t first_dim_len, const void* second_dim,
    int64_t second_dim_count, const void* packing_key,
    int64_t packing_key_count, void* out, int threads, int condensed_db,
    double* stage_ms, char* err, size_t err_len) {
  Status s;
  if (prm->coeff_bits == 32) {
    using T = uint32_t;
    s = ProcessResponse<T>(
        *prm, mode, db_kind, db, db_cols, pack_kind, pack, pack_cols,
        static_cast<const T*>(a_tilde_agg), static_cast<const T*>(t_vec_h),
        static_cast<const T*>(second_dim_a), static_cast<const T*>(first_dim),
        first_dim_len, static_cast<const T*>(second_dim), second_dim_count,
        static_cast<const T*>(packing_key), packing_key_count,
        static_cast<T*>(out), threads, stage_ms, condensed_db != 0);
  } else {
    using T = uint64_t;
    s = ProcessResponse<T>(
        *prm, mode, db_kind, db, db_cols, pack_kind, pack, pack_cols,
        static_cast<const T*>(a_tilde_agg), static_cast<const T*>(t_vec_h),
        static_cast<const T*>(second_dim_a), static_cast<const T*>(first_dim),
        first_dim_len, static_cast<const T*>(second_dim), second_dim_count,
        static_cast<const T*>(packing_key), packing_key_count,
        static_cast<T*>(out), threads, stage_ms, condensed_db != 0);
  }
  return Report(s, err, err_len);
}

int orc_process_response(const orc_params* prm, int mode, int db_kind,
                         const void* db, int64_t db_cols, int pack_kind,
                         const void* pack, int64_t pack_cols,
                         const void* a_tilde_agg, const void* t_vec_h,
                         const void* second_dim_a, const void* first_dim,
                         int64_t first_dim_len, const void* second_dim,
                         int64_t second_dim_count, const void* packing_key,
                         int64_t packing_key_count, void* out, char* err,
                         size_t err_len) {
  Status s;
  if (prm->coeff_bits == 32) {
    using T = uint32_t;
    s = ProcessResponse<T>(
        *prm, mode, db_kind, db, db_cols, pack_kind, pack, pack_cols,
        static_cast<const T*>(a_tilde_agg), static_cast<const T*>(t_vec_h),
        static_cast<const T*>(second_dim_a), static_cast<const T*>(first_dim),
        first_dim_len, static_cast<const T*>(second_dim), second_dim_count,
        static_cast<const T*>(packing_key), packing_key_count,
        static_cast<T*>(out), 1);
  } else {
    using T = uint64_t;
    s = ProcessResponse<T>(
        *prm, mode, db_kind, db, db_cols, pack_kind, pack, pack_cols,
        static_cast<const T*>(a_tilde_agg), static_cast<const T*>(t_vec_h),
        static_cast<const T*>(second_dim_a), static_cast<const T*>(first_dim),
        first_dim_len, static_cast<const T*>(second_dim), second_dim_count,
        static_cast<const T*>(packing_key), packing_key_count,
        static_cast<T*>(out), 1);
  }
  return Report(s, err, err_len);
}

int orc_preprocess_matrix_pack(int coeff_bits, int mode, int log_modulus,
                               int log_digit, int num_digits, int d,
                               const void* a_is, const void* w_vec_g,
                               const void* w_vec_h, void* a_tilde_agg,
                               int64_t* matrix, void* t_vec_h, void* t_vec_g,
                               void* t_vec_gh, char* err, size_t err_len) {
  if (d < 4 || (d & (d - 1)) != 0) {
    return Report(Error(kInvalidArgument, "d must be a power of two >= 4."), err,
                  err_len);
  }
  const size_t n = static_cast<size_t>(d / 2 - 1) * num_digits * d;
  Status s;
  auto run = [&](auto tag) {
    using T = decltype(tag);
    std::vector<T> g(n), gh(n);
    s = PreprocessPack<T>(mode, log_modulus, log_digit, num_digits, d,
                          static_cast<const T*>(a_is), static_cast<const T*>(w_vec_g),
                          static_cast<const T*>(w_vec_h), static_cast<T*>(a_tilde_agg),
                          g.data(), gh.data(), static_cast<T*>(t_vec_h));
    if (!s.ok()) return;
    if (matrix != nullptr) {
      BuildPreprocessMatrix<T>(log_modulus, num_digits, d, g.data(), gh.data(), matrix);
    }
    if (t_vec_g != nullptr) std::copy(g.begin(), g.end(), static_cast<T*>(t_vec_g));
    if (t_vec_gh != nullptr) std::copy(gh.begin(), gh.end(), static_cast<T*>(t_vec_gh));
  };
  if (coeff_bits == 32) {
    run(uint32_t{});
  } else if (coeff_bits == 64) {
    run(uint64_t{});
  } else {
    s = Error(kInvalidArgument, "coeff_bits must be 32 or 64.");
  }
  return Report(s, err, err_len);
}

int orc_pack(int coeff_bits, int mode, int log_modulus, int log_digit,
             int num_digits, int d, const void* b, const void* y_vec_g,
             const void* y_vec_h, const void* t_vec_g, const void* t_vec_gh,
             const void* t_vec_h, void* b_agg, char* err, size_t err_len) {
  Status s;
  if (coeff_bits == 32) {
    using T = uint32_t;
    s = Pack<T>(mode, log_modulus, log_digit, num_digits, d, static_cast<const T*>(b),
                static_cast<const T*>(y_vec_g), static_cast<const T*>(y_vec_h),
                static_cast<const T*>(t_vec_g), static_cast<const T*>(t_vec_gh),
                static_cast<const T*>(t_vec_h), static_cast<T*>(b_agg));
  } else if (coeff_bits == 64) {
    using T = uint64_t;
    s = Pack<T>(mode, log_modulus, log_digit, num_digits, d, static_cast<const T*>(b),
                static_cast<const T*>(y_vec_g), static_cast<const T*>(y_vec_h),
                static_cast<const T*>(t_vec_g), static_cast<const T*>(t_vec_gh),
                static_cast<const T*>(t_vec_h), static_cast<T*>(b_agg));
  } else {
    s = Error(kInvalidArgument, "coeff_bits must be 32 or 64.");
  }
  return Report(s, err, err_len);
}

int orc_interpolate(int value_bits, const void* db_row, int d, int t,
                    uint32_t plaintext_modulus, void* out, char* err,
                    size_t err_len) {
  Status s;
  switch (value_bits) {
    case 8:
      s = Interpolate<uint8_t>(static_cast<const uint8_t*>(db_row), d, t,
                               plaintext_modulus, static_cast<uint8_t*>(out));
      break;
    case 16:
      s = Interpolate<uint16_t>(static_cast<const uint16_t*>(db_row), d, t,
                                plaintext_modulus, static_cast<uint16_t*>(out));
      break;
    case 32:
      s = Interpolate<uint32_t>(static_cast<const uint32_t*>(db_row), d, t,
                                plaintext_modulus, static_cast<uint32_t*>(out));
      break;
    default:
      s = Error(kInvalidArgument, "value_bits must be 8, 16 or 32.");
  }
  return Report(s, err, err_len);
}

}  // extern "C"
