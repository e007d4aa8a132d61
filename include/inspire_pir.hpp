// C++ mirror of the reference's PirServer API over the C ABI (inspire_pir.h).
//
// The reference's server interface (crypto/pir/server/pir_server.h:40-72):
//   template <typename DbDataType, typename CoeffType, typename MatCoeffType>
//   class PirServer {
//     static StatusOr<unique_ptr<PirServer>> Create(params, preprocessed data);
//     static StatusOr<unique_ptr<PirServer>> LoadFromBuffer(params, buf, size);
//     static StatusOr<unique_ptr<PirServer>> LoadFromFile(params, path);
//     Status SaveToFile(path) const;
//     StatusOr<PirResponse> ProcessResponse(const PirRequest&) const;
//     Duration GetDbMultiplyTime() / GetPackingTime() / GetPolyEvalTime();
//   };
// This header keeps those names, argument meanings and status codes with
// plain standard-library types (the reference's abseil, Polynomial and
// Matrix types are not part of this build): polynomials are std::vector
// of d coefficients, matrices row-major std::vector. Header-only; link
// against libinspire_gb300.so.
#ifndef INSPIRE_PIR_HPP_
#define INSPIRE_PIR_HPP_

#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "inspire_pir.h"

namespace inspire_gb300 {

// absl::Status shape: code 0 = OK, otherwise the absl::StatusCode number.
class Status {
 public:
  Status() = default;
  Status(int code, std::string message) : code_(code), message_(std::move(message)) {}
  bool ok() const { return code_ == INSPIRE_OK; }
  int code() const { return code_; }
  const std::string& message() const { return message_; }

 private:
  int code_ = INSPIRE_OK;
  std::string message_;
};

template <typename T>
class StatusOr {
 public:
  StatusOr(Status s) : status_(std::move(s)) {}  // NOLINT: absl-style
  StatusOr(T v) : value_(std::move(v)) {}        // NOLINT
  bool ok() const { return status_.ok(); }
  const Status& status() const { return status_; }
  T& value() { return value_; }
  T& operator*() { return value_; }
  T* operator->() { return &value_; }

 private:
  Status status_;
  T value_{};
};

template <typename T>
constexpr int32_t KindOf() {
  if (std::is_same_v<T, uint8_t>) return INSPIRE_U8;
  if (std::is_same_v<T, uint16_t>) return INSPIRE_U16;
  if (std::is_same_v<T, uint32_t>) return INSPIRE_U32;
  if (std::is_same_v<T, uint64_t>) return INSPIRE_U64;
  if (std::is_same_v<T, int16_t>) return INSPIRE_I16;
  return INSPIRE_I32;
}

// PirParams<CoeffType> (crypto/pir/pir_params.h:36-105), flattened.
struct PirParams {
  int log_degree = 11;
  int log_modulus = 32;
  int log_modulus1_after_switch = 29;
  int log_modulus2_after_switch = 18;
  int pack_log_digit = 19, pack_num_digits = 2;
  int eval_log_digit = 19, eval_num_digits = 3;
  int num_entries = 0;
  int interpolation_degree = 1;
  int entry_size_multiple = 1;
  uint64_t plaintext_modulus = 65535;
};

// PirRequest / PirResponse (crypto/pir/pir_params.h:196-216).
template <typename CoeffType>
struct PirRequest {
  std::vector<CoeffType> first_dimension_query;
  std::vector<std::vector<CoeffType>> second_dimension_query;  // 2*ne polys
  std::vector<std::vector<CoeffType>> packing_key;             // 2*k polys
};

template <typename CoeffType>
struct RlweCiphertext {
  std::vector<CoeffType> a, b;
};

template <typename CoeffType>
struct PirResponse {
  std::vector<RlweCiphertext<CoeffType>> ciphertexts;  // l of them
};

// The combined server material (PirServer::Create's VerticalConcatenate
// output): DB (l*t*d x db_cols), pack matrix (l*t*d x k*d), and per slice
// a_tilde_agg, t_vec_h (k polys), then second_dim_a (2*ne polys).
template <typename DbDataType, typename CoeffType, typename MatCoeffType>
struct CombinedMaterial {
  std::vector<DbDataType> db;
  int64_t db_rows = 0, db_cols = 0;
  std::vector<MatCoeffType> pack;
  int64_t pack_rows = 0, pack_cols = 0;
  std::vector<std::vector<CoeffType>> a_tilde_agg, t_vec_h, second_dim_a;
};

template <typename DbDataType, typename CoeffType, typename MatCoeffType>
class PirServer {
 public:
  using Material = CombinedMaterial<DbDataType, CoeffType, MatCoeffType>;

  static StatusOr<std::unique_ptr<PirServer>> Create(const PirParams& params,
                                                     const Material& m) {
    inspire_pir_params p = ToC(params);
    std::vector<CoeffType> a = Flatten(m.a_tilde_agg), th = Flatten(m.t_vec_h),
                           sda = Flatten(m.second_dim_a);
    const int64_t d = int64_t{1} << params.log_degree;
    inspire_pir_server* h = nullptr;
    char err[512];
    const int rc = inspire_pir_server_create(
        &p, m.db.data(), m.db_rows, m.db_cols, m.pack.data(), m.pack_rows, m.pack_cols,
        a.data(), static_cast<int64_t>(a.size()) / d, th.data(),
        static_cast<int64_t>(th.size()) / d, sda.data(), static_cast<int64_t>(sda.size()) / d,
        &h, err, sizeof(err));
    if (rc != INSPIRE_OK) return Status(rc, err);
    return std::unique_ptr<PirServer>(new PirServer(params, h));
  }

  static StatusOr<std::unique_ptr<PirServer>> LoadFromBuffer(const PirParams& params,
                                                             const uint8_t* buffer,
                                                             size_t size) {
    inspire_pir_params p = ToC(params);
    inspire_pir_server* h = nullptr;
    char err[512];
    const int rc = inspire_pir_server_load(&p, buffer, size, &h, err, sizeof(err));
    if (rc != INSPIRE_OK) return Status(rc, err);
    return std::unique_ptr<PirServer>(new PirServer(params, h));
  }

  static StatusOr<std::unique_ptr<PirServer>> LoadFromFile(const PirParams& params,
                                                           const std::string& path) {
    inspire_pir_params p = ToC(params);
    inspire_pir_server* h = nullptr;
    char err[512];
    const int rc = inspire_pir_server_load_file(&p, path.c_str(), &h, err, sizeof(err));
    if (rc != INSPIRE_OK) return Status(rc, err);
    return std::unique_ptr<PirServer>(new PirServer(params, h));
  }

  Status SaveToFile(const std::string& path) const {
    char err[512];
    const int rc = inspire_pir_server_save_file(h_, path.c_str(), err, sizeof(err));
    return rc == INSPIRE_OK ? Status() : Status(rc, err);
  }

  StatusOr<PirResponse<CoeffType>> ProcessResponse(const PirRequest<CoeffType>& req) const {
    const int64_t d = int64_t{1} << params_.log_degree;
    std::vector<CoeffType> sd = Flatten(req.second_dimension_query);
    std::vector<CoeffType> pk = Flatten(req.packing_key);
    const int l = params_.entry_size_multiple;
    std::vector<CoeffType> out(static_cast<size_t>(2) * l * d);
    char err[512];
    const int rc = inspire_pir_process_response(
        h_, req.first_dimension_query.data(),
        static_cast<int64_t>(req.first_dimension_query.size()), sd.data(),
        static_cast<int64_t>(req.second_dimension_query.size()), pk.data(),
        static_cast<int64_t>(req.packing_key.size()), out.data(), err, sizeof(err));
    if (rc != INSPIRE_OK) return Status(rc, err);
    PirResponse<CoeffType> resp;
    for (int k = 0; k < l; ++k) {
      RlweCiphertext<CoeffType> ct;
      ct.a.assign(out.begin() + 2 * k * d, out.begin() + (2 * k + 1) * d);
      ct.b.assign(out.begin() + (2 * k + 1) * d, out.begin() + (2 * k + 2) * d);
      resp.ciphertexts.push_back(std::move(ct));
    }
    return resp;
  }

  // Accumulated times in milliseconds (the reference returns absl::Duration).
  double GetDbMultiplyTime() const { return Times()[0]; }
  double GetPackingTime() const { return Times()[1]; }
  double GetPolyEvalTime() const { return Times()[2]; }

  inspire_pir_server* handle() const { return h_; }
  ~PirServer() { inspire_pir_server_destroy(h_); }
  PirServer(const PirServer&) = delete;
  PirServer& operator=(const PirServer&) = delete;

 private:
  PirServer(const PirParams& p, inspire_pir_server* h) : params_(p), h_(h) {}

  static inspire_pir_params ToC(const PirParams& q) {
    inspire_pir_params p{};
    p.coeff_bits = 8 * sizeof(CoeffType);
    p.db_kind = KindOf<DbDataType>();
    p.mat_kind = KindOf<MatCoeffType>();
    p.log_degree = q.log_degree;
    p.log_modulus = q.log_modulus;
    p.log_modulus1_after_switch = q.log_modulus1_after_switch;
    p.log_modulus2_after_switch = q.log_modulus2_after_switch;
    p.pack_log_digit = q.pack_log_digit;
    p.pack_num_digits = q.pack_num_digits;
    p.eval_log_digit = q.eval_log_digit;
    p.eval_num_digits = q.eval_num_digits;
    p.num_entries = q.num_entries;
    p.interpolation_degree = q.interpolation_degree;
    p.entry_size_multiple = q.entry_size_multiple;
    p.plaintext_modulus = q.plaintext_modulus;
    return p;
  }

  static std::vector<CoeffType> Flatten(const std::vector<std::vector<CoeffType>>& polys) {
    std::vector<CoeffType> out;
    for (const auto& p : polys) out.insert(out.end(), p.begin(), p.end());
    return out;
  }

  std::vector<double> Times() const {
    double t[3] = {0, 0, 0};
    inspire_pir_server_timings(h_, &t[0], &t[1], &t[2]);
    return {t[0], t[1], t[2]};
  }

  PirParams params_;
  inspire_pir_server* h_;
};

// GadgetParams (crypto/encryption.h) and PreprocessMatrixPackOutput
// (crypto/lwes_to_rlwe.h:42-47); the matrix is row-major d x (num_digits*d).
struct GadgetParams {
  int log_digit = 19;
  int num_digits = 2;
};

template <typename CoeffType, typename MatCoeffType>
struct PreprocessMatrixPackOutput {
  std::vector<CoeffType> a_tilde_agg;
  std::vector<MatCoeffType> matrix;
  int64_t rows = 0, cols = 0;
  std::vector<std::vector<CoeffType>> t_vec_h;
};

// PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:414-446) of one slice on the
// GPU: a_is are the slice's d LWE a-vectors (d words each), w_vec_g / w_vec_h
// the key-switching a-parts (num_digits polynomials each). The reference's
// RlweParams enters as its log modulus.
template <typename CoeffType, typename MatCoeffType>
StatusOr<PreprocessMatrixPackOutput<CoeffType, MatCoeffType>> PreprocessMatrixPack(
    int log_modulus, const std::vector<std::vector<CoeffType>>& a_is,
    const std::vector<std::vector<CoeffType>>& w_vec_g,
    const std::vector<std::vector<CoeffType>>& w_vec_h, const GadgetParams& gadget) {
  const int d = static_cast<int>(a_is.size());
  const int k = gadget.num_digits;
  std::vector<CoeffType> hint;
  for (const auto& row : a_is) hint.insert(hint.end(), row.begin(), row.end());
  std::vector<CoeffType> pack;
  for (const auto& p : w_vec_g) pack.insert(pack.end(), p.begin(), p.end());
  for (const auto& p : w_vec_h) pack.insert(pack.end(), p.begin(), p.end());
  if (static_cast<int64_t>(hint.size()) != static_cast<int64_t>(d) * d ||
      static_cast<int64_t>(pack.size()) !=
          static_cast<int64_t>(w_vec_g.size() + w_vec_h.size()) * d) {
    return Status(INSPIRE_INVALID_ARGUMENT, "a_is must be d vectors of d words.");
  }
  PreprocessMatrixPackOutput<CoeffType, MatCoeffType> out;
  out.rows = d;
  out.cols = static_cast<int64_t>(k) * d;
  out.a_tilde_agg.resize(d);
  out.matrix.resize(static_cast<size_t>(out.rows * out.cols));
  std::vector<CoeffType> th(static_cast<size_t>(k > 0 ? k : 0) * d);
  char err[512];
  const int rc = inspire_preprocess_matrix_pack(
      8 * sizeof(CoeffType), KindOf<MatCoeffType>(), log_modulus, gadget.log_digit, k, d, 1,
      hint.data(), d, pack.data(), static_cast<int64_t>(w_vec_g.size() + w_vec_h.size()),
      out.a_tilde_agg.data(), out.matrix.data(), th.data(), 0, nullptr, err, sizeof(err));
  if (rc != INSPIRE_OK) return Status(rc, err);
  for (int l = 0; l < k; ++l) {
    out.t_vec_h.emplace_back(th.begin() + static_cast<size_t>(l) * d,
                             th.begin() + static_cast<size_t>(l + 1) * d);
  }
  return out;
}

}  // namespace inspire_gb300

#endif  // INSPIRE_PIR_HPP_
