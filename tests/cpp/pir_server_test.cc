// C++ test of the PirServer mirror (include/inspire_pir.hpp) over the C ABI,
// structured like the reference's crypto/pir/server/pir_server_test.cc:
// responses against the CPU oracle (test infrastructure, linked only here),
// the request validation messages, and SaveToFile / LoadFromFile giving a
// server that answers identically. Exit status 0 when every check passes.
#include <cstdint>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "inspire_pir.hpp"
#include "pir_oracle.h"

namespace {

int failures = 0;

#define CHECK(cond, what)                                   \
  do {                                                      \
    if (!(cond)) {                                          \
      std::fprintf(stderr, "FAILED: %s (%s:%d)\n", what,    \
                   __FILE__, __LINE__);                     \
      ++failures;                                           \
    }                                                       \
  } while (0)

using Server = inspire_gb300::PirServer<uint16_t, uint32_t, int32_t>;

struct Case {
  int log_d, t, l, n;
};

void RunCase(const Case& c, const std::string& dir) {
  const int d = 1 << c.log_d, k = 2, ne = 3;
  inspire_gb300::PirParams params;
  params.log_degree = c.log_d;
  params.log_modulus = 32;
  params.log_modulus1_after_switch = 16 + c.log_d + 2 < 32 ? 16 + c.log_d + 2 : 32;
  params.log_modulus2_after_switch = 18;
  params.num_entries = c.n;
  params.interpolation_degree = c.t;
  params.entry_size_multiple = c.l;
  const int64_t rows = static_cast<int64_t>(c.l) * c.t * d, cols = c.n / c.t;
  std::mt19937_64 rng(12345 + c.log_d);
  Server::Material m;
  m.db_rows = rows;
  m.db_cols = cols;
  m.db.resize(rows * cols);
  for (auto& x : m.db) x = static_cast<uint16_t>(rng() % 65535);
  m.pack_rows = rows;
  m.pack_cols = static_cast<int64_t>(k) * d;
  m.pack.resize(rows * k * d);
  for (auto& x : m.pack) x = static_cast<int32_t>(rng() % (1 << 24)) - (1 << 23);
  auto poly = [&](bool digit) {
    std::vector<uint32_t> p(d);
    for (auto& x : p) {
      x = digit ? static_cast<uint32_t>(static_cast<int32_t>(rng() % (1 << 19)) - (1 << 18))
                : static_cast<uint32_t>(rng());
    }
    return p;
  };
  for (int s = 0; s < c.l * c.t; ++s) {
    m.a_tilde_agg.push_back(poly(false));
    for (int j = 0; j < k; ++j) m.t_vec_h.push_back(poly(true));
  }
  if (c.t > 1) {
    for (int j = 0; j < 2 * ne; ++j) m.second_dim_a.push_back(poly(false));
  }
  auto server = Server::Create(params, m);
  CHECK(server.ok(), "Create");
  if (!server.ok()) return;

  inspire_gb300::PirRequest<uint32_t> req;
  req.first_dimension_query.resize(cols);
  for (auto& x : req.first_dimension_query) x = static_cast<uint32_t>(rng());
  if (c.t > 1) {
    for (int j = 0; j < 2 * ne; ++j) req.second_dimension_query.push_back(poly(false));
  }
  for (int j = 0; j < 2 * k; ++j) req.packing_key.push_back(poly(false));
  auto resp = (*server)->ProcessResponse(req);
  CHECK(resp.ok(), "ProcessResponse");
  if (!resp.ok()) return;

  // The oracle on the same bytes.
  orc_params op{32, c.log_d, 32, params.log_modulus1_after_switch,
                params.log_modulus2_after_switch, 19, k, 19, ne, c.n, c.t, c.l};
  std::vector<uint32_t> a, th, sda, sd, pk;
  for (auto& p : m.a_tilde_agg) a.insert(a.end(), p.begin(), p.end());
  for (auto& p : m.t_vec_h) th.insert(th.end(), p.begin(), p.end());
  for (auto& p : m.second_dim_a) sda.insert(sda.end(), p.begin(), p.end());
  for (auto& p : req.second_dimension_query) sd.insert(sd.end(), p.begin(), p.end());
  for (auto& p : req.packing_key) pk.insert(pk.end(), p.begin(), p.end());
  std::vector<uint32_t> want(static_cast<size_t>(2) * c.l * d);
  char err[512];
  const int rc = orc_process_response(
      &op, ORC_MODE_EXACT, ORC_U16, m.db.data(), cols, ORC_I32, m.pack.data(), k * d,
      a.data(), th.data(), sda.data(), req.first_dimension_query.data(), cols, sd.data(),
      static_cast<int64_t>(req.second_dimension_query.size()), pk.data(),
      static_cast<int64_t>(req.packing_key.size()), want.data(), err, sizeof(err));
  CHECK(rc == 0, "oracle");
  bool same = resp->ciphertexts.size() == static_cast<size_t>(c.l);
  for (int s = 0; same && s < c.l; ++s) {
    for (int j = 0; j < d; ++j) {
      same = same && resp->ciphertexts[s].a[j] == want[(2 * s) * d + j] &&
             resp->ciphertexts[s].b[j] == want[(2 * s + 1) * d + j];
    }
  }
  CHECK(same, "response equals the oracle's");

  // Request validation (pir_server.cc:160-205).
  auto bad = req;
  bad.packing_key.pop_back();
  auto r1 = (*server)->ProcessResponse(bad);
  CHECK(!r1.ok() && r1.status().code() == INSPIRE_INVALID_ARGUMENT &&
            r1.status().message() == "Packing key must contain 2 * num_digits polynomials.",
        "packing key validation");
  bad = req;
  bad.first_dimension_query.resize(cols + 1);
  auto r2 = (*server)->ProcessResponse(bad);
  CHECK(!r2.ok() && r2.status().message().find("First dimension query size") == 0,
        "first dimension validation");

  // SaveToFile / LoadFromFile (pir_server_test.cc:527-679).
  const std::string path = dir + "/server_" + std::to_string(c.log_d) + ".img";
  CHECK((*server)->SaveToFile(path).ok(), "SaveToFile");
  auto loaded = Server::LoadFromFile(params, path);
  CHECK(loaded.ok(), "LoadFromFile");
  if (loaded.ok()) {
    auto resp2 = (*loaded)->ProcessResponse(req);
    CHECK(resp2.ok(), "ProcessResponse after load");
    bool same2 = resp2.ok();
    for (int s = 0; same2 && s < c.l; ++s) {
      same2 = resp2->ciphertexts[s].a == resp->ciphertexts[s].a &&
              resp2->ciphertexts[s].b == resp->ciphertexts[s].b;
    }
    CHECK(same2, "loaded server answers identically");
  }
  auto missing = Server::LoadFromFile(params, dir + "/missing.img");
  CHECK(!missing.ok() && missing.status().message() == "Failed to read file.",
        "missing file");
  CHECK((*server)->GetDbMultiplyTime() > 0, "timers");
}

}  // namespace

// PreprocessMatrixPack through the C++ mirror against the oracle's
// restatement (d = 64, the reference test's degree; int32 matrix entries).
void PreprocessCase(int log_q, int log_digit, int k) {
  const int d = 64;
  std::mt19937_64 g(1000 + log_q);
  const uint32_t mask = log_q >= 32 ? 0xFFFFFFFFu : ((1u << log_q) - 1);
  std::vector<std::vector<uint32_t>> a_is(d, std::vector<uint32_t>(d));
  for (auto& row : a_is)
    for (auto& x : row) x = static_cast<uint32_t>(g()) & mask;
  std::vector<std::vector<uint32_t>> wg(k, std::vector<uint32_t>(d)), wh = wg;
  for (auto* v : {&wg, &wh})
    for (auto& p : *v)
      for (auto& x : p) x = static_cast<uint32_t>(g()) & mask;
  auto got = inspire_gb300::PreprocessMatrixPack<uint32_t, int32_t>(
      log_q, a_is, wg, wh, inspire_gb300::GadgetParams{log_digit, k});
  CHECK(got.ok(), "PreprocessMatrixPack");
  if (!got.ok()) return;
  std::vector<uint32_t> flat_a, flat_g, flat_h;
  for (auto& r : a_is) flat_a.insert(flat_a.end(), r.begin(), r.end());
  for (auto& p : wg) flat_g.insert(flat_g.end(), p.begin(), p.end());
  for (auto& p : wh) flat_h.insert(flat_h.end(), p.begin(), p.end());
  std::vector<uint32_t> a(d), th(static_cast<size_t>(k) * d);
  std::vector<int64_t> mat(static_cast<size_t>(d) * k * d);
  char err[512];
  const int rc = orc_preprocess_matrix_pack(32, ORC_MODE_EXACT, log_q, log_digit, k, d,
                                            flat_a.data(), flat_g.data(), flat_h.data(),
                                            a.data(), mat.data(), th.data(), nullptr,
                                            nullptr, err, sizeof(err));
  CHECK(rc == 0, "oracle PreprocessMatrixPack");
  CHECK(got->a_tilde_agg == a, "a_tilde_agg");
  bool th_ok = true;
  for (int l = 0; l < k; ++l)
    for (int j = 0; j < d; ++j) th_ok &= got->t_vec_h[l][j] == th[static_cast<size_t>(l) * d + j];
  CHECK(th_ok, "t_vec_h");
  bool m_ok = true;
  for (size_t i = 0; i < mat.size(); ++i) m_ok &= got->matrix[i] == static_cast<int32_t>(mat[i]);
  CHECK(m_ok, "matrix");
}

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  RunCase({8, 4, 1, 4 * 512}, dir);    // d = 256, t = 4
  RunCase({11, 2, 2, 2 * 1024}, dir);  // d = 2048, t = 2, l = 2
  RunCase({7, 1, 1, 256}, dir);        // t = 1: no EvalPoly
  PreprocessCase(32, 19, 2);
  PreprocessCase(27, 4, 5);
  if (failures == 0) std::printf("pir_server_test: all checks passed\n");
  return failures == 0 ? 0 : 1;
}
