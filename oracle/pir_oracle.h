// CPU oracle for the ReinsPIRe online answer path.
//
// TEST INFRASTRUCTURE ONLY. This library is a plain C++17 restatement of the
// reference server algorithm (google/InsPIRe, crypto/...). It exists so that the
// test-suite, the smoke check and the CPU-baseline leg of the benchmark can
// check the CUDA path against it. Nothing in the product (inspire_gb300/, the
// C-ABI library) links, loads or calls it.
//
// Two negacyclic-product modes are provided:
//   ORC_MODE_EXACT  : the exact integer result that the reference's
//                     InnerProductFft computes whenever its FP64 rounding is
//                     exact (the reference's own tests assert FFT == NTT).
//   ORC_MODE_FP64   : a restatement of the reference FP64 FFT path
//                     (crypto/polynomial_fft.cc:68-197, crypto/fft.h:50-151),
//                     same chunk rules, same radix-2 loop order, std::complex.
//
// Every entry point returns 0 on success, or a non-zero status code with a
// message copied into `err` (mirroring absl::StatusCode numbering:
// 3 = INVALID_ARGUMENT, 9 = FAILED_PRECONDITION, 13 = INTERNAL).
#ifndef INSPIRE_ORACLE_PIR_ORACLE_H_
#define INSPIRE_ORACLE_PIR_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_MODE_EXACT = 0, ORC_MODE_FP64 = 1 };

// Element kinds of a Matrix<T> (crypto/matrix.h:35-156).
enum {
  ORC_U8 = 0,
  ORC_U16 = 1,
  ORC_U32 = 2,
  ORC_U64 = 3,
  ORC_I16 = 4,
  ORC_I32 = 5
};

// Parameters of one PirServer instance (crypto/pir/pir_params.h:36-105,
// crypto/encryption.h:30-98).
typedef struct {
  int32_t coeff_bits;          // 32 or 64: CoeffType
  int32_t log_degree;          // d = 1 << log_degree
  int32_t log_modulus;         // RlweParams::LogModulus()
  int32_t log_modulus1_after_switch;
  int32_t log_modulus2_after_switch;
  int32_t pack_log_digit;
  int32_t pack_num_digits;
  int32_t eval_log_digit;
  int32_t eval_num_digits;
  int32_t num_entries;
  int32_t interpolation_degree;
  int32_t entry_size_multiple;
} orc_params;

// Matrix::Multiply (crypto/matrix.h:167-195): out[r] = sum_c M[r][c]*v[c]
// in CoeffType arithmetic; signed matrix entries are sign-extended.
// `v` and `out` hold coeff_bits-wide words.
int orc_matrix_multiply(int mat_kind, int coeff_bits, const void* mat,
                        int64_t rows, int64_t cols, const void* v, void* out,
                        char* err, size_t err_len);

// CondensedMultiply<uint16_t/int32_t/uint8_t> (crypto/matrix.cc:261-462):
// the u64-lane restatement. `lanes` is the SIMD width in u64 lanes (8 for
// AVX-512); cols must be a multiple of (values-per-word * lanes).
int orc_condensed_multiply(int mat_kind, const void* mat, int64_t rows,
                           int64_t cols, const uint64_t* v, uint64_t* out,
                           int lanes, char* err, size_t err_len);

// Polynomial::InnerProductFft (crypto/polynomial_fft.cc:68-197).
// u and v are n polynomials of length d, stored back to back.
int orc_inner_product(int coeff_bits, int mode, const void* u, const void* v,
                      int n, int d, int u_bits, int v_bits, int chunk_bits,
                      int u_is_signed, void* out, char* err, size_t err_len);

// Polynomial ring helpers (crypto/polynomial.cc:254-456).
int orc_gadget_inv(int coeff_bits, const void* p, int d, int log_modulus,
                   int log_digit, int num_digits, void* out, char* err,
                   size_t err_len);
int orc_signed_gadget_inv(int coeff_bits, const void* p, int d,
                          int log_modulus, int log_digit, int num_digits,
                          void* out, char* err, size_t err_len);
int orc_rescale(int coeff_bits, const void* p, int d, int log_cur, int log_new,
                void* out);
int orc_automorph(int coeff_bits, const void* p, int d, int power, void* out,
                  char* err, size_t err_len);

// FinalizeMatrixPack (crypto/lwes_to_rlwe.cc:448-479): writes the b part of
// the packed ciphertext (the a part is a_tilde_agg unchanged).
int orc_finalize_matrix_pack(const orc_params* prm, int mode, const void* b,
                             const void* b_agg_partial, const void* y_vec_h,
                             const void* t_vec_h, void* out_b, char* err,
                             size_t err_len);

// ExternalProduct (crypto/external_product.cc:35-114). ct = (a, b);
// rgsw holds u[0..nd) then v[0..nd), each an (a, b) pair of polynomials.
int orc_external_product(const orc_params* prm, int mode, const void* ct_a,
                         const void* ct_b, const void* rgsw, void* out_a,
                         void* out_b, char* err, size_t err_len);

// PirServer::ProcessResponse (crypto/pir/server/pir_server.cc:154-306) over
// the combined server material:
//   db            : (l*t*d) x db_cols, row-major, db_kind elements
//   pack          : (l*t*d) x pack_cols, row-major, pack_kind elements
//   a_tilde_agg   : l*t polynomials
//   t_vec_h       : l*t*pack_num_digits polynomials
//   second_dim_a  : 2*eval_num_digits polynomials (unused when t == 1)
//   first_dim     : first_dim_len coefficients
//   second_dim    : second_dim_count polynomials
//   packing_key   : packing_key_count polynomials
//   out           : l ciphertexts, each a then b (2*l*d coefficients)
// `threads` > 1 splits the DB product over threads (CPU baseline only).
int orc_process_response(const orc_params* prm, int mode, int db_kind,
                         const void* db, int64_t db_cols, int pack_kind,
                         const void* pack, int64_t pack_cols,
                         const void* a_tilde_agg, const void* t_vec_h,
                         const void* second_dim_a, const void* first_dim,
                         int64_t first_dim_len, const void* second_dim,
                         int64_t second_dim_count, const void* packing_key,
                         int64_t packing_key_count, void* out, char* err,
                         size_t err_len);

// orc_process_response with the reference's stage timers
// (pir_server.cc:214-285): stage_ms[0] = DB product, [1] = packing (pack
// product + FinalizeMatrixPack), [2] = EvalPoly, in milliseconds. `threads`
// splits the two products over host threads (1 = the single-threaded
// reference); condensed_db != 0 runs a u8 / u16 DB with a u64 CoeffType
// through the condensed-word product the reference uses for that case
// (matrix.cc:261-318, 376-462). Used by the CPU baseline.
int orc_process_response_staged(
    const orc_params* prm, int mode, int db_kind, const void* db,
    int64_t db_cols, int pack_kind, const void* pack, int64_t pack_cols,
    const void* a_tilde_agg, const void* t_vec_h, const void* second_dim_a,
    const void* first_dim, int64_t first_dim_len, const void* second_dim,
    int64_t second_dim_count, const void* packing_key,
    int64_t packing_key_count, void* out, int threads, int condensed_db,
    double* stage_ms, char* err, size_t err_len);

// Interpolate (crypto/db_row_interpolation.cc:115-228) for one group of t
// records of d values each, values of width value_bits (8, 16 or 32).
int orc_interpolate(int value_bits, const void* db_row, int d, int t,
                    uint32_t plaintext_modulus, void* out, char* err,
                    size_t err_len);

// PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:163-446) for one slice:
//   a_is     : d LWE a-vectors of d words (row i = a_i)
//   w_vec_g  : num_digits polynomials (key-switching a-parts for X -> X^5)
//   w_vec_h  : num_digits polynomials (for X -> X^{2d-1})
// Writes a_tilde_agg (d words), t_vec_h (num_digits polynomials), and when
// not null the d x (num_digits*d) matrix as centred signed 64-bit entries and
// the (d/2-1) x num_digits x d digit polynomials t_vec_g / t_vec_gh.
int orc_preprocess_matrix_pack(int coeff_bits, int mode, int log_modulus,
                               int log_digit, int num_digits, int d,
                               const void* a_is, const void* w_vec_g,
                               const void* w_vec_h, void* a_tilde_agg,
                               int64_t* matrix, void* t_vec_h, void* t_vec_g,
                               void* t_vec_gh, char* err, size_t err_len);

// Pack (crypto/lwes_to_rlwe.cc:356-412): b_agg of the packed ciphertext from
// the LWE b-values and the key-switching b-parts, by automorphisms.
int orc_pack(int coeff_bits, int mode, int log_modulus, int log_digit,
             int num_digits, int d, const void* b, const void* y_vec_g,
             const void* y_vec_h, const void* t_vec_g, const void* t_vec_gh,
             const void* t_vec_h, void* b_agg, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif  // INSPIRE_ORACLE_PIR_ORACLE_H_
