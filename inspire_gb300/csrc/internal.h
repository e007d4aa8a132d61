// Internal launch interfaces shared by the translation units of the library.
// Nothing here is part of the public C ABI (include/inspire_pir.h).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace inspire {

// Element kinds, numbered as in the public header.
enum ElemKind : int {
  kU8 = 0,
  kU16 = 1,
  kU32 = 2,
  kU64 = 3,
  kI16 = 4,
  kI32 = 5,
};

int elem_size(int kind);

// out[q][r] = sum_c db[r][c] * q1[q][c] + sum_j pk[r][j] * yg[q][j]  (mod 2^w)
// for q < nq, r < rows. Either matrix may be absent (nullptr, 0 columns).
// Returns a cudaError_t from the launch.
cudaError_t launch_fused_gemv(int coeff_bits, int db_kind, const void* db,
                              int64_t db_cols, const void* q1,
                              int64_t q1_stride, int pk_kind, const void* pk,
                              int64_t pk_cols, const void* yg,
                              int64_t yg_stride, void* out, int64_t out_stride,
                              int64_t rows, int nq, cudaStream_t stream);

}  // namespace inspire
