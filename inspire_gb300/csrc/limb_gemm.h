// Batched DB/pack product on the tensor cores with exact 8-bit limbs.
// Declared here, implemented in limb_gemm.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

namespace inspire {

// Per-batch state of the tensor engine (the request byte planes and their
// TMA descriptors). One per in-flight batch.
class LimbScratch {
 public:
  virtual ~LimbScratch() = default;
};

class LimbGemm {
 public:
  // Prepares the limb planes of the server matrices. Leaves *out empty when
  // the parameters are outside what the tensor-core engine supports.
  static void Create(int coeff_bits, int db_kind, const void* db, int64_t rows,
                     int64_t db_cols, int mat_kind, const void* pack,
                     int64_t pack_cols, std::unique_ptr<LimbGemm>* out);
  virtual ~LimbGemm() = default;
  virtual std::unique_ptr<LimbScratch> NewScratch() = 0;
  // Device bytes the scratch for `batch` requests holds.
  virtual int64_t ScratchBytes(int batch) const = 0;
  // Allocates the scratch for up to `batch` requests now (Run allocates on
  // first use otherwise).
  virtual cudaError_t Reserve(LimbScratch* scratch, int batch) = 0;
  // out[q][r] = db[r] . q1[q] + pack[r] . yg[q]  (mod 2^w), q < batch.
  virtual cudaError_t Run(int batch, const void* q1, int64_t q1_stride,
                          const void* yg, int64_t yg_stride, void* out,
                          LimbScratch* scratch, cudaStream_t stream) = 0;
  // Autotuner: times the split-K factors for this batch size on these
  // operands, keeps the fastest for later Runs of the same padded batch
  // size and reports it. Synchronises the stream.
  virtual cudaError_t Tune(int batch, const void* q1, int64_t q1_stride,
                           const void* yg, int64_t yg_stride, void* out,
                           LimbScratch* scratch, cudaStream_t stream,
                           int* chosen, float* best_ms) = 0;
  // Returns (and clears) the kernel's error flag: non-zero when a pipeline
  // wait timed out in a previous launch. Synchronous.
  virtual int CheckError() = 0;
};

}  // namespace inspire
