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

// Forms of the product kernel: the DB as resident fp16 digit planes, or
// the DB read as stored (u16) and split into digits in shared memory.
constexpr int kFormPlanes = 0;
constexpr int kFormRaw = 1;
// Or-ed into a form: the narrow (16-request) request tile.
constexpr int kFormNarrow = 2;

class LimbGemm {
 public:
  // Prepares the limb planes of the server matrices (the pack matrix's
  // always; the DB's only with db_planes, else the DB is read as stored:
  // `db` must stay valid while the engine lives). Leaves *out empty when
  // the parameters are outside what the tensor-core engine supports.
  static void Create(int coeff_bits, int db_kind, const void* db, int64_t rows,
                     int64_t db_cols, int mat_kind, const void* pack,
                     int64_t pack_cols, bool db_planes, std::unique_ptr<LimbGemm>* out);
  virtual ~LimbGemm() = default;
  virtual std::unique_ptr<LimbScratch> NewScratch() = 0;
  // Device bytes the scratch for `batch` requests holds.
  virtual int64_t ScratchBytes(int batch) const = 0;
  // Allocates the scratch for up to `batch` requests now (Run allocates on
  // first use otherwise).
  virtual cudaError_t Reserve(LimbScratch* scratch, int batch) = 0;
  // out[q][r] = db[r] . q1[q] + pack[r] . yg[q]  (mod 2^w), q < batch.
  // out_bits: the low bits of each word the caller reads (0: all w); the
  // words are exact mod 2^out_bits at least, and a Z_2^64 product read mod
  // 2^56 or less skips its top digit position.
  virtual cudaError_t Run(int batch, const void* q1, int64_t q1_stride,
                          const void* yg, int64_t yg_stride, void* out,
                          LimbScratch* scratch, cudaStream_t stream, int out_bits) = 0;
  // Run with a given form (kFormPlanes or kFormRaw, | kFormNarrow for the
  // 16-request tile) and split-K factor (split <= 0: the tuned or heuristic
  // one); cudaErrorNotSupported when the form is unavailable.
  virtual cudaError_t RunForm(int batch, const void* q1, int64_t q1_stride,
                              const void* yg, int64_t yg_stride, void* out,
                              LimbScratch* scratch, cudaStream_t stream, int form,
                              int split, int out_bits) = 0;
  // Autotuner: times the split-K factors of every available form for this
  // batch size on these operands, keeps the fastest (factor, form) for
  // later Runs of the same padded batch size and reports it. Synchronises
  // the stream.
  virtual cudaError_t Tune(int batch, const void* q1, int64_t q1_stride,
                           const void* yg, int64_t yg_stride, void* out,
                           LimbScratch* scratch, cudaStream_t stream, int out_bits,
                           int* chosen, int* chosen_form, float* best_ms) = 0;
  // Device bytes the engine keeps resident (digit planes).
  virtual int64_t ResidentBytes() const = 0;
  // Returns (and clears) the kernel's error flag: non-zero when a pipeline
  // wait timed out in a previous launch. Synchronous.
  virtual int CheckError() = 0;
};

}  // namespace inspire
