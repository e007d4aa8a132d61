#include "limb_gemm.h"

namespace inspire {

void LimbGemm::Create(int, int, const void*, int64_t, int64_t, int, const void*,
                      int64_t, std::unique_ptr<LimbGemm>* out) {
  out->reset();
}

}  // namespace inspire
