// Instantiation unit of the bp model kernels (compiled in parallel with the
// other models).
#include "kernels.cuh"

namespace gelio {
GELIO_DEFINE_MODEL_ENTRIES(bp, kModelBp)
}  // namespace gelio
