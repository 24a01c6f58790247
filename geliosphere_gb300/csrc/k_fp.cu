// Instantiation unit of the fp model kernels (compiled in parallel with the
// other models).
#include "kernels.cuh"

namespace gelio {
GELIO_DEFINE_MODEL_ENTRIES(fp, kModelFp)
}  // namespace gelio
