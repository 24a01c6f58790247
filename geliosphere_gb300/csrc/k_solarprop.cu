// Instantiation unit of the solarprop model kernels (compiled in parallel with the
// other models).
#include "kernels.cuh"

namespace gelio {
GELIO_DEFINE_MODEL_ENTRIES(solarprop, kModelSolarProp)
}  // namespace gelio
