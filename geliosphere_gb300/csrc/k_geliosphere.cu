// Instantiation unit of the geliosphere model kernels (compiled in parallel with the
// other models).
#include "kernels.cuh"

namespace gelio {
GELIO_DEFINE_MODEL_ENTRIES(geliosphere, kModelGeliosphere)
}  // namespace gelio
