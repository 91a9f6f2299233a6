// Born forward step with FP32 levels in the reference's operation order and
// the Born coupling formed exactly as the reference's double expression
// (born_couple.h); the other steps of this storage are the FP32 kernels.
#include "born_step_impl.cuh"

namespace born {

BORN_DEFINE_STORAGE_ENTRY(kStoreF32Exact, f32exact)

}  // namespace born
