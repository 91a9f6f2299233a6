// Fused time-step kernels with FP32 levels and fused multiply-add
// arithmetic (not bit-identical to the reference order): source, forward and
// adjoint modes, single-shot and batched launches.
#include "born_step_impl.cuh"

namespace born {

BORN_DEFINE_STORAGE_ENTRY(kStoreF32Fused, f32fused)

}  // namespace born
