// Fused time-step kernels with BF16 wavefield storage (per-level
// power-of-two scales, FP32 arithmetic): source, forward and adjoint modes,
// single-shot and batched launches.
#include "born_step_impl.cuh"

namespace born {

BORN_DEFINE_STORAGE_ENTRY(kStoreBF16, bf16)

}  // namespace born
