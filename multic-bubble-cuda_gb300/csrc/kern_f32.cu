// Update kernels instantiated for float32 f and Q2.30 g population storage.
#include "kernels.cuh"

namespace mcb {
MCB_STORAGE_LAUNCHERS(StF32, f32)
}  // namespace mcb
