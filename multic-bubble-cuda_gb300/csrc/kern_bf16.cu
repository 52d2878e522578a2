// Update kernels instantiated for bfloat16 deviation form population storage.
#include "kernels.cuh"

namespace mcb {
MCB_STORAGE_LAUNCHERS(StB16, bf16)
}  // namespace mcb
