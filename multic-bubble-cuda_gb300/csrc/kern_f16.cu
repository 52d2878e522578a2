// Update kernels instantiated for float16 deviation form population storage.
#include "kernels.cuh"

namespace mcb {
MCB_STORAGE_LAUNCHERS(StH16, f16)
}  // namespace mcb
