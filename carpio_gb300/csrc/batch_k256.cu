// k_batch<256>: the batched solver's kernel for 256-thread CTAs, compiled in
// its own translation unit so the block sizes build in parallel.
#include "batch_dev.cuh"

namespace cg_batch {
const void* kernel_256() { return (const void*)k_batch<256>; }
}  // namespace cg_batch
