// k_batch<512>: the batched solver's kernel for 512-thread CTAs, compiled in
// its own translation unit so the block sizes build in parallel.
#include "batch_dev.cuh"

namespace cg_batch {
const void* kernel_512() { return (const void*)k_batch<512>; }
}  // namespace cg_batch
