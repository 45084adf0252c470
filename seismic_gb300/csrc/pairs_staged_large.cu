// Staged pair form, the launches for P = 2048 and 4096 (a translation unit of
// its own so that the kernel's instances compile in parallel with
// pairs_staged.cu's).
#include "staged_core.cuh"

namespace seismic {

cudaError_t launch_pairs_staged_large(int P, const PairArgs &a, int sm_count, cudaStream_t s) {
  switch (P) {
    case 2048: return launch_staged_p<2048>(a, sm_count, s);
    case 4096: return launch_staged_p<4096>(a, sm_count, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace seismic
