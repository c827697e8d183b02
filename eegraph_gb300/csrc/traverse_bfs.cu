// traverse_bfs.cu -- instantiation of the persistent push kernels for BFS (templates in traverse.cuh).
#include "traverse.cuh"

namespace eeg {
namespace trav {

eeg_status launch_bfs(const TravArgs& args, bool td, uint32_t K, int device, uint32_t bps, cudaStream_t st) {
    return td ? launch_k<OP_BFS, true>(args, K, device, bps, st) : launch_k<OP_BFS, false>(args, K, device, bps, st);
}

}  // namespace trav
}  // namespace eeg
