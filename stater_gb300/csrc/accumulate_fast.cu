// FP32 form of the stage-1 accumulation (FMA contraction on, reciprocal of n
// shared by all moments of a sample).
#include "acc_kernels.cuh"

namespace stater {

cudaError_t launch_acc_fast_f32(const AccParams &P, int max_moment, cudaStream_t s) {
    return launch_acc<float, true>(P, max_moment, s);
}

}  // namespace stater
