// pp_mixed_v0.cu -- PP_MIXED tile shape 0: 4 warps x 64 nodes per CTA, register
// budget for 8 resident CTAs per SM (kernel template in pp_mixed.cuh).
#include "pp_mixed.cuh"

namespace pp {
namespace mixed {

int launch_mixed_shape0(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    return launch_shape<4, 8>(a, parity, l, st);
}

}  // namespace mixed
}  // namespace pp
