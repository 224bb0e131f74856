// pp_mixed_v2.cu -- PP_MIXED tile shape 2: 4 warps x 64 nodes per CTA, register
// budget for 6 resident CTAs per SM (kernel template in pp_mixed.cuh).
#include "pp_mixed.cuh"

namespace pp {
namespace mixed {

int launch_mixed_shape2(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    return launch_shape<4, 6>(a, parity, l, st);
}

}  // namespace mixed
}  // namespace pp
