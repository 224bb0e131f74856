// pp_mixed_v2.cu -- PP_MIXED tile shape 2: 8 warps x 128 nodes per CTA, register
// budget for 3 resident CTAs per SM (for the bond-type and compensated
// instances, which need more registers; kernel template in pp_mixed.cuh).
#include "pp_mixed.cuh"

namespace pp {
namespace mixed {

int launch_mixed_shape2(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    return launch_shape<8, 3>(a, parity, l, st);
}

}  // namespace mixed
}  // namespace pp
