// pp_tiled_v1.cu -- tiled PP_MIXED tile shape 1: 4 warps, register budget for 8 resident CTAs per SM
// (kernel template in pp_tiled.cuh).
#include "pp_tiled.cuh"

namespace pp {
namespace tiled {

int launch_tiled_shape1(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st) {
    return launch_tiled_shape<4, 8>(a, t, parity, l, st);
}

}  // namespace tiled
}  // namespace pp
