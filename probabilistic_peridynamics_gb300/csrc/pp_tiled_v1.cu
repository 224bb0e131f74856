// pp_tiled_v1.cu -- tiled PP_MIXED tile shape 1: 8 warps, register budget for 3 resident CTAs per SM (bond types, compensated sums)
// (kernel template in pp_tiled.cuh).
#include "pp_tiled.cuh"

namespace pp {
namespace tiled {

int launch_tiled_shape1(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st) {
    return launch_tiled_shape<8, 3>(a, t, parity, l, st);
}

}  // namespace tiled
}  // namespace pp
