// pp_tiled_v2.cu -- tiled PP_MIXED tile shape 2: 16 warps, register budget for 2 resident CTAs per SM
// (kernel template in pp_tiled.cuh).
#include "pp_tiled.cuh"

namespace pp {
namespace tiled {

int launch_tiled_shape2(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st) {
    return launch_tiled_shape<16, 2>(a, t, parity, l, st);
}

}  // namespace tiled
}  // namespace pp
