// pp_tiled_v0.cu -- tiled PP_MIXED tile shape 0: 8 warps, register budget for 4 resident CTAs per SM
// (kernel template in pp_tiled.cuh).
#include "pp_tiled.cuh"

namespace pp {
namespace tiled {

int launch_tiled_shape0(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st) {
    return launch_tiled_shape<8, 4>(a, t, parity, l, st);
}

}  // namespace tiled
}  // namespace pp
