// pp_fused.cuh -- declarations shared by the fused-step translation units.
#pragma once

#include "pp_common.cuh"

namespace pp {

// Boundary-condition magnitudes of one launch: by value, or read on the
// device from dmags/fmags at index k_off (+ *base in graph replays).
struct Launch {
    double disp, force;
    const double* dmags;
    const double* fmags;
    const int64_t* base;
    int64_t k_off;
};

struct StepMags {
    double disp;
    double force;
};

__device__ __forceinline__ StepMags step_mags(const Launch& l) {
    if (l.dmags == nullptr) return StepMags{l.disp, l.force};
    const int64_t idx = (l.base ? *l.base : 0) + l.k_off;
    return StepMags{l.dmags[idx], l.fmags[idx]};
}

// Launches one PP_MIXED step (pp_mixed.cu); returns a PP_* status.
int launch_mixed_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st);

// Checks of the PP_MIXED arguments beyond the common ones (pp_mixed.cu).
int validate_mixed(const pp_fused_args& a);

// All argument checks of a fused step (pp_fused.cu).
int validate_fused(const pp_fused_args& a);

// Launches one fused step of either precision (pp_fused.cu).
int launch_fused_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st);

}  // namespace pp
