// pp_plain.cu -- reference-structured binary64 kernels ("plain" step).
//
// Separate launches for bond force, displacement update and damage, as
// PeriPy's OpenCL integrators issue them (peripy/integrators.py:256-283,
// 530-541, 635-648, 751-764).  One warp owns one node; its lanes stride the
// node's neighbour slots and the slot forces are summed in the work-group
// tree order (pp_common.cuh), so results are bit-identical to the reference
// arithmetic.  These kernels are bound by the FP64 pipe on GB300.
#include "pp_bond_f64.cuh"

namespace pp {
namespace {

constexpr int kWarpsPerBlock = 8;

template <int SL, bool CORR, bool TYPES>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_bond_force(pp_bond_force_args a) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (i >= a.nnodes) return;  // warp-uniform
    const F64Bond b{a.r0,
                    a.u,
                    a.vols,
                    a.nlist,
                    a.stiffness_corrections,
                    a.bond_types,
                    a.regimes,
                    a.bond_stiffness_table,
                    a.critical_stretch_table,
                    a.plus_cs,
                    nullptr,  // the plain step recomputes |xi| as the reference does
                    a.bond_stiffness,
                    a.critical_stretch,
                    a.nregimes};
    const d3 ri{a.r0[3 * (int64_t)i], a.r0[3 * (int64_t)i + 1], a.r0[3 * (int64_t)i + 2]};
    const d3 ui{a.u[3 * (int64_t)i], a.u[3 * (int64_t)i + 1], a.u[3 * (int64_t)i + 2]};
    const int64_t row = (int64_t)i * a.max_neigh;
    int intact = 0;
    const d3 f = tree_reduce_f64<SL>(lane, a.max_neigh, [&](int k) {
        return f64_slot<CORR, TYPES>(b, row + k, ri, ui, intact);
    });
    if (lane == 0) {
        const int64_t o = 3 * (int64_t)i;
        a.body_force[o] = f.x;
        a.body_force[o + 1] = f.y;
        a.body_force[o + 2] = f.z;
        a.force[o] = force_with_bc(f.x, a.fc_types[o], a.fc_values[o], a.fc_scale);
        a.force[o + 1] = force_with_bc(f.y, a.fc_types[o + 1], a.fc_values[o + 1], a.fc_scale);
        a.force[o + 2] = force_with_bc(f.z, a.fc_types[o + 2], a.fc_values[o + 2], a.fc_scale);
    }
}

template <int SL>
int launch_bond_force(const pp_bond_force_args& a, cudaStream_t st) {
    const dim3 grid((a.nnodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
    const dim3 block(kWarpsPerBlock * 32);
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    if (!corr && !types) k_bond_force<SL, false, false><<<grid, block, 0, st>>>(a);
    if (corr && !types) k_bond_force<SL, true, false><<<grid, block, 0, st>>>(a);
    if (!corr && types) k_bond_force<SL, false, true><<<grid, block, 0, st>>>(a);
    if (corr && types) k_bond_force<SL, true, true><<<grid, block, 0, st>>>(a);
    return launch_status();
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_damage(const int32_t* __restrict__ nlist, const int32_t* __restrict__ family,
             int32_t* __restrict__ n_neigh, double* __restrict__ damage, int nnodes,
             int max_neigh) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (i >= nnodes) return;
    const int64_t row = (int64_t)i * max_neigh;
    int count = 0;
    for (int k0 = 0; k0 < max_neigh; k0 += 32) {
        const int k = k0 + lane;
        const bool intact = k < max_neigh && nlist[row + k] != -1;
        count += __popc(__ballot_sync(kFull, intact));
    }
    if (lane == 0) {
        n_neigh[i] = count;
        damage[i] = damage_of(count, family[i]);
    }
}

__global__ void k_update_euler(const double* __restrict__ force, double* __restrict__ u,
                               const int32_t* __restrict__ bc_types,
                               const double* __restrict__ bc_values, double bc_scale,
                               double dt, int64_t ndof) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ndof) return;
    u[i] = euler_u(u[i], force[i], bc_types[i], bc_values[i], bc_scale, dt);
}

template <int KIND>
__global__ void k_update_dynamic(const double* __restrict__ force, double* __restrict__ u,
                                 double* __restrict__ ud, double* __restrict__ udd,
                                 const int32_t* __restrict__ bc_types,
                                 const double* __restrict__ bc_values,
                                 const double* __restrict__ densities, double bc_scale,
                                 double damping, double dt, int64_t ndof) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ndof) return;
    double v = ud[i];
    double a = udd[i];
    double x;
    if constexpr (KIND == PP_EULER_CROMER)
        x = euler_cromer_u(u[i], v, a, force[i], bc_types[i], bc_values[i], densities[i],
                           bc_scale, damping, dt);
    else
        x = velocity_verlet_u(u[i], v, a, force[i], bc_types[i], bc_values[i], densities[i],
                              bc_scale, damping, dt);
    ud[i] = v;
    udd[i] = a;
    u[i] = x;
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_bond_force(const pp_bond_force_args* args, void* stream) {
    if (!args) return PP_ERROR_INVALID_VALUE;
    const pp_bond_force_args& a = *args;
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(a.max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.u || !a.force || !a.body_force || !a.r0 || !a.vols || !a.nlist || !a.fc_types ||
        !a.fc_values)
        return PP_ERROR_INVALID_VALUE;
    if (a.bond_types && (!a.regimes || !a.plus_cs || !a.bond_stiffness_table ||
                         !a.critical_stretch_table || a.nregimes < 1 || a.nbond_types < 1))
        return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (a.max_neigh > 32 ? a.max_neigh / 32 : 1) {
        case 1: return launch_bond_force<1>(a, st);
        case 2: return launch_bond_force<2>(a, st);
        case 4: return launch_bond_force<4>(a, st);
        case 8: return launch_bond_force<8>(a, st);
        case 16: return launch_bond_force<16>(a, st);
        case 32: return launch_bond_force<32>(a, st);
    }
    return PP_ERROR_MAX_NEIGH;
}

extern "C" int pp_damage(const int32_t* nlist, const int32_t* family, int32_t* n_neigh,
                         double* damage, int32_t nnodes, int32_t max_neigh, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!nlist || !family || !n_neigh || !damage) return PP_ERROR_INVALID_VALUE;
    const dim3 grid((nnodes + kWarpsPerBlock - 1) / kWarpsPerBlock);
    k_damage<<<grid, kWarpsPerBlock * 32, 0, static_cast<cudaStream_t>(stream)>>>(
        nlist, family, n_neigh, damage, nnodes, max_neigh);
    return launch_status();
}

extern "C" int pp_update_displacement_euler(const double* force, double* u,
                                            const int32_t* bc_types, const double* bc_values,
                                            double bc_scale, double dt, int64_t ndof,
                                            void* stream) {
    if (ndof < 0) return PP_ERROR_INVALID_VALUE;
    if (ndof == 0) return PP_SUCCESS;
    if (!force || !u || !bc_types || !bc_values) return PP_ERROR_INVALID_VALUE;
    const int64_t grid = (ndof + 255) / 256;
    k_update_euler<<<(unsigned)grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        force, u, bc_types, bc_values, bc_scale, dt, ndof);
    return launch_status();
}

template <int KIND>
static int update_dynamic(const double* force, double* u, double* ud, double* udd,
                          const int32_t* bc_types, const double* bc_values,
                          const double* densities, double bc_scale, double damping, double dt,
                          int64_t ndof, void* stream) {
    if (ndof < 0) return PP_ERROR_INVALID_VALUE;
    if (ndof == 0) return PP_SUCCESS;
    if (!force || !u || !ud || !udd || !bc_types || !bc_values || !densities)
        return PP_ERROR_INVALID_VALUE;
    const int64_t grid = (ndof + 255) / 256;
    k_update_dynamic<KIND><<<(unsigned)grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        force, u, ud, udd, bc_types, bc_values, densities, bc_scale, damping, dt, ndof);
    return launch_status();
}

extern "C" int pp_update_displacement_euler_cromer(const double* force, double* u, double* ud,
                                                   double* udd, const int32_t* bc_types,
                                                   const double* bc_values,
                                                   const double* densities, double bc_scale,
                                                   double damping, double dt, int64_t ndof,
                                                   void* stream) {
    return update_dynamic<PP_EULER_CROMER>(force, u, ud, udd, bc_types, bc_values, densities,
                                           bc_scale, damping, dt, ndof, stream);
}

extern "C" int pp_update_displacement_velocity_verlet(
    const double* force, double* u, double* ud, double* udd, const int32_t* bc_types,
    const double* bc_values, const double* densities, double bc_scale, double damping,
    double dt, int64_t ndof, void* stream) {
    return update_dynamic<PP_VELOCITY_VERLET>(force, u, ud, udd, bc_types, bc_values,
                                              densities, bc_scale, damping, dt, ndof, stream);
}

extern "C" const char* pp_status_string(int status) {
    switch (status) {
        case PP_SUCCESS: return "success";
        case PP_ERROR_INVALID_VALUE: return "invalid value (size, pointer or flag)";
        case PP_ERROR_MAX_NEIGH: return "max_neigh must be a power of two in [1, 1024]";
        case PP_ERROR_MISALIGNED: return "pointer not 16-byte aligned";
        case PP_ERROR_UNSUPPORTED: return "unsupported option combination";
        case PP_ERROR_CUDA: return "CUDA runtime error";
        case PP_ERROR_TOO_LARGE: return "nsteps exceeds PP_STATIC_MAX_STEPS";
    }
    return "unknown status";
}

extern "C" int pp_abi_version(void) { return PP_ABI_VERSION; }
