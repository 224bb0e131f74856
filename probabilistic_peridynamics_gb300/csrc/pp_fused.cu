// pp_fused.cu -- one launch per time step: stretch, break / regime update,
// bond force, per-node reduction, force boundary conditions, intact count
// and the integrator update.
//
// This unit holds the PP_FLOAT64 kernel, the argument checks, and the
// entry points pp_fused_step / pp_fused_run (which dispatch PP_MIXED to
// pp_mixed.cu).
//
// PP_FLOAT64: one warp per node; the binary64 bond arithmetic of
// pp_bond_f64.cuh summed in the work-group tree order, then the reference
// integrator formulas (euler.cl:23, euler_cromer.cl:55-58,
// velocity_verlet.cl:90-94) applied by lanes 0..2 (one DOF each).  The
// results are bit-identical to the plain kernels.  Displacements are
// double-buffered (read slot `parity`, write parity ^ 1); velocities and
// accelerations belong to their node's warp alone and are updated in place.
#include "pp_bond_f64.cuh"
#include "pp_fused.cuh"

namespace pp {
namespace {

constexpr int kDefaultWarps = 8;

// One warp per node for the bond phase; the node updates of the block's
// nodes then run one thread per DOF (the update's binary64 instructions
// would otherwise occupy GB300's FP64 pipe for a whole warp per 3 lanes).
template <int SL, bool CORR, bool TYPES>
__global__ void __launch_bounds__(256) k_fused_f64(pp_fused_args a, int parity, Launch l) {
    __shared__ double s_f[32][3];
    __shared__ int s_cnt[32];
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5;
    const int node0 = blockIdx.x * wpb;
    const int i = node0 + warp;
    const StepMags m = step_mags(l);
    const double* __restrict__ u = a.u[parity];
    if (i < a.nnodes) {  // warp-uniform
        const F64Bond b{a.r0,
                        u,
                        a.vols,
                        a.nlist,
                        a.stiffness_corrections,
                        a.bond_types,
                        a.regimes,
                        a.bond_stiffness_table,
                        a.critical_stretch_table,
                        a.plus_cs,
                        a.bond_length,
                        a.bond_stiffness,
                        a.node_instance ? a.instance_s0[a.node_instance[i]] : a.critical_stretch,
                        a.nregimes};
        const int64_t o3 = 3 * (int64_t)i;
        const d3 ri{a.r0[o3], a.r0[o3 + 1], a.r0[o3 + 2]};
        const d3 ui{u[o3], u[o3 + 1], u[o3 + 2]};
        const int64_t row = (int64_t)i * a.max_neigh;
        int intact = 0;
        const d3 f = tree_reduce_f64<SL>(lane, a.max_neigh, [&](int k) {
            return f64_slot<CORR, TYPES>(b, row + k, ri, ui, intact);
        });
        const int count = __reduce_add_sync(kFull, intact);
        if (lane == 0) {
            s_f[warp][0] = f.x;
            s_f[warp][1] = f.y;
            s_f[warp][2] = f.z;
            s_cnt[warp] = count;
        }
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t < 3 * wpb) {
        const int li = t / 3, d = t % 3;
        const int n = node0 + li;
        if (n < a.nnodes) {
            const int64_t o = 3 * (int64_t)n + d;
            const double body = s_f[li][d];
            a.body_force[o] = body;
            const double frc = force_with_bc(body, a.fc_types[o], a.fc_values[o], m.force);
            a.force[o] = frc;
            const int bct = a.bc_types[o];
            const double bcv = a.bc_values[o];
            double unew;
            if (a.integrator == PP_EULER) {
                unew = euler_u(u[o], frc, bct, bcv, m.disp, a.dt);
            } else {
                double v = a.ud[o];
                double acc = a.udd[o];
                if (a.integrator == PP_EULER_CROMER)
                    unew = euler_cromer_u(u[o], v, acc, frc, bct, bcv, a.densities[o], m.disp,
                                          a.damping, a.dt);
                else
                    unew = velocity_verlet_u(u[o], v, acc, frc, bct, bcv, a.densities[o],
                                             m.disp, a.damping, a.dt);
                a.ud[o] = v;
                a.udd[o] = acc;
            }
            a.u[parity ^ 1][o] = unew;
        }
    } else if (t < 4 * wpb) {
        const int n = node0 + (t - 3 * wpb);
        if (n < a.nnodes) {
            const int count = s_cnt[t - 3 * wpb];
            a.n_neigh[n] = count;
            a.damage[n] = damage_of(count, a.family[n]);
        }
    }
}

// One thread per slot: |r0[j] - r0[i]| as the bond body computes it.
__global__ void k_bond_lengths(const double* __restrict__ r0, const int32_t* __restrict__ nlist,
                               int nnodes, int max_neigh, double* __restrict__ length) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= (int64_t)nnodes * max_neigh) return;
    const int j = nlist[g];
    const int64_t i = g / max_neigh;
    double len = 0.0;
    if (j >= 0 && j < nnodes) {
        const double x = dsub(r0[3 * (int64_t)j], r0[3 * i]);
        const double y = dsub(r0[3 * (int64_t)j + 1], r0[3 * i + 1]);
        const double z = dsub(r0[3 * (int64_t)j + 2], r0[3 * i + 2]);
        len = dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)));
    }
    length[g] = len;
}

__global__ void k_set_base(int64_t* base, int64_t v) { *base = v; }
__global__ void k_advance_base(int64_t* base, int64_t by) { *base += by; }

}  // namespace

int validate_fused(const pp_fused_args& a) {
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(a.max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (a.integrator < PP_EULER || a.integrator > PP_VELOCITY_VERLET) return PP_ERROR_INVALID_VALUE;
    if (a.nodes_per_block < 0 || a.nodes_per_block > 8) return PP_ERROR_INVALID_VALUE;
    if (a.reserved != 0 || a.reserved2 != 0) return PP_ERROR_INVALID_VALUE;
    if (a.flags & ~PP_FLAG_COMPENSATED) return PP_ERROR_INVALID_VALUE;
    // compensation applies to the FP32 force sums of PP_MIXED only
    if ((a.flags & PP_FLAG_COMPENSATED) && a.precision != PP_MIXED) return PP_ERROR_UNSUPPORTED;
    if (a.node_instance &&
        (a.bond_types || !a.instance_s0 || a.ninstances < 1 || a.ninstances > 256))
        return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.r0 || !a.vols || !a.family || !a.bc_types || !a.bc_values || !a.fc_types ||
        !a.fc_values || !a.nlist || !a.n_neigh)
        return PP_ERROR_INVALID_VALUE;
    if (a.integrator != PP_EULER && !a.densities) return PP_ERROR_INVALID_VALUE;
    if (a.bond_types && (!a.regimes || !a.plus_cs || !a.bond_stiffness_table ||
                         !a.critical_stretch_table || a.nregimes < 1 || a.nbond_types < 1))
        return PP_ERROR_INVALID_VALUE;
    if (a.precision == PP_FLOAT64) {
        if (!a.u[0] || !a.u[1] || !a.force || !a.body_force || !a.damage)
            return PP_ERROR_INVALID_VALUE;
        if (a.integrator != PP_EULER && (!a.ud || !a.udd)) return PP_ERROR_INVALID_VALUE;
        return PP_SUCCESS;
    }
    if (a.precision == PP_MIXED) return validate_mixed(a);
    return PP_ERROR_INVALID_VALUE;
}

namespace {

template <int SL, bool CORR, bool TYPES>
void launch_f64_variant(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const int wpb = a.nodes_per_block > 0 ? a.nodes_per_block : kDefaultWarps;
    const dim3 grid((a.nnodes + wpb - 1) / wpb), block(32 * wpb);
    k_fused_f64<SL, CORR, TYPES><<<grid, block, 0, st>>>(a, parity, l);
}

template <int SL>
void launch_f64_sl(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    if (!corr && !types) launch_f64_variant<SL, false, false>(a, parity, l, st);
    if (corr && !types) launch_f64_variant<SL, true, false>(a, parity, l, st);
    if (!corr && types) launch_f64_variant<SL, false, true>(a, parity, l, st);
    if (corr && types) launch_f64_variant<SL, true, true>(a, parity, l, st);
}

}  // namespace

int launch_fused_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    if (a.precision == PP_MIXED) return launch_mixed_step(a, parity, l, st);
    switch (a.max_neigh > 32 ? a.max_neigh / 32 : 1) {
        case 1: launch_f64_sl<1>(a, parity, l, st); break;
        case 2: launch_f64_sl<2>(a, parity, l, st); break;
        case 4: launch_f64_sl<4>(a, parity, l, st); break;
        case 8: launch_f64_sl<8>(a, parity, l, st); break;
        case 16: launch_f64_sl<16>(a, parity, l, st); break;
        case 32: launch_f64_sl<32>(a, parity, l, st); break;
        default: return PP_ERROR_MAX_NEIGH;
    }
    return launch_status();
}

}  // namespace pp

using namespace pp;

extern "C" int pp_fused_step(const pp_fused_args* args, int32_t parity,
                             double displacement_bc_magnitude, double force_bc_magnitude,
                             void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const int v = validate_fused(*args);
    if (v != PP_SUCCESS || args->nnodes == 0) return v;
    const Launch l{displacement_bc_magnitude, force_bc_magnitude, nullptr, nullptr, nullptr, 0};
    return launch_fused_step(*args, parity, l, static_cast<cudaStream_t>(stream));
}

extern "C" int pp_fused_run(const pp_fused_args* args, int32_t parity, int64_t nsteps,
                            const double* disp_mags, const double* force_mags, int64_t first,
                            int32_t use_graph, int32_t chunk, int64_t* step_base,
                            void* stream) {
    if (!args || (parity != 0 && parity != 1) || nsteps < 0 || first < 0)
        return PP_ERROR_INVALID_VALUE;
    if (!disp_mags || !force_mags) return PP_ERROR_INVALID_VALUE;
    const int v = validate_fused(*args);
    if (v != PP_SUCCESS || args->nnodes == 0 || nsteps == 0) return v;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int64_t done = 0;
    int p = parity;
    // Graph replay needs a capturable (non-legacy) stream, an even chunk
    // (so the parity pattern repeats) and a scratch word for the step index.
    if (use_graph && st != nullptr && step_base != nullptr && chunk >= 2 && (chunk & 1) == 0 &&
        nsteps >= 2 * (int64_t)chunk) {
        k_set_base<<<1, 1, 0, st>>>(step_base, first);
        if (launch_status() != PP_SUCCESS) return PP_ERROR_CUDA;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return PP_ERROR_CUDA;
        int rc = PP_SUCCESS;
        for (int k = 0; k < chunk && rc == PP_SUCCESS; ++k) {
            const Launch l{0.0, 0.0, disp_mags, force_mags, step_base, k};
            rc = launch_fused_step(*args, p ^ (k & 1), l, st);
        }
        if (rc == PP_SUCCESS) {
            k_advance_base<<<1, 1, 0, st>>>(step_base, chunk);
            rc = launch_status();
        }
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (rc != PP_SUCCESS || ec != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return PP_ERROR_CUDA;
        }
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            cudaGraphDestroy(graph);
            return PP_ERROR_CUDA;
        }
        const int64_t reps = nsteps / chunk;
        for (int64_t r = 0; r < reps && rc == PP_SUCCESS; ++r)
            if (cudaGraphLaunch(exec, st) != cudaSuccess) rc = PP_ERROR_CUDA;
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        if (rc != PP_SUCCESS) return rc;
        done = reps * chunk;  // chunk is even: parity unchanged
    }
    for (int64_t k = done; k < nsteps; ++k) {
        const Launch l{0.0, 0.0, disp_mags, force_mags, nullptr, first + k};
        const int rc = launch_fused_step(*args, p, l, st);
        if (rc != PP_SUCCESS) return rc;
        p ^= 1;
    }
    return PP_SUCCESS;
}

extern "C" int pp_bond_lengths(const double* r0, const int32_t* nlist, int32_t nnodes,
                               int32_t max_neigh, double* length, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (max_neigh < 1 || max_neigh > 1024) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!r0 || !nlist || !length) return PP_ERROR_INVALID_VALUE;
    const int64_t slots = (int64_t)nnodes * max_neigh;
    k_bond_lengths<<<(unsigned)((slots + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        r0, nlist, nnodes, max_neigh, length);
    return launch_status();
}
