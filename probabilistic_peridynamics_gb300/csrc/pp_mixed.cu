// pp_mixed.cu -- PP_MIXED set-up (pack, export, bond extent), argument
// checks and dispatch of a step to its tile shape.  The kernel itself is in
// pp_mixed.cuh, instantiated per tile shape in pp_mixed_v*.cu.
#include "pp_tiled.cuh"

namespace pp {
namespace tiling {
int tile_export(const pp_fused_args& a, cudaStream_t st);
int validate_tiling(const pp_fused_args& a);
}  // namespace tiling

namespace mixed {
namespace {

// ------------------------------------------------------ pack / export
// Node i of the mixed layout from reference node perm[i] (perm NULL: i).
__global__ void k_mixed_pack(pp_fused_args a, int parity, const int32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nnodes) return;
    const int64_t src = perm ? perm[i] : i;
    const int64_t o = 3 * src;
    int4 q;
    const double inv = 1.0 / a.pos_scale;  // pos_scale is a power of two: exact
    q.x = (int)llrint((a.r0[o] - a.pos_origin[0]) * inv);
    q.y = (int)llrint((a.r0[o + 1] - a.pos_origin[1]) * inv);
    q.z = (int)llrint((a.r0[o + 2] - a.pos_origin[2]) * inv);
    const double w = a.bond_types ? a.vols[src] : a.bond_stiffness * a.vols[src];
    q.w = __float_as_int((float)w);
    float* rec = a.rec[parity] + 8 * (int64_t)i;
    reinterpret_cast<int4*>(rec)[0] = q;
    const double* u = a.u[parity];
    float umax = 0.f;
    int fl = 0;
    for (int d = 0; d < 3; ++d) {
        const df x = df_from_double(u[o + d]);
        rec[4 + d] = x.hi;
        a.ulo[parity][4 * (int64_t)i + d] = x.lo;
        umax = fmaxf(umax, fabsf(x.hi));
        fl |= (a.bc_types[o + d] != 0) << d;
        fl |= (a.fc_types[o + d] != 0) << (3 + d);
    }
    a.nflags[i] = fl;
    rec[7] = umax * (1.0f + 1.2e-7f);
    if (a.umax) atomicMax(reinterpret_cast<int*>(a.umax), __float_as_int(umax * (1.0f + 1.2e-7f)));
    a.ulo[parity][4 * (int64_t)i + 3] = 0.f;
    if (a.vel) {
        for (int d = 0; d < 3; ++d) {
            const df v = df_from_double(a.ud ? a.ud[o + d] : 0.0);
            a.vel[8 * (int64_t)i + d] = v.hi;
            a.vel[8 * (int64_t)i + 4 + d] = v.lo;
            a.acc[4 * (int64_t)i + d] = a.udd ? (float)a.udd[o + d] : 0.f;
            a.rho32[4 * (int64_t)i + d] = a.densities ? (float)(1.0 / a.densities[o + d]) : 1.f;
        }
        a.vel[8 * (int64_t)i + 3] = 0.f;
        a.vel[8 * (int64_t)i + 7] = 0.f;
        a.acc[4 * (int64_t)i + 3] = 0.f;
        a.rho32[4 * (int64_t)i + 3] = 1.f;
    }
    if (a.sc32 && !perm) {
        const int64_t row = (int64_t)i * a.max_neigh;
        for (int k = 0; k < a.max_neigh; ++k)
            a.sc32[row + k] = (float)a.stiffness_corrections[row + k];
    }
}

// Reference node perm[i] (perm NULL: i) from node i of the mixed layout;
// with a tiling, n_neigh and damage from the tiling's intact counts.
__global__ void k_mixed_export(pp_fused_args a, int parity, const int32_t* __restrict__ perm,
                               const int32_t* __restrict__ tile_n_neigh) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nnodes) return;
    const int64_t dst = perm ? perm[i] : i;
    const int64_t o = 3 * dst;
    for (int d = 0; d < 3; ++d) {
        a.u[parity][o + d] =
            df_to_double(df{a.rec[parity][8 * (int64_t)i + 4 + d], a.ulo[parity][4 * (int64_t)i + d]});
        if (a.vel && a.ud)
            a.ud[o + d] =
                df_to_double(df{a.vel[8 * (int64_t)i + d], a.vel[8 * (int64_t)i + 4 + d]});
        if (a.acc && a.udd) a.udd[o + d] = (double)a.acc[4 * (int64_t)i + d];
        if (a.force) a.force[o + d] = (double)a.frc[8 * (int64_t)i + d];
        if (a.body_force) a.body_force[o + d] = (double)a.frc[8 * (int64_t)i + 4 + d];
    }
    if (tile_n_neigh) {
        a.n_neigh[dst] = tile_n_neigh[i];
        if (a.damage) a.damage[dst] = damage_of(tile_n_neigh[i], a.family[dst]);
    } else if (a.damage) {
        a.damage[i] = damage_of(a.n_neigh[i], a.family[i]);
    }
}

__global__ void k_init_extent(unsigned long long* p) {
    p[0] = 0ull;                                               // max component
    p[1] = (unsigned long long)__double_as_longlong(1.0e300);  // min length
}

// Warp per node: max |r0[j][d] - r0[i][d]| and min |r0[j] - r0[i]| over the
// row's bonds (non-negative doubles order as unsigned integers).
__global__ void k_bond_extent(const int32_t* __restrict__ nlist, const double* __restrict__ r0,
                              int nnodes, int max_neigh, unsigned long long* out) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= nnodes) return;
    double mx = 0.0, mn = 1.0e300;
    for (int k = lane; k < max_neigh; k += 32) {
        const int j = nlist[(int64_t)i * max_neigh + k];
        if (j < 0 || j >= nnodes) continue;
        double l2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double x = r0[3 * (int64_t)j + d] - r0[3 * (int64_t)i + d];
            mx = fmax(mx, fabs(x));
            l2 += x * x;
        }
        mn = fmin(mn, sqrt(l2));
    }
    for (int off = 16; off >= 1; off >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(kFull, mx, off));
        mn = fmin(mn, __shfl_xor_sync(kFull, mn, off));
    }
    if (lane == 0) {
        atomicMax(out, (unsigned long long)__double_as_longlong(mx));
        atomicMin(out + 1, (unsigned long long)__double_as_longlong(mn));
    }
}

}  // namespace
}  // namespace mixed

int validate_mixed(const pp_fused_args& a) {
    using mixed::kMaxTable;
    if (!a.rec[0] || !a.rec[1] || !a.ulo[0] || !a.ulo[1] || !a.frc || !a.nflags)
        return PP_ERROR_INVALID_VALUE;
    if (!aligned32(a.rec[0]) || !aligned32(a.rec[1]) || !aligned16(a.ulo[0]) ||
        !aligned16(a.ulo[1]) || !aligned16(a.frc))
        return PP_ERROR_MISALIGNED;
    if (a.integrator != PP_EULER && (!a.vel || !a.acc || !a.rho32)) return PP_ERROR_INVALID_VALUE;
    if (a.tiling) {
        const int rc = tiling::validate_tiling(a);
        if (rc != PP_SUCCESS) return rc;
    } else if (a.stiffness_corrections && !a.sc32) {
        return PP_ERROR_INVALID_VALUE;
    }
    if (a.bond_types && a.nbond_types * a.nregimes > kMaxTable) return PP_ERROR_UNSUPPORTED;
    if (!(a.pos_scale > 0.0)) return PP_ERROR_INVALID_VALUE;
    if (a.variant < 0 || a.variant >= PP_MIXED_VARIANTS) return PP_ERROR_INVALID_VALUE;
    if (!a.umax || !a.status) return PP_ERROR_INVALID_VALUE;
    if (a.max_neigh > 256) return PP_ERROR_UNSUPPORTED;
    if (a.node_instance && a.ninstances > kMaxTable) return PP_ERROR_UNSUPPORTED;
    return PP_SUCCESS;
}

int launch_mixed_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    if (a.tiling) {
        // the node arrays the step reads by node, in internal order
        const pp_tiling& t = *a.tiling;
        pp_fused_args ai = a;
        ai.r0 = t.r0;
        ai.bc_values = t.bc_values;
        ai.fc_values = t.fc_values;
        ai.n_neigh = t.n_neigh;
        ai.node_instance = t.node_instance;
        ai.tiling = nullptr;
        switch (a.variant) {
            case 0: return tiled::launch_tiled_shape0(ai, t, parity, l, st);
            case 1: return tiled::launch_tiled_shape1(ai, t, parity, l, st);
            case 2: return tiled::launch_tiled_shape2(ai, t, parity, l, st);
        }
        return PP_ERROR_INVALID_VALUE;
    }
    switch (a.variant) {
        case 0: return mixed::launch_mixed_shape0(a, parity, l, st);
        case 1: return mixed::launch_mixed_shape1(a, parity, l, st);
        case 2: return mixed::launch_mixed_shape2(a, parity, l, st);
    }
    return PP_ERROR_INVALID_VALUE;
}

}  // namespace pp

using namespace pp;
using namespace pp::mixed;

extern "C" int pp_bond_extent(const int32_t* nlist, const double* r0, int32_t nnodes,
                              int32_t max_neigh, double* extent, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (!extent) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* out = reinterpret_cast<unsigned long long*>(extent);
    k_init_extent<<<1, 1, 0, st>>>(out);
    if (nnodes > 0) {
        if (!nlist || !r0) return PP_ERROR_INVALID_VALUE;
        k_bond_extent<<<(nnodes + 7) / 8, 256, 0, st>>>(nlist, r0, nnodes, max_neigh, out);
    }
    return launch_status();
}

extern "C" int pp_mixed_pack(const pp_fused_args* args, int32_t parity, void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0 || !is_pow2_le_1024(a.max_neigh)) return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.r0 || !a.vols || !a.u[parity] || !a.rec[parity] || !a.ulo[parity] || !a.nflags ||
        !a.bc_types || !a.fc_types || !(a.pos_scale > 0.0))
        return PP_ERROR_INVALID_VALUE;
    if (!aligned32(a.rec[parity]) || !aligned16(a.ulo[parity])) return PP_ERROR_MISALIGNED;
    if (a.vel && (!a.acc || !a.rho32)) return PP_ERROR_INVALID_VALUE;
    if (a.sc32 && !a.stiffness_corrections) return PP_ERROR_INVALID_VALUE;
    if (a.tiling && !a.tiling->perm) return PP_ERROR_INVALID_VALUE;
    k_mixed_pack<<<(a.nnodes + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        a, parity, a.tiling ? a.tiling->perm : nullptr);
    return launch_status();
}

extern "C" int pp_mixed_export(const pp_fused_args* args, int32_t parity, void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.u[parity] || !a.rec[parity] || !a.ulo[parity] || !a.frc || !a.n_neigh || !a.family)
        return PP_ERROR_INVALID_VALUE;
    if (a.tiling && (!a.tiling->perm || !a.tiling->n_neigh)) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_mixed_export<<<(a.nnodes + 255) / 256, 256, 0, st>>>(
        a, parity, a.tiling ? a.tiling->perm : nullptr, a.tiling ? a.tiling->n_neigh : nullptr);
    const int rc = launch_status();
    if (rc != PP_SUCCESS || !a.tiling) return rc;
    return tiling::tile_export(a, st);
}
