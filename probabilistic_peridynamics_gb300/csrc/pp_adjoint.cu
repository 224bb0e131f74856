// pp_adjoint.cu -- reverse (adjoint) step of the Euler time step with
// per-bond stiffness and a frozen bond set, for gradients of a
// displacement loss.
//
// Forward step (run with pp_fused_step, PP_FLOAT64, stiffness corrections =
// per-bond stiffness k_b, bond_stiffness = 1, critical_stretch = +inf so
// the bond set stays frozen):
//   u'_m = u_m + dt f_m(u)   on free DOFs,   u'_m = c * bc_values on BC DOFs
//   f_m  = sum_{b=(m,j)} k_b vol_j s_b p_b/|p_b|,  p_b = xi_b + u_j - u_m,
//   s_b  = (|p_b| - |xi_b|)/|xi_b|            (peridynamics.cl:65-87, :214)
// Reverse of one step, with mu = lambda' masked to the free DOFs:
//   lambda_m = mu_m + dt sum_{b=(m,j)} G_b (k_(j,m) vol_m mu_j - k_b vol_j mu_m)
//   G(p)     = p^ p^T / |xi| + (s/|p|)(I - p^ p^T)      (symmetric, even in p)
//   dL/dk_b += dt vol_j s_b (mu_m . p^_b)
// The first sum gathers the contribution of the reverse bond (j, m) from
// row m itself: G is the same for both directions of a bond, and the
// reverse bond's stiffness is found through the partner slot.  One warp per
// node, no atomics: the gradient is deterministic.
#include "pp_common.cuh"

namespace pp {
namespace {

constexpr int kWarps = 8;

__global__ void __launch_bounds__(kWarps * 32)
    k_partner_slots(const int32_t* __restrict__ nlist, int nnodes, int L,
                    int32_t* __restrict__ partner) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (i >= nnodes) return;
    for (int s = lane; s < L; s += 32) {
        const int j = nlist[(int64_t)i * L + s];
        int found = -1;
        if (j >= 0 && j < nnodes) {
            const int32_t* row = nlist + (int64_t)j * L;
            for (int q = 0; q < L; ++q)
                if (row[q] == i) {
                    found = q;
                    break;
                }
        }
        partner[(int64_t)i * L + s] = found;
    }
}

__global__ void __launch_bounds__(kWarps * 32)
    k_adjoint_backward(pp_adjoint_args a, const double* __restrict__ u,
                       const double* __restrict__ lam_next, double* __restrict__ lam,
                       double* __restrict__ grad_k) {
    const int lane = threadIdx.x & 31;
    const int m = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (m >= a.nnodes) return;  // warp-uniform
    const int L = a.max_neigh;
    const int64_t o3 = 3 * (int64_t)m;
    const double rmx = a.r0[o3], rmy = a.r0[o3 + 1], rmz = a.r0[o3 + 2];
    const double umx = u[o3], umy = u[o3 + 1], umz = u[o3 + 2];
    // mu = lambda_next on the free DOFs of node m
    const double mmx = a.bc_types[o3] ? 0.0 : lam_next[o3];
    const double mmy = a.bc_types[o3 + 1] ? 0.0 : lam_next[o3 + 1];
    const double mmz = a.bc_types[o3 + 2] ? 0.0 : lam_next[o3 + 2];
    const double vol_m = a.vols[m];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int s = lane; s < L; s += 32) {
        const int64_t gid = (int64_t)m * L + s;
        const int j = a.nlist[gid];
        if (j == -1) continue;
        const int64_t j3 = 3 * (int64_t)j;
        const double xx = a.r0[j3] - rmx, xy = a.r0[j3 + 1] - rmy, xz = a.r0[j3 + 2] - rmz;
        const double px = u[j3] - umx + xx, py = u[j3 + 1] - umy + xy, pz = u[j3 + 2] - umz + xz;
        const double xi = sqrt(xx * xx + xy * xy + xz * xz);
        const double y = sqrt(px * px + py * py + pz * pz);
        const double st = (y - xi) / xi;
        const double hx = px / y, hy = py / y, hz = pz / y;
        const double mjx = a.bc_types[j3] ? 0.0 : lam_next[j3];
        const double mjy = a.bc_types[j3 + 1] ? 0.0 : lam_next[j3 + 1];
        const double mjz = a.bc_types[j3 + 2] ? 0.0 : lam_next[j3 + 2];
        const double kb = a.stiffness[gid];
        const int q = a.partner[gid];
        const double krev =
            (q >= 0 && a.nlist[(int64_t)j * L + q] == m) ? a.stiffness[(int64_t)j * L + q] : 0.0;
        // v = k_(j,m) vol_m mu_j - k_b vol_j mu_m
        const double vol_j = a.vols[j];
        const double vx = krev * vol_m * mjx - kb * vol_j * mmx;
        const double vy = krev * vol_m * mjy - kb * vol_j * mmy;
        const double vz = krev * vol_m * mjz - kb * vol_j * mmz;
        // G v = (h.v)/|xi| h + (s/|p|)(v - (h.v) h)
        const double hv = hx * vx + hy * vy + hz * vz;
        const double c1 = hv / xi, c2 = st / y;
        ax += c1 * hx + c2 * (vx - hv * hx);
        ay += c1 * hy + c2 * (vy - hv * hy);
        az += c1 * hz + c2 * (vz - hv * hz);
        // dL/dk_b += dt vol_j s_b (mu_m . h)
        grad_k[gid] += a.dt * vol_j * st * (mmx * hx + mmy * hy + mmz * hz);
    }
    for (int off = 16; off >= 1; off >>= 1) {
        ax += __shfl_xor_sync(kFull, ax, off);
        ay += __shfl_xor_sync(kFull, ay, off);
        az += __shfl_xor_sync(kFull, az, off);
    }
    if (lane == 0) {
        lam[o3] = mmx + a.dt * ax;
        lam[o3 + 1] = mmy + a.dt * ay;
        lam[o3 + 2] = mmz + a.dt * az;
    }
}

// First step at which each slot is seen broken.
__global__ void k_mark_breaks(const int32_t* __restrict__ nlist, int32_t* __restrict__ break_step,
                              int64_t nslots, int32_t t) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g < nslots && nlist[g] == -1 && break_step[g] > t) break_step[g] = t;
}

// The bond set in force during step t.
__global__ void k_bonds_at_step(const int32_t* __restrict__ nlist0,
                                const int32_t* __restrict__ break_step, int64_t nslots,
                                int32_t t, int32_t* __restrict__ nlist_t) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g < nslots) nlist_t[g] = break_step[g] > t ? nlist0[g] : -1;
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_mark_breaks(const int32_t* nlist, int32_t* break_step, int64_t nslots,
                              int32_t t, void* stream) {
    if (nslots < 0) return PP_ERROR_INVALID_VALUE;
    if (nslots == 0) return PP_SUCCESS;
    if (!nlist || !break_step) return PP_ERROR_INVALID_VALUE;
    k_mark_breaks<<<(unsigned)((nslots + 255) / 256), 256, 0,
                    static_cast<cudaStream_t>(stream)>>>(nlist, break_step, nslots, t);
    return launch_status();
}

extern "C" int pp_bonds_at_step(const int32_t* nlist0, const int32_t* break_step, int64_t nslots,
                                int32_t t, int32_t* nlist_t, void* stream) {
    if (nslots < 0) return PP_ERROR_INVALID_VALUE;
    if (nslots == 0) return PP_SUCCESS;
    if (!nlist0 || !break_step || !nlist_t) return PP_ERROR_INVALID_VALUE;
    k_bonds_at_step<<<(unsigned)((nslots + 255) / 256), 256, 0,
                      static_cast<cudaStream_t>(stream)>>>(nlist0, break_step, nslots, t,
                                                           nlist_t);
    return launch_status();
}

extern "C" int pp_partner_slots(const int32_t* nlist, int32_t nnodes, int32_t max_neigh,
                                int32_t* partner, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!nlist || !partner) return PP_ERROR_INVALID_VALUE;
    k_partner_slots<<<(nnodes + kWarps - 1) / kWarps, kWarps * 32, 0,
                      static_cast<cudaStream_t>(stream)>>>(nlist, nnodes, max_neigh, partner);
    return launch_status();
}

extern "C" int pp_adjoint_backward(const pp_adjoint_args* args, const double* u,
                                   const double* lam_next, double* lam, double* grad_k,
                                   void* stream) {
    if (!args) return PP_ERROR_INVALID_VALUE;
    const pp_adjoint_args& a = *args;
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(a.max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.r0 || !a.vols || !a.nlist || !a.partner || !a.bc_types || !a.stiffness || !u ||
        !lam_next || !lam || !grad_k || lam == lam_next)
        return PP_ERROR_INVALID_VALUE;
    k_adjoint_backward<<<(a.nnodes + kWarps - 1) / kWarps, kWarps * 32, 0,
                         static_cast<cudaStream_t>(stream)>>>(a, u, lam_next, lam, grad_k);
    return launch_status();
}
