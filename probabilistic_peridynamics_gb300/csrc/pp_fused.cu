// pp_fused.cu -- one launch per time step: stretch, break / regime update,
// bond force, per-node reduction, force boundary conditions, intact count
// and the integrator update, for one warp per node.
//
// Two arithmetic variants share the structure:
//
// * PP_FLOAT64: the binary64 bond arithmetic of pp_bond_f64.cuh and the
//   work-group tree order, then the reference integrator formulas
//   (euler.cl:23, euler_cromer.cl:55-58, velocity_verlet.cl:90-94) applied
//   by lanes 0..2 (one DOF each).  Bit-identical to the plain kernels.
//
// * PP_MIXED: FP32 bond arithmetic on compact gathers (int4 fixed-point
//   positions + volume, float4 displacement), an exact binary64 stretch test
//   only where the FP32 stretch lies within its error band of a critical
//   stretch, an FP32 warp reduction (optionally compensated), and the
//   integrator update in double-float arithmetic.  No binary64 instruction
//   runs per bond or per node unless a bond needs the exact test or a node
//   carries a boundary condition; on GB300 the FP64 pipe is ~1/64 of FP32.
//
// Displacements are double-buffered (read slot `parity`, write parity ^ 1).
// Velocities and accelerations belong to their node's warp alone and are
// updated in place.
#include "pp_bond_f64.cuh"

namespace pp {
namespace {

constexpr int kDefaultWarps = 8;
constexpr int kMaxTable = 256;  // nbond_types * nregimes handled by the mixed kernel

struct StepMags {
    double disp;
    double force;
};

// Magnitudes of this step: by value, or from device arrays indexed by
// k_off (+ *base when base != nullptr, the graph-replay case).
__device__ __forceinline__ StepMags step_mags(double disp, double force, const double* dmags,
                                              const double* fmags, const int64_t* base,
                                              int64_t k_off) {
    if (dmags == nullptr) return StepMags{disp, force};
    const int64_t idx = (base ? *base : 0) + k_off;
    return StepMags{dmags[idx], fmags[idx]};
}

// ------------------------------------------------------------------ FP64
template <int SL, bool CORR, bool TYPES>
__global__ void __launch_bounds__(256)
    k_fused_f64(pp_fused_args a, int parity, double disp_in, double force_in,
                const double* __restrict__ dmags, const double* __restrict__ fmags,
                const int64_t* __restrict__ base, int64_t k_off) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int i = blockIdx.x * wpb + (threadIdx.x >> 5);
    if (i >= a.nnodes) return;  // warp-uniform
    const StepMags m = step_mags(disp_in, force_in, dmags, fmags, base, k_off);
    const double* __restrict__ u = a.u[parity];
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
                    a.bond_stiffness,
                    a.critical_stretch,
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
    const double fx = __shfl_sync(kFull, f.x, 0);
    const double fy = __shfl_sync(kFull, f.y, 0);
    const double fz = __shfl_sync(kFull, f.z, 0);
    if (lane < 3) {
        const int64_t o = o3 + lane;
        const double body = lane == 0 ? fx : (lane == 1 ? fy : fz);
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
                unew = velocity_verlet_u(u[o], v, acc, frc, bct, bcv, a.densities[o], m.disp,
                                         a.damping, a.dt);
            a.ud[o] = v;
            a.udd[o] = acc;
        }
        a.u[parity ^ 1][o] = unew;
    }
    if (lane == 0) {
        a.n_neigh[i] = count;
        a.damage[i] = damage_of(count, a.family[i]);
    }
}

// ----------------------------------------------------------------- mixed
struct MixedConst {
    float h;        // fixed-point step of pos_q (a power of two)
    float geo;      // sqrt(3) * h: bound on the geometric rounding of xi
    float k;        // bond stiffness (PMB)
    float s0;       // critical stretch (PMB), rounded to float
    float dt_hi, dt_lo;      // dt as a double-float pair
    float half_hi, half_lo;  // dt/2 as a double-float pair
    float damping;
};

// Binary64 stretch of bond (i, j) from the reference r0 and the exact
// double-float displacement, in the reference operation order
// (peridynamics.cl:65-75).
__device__ __noinline__ double exact_stretch(const pp_fused_args& a, int parity, int i, int j) {
    const float4 hi_i = ldg_f4(a.uhi[parity], i), lo_i = ldg_f4(a.ulo[parity], i);
    const float4 hi_j = ldg_f4(a.uhi[parity], j), lo_j = ldg_f4(a.ulo[parity], j);
    const double* ri = a.r0 + 3 * (int64_t)i;
    const double* rj = a.r0 + 3 * (int64_t)j;
    const double uix = dadd((double)hi_i.x, (double)lo_i.x);
    const double uiy = dadd((double)hi_i.y, (double)lo_i.y);
    const double uiz = dadd((double)hi_i.z, (double)lo_i.z);
    const double ujx = dadd((double)hi_j.x, (double)lo_j.x);
    const double ujy = dadd((double)hi_j.y, (double)lo_j.y);
    const double ujz = dadd((double)hi_j.z, (double)lo_j.z);
    const double xi_x = dsub(rj[0], ri[0]);
    const double xi_y = dsub(rj[1], ri[1]);
    const double xi_z = dsub(rj[2], ri[2]);
    const double xe_x = dadd(dsub(ujx, uix), xi_x);
    const double xe_y = dadd(dsub(ujy, uiy), xi_y);
    const double xe_z = dadd(dsub(ujz, uiz), xi_z);
    const double xi = dsqrt(dadd(dadd(dmul(xi_x, xi_x), dmul(xi_y, xi_y)), dmul(xi_z, xi_z)));
    const double y = dsqrt(dadd(dadd(dmul(xe_x, xe_x), dmul(xe_y, xe_y)), dmul(xe_z, xe_z)));
    return ddiv(dsub(y, xi), xi);
}

// Decide (stretch < threshold) as binary64 would: from the FP32 stretch when
// it is farther than the error band from the threshold, else from the exact
// binary64 stretch (computed at most once per bond).
struct ExactTest {
    const pp_fused_args& a;
    int parity, i, j;
    float s, band;
    bool have;
    double s64;
    __device__ __forceinline__ bool lt(float thr_f, double thr) {
        const float d = s - thr_f;
        if (fabsf(d) > band + 6.0e-8f * fabsf(thr_f)) return d < 0.0f;
        if (!have) {
            s64 = exact_stretch(a, parity, i, j);
            have = true;
        }
        return s64 < thr;
    }
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}
__device__ __forceinline__ float warp_sum_comp(float s, float c) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const float so = __shfl_xor_sync(kFull, s, off);
        const float co = __shfl_xor_sync(kFull, c, off);
        const df t = two_sum(s, so);
        s = t.hi;
        c = __fadd_rn(__fadd_rn(c, co), t.lo);
    }
    return __fadd_rn(s, c);
}

template <int SL, bool CORR, bool TYPES>
__global__ void __launch_bounds__(256)
    k_fused_mixed(pp_fused_args a, MixedConst c, int parity, double disp_in, double force_in,
                  const double* __restrict__ dmags, const double* __restrict__ fmags,
                  const int64_t* __restrict__ base, int64_t k_off) {
    __shared__ float thr_f[TYPES ? kMaxTable : 1];
    __shared__ float k_f[TYPES ? kMaxTable : 1];
    __shared__ float c_f[TYPES ? kMaxTable : 1];
    if constexpr (TYPES) {
        const int nt = a.nbond_types * a.nregimes;
        for (int t = threadIdx.x; t < nt; t += blockDim.x) {
            thr_f[t] = (float)a.critical_stretch_table[t];
            k_f[t] = (float)a.bond_stiffness_table[t];
            c_f[t] = (float)a.plus_cs[t];
        }
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int i = blockIdx.x * wpb + (threadIdx.x >> 5);
    if (i >= a.nnodes) return;  // warp-uniform
    const int L = a.max_neigh;
    const int64_t row = (int64_t)i * L;
    const float* __restrict__ uhi = a.uhi[parity];
    const int4 qi = ldg_i4(a.pos_q, i);
    const float4 ui = ldg_f4(uhi, i);
    const bool comp = (a.flags & PP_FLAG_COMPENSATED) != 0;

    float sx = 0.f, sy = 0.f, sz = 0.f;  // force sums
    float cx = 0.f, cy = 0.f, cz = 0.f;  // compensation terms
    int intact = 0;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
        const int slot = lane + 32 * k;
        if (SL == 1 && slot >= L) continue;
        const int64_t gid = row + slot;
        const int jr = a.nlist[gid];
        const bool valid = jr != -1;
        const int j = valid ? jr : i;  // keep the gathers unconditional
        const int4 qj = ldg_i4(a.pos_q, j);
        const float4 uj = ldg_f4(uhi, j);
        if (!valid) continue;
        const float xix = (float)(qj.x - qi.x) * c.h;
        const float xiy = (float)(qj.y - qi.y) * c.h;
        const float xiz = (float)(qj.z - qi.z) * c.h;
        const float ex = uj.x - ui.x, ey = uj.y - ui.y, ez = uj.z - ui.z;
        const float px = xix + ex, py = xiy + ey, pz = xiz + ez;
        const float xi2 = fmaf(xix, xix, fmaf(xiy, xiy, xiz * xiz));
        const float y2 = fmaf(px, px, fmaf(py, py, pz * pz));
        const float xe = fmaf(xix, ex, fmaf(xiy, ey, xiz * ez));
        const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
        const float rxi = rsqrtf(xi2);
        const float ry = rsqrtf(y2);
        const float xil = xi2 * rxi;
        const float yl = y2 * ry;
        // s = (|p| - |xi|)/|xi| without cancellation: (2 xi.e + e.e)/(|xi|(|p|+|xi|))
        const float s = __fdividef(fmaf(2.0f, xe, ee) * rxi, yl + xil);
        // Error band of s against the binary64 stretch of the same state.
        const float einf = fmaxf(fabsf(ex), fmaxf(fabsf(ey), fabsf(ez)));
        const float r = 1.7320508f * einf * rxi;  // >= |e|/|xi|
        const float as = fabsf(s);
        const float band =
            2.0f * (fmaf(c.geo, rxi, 1.1e-7f) * (2.0f * r + as) +
                    1.1e-7f * (ui.w + uj.w + einf) * rxi + 1.0e-6f * (2.0f * r + r * r + as)) +
            1.0e-12f;
        ExactTest t{a, parity, i, j, s, band, false, 0.0};
        float fk;
        if constexpr (!TYPES) {
            if (!t.lt(c.s0, a.critical_stretch)) {
                a.nlist[gid] = -1;
                continue;
            }
            fk = s * c.k;
        } else {
            const int nr = a.nregimes;
            const int bt = a.bond_types[gid] * nr;
            int reg = a.regimes[gid];
            const int rc = reg < 0 ? 0 : (reg >= nr ? nr - 1 : reg);
            if (t.lt(thr_f[bt + rc], a.critical_stretch_table[bt + rc])) {
                if (reg > 0 && rc > 0 &&
                    t.lt(thr_f[bt + rc - 1], a.critical_stretch_table[bt + rc - 1])) {
                    reg -= 1;
                    a.regimes[gid] = reg;
                }
            } else {
                reg += 1;
                a.regimes[gid] = reg;
            }
            if (reg >= nr) {
                a.nlist[gid] = -1;
                continue;
            }
            const int rr = reg < 0 ? 0 : reg;
            fk = fmaf(s, k_f[bt + rr], c_f[bt + rr]);
        }
        if constexpr (CORR) fk *= __ldg(a.sc32 + gid);
        const float fv = fk * __int_as_float(qj.w) * ry;
        intact += 1;
        if (comp) {
            df q = two_sum(sx, fv * px);
            sx = q.hi;
            cx += q.lo;
            q = two_sum(sy, fv * py);
            sy = q.hi;
            cy += q.lo;
            q = two_sum(sz, fv * pz);
            sz = q.hi;
            cz += q.lo;
        } else {
            sx = fmaf(fv, px, sx);
            sy = fmaf(fv, py, sy);
            sz = fmaf(fv, pz, sz);
        }
    }
    float fx, fy, fz;
    if (comp) {
        fx = warp_sum_comp(sx, cx);
        fy = warp_sum_comp(sy, cy);
        fz = warp_sum_comp(sz, cz);
    } else {
        fx = warp_sum(sx);
        fy = warp_sum(sy);
        fz = warp_sum(sz);
    }
    const int count = __reduce_add_sync(kFull, intact);
    const StepMags m = step_mags(disp_in, force_in, dmags, fmags, base, k_off);
    // Lanes 0..2 update one DOF each; every lane takes part in the
    // shuffles that assemble max|u| for the gather record.
    const int d = lane < 3 ? lane : 0;
    const int64_t o = 3 * (int64_t)i + d;
    const float body = d == 0 ? fx : (d == 1 ? fy : fz);
    float hi_new = 0.f, lo_new = 0.f;
    if (lane < 3) {
        float frc = body;
        if (a.fc_types[o] != 0)
            frc = (float)((double)body + m.force * a.fc_values[o]);
        const float* ulo_in = a.ulo[parity];
        df uu{uhi[4 * (int64_t)i + d], ulo_in[4 * (int64_t)i + d]};
        const df dt{c.dt_hi, c.dt_lo};
        const df half{c.half_hi, c.half_lo};
        const int bct = a.bc_types[o];
        if (a.integrator == PP_EULER) {
            uu = df_add(uu, df_mul_f(dt, frc));
        } else {
            float* vel = a.vel;
            df v{vel[8 * (int64_t)i + d], vel[8 * (int64_t)i + 4 + d]};
            const float rho = a.rho32[4 * (int64_t)i + d];
            float acc;
            if (a.integrator == PP_EULER_CROMER) {
                acc = __fdiv_rn(frc - c.damping * v.hi, rho);
                v = df_add(v, df_mul_f(dt, acc));
                uu = df_add(uu, df_mul(dt, v));
            } else {
                const float acc_prev = a.acc[4 * (int64_t)i + d];
                const df v1 = df_add(v, df_mul_f(half, acc_prev));
                acc = __fdiv_rn(frc - c.damping * v1.hi, rho);
                v = df_add(v1, df_mul_f(half, acc));
                uu = df_add(uu, df_mul(dt, df_add(v, df_mul_f(half, acc))));
            }
            vel[8 * (int64_t)i + d] = v.hi;
            vel[8 * (int64_t)i + 4 + d] = v.lo;
            a.acc[4 * (int64_t)i + d] = acc;
        }
        if (bct != 0) uu = df_from_double(m.disp * a.bc_values[o]);
        hi_new = uu.hi;
        lo_new = uu.lo;
        a.frc[8 * (int64_t)i + d] = frc;
        a.frc[8 * (int64_t)i + 4 + d] = body;
    }
    // max |u| over the three components for the next step's error band.
    float umax = fabsf(hi_new);
    umax = fmaxf(umax, __shfl_sync(kFull, umax, 1));
    umax = fmaxf(umax, __shfl_sync(kFull, umax, 2));
    if (lane < 3) {
        a.uhi[parity ^ 1][4 * (int64_t)i + d] = hi_new;
        a.ulo[parity ^ 1][4 * (int64_t)i + d] = lo_new;
    }
    if (lane == 0) {
        a.uhi[parity ^ 1][4 * (int64_t)i + 3] = umax * (1.0f + 1.2e-7f);
        a.n_neigh[i] = count;
    }
}

// ------------------------------------------------------ pack / export
__global__ void k_mixed_pack(pp_fused_args a, int parity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nnodes) return;
    const int64_t o = 3 * (int64_t)i;
    int4 q;
    const double inv = 1.0 / a.pos_scale;  // pos_scale is a power of two: exact
    q.x = (int)llrint((a.r0[o] - a.pos_origin[0]) * inv);
    q.y = (int)llrint((a.r0[o + 1] - a.pos_origin[1]) * inv);
    q.z = (int)llrint((a.r0[o + 2] - a.pos_origin[2]) * inv);
    q.w = __float_as_int((float)a.vols[i]);
    reinterpret_cast<int4*>(a.pos_q)[i] = q;
    const double* u = a.u[parity];
    float umax = 0.f;
    for (int d = 0; d < 3; ++d) {
        const df x = df_from_double(u[o + d]);
        a.uhi[parity][4 * (int64_t)i + d] = x.hi;
        a.ulo[parity][4 * (int64_t)i + d] = x.lo;
        umax = fmaxf(umax, fabsf(x.hi));
    }
    a.uhi[parity][4 * (int64_t)i + 3] = umax * (1.0f + 1.2e-7f);
    a.ulo[parity][4 * (int64_t)i + 3] = 0.f;
    if (a.vel) {
        for (int d = 0; d < 3; ++d) {
            const df v = df_from_double(a.ud ? a.ud[o + d] : 0.0);
            a.vel[8 * (int64_t)i + d] = v.hi;
            a.vel[8 * (int64_t)i + 4 + d] = v.lo;
            a.acc[4 * (int64_t)i + d] = a.udd ? (float)a.udd[o + d] : 0.f;
            a.rho32[4 * (int64_t)i + d] = a.densities ? (float)a.densities[o + d] : 1.f;
        }
        a.vel[8 * (int64_t)i + 3] = 0.f;
        a.vel[8 * (int64_t)i + 7] = 0.f;
        a.acc[4 * (int64_t)i + 3] = 0.f;
        a.rho32[4 * (int64_t)i + 3] = 1.f;
    }
    if (a.sc32) {
        const int64_t row = (int64_t)i * a.max_neigh;
        for (int k = 0; k < a.max_neigh; ++k)
            a.sc32[row + k] = (float)a.stiffness_corrections[row + k];
    }
}

__global__ void k_mixed_export(pp_fused_args a, int parity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nnodes) return;
    const int64_t o = 3 * (int64_t)i;
    for (int d = 0; d < 3; ++d) {
        a.u[parity][o + d] =
            df_to_double(df{a.uhi[parity][4 * (int64_t)i + d], a.ulo[parity][4 * (int64_t)i + d]});
        if (a.vel && a.ud)
            a.ud[o + d] =
                df_to_double(df{a.vel[8 * (int64_t)i + d], a.vel[8 * (int64_t)i + 4 + d]});
        if (a.acc && a.udd) a.udd[o + d] = (double)a.acc[4 * (int64_t)i + d];
        if (a.force) a.force[o + d] = (double)a.frc[8 * (int64_t)i + d];
        if (a.body_force) a.body_force[o + d] = (double)a.frc[8 * (int64_t)i + 4 + d];
    }
    if (a.damage) a.damage[i] = damage_of(a.n_neigh[i], a.family[i]);
}

__global__ void k_set_base(int64_t* base, int64_t v) { *base = v; }
__global__ void k_advance_base(int64_t* base, int64_t by) { *base += by; }

// ----------------------------------------------------------- dispatch
int validate(const pp_fused_args& a) {
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(a.max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (a.integrator < PP_EULER || a.integrator > PP_VELOCITY_VERLET) return PP_ERROR_INVALID_VALUE;
    if (a.nodes_per_block < 0 || a.nodes_per_block > 32) return PP_ERROR_INVALID_VALUE;
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
    } else if (a.precision == PP_MIXED) {
        if (!a.pos_q || !a.uhi[0] || !a.uhi[1] || !a.ulo[0] || !a.ulo[1] || !a.frc)
            return PP_ERROR_INVALID_VALUE;
        if (!aligned16(a.pos_q) || !aligned16(a.uhi[0]) || !aligned16(a.uhi[1]) ||
            !aligned16(a.ulo[0]) || !aligned16(a.ulo[1]) || !aligned16(a.frc))
            return PP_ERROR_MISALIGNED;
        if (a.integrator != PP_EULER && (!a.vel || !a.acc || !a.rho32))
            return PP_ERROR_INVALID_VALUE;
        if (a.stiffness_corrections && !a.sc32) return PP_ERROR_INVALID_VALUE;
        if (a.bond_types && a.nbond_types * a.nregimes > kMaxTable) return PP_ERROR_UNSUPPORTED;
        if (!(a.pos_scale > 0.0)) return PP_ERROR_INVALID_VALUE;
    } else {
        return PP_ERROR_INVALID_VALUE;
    }
    return PP_SUCCESS;
}

MixedConst mixed_const(const pp_fused_args& a) {
    MixedConst c;
    c.h = (float)a.pos_scale;
    c.geo = 1.7320508f * c.h;
    c.k = (float)a.bond_stiffness;
    c.s0 = (float)a.critical_stretch;
    c.dt_hi = (float)a.dt;
    c.dt_lo = (float)(a.dt - (double)c.dt_hi);
    const double half = a.dt / 2;
    c.half_hi = (float)half;
    c.half_lo = (float)(half - (double)c.half_hi);
    c.damping = (float)a.damping;
    return c;
}

struct Launch {
    double disp, force;
    const double* dmags;
    const double* fmags;
    const int64_t* base;
    int64_t k_off;
};

template <int SL, bool CORR, bool TYPES>
void launch_variant(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const int wpb = a.nodes_per_block > 0 ? a.nodes_per_block : kDefaultWarps;
    const dim3 grid((a.nnodes + wpb - 1) / wpb), block(32 * wpb);
    if (a.precision == PP_FLOAT64)
        k_fused_f64<SL, CORR, TYPES><<<grid, block, 0, st>>>(a, parity, l.disp, l.force, l.dmags,
                                                             l.fmags, l.base, l.k_off);
    else
        k_fused_mixed<SL, CORR, TYPES><<<grid, block, 0, st>>>(
            a, mixed_const(a), parity, l.disp, l.force, l.dmags, l.fmags, l.base, l.k_off);
}

template <int SL>
void launch_sl(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    if (!corr && !types) launch_variant<SL, false, false>(a, parity, l, st);
    if (corr && !types) launch_variant<SL, true, false>(a, parity, l, st);
    if (!corr && types) launch_variant<SL, false, true>(a, parity, l, st);
    if (corr && types) launch_variant<SL, true, true>(a, parity, l, st);
}

int launch_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    switch (a.max_neigh > 32 ? a.max_neigh / 32 : 1) {
        case 1: launch_sl<1>(a, parity, l, st); break;
        case 2: launch_sl<2>(a, parity, l, st); break;
        case 4: launch_sl<4>(a, parity, l, st); break;
        case 8: launch_sl<8>(a, parity, l, st); break;
        case 16: launch_sl<16>(a, parity, l, st); break;
        case 32: launch_sl<32>(a, parity, l, st); break;
        default: return PP_ERROR_MAX_NEIGH;
    }
    return launch_status();
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_fused_step(const pp_fused_args* args, int32_t parity,
                             double displacement_bc_magnitude, double force_bc_magnitude,
                             void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const int v = validate(*args);
    if (v != PP_SUCCESS || args->nnodes == 0) return v;
    const Launch l{displacement_bc_magnitude, force_bc_magnitude, nullptr, nullptr, nullptr, 0};
    return launch_step(*args, parity, l, static_cast<cudaStream_t>(stream));
}

extern "C" int pp_fused_run(const pp_fused_args* args, int32_t parity, int64_t nsteps,
                            const double* disp_mags, const double* force_mags, int64_t first,
                            int32_t use_graph, int32_t chunk, int64_t* step_base,
                            void* stream) {
    if (!args || (parity != 0 && parity != 1) || nsteps < 0 || first < 0)
        return PP_ERROR_INVALID_VALUE;
    if (!disp_mags || !force_mags) return PP_ERROR_INVALID_VALUE;
    const int v = validate(*args);
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
            rc = launch_step(*args, p ^ (k & 1), l, st);
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
        const int rc = launch_step(*args, p, l, st);
        if (rc != PP_SUCCESS) return rc;
        p ^= 1;
    }
    return PP_SUCCESS;
}

extern "C" int pp_mixed_pack(const pp_fused_args* args, int32_t parity, void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0 || !is_pow2_le_1024(a.max_neigh)) return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.r0 || !a.vols || !a.u[parity] || !a.pos_q || !a.uhi[parity] || !a.ulo[parity] ||
        !(a.pos_scale > 0.0))
        return PP_ERROR_INVALID_VALUE;
    if (!aligned16(a.pos_q) || !aligned16(a.uhi[parity]) || !aligned16(a.ulo[parity]))
        return PP_ERROR_MISALIGNED;
    if (a.vel && (!a.acc || !a.rho32)) return PP_ERROR_INVALID_VALUE;
    if (a.sc32 && !a.stiffness_corrections) return PP_ERROR_INVALID_VALUE;
    k_mixed_pack<<<(a.nnodes + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, parity);
    return launch_status();
}

extern "C" int pp_mixed_export(const pp_fused_args* args, int32_t parity, void* stream) {
    if (!args || (parity != 0 && parity != 1)) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.u[parity] || !a.uhi[parity] || !a.ulo[parity] || !a.frc || !a.n_neigh || !a.family)
        return PP_ERROR_INVALID_VALUE;
    k_mixed_export<<<(a.nnodes + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(a,
                                                                                       parity);
    return launch_status();
}
