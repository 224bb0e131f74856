// pp_mixed.cu -- PP_MIXED fused step: FP32 bond arithmetic on compact
// gathers, the break / regime decision taken exactly as binary64 would on
// the same state, and double-float node state.
//
// Structure of one launch (one CTA = 8 warps = 64 consecutive nodes):
//
//  1. Bond phase, one warp per node (8 nodes per warp, the CTA's warps
//     working on 8 consecutive nodes at a time so their neighbourhoods share
//     L1 lines).  For the lane's max_neigh/32 slots: load all neighbour
//     indices, then all gathers (int4 fixed-point position + k*vol, float4
//     displacement + max|u|), then the FP32 bond arithmetic.  A slot whose
//     FP32 stretch lies within the proven error band of a critical stretch
//     is deferred to a slow path that evaluates the binary64 stretch of
//     peridynamics.cl:65-75 from the reference r0 and the exact
//     double-float displacement.  The four per-node sums (force x, y, z and
//     the intact count) are reduced with a 6-shuffle transposed butterfly
//     and parked in shared memory.
//  2. Node phase, all 256 threads: thread (node, component) applies the
//     force boundary condition and the integrator update of one DOF in
//     double-float arithmetic; every load and store of the node state is a
//     contiguous 1 KB access per CTA.
//
// Integer-to-float conversion uses the exponent trick
// float(q) = bits(0x4B400000 + q) - 1.5*2^23 (exact for |q| < 2^22), folded
// with the fixed-point scale into one FMA: on GB300 the I2F instruction
// runs on the FP64 pipe, which would otherwise bound this kernel.
//
// This translation unit is compiled with -ftz=true -prec-div=false
// -prec-sqrt=false: every FP32 rounding and approximation is covered by the
// error band; the double-float operations use explicit _rn intrinsics and
// the binary64 slow path is unaffected by those flags.
#include "pp_bond_f64.cuh"
#include "pp_fused.cuh"

namespace pp {
namespace {

constexpr int kWarps = 8;
constexpr int kChunk = 64;  // nodes per CTA
constexpr int kMaxTable = 256;

constexpr int kMagicI = 0x4B400000;  // bit pattern of 1.5 * 2^23
constexpr float kMagicF = 12582912.0f;

struct MixedConst {
    float h;       // fixed-point step (a power of two)
    float mh;      // -kMagicF * h
    float geo;     // sqrt(3) * h: bound on the rounding of each xi
    float s0;      // critical stretch (PMB), rounded to float
    float s0_err;  // 6e-8 * |s0|: rounding of s0 to float
    float dt_hi, dt_lo;
    float half_hi, half_lo;
    float damping;
};

// FP32 quantities of one bond (i -> j).
struct Bond32 {
    float px, py, pz;  // deformed bond vector
    float s;           // stretch
    float ry;          // 1 / |p|
    float band;        // bound on |s - s64|
};

__device__ __forceinline__ float fixed_diff(int qj, int qi, const MixedConst& c) {
    return fmaf(__int_as_float(qj - qi + kMagicI), c.h, c.mh);
}

__device__ __forceinline__ Bond32 bond32(const int4& qi, const float4& ui, const int4& qj,
                                         const float4& uj, const MixedConst& c) {
    const float xx = fixed_diff(qj.x, qi.x, c);
    const float xy = fixed_diff(qj.y, qi.y, c);
    const float xz = fixed_diff(qj.z, qi.z, c);
    const float ex = uj.x - ui.x, ey = uj.y - ui.y, ez = uj.z - ui.z;
    Bond32 b;
    b.px = xx + ex;
    b.py = xy + ey;
    b.pz = xz + ez;
    const float mx = b.px + xx, my = b.py + xy, mz = b.pz + xz;  // 2 xi + e
    const float xi2 = fmaf(xx, xx, fmaf(xy, xy, xz * xz));
    const float y2 = fmaf(b.px, b.px, fmaf(b.py, b.py, b.pz * b.pz));
    const float num = fmaf(ex, mx, fmaf(ey, my, ez * mz));  // |p|^2 - |xi|^2
    const float rxi = rsqrtf(xi2);
    b.ry = rsqrtf(y2);
    const float lsum = fmaf(y2, b.ry, xi2 * rxi);  // |p| + |xi|
    b.s = __fdividef(num * rxi, lsum);
    // Error band against the binary64 stretch of the same state:
    //   geometry (fixed-point rounding of xi), displacement rounding to
    //   float, FP32 arithmetic (<= 1e-6 relative), safety factor 2.
    const float einf = fmaxf(fabsf(ex), fmaxf(fabsf(ey), fabsf(ez)));
    const float r = 1.7320508f * einf * rxi;  // >= |e| / |xi|
    const float as = fabsf(b.s);
    const float t2 = fmaf(2.0f, r, as);                          // 2r + |s|
    const float geo = fmaf(c.geo, rxi, 1.1e-7f);                 // |dxi|/|xi|
    const float uterm = 1.1e-7f * (ui.w + uj.w + einf) * rxi;    // float u
    const float arith = 1.0e-6f * fmaf(r, r, t2);                // 2r + r^2 + |s|
    b.band = fmaf(2.0f, fmaf(geo, t2, uterm + arith), 1.0e-12f);
    return b;
}

// Two bonds (i -> a, i -> b) at once in packed FP32x2 arithmetic (.x = a,
// .y = b); the same operations and error band as bond32.
struct Bond32x2 {
    float2 px, py, pz, s, ry, band;
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

__device__ __forceinline__ Bond32x2 bond32x2(const int4& qi, const float4& ui, const int4& qa,
                                             const float4& ua, const int4& qb,
                                             const float4& ub, const MixedConst& c) {
    const float2 H = f2(c.h), MH = f2(c.mh);
    const float2 xx = __ffma2_rn(
        f2(__int_as_float(qa.x - qi.x + kMagicI), __int_as_float(qb.x - qi.x + kMagicI)), H, MH);
    const float2 xy = __ffma2_rn(
        f2(__int_as_float(qa.y - qi.y + kMagicI), __int_as_float(qb.y - qi.y + kMagicI)), H, MH);
    const float2 xz = __ffma2_rn(
        f2(__int_as_float(qa.z - qi.z + kMagicI), __int_as_float(qb.z - qi.z + kMagicI)), H, MH);
    const float2 ex = f2(ua.x - ui.x, ub.x - ui.x);
    const float2 ey = f2(ua.y - ui.y, ub.y - ui.y);
    const float2 ez = f2(ua.z - ui.z, ub.z - ui.z);
    Bond32x2 b;
    b.px = __fadd2_rn(xx, ex);
    b.py = __fadd2_rn(xy, ey);
    b.pz = __fadd2_rn(xz, ez);
    const float2 mx = __fadd2_rn(b.px, xx), my = __fadd2_rn(b.py, xy), mz = __fadd2_rn(b.pz, xz);
    const float2 xi2 = __ffma2_rn(xx, xx, __ffma2_rn(xy, xy, __fmul2_rn(xz, xz)));
    const float2 y2 = __ffma2_rn(b.px, b.px, __ffma2_rn(b.py, b.py, __fmul2_rn(b.pz, b.pz)));
    const float2 num = __ffma2_rn(ex, mx, __ffma2_rn(ey, my, __fmul2_rn(ez, mz)));
    const float2 rxi = f2(rsqrtf(xi2.x), rsqrtf(xi2.y));
    b.ry = f2(rsqrtf(y2.x), rsqrtf(y2.y));
    const float2 lsum = __ffma2_rn(y2, b.ry, __fmul2_rn(xi2, rxi));
    const float2 rl = f2(__fdividef(1.0f, lsum.x), __fdividef(1.0f, lsum.y));
    b.s = __fmul2_rn(__fmul2_rn(num, rxi), rl);
    const float2 einf = f2(fmaxf(fabsf(ex.x), fmaxf(fabsf(ey.x), fabsf(ez.x))),
                           fmaxf(fabsf(ex.y), fmaxf(fabsf(ey.y), fabsf(ez.y))));
    const float2 r = __fmul2_rn(einf, __fmul2_rn(rxi, f2(1.7320508f)));
    const float2 t2 = __ffma2_rn(f2(2.0f), r, f2(fabsf(b.s.x), fabsf(b.s.y)));
    const float2 geo = __ffma2_rn(f2(c.geo), rxi, f2(1.1e-7f));
    const float2 uw = __fadd2_rn(f2(ui.w + ua.w, ui.w + ub.w), einf);
    const float2 uterm = __fmul2_rn(__fmul2_rn(f2(1.1e-7f), uw), rxi);
    const float2 arith = __fmul2_rn(f2(1.0e-6f), __ffma2_rn(r, r, t2));
    b.band = __ffma2_rn(f2(2.0f), __ffma2_rn(geo, t2, __fadd2_rn(uterm, arith)), f2(1.0e-12f));
    return b;
}

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

// Regime logic of bond_force3/4 (peridynamics.cl:345-367) on an exact
// decision function lt(threshold index) = (s < critical_stretch[idx]).
// Returns the new regime (>= nregimes means broken).
template <class Lt>
__device__ __forceinline__ int next_regime(int reg, int base, int nr, Lt&& lt) {
    const int rc = reg < 0 ? 0 : (reg >= nr ? nr - 1 : reg);
    if (lt(base + rc)) {
        if (reg > 0 && rc > 0 && lt(base + rc - 1)) return reg - 1;
        return reg;
    }
    return reg + 1;
}

// Sum (x, y, z, w) over the warp: 6 shuffles.  Lanes 0-7 end with the x
// total, 8-15 y, 16-23 z, 24-31 w.
__device__ __forceinline__ float reduce4(float x, float y, float z, float w, int lane) {
    const bool up16 = lane & 16;
    const float a_keep = up16 ? z : x, a_send = up16 ? x : z;
    const float b_keep = up16 ? w : y, b_send = up16 ? y : w;
    const float a = a_keep + __shfl_xor_sync(kFull, a_send, 16);
    const float b = b_keep + __shfl_xor_sync(kFull, b_send, 16);
    const bool up8 = lane & 8;
    float v = (up8 ? b : a) + __shfl_xor_sync(kFull, up8 ? a : b, 8);
    v += __shfl_xor_sync(kFull, v, 4);
    v += __shfl_xor_sync(kFull, v, 2);
    v += __shfl_xor_sync(kFull, v, 1);
    return v;
}

template <int SL, bool CORR, bool TYPES, int MINB>
__global__ void __launch_bounds__(kWarps * 32, MINB)
    k_mixed(pp_fused_args a, MixedConst c, int parity, Launch l) {
    __shared__ float4 s_frc[kChunk];
    __shared__ float s_thr[TYPES ? kMaxTable : 1];
    __shared__ float s_k[TYPES ? kMaxTable : 1];
    __shared__ float s_c[TYPES ? kMaxTable : 1];
    if constexpr (TYPES) {
        const int nt = a.nbond_types * a.nregimes;
        for (int t = threadIdx.x; t < nt; t += blockDim.x) {
            s_thr[t] = (float)a.critical_stretch_table[t];
            s_k[t] = (float)a.bond_stiffness_table[t];
            s_c[t] = (float)a.plus_cs[t];
        }
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int node0 = blockIdx.x * kChunk;
    const int L = a.max_neigh;
    const int nr = a.nregimes;
    const float* __restrict__ uhi = a.uhi[parity];

    // ------------------------------------------------------- bond phase
    for (int t = 0; t < kChunk / kWarps; ++t) {
        const int li = t * kWarps + warp;
        const int i = node0 + li;
        if (i >= a.nnodes) break;  // warp-uniform
        const int64_t row = (int64_t)i * L;
        const int4 qi = ldg_i4(a.pos_q, i);
        const float4 ui = ldg_f4(uhi, i);
        int jr[SL];
#pragma unroll
        for (int k = 0; k < SL; ++k) {
            const int slot = lane + 32 * k;
            jr[k] = (SL > 1 || slot < L) ? __ldcs(a.nlist + row + slot) : -1;
        }
        int4 qj[SL];
        float4 uj[SL];
        float sc[SL];
        int bt[SL], rg[SL];
#pragma unroll
        for (int k = 0; k < SL; ++k) {
            // An empty slot gets a harmless stand-in (one fixed-point step
            // away, same displacement) so that all arithmetic stays finite.
            if (jr[k] != -1) {
                qj[k] = ldg_i4(a.pos_q, jr[k]);
                uj[k] = ldg_f4(uhi, jr[k]);
            } else {
                qj[k] = make_int4(qi.x + 1, qi.y, qi.z, 0);
                uj[k] = ui;
            }
            const int64_t gid = row + lane + 32 * k;
            if constexpr (CORR) sc[k] = jr[k] != -1 ? __ldcs(a.sc32 + gid) : 0.f;
            if constexpr (TYPES) {
                bt[k] = jr[k] != -1 ? __ldcs(a.bond_types + gid) * nr : 0;
                rg[k] = jr[k] != -1 ? a.regimes[gid] : 0;
            }
        }
        float sx = 0.f, sy = 0.f, sz = 0.f;
        float cnt = 0.f;
        unsigned amb = 0u;
        // Decide one bond from its FP32 stretch; returns the force factor
        // (force = factor * p) or 0.  Ambiguous slots are deferred.
        auto decide = [&](int k, float s, float band, float ry) -> float {
            if (jr[k] == -1) return 0.0f;
            const int64_t gid = row + lane + 32 * k;
            float w = __int_as_float(qj[k].w);  // k*vol (PMB) or vol (types)
            bool intact;
            if constexpr (!TYPES) {
                const float d = s - c.s0;
                if (!(fabsf(d) > band + c.s0_err)) {
                    amb |= 1u << k;
                    return 0.0f;
                }
                intact = d < 0.0f;
                w *= s;
            } else {
                bool ambiguous = false;
                const int reg = next_regime(rg[k], bt[k], nr, [&](int idx) {
                    const float thr = s_thr[idx];
                    const float d = s - thr;
                    if (!(fabsf(d) > band + 6.0e-8f * fabsf(thr))) ambiguous = true;
                    return d < 0.0f;
                });
                if (ambiguous) {
                    amb |= 1u << k;
                    return 0.0f;
                }
                if (reg != rg[k]) a.regimes[gid] = reg;
                intact = reg < nr;
                if (intact) w *= fmaf(s, s_k[bt[k] + reg], s_c[bt[k] + reg]);
            }
            if (!intact) {
                a.nlist[gid] = -1;
                return 0.0f;
            }
            if constexpr (CORR) w *= sc[k];
            cnt += 1.0f;
            return w * ry;
        };
        if constexpr (SL == 1) {
            const Bond32 b = bond32(qi, ui, qj[0], uj[0], c);
            const float fv = decide(0, b.s, b.band, b.ry);
            sx = fv * b.px;
            sy = fv * b.py;
            sz = fv * b.pz;
        } else {
            float2 ax = f2(0.0f), ay = f2(0.0f), az = f2(0.0f);
#pragma unroll
            for (int k = 0; k < SL / 2; ++k) {
                const int kb = k + SL / 2;
                if (jr[k] == -1 && jr[kb] == -1) continue;
                const Bond32x2 b = bond32x2(qi, ui, qj[k], uj[k], qj[kb], uj[kb], c);
                const float2 fv = f2(decide(k, b.s.x, b.band.x, b.ry.x),
                                     decide(kb, b.s.y, b.band.y, b.ry.y));
                ax = __ffma2_rn(fv, b.px, ax);
                ay = __ffma2_rn(fv, b.py, ay);
                az = __ffma2_rn(fv, b.pz, az);
            }
            sx = ax.x + ax.y;
            sy = ay.x + ay.y;
            sz = az.x + az.y;
        }
        // Slow path: slots whose FP32 stretch is too close to a critical
        // stretch are decided on the binary64 stretch.
        if (__any_sync(kFull, amb != 0u)) {
#pragma unroll
            for (int k = 0; k < SL; ++k) {
                if (!((amb >> k) & 1u)) continue;
                const int64_t gid = row + lane + 32 * k;
                const int j = jr[k];
                const Bond32 b = bond32(qi, ui, qj[k], uj[k], c);
                const double s64 = exact_stretch(a, parity, i, j);
                float w = __int_as_float(qj[k].w);
                bool intact;
                if constexpr (!TYPES) {
                    intact = s64 < a.critical_stretch;
                } else {
                    const int reg = next_regime(rg[k], bt[k], nr, [&](int idx) {
                        return s64 < a.critical_stretch_table[idx];
                    });
                    if (reg != rg[k]) a.regimes[gid] = reg;
                    intact = reg < nr;
                    if (intact) w *= fmaf(b.s, s_k[bt[k] + reg], s_c[bt[k] + reg]);
                }
                if (!intact) {
                    a.nlist[gid] = -1;
                    continue;
                }
                float fv = TYPES ? w * b.ry : b.s * w * b.ry;
                if constexpr (CORR) fv *= sc[k];
                sx = fmaf(fv, b.px, sx);
                sy = fmaf(fv, b.py, sy);
                sz = fmaf(fv, b.pz, sz);
                cnt += 1.0f;
            }
        }
        const float v = reduce4(sx, sy, sz, cnt, lane);
        if ((lane & 7) == 0) reinterpret_cast<float*>(&s_frc[li])[lane >> 3] = v;
    }
    __syncthreads();

    // ------------------------------------------------------- node phase
    const int li = threadIdx.x >> 2;
    const int comp = threadIdx.x & 3;
    const int i = node0 + li;
    const bool active = i < a.nnodes;
    const StepMags m = step_mags(l);
    const float4 fr = s_frc[li];
    const int64_t o4 = 4 * (int64_t)i + comp;
    float hi_new = 0.f, lo_new = 0.f;
    if (active && comp < 3) {
        const float body = comp == 0 ? fr.x : (comp == 1 ? fr.y : fr.z);
        const int fl = a.nflags[i];
        const int64_t o3 = 3 * (int64_t)i + comp;
        float frc = body;
        if ((fl >> (3 + comp)) & 1) frc = (float)((double)body + m.force * a.fc_values[o3]);
        df uu{uhi[o4], a.ulo[parity][o4]};
        const df dt{c.dt_hi, c.dt_lo};
        if (a.integrator == PP_EULER) {
            uu = df_add(uu, df_mul_f(dt, frc));
        } else {
            const df half{c.half_hi, c.half_lo};
            const int64_t o8 = 8 * (int64_t)i + comp;
            df v{a.vel[o8], a.vel[o8 + 4]};
            const float rho = a.rho32[o4];
            float acc;
            if (a.integrator == PP_EULER_CROMER) {
                acc = __fdiv_rn(frc - c.damping * v.hi, rho);
                v = df_add(v, df_mul_f(dt, acc));
                uu = df_add(uu, df_mul(dt, v));
            } else {
                const df v1 = df_add(v, df_mul_f(half, a.acc[o4]));
                acc = __fdiv_rn(frc - c.damping * v1.hi, rho);
                v = df_add(v1, df_mul_f(half, acc));
                uu = df_add(uu, df_mul(dt, df_add(v, df_mul_f(half, acc))));
            }
            a.vel[o8] = v.hi;
            a.vel[o8 + 4] = v.lo;
            a.acc[o4] = acc;
        }
        if (fl & (1 << comp)) uu = df_from_double(m.disp * a.bc_values[o3]);
        hi_new = uu.hi;
        lo_new = uu.lo;
        a.frc[8 * (int64_t)i + comp] = frc;
        a.frc[8 * (int64_t)i + 4 + comp] = body;
    }
    // max |u| of the node for the next step's error band (quad shuffle)
    float um = fabsf(hi_new);
    um = fmaxf(um, __shfl_xor_sync(kFull, um, 1));
    um = fmaxf(um, __shfl_xor_sync(kFull, um, 2));
    if (active) {
        if (comp < 3) {
            a.uhi[parity ^ 1][o4] = hi_new;
            a.ulo[parity ^ 1][o4] = lo_new;
        } else {
            a.uhi[parity ^ 1][o4] = um * (1.0f + 1.2e-7f);
            a.ulo[parity ^ 1][o4] = 0.f;
            a.n_neigh[i] = (int)fr.w;
        }
    }
}

MixedConst mixed_const(const pp_fused_args& a) {
    MixedConst c;
    c.h = (float)a.pos_scale;
    c.mh = -kMagicF * c.h;
    c.geo = 1.7320508f * c.h;
    c.s0 = (float)a.critical_stretch;
    c.s0_err = 6.0e-8f * fabsf(c.s0);
    c.dt_hi = (float)a.dt;
    c.dt_lo = (float)(a.dt - (double)c.dt_hi);
    const double half = a.dt / 2;
    c.half_hi = (float)half;
    c.half_lo = (float)(half - (double)c.half_hi);
    c.damping = (float)a.damping;
    return c;
}

template <int SL, bool CORR, bool TYPES>
void launch_variant(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const dim3 grid((a.nnodes + kChunk - 1) / kChunk), block(kWarps * 32);
    // variant 0: register budget for 2 resident CTAs per SM, 1: for 3.
    if (a.variant == 1)
        k_mixed<SL, CORR, TYPES, 3><<<grid, block, 0, st>>>(a, mixed_const(a), parity, l);
    else
        k_mixed<SL, CORR, TYPES, 2><<<grid, block, 0, st>>>(a, mixed_const(a), parity, l);
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
    const double w = a.bond_types ? a.vols[i] : a.bond_stiffness * a.vols[i];
    q.w = __float_as_int((float)w);
    reinterpret_cast<int4*>(a.pos_q)[i] = q;
    const double* u = a.u[parity];
    float umax = 0.f;
    int fl = 0;
    for (int d = 0; d < 3; ++d) {
        const df x = df_from_double(u[o + d]);
        a.uhi[parity][4 * (int64_t)i + d] = x.hi;
        a.ulo[parity][4 * (int64_t)i + d] = x.lo;
        umax = fmaxf(umax, fabsf(x.hi));
        fl |= (a.bc_types[o + d] != 0) << d;
        fl |= (a.fc_types[o + d] != 0) << (3 + d);
    }
    a.nflags[i] = fl;
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

__global__ void k_zero_u64(unsigned long long* p) { *p = 0ull; }

// Warp per node: max |r0[j][d] - r0[i][d]| over the row's bonds.
__global__ void k_bond_extent(const int32_t* __restrict__ nlist, const double* __restrict__ r0,
                              int nnodes, int max_neigh, unsigned long long* out) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= nnodes) return;
    double mx = 0.0;
    for (int k = lane; k < max_neigh; k += 32) {
        const int j = nlist[(int64_t)i * max_neigh + k];
        if (j < 0 || j >= nnodes) continue;
        for (int d = 0; d < 3; ++d)
            mx = fmax(mx, fabs(r0[3 * (int64_t)j + d] - r0[3 * (int64_t)i + d]));
    }
    for (int off = 16; off >= 1; off >>= 1) mx = fmax(mx, __shfl_xor_sync(kFull, mx, off));
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

}  // namespace

int validate_mixed(const pp_fused_args& a) {
    if (!a.pos_q || !a.uhi[0] || !a.uhi[1] || !a.ulo[0] || !a.ulo[1] || !a.frc || !a.nflags)
        return PP_ERROR_INVALID_VALUE;
    if (!aligned16(a.pos_q) || !aligned16(a.uhi[0]) || !aligned16(a.uhi[1]) ||
        !aligned16(a.ulo[0]) || !aligned16(a.ulo[1]) || !aligned16(a.frc))
        return PP_ERROR_MISALIGNED;
    if (a.integrator != PP_EULER && (!a.vel || !a.acc || !a.rho32)) return PP_ERROR_INVALID_VALUE;
    if (a.stiffness_corrections && !a.sc32) return PP_ERROR_INVALID_VALUE;
    if (a.bond_types && a.nbond_types * a.nregimes > kMaxTable) return PP_ERROR_UNSUPPORTED;
    if (!(a.pos_scale > 0.0)) return PP_ERROR_INVALID_VALUE;
    if (a.variant < 0 || a.variant >= PP_MIXED_VARIANTS) return PP_ERROR_INVALID_VALUE;
    return PP_SUCCESS;
}

int launch_mixed_step(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    switch (a.max_neigh > 32 ? a.max_neigh / 32 : 1) {
        case 1: launch_sl<1>(a, parity, l, st); break;
        case 2: launch_sl<2>(a, parity, l, st); break;
        case 4: launch_sl<4>(a, parity, l, st); break;
        case 8: launch_sl<8>(a, parity, l, st); break;
        default: return PP_ERROR_UNSUPPORTED;  // max_neigh > 256
    }
    return launch_status();
}

}  // namespace pp

using namespace pp;

extern "C" int pp_bond_extent(const int32_t* nlist, const double* r0, int32_t nnodes,
                              int32_t max_neigh, double* extent, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (!is_pow2_le_1024(max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (!extent) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* out = reinterpret_cast<unsigned long long*>(extent);
    k_zero_u64<<<1, 1, 0, st>>>(out);
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
    if (!a.r0 || !a.vols || !a.u[parity] || !a.pos_q || !a.uhi[parity] || !a.ulo[parity] ||
        !a.nflags || !a.bc_types || !a.fc_types || !(a.pos_scale > 0.0))
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
