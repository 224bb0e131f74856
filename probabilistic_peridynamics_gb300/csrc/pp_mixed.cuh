// pp_mixed.cuh -- the PP_MIXED fused step kernel (templates), shared by the
// translation units that instantiate its tile shapes (pp_mixed_v*.cu).
//
// FP32 bond arithmetic on 32-byte node records gathered with one 256-bit
// load per bond, the break / regime decision taken exactly as binary64
// would on the same state, and double-float node state.
//
// Structure of one launch (one CTA = W warps, chunks of 16 W consecutive
// nodes, persistent over the chunks):
//
//  1. Bond phase.  Rows of 64 or more slots: four consecutive nodes per
//     warp, eight lanes per node, lane t taking slots t, t + 8, ... four at
//     a time (bond_phase_group); the slot indices of the next batch are
//     loaded while a batch computes, and one gather instruction reaches the
//     first neighbours of four neighbouring nodes, mostly the same L1
//     lines.  Rows of 32 slots or fewer: one warp per node, lane l taking
//     slot l (bond_phase_node).  Each slot costs one 256-bit record gather
//     and the FP32 bond arithmetic; a clearly intact bond is decided by one
//     compare, every other one (breaking, or close to a critical stretch)
//     in a per-node slow path, where the bond's own error band or else the
//     binary64 stretch of peridynamics.cl:65-75, from the reference r0 and
//     the exact double-float displacement, decides.  The four per-node sums
//     (force x, y, z and the intact count) are reduced with a transposed
//     butterfly and parked in shared memory.  No shared-memory staging of
//     the neighbour list, so L1 keeps its full capacity for the records.
//  2. Node phase, all threads: thread (node, component) applies the force
//     boundary condition and the integrator update of one DOF in
//     double-float arithmetic and writes one word of each half of the
//     node's next record; every load and store of the node state is
//     contiguous per CTA.
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
#pragma once


#include "pp_bond_f64.cuh"
#include "pp_fused.cuh"

namespace pp {
namespace mixed {

constexpr int kMaxTable = 256;
constexpr int kNodesPerWarp = 16;  // a CTA of W warps owns chunks of 16*W nodes
constexpr int kLanesPerNode = 8;   // rows of 64+ slots: 32/8 nodes per warp

constexpr int kMagicI = 0x4B400000;  // bit pattern of 1.5 * 2^23
constexpr float kMagicF = 12582912.0f;

struct MixedConst {
    float h;        // fixed-point step (a power of two)
    float mh;       // -kMagicF * h
    float geo;      // sqrt(3) * h: bound on the rounding of each xi
    float rxi_max;  // 1 / (smallest bond length)
    float s0;       // critical stretch (PMB), rounded to float
    float s0_err;   // 6e-8 * |s0|: rounding of s0 to float
    float dt_hi, dt_lo;
    float half_hi, half_lo;
    float damping;
};

// FP32 quantities of one bond (i -> j).
struct Bond32 {
    float px, py, pz;  // deformed bond vector
    float s;           // stretch
    float ry;          // 1 / |p|
    float rxi;         // 1 / |xi|
};

// One node record {q, w; u, m} (32 bytes, 32-byte aligned) in one 256-bit
// read-only load: a step never writes the records it reads.
struct Rec {
    int4 q;
    float4 u;
};

__device__ __forceinline__ Rec load_rec(const float* rec, int64_t i) {
    float v[8];
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
          "=f"(v[7])
        : "l"(rec + 8 * i));
    Rec r;
    r.q = make_int4(__float_as_int(v[0]), __float_as_int(v[1]), __float_as_int(v[2]),
                    __float_as_int(v[3]));
    r.u = make_float4(v[4], v[5], v[6], v[7]);
    return r;
}

// Neighbour-list word that the step reads once and may overwrite (-1 on a
// break) later in the same thread: a coherent load that does not allocate
// in L1, which is kept for the node records.
__device__ __forceinline__ int load_slot(const int32_t* p) {
    int v;
    asm volatile("ld.global.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ float fixed_diff(int qj, int qi, const MixedConst& c) {
    return fmaf(__int_as_float(qj - qi + kMagicI), c.h, c.mh);
}

// FP32 quantities of a bond from its exact reference vector xi = (xx, xy,
// xz) and the displacement halves of both ends.
__device__ __forceinline__ Bond32 bond32_xi(float xx, float xy, float xz, const float4& ui,
                                            const float4& uj) {
    const float ex = uj.x - ui.x, ey = uj.y - ui.y, ez = uj.z - ui.z;
    Bond32 b;
    b.px = xx + ex;
    b.py = xy + ey;
    b.pz = xz + ez;
    const float mx = b.px + xx, my = b.py + xy, mz = b.pz + xz;  // 2 xi + e
    const float xi2 = fmaf(xx, xx, fmaf(xy, xy, xz * xz));
    const float y2 = fmaf(b.px, b.px, fmaf(b.py, b.py, b.pz * b.pz));
    const float num = fmaf(ex, mx, fmaf(ey, my, ez * mz));  // |p|^2 - |xi|^2
    b.rxi = rsqrtf(xi2);
    b.ry = rsqrtf(y2);
    const float lsum = fmaf(y2, b.ry, xi2 * b.rxi);  // |p| + |xi|
    // s = (|p| - |xi|)/|xi| without cancellation: (2 xi.e + e.e)/(|xi|(|p|+|xi|))
    b.s = __fdividef(num * b.rxi, lsum);
    return b;
}

// bond32_xi of two bonds (a, b) of node i at once, on the paired FP32
// instructions of sm_100 and later (__fadd2_rn, __fmul2_rn, __ffma2_rn: per
// component the same IEEE round-to-nearest operation as the scalar one).
// Every component goes through the operations of bond32_xi in the same order,
// so half h is bit for bit bond32_xi of bond h; the approximate rsqrt and
// division stay scalar calls of the same intrinsics.
struct Bond32x2 {
    float2 px, py, pz, s, ry, rxi;
    __device__ __forceinline__ Bond32 half(int h) const {
        Bond32 b;
        b.px = h ? px.y : px.x;
        b.py = h ? py.y : py.x;
        b.pz = h ? pz.y : pz.x;
        b.s = h ? s.y : s.x;
        b.ry = h ? ry.y : ry.x;
        b.rxi = h ? rxi.y : rxi.x;
        return b;
    }
};

__device__ __forceinline__ Bond32x2 bond32_xi2(float2 xx, float2 xy, float2 xz, const float4& ui,
                                               const float4& uja, const float4& ujb) {
    const float2 ex = make_float2(uja.x - ui.x, ujb.x - ui.x);
    const float2 ey = make_float2(uja.y - ui.y, ujb.y - ui.y);
    const float2 ez = make_float2(uja.z - ui.z, ujb.z - ui.z);
    Bond32x2 b;
    b.px = __fadd2_rn(xx, ex);
    b.py = __fadd2_rn(xy, ey);
    b.pz = __fadd2_rn(xz, ez);
    const float2 mx = __fadd2_rn(b.px, xx), my = __fadd2_rn(b.py, xy), mz = __fadd2_rn(b.pz, xz);
    const float2 xi2 = __ffma2_rn(xx, xx, __ffma2_rn(xy, xy, __fmul2_rn(xz, xz)));
    const float2 y2 = __ffma2_rn(b.px, b.px, __ffma2_rn(b.py, b.py, __fmul2_rn(b.pz, b.pz)));
    const float2 num = __ffma2_rn(ex, mx, __ffma2_rn(ey, my, __fmul2_rn(ez, mz)));
    b.rxi = make_float2(rsqrtf(xi2.x), rsqrtf(xi2.y));
    b.ry = make_float2(rsqrtf(y2.x), rsqrtf(y2.y));
    const float2 lsum = __ffma2_rn(y2, b.ry, __fmul2_rn(xi2, b.rxi));
    const float2 t = __fmul2_rn(num, b.rxi);
    b.s = make_float2(__fdividef(t.x, lsum.x), __fdividef(t.y, lsum.y));
    return b;
}

// The same from the fixed-point positions: xi = h (q_j - q_i), exact.
__device__ __forceinline__ Bond32 bond32(const int4& qi, const float4& ui, const int4& qj,
                                         const float4& uj, const MixedConst& c) {
    return bond32_xi(fixed_diff(qj.x, qi.x, c), fixed_diff(qj.y, qi.y, c),
                     fixed_diff(qj.z, qi.z, c), ui, uj);
}

// Bound on |s - s64| for one bond: s64 is the binary64 stretch of the same
// state (reference formula).  Terms: geometry (fixed-point rounding of xi,
// <= sqrt(3) h per bond vector), the rounding of the displacement to float
// (<= 2^-24 |u| per component), FP32 arithmetic (<= 1e-6 relative, which
// covers the approximate rsqrt and division), times a safety factor 2.
__device__ __forceinline__ float band32(const float4& ui, const float4& uj, const Bond32& b,
                                        const MixedConst& c) {
    const float einf =
        fmaxf(fabsf(uj.x - ui.x), fmaxf(fabsf(uj.y - ui.y), fabsf(uj.z - ui.z)));
    const float r = 1.7320508f * einf * b.rxi;  // >= |e| / |xi|
    const float t2 = fmaf(2.0f, r, fabsf(b.s));
    const float geo = fmaf(c.geo, b.rxi, 1.1e-7f);
    const float uterm = 1.1e-7f * (ui.w + uj.w + einf) * b.rxi;
    const float arith = 1.0e-6f * fmaf(r, r, t2);
    return fmaf(2.0f, fmaf(geo, t2, uterm + arith), 1.0e-12f);
}

// A bound of band32 valid for every bond of the step, affine in |s|:
// band32 <= quick_a + quick_c * |s|, from the running max |u| (U) and the
// shortest bond.  Decides almost every bond with three instructions.
struct QuickBand {
    float a, c;
};

__device__ __forceinline__ QuickBand quick_band(float U, const MixedConst& c) {
    const float geo = fmaf(c.geo, c.rxi_max, 1.1e-7f);
    const float R = 3.5f * U * c.rxi_max;  // >= sqrt(3) * (|u_i| + |u_j|)(1 + eps) / |xi|
    QuickBand q;
    q.a = 2.0f * (geo * 2.0f * R + 1.1e-7f * 4.1f * U * c.rxi_max +
                  1.0e-6f * fmaf(R, R, 2.0f * R)) +
          1.0e-12f;
    q.c = 2.0f * (geo + 1.0e-6f);
    return q;
}

// Binary64 stretch of bond (i, j) from the reference r0 and the exact
// double-float displacement, in the reference operation order
// (peridynamics.cl:65-75).
static __device__ __noinline__ double exact_stretch(const pp_fused_args& a, int parity, int i, int j) {
    // the displacement halves of the records (16-byte loads: ptxas 13.0
    // fails on a 256-bit load inside a non-inlined function)
    const float4 hi_i = ldg_f4(a.rec[parity], 2 * (int64_t)i + 1), lo_i = ldg_f4(a.ulo[parity], i);
    const float4 hi_j = ldg_f4(a.rec[parity], 2 * (int64_t)j + 1), lo_j = ldg_f4(a.ulo[parity], j);
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

// Regime logic of bond_force3/4 (peridynamics.cl:345-367) on a decision
// function lt(threshold index) = (s < critical_stretch[idx]).
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

// Compensated accumulation s + c += a * b: the rounding error of the
// product (FMA) and of the sum (TwoSum, Knuth) go to the carry c.
template <bool COMP>
__device__ __forceinline__ void acc_mul(float& s, float& c, float a, float b) {
    if constexpr (COMP) {
        const float t = __fmul_rn(a, b);
        const float pe = fmaf(a, b, -t);
        const float ns = __fadd_rn(s, t);
        const float bp = __fsub_rn(ns, s);
        const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(ns, bp)), __fsub_rn(t, bp));
        c = __fadd_rn(c, __fadd_rn(e, pe));
        s = ns;
    } else {
        s = fmaf(a, b, s);
    }
}

// (v, c) += (w, d) with the rounding error of v + w added to the carry.
__device__ __forceinline__ void two_sum_into(float& v, float& c, float w, float d) {
    const float ns = __fadd_rn(v, w);
    const float bp = __fsub_rn(ns, v);
    const float e = __fadd_rn(__fsub_rn(v, __fsub_rn(ns, bp)), __fsub_rn(w, bp));
    c = __fadd_rn(c, __fadd_rn(d, e));
    v = ns;
}

// reduce4 on compensated pairs (x + cx, ...): the same lane layout, the
// result rounded once at the end.
__device__ __forceinline__ float reduce4c(float x, float cx, float y, float cy, float z,
                                          float cz, float w, int lane) {
    const bool up16 = lane & 16;
    float a = up16 ? z : x, ac = up16 ? cz : cx;
    float b = up16 ? w : y, bc = up16 ? 0.f : cy;
    const float as = up16 ? x : z, asc = up16 ? cx : cz;
    const float bs = up16 ? y : w, bsc = up16 ? cy : 0.f;
    two_sum_into(a, ac, __shfl_xor_sync(kFull, as, 16), __shfl_xor_sync(kFull, asc, 16));
    two_sum_into(b, bc, __shfl_xor_sync(kFull, bs, 16), __shfl_xor_sync(kFull, bsc, 16));
    const bool up8 = lane & 8;
    float v = up8 ? b : a, vc = up8 ? bc : ac;
    two_sum_into(v, vc, __shfl_xor_sync(kFull, up8 ? a : b, 8),
                 __shfl_xor_sync(kFull, up8 ? ac : bc, 8));
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1)
        two_sum_into(v, vc, __shfl_xor_sync(kFull, v, off), __shfl_xor_sync(kFull, vc, off));
    return __fadd_rn(v, vc);
}

template <int CH>
struct alignas(16) MixedShared {
    float4 frc[CH];
    float thr[kMaxTable], k[kMaxTable], c[kMaxTable];  // regime tables or
                                                        // instance thresholds
    float tlo[kMaxTable], thi[kMaxTable];              // Thresholds of thr[]
};

// Stretch thresholds that decide a bond against critical stretch s0 without
// its own band: s < lo is intact and s > hi broken for every bond of the
// step, from |s - s0| > quick.a + quick.c |s| + s0err solved for s (both
// signs of s), widened by 5e-7 relative to cover their own rounding.
struct Thresholds {
    float lo, hi;
};

__device__ __forceinline__ Thresholds thresholds(float s0f, float s0err, const QuickBand& q) {
    const float x = s0f - q.a - s0err;  // s < s0 side
    const float y = s0f + q.a + s0err;  // s > s0 side
    float lo = x >= 0.0f ? x / (1.0f + q.c) : x / (1.0f - q.c);
    float hi = y > 0.0f ? y / (1.0f - q.c) : y / (1.0f + q.c);
    lo -= fmaf(fabsf(lo), 5.0e-7f, 1.0e-30f);
    hi += fmaf(fabsf(hi), 5.0e-7f, 1.0e-30f);
    return {lo, hi};
}

// Bond phase of one node (one warp): returns nothing, parks the reduced
// (force x, y, z, intact count) of local node li in sh.frc[li].  COMP:
// compensated force sums (acc_mul, reduce4c).
//
// A broken or padding slot (-1) gathers node i itself instead of branching
// around the loads: its bond vector is exactly 0, so its (discarded, weight
// 0) contribution stays finite.
template <int SL, bool CORR, bool TYPES, bool COMP, class Shared>
__device__ __forceinline__ void bond_phase_node(const pp_fused_args& a, const MixedConst& c,
                                                const QuickBand& qb, const Thresholds& th0,
                                                Shared& sh, const int (&jr)[SL], int parity,
                                                int i, int li, int lane) {
    const int L = a.max_neigh;
    const int nr = a.nregimes;
    const int64_t row = (int64_t)i * L;
    const float* __restrict__ rec = a.rec[parity];
    const Rec ri = load_rec(rec, i);
    const int4 qi = ri.q;
    const float4 ui = ri.u;
    // critical stretch of this node (per instance when batched)
    float s0f = c.s0, s0err = c.s0_err;
    double s0d = a.critical_stretch;
    Thresholds th = th0;
    if (!TYPES && a.node_instance) {
        const int inst = a.node_instance[i];
        s0f = sh.thr[inst];
        s0err = 6.0e-8f * fabsf(s0f);
        s0d = a.instance_s0[inst];
        th.lo = sh.tlo[inst];
        th.hi = sh.thi[inst];
    }
    // this lane's slots: lane + 32 k (consecutive lanes gather consecutive
    // neighbours of the row)
    const int64_t g0 = row + lane;
    int32_t* const nl_g = a.nlist + g0;
    int4 qj[SL];
    float4 uj[SL];
    float sc[SL];
    int bt[SL], rg[SL];
#pragma unroll
    for (int k = 0; k < SL; ++k) {
        if constexpr (CORR) sc[k] = (SL > 1 || lane < L) ? __ldcs(a.sc32 + g0 + 32 * k) : 0.f;
        if constexpr (TYPES) {
            bt[k] = jr[k] != -1 ? __ldcs(a.bond_types + g0 + 32 * k) * nr : 0;
            rg[k] = jr[k] != -1 ? a.regimes[g0 + 32 * k] : 0;
        }
    }
#pragma unroll
    for (int k = 0; k < SL; ++k) {
        const Rec rj = load_rec(rec, jr[k] < 0 ? i : jr[k]);
        qj[k] = rj.q;
        uj[k] = rj.u;
    }
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float cx = 0.f, cy = 0.f, cz = 0.f;  // carries (COMP)
    float cnt = 0.f;
    unsigned amb = 0u;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
        const bool valid = jr[k] != -1;
        const Bond32 b = bond32(qi, ui, qj[k], uj[k], c);
        float w = __int_as_float(qj[k].w);  // k*vol (PMB) or vol (types)
        bool intact;
        if constexpr (!TYPES) {
            // clearly intact below th.lo; every other bond (clearly broken
            // above th.hi, or between: own band, then binary64) is decided
            // in the slow path below, where breaks are written
            intact = valid && b.s < th.lo;
            if (valid && !intact) amb |= 1u << k;
            w *= b.s;
        } else {
            if (!valid) continue;
            bool ambiguous = false;
            const int reg = next_regime(rg[k], bt[k], nr, [&](int idx) {
                if (b.s < sh.tlo[idx]) return true;
                if (b.s > sh.thi[idx]) return false;
                const float thr = sh.thr[idx];
                const float d = b.s - thr;
                if (!(fabsf(d) > band32(ui, uj[k], b, c) + 6.0e-8f * fabsf(thr)))
                    ambiguous = true;
                return d < 0.0f;
            });
            if (ambiguous) {
                amb |= 1u << k;
                continue;
            }
            if (reg != rg[k]) a.regimes[g0 + 32 * k] = reg;
            intact = reg < nr;
            if (!intact) {
                nl_g[32 * k] = -1;
                continue;
            }
            w *= fmaf(b.s, sh.k[bt[k] + reg], sh.c[bt[k] + reg]);
        }
        float fv = intact ? w * b.ry : 0.0f;
        if constexpr (CORR) fv *= sc[k];
        acc_mul<COMP>(sx, cx, fv, b.px);
        acc_mul<COMP>(sy, cy, fv, b.py);
        acc_mul<COMP>(sz, cz, fv, b.pz);
        cnt += intact ? 1.0f : 0.0f;
    }
    // Slow path: slots that break, or whose FP32 stretch is too close to a
    // critical stretch (decided on the binary64 stretch).
    if (__any_sync(kFull, amb != 0u)) {
#pragma unroll
        for (int k = 0; k < SL; ++k) {
            if (!((amb >> k) & 1u)) continue;
            // gathered again: keeping the first loop's records live until
            // here would cost the common path their registers
            const Rec rj = load_rec(rec, jr[k]);
            const Bond32 b = bond32(qi, ui, rj.q, rj.u, c);
            float w = __int_as_float(rj.q.w);
            bool intact;
            if constexpr (!TYPES) {
                // clearly broken, or the bond's own error band decides;
                // else binary64
                const float d = b.s - s0f;
                if (b.s > th.hi)
                    intact = false;
                else if (fabsf(d) > band32(ui, rj.u, b, c) + s0err)
                    intact = d < 0.0f;
                else
                    intact = exact_stretch(a, parity, i, jr[k]) < s0d;
                w *= b.s;
            } else {
                const double s64 = exact_stretch(a, parity, i, jr[k]);
                const int reg = next_regime(rg[k], bt[k], nr, [&](int idx) {
                    return s64 < a.critical_stretch_table[idx];
                });
                if (reg != rg[k]) a.regimes[g0 + 32 * k] = reg;
                intact = reg < nr;
                if (intact) w *= fmaf(b.s, sh.k[bt[k] + reg], sh.c[bt[k] + reg]);
            }
            if (!intact) {
                nl_g[32 * k] = -1;
                continue;
            }
            float fv = w * b.ry;
            if constexpr (CORR) fv *= sc[k];
            acc_mul<COMP>(sx, cx, fv, b.px);
            acc_mul<COMP>(sy, cy, fv, b.py);
            acc_mul<COMP>(sz, cz, fv, b.pz);
            cnt += 1.0f;
        }
    }
    float v;
    if constexpr (COMP)
        v = reduce4c(sx, cx, sy, cy, sz, cz, cnt, lane);
    else
        v = reduce4(sx, sy, sz, cnt, lane);
    if ((lane & 7) == 0) reinterpret_cast<float*>(&sh.frc[li])[lane >> 3] = v;
}

// Sum (x, y, z, w) over each group of 8 lanes (lanes 8g .. 8g + 7): 4
// shuffles.  Lanes 8g + 2c and 8g + 2c + 1 end with channel c (x, y, z, w).
__device__ __forceinline__ float reduce4_8(float x, float y, float z, float w, int lane) {
    const bool b2 = lane & 4;
    const float a_keep = b2 ? z : x, a_send = b2 ? x : z;
    const float b_keep = b2 ? w : y, b_send = b2 ? y : w;
    const float p = a_keep + __shfl_xor_sync(kFull, a_send, 4);
    const float q = b_keep + __shfl_xor_sync(kFull, b_send, 4);
    const bool b1 = lane & 2;
    float v = (b1 ? q : p) + __shfl_xor_sync(kFull, b1 ? p : q, 2);
    v += __shfl_xor_sync(kFull, v, 1);
    return v;
}

// reduce4_8 on compensated pairs, rounded once at the end.
__device__ __forceinline__ float reduce4c_8(float x, float cx, float y, float cy, float z,
                                            float cz, float w, int lane) {
    const bool b2 = lane & 4;
    float p = b2 ? z : x, pc = b2 ? cz : cx;
    float q = b2 ? w : y, qc = b2 ? 0.f : cy;
    const float ps = b2 ? x : z, psc = b2 ? cx : cz;
    const float qs = b2 ? y : w, qsc = b2 ? cy : 0.f;
    two_sum_into(p, pc, __shfl_xor_sync(kFull, ps, 4), __shfl_xor_sync(kFull, psc, 4));
    two_sum_into(q, qc, __shfl_xor_sync(kFull, qs, 4), __shfl_xor_sync(kFull, qsc, 4));
    const bool b1 = lane & 2;
    float v = b1 ? q : p, vc = b1 ? qc : pc;
    two_sum_into(v, vc, __shfl_xor_sync(kFull, b1 ? p : q, 2),
                 __shfl_xor_sync(kFull, b1 ? pc : qc, 2));
    two_sum_into(v, vc, __shfl_xor_sync(kFull, v, 1), __shfl_xor_sync(kFull, vc, 1));
    return __fadd_rn(v, vc);
}

// Sum (x, y, z, w) over each group of LPN lanes (8 or 16): channel c ends
// in lanes 2c and 2c + 1 of the group (reduce4_8 after one more stage).
template <int LPN>
__device__ __forceinline__ float reduce4_group(float x, float y, float z, float w, int lane) {
    if constexpr (LPN == 16) {
        x += __shfl_xor_sync(kFull, x, 8);
        y += __shfl_xor_sync(kFull, y, 8);
        z += __shfl_xor_sync(kFull, z, 8);
        w += __shfl_xor_sync(kFull, w, 8);
    }
    return reduce4_8(x, y, z, w, lane);
}

template <int LPN>
__device__ __forceinline__ float reduce4c_group(float x, float cx, float y, float cy, float z,
                                                float cz, float w, int lane) {
    if constexpr (LPN == 16) {
        two_sum_into(x, cx, __shfl_xor_sync(kFull, x, 8), __shfl_xor_sync(kFull, cx, 8));
        two_sum_into(y, cy, __shfl_xor_sync(kFull, y, 8), __shfl_xor_sync(kFull, cy, 8));
        two_sum_into(z, cz, __shfl_xor_sync(kFull, z, 8), __shfl_xor_sync(kFull, cz, 8));
        w += __shfl_xor_sync(kFull, w, 8);
    }
    return reduce4c_8(x, cx, y, cy, z, cz, w, lane);
}

// Bond phase of four nodes per warp, eight lanes each (rows of 64 or more
// slots).  The group of lanes 8g .. 8g + 7 works on node i (local li) and
// lane 8g + t takes slots t, t + 8, ..., SPL of them, G at a time.  The
// warp's four nodes are consecutive, so one gather instruction reaches the
// first neighbours of four neighbouring nodes: mostly the same L1 lines.
// i >= nnodes: no node; the lanes only join the warp's shuffles.
//
// jn holds the first G slot indices of this lane (loaded ahead); each batch
// loads the next batch's indices before its own arithmetic, and the last
// one loads the first batch of node i_next.
template <int LPN, int SPL, int G, bool CORR, bool TYPES, bool COMP, class Shared>
__device__ __forceinline__ void bond_phase_group(const pp_fused_args& a, const MixedConst& c,
                                                 const Thresholds& th0, Shared& sh, int parity,
                                                 int i, int li, int lane, int (&jn)[G],
                                                 int i_next) {
    const int sub = lane & (LPN - 1);
    const bool node_ok = i < a.nnodes;
    const int ie = node_ok ? i : 0;
    const int L = a.max_neigh;
    const int nr = a.nregimes;
    const float* __restrict__ rec = a.rec[parity];
    const Rec ri = load_rec(rec, ie);
    const int4 qi = ri.q;
    const float4 ui = ri.u;
    // critical stretch of this node (per instance when batched)
    float s0f = c.s0, s0err = c.s0_err;
    double s0d = a.critical_stretch;
    Thresholds th = th0;
    if (!TYPES && a.node_instance) {
        const int inst = a.node_instance[ie];
        s0f = sh.thr[inst];
        s0err = 6.0e-8f * fabsf(s0f);
        s0d = a.instance_s0[inst];
        th.lo = sh.tlo[inst];
        th.hi = sh.thi[inst];
    }
    const int64_t g0 = (int64_t)ie * L + sub;
    int32_t* const nl_g = a.nlist + g0;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float cx = 0.f, cy = 0.f, cz = 0.f;  // carries (COMP)
    float cnt = 0.f;
    unsigned amb = 0u;
#pragma unroll
    for (int k0 = 0; k0 < SPL; k0 += G) {
        int jr[G];
        float sc[G];
        int bt[G], rg[G];
#pragma unroll
        for (int kk = 0; kk < G; ++kk) jr[kk] = jn[kk];
        if (k0 + G < SPL) {
#pragma unroll
            for (int kk = 0; kk < G; ++kk)
                jn[kk] = node_ok ? load_slot(nl_g + LPN * (k0 + G + kk)) : -1;
        } else {
            const int64_t gn = (int64_t)i_next * L + sub;
#pragma unroll
            for (int kk = 0; kk < G; ++kk)
                jn[kk] = i_next < a.nnodes ? load_slot(a.nlist + gn + LPN * kk) : -1;
        }
#pragma unroll
        for (int kk = 0; kk < G; ++kk) {
            const int k = k0 + kk;
            if constexpr (CORR) sc[kk] = node_ok ? __ldcs(a.sc32 + g0 + LPN * k) : 0.f;
            if constexpr (TYPES) {
                bt[kk] = jr[kk] != -1 ? __ldcs(a.bond_types + g0 + LPN * k) * nr : 0;
                rg[kk] = jr[kk] != -1 ? a.regimes[g0 + LPN * k] : 0;
            }
        }
        int4 qj[G];
        float4 uj[G];
#pragma unroll
        for (int kk = 0; kk < G; ++kk) {
            const Rec rj = load_rec(rec, jr[kk] < 0 ? ie : jr[kk]);
            qj[kk] = rj.q;
            uj[kk] = rj.u;
        }
#pragma unroll
        for (int kk = 0; kk < G; ++kk) {
            const int k = k0 + kk;
            const bool valid = jr[kk] != -1;
            const Bond32 b = bond32(qi, ui, qj[kk], uj[kk], c);
            float w = __int_as_float(qj[kk].w);  // k*vol (PMB) or vol (types)
            bool intact;
            if constexpr (!TYPES) {
                // clearly intact below th.lo; every other bond is decided in
                // the slow path below, where breaks are written
                intact = valid && b.s < th.lo;
                if (valid && !intact) amb |= 1u << k;
                w *= b.s;
            } else {
                if (!valid) continue;
                bool ambiguous = false;
                const int reg = next_regime(rg[kk], bt[kk], nr, [&](int idx) {
                    if (b.s < sh.tlo[idx]) return true;
                    if (b.s > sh.thi[idx]) return false;
                    const float thr = sh.thr[idx];
                    const float d = b.s - thr;
                    if (!(fabsf(d) > band32(ui, uj[kk], b, c) + 6.0e-8f * fabsf(thr)))
                        ambiguous = true;
                    return d < 0.0f;
                });
                if (ambiguous) {
                    amb |= 1u << k;
                    continue;
                }
                if (reg != rg[kk]) a.regimes[g0 + LPN * k] = reg;
                intact = reg < nr;
                if (!intact) {
                    nl_g[LPN * k] = -1;
                    continue;
                }
                w *= fmaf(b.s, sh.k[bt[kk] + reg], sh.c[bt[kk] + reg]);
            }
            float fv = intact ? w * b.ry : 0.0f;
            if constexpr (CORR) fv *= sc[kk];
            acc_mul<COMP>(sx, cx, fv, b.px);
            acc_mul<COMP>(sy, cy, fv, b.py);
            acc_mul<COMP>(sz, cz, fv, b.pz);
            cnt += intact ? 1.0f : 0.0f;
        }
    }
    // Slow path: slots that break, or whose FP32 stretch is too close to a
    // critical stretch.  Their indices, records and tables are read again
    // (the hot loop keeps nothing for them; no slot was written yet).
    if (__any_sync(kFull, amb != 0u)) {
#pragma unroll 1
        for (int k = 0; k < SPL; ++k) {
            if (!((amb >> k) & 1u)) continue;
            const int j = load_slot(nl_g + LPN * k);
            const Rec rj = load_rec(rec, j);
            const Bond32 b = bond32(qi, ui, rj.q, rj.u, c);
            float w = __int_as_float(rj.q.w);
            bool intact;
            if constexpr (!TYPES) {
                // clearly broken, or the bond's own error band decides;
                // else binary64
                const float d = b.s - s0f;
                if (b.s > th.hi)
                    intact = false;
                else if (fabsf(d) > band32(ui, rj.u, b, c) + s0err)
                    intact = d < 0.0f;
                else
                    intact = exact_stretch(a, parity, i, j) < s0d;
                w *= b.s;
            } else {
                const double s64 = exact_stretch(a, parity, i, j);
                const int btk = __ldcs(a.bond_types + g0 + LPN * k) * nr;
                const int rgk = a.regimes[g0 + LPN * k];
                const int reg = next_regime(rgk, btk, nr, [&](int idx) {
                    return s64 < a.critical_stretch_table[idx];
                });
                if (reg != rgk) a.regimes[g0 + LPN * k] = reg;
                intact = reg < nr;
                if (intact) w *= fmaf(b.s, sh.k[btk + reg], sh.c[btk + reg]);
            }
            if (!intact) {
                nl_g[LPN * k] = -1;
                continue;
            }
            float fv = w * b.ry;
            if constexpr (CORR) fv *= __ldcs(a.sc32 + g0 + LPN * k);
            acc_mul<COMP>(sx, cx, fv, b.px);
            acc_mul<COMP>(sy, cy, fv, b.py);
            acc_mul<COMP>(sz, cz, fv, b.pz);
            cnt += 1.0f;
        }
    }
    float v;
    if constexpr (COMP)
        v = reduce4c_group<LPN>(sx, cx, sy, cy, sz, cz, cnt, lane);
    else
        v = reduce4_group<LPN>(sx, sy, sz, cnt, lane);
    if (node_ok && sub < 8 && (sub & 1) == 0)
        reinterpret_cast<float*>(&sh.frc[li])[sub >> 1] = v;
}

// The step's inputs of DOF `comp` of node i, read from the global arrays
// (each only where node_update needs it).
struct GlobalDof {
    const pp_fused_args& a;
    int parity;
    int64_t i;
    int comp;
    __device__ __forceinline__ int flags() const { return a.nflags[i]; }
    __device__ __forceinline__ float u_hi() const { return a.rec[parity][8 * i + 4 + comp]; }
    __device__ __forceinline__ float u_lo() const { return a.ulo[parity][4 * i + comp]; }
    __device__ __forceinline__ float v_hi() const { return a.vel[8 * i + comp]; }
    __device__ __forceinline__ float v_lo() const { return a.vel[8 * i + 4 + comp]; }
    __device__ __forceinline__ float rinv() const { return a.rho32[4 * i + comp]; }
    __device__ __forceinline__ float acc() const { return a.acc[4 * i + comp]; }
    // record word `comp` (position or weight), copied to the next record
    __device__ __forceinline__ float qword() const { return a.rec[parity][8 * i + comp]; }
};

// Update of DOF `comp` of node i (comp 3: the record's fourth word) from its
// force component `fc` (comp 3: the intact-bond count) and the inputs that
// `in` reads (GlobalDof or a staged copy).  The four components of a node
// sit on lanes S apart (xor shuffles by S and 2S); lanes with `active` false
// only join the warp's shuffles.  Returns the node's max |u| for the running
// maximum (0 on inactive lanes).
template <int S, class In>
__device__ __forceinline__ float node_update(const pp_fused_args& a, const MixedConst& c,
                                             const StepMags& m, int parity, int i, int comp,
                                             bool active, float fc, const In& in) {
    const int64_t o4 = 4 * (int64_t)i + comp;
    const int64_t o3 = 3 * (int64_t)i + comp;
    const int fl = active ? in.flags() : 0;
    const bool dof = active && comp < 3;
    // Boundary conditions are binary64 (slow on GB300's FP64 pipe): taken
    // only by warps that hold a boundary DOF.
    const bool fbc = dof && ((fl >> (3 + comp)) & 1);
    const bool dbc = dof && ((fl >> comp) & 1);
    const bool any_fbc = __any_sync(kFull, fbc);
    const bool any_dbc = __any_sync(kFull, dbc);
    float hi_new = 0.f, lo_new = 0.f;
    if (dof) {
        const float body = fc;
        float frc = body;
        if (any_fbc && fbc) frc = (float)((double)body + m.force * a.fc_values[o3]);
        df uu{in.u_hi(), in.u_lo()};
        const df dt{c.dt_hi, c.dt_lo};
        if (a.integrator == PP_EULER) {
            uu = df_add(uu, df_mul_f(dt, frc));
        } else {
            const df half{c.half_hi, c.half_lo};
            const int64_t o8 = 8 * (int64_t)i + comp;
            df v{in.v_hi(), in.v_lo()};
            const float rinv = in.rinv();  // 1 / density
            float acc;
            if (a.integrator == PP_EULER_CROMER) {
                acc = (frc - c.damping * v.hi) * rinv;
                v = df_add(v, df_mul_f(dt, acc));
                uu = df_add(uu, df_mul(dt, v));
            } else {
                const df v1 = df_add(v, df_mul_f(half, in.acc()));
                acc = (frc - c.damping * v1.hi) * rinv;
                v = df_add(v1, df_mul_f(half, acc));
                uu = df_add(uu, df_mul(dt, df_add(v, df_mul_f(half, acc))));
            }
            a.vel[o8] = v.hi;
            a.vel[o8 + 4] = v.lo;
            a.acc[o4] = acc;
        }
        if (any_dbc && dbc) uu = df_from_double(m.disp * a.bc_values[o3]);
        hi_new = uu.hi;
        lo_new = uu.lo;
        a.frc[8 * (int64_t)i + comp] = frc;
        a.frc[8 * (int64_t)i + 4 + comp] = body;
    }
    // max |u| of the node (shuffles within its four lanes) for the next
    // step's error bounds
    float um = fabsf(hi_new);
    um = fmaxf(um, __shfl_xor_sync(kFull, um, S));
    um = fmaxf(um, __shfl_xor_sync(kFull, um, 2 * S));
    um *= 1.0f + 1.2e-7f;
    if (active) {
        // the whole record: position word comp, displacement word 4 + comp
        const int64_t o8 = 8 * (int64_t)i + comp;
        a.rec[parity ^ 1][o8] = in.qword();
        if (comp < 3) {
            a.rec[parity ^ 1][o8 + 4] = hi_new;
            a.ulo[parity ^ 1][o4] = lo_new;
        } else {
            a.rec[parity ^ 1][o8 + 4] = um;
            a.ulo[parity ^ 1][o4] = 0.f;
            a.n_neigh[i] = (int)fc;
        }
    }
    return active ? um : 0.f;
}

// Raise the running max |u| of the model to the warp's largest `um`
// (non-negative floats order as ints).
__device__ __forceinline__ void raise_umax(const pp_fused_args& a, float um) {
    const int wmax = __reduce_max_sync(kFull, __float_as_int(um));
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(reinterpret_cast<int*>(a.umax), wmax);
}

// Node phase of one chunk: thread (node, component) updates one DOF of
// node node0 + li; nodes at iend and beyond only join the warp's shuffles.
// Returns the node's max |u| (0 beyond iend).
template <class Shared>
__device__ __forceinline__ float node_phase(const pp_fused_args& a, const MixedConst& c,
                                            const Shared& sh, const StepMags& m, int parity,
                                            int node0, int li, int iend) {
    const int comp = threadIdx.x & 3;
    const int i = node0 + li;
    const float4 fr = sh.frc[li];
    const float fc = comp == 0 ? fr.x : (comp == 1 ? fr.y : (comp == 2 ? fr.z : fr.w));
    return node_update<1>(a, c, m, parity, i, comp, i < iend, fc, GlobalDof{a, parity, i, comp});
}

// One CTA of W warps loops over chunks of 16*W consecutive nodes (chunks
// strided by the grid: a persistent launch).  Warp w takes nodes w, W + w,
// ... of the chunk, so the CTA's warps work on W consecutive nodes at a time
// and share their neighbours in L1.  Each warp loads the neighbour indices
// of its next node while it works on the current one.
template <int SL, bool CORR, bool TYPES, bool COMP, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
    k_mixed(pp_fused_args a, MixedConst c, int parity, Launch l) {
    constexpr int kChunk = kNodesPerWarp * W;
    __shared__ MixedShared<kChunk> sh;
    const int L = a.max_neigh;
    const int nchunks = (a.nnodes + kChunk - 1) / kChunk;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // error bounds of this step: running max |u| and the shortest bond
    const float U = __ldcg(a.umax);
    const QuickBand qb = quick_band(U, c);
    if constexpr (TYPES) {
        const int nt = a.nbond_types * a.nregimes;
        for (int t = threadIdx.x; t < nt; t += blockDim.x) {
            const float thr = (float)a.critical_stretch_table[t];
            const Thresholds th = thresholds(thr, 6.0e-8f * fabsf(thr), qb);
            sh.thr[t] = thr;
            sh.tlo[t] = th.lo;
            sh.thi[t] = th.hi;
            sh.k[t] = (float)a.bond_stiffness_table[t];
            sh.c[t] = (float)a.plus_cs[t];
        }
    } else {
        if (a.node_instance)
            for (int t = threadIdx.x; t < a.ninstances; t += blockDim.x) {
                const float thr = (float)a.instance_s0[t];
                const Thresholds th = thresholds(thr, 6.0e-8f * fabsf(thr), qb);
                sh.thr[t] = thr;
                sh.tlo[t] = th.lo;
                sh.thi[t] = th.hi;
            }
    }
    __syncthreads();
    const StepMags m = step_mags(l);
    const Thresholds th0 = thresholds(c.s0, c.s0_err, qb);
    // this thread's largest max |u| (node phases), raised once per warp at
    // the end
    float um = 0.f;
    if constexpr (SL >= 2) {
        // kNPW consecutive nodes per warp, kLPN lanes each
        constexpr int kLPN = kLanesPerNode;
        constexpr int kNPW = 32 / kLPN;
        // slots per batch: 4; 2 with bond types, whose regime state and
        // tables would otherwise hold enough registers per slot to cost a
        // resident CTA (composite: 0.334 vs 0.367 ms per step)
        constexpr int kG = TYPES ? 2 : 4;
        const int grp = lane / kLPN, sub = lane % kLPN;
        auto first_batch = [&](int i, int (&jn)[kG]) {
#pragma unroll
            for (int kk = 0; kk < kG; ++kk)
                jn[kk] = i < a.nnodes ? load_slot(a.nlist + (int64_t)i * L + sub + kLPN * kk) : -1;
        };
        int jn[kG];
        first_batch(blockIdx.x * kChunk + warp * kNPW + grp, jn);
        for (int chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
            const int node0 = chunk * kChunk;
            for (int t = 0; t < kNodesPerWarp / kNPW; ++t) {
                const int first = (t * W + warp) * kNPW;
                if (node0 + first >= a.nnodes) break;  // warp-uniform
                const int li = first + grp;
                const int i_next = t + 1 < kNodesPerWarp / kNPW
                                       ? node0 + li + W * kNPW
                                       : (chunk + gridDim.x) * kChunk + warp * kNPW + grp;
                bond_phase_group<kLPN, SL * 32 / kLPN, kG, CORR, TYPES, COMP>(
                    a, c, th0, sh, parity, node0 + li, li, lane, jn, i_next);
            }
            __syncthreads();
            for (int li = threadIdx.x >> 2; li < kChunk; li += blockDim.x >> 2)
                um = fmaxf(um, node_phase(a, c, sh, m, parity, node0, li, a.nnodes));
            __syncthreads();
        }
        raise_umax(a, um);
        return;
    }
    const bool has = SL > 1 || lane < L;
    // neighbour slots of node i (-1 beyond the row or past the last node)
    auto load_row = [&](int i, int (&jr)[SL]) {
#pragma unroll
        for (int k = 0; k < SL; ++k)
            jr[k] = (i < a.nnodes && has) ? load_slot(a.nlist + (int64_t)i * L + lane + 32 * k)
                                          : -1;
    };
    int jn[SL];
    load_row(blockIdx.x * kChunk + warp, jn);
    for (int chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
        const int node0 = chunk * kChunk;
        for (int t = 0; t < kNodesPerWarp; ++t) {
            const int li = t * W + warp;
            const int i = node0 + li;
            if (i >= a.nnodes) break;  // warp-uniform
            int jr[SL];
#pragma unroll
            for (int k = 0; k < SL; ++k) jr[k] = jn[k];
            const int next = t + 1 < kNodesPerWarp ? i + W : (chunk + gridDim.x) * kChunk + warp;
            load_row(next, jn);
            bond_phase_node<SL, CORR, TYPES, COMP>(a, c, qb, th0, sh, jr, parity, i, li, lane);
        }
        __syncthreads();
        for (int li = threadIdx.x >> 2; li < kChunk; li += blockDim.x >> 2)
            um = fmaxf(um, node_phase(a, c, sh, m, parity, node0, li, a.nnodes));
        __syncthreads();
    }
    raise_umax(a, um);
}

inline MixedConst mixed_const(const pp_fused_args& a) {
    MixedConst c;
    c.h = (float)a.pos_scale;
    c.mh = -kMagicF * c.h;
    c.geo = 1.7320508f * c.h;
    c.rxi_max = a.min_bond > 0.0 ? (float)(1.0 / a.min_bond) : 3.0e38f;
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

inline int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            n = 1;
    }
    return n;
}

// Persistent launch: as many CTAs as fit on the device at once (cached per
// kernel instance and shared-memory size).
template <int SL, bool CORR, bool TYPES, bool COMP, int W, int MINB>
int launch_instance(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    constexpr int kChunk = kNodesPerWarp * W;
    auto kernel = k_mixed<SL, CORR, TYPES, COMP, W, MINB>;
    static int cached_grid = 0;
    if (cached_grid == 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, W * 32, 0) !=
                cudaSuccess ||
            per_sm < 1)
            return PP_ERROR_CUDA;
        cached_grid = per_sm * sm_count();
    }
    const int nchunks = (a.nnodes + kChunk - 1) / kChunk;
    const int grid = nchunks < cached_grid ? nchunks : cached_grid;
    kernel<<<grid, W * 32, 0, st>>>(a, mixed_const(a), parity, l);
    return launch_status();
}

// All kernel instances of one tile shape (W warps, register budget MINB).
template <int W, int MINB, bool COMP>
int launch_shape_comp(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    const int sl = a.max_neigh > 32 ? a.max_neigh / 32 : 1;
#define PP_LAUNCH_SL(S)                                                                      \
    if (sl == S) {                                                                           \
        if (!corr && !types) return launch_instance<S, false, false, COMP, W, MINB>(a, parity, l, st); \
        if (corr && !types) return launch_instance<S, true, false, COMP, W, MINB>(a, parity, l, st);  \
        if (!corr && types) return launch_instance<S, false, true, COMP, W, MINB>(a, parity, l, st);  \
        return launch_instance<S, true, true, COMP, W, MINB>(a, parity, l, st);                       \
    }
    PP_LAUNCH_SL(1)
    PP_LAUNCH_SL(2)
    PP_LAUNCH_SL(4)
    PP_LAUNCH_SL(8)
#undef PP_LAUNCH_SL
    return PP_ERROR_UNSUPPORTED;  // max_neigh > 256
}

// All kernel instances of one tile shape (W warps, register budget MINB).
template <int W, int MINB>
int launch_shape(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st) {
    if (a.flags & PP_FLAG_COMPENSATED) return launch_shape_comp<W, MINB, true>(a, parity, l, st);
    return launch_shape_comp<W, MINB, false>(a, parity, l, st);
}

// Launchers of the tile shapes, one translation unit each (pp_mixed_v*.cu).
int launch_mixed_shape0(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st);
int launch_mixed_shape1(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st);
int launch_mixed_shape2(const pp_fused_args& a, int parity, const Launch& l, cudaStream_t st);

}  // namespace mixed
}  // namespace pp
