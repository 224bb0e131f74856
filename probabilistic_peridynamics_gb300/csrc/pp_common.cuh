// pp_common.cuh -- device helpers shared by the step kernels.
//
// * Exact binary64 operations (__dadd_rn & co.) so that no compiler flag can
//   contract or reorder the reference arithmetic of peripy/cl/*.cl.
// * The work-group tree reduction of peripy/cl/peridynamics.cl:105-115,
//   restated for one warp per node: lane l owns slots l, l+32, l+64, ...;
//   the first log2(max_neigh/32) tree steps combine a lane's own slots in
//   registers, the last five are warp shuffles.  The association order is
//   the same as the work-group tree, so binary64 sums are bit-identical.
// * Double-float ("FP32 pair") arithmetic for the mixed-precision node state
//   (error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum and the
//   FMA-based TwoProduct; the pair operations follow the double-double
//   algorithms of Hida, Li and Bailey's QD library, restated for float).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pp_gb300.h"

namespace pp {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------- binary64
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

struct d3 {
    double x, y, z;
};

__device__ __forceinline__ d3 d3_zero() { return d3{0.0, 0.0, 0.0}; }
__device__ __forceinline__ d3 d3_add(d3 a, d3 b) {
    return d3{dadd(a.x, b.x), dadd(a.y, b.y), dadd(a.z, b.z)};
}
__device__ __forceinline__ d3 d3_shfl_down(d3 v, int off) {
    return d3{__shfl_down_sync(kFull, v.x, off), __shfl_down_sync(kFull, v.y, off),
              __shfl_down_sync(kFull, v.z, off)};
}

// Reduce per-slot binary64 vectors of one node held by one warp, in the
// work-group tree order.  SL = slots per lane = max(1, L/32).  `slot(k)`
// returns the contribution of slot k and is called exactly once for every
// slot < L (and for no other), on all lanes together.  The sum ends in lane 0.
template <int SL, class SlotFn>
__device__ __forceinline__ d3 tree_reduce_f64(int lane, int L, SlotFn&& slot) {
    d3 v;
    if constexpr (SL == 1) {
        v = (lane < L) ? slot(lane) : d3_zero();
        for (int off = (L >> 1) < 16 ? (L >> 1) : 16; off >= 1; off >>= 1)
            v = d3_add(v, d3_shfl_down(v, off));
        return v;
    } else {
        constexpr int H = SL / 2;
        d3 p[H];
#pragma unroll
        for (int k = 0; k < H; ++k) {
            d3 a = slot(lane + 32 * k);
            d3 b = slot(lane + 32 * (k + H));
            p[k] = d3_add(a, b);  // tree step i = L/2
        }
#pragma unroll
        for (int w = H / 2; w >= 1; w >>= 1) {
#pragma unroll
            for (int k = 0; k < w; ++k) p[k] = d3_add(p[k], p[k + w]);
        }
        v = p[0];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) v = d3_add(v, d3_shfl_down(v, off));
        return v;
    }
}

// ------------------------------------------------------------ double-float
struct df {
    float hi, lo;
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df{s, e};
}
// Dekker's Fast2Sum (requires |a| >= |b| or a == 0).
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return df{s, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
    df s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
// TwoProduct via FMA, plus cross terms.
__device__ __forceinline__ df df_mul(df a, df b) {
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_from_double(double x) {
    float hi = __double2float_rn(x);
    float lo = __double2float_rn(x - (double)hi);
    return df{hi, lo};
}
__device__ __forceinline__ double df_to_double(df a) {
    return (double)a.hi + (double)a.lo;  // exact: |lo| <= ulp(hi)/2
}

// ------------------------------------------------------------- utilities
__device__ __forceinline__ float4 ldg_f4(const float* p, int64_t i) {
    return __ldg(reinterpret_cast<const float4*>(p) + i);
}
__device__ __forceinline__ int4 ldg_i4(const int32_t* p, int64_t i) {
    return __ldg(reinterpret_cast<const int4*>(p) + i);
}

inline bool is_pow2_le_1024(int32_t x) { return x >= 1 && x <= 1024 && (x & (x - 1)) == 0; }

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline bool aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31u) == 0; }

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PP_SUCCESS : PP_ERROR_CUDA;
}

}  // namespace pp
