// pp_tiled.cuh -- the PP_MIXED fused step on the tiled layout (templates),
// shared by the translation units that instantiate its tile shapes
// (pp_tiled_v*.cu).  Layout and set-up: pp_gb300.h (pp_tiling) and
// pp_tiling.cu.
//
// Same arithmetic and the same exact break / regime decision as k_mixed
// (pp_mixed.cuh), with the neighbour records gathered from shared memory:
//
//  0. A persistent CTA takes tiles from a device counter (t.sched[0]; the
//     last CTA to finish resets both counter words for the next launch:
//     no CTA waits for another).
//  1. Staging: the records of the tile's halo (every node its bonds reach,
//     ascending) are copied from the state slot into shared memory with
//     16-byte cp.async, as two arrays (positions + weight, displacements +
//     max|u|) so that eight lanes reading eight consecutive records hit
//     eight different bank quads.
//  2. Bond phase: four nodes per warp, eight lanes per node; lane l reads
//     its row entries 16 m + l and 16 m + 8 + l as one 32-bit word of two
//     16-bit halo indices (the next two words are loaded while a batch of
//     four computes), gathers both records from shared memory and does the
//     FP32 bond arithmetic of bond32; a clearly intact bond is decided by
//     one compare, every other one in the per-node slow path (own error
//     band, else the binary64 stretch from the reference r0 and the exact
//     double-float displacement, peridynamics.cl:65-91).  A break writes
//     0xFFFF into the entry.  The four per-node sums are reduced over the
//     eight lanes (4 shuffles) and parked in shared memory.
//  3. Node phase: as k_mixed (double-float update, next records written
//     with coalesced stores), for the tile's nodes.
//
// Every index read from the tiling is checked before it addresses shared
// memory: a tile with more than PP_TILE_NODES_MAX nodes or a halo longer
// than its capacity is skipped and reported in the status word
// (PP_STATUS_BAD_TILING); an entry >= the halo length is a broken bond.
#pragma once

#include "pp_mixed.cuh"

namespace pp {
namespace tiled {

using namespace mixed;

constexpr int kTileNodes = PP_TILE_NODES_MAX;

struct Tables {
    float thr[kMaxTable], k[kMaxTable], c[kMaxTable];  // regime tables or
                                                        // instance thresholds
    float tlo[kMaxTable], thi[kMaxTable];              // thresholds of thr[]
};

// node_phase reads the parked sums as sh.frc[li]
struct FrcView {
    const float4* frc;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// A word of two entries, read once and possibly overwritten later by the
// same thread (a break): coherent, no L1 allocation.
__device__ __forceinline__ uint32_t load_word(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.global.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t load_u16x2(const uint8_t* p) {
    return static_cast<uint32_t>(__ldcs(reinterpret_cast<const unsigned short*>(p)));
}

// Bond phase of one node (eight lanes, lane `lane & 7` of them): internal
// node n0 + li of tile `tile`, its record at halo index own0 + li.  Parks
// (force x, y, z, intact count) in sfrc[li].  li >= nt: no node; the lanes
// only join the warp's shuffles.
template <bool CORR, bool TYPES, bool COMP>
__device__ __forceinline__ void bond_tile(const pp_fused_args& a, const pp_tiling& t,
                                          const MixedConst& c, const Thresholds& th0,
                                          const Tables& tab, const int4* __restrict__ sq,
                                          const float4* __restrict__ su,
                                          float4* __restrict__ sfrc, int parity, int tile,
                                          int n0, int nt, int nh, int own0, int li, int lane) {
    const int sub = lane & 7;
    const bool node_ok = li < nt;
    const int lic = node_ok ? li : 0;
    const int i = n0 + lic;
    const int own = own0 + lic;
    const int4 qi = sq[own];
    const float4 ui = su[own];
    const int nr = a.nregimes;
    float s0f = c.s0, s0err = c.s0_err;
    double s0d = a.critical_stretch;
    Thresholds th = th0;
    if (!TYPES && a.node_instance) {
        const int inst = a.node_instance[i];
        s0f = tab.thr[inst];
        s0err = 6.0e-8f * fabsf(s0f);
        s0d = a.instance_s0[inst];
        th.lo = tab.tlo[inst];
        th.hi = tab.thi[inst];
    }
    int np = 0;  // 32-bit words (pairs of entries) per lane
    int64_t rowE = 0;
    if (node_ok) {
        const int r0 = t.row_off[i];
        np = t.row_off[i + 1] - r0;
        rowE = 16 * (int64_t)r0;
    }
    const int npw = __reduce_max_sync(kFull, np);
    // this lane's entry position of word m, half h: lp + 16 m + h
    const int64_t lp = rowE + 2 * sub;
    const uint32_t* ew = reinterpret_cast<const uint32_t*>(t.entry) + (lp >> 1);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float cx = 0.f, cy = 0.f, cz = 0.f;  // carries (COMP)
    float cnt = 0.f;
    unsigned amb = 0u;
    uint32_t wn0 = np > 0 ? load_word(ew) : 0xFFFFFFFFu;
    uint32_t wn1 = np > 1 ? load_word(ew + 8) : 0xFFFFFFFFu;
    for (int m0 = 0; m0 < npw; m0 += 2) {
        const uint32_t w0 = wn0, w1 = wn1;
        wn0 = m0 + 2 < np ? load_word(ew + 8 * (m0 + 2)) : 0xFFFFFFFFu;
        wn1 = m0 + 3 < np ? load_word(ew + 8 * (m0 + 3)) : 0xFFFFFFFFu;
        const int e[4] = {static_cast<int>(w0 & 0xFFFFu), static_cast<int>(w0 >> 16),
                          static_cast<int>(w1 & 0xFFFFu), static_cast<int>(w1 >> 16)};
        float sc[4];
        int bt[4], rg[4];
        if constexpr (CORR) {
            const float2 z = make_float2(0.f, 0.f);
            const float2 c0 =
                m0 < np ? __ldcs(reinterpret_cast<const float2*>(t.correction + lp + 16 * m0)) : z;
            const float2 c1 = m0 + 1 < np ? __ldcs(reinterpret_cast<const float2*>(
                                                t.correction + lp + 16 * (m0 + 1)))
                                          : z;
            sc[0] = c0.x;
            sc[1] = c0.y;
            sc[2] = c1.x;
            sc[3] = c1.y;
        }
        if constexpr (TYPES) {
            const uint32_t b0 = m0 < np ? load_u16x2(t.bond_type + lp + 16 * m0) : 0u;
            const uint32_t b1 = m0 + 1 < np ? load_u16x2(t.bond_type + lp + 16 * (m0 + 1)) : 0u;
            const uint32_t g0 = m0 < np ? load_u16x2(t.regime + lp + 16 * m0) : 0u;
            const uint32_t g1 = m0 + 1 < np ? load_u16x2(t.regime + lp + 16 * (m0 + 1)) : 0u;
            bt[0] = (b0 & 0xFF) * nr;
            bt[1] = (b0 >> 8) * nr;
            bt[2] = (b1 & 0xFF) * nr;
            bt[3] = (b1 >> 8) * nr;
            rg[0] = g0 & 0xFF;
            rg[1] = g0 >> 8;
            rg[2] = g1 & 0xFF;
            rg[3] = g1 >> 8;
        }
        int4 qj[4];
        float4 uj[4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int ee = e[kk] < nh ? e[kk] : own;
            qj[kk] = sq[ee];
            uj[kk] = su[ee];
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int k = 2 * m0 + kk;  // word k >> 1, half k & 1
            const bool valid = e[kk] < nh;
            const Bond32 b = bond32(qi, ui, qj[kk], uj[kk], c);
            float w = __int_as_float(qj[kk].w);  // k*vol (PMB) or vol (types)
            bool intact;
            if constexpr (!TYPES) {
                intact = valid && b.s < th.lo;
                if (valid && !intact) amb |= 1u << k;
                w *= b.s;
            } else {
                if (!valid) continue;
                bool ambiguous = false;
                const int reg = next_regime(rg[kk], bt[kk], nr, [&](int idx) {
                    if (b.s < tab.tlo[idx]) return true;
                    if (b.s > tab.thi[idx]) return false;
                    const float thr = tab.thr[idx];
                    const float d = b.s - thr;
                    if (!(fabsf(d) > band32(ui, uj[kk], b, c) + 6.0e-8f * fabsf(thr)))
                        ambiguous = true;
                    return d < 0.0f;
                });
                if (ambiguous) {
                    amb |= 1u << k;
                    continue;
                }
                const int64_t pos = lp + 16 * (k >> 1) + (k & 1);
                if (reg != rg[kk]) t.regime[pos] = static_cast<uint8_t>(reg);
                intact = reg < nr;
                if (!intact) {
                    t.entry[pos] = 0xFFFF;
                    continue;
                }
                w *= fmaf(b.s, tab.k[bt[kk] + reg], tab.c[bt[kk] + reg]);
            }
            float fv = intact ? w * b.ry : 0.0f;
            if constexpr (CORR) fv *= sc[kk];
            acc_mul<COMP>(sx, cx, fv, b.px);
            acc_mul<COMP>(sy, cy, fv, b.py);
            acc_mul<COMP>(sz, cz, fv, b.pz);
            cnt += intact ? 1.0f : 0.0f;
        }
    }
    // Slow path: entries that break, or whose FP32 stretch is too close to
    // a critical stretch.  Their halo index is read again; the records come
    // from shared memory.
    if (__any_sync(kFull, amb != 0u)) {
        const int32_t* hl = t.halo + (int64_t)tile * t.halo_cap;
#pragma unroll 1
        for (unsigned bits = amb; bits != 0u; bits &= bits - 1u) {
            const int k = __ffs(bits) - 1;
            const int64_t pos = lp + 16 * (k >> 1) + (k & 1);
            const int e = t.entry[pos];
            if (e >= nh) continue;  // cannot happen: it was valid above
            const int j = hl[e];
            const int4 qj = sq[e];
            const float4 uj = su[e];
            const Bond32 b = bond32(qi, ui, qj, uj, c);
            float w = __int_as_float(qj.w);
            bool intact;
            if constexpr (!TYPES) {
                const float d = b.s - s0f;
                if (b.s > th.hi)
                    intact = false;
                else if (fabsf(d) > band32(ui, uj, b, c) + s0err)
                    intact = d < 0.0f;
                else
                    intact = exact_stretch(a, parity, i, j) < s0d;
                w *= b.s;
            } else {
                const double s64 = exact_stretch(a, parity, i, j);
                const int btk = t.bond_type[pos] * nr;
                const int rgk = t.regime[pos];
                const int reg = next_regime(rgk, btk, nr, [&](int idx) {
                    return s64 < a.critical_stretch_table[idx];
                });
                if (reg != rgk) t.regime[pos] = static_cast<uint8_t>(reg);
                intact = reg < nr;
                if (intact) w *= fmaf(b.s, tab.k[btk + reg], tab.c[btk + reg]);
            }
            if (!intact) {
                t.entry[pos] = 0xFFFF;
                continue;
            }
            float fv = w * b.ry;
            if constexpr (CORR) fv *= t.correction[pos];
            acc_mul<COMP>(sx, cx, fv, b.px);
            acc_mul<COMP>(sy, cy, fv, b.py);
            acc_mul<COMP>(sz, cz, fv, b.pz);
            cnt += 1.0f;
        }
    }
    float v;
    if constexpr (COMP)
        v = reduce4c_group<8>(sx, cx, sy, cy, sz, cz, cnt, lane);
    else
        v = reduce4_group<8>(sx, sy, sz, cnt, lane);
    if (node_ok && sub < 8 && (sub & 1) == 0) reinterpret_cast<float*>(&sfrc[li])[sub >> 1] = v;
}

// One persistent CTA of W warps takes tiles until none are left.
template <bool CORR, bool TYPES, bool COMP, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
    k_tiled(pp_fused_args a, pp_tiling t, MixedConst c, int parity, Launch l) {
    extern __shared__ __align__(16) unsigned char dsm[];
    int4* sq = reinterpret_cast<int4*>(dsm);
    float4* su = reinterpret_cast<float4*>(dsm + 16 * static_cast<size_t>(t.halo_cap));
    __shared__ __align__(16) float4 sfrc[kTileNodes];
    __shared__ Tables tab;
    __shared__ int s_tile;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // error bounds of this step: running max |u| and the shortest bond
    const float U = __ldcg(a.umax);
    const QuickBand qb = quick_band(U, c);
    if constexpr (TYPES) {
        const int nt = a.nbond_types * a.nregimes;
        for (int k = threadIdx.x; k < nt; k += blockDim.x) {
            const float thr = (float)a.critical_stretch_table[k];
            const Thresholds th = thresholds(thr, 6.0e-8f * fabsf(thr), qb);
            tab.thr[k] = thr;
            tab.tlo[k] = th.lo;
            tab.thi[k] = th.hi;
            tab.k[k] = (float)a.bond_stiffness_table[k];
            tab.c[k] = (float)a.plus_cs[k];
        }
    } else {
        if (a.node_instance)
            for (int k = threadIdx.x; k < a.ninstances; k += blockDim.x) {
                const float thr = (float)a.instance_s0[k];
                const Thresholds th = thresholds(thr, 6.0e-8f * fabsf(thr), qb);
                tab.thr[k] = thr;
                tab.tlo[k] = th.lo;
                tab.thi[k] = th.hi;
            }
    }
    const StepMags m = step_mags(l);
    const Thresholds th0 = thresholds(c.s0, c.s0_err, qb);
    if (threadIdx.x == 0) s_tile = atomicAdd(t.sched, 1);
    __syncthreads();
    int tile = s_tile;
    while (tile < t.ntiles) {
        const int n0 = t.tile_start[tile];
        const int nt = t.tile_start[tile + 1] - n0;
        const int nh = t.halo_count[tile];
        const int own0 = t.own_off[tile];
        const bool ok = nt >= 0 && nt <= kTileNodes && nh >= 0 && nh <= t.halo_cap &&
                        own0 >= 0 && own0 + nt <= nh && n0 >= 0 && n0 + nt <= a.nnodes;
        if (ok) {
            const int32_t* hl = t.halo + (int64_t)tile * t.halo_cap;
            const float* rec = a.rec[parity];
            for (int h = threadIdx.x; h < nh; h += blockDim.x) {
                int idx = hl[h];
                idx = static_cast<unsigned>(idx) < static_cast<unsigned>(a.nnodes) ? idx : 0;
                cp_async16(&sq[h], rec + 8 * (int64_t)idx);
                cp_async16(&su[h], rec + 8 * (int64_t)idx + 4);
            }
            cp_async_wait_all();
            __syncthreads();
            for (int base = warp * 4; base < nt; base += W * 4)  // warp-uniform
                bond_tile<CORR, TYPES, COMP>(a, t, c, th0, tab, sq, su, sfrc, parity, tile, n0,
                                             nt, nh, own0, base + (lane >> 3), lane);
            __syncthreads();
            for (int li = threadIdx.x >> 2; li < kTileNodes; li += blockDim.x >> 2)
                node_phase(a, c, FrcView{sfrc}, m, parity, n0, li, n0 + nt);
        } else if (threadIdx.x == 0) {
            atomicExch(a.status, PP_STATUS_BAD_TILING);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_tile = atomicAdd(t.sched, 1);
        __syncthreads();
        tile = s_tile;
    }
    // the last CTA to finish leaves both counter words zero for the next
    // launch (every CTA has taken its last tile by then)
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(t.sched + 1, 1) == static_cast<int>(gridDim.x) - 1) {
            t.sched[0] = 0;
            t.sched[1] = 0;
        }
    }
}

// Persistent launch: as many CTAs as fit on the device at once for this
// halo capacity (cached per kernel instance and capacity).
template <bool CORR, bool TYPES, bool COMP, int W, int MINB>
int launch_tiled_instance(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                          cudaStream_t st) {
    auto kernel = k_tiled<CORR, TYPES, COMP, W, MINB>;
    static int cached_cap = -1, cached_grid = 0;
    const size_t dyn = 32 * static_cast<size_t>(t.halo_cap);
    if (cached_cap != t.halo_cap) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(dyn)) != cudaSuccess)
            return PP_ERROR_CUDA;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, W * 32, dyn) !=
                cudaSuccess ||
            per_sm < 1)
            return PP_ERROR_UNSUPPORTED;  // halo capacity too large for shared memory
        cached_grid = per_sm * sm_count();
        cached_cap = t.halo_cap;
    }
    const int grid = t.ntiles < cached_grid ? t.ntiles : cached_grid;
    if (grid < 1) return PP_SUCCESS;
    kernel<<<grid, W * 32, dyn, st>>>(a, t, mixed_const(a), parity, l);
    return launch_status();
}

template <int W, int MINB, bool COMP>
int launch_tiled_comp(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                      cudaStream_t st) {
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    if (!corr && !types) return launch_tiled_instance<false, false, COMP, W, MINB>(a, t, parity, l, st);
    if (corr && !types) return launch_tiled_instance<true, false, COMP, W, MINB>(a, t, parity, l, st);
    if (!corr && types) return launch_tiled_instance<false, true, COMP, W, MINB>(a, t, parity, l, st);
    return launch_tiled_instance<true, true, COMP, W, MINB>(a, t, parity, l, st);
}

// All kernel instances of one tile shape (W warps, register budget MINB).
template <int W, int MINB>
int launch_tiled_shape(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                       cudaStream_t st) {
    if (a.flags & PP_FLAG_COMPENSATED) return launch_tiled_comp<W, MINB, true>(a, t, parity, l, st);
    return launch_tiled_comp<W, MINB, false>(a, t, parity, l, st);
}

// Launchers of the tile shapes, one translation unit each (pp_tiled_v*.cu).
int launch_tiled_shape0(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st);
int launch_tiled_shape1(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st);
int launch_tiled_shape2(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                        cudaStream_t st);

}  // namespace tiled
}  // namespace pp
