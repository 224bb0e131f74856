// pp_tiled.cuh -- the PP_MIXED fused step on the tiled layout (templates),
// shared by the translation units that instantiate its tile shapes
// (pp_tiled_v*.cu).  Layout and set-up: pp_gb300.h (pp_tiling) and
// pp_tiling.cu.
//
// Same arithmetic and the same exact break / regime decision as k_mixed
// (pp_mixed.cuh), with the neighbour records gathered from shared memory:
//
//  0. A persistent CTA takes tiles from a device counter (t.sched[0]; the
//     next tile is fetched while the current one computes; the last CTA to
//     finish resets both counter words for the next launch: no CTA waits
//     for another).
//  1. Staging: the records of the tile's halo (every node its bonds reach,
//     ascending) go to shared memory as two arrays, so that eight lanes
//     reading eight consecutive records hit eight different bank quads:
//     the displacement halves and max|u| by 16-byte cp.async, the
//     positions converted to floats relative to the tile's reference point
//     (exact: |q - ref| < 2^22 fixed-point steps) with the weight.  A bond
//     vector is then one subtraction per component, exactly h (q_j - q_i).
//  2. Bond phase: four nodes per warp, eight lanes per node; lane l reads
//     its row entries 16 m + l and 16 m + 8 + l as one 32-bit word of two
//     16-bit entries (the next words are loaded while a batch computes),
//     gathers both records from shared memory and does the FP32 bond
//     arithmetic of bond32_xi, two bonds per paired FP32 instruction
//     (bond32_xi2); a clearly intact bond is decided by one compare, every
//     other one in the per-node slow path (own error band, else the
//     binary64 stretch from the reference r0 and the exact double-float
//     displacement, peridynamics.cl:65-91).  A break writes the node's own
//     entry.  The four per-node sums are reduced over the eight lanes (4
//     shuffles).
//  3. Node update, right after the bond phase of each warp's two groups of
//     four nodes, by the lanes that hold the sums (every lane: the even
//     lanes of each eight update a node of the first group, the odd lanes
//     one of the second): the double-float update of k_mixed's node phase
//     (node_update), so its loads wait while other warps compute bonds,
//     with no barrier and no shared-memory round trip.  The running max |u|
//     is raised once per warp when the CTA ends.
//
// Entries are byte offsets (16 x halo index) into the staged arrays, so a
// gather is one shared load at an immediate offset; a broken bond or
// padding holds the node's own entry.  Every count read from the tiling is
// checked before it addresses shared or global memory: a tile with more
// than PP_TILE_NODES_MAX nodes or a halo longer than the tiling's halo_cap
// (the set-up marks a tile to split with halo_cap + 1) is skipped and
// reported in the status word (PP_STATUS_BAD_TILING).
#pragma once

#include "pp_mixed.cuh"

namespace pp {
namespace tiled {

using namespace mixed;

constexpr int kTileNodes = PP_TILE_NODES_MAX;
constexpr int kHaloCap = PP_TILE_HALO_MAX;  // staged records per CTA

// dynamic shared memory: positions at byte 0, displacements at kSuOffset,
// then (kTabOffset) the regime tables or instance thresholds, allocated
// only for the launches that read them (bond types, batch instances)
constexpr int kSuOffset = 16 * kHaloCap;
constexpr int kTabOffset = 32 * kHaloCap;

// One entry of the regime tables (bond types: index type * nregimes +
// regime) or of the per-instance thresholds (batch instances): 32 bytes, so
// that every field is at a fixed offset from the entry.
struct TabEntry {
    float thr, k, c;  // critical stretch (rounded to float), stiffness, plus_cs
    float tlo, thi;   // thresholds of thr (clearly below / clearly above)
    float pad[3];
};

// Dynamic shared memory of a launch: the halo arrays, plus the table
// entries the step reads (none for plain PMB).
inline size_t dyn_smem(const pp_fused_args& a) {
    const int entries = a.bond_types ? a.nbond_types * a.nregimes
                                     : (a.node_instance ? a.ninstances : 0);
    return static_cast<size_t>(kTabOffset) + sizeof(TabEntry) * static_cast<size_t>(entries);
}

// Staged record at byte offset `off` (an entry) of the array at `base`.
__device__ __forceinline__ float4 staged(const unsigned char* base, int off) {
    return *reinterpret_cast<const float4*>(base + off);
}

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
// node n0 + li of tile `tile`, its staged record at halo index own0 + li
// (entry own0 + li times 16, which its broken bonds and padding hold).
// Returns the node's sums reduced over the eight lanes: force x on lanes 0
// and 1 of the eight, y on 2 and 3, z on 4 and 5, the intact count on 6 and
// 7.  li >= nt: no node; the lanes only join the warp's shuffles.  NW: the
// most 32-bit entry words a lane can have (max_neigh / 16); the loop over
// them is unrolled, so every entry's bit and offset are constants, and
// stops at the warp's longest row.  A batch takes G entries (G / 2 words).
//
// dsm: the staged positions relative to the tile's reference point
// (float(q - ref) h, exact) with the weight, then (kSuOffset) the
// displacement halves with max|u|.  The bond vector xj - xi is exactly
// h (q_j - q_i), as in k_mixed.
//
// srow: the tile's row offsets (units of 16 entries) relative to its first
// row, which starts at entry tileE.
template <int NW, int G, bool CORR, bool TYPES, bool COMP>
__device__ __forceinline__ float bond_tile(const pp_fused_args& a, const pp_tiling& t,
                                           const MixedConst& c, const Thresholds& th0,
                                           const TabEntry* __restrict__ tab,
                                           const unsigned char* __restrict__ dsm,
                                           const int* __restrict__ srow, int64_t tileE, int parity,
                                           int tile, int n0, int nt, int own0, int li, int lane) {
    constexpr int GW = G / 2;  // words per batch
    const int sub = lane & 7;
    const bool node_ok = li < nt;
    const int lic = node_ok ? li : 0;
    const int i = n0 + lic;
    const int self = 16 * (own0 + lic);  // this node's own entry
    const float4 xi = staged(dsm, self);
    const float4 ui = staged(dsm + kSuOffset, self);
    const int nr = a.nregimes;
    float s0f = c.s0, s0err = c.s0_err;
    double s0d = a.critical_stretch;
    Thresholds th = th0;
    if (!TYPES && a.node_instance) {
        const int inst = a.node_instance[i];
        s0f = tab[inst].thr;
        s0err = 6.0e-8f * fabsf(s0f);
        s0d = a.instance_s0[inst];
        th.lo = tab[inst].tlo;
        th.hi = tab[inst].thi;
    }
    const int np = node_ok ? srow[lic + 1] - srow[lic] : 0;  // words of this lane
    const int npw = __reduce_max_sync(kFull, np);
    // this lane's entry position of word m, half h: lp + 16 m + h
    const int64_t lp = tileE + 16 * (int64_t)srow[lic] + 2 * sub;
    const uint32_t* ew = reinterpret_cast<const uint32_t*>(t.entry) + (lp >> 1);
    const uint32_t none = static_cast<uint32_t>(self) * 0x10001u;  // two own entries
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float cx = 0.f, cy = 0.f, cz = 0.f;  // carries (COMP)
    float cnt = 0.f;
    unsigned amb = 0u;
    uint32_t wn[GW];
#pragma unroll
    for (int g = 0; g < GW; ++g) wn[g] = g < np ? load_word(ew + 8 * g) : none;
#pragma unroll
    for (int m0 = 0; m0 < NW; m0 += GW) {
        if (m0 >= npw) break;  // warp-uniform
        uint32_t w[GW];
#pragma unroll
        for (int g = 0; g < GW; ++g) {
            w[g] = wn[g];
            if (m0 + GW < NW) wn[g] = m0 + GW + g < np ? load_word(ew + 8 * (m0 + GW + g)) : none;
        }
        int e[G];
#pragma unroll
        for (int g = 0; g < GW; ++g) {
            e[2 * g] = static_cast<int>(w[g] & 0xFFFFu);
            e[2 * g + 1] = static_cast<int>(w[g] >> 16);
        }
        float sc[G];
        int bt[G], rg[G];
#pragma unroll
        for (int g = 0; g < GW; ++g) {
            const int m = m0 + g;
            if constexpr (CORR) {
                const float2 cv =
                    m < np ? __ldcs(reinterpret_cast<const float2*>(t.correction + lp + 16 * m))
                           : make_float2(0.f, 0.f);
                sc[2 * g] = cv.x;
                sc[2 * g + 1] = cv.y;
            }
            if constexpr (TYPES) {
                const uint32_t bb = m < np ? load_u16x2(t.bond_type + lp + 16 * m) : 0u;
                const uint32_t gg = m < np ? load_u16x2(t.regime + lp + 16 * m) : 0u;
                bt[2 * g] = (bb & 0xFF) * nr;
                bt[2 * g + 1] = (bb >> 8) * nr;
                rg[2 * g] = gg & 0xFF;
                rg[2 * g + 1] = gg >> 8;
            }
        }
        float4 xj[G], uj[G];
#pragma unroll
        for (int kk = 0; kk < G; ++kk) {
            xj[kk] = staged(dsm, e[kk]);
            uj[kk] = staged(dsm + kSuOffset, e[kk]);
        }
        // the FP32 bond arithmetic of the batch, two bonds per instruction
        Bond32x2 bp[G / 2];
#pragma unroll
        for (int q = 0; q < G / 2; ++q) {
            const float4 &xa = xj[2 * q], &xb = xj[2 * q + 1];
            bp[q] = bond32_xi2(make_float2(xa.x - xi.x, xb.x - xi.x),
                               make_float2(xa.y - xi.y, xb.y - xi.y),
                               make_float2(xa.z - xi.z, xb.z - xi.z), ui, uj[2 * q], uj[2 * q + 1]);
        }
#pragma unroll
        for (int kk = 0; kk < G; ++kk) {
            const int k = 2 * m0 + kk;  // word k >> 1, half k & 1
            const bool valid = e[kk] != self;
            const Bond32 b = bp[kk >> 1].half(kk & 1);
            float wt = xj[kk].w;  // k*vol (PMB) or vol (types)
            if constexpr (!TYPES) {
                // clearly intact below th.lo; every other bond is decided in
                // the slow path below, where breaks are written
                const bool intact = valid && b.s < th.lo;
                if (valid && !intact) amb |= 1u << k;
                if (intact) {
                    float fv = (wt * b.s) * b.ry;
                    if constexpr (CORR) fv *= sc[kk];
                    acc_mul<COMP>(sx, cx, fv, b.px);
                    acc_mul<COMP>(sy, cy, fv, b.py);
                    acc_mul<COMP>(sz, cz, fv, b.pz);
                    cnt += 1.0f;
                }
            } else {
                if (!valid) continue;
                bool ambiguous = false;
                const int reg = next_regime(rg[kk], bt[kk], nr, [&](int idx) {
                    if (b.s < tab[idx].tlo) return true;
                    if (b.s > tab[idx].thi) return false;
                    const float thr = tab[idx].thr;
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
                if (reg >= nr) {
                    t.entry[pos] = static_cast<uint16_t>(self);
                    continue;
                }
                wt *= fmaf(b.s, tab[bt[kk] + reg].k, tab[bt[kk] + reg].c);
                float fv = wt * b.ry;
                if constexpr (CORR) fv *= sc[kk];
                acc_mul<COMP>(sx, cx, fv, b.px);
                acc_mul<COMP>(sy, cy, fv, b.py);
                acc_mul<COMP>(sz, cz, fv, b.pz);
                cnt += 1.0f;
            }
        }
    }
    // Slow path: entries that break, or whose FP32 stretch is too close to
    // a critical stretch.  Their entry is read again; the records come from
    // shared memory.
    if (__any_sync(kFull, amb != 0u)) {
        const int32_t* hl = t.halo + (int64_t)tile * t.halo_cap;
#pragma unroll 1
        for (unsigned bits = amb; bits != 0u; bits &= bits - 1u) {
            const int k = __ffs(bits) - 1;
            const int64_t pos = lp + 16 * (k >> 1) + (k & 1);
            const int e = t.entry[pos];
            if (e == self) continue;  // cannot happen: it was valid above
            const int j = hl[e >> 4];
            if (static_cast<unsigned>(j) >= static_cast<unsigned>(a.nnodes)) continue;
            const float4 xj = staged(dsm, e);
            const float4 uj = staged(dsm + kSuOffset, e);
            const Bond32 b = bond32_xi(xj.x - xi.x, xj.y - xi.y, xj.z - xi.z, ui, uj);
            float wt = xj.w;
            bool intact;
            if constexpr (!TYPES) {
                const float d = b.s - s0f;
                if (b.s > th.hi)
                    intact = false;
                else if (fabsf(d) > band32(ui, uj, b, c) + s0err)
                    intact = d < 0.0f;
                else
                    intact = exact_stretch(a, parity, i, j) < s0d;
                wt *= b.s;
            } else {
                const double s64 = exact_stretch(a, parity, i, j);
                const int btk = t.bond_type[pos] * nr;
                const int rgk = t.regime[pos];
                const int reg = next_regime(rgk, btk, nr, [&](int idx) {
                    return s64 < a.critical_stretch_table[idx];
                });
                if (reg != rgk) t.regime[pos] = static_cast<uint8_t>(reg);
                intact = reg < nr;
                if (intact) wt *= fmaf(b.s, tab[btk + reg].k, tab[btk + reg].c);
            }
            if (!intact) {
                t.entry[pos] = static_cast<uint16_t>(self);
                continue;
            }
            float fv = wt * b.ry;
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
    return v;
}

// One persistent CTA of W warps takes tiles until none are left.
template <int NW, bool CORR, bool TYPES, bool COMP, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
    k_tiled(pp_fused_args a, pp_tiling t, MixedConst c, int parity, Launch l) {
    // entries per batch: 4; 2 with bond types, whose regime state and
    // tables hold more registers per entry
    constexpr int kG = TYPES ? 2 : 4;
    extern __shared__ __align__(16) unsigned char dsm[];
    float4* sp = reinterpret_cast<float4*>(dsm);
    float4* su = reinterpret_cast<float4*>(dsm + kSuOffset);
    __shared__ int srow[kTileNodes + 1];
    TabEntry* tab = reinterpret_cast<TabEntry*>(dsm + kTabOffset);  // (when allocated)
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
            tab[k].thr = thr;
            tab[k].tlo = th.lo;
            tab[k].thi = th.hi;
            tab[k].k = (float)a.bond_stiffness_table[k];
            tab[k].c = (float)a.plus_cs[k];
        }
    } else {
        if (a.node_instance)
            for (int k = threadIdx.x; k < a.ninstances; k += blockDim.x) {
                const float thr = (float)a.instance_s0[k];
                const Thresholds th = thresholds(thr, 6.0e-8f * fabsf(thr), qb);
                tab[k].thr = thr;
                tab[k].tlo = th.lo;
                tab[k].thi = th.hi;
            }
    }
    const StepMags m = step_mags(l);
    const Thresholds th0 = thresholds(c.s0, c.s0_err, qb);
    if (threadIdx.x == 0) s_tile = atomicAdd(t.sched, 1);
    __syncthreads();
    int tile = s_tile;
    float um = 0.f;  // this thread's largest max |u| (node updates)
    while (tile < t.ntiles) {
        const int n0 = t.tile_start[tile];
        const int nt = t.tile_start[tile + 1] - n0;
        const int nh = t.halo_count[tile];
        const int own0 = t.own_off[tile];
        // (halo_cap <= kHaloCap is checked on the host; a halo count above
        // halo_cap is also the set-up's mark of a tile to split)
        const bool ok = nt >= 0 && nt <= kTileNodes && nh >= 0 && nh <= t.halo_cap &&
                        own0 >= 0 && own0 + nt <= nh && n0 >= 0 && n0 + nt <= a.nnodes;
        if (ok) {
            const int32_t* hl = t.halo + (int64_t)tile * t.halo_cap;
            const float* rec = a.rec[parity];
            const int4 ref = reinterpret_cast<const int4*>(t.tile_ref)[tile];
            // the displacement halves by cp.async; positions converted to
            // floats relative to the tile's reference point on the way.
            if constexpr (!CORR && !TYPES) {
                // In chunks of kPer records per thread, the halo indices of
                // a chunk all loaded before its records: a chunk waits on two
                // load latencies, not two per record.  (The instances with
                // corrections or bond types hold more state across the
                // staging, and the chunk's registers cost them more than
                // the latency saves: measured on the batched and composite
                // forms.)
                constexpr int kPer = 3;
#pragma unroll 1
                for (int h0 = 0; h0 < nh; h0 += kPer * W * 32) {
                    int idx[kPer];
#pragma unroll
                    for (int r = 0; r < kPer; ++r) {
                        const int h = h0 + threadIdx.x + r * W * 32;
                        const int j = h < nh ? hl[h] : 0;
                        idx[r] =
                            static_cast<unsigned>(j) < static_cast<unsigned>(a.nnodes) ? j : 0;
                    }
                    int4 q[kPer];
#pragma unroll
                    for (int r = 0; r < kPer; ++r) {
                        const int h = h0 + threadIdx.x + r * W * 32;
                        if (h < nh) {
                            cp_async16(&su[h], rec + 8 * (int64_t)idx[r] + 4);
                            q[r] = __ldg(reinterpret_cast<const int4*>(rec + 8 * (int64_t)idx[r]));
                        }
                    }
#pragma unroll
                    for (int r = 0; r < kPer; ++r) {
                        const int h = h0 + threadIdx.x + r * W * 32;
                        if (h < nh)
                            sp[h] = make_float4(
                                fixed_diff(q[r].x, ref.x, c), fixed_diff(q[r].y, ref.y, c),
                                fixed_diff(q[r].z, ref.z, c), __int_as_float(q[r].w));
                    }
                }
            } else {
                for (int h = threadIdx.x; h < nh; h += blockDim.x) {
                    int idx = hl[h];
                    idx = static_cast<unsigned>(idx) < static_cast<unsigned>(a.nnodes) ? idx : 0;
                    cp_async16(&su[h], rec + 8 * (int64_t)idx + 4);
                    const int4 q = __ldg(reinterpret_cast<const int4*>(rec + 8 * (int64_t)idx));
                    sp[h] = make_float4(fixed_diff(q.x, ref.x, c), fixed_diff(q.y, ref.y, c),
                                        fixed_diff(q.z, ref.z, c), __int_as_float(q.w));
                }
            }
            // row offsets of the tile, relative to its first row
            const int rbase = t.row_off[n0];
            for (int k = threadIdx.x; k <= nt; k += blockDim.x)
                srow[k] = t.row_off[n0 + k] - rbase;
            cp_async_wait_all();
            __syncthreads();
            // the next tile, fetched while this one computes (read after the
            // barrier that ends this tile; rewritten only after the next
            // staging barrier)
            if (threadIdx.x == 0) s_tile = atomicAdd(t.sched, 1);
            const int64_t tileE = 16 * (int64_t)rbase;
            // Two groups of four nodes per warp, then one node update of all
            // eight with every lane: the even lanes of each eight update the
            // first group's node, the odd lanes the second's (each lane holds
            // component (lane & 7) / 2 of both sums).
            for (int base = warp * 8; base < nt; base += W * 8) {  // warp-uniform
                const int la = base + (lane >> 3), lb = la + 4;
                float va = 0.f, vb = 0.f;
#pragma unroll 1
                for (int g = 0; g < 2; ++g) {  // one copy of the bond loop
                    const float v = bond_tile<NW, kG, CORR, TYPES, COMP>(
                        a, t, c, th0, tab, dsm, srow, tileE, parity, tile, n0, nt, own0,
                        la + 4 * g, lane);
                    if (g == 0)
                        va = v;
                    else
                        vb = v;
                }
                const bool odd = lane & 1;
                const int li = odd ? lb : la;
                const int comp = (lane & 7) >> 1;
                const int i = n0 + li;
                um = fmaxf(um, node_update<2>(a, c, m, parity, i, comp, li < nt, odd ? vb : va,
                                              GlobalDof{a, parity, i, comp}));
            }
        } else {
            if (threadIdx.x == 0) {
                atomicExch(a.status, PP_STATUS_BAD_TILING);
                s_tile = atomicAdd(t.sched, 1);
            }
        }
        // every warp is done with the staged halo (and s_tile is set)
        __syncthreads();
        tile = s_tile;
    }
    raise_umax(a, um);
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

// Persistent launch: as many CTAs as fit on the device at once (cached per
// kernel instance).
template <int NW, bool CORR, bool TYPES, bool COMP, int W, int MINB>
int launch_tiled_instance(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                          cudaStream_t st) {
    auto kernel = k_tiled<NW, CORR, TYPES, COMP, W, MINB>;
    // resident CTAs per SM: cached per kernel instance for the last
    // dynamic shared-memory size (it varies with the table entries).  Two
    // host threads racing here can only pair a size with another size's
    // grid: a grid that does not fit at once still completes (the CTAs take
    // tiles from the counter and never wait for one another).
    static size_t cached_dyn = 0;
    static int cached_grid = 0;
    const size_t dyn = dyn_smem(a);
    if (cached_grid == 0 || cached_dyn != dyn) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kTabOffset + sizeof(TabEntry) * kMaxTable)) !=
            cudaSuccess)
            return PP_ERROR_CUDA;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, W * 32, dyn) !=
                cudaSuccess ||
            per_sm < 1)
            return PP_ERROR_UNSUPPORTED;
        cached_grid = per_sm * sm_count();
        cached_dyn = dyn;
    }
    const int cg = cached_grid;
    const int grid = t.ntiles < cg ? t.ntiles : cg;
    if (grid < 1) return PP_SUCCESS;
    kernel<<<grid, W * 32, dyn, st>>>(a, t, mixed_const(a), parity, l);
    return launch_status();
}

template <int NW, int W, int MINB, bool COMP>
int launch_tiled_nw(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                    cudaStream_t st) {
    const bool corr = a.stiffness_corrections != nullptr;
    const bool types = a.bond_types != nullptr;
    if (!corr && !types)
        return launch_tiled_instance<NW, false, false, COMP, W, MINB>(a, t, parity, l, st);
    if (corr && !types)
        return launch_tiled_instance<NW, true, false, COMP, W, MINB>(a, t, parity, l, st);
    if (!corr && types)
        return launch_tiled_instance<NW, false, true, COMP, W, MINB>(a, t, parity, l, st);
    return launch_tiled_instance<NW, true, true, COMP, W, MINB>(a, t, parity, l, st);
}

// All kernel instances of one tile shape (W warps, register budget MINB):
// rows of at most 32, 64, 128 or 256 entries (max_neigh).
template <int W, int MINB>
int launch_tiled_shape(const pp_fused_args& a, const pp_tiling& t, int parity, const Launch& l,
                       cudaStream_t st) {
    const bool comp = (a.flags & PP_FLAG_COMPENSATED) != 0;
#define PP_TILED_NW(N)                                                        \
    if (a.max_neigh <= 16 * (N))                                              \
        return comp ? launch_tiled_nw<N, W, MINB, true>(a, t, parity, l, st) \
                    : launch_tiled_nw<N, W, MINB, false>(a, t, parity, l, st);
    PP_TILED_NW(2)
    PP_TILED_NW(4)
    PP_TILED_NW(8)
    PP_TILED_NW(16)
#undef PP_TILED_NW
    return PP_ERROR_UNSUPPORTED;  // max_neigh > 256
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
