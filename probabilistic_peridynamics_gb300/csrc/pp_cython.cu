// pp_cython.cu -- the time step of PeriPy's CPU integrator `Euler`
// (peripy/integrators.py:303-459), whose arithmetic is the Cython module
// peripy/peridynamics.pyx, on the GPU with the same results bit for bit.
//
// The Cython step is sequential over the nodes, and its results depend on
// that order in three places; each is reproduced per row or per node.
//
// break_bonds (peridynamics.pyx:102-156).  Node i, in ascending order,
// scans its row; a bond (i, j) with i < j whose |strain| is not below the
// critical strain is swap-removed from row i (the last entry moves into the
// hole, which is then examined again; the vacated slot keeps its stale
// value) and i is swap-removed from row j (first match).  Whether a bond
// breaks depends only on positions, so the final state of row i is that of
// (1) the removals made by its lower neighbours k < i, in ascending k, then
// (2) its own scan.  k_cy_break gives one warp to each row and applies
// exactly these edits to a copy of the row in shared memory.  This holds for
// symmetric neighbour lists (j in row i exactly when i is in row j), which
// Model builds and every removal keeps.
//
// bond_force (peridynamics.pyx:34-99).  Node i's force is the sequential
// sum, starting from 0, of -f * vol[k] for its lower neighbours k in
// ascending k (row k's loop subtracts them), then +f * vol[j] for its upper
// neighbours in row order, then the force boundary condition.  k_cy_force
// computes the terms of a row in parallel and sums them in that order.
//
// Distances and strains follow spatial.pyx: ceuclid(r1, r2) =
// sqrt((d0*d0 + d1*d1) + d2*d2) with d = r2 - r1, strain = (l - l0) / l0,
// with r = coords + u as Euler forms it; every operation is an explicitly
// rounded binary64 operation (no contraction), as the reference's C code
// compiles without fused multiply-adds.
#include "pp_common.cuh"

namespace pp {
namespace {

constexpr int kMaxWidth = 1024;

struct V3 {
    double x, y, z;
};

__device__ __forceinline__ V3 pos(const double* __restrict__ coords, const double* __restrict__ u,
                                  int i) {
    const int64_t o = 3 * (int64_t)i;
    return {dadd(coords[o], u[o]), dadd(coords[o + 1], u[o + 1]), dadd(coords[o + 2], u[o + 2])};
}

__device__ __forceinline__ V3 at(const double* __restrict__ a, int i) {
    const int64_t o = 3 * (int64_t)i;
    return {a[o], a[o + 1], a[o + 2]};
}

// ceuclid(r1, r2) (spatial.pyx:20-31)
__device__ __forceinline__ double ceuclid(const V3& r1, const V3& r2) {
    double d0 = dsub(r2.x, r1.x), d1 = dsub(r2.y, r1.y), d2 = dsub(r2.z, r1.z);
    d0 = dmul(d0, d0);
    d1 = dmul(d1, d1);
    d2 = dmul(d2, d2);
    return dsqrt(dadd(dadd(d0, d1), d2));
}

// cstrain2(l, r10, r20) (spatial.pyx:87-97)
__device__ __forceinline__ double cstrain2(double l, const V3& r10, const V3& r20) {
    const double l0 = ceuclid(r10, r20);
    return ddiv(dsub(l, l0), l0);
}

// Does the bond between lo < hi break (break_bonds' test, pyx:133)?
__device__ __forceinline__ bool cy_breaks(const double* coords, const double* u, int lo, int hi,
                                          double critical) {
    const double l = ceuclid(pos(coords, u, lo), pos(coords, u, hi));
    const double s = cstrain2(l, at(coords, lo), at(coords, hi));
    return !(fabs(s) < critical);
}

constexpr int kLower = 1;   // entry j < i
constexpr int kUpper = 2;   // entry j > i
constexpr int kBroken = 4;  // the bond breaks this step

// One warp per row.  rows: kWarps x width entries, flags likewise.
template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32)
    k_cy_break(const double* __restrict__ coords, const double* __restrict__ u,
               int32_t* __restrict__ nlist, int32_t* __restrict__ n_neigh, int nnodes, int width,
               double critical) {
    extern __shared__ int32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * kWarps + warp;
    if (i >= nnodes) return;  // warp-uniform
    int32_t* row = smem + (size_t)warp * width;
    int32_t* flag = smem + (size_t)(kWarps + warp) * width;
    int32_t* g = nlist + (int64_t)i * width;
    const int cnt0 = min(max(n_neigh[i], 0), width);
    bool any = false;
    for (int p = lane; p < cnt0; p += 32) {
        const int j = g[p];
        int f = 0;
        if (j >= 0 && j < nnodes && j != i) {
            f = j < i ? kLower : kUpper;
            if (cy_breaks(coords, u, j < i ? j : i, j < i ? i : j, critical)) f |= kBroken;
        }
        row[p] = j;
        flag[p] = f;
        any |= (f & kBroken) != 0;
    }
    if (!__any_sync(kFull, any)) return;  // nothing breaks: the row is unchanged
    __syncwarp();
    int cnt = cnt0;
    // (1) removals by the lower neighbours, in ascending neighbour index
    int last = -1;
    while (true) {
        int best = INT32_MAX;
        for (int p = lane; p < cnt; p += 32)
            if ((flag[p] & (kLower | kBroken)) == (kLower | kBroken) && row[p] > last &&
                row[p] < best)
                best = row[p];
        for (int off = 16; off > 0; off >>= 1) best = min(best, __shfl_xor_sync(kFull, best, off));
        if (best == INT32_MAX) break;
        last = best;
        int hit = -1;
        for (int p0 = 0; p0 < cnt && hit < 0; p0 += 32) {
            const int p = p0 + lane;
            const unsigned m = __ballot_sync(kFull, p < cnt && row[p] == best);
            if (m) hit = p0 + __ffs(m) - 1;
        }
        if (hit >= 0) {
            if (lane == 0) {
                row[hit] = row[cnt - 1];
                flag[hit] = flag[cnt - 1];
            }
            --cnt;
        }
        __syncwarp();
    }
    // (2) the row's own scan: broken upper bonds are swap-removed
    int next = 0;
    while (true) {
        int hit = -1;
        for (int p0 = next; p0 < cnt && hit < 0; p0 += 32) {
            const int p = p0 + lane;
            const unsigned m =
                __ballot_sync(kFull, p < cnt && (flag[p] & (kUpper | kBroken)) == (kUpper | kBroken));
            if (m) hit = p0 + __ffs(m) - 1;
        }
        if (hit < 0) break;
        if (lane == 0) {
            row[hit] = row[cnt - 1];
            flag[hit] = flag[cnt - 1];
        }
        --cnt;
        next = hit;
        __syncwarp();
    }
    __syncwarp();
    for (int p = lane; p < cnt0; p += 32) g[p] = row[p];
    if (lane == 0) n_neigh[i] = cnt;
}

// One warp per node.  Per warp in shared memory: the terms of its row (3
// doubles per entry) and the summation order (entry positions).
template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32)
    k_cy_force(const double* __restrict__ coords, const double* __restrict__ u,
               const int32_t* __restrict__ nlist, const int32_t* __restrict__ n_neigh,
               const double* __restrict__ vol, double k, const double* __restrict__ fc_values,
               const int32_t* __restrict__ fc_types, double fc_scale, int nnodes, int width,
               double* __restrict__ force) {
    extern __shared__ double dsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * kWarps + warp;
    if (i >= nnodes) return;  // warp-uniform
    double* term = dsm + (size_t)warp * 3 * width;
    int32_t* order = reinterpret_cast<int32_t*>(dsm + (size_t)kWarps * 3 * width) +
                     (size_t)warp * width;
    int32_t* key = order + (size_t)kWarps * width;
    const int32_t* g = nlist + (int64_t)i * width;
    const int cnt = min(max(n_neigh[i], 0), width);
    const V3 ri = pos(coords, u, i);
    const V3 r0i = at(coords, i);
    // terms; key = j for a lower neighbour (summed first, ascending j),
    // nnodes + position for an upper one (then in row order), -1 for none
    for (int p = lane; p < cnt; p += 32) {
        const int j = g[p];
        int kk = -1;
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
        if (j >= 0 && j < nnodes && j != i) {
            const V3 rj = pos(coords, u, j);
            const V3 r0j = at(coords, j);
            if (j < i) {
                // row j's loop: f = fn * (r[i] - r[j]), force[i] -= f * vol[j]
                const double l = ceuclid(rj, ri);
                const double fn = ddiv(dmul(cstrain2(l, r0j, r0i), k), l);
                t0 = dmul(dmul(fn, dsub(ri.x, rj.x)), vol[j]);
                t1 = dmul(dmul(fn, dsub(ri.y, rj.y)), vol[j]);
                t2 = dmul(dmul(fn, dsub(ri.z, rj.z)), vol[j]);
                kk = j;
            } else {
                // row i's loop: f = fn * (r[j] - r[i]), force[i] += f * vol[j]
                const double l = ceuclid(ri, rj);
                const double fn = ddiv(dmul(cstrain2(l, r0i, r0j), k), l);
                t0 = dmul(dmul(fn, dsub(rj.x, ri.x)), vol[j]);
                t1 = dmul(dmul(fn, dsub(rj.y, ri.y)), vol[j]);
                t2 = dmul(dmul(fn, dsub(rj.z, ri.z)), vol[j]);
                kk = nnodes + p;
            }
        }
        term[3 * p] = t0;
        term[3 * p + 1] = t1;
        term[3 * p + 2] = t2;
        key[p] = kk;
    }
    __syncwarp();
    // summation order: rank of each key among the row's keys (keys are
    // distinct; entries without a bond are left out)
    int used = 0;
    for (int p = 0; p < cnt; ++p) used += key[p] >= 0;
    for (int p = lane; p < cnt; p += 32) {
        const int kp = key[p];
        if (kp < 0) continue;
        int rank = 0;
        for (int q = 0; q < cnt; ++q) rank += key[q] >= 0 && key[q] < kp;
        order[rank] = p;
    }
    __syncwarp();
    if (lane < 3) {
        double acc = 0.0;
        for (int r = 0; r < used; ++r) {
            const int p = order[r];
            const double t = term[3 * p + lane];
            acc = key[p] < nnodes ? dsub(acc, t) : dadd(acc, t);
        }
        const int64_t o = 3 * (int64_t)i + lane;
        if (fc_types[o] != 0) acc = dadd(acc, dmul(fc_scale, fc_values[o]));
        force[o] = acc;
    }
}

// break_bonds then bond_force in one pass, one warp per node: each entry's
// length and strain are computed once (with the lower node first, as both
// Cython functions compute them), the row is edited as k_cy_break edits it
// (the values move with their entries), and the surviving entries' terms
// are summed in k_cy_force's order.  The force of node i depends only on
// its own row after the breaks, so no other warp is involved.
// With l0c (the per-slot reference lengths, (nnodes, width), kept in the
// order of the row's entries) the reference length is read instead of
// computed, and moves with its entry.  Shared memory per warp and slot:
// entry, flag, key, order (int32); length, strain, reference length and
// three terms (double).
template <int kWarps>
__global__ void __launch_bounds__(kWarps * 32)
    k_cy_break_force(const double* __restrict__ coords, const double* __restrict__ u,
                     int32_t* __restrict__ nlist, int32_t* __restrict__ n_neigh,
                     const double* __restrict__ vol, double k, double critical,
                     const double* __restrict__ fc_values, const int32_t* __restrict__ fc_types,
                     double fc_scale, int nnodes, int width, double* __restrict__ force,
                     double* __restrict__ l0c) {
    extern __shared__ double fsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * kWarps + warp;
    if (i >= nnodes) return;  // warp-uniform
    double* len = fsm + (size_t)warp * 6 * width;
    double* str = len + width;
    double* ref = str + width;
    double* term = ref + width;
    int32_t* ibase = reinterpret_cast<int32_t*>(fsm + (size_t)kWarps * 6 * width);
    int32_t* row = ibase + (size_t)warp * 4 * width;
    int32_t* flag = row + width;
    int32_t* key = flag + width;
    int32_t* order = key + width;
    int32_t* g = nlist + (int64_t)i * width;
    const int cnt0 = min(max(n_neigh[i], 0), width);
    const V3 ri = pos(coords, u, i);
    const V3 r0i = at(coords, i);
    double* gl0 = l0c ? l0c + (int64_t)i * width : nullptr;
    bool any = false;
    for (int p = lane; p < cnt0; p += 32) {
        const int j = g[p];
        int f = 0;
        double l = 0.0, st = 0.0, l0 = gl0 ? gl0[p] : 0.0;
        if (j >= 0 && j < nnodes && j != i) {
            const V3 rj = pos(coords, u, j);
            const V3 r0j = at(coords, j);
            // cstrain2 with the lower node first; the cached l0 is the
            // same value (ceuclid of the two reference positions)
            if (j < i) {
                l = ceuclid(rj, ri);
                if (!gl0) l0 = ceuclid(r0j, r0i);
                f = kLower;
            } else {
                l = ceuclid(ri, rj);
                if (!gl0) l0 = ceuclid(r0i, r0j);
                f = kUpper;
            }
            st = ddiv(dsub(l, l0), l0);
            if (!(fabs(st) < critical)) f |= kBroken;
        }
        row[p] = j;
        flag[p] = f;
        len[p] = l;
        str[p] = st;
        ref[p] = l0;
        any |= (f & kBroken) != 0;
    }
    const bool edited = __any_sync(kFull, any);
    __syncwarp();
    int cnt = cnt0;
    if (edited) {
        auto move = [&](int to, int from) {
            row[to] = row[from];
            flag[to] = flag[from];
            len[to] = len[from];
            str[to] = str[from];
            ref[to] = ref[from];
        };
        int last = -1;
        while (true) {
            int best = INT32_MAX;
            for (int p = lane; p < cnt; p += 32)
                if ((flag[p] & (kLower | kBroken)) == (kLower | kBroken) && row[p] > last &&
                    row[p] < best)
                    best = row[p];
            for (int off = 16; off > 0; off >>= 1)
                best = min(best, __shfl_xor_sync(kFull, best, off));
            if (best == INT32_MAX) break;
            last = best;
            int hit = -1;
            for (int p0 = 0; p0 < cnt && hit < 0; p0 += 32) {
                const int p = p0 + lane;
                const unsigned m = __ballot_sync(kFull, p < cnt && row[p] == best);
                if (m) hit = p0 + __ffs(m) - 1;
            }
            if (hit >= 0) {
                if (lane == 0) move(hit, cnt - 1);
                --cnt;
            }
            __syncwarp();
        }
        int next = 0;
        while (true) {
            int hit = -1;
            for (int p0 = next; p0 < cnt && hit < 0; p0 += 32) {
                const int p = p0 + lane;
                const unsigned m = __ballot_sync(
                    kFull, p < cnt && (flag[p] & (kUpper | kBroken)) == (kUpper | kBroken));
                if (m) hit = p0 + __ffs(m) - 1;
            }
            if (hit < 0) break;
            if (lane == 0) move(hit, cnt - 1);
            --cnt;
            next = hit;
            __syncwarp();
        }
        __syncwarp();
        for (int p = lane; p < cnt0; p += 32) {
            g[p] = row[p];
            if (gl0) gl0[p] = ref[p];
        }
        if (lane == 0) n_neigh[i] = cnt;
    }
    // bond_force on the edited row
    for (int p = lane; p < cnt; p += 32) {
        const int f = flag[p];
        int kk = -1;
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
        if (f & (kLower | kUpper)) {
            const int j = row[p];
            const V3 rj = pos(coords, u, j);
            const double fn = ddiv(dmul(str[p], k), len[p]);
            if (f & kLower) {
                t0 = dmul(dmul(fn, dsub(ri.x, rj.x)), vol[j]);
                t1 = dmul(dmul(fn, dsub(ri.y, rj.y)), vol[j]);
                t2 = dmul(dmul(fn, dsub(ri.z, rj.z)), vol[j]);
                kk = j;
            } else {
                t0 = dmul(dmul(fn, dsub(rj.x, ri.x)), vol[j]);
                t1 = dmul(dmul(fn, dsub(rj.y, ri.y)), vol[j]);
                t2 = dmul(dmul(fn, dsub(rj.z, ri.z)), vol[j]);
                kk = nnodes + p;
            }
        }
        term[3 * p] = t0;
        term[3 * p + 1] = t1;
        term[3 * p + 2] = t2;
        key[p] = kk;
    }
    __syncwarp();
    int used = 0;
    for (int p = 0; p < cnt; ++p) used += key[p] >= 0;
    for (int p = lane; p < cnt; p += 32) {
        const int kp = key[p];
        if (kp < 0) continue;
        int rank = 0;
        for (int q = 0; q < cnt; ++q) rank += key[q] >= 0 && key[q] < kp;
        order[rank] = p;
    }
    __syncwarp();
    if (lane < 3) {
        double acc = 0.0;
        for (int r = 0; r < used; ++r) {
            const int p = order[r];
            const double t = term[3 * p + lane];
            acc = key[p] < nnodes ? dsub(acc, t) : dadd(acc, t);
        }
        const int64_t o = 3 * (int64_t)i + lane;
        if (fc_types[o] != 0) acc = dadd(acc, dmul(fc_scale, fc_values[o]));
        force[o] = acc;
    }
}

// update_displacement (peridynamics.pyx:159-184)
__global__ void k_cy_update(double* __restrict__ u, const double* __restrict__ bc_values,
                            const int32_t* __restrict__ bc_types,
                            const double* __restrict__ force, double bc_scale, double dt,
                            int64_t ndof) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= ndof) return;
    u[o] = bc_types[o] == 0 ? dadd(u[o], dmul(dt, force[o])) : dmul(bc_scale, bc_values[o]);
}

// damage (peridynamics.pyx:5-31): (family - n_neigh) / family
__global__ void k_cy_damage(const int32_t* __restrict__ n_neigh, const int32_t* __restrict__ family,
                            int nnodes, double* __restrict__ damage) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnodes) return;
    const double f = (double)family[i];
    damage[i] = ddiv(dsub(f, (double)n_neigh[i]), f);
}

// Symmetry of compact rows: every entry j of row i (first n_neigh[i]
// entries, width `w`) must be a node whose row holds i exactly as often as
// row i holds j.  One warp per row; lane l takes entries l, l + 32, ... and
// counts both multiplicities by scanning the two rows.  *bad counts the
// entries that fail (out of range, or unequal multiplicities).
__global__ void k_cy_symmetric(const int32_t* __restrict__ nlist,
                               const int32_t* __restrict__ n_neigh, int nnodes, int w,
                               unsigned int* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= nnodes) return;
    const int ni = min(max(n_neigh[i], 0), w);
    const int32_t* ri = nlist + (int64_t)i * w;
    unsigned int nbad = 0;
    for (int k = lane; k < ni; k += 32) {
        const int j = ri[k];
        if (j < 0 || j >= nnodes) {
            ++nbad;
            continue;
        }
        const int nj = min(max(n_neigh[j], 0), w);
        const int32_t* rj = nlist + (int64_t)j * w;
        int fwd = 0, back = 0;
        for (int t = 0; t < ni; ++t) fwd += ri[t] == j;
        for (int t = 0; t < nj; ++t) back += rj[t] == i;
        nbad += fwd != back;
    }
    nbad = __reduce_add_sync(kFull, nbad);
    if (lane == 0 && nbad) atomicAdd(bad, nbad);
}

constexpr int kBreakWarps = 4;

int warps_for(size_t per_warp) {
    // up to 4 warps per block within 48 KB of shared memory
    int w = 4;
    while (w > 1 && per_warp * w > 48 * 1024) w >>= 1;
    return w;
}

template <int W>
int launch_force(const double* coords, const double* u, const int32_t* nlist,
                 const int32_t* n_neigh, const double* vol, double k, const double* fcv,
                 const int32_t* fct, double scale, int n, int width, double* force,
                 cudaStream_t st) {
    const size_t smem = (size_t)W * width * (3 * sizeof(double) + 2 * sizeof(int32_t));
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_cy_force<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return PP_ERROR_CUDA;
    k_cy_force<W><<<(n + W - 1) / W, W * 32, smem, st>>>(coords, u, nlist, n_neigh, vol, k, fcv,
                                                         fct, scale, n, width, force);
    return launch_status();
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_cy_break_bonds(const double* coords, const double* u, int32_t* nlist,
                                 int32_t* n_neigh, int32_t nnodes, int32_t max_neigh,
                                 double critical_strain, void* stream) {
    if (nnodes < 0 || max_neigh < 0) return PP_ERROR_INVALID_VALUE;
    if (max_neigh > kMaxWidth) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0 || max_neigh == 0) return PP_SUCCESS;
    if (!coords || !u || !nlist || !n_neigh) return PP_ERROR_INVALID_VALUE;
    const size_t smem = (size_t)2 * kBreakWarps * max_neigh * sizeof(int32_t);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_cy_break<kBreakWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return PP_ERROR_CUDA;
    k_cy_break<kBreakWarps>
        <<<(nnodes + kBreakWarps - 1) / kBreakWarps, kBreakWarps * 32, smem,
           static_cast<cudaStream_t>(stream)>>>(coords, u, nlist, n_neigh, nnodes, max_neigh,
                                                critical_strain);
    return launch_status();
}

extern "C" int pp_cy_bond_force(const double* coords, const double* u, const int32_t* nlist,
                                const int32_t* n_neigh, const double* volume,
                                double bond_stiffness, const double* force_bc_values,
                                const int32_t* force_bc_types, double force_bc_scale,
                                int32_t nnodes, int32_t max_neigh, double* force, void* stream) {
    if (nnodes < 0 || max_neigh < 0) return PP_ERROR_INVALID_VALUE;
    if (max_neigh > kMaxWidth) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!coords || !u || (max_neigh > 0 && !nlist) || !n_neigh || !volume || !force_bc_values ||
        !force_bc_types || !force)
        return PP_ERROR_INVALID_VALUE;
    const int width = max_neigh > 0 ? max_neigh : 1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (warps_for((size_t)width * (3 * sizeof(double) + 2 * sizeof(int32_t)))) {
        case 4:
            return launch_force<4>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                   force_bc_values, force_bc_types, force_bc_scale, nnodes,
                                   max_neigh, force, st);
        case 2:
            return launch_force<2>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                   force_bc_values, force_bc_types, force_bc_scale, nnodes,
                                   max_neigh, force, st);
        default:
            return launch_force<1>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                   force_bc_values, force_bc_types, force_bc_scale, nnodes,
                                   max_neigh, force, st);
    }
}

namespace {

template <int W>
int launch_break_force(const double* coords, const double* u, int32_t* nlist, int32_t* n_neigh,
                       const double* vol, double k, double critical, const double* fcv,
                       const int32_t* fct, double scale, int n, int width, double* force,
                       double* l0c, cudaStream_t st) {
    const size_t smem = (size_t)W * width * (6 * sizeof(double) + 4 * sizeof(int32_t));
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_cy_break_force<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return PP_ERROR_CUDA;
    k_cy_break_force<W><<<(n + W - 1) / W, W * 32, smem, st>>>(
        coords, u, nlist, n_neigh, vol, k, critical, fcv, fct, scale, n, width, force, l0c);
    return launch_status();
}

}  // namespace

extern "C" int pp_cy_break_and_force(const double* coords, const double* u, int32_t* nlist,
                                     int32_t* n_neigh, const double* volume,
                                     double bond_stiffness, double critical_strain,
                                     const double* force_bc_values,
                                     const int32_t* force_bc_types, double force_bc_scale,
                                     int32_t nnodes, int32_t max_neigh, double* force,
                                     double* bond_length, void* stream) {
    if (nnodes < 0 || max_neigh < 0) return PP_ERROR_INVALID_VALUE;
    if (max_neigh > kMaxWidth) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!coords || !u || (max_neigh > 0 && !nlist) || !n_neigh || !volume || !force_bc_values ||
        !force_bc_types || !force)
        return PP_ERROR_INVALID_VALUE;
    const int width = max_neigh > 0 ? max_neigh : 1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (warps_for((size_t)width * (6 * sizeof(double) + 4 * sizeof(int32_t)))) {
        case 4:
            return launch_break_force<4>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                         critical_strain, force_bc_values, force_bc_types,
                                         force_bc_scale, nnodes, max_neigh, force, bond_length,
                                         st);
        case 2:
            return launch_break_force<2>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                         critical_strain, force_bc_values, force_bc_types,
                                         force_bc_scale, nnodes, max_neigh, force, bond_length,
                                         st);
        default:
            return launch_break_force<1>(coords, u, nlist, n_neigh, volume, bond_stiffness,
                                         critical_strain, force_bc_values, force_bc_types,
                                         force_bc_scale, nnodes, max_neigh, force, bond_length,
                                         st);
    }
}

extern "C" int pp_cy_update_displacement(double* u, const double* bc_values,
                                         const int32_t* bc_types, const double* force,
                                         double bc_scale, double dt, int32_t nnodes,
                                         void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (nnodes == 0) return PP_SUCCESS;
    if (!u || !bc_values || !bc_types || !force) return PP_ERROR_INVALID_VALUE;
    const int64_t ndof = 3 * (int64_t)nnodes;
    k_cy_update<<<(unsigned)((ndof + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        u, bc_values, bc_types, force, bc_scale, dt, ndof);
    return launch_status();
}

extern "C" int pp_cy_check_symmetric(const int32_t* nlist, const int32_t* n_neigh,
                                     int32_t nnodes, int32_t width, uint32_t* bad,
                                     void* stream) {
    if (nnodes < 0 || width < 0 || width > 1024 || !bad) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(bad, 0, sizeof(uint32_t), st) != cudaSuccess) return PP_ERROR_CUDA;
    if (nnodes == 0 || width == 0) return PP_SUCCESS;
    if (!nlist || !n_neigh) return PP_ERROR_INVALID_VALUE;
    k_cy_symmetric<<<(nnodes + 7) / 8, 256, 0, st>>>(nlist, n_neigh, nnodes, width, bad);
    return launch_status();
}

extern "C" int pp_cy_damage(const int32_t* n_neigh, const int32_t* family, int32_t nnodes,
                            double* damage, void* stream) {
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    if (nnodes == 0) return PP_SUCCESS;
    if (!n_neigh || !family || !damage) return PP_ERROR_INVALID_VALUE;
    k_cy_damage<<<(nnodes + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n_neigh, family, nnodes, damage);
    return launch_status();
}
