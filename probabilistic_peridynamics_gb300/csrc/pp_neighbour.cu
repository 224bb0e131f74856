// pp_neighbour.cu -- neighbour families on the GPU: every pair of nodes
// closer than the horizon, in the CL layout (rows in ascending node order,
// -1 padding to a power-of-two width).  Replaces the host KD-tree search of
// Model._set_neighbour_list (peripy/model.py:536-597, sklearn KDTree
// query_radius), whose neighbour sets it reproduces.
//
// Nodes are binned into cubic cells of edge >= horizon (a counting sort:
// per-cell counts, one scan, a scatter that decrements each cell's end), so
// a node's neighbours lie in its own and the 26 adjacent cells.  One warp
// per node then tests the candidates of those cells, compacts the hits with
// a ballot, and finally writes its row sorted (rank sort in shared memory:
// the neighbour indices of a row are distinct).  A pair is a neighbour pair
// when (dx*dx + dy*dy) + dz*dz <= horizon*horizon in binary64, in that
// order, with no contraction.
#include <climits>

#include "pp_common.cuh"

namespace pp {
namespace {

constexpr int kRowWarps = 4;

__device__ __forceinline__ int3 cell_of(const double* __restrict__ r, int i, const double3 lo,
                                        double inv_cell, int3 dims) {
    int3 c;
    c.x = (int)floor((r[3 * (int64_t)i] - lo.x) * inv_cell);
    c.y = (int)floor((r[3 * (int64_t)i + 1] - lo.y) * inv_cell);
    c.z = (int)floor((r[3 * (int64_t)i + 2] - lo.z) * inv_cell);
    c.x = min(max(c.x, 0), dims.x - 1);
    c.y = min(max(c.y, 0), dims.y - 1);
    c.z = min(max(c.z, 0), dims.z - 1);
    return c;
}

__device__ __forceinline__ int64_t cell_index(int3 c, int3 dims) {
    return ((int64_t)c.x * dims.y + c.y) * dims.z + c.z;
}

// cs[c + 1] += 1 for the cell c of every node (cs zeroed by the caller).
__global__ void k_cell_count(const double* __restrict__ r, int n, double3 lo, double inv_cell,
                             int3 dims, int32_t* __restrict__ cs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(&cs[cell_index(cell_of(r, i, lo, inv_cell, dims), dims) + 1], 1);
}

// Inclusive scan of cs[1 .. ncells] in place, one block, chunks of 1024.
__global__ void __launch_bounds__(1024) k_cell_scan(int32_t* __restrict__ cs, int64_t ncells) {
    __shared__ int32_t warp_sums[32];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 1; base <= ncells; base += 1024) {
        const int64_t k = base + threadIdx.x;
        int32_t v = k <= ncells ? cs[k] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const int32_t t = __shfl_up_sync(kFull, v, off);
            if (lane >= off) v += t;
        }
        if (lane == 31) warp_sums[warp] = v;
        __syncthreads();
        if (warp == 0) {
            int32_t w = warp_sums[lane];
            for (int off = 1; off < 32; off <<= 1) {
                const int32_t t = __shfl_up_sync(kFull, w, off);
                if (lane >= off) w += t;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const int32_t total = v + (warp > 0 ? warp_sums[warp - 1] : 0) + carry;
        if (k <= ncells) cs[k] = total;
        __syncthreads();
        if (threadIdx.x == 1023) carry = total;
        __syncthreads();
    }
}

// Scatter: a node takes the last free place of its cell.  Afterwards
// cs[c + 1] is the start of cell c (its end was decremented count times).
__global__ void k_cell_fill(const double* __restrict__ r, int n, double3 lo, double inv_cell,
                            int3 dims, int32_t* __restrict__ cs, int32_t* __restrict__ order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t c = cell_index(cell_of(r, i, lo, inv_cell, dims), dims);
    order[atomicSub(&cs[c + 1], 1) - 1] = i;
}

__device__ __forceinline__ bool within(const double* __restrict__ r, int i, int j, double h2) {
    const double dx = __dsub_rn(r[3 * (int64_t)j], r[3 * (int64_t)i]);
    const double dy = __dsub_rn(r[3 * (int64_t)j + 1], r[3 * (int64_t)i + 1]);
    const double dz = __dsub_rn(r[3 * (int64_t)j + 2], r[3 * (int64_t)i + 2]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return d2 <= h2;
}

// One warp per node.  nlist == NULL: count only (family).  Else the row is
// collected (unsorted) in shared memory, rank-sorted into nlist and padded
// with -1; a row longer than max_neigh sets *overflow and is truncated.
__global__ void __launch_bounds__(kRowWarps * 32)
    k_rows(const double* __restrict__ r, int n, double h2, double3 lo, double inv_cell, int3 dims,
           const int32_t* __restrict__ cs, const int32_t* __restrict__ order, int max_neigh,
           int32_t* __restrict__ nlist, int32_t* __restrict__ family, int32_t* overflow) {
    extern __shared__ int32_t rows[];  // kRowWarps x max_neigh
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * kRowWarps + warp;
    if (i >= n) return;  // warp-uniform
    int32_t* row = rows + (size_t)warp * max_neigh;
    const int3 ci = cell_of(r, i, lo, inv_cell, dims);
    const int64_t ncells = (int64_t)dims.x * dims.y * dims.z;
    int cnt = 0;
    for (int ox = -1; ox <= 1; ++ox) {
        const int cx = ci.x + ox;
        if (cx < 0 || cx >= dims.x) continue;
        for (int oy = -1; oy <= 1; ++oy) {
            const int cy = ci.y + oy;
            if (cy < 0 || cy >= dims.y) continue;
            for (int oz = -1; oz <= 1; ++oz) {
                const int cz = ci.z + oz;
                if (cz < 0 || cz >= dims.z) continue;
                const int64_t c = cell_index(make_int3(cx, cy, cz), dims);
                const int beg = cs[c + 1];
                const int end = c + 1 < ncells ? cs[c + 2] : n;
                for (int k0 = beg; k0 < end; k0 += 32) {
                    const int k = k0 + lane;
                    const int j = k < end ? order[k] : -1;
                    const bool hit = j >= 0 && j != i && within(r, i, j, h2);
                    const unsigned m = __ballot_sync(kFull, hit);
                    if (hit && nlist) {
                        const int pos = cnt + __popc(m & ((1u << lane) - 1u));
                        if (pos < max_neigh) row[pos] = j;
                    }
                    cnt += __popc(m);
                }
            }
        }
    }
    if (lane == 0) family[i] = cnt;
    if (!nlist) return;
    if (cnt > max_neigh) {
        if (lane == 0) atomicExch(overflow, 1);
        cnt = max_neigh;
    }
    __syncwarp();
    int32_t* out = nlist + (int64_t)i * max_neigh;
    for (int e = lane; e < cnt; e += 32) {
        const int v = row[e];
        int rank = 0;
        for (int k = 0; k < cnt; ++k) rank += row[k] < v;
        out[rank] = v;
    }
    for (int e = cnt + lane; e < max_neigh; e += 32) out[e] = -1;
}

// ---- initial crack ---------------------------------------------------------
// Every pair c = (i, j) of the crack list is two edits: "remove j from row i"
// with key 2c and "remove i from row j" with key 2c + 1.  The edits are
// grouped by row with a counting sort (cs: per-row counts, the scan above,
// a decrement-scatter), and one warp per row applies its edits in key order,
// which is the order in which the sequential loop over the crack list meets
// them.  Edits of different rows commute, so the result is the sequential
// one.

// A pair's index selects a row counting from the end when negative, as an
// index of the reference's memoryviews does; the node looked for in the
// other row is the index as given.
__device__ __forceinline__ int crack_row(int i, int nnodes) { return i < 0 ? i + nnodes : i; }

// cs[row + 1] += 1 for both rows of every pair (cs zeroed by the caller); an
// index outside [-nnodes, nnodes) sets *bad.
__global__ void k_crack_count(const int32_t* __restrict__ crack, int npairs, int nnodes,
                              int32_t* __restrict__ cs, int32_t* bad) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npairs) return;
    const int i = crack[2 * (int64_t)c], j = crack[2 * (int64_t)c + 1];
    if (i < -nnodes || i >= nnodes || j < -nnodes || j >= nnodes) {
        atomicExch(bad, 1);
        return;
    }
    atomicAdd(&cs[crack_row(i, nnodes) + 1], 1);
    atomicAdd(&cs[crack_row(j, nnodes) + 1], 1);
}

// Scatter the edits into their rows' segments (nothing when *bad is set:
// the crack list is then rejected as a whole).  Afterwards cs[row + 1] is
// the start of the row's segment.
__global__ void k_crack_fill(const int32_t* __restrict__ crack, int npairs, int nnodes,
                             int32_t* __restrict__ cs, const int32_t* __restrict__ bad,
                             int32_t* __restrict__ key, int32_t* __restrict__ target) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= npairs || *bad) return;
    const int i = crack[2 * (int64_t)c], j = crack[2 * (int64_t)c + 1];
    int p = atomicSub(&cs[crack_row(i, nnodes) + 1], 1) - 1;
    key[p] = 2 * c;
    target[p] = j;
    p = atomicSub(&cs[crack_row(j, nnodes) + 1], 1) - 1;
    key[p] = 2 * c + 1;
    target[p] = i;
}

// One warp per row.  Edits are taken in ascending key order (a warp-wide
// minimum over the keys above the last one applied: keys are distinct).  An
// edit looks for the target among the row's first n_neigh entries; the
// first hit takes the row's last entry, whose slot becomes -1, and the count
// drops by one.  A target that is not found leaves the row as it is.
__global__ void __launch_bounds__(kRowWarps * 32)
    k_crack_apply(int nnodes, int max_neigh, int total, const int32_t* __restrict__ cs,
                  const int32_t* __restrict__ bad, const int32_t* __restrict__ key,
                  const int32_t* __restrict__ target, int32_t* __restrict__ nlist,
                  int32_t* __restrict__ n_neigh) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kRowWarps + (threadIdx.x >> 5);
    if (i >= nnodes || *bad) return;  // warp-uniform
    const int beg = cs[i + 1];
    const int end = i + 1 < nnodes ? cs[i + 2] : total;
    if (beg >= end) return;
    int32_t* row = nlist + (int64_t)i * max_neigh;
    int cnt = min(max(n_neigh[i], 0), max_neigh);
    int last = -1;
    for (int e = beg; e < end; ++e) {
        int best = INT_MAX, who = -1;
        for (int k = beg + lane; k < end; k += 32) {
            const int v = key[k];
            if (v > last && v < best) {
                best = v;
                who = k;
            }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const int ob = __shfl_xor_sync(kFull, best, off);
            const int ow = __shfl_xor_sync(kFull, who, off);
            if (ob < best) {
                best = ob;
                who = ow;
            }
        }
        last = best;
        const int b = target[who];
        int hit = -1;
        for (int k0 = 0; k0 < cnt && hit < 0; k0 += 32) {
            const int k = k0 + lane;
            const unsigned m = __ballot_sync(kFull, k < cnt && row[k] == b);
            if (m) hit = k0 + __ffs(m) - 1;
        }
        if (hit >= 0) {
            if (lane == 0) {
                row[hit] = row[cnt - 1];
                row[cnt - 1] = -1;
            }
            --cnt;
        }
        __syncwarp();
    }
    if (lane == 0) n_neigh[i] = cnt;
}

}  // namespace
}  // namespace pp

using namespace pp;

namespace {

int grid_args(const double* lo, double cell, const int32_t* dims, double3& lo3, int3& d3,
              int64_t& ncells) {
    if (!lo || !dims || !(cell > 0.0)) return PP_ERROR_INVALID_VALUE;
    if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return PP_ERROR_INVALID_VALUE;
    ncells = (int64_t)dims[0] * dims[1] * dims[2];
    if (ncells > (int64_t)INT32_MAX - 2) return PP_ERROR_TOO_LARGE;
    lo3 = make_double3(lo[0], lo[1], lo[2]);
    d3 = make_int3(dims[0], dims[1], dims[2]);
    return PP_SUCCESS;
}

}  // namespace

extern "C" int pp_neighbour_cells(const double* coords, int32_t nnodes, const double* lo,
                                  double cell, const int32_t* dims, int32_t* cell_start,
                                  int32_t* order, void* stream) {
    double3 lo3;
    int3 d3;
    int64_t ncells = 0;
    if (nnodes < 0) return PP_ERROR_INVALID_VALUE;
    const int g = grid_args(lo, cell, dims, lo3, d3, ncells);
    if (g != PP_SUCCESS) return g;
    if (!cell_start) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(cell_start, 0, (size_t)(ncells + 1) * sizeof(int32_t), st) != cudaSuccess)
        return PP_ERROR_CUDA;
    if (nnodes == 0) return launch_status();
    if (!coords || !order) return PP_ERROR_INVALID_VALUE;
    const double inv = 1.0 / cell;
    const unsigned blocks = (unsigned)((nnodes + 255) / 256);
    k_cell_count<<<blocks, 256, 0, st>>>(coords, nnodes, lo3, inv, d3, cell_start);
    k_cell_scan<<<1, 1024, 0, st>>>(cell_start, ncells);
    k_cell_fill<<<blocks, 256, 0, st>>>(coords, nnodes, lo3, inv, d3, cell_start, order);
    return launch_status();
}

extern "C" int pp_neighbour_rows(const double* coords, int32_t nnodes, double horizon,
                                 const double* lo, double cell, const int32_t* dims,
                                 const int32_t* cell_start, const int32_t* order,
                                 int32_t max_neigh, int32_t* nlist, int32_t* family,
                                 int32_t* overflow, void* stream) {
    double3 lo3;
    int3 d3;
    int64_t ncells = 0;
    if (nnodes < 0 || !(horizon >= 0.0)) return PP_ERROR_INVALID_VALUE;
    const int g = grid_args(lo, cell, dims, lo3, d3, ncells);
    if (g != PP_SUCCESS) return g;
    // neighbours must lie in the 27 cells around a node's cell, with room for
    // the rounding of the cell coordinates
    if (!(cell > horizon * (1.0 + 1e-9))) return PP_ERROR_INVALID_VALUE;
    if (nlist && !is_pow2_le_1024(max_neigh)) return PP_ERROR_MAX_NEIGH;
    if (nnodes == 0) return PP_SUCCESS;
    if (!coords || !cell_start || !order || !family || (nlist && !overflow))
        return PP_ERROR_INVALID_VALUE;
    const int width = nlist ? max_neigh : 0;
    const size_t smem = (size_t)kRowWarps * width * sizeof(int32_t);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return PP_ERROR_CUDA;
    k_rows<<<(nnodes + kRowWarps - 1) / kRowWarps, kRowWarps * 32, smem,
             static_cast<cudaStream_t>(stream)>>>(coords, nnodes, horizon * horizon,
                                                   lo3, 1.0 / cell, d3, cell_start, order,
                                                   width, nlist, family, overflow);
    return launch_status();
}

extern "C" int pp_create_crack(const int32_t* crack, int32_t npairs, int32_t nnodes,
                               int32_t max_neigh, int32_t* nlist, int32_t* n_neigh,
                               int32_t* scratch, int32_t* bad, void* stream) {
    if (npairs < 0 || nnodes < 0 || max_neigh < 1) return PP_ERROR_INVALID_VALUE;
    if ((int64_t)npairs > (INT32_MAX - 1) / 2) return PP_ERROR_TOO_LARGE;
    if (nnodes == INT32_MAX) return PP_ERROR_TOO_LARGE;
    if (npairs == 0) return PP_SUCCESS;
    if (!crack || !nlist || !n_neigh || !scratch || !bad) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // scratch: cs (nnodes + 1), then key and target (2 npairs each)
    int32_t* cs = scratch;
    int32_t* key = cs + (int64_t)nnodes + 1;
    int32_t* target = key + 2 * (int64_t)npairs;
    if (cudaMemsetAsync(cs, 0, ((size_t)nnodes + 1) * sizeof(int32_t), st) != cudaSuccess ||
        cudaMemsetAsync(bad, 0, sizeof(int32_t), st) != cudaSuccess)
        return PP_ERROR_CUDA;
    const unsigned blocks = (unsigned)((npairs + 255) / 256);
    k_crack_count<<<blocks, 256, 0, st>>>(crack, npairs, nnodes, cs, bad);
    if (nnodes > 0) k_cell_scan<<<1, 1024, 0, st>>>(cs, nnodes);
    k_crack_fill<<<blocks, 256, 0, st>>>(crack, npairs, nnodes, cs, bad, key, target);
    if (nnodes > 0)
        k_crack_apply<<<(nnodes + kRowWarps - 1) / kRowWarps, kRowWarps * 32, 0, st>>>(
            nnodes, max_neigh, 2 * npairs, cs, bad, key, target, nlist, n_neigh);
    return launch_status();
}
