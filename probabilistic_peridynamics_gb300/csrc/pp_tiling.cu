// pp_tiling.cu -- set-up of the tiled layout of the PP_MIXED step
// (pp_tile_halos, pp_tile_rows) and its conversion back to the reference
// neighbour list and regimes at write time (tile_export, called by
// pp_mixed_export).
//
// The layout (declared in pp_gb300.h): nodes renumbered into tiles of at
// most PP_TILE_NODES_MAX; per tile the ascending list of internal nodes its
// bonds reach (the halo); per node a CSR row of 16-bit halo indices in the
// reference row's slot order, stored so that lane l of a node's eight
// lanes reads row entries 16 m + l and 16 m + 8 + l as one 32-bit word.
#include "pp_fused.cuh"

namespace pp {
namespace tiling {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int lower_bound(const int* a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Position of row entry p within its row (see the file comment).
__device__ __forceinline__ int entry_pos(int p) {
    return 16 * (p >> 4) + 2 * (p & 7) + ((p >> 3) & 1);
}

__device__ __forceinline__ bool valid_node(int j, int n) { return j >= 0 && j < n; }

// One CTA per tile: the set of internal nodes the tile's bonds reach (and
// its own nodes) in a shared-memory hash set (open addressing, hc slots,
// a power of two >= 2 * the sorted capacity sc), then sorted (bitonic) into
// the halo.  Each node's row length (intact slots rounded up to 16) goes
// to row_off[i + 1] in units of 16 entries.
// Fixed-point position of reference node o (the formula of pp_mixed_pack).
__device__ __forceinline__ int fixed_pos(const double* r0, int64_t o, int d, const double* origin,
                                         double inv_scale) {
    return (int)llrint((r0[3 * o + d] - origin[d]) * inv_scale);
}

struct Frame {
    double origin[3];
    double inv_scale;  // 1 / pos_scale (a power of two: exact)
};

// The largest |q - ref| a staged position may have (exact float
// conversion of q - ref by the 1.5 * 2^23 exponent trick).
constexpr int kRefReach = (1 << 22) - 1;

__global__ void k_tile_halos(const int32_t* __restrict__ nlist, int L, int n,
                             const int32_t* __restrict__ perm, const int32_t* __restrict__ inv,
                             const int32_t* __restrict__ tile_start, int halo_cap, int hc,
                             int sc, int32_t* __restrict__ halo, int32_t* __restrict__ halo_count,
                             int32_t* __restrict__ own_off, int32_t* __restrict__ row_off,
                             int32_t* __restrict__ tile_ref, const double* __restrict__ r0,
                             Frame frame) {
    extern __shared__ int smem[];
    int* hs = smem;        // hash slots, -1 = empty
    int* keys = smem + hc;  // compacted, then sorted
    __shared__ int count, placed, far;
    __shared__ int qlo[3], qhi[3];
    const int t = blockIdx.x;
    const int n0 = tile_start[t], n1 = tile_start[t + 1];
    const int nt = n1 - n0;
    for (int k = threadIdx.x; k < hc; k += blockDim.x) hs[k] = -1;
    if (threadIdx.x == 0) {
        count = 0;
        placed = 0;
        far = 0;
        for (int d = 0; d < 3; ++d) {
            qlo[d] = 0x7FFFFFFF;
            qhi[d] = -0x7FFFFFFF;
        }
        if (t == 0) row_off[0] = 0;
    }
    __syncthreads();
    const unsigned shift = 32u - (unsigned)(__ffs(hc) - 1);  // hc = 2^(ffs-1)
    auto insert = [&](int key) {
        if (*(volatile int*)&count > halo_cap) return;  // overflow: stop
        unsigned h = ((unsigned)key * 0x9E3779B1u) >> shift;
        for (int probe = 0; probe < hc; ++probe) {
            const int old = atomicCAS(&hs[h], -1, key);
            if (old == -1) {
                atomicAdd(&count, 1);
                return;
            }
            if (old == key) return;
            h = (h + 1) & (hc - 1);
        }
    };
    for (int li = threadIdx.x; li < nt; li += blockDim.x) {
        insert(n0 + li);
        const int64_t o = perm[n0 + li];
        for (int d = 0; d < 3; ++d) {
            const int q = fixed_pos(r0, o, d, frame.origin, frame.inv_scale);
            atomicMin(&qlo[d], q);
            atomicMax(&qhi[d], q);
        }
    }
    // bonds: warp per node, lanes over slots; row lengths on the way
    const int lane = threadIdx.x & 31;
    for (int li = threadIdx.x >> 5; li < nt; li += blockDim.x >> 5) {
        const int o = perm[n0 + li];
        const int32_t* row = nlist + (int64_t)o * L;
        int cnt = 0;
        for (int s0 = 0; s0 < L; s0 += 32) {
            const int s = s0 + lane;
            const int j = s < L ? row[s] : -1;
            const bool ok = valid_node(j, n);
            cnt += __popc(__ballot_sync(kFull, ok));
            if (ok) insert(inv[j]);
        }
        if (lane == 0) row_off[n0 + li + 1] = (cnt + 15) >> 4;
    }
    __syncthreads();
    const int nh = count;
    if (nh > halo_cap) {
        if (threadIdx.x == 0) halo_count[t] = nh;
        return;
    }
    for (int k = threadIdx.x; k < hc; k += blockDim.x)
        if (hs[k] != -1) keys[atomicAdd(&placed, 1)] = hs[k];
    __syncthreads();
    int p2 = 1;
    while (p2 < nh) p2 <<= 1;
    for (int k = nh + threadIdx.x; k < p2; k += blockDim.x) keys[k] = 0x7FFFFFFF;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < p2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int a = keys[i], b = keys[ixj];
                    if ((a > b) == ((i & k) == 0)) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    // reference point: the middle of the tile's own bounding box; every
    // halo node must lie within kRefReach fixed-point steps of it
    int ref[3];
    for (int d = 0; d < 3; ++d)
        ref[d] = nt > 0 ? (int)(((long long)qlo[d] + (long long)qhi[d]) >> 1) : 0;
    for (int k = threadIdx.x; k < nh; k += blockDim.x) {
        const int64_t o = perm[keys[k]];
        for (int d = 0; d < 3; ++d) {
            const long long dq =
                (long long)fixed_pos(r0, o, d, frame.origin, frame.inv_scale) - ref[d];
            if (dq > kRefReach || dq < -kRefReach) far = 1;
        }
    }
    __syncthreads();
    if (far) {
        if (threadIdx.x == 0) halo_count[t] = halo_cap + 1;
        return;
    }
    int32_t* out = halo + (int64_t)t * halo_cap;
    for (int k = threadIdx.x; k < nh; k += blockDim.x) out[k] = keys[k];
    if (threadIdx.x == 0) {
        halo_count[t] = nh;
        own_off[t] = nt > 0 ? lower_bound(keys, nh, n0) : 0;
        for (int d = 0; d < 3; ++d) tile_ref[4 * t + d] = ref[d];
        tile_ref[4 * t + 3] = 0;
    }
}

// In-place inclusive scan of row_off[1..n] by one CTA of 1024 threads
// (each thread scans a contiguous chunk; the chunk totals are scanned with
// warp shuffles).  Set-up only.
__global__ void k_scan_rows(int32_t* __restrict__ row_off, int n) {
    __shared__ long long warp_tot[32];
    const int tid = threadIdx.x;
    const int64_t chunk = ((int64_t)n + blockDim.x - 1) / blockDim.x;
    const int64_t a = 1 + tid * chunk;
    const int64_t b = a + chunk < (int64_t)n + 1 ? a + chunk : (int64_t)n + 1;
    long long local = 0;
    for (int64_t k = a; k < b; ++k) local += row_off[k];
    // exclusive scan of the thread totals
    const int lane = tid & 31, warp = tid >> 5;
    long long incl = local;
    for (int off = 1; off < 32; off <<= 1) {
        const long long v = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const long long v = __shfl_up_sync(kFull, w, off);
            if (lane >= off) w += v;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    long long run = incl - local + (warp > 0 ? warp_tot[warp - 1] : 0);
    for (int64_t k = a; k < b; ++k) {
        run += row_off[k];
        row_off[k] = run > 0x7FFFFFFFLL ? -1 : (int32_t)run;  // -1: too many entries
    }
}

// One CTA per tile: the rows of its nodes (warp per node) from the
// reference row, in slot order, with halo indices found in the sorted halo
// (shared memory), stored as 16 x index; padding entries hold the node's
// own entry, slot 0xFF.  Also the initial intact count per node.
__global__ void k_tile_rows(const int32_t* __restrict__ nlist, int L, int n,
                            const int32_t* __restrict__ bond_types,
                            const int32_t* __restrict__ regimes,
                            const double* __restrict__ corrections, pp_tiling t) {
    extern __shared__ int hl[];
    const int tile = blockIdx.x;
    const int n0 = t.tile_start[tile], n1 = t.tile_start[tile + 1];
    // a count above the capacity (an unsplit tile) never addresses past it
    const int nh = min(max(t.halo_count[tile], 0), t.halo_cap);
    const int32_t* src = t.halo + (int64_t)tile * t.halo_cap;
    for (int k = threadIdx.x; k < nh; k += blockDim.x) hl[k] = src[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int own0 = t.own_off[tile];
    for (int i = n0 + (threadIdx.x >> 5); i < n1; i += blockDim.x >> 5) {
        const int o = t.perm[i];
        const uint16_t self = (uint16_t)(16 * (own0 + (i - n0)));
        const int64_t ref = (int64_t)o * L;
        const int64_t rowE = 16 * (int64_t)t.row_off[i];
        const int len = 16 * (t.row_off[i + 1] - t.row_off[i]);
        int base = 0;
        for (int s0 = 0; s0 < L; s0 += 32) {
            const int s = s0 + lane;
            const int j = s < L ? nlist[ref + s] : -1;
            const bool ok = valid_node(j, n);
            const unsigned bal = __ballot_sync(kFull, ok);
            if (ok) {
                const int p = base + __popc(bal & below);
                const int64_t pos = rowE + entry_pos(p);
                const int key = t.inv[j];
                const int e = lower_bound(hl, nh, key);
                t.entry[pos] = e < nh && hl[e] == key ? (uint16_t)(16 * e) : self;
                t.slot[pos] = (uint8_t)s;
                if (t.bond_type) t.bond_type[pos] = (uint8_t)bond_types[ref + s];
                if (t.regime) t.regime[pos] = (uint8_t)regimes[ref + s];
                if (t.correction) t.correction[pos] = (float)corrections[ref + s];
            }
            base += __popc(bal);
        }
        for (int p = base + lane; p < len; p += 32) {
            const int64_t pos = rowE + entry_pos(p);
            t.entry[pos] = self;
            t.slot[pos] = 0xFF;
            if (t.bond_type) t.bond_type[pos] = 0;
            if (t.regime) t.regime[pos] = 0;
            if (t.correction) t.correction[pos] = 0.0f;
        }
        if (lane == 0) t.n_neigh[i] = base;
    }
}

// Internal-order copies of the node arrays the step reads by node.
__global__ void k_tile_nodes(const double* __restrict__ r0, const double* __restrict__ bc_values,
                             const double* __restrict__ fc_values,
                             const int32_t* __restrict__ node_instance, int n, pp_tiling t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t o = t.perm[i];
    for (int d = 0; d < 3; ++d) {
        t.r0[3 * (int64_t)i + d] = r0[3 * o + d];
        t.bc_values[3 * (int64_t)i + d] = bc_values[3 * o + d];
        t.fc_values[3 * (int64_t)i + d] = fc_values[3 * o + d];
    }
    if (t.node_instance) t.node_instance[i] = node_instance[o];
}

// Bonds broken since pp_tile_rows (an entry equal to the node's own entry,
// slot != 0xFF) become -1 in the reference neighbour list; regimes are
// copied back.  Warp per internal node (its tile found by bisection).
__global__ void k_tile_export(int32_t* __restrict__ nlist, int32_t* __restrict__ regimes, int L,
                              int n, pp_tiling t) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    int lo = 0, hi = t.ntiles;  // the tile with tile_start[tile] <= i
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t.tile_start[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    const int self = 16 * (t.own_off[lo] + (i - t.tile_start[lo]));
    const int64_t ref = (int64_t)t.perm[i] * L;
    const int64_t rowE = 16 * (int64_t)t.row_off[i];
    const int len = 16 * (t.row_off[i + 1] - t.row_off[i]);
    for (int q = lane; q < len; q += 32) {
        const int s = t.slot[rowE + q];
        if (s == 0xFF || s >= L) continue;
        if (t.entry[rowE + q] == self) nlist[ref + s] = -1;
        if (regimes && t.regime) regimes[ref + s] = t.regime[rowE + q];
    }
}

int next_pow2(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

int check_tiling(const pp_fused_args& a, const pp_tiling* t) {
    if (!t) return PP_ERROR_INVALID_VALUE;
    if (t->ntiles < 0 || (a.nnodes > 0 && t->ntiles < 1)) return PP_ERROR_INVALID_VALUE;
    if (t->halo_cap < 1 || t->halo_cap > PP_TILE_HALO_MAX) return PP_ERROR_INVALID_VALUE;
    if (!t->perm || !t->inv || !t->tile_start || !t->halo || !t->halo_count || !t->own_off ||
        !t->tile_ref || !t->row_off || !t->r0 || !t->bc_values || !t->fc_values ||
        !t->n_neigh || !t->sched)
        return PP_ERROR_INVALID_VALUE;
    return PP_SUCCESS;
}

}  // namespace

// Used by pp_mixed_export.
int tile_export(const pp_fused_args& a, cudaStream_t st) {
    const pp_tiling* t = a.tiling;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.nlist || !t->entry || !t->slot) return PP_ERROR_INVALID_VALUE;
    k_tile_export<<<(a.nnodes + 7) / 8, 256, 0, st>>>(a.nlist, a.regimes, a.max_neigh, a.nnodes,
                                                      *t);
    return launch_status();
}

int validate_tiling(const pp_fused_args& a) {
    const int rc = check_tiling(a, a.tiling);
    if (rc != PP_SUCCESS) return rc;
    const pp_tiling* t = a.tiling;
    if (!t->entry) return PP_ERROR_INVALID_VALUE;
    if (a.bond_types && (!t->bond_type || !t->regime)) return PP_ERROR_INVALID_VALUE;
    if (a.stiffness_corrections && !t->correction) return PP_ERROR_INVALID_VALUE;
    if (a.node_instance && !t->node_instance) return PP_ERROR_INVALID_VALUE;
    if (!aligned16(t->entry)) return PP_ERROR_MISALIGNED;
    if ((t->correction && !aligned16(t->correction)) || (t->bond_type && !aligned16(t->bond_type)) ||
        (t->regime && !aligned16(t->regime)))
        return PP_ERROR_MISALIGNED;
    return PP_SUCCESS;
}

}  // namespace tiling
}  // namespace pp

using namespace pp;
using namespace pp::tiling;

extern "C" int pp_tile_halos(const pp_fused_args* args, const pp_tiling* t, void* stream) {
    if (!args) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0 || !is_pow2_le_1024(a.max_neigh) || a.max_neigh > 256)
        return PP_ERROR_INVALID_VALUE;
    int rc = check_tiling(a, t);
    if (rc != PP_SUCCESS) return rc;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.nlist || !a.r0 || !(a.pos_scale > 0.0)) return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Frame frame;
    for (int d = 0; d < 3; ++d) frame.origin[d] = a.pos_origin[d];
    frame.inv_scale = 1.0 / a.pos_scale;
    const int sc = next_pow2(t->halo_cap);
    const int hc = 2 * (sc < 512 ? 512 : sc);
    const size_t bytes = (size_t)(hc + sc) * sizeof(int);
    if (bytes > 48 * 1024) return PP_ERROR_UNSUPPORTED;
    k_tile_halos<<<t->ntiles, kThreads, bytes, st>>>(
        a.nlist, a.max_neigh, a.nnodes, t->perm, t->inv, t->tile_start, t->halo_cap, hc, sc,
        t->halo, t->halo_count, t->own_off, t->row_off, t->tile_ref, a.r0, frame);
    rc = launch_status();
    if (rc != PP_SUCCESS) return rc;
    k_scan_rows<<<1, 1024, 0, st>>>(t->row_off, a.nnodes);
    return launch_status();
}

extern "C" int pp_tile_rows(const pp_fused_args* args, const pp_tiling* t, void* stream) {
    if (!args) return PP_ERROR_INVALID_VALUE;
    const pp_fused_args& a = *args;
    if (a.nnodes < 0 || !is_pow2_le_1024(a.max_neigh) || a.max_neigh > 256)
        return PP_ERROR_INVALID_VALUE;
    int rc = check_tiling(a, t);
    if (rc != PP_SUCCESS) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(t->sched, 0, 2 * sizeof(int32_t), st) != cudaSuccess) return PP_ERROR_CUDA;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.nlist || !t->entry || !t->slot || !a.r0 || !a.bc_values || !a.fc_values)
        return PP_ERROR_INVALID_VALUE;
    if ((t->bond_type || t->regime) && (!a.bond_types || !a.regimes)) return PP_ERROR_INVALID_VALUE;
    if (t->correction && !a.stiffness_corrections) return PP_ERROR_INVALID_VALUE;
    if (t->node_instance && !a.node_instance) return PP_ERROR_INVALID_VALUE;
    k_tile_rows<<<t->ntiles, kThreads, (size_t)t->halo_cap * sizeof(int), st>>>(
        a.nlist, a.max_neigh, a.nnodes, a.bond_types, a.regimes, a.stiffness_corrections, *t);
    rc = launch_status();
    if (rc != PP_SUCCESS) return rc;
    k_tile_nodes<<<(a.nnodes + 255) / 256, 256, 0, st>>>(a.r0, a.bc_values, a.fc_values,
                                                        a.node_instance, a.nnodes, *t);
    return launch_status();
}
