// pp_writes.cu -- the sums Model.simulate records at every write step
// (peripy/model.py:1320-1366), computed on the device so that a write needs
// to bring back only what the mesh file holds (u and damage).
//
// Model sums.  The reference takes np.sum over each (nnodes, 3) state array,
// over force * volume[:, None] and body_force * volume[:, None], and over
// damage.  NumPy's float64 sum of a contiguous array is 0.0 + P(a, n), with
// P its pairwise summation:
//   n < 8:        ((0.0 + a[0]) + a[1]) + ...
//   8 <= n <= 128: eight running sums r[j] = a[j] + a[j + 8] + ... over the
//                 first n - n % 8 elements, ((r0 + r1) + (r2 + r3)) +
//                 ((r4 + r5) + (r6 + r7)), then the last n % 8 elements in
//                 order
//   n > 128:      P(a, m) + P(a + m, n - m) with m = n / 2 rounded down to a
//                 multiple of 8.
// The split depends on n only, so pp_pairwise_plan writes the tree once on
// the host: its leaves (first element, length) and its inner nodes ordered
// by height.  k_sum_leaves evaluates every leaf of every array in parallel;
// k_sum_tree then adds the inner nodes one height at a time in one block per
// array.  Every operation is an explicitly rounded binary64 add or multiply
// (no contraction), so the sums are NumPy's bit for bit.
//
// Tip sums.  For each tip type the reference adds u[i, j], ud[i, j],
// udd[i, j], force[i, j] * volume[i] and body_force[i, j] * volume[i] over
// its (node, dof) list in order, starting from 0.0: one thread per tip type
// and quantity does the same sequential sum.
#include <vector>

#include "pp_common.cuh"

namespace pp {
namespace {

constexpr int kLeafMax = 128;
constexpr int kArrays = 6;  // u, ud, udd, force * vol, body_force * vol, damage

struct SumSource {
    const double* x;       // NULL: an array of zeros
    const double* scale;   // NULL, or vol: element k is x[k] * scale[k / 3]
};

__device__ __forceinline__ double element(const SumSource& s, int64_t k) {
    const double v = s.x[k];
    return s.scale ? __dmul_rn(v, s.scale[k / 3]) : v;
}

__device__ double leaf_sum(const SumSource& s, int64_t lo, int n) {
    if (n < 8) {
        double r = 0.0;
        for (int k = 0; k < n; ++k) r = __dadd_rn(r, element(s, lo + k));
        return r;
    }
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = element(s, lo + j);
    const int body = n - n % 8;
    int i = 8;
    for (; i < body; i += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = __dadd_rn(r[j], element(s, lo + i + j));
    }
    double res = __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[1]), __dadd_rn(r[2], r[3])),
                           __dadd_rn(__dadd_rn(r[4], r[5]), __dadd_rn(r[6], r[7])));
    for (; i < n; ++i) res = __dadd_rn(res, element(s, lo + i));
    return res;
}

struct SumJob {
    SumSource src[kArrays];
    const int32_t* plan[kArrays];  // plan3 for the first five, plan1 for damage
    double* val[kArrays];          // leaf values, then inner-node values
};

// Plan header: [0] leaves, [1] inner nodes, [2] heights, [3] elements; then
// leaf first elements, leaf lengths, inner left, inner right (value
// indices: leaves first, inner nodes after them), height offsets.
__device__ __forceinline__ const int32_t* leaf_lo(const int32_t* p) { return p + 4; }
__device__ __forceinline__ const int32_t* leaf_len(const int32_t* p) { return p + 4 + p[0]; }
__device__ __forceinline__ const int32_t* inner_left(const int32_t* p) { return p + 4 + 2 * p[0]; }
__device__ __forceinline__ const int32_t* inner_right(const int32_t* p) {
    return p + 4 + 2 * p[0] + p[1];
}
__device__ __forceinline__ const int32_t* height_off(const int32_t* p) {
    return p + 4 + 2 * p[0] + 2 * p[1];
}

// Work item w < 5 * leaves3 + leaves1: array w / leaves3 (the first five) or
// damage.
__global__ void __launch_bounds__(256)
    k_sum_leaves(SumJob job, int leaves3, int leaves1) {
    const int64_t total = 5 * (int64_t)leaves3 + leaves1;
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total;
         w += (int64_t)gridDim.x * blockDim.x) {
        int a, t;
        if (w < 5 * (int64_t)leaves3) {
            a = (int)(w / leaves3);
            t = (int)(w % leaves3);
        } else {
            a = 5;
            t = (int)(w - 5 * (int64_t)leaves3);
        }
        if (!job.src[a].x) continue;
        const int32_t* p = job.plan[a];
        job.val[a][t] = leaf_sum(job.src[a], leaf_lo(p)[t], leaf_len(p)[t]);
    }
}

// Blocks 0..5: the inner nodes of one array's tree, one height at a time,
// then sums[a] = 0.0 + root.  Block 6 (when there are tips): the tip sums.
__global__ void __launch_bounds__(256)
    k_sum_tree(SumJob job, const double* __restrict__ volume, int ntips,
               const int32_t* __restrict__ tip_offsets, const int32_t* __restrict__ tip_entries,
               double* __restrict__ sums) {
    if (blockIdx.x < kArrays) {
        const int a = blockIdx.x;
        const int32_t* p = job.plan[a];
        const int leaves = p[0], inner = p[1], heights = p[2];
        double* val = job.val[a];
        if (!job.src[a].x || leaves == 0) {
            if (threadIdx.x == 0) sums[a] = 0.0;
            return;
        }
        const int32_t* left = inner_left(p);
        const int32_t* right = inner_right(p);
        const int32_t* off = height_off(p);
        for (int h = 0; h < heights; ++h) {
            for (int k = off[h] + threadIdx.x; k < off[h + 1]; k += blockDim.x)
                val[leaves + k] = __dadd_rn(val[left[k]], val[right[k]]);
            __syncthreads();
        }
        if (threadIdx.x == 0) sums[a] = __dadd_rn(0.0, val[inner > 0 ? leaves + inner - 1 : 0]);
        return;
    }
    // tips: thread q = 5 * tip + quantity
    for (int q = threadIdx.x; q < 5 * ntips; q += blockDim.x) {
        const int tip = q / 5, what = q % 5;
        const SumSource s = job.src[what];
        double acc = 0.0;
        if (s.x) {
            for (int e = tip_offsets[tip]; e < tip_offsets[tip + 1]; ++e) {
                const int i = tip_entries[2 * (int64_t)e], j = tip_entries[2 * (int64_t)e + 1];
                const double v = s.x[3 * (int64_t)i + j];
                acc = __dadd_rn(acc, s.scale ? __dmul_rn(v, volume[i]) : v);
            }
        }
        sums[kArrays + q] = acc;
    }
}

// ---- host: the pairwise tree of n elements ---------------------------------
struct PlanBuilder {
    std::vector<int32_t> lo, len;             // leaves in order
    std::vector<int32_t> left, right, height;  // inner nodes in creation order
    // child references: >= 0 leaf index, < 0 inner node -(id + 1)
    int32_t add(int64_t first, int64_t n, int32_t& h) {
        if (n <= kLeafMax) {
            lo.push_back((int32_t)first);
            len.push_back((int32_t)n);
            h = 0;
            return (int32_t)lo.size() - 1;
        }
        int64_t m = n / 2;
        m -= m % 8;
        int32_t hl = 0, hr = 0;
        const int32_t l = add(first, m, hl);
        const int32_t r = add(first + m, n - m, hr);
        left.push_back(l);
        right.push_back(r);
        h = 1 + (hl > hr ? hl : hr);
        height.push_back(h);
        return -(int32_t)left.size();
    }
};

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int64_t pp_pairwise_plan(int64_t n, int32_t* plan, int64_t capacity) {
    if (n < 0 || n > INT32_MAX) return -1;
    PlanBuilder b;
    if (n > 0) {
        int32_t h = 0;
        b.add(0, n, h);
    }
    const int64_t leaves = (int64_t)b.lo.size(), inner = (int64_t)b.left.size();
    int32_t heights = 0;
    for (int32_t h : b.height) heights = h > heights ? h : heights;
    const int64_t need = 4 + 2 * leaves + 2 * inner + heights + 1;
    if (!plan || capacity < need) return need;
    // inner nodes ordered by height (stable), value index leaves + position
    std::vector<int32_t> off(heights + 2, 0);
    for (int32_t h : b.height) ++off[h];  // heights are 1..heights
    for (int32_t h = 1, acc = 0; h <= heights + 1; ++h) {
        const int32_t c = off[h];
        off[h] = acc;
        acc += c;
    }
    std::vector<int32_t> pos(inner);
    for (int64_t k = 0; k < inner; ++k) pos[k] = off[b.height[k]]++;
    auto ref = [&](int32_t r) -> int32_t {
        return r >= 0 ? r : (int32_t)(leaves + pos[-r - 1]);
    };
    int32_t* p = plan;
    p[0] = (int32_t)leaves;
    p[1] = (int32_t)inner;
    p[2] = heights;
    p[3] = (int32_t)n;
    int32_t* lo = p + 4;
    int32_t* len = lo + leaves;
    int32_t* lft = len + leaves;
    int32_t* rgt = lft + inner;
    int32_t* hoff = rgt + inner;
    for (int64_t t = 0; t < leaves; ++t) {
        lo[t] = b.lo[t];
        len[t] = b.len[t];
    }
    for (int64_t k = 0; k < inner; ++k) {
        lft[pos[k]] = ref(b.left[k]);
        rgt[pos[k]] = ref(b.right[k]);
    }
    // after the placement pass off[h] is the end of height h, which is the
    // start of height h + 1: hoff[h - 1] = start of height h
    hoff[0] = 0;
    for (int32_t h = 1; h <= heights; ++h) hoff[h] = off[h];
    return need;
}

extern "C" int pp_write_sums(const pp_write_sums_args* a, void* stream) {
    if (!a || a->nnodes < 0 || a->ntips < 0) return PP_ERROR_INVALID_VALUE;
    if (3 * (int64_t)a->nnodes > INT32_MAX) return PP_ERROR_TOO_LARGE;
    if (!a->sums || !a->plan3 || !a->plan1 || !a->scratch) return PP_ERROR_INVALID_VALUE;
    if (a->nnodes > 0 && (!a->u || !a->damage || !a->volume)) return PP_ERROR_INVALID_VALUE;
    if (a->ntips > 0 && (!a->tip_offsets || !a->tip_entries)) return PP_ERROR_INVALID_VALUE;
    if (a->leaves3 < 0 || a->values3 < a->leaves3 || a->leaves1 < 0 ||
        a->values1 < a->leaves1)
        return PP_ERROR_INVALID_VALUE;
    SumJob job;
    const double* xs[kArrays] = {a->u, a->ud, a->udd, a->force, a->body_force, a->damage};
    for (int k = 0; k < kArrays; ++k) {
        job.src[k].x = xs[k];
        job.src[k].scale = (k == 3 || k == 4) ? a->volume : nullptr;
        job.plan[k] = k < 5 ? a->plan3 : a->plan1;
        job.val[k] = a->scratch + (k < 5 ? (int64_t)k * a->values3 : 5 * (int64_t)a->values3);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t work = 5 * (int64_t)a->leaves3 + a->leaves1;
    if (work > 0) {
        const int64_t want = (work + 255) / 256;
        const unsigned blocks = (unsigned)(want < 152 * 8 ? want : 152 * 8);
        k_sum_leaves<<<blocks, 256, 0, st>>>(job, a->leaves3, a->leaves1);
    }
    k_sum_tree<<<kArrays + (a->ntips > 0 ? 1 : 0), 256, 0, st>>>(
        job, a->volume, a->ntips, a->tip_offsets, a->tip_entries, a->sums);
    return launch_status();
}
