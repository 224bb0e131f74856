// pp_corrections.cu -- per-bond stiffness correction factors on the GPU:
// the conical micromodulus function, the partial-volume (HHB) correction and
// the volume-method surface correction of peripy/correction.pyx:5-277, as
// Model.__init__ applies them (peripy/model.py:349-375): each factor
// multiplies the (nnodes, max_neigh) correction array in that order.
//
// The reference visits each pair once, from its lower node a to b > a: it
// multiplies the slot (a -> b) and the first slot (b -> a) of b's row.  So
// here a slot (i -> j) takes the pair's factor when i < j, or when i > j and
// it is the first slot of i's row that holds j and j's row holds i.  The
// factors depend on the pair only (the distance and the sum of the family
// volumes are symmetric), computed in binary64 in the reference's order:
//   l0 = sqrt((dx*dx + dy*dy) + dz*dz), d = r0[b] - r0[a]   (spatial.pyx:20-31)
//   conical:        (h - l0) / h for l0 <= h, else 0           (:268-277)
//   partial volume: 1 for l0 <= H - R, (H + R - l0) / (2 R) for l0 <= H + R,
//                   else 0                                       (:159-176)
//   surface:        2 V_bulk / (V_a + V_b), V the family volume  (:5-108)
// Only the first n_neigh[i] slots of each row are bonds.
#include "pp_common.cuh"

namespace pp {
namespace {

__device__ __forceinline__ double pair_length(const double* __restrict__ r, int a, int b) {
    const double dx = __dsub_rn(r[3 * (int64_t)b], r[3 * (int64_t)a]);
    const double dy = __dsub_rn(r[3 * (int64_t)b + 1], r[3 * (int64_t)a + 1]);
    const double dz = __dsub_rn(r[3 * (int64_t)b + 2], r[3 * (int64_t)a + 2]);
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// Family volume of each node: the volumes of its bonds' far ends, summed in
// slot order (correction.pyx:88-94), or n_neigh * average volume.
__global__ void k_family_volume(pp_corrections_args a, double* __restrict__ fv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nnodes) return;
    const int nn = a.n_neigh[i];
    if (a.surface_correction == 0) {
        fv[i] = __dmul_rn((double)nn, a.average_volume);
        return;
    }
    double t = 0.0;
    const int32_t* row = a.nlist + (int64_t)i * a.max_neigh;
    for (int s = 0; s < nn; ++s) t = __dadd_rn(t, a.volume[row[s]]);
    fv[i] = t;
}

__device__ __forceinline__ bool row_holds(const pp_corrections_args& a, int i, int j, int upto) {
    const int32_t* row = a.nlist + (int64_t)i * a.max_neigh;
    for (int s = 0; s < upto; ++s)
        if (row[s] == j) return true;
    return false;
}

// One thread per slot.
__global__ void k_corrections(pp_corrections_args a, const double* __restrict__ fv) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= (int64_t)a.nnodes * a.max_neigh) return;
    const int i = (int)(g / a.max_neigh);
    const int s = (int)(g % a.max_neigh);
    if (s >= a.n_neigh[i]) return;
    const int j = a.nlist[g];
    if (j < 0 || j >= a.nnodes || j == i) return;
    if (j < i) {
        // the reference reaches this slot from j's row: only the first slot
        // of i's row holding j, and only when j's row holds i
        if (row_holds(a, i, j, s)) return;
        if (!row_holds(a, j, i, a.n_neigh[j])) return;
    }
    const int lo = min(i, j), hi = max(i, j);
    double c = a.corrections[g];
    if (a.micromodulus_function == 0 || a.volume_correction == 0) {
        const double l0 = pair_length(a.r0, lo, hi);
        if (a.micromodulus_function == 0) {
            const double h = a.micromodulus_horizon;
            c = __dmul_rn(c, l0 <= h ? __ddiv_rn(__dsub_rn(h, l0), h) : 0.0);
        }
        if (a.volume_correction == 0) {
            const double H = a.vc_horizon, R = a.vc_node_radius;
            double f;
            if (l0 <= __dsub_rn(H, R))
                f = 1.0;
            else if (l0 <= __dadd_rn(H, R))
                f = __ddiv_rn(__dsub_rn(__dadd_rn(H, R), l0), __dmul_rn(2.0, R));
            else
                f = 0.0;
            c = __dmul_rn(c, f);
        }
    }
    if (a.surface_correction == 0 || a.surface_correction == 1)
        c = __dmul_rn(c, __ddiv_rn(__dmul_rn(2.0, a.family_volume_bulk), __dadd_rn(fv[lo], fv[hi])));
    a.corrections[g] = c;
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_stiffness_corrections(const pp_corrections_args* args, void* stream) {
    if (!args) return PP_ERROR_INVALID_VALUE;
    const pp_corrections_args& a = *args;
    if (a.nnodes < 0 || a.max_neigh < 1 || a.reserved != 0) return PP_ERROR_INVALID_VALUE;
    if (a.micromodulus_function < -1 || a.micromodulus_function > 0 ||
        a.volume_correction < -1 || a.volume_correction > 0 || a.surface_correction < -1 ||
        a.surface_correction > 1)
        return PP_ERROR_INVALID_VALUE;
    if (a.nnodes == 0) return PP_SUCCESS;
    if (!a.nlist || !a.n_neigh || !a.corrections) return PP_ERROR_INVALID_VALUE;
    if ((a.micromodulus_function == 0 || a.volume_correction == 0) && !a.r0)
        return PP_ERROR_INVALID_VALUE;
    const bool surface = a.surface_correction >= 0;
    if (surface && (!a.family_volume || (a.surface_correction == 1 && !a.volume)))
        return PP_ERROR_INVALID_VALUE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (surface) k_family_volume<<<(a.nnodes + 255) / 256, 256, 0, st>>>(a, a.family_volume);
    const int64_t slots = (int64_t)a.nnodes * a.max_neigh;
    k_corrections<<<(unsigned)((slots + 255) / 256), 256, 0, st>>>(a, a.family_volume);
    return launch_status();
}
