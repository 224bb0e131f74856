// pp_static.cu -- fused steps that allocate nothing (pp_fused_run_static).
//
// For callers that cannot allocate device memory: the only device memory
// this path needs beyond the caller's simulation arrays -- the device copy
// of the boundary-condition magnitude schedule, and, for the mixed step,
// the running max |u| and the status word -- lives in one file-scope
// __device__ array, loaded with the library and kept until exit.  Its
// device address is looked up once per device (cudaGetSymbolAddress, with
// that device current) by the first call on that device.  All calls share
// the array and leave their contents in it; calls whose work overlaps on
// the GPU race on it.
#include <mutex>

#include "pp_fused.cuh"

namespace pp {
namespace {

struct StaticScratch {
    double mags[2 * PP_STATIC_MAX_STEPS];  // displacement, then force magnitudes
    float umax;                            // running max |u| (PP_MIXED)
    int32_t status;                        // PP_STATUS_* of the last call
};

__device__ __align__(256) StaticScratch g_static_scratch;

constexpr int kMaxDevices = 64;
StaticScratch* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of g_static_scratch on the current device (looked up once).
int scratch_address(StaticScratch** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PP_ERROR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PP_ERROR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return PP_ERROR_CUDA;
        g_scratch_addr[dev] = static_cast<StaticScratch*>(p);
    }
    *out = g_scratch_addr[dev];
    return PP_SUCCESS;
}

__global__ void k_reset_words(StaticScratch* s) {
    s->umax = 0.0f;
    s->status = PP_STATUS_OK;
}

// Running max |u| of the state: max over nodes of the gathered max|u|
// (the .w of each displacement record), as the mixed step maintains it.
__global__ void k_umax_of_state(const float* __restrict__ rec, int nnodes, StaticScratch* s) {
    float m = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnodes; i += gridDim.x * blockDim.x)
        m = fmaxf(m, rec[8 * (int64_t)i + 7]);
    const int w = __reduce_max_sync(kFull, __float_as_int(m));
    if ((threadIdx.x & 31) == 0 && w > 0) atomicMax(reinterpret_cast<int*>(&s->umax), w);
}

}  // namespace
}  // namespace pp

using namespace pp;

extern "C" int pp_fused_run_static(const pp_fused_args* args, int32_t parity, int64_t nsteps,
                                   const double* disp_mags, const double* force_mags,
                                   void* stream) {
    if (!args || (parity != 0 && parity != 1) || nsteps < 0) return PP_ERROR_INVALID_VALUE;
    if (nsteps > PP_STATIC_MAX_STEPS) return PP_ERROR_TOO_LARGE;
    if (nsteps > 0 && (!disp_mags || !force_mags)) return PP_ERROR_INVALID_VALUE;
    StaticScratch* s = nullptr;
    int rc = scratch_address(&s);
    if (rc != PP_SUCCESS) return rc;
    pp_fused_args a = *args;
    if (a.precision == PP_MIXED) {
        a.umax = &s->umax;
        a.status = &s->status;
    }
    rc = validate_fused(a);
    if (rc != PP_SUCCESS) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_reset_words<<<1, 1, 0, st>>>(s);
    if (launch_status() != PP_SUCCESS) return PP_ERROR_CUDA;
    if (a.nnodes == 0 || nsteps == 0) return PP_SUCCESS;
    const size_t bytes = (size_t)nsteps * sizeof(double);
    if (cudaMemcpyAsync(s->mags, disp_mags, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(s->mags + PP_STATIC_MAX_STEPS, force_mags, bytes, cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
        return PP_ERROR_CUDA;
    if (a.precision == PP_MIXED) {
        const int blocks = (a.nnodes + 255) / 256 < 1024 ? (a.nnodes + 255) / 256 : 1024;
        k_umax_of_state<<<blocks, 256, 0, st>>>(a.rec[parity], a.nnodes, s);
        if (launch_status() != PP_SUCCESS) return PP_ERROR_CUDA;
    }
    int p = parity;
    for (int64_t k = 0; k < nsteps; ++k) {
        const Launch l{0.0, 0.0, s->mags, s->mags + PP_STATIC_MAX_STEPS, nullptr, k};
        rc = launch_fused_step(a, p, l, st);
        if (rc != PP_SUCCESS) return rc;
        p ^= 1;
    }
    return PP_SUCCESS;
}

extern "C" int pp_static_status(int32_t* status, void* stream) {
    if (!status) return PP_ERROR_INVALID_VALUE;
    StaticScratch* s = nullptr;
    const int rc = scratch_address(&s);
    if (rc != PP_SUCCESS) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(status, &s->status, sizeof(int32_t), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PP_ERROR_CUDA;
    return PP_SUCCESS;
}
