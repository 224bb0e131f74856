// pp_static.cu -- fused steps that allocate nothing (pp_fused_run_static).
//
// For callers that cannot allocate device memory: the only device memory
// this path needs beyond the caller's simulation arrays -- the device copy
// of the boundary-condition magnitude schedule, and, for the mixed step,
// the running max |u| and the status word -- lives in one file-scope
// __device__ array, loaded with the library and kept until exit.  Its
// device address is looked up (cudaGetSymbolAddress, with the device
// current) by the first call in each CUDA context: the address is cached
// per device together with the context's unique ID (cuCtxGetId), so a
// device reset or a re-created primary context makes the next call look it
// up again.  All calls share the array and leave their contents in it;
// calls whose work overlaps on the GPU race on it.
#include <cuda.h>  // CUcontext, CUresult (the driver calls go through entry points)

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
struct CachedAddress {
    unsigned long long ctx_id;  // cuCtxGetId of the context it belongs to
    StaticScratch* addr;
};
CachedAddress g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique ID of the current context (0 when there is none yet).
int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_current || !get_id) return PP_ERROR_CUDA;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS) return PP_ERROR_CUDA;
    *id = 0;
    if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return PP_ERROR_CUDA;
    return PP_SUCCESS;
}

// Device address of g_static_scratch in the current context (looked up by
// the first call in each context).
int scratch_address(StaticScratch** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PP_ERROR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PP_ERROR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc != PP_SUCCESS) return rc;
    CachedAddress& c = g_scratch_addr[dev];
    if (id == 0 || !c.addr || c.ctx_id != id) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return PP_ERROR_CUDA;
        // the lookup makes the primary context current if none was
        rc = current_context_id(&id);
        if (rc != PP_SUCCESS || id == 0) return PP_ERROR_CUDA;
        c.addr = static_cast<StaticScratch*>(p);
        c.ctx_id = id;
    }
    *out = c.addr;
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
