// pp_host.cu -- page-locking of caller host arrays for the write-step copies.
//
// The library links its own (static) CUDA runtime, so a failed registration
// leaves its error in this runtime, where it is cleared here, and not in the
// runtime of the caller (torch's, for the Python integrators), whose next
// launch check would otherwise report it at an unrelated call.  The pages
// are registered with the device's primary context, which every runtime in
// the process shares, so copies issued by the caller's runtime see them as
// page-locked.
#include "pp_common.cuh"

extern "C" int pp_host_register(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return PP_ERROR_INVALID_VALUE;
    if (cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) != cudaSuccess) {
        (void)cudaGetLastError();  // non-sticky: clear it
        return PP_ERROR_CUDA;
    }
    return PP_SUCCESS;
}

extern "C" int pp_host_unregister(void* ptr) {
    if (!ptr) return PP_ERROR_INVALID_VALUE;
    if (cudaHostUnregister(ptr) != cudaSuccess) {
        (void)cudaGetLastError();
        return PP_ERROR_CUDA;
    }
    return PP_SUCCESS;
}
