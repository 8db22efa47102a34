// Error reporting and version of the sfem_gb300 C ABI.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace sfem_gb300 {

static thread_local char g_last_error[1024] = "";

int set_error(const char *fmt, ...) {
    va_list args;
    va_start(args, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, args);
    va_end(args);
    return SFEM_GB300_FAILURE;
}

int check_launch(const char *what) {
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        return set_error("%s: CUDA launch failed: %s", what, cudaGetErrorString(err));
    }
    return SFEM_GB300_SUCCESS;
}

}  // namespace sfem_gb300

extern "C" const char *sfem_gb300_last_error(void) { return sfem_gb300::g_last_error; }

extern "C" const char *sfem_gb300_version(void) { return "sfem_gb300 0.1 (sm_103a)"; }
