// runtime.cpp -- error reporting, device selection, pointer kinds, constants.
#include <cstdarg>
#include <mutex>

#include "ucfd_internal.h"

namespace ucfd {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

void fail(ucfd_status_t st, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    throw Error{st};
}

static std::once_flag g_dev_once;
static int g_sm_count = 0;
static cudaError_t g_dev_err = cudaSuccess;

int ensure_device() {
    std::call_once(g_dev_once, [] {
        int dev = 0;
        g_dev_err = cudaGetDevice(&dev);
        if (g_dev_err == cudaSuccess) g_dev_err = cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_dev_err != cudaSuccess) cudaGetLastError();
    });
    if (g_dev_err != cudaSuccess)
        fail(UCFD_ERR_CUDA, "no usable CUDA device: %s", cudaGetErrorString(g_dev_err));
    return 0;
}

int sm_count() {
    ensure_device();
    return g_sm_count;
}

bool is_device_ptr(const void *ptr) {
    if (!ptr) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

Constants &constants() {
    static Constants c;
    return c;
}

}  // namespace ucfd

extern "C" {

const char *UCFDGetLastError(void) { return ucfd::g_last_error.c_str(); }

ucfd_status_t UCFDSetConstants(UCFDReal gamma, UCFDReal pmin, UCFDReal betast) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(gamma > 1.0, "gamma must exceed 1 (got %g)", gamma);
    ucfd::constants().gamma = gamma;
    ucfd::constants().pmin = pmin;
    ucfd::constants().betast = betast;
    UCFD_API_END
}

const char *UCFDVersion(void) { return "ucfd_gb300 1.0 (sm_103a)"; }

ucfd_status_t UCFDDeviceInfo(char *name, size_t len, int *sm) {
    UCFD_API_BEGIN
    ucfd::ensure_device();
    int dev = 0;
    UCFD_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    UCFD_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (name && len) {
        std::strncpy(name, prop.name, len - 1);
        name[len - 1] = 0;
    }
    if (sm) *sm = prop.multiProcessorCount;
    UCFD_API_END
}

}  // extern "C"
