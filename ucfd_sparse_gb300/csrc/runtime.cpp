// runtime.cpp -- error reporting, device selection, pointer kinds, constants.
#include <cstdarg>
#include <atomic>
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

// ---- timed host<->device copies (UCFDSetTransferTiming) ------------------
namespace {
std::mutex g_xfer_mu;
bool g_xfer_on = false;
UCFDTransferStats g_xfer{};

void timed_copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    bool on;
    {
        std::lock_guard<std::mutex> lk(g_xfer_mu);
        on = g_xfer_on;
    }
    if (!on) {
        UCFD_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, s));
        return;
    }
    thread_local cudaEvent_t ev[2] = {nullptr, nullptr};
    if (!ev[0]) {
        UCFD_CUDA(cudaEventCreate(&ev[0]));
        UCFD_CUDA(cudaEventCreate(&ev[1]));
    }
    UCFD_CUDA(cudaEventRecord(ev[0], s));
    UCFD_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, s));
    UCFD_CUDA(cudaEventRecord(ev[1], s));
    UCFD_CUDA(cudaEventSynchronize(ev[1]));
    float ms = 0.f;
    UCFD_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    std::lock_guard<std::mutex> lk(g_xfer_mu);
    if (kind == cudaMemcpyHostToDevice) {
        g_xfer.h2d_ms += ms;
        g_xfer.h2d_bytes += (double)bytes;
        g_xfer.h2d_copies++;
    } else {
        g_xfer.d2h_ms += ms;
        g_xfer.d2h_bytes += (double)bytes;
        g_xfer.d2h_copies++;
    }
}
}  // namespace

void copy_h2d(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    timed_copy(dst, src, bytes, cudaMemcpyHostToDevice, s);
}
void copy_d2h(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    timed_copy(dst, src, bytes, cudaMemcpyDeviceToHost, s);
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

namespace {
std::atomic<int> g_host_access{UCFD_HOST_MAP};
}

const void *host_mapped(const void *ptr) {
    if (!ptr || g_host_access.load(std::memory_order_relaxed) != UCFD_HOST_MAP) return nullptr;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
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

ucfd_status_t UCFDSetTransferTiming(int on) {
    UCFD_API_BEGIN
    std::lock_guard<std::mutex> lk(ucfd::g_xfer_mu);
    if (on) ucfd::g_xfer = UCFDTransferStats{};
    ucfd::g_xfer_on = on != 0;
    UCFD_API_END
}

ucfd_status_t UCFDSetHostArrayAccess(int mode) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mode == UCFD_HOST_STAGE || mode == UCFD_HOST_MAP,
                 "host array access must be UCFD_HOST_STAGE (0) or UCFD_HOST_MAP (1), got %d", mode);
    ucfd::g_host_access.store(mode, std::memory_order_relaxed);
    UCFD_API_END
}

int UCFDGetHostArrayAccess(void) { return ucfd::g_host_access.load(std::memory_order_relaxed); }

ucfd_status_t UCFDGetTransferStats(UCFDTransferStats *stats) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(stats, "UCFDGetTransferStats: null argument");
    std::lock_guard<std::mutex> lk(ucfd::g_xfer_mu);
    *stats = ucfd::g_xfer;
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
