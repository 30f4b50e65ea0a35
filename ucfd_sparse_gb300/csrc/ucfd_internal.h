// ucfd_internal.h -- host-side runtime shared by the C-ABI translation units:
// error reporting, device buffers, host/device pointer detection, staging.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ucfd_gb300.h"

namespace ucfd {

// ---- errors -----------------------------------------------------------------
void set_error(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
void clear_error();

struct Error {
    ucfd_status_t st;
};

// Throwing helpers used inside the library; every C entry point catches and
// converts to a status (see UCFD_API_BEGIN / UCFD_API_END).
[[noreturn]] void fail(ucfd_status_t st, const char *fmt, ...) __attribute__((format(printf, 2, 3)));

inline void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
    if (e != cudaSuccess) fail(UCFD_ERR_CUDA, "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
}
#define UCFD_CUDA(call) ::ucfd::cuda_check((call), #call, __FILE__, __LINE__)
#define UCFD_CHECK_LAUNCH() ::ucfd::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)
#define UCFD_REQUIRE(cond, ...) \
    do { if (!(cond)) ::ucfd::fail(UCFD_ERR_ARGUMENT, __VA_ARGS__); } while (0)

#define UCFD_API_BEGIN try { ::ucfd::clear_error();
#define UCFD_API_END                                                       \
    }                                                                      \
    catch (const ::ucfd::Error &e) { return e.st; }                        \
    catch (const std::bad_alloc &) {                                       \
        ::ucfd::set_error("host allocation failed");                       \
        return UCFD_ERR_NOMEM;                                             \
    }                                                                      \
    catch (...) {                                                          \
        ::ucfd::set_error("unexpected exception");                         \
        return UCFD_FAILED;                                                \
    }                                                                      \
    return UCFD_SUCCESS;

// ---- device buffers ---------------------------------------------------------
// Owning, growable device allocation.  Never shrinks; realloc discards data.
// Host -> device / device -> host copy of `bytes` on stream s
// (cudaMemcpyAsync), counted and, while UCFDSetTransferTiming is on, timed.
void copy_h2d(void *dst, const void *src, size_t bytes, cudaStream_t s);
void copy_d2h(void *dst, const void *src, size_t bytes, cudaStream_t s);

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    T *ensure(size_t count) {
        if (count <= n && p) return p;
        release();
        size_t bytes = (count ? count : 1) * sizeof(T);
        cudaError_t e = cudaMalloc((void **)&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            fail(UCFD_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        }
        n = count;
        return p;
    }
    void upload(const T *host, size_t count, cudaStream_t s) {
        ensure(count);
        if (count) copy_h2d(p, host, count * sizeof(T), s);
    }
    void zero(size_t count, cudaStream_t s) {
        ensure(count);
        if (count) UCFD_CUDA(cudaMemsetAsync(p, 0, count * sizeof(T), s));
    }
};

// Pinned host staging buffer.
template <typename T>
struct PinnedBuf {
    T *p = nullptr;
    size_t n = 0;
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
    T *ensure(size_t count) {
        if (count <= n && p) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        UCFD_CUDA(cudaMallocHost((void **)&p, (count ? count : 1) * sizeof(T)));
        n = count;
        return p;
    }
};

// ---- pointer kinds ----------------------------------------------------------
// Under UCFD_HOST_MAP (UCFDSetHostArrayAccess): the device address of
// page-locked host memory (pinned or registered), which kernels can read in
// place over the host link; otherwise nullptr (stage the array instead).
const void *host_mapped(const void *ptr);

// True when the GPU can dereference ptr directly (device or managed memory).
bool is_device_ptr(const void *ptr);

// View of a caller array on the device: the caller's pointer when it is
// device memory, otherwise a staged copy in `stage`.
template <typename T>
const T *device_view(const T *ptr, size_t count, DevBuf<T> &stage, cudaStream_t s) {
    if (!ptr) return nullptr;
    if (is_device_ptr(ptr)) return ptr;
    stage.upload(ptr, count, s);
    return stage.p;
}

// Copy of a caller array (host or device) into host memory.
template <typename T>
void to_host(const T *ptr, size_t count, std::vector<T> &out) {
    out.resize(count);
    if (!count) return;
    if (is_device_ptr(ptr))
        UCFD_CUDA(cudaMemcpy(out.data(), ptr, count * sizeof(T), cudaMemcpyDeviceToHost));
    else
        std::memcpy(out.data(), ptr, count * sizeof(T));
}

// Process-wide device setup: selects the current device once and returns its SM count.
int sm_count();
int ensure_device();

// Gas constants (flux.h:18-26 defaults).
struct Constants {
    double gamma = 1.4, pmin = 1e-13, betast = 0.09;
};
Constants &constants();

}  // namespace ucfd
