// noalloc.cu -- UCFDBLUSGS_ResidualNoAlloc: the FP64 residual norm of a
// prepared block LU-SGS system computed without any allocation.
//
// Who needs it: a CFD code that hands its whole device-memory budget to its
// own pool allocator at start-up and forbids allocations afterwards, or one
// whose time-step loop must not stall on cudaMalloc (which can synchronise
// the device), still has to monitor the linear residual every iteration.
// UCFDBLUSGS_Residual grows private reduction buffers on first use; this
// variant keeps its partial sums in a fixed file-scope device array instead
// and calls no cudaMalloc, cudaFree or allocating library routine.
//
// Limits and sharing rules:
//  * the scratch array holds 2 * kMaxBlocks partial sums plus 2 totals
//    (64 KiB); one block covers up to kCellsPerBlock cells, so systems with
//    more than kMaxBlocks * kCellsPerBlock = 8,388,608 cells are rejected
//    (UCFD_ERR_ARGUMENT);
//  * every GPU that loads the library holds this array until the process
//    exits;
//  * all calls share the array and it keeps the last call's contents; every
//    slot a call reads is written by that same call first, so nothing has to
//    start at zero -- but two calls whose kernels overlap on the GPU (e.g.
//    issued on different streams without ordering) race on it;
//  * the call runs on the device that holds the handle's arrays: it makes
//    that device current for its duration and restores the caller's device
//    before returning;
//  * the first call on a device does the set-up: with that device current it
//    looks up the array's device address (cudaGetSymbolAddress) and caches
//    it, so make that first call before any stream capture begins;
//  * like UCFDBLUSGS_Residual the call returns only after the result has
//    been written (it synchronises the handle's stream).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>

#include "../../include/ucfdlusgs.h"
#include "kargs.h"
#include "flowsys_view.h"
#include "ucfd_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 4096;
constexpr int kCellsPerBlock = 2048;  // 8 cells per thread
constexpr long long kMaxCells = (long long)kMaxBlocks * kCellsPerBlock;
constexpr int kMaxDevices = 64;

// 2 partial sums per block (r.r, rhs.rhs) followed by the 2 totals.
static __device__ __align__(256) double g_resid_scratch[2 * kMaxBlocks + 2];

// device address of g_resid_scratch per device, filled on a device's first
// call; concurrent first calls store the same value
std::atomic<double *> g_scratch_addr[kMaxDevices];

// Makes `dev` current for the scope of a call and restores the caller's
// device afterwards (also when the call fails).
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        UCFD_CUDA(cudaGetDevice(&prev));
        if (prev != dev) UCFD_CUDA(cudaSetDevice(dev));
        else prev = -1;
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

__device__ inline double warp_block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// Grid-stride variant of the FP64 residual kernel: per cell
// r = rhs - D x - sum_f J x_nb fv (same per-cell arithmetic; fa == nullptr:
// the blocks are M = D^-1 J fv and r = rhs - D (x + sum_f M x_nb)), per block the
// partial sums of r^2 and rhs^2 go to scratch[2 b], scratch[2 b + 1].
template <typename Sx, int B>
__global__ void __launch_bounds__(kThreads) residual_noalloc_kernel(long long N, int P, const int *nei,
                                                                    const double *fa, const double *rv,
                                                                    const double *J64, const double *D,
                                                                    const double *rhs64, const Sx *x,
                                                                    double *scratch) {
    __shared__ double sh[32];
    constexpr int B2 = B * B;
    double rr = 0.0, bb = 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        double res[B], xk[B], t[B];
#pragma unroll
        for (int c = 0; c < B; ++c) xk[c] = t[c] = (double)x[c * N + k];
#pragma unroll
        for (int r = 0; r < B; ++r) {
            double v = rhs64[r * N + k];
            bb += v * v;
            if (fa) {
#pragma unroll
                for (int c = 0; c < B; ++c) v -= D[::ucfd::tile_index(k, r * B + c, B2)] * xk[c];
            }
            res[r] = v;
        }
        for (int p = 0; p < P; ++p) {
            const int nb = nei[p * N + k];
            if (nb < 0) break;
            const double fv = fa ? fa[p * N + k] * rv[k] : 1.0;
            double xn[B];
#pragma unroll
            for (int c = 0; c < B; ++c) xn[c] = (double)x[c * N + nb];
#pragma unroll
            for (int r = 0; r < B; ++r) {
                double val = 0.0;
#pragma unroll
                for (int c = 0; c < B; ++c)
                    val += J64[::ucfd::tile_index(k, (long long)p * B2 + r * B + c, (long long)P * B2)] * xn[c];
                if (fa) res[r] -= val * fv;
                else t[r] += val;
            }
        }
        if (!fa) {
            // M form: r = rhs - D (x + sum_f M x_nb)
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
                for (int c = 0; c < B; ++c) res[r] -= D[::ucfd::tile_index(k, r * B + c, B2)] * t[c];
        }
#pragma unroll
        for (int r = 0; r < B; ++r) rr += res[r] * res[r];
    }
    rr = warp_block_sum(rr, sh);
    bb = warp_block_sum(bb, sh);
    if (threadIdx.x == 0) {
        scratch[2 * blockIdx.x] = rr;
        scratch[2 * blockIdx.x + 1] = bb;
    }
}

// Totals of the nb partial pairs into scratch[2 kMaxBlocks + {0, 1}]; with
// out != nullptr also writes the relative residual there (device output).
__global__ void __launch_bounds__(1024) residual_noalloc_total_kernel(int nb, double *scratch, double *out) {
    __shared__ double sh[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        a += scratch[2 * i];
        b += scratch[2 * i + 1];
    }
    a = warp_block_sum(a, sh);
    b = warp_block_sum(b, sh);
    if (threadIdx.x == 0) {
        scratch[2 * kMaxBlocks] = a;
        scratch[2 * kMaxBlocks + 1] = b;
        if (out) {
            const double rn = sqrt(a), bn = sqrt(b);
            *out = bn > 0 ? rn / bn : rn;
        }
    }
}

template <typename Sx>
void launch(const ucfd::BlockSystemView &v, const Sx *x, double *scratch, int nb, cudaStream_t s) {
    switch (v.B) {
        case 4:
            residual_noalloc_kernel<Sx, 4><<<nb, kThreads, 0, s>>>(v.N, v.P, v.nei, v.fa, v.rv, v.J64, v.D, v.rhs64, x,
                                                                    scratch);
            break;
        case 5:
            residual_noalloc_kernel<Sx, 5><<<nb, kThreads, 0, s>>>(v.N, v.P, v.nei, v.fa, v.rv, v.J64, v.D, v.rhs64, x,
                                                                    scratch);
            break;
        default:
            ucfd::fail(UCFD_ERR_UNSUPPORTED, "UCFDBLUSGS_ResidualNoAlloc: block size %d not built (4 or 5)", v.B);
    }
}

}  // namespace

extern "C" ucfd_status_t UCFDBLUSGS_ResidualNoAlloc(FlowSys sys, UCFDReal *relres) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(sys && relres, "UCFDBLUSGS_ResidualNoAlloc: null argument");
    ucfd::BlockSystemView v;
    if (!ucfd::flowsys_block_view(sys, v))
        ucfd::fail(UCFD_ERR_STATE, "UCFDBLUSGS_ResidualNoAlloc: the block system must be packed and prepared first "
                                   "(UCFDBLUSGS_Pack + UCFDBLUSGS_NSPrepare)");
    UCFD_REQUIRE(v.N <= kMaxCells,
                 "UCFDBLUSGS_ResidualNoAlloc: %lld cells exceed the fixed scratch capacity of %lld cells "
                 "(use UCFDBLUSGS_Residual)", v.N, kMaxCells);
    // the device that holds the handle's prepared arrays
    cudaPointerAttributes pa{};
    UCFD_CUDA(cudaPointerGetAttributes(&pa, v.D));
    const int dev = pa.device;
    UCFD_REQUIRE(pa.type == cudaMemoryTypeDevice && dev >= 0 && dev < kMaxDevices,
                 "UCFDBLUSGS_ResidualNoAlloc: the handle's arrays are not on a CUDA device below %d", kMaxDevices);
    DeviceScope on(dev);
    if (!g_scratch_addr[dev].load(std::memory_order_acquire)) {
        // set-up, once per device, with that device current
        void *p = nullptr;
        UCFD_CUDA(cudaGetSymbolAddress(&p, g_resid_scratch));
        g_scratch_addr[dev].store((double *)p, std::memory_order_release);
    }
    double *scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
    cudaStream_t s = (cudaStream_t)v.stream;
    const int nb = (int)((v.N + kCellsPerBlock - 1) / kCellsPerBlock);
    if (v.x64) launch<double>(v, v.x64, scratch, nb, s);
    else launch<float>(v, v.x32, scratch, nb, s);
    const bool out_dev = ucfd::is_device_ptr(relres);
    residual_noalloc_total_kernel<<<1, 1024, 0, s>>>(nb, scratch, out_dev ? relres : nullptr);
    UCFD_CHECK_LAUNCH();
    if (!out_dev) {
        double tot[2];
        UCFD_CUDA(cudaMemcpyAsync(tot, scratch + 2 * kMaxBlocks, sizeof(tot), cudaMemcpyDeviceToHost, s));
        UCFD_CUDA(cudaStreamSynchronize(s));
        const double rn = std::sqrt(tot[0]), bn = std::sqrt(tot[1]);
        *relres = bn > 0 ? rn / bn : rn;
    } else {
        UCFD_CUDA(cudaStreamSynchronize(s));
    }
    UCFD_API_END
}
