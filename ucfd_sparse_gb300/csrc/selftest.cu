// selftest.cu -- UCFDSelfTestTimeouts: shows on the device that the two
// kinds of bounded wait used by the sweeps give up and report instead of
// hanging.
//
//  * the grid barrier of the persistent scalar sweep (grid_barrier_bounded):
//    its arrival counter starts far above the grid size, so the last
//    arrival that would release the barrier never comes;
//  * the mbarrier wait of the bulk-copy block sweep
//    (ucfd::dev::mbar_wait_bounded): a fresh barrier expecting one arrival
//    that nobody makes and no copy.
//
// Both waits run out after a few thousand polls, set their error flag and
// return; the kernels end normally and the context stays usable.  Nothing
// faults: every access is in bounds and nothing waits without a limit.
#define UCFD_KNS kselftest
#include "kernels_lusgs.cuh"
#include "ucfd_internal.h"

namespace {

__global__ void barrier_timeout_kernel(unsigned *bar, int *err, long long max_spin, int *released) {
    const bool ok = kselftest::grid_barrier_bounded(bar, bar + 1, err, max_spin);
    if (threadIdx.x == 0 && ok) atomicAdd(released, 1);
}

__global__ void mbarrier_timeout_kernel(int *err, long long max_spin) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        ::ucfd::dev::mbar_init(&bar, 1);
        ::ucfd::dev::fence_mbar_init();
    }
    __syncthreads();
    const bool done = ::ucfd::dev::mbar_wait_bounded(&bar, 0, max_spin);
    if (!done && threadIdx.x == 0) atomicExch(err, 1);
}

}  // namespace

extern "C" {

ucfd_status_t UCFDSelfTestTimeouts(int *barrier_timed_out, int *mbarrier_timed_out) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(barrier_timed_out && mbarrier_timed_out, "null argument");
    ucfd::ensure_device();
    ucfd::DevBuf<unsigned> bar;
    ucfd::DevBuf<int> flags;
    const unsigned init[2] = {1000000u, 0u};  // arrivals already far past the grid size
    bar.upload(init, 2, nullptr);
    flags.zero(3, nullptr);
    constexpr long long kSpin = 2000;
    barrier_timeout_kernel<<<2, 64>>>(bar.p, flags.p, kSpin, flags.p + 2);
    UCFD_CHECK_LAUNCH();
    mbarrier_timeout_kernel<<<1, 32>>>(flags.p + 1, kSpin);
    UCFD_CHECK_LAUNCH();
    int h[3] = {0, 0, 0};
    UCFD_CUDA(cudaMemcpy(h, flags.p, sizeof(h), cudaMemcpyDeviceToHost));
    *barrier_timed_out = (h[0] == 1 && h[2] == 0) ? 1 : 0;
    *mbarrier_timed_out = h[1] == 1 ? 1 : 0;
    UCFD_API_END
}

}  // extern "C"
