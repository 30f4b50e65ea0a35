// gm_launchers.cuh -- launchers of the GMRES orthogonalisation kernels
// (gm_dots_kernel, gm_update_kernel), compiled in a translation unit of
// their own (kern_gm.cu): one kernel per vector count makes them the
// longest part of the build.
#pragma once

#include "launch.h"
#include "kernels_krylov.cuh"
#include "ucfd_internal.h"

namespace UCFD_KNS {

// The orthogonalisation kernels run every product of the compiled bound KM
// (entries past K read as zero), and their FP64 pipe is what bounds them; so
// K up to 16 gets a kernel of its own (KM = K) and larger K the next multiple
// of 8 (the chunk the dots kernel walks V in).
#define UCFD_GM_SWITCH(K, CALL)                                                                       \
    switch (K) {                                                                                     \
        case 1: { constexpr int KM = 1; CALL; break; }    case 2: { constexpr int KM = 2; CALL; break; }   \
        case 3: { constexpr int KM = 3; CALL; break; }    case 4: { constexpr int KM = 4; CALL; break; }   \
        case 5: { constexpr int KM = 5; CALL; break; }    case 6: { constexpr int KM = 6; CALL; break; }   \
        case 7: { constexpr int KM = 7; CALL; break; }    case 8: { constexpr int KM = 8; CALL; break; }   \
        case 9: { constexpr int KM = 9; CALL; break; }    case 10: { constexpr int KM = 10; CALL; break; } \
        case 11: { constexpr int KM = 11; CALL; break; }  case 12: { constexpr int KM = 12; CALL; break; } \
        case 13: { constexpr int KM = 13; CALL; break; }  case 14: { constexpr int KM = 14; CALL; break; } \
        case 15: { constexpr int KM = 15; CALL; break; }  case 16: { constexpr int KM = 16; CALL; break; } \
        default:                                                                                     \
            if (K <= 24) { constexpr int KM = 24; CALL; }                                            \
            else { constexpr int KM = 32; CALL; }                                                    \
    }

void gm_dots(long long n, int K, const double *V, long long ldv, const double *w, double *part,
             cudaStream_t s) {
    if (K < 1 || K > kMaxK) ::ucfd::fail(UCFD_ERR_ARGUMENT, "gm_dots: %d vectors (1..%d)", K, kMaxK);
    const int g = gm_grid(n);
    UCFD_GM_SWITCH(K, (gm_dots_kernel<KM><<<g, kBlock, 0, s>>>(n, K, V, ldv, w, part)));
}

void gm_update(long long n, int K, const double *V, long long ldv, const double *h, double *w, int mode,
               double *part, cudaStream_t s) {
    if (K < 1 || K > kMaxK) ::ucfd::fail(UCFD_ERR_ARGUMENT, "gm_update: %d vectors (1..%d)", K, kMaxK);
    const int g = gm_grid(n);
    UCFD_GM_SWITCH(K, (gm_update_kernel<KM><<<g, kBlock, 0, s>>>(n, K, V, ldv, h, w, mode, part)));
}
#undef UCFD_GM_SWITCH

}  // namespace UCFD_KNS
