// flowsys_view.h -- read-only view of a prepared FlowSys block system, for
// entry points that compute on it without touching its allocations.
#pragma once

#include "../../include/ucfdlusgs.h"

namespace ucfd {

struct BlockSystemView {
    long long N = 0;        // internal cells
    int P = 0;              // ELL width
    int B = 0;              // NS block size (nfvars)
    const int *nei = nullptr;
    // fa == nullptr: J64 holds M = D^-1 J fa rv (the FP64 fused multiply-add
    // mode's sweep blocks); the residual is then rhs - D (x + sum_f M x_nb)
    const double *fa = nullptr, *rv = nullptr, *J64 = nullptr, *D = nullptr, *rhs64 = nullptr;
    const double *x64 = nullptr;  // current increment (FP64), or
    const float *x32 = nullptr;   // current increment (FP32 sweeps)
    void *stream = nullptr;       // cudaStream_t of the handle
};

// Fills v for a FlowSys whose BLU-SGS system has been packed and prepared;
// returns false (and leaves v untouched) otherwise.  Never allocates.
bool flowsys_block_view(FlowSys s, BlockSystemView &v);

}  // namespace ucfd
