// kern_gm.cu -- the GMRES orthogonalisation kernels (FMA contraction on),
// one instantiation per vector count, in a translation unit of their own so
// that they compile in parallel with the rest.  The kernel headers are
// compiled here in a namespace of their own (their non-template kernels are
// also defined in kern_fast.cu); kfast::gm_dots / gm_update forward to it.
#define UCFD_KNS kfast_gm
#include "gm_launchers.cuh"

namespace kfast {
void gm_dots(long long n, int K, const double *V, long long ldv, const double *w, double *part, cudaStream_t s) {
    kfast_gm::gm_dots(n, K, V, ldv, w, part, s);
}
void gm_update(long long n, int K, const double *V, long long ldv, const double *h, double *w, int mode,
               double *part, cudaStream_t s) {
    kfast_gm::gm_update(n, K, V, ldv, h, w, mode, part, s);
}
}  // namespace kfast
