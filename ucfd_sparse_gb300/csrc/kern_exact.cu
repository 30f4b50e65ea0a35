// kern_exact.cu -- FP64 kernels built with -fmad=false: no multiply-add
// contraction, so each cell's arithmetic is the reference's operation by
// operation (IEEE-rounded division and multiply/add, same order).
#define UCFD_KNS kexact
#define UCFD_KEXACT 1
#include "launchers.cuh"

namespace kexact {
template void scalar_sweep<double>(const ::ucfd::ScalarSweepArgs<double> &, int, int, int, int, int, cudaStream_t);
template void scalar_sweep_persistent<double>(const ::ucfd::ScalarSweepArgs<double> &, int, int, int, int,
                                              const int *, int, unsigned *, int *, long long, cudaStream_t);
template void legacy_pre<double>(int, int, double, const double *, const double *, double *, const double *, cudaStream_t);
template void legacy_update<double>(int, int, int, double *, const double *, cudaStream_t);
template void fs_lusgs_pack<double>(int, int, int, long long, double, double, const int *, const int *, const double *,
                                    const double *, const double *, const double *, double *, double *, double *, cudaStream_t);
template void fs_lusgs_update<double>(int, int, long long, const int *, const int *, const double *, double *, int, cudaStream_t);
template void fs_lusgs_prepare<double>(long long, int, int, int, double, const int *, const double *, const double *,
                                       const double *, const double *, double *, cudaStream_t);
template void fs_lusgs_prepare_both<double>(long long, int, int, int, double, const int *, const double *,
                                            const double *, const double *, const double *, const double *,
                                            double *, cudaStream_t);
template void gather_idx<double>(long long, const int *, const double *, double *, cudaStream_t);
template void fs_blusgs_pack<double>(int, int, int, long long, double, const int *, const int *, const double *,
                                     const double *, double *, double *, double *, cudaStream_t);
template void fs_blusgs_prepare<double>(int, long long, int, long long, const int *, const int *, const int8_t *,
                                        const double *, const double *, const double *, const double *, double *,
                                        double *, double *, double *, double *, double *, cudaStream_t);
template void fs_blusgs_sweep<double>(int, int, int, long long, int, int, const int *, const double *, const double *,
                                      const double *, const double *, const double *, double *, int, int,
                                      int *, long long,
                                      const ::ucfd::SweepSplit<double> &, cudaStream_t);
template void fs_blusgs_residual<double, double>(int, long long, int, int, int, const int *, const double *,
                                                 const double *, const double *, const double *, const double *,
                                                 const double *, double *, double *, int, int *, cudaStream_t);
template void fs_blusgs_subres<double>(int, int, long long, const int *, const int *, const double *, const double *,
                                       double *, double *, cudaStream_t);
template void fs_blusgs_update<double>(int, int, long long, const int *, const int *, const double *, double *, cudaStream_t);
template void bsr_spmv<double, double>(int, int, int, const int *, const double *, double, const double *, double,
                                       double *, int, cudaStream_t);
template void pc_prepare<double>(int, int, const int *, const long long *, const double *, double *, double *, int,
                                 cudaStream_t);
template void pc_lower<double>(int, int, int, int, int, const int *, const double *, const double *, double *, int,
                               int, cudaStream_t);
template void pc_upper<double>(int, int, int, int, int, const int *, const double *, const double *, double *, int,
                               int, cudaStream_t);
template void gather_rows<double, double>(int, int, const int *, const double *, double *, cudaStream_t);
template void scatter_rows<double, double>(int, int, const int *, const double *, double *, cudaStream_t);
}  // namespace kexact
