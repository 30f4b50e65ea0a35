// kern_fast.cu -- kernels built with FMA contraction: FP64 (fast mode) and
// FP32 instantiations, mixed-precision helpers and the GMRES reductions.
#define UCFD_KNS kfast
#include "launchers.cuh"

namespace kfast {
#define UCFD_INST_T(T)                                                                                          \
    template void scalar_sweep<T>(const ::ucfd::ScalarSweepArgs<T> &, int, int, int, int, int, cudaStream_t);  \
    template void face_list_geo<T>(long long, long long, int, const int *, const T *, const T *, const T *,    \
                                   T *, cudaStream_t);                                                         \
    template void scalar_sweep_persistent<T>(const ::ucfd::ScalarSweepArgs<T> &, int, int, int, int,           \
                                             const int *, int, unsigned *, int *, long long, cudaStream_t);    \
    template void legacy_pre<T>(int, int, T, const T *, const T *, T *, const T *, cudaStream_t);              \
    template void legacy_update<T>(int, int, int, T *, const T *, cudaStream_t);                               \
    template void fs_lusgs_pack<T>(int, int, int, long long, double, double, const int *, const int *,         \
                                   const double *, const double *, const double *, const double *, T *, T *,   \
                                   T *, cudaStream_t);                                                         \
    template void fs_lusgs_update<T>(int, int, long long, const int *, const int *, const T *, double *, int,  \
                                     cudaStream_t);                                                            \
    template void fs_lusgs_prepare<T>(long long, int, int, int, T, const int *, const T *, const T *,          \
                                      const T *, const T *, T *, cudaStream_t);                                \
    template void fs_lusgs_prepare_both<T>(long long, int, int, int, T, const int *, const T *, const T *,     \
                                           const T *, const T *, const T *, T *, cudaStream_t);                \
    template void gather_idx<T>(long long, const int *, const double *, T *, cudaStream_t);                    \
    template void fs_blusgs_pack<T>(int, int, int, long long, double, const int *, const int *,                \
                                    const double *, const double *, T *, double *, double *, cudaStream_t);    \
    template void fs_blusgs_prepare<T>(int, long long, int, long long, const int *, const int *,               \
                                       const int8_t *, const double *, const double *, const double *,         \
                                       const double *, double *, double *, T *, T *, double *, double *,       \
                                       cudaStream_t);                                                          \
    template void fs_blusgs_sweep<T>(int, int, int, long long, int, int, const int *, const T *, const T *,    \
                                     const T *, const T *, const T *, T *, int, int, int *, long long,         \
                                     const ::ucfd::SweepSplit<T> &, cudaStream_t);                                                            \
    template void fs_blusgs_residual<T, T>(int, long long, int, int, int, const int *, const double *,         \
                                           const double *, const double *, const double *, const double *,     \
                                           const T *, T *, double *, int, int *, cudaStream_t);                \
    template void fs_blusgs_rhs_solve<T>(int, long long, int, const T *, const T *, T *, cudaStream_t);        \
    template void fs_blusgs_subres<T>(int, int, long long, const int *, const int *, const double *,           \
                                      const T *, T *, double *, cudaStream_t);                                 \
    template void fs_blusgs_update<T>(int, int, long long, const int *, const int *, const T *, double *,      \
                                      cudaStream_t);                                                           \
    template void bsr_spmv<T, T>(int, int, int, const int *, const T *, double, const double *, double,        \
                                 double *, int, cudaStream_t);                                                 \
    template void pc_prepare<T>(int, int, const int *, const long long *, const double *, double *, T *, int,  \
                                cudaStream_t);                                                                 \
    template void pc_lower<T>(int, int, int, int, int, const int *, const T *, const T *, T *, int, int,       \
                              cudaStream_t);                                                                   \
    template void pc_upper<T>(int, int, int, int, int, const int *, const T *, const T *, T *, int, int,       \
                              cudaStream_t);
UCFD_INST_T(double)
UCFD_INST_T(float)
#undef UCFD_INST_T
#define UCFD_INST_ADJ(T)                                                                                       \
    template void adj_upper<T>(const ::ucfd::AdjArgs &, int, int, T, T, const T *, const T *, const T *,      \
                               const T *, const T *, const T *, const T *, const T *, T *, T *, T *,          \
                               cudaStream_t);                                                                 \
    template void adj_lower<T>(const ::ucfd::AdjArgs &, int, int, T, T, T, const T *, const T *, const T *,    \
                               const T *, const T *, const T *, const T *, const T *, T *, const T *, T *,    \
                               T *, T *, cudaStream_t);
UCFD_INST_ADJ(double)
UCFD_INST_ADJ(float)
#undef UCFD_INST_ADJ
template void fs_blusgs_residual<double, float>(int, long long, int, int, int, const int *, const double *,
                                                const double *, const double *, const double *, const double *,
                                                const double *, float *, double *, int, int *, cudaStream_t);
template void gather_rows<double, double>(int, int, const int *, const double *, double *, cudaStream_t);
template void scatter_rows<double, double>(int, int, const int *, const double *, double *, cudaStream_t);
template void gather_rows<double, float>(int, int, const int *, const double *, float *, cudaStream_t);
template void scatter_rows<float, double>(int, int, const int *, const float *, double *, cudaStream_t);
template void ell_gather<double>(int, int, int, const int *, const double *, double *, cudaStream_t);
template void ell_gather<float>(int, int, int, const int *, const double *, float *, cudaStream_t);
template void convert<double, float>(long long, const double *, float *, cudaStream_t);
template void convert<float, double>(long long, const float *, double *, cudaStream_t);
template void axpy_into<float>(long long, const float *, double *, cudaStream_t);
template void axpy_into<double>(long long, const double *, double *, cudaStream_t);
template void axpy_norm<double>(long long, const double *, double *, double *, double *, cudaStream_t);
template void axpy_norm<float>(long long, const float *, float *, double *, double *, cudaStream_t);
}  // namespace kfast
