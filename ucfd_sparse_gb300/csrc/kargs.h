// kargs.h -- plain argument structs shared by host code and kernels.
#pragma once

namespace ucfd {

// One launch of the scalar LU-SGS sweep over a range of cells that are
// independent of each other (one colour or one level).
template <typename T>
struct ScalarSweepArgs {
    int t0, t1;            // cell slots t in [t0, t1)
    const int *cells;      // cell = cells ? cells[t] : t
    const int *lcolor;     // colour test (array layout) or nullptr
    int lo, hi;            // index test (level-major layout): lower nb < lo, upper nb >= hi
    int nface;
    long long ld;          // cell stride of every [..][ld] array
    const int *nei;        // [nface][ld]  (-1 = padding)
    const T *fa;           // [nface][ld]  face area (fnorm_vol when rv == nullptr)
    const T *rv;           // [ld] reciprocal volume or nullptr
    const T *nrm;          // [nface][ndims][ld] outward unit normals
    const T *lam;          // [nface][ld] spectral radius
    const T *u;            // [nvars][ld]
    const T *nbsrc;        // [nvars][ld] neighbour increments
    const T *own_in;       // [nvars][ld]
    T *own_out;            // [nvars][ld]
    const T *diag;         // diag[v*diag_vs + cell]
    long long diag_vs;
    T kappa, gamma, pmin;
    int upper;
};

// One colour of a transposed (adjoint) colored LU-SGS sweep.
struct AdjArgs {
    int t0, t1;          // icolor slots of the colour
    int neles, nface;
    const int *icolor, *lcolor, *nei, *rface;
};

}  // namespace ucfd
