// kargs.h -- plain argument structs shared by host code and kernels.
#pragma once

#ifdef __CUDACC__
#define UCFD_HD __host__ __device__
#else
#define UCFD_HD
#endif

namespace ucfd {

// Cell-tiled layout of the per-cell block arrays (J, LU, D of block
// LU-SGS): internal cells are grouped in tiles of 32 consecutive cells and
// element j (of m per cell) of cell k sits at ((k / 32) * m + j) * 32 + k % 32.
// A warp on one tile reads each element as one 128-byte (FP32) line, and
// all m elements of a tile are one contiguous block (a single bulk copy).
constexpr int kCellTile = 32;
UCFD_HD inline long long tile_index(long long k, long long j, long long m) {
    return (((k >> 5) * m + j) << 5) + (k & 31);
}
UCFD_HD inline long long tiled_size(long long N, long long m) { return ((N + 31) >> 5) * m * 32; }

// Term of the structure fingerprints (sum over i, wrapping): the splitmix64
// finaliser (Steele, Lea and Flood 2014) of the index in the high word and
// the value in the low word.  The same function on the host and the device.
UCFD_HD inline unsigned long long fingerprint_mix(long long i, int v) {
    unsigned long long z = ((unsigned long long)i << 32) ^ (unsigned)v;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

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
    const T *tlam;         // [nface][ld] spectral radius of the turbulence system when one launch
                           // sweeps both systems (rans == 2), else unused
    const void *geo4;      // FP32, both systems: float4 [nface][ld] (normal, fa * rv) per cell-face,
                           // read instead of nrm / fa / rv (nullptr: not packed)
    const void *lam2;      // with geo4: float2 [nface][ld] (lam, tlam) per cell-face
    const T *u;            // [nvars][ld]
    const T *nbsrc;        // [nvars][ld] neighbour increments
    const T *own_in;       // [nvars][ld]
    T *own_out;            // [nvars][ld]
    const T *diag;         // diag[v*diag_vs + cell]
    long long diag_vs;
    T kappa, gamma, pmin;
    int upper;
    int regcap;            // 0, or 3 / 4: the kernel built for that many blocks of 256 threads per SM
                           // (at most 80 / 64 registers)
    int pair;              // 1: two threads per cell (faces 0-2 / 3-5; ELL width <= 6, per-level launches)
    // one thread per active face (per-level launches): the faces of this
    // sweep direction whose neighbour lies in an earlier level, cell by cell
    // in face order
    int facelist;          // 1: use the list
    int cpb;               // cells per block (0: a third of the block's threads)
    const int *fl_off;     // [ld + 1] first list entry of each cell
    const int *fl_nb;      // [E] neighbour cell of each entry
    const int *fl_q;       // [E] ELL slot f * ld + cell of each entry (spectral radius)
    const T *fl_geo;       // [E][4] outward normal (zero-padded to 3 components) and fa * rv
};

// Block LU-SGS sweeps of the fast build (M = D^-1 J fv blocks): a cell's
// face products are summed by the level of the neighbour -- S_lo over
// earlier levels, S_up over later ones -- and du = c - S_lo - S_up.  A
// lower sweep reaches a cell after every earlier level and before every
// later one, an upper sweep the other way round, so the side a sweep does
// not update is the sum the previous (opposite) sweep formed with the same
// increments.  part keeps each sweep's own side for the next one; with
// full == 0 a sweep reads the other side from part instead of loading
// those faces again.  Either way the values are the same, bit for bit.
// (A face to the cell itself goes with the other side's sum; a mesh with
// such faces always sweeps in full mode.)
template <typename S>
struct SweepSplit {
    S *part = nullptr;  // [nvars][N] sums of the sweep's own side (nullptr: exact build, no split)
    int upper = 0;      // this sweep's direction
    int full = 1;       // 1: form both sides; 0: the other side from part
};

// One colour of a transposed (adjoint) colored LU-SGS sweep.
struct AdjArgs {
    int t0, t1;          // icolor slots of the colour
    int neles, nface;
    const int *icolor, *lcolor, *nei, *rface;
};

}  // namespace ucfd
