/*
 * ucfdmesh.h -- connectivity and colouring helpers of libucfd_gb300.so
 * (host code, no GPU needed).
 *
 * UCFDMakeNeiEle / UCFDMakeColoring replace the reference example
 * utilities make_nei_ele and make_coloring (examples/utils/pbutils.c:43-84
 * and 98-121, pbutils.py:4-56) with identical output; the checkerboard
 * follows pbutils.py (correct for odd cell counts, where pbutils.c
 * overruns its first half).  The greedy colouring and the level schedule
 * are this library's: the reference has no general colouring.
 */
#pragma once

#include "ucfd_gb300.h"

#if defined(__cplusplus)
extern "C" {
#endif

/* nei_ele [6][m*n*l], face order -x,+x,-y,+y,-z,+z, boundary -> self */
UCFD_EXTERN ucfd_status_t UCFDMakeNeiEle(int m, int n, int l, int *nei_ele);
/* icolor [m*n*l]: cells with even x+y+z in index order, then odd ones */
UCFD_EXTERN ucfd_status_t UCFDMakeColoring(int m, int n, int l, int *icolor);

/* Greedy first-fit colouring of a [nface][neles] neighbour table, cells
 * visited in index order; entries equal to the cell itself or < 0 are
 * ignored.  Outputs: lcolor [neles] (1-based colour), icolor [neles]
 * (cells grouped by colour, ascending index within a colour), ranges
 * [ncolors] (exclusive end of each colour in icolor; room for 64) and the
 * number of colours. */
UCFD_EXTERN ucfd_status_t UCFDGreedyColoring(int neles, int nface, const int *nei_ele,
                                             int *lcolor, int *icolor, int *ranges,
                                             int *ncolors);
/* The same for a CSR graph (rowptr [n+1], colidx [nnz]). */
UCFD_EXTERN ucfd_status_t UCFDGreedyColoringCSR(int n, const int *rowptr, const int *colidx,
                                                int *lcolor, int *icolor, int *ranges,
                                                int *ncolors);
/* First-fit greedy colouring of a CSR graph visiting the cells in
 * breadth-first order from a pseudo-peripheral cell (fewer colours than
 * index order: two on a bipartite hexahedral mesh); same outputs as
 * UCFDGreedyColoringCSR.  No counterpart in the reference (its colourings
 * come from the caller or examples/utils/pbutils). */
UCFD_EXTERN ucfd_status_t UCFDBFSColoringCSR(int n, const int *rowptr, const int *colidx,
                                             int *lcolor, int *icolor, int *ranges, int *ncolors);

#if defined(__cplusplus)
}
#endif
