// graph.h -- host-side graph utilities: sweep schedules and colourings.
#pragma once

#include <cstdint>
#include <vector>

namespace ucfd {

// A sweep schedule: cells grouped in levels, every level an independent
// set, processed in increasing order by lower sweeps and in decreasing
// order by upper sweeps.  perm[k] is the original index of internal cell k
// (level-major, original order inside a level); iperm is its inverse.
struct Schedule {
    int nlev = 0;
    std::vector<int> lev_off;  // size nlev + 1
    std::vector<int> perm, iperm;
};

// Levels that reproduce a natural-order Gauss-Seidel sweep of a CSR graph:
// level(i) = 1 + max level over neighbours j < i of the symmetrised graph
// (self entries and entries < 0 ignored).  Adjacent cells always land in
// different levels, the higher-indexed one later.
Schedule schedule_natural(int n, const int *rowptr, const int *colidx);

// Levels = colours (dense rank of the colour values).  Throws
// UCFD_ERR_ARGUMENT when two neighbours share a colour.
Schedule schedule_colored(int n, const int *rowptr, const int *colidx, const int *color);

// Greedy first-fit colouring in index order (neighbours from the
// symmetrised graph); returns 0-based colours and the colour count.
std::vector<int> greedy_color_csr(int n, const int *rowptr, const int *colidx, int *ncolors);
// First-fit greedy colouring visiting the cells in breadth-first order
// (bfs_rank): two colours on a bipartite graph such as a hexahedral mesh.
std::vector<int> greedy_color_bfs(int n, const int *rowptr, const int *colidx, int *ncolors);

// Breadth-first order of the symmetrised graph started from a
// pseudo-peripheral cell (each connected component in turn): rank[i] is
// the position of cell i.  Graph neighbours get nearby ranks, so sorting
// the cells of each level by it makes neighbour gathers of consecutive
// threads hit nearby memory.
std::vector<int> bfs_rank(int n, const int *rowptr, const int *colidx);

// Reorder the cells inside every level by key (does not change results:
// the cells of a level are independent).
void sort_levels_by(Schedule &s, const std::vector<int> &key);
// The same with a major and a minor key.
void sort_levels_by(Schedule &s, const std::vector<int> &major, const std::vector<int> &minor);

// Symmetrised adjacency (CSR, no self entries, no duplicates).
void symmetrize(int n, const int *rowptr, const int *colidx, std::vector<int> &srp,
                std::vector<int> &sci);

}  // namespace ucfd
