// graph.cpp -- sweep schedules, colourings and the reference's box
// connectivity helpers (examples/utils/pbutils.{c,py}).
#include "graph.h"

#include <algorithm>
#include <numeric>

#include "../../include/ucfdmesh.h"
#include "ucfd_internal.h"

namespace ucfd {

void symmetrize(int n, const int *rowptr, const int *colidx, std::vector<int> &srp,
                std::vector<int> &sci) {
    std::vector<int> deg(n + 1, 0);
    for (int r = 0; r < n; ++r)
        for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
            const int c = colidx[p];
            if (c < 0 || c == r) continue;
            UCFD_REQUIRE(c < n, "neighbour index %d of row %d out of range [0, %d)", c, r, n);
            deg[r]++;
            deg[c]++;
        }
    srp.assign(n + 1, 0);
    for (int r = 0; r < n; ++r) srp[r + 1] = srp[r] + deg[r];
    sci.resize(srp[n]);
    std::vector<int> fill(srp.begin(), srp.end() - 1);
    for (int r = 0; r < n; ++r)
        for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
            const int c = colidx[p];
            if (c < 0 || c == r) continue;
            sci[fill[r]++] = c;
            sci[fill[c]++] = r;
        }
    // sort + dedupe each row
    std::vector<int> nrp(n + 1, 0);
    size_t w = 0;
    for (int r = 0; r < n; ++r) {
        auto b = sci.begin() + srp[r], e = sci.begin() + srp[r + 1];
        std::sort(b, e);
        auto last = std::unique(b, e);
        for (auto it = b; it != last; ++it) sci[w++] = *it;
        nrp[r + 1] = (int)w;
    }
    sci.resize(w);
    srp.swap(nrp);
}

static Schedule from_levels(int n, const std::vector<int> &lev, int nlev) {
    Schedule s;
    s.nlev = nlev;
    s.lev_off.assign(nlev + 1, 0);
    for (int i = 0; i < n; ++i) s.lev_off[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) s.lev_off[l + 1] += s.lev_off[l];
    s.perm.resize(n);
    s.iperm.resize(n);
    std::vector<int> fill(s.lev_off.begin(), s.lev_off.end() - 1);
    for (int i = 0; i < n; ++i) {
        const int k = fill[lev[i]]++;
        s.perm[k] = i;
        s.iperm[i] = k;
    }
    return s;
}

Schedule schedule_natural(int n, const int *rowptr, const int *colidx) {
    std::vector<int> srp, sci;
    symmetrize(n, rowptr, colidx, srp, sci);
    std::vector<int> lev(n, 0);
    int nlev = n > 0 ? 1 : 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int p = srp[i]; p < srp[i + 1]; ++p) {
            const int j = sci[p];
            if (j < i && lev[j] + 1 > l) l = lev[j] + 1;
        }
        lev[i] = l;
        if (l + 1 > nlev) nlev = l + 1;
    }
    return from_levels(n, lev, nlev);
}

Schedule schedule_colored(int n, const int *rowptr, const int *colidx, const int *color) {
    for (int r = 0; r < n; ++r)
        for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
            const int c = colidx[p];
            if (c < 0 || c == r) continue;
            UCFD_REQUIRE(c < n, "neighbour index %d of row %d out of range", c, r);
            UCFD_REQUIRE(color[c] != color[r],
                         "invalid colouring: neighbours %d and %d share colour %d", r, c, color[r]);
        }
    std::vector<int> vals(color, color + n);
    std::sort(vals.begin(), vals.end());
    vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
    std::vector<int> lev(n);
    for (int i = 0; i < n; ++i)
        lev[i] = (int)(std::lower_bound(vals.begin(), vals.end(), color[i]) - vals.begin());
    return from_levels(n, lev, (int)vals.size());
}

static int bfs_from(int start, const std::vector<int> &srp, const std::vector<int> &sci, std::vector<int> &dist,
                    std::vector<int> &order) {
    // returns the last cell reached (a far cell); appends the visit order
    size_t head = order.size();
    order.push_back(start);
    dist[start] = 0;
    int last = start;
    while (head < order.size()) {
        const int i = order[head++];
        last = i;
        for (int p = srp[i]; p < srp[i + 1]; ++p) {
            const int j = sci[p];
            if (dist[j] < 0) {
                dist[j] = dist[i] + 1;
                order.push_back(j);
            }
        }
    }
    return last;
}

std::vector<int> bfs_rank(int n, const int *rowptr, const int *colidx) {
    std::vector<int> srp, sci;
    symmetrize(n, rowptr, colidx, srp, sci);
    std::vector<int> dist(n, -1), order;
    order.reserve(n);
    std::vector<int> scratch_dist(n, -1), scratch;
    for (int s = 0; s < n; ++s) {
        if (dist[s] >= 0) continue;
        // pseudo-peripheral start: the cell farthest from s in its component
        scratch.clear();
        const int far = bfs_from(s, srp, sci, scratch_dist, scratch);
        for (int v : scratch) scratch_dist[v] = -1;
        bfs_from(far, srp, sci, dist, order);
    }
    std::vector<int> rank(n);
    for (int k = 0; k < n; ++k) rank[order[k]] = k;
    return rank;
}

void sort_levels_by(Schedule &s, const std::vector<int> &key) {
    for (int l = 0; l < s.nlev; ++l) {
        auto b = s.perm.begin() + s.lev_off[l], e = s.perm.begin() + s.lev_off[l + 1];
        std::sort(b, e, [&](int a, int c) { return key[a] < key[c]; });
    }
    for (int k = 0; k < (int)s.perm.size(); ++k) s.iperm[s.perm[k]] = k;
}

void sort_levels_by(Schedule &s, const std::vector<int> &major, const std::vector<int> &minor) {
    for (int l = 0; l < s.nlev; ++l) {
        auto b = s.perm.begin() + s.lev_off[l], e = s.perm.begin() + s.lev_off[l + 1];
        std::sort(b, e, [&](int a, int c) { return major[a] != major[c] ? major[a] < major[c] : minor[a] < minor[c]; });
    }
    for (int k = 0; k < (int)s.perm.size(); ++k) s.iperm[s.perm[k]] = k;
}

std::vector<int> greedy_color_csr(int n, const int *rowptr, const int *colidx, int *ncolors) {
    std::vector<int> srp, sci;
    symmetrize(n, rowptr, colidx, srp, sci);
    std::vector<int> col(n, -1);
    std::vector<int> mark;  // mark[c] == i when colour c is taken by a neighbour of i
    int nc = 0;
    for (int i = 0; i < n; ++i) {
        for (int p = srp[i]; p < srp[i + 1]; ++p) {
            const int c = col[sci[p]];
            if (c >= 0) {
                if ((int)mark.size() <= c) mark.resize(c + 1, -1);
                mark[c] = i;
            }
        }
        int c = 0;
        while (c < (int)mark.size() && mark[c] == i) ++c;
        col[i] = c;
        if (c + 1 > nc) nc = c + 1;
    }
    if (ncolors) *ncolors = nc;
    return col;
}

std::vector<int> greedy_color_bfs(int n, const int *rowptr, const int *colidx, int *ncolors) {
    std::vector<int> srp, sci;
    symmetrize(n, rowptr, colidx, srp, sci);
    const std::vector<int> rank = bfs_rank(n, rowptr, colidx);
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[rank[i]] = i;
    std::vector<int> col(n, -1);
    std::vector<int> mark;  // mark[c] == step when colour c is taken by a neighbour
    int nc = 0;
    for (int step = 0; step < n; ++step) {
        const int i = order[step];
        for (int p = srp[i]; p < srp[i + 1]; ++p) {
            const int c = col[sci[p]];
            if (c >= 0) {
                if ((int)mark.size() <= c) mark.resize(c + 1, -1);
                mark[c] = step;
            }
        }
        int c = 0;
        while (c < (int)mark.size() && mark[c] == step) ++c;
        col[i] = c;
        if (c + 1 > nc) nc = c + 1;
    }
    if (ncolors) *ncolors = nc;
    return col;
}

}  // namespace ucfd

// ---------------------------------------------------------------------------
// C ABI (ucfdmesh.h)
// ---------------------------------------------------------------------------
extern "C" {

// make_nei_ele: examples/utils/pbutils.c:43-84 / pbutils.py:4-36.
ucfd_status_t UCFDMakeNeiEle(int m, int n, int l, int *adj) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(adj && m > 0 && n > 0 && l > 0, "UCFDMakeNeiEle: bad arguments");
    const long long mn = (long long)m * n, N = mn * l;
    UCFD_REQUIRE(N < (1ll << 31), "UCFDMakeNeiEle: %lld cells overflow int32", N);
    for (int z = 0; z < l; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < m; ++x) {
                const long long i = x + (long long)m * y + mn * z;
                adj[0 * N + i] = (int)(x > 0 ? i - 1 : i);
                adj[1 * N + i] = (int)(x + 1 < m ? i + 1 : i);
                adj[2 * N + i] = (int)(y > 0 ? i - m : i);
                adj[3 * N + i] = (int)(y + 1 < n ? i + m : i);
                adj[4 * N + i] = (int)(z > 0 ? i - mn : i);
                adj[5 * N + i] = (int)(z + 1 < l ? i + mn : i);
            }
    UCFD_API_END
}

// make_coloring: pbutils.py:39-56 (even x+y+z first, then odd, index order).
ucfd_status_t UCFDMakeColoring(int m, int n, int l, int *icolor) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(icolor && m > 0 && n > 0 && l > 0, "UCFDMakeColoring: bad arguments");
    const long long N = (long long)m * n * l;
    long long ne = 0;
    for (long long i = 0; i < N; ++i) {
        const long long x = i % m, y = (i / m) % n, z = i / ((long long)m * n);
        if (((x + y + z) & 1) == 0) ne++;
    }
    long long a = 0, b = ne;
    for (long long i = 0; i < N; ++i) {
        const long long x = i % m, y = (i / m) % n, z = i / ((long long)m * n);
        if (((x + y + z) & 1) == 0) icolor[a++] = (int)i;
        else icolor[b++] = (int)i;
    }
    UCFD_API_END
}

static ucfd_status_t color_out(int n, const std::vector<int> &col, int nc, int *lcolor, int *icolor,
                               int *ranges, int *ncolors) {
    UCFD_REQUIRE(nc <= 64 || !ranges, "greedy colouring needed %d colours (> 64)", nc);
    std::vector<int> cnt(nc + 1, 0);
    for (int i = 0; i < n; ++i) cnt[col[i] + 1]++;
    for (int c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    if (ranges)
        for (int c = 0; c < nc; ++c) ranges[c] = cnt[c + 1];
    if (icolor) {
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int i = 0; i < n; ++i) icolor[fill[col[i]]++] = i;
    }
    if (lcolor)
        for (int i = 0; i < n; ++i) lcolor[i] = col[i] + 1;
    if (ncolors) *ncolors = nc;
    return UCFD_SUCCESS;
}

ucfd_status_t UCFDGreedyColoringCSR(int n, const int *rowptr, const int *colidx, int *lcolor,
                                    int *icolor, int *ranges, int *ncolors) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(n >= 0 && rowptr && colidx, "UCFDGreedyColoringCSR: bad arguments");
    int nc = 0;
    std::vector<int> col = ucfd::greedy_color_csr(n, rowptr, colidx, &nc);
    color_out(n, col, nc, lcolor, icolor, ranges, ncolors);
    UCFD_API_END
}

ucfd_status_t UCFDBFSColoringCSR(int n, const int *rowptr, const int *colidx, int *lcolor, int *icolor,
                                 int *ranges, int *ncolors) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(n >= 0 && rowptr && colidx, "UCFDBFSColoringCSR: bad arguments");
    int nc = 0;
    std::vector<int> col = ucfd::greedy_color_bfs(n, rowptr, colidx, &nc);
    color_out(n, col, nc, lcolor, icolor, ranges, ncolors);
    UCFD_API_END
}

ucfd_status_t UCFDGreedyColoring(int neles, int nface, const int *nei_ele, int *lcolor,
                                 int *icolor, int *ranges, int *ncolors) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(neles >= 0 && nface > 0 && nei_ele, "UCFDGreedyColoring: bad arguments");
    std::vector<int> rp(neles + 1), ci((size_t)neles * nface);
    for (int i = 0; i <= neles; ++i) rp[i] = i * nface;
    for (int i = 0; i < neles; ++i)
        for (int f = 0; f < nface; ++f) ci[(size_t)i * nface + f] = nei_ele[(size_t)f * neles + i];
    int nc = 0;
    std::vector<int> col = ucfd::greedy_color_csr(neles, rp.data(), ci.data(), &nc);
    color_out(neles, col, nc, lcolor, icolor, ranges, ncolors);
    UCFD_API_END
}

}  // extern "C"
