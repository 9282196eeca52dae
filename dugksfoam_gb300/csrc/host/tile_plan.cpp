// Tile plan construction (see tile_plan.h).
//
// Tiles come from recursive coordinate bisection of the cell centres: a range
// of c cells is split along its longest extent into parts holding whole
// multiples of the tile size N, so the leaves are box-shaped blobs of N cells
// and the depth-first leaf order keeps consecutive tiles spatially adjacent
// (their halo rows are re-read from L2 while both are in flight).  N is the
// largest size (binary search) for which every tile's shared-memory footprint
// -- rows of T u H1 u H2 plus face/cell accumulators -- fits the budget.
#include "tile_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace dugks {
namespace {

inline int other(const Mesh& m, int j) {  // neighbour across cell-face entry j (internal faces)
    const int f = m.cellFace[j];
    return m.cellSide[j] == 0 ? m.neighbour[f] : m.owner[f];
}

// Sets of a candidate tile: lc = T, then H1, then H2 (stamp-marked).
struct Sets {
    std::vector<int> mark;  // stamp*3 + {0,1,2}
    int stamp = 0;
    TileDims d;
    int &nT = d.nT, &nT1 = d.nT1, &nT2 = d.nT2, &nFA = d.nFA, &nFB = d.nFB, &nEnt = d.nEnt;
    std::vector<int> lc;
    explicit Sets(int nC) : mark(nC, -1) {}
    bool in(int c) const { return mark[c] >= stamp * 3 && mark[c] <= stamp * 3 + 2; }
    bool inT(int c) const { return mark[c] == stamp * 3; }
    void build(const Mesh& m, const int* cells, int n, int rings) {
        ++stamp;
        lc.assign(cells, cells + n);
        for (int i = 0; i < n; ++i) mark[cells[i]] = stamp * 3;
        nT = n;
        auto ring = [&](int from, int to, int tag) {
            for (int i = from; i < to; ++i) {
                const int c = lc[i];
                for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                    if (m.cellFace[j] >= m.nI) continue;
                    const int o = other(m, j);
                    if (in(o)) continue;
                    mark[o] = stamp * 3 + tag;
                    lc.push_back(o);
                }
            }
        };
        ring(0, nT, 1);
        nT1 = (int)lc.size();
        if (rings == 2) ring(nT, nT1, 2);
        nT2 = (int)lc.size();
        nFA = nFB = nEnt = 0;
        for (int i = 0; i < nT; ++i) {
            const int c = lc[i];
            for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                const int f = m.cellFace[j];
                if (f >= m.nI || m.cellSide[j] == 0) ++nFA, ++nFB;
                else if (!inT(m.owner[f])) ++nFB;
            }
        }
        const int nSt = rings == 2 ? nT1 : nT;  // cells with a stencil
        for (int i = 0; i < nSt; ++i) nEnt += m.cellOff[lc[i] + 1] - m.cellOff[lc[i]];
    }
};

}  // namespace

namespace {

void rcb(const Mesh& m, std::vector<int>& cells, int b, int e, int N, std::vector<std::pair<int, int>>& parts) {
    const int c = e - b;
    if (c <= N) {
        parts.push_back({b, e});
        return;
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], m.C[3 * (size_t)cells[i] + k]);
            hi[k] = std::max(hi[k], m.C[3 * (size_t)cells[i] + k]);
        }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (hi[k] - lo[k] > hi[ax] - lo[ax]) ax = k;
    const int np = (c + N - 1) / N;
    const int left = (int)((long long)c * (np / 2) / np);
    std::nth_element(cells.begin() + b, cells.begin() + b + left, cells.begin() + e, [&](int x, int y) {
        return m.C[3 * (size_t)x + ax] < m.C[3 * (size_t)y + ax];
    });
    rcb(m, cells, b, b + left, N, parts);
    rcb(m, cells, b + left, e, N, parts);
}

}  // namespace

bool build_tile_plan(const Mesh& m, int maxTileCells, const SmemFn& smem, size_t budget, TilePlan& p,
                     std::string& err, int rings, int waveSlots) {
    if (rings != 1 && rings != 2) { err = "tile plan: rings must be 1 or 2"; return false; }
    const int nC = m.nC, nI = m.nI;
    if (maxTileCells < 1) { err = "tile size must be positive"; return false; }
    p = TilePlan();
    Sets S(nC);
    std::vector<int> cells(nC);
    std::vector<std::pair<int, int>> parts;
    auto partition = [&](int N) {
        for (int c = 0; c < nC; ++c) cells[c] = c;
        parts.clear();
        rcb(m, cells, 0, nC, N, parts);
    };
    auto fits = [&](int N) {
        partition(N);
        for (auto& pr : parts) {
            S.build(m, cells.data() + pr.first, pr.second - pr.first, rings);
            if (smem(S.d) > budget) return false;
        }
        return true;
    };
    int lo = 1, hi = std::min(maxTileCells, nC);
    if (!fits(lo)) { err = "tile plan: a single cell and its halo exceed the shared-memory budget"; return false; }
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (fits(mid)) lo = mid;
        else hi = mid - 1;
    }
    if (waveSlots > 0) {  // fill the last wave: the smallest size with no more waves
        partition(lo);
        const long long slots = ((long long)parts.size() + waveSlots - 1) / waveSlots * waveSlots;
        int a = 1, b = lo;  // smallest N in [1, lo] with count(N) <= slots (count falls as N grows)
        while (a < b) {
            const int mid = (a + b) / 2;
            partition(mid);
            if ((long long)parts.size() <= slots) b = mid;
            else a = mid + 1;
        }
        lo = a;  // smaller tiles than a size that fits: they fit too
    }
    partition(lo);
    p.tileCells = lo;
    std::vector<int> loc(nC, -1);
    int t = 0;
    for (auto& pr : parts) {
        S.build(m, cells.data() + pr.first, pr.second - pr.first, rings);
        // ---- emit the tile
        TileHdr h{};
        const std::vector<int>& lc = S.lc;
        h.nT = S.nT;
        h.nT1 = S.nT1;
        h.nT2 = S.nT2;
        h.cellStart = (int)p.cells.size();
        for (int i = 0; i < h.nT2; ++i) {
            loc[lc[i]] = i;
            p.cells.push_back(lc[i]);
        }
        // stencils of T u H1 (rings = 2) or T (rings = 1), entries in global face order
        const int nSt = rings == 2 ? h.nT1 : h.nT;
        h.stStart = (int)p.stOff.size();
        for (int i = 0; i < nSt; ++i) {
            const int c = lc[i];
            p.stOff.push_back((int)p.stEnt.size());
            for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                const int f = m.cellFace[j];
                if (f < nI) {
                    const int o = other(m, j);
                    if (!S.in(o)) { err = "tile plan: stencil cell outside the two-ring halo"; return false; }
                    p.stEnt.push_back(loc[o]);
                    const double* L = m.cellSide[j] == 0 ? &m.pVec[3 * (size_t)f] : &m.nVec[3 * (size_t)f];
                    p.stL.insert(p.stL.end(), L, L + 3);
                } else {
                    const int w = f - nI;
                    p.stEnt.push_back(-(w + 1));
                    p.stL.insert(p.stL.end(), &m.bVec[3 * (size_t)w], &m.bVec[3 * (size_t)w] + 3);
                }
            }
        }
        p.stOff.push_back((int)p.stEnt.size());
        h.nEnt = (int)p.stEnt.size() - p.stOff[h.stStart];
        // faces: owned first (internal with owner in T, then walls of T), then
        // internal faces with neighbour in T and owner outside T.
        std::vector<std::pair<int, int>> owned, extra;  // (global face order key, active face)
        for (int i = 0; i < h.nT; ++i) {
            const int c = lc[i];
            for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                const int f = m.cellFace[j];
                if (f < nI) {
                    if (m.cellSide[j] == 0) owned.push_back({f, f});
                    else if (!S.inT(m.owner[f])) extra.push_back({f, f});
                } else {
                    owned.push_back({m.wallFace[f - nI], f});
                }
            }
        }
        std::sort(owned.begin(), owned.end());
        std::sort(extra.begin(), extra.end());
        h.faceStart = (int)p.faces.size();
        h.nFA = (int)owned.size();
        h.nFB = h.nFA + (int)extra.size();
        std::vector<int> fa;
        for (auto& x : owned) fa.push_back(x.second);
        for (auto& x : extra) fa.push_back(x.second);
        for (int a : fa) {
            TileFace r{};
            r.a = a;
            if (a < nI) {
                r.ownL = loc[m.owner[a]];
                r.neiL = loc[m.neighbour[a]];
                r.w = -1;
            } else {
                r.w = a - nI;
                r.ownL = loc[m.wallCell[r.w]];
                r.neiL = -1;
            }
            if (r.ownL < 0 || r.ownL >= h.nT1 || (a < nI && (r.neiL < 0 || r.neiL >= h.nT1))) {
                err = "tile plan: face cell outside T u H1";
                return false;
            }
            const bool stO = r.ownL < nSt, stN = r.neiL >= 0 && r.neiL < nSt;
            r.stO0 = stO ? p.stOff[h.stStart + r.ownL] : 0;
            r.stO1 = stO ? p.stOff[h.stStart + r.ownL + 1] : 0;
            r.stN0 = stN ? p.stOff[h.stStart + r.neiL] : 0;
            r.stN1 = stN ? p.stOff[h.stStart + r.neiL + 1] : 0;
            p.faces.push_back(r);
        }
        // greedy colouring: faces of one colour touch distinct cells of T
        std::vector<int> color(h.nFB, -1);
        std::vector<uint64_t> used(h.nT, 0);
        int ncol = 0;
        for (int k = 0; k < h.nFB; ++k) {
            const TileFace& r = p.faces[h.faceStart + k];
            uint64_t busy = 0;
            if (r.ownL < h.nT) busy |= used[r.ownL];
            if (r.neiL >= 0 && r.neiL < h.nT) busy |= used[r.neiL];
            int col = 0;
            while (col < 64 && (busy >> col & 1)) ++col;
            if (col == 64) { err = "tile plan: more than 64 face colours"; return false; }
            color[k] = col;
            ncol = std::max(ncol, col + 1);
            if (r.ownL < h.nT) used[r.ownL] |= 1ULL << col;
            if (r.neiL >= 0 && r.neiL < h.nT) used[r.neiL] |= 1ULL << col;
        }
        h.colStart = (int)p.colorOff.size();
        h.permStart = (int)p.colorPerm.size();
        h.nColors = ncol;
        int acc = 0;
        for (int col = 0; col < ncol; ++col) {
            p.colorOff.push_back(acc);
            for (int k = 0; k < h.nFB; ++k)
                if (color[k] == col) { p.colorPerm.push_back(k); ++acc; }
        }
        p.colorOff.push_back(acc);
        p.maxT = std::max(p.maxT, h.nT);
        p.maxT2 = std::max(p.maxT2, h.nT2);
        p.maxFA = std::max(p.maxFA, h.nFA);
        p.maxFB = std::max(p.maxFB, h.nFB);
        p.sumT += h.nT;
        p.sumT2 += h.nT2;
        for (int c : lc) loc[c] = -1;
        p.hdr.push_back(h);
        ++t;
    }
    p.nTiles = t;
    return true;
}

}  // namespace dugks
