// Tile plan construction (see tile_plan.h).
#include "tile_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace dugks {
namespace {

uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

}  // namespace

bool build_tile_plan(const Mesh& m, int tileCells, TilePlan& p, std::string& err) {
    const int nC = m.nC, nI = m.nI;
    if (tileCells < 1) { err = "tile size must be positive"; return false; }
    p = TilePlan();
    p.tileCells = tileCells;

    // ---- Morton order of cell centres
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < nC; ++c)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], m.C[3 * (size_t)c + k]);
            hi[k] = std::max(hi[k], m.C[3 * (size_t)c + k]);
        }
    std::vector<std::pair<uint64_t, int>> key(nC);
    for (int c = 0; c < nC; ++c) {
        uint64_t code = 0;
        for (int k = 0; k < 3; ++k) {
            double span = hi[k] - lo[k];
            double t = span > 0 ? (m.C[3 * (size_t)c + k] - lo[k]) / span : 0.0;
            uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, t * 2097151.0));
            code |= spread3(q) << k;
        }
        key[c] = {code, c};
    }
    std::sort(key.begin(), key.end());

    // cell -> (neighbour cell) adjacency through internal faces, per cell in face order
    std::vector<int> mark(nC, -1), loc(nC, -1);
    const int nTiles = (nC + tileCells - 1) / tileCells;
    p.nTiles = nTiles;
    p.hdr.resize(nTiles);
    for (int t = 0; t < nTiles; ++t) {
        TileHdr h{};
        const int b = t * tileCells, e = std::min(nC, b + tileCells);
        std::vector<int> lc;  // local cells
        for (int i = b; i < e; ++i) lc.push_back(key[i].second);
        for (int c : lc) mark[c] = t * 3;          // T
        h.nT = (int)lc.size();
        auto ring = [&](int from, int to, int tag) {
            for (int i = from; i < to; ++i) {
                int c = lc[i];
                for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                    int f = m.cellFace[j];
                    if (f >= nI) continue;
                    int o = m.cellSide[j] == 0 ? m.neighbour[f] : m.owner[f];
                    if (mark[o] >= t * 3 && mark[o] <= t * 3 + 2) continue;
                    mark[o] = tag;
                    lc.push_back(o);
                }
            }
        };
        ring(0, h.nT, t * 3 + 1);
        h.nT1 = (int)lc.size();
        ring(h.nT, h.nT1, t * 3 + 2);
        h.nT2 = (int)lc.size();
        h.cellStart = (int)p.cells.size();
        for (int i = 0; i < h.nT2; ++i) {
            loc[lc[i]] = i;
            p.cells.push_back(lc[i]);
        }
        // stencils of T u H1, entries in global face order
        h.stStart = (int)p.stOff.size();
        for (int i = 0; i < h.nT1; ++i) {
            int c = lc[i];
            p.stOff.push_back((int)p.stEnt.size());
            for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                int f = m.cellFace[j];
                if (f < nI) {
                    int side = m.cellSide[j];
                    int o = side == 0 ? m.neighbour[f] : m.owner[f];
                    if (loc[o] < 0 || mark[o] < t * 3 || mark[o] > t * 3 + 2) {
                        err = "tile plan: stencil cell outside the two-ring halo";
                        return false;
                    }
                    p.stEnt.push_back(loc[o]);
                    const double* L = side == 0 ? &m.pVec[3 * (size_t)f] : &m.nVec[3 * (size_t)f];
                    p.stL.insert(p.stL.end(), L, L + 3);
                } else {
                    int w = f - nI;
                    p.stEnt.push_back(-(w + 1));
                    p.stL.insert(p.stL.end(), &m.bVec[3 * (size_t)w], &m.bVec[3 * (size_t)w] + 3);
                }
            }
        }
        p.stOff.push_back((int)p.stEnt.size());
        // faces: owned first (internal with owner in T, then walls of T), then
        // internal faces with neighbour in T and owner outside T.
        std::vector<std::pair<int, int>> owned, extra;  // (global face order key, active face)
        for (int i = 0; i < h.nT; ++i) {
            int c = lc[i];
            for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                int f = m.cellFace[j];
                if (f < nI) {
                    if (m.cellSide[j] == 0) owned.push_back({f, f});
                    else if (mark[m.owner[f]] != t * 3) extra.push_back({f, f});
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
            r.stO0 = p.stOff[h.stStart + r.ownL];
            r.stO1 = p.stOff[h.stStart + r.ownL + 1];
            r.stN0 = r.neiL >= 0 ? p.stOff[h.stStart + r.neiL] : 0;
            r.stN1 = r.neiL >= 0 ? p.stOff[h.stStart + r.neiL + 1] : 0;
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
        for (int c : lc) { loc[c] = -1; }
        p.hdr[t] = h;
    }
    return true;
}

}  // namespace dugks
