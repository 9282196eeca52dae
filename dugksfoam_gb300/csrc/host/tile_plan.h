// Tile plan for the fused sweeps: cells grouped into spatially compact tiles
// (Morton order of centroids), each with the two rings of neighbour cells the
// on-chip least-squares gradient and upwind reconstruction need.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "mesh.h"

namespace dugks {

// Per-tile header (device-visible POD).
struct TileHdr {
    int32_t cellStart;   // into tileCells
    int32_t nT, nT1, nT2;// |T|, |T u H1|, |T u H1 u H2|; local cells ordered T, H1, H2
    int32_t stStart;     // into stOff (nT1+1 entries from here)
    int32_t faceStart;   // into face arrays
    int32_t nFA;         // faces owned by the tile (sweep A): internal faces with owner in T, walls of T
    int32_t nFB;         // all faces of T's cells (sweep B); the first nFA are the owned ones
    int32_t colStart;    // into colorPerm / colorOff
    int32_t nColors;
    int32_t permStart;   // into colorPerm (nFB entries, grouped by colour)
    int32_t nEnt;        // stencil entries of T u H1 (from stOff[stStart])
};

// Face record (device-visible POD).
struct TileFace {
    int32_t ownL, neiL;  // local cell indices (neiL = -1 on walls)
    int32_t a;           // active face index (internal f, or nI + wall)
    int32_t w;           // wall index or -1
    int32_t stO0, stO1;  // stencil entries [stO0, stO1) of the owner cell
    int32_t stN0, stN1;  // stencil entries of the neighbour cell (empty on walls)
};

struct TilePlan {
    int nTiles = 0, tileCells = 0;
    int maxT = 0, maxT2 = 0, maxFA = 0, maxFB = 0;
    long long sumT = 0, sumT2 = 0;  // halo ratio = sumT2 / sumT
    std::vector<TileHdr> hdr;
    std::vector<int32_t> cells;     // local -> global cell
    std::vector<int32_t> stOff;     // per tile (nT1+1) offsets into stEnt (absolute)
    std::vector<int32_t> stEnt;     // other local cell (>= 0) or -(wall+1)
    std::vector<double> stL;        // [nEnt][3] least-squares vector of the entry
    std::vector<TileFace> faces;    // per tile nFB records
    std::vector<int32_t> colorOff;  // per tile nColors+1 (relative to the tile's face block)
    std::vector<int32_t> colorPerm; // per tile nFB local face ids grouped by colour
};

// Sizes of one tile: |T|, |T u H1|, |T u H1 u H2|, owned faces (sweep A),
// faces of T's cells (sweep B) and stencil entries of T u H1.
struct TileDims {
    int nT = 0, nT1 = 0, nT2 = 0, nFA = 0, nFB = 0, nEnt = 0;
};

// Shared-memory bytes a tile needs.
using SmemFn = std::function<size_t(const TileDims&)>;

// Build the plan: compact BFS tiles of at most maxTileCells cells, each the
// largest that fits `budget` bytes of shared memory.
//
// rings = 2: rows of T u H1 u H2, stencils of T u H1 (a face's two upwind
// candidates both have their gradients in the tile).  rings = 1: rows of
// T u H1, stencils of T only (nT2 == nT1); a face's stencil range is set for
// the sides whose cell is in T and empty otherwise.
//
// waveSlots > 0 (tiles that run at once: SMs x tiles per SM): after the
// largest fitting tile size is found, the tiles are shrunk to the smallest
// size whose count still fills the same number of waves, so that the last
// wave is (nearly) full instead of leaving SMs idle.
bool build_tile_plan(const Mesh& m, int maxTileCells, const SmemFn& smem, size_t budget, TilePlan& p,
                     std::string& err, int rings = 2, int waveSlots = 0);

}  // namespace dugks
