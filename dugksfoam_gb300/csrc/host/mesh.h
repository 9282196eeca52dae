// Host-side finite-volume mesh data for the DUGKS engine.
//
// Geometry follows OpenFOAM primitiveMesh semantics (triangle-fan faces,
// pyramid-decomposed cells) and the fv layer the reference relies on:
// boundary delta d_b = n (n.(Cf - C_P)), deltaCoeff = 1/|d|, least-squares
// vectors with 1/|d|^2 weights over internal and non-empty boundary faces
// (zeroBoundaryGrad/invDistLeastSquaresVectors.C:100-172 in the reference).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dugks {

struct MeshInput {
    int nPoints = 0;
    const double* points = nullptr;
    int nCells = 0, nFaces = 0, nInternal = 0;
    const int32_t* faceOffsets = nullptr;
    const int32_t* faceVerts = nullptr;
    const int32_t* owner = nullptr;
    const int32_t* neighbour = nullptr;
    int nPatches = 0;
    const int32_t* patchStart = nullptr;
    const int32_t* patchSize = nullptr;
    const int32_t* patchKind = nullptr;  // dugks_patch_kind
};

struct Mesh {
    int nC = 0, nF = 0, nI = 0, nB = 0;
    int D = 3;                     // number of solution directions
    bool emptyDir[3] = {false, false, false};
    std::vector<double> C, V;      // cell centres [nC][3], volumes
    std::vector<double> Cf, Sf;    // all faces [nF][3]
    std::vector<int32_t> owner, neighbour;
    std::vector<int32_t> bKind;    // per boundary face
    std::vector<int32_t> bPatch;   // per boundary face
    // Active faces = internal faces followed by non-empty boundary faces
    // ("wall" faces below: every non-empty boundary face, whatever its kind).
    int nW = 0;                    // active boundary faces
    std::vector<int32_t> wallFace; // global face index of wall face w
    std::vector<int32_t> wallCell;
    std::vector<int32_t> wallPatch;
    std::vector<int32_t> wallKind; // dugks_patch_kind of boundary face w
    std::vector<int32_t> globalToWall; // boundary face b -> w or -1
    std::vector<double> dcI;       // internal deltaCoeffs [nI]
    std::vector<double> pVec, nVec;// internal LS vectors [nI][3]
    std::vector<double> bVec;      // wall LS vectors [nW][3]
    std::vector<double> dcW;       // wall deltaCoeffs [nW]
    std::vector<double> nHatW;     // wall unit normals [nW][3]
    // cell -> active faces, increasing global face index
    std::vector<int32_t> cellOff;  // [nC+1]
    std::vector<int32_t> cellFace; // active face index (internal f, or nI + w)
    std::vector<int8_t> cellSide;  // 0: cell is owner, 1: cell is neighbour
    std::vector<double> lerpW;     // linear interpolation weights (internal)
};

// Builds geometry, connectivity and LS vectors.  Returns false with a message
// on inconsistent input.
bool build_mesh(const MeshInput& in, Mesh& m, std::string& err);

}  // namespace dugks
