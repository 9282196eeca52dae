// OpenFOAM ASCII case I/O for the DUGKS engine.
//
// Reads the inputs dugksFoam reads (src/dugksFoam.C:48-54, createFields.H,
// fvDVM.C:886-933, fvDVM.C:56-117): constant/polyMesh/{points,faces,owner,
// neighbour,boundary}, 0/{rho,U,T}, constant/DVMProperties,
// constant/{Xis,weights}, system/controlDict.  Writes volume fields in the
// same ASCII format (runTime.write(), dugksFoam.C:81).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace dugks {

struct FoamCase {
    // mesh
    std::vector<double> points;
    std::vector<int32_t> faceOffsets, faceVerts, owner, neighbour;
    int nCells = 0, nFaces = 0, nInternal = 0;
    std::vector<std::string> patchNames, patchTypes;   // polyMesh boundary
    std::vector<int32_t> patchStart, patchSize;
    std::vector<std::string> rhoBC;                     // 0/rho patch types
    std::vector<int32_t> patchKind;                     // dugks_patch_kind
    // fields
    std::vector<double> rho0, U0, T0;                   // internal
    std::vector<double> wallU, wallT;                   // U, T patch values per boundary face
    std::vector<double> bndRho;                         // rho patch values per boundary face
    std::vector<double> patchPressure;                  // pressureIn / pressureOut per patch
    std::vector<int32_t> patchTzg, patchUzg;            // per patch: 0/T, 0/U type zeroGradient
    // DVMProperties
    int nDV = 0;
    double xiMax = 0, xiMin = 0;
    double R = 0, omega = 0, Tref = 0, muRef = 0, Pr = 0;
    int KInner = 0;
    std::string macroFlux = "no";
    std::vector<double> xis, weights;
    std::vector<int32_t> dfCells;                       // DFwriteCellList
    // controlDict
    std::map<std::string, std::string> control;
    double deltaT = 0;
};

bool read_foam_case(const std::string& dir, FoamCase& c, std::string& err);

// An OpenFOAM scalarList file (class scalarList, 17 significant digits).
bool write_scalar_list(const std::string& path, const std::string& object, const double* v, int n,
                       std::string& err);

// One patch of a written vol field: "empty" patches carry no value.
struct PatchOut {
    std::string name, type;
    std::vector<double> values;  // ncomp per face
    std::string extra;           // one more "keyword value" entry (e.g. "pressureIn 1e5"), or empty
};

// Write a vol field in OpenFOAM ASCII (volScalarField / volVectorField /
// volTensorField by ncomp = 1 / 3 / 9), full double precision (17 digits).
// internal == nullptr writes a uniform zero internal field.
bool write_vol_field(const std::string& path, const std::string& name, const std::string& dims, int ncomp,
                     const double* internal, int n, const std::vector<PatchOut>& patches, std::string& err);

}  // namespace dugks
