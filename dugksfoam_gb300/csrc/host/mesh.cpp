// Mesh geometry, connectivity and least-squares vectors (see mesh.h).
#include "mesh.h"

#include <cmath>
#include <cstring>

#include "dugks/dugks.h"

namespace dugks {
namespace {

struct V3 {
    double x, y, z;
};
inline V3 v3(const double* p) { return {p[0], p[1], p[2]}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double magSqr(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline void put(double* p, V3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }

// Face centre and area vector: exact for triangles, triangle fan about the
// vertex average otherwise (primitiveMesh::makeFaceCentresAndAreas).
void faceGeometry(const double* pts, const int32_t* fv, int n, V3& Cf, V3& Sf) {
    if (n == 3) {
        V3 p0 = v3(pts + 3 * fv[0]), p1 = v3(pts + 3 * fv[1]), p2 = v3(pts + 3 * fv[2]);
        Cf = (1.0 / 3.0) * V3{p0.x + p1.x + p2.x, p0.y + p1.y + p2.y, p0.z + p1.z + p2.z};
        Sf = 0.5 * cross(p1 - p0, p2 - p0);
        return;
    }
    V3 avg{0, 0, 0};
    for (int i = 0; i < n; ++i) avg = avg + v3(pts + 3 * fv[i]);
    avg = {avg.x / n, avg.y / n, avg.z / n};
    V3 sumN{0, 0, 0}, sumAc{0, 0, 0};
    double sumA = 0.0;
    for (int i = 0; i < n; ++i) {
        V3 p = v3(pts + 3 * fv[i]);
        V3 pn = v3(pts + 3 * fv[(i + 1) % n]);
        V3 c = V3{p.x + pn.x + avg.x, p.y + pn.y + avg.y, p.z + pn.z + avg.z};
        V3 nv = cross(pn - p, avg - p);
        double a = std::sqrt(magSqr(nv));
        sumN = sumN + nv;
        sumA += a;
        sumAc = sumAc + a * c;
    }
    if (sumA < 1e-150) {
        Cf = avg;
        Sf = {0, 0, 0};
    } else {
        Cf = V3{(1.0 / 3.0) * sumAc.x / sumA, (1.0 / 3.0) * sumAc.y / sumA, (1.0 / 3.0) * sumAc.z / sumA};
        Sf = 0.5 * sumN;
    }
}

// Symmetric 3x3 (xx,xy,xz,yy,yz,zz) inverse by the adjugate.
void invSymm(const double* t, double* r) {
    const double xx = t[0], xy = t[1], xz = t[2], yy = t[3], yz = t[4], zz = t[5];
    const double det = xx * yy * zz + xy * yz * xz + xz * xy * yz - xx * yz * yz - xy * xy * zz - xz * yy * xz;
    r[0] = (yy * zz - yz * yz) / det;
    r[1] = (xz * yz - xy * zz) / det;
    r[2] = (xy * yz - xz * yy) / det;
    r[3] = (xx * zz - xz * xz) / det;
    r[4] = (xy * xz - xx * yz) / det;
    r[5] = (xx * yy - xy * xy) / det;
}

V3 symmDot(const double* t, V3 d) {
    return {t[0] * d.x + t[1] * d.y + t[2] * d.z, t[1] * d.x + t[3] * d.y + t[4] * d.z,
            t[2] * d.x + t[4] * d.y + t[5] * d.z};
}

}  // namespace

bool build_mesh(const MeshInput& in, Mesh& m, std::string& err) {
    const int nC = in.nCells, nF = in.nFaces, nI = in.nInternal, nB = nF - nI;
    if (nC <= 0 || nF <= 0 || nI < 0 || nB < 0 || !in.points || !in.faceOffsets || !in.faceVerts || !in.owner ||
        (nI > 0 && !in.neighbour)) {
        err = "mesh: missing or inconsistent sizes/pointers";
        return false;
    }
    m.nC = nC; m.nF = nF; m.nI = nI; m.nB = nB;
    m.owner.assign(in.owner, in.owner + nF);
    m.neighbour.assign(in.neighbour, in.neighbour + nI);
    for (int f = 0; f < nF; ++f) {
        if (m.owner[f] < 0 || m.owner[f] >= nC) { err = "mesh: owner index out of range"; return false; }
        int n = in.faceOffsets[f + 1] - in.faceOffsets[f];
        if (n < 3) { err = "mesh: face with fewer than 3 vertices"; return false; }
        for (int k = in.faceOffsets[f]; k < in.faceOffsets[f + 1]; ++k)
            if (in.faceVerts[k] < 0 || in.faceVerts[k] >= in.nPoints) { err = "mesh: point index out of range"; return false; }
    }
    for (int f = 0; f < nI; ++f)
        if (m.neighbour[f] < 0 || m.neighbour[f] >= nC || m.neighbour[f] == m.owner[f]) {
            err = "mesh: neighbour index out of range";
            return false;
        }
    m.bKind.assign(nB, -1);
    m.bPatch.assign(nB, -1);
    for (int p = 0; p < in.nPatches; ++p) {
        int s = in.patchStart[p] - nI, e = s + in.patchSize[p];
        if (s < 0 || e > nB) { err = "mesh: patch range outside boundary faces"; return false; }
        int kind = in.patchKind[p];
        if (kind < DUGKS_PATCH_EMPTY || kind > DUGKS_PATCH_SYMMETRY_PLANE) {
            err = "mesh: unsupported patch kind";
            return false;
        }
        for (int b = s; b < e; ++b) { m.bKind[b] = kind; m.bPatch[b] = p; }
    }
    for (int b = 0; b < nB; ++b)
        if (m.bKind[b] < 0) { err = "mesh: boundary face not covered by any patch"; return false; }

    // ---- primitiveMesh geometry (all faces, empty ones included)
    m.Cf.assign(3 * (size_t)nF, 0.0);
    m.Sf.assign(3 * (size_t)nF, 0.0);
    for (int f = 0; f < nF; ++f) {
        V3 cf, sf;
        faceGeometry(in.points, in.faceVerts + in.faceOffsets[f], in.faceOffsets[f + 1] - in.faceOffsets[f], cf, sf);
        put(&m.Cf[3 * f], cf);
        put(&m.Sf[3 * f], sf);
    }
    std::vector<V3> cEst(nC, V3{0, 0, 0});
    std::vector<int> nCF(nC, 0);
    for (int f = 0; f < nF; ++f) { cEst[m.owner[f]] = cEst[m.owner[f]] + v3(&m.Cf[3 * f]); nCF[m.owner[f]]++; }
    for (int f = 0; f < nI; ++f) { cEst[m.neighbour[f]] = cEst[m.neighbour[f]] + v3(&m.Cf[3 * f]); nCF[m.neighbour[f]]++; }
    for (int c = 0; c < nC; ++c) {
        if (nCF[c] == 0) { err = "mesh: cell without faces"; return false; }
        cEst[c] = {cEst[c].x / nCF[c], cEst[c].y / nCF[c], cEst[c].z / nCF[c]};
    }
    std::vector<V3> cC(nC, V3{0, 0, 0});
    m.V.assign(nC, 0.0);
    for (int f = 0; f < nF; ++f) {
        int o = m.owner[f];
        V3 cf = v3(&m.Cf[3 * f]);
        double pyr3 = dot(v3(&m.Sf[3 * f]), cf - cEst[o]);
        V3 pc = (3.0 / 4.0) * cf + (1.0 / 4.0) * cEst[o];
        cC[o] = cC[o] + pyr3 * pc;
        m.V[o] += pyr3;
    }
    for (int f = 0; f < nI; ++f) {
        int n = m.neighbour[f];
        V3 cf = v3(&m.Cf[3 * f]);
        double pyr3 = dot(v3(&m.Sf[3 * f]), cEst[n] - cf);
        V3 pc = (3.0 / 4.0) * cf + (1.0 / 4.0) * cEst[n];
        cC[n] = cC[n] + pyr3 * pc;
        m.V[n] += pyr3;
    }
    m.C.assign(3 * (size_t)nC, 0.0);
    for (int c = 0; c < nC; ++c) {
        if (!(m.V[c] > 0.0)) { err = "mesh: non-positive cell volume (check face orientation)"; return false; }
        put(&m.C[3 * c], V3{cC[c].x / m.V[c], cC[c].y / m.V[c], cC[c].z / m.V[c]});
        m.V[c] *= (1.0 / 3.0);
    }

    // ---- solution directions from the empty patches' normals
    double ed[3] = {0, 0, 0};
    int nEmpty = 0;
    for (int b = 0; b < nB; ++b) {
        if (m.bKind[b] != DUGKS_PATCH_EMPTY) continue;
        const double* s = &m.Sf[3 * (nI + b)];
        double mg = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
        for (int k = 0; k < 3; ++k) ed[k] += std::fabs(s[k]) / mg;
        nEmpty++;
    }
    m.D = 3;
    if (nEmpty) {
        double mg = std::sqrt(ed[0] * ed[0] + ed[1] * ed[1] + ed[2] * ed[2]);
        for (int k = 0; k < 3; ++k)
            if (ed[k] / mg > 1e-6) { m.emptyDir[k] = true; m.D--; }
    }

    // ---- wall (active boundary) faces
    m.globalToWall.assign(nB, -1);
    m.wallFace.clear(); m.wallCell.clear(); m.wallPatch.clear(); m.wallKind.clear();
    for (int b = 0; b < nB; ++b) {
        if (m.bKind[b] == DUGKS_PATCH_EMPTY) continue;
        m.globalToWall[b] = (int)m.wallFace.size();
        m.wallFace.push_back(nI + b);
        m.wallCell.push_back(m.owner[nI + b]);
        m.wallPatch.push_back(m.bPatch[b]);
        m.wallKind.push_back(m.bKind[b]);
    }
    m.nW = (int)m.wallFace.size();

    // ---- deltas and deltaCoeffs
    m.dcI.assign(nI, 0.0);
    for (int f = 0; f < nI; ++f) {
        V3 d = v3(&m.C[3 * m.neighbour[f]]) - v3(&m.C[3 * m.owner[f]]);
        m.dcI[f] = 1.0 / std::sqrt(magSqr(d));
    }
    std::vector<V3> dW(m.nW);
    m.dcW.assign(m.nW, 0.0);
    m.nHatW.assign(3 * (size_t)m.nW, 0.0);
    for (int w = 0; w < m.nW; ++w) {
        int f = m.wallFace[w], P = m.wallCell[w];
        V3 S = v3(&m.Sf[3 * f]);
        double magSf = std::sqrt(magSqr(S));
        V3 n{S.x / magSf, S.y / magSf, S.z / magSf};
        double s = dot(n, v3(&m.Cf[3 * f]) - v3(&m.C[3 * P]));
        dW[w] = s * n;
        put(&m.nHatW[3 * w], n);
        m.dcW[w] = 1.0 / std::sqrt(magSqr(dW[w]));
    }

    // ---- least-squares vectors
    std::vector<double> dd(6 * (size_t)nC, 0.0);
    auto addW = [&](int c, V3 d) {
        double m2 = magSqr(d);
        double w6[6] = {d.x * d.x / m2, d.x * d.y / m2, d.x * d.z / m2, d.y * d.y / m2, d.y * d.z / m2, d.z * d.z / m2};
        for (int k = 0; k < 6; ++k) dd[6 * (size_t)c + k] += w6[k];
    };
    for (int f = 0; f < nI; ++f) {
        V3 d = v3(&m.C[3 * m.neighbour[f]]) - v3(&m.C[3 * m.owner[f]]);
        addW(m.owner[f], d);
        addW(m.neighbour[f], d);
    }
    for (int w = 0; w < m.nW; ++w) addW(m.wallCell[w], dW[w]);
    std::vector<double> inv(6 * (size_t)nC);
    const int diag[3] = {0, 3, 5};
    for (int c = 0; c < nC; ++c) {
        double t[6];
        std::memcpy(t, &dd[6 * (size_t)c], sizeof(t));
        for (int k = 0; k < 3; ++k) if (m.emptyDir[k]) t[diag[k]] += 1.0;
        invSymm(t, &inv[6 * (size_t)c]);
        for (int k = 0; k < 3; ++k) if (m.emptyDir[k]) inv[6 * (size_t)c + diag[k]] -= 1.0;
        for (int k = 0; k < 6; ++k)
            if (!std::isfinite(inv[6 * (size_t)c + k])) { err = "mesh: singular least-squares matrix"; return false; }
    }
    m.pVec.assign(3 * (size_t)nI, 0.0);
    m.nVec.assign(3 * (size_t)nI, 0.0);
    for (int f = 0; f < nI; ++f) {
        int o = m.owner[f], n = m.neighbour[f];
        V3 d = v3(&m.C[3 * n]) - v3(&m.C[3 * o]);
        double m2 = magSqr(d);
        V3 a = symmDot(&inv[6 * (size_t)o], d), b = symmDot(&inv[6 * (size_t)n], d);
        put(&m.pVec[3 * f], V3{a.x / m2, a.y / m2, a.z / m2});
        put(&m.nVec[3 * f], V3{-(b.x / m2), -(b.y / m2), -(b.z / m2)});
    }
    m.bVec.assign(3 * (size_t)m.nW, 0.0);
    for (int w = 0; w < m.nW; ++w) {
        double m2 = magSqr(dW[w]);
        V3 a = symmDot(&inv[6 * (size_t)m.wallCell[w]], dW[w]);
        put(&m.bVec[3 * w], V3{a.x / m2, a.y / m2, a.z / m2});
    }

    // ---- cell -> active faces (increasing global face index)
    m.cellOff.assign(nC + 1, 0);
    for (int f = 0; f < nI; ++f) { m.cellOff[m.owner[f] + 1]++; m.cellOff[m.neighbour[f] + 1]++; }
    for (int w = 0; w < m.nW; ++w) m.cellOff[m.wallCell[w] + 1]++;
    for (int c = 0; c < nC; ++c) m.cellOff[c + 1] += m.cellOff[c];
    m.cellFace.assign(m.cellOff[nC], 0);
    m.cellSide.assign(m.cellOff[nC], 0);
    std::vector<int> fill(nC, 0);
    for (int f = 0; f < nF; ++f) {
        if (f < nI) {
            int o = m.owner[f], n = m.neighbour[f];
            int jo = m.cellOff[o] + fill[o]++, jn = m.cellOff[n] + fill[n]++;
            m.cellFace[jo] = f; m.cellSide[jo] = 0;
            m.cellFace[jn] = f; m.cellSide[jn] = 1;
        } else {
            int w = m.globalToWall[f - nI];
            if (w < 0) continue;
            int o = m.owner[f];
            int j = m.cellOff[o] + fill[o]++;
            m.cellFace[j] = nI + w;
            m.cellSide[j] = 0;
        }
    }

    // ---- linear interpolation weights (surfaceInterpolation::makeWeights)
    m.lerpW.assign(nI, 0.5);
    for (int f = 0; f < nI; ++f) {
        V3 S = v3(&m.Sf[3 * f]), cf = v3(&m.Cf[3 * f]);
        double so = std::fabs(dot(S, cf - v3(&m.C[3 * m.owner[f]])));
        double sn = std::fabs(dot(S, v3(&m.C[3 * m.neighbour[f]]) - cf));
        m.lerpW[f] = sn / (so + sn);
    }
    return true;
}

}  // namespace dugks
