"""Vectorised mesh geometry for case preparation (time-step sizing, checks).

Face centres/areas use the triangle fan about the point average and cell
centres/volumes the pyramid decomposition about the face-centre average
(OpenFOAM primitiveMesh semantics).  The engine computes its own geometry in
C++ (csrc/host/mesh.cpp); this module only sizes dt and checks cases.
"""
from __future__ import annotations

import numpy as np

__all__ = ["face_centres_areas", "cell_centres_volumes"]


def face_centres_areas(mesh):
    pts = mesh["points"]
    off = mesh["face_offsets"]
    fv = mesh["face_verts"]
    nF = len(off) - 1
    Cf = np.zeros((nF, 3))
    Sf = np.zeros((nF, 3))
    sizes = np.diff(off)
    for n in np.unique(sizes):
        sel = np.nonzero(sizes == n)[0]
        idx = off[sel][:, None] + np.arange(n)[None, :]
        P = pts[fv[idx]]  # (m, n, 3)
        if n == 3:
            Cf[sel] = (1.0 / 3.0) * (P[:, 0] + P[:, 1] + P[:, 2])
            Sf[sel] = 0.5 * np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
            continue
        fc = P.mean(1)
        Pn = np.roll(P, -1, axis=1)
        c = P + Pn + fc[:, None, :]
        nv = np.cross(Pn - P, fc[:, None, :] - P)
        a = np.sqrt((nv * nv).sum(2))
        sumA = a.sum(1)
        Cf[sel] = (1.0 / 3.0) * (a[:, :, None] * c).sum(1) / sumA[:, None]
        Sf[sel] = 0.5 * nv.sum(1)
    return Cf, Sf


def cell_centres_volumes(mesh):
    Cf, Sf = face_centres_areas(mesh)
    own = mesh["owner"]
    nei = mesh["neighbour"]
    nI = len(nei)
    nC = mesh["n_cells"]
    cEst = np.zeros((nC, 3))
    cnt = np.zeros(nC)
    np.add.at(cEst, own, Cf)
    np.add.at(cnt, own, 1)
    np.add.at(cEst, nei, Cf[:nI])
    np.add.at(cnt, nei, 1)
    cEst /= cnt[:, None]
    pyr = (Sf * (Cf - cEst[own])).sum(1)
    pc = 0.75 * Cf + 0.25 * cEst[own]
    C = np.zeros((nC, 3))
    V = np.zeros(nC)
    np.add.at(C, own, pyr[:, None] * pc)
    np.add.at(V, own, pyr)
    pyr = (Sf[:nI] * (cEst[nei] - Cf[:nI])).sum(1)
    pc = 0.75 * Cf[:nI] + 0.25 * cEst[nei]
    np.add.at(C, nei, pyr[:, None] * pc)
    np.add.at(V, nei, pyr)
    C /= V[:, None]
    V /= 3.0
    return C, V
