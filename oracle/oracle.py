"""TEST INFRASTRUCTURE ONLY: Python access to the FP64 DUGKS oracle.

* ``Oracle`` wraps oracle/_build/liboracle.so (the C restatement of
  fvDVM::evolution, src/fvDVM/fvDVM/fvDVM.C:1086-1108, in the reference's
  operation and summation order).  Used by tests, the smoke check and the
  benchmark's CPU leg only -- never by the engine.
* ``NumpyOracle`` is a second, independent restatement (numpy, DV-innermost
  arrays, vectorised) used to cross-check the C oracle on small meshes.

Parity status: UNPINNED (the reference has no golden outputs and cannot be
built without OpenFOAM + MPI); the DV-grid generator is pinned to the demo
case's Xis/weights files.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

PATCH_EMPTY = 0
PATCH_MAXWELL = 1
# rho boundary-condition type -> patch kind (dugks_oracle.h; the same numbering
# as the engine's dugks_patch_kind)
BC_KINDS = {"empty": 0, "calculatedMaxwell": 1, "zeroGradient": 2, "fixedValue": 3, "farField": 4,
            "pressureIn": 5, "pressureOut": 6, "symmetryMod": 7, "symmetryPlane": 8}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Case(C.Structure):
    _fields_ = [
        ("nPoints", C.c_int), ("points", _dp),
        ("nCells", C.c_int), ("nFaces", C.c_int), ("nInternalFaces", C.c_int),
        ("faceOffsets", _ip), ("faceVerts", _ip), ("owner", _ip), ("neighbour", _ip),
        ("nPatches", C.c_int), ("patchStart", _ip), ("patchSize", _ip), ("patchKind", _ip),
        ("Ub", _dp), ("Tb", _dp), ("rhob", _dp), ("patchPressure", _dp), ("patchTzg", _ip), ("patchUzg", _ip),
        ("nXiPerDim", C.c_int), ("xis", _dp), ("weights", _dp), ("xiMax", C.c_double),
        ("R", C.c_double), ("omega", C.c_double), ("Tref", C.c_double), ("muRef", C.c_double),
        ("Pr", C.c_double), ("KInner", C.c_int),
        ("rho0", _dp), ("U0", _dp), ("T0", _dp),
    ]


def build():
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = C.CDLL(LIB_PATH)
        lib.oracle_create.restype = C.c_void_p
        lib.oracle_create.argtypes = [C.POINTER(_Case)]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        lib.oracle_step.argtypes = [C.c_void_p, C.c_double, C.c_int]
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_nsolutiond.argtypes = [C.c_void_p]
        lib.oracle_ndv.argtypes = [C.c_void_p]
        for name in ("oracle_get_cell", "oracle_get_face"):
            getattr(lib, name).argtypes = [C.c_void_p] + [_dp] * 5
        lib.oracle_get_wall.argtypes = [C.c_void_p, _dp, _dp, _dp]
        lib.oracle_get_boundary.argtypes = [C.c_void_p, _dp, _dp, _dp]
        lib.oracle_get_dist.argtypes = [C.c_void_p, _dp, _dp]
        lib.oracle_set_dist.argtypes = [C.c_void_p, _dp, _dp]
        lib.oracle_get_geometry.argtypes = [C.c_void_p] + [_dp] * 8
        lib.oracle_get_dv.argtypes = [C.c_void_p, _dp, _dp]
        lib.oracle_conum.argtypes = [C.c_void_p, C.c_double, _dp, _dp]
        _lib = lib
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def patch_bc(p):
    """rho boundary-condition type of a case patch (explicit "bc", else from the mesh type)."""
    if "bc" in p:
        return p["bc"]
    return {"empty": "empty", "wall": "calculatedMaxwell", "symmetryPlane": "symmetryPlane"}[p["type"]]


def patch_zero_gradient(mesh, field):
    """Per patch: 1 when the boundary condition of ``field`` (U or T) is
    zeroGradient (patch entry "T_bc"/"U_bc" == "zeroGradient"), else 0."""
    return np.array([1 if p.get(field + "_bc") == "zeroGradient" else 0 for p in mesh["patches"]], np.int32)


def patch_kinds(mesh):
    return np.array([BC_KINDS[patch_bc(p)] for p in mesh["patches"]], np.int32)


class Oracle:
    """FP64 reference-order DUGKS step on the CPU (C restatement)."""

    def __init__(self, case, threads: int | None = None):
        lib = _load()
        if threads:
            lib.oracle_set_threads(int(threads))
        m = case["mesh"]
        g = case["gas"]
        keep = dict(
            points=np.ascontiguousarray(m["points"], np.float64),
            off=np.ascontiguousarray(m["face_offsets"], np.int32),
            fv=np.ascontiguousarray(m["face_verts"], np.int32),
            own=np.ascontiguousarray(m["owner"], np.int32),
            nei=np.ascontiguousarray(m["neighbour"], np.int32),
            ps=np.array([p["startFace"] for p in m["patches"]], np.int32),
            pn=np.array([p["nFaces"] for p in m["patches"]], np.int32),
            pk=patch_kinds(m),
            Ub=np.ascontiguousarray(case["Ub"], np.float64),
            Tb=np.ascontiguousarray(case["Tb"], np.float64),
            rhob=np.ascontiguousarray(case.get("rhob", np.zeros(len(case["Tb"]))), np.float64),
            pp=np.ascontiguousarray([p.get("pressure", 0.0) for p in m["patches"]], np.float64),
            tzg=patch_zero_gradient(m, "T"), uzg=patch_zero_gradient(m, "U"),
            xis=np.ascontiguousarray(case["xis"], np.float64),
            w=np.ascontiguousarray(case["weights"], np.float64),
            rho0=np.ascontiguousarray(case["rho0"], np.float64),
            U0=np.ascontiguousarray(case["U0"], np.float64),
            T0=np.ascontiguousarray(case["T0"], np.float64),
        )
        cs = _Case(
            nPoints=len(keep["points"]), points=_d(keep["points"]),
            nCells=int(m["n_cells"]), nFaces=len(keep["off"]) - 1, nInternalFaces=len(keep["nei"]),
            faceOffsets=_i(keep["off"]), faceVerts=_i(keep["fv"]), owner=_i(keep["own"]),
            neighbour=_i(keep["nei"]), nPatches=len(keep["ps"]), patchStart=_i(keep["ps"]),
            patchSize=_i(keep["pn"]), patchKind=_i(keep["pk"]), Ub=_d(keep["Ub"]), Tb=_d(keep["Tb"]),
            rhob=_d(keep["rhob"]), patchPressure=_d(keep["pp"]), patchTzg=_i(keep["tzg"]), patchUzg=_i(keep["uzg"]),
            nXiPerDim=len(keep["xis"]), xis=_d(keep["xis"]), weights=_d(keep["w"]),
            xiMax=float(case["xi_max"]), R=g["R"], omega=g["omega"], Tref=g["Tref"],
            muRef=g["muRef"], Pr=g["Pr"], KInner=int(g["KInner"]),
            rho0=_d(keep["rho0"]), U0=_d(keep["U0"]), T0=_d(keep["T0"]),
        )
        self._lib = lib
        self._h = lib.oracle_create(C.byref(cs))
        self.nC = int(m["n_cells"])
        self.nF = len(keep["off"]) - 1
        self.nI = len(keep["nei"])
        self.nB = self.nF - self.nI
        self.D = lib.oracle_nsolutiond(self._h)
        self.nV = lib.oracle_ndv(self._h)

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt, n=1):
        self._lib.oracle_step(self._h, float(dt), int(n))

    def cell(self):
        n = self.nC
        rho, U, T, q, tau = np.zeros(n), np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3)), np.zeros(n)
        self._lib.oracle_get_cell(self._h, _d(rho), _d(U), _d(T), _d(q), _d(tau))
        return dict(rho=rho, U=U, T=T, q=q, tau=tau)

    def face(self):
        n = self.nF
        rho, U, T, q, tau = np.zeros(n), np.zeros((n, 3)), np.zeros(n), np.zeros((n, 3)), np.zeros(n)
        self._lib.oracle_get_face(self._h, _d(rho), _d(U), _d(T), _d(q), _d(tau))
        return dict(rho=rho, U=U, T=T, q=q, tau=tau)

    def wall(self):
        n = self.nB
        r, q, s = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 9))
        self._lib.oracle_get_wall(self._h, _d(r), _d(q), _d(s))
        return dict(rhoW=r, qWall=q, stressWall=s)

    def boundary(self):
        n = self.nB
        r, U, T = np.zeros(n), np.zeros((n, 3)), np.zeros(n)
        self._lib.oracle_get_boundary(self._h, _d(r), _d(U), _d(T))
        return dict(rho=r, U=U, T=T)

    def dist(self):
        g = np.zeros((self.nV, self.nC))
        h = np.zeros((self.nV, self.nC))
        self._lib.oracle_get_dist(self._h, _d(g), _d(h))
        return g, h

    def set_dist(self, g, h):
        g = np.ascontiguousarray(g, np.float64)
        h = np.ascontiguousarray(h, np.float64)
        self._lib.oracle_set_dist(self._h, _d(g), _d(h))

    def geometry(self):
        nC, nF, nI, nB = self.nC, self.nF, self.nI, self.nB
        out = dict(C=np.zeros((nC, 3)), V=np.zeros(nC), Cf=np.zeros((nF, 3)), Sf=np.zeros((nF, 3)),
                   pVec=np.zeros((nI, 3)), nVec=np.zeros((nI, 3)), bVec=np.zeros((nB, 3)),
                   deltaCoeffs=np.zeros(nF))
        self._lib.oracle_get_geometry(self._h, *(_d(out[k]) for k in
                                                 ("C", "V", "Cf", "Sf", "pVec", "nVec", "bVec", "deltaCoeffs")))
        return out

    def dv(self):
        xi = np.zeros((self.nV, 3))
        w = np.zeros(self.nV)
        self._lib.oracle_get_dv(self._h, _d(xi), _d(w))
        return xi, w

    def conum(self, dt):
        a, b = C.c_double(), C.c_double()
        self._lib.oracle_conum(self._h, float(dt), C.byref(a), C.byref(b))
        return a.value, b.value


# --------------------------------------------------------------------------
class NumpyOracle:
    """Independent vectorised FP64 restatement (DV-innermost arrays).

    Same algorithm as fvDVM::evolution (fvDVM.C:1086-1108) written as whole-
    array operations: it does not share code or summation order with the C
    oracle, so agreement to ~1e-13 cross-checks both.  Small meshes only.
    Boundary types as the C oracle (every rho type of BC_KINDS); symmetry
    patches copy from a snapshot, which equals symmetryPlane's index-order
    assignment on grids symmetric about 0.
    """

    def __init__(self, case):
        o = Oracle(case)  # geometry and DV set from the C oracle's set-up
        geo = o.geometry()
        self.xi, self.w = o.dv()
        self.D = o.D
        o.close()
        m = case["mesh"]
        g = case["gas"]
        self.R, self.omega, self.Tref, self.muRef, self.Pr, self.K = (
            g["R"], g["omega"], g["Tref"], g["muRef"], g["Pr"], int(g["KInner"]))
        nF = len(m["face_offsets"]) - 1
        nI = len(m["neighbour"])
        self.nI = nI
        self.own = np.asarray(m["owner"][:nI])
        self.nei = np.asarray(m["neighbour"])
        kinds = np.zeros(nF - nI, np.int32)
        press = np.zeros(nF - nI)
        first = np.zeros(nF - nI, np.int64)
        zgT = np.zeros(nF - nI, bool)
        zgU = np.zeros(nF - nI, bool)
        for p in m["patches"]:
            sl = slice(p["startFace"] - nI, p["startFace"] - nI + p["nFaces"])
            kinds[sl] = BC_KINDS[patch_bc(p)]
            press[sl] = p.get("pressure", 0.0)
            first[sl] = p["startFace"]
            zgT[sl] = p.get("T_bc") == "zeroGradient"
            zgU[sl] = p.get("U_bc") == "zeroGradient"
        wall = np.nonzero(kinds != PATCH_EMPTY)[0]  # every active boundary face
        self.kind = kinds[wall]
        self.pB = press[wall]
        self.zgT, self.zgU = zgT[wall], zgU[wall]
        self.wb = wall
        self.wf = nI + wall
        self.wc = np.asarray(m["owner"])[self.wf]
        self.C, self.V = geo["C"], geo["V"]
        self.Cf, self.Sf = geo["Cf"], geo["Sf"]
        self.pV, self.nV_ = geo["pVec"], geo["nVec"]
        self.bV = geo["bVec"][wall]
        self.dcB = geo["deltaCoeffs"][nI:][wall]
        Sw = self.Sf[self.wf]
        self.nHat = Sw / np.linalg.norm(Sw, axis=1)[:, None]
        self.Uw = np.array(case["Ub"][wall], float)
        self.Tw = np.array(case["Tb"][wall], float)
        self.rhob = np.array(case.get("rhob", np.zeros(nF - nI))[wall], float)
        S0 = geo["Sf"][first[wall]]
        self.mirror = self._mirrors(S0)  # [nb][nV] mirror DV (symmetry faces)
        self.inS0 = (S0 @ self.xi.T) <= 0
        nC = m["n_cells"]
        self.rho = np.array(case["rho0"], float)
        self.U = np.array(case["U0"], float)
        self.T = np.array(case["T0"], float)
        self.q = np.zeros((nC, 3))
        self.g, self.h = self._shakhov(self.rho, self.U, self.T, self.q)
        self.tau = self._tau(self.T, self.rho)
        self.Gg = np.zeros((len(wall), len(self.w)))
        self.Gh = np.zeros_like(self.Gg)
        self._zero_gradient_tu()  # zeroGradient U/T patches start at the owner cells' values
        xs_w = Sw @ self.xi.T
        Tpos = np.where(self.Tw > 0, self.Tw, 1.0)
        M = self._maxwell(self.Uw, Tpos)
        self.inc = np.where(xs_w < 0, -self.w[None, :] * xs_w * M, 0.0).sum(1)
        # mixed (rho fixedValue): frozen Maxwellian of the initial patch values
        self.mixG = self.rhob[:, None] * M
        self.mixH = (self.K + 3 - self.D) * self.R * Tpos[:, None] * self.mixG
        self._pressure_bc()  # the constructor's initial update (fvDVM.C:1067-1071)

    def _mirrors(self, S0):
        """round(|n . (symX, symY, symZ)|) per face and DV (fvDVM.C:140-221)."""
        nV, D = len(self.w), self.D
        M = int(round(nV ** (1.0 / D)))
        v = np.arange(nV)
        ix = v % M
        iy = (v // M) % M if D == 3 else (v // M if D == 2 else 0 * v)
        iz = v // (M * M) if D == 3 else 0 * v
        if D == 3:
            sx = iz * M * M + iy * M + (M - ix - 1)
            sy = iz * M * M + (M - iy - 1) * M + ix
            sz = (M - iz - 1) * M * M + iy * M + ix
        elif D == 2:
            sx, sy, sz = iy * M + (M - ix - 1), (M - iy - 1) * M + ix, 0 * v
        else:
            sx, sy, sz = M - ix - 1, 0 * v, 0 * v
        n = S0 / np.linalg.norm(S0, axis=1)[:, None]
        t = np.rint(np.abs(n[:, 0:1] * sx + n[:, 1:2] * sy + n[:, 2:3] * sz)).astype(np.int64)
        return np.clip(t, 0, nV - 1)

    def _shakhov(self, rho, U, T, q):
        R, Pr, D, K = self.R, self.Pr, self.D, self.K
        c = self.xi[None, :, :] - U[:, None, :]
        RT = (R * T)[:, None]
        c2 = (c * c).sum(2) / RT
        cq = (c * q[:, None, :]).sum(2) / (5.0 * rho[:, None] * RT * RT)
        gB = rho[:, None] / (2 * np.pi * RT) ** (D / 2.0) * np.exp(-c2 / 2)
        p = (1 - Pr) * cq
        g = (1 + p * (c2 - D - 2)) * gB
        h = ((K + 3 - D) + p * ((c2 - D) * (K + 3 - D) - 2 * K)) * gB * RT
        return g, h

    def _maxwell(self, U, T):
        c = self.xi[None, :, :] - U[:, None, :]
        RT = (self.R * T)[:, None]
        return 1.0 / (2 * np.pi * RT) ** (self.D / 2.0) * np.exp(-(c * c).sum(2) / (2 * RT))

    def _tau(self, T, rho):
        return self.muRef * (T / self.Tref) ** self.omega / rho / T / self.R

    def _moments(self, g, h, dtfac):
        w = self.w[None, :]
        rho = (w * g).sum(1)
        U = (w[:, :, None] * g[:, :, None] * self.xi[None]).sum(1) / rho[:, None]
        E = 0.5 * (w * ((self.xi ** 2).sum(1)[None] * g + h)).sum(1)
        T = (E - 0.5 * rho * (U * U).sum(1)) / ((self.K + 3) / 2.0 * self.R * rho)
        tau = self._tau(T, rho)
        c = self.xi[None] - U[:, None]
        s = (c * c).sum(2) * g + h
        q = 0.5 * (w[:, :, None] * c * s[:, :, None]).sum(1)
        q *= (2 * tau / (2 * tau + dtfac * self.Pr))[:, None]
        return rho, U, T, tau, q

    def step(self, dt, n=1):
        for _ in range(n):
            self._step(dt)

    def _step(self, dt):
        nI = self.nI
        own, nei = self.own, self.nei
        xi = self.xi
        a = (1.5 * dt / (2 * self.tau + dt))[:, None]
        ge, he = self._shakhov(self.rho, self.U, self.T, self.q)
        gb = (1 - a) * self.g + a * ge
        hb = (1 - a) * self.h + a * he
        grads = []
        newG = []
        for f, G in ((gb, self.Gg), (hb, self.Gh)):
            d = f[nei] - f[own]
            grad = np.zeros(f.shape + (3,))
            np.add.at(grad, own, self.pV[:, None, :] * d[:, :, None])
            np.add.at(grad, nei, -self.nV_[:, None, :] * d[:, :, None])
            phib = f[self.wc] + G / self.dcB[:, None]
            phib = np.where((self.kind == 8)[:, None], f[self.wc], phib)  # symmetryPlane: internal value
            np.add.at(grad, self.wc, self.bV[:, None, :] * (phib - f[self.wc])[:, :, None])
            grads.append(grad)
            newG.append((grad[self.wc] * self.nHat[:, None, :]).sum(2))
        self.Gg, self.Gh = newG
        xsI = self.Sf[:nI] @ xi.T
        shift = 0.5 * xi * dt

        def recon(f, grad, cells, Cf):
            r = Cf[:, None, :] - self.C[cells][:, None, :] - shift[None]
            return f[cells] + (grad[cells] * r).sum(2)

        gs = []
        for f, grad in ((gb, grads[0]), (hb, grads[1])):
            fo = recon(f, grad, own, self.Cf[:nI])
            fn = recon(f, grad, nei, self.Cf[:nI])
            gs.append(np.where(xsI >= 1e-300, fo, np.where(xsI < -1e-300, fn, 0.5 * (fn + fo))))
        gI, hI = gs
        xsW = self.Sf[self.wf] @ xi.T
        gWo = recon(gb, grads[0], self.wc, self.Cf[self.wf])
        hWo = recon(hb, grads[1], self.wc, self.Cf[self.wf])
        out = np.where(xsW > 0, self.w[None] * xsW * gWo, 0.0).sum(1)
        rhoW = out / np.abs(self.inc)
        k = self.kind[:, None]
        Tpos = np.where(self.Tw > 0, self.Tw, 1.0)
        hfac = (self.R * Tpos)[:, None] * (self.K + 3 - self.D)
        Mw = rhoW[:, None] * self._maxwell(self.Uw, Tpos)
        Mf = self.rhob[:, None] * self._maxwell(self.U[self.wc], Tpos)  # farField / pressure incoming
        sym = (k == 7) | (k == 8)
        out_ = np.where(sym, xsW > -1e-300, xsW > 0)
        rows = np.arange(len(self.wc))[:, None]
        gM, hM = gWo[rows, self.mirror], hWo[rows, self.mirror]
        gIn = np.select([k == 1, k == 3, (k >= 4) & (k <= 6)], [Mw, self.mixG, Mf], gM)
        hIn = np.select([k == 1, k == 3, (k >= 4) & (k <= 6)], [Mw * hfac, self.mixH, Mf * hfac], hM)
        inc = np.where(sym, self.inS0, ~out_)
        gW = np.where(inc, gIn, gWo)
        hW = np.where(inc, hIn, hWo)
        zg = k == 2
        gW = np.where(zg, gb[self.wc], gW)
        hW = np.where(zg, hb[self.wc], hW)
        gF = np.concatenate([gI, gW])
        hF = np.concatenate([hI, hW])
        rF, UF, TF, tF, qF = self._moments(gF, hF, 0.5 * dt)
        b = (0.5 * dt / (2 * tF + 0.5 * dt))[:, None]
        geF, heF = self._shakhov(rF, UF, TF, qF)
        plane = np.concatenate([np.zeros_like(xsI, bool), np.broadcast_to(k == 8, xsW.shape)])
        gF = np.where(plane, (1 - b) * gF + b * geF, gF)  # symmetryPlane takes the field assignment
        hF = np.where(plane, (1 - b) * hF + b * heF, hF)
        relax = np.concatenate([np.ones_like(xsI, bool), xsW > 0])
        gF = np.where(relax, (1 - b) * gF + b * geF, gF)
        hF = np.where(relax, (1 - b) * hF + b * heF, hF)
        gt = -1.0 / 3 * self.g + 4.0 / 3 * gb
        ht = -1.0 / 3 * self.h + 4.0 / 3 * hb
        xsA = np.concatenate([xsI, xsW])
        Vo = self.V
        fo = np.concatenate([own, self.wc])
        for t, f in ((gt, gF), (ht, hF)):
            flux = xsA * f * dt
            np.add.at(t, fo, -flux / Vo[fo][:, None])
            np.add.at(t, nei, flux[:nI] / Vo[nei][:, None])
        self.g, self.h = gt, ht
        self.rho, self.U, self.T, self.tau, self.q = self._moments(self.g, self.h, dt)
        self.faces = dict(rho=rF, U=UF, T=TF, q=qF, tau=tF, rhoW=rhoW)
        self._zero_gradient_tu()
        self._pressure_bc()

    def _zero_gradient_tu(self):
        """U/T correctBoundaryConditions (fvDVM.C:697-699): zeroGradient patches
        take their owner cells' values."""
        self.Tw = np.where(self.zgT, self.T[self.wc], self.Tw)
        self.Uw = np.where(self.zgU[:, None], self.U[self.wc], self.Uw)

    def _pressure_bc(self):
        """fvDVM::updatePressureInOutBC (fvDVM.C:730-806) from the current cell macros."""
        R, K = self.R, self.K
        for i in np.nonzero((self.kind == 5) | (self.kind == 6))[0]:
            c = self.wc[i]
            S = self.Sf[self.wf[i]]
            n = S / np.sqrt((S * S).sum())
            Ui, Ti, ri, p = self.U[c], self.T[c], self.rho[c], self.pB[i]
            ai = np.sqrt(R * Ti * (K + 5) / (K + 3))
            Un = (Ui * n).sum()
            if self.kind[i] == 5:
                self.rhob[i] = p / R / self.Tw[i]
                UnIn = Un + (p - ri * R * Ti) / ri / ai
            else:
                self.rhob[i] = ri + (p - ri * R * Ti) / ai / ai
                self.Tw[i] = p / (R * ri)
                UnIn = Un + (ri * R * Ti - p) / ri / ai
            self.Uw[i] = UnIn * n + (Ui - Un * n)


    def cell(self):
        return dict(rho=self.rho.copy(), U=self.U.copy(), T=self.T.copy(), q=self.q.copy(),
                    tau=self.tau.copy())
