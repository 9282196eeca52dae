"""Synthetic DUGKS cases: OpenFOAM-ordered meshes, gas parameters, DV grids.

A case is a plain dict of numpy arrays that both the C-ABI descriptor
(``dugks_case_desc``) and the OpenFOAM case writer (``foamio.write_case``)
consume.  Meshes follow OpenFOAM polyMesh conventions: internal faces first,
sorted by (owner, neighbour) with owner < neighbour and the face normal
pointing owner -> neighbour; boundary faces grouped by patch with outward
normals; 2D meshes are one cell thick with an ``empty`` front/back patch.

Gas parameters follow the demo case's ``para.py`` (demo/cavity/para.py:20-46):
hard-sphere mu-bar from Kn, argon mass and diameter for rho0, and
mu_ref = rho0 * sqrt(2 R T0) * L * mu-bar.

Named workloads (all lid-driven cavities with diffuse Maxwell walls):

* ``cavity2d``      -- N x N uniform quads (61 x 61, Kn 0.075, 28^2 DVs: the
                       CPU-runnable case);
* ``delaunay2d``    -- ~100k seeded Delaunay triangles extruded to prisms
                       (49 200 uniform interior points + 400 nodes per side,
                       Kn 0.01, 32^2 DVs);
* ``cavity3d``      -- 48^3 uniform hexes (Kn 0.1, 20^3 DVs);
* ``batch_instances`` -- seeded instance list for the batched runner;
* ``cavity2d`` with ``bottom_patch=True`` -- the 128^2 adjoint case.
"""
from __future__ import annotations

import math

import numpy as np

from .dvgrid import gauss_hermite_half_range, newton_cotes

__all__ = [
    "gas_from_kn", "structured_mesh", "delaunay_mesh", "make_case", "cavity2d",
    "delaunay2d", "cavity3d", "batch_instances", "stable_dt", "cell_stable_dt", "case_dt", "mesh_info",
]

K_BOLTZ = 1.38066e-23
M_ARGON = 6.63e-26
D_ARGON = 4.17e-10


def gas_from_kn(Kn: float, R: float = 208.0, T0: float = 273.0, L: float = 1.0,
                omega: float = 0.81, Pr: float = 2.0 / 3.0):
    """Gas properties and rho0 for a given Knudsen number (para.py:20-46)."""
    alpha, omega_hs = 1.0, 0.5
    mu_bar = 5.0 * (alpha + 1.0) * (alpha + 2.0) * math.sqrt(math.pi) * Kn / (
        4.0 * alpha * (5.0 - 2 * omega_hs) * (7.0 - 2.0 * omega_hs))
    mfp = L * Kn
    rho0 = M_ARGON / (mfp * math.sqrt(2.0) * math.pi * D_ARGON * D_ARGON)
    C = math.sqrt(2 * R * T0)
    mu = rho0 * C * L * mu_bar
    return dict(R=R, omega=omega, Tref=T0, muRef=mu, Pr=Pr, KInner=0), rho0


# ----------------------------------------------------------------- meshes
def _sort_internal(owner, neigh, faces):
    order = np.lexsort((neigh, owner))
    return owner[order], neigh[order], faces[order]


def structured_mesh(nx: int, ny: int, nz: int = 1, lx=1.0, ly=1.0, lz=None, two_d=True,
                    bottom_patch=False, patch_defs=None):
    """Uniform hex mesh of [0,lx]x[0,ly]x[0,lz] in OpenFOAM order.

    2D (two_d=True): nz must be 1 and front/back form an ``empty`` patch.
    Patches: movingWall (y = ly), fixedWalls (the other walls; bottomWall
    separately when ``bottom_patch``), frontAndBack (2D only).  ``patch_defs``
    replaces them: a list of (name, mesh type, sides, rho boundary type or
    None) with sides among x0 x1 y0 y1 z0 z1 (2D adds frontAndBack itself).
    """
    if two_d:
        assert nz == 1
        lz = (lx / nx) if lz is None else lz
    else:
        lz = lz if lz is not None else 1.0
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    zs = np.linspace(0.0, lz, nz + 1)
    P = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i  # noqa: E731
    Cl = lambda i, j, k: (k * ny + j) * nx + i  # noqa: E731
    kk, jj, ii = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    points = np.stack([xs[ii.ravel()], ys[jj.ravel()], zs[kk.ravel()]], axis=1)

    own, nei, fcs = [], [], []
    # x-faces, normal +x
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(1, nx), indexing="ij")
    k, j, i = k.ravel(), j.ravel(), i.ravel()
    own.append(Cl(i - 1, j, k)); nei.append(Cl(i, j, k))
    fcs.append(np.stack([P(i, j, k), P(i, j + 1, k), P(i, j + 1, k + 1), P(i, j, k + 1)], 1))
    # y-faces, normal +y
    k, j, i = np.meshgrid(np.arange(nz), np.arange(1, ny), np.arange(nx), indexing="ij")
    k, j, i = k.ravel(), j.ravel(), i.ravel()
    own.append(Cl(i, j - 1, k)); nei.append(Cl(i, j, k))
    fcs.append(np.stack([P(i, j, k), P(i, j, k + 1), P(i + 1, j, k + 1), P(i + 1, j, k)], 1))
    if nz > 1:
        k, j, i = np.meshgrid(np.arange(1, nz), np.arange(ny), np.arange(nx), indexing="ij")
        k, j, i = k.ravel(), j.ravel(), i.ravel()
        own.append(Cl(i, j, k - 1)); nei.append(Cl(i, j, k))
        fcs.append(np.stack([P(i, j, k), P(i + 1, j, k), P(i + 1, j + 1, k), P(i, j + 1, k)], 1))
    owner, neigh, faces = _sort_internal(np.concatenate(own), np.concatenate(nei), np.concatenate(fcs))

    def bfaces(which):
        if which == "x0":
            k, j = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij"); k, j = k.ravel(), j.ravel()
            return Cl(0, j, k), np.stack([P(0, j, k), P(0, j, k + 1), P(0, j + 1, k + 1), P(0, j + 1, k)], 1)
        if which == "x1":
            k, j = np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij"); k, j = k.ravel(), j.ravel()
            return Cl(nx - 1, j, k), np.stack([P(nx, j, k), P(nx, j + 1, k), P(nx, j + 1, k + 1), P(nx, j, k + 1)], 1)
        if which == "y0":
            k, i = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij"); k, i = k.ravel(), i.ravel()
            return Cl(i, 0, k), np.stack([P(i, 0, k), P(i + 1, 0, k), P(i + 1, 0, k + 1), P(i, 0, k + 1)], 1)
        if which == "y1":
            k, i = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij"); k, i = k.ravel(), i.ravel()
            return Cl(i, ny - 1, k), np.stack([P(i, ny, k), P(i, ny, k + 1), P(i + 1, ny, k + 1), P(i + 1, ny, k)], 1)
        if which == "z0":
            j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij"); j, i = j.ravel(), i.ravel()
            return Cl(i, j, 0), np.stack([P(i, j, 0), P(i, j + 1, 0), P(i + 1, j + 1, 0), P(i + 1, j, 0)], 1)
        if which == "z1":
            j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij"); j, i = j.ravel(), i.ravel()
            return Cl(i, j, nz - 1), np.stack([P(i, j, nz), P(i + 1, j, nz), P(i + 1, j + 1, nz), P(i, j + 1, nz)], 1)
        raise KeyError(which)

    def group(sides):
        cs, fs = zip(*(bfaces(s) for s in sides))
        c, f = np.concatenate(cs), np.concatenate(fs)
        o = np.argsort(c, kind="stable")
        return c[o], f[o]

    if patch_defs is None:
        patch_defs = [("movingWall", "wall", ["y1"], None)]
        if bottom_patch:
            patch_defs.append(("fixedWalls", "wall", ["x0", "x1"] + ([] if two_d else ["z0", "z1"]), None))
            patch_defs.append(("bottomWall", "wall", ["y0"], None))
        else:
            patch_defs.append(("fixedWalls", "wall", ["x0", "x1", "y0"] + ([] if two_d else ["z0", "z1"]), None))
    else:
        patch_defs = list(patch_defs)
    if two_d:
        patch_defs.append(("frontAndBack", "empty", ["z0", "z1"], None))
    b_own, b_faces, patches = [], [], []
    start = len(owner)
    for name, ptype, sides, bc in patch_defs:
        c, f = group(sides)
        b_own.append(c); b_faces.append(f)
        patches.append(dict(name=name, type=ptype, startFace=start, nFaces=len(c)))
        if bc is not None:
            patches[-1]["bc"] = bc
        start += len(c)
    all_faces = np.concatenate([faces] + b_faces).astype(np.int32)
    mesh = dict(
        points=points.astype(np.float64),
        face_offsets=np.arange(0, 4 * len(all_faces) + 1, 4, dtype=np.int32),
        face_verts=all_faces.ravel().astype(np.int32),
        owner=np.concatenate([owner] + b_own).astype(np.int32),
        neighbour=neigh.astype(np.int32),
        n_cells=nx * ny * nz,
        patches=patches,
    )
    return mesh


def _morton_order(xy: np.ndarray, bits: int = 16) -> np.ndarray:
    q = np.clip((xy - xy.min(0)) / np.maximum(np.ptp(xy, 0), 1e-300) * (2 ** bits - 1), 0, 2 ** bits - 1)
    q = q.astype(np.uint64)

    def spread(v):
        v = v & np.uint64(0xFFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
        return v

    key = spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1))
    return np.argsort(key, kind="stable")


def delaunay_mesh(n_interior: int = 49200, n_side: int = 400, seed: int = 0, dz=None,
                  bottom_patch=False):
    """Seeded Delaunay triangulation of the unit square, extruded to prisms.

    Interior points: ``default_rng(seed).uniform(size=(n_interior, 2))``;
    boundary: n_side nodes per side at t = k/n_side.  Cells are renumbered
    along a Morton curve of their centroids.
    """
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    inner = rng.uniform(0.0, 1.0, size=(n_interior, 2))
    t = np.arange(n_side) / n_side
    per = np.concatenate([
        np.stack([t, np.zeros_like(t)], 1),
        np.stack([np.ones_like(t), t], 1),
        np.stack([1.0 - t, np.ones_like(t)], 1),
        np.stack([np.zeros_like(t), 1.0 - t], 1),
    ])
    pts = np.concatenate([per, inner])
    tri = Delaunay(pts).simplices.astype(np.int64)
    a, b, c = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    flip = area2 < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    tri = tri[np.abs(area2) > 1e-14]
    cen = pts[tri].mean(1)
    tri = tri[_morton_order(cen)]
    nT = len(tri)
    n = len(pts)
    if dz is None:
        dz = 1.0 / n_side
    points = np.concatenate([np.c_[pts, np.zeros(n)], np.c_[pts, np.full(n, dz)]])
    # directed CCW edges per triangle
    ea = tri.ravel()
    eb = tri[:, [1, 2, 0]].ravel()
    et = np.repeat(np.arange(nT), 3)
    lo, hi = np.minimum(ea, eb), np.maximum(ea, eb)
    key = lo * n + hi
    order = np.argsort(key, kind="stable")
    key_s = key[order]
    first = np.ones(len(key_s), bool)
    first[1:] = key_s[1:] != key_s[:-1]
    grp = np.cumsum(first) - 1
    cnt = np.bincount(grp)
    idx_first = order[first]
    internal_g = np.nonzero(cnt == 2)[0]
    starts = np.nonzero(first)[0]
    i1 = order[starts[internal_g]]
    i2 = order[starts[internal_g] + 1]
    t1, t2 = et[i1], et[i2]
    own = np.minimum(t1, t2)
    nei = np.maximum(t1, t2)
    # edge as traversed CCW by the owner gives an outward (owner->neighbour) normal
    own_edge = np.where(t1 == own, i1, i2)
    qa, qb = ea[own_edge], eb[own_edge]
    ifaces = np.stack([qa, qb, qb + n, qa + n], 1)
    owner, neigh, faces = _sort_internal(own, nei, ifaces)
    bnd_g = np.nonzero(cnt == 1)[0]
    bi = order[starts[bnd_g]]
    bt, ba, bb = et[bi], ea[bi], eb[bi]
    mid = 0.5 * (pts[ba] + pts[bb])
    bfaces = np.stack([ba, bb, bb + n, ba + n], 1)
    top = np.abs(mid[:, 1] - 1.0) < 1e-12
    bottom = np.abs(mid[:, 1]) < 1e-12
    groups = [("movingWall", "wall", top)]
    if bottom_patch:
        groups.append(("fixedWalls", "wall", ~top & ~bottom))
        groups.append(("bottomWall", "wall", bottom))
    else:
        groups.append(("fixedWalls", "wall", ~top))
    patches, bo, bf = [], [], []
    start = len(owner)
    for name, ptype, m in groups:
        o = np.argsort(bt[m], kind="stable")
        bo.append(bt[m][o]); bf.append(bfaces[m][o])
        patches.append(dict(name=name, type=ptype, startFace=start, nFaces=int(m.sum())))
        start += int(m.sum())
    # front (z=0, normal -z) and back (z=dz, normal +z) triangles
    fb_own = np.concatenate([np.arange(nT), np.arange(nT)])
    fb = [tri[:, [0, 2, 1]], tri + n]
    patches.append(dict(name="frontAndBack", type="empty", startFace=start, nFaces=2 * nT))
    quads = np.concatenate([faces] + bf).astype(np.int32)
    tris = np.concatenate(fb).astype(np.int32)
    nq, nt3 = len(quads), len(tris)
    offsets = np.concatenate([np.arange(0, 4 * nq + 1, 4), 4 * nq + np.arange(3, 3 * nt3 + 1, 3)]).astype(np.int32)
    mesh = dict(
        points=points.astype(np.float64),
        face_offsets=offsets,
        face_verts=np.concatenate([quads.ravel(), tris.ravel()]).astype(np.int32),
        owner=np.concatenate([owner] + bo + [fb_own]).astype(np.int32),
        neighbour=neigh.astype(np.int32),
        n_cells=nT,
        patches=patches,
    )
    return mesh


def mesh_info(mesh):
    nF = len(mesh["face_offsets"]) - 1
    nI = len(mesh["neighbour"])
    return dict(n_cells=mesh["n_cells"], n_faces=nF, n_internal=nI,
                n_wall=sum(p["nFaces"] for p in mesh["patches"] if p["type"] == "wall"))


# ------------------------------------------------------------------ cases
def make_case(mesh, gas, rho0, nxi, xi_max, two_d=True, lid_u=50.0, T0=273.0, Tw=None,
              grid="nc", C_gh=None, lid_patch="movingWall", bvals=None):
    """Assemble a case dict: mesh + gas + DV grid + initial rest equilibrium.

    Wall velocity: ``lid_u`` in +x on ``lid_patch``, zero elsewhere.  Wall
    temperature: ``Tw`` (scalar, or dict patch-name -> scalar/array), else T0.
    ``bvals``: patch name -> dict(rho=, U=, T=, pressure=) patch values of the
    other boundary types (fixedValue, farField, pressureIn/Out).
    """
    nC = mesh["n_cells"]
    nF = len(mesh["face_offsets"]) - 1
    nI = len(mesh["neighbour"])
    nB = nF - nI
    Ub = np.zeros((nB, 3))
    Tb = np.full(nB, float(T0))
    rhob = np.zeros(nB)
    for p in mesh["patches"]:
        s, e = p["startFace"] - nI, p["startFace"] - nI + p["nFaces"]
        bv = (bvals or {}).get(p["name"])
        if bv is not None:
            rhob[s:e] = bv.get("rho", rho0)
            Ub[s:e] = bv.get("U", (0.0, 0.0, 0.0))
            Tb[s:e] = bv.get("T", T0)
            if "pressure" in bv:
                p["pressure"] = float(bv["pressure"])
            for f in ("T", "U"):  # zeroGradient T / U: the patch follows its owner cells
                if bv.get(f + "_bc"):
                    p[f + "_bc"] = bv[f + "_bc"]
            continue
        if p["type"] != "wall":
            Tb[s:e] = 0.0
            continue
        if p["name"] == lid_patch:
            Ub[s:e, 0] = lid_u
        if Tw is not None:
            val = Tw.get(p["name"], T0) if isinstance(Tw, dict) else Tw
            Tb[s:e] = val
    if grid == "nc":
        xis, w = newton_cotes(xi_max, nxi)
    else:
        xis, w = gauss_hermite_half_range(C_gh, nxi)
    return dict(
        mesh=mesh,
        gas=gas,
        xis=np.asarray(xis, np.float64),
        weights=np.asarray(w, np.float64),
        xi_max=float(xi_max),
        rho0=np.full(nC, rho0),
        U0=np.zeros((nC, 3)),
        T0=np.full(nC, float(T0)),
        Ub=Ub,
        Tb=Tb,
        rhob=rhob,
        two_d=two_d,
    )


def stable_dt(case, cfl=0.5):
    """dt with max Courant number ``cfl`` at rest (fvDVM::getCoNum with Usurf = 0)."""
    mesh = case["mesh"]
    from .geometry import cell_centres_volumes

    C, _ = cell_centres_volumes(mesh)
    d = C[mesh["neighbour"]] - C[mesh["owner"][: len(mesh["neighbour"])]]
    dc = 1.0 / np.sqrt((d * d).sum(1))
    D = 1 if case.get("one_d") else (2 if case["two_d"] else 3)
    return cfl / (dc.max() * math.sqrt(D) * case["xi_max"])


def cell_stable_dt(case, cfl=0.5):
    """dt with a cell-based Courant number: cfl * min_c(V_c / sum_f |S_f|) / (sqrt(D) xi_max).

    Used for unstructured meshes, where the centroid-distance Courant number of
    fvDVM::getCoNum under-estimates the stiffness of sliver cells (random
    Delaunay triangulations are unstable at the reference rule, even at 1/4).
    """
    from .geometry import cell_centres_volumes, face_centres_areas

    mesh = case["mesh"]
    _, V = cell_centres_volumes(mesh)
    _, Sf = face_centres_areas(mesh)
    nI = len(mesh["neighbour"])
    own = np.asarray(mesh["owner"])
    active = np.ones(len(own), bool)
    for p in mesh["patches"]:
        if p["type"] == "empty":
            active[p["startFace"]:p["startFace"] + p["nFaces"]] = False
    A = np.linalg.norm(Sf, axis=1)
    area = np.zeros(mesh["n_cells"])
    np.add.at(area, own[active], A[active])
    np.add.at(area, np.asarray(mesh["neighbour"]), A[:nI])
    D = 2 if case["two_d"] else 3
    return cfl * (V / area).min() / (math.sqrt(D) * case["xi_max"])


def case_dt(case, cfl=0.5):
    """The time step a workload runs at: cell-based for unstructured meshes."""
    return cell_stable_dt(case, cfl) if case.get("unstructured") else stable_dt(case, cfl)


def cavity2d(n=61, Kn=0.075, nxi=28, bottom_patch=False, lid_u=50.0, Tw=None):
    """2D lid-driven cavity on n x n quads (default: the 61^2, 28^2-DV case)."""
    gas, rho0 = gas_from_kn(Kn)
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 273.0)
    mesh = structured_mesh(n, n, 1, two_d=True, bottom_patch=bottom_patch)
    return make_case(mesh, gas, rho0, nxi, xi_max, two_d=True, lid_u=lid_u, Tw=Tw)


def delaunay2d(n_interior=49200, n_side=400, seed=0, Kn=0.01, nxi=32):
    """2D unstructured cavity on ~100k Delaunay triangles (prisms)."""
    gas, rho0 = gas_from_kn(Kn)
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 273.0)
    mesh = delaunay_mesh(n_interior, n_side, seed)
    case = make_case(mesh, gas, rho0, nxi, xi_max, two_d=True)
    case["unstructured"] = True
    return case


def cavity3d(n=48, Kn=0.1, nxi=20):
    """3D cubic lid-driven cavity on n^3 hexes."""
    gas, rho0 = gas_from_kn(Kn)
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 273.0)
    mesh = structured_mesh(n, n, n, lz=1.0, two_d=False)
    return make_case(mesh, gas, rho0, nxi, xi_max, two_d=False)


def channel2d(nx=40, ny=20, Kn=0.1, nxi=24, p_ratio=1.2, inlet_T_zero_gradient=False):
    """2D channel [0,2]x[0,1] in reduced units (R = 1/2, T0 = 1, rho0 = 1, so
    2 R T0 = 1): pressureIn (x = 0) at p_ratio p0, pressureOut (x = 2) at
    p0 = rho0 R T0, diffuse walls top and bottom (``inlet_T_zero_gradient``:
    the inlet's T is zeroGradient, so rho_b = p/(R T_b) follows the inlet
    cells' temperature).  Long runs need >= 24
    velocities per direction on [-4, 4]: on 16 the pressureOut feedback
    (rho_b, T_b from the owner cell's macros) drifts and the run blows up
    within a few hundred steps (in the oracle and the engine alike)."""
    gas, _ = gas_from_kn(Kn, R=0.5, T0=1.0)
    rho0 = 1.0
    gas["muRef"] = gas["muRef"] / _ * rho0  # mu = rho0 C L mu_bar with this rho0
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 1.0)
    p0 = rho0 * gas["R"] * 1.0
    mesh = structured_mesh(nx, ny, 1, lx=2.0, ly=1.0, lz=1.0 / ny, two_d=True, patch_defs=[
        ("inlet", "patch", ["x0"], "pressureIn"), ("outlet", "patch", ["x1"], "pressureOut"),
        ("walls", "wall", ["y0", "y1"], None)])
    return make_case(mesh, gas, rho0, nxi, xi_max, two_d=True, lid_u=0.0, T0=1.0, bvals={
        "inlet": dict(T=1.0, pressure=p_ratio * p0, T_bc="zeroGradient" if inlet_T_zero_gradient else None),
        "outlet": dict(T=1.0, pressure=p0)})


def open_box2d(n=24, Kn=0.1, nxi=28, u_in=60.0, zero_gradient_tu=False):
    """2D box with one patch of each open type: farField at x = 0 (rho0, 300 K),
    zeroGradient at x = 1, fixedValue (mixed) at y = 1 moving at u_in, a
    diffuse wall at y = 0.  ``zero_gradient_tu``: the farField and outflow
    patches have zeroGradient T and U (the farField's incoming Maxwellian then
    takes the temperature of its owner cells), and the initial temperature
    rises linearly from 273 K to 300 K across the box.  (Like the cavity, long
    runs on [-4, 4] sqrt(2 R T0) need ~28 velocities per direction; 16 blow up
    within ~1000 steps.)"""
    gas, rho0 = gas_from_kn(Kn)
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 273.0)
    mesh = structured_mesh(n, n, 1, two_d=True, patch_defs=[
        ("farfield", "patch", ["x0"], "farField"), ("outflow", "patch", ["x1"], "zeroGradient"),
        ("top", "patch", ["y1"], "fixedValue"), ("bottom", "wall", ["y0"], None)])
    zg = "zeroGradient" if zero_gradient_tu else None
    case = make_case(mesh, gas, rho0, nxi, xi_max, two_d=True, lid_u=0.0, bvals={
        "farfield": dict(rho=rho0, T=300.0, T_bc=zg, U_bc=zg), "top": dict(rho=1.1 * rho0, U=(u_in, 0.0, 0.0), T=290.0),
        "outflow": dict(T=273.0, T_bc=zg, U_bc=zg)})
    if zero_gradient_tu:
        from .geometry import cell_centres_volumes

        C, _ = cell_centres_volumes(mesh)
        case["T0"] = 300.0 - 27.0 * C[:, 0]
    return case


def half_cavity2d(nx=15, ny=30, Kn=0.075, nxi=28, sym="symmetryPlane"):
    """Left half [0,0.5]x[0,1] of the lid-driven cavity with a symmetry patch at
    x = 0.5 (the layout of the reference demo testSymmetry/symmetry):
    ``sym`` = "symmetryPlane" (constraint patch) or "symmetryMod" (DVMsymmetry)."""
    gas, rho0 = gas_from_kn(Kn)
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * 273.0)
    mtype = "symmetryPlane" if sym == "symmetryPlane" else "wall"
    mesh = structured_mesh(nx, ny, 1, lx=0.5, ly=1.0, lz=1.0 / ny, two_d=True, patch_defs=[
        ("movingWall", "wall", ["y1"], None), ("fixedWalls", "wall", ["x0", "y0"], None),
        ("symmetryWall", mtype, ["x1"], sym)])
    return make_case(mesh, gas, rho0, nxi, xi_max, two_d=True, bvals={"symmetryWall": dict(T=273.0)})


def tube1d(nx=100, Kn=0.05, nxi=32, rho_ratio=4.0):
    """1D closed shock tube [0,1] in reduced units (R = 1/2, T0 = 1): rho = 1
    on the left half and 1/rho_ratio on the right, at rest, diffuse walls at
    both ends; y and z faces are empty patches, so the case is 1D (M velocities)."""
    gas, _ = gas_from_kn(Kn, R=0.5, T0=1.0)
    gas["muRef"] = gas["muRef"] / _
    xi_max = 5.0 * math.sqrt(2 * gas["R"] * 1.0)
    mesh = structured_mesh(nx, 1, 1, lx=1.0, ly=1.0 / nx, lz=1.0 / nx, two_d=True, patch_defs=[
        ("left", "wall", ["x0"], None), ("right", "wall", ["x1"], None), ("sides", "empty", ["y0", "y1"], None)])
    case = make_case(mesh, gas, 1.0, nxi, xi_max, two_d=True, lid_u=0.0, T0=1.0, lid_patch="none")
    xc = (np.arange(nx) + 0.5) / nx
    case["rho0"] = np.where(xc < 0.5, 1.0, 1.0 / rho_ratio)
    case["one_d"] = True
    return case


def batch_case(inst):
    """Case dict of one batch instance: N x N lid-driven cavity, M x M DVs,
    its Kn, lid speed and wall temperature (all walls at Tw; initial T = Tw)."""
    gas, rho0 = gas_from_kn(inst["Kn"], T0=inst["Tw"])
    xi_max = 4.0 * math.sqrt(2 * gas["R"] * inst["Tw"])
    mesh = structured_mesh(inst["N"], inst["N"], 1, two_d=True)
    return make_case(mesh, gas, rho0, inst["M"], xi_max, two_d=True, lid_u=inst["lid_u"], T0=inst["Tw"],
                     Tw=inst["Tw"])


def batch_instances(count=64, steps=2000):
    """Seeded parameter list of independent 2D cavities (one rng per instance)."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(i)
        N = int(rng.integers(32, 129))
        M = int(rng.integers(16, 41))
        Kn = float(10 ** rng.uniform(math.log10(0.01), math.log10(1.0)))
        lid = float(rng.uniform(10.0, 100.0))
        Tw = float(rng.uniform(250.0, 350.0))
        out.append(dict(N=N, M=M, Kn=Kn, lid_u=lid, Tw=Tw, steps=steps))
    return out
