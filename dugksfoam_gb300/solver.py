"""Python binding of the GB300 DUGKS engine (ctypes over include/dugks/dugks.h).

``FvDVM`` mirrors the reference solver class Foam::fvDVM
(src/fvDVM/fvDVM/fvDVM.H:78-377): ``evolution()``, ``getCoNum()``,
``rhoVol()``, ``Uvol()``, ``Tvol()``, ``qVol()``, ``tauVol()`` keep the
reference's names and meaning.  There is no CPU fallback: if libdugks.so is
missing or no CUDA device is present, construction raises ``DugksError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libdugks.so")

FP64 = 0
FP32_FP64MOM = 1
PIPE_AUTO, PIPE_REFERENCE, PIPE_FUSED = 0, 1, 2
PATCH_EMPTY, PATCH_MAXWELL = 0, 1
# dugks_patch_kind by rho boundary-condition type (include/dugks/dugks.h)
BC_KINDS = {"empty": 0, "calculatedMaxwell": 1, "zeroGradient": 2, "fixedValue": 3, "farField": 4,
            "pressureIn": 5, "pressureOut": 6, "symmetryMod": 7, "symmetryPlane": 8}

ERRORS = {0: "OK", 1: "DUGKS_ERR_ARG", 2: "DUGKS_ERR_IO", 3: "DUGKS_ERR_UNSUPPORTED", 4: "DUGKS_ERR_CUDA",
          5: "DUGKS_ERR_NUMERIC", 6: "DUGKS_ERR_TIMEOUT", 7: "DUGKS_ERR_OOM", 8: "DUGKS_ERR_BOUNDS"}

# Every entry point declared in include/dugks/dugks.h.
EXPORTS = [
    "dugks_create", "dugks_create_from_case_dir", "dugks_destroy", "dugks_last_error", "dugks_global_error",
    "dugks_get_info", "dugks_set_dt", "dugks_get_dt", "dugks_set_stream", "dugks_step", "dugks_synchronize",
    "dugks_get_conum", "dugks_get_macros", "dugks_get_face_macros", "dugks_get_wall", "dugks_get_boundary", "dugks_get_residual",
    "dugks_get_dist", "dugks_set_dist", "dugks_checkpoint_size", "dugks_checkpoint_save",
    "dugks_checkpoint_load", "dugks_profile_step", "dugks_launches_per_step", "dugks_macros_noalloc",
    "dugks_inspect_case_dir", "dugks_write_time", "dugks_write_df_on_cells",
    "dugks_objective_value", "dugks_objective_tangent", "dugks_objective_adjoint",
    "dugks_batch_create", "dugks_batch_destroy", "dugks_batch_last_error", "dugks_batch_set_dt", "dugks_batch_step",
    "dugks_batch_synchronize", "dugks_batch_get_macros", "dugks_batch_get_info", "dugks_batch_set_wait_limit",
    "dugks_checked_build",
]


class DugksError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class CaseDesc(C.Structure):
    _fields_ = [
        ("n_points", C.c_int32), ("points", _dp),
        ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_internal_faces", C.c_int32),
        ("face_offsets", _ip), ("face_verts", _ip), ("owner", _ip), ("neighbour", _ip),
        ("n_patches", C.c_int32), ("patch_start", _ip), ("patch_size", _ip), ("patch_kind", _ip),
        ("wall_U", _dp), ("wall_T", _dp), ("bnd_rho", _dp), ("patch_pressure", _dp),
        ("n_xi_per_dim", C.c_int32), ("xis", _dp), ("weights", _dp), ("xi_max", C.c_double),
        ("R", C.c_double), ("omega", C.c_double), ("Tref", C.c_double), ("muRef", C.c_double),
        ("Pr", C.c_double), ("KInner", C.c_int32),
        ("rho0", _dp), ("U0", _dp), ("T0", _dp),
        ("precision", C.c_int32), ("pipeline", C.c_int32), ("device", C.c_int32),
        ("patch_T_zero_gradient", _ip), ("patch_U_zero_gradient", _ip),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_internal_faces", C.c_int32),
        ("n_wall_faces", C.c_int32), ("n_dv", C.c_int32), ("n_dv_padded", C.c_int32),
        ("n_solution_d", C.c_int32), ("has_h", C.c_int32), ("precision", C.c_int32), ("pipeline", C.c_int32),
        ("dt", C.c_double), ("step_count", C.c_int64), ("device_bytes", C.c_size_t),
        ("n_xi_per_dim", C.c_int32), ("KInner", C.c_int32), ("xi_max", C.c_double), ("R", C.c_double),
        ("omega", C.c_double), ("Tref", C.c_double), ("muRef", C.c_double), ("Pr", C.c_double),
    ]


class CaseSummary(C.Structure):
    _fields_ = [
        ("n_points", C.c_int32), ("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_internal_faces", C.c_int32),
        ("n_patches", C.c_int32), ("n_wall_faces", C.c_int32), ("n_empty_faces", C.c_int32),
        ("n_xi_per_dim", C.c_int32), ("KInner", C.c_int32),
        ("xi_max", C.c_double), ("R", C.c_double), ("omega", C.c_double), ("Tref", C.c_double),
        ("muRef", C.c_double), ("Pr", C.c_double), ("delta_t", C.c_double),
        ("rho_sum", C.c_double), ("T_sum", C.c_double), ("n_df_cells", C.c_int32),
    ]


class ObjectiveDesc(C.Structure):
    _fields_ = [("n_steps", C.c_int32), ("avg_first", C.c_int32), ("q_patch", C.c_int32),
                ("stress_patch", C.c_int32), ("checkpoint_every", C.c_int32)]


class BatchInfo(C.Structure):
    _fields_ = [("n_cases", C.c_int32), ("dv_per_lane", C.c_int32), ("tile_cap", C.c_int32), ("groups", C.c_int32),
                ("launches_per_step", C.c_int32), ("steps_per_graph", C.c_int32), ("n_tuned", C.c_int32),
                ("cells", C.c_int64), ("cell_dv", C.c_int64),
                ("tuned_dv_per_lane", C.c_int32 * 8), ("tuned_tile_cap", C.c_int32 * 8), ("tuned_groups", C.c_int32 * 8),
                ("tuned_ms_per_step", C.c_double * 8)]


_libs = {}


def load_library(path: str | None = None):
    """Load libdugks.so, or the library at ``path`` (the index-checked build
    libdugks_checked.so), once per path (raises if it has not been built)."""
    path = path or LIB_PATH
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise DugksError(4, f"{path} not built; run dugksfoam_gb300.build.build()")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.dugks_create.argtypes = [C.POINTER(CaseDesc), C.POINTER(vp)]
    lib.dugks_create_from_case_dir.argtypes = [C.c_char_p, C.c_int32, C.POINTER(vp)]
    lib.dugks_destroy.argtypes = [vp]
    lib.dugks_last_error.argtypes = [vp]
    lib.dugks_last_error.restype = C.c_char_p
    lib.dugks_global_error.restype = C.c_char_p
    lib.dugks_get_info.argtypes = [vp, C.POINTER(Info)]
    lib.dugks_set_dt.argtypes = [vp, C.c_double]
    lib.dugks_get_dt.argtypes = [vp, _dp]
    lib.dugks_set_stream.argtypes = [vp, vp]
    lib.dugks_step.argtypes = [vp, C.c_int32]
    lib.dugks_synchronize.argtypes = [vp]
    lib.dugks_get_conum.argtypes = [vp, _dp, _dp]
    lib.dugks_get_macros.argtypes = [vp] + [_dp] * 5
    lib.dugks_get_face_macros.argtypes = [vp] + [_dp] * 5
    lib.dugks_get_wall.argtypes = [vp, C.c_int32, _dp, _dp, _dp]
    lib.dugks_get_boundary.argtypes = [vp, C.c_int32, _dp, _dp, _dp]
    lib.dugks_get_residual.argtypes = [vp, _dp]
    lib.dugks_get_dist.argtypes = [vp, _dp, _dp]
    lib.dugks_set_dist.argtypes = [vp, _dp, _dp]
    lib.dugks_checkpoint_size.argtypes = [vp, C.POINTER(C.c_size_t)]
    lib.dugks_checkpoint_save.argtypes = [vp, C.c_void_p, C.c_size_t]
    lib.dugks_checkpoint_load.argtypes = [vp, C.c_void_p, C.c_size_t]
    lib.dugks_profile_step.argtypes = [vp, C.c_int32, C.c_char_p, C.c_size_t, _dp, C.c_int32, _ip]
    lib.dugks_launches_per_step.argtypes = [vp, _ip]
    lib.dugks_macros_noalloc.argtypes = [vp] + [vp] * 6
    lib.dugks_inspect_case_dir.argtypes = [C.c_char_p, C.POINTER(CaseSummary)]
    lib.dugks_write_time.argtypes = [vp, C.c_char_p, C.c_char_p]
    lib.dugks_write_df_on_cells.argtypes = [vp, C.c_char_p, _ip, C.c_int32]
    op = C.POINTER(ObjectiveDesc)
    lib.dugks_objective_value.argtypes = [vp, op, _dp]
    lib.dugks_objective_tangent.argtypes = [vp, op, _dp, C.c_double, _dp, _dp]
    lib.dugks_objective_adjoint.argtypes = [vp, op, _dp, _dp, _dp]
    lib.dugks_batch_create.argtypes = [C.POINTER(CaseDesc), C.c_int32, C.c_int32, C.POINTER(vp)]
    lib.dugks_batch_destroy.argtypes = [vp]
    lib.dugks_batch_last_error.argtypes = [vp]
    lib.dugks_batch_last_error.restype = C.c_char_p
    lib.dugks_batch_set_dt.argtypes = [vp, C.c_int32, C.c_double]
    lib.dugks_batch_step.argtypes = [vp, C.c_int32]
    lib.dugks_batch_synchronize.argtypes = [vp]
    lib.dugks_batch_get_macros.argtypes = [vp, C.c_int32] + [_dp] * 4
    lib.dugks_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    lib.dugks_batch_set_wait_limit.argtypes = [vp, C.c_int64]
    _libs[path] = lib
    return lib


def inspect_case_dir(path):
    """Sizes and parameters of an OpenFOAM case directory (host only, no GPU)."""
    lib = load_library()
    out = CaseSummary()
    rc = lib.dugks_inspect_case_dir(str(path).encode(), C.byref(out))
    if rc != 0:
        raise DugksError(rc, lib.dugks_global_error().decode())
    return {k: getattr(out, k) for k, _ in CaseSummary._fields_}


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip)


def patch_bc(p):
    """rho boundary-condition type of a case patch: its "bc" entry, else from the mesh patch type."""
    if "bc" in p:
        return p["bc"]
    return {"empty": "empty", "wall": "calculatedMaxwell", "symmetryPlane": "symmetryPlane"}[p["type"]]


def _kinds(mesh):
    return np.array([BC_KINDS[patch_bc(p)] for p in mesh["patches"]], np.int32)


def case_desc(case, precision=FP64, pipeline=PIPE_AUTO, device=0):
    """dugks_case_desc of a case dict; returns (desc, arrays the desc points into)."""
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
        pk=_kinds(m),
        Ub=np.ascontiguousarray(case["Ub"], np.float64),
        Tb=np.ascontiguousarray(case["Tb"], np.float64),
        rhob=np.ascontiguousarray(case.get("rhob", np.zeros(len(case["Tb"]))), np.float64),
        pp=np.ascontiguousarray([p.get("pressure", 0.0) for p in m["patches"]], np.float64),
        tzg=np.array([1 if p.get("T_bc") == "zeroGradient" else 0 for p in m["patches"]], np.int32),
        uzg=np.array([1 if p.get("U_bc") == "zeroGradient" else 0 for p in m["patches"]], np.int32),
        xis=np.ascontiguousarray(case["xis"], np.float64),
        w=np.ascontiguousarray(case["weights"], np.float64),
        rho0=np.ascontiguousarray(case["rho0"], np.float64),
        U0=np.ascontiguousarray(case["U0"], np.float64),
        T0=np.ascontiguousarray(case["T0"], np.float64),
    )
    d = CaseDesc(
        n_points=len(keep["points"]), points=_d(keep["points"]), n_cells=int(m["n_cells"]),
        n_faces=len(keep["off"]) - 1, n_internal_faces=len(keep["nei"]), face_offsets=_i(keep["off"]),
        face_verts=_i(keep["fv"]), owner=_i(keep["own"]), neighbour=_i(keep["nei"]),
        n_patches=len(keep["ps"]), patch_start=_i(keep["ps"]), patch_size=_i(keep["pn"]),
        patch_kind=_i(keep["pk"]), wall_U=_d(keep["Ub"]), wall_T=_d(keep["Tb"]),
        bnd_rho=_d(keep["rhob"]), patch_pressure=_d(keep["pp"]),
        n_xi_per_dim=len(keep["xis"]), xis=_d(keep["xis"]), weights=_d(keep["w"]),
        xi_max=float(case["xi_max"]), R=g["R"], omega=g["omega"], Tref=g["Tref"], muRef=g["muRef"],
        Pr=g["Pr"], KInner=int(g["KInner"]), rho0=_d(keep["rho0"]), U0=_d(keep["U0"]), T0=_d(keep["T0"]),
        precision=int(precision), pipeline=int(pipeline), device=int(device),
        patch_T_zero_gradient=_i(keep["tzg"]), patch_U_zero_gradient=_i(keep["uzg"]),
    )
    return d, keep


class FvDVM:
    """One DUGKS case resident on one GPU (the reference's fvDVM)."""

    def __init__(self, case=None, precision=FP64, pipeline=PIPE_AUTO, device=0, _handle=None, lib_path=None):
        self._lib = load_library(lib_path)
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            d, self._keep = case_desc(case, precision, pipeline, device)
            rc = self._lib.dugks_create(C.byref(d), C.byref(self._h))
            if rc != 0:
                raise DugksError(rc, self._lib.dugks_global_error().decode())
        info = self.info()
        self.nCells = info["n_cells"]
        self.nDV = info["n_dv"]
        self.nFaceMacros = info["n_internal_faces"] + info["n_wall_faces"]

    @classmethod
    def from_case_dir(cls, path, precision=FP64):
        lib = load_library()
        h = C.c_void_p()
        rc = lib.dugks_create_from_case_dir(str(path).encode(), int(precision), C.byref(h))
        if rc != 0:
            raise DugksError(rc, lib.dugks_global_error().decode())
        return cls(_handle=h)

    # ------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.dugks_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise DugksError(rc, self._lib.dugks_last_error(self._h).decode())

    # ------------------------------------------------------------- controls
    def info(self):
        i = Info()
        self._check(self._lib.dugks_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in Info._fields_}

    def set_dt(self, dt):
        self._check(self._lib.dugks_set_dt(self._h, float(dt)))

    @property
    def dt(self):
        v = C.c_double()
        self._check(self._lib.dugks_get_dt(self._h, C.byref(v)))
        return v.value

    def set_stream(self, stream_ptr):
        self._check(self._lib.dugks_set_stream(self._h, C.c_void_p(stream_ptr)))

    def evolution(self, nsteps=1):
        """fvDVM::evolution() ``nsteps`` times (asynchronous)."""
        self._check(self._lib.dugks_step(self._h, int(nsteps)))

    def synchronize(self):
        self._check(self._lib.dugks_synchronize(self._h))

    def getCoNum(self):
        a, b = C.c_double(), C.c_double()
        self._check(self._lib.dugks_get_conum(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    # ------------------------------------------------------------ accessors
    def macros(self):
        n = self.nCells
        out = dict(rho=np.empty(n), U=np.empty((n, 3)), T=np.empty(n), q=np.empty((n, 3)), tau=np.empty(n))
        self._check(self._lib.dugks_get_macros(self._h, *(_d(out[k]) for k in ("rho", "U", "T", "q", "tau"))))
        return out

    def macros_into(self, rho, U, T, q):
        """Copy cell macros into caller-owned (e.g. pinned) float64 buffers."""
        self._check(self._lib.dugks_get_macros(self._h, _d(rho), _d(U), _d(T), _d(q), None))

    def rhoVol(self):
        return self.macros()["rho"]

    def Uvol(self):
        return self.macros()["U"]

    def Tvol(self):
        return self.macros()["T"]

    def qVol(self):
        return self.macros()["q"]

    def tauVol(self):
        return self.macros()["tau"]

    # fvDVMI.H:67-155: face fields (internal faces, then non-empty boundary faces)
    # and parameters
    def rhoSurf(self):
        return self.face_macros()["rho"]

    def Usurf(self):
        return self.face_macros()["U"]

    def Tsurf(self):
        return self.face_macros()["T"]

    def qSurf(self):
        return self.face_macros()["q"]

    def tauSurf(self):
        return self.face_macros()["tau"]

    def nXi(self):
        return self.info()["n_dv"]

    def nXiPerDim(self):
        return self.info()["n_xi_per_dim"]

    def xiMax(self):
        return self.info()["xi_max"]

    def R(self):
        return self.info()["R"]

    def omega(self):
        return self.info()["omega"]

    def Tref(self):
        return self.info()["Tref"]

    def muRef(self):
        return self.info()["muRef"]

    def Pr(self):
        return self.info()["Pr"]

    def KInner(self):
        return self.info()["KInner"]

    def face_macros(self):
        n = self.nFaceMacros
        out = dict(rho=np.empty(n), U=np.empty((n, 3)), T=np.empty(n), q=np.empty((n, 3)), tau=np.empty(n))
        self._check(self._lib.dugks_get_face_macros(self._h, *(_d(out[k]) for k in ("rho", "U", "T", "q", "tau"))))
        return out

    def wall(self, patch, n_faces):
        out = dict(rhoW=np.empty(n_faces), qWall=np.empty((n_faces, 3)), stressWall=np.empty((n_faces, 9)))
        self._check(self._lib.dugks_get_wall(self._h, int(patch), _d(out["rhoW"]), _d(out["qWall"]),
                                             _d(out["stressWall"])))
        return out

    def boundary(self, patch, n_faces):
        """rho, U, T patch values of one non-empty patch (rho_w on walls)."""
        out = dict(rho=np.empty(n_faces), U=np.empty((n_faces, 3)), T=np.empty(n_faces))
        self._check(self._lib.dugks_get_boundary(self._h, int(patch), _d(out["rho"]), _d(out["U"]), _d(out["T"])))
        return out

    def residual(self):
        r = np.empty(3)
        self._check(self._lib.dugks_get_residual(self._h, _d(r)))
        return dict(U=r[0], T=r[1], rho=r[2])

    def dist(self):
        g = np.empty((self.nCells, self.nDV))
        h = np.empty((self.nCells, self.nDV))
        self._check(self._lib.dugks_get_dist(self._h, _d(g), _d(h)))
        return g, h

    def set_dist(self, g, h=None):
        g = np.ascontiguousarray(g, np.float64)
        h = None if h is None else np.ascontiguousarray(h, np.float64)
        self._check(self._lib.dugks_set_dist(self._h, _d(g), _d(h)))

    def writeDFonCells(self, case_dir, cells=None):
        """fvDVM::writeDFonCells: case_dir/0/DF<id> with g~ of each cell (cells=None:
        the case directory's DFwriteCellList)."""
        if cells is None:
            rc = self._lib.dugks_write_df_on_cells(self._h, str(case_dir).encode(), None, 0)
        else:
            ids = np.ascontiguousarray(cells, np.int32)
            rc = self._lib.dugks_write_df_on_cells(self._h, str(case_dir).encode(), _i(ids), len(ids))
        self._check(rc)

    def write(self, case_dir, time_name):
        """runTime.write(): rho, U, T, q, qSurf, stressSurf into case_dir/time_name (dugksFoam.C:81)."""
        self._check(self._lib.dugks_write_time(self._h, str(case_dir).encode(), str(time_name).encode()))

    # ------------------------------------------------------------ gradient harness
    @staticmethod
    def _obj(n_steps, avg_first, q_patch, stress_patch, checkpoint_every):
        return ObjectiveDesc(int(n_steps), int(avg_first), int(q_patch), int(stress_patch), int(checkpoint_every))

    def objective_value(self, n_steps, avg_first, q_patch=-1, stress_patch=-1, checkpoint_every=100):
        """FP64 wall objective over steps [avg_first, n_steps) from the initial state."""
        o = self._obj(n_steps, avg_first, q_patch, stress_patch, checkpoint_every)
        J = C.c_double()
        self._check(self._lib.dugks_objective_value(self._h, C.byref(o), C.byref(J)))
        return J.value

    def objective_tangent(self, dTw, ds, n_steps, avg_first, q_patch=-1, stress_patch=-1, checkpoint_every=100):
        """(J, dJ) along (dTw per wall face, ds): FP64 tangent-linear step."""
        o = self._obj(n_steps, avg_first, q_patch, stress_patch, checkpoint_every)
        d = np.ascontiguousarray(dTw, np.float64)
        J, dJ = C.c_double(), C.c_double()
        self._check(self._lib.dugks_objective_tangent(self._h, C.byref(o), _d(d), float(ds), C.byref(J), C.byref(dJ)))
        return J.value, dJ.value

    def objective_adjoint(self, n_steps, avg_first, q_patch=-1, stress_patch=-1, checkpoint_every=100):
        """(J, dJ/dTw per wall face, dJ/ds): hand-written adjoint of the FP64 step."""
        o = self._obj(n_steps, avg_first, q_patch, stress_patch, checkpoint_every)
        info = self.info()
        g = np.zeros(max(info["n_wall_faces"], 1))
        J, gs = C.c_double(), C.c_double()
        self._check(self._lib.dugks_objective_adjoint(self._h, C.byref(o), C.byref(J), _d(g), C.byref(gs)))
        return J.value, g[: info["n_wall_faces"]], gs.value

    def checkpoint(self) -> bytes:
        n = C.c_size_t()
        self._check(self._lib.dugks_checkpoint_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._check(self._lib.dugks_checkpoint_save(self._h, buf, n.value))
        return buf.raw

    def restore(self, data: bytes):
        buf = C.create_string_buffer(data, len(data))
        self._check(self._lib.dugks_checkpoint_load(self._h, buf, len(data)))

    def profile(self, nsteps=3):
        names = C.create_string_buffer(4096)
        ms = np.zeros(64)
        nk = C.c_int32()
        self._check(self._lib.dugks_profile_step(self._h, int(nsteps), names, 4096, _d(ms), 64, C.byref(nk)))
        nm = names.value.decode().strip().split("\n")
        return dict(zip(nm, ms[: nk.value].tolist()))

    def launches_per_step(self):
        n = C.c_int32()
        self._check(self._lib.dugks_launches_per_step(self._h, C.byref(n)))
        return n.value


class Batch:
    """Independent 2D cases advanced together (dugks_batch_*): one launch per
    pass over all cases, two steps per CUDA graph, autotuned DVs per lane and
    tile cap; or (``persistent=True``) every pass of every step in one
    cooperative launch.  Every case uses the FP32 / FP64-moment pipeline."""

    def __init__(self, case_list, autotune=True, device=0, persistent=False):
        self._lib = load_library()
        self._h = C.c_void_p()
        descs, self._keep = [], []
        for c in case_list:
            d, k = case_desc(c, FP32_FP64MOM, PIPE_FUSED, device)
            descs.append(d)
            self._keep.append(k)
        arr = (CaseDesc * len(descs))(*descs)
        mode = 2 if persistent else int(bool(autotune))
        rc = self._lib.dugks_batch_create(arr, len(descs), mode, C.byref(self._h))
        if rc != 0:
            raise DugksError(rc, self._lib.dugks_global_error().decode())
        self.cells = [int(c["mesh"]["n_cells"]) for c in case_list]

    def _check(self, rc):
        if rc != 0:
            raise DugksError(rc, self._lib.dugks_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.dugks_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_dt(self, i, dt):
        self._check(self._lib.dugks_batch_set_dt(self._h, int(i), float(dt)))

    def step(self, n):
        self._check(self._lib.dugks_batch_step(self._h, int(n)))

    def set_wait_limit(self, polls):
        """Polls a grid-barrier wait of the persistent kernel makes before giving up."""
        self._check(self._lib.dugks_batch_set_wait_limit(self._h, int(polls)))

    def synchronize(self):
        self._check(self._lib.dugks_batch_synchronize(self._h))

    def macros(self, i):
        n = self.cells[i]
        out = dict(rho=np.empty(n), U=np.empty((n, 3)), T=np.empty(n), q=np.empty((n, 3)))
        self._check(self._lib.dugks_batch_get_macros(self._h, int(i), _d(out["rho"]), _d(out["U"]), _d(out["T"]),
                                                     _d(out["q"])))
        return out

    def info(self):
        b = BatchInfo()
        self._check(self._lib.dugks_batch_get_info(self._h, C.byref(b)))
        r = {k: getattr(b, k) for k, _ in BatchInfo._fields_}
        n = b.n_tuned
        r["tuned"] = [dict(dv_per_lane=b.tuned_dv_per_lane[k], tile_cap=b.tuned_tile_cap[k], groups=b.tuned_groups[k],
                           ms_per_step=b.tuned_ms_per_step[k]) for k in range(n)]
        for k in ("tuned_dv_per_lane", "tuned_tile_cap", "tuned_groups", "tuned_ms_per_step"):
            r.pop(k)
        return r
