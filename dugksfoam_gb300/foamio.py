"""OpenFOAM ASCII case files for the engine.

``write_case`` writes a case dict (``cases.make_case``) as the directory
dugksFoam reads (doc/demo.tex; demo/cavity): ``constant/polyMesh/{points,
faces,owner,neighbour,boundary}``, ``0/{rho,U,T}`` with ``calculatedMaxwell``
density walls (``calculatedMaxwellFvPatchField``) and ``fixedValue`` U/T walls,
``constant/DVMProperties`` (``fvDVMparas``, ``gasProperties``),
``constant/Xis``, ``constant/weights`` and ``system/controlDict``.

``read_vol_field`` parses a vol field written by OpenFOAM or by
``dugks_write_time`` (uniform / nonuniform internal fields and patch values).
"""
from __future__ import annotations

import os
import re

import numpy as np

_HEADER = """FoamFile
{{
    version     2.0;
    format      ascii;
    class       {cls};
    location    "{loc}";
    object      {obj};
}}

"""


def _f(x):
    return repr(float(x))


def _write(path, cls, loc, obj, body):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        fh.write(_HEADER.format(cls=cls, loc=loc, obj=obj))
        fh.write(body)


def _scalar_list(v):
    return f"{len(v)}\n(\n" + "\n".join(_f(x) for x in v) + "\n)\n"


def _vector_list(v):
    return f"{len(v)}\n(\n" + "\n".join(f"({_f(a)} {_f(b)} {_f(c)})" for a, b, c in v) + "\n)\n"


def _field(path, cls, obj, dims, internal, patches, vector):
    """internal: array; patches: list of (name, type, values or None[, extra "key value" entry])."""
    kind = "vector" if vector else "scalar"
    lst = _vector_list(internal) if vector else _scalar_list(internal)
    body = f"dimensions      {dims};\n\ninternalField   nonuniform List<{kind}>\n{lst};\n\nboundaryField\n{{\n"
    for name, typ, val, *extra in patches:
        body += f"    {name}\n    {{\n        type            {typ};\n"
        for e in extra:
            key, v = e.split(" ", 1)
            body += f"        {key:<16}{v};\n"
        if val is not None:
            body += f"        value           nonuniform List<{kind}>\n"
            body += (_vector_list(val) if vector else _scalar_list(val)) + ";\n"
        body += "    }\n"
    body += "}\n"
    _write(path, cls, "0", obj, body)


def write_case(case, path, delta_t=None, end_time=None, df_cells=None):
    """Write ``case`` (a ``cases.make_case`` dict) as an OpenFOAM case directory
    (``df_cells``: DFwriteCellList of DVMProperties, written as a counted list)."""
    m = case["mesh"]
    pm = os.path.join(path, "constant", "polyMesh")
    pts = np.asarray(m["points"], np.float64)
    _write(os.path.join(pm, "points"), "vectorField", "constant/polyMesh", "points", _vector_list(pts))
    off = np.asarray(m["face_offsets"])
    fv = np.asarray(m["face_verts"])
    faces = [fv[off[i]:off[i + 1]] for i in range(len(off) - 1)]
    body = f"{len(faces)}\n(\n" + "\n".join(f"{len(f)}(" + " ".join(str(int(x)) for x in f) + ")" for f in faces)
    _write(os.path.join(pm, "faces"), "faceList", "constant/polyMesh", "faces", body + "\n)\n")
    own = np.asarray(m["owner"])
    nei = np.asarray(m["neighbour"])
    _write(os.path.join(pm, "owner"), "labelList", "constant/polyMesh", "owner",
           f"{len(own)}\n(\n" + "\n".join(str(int(x)) for x in own) + "\n)\n")
    _write(os.path.join(pm, "neighbour"), "labelList", "constant/polyMesh", "neighbour",
           f"{len(nei)}\n(\n" + "\n".join(str(int(x)) for x in nei) + "\n)\n")
    body = f"{len(m['patches'])}\n(\n"
    for p in m["patches"]:
        body += (f"    {p['name']}\n    {{\n        type            {p['type']};\n"
                 f"        nFaces          {int(p['nFaces'])};\n        startFace       {int(p['startFace'])};\n    }}\n")
    _write(os.path.join(pm, "boundary"), "polyBoundaryMesh", "constant/polyMesh", "boundary", body + ")\n")
    # 0/ fields
    nI = len(nei)
    Ub, Tb = np.asarray(case["Ub"]), np.asarray(case["Tb"])
    prho, pU, pT = [], [], []
    rhob = np.asarray(case.get("rhob", np.zeros(len(Tb))))
    for p in m["patches"]:
        s, e = p["startFace"] - nI, p["startFace"] - nI + p["nFaces"]
        bc = p.get("bc", {"wall": "calculatedMaxwell"}.get(p["type"], p["type"]))
        if bc == "calculatedMaxwell":
            prho.append((p["name"], "calculatedMaxwell", np.ones(p["nFaces"])))
            pU.append((p["name"], "fixedValue", Ub[s:e]))
            pT.append((p["name"], "fixedValue", Tb[s:e]))
        elif bc in ("empty", "symmetryPlane"):
            for lst in (prho, pU, pT):
                lst.append((p["name"], bc, None))
        else:  # zeroGradient, fixedValue, farField, pressureIn, pressureOut, symmetryMod
            extra = [f"{bc} {_f(p['pressure'])}"] if bc in ("pressureIn", "pressureOut") else []
            prho.append((p["name"], bc, rhob[s:e], *extra))
            pU.append((p["name"], "zeroGradient", None) if p.get("U_bc") == "zeroGradient"
                      else (p["name"], "fixedValue", Ub[s:e]))
            pT.append((p["name"], "zeroGradient", None) if p.get("T_bc") == "zeroGradient"
                      else (p["name"], "fixedValue", Tb[s:e]))
    z = os.path.join(path, "0")
    _field(os.path.join(z, "rho"), "volScalarField", "rho", "[1 -3 0 0 0 0 0]", case["rho0"], prho, False)
    _field(os.path.join(z, "U"), "volVectorField", "U", "[0 1 -1 0 0 0 0]", case["U0"], pU, True)
    _field(os.path.join(z, "T"), "volScalarField", "T", "[0 0 0 1 0 0 0]", case["T0"], pT, False)
    g = case["gas"]
    xm = float(case["xi_max"])
    body = (f"fvDVMparas\n{{\n    xiMax           xiMax [0 1 -1 0 0 0 0] {_f(xm)};\n"
            f"    xiMin           xiMin [0 1 -1 0 0 0 0] {_f(-xm)};\n    nDV             {len(case['xis'])};\n"
            f"    macroFlux       no;\n}}\n\ngasProperties\n{{\n    R               R [0 2 -2 -1 0 0 0] {_f(g['R'])};\n"
            f"    omega           {_f(g['omega'])};\n    Tref            Tref [0 0 0 1 0 0 0] {_f(g['Tref'])};\n"
            f"    muRef           muRef [1 -1 -1 0 0 0 0] {_f(g['muRef'])};\n    Pr              {_f(g['Pr'])};\n"
            f"    KInner          {int(g['KInner'])};\n}}\n")
    if df_cells is not None:
        body += f"\nDFwriteCellList {len(df_cells)}(" + " ".join(str(int(c)) for c in df_cells) + ");\n"
    _write(os.path.join(path, "constant", "DVMProperties"), "dictionary", "constant", "DVMProperties", body)
    _write(os.path.join(path, "constant", "Xis"), "scalarList", "constant", "Xis", _scalar_list(case["xis"]))
    _write(os.path.join(path, "constant", "weights"), "scalarList", "constant", "weights",
           _scalar_list(case["weights"]))
    dt = delta_t if delta_t is not None else 1e-6
    body = (f"application     dugksFoam;\nstartFrom       startTime;\nstartTime       0;\nstopAt          endTime;\n"
            f"endTime         {_f(end_time if end_time is not None else 1000 * dt)};\ndeltaT          {_f(dt)};\n"
            f"writeControl    timeStep;\nwriteInterval   100;\nadjustTimeStep  no;\n")
    _write(os.path.join(path, "system", "controlDict"), "dictionary", "system", "controlDict", body)


_NUM = r"[-+0-9.eEinfa]+"


def _strip_comments(t):
    t = re.sub(r"/\*.*?\*/", " ", t, flags=re.S)
    return re.sub(r"//[^\n]*", " ", t)


def _values(txt, ncomp):
    """Values of a field entry ('uniform x' / 'nonuniform List<..> n(...)')."""
    txt = txt.strip()
    if txt.startswith("uniform"):
        nums = [float(x) for x in re.findall(_NUM, txt[len("uniform"):])]
        return np.array(nums[:ncomp]), True
    body = txt[txt.index(">") + 1:]
    nums = [float(x) for x in re.findall(_NUM, body)]
    n = int(nums[0])
    return np.array(nums[1:1 + n * ncomp]).reshape(n, ncomp) if ncomp > 1 else np.array(nums[1:1 + n]), False


def read_vol_field(path):
    """Parse a vol field: returns (internal, {patch: (type, values or None)})."""
    t = _strip_comments(open(path).read())
    cls = re.search(r"class\s+(\w+)\s*;", t).group(1)
    ncomp = {"volScalarField": 1, "volVectorField": 3, "volTensorField": 9}[cls]
    i0 = t.index("internalField")
    i1, depth = i0, 0
    while not (t[i1] == ";" and depth == 0):  # end of the entry: ';' outside parentheses
        depth += (t[i1] == "(") - (t[i1] == ")")
        i1 += 1
    internal, _ = _values(t[i0 + len("internalField"):i1], ncomp)
    patches = {}
    bf = t[t.index("boundaryField"):]
    for mm in re.finditer(r"(\w+)\s*\{\s*type\s+(\w+)\s*;(.*?)\}", bf[bf.index("{") + 1:], flags=re.S):
        name, typ, rest = mm.group(1), mm.group(2), mm.group(3)
        val = None
        if "value" in rest:
            v = rest[rest.index("value") + len("value"):]
            v = v[: v.rindex(";")]
            val, _ = _values(v, ncomp)
        patches[name] = (typ, val)
    return internal, patches
