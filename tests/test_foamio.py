"""OpenFOAM case I/O: the Python case writer against the engine's C++ reader
(host-only entry point dugks_inspect_case_dir), the reader against the
reference's own demo case (src-tree fixture demo/cavity, read in place when
the reference tree is present), and the vol-field parser."""
import os
import re

import numpy as np
import pytest

from conftest import reference_path

REF_DEMO = reference_path("demo", "cavity")


def _case():
    from dugksfoam_gb300 import cases

    return cases.cavity2d(n=7, nxi=8)


def test_written_case_reads_back(built_lib, tmp_path):
    from dugksfoam_gb300 import foamio, solver

    case = _case()
    foamio.write_case(case, tmp_path, delta_t=3.25e-6)
    s = solver.inspect_case_dir(tmp_path)
    m = case["mesh"]
    nI = len(m["neighbour"])
    assert s["n_cells"] == m["n_cells"]
    assert s["n_faces"] == len(m["face_offsets"]) - 1
    assert s["n_internal_faces"] == nI
    assert s["n_points"] == len(m["points"])
    assert s["n_patches"] == len(m["patches"])
    assert s["n_wall_faces"] == sum(p["nFaces"] for p in m["patches"] if p["type"] == "wall")
    assert s["n_empty_faces"] == sum(p["nFaces"] for p in m["patches"] if p["type"] == "empty")
    assert s["n_xi_per_dim"] == len(case["xis"])
    g = case["gas"]
    for k in ("R", "omega", "Tref", "muRef", "Pr"):
        assert s[k] == g[k], k  # 17-digit round trip is exact
    assert s["xi_max"] == case["xi_max"]
    assert s["delta_t"] == 3.25e-6
    assert s["rho_sum"] == pytest.approx(float(np.sum(case["rho0"])), rel=1e-15)
    assert s["T_sum"] == pytest.approx(float(np.sum(case["T0"])), rel=1e-15)


def test_vol_field_parser_round_trip(tmp_path):
    from dugksfoam_gb300 import foamio

    case = _case()
    foamio.write_case(case, tmp_path)
    rho, prho = foamio.read_vol_field(tmp_path / "0" / "rho")
    U, pU = foamio.read_vol_field(tmp_path / "0" / "U")
    assert np.array_equal(rho, case["rho0"]) and np.array_equal(U, case["U0"])
    nI = len(case["mesh"]["neighbour"])
    for p in case["mesh"]["patches"]:
        if p["type"] == "wall":
            s, e = p["startFace"] - nI, p["startFace"] - nI + p["nFaces"]
            assert prho[p["name"]][0] == "calculatedMaxwell"
            assert pU[p["name"]][0] == "fixedValue" and np.array_equal(pU[p["name"]][1], case["Ub"][s:e])
        else:
            assert pU[p["name"]] == ("empty", None)


def test_missing_field_and_unsupported_bc_are_errors(built_lib, tmp_path):
    from dugksfoam_gb300 import foamio, solver

    foamio.write_case(_case(), tmp_path)
    os.remove(tmp_path / "0" / "T")
    with pytest.raises(solver.DugksError) as e:
        solver.inspect_case_dir(tmp_path)
    assert e.value.code == 2  # DUGKS_ERR_IO
    foamio.write_case(_case(), tmp_path)
    t = (tmp_path / "0" / "rho").read_text().replace("calculatedMaxwell", "totalPressure", 1)
    (tmp_path / "0" / "rho").write_text(t)
    with pytest.raises(solver.DugksError) as e:
        solver.inspect_case_dir(tmp_path)
    assert e.value.code == 3  # DUGKS_ERR_UNSUPPORTED


@pytest.mark.skipif(not REF_DEMO or not os.path.isdir(REF_DEMO),
                    reason="reference demo case not present (set DUGKS_REFERENCE_ROOT)")
def test_reference_demo_case(built_lib):
    """demo/cavity: 3600 cells, 14520 faces, 7080 internal (owner file note),
    the 28-point velocity grid; gas constants as in its DVMProperties.  Its
    empty patch is listed as frontAndBack in polyMesh/boundary and not in the
    fields (which name frontAndBackPlanes): read as empty, as OpenFOAM does."""
    from dugksfoam_gb300 import solver

    s = solver.inspect_case_dir(REF_DEMO)
    note = open(os.path.join(REF_DEMO, "constant/polyMesh/owner")).read()
    n = {k: int(v) for k, v in re.findall(r"n(Points|Cells|Faces|InternalFaces):\s*(\d+)", note)}
    assert (s["n_points"], s["n_cells"], s["n_faces"], s["n_internal_faces"]) == (
        n["Points"], n["Cells"], n["Faces"], n["InternalFaces"]) == (7442, 3600, 14520, 7080)
    assert s["n_xi_per_dim"] == 28 and s["n_wall_faces"] == 240 and s["n_empty_faces"] == 7200
    dvm = open(os.path.join(REF_DEMO, "constant/DVMProperties")).read()
    for k in ("R", "omega", "Tref", "muRef", "Pr"):
        v = float(re.search(rf"\n\s*{k}\s[^;]*?([-+0-9.eE]+)\s*;", dvm).group(1))
        assert s[k] == v, k


def test_df_write_cell_list_is_read(built_lib, tmp_path):
    """DFwriteCellList of DVMProperties (fvDVM.C:1067), counted or plain list;
    a cell out of range is an error."""
    from dugksfoam_gb300 import foamio, solver

    case = _case()
    foamio.write_case(case, tmp_path, df_cells=[0, 5, 17])
    assert solver.inspect_case_dir(tmp_path)["n_df_cells"] == 3
    dvm = tmp_path / "constant" / "DVMProperties"
    dvm.write_text(dvm.read_text().replace("DFwriteCellList 3(0 5 17);", "DFwriteCellList (4 9);"))
    assert solver.inspect_case_dir(tmp_path)["n_df_cells"] == 2
    dvm.write_text(dvm.read_text().replace("DFwriteCellList (4 9);", "DFwriteCellList (4 100000);"))
    with pytest.raises(solver.DugksError) as e:
        solver.inspect_case_dir(tmp_path)
    assert e.value.code == 2  # DUGKS_ERR_IO
