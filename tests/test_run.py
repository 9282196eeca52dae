"""The dugksFoam application loop (dugksfoam_gb300/run.py): controlDict
reading, the damped time-step rule of setDeltaTvar.H and the output clock, on
the CPU; the loop itself on a GPU."""
import json
import os

import pytest

from conftest import reference_path

REF_DEMO = reference_path("demo", "cavity")


def test_control_dict_and_defaults(tmp_path):
    from dugksfoam_gb300 import cases, foamio, run

    case = cases.cavity2d(n=5, nxi=6)
    foamio.write_case(case, tmp_path, delta_t=2.5e-6, end_time=1e-3)
    c = run.time_controls(run.read_control_dict(tmp_path))
    assert c["dt"] == 2.5e-6 and c["end"] == 1e-3 and c["write_control"] == "timeStep"
    assert c["write_interval"] == 100 and c["adjust"] is False
    # readTimeControlsExplicit.H defaults
    assert (c["max_co"], c["converge_tol"], c["check_steps"]) == (1.0, 1e-9, 1)


def test_set_delta_t_rule():
    from dugksfoam_gb300 import run

    # reduction is immediate, increase damped to 1 + 0.1 f and at most 1.2x
    assert run.new_delta_t(1.0, 2.0, 1.0, 1e15) == pytest.approx(0.5 / (1 + 1e-15 / 2.0))
    assert run.new_delta_t(1.0, 0.5, 1.0, 1e15) == pytest.approx(1.2)
    assert run.new_delta_t(1.0, 0.95, 1.0, 1e15) == pytest.approx(1.0 / 0.95, rel=1e-12)
    assert run.new_delta_t(1.0, 1.0 / 1.15, 1.0, 1e15) == pytest.approx(1.0 + 0.1 * 1.15, rel=1e-12)
    assert run.new_delta_t(1.0, 0.5, 1.0, 0.7) == 0.7


def test_output_clock():
    from dugksfoam_gb300 import run

    steps = run.OutputClock(dict(write_control="timeStep", write_interval=3.0, start=0.0))
    assert [s for s in range(1, 10) if steps(s, 0.0)] == [3, 6, 9]
    clock = run.OutputClock(dict(write_control="adjustableRunTime", write_interval=0.1, start=0.0))
    hits = [round(t, 3) for t in [0.04 * k for k in range(1, 13)] if clock(0, t)]
    assert hits == [0.12, 0.2, 0.32, 0.4]
    assert run.time_name(0.000125) == "0.000125" and run.time_name(2.0) == "2"


@pytest.mark.gpu
def test_loop_writes_time_directories(built_lib, tmp_path, capsys):
    from dugksfoam_gb300 import cases, foamio, run, solver

    case = cases.cavity2d(n=8, nxi=8)
    foamio.write_case(case, tmp_path, delta_t=cases.stable_dt(case), df_cells=[2])
    cd = (tmp_path / "system" / "controlDict").read_text().replace("writeInterval   100;", "writeInterval   3;")
    (tmp_path / "system" / "controlDict").write_text(cd + "convergeCheckSteps 2;\n")
    it, t = run.run(tmp_path, solver.FP64, max_steps=6)
    assert it == 6
    lines = [json.loads(x) for x in capsys.readouterr().out.splitlines()]
    assert [x["step"] for x in lines] == [2, 4, 6] and all(x["U_change"] > 0 for x in lines)
    written = sorted(p.name for p in tmp_path.iterdir() if p.name not in ("0", "constant", "system"))
    assert len(written) == 2 and (tmp_path / "0" / "DF2").exists()


@pytest.mark.skipif(not REF_DEMO or not os.path.isdir(REF_DEMO),
                    reason="reference demo case not present (set DUGKS_REFERENCE_ROOT)")
def test_reference_demo_control_dict():
    """The reference demo's controlDict: adjustable time step at maxCo 0.8,
    writes every 1000 steps, 9-digit time names."""
    from dugksfoam_gb300 import run

    c = run.time_controls(run.read_control_dict(REF_DEMO))
    assert c["adjust"] and c["max_co"] == 0.8 and c["max_dt"] == 1.0
    assert (c["dt"], c["end"], c["write_control"], c["write_interval"]) == (4e-4, 200.0, "timeStep", 1000.0)
    assert c["time_precision"] == 9


def test_adjustable_run_time_lands_on_write_times():
    """Time::adjustDeltaT under adjustableRunTime: the step is reshaped so that
    a whole number of steps reaches the next write time (2x up, 5x down)."""
    from dugksfoam_gb300 import run

    c = dict(write_control="adjustableRunTime", write_interval=0.1, start=0.0)
    assert run.adjust_to_write_time(0.03, 0.0, c, 0) == pytest.approx(0.1 / 4)
    assert run.adjust_to_write_time(0.03, 0.08, c, 0) == pytest.approx(0.02)
    assert run.adjust_to_write_time(0.001, 0.0995, c, 0) == pytest.approx(0.0005)
    assert run.adjust_to_write_time(0.5, 0.0, c, 0) == pytest.approx(0.1)  # shrink at most 5x
    c2 = dict(c, write_control="timeStep")
    assert run.adjust_to_write_time(0.03, 0.0, c2, 0) == 0.03
    # a loop that follows the adjusted step hits every write time exactly
    t, dt, clock, hits = 0.0, 0.03, run.OutputClock(c), []
    while t < 0.4 - 0.5 * dt:
        dt = run.adjust_to_write_time(dt, t, c, clock.index)
        t += dt
        if clock(0, t):
            hits.append(t)
    assert hits == pytest.approx([0.1, 0.2, 0.3, 0.4], abs=1e-12)


def test_run_condition_follows_time_run():
    """Time::run() is value() < endTime - 0.5 deltaT: a step that does not
    divide endTime takes no step past it."""
    t, dt, end, n = 0.0, 0.3, 1.0, 0
    while t < end - 0.5 * dt:
        t += dt
        n += 1
    assert n == 3
