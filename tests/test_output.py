"""The output loop (nlmech_gb300/output.py): FDModel::integrate's output
schedule, model::Output's files and checkOutputCriteria.

The loop is host logic over any model with the FDModel methods; these CPU
tests drive it with the oracle's model and compare the chunked loop with a
step-by-step transcription of the reference's loop (fDModel.cpp:335-374).
"""
import os

import numpy as np
import pytest

import refcases
from nlmech_gb300 import output, vtu
from oracle import oracle as orc


def _naive_integrate(model, deck, nsteps):
    """fDModel.cpp:352-373 one step at a time, with the crack check after
    every step as the reference does it."""
    crit = output.OutputCriteria(deck)
    os.makedirs(deck.path, exist_ok=True)
    pending = [c for c in model.problem.cracks if c.activation_time >= 0]
    files, Z = [], np.zeros(model.n, dtype=np.float32)
    n0 = model.time()[1]
    if n0 == 0:  # output at the beginning (fDModel.cpp:335-339)
        model.run(0)
        post = output.post_process(model, deck)
        Z = post["damage"][1]
        files.append(output.write_output(model, deck, 0, crit.dt_out_criteria, post))
    for _ in range(nsteps):
        model.run(1)
        t, n = model.time()
        if n % crit.dt_out == 0 and n >= crit.dt_out:
            post = output.post_process(model, deck)
            Z = post["damage"][1]
            files.append(output.write_output(model, deck, n, crit.dt_out_criteria, post))
            if crit.stop:
                return n - n0, files
            crit.check(n, Z, model.problem.x)
        for c in pending:
            if output._dlt(c.activation_time, t):
                pending.remove(c)
                crit.check(n, Z, model.problem.x)
                break
    return nsteps, files


def test_output_schedule_and_files(tmp_path):
    p = refcases.loads_nofail_plate()
    m = orc.OracleFD(p)
    tags = ["Displacement", "Velocity", "Force", "Force_Density", "Damage_Phi", "Damage_Z",
            "Strain_Energy", "Work_Done", "Fixity", "Node_Volume", "Total_Energy",
            "Fracture_Perienergy_Total", "Neighbors"]
    deck = output.OutputDeck(path=str(tmp_path) + "/", tags=tags, dt_out=50)
    steps, files = output.integrate(m, deck, 120)
    assert steps == 120 and [os.path.basename(f) for f in files] == [
        "output_0.vtu", "output_1.vtu", "output_2.vtu"]
    d = vtu.read_vtu(files[-1])
    o = orc.OracleFD(p)
    o.run(100)
    u, v, f = o.state()
    phi, Z = o.damage()
    e, tot = o.energies()
    assert d["TIME"][0] == o.time()[0]
    assert np.array_equal(d["Displacement"], u) and np.array_equal(d["Velocity"], v)
    assert np.array_equal(d["Force"], f * p.volume[:, None])
    assert np.array_equal(d["Damage_Z"], Z) and np.array_equal(d["Damage_Phi"], phi)
    assert np.array_equal(d["Strain_Energy"], e[0]) and np.array_equal(d["Work_Done"], e[1])
    assert np.array_equal(d["Fixity"], o.fixity())
    assert d["Total_Energy"][0] == tot[0] - tot[1] + tot[2]
    rowptr, _ = o.neighbors()
    assert np.array_equal(d["Neighbors"], np.diff(rowptr))
    assert np.array_equal(d["Points"], p.x + u)
    assert m.time()[1] == 120


def test_criteria_transitions(tmp_path):
    deck = output.OutputDeck(dt_out=100, criteria="max_Z_stop", dt_out_criteria=10,
                             criteria_params=[0.9, 1.0, 0.0, 0.0, 1.0, 1.0], path=str(tmp_path))
    x = np.array([[0.5, 0.5, 0.], [2.0, 2.0, 0.]])
    c = output.OutputCriteria(deck)
    c.check(50, np.array([0.95, 0.], np.float32), x)    # not a multiple of 100
    assert c.dt_out == 100
    c.check(100, np.array([0.5, 0.], np.float32), x)    # below the switch level
    assert c.dt_out == 100
    c.check(200, np.array([1.2, 0.], np.float32), x)    # switch; no stop in the same call
    assert c.dt_out == 10 and not c.stop
    c.check(300, np.array([0.5, 5.0], np.float32), x)   # high Z outside the rectangle
    assert not c.stop
    c.check(400, np.array([1.5, 0.], np.float32), x)    # inside: back to 100 and stop
    assert c.dt_out == 100 and c.stop
    txt = open(os.path.join(str(tmp_path), "dt_out_change.info")).read()
    assert txt == ("Large_Dt_To_Small_Dt:\n  N: 200\n  dN: 20\n"
                   "Small_Dt_To_Large_Dt:\n  N: 400\n  dN: 40\n")
    # max_Z switches once and never stops
    deck = output.OutputDeck(dt_out=100, criteria="max_Z", dt_out_criteria=10,
                             criteria_params=[0.9], path=str(tmp_path))
    c = output.OutputCriteria(deck)
    c.check(100, np.array([1.0], np.float32), x[:1])
    c.check(200, np.array([9.0], np.float32), x[:1])
    assert c.dt_out == 10 and not c.stop


@pytest.mark.parametrize("timed", [False, True])
def test_chunked_loop_equals_step_by_step(tmp_path, timed):
    """max_Z_stop on a growing crack (and timed cracks whose cut triggers a
    check): the chunked loop writes the same files and stops at the same
    step as the step-by-step loop."""
    # timed: a crack is cut at the end of step 16, a multiple of the interval,
    # so the check that its cut triggers runs right after the output's one
    make = refcases.timed_crack_plate if timed else refcases.fracture_plate
    deck = output.OutputDeck(tags=["Damage_Z"], dt_out=16 if timed else 40,
                             criteria="max_Z_stop", dt_out_criteria=8,
                             criteria_params=[0.5, 1.0, 0.0, 0.0, 0.048, 0.048])
    runs = []
    for kind in ("chunked", "naive"):
        deck.path = str(tmp_path / kind) + "/"
        m = orc.OracleFD(make())
        fn = output.integrate if kind == "chunked" else _naive_integrate
        steps, files = fn(m, deck, 300)
        names = [os.path.basename(f) for f in files]
        zs = [vtu.read_vtu(f)["Damage_Z"] for f in files]
        info = open(os.path.join(deck.path, "dt_out_change.info")).read()
        runs.append((steps, names, zs, info))
    (s1, n1, z1, i1), (s2, n2, z2, i2) = runs
    assert s1 == s2 and n1 == n2 and i1 == i2
    assert all(np.array_equal(a, b) for a, b in zip(z1, z2))
    assert "Large_Dt_To_Small_Dt" in i1 and s1 < 300  # switched and stopped
