"""Decks run end to end on the GPU (nlmech_gb300/run.py): an explicit deck
with a CSV mesh, timed crack, no-fail region, angled force region, initial
velocity and output criteria against the same deck run on the oracle's model;
a quasi-static 1-D deck (the reference's qsModel/1D setup, written from its
stored mesh) against the reference's stored result."""
import json
import os

import numpy as np
import pytest

from nlmech_gb300 import abi, deckfile, output, run, vtu
from oracle import oracle as orc
from test_deckfile import _write_deck

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_fd_deck_matches_oracle(gpu, tmp_path):
    _write_deck(tmp_path)
    deck = deckfile.read_deck(str(tmp_path / "input.yaml"))
    deck.output.tags = ["Displacement", "Velocity", "Damage_Z", "Strain_Energy"]
    deck.output.path = str(tmp_path / "gpu") + "/"
    model, steps, files = run.run_fd(deck, abi.FP64, graph=8)
    deck_o = deckfile.read_deck(str(tmp_path / "input.yaml"))
    deck_o.output.tags = deck.output.tags
    deck_o.output.path = str(tmp_path / "cpu") + "/"
    so, fo = output.integrate(orc.OracleFD(deck_o.problem), deck_o.output, deck_o.time_steps)
    assert steps == so and [os.path.basename(f) for f in files] == [os.path.basename(f) for f in fo]
    assert len(files) > 4
    for a, b in zip(files, fo):
        da, db = vtu.read_vtu(a), vtu.read_vtu(b)
        assert da["TIME"][0] == db["TIME"][0]
        scale = max(np.abs(db["Displacement"]).max(), 1e-300)
        assert np.abs(da["Displacement"] - db["Displacement"]).max() <= 1e-12 * scale
        assert np.abs(da["Damage_Z"] - db["Damage_Z"]).max() <= 1e-5


QS_DECK = """
Model:
  Dimension: 1
  Discretization_Type:
    Spatial: finite_difference
    Time: quasi_static
  Final_Time: {final_time}
  Time_Steps: {time_steps}
  Horizon: {horizon}
  Horizon_h_Ratio: {h_ratio}
Mesh:
  File: mesh.csv
Material:
  Type: ElasticState
  Density: {density}
  Compute_From_Classical: true
  E: {E}
Displacement_BC:
  Sets: {n_ubc}
{ubc}
Force_BC:
  Sets: {n_fbc}
{fbc}
Solver:
  Type: CG
  Max_Iteration: {max_iters}
  Tolerance: {tol}
  Perturbation: {perturbation}
Output:
  Path: ./out/
  Tags:
    - Displacement
    - Force
  Output_Interval: 1
"""


def _bc_text(bcs):
    out = []
    for k, b in enumerate(bcs, 1):
        out.append("  Set_%d:\n    Location:\n      Line: [%r, %r]\n    Direction: [%s]\n"
                   "    Time_Function:\n      Type: %s\n      Parameters: [%s]\n"
                   "    Spatial_Function:\n      Type: %s\n      Parameters: [%s]"
                   % (k, b["x1"], b["x2"], ", ".join(str(d) for d in b["dir"]), b["time_fn"],
                      ", ".join(repr(v) for v in b["time_params"]), b["spatial_fn"],
                      ", ".join(repr(v) for v in b["spatial_params"])))
    return "\n".join(out)


def test_qs_1d_deck_matches_reference_result(gpu, tmp_path):
    z = np.load(os.path.join(GOLD, "qs_1d.npz"))
    deck = json.loads(str(z["deck"]))
    with open(tmp_path / "mesh.csv", "w") as fh:
        fh.write("id,x,volume\n")
        for i, (p, v) in enumerate(zip(z["x"], z["volume"])):
            fh.write("%d,%.17g,%.17g\n" % (i, p[0], v))
    (tmp_path / "input.yaml").write_text(QS_DECK.format(
        ubc=_bc_text(deck["ubc"]), fbc=_bc_text(deck["fbc"]), n_ubc=len(deck["ubc"]),
        n_fbc=len(deck["fbc"]), **{k: deck[k] for k in (
            "final_time", "time_steps", "horizon", "h_ratio", "density", "E", "max_iters",
            "tol", "perturbation")}))
    d = deckfile.read_deck(str(tmp_path / "input.yaml"))
    q, iters, files = run.run_qs(d)
    assert len(files) == deck["time_steps"] + 1
    last = vtu.read_vtu(files[-1])
    err = np.sqrt((np.linalg.norm(last["Displacement"] - z["displacement"], axis=1) ** 2).sum())
    assert err < deck["compare_tol"], err
