"""The output loop on the GPU model (FP64, CUDA-graph replay on) against the
same loop on the oracle's model: same output steps, same stop step, same
criteria log, and fields within the FP64 bars (Damage_Z to float rounding,
u within 1e-12 of its scale)."""
import os

import numpy as np
import pytest

import refcases
from nlmech_gb300 import abi, output, vtu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("timed", [False, True])
def test_gpu_output_loop_matches_oracle(gpu, oracle, tmp_path, timed):
    make = refcases.timed_crack_plate if timed else refcases.fracture_plate
    tags = ["Displacement", "Damage_Z", "Strain_Energy", "Total_Energy", "Reaction_Force",
            "Total_Reaction_Force"]
    deck = output.OutputDeck(tags=tags, dt_out=16 if timed else 40, criteria="max_Z_stop",
                             dt_out_criteria=8,
                             criteria_params=[0.5, 1.0, 0.0, 0.0, 0.048, 0.048])
    runs = []
    for kind in ("gpu", "oracle"):
        deck.path = str(tmp_path / kind) + "/"
        if kind == "gpu":
            m = gpu.FDModel(make(), precision=abi.FP64)
            m.set_graph(8)
        else:
            m = oracle.OracleFD(make())
        steps, files = output.integrate(m, deck, 300)
        info = open(os.path.join(deck.path, "dt_out_change.info")).read()
        runs.append((steps, [os.path.basename(f) for f in files],
                     [vtu.read_vtu(f) for f in files], info))
    (s1, n1, d1, i1), (s2, n2, d2, i2) = runs
    assert s1 == s2 and n1 == n2 and i1 == i2 and s1 < 300
    for a, b in zip(d1, d2):
        assert a["TIME"][0] == b["TIME"][0]
        assert np.abs(a["Damage_Z"] - b["Damage_Z"]).max() <= 1e-5 * max(1., b["Damage_Z"].max())
        u, uo = a["Displacement"], b["Displacement"]
        assert np.abs(u - uo).max() <= 1e-12 * max(np.abs(uo).max(), 1e-300)
        assert np.abs(a["Strain_Energy"] - b["Strain_Energy"]).max() <= \
            1e-6 * np.abs(b["Strain_Energy"]).max()
