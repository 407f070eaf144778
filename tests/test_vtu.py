"""VTU files in the reference's encoding: written here, read back by this
module and by the independent decoder that reads the reference's own
stored results (tests/golden/make_golden.py)."""
import os
import sys

import numpy as np
import pytest

from nlmech_gb300 import vtu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402


def test_vtu_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    n = 50000  # several compression blocks per array
    x = rng.uniform(size=(n, 3))
    u, v, f = (rng.normal(size=(n, 3)) for _ in range(3))
    vol = rng.uniform(1, 2, size=n)
    phi = rng.uniform(size=n).astype(np.float32)
    fix = rng.integers(0, 8, size=n).astype(np.uint8)
    p = tmp_path / "out.vtu"
    vtu.write_vtu(p, x, u=u, v=v, f=f, volume=vol, phi=phi, Z=phi * 2, fixity=fix, time=1.5e-6)
    for reader in (vtu.read_vtu, make_golden.read_vtu if hasattr(make_golden, "read_vtu") else None):
        if reader is None:
            continue
        d = reader(str(p))
        assert np.array_equal(d["Points"], x + u)
        assert np.array_equal(d["Displacement"], u)
        assert np.array_equal(d["Velocity"], v)
        assert np.array_equal(d["Force_Density"], f)
        assert np.array_equal(d["Force"], f * vol[:, None])
        assert np.array_equal(d["Node_Volume"], vol)
        assert np.array_equal(d["Damage_Phi"], phi)
        assert np.array_equal(d["Damage_Z"], phi * 2)
        assert np.array_equal(d["Fixity"], fix)
        assert d["TIME"][0] == 1.5e-6


def test_vtu_reads_reference_results():
    path = os.path.join(make_golden.REF, "examples/qsModel/2D/output_res.vtu")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    a = vtu.read_vtu(path)
    b = make_golden.read_vtu(path)
    assert set(a) == set(b)
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert a["Displacement"].shape == (289, 3)
