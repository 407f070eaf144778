"""Post-processing energies (nlm_fd_energies) and reaction force
(nlm_fd_reaction_force) against the oracle's
restatement of FDModel::computePostProcFields (fDModel.cpp:651-778).

FP64 plain mode follows the reference's operation order, so per-node fields
agree to float rounding (1e-6 of the field's scale: the FP64 sums differ in
the last bits of exp() before the float conversion).  FP32-compensated mode
is compared through the totals (1e-3 relative), like its displacement bar.
The property test needs no oracle: with velocity Verlet and no bond
breaking, strain + kinetic energy is conserved to 1% over 100 steps.
"""
import numpy as np
import pytest

import refcases
from nlmech_gb300 import abi, configs

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _rel_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _compare(m, o, what):
    e, t = m.energies()
    eo, to = o.energies()
    for q, name in enumerate(("strain", "work", "kinetic", "fracture")):
        if np.abs(eo[q]).max() == 0:
            assert np.abs(e[q]).max() == 0, what + " " + name
            continue
        assert _rel_max(e[q], eo[q]) <= RTOL, what + " " + name
        assert abs(t[q] - to[q]) <= 1e-5 * np.abs(eo[q]).sum(), what + " total " + name


def test_energies_fp64_loads_parity(gpu, oracle):
    """Force BCs in time and space (work done), no-fail layer, crack growth."""
    p = refcases.loads_nofail_plate()
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    for n in (1, 49, 150):
        m.run(n)
        o.run(n)
        _compare(m, o, "step %d" % n)
    e, _ = o.energies()
    assert (e[1] != 0).any() and (e[3] != 0).any()


def test_energies_fp64_fracture_and_3d(gpu, oracle):
    for p, n in ((refcases.fracture_plate(), 300), (refcases.cube3d(10), 60)):
        m = gpu.FDModel(p, precision=abi.FP64)
        o = oracle.OracleFD(p)
        m.run(n)
        o.run(n)
        _compare(m, o, "dim %d" % p.dim)


def test_energies_fp32c_totals(gpu, oracle):
    p = refcases.fracture_plate()
    m = gpu.FDModel(p, precision=abi.FP32C)
    o = oracle.OracleFD(p)
    m.run(300)
    o.run(300)
    e, t = m.energies()
    eo, to = o.energies()
    assert int(o.bond_state().sum()) > 0
    for q in (0, 2):
        assert abs(t[q] - to[q]) <= 1e-3 * abs(to[q]), q
        assert np.linalg.norm(e[q] - eo[q]) <= 1e-3 * np.linalg.norm(eo[q]), q


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32C])
def test_energy_conservation(gpu, precision):
    p = refcases.cube3d(10)
    p.v0 = p.v0 * 0.02  # no bond reaches its critical strain
    m = gpu.FDModel(p, precision=precision)
    _, t0 = m.energies()
    tot0 = t0[0] + t0[2]
    for _ in range(5):
        m.run(20)
        _, t = m.energies()
        assert abs(t[0] + t[2] - tot0) <= 1e-2 * tot0, (t, t0)
    assert m.count_broken() == 0


def test_energies_unsupported_for_elastic_state(gpu):
    m = gpu.FDModel(configs.elastic_state_cube(8, 1e-3), precision=abi.FP64)
    with pytest.raises(gpu.NLMError):
        m.energies()


def test_reaction_force_fp32c_and_limits(gpu):
    """Reaction_Force in FP32C against the reference's golden output (1e-3
    relative L2: the FP32C state's own bar is 1e-5 on u, and the bond forces
    difference it), and the 3-D model refuses the 2-D layer definition."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "rnp_ref_reaction_plate.npz"))
    m = gpu.FDModel(refcases.reaction_plate(), precision=abi.FP32C)
    m.run(int(z["steps"]))
    R, tot, s = m.reaction_force()
    assert np.linalg.norm(R - z["reaction"]) <= 1e-3 * np.linalg.norm(z["reaction"])
    assert np.array_equal(np.abs(R).sum(axis=1) > 0, np.abs(z["reaction"]).sum(axis=1) > 0)
    m3 = gpu.FDModel(refcases.cube3d(8), precision=abi.FP64)
    with pytest.raises(gpu.NLMError):
        m3.reaction_force()
