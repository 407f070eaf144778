"""The oracle's RNPBond restatement against the reference's own sources.

oracle/refshim compiles NLMech's neighbor.cpp, fracture.cpp,
interiorFlags.cpp, rnpBond.cpp, uLoading.cpp and fLoading.cpp unmodified and
drives them through FDModel's velocity-Verlet loop.  Neighbour lists,
pre-crack bits, fixity, broken bonds and u, v, f must agree bit for bit.
The direct runs need the reference source tree (skipped where it is
absent); the oracle is also checked against the committed outputs of those
runs (tests/golden/rnp_ref_*.npz, written by tests/golden/make_rnp_golden.py).
"""
import numpy as np
import pytest

from nlmech_gb300 import configs
from oracle import oracle as orc

from refcases import (GOLDEN_CASES, contact_plate, cube3d, fracture_plate, gaussian_params_plate,
                      gaussian_plate, loads_nofail_plate, reaction_plate, timed_crack_plate)

needs_ref = pytest.mark.skipif(not orc.refshim_available(),
                               reason="reference source tree not present")


def _same_run(p, steps, chunks=2):
    r = orc.RefRNP(p)
    o = orc.OracleFD(p)
    ra, ca = r.neighbors()
    oa, oc = o.neighbors()
    assert np.array_equal(ra, oa) and np.array_equal(ca, oc)
    assert np.array_equal(r.bond_state(), o.bond_state())
    assert np.array_equal(r.fixity(), o.fixity())
    done = 0
    for k in range(chunks):
        n = steps // chunks if k < chunks - 1 else steps - done
        r.run(n)
        o.run(n)
        done += n
        for a, b in zip(r.state(), o.state()):
            assert np.array_equal(a, b), np.abs(a - b).max()
        assert np.array_equal(r.bond_state(), o.bond_state())
        assert r.time() == o.time()
    return r, o


@needs_ref
def test_refshim_config0_bit_exact():
    _same_run(configs.config0(), 300)


@needs_ref
def test_refshim_fracture_bit_exact():
    r, o = _same_run(fracture_plate(), 300, chunks=3)
    assert int(r.bond_state().sum()) > int(orc.RefRNP(fracture_plate()).bond_state().sum()) + 100


@needs_ref
def test_refshim_loads_nofail_influence_bit_exact():
    _same_run(loads_nofail_plate(), 200)


@needs_ref
def test_refshim_gaussian_influence_bit_exact():
    """GaussianInfluenceFn with the default parameters and with parameters
    from the deck (influenceFn.h:278-402)."""
    r, _ = _same_run(gaussian_plate(), 300, chunks=3)
    assert int(r.bond_state().sum()) > int(orc.RefRNP(gaussian_plate()).bond_state().sum()) + 50
    _same_run(gaussian_params_plate(), 200)


@needs_ref
def test_refshim_3d_bit_exact():
    _same_run(cube3d(), 100)


@needs_ref
def test_refshim_contact_bit_exact():
    _same_run(contact_plate(), 300, chunks=3)


@needs_ref
def test_refshim_timed_cracks_bit_exact():
    """Fracture::addCrack after every step's output: the crack at t = 0 is
    cut before step 2, the two at 3e-7 s before steps 17 and 18 (one per
    step)."""
    p = timed_crack_plate()
    r = orc.RefRNP(p)
    o = orc.OracleFD(p)
    counts = [int(r.bond_state().sum())]
    for n in (1, 14, 1, 1, 1, 182):
        r.run(n)
        o.run(n)
        assert np.array_equal(r.bond_state(), o.bond_state())
        for a, b in zip(r.state(), o.state()):
            assert np.array_equal(a, b)
        counts.append(int(r.bond_state().sum()))
    d = np.diff(counts)  # after steps 1, 15, 16, 17, 18, 200
    assert d[0] < 50 and d[1] > 200 and d[2] < 50 and d[3] > 200 and d[4] > 200, counts


@needs_ref
@pytest.mark.parametrize("make,steps", [(loads_nofail_plate, 200), (fracture_plate, 300),
                                        (cube3d, 50)])
def test_refshim_energies_bit_exact(make, steps):
    """computePostProcFields energies from the reference's getBondEF and
    FLoading against the oracle's restatement."""
    r = orc.RefRNP(make())
    o = orc.OracleFD(make())
    r.run(steps)
    o.run(steps)
    eo, tot = o.energies()
    assert np.array_equal(r.energies(), eo)
    assert np.allclose(tot, eo.astype(np.float64).sum(axis=1), rtol=1e-12, atol=0)


@needs_ref
def test_refshim_reaction_force_bit_exact():
    """Reaction_Force of FDModel::computeForce from the reference's getBondEF
    and doLinesIntersect against the oracle: non-zero on the 1 m plate, zero
    on the 1 mm plate (the truncated orientation test)."""
    for make, steps, nonzero in ((reaction_plate, 200, True), (fracture_plate, 300, False)):
        r = orc.RefRNP(make())
        o = orc.OracleFD(make())
        r.run(steps)
        o.run(steps)
        R, tot, s = o.reaction_force()
        assert np.array_equal(r.reaction_force(), R)
        assert np.array_equal(tot, np.sqrt((R * R).sum(axis=1)))
        assert (np.abs(R).sum() > 0) == nonzero


@needs_ref
def test_refshim_critical_stretch():
    p = configs.config0()
    r = orc.RefRNP(p)
    prm = orc.rnp_params(p.material, 2, p.horizon)
    for rr in (1e-3, 2.5e-3, 4e-3):
        assert r.sc(rr) == prm["rbar"] / np.sqrt(rr)


# ---- committed outputs of the reference sources (no reference tree needed) --
import os  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_oracle_matches_reference_golden(name):
    make, steps = GOLDEN_CASES[name]
    z = np.load(os.path.join(GOLDEN, "rnp_ref_%s.npz" % name))
    o = orc.OracleFD(make())
    rowptr, cols = o.neighbors()
    assert np.array_equal(rowptr, z["rowptr"]) and np.array_equal(cols, z["cols"])
    assert np.array_equal(o.bond_state(), z["precrack"])
    assert np.array_equal(o.fixity(), z["fixity"])
    o.run(steps)
    u, v, f = o.state()
    for a, k in ((u, "u"), (v, "v"), (f, "f")):
        assert np.array_equal(a, z[k]), k
    assert np.array_equal(o.bond_state(), z["broken"])
    assert o.time() == (float(z["time"]), int(z["steps"]))
    assert np.array_equal(o.energies()[0], z["energies"])
    if "reaction" in z.files:
        assert np.array_equal(o.reaction_force()[0], z["reaction"])
