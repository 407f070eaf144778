"""The CPU oracle against the reference's own stored results and invariants.

Golden data: examples/qsModel/{1D,2D}/output_res.vtu of NLMech, decoded into
tests/golden/qs_{1d,2d}.npz by tests/golden/make_golden.py.  The reference
test compares Displacement and Force with the `dc` tool at L2 < 1e-7
(examples/qsModel/*/input_compare.yaml, tools/dc/src/fdSimple.cpp:164-176).
"""
import json
import os

import numpy as np
import pytest

from nlmech_gb300 import configs
from nlmech_gb300.decks import BC, MaterialDeck, Problem

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_problem(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    deck = json.loads(str(z["deck"]))

    def bcs(lst):
        return [BC(region=b["region"], x1=b["x1"], x2=b["x2"], direction=b["dir"],
                   time_fn=b["time_fn"], time_params=b["time_params"],
                   spatial_fn=b["spatial_fn"], spatial_params=b["spatial_params"]) for b in lst]

    mat = MaterialDeck(kind="ElasticState", density=deck["density"], E=deck.get("E", -1.0),
                       K=deck.get("K", -1.0), G=deck.get("G", -1.0),
                       plane_strain=deck.get("plane_strain", False))
    p = Problem(dim=deck["dim"], x=z["x"], volume=z["volume"], horizon=deck["horizon"],
                mesh_size=deck["horizon"] / deck["h_ratio"], material=mat,
                ubc=bcs(deck["ubc"]), fbc=bcs(deck["fbc"]))
    return p, z, deck


def _l2(a, b):
    # tools/dc/src/fdSimple.cpp:164-176: sqrt(sum_i |a_i - b_i|^2)
    return float(np.sqrt((np.linalg.norm(a - b, axis=1) ** 2).sum()))


@pytest.mark.parametrize("name", ["qs_1d", "qs_2d"])
@pytest.mark.parametrize("jac", [0, 1])
def test_qs_golden(oracle, name, jac):
    p, z, deck = _golden_problem(name)
    prm = oracle.QSParams(jacobian=jac, solver=0, max_iters=deck["max_iters"], tol=deck["tol"],
                          tol_relative=0, perturbation=deck["perturbation"], lin_max_iters=1000,
                          lin_tol=1e-12, dt=deck["final_time"] / deck["time_steps"])
    q = oracle.OracleQS(p, prm)
    iters, res = q.solve(deck["time_steps"])
    assert res < deck["tol"]
    u, f = q.get()
    tol = deck["compare_tol"]
    assert _l2(u, z["displacement"]) < tol
    assert _l2(f, z["force"]) < 1e-6 * max(1.0, np.abs(z["force"]).max())
    if name == "qs_2d" and jac == 1:
        # full-block Jacobian: Newton converges quadratically
        assert iters[0] <= 5


@pytest.mark.parametrize("name", ["qs_1d", "qs_2d"])
def test_golden_neighbor_counts(oracle, name):
    p, z, deck = _golden_problem(name)
    rp, cols = oracle.neighbors(p.x, p.horizon, dim=p.dim, grid=False)
    assert np.array_equal(np.diff(rp), z["neighbors"].astype(np.int64))


def test_neighbors_brute_equals_grid(oracle):
    x, _ = configs.grid2d(40, 30, 1e-3, jitter=0.05, seed=3)
    for ratio in (3, 4):
        a = oracle.neighbors(x, ratio * 1e-3, dim=2, grid=False)
        b = oracle.neighbors(x, ratio * 1e-3, dim=2, grid=True)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    x3, _ = configs.grid3d(9, 8, 7, 1e-3, seed=4)
    a = oracle.neighbors(x3, 3e-3, dim=3, grid=False)
    b = oracle.neighbors(x3, 3e-3, dim=3, grid=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_neighbor_predicate_excludes_horizon(oracle):
    # compare.cpp:30-33: a node at exactly the horizon is not a neighbour,
    # neither is one within the 1e-5 relative band below it.
    d = 1.0
    x = np.array([[0, 0, 0], [d, 0, 0], [0, d * (1 - 2e-6), 0], [0, -d * (1 - 2e-5), 0.]])
    rp, cols = oracle.neighbors(x, d, dim=2, grid=False)
    assert list(cols[rp[0]:rp[1]]) == [3]
    assert oracle.lib().orc_definitely_less_than(ctypes_double(1.0), ctypes_double(1.0 + 2e-5))
    assert not oracle.lib().orc_definitely_less_than(ctypes_double(1.0), ctypes_double(1.0 + 5e-6))


def ctypes_double(v):
    import ctypes
    return ctypes.c_double(v)


def test_rnp_parameters(oracle):
    # config-0 material, J = 1, 2-D plane stress (rnpBond.cpp:99-189)
    m = configs.glass_rnp()
    r = oracle.rnp_params(m, 2, 4e-3)
    assert r["nu"] == pytest.approx(1 / 3)
    assert r["M"] == pytest.approx(1 / 3)
    assert r["lambda"] == pytest.approx(72e9 / 3 / ((4 / 3) * (1 / 3)))
    assert r["C"] == pytest.approx(np.pi * 3.8 / (4 / 3))
    assert r["beta"] == pytest.approx(4 * r["lambda"] / (r["C"] / 3))
    assert r["rbar"] == pytest.approx(np.sqrt(0.5 / r["beta"]))
    assert r["invF"] == pytest.approx(np.pi * (4e-3) ** 3)


def test_precrack_is_symmetric_and_local(oracle):
    p = configs.rnp_plate(40, 1e-3, 4, 0.01, 0.1, 2e-8, 10, seed=1)
    o = oracle.OracleFD(p)
    rp, cols = o.neighbors()
    b = o.bond_state()
    assert b.sum() > 0
    pairs = set()
    for i in range(p.n):
        for k in range(rp[i], rp[i + 1]):
            if b[k]:
                pairs.add((i, int(cols[k])))
    # a bond cut from one side is cut from the other (both ends tested)
    assert all((j, i) in pairs for (i, j) in pairs)
    # every cut bond straddles y = 0.02 inside x in [0.015, 0.025]
    for (i, j) in pairs:
        yi, yj = p.x[i, 1], p.x[j, 1]
        assert (yi - 0.02) * (yj - 0.02) <= 0


def test_fd_run_conserves_without_load(oracle):
    # no BC, no crack, zero initial state: nothing moves
    p = configs.rnp_plate(20, 1e-3, 3, 0.0, 0.1, 2e-8, 10)
    p.ubc = []
    o = oracle.OracleFD(p)
    o.run(5)
    u, v, f = o.state()
    assert np.abs(u).max() == 0 and np.abs(v).max() == 0


def test_fd_rigid_translation_is_force_free(oracle):
    p = configs.rnp_plate(16, 1e-3, 3, 0.0, 0.1, 2e-8, 10)
    p.ubc = []
    p.u0 = np.tile([1e-6, -2e-6, 0.0], (p.n, 1))
    o = oracle.OracleFD(p)
    o.run(1)
    u, v, f = o.state()
    assert np.abs(f).max() < 1e-6 * 1e9


def test_fd_momentum_balance(oracle):
    # internal forces are pairwise equal and opposite when all volumes match
    p = configs.rnp_plate(24, 1e-3, 3, 0.0, 0.1, 2e-8, 10, jitter=0.0)
    p.ubc = []
    rng = np.random.default_rng(0)
    p.u0 = np.zeros((p.n, 3))
    p.u0[:, :2] = rng.normal(scale=1e-8, size=(p.n, 2))
    o = oracle.OracleFD(p)
    f = o.eval_force()
    tot = f.sum(axis=0)
    assert np.abs(tot).max() < 1e-9 * np.abs(f).sum()


def test_config_shapes():
    p = configs.config0()
    assert p.n == 10000 and p.horizon == pytest.approx(4e-3)
    assert len(p.ubc) == 2 and len(p.cracks) == 1
    assert np.all(np.abs(p.x[:, 0] - (np.round(p.x[:, 0] / 1e-3 - 0.5) + 0.5) * 1e-3) <= 0.05e-3 + 1e-15)
