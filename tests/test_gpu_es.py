"""Parity of the CUDA ElasticState two-pass explicit path with the oracle.

The reference has no explicit ElasticState model and no ElasticState damage;
the build defines them (gather form of the QS half-force scatter, break when
e/|X| > s_c, broken bonds excluded from dilatation and force).  The oracle
implements the same definition in plain FP64 and is itself pinned to the
reference's quasi-static golden results through the shared ElasticState
arithmetic (tests/test_oracle.py).
"""
import numpy as np
import pytest

from nlmech_gb300 import abi, configs
from nlmech_gb300.decks import BC

pytestmark = pytest.mark.gpu


def rel_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def pairs(rowptr, cols, broken):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    sel = broken.astype(bool)
    return set(zip(rows[sel].tolist(), cols[sel].tolist()))


def cube(n=14, vscale=20.0, ref_compat=False, sc=5e-4, seed=0):
    p = configs.elastic_state_cube(n, 1e-3, sc=sc, seed=seed, ref_compat=ref_compat)
    p.v0 = p.v0 * vscale
    return p


@pytest.mark.parametrize("ref_compat", [False, True])
def test_es3d_fp64_parity(gpu, oracle, ref_compat):
    p = cube(ref_compat=ref_compat)
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    rowptr, cols = o.neighbors()
    assert np.array_equal(m.bond_state(), o.bond_state())  # notch bonds
    for n in (1, 79):
        m.run(n)
        o.run(n)
    u, v, f = m.state()
    uo, vo, fo = o.state()
    assert rel_max(u, uo) <= 1e-12
    assert rel_max(v, vo) <= 1e-12
    assert rel_max(f, fo) <= 1e-12
    assert pairs(rowptr, cols, m.bond_state()) == pairs(rowptr, cols, o.bond_state())
    phi, Z = m.damage()
    phio, Zo = o.damage()
    assert np.abs(phi - phio).max() <= 1e-6


def test_es3d_breaks_bonds(gpu, oracle):
    p = cube(vscale=200.0)
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    b0 = int(o.bond_state().sum())
    m.run(60)
    o.run(60)
    rowptr, cols = o.neighbors()
    assert int(o.bond_state().sum()) > b0
    assert pairs(rowptr, cols, m.bond_state()) == pairs(rowptr, cols, o.bond_state())
    assert rel_max(m.state()[0], o.state()[0]) <= 1e-12


def test_es2d_fp64_parity(gpu, oracle):
    for plane_strain in (False, True):
        p = configs.rnp_plate(36, 1e-3, 3, 0.008, 0.5, 1e-8, 100, seed=4)
        p.material = configs.MaterialDeck(kind="ElasticState", density=2440.0, K=40e9, G=30e9,
                                          plane_strain=plane_strain, es_sc=2e-3)
        m = gpu.FDModel(p, precision=abi.FP64)
        o = oracle.OracleFD(p)
        m.run(100)
        o.run(100)
        u, v, f = m.state()
        uo, vo, fo = o.state()
        assert rel_max(u, uo) <= 1e-12 and rel_max(v, vo) <= 1e-12 and rel_max(f, fo) <= 1e-12


@pytest.mark.parametrize("decomp", [abi.DECOMP_THREAD, abi.DECOMP_TILE_LOCAL])
def test_es3d_fp32c_error(gpu, oracle, decomp):
    """FP32C against the FP64 oracle, thread-per-node kernels and tile-frame
    kernels (neighbours staged in shared memory), same bar."""
    p = cube(vscale=20.0)
    o = oracle.OracleFD(p)
    o.run(200)
    uo = o.state()[0]
    rowptr, cols = o.neighbors()
    bo = pairs(rowptr, cols, o.bond_state())
    m = gpu.FDModel(p, precision=abi.FP32C, decomposition=decomp)
    assert m.decomposition() == decomp
    m.run(200)
    u = m.state()[0]
    assert rel_l2(u, uo) <= 1e-5
    bm = pairs(rowptr, cols, m.bond_state())
    assert len(bm ^ bo) <= 1e-3 * max(len(bo), 1) + 2


@pytest.mark.parametrize("decomp", [abi.DECOMP_THREAD, abi.DECOMP_TILE_LOCAL])
def test_es2d_fp32c_error(gpu, oracle, decomp):
    p = configs.rnp_plate(36, 1e-3, 3, 0.008, 0.5, 1e-8, 100, seed=4)
    p.material = configs.MaterialDeck(kind="ElasticState", density=2440.0, K=40e9, G=30e9,
                                      es_sc=2e-3)
    m = gpu.FDModel(p, precision=abi.FP32C, decomposition=decomp)
    o = oracle.OracleFD(p)
    m.run(100)
    o.run(100)
    assert rel_l2(m.state()[0], o.state()[0]) <= 1e-5
    assert rel_l2(m.state()[1], o.state()[1]) <= 1e-4


def test_es3d_fp32c_tile_matches_thread_large(gpu):
    """40^3 nodes (250 tiles, most of them interior with full halos, some
    across jumps of the Morton order): the tile-frame kernels follow the
    thread kernels through breaking."""
    p = configs.elastic_state_cube(40, 1e-3, sc=5e-4, seed=3)
    p.v0 = p.v0 * 50.0
    a = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_THREAD)
    b = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    a.run(150)
    b.run(150)
    assert a.count_broken() > 0
    assert abs(a.count_broken() - b.count_broken()) <= 1e-3 * a.count_broken() + 2
    assert rel_l2(b.state()[0], a.state()[0]) <= 1e-5
    assert rel_l2(b.state()[1], a.state()[1]) <= 1e-4


def test_es_central_difference(gpu, oracle):
    p = cube(n=12, vscale=20.0)
    p.scheme = abi.CENTRAL_DIFFERENCE
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    m.run(50)
    o.run(50)
    assert rel_max(m.state()[0], o.state()[0]) <= 1e-12
    t = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    t.run(50)
    assert rel_l2(t.state()[0], o.state()[0]) <= 1e-5
