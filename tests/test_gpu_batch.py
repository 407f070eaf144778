"""Batched specimens and CUDA-graph replay.

A batch steps many independent plates in one launch per node-count bucket;
each plate must match its own oracle run (FP32C tolerance), its neighbour
and pre-crack sets must equal a separate model's, and graph replay must give
bit-identical results to plain launches.
"""
import numpy as np
import pytest

from nlmech_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def pairs(rowptr, cols, broken):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    sel = broken.astype(bool)
    return set(zip(rows[sel].tolist(), cols[sel].tolist()))


def small_ensemble(n=7, seed=3):
    return configs.ensemble(nplates=n, nmin=600, nmax=3000, seed=seed, steps=300)


@pytest.mark.parametrize("decomp", [None, abi.DECOMP_THREAD, abi.DECOMP_TILE_LOCAL])
def test_batch_matches_oracle_per_plate(gpu, oracle, decomp):
    """Autotuned buckets, thread kernels, and tile-frame kernels whose tiles
    straddle specimens of a few hundred to a few thousand nodes."""
    plates = small_ensemble()
    b = gpu.Batch(plates, decomposition=decomp)
    if decomp is not None:
        assert all(dc == decomp for _, dc in b.buckets())
    assert b.nnz() == sum(b.nnz(s) for s in range(len(plates)))
    bond0 = [b.bond_state(s) for s in range(len(plates))]
    b.run(300)
    for s, p in enumerate(plates):
        o = oracle.OracleFD(p)
        rowptr, cols = o.neighbors()
        assert b.nnz(s) == len(cols)
        assert np.array_equal(bond0[s], o.bond_state())  # pre-cracks
        o.run(300)
        u = b.state(s)[0]
        uo = o.state()[0]
        assert rel_l2(u, uo) <= 1e-5, s
        d = len(pairs(rowptr, cols, b.bond_state(s)) ^ pairs(rowptr, cols, o.bond_state()))
        assert d <= 1e-3 * max(int(o.bond_state().sum()), 1) + 2, s
    assert b.time()[1] == 300


@pytest.mark.parametrize("decomp", [abi.DECOMP_THREAD, abi.DECOMP_TILE_LOCAL])
def test_batch_graph_replay_is_bit_identical(gpu, decomp):
    plates = small_ensemble(n=5, seed=8)
    a = gpu.Batch(plates, decomposition=decomp)
    a.run(101)
    g = gpu.Batch(plates, decomposition=decomp)
    g.set_graph(20)
    g.run(101)
    assert a.time() == g.time()
    for s in range(len(plates)):
        for x, y in zip(a.state(s), g.state(s)):
            assert np.array_equal(x, y)
        assert np.array_equal(a.bond_state(s), g.bond_state(s))


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32C])
def test_fd_graph_replay_is_bit_identical(gpu, prec):
    p = configs.config0()
    a = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
    a.run(130)
    g = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
    g.set_graph(16)
    g.run(70)
    g.run(60)
    assert a.time() == g.time()
    for x, y in zip(a.state(), g.state()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.bond_state(), g.bond_state())


def test_batch_rejects_mixed_inputs(gpu):
    plates = small_ensemble(n=2)
    plates[1] = configs.rnp_plate(20, 1e-3, 3, 0.0, 0.1, 1e-8, 10)  # other dt
    with pytest.raises(gpu.NLMError):
        gpu.Batch(plates)
