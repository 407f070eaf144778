"""Parity of the CUDA RNPBond explicit path with the CPU oracle.

Bars (the benchmark spec): neighbour lists bit-exact (identical sorted index sets);
broken-bond set identical and u, v, f within 1e-12 relative in FP64 plain
mode; FP32-compensated mode within 1e-5 relative L2 of the FP64 displacement
and at most 0.1% differing broken bonds.
"""
import numpy as np
import pytest

from nlmech_gb300 import abi, configs
from nlmech_gb300.decks import BC

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12     # relative to the largest magnitude of the field
FP32_L2 = 1e-5        # relative L2 of u against the FP64 oracle
FP32_BROKEN = 1e-3    # fraction of differing broken bonds


def rel_max(a, b):
    s = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / s)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def bonds_as_pairs(rowptr, cols, broken):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    sel = broken.astype(bool)
    return set(zip(rows[sel].tolist(), cols[sel].tolist()))


def test_neighbor_search_bit_exact(gpu, oracle):
    for ratio, seed in ((4, 0), (3, 1)):
        x, _ = configs.grid2d(100, 100, 1e-3, seed=seed)
        a = gpu.neighbor_search(x, ratio * 1e-3, dim=2)
        b = oracle.neighbors(x, ratio * 1e-3, dim=2, grid=False)
        assert np.array_equal(a[0], b[0])
        assert np.array_equal(a[1], b[1])
    x3, _ = configs.grid3d(14, 13, 12, 1e-3, seed=2)
    a = gpu.neighbor_search(x3, 3e-3, dim=3)
    b = oracle.neighbors(x3, 3e-3, dim=3, grid=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_neighbor_search_edge_cases(gpu, oracle):
    # single node, two nodes at exactly the horizon, empty
    a = gpu.neighbor_search(np.zeros((1, 3)), 1.0)
    assert list(a[0]) == [0, 0]
    x = np.array([[0., 0, 0], [1., 0, 0], [0., 0.5, 0]])
    a = gpu.neighbor_search(x, 1.0)
    b = oracle.neighbors(x, 1.0, grid=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    a = gpu.neighbor_search(np.zeros((0, 3)), 1.0)
    assert list(a[0]) == [0]
    # coincident points and a dense cluster
    rng = np.random.default_rng(5)
    x = np.zeros((300, 3))
    x[:, :2] = rng.uniform(0, 1e-3, size=(300, 2))
    x[10] = x[11]
    a = gpu.neighbor_search(x, 2e-4)
    b = oracle.neighbors(x, 2e-4, grid=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_model_neighbors_and_precrack(gpu, oracle):
    p = configs.config0()
    o = oracle.OracleFD(p, grid_neighbors=False)
    rb, cb = o.neighbors()
    for prec in (abi.FP64, abi.FP32C):
        m = gpu.FDModel(p, precision=prec)
        ra, ca = m.neighbors()
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
        assert np.array_equal(m.bond_state(), o.bond_state())
        assert m.count_broken() == int(o.bond_state().sum())


def _compare_fp64(m, o, rowptr, cols, what=""):
    u, v, f = m.state()
    uo, vo, fo = o.state()
    assert rel_max(u, uo) <= FP64_RTOL, what + " u"
    assert rel_max(v, vo) <= FP64_RTOL, what + " v"
    assert rel_max(f, fo) <= FP64_RTOL, what + " f"
    bm, bo = m.bond_state(), o.bond_state()
    assert bonds_as_pairs(rowptr, cols, bm) == bonds_as_pairs(rowptr, cols, bo), what + " bonds"
    assert m.time() == o.time()


def test_fp64_config0_parity(gpu, oracle):
    """Config 0 in full: 100x100 plate, 1000 Verlet steps, FP64 plain."""
    p = configs.config0()
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    rowptr, cols = o.neighbors()
    done = 0
    for n in (1, 9, 190, 800):
        m.run(n)
        o.run(n)
        done += n
        _compare_fp64(m, o, rowptr, cols, "step %d" % done)
    assert int(o.bond_state().sum()) > 10000  # the crack has grown
    phi, Z = m.damage()
    phio, Zo = o.damage()
    assert np.abs(phi - phio).max() <= 1e-6
    assert np.abs(Z - Zo).max() <= 1e-5 * max(1.0, np.abs(Zo).max())


def test_fp64_central_difference_parity(gpu, oracle):
    p = configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)
    m = gpu.FDModel(p, precision=abi.FP64, scheme=abi.CENTRAL_DIFFERENCE)
    p2 = configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)
    p2.scheme = abi.CENTRAL_DIFFERENCE
    o = oracle.OracleFD(p2)
    rowptr, cols = o.neighbors()
    m.run(300)
    o.run(300)
    _compare_fp64(m, o, rowptr, cols, "CD")


def test_fp64_loads_nofail_influence(gpu, oracle):
    """Force BC, a sin-in-time displacement BC, no-fail boundary layer and a
    linear influence function, all through the same step kernel."""
    p = configs.rnp_plate(40, 1e-3, 3, 0.01, 0.3, 2e-8, 200, seed=11)
    p.material.influence_type = 1
    p.material.influence_params = []
    p.fbc = [BC(region="rectangle", x1=0.0, x2=0.004, y1=0.0, y2=0.04, direction=[1],
                time_fn="linear", time_params=[1.0], spatial_fn="constant",
                spatial_params=[-2e12]),
             BC(region="rectangle", x1=0.0, x2=0.002, y1=0.0, y2=0.04, direction=[1, 2],
                time_fn="sin", time_params=[1.0, 2e4], spatial_fn="linear_y",
                spatial_params=[1e14])]
    p.ubc.append(BC(region="rectangle", x1=0.036, x2=0.041, y1=0.01, y2=0.03, direction=[1],
                    time_fn="sin", time_params=[1e-7, 5e4], spatial_fn="constant",
                    spatial_params=[1.0]))
    p.no_fail = abi.NOFAIL_COMPUTE
    p.no_fail_tol = 2e-3
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    rowptr, cols = o.neighbors()
    m.run(200)
    o.run(200)
    u, v, f = m.state()
    uo, vo, fo = o.state()
    # sin/cos of the BC and exp of the bond are libm-vs-CUDA last-ulp apart
    assert rel_max(u, uo) <= 1e-11
    assert rel_max(v, vo) <= 1e-11
    assert rel_max(f, fo) <= 1e-11
    assert bonds_as_pairs(rowptr, cols, m.bond_state()) == bonds_as_pairs(rowptr, cols, o.bond_state())


def test_fp64_3d_rnp_parity(gpu, oracle):
    x, vol = configs.grid3d(14, 14, 14, 1e-3, seed=3)
    p = configs.rnp_plate(8, 1e-3, 3, 0.0, 0.1, 2e-8, 10)
    p.dim = 3
    p.x, p.volume = x, vol
    p.horizon = 3e-3
    p.cracks = []
    p.ubc = [BC(region="cuboid", x1=-1, x2=1, y1=-1, y2=1, z1=-1, z2=2e-3, direction=[3],
                time_fn="linear", time_params=[-0.5]),
             BC(region="cuboid", x1=-1, x2=1, y1=-1, y2=1, z1=12e-3, z2=1, direction=[3],
                time_fn="linear", time_params=[0.5])]
    m = gpu.FDModel(p, precision=abi.FP64)
    o = oracle.OracleFD(p)
    rowptr, cols = o.neighbors()
    m.run(150)
    o.run(150)
    _compare_fp64(m, o, rowptr, cols, "3D")


def test_fp32c_config0_error(gpu, oracle):
    """FP32-compensated against the FP64 oracle on config 0 (1000 steps)."""
    p = configs.config0()
    o = oracle.OracleFD(p)
    o.run(1000)
    uo, vo, fo = o.state()
    rowptr, cols = o.neighbors()
    bo = bonds_as_pairs(rowptr, cols, o.bond_state())
    for dec in (abi.DECOMP_THREAD, abi.DECOMP_THREAD1, abi.DECOMP_WARP, abi.DECOMP_TILE,
                abi.DECOMP_TILE_LOCAL,
                abi.DECOMP_AUTO):
        m = gpu.FDModel(p, precision=abi.FP32C, decomposition=dec)
        m.run(1000)
        u, v, f = m.state()
        assert rel_l2(u, uo) <= FP32_L2
        bm = bonds_as_pairs(rowptr, cols, m.bond_state())
        ndiff = len(bm ^ bo)
        assert ndiff <= FP32_BROKEN * max(len(bo), 1), (ndiff, len(bo))


def test_step_host_matches_run(gpu):
    """Host-resident drop-in: calls that pass back the previous arrays
    continue the run bit for bit."""
    p = configs.rnp_plate(30, 1e-3, 3, 0.008, 0.1, 2e-8, 50, seed=2)
    for prec in (abi.FP64, abi.FP32C):
        a = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        a.run(20)
        ua, va, fa = a.state()
        b = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        u = np.zeros((p.n, 3))
        v = np.zeros((p.n, 3))
        f = np.zeros((p.n, 3))
        b.step_host(u, v, f, nsteps=5)
        for _ in range(15):
            b.step_host(u, v, f, nsteps=1)
        assert b.time() == a.time()
        if prec == abi.FP64:
            assert np.array_equal(u, ua) and np.array_equal(v, va) and np.array_equal(f, fa)
        else:
            assert rel_max(u, ua) < 1e-12 and rel_max(v, va) < 1e-9


def test_step_host_rejects_nonfinite_state(gpu):
    """A non-finite value in the host state is found on the device before
    the state is replaced: the call fails and the model is unchanged."""
    p = configs.rnp_plate(30, 1e-3, 3, 0.008, 0.1, 2e-8, 50, seed=2)
    m = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_THREAD)
    u, v, f = np.zeros((p.n, 3)), np.zeros((p.n, 3)), np.zeros((p.n, 3))
    m.step_host(u, v, f, nsteps=3)
    t0 = m.time()
    u0 = m.state()[0].copy()
    bad = v.copy()
    bad[7, 1] = np.nan
    with pytest.raises(gpu.NLMError):
        m.step_host(u, bad, f, nsteps=1)
    assert m.time() == t0
    assert np.array_equal(m.state()[0], u0)


def test_runs_are_deterministic(gpu):
    p = configs.config0()
    for prec in (abi.FP64, abi.FP32C):
        r = []
        for _ in range(2):
            m = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
            m.run(300)
            r.append(m.state() + (m.bond_state(),))
        for a, b in zip(r[0], r[1]):
            assert np.array_equal(a, b)


def test_tile_decomposition_bit_identical_to_thread(gpu):
    """The tile kernel runs the thread kernel's bond loop on staged copies:
    same bond order, same arithmetic, bit-identical state."""
    for p in (configs.config0(), configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)):
        a = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_THREAD)
        b = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE)
        assert b.decomposition() == abi.DECOMP_TILE
        a.run(300)
        b.run(300)
        for x, y in zip(a.state(), b.state()):
            assert np.array_equal(x, y)
        assert np.array_equal(a.bond_state(), b.bond_state())


def test_tile_decomposition_rejected_where_unsupported(gpu):
    p = configs.config0()
    for dec in (abi.DECOMP_TILE, abi.DECOMP_TILE_LOCAL):
        with pytest.raises(gpu.NLMError):
            gpu.FDModel(p, precision=abi.FP64, decomposition=dec)
    # ElasticState has the tile-frame kernels only
    q = configs.elastic_state_cube(8, 1e-3)
    with pytest.raises(gpu.NLMError):
        gpu.FDModel(q, precision=abi.FP32C, decomposition=abi.DECOMP_TILE)
    assert gpu.FDModel(q, precision=abi.FP32C,
                       decomposition=abi.DECOMP_TILE_LOCAL).decomposition() == abi.DECOMP_TILE_LOCAL


def test_checkpoint_restart_continues_the_run(gpu, tmp_path):
    """Save after 150 steps of a growing crack, load into a fresh handle,
    run on: the state, broken bonds and time equal those of the run that
    never stopped (bit for bit in FP64, FP32C within its split rounding)."""
    p = configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)
    for prec in (abi.FP64, abi.FP32C):
        a = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        a.run(150)
        path = tmp_path / ("ckpt_%d.bin" % prec)
        a.save(path)
        a.run(150)
        b = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        b.load(path)
        b.run(150)
        assert b.time() == a.time()
        assert np.array_equal(b.bond_state(), a.bond_state())
        assert int(a.bond_state().sum()) > 1000
        ua, va, fa = a.state()
        ub, vb, fb = b.state()
        if prec == abi.FP64:
            assert np.array_equal(ua, ub) and np.array_equal(va, vb) and np.array_equal(fa, fb)
        else:
            assert rel_max(ub, ua) < 1e-12 and rel_max(vb, va) < 1e-9
    # a checkpoint of another model is refused
    q = gpu.FDModel(configs.rnp_plate(40, 1e-3, 3, 0.01, 0.5, 2e-8, 10, seed=1))
    with pytest.raises(gpu.NLMError):
        q.load(path)


def test_checkpoint_with_nonfinite_state_leaves_model_unchanged(gpu, tmp_path):
    """A checkpoint whose state holds a NaN is refused before the handle
    changes: time, step, bond state and u stay those of the running model,
    and a sound checkpoint loads afterwards."""
    p = configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)
    a = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_THREAD)
    a.run(150)
    good = tmp_path / "good.bin"
    a.save(good)
    raw = bytearray(good.read_bytes())
    header = 72  # CkptHeader: magic, 5 int32, uint32, 3 int64, 2 doubles
    raw[header + 8 * 16: header + 8 * 17] = np.array([np.nan]).tobytes()  # u of node 5, y
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    b = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_THREAD)
    b.run(20)
    t0, bonds0, u0 = b.time(), b.bond_state(), b.state()[0]
    with pytest.raises(gpu.NLMError) as e:
        b.load(bad)
    assert e.value.code == 7  # NLM_ERR_NONFINITE
    assert b.time() == t0
    assert np.array_equal(b.bond_state(), bonds0)
    assert np.array_equal(b.state()[0], u0)
    b.load(good)
    assert b.time() == a.time()
    assert np.array_equal(b.bond_state(), a.bond_state())


def test_write_vtu_output_step(gpu, tmp_path):
    from nlmech_gb300 import vtu
    p = configs.rnp_plate(30, 1e-3, 3, 0.008, 0.3, 2e-8, 50, seed=2)
    m = gpu.FDModel(p, precision=abi.FP64)
    m.run(50)
    path = tmp_path / "output_50.vtu"
    m.write_vtu(path)
    d = vtu.read_vtu(str(path))
    u, v, f = m.state()
    phi, Z = m.damage()
    assert np.array_equal(d["Displacement"], u) and np.array_equal(d["Velocity"], v)
    assert np.array_equal(d["Points"], p.x + u)
    assert np.array_equal(d["Force"], f * p.volume[:, None])
    assert np.array_equal(d["Damage_Phi"], phi) and np.array_equal(d["Damage_Z"], Z)
    assert d["TIME"][0] == m.time()[0]


def test_timed_cracks_with_graph_replay(gpu, oracle):
    """Timed cracks (Fracture::addCrack after every step) with and without
    CUDA-graph replay: a graph chunk in which a crack falls due runs step by
    step, so the broken bonds and u equal the oracle's at every check."""
    import refcases
    p = refcases.timed_crack_plate()
    o = oracle.OracleFD(p)
    rowptr, cols = o.neighbors()
    runs = []
    for prec, graph, dec in ((abi.FP64, 0, abi.DECOMP_THREAD), (abi.FP64, 8, abi.DECOMP_THREAD),
                             (abi.FP32C, 8, abi.DECOMP_TILE)):
        m = gpu.FDModel(p, precision=prec, decomposition=dec)
        m.set_graph(graph)
        runs.append((prec, m))
    for n in (1, 15, 1, 1, 22, 160):
        o.run(n)
        ref = bonds_as_pairs(rowptr, cols, o.bond_state())
        uo = o.state()[0]
        for prec, m in runs:
            m.run(n)
            assert m.time() == o.time()
            got = bonds_as_pairs(rowptr, cols, m.bond_state())
            if prec == abi.FP64:
                assert got == ref
                assert rel_max(m.state()[0], uo) <= FP64_RTOL
            else:
                assert len(got ^ ref) <= FP32_BROKEN * len(ref)
                assert rel_l2(m.state()[0], uo) <= FP32_L2


def test_timed_crack_checkpoint_between_activations(gpu, tmp_path):
    """A checkpoint taken after step 17 (one of the two cracks due at 3e-7 s
    cut) restarts with the second still pending: it is cut before step 18."""
    import refcases
    p = refcases.timed_crack_plate()
    a = gpu.FDModel(p, precision=abi.FP64)
    a.run(17)
    path = tmp_path / "timed.bin"
    a.save(path)
    n17 = int(a.bond_state().sum())
    a.run(24)
    b = gpu.FDModel(p, precision=abi.FP64)
    b.load(path)
    b.run(1)
    assert int(b.bond_state().sum()) > n17 + 200  # the pending crack
    b.run(23)
    assert np.array_equal(a.bond_state(), b.bond_state())
    assert np.array_equal(a.state()[0], b.state()[0])


def test_timed_cracks_rejected_by_batch_and_qs(gpu):
    import refcases
    p = refcases.timed_crack_plate()
    with pytest.raises(gpu.NLMError):
        gpu.Batch([p])
    q = configs.qs_plate(nx=40)
    q.cracks[0].activation_time = 1.0
    with pytest.raises(gpu.NLMError):
        gpu.QSModel(q, gpu.qs_params())


def test_bc_function_names_checked_like_the_reference(gpu):
    """ULoading accepts only constant / sin_* / linear_* spatial functions and
    FLoading no quadratic time function (uLoading.cpp:35-53,
    fLoading.cpp:33-52): such decks are refused, not run."""
    p = configs.rnp_plate(20, 1e-3, 3, 0.0, 0.1, 2e-8, 10)
    p.ubc[0].spatial_fn = "hat_x"
    with pytest.raises(gpu.NLMError):
        gpu.FDModel(p)
    p = configs.rnp_plate(20, 1e-3, 3, 0.0, 0.1, 2e-8, 10)
    p.fbc = [BC(region="rectangle", x1=0.0, x2=0.02, y1=0.0, y2=0.02, direction=[1],
                time_fn="quadratic", time_params=[1.0, 1.0])]
    with pytest.raises(gpu.NLMError):
        gpu.FDModel(p)


def test_graph_replay_with_force_loads(gpu):
    """Force_BC loads evaluated inside the graph at each step's time: the same
    state as plain launches, bit for bit (FP64)."""
    import refcases
    runs = []
    for graph in (0, 8):
        m = gpu.FDModel(refcases.loads_nofail_plate(), precision=abi.FP64)
        m.set_graph(graph)
        m.run(3)
        m.run(61)
        runs.append(m.state())
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_step_host_in_place_matches_copies(gpu):
    """Page-locked arrays are read and written in place by kernels; pageable
    ones go through copies.  Both give the same state bit for bit, keep the
    caller's z of u and v in 2-D, write f's z as 0, and refuse a non-finite
    input without touching the model."""
    torch = pytest.importorskip("torch")
    p = configs.rnp_plate(30, 1e-3, 3, 0.008, 0.1, 2e-8, 50, seed=2)
    n = p.n
    for prec in (abi.FP64, abi.FP32C):
        a = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        b = gpu.FDModel(p, precision=prec, decomposition=abi.DECOMP_THREAD)
        host = [np.zeros((n, 3)) for _ in range(3)]
        pin = [torch.zeros((n, 3), dtype=torch.float64).pin_memory() for _ in range(3)]
        for arr in (host[0], host[1], pin[0].numpy(), pin[1].numpy()):
            arr[:, 2] = 7.0
        ptrs = [t.data_ptr() for t in pin]
        for k in range(4):
            a.step_host(*host, nsteps=3)
            b.step_host_ptr(*ptrs, nsteps=3)
        assert a.host_io() == 0 and b.host_io() == 1
        for x, y in zip(host, pin):
            assert np.array_equal(x, y.numpy())
        assert np.all(host[0][:, 2] == 7.0) and np.all(host[1][:, 2] == 7.0)
        assert np.all(host[2][:, 2] == 0.0)
        t0, u0 = b.time(), b.state()[0].copy()
        pin[1].numpy()[5, 0] = np.inf
        with pytest.raises(gpu.NLMError):
            b.step_host_ptr(*ptrs, nsteps=1)
        assert b.time() == t0 and np.array_equal(b.state()[0], u0)


def _pinned_state(torch, n):
    pin = [torch.zeros((n, 3), dtype=torch.float64).pin_memory() for _ in range(3)]
    pin[0].numpy()[:, 2] = 7.0
    pin[1].numpy()[:, 2] = -3.0
    return pin, [t.data_ptr() for t in pin]


@pytest.mark.parametrize("nx,shuffle", [(300, False), (800, False), (300, True)])
def test_step_host_banded_matches_copies(gpu, nx, shuffle):
    """Page-locked arrays of a large 2-D FP32C model on a tile decomposition
    move in caller-order bands whose copies overlap the step (host_io 2: six
    bands at 300 x 300, seven at 800 x 800, with late nodes where tiles
    straddle a jump of the Morton order).  Arrays, state and bond bits
    match the copy path bit for bit, through breaking at the loaded edges.
    With the caller's nodes in random order every band touches every tile:
    the schedule degenerates (most nodes late or released at the end) and
    must still be exact."""
    torch = pytest.importorskip("torch")
    p = configs.rnp_plate(nx, 1e-4, 3, 0.2 * nx * 1e-4, 50.0, 2e-9, 50, seed=4)
    if shuffle:
        order = np.random.default_rng(5).permutation(p.n)
        p.x = np.ascontiguousarray(np.asarray(p.x).reshape(-1, 3)[order])
        p.volume = np.ascontiguousarray(np.asarray(p.volume)[order])
    n = p.n
    a = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    b = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    host = [np.zeros((n, 3)) for _ in range(3)]
    host[0][:, 2] = 7.0
    host[1][:, 2] = -3.0
    pin, ptrs = _pinned_state(torch, n)
    for k in range(13):
        a.step_host(*host, nsteps=1)
        b.step_host_ptr(*ptrs, nsteps=1)
        if k > 0:
            assert a.host_io() == 0 and b.host_io() == 2
    assert a.time() == b.time()
    for x, y in zip(host, pin):
        assert np.array_equal(x, y.numpy())
    assert a.count_broken() > 0
    assert np.array_equal(a.bond_state(), b.bond_state())
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    a.run(3)
    b.run(3)
    assert np.array_equal(a.state()[0], b.state()[0])


def test_step_host_banded_falls_back_when_buffers_fail(gpu):
    """With the handle's device allocations capped below what the banded
    path stages (about 200 bytes per node) but above what the in-place path
    needs (about 70), the first banded call frees what it had set up and the
    in-place path serves it and every later call: results equal the copy
    path bit for bit and no error text is left behind."""
    torch = pytest.importorskip("torch")
    p = configs.rnp_plate(300, 1e-4, 3, 0.006, 50.0, 2e-9, 50, seed=4)
    n = p.n
    a = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    b = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    host = [np.zeros((n, 3)) for _ in range(3)]
    host[0][:, 2] = 7.0
    host[1][:, 2] = -3.0
    pin, ptrs = _pinned_state(torch, n)
    a.step_host(*host, nsteps=1)
    b.step_host_ptr(*ptrs, nsteps=1)
    b.set_alloc_limit(80 * n + 4096)
    for _ in range(6):
        a.step_host(*host, nsteps=1)
        b.step_host_ptr(*ptrs, nsteps=1)
        assert a.host_io() == 0 and b.host_io() == 1
    assert gpu.load().nlm_last_error() == b""
    for x, y in zip(host, pin):
        assert np.array_equal(x, y.numpy())
    assert np.array_equal(a.bond_state(), b.bond_state())
    b.set_alloc_limit(-1)


def test_step_host_banded_rejects_nonfinite(gpu):
    """A non-finite value in the last band is found after earlier bands were
    already written back: the call fails, the model (time, state, bond bits)
    is unchanged and the caller's arrays hold their input again."""
    torch = pytest.importorskip("torch")
    p = configs.rnp_plate(300, 1e-4, 3, 0.006, 50.0, 2e-9, 50, seed=4)
    n = p.n
    m = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
    pin, ptrs = _pinned_state(torch, n)
    for _ in range(6):
        m.step_host_ptr(*ptrs, nsteps=1)
    assert m.host_io() == 2 and m.count_broken() > 0
    t0, st0, bonds0 = m.time(), m.state(), m.bond_state()
    pin[1].numpy()[n - 5, 0] = np.inf
    keep = [t.numpy().copy() for t in pin]
    with pytest.raises(gpu.NLMError):
        m.step_host_ptr(*ptrs, nsteps=1)
    assert m.time() == t0
    for x, y in zip(m.state(), st0):
        assert np.array_equal(x, y)
    assert np.array_equal(m.bond_state(), bonds0)
    for t, k in zip(pin, keep):
        assert np.array_equal(t.numpy(), k)
    # with the value put back the run continues
    pin[1].numpy()[n - 5, 0] = st0[1][n - 5, 0]
    m.step_host_ptr(*ptrs, nsteps=1)
    assert m.time() > t0


def test_tile_frame_interior_prefix_is_exact(gpu):
    """The tile-frame kernel evaluates the leading bonds of a row that lie
    certainly inside the horizon's interior (r <= check_low - 1e-3 h, where
    the volume factor min(1, (check_up - r) / h) is 1) without forming the
    factor (rnpBond.cpp:242-256); it does so for a constant influence
    function only.  The linear influence function J = 1 + 0 r / delta has
    the same constants and multiplies every bond by exactly 1, but takes the
    general path for every bond.  Both runs of the 100 x 100 plate (crack
    growing, 600 steps) agree bit for bit."""
    import dataclasses
    p0 = configs.config0()
    p1 = dataclasses.replace(p0, material=dataclasses.replace(
        p0.material, influence_type=1, influence_params=[1.0, 0.0]))
    out = []
    for p in (p0, p1):
        m = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_TILE_LOCAL)
        pre = np.count_nonzero(m.bond_state())
        m.run(600)
        out.append((m.state(), m.bond_state(), pre))
        m.close()
    (s0, b0, pre0), (s1, b1, _) = out
    for a, b in zip(s0, s1):
        assert np.array_equal(a, b)
    assert np.array_equal(b0, b1)
    assert np.count_nonzero(b0) > pre0  # the crack grew
