"""Seeded synthetic specimens with the shapes of the benchmark workloads.

No dataset is involved: every workload is a jittered grid built from a fixed
seed.  Conventions shared by all generators:

* cell-centred nodes x = (i + 1/2) h (and y, z), each moved by a seeded
  uniform offset in [-jitter*h, +jitter*h] per coordinate;
* nodal volume h^dim, mesh size h, horizon = ratio * h;
* the reference deck fields (Material, Displacement_BC, Fracture) are filled
  the way an NLMech input file would fill them.
"""
import numpy as np

from . import abi
from .decks import BC, Crack, MaterialDeck, Problem  # noqa: F401


def glass_rnp(plane_strain=False):
    """E = 72 GPa, rho = 2440 kg/m^3, Gc = 3.8 J/m^2, constant influence J = 1."""
    return MaterialDeck(kind="RNPBond", density=2440.0, E=72e9, Gc=3.8,
                        plane_strain=plane_strain, influence_type=0,
                        influence_params=[1.0])


def grid2d(nx, ny, h, jitter=0.05, seed=0):
    rng = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = np.zeros((nx * ny, 3))
    x[:, 0] = (ii.ravel() + 0.5) * h
    x[:, 1] = (jj.ravel() + 0.5) * h
    if jitter > 0:
        x[:, :2] += rng.uniform(-jitter * h, jitter * h, size=(nx * ny, 2))
    vol = np.full(nx * ny, h * h)
    return x, vol


def grid3d(nx, ny, nz, h, jitter=0.05, seed=0):
    rng = np.random.default_rng(seed)
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n = nx * ny * nz
    x = np.zeros((n, 3))
    x[:, 0] = (ii.ravel() + 0.5) * h
    x[:, 1] = (jj.ravel() + 0.5) * h
    x[:, 2] = (kk.ravel() + 0.5) * h
    if jitter > 0:
        x += rng.uniform(-jitter * h, jitter * h, size=(n, 3))
    vol = np.full(n, h ** 3)
    return x, vol


def rnp_plate(nx, h, ratio, crack_len, speed, dt, steps, seed=0, layers=3, ny=None,
              jitter=0.05, name=""):
    """2-D RNPBond plate nx x ny, centred horizontal pre-crack, top/bottom
    layers pulled apart at +-speed in y (Displacement_BC, linear in time)."""
    ny = nx if ny is None else ny
    x, vol = grid2d(nx, ny, h, jitter, seed)
    W, H = nx * h, ny * h
    ubc = [
        BC(region="rectangle", x1=-h, x2=W + h, y1=-h, y2=layers * h, direction=[2],
           time_fn="linear", time_params=[-speed], spatial_fn="constant", spatial_params=[1.0]),
        BC(region="rectangle", x1=-h, x2=W + h, y1=H - layers * h, y2=H + h, direction=[2],
           time_fn="linear", time_params=[speed], spatial_fn="constant", spatial_params=[1.0]),
    ]
    cracks = []
    if crack_len > 0:
        yc = 0.5 * H
        cracks.append(Crack(kind="edge", orientation=1, pb=(0.5 * W - 0.5 * crack_len, yc),
                            pt=(0.5 * W + 0.5 * crack_len, yc)))
    return Problem(dim=2, x=x, volume=vol, horizon=ratio * h, mesh_size=h,
                   material=glass_rnp(), ubc=ubc, cracks=cracks, dt=dt, steps=steps,
                   name=name)


def config0(seed=0):
    """100 x 100 plate, h = 1e-3 m, horizon 4h, 0.02 m centre pre-crack,
    +-0.1 m/s edge loading, velocity-Verlet dt = 2e-8 s, 1000 steps."""
    return rnp_plate(100, 1e-3, 4, 0.02, 0.1, 2e-8, 1000, seed=seed, name="rnp2d_100x100_d4h")


def config1(seed=0):
    """1000 x 1000 plate, h = 1e-4 m, horizon 3h, 2 mm pre-crack, +-0.1 m/s,
    dt = 2e-9 s, 5000 steps."""
    return rnp_plate(1000, 1e-4, 3, 2e-3, 0.1, 2e-9, 5000, seed=seed,
                     name="rnp2d_1000x1000_d3h")


def elastic_state_cube(n, h, ratio=3, sc=5e-4, dt=1e-8, steps=2000, seed=0, jitter=0.05,
                       ref_compat=False, name=""):
    """3-D ElasticState cube n^3 (K = 40 GPa, G = 30 GPa, rho = 2440),
    half-depth planar notch at mid-height z, opposite z-faces given seeded
    random initial velocities +-U[0.05, 0.2] m/s."""
    x, vol = grid3d(n, n, n, h, jitter, seed)
    L = n * h
    mat = MaterialDeck(kind="ElasticState", density=2440.0, K=40e9, G=30e9, es_sc=sc,
                       es_ref_compat=ref_compat)
    rng = np.random.default_rng(seed + 1)
    v0 = np.zeros_like(x)
    bot = x[:, 2] < h
    top = x[:, 2] > L - h
    v0[bot, 2] = -rng.uniform(0.05, 0.2, size=int(bot.sum()))
    v0[top, 2] = rng.uniform(0.05, 0.2, size=int(top.sum()))
    notch = Crack(kind="plane", z0=0.5 * L, lo=(-h, -h), hi=(0.5 * L, L + h))
    return Problem(dim=3, x=x, volume=vol, horizon=ratio * h, mesh_size=h, material=mat,
                   cracks=[notch], dt=dt, steps=steps, v0=v0, name=name)


def config2(seed=0):
    return elastic_state_cube(100, 1e-3, seed=seed, name="es3d_100cube_d3h")


def ensemble(nplates=256, nmin=5000, nmax=200000, seed=0, steps=1000):
    """Batched ensemble: plate i has N_i ~ U[nmin, nmax] nodes on a square grid,
    horizon 4h, crack length U[0.1, 0.4] W, speed log-U[0.01, 1] m/s."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(nplates):
        N = int(rng.integers(nmin, nmax + 1))
        nx = max(8, int(round(np.sqrt(N))))
        h = 0.1 / nx
        frac = rng.uniform(0.1, 0.4)
        speed = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        out.append(rnp_plate(nx, h, 4, frac * nx * h, speed, 2e-8, steps, seed=seed + 1000 + p,
                             name="plate%03d" % p))
    return out


def qs_plate(nx=200, h=5e-4, ratio=3, crack_frac=0.2, crack_center=(0.5, 0.5), du=1e-6,
             layers=3, jitter=0.0, seed=0, name=""):
    """Quasi-static RNPBond plate: nx x nx nodes, bottom `layers` rows fixed in
    x and y, top rows clamped in x and prescribed u_y = du * k at load step k
    (Displacement_BC, linear in the load parameter with dt = 1), horizontal
    pre-crack of length crack_frac * W centred at crack_center * W.  Clamping
    the top rows in x leaves no rigid-body mode once the crack has separated
    the plate."""
    x, vol = grid2d(nx, nx, h, jitter, seed)
    W = nx * h
    top = dict(region="rectangle", x1=-h, x2=W + h, y1=W - layers * h, y2=W + h)
    ubc = [
        BC(region="rectangle", x1=-h, x2=W + h, y1=-h, y2=layers * h, direction=[1, 2],
           time_fn="constant", time_params=[0.0], spatial_fn="constant", spatial_params=[1.0]),
        BC(direction=[1], time_fn="constant", time_params=[0.0], spatial_fn="constant",
           spatial_params=[1.0], **top),
        BC(direction=[2], time_fn="linear", time_params=[du], spatial_fn="constant",
           spatial_params=[1.0], **top),
    ]
    cx, cy = crack_center[0] * W, crack_center[1] * W
    L = crack_frac * W
    cracks = [Crack(kind="edge", orientation=1, pb=(cx - 0.5 * L, cy), pt=(cx + 0.5 * L, cy))]
    return Problem(dim=2, x=x, volume=vol, horizon=ratio * h, mesh_size=h, material=glass_rnp(),
                   ubc=ubc, cracks=cracks, dt=1.0, steps=100, name=name)


def config4(seed=0):
    """200 x 200 quasi-static plate, horizon 3h, centred 0.2 W pre-crack, 100
    load steps of 1e-6 m on the top edge, bottom edge fixed."""
    return qs_plate(200, name="qs_rnp2d_200x200_d3h")


def qs_training_geometry(seed, nx=200):
    """Seeded pre-crack length U[0.1, 0.3] W and centre U[0.35, 0.65]^2 W."""
    rng = np.random.default_rng(10_000 + seed)
    frac = float(rng.uniform(0.1, 0.3))
    c = (float(rng.uniform(0.35, 0.65)), float(rng.uniform(0.35, 0.65)))
    return qs_plate(nx, crack_frac=frac, crack_center=c, name="qs_seed%d" % seed)
