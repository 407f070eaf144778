"""Model descriptions mirroring the reference's input decks.

The reference reads a YAML file into deck structs (src/inp/input.cpp,
src/inp/decks/*.h).  Here a ``Problem`` holds the same fields as plain Python
values and numpy arrays, and ``Problem.desc()`` packs them into the C struct
``nlm_fd_desc`` of include/nlmgpu.h that both the CUDA library and the CPU
oracle take.
"""
from dataclasses import dataclass, field
from typing import List, Optional
import ctypes as C

import numpy as np

from . import abi


@dataclass
class BC:
    """One Displacement_BC / Force_BC set (inp::BCData, loadingDeck.h)."""
    region: str = "rectangle"
    x1: float = 0.0
    x2: float = 0.0
    y1: float = 0.0
    y2: float = 0.0
    z1: float = 0.0
    z2: float = 0.0
    r1: float = 0.0
    r2: float = 0.0
    direction: List[int] = field(default_factory=lambda: [1])  # 1-based, as in the deck
    time_fn: str = "constant"
    time_params: List[float] = field(default_factory=lambda: [0.0])
    spatial_fn: str = "constant"
    spatial_params: List[float] = field(default_factory=lambda: [1.0])
    theta: float = 0.0  # angled_rectangle: Location.Angle

    def to_c(self):
        s = abi.BCSet()
        s.region = abi.REGION[self.region]
        for k in ("x1", "x2", "y1", "y2", "z1", "z2", "r1", "r2", "theta"):
            setattr(s, k, float(getattr(self, k)))
        mask = 0
        for d in self.direction:
            if d not in (1, 2, 3):
                raise ValueError("direction must be 1, 2 or 3")
            mask |= 1 << (d - 1)
        s.dir_mask = mask
        s.time_fn = abi.TIME_FN[self.time_fn]
        for i, v in enumerate(self.time_params[:4]):
            s.time_params[i] = float(v)
        s.spatial_fn = abi.SPATIAL_FN[self.spatial_fn]
        for i, v in enumerate(self.spatial_params[:2]):
            s.spatial_params[i] = float(v)
        return s


@dataclass
class Crack:
    """A crack: inp::EdgeCrack (2-D) or a planar patch (3-D).
    activation_time < 0 (the default, as in fractureDeck.h:103): a pre-crack;
    >= 0: "Activation_Time", cut by the explicit model during the run."""
    kind: str = "edge"
    orientation: int = 1
    pb: tuple = (0.0, 0.0)
    pt: tuple = (0.0, 0.0)
    theta: float = 0.0
    z0: float = 0.0
    lo: tuple = (0.0, 0.0)
    hi: tuple = (0.0, 0.0)
    activation_time: float = -1.0

    def to_c(self):
        c = abi.Crack()
        c.kind = abi.CRACK_EDGE if self.kind == "edge" else abi.CRACK_PLANE
        c.orientation = int(self.orientation)
        c.pb[0], c.pb[1] = self.pb
        c.pt[0], c.pt[1] = self.pt
        c.theta = float(self.theta)
        c.z0 = float(self.z0)
        c.lo[0], c.lo[1] = self.lo
        c.hi[0], c.hi[1] = self.hi
        c.timed = int(self.activation_time >= 0.)
        c.activation_time = float(self.activation_time)
        return c


@dataclass
class MaterialDeck:
    """inp::MaterialDeck fields (materialDeck.h); -1 = not given."""
    kind: str = "RNPBond"
    density: float = 1.0
    E: float = -1.0
    G: float = -1.0
    K: float = -1.0
    Gc: float = -1.0
    KIc: float = -1.0
    plane_strain: bool = False
    influence_type: int = 0
    influence_params: List[float] = field(default_factory=list)
    irreversible: bool = True
    check_sc_factor: float = 1.0
    compute_from_classical: bool = True
    bond_params: List[float] = field(default_factory=lambda: [0.0, 0.0])
    es_sc: float = 0.0
    es_ref_compat: bool = False
    apply_contact: bool = False

    def to_c(self):
        m = abi.Material()
        m.kind = abi.RNP_BOND if self.kind in ("RNPBond", "PDBond") else abi.ELASTIC_STATE
        m.density = self.density
        m.E, m.G, m.K, m.Gc, m.KIc = self.E, self.G, self.K, self.Gc, self.KIc
        m.plane_strain = int(self.plane_strain)
        m.influence_type = self.influence_type
        m.n_influence_params = len(self.influence_params)
        for i, v in enumerate(self.influence_params[:2]):
            m.influence_params[i] = v
        m.irreversible = int(self.irreversible)
        m.check_sc_factor = self.check_sc_factor
        m.compute_from_classical = int(self.compute_from_classical)
        m.bond_params[0], m.bond_params[1] = self.bond_params[:2]
        m.es_sc = self.es_sc
        m.es_ref_compat = int(self.es_ref_compat)
        m.apply_contact = int(self.apply_contact)
        return m


@dataclass
class Problem:
    """Everything FDModel reads from its decks for one specimen."""
    dim: int
    x: np.ndarray            # (n, 3) float64 reference coordinates
    volume: np.ndarray       # (n,) float64
    horizon: float
    mesh_size: float
    material: MaterialDeck
    ubc: List[BC] = field(default_factory=list)
    fbc: List[BC] = field(default_factory=list)
    cracks: List[Crack] = field(default_factory=list)
    no_fail: int = abi.NOFAIL_OFF
    no_fail_tol: float = 0.0
    dt: float = 0.0
    steps: int = 0
    scheme: int = abi.VELOCITY_VERLET
    precision: int = abi.FP64
    decomposition: int = abi.DECOMP_AUTO
    u0: Optional[np.ndarray] = None
    v0: Optional[np.ndarray] = None
    name: str = ""
    # No_Fail_Region.Region_k: ("Circle", [cx, cy, cz, r]) or
    # ("Rectangle", [x1, y1, x2, y2]) (interiorFlags.cpp:76-90)
    nofail_regions: List[tuple] = field(default_factory=list)

    @property
    def n(self):
        return int(self.x.shape[0])

    def desc(self, precision=None, decomposition=None, scheme=None):
        """Return (nlm_fd_desc, keepalive) for this problem."""
        x = np.ascontiguousarray(self.x, dtype=np.float64).reshape(-1, 3)
        vol = np.ascontiguousarray(self.volume, dtype=np.float64)
        keep = [x, vol]
        d = abi.FDDesc()
        d.dim = self.dim
        d.n_nodes = x.shape[0]
        d.x = abi.dptr(x)
        d.volume = abi.dptr(vol)
        d.horizon = self.horizon
        d.mesh_size = self.mesh_size
        d.material = self.material.to_c()
        ub = (abi.BCSet * max(1, len(self.ubc)))(*[b.to_c() for b in self.ubc])
        fb = (abi.BCSet * max(1, len(self.fbc)))(*[b.to_c() for b in self.fbc])
        ck = (abi.Crack * max(1, len(self.cracks)))(*[c.to_c() for c in self.cracks])
        keep += [ub, fb, ck]
        d.n_ubc, d.ubc = len(self.ubc), ub
        d.n_fbc, d.fbc = len(self.fbc), fb
        d.n_cracks, d.cracks = len(self.cracks), ck
        d.no_fail = self.no_fail
        d.no_fail_tol = self.no_fail_tol
        if self.nofail_regions:
            regs = (abi.NoFailRegion * len(self.nofail_regions))()
            for k, (kind, prm) in enumerate(self.nofail_regions):
                if kind not in ("Circle", "Rectangle"):
                    raise ValueError("no-fail region type must be Circle or Rectangle")
                regs[k].kind = abi.NOFAIL_CIRCLE if kind == "Circle" else abi.NOFAIL_RECTANGLE
                for q, v in enumerate(list(prm)[:4]):
                    regs[k].params[q] = float(v)
            keep.append(regs)
            d.n_nofail_regions, d.nofail_regions = len(self.nofail_regions), regs
        d.dt = self.dt
        d.scheme = self.scheme if scheme is None else scheme
        d.precision = self.precision if precision is None else precision
        d.decomposition = self.decomposition if decomposition is None else decomposition
        for nm in ("u0", "v0"):
            a = getattr(self, nm)
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)
                keep.append(a)
                setattr(d, nm, abi.dptr(a))
        return d, keep
