"""The reference's input decks (YAML files read by inp::Input,
src/inp/input.cpp) turned into a Problem, an OutputDeck and the solver
settings, so a deck written for NLMech runs here unchanged:

    deck = read_deck("examples/fdModel/crack_propagation/input.yaml")
    model = gpu.FDModel(deck.problem)
    output.integrate(model, deck.output, deck.problem.steps)

or from the command line, ``python -m nlmech_gb300.run -i input.yaml``.

``parse_yaml`` reads the part of YAML the decks use: nested block mappings,
block sequences ("- item"), flow sequences ("[a, b]"), scalars and comments.
A key given twice in one mapping keeps its first value, which is the one
yaml-cpp's node lookup returns.
"""
import math
import os
import re
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi, meshfile
from .decks import BC, Crack, MaterialDeck, Problem
from .output import OutputDeck


class DeckError(ValueError):
    """A deck the reference would refuse (it prints the message and exits)."""


# ---------------------------------------------------------------------------
# YAML subset

def _scalar(tok):
    t = tok.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if low in ("~", "null", ""):
        return None
    if re.fullmatch(r"[-+]?\d+", t):
        return int(t)
    try:
        return float(t)
    except ValueError:
        return t


def _value(text):
    t = text.strip()
    if t.startswith("["):
        if not t.endswith("]"):
            raise DeckError("unterminated flow sequence: " + t)
        body = t[1:-1].strip()
        return [] if not body else [_scalar(v) for v in body.split(",")]
    return _scalar(t)


def _strip_comment(line):
    out, quote = [], None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def parse_yaml(text):
    lines = []
    for raw in text.splitlines():
        ln = _strip_comment(raw.replace("\t", "    "))
        if ln.strip():
            lines.append((len(ln) - len(ln.lstrip(" ")), ln.strip()))
    pos = [0]

    def block(indent):
        if pos[0] >= len(lines):
            return None
        ind, txt = lines[pos[0]]
        if txt.startswith("- ") or txt == "-":
            return seq(ind)
        return mapping(ind)

    def seq(ind):
        out = []
        while pos[0] < len(lines):
            i, txt = lines[pos[0]]
            if i != ind or not (txt.startswith("- ") or txt == "-"):
                break
            item = txt[1:].strip()
            pos[0] += 1
            if not item:
                out.append(block(ind + 1))
            elif re.match(r"^[^\[\]'\"]+?:(\s|$)", item):
                # "- key: value": a mapping item whose keys line up after "- "
                lines.insert(pos[0], (ind + 2, item))
                out.append(mapping(ind + 2))
            else:
                out.append(_value(item))
        return out

    def mapping(ind):
        out = {}
        while pos[0] < len(lines):
            i, txt = lines[pos[0]]
            if i < ind:
                break
            if i > ind:
                raise DeckError("bad indentation near: " + txt)
            m = re.match(r"^([^:]+?)\s*:(?:\s+(.*)|)$", txt)
            if not m:
                raise DeckError("expected 'key: value' near: " + txt)
            key, rest = m.group(1).strip(), (m.group(2) or "").strip()
            pos[0] += 1
            if rest:
                val = _value(rest)
            elif pos[0] < len(lines) and (lines[pos[0]][0] > ind or (
                    lines[pos[0]][0] == ind and lines[pos[0]][1].startswith("-"))):
                val = block(lines[pos[0]][0])
            else:
                val = None
            if key not in out:
                out[key] = val
        return out

    return block(0) or {}


# ---------------------------------------------------------------------------
# inp::Input

@dataclass
class InputDeck:
    problem: Problem
    output: OutputDeck
    time_scheme: str                    # Model.Discretization_Type.Time
    spatial: str                        # Model.Discretization_Type.Spatial
    final_time: float
    time_steps: int
    solver: dict = field(default_factory=dict)   # Solver block
    restart: Optional[dict] = None               # Restart block (File, Step)
    post_processing: bool = True
    path: str = ""

    @property
    def quasi_static(self):
        return self.time_scheme == "quasi_static"


def _get(d, *keys):
    for k in keys:
        if not isinstance(d, dict) or k not in d:
            return None
        d = d[k]
    return d


def _floats(v, what, n=None):
    if v is None:
        return []
    vals = [float(x) for x in (v if isinstance(v, list) else [v])]
    if n is not None and len(vals) != n:
        raise DeckError("Error: Check %s data." % what)
    return vals


def _bc_sets(cfg, tag):
    """inp::Input::setLoadingDeck (input.cpp:418-560)."""
    out = []
    blk = cfg.get(tag)
    if not blk:
        return out
    for s in range(1, int(blk.get("Sets", 0)) + 1):
        e = blk.get("Set_%d" % s) or {}
        loc = e.get("Location") or {}
        bc = BC()
        if "Line" in loc:
            x = _floats(loc["Line"], "Line data in " + tag, 2)
            bc.region, bc.x1, bc.x2 = "line", x[0], x[1]
        elif "Rectangle" in loc:
            x = _floats(loc["Rectangle"], "Rectangle data in " + tag, 4)
            bc.region, bc.x1, bc.y1, bc.x2, bc.y2 = "rectangle", x[0], x[1], x[2], x[3]
        elif "Angled_Rectangle" in loc:
            x = _floats(loc["Angled_Rectangle"], "Rectangle data in " + tag, 4)
            bc.region, bc.x1, bc.y1, bc.x2, bc.y2 = "angled_rectangle", x[0], x[1], x[2], x[3]
            bc.theta = float(loc.get("Angle"))
            alpha = math.atan((bc.y2 - bc.y1) / (bc.x2 - bc.x1))
            if _dgt(0.0, alpha):
                alpha = alpha + math.pi
            if _dgt(bc.theta, alpha) or abs(alpha - bc.theta) <= 1.0e-5:
                raise DeckError("Error: Check angled rectangle. Either angle of diagonal is "
                                "smaller than theta or it is very close to theta")
        elif "Point" in loc and "Radius" in loc:
            x = _floats(loc["Point"], "Point data in " + tag, 2)
            r = _floats(loc["Radius"], "Radii data in " + tag, 1)
            bc.region, bc.x1, bc.y1, bc.r1 = "circle", x[0], x[1], r[0]
        elif "Point" in loc and "Radii" in loc:
            x = _floats(loc["Point"], "Point data in " + tag, 2)
            r = _floats(loc["Radii"], "Radii data in " + tag, 2)
            bc.region, bc.x1, bc.y1, bc.r1, bc.r2 = "torus", x[0], x[1], r[0], r[1]
        elif "Cuboid" in loc:
            x = _floats(loc["Cuboid"], "Cuboid data in " + tag, 6)
            bc.region = "cuboid"
            bc.x1, bc.y1, bc.z1, bc.x2, bc.y2, bc.z2 = x
        elif "Displacement_from_pum" in loc:
            raise DeckError("Displacement_from_pum (PUM coupling) is not part of this library")
        else:
            raise DeckError("Error: no Location in %s Set_%d" % (tag, s))
        bc.direction = [int(d) for d in (e.get("Direction") or [])]
        tf = e.get("Time_Function") or {}
        bc.time_fn = str(tf.get("Type", "constant"))
        bc.time_params = _floats(tf.get("Parameters"), "time parameters") or [0.0]
        sf = e.get("Spatial_Function") or {}
        bc.spatial_fn = str(sf.get("Type", "constant"))
        bc.spatial_params = _floats(sf.get("Parameters"), "spatial parameters") or [1.0]
        for name, table in ((bc.time_fn, abi.TIME_FN), (bc.spatial_fn, abi.SPATIAL_FN)):
            if name not in table:
                raise DeckError("Error: %s function type = %s not recognised" % (tag, name))
        out.append(bc)
    return out


def _dgt(a, b):
    return (a - b) > max(abs(a), abs(b)) * 1e-5


def _material(cfg, dim):
    """inp::Input::setMaterialDeck (input.cpp:562-670)."""
    e = cfg.get("Material") or {}
    if "Type" not in e:
        raise DeckError("Error: Please specify the material type.")
    kind = str(e["Type"])
    if kind == "PDBond":
        kind = "RNPBond"
    if kind not in ("RNPBond", "ElasticState"):
        raise DeckError("material type %s: the library has RNPBond and ElasticState" % kind)
    if "Density" not in e:
        raise DeckError("Error: Please specify the density of the material.")
    for k in ("Lambda", "Mu", "Poisson_Ratio"):
        if k in e:
            raise DeckError("Material.%s: give E/G/K instead" % k)
    m = MaterialDeck(kind=kind, density=float(e["Density"]))
    m.plane_strain = bool(e.get("Is_Plane_Strain", False))
    m.compute_from_classical = bool(e.get("Compute_From_Classical", True))
    for k in ("E", "G", "K", "Gc", "KIc"):
        if k in e:
            setattr(m, k, float(e[k]))
    bp = e.get("Bond_Potential") or {}
    if "Check_Sc_Factor" in bp:
        m.check_sc_factor = float(bp["Check_Sc_Factor"])
    if "Irreversible_Bond_Fracture" in bp:
        m.irreversible = bool(bp["Irreversible_Bond_Fracture"])
    if "Parameters" in bp:
        m.bond_params = (_floats(bp["Parameters"], "Bond_Potential.Parameters") + [0.0, 0.0])[:2]
    inf = e.get("Influence_Function") or {}
    if "Type" in inf:
        m.influence_type = int(inf["Type"])
    if "Parameters" in inf:
        m.influence_params = _floats(inf["Parameters"], "Influence_Function.Parameters")
    if "No_Penetration" in e:
        m.apply_contact = bool(e["No_Penetration"])
    return m


def _cracks(cfg, dim):
    """inp::Input::setFractureDeck (input.cpp:282-353)."""
    blk = _get(cfg, "Fracture", "Cracks") or {}
    n = int(blk.get("Sets", 0) or 0)
    if n and dim != 2:
        raise DeckError("Error: Pre-cracks can only be prescribed for material in dimension 2.")
    out = []
    for s in range(1, n + 1):
        e = blk.get("Set_%d" % s) or {}
        c = Crack(kind="edge", orientation=int(e.get("Orientation", 1)))
        if "Line" not in e:
            raise DeckError("Error: Need Line data for complete specification of pre-crack.")
        x = _floats(e["Line"], "Line (crack)", 4)
        c.pb, c.pt = (x[0], x[1]), (x[2], x[3])
        if c.orientation == 0:
            if "Angle" not in e:
                raise DeckError("Error: Need Angle data for crack with arbitrary orientation.")
            c.theta = float(e["Angle"])
        if "Activation_Time" in e:
            c.activation_time = float(e["Activation_Time"])
        out.append(c)
    return out


def _ic(cfg, x, dim):
    """InitialCondition (initialCondition.cpp:20-82): Gaussian and double
    Gaussian profiles in 2-D (util::function::gaussian2d / doubleGaussian2d,
    utilFunction.cpp:66-102)."""
    out = []
    for key in ("Displacement", "Velocity"):
        e = _get(cfg, "Initial_Condition", key)
        if not e:
            out.append(None)
            continue
        if "File" in e:
            raise DeckError("Initial_Condition.%s.File: give the state through u0/v0" % key)
        typ = str(e.get("Type", ""))
        p = _floats(e.get("Parameters"), "Initial_Condition parameters")
        if dim != 2 or typ not in ("gaussian", "double_gaussian"):
            raise DeckError("Error: Check initial condition flag = %s. Currently only guassian "
                            "and double_guassian type functions are supported in 2-d." % typ)

        def g(cx, cy, amp, beta):
            d0, d1, d2 = x[:, 0] - cx, x[:, 1] - cy, x[:, 2] - 0.
            r = np.sqrt(d0 * d0 + d1 * d1 + d2 * d2)
            return amp * np.exp(-(r * r) / beta)

        a = np.zeros((x.shape[0], 3))
        for d in range(dim):
            if typ == "gaussian":
                if len(p) < 6:
                    raise DeckError("Error: Not enough parameters to compute guassian 2-d function.")
                a[:, d] = g(p[0], p[1], p[5], p[4]) * p[2 + d]
            else:
                if len(p) < 10:
                    raise DeckError("Error: Not enough parameters to compute guassian 2-d function.")
                a[:, d] = g(p[0], p[1], p[9], p[8]) * p[4 + d] + g(p[2], p[3], p[9], p[8]) * p[6 + d]
        out.append(a)
    return out


def read_deck(path, mesh=None):
    """inp::Input (input.cpp:23-60) for the models this library runs.  The
    mesh file is read relative to the deck's folder unless ``mesh`` (a
    meshfile.Mesh) is given."""
    with open(path) as fh:
        cfg = parse_yaml(fh.read())
    base = os.path.dirname(os.path.abspath(path))
    model = cfg.get("Model") or {}
    if "Dimension" not in model:
        raise DeckError("Error: Please specify the dimension.")
    dim = int(model["Dimension"])
    scheme = str(_get(model, "Discretization_Type", "Time") or "")
    spatial = str(_get(model, "Discretization_Type", "Spatial") or "")
    horizon = model.get("Horizon")
    ratio = model.get("Horizon_h_Ratio")
    h = model.get("Mesh_Size")
    if horizon is None:
        if ratio is None or h is None:
            raise DeckError("Error: Horizon is not provided. In this case Horizon_h_Ratio and "
                            "Mesh_Size are necessary to compute horizon.")
        horizon = float(h) * float(int(ratio))
    horizon = float(horizon)
    if h is None and ratio is not None:
        h = horizon / float(int(ratio))
    t_final = float(model.get("Final_Time", 0.0) or 0.0)
    nt = int(model.get("Time_Steps", 0) or 0)
    if abs(t_final) < 1.0e-10 or nt <= 0:
        raise DeckError("Error: Check Final_Time and Time_Steps data.")
    dt = t_final / nt
    if spatial != "finite_difference":
        raise DeckError("spatial discretisation %r: the library runs finite_difference models"
                        % spatial)
    if scheme not in ("velocity_verlet", "central_difference", "quasi_static"):
        raise DeckError("time discretisation %r is not known" % scheme)

    mblk = cfg.get("Mesh") or {}
    if mesh is None:
        if "File" not in mblk:
            raise DeckError("Error: Please specify mesh filename.")
        mesh = meshfile.read_mesh(os.path.join(base, str(mblk["File"])), dim,
                                  centroid_based=bool(mblk.get("Is_Centroid_Based_Discretization",
                                                               False)))
    if h is None or float(h) < 1.0e-12:
        h = meshfile.mesh_size(mesh.nodes)
    h = float(h)
    vol = np.asarray(mesh.volumes, dtype=np.float64)
    small = np.nonzero(vol < 0.01 * h ** dim)[0]
    if len(small):
        i = int(small[0])
        raise DeckError("Error: Check nodal volume %g is less than %g, Node = %d"
                        % (vol[i], 0.01 * h ** dim, i))

    x = np.asarray(mesh.nodes, dtype=np.float64).reshape(-1, 3)
    material = _material(cfg, dim)
    prob = Problem(dim=dim, x=x, volume=vol, horizon=horizon, mesh_size=h, material=material,
                   ubc=_bc_sets(cfg, "Displacement_BC"), fbc=_bc_sets(cfg, "Force_BC"),
                   cracks=_cracks(cfg, dim), dt=dt, steps=nt,
                   scheme=abi.CENTRAL_DIFFERENCE if scheme == "central_difference"
                   else abi.VELOCITY_VERLET, name=os.path.basename(path))
    nf = cfg.get("No_Fail_Region")
    if nf:
        prob.no_fail_tol = horizon * float(nf.get("Factor"))
        prob.no_fail = (abi.NOFAIL_COMPUTE if bool(nf.get("Compute_And_Not_Store", False))
                        else abi.NOFAIL_DATA)
        for r in range(1, int(nf.get("Num_Regions", 0) or 0) + 1):
            reg = nf.get("Region_%d" % r) or {}
            if "Type" not in reg:
                raise DeckError("Error: Region type must be provided for no-fail region")
            prob.nofail_regions.append((str(reg["Type"]), _floats(reg.get("Parameters"),
                                                                  "no-fail region")))
    prob.u0, prob.v0 = _ic(cfg, x, dim)

    oblk = cfg.get("Output") or {}
    crit = oblk.get("Output_Criteria") or {}
    dt_out = int(oblk.get("Output_Interval", 0) or 0)
    out = OutputDeck(path=os.path.join(base, str(oblk.get("Path", "./"))),
                     tags=[str(t) for t in (oblk.get("Tags") or [])], dt_out=dt_out,
                     criteria=str(crit.get("Type", "") or ""),
                     dt_out_criteria=int(crit.get("New_Interval", dt_out) or dt_out),
                     criteria_params=_floats(crit.get("Parameters"), "Output_Criteria"),
                     post_processing=bool(_get(cfg, "Policy", "Enable_PostProcessing")
                                          if _get(cfg, "Policy", "Enable_PostProcessing")
                                          is not None else True))
    if str(oblk.get("File_Format", "vtu")) != "vtu":
        raise DeckError("Output.File_Format: the library writes vtu")
    solver = cfg.get("Solver") or {}
    restart = None
    if cfg.get("Restart"):
        rb = cfg["Restart"]
        if "File" not in rb:
            raise DeckError("Error: Please specify the file for restart.")
        if "Step" not in rb:
            raise DeckError("Error: Please specify the time step from which to restart the "
                            "simulation.")
        restart = {"file": os.path.join(base, str(rb["File"])), "step": int(rb["Step"])}
    return InputDeck(problem=prob, output=out, time_scheme=scheme, spatial=spatial,
                     final_time=t_final, time_steps=nt, solver=solver, restart=restart,
                     post_processing=out.post_processing, path=os.path.abspath(path))
