"""The explicit model's output loop: FDModel::integrate's output schedule
(src/model/fd/fDModel.cpp:335-374), model::Output's VTU files
(src/model/util.cpp:4-191) and the output criteria of
FDModel::checkOutputCriteria (fDModel.cpp:780-915).

    deck = OutputDeck(path="out/", tags=["Displacement", "Damage_Z"], dt_out=100,
                      criteria="max_Z_stop", dt_out_criteria=10,
                      criteria_params=[0.9, 1.0, x0, y0, x1, y1])
    integrate(model, deck, nsteps=problem.steps)

The steps run on the GPU in chunks that end at the next step where output
or a criteria check can happen; post-processing (damage, energies, reaction
force) runs on the GPU only at output steps and only for the tags asked for.
"""
import math
import os
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import vtu


def _dlt(a, b):
    """util::compare::definitelyLessThan (src/util/compare.cpp)."""
    return (b - a) > max(abs(a), abs(b)) * 1e-5


def _dgt(a, b):
    """util::compare::definitelyGreaterThan (src/util/compare.cpp)."""
    return (a - b) > max(abs(a), abs(b)) * 1e-5


def _bbox(x):
    """fe::Mesh::computeBBox (mesh.cpp:311-324): both corners start at the
    origin and widen with definitelyLessThan."""
    lo, hi = [0., 0., 0.], [0., 0., 0.]
    for p in np.asarray(x, dtype=np.float64).reshape(-1, 3):
        for d in range(3):
            if _dlt(p[d], lo[d]):
                lo[d] = float(p[d])
            if _dlt(hi[d], p[d]):
                hi[d] = float(p[d])
    return lo, hi


@dataclass
class OutputDeck:
    """inp::OutputDeck (src/inp/decks/outputDeck.h) fields of the loop."""
    path: str = "./"                     # Output.Path
    tags: List[str] = field(default_factory=lambda: ["Displacement", "Velocity"])
    dt_out: int = 0                      # Output_Interval (0: no output)
    criteria: str = ""                   # Output_Criteria.Type: "", "max_Z", "max_Z_stop"
    dt_out_criteria: int = 0             # Output_Criteria.New_Interval (0: dt_out)
    criteria_params: List[float] = field(default_factory=list)  # Output_Criteria.Parameters
    post_processing: bool = True         # Policy: Enable_PostProcessing


class OutputCriteria:
    """FDModel::checkOutputCriteria (fDModel.cpp:780-915).  The reference
    keeps the two "changed" flags as function statics; here they belong to
    the object, one per run."""

    def __init__(self, deck):
        self.criteria = deck.criteria
        self.params = list(deck.criteria_params)
        self.path = deck.path
        self.dt_out = int(deck.dt_out)
        self.dt_out_old = int(deck.dt_out)
        self.dt_out_criteria = int(deck.dt_out_criteria or deck.dt_out)
        self.changed_to_small = False
        self.changed_back_to_large = False
        self.stop = False

    def _dump(self, title, n, mode):
        with open(os.path.join(self.path, "dt_out_change.info"), mode) as fh:
            fh.write("%s:\n  N: %d\n  dN: %d\n" % (title, n, n // self.dt_out_criteria))

    def check(self, n, Z, x):
        """One check at step n with the damage function Z of the last
        post-processing and the reference positions x."""
        if not self.criteria or self.dt_out_old == self.dt_out_criteria:
            return
        if n % self.dt_out_old != 0:
            return
        if self.criteria not in ("max_Z", "max_Z_stop"):
            return
        if self.criteria == "max_Z" and self.dt_out == self.dt_out_criteria:
            return
        changed_now = False
        if self.dt_out > self.dt_out_criteria and not self.changed_to_small:
            zmax = float(np.max(Z)) if len(Z) else 0.
            if _dgt(zmax, self.params[0]):
                self.dt_out = self.dt_out_criteria
                self._dump("Large_Dt_To_Small_Dt", n, "w")
                self.changed_to_small = True
                changed_now = True
        if (not changed_now and not self.changed_back_to_large and
                self.criteria == "max_Z_stop" and self.dt_out < self.dt_out_old):
            ps = self.params
            ref_z = ps[1]
            lo, hi = [0., 0., 0.], [0., 0., 0.]
            if len(ps) == 6:
                lo, hi = [ps[2], ps[3], 0.], [ps[4], ps[5], 0.]
            elif len(ps) == 8:
                lo, hi = ps[2:5], ps[5:8]
            x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
            Zd = np.asarray(Z, dtype=np.float64)
            found = False
            for i in np.nonzero(Zd > ref_z)[0]:  # candidates; the tests below decide
                p = x[i]
                # util::geometry::isPointInsideRectangle (utilGeom.cpp:52-58)
                inside = not (_dlt(p[0], lo[0] - 1.0e-12) or _dlt(p[1], lo[1] - 1.0e-12) or
                              _dgt(p[0], hi[0] + 1.0e-12) or _dgt(p[1], hi[1] + 1.0e-12))
                if inside and _dgt(float(Zd[i]), ref_z):
                    found = True
                    break
            if found:
                self.dt_out = self.dt_out_old
                self._dump("Small_Dt_To_Large_Dt", n, "a")
                self.changed_back_to_large = True
                self.stop = True


def _int_accumulate(values):
    """std::accumulate(begin, end, 0): the int initial value makes every
    partial sum an int (truncation toward zero)."""
    acc = 0
    for v in values:
        acc = int(math.trunc(acc + float(v)))
    return acc


def write_output(model, deck, n, dt_out_criteria, post=None):
    """model::Output (util.cpp:4-191) for step n: output_<n / New_Interval>.vtu
    in deck.path with the deck's tags, in the reference's order."""
    tags = set(deck.tags)
    x = np.asarray(model.problem.x, dtype=np.float64).reshape(-1, 3)
    vol = np.asarray(model.problem.volume, dtype=np.float64)
    u, v, f = model.state()
    t, _ = model.time()
    pd, fd = [], []
    if "Displacement" in tags:
        pd.append(("Displacement", u))
    if "Velocity" in tags:
        pd.append(("Velocity", v))
    if "Force" in tags:
        pd.append(("Force", f * vol[:, None]))
    fd.append(("TIME", t))
    if deck.post_processing:
        post = post if post is not None else post_process(model, deck)
        if "Force_Density" in tags:
            pd.append(("Force_Density", f))
        if "Reaction_Force" in tags and "reaction" in post:
            pd.append(("Reaction_Force", post["reaction"][0]))
        if "Total_Reaction_Force" in tags and "reaction" in post:
            lo, hi = _bbox(x)
            delta = model.problem.horizon
            area = (abs(hi[0] - lo[0]) - delta) * (abs(hi[1] - lo[1]) - delta)
            fd.append(("Total_Reaction_Force",
                       _int_accumulate(post["reaction"][1]) * area))
        e = post.get("energies")
        if "Strain_Energy" in tags and e is not None:
            pd.append(("Strain_Energy", e[0][0]))
        if "Work_Done" in tags and e is not None:
            pd.append(("Work_Done", e[0][1]))
        if "Fixity" in tags:
            pd.append(("Fixity", model.fixity()))
        if "Node_Volume" in tags:
            pd.append(("Node_Volume", vol))
        if "Damage_Phi" in tags:
            pd.append(("Damage_Phi", post["damage"][0]))
        if "Damage_Z" in tags:
            pd.append(("Damage_Z", post["damage"][1]))
        if e is not None:
            if "Fracture_Perienergy_Bond" in tags:
                pd.append(("Fracture_Perienergy_Bond", e[0][3]))
            if "Fracture_Perienergy_Total" in tags:
                pd.append(("Fracture_Perienergy_Total", e[0][3]))
            tot = e[1]
            if "Total_Energy" in tags:
                fd.append(("Total_Energy", tot[0] - tot[1] + tot[2]))
            if "Total_Fracture_Perienergy_Bond" in tags:
                fd.append(("Total_Fracture_Perienergy_Bond", tot[3]))
            if "Total_Fracture_Perienergy_Total" in tags:
                fd.append(("Total_Fracture_Perienergy_Total", tot[3]))
        if "Neighbors" in tags:
            rowptr, _ = model.neighbors()
            pd.append(("Neighbors", np.diff(rowptr).astype(np.uint64)))
    name = os.path.join(deck.path, "output_%d.vtu" % (n // dt_out_criteria))
    vtu.write_points(name, x + u, pd, fd)
    return name


_ENERGY_TAGS = {"Strain_Energy", "Work_Done", "Fracture_Perienergy_Bond",
                "Fracture_Perienergy_Total", "Total_Energy", "Total_Fracture_Perienergy_Bond",
                "Total_Fracture_Perienergy_Total"}


def post_process(model, deck):
    """FDModel::computePostProcFields (fDModel.cpp:651-778) on the GPU, for
    the fields the deck's tags and criteria read."""
    tags = set(deck.tags)
    out = {"damage": model.damage()}  # Z feeds the output criteria as well
    if tags & _ENERGY_TAGS:
        out["energies"] = model.energies()
    if tags & {"Reaction_Force", "Total_Reaction_Force"}:
        out["reaction"] = model.reaction_force()
    return out


def integrate(model, deck, nsteps, on_output=None):
    """FDModel::integrate's loop (fDModel.cpp:335-374) for nsteps more steps:
    output every dt_out steps (from step dt_out on), stop when max_Z_stop
    fires, the output criteria checked after each output and after a step
    whose end cuts a timed crack.  Returns (steps run, files written)."""
    crit = OutputCriteria(deck)
    if deck.dt_out <= 0:
        model.run(nsteps)
        return nsteps, []
    os.makedirs(deck.path, exist_ok=True)
    t0, n0 = model.time()
    files = []
    Z = np.zeros(model.n, dtype=np.float32)
    if n0 == 0:
        # the output at the beginning (fDModel.cpp:335-339): loads and forces
        # at t = 0, then output_0
        model.run(0)
        post = post_process(model, deck) if deck.post_processing else None
        if post is not None:
            Z = post["damage"][1]
        files.append(write_output(model, deck, 0, crit.dt_out_criteria, post))
        if on_output is not None:
            on_output(0, files[-1])
    pending = [c for c in model.problem.cracks if c.activation_time >= 0]
    t = t0
    n = n0
    n_end = n0 + nsteps
    x = model.problem.x
    while n < n_end:
        # next step at which output or a check may act (a crack's check is
        # only effective at multiples of the old interval)
        nxt = n + 1
        while nxt < n_end and nxt % crit.dt_out != 0 and nxt % crit.dt_out_old != 0:
            nxt += 1
        # the reference accumulates the time step by step
        k0 = n
        cut_at = []
        while k0 < nxt:
            k0 += 1
            t = t + model.problem.dt
            for c in pending:
                if _dlt(c.activation_time, t):
                    pending.remove(c)
                    cut_at.append(k0)
                    break
        model.run(nxt - n)
        n = nxt
        if n % crit.dt_out == 0 and n >= crit.dt_out:
            post = post_process(model, deck) if deck.post_processing else None
            if post is not None:
                Z = post["damage"][1]
            files.append(write_output(model, deck, n, crit.dt_out_criteria, post))
            if on_output is not None:
                on_output(n, files[-1])
            if crit.stop:
                return n - n0, files
            crit.check(n, Z, x)
        if n in cut_at:
            crit.check(n, Z, x)
    return n - n0, files
