"""Learned warm start of the quasi-static Newton load steps.

A per-node MLP (10 -> 128 x 3 -> 2, ReLU; BF16 GEMMs accumulating in FP32 on
the tensor cores, nlm_mlp_*) predicts the displacement increment of load
step k from local features.  The start handed to nlm_qs_load_step is

    u_guess = u_{k-1} + du_{k-1} + s * y

where du_{k-1} = u_{k-1} - u_{k-2} is the last increment, s the magnitude of
the prescribed boundary increment per step and y the network output, so the
network learns how the increment changes from one step to the next.
nlm_qs_load_step judges the start by the linear model of the residual at
the previous converged state and keeps it if it cuts the linearised
residual of the plain start (the previous displacement with the new
boundary values, QuasiStaticModel::solver, QuasiStaticModel.cpp:280-312) at
least tenfold; otherwise it starts from the plain start.  Newton then runs
to the same tolerance either way.

Features per node (float32, in this order):
  0, 1  reference position (x - x_min) / W, (y - y_min) / W
  2, 3  du_{k-1} / s
  4, 5  (du_{k-1} - du_{k-2}) / s
  6     damage of the node at u_{k-1}
  7     prescribed increment of the node this step / s (largest component)
  8     1 if a displacement component of the node is prescribed, else 0
  9     k / K  (load fraction)
Target: (du_k - du_{k-1}) / s, two components.

Training data are the load steps of the plain solver itself over seeded
pre-crack geometries (configs.qs_training_geometry).  Command line:

  python -m nlmech_gb300.warmstart train  [--seeds 20] [--steps 100] [--out F]
  python -m nlmech_gb300.warmstart eval   [--weights F] [--seeds 100 101]
"""
import argparse
import json
import os
import time

import numpy as np

from . import configs, gpu

N_FEAT = 10
N_OUT = 2
HIDDEN = 128
LAYERS = 3
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart_mlp.npz")
TARGET_CLIP = 5.0    # targets (units of s) beyond this are clipped for training
FEATURE_CLIP = 8.0   # increment features (units of s) are clipped to +-8
DETACHED = 0.999     # nodes with damage above this keep the plain start
DEADZONE = 0.5       # network outputs below this (units of s) count as zero
# Newton-Krylov forcing term of the evaluation runs (both arms): an iteration
# whose residual is already near the target solves its linear system to
# min(0.1, 0.1 target / ||r||) instead of 1e-4, so a good start is not paid
# back with a linear solve more accurate than the step needs
LIN_TOL_GAMMA = 0.1


def _rect_mask(x, b):
    if b.region != "rectangle":
        raise ValueError("warm-start features support rectangle displacement regions")
    return ((x[:, 0] >= b.x1) & (x[:, 0] <= b.x2) & (x[:, 1] >= b.y1) & (x[:, 1] <= b.y2))


def _rate(b):
    if b.time_fn == "constant":
        return 0.0
    if b.time_fn == "linear":
        return float(b.time_params[0]) * float(b.spatial_params[0] if b.spatial_fn == "constant" else 1.0)
    raise ValueError("warm-start features support constant and linear displacement loads")


class Features:
    """Per-node feature rows of one specimen (2-D quasi-static plate)."""

    def __init__(self, problem, nsteps):
        if problem.dim != 2:
            raise ValueError("the warm start is for 2-D specimens")
        x = problem.x
        lo = x[:, :2].min(axis=0)
        span = max(float((x[:, :2].max(axis=0) - lo).max()), problem.mesh_size)
        self.n = problem.n
        self.K = max(int(nsteps), 1)
        self.pos = ((x[:, :2] - lo) / span).astype(np.float32)
        inc = np.zeros(self.n)
        fixed = np.zeros(self.n, dtype=bool)
        for b in problem.ubc:
            m = _rect_mask(x, b)
            fixed |= m
            inc[m] = np.maximum(inc[m], abs(_rate(b)) * problem.dt)
        self.s = float(inc.max()) if inc.max() > 0 else problem.mesh_size * 1e-3
        self.inc = (inc / self.s).astype(np.float32)
        self.fixed = fixed.astype(np.float32)

    def rows(self, k, d1, d2, phi):
        F = np.empty((self.n, N_FEAT), dtype=np.float32)
        F[:, 0:2] = self.pos
        F[:, 2:4] = np.clip(d1 / self.s, -FEATURE_CLIP, FEATURE_CLIP)
        F[:, 4:6] = np.clip((d1 - d2) / self.s, -FEATURE_CLIP, FEATURE_CLIP)
        F[:, 6] = phi
        F[:, 7] = self.inc
        F[:, 8] = self.fixed
        F[:, 9] = k / self.K
        return F

    def target(self, d, d1):
        return np.clip((d - d1) / self.s, -TARGET_CLIP, TARGET_CLIP).astype(np.float32)

    def guess(self, u_prev, d1, y, phi, deadzone=DEADZONE):
        """Start displacement (n, 3) from the network output y (n, 2) (None:
        the increment is repeated unchanged).  Outputs inside the dead zone
        are taken as zero: where the last increment already predicts the
        next one to Newton accuracy (steady loading) a small network error
        would otherwise cost a Newton iteration.  Nodes that have lost
        (almost) all their bonds keep their previous position."""
        g = np.zeros((self.n, 3))
        g[:, :2] = u_prev + d1
        if y is not None:
            y = np.clip(y, -TARGET_CLIP, TARGET_CLIP)
            y = np.where(np.abs(y) < deadzone, 0.0, y)
            g[:, :2] += self.s * y
        det = phi > DETACHED
        g[det, :2] = u_prev[det]
        return g


def run_steps(problem, nsteps, params=None, model=None, record=False, log=None,
              secant=False, deadzone=DEADZONE, start="network"):
    """Run nsteps load steps: plain (no model), with the learned start
    (model; start="network": the network's start, "best": the better of the
    network's start and the repeated last increment by the linearised
    residual), or with the last increment repeated (secant=True, the
    ablation of the learned start without its network).

    Returns a dict of per-step statistics, wall time, the final state and,
    with record=True, the (features, targets) rows of every step."""
    q = gpu.QSModel(problem, params or gpu.qs_params())
    fb = Features(problem, nsteps)
    n = problem.n
    u_prev = np.zeros((n, 2))
    d1 = np.zeros((n, 2))
    d2 = np.zeros((n, 2))
    phi = np.zeros(n, dtype=np.float32)
    stats, X, T = [], [], []
    mlp_s = 0.0  # wall time of the network's inference calls (host in, host out)

    def infer(F):
        nonlocal mlp_s
        t = time.perf_counter()
        y = model.forward(F)
        mlp_s += time.perf_counter() - t
        return y

    t0 = time.perf_counter()
    for k in range(nsteps):
        hist = model is not None or record or secant
        F = fb.rows(k, d1, d2, phi) if (model is not None or record) else None
        if model is not None and start == "best":
            st = q.load_step(candidates=[fb.guess(u_prev, d1, None, phi),
                                         fb.guess(u_prev, d1, infer(F), phi, deadzone)])
        elif model is not None:
            st = q.load_step(fb.guess(u_prev, d1, infer(F), phi, deadzone))
        elif secant:
            st = q.load_step(fb.guess(u_prev, d1, None, phi))
        else:
            st = q.load_step()
        if hist:
            # history for the next step's features (the plain run needs none)
            u = q.state()[:, :2]
            d = u - u_prev
            if record:
                keep = phi <= DETACHED  # detached nodes carry no information
                X.append(F[keep])
                T.append(fb.target(d, d1)[keep])
            d2, d1, u_prev = d1, d, u
            phi = q.damage()[0]
        stats.append(st)
        if log:
            log("step %3d newton %3d cg %6d guess %d broken %6d res %.3g -> %.3g  %.1f ms" % (
                k, st["newton_iters"], st["lin_iters"], st["used_guess"], st["broken"],
                st["res_start"], st["res_final"], st["ms"]))
    wall = time.perf_counter() - t0
    out = {"stats": stats, "wall_s": wall, "mlp_s": mlp_s, "u": q.state(),
           "bonds": q.bond_state()}
    if record:
        out["X"] = np.concatenate(X)
        out["T"] = np.concatenate(T)
    q.close()
    return out


def summary(run):
    st = run["stats"]
    tol_ok = all(s["res_final"] <= 1e-8 * s["res_plain"] for s in st)
    return {"newton_iters": int(sum(s["newton_iters"] for s in st)),
            "cg_iters": int(sum(s["lin_iters"] for s in st)),
            "guess_used": int(sum(1 for s in st if s["used_guess"])),

            "wall_s": round(run["wall_s"], 4),
            "mlp_infer_s": round(run.get("mlp_s", 0.0), 4),
            "solver_ms": round(sum(s["ms"] for s in st), 2),
            "all_steps_converged": bool(tol_ok)}


def load_model(path=WEIGHTS):
    z = np.load(path)
    shape = tuple(int(v) for v in z["shape"])
    m = gpu.MLP(*shape)
    m.set_params(z["params"])
    return m


def train(seeds, nsteps, out, epochs=8, batch=8192, lr=3e-4, max_newton=500, log=print):
    params = gpu.qs_params(max_newton=max_newton)
    X, T = [], []
    t0 = time.perf_counter()
    for sd in seeds:
        r = run_steps(configs.qs_training_geometry(sd), nsteps, params, record=True)
        X.append(r["X"])
        T.append(r["T"])
        log("seed %d: %s" % (sd, json.dumps(summary(r))))
    X = np.concatenate(X)
    T = np.concatenate(T)
    gen_s = time.perf_counter() - t0
    log("data: %d rows from %d load steps in %.1f s" % (X.shape[0], len(seeds) * nsteps, gen_s))
    m = gpu.MLP(N_FEAT, HIDDEN, LAYERS, N_OUT, seed=1234)
    m.set_data(X, T)
    t1 = time.perf_counter()
    losses = []
    for e in range(epochs):
        lr_e = lr * 0.5 * (1 + np.cos(np.pi * e / epochs))
        losses += list(m.train(1, batch=batch, lr=float(lr_e), seed=e))
        log("epoch %d lr %.2e loss %.4g" % (e, lr_e, losses[-1]))
    train_s = time.perf_counter() - t1
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.savez(out, params=m.params(), shape=np.array([N_FEAT, HIDDEN, LAYERS, N_OUT]),
             seeds=np.array(seeds), steps=nsteps, losses=np.array(losses, dtype=np.float32),
             rows=X.shape[0], gen_s=gen_s, train_s=train_s)
    log("trained %d epochs in %.1f s -> %s" % (epochs, train_s, out))
    return m


def evaluate(model, problems, nsteps, max_newton=500, log=print, deadzone=DEADZONE,
             ablation=True, lin_tol_gamma=LIN_TOL_GAMMA):
    """Plain vs learned start (and, with ablation, the secant start without
    the network) on each problem, every load step to the same tolerance and
    with the same Newton-Krylov settings in every arm."""
    params = gpu.qs_params(max_newton=max_newton, lin_tol_gamma=lin_tol_gamma)
    res = {}
    for p in problems:
        a = run_steps(p, nsteps, params)
        b = run_steps(p, nsteps, params, model=model, deadzone=deadzone)
        sa, sb = summary(a), summary(b)
        du = np.linalg.norm(b["u"] - a["u"]) / max(np.linalg.norm(a["u"]), 1e-300)
        diff = int(np.count_nonzero((a["bonds"] != 0) != (b["bonds"] != 0)))
        res[p.name] = {"plain": sa, "learned": sb,
                       "speedup_wall": round(sa["wall_s"] / sb["wall_s"], 3),
                       "newton_ratio": round(sa["newton_iters"] / max(sb["newton_iters"], 1), 3),
                       "u_rel_l2_vs_plain": float(du), "broken_bonds_differing": diff,
                       "broken_bonds_plain": int(np.count_nonzero(a["bonds"]))}
        if ablation:
            for key, kw in (("secant_only", dict(secant=True)),
                            ("best_of_two", dict(model=model, deadzone=deadzone, start="best"))):
                c = run_steps(p, nsteps, params, **kw)
                sc = summary(c)
                sc["speedup_wall"] = round(sa["wall_s"] / c["wall_s"], 3)
                sc["u_rel_l2_vs_plain"] = float(np.linalg.norm(c["u"] - a["u"]) /
                                                max(np.linalg.norm(a["u"]), 1e-300))
                sc["broken_bonds_differing"] = int(np.count_nonzero((a["bonds"] != 0) !=
                                                                    (c["bonds"] != 0)))
                res[p.name][key] = sc
        log("%s: %s" % (p.name, json.dumps(res[p.name])))
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("mode", choices=["train", "eval"])
    ap.add_argument("--seeds", type=int, nargs="*", default=None)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--nx", type=int, default=200)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--deadzone", type=float, nargs="*", default=[DEADZONE])
    a = ap.parse_args(argv)
    if a.mode == "train":
        seeds = a.seeds if a.seeds else list(range(20))
        train(seeds, a.steps, a.out, epochs=a.epochs)
    else:
        seeds = a.seeds if a.seeds else [100, 101]
        m = load_model(a.weights)
        probs = [configs.config4()] + [configs.qs_training_geometry(s, a.nx) for s in seeds]
        for k, dz in enumerate(a.deadzone):
            print("deadzone", dz)
            print(json.dumps(evaluate(m, probs, a.steps, deadzone=dz, ablation=k == 0), indent=1))


if __name__ == "__main__":
    main()
