"""Run a deck of the reference on the GPU, the way its executable does
(src/main.cpp:40-90): a finite-difference deck with velocity_verlet or
central_difference time stepping runs FDModel<RNPBond> (here also
ElasticState), a quasi_static deck runs QuasiStaticModel<ElasticState>.

    python -m nlmech_gb300.run -i input.yaml [--precision fp32c] [--graph 8]

Output files go where the deck's Output.Path says, relative to the deck.
"""
import argparse
import json
import os
import time

import numpy as np

from . import abi, deckfile, gpu, output, vtu


def _restart_state(model, deck):
    """FDModel::restart (fDModel.cpp:102-131): u and v from the restart file,
    d_n = Restart.Step, d_time = d_n dt."""
    d = vtu.read_vtu(deck.restart["file"])
    u = np.asarray(d["Displacement"], dtype=np.float64).reshape(-1, 3)
    v = np.asarray(d["Velocity"], dtype=np.float64).reshape(-1, 3)
    model.set_state(u, v)
    step = deck.restart["step"]
    model.set_time(float(step) * deck.problem.dt, step)
    return step


def run_fd(deck, precision=abi.FP64, graph=0, on_output=None):
    model = gpu.FDModel(deck.problem, precision=precision)
    if graph:
        model.set_graph(graph)
    start = _restart_state(model, deck) if deck.restart else 0
    steps, files = output.integrate(model, deck.output, deck.time_steps - start,
                                    on_output=on_output)
    return model, steps, files


def _qs_output(q, deck, n, t):
    """model::Output for the quasi-static model's fields (util.cpp:4-191)."""
    tags = set(deck.output.tags)
    p = deck.problem
    u, f = q.get()
    pd = []
    if "Displacement" in tags:
        pd.append(("Displacement", u))
    if "Velocity" in tags:
        pd.append(("Velocity", np.zeros_like(u)))
    if "Force" in tags:
        pd.append(("Force", f))
    if "Node_Volume" in tags:
        pd.append(("Node_Volume", np.asarray(p.volume, dtype=np.float64)))
    if "Neighbors" in tags:
        rowptr, _ = gpu.neighbor_search(p.x, p.horizon, dim=p.dim)
        pd.append(("Neighbors", np.diff(rowptr).astype(np.uint64)))
    dt_c = deck.output.dt_out_criteria or 1
    os.makedirs(deck.output.path, exist_ok=True)
    name = os.path.join(deck.output.path, "output_%d.vtu" % (n // dt_c))
    x = np.asarray(p.x, dtype=np.float64).reshape(-1, 3)
    vtu.write_points(name, x + u, pd, [("TIME", t)])
    return name


def run_qs(deck):
    """QuasiStaticModel::solver (QuasiStaticModel.cpp:526-594): output of the
    initial state, then one output after each load step."""
    s = deck.solver
    prm = gpu.esqs_params(max_iters=int(s.get("Max_Iteration", 100)),
                          tol=float(s.get("Tolerance", 1e-6)),
                          perturbation=float(s.get("Perturbation", 1e-7)),
                          dt=deck.problem.dt)
    q = gpu.ESQSModel(deck.problem, prm)
    files = [_qs_output(q, deck, 0, 0.0)]
    iters = []
    for n in range(1, deck.time_steps + 1):
        it, _, res = q.solve(1)
        iters.append((it[0], res))
        files.append(_qs_output(q, deck, n, n * deck.problem.dt))
    return q, iters, files


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("-i", "--input", required=True, help="the deck (YAML)")
    ap.add_argument("--precision", choices=["fp64", "fp32c"], default="fp64")
    ap.add_argument("--graph", type=int, default=0, help="steps per CUDA graph (0: off)")
    ap.add_argument("--out", default=None, help="output folder instead of the deck's Output.Path")
    args = ap.parse_args(argv)
    t0 = time.time()
    deck = deckfile.read_deck(args.input)
    if args.out:
        deck.output.path = args.out
    if deck.quasi_static:
        _, iters, files = run_qs(deck)
        summary = {"model": "QuasiStaticModel<ElasticState>", "load_steps": len(iters),
                   "newton": [i for i, _ in iters], "residual": [r for _, r in iters]}
    else:
        prec = abi.FP64 if args.precision == "fp64" else abi.FP32C
        model, steps, files = run_fd(deck, prec, args.graph)
        summary = {"model": "FDModel<%s>" % deck.problem.material.kind, "steps": steps,
                   "time": model.time()[0], "broken_bonds": model.count_broken()}
    summary.update({"outputs": len(files), "seconds": round(time.time() - t0, 3)})
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
