#!/usr/bin/env python
"""Headline benchmark: explicit RNPBond peridynamics step on one GB300.

Workload (default): the 1000 x 1000 node plate (h = 1e-4 m, horizon 3h,
seeded +-0.05h jitter, 2 mm centre pre-crack, top/bottom 3-node layers pulled
at +-0.1 m/s, velocity-Verlet dt = 2e-9 s).  A step is one Verlet step: one
fused force + integrate launch over every node.  The metric is bond-updates/s
= directed bonds x steps / time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is the FP32-compensated device throughput with
the state resident in HBM; `fp64_plain` is the same run in FP64 plain mode;
`e2e` is measured through the host-resident drop-in call nlm_fd_step_host,
copying u, v, f in and out of pinned host memory every step.  The
`--impl reference` arm times the CPU restatement of the reference (oracle/)
on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bond-updates/s FP32 vs FP64 plain; QS Newton s, learned vs plain @1e-8 res"
UNIT = "bond-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1000, help="plate nodes per side")
    ap.add_argument("--fp64-steps", type=int, default=200)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-steps", type=int, default=30)
    ap.add_argument("--es-steps", type=int, default=50,
                    help="steps of the 100^3 ElasticState cube (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--qs-steps", type=int, default=100,
                    help="quasi-static load steps of the learned vs plain warm-start comparison "
                         "(200 x 200 plate); 0 skips it")
    ap.add_argument("--decomp", default="auto", choices=["auto", "thread", "thread1", "warp", "tile", "tilel"])
    ap.add_argument("--workload", default="plate", choices=["plate", "ensemble"],
                    help="plate: 1000x1000 RNPBond plate (headline); ensemble: 256 plates "
                         "of 5k-200k nodes batched, against sequential single-plate runs")
    ap.add_argument("--plates", type=int, default=256)
    ap.add_argument("--seq-plates", type=int, default=16,
                    help="plates timed one by one for the sequential comparison")
    ap.add_argument("--graph", type=int, default=50,
                    help="steps per CUDA graph in the timed FP32C run (0: launches one by one)")
    ap.add_argument("--err-steps", type=int, default=5000,
                    help="steps of the FP32C-vs-FP64 error run on the plate (0: skip)")
    ap.add_argument("--es-err-steps", type=int, default=200,
                    help="steps of the FP32C-vs-FP64 error run on the 100^3 cube (0: skip)")
    ap.add_argument("--ens-plates", type=int, default=32,
                    help="plates of the batched-ensemble line in the default run (0: skip)")
    ap.add_argument("--ens-steps", type=int, default=200)
    ap.add_argument("--qs-heldout", default="100,101",
                    help="held-out training-geometry seeds also timed learned vs plain")
    ap.add_argument("--cpu1-steps", type=int, default=2,
                    help="steps of the 1-thread CPU baseline leg (0: skip)")
    ap.add_argument("--quick", action="store_true",
                    help="FP32C timed run only (profiling driver)")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Ranks:
    """Barrier and reductions over the ranks of a replicas run: one process
    per GPU, each stepping its own specimen (seed = rank); the job's time is
    the slowest rank's, its work the sum over ranks.  With one rank no
    process group exists.  device "cuda" synchronises the GPU around each
    barrier; "cpu" (a gloo group) is for tests of the reduction logic."""

    def __init__(self, world, device="cuda"):
        self.world = world
        self.device = device

    def _sync(self):
        if self.device == "cuda":
            import torch
            torch.cuda.synchronize()

    def barrier(self):
        self._sync()
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()
            self._sync()

    def _reduce(self, v, op):
        if self.world == 1:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        import torch.distributed as dist
        return self._reduce(v, dist.ReduceOp.MAX)

    def sum(self, v):
        import torch.distributed as dist
        return self._reduce(v, dist.ReduceOp.SUM)


def throughput(bonds_per_rank, steps, seconds_per_rank, ranks):
    """Whole-job bond-updates/s: the bonds of every rank's specimen times the
    steps, over the slowest rank's time."""
    return ranks.sum(float(bonds_per_rank)) * steps / ranks.max(seconds_per_rank)


def problem(nx, seed):
    from nlmech_gb300 import configs
    if nx == 1000:
        p = configs.config1(seed=seed)
    else:
        p = configs.rnp_plate(nx, 0.1 / nx, 3, 0.02 * 0.1, 0.1, 2e-9, 5000, seed=seed)
    return p


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


KERNELS = {1: ("k_rnp32_thread", "rnp_fp32_step_plate1000.md"),
           2: ("k_rnp32_warp", None), 3: ("k_rnp32_thread1", None),
           4: ("k_rnp32_tile", None),
           5: ("k_rnp32_tilel", "rnp_fp32_tilel_step_plate1000.md")}


def profiled_traffic(decomp=1):
    """dram bytes per launch of the step kernel from the committed ncu summary."""
    name = KERNELS.get(decomp, (None, None))[1]
    if name is None:
        return None
    p = os.path.join(ROOT, "profiles", name)
    try:
        for ln in open(p):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo) and core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() == "Model name":
                name = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not name:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith("model name"):
                    name = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"model": name or "unknown", "nproc": os.cpu_count()}


# The port against the reference's own FDModel<RNPBond> sources compiled with
# OpenMP loops (oracle/refshim), same 200 x 200 plate, same 8 x86 cores,
# identical results: the port ran 3.4x faster (1.9e8 vs 5.5e7 bond-updates/s).
# The reference tree is not on the GPU machine, so the refshim cannot be
# timed there.
PORT_OVER_REFSHIM_X86 = 3.4


def cpu_baseline(nx, steps, threads=None, steps1=0):
    """The oracle (CPU restatement of FDModel<RNPBond>) on a bounded sample,
    with all host threads, and (steps1 > 0) on one thread."""
    from oracle import oracle as orc
    if threads:
        orc.set_threads(threads)
    p = problem(nx, 0)
    o = orc.OracleFD(p)
    nnz = o.nnz()
    o.run(1)  # step-0 force evaluation and one step, untimed
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    out = {"value": nnz * steps / dt, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
           "sample": "%d Verlet steps of the %dx%d plate (%d bonds), after 1 untimed step"
                     % (steps, nx, nx, nnz),
           "cpu": cpu_model(),
           "port_over_reference_code": {
               "factor": PORT_OVER_REFSHIM_X86,
               "note": "the port against the reference's own sources (refshim, OpenMP) on "
                       "8 x86 cores of the build machine, 200 x 200 plate; the reference "
                       "tree is not on the GPU machine, so its own code is not timed here"}}
    if steps1 > 0:
        nt = orc.num_threads()
        orc.set_threads(1)
        t0 = time.perf_counter()
        o.run(steps1)
        d1 = time.perf_counter() - t0
        orc.set_threads(nt)
        out["one_thread"] = {"value": nnz * steps1 / d1, "unit": UNIT, "cores": 1,
                             "sample": "%d further Verlet steps of the same run" % steps1}
    return out


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    steps = min(a.steps, a.cpu_steps)
    cb = cpu_baseline(a.nx, steps)
    cb["sample"] += "; K=%d requested, %d timed (bounded CPU sample)" % (a.steps, steps)
    nnz = float(cb["sample"].split("(")[1].split()[0])
    out = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
           "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": 1e3 * nnz / cb["value"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered plate)",
           "config": {"workload": "rnp2d_plate_%dx%d_d3h_verlet" % (a.nx, a.nx),
                      "nodes": a.nx * a.nx},
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


DTYPE = ("f32 bond arithmetic and force sums; u, v held as double-float f32 (hi, lo) "
         "pairs (~48-bit significand), not f64")
DECOMP_NAMES = {1: "thread-per-node, 4-bond groups", 2: "warp-per-node",
                3: "thread-per-node, 1 bond/iteration",
                4: "256-node tiles staged in shared memory",
                5: "256-node tiles staged in shared memory, tile-frame FP32 bond data"}


def hot_path_bytes(nnz, n):
    """Compulsory bytes of one FP32C 2-D RNPBond step in the hot-path byte
    model: 4 B neighbour id + 0.25 B bond bit read and write per directed
    bond; x (8 B FP32 offset) + V 4 + flags 1 + rowptr 4 + u read/write 32 +
    v read/write 32 = 81 B per node."""
    return 4.25 * nnz + 81.0 * n


def design_bytes(nnz, n):
    """The same with this design's per-node arrays: the velocity-Verlet
    half-kick reads the previous step's force, so f (2 x f32) is read and
    written each step (16 B), and the row length (2 B) replaces the rowptr:
    x split + V 16 + flags 1 + row length 2 + u 32 + v 32 + f 16 = 99 B."""
    return 4.25 * nnz + 99.0 * n


def warm_graphs(m, G):
    """Capture both ping-pong phases' step graphs before a timed run."""
    if G <= 0:
        return
    m.set_graph(G)
    m.run(G + 1)
    m.run(G)


def run_ours(a):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from nlmech_gb300 import abi, accuracy, build, gpu
    build.build()
    gpu.set_device(local)
    p = problem(a.nx, seed=rank)
    n = p.n

    ranks = Ranks(world, "cuda")
    barrier_sync, max_over_ranks, sum_over_ranks = ranks.barrier, ranks.max, ranks.sum

    # ---- FP32-compensated (headline) ----
    dmap = {"auto": abi.DECOMP_AUTO, "thread": abi.DECOMP_THREAD,
            "thread1": abi.DECOMP_THREAD1, "warp": abi.DECOMP_WARP, "tile": abi.DECOMP_TILE,
            "tilel": abi.DECOMP_TILE_LOCAL}
    m = gpu.FDModel(p, precision=abi.FP32C, decomposition=dmap[a.decomp])
    nnz = m.nnz()
    dcode = m.decomposition()
    decomp = DECOMP_NAMES.get(dcode, "?")
    warm_graphs(m, a.graph)
    m.run(a.warmup)
    barrier_sync()
    with ClockSampler(local) as cs:
        ms = m.run_timed(a.steps)
    barrier_sync()
    ms = max_over_ranks(ms)
    total_bonds = sum_over_ranks(float(nnz))
    value = total_bonds * a.steps / (ms * 1e-3)
    clocks = cs.summary()
    if a.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "quick": True,
                              "ms_per_step": ms / a.steps, "steps": a.steps,
                              "decomposition": decomp, "clocks": clocks}))
        return 0
    broken = m.count_broken()
    m.close()

    # ---- FP64 plain ----
    m64 = gpu.FDModel(p, precision=abi.FP64)
    m64.run(3)
    barrier_sync()
    ms64 = m64.run_timed(a.fp64_steps)
    barrier_sync()
    ms64 = max_over_ranks(ms64)
    value64 = total_bonds * a.fp64_steps / (ms64 * 1e-3)
    m64.close()

    # ---- FP32C error against FP64 plain, same problem, full run ----
    errors = None
    if a.err_steps > 0:
        errors = accuracy.fp32c_error(p, a.err_steps, decomposition=dcode)
        errors["decomposition"] = DECOMP_NAMES.get(errors["decomposition"], "?")

    # ---- 3-D ElasticState cube (two-pass kernels), reported beside ----
    es = None
    if a.es_steps > 0:
        from nlmech_gb300 import configs
        pe = configs.config2(seed=rank)
        es = {"workload": "es3d_cube_100^3_d3h_verlet", "nodes": pe.n}
        for prec, key, k in ((abi.FP32C, "fp32c", a.es_steps), (abi.FP64, "fp64_plain",
                                                                  max(3, a.es_steps // 10))):
            mm = gpu.FDModel(pe, precision=prec)
            mm.run(2)
            barrier_sync()
            t = max_over_ranks(mm.run_timed(k))
            es["bonds"] = mm.nnz()
            es[key] = {"value": sum_over_ranks(float(mm.nnz())) * k / (t * 1e-3), "unit": UNIT,
                       "steps": k, "ms_per_step": t / k}
            mm.close()
        if a.es_err_steps > 0:
            es["errors"] = accuracy.fp32c_error(pe, a.es_err_steps)
            es["errors"]["decomposition"] = DECOMP_NAMES.get(es["errors"]["decomposition"], "?")

    # ---- end to end through the host-resident drop-in call ----
    # the step kernel the device-resident run used (autotuned there, or named)
    me = gpu.FDModel(p, precision=abi.FP32C, decomposition=dcode)
    bufs = [torch.zeros((n, 3), dtype=torch.float64).pin_memory() for _ in range(3)]
    ptrs = [b.data_ptr() for b in bufs]
    me.step_host_ptr(*ptrs, nsteps=1)  # step 0 + first step (untimed)
    for _ in range(3):
        me.step_host_ptr(*ptrs, nsteps=1)
    barrier_sync()
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        me.step_host_ptr(*ptrs, nsteps=1)
    barrier_sync()
    te = max_over_ranks(time.perf_counter() - t0)
    e2e_value = total_bonds * a.e2e_steps / te
    e2e_io = me.host_io()
    me.close()

    ens = None
    if a.ens_plates > 0 and world == 1:
        ens = ensemble_line(a.ens_plates, a.ens_steps, a.warmup, a.ens_plates)

    if rank != 0:
        return 0
    peaks = measured_peaks()
    if peaks and peaks.get("hbm_gbs"):
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    # one step-kernel launch per step: the kernel's mean duration is the timed
    # region's device time over its steps (CUDA events on the handle's stream)
    kms = ms / a.steps
    alg = hot_path_bytes(nnz, n)
    achieved = alg / (kms * 1e-3) / 1e9
    traffic = profiled_traffic(dcode)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
        "data": "synthetic (seeded jittered plate)",
        "config": {"workload": "rnp2d_plate_%dx%d_d3h_verlet" % (a.nx, a.nx), "nodes": n,
                   "bonds": nnz, "horizon": "3h", "dt": p.dt, "precision": "fp32c",
                   "decomposition": decomp + (" (autotuned)" if a.decomp == "auto" else ""),
                   "graph_steps": a.graph,
                   "l2": "inputs larger than L2: %.0f MB moved per step vs 129 MB L2"
                         % (design_bytes(nnz, n) / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "errors": errors,
        "fp64_plain": {"value": value64, "unit": UNIT, "steps": a.fp64_steps,
                       "ms_per_step": ms64 / a.fp64_steps, "dtype": "f64"},
        "fp32_over_fp64": value / value64,
        "es3d": es,
        "broken_bonds_after_run": broken,
        "e2e": {"value": e2e_value, "unit": UNIT, "steps": a.e2e_steps,
                "h2d_bytes_per_step": 3 * 3 * 8 * n, "d2h_bytes_per_step": 3 * 3 * 8 * n,
                "call": "nlm_fd_step_host (u, v, f in/out of pinned host memory each step)",
                "host_io": {0: "copies", 1: "in place", 2: "banded copies overlapping the step"}
                .get(e2e_io, e2e_io)},
        "gpu_launches": a.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_src,
                     "kernel": KERNELS.get(dcode, ("?", None))[0],
                     "kernel_ms": kms, "bytes_per_launch": alg,
                     "bytes_model": "4.25 B per directed bond + 81 B per node",
                     "design_bytes_per_launch": design_bytes(nnz, n),
                     "design_frac": design_bytes(nnz, n) / (kms * 1e-3) / 1e9 / peak,
                     "dram_frac": (traffic / (kms * 1e-3) / 1e9 / peak) if traffic else None,
                     "timing": "kernel_ms = timed region / steps (one launch per step)"},
        "clocks": clocks,
    }
    if ens is not None:
        out["ensemble"] = ens
    if a.qs_steps > 0:
        seeds = [int(s) for s in a.qs_heldout.split(",") if s.strip()]
        out["qs_warm_start"] = qs_warm_start(a.qs_steps, seeds)
    if not a.no_cpu:
        out["cpu_baseline"] = cpu_baseline(a.nx, a.cpu_steps, steps1=a.cpu1_steps)
    print(json.dumps(out))
    return 0


def qs_warm_start(steps, heldout=()):
    """Quasi-static Newton on the 200 x 200 pre-cracked RNP plate (top edge
    +1e-6 m per load step, bottom fixed, relative residual 1e-8): plain
    previous-step start vs the learned BF16 MLP start, wall time of the whole
    load-step loop including feature building and inference; then the same
    on held-out training-geometry seeds."""
    from nlmech_gb300 import configs, warmstart as ws
    if not os.path.exists(ws.WEIGHTS):
        return {"unavailable": "warm-start weights not found"}
    z = np.load(ws.WEIGHTS)
    model = ws.load_model()
    p = configs.config4()
    res = ws.evaluate(model, [p], steps, log=lambda *_: None)[p.name]
    res.update({"workload": "qs_rnp2d_200x200_d3h_precrack0.2W", "load_steps": steps,
                "tolerance": "||r|| <= 1e-8 ||r0|| every load step",
                "krylov": "PCG to 1e-4, loosened to min(0.1, %g target/||r||) for Newton "
                          "iterations already near the target; the same in every arm"
                          % ws.LIN_TOL_GAMMA,
                "mlp": "10 -> 128 x 3 -> 2, bf16 GEMMs with fp32 accumulation",
                "trained_on": "%d load steps of %d seeded pre-crack geometries (held out here)"
                              % (int(z["steps"]) * len(z["seeds"]), len(z["seeds"]))})
    if heldout:
        ps = [configs.qs_training_geometry(s) for s in heldout]
        r = ws.evaluate(model, ps, steps, log=lambda *_: None, ablation=False)
        res["heldout"] = {}
        for s, q in zip(heldout, ps):
            e = r[q.name]
            res["heldout"]["seed%d" % s] = {
                k: e[k] for k in ("speedup_wall", "newton_ratio", "u_rel_l2_vs_plain",
                                  "broken_bonds_differing", "broken_bonds_plain") if k in e}
            res["heldout"]["seed%d" % s]["plain_wall_s"] = e["plain"]["wall_s"]
            res["heldout"]["seed%d" % s]["learned_wall_s"] = e["learned"]["wall_s"]
    return res


def ensemble_line(nplates, steps, warmup, seq_plates, graph=20):
    """Batched ensemble against the same plates run one after another as
    separate autotuned models (each with its own step graphs)."""
    import torch
    from nlmech_gb300 import abi, configs, gpu
    plates = configs.ensemble(nplates=nplates, steps=steps)
    t0 = time.perf_counter()
    b = gpu.Batch(plates)
    setup_s = time.perf_counter() - t0
    nnz = b.nnz()
    b.set_graph(graph)
    b.run(graph + 1)
    b.run(graph)
    b.run(warmup)
    torch.cuda.synchronize()
    with ClockSampler(0) as cs:
        ms = b.run_timed(steps)
    torch.cuda.synchronize()
    value = nnz * steps / (ms * 1e-3)
    names = {1: "thread", 2: "warp", 3: "thread1", 5: "tile-frame"}
    buckets = [{"nodes": int(nd), "decomposition": names.get(dc, dc)} for nd, dc in b.buckets()]
    b.close()
    seq_ms, seq_bonds = 0.0, 0
    for p in plates[:seq_plates]:
        m = gpu.FDModel(p, precision=abi.FP32C, decomposition=abi.DECOMP_AUTO)
        warm_graphs(m, graph)
        m.run(warmup)
        seq_ms += m.run_timed(steps)
        seq_bonds += m.nnz()
        m.close()
    seq_value = seq_bonds * steps / (seq_ms * 1e-3)
    return {"workload": "rnp2d_ensemble_%d_plates_5k-200k_d4h" % nplates, "plates": nplates,
            "nodes": int(sum(p.n for p in plates)), "bonds": nnz, "steps": steps,
            "graph_steps": graph, "buckets": buckets, "setup_s": setup_s,
            "value": value, "unit": UNIT, "ms_per_step": ms / steps,
            "sequential": {"value": seq_value, "unit": UNIT, "plates_timed": seq_plates,
                           "note": "plates run one after another as separate models"},
            "batched_over_sequential": value / seq_value, "clocks": cs.summary()}


def run_ensemble(a):
    """Batched ensemble line alone (--workload ensemble)."""
    from nlmech_gb300 import build
    build.build()
    e = ensemble_line(a.plates, a.steps, a.warmup, a.seq_plates)
    out = {"metric": METRIC, "value": e["value"], "unit": UNIT, "n_gpus": 1, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": e["ms_per_step"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
           "data": "synthetic (seeded plates)",
           "config": {"workload": e["workload"], "plates": e["plates"], "nodes": e["nodes"],
                      "bonds": e["bonds"], "graph_steps": e["graph_steps"],
                      "buckets": e["buckets"], "setup_s": e["setup_s"]},
           "sequential": e["sequential"],
           "batched_over_sequential": e["batched_over_sequential"], "clocks": e["clocks"]}
    print(json.dumps(out))
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.workload == "ensemble":
        return run_ensemble(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
