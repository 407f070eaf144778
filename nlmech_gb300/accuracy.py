"""Error of an FP32-compensated run against the FP64 plain run of the same problem.

Both runs go through the GPU library: the FP64 plain path keeps the
reference's operation order (rnpBond.cpp:216-301, fDModel.cpp:445-582) and
matches the reference's own code to 1e-12, so it stands in for the FP64
reference at sizes where the CPU cannot run 5000 steps.  The reported fields
are those every FP32C result states:

* ``u_rel_l2``, ``v_rel_l2`` -- ||a - b||_2 / ||b||_2 over all nodes and
  components (b the FP64 field);
* ``damage_max_abs_diff`` -- max_i |phi_i(FP32C) - phi_i(FP64)|, phi the
  damage of computePostProcFields (fDModel.cpp:716-717);
* ``broken_bonds_differing`` -- the number of directed bonds (id_i, id_j)
  broken in one run and intact in the other, and its fraction of the FP64
  run's broken bonds;
* ``neighbors_identical`` -- both handles hold the same neighbour rows.
"""
import time

import numpy as np

from . import abi


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def compare_states(m32, m64):
    """Error fields of handle m32 against handle m64 (same problem, same
    number of steps)."""
    r32, c32 = m32.neighbors()
    r64, c64 = m64.neighbors()
    same_nb = bool(np.array_equal(r32, r64) and np.array_equal(c32, c64))
    u32, v32, _ = m32.state()
    u64, v64, _ = m64.state()
    b32, b64 = m32.bond_state(), m64.bond_state()
    if same_nb:
        ndiff = int(np.count_nonzero(b32 != b64))
    else:
        ndiff = len(_pairs(r32, c32, b32) ^ _pairs(r64, c64, b64))
    nb64 = int(np.count_nonzero(b64))
    phi32, _ = m32.damage()
    phi64, _ = m64.damage()
    return {
        "u_rel_l2": rel_l2(u32, u64),
        "v_rel_l2": rel_l2(v32, v64),
        "damage_max_abs_diff": float(np.abs(phi32.astype(np.float64) - phi64).max())
        if len(phi64) else 0.0,
        "broken_bonds_fp64": nb64,
        "broken_bonds_fp32c": int(np.count_nonzero(b32)),
        "broken_bonds_differing": ndiff,
        "broken_bonds_differing_frac": ndiff / max(nb64, 1),
        "neighbors_identical": same_nb,
    }


def _pairs(rowptr, cols, broken):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    sel = broken.astype(bool)
    return set(zip(rows[sel].tolist(), cols[sel].tolist()))


def fp32c_error(problem, steps, decomposition=None):
    """Run `problem` for `steps` steps in FP64 plain and in FP32C (the given
    decomposition, or the autotuner's pick) from the same initial state and
    return the error fields, the FP32C decomposition and both wall times."""
    from . import gpu
    dec = abi.DECOMP_AUTO if decomposition is None else decomposition
    t0 = time.perf_counter()
    m64 = gpu.FDModel(problem, precision=abi.FP64)
    m64.run(steps)
    m64.sync()
    t64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    m32 = gpu.FDModel(problem, precision=abi.FP32C, decomposition=dec)
    m32.run(steps)
    m32.sync()
    t32 = time.perf_counter() - t0
    out = compare_states(m32, m64)
    out.update({"steps": int(steps), "decomposition": m32.decomposition(),
                "fp64_wall_s": t64, "fp32c_wall_s": t32})
    m32.close()
    m64.close()
    return out
