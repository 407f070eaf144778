"""ctypes binding of libnlmgpu.so, shaped like the reference's FDModel.

The reference constructs ``model::FDModel<RNPBond>(deck)`` and the constructor
runs the whole simulation (src/model/fd/fDModel.cpp:47-67).  Here the same
steps are split so that a caller can drive and inspect them:

    m = FDModel(problem)       # initHObjects + init (neighbours, cracks, loads)
    m.run(nsteps)              # integrate(): nsteps Verlet / CD steps
    u, v, f = m.state()        # DataManager displacement / velocity / force

There is no CPU fallback: if libnlmgpu.so is missing or no GPU is present the
calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnlmgpu.so")

_lib = None


class NLMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libnlmgpu error %d: %s" % (code, msg))
        self.code = code


def load(path=None):
    """Load libnlmgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libnlmgpu.so not built at %s (run nlmech_gb300/build.py)" % p)
    L = C.CDLL(p)
    L.nlm_last_error.restype = C.c_char_p
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise NLMError(rc, load().nlm_last_error().decode())


def device_count():
    c = C.c_int()
    _check(load().nlm_device_count(C.byref(c)))
    return c.value


def set_device(dev):
    _check(load().nlm_set_device(C.c_int(int(dev))))


def neighbor_search(x, horizon, dim=2):
    """GPU cell-list neighbour lists in original ids (rowptr int64, cols int32)."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    n = x.shape[0]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    L = load()
    _check(L.nlm_neighbor_search(C.c_int(dim), C.c_int64(n), abi.dptr(x), C.c_double(horizon),
                                 abi.ptr(rowptr, C.c_int64), C.POINTER(C.c_int32)()))
    cols = np.zeros(int(rowptr[-1]), dtype=np.int32)
    _check(L.nlm_neighbor_search(C.c_int(dim), C.c_int64(n), abi.dptr(x), C.c_double(horizon),
                                 abi.ptr(rowptr, C.c_int64), abi.ptr(cols, C.c_int32)))
    return rowptr, cols


class FDModel:
    """model::FDModel<T> on the GPU (T chosen by problem.material.kind)."""

    def __init__(self, problem, precision=None, decomposition=None, scheme=None):
        self.problem = problem
        d, self._keep = problem.desc(precision=precision, decomposition=decomposition,
                                     scheme=scheme)
        self.precision = d.precision
        h = C.c_void_p()
        _check(load().nlm_fd_create(C.byref(d), C.byref(h)))
        self.h = h
        self.n = problem.n

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.nlm_fd_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def nnz(self):
        v = C.c_int64()
        _check(load().nlm_fd_num_bonds(self.h, C.byref(v)))
        return v.value

    def neighbors(self):
        rowptr = np.zeros(self.n + 1, dtype=np.int64)
        cols = np.zeros(self.nnz(), dtype=np.int32)
        _check(load().nlm_fd_get_neighbors(self.h, abi.ptr(rowptr, C.c_int64),
                                           abi.ptr(cols, C.c_int32)))
        return rowptr, cols

    def run(self, nsteps):
        _check(load().nlm_fd_run(self.h, C.c_int64(int(nsteps))))

    def sync(self):
        _check(load().nlm_fd_sync(self.h))

    def state(self):
        u = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        _check(load().nlm_fd_get_state(self.h, abi.dptr(u), abi.dptr(v), abi.dptr(f)))
        return u, v, f

    def set_state(self, u=None, v=None):
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        _check(load().nlm_fd_set_state(self.h, abi.dptr(u), abi.dptr(v)))

    def write_vtu(self, path, tags=("Displacement", "Velocity", "Force", "Damage_Phi",
                                    "Damage_Z")):
        """One output step in the reference's VTU layout (model::Output,
        src/model/util.cpp:4-191): points at x + u and the requested tags."""
        from . import vtu
        u, v, f = self.state()
        phi = Z = None
        if "Damage_Phi" in tags or "Damage_Z" in tags:
            phi, Z = self.damage()
        t, _ = self.time()
        vtu.write_vtu(path, self.problem.x, u=u,
                      v=v if "Velocity" in tags else None,
                      f=f if ("Force" in tags or "Force_Density" in tags) else None,
                      volume=self.problem.volume,
                      phi=phi if "Damage_Phi" in tags else None,
                      Z=Z if "Damage_Z" in tags else None, time=t)

    def set_bond_state(self, broken):
        b = np.ascontiguousarray(broken, dtype=np.uint8)
        _check(load().nlm_fd_set_bond_state(self.h, abi.ptr(b, C.c_uint8)))

    def save(self, path):
        """Checkpoint u, v, f, bond state, step and time to a binary file."""
        _check(load().nlm_fd_save(self.h, str(path).encode()))

    def load(self, path):
        """Continue from a checkpoint written by save() for the same model."""
        _check(load().nlm_fd_load(self.h, str(path).encode()))

    def step_host(self, u, v, f, nsteps=1):
        """Drop-in step on host arrays u, v, f (3 doubles per node, updated
        in place); passing back the previous call's arrays continues the run."""
        _check(load().nlm_fd_step_host(self.h, abi.dptr(u), abi.dptr(v), abi.dptr(f),
                                       C.c_int64(int(nsteps))))

    def step_host_ptr(self, u_ptr, v_ptr, f_ptr, nsteps=1):
        """Same as step_host with raw host addresses (e.g. pinned buffers)."""
        P = C.POINTER(C.c_double)
        _check(load().nlm_fd_step_host(self.h, C.cast(u_ptr, P), C.cast(v_ptr, P),
                                       C.cast(f_ptr, P), C.c_int64(int(nsteps))))

    def host_io(self):
        """How the last step_host moved the arrays: 0 copies (pageable
        arrays), 1 read and written in place by kernels (page-locked), 2 in
        caller-order bands overlapped with the step (page-locked, one FP32C
        2-D step on a tile decomposition)."""
        m = C.c_int()
        _check(load().nlm_fd_host_io(self.h, C.byref(m)))
        return m.value

    def set_alloc_limit(self, nbytes):
        """Cap the device bytes the handle may still allocate (< 0: no cap)."""
        _check(load().nlm_fd_set_alloc_limit(self.h, C.c_int64(int(nbytes))))

    def run_timed(self, nsteps):
        """Run nsteps; returns the device time in ms (CUDA events on the
        handle's stream)."""
        ms = C.c_double()
        _check(load().nlm_fd_run_timed(self.h, C.c_int64(int(nsteps)), C.byref(ms)))
        return ms.value

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        _check(load().nlm_fd_get_time(self.h, C.byref(t), C.byref(n)))
        return t.value, n.value

    def bond_state(self):
        b = np.zeros(self.nnz(), dtype=np.uint8)
        _check(load().nlm_fd_get_bond_state(self.h, abi.ptr(b, C.c_uint8)))
        return b

    def count_broken(self):
        c = C.c_int64()
        _check(load().nlm_fd_count_broken(self.h, C.byref(c)))
        return c.value

    def damage(self):
        phi = np.zeros(self.n, dtype=np.float32)
        Z = np.zeros(self.n, dtype=np.float32)
        _check(load().nlm_fd_damage(self.h, abi.ptr(phi, C.c_float), abi.ptr(Z, C.c_float)))
        return phi, Z

    def set_time(self, time, step):
        """Start at this step and time (a restart); before the first step."""
        _check(load().nlm_fd_set_time(self.h, C.c_double(float(time)), C.c_int64(int(step))))

    def fixity(self):
        fx = np.zeros(self.n, dtype=np.uint8)
        _check(load().nlm_fd_get_fixity(self.h, abi.ptr(fx, C.c_uint8)))
        return fx

    def energies(self):
        """(strain, work, kinetic, fracture) per node (float32) and their
        sums, as computePostProcFields (fDModel.cpp:651-778) forms them."""
        e = np.zeros((4, self.n), dtype=np.float32)
        tot = np.zeros(4)
        _check(load().nlm_fd_energies(self.h, *[abi.ptr(e[q], C.c_float) for q in range(4)],
                  abi.dptr(tot)))
        return e, tot

    def reaction_force(self):
        """Reaction_Force (n, 3), Total_Reaction_Force (n,) and the sum (3,)
        of FDModel::computeForce (fDModel.cpp:543-605)."""
        R = np.zeros((self.n, 3))
        t = np.zeros(self.n)
        s = np.zeros(3)
        _check(load().nlm_fd_reaction_force(self.h, abi.dptr(R), abi.dptr(t), abi.dptr(s)))
        return R, t, s

    def decomposition(self):
        d = C.c_int()
        _check(load().nlm_fd_decomposition(self.h, C.byref(d)))
        return d.value

    def set_timing(self, on):
        _check(load().nlm_fd_set_timing(self.h, C.c_int(int(on))))

    def kernel_stats(self, reset=True):
        ms = C.c_double()
        L = C.c_int64()
        b = C.c_double()
        _check(load().nlm_fd_kernel_stats(self.h, C.c_int(int(reset)), C.byref(ms), C.byref(L),
                                          C.byref(b)))
        return ms.value, L.value, b.value


def _fd_set_graph(self, steps_per_graph):
    """Replay the step loop from CUDA graphs of this many steps (0: off)."""
    _check(load().nlm_fd_set_graph(self.h, C.c_int(int(steps_per_graph))))


FDModel.set_graph = _fd_set_graph


class Batch:
    """Many independent RNPBond specimens stepped together (FP32C).
    decomposition: None keeps each problem's own (autotuned per node-count
    bucket unless every problem names the same one); a DECOMP_* value is used
    for every bucket."""

    def __init__(self, problems, scheme=None, decomposition=None):
        self.problems = list(problems)
        descs, self._keep = [], []
        for p in self.problems:
            d, keep = p.desc(precision=abi.FP32C, scheme=scheme, decomposition=decomposition)
            descs.append(d)
            self._keep.append(keep)
        arr = (abi.FDDesc * len(descs))(*descs)
        self._keep.append(arr)
        h = C.c_void_p()
        _check(load().nlm_batch_create(arr, C.c_int(len(descs)), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.nlm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def nnz(self, s=-1):
        v = C.c_int64()
        _check(load().nlm_batch_num_bonds(self.h, C.c_int(s), C.byref(v)))
        return v.value

    def run(self, nsteps):
        _check(load().nlm_batch_run(self.h, C.c_int64(int(nsteps))))

    def run_timed(self, nsteps):
        ms = C.c_double()
        _check(load().nlm_batch_run_timed(self.h, C.c_int64(int(nsteps)), C.byref(ms)))
        return ms.value

    def set_graph(self, steps_per_graph):
        _check(load().nlm_batch_set_graph(self.h, C.c_int(int(steps_per_graph))))

    def state(self, s):
        n = self.problems[s].n
        u = np.zeros((n, 3))
        v = np.zeros((n, 3))
        f = np.zeros((n, 3))
        _check(load().nlm_batch_get_state(self.h, C.c_int(s), abi.dptr(u), abi.dptr(v),
                                          abi.dptr(f)))
        return u, v, f

    def bond_state(self, s):
        b = np.zeros(self.nnz(s), dtype=np.uint8)
        _check(load().nlm_batch_get_bond_state(self.h, C.c_int(s), abi.ptr(b, C.c_uint8)))
        return b

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        _check(load().nlm_batch_get_time(self.h, C.byref(t), C.byref(n)))
        return t.value, n.value

    def buckets(self):
        nb = C.c_int()
        nodes = (C.c_int64 * 8)()
        dec = (C.c_int * 8)()
        _check(load().nlm_batch_buckets(self.h, C.byref(nb), nodes, dec))
        return [(nodes[k], dec[k]) for k in range(nb.value)]


def qs_params(max_newton=30, tol=1e-8, lin_max_iters=20000, lin_tol=1e-4, break_bonds=True,
              max_break_rounds=50, guess_accept=0.1, krylov_launch=0, wait_limit_s=1.0,
              barrier_extra=0, lin_tol_gamma=0.0):
    """nlm_qs_params; krylov_launch 0: the FP32 Krylov solve in two launches
    per iteration, 1: in one cooperative launch per solve; barrier_extra > 0
    only to test the bounded barrier wait (wait_limit_s) of the latter;
    lin_tol_gamma > 0 loosens the Krylov tolerance of a Newton iteration
    whose residual is already near the target."""
    return abi.QSParams(max_newton, tol, lin_max_iters, lin_tol, int(break_bonds),
                        max_break_rounds, guess_accept, int(krylov_launch),
                        float(wait_limit_s), int(barrier_extra), float(lin_tol_gamma))


class QSModel:
    """Quasi-static Newton load steps (QuasiStaticModel<RNPBond> on the GPU)."""

    def __init__(self, problem, params=None):
        self.problem = problem
        d, self._keep = problem.desc(precision=abi.FP64)
        self.params = params or qs_params()
        h = C.c_void_p()
        _check(load().nlm_qs_create(C.byref(d), C.byref(self.params), C.byref(h)))
        self.h = h
        self.n = problem.n

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.nlm_qs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def load_step(self, guess=None, candidates=None):
        """One load step from the plain start, a guess ((n, 3) displacement)
        or the best of several candidate starts (list of (n, 3)); stats
        "used_guess" is the 1-based index of the start used (0: plain)."""
        st = abi.QSStats()
        if candidates is not None:
            g = np.ascontiguousarray(np.stack([np.asarray(c, dtype=np.float64).reshape(-1, 3)
                                               for c in candidates]))
            _check(load().nlm_qs_load_step_candidates(self.h, abi.dptr(g), C.c_int(g.shape[0]),
                                                      C.byref(st)))
            return st.as_dict()
        g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64)
        _check(load().nlm_qs_load_step(self.h, abi.dptr(g), C.byref(st)))
        return st.as_dict()

    def state(self):
        u = np.zeros((self.n, 3))
        _check(load().nlm_qs_get_state(self.h, abi.dptr(u)))
        return u

    def nnz(self):
        v = C.c_int64()
        _check(load().nlm_qs_num_bonds(self.h, C.byref(v)))
        return v.value

    def bond_state(self):
        b = np.zeros(self.nnz(), dtype=np.uint8)
        _check(load().nlm_qs_get_bond_state(self.h, abi.ptr(b, C.c_uint8)))
        return b

    def damage(self):
        phi = np.zeros(self.n, dtype=np.float32)
        Z = np.zeros(self.n, dtype=np.float32)
        _check(load().nlm_qs_damage(self.h, abi.ptr(phi, C.c_float), abi.ptr(Z, C.c_float)))
        return phi, Z


def esqs_params(max_iters=200, tol=1e-6, perturbation=1e-7, jacobian=0, tol_relative=False,
                lin_max_iters=5000, lin_tol=1e-12, dt=1.0):
    """Solver deck of QuasiStaticModel (Max_Iteration, Tolerance,
    Perturbation) plus the BiCGSTAB cap and tolerance."""
    return abi.ESQSParams(jacobian=int(jacobian), max_iters=int(max_iters), tol=float(tol),
                          tol_relative=int(bool(tol_relative)), perturbation=float(perturbation),
                          lin_max_iters=int(lin_max_iters), lin_tol=float(lin_tol), dt=float(dt))


class ESQSModel:
    """QuasiStaticModel<ElasticState> on the GPU (nlm_esqs_*)."""

    def __init__(self, problem, params=None):
        self.problem = problem
        self.params = params if params is not None else esqs_params()
        d, self._keep = problem.desc(precision=abi.FP64)
        h = C.c_void_p()
        _check(load().nlm_esqs_create(C.byref(d), C.byref(self.params), C.byref(h)))
        self.h = h
        self.n = problem.n

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.nlm_esqs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def solve(self, nsteps=1):
        """nsteps load steps: (Newton iterations per step, BiCGSTAB
        iterations per step, final residual norm)."""
        it = (C.c_int * max(1, nsteps))()
        li = (C.c_int * max(1, nsteps))()
        res = C.c_double()
        _check(load().nlm_esqs_solve(self.h, C.c_int(int(nsteps)), it, li, C.byref(res)))
        return list(it)[:nsteps], list(li)[:nsteps], res.value

    def get(self):
        """u (n, 3) and the output's "Force" f_i V_i (n, 3)."""
        u = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        _check(load().nlm_esqs_get_state(self.h, abi.dptr(u), abi.dptr(f)))
        return u, f


def mlp_layout(n_in, n_hidden, n_layers, n_out):
    """[(d_in, d_out, w_offset, b_offset)] of the nlm_mlp parameter vector."""
    r16 = lambda v: (v + 15) // 16 * 16
    dims = [r16(n_in)] + [r16(n_hidden)] * n_layers + [(n_out + 7) // 8 * 8]
    out, off = [], 0
    for l in range(n_layers + 1):
        di, do = dims[l], dims[l + 1]
        out.append((di, do, off, off + di * do))
        off += di * do + do
    return out


class MLP:
    """Per-node MLP with BF16 tensor-core GEMMs (nlm_mlp_*)."""

    def __init__(self, n_in=10, n_hidden=128, n_layers=3, n_out=2, seed=0):
        self.shape = (n_in, n_hidden, n_layers, n_out)
        h = C.c_void_p()
        _check(load().nlm_mlp_create(C.c_int(n_in), C.c_int(n_hidden), C.c_int(n_layers),
                                     C.c_int(n_out), C.c_uint64(seed), C.byref(h)))
        self.h = h
        c = C.c_int64()
        _check(load().nlm_mlp_num_params(self.h, C.byref(c)))
        self.nparams = c.value
        self.layout = mlp_layout(*self.shape)

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.nlm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        _check(load().nlm_mlp_get_params(self.h, abi.ptr(p, C.c_float)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _check(load().nlm_mlp_set_params(self.h, abi.ptr(p, C.c_float)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((x.shape[0], self.shape[3]), dtype=np.float32)
        _check(load().nlm_mlp_forward(self.h, abi.ptr(x, C.c_float), C.c_int64(x.shape[0]),
                                      abi.ptr(y, C.c_float)))
        return y

    def grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_float()
        _check(load().nlm_mlp_grad(self.h, abi.ptr(x, C.c_float), abi.ptr(t, C.c_float),
                                   C.c_int64(x.shape[0]), C.byref(loss), abi.ptr(g, C.c_float)))
        return loss.value, g

    def set_data(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        _check(load().nlm_mlp_set_data(self.h, abi.ptr(x, C.c_float), abi.ptr(t, C.c_float),
                                       C.c_int64(x.shape[0])))

    def train(self, epochs, batch=4096, lr=1e-3, seed=0, losses=True):
        out = np.zeros(max(epochs, 1), dtype=np.float32)
        _check(load().nlm_mlp_train(self.h, C.c_int(epochs), C.c_int(batch), C.c_float(lr),
                                    C.c_uint64(seed),
                                    abi.ptr(out, C.c_float) if losses else None))
        return out[:epochs]
