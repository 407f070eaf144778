"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by bench.py's CPU-baseline leg
and by __graft_entry__.smoke() as the checker.  The product package
(nlmech_gb300) never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from nlmech_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False):
    """Compile liboracle.so with the Makefile beside this file."""
    src = [os.path.join(HERE, f) for f in ("nlm_oracle.cpp", "nlm_oracle.h")]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in src)):
        return LIB
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB


class QSParams(C.Structure):
    _fields_ = [
        ("jacobian", C.c_int),
        ("solver", C.c_int),
        ("max_iters", C.c_int),
        ("tol", C.c_double),
        ("tol_relative", C.c_int),
        ("perturbation", C.c_double),
        ("lin_max_iters", C.c_int),
        ("lin_tol", C.c_double),
        ("dt", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_last_error.restype = C.c_char_p
        for nm in ("orc_fd_create", "orc_qs_create"):
            getattr(L, nm).restype = C.c_int
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle error %d: %s" % (rc, lib().orc_last_error().decode()))


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())


def neighbors(x, horizon, dim=2, grid=True):
    """CSR neighbour lists (rowptr int64 n+1, cols int32), rows ascending."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    n = x.shape[0]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    L = lib()
    fn = L.orc_neighbors_grid if grid else L.orc_neighbors_brute
    args = ([C.c_int(dim)] if grid else []) + [C.c_int64(n), abi.dptr(x), C.c_double(horizon)]
    _check(fn(*args, abi.ptr(rowptr, C.c_int64), C.POINTER(C.c_int32)()))
    cols = np.zeros(int(rowptr[-1]), dtype=np.int32)
    _check(fn(*args, abi.ptr(rowptr, C.c_int64), abi.ptr(cols, C.c_int32)))
    return rowptr, cols


def rnp_params(material, dim, horizon):
    out = (C.c_double * 7)()
    m = material.to_c()
    _check(lib().orc_rnp_params(C.byref(m), C.c_int(dim), C.c_double(horizon), out))
    keys = ("C", "beta", "rbar", "invF", "M", "nu", "lambda")
    return dict(zip(keys, list(out)))


class OracleFD:
    """FDModel restated on the CPU (explicit dynamics)."""

    def __init__(self, problem, grid_neighbors=True):
        self.problem = problem
        d, self._keep = problem.desc()
        h = C.c_void_p()
        _check(lib().orc_fd_create(C.byref(d), C.c_int(int(grid_neighbors)), C.byref(h)))
        self.h = h
        self.n = problem.n

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_fd_destroy(self.h)
            self.h = None

    def nnz(self):
        v = C.c_int64()
        _check(lib().orc_fd_num_bonds(self.h, C.byref(v)))
        return v.value

    def neighbors(self):
        rowptr = np.zeros(self.n + 1, dtype=np.int64)
        cols = np.zeros(self.nnz(), dtype=np.int32)
        _check(lib().orc_fd_get_neighbors(self.h, abi.ptr(rowptr, C.c_int64), abi.ptr(cols, C.c_int32)))
        return rowptr, cols

    def run(self, nsteps):
        _check(lib().orc_fd_run(self.h, C.c_int64(nsteps)))

    def state(self):
        u = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        _check(lib().orc_fd_get_state(self.h, abi.dptr(u), abi.dptr(v), abi.dptr(f)))
        return u, v, f

    def set_state(self, u=None, v=None):
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        _check(lib().orc_fd_set_state(self.h, abi.dptr(u), abi.dptr(v)))

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        _check(lib().orc_fd_get_time(self.h, C.byref(t), C.byref(n)))
        return t.value, n.value

    def bond_state(self):
        b = np.zeros(self.nnz(), dtype=np.uint8)
        _check(lib().orc_fd_get_bond_state(self.h, abi.ptr(b, C.c_uint8)))
        return b

    def set_bond_state(self, b):
        b = np.ascontiguousarray(b, dtype=np.uint8)
        _check(lib().orc_fd_set_bond_state(self.h, abi.ptr(b, C.c_uint8)))

    def fixity(self):
        f = np.zeros(self.n, dtype=np.uint8)
        _check(lib().orc_fd_get_fixity(self.h, abi.ptr(f, C.c_uint8)))
        return f

    def damage(self):
        phi = np.zeros(self.n, dtype=np.float32)
        Z = np.zeros(self.n, dtype=np.float32)
        _check(lib().orc_fd_damage(self.h, abi.ptr(phi, C.c_float), abi.ptr(Z, C.c_float)))
        return phi, Z

    def energies(self):
        """(strain, work, kinetic, fracture) per node (float32) and their
        sums, as computePostProcFields (fDModel.cpp:651-778) forms them."""
        e = np.zeros((4, self.n), dtype=np.float32)
        tot = np.zeros(4)
        _check(lib().orc_fd_energies(self.h, *[abi.ptr(e[q], C.c_float) for q in range(4)],
                  abi.dptr(tot)))
        return e, tot

    def reaction_force(self):
        """Reaction_Force (n, 3), Total_Reaction_Force (n,) and the sum (3,)
        of FDModel::computeForce (fDModel.cpp:543-605)."""
        R = np.zeros((self.n, 3))
        t = np.zeros(self.n)
        s = np.zeros(3)
        _check(lib().orc_fd_reaction_force(self.h, abi.dptr(R), abi.dptr(t), abi.dptr(s)))
        return R, t, s

    def es_fields(self):
        om = np.zeros(self.nnz())
        m = np.zeros(self.n)
        th = np.zeros(self.n)
        _check(lib().orc_fd_es_fields(self.h, abi.dptr(om), abi.dptr(m), abi.dptr(th)))
        return om, m, th

    def eval_force(self):
        f = np.zeros((self.n, 3))
        _check(lib().orc_fd_eval_force(self.h, abi.dptr(f)))
        return f


class OracleQS:
    """QuasiStaticModel<ElasticState> restated on the CPU."""

    def __init__(self, problem, params):
        d, self._keep = problem.desc()
        h = C.c_void_p()
        self.params = params
        _check(lib().orc_qs_create(C.byref(d), C.byref(params), C.byref(h)))
        self.h = h
        self.n = problem.n

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_qs_destroy(self.h)
            self.h = None

    def solve(self, nsteps):
        iters = (C.c_int * nsteps)()
        res = C.c_double()
        _check(lib().orc_qs_solve(self.h, C.c_int(nsteps), iters, C.byref(res)))
        return list(iters), res.value

    def get(self):
        u = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        nnz = C.c_int64()
        _check(lib().orc_qs_get(self.h, abi.dptr(u), abi.dptr(f), C.byref(nnz)))
        return u, f


class QSRStats(C.Structure):
    _fields_ = [
        ("newton_iters", C.c_int),
        ("lin_iters", C.c_int),
        ("break_rounds", C.c_int),
        ("used_guess", C.c_int),
        ("broken", C.c_int64),
        ("res_plain", C.c_double),
        ("res_start", C.c_double),
        ("res_final", C.c_double),
    ]


class OracleQSR:
    """Quasi-static RNPBond restated on the CPU (same definition as the GPU)."""

    def __init__(self, problem, max_newton=30, tol=1e-8, lin_max_iters=20000, lin_tol=1e-4,
                 break_bonds=True, max_break_rounds=50):
        d, self._keep = problem.desc()
        h = C.c_void_p()
        _check(lib().orc_qsr_create(C.byref(d), C.c_int(max_newton), C.c_double(tol),
                                    C.c_int(lin_max_iters), C.c_double(lin_tol),
                                    C.c_int(int(break_bonds)), C.c_int(max_break_rounds),
                                    C.byref(h)))
        self.h = h
        self.n = problem.n
        self.problem = problem

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_qsr_destroy(self.h)
            self.h = None

    def load_step(self, guess=None):
        st = QSRStats()
        g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64)
        _check(lib().orc_qsr_load_step(self.h, abi.dptr(g), C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def state(self):
        u = np.zeros((self.n, 3))
        _check(lib().orc_qsr_get_state(self.h, abi.dptr(u)))
        return u

    def bond_state(self):
        rp, cols = neighbors(self.problem.x, self.problem.horizon, dim=self.problem.dim)
        b = np.zeros(len(cols), dtype=np.uint8)
        _check(lib().orc_qsr_get_bond_state(self.h, abi.ptr(b, C.c_uint8)))
        return b


# ---- the reference's own RNPBond sources (oracle/refshim) -------------------
def _recipe_reference_tree():
    """The tree the refshim recipe (refshim/Makefile) compiles from: its
    `REF ?=` default, the one place that names where the tree lies."""
    try:
        for ln in open(os.path.join(HERE, "refshim", "Makefile")):
            if ln.startswith("REF ?="):
                return ln.split("=", 1)[1].strip()
    except OSError:
        pass
    return ""


# NLMECH_REFERENCE overrides the recipe's default; where neither holds the
# tree, the checks that need it are skipped.
REF_TREE = os.environ.get("NLMECH_REFERENCE") or _recipe_reference_tree()
REF_LIB = os.path.join(HERE, "_ref", "libref_rnp.so")
_ref = None


def refshim_available():
    """True if libref_rnp.so exists or the reference tree is here to build it."""
    return os.path.exists(REF_LIB) or os.path.isdir(os.path.join(REF_TREE, "src"))


def build_refshim():
    """Compile the reference's RNPBond sources with oracle/refshim/Makefile."""
    if not os.path.isdir(os.path.join(REF_TREE, "src")):
        if os.path.exists(REF_LIB):
            return REF_LIB
        raise RuntimeError("reference tree not found at %s" % REF_TREE)
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "refshim"),
                           "REF=" + REF_TREE])
    return REF_LIB


def ref_lib():
    global _ref
    if _ref is None:
        build_refshim()
        L = C.CDLL(REF_LIB)
        L.ref_rnp_last_error.restype = C.c_char_p
        _ref = L
    return _ref


class RefRNP:
    """The reference's Neighbor, Fracture, InteriorFlags, ULoading/FLoading
    and RNPBond::getBondEF driven through FDModel's velocity-Verlet loop."""

    def __init__(self, problem):
        d, self._keep = problem.desc()
        h = C.c_void_p()
        self._chk(ref_lib().ref_rnp_create(C.byref(d), C.byref(h)))
        self.h = h
        self.n = problem.n

    @staticmethod
    def _chk(rc):
        if rc != 0:
            raise RuntimeError("refshim error: %s" % ref_lib().ref_rnp_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_rnp_destroy(self.h)
            self.h = None

    def nnz(self):
        v = C.c_int64()
        self._chk(ref_lib().ref_rnp_num_bonds(self.h, C.byref(v)))
        return v.value

    def neighbors(self):
        rowptr = np.zeros(self.n + 1, dtype=np.int64)
        cols = np.zeros(self.nnz(), dtype=np.int32)
        self._chk(ref_lib().ref_rnp_get_neighbors(self.h, abi.ptr(rowptr, C.c_int64),
                                                  abi.ptr(cols, C.c_int32)))
        return rowptr, cols

    def bond_state(self):
        b = np.zeros(self.nnz(), dtype=np.uint8)
        self._chk(ref_lib().ref_rnp_get_bond_state(self.h, abi.ptr(b, C.c_uint8)))
        return b

    def fixity(self):
        f = np.zeros(self.n, dtype=np.uint8)
        self._chk(ref_lib().ref_rnp_get_fixity(self.h, abi.ptr(f, C.c_uint8)))
        return f

    def run(self, nsteps):
        self._chk(ref_lib().ref_rnp_run(self.h, C.c_int64(nsteps)))

    def state(self):
        u = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        self._chk(ref_lib().ref_rnp_get_state(self.h, abi.dptr(u), abi.dptr(v), abi.dptr(f)))
        return u, v, f

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        self._chk(ref_lib().ref_rnp_get_time(self.h, C.byref(t), C.byref(n)))
        return t.value, n.value

    def sc(self, r):
        v = C.c_double()
        self._chk(ref_lib().ref_rnp_sc(self.h, C.c_double(r), C.byref(v)))
        return v.value

    def energies(self):
        """(strain, work, kinetic, fracture) per node from the reference's
        getBondEF, FLoading::apply and computePostProcFields formulas."""
        e = np.zeros((4, self.n), dtype=np.float32)
        self._chk(ref_lib().ref_rnp_energies(self.h, *[abi.ptr(e[q], C.c_float) for q in range(4)]))
        return e

    def reaction_force(self):
        """Reaction_Force (n, 3) from the reference's getBondEF and
        util::geometry::doLinesIntersect."""
        R = np.zeros((self.n, 3))
        self._chk(ref_lib().ref_rnp_reaction_force(self.h, abi.dptr(R)))
        return R


def ref_mesh_volumes(dim, nodes, element_type, elements):
    """The reference's own fe::Mesh::computeVol (mesh.cpp:231-309) on a mesh
    given as nodes (n, 3) and element connectivity (refshim; test use)."""
    x = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
    E = np.ascontiguousarray(elements, dtype=np.int64)
    vol = np.zeros(x.shape[0])
    rc = ref_lib().ref_mesh_volumes(C.c_int(dim), C.c_int64(x.shape[0]), abi.dptr(x),
                                   C.c_int(int(element_type)), C.c_int64(E.shape[0]),
                                   abi.ptr(E, C.c_int64), abi.dptr(vol))
    if rc != 0:
        raise RuntimeError("refshim error: %s" % ref_lib().ref_rnp_last_error().decode())
    return vol
