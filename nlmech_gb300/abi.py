"""ctypes mirror of include/nlmgpu.h.

Only plain data: the structs that describe a peridynamics model and the enum
values.  Field order and types must match the C header exactly.
"""
import ctypes as C

# status codes
NLM_OK = 0
NLM_ERR_INVALID = 1
NLM_ERR_CUDA = 2
NLM_ERR_OOM = 3
NLM_ERR_TIMEOUT = 4
NLM_ERR_UNSUPPORTED = 5
NLM_ERR_STATE = 6
NLM_ERR_NONFINITE = 7

# material kinds
RNP_BOND = 0
ELASTIC_STATE = 1
# precision
FP64 = 0
FP32C = 1
# integration scheme
VELOCITY_VERLET = 0
CENTRAL_DIFFERENCE = 1
# decomposition
DECOMP_AUTO = 0
DECOMP_THREAD = 1
DECOMP_WARP = 2
DECOMP_THREAD1 = 3
DECOMP_TILE = 4
DECOMP_TILE_LOCAL = 5
# regions
REGION = {"rectangle": 0, "line": 1, "circle": 2, "torus": 3, "cuboid": 4,
          "angled_rectangle": 5}
TIME_FN = {"constant": 0, "linear": 1, "quadratic": 2, "sin": 3,
           "linear_step": 4, "linear_slow_fast": 5}
SPATIAL_FN = {"constant": 0, "sin_x": 1, "sin_y": 2, "sin_z": 3,
              "linear_x": 4, "linear_y": 5, "linear_z": 6,
              "hat_x": 7, "hat_y": 8, "hat_z": 9, "line_load": 10}
CRACK_EDGE = 0
CRACK_PLANE = 1
NOFAIL_OFF = 0
NOFAIL_COMPUTE = 1
NOFAIL_DATA = 2


class BCSet(C.Structure):
    _fields_ = [
        ("region", C.c_int),
        ("x1", C.c_double), ("x2", C.c_double),
        ("y1", C.c_double), ("y2", C.c_double),
        ("z1", C.c_double), ("z2", C.c_double),
        ("r1", C.c_double), ("r2", C.c_double),
        ("dir_mask", C.c_int),
        ("time_fn", C.c_int),
        ("time_params", C.c_double * 4),
        ("spatial_fn", C.c_int),
        ("spatial_params", C.c_double * 2),
        ("theta", C.c_double),
    ]


class Crack(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("orientation", C.c_int),
        ("pb", C.c_double * 2),
        ("pt", C.c_double * 2),
        ("theta", C.c_double),
        ("z0", C.c_double),
        ("lo", C.c_double * 2),
        ("hi", C.c_double * 2),
        ("timed", C.c_int),
        ("activation_time", C.c_double),
    ]


class NoFailRegion(C.Structure):
    _fields_ = [("kind", C.c_int), ("params", C.c_double * 4)]


NOFAIL_CIRCLE = 0
NOFAIL_RECTANGLE = 1


class Material(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("density", C.c_double),
        ("E", C.c_double), ("G", C.c_double), ("K", C.c_double),
        ("Gc", C.c_double), ("KIc", C.c_double),
        ("plane_strain", C.c_int),
        ("influence_type", C.c_int),
        ("n_influence_params", C.c_int),
        ("influence_params", C.c_double * 2),
        ("irreversible", C.c_int),
        ("check_sc_factor", C.c_double),
        ("compute_from_classical", C.c_int),
        ("bond_params", C.c_double * 2),
        ("es_sc", C.c_double),
        ("es_ref_compat", C.c_int),
        ("apply_contact", C.c_int),
    ]


class FDDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("n_nodes", C.c_int64),
        ("x", C.POINTER(C.c_double)),
        ("volume", C.POINTER(C.c_double)),
        ("horizon", C.c_double),
        ("mesh_size", C.c_double),
        ("material", Material),
        ("n_ubc", C.c_int),
        ("ubc", C.POINTER(BCSet)),
        ("n_fbc", C.c_int),
        ("fbc", C.POINTER(BCSet)),
        ("n_cracks", C.c_int),
        ("cracks", C.POINTER(Crack)),
        ("no_fail", C.c_int),
        ("no_fail_tol", C.c_double),
        ("dt", C.c_double),
        ("scheme", C.c_int),
        ("precision", C.c_int),
        ("decomposition", C.c_int),
        ("u0", C.POINTER(C.c_double)),
        ("v0", C.POINTER(C.c_double)),
        ("n_nofail_regions", C.c_int),
        ("nofail_regions", C.POINTER(NoFailRegion)),
    ]


def dptr(a):
    """Pointer to the data of a C-contiguous float64 numpy array (or NULL)."""
    if a is None:
        return C.POINTER(C.c_double)()
    assert a.dtype.name == "float64" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ptr(a, ctype):
    if a is None:
        return C.POINTER(ctype)()
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


class QSParams(C.Structure):
    _fields_ = [
        ("max_newton", C.c_int),
        ("tol", C.c_double),
        ("lin_max_iters", C.c_int),
        ("lin_tol", C.c_double),
        ("break_bonds", C.c_int),
        ("max_break_rounds", C.c_int),
        ("guess_accept", C.c_double),
        ("krylov_launch", C.c_int),
        ("wait_limit_s", C.c_double),
        ("barrier_extra", C.c_int),
        ("lin_tol_gamma", C.c_double),
    ]


class ESQSParams(C.Structure):
    """nlm_esqs_params: the quasi-static ElasticState solver (Solver deck)."""
    _fields_ = [
        ("jacobian", C.c_int),
        ("max_iters", C.c_int),
        ("tol", C.c_double),
        ("tol_relative", C.c_int),
        ("perturbation", C.c_double),
        ("lin_max_iters", C.c_int),
        ("lin_tol", C.c_double),
        ("dt", C.c_double),
    ]


class QSStats(C.Structure):
    _fields_ = [
        ("newton_iters", C.c_int),
        ("lin_iters", C.c_int),
        ("break_rounds", C.c_int),
        ("used_guess", C.c_int),
        ("broken", C.c_int64),
        ("res_plain", C.c_double),
        ("res_start", C.c_double),
        ("res_final", C.c_double),
        ("ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}
