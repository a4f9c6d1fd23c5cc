"""ctypes binding of the C-ABI in include/ouranos_gb300.h.

The shared library is built in-tree by ouranos_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for the operator.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libouranos_gb300.so")

OK = 0
ERR_BAD_INPUT = -1
ERR_CUDA = -2
ERR_TIMEOUT = -3
ERR_UNSUPPORTED = -4
ERR_NO_DEVICE = -5
ERR_NOT_CONVERGED = -6

BC_VACUUM, BC_ISOTROPIC, BC_MOST_NORMAL, BC_REFLECTIVE = 0, 1, 2, 3
QUAD_LS, QUAD_GLC = 0, 1
HARM_ORTHONORMAL, HARM_REFERENCE = 0, 1
FP64, FP32 = 0, 1
FP64_NATIVE, FP64_DF64, FP64_DF64_SWEEP, FP64_DF64_SWEEP_TC = 0, 1, 2, 3
FP32_CONTRACT_CUDA_CORES, FP32_CONTRACT_TENSOR = 0, 1
SOLVER_SI, SOLVER_GMRES, SOLVER_BICGSTAB, SOLVER_FGMRES_MIXED, SOLVER_FGMRES_LEARNED = 0, 1, 2, 3, 4
SOLVER_WARM_START = 0x100
SOLVER_DSA = 0x200

# every symbol include/ouranos_gb300.h declares
EXPORTS = [
    "ouranos_quadrature_sizes", "ouranos_quadrature_build",
    "ouranos_rt_create", "ouranos_rt_destroy", "ouranos_rt_set_group",
    "ouranos_rt_set_precision", "ouranos_rt_set_fp64_contractions", "ouranos_rt_set_fp32_contractions", "ouranos_rt_vector_length", "ouranos_rt_n_tasks",
    "ouranos_rt_scattering_source", "ouranos_rt_sweep", "ouranos_rt_apply",
    "ouranos_rt_sweep_rhs", "ouranos_rt_task_levels", "ouranos_wavefront_levels",
    "ouranos_rt_set_stream", "ouranos_rt_last_error",
    "ouranos_rt_last_sweep_ms", "ouranos_rt_set_tiling", "ouranos_rt_get_tiling",
    "ouranos_rt_set_wait_limit", "ouranos_rt_debug_wait_bias", "ouranos_solve",
    "ouranos_rt_apply_noalloc",
    "ouranos_cnn_create", "ouranos_cnn_destroy", "ouranos_cnn_n_params", "ouranos_cnn_get_params",
    "ouranos_cnn_set_params", "ouranos_cnn_forward", "ouranos_cnn_gradients",
    "ouranos_cnn_train_step", "ouranos_cnn_last_error", "ouranos_rt_set_preconditioner",
    "ouranos_rt_pc_features", "ouranos_rt_pc_target", "ouranos_rt_pc_apply", "ouranos_rt_pc_dsa_apply",
    "ouranos_batch_create", "ouranos_batch_destroy", "ouranos_batch_layout", "ouranos_batch_apply",
    "ouranos_batch_rhs", "ouranos_batch_solve", "ouranos_batch_autotune", "ouranos_batch_set_graphs",
    "ouranos_batch_stats", "ouranos_batch_last_error",
    "ouranos_rt_set_time_step", "ouranos_rt_set_source", "ouranos_rt_time_advance",
    "ouranos_rt_get_angular_flux", "ouranos_rt_set_angular_flux",
    "ouranos_rt_set_dsa", "ouranos_rt_dsa_apply", "ouranos_solve_multigroup", "ouranos_batch_set_dsa",
    "ouranos_batch_dsa_apply",
]


class ProblemDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("fe_order", C.c_int), ("n_cells", C.c_int * 3),
        ("lower", C.c_double * 3), ("upper", C.c_double * 3), ("n_groups", C.c_int),
        ("n_dir", C.c_int), ("n_mom", C.c_int),
        ("omega", C.c_void_p), ("m2d", C.c_void_p), ("d2m", C.c_void_p),
        ("moment_l", C.c_void_p), ("most_normal", C.c_void_p), ("weight_sum", C.c_double),
        ("n_materials", C.c_int), ("l_max", C.c_int),
        ("sigma_t", C.c_void_p), ("sigma_s", C.c_void_p),
        ("material_id", C.c_void_p), ("source_id", C.c_void_p),
        ("n_sources", C.c_int), ("source", C.c_void_p),
        ("bc_type", C.c_int * 6), ("inc_flux", C.c_void_p), ("cell_order", C.c_void_p),
    ]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("restarts", C.c_int), ("residual", C.c_double),
                ("seconds", C.c_double), ("converged", C.c_int)]


class MultigroupInfo(C.Structure):
    _fields_ = [("outer_iterations", C.c_int), ("inner_iterations", C.c_int), ("change", C.c_double),
                ("seconds", C.c_double), ("converged", C.c_int)]


class OuranosError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ouranos error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("ouranos_gb300 native library missing at %s; run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i, d, l, sz = C.c_void_p, C.c_int, C.c_double, C.c_long, C.c_size_t
    sig = {
        "ouranos_quadrature_sizes": [i, i, i, i, C.POINTER(i), C.POINTER(i)],
        "ouranos_quadrature_build": [i, i, i, i, d, i, i, vp, vp, vp, vp, vp, vp],
        "ouranos_rt_create": [C.POINTER(ProblemDesc), i, C.POINTER(vp)],
        "ouranos_rt_destroy": [vp],
        "ouranos_rt_set_group": [vp, i],
        "ouranos_rt_set_precision": [vp, i],
        "ouranos_rt_set_fp64_contractions": [vp, i],
        "ouranos_rt_set_fp32_contractions": [vp, i],
        "ouranos_rt_vector_length": [vp, C.POINTER(l)],
        "ouranos_rt_n_tasks": [vp, C.POINTER(l)],
        "ouranos_rt_scattering_source": [vp, vp],
        "ouranos_rt_sweep": [vp, vp, vp],
        "ouranos_rt_apply": [vp, vp, vp],
        "ouranos_rt_sweep_rhs": [vp, vp, vp],
        "ouranos_rt_task_levels": [vp, vp],
        "ouranos_wavefront_levels": [i, vp, i, vp, vp],
        "ouranos_rt_set_stream": [vp, vp],
        "ouranos_rt_last_error": [vp, C.c_char_p, sz],
        "ouranos_rt_last_sweep_ms": [vp, C.POINTER(d), C.POINTER(i)],
        "ouranos_rt_set_tiling": [vp, i, i, i],
        "ouranos_rt_get_tiling": [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)],
        "ouranos_rt_set_wait_limit": [vp, d],
        "ouranos_rt_debug_wait_bias": [vp, i],
        "ouranos_solve": [vp, i, i, i, d, vp, vp, vp, C.POINTER(SolveInfo)],
        "ouranos_rt_apply_noalloc": [vp, vp, vp],
        "ouranos_batch_create": [C.POINTER(ProblemDesc), i, i, C.POINTER(vp)],
        "ouranos_batch_destroy": [vp],
        "ouranos_batch_layout": [vp, C.POINTER(i), C.POINTER(l), vp],
        "ouranos_batch_apply": [vp, i, vp, vp],
        "ouranos_batch_rhs": [vp, vp],
        "ouranos_batch_solve": [vp, i, i, i, d, vp, vp],
        "ouranos_batch_autotune": [vp, i, i, vp],
        "ouranos_batch_set_graphs": [vp, i],
        "ouranos_batch_stats": [vp, C.POINTER(d), C.POINTER(i)],
        "ouranos_batch_last_error": [vp, C.c_char_p, sz],
        "ouranos_rt_set_time_step": [vp, d],
        "ouranos_rt_set_source": [vp, vp],
        "ouranos_rt_time_advance": [vp, i, i, i, d, vp, C.POINTER(SolveInfo)],
        "ouranos_rt_get_angular_flux": [vp, vp],
        "ouranos_rt_set_angular_flux": [vp, vp],
        "ouranos_rt_set_dsa": [vp, i],
        "ouranos_rt_dsa_apply": [vp, vp, vp],
        "ouranos_solve_multigroup": [vp, i, i, i, d, i, d, vp, C.POINTER(MultigroupInfo)],
        "ouranos_batch_set_dsa": [vp, i],
        "ouranos_batch_dsa_apply": [vp, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = i
    _lib = L
    return L


def last_error(handle):
    buf = C.create_string_buffer(512)
    if handle:
        lib().ouranos_rt_last_error(handle, buf, 512)
    return buf.value.decode(errors="replace")


def check(rc, handle=None):
    if rc != OK:
        raise OuranosError(rc, last_error(handle) if handle else "")
    return rc
