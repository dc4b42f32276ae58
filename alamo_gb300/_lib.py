"""ctypes loader of the in-tree CUDA library ``_build/libagb.so``.

The library is the product: there is no Python or CPU fallback.  If the
shared object is missing, ``lib()`` raises with the build command.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libagb.so")

# every symbol include/agb.h declares
EXPORTS = [
    "agb_default_opts", "agb_elastic_create", "agb_elastic_destroy", "agb_elastic_set_opts",
    "agb_elastic_set_stream", "agb_elastic_set_model", "agb_elastic_get_model", "agb_elastic_set_bc",
    "agb_elastic_prepare", "agb_elastic_num_levels", "agb_elastic_level_dims", "agb_elastic_fapply",
    "agb_elastic_fapply_f32", "agb_elastic_diagonal", "agb_elastic_fsmooth", "agb_elastic_residual",
    "agb_elastic_fsmooth_f32", "agb_elastic_residual_f32", "agb_elastic_residual_dfloat",
    "agb_elastic_restrict", "agb_elastic_prolong_add", "agb_elastic_vcycle", "agb_elastic_bc_init", "agb_elastic_build_rhs",
    "agb_linear_solve", "agb_newton_solve", "agb_elastic_stress_strain", "agb_profile_enable",
    "agb_profile_reset", "agb_profile_get", "agb_profile_bytes", "agb_launch_count", "agb_cubic_stiffness", "agb_synth_uniform",
    "agb_synth_inclusion_iso", "agb_synth_voronoi_cubic", "agb_synth_spheres_iso", "agb_synth_spheres_diffuse",
    "agb_status_string",
    "agb_last_error", "agb_version", "agb_residual_norms_noalloc",
    "agb_unet_create", "agb_unet_destroy", "agb_unet_num_params", "agb_unet_get_params", "agb_unet_set_params",
    "agb_unet_train_step", "agb_unet_predict", "agb_elastic_learned_guess", "agb_conv3_bf16", "agb_conv3_wgrad_bf16",
    "agb_newton_solve_n", "agb_elastic_set_psi", "agb_newton_solve_guess", "agb_elastic_tensor",
    "agb_newton_solve_neohookean", "agb_composite_create", "agb_composite_destroy", "agb_composite_level_dims",
    "agb_composite_set_bc", "agb_composite_set_model", "agb_composite_solve",
]

AGB_OK, AGB_NOT_CONVERGED, AGB_NAN, AGB_BAD_ARG, AGB_CUDA_ERROR, AGB_NOT_READY, AGB_OUT_OF_MEMORY, AGB_LIMIT = range(8)
MEM_HOST, MEM_DEVICE = 0, 1
SYM_ISOTROPIC, SYM_MAJORMINOR, SYM_MAJOR = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1
SOLVER_VCYCLE, SOLVER_FGMRES = 0, 1
BOTTOM_BICGSTAB, BOTTOM_DIRECT, BOTTOM_SMOOTHER = 0, 1, 2
SMOOTHER_JACOBI, SMOOTHER_GS = 0, 1
OUTER_FP64, OUTER_DFLOAT = 0, 1
PRECOND_V, PRECOND_F = 0, 1
K_FAPPLY_F64, K_JACOBI_F64, K_RESIDUAL_F64, K_FAPPLY_F32, K_JACOBI_F32, K_RESIDUAL_F32, K_RESTRICT, K_PROLONG, \
    K_BOTTOM, K_KRYLOV, K_RESIDUAL_DF = range(11)


class SolverOpts(ctypes.Structure):
    """agb_solver_opts (include/agb.h)."""
    _fields_ = [
        ("max_iter", ctypes.c_int),
        ("pre_smooth", ctypes.c_int),
        ("post_smooth", ctypes.c_int),
        ("final_smooth", ctypes.c_int),
        ("bottom_smooth", ctypes.c_int),
        ("bottom_max_iter", ctypes.c_int),
        ("bottom_tol_rel", ctypes.c_double),
        ("bottom_tol_abs", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("max_coarsening_level", ctypes.c_int),
        ("fixed_iter", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("inner_cycles", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("krylov_dim", ctypes.c_int),
        ("inner_tol", ctypes.c_double),
        ("bottom_solver", ctypes.c_int),
        ("fine_kernel", ctypes.c_int),
        ("krylov_reorth", ctypes.c_int),
        ("tma_min_nodes", ctypes.c_int),
        ("max_fmg_iter", ctypes.c_int),
        ("smoother", ctypes.c_int),
        ("outer_residual", ctypes.c_int),
        ("precond_cycle", ctypes.c_int),
    ]


class SolveReport(ctypes.Structure):
    """agb_solve_report (include/agb.h)."""
    _fields_ = [
        ("status", ctypes.c_int),
        ("iters", ctypes.c_int),
        ("nlevels", ctypes.c_int),
        ("bottom_iters", ctypes.c_int),
        ("fp64_residuals", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("resnorm0", ctypes.c_double),
        ("rhsnorm0", ctypes.c_double),
        ("final_resnorm", ctypes.c_double),
        ("final_resnorm_l2", ctypes.c_double),
        ("rhsnorm_l2", ctypes.c_double),
        ("seconds", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


_lib = None


class AgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (status_string(status), msg))
        self.status = status


def lib():
    """Load libagb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libagb.so not built: run `python -m alamo_gb300.build` (needs nvcc)")
        L = ctypes.CDLL(LIB_PATH)
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        L.agb_status_string.restype = ctypes.c_char_p
        L.agb_last_error.restype = ctypes.c_char_p
        L.agb_version.restype = ctypes.c_char_p
        _lib = L
    return _lib


def status_string(s):
    return lib().agb_status_string(int(s)).decode()


def last_error():
    return lib().agb_last_error().decode()


def check(status, allow=(AGB_OK,)):
    if status not in allow:
        raise AgbError(status, last_error())
    return status
