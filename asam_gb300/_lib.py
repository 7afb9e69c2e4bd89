"""ctypes binding of libasam_gb300.so (the C-ABI declared in include/asam_gb300.h).

The library is built in-tree by :func:`asam_gb300.build.build_library`.  There
is no CPU fallback: if the library or a CUDA device is missing, the calls
raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libasam_gb300.so"

STATUS = {
    0: "ASAM_OK",
    1: "ASAM_NOT_CONVERGED",
    2: "ASAM_BREAKDOWN",
    3: "ASAM_NAN_DETECTED",
    4: "ASAM_BAD_ARG",
    5: "ASAM_CUDA_ERROR",
    6: "ASAM_NO_DEVICE",
    7: "ASAM_IO_ERROR",
    8: "ASAM_UNSUPPORTED",
}
ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN = 0, 1, 2
ASAM_CUDA_ERROR = 5
ASAM_BAD_ARG, ASAM_IO_ERROR, ASAM_UNSUPPORTED = 4, 7, 8


class AsamConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("periodic_x", C.c_int), ("periodic_y", C.c_int), ("periodic_z", C.c_int),
        ("ncomp", C.c_int), ("rho_pos", C.c_int), ("method", C.c_int),
        ("bicgstab_maxiter", C.c_int), ("bicgstab_tol", C.c_double), ("gs_iter", C.c_int),
        ("precision", C.c_int), ("inner_precond", C.c_int), ("inner_gs_iter", C.c_int),
        ("gs_schedule", C.c_int), ("gs_group", C.c_int),
    ]


class AsamProjConfig(C.Structure):
    _fields_ = [
        ("ref_level", C.c_int), ("gauss_iter2", C.c_int), ("gauss_iter3", C.c_int),
        ("mult_iter2", C.c_int), ("mult_iter3", C.c_int), ("step_gmres", C.c_int),
        ("max_restart", C.c_int), ("tol", C.c_double), ("fac_anela", C.c_double), ("prefac2", C.c_double),
    ]


class AsamDynConfig(C.Structure):
    _fields_ = [
        ("th_pos", C.c_int), ("rv_pos", C.c_int), ("rc_pos", C.c_int), ("rr_pos", C.c_int), ("ri_pos", C.c_int),
        ("mom_pos", C.c_int * 6), ("pgradient", C.c_int), ("buoyancy", C.c_int), ("free_slip", C.c_int),
        ("wall_no_slip", C.c_int), ("grav", C.c_double),
    ]


class AsamRestartHeader(C.Structure):
    _fields_ = [("time", C.c_double), ("gmv_step", C.c_int), ("output_time", C.c_double)]


class AsamRestartBlock(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("ncomp", C.c_int), ("nfrac", C.c_int),
                ("c", C.c_void_p), ("uf", C.c_void_p), ("vf", C.c_void_p), ("wf", C.c_void_p)]


class AsamWeight2Block(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("origin", C.c_double * 3),
                ("dx", C.c_void_p), ("dy", C.c_void_p), ("dz", C.c_void_p),
                ("fu", C.c_void_p), ("fv", C.c_void_p), ("fw", C.c_void_p), ("volc", C.c_void_p),
                ("nmid", C.c_int * 3), ("mid_ijk", C.c_void_p * 3), ("mid_xs", C.c_void_p * 3),
                ("nbound", C.c_int), ("struct_bound", C.c_int), ("nsoil", C.c_int),
                ("bound_ijk", C.c_void_p), ("bound_xs", C.c_void_p), ("bound_surf", C.c_void_p),
                ("land_class", C.c_void_p), ("soil_type", C.c_void_p),
                ("normal", C.c_void_p), ("fl", C.c_void_p), ("dl", C.c_void_p)]


class AsamWeight2Options(C.Structure):
    _fields_ = [("periodic", C.c_int * 3), ("nr_soil_layers", C.c_int), ("land_class_def", C.c_int),
                ("real_island", C.c_int), ("expect", C.c_int * 3)]


class AsamTriTbCoefs(C.Structure):
    _fields_ = [("beta0_dtp", C.c_double), ("fac1_l", C.c_double), ("fac1_r", C.c_double),
                ("grav_comp", C.c_double), ("fac_anela", C.c_double), ("fac2_l", C.c_double),
                ("fac2_r", C.c_double), ("fac3_l", C.c_double), ("fac3_r", C.c_double)]


# (name, restype, argtypes) of every exported entry point of include/asam_gb300.h
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p
SIGNATURES = [
    ("asam_create", C.c_int, [C.POINTER(AsamConfig), _V, _V, _V, _V, C.POINTER(C.c_void_p)]),
    ("asam_destroy", C.c_int, [_V]),
    ("asam_set_stream", C.c_int, [_V, _V]),
    ("asam_set_graphs", C.c_int, [_V, C.c_int]),
    ("asam_state_device_ptr", C.c_int, [_V, C.POINTER(C.c_void_p)]),
    ("asam_synchronize", C.c_int, [_V]),
    ("asam_set_velocity", C.c_int, [_V, _V, _V, _V]),
    ("asam_exchange_cell", C.c_int, [_V, C.c_int, _V]),
    ("asam_set_boundary", C.c_int, [_V, C.POINTER(C.c_int)]),
    ("asam_set_boundary_data", C.c_int, [_V, _V, _V, _V]),
    ("asam_boundary_condition", C.c_int, [_V, _V]),
    ("asam_set_diffusion", C.c_int, [_V, _V, _V, C.c_int]),
    ("asam_fcn", C.c_int, [_V, _V, _V]),
    ("asam_div", C.c_int, [_V, _V]),
    ("asam_jac", C.c_int, [_V, _V, C.c_double]),
    ("asam_get_jac", C.c_int, [_V, _V]),
    ("asam_set_jac", C.c_int, [_V, _V]),
    ("asam_matvec", C.c_int, [_V, _V, _V]),
    ("asam_psolve", C.c_int, [_V, _V, _V]),
    ("asam_inner_psolve", C.c_int, [_V, _V, _V]),
    ("asam_bicgstab", C.c_int, [_V, _V, _V, _I, _D]),
    ("asam_ros_step", C.c_int, [_V, _V, C.c_double, _I, _D]),
    ("asam_total_scalar", C.c_int, [_V, _V, C.c_int, _D]),
    ("asam_fcn_tlm", C.c_int, [_V, _V, C.c_int, _V, _V]),
    ("asam_fcn_adj", C.c_int, [_V, _V, C.c_int, _V, _V]),
    ("asam_matvec_adj", C.c_int, [_V, _V, _V]),
    ("asam_bicgstab_adj", C.c_int, [_V, _V, _V, _I, _D]),
    ("asam_ros_step_tlm", C.c_int, [_V, _V, C.c_int, _V, _V, C.c_double, C.c_double]),
    ("asam_ros_step_adj", C.c_int, [_V, _V, C.c_int, _V, _V, C.c_double, C.c_double]),
    ("asam_tracer_gradient", C.c_int, [_V, _V, C.c_int, C.c_int, C.c_double, C.c_int, _V, C.c_double, _D, _V]),
    ("asam_tracer_wind_gradient", C.c_int,
     [_V, _V, C.c_int, C.c_int, C.c_double, C.c_int, _V, C.c_double, _D, _V, _V, _V, _V, _V]),
    ("asam_tri_solve", C.c_int, [C.c_int, C.c_int, _V, _V, _V, _V]),
    ("asam_tri_matvec", C.c_int, [C.c_int, C.c_int, _V, _V, _V, _V, _V]),
    ("asam_tri_tb_compute", C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(AsamTriTbCoefs)] + [_V] * 10),
    ("asam_tri_tb_compute_2d", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(AsamTriTbCoefs)] + [_V] * 16),
    ("asam_tri_tb_compute_3d", C.c_int,
     [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(AsamTriTbCoefs)] + [_V] * 22),
    ("asam_tri_tb_matvec_3d", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int] + [_V] * 9),
    ("asam_tri_tb_gauss_seidel_2d", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int] + [_V] * 7 + [C.c_int]),
    ("asam_tri_tb_restrict_2d", C.c_int, [C.c_int, C.c_int, C.c_int, _V, _V]),
    ("asam_tri_tb_prolong_2d", C.c_int, [C.c_int, C.c_int, C.c_int, _V, _V]),
    ("asam_tri_tb_multigrid_2d", C.c_int, [C.c_int, C.c_int, C.c_int, _V, _V] + [_V] * 7 + [C.c_int, C.c_int]),
    ("asam_tri_tb_multigrid_3d", C.c_int, [C.c_int, C.c_int] + [_V] * 4 + [_V] * 9 + [C.c_int] * 4),
    ("asam_tri_tb_hier_create", C.c_int, [C.c_int] * 5 + [C.POINTER(AsamTriTbCoefs), _V, _V, _V, _V, C.POINTER(_V)]),
    ("asam_tri_tb_hier_get", C.c_int, [_V, C.c_int, C.c_int, C.c_int, _V]),
    ("asam_tri_tb_hier_vcycle", C.c_int, [_V, _V, _V] + [C.c_int] * 4),
    ("asam_tri_tb_hier_set_zebra", C.c_int, [_V, C.c_int]),
    ("asam_tri_tb_hier_destroy", None, [_V]),
    ("asam_tri_tb_solve", C.c_int, [C.c_int, C.c_int, _V, _V, _V, _V]),
    ("asam_tri_tb_matvec", C.c_int, [C.c_int, C.c_int, _V, _V, _V, _V, _V]),
    ("asam_tri_solve_noalloc", C.c_int, [C.c_int, C.c_int, _V, _V, _V, _V, _V]),
    ("asam_proj_setup", C.c_int, [_V, C.POINTER(AsamProjConfig), _V, _V, _V, _V]),
    ("asam_proj_weights", C.c_int, [_V, _V, _V, _V, _V, _V, _V, _V, _V]),
    ("asam_proj_weights_density", C.c_int, [_V, _V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _V]),
    ("asam_proj_get_weights", C.c_long, [_V, C.c_int, _V]),
    ("asam_lapl_compute", C.c_int, [_V, C.c_double, C.c_double]),
    ("asam_lapl_get", C.c_long, [_V, C.c_int, C.c_int, C.c_int, _V]),
    ("asam_lapl_matvec", C.c_int, [_V, _V, _V]),
    ("asam_lapl_vcycle", C.c_int, [_V, _V, _V]),
    ("asam_solve_sound", C.c_int, [_V, _V, _V, _I, _D]),
    ("asam_proj_face_count", C.c_long, [_V]),
    ("asam_proj_matvec1", C.c_int, [_V, _V, _V]),
    ("asam_proj_psolve1", C.c_int, [_V, _V, _V]),
    ("asam_lapl_get_dirichlet", C.c_long, [_V, C.c_int, C.c_int, C.c_int, _V]),
    ("asam_lapl_vcycle_dirichlet", C.c_int, [_V, _V, _V]),
    ("asam_project_vel_face", C.c_int, [_V, _V, _V, _V, _V, _V, C.c_int, C.c_int, _I, C.c_int, _V, _I, _D]),
    ("asam_proj_vcycles", C.c_longlong, [_V]),
    ("asam_proj_set_precision", C.c_int, [_V, C.c_int]),
    ("asam_proj_set_preconditioner", C.c_int, [_V, C.c_int]),
    ("asam_proj_set_pre_schedule", C.c_int, [_V, C.c_int, C.c_int]),
    ("asam_probe_fp64_chain", C.c_int, [C.c_int, C.c_int, C.c_int, _D]),
    ("asam_set_wait_limit", C.c_int, [_V, C.c_int]),
    ("asam_dyn_setup", C.c_int, [_V, C.POINTER(AsamDynConfig), _I, C.c_int, _I, C.c_int]),
    ("asam_face_to_cell", C.c_int, [_V, _V, _V, _V, _V]),
    ("asam_cell_to_face", C.c_int, [_V, _V, _V, _V, _V]),
    ("asam_thermo", C.c_int, [_V, _V, _V, _V]),
    ("asam_fcn_dyn", C.c_int, [_V, _V, _V, _V]),
    ("asam_ros_step_dyn", C.c_int, [_V, _V, C.c_double, _I, _D, _I, _D]),
    ("asam_get_velocity", C.c_int, [_V, _V, _V, _V]),
    ("asam_ros_coeffs", C.c_int, [C.c_int, _D, _D, _D, _D]),
    ("asam_autotune", C.c_int, [_V, _V, C.c_double, _I, _D]),
    ("asam_state_dot", C.c_int, [_V, _V, _D]),
    ("asam_batch_create", C.c_int, [C.c_int, _V, C.c_int, C.POINTER(C.c_void_p)]),
    ("asam_batch_destroy", C.c_int, [_V]),
    ("asam_batch_ros_step", C.c_int, [_V, _V, _D, C.c_int, _I, _D, _I]),
    ("asam_batch_set_graph", C.c_int, [_V, C.c_int]),
    ("asam_npad", C.c_longlong, [C.POINTER(AsamConfig)]),
    ("asam_probe_fp64_fma", C.c_int, [C.c_int, _D]),
    ("asam_launch_count", C.c_longlong, []),
    ("asam_restart_write", C.c_int, [C.c_char_p, C.POINTER(AsamRestartHeader), C.c_int, C.POINTER(AsamRestartBlock)]),
    ("asam_restart_read", C.c_int, [C.c_char_p, C.POINTER(AsamRestartHeader), C.c_int, C.POINTER(AsamRestartBlock)]),
    ("asam_restart_file_name", C.c_int, [C.c_char_p, C.c_int, C.c_char_p, C.c_int]),
    ("asam_restart_set_max_subrecord", C.c_int, [C.c_longlong]),
    ("asam_weight2_open", C.c_int, [C.c_char_p, C.c_int, C.POINTER(AsamWeight2Options), C.POINTER(C.c_void_p),
                                     C.POINTER(AsamWeight2Block)]),
    ("asam_weight2_fetch", C.c_int, [_V, C.POINTER(AsamWeight2Block)]),
    ("asam_weight2_close", None, [_V]),
    ("asam_weight2_write", C.c_int, [C.c_char_p, C.c_int, C.POINTER(AsamWeight2Block), C.POINTER(C.c_int)]),
    ("asam_probe_div", C.c_int, [C.c_longlong, C.c_longlong, C.c_int, C.POINTER(C.c_longlong)]),
    ("asam_last_error", C.c_char_p, []),
]

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with asam_gb300.build.build_library() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class AsamError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = load()
        msg = lib.asam_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)} {msg}")
        self.status = status


def check(status: int, where: str, allow=(ASAM_OK,)) -> int:
    if status not in allow:
        raise AsamError(status, where)
    return status


def ptr(a: np.ndarray) -> int:
    """Address of a C-contiguous float64 array."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 numpy array")
    return a.ctypes.data
