"""ctypes binding of libtopopt_gb300.so (the C ABI in include/topopt_gb300.h).

The shared library is the only compute backend.  Loading fails loudly when it
is missing or was built for another machine; nothing falls back to the CPU.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libtopopt_gb300.so")

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
    4: "linear solve did not converge", 5: "Krylov breakdown", 6: "NaN or Inf encountered",
    7: "call order violated", 8: "device wait timed out",
}


class TopoError(RuntimeError):
    """A non-zero status from the C ABI (the PetscErrorCode of the reference)."""

    def __init__(self, status, where, message=""):
        self.status = status
        super().__init__("%s failed: %s (status %d)%s" % (where, STATUS.get(status, "?"), status,
                                                          (": " + message) if message else ""))


class LEParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("hx", C.c_double), ("hy", C.c_double), ("hz", C.c_double),
        ("nu", C.c_double),
        ("nlvls", C.c_int), ("ncp", C.c_int), ("tsc", C.c_int),
        ("t1", C.c_double),
        ("ti", C.c_int), ("objective", C.c_int), ("sInt", C.c_int), ("mInt", C.c_int),
        ("boundaries", C.c_int), ("loadloc", C.c_int), ("optregion", C.c_int), ("loadsignal", C.c_int),
        ("dalpha", C.c_double), ("dbeta", C.c_double),
        ("mixed", C.c_int), ("rtol", C.c_double), ("maxit", C.c_int), ("smooth", C.c_int),
        ("cheb_ratio", C.c_double), ("use_graphs", C.c_int),
        ("coarse_dense_max", C.c_int), ("coarse_smooth", C.c_int), ("sens_fp32", C.c_int),
        ("inner_tol", C.c_double), ("inner_maxit", C.c_int), ("adaptive_kappa", C.c_double),
        ("extrapolate", C.c_int), ("mass_precond", C.c_int), ("mass_precond_share", C.c_double),
        ("mass_precond_smooth", C.c_int), ("reduction", C.c_int), ("basis", C.c_int), ("omega0", C.c_double),
        ("load2_node", C.c_int), ("load2_phase", C.c_double), ("out_dof", C.c_int),
    ]


class LEStats(C.Structure):
    _fields_ = [("cg_iterations", C.c_longlong), ("solves", C.c_longlong), ("device_bytes", C.c_double),
                ("last_fx", C.c_double), ("graph_body_launches", C.c_longlong), ("mg_solves", C.c_longlong),
                ("step_precond", C.c_int), ("replacements", C.c_longlong)]


EXPORTS = [
    "topo_le_default_params", "topo_le_create", "topo_le_destroy",
    "topo_le_complete_initial_state", "topo_le_complete_initial_state_dev",
    "topo_le_generate_checkpoints",
    "topo_le_compute_objective_sensitivities", "topo_le_compute_objective_sensitivities_dev",
    "topo_le_volume_constraint", "topo_le_volume_constraint_dev",
    "topo_le_get_state", "topo_le_get_checkpoint", "topo_le_set_initial_displacement", "topo_le_get_restart_state", "topo_le_apply_km", "topo_le_get_stats", "topo_le_time_apply",
    "topo_le_kernel_timing", "topo_volume_constraint_noalloc_dev", "topo_le_reduced_system", "topo_vec_scale_dev",
    "topo_box_element_matrices", "topo_sommg_create", "topo_sommg_destroy", "topo_sommg_construct_basis",
    "topo_sommg_get", "topo_sommg_gram_dev",
    "topo_pdefilt_create", "topo_pdefilt_destroy", "topo_pdefilt_filter_project", "topo_pdefilt_filter_project_dev",
    "topo_filter_project", "topo_filter_project_dev", "topo_filter_gradients", "topo_filter_gradients_dev",
    "topo_filter_mnd", "topo_filter_mnd_dev",
    "topo_densfilt_create", "topo_densfilt_destroy", "topo_densfilt_filter_project",
    "topo_densfilt_filter_project_dev", "topo_densfilt_gradients", "topo_densfilt_gradients_dev",
    "topo_densfilt_mnd", "topo_densfilt_mnd_dev",
    "topo_mma_create", "topo_mma_create_restart", "topo_mma_create_restart_dev", "topo_mma_restart",
    "topo_mma_restart_dev", "topo_mma_destroy", "topo_mma_set_asymptotes", "topo_mma_set_outer_movelimit",
    "topo_mma_set_outer_movelimit_dev", "topo_mma_design_change",
    "topo_mma_update", "topo_mma_update_dev", "topo_mma_design_change_dev", "topo_mma_kkt_residual_dev",
    "topo_petsc_vec_write", "topo_petsc_vec_read",
    "topo_mpiio_create", "topo_mpiio_destroy", "topo_mpiio_write", "topo_mpiio_flush", "topo_le_set_output",
    "topo_kernel_launches", "topo_last_error", "topo_status_str",
]

_lib = None


def load(path=None):
    """Load (once) and return the ctypes handle of libtopopt_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libtopopt_gb300.so not found at %s: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)" % p)
    L = C.CDLL(p)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    d = C.c_double
    pp = C.POINTER(C.c_void_p)
    sig = {
        "topo_le_default_params": (None, [C.POINTER(LEParams), ip, ip, ip]),
        "topo_le_create": (ip, [pp, C.POINTER(LEParams)]),
        "topo_le_destroy": (None, [vp]),
        "topo_le_complete_initial_state": (ip, [vp, vp, d, d, d, d, d, d]),
        "topo_le_complete_initial_state_dev": (ip, [vp, vp, d, d, d, d, d, d]),
        "topo_le_generate_checkpoints": (ip, [vp]),
        "topo_le_compute_objective_sensitivities": (ip, [vp, dp, vp]),
        "topo_le_compute_objective_sensitivities_dev": (ip, [vp, dp, vp]),
        "topo_le_volume_constraint": (ip, [vp, dp, vp, vp, d]),
        "topo_le_volume_constraint_dev": (ip, [vp, dp, vp, vp, d]),
        "topo_le_get_checkpoint": (ip, [vp, ip, vp, vp, vp]),
        "topo_le_set_initial_displacement": (ip, [vp, vp, ip]),
        "topo_le_get_restart_state": (ip, [vp, vp, vp, vp]),
        "topo_le_get_state": (ip, [vp, ip, ip, vp]),
        "topo_le_apply_km": (ip, [vp, vp, vp, vp]),
        "topo_le_get_stats": (ip, [vp, C.POINTER(LEStats)]),
        "topo_le_time_apply": (ip, [vp, ip, ip, ip, dp]),
        "topo_le_kernel_timing": (ip, [vp, ip, ip, dp, C.POINTER(C.c_longlong)]),
        "topo_le_reduced_system": (ip, [vp, vp, vp, vp, vp]),
        "topo_volume_constraint_noalloc_dev": (ip, [C.c_longlong, dp, vp, vp, d]),
        "topo_vec_scale_dev": (ip, [vp, C.c_longlong, d]),
        "topo_box_element_matrices": (None, [d, d, d, d, vp, vp]),
        "topo_sommg_create": (ip, [pp, vp, ip]),
        "topo_sommg_destroy": (None, [vp]),
        "topo_sommg_construct_basis": (ip, [vp, d]),
        "topo_sommg_get": (ip, [vp, vp, vp, vp, vp, vp]),
        "topo_sommg_gram_dev": (ip, [vp, C.c_longlong, vp, C.c_longlong, C.c_longlong, ip, vp]),
        "topo_pdefilt_create": (ip, [pp, ip, ip, ip, d, d, d, d, d, ip]),
        "topo_pdefilt_destroy": (None, [vp]),
        "topo_pdefilt_filter_project": (ip, [vp, vp, vp]),
        "topo_pdefilt_filter_project_dev": (ip, [vp, vp, vp]),
        "topo_filter_project": (ip, [vp, vp, vp, vp, ip, d, d]),
        "topo_filter_project_dev": (ip, [vp, vp, vp, vp, ip, d, d]),
        "topo_filter_gradients": (ip, [vp, vp, vp, ip, vp, ip, d, d]),
        "topo_filter_gradients_dev": (ip, [vp, vp, vp, ip, vp, ip, d, d]),
        "topo_filter_mnd": (ip, [vp, vp, dp]),
        "topo_filter_mnd_dev": (ip, [vp, vp, dp]),
        "topo_densfilt_create": (ip, [pp, ip, ip, ip, d, d, d, ip, d]),
        "topo_densfilt_destroy": (None, [vp]),
        "topo_densfilt_filter_project": (ip, [vp, vp, vp, vp, ip, d, d]),
        "topo_densfilt_filter_project_dev": (ip, [vp, vp, vp, vp, ip, d, d]),
        "topo_densfilt_gradients": (ip, [vp, vp, vp, vp, ip, vp, ip, d, d]),
        "topo_densfilt_gradients_dev": (ip, [vp, vp, vp, vp, ip, vp, ip, d, d]),
        "topo_densfilt_mnd": (ip, [vp, vp, dp]),
        "topo_densfilt_mnd_dev": (ip, [vp, vp, dp]),
        "topo_petsc_vec_write": (ip, [C.c_char_p, ip, vp, C.c_longlong, ip]),
        "topo_petsc_vec_read": (ip, [C.c_char_p, ip, vp, C.c_longlong, ip]),
        "topo_mpiio_create": (ip, [pp, ip, ip, ip, dp, ip, C.c_char_p, ip, C.c_char_p, C.c_char_p, ip]),
        "topo_mpiio_destroy": (None, [vp]),
        "topo_mpiio_write": (ip, [vp, C.c_ulonglong, pp, ip, pp, ip, ip, vp]),
        "topo_mpiio_flush": (ip, [vp]),
        "topo_le_set_output": (ip, [vp, vp]),
        "topo_mma_create": (ip, [pp, ip, ip, vp, vp, vp]),
        "topo_mma_create_restart": (ip, [pp, ip, ip, ip, vp, vp, vp, vp, vp, vp, vp]),
        "topo_mma_create_restart_dev": (ip, [pp, ip, ip, ip, vp, vp, vp, vp, vp, vp, vp]),
        "topo_mma_restart": (ip, [vp, vp, vp, vp, vp]),
        "topo_mma_restart_dev": (ip, [vp, vp, vp, vp, vp]),
        "topo_mma_destroy": (None, [vp]),
        "topo_mma_set_asymptotes": (ip, [vp, d, d, d]),
        "topo_mma_set_outer_movelimit": (ip, [vp, d, d, d, vp, vp, vp]),
        "topo_mma_set_outer_movelimit_dev": (ip, [vp, d, d, d, vp, vp, vp]),
        "topo_mma_design_change": (ip, [vp, vp, vp, dp]),
        "topo_mma_update": (ip, [vp, vp, vp, vp, vp, vp, vp]),
        "topo_mma_update_dev": (ip, [vp, vp, vp, vp, vp, vp, vp]),
        "topo_mma_design_change_dev": (ip, [vp, vp, vp, dp]),
        "topo_mma_kkt_residual_dev": (ip, [vp, vp, vp, vp, vp, vp, vp, dp, dp]),
        "topo_kernel_launches": (C.c_longlong, []),
        "topo_last_error": (C.c_char_p, []),
        "topo_status_str": (C.c_char_p, [ip]),
    }
    for name in EXPORTS:
        f = getattr(L, name)  # AttributeError if the library lacks an export
        res, args = sig[name]
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status, where):
    if status != 0:
        msg = load().topo_last_error()
        raise TopoError(status, where, msg.decode() if msg else "")
    return status
