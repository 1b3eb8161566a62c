"""ctypes binding of the C ABI declared in include/mstcfd.h.

Loads the in-tree ``lib/libmstcfd.so`` (building it first when it is missing
and nvcc is available).  There is no fallback: if the library cannot be
loaded, every entry point raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)

OK, EINVAL, EMESH, ECUDA, EDIVERGED, ETIMEOUT, ENOMEM, EUNSUPPORTED = range(8)
FLUX_AUSM, FLUX_ROE = 0, 1
LIMITER_NONE, LIMITER_MINMOD, LIMITER_VANLEER, LIMITER_VANALBADA = range(4)
PREC_FP64_EXACT, PREC_FP64, PREC_FP32 = range(3)
LU_ILUSGS, LU_GS = range(2)
TIME_EULER, TIME_RK2 = range(2)
DT_FIXED, DT_CFL_GLOBAL, DT_CFL_LOCAL = range(3)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint8)


class Params(C.Structure):
    _fields_ = [("flux", C.c_int), ("order", C.c_int), ("limiter", C.c_int),
                ("precision", C.c_int), ("time_scheme", C.c_int),
                ("dt_mode", C.c_int), ("dt", C.c_double), ("cfl", C.c_double),
                ("inlet_q", C.c_double * 4), ("reference_quirks", C.c_int),
                ("viscous", C.c_int), ("mu", C.c_double), ("lambda_", C.c_double),
                ("kappa", C.c_double), ("cv", C.c_double), ("reserved", C.c_int * 6)]


class MeshDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("node_xy", _dp), ("n_cells", C.c_int),
                ("n_faces", C.c_int), ("face_nodes", _ip), ("face_cells", _ip),
                ("n_zones", C.c_int), ("zones", _ip), ("c1_shift", _dp)]


class Mesh3DInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in (
        "n_nodes", "n_cells", "n_faces", "n_int_faces", "n_zones", "n_face_nodes",
        "n_cell_faces", "n_cell_nodes", "n_inner", "n_bond1", "n_bond2")]


class Mesh3DArrays(C.Structure):
    _fields_ = [("node_xyz", _dp), ("face_ptr", _ip), ("face_nodes", _ip), ("face_cells", _ip),
                ("face_type", _ip), ("face_ctr", _dp), ("face_dir", _dp), ("face_area", _dp),
                ("face_eta0", _dp), ("face_cmd", _dp), ("face_dac", _ip), ("face_flag", _up),
                ("face_flag_set", _up), ("cell_ptr", _ip), ("cell_faces", _ip),
                ("cell_nb", _ip), ("cell_dof", _dp), ("cell_eta0c", _dp), ("cell_ctr", _dp),
                ("cell_vol", _dp), ("cell_vol_fixed", _dp), ("cell_node_ptr", _ip),
                ("cell_nodes", _ip), ("inner", _ip), ("bond1", _ip), ("bond2", _ip),
                ("cell_n_lower", _ip)]


class Params3D(C.Structure):
    _fields_ = [("precision", C.c_int), ("order", C.c_int), ("limiter", C.c_int),
                ("viscous", C.c_int), ("mu", C.c_double), ("lambda_", C.c_double),
                ("kappa", C.c_double), ("cv", C.c_double), ("inlet_q", C.c_double * 5),
                ("cfl", C.c_double)]


class Ctx3DInfo(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("n_tiles", C.c_int),
                ("max_tile_faces", C.c_int), ("n_cell_faces", C.c_int), ("n_borrowed", C.c_int),
                ("device_bytes", C.c_size_t)]


class CaseParams(C.Structure):
    _fields_ = [("inlet_q", C.c_double * 4), ("mu", C.c_double), ("lambda_", C.c_double),
                ("kappa", C.c_double), ("cv", C.c_double)]


class ImplicitParams(C.Structure):
    _fields_ = [("cfl0", C.c_double), ("cfl_max", C.c_double), ("omega", C.c_double),
                ("tol", C.c_double), ("freeze_tol", C.c_double), ("fp32_until", C.c_double),
                ("max_iter", C.c_int), ("graph_iters", C.c_int),
                ("autotune", C.c_int), ("sweep_fp32", C.c_int), ("p_floor", C.c_double),
                ("fp32_window", C.c_int), ("refreeze_window", C.c_int),
                ("stall_window", C.c_int), ("restart_after", C.c_int),
                ("restart_projected", C.c_int)]


class BatchInfo(C.Structure):
    _fields_ = [("n_cases", C.c_int), ("n_cells", C.c_int), ("n_faces", C.c_int),
                ("n_colors", C.c_int), ("sweep_threads", C.c_int), ("graph_iters", C.c_int)]


class BatchResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("total_iterations", C.c_int),
                ("n_converged", C.c_int), ("ms", C.c_double), ("n_diverged", C.c_int),
                ("n_stalled", C.c_int), ("n_restarted", C.c_int)]


CASE_DIVERGED = -2  # mst_batch_case_status: the case was retired as diverged
CASE_STALLED = -3   # ... retired by the stall_window test


class MeshInfo(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "n_nodes", "n_cells", "n_faces", "n_int_faces", "n_zones",
        "n_cell_faces", "n_inner", "n_bond1", "n_bond2", "n_tiles", "n_borrowed", "n_halo",
        "n_halo_cells", "n_halo_cell_faces")]


class MeshArrays(C.Structure):
    _fields_ = [("face_ctr", _dp), ("face_dir", _dp), ("face_area", _dp),
                ("face_eta0", _dp), ("face_dac", _ip), ("face_flag", _up),
                ("face_cells", _ip), ("cell_ptr", _ip), ("cell_faces", _ip),
                ("cell_nb", _ip), ("cell_dof", _dp), ("cell_eta0c", _dp),
                ("cell_ctr", _dp), ("cell_vol", _dp), ("inner", _ip),
                ("bond1", _ip), ("bond2", _ip), ("cell_perm", _ip),
                ("face_perm", _ip)]


class Norms(C.Structure):
    _fields_ = [("linf_change", C.c_double * 4), ("l2_resid", C.c_double * 4),
                ("dt", C.c_double), ("time", C.c_double), ("mass", C.c_double)]


class SimpleParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("alpha_p", C.c_double), ("n_inner", C.c_int),
                ("wall_smooth", C.c_int), ("inlet", C.c_double * 4), ("p_out", C.c_double),
                ("cluster", C.c_int), ("reserved", C.c_int * 3)]


class SimpleInfo(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("cluster", C.c_int),
                ("threads", C.c_int), ("momentum_levels", C.c_int),
                ("pressure_levels", C.c_int), ("last_steps", C.c_int),
                ("batch_cluster", C.c_int)]


class MstError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"mstcfd status {status}: {msg}")
        self.status = status


_lib = None


def lib_path():
    return os.path.join(_PKG, "lib", "libmstcfd.so")


def load():
    """Load (building if needed) the CUDA library; raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "_mstcfd_build", os.path.join(_PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(path)
    sigs = {
        "mst_params_default": (None, [C.POINTER(Params)]),
        "mst_mesh_read_msh": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
        "mst_mesh_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(C.c_void_p)]),
        "mst_mesh_destroy": (None, [C.c_void_p]),
        "mst_mesh_get_info": (C.c_int, [C.c_void_p, C.POINTER(MeshInfo)]),
        "mst_mesh_get_arrays": (C.c_int, [C.c_void_p, C.POINTER(MeshArrays)]),
        "mst_ctx_create": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(C.c_void_p)]),
        "mst_ctx_destroy": (C.c_int, [C.c_void_p]),
        "mst_ctx_set_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
        "mst_set_dt": (C.c_int, [C.c_void_p, C.c_double]),
        "mst_set_state": (C.c_int, [C.c_void_p, _dp, C.c_size_t]),
        "mst_get_state": (C.c_int, [C.c_void_p, _dp, C.c_size_t]),
        "mst_get_new_state": (C.c_int, [C.c_void_p, _dp, C.c_size_t]),
        "mst_solve": (C.c_int, [C.c_void_p]),
        "mst_update_new_to_old": (C.c_int, [C.c_void_p]),
        "mst_get_residual": (C.c_int, [C.c_void_p, _dp, C.c_size_t]),
        "mst_get_face_flux": (C.c_int, [C.c_void_p, _dp]),
        "mst_get_gradient": (C.c_int, [C.c_void_p, _dp]),
        "mst_step": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(Norms)]),
        "mst_get_time": (C.c_int, [C.c_void_p, _dp]),
        "mst_last_timing": (C.c_int, [C.c_void_p, _dp, _ip]),
        "mst_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
        "mst_profile_reset": (C.c_int, [C.c_void_p]),
        "mst_profile_count": (C.c_int, [C.c_void_p]),
        "mst_profile_get": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t,
                                      _ip, _dp]),
        "mst_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
        "mst_host_free": (C.c_int, [C.c_void_p]),
        "mst_device_count": (C.c_int, [_ip]),
        "mst_set_device": (C.c_int, [C.c_int]),
        "mst_probe_fp64_rate": (C.c_int, [_dp]),
        "mst_set_wait_limit": (C.c_int, [C.c_longlong]),
        "mst_step_host_jobs": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p),
                                         C.POINTER(C.c_void_p), C.c_int]),
        "mst_solve_device_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p]),
        "mst_node_values": (C.c_int, [C.c_void_p, _dp, _dp]),
        "mst_write_plt": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
        "mst_write_cell_text": (C.c_int, [C.c_void_p, C.c_char_p]),
        "mst_read_cell_text": (C.c_int, [C.c_void_p, C.c_char_p]),
        "mst_checkpoint_save": (C.c_int, [C.c_void_p, C.c_char_p]),
        "mst_checkpoint_load": (C.c_int, [C.c_void_p, C.c_char_p]),
        "mst_implicit_params_default": (None, [C.POINTER(ImplicitParams)]),
        "mst_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(CaseParams), C.c_int,
                                       C.POINTER(Params), C.POINTER(ImplicitParams),
                                       C.POINTER(C.c_void_p)]),
        "mst_batch_destroy": (C.c_int, [C.c_void_p]),
        "mst_batch_info": (C.c_int, [C.c_void_p, C.POINTER(BatchInfo)]),
        "mst_batch_colors": (C.c_int, [C.c_void_p, _ip]),
        "mst_batch_set_state": (C.c_int, [C.c_void_p, _dp]),
        "mst_batch_set_l2_ref": (C.c_int, [C.c_void_p, _dp]),
        "mst_batch_get_state": (C.c_int, [C.c_void_p, _dp]),
        "mst_batch_iterate": (C.c_int, [C.c_void_p, C.c_int]),
        "mst_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(BatchResult)]),
        "mst_batch_case_status": (C.c_int, [C.c_void_p, _ip, _dp, _dp]),
        "mst_batch_set_fallback": (C.c_int, [C.c_void_p, _dp]),
        "mst_batch_restart": (C.c_int, [C.c_void_p, _ip, C.c_int]),
        "mst_batch_case_restarts": (C.c_int, [C.c_void_p, _ip]),
        "mst_tc_gemm_check": (C.c_int, [C.POINTER(C.c_uint16), C.POINTER(C.c_uint16), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int]),
        "mst_mpnn_num_params": (C.c_int, []),
        "mst_mpnn_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
        "mst_mpnn_destroy": (C.c_int, [C.c_void_p]),
        "mst_mpnn_set_graph": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_float), _ip, _ip]),
        "mst_mpnn_set_targets": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "mst_mpnn_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "mst_mpnn_backward": (C.c_int, [C.c_void_p, _dp]),
        "mst_mpnn_get": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_float)]),
        "mst_mpnn_set_weights": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
        "mst_mpnn_adam_step": (C.c_int, [C.c_void_p, C.c_float]),
        "mst_mpnn_profile": (C.c_int, [C.c_void_p, C.c_int]),
        "mst_mpnn_profile_read": (C.c_int, [C.c_void_p, _dp]),
        "mst_mesh3d_read_msh": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
        "mst_mesh3d_get_info": (C.c_int, [C.c_void_p, C.POINTER(Mesh3DInfo)]),
        "mst_mesh3d_get_arrays": (C.c_int, [C.c_void_p, C.POINTER(Mesh3DArrays)]),
        "mst_mesh3d_destroy": (None, [C.c_void_p]),
        "mst_mesh3d_from_arrays": (C.c_int, [C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, _ip,
                                             C.c_int, _ip, _dp, C.POINTER(C.c_void_p)]),
        "mst_params3d_default": (None, [C.POINTER(Params3D)]),
        "mst_ctx3d_create": (C.c_int, [C.c_void_p, C.POINTER(Params3D), C.POINTER(C.c_void_p)]),
        "mst_ctx3d_destroy": (C.c_int, [C.c_void_p]),
        "mst_ctx3d_info_get": (C.c_int, [C.c_void_p, C.POINTER(Ctx3DInfo)]),
        "mst_ctx3d_set_state": (C.c_int, [C.c_void_p, _dp]),
        "mst_ctx3d_get_state": (C.c_int, [C.c_void_p, _dp]),
        "mst_ctx3d_residual": (C.c_int, [C.c_void_p, _dp]),
        "mst_ctx3d_gradient": (C.c_int, [C.c_void_p, _dp]),
        "mst_ctx3d_step": (C.c_int, [C.c_void_p, C.c_int, C.c_double, _dp]),
        "mst_ctx3d_last_timing": (C.c_int, [C.c_void_p, _dp, _ip]),
        "mst_ctx3d_kinetic_energy": (C.c_int, [C.c_void_p, _dp, _dp]),
        "mst_ctx3d_profile": (C.c_int, [C.c_void_p, C.c_int]),
        "mst_ctx3d_profile_count": (C.c_int, [C.c_void_p]),
        "mst_ctx3d_profile_get": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t, _ip,
                                            _dp]),
        "mst_lu_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip, _ip, _dp,
                                    C.POINTER(C.c_void_p)]),
        "mst_lu_solve": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _ip]),
        "mst_lu_levels": (C.c_int, [C.c_void_p, _ip, _ip]),
        "mst_lu_destroy": (C.c_int, [C.c_void_p]),
        "mst_simple_default_params": (C.c_int, [C.POINTER(SimpleParams)]),
        "mst_q_to_puvt": (C.c_int, [C.c_int, _dp, _dp]),
        "mst_simple_create": (C.c_int, [C.c_void_p, C.POINTER(SimpleParams),
                                        C.POINTER(C.c_void_p)]),
        "mst_simple_set_state": (C.c_int, [C.c_void_p, _dp, _dp]),
        "mst_simple_get_state": (C.c_int, [C.c_void_p, _dp, _dp]),
        "mst_simple_step": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "mst_simple_rows": (C.c_int, [C.c_void_p, _dp, _ip]),
        "mst_simple_step_batch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, _dp]),
        "mst_simple_get_info": (C.c_int, [C.c_void_p, C.POINTER(SimpleInfo)]),
        "mst_simple_destroy": (C.c_int, [C.c_void_p]),
        "mst_last_error": (C.c_char_p, []),
        "mst_abi_version": (C.c_int, []),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != OK:
        raise MstError(status, load().mst_last_error().decode(errors="replace"))


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def params(**kw):
    """mst_params with the reference defaults, overridden by keywords."""
    p = Params()
    load().mst_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "inlet_q":
            for i in range(4):
                p.inlet_q[i] = float(v[i])
        elif not hasattr(p, k):
            raise KeyError(k)
        else:
            setattr(p, k, v)
    return p


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a
