"""ctypes binding of liblvgpu.so (declarations in include/lvgpu.h).

The library is the only compute path of this package: when it is missing or
fails to load, every entry point raises instead of falling back to anything.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblvgpu.so")

LV_OK = 0
LV_ERR = {
    1: "NAN_VELOCITY", 2: "MESH_DESTROYED", 3: "EDGE_OVERFLOW", 4: "CELL_OVERFLOW", 5: "CG_MAXITER",
    6: "BAD_ARGUMENT", 7: "CUDA", 8: "NOT_MESHED", 9: "LEARNED_WORSE", 10: "NONFINITE_POSITION",
    11: "BARRIER_TIMEOUT",
}
LV_MAX_EDGES = 20

FIELDS = {"x": (0, 2), "v": (1, 2), "e": (2, 1), "P": (3, 1), "rho": (4, 1), "c2": (5, 1), "dv": (6, 2),
          "mass": (7, 1), "momentum": (8, 2), "energy": (9, 1), "phase": (10, 1), "quality": (11, 1),
          "D": (12, 4), "mu": (13, 1), "T": (14, 1), "k": (15, 1), "cV": (16, 1), "area": (20, 1),
          "centroid": (21, 2)}

METHODS = {"jacobi_pcg": 0, "mixed_ir": 1, "learned_pcg": 2, "minres": 3}


class LvParams(C.Structure):
    _fields_ = [("xmin", C.c_double * 2), ("xmax", C.c_double * 2), ("dr", C.c_double), ("h", C.c_double),
                ("r_max", C.c_double), ("xperiodic", C.c_int32), ("yperiodic", C.c_int32),
                ("capacity", C.c_int32), ("device", C.c_int32)]


class LvSolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("outer", C.c_int32), ("method", C.c_int32),
                ("rel_residual", C.c_double)]


# name -> (restype, argtypes); every symbol include/lvgpu.h declares
_vp, _d, _i32, _i64 = C.c_void_p, C.c_double, C.c_int32, C.c_int64
_pd, _pi32, _pi64 = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
_pst = C.POINTER(LvSolveStats)
SIGNATURES = {
    "lv_create": (_vp, [C.POINTER(LvParams)]),
    "lv_destroy": (C.c_int, [_vp]),
    "lv_last_error": (C.c_char_p, [_vp]),
    "lv_status": (C.c_int, [_vp]),
    "lv_synchronize": (C.c_int, [_vp]),
    "lv_set_positions": (C.c_int, [_vp, _i32, _pd]),
    "lv_num_particles": (_i32, [_vp]),
    "lv_set_field": (C.c_int, [_vp, _i32, _pd]),
    "lv_get_field": (C.c_int, [_vp, _i32, _pd]),
    "lv_set_fields": (C.c_int, [_vp, _i32, _pi32, C.POINTER(C.c_void_p)]),
    "lv_get_fields": (C.c_int, [_vp, _i32, _pi32, C.POINTER(C.c_void_p)]),
    "lv_field_device_ptr": (_vp, [_vp, _i32]),
    "lv_remesh": (C.c_int, [_vp]),
    "lv_remesh_async": (C.c_int, [_vp]),
    "lv_get_geometry": (C.c_int, [_vp, _pi32, _pd, _pi32]),
    "lv_get_faces": (C.c_int, [_vp, _pi64, _pi64, _pi32, _pd, _pd, _pd, _pd]),
    "lv_get_cell_list": (C.c_int, [_vp, _pi64, _pi64, _pi32, _pi32]),
    "lv_move": (C.c_int, [_vp, _d]),
    "lv_ideal_eos": (C.c_int, [_vp, _d, _d]),
    "lv_stiffened_eos": (C.c_int, [_vp, _d, _d]),
    "lv_find_rho": (C.c_int, [_vp]),
    "lv_gravity_step": (C.c_int, [_vp, _d, _d, _d]),
    "lv_pressure_step": (C.c_int, [_vp, _d]),
    "lv_find_D": (C.c_int, [_vp]),
    "lv_viscous_step": (C.c_int, [_vp, _d, _i32]),
    "lv_bdary_friction": (C.c_int, [_vp, _pd, _d]),
    "lv_find_dv": (C.c_int, [_vp, _d, _d]),
    "lv_relaxation_step": (C.c_int, [_vp, _d, _i32]),
    "lv_set_solver": (C.c_int, [_vp, _i32, _d, _i32]),
    "lv_find_pressure": (C.c_int, [_vp, _d, _i32, _pd, _pst]),
    "lv_pressure_operator": (C.c_int, [_vp, _d]),
    "lv_pressure_rhs": (C.c_int, [_vp, _d, _i32, _pd]),
    "lv_export_system": (C.c_int, [_vp, _pi64, _pd, _pi64, _pi32, _pd, _pd]),
    "lv_solve": (C.c_int, [_vp, _pd, _pd, _pst]),
    "lv_operator_apply": (C.c_int, [_vp, _pd, _pd]),
    "lv_multiphase_projection": (C.c_int, [_vp, _d, _pst]),
    "lv_learn_set_pattern": (C.c_int, [_vp, _i32]),
    "lv_learn_get_pattern": (C.c_int32, [_vp]),
    "lv_learn_factor2": (C.c_int, [_vp, _pi64, _pi64, _pi32, C.POINTER(C.c_float)]),
    "lv_nearest_polygon": (C.c_int, [_vp, _i32, _pd, _pi32]),
    "lv_movingls": (C.c_int, [_vp, _i32, _i32, _pi32, _pd, _d, _pd]),
    "lv_point_value": (C.c_int, [_vp, _i32, _pd, _pd, _pd]),
    "lv_get_timings": (C.c_int, [_vp, _pd, _i32]),
    "lv_reset_timings": (C.c_int, [_vp]),
    "lv_launch_count": (_i64, [_vp]),
    "lv_stream": (_vp, [_vp]),
    "lv_kernel_timing": (C.c_int, [_vp, _i32]),
    "lv_kernel_time": (C.c_int, [_vp, _i32, _pi64, _pd, _i32]),
    "lv_solver_counters": (C.c_int, [_vp, _pi64, _pi64]),
    "lv_solver_unconverged": (C.c_int, [_vp, _pi64]),
    "lv_set_wait_limit": (C.c_int, [_vp, _i64]),
    "lv_get_boundary_edges": (C.c_int, [_vp, _pi64, _pd, _pi32]),
    "lv_find_pressure_edges": (C.c_int, [_vp, _d, _i32, _i64, _pd, _pst]),
    "lv_bdary_friction_edges": (C.c_int, [_vp, _i64, _pd, C.POINTER(C.c_uint8), _d]),
    "lv_viscous_solve": (C.c_int, [_vp, _d, _pst]),
    "lv_ideal_temperature": (C.c_int, [_vp]),
    "lv_fourier_step": (C.c_int, [_vp, _d]),
    "lv_heat_from_bdary_edges": (C.c_int, [_vp, _i64, _pd, _d, _d]),
    "lv_solver_halo": (C.c_int, [_vp, _pi32]),
    "lv_solver_forget": (C.c_int, [_vp]),
    "lv_mesh_captures": (C.c_int, [_vp, _pi32]),
    "lv_learn_init": (C.c_int, [_vp, C.c_uint64]),
    "lv_learn_num_params": (_i32, []),
    "lv_learn_get_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "lv_learn_set_params": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "lv_learn_add_system": (C.c_int, [_vp]),
    "lv_learn_num_systems": (_i32, [_vp]),
    "lv_learn_clear_systems": (C.c_int, [_vp]),
    "lv_learn_train": (C.c_int, [_vp, _i32, C.c_float, _i32, C.c_uint64, C.POINTER(C.c_float)]),
    "lv_learn_loss_grad": (C.c_int, [_vp, _i32, C.POINTER(C.c_float), _i32, C.c_uint64, _pd,
                                     C.POINTER(C.c_float)]),
    "lv_learn_factor": (C.c_int, [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "lv_pcg_solve_noalloc": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _d, _i32, _vp, _pi32, _pd]),
}
KERNEL_FAMILIES = {"bin": 0, "clip": 1, "pcg": 2, "rhs": 3, "ops": 4, "learn": 5}

_LIB = None


class LvError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{LV_ERR.get(code, code)}: {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Load liblvgpu.so and bind every exported symbol (raises if absent)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise RuntimeError(f"liblvgpu.so not built ({path}); run lagrangianvoronoi.jl_gb300/build.py")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def ptr(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))
