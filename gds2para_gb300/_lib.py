"""ctypes binding of libgds2para_gb300.so (the C ABI in include/gds2para_gb300.h).

The library is built in-tree by gds2para_gb300.build; loading fails loudly
when it is missing -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

# Every symbol the public header declares.
EXPORTS = [
    "g2p_last_error", "g2p_version", "g2p_default_params",
    "g2p_mesh_create", "g2p_mesh_destroy", "g2p_mesh_sizes",
    "g2p_index_maps", "g2p_generate_stiff", "g2p_export_stiff",
    "g2p_assemble_v0", "g2p_export_v0", "g2p_export_laplacian",
    "g2p_hypre_solve", "g2p_solver_create", "g2p_solver_solve", "g2p_solver_destroy",
    "g2p_para_generator", "g2p_launch_count", "g2p_profile_begin", "g2p_profile_end", "g2p_profile_report",
    "g2p_map_edge_noalloc", "g2p_profile_buckets",
    "g2p_server_create", "g2p_server_submit", "g2p_server_wait", "g2p_server_destroy",
    "g2p_mesh_mark", "g2p_mesh_mark_polygons",
    "g2p_convert_param", "g2p_write_touchstone", "g2p_write_citi",
    "g2p_ybus_from_param", "g2p_write_xyce", "g2p_write_spef", "g2p_terminate_port", "g2p_y_from_circuit",
    "g2p_gdsii_read", "g2p_polygons_size", "g2p_polygons_get", "g2p_polygons_free", "g2p_mesh_grid",
    "g2p_stiff_apply", "g2p_sim_input_read", "g2p_sim_input_sizes", "g2p_sim_input_get", "g2p_sim_input_free",
    "g2p_find_vh", "g2p_export_vh", "g2p_set_vh", "g2p_para_generator_vh", "g2p_hessenberg_eig",
]

STATUS = {0: "G2P_OK", 1: "G2P_ERR_INVALID", 2: "G2P_ERR_CUDA", 3: "G2P_ERR_NOMEM", 4: "G2P_ERR_NOT_CONVERGED",
          5: "G2P_ERR_UNSUPPORTED", 6: "G2P_ERR_STATE", 7: "G2P_ERR_ADMISSION"}
G2P_OK, G2P_ERR_NOT_CONVERGED = 0, 4
G2P_PREC_FP64, G2P_PREC_MIXED, G2P_PREC_FP64_PC32 = 0, 1, 2


class MeshDescC(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("xn", C.c_void_p), ("yn", C.c_void_p), ("zn", C.c_void_p),
                ("stack_epsn", C.c_void_p), ("stack_sign", C.c_void_p),
                ("mark_node", C.c_void_p), ("mark_edge", C.c_void_p),
                ("num_cdt", C.c_int64), ("mark_port", C.c_void_p), ("cdt_return", C.c_void_p),
                ("num_ports", C.c_int32), ("port_side_ptr", C.c_void_p), ("side_edge_ptr", C.c_void_p),
                ("side_edges", C.c_void_p), ("side_area", C.c_void_p), ("side_dir", C.c_void_p),
                ("freq_start", C.c_double), ("freq_end", C.c_double), ("freq_unit", C.c_double),
                ("nfreq", C.c_int32), ("freq_scale", C.c_int32)]


class SolverParams(C.Structure):
    _fields_ = [("precision", C.c_int32), ("restart", C.c_int32), ("maxit", C.c_int32), ("rtol", C.c_double),
                ("smoother_degree", C.c_int32), ("coarse_size", C.c_int32), ("strength", C.c_double),
                ("max_levels", C.c_int32), ("inner_rtol", C.c_double), ("inner_maxit", C.c_int32),
                ("batch", C.c_int32), ("use_graphs", C.c_int32), ("autotune", C.c_int32),
                ("inner_restart", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("rel_residual", C.c_double),
                ("levels", C.c_int32), ("converged", C.c_int32), ("coarse_rows", C.c_int64),
                ("setup_ms", C.c_double), ("solve_ms", C.c_double)]


class Sizes(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("bden", "leng_S", "leng_v0d", "leng_v0c", "nnz_v0d", "nnz_v0c",
                                          "nnz_ad", "nnz_ac")]


class ExtractStats(C.Structure):
    _fields_ = [("sizes", Sizes), ("solves", C.c_int32), ("total_iterations", C.c_int32),
                ("max_rel_residual", C.c_double), ("assembly_ms", C.c_double), ("setup_ms", C.c_double),
                ("solve_ms", C.c_double), ("total_ms", C.c_double), ("ad_levels", C.c_int32),
                ("ac_levels", C.c_int32), ("rhs_block", C.c_int32), ("ad_degree", C.c_int32),
                ("ac_strength", C.c_double), ("ac_precision", C.c_int32), ("ac_iterations", C.c_int32)]


class BoxC(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("x0", "x1", "y0", "y1", "z0", "z1")]


class PortSideC(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("sx", "sy", "sz", "rx", "ry", "rz")]


class JobTimes(C.Structure):
    _fields_ = [("queued_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
                ("footprint_estimate", C.c_int64), ("footprint_measured", C.c_int64), ("ran_alone", C.c_int32)]


class G2PError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} missing: run gds2para_gb300.build")
        _build.build()
    L = C.CDLL(path)
    vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    L.g2p_last_error.restype = C.c_char_p
    L.g2p_version.restype = C.c_char_p
    L.g2p_default_params.argtypes = [C.POINTER(SolverParams), i32]
    L.g2p_default_params.restype = None
    L.g2p_mesh_create.argtypes = [C.POINTER(MeshDescC), C.POINTER(vp)]
    L.g2p_mesh_destroy.argtypes = [vp]
    L.g2p_mesh_sizes.argtypes = [vp, C.POINTER(Sizes)]
    L.g2p_index_maps.argtypes = [vp, C.POINTER(i64), vp]
    L.g2p_generate_stiff.argtypes = [vp, C.POINTER(i64)]
    L.g2p_export_stiff.argtypes = [vp, vp, vp, vp]
    L.g2p_assemble_v0.argtypes = [vp, C.POINTER(Sizes)]
    L.g2p_export_v0.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.g2p_export_laplacian.argtypes = [vp, i32, vp, vp, vp]
    L.g2p_hypre_solve.argtypes = [vp, vp, vp, i64, vp, i64, vp]
    L.g2p_solver_create.argtypes = [vp, vp, vp, i64, i64, C.POINTER(SolverParams), C.POINTER(vp)]
    L.g2p_solver_solve.argtypes = [vp, vp, vp, i32, C.POINTER(SolveStats)]
    L.g2p_solver_destroy.argtypes = [vp]
    L.g2p_para_generator.argtypes = [vp, C.POINTER(SolverParams), vp, C.POINTER(ExtractStats)]
    L.g2p_launch_count.restype = C.c_int64
    L.g2p_launch_count.argtypes = []
    L.g2p_profile_begin.restype = None
    L.g2p_profile_begin.argtypes = []
    L.g2p_profile_end.argtypes = [C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i64)]
    L.g2p_profile_report.restype = C.c_int64
    L.g2p_profile_report.argtypes = [C.c_char_p, i64]
    L.g2p_mesh_mark.argtypes = [i64, i64, i64, vp, vp, vp, vp, i64, i32, vp, vp, vp, vp, C.POINTER(i64),
                                vp, vp, i64, vp, vp, i64, vp, vp]
    L.g2p_mesh_mark_polygons.argtypes = [i64, i64, i64, vp, vp, vp, i64, vp, vp, vp, vp, i32, vp, vp, vp, vp, vp,
                                         C.POINTER(i64), vp, vp, i64, vp, vp, i64, vp, vp]
    L.g2p_server_create.argtypes = [i64, i32, C.POINTER(vp)]
    L.g2p_server_submit.argtypes = [vp, C.POINTER(MeshDescC), C.POINTER(SolverParams), C.POINTER(i64)]
    L.g2p_server_wait.argtypes = [vp, i64, vp, C.POINTER(ExtractStats), C.POINTER(JobTimes)]
    L.g2p_server_destroy.argtypes = [vp]
    L.g2p_profile_buckets.restype = None
    L.g2p_profile_buckets.argtypes = [C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i64)]
    L.g2p_map_edge_noalloc.argtypes = [i64, i64, i64, vp, vp, i64, vp, vp, vp]
    L.g2p_convert_param.argtypes = [C.c_char, C.c_char, i32, i32, vp, vp, vp]
    L.g2p_write_touchstone.argtypes = [C.c_char_p, C.c_char, i32, i32, vp, vp, vp, C.c_char_p]
    L.g2p_write_citi.argtypes = [C.c_char_p, C.c_char, i32, i32, vp, vp, C.c_char_p]
    L.g2p_ybus_from_param.argtypes = [C.c_char, i32, dbl, vp, vp, vp]
    L.g2p_terminate_port.argtypes = [C.c_char, i32, i32, vp, i32, i32, vp, vp, vp]
    L.g2p_y_from_circuit.argtypes = [i32, i32, vp, vp, vp, vp]
    L.g2p_write_xyce.argtypes = [C.c_char_p, C.c_char_p, i32, C.POINTER(C.c_char_p), dbl, vp, vp, dbl]
    L.g2p_write_spef.argtypes = [C.c_char_p, C.c_char_p, i32, C.POINTER(C.c_char_p), C.c_char_p, vp, vp, dbl]
    L.g2p_gdsii_read.argtypes = [C.c_char_p, vp, i32, C.POINTER(vp)]
    L.g2p_polygons_size.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
    L.g2p_polygons_get.argtypes = [vp, vp, vp, vp, vp]
    L.g2p_polygons_free.argtypes = [vp]
    L.g2p_polygons_free.restype = None
    L.g2p_mesh_grid.argtypes = [vp, i64, vp, vp, vp, i32, vp, i32, vp, i64, i64, vp, vp, vp, vp, vp, vp]
    L.g2p_sim_input_read.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.g2p_sim_input_sizes.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
    L.g2p_sim_input_get.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.g2p_sim_input_free.argtypes = [vp]
    L.g2p_sim_input_free.restype = None
    L.g2p_stiff_apply.argtypes = [vp, i32, i32, vp, vp, C.POINTER(dbl)]
    L.g2p_find_vh.argtypes = [vp, i32, C.POINTER(i64)]
    L.g2p_export_vh.argtypes = [vp, vp]
    L.g2p_set_vh.argtypes = [vp, vp, i64]
    L.g2p_para_generator_vh.argtypes = [vp, C.POINTER(SolverParams), i32, vp, vp, C.POINTER(ExtractStats)]
    L.g2p_hessenberg_eig.argtypes = [i64, vp, vp, vp]
    for name in EXPORTS:
        if name not in ("g2p_last_error", "g2p_version", "g2p_default_params", "g2p_launch_count",
                        "g2p_profile_begin", "g2p_profile_report", "g2p_profile_buckets", "g2p_polygons_free",
                        "g2p_sim_input_free"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def profile_report() -> str:
    L = load()
    n = L.g2p_profile_report(None, 0)
    buf = C.create_string_buffer(int(n) + 1)
    L.g2p_profile_report(buf, int(n) + 1)
    return buf.value.decode()


def check(status: int, allow=(G2P_OK,)):
    if status not in allow:
        raise G2PError(status, load().g2p_last_error().decode(errors="replace"))
    return status
