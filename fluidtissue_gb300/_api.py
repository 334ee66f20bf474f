"""ctypes declarations of the solver entry points in include/fts.h."""
from __future__ import annotations

import ctypes as C


class FtsMesh(C.Structure):
    _fields_ = [
        ("np", C.c_int64),
        ("nt", C.c_int64),
        ("xyz", C.POINTER(C.c_float)),
        ("tets", C.POINTER(C.c_int32)),
        ("boundary", C.POINTER(C.c_uint8)),
    ]


class FtsParams(C.Structure):
    _fields_ = [
        ("velocity_degree", C.c_int32),
        ("alpha", C.c_double),
        ("eps", C.c_double),
        ("tol", C.c_double),
        ("max_iter", C.c_int32),
        ("mu_interior", C.c_double),
        ("mu_exterior", C.c_double),
        ("mu_profile", C.c_int32),
        ("gf_growth", C.c_double),
        ("level_sink", C.c_double),
        ("growth_threshold", C.c_double),
        ("rd_iterations", C.c_double),
        ("gf_production", C.c_double),
        ("advection_dt", C.c_double),
        ("surface_tension", C.c_double),
        ("precision", C.c_int32),
        ("solver", C.c_int32),
        ("preconditioner", C.c_int32),
        ("operator_kind", C.c_int32),
        ("warm_start", C.c_int32),
        ("device", C.c_int32),
        ("inner_tol", C.c_double),
        ("verbose", C.c_int32),
        ("time_kernels", C.c_int32),
    ]


class FtsStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("solved", C.c_int32),
        ("iterations", C.c_int64),
        ("iterations_fp32", C.c_int64),
        ("outer_iterations", C.c_int32),
        ("rel_residual", C.c_double),
        ("error_estimate", C.c_double),
        ("mu_min", C.c_double),
        ("mu_max", C.c_double),
        ("f_norm", C.c_double),
        ("ms_assembly", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_total", C.c_double),
        ("device_bytes", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("spmv_launches", C.c_int64),
        ("ms_spmv", C.c_double),
        ("spmv_bytes", C.c_double),
        ("spmv_bytes_fp64", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class FtsBatchConfig(C.Structure):
    _fields_ = [
        ("threads", C.c_int32),
        ("chunk_rows", C.c_int32),
        ("tpr", C.c_int32),
        ("blocks", C.c_int32),
        ("ms_per_sweep", C.c_double),
        ("graph", C.c_int32),
        ("spmv_format", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class FtsRdParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("iterations", C.c_int64),
        ("act", C.c_double), ("da", C.c_double), ("dega", C.c_double),
        ("inh", C.c_double), ("di", C.c_double), ("degi", C.c_double),
        ("gf_production", C.c_double),
        ("gf_diffusion", C.c_double),
        ("gf_degradation", C.c_double),
        ("gf_inhibition", C.c_double),
    ]


class FtsRdStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("alive", C.c_int32),
        ("interior_nodes", C.c_int64),
        ("interior_elements", C.c_int64),
        ("steps", C.c_int64),
        ("ms_setup", C.c_double),
        ("ms_steps", C.c_double),
        ("ms_total", C.c_double),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class FtsDistStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("blocks", C.c_int32),
        ("points_scanned", C.c_int64),
        ("ms_setup", C.c_double),
        ("ms_kernel", C.c_double),
        ("ms_total", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


DIST_PRUNED, DIST_EXHAUSTIVE = 0, 1


class FtsLsParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("tol", C.c_double),
        ("max_iter", C.c_int64),
        ("reset", C.c_int32),
    ]


class FtsLsStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_int64),
        ("error", C.c_double),
        ("interface_points", C.c_int64),
        ("ms_assembly", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_reset", C.c_double),
        ("ms_total", C.c_double),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class FtsStStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("interface_points", C.c_int64),
        ("area", C.c_double),
        ("ms_kernels", C.c_double),
        ("ms_total", C.c_double),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}

PREC_FP64, PREC_MIXED = 0, 1
SOLVER_MINRES, SOLVER_BICGSTAB = 0, 1
PC_AUTO, PC_JACOBI, PC_MULTIGRID, PC_MULTIGRID_DIAG = 0, 1, 2, 3
OP_AUTO, OP_ASSEMBLED, OP_MATFREE, OP_STENCIL = 0, 1, 2, 3

STATUS = {
    0: "FTS_OK", 1: "FTS_ERR_BAD_INPUT", 2: "FTS_ERR_DEGENERATE_ELEMENT",
    3: "FTS_ERR_NOT_CONVERGED", 4: "FTS_ERR_CUDA", 5: "FTS_ERR_OOM",
    6: "FTS_ERR_UNSUPPORTED", 7: "FTS_ERR_NAN", 8: "FTS_ERR_TIMEOUT",
}

# Every symbol include/fts.h declares, with (restype, argtypes).
_P = C.POINTER
_vp = C.c_void_p
_dp = _P(C.c_double)
SIGNATURES = {
    "fts_params_default": (None, [_P(FtsParams)]),
    "fts_create": (C.c_int, [_P(FtsMesh), _P(FtsParams), _P(_vp)]),
    "fts_solve": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _P(FtsStats)]),
    "fts_solve_device": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _P(FtsStats)]),
    "fts_set_stream": (C.c_int, [_vp, _vp]),
    "fts_update_params": (C.c_int, [_vp, _P(FtsParams)]),
    "fts_reset_guess": (C.c_int, [_vp]),
    "fts_destroy": (None, [_vp]),
    "fts_status_string": (C.c_char_p, [C.c_int]),
    "fts_last_error": (C.c_char_p, [_vp]),
    "fts_get_sizes": (C.c_int, [_vp, _P(C.c_int64), _P(C.c_int64), _P(C.c_int64)]),
    "fts_get_system": (C.c_int, [_vp, _P(C.c_int32), _P(C.c_int32), _dp, _dp]),
    "fts_apply": (C.c_int, [_vp, C.c_int32, _dp, _dp]),
    "fts_bsr_residual_noalloc": (C.c_int, [C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fts_batch_create": (C.c_int, [C.c_int32, _P(FtsMesh), _P(FtsParams), _P(_vp)]),
    "fts_batch_solve": (C.c_int, [_vp, _P(_dp), _P(_dp), _P(_dp), _P(_dp), _P(FtsStats)]),
    "fts_batch_solve_device": (C.c_int, [_vp, _P(_vp), _P(_vp), _P(_vp), _P(_vp), _P(FtsStats)]),
    "fts_batch_get_config": (C.c_int, [_vp, _P(FtsBatchConfig)]),
    "fts_batch_set_stream": (C.c_int, [_vp, _vp]),
    "fts_batch_set_barrier_limit": (C.c_int, [_vp, C.c_double, C.c_int32]),
    "fts_batch_last_error": (C.c_char_p, [_vp]),
    "fts_batch_destroy": (None, [_vp]),
    "fts_rd_create": (C.c_int, [_P(FtsMesh), C.c_int32, _P(_vp)]),
    "fts_rd_solve": (C.c_int, [_vp, _P(FtsRdParams), _dp, _P(C.c_int32), C.c_int32, _dp, _dp,
                               _dp, _P(FtsRdStats)]),
    "fts_rd_destroy": (None, [_vp]),
    "fts_rd_last_error": (C.c_char_p, [_vp]),
    "fts_dist_create": (C.c_int, [_P(C.c_float), C.c_int64, C.c_int32, _P(_vp)]),
    "fts_dist_reset": (C.c_int, [_vp, _P(C.c_float), C.c_int32, _dp, C.c_int32,
                                 _P(FtsDistStats)]),
    "fts_dist_destroy": (None, [_vp]),
    "fts_dist_last_error": (C.c_char_p, [_vp]),
    "fts_ls_create": (C.c_int, [_P(FtsMesh), C.c_int32, _P(_vp)]),
    "fts_ls_update": (C.c_int, [_vp, _P(FtsLsParams), _dp, _dp, _P(FtsLsStats)]),
    "fts_ls_destroy": (None, [_vp]),
    "fts_ls_last_error": (C.c_char_p, [_vp]),
    "fts_ls_reset_values": (C.c_int, [_vp, _dp]),
    "fts_ls_distance_reset": (C.c_int, [_vp, _dp, _dp]),
    "fts_ls_surface_tension": (C.c_int, [_vp, _dp, _dp, C.c_double, C.c_int32, _dp,
                                         _P(FtsStStats)]),
}

NOALLOC_MAX_NODES = 1048576


def declare(lib: C.CDLL) -> None:
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
