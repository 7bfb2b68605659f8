"""ctypes binding of libpunc_gpu.so (the C ABI declared in include/punc_gpu.h).

The library must exist: nothing here falls back to a CPU path.  Build it with
`python -c "import __graft_entry__ as g; g.build()"` or
`python puncpp_gb300/build_lib.py`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpunc_gpu.so")
ABI_VERSION = 3   # include/punc_gpu.h PG_ABI_VERSION, which these structures follow

PG_OK = 0
STATUS_NAMES = {
    0: "PG_OK", 1: "PG_ERR_ARG", 2: "PG_ERR_CUDA", 3: "PG_ERR_MESH", 4: "PG_ERR_CAPACITY",
    5: "PG_ERR_WALK_LIMIT", 6: "PG_ERR_NOT_CONVERGED", 7: "PG_ERR_STATE", 8: "PG_ERR_SINGULAR",
}
PG_FP64, PG_MIXED = 0, 1
(PG_ERR_ARG, PG_ERR_CUDA, PG_ERR_MESH, PG_ERR_CAPACITY, PG_ERR_WALK_LIMIT, PG_ERR_NOT_CONVERGED, PG_ERR_STATE,
 PG_ERR_SINGULAR) = range(1, 9)

(T_CELL_VERTICES, T_BARYCENTRIC, T_PLANES, T_NEIGHBOURS, T_CELL_DOFS, T_VOLUME, T_DV_INV,
 T_CSR_ROWPTR, T_CSR_COL, T_STIFFNESS, T_MASS, T_EXT_FACETS, T_BC_KIND, T_OBJ_FACETS) = range(14)
_TABLE_DTYPE = {T_CELL_VERTICES: np.int64, T_BARYCENTRIC: np.float64, T_PLANES: np.float64,
                T_NEIGHBOURS: np.int64, T_CELL_DOFS: np.int64, T_VOLUME: np.float64, T_DV_INV: np.float64,
                T_CSR_ROWPTR: np.int64, T_CSR_COL: np.int64, T_STIFFNESS: np.float64, T_MASS: np.float64,
                T_EXT_FACETS: np.float64, T_BC_KIND: np.int64, T_OBJ_FACETS: np.float64}


class PgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int64), ("coords", C.POINTER(C.c_double)),
                ("n_cells", C.c_int64), ("cells", C.POINTER(C.c_int64)),
                ("n_boundary_facets", C.c_int64), ("bfacet_vertices", C.POINTER(C.c_int64)),
                ("bfacet_tags", C.POINTER(C.c_int32)),
                ("n_dofs", C.c_int64), ("vertex_to_dof", C.POINTER(C.c_int64))]


class Config(C.Structure):
    _fields_ = [("precision", C.c_int32), ("periodic", C.c_int32), ("eps0", C.c_double),
                ("particle_capacity", C.c_int64), ("max_walk_steps", C.c_int32),
                ("sort_interval", C.c_int32), ("pcg_rtol", C.c_double), ("pcg_atol", C.c_double),
                ("pcg_max_iter", C.c_int32), ("pcg_warm_start", C.c_int32), ("ext_E", C.c_double * 3),
                ("circuit_resolve", C.c_int32), ("pcg_precision", C.c_int32), ("pcg_precond", C.c_int32)]


class Object(C.Structure):
    _fields_ = [("bnd_id", C.c_int64), ("charge", C.c_double), ("current", C.c_double),
                ("potential", C.c_double)]


class Source(C.Structure):
    _fields_ = [("node_a", C.c_int32), ("node_b", C.c_int32), ("value", C.c_double)]


class Species(C.Structure):
    _fields_ = [("q", C.c_double), ("m", C.c_double), ("n", C.c_double), ("vth", C.c_double),
                ("vd", C.c_double * 3), ("vdf_range", C.c_double)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("solves", C.c_int32), ("residual", C.c_double),
                ("rhs_norm", C.c_double)]


class StepArgs(C.Structure):
    _fields_ = [("dt", C.c_double), ("B", C.c_double * 3), ("first_step", C.c_int32),
                ("use_accel", C.c_int32), ("periodic_move", C.c_int32), ("Ld", C.c_double * 3),
                ("inject", C.c_int32), ("seed", C.c_uint64), ("step", C.c_uint64), ("E0", C.c_double * 3),
                ("efield_cg1", C.c_int32), ("potential_energy", C.c_int32)]


class StepResult(C.Structure):
    _fields_ = [("KE", C.c_double), ("n_particles", C.c_int64), ("n_absorbed", C.c_int64),
                ("n_injected", C.c_int64), ("pcg_iterations", C.c_int32), ("pcg_residual", C.c_double),
                ("PE", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("threads", C.c_int32), ("blocks_per_sm", C.c_int32), ("dep_agg", C.c_int32),
                ("sort_interval", C.c_int32), ("pass_ms", C.c_double), ("sort_ms", C.c_double)]


MAX_AMG_LEVELS = 12


class PoissonLayout(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("nnz", C.c_int64), ("sell_entries", C.c_int64),
                ("precond", C.c_int32), ("levels", C.c_int32),
                ("level_rows", C.c_int64 * MAX_AMG_LEVELS), ("level_nnz", C.c_int64 * MAX_AMG_LEVELS),
                ("level_nnz_p", C.c_int64 * MAX_AMG_LEVELS), ("cycle_nnz_g", C.c_int64),
                ("cycle_nnz_u1", C.c_int64), ("cycle_bytes", C.c_int64)]


# Every entry point of include/punc_gpu.h with its argument types.
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
SIGNATURES = {
    "pg_abi_version": ([], C.c_int32),
    "pg_last_error": ([], C.c_char_p),
    "pg_philox4x32_10": ([C.POINTER(C.c_uint32)] * 3, C.c_int),
    "pg_mesh_build": ([C.POINTER(MeshDesc), C.c_double, C.POINTER(_P)], C.c_int),
    "pg_mesh_array": ([_P, C.c_int32, C.POINTER(C.c_void_p), _I64], C.c_int),
    "pg_mesh_free": ([_P], C.c_int),
    "pg_create": ([_P, C.POINTER(Config), C.POINTER(_P)], C.c_int),
    "pg_destroy": ([_P], C.c_int),
    "pg_status_detail": ([_P, _I32, _I64], C.c_int),
    "pg_add_particles": ([_P, _D, _D, C.c_int64, C.c_double, C.c_double, _I64], C.c_int),
    "pg_num_particles": ([_P, _I64, _I64, _I64], C.c_int),
    "pg_add_particles_range": ([_P, _D, _D, C.c_int64, C.c_double, C.c_double, C.c_int32, C.c_int32, _I64], C.c_int),
    "pg_set_injection_streams": ([_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)], C.c_int),
    "pg_get_particles": ([_P, C.c_int64, _D, _D, _D, _D, _I64, _I64, _I64], C.c_int),
    "pg_locate": ([_P, _D, C.c_int64, _I64], C.c_int),
    "pg_efield_dg0": ([_P, _D], C.c_int),
    "pg_set_efield": ([_P, _D], C.c_int),
    "pg_get_efield": ([_P, _D], C.c_int),
    "pg_accel": ([_P, C.c_double, _D], C.c_int),
    "pg_boris": ([_P, _D, C.c_double, _D], C.c_int),
    "pg_move": ([_P, C.c_double], C.c_int),
    "pg_move_periodic": ([_P, C.c_double, _D], C.c_int),
    "pg_update": ([_P, C.POINTER(Object), C.c_int32, C.c_double], C.c_int),
    "pg_absorbed_counts": ([_P, _I64, C.c_int32, C.c_int32, _D, _D, _I32], C.c_int),
    "pg_relocate": ([_P, _D, _I64, C.c_int64, C.c_int32, _I64, _I32], C.c_int),
    "pg_kinetic_energy": ([_P, _D], C.c_int),
    "pg_distribute_cg1": ([_P, _D], C.c_int),
    "pg_set_rho": ([_P, _D], C.c_int),
    "pg_poisson_solve": ([_P, C.POINTER(Object), C.c_int32, _D, C.POINTER(SolveInfo)], C.c_int),
    "pg_circuit_cm_setup": ([_P, C.POINTER(Source), C.c_int32, C.POINTER(Source), C.c_int32, C.c_double], C.c_int),
    "pg_solve_circuit": ([_P, C.POINTER(Object), C.c_int32, _D, C.POINTER(SolveInfo)], C.c_int),
    "pg_get_phi": ([_P, _D], C.c_int),
    "pg_get_phi_async": ([_P, _D], C.c_int),
    "pg_get_rho": ([_P, _D], C.c_int),
    "pg_get_capacitance": ([_P, _D], C.c_int),
    "pg_create_flux": ([_P, C.POINTER(Species), C.c_int32], C.c_int),
    "pg_inject": ([_P, C.c_double, C.c_uint64, C.c_uint64, _I64], C.c_int),
    "pg_step": ([_P, C.POINTER(StepArgs), C.POINTER(Object), C.c_int32, C.POINTER(StepResult)], C.c_int),
    "pg_sort": ([_P], C.c_int),
    "pg_adjoint_forward": ([_P, C.POINTER(StepArgs), C.POINTER(Object), C.c_int32, C.c_int32, C.c_int32, _D, _D],
                           C.c_int),
    "pg_adjoint_backward": ([_P, _D, C.c_int64, _D, _D], C.c_int),
    "pg_adjoint_potential_gradient": ([_P, _D, C.c_int32], C.c_int),
    "pg_adjoint_release": ([_P], C.c_int),
    "pg_set_tuning": ([_P, C.POINTER(Tuning)], C.c_int),
    "pg_get_tuning": ([_P, C.POINTER(Tuning)], C.c_int),
    "pg_autotune": ([_P, C.POINTER(StepArgs), C.POINTER(Object), C.c_int32, C.c_int32, C.POINTER(Tuning)], C.c_int),
    "pg_amg_set_strength": ([_P, C.c_double], C.c_int),
    "pg_amg_get_strength": ([_P, _D], C.c_int),
    "pg_autotune_amg": ([_P, C.POINTER(StepArgs), C.POINTER(Object), C.c_int32, C.c_int32, _D, C.c_int32, _D, _D],
                        C.c_int),
    "pg_run_steps": ([_P, C.POINTER(StepArgs), C.POINTER(Object), C.c_int32, C.c_int32, C.c_int32,
                      C.POINTER(StepResult)], C.c_int),
    "pg_stage_times": ([_P, _D, C.c_int32, _I32], C.c_int),
    "pg_stage_name": ([_P, C.c_int32], C.c_char_p),
    "pg_set_profiling": ([_P, C.c_int32], C.c_int),
    "pg_event_record": ([_P, C.c_int32], C.c_int),
    "pg_event_elapsed": ([_P, C.c_int32, C.c_int32, _D], C.c_int),
    "pg_synchronize": ([_P], C.c_int),
    "pg_launch_count": ([_I64], C.c_int),
    "pg_esolver_solve": ([_P, _D, C.POINTER(SolveInfo)], C.c_int),
    "pg_potential_energy": ([_P, _D], C.c_int),
    "pg_population_save": ([_P, C.c_char_p, C.c_int32], C.c_int),
    "pg_population_load": ([_P, C.c_char_p, C.c_int32, _I64], C.c_int),
    "pg_density_cg1": ([_P, C.c_double, C.c_double, _D, _D], C.c_int),
    "pg_density_dg0": ([_P, C.c_double, C.c_double, _D, _D], C.c_int),
    "pg_statistics": ([_P, _D], C.c_int),
    "pg_set_efield_cg1": ([_P, _D], C.c_int),
    "pg_get_efield_cg1": ([_P, _D], C.c_int),
    "pg_accel_cg1": ([_P, C.c_double, _D], C.c_int),
    "pg_boris_cg1": ([_P, _D, C.c_double, _D], C.c_int),
    "pg_poisson_layout_get": ([_P, C.POINTER(PoissonLayout)], C.c_int),
    "pg_pcg_solve_noalloc": ([C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                              C.c_double, C.c_int32, C.c_void_p, _I32, _D], C.c_int),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it first (puncpp_gb300/build_lib.py)")
    lib = C.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.pg_abi_version() != ABI_VERSION:
        raise ImportError(f"{path}: ABI version {lib.pg_abi_version()}, these bindings follow {ABI_VERSION} "
                          "(rebuild the library)")
    _lib = lib
    return lib


def check(rc: int):
    if rc != PG_OK:
        msg = load().pg_last_error()
        raise PgError(rc, msg.decode() if msg else "")


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def i64ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_I64)


def i32ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I32)
