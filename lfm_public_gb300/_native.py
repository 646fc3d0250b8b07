"""ctypes binding of the C ABI in include/lfm_gpu.h.

The library is the in-tree ``liblfm_gpu.so``; importing a solver without it is
an error (there is no CPU fallback). The oracle's binding lives beside the
oracle (``oracle/port``), outside this package.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "liblfm_gpu.so")

LFM_FP64 = 0
LFM_FP32_BULK = 1
LFM_RENUMBER_NONE, LFM_RENUMBER_RCM, LFM_RENUMBER_HILBERT, LFM_RENUMBER_HPATH = 0, 1, 2, 3
# lfm_status codes (include/lfm_gpu.h)
LFM_OK = 0
LFM_ERR_INVALID = -1
LFM_ERR_IO = -2
LFM_ERR_CUDA = -3
LFM_ERR_NOMEM = -4
LFM_ERR_NUMERIC = -5
LFM_ERR_UNSUPPORTED = -6

_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)


class SolverDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("nq", C.c_int), ("solver", C.c_int), ("rk_order", C.c_int), ("minmod", C.c_int),
        ("residuals", C.c_int),
        ("n_cells", C.c_int64), ("n_cells0", C.c_int64), ("n_ghosts", C.c_int64), ("n_faces", C.c_int64),
        ("face_p", _i64p), ("face_n", _i64p), ("face_ghost", C.POINTER(C.c_uint8)),
        ("S", _dp), ("d", _dp), ("w", _dp), ("smag", _dp), ("dmag_inv", _dp), ("dnorm", _dp), ("delta_mag", _dp),
        ("K", _dp), ("vol_inv", _dp), ("sponge", _dp),
        ("ghost_cell", _i64p), ("ghost_kind", C.POINTER(C.c_int)),
        ("cell_face_offsets", _i64p), ("cell_faces", _i64p), ("cell_face_sign", C.POINTER(C.c_int8)),
        ("cell_s_offsets", _i64p), ("cell_s", _dp), ("q0", _dp),
        ("gamma", C.c_double), ("Rgas", C.c_double), ("rhoInf", C.c_double), ("EInf", C.c_double),
        ("pInf", C.c_double), ("TInf", C.c_double), ("UInf", C.c_double * 3), ("mu", C.c_double), ("Cp", C.c_double),
        ("PrInv", C.c_double), ("rkA", _dp), ("rkB", _dp),
        ("n_halos", C.c_int64), ("halo_src_part", _i64p), ("halo_src_cell", _i64p),
        ("ghost_patch", C.POINTER(C.c_int32)), ("smag_c", _dp),
    ]


class PolyMesh(C.Structure):
    _fields_ = [
        ("n_points", C.c_int64), ("points", _dp), ("n_faces", C.c_int64), ("face_offsets", _i64p),
        ("face_points", _i64p), ("owner", _i64p), ("n_internal_faces", C.c_int64), ("neighbour", _i64p),
        ("n_patches", C.c_int), ("patch_name", C.POINTER(C.c_char_p)), ("patch_type", C.POINTER(C.c_char_p)),
        ("patch_start", _i64p), ("patch_size", _i64p), ("patch_neighbour", C.POINTER(C.c_char_p)),
        ("cell_submesh", _i64p), ("n_cells", C.c_int64),
    ]


class Params(C.Structure):
    _fields_ = [
        ("solver", C.c_int), ("dimension", C.c_int), ("rk_order", C.c_int), ("minmod", C.c_int), ("laminar", C.c_int),
        ("residuals", C.c_int), ("p_inf", C.c_double), ("T_inf", C.c_double), ("U_inf", C.c_double * 3),
        ("Ls", C.c_double), ("mach", C.c_double), ("k_sponge", C.c_double), ("Cp", C.c_double),
        ("mol_weight", C.c_double), ("mu", C.c_double), ("Pr", C.c_double), ("renumber", C.c_int),
    ]


class Fields(C.Structure):
    _fields_ = [("p", _dp), ("T", _dp), ("U", _dp), ("alpha", _dp)]


class SolverOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("block", C.c_int)]


class BatchOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("rk_order", C.c_int), ("arena_bytes", C.c_size_t), ("max_cases", C.c_int)]


class BatchTuning(C.Structure):
    _fields_ = [("block", C.c_int), ("items_per_thread", C.c_int), ("blocks_per_sm", C.c_int),
                ("cooperative", C.c_int), ("phased", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


LFM_FLUX_FACE, LFM_FLUX_CELL, LFM_FLUX_STAGED = 0, 1, 2
FLUX_KERNEL_NAMES = {LFM_FLUX_FACE: "face", LFM_FLUX_CELL: "cell", LFM_FLUX_STAGED: "staged"}


class SolverTuning(C.Structure):
    _fields_ = [("flux_kernel", C.c_int), ("staging_depth", C.c_int), ("staging_faces", C.c_int),
                ("ms_per_step", C.c_float)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["flux_kernel"] = FLUX_KERNEL_NAMES.get(self.flux_kernel, self.flux_kernel)
        return d


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("rk_order", C.c_int), ("arena_bytes", C.c_size_t), ("max_cases", C.c_int),
                ("chunk_steps", C.c_int), ("max_bypass", C.c_int), ("tuning", BatchTuning), ("solo_cells", C.c_int64),
                ("max_solo", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("status", C.c_int), ("cells", C.c_int64), ("steps", C.c_int),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("footprint_bytes", C.c_size_t), ("steps_done", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int), ("running", C.c_int), ("completed", C.c_int64), ("chunks", C.c_int64),
                ("t_now", C.c_double), ("busy_s", C.c_double), ("cell_stages", C.c_double)]


class LfmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lfm error {code}: {msg}")
        self.code = code


_lib: Optional[C.CDLL] = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Loads liblfm_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    vp = C.c_void_p
    sig = {
        "lfm_last_error": ([], C.c_char_p), "lfm_version": ([], C.c_char_p),
        "lfm_solver_stats_reset": ([vp], C.c_int), "lfm_solver_stats_accumulate": ([vp, C.c_int], C.c_int),
        "lfm_solver_stats_get": ([vp, C.c_int, _dp, _dp], C.c_int),
        "lfm_solver_forces": ([vp, C.c_int, C.POINTER(C.c_int32), _dp, _dp], C.c_int),
        "lfm_solver_probes_set": ([vp, C.c_int, C.POINTER(C.c_int64), C.c_int], C.c_int),
        "lfm_solver_probes_record": ([vp], C.c_int),
        "lfm_solver_probes_read": ([vp, _dp, C.POINTER(C.c_int)], C.c_int),
        "lfm_partitioned_solver": ([vp, C.c_int, C.POINTER(vp)], C.c_int),
        "lfm_solver_advance": ([vp, _dp, C.c_int, C.c_double, _dp], C.c_int),
        "lfm_batch_advance": ([vp, C.c_int, C.POINTER(C.c_int), C.POINTER(_dp), C.c_int, C.POINTER(_dp)], C.c_int),
        "lfm_tiles_stats": ([C.POINTER(SolverDesc), C.c_int, C.c_int, C.POINTER(C.c_int64)], C.c_int),
        "lfm_case_open": ([C.c_char_p, C.c_int, C.POINTER(vp)], C.c_int),
        "lfm_case_from_polymesh": ([C.POINTER(PolyMesh), C.POINTER(Params), C.POINTER(Fields), C.POINTER(vp)],
                                   C.c_int),
        "lfm_case_describe": ([vp, C.POINTER(SolverDesc)], C.c_int),
        "lfm_case_time": ([vp, _dp, _dp, _dp, C.POINTER(C.c_int), _dp], C.c_int),
        "lfm_case_cell_ids": ([vp, _i64p], C.c_int),
        "lfm_case_free": ([vp], None),
        "lfm_solver_create": ([C.POINTER(SolverDesc), C.POINTER(SolverOpts), C.POINTER(vp)], C.c_int),
        "lfm_solver_destroy": ([vp], None),
        "lfm_solver_set_state": ([vp, _dp], C.c_int),
        "lfm_solver_get_state": ([vp, _dp], C.c_int),
        "lfm_solver_stage": ([vp, C.c_int, C.c_double], C.c_int),
        "lfm_solver_step": ([vp, C.c_int, C.c_double], C.c_int),
        "lfm_solver_step_timed": ([vp, C.c_int, C.c_double, C.POINTER(C.c_float)], C.c_int),
        "lfm_solver_cfl": ([vp, C.c_double, _dp], C.c_int),
        "lfm_solver_min_dt": ([vp, C.c_double, _dp], C.c_int),
        "lfm_solver_residual": ([vp, _dp], C.c_int),
        "lfm_solver_cell_residual": ([vp, _dp], C.c_int),
        "lfm_solver_residual_noalloc": ([vp, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p], C.c_int),
        "lfm_solver_sync": ([vp], C.c_int),
        "lfm_solver_launches_per_step": ([vp, C.POINTER(C.c_int)], C.c_int),
        "lfm_solver_flush_l2": ([vp, C.c_size_t], C.c_int),
        "lfm_solver_bench": ([vp, C.c_int, C.c_double, C.c_size_t, C.POINTER(C.c_float)], C.c_int),
        "lfm_solver_profile_step": ([vp, C.c_double, C.c_int, C.POINTER(C.c_float)], C.c_int),
        "lfm_solver_kernel_name": ([C.c_int], C.c_char_p),
        "lfm_solver_get_tuning": ([vp, C.POINTER(SolverTuning)], C.c_int),
        "lfm_solver_set_tuning": ([vp, C.POINTER(SolverTuning)], C.c_int),
        "lfm_solver_autotune": ([vp, C.c_double, C.c_int, C.c_size_t, C.POINTER(SolverTuning),
                                 C.POINTER(SolverTuning), C.c_int, C.POINTER(C.c_int)], C.c_int),
        "lfm_pcase_open": ([C.c_char_p, C.c_int, C.POINTER(vp)], C.c_int),
        "lfm_pcase_parts": ([vp, C.POINTER(C.c_int)], C.c_int),
        "lfm_pcase_describe": ([vp, C.c_int, C.POINTER(SolverDesc)], C.c_int),
        "lfm_pcase_cell_global": ([vp, C.c_int, _i64p], C.c_int),
        "lfm_pcase_time": ([vp, _dp, _dp, _dp, C.POINTER(C.c_int), _dp], C.c_int),
        "lfm_pcase_free": ([vp], None),
        "lfm_partitioned_create": ([C.POINTER(C.POINTER(SolverDesc)), C.c_int, C.POINTER(SolverOpts), C.POINTER(vp)],
                                   C.c_int),
        "lfm_partitioned_destroy": ([vp], None),
        "lfm_partitioned_set_state": ([vp, C.c_int, _dp], C.c_int),
        "lfm_partitioned_get_state": ([vp, C.c_int, _dp], C.c_int),
        "lfm_partitioned_step": ([vp, C.c_int, C.c_double], C.c_int),
        "lfm_partitioned_sync": ([vp], C.c_int),
        "lfm_selftest_fp_convert": ([C.c_int64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint32)], C.c_int),
        "lfm_batch_create": ([C.POINTER(BatchOpts), C.POINTER(vp)], C.c_int),
        "lfm_batch_destroy": ([vp], None),
        "lfm_batch_case_bytes": ([C.POINTER(SolverDesc), C.POINTER(C.c_size_t)], C.c_int),
        "lfm_batch_add": ([vp, C.POINTER(SolverDesc), C.c_double, C.POINTER(C.c_int)], C.c_int),
        "lfm_batch_remove": ([vp, C.c_int], C.c_int),
        "lfm_batch_set_state": ([vp, C.c_int, _dp], C.c_int),
        "lfm_batch_get_state": ([vp, C.c_int, _dp], C.c_int),
        "lfm_batch_step": ([vp, C.c_int], C.c_int),
        "lfm_batch_sync": ([vp], C.c_int),
        "lfm_batch_case_status": ([vp, C.c_int, C.POINTER(C.c_int)], C.c_int),
        "lfm_batch_memory": ([vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], C.c_int),
        "lfm_batch_cells": ([vp, _i64p, C.POINTER(C.c_int)], C.c_int),
        "lfm_batch_get_tuning": ([vp, C.POINTER(BatchTuning)], C.c_int),
        "lfm_batch_set_tuning": ([vp, C.POINTER(BatchTuning)], C.c_int),
        "lfm_batch_autotune": ([vp, C.c_int, C.POINTER(BatchTuning)], C.c_int),
        "lfm_batch_bench": ([vp, C.c_int, C.c_size_t, C.POINTER(C.c_float)], C.c_int),
        "lfm_batch_launches_per_step": ([vp, C.POINTER(C.c_int)], C.c_int),
        "lfm_batch_debug_barrier": ([vp, C.c_int], C.c_int),
        "lfm_server_create": ([C.POINTER(ServerOpts), C.POINTER(vp)], C.c_int),
        "lfm_server_destroy": ([vp], None),
        "lfm_server_submit": ([vp, C.POINTER(SolverDesc), C.c_double, C.c_int, C.POINTER(C.c_int64)], C.c_int),
        "lfm_server_info": ([vp, C.c_int64, C.POINTER(RequestInfo)], C.c_int),
        "lfm_server_wait": ([vp, C.c_int64, C.c_double, C.POINTER(C.c_int)], C.c_int),
        "lfm_server_result": ([vp, C.c_int64, _dp, C.POINTER(RequestInfo)], C.c_int),
        "lfm_server_get_stats": ([vp, C.POINTER(ServerStats)], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = load_library().lfm_last_error().decode(errors="replace")
        raise LfmError(rc, msg)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class CaseHandle:
    """An lfm_case: the host-side solver setup of one case."""

    def __init__(self, handle: C.c_void_p, keep=()):
        self._h = handle
        self._keep = keep
        self.desc = SolverDesc()
        check(load_library().lfm_case_describe(self._h, C.byref(self.desc)))

    @classmethod
    def open(cls, root: str, rank: int = -1) -> "CaseHandle":
        lib = load_library()
        h = C.c_void_p()
        check(lib.lfm_case_open(root.encode(), rank, C.byref(h)))
        return cls(h)

    @classmethod
    def from_case(cls, case, renumber: int = 0) -> "CaseHandle":
        """From an in-memory lfm_public_gb300.cases.Case; ``renumber``: solver
        order inside each submesh (LFM_RENUMBER_NONE / _RCM / _HILBERT)."""
        lib = load_library()
        pts = np.ascontiguousarray(case.points, dtype=np.float64)
        fo = np.ascontiguousarray(case.face_offsets, dtype=np.int64)
        fp = np.ascontiguousarray(case.face_points, dtype=np.int64)
        own = np.ascontiguousarray(case.owner, dtype=np.int64)
        nei = np.ascontiguousarray(case.neighbour, dtype=np.int64)
        names = (C.c_char_p * len(case.patches))(*[p.name.encode() for p in case.patches])
        types = (C.c_char_p * len(case.patches))(*[p.type.encode() for p in case.patches])
        nbrs = (C.c_char_p * len(case.patches))(*[(p.neighbour.encode() if p.neighbour else None)
                                                  for p in case.patches])
        starts = np.array([p.start for p in case.patches], dtype=np.int64)
        sizes = np.array([p.size for p in case.patches], dtype=np.int64)
        m = PolyMesh(n_points=pts.shape[0], points=_ptr(pts, C.c_double), n_faces=own.shape[0],
                     face_offsets=_ptr(fo, C.c_int64), face_points=_ptr(fp, C.c_int64), owner=_ptr(own, C.c_int64),
                     n_internal_faces=nei.shape[0], neighbour=_ptr(nei, C.c_int64), n_patches=len(case.patches),
                     patch_name=names, patch_type=types, patch_start=_ptr(starts, C.c_int64),
                     patch_size=_ptr(sizes, C.c_int64), patch_neighbour=nbrs, cell_submesh=None,
                     n_cells=case.n_cells)
        pr = case.params()
        prm = Params(solver=pr["solver"], dimension=pr["dimension"], rk_order=pr["rk_order"], minmod=pr["minmod"],
                     laminar=pr["laminar"], residuals=pr["residuals"], p_inf=pr["p_inf"], T_inf=pr["T_inf"],
                     U_inf=(C.c_double * 3)(*pr["U_inf"]), Ls=pr["Ls"], mach=pr["mach"], k_sponge=pr["k_sponge"],
                     Cp=pr["Cp"], mol_weight=pr["mol_weight"], mu=pr["mu"], Pr=pr["Pr"], renumber=renumber)
        p = np.ascontiguousarray(case.fields["p"], dtype=np.float64)
        T = np.ascontiguousarray(case.fields["T"], dtype=np.float64)
        U = np.ascontiguousarray(case.fields["U"], dtype=np.float64)
        al = case.fields.get("alpha")
        al = np.ascontiguousarray(al, dtype=np.float64) if al is not None else None
        fl = Fields(p=_ptr(p, C.c_double), T=_ptr(T, C.c_double), U=_ptr(U, C.c_double),
                    alpha=_ptr(al, C.c_double) if al is not None else None)
        h = C.c_void_p()
        check(lib.lfm_case_from_polymesh(C.byref(m), C.byref(prm), C.byref(fl), C.byref(h)))
        return cls(h)

    def time(self):
        lib = load_library()
        dt, t0, t1, mc = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        adj = C.c_int()
        check(lib.lfm_case_time(self._h, C.byref(dt), C.byref(t0), C.byref(t1), C.byref(adj), C.byref(mc)))
        return dict(delta_t=dt.value, start_time=t0.value, end_time=t1.value, adjust=bool(adj.value),
                    max_co=mc.value)

    def cell_ids(self) -> np.ndarray:
        out = np.empty(self.desc.n_cells, dtype=np.int64)
        check(load_library().lfm_case_cell_ids(self._h, _ptr(out, C.c_int64)))
        return out

    def q0(self) -> np.ndarray:
        d = self.desc
        return np.ctypeslib.as_array(d.q0, shape=(d.nq * d.n_cells,)).reshape(d.nq, d.n_cells).copy()

    def array(self, name: str, shape, dtype=np.float64) -> np.ndarray:
        ptr = getattr(self.desc, name)
        return np.ctypeslib.as_array(ptr, shape=shape).copy()

    def close(self):
        if self._h:
            load_library().lfm_case_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """An lfm_solver on one GPU."""

    def __init__(self, case: CaseHandle, precision: int = LFM_FP64, device: int = 0):
        lib = load_library()
        self.case = case
        self.nq = case.desc.nq
        self.n_cells = case.desc.n_cells
        opts = SolverOpts(precision=precision, device=device, block=0)
        h = C.c_void_p()
        check(lib.lfm_solver_create(C.byref(case.desc), C.byref(opts), C.byref(h)))
        self._h = h

    def set_state(self, q: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.nq, self.n_cells)
        check(load_library().lfm_solver_set_state(self._h, _ptr(q, C.c_double)))

    def get_state(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """State [nq][n_cells] in solver order, into ``out`` when given (a
        C-contiguous float64 array of that shape, e.g. in pinned memory)."""
        if out is None:
            out = np.empty((self.nq, self.n_cells), dtype=np.float64)
        elif out.dtype != np.float64 or out.shape != (self.nq, self.n_cells) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape (nq, n_cells)")
        check(load_library().lfm_solver_get_state(self._h, _ptr(out, C.c_double)))
        return out

    def step(self, nsteps: int, dt: float):
        check(load_library().lfm_solver_step(self._h, nsteps, dt))

    def advance(self, q_in: Optional[np.ndarray], nsteps: int, dt: float, q_out: Optional[np.ndarray] = None):
        """Host state in (or None), nsteps steps, host state out (into q_out,
        a C-contiguous float64 (nq, n_cells) array, or None), one sync."""
        shape = (self.nq, self.n_cells)
        for a in (q_in, q_out):
            if a is not None and (a.dtype != np.float64 or a.shape != shape or not a.flags.c_contiguous):
                raise ValueError("states must be C-contiguous float64 arrays of shape (nq, n_cells)")
        pin = _ptr(q_in, C.c_double) if q_in is not None else None
        pout = _ptr(q_out, C.c_double) if q_out is not None else None
        check(load_library().lfm_solver_advance(self._h, pin, nsteps, dt, pout))
        return q_out

    def stage(self, rk: int, dt: float):
        check(load_library().lfm_solver_stage(self._h, rk, dt))

    def step_timed(self, nsteps: int, dt: float) -> float:
        ms = C.c_float()
        check(load_library().lfm_solver_step_timed(self._h, nsteps, dt, C.byref(ms)))
        return ms.value

    def sync(self):
        check(load_library().lfm_solver_sync(self._h))

    def cfl(self, dt: float) -> float:
        v = C.c_double()
        check(load_library().lfm_solver_cfl(self._h, dt, C.byref(v)))
        return v.value

    def min_dt(self, max_co: float) -> float:
        v = C.c_double()
        check(load_library().lfm_solver_min_dt(self._h, max_co, C.byref(v)))
        return v.value

    def residual(self) -> np.ndarray:
        out = np.empty(self.nq)
        check(load_library().lfm_solver_residual(self._h, _ptr(out, C.c_double)))
        return out

    def bench(self, nsteps: int, dt: float, flush_bytes: int = 512 << 20) -> np.ndarray:
        ms = (C.c_float * nsteps)()
        check(load_library().lfm_solver_bench(self._h, nsteps, dt, flush_bytes, ms))
        return np.array(ms[:], dtype=np.float64)

    def flush_l2(self, nbytes: int = 512 << 20):
        check(load_library().lfm_solver_flush_l2(self._h, nbytes))

    def cell_residual(self) -> np.ndarray:
        out = np.empty((self.nq, self.n_cells), dtype=np.float64)
        check(load_library().lfm_solver_cell_residual(self._h, _ptr(out, C.c_double)))
        return out

    # post-processing ------------------------------------------------------
    def stats_reset(self):
        check(load_library().lfm_solver_stats_reset(self._h))

    def stats_accumulate(self, n: int):
        check(load_library().lfm_solver_stats_accumulate(self._h, n))

    def stats_get(self, n: int):
        """(p_avg, p_rms) per cell, solver order."""
        a = np.empty(self.n_cells)
        r = np.empty(self.n_cells)
        check(load_library().lfm_solver_stats_get(self._h, n, _ptr(a, C.c_double), _ptr(r, C.c_double)))
        return a, r

    def forces(self, patches) -> tuple:
        """(pressure, viscous) force [len(patches)][dim] on the given patches."""
        p = np.ascontiguousarray(patches, dtype=np.int32)
        D = self.case.desc.dim
        fp = np.empty((len(p), D))
        fv = np.empty((len(p), D))
        check(load_library().lfm_solver_forces(self._h, len(p), _ptr(p, C.c_int32), _ptr(fp, C.c_double),
                                               _ptr(fv, C.c_double)))
        return fp, fv

    def probes_set(self, cells, capacity: int):
        c = np.ascontiguousarray(cells, dtype=np.int64)
        self._nprobes = len(c)
        self._probe_cap = capacity
        check(load_library().lfm_solver_probes_set(self._h, len(c), _ptr(c, C.c_int64), capacity))

    def probes_record(self):
        check(load_library().lfm_solver_probes_record(self._h))

    def probes_read(self) -> np.ndarray:
        out = np.empty((max(self._probe_cap, 1), self._nprobes))
        n = C.c_int()
        check(load_library().lfm_solver_probes_read(self._h, _ptr(out, C.c_double), C.byref(n)))
        return out[:n.value]

    def launches_per_step(self) -> int:
        v = C.c_int()
        check(load_library().lfm_solver_launches_per_step(self._h, C.byref(v)))
        return v.value

    def tuning(self) -> SolverTuning:
        t = SolverTuning()
        check(load_library().lfm_solver_get_tuning(self._h, C.byref(t)))
        return t

    def set_tuning(self, flux_kernel: int, staging_depth: int = 0, staging_faces: int = 0):
        t = SolverTuning(flux_kernel, staging_depth, staging_faces, 0.0)
        check(load_library().lfm_solver_set_tuning(self._h, C.byref(t)))

    def autotune(self, dt: float, trial_steps: int = 5, flush_bytes: int = 512 << 20, tried: list = None
                 ) -> SolverTuning:
        """Times every applicable flux kernel configuration and keeps the
        fastest (lfm_solver_autotune); the state is restored. `tried`, a list,
        receives every configuration timed."""
        t = SolverTuning()
        cap = 32
        arr = (SolverTuning * cap)()
        n = C.c_int()
        check(load_library().lfm_solver_autotune(self._h, dt, trial_steps, flush_bytes, C.byref(t), arr, cap,
                                                 C.byref(n)))
        if tried is not None:
            tried.extend(arr[i] for i in range(min(n.value, cap)))
        return t

    def profile_step(self, dt: float) -> dict:
        """ms per time step of each kernel; kernels that did not run are left out."""
        lib = load_library()
        n = 7
        ms = (C.c_float * n)()
        check(lib.lfm_solver_profile_step(self._h, dt, n, ms))
        names = [lib.lfm_solver_kernel_name(i).decode() for i in range(n)]
        if ms[5] > 0:   # fused tile stages
            return {names[5]: ms[5]}
        if ms[6] != 0:  # fused flux + update stages
            return {names[i]: ms[i] for i in (0, 1, 2, 6)}
        return {names[i]: ms[i] for i in range(5)}

    def close(self):
        if getattr(self, "_h", None):
            load_library().lfm_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PartitionedCase:
    """An lfm_pcase: every partition (processor0..N-1) of a decomposed case."""

    def __init__(self, root: str, nparts: int):
        lib = load_library()
        h = C.c_void_p()
        check(lib.lfm_pcase_open(root.encode(), nparts, C.byref(h)))
        self._h = h
        self.nparts = nparts
        self.descs = []
        for p in range(nparts):
            d = SolverDesc()
            check(lib.lfm_pcase_describe(h, p, C.byref(d)))
            self.descs.append(d)

    def cell_global(self, part: int) -> np.ndarray:
        out = np.empty(self.descs[part].n_cells, dtype=np.int64)
        check(load_library().lfm_pcase_cell_global(self._h, part, _ptr(out, C.c_int64)))
        return out

    def delta_t(self) -> float:
        v = C.c_double()
        check(load_library().lfm_pcase_time(self._h, C.byref(v), None, None, None, None))
        return v.value

    def q0(self, part: int) -> np.ndarray:
        d = self.descs[part]
        return np.ctypeslib.as_array(d.q0, shape=(d.nq * d.n_cells,)).reshape(d.nq, d.n_cells).copy()

    def close(self):
        if getattr(self, "_h", None):
            load_library().lfm_pcase_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Partitioned:
    """An lfm_partitioned: every partition of a decomposed case on one GPU,
    halos exchanged by on-device copies."""

    def __init__(self, pcase: PartitionedCase, precision: int = LFM_FP64, device: int = 0):
        lib = load_library()
        self.pcase = pcase
        arr = (C.POINTER(SolverDesc) * pcase.nparts)(*[C.pointer(d) for d in pcase.descs])
        opts = SolverOpts(precision=precision, device=device, block=0)
        h = C.c_void_p()
        check(lib.lfm_partitioned_create(arr, pcase.nparts, C.byref(opts), C.byref(h)))
        self._h = h

    def step(self, nsteps: int, dt: float):
        check(load_library().lfm_partitioned_step(self._h, nsteps, dt))

    def sync(self):
        check(load_library().lfm_partitioned_sync(self._h))

    def set_state(self, part: int, q: np.ndarray):
        d = self.pcase.descs[part]
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(d.nq, d.n_cells)
        check(load_library().lfm_partitioned_set_state(self._h, part, _ptr(q, C.c_double)))

    def get_state(self, part: int) -> np.ndarray:
        d = self.pcase.descs[part]
        out = np.empty((d.nq, d.n_cells), dtype=np.float64)
        check(load_library().lfm_partitioned_get_state(self._h, part, _ptr(out, C.c_double)))
        return out

    def global_state(self, n_global: int) -> np.ndarray:
        """State of the whole case [nq][n_global] by global (undecomposed) cell."""
        nq = self.pcase.descs[0].nq
        out = np.full((nq, n_global), np.nan)
        for p in range(self.pcase.nparts):
            out[:, self.pcase.cell_global(p)] = self.get_state(p)
        return out

    def close(self):
        if getattr(self, "_h", None):
            load_library().lfm_partitioned_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """An lfm_batch: many cases advanced together (FP32-bulk) on one GPU."""

    def __init__(self, device: int = 0, rk_order: int = 5, arena_bytes: int = 0, max_cases: int = 256):
        lib = load_library()
        opts = BatchOpts(device=device, rk_order=rk_order, arena_bytes=arena_bytes, max_cases=max_cases)
        h = C.c_void_p()
        check(lib.lfm_batch_create(C.byref(opts), C.byref(h)))
        self._h = h
        self._cases = {}

    @staticmethod
    def case_bytes(case: CaseHandle) -> int:
        v = C.c_size_t()
        check(load_library().lfm_batch_case_bytes(C.byref(case.desc), C.byref(v)))
        return v.value

    def add(self, case: CaseHandle, dt: float) -> int:
        s = C.c_int()
        check(load_library().lfm_batch_add(self._h, C.byref(case.desc), dt, C.byref(s)))
        self._cases[s.value] = case
        return s.value

    def remove(self, slot: int):
        check(load_library().lfm_batch_remove(self._h, slot))
        self._cases.pop(slot, None)

    def set_state(self, slot: int, q: np.ndarray):
        d = self._cases[slot].desc
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(d.nq, d.n_cells)
        check(load_library().lfm_batch_set_state(self._h, slot, _ptr(q, C.c_double)))

    def get_state(self, slot: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        d = self._cases[slot].desc
        if out is None:
            out = np.empty((d.nq, d.n_cells), dtype=np.float64)
        check(load_library().lfm_batch_get_state(self._h, slot, _ptr(out, C.c_double)))
        return out

    def step(self, nsteps: int = 1):
        check(load_library().lfm_batch_step(self._h, nsteps))

    def advance(self, slots, q_in, nsteps: int, q_out):
        """lfm_batch_advance: the states q_in[i] (or None) of slots[i] in,
        nsteps steps, the states out into q_out[i] (or None), one sync. The
        arrays are C-contiguous float64 (nq, n_cells) of their case."""
        n = len(slots)

        def ptrs(arrs):
            if arrs is None:
                return None
            out = (_dp * n)()
            for i, (s, a) in enumerate(zip(slots, arrs)):
                if a is None:
                    continue
                d = self._cases[s].desc
                if a.dtype != np.float64 or a.shape != (d.nq, d.n_cells) or not a.flags.c_contiguous:
                    raise ValueError("states must be C-contiguous float64 arrays of shape (nq, n_cells)")
                out[i] = _ptr(a, C.c_double)
            return out

        pin, pout = ptrs(q_in), ptrs(q_out)
        sl = (C.c_int * n)(*slots)
        check(load_library().lfm_batch_advance(self._h, n, sl, pin, nsteps, pout))

    def sync(self):
        check(load_library().lfm_batch_sync(self._h))

    def case_status(self, slot: int) -> int:
        v = C.c_int()
        check(load_library().lfm_batch_case_status(self._h, slot, C.byref(v)))
        return v.value

    def memory(self) -> dict:
        a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
        check(load_library().lfm_batch_memory(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"largest_free": a.value, "total_free": b.value, "arena": c.value}

    def cells(self) -> int:
        n = C.c_int64()
        check(load_library().lfm_batch_cells(self._h, C.byref(n), None))
        return n.value

    def tuning(self) -> dict:
        t = BatchTuning()
        check(load_library().lfm_batch_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, block: int, items_per_thread: int = 1, blocks_per_sm: int = 0, cooperative: int = 1,
                   phased: int = 0):
        t = BatchTuning(block=block, items_per_thread=items_per_thread, blocks_per_sm=blocks_per_sm,
                        cooperative=cooperative, phased=phased)
        check(load_library().lfm_batch_set_tuning(self._h, C.byref(t)))

    def autotune(self, trial_steps: int = 2) -> dict:
        t = BatchTuning()
        check(load_library().lfm_batch_autotune(self._h, trial_steps, C.byref(t)))
        return t.as_dict()

    def bench(self, nsteps: int, flush_bytes: int = 512 << 20) -> np.ndarray:
        ms = (C.c_float * nsteps)()
        check(load_library().lfm_batch_bench(self._h, nsteps, flush_bytes, ms))
        return np.array(ms[:], dtype=np.float64)

    # post-processing ------------------------------------------------------
    def stats_reset(self):
        check(load_library().lfm_solver_stats_reset(self._h))

    def stats_accumulate(self, n: int):
        check(load_library().lfm_solver_stats_accumulate(self._h, n))

    def stats_get(self, n: int):
        """(p_avg, p_rms) per cell, solver order."""
        a = np.empty(self.n_cells)
        r = np.empty(self.n_cells)
        check(load_library().lfm_solver_stats_get(self._h, n, _ptr(a, C.c_double), _ptr(r, C.c_double)))
        return a, r

    def forces(self, patches) -> tuple:
        """(pressure, viscous) force [len(patches)][dim] on the given patches."""
        p = np.ascontiguousarray(patches, dtype=np.int32)
        D = self.case.desc.dim
        fp = np.empty((len(p), D))
        fv = np.empty((len(p), D))
        check(load_library().lfm_solver_forces(self._h, len(p), _ptr(p, C.c_int32), _ptr(fp, C.c_double),
                                               _ptr(fv, C.c_double)))
        return fp, fv

    def probes_set(self, cells, capacity: int):
        c = np.ascontiguousarray(cells, dtype=np.int64)
        self._nprobes = len(c)
        self._probe_cap = capacity
        check(load_library().lfm_solver_probes_set(self._h, len(c), _ptr(c, C.c_int64), capacity))

    def probes_record(self):
        check(load_library().lfm_solver_probes_record(self._h))

    def probes_read(self) -> np.ndarray:
        out = np.empty((max(self._probe_cap, 1), self._nprobes))
        n = C.c_int()
        check(load_library().lfm_solver_probes_read(self._h, _ptr(out, C.c_double), C.byref(n)))
        return out[:n.value]

    def launches_per_step(self) -> int:
        v = C.c_int()
        check(load_library().lfm_batch_launches_per_step(self._h, C.byref(v)))
        return v.value

    def debug_barrier(self, extra_arrivals: int):
        """Failure-detection test aid (lfm_batch_debug_barrier): the stage
        kernel's grid barriers wait for that many blocks beyond the grid."""
        check(load_library().lfm_batch_debug_barrier(self._h, extra_arrivals))

    def close(self):
        if getattr(self, "_h", None):
            load_library().lfm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """An lfm_server: continuous batching of solve requests on one GPU
    (thread-safe; the worker runs in the library)."""

    def __init__(self, device: int = 0, rk_order: int = 5, arena_bytes: int = 0, max_cases: int = 256,
                 chunk_steps: int = 50, max_bypass: int = 0, tuning: Optional[tuple] = None, solo_cells: int = 0,
                 max_solo: int = 0):
        t = BatchTuning()
        if tuning:
            t.block, t.items_per_thread, t.blocks_per_sm = tuning[:3]
            t.cooperative = tuning[3] if len(tuning) > 3 else 1
        opts = ServerOpts(device=device, rk_order=rk_order, arena_bytes=arena_bytes, max_cases=max_cases,
                          chunk_steps=chunk_steps, max_bypass=max_bypass, tuning=t, solo_cells=solo_cells,
                          max_solo=max_solo)
        h = C.c_void_p()
        check(load_library().lfm_server_create(C.byref(opts), C.byref(h)))
        self._h = h
        self._shape = {}

    def submit(self, case: CaseHandle, dt: float, nsteps: int) -> int:
        i = C.c_int64()
        check(load_library().lfm_server_submit(self._h, C.byref(case.desc), dt, nsteps, C.byref(i)))
        self._shape[i.value] = (case.desc.nq, case.desc.n_cells)
        return i.value

    def info(self, rid: int) -> dict:
        r = RequestInfo()
        check(load_library().lfm_server_info(self._h, rid, C.byref(r)))
        return r.as_dict()

    def wait(self, rid: int, timeout: float = -1.0) -> bool:
        d = C.c_int()
        check(load_library().lfm_server_wait(self._h, rid, timeout, C.byref(d)))
        return bool(d.value)

    def result(self, rid: int):
        """(state [nq][n_cells], info dict) of a done request; releases it."""
        nq, nc = self._shape.pop(rid)
        q = np.empty((nq, nc), dtype=np.float64)
        r = RequestInfo()
        check(load_library().lfm_server_result(self._h, rid, _ptr(q, C.c_double), C.byref(r)))
        return q, r.as_dict()

    def stats(self) -> dict:
        s = ServerStats()
        check(load_library().lfm_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if getattr(self, "_h", None):
            load_library().lfm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_fp_convert(f32_bits: np.ndarray, f64_bits: np.ndarray):
    """Device integer-pipe conversions of the FP32-bulk kernels over bit
    patterns: (binary64 bits of each binary32, binary32 bits of each binary64)."""
    a = np.ascontiguousarray(f32_bits, dtype=np.uint32)
    b = np.ascontiguousarray(f64_bits, dtype=np.uint64)
    if a.size != b.size:
        raise ValueError("both inputs need the same length")
    o64 = np.empty(a.size, dtype=np.uint64)
    o32 = np.empty(a.size, dtype=np.uint32)
    rc = load_library().lfm_selftest_fp_convert(a.size, _ptr(a, C.c_uint32), _ptr(b, C.c_uint64),
                                                _ptr(o64, C.c_uint64), _ptr(o32, C.c_uint32))
    if rc != 0:
        raise LfmError(rc, "conversion self-test failed to run")
    return o64, o32
