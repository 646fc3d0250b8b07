"""ctypes binding of the oracle port (``oracle/port/liblfm_port.so``).

TEST INFRASTRUCTURE ONLY: tests, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` use it as the checker and the CPU baseline. The product path
never imports it. The port library carries its own case set-up
(``lfm_port_setup.c``), so ``PortCase.from_case`` builds a description
without loading the device library; ``run``/``cfl``/``min_dt`` also accept a
product ``CaseHandle`` (anything with a ``desc``), for tests that hold the
two set-ups side by side.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

# The C structures of include/lfm_gpu.h (plain ctypes declarations; importing
# them loads no library).
from lfm_public_gb300._native import Fields, Params, PolyMesh, SolverDesc

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "liblfm_port.so")

_dp = C.POINTER(C.c_double)
_port: Optional[C.CDLL] = None


def load(path: str = PORT_PATH) -> C.CDLL:
    """Loads liblfm_port.so (built by lfm_public_gb300.build.build_port)."""
    global _port
    if _port is not None:
        return _port
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with lfm_public_gb300.build.build_port()")
    lib = C.CDLL(path)
    vp = C.c_void_p
    sig = {
        "lfm_port_run": ([C.POINTER(SolverDesc), _dp, C.c_int, C.c_double, _dp], C.c_int),
        "lfm_port_run_cell_residual": ([C.POINTER(SolverDesc), _dp, C.c_int, C.c_double, _dp], C.c_int),
        "lfm_port_cfl": ([C.POINTER(SolverDesc), _dp, C.c_double, _dp], C.c_int),
        "lfm_port_min_dt": ([C.POINTER(SolverDesc), _dp, C.c_double, _dp], C.c_int),
        "lfm_port_case_build": ([C.POINTER(PolyMesh), C.POINTER(Params), C.POINTER(Fields), C.POINTER(vp)],
                                C.c_int),
        "lfm_port_case_describe": ([vp, C.POINTER(SolverDesc)], C.c_int),
        "lfm_port_case_free": ([vp], None),
        "lfm_port_case_cell_ids": ([vp, C.POINTER(C.c_int64)], C.c_int),
        "lfm_port_last_error": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _port = lib
    return lib


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def polymesh_args(case, renumber: int = 0):
    """The C structures (polyMesh, parameters, fields) of an in-memory
    ``lfm_public_gb300.cases.Case``, with the arrays they point into (keep
    the returned tuple alive while the structures are used)."""
    i64 = C.c_int64
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
                 face_offsets=_ptr(fo, i64), face_points=_ptr(fp, i64), owner=_ptr(own, i64),
                 n_internal_faces=nei.shape[0], neighbour=_ptr(nei, i64), n_patches=len(case.patches),
                 patch_name=names, patch_type=types, patch_start=_ptr(starts, i64), patch_size=_ptr(sizes, i64),
                 patch_neighbour=nbrs, cell_submesh=None, n_cells=case.n_cells)
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
    keep = (pts, fo, fp, own, nei, names, types, nbrs, starts, sizes, p, T, U, al)
    return m, prm, fl, keep


class PortCase:
    """A case set up by the oracle itself (lfm_port_case_build)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.desc = SolverDesc()
        rc = load().lfm_port_case_describe(self._h, C.byref(self.desc))
        if rc != 0:
            raise RuntimeError("lfm_port_case_describe failed")

    @classmethod
    def from_case(cls, case) -> "PortCase":
        lib = load()
        m, prm, fl, keep = polymesh_args(case)
        h = C.c_void_p()
        rc = lib.lfm_port_case_build(C.byref(m), C.byref(prm), C.byref(fl), C.byref(h))
        del keep
        if rc != 0:
            raise RuntimeError("oracle case set-up failed: " + lib.lfm_port_last_error().decode(errors="replace"))
        return cls(h)

    def cell_ids(self) -> np.ndarray:
        """polyMesh cell label of each solver-order cell."""
        out = np.empty(self.desc.n_cells, dtype=np.int64)
        load().lfm_port_case_cell_ids(self._h, _ptr(out, C.c_int64))
        return out

    def q0(self) -> np.ndarray:
        d = self.desc
        return np.ctypeslib.as_array(d.q0, shape=(d.nq * d.n_cells,)).reshape(d.nq, d.n_cells).copy()

    def close(self):
        if self._h:
            load().lfm_port_case_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(case, q: np.ndarray, nsteps: int, dt: float, residual: bool = False):
    """The oracle on a copy of q: (q after nsteps, summed squared residual or None)."""
    qq = np.ascontiguousarray(q, dtype=np.float64).copy()
    res = np.zeros(case.desc.nq)
    rc = load().lfm_port_run(C.byref(case.desc), _ptr(qq, C.c_double), nsteps, dt,
                             _ptr(res, C.c_double) if residual else None)
    if rc != 0:
        raise RuntimeError(f"oracle port failed with {rc}")
    return qq, (res if residual else None)


def cell_residual(case, q: np.ndarray, nsteps: int, dt: float):
    """The oracle: (q after nsteps, per-cell stage-0 residual of the last step)."""
    qq = np.ascontiguousarray(q, dtype=np.float64).copy()
    res = np.zeros((case.desc.nq, case.desc.n_cells))
    rc = load().lfm_port_run_cell_residual(C.byref(case.desc), _ptr(qq, C.c_double), nsteps, dt,
                                           _ptr(res, C.c_double))
    if rc != 0:
        raise RuntimeError(f"oracle port failed with {rc}")
    return qq, res


def cfl(case, q: np.ndarray, dt: float) -> float:
    v = C.c_double()
    qq = np.ascontiguousarray(q, dtype=np.float64)
    load().lfm_port_cfl(C.byref(case.desc), _ptr(qq, C.c_double), dt, C.byref(v))
    return v.value


def min_dt(case, q: np.ndarray, max_co: float) -> float:
    v = C.c_double()
    qq = np.ascontiguousarray(q, dtype=np.float64)
    load().lfm_port_min_dt(C.byref(case.desc), _ptr(qq, C.c_double), max_co, C.byref(v))
    return v.value
