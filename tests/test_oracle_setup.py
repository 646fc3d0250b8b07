"""The oracle's own case set-up (oracle/port/lfm_port_setup.c) against the
product's (lfm_case_from_polymesh), array by array and bit for bit.

The product's set-up is pinned to the reference build by the golden fixtures;
this pins the oracle's independent restatement to it, so that the CPU
baseline and the checks that use the oracle need nothing from the device
library. No GPU is used.
"""
import ctypes as C

import numpy as np
import pytest

import oracle.port as P
from lfm_public_gb300 import _native as N, cases
from tests.helpers import golden_names, load_golden


def _arr(desc, name, n, ctype):
    ptr = getattr(desc, name)
    if not ptr:
        return None
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,)).copy()


def _fields(desc):
    D, nc, nf, ng = desc.dim, desc.n_cells, desc.n_faces, desc.n_ghosts
    ncf = int(_arr(desc, "cell_face_offsets", nc + 1, C.c_int64)[-1])
    ncs = int(_arr(desc, "cell_s_offsets", nc + 1, C.c_int64)[-1])
    out = {
        "face_p": _arr(desc, "face_p", nf, C.c_int64), "face_n": _arr(desc, "face_n", nf, C.c_int64),
        "face_ghost": _arr(desc, "face_ghost", nf, C.c_uint8),
        "cell_face_offsets": _arr(desc, "cell_face_offsets", nc + 1, C.c_int64),
        "cell_faces": _arr(desc, "cell_faces", ncf, C.c_int64),
        "cell_face_sign": _arr(desc, "cell_face_sign", ncf, C.c_int8),
        "cell_s_offsets": _arr(desc, "cell_s_offsets", nc + 1, C.c_int64),
        "ghost_cell": _arr(desc, "ghost_cell", ng, C.c_int64), "ghost_kind": _arr(desc, "ghost_kind", ng, C.c_int),
        "ghost_patch": _arr(desc, "ghost_patch", ng, C.c_int32),
        "rkA": _arr(desc, "rkA", desc.rk_order, C.c_double), "rkB": _arr(desc, "rkB", desc.rk_order, C.c_double),
    }
    for name, n in [("S", D * nf), ("d", D * nf), ("w", nf), ("smag", nf), ("dmag_inv", nf), ("dnorm", D * nf),
                    ("delta_mag", nf), ("K", D * nf), ("vol_inv", nc), ("sponge", nc), ("cell_s", D * ncs),
                    ("q0", desc.nq * nc), ("smag_c", nc)]:
        out[name] = _arr(desc, name, n, C.c_double)
    for k in ("dim", "nq", "solver", "rk_order", "minmod", "residuals", "n_cells", "n_cells0", "n_ghosts", "n_faces",
              "n_halos", "gamma", "Rgas", "rhoInf", "EInf", "pInf", "TInf", "mu", "Cp", "PrInv"):
        out[k] = getattr(desc, k)
    out["UInf"] = tuple(desc.UInf)
    return out


def assert_same_setup(case):
    ch = N.CaseHandle.from_case(case)
    pc = P.PortCase.from_case(case)
    a, b = _fields(ch.desc), _fields(pc.desc)
    assert a.keys() == b.keys()
    for k in a:
        x, y = a[k], b[k]
        if isinstance(x, np.ndarray) or isinstance(y, np.ndarray):
            assert x is not None and y is not None, k
            assert x.dtype == y.dtype and x.shape == y.shape, k
            # bitwise (NaN-free arrays; -0.0 and 0.0 are told apart)
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k
        else:
            assert x == y or (x is None and y is None), (k, x, y)
    return ch, pc


@pytest.mark.parametrize("name", golden_names())
def test_setup_matches_product_on_fixture_meshes(name):
    case, _ = load_golden(name)
    assert_same_setup(case)


@pytest.mark.parametrize("make", [
    lambda: cases.vortex_case(n=20, solver=0),
    lambda: cases.cylinder_case(n_theta=48, n_r=24, solver=1, minmod=True, noise=0.01, seed=3),
    lambda: cases.cylinder_case(n_theta=16, n_r=8, n_span=4, solver=2, reynolds=3900.0, noise=0.01, seed=7),
    lambda: cases.tri_case(n=12, seed=4, solver=1),
    lambda: cases.hybrid_case(n=10, seed=2),
    lambda: cases.prism_case(n=6, nz=3, seed=1),
    lambda: cases.tet_case(n=4, nz=2, seed=2),
])
def test_setup_matches_product_on_generated_meshes(make):
    assert_same_setup(make())


def test_oracle_runs_the_same_on_either_setup():
    """The stage loop gives the same bits on either description."""
    case = cases.cylinder_case(n_theta=24, n_r=12, solver=0, minmod=True, noise=0.02, seed=9, reynolds=150.0)
    ch, pc = assert_same_setup(case)
    qa, _ = P.run(ch, ch.q0(), 3, case.delta_t)
    qb, _ = P.run(pc, pc.q0(), 3, case.delta_t)
    assert np.array_equal(qa, qb)


def test_setup_rejects_renumbering_and_bad_input():
    case = cases.vortex_case(n=8)
    m, prm, fl, keep = P.polymesh_args(case, renumber=1)
    h = C.c_void_p()
    assert P.load().lfm_port_case_build(C.byref(m), C.byref(prm), C.byref(fl), C.byref(h)) != 0
    m, prm, fl, keep = P.polymesh_args(case)
    prm.dimension = 4
    assert P.load().lfm_port_case_build(C.byref(m), C.byref(prm), C.byref(fl), C.byref(h)) != 0
