"""The oracle port against the reference solver run here on fresh cases.

Needs oracle/_ref/lfm_oracle, which is built from the reference's own sources
(oracle/Makefile); skipped where those sources are not present.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import oracle.port as P
from lfm_public_gb300 import _native as N, cases
from tests.helpers import primitives

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "lfm_oracle")

pytestmark = pytest.mark.skipif(not os.path.exists(ORACLE), reason="reference oracle not built on this machine")


def _run_both(case, n):
    tmp = tempfile.mkdtemp(prefix="lfm_ref_")
    try:
        cases.write_case(case, tmp, n_steps=n)
        r = subprocess.run([ORACLE], cwd=tmp, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        ref = cases.read_result_fields(tmp)
        ch = N.CaseHandle.open(tmp)   # the file route: plugins read the case directory
        q, _ = P.run(ch, ch.q0(), n, ch.time()["delta_t"])
        return ch, q, ref
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


@pytest.mark.parametrize("seed", [11, 12])
def test_random_triangulation_bitwise(seed):
    case = cases.tri_case(n=6, seed=seed, solver=seed % 2, beta=2.0 + seed % 3)
    ch, q, ref = _run_both(case, 5)
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 2)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(p, ref["p"][ids])


def test_viscous_cylinder_ausm_bitwise():
    case = cases.cylinder_case(n_theta=20, n_r=10, r1=8, first=0.05, Ls=2, solver=2, minmod=True, noise=0.05,
                               seed=5, reynolds=40.0)
    ch, q, ref = _run_both(case, 6)
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 2)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(U, ref["U"][ids][:, :2].T)


@pytest.mark.parametrize("rk", [0, 1, 2, 3, 4])
def test_rk_orders_bitwise(rk):
    """Every rkOrder the reference accepts: 0 and 1 forward Euler (0 runs no
    stage: the state stays), 2 the two-stage set, 3 the first three stages of
    the four-stage low-storage set, 4 all four (src/cfd_v0.cpp:86-128; the
    stage loop runs rkOrder stages, src/mesh_solver.cpp:500)."""
    case = cases.cylinder_case(n_theta=16, n_r=8, r1=6, first=0.05, Ls=2, solver=rk % 2, minmod=True, noise=0.05,
                               seed=9, reynolds=60.0)
    case.rk_order = rk
    ch, q, ref = _run_both(case, 4)
    assert ch.desc.rk_order == rk
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 2)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(p, ref["p"][ids])
    if rk == 0:
        assert np.array_equal(q, ch.q0())


@pytest.mark.parametrize("make", [lambda: cases.vortex_case(n=1), lambda: cases.vortex_case(n=2),
                                  lambda: cases.vortex_case(n=3, ny=1), lambda: cases.tri_case(n=1, seed=3),
                                  lambda: cases.tri_case(n=2, seed=3, solver=1)],
                         ids=["1cell", "2x2", "3x1", "2tri", "8tri"])
def test_tiny_meshes_bitwise(make):
    """The smallest meshes: one cell (no internal face), every cell in the
    boundary submesh, two triangles."""
    case = make()
    ch, q, ref = _run_both(case, 3)
    assert ch.desc.n_cells0 == ch.desc.n_cells   # no interior submesh
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 2)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(p, ref["p"][ids])


@pytest.mark.parametrize("frac", [0.0, 1.0])
def test_polygon_mesh_generator_bitwise(frac):
    """The loop-based polygon generator behind the mixed-cell meshes gives the
    reference's results on all-quad and all-triangle grids. (A mesh that
    mixes quadrilaterals and triangles in one submesh stops the reference:
    its reorder_faces reads every one of the solver's FACE_CNT neighbour
    slots, src/cfd_v0.cpp:298-304, and a triangle's fourth is unset. The
    device path runs such meshes; tests/test_gpu_parity.py checks them
    against the oracle.)"""
    case = cases.hybrid_case(n=5, tri_fraction=frac, seed=3 + int(frac))
    ch, q, ref = _run_both(case, 4)
    assert ch.desc.n_cells == (50 if frac else 25)
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 2)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(p, ref["p"][ids])


@pytest.mark.parametrize("make,faces", [
    (lambda: cases.prism_case(n=4, nz=2, seed=1), 5),
    (lambda: cases.prism_case(n=5, nz=3, seed=2, solver=1), 5),
    (lambda: cases.tet_case(n=3, nz=2, seed=1), 4),
    (lambda: cases.tet_case(n=3, nz=2, seed=2, solver=2), 4),
], ids=["prism_m1", "prism_m2", "tet_m1", "tet_ausm"])
def test_3d_prisms_and_tetrahedra_bitwise(make, faces):
    """The reference's 3D solvers for five and four faces a cell
    (src/mesh_solver.cpp:56-70): extruded triangular prisms and Kuhn
    tetrahedra."""
    case = make()
    ch, q, ref = _run_both(case, 3)
    offs = np.ctypeslib.as_array(ch.desc.cell_face_offsets, shape=(ch.desc.n_cells + 1,))
    assert set(np.diff(offs).tolist()) == {faces}
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 3)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(p, ref["p"][ids])


@pytest.mark.parametrize("make", [lambda: cases.prism_case(n=4, nz=3, seed=5, solver=1),
                                  lambda: cases.tet_case(n=3, nz=2, seed=6, solver=0)], ids=["prism_m2", "tet_m1"])
def test_smagorinsky_les_on_prisms_and_tetrahedra_bitwise(make):
    """Smagorinsky LES (simulationType LES; the model constant built from
    each cell's volume) on 3D cells of five and four faces."""
    case = make()
    case.laminar = False
    case.mu = 1.8e-3
    ch, q, ref = _run_both(case, 3)
    assert ch.desc.smag_c
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, 3)
    assert np.array_equal(r, ref["rho"][ids]) and np.array_equal(E, ref["E"][ids])
    assert np.array_equal(U, ref["U"][ids].T)
