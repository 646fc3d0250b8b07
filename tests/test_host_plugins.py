"""Host layer: dictionary grammar, polyMesh reader, geometry, solver setup and
the error behaviour of the C ABI (no GPU needed)."""
import ctypes as C
import os
import re
import shutil
import tempfile

import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture()
def tmpdir_case():
    d = tempfile.mkdtemp(prefix="lfm_host_")
    yield d
    shutil.rmtree(d, ignore_errors=True)


def test_file_route_equals_memory_route(tmpdir_case):
    case = cases.cylinder_case(n_theta=12, n_r=6, r1=6, first=0.1, Ls=2, solver=2, minmod=True, noise=0.01)
    cases.write_case(case, tmpdir_case, n_steps=3)
    a = N.CaseHandle.open(tmpdir_case)
    b = N.CaseHandle.from_case(case)
    da, db = a.desc, b.desc
    for k in ("dim", "nq", "solver", "rk_order", "minmod", "n_cells", "n_cells0", "n_ghosts", "n_faces"):
        assert getattr(da, k) == getattr(db, k), k
    nf, D = da.n_faces, da.dim
    for name, shape in (("S", D * nf), ("d", D * nf), ("w", nf), ("K", D * nf), ("dmag_inv", nf),
                        ("vol_inv", da.n_cells), ("sponge", da.n_cells)):
        assert np.array_equal(a.array(name, (shape,)), b.array(name, (shape,))), name
    assert np.array_equal(a.q0(), b.q0())
    assert a.time()["delta_t"] == pytest.approx(case.delta_t, rel=1e-15)


def test_geometry_closed_cells_and_volumes():
    case = cases.tri_case(n=6, seed=1)
    ch = N.CaseHandle.from_case(case)
    d = ch.desc
    nf, nc = d.n_faces, d.n_cells
    S = ch.array("S", (2 * nf,)).reshape(2, nf)
    offs = ch.array("cell_face_offsets", (nc + 1,), np.int64)
    faces = ch.array("cell_faces", (offs[-1],), np.int64)
    sign = ch.array("cell_face_sign", (offs[-1],), np.int8)
    # every cell's outward face vectors (valid faces) close: sum S = 0
    for c in range(nc):
        tot = np.zeros(2)
        for e in range(offs[c], offs[c + 1]):
            tot += sign[e] * S[:, faces[e]]
        assert np.abs(tot).max() < 1e-12
    vol = 1.0 / ch.array("vol_inv", (nc,))
    assert np.all(vol > 0)
    assert vol.sum() == pytest.approx(400.0, rel=1e-12)   # [-10,10]^2 x 1


@pytest.mark.parametrize("make,volume,faces", [
    (lambda: cases.hybrid_case(n=6, tri_fraction=0.5, seed=1), 400.0, {3, 4}),
    (lambda: cases.prism_case(n=5, nz=3, seed=2), 1600.0, {5}),
    (lambda: cases.tet_case(n=3, nz=2, seed=1), 1600.0, {4}),
], ids=["quad+tri", "prisms", "tets"])
def test_generated_element_meshes_are_closed(make, volume, faces):
    """The mixed-polygon, prism and tetrahedron generators: every cell closed
    (its outward face vectors sum to zero), positive volumes filling the box,
    the expected faces per cell."""
    case = make()
    ch = N.CaseHandle.from_case(case)
    d = ch.desc
    nf, nc, D = d.n_faces, d.n_cells, d.dim
    S = ch.array("S", (D * nf,)).reshape(D, nf)
    offs = ch.array("cell_face_offsets", (nc + 1,), np.int64)
    fl = ch.array("cell_faces", (offs[-1],), np.int64)
    sign = ch.array("cell_face_sign", (offs[-1],), np.int8)
    assert set(np.diff(offs).tolist()) == faces
    for c in range(nc):
        tot = np.zeros(D)
        for e in range(offs[c], offs[c + 1]):
            tot += sign[e] * S[:, fl[e]]
        assert np.abs(tot).max() < 1e-11 * max(1.0, np.abs(S).max()), c
    vol = 1.0 / ch.array("vol_inv", (nc,))
    assert np.all(vol > 0)
    assert vol.sum() == pytest.approx(volume, rel=1e-12)


def test_ownership_and_processing_order():
    case = cases.vortex_case(n=8)
    ch = N.CaseHandle.from_case(case)
    d = ch.desc
    nf, nc = d.n_faces, d.n_cells
    P = ch.array("face_p", (nf,), np.int64)
    Nn = ch.array("face_n", (nf,), np.int64)
    assert np.all(np.diff(P) >= 0)
    assert np.all(Nn > P)                     # owned faces point to later cells or ghosts
    assert d.n_ghosts == 4 * 8                # inlet, outlet, two walls
    internal = Nn < nc
    assert internal.sum() == 2 * 8 * 7        # each internal face exactly once
    sm0 = d.n_cells0
    assert 0 < sm0 < nc                       # boundary submesh then interior


def test_submesh_split_marks_boundary_cells():
    case = cases.vortex_case(n=10)
    ch = N.CaseHandle.from_case(case)
    ids = ch.cell_ids()
    sm0 = set(ids[:ch.desc.n_cells0].tolist())
    for c in range(case.n_cells):
        i, j = c % 10, c // 10
        touches = i in (0, 9) or j in (0, 9) or i in (1, 8) and j in (0, 9)
        # cells sharing a point with the boundary: the outer ring only (a
        # point-based test also catches diagonal neighbours of corner cells,
        # which are already in the ring on a structured grid)
        assert (c in sm0) == (i in (0, 9) or j in (0, 9)), (i, j)


def _write_dicts(tmp, case, **over):
    cases.write_case(case, tmp, n_steps=2)
    for rel, old, new in over.get("edits", []):
        p = os.path.join(tmp, rel)
        s = open(p).read()
        assert old in s, (rel, old)
        open(p, "w").write(s.replace(old, new))


def test_dictionary_grammar(tmpdir_case):
    case = cases.vortex_case(n=6)
    _write_dicts(tmpdir_case, case, edits=[
        ("system/fvSchemes", "    solver          0;",
         "    // comment\n    solver          /* inline */ 1;\n    minmodExists yes;"),
        ("system/controlDict", "haveResiduals   false", "haveResiduals   on"),
    ])
    ch = N.CaseHandle.open(tmpdir_case)
    assert ch.desc.solver == 1
    assert ch.desc.residuals == 1


def test_missing_dictionary_is_an_io_error(tmpdir_case):
    case = cases.vortex_case(n=6)
    cases.write_case(case, tmpdir_case, n_steps=2)
    os.remove(os.path.join(tmpdir_case, "constant", "spongeDict"))
    with pytest.raises(N.LfmError) as e:
        N.CaseHandle.open(tmpdir_case)
    assert e.value.code == -2 and "spongeDict" in str(e.value)


def test_missing_mandatory_key(tmpdir_case):
    case = cases.vortex_case(n=6)
    _write_dicts(tmpdir_case, case, edits=[("constant/spongeDict", "Ls      2.0;", "")])
    with pytest.raises(N.LfmError) as e:
        N.CaseHandle.open(tmpdir_case)
    assert "Ls" in str(e.value)


def test_turbulent_case_selects_smagorinsky(tmpdir_case):
    """simulationType other than laminar: the Smagorinsky LES viscous pass
    (calc_VIS_Smagorinsky): every cell gets its model constant
    -2 (0.16 V^(1/3))^2."""
    case = cases.vortex_case(n=6)
    _write_dicts(tmpdir_case, case, edits=[("constant/turbulenceProperties", "laminar", "LES")])
    ch = N.CaseHandle.open(tmpdir_case)
    d = ch.desc
    c = np.ctypeslib.as_array(d.smag_c, shape=(d.n_cells,))
    vol = 1.0 / np.ctypeslib.as_array(d.vol_inv, shape=(d.n_cells,))
    np.testing.assert_allclose(c, -2.0 * (0.16 * vol ** (1.0 / 3.0)) ** 2, rtol=1e-15)
    lam = cases.vortex_case(n=6)
    _write_dicts(tmpdir_case, lam)
    assert not N.CaseHandle.open(tmpdir_case).desc.smag_c


def test_bad_solver_id(tmpdir_case):
    case = cases.vortex_case(n=6)
    _write_dicts(tmpdir_case, case, edits=[("system/fvSchemes", "solver          0;", "solver          7;")])
    with pytest.raises(N.LfmError) as e:
        N.CaseHandle.open(tmpdir_case)
    assert e.value.code == -1


def test_missing_case_directory():
    with pytest.raises(N.LfmError) as e:
        N.CaseHandle.open("/nonexistent/lfm/case")
    assert e.value.code == -2


def test_solver_create_rejects_bad_description():
    lib = N.load_library()
    h = C.c_void_p()
    assert lib.lfm_solver_create(None, None, C.byref(h)) == -1
    d = N.SolverDesc(dim=4, nq=6)
    assert lib.lfm_solver_create(C.byref(d), None, C.byref(h)) == -1
    assert b"dim" in lib.lfm_last_error()


def test_advance_calls_reject_bad_arguments():
    """lfm_solver_advance / lfm_batch_advance: a null handle or a negative
    count is LFM_ERR_INVALID before any device work."""
    lib = N.load_library()
    assert lib.lfm_solver_advance(None, None, 1, 1e-3, None) == N.LFM_ERR_INVALID
    assert lib.lfm_batch_advance(None, 0, None, None, 1, None) == N.LFM_ERR_INVALID
    assert b"bad argument" in lib.lfm_last_error()


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "lfm_gpu.h")).read()
    names = set(re.findall(r"\b(lfm_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 20
    lib = N.load_library()
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert N.load_library().lfm_version().startswith(b"lfm_public_gb300")


def test_time_names_and_write_control(tmpdir_case):
    case = cases.vortex_case(n=6)
    cases.write_case(case, tmpdir_case, n_steps=4, write_interval=2)
    t = N.CaseHandle.open(tmpdir_case).time()
    assert t["end_time"] == pytest.approx(4 * case.delta_t)
    assert not t["adjust"]
