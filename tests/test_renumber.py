"""Cell renumbering (reverse Cuthill-McKee, Hilbert, the reference's
Hamiltonian path) of the solver order.

The polyMesh keeps its numbering; only the solver's cell order inside each
submesh changes, so results are those of the polyMesh order up to the
summation order of each cell's faces (FP64 within 1e-12 of the oracle run on
the unrenumbered case)."""
import numpy as np
import pytest

import oracle.port as P
from lfm_public_gb300 import _native as N, cases


def _order_stats(ch):
    d = ch.desc
    nf, nc, n0 = d.n_faces, d.n_cells, d.n_cells0
    fp = np.ctypeslib.as_array(d.face_p, shape=(nf,))
    fn = np.ctypeslib.as_array(d.face_n, shape=(nf,))
    m = (fn < nc) & (fp >= n0) & (fn >= n0)   # faces inside the interior submesh
    dist = np.abs(fp[m] - fn[m])
    return int(dist.max()), float(dist.mean())


@pytest.fixture(scope="module")
def shuffled():
    c = cases.cylinder_case(n_theta=48, n_r=24, r1=10, first=0.03, Ls=3, solver=1, noise=0.02)
    perm = np.random.default_rng(1).permutation(c.n_cells)
    return c, cases.renumber_cells(c, perm), perm


def test_renumber_cells_is_a_relabelling(shuffled):
    c, cs, perm = shuffled
    a = N.CaseHandle.from_case(c)
    b = N.CaseHandle.from_case(cs)
    assert a.desc.n_faces == b.desc.n_faces and a.desc.n_ghosts == b.desc.n_ghosts
    # the same geometry per cell, in the new labels
    va = np.ctypeslib.as_array(a.desc.vol_inv, shape=(c.n_cells,))[np.argsort(a.cell_ids())]
    vb = np.ctypeslib.as_array(b.desc.vol_inv, shape=(c.n_cells,))[np.argsort(b.cell_ids())]
    np.testing.assert_allclose(vb, va[perm], rtol=1e-12)


METHODS = [N.LFM_RENUMBER_RCM, N.LFM_RENUMBER_HILBERT, N.LFM_RENUMBER_HPATH]


@pytest.mark.parametrize("method", METHODS)
def test_renumbering_restores_locality(shuffled, method):
    c, cs, _ = shuffled
    base = _order_stats(N.CaseHandle.from_case(cs))
    ch = N.CaseHandle.from_case(cs, renumber=method)
    ids = ch.cell_ids()
    assert sorted(ids.tolist()) == list(range(c.n_cells))
    bw, mean = _order_stats(ch)
    assert mean < base[1] / 5, (mean, base)
    if method == N.LFM_RENUMBER_RCM:
        assert bw <= 2 * 48, bw   # about one ring of the O-grid


@pytest.mark.parametrize("method", METHODS)
def test_renumbered_case_matches_oracle(shuffled, method):
    c, cs, _ = shuffled
    n = 10
    a = N.CaseHandle.from_case(cs)
    qa, _ = P.run(a, a.q0(), n, c.delta_t)
    b = N.CaseHandle.from_case(cs, renumber=method)
    qb, _ = P.run(b, b.q0(), n, c.delta_t)
    ga = np.empty_like(qa)
    ga[:, a.cell_ids()] = qa
    gb = np.empty_like(qb)
    gb[:, b.cell_ids()] = qb
    err = np.linalg.norm(gb - ga, axis=1) / np.linalg.norm(ga, axis=1)
    assert np.all(err <= 1e-12), err


def test_controldict_renumber_option(tmp_path, shuffled):
    _, cs, _ = shuffled
    root = str(tmp_path / "c")
    cases.write_case(cs, root, n_steps=2)
    cd = tmp_path / "c" / "system" / "controlDict"
    cd.write_text(cd.read_text().replace("    doublePrecision true;", "    doublePrecision true;\n    renumber        rcm;"))
    ch = N.CaseHandle.open(root)
    assert _order_stats(ch)[0] <= 2 * 48
    cd.write_text(cd.read_text().replace("renumber        rcm;", "renumber        bogus;"))
    with pytest.raises(N.LfmError):
        N.CaseHandle.open(root)


@pytest.mark.gpu
@pytest.mark.parametrize("method", METHODS)
def test_renumbered_device_run_matches_oracle(shuffled, method):
    c, cs, _ = shuffled
    n = 10
    a = N.CaseHandle.from_case(cs)
    qa, _ = P.run(a, a.q0(), n, c.delta_t)
    ga = np.empty_like(qa)
    ga[:, a.cell_ids()] = qa
    b = N.CaseHandle.from_case(cs, renumber=method)
    for prec, tol in ((N.LFM_FP64, 1e-12), (N.LFM_FP32_BULK, 1e-5)):
        s = N.Solver(b, precision=prec)
        s.step(n, c.delta_t)
        s.sync()
        q = s.get_state()
        s.close()
        g = np.empty_like(q)
        g[:, b.cell_ids()] = q
        err = np.linalg.norm(g - ga, axis=1) / np.linalg.norm(ga, axis=1)
        assert np.all(err <= tol), (prec, err)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("make", [lambda: cases.prism_case(n=6, nz=3, seed=8, solver=1),
                                  lambda: cases.tet_case(n=4, nz=3, seed=9, solver=0)], ids=["prisms", "tets"])
def test_renumbered_3d_elements_match_oracle(make, method):
    """RCM and the 3D Hilbert order on prisms and tetrahedra: a permutation
    of the solver order whose oracle run matches the unrenumbered one to
    1e-12 (momentum as one vector: the prisms' w stays at rounding level)."""
    from tests.helpers import rel_l2_vec
    c = make()
    n = 5
    a = N.CaseHandle.from_case(c)
    b = N.CaseHandle.from_case(c, renumber=method)
    assert sorted(b.cell_ids().tolist()) == list(range(c.n_cells))
    qa, _ = P.run(a, a.q0(), n, c.delta_t)
    qb, _ = P.run(b, b.q0(), n, c.delta_t)
    ga = np.empty_like(qa)
    ga[:, a.cell_ids()] = qa
    gb = np.empty_like(qb)
    gb[:, b.cell_ids()] = qb
    err = rel_l2_vec(gb, ga, 3)
    assert np.all(err <= 1e-12), err


def _consecutive_adjacent(ch):
    """Fractions of consecutive solver cells that share a face, in the
    boundary and in the interior submesh."""
    d = ch.desc
    nf, nc, n0 = d.n_faces, d.n_cells, d.n_cells0
    fp = np.ctypeslib.as_array(d.face_p, shape=(nf,))
    fn = np.ctypeslib.as_array(d.face_n, shape=(nf,))
    m = fn < nc
    adj = set(zip(np.minimum(fp[m], fn[m]).tolist(), np.maximum(fp[m], fn[m]).tolist()))

    def frac(lo, hi):
        return sum((i, i + 1) in adj for i in range(lo, hi - 1)) / max(1, hi - lo - 1)
    return frac(0, n0), frac(n0, nc)


@pytest.mark.parametrize("make", [
    lambda: cases.vortex_case(n=32),
    lambda: cases.cylinder_case(n_theta=48, n_r=24, r1=10, first=0.03, Ls=3),
    lambda: cases.tri_case(n=12, seed=3),
    lambda: cases.hybrid_case(n=10, seed=2),
], ids=["quads", "o-grid", "triangles", "quads+triangles"])
def test_hpath_order_is_a_hamiltonian_walk(make):
    """The reference's hpath method (hpathRenumber/hpathRenumber.C:127-180)
    orders the boundary cells as one walk and the interior cells as another,
    the cells a walk had to skip following it: consecutive cells share a
    face almost everywhere (a random order: almost nowhere)."""
    c = make()
    ch = N.CaseHandle.from_case(c, renumber=N.LFM_RENUMBER_HPATH)
    assert sorted(ch.cell_ids().tolist()) == list(range(c.n_cells))
    b, i = _consecutive_adjacent(ch)
    assert b >= 0.9 and i >= 0.9, (b, i)
    # from a randomly numbered polyMesh the interior walk is found as well;
    # the boundary walk moves to the nearest boundary cell within ten rings,
    # so on an O-grid (wall ring and outer ring 24 cells apart) it covers one
    # ring and the other follows in polyMesh order, as in the reference
    cs = cases.renumber_cells(c, np.random.default_rng(5).permutation(c.n_cells))
    b2, i2 = _consecutive_adjacent(N.CaseHandle.from_case(cs, renumber=N.LFM_RENUMBER_HPATH))
    assert i2 >= 0.9 and b2 >= 0.45, (b2, i2)


def test_controldict_accepts_hpath(tmp_path, shuffled):
    _, cs, _ = shuffled
    root = str(tmp_path / "c")
    cases.write_case(cs, root, n_steps=2)
    cd = tmp_path / "c" / "system" / "controlDict"
    cd.write_text(cd.read_text().replace("    doublePrecision true;", "    doublePrecision true;\n    renumber        hpath;"))
    ch = N.CaseHandle.open(root)
    b, i = _consecutive_adjacent(ch)
    assert i >= 0.9 and b >= 0.45, (b, i)
