"""Decomposed cases (processor0..N-1, as decomposePar writes them): the host
side that replaces the reference's MPI set-up of processor faces
(src/mesh_reader.cpp:374-611). CPU only: every partition's description must
reproduce, face by face, the geometry of the same face in the undecomposed
case, and every halo must point at the cell across its processor face."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases


def _arr(ptr, n, dtype=np.float64):
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype)


def _face_table(desc, gid):
    """(P global cell, N global cell or -1) -> (S, d, w) of every flux face."""
    nf, D = desc.n_faces, desc.dim
    fp, fn = _arr(desc.face_p, nf, np.int64), _arr(desc.face_n, nf, np.int64)
    S = _arr(desc.S, D * nf).reshape(D, nf)
    d = _arr(desc.d, D * nf).reshape(D, nf)
    w = _arr(desc.w, nf)
    nc, ng = desc.n_cells, desc.n_ghosts
    out = {}
    hs = _arr(desc.halo_src_cell, desc.n_halos, np.int64) if desc.n_halos else None
    hp = _arr(desc.halo_src_part, desc.n_halos, np.int64) if desc.n_halos else None
    for f in range(nf):
        p = gid[0][fp[f]]
        if fn[f] < nc:
            n = gid[0][fn[f]]
        elif fn[f] < nc + ng:
            continue   # boundary ghost
        else:
            h = fn[f] - nc - ng
            n = gid[1][hp[h]][hs[h]]
        out[(int(p), int(n))] = (S[:, f], d[:, f], w[f])
    return out


@pytest.mark.parametrize("method,span", [("x", 1), ("random", 1), ("x", 4)])
def test_partitions_reproduce_whole_case_geometry(tmp_path, method, span):
    case = cases.cylinder_case(n_theta=24, n_r=10, r1=8, first=0.05, Ls=3, solver=1, minmod=True, noise=0.01,
                               n_span=span)
    root = str(tmp_path / "case")
    part = cases.decompose_case(case, root, 3, method=method, seed=5)
    whole = N.CaseHandle.open(root)
    wid = whole.cell_ids()
    wt = _face_table(whole.desc, (wid, None))
    pc = N.PartitionedCase(root, 3)
    gids = [pc.cell_global(p) for p in range(3)]
    assert sorted(np.concatenate(gids).tolist()) == list(range(case.n_cells))
    n_halo = 0
    for p in range(3):
        d = pc.descs[p]
        n_halo += d.n_halos
        assert np.all(part[gids[p]] == p)
        pt = _face_table(d, (gids[p], gids))
        for key, (S, dv, w) in pt.items():
            # a face a partition owns, or a processor face (owned on both sides)
            if key in wt:
                S0, d0, w0 = wt[key]
            else:
                S0, d0, w0 = wt[(key[1], key[0])]
                S0, d0, w0 = -S0, -d0, 1.0 - w0
            assert np.allclose(S, S0, rtol=1e-12, atol=1e-14), key
            assert np.allclose(dv, d0, rtol=1e-11, atol=1e-12), key
            assert abs(w - w0) < 1e-11, key
    assert n_halo > 0
    pc.close()


@pytest.mark.parametrize("make", [lambda: cases.tet_case(n=4, nz=3, seed=2, solver=1),
                                  lambda: cases.hybrid_case(n=8, tri_fraction=0.4, seed=3)], ids=["tets", "quad+tri"])
def test_partitions_of_element_meshes_reproduce_geometry(tmp_path, make):
    """Random partitions of a tetrahedral and of a mixed quadrilateral /
    triangle mesh: every face of every partition is the undecomposed face."""
    case = make()
    root = str(tmp_path / "case")
    cases.decompose_case(case, root, 3, method="random", seed=7)
    whole = N.CaseHandle.open(root)
    wt = _face_table(whole.desc, (whole.cell_ids(), None))
    pc = N.PartitionedCase(root, 3)
    gids = [pc.cell_global(p) for p in range(3)]
    assert sorted(np.concatenate(gids).tolist()) == list(range(case.n_cells))
    n_halo = 0
    for p in range(3):
        d = pc.descs[p]
        n_halo += d.n_halos
        for key, (S, dv, w) in _face_table(d, (gids[p], gids)).items():
            if key in wt:
                S0, d0, w0 = wt[key]
            else:
                S0, d0, w0 = wt[(key[1], key[0])]
                S0, d0, w0 = -S0, -d0, 1.0 - w0
            assert np.allclose(S, S0, rtol=1e-12, atol=1e-14), key
            assert np.allclose(dv, d0, rtol=1e-11, atol=1e-12), key
            assert abs(w - w0) < 1e-11, key
    assert n_halo > 0
    pc.close()


def test_whole_case_open_rejects_a_single_partition(tmp_path):
    case = cases.vortex_case(n=12)
    root = str(tmp_path / "case")
    cases.decompose_case(case, root, 2)
    with pytest.raises(N.LfmError) as e:
        N.CaseHandle.open(root, rank=0)
    assert b"partition" in N.load_library().lfm_last_error() or "partition" in str(e.value)


def test_cyclic_pair_across_partitions_is_rejected(tmp_path):
    case = cases.cylinder_case(n_theta=16, n_r=8, r1=6, first=0.05, Ls=2, n_span=4)
    with pytest.raises(ValueError, match="cyclic"):
        cases.decompose_case(case, str(tmp_path / "c"), 3, method="random", seed=1)
