"""Tiles of the fused FP32-bulk stage kernel (host builder; every local index
is checked against its tile's counts by the builder itself)."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases


def _stats(ch, tile_cells, max_local=1 << 30):
    out = (N.C.c_int64 * 5)()
    N.check(N.load_library().lfm_tiles_stats(N.C.byref(ch.desc), tile_cells, max_local, out))
    return dict(zip(("tiles", "max_local_cells", "max_local_faces", "local_cells", "flux_faces"), out[:]))


@pytest.mark.parametrize("make,renumber", [
    (lambda: cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=0), N.LFM_RENUMBER_NONE),
    (lambda: cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=0), N.LFM_RENUMBER_HILBERT),
    (lambda: cases.cylinder_case(n_theta=32, n_r=16, r1=10, first=0.03, Ls=3, solver=2, n_span=8), N.LFM_RENUMBER_HILBERT),
    (lambda: cases.tri_case(n=40, seed=9, solver=1), N.LFM_RENUMBER_RCM),
    (lambda: cases.vortex_case(n=48, solver=1, mu=1e-3), N.LFM_RENUMBER_NONE),
])
@pytest.mark.parametrize("tile_cells,max_local", [(1, 1 << 30), (97, 1 << 30), (256, 1 << 30), (256, 300)])
def test_tiles_cover_every_cell_once(make, renumber, tile_cells, max_local):
    ch = N.CaseHandle.from_case(make(), renumber=renumber)
    st = _stats(ch, tile_cells, max_local)
    nc = ch.desc.n_cells
    if max_local >= 1 << 30:
        assert st["tiles"] == -(-nc // tile_cells)
    else:   # oversized runs are halved until they fit (or are single cells)
        assert st["tiles"] >= -(-nc // tile_cells)
        assert st["max_local_cells"] <= max_local or st["tiles"] == nc
    # every cell of a tile and at least its neighbours are staged
    assert st["local_cells"] >= nc
    assert st["flux_faces"] >= ch.desc.n_faces


def test_hilbert_tiles_are_compact():
    c = cases.cylinder_case(n_theta=48, n_r=512, r1=30, first=0.01, Ls=8, solver=0)   # radial lines of 512
    strip = _stats(N.CaseHandle.from_case(c), 256)
    # cells staged per tile cell: a 256-cell run of a radial line is a strip
    # (two rings on both sides of it); renumbered, the runs are compact
    assert strip["local_cells"] > 4.5 * c.n_cells
    for method in (N.LFM_RENUMBER_RCM, N.LFM_RENUMBER_HILBERT):
        compact = _stats(N.CaseHandle.from_case(c, renumber=method), 256)
        assert compact["local_cells"] < 0.6 * strip["local_cells"], method
