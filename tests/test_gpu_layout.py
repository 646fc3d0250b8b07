"""Device storage layouts that must not change a single bit.

Flux faces stored by owned-face slot (every cell's first owned face, then
every cell's second, ...) instead of the reference's processing order: each
face's rhs is computed from the same data and each cell still sums its faces
in processing order, so states, residuals and wall forces keep their bits,
in both precisions, 2D and 3D."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [N.LFM_FP64, N.LFM_FP32_BULK], ids=["fp64", "fp32_bulk"])
@pytest.mark.parametrize("make", [
    lambda: cases.cylinder_case(n_theta=48, n_r=24, r1=10, first=0.03, Ls=3, solver=0, minmod=True, noise=0.02,
                                seed=2, reynolds=150.0),
    lambda: cases.cylinder_case(n_theta=16, n_r=8, n_span=6, r1=6, first=0.05, Ls=2, solver=2, minmod=True,
                                noise=0.01, seed=4, reynolds=300.0),
    lambda: cases.tet_case(n=4, nz=3, seed=9, solver=1),
], ids=["o-grid-m1", "wake-3d-ausm", "tets-m2"])
def test_slot_face_order_keeps_the_bits(monkeypatch, make, precision):
    case = make()
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    walls = [i for i, p in enumerate(case.patches) if p.type == "wall"]
    out = {}
    for order in ("processing", "slot"):
        monkeypatch.setenv("LFM_FACE_ORDER", order)
        s = N.Solver(ch, precision=precision)
        s.step(6, case.delta_t)
        s.sync()
        q = s.get_state()
        res = s.cell_residual()
        f = s.forces(walls) if walls else (np.zeros(1), np.zeros(1))
        out[order] = (q, res, f[0], f[1])
        s.close()
    for a, b in zip(out["processing"], out["slot"]):
        assert np.array_equal(a, b)
