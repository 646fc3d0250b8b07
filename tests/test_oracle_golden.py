"""The oracle port against the reference's own outputs (golden fixtures).

The fixtures hold the fields the reference solver wrote (built from its own
sources, tests/golden/make_golden.py). The port is fed by this build's case
setup through the in-memory C ABI; both are compiled without FMA contraction,
so the match is exact up to the last bit on any host.
"""
import numpy as np
import pytest

import oracle.port as P
from lfm_public_gb300 import _native as N
from tests.helpers import golden_names, load_golden, primitives


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_bitwise(name):
    case, z = load_golden(name)
    ch = N.CaseHandle.from_case(case)
    q, _ = P.run(ch, ch.q0(), int(z["n_steps"]), case.delta_t)
    ids = ch.cell_ids()
    r, U, E, p = primitives(q, ch.desc.gamma, case.dim)
    assert np.array_equal(r, z["ref_rho"][ids])
    assert np.array_equal(E, z["ref_E"][ids])
    assert np.array_equal(p, z["ref_p"][ids])
    assert np.array_equal(U, z["ref_U"][ids][:, :case.dim].T)


@pytest.mark.parametrize("name", golden_names())
def test_port_cfl_matches_reference(name):
    case, z = load_golden(name)
    ch = N.CaseHandle.from_case(case)
    q, _ = P.run(ch, ch.q0(), int(z["n_steps"]), case.delta_t)
    cfl = P.cfl(ch, q, case.delta_t)
    # the reference prints 10 significant digits
    assert abs(cfl - float(z["ref_cfl"])) <= 1e-9 * abs(cfl)


def test_fixtures_cover_the_schemes_and_shapes():
    names = golden_names()
    assert any("m1" in n for n in names) and any("m2" in n for n in names) and any("ausm" in n for n in names)
    assert any("3d" in n for n in names) and any("tri" in n for n in names)
    # the 3D element types of the reference's 5- and 4-face solvers, one cell, rkOrder 3
    assert {"prism5x3_m2_3d", "tet3x2_ausm_3d", "vortex1_m1", "cyl16x8_m1_rk3"} <= set(names)
    assert load_golden("cyl16x8_m1_rk3")[0].rk_order == 3


def test_port_cell_residual_matches_reference_bitwise():
    case, z = load_golden("vortex12x20_m1_res")
    ch = N.CaseHandle.from_case(case)
    _, res = P.cell_residual(ch, ch.q0(), int(z["n_steps"]), case.delta_t)
    ids = ch.cell_ids()
    for v, name in enumerate(["rhoRES", "uRES", "vRES", "eRES"]):
        assert np.array_equal(res[v], z["ref_" + name][ids]), name
