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
from tests.helpers import adaptive_run, adjust_names, config_case, golden_names, load_golden, primitives


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


@pytest.mark.parametrize("name", adjust_names())
def test_port_adaptive_dt_matches_reference(name):
    """adjustTimeStep yes: the reference's compute_dt minimum sets every next
    dt (src/cfd_v0.cpp:2912-2942, src/mesh_solver.cpp:705-716). The oracle,
    set up by its own code and run through the same time loop, takes the same
    number of steps, prints the same dt and time at every step (10 significant
    digits, the reference's output precision) and ends on the reference's
    fields bit for bit."""
    case, z = load_golden(name)
    pc = P.PortCase.from_case(case)
    state = {"q": pc.q0()}
    max_co = float(z["max_co"])

    def step(dt):
        state["q"], _ = P.run(pc, state["q"], 1, dt)

    dts, times = adaptive_run(step, lambda: P.min_dt(pc, state["q"], max_co), case, z)
    assert len(dts) == len(z["ref_dt"])
    np.testing.assert_allclose(dts, z["ref_dt"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(times, z["ref_time"], rtol=1e-9, atol=0)
    ids = pc.cell_ids()
    r, U, E, p = primitives(state["q"], pc.desc.gamma, case.dim)
    assert np.array_equal(r, z["ref_rho"][ids]) and np.array_equal(E, z["ref_E"][ids])
    assert np.array_equal(p, z["ref_p"][ids])


def test_port_matches_reference_at_configured_cylinder_size():
    """The 768 x 512 cylinder for 20 steps (100 RK stages): the oracle, set up
    by its own code, gives the reference's written fields bit for bit on the
    fixture's 4096 sampled cells."""
    case, z = config_case("cfg_cyl768x512_m1_20")
    pc = P.PortCase.from_case(case)
    q, _ = P.run(pc, pc.q0(), int(z["n_steps"]), case.delta_t)
    inv = np.empty(pc.desc.n_cells, dtype=np.int64)
    inv[pc.cell_ids()] = np.arange(pc.desc.n_cells)
    r, U, E, p = primitives(q[:, inv[z["sample"]]], pc.desc.gamma, case.dim)
    assert np.array_equal(r, z["ref_rho"]) and np.array_equal(E, z["ref_E"]) and np.array_equal(p, z["ref_p"])
