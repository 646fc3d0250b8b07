"""FP64 device path against the reference (golden fixtures) and the oracle.

Parity bar: relative L2 per conserved field <= 1e-12 after the fixture's RK
steps (100 RK stages for the 2D fixtures), and bitwise reproducibility run to
run."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases
from tests.helpers import golden_names, load_golden, reference_conserved, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gpu_run(ch, nsteps, dt, precision=N.LFM_FP64):
    s = N.Solver(ch, precision=precision)
    s.step(nsteps, dt)
    s.sync()
    q = s.get_state()
    s.close()
    return q


@pytest.mark.parametrize("name", golden_names())
def test_fp64_matches_reference_fixture(name):
    case, z = load_golden(name)
    ch = N.CaseHandle.from_case(case)
    q = _gpu_run(ch, int(z["n_steps"]), case.delta_t)
    ref = reference_conserved(z, ch.cell_ids(), case.dim)
    err = rel_l2(q, ref)
    assert np.all(err <= TOL), err


@pytest.mark.parametrize("solver,minmod", [(0, True), (1, False), (2, True), (2, False)])
def test_fp64_matches_oracle_cylinder(solver, minmod):
    case = cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=solver, minmod=minmod,
                               noise=0.02, seed=7)
    ch = N.CaseHandle.from_case(case)
    n = 20
    q_gpu = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = N.port_run(ch, ch.q0(), n, case.delta_t)
    assert np.all(rel_l2(q_gpu, q_ref) <= TOL), rel_l2(q_gpu, q_ref)


def test_fp64_matches_oracle_3d_and_triangles():
    for case, n in ((cases.cylinder_case(n_theta=32, n_r=16, r1=10, first=0.03, Ls=3, solver=2, minmod=True,
                                         n_span=8, noise=0.01), 10),
                    (cases.tri_case(n=40, seed=9, solver=0, beta=4.0), 20)):
        ch = N.CaseHandle.from_case(case)
        q_gpu = _gpu_run(ch, n, case.delta_t)
        q_ref, _ = N.port_run(ch, ch.q0(), n, case.delta_t)
        assert np.all(rel_l2(q_gpu, q_ref) <= TOL), (case.name, rel_l2(q_gpu, q_ref))


def test_bitwise_reproducible_and_stage_api_equivalent():
    case = cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=2, minmod=True, noise=0.02)
    ch = N.CaseHandle.from_case(case)
    q1 = _gpu_run(ch, 5, case.delta_t)
    q2 = _gpu_run(ch, 5, case.delta_t)
    assert np.array_equal(q1, q2)
    s = N.Solver(ch)
    for _ in range(5):
        for k in range(ch.desc.rk_order):
            s.stage(k, case.delta_t)
    s.sync()
    assert np.array_equal(s.get_state(), q1)


def test_cfl_and_dt_reductions_match_oracle():
    case = cases.vortex_case(n=48, mu=1e-3)
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    s.step(3, case.delta_t)
    q = s.get_state()
    assert s.cfl(case.delta_t) == pytest.approx(N.port_cfl(ch, q, case.delta_t), rel=1e-14)
    assert s.min_dt(0.5) == pytest.approx(N.port_min_dt(ch, q, 0.5), rel=1e-14)


def test_residual_matches_oracle():
    case = cases.vortex_case(n=32, mu=1e-3)
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    s.step(4, case.delta_t)
    gpu_res = s.residual()
    _, port_res = N.port_run(ch, ch.q0(), 4, case.delta_t, residual=True)
    assert np.allclose(gpu_res, port_res, rtol=1e-10, atol=0)


def test_non_finite_state_is_reported():
    # a patch with no boundary condition keeps a zero ghost state, as in the
    # reference, and the flux through it is not finite
    case = cases.vortex_case(n=12)
    for p in case.patches:
        if p.name == "walls":
            p.type = "symmetryPlane"
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    s.step(2, case.delta_t)
    with pytest.raises(N.LfmError) as e:
        s.sync()
    assert e.value.code == -5


def test_full_size_cylinder_matches_oracle():
    """The 768 x 512 cylinder workload, two time steps (10 RK stages)."""
    case = cases.cylinder_case(solver=0, minmod=True)
    ch = N.CaseHandle.from_case(case)
    q_gpu = _gpu_run(ch, 2, case.delta_t)
    q_ref, _ = N.port_run(ch, ch.q0(), 2, case.delta_t)
    assert np.all(rel_l2(q_gpu, q_ref) <= TOL), rel_l2(q_gpu, q_ref)


def test_cell_residual_matches_reference_fixture():
    case, z = load_golden("vortex12x20_m1_res")
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    s.step(int(z["n_steps"]), case.delta_t)
    res = s.cell_residual()
    ids = ch.cell_ids()
    ref = np.vstack([z["ref_" + n][ids] for n in ("rhoRES", "uRES", "vRES", "eRES")])
    assert np.all(rel_l2(res, ref) <= 1e-10), rel_l2(res, ref)
