"""FP64 device path against the reference (golden fixtures) and the oracle.

Parity bar: relative L2 per conserved field <= 1e-12 after the fixture's RK
steps (100 RK stages for the 2D fixtures), and bitwise reproducibility run to
run."""
import numpy as np
import pytest

import oracle.port as P
from lfm_public_gb300 import _native as N, acoustics, cases
from tests.helpers import (adaptive_run, adjust_names, config_case, golden_names, load_golden, primitives,
                           reference_conserved, rel_l2, rel_l2_vec)

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
    err = rel_l2_vec(q, ref, case.dim)   # the prisms' w is rounding noise
    assert np.all(err <= TOL), err


@pytest.mark.parametrize("name", adjust_names())
def test_fp64_adaptive_dt_matches_reference(name):
    """adjustTimeStep yes through the C ABI: one step at a time, the next dt
    from lfm_solver_min_dt (compute_dt's deterministic minimum on the
    device). Same step count as the reference, every dt and time within
    1e-9 (the reference prints 10 significant digits), final fields within
    1e-12."""
    case, z = load_golden(name)
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch, precision=N.LFM_FP64)
    max_co = float(z["max_co"])
    dts, times = adaptive_run(lambda dt: s.step(1, dt), lambda: s.min_dt(max_co), case, z)
    s.sync()
    q = s.get_state()
    s.close()
    assert len(dts) == len(z["ref_dt"])
    np.testing.assert_allclose(dts, z["ref_dt"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(times, z["ref_time"], rtol=1e-9, atol=0)
    err = rel_l2_vec(q, reference_conserved(z, ch.cell_ids(), case.dim), case.dim)
    assert np.all(err <= TOL), err


@pytest.mark.parametrize("solver,minmod", [(0, True), (1, False), (2, True), (2, False)])
def test_fp64_matches_oracle_cylinder(solver, minmod):
    case = cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=solver, minmod=minmod,
                               noise=0.02, seed=7)
    ch = N.CaseHandle.from_case(case)
    n = 20
    q_gpu = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    assert np.all(rel_l2(q_gpu, q_ref) <= TOL), rel_l2(q_gpu, q_ref)


def test_fp64_matches_oracle_3d_and_triangles():
    for case, n in ((cases.cylinder_case(n_theta=32, n_r=16, r1=10, first=0.03, Ls=3, solver=2, minmod=True,
                                         n_span=8, noise=0.01), 10),
                    (cases.tri_case(n=40, seed=9, solver=0, beta=4.0), 20)):
        ch = N.CaseHandle.from_case(case)
        q_gpu = _gpu_run(ch, n, case.delta_t)
        q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
        assert np.all(rel_l2(q_gpu, q_ref) <= TOL), (case.name, rel_l2(q_gpu, q_ref))


@pytest.mark.parametrize("rk", [0, 1, 2, 3, 4])
def test_rk_orders_match_oracle(rk):
    """rkOrder 0-4 (5 is every other test's): FP64 within 1e-12 of the
    oracle, FP32-bulk p' within 1e-3 of FP64, and a batch of rkOrder-rk
    cases bitwise the single-case FP32-bulk solver (rkOrder 0: no stage, the
    state stays; batches take 1 and above)."""
    case = cases.cylinder_case(n_theta=48, n_r=24, r1=15, first=0.02, Ls=4, solver=rk % 3, minmod=True, noise=0.02)
    case.rk_order = rk
    ch = N.CaseHandle.from_case(case)
    assert ch.desc.rk_order == rk
    n = 10
    q64 = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    assert np.all(rel_l2(q64, q_ref) <= TOL), rel_l2(q64, q_ref)
    q32 = _gpu_run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    assert acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, case.dim, case.p_inf) <= 1e-3
    if rk == 0:
        assert np.array_equal(q64, ch.q0())
        return
    b = N.Batch(rk_order=rk, arena_bytes=256 << 20)
    slot = b.add(ch, case.delta_t)
    b.step(n)
    b.sync()
    assert np.array_equal(b.get_state(slot), q32)
    b.close()


@pytest.mark.parametrize("make", [lambda: cases.vortex_case(n=1), lambda: cases.vortex_case(n=2),
                                  lambda: cases.vortex_case(n=3, ny=1), lambda: cases.tri_case(n=1, seed=3),
                                  lambda: cases.tri_case(n=2, seed=3, solver=1)],
                         ids=["1cell", "2x2", "3x1", "2tri", "8tri"])
def test_tiny_meshes(make):
    """One cell (no internal face), meshes without interior submesh, two
    triangles: FP64 within 1e-12 of the oracle, FP32-bulk near FP64 and the
    batch bitwise the single-case FP32-bulk solver."""
    case = make()
    ch = N.CaseHandle.from_case(case)
    n = 5
    q64 = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    # momentum as one vector field: on these symmetric meshes a momentum
    # component can be pure rounding noise (1e-8 against 1e2)
    err = lambda a, b: rel_l2_vec(a, b, case.dim)  # noqa: E731
    assert np.all(err(q64, q_ref) <= TOL), err(q64, q_ref)
    q32 = _gpu_run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    assert np.all(err(q32, q64) <= 1e-5), err(q32, q64)
    b = N.Batch(arena_bytes=64 << 20)
    slot = b.add(ch, case.delta_t)
    b.step(n)
    b.sync()
    assert np.array_equal(b.get_state(slot), q32)
    b.close()


@pytest.mark.parametrize("solver", [0, 1, 2])
def test_mixed_quad_triangle_mesh(solver):
    """Quadrilaterals and triangles in one mesh (cells of 4 and 3 faces; the
    reference itself stops on such a submesh, so the oracle is the bar): FP64
    within 1e-12 of the oracle, FP32-bulk p' within 1e-3 and the batch
    bitwise the single-case FP32-bulk solver."""
    case = cases.hybrid_case(n=24, tri_fraction=0.4, seed=5 + solver, solver=solver, beta=3.0)
    ch = N.CaseHandle.from_case(case)
    offs = np.ctypeslib.as_array(ch.desc.cell_face_offsets, shape=(ch.desc.n_cells + 1,))
    assert set(np.diff(offs).tolist()) == {3, 4}
    n = 20
    q64 = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    assert np.all(rel_l2(q64, q_ref) <= TOL), rel_l2(q64, q_ref)
    q32 = _gpu_run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    assert acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, case.dim, case.p_inf) <= 1e-3
    b = N.Batch(arena_bytes=64 << 20)
    slot = b.add(ch, case.delta_t)
    b.step(n)
    b.sync()
    assert np.array_equal(b.get_state(slot), q32)
    b.close()


@pytest.mark.parametrize("make", [lambda: cases.prism_case(n=10, nz=4, seed=3, solver=1),
                                  lambda: cases.tet_case(n=6, nz=3, seed=4, solver=2)], ids=["prisms", "tets"])
def test_3d_prisms_and_tetrahedra(make):
    """Cells of five and four faces in 3D: FP64 within 1e-12 of the oracle,
    FP32-bulk p' within 1e-3, and the batch bitwise the single-case FP32-bulk
    solver (whose 3D update pads these cells' rows of the fixed-width face
    table)."""
    case = make()
    ch = N.CaseHandle.from_case(case)
    n = 10
    q64 = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    # momentum as one vector: the prisms' w stays zero up to rounding (1e-12 against 6e3)
    err = rel_l2_vec(q64, q_ref, case.dim)
    assert np.all(err <= TOL), err
    q32 = _gpu_run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    assert acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, case.dim, case.p_inf) <= 1e-3
    b = N.Batch(arena_bytes=64 << 20)
    slot = b.add(ch, case.delta_t)
    b.step(n)
    b.sync()
    assert np.array_equal(b.get_state(slot), q32)
    b.close()


def test_smagorinsky_les_on_tetrahedra():
    """Smagorinsky LES on 3D cells of four faces: FP64 within 1e-12 of the
    oracle (itself bitwise the reference build on such meshes), FP32-bulk p'
    within 1e-3."""
    case = cases.tet_case(n=6, nz=3, seed=7, solver=1)
    case.laminar = False
    case.mu = 1.8e-3
    ch = N.CaseHandle.from_case(case)
    assert ch.desc.smag_c
    n = 10
    q64 = _gpu_run(ch, n, case.delta_t)
    q_ref, _ = P.run(ch, ch.q0(), n, case.delta_t)
    err = rel_l2_vec(q64, q_ref, case.dim)
    assert np.all(err <= TOL), err
    q32 = _gpu_run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    assert acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, case.dim, case.p_inf) <= 1e-3


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
    assert s.cfl(case.delta_t) == pytest.approx(P.cfl(ch, q, case.delta_t), rel=1e-14)
    assert s.min_dt(0.5) == pytest.approx(P.min_dt(ch, q, 0.5), rel=1e-14)


def test_residual_matches_oracle():
    case = cases.vortex_case(n=32, mu=1e-3)
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    s.step(4, case.delta_t)
    gpu_res = s.residual()
    _, port_res = P.run(ch, ch.q0(), 4, case.delta_t, residual=True)
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
    """The 768 x 512 cylinder workload, 20 time steps (100 RK stages), every
    cell against the oracle set up by its own code."""
    case = cases.cylinder_case(solver=0, minmod=True)
    ch = N.CaseHandle.from_case(case)
    q_gpu = _gpu_run(ch, 20, case.delta_t)
    pc = P.PortCase.from_case(case)
    q_ref, _ = P.run(pc, pc.q0(), 20, case.delta_t)
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


def _sample_conserved(z, q, ids, dim, gamma):
    """The device state at the fixture's sampled polyMesh cells, as the
    reference's written rho, E, p; and the reference's."""
    inv = np.empty_like(ids)
    inv[ids] = np.arange(len(ids))
    cells = inv[z["sample"]]
    r, U, E, p = primitives(q[:, cells], gamma, dim)
    return {"rho": r, "E": E, "p": p}, {k: z["ref_" + k] for k in ("rho", "E", "p")}


@pytest.mark.parametrize("name", ["cfg_vortex256_m1_1000", "cfg_cyl768x512_m1_20"])
def test_configured_workload_matches_reference(name):
    """The configured workloads at full size and length against the reference
    solver run with the same settings: the 256 x 256 isentropic vortex for
    1000 steps (5000 RK stages) and the 768 x 512 cylinder for 20 steps
    (100 RK stages). FP64: rho, E and p within 1e-12 relative L2 on 4096
    seeded cells, and the whole-field norms within 1e-12; FP32-bulk: acoustic
    pressure within 1e-3 there."""
    case, z = config_case(name)
    ch = N.CaseHandle.from_case(case)
    n = int(z["n_steps"])
    ids = ch.cell_ids()
    for prec in (N.LFM_FP64, N.LFM_FP32_BULK):
        q = _gpu_run(ch, n, case.delta_t, precision=prec)
        got, ref = _sample_conserved(z, q, ids, case.dim, ch.desc.gamma)
        if prec == N.LFM_FP64:
            for k in got:
                assert rel_l2(got[k][None], ref[k][None])[0] <= TOL, k
            r, U, E, p = primitives(q, ch.desc.gamma, case.dim)
            for k, v in (("rho", r), ("E", E), ("p", p)):
                assert abs(np.linalg.norm(v) - float(z["ref_norm_" + k])) <= TOL * float(z["ref_norm_" + k]), k
        else:
            pp = got["p"] - case.p_inf
            pr = ref["p"] - case.p_inf
            assert np.linalg.norm(pp - pr) <= 1e-3 * np.linalg.norm(pr)
