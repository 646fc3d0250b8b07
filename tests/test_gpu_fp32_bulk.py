"""FP32-bulk form against the FP64 path.

The FP32-bulk form keeps the RK registers, ghost states and geometry in FP64
and evaluates fluxes, limiter and residual sums in FP32 on perturbations from
the free stream. Bar: the acoustic pressure p' = p - p_inf after the same
steps has a relative L2 error <= 1e-3 against the FP64 result (which itself
matches the oracle to 1e-12), over all cells and over a probe ring; the
conserved fields stay within 1e-5 relative L2; results are bitwise
reproducible run to run."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, acoustics, cases
from tests.helpers import load_golden, rel_l2

pytestmark = pytest.mark.gpu
ACOUSTIC_TOL = 1e-3
CONSERVED_TOL = 1e-5


def _run(ch, nsteps, dt, precision):
    s = N.Solver(ch, precision=precision)
    s.step(nsteps, dt)
    s.sync()
    q = s.get_state()
    s.close()
    return q


def _compare(case, nsteps, probes_radius=None):
    ch = N.CaseHandle.from_case(case)
    q64 = _run(ch, nsteps, case.delta_t, N.LFM_FP64)
    q32 = _run(ch, nsteps, case.delta_t, N.LFM_FP32_BULK)
    g = ch.desc.gamma
    err = acoustics.acoustic_rel_l2(q32, q64, g, case.dim, case.p_inf)
    cons = rel_l2(q32, q64)
    probe_err = None
    if probes_radius is not None:
        cells = acoustics.probe_ring(case.cell_centres, ch.cell_ids(), probes_radius)
        probe_err = acoustics.acoustic_rel_l2(q32, q64, g, case.dim, case.p_inf, cells)
    return err, probe_err, cons


@pytest.mark.parametrize("solver", [0, 1, 2])
def test_fp32_bulk_cylinder_acoustic_pressure(solver):
    case = cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=solver, minmod=True,
                               noise=0.02, seed=7)
    err, probe_err, cons = _compare(case, 200, probes_radius=15.0)
    print(f"solver {solver}: p' rel L2 {err:.3e}, probes {probe_err:.3e}, conserved {cons}")
    assert err <= ACOUSTIC_TOL and probe_err <= ACOUSTIC_TOL, (err, probe_err)
    assert np.all(cons <= CONSERVED_TOL), cons


def test_fp32_bulk_vortex_3d_and_triangles():
    for case, n in ((cases.vortex_case(n=64, mu=1e-3), 100),
                    (cases.cylinder_case(n_theta=32, n_r=16, r1=10, first=0.03, Ls=3, solver=2, minmod=True,
                                         n_span=8, noise=0.01), 40),
                    (cases.tri_case(n=40, seed=9, solver=1, beta=4.0), 60)):
        err, _, cons = _compare(case, n)
        print(f"{case.name}: p' rel L2 {err:.3e}, conserved {cons}")
        assert err <= ACOUSTIC_TOL, (case.name, err)
        assert np.all(cons <= CONSERVED_TOL), (case.name, cons)


def test_fp32_bulk_bitwise_reproducible_and_stage_api():
    case = cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=2, minmod=True, noise=0.02)
    ch = N.CaseHandle.from_case(case)
    q1 = _run(ch, 5, case.delta_t, N.LFM_FP32_BULK)
    q2 = _run(ch, 5, case.delta_t, N.LFM_FP32_BULK)
    assert np.array_equal(q1, q2)
    s = N.Solver(ch, precision=N.LFM_FP32_BULK)
    for _ in range(5):
        for k in range(ch.desc.rk_order):
            s.stage(k, case.delta_t)
    s.sync()
    assert np.array_equal(s.get_state(), q1)
    s.close()


@pytest.mark.parametrize("precision", [N.LFM_FP64, N.LFM_FP32_BULK])
def test_advance_is_set_state_step_get_state(precision):
    """lfm_solver_advance (state in, steps, state out, one synchronisation)
    gives the bits of set_state + step + get_state, step by step, and a
    None input or output skips that copy."""
    case = cases.cylinder_case(n_theta=48, n_r=24, r1=15, first=0.02, Ls=4, solver=1, minmod=True, noise=0.02)
    ch = N.CaseHandle.from_case(case)
    dt = case.delta_t
    a = N.Solver(ch, precision=precision)
    b = N.Solver(ch, precision=precision)
    host = np.ascontiguousarray(a.get_state())
    out = np.empty_like(host)
    for _ in range(3):
        b.set_state(host)
        b.step(1, dt)
        b.sync()
        ref = b.get_state()
        a.advance(host, 1, dt, out)
        assert np.array_equal(out, ref)
        host = out.copy()
    a.advance(None, 2, dt, None)
    b.step(2, dt)
    b.sync()
    a.advance(None, 0, dt, out)
    assert np.array_equal(out, b.get_state())
    with pytest.raises(ValueError):
        a.advance(host[:, :-1].copy(), 1, dt, None)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [N.LFM_FP64, N.LFM_FP32_BULK])
def test_advance_between_page_locked_states_is_one_graph(precision):
    """With page-locked host states lfm_solver_advance replays one captured
    graph (copy in, conversion, primitives, steps, conversion, copy out, the
    non-finite flag): the bits of set_state + step + get_state, for repeated
    calls on the same buffers, a new dt and several steps, and a non-finite
    state is reported."""
    torch = pytest.importorskip("torch")
    case = cases.cylinder_case(n_theta=48, n_r=24, r1=15, first=0.02, Ls=4, solver=2, minmod=True, noise=0.02)
    ch = N.CaseHandle.from_case(case)
    a = N.Solver(ch, precision=precision)
    b = N.Solver(ch, precision=precision)
    shape = (ch.desc.nq, ch.desc.n_cells)
    hin = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hout = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hin[:] = a.get_state()
    for dt, nsteps in ((case.delta_t, 1), (case.delta_t, 1), (0.5 * case.delta_t, 1), (case.delta_t, 3)):
        b.set_state(hin)
        b.step(nsteps, dt)
        b.sync()
        ref = b.get_state()
        a.advance(hin, nsteps, dt, hout)
        assert np.array_equal(hout, ref)
        hin[:] = hout
    # the solver keeps working through its other calls afterwards
    a.step(1, case.delta_t)
    b.step(1, case.delta_t)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_state(), b.get_state())
    hin[0, 5] = np.nan
    with pytest.raises(N.LfmError) as e:
        a.advance(hin, 1, case.delta_t, hout)
    assert e.value.code == N.LFM_ERR_NUMERIC
    a.close()
    b.close()


def test_fp32_bulk_free_stream_is_preserved():
    # A uniform free stream (inlet, outlet and walls) has zero perturbation in
    # the interior and FP64-derived ghost primitives: the state may move only
    # by FP64 rounding.
    case = cases.vortex_case(n=32, beta=0.0)
    ch = N.CaseHandle.from_case(case)
    q = _run(ch, 10, case.delta_t, N.LFM_FP32_BULK)
    q0 = ch.q0()
    d = case.dim
    scale = np.array([np.abs(q0[0]).max()] + [np.abs(q0[1:1 + d]).max()] * d + [np.abs(q0[d + 1]).max()])
    assert np.max(np.abs(q - q0) / scale[:, None]) < 1e-13


def test_fp32_bulk_residual_and_cell_residual():
    case = cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=0, minmod=True, noise=0.02)
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    s64 = N.Solver(ch, precision=N.LFM_FP64)
    s32 = N.Solver(ch, precision=N.LFM_FP32_BULK)
    for s in (s64, s32):
        s.step(3, case.delta_t)
        s.sync()
    r64, r32 = s64.cell_residual(), s32.cell_residual()
    # residuals are differences of fluxes; compare against the largest value per field
    scale = np.abs(r64).max(axis=1, keepdims=True)
    assert np.max(np.abs(r32 - r64) / scale) < 1e-4
    s64.close()
    s32.close()


def _conversion_inputs():
    rng = np.random.default_rng(1)
    f32 = rng.integers(0, 2 ** 32, size=100000, dtype=np.uint64).astype(np.uint32)
    edge32 = np.array([0, 0x80000000, 1, 0x80000001, 0x7fffff, 0x800000, 0x7f7fffff, 0x7f800000, 0xff800000,
                       0x7fc00000, 0x3f800000], dtype=np.uint32)
    f32 = np.concatenate([f32, edge32])
    bits = rng.integers(0, 2 ** 63, size=40000, dtype=np.uint64)
    vals = (rng.standard_normal(40000) * np.exp(rng.uniform(-100, 100, 40000))).view(np.uint64)
    fl = rng.standard_normal(20000).astype(np.float32)
    ties = (fl.astype(np.float64) + np.spacing(fl).astype(np.float64) / 2).view(np.uint64)   # halfway cases
    sub = rng.uniform(0, 2e-38, 11).view(np.uint64)                                           # binary32 subnormals
    edge64 = np.array([
        0x47EFFFFFE0000000, 0x47EFFFFFF0000000, 0x47EFFFFFEFFFFFFF, 0xC7EFFFFFF0000000,   # FLT_MAX, tie -> inf
        0x47F0000000000000, 0x47E0000000000000,                                         # 2^128, 2^127
        0x3FF0000010000000, 0x3FF0000030000000, 0x3FF0000010000001, 0x3FF000000FFFFFFF,   # ties even / odd
        0x3FFFFFFFF0000000, 0xBFFFFFFFF0000001,                                         # carry into the exponent
        0x3810000000000000, 0x380FFFFFFFFFFFFF, 0x380FFFFFF0000000, 0x3800000000000000,   # smallest normal float
        0x0000000000000001, 0x8000000000000000, 0x0000000000000000, 0x7FF0000000000000,
        0x7FF8000000000001, 0xFFF0000000000000], dtype=np.uint64)
    f64 = np.concatenate([edge64, bits, vals, ties, sub])[:f32.size]
    return f32, f64


def test_integer_pipe_conversions_match_ieee():
    # The FP32-bulk kernels convert between FP32 and FP64 with integer
    # operations; they must equal IEEE 754 conversions bit for bit (NaNs: any NaN).
    f32, f64 = _conversion_inputs()
    o64, o32 = N.selftest_fp_convert(f32, f64)
    with np.errstate(invalid="ignore", over="ignore"):
        r64 = f32.view(np.float32).astype(np.float64).view(np.uint64)
        r32 = f64.view(np.float64).astype(np.float32).view(np.uint32)
    nan64 = np.isnan(r64.view(np.float64))
    assert np.array_equal(o64[~nan64], r64[~nan64])
    assert np.all(np.isnan(o64[nan64].view(np.float64)))
    nan32 = np.isnan(r32.view(np.float32))
    assert np.array_equal(o32[~nan32], r32[~nan32])
    assert np.all(np.isnan(o32[nan32].view(np.float32)))


@pytest.mark.parametrize("make,tiled", [
    (lambda: cases.cylinder_case(n_theta=96, n_r=64, r1=30, first=0.01, Ls=8, solver=0, minmod=True, noise=0.02),
     True),
    (lambda: cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=2, minmod=True, noise=0.02),
     True),
    (lambda: cases.tri_case(n=40, seed=9, solver=1, beta=4.0), True),
    # a small 3D mesh stages over 8 cells per tile cell: the solver keeps the
    # separate kernels
    (lambda: cases.cylinder_case(n_theta=24, n_r=12, r1=8, first=0.04, Ls=3, solver=1, n_span=6, noise=0.01),
     False),
])
def test_fused_tile_stages_are_bitwise_the_separate_kernels(make, tiled, monkeypatch):
    """The fused tile stage (one kernel per stage, tile data staged in shared
    memory; opt-in) gives the bits of the separate kernels."""
    case = make()
    ch = N.CaseHandle.from_case(case, renumber=N.LFM_RENUMBER_HILBERT)
    n = 7   # odd: the run ends on the second primitive buffer
    monkeypatch.setenv("LFM_TILE_CELLS", "0")
    q0 = _run(ch, n, case.delta_t, N.LFM_FP32_BULK)
    monkeypatch.setenv("LFM_TILE_CELLS", "128")
    s = N.Solver(ch, precision=N.LFM_FP32_BULK)
    assert (s.launches_per_step() == ch.desc.rk_order) == tiled   # one fused kernel per stage
    s.step(n, case.delta_t)
    s.sync()
    q1 = s.get_state()
    # stepping on after a single-stage call (primitives rebuilt in buffer 0)
    s.stage(0, case.delta_t)
    s.sync()
    s.close()
    assert np.array_equal(q0, q1)


def test_smagorinsky_les_fp32_bulk_and_batch():
    """Smagorinsky LES: the FP32-bulk form stays within the acoustic bar of
    the FP64 path (which the les_* fixtures pin to the reference); the batch
    engine refuses LES cases."""
    case, _ = load_golden("les_cyl24x12_m2")
    assert not case.laminar
    ch = N.CaseHandle.from_case(case)
    assert ch.desc.smag_c
    q64 = _run(ch, 40, case.delta_t, N.LFM_FP64)
    q32 = _run(ch, 40, case.delta_t, N.LFM_FP32_BULK)
    err = acoustics.acoustic_rel_l2(q32, q64, ch.desc.gamma, case.dim, case.p_inf)
    assert err <= ACOUSTIC_TOL, err
    b = N.Batch(arena_bytes=64 << 20, max_cases=2)
    with pytest.raises(N.LfmError):
        b.add(ch, case.delta_t)
    b.close()


@pytest.mark.parametrize("solver,minmod,mu", [(0, True, 1e-3), (1, False, 1e-3), (2, True, 1e-3), (0, False, 0.0)])
def test_fused_flux_update_gives_the_separate_kernels_bits(monkeypatch, solver, minmod, mu):
    """The fused flux + update stage (each cell evaluates the rhs of its own
    faces, the next stage's primitives go to a second buffer) gives the bits
    of the separate flux and update kernels, through stepping, single steps,
    lfm_solver_advance and the residual."""
    case = cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=solver, minmod=minmod,
                               noise=0.02, seed=3)
    case.mu = mu
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("LFM_FLUX_UPDATE", mode)
        s = N.Solver(ch, precision=N.LFM_FP32_BULK)
        s.step(7, case.delta_t)   # an odd stage count per step: the buffers swap
        s.sync()
        q7 = s.get_state()
        res = s.cell_residual()
        host = np.ascontiguousarray(q7.copy())
        outq = np.empty_like(host)
        s.advance(host, 3, case.delta_t, outq)
        out[mode] = (q7, res, outq)
        s.close()
    for a, b in zip(out["0"], out["1"]):
        assert np.array_equal(a, b)


def _staged_cases():
    return {
        "cyl2d_m1": lambda: cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=0, minmod=True,
                                                noise=0.02, seed=3),
        "cyl2d_m2": lambda: cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=1, minmod=False,
                                                noise=0.02, seed=4),
        "vortex_inviscid": lambda: cases.vortex_case(n=40, solver=0),
        "tri_m2": lambda: cases.tri_case(n=24, seed=4, solver=1),
        "cyl3d_m2": lambda: cases.cylinder_case(n_theta=24, n_r=12, n_span=6, solver=1, reynolds=3900.0, noise=0.01,
                                                seed=7),
    }


@pytest.mark.parametrize("name,stages,faces", [
    ("cyl2d_m1", 2, 128), ("cyl2d_m1", 3, 96), ("cyl2d_m1", 4, 256), ("cyl2d_m2", 2, 96),
    ("vortex_inviscid", 2, 128), ("tri_m2", 3, 32), ("cyl3d_m2", 2, 128), ("cyl3d_m2", 3, 160),
    ("cyl2d_m1", 1, 256), ("cyl2d_m2", 1, 256), ("vortex_inviscid", 1, 256), ("tri_m2", 1, 256), ("cyl3d_m2", 1, 256),
])
def test_staged_flux_gives_the_plain_kernels_bits(monkeypatch, name, stages, faces):
    """The staged flux kernel (the values of each face copied into shared
    memory ahead of use, chunks of `faces` faces per block, `stages` buffers
    per thread) gives the bits of the plain flux kernel: face counts that
    are not a multiple of the chunk, boundary faces, inviscid and viscous
    cases, 2D and 3D, through stepping, lfm_solver_advance and the residual."""
    case = _staged_cases()[name]()
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    assert ch.desc.n_faces % faces != 0 or faces == 32
    monkeypatch.setenv("LFM_FLUX_UPDATE", "0")
    out = {}
    for mode in ("0", str(stages)):
        monkeypatch.setenv("LFM_FLUX_STAGES", mode)
        monkeypatch.setenv("LFM_FLUX_FACES", str(faces))
        s = N.Solver(ch, precision=N.LFM_FP32_BULK)
        s.step(4, case.delta_t)
        s.sync()
        q = s.get_state()
        res = s.cell_residual()
        host = np.ascontiguousarray(q.copy())
        outq = np.empty_like(host)
        s.advance(host, 2, case.delta_t, outq)
        out[mode] = (q, res, outq)
        s.close()
    assert np.isfinite(out["0"][0]).all()
    for a, b in zip(out["0"], out[str(stages)]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["cyl2d_m1", "cyl2d_m2", "vortex_inviscid", "tri_m2", "cyl3d_m2"])
def test_cell_centred_flux_gives_the_plain_kernels_bits(monkeypatch, name):
    """The cell-centred flux kernel (one thread per cell over the faces it
    owns, the cell's own rows read once) gives the plain flux kernel's bits,
    through stepping, lfm_solver_advance and the residual."""
    case = _staged_cases()[name]()
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    monkeypatch.setenv("LFM_FLUX_UPDATE", "0")
    monkeypatch.setenv("LFM_FLUX_STAGES", "0")
    out = {}
    for m in ("0", "1"):
        monkeypatch.setenv("LFM_FLUX_CELL", m)
        s = N.Solver(ch, precision=N.LFM_FP32_BULK)
        s.step(4, case.delta_t)
        s.sync()
        q = s.get_state()
        res = s.cell_residual()
        host = np.ascontiguousarray(q.copy())
        outq = np.empty_like(host)
        s.advance(host, 2, case.delta_t, outq)
        out[m] = (q, res, outq)
        s.close()
    assert np.isfinite(out["0"][0]).all()
    for a, b in zip(out["0"], out["1"]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["cyl2d_m1", "cyl3d_m2"])
def test_flux_autotune_restores_the_state_and_keeps_the_bits(monkeypatch, name):
    """lfm_solver_autotune times the face, cell and staged flux kernels (the
    staging depths 1..4) and keeps the fastest; the state is restored, and
    stepping on with the chosen kernel gives the bits of an untuned solver."""
    case = _staged_cases()[name]()
    ch = N.CaseHandle.from_case(case)
    monkeypatch.setenv("LFM_FLUX_UPDATE", "0")
    ref = N.Solver(ch, precision=N.LFM_FP32_BULK)
    ref.step(6, case.delta_t)
    ref.sync()
    q_ref = ref.get_state()
    ref.close()
    s = N.Solver(ch, precision=N.LFM_FP32_BULK)
    s.step(3, case.delta_t)
    s.sync()
    q3 = s.get_state()
    t = s.autotune(case.delta_t, trial_steps=3, flush_bytes=1 << 20)
    assert t.flux_kernel in (N.LFM_FLUX_FACE, N.LFM_FLUX_CELL, N.LFM_FLUX_STAGED)
    assert t.ms_per_step > 0
    assert s.tuning().flux_kernel == t.flux_kernel
    assert np.array_equal(s.get_state(), q3)
    s.step(3, case.delta_t)
    s.sync()
    assert np.array_equal(s.get_state(), q_ref)
    # every variant by hand
    for kern, depth, faces in [(N.LFM_FLUX_FACE, 0, 0), (N.LFM_FLUX_CELL, 0, 0), (N.LFM_FLUX_STAGED, 1, 256),
                               (N.LFM_FLUX_STAGED, 3, 96)]:
        s.set_tuning(kern, depth, faces)
        s.set_state(ch.q0())
        s.step(6, case.delta_t)
        s.sync()
        assert np.array_equal(s.get_state(), q_ref), (kern, depth, faces)
    with pytest.raises(N.LfmError):
        s.set_tuning(N.LFM_FLUX_STAGED, 5, 128)
    with pytest.raises(N.LfmError):
        s.set_tuning(N.LFM_FLUX_STAGED, 2, 48)
    s.close()


def test_flux_tuning_where_the_variants_do_not_apply():
    """FP64 solvers and M2AUSM report the face kernel and refuse the others;
    lfm_solver_autotune times the one configuration they have."""
    case = cases.cylinder_case(n_theta=32, n_r=16, r1=20, first=0.02, Ls=5, solver=2, minmod=True)
    ch = N.CaseHandle.from_case(case)
    for prec in (N.LFM_FP64, N.LFM_FP32_BULK):
        s = N.Solver(ch, precision=prec)
        assert s.tuning().flux_kernel == N.LFM_FLUX_FACE
        s.set_tuning(N.LFM_FLUX_FACE)
        with pytest.raises(N.LfmError):
            s.set_tuning(N.LFM_FLUX_CELL)
        t = s.autotune(case.delta_t, trial_steps=2, flush_bytes=1 << 20)
        assert t.flux_kernel == N.LFM_FLUX_FACE and t.ms_per_step > 0
        s.close()
