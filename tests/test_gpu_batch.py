"""Batch engine: many cases advanced by one persistent kernel per RK stage.

Bar: a case advanced inside a batch -- whatever else is in the batch (and so
whichever stage-kernel variant runs), whenever it joined, whatever launch
shape the autotuner picked -- ends bit for bit where it ends alone in a batch
and where the single-case FP32-bulk solver ends; its acoustic pressure stays
within 1e-3 relative L2 of the FP64 path; the arena admits by footprint."""
import numpy as np
import pytest

from lfm_public_gb300 import _native as N, acoustics, cases

pytestmark = pytest.mark.gpu


def _single(ch, n, dt, precision=N.LFM_FP32_BULK):
    s = N.Solver(ch, precision=precision)
    s.step(n, dt)
    s.sync()
    q = s.get_state()
    s.close()
    return q


def _alone(ch, n, dt, shape=None):
    b = N.Batch(arena_bytes=N.Batch.case_bytes(ch) + (1 << 20), max_cases=1)
    if shape:
        b.set_tuning(*shape)
    s = b.add(ch, dt)
    b.step(n)
    b.sync()
    q = b.get_state(s)
    b.close()
    return q


def _mixed_cases():
    spec = cases.sweep_spec(n_cases=6, seed=11, cells_min=2e3, cells_max=2e4)
    cs = [cases.sweep_case(x) for x in spec]
    cs.append(cases.cylinder_case(n_theta=48, n_r=24, r1=15, first=0.02, Ls=4, solver=2, minmod=True, noise=0.02))
    cs.append(cases.cylinder_case(n_theta=24, n_r=12, r1=8, first=0.04, Ls=3, solver=1, minmod=False, n_span=6,
                                  noise=0.01))
    return cs


def test_batch_mix_matches_alone_and_single_solver_bitwise():
    cs = _mixed_cases()
    chs = [N.CaseHandle.from_case(c) for c in cs]
    b = N.Batch(arena_bytes=512 << 20)
    slots = [b.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    n = 12
    b.step(n)
    b.sync()
    for s, ch, c in zip(slots, chs, cs):
        q = b.get_state(s)
        assert np.array_equal(q, _alone(ch, n, c.delta_t)), c.name
        # the FP32-bulk kernels are compiled without implicit FMA contraction,
        # so the single-case solver's kernels round exactly as the batch's
        assert np.array_equal(q, _single(ch, n, c.delta_t)), c.name
    b.close()


def test_single_solver_ghost_pass_variants_bitwise():
    """Above a size threshold the single-case solver prepares its ghosts in a
    separate kernel instead of inside the update; both give the batch's bits
    (the batch always writes ghosts from the update). 3D single-case updates
    gather through the fixed-width cell -> face table, the batch through the
    face list: the same sums in the same order."""
    case = cases.cylinder_case(n_theta=96, n_r=48, r1=12, first=0.03, Ls=3, solver=1, minmod=False, n_span=64,
                               noise=0.01)   # 294,912 cells: above the 3D threshold
    ch = N.CaseHandle.from_case(case)
    assert ch.desc.n_cells > (1 << 18)
    n = 8
    assert np.array_equal(_single(ch, n, case.delta_t), _alone(ch, n, case.delta_t))


def test_batch_advance_is_the_separate_calls():
    """lfm_batch_advance (every state in, steps, every state out, one sync)
    gives the bits of set_state per case, step and get_state per case; None
    keeps a case's state or skips its copy out."""
    cs = _mixed_cases()[:4]
    chs = [N.CaseHandle.from_case(c) for c in cs]
    a = N.Batch(arena_bytes=256 << 20)
    b = N.Batch(arena_bytes=256 << 20)
    sa = [a.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    sb = [b.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    hosts = [np.ascontiguousarray(ch.q0()) for ch in chs]
    outs = [np.empty_like(h) for h in hosts]
    for _ in range(2):
        for s, h in zip(sb, hosts):
            b.set_state(s, h)
        b.step(2)
        refs = [b.get_state(s) for s in sb]
        a.advance(sa, hosts, 2, outs)
        for o, r in zip(outs, refs):
            assert np.array_equal(o, r)
        hosts = [o.copy() for o in outs]
    # keep case 0's state (None in), skip case 1's copy out (None out); a
    # state read out and set again is q_ref + q' rounded, so the reference
    # batch sets the same ones
    keep0, keep1 = outs[0].copy(), outs[1].copy()
    for s, h in zip(sb[1:], hosts[1:]):
        b.set_state(s, h)
    b.step(1)
    a.advance(sa, [None] + hosts[1:], 1, [outs[0], None] + outs[2:])
    assert np.array_equal(outs[0], b.get_state(sb[0])) and not np.array_equal(outs[0], keep0)
    assert np.array_equal(outs[1], keep1)   # not written
    assert np.array_equal(a.get_state(sa[1]), b.get_state(sb[1]))
    for s, o in zip(sb[2:], outs[2:]):
        assert np.array_equal(o, b.get_state(s))
    a.close()
    b.close()


def test_batch_join_leave_between_steps():
    cs = _mixed_cases()[:4]
    chs = [N.CaseHandle.from_case(c) for c in cs]
    b = N.Batch(arena_bytes=256 << 20, max_cases=8)
    s0 = b.add(chs[0], cs[0].delta_t)
    s1 = b.add(chs[1], cs[1].delta_t)
    b.step(5)
    b.remove(s0)
    s2 = b.add(chs[2], cs[2].delta_t)
    s3 = b.add(chs[3], cs[3].delta_t)
    b.step(7)
    b.sync()
    assert np.array_equal(b.get_state(s1), _alone(chs[1], 12, cs[1].delta_t))
    assert np.array_equal(b.get_state(s2), _alone(chs[2], 7, cs[2].delta_t))
    assert np.array_equal(b.get_state(s3), _alone(chs[3], 7, cs[3].delta_t))
    b.close()


def test_batch_autotune_restores_state_and_keeps_results():
    cs = _mixed_cases()[:5]
    chs = [N.CaseHandle.from_case(c) for c in cs]
    b = N.Batch(arena_bytes=256 << 20)
    slots = [b.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    b.step(3)
    b.sync()
    before = [b.get_state(s) for s in slots]
    t = b.autotune(trial_steps=1)
    assert t["block"] in (128, 256, 512) and t["items_per_thread"] >= 1
    for s, q in zip(slots, before):
        assert np.array_equal(b.get_state(s), q)
    b.step(4)
    b.sync()
    for s, ch, c in zip(slots, chs, cs):
        assert np.array_equal(b.get_state(s), _alone(ch, 7, c.delta_t)), (c.name, t)
    b.close()


@pytest.mark.parametrize("shape", [(128, 1, 0), (256, 4, 1), (512, 2, 0), (128, 2, 0, 1, 1), (256, 1, 2, 1, 1)])
def test_batch_launch_shapes_agree(shape):
    """Persistent and phased (one kernel per phase) launch modes, any shape:
    the same bits."""
    cs = _mixed_cases()[:3]
    chs = [N.CaseHandle.from_case(c) for c in cs]
    b = N.Batch(arena_bytes=128 << 20)
    b.set_tuning(*shape)
    slots = [b.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    b.step(6)
    b.sync()
    for s, ch, c in zip(slots, chs, cs):
        assert np.array_equal(b.get_state(s), _alone(ch, 6, c.delta_t)), (c.name, shape)
    b.close()


def test_batch_admission_by_footprint():
    c = cases.vortex_case(n=64)
    ch = N.CaseHandle.from_case(c)
    need = N.Batch.case_bytes(ch)
    b = N.Batch(arena_bytes=2 * need + 4096, max_cases=8)
    s0 = b.add(ch, c.delta_t)
    s1 = b.add(ch, c.delta_t)
    with pytest.raises(N.LfmError) as e:
        b.add(ch, c.delta_t)
    assert e.value.code == N.LFM_ERR_NOMEM
    b.remove(s0)
    assert b.memory()["largest_free"] >= need
    s2 = b.add(ch, c.delta_t)
    assert s2 == s0
    b.step(2)
    b.sync()
    assert np.array_equal(b.get_state(s1), b.get_state(s2))
    b.close()


def test_batch_acoustic_pressure_against_fp64():
    cs = _mixed_cases()
    chs = [N.CaseHandle.from_case(c) for c in cs]
    b = N.Batch(arena_bytes=512 << 20)
    slots = [b.add(ch, c.delta_t) for ch, c in zip(chs, cs)]
    n = 60
    b.step(n)
    b.sync()
    for s, ch, c in zip(slots, chs, cs):
        q64 = _single(ch, n, c.delta_t, N.LFM_FP64)
        err = acoustics.acoustic_rel_l2(b.get_state(s), q64, ch.desc.gamma, c.dim, c.p_inf)
        assert err <= 1e-3, (c.name, err)
    b.close()


def test_grid_barrier_wait_is_bounded():
    """Failure detection without a GPU fault: a grid barrier made to wait for
    one block more than the grid has (a count nothing reaches) gives up after
    its bounded wait (about a second); the kernel returns, lfm_batch_sync
    reports LFM_ERR_CUDA, and the context stays usable: a fresh batch then
    steps and gives the single-case solver's bits."""
    import time
    case = cases.vortex_case(n=32, solver=1)
    ch = N.CaseHandle.from_case(case)
    b = N.Batch(arena_bytes=N.Batch.case_bytes(ch) + (1 << 20), max_cases=1)
    b.add(ch, case.delta_t)
    b.set_tuning(128, 1, 1, cooperative=1, phased=0)
    b.debug_barrier(1)
    t0 = time.perf_counter()
    b.step(1)
    with pytest.raises(N.LfmError) as e:
        b.sync()
    waited = time.perf_counter() - t0
    b.close()
    assert e.value.code == N.LFM_ERR_CUDA and "barrier" in str(e.value)
    assert waited < 10.0, waited
    # the same GPU context, a fresh batch
    q = _alone(ch, 3, case.delta_t, shape=(128, 1, 1))
    assert np.array_equal(q, _single(ch, 3, case.delta_t))
