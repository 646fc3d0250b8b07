"""Request server: continuous batching with admission by HBM footprint.

Bar: every request's result is the same alone and in the mix -- bit for bit,
since the batch computes each case with the same kernels whatever else runs
-- and within the acoustic tolerance (1e-3 relative L2 of p') of the FP64
path; requests admitted while others run finish with exact step counts; a
request larger than the arena is refused, one whose state becomes
non-finite is retired with LFM_ERR_NUMERIC without disturbing the others."""
import dataclasses
import time

import numpy as np
import pytest

from lfm_public_gb300 import _native as N, acoustics, cases

pytestmark = pytest.mark.gpu


def _requests():
    out = [(cases.vortex_case(n=48, mach=0.3, beta=3.0, solver=0), 37),
           (cases.cylinder_case(n_theta=48, n_r=24, r1=15, first=0.02, Ls=4, solver=2, minmod=True, noise=0.02), 23),
           (cases.cylinder_case(n_theta=24, n_r=12, r1=8, first=0.04, Ls=3, solver=1, n_span=6, noise=0.01), 11),
           (cases.vortex_case(n=96, mach=0.5, beta=5.0, solver=1), 64),
           (cases.tri_case(n=24, seed=3, solver=1, mach=0.2, beta=2.0), 19)]
    return [(c, N.CaseHandle.from_case(c), n) for c, n in out]


def _alone(ch, dt, n, **kw):
    srv = N.Server(arena_bytes=N.Batch.case_bytes(ch) + (1 << 20), max_cases=1, **kw)
    rid = srv.submit(ch, dt, n)
    assert srv.wait(rid, 60.0)
    q, info = srv.result(rid)
    srv.close()
    assert info["status"] == N.LFM_OK
    return q


def test_results_same_alone_and_in_the_mix():
    reqs = _requests()
    srv = N.Server(arena_bytes=256 << 20, chunk_steps=7)
    ids = []
    for k, (c, ch, n) in enumerate(reqs):
        ids.append(srv.submit(ch, c.delta_t, n))
        if k % 2 == 1:
            time.sleep(0.05)      # later requests arrive while earlier ones run
    results = {}
    for rid in ids:
        assert srv.wait(rid, 60.0)
        results[rid] = srv.result(rid)
    st = srv.stats()
    srv.close()
    for rid, (c, ch, n) in zip(ids, reqs):
        q, info = results[rid]
        assert info["status"] == N.LFM_OK and info["steps"] == n
        assert info["t_submit"] <= info["t_admit"] <= info["t_done"]
        assert np.array_equal(q, _alone(ch, c.delta_t, n)), c.name
        s64 = N.Solver(ch, precision=N.LFM_FP64)
        s64.step(n, c.delta_t)
        q64 = s64.get_state()
        s64.close()
        err = acoustics.acoustic_rel_l2(q, q64, ch.desc.gamma, c.dim, c.p_inf)
        assert err <= 1e-3, (c.name, err)
    assert st["completed"] == len(reqs)


def test_admission_waits_for_footprint():
    c = cases.vortex_case(n=64)
    ch = N.CaseHandle.from_case(c)
    need = N.Batch.case_bytes(ch)
    srv = N.Server(arena_bytes=2 * need + 4096, chunk_steps=5)
    ids = [srv.submit(ch, c.delta_t, 40) for _ in range(5)]
    infos = []
    for rid in ids:
        assert srv.wait(rid, 60.0)
        q, info = srv.result(rid)
        infos.append((q, info))
    srv.close()
    # at most two fit at once: the third is admitted only after one is done
    done = sorted(i["t_done"] for _, i in infos)
    third_admit = sorted(i["t_admit"] for _, i in infos)[2]
    assert third_admit >= done[0]
    for q, info in infos[1:]:
        assert info["status"] == N.LFM_OK
        assert np.array_equal(q, infos[0][0])


def test_oversized_request_is_refused_and_others_run():
    small = cases.vortex_case(n=32)
    big = cases.vortex_case(n=96)
    chs, chb = N.CaseHandle.from_case(small), N.CaseHandle.from_case(big)
    srv = N.Server(arena_bytes=N.Batch.case_bytes(chs) + (1 << 16))
    rb = srv.submit(chb, big.delta_t, 5)
    rs = srv.submit(chs, small.delta_t, 5)
    assert srv.wait(rb, 30.0) and srv.wait(rs, 30.0)
    _, ib = srv.result(rb)
    qs, is_ = srv.result(rs)
    srv.close()
    assert ib["status"] == N.LFM_ERR_NOMEM
    assert is_["status"] == N.LFM_OK
    assert np.array_equal(qs, _alone(chs, small.delta_t, 5))


@pytest.mark.parametrize("solo_cells", [0, 1])
def test_nonfinite_request_is_retired_alone(solo_cells):
    """Batched (solo_cells 0) or each on its own solver (solo_cells 1)."""
    # A patch without a boundary condition keeps a zero ghost state (as in the
    # reference): the first flux through it is non-finite.
    bad = cases.vortex_case(n=32)
    bad.patches = [dataclasses.replace(p, name="side") if p.name == "outlet" else p for p in bad.patches]
    good = cases.vortex_case(n=40)
    chb, chg = N.CaseHandle.from_case(bad), N.CaseHandle.from_case(good)
    srv = N.Server(arena_bytes=64 << 20, chunk_steps=4, solo_cells=solo_cells)
    rb = srv.submit(chb, bad.delta_t, 20)
    rg = srv.submit(chg, good.delta_t, 20)
    assert srv.wait(rb, 30.0) and srv.wait(rg, 30.0)
    _, ib = srv.result(rb)
    qg, ig = srv.result(rg)
    srv.close()
    assert ib["status"] == N.LFM_ERR_NUMERIC
    assert ig["status"] == N.LFM_OK
    assert np.array_equal(qg, _alone(chg, good.delta_t, 20))


@pytest.mark.parametrize("max_solo", [1, 2])
def test_solo_requests_give_the_batched_bits(max_solo):
    """Requests of at least solo_cells cells run on their own single-case
    FP32-bulk solver beside the batch; every result keeps the bits of the
    same request run alone in the batch, and the server's counters add up
    (cell-stage updates = cells x steps x stages of every request)."""
    reqs = _requests()
    sizes = [ch.desc.n_cells for _, ch, _ in reqs]
    solo_cells = 2000
    assert any(n >= solo_cells for n in sizes) and any(n < solo_cells for n in sizes)
    srv = N.Server(arena_bytes=256 << 20, chunk_steps=7, solo_cells=solo_cells, max_solo=max_solo)
    ids = [srv.submit(ch, c.delta_t, n) for c, ch, n in reqs]
    for rid in ids:
        assert srv.wait(rid, 60.0)
    st = srv.stats()
    results = [srv.result(rid) for rid in ids]
    srv.close()
    for (q, info), (c, ch, n) in zip(results, reqs):
        assert info["status"] == N.LFM_OK and info["steps"] == n and info["steps_done"] == n
        assert np.array_equal(q, _alone(ch, c.delta_t, n)), c.name
    assert st["cell_stages"] == sum(ch.desc.n_cells * n * 5 for _, ch, n in reqs)
    assert 0 < st["busy_s"] <= st["t_now"]


def test_solo_request_runs_an_les_case():
    """The batch refuses Smagorinsky LES cases; a solo request runs one on
    its own solver, with the single-case FP32-bulk solver's bits."""
    from tests.helpers import load_golden
    case, _ = load_golden("les_cyl24x12_m2")
    ch = N.CaseHandle.from_case(case)
    n = 9
    srv = N.Server(arena_bytes=64 << 20, solo_cells=1)
    rid = srv.submit(ch, case.delta_t, n)
    assert srv.wait(rid, 60.0)
    q, info = srv.result(rid)
    srv.close()
    assert info["status"] == N.LFM_OK
    s = N.Solver(ch, precision=N.LFM_FP32_BULK)
    s.step(n, case.delta_t)
    s.sync()
    assert np.array_equal(q, s.get_state())
    s.close()


def test_server_closes_while_solo_solvers_are_built():
    """Closing a server with solo requests queued, being built and running
    returns (the worker and the solver-building thread stop; their solvers
    are freed), and a new server on the same device serves normally."""
    c = cases.vortex_case(n=160, solver=0)
    ch = N.CaseHandle.from_case(c)
    srv = N.Server(arena_bytes=64 << 20, solo_cells=1, max_solo=2, chunk_steps=5)
    for _ in range(6):
        srv.submit(ch, c.delta_t, 200)
    time.sleep(0.05)
    t0 = time.time()
    srv.close()
    assert time.time() - t0 < 30.0
    small = cases.vortex_case(n=24)
    chs = N.CaseHandle.from_case(small)
    q = _alone(chs, small.delta_t, 7)
    assert np.isfinite(q).all()
