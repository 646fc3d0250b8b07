"""Post-processing on the device against the reference (post_* golden
fixtures: the reference run with haveAverage and haveForces).

* pAvg / pRMS (postProcAverage, src/cfd_v0.cpp:3083-3104): per-cell sums
  accumulated on the device after every step from tStartAverage on.
  Bar: pAvg relative L2 <= 1e-12; pRMS, a root of sums of squared
  fluctuations (differences of nearby pressures), <= 1e-8.
* Wall forces (postProcForces, src/cfd_v0.cpp:3169-3250): pressure and
  viscous force of every record. Bar: each force vector within 1e-10 of the
  magnitude of the reference's.
Both through the C ABI and through the lfm_solve_gpu driver (its
output/postProcess_Forces_1 and pAvg / pRMS fields)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases
from tests.golden.make_golden import read_forces
import re

from tests.helpers import adjust_names, load_golden, rel_l2

pytestmark = pytest.mark.gpu
POST = ["post_cyl24x12_m2", "post_cyl16x8x4_ausm_3d"]
CLI = os.path.join(os.path.dirname(N.LIB_PATH), "lfm_solve_gpu")


def _wall_patches(case):
    return [i for i, p in enumerate(case.patches) if p.type == "wall"]


def _check_forces(rows, ref, dim):
    assert rows.shape == ref.shape, (rows.shape, ref.shape)
    np.testing.assert_allclose(rows[:, 0], ref[:, 0], rtol=1e-13, atol=0)
    for r in range(ref.shape[0]):
        for blk in range(3):   # Fp, Fv, Fp + Fv
            a = rows[r, 1 + blk * dim:1 + (blk + 1) * dim]
            b = ref[r, 1 + blk * dim:1 + (blk + 1) * dim]
            scale = max(np.linalg.norm(b), 1e-300)
            assert np.linalg.norm(a - b) <= 1e-10 * scale, (r, blk, a, b)


@pytest.mark.parametrize("name", POST)
@pytest.mark.parametrize("precision", [N.LFM_FP64])
def test_stats_and_forces_through_the_c_abi(name, precision):
    case, z = load_golden(name)
    n, start, save = int(z["n_steps"]), int(z["average_start"]), int(z["save_forces_step"])
    ch = N.CaseHandle.from_case(case)
    ids = ch.cell_ids()
    s = N.Solver(ch, precision=precision)
    walls = _wall_patches(case)
    assert walls
    s.stats_reset()
    rows = []

    def record(t):
        fp, fv = s.forces(walls)
        rows.append(np.concatenate([[t], fp[0], fv[0], fp[0] + fv[0]]))

    record(0.0)
    t = 0.0
    for k in range(1, n + 1):
        s.step(1, case.delta_t)
        t += case.delta_t
        s.stats_accumulate(k - start)
        if k % save == 0:
            record(t)
    s.sync()
    pa, pr = s.stats_get(n - start)
    s.close()
    assert rel_l2(pa[None], z["ref_pAvg"][ids][None])[0] <= 1e-12
    assert rel_l2(pr[None], z["ref_pRMS"][ids][None])[0] <= 1e-8
    _check_forces(np.array(rows), z["ref_forces"], case.dim)


def test_fp32_bulk_forces_and_stats_near_fp64():
    """FP32-bulk: the ghost state of a force record is the last stage's
    starting state recovered from the update (q' - B dq), as the FP64 path and
    the reference use; forces and statistics stay close to the FP64 path's."""
    case, z = load_golden("post_cyl24x12_m2")
    ch = N.CaseHandle.from_case(case)
    walls = _wall_patches(case)
    out = []
    for prec in (N.LFM_FP64, N.LFM_FP32_BULK):
        s = N.Solver(ch, precision=prec)
        s.stats_reset()
        for k in range(1, 21):
            s.step(1, case.delta_t)
            s.stats_accumulate(k)
        fp, fv = s.forces(walls)
        pa, pr = s.stats_get(20)
        out.append((fp, fv, pa, pr))
        s.close()
    (fp64, fv64, pa64, pr64), (fp32, fv32, pa32, pr32) = out
    assert np.linalg.norm(fp32 - fp64) <= 1e-4 * np.linalg.norm(fp64)
    assert np.linalg.norm(fv32 - fv64) <= 1e-4 * np.linalg.norm(fv64)
    assert rel_l2(pa32[None], pa64[None])[0] <= 1e-7   # of p ~ 1e5 Pa: 0.01 Pa
    assert rel_l2(pr32[None], pr64[None])[0] <= 1e-3


def test_probes_record_pressure_history():
    case = cases.cylinder_case(n_theta=48, n_r=24, r1=10, first=0.03, Ls=3, solver=1, noise=0.02)
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch, precision=N.LFM_FP64)
    cells = np.array([0, 17, ch.desc.n_cells - 1], dtype=np.int64)
    s.probes_set(cells, capacity=8)
    hist = []
    for _ in range(5):
        s.step(1, case.delta_t)
        s.probes_record()
        q = s.get_state()
        r, m, E = q[0, cells], q[1:3, cells], q[3, cells]
        u2 = ((m / r) ** 2).sum(axis=0)
        hist.append(r * (ch.desc.gamma - 1) * (E / r - 0.5 * u2) - case.p_inf)
    h = s.probes_read()
    s.close()
    assert h.shape == (5, 3)
    np.testing.assert_allclose(h, np.array(hist), rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("name", POST)
def test_driver_writes_reference_post_processing(tmp_path, name):
    if not os.path.exists(CLI):
        pytest.fail(f"{CLI} is missing: build() makes it")
    case, z = load_golden(name)
    n, start, save = int(z["n_steps"]), int(z["average_start"]), int(z["save_forces_step"])
    root = str(tmp_path / "case")
    cases.write_case(case, root, n_steps=n, post=dict(haveAverage=True, tStartAverage=case.delta_t * start,
                                                      haveForces=True, saveForcesStep=save, printInfoFreq=n))
    os.makedirs(os.path.join(root, "output"))
    r = subprocess.run([CLI], cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    rows = read_forces(os.path.join(root, "output", "postProcess_Forces_1"))
    _check_forces(rows, z["ref_forces"], case.dim)
    head = open(os.path.join(root, "output", "postProcess_Forces_1")).readline()
    assert head.split() == ["time"] + [f"F{a},{x}" for a in "pv" for x in "xyz"[:case.dim]] + \
        [w for x in "xyz"[:case.dim] for w in (f"Fp,{x}", "+", f"Fv,{x}")]
    f = cases.read_result_fields(root, names=("rho", "pAvg", "pRMS"))
    assert rel_l2(f["pAvg"][None], z["ref_pAvg"][None])[0] <= 1e-12
    assert rel_l2(f["pRMS"][None], z["ref_pRMS"][None])[0] <= 1e-8
    assert rel_l2(f["rho"][None], z["ref_rho"][None])[0] <= 1e-12
    shutil.rmtree(root, ignore_errors=True)


@pytest.mark.parametrize("name,nparts,method", [("post_cyl24x12_m2", 3, "random"), ("post_cyl24x12_m2", 2, "x")])
def test_driver_runs_decomposed_case(tmp_path, name, nparts, method):
    """`lfm_solve_gpu -p` on processor0..N-1 (the reference's
    `mpirun -np N lfm_solve -p`): every partition in one process on the GPU,
    each writing its processor directory; reassembled fields, statistics and
    the summed wall forces match the reference's undecomposed run."""
    case, z = load_golden(name)
    n, start, save = int(z["n_steps"]), int(z["average_start"]), int(z["save_forces_step"])
    root = str(tmp_path / "case")
    part = cases.decompose_case(case, root, nparts, method=method, seed=4, n_steps=n,
                                post=dict(haveAverage=True, tStartAverage=case.delta_t * start, haveForces=True,
                                          saveForcesStep=save, printInfoFreq=n))
    os.makedirs(os.path.join(root, "output"))
    r = subprocess.run([CLI, "-p"], cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "partitions   : %d" % nparts in r.stdout
    glob = {k: np.full(case.n_cells, np.nan) for k in ("rho", "p", "pAvg", "pRMS")}
    for p in range(nparts):
        f = cases.read_result_fields(os.path.join(root, f"processor{p}"), names=tuple(glob))
        cells = np.nonzero(part == p)[0]
        for k in glob:
            glob[k][cells] = f[k]
    for k, tol in (("rho", 1e-12), ("p", 1e-12), ("pAvg", 1e-12), ("pRMS", 1e-8)):
        assert np.all(np.isfinite(glob[k])), k
        assert rel_l2(glob[k][None], z["ref_" + k][None])[0] <= tol, k
    rows = read_forces(os.path.join(root, "output", "postProcess_Forces_1"))
    _check_forces(rows, z["ref_forces"], case.dim)


@pytest.mark.parametrize("name", adjust_names())
def test_driver_adaptive_dt_matches_reference(tmp_path, name):
    """lfm_solve_gpu with adjustTimeStep yes: every step's printed time and
    dt (printInfoFreq 1) are the reference's to its printed precision, the
    run ends after the same step, and the final fields match within 1e-12."""
    if not os.path.exists(CLI):
        pytest.fail(f"{CLI} is missing: build() makes it")
    case, z = load_golden(name)
    root = str(tmp_path / "case")
    cases.write_case(case, root, n_steps=int(z["n_steps"]), write_interval=1, post=dict(printInfoFreq=1),
                     adjust_time_step=True, max_co=float(z["max_co"]))
    r = subprocess.run([CLI], cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    rows = np.array([(int(a), float(b), float(c)) for a, b, c in
                     re.findall(r"Time step:\s*(\d+)\s+Time:\s*([0-9eE+\-.]+)\s+dt:\s*([0-9eE+\-.]+)", r.stdout)])
    assert rows.shape[0] == len(z["ref_dt"]), r.stdout[-1500:]
    np.testing.assert_array_equal(rows[:, 0], z["ref_step"])
    np.testing.assert_allclose(rows[:, 1], z["ref_time"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(rows[:, 2], z["ref_dt"], rtol=1e-9, atol=0)
    f = cases.read_result_fields(root, names=("rho", "E", "p"))
    for k in ("rho", "E", "p"):
        assert rel_l2(f[k][None], z["ref_" + k][None])[0] <= 1e-12, k
    shutil.rmtree(root, ignore_errors=True)
