"""Generates the golden fixtures of tests/golden/ by running the reference.

Each fixture is a small synthetic case (mesh, initial fields, dictionary
values) together with the fields the reference solver wrote after n_steps
time steps: rho, U, E, p per polyMesh cell, and the CFL it printed. The
reference is built from its own sources by oracle/Makefile (oracle/_ref/
lfm_oracle); this script only runs where those sources exist. The post_*
fixtures also hold the reference's pAvg / pRMS fields and its wall-force
records (haveAverage, haveForces). Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lfm_public_gb300 import cases  # noqa: E402

ORACLE = os.path.join(ROOT, "oracle", "_ref", "lfm_oracle")

# name -> (generator, kwargs, n_steps)
FIXTURES = {
    "vortex16_m1_visc": (cases.vortex_case, dict(n=16, mu=1e-3), 20),
    "vortex16_m2": (cases.vortex_case, dict(n=16, solver=1), 20),
    "vortex12x20_m1_res": (cases.vortex_case, dict(n=12, ny=20, mu=2e-3, beta=3.0), 20),
    "cyl24x12_m1_minmod": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=0,
                                                     minmod=True), 20),
    "cyl24x12_m2": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=1,
                                              minmod=True, noise=0.02), 20),
    "cyl24x12_ausm_minmod": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=2,
                                                       minmod=True, noise=0.02), 20),
    "cyl24x12_ausm_nominmod": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=2,
                                                         minmod=False, noise=0.02), 20),
    "cyl16x8x4_m2_3d": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=10, first=0.05, Ls=3, solver=1, n_span=4,
                                                  noise=0.01), 10),
    "cyl16x8x4_m1_3d": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=10, first=0.05, Ls=3, solver=0, n_span=4,
                                                  noise=0.01), 10),
    "cyl16x8x4_ausm_3d": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=10, first=0.05, Ls=3, solver=2, n_span=4,
                                                    noise=0.01), 10),
    "tri8_m1": (cases.tri_case, dict(n=8, seed=3), 20),
    "tri8_m2": (cases.tri_case, dict(n=8, seed=4, solver=1), 20),
    # Smagorinsky LES (turbulenceProperties simulationType LES)
    "les_cyl24x12_m2": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=1,
                                                  minmod=False, noise=0.05, reynolds=50.0), 20),
    "les_cyl16x8x4_m1_3d": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=10, first=0.05, Ls=3, solver=0,
                                                      n_span=4, noise=0.05, reynolds=50.0), 10),
    # the reference's 3D solvers for five and four faces a cell
    "prism5x3_m2_3d": (cases.prism_case, dict(n=5, nz=3, seed=2, solver=1), 10),
    "tet3x2_ausm_3d": (cases.tet_case, dict(n=3, nz=2, seed=2, solver=2), 10),
    # edge cases: one cell (no internal face), rkOrder 3 (three stages of the four-stage set)
    "vortex1_m1": (cases.vortex_case, dict(n=1), 5),
    "cyl16x8_m1_rk3": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=6, first=0.05, Ls=2, solver=0, minmod=True,
                                                 noise=0.05, seed=9, reynolds=60.0), 10),
}


def case_to_arrays(case: cases.Case) -> dict:
    out = dict(points=case.points, face_offsets=case.face_offsets, face_points=case.face_points,
               owner=case.owner, neighbour=case.neighbour, n_cells=np.int64(case.n_cells),
               cell_centres=case.cell_centres, dim=np.int64(case.dim),
               patch_names=np.array([p.name for p in case.patches]),
               patch_types=np.array([p.type for p in case.patches]),
               patch_start=np.array([p.start for p in case.patches], dtype=np.int64),
               patch_size=np.array([p.size for p in case.patches], dtype=np.int64),
               patch_neighbour=np.array([p.neighbour or "" for p in case.patches]))
    for k, v in case.fields.items():
        out["field_" + k] = v
    for k in ("solver", "rk_order", "minmod", "residuals", "laminar", "p_inf", "T_inf", "Ls", "mach", "k_sponge",
              "Cp", "mol_weight", "mu", "Pr", "delta_t"):
        out["param_" + k] = np.float64(getattr(case, k))
    out["param_U_inf"] = np.array(case.U_inf, dtype=np.float64)
    return out


def arrays_to_case(z) -> cases.Case:
    patches = [cases.Patch(str(n), str(t), int(s), int(z_), (str(nb) or None))
               for n, t, s, z_, nb in zip(z["patch_names"], z["patch_types"], z["patch_start"], z["patch_size"],
                                          z["patch_neighbour"])]
    c = cases.Case(name="golden", dim=int(z["dim"]), points=z["points"], face_offsets=z["face_offsets"],
                   face_points=z["face_points"], owner=z["owner"], neighbour=z["neighbour"], patches=patches,
                   n_cells=int(z["n_cells"]), cell_centres=z["cell_centres"])
    c.fields = {k[6:]: z[k] for k in z.files if k.startswith("field_")}
    for k in ("solver", "rk_order"):
        setattr(c, k, int(z["param_" + k]))
    for k in ("minmod", "residuals"):
        setattr(c, k, bool(z["param_" + k]))
    c.laminar = bool(z["param_laminar"]) if "param_laminar" in z.files else True
    for k in ("p_inf", "T_inf", "Ls", "mach", "k_sponge", "Cp", "mol_weight", "mu", "Pr", "delta_t"):
        setattr(c, k, float(z["param_" + k]))
    c.U_inf = tuple(float(x) for x in z["param_U_inf"])
    return c


def run_reference(case: cases.Case, n_steps: int, workdir: str):
    cases.write_case(case, workdir, n_steps=n_steps)
    # print the CFL once, at the last step
    cd = os.path.join(workdir, "system", "controlDict")
    txt = open(cd).read().replace(f"printInfoFreq   {case.print_freq}", f"printInfoFreq   {n_steps}")
    if case.residuals:
        txt = txt.replace("saveResiduals   false", "saveResiduals   true")
    open(cd, "w").write(txt)
    r = subprocess.run([ORACLE], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference run failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
    m = re.findall(r"CFL:\s*([0-9eE+\-.]+)", r.stdout)
    cfl = float(m[-1]) if m else float("nan")
    fields = cases.read_result_fields(workdir)
    if case.residuals:
        fields.update(cases.read_result_fields(workdir, names=["rhoRES", "uRES", "vRES", "eRES"][:case.dim + 2]
                                               if case.dim == 2 else ["rhoRES", "uRES", "vRES", "wRES", "eRES"]))
    return fields, cfl, r.stdout


# Adaptive time step (adjustTimeStep yes): the reference's compute_dt and its
# MPI_Allreduce(MIN) (src/cfd_v0.cpp:2912-2942, src/mesh_solver.cpp:705-716)
# set each next dt; printInfoFreq 1 prints every step's time and new dt, and
# every step is written (the run ends at endTime, before step n_steps).
# name -> (generator, kwargs, nominal n_steps, maxCo)
ADJUST_FIXTURES = {
    "vortex16_m2_adjustdt": (cases.vortex_case, dict(n=16, solver=1, mu=1e-3), 20, 0.2),
    "cyl24x12_m1_adjustdt": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=0,
                                                       minmod=True, noise=0.02), 20, 0.25),
}

_STEP_LINE = re.compile(r"Time step:\s*(\d+)\s+Time:\s*([0-9eE+\-.]+)\s+dt:\s*([0-9eE+\-.]+)")


def run_reference_adjust(case: cases.Case, n_steps: int, max_co: float, workdir: str):
    cases.write_case(case, workdir, n_steps=n_steps, write_interval=1, post=dict(printInfoFreq=1),
                     adjust_time_step=True, max_co=max_co)
    r = subprocess.run([ORACLE], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference run failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
    rows = np.array([(int(a), float(b), float(c)) for a, b, c in _STEP_LINE.findall(r.stdout)])
    return cases.read_result_fields(workdir), rows


def main_adjust():
    for name, (gen, kw, n, max_co) in ADJUST_FIXTURES.items():
        case = gen(n_steps=n, **kw)
        tmp = tempfile.mkdtemp(prefix="lfm_golden_")
        try:
            res, rows = run_reference_adjust(case, n, max_co, tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        arrs = case_to_arrays(case)
        arrs.update({f"ref_{k}": v for k, v in res.items()})
        arrs["n_steps"] = np.int64(n)
        arrs["max_co"] = np.float64(max_co)
        arrs["ref_step"] = rows[:, 0].astype(np.int64)
        arrs["ref_time"] = rows[:, 1]
        arrs["ref_dt"] = rows[:, 2]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(f"{name}: {case.n_cells} cells, {len(rows)} steps to endTime {case.delta_t * n:.6g}, "
              f"dt {rows[0, 2]:.6g} .. {rows[-1, 2]:.6g}")


# The configured workloads at full size and length, checked against the
# reference: the mesh is regenerated from its generator (the fixture holds a
# digest of the generated mesh and initial fields, which the test checks),
# and the fixture keeps the reference's fields on a seeded sample of cells.
# name -> (generator, kwargs, n_steps)
CONFIG_FIXTURES = {
    # 2D isentropic vortex, 256 x 256, M1, rkOrder 5, CFL 0.5, 1000 steps
    "cfg_vortex256_m1_1000": (cases.vortex_case, dict(n=256, solver=0), 1000),
    # 2D cylinder O-grid 768 x 512, M1, minmod on, 20 steps (100 RK stages)
    "cfg_cyl768x512_m1_20": (cases.cylinder_case, dict(n_theta=768, n_r=512, solver=0, minmod=True), 20),
}
SAMPLE_CELLS = 4096


def case_fingerprint(case: cases.Case) -> dict:
    """Values that pin a regenerated case to the one the reference ran: the
    norms of the points and of every initial field, dt, and the initial
    fields on the sampled cells. They are compared with a relative tolerance:
    numpy's transcendental functions may differ in the last bit between
    hosts, which moves a 1000-step FP64 result by far less than 1e-12."""
    cells = sample_cells(case.n_cells)
    out = {"fp_points_norm": np.float64(np.linalg.norm(case.points)), "fp_delta_t": np.float64(case.delta_t),
           "fp_n_faces": np.int64(len(case.owner)), "fp_n_internal": np.int64(len(case.neighbour))}
    for k in sorted(case.fields):
        v = np.asarray(case.fields[k], dtype=np.float64)
        out["fp_norm_" + k] = np.float64(np.linalg.norm(v))
        out["fp_sample_" + k] = v[cells]
    return out


def sample_cells(n_cells: int) -> np.ndarray:
    return np.sort(np.random.default_rng(20261204).choice(n_cells, size=min(SAMPLE_CELLS, n_cells), replace=False))


def main_config():
    import json
    for name, (gen, kw, n) in CONFIG_FIXTURES.items():
        case = gen(**kw)
        tmp = tempfile.mkdtemp(prefix="lfm_golden_")
        try:
            res, cfl, _ = run_reference(case, n, tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        cells = sample_cells(case.n_cells)
        arrs = {"generator": np.array(gen.__name__), "kwargs": np.array(json.dumps(kw)),
                "n_steps": np.int64(n), "n_cells": np.int64(case.n_cells), "sample": cells,
                "ref_cfl": np.float64(cfl)}
        arrs.update(case_fingerprint(case))
        for k in ("rho", "E", "p"):
            arrs["ref_" + k] = res[k][cells]
            arrs["ref_norm_" + k] = np.float64(np.linalg.norm(res[k]))
        arrs["ref_U"] = res["U"][cells]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(f"{name}: {case.n_cells} cells, {n} steps, {len(cells)} sampled cells, CFL {cfl}")


# Post-processing fixtures: the same runs with haveAverage (pAvg, pRMS fields)
# and haveForces (output/postProcess_Forces_1) switched on.
# name -> (generator, kwargs, n_steps, averaging start step, saveForcesStep)
POST_FIXTURES = {
    "post_cyl24x12_m2": (cases.cylinder_case, dict(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=1,
                                                   minmod=False, noise=0.02), 20, 5, 5),
    "post_cyl16x8x4_ausm_3d": (cases.cylinder_case, dict(n_theta=16, n_r=8, r1=10, first=0.05, Ls=3, solver=2,
                                                         n_span=4, noise=0.01), 10, 3, 2),
}


def read_forces(path: str) -> np.ndarray:
    """Rows of a postProcess_Forces file: time, Fp[D], Fv[D], Fp + Fv[D]."""
    rows = [ln.split() for ln in open(path).read().splitlines()[1:] if ln.strip()]
    return np.array(rows, dtype=np.float64)


def run_reference_post(case: cases.Case, n_steps: int, start: int, save_step: int, workdir: str):
    post = dict(haveAverage=True, tStartAverage=case.delta_t * start, haveForces=True, saveForcesStep=save_step,
                printInfoFreq=n_steps)
    cases.write_case(case, workdir, n_steps=n_steps, post=post)
    os.makedirs(os.path.join(workdir, "output"), exist_ok=True)
    r = subprocess.run([ORACLE], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference run failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
    m = re.findall(r"CFL:\s*([0-9eE+\-.]+)", r.stdout)
    fields = cases.read_result_fields(workdir, names=("rho", "E", "p", "U", "pAvg", "pRMS"))
    forces = read_forces(os.path.join(workdir, "output", "postProcess_Forces_1"))
    return fields, forces, float(m[-1]) if m else float("nan")


def main_post():
    for name, (gen, kw, n, start, save) in POST_FIXTURES.items():
        case = gen(n_steps=n, **kw)
        tmp = tempfile.mkdtemp(prefix="lfm_golden_")
        try:
            res, forces, cfl = run_reference_post(case, n, start, save, tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        arrs = case_to_arrays(case)
        arrs.update({f"ref_{k}": v for k, v in res.items()})
        arrs["ref_forces"] = forces
        arrs["ref_cfl"] = np.float64(cfl)
        arrs["n_steps"] = np.int64(n)
        arrs["average_start"] = np.int64(start)
        arrs["save_forces_step"] = np.int64(save)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(f"{name}: {case.n_cells} cells, {n} steps, {forces.shape[0]} force records")


def main(only=()):
    """Writes every fixture, or only the named ones."""
    if not os.path.exists(ORACLE):
        raise SystemExit(f"{ORACLE} is missing: run `make -C oracle` where the reference sources exist")
    if not only:
        main_post()
        main_adjust()
        main_config()
    if any(n in ADJUST_FIXTURES for n in only):
        main_adjust()
    if any(n in CONFIG_FIXTURES for n in only):
        main_config()
    for name, (gen, kw, n) in FIXTURES.items():
        if only and name not in only:
            continue
        case = gen(n_steps=n, **kw)
        if name.endswith("_res"):
            case.residuals = True
        if name.startswith("les_"):
            case.laminar = False
        m = re.search(r"_rk(\d)$", name)
        if m:
            case.rk_order = int(m.group(1))
        tmp = tempfile.mkdtemp(prefix="lfm_golden_")
        try:
            res, cfl, _ = run_reference(case, n, tmp)
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        arrs = case_to_arrays(case)
        arrs.update({f"ref_{k}": v for k, v in res.items()})
        arrs["ref_cfl"] = np.float64(cfl)
        arrs["n_steps"] = np.int64(n)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(f"{name}: {case.n_cells} cells, {n} steps, CFL {cfl}")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
