"""Shared helpers of the test suite."""
import glob
import os

import numpy as np

from lfm_public_gb300 import _native as N
from tests.golden.make_golden import arrays_to_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """Fixtures of runs at constant dt (every fixture but the adaptive-dt ones)."""
    return sorted(n for n in (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if not n.endswith("_adjustdt") and not n.startswith("cfg_"))


def adjust_names():
    """Fixtures of runs with adjustTimeStep yes (the reference's dt sequence)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*_adjustdt.npz")))


def adaptive_run(step, min_dt, case, z):
    """The reference's adaptive time loop (src/mesh_solver.cpp:474-740 with the
    run-time manager's running(): time < endTime - deltaT/2): step(dt) runs
    one time step, min_dt() is compute_dt's minimum on the new state, and
    the time advances by that new dt. Returns the new dts and times."""
    end = case.delta_t * int(z["n_steps"])
    dt, t, dts, times = case.delta_t, 0.0, [], []
    while t < end - 0.5 * dt:
        step(dt)
        dt = min_dt()
        t += dt
        dts.append(dt)
        times.append(t)
    return np.array(dts), np.array(times)


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    case = arrays_to_case(z)
    return case, z


def reference_conserved(z, ids, dim):
    """Conserved state in solver order from the reference's written fields."""
    rho = z["ref_rho"][ids]
    U = z["ref_U"][ids][:, :dim].T
    E = z["ref_E"][ids]
    return np.vstack([rho[None], rho[None] * U, (rho * E)[None]])


def primitives(q, gamma, dim):
    """rho, U, E, p as the reference's updateSolutionPrimitives computes them
    (src/cfd_v0.cpp:3010-3025)."""
    r = q[0]
    U = q[1:1 + dim] / r
    E = q[dim + 1] / r
    um2 = U[0] * U[0]
    for k in range(1, dim):
        um2 = um2 + U[k] * U[k]
    p = r * (gamma - 1) * (E - 0.5 * um2)
    return r, U, E, p


def rel_l2_vec(a, b, dim):
    """rel_l2 with the momentum rows measured as one vector field: each
    component's error against the norm of the whole momentum (a component
    that stays zero up to rounding, such as w in a flow uniform along z,
    would otherwise compare rounding noise with rounding noise)."""
    e = rel_l2(a, b)
    m = slice(1, 1 + dim)
    e[m] = np.linalg.norm(a[m] - b[m], axis=1) / np.linalg.norm(b[m])
    return e


def rel_l2(a, b):
    """Relative L2 error of each conserved field (rows); a field that is zero
    in b counts 0 when a matches it exactly and infinity otherwise."""
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(den > 0, num / np.where(den > 0, den, 1.0), np.where(num > 0, np.inf, 0.0))


def config_case(name):
    """A configured workload (cfg_* fixture) regenerated from its generator,
    checked against the fingerprint the fixture recorded when the reference
    ran it (relative 1e-13: the inputs may differ in the last bit between
    hosts, which no 1e-12 parity check can see)."""
    import json

    from lfm_public_gb300 import cases
    from tests.golden.make_golden import case_fingerprint
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    case = getattr(cases, str(z["generator"]))(**json.loads(str(z["kwargs"])))
    fp = case_fingerprint(case)
    for k, v in fp.items():
        ref = z[k]
        if np.issubdtype(np.asarray(v).dtype, np.integer):
            assert int(v) == int(ref), k
        else:
            assert np.allclose(v, ref, rtol=1e-13, atol=0), k
    return case, z
