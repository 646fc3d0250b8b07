"""Shared helpers of the test suite."""
import glob
import os

import numpy as np

from lfm_public_gb300 import _native as N
from tests.golden.make_golden import arrays_to_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


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
