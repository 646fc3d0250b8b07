"""Acoustic-pressure comparison of two solver states.

The FP32-bulk form is judged by the pressure fluctuation p' = p - p_inf it
produces: its relative L2 error against an FP64 result of the same case and
step count, over all cells or over a ring of probes (the aeroacoustic
cylinder records p' on 72 probes at r = 50 D).
"""
from __future__ import annotations

import math

import numpy as np


def pressure(q: np.ndarray, gamma: float, dim: int) -> np.ndarray:
    """p = (gamma - 1) (rho E - |rho u|^2 / (2 rho)) of a conserved state
    [nq][n] (solver order)."""
    rho = q[0]
    ke = 0.5 * np.sum(q[1:1 + dim] ** 2, axis=0) / rho
    return (gamma - 1.0) * (q[dim + 1] - ke)


def acoustic_rel_l2(q: np.ndarray, q_ref: np.ndarray, gamma: float, dim: int, p_inf: float,
                    cells: np.ndarray | None = None) -> float:
    """||p'(q) - p'(q_ref)|| / ||p'(q_ref)|| with p' = p - p_inf, over ``cells``
    (solver-order indices) or all cells."""
    p = pressure(q, gamma, dim)
    pr = pressure(q_ref, gamma, dim)
    if cells is not None:
        p, pr = p[cells], pr[cells]
    den = float(np.linalg.norm(pr - p_inf))
    return float(np.linalg.norm(p - pr)) / den if den > 0 else float("inf")


def probe_ring(centres: np.ndarray, solver_ids: np.ndarray, radius: float, n: int = 72) -> np.ndarray:
    """Solver-order indices of the cells nearest to n probes equally spaced on
    the circle of ``radius`` about the origin (z ignored). ``centres`` are the
    case's cell centres, ``solver_ids`` the case cell id of each solver cell."""
    inv = np.empty(len(solver_ids), dtype=np.int64)
    inv[solver_ids] = np.arange(len(solver_ids))
    th = 2 * math.pi * np.arange(n) / n
    px, py = radius * np.cos(th), radius * np.sin(th)
    out = np.empty(n, dtype=np.int64)
    cx, cy = centres[:, 0], centres[:, 1]
    for k in range(n):
        out[k] = inv[int(np.argmin((cx - px[k]) ** 2 + (cy - py[k]) ** 2))]
    return out
