"""Synthetic OpenFOAM cases for the explicit time step.

The reference is validated on OpenFOAM cases (polyMesh + 0/{p,T,U,alpha} +
system/ and constant/ dictionaries, reference README.md:89-160). Its example
meshes are not shipped, so every case here is generated from a seed:

* ``vortex_case``     -- uniform quad grid of [-L, L]^2 with an isentropic vortex
                         (2D isentropic vortex advection workload, 256x256).
* ``cylinder_case``   -- stretched O-grid around a cylinder of diameter 1, wall
                         on the cylinder, inlet/outlet on the outer circle
                         (2D cylinder aeroacoustics workload, 768x512; with
                         ``n_span`` > 1 the section is extruded with cyclic
                         spanwise patches, the 3D wake workload).
* ``tri_case``        -- jittered triangulation of a square (split quads).

A case is a :class:`Case`: polyMesh arrays (points, CSR faces, owner,
neighbour, patches), initial fields per cell and the dictionary values. It can
be written as an OpenFOAM case directory (``write_case``) for the file-based
path (CPolyMeshReaderOF / CDictReaderOF) or handed to the C ABI directly.

Cell ordering follows the generator's natural index (i fastest). The
free-stream, vortex and sponge formulas are stated in each generator.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

RUNIVERSAL = 8.31447  # J/(mol K), as the reference (api/cfdv0_solver.h:138)


@dataclass
class Patch:
    name: str
    type: str
    start: int
    size: int
    neighbour: Optional[str] = None
    my_proc: Optional[int] = None          # processor patches (decomposed cases)
    neighb_proc: Optional[int] = None


@dataclass
class Case:
    name: str
    dim: int
    points: np.ndarray            # (n_points, 3)
    face_offsets: np.ndarray      # (n_faces + 1,) int64
    face_points: np.ndarray       # int64
    owner: np.ndarray             # (n_faces,) int64
    neighbour: np.ndarray         # (n_internal,) int64
    patches: List[Patch]
    n_cells: int
    cell_centres: np.ndarray      # (n_cells, 3) vertex-average estimate
    fields: Dict[str, np.ndarray] = field(default_factory=dict)   # p, T, U (n,3), alpha
    # dictionary values
    solver: int = 0
    rk_order: int = 5
    minmod: bool = False
    residuals: bool = False
    laminar: bool = True          # False: Smagorinsky LES viscous terms (turbulenceProperties LES)
    p_inf: float = 101325.0
    T_inf: float = 300.0
    U_inf: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    Ls: float = 0.0
    mach: float = 0.0
    k_sponge: float = 0.434294481903252
    Cp: float = 1005.0
    mol_weight: float = 28.96
    mu: float = 0.0
    Pr: float = 0.71
    delta_t: float = 1e-5
    n_steps: int = 10
    print_freq: int = 1000000
    write_precision: int = 17

    @property
    def n_faces(self) -> int:
        return int(self.owner.shape[0])

    @property
    def Rgas(self) -> float:
        return RUNIVERSAL / self.mol_weight * 1000

    @property
    def gamma(self) -> float:
        return self.Cp / (self.Cp - self.Rgas)

    @property
    def rho_inf(self) -> float:
        return self.p_inf / (self.Rgas * self.T_inf)

    def params(self) -> dict:
        return dict(solver=self.solver, dimension=self.dim, rk_order=self.rk_order, minmod=int(self.minmod),
                    laminar=int(self.laminar), residuals=int(self.residuals), p_inf=self.p_inf, T_inf=self.T_inf,
                    U_inf=tuple(self.U_inf), Ls=self.Ls, mach=self.mach, k_sponge=self.k_sponge, Cp=self.Cp,
                    mol_weight=self.mol_weight, mu=self.mu, Pr=self.Pr)


# ---------------------------------------------------------------------------
# structured hexahedral blocks
# ---------------------------------------------------------------------------
def _quad_faces(a, b, c, d):
    return np.stack([a, b, c, d], axis=-1).reshape(-1, 4)


def structured_block(X: np.ndarray, periodic_j: bool, boundary: Dict[str, Tuple[str, str]],
                     cyclic_k: Optional[Tuple[str, str]] = None):
    """polyMesh of a structured block of hexahedra.

    X: point coordinates (ni+1, nj', nk+1, 3) with nj' = nj when periodic_j
    (index j wraps) else nj + 1; the index map (i, j, k) -> x must be
    right-handed. ``boundary`` maps the block sides "i0", "i1", "j0", "j1",
    "k0", "k1" to (patch name, patch type); several sides may share one patch
    name. ``cyclic_k`` names the (k0, k1) cyclic pair instead of k sides.
    Returns (points, face_offsets, face_points, owner, neighbour, patches,
    n_cells, cell_centres).
    """
    ni = X.shape[0] - 1
    nj = X.shape[1] if periodic_j else X.shape[1] - 1
    nk = X.shape[2] - 1
    NJp = X.shape[1]
    points = X.transpose(2, 1, 0, 3).reshape(-1, 3)  # i fastest, then j, then k

    def pid(i, j, k):
        jj = np.mod(j, nj) if periodic_j else j
        return i + (ni + 1) * (jj + NJp * k)

    def cid(i, j, k):
        return i + ni * (j + nj * k)

    n_cells = ni * nj * nk
    # +i faces at index plane i (points of plane i), +j at plane j, +k at plane k
    def face_i(i, j, k):
        return _quad_faces(pid(i, j, k), pid(i, j + 1, k), pid(i, j + 1, k + 1), pid(i, j, k + 1))

    def face_j(i, j, k):
        return _quad_faces(pid(i, j, k), pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j, k))

    def face_k(i, j, k):
        return _quad_faces(pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k))

    int_faces, int_own, int_nei = [], [], []
    # i interfaces
    if ni > 1:
        I, J, K = np.meshgrid(np.arange(1, ni), np.arange(nj), np.arange(nk), indexing="ij")
        I, J, K = I.ravel(), J.ravel(), K.ravel()
        int_faces.append(face_i(I, J, K))
        int_own.append(cid(I - 1, J, K))
        int_nei.append(cid(I, J, K))
    # j interfaces
    jr = np.arange(1, nj)
    if jr.size:
        I, J, K = np.meshgrid(np.arange(ni), jr, np.arange(nk), indexing="ij")
        I, J, K = I.ravel(), J.ravel(), K.ravel()
        int_faces.append(face_j(I, J, K))
        int_own.append(cid(I, J - 1, K))
        int_nei.append(cid(I, J, K))
    if periodic_j:
        I, K = np.meshgrid(np.arange(ni), np.arange(nk), indexing="ij")
        I, K = I.ravel(), K.ravel()
        J = np.zeros_like(I)
        f = face_j(I, J, K)[:, ::-1]   # normal from cell j=0 (owner) towards j=nj-1
        int_faces.append(f)
        int_own.append(cid(I, J, K))
        int_nei.append(cid(I, J + nj - 1, K))
    if nk > 1:
        I, J, K = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(1, nk), indexing="ij")
        I, J, K = I.ravel(), J.ravel(), K.ravel()
        int_faces.append(face_k(I, J, K))
        int_own.append(cid(I, J, K - 1))
        int_nei.append(cid(I, J, K))
    if not int_faces:   # a single cell: no internal face
        int_faces, int_own, int_nei = [np.zeros((0, 4), dtype=np.int64)], [np.zeros(0, np.int64)], \
            [np.zeros(0, np.int64)]
    F = np.concatenate(int_faces)
    own = np.concatenate(int_own)
    nei = np.concatenate(int_nei)
    sw = own > nei
    own[sw], nei[sw] = nei[sw], own[sw].copy()
    order = np.lexsort((nei, own))
    F, own, nei = F[order], own[order], nei[order]

    # boundary sides
    sides = {}
    I, J = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
    if not periodic_j:
        I2, K2 = np.meshgrid(np.arange(ni), np.arange(nk), indexing="ij")
        I2, K2 = I2.ravel(), K2.ravel()
        sides["j0"] = (face_j(I2, 0 * I2, K2)[:, ::-1], cid(I2, 0 * I2, K2))
        sides["j1"] = (face_j(I2, 0 * I2 + nj, K2), cid(I2, 0 * I2 + nj - 1, K2))
    J2, K2 = np.meshgrid(np.arange(nj), np.arange(nk), indexing="ij")
    J2, K2 = J2.ravel(), K2.ravel()
    sides["i0"] = (face_i(0 * J2, J2, K2)[:, ::-1], cid(0 * J2, J2, K2))
    sides["i1"] = (face_i(0 * J2 + ni, J2, K2), cid(0 * J2 + ni - 1, J2, K2))
    I3, J3 = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
    I3, J3 = I3.ravel(order="F"), J3.ravel(order="F")
    sides["k0"] = (face_k(I3, J3, 0 * I3)[:, ::-1], cid(I3, J3, 0 * I3))
    sides["k1"] = (face_k(I3, J3, 0 * I3 + nk), cid(I3, J3, 0 * I3 + nk - 1))

    patch_faces: Dict[str, List] = {}
    patch_types: Dict[str, str] = {}
    patch_order: List[str] = []
    for side, (pname, ptype) in boundary.items():
        if pname not in patch_faces:
            patch_faces[pname] = []
            patch_types[pname] = ptype
            patch_order.append(pname)
        patch_faces[pname].append(sides[side])
    if cyclic_k is not None:
        for side, pname, nb in (("k0", cyclic_k[0], cyclic_k[1]), ("k1", cyclic_k[1], cyclic_k[0])):
            patch_faces[pname] = [sides[side]]
            patch_types[pname] = "cyclic:" + nb
            patch_order.append(pname)

    faces = [F]
    owners = [own]
    patches = []
    start = F.shape[0]
    for pname in patch_order:
        fl = np.concatenate([x[0] for x in patch_faces[pname]])
        ol = np.concatenate([x[1] for x in patch_faces[pname]])
        faces.append(fl)
        owners.append(ol)
        ptype = patch_types[pname]
        nb = None
        if ptype.startswith("cyclic:"):
            nb = ptype.split(":", 1)[1]
            ptype = "cyclic"
        patches.append(Patch(pname, ptype, start, int(fl.shape[0]), nb))
        start += int(fl.shape[0])
    allF = np.concatenate(faces).astype(np.int64)
    face_offsets = np.arange(0, 4 * allF.shape[0] + 1, 4, dtype=np.int64)
    owner = np.concatenate(owners).astype(np.int64)
    # vertex-average cell centres
    i0, j0, k0 = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    cc = np.zeros((ni, nj, nk, 3))
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                cc += points[pid(i0 + di, j0 + dj, k0 + dk)]
    cc /= 8.0
    cell_centres = cc.transpose(2, 1, 0, 3).reshape(-1, 3)
    return (points.astype(np.float64), face_offsets, allF.ravel(), owner, nei.astype(np.int64), patches, n_cells,
            cell_centres)


def _build(name, dim, block, **kw) -> Case:
    points, fo, fp, owner, nei, patches, nc, cc = block
    return Case(name=name, dim=dim, points=points, face_offsets=fo, face_points=fp, owner=owner, neighbour=nei,
                patches=patches, n_cells=nc, cell_centres=cc, **kw)


# ---------------------------------------------------------------------------
# flow states
# ---------------------------------------------------------------------------
def sound_speed(case: Case) -> float:
    return math.sqrt(case.gamma * case.Rgas * case.T_inf)


def isentropic_vortex(case: Case, x: np.ndarray, y: np.ndarray, beta: float, radius: float = 1.0):
    """Shu's isentropic vortex on the free stream of ``case``.

    With r^2 = (x^2 + y^2)/radius^2 and the velocity scale sqrt(R T_inf):
      u = U_inf + sqrt(R T_inf) beta/(2 pi) exp((1 - r^2)/2) (-y, x)/radius
      T/T_inf = 1 - (gamma - 1) beta^2 / (8 gamma pi^2) exp(1 - r^2)
      p = p_inf (T/T_inf)^(gamma/(gamma-1))
    """
    g = case.gamma
    r2 = (x * x + y * y) / (radius * radius)
    scale = math.sqrt(case.Rgas * case.T_inf)
    amp = scale * beta / (2 * math.pi) * np.exp(0.5 * (1 - r2))
    u = case.U_inf[0] - amp * y / radius
    v = case.U_inf[1] + amp * x / radius
    Tr = 1 - (g - 1) * beta * beta / (8 * g * math.pi ** 2) * np.exp(1 - r2)
    T = case.T_inf * Tr
    p = case.p_inf * Tr ** (g / (g - 1))
    return p, T, u, v


def acoustic_dt(case: Case, cfl: float, u: np.ndarray, T: np.ndarray, h: np.ndarray) -> float:
    """dt = cfl * min over cells of h / (|u| + c), h the cell's smallest width."""
    c = np.sqrt(case.gamma * case.Rgas * T)
    return float(cfl * np.min(h / (np.abs(u) + c)))


def _uniform_fields(case: Case, noise: float = 0.0, seed: int = 0):
    n = case.n_cells
    U = np.tile(np.asarray(case.U_inf, dtype=np.float64), (n, 1))
    if noise > 0:
        rng = np.random.default_rng(seed)
        umag = math.sqrt(sum(x * x for x in case.U_inf))
        U[:, :case.dim] += rng.uniform(-noise, noise, size=(n, case.dim)) * umag
    case.fields["U"] = U
    case.fields["p"] = np.full(n, case.p_inf)
    case.fields["T"] = np.full(n, case.T_inf)


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------
def vortex_case(n: int = 256, half: float = 10.0, mach: float = 0.5, beta: float = 5.0, solver: int = 0,
                n_steps: int = 1000, cfl: float = 0.5, mu: float = 0.0, ny: Optional[int] = None,
                mol_weight: float = 28.9647) -> Case:
    """2D isentropic vortex advection: n x ny quads on [-half, half]^2, one cell
    thick (z in [0,1], empty front/back), 'inlet' patch at x=-half, 'outlet'
    patch at x=+half (type patch), 'walls' (type wall) at y=+-half. gamma=1.4
    through Cp = 3.5 R. Sponge: alpha = half - x (distance from the outlet),
    Ls = 2, k = 0.434294481903252. Euler (mu = 0) unless ``mu`` is given."""
    ny = n if ny is None else ny
    xs = np.linspace(-half, half, n + 1)
    ys = np.linspace(-half, half, ny + 1)
    X = np.zeros((n + 1, ny + 1, 2, 3))
    X[..., 0] = xs[:, None, None]
    X[..., 1] = ys[None, :, None]
    X[..., 2] = np.array([0.0, 1.0])[None, None, :]
    blk = structured_block(X, False, {"i0": ("inlet", "patch"), "i1": ("outlet", "patch"), "j0": ("walls", "wall"),
                                      "j1": ("walls", "wall"), "k0": ("frontAndBack", "empty"),
                                      "k1": ("frontAndBack", "empty")})
    R = RUNIVERSAL / mol_weight * 1000
    case = _build(f"vortex{n}x{ny}", 2, blk, solver=solver, Cp=3.5 * R, mol_weight=mol_weight, mu=mu, Pr=0.71,
                  p_inf=101325.0, T_inf=300.0, mach=mach, Ls=2.0, n_steps=n_steps)
    c = sound_speed(case)
    case.U_inf = (mach * c, 0.0, 0.0)
    x, y = case.cell_centres[:, 0], case.cell_centres[:, 1]
    p, T, u, v = isentropic_vortex(case, x, y, beta)
    case.fields = {"p": p, "T": T, "U": np.stack([u, v, np.zeros_like(u)], axis=1), "alpha": half - x}
    h = np.full(case.n_cells, min(2 * half / n, 2 * half / ny))
    case.delta_t = acoustic_dt(case, cfl, np.hypot(u, v), T, h)
    return case


def _geometric_ratio(first: float, total: float, n: int) -> float:
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = first * (mid ** n - 1) / (mid - 1)
        lo, hi = (mid, hi) if s < total else (lo, mid)
    return 0.5 * (lo + hi)


def cylinder_case(n_theta: int = 768, n_r: int = 512, r0: float = 0.5, r1: float = 100.0, first: float = 0.002,
                  mach: float = 0.2, reynolds: float = 150.0, solver: int = 0, minmod: bool = True,
                  n_span: int = 1, span: float = math.pi, Ls: float = 20.0, noise: float = 0.0,
                  seed: int = 3900, n_steps: int = 20000, cfl: float = 0.5) -> Case:
    """Stretched O-grid around a cylinder of diameter 1 (radius r0): n_r cells
    radially with first width ``first`` and geometric growth to r1, n_theta
    cells azimuthally (the seam is an internal face). Patches: 'cylinder'
    (wall), outer circle split into 'inlet' (x < 0) and 'outlet' (x >= 0)
    (type patch), 'frontAndBack' (empty) in 2D or the cyclic pair
    'periodic_m'/'periodic_p' over ``span`` with ``n_span`` cells in 3D.
    Flow: M, Re on diameter 1, Pr 0.71, Cp 1005, molWeight 28.96, T_inf 300 K,
    p_inf 101325 Pa, mu = rho_inf U_inf / Re. Sponge: alpha = r1 - r (distance
    from the outer boundary), Ls in diameters. Initial field: free stream plus
    uniform noise of +-``noise`` U_inf per velocity component (seeded)."""
    q = _geometric_ratio(first, r1 - r0, n_r)
    rs = r0 + np.concatenate([[0.0], first * (q ** np.arange(1, n_r + 1) - 1) / (q - 1)])
    rs[-1] = r1
    th = np.linspace(0.0, 2 * math.pi, n_theta, endpoint=False)
    nk = n_span
    zs = np.linspace(0.0, span if n_span > 1 else 1.0, nk + 1)
    X = np.zeros((n_r + 1, n_theta, nk + 1, 3))
    X[..., 0] = rs[:, None, None] * np.cos(th)[None, :, None]
    X[..., 1] = rs[:, None, None] * np.sin(th)[None, :, None]
    X[..., 2] = zs[None, None, :]
    if n_span > 1:
        blk = structured_block(X, True, {"i0": ("cylinder", "wall"), "i1": ("outer", "patch")},
                               cyclic_k=("periodic_m", "periodic_p"))
        dim = 3
    else:
        blk = structured_block(X, True, {"i0": ("cylinder", "wall"), "i1": ("outer", "patch"),
                                         "k0": ("frontAndBack", "empty"), "k1": ("frontAndBack", "empty")})
        dim = 2
    blk = _split_outer(blk, n_theta, nk)
    case = _build(f"cylinder{n_theta}x{n_r}x{n_span}", dim, blk, solver=solver, minmod=minmod, Cp=1005.0,
                  mol_weight=28.96, Pr=0.71, p_inf=101325.0, T_inf=300.0, mach=mach, Ls=Ls, n_steps=n_steps)
    c = sound_speed(case)
    case.U_inf = (mach * c, 0.0, 0.0)
    case.mu = case.rho_inf * case.U_inf[0] * (2 * r0) / reynolds
    _uniform_fields(case, noise=noise, seed=seed)
    r = np.hypot(case.cell_centres[:, 0], case.cell_centres[:, 1])
    case.fields["alpha"] = r1 - r
    # smallest cell width: radial width or arc length
    ir = np.arange(case.n_cells) % n_r
    dr = np.diff(rs)[ir]
    arc = 2 * math.pi * rs[ir] / n_theta
    h = np.minimum(dr, arc)
    if n_span > 1:
        h = np.minimum(h, span / n_span)
    U = case.fields["U"]
    case.delta_t = acoustic_dt(case, cfl, np.linalg.norm(U, axis=1), case.fields["T"], h)
    return case


def _split_outer(blk, n_theta, nk):
    """Splits the 'outer' patch into 'inlet' (face centre x < 0) and 'outlet'."""
    points, fo, fp, owner, nei, patches, nc, cc = blk
    out = [p for p in patches if p.name == "outer"][0]
    F = fp.reshape(-1, 4)
    sl = slice(out.start, out.start + out.size)
    xc = points[F[sl]].mean(axis=1)[:, 0]
    inlet = np.nonzero(xc < 0)[0]
    outlet = np.nonzero(xc >= 0)[0]
    idx = np.concatenate([inlet, outlet]) + out.start
    Fo = F[out.start:out.start + out.size].copy()
    Oo = owner[out.start:out.start + out.size].copy()
    F[out.start:out.start + out.size] = F[idx]
    owner[out.start:out.start + out.size] = owner[idx]
    del Fo, Oo
    new = []
    for p in patches:
        if p.name == "outer":
            new.append(Patch("inlet", "patch", p.start, int(inlet.size)))
            new.append(Patch("outlet", "patch", p.start + int(inlet.size), int(outlet.size)))
        else:
            new.append(p)
    return points, fo, F.ravel(), owner, nei, new, nc, cc


def tri_case(n: int = 64, half: float = 10.0, jitter: float = 0.2, seed: int = 0, mach: float = 0.5,
             beta: float = 5.0, solver: int = 0, n_steps: int = 100, cfl: float = 0.5) -> Case:
    """Jittered triangulation of [-half, half]^2: an n x n grid whose interior
    vertices move by U(-jitter, jitter) h in x and y, every quad split along a
    random diagonal (2 n^2 triangles), extruded one cell thick. Patches and
    flow as ``vortex_case``."""
    rng = np.random.default_rng(seed)
    h = 2 * half / n
    xs = np.linspace(-half, half, n + 1)
    XX, YY = np.meshgrid(xs, xs, indexing="ij")
    inner = np.zeros_like(XX, dtype=bool)
    inner[1:-1, 1:-1] = True
    XX = XX + np.where(inner, rng.uniform(-jitter, jitter, XX.shape) * h, 0.0)
    YY = YY + np.where(inner, rng.uniform(-jitter, jitter, YY.shape) * h, 0.0)
    nodes = np.stack([XX.ravel(), YY.ravel()], axis=1)
    vid = lambda i, j: i * (n + 1) + j  # noqa: E731
    I, J = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    I, J = I.ravel(), J.ravel()
    a, b, c, d = vid(I, J), vid(I + 1, J), vid(I + 1, J + 1), vid(I, J + 1)   # ccw quad
    diag = rng.integers(0, 2, size=I.size).astype(bool)
    t1 = np.where(diag[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
    t2 = np.where(diag[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
    tris = np.empty((2 * I.size, 3), dtype=np.int64)
    tris[0::2], tris[1::2] = t1, t2
    case = _prism_mesh(nodes, tris, half, f"tri{n}", solver=solver, n_steps=n_steps)
    c0 = sound_speed(case)
    case.U_inf = (mach * c0, 0.0, 0.0)
    case.mach = mach
    x, y = case.cell_centres[:, 0], case.cell_centres[:, 1]
    p, T, u, v = isentropic_vortex(case, x, y, beta)
    case.fields = {"p": p, "T": T, "U": np.stack([u, v, np.zeros_like(u)], axis=1), "alpha": half - x}
    case.delta_t = acoustic_dt(case, cfl, np.hypot(u, v), T, np.full(case.n_cells, 0.5 * h * (1 - 2 * jitter)))
    return case


def hybrid_case(n: int = 16, tri_fraction: float = 0.5, half: float = 10.0, jitter: float = 0.2, seed: int = 0,
                mach: float = 0.5, beta: float = 5.0, solver: int = 0, n_steps: int = 100, cfl: float = 0.5) -> Case:
    """Mixed quadrilaterals and triangles on [-half, half]^2: the jittered
    n x n grid of ``tri_case`` with a random tri_fraction of its quads split
    along a random diagonal, extruded one cell thick (cells of 4 and 3 faces
    in one mesh; the reference sizes its solver for 4 and leaves a triangle's
    fourth slot empty). Patches and flow as ``vortex_case``."""
    rng = np.random.default_rng(seed)
    h = 2 * half / n
    xs = np.linspace(-half, half, n + 1)
    XX, YY = np.meshgrid(xs, xs, indexing="ij")
    inner = np.zeros_like(XX, dtype=bool)
    inner[1:-1, 1:-1] = True
    XX = XX + np.where(inner, rng.uniform(-jitter, jitter, XX.shape) * h, 0.0)
    YY = YY + np.where(inner, rng.uniform(-jitter, jitter, YY.shape) * h, 0.0)
    nodes = np.stack([XX.ravel(), YY.ravel()], axis=1)
    polys = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            if rng.uniform() < tri_fraction:
                if rng.integers(0, 2):
                    polys += [(a, b, c), (a, c, d)]
                else:
                    polys += [(a, b, d), (b, c, d)]
            else:
                polys.append((a, b, c, d))
    case = _polygon_mesh(nodes, polys, half, f"hybrid{n}", solver=solver, n_steps=n_steps)
    c0 = sound_speed(case)
    case.U_inf = (mach * c0, 0.0, 0.0)
    case.mach = mach
    x, y = case.cell_centres[:, 0], case.cell_centres[:, 1]
    p, T, u, v = isentropic_vortex(case, x, y, beta)
    case.fields = {"p": p, "T": T, "U": np.stack([u, v, np.zeros_like(u)], axis=1), "alpha": half - x}
    case.delta_t = acoustic_dt(case, cfl, np.hypot(u, v), T, np.full(case.n_cells, 0.5 * h * (1 - 2 * jitter)))
    return case


def _polyhedral_mesh(pts: np.ndarray, cells, half: float, name: str, **kw) -> Case:
    """3D polyMesh from convex cells given as lists of faces (vertex tuples in
    cyclic order, either orientation): each face is oriented outward from its
    cell by the cell-centroid test, a face shared by two cells is internal
    (owner the lower cell, oriented outward from it), the others form the
    patches inlet (x = -half), outlet (x = +half) and walls. A loop over the
    cells: for test-sized meshes."""
    T = len(cells)
    cc = np.zeros((T, 3))
    shared = {}
    for t, faces in enumerate(cells):
        verts = sorted({v for f in faces for v in f})
        c = pts[verts].mean(axis=0)
        cc[t] = c
        for f in faces:
            f = tuple(f)
            P = pts[list(f)]
            nrm = np.cross(P[1] - P[0], P[2] - P[0])
            if np.dot(nrm, P.mean(axis=0) - c) < 0:
                f = f[::-1]
            shared.setdefault(tuple(sorted(f)), []).append((t, f))
    internal, boundary = [], []
    for es in shared.values():
        if len(es) == 2:
            (t0, f0), (t1, f1) = sorted(es, key=lambda e: e[0])
            internal.append((t0, t1, f0))
        else:
            boundary.append(es[0])
    internal.sort(key=lambda e: (e[0], e[1]))
    tol = 1e-9 * half
    groups = {"inlet": [], "outlet": [], "walls": []}
    for t, f in boundary:
        mx = pts[list(f), 0].mean()
        groups["inlet" if mx < -half + tol else "outlet" if mx > half - tol else "walls"].append((t, f))
    faces = [f for _, _, f in internal]
    owner = [t for t, _, _ in internal]
    neighbour = [t1 for _, t1, _ in internal]
    patches = []
    start = len(faces)
    for pname, ptype in (("inlet", "patch"), ("outlet", "patch"), ("walls", "wall")):
        for t, f in groups[pname]:
            faces.append(f)
            owner.append(t)
        patches.append(Patch(pname, ptype, start, len(groups[pname])))
        start += len(groups[pname])
    face_points = np.array([v for f in faces for v in f], dtype=np.int64)
    face_offsets = np.concatenate([[0], np.cumsum([len(f) for f in faces])]).astype(np.int64)
    R = RUNIVERSAL / 28.9647 * 1000
    return Case(name=name, dim=3, points=pts, face_offsets=face_offsets, face_points=face_points,
                owner=np.array(owner, dtype=np.int64), neighbour=np.array(neighbour, dtype=np.int64),
                patches=patches, n_cells=T, cell_centres=cc, Cp=3.5 * R, mol_weight=28.9647, Pr=0.71, Ls=2.0, **kw)


def _vortex_tube(case: Case, half: float, beta: float, mach: float, h: float, cfl: float) -> Case:
    c0 = sound_speed(case)
    case.U_inf = (mach * c0, 0.0, 0.0)
    case.mach = mach
    x, y = case.cell_centres[:, 0], case.cell_centres[:, 1]
    p, T, u, v = isentropic_vortex(case, x, y, beta)
    case.fields = {"p": p, "T": T, "U": np.stack([u, v, np.zeros_like(u)], axis=1), "alpha": half - x}
    case.delta_t = acoustic_dt(case, cfl, np.hypot(u, v), T, np.full(case.n_cells, h))
    return case


def prism_case(n: int = 8, nz: int = 3, half: float = 10.0, depth: float = 4.0, jitter: float = 0.2, seed: int = 0,
               mach: float = 0.5, beta: float = 3.0, solver: int = 0, n_steps: int = 100, cfl: float = 0.5) -> Case:
    """3D triangular prisms (five faces a cell): the jittered triangulation of
    ``tri_case`` extruded into nz layers over z in [0, depth]; walls at the
    ends in z, an isentropic vortex tube along z."""
    rng = np.random.default_rng(seed)
    h = 2 * half / n
    xs = np.linspace(-half, half, n + 1)
    XX, YY = np.meshgrid(xs, xs, indexing="ij")
    inner = np.zeros_like(XX, dtype=bool)
    inner[1:-1, 1:-1] = True
    XX = XX + np.where(inner, rng.uniform(-jitter, jitter, XX.shape) * h, 0.0)
    YY = YY + np.where(inner, rng.uniform(-jitter, jitter, YY.shape) * h, 0.0)
    nn = (n + 1) * (n + 1)
    zs = np.linspace(0.0, depth, nz + 1)
    pts = np.zeros((nn * (nz + 1), 3))
    for k in range(nz + 1):
        pts[k * nn:(k + 1) * nn, 0] = XX.ravel()
        pts[k * nn:(k + 1) * nn, 1] = YY.ravel()
        pts[k * nn:(k + 1) * nn, 2] = zs[k]
    tris = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            tris += [(a, b, c), (a, c, d)] if rng.integers(0, 2) else [(a, b, d), (b, c, d)]
    cells = []
    for k in range(nz):
        lo, hi = k * nn, (k + 1) * nn
        for (a, b, c) in tris:
            tri_lo, tri_hi = (a + lo, b + lo, c + lo), (a + hi, b + hi, c + hi)
            sides = [(u + lo, w + lo, w + hi, u + hi) for u, w in ((a, b), (b, c), (c, a))]
            cells.append([tri_lo, tri_hi] + sides)
    case = _polyhedral_mesh(pts, cells, half, f"prism{n}x{nz}", solver=solver, n_steps=n_steps)
    return _vortex_tube(case, half, beta, mach, min(0.5 * h * (1 - 2 * jitter), 0.5 * depth / nz), cfl)


def tet_case(n: int = 5, nz: int = 2, half: float = 10.0, depth: float = 4.0, seed: int = 0, mach: float = 0.5,
             beta: float = 3.0, solver: int = 0, n_steps: int = 100, cfl: float = 0.5) -> Case:
    """3D tetrahedra (four faces a cell): an n x n x nz box of hexahedra over
    [-half, half]^2 x [0, depth], each split into the six tetrahedra of its
    main diagonal (Kuhn's subdivision, conforming between neighbours); walls
    at the ends in z, an isentropic vortex tube along z. seed jitters the
    interior vertices in x and y by up to 15 % of the spacing."""
    import itertools
    rng = np.random.default_rng(seed)
    h = 2 * half / n
    xs, zs = np.linspace(-half, half, n + 1), np.linspace(0.0, depth, nz + 1)
    X, Y, Z = np.meshgrid(xs, xs, zs, indexing="ij")
    inner = np.zeros_like(X, dtype=bool)
    inner[1:-1, 1:-1, :] = True
    X = X + np.where(inner, rng.uniform(-0.15, 0.15, X.shape) * h, 0.0)
    Y = Y + np.where(inner, rng.uniform(-0.15, 0.15, Y.shape) * h, 0.0)
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    vid = lambda i, j, k: (i * (n + 1) + j) * (nz + 1) + k  # noqa: E731
    cells = []
    for i in range(n):
        for j in range(n):
            for k in range(nz):
                for perm in itertools.permutations(range(3)):
                    p = [0, 0, 0]
                    path = [vid(i, j, k)]
                    for ax in perm:
                        p[ax] += 1
                        path.append(vid(i + p[0], j + p[1], k + p[2]))
                    cells.append([tuple(path[m] for m in range(4) if m != skip) for skip in range(4)])
    case = _polyhedral_mesh(pts, cells, half, f"tet{n}x{nz}", solver=solver, n_steps=n_steps)
    return _vortex_tube(case, half, beta, mach, 0.2 * min(h, depth / nz), cfl)


def _polygon_mesh(nodes, polys, half, name, **kw) -> Case:
    """polyMesh of counter-clockwise polygons (any vertex counts) extruded one
    cell thick in z, patches as ``_prism_mesh``. A loop over the cells: for
    test-sized meshes."""
    N = nodes.shape[0]
    T = len(polys)
    pts = np.zeros((2 * N, 3))
    pts[:N, :2] = nodes
    pts[N:, :2] = nodes
    pts[N:, 2] = 1.0
    edges = {}
    for t, pv in enumerate(polys):
        for k in range(len(pv)):
            a, b = pv[k], pv[(k + 1) % len(pv)]
            edges.setdefault((min(a, b), max(a, b)), []).append((t, a, b))
    internal, boundary = [], []
    for es in edges.values():
        if len(es) == 2:
            (t0, a0, b0), (t1, a1, b1) = es
            if t0 > t1:
                (t0, a0, b0), (t1, a1, b1) = (t1, a1, b1), (t0, a0, b0)
            internal.append((t0, t1, (a0, b0, b0 + N, a0 + N)))   # as seen by the owner
        else:
            t, a, b = es[0]
            boundary.append((t, (a, b, b + N, a + N)))
    internal.sort(key=lambda e: (e[0], e[1]))
    tol = 1e-9 * half
    groups = {"inlet": [], "outlet": [], "walls": []}
    for t, f in boundary:
        mx = 0.5 * (nodes[f[0], 0] + nodes[f[1], 0])
        groups["inlet" if mx < -half + tol else "outlet" if mx > half - tol else "walls"].append((t, f))
    faces = [f for _, _, f in internal]
    owner = [t for t, _, _ in internal]
    neighbour = [t1 for _, t1, _ in internal]
    patches = []
    start = len(faces)
    for pname, ptype in (("inlet", "patch"), ("outlet", "patch"), ("walls", "wall")):
        for t, f in groups[pname]:
            faces.append(f)
            owner.append(t)
        patches.append(Patch(pname, ptype, start, len(groups[pname])))
        start += len(groups[pname])
    for t, pv in enumerate(polys):        # back (z = 0), normal -z
        faces.append(tuple(pv[::-1]))
        owner.append(t)
    for t, pv in enumerate(polys):        # front (z = 1), normal +z
        faces.append(tuple(v + N for v in pv))
        owner.append(t)
    patches.append(Patch("frontAndBack", "empty", start, 2 * T))
    face_points = np.array([v for f in faces for v in f], dtype=np.int64)
    face_offsets = np.concatenate([[0], np.cumsum([len(f) for f in faces])]).astype(np.int64)
    cc = np.zeros((T, 3))
    cc[:, :2] = np.array([nodes[list(pv)].mean(axis=0) for pv in polys])
    cc[:, 2] = 0.5
    R = RUNIVERSAL / 28.9647 * 1000
    return Case(name=name, dim=2, points=pts, face_offsets=face_offsets, face_points=face_points,
                owner=np.array(owner, dtype=np.int64), neighbour=np.array(neighbour, dtype=np.int64),
                patches=patches, n_cells=T, cell_centres=cc, Cp=3.5 * R, mol_weight=28.9647, Pr=0.71, Ls=2.0, **kw)


def _prism_mesh(nodes, tris, half, name, **kw) -> Case:
    N = nodes.shape[0]
    T = tris.shape[0]
    pts = np.zeros((2 * N, 3))
    pts[:N, :2] = nodes
    pts[N:, :2] = nodes
    pts[N:, 2] = 1.0
    # edges a->b of each ccw triangle
    ea = tris.ravel()
    eb = np.roll(tris, -1, axis=1).ravel()
    et = np.repeat(np.arange(T), 3)
    lo, hi = np.minimum(ea, eb), np.maximum(ea, eb)
    key = lo * (2 * N) + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    first = np.ones_like(ks, dtype=bool)
    first[1:] = ks[1:] != ks[:-1]
    grp = np.cumsum(first) - 1
    counts = np.bincount(grp)
    # internal edges: groups of two
    g2 = np.nonzero(counts == 2)[0]
    starts = np.nonzero(first)[0]
    e0 = order[starts[g2]]
    e1 = order[starts[g2] + 1]
    t0, t1 = et[e0], et[e1]
    own = np.minimum(t0, t1)
    nei = np.maximum(t0, t1)
    oe = np.where(t0 < t1, e0, e1)     # edge as seen by the owner (ccw in owner)
    A, B = ea[oe], eb[oe]
    fint = np.stack([A, B, B + N, A + N], 1)
    srt = np.lexsort((nei, own))
    fint, own, nei = fint[srt], own[srt], nei[srt]
    # boundary edges
    g1 = np.nonzero(counts == 1)[0]
    eb1 = order[starts[g1]]
    A, B, tb = ea[eb1], eb[eb1], et[eb1]
    fb = np.stack([A, B, B + N, A + N], 1)
    mid = 0.5 * (nodes[A] + nodes[B])
    tol = 1e-9 * half
    groups = [("inlet", "patch", mid[:, 0] < -half + tol), ("outlet", "patch", mid[:, 0] > half - tol)]
    rest = ~(groups[0][2] | groups[1][2])
    groups.append(("walls", "wall", rest))
    faces = [fint]
    owners = [own]
    patches = []
    start = fint.shape[0]
    for pname, ptype, msk in groups:
        faces.append(fb[msk])
        owners.append(tb[msk])
        patches.append(Patch(pname, ptype, start, int(msk.sum())))
        start += int(msk.sum())
    # front/back triangles: back (z=0) normal -z, front normal +z
    back = tris[:, [0, 2, 1]]
    front = tris + N
    fo_quads = np.concatenate(faces).astype(np.int64)
    nq = fo_quads.shape[0]
    face_points = np.concatenate([fo_quads.ravel(), back.ravel(), front.ravel()]).astype(np.int64)
    face_offsets = np.concatenate([np.arange(0, 4 * nq + 1, 4), 4 * nq + 3 * np.arange(1, 2 * T + 1)]).astype(np.int64)
    owner = np.concatenate(owners + [np.arange(T), np.arange(T)]).astype(np.int64)
    patches.append(Patch("frontAndBack", "empty", start, 2 * T))
    cc = np.zeros((T, 3))
    cc[:, :2] = nodes[tris].mean(axis=1)
    cc[:, 2] = 0.5
    R = RUNIVERSAL / 28.9647 * 1000
    return Case(name=name, dim=2, points=pts, face_offsets=face_offsets, face_points=face_points, owner=owner,
                neighbour=nei.astype(np.int64), patches=patches, n_cells=T, cell_centres=cc, Cp=3.5 * R,
                mol_weight=28.9647, Pr=0.71, Ls=2.0, **kw)


def sweep_spec(n_cases: int = 64, seed: int = 20261203, cells_min: float = 16e3, cells_max: float = 1e6):
    """Parameters of a batched sweep: for case k, a quad grid (even k) or a
    jittered triangulation (odd k) with a cell count log-uniform in
    [cells_min, cells_max], Mach U(0.1, 0.6), vortex strength U(1, 5) and the
    M1 or M2 scheme at random. Returns a list of dicts (kind, n, cells, mach,
    beta, solver, seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_cases):
        cells = math.exp(rng.uniform(math.log(cells_min), math.log(cells_max)))
        mach = float(rng.uniform(0.1, 0.6))
        beta = float(rng.uniform(1.0, 5.0))
        solver = int(rng.integers(0, 2))
        sub = int(rng.integers(0, 2 ** 31 - 1))
        if k % 2 == 0:
            n = max(8, int(round(math.sqrt(cells))))
            out.append(dict(kind="quad", n=n, cells=n * n, mach=mach, beta=beta, solver=solver, seed=sub))
        else:
            n = max(8, int(round(math.sqrt(cells / 2))))
            out.append(dict(kind="tri", n=n, cells=2 * n * n, mach=mach, beta=beta, solver=solver, seed=sub))
    return out


def sweep_case(spec: dict) -> Case:
    """The case of one ``sweep_spec`` entry (isentropic vortex on [-10, 10]^2)."""
    if spec["kind"] == "quad":
        return vortex_case(n=spec["n"], mach=spec["mach"], beta=spec["beta"], solver=spec["solver"])
    return tri_case(n=spec["n"], seed=spec["seed"], mach=spec["mach"], beta=spec["beta"], solver=spec["solver"])


# ---------------------------------------------------------------------------
# OpenFOAM case writer
# ---------------------------------------------------------------------------
_BANNER = "/* generated by lfm_public_gb300.cases */\n"


def _header(cls: str, obj: str, location: str = "", binary: bool = False) -> str:
    loc = f'    location    "{location}";\n' if location else ""
    fmt = ('binary;\n    arch        "LSB;label=32;scalar=64";\n' if binary else "ascii;\n")
    return (_BANNER + "FoamFile\n{\n    version     2.0;\n    format      " + fmt +
            f"    class       {cls};\n{loc}    object      {obj};\n}}\n\n")


def _binary_list(f, arr: np.ndarray, n: int) -> None:
    """An OpenFOAM binary list body: the count, then '(' raw bytes ')'
    (little-endian; labels int32, scalars float64)."""
    f.write(f"{n}\n(".encode())
    f.write(np.ascontiguousarray(arr).tobytes())
    f.write(b")\n")


def _fmt(x: float) -> str:
    return repr(float(x))


def write_polymesh_binary(case: Case, d: str) -> None:
    """The polyMesh in OpenFOAM's binary format (points, faceCompactList
    faces, owner and neighbour as raw little-endian arrays)."""
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "points"), "wb") as f:
        f.write(_header("vectorField", "points", "constant/polyMesh", True).encode())
        _binary_list(f, np.asarray(case.points, dtype="<f8"), case.points.shape[0])
    with open(os.path.join(d, "faces"), "wb") as f:
        f.write(_header("faceCompactList", "faces", "constant/polyMesh", True).encode())
        _binary_list(f, np.asarray(case.face_offsets, dtype="<i4"), len(case.face_offsets))
        _binary_list(f, np.asarray(case.face_points, dtype="<i4"), len(case.face_points))
    for name, arr in (("owner", case.owner), ("neighbour", case.neighbour)):
        with open(os.path.join(d, name), "wb") as f:
            f.write(_header("labelList", name, "constant/polyMesh", True).encode())
            _binary_list(f, np.asarray(arr, dtype="<i4"), arr.shape[0])


def write_polymesh(case: Case, d: str, binary: bool = False) -> None:
    os.makedirs(d, exist_ok=True)
    if binary:
        write_polymesh_binary(case, d)
        _write_boundary(case, d)
        return
    with open(os.path.join(d, "points"), "w") as f:
        f.write(_header("vectorField", "points", "constant/polyMesh"))
        f.write(f"{case.points.shape[0]}\n(\n")
        f.write("\n".join(f"({_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])})" for p in case.points))
        f.write("\n)\n")
    with open(os.path.join(d, "faces"), "w") as f:
        f.write(_header("faceList", "faces", "constant/polyMesh"))
        fo, fp = case.face_offsets, case.face_points
        f.write(f"{case.n_faces}\n(\n")
        lines = []
        for i in range(case.n_faces):
            pts = fp[fo[i]:fo[i + 1]]
            lines.append(f"{len(pts)}(" + " ".join(str(int(v)) for v in pts) + ")")
        f.write("\n".join(lines))
        f.write("\n)\n")
    for name, arr in (("owner", case.owner), ("neighbour", case.neighbour)):
        with open(os.path.join(d, name), "w") as f:
            f.write(_header("labelList", name, "constant/polyMesh"))
            f.write(f"{arr.shape[0]}\n(\n" + "\n".join(str(int(v)) for v in arr) + "\n)\n")
    _write_boundary(case, d)


def _write_boundary(case: Case, d: str) -> None:
    with open(os.path.join(d, "boundary"), "w") as f:
        f.write(_header("polyBoundaryMesh", "boundary", "constant/polyMesh"))
        f.write(f"{len(case.patches)}\n(\n")
        for p in case.patches:
            f.write(f"    {p.name}\n    {{\n        type            {p.type};\n")
            if p.neighbour:
                f.write(f"        neighbourPatch  {p.neighbour};\n")
            if p.neighb_proc is not None:
                f.write(f"        myProcNo        {p.my_proc};\n        neighbProcNo    {p.neighb_proc};\n")
            f.write(f"        nFaces          {p.size};\n        startFace       {p.start};\n    }}\n")
        f.write(")\n")


def _boundary_block(case: Case) -> str:
    out = "\n"
    for p in case.patches:
        t = p.type if p.type in ("empty", "cyclic", "processor") else "zeroGradient"
        out += f"    {p.name}\n    {{\n        type            {t};\n    }}\n"
    return out


def write_field(case: Case, d: str, name: str, values: np.ndarray, dims: str, binary: bool = False) -> None:
    vec = values.ndim == 2
    cls = "volVectorField" if vec else "volScalarField"
    if binary:
        with open(os.path.join(d, name), "wb") as f:
            f.write(_header(cls, name, "0", True).encode())
            f.write(f"dimensions      {dims};\n\ninternalField   nonuniform List<{'vector' if vec else 'scalar'}> \n"
                    .encode())
            _binary_list(f, np.asarray(values, dtype="<f8"), values.shape[0])
            f.write(("\n;\n\nboundaryField\n{" + _boundary_block(case) + "}\n").encode())
        return
    with open(os.path.join(d, name), "w") as f:
        f.write(_header(cls, name, "0"))
        f.write(f"dimensions      {dims};\n\n")
        f.write(f"internalField   nonuniform List<{'vector' if vec else 'scalar'}> \n{values.shape[0]}\n(\n")
        if vec:
            f.write("\n".join(f"({_fmt(v[0])} {_fmt(v[1])} {_fmt(v[2])})" for v in values))
        else:
            f.write("\n".join(_fmt(v) for v in values))
        f.write("\n)\n;\n\nboundaryField\n{" + _boundary_block(case) + "}\n")


def write_case(case: Case, root: str, n_steps: Optional[int] = None, write_interval: Optional[int] = None,
               post: Optional[dict] = None, adjust_time_step: bool = False, max_co: float = 0.5,
               binary: bool = False) -> str:
    """Writes ``case`` as an OpenFOAM case directory under ``root``. ``post``
    sets lfm/post entries of controlDict (haveAverage, tStartAverage,
    haveForces, saveForcesStep, printInfoFreq, ...); ``adjust_time_step`` and
    ``max_co`` its adjustTimeStep and maxCo (endTime stays n_steps x deltaT);
    ``binary`` writes the polyMesh and the initial fields in OpenFOAM's binary
    format and sets writeFormat binary."""
    pe = {"haveProbes": "false", "haveSampling": "false", "haveAverage": "false", "haveForces": "false",
          "haveResiduals": "true" if case.residuals else "false", "printInfoFreq": str(case.print_freq),
          "saveResiduals": "false", "saveBlendFactor": "false"}
    for k, v in (post or {}).items():
        pe[k] = ("true" if v else "false") if isinstance(v, bool) else (_fmt(v) if isinstance(v, float) else str(v))
    n_steps = case.n_steps if n_steps is None else n_steps
    wi = n_steps if write_interval is None else write_interval
    os.makedirs(root, exist_ok=True)
    for sub in ("system", "constant", "0"):
        os.makedirs(os.path.join(root, sub), exist_ok=True)
    write_polymesh(case, os.path.join(root, "constant", "polyMesh"), binary=binary)
    z = os.path.join(root, "0")
    write_field(case, z, "p", case.fields["p"], "[1 -1 -2 0 0 0 0]", binary)
    write_field(case, z, "T", case.fields["T"], "[0 0 0 1 0 0 0]", binary)
    write_field(case, z, "U", case.fields["U"], "[0 1 -1 0 0 0 0]", binary)
    if "alpha" in case.fields:
        write_field(case, z, "alpha", case.fields["alpha"], "[0 1 0 0 0 0 0]", binary)
    end = case.delta_t * n_steps
    with open(os.path.join(root, "system", "controlDict"), "w") as f:
        f.write(_header("dictionary", "controlDict", "system"))
        f.write("lfm\n{\n    commType        2;\n    haloCommType    1;\n    doublePrecision true;\n"
                "    post\n    {\n" + "".join(f"        {k:<15} {v};\n" for k, v in pe.items()) + "    }\n}\n\n")
        f.write(f"startFrom       startTime;\nstartTime       0;\nstopAt          endTime;\n"
                f"endTime         {_fmt(end)};\ndeltaT          {_fmt(case.delta_t)};\n"
                f"writeControl    timeStep;\nwriteInterval   {wi};\nwriteFormat     {'binary' if binary else 'ascii'};\n"
                f"writePrecision  {case.write_precision};\ntimeFormat      general;\ntimePrecision   12;\n"
                f"adjustTimeStep  {'yes' if adjust_time_step else 'no'};\nmaxCo           {_fmt(max_co)};\n")
    with open(os.path.join(root, "system", "fvSchemes"), "w") as f:
        f.write(_header("dictionary", "fvSchemes", "system"))
        f.write(f"lfm\n{{\n    solver          {case.solver};\n    dimension       {case.dim};\n"
                f"    rkOrder         {case.rk_order};\n    minmodExists    {'true' if case.minmod else 'false'};\n"
                "    constantTimeStep true;\n}\n")
    with open(os.path.join(root, "constant", "spongeDict"), "w") as f:
        f.write(_header("dictionary", "spongeDict", "constant"))
        f.write(f"Ls      {_fmt(case.Ls)};\nM       {_fmt(case.mach)};\npinf    {_fmt(case.p_inf)};\n"
                f"Tinf    {_fmt(case.T_inf)};\nUinf_x  {_fmt(case.U_inf[0])};\nUinf_y  {_fmt(case.U_inf[1])};\n"
                f"Uinf_z  {_fmt(case.U_inf[2])};\nk       {_fmt(case.k_sponge)};\n")
    with open(os.path.join(root, "constant", "thermophysicalProperties"), "w") as f:
        f.write(_header("dictionary", "thermophysicalProperties", "constant"))
        f.write("mixture\n{\n    specie\n    {\n        nMoles          1;\n"
                f"        molWeight       {_fmt(case.mol_weight)};\n    }}\n    thermodynamics\n    {{\n"
                f"        Cp              {_fmt(case.Cp)};\n        Hf              0;\n    }}\n"
                f"    transport\n    {{\n        mu              {_fmt(case.mu)};\n"
                f"        Pr              {_fmt(case.Pr)};\n    }}\n}}\n")
    with open(os.path.join(root, "constant", "turbulenceProperties"), "w") as f:
        f.write(_header("dictionary", "turbulenceProperties", "constant"))
        f.write("simulationType  " + ("laminar" if case.laminar else "LES") + ";\n")
    return root


def read_result_fields(root: str, names=("rho", "E", "p", "U")):
    """Reads fields (default rho, U, E, p) of the latest time directory written by a run."""
    times = []
    for name in os.listdir(root):
        try:
            t = float(name)
        except ValueError:
            continue
        if t > 0:
            times.append((t, name))
    if not times:
        raise FileNotFoundError(f"no result time directory under {root}")
    tdir = os.path.join(root, max(times)[1])
    out = {}
    for name in names:
        out[name] = _read_internal_field(os.path.join(tdir, name))
    return out


def _read_internal_field(path: str) -> np.ndarray:
    raw = open(path, "rb").read()
    head = raw[:raw.index(b"internalField")].decode(errors="replace")
    if "binary" in head.split("}", 1)[0]:
        # nonuniform List<...> N ( raw little-endian float64 )
        i = raw.index(b"internalField")
        j = raw.index(b"(", i)
        n = int(raw[i:j].split()[-1])
        width = 3 if b"List<vector>" in raw[i:j] else 1
        vals = np.frombuffer(raw[j + 1:j + 1 + 8 * n * width], dtype="<f8").copy()
        return vals.reshape(n, 3) if width == 3 else vals
    txt = raw.decode()
    i = txt.index("internalField")
    rest = txt[i:]
    if "nonuniform" not in rest.split("\n", 1)[0]:
        raise ValueError(f"{path}: expected a nonuniform internalField")
    j = rest.index("(")
    n = int(rest[:j].split()[-1])
    body = rest[j + 1:]
    if body.lstrip().startswith("("):
        vals = np.array(body.replace("(", " ").replace(")", " ").split()[:3 * n], dtype=np.float64)
        return vals.reshape(n, 3)
    return np.array(body.split()[:n], dtype=np.float64)


# ---------------------------------------------------------------------------
# cell renumbering of a polyMesh (what renumberMesh writes)
# ---------------------------------------------------------------------------
def renumber_cells(case: Case, order: np.ndarray) -> Case:
    """The same case with its cells renumbered: new cell i is old cell
    ``order[i]``. Internal faces are flipped where the new owner label would
    exceed the neighbour's (point order reversed, first point kept) and
    sorted upper-triangular; boundary faces keep their patches and order."""
    import copy
    order = np.asarray(order, dtype=np.int64)
    n = case.n_cells
    if sorted(order.tolist()) != list(range(n)):
        raise ValueError("order is not a permutation of the cells")
    inv = np.empty(n, dtype=np.int64)
    inv[order] = np.arange(n)
    n_int = case.neighbour.shape[0]
    fo, fp = case.face_offsets, case.face_points
    own = inv[case.owner]
    nbr = inv[case.neighbour]
    flip = own[:n_int] > nbr
    lo = np.where(flip, nbr, own[:n_int])
    hi = np.where(flip, own[:n_int], nbr)
    perm = np.lexsort((hi, lo))
    faces = [(int(f), bool(flip[f])) for f in perm] + [(f, False) for f in range(n_int, case.n_faces)]
    offs, pts = [0], []
    for f, fl in faces:
        v = fp[fo[f]:fo[f + 1]]
        if fl:
            v = np.concatenate([v[:1], v[1:][::-1]])
        pts.append(v)
        offs.append(offs[-1] + v.size)
    out = copy.copy(case)
    out.face_offsets = np.array(offs, dtype=np.int64)
    out.face_points = np.concatenate(pts).astype(np.int64)
    out.owner = np.concatenate([lo[perm], own[n_int:]]).astype(np.int64)
    out.neighbour = hi[perm].astype(np.int64)
    out.cell_centres = case.cell_centres[order]
    out.fields = {k: v[order] for k, v in case.fields.items()}
    out.name = case.name + ".renumbered"
    return out


# ---------------------------------------------------------------------------
# decomposition into processor partitions (what decomposePar writes)
# ---------------------------------------------------------------------------
def partition_cells(case: Case, nparts: int, method: str = "x", seed: int = 0) -> np.ndarray:
    """Partition of every cell: slabs along x ("x"), contiguous index ranges
    ("index") or a seeded random assignment ("random", many processor faces)."""
    n = case.n_cells
    if method == "x":
        # cells with the same x (to 1e-9) share a partition, so that an
        # extruded case keeps each spanwise column - and its cyclic pair - whole
        xs, inv, counts = np.unique(np.round(case.cell_centres[:, 0], 9), return_inverse=True, return_counts=True)
        first = np.cumsum(counts) - counts
        return (first[inv] * nparts // n).astype(np.int64)
    if method == "index":
        return np.arange(n) * nparts // n
    if method == "random":
        return np.random.default_rng(seed).integers(0, nparts, size=n)
    raise ValueError(f"unknown partition method {method}")


def _write_label_list(path: str, obj: str, values) -> None:
    with open(path, "w") as f:
        f.write(_header("labelList", obj, "constant/polyMesh"))
        f.write(f"{len(values)}\n(\n" + "\n".join(str(int(v)) for v in values) + "\n)\n")


def decompose_case(case: Case, root: str, nparts: int, method: str = "x", seed: int = 0, **kw) -> np.ndarray:
    """Writes ``case`` under ``root`` (dictionaries and the whole mesh) and its
    decomposition into ``root``/processor0..nparts-1, as decomposePar does:
    each partition's cells and points renumbered in global order, its internal
    faces, the original patches restricted to its cells, and one processor
    patch per neighbouring partition (faces in global order on both sides; the
    side that does not own a face globally stores it flipped, with a negative
    faceProcAddressing), plus cell/face/point/boundaryProcAddressing and the
    initial fields. A cyclic pair must join cells of one partition (the "x"
    method keeps spanwise columns whole); processorCyclic patches are not
    written. Returns the partition of every cell."""
    part = partition_cells(case, nparts, method, seed)
    byname = {pt.name: pt for pt in case.patches}
    for pt in case.patches:
        if pt.type != "cyclic":
            continue
        nb = byname[pt.neighbour]
        a = part[case.owner[pt.start:pt.start + pt.size]]
        b = part[case.owner[nb.start:nb.start + nb.size]]
        if not np.array_equal(a, b):
            raise ValueError(f"cyclic patch {pt.name} pairs cells of different partitions "
                             "(processorCyclic patches are not supported)")
    write_case(case, root, **kw)
    fo, fp = case.face_offsets, case.face_points
    owner, nbr = case.owner, case.neighbour
    n_int = nbr.shape[0]
    for p in range(nparts):
        cells = np.nonzero(part == p)[0]
        lcell = np.full(case.n_cells, -1, dtype=np.int64)
        lcell[cells] = np.arange(cells.size)
        faces, flip, fown, fnbr = [], [], [], []
        # internal faces of the partition (global order is upper-triangular and
        # the renumbering is monotone, so the order stays valid)
        inner = np.nonzero((part[owner[:n_int]] == p) & (part[nbr] == p))[0]
        faces += inner.tolist()
        flip += [False] * inner.size
        fown += lcell[owner[inner]].tolist()
        fnbr += lcell[nbr[inner]].tolist()
        patches = []
        bmap = []
        for bi, pt in enumerate(case.patches):
            gf = np.arange(pt.start, pt.start + pt.size)
            gf = gf[part[owner[gf]] == p]
            patches.append(Patch(pt.name, pt.type, len(faces), int(gf.size), neighbour=pt.neighbour))
            bmap.append(bi)
            faces += gf.tolist()
            flip += [False] * gf.size
            fown += lcell[owner[gf]].tolist()
        gi = np.arange(n_int)
        po, pn = part[owner[:n_int]], part[nbr]
        for q in range(nparts):
            if q == p:
                continue
            mine = gi[(po == p) & (pn == q)]
            theirs = gi[(po == q) & (pn == p)]
            gf = np.sort(np.concatenate([mine, theirs]))
            if gf.size == 0:
                continue
            patches.append(Patch(f"procBoundary{p}to{q}", "processor", len(faces), int(gf.size), my_proc=p,
                                 neighb_proc=q))
            bmap.append(-1)
            own_side = po[gf] == p
            faces += gf.tolist()
            flip += (~own_side).tolist()
            fown += np.where(own_side, lcell[owner[gf]], lcell[nbr[gf]]).tolist()
        # points in global order
        used = np.unique(np.concatenate([fp[fo[f]:fo[f + 1]] for f in faces]))
        lpt = np.full(case.points.shape[0], -1, dtype=np.int64)
        lpt[used] = np.arange(used.size)
        offs, pts = [0], []
        for f, fl in zip(faces, flip):
            v = fp[fo[f]:fo[f + 1]]
            if fl:   # reversed orientation, first point kept (OpenFOAM's face::reverseFace)
                v = np.concatenate([v[:1], v[1:][::-1]])
            pts.append(lpt[v])
            offs.append(offs[-1] + v.size)
        local = Case(name=f"{case.name}.p{p}", dim=case.dim, points=case.points[used],
                     face_offsets=np.array(offs, dtype=np.int64), face_points=np.concatenate(pts).astype(np.int64),
                     owner=np.array(fown, dtype=np.int64), neighbour=np.array(fnbr, dtype=np.int64), patches=patches,
                     n_cells=int(cells.size), cell_centres=case.cell_centres[cells])
        pdir = os.path.join(root, f"processor{p}")
        mesh = os.path.join(pdir, "constant", "polyMesh")
        write_polymesh(local, mesh)
        _write_label_list(os.path.join(mesh, "cellProcAddressing"), "cellProcAddressing", cells)
        fpa = [(-(f + 1) if fl else (f + 1)) for f, fl in zip(faces, flip)]
        _write_label_list(os.path.join(mesh, "faceProcAddressing"), "faceProcAddressing", fpa)
        _write_label_list(os.path.join(mesh, "pointProcAddressing"), "pointProcAddressing", used)
        _write_label_list(os.path.join(mesh, "boundaryProcAddressing"), "boundaryProcAddressing", bmap)
        z = os.path.join(pdir, "0")
        os.makedirs(z, exist_ok=True)
        write_field(local, z, "p", case.fields["p"][cells], "[1 -1 -2 0 0 0 0]")
        write_field(local, z, "T", case.fields["T"][cells], "[0 0 0 1 0 0 0]")
        write_field(local, z, "U", case.fields["U"][cells], "[0 1 -1 0 0 0 0]")
        if "alpha" in case.fields:
            write_field(local, z, "alpha", case.fields["alpha"][cells], "[0 1 0 0 0 0 0]")
    return part
