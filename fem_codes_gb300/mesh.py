"""Synthetic structured triangle meshes and problem coefficients.

The mesh topology is the reference's structured generator with the diagonal
leaning right (Gerador_de_Malhas/Structured_Mesh/geraMalha.c:113-138): nodes
numbered row by row, x fastest; cell (i, j) with corners a=(i,j), b=(i+1,j),
c=(i+1,j+1), d=(i,j+1) is split into elements (a, b, c) and (a, c, d), stored
cell by cell.  Coordinates are x = i/nx * Lx so that boundary nodes land
exactly on 0 and Lx (the reference classifies boundaries with exact
comparisons, Preprocess.c:112-123).  Interior nodes may be perturbed by a
seeded uniform offset in [-frac*h, +frac*h] per coordinate.

Node ``Type`` follows the reference's mesh format (Preprocess.c:73-81):
``Type >= 1`` is an unknown, ``Type == 0`` a prescribed (Dirichlet) node.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Velocity of the skew-advection problem: (cos 30deg, sin 30deg).  sin 30deg is
# written as the exact 0.5.
SKEW_BETA = (0.86602540378443865, 0.5)


@dataclasses.dataclass
class Mesh:
    nx: int
    ny: int
    x: np.ndarray          # float64 [nnodes]
    y: np.ndarray          # float64 [nnodes]
    vert: np.ndarray       # int32 [nel, 3]

    @property
    def nnodes(self) -> int:
        return int(self.x.shape[0])

    @property
    def nel(self) -> int:
        return int(self.vert.shape[0])


def structured_mesh(nx: int, ny: int, lx: float = 1.0, ly: float = 1.0,
                    perturb: float = 0.0, seed: int = 1234) -> Mesh:
    """Structured nx-by-ny cell mesh of 2*nx*ny linear triangles."""
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = (ii.astype(np.float64) / nx) * lx
    y = (jj.astype(np.float64) / ny) * ly
    x = x.reshape(-1).copy()
    y = y.reshape(-1).copy()
    if perturb > 0.0:
        rng = np.random.default_rng(seed)
        hx, hy = lx / nx, ly / ny
        dx = rng.uniform(-perturb * hx, perturb * hx, size=x.shape)
        dy = rng.uniform(-perturb * hy, perturb * hy, size=y.shape)
        interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
        interior = interior.reshape(-1)
        x[interior] += dx[interior]
        y[interior] += dy[interior]
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    a = (cj * (nx + 1) + ci).reshape(-1)
    b = a + 1
    c = b + (nx + 1)
    d = a + (nx + 1)
    vert = np.empty((2 * nx * ny, 3), dtype=np.int32)
    vert[0::2] = np.stack([a, b, c], axis=1)
    vert[1::2] = np.stack([a, c, d], axis=1)
    return Mesh(nx, ny, x, y, vert)


@dataclasses.dataclass
class TransportProblem:
    """Coefficients of a steady scalar transport problem, evaluated the way the
    reference's Build_K_F_SUPG.c:61-84 evaluates its plug-in callbacks:
    velocity at the element centroid, source at each vertex, prescribed value
    at each node."""
    name: str
    k: float                 # conductivity (kx == ky)
    gamma: float             # reaction
    node_type: np.ndarray    # int32 [nnodes]
    beta: np.ndarray         # float64 [nel, 2]
    fsrc: np.ndarray         # float64 [nel, 3]
    upresc: np.ndarray       # float64 [nnodes]


def skew_problem(mesh: Mesh, k: float = 1e-4) -> TransportProblem:
    """Skew advection-diffusion on the unit square: beta = (cos30, sin30),
    f = 0, gamma = 0; nodes on x = 0 or y = 0 prescribed, u = 1 on x = 0 for
    y > 0.3 and 0 elsewhere on that inflow boundary."""
    presc = (mesh.x == 0.0) | (mesh.y == 0.0)
    node_type = np.where(presc, 0, 1).astype(np.int32)
    beta = np.empty((mesh.nel, 2), dtype=np.float64)
    beta[:, 0] = SKEW_BETA[0]
    beta[:, 1] = SKEW_BETA[1]
    fsrc = np.zeros((mesh.nel, 3), dtype=np.float64)
    upresc = np.where((mesh.x == 0.0) & (mesh.y > 0.3), 1.0, 0.0)
    return TransportProblem("SKEW", k, 0.0, node_type, beta, fsrc, upresc)


def rotated_problem(mesh: Mesh, angle: float, k: float, seed: int = 0) -> TransportProblem:
    """Constant-velocity transport at an arbitrary angle (used for the learned
    preconditioner's training distribution): inflow edges prescribed by the
    sign of beta.n, unit value on the left half of the inflow."""
    bx, by = math.cos(angle), math.sin(angle)
    inflow = np.zeros(mesh.nnodes, dtype=bool)
    if bx > 0:
        inflow |= mesh.x == 0.0
    if bx < 0:
        inflow |= mesh.x == mesh.x.max()
    if by > 0:
        inflow |= mesh.y == 0.0
    if by < 0:
        inflow |= mesh.y == mesh.y.max()
    node_type = np.where(inflow, 0, 1).astype(np.int32)
    beta = np.empty((mesh.nel, 2), dtype=np.float64)
    beta[:, 0] = bx
    beta[:, 1] = by
    fsrc = np.zeros((mesh.nel, 3), dtype=np.float64)
    s = mesh.x + mesh.y
    upresc = np.where(inflow & (s > 0.3 * s.max()), 1.0, 0.0)
    return TransportProblem("ROT", k, 0.0, node_type, beta, fsrc, upresc)


def element_types(mesh: Mesh) -> np.ndarray:
    """Element boundary class of Preprocess.c:108-152 (1..4 edge on x=0, y=0,
    x=1, y=1; 5..8 corners; -1 interior)."""
    v = mesh.vert
    c1 = (mesh.x[v] == 0.0).sum(1)
    c2 = (mesh.y[v] == 0.0).sum(1)
    c3 = (mesh.x[v] == 1.0).sum(1)
    c4 = (mesh.y[v] == 1.0).sum(1)
    t = np.full(mesh.nel, -1, dtype=np.int32)
    # Evaluate in reverse priority so that earlier branches win.
    t[c4 == 2] = 4
    t[c3 == 2] = np.where((c3 == c4)[c3 == 2], 7, 3)
    t[c2 == 2] = np.where((c2 == c3)[c2 == 2], 6, 2)
    m1 = c1 == 2
    t[m1] = np.where((c1 == c2)[m1], 5, np.where((c1 == c4)[m1], 8, 1))
    return t


@dataclasses.dataclass
class EulerProblem:
    """A 2D Euler problem on a mesh: equation numbering node_id [nnodes, 4]
    (-1 prescribed; Fill_ID.c:3-39 numbers node by node, dof by dof), the
    prescribed conservative values upresc [nnodes, 4] (rho, rho u, rho v,
    rho E), the initial solution u0 [neq+1] and gamma."""
    name: str
    node_id: np.ndarray
    neq: int
    upresc: np.ndarray
    u0: np.ndarray
    gamma: float


def refletido_problem(mesh: Mesh) -> EulerProblem:
    """Reflected oblique shock (03_Euler_Equations/2D/REFLETIDO): inflow x = 0
    with (1, 2.9, 0, 5.990715) and top y = ymax with (1.7, 4.452878,
    -0.860744, 9.870181681) fully prescribed, rho v = 0 on the bottom wall
    y = 0, free outflow; initial state the inflow state
    (REFLETIDO_InitialSolution.c, REFLETIDO_*presc.c: the left boundary
    wins at shared corners)."""
    x, y = mesh.x, mesh.y
    left = np.abs(x) <= 1e-15
    top = y == y.max()
    bottom = np.abs(y) <= 1e-15
    presc = np.zeros((mesh.nnodes, 4), dtype=bool)
    presc[left | top, :] = True
    presc[bottom, 2] = True
    node_id = np.full((mesh.nnodes, 4), -1, np.int32)
    neq = int((~presc).sum())
    node_id[~presc] = np.arange(neq, dtype=np.int32)
    upresc = np.empty((mesh.nnodes, 4))
    upresc[:, 0] = np.where(left, 1.0, 1.7)
    upresc[:, 1] = np.where(left, 2.9, 4.452878)
    upresc[:, 2] = np.where(left | bottom, 0.0, -0.860744)
    upresc[:, 3] = np.where(left, 5.990715, 9.870181681)
    init = np.array([1.0, 2.9, 0.0, 5.990715])
    u0 = np.zeros(neq + 1)
    free = node_id >= 0
    u0[node_id[free]] = np.broadcast_to(init, node_id.shape)[free]
    return EulerProblem("REFLETIDO", node_id, neq, upresc, u0, 1.4)


def euler_cfl_dt(mesh: Mesh, cfl: float = 5.0, speed: float = 2.9, sound: float = 1.0) -> float:
    """Time step from a CFL number, dt = CFL * h / (|v| + c), h the smaller
    cell size (the reference's decks give dt directly)."""
    h = min(float(mesh.x.max() - mesh.x.min()) / mesh.nx, float(mesh.y.max() - mesh.y.min()) / mesh.ny)
    return cfl * h / (speed + sound)


@dataclasses.dataclass
class NSProblem:
    """A steady incompressible Navier-Stokes problem: numbering node_id
    [nnodes, 3] (u, v, p; -1 prescribed; Fill_ID.c numbers node by node),
    prescribed values upresc [nnodes, 3], nodal body force f [nnodes, 2],
    Reynolds number and the reference velocity of the local Reynolds number."""
    name: str
    node_id: np.ndarray
    neq: int
    upresc: np.ndarray
    f: np.ndarray
    re: float
    velmax: float


def cavity_lid(x: float, y: float) -> float:
    """CAVITY_v1presc.c: u = 1 on the lid y = 1 with cosine ramps over
    x < 0.1 and x > 0.9, 0 elsewhere (evaluated with the C library's cos)."""
    pi, eps1 = 3.14159265359, 0.1
    eps2 = 1.0 - eps1
    if abs(y - 1.0) <= 1e-15:
        if x < eps1:
            c = 1 - math.cos((eps1 - x) * pi / eps1)
            return 1.0 - 0.25 * c * c
        if x > eps2:
            c = 1 - math.cos((x - eps2) * pi / eps1)
            return 1.0 - 0.25 * c * c
        return 1.0
    return 0.0


def cavity_problem(mesh: Mesh, re: float = 1000.0, lid: str = "smooth") -> NSProblem:
    """Lid-driven cavity on the unit square: velocity prescribed on the whole
    boundary (the lid by CAVITY_v1presc.c, or u = 1 on the whole lid with
    lid="unit"), pressure pinned to 0 at node 0 (the corner x = y = 0)."""
    x, y = mesh.x, mesh.y
    bnd = (x == x.min()) | (x == x.max()) | (y == y.min()) | (y == y.max())
    presc = np.zeros((mesh.nnodes, 3), dtype=bool)
    presc[bnd, 0:2] = True
    presc[0, 2] = True
    node_id = np.full((mesh.nnodes, 3), -1, np.int32)
    neq = int((~presc).sum())
    node_id[~presc] = np.arange(neq, dtype=np.int32)
    upresc = np.zeros((mesh.nnodes, 3))
    if lid == "unit":
        upresc[:, 0] = np.where(np.abs(y - 1.0) <= 1e-15, 1.0, 0.0)
    else:
        upresc[:, 0] = [cavity_lid(float(a), float(b)) for a, b in zip(x, y)]
    return NSProblem("CAVITY", node_id, neq, upresc, np.zeros((mesh.nnodes, 2)), float(re), 1.0)
