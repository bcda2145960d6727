"""FP64 CPU restatement of eQ's trap-layer field step (the oracle).

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module; only
tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it, and
only as the checker / the timed CPU baseline.

What it restates, element by element:

* Mesh: ``RectangleMesh(p0, p1, nx, ny, "right")`` (src/fHSL.cpp:164-172).  Vertex
  (i, j) sits at (j*W/nx, i*H/ny) with natural index k = j + i*(nx+1); each square
  splits into the triangles (v0, v1, v3) and (v0, v2, v3) with v0 = k, v1 = k+1,
  v2 = k+nx+1, v3 = k+nx+2, i.e. the diagonal runs (i, j)-(i+1, j+1).
* Bilinear form ``a`` of fenics/hslD.ufl:31-49, as tabulated by the generated cell
  kernel fenics/hslD.h:3103-3262: consistent P1 mass (|J|/12 diagonal, |J|/24 off
  diagonal) plus dt * (A grad u) . grad v with A = D*[[D11, D12], [D12, D22]], the
  nodal tensor fields interpolated at the 3-point degree-2 rule.
* Robin facet terms dt*r*(u - s)*v on ds(1)/ds(2) (fenics/hslD.h:3264-3445 and
  3534-3693): facet mass |e|/3, |e|/6 and load |e|/2.
* Linear form ``L`` = (u0 + dt*f) v (fenics/hslD.h:3446-3533); f = 0 in the
  reference (src/fHSL.h:201), so b = M u0.
* Dirichlet rows: identity with the wall value (DOLFIN DirichletBC.apply) on the
  walls selected by the trap type (src/fHSL.h:456-504, src/fHSL.cpp:557-569).
* Boundary flux functional -grad(u).n ds (fenics/boundary.ufl:9-12) scaled by
  D*dt into ``totalBoundaryFlux`` (src/fHSL.cpp:156-160).

Extensions required by the synthetic workloads, with no form in the reference:

* reaction -g*c, implicit: the mass block is scaled by (1 + dt*g);
* point cells: load dt * sum_i s_i * phi(x_i) on the containing triangle
  (barycentric), and gather c(x_i) = sum_j phi_j(x_i) c_j;
* Galerkin advection dt * (v . grad u) * w (the non-conservative, SUPG-free form
  of fenics/AdvectionDiffusion.ufl:62, extended to 2D with a P1 velocity).

The solve is a sparse direct LU (scipy SuperLU), FP64, like DOLFIN's default
LinearVariationalSolver path.  Parity is unpinned by the reference's own tests
(it has none); it is pinned instead by the reference's own element kernels
compiled from fenics/hslD.h (see ``oracle/ref_kernels.py``) and by analytic
known answers in the tests.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

WALL_BOTTOM, WALL_TOP, WALL_LEFT, WALL_RIGHT = 1, 2, 4, 8

# 3-point degree-2 rule on the reference triangle, as in fenics/hslD.h:3152-3157:
# weights 1/6 each; P1 basis values at the points.
_QW = np.array([1.0 / 6.0] * 3)
_QPHI = np.array([[2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0],
                  [1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0],
                  [1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0]])


class RightMesh:
    """Structured triangulation of [0, W] x [0, H] with nx x ny squares.

    diagonal "right" (the reference's RectangleMesh(..., "right"), src/fHSL.cpp:171)
    cuts each square along (i, j)-(i+1, j+1); "left" along (i, j+1)-(i+1, j).  The
    direction comes from DOLFIN, which is not part of the reference tree, so it is a
    switch here; "right" is what the GPU library implements.
    """

    def __init__(self, W: float, H: float, nx: int, ny: int, diagonal: str = "right"):
        if diagonal not in ("right", "left"):
            raise ValueError(diagonal)
        self.W, self.H, self.nx, self.ny = float(W), float(H), int(nx), int(ny)
        self.diagonal = diagonal
        self.hx, self.hy = self.W / nx, self.H / ny
        jj, ii = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1))
        self.coords = np.stack([jj.ravel() * self.hx, ii.ravel() * self.hy], axis=1)
        sj, si = np.meshgrid(np.arange(nx), np.arange(ny))
        v0 = (sj + si * (nx + 1)).ravel()
        v1, v2, v3 = v0 + 1, v0 + nx + 1, v0 + nx + 2
        self.cells = np.empty((2 * nx * ny, 3), dtype=np.int64)
        if diagonal == "right":
            # per square: lower-right (v0, v1, v3), then upper-left (v0, v2, v3)
            self.cells[0::2] = np.stack([v0, v1, v3], axis=1)
            self.cells[1::2] = np.stack([v0, v2, v3], axis=1)
        else:
            # per square: lower-left (v0, v1, v2), then upper-right (v1, v2, v3)
            self.cells[0::2] = np.stack([v0, v1, v2], axis=1)
            self.cells[1::2] = np.stack([v1, v2, v3], axis=1)

    @property
    def n_nodes(self) -> int:
        return (self.nx + 1) * (self.ny + 1)

    def wall_nodes(self, walls: int) -> np.ndarray:
        i = np.arange(self.n_nodes) // (self.nx + 1)
        j = np.arange(self.n_nodes) % (self.nx + 1)
        m = np.zeros(self.n_nodes, dtype=bool)
        if walls & WALL_BOTTOM:
            m |= i == 0
        if walls & WALL_TOP:
            m |= i == self.ny
        if walls & WALL_LEFT:
            m |= j == 0
        if walls & WALL_RIGHT:
            m |= j == self.nx
        return m


def _geometry(mesh: RightMesh):
    """Per-triangle Jacobian pieces in the order fenics/hslD.h:3158-3169 uses them."""
    return _geometry_of(mesh.coords[mesh.cells])


def _geometry_of(c: np.ndarray):
    """Same for explicit triangles c (T, 3, 2)."""
    J_c0 = c[:, 1, 0] - c[:, 0, 0]
    J_c1 = c[:, 2, 0] - c[:, 0, 0]
    J_c2 = c[:, 1, 1] - c[:, 0, 1]
    J_c3 = c[:, 2, 1] - c[:, 0, 1]
    detJ = J_c0 * J_c3 - J_c1 * J_c2
    # K = J^{-1}; reference gradients of P1: dphi/dX = [-1, 1, 0], dphi/dY = [-1, 0, 1]
    K00, K01 = J_c3 / detJ, -J_c1 / detJ
    K10, K11 = -J_c2 / detJ, J_c0 / detJ
    dX = np.array([-1.0, 1.0, 0.0])
    dY = np.array([-1.0, 0.0, 1.0])
    gx = K00[:, None] * dX[None, :] + K10[:, None] * dY[None, :]  # d phi_a / dx
    gy = K01[:, None] * dX[None, :] + K11[:, None] * dY[None, :]  # d phi_a / dy
    return detJ, np.abs(detJ), gx, gy


def tabulate_a(mesh: RightMesh, D: float, dt: float, D11=None, D22=None, D12=None,
               mass_scale: float = 1.0) -> np.ndarray:
    """Element matrices of hslD's cell integral (fenics/hslD.h:3123-3262), (T, 3, 3).

    ``mass_scale`` multiplies the mass block (1 + dt*g for the reaction extension);
    at 1.0 this is exactly the reference's form.
    """
    n = mesh.n_nodes
    D11 = np.ones(n) if D11 is None else np.asarray(D11, dtype=np.float64)
    D22 = np.ones(n) if D22 is None else np.asarray(D22, dtype=np.float64)
    D12 = np.zeros(n) if D12 is None else np.asarray(D12, dtype=np.float64)
    _, adet, gx, gy = _geometry(mesh)
    cells = mesh.cells
    # tensor coefficients interpolated at the 3 quadrature points, weighted
    t11 = np.einsum('q,qc,tc->t', _QW, _QPHI, D11[cells])
    t22 = np.einsum('q,qc,tc->t', _QW, _QPHI, D22[cells])
    t12 = np.einsum('q,qc,tc->t', _QW, _QPHI, D12[cells])
    stiff = (t11[:, None, None] * gx[:, :, None] * gx[:, None, :]
             + t22[:, None, None] * gy[:, :, None] * gy[:, None, :]
             + t12[:, None, None] * (gx[:, :, None] * gy[:, None, :]
                                     + gy[:, :, None] * gx[:, None, :]))
    stiff *= D * dt * adet[:, None, None]
    mass = np.array([[2.0, 1.0, 1.0], [1.0, 2.0, 1.0], [1.0, 1.0, 2.0]]) / 24.0
    return stiff + mass_scale * adet[:, None, None] * mass[None, :, :]


def tabulate_mass(mesh: RightMesh) -> np.ndarray:
    """Element mass matrices: the u0*v part of hslD's linear form (hslD.h:3466-3533)."""
    _, adet, _, _ = _geometry(mesh)
    mass = np.array([[2.0, 1.0, 1.0], [1.0, 2.0, 1.0], [1.0, 1.0, 2.0]]) / 24.0
    return adet[:, None, None] * mass[None, :, :]


def tabulate_advection(mesh: RightMesh, dt: float, vx: np.ndarray, vy: np.ndarray) -> np.ndarray:
    """Galerkin advection dt * int (v . grad phi_b) phi_a, (T, 3, 3); v is P1 nodal."""
    _, adet, gx, gy = _geometry(mesh)
    cells = mesh.cells
    vxq = np.einsum('qc,tc->tq', _QPHI, vx[cells])  # velocity at quadrature points
    vyq = np.einsum('qc,tc->tq', _QPHI, vy[cells])
    # sum_q w_q phi_a(q) (v(q) . grad phi_b)
    conv = (np.einsum('q,qa,tq,tb->tab', _QW, _QPHI, vxq, gx)
            + np.einsum('q,qa,tq,tb->tab', _QW, _QPHI, vyq, gy))
    return dt * adet[:, None, None] * conv


# --- single-element tensors (the unit the reference's generated kernels compute) ---
_MASS_REF = np.array([[2.0, 1.0, 1.0], [1.0, 2.0, 1.0], [1.0, 1.0, 2.0]]) / 24.0


def element_a(coords, D11, D22, D12, D, dt) -> np.ndarray:
    """Bilinear cell tensor of hslD on one triangle (cf. fenics/hslD.h:3123-3262)."""
    c = np.asarray(coords, dtype=np.float64).reshape(1, 3, 2)
    _, adet, gx, gy = _geometry_of(c)
    t = [float(np.einsum('q,qc,c->', _QW, _QPHI, np.asarray(v, dtype=np.float64)))
         for v in (D11, D22, D12)]
    stiff = (t[0] * np.outer(gx[0], gx[0]) + t[1] * np.outer(gy[0], gy[0])
             + t[2] * (np.outer(gx[0], gy[0]) + np.outer(gy[0], gx[0])))
    return D * dt * adet[0] * stiff + adet[0] * _MASS_REF


def element_L(coords, u0, dt, f) -> np.ndarray:
    """Linear cell tensor (u0 + dt f) v on one triangle (cf. fenics/hslD.h:3446-3533)."""
    c = np.asarray(coords, dtype=np.float64).reshape(1, 3, 2)
    _, adet, _, _ = _geometry_of(c)
    return adet[0] * _MASS_REF @ np.asarray(u0, dtype=np.float64) + dt * f * adet[0] / 6.0


def _facet_vertices(facet: int):
    """Local vertices of facet `facet` (the edge opposite vertex `facet`)."""
    return [v for v in range(3) if v != facet]


def facet_a(coords, facet, dt, r) -> np.ndarray:
    """Robin facet tensor dt r u v on one exterior facet (cf. fenics/hslD.h:3264-3445)."""
    c = np.asarray(coords, dtype=np.float64)
    a, b = _facet_vertices(facet)
    L = float(np.hypot(*(c[b] - c[a])))
    A = np.zeros((3, 3))
    A[np.ix_([a, b], [a, b])] = dt * r * L * np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]])
    return A


def facet_L(coords, facet, dt, r, s) -> np.ndarray:
    """Robin facet load dt r s v (cf. fenics/hslD.h:3534-3693)."""
    c = np.asarray(coords, dtype=np.float64)
    a, b = _facet_vertices(facet)
    L = float(np.hypot(*(c[b] - c[a])))
    out = np.zeros(3)
    out[[a, b]] = dt * r * s * L / 2.0
    return out


def facet_flux(coords, u, facet) -> float:
    """-grad(u).n |e| of a P1 field on one exterior facet (cf. fenics/boundary.ufl:11)."""
    c = np.asarray(coords, dtype=np.float64).reshape(1, 3, 2)
    _, _, gx, gy = _geometry_of(c)
    u = np.asarray(u, dtype=np.float64)
    grad = np.array([gx[0] @ u, gy[0] @ u])
    a, b = _facet_vertices(facet)
    e = c[0, b] - c[0, a]
    L = float(np.hypot(*e))
    n = np.array([e[1], -e[0]]) / L
    # outward: away from the opposite vertex
    if np.dot(n, c[0, facet] - c[0, a]) > 0:
        n = -n
    return float(-np.dot(grad, n) * L)


def robin_facets(mesh: RightMesh, wall: int):
    """Boundary edges (node pairs) of one wall and their lengths."""
    nx, ny = mesh.nx, mesh.ny
    if wall == WALL_BOTTOM:
        a = np.arange(nx); e = np.stack([a, a + 1], 1); L = mesh.hx
    elif wall == WALL_TOP:
        a = ny * (nx + 1) + np.arange(nx); e = np.stack([a, a + 1], 1); L = mesh.hx
    elif wall == WALL_LEFT:
        a = np.arange(ny) * (nx + 1); e = np.stack([a, a + nx + 1], 1); L = mesh.hy
    else:
        a = np.arange(ny) * (nx + 1) + nx; e = np.stack([a, a + nx + 1], 1); L = mesh.hy
    return e, L


def _assemble(mesh: RightMesh, Ae: np.ndarray) -> sp.csr_matrix:
    rows = np.repeat(mesh.cells, 3, axis=1).ravel()
    cols = np.tile(mesh.cells, (1, 3)).ravel()
    n = mesh.n_nodes
    return sp.coo_matrix((Ae.ravel(), (rows, cols)), shape=(n, n)).tocsr()


def point_weights(mesh: RightMesh, xy: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Containing triangle of each point and its P1 barycentric weights.

    Returns (nodes (n, 3) int64, weights (n, 3)).  Points on the square diagonal
    belong to the lower-right triangle; points on the far walls to the last square.
    """
    xy = np.asarray(xy, dtype=np.float64).reshape(-1, 2)
    nx, ny = mesh.nx, mesh.ny
    X = xy[:, 0] / mesh.hx
    Y = xy[:, 1] / mesh.hy
    j = np.clip(np.floor(X).astype(np.int64), 0, nx - 1)
    i = np.clip(np.floor(Y).astype(np.int64), 0, ny - 1)
    xi = X - j
    eta = Y - i
    v0 = j + i * (nx + 1)
    nodes = np.empty((len(xy), 3), dtype=np.int64)
    w = np.empty((len(xy), 3))
    if getattr(mesh, "diagonal", "right") == "left":
        # lower-left (v0, v1, v2) where xi + eta <= 1, else upper-right (v1, v2, v3)
        low = xi + eta <= 1.0
        nodes[:, 0] = np.where(low, v0, v0 + 1)
        nodes[:, 1] = np.where(low, v0 + 1, v0 + nx + 1)
        nodes[:, 2] = np.where(low, v0 + nx + 1, v0 + nx + 2)
        w[:, 0] = np.where(low, 1.0 - xi - eta, 1.0 - eta)
        w[:, 1] = np.where(low, xi, 1.0 - xi)
        w[:, 2] = np.where(low, eta, xi + eta - 1.0)
        return nodes, w
    lower = xi >= eta
    nodes[:, 0] = v0
    nodes[:, 1] = np.where(lower, v0 + 1, v0 + nx + 1)
    nodes[:, 2] = v0 + nx + 2
    w[:, 0] = np.where(lower, 1.0 - xi, 1.0 - eta)
    w[:, 1] = np.where(lower, xi - eta, eta - xi)
    w[:, 2] = np.where(lower, eta, xi)
    return nodes, w


def point_load(mesh: RightMesh, xy: np.ndarray, s: np.ndarray, scale: float = 1.0) -> np.ndarray:
    """Nodal load scale * sum_i s_i phi(x_i), summed in cell order."""
    nodes, w = point_weights(mesh, xy)
    F = np.zeros(mesh.n_nodes)
    np.add.at(F, nodes.ravel(), (w * (scale * np.asarray(s))[:, None]).ravel())
    return F


def gather(mesh: RightMesh, u: np.ndarray, xy: np.ndarray) -> np.ndarray:
    nodes, w = point_weights(mesh, xy)
    return np.sum(u[nodes] * w, axis=1)


def boundary_flux_integral(mesh: RightMesh, u: np.ndarray) -> float:
    """-int_{dOmega} grad(u).n ds for P1 u (fenics/boundary.ufl:11).

    Each boundary edge takes the gradient of the one triangle it bounds: bottom
    edges the lower-right triangle (v0, v1, v3), top edges the upper-left one
    (v0, v2, v3), left edges the upper-left one, right edges the lower-right one.
    """
    nx, ny = mesh.nx, mesh.ny
    hx, hy = mesh.hx, mesh.hy
    U = u.reshape(ny + 1, nx + 1)
    if getattr(mesh, "diagonal", "right") == "left":
        # bottom and left edges bound the lower-left triangle (v0, v1, v2), top and
        # right edges the upper-right one (v1, v2, v3)
        fb = np.sum((U[1, :-1] - U[0, :-1]) / hy) * hx
        ft = np.sum(-(U[ny, 1:] - U[ny - 1, 1:]) / hy) * hx
        fl = np.sum((U[:-1, 1] - U[:-1, 0]) / hx) * hy
        fr = np.sum(-(U[1:, nx] - U[1:, nx - 1]) / hx) * hy
        return float(fb + ft + fl + fr)
    # bottom (n = (0,-1)): -du/dy on triangle (v0,v1,v3) = (u3 - u1)/hy
    fb = np.sum((U[1, 1:] - U[0, 1:]) / hy) * hx
    # top (n = (0,1)): -du/dy on (v0,v2,v3) = -(u2 - u0)/hy, u2 = U[ny, j], u0 = U[ny-1, j]
    ft = np.sum(-(U[ny, :-1] - U[ny - 1, :-1]) / hy) * hx
    # left (n = (-1,0)): du/dx on (v0,v2,v3) = (u3 - u2)/hx with u2 = U[i+1,0], u3 = U[i+1,1]
    fl = np.sum((U[1:, 1] - U[1:, 0]) / hx) * hy
    # right (n = (1,0)): -du/dx on (v0,v1,v3) = -(u1 - u0)/hx with u1 = U[i,nx], u0 = U[i,nx-1]
    fr = np.sum(-(U[:-1, nx] - U[:-1, nx - 1]) / hx) * hy
    return float(fb + ft + fl + fr)


class HsldOracle:
    """Backward-Euler step of one species on one trap, FP64 direct solve.

    System: (alpha*M + dt*D*K(tensor) + dt*C(v) + R) u^{n+1} = M u^n + F + r
    with alpha = 1 + dt*g; Dirichlet rows replaced by identity and value 0.
    With g = 0, no advection and F folded into u^n this is exactly the reference
    step u0 <- solution_vector; LVS->solve() (src/fHSL.cpp:104-108).
    """

    def __init__(self, W, H, nx, ny, D, dt, g=0.0, walls=WALL_BOTTOM, D11=None, D22=None,
                 D12=None, velocity=None, robin=None, factor=True, diagonal="right"):
        self.mesh = RightMesh(W, H, nx, ny, diagonal)
        self.D, self.dt, self.g, self.walls = float(D), float(dt), float(g), int(walls)
        m = self.mesh
        Ae = tabulate_a(m, self.D, self.dt, D11, D22, D12, mass_scale=1.0 + self.dt * self.g)
        if velocity is not None:
            vx, vy = velocity(m.coords[:, 0], m.coords[:, 1])
            Ae = Ae + tabulate_advection(m, self.dt, np.broadcast_to(vx, (m.n_nodes,)).astype(float),
                                         np.broadcast_to(vy, (m.n_nodes,)).astype(float))
        A = _assemble(m, Ae)
        self.robin_load = np.zeros(m.n_nodes)
        if robin:
            # robin = {wall_bit: (rate, external_value)}: dt*r*(u - s)*v on that wall
            Rr, Rc, Rv = [], [], []
            for wall, (r, s) in robin.items():
                e, L = robin_facets(m, wall)
                fm = self.dt * r * L * np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]])
                for a in range(2):
                    for b in range(2):
                        Rr.append(e[:, a]); Rc.append(e[:, b])
                        Rv.append(np.full(len(e), fm[a, b]))
                np.add.at(self.robin_load, e.ravel(), self.dt * r * s * L / 2.0)
            A = A + sp.coo_matrix((np.concatenate(Rv), (np.concatenate(Rr), np.concatenate(Rc))),
                                  shape=A.shape).tocsr()
        self.M = _assemble(m, tabulate_mass(m))
        self.A_full = A  # before the Dirichlet rows are replaced (for the balance)
        self.dir = m.wall_nodes(self.walls)
        # DirichletBC.apply: zero the row, unit diagonal, rhs = wall value (0)
        Dm = sp.diags((~self.dir).astype(np.float64))
        A = (Dm @ A + sp.diags(self.dir.astype(np.float64))).tocsc()
        self.A = A
        self.lu = spla.splu(A) if factor else None

    def rhs(self, u: np.ndarray, F: Optional[np.ndarray] = None,
            dvals: Optional[np.ndarray] = None) -> np.ndarray:
        b = self.M @ u + self.robin_load
        if F is not None:
            b = b + F
        # DirichletBC.apply: the wall rows take the wall values (0 unless given)
        b[self.dir] = 0.0 if dvals is None else np.asarray(dvals)[self.dir]
        return b

    def step(self, u: np.ndarray, F: Optional[np.ndarray] = None,
             dvals: Optional[np.ndarray] = None) -> np.ndarray:
        b = self.rhs(u, F, dvals)
        if self.lu is None:
            return spla.spsolve(self.A, b)
        return self.lu.solve(b)

    def balance(self, u_new: np.ndarray, u_old: np.ndarray,
                F: Optional[np.ndarray] = None) -> dict:
        """Discrete balance of one step from the assembled matrices.  r = A_full u_new
        - M u_old - F_full on every row (A_full without the Dirichlet replacement,
        F_full the point load plus the Robin load); its sum over the Dirichlet rows is
        minus the wall outflow, over the free rows the drift.  The decay and operator
        terms split 1'A_full u_new - 1'M u_new (the stiffness sums to zero)."""
        Ff = self.robin_load + (0.0 if F is None else F)
        r = self.A_full @ u_new - self.M @ u_old - Ff
        mass = float(np.sum(self.M @ u_new))
        decay = self.dt * self.g * mass
        total_op = float(np.sum(self.A_full @ u_new))
        return {"mass": mass, "mass_prev": float(np.sum(self.M @ u_old)),
                "load": float(np.sum(Ff)), "decay": decay,
                "operator_loss": total_op - (1.0 + self.dt * self.g) * mass,
                "wall_outflow": -float(np.sum(r[self.dir])),
                "drift": float(np.sum(r[~self.dir]))}

    def total_mass(self, u: np.ndarray) -> float:
        return float(np.sum(self.M @ u))

    def boundary_flux(self, u: np.ndarray) -> float:
        """totalBoundaryFlux = D * dt * (-int grad u . n ds) (src/fHSL.cpp:160)."""
        return self.D * self.dt * boundary_flux_integral(self.mesh, u)


def run_trap(trap, steps: Optional[int] = None, snapshots=(), oracles=None):
    """Run a workload ``Trap`` (eq_gb300.workloads) with the oracle.

    Returns dict with final nodal fields per species (grid order), per-cell
    concentrations per species at the final time, and requested snapshots.
    Single species: F = dt * sum s_i phi(x_i), constant.
    Two species (sender/receiver): explicit per-cell sources from the previous
    step's gathered concentrations:
        sigma1_i = [sender] * s_i - 0.05 * c1(x_i)
        sigma2_i = [receiver] * 0.5 * c1(x_i) / (0.1 + c1(x_i)) - 0.05 * c2(x_i)
    """
    steps = trap.steps if steps is None else steps
    ns = trap.n_species
    vel = None
    if trap.adv_u:
        u_, L_ = trap.adv_u, trap.adv_len
        vel = lambda x, y: (np.zeros_like(x), -u_ * y / L_)
    if oracles is None:
        oracles = [HsldOracle(trap.W, trap.H, trap.nx, trap.ny, trap.D[k], trap.dt, trap.g[k],
                              trap.walls, velocity=vel) for k in range(ns)]
    mesh = oracles[0].mesh
    u = [np.zeros(mesh.n_nodes) for _ in range(ns)]
    snaps = {}
    nodes, w = point_weights(mesh, trap.cell_xy)
    if ns == 1:
        F = point_load(mesh, trap.cell_xy, trap.cell_s, scale=trap.dt)
    for n in range(1, steps + 1):
        if ns == 1:
            u[0] = oracles[0].step(u[0], F)
        else:
            c1 = np.sum(u[0][nodes] * w, axis=1)
            c2 = np.sum(u[1][nodes] * w, axis=1)
            sig1 = trap.cell_kind * trap.cell_s - 0.05 * c1
            sig2 = (1 - trap.cell_kind) * 0.5 * c1 / (0.1 + c1) - 0.05 * c2
            F1 = point_load(mesh, trap.cell_xy, sig1, scale=trap.dt)
            F2 = point_load(mesh, trap.cell_xy, sig2, scale=trap.dt)
            u = [oracles[0].step(u[0], F1), oracles[1].step(u[1], F2)]
        if n in snapshots:
            snaps[n] = [x.copy() for x in u]
    cells = [np.sum(x[nodes] * w, axis=1) for x in u]
    return {"u": u, "cells": cells, "snapshots": snaps, "oracles": oracles}
