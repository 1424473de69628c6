"""Electrostatic set-up: per-electrode unit basis fields of the Laplace problem.

The reference solves one Laplace problem with FEniCS every time a voltage
changes (``init_V`` / ``update_V``, kmc_dopant_networks.py:706-822): P1
elements on a ``RectangleMesh`` of ``int(xdim//res) x int(ydim//res)`` cells
(kmc_dopant_networks.py:771-777, default diagonal "right"), Dirichlet data on
the whole boundary given by a C++ ternary expression (kmc_dopant_networks.py:
733-763): an electrode is its voltage on the boundary segment
``[c - xdim/10, c + xdim/10]`` of its edge, and the rest of the boundary is the
chemical potential ``mu``.

Here the problem is linear in the boundary data, so it is solved once per
geometry for unit data on each electrode (and on the ``mu`` part of the
boundary); any voltage vector is then the superposition
``V = sum_e V_e * phi_e + mu * phi_mu`` (the same linear-rescale idea as
kmc_dopant_networks_utils.py:660-676).  On a uniform mesh of right triangles
the P1 stiffness matrix is the (anisotropic) 5-point finite-difference
stencil: the hypotenuse couplings vanish because the cotangent of the right
angle is zero.  So the nodal values below equal the FEniCS solution, and
``interpolate_p1`` reproduces FEniCS point evaluation on the same
triangulation.  This is host set-up in FP64 and is not on the hop path.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

__all__ = ["BasisFields", "boundary_owner", "solve_basis_fields", "solve_basis_fields_gpu",
           "interpolate_p1", "default_cells", "boundary_grids"]


def default_cells(length: float, res: float) -> int:
    """Number of mesh cells along one side, computed exactly as the reference
    does (``int(xdim//res)``, kmc_dopant_networks.py:774-777).

    Note the float floor division: ``1 // 0.01 == 99``, so the reference's
    default ``res = min(xdim, ydim)/100`` gives 99 cells (100 vertices)."""
    return int(length // res)


def boundary_owner(xs, ys, xdim, ydim, electrodes, surplus=None):
    """For each boundary vertex return the index of the electrode that the
    reference's boundary expression assigns to it, or -1 for ``mu``.

    ``electrodes`` is a (P, >=2) array of electrode x, y positions (transport
    electrodes first, static electrodes after, the order of the expression
    string).  The first matching electrode wins, as in the C++ ternary chain
    (kmc_dopant_networks.py:742-761).  Comparisons are exact float
    comparisons, as in the compiled expression."""
    if surplus is None:
        surplus = xdim / 10
    owner = np.full(np.shape(xs), -1, dtype=np.int64)
    for e in range(len(electrodes) - 1, -1, -1):   # reverse: first match wins
        ex, ey = float(electrodes[e][0]), float(electrodes[e][1])
        if ex == 0 or ex == xdim:
            m = (xs == ex) & (ys >= ey - surplus) & (ys <= ey + surplus)
        else:
            m = (xs >= ex - surplus) & (xs <= ex + surplus) & (ys == ey)
        owner[m] = e
    return owner


class BasisFields:
    """Unit-voltage solutions on the vertex grid.

    ``fields[k]`` for k < n_el is the potential with electrode k at 1 and all
    other boundary data 0; ``fields[n_el]`` is the potential with the ``mu``
    part of the boundary at 1 and every electrode at 0."""

    def __init__(self, fields, xdim, ydim, nx, ny, dim):
        self.fields = fields
        self.xdim, self.ydim = float(xdim), float(ydim)
        self.nx, self.ny = int(nx), int(ny)
        self.dim = dim

    @property
    def n_basis(self):
        return self.fields.shape[0]

    def potential(self, voltages, mu=0.0):
        """Nodal potential for one voltage vector (length n_basis-1)."""
        v = np.asarray(voltages, dtype=np.float64)
        out = np.tensordot(v, self.fields[:-1], axes=(0, 0))
        return out + float(mu) * self.fields[-1]

    def sample(self, points):
        """Basis values at points: array (n_basis, n_points).  P1 interpolation
        on the reference's triangulation."""
        pts = np.asarray(points, dtype=np.float64)
        return np.stack([interpolate_p1(f, self, pts) for f in self.fields])


def solve_basis_fields(xdim, ydim, electrodes, nx, ny=None, surplus=None):
    """Solve the Laplace problem for unit data on each electrode and on mu.

    electrodes: (P, >=2) positions (transport then static electrodes).
    nx, ny: number of cells per side (``default_cells`` gives the
    reference's count).  ydim == 0 selects the 1D problem."""
    electrodes = np.asarray(electrodes, dtype=np.float64)
    electrodes = electrodes.reshape(-1, electrodes.shape[-1] if electrodes.ndim == 2 else 2)
    P = electrodes.shape[0]
    if ydim == 0:
        # 1D: IntervalMesh(int(xdim//res), 0, xdim); boundary = the two end
        # points, value "x[0] == e_x ? e : mu" (kmc_dopant_networks.py:736-739).
        xs = np.arange(nx + 1) * (xdim / nx)
        fields = np.zeros((P + 1, nx + 1))
        for end, xv in ((0, 0.0), (nx, float(xdim))):
            owner = -1
            for e in range(P):
                if float(electrodes[e, 0]) == xv:
                    owner = e
                    break
            k = owner if owner >= 0 else P
            # exact linear solution between the end values
            prof = xs / xdim if end == nx else 1.0 - xs / xdim
            fields[k] += prof
        return BasisFields(fields, xdim, 0.0, nx, 0, 1)

    if ny is None:
        ny = nx
    hx, hy = xdim / nx, ydim / ny
    # Vertex coordinates as the mesh generator computes them: a + i*(b-a)/n.
    gx = np.arange(nx + 1) * hx
    gy = np.arange(ny + 1) * hy
    X, Y = np.meshgrid(gx, gy)          # [iy, ix]
    on_b = np.zeros((ny + 1, nx + 1), dtype=bool)
    on_b[0, :] = on_b[-1, :] = on_b[:, 0] = on_b[:, -1] = True
    owner = boundary_owner(X[on_b], Y[on_b], xdim, ydim, electrodes, surplus)

    # Boundary data per basis: (P+1, n_boundary)
    nb = owner.shape[0]
    bdata = np.zeros((P + 1, nb))
    for k in range(P):
        bdata[k, owner == k] = 1.0
    bdata[P, owner < 0] = 1.0

    # Interior system: anisotropic 5-point stencil (P1 on right triangles).
    mi, mj = ny - 1, nx - 1
    n_int = mi * mj
    cx, cy = hy / hx, hx / hy
    idx = -np.ones((ny + 1, nx + 1), dtype=np.int64)
    idx[1:-1, 1:-1] = np.arange(n_int).reshape(mi, mj)
    bidx = -np.ones((ny + 1, nx + 1), dtype=np.int64)
    bidx[on_b] = np.arange(nb)

    rows, cols, vals = [], [], []
    rhs_rows, rhs_b, rhs_w = [], [], []
    I, J = np.meshgrid(np.arange(1, ny), np.arange(1, nx), indexing="ij")
    I, J = I.ravel(), J.ravel()
    me = idx[I, J]
    rows.append(me); cols.append(me); vals.append(np.full(me.shape, 2 * (cx + cy)))
    for di, dj, w in ((0, -1, cx), (0, 1, cx), (-1, 0, cy), (1, 0, cy)):
        ni, nj = I + di, J + dj
        nb_int = idx[ni, nj]
        inside = nb_int >= 0
        rows.append(me[inside]); cols.append(nb_int[inside]); vals.append(np.full(inside.sum(), -w))
        rhs_rows.append(me[~inside]); rhs_b.append(bidx[ni[~inside], nj[~inside]])
        rhs_w.append(np.full((~inside).sum(), w))
    A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n_int, n_int))
    rr, bb, ww = map(np.concatenate, (rhs_rows, rhs_b, rhs_w))
    B = np.zeros((n_int, P + 1))
    for k in range(P + 1):
        np.add.at(B[:, k], rr, ww * bdata[k, bb])
    sol = spla.splu(A).solve(B)          # (n_int, P+1)

    fields = np.zeros((P + 1, ny + 1, nx + 1))
    for k in range(P + 1):
        f = fields[k]
        f[on_b] = bdata[k]
        f[1:-1, 1:-1] = sol[:, k].reshape(mi, mj)
    return BasisFields(fields, xdim, ydim, nx, ny, 2)


def interpolate_p1(field, basis: BasisFields, pts, diagonal="right"):
    """Evaluate the piecewise-linear interpolant of nodal ``field`` at points.

    2D: cell (ix, iy) is split along the diagonal from (ix, iy) to
    (ix+1, iy+1) ("right", the mesh generator's default) or from (ix+1, iy)
    to (ix, iy+1) ("left")."""
    pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
    if basis.dim == 1:
        x = pts[:, 0]
        h = basis.xdim / basis.nx
        s = x / h
        ix = np.clip(np.floor(s).astype(np.int64), 0, basis.nx - 1)
        t = s - ix
        return field[ix] * (1 - t) + field[ix + 1] * t
    hx, hy = basis.xdim / basis.nx, basis.ydim / basis.ny
    sx, sy = pts[:, 0] / hx, pts[:, 1] / hy
    ix = np.clip(np.floor(sx).astype(np.int64), 0, basis.nx - 1)
    iy = np.clip(np.floor(sy).astype(np.int64), 0, basis.ny - 1)
    xi, eta = sx - ix, sy - iy
    f00 = field[iy, ix]
    f10 = field[iy, ix + 1]
    f01 = field[iy + 1, ix]
    f11 = field[iy + 1, ix + 1]
    if diagonal == "right":
        lower = xi >= eta
        v_lo = f00 + xi * (f10 - f00) + eta * (f11 - f10)
        v_up = f00 + eta * (f01 - f00) + xi * (f11 - f01)
        return np.where(lower, v_lo, v_up)
    lower = (xi + eta) <= 1.0
    v_lo = f00 + xi * (f10 - f00) + eta * (f01 - f00)
    v_up = f11 + (1 - xi) * (f01 - f11) + (1 - eta) * (f10 - f11)
    return np.where(lower, v_lo, v_up)


def boundary_grids(xdim, ydim, electrodes, nx, ny, surplus=None):
    """Nodal grids (P+1, ny+1, nx+1) carrying each basis field's boundary
    data (electrode k at 1 in field k, the mu boundary at 1 in field P);
    interior entries are 0."""
    electrodes = np.asarray(electrodes, dtype=np.float64)
    electrodes = electrodes.reshape(-1, electrodes.shape[-1] if electrodes.ndim == 2 else 2)
    P = electrodes.shape[0]
    hx, hy = xdim / nx, ydim / ny
    X, Y = np.meshgrid(np.arange(nx + 1) * hx, np.arange(ny + 1) * hy)
    on_b = np.zeros((ny + 1, nx + 1), dtype=bool)
    on_b[0, :] = on_b[-1, :] = on_b[:, 0] = on_b[:, -1] = True
    owner = boundary_owner(X[on_b], Y[on_b], xdim, ydim, electrodes, surplus)
    grids = np.zeros((P + 1, ny + 1, nx + 1))
    for k in range(P):
        grids[k][on_b] = (owner == k).astype(np.float64)
    grids[P][on_b] = (owner < 0).astype(np.float64)
    return grids


def solve_basis_fields_gpu(xdim, ydim, electrodes, nx, ny=None, surplus=None, dev=None):
    """The basis fields of ``solve_basis_fields``, solved on the device by
    kmc_laplace_basis (sine-transform direct solve of the same 5-point
    system).  2D only."""
    import ctypes as C
    import torch
    from ._native import lib, check
    if ydim == 0:
        return solve_basis_fields(xdim, ydim, electrodes, nx)
    ny = nx if ny is None else ny
    grids = boundary_grids(xdim, ydim, electrodes, nx, ny, surplus)
    d = torch.device(dev if dev is not None else "cuda")
    g = torch.as_tensor(grids, dtype=torch.float64).to(d).contiguous()
    L = lib()
    wsb = L.kmc_laplace_workspace_size(nx, ny, grids.shape[0])
    ws = torch.empty(max(int(wsb), 8), dtype=torch.uint8, device=d)
    st = C.c_void_p(torch.cuda.current_stream(d).cuda_stream)
    check(L.kmc_laplace_basis(nx, ny, xdim / nx, ydim / ny, grids.shape[0], C.c_void_p(g.data_ptr()),
                              C.c_void_p(ws.data_ptr()), wsb, st))
    torch.cuda.synchronize(d)
    return BasisFields(g.cpu().numpy(), xdim, ydim, nx, ny, 2)
