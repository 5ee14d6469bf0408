"""Seeded synthetic problems for the sparse-solver hot path.

Every generator is deterministic (numpy ``default_rng`` with a fixed seed) and
returns plain numpy arrays: CSR matrices as ``(rowptr int32, colidx int32,
values float64)`` with ascending column indices in every row, vectors as
``float64``.  The same arrays feed the CPU oracle and the GPU library, so the
two see bit-identical inputs.

The operators mirror the reference's structured test problems:

* 2D 5-point / 3D 7-point Laplacians with homogeneous Dirichlet boundaries
  eliminated (the DMDA stencils of
  ``utopia/tests/test_problems/large_scale_benchmark/utopia_Poisson3D.hpp:143-339``,
  unscaled: diagonal 4 or 6, off-diagonals -1).
* Vertex-centred (bi/tri)linear interpolation between nested grids, the
  transfer that ``PetscMultilevelTestProblem`` obtains from
  ``DMCreateInterpolation``
  (``utopia/tests/test_problems/utopia_PetscMultilevelTestProblem.hpp:32-86``),
  restricted to interior nodes: coarse node ``i`` sits on fine node ``2i+1``.
"""

from __future__ import annotations

import numpy as np

try:  # scipy is only needed for the interpolation operators and the random field
    import scipy.sparse as _sp
except Exception:  # pragma: no cover
    _sp = None


# --------------------------------------------------------------------------------------
# CSR helpers
# --------------------------------------------------------------------------------------
class CSR:
    """Host CSR matrix (int32 indices, float64 values, sorted columns)."""

    __slots__ = ("nrows", "ncols", "rowptr", "colidx", "values")

    def __init__(self, nrows, ncols, rowptr, colidx, values):
        self.nrows = int(nrows)
        self.ncols = int(ncols)
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.colidx = np.ascontiguousarray(colidx, dtype=np.int32)
        self.values = np.ascontiguousarray(values, dtype=np.float64)

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    @property
    def shape(self):
        return (self.nrows, self.ncols)

    def to_scipy(self):
        return _sp.csr_matrix((self.values, self.colidx, self.rowptr), shape=self.shape)

    @staticmethod
    def from_scipy(m) -> "CSR":
        m = m.tocsr()
        m.sort_indices()
        return CSR(m.shape[0], m.shape[1], m.indptr, m.indices, m.data)

    def matvec(self, x):
        """y = A x in float64 (numpy, for tests and problem set-up only)."""
        rows = np.repeat(np.arange(self.nrows), np.diff(self.rowptr))
        return np.bincount(rows, weights=self.values * x[self.colidx], minlength=self.nrows)


def _stencil_csr(n, cols, vals, valid):
    """Compress an (n, k) stencil table (columns ascending along axis 1) into CSR."""
    counts = valid.sum(axis=1, dtype=np.int64)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rowptr[1:])
    if rowptr[-1] >= 2**31:
        raise ValueError("nnz exceeds int32 CSR indexing")
    return CSR(n, n, rowptr.astype(np.int32), cols[valid].astype(np.int32), vals[valid])


def laplacian_2d(nx: int, ny: int | None = None) -> CSR:
    """Unscaled 5-point Laplacian on an nx*ny interior grid, index = y*nx + x."""
    ny = nx if ny is None else ny
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    x = idx % nx
    y = idx // nx
    offs = [-nx, -1, 0, 1, nx]
    valid = np.stack([y > 0, x > 0, np.ones(n, bool), x < nx - 1, y < ny - 1], axis=1)
    cols = idx[:, None] + np.asarray(offs)[None, :]
    vals = np.broadcast_to(np.array([-1.0, -1.0, 4.0, -1.0, -1.0]), (n, 5))
    return _stencil_csr(n, cols, vals, valid)


def laplacian_3d(nx: int, ny: int | None = None, nz: int | None = None) -> CSR:
    """Unscaled 7-point Laplacian on an nx*ny*nz interior grid, index = (z*ny + y)*nx + x."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64)
    x = idx % nx
    y = (idx // nx) % ny
    z = idx // (nx * ny)
    pl = nx * ny
    offs = [-pl, -nx, -1, 0, 1, nx, pl]
    valid = np.stack(
        [z > 0, y > 0, x > 0, np.ones(n, bool), x < nx - 1, y < ny - 1, z < nz - 1], axis=1
    )
    cols = idx[:, None] + np.asarray(offs)[None, :]
    vals = np.broadcast_to(np.array([-1.0, -1.0, -1.0, 6.0, -1.0, -1.0, -1.0]), (n, 7))
    return _stencil_csr(n, cols, vals, valid)


def diffusion_3d_faces(kx, ky, kz, kbx, kby, kbz) -> CSR:
    """7-point operator of -div(k grad u) from face conductances.

    ``kx[z,y,x]`` couples (x,y,z)-(x+1,y,z) (shape (N,N,N-1)); ``ky``/``kz`` alike.
    ``kbx`` (shape (N,N,2)) holds the Dirichlet boundary-face conductances of the
    x=0 and x=N-1 faces; ``kby``/``kbz`` alike.  A_ii is the sum of the node's
    face conductances, A_ij = -k_face.
    """
    nz, ny, nxm1 = kx.shape
    nx = nxm1 + 1
    n = nx * ny * nz
    shp = (nz, ny, nx)
    zero = np.zeros(shp)
    # conductance to each of the six neighbours, (0 where the neighbour is the boundary)
    c_xm = zero.copy(); c_xm[:, :, 1:] = kx
    c_xp = zero.copy(); c_xp[:, :, :-1] = kx
    c_ym = zero.copy(); c_ym[:, 1:, :] = ky
    c_yp = zero.copy(); c_yp[:, :-1, :] = ky
    c_zm = zero.copy(); c_zm[1:, :, :] = kz
    c_zp = zero.copy(); c_zp[:-1, :, :] = kz
    diag = c_xm + c_xp + c_ym + c_yp + c_zm + c_zp
    diag[:, :, 0] += kbx[:, :, 0]
    diag[:, :, -1] += kbx[:, :, 1]
    diag[:, 0, :] += kby[:, :, 0]
    diag[:, -1, :] += kby[:, :, 1]
    diag[0, :, :] += kbz[:, :, 0]
    diag[-1, :, :] += kbz[:, :, 1]
    idx = np.arange(n, dtype=np.int64)
    x = idx % nx
    y = (idx // nx) % ny
    z = idx // (nx * ny)
    pl = nx * ny
    offs = [-pl, -nx, -1, 0, 1, nx, pl]
    valid = np.stack(
        [z > 0, y > 0, x > 0, np.ones(n, bool), x < nx - 1, y < ny - 1, z < nz - 1], axis=1
    )
    cols = idx[:, None] + np.asarray(offs)[None, :]
    vals = np.stack(
        [-c_zm.ravel(), -c_ym.ravel(), -c_xm.ravel(), diag.ravel(),
         -c_xp.ravel(), -c_yp.ravel(), -c_zp.ravel()], axis=1)
    return _stencil_csr(n, cols, vals, valid)


# --------------------------------------------------------------------------------------
# Interpolation (prolongation) operators, coarse -> fine
# --------------------------------------------------------------------------------------
def _interp_1d(nf: int):
    """1D vertex-centred linear interpolation on interior nodes, nf even -> nc = nf/2.

    Coarse node i sits on fine node 2i+1 (weight 1); fine node 2i (i >= 1) takes
    1/2 from coarse i-1 and i; fine node 0 takes 1/2 from coarse 0 (its other
    neighbour is the Dirichlet boundary, value 0).
    """
    if nf % 2:
        raise ValueError("fine size must be even")
    nc = nf // 2
    rows, cols, vals = [], [], []
    for f in range(nf):
        if f % 2 == 1:
            rows.append(f); cols.append((f - 1) // 2); vals.append(1.0)
        else:
            i = f // 2
            if i - 1 >= 0:
                rows.append(f); cols.append(i - 1); vals.append(0.5)
            rows.append(f); cols.append(i); vals.append(0.5)
    return _sp.csr_matrix((vals, (rows, cols)), shape=(nf, nc))


def interpolation_2d(nf: int) -> CSR:
    p = _interp_1d(nf)
    return CSR.from_scipy(_sp.kron(p, p, format="csr"))


def interpolation_3d(nf: int) -> CSR:
    p = _interp_1d(nf)
    return CSR.from_scipy(_sp.kron(_sp.kron(p, p, format="csr"), p, format="csr"))


def hierarchy_3d(nf: int, n_levels: int):
    """Interpolation operators ordered coarse -> fine (the order
    ``LinearMultiLevel::set_transfer_operators`` expects,
    utopia/solvers/multilevel/utopia_LinearMultiLevel.hpp:58-79)."""
    sizes = [nf >> l for l in range(n_levels)]
    ops = [interpolation_3d(s) for s in sizes[:-1]]
    return ops[::-1]


def hierarchy_2d(nf: int, n_levels: int):
    sizes = [nf >> l for l in range(n_levels)]
    ops = [interpolation_2d(s) for s in sizes[:-1]]
    return ops[::-1]


# --------------------------------------------------------------------------------------
# Random fields
# --------------------------------------------------------------------------------------
def gaussian_field(rng, shape, corr_len: float):
    """White noise smoothed separably by a Gaussian of std ``corr_len`` cells
    (periodic wrap), renormalised to zero mean and unit standard deviation."""
    from scipy.ndimage import gaussian_filter

    g = rng.standard_normal(shape)
    g = gaussian_filter(g, sigma=corr_len, mode="wrap", truncate=4.0)
    g = (g - g.mean()) / g.std()
    return g


def lognormal_diffusion_3d(N: int, seed: int, sigma: float = 1.0, corr_len: float = 8.0):
    """-div(k grad u) on N^3 with k = exp(sigma * g), g a unit Gaussian field.

    Interior face conductance k_f = exp((g_i + g_j) / 2); Dirichlet boundary faces
    exp(g_i).  Returns (A, g, rng) so callers continue the same random stream.
    """
    rng = np.random.default_rng(seed)
    g = sigma * gaussian_field(rng, (N, N, N), corr_len)
    kx = np.exp(0.5 * (g[:, :, 1:] + g[:, :, :-1]))
    ky = np.exp(0.5 * (g[:, 1:, :] + g[:, :-1, :]))
    kz = np.exp(0.5 * (g[1:, :, :] + g[:-1, :, :]))
    eg = np.exp(g)
    kbx = np.stack([eg[:, :, 0], eg[:, :, -1]], axis=2)
    kby = np.stack([eg[:, 0, :], eg[:, -1, :]], axis=2)
    kbz = np.stack([eg[0, :, :], eg[-1, :, :]], axis=2)
    return diffusion_3d_faces(kx, ky, kz, kbx, kby, kbz), g, rng


# --------------------------------------------------------------------------------------
# Graph problem with per-edge log-conductances (differentiable solve)
# --------------------------------------------------------------------------------------
class EdgeGraph:
    """7-point grid graph with E interior edges, ordered x-edges, y-edges, z-edges.

    ``src < dst`` for every edge.  ``pos_ij``/``pos_ji`` are the CSR positions of
    A[src,dst] and A[dst,src], ``diag_pos`` the position of every diagonal entry,
    so edge data can be scattered onto the sparsity pattern directly.
    """

    def __init__(self, N: int):
        self.N = N
        n = N ** 3
        idx = np.arange(n, dtype=np.int64).reshape(N, N, N)
        ex = (idx[:, :, :-1].ravel(), idx[:, :, 1:].ravel())
        ey = (idx[:, :-1, :].ravel(), idx[:, 1:, :].ravel())
        ez = (idx[:-1, :, :].ravel(), idx[1:, :, :].ravel())
        self.src = np.concatenate([ex[0], ey[0], ez[0]]).astype(np.int32)
        self.dst = np.concatenate([ex[1], ey[1], ez[1]]).astype(np.int32)
        self.n = n
        self.E = int(self.src.size)
        # boundary-face count per node (unit conductance Dirichlet faces)
        x = np.arange(n) % N
        y = (np.arange(n) // N) % N
        z = np.arange(n) // (N * N)
        self.nbnd = ((x == 0).astype(np.int64) + (x == N - 1) + (y == 0) + (y == N - 1)
                     + (z == 0) + (z == N - 1)).astype(np.float64)
        lap = laplacian_3d(N)
        self.rowptr = lap.rowptr
        self.colidx = lap.colidx
        self.diag_pos = self._positions(np.arange(n), np.arange(n))
        self.pos_ij = self._positions(self.src, self.dst)
        self.pos_ji = self._positions(self.dst, self.src)

    def _positions(self, rows, cols):
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        start = self.rowptr[rows].astype(np.int64)
        cnt = (self.rowptr[rows + 1] - self.rowptr[rows]).astype(np.int64)
        out = np.full(rows.size, -1, dtype=np.int64)
        for k in range(7):
            m = (k < cnt) & (out < 0)
            hit = m & (self.colidx[np.minimum(start + k, self.colidx.size - 1)] == cols)
            out[hit] = start[hit] + k
        assert (out >= 0).all()
        return out.astype(np.int32)

    def edge_of_pos(self):
        """Edge id of every CSR entry of the Laplacian pattern (-1 on the diagonal)."""
        eop = np.full(self.colidx.size, -1, dtype=np.int32)
        e = np.arange(self.E, dtype=np.int32)
        eop[self.pos_ij] = e
        eop[self.pos_ji] = e
        return eop

    def assemble(self, theta) -> CSR:
        """A(theta) = sum_e exp(theta_e) (e_i - e_j)(e_i - e_j)^T + unit Dirichlet faces."""
        k = np.exp(np.asarray(theta, dtype=np.float64))
        vals = np.zeros(self.colidx.size)
        diag = self.nbnd.copy()
        np.add.at(diag, self.src, k)
        np.add.at(diag, self.dst, k)
        vals[self.diag_pos] = diag
        vals[self.pos_ij] = -k
        vals[self.pos_ji] = -k
        return CSR(self.n, self.n, self.rowptr, self.colidx, vals)


# --------------------------------------------------------------------------------------
# The five workloads
# --------------------------------------------------------------------------------------
def poisson2d_cg(N: int = 256, seed: int = 0):
    """CG + Jacobi on the 2D 5-point Laplacian, b ~ U[-1,1], x0 = 0."""
    A = laplacian_2d(N)
    b = np.random.default_rng(seed).uniform(-1.0, 1.0, A.nrows)
    return A, b


def poisson3d_mg(N: int = 128, n_levels: int = 4, seed: int = 1):
    """MG-PCG on the 3D 7-point Laplacian with trilinear transfers, b ~ U[-1,1]."""
    A = laplacian_3d(N)
    b = np.random.default_rng(seed).uniform(-1.0, 1.0, A.nrows)
    return A, hierarchy_3d(N, n_levels), b


def lognormal_mg(N: int = 192, n_levels: int = 5, seed: int = 2):
    """Variable-coefficient diffusion, lognormal k (sigma 1, correlation 8 cells)."""
    A, g, rng = lognormal_diffusion_3d(N, seed)
    b = rng.uniform(-1.0, 1.0, A.nrows)
    return A, hierarchy_3d(N, n_levels), b


def obstacle_qp(N: int = 1024, seed: int = 3, n_bumps: int = 8, rhs: float = -1.0):
    """Box-constrained QP min 1/2 x'Ax - b'x, x >= l, on the 2D 5-point Laplacian.

    l(x,y) = 0.3 * sum_k exp(-|p - c_k|^2 / (2 w_k^2)) - 0.2 at p = ((i+1)h, (j+1)h),
    h = 1/(N+1), c_k ~ U[0,1]^2, w_k ~ U[0.02, 0.1]; upper bound +inf (the largest
    double, as ``BoxConstraints::fill_empty_bounds`` uses).
    """
    A = laplacian_2d(N)
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, (n_bumps, 2))
    w = rng.uniform(0.02, 0.1, n_bumps)
    h = 1.0 / (N + 1)
    px = (np.arange(N) + 1) * h
    X, Y = np.meshgrid(px, px, indexing="xy")  # X[j, i] = x_i, row-major index j*N + i
    lb = np.zeros((N, N))
    for k in range(n_bumps):
        lb += np.exp(-((X - c[k, 0]) ** 2 + (Y - c[k, 1]) ** 2) / (2.0 * w[k] ** 2))
    lb = 0.3 * lb - 0.2
    b = np.full(A.nrows, rhs)
    ub = np.full(A.nrows, np.finfo(np.float64).max)
    return A, b, lb.ravel(), ub


def graph_adjoint(N: int = 128, seed: int = 4, seed_target: int = 5):
    """Per-edge log-conductance graph problem for the differentiable solve."""
    G = EdgeGraph(N)
    rng = np.random.default_rng(seed)
    theta = rng.normal(0.0, 0.5, G.E).astype(np.float32)
    b = rng.uniform(-0.01, 0.01, G.n)
    c = N // 2
    b[(c * N + c) * N + c] += 1.0
    theta_t = np.random.default_rng(seed_target).normal(0.0, 0.5, G.E).astype(np.float32)
    return G, theta, b, theta_t


def laplacian_1d_dirichlet(n: int) -> CSR:
    """assemble_laplacian_1D(A, bc=true) (utopia/tests/test_problems/utopia_assemble_laplacian_1D.hpp:11-40):
    rows 0 and n-1 are the identity, interior rows (-1, 2, -1) including the columns of the boundary."""
    rows, cols, vals = [0, n - 1], [0, n - 1], [1.0, 1.0]
    for i in range(1, n - 1):
        rows += [i, i, i]
        cols += [i - 1, i, i + 1]
        vals += [-1.0, 2.0, -1.0]
    return CSR.from_scipy(_sp.csr_matrix((vals, (rows, cols)), shape=(n, n)))


def qp_test_problem_1d(n: int = 20):
    """QPSolverTestProblem::run (utopia/tests/test_problems/utopia_QPSolverTestProblem.hpp:29-97):
    the 1D Laplacian (-1, 2, -1) with rows 0 and n-1 set to the identity (their off-diagonal entry
    kept as an explicit zero), rhs 1 with 0 at both ends, upper bound 30; returns A, rhs, ub."""
    rows, cols, vals = [0, 0, n - 1, n - 1], [0, 1, n - 2, n - 1], [1.0, 0.0, 0.0, 1.0]
    for i in range(1, n - 1):
        rows += [i, i, i]
        cols += [i - 1, i, i + 1]
        vals += [-1.0, 2.0, -1.0]
    A = _sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    b = np.ones(n)
    b[0] = b[-1] = 0.0
    return CSR.from_scipy(A), b, np.full(n, 30.0)


def block_rotation(n: int, seed: int, reflection: bool = False) -> CSR:
    """An orthogonal sparse matrix: independent 2 x 2 rotations [[c, -s], [s, c]] of the pairs
    (2k, 2k+1) by random angles, or with reflection=True the symmetric reflections
    [[c, s], [s, -c]] (the last row the identity when n is odd) -- stand-ins for a contact basis."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(0.0, 2.0 * np.pi, n // 2)
    c, s = np.cos(th), np.sin(th)
    i = np.arange(n // 2) * 2
    rows = np.concatenate([i, i, i + 1, i + 1] + ([np.array([n - 1])] if n % 2 else []))
    cols = np.concatenate([i, i + 1, i, i + 1] + ([np.array([n - 1])] if n % 2 else []))
    blocks = [c, s, s, -c] if reflection else [c, -s, s, c]
    vals = np.concatenate(blocks + ([np.array([1.0])] if n % 2 else []))
    return CSR.from_scipy(_sp.csr_matrix((vals, (rows, cols)), shape=(n, n)))


def random_spd_graph(n: int, degree: int, seed: int) -> CSR:
    """Weighted graph Laplacian of a random graph plus a small diagonal shift (SPD, unstructured)."""
    rng = np.random.default_rng(seed)
    i = np.repeat(np.arange(n), degree)
    j = rng.integers(0, n, n * degree)
    keep = i != j
    w = rng.uniform(0.1, 2.0, keep.sum())
    W = _sp.coo_matrix((w, (i[keep], j[keep])), shape=(n, n)).tocsr()
    W = W + W.T
    L = _sp.diags(np.asarray(W.sum(axis=1)).ravel() + 1e-3) - W
    L = L.tocsr()
    L.sort_indices()
    return CSR.from_scipy(L)


def convection_diffusion_2d(n: int, peclet: float = 20.0) -> CSR:
    """-Laplace(u) + c . grad(u) on n x n interior nodes, 5-point diffusion and first-order upwind
    convection with c = (peclet, peclet / 2): a nonsymmetric M-matrix (BiCGStab test operator)."""
    h = 1.0 / (n + 1)
    cx, cy = peclet, peclet / 2
    main = 4.0 / h**2 + (cx + cy) / h
    T = _sp.diags([-1.0 / h**2 - cx / h, 0.0, -1.0 / h**2], [-1, 0, 1], shape=(n, n))
    Ty = _sp.diags([-1.0 / h**2 - cy / h, 0.0, -1.0 / h**2], [-1, 0, 1], shape=(n, n))
    I = _sp.identity(n)
    A = (_sp.kron(I, T) + _sp.kron(Ty, I) + main * _sp.identity(n * n)).tocsr()
    A.sort_indices()
    return CSR.from_scipy(A)


def poisson1d_obstacle_multilevel(n_levels: int = 6, n_coarse_elements: int = 50, lower: float = -0.8,
                                  upper: float = 200.0):
    """The monotone multigrid case of utopia/tests/utopia_QPSolverTest.cpp:715-771 on the problem of
    MultiLevelTestProblem1D<Poisson1D> (utopia/tests/test_problems/large_scale_benchmark/
    utopia_MultilevelTestProblem1D.hpp:61-150, utopia_Poisson1D.hpp problem type 2):

    * level sizes n_0 = n_coarse_elements + 1, n_{l+1} = 2 (n_l - 1) + 1;
    * interpolation n_l -> n_{l+1}: fine row 2j takes coarse j with weight 1, fine row 2j+1 takes
      coarse j and j+1 with weight 1/2; on the finest transfer (remove_bc) the entries (0, 0) and
      (n-1, n_c-1) are zero (kept in the structure);
    * H = (1/h) tridiag(-1, 2, -1) with rows 0 and n-1 replaced by identity rows, h = 1/(n-1);
    * the right-hand side is the gradient at the boundary values (all zero): -10 h on the interior,
      0 on the boundary; box lower <= x <= upper.

    Returns (H, g, lb, ub, interpolations ordered coarse -> fine)."""
    sizes = [n_coarse_elements + 1]
    for _ in range(1, n_levels):
        sizes.append((sizes[-1] - 1) * 2 + 1)
    Ps = []
    for i in range(n_levels - 1):
        nc, nf = sizes[i], sizes[i + 1]
        rows, cols, vals = [], [], []
        for j in range(nc):
            rows.append(2 * j); cols.append(j); vals.append(1.0)
            if j + 1 < nc:
                rows += [2 * j + 1, 2 * j + 1]; cols += [j, j + 1]; vals += [0.5, 0.5]
        if i == n_levels - 2:
            vals[0] = 0.0                                  # (0, 0)
            last = [k for k in range(len(rows)) if rows[k] == nf - 1 and cols[k] == nc - 1][0]
            vals[last] = 0.0                               # (n-1, n_c-1)
        m = _sp.coo_matrix((vals, (rows, cols)), shape=(nf, nc)).tocsr()
        m.sort_indices()
        Ps.append(CSR(nf, nc, m.indptr, m.indices, m.data))
    n = sizes[-1]
    h = 1.0 / (n - 1)
    rows, cols, vals = [0, n - 1], [0, n - 1], [1.0, 1.0]
    for i in range(1, n - 1):
        rows += [i, i, i]
        cols += [i - 1, i, i + 1]
        vals += [-1.0 / h, 2.0 / h, -1.0 / h]
    H = CSR.from_scipy(_sp.csr_matrix((vals, (rows, cols)), shape=(n, n)))
    g = np.full(n, -10.0 * h)
    g[0] = g[-1] = 0.0
    return H, g, np.full(n, lower), np.full(n, upper), Ps
