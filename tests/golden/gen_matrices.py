"""Synthetic sparse systems for the solve phase (numpy implementation).

These stand in for the SuiteSparse matrices the reference's run scripts use
(Matrix/README.md:3-13), which are not shipped.  Every generator returns an FP64
CSR matrix (rptr, cind, val) with rows in natural (x fastest) order and columns
sorted inside each row, Dirichlet boundaries (neighbours outside the grid are
dropped).  The product's C++ generators (sc23-ad_gb300/csrc/host/generators.cpp)
build the same arrays; tests/test_generators.py checks that they agree.

Random numbers come from splitmix64 so that the C++ and numpy versions draw the
same stream: u = (z >> 11) * 2^-53 in [0, 1).
"""
import numpy as np

_M64 = (1 << 64) - 1


def splitmix64(seed, n):
    """n outputs of splitmix64 started at `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, n):
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _assemble(n_rows, rows, cols, vals):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rptr = np.zeros(n_rows + 1, dtype=np.int32)
    np.add.at(rptr, rows + 1, 1)
    rptr = np.cumsum(rptr).astype(np.int32)
    return rptr, cols.astype(np.int32), vals.astype(np.float64)


def _stencil(dims, offsets, coef_fn):
    """Generic structured-grid assembly. coef_fn(idx_grid, off) -> value array or scalar."""
    shape = tuple(dims)
    N = int(np.prod(shape))
    grid = np.indices(shape[::-1]).reshape(len(shape), -1)[::-1]  # grid[0] = x (fastest)
    rows_l, cols_l, vals_l = [], [], []
    strides = [1]
    for d in dims[:-1]:
        strides.append(strides[-1] * d)
    row_ids = np.arange(N, dtype=np.int64)
    for off in offsets:
        ok = np.ones(N, dtype=bool)
        col = row_ids.copy()
        for ax, o in enumerate(off):
            c = grid[ax] + o
            ok &= (c >= 0) & (c < dims[ax])
            col = col + o * strides[ax]
        v = coef_fn(off)
        v = np.broadcast_to(np.asarray(v, dtype=np.float64), (N,))
        rows_l.append(row_ids[ok])
        cols_l.append(col[ok])
        vals_l.append(v[ok])
    return _assemble(N, np.concatenate(rows_l), np.concatenate(cols_l), np.concatenate(vals_l))


def poisson2d(n):
    """5-point Laplacian on an n x n grid: 4 on the diagonal, -1 off it."""
    offs = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)]
    return _stencil([n, n], offs, lambda o: 4.0 if o == (0, 0) else -1.0)


def poisson3d(n):
    """7-point Laplacian on an n^3 grid: 6 on the diagonal, -1 off it."""
    offs = [(0, 0, 0)] + [tuple(int(a == ax) * s for a in range(3)) for ax in range(3) for s in (1, -1)]
    return _stencil([n, n, n], offs, lambda o: 6.0 if o == (0, 0, 0) else -1.0)


def aniso2d(n, eps):
    """5-point anisotropic diffusion: -u_xx - eps*u_yy."""
    offs = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)]

    def c(o):
        if o == (0, 0):
            return 2.0 + 2.0 * eps
        return -1.0 if o[1] == 0 else -eps
    return _stencil([n, n], offs, c)


def stencil27(n, seed):
    """27-point SPD stencil: off-diagonals -1, diagonal 26 + delta, delta ~ U[0.1, 1] per row."""
    N = n ** 3
    delta = 0.1 + 0.9 * uniform01(seed, N)
    offs = [(a, b, c) for c in (-1, 0, 1) for b in (-1, 0, 1) for a in (-1, 0, 1)]
    return _stencil([n, n, n], offs, lambda o: (26.0 + delta) if o == (0, 0, 0) else -1.0)


def convdiff3d(n, pe):
    """Upwinded convection-diffusion -lap(u) + beta.grad(u), beta = pe*(1,1,1)/sqrt(3),
    unit cube, h = 1/(n+1), scaled by h^2: diagonal 6 + h*|beta|_1, the upwind
    (minus-side) neighbour of each axis gets -1 - h*beta_axis, the other -1."""
    h = 1.0 / (n + 1)
    b = pe / np.sqrt(3.0)
    offs = [(0, 0, 0)] + [tuple(int(a == ax) * s for a in range(3)) for ax in range(3) for s in (1, -1)]

    def c(o):
        if o == (0, 0, 0):
            return 6.0 + 3.0 * h * b
        return (-1.0 - h * b) if sum(o) < 0 else -1.0
    return _stencil([n, n, n], offs, c)


def varcoef3d(n, sigma, seed):
    """7-point variable-coefficient diffusion: cell coefficients k = exp(sigma*z),
    z ~ N(0,1) (Box-Muller on splitmix64 uniforms), face coefficient the harmonic
    mean 2 k1 k2 / (k1 + k2); boundary faces use the cell's own k.  The diagonal
    is the sum of the row's face coefficients, off-diagonals are minus the face
    coefficient."""
    N = n ** 3
    u1 = uniform01(seed, N)
    u2 = uniform01(seed + 1, N)
    z = np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(2.0 * np.pi * u2)
    k = np.exp(sigma * z)
    grid = np.indices((n, n, n)).reshape(3, -1)[::-1]
    rows_l, cols_l, vals_l = [], [], []
    diag = np.zeros(N)
    ids = np.arange(N)
    strides = [1, n, n * n]
    for ax in range(3):
        for s in (1, -1):
            c = grid[ax] + s
            ok = (c >= 0) & (c < n)
            nb = ids + s * strides[ax]
            kf = np.where(ok, 2.0 * k * k[np.where(ok, nb, ids)] / (k + k[np.where(ok, nb, ids)]), k)
            diag += kf
            rows_l.append(ids[ok]); cols_l.append(nb[ok]); vals_l.append(-kf[ok])
    rows_l.append(ids); cols_l.append(ids); vals_l.append(diag)
    return _assemble(N, np.concatenate(rows_l), np.concatenate(cols_l), np.concatenate(vals_l))


def spmv(rptr, cind, val, x):
    """Row-sequential FP64 CSR product (the order of matrix/spmat.hpp:43-52)."""
    N = len(rptr) - 1
    y = np.zeros(N)
    for i in range(N):
        s = 0.0
        for j in range(rptr[i], rptr[i + 1]):
            s += val[j] * x[cind[j]]
        y[i] = s
    return y


def rhs(rptr, cind, val, seed):
    """x* ~ U[-1, 1] from splitmix64(seed) and b = A x* (FP64, row order)."""
    N = len(rptr) - 1
    xs = uniform01(seed, N) * 2.0 - 1.0
    # vectorised row-order sum: accumulate column slot by slot (same order as a
    # sequential loop over each row because slots are visited left to right)
    lens = np.diff(rptr)
    y = np.zeros(N)
    for k in range(int(lens.max())):
        has = lens > k
        idx = rptr[:-1][has] + k
        y[has] = y[has] + val[idx] * xs[cind[idx]]
    return xs, y


def write_mtx(path, rptr, cind, val):
    N = len(rptr) - 1
    rows = np.repeat(np.arange(N), np.diff(rptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{N} {N} {len(val)}\n")
        lines = [f"{r + 1} {c + 1} {v:.17g}\n" for r, c, v in zip(rows, cind, val)]
        f.write("".join(lines))
