"""TEST INFRASTRUCTURE ONLY: numpy / scipy.sparse restatement of the projected
operators of the reduced model.  Used by tests/ as the checker of the GPU
build (plume_reduced_build_products, include/plume_reduced.h), never by the
product.

Follows src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:
  buildOutOfCoreMatrices        (1355-1490)  which operator meets which bases;
  buildFlatA                    (2162-2200)  peeled 7-point Poisson matrix:
                                diagonal = number of non-obstacle face
                                neighbours, -1 to each interior neighbour;
  computeVelocityToDivergence   (1989-2107)  peeled divergence, with the
                                one-sided / mirrored rows at the faces chosen
                                by the wall flags (entries accumulate with +=);
  buildPeeledDampingMatrixFlat  (2112-2157)  (1 - w) on the diagonal, w / 6 to
                                each interior neighbour, w = 0.9;
  computePressureToVelocity     (627-695)    peeled gradient, one-sided at the
                                first and last interior index;
and src/linearalgebra:
  SPARSE_MATRIX_ARRAY::projectVerySparse (SPARSE_MATRIX_ARRAY.cpp:76-123)
                                final(y, x) = sum left(col, y) M(row, col)
                                right(row, x), i.e. left^T M^T right;
  SPARSE_MATRIX::project        (SPARSE_MATRIX.cpp:447-471)  left^T (M right);
  EIGEN::transposeProduct       (EIGEN.cpp:463-472)          left^T right.
The wall obstacles are FLUID_3D_MIC's constructor's (FLUID_3D_MIC.cpp:121-158):
a face slab is an obstacle when its flag is 1.  Flags: (front, back, left,
right, top, bottom) = (z low, z high, x low, x high, y high, y low).
Parity of this restatement is pinned to the reference's own constructor
(oracle/_ref/reduced_ref) through tests/golden/ref_reduced_*.npz and
ref_products_mixed_10x12x8.npz.
"""
import numpy as np
import scipy.sparse as sp


def _peeled(res):
    X, Y, Z = (int(v) for v in res)
    return X - 2, Y - 2, Z - 2


def _coords(res):
    nx, ny, nz = _peeled(res)
    i = np.arange(nx * ny * nz)
    return i, i % nx, (i // nx) % ny, i // (nx * ny)


def flat_a(res, bc):
    """buildFlatA on the wall obstacles of `bc`: N_int x N_int."""
    nx, ny, nz = _peeled(res)
    i, x, y, z = _coords(res)
    front, back, left, right, top, bottom = (int(b) for b in bc)
    diag = np.full(i.size, 6.0)
    diag -= (x == 0) * (left == 1) + (x == nx - 1) * (right == 1)
    diag -= (y == 0) * (bottom == 1) + (y == ny - 1) * (top == 1)
    diag -= (z == 0) * (front == 1) + (z == nz - 1) * (back == 1)
    rows, cols, vals = [i], [i], [diag]
    for ok, step in ((x != 0, -1), (x != nx - 1, 1), (y != 0, -nx), (y != ny - 1, nx),
                     (z != 0, -nx * ny), (z != nz - 1, nx * ny)):
        rows.append(i[ok])
        cols.append(i[ok] + step)
        vals.append(np.full(int(ok.sum()), -1.0))
    n = i.size
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def velocity_to_divergence(res, bc, dx):
    """computeVelocityToDivergence: N_int x 3 N_int (duplicates summed, as
    the reference's += does)."""
    nx, ny, nz = _peeled(res)
    i, x, y, z = _coords(res)
    front, back, left, right, top, bottom = (int(b) for b in bc)
    coeff = -dx * 0.5
    rows, cols, vals = [], [], []

    def add(mask, col, v):
        rows.append(i[mask])
        cols.append(col[mask])
        vals.append(np.full(int(mask.sum()), v))

    for comp, pos, n_axis, step, hi_bc, lo_bc in ((0, x, nx, 1, right, left), (1, y, ny, nx, top, bottom),
                                                    (2, z, nz, nx * ny, back, front)):
        hi, lo = pos == n_axis - 1, pos == 0
        # the high-side term
        add(~hi, 3 * (i + step) + comp, coeff)
        if hi_bc != 0:
            add(hi, 3 * i + comp, -coeff)
        else:
            add(hi, 3 * (i - step) + comp, coeff)
        # the low-side term
        add(~lo, 3 * (i - step) + comp, -coeff)
        if lo_bc != 0:
            add(lo, 3 * i + comp, coeff)
        else:
            add(lo, 3 * (i + step) + comp, -coeff)
    n = i.size
    m = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, 3 * n))
    return m.tocsr()  # sums duplicates


def damping(res, w=0.9):
    """buildPeeledDampingMatrixFlat: 3 N_int x 3 N_int."""
    nx, ny, nz = _peeled(res)
    i, x, y, z = _coords(res)
    sixth = (1.0 / 6.0) * w
    rows, cols, vals = [], [], []
    for c in range(3):
        r = 3 * i + c
        rows.append(r)
        cols.append(r)
        vals.append(np.full(i.size, 1.0 - w))
        for ok, step in ((x != nx - 1, 1), (x != 0, -1), (y != ny - 1, nx), (y != 0, -nx),
                         (z != nz - 1, nx * ny), (z != 0, -nx * ny)):
            rows.append(r[ok])
            cols.append(3 * (i[ok] + step) + c)
            vals.append(np.full(int(ok.sum()), sixth))
    n = 3 * i.size
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def pressure_to_velocity(res, dx):
    """computePressureToVelocity: 3 N_int x N_int."""
    nx, ny, nz = _peeled(res)
    i, x, y, z = _coords(res)
    inv, half = 1.0 / dx, 0.5 / dx
    rows, cols, vals = [], [], []
    for comp, pos, n_axis, step in ((0, x, nx, 1), (1, y, ny, nx), (2, z, nz, nx * ny)):
        first, last = pos == 0, pos == n_axis - 1
        mid = ~first & ~last
        for mask, (c1, v1), (c2, v2) in ((first, (step, -inv), (0, inv)),
                                         (last & ~first, (0, -inv), (-step, inv)),
                                         (mid, (step, -half), (-step, half))):
            for off, v in ((c1, v1), (c2, v2)):
                rows.append(3 * i[mask] + comp)
                cols.append(i[mask] + off)
                vals.append(np.full(int(mask.sum()), v))
    n = i.size
    m = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(3 * n, n))
    return m.tocsr()


def products(res, bc, Up, Upp, Upd, Uf):
    """buildOutOfCoreMatrices: dict of the six projected operators, keyed by
    their file names without `.matrix`."""
    dx = 1.0 / max(int(v) for v in res)
    A = flat_a(res, bc)
    Ar = Up.T @ (A.T @ Up)
    vtod = Up.T @ (velocity_to_divergence(res, bc, dx) @ Upp)
    damp = Upp.T @ (damping(res).T @ Upd)
    ptof = Uf.T @ Upp
    ptov = Uf.T @ (pressure_to_velocity(res, dx) @ Up)
    inverse = np.linalg.inv(Ar)
    return {"projected.A": Ar, "projected.vtod": vtod, "damping.peeled": damp, "projected.ptof": ptof,
            "projected.ptov": ptov, "inverseProduct": (ptov @ inverse) @ vtod}
