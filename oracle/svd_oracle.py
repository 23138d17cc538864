"""TEST INFRASTRUCTURE ONLY: numpy restatement of the reference's snapshot SVD
(svdOutOfCoreMultiple).  Used by tests/ as the checker of the GPU path
(include/plume_svd.h), never by the product.

Follows src/linearalgebra/BIG_MATRIX.cpp:
  outOfCoreQR  (100-259)  modified Gram-Schmidt, column by column: norm, scale,
                          then R(i, j) = q_i . a_j and a_j -= R(i, j) q_i for
                          every later column j (the block structure of the
                          reference only streams columns; the arithmetic is
                          this sequence);
  outOfCoreSVD (264-436)  SVD of R (the reference calls Eigen's JacobiSVD; here
                          LAPACK through numpy: the same singular values and,
                          up to sign, vectors), PCA values S^2, the kept count
                          (first ratio below the threshold stops it), and
                          U = Q U_R[:, :kept];
  writeFinalU  (613-647)  int32 rows, cols, then U row by row.
Parity of this restatement is pinned to the reference's own program
(oracle/_ref/svd_ref, built by `make -C oracle ref`) through the fixtures of
tests/golden/make_golden.py.
"""
import numpy as np


def read_stream(prefix):
    """(A, rows, cols): the snapshot matrix (n x m, one snapshot per column) of
    <prefix>.dims / <prefix>.transpose."""
    rows, cols = np.fromfile(prefix + ".dims", dtype="<i4")[:2]
    data = np.fromfile(prefix + ".transpose", dtype="<f8", count=int(rows) * int(cols))
    return data.reshape(int(rows), int(cols)).T.copy(), int(rows), int(cols)


def mgs(A):
    """BIG_MATRIX::outOfCoreQR on an in-memory A: (Q, R)."""
    A = np.array(A, dtype=np.float64, copy=True)
    m = A.shape[1]
    R = np.zeros((m, m))
    for i in range(m):
        norm = np.sqrt(A[:, i] @ A[:, i])
        R[i, i] = norm
        A[:, i] *= 1.0 / norm
        if i + 1 < m:
            dots = A[:, i] @ A[:, i + 1:]
            R[i, i + 1:] = dots
            A[:, i + 1:] -= np.outer(A[:, i], dots)
    return A, R


def kept_columns(pca, threshold):
    keep = 0
    for v in pca:
        if v / pca[0] < threshold:
            break
        keep += 1
    return keep


def svd_stream(A, threshold=1e-9):
    """(pca values, kept, U) of BIG_MATRIX::outOfCoreSVD for A."""
    Q, R = mgs(A)
    UR, S, _ = np.linalg.svd(R)
    pca = S * S
    keep = kept_columns(pca, threshold)
    return pca, keep, Q @ UR[:, :keep]


def read_u(path):
    """EIGEN::read layout of writeFinalU: int32 rows, cols, row-major doubles."""
    hdr = np.fromfile(path, dtype="<i4", count=2)
    rows, cols = int(hdr[0]), int(hdr[1])
    return np.fromfile(path, dtype="<f8", offset=8, count=rows * cols).reshape(rows, cols)


def read_vector(path):
    """VECTOR::write layout: int32 size, then doubles."""
    n = int(np.fromfile(path, dtype="<i4", count=1)[0])
    return np.fromfile(path, dtype="<f8", offset=4, count=n)


def align_signs(U, ref):
    """U with each column's sign flipped to agree with ref's (singular vectors
    are unique up to sign)."""
    s = np.sign(np.sum(U * ref, axis=0))
    s[s == 0] = 1.0
    return U * s
