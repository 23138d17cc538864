/*
 * plume_svd.h -- the snapshot SVD of the reduced-model pipeline on the GPU.
 *
 * Replaces, for a C / ctypes caller:
 *   src/linearalgebra/BIG_MATRIX.cpp:100-259   outOfCoreQR  (modified Gram-Schmidt
 *                                               of the snapshot columns)
 *   src/linearalgebra/BIG_MATRIX.cpp:264-436   outOfCoreSVD (SVD of R, PCA values,
 *                                               kept columns, U = Q U_R)
 *   src/linearalgebra/BIG_MATRIX.cpp:613-647   writeFinalU
 *   projects/svdOutOfCoreMultiple/svdOutOfCoreMultiple.cpp:87-177  the stage
 *                                               (binary bin/svdOutOfCoreMultiple)
 *
 * Input: the stream files that appendStreams writes (<prefix>.dims = int32 rows,
 * cols; <prefix>.transpose = rows snapshots of cols doubles each).  The snapshot
 * matrix A has n = cols rows and m = rows columns; it is held whole in HBM (the
 * reference streams blocks of it through host memory because its host had
 * 92 GB), factored A = Q R by modified Gram-Schmidt in FP64, R = U_R S V^T by a
 * one-sided Jacobi SVD in FP64, and U = Q U_R[:, :kept] is formed by a tiled
 * FP64 GEMM.  PCA values are S^2; columns are kept while S_k^2 / S_0^2 is not
 * below the discard threshold (the reference's loop, BIG_MATRIX.cpp:320-326).
 *
 * Outputs, in the reference's formats:
 *   u_path: int32 rows, int32 cols, then rows x cols doubles row by row
 *           (writeFinalU; read by EIGEN::read);
 *   <scratch><stream name>.singularValues.vector: int32 size, then the PCA
 *           values (VECTOR::write, BIG_MATRIX.cpp:331-339, with the
 *           reference's file-name rule);
 *   pca_path: the same PCA vector (the reference copies a scratch file that
 *           nothing writes and so leaves it empty; here it holds the values).
 * Singular vectors are unique up to sign: a column of U may have the opposite
 * sign of the reference's (Eigen's JacobiSVD picks its own).
 */
#ifndef PLUME_SVD_H
#define PLUME_SVD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plume_svd_info {
  int32_t rows;    /* n: values per snapshot                                  */
  int32_t cols;    /* m: snapshots                                            */
  int32_t kept;    /* columns of U written                                    */
  int32_t sweeps;  /* Jacobi sweeps until no pair needed a rotation           */
  double ms_qr;    /* device time of the Gram-Schmidt QR                      */
  double ms_svd;   /* device time of the SVD of R                             */
  double ms_u;     /* device time of U = Q U_R                                */
  double ms_io;    /* host time reading the stream and writing U              */
} plume_svd_info;

/* BIG_MATRIX::outOfCoreSVD(prefix, reduced_path, threshold) followed by
   writeFinalU(u_path) and the PCA copy to pca_path (NULL: not written).
   reduced_path only feeds the reference's name rule for the singular-value
   file under scratch_path.  Returns a plume_status; the text of a failure is
   plume_last_error(NULL). */
int plume_svd_stream(const char* prefix, const char* reduced_path, const char* scratch_path,
                     double discard_threshold, const char* u_path, const char* pca_path,
                     int32_t device, plume_svd_info* info);

/* The same factorisation on snapshots already in host memory: `columns` holds
   m columns of n doubles (column j at columns + j n).  pca (m doubles) gets
   the PCA values S^2 in decreasing order; u (n x m doubles, may be NULL) gets
   U = Q U_R with the kept columns first, column-major (column k at u + k n),
   *kept their count.  Columns past *kept are left untouched. */
int plume_svd_columns(const double* columns, int32_t n, int32_t m, double discard_threshold,
                      int32_t device, double* pca, double* u, int32_t* kept,
                      plume_svd_info* info);

/* verifyResults (svdOutOfCoreMultiple.cpp:59-79): for each of the first
   `count` columns c of the stream, |c - U U^T c| with U the file at u_path
   (EIGEN::read layout), computed on the GPU.  diffs: count doubles. */
int plume_svd_verify(const char* prefix, const char* u_path, int32_t count, int32_t device,
                     double* diffs);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_SVD_H */
