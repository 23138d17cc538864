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

#include "plume.h"

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

/* ---- snapshots kept in HBM: the streams without the disk round trip ----
 * A plume_snapshots object collects, from one plume handle, the rows that
 * FLUID_3D_MIC::appendStreams (FLUID_3D_MIC.cpp:1329-1477) would append to
 * one stream file -- the peeled field (interior cells, x fastest, vector
 * components interleaved), kept only when its 2-norm exceeds 1e-7 -- as
 * FP64 columns of a device matrix, and factors them in place with the same
 * SVD as plume_svd_stream. */
typedef enum plume_stream {
  PLUME_STREAM_FINAL = 0,   /* velocity            (velocity.final.matrix)      */
  PLUME_STREAM_PREPROJECT,  /* preprojection       (velocity.preproject.matrix) */
  PLUME_STREAM_PREDIFFUSE,  /* prediffusion        (velocity.prediffuse.matrix) */
  PLUME_STREAM_PREADVECT,   /* preadvection        (velocity.preadvect.matrix)  */
  PLUME_STREAM_IOP,         /* postIOP             (velocity.iop.matrix)        */
  PLUME_STREAM_PRESSURE     /* pressure, then divergence (pressure.matrix)      */
} plume_stream;

typedef struct plume_snapshots plume_snapshots;

/* Room for `capacity` rows of the handle's `stream` on the handle's device.
   The handle must outlive the object. */
int plume_snapshots_create(plume_handle* h, int32_t stream, int32_t capacity, plume_snapshots** out);
void plume_snapshots_destroy(plume_snapshots* s);
/* Appends this step's rows (waits for the handle's stream); *appended = rows
   kept (0..2).  PLUME_ERR_STATE when the field is not kept or the capacity is
   reached. */
int plume_snapshots_append(plume_snapshots* s, int32_t* appended);
/* rows = snapshots held, cols = values per snapshot (the stream's dims). */
int plume_snapshots_dims(plume_snapshots* s, int32_t* rows, int32_t* cols);
/* The held rows in the stream file's layout (rows * cols doubles). */
int plume_snapshots_download(plume_snapshots* s, double* dst, size_t n);
/* BIG_MATRIX::outOfCoreSVD + writeFinalU on the held rows, which it consumes
   (the matrix becomes Q; the object is empty afterwards).  u_path / pca_path
   may be NULL (not written); pca (rows doubles) and kept may be NULL. */
int plume_snapshots_svd(plume_snapshots* s, double discard_threshold, const char* u_path,
                        const char* pca_path, double* pca, int32_t* kept, plume_svd_info* info);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_SVD_H */
