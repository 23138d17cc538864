// matrix_file.cuh -- the reference's dense matrix files on the host and their
// column-major copies in HBM, shared by reduced.cu and products.cu.
//
// EIGEN::read / EIGEN::write (src/linearalgebra/EIGEN.cpp:195-213, 294-310):
// int32 rows, int32 cols, then rows x cols doubles row by row.  On the device
// a basis is column-major (column k of an n-row basis at U + k n), so that a
// warp reading one column reads consecutive rows.
#ifndef PLUME_MATRIX_FILE_CUH
#define PLUME_MATRIX_FILE_CUH

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/plume.h"

namespace plume {
namespace matrix_file {
namespace {

bool read_matrix_file(FILE* f, int& rows, int& cols, std::vector<double>& data) {
  bool ok = fread(&rows, sizeof(int), 1, f) == 1 && fread(&cols, sizeof(int), 1, f) == 1 && rows >= 0 && cols >= 0;
  if (ok) {
    data.resize((size_t)rows * cols);
    ok = fread(data.data(), sizeof(double), data.size(), f) == data.size();
  }
  return ok;
}

bool read_matrix(const std::string& path, int& rows, int& cols, std::vector<double>& data) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  const bool ok = read_matrix_file(f, rows, cols, data);
  fclose(f);
  return ok;
}

// The (rows, cols) header alone.
bool read_matrix_dims(const std::string& path, int& rows, int& cols) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  const bool ok = fread(&rows, sizeof(int), 1, f) == 1 && fread(&cols, sizeof(int), 1, f) == 1;
  fclose(f);
  return ok;
}

bool write_matrix_file(FILE* f, int rows, int cols, const double* data) {
  return fwrite(&rows, sizeof(int), 1, f) == 1 && fwrite(&cols, sizeof(int), 1, f) == 1 &&
         fwrite(data, sizeof(double), (size_t)rows * cols, f) == (size_t)rows * cols;
}

// A column-major rows x cols matrix to its file (row by row).
bool write_matrix_colmajor(const std::string& path, int rows, int cols, const double* cm) {
  std::vector<double> rm((size_t)rows * cols);
  for (int i = 0; i < rows; i++)
    for (int j = 0; j < cols; j++) rm[(size_t)i * cols + j] = cm[(size_t)j * rows + i];
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const bool ok = write_matrix_file(f, rows, cols, rm.data());
  return fclose(f) == 0 && ok;
}

template <typename Ptr>
cudaError_t upload(Ptr*& dst, const std::vector<Ptr>& src) {
  cudaError_t e = cudaMalloc(&dst, std::max<size_t>(1, src.size()) * sizeof(Ptr));
  if (e == cudaSuccess && !src.empty())
    e = cudaMemcpy(dst, src.data(), src.size() * sizeof(Ptr), cudaMemcpyHostToDevice);
  return e;
}

// row-major (rows x cols) -> column-major, 32 x 32 tiles
__global__ void k_transpose(const double* in, size_t rows, int cols, double* out) {
  __shared__ double tile[32][33];
  const size_t r0 = (size_t)blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const size_t r = r0 + dy;
    const int c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[dy][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int c = c0 + dy;
    const size_t r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][dy];
  }
}

// An n x r row-major basis from its file, to the device as column-major.
int upload_basis(const std::string& path, size_t n_expected, double*& dst, int& cols, std::string& err) {
  int rows = 0;
  std::vector<double> h;
  if (!read_matrix(path, rows, cols, h)) {
    err = "could not read " + path;
    return PLUME_ERR_IO;
  }
  if ((size_t)rows != n_expected) {
    err = path + " does not match the grid (" + std::to_string(rows) + " rows, expected " +
          std::to_string(n_expected) + ")";
    return PLUME_ERR_IO;
  }
  double* tmp = nullptr;
  if (cudaMalloc(&tmp, std::max<size_t>(1, h.size()) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dst, std::max<size_t>(1, h.size()) * sizeof(double)) != cudaSuccess) {
    if (tmp) cudaFree(tmp);
    err = "basis does not fit on the device";
    return PLUME_ERR_OOM;
  }
  int rc = PLUME_OK;
  if (!h.empty()) {
    if (cudaMemcpy(tmp, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = PLUME_ERR_CUDA;
    if (rc == PLUME_OK) {
      const dim3 grid((unsigned)((n_expected + 31) / 32), (unsigned)((cols + 31) / 32));
      k_transpose<<<grid, dim3(32, 8)>>>(tmp, n_expected, cols, dst);
      if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = PLUME_ERR_CUDA;
    }
  }
  cudaFree(tmp);
  if (rc != PLUME_OK) err = "basis upload failed";
  return rc;
}

}  // namespace
}  // namespace matrix_file
}  // namespace plume

#endif  // PLUME_MATRIX_FILE_CUH
