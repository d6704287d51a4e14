// Deformable-mirror projection for separable influence functions.
//
// The reference's Gaussian IF (OOPAO/DeformableMirror.py:572-600) with no
// anamorphosis angle is exp(-a (X-x0)^2) * exp(-c (Y-y0)^2), and on a
// Cartesian actuator grid (no rotation) x0 takes one of nx values and y0 one
// of ny.  Then
//
//   opd[b][y][x] = sum_a coefs[a][b] * modes[y*res+x][a]
//                = sum_j gy[j][y] * T[b][j][x],   T[b][j][x] = sum_i C_b[j][i] gx[i][x]
//
// with C_b[j][i] the coefficient of the actuator in grid cell (j, i) (zero
// where the grid has no valid actuator).  Two small contractions replace the
// dense product over res^2 x n_act: 2*ny*res*(nx + res) flops per frame
// instead of 2*res^2*n_act, and the factors (nx + ny) x res floats stay in L2.
#include "common.cuh"

namespace {

constexpr int kSepThreads = 256;

// T[b][j][x] = sum_i C_b[j][i] gx[i][x]; one CTA per (grid row j, item b).
__global__ void __launch_bounds__(kSepThreads) dm_sep_rows(const float* __restrict__ gx,
                                                           const int* __restrict__ grid_act,
                                                           const float* __restrict__ coefs, int n_act, int nx,
                                                           int ny, int res, int batch, float* __restrict__ t) {
  extern __shared__ float crow[];  // [nx]
  const int j = blockIdx.x, b = blockIdx.y;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const int a = grid_act[j * nx + i];
    crow[i] = (a >= 0 && a < n_act) ? coefs[(size_t)a * batch + b] : 0.f;
  }
  __syncthreads();
  float* out = t + ((size_t)b * ny + j) * res;
  for (int x = threadIdx.x; x < res; x += blockDim.x) {
    float acc = 0.f;
    for (int i = 0; i < nx; i++) acc = fmaf(crow[i], __ldg(gx + (size_t)i * res + x), acc);
    out[x] = acc;
  }
}

// opd[b][y][x] = scale * sum_j gy[j][y] T[b][j][x] (+ base); one CTA per (row y, item b).
__global__ void __launch_bounds__(kSepThreads) dm_sep_cols(const float* __restrict__ gy,
                                                           const float* __restrict__ t, int ny, int res,
                                                           float scale, const float* __restrict__ base,
                                                           float* __restrict__ opd) {
  extern __shared__ float gcol[];  // [ny]
  const int y = blockIdx.x, b = blockIdx.y;
  for (int j = threadIdx.x; j < ny; j += blockDim.x) gcol[j] = gy[(size_t)j * res + y];
  __syncthreads();
  const float* tb = t + (size_t)b * ny * res;
  const size_t row = ((size_t)b * res + y) * res;
  for (int x = threadIdx.x; x < res; x += blockDim.x) {
    float acc = 0.f;
    for (int j = 0; j < ny; j++) acc = fmaf(gcol[j], tb[(size_t)j * res + x], acc);
    opd[row + x] = acc * scale + (base ? base[row + x] : 0.f);
  }
}

}  // namespace

extern "C" size_t oopao_dm_sep_workspace_bytes(int ny, int res, int batch) {
  if (ny < 1 || res < 1 || batch < 1) return 0;
  return sizeof(float) * (size_t)batch * ny * res;
}

extern "C" int oopao_dm_opd_sep_f32(const float* gx, const float* gy, const int* grid_act, int nx, int ny,
                                    const float* coefs, int n_act, int res, int batch, float scale,
                                    const float* base, float* opd, void* ws, size_t ws_bytes, void* stream) {
  OOPAO_CHECK_ARG(gx && gy && grid_act && coefs && opd && ws, "NULL argument");
  OOPAO_CHECK_ARG(nx > 0 && ny > 0 && n_act > 0 && res > 0 && batch > 0, "sizes must be positive");
  OOPAO_CHECK_ARG(nx <= 8192 && ny <= 8192, "grid larger than 8192 actuators per side");
  OOPAO_CHECK_ARG(ws_bytes >= oopao_dm_sep_workspace_bytes(ny, res, batch), "workspace too small");
  OOPAO_CHECK_ARG(batch <= 65535, "batch larger than 65535");
  cudaStream_t st = (cudaStream_t)stream;
  float* t = (float*)ws;
  dm_sep_rows<<<dim3(ny, batch), kSepThreads, sizeof(float) * nx, st>>>(gx, grid_act, coefs, n_act, nx, ny, res,
                                                                         batch, t);
  dm_sep_cols<<<dim3(res, batch), kSepThreads, sizeof(float) * ny, st>>>(gy, t, ny, res, scale, base, opd);
  oopao_count_launches(2);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
