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

// Both contractions in one launch for grids whose operands fit in shared
// memory.  A CTA owns kSepTile columns x kSepRows rows of the OPD.  It first
// issues every global load it needs at once (the gathered coefficient grid
// C_b, the kSepTile columns of gx and the kSepRows columns of gy), then forms
// the kSepTile columns of T and the output block from shared memory, so its
// path holds about two memory round trips.  The projection is ~2.5 MFLOP per
// 240 x 240 frame; latency, not arithmetic, sets its time.
constexpr int kSepTile = 16;
constexpr int kSepRows = 64;
constexpr int kSepPerThread = kSepRows * kSepTile / 256;  // 4 rows per thread

__host__ __device__ constexpr size_t sep_fused_floats(int nx, int ny) {
  return (size_t)nx * ny + (size_t)nx * kSepTile + (size_t)ny * kSepRows + (size_t)ny * kSepTile;
}
constexpr size_t kSepFusedFloats = 24576;  // 96 KB of dynamic shared memory

__global__ void __launch_bounds__(256) dm_sep_fused(const float* __restrict__ gx, const float* __restrict__ gy,
                                                    const int* __restrict__ grid_act,
                                                    const float* __restrict__ coefs, int n_act, int nx, int ny,
                                                    int res, int batch, float scale,
                                                    const float* __restrict__ base, float* __restrict__ opd) {
  extern __shared__ float sm[];
  float* cm = sm;                          // [ny][nx]   C_b
  float* gxb = cm + nx * ny;               // [nx][kSepTile]
  float* gyb = gxb + nx * kSepTile;        // [ny][kSepRows]
  float* tb = gyb + ny * kSepRows;         // [ny][kSepTile]
  const int x0 = blockIdx.x * kSepTile, y0 = blockIdx.y * kSepRows, b = blockIdx.z;
  const int tid = threadIdx.x;
#pragma unroll 4
  for (int e = tid; e < nx * ny; e += 256) {
    const int a = grid_act[e];
    cm[e] = (a >= 0 && a < n_act) ? coefs[(size_t)a * batch + b] : 0.f;
  }
#pragma unroll 4
  for (int e = tid; e < nx * kSepTile; e += 256) {
    const int x = x0 + e % kSepTile;
    gxb[e] = x < res ? __ldg(gx + (size_t)(e / kSepTile) * res + x) : 0.f;
  }
#pragma unroll 4
  for (int e = tid; e < ny * kSepRows; e += 256) {
    const int y = y0 + e % kSepRows;
    gyb[e] = y < res ? __ldg(gy + (size_t)(e / kSepRows) * res + y) : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < ny * kSepTile; e += 256) {
    const int j = e / kSepTile, xx = e % kSepTile;
    float acc = 0.f;
    for (int i = 0; i < nx; i++) acc = fmaf(cm[j * nx + i], gxb[i * kSepTile + xx], acc);
    tb[e] = acc;
  }
  __syncthreads();
  const int xx = tid % kSepTile, r0 = tid / kSepTile, x = x0 + xx;
  float acc[kSepPerThread];
#pragma unroll
  for (int k = 0; k < kSepPerThread; k++) acc[k] = 0.f;
  for (int j = 0; j < ny; j++) {
    const float t = tb[j * kSepTile + xx];
#pragma unroll
    for (int k = 0; k < kSepPerThread; k++) acc[k] = fmaf(gyb[j * kSepRows + r0 + 16 * k], t, acc[k]);
  }
  if (x < res) {
#pragma unroll
    for (int k = 0; k < kSepPerThread; k++) {
      const int y = y0 + r0 + 16 * k;
      if (y < res) {
        const size_t o = ((size_t)b * res + y) * res + x;
        opd[o] = acc[k] * scale + (base ? base[o] : 0.f);
      }
    }
  }
}

// Second contraction for large batches: opd[b] = scale * Gy^T T[b] (+ base),
// a register-tiled FP32 GEMM per item (M = N = res, K = ny).  A CTA owns a
// 64 x 64 block of one item's OPD; each of its 256 threads accumulates a
// 4 x 4 sub-block (rows 4*ty.., columns 4*tx..) from float4 reads of the
// 16-deep shared-memory slices of Gy (as [k][y]) and T[b] (as [k][x]).
constexpr int kTileM = 64, kTileN = 64, kTileK = 16;

__global__ void __launch_bounds__(256) dm_sep_cols_tiled(const float* __restrict__ gy, const float* __restrict__ t,
                                                         int ny, int res, float scale,
                                                         const float* __restrict__ base, float* __restrict__ opd) {
  __shared__ __align__(16) float as[kTileK][kTileM];  // gy[k0 + k][y0 + m]
  __shared__ __align__(16) float bs[kTileK][kTileN];  // T[b][k0 + k][x0 + n]
  const int b = blockIdx.z, y0 = blockIdx.y * kTileM, x0 = blockIdx.x * kTileN;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const float* tb = t + (size_t)b * ny * res;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < ny; k0 += kTileK) {
#pragma unroll
    for (int r = 0; r < kTileK * kTileM / 256; r++) {
      const int e = tid + 256 * r, k = e / kTileM, m = e % kTileM;
      const int kk = k0 + k, y = y0 + m, x = x0 + m;
      as[k][m] = (kk < ny && y < res) ? __ldg(gy + (size_t)kk * res + y) : 0.f;
      bs[k][m] = (kk < ny && x < res) ? tb[(size_t)kk * res + x] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kTileK; k++) {
      const float4 a = *reinterpret_cast<const float4*>(&as[k][4 * ty]);
      const float4 c = *reinterpret_cast<const float4*>(&bs[k][4 * tx]);
      const float av[4] = {a.x, a.y, a.z, a.w}, cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], cv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int y = y0 + 4 * ty + i;
    if (y >= res) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int x = x0 + 4 * tx + j;
      if (x < res) {
        const size_t o = ((size_t)b * res + y) * res + x;
        opd[o] = acc[i][j] * scale + (base ? base[o] : 0.f);
      }
    }
  }
}

// Batches from this size on take the two launches (T, then the tiled
// GEMM): measured on GB300 the fused kernel, which recomputes T per row
// block, wins below it.
constexpr int kSepTiledMinBatch = 16;

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
  if (batch >= kSepTiledMinBatch) {
    float* t = (float*)ws;
    dm_sep_rows<<<dim3(ny, batch), kSepThreads, sizeof(float) * nx, st>>>(gx, grid_act, coefs, n_act, nx, ny, res,
                                                                           batch, t);
    dm_sep_cols_tiled<<<dim3(ceil_div(res, kTileN), ceil_div(res, kTileM), batch), 256, 0, st>>>(gy, t, ny, res, scale,
                                                                                               base, opd);
    oopao_count_launches(2);
    OOPAO_CUDA_TRY(cudaGetLastError());
    return OOPAO_OK;
  }
  if (sep_fused_floats(nx, ny) <= kSepFusedFloats) {
    const dim3 grid(ceil_div(res, kSepTile), ceil_div(res, kSepRows), batch);
    const size_t smem = sizeof(float) * sep_fused_floats(nx, ny);
    if (smem > 48 * 1024)
      OOPAO_CUDA_TRY(cudaFuncSetAttribute(dm_sep_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dm_sep_fused<<<grid, 256, smem, st>>>(gx, gy, grid_act, coefs, n_act, nx, ny, res, batch, scale, base, opd);
    oopao_count_launches(1);
    OOPAO_CUDA_TRY(cudaGetLastError());
    return OOPAO_OK;
  }
  float* t = (float*)ws;
  dm_sep_rows<<<dim3(ny, batch), kSepThreads, sizeof(float) * nx, st>>>(gx, grid_act, coefs, n_act, nx, ny, res,
                                                                         batch, t);
  dm_sep_cols<<<dim3(res, batch), kSepThreads, sizeof(float) * ny, st>>>(gy, t, ny, res, scale, base, opd);
  oopao_count_launches(2);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
