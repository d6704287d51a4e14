// Deformable-mirror influence-function projection, FP32 path.
//
// dm.coefs setter (OOPAO/DeformableMirror.py:651-686): OPD = modes @ coefs with
// modes [n_pix, n_act] and coefs [n_act] or [n_act, B].  Here the IF matrix is
// stored transposed, modes_t [n_act][n_pix], so that a warp reads consecutive
// pixels of one actuator, and the output is batch-major opd [B][n_pix] (each
// batch item a contiguous res x res map, the layout the pyramid passes read).
//
// batch <= 8: one thread per pixel accumulates all batch columns (GEMV-like,
// bound by reading modes_t once); coefficients are staged through shared
// memory in chunks.  batch > 8: 64x64 register-tiled SGEMM.
#include "common.cuh"

namespace {

constexpr int kGemvThreads = 256;
constexpr int kGemvChunk = 512;  // actuators staged per pass

template <int NB>
__global__ void __launch_bounds__(kGemvThreads) dm_gemv(const float* __restrict__ modes_t,
                                                        const float* __restrict__ coefs, int n_act,
                                                        int n_pix, int batch, float scale,
                                                        float* __restrict__ opd,
                                                        const float* __restrict__ base) {
  __shared__ float cs[kGemvChunk * NB];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  float acc[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) acc[b] = 0.f;
  for (int a0 = 0; a0 < n_act; a0 += kGemvChunk) {
    const int na = min(kGemvChunk, n_act - a0);
    __syncthreads();
    for (int t = threadIdx.x; t < na * NB; t += blockDim.x) {
      const int a = t / NB, b = t % NB;
      cs[t] = (b < batch) ? coefs[(size_t)(a0 + a) * batch + b] : 0.f;
    }
    __syncthreads();
    if (p < n_pix) {
      const float* m = modes_t + (size_t)a0 * n_pix + p;
      for (int a = 0; a < na; a++) {
        const float v = __ldg(m + (size_t)a * n_pix);
#pragma unroll
        for (int b = 0; b < NB; b++) acc[b] = fmaf(v, cs[a * NB + b], acc[b]);
      }
    }
  }
  if (p < n_pix) {
#pragma unroll
    for (int b = 0; b < NB; b++)
      if (b < batch) opd[(size_t)b * n_pix + p] = acc[b] * scale + (base ? base[(size_t)b * n_pix + p] : 0.f);
  }
}

constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) dm_gemm(const float* __restrict__ modes_t,
                                               const float* __restrict__ coefs, int n_act, int n_pix,
                                               int batch, float scale, float* __restrict__ opd,
                                               const float* __restrict__ base) {
  __shared__ float As[BK][BM];  // coefs[a][b]
  __shared__ float Bs[BK][BN];  // modes_t[a][p]
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int b0 = blockIdx.y * BM, p0 = blockIdx.x * BN;
  float acc[4][4] = {};
  for (int a0 = 0; a0 < n_act; a0 += BK) {
    for (int t = threadIdx.x; t < BK * BM; t += 256) {
      const int kk = t / BM, m = t % BM;
      const int a = a0 + kk, b = b0 + m;
      As[kk][m] = (a < n_act && b < batch) ? coefs[(size_t)a * batch + b] : 0.f;
    }
    for (int t = threadIdx.x; t < BK * BN; t += 256) {
      const int kk = t / BN, nn = t % BN;
      const int a = a0 + kk, p = p0 + nn;
      Bs[kk][nn] = (a < n_act && p < n_pix) ? modes_t[(size_t)a * n_pix + p] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      float af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; i++) af[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) bf[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(af[i], bf[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int b = b0 + ty * 4 + i;
    if (b >= batch) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int p = p0 + tx * 4 + j;
      if (p < n_pix)
        opd[(size_t)b * n_pix + p] = acc[i][j] * scale + (base ? base[(size_t)b * n_pix + p] : 0.f);
    }
  }
}

// Adjoint of the projection: out[a][b] = scale * sum_p modes_t[a][p] g[b][p].
// One CTA per (actuator, group of 8 batch columns); fixed-order block
// reduction, so the result is deterministic.
constexpr int kVjpCols = 8;

__global__ void __launch_bounds__(256) dm_vjp(const float* __restrict__ modes_t, const float* __restrict__ g,
                                              int n_act, int n_pix, int batch, float scale,
                                              float* __restrict__ out) {
  __shared__ float red[kVjpCols][8];
  const int a = blockIdx.x, b0 = blockIdx.y * kVjpCols;
  const float* m = modes_t + (size_t)a * n_pix;
  float acc[kVjpCols];
#pragma unroll
  for (int c = 0; c < kVjpCols; c++) acc[c] = 0.f;
  for (int p = threadIdx.x; p < n_pix; p += blockDim.x) {
    const float v = m[p];
#pragma unroll
    for (int c = 0; c < kVjpCols; c++)
      if (b0 + c < batch) acc[c] = fmaf(v, g[(size_t)(b0 + c) * n_pix + p], acc[c]);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < kVjpCols; c++) {
    float s = acc[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) red[c][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < kVjpCols && b0 + (int)threadIdx.x < batch) {
    float s = 0.f;
    for (int i = 0; i < 8; i++) s += red[threadIdx.x][i];
    out[(size_t)a * batch + b0 + threadIdx.x] = s * scale;
  }
}

}  // namespace

extern "C" int oopao_dm_vjp_f32(const float* modes_t, const float* g, int n_act, int n_pix, int batch, float scale,
                                float* out, void* stream) {
  OOPAO_CHECK_ARG(modes_t && g && out, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && batch > 0, "sizes must be positive");
  dim3 grid(n_act, ceil_div(batch, kVjpCols));
  dm_vjp<<<grid, 256, 0, (cudaStream_t)stream>>>(modes_t, g, n_act, n_pix, batch, scale, out);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_dm_opd_acc_f32(const float* modes_t, const float* coefs, int n_act, int n_pix, int batch,
                                    float scale, const float* base, float* opd, void* stream) {
  OOPAO_CHECK_ARG(modes_t && coefs && opd, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && batch > 0, "sizes must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const int g = ceil_div(n_pix, kGemvThreads);
  if (batch == 1) {
    dm_gemv<1><<<g, kGemvThreads, 0, st>>>(modes_t, coefs, n_act, n_pix, batch, scale, opd, base);
  } else if (batch <= 4) {
    dm_gemv<4><<<g, kGemvThreads, 0, st>>>(modes_t, coefs, n_act, n_pix, batch, scale, opd, base);
  } else if (batch <= 8) {
    dm_gemv<8><<<g, kGemvThreads, 0, st>>>(modes_t, coefs, n_act, n_pix, batch, scale, opd, base);
  } else {
    dim3 grid(ceil_div(n_pix, BN), ceil_div(batch, BM));
    dm_gemm<<<grid, 256, 0, st>>>(modes_t, coefs, n_act, n_pix, batch, scale, opd, base);
  }
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_dm_opd_f32(const float* modes_t, const float* coefs, int n_act, int n_pix,
                                int batch, float scale, float* opd, void* stream) {
  return oopao_dm_opd_acc_f32(modes_t, coefs, n_act, n_pix, batch, scale, nullptr, opd, stream);
}
