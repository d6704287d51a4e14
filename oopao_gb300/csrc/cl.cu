// Closed-loop step kernels (tutorials/AO_closed_loop_Pyramid_WFS.py:601-639,
// OOPAO/closed_loop/run_cl.py:176-217): turbulence OPD of the step, DM shape
// added to it, reconstructor MVM + integrator, residual wavefront RMS.
//
// A device step counter drives the time index, so a CUDA graph capturing one
// step replays every later step without host involvement: the screen kernel
// reads the counter, the integrator kernel advances it.
#include <cooperative_groups.h>

#include "common.cuh"

namespace {

struct ScreenLayer {
  const float* screen;  // [h][w] OPD (m), periodic
  int h, w;
  float y0, x0;         // position of pupil pixel (0,0) at step 0 (pixels)
  float vy, vx;         // displacement per step (pixels)
};

constexpr int kMaxLayers = 35;

struct ScreenArgs {
  ScreenLayer layer[kMaxLayers];
  int n_layers, res;
  const int* step;
  float* opd;  // [res][res]
};

__device__ __forceinline__ int wrap(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// Frozen flow: each layer is translated by (vy, vx) pixels per step and
// sampled bilinearly (periodic screens); layers are summed.
__global__ void cl_screen(ScreenArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.res * a.res) return;
  const int i = p / a.res, j = p - (p / a.res) * a.res;
  const float t = (float)(*a.step);
  float s = 0.f;
  for (int q = 0; q < a.n_layers; q++) {
    const ScreenLayer& L = a.layer[q];
    const float y = L.y0 + i + L.vy * t, x = L.x0 + j + L.vx * t;
    const float fy = floorf(y), fx = floorf(x);
    const float dy = y - fy, dx = x - fx;
    const int y0 = wrap((int)fy, L.h), x0 = wrap((int)fx, L.w);
    const int y1 = wrap(y0 + 1, L.h), x1 = wrap(x0 + 1, L.w);
    const float v00 = L.screen[(size_t)y0 * L.w + x0], v01 = L.screen[(size_t)y0 * L.w + x1];
    const float v10 = L.screen[(size_t)y1 * L.w + x0], v11 = L.screen[(size_t)y1 * L.w + x1];
    s += (1.f - dy) * ((1.f - dx) * v00 + dx * v01) + dy * ((1.f - dx) * v10 + dx * v11);
  }
  a.opd[p] = s;
}

// coefs[a] -= gain * sum_j R[a][j] s[j].  Four warps per actuator, each over
// an interleaved quarter of the signals; block 0 thread 0 advances the step
// counter.
constexpr int kIntActPerBlock = 2;  // 256 threads = 2 actuators x 4 warps

// One lane's share of row . s (the 128 lanes of an actuator interleave).
// VEC4: 16-byte loads (row and s 16-byte aligned, n_sig % 4 == 0), four of
// each in flight, so a 2.5k-signal row is read in about one round trip;
// otherwise eight scalar loads in flight.
template <bool VEC4>
__device__ __forceinline__ float row_dot_part(const float* __restrict__ r, const float* __restrict__ s, int n_sig,
                                              int lane128) {
  float acc = 0.f;
  if constexpr (VEC4) {
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const float4* s4 = reinterpret_cast<const float4*>(s);
    const int n4 = n_sig >> 2;
    int j = lane128;
    for (; j + 3 * 128 < n4; j += 4 * 128) {
      float4 rv[4], sv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        rv[u] = r4[j + u * 128];
        sv[u] = s4[j + u * 128];
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        acc = fmaf(rv[u].x, sv[u].x, acc);
        acc = fmaf(rv[u].y, sv[u].y, acc);
        acc = fmaf(rv[u].z, sv[u].z, acc);
        acc = fmaf(rv[u].w, sv[u].w, acc);
      }
    }
    for (; j < n4; j += 128) {
      const float4 rv = r4[j], sv = s4[j];
      acc = fmaf(rv.x, sv.x, acc);
      acc = fmaf(rv.y, sv.y, acc);
      acc = fmaf(rv.z, sv.z, acc);
      acc = fmaf(rv.w, sv.w, acc);
    }
  } else {
    int j = lane128;
    for (; j + 7 * 128 < n_sig; j += 8 * 128) {
      float rv[8], sv[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        rv[u] = r[j + u * 128];
        sv[u] = s[j + u * 128];
      }
#pragma unroll
      for (int u = 0; u < 8; u++) acc = fmaf(rv[u], sv[u], acc);
    }
    for (; j < n_sig; j += 128) acc = fmaf(r[j], s[j], acc);
  }
  return acc;
}

template <bool VEC4>
__global__ void __launch_bounds__(256) cl_integrate(const float* __restrict__ R, const float* __restrict__ s,
                                                    int n_act, int n_sig, float gain, float* __restrict__ coefs,
                                                    int* step) {
  __shared__ float red[8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int act = blockIdx.x * kIntActPerBlock + (w >> 2), part = w & 3;
  float acc = 0.f;
  if (act < n_act) acc = row_dot_part<VEC4>(R + (size_t)act * n_sig, s, n_sig, part * 32 + lane);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[w] = acc;
  __syncthreads();
  if (threadIdx.x < kIntActPerBlock) {
    const int a = blockIdx.x * kIntActPerBlock + threadIdx.x;
    if (a < n_act) {
      const float* q = red + 4 * threadIdx.x;
      coefs[a] -= gain * ((q[0] + q[1]) + (q[2] + q[3]));
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && step) *step += 1;
}

// Modal commands with optical-gain compensation (the GSC tutorial,
// tutorials/AO_closed_loop_Pyramid_WFS_GSC.py: M2C @ diag(1/og) @ M @ s):
// y[m] = (M[m] . s) / og[m] from step og_start on (og = 1 before).  Same
// layout and load pattern as cl_integrate.
template <bool VEC4>
__global__ void __launch_bounds__(256) cl_modal(const float* __restrict__ M, const float* __restrict__ s,
                                                int n_modes, int n_sig, const double* __restrict__ og, int og_start,
                                                const int* __restrict__ step, float* __restrict__ y) {
  __shared__ float red[8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mode = blockIdx.x * kIntActPerBlock + (w >> 2), part = w & 3;
  float acc = 0.f;
  if (mode < n_modes) acc = row_dot_part<VEC4>(M + (size_t)mode * n_sig, s, n_sig, part * 32 + lane);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[w] = acc;
  __syncthreads();
  if (threadIdx.x < kIntActPerBlock) {
    const int m = blockIdx.x * kIntActPerBlock + threadIdx.x;
    if (m < n_modes) {
      const float* q = red + 4 * threadIdx.x;
      const float v = (q[0] + q[1]) + (q[2] + q[3]);
      const bool comp = og != nullptr && (step == nullptr || *step >= og_start);
      y[m] = comp ? v / (float)og[m] : v;
    }
  }
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// Sum over the CTA (blockDim.x = 1024) of one float per thread.
__device__ float cta_sum_1024(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    float t = red[l];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) red[32] = t;
  }
  __syncthreads();
  const float r = red[32];
  __syncthreads();
  return r;
}

// RMS of (opd - mean) over the pupil pixels idx[0..npup) -> out[*step].
// A cluster of kRmsCtas CTAs splits the pixels into contiguous chunks; each
// CTA takes its chunk's mean and sum of squared deviations in two passes with
// compensated float32 sums (float64 is a narrow pipe on this part, and the
// two-pass form avoids the cancellation of sum(v^2)/n - mean^2).  CTA 0 then
// reads the chunk results through distributed shared memory and merges them
// in rank order (Chan et al.: M2 = sum M2_c + sum n_c (mean_c - mean)^2).
constexpr int kRmsCtas = 8;

__global__ void __cluster_dims__(kRmsCtas, 1, 1) __launch_bounds__(1024)
    cl_pupil_rms(const float* __restrict__ opd, const int* __restrict__ idx, int npup, const int* step, float* out,
                 int out_len) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ float red[33];
  __shared__ float part[3];  // n, mean, M2 of this CTA's chunk
  const int rank = (int)cluster.block_rank();
  const int chunk = (npup + kRmsCtas - 1) / kRmsCtas;
  const int i0 = rank * chunk, i1 = min(npup, i0 + chunk);
  const int cnt = max(0, i1 - i0);
  float s = 0.f, c = 0.f;
  for (int i = i0 + threadIdx.x; i < i1; i += 1024) kahan_add(s, c, opd[idx[i]]);
  const float chunk_sum = cta_sum_1024(s, red);
  const float mean = cnt > 0 ? chunk_sum / (float)cnt : 0.f;
  float q = 0.f, cq = 0.f;
  for (int i = i0 + threadIdx.x; i < i1; i += 1024) {
    const float d = opd[idx[i]] - mean;
    kahan_add(q, cq, d * d);
  }
  const float m2 = cta_sum_1024(q, red);
  if (threadIdx.x == 0) {
    part[0] = (float)cnt;
    part[1] = mean;
    part[2] = m2;
  }
  cluster.sync();
  if (rank == 0 && threadIdx.x == 0) {
    float n_r[kRmsCtas], mean_r[kRmsCtas], m2_r[kRmsCtas];
    float tot = 0.f, sum = 0.f;
    for (int r = 0; r < kRmsCtas; r++) {
      const float* pr = cluster.map_shared_rank(part, r);
      n_r[r] = pr[0];
      mean_r[r] = pr[1];
      m2_r[r] = pr[2];
      tot += n_r[r];
      sum += n_r[r] * mean_r[r];
    }
    const float mu = sum / tot;
    float m2t = 0.f;
    for (int r = 0; r < kRmsCtas; r++) {
      const float d = mean_r[r] - mu;
      m2t += m2_r[r] + n_r[r] * d * d;
    }
    const int t = step ? *step : 0;
    if (t >= 0 && t < out_len) out[t] = sqrtf(m2t / tot);
  }
  cluster.sync();  // the other CTAs' shared memory stays alive until CTA 0 has read it
}

}  // namespace

extern "C" int oopao_cl_screen(int n_layers, const float* const* screens, const int* heights, const int* widths,
                               const float* y0, const float* x0, const float* vy, const float* vx, int res,
                               const int* step, float* opd, void* stream) {
  OOPAO_CHECK_ARG(n_layers >= 1 && n_layers <= kMaxLayers, "1 to 35 layers");
  OOPAO_CHECK_ARG(screens && heights && widths && y0 && x0 && vy && vx && step && opd, "NULL argument");
  ScreenArgs a;
  a.n_layers = n_layers;
  a.res = res;
  a.step = step;
  a.opd = opd;
  for (int q = 0; q < n_layers; q++) {
    OOPAO_CHECK_ARG(screens[q] && heights[q] > 1 && widths[q] > 1, "bad layer");
    a.layer[q] = ScreenLayer{screens[q], heights[q], widths[q], y0[q], x0[q], vy[q], vx[q]};
  }
  cl_screen<<<ceil_div(res * res, 256), 256, 0, (cudaStream_t)stream>>>(a);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

namespace {
// 16-byte loads of every row of a row-major [rows][n_sig] matrix and of s.
bool vec4_ok(const float* m, const float* s, int n_sig) {
  return n_sig % 4 == 0 && reinterpret_cast<uintptr_t>(m) % 16 == 0 && reinterpret_cast<uintptr_t>(s) % 16 == 0;
}
}  // namespace

extern "C" int oopao_cl_integrate(const float* R, const float* s, int n_act, int n_sig, float gain, float* coefs,
                                  int* step, void* stream) {
  OOPAO_CHECK_ARG(R && s && coefs, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_sig > 0, "sizes must be positive");
  const int g = ceil_div(n_act, kIntActPerBlock);
  if (vec4_ok(R, s, n_sig))
    cl_integrate<true><<<g, 256, 0, (cudaStream_t)stream>>>(R, s, n_act, n_sig, gain, coefs, step);
  else
    cl_integrate<false><<<g, 256, 0, (cudaStream_t)stream>>>(R, s, n_act, n_sig, gain, coefs, step);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_cl_modal(const float* M, const float* s, int n_modes, int n_sig, const double* og,
                              int og_start, const int* step, float* y, void* stream) {
  OOPAO_CHECK_ARG(M && s && y, "NULL argument");
  OOPAO_CHECK_ARG(n_modes > 0 && n_sig > 0, "sizes must be positive");
  const int g = ceil_div(n_modes, kIntActPerBlock);
  if (vec4_ok(M, s, n_sig))
    cl_modal<true><<<g, 256, 0, (cudaStream_t)stream>>>(M, s, n_modes, n_sig, og, og_start, step, y);
  else
    cl_modal<false><<<g, 256, 0, (cudaStream_t)stream>>>(M, s, n_modes, n_sig, og, og_start, step, y);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_cl_pupil_rms(const float* opd, const int* idx, int npup, const int* step, float* out,
                                  int out_len, void* stream) {
  OOPAO_CHECK_ARG(opd && idx && out && npup > 0, "bad argument");
  cl_pupil_rms<<<kRmsCtas, 1024, 0, (cudaStream_t)stream>>>(opd, idx, npup, step, out, out_len);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
