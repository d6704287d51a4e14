// Infinite-phase-screen atmosphere on the GPU (frozen flow with ring
// extrusion), the per-step part of OOPAO/Atmosphere.py updateLayer / add_row
// (:410-531) and fill_OPD_support (:589-622) for an on-axis source.
//
// Every layer keeps its phase map (radians, float64, n x n with n = res + 6)
// in two ping-pong buffers.  The host precomputes, for every step, the
// integer one-pixel moves of each layer (the reference's add_row calls, at
// most `slots` per step) and the sub-pixel offset left in its buffer, and
// draws the extrusion normals from each layer's RandomState; the kernels read
// the entries of the step held in a device counter, so the same launches
// serve eager updates and a captured CUDA graph.
//
//   atm_boil     boiling (apply_boiling :387-408): map = alpha map + beta phi
//                for the layers that boil, before the step's moves
//   atm_shift    one add_row slot: interior one-pixel move (or plain copy
//                when the slot is idle), map[s%2] -> map[(s+1)%2]
//   atm_extrude  the new outer ring X = A Z + B w (float64), Z = the inner
//                ring of the moved interior
//   atm_minmax   value range of each map (the clip of the cubic warp)
//   atm_opd      bicubic (Keys, a = -0.5) sub-pixel shift of every layer,
//                clipped, cropped to the pupil footprint, scaled by
//                lambda/2pi * sqrt(fractional r0) and summed -> OPD [res][res]
#include <cfloat>

#include "common.cuh"

namespace {

struct AtmEntry {
  int active, dx, dy, normal;  // move (dx, dy) of the slot; row of its normals
};

__device__ __forceinline__ int atm_step(const int* step, int n_steps, int* err) {
  const int t = *step;
  if (t < 0 || t >= n_steps) {
    if (err) atomicExch(err, 1);
    return -1;
  }
  return t;
}

__global__ void atm_shift(const double* __restrict__ src, double* __restrict__ dst, const AtmEntry* __restrict__ sched,
                          const int* step, int n_steps, int slots, int slot, int n_layers, int n, int* err) {
  const int l = blockIdx.y;
  const int t = atm_step(step, n_steps, err);
  const size_t nn = (size_t)n * n;
  const double* s = src + l * nn;
  double* d = dst + l * nn;
  AtmEntry e{0, 0, 0, 0};
  if (t >= 0) e = sched[((size_t)t * n_layers + l) * slots + slot];
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n), x = (int)(i % n);
    const bool interior = y > 0 && y < n - 1 && x > 0 && x < n - 1;
    if (e.active && interior) {
      // output (y, x) reads input (y - dy, x - dx): one-pixel translation
      d[i] = s[(size_t)(y - e.dy) * n + (x - e.dx)];
    } else {
      d[i] = s[i];
    }
  }
}

// one warp per ring pixel: X[o] = sum_i A[o][i] Z[i] + sum_j B[o][j] w[j]
__global__ void atm_extrude(double* __restrict__ map, const double* __restrict__ A, const double* __restrict__ B,
                            const int* __restrict__ inner_idx, const int* __restrict__ outer_idx,
                            const double* __restrict__ normals, const AtmEntry* __restrict__ sched, const int* step,
                            int n_steps, int slots, int slot, int n_layers, int n, int n_inner, int n_outer,
                            int* err) {
  extern __shared__ double z[];
  const int l = blockIdx.y;
  const int t = atm_step(step, n_steps, err);
  if (t < 0) return;
  const AtmEntry e = sched[((size_t)t * n_layers + l) * slots + slot];
  if (!e.active) return;
  double* m = map + (size_t)l * n * n;
  for (int i = threadIdx.x; i < n_inner; i += blockDim.x) z[i] = m[inner_idx[i]];
  __syncthreads();
  const double* w = normals + (size_t)e.normal * n_outer;
  const int warps = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int o = blockIdx.x * warps + (threadIdx.x >> 5); o < n_outer; o += gridDim.x * warps) {
    const double* a = A + (size_t)o * n_inner;
    const double* b = B + (size_t)o * n_outer;
    double acc = 0.0;
    for (int i = lane; i < n_inner; i += 32) acc = fma(a[i], z[i], acc);
    for (int j = lane; j < n_outer; j += 32) acc = fma(b[j], w[j], acc);
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
    if (lane == 0) m[outer_idx[o]] = acc;
  }
}

constexpr int kRangeBlocks = 32;  // partial value ranges per layer

// Float32 mirror of each map (what the OPD interpolation reads; the maps
// themselves stay float64 for the extrusion) and its partial value ranges:
// block b of layer l covers a contiguous chunk; range[l][b] = (min, max) of
// the float32 values, which is the float32 rounding of the float64 range.
// One float64 -> float32 conversion per pixel here replaces sixteen per
// output pixel and layer in the interpolation.
__global__ void atm_minmax(const double* __restrict__ map, float* __restrict__ mirror, double* __restrict__ range,
                           int n) {
  __shared__ float lo_s[32], hi_s[32];
  const int l = blockIdx.y, b = blockIdx.x;
  const double* m = map + (size_t)l * n * n;
  float* mf = mirror + (size_t)l * n * n;
  const int nn = n * n, chunk = (nn + gridDim.x - 1) / gridDim.x;
  const int i0 = b * chunk, i1 = min(nn, i0 + chunk);
  float lo = FLT_MAX, hi = -FLT_MAX;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const float v = (float)m[i];
    mf[i] = v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  for (int s = 16; s > 0; s >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, s));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, s));
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    lo_s[wid] = lo;
    hi_s[wid] = hi;
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    lo = lane < nw ? lo_s[lane] : FLT_MAX;
    hi = lane < nw ? hi_s[lane] : -FLT_MAX;
    for (int s = 16; s > 0; s >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, s));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, s));
    }
    if (lane == 0) {
      range[((size_t)l * gridDim.x + b) * 2] = lo;
      range[((size_t)l * gridDim.x + b) * 2 + 1] = hi;
    }
  }
}

// Weights of the Keys cubic convolution (a = -0.5) at offset x in [0, 1):
// f1 + x/2 (f2 - f0 + x (2 f0 - 5 f1 + 4 f2 - f3 + x (3 (f1 - f2) + f3 - f0)))
__device__ __forceinline__ void keys_weights(float x, float* w) {
  const float x2 = x * x, x3 = x2 * x;
  w[0] = 0.5f * (-x + 2.f * x2 - x3);
  w[1] = 1.f + 0.5f * (-5.f * x2 + 3.f * x3);
  w[2] = 0.5f * (x + 4.f * x2 - 3.f * x3);
  w[3] = 0.5f * (-x2 + x3);
}

__device__ __forceinline__ float map_at(const float* m, int n, int r, int c) {
  return (r >= 0 && r < n && c >= 0 && c < n) ? m[(size_t)r * n + c] : 0.f;
}

constexpr int kMaxAtmLayers = 64;

// The sub-pixel offset is the same for every pixel of a layer, so the
// per-layer integer base, separable weights and value range are set up once
// per block in shared memory; each pixel is then 16 loads and FP32 FMAs per
// layer (the interpolated values are rounded to float32 like the output).
__global__ void atm_opd(const float* __restrict__ mirror, const double* __restrict__ range,
                        const double2* __restrict__ buff, const int* step, int n_steps, int use_buff,
                        const double* __restrict__ scale, int n_layers, int n, int res, int off, float* __restrict__ opd,
                        int* err) {
  __shared__ float wr_s[kMaxAtmLayers][4], wc_s[kMaxAtmLayers][4], lo_s[kMaxAtmLayers], hi_s[kMaxAtmLayers],
      sc_s[kMaxAtmLayers];
  __shared__ int dr_s[kMaxAtmLayers], dc_s[kMaxAtmLayers];
  int t = -1;
  if (use_buff) {
    t = atm_step(step, n_steps, err);
    if (t < 0) return;
  }
  for (int l = threadIdx.x; l < n_layers; l += blockDim.x) {
    double tx = 0.0, ty = 0.0;
    if (use_buff) {
      const double2 b = buff[(size_t)t * n_layers + l];
      tx = b.x;
      ty = b.y;
    }
    // output pixel (r, c) of the warped map reads (r - ty, c - tx)
    const double fr = floor(-ty), fc = floor(-tx);
    dr_s[l] = (int)fr;
    dc_s[l] = (int)fc;
    keys_weights((float)(-ty - fr), wr_s[l]);
    keys_weights((float)(-tx - fc), wc_s[l]);
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (int b = 0; b < kRangeBlocks; b++) {
      lo = fminf(lo, (float)range[((size_t)l * kRangeBlocks + b) * 2]);
      hi = fmaxf(hi, (float)range[((size_t)l * kRangeBlocks + b) * 2 + 1]);
    }
    lo_s[l] = lo;
    hi_s[l] = hi;
    sc_s[l] = (float)scale[l];
  }
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= res * res) return;
  const int y = p / res, x = p % res;
  float acc = 0.f;
  for (int l = 0; l < n_layers; l++) {
    const float* m = mirror + (size_t)l * n * n;
    // the OPD crop starts `off` pixels into the map
    const int r0 = y + off + dr_s[l], c0 = x + off + dc_s[l];
    float v = 0.f;
#pragma unroll
    for (int pr = 0; pr < 4; pr++) {
      const int r = r0 + pr - 1;
      const float row = wc_s[l][0] * map_at(m, n, r, c0 - 1) + wc_s[l][1] * map_at(m, n, r, c0) +
                        wc_s[l][2] * map_at(m, n, r, c0 + 1) + wc_s[l][3] * map_at(m, n, r, c0 + 2);
      v = fmaf(wr_s[l][pr], row, v);
    }
    v = fminf(fmaxf(v, lo_s[l]), hi_s[l]);
    acc = fmaf(v, sc_s[l], acc);
  }
  opd[p] = acc;
}

struct AtmBoil {
  int layer[kMaxAtmLayers];  // map of boiling layer k
  double alpha[kMaxAtmLayers], beta[kMaxAtmLayers];
};

// Boiling (AR(1) decorrelation) of the maps before the step's moves:
// map_l = alpha_k map_l + beta_k phi[t][k] for the k-th boiling layer.  The
// products and the sum are rounded separately (no fused multiply-add), as
// the float64 host arithmetic of the same update.
__global__ void atm_boil(double* __restrict__ maps, const double* __restrict__ phi, AtmBoil b, const int* step,
                         int n_steps, int n_boil, int n, int* err) {
  int t = 0;
  if (step != nullptr) {
    t = atm_step(step, n_steps, err);
    if (t < 0) return;
  }
  const int k = blockIdx.y;
  const size_t nn = (size_t)n * n;
  double* m = maps + (size_t)b.layer[k] * nn;
  const double* f = phi + ((size_t)t * n_boil + k) * nn;
  const double a = b.alpha[k], c = b.beta[k];
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (size_t)gridDim.x * blockDim.x)
    m[i] = __dadd_rn(__dmul_rn(a, m[i]), __dmul_rn(c, f[i]));
}

__global__ void atm_advance(int* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

}  // namespace

extern "C" int oopao_atm_update(double* maps, float* mirror, int n_layers, int n, int slots, const void* sched,
                                const double* buff, int n_steps, const double* A, const double* B, const int* inner_idx,
                                const int* outer_idx, int n_inner, int n_outer, const double* normals,
                                double* range, const double* scale, int res, float* opd, int* step, int advance,
                                int* err, void* stream) {
  OOPAO_CHECK_ARG(maps && mirror && scale && opd && step && range, "NULL argument");
  OOPAO_CHECK_ARG(n_layers > 0 && n_layers <= kMaxAtmLayers && n >= 8 && res > 0 && res <= n - 6 && slots >= 0 &&
                      slots % 2 == 0,
                  "bad sizes (1 to 64 layers, n >= res + 6, an even number of slots)");
  OOPAO_CHECK_ARG(slots == 0 || (sched && A && B && inner_idx && outer_idx && normals && n_inner > 0 && n_outer > 0),
                  "moving layers need the schedule, A, B, ring indices and normals");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t nn = (size_t)n * n;
  const AtmEntry* e = reinterpret_cast<const AtmEntry*>(sched);
  double* buf[2] = {maps, maps + (size_t)n_layers * nn};
  int launches = 0;
  for (int s = 0; s < slots; s++) {
    const dim3 g1((unsigned)ceil_div((int)nn, 256), n_layers);
    atm_shift<<<g1, 256, 0, st>>>(buf[s & 1], buf[(s + 1) & 1], e, step, n_steps, slots, s, n_layers, n, err);
    const dim3 g2((unsigned)ceil_div(n_outer, 8), n_layers);
    atm_extrude<<<g2, 256, sizeof(double) * n_inner, st>>>(buf[(s + 1) & 1], A, B, inner_idx, outer_idx, normals, e,
                                                          step, n_steps, slots, s, n_layers, n, n_inner, n_outer,
                                                          err);
    launches += 2;
  }
  atm_minmax<<<dim3(kRangeBlocks, n_layers), 256, 0, st>>>(maps, mirror, range, n);
  const int off = (n - res) / 2;  // crop of the warped map: [1:-1] then the pupil footprint
  atm_opd<<<ceil_div(res * res, 256), 256, 0, st>>>(mirror, range, reinterpret_cast<const double2*>(buff), step,
                                                   n_steps, buff != nullptr ? 1 : 0, scale, n_layers, n, res, off,
                                                   opd, err);
  launches += 2;
  if (advance) {
    atm_advance<<<1, 32, 0, st>>>(step);
    launches += 1;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_atm_boil(double* maps, int n_layers, int n, const double* phi, int n_boil, const int* layers,
                              const double* alpha, const double* beta, const int* step, int n_steps, int* err,
                              void* stream) {
  OOPAO_CHECK_ARG(maps && phi && layers && alpha && beta, "NULL argument");
  OOPAO_CHECK_ARG(n_layers > 0 && n_layers <= kMaxAtmLayers && n >= 8 && n_boil >= 1 && n_boil <= n_layers,
                  "bad sizes (1 to 64 layers, 1 to n_layers boiling layers)");
  OOPAO_CHECK_ARG(step != nullptr ? n_steps >= 1 : n_steps == 1,
                  "a table of steps needs the device step counter; without it the table holds one step");
  AtmBoil b{};
  for (int k = 0; k < n_boil; k++) {
    OOPAO_CHECK_ARG(layers[k] >= 0 && layers[k] < n_layers && (k == 0 || layers[k] > layers[k - 1]),
                    "boiling layers must be distinct, increasing and below n_layers");
    b.layer[k] = layers[k];
    b.alpha[k] = alpha[k];
    b.beta[k] = beta[k];
  }
  const size_t nn = (size_t)n * n;
  const dim3 g((unsigned)ceil_div((int)nn, 256), n_boil);
  atm_boil<<<g, 256, 0, (cudaStream_t)stream>>>(maps, phi, b, step, n_steps, n_boil, n, err);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
