// Modulated pyramid WFS propagation on GB300 (sm_103a).
//
// Per modulation point k the reference computes (OOPAO/Pyramid.py:612-646)
//     E_k = A * exp(i (phi + TT_k))          placed at rows/cols [off, off+res)
//     F_k = fft2(E_k * phasor)               N x N
//     G_k = ifft2(F_k * mask)
//     raw = sum_k |G_k|^2                    (:741-751)
// and the camera sums raw over N/cam x N/cam blocks (:1178-1203).
//
// The phasor exp(-i pi (N+1)/N (x+y)) and the modulation tilt
// x_k*Tip + y_k*Tilt are both separable in (row, col), so E_k*phasor =
// A e^{i phi} * rowfac_k[col] * colfac_k[row].  The 2-D transforms are split
// into three fused passes over shared-memory line FFTs (fft.cuh):
//   pass 1 (rows_fwd):  build the field for `res` non-zero rows, forward
//                       row FFT, store Y[b,k] (res x N).
//   pass 2 (cols):      per column: gather the res non-zero entries, forward
//                       FFT, multiply the mask column, inverse FFT, store
//                       Z[b,k] (N x N).
//   pass 3 (rows_inv):  per row: inverse FFT of Z rows for a range of points,
//                       accumulate |.|^2 over them, store a partial sum.
//   pass 4 (bin):       sum the partials, bin N/cam x N/cam -> camera frame,
//                       optionally write raw_data.
// The 1/N^2 of numpy's ifft2 is folded into rowfac.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft.cuh"

namespace {

constexpr int kThreads = 256;
constexpr size_t kSmemLimit = 227 * 1024;
// Measured on GB300: passes small enough to keep the intermediates in L2
// (<= 128 MiB) lose to large passes streaming through HBM, because the
// per-pass launch gaps and the small grids cost more than the DRAM traffic
// at these sizes (the passes are issue-bound, not bandwidth-bound).
constexpr size_t kDefaultPassBudget = 4ull << 30;

}  // namespace

// Per-kernel CUDA-event timing of oopao_pwfs_measure (bench instrumentation):
// a start/end event pair on the launching stream around every launch, tagged
// with its stage (0 rows, 1 columns, 2 row inverse, 3 reduce/bin).
struct PwfsProfile {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  std::vector<int> stage;  // stage id of each start/end pair
  size_t used = 0;
  bool open = false;
  cudaEvent_t next() {
    if (used == pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      pool.push_back(e);
    }
    return pool[used++];
  }
  // called twice per launch: before (opens a pair) and after (closes it)
  void mark(int s, cudaStream_t st) {
    cudaEvent_t e = next();
    if (!e) return;
    cudaEventRecord(e, st);
    if (!open) stage.push_back(s);
    open = !open;
  }
};

struct oopao_pwfs_plan {
  int device;
  PwfsProfile* prof;
  int res, n, cam, k, bin, off;
  int psf_centering;
  FftPlan fft;
  float2* d_tw;      // [n]      exp(-2 pi i t / n)
  float2* d_mask;    // [n*n]
  float2* d_rowfac;  // [k*res]  exp(i x_k t_j s) rho(j+off) / n^2 (per point)
  float2* d_colfac;  // [k*res]  exp(i y_k t_i s) rho(i+off)
  // points with equal x_k share their row transform (a symmetric modulation
  // circle has ~K/2+1 distinct x_k): group table and point -> group map
  int ngroups;
  float2* d_growfac;  // [ngroups*res]
  int* d_group;       // [k]
  // adjoint column pass: conjugate mask and a unit row phasor [k][n]
  float2* d_mask_conj;
  float2* d_ones;
  float* d_amp;      // [res*res]
  float* d_weights;  // [k] or null; allocated once, freed with the plan
  bool weights_on;   // launches read d_weights (else the plain sum)
  // launch shape
  int rows_per_cta, cols_per_cta, inv_rows_per_cta;
  int ksplit;        // partial slots over modulation points (divides k; 0 = automatic)
  size_t l2_budget;  // bytes of FFT intermediates per pass (kept L2-resident)
  const struct FastPasses* fast;  // compile-time plan for n, or null (generic kernels)
  int variant;                    // 1 = use `fast` when available, 0 = generic
  int inv_target_ctas;            // row-inverse CTAs wanted per launch (2 resident waves)
  int cols3_ctas;                 // resident CTAs of the persistent column pass (0 = not used)
  int n_masks;                    // Fourier masks measured together (1, or Bi-O Edge's 4)
  float2* d_masks;                // [n_masks][n][n] when n_masks > 1
  int* d_err;                     // device error word (bounded waits of the persistent column pass)
  // two-pass path for a mask that factorises per axis (pwfs_sep.cuh)
  const struct SepPasses* sep;    // compile-time two-pass plan for n, or null
  bool mask_sep;                  // mask == mcol (x) mrow within float32 rounding
  bool sep_on;                    // oopao_pwfs_set_separable (default on)
  float2* d_mrow;                 // [n] factor along a row (column frequency)
  float2* d_mcol;                 // [n] factor along a column (row frequency)
  int sep_cols_ctas;              // resident column-pass CTAs on this device
  // the two-pass plan of the tangent and adjoint passes: the first
  // candidate, whatever the measure calls were tuned to (their kernel forms
  // differ), and its resident column-pass CTAs
  const struct SepPasses* sep_ad;
  int sep_ad_ctas;
  // Masks that each vary along one focal-plane axis only (the Bi-O Edge knife
  // edges, OOPAO/BioEdge.py:331-392, without their tip/tilt shifts).  The
  // filter then acts on the lines of that axis alone, and |G_k|^2 no longer
  // depends on the point's phasor along the other axis: the frame of such a
  // mask is sum over the groups of points sharing that axis' phasor of
  // (their weight) |filtered line|^2 (measure_edge).
  bool edge_1d;
  int edge_axis[8];               // 0: the mask varies along x (a row), 1: along y (a column)
  float2* d_edge_filt;            // [n_masks][n] the 1-D factors, pupil offset folded in
  int nygroups;                   // points with equal y_k
  float2* d_ygrowfac;             // [nygroups*res] their column phasor, with the 1/n^2 of ifft2
  float* d_gsum;                  // [2][k] points per x-group, per y-group (unweighted)
  float* d_gsum_w;                // [2][k] weights summed per x-group, per y-group
  int* h_group;                   // [k] x-group of each point (host)
  int* h_ygroup;                  // [k] y-group of each point (host)
  // signal processing
  int sp_mode, nq, n2d, n_signal, cam2;
  int q_r0[4], q_c0[4];
  float slopes_units, norma_const;
  unsigned char* d_valid;
  float* d_ref2d;
  int* d_sig_index;
  int* d_sig_inv;  // [n2d] signal entry of each 2-D map cell, or -1
};

static const float* weights_of(const oopao_pwfs_plan* p) { return p->weights_on ? p->d_weights : nullptr; }

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Pupil field amp * exp(i opd * scale) of each item, computed once per pass
// (shared by every modulation point).
__global__ void pwfs_field(const float* __restrict__ opd, float scale, const float* __restrict__ amp,
                           float2* __restrict__ field, int npix) {
  pdl_wait();
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float am = amp[i];
  float2 v = make_float2(0.f, 0.f);
  if (am != 0.f) {
    float s, c;
    sincosf(opd[(size_t)b * npix + i] * scale, &s, &c);
    v = make_float2(am * c, am * s);
  }
  field[(size_t)b * npix + i] = v;
}

struct RowsFwdArgs {
  FftPlan fft;
  const float2* tw;
  const float2* field;   // [B][res][res] amp * exp(i phase) of this pass's items
  const float2* rowfac;  // [groups][res] column-direction phasor of each row-transform group
  float2* y;             // [B][ng][res][n] row transforms of groups [g0, g0+ng)
  int res, n, g0, ng, off, lines;
};

__global__ void __launch_bounds__(kThreads) pwfs_rows_fwd(RowsFwdArgs a) {
  extern __shared__ float2 smem[];
  const int n = a.n;
  float2* tw = smem;
  float2* buf0 = smem + n;
  float2* buf1 = buf0 + a.lines * n;
  const int tid = threadIdx.x;
  const int b = blockIdx.z, g = blockIdx.y, i0 = blockIdx.x * a.lines;
  const int nl = min(a.lines, a.res - i0);
  for (int t = tid; t < n; t += blockDim.x) tw[t] = a.tw[t];
  const float2* fld = a.field + (size_t)b * a.res * a.res;
  const float2* rf = a.rowfac + (size_t)(a.g0 + g) * a.res;
  for (int idx = tid; idx < a.lines * n; idx += blockDim.x) {
    const int line = idx / n;
    const int x = idx - line * n;
    const int j = x - a.off;
    float2 v = make_float2(0.f, 0.f);
    if (line < nl && j >= 0 && j < a.res) v = cmul(fld[(i0 + line) * a.res + j], rf[j]);
    buf0[idx] = v;
  }
  __syncthreads();
  float2* out = fft_lines<false>(buf0, buf1, a.fft, tw, nl, n, tid, blockDim.x);
  float2* y = a.y + (((size_t)b * a.ng + g) * a.res + i0) * n;
  for (int idx = tid; idx < nl * n; idx += blockDim.x) y[idx] = out[idx];
}

struct ColsArgs {
  FftPlan fft;
  const float2* tw;
  const float2* mask;    // [n][n]
  const float2* y;       // [B][ng][res][n]
  const int* group;      // [K] row-transform group of each point, or null (group = point - k0)
  const float2* colfac;  // [K][res] row-direction phasor of each point
  float2* z;             // [B][kp][n][n] for the points [k0, k0+kp)
  int res, n, k0, kp, ng, off, cols;
  // focal-plane (modulation) camera: sum over points of |F_k|^2 * focal_scale
  // into [B][n][n] (atomic adds), or null
  float* focal;
  float focal_scale;
  // persistent column pass (pwfs_cols3): items in this pass, error word
  int items;
  int* err;
  // several masks (pwfs_cols2m): mask = [n_masks][n][n]
  int n_masks;
};

__global__ void __launch_bounds__(kThreads) pwfs_cols(ColsArgs a) {
  extern __shared__ float2 smem[];
  const int n = a.n, C = a.cols;
  float2* tw = smem;
  float2* buf0 = smem + n;
  float2* buf1 = buf0 + C * n;
  const int tid = threadIdx.x;
  const int b = blockIdx.z, kk = blockIdx.y, c0 = blockIdx.x * C;
  const int kabs = a.k0 + kk;
  const int g = a.group ? a.group[kabs] : kk;
  for (int t = tid; t < n; t += blockDim.x) tw[t] = a.tw[t];
  const float2* y = a.y + ((size_t)b * a.ng + g) * a.res * n;
  const float2* cf = a.colfac + (size_t)kabs * a.res;
  // gather: column c of the tile becomes line c; rows outside [off, off+res) are zero
  for (int idx = tid; idx < C * n; idx += blockDim.x) {
    const int c = idx % C;
    const int r = idx / C;
    const int i = r - a.off;
    float2 v = make_float2(0.f, 0.f);
    if (c0 + c < n && i >= 0 && i < a.res) v = cmul(y[(size_t)i * n + c0 + c], cf[i]);
    buf0[c * n + r] = v;
  }
  __syncthreads();
  float2* f = fft_lines<false>(buf0, buf1, a.fft, tw, C, n, tid, blockDim.x);
  float2* other = (f == buf0) ? buf1 : buf0;
  for (int idx = tid; idx < C * n; idx += blockDim.x) {
    const int c = idx % C;
    const int r = idx / C;
    if (c0 + c < n) {
      if (a.focal) atomicAdd(a.focal + ((size_t)b * n + r) * n + c0 + c, a.focal_scale * cabs2(f[c * n + r]));
      f[c * n + r] = cmul(f[c * n + r], a.mask[(size_t)r * n + c0 + c]);
    }
  }
  __syncthreads();
  float2* gg = fft_lines<true>(f, other, a.fft, tw, C, n, tid, blockDim.x);
  float2* z = a.z + ((size_t)b * a.kp + kk) * n * n;
  for (int idx = tid; idx < C * n; idx += blockDim.x) {
    const int c = idx % C;
    const int r = idx / C;
    if (c0 + c < n) z[(size_t)r * n + c0 + c] = gg[c * n + r];
  }
}

struct RowsInvArgs {
  FftPlan fft;
  const float2* tw;
  const float2* z;       // [B][K][n][n]
  const float* weights;  // [K] or null
  float* partial;        // [B][ksplit][n][n] un-binned partial sums, or null
  float* binned;         // [B][ksplit][cam][cam] binned partial sums (fused binning)
  // this pass holds points [k0, k0+kp) of each item and processes slots
  // [s0, s0+gridDim.y); slot s sums points [s*slot_pts, (s+1)*slot_pts)
  int n, k0, kp, s0, slot_pts, ksplit, lines, bin, cam;
};

__global__ void __launch_bounds__(kThreads) pwfs_rows_inv(RowsInvArgs a) {
  extern __shared__ float2 smem[];
  const int n = a.n;
  float2* tw = smem;
  float2* buf0 = smem + n;
  float2* buf1 = buf0 + a.lines * n;
  float* acc = reinterpret_cast<float*>(buf1 + a.lines * n);
  const int tid = threadIdx.x;
  const int b = blockIdx.z, slot = a.s0 + blockIdx.y, r0 = blockIdx.x * a.lines;
  const int nl = min(a.lines, n - r0);
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  for (int t = tid; t < n; t += blockDim.x) tw[t] = a.tw[t];
  for (int idx = tid; idx < a.lines * n; idx += blockDim.x) acc[idx] = 0.f;
  for (int kk = kbeg; kk < kend; kk++) {
    const float2* z = a.z + (((size_t)b * a.kp + (kk - a.k0)) * n + r0) * n;
    for (int idx = tid; idx < nl * n; idx += blockDim.x) buf0[idx] = z[idx];
    __syncthreads();
    float2* g = fft_lines<true>(buf0, buf1, a.fft, tw, nl, n, tid, blockDim.x);
    const float w = a.weights ? a.weights[kk] : 1.f;
    for (int idx = tid; idx < nl * n; idx += blockDim.x) acc[idx] = fmaf(w, cabs2(g[idx]), acc[idx]);
    __syncthreads();
  }
  float* p = a.partial + (((size_t)b * a.ksplit + slot) * n + r0) * n;
  for (int idx = tid; idx < nl * n; idx += blockDim.x) p[idx] = acc[idx];
}

#include "pwfs_fast.cuh"
#include "pwfs_sep.cuh"
namespace {
// Compile-time plans (N = R1*R2, T threads per line, lines per CTA of the
// three passes).  Sizes without an entry use the generic kernels.
// Candidates per N (the autotuner picks one per plan).  Row-inverse lines per
// CTA are a multiple of the usual N/cam so the detector binning fuses into
// that pass (6 for the default geometry).
int fast_candidates(int n, const FastPasses** out) {
  static const FastPasses f72[] = {make_fast<72, 8, 9, 9, 16, 16, 12>()};
  static const FastPasses f96[] = {make_fast<96, 8, 12, 12, 16, 16, 12>()};
  static const FastPasses f112[] = {make_fast<112, 16, 7, 8, 16, 16, 16>()};
  static const FastPasses f128[] = {make_fast<128, 16, 8, 8, 16, 16, 16>()};
  static const FastPasses f240[] = {make_fast<240, 16, 15, 16, 16, 16, 12>()};
  static const FastPasses f264[] = {make_fast<264, 24, 11, 12, 16, 16, 12>(),
                                    make_fast<264, 24, 11, 24, 8, 8, 12>(),
                                    make_fast<264, 11, 24, 12, 16, 16, 12>(),
                                    make_fast<264, 12, 22, 12, 16, 16, 12>(),
                                    make_fast3<264, 12, 22, 12, 16, 16, 12, 8>()};
  static const FastPasses f480[] = {make_fast<480, 24, 20, 12, 16, 8, 12>()};
  static const FastPasses f504[] = {make_fast<504, 24, 21, 12, 16, 8, 12>(),
                                    make_fast<504, 24, 21, 24, 8, 8, 12>(),
                                    make_fast<504, 21, 24, 12, 16, 8, 12>(),
                                    make_fast<504, 24, 21, 24, 8, 16, 6>()};
  static const FastPasses f1920[] = {make_fast<1920, 48, 40, 48, 2, 8, 6>(),
                                     make_fast<1920, 48, 40, 48, 2, 4, 6>(),
                                     make_fast<1920, 48, 40, 48, 2, 2, 6>(),
                                     make_fast<1920, 40, 48, 48, 2, 4, 6>()};
#define OOPAO_CANDS(arr) (*out = arr, (int)(sizeof(arr) / sizeof(arr[0])))
  switch (n) {
    case 72: return OOPAO_CANDS(f72);
    case 96: return OOPAO_CANDS(f96);
    case 112: return OOPAO_CANDS(f112);
    case 128: return OOPAO_CANDS(f128);
    case 240: return OOPAO_CANDS(f240);
    case 264: return OOPAO_CANDS(f264);
    case 480: return OOPAO_CANDS(f480);
    case 504: return OOPAO_CANDS(f504);
    case 1920: return OOPAO_CANDS(f1920);
    default: *out = nullptr; return 0;
  }
#undef OOPAO_CANDS
}

constexpr int kTargetCtas = 2 * 152;  // row-inverse CTAs wanted by the generic kernels

// Variant a plan starts with (0-based index into the candidates): the
// fastest measured on GB300 over batch 1 to 100; the autotuner may pick
// another per batch.
int fast_default_index(int n) {
  switch (n) {
    case 264: return 3;  // 12 x 22, one stage-B butterfly per thread
    case 504: return 3;  // 24 x 21, 24 threads per line, 6-row inverse blocks
    default: return 0;
  }
}

const FastPasses* fast_passes(int n, int idx = 0) {
  const FastPasses* c = nullptr;
  const int cnt = fast_candidates(n, &c);
  return (idx >= 0 && idx < cnt) ? c + idx : nullptr;
}

// Opt the variant's kernels into their shared memory and return, in
// *inv_target, two resident waves of row-inverse CTAs on this device and, in
// *cols3_ctas, the resident CTAs of its persistent column pass for pupils of
// `res` pixels (0 when the variant has none or res is above a TMA box).
cudaError_t fast_attrs(const FastPasses* f, int res, int* inv_target, int* cols3_ctas) {
  cudaError_t e = cudaFuncSetAttribute(f->rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->smem_rows);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(f->cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->smem_cols);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(f->inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->smem_inv);
  if (e == cudaSuccess && f->cols_m)
    e = cudaFuncSetAttribute(f->cols_m, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->smem_cols_m);
  int dev = 0, sms = 0, occ = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, f->inv, f->t * f->l_inv, f->smem_inv);
  if (e == cudaSuccess) *inv_target = 2 * sms * std::max(occ, 1);
  *cols3_ctas = 0;
  if (e == cudaSuccess && f->cols3 && res <= 256) {
    const size_t sm3 = f->smem_cols3(res);
    int occ3 = 0;
    e = cudaFuncSetAttribute(f->cols3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ3, f->cols3, f->t * f->l_cols3, sm3);
    if (e == cudaSuccess) *cols3_ctas = occ3 * sms;
  }
  return e;
}

// 2-D TMA map of the row transforms Y [rows][n] complex64, viewed as float32
// pairs, with [res][l3] boxes (l3 columns of res rows).
int encode_y_map(CUtensorMap* map, const float2* y, int n, size_t rows, int l3, int res) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tma::encode_fn();
  if (!fn) {
    oopao_set_last_error("cuTensorMapEncodeTiled is not available from the driver", __FILE__, __LINE__);
    return OOPAO_ERR_CUDA;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)2 * n, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)n * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)(2 * l3), (cuuint32_t)res};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(y), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    oopao_set_last_error("cuTensorMapEncodeTiled rejected the row-transform map", __FILE__, __LINE__);
    return OOPAO_ERR_INVALID;
  }
  return OOPAO_OK;
}
}  // namespace

// One CTA per (camera row, batch item); thread = camera column.  Also writes
// raw_data rows (sum of partials) when requested.
__global__ void pwfs_bin(const float* __restrict__ partial, float* __restrict__ frame,
                         float* __restrict__ raw, int n, int cam, int bin, int ksplit) {
  const int b = blockIdx.y, cy = blockIdx.x;
  const float* p = partial + (size_t)b * ksplit * n * n;
  if (raw) {
    for (int idx = threadIdx.x; idx < bin * n; idx += blockDim.x) {
      const int y = cy * bin + idx / n, x = idx % n;
      float s = 0.f;
      for (int q = 0; q < ksplit; q++) s += p[((size_t)q * n + y) * n + x];
      raw[((size_t)b * n + y) * n + x] = s;
    }
  }
  for (int cx = threadIdx.x; cx < cam; cx += blockDim.x) {
    float s = 0.f;
    for (int dy = 0; dy < bin; dy++) {
      float row = 0.f;
      for (int dx = 0; dx < bin; dx++) {
        float v = 0.f;
        for (int q = 0; q < ksplit; q++) v += p[((size_t)q * n + cy * bin + dy) * n + cx * bin + dx];
        row += v;
      }
      s += row;
    }
    frame[((size_t)b * cam + cy) * cam + cx] = s;
  }
}

// Deterministic block sum (fixed tree for a fixed blockDim).
__device__ float block_sum(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  float t = 0.f;
  if (w == 0) {
    t = (l < nw) ? red[l] : 0.f;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) red[32] = t;
  }
  __syncthreads();
  const float r = red[32];
  __syncthreads();
  return r;
}

struct SignalArgs {
  const float* frame;        // [B][cam][cam]
  const unsigned char* valid;
  const float* ref2d;        // or null
  const int* sig_index;      // [n_signal]
  const int* sig_inv;        // [n2d] signal entry of each 2-D cell, or -1
  float* signal_2d;          // [B][n2d]
  float* signal;             // [B][n_signal]
  float* norma;              // [B] or null
  int mode, cam, nq, n2d, n_signal, n_valid;
  int q_r0[4], q_c0[4];
  float units, norma_const;
};

// Quadrant cells per thread that the slopes path keeps in registers between
// the flux reduction and the output (nq^2 <= kSigCells * blockDim).
constexpr int kSigCells = 8;

__global__ void pwfs_signal(SignalArgs a) {
  __shared__ float red[33];
  pdl_wait();
  const int b = blockIdx.x;
  const float* fr = a.frame + (size_t)b * a.cam * a.cam;
  float* s2 = a.signal_2d + (size_t)b * a.n2d;
  float* sg = a.signal + (size_t)b * a.n_signal;
  const bool slopes = a.mode <= 2;
  const int nq2s = a.nq * a.nq;
  if (slopes && nq2s <= kSigCells * (int)blockDim.x) {
    // one read of the frame: every load of a cell (four quadrant pixels, its
    // reference slopes and signal slots) is issued before the reduction; the
    // per-thread flux sums run over the same cells in the same order as the
    // general path below, so both give the same bits
    float sx[kSigCells], sy[kSigCells], rx[kSigCells], ry[kSigCells];
    int ex[kSigCells], ey[kSigCells];
    float part = 0.f;
#pragma unroll
    for (int k = 0; k < kSigCells; k++) {
      const int idx = threadIdx.x + k * blockDim.x;
      sx[k] = sy[k] = rx[k] = ry[k] = 0.f;
      ex[k] = ey[k] = -1;
      if (idx < nq2s) {
        const int r = idx / a.nq, c = idx % a.nq;
        const float i1 = fr[(a.q_r0[0] + r) * a.cam + a.q_c0[0] + c];
        const float i2 = fr[(a.q_r0[1] + r) * a.cam + a.q_c0[1] + c];
        const float i3 = fr[(a.q_r0[2] + r) * a.cam + a.q_c0[2] + c];
        const float i4 = fr[(a.q_r0[3] + r) * a.cam + a.q_c0[3] + c];
        if (a.ref2d) {
          rx[k] = a.ref2d[idx];
          ry[k] = a.ref2d[nq2s + idx];
        }
        ex[k] = a.sig_inv[idx];
        ey[k] = a.sig_inv[nq2s + idx];
        if (a.valid[idx]) {
          sx[k] = ((i1 - i2) + i4) - i3;
          sy[k] = ((i1 - i4) + i2) - i3;
          if (a.mode == 0) part += ((i1 + i2) + i3) + i4;
        }
      }
    }
    if (a.mode == 2)
      for (int idx = threadIdx.x; idx < a.cam * a.cam; idx += blockDim.x) part += fr[idx];
    const float tot = block_sum(part, red);
    const float norma = a.mode == 0 ? tot / (float)a.n_valid
                      : a.mode == 2 ? tot / (float)(a.cam * a.cam) : a.norma_const;
#pragma unroll
    for (int k = 0; k < kSigCells; k++) {
      const int idx = threadIdx.x + k * blockDim.x;
      if (idx < nq2s) {
        const float vx = (sx[k] / norma - rx[k]) * a.units, vy = (sy[k] / norma - ry[k]) * a.units;
        s2[idx] = vx;
        s2[nq2s + idx] = vy;
        if (ex[k] >= 0) sg[ex[k]] = vx;
        if (ey[k] >= 0) sg[ey[k]] = vy;
      }
    }
    if (a.norma && threadIdx.x == 0) a.norma[b] = norma;
    return;
  }
  float part = 0.f;
  if (slopes) {
    const int nq2 = a.nq * a.nq;
    if (a.mode == 0) {
      for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
        if (!a.valid[idx]) continue;
        const int r = idx / a.nq, c = idx % a.nq;
        const float i1 = fr[(a.q_r0[0] + r) * a.cam + a.q_c0[0] + c];
        const float i2 = fr[(a.q_r0[1] + r) * a.cam + a.q_c0[1] + c];
        const float i3 = fr[(a.q_r0[2] + r) * a.cam + a.q_c0[2] + c];
        const float i4 = fr[(a.q_r0[3] + r) * a.cam + a.q_c0[3] + c];
        part += ((i1 + i2) + i3) + i4;
      }
    } else if (a.mode == 2) {
      for (int idx = threadIdx.x; idx < a.cam * a.cam; idx += blockDim.x) part += fr[idx];
    }
  } else if (a.mode == 3) {
    for (int idx = threadIdx.x; idx < a.cam * a.cam; idx += blockDim.x)
      if (a.valid[idx]) part += fr[idx];
  } else if (a.mode == 5 || a.mode == 6) {
    for (int idx = threadIdx.x; idx < a.cam * a.cam; idx += blockDim.x) part += fr[idx];
  }
  const float tot = block_sum(part, red);
  float norma;
  switch (a.mode) {
    case 0: norma = tot / (float)a.n_valid; break;
    case 2: case 5: norma = tot / (float)(a.cam * a.cam); break;
    case 3: case 6: norma = tot; break;
    default: norma = a.norma_const; break;
  }
  if (slopes) {
    const int nq2 = a.nq * a.nq;
    for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
      const int r = idx / a.nq, c = idx % a.nq;
      float sx = 0.f, sy = 0.f;
      if (a.valid[idx]) {
        const float i1 = fr[(a.q_r0[0] + r) * a.cam + a.q_c0[0] + c];
        const float i2 = fr[(a.q_r0[1] + r) * a.cam + a.q_c0[1] + c];
        const float i3 = fr[(a.q_r0[2] + r) * a.cam + a.q_c0[2] + c];
        const float i4 = fr[(a.q_r0[3] + r) * a.cam + a.q_c0[3] + c];
        sx = ((i1 - i2) + i4) - i3;
        sy = ((i1 - i4) + i2) - i3;
      }
      const float rx = a.ref2d ? a.ref2d[idx] : 0.f;
      const float ry = a.ref2d ? a.ref2d[nq2 + idx] : 0.f;
      const float vx = (sx / norma - rx) * a.units, vy = (sy / norma - ry) * a.units;
      s2[idx] = vx;
      s2[nq2 + idx] = vy;
      // signal = signal_2D[validSignal], written from the same registers
      const int ex = a.sig_inv[idx], ey = a.sig_inv[nq2 + idx];
      if (ex >= 0) sg[ex] = vx;
      if (ey >= 0) sg[ey] = vy;
    }
  } else {
    for (int idx = threadIdx.x; idx < a.cam * a.cam; idx += blockDim.x) {
      const float rr = a.ref2d ? a.ref2d[idx] : 0.f;
      const float v = fr[idx] / norma - rr;
      s2[idx] = v;
      const int e = a.sig_inv[idx];
      if (e >= 0) sg[e] = v;
    }
  }
  if (a.norma && threadIdx.x == 0) a.norma[b] = norma;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

namespace {

size_t rows_smem(int n, int lines) { return (size_t)(n + 2 * lines * n) * sizeof(float2); }
size_t inv_smem(int n, int lines) { return rows_smem(n, lines) + (size_t)lines * n * sizeof(float); }

int max_lines(int n, bool with_acc) {
  int l = 32;
  while (l > 1 && (with_acc ? inv_smem(n, l) : rows_smem(n, l)) > kSmemLimit) l--;
  return l;
}

void free_plan(oopao_pwfs_plan* p) {
  if (!p) return;
  if (p->prof) {
    for (cudaEvent_t e : p->prof->pool) cudaEventDestroy(e);
    delete p->prof;
  }
  cudaFree(p->d_tw);
  cudaFree(p->d_mask);
  cudaFree(p->d_rowfac);
  cudaFree(p->d_colfac);
  cudaFree(p->d_growfac);
  cudaFree(p->d_group);
  cudaFree(p->d_mask_conj);
  cudaFree(p->d_ones);
  cudaFree(p->d_sig_inv);
  cudaFree(p->d_amp);
  cudaFree(p->d_weights);
  cudaFree(p->d_valid);
  cudaFree(p->d_ref2d);
  cudaFree(p->d_sig_index);
  cudaFree(p->d_err);
  cudaFree(p->d_masks);
  cudaFree(p->d_mrow);
  cudaFree(p->d_mcol);
  cudaFree(p->d_edge_filt);
  cudaFree(p->d_ygrowfac);
  cudaFree(p->d_gsum);
  cudaFree(p->d_gsum_w);
  free(p->h_group);
  free(p->h_ygroup);
  free(p);
}

// Rank-one factorisation M[r][c] = mcol[r] * mrow[c] of an n x n complex
// mask: pivot on the entry of largest modulus, mrow = the pivot's row,
// mcol = the pivot's column / pivot.  Accepted when the float32 factors
// reproduce every entry within 1e-6 of max|M| (the mask itself is stored in
// complex64, ~6e-8 rounding).  The reference's four-face mask factorises
// whenever the faces share one shift and there is no rooftop or rotation.
bool factor_mask(const float2* m, int n, std::vector<float2>* mrow, std::vector<float2>* mcol) {
  const size_t nn = (size_t)n * n;
  size_t piv = 0;
  double best = -1.0;
  for (size_t i = 0; i < nn; i++) {
    const double a = (double)m[i].x * m[i].x + (double)m[i].y * m[i].y;
    if (a > best) { best = a; piv = i; }
  }
  if (!(best > 0.0)) return false;
  const int r0 = (int)(piv / n), c0 = (int)(piv % n);
  const double pr = m[piv].x, pi = m[piv].y, pa = pr * pr + pi * pi;
  mrow->resize(n);
  mcol->resize(n);
  for (int c = 0; c < n; c++) (*mrow)[c] = m[(size_t)r0 * n + c];
  for (int r = 0; r < n; r++) {
    const double ar = m[(size_t)r * n + c0].x, ai = m[(size_t)r * n + c0].y;
    (*mcol)[r] = make_float2((float)((ar * pr + ai * pi) / pa), (float)((ai * pr - ar * pi) / pa));
  }
  const double tol = 1e-6 * sqrt(best);
  for (int r = 0; r < n; r++) {
    const double ur = (*mcol)[r].x, ui = (*mcol)[r].y;
    for (int c = 0; c < n; c++) {
      const double vr = (*mrow)[c].x, vi = (*mrow)[c].y;
      const float2 e = m[(size_t)r * n + c];
      const double dr = ur * vr - ui * vi - e.x, di = ur * vi + ui * vr - e.y;
      if (dr * dr + di * di > tol * tol) return false;
    }
  }
  return true;
}

// Opt a two-pass plan's kernels into their shared memory for pupils of
// `res` pixels and return in *ctas its resident column-pass CTAs on this
// device.
cudaError_t sep_attrs_for(const SepPasses* s, int res, int* ctas) {
  cudaError_t e = cudaFuncSetAttribute(s->rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_rows);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(s->rows_int, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_rows);
  for (int m = 0; m < 3 && e == cudaSuccess; m++)
    e = cudaFuncSetAttribute(s->cols[m], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_cols(res));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(s->cols_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_cols(res));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(s->rows_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_rows);
  int dev = 0, sms = 0, occ = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, s->cols[kSepIntensity], s->t * s->l_cols,
                                                      s->smem_cols(res));
  if (e == cudaSuccess) *ctas = sms * std::max(occ, 1);
  return e;
}

cudaError_t sep_attrs(oopao_pwfs_plan* p) {
  cudaError_t e = sep_attrs_for(p->sep, p->res, &p->sep_cols_ctas);
  if (e == cudaSuccess) e = sep_attrs_for(p->sep_ad, p->res, &p->sep_ad_ctas);
  return e;
}

// A two-pass plan serves pupils of `res` pixels when its column pass fits in
// shared memory, the 16-byte tile copies see an even pupil, and the pupil
// lies within the stage-A inputs the plan reads (res <= nz * r2).
bool sep_fits(const SepPasses* s, int res) {
  return res % 2 == 0 && s->smem_cols(res) <= kSmemLimit && (res + s->r2 - 1) / s->r2 <= s->nz;
}

// Two-pass set-up for mask 0 of the plan: factorise it, upload the factors
// and prepare the kernels.  A mask that does not factorise (or an n without
// a two-pass plan) leaves mask_sep false.
cudaError_t sep_setup(oopao_pwfs_plan* p, const float* mask_host) {
  p->mask_sep = false;
  // 16-byte tile copies need an even pupil; the column pass must fit in shared memory
  if (!p->sep || !sep_fits(p->sep, p->res)) return cudaSuccess;
  std::vector<float2> mrow, mcol;
  if (!factor_mask(reinterpret_cast<const float2*>(mask_host), p->n, &mrow, &mcol)) return cudaSuccess;
  // The passes place the pupil at rows and columns [0, res) of the grid
  // instead of [off, off+res): F(x) = exp(-2 pi i u off/N) F(x shifted by
  // off), so the shift folds into each factor as that linear phase and the
  // outputs are unchanged.  The forward transforms then see their non-zero
  // inputs at the start of each line.
  for (int u = 0; u < p->n; u++) {
    const long long m = ((long long)u * p->off) % p->n;
    const double a = -2.0 * M_PI * (double)m / p->n, cr = cos(a), ci = sin(a);
    for (std::vector<float2>* f : {&mrow, &mcol}) {
      const double fr = (*f)[u].x, fi = (*f)[u].y;
      (*f)[u] = make_float2((float)(fr * cr - fi * ci), (float)(fr * ci + fi * cr));
    }
  }
  cudaError_t e = cudaSuccess;
  if (!p->d_mrow) e = cudaMalloc((void**)&p->d_mrow, sizeof(float2) * p->n);
  if (e == cudaSuccess && !p->d_mcol) e = cudaMalloc((void**)&p->d_mcol, sizeof(float2) * p->n);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_mrow, mrow.data(), sizeof(float2) * p->n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_mcol, mcol.data(), sizeof(float2) * p->n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = sep_attrs(p);
  if (e == cudaSuccess) p->mask_sep = true;
  return e;
}

// Masks that each vary along one axis only: mask m is f_m[c] on every row
// (axis 0) or g_m[r] on every column (axis 1), within 1e-6 of max|M| (the
// tolerance of factor_mask).  Such a mask filters the lines of one axis and
// leaves the other untouched, so measure_edge needs the filtered lines of
// each axis only.  The factors carry the pupil-offset phase of sep_setup.
// Leaves edge_1d false when a mask is two-dimensional or no two-pass plan
// serves n.
cudaError_t edge_setup(oopao_pwfs_plan* p, int n_masks, const float* masks_host) {
  p->edge_1d = false;
  if (!p->sep || !sep_fits(p->sep, p->res) || n_masks < 1 || n_masks > 8) return cudaSuccess;
  const int n = p->n;
  const size_t nn = (size_t)n * n;
  const float2* all = reinterpret_cast<const float2*>(masks_host);
  std::vector<float2> filt((size_t)n_masks * n);
  int axis[8];
  for (int m = 0; m < n_masks; m++) {
    const float2* M = all + (size_t)m * nn;
    double mx = 0.0;
    for (size_t i = 0; i < nn; i++) mx = std::max(mx, (double)M[i].x * M[i].x + (double)M[i].y * M[i].y);
    const double tol2 = 1e-12 * mx;
    auto same = [&](const float2& a, const float2& b) {
      const double dr = (double)a.x - b.x, di = (double)a.y - b.y;
      return dr * dr + di * di <= tol2;
    };
    bool along_x = true, along_y = true;
    for (int r = 0; r < n && (along_x || along_y); r++)
      for (int c = 0; c < n && (along_x || along_y); c++) {
        if (along_x && !same(M[(size_t)r * n + c], M[c])) along_x = false;
        if (along_y && !same(M[(size_t)r * n + c], M[(size_t)r * n])) along_y = false;
      }
    if (!along_x && !along_y) return cudaSuccess;
    axis[m] = along_x ? 0 : 1;
    for (int u = 0; u < n; u++) {
      const float2 f = along_x ? M[u] : M[(size_t)u * n];
      const long long q = ((long long)u * p->off) % n;
      const double a = -2.0 * M_PI * (double)q / n, cr = cos(a), ci = sin(a);
      filt[(size_t)m * n + u] = make_float2((float)(f.x * cr - f.y * ci), (float)(f.x * ci + f.y * cr));
    }
  }
  cudaError_t e = cudaSuccess;
  if (!p->d_edge_filt) e = cudaMalloc((void**)&p->d_edge_filt, sizeof(float2) * 8 * n);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_edge_filt, filt.data(), sizeof(float2) * filt.size(), cudaMemcpyHostToDevice);
  int ctas = 0;
  if (e == cudaSuccess) e = sep_attrs_for(p->sep, p->res, &ctas);
  if (e != cudaSuccess) return e;
  for (int m = 0; m < n_masks; m++) p->edge_axis[m] = axis[m];
  p->edge_1d = true;
  return cudaSuccess;
}

// numpy.linspace(-pi, pi, res)[j]
double tt_grid(int j, int res) {
  if (res == 1) return -M_PI;
  if (j == res - 1) return M_PI;
  return -M_PI + j * (2.0 * M_PI / (res - 1));
}

}  // namespace

extern "C" int oopao_pwfs_plan_create(oopao_pwfs_plan** out, int res, int n, int cam, int k,
                                      const float* mask_host, const double* path_host,
                                      double tt_scale, int psf_centering) {
  OOPAO_CHECK_ARG(out != nullptr, "plan pointer is NULL");
  *out = nullptr;
  OOPAO_CHECK_ARG(res > 0 && n >= res && (n - res) % 2 == 0, "need n_fft >= res with n_fft-res even");
  OOPAO_CHECK_ARG(cam > 0 && n % cam == 0, "n_fft must be a multiple of the camera size");
  OOPAO_CHECK_ARG(k >= 1, "n_theta must be >= 1");
  OOPAO_CHECK_ARG(mask_host != nullptr, "mask is NULL");
  OOPAO_CHECK_ARG(path_host != nullptr || k == 1, "modulation path is NULL");
  FftPlan fp;
  if (!fft_make_plan(n, &fp)) {
    oopao_set_last_error("FFT size has a prime factor > 13 or too many stages", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  oopao_pwfs_plan* p = (oopao_pwfs_plan*)calloc(1, sizeof(oopao_pwfs_plan));
  OOPAO_CHECK_ARG(p != nullptr, "out of host memory");
  cudaGetDevice(&p->device);
  p->prof = new PwfsProfile();
  p->res = res; p->n = n; p->cam = cam; p->k = k; p->bin = n / cam; p->off = (n - res) / 2;
  p->psf_centering = psf_centering;
  p->fft = fp;
  p->rows_per_cta = std::min(8, max_lines(n, false));
  p->cols_per_cta = std::min(16, max_lines(n, false));
  p->inv_rows_per_cta = std::min(8, max_lines(n, true));
  p->ksplit = 0;  // automatic
  p->n_masks = 1;
  p->l2_budget = kDefaultPassBudget;
  p->slopes_units = 1.f;
  p->sp_mode = -1;

  std::vector<float2> tw(n), rowfac((size_t)k * res), colfac((size_t)k * res);
  for (int t = 0; t < n; t++) {
    const double a = -2.0 * M_PI * (double)t / n;
    tw[t] = make_float2((float)cos(a), (float)sin(a));
  }
  // rho(t): centring phasor exp(-i pi (N+1) t / N), or (-1)^t for the
  // fftshift of the 1-pixel-centred mask; 1/N^2 of ifft2 folded into rowfac.
  auto rho = [&](int t, double* re, double* im) {
    if (psf_centering) {
      const long long m = ((long long)(n + 1) * t) % (2LL * n);
      const double a = -M_PI * (double)m / n;
      *re = cos(a); *im = sin(a);
    } else {
      *re = (t % 2) ? -1.0 : 1.0; *im = 0.0;
    }
  };
  const double inv_n2 = 1.0 / ((double)n * (double)n);
  for (int kk = 0; kk < k; kk++) {
    const double xk = path_host ? path_host[2 * kk] : 0.0;
    const double yk = path_host ? path_host[2 * kk + 1] : 0.0;
    for (int j = 0; j < res; j++) {
      const double t = tt_grid(j, res) * tt_scale;
      double pr, pi;
      rho(j + p->off, &pr, &pi);
      const double ax = xk * t, ay = yk * t;
      const double cr = cos(ax), ci = sin(ax);
      rowfac[(size_t)kk * res + j] = make_float2((float)((cr * pr - ci * pi) * inv_n2),
                                                 (float)((cr * pi + ci * pr) * inv_n2));
      const double dr = cos(ay), di = sin(ay);
      colfac[(size_t)kk * res + j] = make_float2((float)(dr * pr - di * pi), (float)(dr * pi + di * pr));
    }
  }
  // row-transform groups: points whose x_k agree to 1e-12 share rowfac
  std::vector<double> gx;
  std::vector<int> group(k);
  std::vector<float2> growfac;
  for (int kk = 0; kk < k; kk++) {
    const double xk = path_host ? path_host[2 * kk] : 0.0;
    int g = -1;
    for (size_t q = 0; q < gx.size(); q++)
      if (fabs(gx[q] - xk) <= 1e-12 * std::max(1.0, fabs(xk))) { g = (int)q; break; }
    if (g < 0) {
      g = (int)gx.size();
      gx.push_back(xk);
      growfac.insert(growfac.end(), rowfac.begin() + (size_t)kk * res, rowfac.begin() + (size_t)(kk + 1) * res);
    }
    group[kk] = g;
  }
  p->ngroups = (int)gx.size();
  // the same for y_k: the column phasors of the points with equal y_k, for
  // masks that vary along y only (with the 1/n^2 the row phasors carry)
  std::vector<double> gy;
  std::vector<int> ygroup(k);
  std::vector<float2> ygrowfac;
  for (int kk = 0; kk < k; kk++) {
    const double yk = path_host ? path_host[2 * kk + 1] : 0.0;
    int g = -1;
    for (size_t q = 0; q < gy.size(); q++)
      if (fabs(gy[q] - yk) <= 1e-12 * std::max(1.0, fabs(yk))) { g = (int)q; break; }
    if (g < 0) {
      g = (int)gy.size();
      gy.push_back(yk);
      for (int j = 0; j < res; j++) {
        const float2 c = colfac[(size_t)kk * res + j];
        ygrowfac.push_back(make_float2((float)(c.x * inv_n2), (float)(c.y * inv_n2)));
      }
    }
    ygroup[kk] = g;
  }
  p->nygroups = (int)gy.size();
  p->h_group = (int*)malloc(sizeof(int) * k);
  p->h_ygroup = (int*)malloc(sizeof(int) * k);
  if (!p->h_group || !p->h_ygroup) {
    free_plan(p);
    oopao_set_last_error("host allocation failed", __FILE__, __LINE__);
    return OOPAO_ERR_CUDA;
  }
  std::vector<float> gsum(2 * (size_t)k, 0.f);
  for (int kk = 0; kk < k; kk++) {
    p->h_group[kk] = group[kk];
    p->h_ygroup[kk] = ygroup[kk];
    gsum[group[kk]] += 1.f;
    gsum[k + ygroup[kk]] += 1.f;
  }
  std::vector<float> ones((size_t)res * res, 0.f);
#define ALLOC_COPY(dst, src, bytes)                                   \
  do {                                                                \
    cudaError_t e1 = cudaMalloc((void**)&(dst), (bytes));             \
    if (e1 == cudaSuccess && (src) != nullptr)                        \
      e1 = cudaMemcpy((dst), (src), (bytes), cudaMemcpyHostToDevice); \
    if (e1 != cudaSuccess) {                                          \
      oopao_set_last_error(cudaGetErrorString(e1), __FILE__, __LINE__); \
      free_plan(p);                                                   \
      return OOPAO_ERR_CUDA;                                          \
    }                                                                 \
  } while (0)
  ALLOC_COPY(p->d_tw, tw.data(), sizeof(float2) * n);
  ALLOC_COPY(p->d_mask, mask_host, sizeof(float2) * (size_t)n * n);
  ALLOC_COPY(p->d_rowfac, rowfac.data(), sizeof(float2) * rowfac.size());
  ALLOC_COPY(p->d_colfac, colfac.data(), sizeof(float2) * colfac.size());
  ALLOC_COPY(p->d_growfac, growfac.data(), sizeof(float2) * growfac.size());
  ALLOC_COPY(p->d_group, group.data(), sizeof(int) * group.size());
  ALLOC_COPY(p->d_ygrowfac, ygrowfac.data(), sizeof(float2) * ygrowfac.size());
  ALLOC_COPY(p->d_gsum, gsum.data(), sizeof(float) * gsum.size());
  ALLOC_COPY(p->d_gsum_w, gsum.data(), sizeof(float) * gsum.size());
  {
    std::vector<float2> mc((size_t)n * n), ones((size_t)k * n, make_float2(1.f, 0.f));
    const float2* m = reinterpret_cast<const float2*>(mask_host);
    for (size_t i = 0; i < mc.size(); i++) mc[i] = make_float2(m[i].x, -m[i].y);
    ALLOC_COPY(p->d_mask_conj, mc.data(), sizeof(float2) * mc.size());
    ALLOC_COPY(p->d_ones, ones.data(), sizeof(float2) * ones.size());
  }
  ALLOC_COPY(p->d_amp, ones.data(), sizeof(float) * ones.size());
#undef ALLOC_COPY
  cudaError_t e = cudaFuncSetAttribute(pwfs_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(pwfs_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(pwfs_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
  p->fast = fast_passes(n, fast_default_index(n));
  p->variant = p->fast ? fast_default_index(n) + 1 : 0;
  p->inv_target_ctas = kTargetCtas;
  p->cols3_ctas = 0;
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->d_err, 0, sizeof(int));
  if (p->fast && e == cudaSuccess) e = fast_attrs(p->fast, res, &p->inv_target_ctas, &p->cols3_ctas);
  {
    const SepPasses* sc = nullptr;
    p->sep = sep_candidates(n, &sc) > 0 ? sc : nullptr;
    p->sep_ad = p->sep;
    p->sep_on = true;
  }
  if (e == cudaSuccess) e = sep_setup(p, mask_host);
  if (e == cudaSuccess) e = edge_setup(p, 1, mask_host);
  if (e != cudaSuccess) {
    oopao_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    free_plan(p);
    return OOPAO_ERR_CUDA;
  }
  *out = p;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_plan_destroy(oopao_pwfs_plan* p) {
  free_plan(p);
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_amplitude(oopao_pwfs_plan* p, const float* amp_host) {
  OOPAO_CHECK_ARG(p && amp_host, "NULL argument");
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_amp, amp_host, sizeof(float) * p->res * p->res, cudaMemcpyHostToDevice));
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_masks(oopao_pwfs_plan* p, int n_masks, const float* masks_host) {
  OOPAO_CHECK_ARG(p && masks_host, "NULL argument");
  OOPAO_CHECK_ARG(n_masks >= 1 && n_masks <= 8, "1 to 8 masks");
  const size_t nn = (size_t)p->n * p->n;
  if (n_masks > 1 && !(p->fast && p->variant >= 1 && p->fast->cols_m)) {
    // move to the first compile-time variant that has the several-mask column pass
    const FastPasses* c = nullptr;
    const int cnt = fast_candidates(p->n, &c);
    int v = 0;
    for (int i = 0; i < cnt && !v; i++)
      if (c[i].cols_m) v = i + 1;
    if (!v) {
      oopao_set_last_error("no compile-time plan with a several-mask column pass for this FFT size", __FILE__,
                           __LINE__);
      return OOPAO_ERR_UNSUPPORTED;
    }
    int target = kTargetCtas, c3 = 0;
    OOPAO_CUDA_TRY(fast_attrs(c + (v - 1), p->res, &target, &c3));
    p->fast = c + (v - 1);
    p->variant = v;
    p->inv_target_ctas = target;
    p->cols3_ctas = c3;
  }
  // mask 0 is also the plan's single mask (spatial consumers, focal camera)
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_mask, masks_host, sizeof(float2) * nn, cudaMemcpyHostToDevice));
  if (p->d_mask_conj) {
    std::vector<float2> mc(nn);
    const float2* m = reinterpret_cast<const float2*>(masks_host);
    for (size_t i = 0; i < nn; i++) mc[i] = make_float2(m[i].x, -m[i].y);
    OOPAO_CUDA_TRY(cudaMemcpy(p->d_mask_conj, mc.data(), sizeof(float2) * nn, cudaMemcpyHostToDevice));
  }
  cudaFree(p->d_masks);
  p->d_masks = nullptr;
  p->mask_sep = false;
  if (n_masks == 1) OOPAO_CUDA_TRY(sep_setup(p, masks_host));
  OOPAO_CUDA_TRY(edge_setup(p, n_masks, masks_host));
  if (n_masks > 1) {
    OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_masks, sizeof(float2) * nn * n_masks));
    OOPAO_CUDA_TRY(cudaMemcpy(p->d_masks, masks_host, sizeof(float2) * nn * n_masks, cudaMemcpyHostToDevice));
  }
  p->n_masks = n_masks;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_n_masks(const oopao_pwfs_plan* p) { return p ? p->n_masks : -1; }

extern "C" int oopao_pwfs_set_weights(oopao_pwfs_plan* p, const float* w) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  // The buffer outlives every switch: a graph captured with the weights on
  // keeps its address.
  if (!w) {
    p->weights_on = false;
    return OOPAO_OK;
  }
  if (!p->d_weights) OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_weights, sizeof(float) * p->k));
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_weights, w, sizeof(float) * p->k, cudaMemcpyHostToDevice));
  // the weights summed over the groups of points that share a phasor
  // (masks that vary along one axis only)
  std::vector<float> gs(2 * (size_t)p->k, 0.f);
  for (int kk = 0; kk < p->k; kk++) {
    gs[p->h_group[kk]] += w[kk];
    gs[p->k + p->h_ygroup[kk]] += w[kk];
  }
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_gsum_w, gs.data(), sizeof(float) * gs.size(), cudaMemcpyHostToDevice));
  p->weights_on = true;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_launch(oopao_pwfs_plan* p, int rows, int cols, int inv_rows, int ksplit) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  if (rows > 0) {
    OOPAO_CHECK_ARG(rows_smem(p->n, rows) <= kSmemLimit, "rows_per_cta exceeds shared memory");
    p->rows_per_cta = rows;
  }
  if (cols > 0) {
    OOPAO_CHECK_ARG(rows_smem(p->n, cols) <= kSmemLimit, "cols_per_cta exceeds shared memory");
    p->cols_per_cta = cols;
  }
  if (inv_rows > 0) {
    OOPAO_CHECK_ARG(inv_smem(p->n, inv_rows) <= kSmemLimit, "inv_rows_per_cta exceeds shared memory");
    p->inv_rows_per_cta = inv_rows;
  }
  if (ksplit >= 0) {
    OOPAO_CHECK_ARG(ksplit == 0 || (ksplit <= p->k && p->k % ksplit == 0),
                    "ksplit must divide n_theta (0 = automatic)");
    p->ksplit = ksplit;
  }
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_pass_budget(oopao_pwfs_plan* p, size_t bytes) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  p->l2_budget = bytes ? bytes : kDefaultPassBudget;
  return OOPAO_OK;
}

namespace {

constexpr int kMaxSlotsBinned = 64;  // partial sums over modulation points, fused binning
constexpr int kMaxSlotsRaw = 8;      // partial sums kept un-binned (raw_data requested)

// How one oopao_pwfs_measure call is cut into passes: each pass holds the
// row/column intermediates of `bc` items x `kp` points, sized to stay
// resident in L2 between the three FFT passes; the row-inverse pass sums
// `slot_pts` points per partial slot.
struct PassPlan {
  bool fast, fused;
  int ksplit, slot_pts, bc, kp;
  size_t unit_bytes, bytes;
};

PassPlan plan_passes(const oopao_pwfs_plan* p, int batch, bool want_raw, size_t units) {
  PassPlan pp;
  const FastPasses* f = (p->variant >= 1) ? p->fast : nullptr;
  pp.fast = f != nullptr;
  pp.fused = pp.fast && !want_raw && (f->l_inv % p->bin == 0);
  const int k = p->k;
  const int nm = p->n_masks;
  pp.unit_bytes = ((size_t)p->res * p->n + (size_t)nm * p->n * p->n) * sizeof(float2);
  if (units < 1) units = 1;
  if (units >= (size_t)k) {
    pp.bc = (int)std::min<size_t>((size_t)batch, units / k);
    pp.kp = k;
  } else {
    pp.bc = 1;
    pp.kp = (int)units;
  }
  const int cap = pp.fused ? kMaxSlotsBinned : kMaxSlotsRaw;
  if (p->ksplit > 0) {
    pp.ksplit = p->ksplit;
  } else {
    const int row_blocks = ceil_div(p->n, pp.fast ? f->l_inv : p->inv_rows_per_cta);
    const int want = ceil_div(pp.fast ? p->inv_target_ctas : kTargetCtas, row_blocks * pp.bc * nm);
    int best = 1;
    for (int d = 1; d <= k && d <= cap; d++) {
      if (k % d) continue;
      best = d;
      if (d >= want) break;
    }
    pp.ksplit = best;
  }
  if (!pp.fused && pp.ksplit > kMaxSlotsRaw) {
    int d = kMaxSlotsRaw;
    while (k % d) d--;
    pp.ksplit = d;
  }
  pp.slot_pts = k / pp.ksplit;
  if (pp.kp < k) pp.kp = std::max(pp.slot_pts, (pp.kp / pp.slot_pts) * pp.slot_pts);
  const size_t part = pp.fused ? (size_t)p->cam * p->cam : (size_t)p->n * p->n;
  pp.bytes = (size_t)pp.bc * pp.kp * pp.unit_bytes + (size_t)pp.bc * nm * pp.ksplit * part * sizeof(float) +
             (size_t)pp.bc * p->res * p->res * sizeof(float2) + 1024;
  return pp;
}

size_t default_units(const oopao_pwfs_plan* p, int batch) {
  const size_t unit = ((size_t)p->res * p->n + (size_t)p->n_masks * p->n * p->n) * sizeof(float2);
  size_t u = std::max<size_t>(1, p->l2_budget / unit);
  return std::min<size_t>(u, (size_t)batch * p->k);
}

}  // namespace

extern "C" size_t oopao_pwfs_workspace_bytes(const oopao_pwfs_plan* p, int batch) {
  if (!p || batch < 1) return 0;
  const size_t u = default_units(p, batch);
  return std::max(plan_passes(p, batch, false, u).bytes, plan_passes(p, batch, true, u).bytes);
}

__global__ void pwfs_reduce_binned(const float* __restrict__ binned, float* __restrict__ frame, int cam2,
                                   int ksplit) {
  pdl_wait();
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cam2) return;
  const float* q = binned + (size_t)b * ksplit * cam2 + i;
  float s = 0.f;
  for (int t = 0; t < ksplit; t++) s += q[(size_t)t * cam2];
  frame[(size_t)b * cam2 + i] = s;
}

// ---- masks that vary along one axis only (measure_edge) ----

// out[b][x][y] = in[b][y][x] for res x res complex maps, through a 32 x 32 tile.
__global__ void __launch_bounds__(256) edge_transpose(const float2* __restrict__ in, float2* __restrict__ out,
                                                      int res) {
  __shared__ float2 tile[32][33];
  const size_t plane = (size_t)res * res;
  const float2* src = in + (size_t)blockIdx.z * plane;
  float2* dst = out + (size_t)blockIdx.z * plane;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  for (int dy = threadIdx.y; dy < 32; dy += 8) {
    const int y = y0 + dy, x = x0 + threadIdx.x;
    if (y < res && x < res) tile[dy][threadIdx.x] = src[(size_t)y * res + x];
  }
  __syncthreads();
  for (int dx = threadIdx.y; dx < 32; dx += 8) {
    const int x = x0 + dx, y = y0 + threadIdx.x;
    if (x < res && y < res) dst[(size_t)x * res + y] = tile[threadIdx.x][dx];
  }
}

struct EdgeBinArgs {
  const float* inten;   // mask m at inten + m * mask_stride: [slices][items][res][n] line intensity
  size_t mask_stride, slice_stride;
  int slices;           // partial sums over slices of groups (pwfs_srows_int)
  int axis[8];
  int res, n, off, cam, bin, n_masks;
  float* frame;         // [items][n_masks][cam][cam]
  float* raw;           // [items][n_masks][n][n] un-binned intensity, or null
};

// Camera frames of masks that vary along one axis only, from the line
// intensities of pwfs_srows_int: lines along x are the pupil rows
// [off, off+res) of the grid, lines along y its pupil columns (the field was
// transposed), the rest of the grid is dark.  One CTA per (camera row, mask,
// item): each thread sums a grid column over the camera row's bin rows
// (writing each grid pixel to raw when asked), then the columns are summed in
// bins.
__global__ void __launch_bounds__(256) edge_bin(EdgeBinArgs a) {
  extern __shared__ float colsum[];  // [n]
  const int cy = blockIdx.x, m = blockIdx.y, b = blockIdx.z;
  const int ax = a.axis[m], res = a.res, n = a.n;
  const float* I = a.inten + m * a.mask_stride + (size_t)b * res * n;
  for (int X = threadIdx.x; X < n; X += blockDim.x) {
    float s = 0.f;
    for (int dy = 0; dy < a.bin; dy++) {
      const int Y = cy * a.bin + dy;
      const int line = ax == 0 ? Y - a.off : X - a.off, pos = ax == 0 ? X : Y;
      float v = 0.f;
      if (line >= 0 && line < res)
        for (int sl = 0; sl < a.slices; sl++) v += I[sl * a.slice_stride + (size_t)line * n + pos];
      if (a.raw) a.raw[(((size_t)b * a.n_masks + m) * n + Y) * n + X] = v;
      s += v;
    }
    colsum[X] = s;
  }
  __syncthreads();
  for (int cx = threadIdx.x; cx < a.cam; cx += blockDim.x) {
    float t = 0.f;
    for (int dx = 0; dx < a.bin; dx++) t += colsum[cx * a.bin + dx];
    a.frame[(((size_t)b * a.n_masks + m) * a.cam + cy) * a.cam + cx] = t;
  }
}

namespace {
int measure_impl(const oopao_pwfs_plan* p, const float* opd, double phase_scale, int batch, float* frame,
                 float* raw, float* focal, void* ws, size_t ws_bytes, void* stream);
}  // namespace

extern "C" int oopao_pwfs_measure(const oopao_pwfs_plan* p, const float* opd, double phase_scale,
                                  int batch, float* frame, float* raw, void* ws, size_t ws_bytes,
                                  void* stream) {
  return measure_impl(p, opd, phase_scale, batch, frame, raw, nullptr, ws, ws_bytes, stream);
}

extern "C" int oopao_pwfs_measure_focal(const oopao_pwfs_plan* p, const float* opd, double phase_scale,
                                        int batch, float* frame, float* raw, float* focal, void* ws,
                                        size_t ws_bytes, void* stream) {
  OOPAO_CHECK_ARG(p && focal, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1, "batch must be >= 1");
  OOPAO_CUDA_TRY(cudaMemsetAsync(focal, 0, sizeof(float) * (size_t)batch * p->n * p->n, (cudaStream_t)stream));
  return measure_impl(p, opd, phase_scale, batch, frame, raw, focal, ws, ws_bytes, stream);
}

namespace {
// The two-pass path serves a call when the plan's single mask factorises,
// a compile-time two-pass plan exists, no focal-plane frame is wanted (it
// needs the 2-D spectrum, which the two passes never form) and the camera
// binning divides the column block (or raw data is wanted).
bool sep_applies(const oopao_pwfs_plan* p, bool focal, bool raw) {
  return p->sep && p->mask_sep && p->sep_on && p->variant >= 1 && p->n_masks == 1 && !focal &&
         (raw || p->sep->l_cols % p->bin == 0);
}

// Slots over modulation points for the two-pass column pass: a divisor d of
// K (at most `cap`) minimising (ctas/resident + 1) * (K/d + 2), the time
// model of CTAs that each sum K/d points after a fixed cost of about two
// points, with one CTA's time of tail.  Against a sweep of every divisor on
// GB300 (20x20 at batch 1/16/100, 40x40 at batch 1/4/16) it picks the
// fastest or one within 3%.
int sep_ksplit(const oopao_pwfs_plan* p, int bc, int cap, bool use_set = true, bool ad = false) {
  if (use_set && p->ksplit > 0 && p->ksplit <= cap) return p->ksplit;
  const SepPasses* s = ad ? p->sep_ad : p->sep;
  const int blocks = p->n / s->l_cols, resident = std::max(1, ad ? p->sep_ad_ctas : p->sep_cols_ctas);
  int best = 1;
  double best_t = 1e300;
  for (int d = 1; d <= p->k && d <= cap; d++) {
    if (p->k % d) continue;
    const double ctas = (double)blocks * d * bc;
    const double t = (ctas / resident + 1.0) * ((double)p->k / d + 2.0);
    if (t < best_t - 1e-9) {
      best_t = t;
      best = d;
    }
  }
  return best;
}

// Workspace of one two-pass chunk of bc items with ks slots.
size_t sep_chunk_bytes(const oopao_pwfs_plan* p, int bc, int ks, bool fused) {
  const size_t y = (size_t)p->ngroups * p->res * p->n * sizeof(float2);
  const size_t f = (size_t)p->res * p->res * sizeof(float2);
  const size_t part = (size_t)ks * (fused ? (size_t)p->cam * p->cam : (size_t)p->n * p->n) * sizeof(float);
  return (size_t)bc * (y + f + part) + 1024;
}

// The frames of masks that each vary along one axis only (edge_setup): per
// chunk of items the field and, for masks along y, its transpose; one
// two-pass row launch per mask over the groups of points that share the
// phasor of its axis (with the mask's 1-D factor as the filter); then
// edge_bin.  No column transform is needed.  OOPAO_ERR_WORKSPACE (nothing
// launched) when one item does not fit.
bool edge_applies(const oopao_pwfs_plan* p, bool focal) {
  return p->edge_1d && p->sep && p->sep_on && p->variant >= 1 && !focal;
}

int measure_edge(const oopao_pwfs_plan* p, const float* opd, double phase_scale, int batch, float* frame,
                 float* raw, char* base, size_t usable, cudaStream_t st) {
  const SepPasses* s = p->sep;
  const int n = p->n, res = p->res, cam = p->cam, nm = p->n_masks;
  bool any_y = false;
  for (int m = 0; m < nm; m++) any_y |= p->edge_axis[m] == 1;
  // slices of groups per row launch: enough CTAs for about two waves
  const int ngmax = std::max(p->ngroups, p->nygroups), blocks = ceil_div(res, s->l_rows);
  const int target = 2 * std::max(1, p->sep_cols_ctas);
  auto slices_for = [&](int nb) { return std::max(1, std::min(ngmax, ceil_div(target, blocks * nb))); };
  // per item: the field (and its transpose), then each mask's line intensity slices
  const int sl1 = slices_for(1);
  auto item_bytes = [&](int sl) {
    return sizeof(float2) * (size_t)res * res * (any_y ? 2 : 1) + sizeof(float) * (size_t)nm * sl * res * n;
  };
  if (item_bytes(sl1) + 1024 > usable) return OOPAO_ERR_WORKSPACE;
  int bc = (int)std::min<size_t>((size_t)batch, (usable - 1024) / item_bytes(sl1));
  const int slices = slices_for(bc);
  float2* field = (float2*)base;
  float2* field_t = field + (size_t)bc * res * res;
  float* inten = (float*)(field_t + (any_y ? (size_t)bc * res * res : 0));
  EdgeBinArgs ea{};
  ea.inten = inten;
  ea.slices = slices;
  ea.slice_stride = (size_t)bc * res * n;
  ea.mask_stride = (size_t)slices * bc * res * n;
  for (int m = 0; m < nm; m++) ea.axis[m] = p->edge_axis[m];
  ea.res = res; ea.n = n; ea.off = p->off; ea.cam = cam; ea.bin = p->bin; ea.n_masks = nm;
  const float* gsum = p->weights_on ? p->d_gsum_w : p->d_gsum;
  // the line phasors carry the 1/n^2 of the 2-D inverse transform, but only
  // one axis goes through the unnormalised transform pair (a gain of n): n^2
  // back in intensity
  const float nsq = (float)n * (float)n;
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    OOPAO_CUDA_TRY(launch_pdl(pwfs_field, dim3(ceil_div(res * res, 256), nb), dim3(256), 0, st,
                              opd + (size_t)b0 * res * res, (float)phase_scale, (const float*)p->d_amp, field,
                              res * res));
    launches++;
    if (any_y) {
      edge_transpose<<<dim3(ceil_div(res, 32), ceil_div(res, 32), nb), dim3(32, 8), 0, st>>>(field, field_t, res);
      launches++;
    }
    for (int m = 0; m < nm; m++) {
      const bool ya = p->edge_axis[m] == 1;
      const int ng = ya ? p->nygroups : p->ngroups, g_per = ceil_div(ng, slices);
      SepRowsIntArgs ra{p->d_tw, ya ? field_t : field, ya ? p->d_ygrowfac : p->d_growfac,
                        p->d_edge_filt + (size_t)m * n, gsum + (ya ? p->k : 0), inten + (size_t)m * ea.mask_stride,
                        ea.slice_stride, res, ng, g_per, nsq};
      // every slice writes its partial sums (a slice past the last group writes zeros)
      OOPAO_CUDA_TRY(launch_pdl(s->rows_int, dim3(blocks, slices, nb), dim3(s->t * s->l_rows), s->smem_rows, st,
                                ra));
      launches++;
    }
    ea.frame = frame + (size_t)b0 * nm * cam * cam;
    ea.raw = raw ? raw + (size_t)b0 * nm * n * n : nullptr;
    edge_bin<<<dim3(cam, nm, nb), 256, sizeof(float) * n, st>>>(ea);
    launches++;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

// Two-pass measurement (pwfs_sep.cuh): field, filtered rows of every
// row-transform group, filtered columns summed over slots of points and
// binned, then the fixed-order sum of the slots.  Returns
// OOPAO_ERR_WORKSPACE (without launching) when one item does not fit.
int measure_sep(const oopao_pwfs_plan* p, const float* opd, double phase_scale, int batch, float* frame,
                float* raw, char* base, size_t usable, cudaStream_t st) {
  const SepPasses* s = p->sep;
  const int n = p->n, res = p->res, k = p->k, cam = p->cam, ng = p->ngroups;
  const bool fused = raw == nullptr;
  const int cap = fused ? kMaxSlotsBinned : kMaxSlotsRaw;
  const size_t item = sep_chunk_bytes(p, 1, 1, fused);
  int bc = (int)std::min<size_t>((size_t)batch, std::max<size_t>(1, p->l2_budget / item));
  int ks = sep_ksplit(p, bc, cap);
  while (bc > 1 && sep_chunk_bytes(p, bc, ks, fused) > usable) {
    bc = (bc + 1) / 2;
    ks = sep_ksplit(p, bc, cap);
  }
  if (sep_chunk_bytes(p, bc, ks, fused) > usable) return OOPAO_ERR_WORKSPACE;
  float2* y = (float2*)base;
  float2* field = y + (size_t)bc * ng * res * n;
  float* part = (float*)(field + (size_t)bc * res * res);
  PwfsProfile* prof = p->prof->enabled ? p->prof : nullptr;
  auto mark = [&](int stage) {
    if (prof) prof->mark(stage, st);
  };
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    mark(0);
    OOPAO_CUDA_TRY(launch_pdl(pwfs_field, dim3(ceil_div(res * res, 256), nb), dim3(256), 0, st,
                              opd + (size_t)b0 * res * res, (float)phase_scale, (const float*)p->d_amp, field,
                              res * res));
    mark(0);
    SepRowsArgs ra{p->d_tw, field, p->d_growfac, p->d_mrow, y, res, ng, 0 /* support at row/column 0 */};
    mark(0);
    OOPAO_CUDA_TRY(launch_pdl(s->rows, dim3(ceil_div(res, s->l_rows), ng, nb), dim3(s->t * s->l_rows), s->smem_rows,
                              st, ra));
    mark(0);
    SepColsArgs ca{p->d_tw, p->d_mcol, y, p->d_group, p->d_colfac, weights_of(p), nullptr, nullptr,
                   fused ? nullptr : part, fused ? part : nullptr, res, 0 /* support at row/column 0 */, ng, k / ks, ks, p->bin, cam};
    mark(1);
    OOPAO_CUDA_TRY(launch_pdl(s->cols[kSepIntensity], dim3(n / s->l_cols, ks, nb), dim3(s->t * s->l_cols),
                              s->smem_cols(res), st, ca));
    mark(1);
    mark(3);
    if (fused) {
      OOPAO_CUDA_TRY(launch_pdl(pwfs_reduce_binned, dim3(ceil_div(cam * cam, 256), nb), dim3(256), 0, st,
                                (const float*)part, frame + (size_t)b0 * cam * cam, cam * cam, ks));
    } else {
      pwfs_bin<<<dim3(cam, nb), 128, 0, st>>>(part, frame + (size_t)b0 * cam * cam,
                                              raw + (size_t)b0 * n * n, n, cam, p->bin, ks);
    }
    mark(3);
    launches += 4;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

int measure_impl(const oopao_pwfs_plan* p, const float* opd, double phase_scale, int batch, float* frame,
                 float* raw, float* focal, void* ws, size_t ws_bytes, void* stream) {
  OOPAO_CHECK_ARG(p && opd && frame && ws, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1, "batch must be >= 1");
  cudaStream_t st = (cudaStream_t)stream;
  uintptr_t base = ((uintptr_t)ws + 255) & ~(uintptr_t)255;
  const size_t usable = ws_bytes > (base - (uintptr_t)ws) ? ws_bytes - (base - (uintptr_t)ws) : 0;
  if (edge_applies(p, focal != nullptr)) {
    const int r = measure_edge(p, opd, phase_scale, batch, frame, raw, (char*)base, usable, st);
    if (r != OOPAO_ERR_WORKSPACE) return r;
  }
  if (sep_applies(p, focal != nullptr, raw != nullptr)) {
    const int r = measure_sep(p, opd, phase_scale, batch, frame, raw, (char*)base, usable, st);
    if (r != OOPAO_ERR_WORKSPACE) return r;  // else the three-pass path below, in smaller passes
  }
  size_t units = default_units(p, batch);
  PassPlan pp = plan_passes(p, batch, raw != nullptr, units);
  while (pp.bytes > usable && units > 1) {
    units = units / 2;
    pp = plan_passes(p, batch, raw != nullptr, units);
  }
  if (pp.bytes > usable) {
    oopao_set_last_error("workspace smaller than one pass needs", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  const int n = p->n, res = p->res, k = p->k, cam = p->cam, nm = p->n_masks;
  float2* y = (float2*)base;
  float2* z = y + (size_t)pp.bc * pp.kp * res * n;
  float2* field = z + (size_t)pp.bc * nm * pp.kp * n * n;
  float* part = (float*)(field + (size_t)pp.bc * res * res);
  const FastPasses* f = pp.fast ? p->fast : nullptr;
  if (nm > 1 && (!f || !f->cols_m)) {
    oopao_set_last_error("several masks need a compile-time plan with one stage-B butterfly per thread",
                         __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  PwfsProfile* prof = p->prof->enabled ? p->prof : nullptr;
  auto mark = [&](int stage) {
    if (prof) prof->mark(stage, st);
  };
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += pp.bc) {
    const int bc = std::min(pp.bc, batch - b0);
    mark(0);
    {
      dim3 g0(ceil_div(res * res, 256), bc);
      pwfs_field<<<g0, 256, 0, st>>>(opd + (size_t)b0 * res * res, (float)phase_scale, p->d_amp, field,
                                     res * res);
    }
    mark(0);
    launches += 1;
    for (int k0 = 0; k0 < k; k0 += pp.kp) {
      const int kc = std::min(pp.kp, k - k0);
      // whole items: one row transform per distinct x_k; otherwise one per point
      const bool grouped = (kc == k);
      const float2* gtab = grouped ? p->d_growfac : p->d_rowfac;
      const int g0 = grouped ? 0 : k0, ng = grouped ? p->ngroups : kc;
      RowsFwdArgs ra{p->fft, p->d_tw, field, gtab, y, res, n, g0, ng, p->off, p->rows_per_cta};
      mark(0);
      if (f) {
        dim3 g1(ceil_div(res, f->l_rows), ng, bc);
        f->rows<<<g1, f->t * f->l_rows, f->smem_rows, st>>>(ra);
      } else {
        dim3 g1(ceil_div(res, p->rows_per_cta), ng, bc);
        pwfs_rows_fwd<<<g1, kThreads, rows_smem(n, p->rows_per_cta), st>>>(ra);
      }
      mark(0);
      ColsArgs ca{p->fft, p->d_tw, p->d_mask, y, grouped ? p->d_group : nullptr, p->d_colfac, z,
                  res, n, k0, kc, ng, p->off, p->cols_per_cta,
                  focal ? focal + (size_t)b0 * n * n : nullptr, (float)((double)n * n)};
      mark(1);
      if (nm > 1) {
        ca.mask = p->d_masks;
        ca.n_masks = nm;
        dim3 g2(ceil_div(n, f->l_cols), kc, bc);
        f->cols_m<<<g2, f->t * f->l_cols, f->smem_cols_m, st>>>(ca);
      } else if (f && p->cols3_ctas > 0) {
        // persistent column pass: each CTA keeps one column block's mask and
        // streams its Y tiles with TMA over the (item, point) units
        CUtensorMap ymap;
        const int es = encode_y_map(&ymap, y, n, (size_t)bc * ng * res, f->l_cols3, res);
        if (es) return es;
        ca.items = bc;
        ca.err = p->d_err;
        const int blocks = n / f->l_cols3;
        const int per = std::max(1, std::min(bc * kc, p->cols3_ctas / blocks));
        f->cols3<<<dim3(blocks, per), f->t * f->l_cols3, f->smem_cols3(res), st>>>(ymap, ca);
      } else if (f) {
        dim3 g2(ceil_div(n, f->l_cols), kc, bc);
        f->cols<<<g2, f->t * f->l_cols, f->smem_cols, st>>>(ca);
      } else {
        dim3 g2(ceil_div(n, p->cols_per_cta), kc, bc);
        pwfs_cols<<<g2, kThreads, rows_smem(n, p->cols_per_cta), st>>>(ca);
      }
      mark(1);
      RowsInvArgs ia{p->fft, p->d_tw, z, weights_of(p), pp.fused ? nullptr : part, pp.fused ? part : nullptr,
                     n, k0, kc, k0 / pp.slot_pts, pp.slot_pts, pp.ksplit, p->inv_rows_per_cta, p->bin, cam};
      mark(2);
      if (f) {
        dim3 g3(ceil_div(n, f->l_inv), kc / pp.slot_pts, bc * nm);
        f->inv<<<g3, f->t * f->l_inv, f->smem_inv, st>>>(ia);
      } else {
        dim3 g3(ceil_div(n, p->inv_rows_per_cta), kc / pp.slot_pts, bc);
        pwfs_rows_inv<<<g3, kThreads, inv_smem(n, p->inv_rows_per_cta), st>>>(ia);
      }
      mark(2);
      launches += 3;
    }
    mark(3);
    if (pp.fused) {
      dim3 g4(ceil_div(cam * cam, 256), bc * nm);
      pwfs_reduce_binned<<<g4, 256, 0, st>>>(part, frame + (size_t)b0 * nm * cam * cam, cam * cam, pp.ksplit);
    } else {
      dim3 g4(cam, bc * nm);
      pwfs_bin<<<g4, 128, 0, st>>>(part, frame + (size_t)b0 * nm * cam * cam,
                                   raw ? raw + (size_t)b0 * nm * n * n : nullptr, n, cam, p->bin, pp.ksplit);
    }
    mark(3);
    launches += 1;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
}  // namespace

extern "C" int oopao_pwfs_set_signal_processing(oopao_pwfs_plan* p, int mode, int nq,
                                                const int* quad_origin, const unsigned char* valid,
                                                const float* ref2d, double units, double norma_const) {
  OOPAO_CHECK_ARG(p && valid, "NULL argument");
  OOPAO_CHECK_ARG(mode >= 0 && mode <= 6, "unknown signal-processing mode");
  const bool slopes = mode <= 2;
  int n2d;
  if (slopes) {
    OOPAO_CHECK_ARG(quad_origin != nullptr && nq > 0, "slopes modes need quadrant geometry");
    for (int q = 0; q < 4; q++) {
      OOPAO_CHECK_ARG(quad_origin[2 * q] >= 0 && quad_origin[2 * q] + nq <= p->cam &&
                          quad_origin[2 * q + 1] >= 0 && quad_origin[2 * q + 1] + nq <= p->cam,
                      "quadrant outside the camera frame");
      p->q_r0[q] = quad_origin[2 * q];
      p->q_c0[q] = quad_origin[2 * q + 1];
    }
    n2d = 2 * nq * nq;
  } else {
    n2d = p->cam * p->cam;
  }
  const int nvalid_cells = slopes ? nq * nq : p->cam * p->cam;
  std::vector<int> idx;
  int nvalid = 0;
  for (int i = 0; i < nvalid_cells; i++) nvalid += valid[i] ? 1 : 0;
  if (slopes) {
    // validSignal = concatenate((validI4Q, validI4Q)); row-major order
    for (int h = 0; h < 2; h++)
      for (int i = 0; i < nvalid_cells; i++)
        if (valid[i]) idx.push_back(h * nvalid_cells + i);
  } else {
    for (int i = 0; i < nvalid_cells; i++)
      if (valid[i]) idx.push_back(i);
  }
  OOPAO_CHECK_ARG(!idx.empty(), "no valid pixel");
  cudaFree(p->d_valid);
  cudaFree(p->d_ref2d);
  cudaFree(p->d_sig_index);
  p->d_valid = nullptr; p->d_ref2d = nullptr; p->d_sig_index = nullptr;
  OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_valid, nvalid_cells));
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_valid, valid, nvalid_cells, cudaMemcpyHostToDevice));
  if (ref2d) {
    OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_ref2d, sizeof(float) * n2d));
    OOPAO_CUDA_TRY(cudaMemcpy(p->d_ref2d, ref2d, sizeof(float) * n2d, cudaMemcpyHostToDevice));
  }
  OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_sig_index, sizeof(int) * idx.size()));
  OOPAO_CUDA_TRY(cudaMemcpy(p->d_sig_index, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice));
  {
    std::vector<int> inv(n2d, -1);
    for (size_t t = 0; t < idx.size(); t++) inv[idx[t]] = (int)t;
    cudaFree(p->d_sig_inv);
    p->d_sig_inv = nullptr;
    OOPAO_CUDA_TRY(cudaMalloc((void**)&p->d_sig_inv, sizeof(int) * inv.size()));
    OOPAO_CUDA_TRY(cudaMemcpy(p->d_sig_inv, inv.data(), sizeof(int) * inv.size(), cudaMemcpyHostToDevice));
  }
  p->sp_mode = mode;
  p->nq = nq;
  p->n2d = n2d;
  p->n_signal = (int)idx.size();
  p->slopes_units = (float)units;
  p->norma_const = (float)norma_const;
  p->cam2 = nvalid;  // number of valid cells
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_n_signal(const oopao_pwfs_plan* p) { return p ? p->n_signal : -1; }

// Tangent / adjoint of the slopesMaps signal (signalProcessing
// OOPAO/Pyramid.py:838-854): s = units (Q/norma - ref), Q = (Sx, Sy) linear
// in the masked quadrants, norma = mean over valid cells of the quadrant sum
// (a constant for slopesMaps_incidence_flux).
struct SignalAdArgs {
  const float* frame0;  // [B or 1][cam][cam] operating-point frames
  int frame0_per_item;
  const float* dframe;  // tangent frames [B][cam][cam]
  const float* sbar;    // signal cotangents [B][n_signal]
  float* dsig2d;        // [B][n2d]
  float* dsig;          // [B][n_signal]
  float* fbar;          // [B][cam][cam]
  const unsigned char* valid;
  const int* sig_index;
  const int* sig_inv;
  int mode, cam, nq, n2d, n_signal, n_valid;
  int q_r0[4], q_c0[4];
  float units, norma_const;
};

__device__ __forceinline__ void quad_values(const float* fr, const SignalAdArgs& a, int r, int c, float* v) {
#pragma unroll
  for (int q = 0; q < 4; q++) v[q] = fr[(a.q_r0[q] + r) * a.cam + a.q_c0[q] + c];
}

__global__ void pwfs_signal_jvp(SignalAdArgs a) {
  __shared__ float red[33];
  const int b = blockIdx.x;
  const float* f0 = a.frame0 + (a.frame0_per_item ? (size_t)b * a.cam * a.cam : 0);
  const float* df = a.dframe + (size_t)b * a.cam * a.cam;
  const int nq2 = a.nq * a.nq;
  float p0 = 0.f, p1 = 0.f;
  for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
    if (!a.valid[idx]) continue;
    float v0[4], v1[4];
    quad_values(f0, a, idx / a.nq, idx % a.nq, v0);
    quad_values(df, a, idx / a.nq, idx % a.nq, v1);
    p0 += ((v0[0] + v0[1]) + v0[2]) + v0[3];
    p1 += ((v1[0] + v1[1]) + v1[2]) + v1[3];
  }
  const float s0 = block_sum(p0, red);
  const float s1 = block_sum(p1, red);
  const float n0 = a.mode == 0 ? s0 / (float)a.n_valid : a.norma_const;
  const float dn = a.mode == 0 ? s1 / (float)a.n_valid : 0.f;
  float* s2 = a.dsig2d + (size_t)b * a.n2d;
  for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
    float sx = 0.f, sy = 0.f, dx = 0.f, dy = 0.f;
    if (a.valid[idx]) {
      float v0[4], v1[4];
      quad_values(f0, a, idx / a.nq, idx % a.nq, v0);
      quad_values(df, a, idx / a.nq, idx % a.nq, v1);
      sx = ((v0[0] - v0[1]) + v0[3]) - v0[2];
      sy = ((v0[0] - v0[3]) + v0[1]) - v0[2];
      dx = ((v1[0] - v1[1]) + v1[3]) - v1[2];
      dy = ((v1[0] - v1[3]) + v1[1]) - v1[2];
    }
    s2[idx] = a.units * (dx / n0 - sx * dn / (n0 * n0));
    s2[nq2 + idx] = a.units * (dy / n0 - sy * dn / (n0 * n0));
  }
  __syncthreads();
  float* sg = a.dsig + (size_t)b * a.n_signal;
  for (int t = threadIdx.x; t < a.n_signal; t += blockDim.x) sg[t] = s2[a.sig_index[t]];
}

__global__ void pwfs_signal_vjp(SignalAdArgs a) {
  __shared__ float red[33];
  const int b = blockIdx.x;
  const float* f0 = a.frame0 + (a.frame0_per_item ? (size_t)b * a.cam * a.cam : 0);
  const float* sb = a.sbar + (size_t)b * a.n_signal;
  const int nq2 = a.nq * a.nq;
  float p0 = 0.f, pq = 0.f;
  for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
    if (!a.valid[idx]) continue;
    float v0[4];
    quad_values(f0, a, idx / a.nq, idx % a.nq, v0);
    p0 += ((v0[0] + v0[1]) + v0[2]) + v0[3];
    const int ix = a.sig_inv[idx], iy = a.sig_inv[nq2 + idx];
    const float qx = ix >= 0 ? sb[ix] : 0.f, qy = iy >= 0 ? sb[iy] : 0.f;
    const float sx = ((v0[0] - v0[1]) + v0[3]) - v0[2];
    const float sy = ((v0[0] - v0[3]) + v0[1]) - v0[2];
    pq += qx * sx + qy * sy;
  }
  const float s0 = block_sum(p0, red);
  const float sq = block_sum(pq, red);
  const float n0 = a.mode == 0 ? s0 / (float)a.n_valid : a.norma_const;
  const float nbar = a.mode == 0 ? -a.units * sq / (n0 * n0) : 0.f;
  const float dn = a.mode == 0 ? nbar / (float)a.n_valid : 0.f;
  float* fb = a.fbar + (size_t)b * a.cam * a.cam;
  for (int i = threadIdx.x; i < a.cam * a.cam; i += blockDim.x) fb[i] = 0.f;
  __syncthreads();
  for (int idx = threadIdx.x; idx < nq2; idx += blockDim.x) {
    if (!a.valid[idx]) continue;
    const int r = idx / a.nq, c = idx % a.nq;
    const int ix = a.sig_inv[idx], iy = a.sig_inv[nq2 + idx];
    const float qx = (ix >= 0 ? sb[ix] : 0.f) * a.units / n0;
    const float qy = (iy >= 0 ? sb[iy] : 0.f) * a.units / n0;
    fb[(a.q_r0[0] + r) * a.cam + a.q_c0[0] + c] = qx + qy + dn;
    fb[(a.q_r0[1] + r) * a.cam + a.q_c0[1] + c] = -qx + qy + dn;
    fb[(a.q_r0[2] + r) * a.cam + a.q_c0[2] + c] = -qx - qy + dn;
    fb[(a.q_r0[3] + r) * a.cam + a.q_c0[3] + c] = qx - qy + dn;
  }
}

namespace {
int signal_ad_args(const oopao_pwfs_plan* p, SignalAdArgs* a) {
  OOPAO_CHECK_ARG(p->sp_mode == 0 || p->sp_mode == 1,
                  "signal tangent/adjoint support slopesMaps and slopesMaps_incidence_flux");
  memset(a, 0, sizeof(*a));
  a->valid = p->d_valid;
  a->sig_index = p->d_sig_index;
  a->sig_inv = p->d_sig_inv;
  a->mode = p->sp_mode;
  a->cam = p->cam;
  a->nq = p->nq;
  a->n2d = p->n2d;
  a->n_signal = p->n_signal;
  a->n_valid = p->cam2;
  for (int q = 0; q < 4; q++) { a->q_r0[q] = p->q_r0[q]; a->q_c0[q] = p->q_c0[q]; }
  a->units = p->slopes_units;
  a->norma_const = p->norma_const;
  return OOPAO_OK;
}
}  // namespace

extern "C" int oopao_pwfs_signal_jvp(const oopao_pwfs_plan* p, const float* frame0, int frame0_batch,
                                     const float* dframe, int batch, float* dsignal_2d, float* dsignal,
                                     void* stream) {
  OOPAO_CHECK_ARG(p && frame0 && dframe && dsignal_2d && dsignal, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1 && (frame0_batch == 1 || frame0_batch == batch), "frame0_batch must be 1 or batch");
  SignalAdArgs a;
  int s = signal_ad_args(p, &a);
  if (s) return s;
  a.frame0 = frame0;
  a.frame0_per_item = frame0_batch != 1;
  a.dframe = dframe;
  a.dsig2d = dsignal_2d;
  a.dsig = dsignal;
  pwfs_signal_jvp<<<batch, 256, 0, (cudaStream_t)stream>>>(a);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_signal_vjp(const oopao_pwfs_plan* p, const float* frame0, int frame0_batch,
                                     const float* sbar, int batch, float* fbar, void* stream) {
  OOPAO_CHECK_ARG(p && frame0 && sbar && fbar, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1 && (frame0_batch == 1 || frame0_batch == batch), "frame0_batch must be 1 or batch");
  SignalAdArgs a;
  int s = signal_ad_args(p, &a);
  if (s) return s;
  a.frame0 = frame0;
  a.frame0_per_item = frame0_batch != 1;
  a.sbar = sbar;
  a.fbar = fbar;
  pwfs_signal_vjp<<<batch, 256, 0, (cudaStream_t)stream>>>(a);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_signal(const oopao_pwfs_plan* p, const float* frame, int batch,
                                 float* signal_2d, float* signal, float* norma, void* stream) {
  OOPAO_CHECK_ARG(p && frame && signal_2d && signal, "NULL argument");
  OOPAO_CHECK_ARG(p->sp_mode >= 0, "signal processing not configured");
  OOPAO_CHECK_ARG(batch >= 1, "batch must be >= 1");
  SignalArgs a;
  a.frame = frame; a.valid = p->d_valid; a.ref2d = p->d_ref2d; a.sig_index = p->d_sig_index;
  a.sig_inv = p->d_sig_inv;
  a.signal_2d = signal_2d; a.signal = signal; a.norma = norma;
  a.mode = p->sp_mode; a.cam = p->cam; a.nq = p->nq; a.n2d = p->n2d; a.n_signal = p->n_signal;
  a.n_valid = p->cam2;
  for (int q = 0; q < 4; q++) { a.q_r0[q] = p->q_r0[q]; a.q_c0[q] = p->q_c0[q]; }
  a.units = p->slopes_units; a.norma_const = p->norma_const;
  OOPAO_CUDA_TRY(launch_pdl(pwfs_signal, dim3(batch), dim3(512), 0, (cudaStream_t)stream, a));
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_profiling(oopao_pwfs_plan* p, int enable) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  p->prof->enabled = enable != 0;
  p->prof->used = 0;
  p->prof->stage.clear();
  p->prof->open = false;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_profile_read(oopao_pwfs_plan* p, double* ms, int* launches) {
  OOPAO_CHECK_ARG(p && ms && launches, "NULL argument");
  PwfsProfile* pr = p->prof;
  for (int s = 0; s < 4; s++) { ms[s] = 0.0; launches[s] = 0; }
  OOPAO_CHECK_ARG(pr->used % 2 == 0 && pr->used / 2 == pr->stage.size(), "profile events out of step");
  if (pr->used) OOPAO_CUDA_TRY(cudaEventSynchronize(pr->pool[pr->used - 1]));
  for (size_t c = 0; c < pr->stage.size(); c++) {
    float t = 0.f;
    OOPAO_CUDA_TRY(cudaEventElapsedTime(&t, pr->pool[2 * c], pr->pool[2 * c + 1]));
    ms[pr->stage[c]] += t;
    launches[pr->stage[c]] += 1;
  }
  pr->used = 0;
  pr->stage.clear();
  return OOPAO_OK;
}

// ---------------------------------------------------------------------------
// Tangent (JVP) and adjoint (VJP) of the propagation, see pwfs_ad.cuh.
// ---------------------------------------------------------------------------
#include "pwfs_ad.cuh"

namespace {

const AdPasses* ad_passes(int n) {
  static const AdPasses a72 = make_ad<72, 8, 9, 9, 12>();
  static const AdPasses a112 = make_ad<112, 16, 7, 8, 16>();
  static const AdPasses a128 = make_ad<128, 16, 8, 8, 16>();
  static const AdPasses a264 = make_ad<264, 24, 11, 12, 12>();
  static const AdPasses a504 = make_ad<504, 24, 21, 12, 12>();
  static const AdPasses a1920 = make_ad<1920, 48, 40, 48, 6>();
  switch (n) {
    case 72: return &a72;
    case 112: return &a112;
    case 128: return &a128;
    case 264: return &a264;
    case 504: return &a504;
    case 1920: return &a1920;
    default: return nullptr;
  }
}

int ad_setup(const oopao_pwfs_plan* p, const AdPasses** out) {
  const AdPasses* a = ad_passes(p->n);
  if (p->n_masks != 1) {
    oopao_set_last_error("tangent/adjoint passes take a plan with one mask", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  if (!a || !p->fast || p->variant < 1) {
    oopao_set_last_error("tangent/adjoint passes exist for n_fft in {72,112,128,264,504,1920} only", __FILE__,
                         __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  cudaError_t e = cudaFuncSetAttribute(a->field, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smem_field);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(a->jvp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smem_jvp);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(a->vjp_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smem_vjp_a);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(a->vjp_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smem_vjp_b);
  if (e != cudaSuccess) {
    oopao_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return OOPAO_ERR_CUDA;
  }
  *out = a;
  return OOPAO_OK;
}

// i * dopd * scale * amp * exp(i opd0 * scale): tangent of the pupil field
__global__ void pwfs_field_tangent(const float* __restrict__ opd0, const float* __restrict__ dopd, float scale,
                                   const float* __restrict__ amp, float2* __restrict__ out, int npix,
                                   int opd0_per_item) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float am = amp[i];
  float2 v = make_float2(0.f, 0.f);
  if (am != 0.f) {
    float s, c;
    sincosf(opd0[(opd0_per_item ? (size_t)b * npix : 0) + i] * scale, &s, &c);
    const float d = dopd[(size_t)b * npix + i] * scale * am;
    v = make_float2(-s * d, c * d);
  }
  out[(size_t)b * npix + i] = v;
}

__global__ void pwfs_reduce_scaled(const float* __restrict__ part, float* __restrict__ out, int m, int ksplit,
                                   float scale) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float* q = part + (size_t)b * ksplit * m + i;
  float s = 0.f;
  for (int t = 0; t < ksplit; t++) s += q[(size_t)t * m];
  out[(size_t)b * m + i] = s * scale;
}

int ad_ksplit(const oopao_pwfs_plan* p, int rows, int bc, int cap) {
  const int want = ceil_div(kTargetCtas, std::max(1, ceil_div(rows, 12) * bc));
  int best = 1;
  for (int d = 1; d <= p->k && d <= cap; d++) {
    if (p->k % d) continue;
    best = d;
    if (d >= want) break;
  }
  return best;
}

size_t ad_item_bytes(const oopao_pwfs_plan* p, int ksplit, bool vjp) {
  const size_t yz = (size_t)p->k * ((size_t)p->res * p->n + (size_t)p->n * p->n) * sizeof(float2);
  const size_t fld = (size_t)p->res * p->res * sizeof(float2);
  const size_t part = (size_t)ksplit * (vjp ? (size_t)p->res * p->res : (size_t)p->cam * p->cam) * sizeof(float);
  return yz + fld + part;
}

}  // namespace

extern "C" size_t oopao_pwfs_ad_workspace_bytes(const oopao_pwfs_plan* p, int batch) {
  if (!p || batch < 1) return 0;
  const size_t g = (size_t)p->k * p->n * p->n * sizeof(float2) + (size_t)p->res * p->res * sizeof(float2);
  size_t per = std::max(ad_item_bytes(p, std::min(p->k, kMaxSlotsBinned), false),
                        ad_item_bytes(p, std::min(p->k, kMaxSlotsBinned), true));
  const size_t cap_items = std::max<size_t>(1, p->l2_budget / per);
  return g + per * std::min<size_t>((size_t)batch, cap_items) + 4096;
}

namespace {
// Tangent through the two passes: the operating point's filtered rows, then
// its fields G_k stored once ([K][N][N], the storing column pass), then per
// chunk of tangents the filtered rows of i dphi W and the tangent column
// pass, which sums 2 w_k Re(conj(G_k) dG_k) against the stored G_k.  Its
// grid puts the items fastest: the items of one (column block, slot) run side
// by side and share the G_k columns through L2.  OOPAO_ERR_WORKSPACE (nothing launched) when one item
// does not fit.
int jvp_sep(const oopao_pwfs_plan* p, const float* opd0, int opd0_batch, const float* dopd, double phase_scale,
            int batch, float* dframe, char* base, size_t usable, cudaStream_t st) {
  const SepPasses* s = p->sep_ad;
  const int n = p->n, res = p->res, k = p->k, cam = p->cam, ng = p->ngroups;
  float2* g = (float2*)base;  // [k][n][n] operating-point fields
  float2* w0 = g + (size_t)k * n * n;
  char* chunk = (char*)(w0 + (size_t)res * res);
  const size_t fixed = (size_t)(chunk - base);
  if (usable <= fixed) return OOPAO_ERR_WORKSPACE;
  const size_t avail = usable - fixed;
  int bc = opd0_batch == 1 ? batch : 1;
  bc = (int)std::min<size_t>((size_t)bc, std::max<size_t>(1, p->l2_budget / sep_chunk_bytes(p, 1, 1, true)));
  // slot counts from the model: a count set for measure calls (autotuner) was
  // timed on another batch and another kernel form
  int ks = sep_ksplit(p, bc, kMaxSlotsBinned, false, true);
  while (bc > 1 && sep_chunk_bytes(p, bc, ks, true) > avail) {
    bc = (bc + 1) / 2;
    ks = sep_ksplit(p, bc, kMaxSlotsBinned, false, true);
  }
  if (sep_chunk_bytes(p, bc, ks, true) > avail) return OOPAO_ERR_WORKSPACE;
  float2* y = (float2*)chunk;
  float2* fld = y + (size_t)bc * ng * res * n;
  float* part = (float*)(fld + (size_t)bc * res * res);
  const int ks0 = sep_ksplit(p, 1, kMaxSlotsBinned, false, true);
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    const float* o0 = opd0 + (opd0_batch == 1 ? 0 : (size_t)b0 * res * res);
    if (b0 == 0 || opd0_batch != 1) {
      pwfs_field<<<dim3(ceil_div(res * res, 256), 1), 256, 0, st>>>(o0, (float)phase_scale, p->d_amp, w0, res * res);
      SepRowsArgs ra{p->d_tw, w0, p->d_growfac, p->d_mrow, y, res, ng, 0 /* support at row/column 0 */};
      s->rows<<<dim3(ceil_div(res, s->l_rows), ng, 1), s->t * s->l_rows, s->smem_rows, st>>>(ra);
      SepColsArgs ca{p->d_tw, p->d_mcol, y, p->d_group, p->d_colfac, nullptr, nullptr, g, nullptr, nullptr,
                     res, 0 /* support at row/column 0 */, ng, k / ks0, ks0, p->bin, cam};
      s->cols[kSepStore]<<<dim3(n / s->l_cols, ks0, 1), s->t * s->l_cols, s->smem_cols(res), st>>>(ca);
      launches += 3;
    }
    pwfs_field_tangent<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(
        o0, dopd + (size_t)b0 * res * res, (float)phase_scale, p->d_amp, fld, res * res, 0);
    SepRowsArgs ra{p->d_tw, fld, p->d_growfac, p->d_mrow, y, res, ng, 0 /* support at row/column 0 */};
    s->rows<<<dim3(ceil_div(res, s->l_rows), ng, nb), s->t * s->l_rows, s->smem_rows, st>>>(ra);
    SepColsArgs ca{p->d_tw, p->d_mcol, y, p->d_group, p->d_colfac, weights_of(p), g, nullptr, nullptr, part,
                   res, 0 /* support at row/column 0 */, ng, k / ks, ks, p->bin, cam};
    s->cols[kSepTangent]<<<dim3(nb, ks, n / s->l_cols), s->t * s->l_cols, s->smem_cols(res), st>>>(ca);
    pwfs_reduce_binned<<<dim3(ceil_div(cam * cam, 256), nb), 256, 0, st>>>(part, dframe + (size_t)b0 * cam * cam,
                                                                           cam * cam, ks);
    launches += 4;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
}  // namespace

extern "C" int oopao_pwfs_jvp(const oopao_pwfs_plan* p, const float* opd0, int opd0_batch, const float* dopd,
                              double phase_scale, int batch, float* dframe, void* ws, size_t ws_bytes,
                              void* stream) {
  OOPAO_CHECK_ARG(p && opd0 && dopd && dframe && ws, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1 && (opd0_batch == 1 || opd0_batch == batch), "opd0_batch must be 1 or batch");
  cudaStream_t st = (cudaStream_t)stream;
  uintptr_t base = ((uintptr_t)ws + 255) & ~(uintptr_t)255;
  OOPAO_CHECK_ARG(ws_bytes > base - (uintptr_t)ws, "workspace too small");
  const size_t usable = ws_bytes - (base - (uintptr_t)ws);
  if (sep_applies(p, false, false) && p->sep_ad->l_cols % p->bin == 0) {
    const int r = jvp_sep(p, opd0, opd0_batch, dopd, phase_scale, batch, dframe, (char*)base, usable, st);
    if (r != OOPAO_ERR_WORKSPACE) return r;  // else the three-pass tangent below
  }
  const AdPasses* ad = nullptr;
  int st0 = ad_setup(p, &ad);
  if (st0) return st0;
  OOPAO_CHECK_ARG(ad->l % p->bin == 0, "tangent pass needs the camera binning to divide its row block");
  const FastPasses* f = p->fast;
  const int n = p->n, res = p->res, k = p->k, cam = p->cam;
  float2* g = (float2*)base;  // [k][n][n] operating-point fields
  float2* w0 = g + (size_t)k * n * n;
  char* chunk = (char*)(w0 + (size_t)res * res);
  const size_t fixed = (size_t)(chunk - (char*)ws);
  OOPAO_CHECK_ARG(usable > fixed, "workspace smaller than the operating-point fields");
  // items per chunk (per-item operating points: one item per chunk)
  int bc = opd0_batch == 1 ? batch : 1;
  int ks = ad_ksplit(p, n, bc, kMaxSlotsBinned);
  while (bc > 1 && fixed + (size_t)bc * ad_item_bytes(p, ks, false) > ws_bytes) {
    bc = (bc + 1) / 2;
    ks = ad_ksplit(p, n, bc, kMaxSlotsBinned);
  }
  if (fixed + (size_t)bc * ad_item_bytes(p, ks, false) > ws_bytes) {
    oopao_set_last_error("workspace smaller than one tangent item", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  float2* y = (float2*)chunk;
  float2* z = y + (size_t)bc * k * res * n;
  float2* fld = z + (size_t)bc * k * n * n;
  float* part = (float*)(fld + (size_t)bc * res * res);
  const int slot_pts = k / ks;
  int launches = 0;
  auto forward_to_z = [&](const float2* field, int nb) {
    RowsFwdArgs ra{p->fft, p->d_tw, field, p->d_growfac, y, res, n, 0, p->ngroups, p->off, 0};
    f->rows<<<dim3(ceil_div(res, f->l_rows), p->ngroups, nb), f->t * f->l_rows, f->smem_rows, st>>>(ra);
    ColsArgs ca{p->fft, p->d_tw, p->d_mask, y, p->d_group, p->d_colfac, z, res, n, 0, k, p->ngroups, p->off, 0};
    f->cols<<<dim3(ceil_div(n, f->l_cols), k, nb), f->t * f->l_cols, f->smem_cols, st>>>(ca);
    launches += 2;
  };
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    if (b0 == 0 || opd0_batch != 1) {
      // operating-point fields G_k of item b0 (or of the shared point)
      const float* o0 = opd0 + (opd0_batch == 1 ? 0 : (size_t)b0 * res * res);
      pwfs_field<<<dim3(ceil_div(res * res, 256), 1), 256, 0, st>>>(o0, (float)phase_scale, p->d_amp, w0,
                                                                  res * res);
      forward_to_z(w0, 1);
      AdFieldArgs fa{p->d_tw, z, g, k};
      ad->field<<<dim3(ceil_div(n, ad->l), k, 1), ad->t * ad->l, ad->smem_field, st>>>(fa);
      launches += 2;
    }
    const float* o0 = opd0 + (opd0_batch == 1 ? 0 : (size_t)b0 * res * res);
    pwfs_field_tangent<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(
        o0, dopd + (size_t)b0 * res * res, (float)phase_scale, p->d_amp, fld, res * res, 0);
    forward_to_z(fld, nb);
    AdJvpArgs ja{p->d_tw, z, g, weights_of(p), part, 0, k, 0, slot_pts, ks, p->bin, cam};
    ad->jvp<<<dim3(nb, ceil_div(n, ad->l), ks), ad->t * ad->l, ad->smem_jvp, st>>>(ja);
    pwfs_reduce_binned<<<dim3(ceil_div(cam * cam, 256), nb), 256, 0, st>>>(part, dframe + (size_t)b0 * cam * cam,
                                                                           cam * cam, ks);
    launches += 3;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

namespace {
// Adjoint through the two passes (pwfs_sep.cuh): per chunk of items, the
// field and the filtered rows of each item's operating point, the adjoint
// column pass (G_k, Gbar_k, conjugate column filter -> V_k on the pupil
// rows), the adjoint row pass (conjugate row filter, Im(. conj(E~_k))
// summed over slots of points) and the fixed-order sum of the slots, scaled
// to OPD units.  OOPAO_ERR_WORKSPACE (nothing launched) when one item does
// not fit.
int vjp_sep(const oopao_pwfs_plan* p, const float* opd, const float* fbar, double phase_scale, int batch,
            float* opd_bar, char* base, size_t usable, cudaStream_t st) {
  const SepPasses* s = p->sep_ad;
  const int n = p->n, res = p->res, k = p->k, cam = p->cam, ng = p->ngroups;
  const int rblocks = ceil_div(res, s->l_rows);
  auto row_slots = [&](int bc) {
    const int want = ceil_div(8 * std::max(1, p->sep_ad_ctas), rblocks * bc);
    int best = 1;
    for (int d = 1; d <= k && d <= kMaxSlotsBinned; d++) {
      if (k % d) continue;
      best = d;
      if (d >= want) break;
    }
    return best;
  };
  auto chunk_bytes = [&](int bc, int ksr) {
    return (size_t)bc * ((size_t)ng * res * n * 8 + (size_t)res * res * 8 + (size_t)k * res * n * 8 +
                         (size_t)ksr * res * res * 4) + 1024;
  };
  int bc = (int)std::min<size_t>((size_t)batch, std::max<size_t>(1, p->l2_budget / chunk_bytes(1, 1)));
  int ksr = row_slots(bc);
  while (bc > 1 && chunk_bytes(bc, ksr) > usable) {
    bc = (bc + 1) / 2;
    ksr = row_slots(bc);
  }
  if (chunk_bytes(bc, ksr) > usable) return OOPAO_ERR_WORKSPACE;
  float2* y = (float2*)base;
  float2* fld = y + (size_t)bc * ng * res * n;
  float2* v = fld + (size_t)bc * res * res;
  float* part = (float*)(v + (size_t)bc * k * res * n);
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    const int ksc = sep_ksplit(p, nb, kMaxSlotsBinned, false, true);
    pwfs_field<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(opd + (size_t)b0 * res * res, (float)phase_scale,
                                                                   p->d_amp, fld, res * res);
    SepRowsArgs ra{p->d_tw, fld, p->d_growfac, p->d_mrow, y, res, ng, 0 /* support at row/column 0 */};
    s->rows<<<dim3(rblocks, ng, nb), s->t * s->l_rows, s->smem_rows, st>>>(ra);
    SepAdjArgs ca{p->d_tw, p->d_mcol, p->d_mrow, y, p->d_group, p->d_colfac, p->d_growfac, weights_of(p),
                  fbar + (size_t)b0 * cam * cam, fld, v, part, res, 0 /* support at row/column 0 */, ng, k / ksc, ksc, p->bin, cam};
    s->cols_adj<<<dim3(n / s->l_cols, ksc, nb), s->t * s->l_cols, s->smem_cols(res), st>>>(ca);
    SepAdjArgs rb = ca;
    rb.slot_pts = k / ksr;
    rb.ksplit = ksr;
    s->rows_adj<<<dim3(rblocks, ksr, nb), s->t * s->l_rows, s->smem_rows, st>>>(rb);
    pwfs_reduce_scaled<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(
        part, opd_bar + (size_t)b0 * res * res, res * res, ksr, (float)phase_scale);
    launches += 5;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
}  // namespace

extern "C" int oopao_pwfs_vjp(const oopao_pwfs_plan* p, const float* opd, const float* fbar, double phase_scale,
                              int batch, float* opd_bar, void* ws, size_t ws_bytes, void* stream) {
  OOPAO_CHECK_ARG(p && opd && fbar && opd_bar && ws, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1, "batch must be >= 1");
  cudaStream_t st = (cudaStream_t)stream;
  if (sep_applies(p, false, false) && p->n % p->bin == 0) {
    uintptr_t b2 = ((uintptr_t)ws + 255) & ~(uintptr_t)255;
    if (ws_bytes > b2 - (uintptr_t)ws) {
      const int r = vjp_sep(p, opd, fbar, phase_scale, batch, opd_bar, (char*)b2, ws_bytes - (b2 - (uintptr_t)ws), st);
      if (r != OOPAO_ERR_WORKSPACE) return r;  // else the three-pass adjoint below
    }
  }
  const AdPasses* ad = nullptr;
  int st0 = ad_setup(p, &ad);
  if (st0) return st0;
  const FastPasses* f = p->fast;
  const int n = p->n, res = p->res, k = p->k, cam = p->cam;
  uintptr_t base = ((uintptr_t)ws + 255) & ~(uintptr_t)255;
  const size_t slack = (size_t)(base - (uintptr_t)ws) + 256;
  int bc = batch;
  int ks = ad_ksplit(p, res, bc, kMaxSlotsBinned);
  while (bc > 1 && slack + (size_t)bc * ad_item_bytes(p, ks, true) > ws_bytes) {
    bc = (bc + 1) / 2;
    ks = ad_ksplit(p, res, bc, kMaxSlotsBinned);
  }
  if (slack + (size_t)bc * ad_item_bytes(p, ks, true) > ws_bytes) {
    oopao_set_last_error("workspace smaller than one adjoint item", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  float2* y = (float2*)base;
  float2* z = y + (size_t)bc * k * res * n;
  float2* fld = z + (size_t)bc * k * n * n;
  float* part = (float*)(fld + (size_t)bc * res * res);
  const int slot_pts = k / ks;
  int launches = 0;
  for (int b0 = 0; b0 < batch; b0 += bc) {
    const int nb = std::min(bc, batch - b0);
    pwfs_field<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(opd + (size_t)b0 * res * res,
                                                                   (float)phase_scale, p->d_amp, fld, res * res);
    RowsFwdArgs ra{p->fft, p->d_tw, fld, p->d_growfac, y, res, n, 0, p->ngroups, p->off, 0};
    f->rows<<<dim3(ceil_div(res, f->l_rows), p->ngroups, nb), f->t * f->l_rows, f->smem_rows, st>>>(ra);
    ColsArgs ca{p->fft, p->d_tw, p->d_mask, y, p->d_group, p->d_colfac, z, res, n, 0, k, p->ngroups, p->off, 0};
    f->cols<<<dim3(ceil_div(n, f->l_cols), k, nb), f->t * f->l_cols, f->smem_cols, st>>>(ca);
    // Gbar and its row FFT, in place over z
    AdVjpAArgs va{p->d_tw, z, z, fbar + (size_t)b0 * cam * cam, weights_of(p), 0, k, p->bin, cam};
    ad->vjp_a<<<dim3(ceil_div(n, ad->l), k, nb), ad->t * ad->l, ad->smem_vjp_a, st>>>(va);
    // column FFT, conj(mask), column IFFT over full columns, in place
    ColsArgs cb{p->fft, p->d_tw, p->d_mask_conj, z, nullptr, p->d_ones, z, n, n, 0, k, k, 0, 0};
    f->cols<<<dim3(ceil_div(n, f->l_cols), k, nb), f->t * f->l_cols, f->smem_cols, st>>>(cb);
    AdVjpBArgs vb{p->d_tw, z, fld, p->d_growfac, p->d_group, 0, p->d_colfac, part, 0, k, 0, slot_pts, ks, res,
                  p->off};
    ad->vjp_b<<<dim3(ceil_div(res, ad->l), ks, nb), ad->t * ad->l, ad->smem_vjp_b, st>>>(vb);
    pwfs_reduce_scaled<<<dim3(ceil_div(res * res, 256), nb), 256, 0, st>>>(
        part, opd_bar + (size_t)b0 * res * res, res * res, ks, (float)phase_scale);
    launches += 7;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_set_variant(oopao_pwfs_plan* p, int variant) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  const FastPasses* c = nullptr;
  const int cnt = fast_candidates(p->n, &c);
  OOPAO_CHECK_ARG(variant >= 0, "variant must be 0 (generic) or a compile-time plan index >= 1");
  if (variant > cnt) {
    oopao_set_last_error("no such compile-time plan for this FFT size", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  if (p->n_masks > 1 && (variant == 0 || !c[variant - 1].cols_m)) {
    oopao_set_last_error("this variant has no several-mask column pass", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  if (variant >= 1) {
    const FastPasses* f = c + (variant - 1);
    int target = kTargetCtas, c3 = 0;
    OOPAO_CUDA_TRY(fast_attrs(f, p->res, &target, &c3));
    p->fast = f;
    p->inv_target_ctas = target;
    p->cols3_ctas = c3;
  }
  p->variant = variant;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_device_status(oopao_pwfs_plan* p, int* code) {
  OOPAO_CHECK_ARG(p && code, "NULL argument");
  OOPAO_CUDA_TRY(cudaMemcpy(code, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  OOPAO_CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_num_variants(const oopao_pwfs_plan* p) {
  if (!p) return -1;
  const FastPasses* c = nullptr;
  return fast_candidates(p->n, &c);
}

extern "C" int oopao_pwfs_variant_info(const oopao_pwfs_plan* p, int variant, int* info) {
  OOPAO_CHECK_ARG(p && info, "NULL argument");
  const FastPasses* c = nullptr;
  const int cnt = fast_candidates(p->n, &c);
  OOPAO_CHECK_ARG(variant >= 1 && variant <= cnt, "no such compile-time plan");
  const FastPasses* f = c + (variant - 1);
  info[0] = f->r1; info[1] = f->r2; info[2] = f->t;
  info[3] = f->l_rows; info[4] = f->l_cols; info[5] = f->l_inv;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_get_variant(const oopao_pwfs_plan* p) { return p ? p->variant : -1; }

extern "C" int oopao_pwfs_set_separable(oopao_pwfs_plan* p, int enable) {
  OOPAO_CHECK_ARG(p, "NULL plan");
  OOPAO_CHECK_ARG(enable >= 0, "enable must be 0 (three passes) or a two-pass plan index >= 1");
  if (enable == 0) {
    p->sep_on = false;
    return OOPAO_OK;
  }
  const SepPasses* c = nullptr;
  const int cnt = sep_candidates(p->n, &c);
  if (enable > cnt) {
    oopao_set_last_error("no such two-pass plan for this FFT size", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  if (p->sep != c + (enable - 1)) {
    const SepPasses* prev = p->sep;
    p->sep = c + (enable - 1);
    if (!sep_fits(p->sep, p->res)) {
      p->sep = prev;
      oopao_set_last_error("that two-pass plan does not fit this pupil", __FILE__, __LINE__);
      return OOPAO_ERR_UNSUPPORTED;
    }
    OOPAO_CUDA_TRY(sep_attrs(p));
  }
  p->sep_on = true;
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_pass_info(const oopao_pwfs_plan* p, int batch, int* info) {
  OOPAO_CHECK_ARG(p && info && batch >= 1, "bad argument");
  const size_t ws = oopao_pwfs_workspace_bytes(p, batch);
  info[1] = p->ngroups;
  if (sep_applies(p, false, false)) {
    int bc = (int)std::min<size_t>((size_t)batch, std::max<size_t>(1, p->l2_budget / sep_chunk_bytes(p, 1, 1, true)));
    int ks = sep_ksplit(p, bc, kMaxSlotsBinned);
    while (bc > 1 && sep_chunk_bytes(p, bc, ks, true) > ws - 256) {
      bc = (bc + 1) / 2;
      ks = sep_ksplit(p, bc, kMaxSlotsBinned);
    }
    info[0] = 1;
    info[2] = ks;
    info[3] = bc;
  } else {
    const PassPlan pp = plan_passes(p, batch, false, default_units(p, batch));
    info[0] = 0;
    info[2] = pp.ksplit;
    info[3] = pp.bc;
  }
  return OOPAO_OK;
}

extern "C" int oopao_pwfs_num_separable(const oopao_pwfs_plan* p) {
  if (!p) return -1;
  const SepPasses* c = nullptr;
  return sep_candidates(p->n, &c);
}

extern "C" int oopao_pwfs_separable(const oopao_pwfs_plan* p) {
  if (!p) return -1;
  if (edge_applies(p, false)) return 2;
  return sep_applies(p, false, false) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Allocation-free measurement.
//
// Some callers cannot allocate device memory when they measure: a real-time
// AO control loop that forbids allocation once it runs (an allocation can
// block on the driver or synchronise the device), or a host framework that
// owns the GPU allocator and exposes no way to obtain scratch memory.  For
// them the FFT intermediates live in a fixed array compiled into this
// library.  Every GPU that loads the library holds these bytes until the
// process exits, so the size is kept modest.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_scratch_addr[kNoAllocMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_pwfs_noalloc_scratch[kNoAllocScratchBytes];

extern "C" int oopao_pwfs_measure_noalloc(const oopao_pwfs_plan* p, const float* opd, double phase_scale,
                                          int batch, float* frame, float* raw, void* stream) {
  OOPAO_CHECK_ARG(p && opd && frame, "NULL argument");
  OOPAO_CHECK_ARG(batch >= 1, "batch must be >= 1");
  OOPAO_CHECK_ARG(!p->prof->enabled,
                  "per-kernel profiling creates CUDA events; disable it for the allocation-free entry point");
  int dev = -1;
  OOPAO_CUDA_TRY(cudaGetDevice(&dev));
  OOPAO_CHECK_ARG(dev >= 0 && dev < kNoAllocMaxDevices, "device index outside the allocation-free scratch table");
  OOPAO_CHECK_ARG(dev == p->device, "the current device is not the device the plan was created on");
  void* scratch = nullptr;
  {
    // set-up, once per device, with that device current: the host-side name
    // of the array is not a device address, so look the address up
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_scratch_addr[dev]) {
      void* addr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&addr, g_pwfs_noalloc_scratch);
      if (e != cudaSuccess || addr == nullptr) {
        oopao_set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "symbol address is NULL", __FILE__,
                             __LINE__);
        return OOPAO_ERR_CUDA;
      }
      g_noalloc_scratch_addr[dev] = addr;
    }
    scratch = g_noalloc_scratch_addr[dev];
  }
  // the smallest pass (one slot of modulation points of one item) must fit
  const PassPlan smallest = plan_passes(p, 1, raw != nullptr, 1);
  if (smallest.bytes > kNoAllocScratchBytes) {
    char msg[200];
    snprintf(msg, sizeof(msg), "one pass of this plan needs %zu bytes, more than the %zu-byte allocation-free scratch",
             smallest.bytes, kNoAllocScratchBytes);
    oopao_set_last_error(msg, __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  // every scratch byte a pass reads is written earlier in the same call, so
  // nothing left by a previous call needs clearing
  return oopao_pwfs_measure(p, opd, phase_scale, batch, frame, raw, scratch, kNoAllocScratchBytes, stream);
}
