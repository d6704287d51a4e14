// Gain-sensing camera on the GPU: optical gains of a modulated pyramid from
// its focal-plane frame, following OOPAO/GainSensingCamera.py (calibration
// :78-95, compute_optical_gains :104-120, split_basis_product :158-173,
// impulse_response :184-185, sensitivity :188-193, optical_gains :196-199).
//
// With s[r][c] = (-1)^(r+c) and an even size n, the centred transform of the
// reference, fftshift(fft2(fftshift(x))) / n, equals s * FFT2(s * x) / n, and
// fftshift(ifft2(fftshift(x))) * n equals s * IFFT2u(s * x) / n with IFFT2u
// the unnormalised inverse.  Every 2-D transform is a row pass then a column
// pass of the shared-memory Stockham FFT (fft.cuh); the sign pattern, the
// inputs and the outputs are fused into the loads and stores:
//
//   basis product   bp[m] = fft3(b_m) * ifft3(b_m) = |fft3(b_m)|^2 for a real
//                   mode b_m zero-padded to n x n; float32 [modes][n*n]
//   impulse resp.   IR = 2 Im(conj(fft3(mask)) fft3(mask * frame / sum(frame)))
//   calibration     W = ifft3(IR_calib);  S_calib[m] = sum_p fft3(IR_calib)[p] W[p] bp[m][p]
//   per frame       S[m] = sum_p fft3(IR_sky)[p] W[p] bp[m][p];  og = Re(S / S_calib)
//
// The contraction over pixels reads bp once per group of frames and is bound
// by HBM bandwidth.  Each mode's bp row is stored divided by its power
// sum_p bp[m][p] = sum b_m^2 (Parseval), which leaves og unchanged and keeps
// every sum near unit scale whatever the units of the basis; sensitivities
// handed out are scaled back in float64.  The device arithmetic is float32
// (float64 is a narrow pipe on this part), summed in a fixed order.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "fft.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kSumThreads = 1024;
constexpr int kModeGroup = 8;        // modes per contraction CTA, one frame per CTA
constexpr int kModeGroupBatch = 4;   // modes per contraction CTA, four frames per CTA
constexpr int kMaxChunks = 64;       // pixel chunks of the contraction
constexpr size_t kSmemBudget = 96 * 1024;

enum { kInMaskFrame = 0, kInReal = 1, kInBasis = 2, kInComplex = 3 };
enum { kOutIr = 0, kOutScaled = 1, kOutWeighted = 2, kOutPower = 3 };

struct RowArgs {
  FftPlan fp;
  const float2* tw;
  int n, lines;
  const float* real_in;   // kInMaskFrame / kInReal: [items][n][n]; kInBasis: [items][n0][n0]
  const float2* cplx_in;  // kInMaskFrame: mask [n][n]; kInComplex: [items][n][n]
  float* row_sums;        // kInMaskFrame: sum of the frame over each CTA's rows, [items][gridDim.x]
  int n0, pad;            // kInBasis: mode placed at (pad, pad)
  float2* out;            // [items][n][n]
};

struct ColArgs {
  FftPlan fp;
  const float2* tw;
  int n, lines;
  const float2* in;          // [items][n][n]
  const float2* aux;         // kOutIr: fft3(mask); kOutWeighted: W
  const float* row_sums;     // kOutIr: the row pass's frame sums, [items][n_row_blocks]
  int n_row_blocks;
  const float* item_scale;   // kOutPower: factor of each item
  float2* out_c;             // kOutScaled / kOutWeighted, [items][n][n]; may be `in`
  float* out_r;              // kOutIr / kOutPower, [items][n][n]
};

constexpr int kLd = 8;  // global loads a thread issues before it uses them

__device__ __forceinline__ float warp_sum_f(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// One CTA transforms `lines` rows of one item; the row is built from the
// inputs with the (-1)^(r+c) sign folded in.  For a frame it also writes the
// sum of its rows of the frame (compensated, fixed order), from which the
// column pass normalises the frame to unit sum.
template <int IN, bool INV>
__global__ void __launch_bounds__(kThreads) gsc_rows(RowArgs a) {
  extern __shared__ float2 sm[];
  __shared__ float red[kThreads / 32];
  const int n = a.n;
  const int r0 = blockIdx.x * a.lines;
  const int nl = min(a.lines, n - r0);
  const size_t item = blockIdx.y;
  const size_t nn = (size_t)n * n;
  float2* A = sm;
  float2* B = sm + (size_t)a.lines * n;
  const int total = nl * n;
  float fs = 0.f, fc = 0.f;
  for (int base = 0; base < total; base += kLd * blockDim.x) {
    float f[kLd];
    float2 m[kLd];
#pragma unroll
    for (int j = 0; j < kLd; j++) {
      const int i = base + j * blockDim.x + threadIdx.x;
      f[j] = 0.f;
      m[j] = make_float2(0.f, 0.f);
      if (i < total) {
        const int l = i / n, c = i - l * n, r = r0 + l;
        if (IN == kInMaskFrame) {
          f[j] = a.real_in[item * nn + (size_t)r * n + c];
          m[j] = a.cplx_in[(size_t)r * n + c];
        } else if (IN == kInReal) {
          f[j] = a.real_in[item * nn + (size_t)r * n + c];
        } else if (IN == kInBasis) {
          const int rr = r - a.pad, cc = c - a.pad;
          if (rr >= 0 && rr < a.n0 && cc >= 0 && cc < a.n0)
            f[j] = a.real_in[item * a.n0 * a.n0 + (size_t)rr * a.n0 + cc];
        } else {
          m[j] = a.cplx_in[item * nn + (size_t)r * n + c];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kLd; j++) {
      const int i = base + j * blockDim.x + threadIdx.x;
      if (i < total) {
        const int l = i / n, c = i - l * n, r = r0 + l;
        const float sg = ((r + c) & 1) ? -1.f : 1.f;
        float2 v;
        if (IN == kInMaskFrame) {
          kahan_add(fs, fc, f[j]);
          v = make_float2(m[j].x * f[j] * sg, m[j].y * f[j] * sg);
        } else if (IN == kInComplex) {
          v = make_float2(m[j].x * sg, m[j].y * sg);
        } else {
          v = make_float2(f[j] * sg, 0.f);
        }
        A[i] = v;
      }
    }
  }
  if (IN == kInMaskFrame) {
    fs = warp_sum_f(fs);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = fs;
  }
  __syncthreads();
  if (IN == kInMaskFrame && threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    a.row_sums[item * gridDim.x + blockIdx.x] = t;
  }
  const float2* res = fft_lines<INV>(A, B, a.fp, a.tw, nl, n, threadIdx.x, blockDim.x);
  float2* out = a.out + item * nn + (size_t)r0 * n;
  for (int i = threadIdx.x; i < total; i += blockDim.x) out[i] = res[i];
}

// One CTA transforms `lines` adjacent columns of one item (each row segment
// is one contiguous load) and applies the centring sign and 1/n on the way
// out.  All of its loads precede its first store, so out_c may alias in.
template <int OUT, bool INV>
__global__ void __launch_bounds__(kThreads) gsc_cols(ColArgs a) {
  extern __shared__ float2 sm[];
  __shared__ float norm_sh;
  const int n = a.n;
  const int c0 = blockIdx.x * a.lines;
  const int nl = min(a.lines, n - c0);
  const size_t item = blockIdx.y;
  const size_t nn = (size_t)n * n;
  float2* A = sm;
  float2* B = sm + (size_t)a.lines * n;
  const float2* in = a.in + item * nn;
  const int total = nl * n;
  if (OUT == kOutIr && threadIdx.x < 32) {
    // 1 / sum of the frame from the row pass's partial sums (fixed order)
    float s = 0.f, c = 0.f;
    for (int k = threadIdx.x; k < a.n_row_blocks; k += 32) kahan_add(s, c, a.row_sums[item * a.n_row_blocks + k]);
    s = warp_sum_f(s);
    if (threadIdx.x == 0) norm_sh = 1.f / s;
  }
  for (int base = 0; base < total; base += kLd * blockDim.x) {
    float2 v[kLd];
#pragma unroll
    for (int j = 0; j < kLd; j++) {
      const int i = base + j * blockDim.x + threadIdx.x;
      if (i < total) {
        const int r = i / nl, l = i - r * nl;
        v[j] = in[(size_t)r * n + c0 + l];
      }
    }
#pragma unroll
    for (int j = 0; j < kLd; j++) {
      const int i = base + j * blockDim.x + threadIdx.x;
      if (i < total) {
        const int r = i / nl, l = i - r * nl;
        A[(size_t)l * n + r] = v[j];
      }
    }
  }
  __syncthreads();
  const float2* res = fft_lines<INV>(A, B, a.fp, a.tw, nl, n, threadIdx.x, blockDim.x);
  const float inv_n = (OUT == kOutIr ? norm_sh : 1.f) / (float)n;
  for (int base = 0; base < total; base += kLd * blockDim.x) {
    float2 w[kLd];
    if (OUT == kOutIr || OUT == kOutWeighted) {
#pragma unroll
      for (int j = 0; j < kLd; j++) {
        const int i = base + j * blockDim.x + threadIdx.x;
        if (i < total) {
          const int r = i / nl, l = i - r * nl;
          w[j] = a.aux[(size_t)r * n + c0 + l];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kLd; j++) {
      const int i = base + j * blockDim.x + threadIdx.x;
      if (i >= total) continue;
      const int r = i / nl, l = i - r * nl, c = c0 + l;
      const size_t p = (size_t)r * n + c;
      const float2 x = res[(size_t)l * n + r];
      const float sg = ((r + c) & 1) ? -inv_n : inv_n;
      const float2 y = make_float2(x.x * sg, x.y * sg);
      if (OUT == kOutIr) {
        a.out_r[item * nn + p] = 2.f * (w[j].x * y.y - w[j].y * y.x);
      } else if (OUT == kOutScaled) {
        a.out_c[item * nn + p] = y;
      } else if (OUT == kOutWeighted) {
        a.out_c[item * nn + p] = cmul(y, w[j]);
      } else {
        a.out_r[item * nn + p] = cabs2(y) * a.item_scale[item];
      }
    }
  }
}


// Power of each mode, sum b^2 = sum_p |fft3(b)|^2: scale[m] = 1 / power
// (1 for an all-zero mode) and norm[m] = power in float64.
__global__ void __launch_bounds__(kSumThreads) gsc_mode_power(const float* __restrict__ basis, size_t n0n0,
                                                              float* __restrict__ scale, double* __restrict__ norm) {
  __shared__ float red[kSumThreads / 32];
  const float* x = basis + blockIdx.x * n0n0;
  float s = 0.f, c = 0.f;
  for (size_t i = threadIdx.x; i < n0n0; i += blockDim.x) {
    const float y = x[i] * x[i] - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  s = warp_sum_f(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.f;
    t = warp_sum_f(t);
    if (threadIdx.x == 0) {
      scale[blockIdx.x] = t > 0.f ? 1.f / t : 1.f;
      norm[blockIdx.x] = t > 0.f ? (double)t : 1.0;
    }
  }
}

// part[chunk][b][m] = sum over the chunk's pixels p of v[b][p] * bp[m][p]
// (complex v, real bp).  A CTA covers BT frames, MG modes and one
// pixel chunk; a thread handles 4 consecutive pixels per step (float4 loads).
// Out-of-range modes and frames are clamped on load and dropped on store.
template <int BT, int MG>
__global__ void __launch_bounds__(kThreads, BT == 4 ? 3 : 2) gsc_contract(const float* __restrict__ bp, const float2* __restrict__ v,
                                                         int n_modes, int n2, int batch, int chunk,
                                                         float2* __restrict__ part) {
  const int b0 = blockIdx.x * BT;  // frame groups vary fastest: CTAs that read
  const int m0 = blockIdx.y * MG;  // the same basis-product rows run together
  const int p0 = blockIdx.z * chunk;
  const int p1 = min(n2, p0 + chunk);
  float ar[BT][MG], ai[BT][MG];
#pragma unroll
  for (int t = 0; t < BT; t++)
#pragma unroll
    for (int g = 0; g < MG; g++) ar[t][g] = ai[t][g] = 0.f;
  constexpr int kUnroll = BT == 1 ? 2 : 1;  // two steps of loads in flight where registers allow
#pragma unroll kUnroll
  for (int p = p0 + 4 * (int)threadIdx.x; p < p1; p += 4 * kThreads) {
    float4 va[BT], vb[BT];
#pragma unroll
    for (int t = 0; t < BT; t++) {
      const int b = min(b0 + t, batch - 1);
      const float4* q = reinterpret_cast<const float4*>(v + (size_t)b * n2 + p);
      va[t] = q[0];
      vb[t] = q[1];
    }
#pragma unroll
    for (int g = 0; g < MG; g++) {
      const int m = min(m0 + g, n_modes - 1);
      const float4 w = __ldg(reinterpret_cast<const float4*>(bp + (size_t)m * n2 + p));
#pragma unroll
      for (int t = 0; t < BT; t++) {
        float re = ar[t][g], im = ai[t][g];
        re = fmaf(va[t].x, w.x, re);
        im = fmaf(va[t].y, w.x, im);
        re = fmaf(va[t].z, w.y, re);
        im = fmaf(va[t].w, w.y, im);
        re = fmaf(vb[t].x, w.z, re);
        im = fmaf(vb[t].y, w.z, im);
        re = fmaf(vb[t].z, w.w, re);
        im = fmaf(vb[t].w, w.w, im);
        ar[t][g] = re;
        ai[t][g] = im;
      }
    }
  }
  __shared__ float red[kThreads / 32][2 * BT * MG];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < BT; t++)
#pragma unroll
    for (int g = 0; g < MG; g++) {
      const float re = warp_sum_f(ar[t][g]);
      const float im = warp_sum_f(ai[t][g]);
      if (lane == 0) {
        red[warp][2 * (t * MG + g)] = re;
        red[warp][2 * (t * MG + g) + 1] = im;
      }
    }
  __syncthreads();
  if (threadIdx.x < 2 * BT * MG) {
    float s = 0.f;
    for (int w = 0; w < kThreads / 32; w++) s += red[w][threadIdx.x];
    const int k = threadIdx.x >> 1, t = k / MG, g = k % MG;
    const int b = b0 + t, m = m0 + g;
    if (b < batch && m < n_modes) {
      float* dst = reinterpret_cast<float*>(part + ((size_t)blockIdx.z * batch + b) * n_modes + m);
      dst[threadIdx.x & 1] = s;
    }
  }
}

// S'[b][m] = sum over chunks (fixed order, compensated).  At a calibration
// (inv_ref == nullptr) it stores ref = S' and inv_ref = 1/S'; otherwise
// og[b][m] = Re(S'[b][m] / ref[m]).  s_out (optional) = S' * norm[m] in
// float64, the sensitivity in the basis' own units.
__global__ void gsc_finish(const float2* __restrict__ part, int n_chunks, int batch, int n_modes,
                           const double* __restrict__ norm, float2* __restrict__ ref, float2* __restrict__ inv_ref,
                           const float2* __restrict__ inv_ref_in, double2* __restrict__ s_out,
                           double* __restrict__ og) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch * n_modes) return;
  float sx = 0.f, sy = 0.f, cx = 0.f, cy = 0.f;
  for (int c = 0; c < n_chunks; c++) {
    const float2 q = part[(size_t)c * batch * n_modes + i];
    const float yx = q.x - cx, yy = q.y - cy;
    const float tx = sx + yx, ty = sy + yy;
    cx = (tx - sx) - yx;
    cy = (ty - sy) - yy;
    sx = tx;
    sy = ty;
  }
  const int m = i % n_modes;
  if (s_out) s_out[i] = make_double2((double)sx * norm[m], (double)sy * norm[m]);
  if (inv_ref_in == nullptr) {
    ref[m] = make_float2(sx, sy);
    const float d = 1.f / (sx * sx + sy * sy);
    inv_ref[m] = make_float2(sx * d, -sy * d);
  } else if (og) {
    const float2 r = inv_ref_in[m];
    og[i] = (double)(sx * r.x - sy * r.y);
  }
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

int lines_for(int n) {
  const int l = (int)(kSmemBudget / (2 * sizeof(float2) * (size_t)n));
  return l < 1 ? 1 : (l > 16 ? 16 : l);
}

template <typename K>
cudaError_t allow_smem(K kernel) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget);
}

}  // namespace

struct oopao_gsc_plan {
  int n = 0, n_modes = 0, n0 = 0;
  FftPlan fp{};
  int max_lines = 1;           // lines per CTA that fit the shared-memory budget
  int n_sm = 148;
  int contract_slots[2] = {0, 0};  // resident contraction CTAs (BT = 1, 4) on the GPU
  float2* tw = nullptr;
  float2* mask = nullptr;      // [n][n]
  float2* mspec = nullptr;     // fft3(mask)
  float* bp = nullptr;         // [n_modes][n*n], each row divided by the mode's power
  float* mode_scale = nullptr; // 1 / power of each mode
  double* mode_norm = nullptr; // power of each mode
  float2* wcal = nullptr;      // ifft3(IR_calib)
  float* ir_calib = nullptr;   // [n][n]
  float2* s_ref = nullptr;     // scaled sensi_calib [n_modes]
  float2* s_inv = nullptr;     // 1 / s_ref
  double2* s_calib = nullptr;  // sensi_calib [n_modes]
  bool have_basis = false;
  bool calibrated = false;
};

namespace {

struct Ws {
  float2* t;
  float* ir;
  float* row_sums;  // [batch][n]
  float2* part;
};

size_t ws_bytes(int n, int n_modes, int batch) {
  const size_t nn = (size_t)n * n;
  return align_up(nn * batch * sizeof(float2)) + align_up(nn * batch * sizeof(float)) +
         align_up((size_t)batch * n * sizeof(float)) + align_up((size_t)kMaxChunks * batch * n_modes * sizeof(float2));
}

Ws carve(void* ws, int n, int n_modes, int batch) {
  const size_t nn = (size_t)n * n;
  char* p = static_cast<char*>(ws);
  Ws w;
  w.t = reinterpret_cast<float2*>(p);
  p += align_up(nn * batch * sizeof(float2));
  w.ir = reinterpret_cast<float*>(p);
  p += align_up(nn * batch * sizeof(float));
  w.row_sums = reinterpret_cast<float*>(p);
  p += align_up((size_t)batch * n * sizeof(float));
  w.part = reinterpret_cast<float2*>(p);
  return w;
}

RowArgs row_args(const oopao_gsc_plan* P, float2* out) {
  RowArgs a{};
  a.fp = P->fp;
  a.tw = P->tw;
  a.n = P->n;
  a.out = out;
  return a;
}

ColArgs col_args(const oopao_gsc_plan* P, const float2* in) {
  ColArgs a{};
  a.fp = P->fp;
  a.tw = P->tw;
  a.n = P->n;
  a.in = in;
  return a;
}

// Lines per CTA for `items` transforms: about three CTAs per SM, at least
// `min_lines` (column passes: 4 columns = one 32-byte sector per row), at
// most what fits the shared-memory budget.  Threads: one per 8 elements.
struct LineLaunch {
  int lines, threads;
  size_t smem;
};

LineLaunch line_launch(const oopao_gsc_plan* P, int items, int min_lines) {
  LineLaunch L;
  L.lines = (int)(((long long)P->n * items + 3LL * P->n_sm - 1) / (3LL * P->n_sm));
  if (L.lines < min_lines) L.lines = min_lines;
  if (L.lines > P->max_lines) L.lines = P->max_lines;
  int t = (L.lines * P->n / 8 + 31) / 32 * 32;
  L.threads = t < 64 ? 64 : (t > kThreads ? kThreads : t);
  L.smem = 2 * sizeof(float2) * (size_t)L.lines * P->n;
  return L;
}

// Returns the number of row blocks (CTAs per item).
template <int IN, bool INV>
int launch_rows(const oopao_gsc_plan* P, RowArgs a, int items, cudaStream_t st) {
  const LineLaunch L = line_launch(P, items, 1);
  a.lines = L.lines;
  const int blocks = ceil_div(P->n, L.lines);
  gsc_rows<IN, INV><<<dim3((unsigned)blocks, (unsigned)items), L.threads, L.smem, st>>>(a);
  return blocks;
}

template <int OUT, bool INV>
void launch_cols(const oopao_gsc_plan* P, ColArgs a, int items, cudaStream_t st) {
  const LineLaunch L = line_launch(P, items, 4);
  a.lines = L.lines;
  gsc_cols<OUT, INV><<<dim3((unsigned)ceil_div(P->n, L.lines), (unsigned)items), L.threads, L.smem, st>>>(a);
}

// Pixel chunks of the contraction: the fewest chunks whose grid fills the
// resident CTA slots to at least 95% of its last wave (else the best fill).
int pick_chunks(int ctas_per_chunk, int slots) {
  int best = 1;
  double best_fill = 0.0;
  for (int c = 1; c <= kMaxChunks; c++) {
    const long long tot = (long long)ctas_per_chunk * c;
    const long long waves = (tot + slots - 1) / slots;
    const double fill = (double)tot / (double)(waves * slots);
    if (fill >= 0.95) return c;
    if (fill > best_fill + 1e-9) {
      best_fill = fill;
      best = c;
    }
  }
  return best;
}

// Contraction of v [batch][n*n] with the basis product, then the sums over
// chunks (gsc_finish: calibration when `calibrating`, else og and the
// optional float64 sensitivities).  Two launches.
void contract(const oopao_gsc_plan* P, const float2* v, int batch, float2* part, bool calibrating, double2* s_out,
              double* og, cudaStream_t st) {
  const int n2 = P->n * P->n;
  const int bt = batch >= 4 ? 4 : 1;
  const int groups = ceil_div(P->n_modes, bt == 4 ? kModeGroupBatch : kModeGroup);
  const int zg = ceil_div(batch, bt);
  int chunks = pick_chunks(groups * zg, P->contract_slots[bt == 4 ? 1 : 0]);
  const int chunk = ceil_div(ceil_div(n2, chunks), 4) * 4;
  chunks = ceil_div(n2, chunk);
  const dim3 g((unsigned)zg, (unsigned)groups, (unsigned)chunks);
  if (bt == 4)
    gsc_contract<4, kModeGroupBatch><<<g, kThreads, 0, st>>>(P->bp, v, P->n_modes, n2, batch, chunk, part);
  else
    gsc_contract<1, kModeGroup><<<g, kThreads, 0, st>>>(P->bp, v, P->n_modes, n2, batch, chunk, part);
  gsc_finish<<<ceil_div(batch * P->n_modes, 256), 256, 0, st>>>(part, chunks, batch, P->n_modes, P->mode_norm,
                                                              P->s_ref, P->s_inv, calibrating ? nullptr : P->s_inv,
                                                              s_out, og);
}

// IR of `batch` frames into ir, then v = fft3(IR) * W into ws.t.  Four launches.
void frames_to_v(const oopao_gsc_plan* P, const float* frames, int batch, float* ir, const Ws& w, cudaStream_t st) {
  RowArgs r = row_args(P, w.t);
  r.real_in = frames;
  r.cplx_in = P->mask;
  r.row_sums = w.row_sums;
  const int blocks = launch_rows<kInMaskFrame, false>(P, r, batch, st);
  ColArgs c = col_args(P, w.t);
  c.aux = P->mspec;
  c.row_sums = w.row_sums;
  c.n_row_blocks = blocks;
  c.out_r = ir;
  launch_cols<kOutIr, false>(P, c, batch, st);
  RowArgs r2 = row_args(P, w.t);
  r2.real_in = ir;
  launch_rows<kInReal, false>(P, r2, batch, st);
  ColArgs c2 = col_args(P, w.t);
  c2.aux = P->wcal;
  c2.out_c = w.t;
  launch_cols<kOutWeighted, false>(P, c2, batch, st);
}

}  // namespace

extern "C" int oopao_gsc_plan_create(oopao_gsc_plan** plan, int n, int n_modes, const float* mask_host) {
  OOPAO_CHECK_ARG(plan && mask_host, "NULL argument");
  OOPAO_CHECK_ARG(n >= 8 && n % 2 == 0 && n_modes > 0, "the mask size must be even and >= 8, n_modes > 0");
  *plan = nullptr;
  oopao_gsc_plan* P = new oopao_gsc_plan();
  P->n = n;
  P->n_modes = n_modes;
  if (!fft_make_plan(n, &P->fp)) {
    delete P;
    oopao_set_last_error("mask size has a prime factor above 13", __FILE__, __LINE__);
    return OOPAO_ERR_UNSUPPORTED;
  }
  P->max_lines = lines_for(n);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&P->n_sm, cudaDevAttrMultiProcessorCount, dev);
  int occ1 = 1, occ4 = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, gsc_contract<1, kModeGroup>, kThreads, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ4, gsc_contract<4, kModeGroupBatch>, kThreads, 0);
  P->contract_slots[0] = (occ1 < 1 ? 1 : occ1) * P->n_sm;
  P->contract_slots[1] = (occ4 < 1 ? 1 : occ4) * P->n_sm;
  const size_t nn = (size_t)n * n;
  std::vector<float2> tw(n);
  for (int t = 0; t < n; t++) {
    const double ang = -2.0 * M_PI * (double)t / (double)n;
    tw[t] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  float2* tmp = nullptr;
  cudaError_t e = cudaSuccess;
  auto fail = [&](cudaError_t err) {
    oopao_set_last_error(cudaGetErrorString(err), __FILE__, __LINE__);
    cudaFree(tmp);
    oopao_gsc_plan_destroy(P);
    return OOPAO_ERR_CUDA;
  };
  if ((e = allow_smem(gsc_rows<kInMaskFrame, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_rows<kInReal, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_rows<kInReal, true>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_rows<kInBasis, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_rows<kInComplex, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_cols<kOutIr, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_cols<kOutScaled, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_cols<kOutScaled, true>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_cols<kOutWeighted, false>)) != cudaSuccess) return fail(e);
  if ((e = allow_smem(gsc_cols<kOutPower, false>)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->tw, n * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->mspec, nn * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->wcal, nn * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->ir_calib, nn * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->s_calib, n_modes * sizeof(double2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->s_ref, n_modes * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->s_inv, n_modes * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->mode_scale, n_modes * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->mode_norm, n_modes * sizeof(double))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&P->mask, nn * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&tmp, nn * sizeof(float2))) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpy(P->tw, tw.data(), n * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpy(P->mask, mask_host, nn * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e);
  // fft3(mask), in single precision as the reference does for its complex64 mask
  RowArgs r = row_args(P, tmp);
  r.cplx_in = P->mask;
  launch_rows<kInComplex, false>(P, r, 1, 0);
  ColArgs c = col_args(P, tmp);
  c.out_c = P->mspec;
  launch_cols<kOutScaled, false>(P, c, 1, 0);
  oopao_count_launches(2);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
  cudaFree(tmp);
  *plan = P;
  return OOPAO_OK;
}

extern "C" int oopao_gsc_plan_destroy(oopao_gsc_plan* plan) {
  if (!plan) return OOPAO_OK;
  cudaFree(plan->tw);
  cudaFree(plan->mask);
  cudaFree(plan->mspec);
  cudaFree(plan->bp);
  cudaFree(plan->wcal);
  cudaFree(plan->ir_calib);
  cudaFree(plan->s_calib);
  cudaFree(plan->s_ref);
  cudaFree(plan->s_inv);
  cudaFree(plan->mode_scale);
  cudaFree(plan->mode_norm);
  delete plan;
  return OOPAO_OK;
}

extern "C" size_t oopao_gsc_workspace_bytes(const oopao_gsc_plan* plan, int batch) {
  if (!plan || batch < 1) return 0;
  return ws_bytes(plan->n, plan->n_modes, batch);
}

extern "C" int oopao_gsc_set_basis(oopao_gsc_plan* plan, const float* basis, int n0, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  OOPAO_CHECK_ARG(plan && basis && workspace, "NULL argument");
  const int n = plan->n;
  OOPAO_CHECK_ARG(n0 > 0 && n0 < n && (n - n0) % 2 == 0,
                  "the basis must be smaller than the mask, with an even difference of sizes");
  const size_t nn = (size_t)n * n;
  int group = (int)(workspace_bytes / (nn * sizeof(float2)));
  if (group < 1) {
    oopao_set_last_error("workspace smaller than one padded mode", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  if (group > 65535) group = 65535;
  if (!plan->bp) OOPAO_CUDA_TRY(cudaMalloc(&plan->bp, (size_t)plan->n_modes * nn * sizeof(float)));
  plan->n0 = n0;
  plan->have_basis = false;
  plan->calibrated = false;
  cudaStream_t st = (cudaStream_t)stream;
  float2* t = static_cast<float2*>(workspace);
  gsc_mode_power<<<plan->n_modes, kSumThreads, 0, st>>>(basis, (size_t)n0 * n0, plan->mode_scale, plan->mode_norm);
  int launches = 1;
  for (int m0 = 0; m0 < plan->n_modes; m0 += group) {
    const int g = plan->n_modes - m0 < group ? plan->n_modes - m0 : group;
    RowArgs r = row_args(plan, t);
    r.real_in = basis + (size_t)m0 * n0 * n0;
    r.n0 = n0;
    r.pad = (n - n0) / 2;
    launch_rows<kInBasis, false>(plan, r, g, st);
    ColArgs c = col_args(plan, t);
    c.out_r = plan->bp + (size_t)m0 * nn;
    c.item_scale = plan->mode_scale + m0;
    launch_cols<kOutPower, false>(plan, c, g, st);
    launches += 2;
  }
  oopao_count_launches(launches);
  OOPAO_CUDA_TRY(cudaGetLastError());
  plan->have_basis = true;
  return OOPAO_OK;
}

extern "C" int oopao_gsc_calibrate(oopao_gsc_plan* plan, const float* frame, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  OOPAO_CHECK_ARG(plan && frame && workspace, "NULL argument");
  OOPAO_CHECK_ARG(plan->have_basis, "oopao_gsc_set_basis must come first");
  if (workspace_bytes < ws_bytes(plan->n, plan->n_modes, 1)) {
    oopao_set_last_error("workspace smaller than oopao_gsc_workspace_bytes(plan, 1)", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Ws w = carve(workspace, plan->n, plan->n_modes, 1);
  plan->calibrated = false;
  // IR_calib
  RowArgs r = row_args(plan, w.t);
  r.real_in = frame;
  r.cplx_in = plan->mask;
  r.row_sums = w.row_sums;
  const int blocks = launch_rows<kInMaskFrame, false>(plan, r, 1, st);
  ColArgs c = col_args(plan, w.t);
  c.aux = plan->mspec;
  c.row_sums = w.row_sums;
  c.n_row_blocks = blocks;
  c.out_r = plan->ir_calib;
  launch_cols<kOutIr, false>(plan, c, 1, st);
  // W = ifft3(IR_calib)
  RowArgs ri = row_args(plan, w.t);
  ri.real_in = plan->ir_calib;
  launch_rows<kInReal, true>(plan, ri, 1, st);
  ColArgs ci = col_args(plan, w.t);
  ci.out_c = plan->wcal;
  launch_cols<kOutScaled, true>(plan, ci, 1, st);
  // v = fft3(IR_calib) * W, then S_calib
  RowArgs rf = row_args(plan, w.t);
  rf.real_in = plan->ir_calib;
  launch_rows<kInReal, false>(plan, rf, 1, st);
  ColArgs cf = col_args(plan, w.t);
  cf.aux = plan->wcal;
  cf.out_c = w.t;
  launch_cols<kOutWeighted, false>(plan, cf, 1, st);
  contract(plan, w.t, 1, w.part, true, plan->s_calib, nullptr, st);
  oopao_count_launches(8);
  OOPAO_CUDA_TRY(cudaGetLastError());
  plan->calibrated = true;
  return OOPAO_OK;
}

extern "C" int oopao_gsc_optical_gains(const oopao_gsc_plan* plan, const float* frames, int batch, double* og,
                                       double* sensitivity, float* ir, void* workspace, size_t workspace_bytes,
                                       void* stream) {
  OOPAO_CHECK_ARG(plan && frames && og && workspace && batch > 0, "NULL argument or batch < 1");
  if (!plan->calibrated) {
    oopao_set_last_error("Optical gains must be initialized first!", __FILE__, __LINE__);
    return OOPAO_ERR_INVALID;
  }
  OOPAO_CHECK_ARG(batch <= 65535, "batch above 65535");
  if (workspace_bytes < ws_bytes(plan->n, plan->n_modes, batch)) {
    oopao_set_last_error("workspace smaller than oopao_gsc_workspace_bytes(plan, batch)", __FILE__, __LINE__);
    return OOPAO_ERR_WORKSPACE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const Ws w = carve(workspace, plan->n, plan->n_modes, batch);
  frames_to_v(plan, frames, batch, ir ? ir : w.ir, w, st);
  contract(plan, w.t, batch, w.part, false, reinterpret_cast<double2*>(sensitivity), og, st);
  oopao_count_launches(6);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_gsc_read(const oopao_gsc_plan* plan, int what, void* dst, void* stream) {
  OOPAO_CHECK_ARG(plan && dst, "NULL argument");
  const size_t nn = (size_t)plan->n * plan->n;
  cudaStream_t st = (cudaStream_t)stream;
  switch (what) {
    case OOPAO_GSC_IR_CALIB:
      OOPAO_CHECK_ARG(plan->calibrated, "not calibrated");
      OOPAO_CUDA_TRY(cudaMemcpyAsync(dst, plan->ir_calib, nn * sizeof(float), cudaMemcpyDeviceToDevice, st));
      return OOPAO_OK;
    case OOPAO_GSC_SENSI_CALIB:
      OOPAO_CHECK_ARG(plan->calibrated, "not calibrated");
      OOPAO_CUDA_TRY(cudaMemcpyAsync(dst, plan->s_calib, plan->n_modes * sizeof(double2), cudaMemcpyDeviceToDevice,
                                     st));
      return OOPAO_OK;
    case OOPAO_GSC_BASIS_PRODUCT:
      OOPAO_CHECK_ARG(plan->have_basis, "no basis");
      OOPAO_CUDA_TRY(cudaMemcpyAsync(dst, plan->bp, (size_t)plan->n_modes * nn * sizeof(float),
                                     cudaMemcpyDeviceToDevice, st));
      return OOPAO_OK;
    case OOPAO_GSC_MODE_POWER:
      OOPAO_CHECK_ARG(plan->have_basis, "no basis");
      OOPAO_CUDA_TRY(cudaMemcpyAsync(dst, plan->mode_norm, plan->n_modes * sizeof(double), cudaMemcpyDeviceToDevice,
                                     st));
      return OOPAO_OK;
    default:
      OOPAO_CHECK_ARG(false, "unknown array");
  }
  return OOPAO_OK;
}
