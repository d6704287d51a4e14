// Shared-memory mixed-radix Stockham FFT for one CTA working on several lines.
//
// A line of length N lives contiguously in shared memory.  A transform is a
// sequence of radix-R stages (R in {2,3,4,5,7,8,9,11,13,16}); stage s with
// span Ns (product of the previous radices) performs, for every butterfly j
// in [0, N/R):
//     k   = j mod Ns
//     x_m = src[j + m*N/R] * W_{Ns*R}^{k*m}        (m = 0..R-1)
//     y   = DFT_R(x)
//     dst[(j-k)*R + k + q*Ns] = y_q                  (q = 0..R-1)
// which leaves the result in natural order after the last stage (Stockham
// auto-sort, ping-pong between two buffers).  Twiddles W_N^t = exp(-2 pi i t/N)
// come from an N-entry table computed in float64 on the host and rounded; the
// inverse transform uses their conjugates and is unnormalised.
#pragma once
#include "common.cuh"
#include "radix_consts.cuh"

#define OOPAO_FFT_MAX_STAGES 8

struct FftPlan {
  int n;
  int nstages;
  int radix[OOPAO_FFT_MAX_STAGES];
};

template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {  // * (-i) forward, * (+i) inverse
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, bool INV>
struct Dft {  // odd R: pairwise-symmetric direct DFT
  static __device__ __forceinline__ void run(float2* v) {
    constexpr int H = (R - 1) / 2;
    float2 a[H], b[H];
#pragma unroll
    for (int m = 1; m <= H; m++) {
      a[m - 1] = cadd(v[m], v[R - m]);
      b[m - 1] = csub(v[m], v[R - m]);
    }
    const float2 x0 = v[0];
    float2 y0 = x0;
#pragma unroll
    for (int m = 0; m < H; m++) y0 = cadd(y0, a[m]);
#pragma unroll
    for (int q = 1; q <= H; q++) {
      float2 A = x0, B = make_float2(0.f, 0.f);
#pragma unroll
      for (int m = 1; m <= H; m++) {
        const int t = (q * m) % R;
        const float c = rad_cos(R, t), s = rad_sin(R, t);
        A.x = fmaf(a[m - 1].x, c, A.x);
        A.y = fmaf(a[m - 1].y, c, A.y);
        B.x = fmaf(b[m - 1].x, s, B.x);
        B.y = fmaf(b[m - 1].y, s, B.y);
      }
      if (!INV) {
        v[q] = make_float2(A.x + B.y, A.y - B.x);
        v[R - q] = make_float2(A.x - B.y, A.y + B.x);
      } else {
        v[q] = make_float2(A.x - B.y, A.y + B.x);
        v[R - q] = make_float2(A.x + B.y, A.y - B.x);
      }
    }
    v[0] = y0;
  }
};

template <bool INV>
struct Dft<2, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

// Radix 3 with the outputs as FMAs on the half-sum: 12 instructions against
// 14 for the generic odd form (whose sine term is a separate product).
template <bool INV>
struct Dft<3, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float s = INV ? -rad_sin(3, 1) : rad_sin(3, 1);
    const float2 a = cadd(v[1], v[2]), b = csub(v[1], v[2]);
    const float2 x0 = v[0];
    const float2 h = make_float2(fmaf(rad_cos(3, 1), a.x, x0.x), fmaf(rad_cos(3, 1), a.y, x0.y));
    v[0] = cadd(x0, a);
    v[1] = make_float2(fmaf(s, b.y, h.x), fmaf(-s, b.x, h.y));
    v[2] = make_float2(fmaf(-s, b.y, h.x), fmaf(s, b.x, h.y));
  }
};

template <bool INV>
struct Dft<4, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    const float2 a2 = cadd(v[1], v[3]), a3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
  }
};

template <bool INV>
struct Dft<8, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    const float h = 0.70710678118654752f;
    // o1 *= W8^1, o2 *= W8^2, o3 *= W8^3 (conjugated for the inverse)
    float2 t;
    if (!INV) {
      t = o[1]; o[1] = make_float2((t.x + t.y) * h, (t.y - t.x) * h);
      o[2] = mul_mi<false>(o[2]);
      t = o[3]; o[3] = make_float2((t.y - t.x) * h, -(t.x + t.y) * h);
    } else {
      t = o[1]; o[1] = make_float2((t.x - t.y) * h, (t.x + t.y) * h);
      o[2] = mul_mi<true>(o[2]);
      t = o[3]; o[3] = make_float2(-(t.x + t.y) * h, (t.x - t.y) * h);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      v[q] = cadd(e[q], o[q]);
      v[q + 4] = csub(e[q], o[q]);
    }
  }
};

template <bool INV>
struct Dft<16, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
      e[i] = v[2 * i];
      o[i] = v[2 * i + 1];
    }
    Dft<8, INV>::run(e);
    Dft<8, INV>::run(o);
#pragma unroll
    for (int q = 1; q < 8; q++) {
      const float c = rad_cos(16, q), s = INV ? rad_sin(16, q) : -rad_sin(16, q);
      o[q] = cmul(o[q], make_float2(c, s));
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      v[q] = cadd(e[q], o[q]);
      v[q + 8] = csub(e[q], o[q]);
    }
  }
};

// One Stockham stage over `nlines` lines (line l at src + l*stride).
template <int R, bool INV>
__device__ __forceinline__ void fft_stage(const float2* __restrict__ src, float2* __restrict__ dst,
                                          int n, int ns, const float2* __restrict__ tw, int nlines,
                                          int stride, int tid, int nthreads) {
  const int nr = n / R;
  const int total = nlines * nr;
  const int tstep = n / (ns * R);
  for (int idx = tid; idx < total; idx += nthreads) {
    const int line = idx / nr;
    const int j = idx - line * nr;
    const float2* s = src + line * stride;
    float2* d = dst + line * stride;
    const int k = j % ns;
    float2 v[R];
#pragma unroll
    for (int m = 0; m < R; m++) v[m] = s[j + m * nr];
    if (ns > 1) {
#pragma unroll
      for (int m = 1; m < R; m++) {
        float2 w = tw[k * m * tstep];
        if (INV) w.y = -w.y;
        v[m] = cmul(v[m], w);
      }
    }
    Dft<R, INV>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; q++) d[base + q * ns] = v[q];
  }
}

// Runs all stages; input in `a`, `b` is scratch of the same shape.  The caller
// synchronises before the call.  Returns the buffer holding the result (a or b);
// every thread of the CTA must call it.
template <bool INV>
__device__ float2* fft_lines(float2* a, float2* b, const FftPlan& p, const float2* __restrict__ tw,
                             int nlines, int stride, int tid, int nthreads) {
  int ns = 1;
  float2* s = a;
  float2* d = b;
  for (int st = 0; st < p.nstages; st++) {
    const int R = p.radix[st];
    switch (R) {
      case 2: fft_stage<2, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 3: fft_stage<3, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 4: fft_stage<4, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 5: fft_stage<5, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 7: fft_stage<7, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 8: fft_stage<8, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 9: fft_stage<9, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 11: fft_stage<11, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 13: fft_stage<13, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      case 16: fft_stage<16, INV>(s, d, p.n, ns, tw, nlines, stride, tid, nthreads); break;
      default: break;
    }
    __syncthreads();
    ns *= R;
    float2* t = s;
    s = d;
    d = t;
  }
  return s;
}

// Host: factor n into supported radices (largest powers of two first, then
// 9, 3, 5, 7, 11, 13).  Returns false when n has another prime factor or
// needs more than OOPAO_FFT_MAX_STAGES stages.
static inline bool fft_make_plan(int n, FftPlan* p) {
  p->n = n;
  p->nstages = 0;
  int m = n;
  int twos = 0;
  while (m % 2 == 0) { m /= 2; twos++; }
  int st[16];
  int ns = 0;
  while (twos >= 4 && twos != 5 && twos != 6) { st[ns++] = 16; twos -= 4; }
  while (twos >= 3) { st[ns++] = 8; twos -= 3; }
  if (twos == 2) st[ns++] = 4;
  if (twos == 1) st[ns++] = 2;
  while (m % 9 == 0) { st[ns++] = 9; m /= 9; }
  const int odd[5] = {3, 5, 7, 11, 13};
  for (int i = 0; i < 5; i++)
    while (m % odd[i] == 0) { st[ns++] = odd[i]; m /= odd[i]; }
  if (m != 1 || ns > OOPAO_FFT_MAX_STAGES || ns == 0) return false;
  p->nstages = ns;
  for (int i = 0; i < ns; i++) p->radix[i] = st[i];
  return true;
}
