// Hand-written tangent (JVP) and adjoint (VJP) passes of the modulated
// pyramid propagation, for the compile-time FFT plans of fft2.cuh.
//
// Notation (per item, per modulation point k; F = unnormalised 2-D DFT,
// F^H its conjugate transpose, M the mask, 1/N^2 of ifft2 folded into E~):
//   E~_k = W * rowfac_k * colfac_k       W = amp * exp(i phi), zero padded
//   G_k  = F^H M F E~_k                   I_k = |G_k|^2, raw = sum_k w_k I_k
// Tangent:  dE~_k = i dphi E~_k,  dG_k = F^H M F dE~_k,
//           dI_k = 2 Re(conj(G_k) dG_k)
// Adjoint:  Gbar_k = 2 w_k rawbar G_k,  E~bar_k = F^H conj(M) F Gbar_k,
//           phibar = sum_k Im(E~bar_k conj(E~_k))   (pupil pixels)
// so both use the forward FFT chain (conjugate mask for the adjoint).  The
// adjoint recomputes each point's field from W instead of storing it.
#pragma once
#include "pwfs_fast.cuh"

struct AdFieldArgs {  // operating-point field rows G_k (one item)
  const float2* tw;
  const float2* z;  // [kp][N][N] column-pass output of the operating point
  float2* g;        // [kp][N][N]
  int kp;
};

// Inverse row FFT of the column-pass output, written as complex rows G_k.
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) ad_rows_field(AdFieldArgs a) {
  constexpr int R2P = pad_odd(R2);
  constexpr int LS = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr int PBA = (R1 + T - 1) / T, PBB = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* twi = sm;
  float2* xb = sm + N;
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int kk = blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < N;
  const float2* z = a.z + ((size_t)kk * N + row) * N;
  float2* x = xb + l * LS;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R1) {
      float2 v[R2];
#pragma unroll
      for (int m = 0; m < R2; m++) v[m] = active ? z[j + m * R1] : make_float2(0.f, 0.f);
      dft<R2, true>(v);
#pragma unroll
      for (int q = 0; q < R2; q++) x[j * R2P + q] = v[q];
    }
  }
  __syncthreads();
  float2* g = a.g + ((size_t)kk * N + row) * N;
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    if (j < R2 && active) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const float2 u = x[m * R2P + j];
        v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
      }
      dft<R1, true>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) g[j + q * R2] = v[q];
    }
  }
}

struct AdJvpArgs {
  const float2* tw;
  const float2* dz;      // [B][kp][N][N] column-pass output of the tangents
  const float2* g;       // [K][N][N] operating-point fields (shared by the batch)
  const float* weights;  // [K] or null
  float* binned;         // [B][ksplit][cam][cam]
  int k0, kp, s0, slot_pts, ksplit, bin, cam;
};

// Tangent of the detector intensity: sum over a slot of points of
// 2 w_k Re(conj(G_k) dG_k), binned to the camera (L % bin == 0).
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) ad_rows_jvp(AdJvpArgs a) {
  constexpr int R2P = pad_odd(R2);
  constexpr int LS = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr int PBA = (R1 + T - 1) / T, PBB = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* twi = sm;
  float2* xb = sm + N;  // [2][L][LS]
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  // grid (items, row blocks, slots): the items of one (row block, slot) run
  // side by side and share the operating-point rows G_k through L2
  const int b = blockIdx.x, slot = a.s0 + blockIdx.z, row = blockIdx.y * L + l;
  const bool active = row < N;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  float acc[PBB][R1];
#pragma unroll
  for (int p = 0; p < PBB; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  __syncthreads();
  for (int kk = kbeg; kk < kend; kk++) {
    float2* x = xb + ((kk - kbeg) & 1) * L * LS + l * LS;
    const float2* z = a.dz + (((size_t)b * a.kp + (kk - a.k0)) * N + row) * N;
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int j = t + p * T;
      if (j < R1) {
        float2 v[R2];
#pragma unroll
        for (int m = 0; m < R2; m++) v[m] = active ? z[j + m * R1] : make_float2(0.f, 0.f);
        dft<R2, true>(v);
#pragma unroll
        for (int q = 0; q < R2; q++) x[j * R2P + q] = v[q];
      }
    }
    __syncthreads();
    const float w2 = 2.f * (a.weights ? a.weights[kk] : 1.f);
    const float2* g = a.g + ((size_t)kk * N + row) * N;
#pragma unroll
    for (int p = 0; p < PBB; p++) {
      const int j = t + p * T;
      if (j < R2 && active) {
        float2 v[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const float2 u = x[m * R2P + j];
          v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
        }
        dft<R1, true>(v);
#pragma unroll
        for (int q = 0; q < R1; q++) {
          const float2 g0 = g[j + q * R2];
          acc[p][q] = fmaf(w2, fmaf(g0.x, v[q].x, g0.y * v[q].y), acc[p][q]);
        }
      }
    }
  }
  __syncthreads();
  float* rows = reinterpret_cast<float*>(xb);  // [L][N]
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    if (j < R2) {
#pragma unroll
      for (int q = 0; q < R1; q++) rows[l * N + j + q * R2] = active ? acc[p][q] : 0.f;
    }
  }
  __syncthreads();
  const int bin = a.bin, cam = a.cam, ncr = L / bin, cr0 = (blockIdx.y * L) / bin;
  float* out = a.binned + ((size_t)b * a.ksplit + slot) * cam * cam;
  for (int i = tid; i < ncr * cam; i += T * L) {
    const int cr = i / cam, cx = i - (i / cam) * cam;
    if (cr0 + cr >= cam) continue;
    float s = 0.f;
    for (int dy = 0; dy < bin; dy++) {
      const float* r = rows + (cr * bin + dy) * N + cx * bin;
      float rs = 0.f;
      for (int dx = 0; dx < bin; dx++) rs += r[dx];
      s += rs;
    }
    out[(cr0 + cr) * cam + cx] = s;
  }
}

struct AdVjpAArgs {
  const float2* tw;
  const float2* z;       // [B][kp][N][N] column-pass output (operating point)
  float2* u;             // [B][kp][N][N] row-FFT of Gbar (may alias z: rows are read before written)
  const float* fbar;     // [B][cam][cam] camera-frame cotangent
  const float* weights;  // [K] or null
  int k0, kp, bin, cam;
};

// Per row: G = inverse row FFT, Gbar = 2 w_k fbar(binned pixel) G, forward
// row FFT of Gbar (first transform of the adjoint chain).  The inverse
// stage-B' outputs of a thread are exactly the forward stage-A inputs.
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) ad_rows_vjp_a(AdVjpAArgs a) {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LS = odd_up(imax(R1 * R2P, R2 * R1P));
  constexpr int PBA = (R1 + T - 1) / T, PBB = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* tw = sm;       // W_N^{j m}:  tw[m*R1 + j]
  float2* twi = sm + N;  // W_N^{-j m}: twi[m*R2 + j]
  float2* x1 = sm + 2 * N;
  float2* x2 = x1 + L * LS;
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int b = blockIdx.z, kk = blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < N;
  const size_t unit = ((size_t)b * a.kp + kk) * N * N;
  const float2* z = a.z + unit + (size_t)row * N;
  float2* xa = x1 + l * LS;
  float2* xc = x2 + l * LS;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R1) {
      float2 v[R2];
#pragma unroll
      for (int m = 0; m < R2; m++) v[m] = active ? z[j + m * R1] : make_float2(0.f, 0.f);
      dft<R2, true>(v);
#pragma unroll
      for (int q = 0; q < R2; q++) xa[j * R2P + q] = v[q];
    }
  }
  __syncthreads();
  const float w2 = 2.f * (a.weights ? a.weights[a.k0 + kk] : 1.f);
  const float* fb = a.fbar + ((size_t)b * a.cam + (active ? row / a.bin : 0)) * a.cam;
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const float2 u = xa[m * R2P + j];
        v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
      }
      dft<R1, true>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) {
        const float s = active ? w2 * fb[(j + q * R2) / a.bin] : 0.f;
        v[q] = make_float2(s * v[q].x, s * v[q].y);
      }
      dft<R1, false>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) xc[j * R1P + q] = v[q];
    }
  }
  __syncthreads();
  float2* u = a.u + unit + (size_t)row * N;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R1 && active) {
      float2 v[R2];
#pragma unroll
      for (int m = 0; m < R2; m++) {
        const float2 w = xc[m * R1P + j];
        v[m] = (m == 0) ? w : cmul(w, tw[m * R1 + j]);
      }
      dft<R2, false>(v);
#pragma unroll
      for (int q = 0; q < R2; q++) u[j + q * R1] = v[q];
    }
  }
}

struct AdVjpBArgs {
  const float2* tw;
  const float2* v;        // [B][kp][N][N] after column FFT, conj(mask), column IFFT
  const float2* field;    // [B][res][res] W
  const float2* rowfac;   // [groups][res]
  const int* group;       // [K] or null (group = point - k0)
  int g0;                 // first row of rowfac for this pass
  const float2* colfac;   // [K][res]
  float* phibar;          // [B][ksplit][res][res]
  int k0, kp, s0, slot_pts, ksplit, res, off;
};

// Last transform of the adjoint chain on the pupil rows, then
// phibar += Im(E~bar conj(E~_k)) on the pupil columns, summed over a slot.
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) ad_rows_vjp_b(AdVjpBArgs a) {
  constexpr int R2P = pad_odd(R2);
  constexpr int LS = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr int PBA = (R1 + T - 1) / T, PBB = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* twi = sm;
  float2* xb = sm + N;  // [2][L][LS]
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int b = blockIdx.z, slot = a.s0 + blockIdx.y;
  const int pr = blockIdx.x * L + l;  // pupil row
  const bool active = pr < a.res;
  const int row = a.off + pr;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  const float2* fld = a.field + ((size_t)b * a.res + (active ? pr : 0)) * a.res;
  float acc[PBB][R1];
#pragma unroll
  for (int p = 0; p < PBB; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  __syncthreads();
  for (int kk = kbeg; kk < kend; kk++) {
    float2* x = xb + ((kk - kbeg) & 1) * L * LS + l * LS;
    const float2* vr = a.v + (((size_t)b * a.kp + (kk - a.k0)) * N + (active ? row : 0)) * N;
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int j = t + p * T;
      if (j < R1) {
        float2 v[R2];
#pragma unroll
        for (int m = 0; m < R2; m++) v[m] = active ? vr[j + m * R1] : make_float2(0.f, 0.f);
        dft<R2, true>(v);
#pragma unroll
        for (int q = 0; q < R2; q++) x[j * R2P + q] = v[q];
      }
    }
    __syncthreads();
    const int g = a.group ? a.group[kk] : (kk - a.k0);
    const float2* rf = a.rowfac + (size_t)(a.g0 + g) * a.res;
    const float2 cf = active ? a.colfac[(size_t)kk * a.res + pr] : make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < PBB; p++) {
      const int j = t + p * T;
      if (j < R2 && active) {
        float2 v[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const float2 u = x[m * R2P + j];
          v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
        }
        dft<R1, true>(v);
#pragma unroll
        for (int q = 0; q < R1; q++) {
          const int pc = j + q * R2 - a.off;
          if (pc >= 0 && pc < a.res) {
            const float2 e = cmul(cmul(fld[pc], rf[pc]), cf);
            acc[p][q] += v[q].y * e.x - v[q].x * e.y;
          }
        }
      }
    }
  }
  if (!active) return;
  float* out = a.phibar + (((size_t)b * a.ksplit + slot) * a.res + pr) * a.res;
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    if (j < R2) {
#pragma unroll
      for (int q = 0; q < R1; q++) {
        const int pc = j + q * R2 - a.off;
        if (pc >= 0 && pc < a.res) out[pc] = acc[p][q];
      }
    }
  }
}

struct AdPasses {
  void (*field)(AdFieldArgs);
  void (*jvp)(AdJvpArgs);
  void (*vjp_a)(AdVjpAArgs);
  void (*vjp_b)(AdVjpBArgs);
  size_t smem_field, smem_jvp, smem_vjp_a, smem_vjp_b;
  int t, l;
};

template <int N, int R1, int R2, int T, int L>
AdPasses make_ad() {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LSI = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr int LSA = odd_up(imax(R1 * R2P, R2 * R1P));
  AdPasses a;
  a.field = ad_rows_field<N, R1, R2, T, L>;
  a.jvp = ad_rows_jvp<N, R1, R2, T, L>;
  a.vjp_a = ad_rows_vjp_a<N, R1, R2, T, L>;
  a.vjp_b = ad_rows_vjp_b<N, R1, R2, T, L>;
  a.smem_field = sizeof(float2) * (N + (size_t)L * LSI);
  a.smem_jvp = sizeof(float2) * (N + 2 * (size_t)L * LSI);
  a.smem_vjp_a = sizeof(float2) * (2 * N + 2 * (size_t)L * LSA);
  a.smem_vjp_b = sizeof(float2) * (N + 2 * (size_t)L * LSI);
  a.t = T;
  a.l = L;
  return a;
}
