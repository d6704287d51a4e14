// Compile-time-planned propagation passes (N = R1*R2), see fft2.cuh.
// Same inputs/outputs as the generic kernels in pwfs.cu; one shared-memory
// exchange per line FFT and the forward->mask->inverse column chain kept in
// registers.
#pragma once
#include "fft2.cuh"
#include "tma.cuh"
#include "xchg.cuh"

// ---- pass 1: forward row FFT of field * row phasor (j-fastest mapping) ----
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) pwfs_rows_fwd2(RowsFwdArgs a) {
  constexpr int R1P = pad_odd(R1);
  constexpr int LS = xchg_stride(R2 * R1P, T, L, R1P, R2, R1);
  constexpr int PBA = (R2 + T - 1) / T, PBB = (R1 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* tw = sm;      // tw[m*R1 + j] = W_N^{j m}
  float2* xb = sm + N;  // [L][LS]
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) tw[i] = a.tw[(i % R1) * (i / R1)];
  const int b = blockIdx.z, g = blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < a.res;
  const int res = a.res, off = a.off;
  const float2* fld = a.field + ((size_t)b * res + row) * res;
  const float2* rf = a.rowfac + (size_t)(a.g0 + g) * res;
  float2* x = xb + l * LS;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2 && active) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const int jc = j + m * R2 - off;
        v[m] = (jc >= 0 && jc < res) ? cmul(fld[jc], rf[jc]) : make_float2(0.f, 0.f);
      }
      dft<R1, false>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) x[j * R1P + q] = v[q];
    }
  }
  __syncthreads();
  float2* y = a.y + (((size_t)b * a.ng + g) * res + row) * N;
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    if (j < R1 && active) {
      float2 v[R2];
#pragma unroll
      for (int m = 0; m < R2; m++) {
        const float2 u = x[m * R1P + j];
        v[m] = (m == 0) ? u : cmul(u, tw[m * R1 + j]);
      }
      dft<R2, false>(v);
#pragma unroll
      for (int q = 0; q < R2; q++) y[j + q * R1] = v[q];
    }
  }
}

// ---- pass 2: column phasor, forward FFT, mask, inverse FFT (l-fastest) ----
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) pwfs_cols2(ColsArgs a) {
  constexpr int LAY1 = cols_layout(R1, R2, T, L), LAY2 = cols_layout(R2, R1, T, L);
  constexpr int R1P = LAY1 >> 16, LS1 = LAY1 & 0xFFFF;
  constexpr int R2P = LAY2 >> 16, LS2 = LAY2 & 0xFFFF;
  constexpr int PBA = (R2 + T - 1) / T;   // forward stage A / inverse stage B' butterflies
  constexpr int PBB = (R1 + T - 1) / T;   // forward stage B / inverse stage A' butterflies
  // one stage-B butterfly per thread: its values stay in registers across a
  // barrier, so the inverse exchange reuses the forward buffer
  constexpr bool ALIAS = PBB == 1;
  extern __shared__ float2 sm[];
  float2* tw = sm;            // tw[m*R1 + j]  = W_N^{j m},  j < R1, m < R2
  float2* twi = sm + N;       // twi[m*R2 + j] = W_N^{-j m}, j < R2, m < R1
  float2* b1 = sm + 2 * N;    // [L][LS1] forward exchange
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;  // [L][LS2] inverse exchange
  const int tid = threadIdx.x;
  const int l = tid % L, t = tid / L;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int b = blockIdx.z, kk = blockIdx.y, c = blockIdx.x * L + l;
  const int kabs = a.k0 + kk;
  const int g = a.group ? a.group[kabs] : kk;
  const bool active = c < N;
  const int res = a.res, off = a.off;
  const float2* y = a.y + ((size_t)b * a.ng + g) * res * N + c;
  const float2* cf = a.colfac + (size_t)kabs * res;
  float2* x1 = b1 + l * LS1;
  float2* x2 = b2 + l * LS2;
  // forward stage A: rows e = j + m*R2, non-zero for off <= e < off + res
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const int i = j + m * R2 - off;
        v[m] = (active && i >= 0 && i < res) ? cmul(y[(size_t)i * N], cf[i]) : make_float2(0.f, 0.f);
      }
      dft<R1, false>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) x1[j * R1P + q] = v[q];
    }
  }
  __syncthreads();
  // forward stage B, mask, inverse stage A' (radix R2, same registers)
  const float2* mk = a.mask + c;
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    float2 v[R2];
    if (j < R1) {
#pragma unroll
      for (int m = 0; m < R2; m++) {
        const float2 u = x1[m * R1P + j];
        v[m] = (m == 0) ? u : cmul(u, tw[m * R1 + j]);
      }
      dft<R2, false>(v);
      if (a.focal && active) {
        // focal-plane camera: |F|^2 of this point, row j + q*R1 of column c
        float* fo = a.focal + (size_t)b * N * N + c;
#pragma unroll
        for (int q = 0; q < R2; q++) atomicAdd(fo + (size_t)(j + q * R1) * N, a.focal_scale * cabs2(v[q]));
      }
#pragma unroll
      for (int q = 0; q < R2; q++) {
        const float2 mq = active ? mk[(size_t)(j + q * R1) * N] : make_float2(0.f, 0.f);
        v[q] = cmul(v[q], mq);
      }
      dft<R2, true>(v);
    }
    if constexpr (ALIAS) __syncthreads();  // every read of the forward exchange is done
    if (j < R1) {
#pragma unroll
      for (int q = 0; q < R2; q++) x2[j * R2P + q] = v[q];
    }
  }
  __syncthreads();
  // inverse stage B' (radix R1, span R2): outputs rows j + q*R2
  float2* z = a.z + ((size_t)b * a.kp + kk) * N * N + c;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const float2 u = x2[m * R2P + j];
        v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
      }
      dft<R1, true>(v);
      if (active) {
#pragma unroll
        for (int q = 0; q < R1; q++) z[(size_t)(j + q * R2) * N] = v[q];
      }
    }
  }
}

// ---- pass 2 for several Fourier masks (Bi-O Edge) ----
// The forward column transform is computed once; for each of the n_masks
// masks the spectrum is multiplied by that mask and transformed back, giving
// one Z per mask ([B][n_masks][kp][N][N]).  Variants with one stage-B
// butterfly per thread only (the spectrum stays in registers across masks).
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) pwfs_cols2m(ColsArgs a) {
  constexpr int LAY1 = cols_layout(R1, R2, T, L), LAY2 = cols_layout(R2, R1, T, L);
  constexpr int R1P = LAY1 >> 16, LS1 = LAY1 & 0xFFFF;
  constexpr int R2P = LAY2 >> 16, LS2 = LAY2 & 0xFFFF;
  constexpr int PBA = (R2 + T - 1) / T;
  static_assert((R1 + T - 1) / T == 1, "one stage-B butterfly per thread");
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* twi = sm + N;
  float2* b1 = sm + 2 * N;   // forward exchange, reused by the inverse exchange
  const int tid = threadIdx.x;
  const int l = tid % L, t = tid / L;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int b = blockIdx.z, kk = blockIdx.y, c = blockIdx.x * L + l;
  const int kabs = a.k0 + kk;
  const int g = a.group ? a.group[kabs] : kk;
  const bool active = c < N;
  const int res = a.res, off = a.off, nm = a.n_masks;
  const float2* y = a.y + ((size_t)b * a.ng + g) * res * N + c;
  const float2* cf = a.colfac + (size_t)kabs * res;
  float2* x1 = b1 + l * LS1;
  float2* x2 = b1 + l * LS2;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const int i = j + m * R2 - off;
        v[m] = (active && i >= 0 && i < res) ? cmul(y[(size_t)i * N], cf[i]) : make_float2(0.f, 0.f);
      }
      dft<R1, false>(v);
#pragma unroll
      for (int q = 0; q < R1; q++) x1[j * R1P + q] = v[q];
    }
  }
  __syncthreads();
  const int j = t;
  float2 spec[R2];  // forward spectrum of column c, rows j + q*R1
  if (j < R1) {
#pragma unroll
    for (int m = 0; m < R2; m++) {
      const float2 u = x1[m * R1P + j];
      spec[m] = (m == 0) ? u : cmul(u, tw[m * R1 + j]);
    }
    dft<R2, false>(spec);
    if (a.focal && active) {
      float* fo = a.focal + (size_t)b * N * N + c;
#pragma unroll
      for (int q = 0; q < R2; q++) atomicAdd(fo + (size_t)(j + q * R1) * N, a.focal_scale * cabs2(spec[q]));
    }
  }
  for (int mi = 0; mi < nm; mi++) {
    float2 v[R2];
    if (j < R1) {
      const float2* mk = a.mask + (size_t)mi * N * N + c;
#pragma unroll
      for (int q = 0; q < R2; q++) {
        const float2 mq = active ? mk[(size_t)(j + q * R1) * N] : make_float2(0.f, 0.f);
        v[q] = cmul(spec[q], mq);
      }
      dft<R2, true>(v);
    }
    __syncthreads();  // earlier reads of the exchange buffer are done
    if (j < R1) {
#pragma unroll
      for (int q = 0; q < R2; q++) x2[j * R2P + q] = v[q];
    }
    __syncthreads();
    float2* z = a.z + (((size_t)b * nm + mi) * a.kp + kk) * N * N + c;
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int jj = t + p * T;
      if (jj < R2) {
        float2 w[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const float2 u = x2[m * R2P + jj];
          w[m] = (m == 0) ? u : cmul(u, twi[m * R2 + jj]);
        }
        dft<R1, true>(w);
        if (active) {
#pragma unroll
          for (int q = 0; q < R1; q++) z[(size_t)(jj + q * R2) * N] = w[q];
        }
      }
    }
  }
}

// ---- pass 2, persistent form ----
// A CTA owns a block of L columns for the whole pass: it loads that block of
// the mask into shared memory once, then loops over (item, point) units,
// bringing each unit's [res][L] tile of Y in with a TMA load issued one unit
// ahead (two tile buffers, one mbarrier each).  The per-unit arithmetic is
// that of pwfs_cols2; global traffic per unit is the Y tile in and Z out.
__host__ __device__ constexpr size_t align128(size_t v) { return (v + 127) / 128 * 128; }

template <int N, int R1, int R2, int T, int L>
struct Cols3Smem {
  static constexpr int LAY1 = cols_layout(R1, R2, T, L), LAY2 = cols_layout(R2, R1, T, L);
  static constexpr int LS1 = LAY1 & 0xFFFF, LS2 = LAY2 & 0xFFFF;
  static constexpr bool ALIAS = (R1 + T - 1) / T == 1;
  static constexpr size_t kXchFloat2 = (size_t)(ALIAS ? imax(LS1, LS2) : LS1 + LS2) * L;
  static constexpr size_t kBars = 0;                                  // 2 mbarriers
  static constexpr size_t kTw = 128;                                  // tw[N], twi[N]
  static constexpr size_t kMask = kTw + 2 * (size_t)N * 8;            // mask block [N][L]
  static constexpr size_t kXch = kMask + (size_t)N * L * 8;           // exchange
  static constexpr size_t kY = align128(kXch + kXchFloat2 * 8);       // two Y tiles
  static __host__ __device__ size_t ytile(int res) { return align128((size_t)res * L * 8); }
  static size_t bytes(int res) { return kY + 2 * ytile(res); }
};

template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) pwfs_cols3(const __grid_constant__ CUtensorMap ymap, ColsArgs a) {
  using S = Cols3Smem<N, R1, R2, T, L>;
  constexpr int R1P = S::LAY1 >> 16, LS1 = S::LS1;
  constexpr int R2P = S::LAY2 >> 16, LS2 = S::LS2;
  constexpr int PBA = (R2 + T - 1) / T;   // forward stage A / inverse stage B' butterflies
  constexpr int PBB = (R1 + T - 1) / T;   // forward stage B / inverse stage A' butterflies
  constexpr bool ALIAS = S::ALIAS;
  extern __shared__ __align__(128) unsigned char smraw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + S::kBars);
  float2* tw = reinterpret_cast<float2*>(smraw + S::kTw);  // tw[m*R1 + j] = W_N^{j m}
  float2* twi = tw + N;                                      // twi[m*R2 + j] = W_N^{-j m}
  float2* mt = reinterpret_cast<float2*>(smraw + S::kMask); // mt[row*L + l] = mask[row][c0 + l]
  float2* b1 = reinterpret_cast<float2*>(smraw + S::kXch);
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int res = a.res, off = a.off;
  float2* ybuf0 = reinterpret_cast<float2*>(smraw + S::kY);
  float2* ybuf1 = reinterpret_cast<float2*>(smraw + S::kY + S::ytile(res));
  const int tid = threadIdx.x;
  const int l = tid % L, t = tid / L;
  const int c0 = blockIdx.x * L, c = c0 + l;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  for (int i = tid; i < N * L; i += T * L) mt[i] = a.mask[(size_t)(i / L) * N + c0 + i % L];
  if (tid == 0) {
    tma::mbar_init(&bar[0], 1);
    tma::mbar_init(&bar[1], 1);
    tma::mbar_init_fence();
  }
  __syncthreads();
  const int units = a.items * a.kp, P = gridDim.y;
  const uint32_t tile_bytes = (uint32_t)res * L * 8;
  auto issue = [&](int u, int s) {
    const int b = u / a.kp, kk = u - (u / a.kp) * a.kp;
    const int g = a.group ? a.group[a.k0 + kk] : kk;
    tma::mbar_expect_tx(&bar[s], tile_bytes);
    tma::load_2d(s ? ybuf1 : ybuf0, &ymap, &bar[s], 2 * c0, (b * a.ng + g) * res);
  };
  int u = blockIdx.y, it = 0;
  bool ok = true;
  if (tid == 0 && u < units) issue(u, 0);
  for (; u < units; u += P, it++) {
    const int s = it & 1;
    // the other buffer was last read before the previous unit's first barrier
    if (tid == 0 && u + P < units) {
      tma::fence_proxy_async();
      issue(u + P, s ^ 1);
    }
    const bool arrived = tma::mbar_wait(&bar[s], (uint32_t)((it >> 1) & 1), a.err, 11);
    if (!__syncthreads_and(arrived)) {
      ok = false;
      break;
    }
    const int b = u / a.kp, kk = u - (u / a.kp) * a.kp;
    const int kabs = a.k0 + kk;
    const float2* yt = (s ? ybuf1 : ybuf0) + l;  // yt[i*L]: row i of this column
    const float2* cf = a.colfac + (size_t)kabs * res;
    float2* x1 = b1 + l * LS1;
    float2* x2 = b2 + l * LS2;
    // forward stage A: rows e = j + m*R2, non-zero for off <= e < off + res
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int j = t + p * T;
      if (j < R2) {
        float2 v[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const int i = j + m * R2 - off;
          v[m] = (i >= 0 && i < res) ? cmul(yt[i * L], cf[i]) : make_float2(0.f, 0.f);
        }
        dft<R1, false>(v);
#pragma unroll
        for (int q = 0; q < R1; q++) x1[j * R1P + q] = v[q];
      }
    }
    __syncthreads();
    // forward stage B, mask (from shared memory), inverse stage A'
#pragma unroll
    for (int p = 0; p < PBB; p++) {
      const int j = t + p * T;
      float2 v[R2];
      if (j < R1) {
#pragma unroll
        for (int m = 0; m < R2; m++) {
          const float2 w = x1[m * R1P + j];
          v[m] = (m == 0) ? w : cmul(w, tw[m * R1 + j]);
        }
        dft<R2, false>(v);
        if (a.focal) {
          float* fo = a.focal + (size_t)b * N * N + c;
#pragma unroll
          for (int q = 0; q < R2; q++) atomicAdd(fo + (size_t)(j + q * R1) * N, a.focal_scale * cabs2(v[q]));
        }
#pragma unroll
        for (int q = 0; q < R2; q++) v[q] = cmul(v[q], mt[(j + q * R1) * L + l]);
        dft<R2, true>(v);
      }
      if constexpr (ALIAS) __syncthreads();  // every read of the forward exchange is done
      if (j < R1) {
#pragma unroll
        for (int q = 0; q < R2; q++) x2[j * R2P + q] = v[q];
      }
    }
    __syncthreads();
    // inverse stage B' (radix R1, span R2): outputs rows j + q*R2
    float2* z = a.z + ((size_t)b * a.kp + kk) * N * N + c;
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int j = t + p * T;
      if (j < R2) {
        float2 v[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const float2 w = x2[m * R2P + j];
          v[m] = (m == 0) ? w : cmul(w, twi[m * R2 + j]);
        }
        dft<R1, true>(v);
#pragma unroll
        for (int q = 0; q < R1; q++) z[(size_t)(j + q * R2) * N] = v[q];
      }
    }
    // the next unit's first barrier (after its wait) orders these exchange
    // reads before its stage-A writes
  }
  if (!ok && tid == 0) {
    // a wait timed out: give the loads still in flight a bounded chance to
    // land before the CTA's shared memory is released
    tma::mbar_wait(&bar[it & 1], (uint32_t)((it >> 1) & 1), nullptr, 0);
    if (u + P < units) tma::mbar_wait(&bar[(it + 1) & 1], (uint32_t)(((it + 1) >> 1) & 1), nullptr, 0);
  }
}

// Row-inverse exchange: double-buffered over modulation points (one barrier
// per point) while both buffers fit in ~110 KB; a single buffer with a second
// barrier per point above that, so that two CTAs still share an SM.
__host__ __device__ constexpr bool inv_double_buffer(int N, int L, int LS) {
  return (size_t)(N + 2 * L * LS) * 8 <= 110 * 1024;
}

// ---- pass 3: row inverse FFT, |.|^2 summed over a slot of points, binning ----
template <int N, int R1, int R2, int T, int L>
__global__ void __launch_bounds__(T* L) pwfs_rows_inv2(RowsInvArgs a) {
  constexpr int R2P = pad_odd(R2);
  constexpr int LS = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr bool DB = inv_double_buffer(N, L, LS);
  constexpr int PBA = (R1 + T - 1) / T;  // inverse stage A' (radix R2) butterflies
  constexpr int PBB = (R2 + T - 1) / T;  // inverse stage B' (radix R1) butterflies
  extern __shared__ float2 sm[];
  float2* twi = sm;          // twi[m*R2 + j] = W_N^{-j m}
  float2* xb = sm + N;       // [2][L][LS]
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
  }
  const int b = blockIdx.z, slot = a.s0 + blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < N;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  float acc[PBB][R1];
#pragma unroll
  for (int p = 0; p < PBB; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  __syncthreads();
  for (int kk = kbeg; kk < kend; kk++) {
    float2* x = xb + (DB ? ((kk - kbeg) & 1) : 0) * L * LS + l * LS;
    if (!DB && kk > kbeg) __syncthreads();  // the previous point's reads of x are done
    const float2* z = a.z + (((size_t)b * a.kp + (kk - a.k0)) * N + row) * N;
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
    const float w = a.weights ? a.weights[kk] : 1.f;
#pragma unroll
    for (int p = 0; p < PBB; p++) {
      const int j = t + p * T;
      if (j < R2) {
        float2 v[R1];
#pragma unroll
        for (int m = 0; m < R1; m++) {
          const float2 u = x[m * R2P + j];
          v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
        }
        dft<R1, true>(v);
#pragma unroll
        for (int q = 0; q < R1; q++) acc[p][q] = fmaf(w, cabs2(v[q]), acc[p][q]);
      }
    }
  }
  if (a.partial) {
    // un-binned partial rows (raw_data requested)
    if (active) {
      float* out = a.partial + (((size_t)b * a.ksplit + slot) * N + row) * N;
#pragma unroll
      for (int p = 0; p < PBB; p++) {
        const int j = t + p * T;
        if (j < R2) {
#pragma unroll
          for (int q = 0; q < R1; q++) out[j + q * R2] = acc[p][q];
        }
      }
    }
    return;
  }
  // fused detector binning: the CTA's L rows are L/bin whole camera rows
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
  const int bin = a.bin, cam = a.cam, ncr = L / bin, cr0 = (blockIdx.x * L) / bin;
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

// ---- registry ----
struct FastPasses {
  int n, r1, r2, t, l_rows, l_cols, l_inv;
  void (*rows)(RowsFwdArgs);
  void (*cols)(ColsArgs);
  void (*inv)(RowsInvArgs);
  size_t smem_rows, smem_cols, smem_inv;
  // persistent column pass (null when the variant has none): L3 columns per CTA
  int l_cols3;
  void (*cols3)(const CUtensorMap, ColsArgs);
  size_t (*smem_cols3)(int res);
  // column pass over several masks (null unless one stage-B butterfly per thread)
  void (*cols_m)(ColsArgs);
  size_t smem_cols_m;
};

template <int N, int R1, int R2, int T, int LR, int LC, int LI>
FastPasses make_fast() {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LSR = xchg_stride(R2 * R1P, T, LR, R1P, R2, R1);
  constexpr int LS1C = cols_layout(R1, R2, T, LC) & 0xFFFF, LS2C = cols_layout(R2, R1, T, LC) & 0xFFFF;
  // the column pass shares one exchange buffer when each thread has one stage-B butterfly
  constexpr int LSC = ((R1 + T - 1) / T == 1) ? imax(LS1C, LS2C) : LS1C + LS2C;
  constexpr int LSI = xchg_stride(R1 * R2P, T, LI, R2P, R1, R2);
  FastPasses f;
  f.n = N; f.r1 = R1; f.r2 = R2; f.t = T; f.l_rows = LR; f.l_cols = LC; f.l_inv = LI;
  f.rows = pwfs_rows_fwd2<N, R1, R2, T, LR>;
  f.cols = pwfs_cols2<N, R1, R2, T, LC>;
  f.inv = pwfs_rows_inv2<N, R1, R2, T, LI>;
  f.smem_rows = sizeof(float2) * (N + (size_t)LR * LSR);
  f.smem_cols = sizeof(float2) * (2 * N + (size_t)LC * LSC);
  f.smem_inv = sizeof(float2) * (N + (inv_double_buffer(N, LI, LSI) ? 2 : 1) * (size_t)LI * LSI);
  f.l_cols3 = 0;
  f.cols3 = nullptr;
  f.smem_cols3 = nullptr;
  f.cols_m = nullptr;
  f.smem_cols_m = 0;
  if constexpr ((R1 + T - 1) / T == 1) {
    f.cols_m = pwfs_cols2m<N, R1, R2, T, LC>;
    f.smem_cols_m = sizeof(float2) * (2 * N + (size_t)LC * imax(LS1C, LS2C));
  }
  return f;
}

// make_fast plus the persistent TMA column pass with L3 columns per CTA.
template <int N, int R1, int R2, int T, int LR, int LC, int LI, int L3>
FastPasses make_fast3() {
  static_assert(N % L3 == 0 && (2 * L3 * 4) % 16 == 0, "column blocks must tile N in 16-byte TMA rows");
  FastPasses f = make_fast<N, R1, R2, T, LR, LC, LI>();
  f.l_cols3 = L3;
  f.cols3 = pwfs_cols3<N, R1, R2, T, L3>;
  f.smem_cols3 = &Cols3Smem<N, R1, R2, T, L3>::bytes;
  return f;
}
