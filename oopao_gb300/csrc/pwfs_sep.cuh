// Two-pass propagation for Fourier masks that factorise per axis.
//
// The reference's four-face mask (OOPAO/Pyramid.py:453-480) with equal face
// shifts, no rooftop and no rotation is exp(-i a(|x| + |y|) + linear terms):
// M[r][c] = mcol[r] * mrow[c].  The 2-D filter then splits into two 1-D
// filters that commute:
//     G_k = F^H M F E~_k = (Fc^H diag(mcol) Fc) (Fr^H diag(mrow) Fr) E~_k
// with E~_k = W * rowfac_k[col] * colfac_k[row] (W = amp e^{i phi}).  The
// row filter only sees rowfac_k, so points that share x_k (the row-transform
// groups of the plan) share it.  Two passes replace the three of the general
// path:
//   rows:  per group g, per pupil row: load W * rowfac_g, forward FFT,
//          * mrow, inverse FFT -> Y'[b][g][row][0..N)            (res rows)
//   cols:  per column block, per slot of points k: load colfac_k * Y'[g(k)]
//          column, forward FFT, * mcol, inverse FFT, accumulate
//          w_k |G_k|^2 in registers, then bin to the camera.
// The N x N field of each point never goes to memory, the per-point work
// drops from (res*ng/K + 3N) to (2 res*ng/K + 2N) line FFTs, and the mask
// read becomes two N-vectors.  The forward->filter->inverse chain of a line
// keeps the spectrum in registers (the inverse runs the radices in reverse
// order, as in pwfs_fast.cuh).
//
// The column pass also has a tangent form (accumulate 2 w_k Re(conj(G_k)
// dG_k) against stored operating-point columns G_k) and a form that stores
// G_k itself, which the JVP uses.
#pragma once
#include "xchg.cuh"

// One line through forward FFT -> diagonal filter -> inverse FFT, by the T
// threads of the line (butterflies j = t, t+T, ...).  load(p, m, j) gives
// input element j + m*R2 of the line (butterfly j = t + p*T; the same
// positions store() receives for the outputs, so one chain's outputs can
// feed the next from registers), filt(u) the filter at frequency u, store(p, j, v)
// receives the outputs v[q] = line[j + q*R2] (q < R1) of butterfly j = t+p*T.
// x1/x2: this line's forward/inverse exchange rows (stage outputs at j*RP+q).
// after_a() runs right after the barrier that ends the input loads.
// Every thread of the CTA calls it (it holds CTA-wide barriers).
// SHARE: x2 is x1 (one exchange buffer, one more barrier; needs one stage-B
// butterfly per thread).  before_last() runs just before the barrier that
// ends the forward half.
// NZ: the line's inputs j + m*R2 are zero for m >= NZ (the pupil sits at
// the start of the line), so stage A reads and transforms only the first NZ.
template <int N, int R1, int R2, int T, int RP1, int RP2, bool SHARE, int NZ, class Load, class Filt, class Store,
          class AfterA, class BeforeLast>
__device__ __forceinline__ void sep_chain_x(int t, float2* x1, float2* x2, const float2* tw, const float2* twi,
                                            Load load, Filt filt, Store store, AfterA after_a,
                                            BeforeLast before_last) {
  constexpr int PBA = (R2 + T - 1) / T;  // forward stage A / inverse stage B' butterflies
  constexpr int PBB = (R1 + T - 1) / T;  // forward stage B / inverse stage A' butterflies
  static_assert(!SHARE || PBB == 1, "a shared exchange needs one stage-B butterfly per thread");
  constexpr bool ALIAS = SHARE;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
      if constexpr (NZ < R1) {
#pragma unroll
        for (int m = 0; m < NZ; m++) v[m] = load(p, m, j);
        dft_front<R1, NZ, false>(v);
      } else {
#pragma unroll
        for (int m = 0; m < R1; m++) v[m] = load(p, m, j);
        dft<R1, false>(v);
      }
#pragma unroll
      for (int q = 0; q < R1; q++) x1[j * RP1 + q] = v[q];
    }
  }
  __syncthreads();
  after_a();
#pragma unroll
  for (int p = 0; p < PBB; p++) {
    const int j = t + p * T;
    float2 v[R2];
    if (j < R1) {
#pragma unroll
      for (int m = 0; m < R2; m++) {
        const float2 u = x1[m * RP1 + j];
        v[m] = (m == 0) ? u : cmul(u, tw[m * R1 + j]);
      }
      dft<R2, false>(v);
#pragma unroll
      for (int q = 0; q < R2; q++) v[q] = cmul(v[q], filt(j + q * R1));
      dft<R2, true>(v);
    }
    if constexpr (ALIAS) __syncthreads();  // every read of the forward exchange is done
    if (j < R1) {
#pragma unroll
      for (int q = 0; q < R2; q++) x2[j * RP2 + q] = v[q];
    }
  }
  before_last();
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
      float2 v[R1];
#pragma unroll
      for (int m = 0; m < R1; m++) {
        const float2 u = x2[m * RP2 + j];
        v[m] = (m == 0) ? u : cmul(u, twi[m * R2 + j]);
      }
      dft<R1, true>(v);
      store(p, j, v);
    }
  }
}

// The chain with the default exchange: shared whenever each thread holds one
// stage-B butterfly.
template <int N, int R1, int R2, int T, int RP1, int RP2, class Load, class Filt, class Store, class AfterA>
__device__ __forceinline__ void sep_chain(int t, float2* x1, float2* x2, const float2* tw, const float2* twi,
                                          Load load, Filt filt, Store store, AfterA after_a) {
  sep_chain_x<N, R1, R2, T, RP1, RP2, (R1 + T - 1) / T == 1, R1>(t, x1, x2, tw, twi, load, filt, store, after_a,
                                                                   [] {});
}

struct SepRowsArgs {
  const float2* tw;      // [N] W_N^t
  const float2* field;   // [B][res][res] pupil field of this pass's items
  const float2* rowfac;  // [groups][res] row-direction phasor of each group
  const float2* mrow;    // [N] mask factor along a row (column frequency)
  float2* y;             // [B][ng][res][N] filtered rows
  int res, ng, off;
};

// Pass 1: filtered rows (j-fastest thread mapping: line = tid / T).
template <int N, int R1, int R2, int T, int L, int NZ>
__global__ void __launch_bounds__(T* L) pwfs_srows(SepRowsArgs a) {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LS1 = xchg_stride(R2 * R1P, T, L, R1P, R2, R1);
  constexpr int LS2 = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr bool ALIAS = (R1 + T - 1) / T == 1;
  extern __shared__ float2 sm[];
  float2* tw = sm;       // tw[m*R1 + j]  = W_N^{j m}
  float2* twi = sm + N;  // twi[m*R2 + j] = W_N^{-j m}
  float2* mf = sm + 2 * N;
  float2* b1 = sm + 3 * N;
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
    mf[i] = a.mrow[i];
  }
  pdl_wait();  // the field comes from the previous kernel
  __syncthreads();
  const int b = blockIdx.z, g = blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < a.res;
  const int res = a.res, off = a.off;
  const float2* fld = a.field + ((size_t)b * res + (active ? row : 0)) * res;
  const float2* rf = a.rowfac + (size_t)g * res;
  float2* y = a.y + (((size_t)b * a.ng + g) * res + row) * N;
  sep_chain_x<N, R1, R2, T, R1P, R2P, ALIAS, NZ>(
      t, b1 + l * LS1, b2 + l * LS2, tw, twi,
      [&](int, int m, int j) {
        const int jc = j + m * R2 - off;
        return (active && jc >= 0 && jc < res) ? cmul(fld[jc], rf[jc]) : make_float2(0.f, 0.f);
      },
      [&](int u) { return mf[u]; },
      [&](int, int j, const float2* v) {
        if (active) {
#pragma unroll
          for (int q = 0; q < R1; q++) y[j + q * R2] = v[q];
        }
      },
      [] {}, [] {});
}

struct SepRowsIntArgs {
  const float2* tw;
  const float2* field;   // [B][res][res]
  const float2* rowfac;  // [ng][res] phasor of each group along the line
  const float2* mrow;    // [N] the 1-D mask factor (filter along the line)
  const float* gw;       // [ng] weight of each group (its points, or their weights)
  float* inten;          // [slices][B][res][N] sum over a slice's groups of gw |filtered line|^2, times scale
  size_t slice_stride;   // floats between slices
  int res, ng, g_per;    // groups, groups per slice (grid y = slices)
  float scale;
};

// Row pass of the one-axis path (masks that vary along the line's axis
// only): per pupil line, the filtered line of every group of the CTA's slice
// of groups, gw |.|^2 summed in registers over them, then written once.  The
// groups' lines never go to memory; slices keep small batches on every SM.
template <int N, int R1, int R2, int T, int L, int NZ>
__global__ void __launch_bounds__(T* L) pwfs_srows_int(SepRowsIntArgs a) {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LS1 = xchg_stride(R2 * R1P, T, L, R1P, R2, R1);
  constexpr int LS2 = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr bool ALIAS = (R1 + T - 1) / T == 1;
  constexpr int PBA = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* twi = sm + N;
  float2* mf = sm + 2 * N;
  float2* b1 = sm + 3 * N;
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
    mf[i] = a.mrow[i];
  }
  pdl_wait();  // the field comes from the previous kernel
  __syncthreads();
  const int b = blockIdx.z, row = blockIdx.x * L + l;
  const bool active = row < a.res;
  const int res = a.res;
  const float2* fld = a.field + ((size_t)b * res + (active ? row : 0)) * res;
  float acc[PBA][R1];
#pragma unroll
  for (int p = 0; p < PBA; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  const int g0 = blockIdx.y * a.g_per, g1 = min(a.ng, g0 + a.g_per);
  for (int g = g0; g < g1; g++) {
    if (ALIAS && g > g0) __syncthreads();  // the previous group's exchange reads are done
    const float2* rf = a.rowfac + (size_t)g * res;
    const float w = a.gw[g];
    sep_chain_x<N, R1, R2, T, R1P, R2P, ALIAS, NZ>(
        t, b1 + l * LS1, b2 + l * LS2, tw, twi,
        [&](int, int m, int j) {
          const int jc = j + m * R2;
          return (active && jc < res) ? cmul(fld[jc], rf[jc]) : make_float2(0.f, 0.f);
        },
        [&](int u) { return mf[u]; },
        [&](int p, int, const float2* v) {
#pragma unroll
          for (int q = 0; q < R1; q++) acc[p][q] = fmaf(w, cabs2(v[q]), acc[p][q]);
        },
        [] {}, [] {});
  }
  if (!active) return;
  float* out = a.inten + blockIdx.y * a.slice_stride + ((size_t)b * res + row) * N;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
#pragma unroll
      for (int q = 0; q < R1; q++) out[j + q * R2] = acc[p][q] * a.scale;
    }
  }
}

struct SepColsArgs {
  const float2* tw;
  const float2* mcol;    // [N] mask factor along a column (row frequency)
  const float2* y;       // [B][ng][res][N] filtered rows
  const int* group;      // [K] row-transform group of each point
  const float2* colfac;  // [K][res] column-direction phasor of each point
  const float* weights;  // [K] or null
  const float2* g0;      // tangent form: operating-point fields [K][N][N], else null
  float2* gout;          // storing form: G_k -> [K][N][N] (item 0 only), else null
  float* partial;        // [B][ksplit][N][N] un-binned sums, or null (then binned)
  float* binned;         // [B][ksplit][cam][cam]
  int res, off, ng, slot_pts, ksplit, bin, cam;
};

// Pass 2: filtered columns, |.|^2 (or the tangent product) summed over a
// slot of points, binned to the camera (l-fastest mapping: consecutive
// threads take consecutive columns, so the Y' loads are row segments).
// Grid (N / L column blocks, slots, items).  MODE: kSepIntensity sums
// w_k |G_k|^2, kSepTangent sums 2 w_k Re(conj(G_k) dG_k) with G_k read from
// g0, kSepStore writes G_k to gout.
constexpr int kSepIntensity = 0, kSepTangent = 1, kSepStore = 2;

// 16-byte asynchronous global -> shared copies (no register staging).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem))),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}

// Shared memory of the column pass: twiddles, filter, exchange, then the
// prefetch buffer of a point's Y' tile [res][L] and colfac row [res].
template <int N, int R1, int R2, int T, int L, bool SHARE = (R1 + T - 1) / T == 1>
struct SepColsSmem {
  static constexpr int LAY1 = cols_layout(R1, R2, T, L), LAY2 = cols_layout(R2, R1, T, L);
  static constexpr int LS1 = LAY1 & 0xFFFF, LS2 = LAY2 & 0xFFFF;
  static constexpr bool ALIAS = SHARE;
  static constexpr size_t kXch = 3 * (size_t)N;                                   // float2 offset
  static constexpr size_t kTiles = kXch + (size_t)L * (ALIAS ? imax(LS1, LS2) : LS1 + LS2);
  static __host__ __device__ size_t tile(int res) { return (size_t)res * (L + 1); }  // float2 per buffer
  static size_t bytes(int res) { return sizeof(float2) * (kTiles + tile(res)); }
};

template <int N, int R1, int R2, int T, int L, int MODE, int MAXREG, bool SHARE, int NZ>
__global__ void __launch_bounds__(T* L) __maxnreg__(MAXREG) pwfs_scols(SepColsArgs a) {
  using S = SepColsSmem<N, R1, R2, T, L, SHARE>;
  constexpr int R1P = S::LAY1 >> 16, LS1 = S::LS1;
  constexpr int R2P = S::LAY2 >> 16, LS2 = S::LS2;
  constexpr int PBA = (R2 + T - 1) / T;
  constexpr bool ALIAS = S::ALIAS;
  static_assert(L % 2 == 0, "16-byte tile copies");
  extern __shared__ __align__(16) float2 sm[];
  float2* tw = sm;
  float2* twi = sm + N;
  float2* mf = sm + 2 * N;
  float2* b1 = sm + S::kXch;
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int res = a.res, off = a.off;
  float2* tile = sm + S::kTiles;  // [res][L] Y' tile, then [res] colfac row
  const int tid = threadIdx.x;
  const int l = tid % L, t = tid / L;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
    mf[i] = a.mcol[i];
  }
  // grid (column blocks, slots, items); the tangent form takes (items,
  // slots, column blocks) instead, so the CTAs of one (column block, slot)
  // for every item of the launch run together and read each G_k tile from
  // HBM once, the others from L2
  const int b = (MODE == kSepTangent) ? blockIdx.x : blockIdx.z;
  const int slot = blockIdx.y, c0 = ((MODE == kSepTangent) ? blockIdx.z : blockIdx.x) * L, c = c0 + l;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  // copies of point kk's Y' tile (res rows x L columns) and colfac row,
  // issued once the previous point's stage A has read the buffer
  auto issue = [&](int kk) {
    const float2* src = a.y + ((size_t)b * a.ng + a.group[kk]) * res * N + c0;
    for (int i = tid; i < res * (L / 2); i += T * L) {
      const int row = i / (L / 2), ch = i - (i / (L / 2)) * (L / 2);
      cp_async16(tile + row * L + 2 * ch, src + (size_t)row * N + 2 * ch);
    }
    const float2* cfs = a.colfac + (size_t)kk * res;
    for (int i = tid; i < res / 2; i += T * L) cp_async16(tile + res * L + 2 * i, cfs + 2 * i);
    cp_async_commit();
  };
  pdl_wait();  // the filtered rows come from the previous kernel
  issue(kbeg);
  float acc[PBA][R1];
#pragma unroll
  for (int p = 0; p < PBA; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  if constexpr (!SHARE) {
    cp_async_wait<0>();
    __syncthreads();
  }
  for (int kk = kbeg; kk < kend; kk++) {
    if constexpr (SHARE) {
      cp_async_wait<0>();
      // the tile is visible to every thread, and the previous point's
      // exchange reads are done (the exchange buffer is reused)
      __syncthreads();
    }
    const float2* yt = tile + l;
    const float2* cf = tile + res * L;
    const float w = a.weights ? a.weights[kk] : 1.f;
    const float2* gi = (MODE == kSepTangent) ? a.g0 + (size_t)kk * N * N + c : nullptr;
    float2* go = (MODE == kSepStore) ? a.gout + (size_t)kk * N * N + c : nullptr;
    sep_chain_x<N, R1, R2, T, R1P, R2P, SHARE, NZ>(
        t, b1 + l * LS1, b2 + l * LS2, tw, twi,
        [&](int, int m, int j) {
          const int i = j + m * R2 - off;
          return (i >= 0 && i < res) ? cmul(yt[i * L], cf[i]) : make_float2(0.f, 0.f);
        },
        [&](int u) { return mf[u]; },
        [&](int p, int j, const float2* v) {
#pragma unroll
          for (int q = 0; q < R1; q++) {
            if constexpr (MODE == kSepStore) {
              go[(size_t)(j + q * R2) * N] = v[q];
            } else if constexpr (MODE == kSepTangent) {
              const float2 gq = gi[(size_t)(j + q * R2) * N];
              acc[p][q] = fmaf(2.f * w, fmaf(gq.x, v[q].x, gq.y * v[q].y), acc[p][q]);
            } else {
              acc[p][q] = fmaf(w, cabs2(v[q]), acc[p][q]);
            }
          }
        },
        [&] {
          if (kk + 1 < kend) issue(kk + 1);
        },
        [&] {
          // separate exchanges: the next point's tile lands before the
          // barrier that ends this point's forward half (its stage A follows
          // this point's stage B' with no barrier in between)
          if constexpr (!SHARE) cp_async_wait<0>();
        });
  }
  if constexpr (MODE == kSepStore) return;
  if (a.partial) {
    float* out = a.partial + ((size_t)b * a.ksplit + slot) * N * N + c;
#pragma unroll
    for (int p = 0; p < PBA; p++) {
      const int j = t + p * T;
      if (j < R2) {
#pragma unroll
        for (int q = 0; q < R1; q++) out[(size_t)(j + q * R2) * N] = acc[p][q];
      }
    }
    return;
  }
  // fused detector binning: the CTA's L columns are L/bin whole camera columns
  __syncthreads();
  float* cols = reinterpret_cast<float*>(b1);  // [L][N]
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
#pragma unroll
      for (int q = 0; q < R1; q++) cols[l * N + j + q * R2] = acc[p][q];
    }
  }
  __syncthreads();
  const int bin = a.bin, cam = a.cam, ncc = L / bin, cc0 = c0 / bin;
  float* out = a.binned + ((size_t)b * a.ksplit + slot) * cam * cam;
  for (int i = tid; i < ncc * cam; i += T * L) {
    const int cr = i / ncc, cx = i - (i / ncc) * ncc;
    float s = 0.f;
    for (int dx = 0; dx < bin; dx++) {
      const float* col = cols + (cx * bin + dx) * N + cr * bin;
      float cs = 0.f;
      for (int dy = 0; dy < bin; dy++) cs += col[dy];
      s += cs;
    }
    out[cr * cam + cc0 + cx] = s;
  }
}

// ---- adjoint (VJP) through the two passes ----
// Per item and point k, with G_k the forward field and the camera cotangent
// fbar: Gbar_k = 2 w_k fbar(binned pixel) G_k; the adjoint of the two 1-D
// filters is the same chain with the conjugate factors (forward FFT,
// * conj(m), inverse FFT: the transposes of the unnormalised transforms),
// so E~bar_k = (Fr^-1 conj(mrow) Fr)(Fc^-1 conj(mcol) Fc) Gbar_k on the
// pupil, and phibar = sum_k Im(E~bar_k conj(E~_k)) with E~_k = W rowfac_k
// colfac_k.  Column pass: G_k from the filtered rows (as in pwfs_scols),
// Gbar_k formed in registers and, as the next chain's stage-A inputs (the
// same thread positions), sent through the conjugate column filter; the
// pupil rows of the result, times conj(colfac_k), go to V_k [res][N].  Row
// pass: per pupil row, each point's V_k row through the conjugate row filter,
// Im(. conj(W rowfac_k)) summed over a slot of points.
struct SepAdjArgs {
  const float2* tw;
  const float2* mcol;    // [N]
  const float2* mrow;    // [N]
  const float2* y;       // [B][ng][res][N] filtered rows of the operating point
  const int* group;      // [K]
  const float2* colfac;  // [K][res]
  const float2* rowfac;  // [groups][res]
  const float* weights;  // [K] or null
  const float* fbar;     // [B][cam][cam] camera-frame cotangent
  const float2* field;   // [B][res][res] W
  float2* v;             // [B][K][res][N]
  float* phibar;         // [B][ksplit][res][res] slot partials (row pass)
  int res, off, ng, slot_pts, ksplit, bin, cam;
};

// Two chains per point with Gbar held between them: 128 registers keep it
// (with 96 it spilled ~300 bytes per thread).
template <int N, int R1, int R2, int T, int L, int NZ>
__global__ void __maxnreg__(128) pwfs_scols_adj(SepAdjArgs a) {
  using S = SepColsSmem<N, R1, R2, T, L>;
  constexpr int R1P = S::LAY1 >> 16, LS1 = S::LS1;
  constexpr int R2P = S::LAY2 >> 16, LS2 = S::LS2;
  constexpr int PBA = (R2 + T - 1) / T;
  constexpr bool ALIAS = S::ALIAS;
  extern __shared__ __align__(16) float2 sm[];
  float2* tw = sm;
  float2* twi = sm + N;
  float2* mf = sm + 2 * N;
  float2* b1 = sm + S::kXch;
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int res = a.res, off = a.off;
  float2* tile = sm + S::kTiles;
  const int tid = threadIdx.x;
  const int l = tid % L, t = tid / L;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
    mf[i] = a.mcol[i];
  }
  const int b = blockIdx.z, slot = blockIdx.y, c0 = blockIdx.x * L, c = c0 + l;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  const float* fb = a.fbar + (size_t)b * a.cam * a.cam + c / a.bin;
  auto issue = [&](int kk) {
    const float2* src = a.y + ((size_t)b * a.ng + a.group[kk]) * res * N + c0;
    for (int i = tid; i < res * (L / 2); i += T * L) {
      const int row = i / (L / 2), ch = i - (i / (L / 2)) * (L / 2);
      cp_async16(tile + row * L + 2 * ch, src + (size_t)row * N + 2 * ch);
    }
    const float2* cfs = a.colfac + (size_t)kk * res;
    for (int i = tid; i < res / 2; i += T * L) cp_async16(tile + res * L + 2 * i, cfs + 2 * i);
    cp_async_commit();
  };
  issue(kbeg);
  for (int kk = kbeg; kk < kend; kk++) {
    cp_async_wait<0>();
    __syncthreads();
    const float2* yt = tile + l;
    const float2* cf = tile + res * L;
    const float w2 = 2.f * (a.weights ? a.weights[kk] : 1.f);
    float2 gb[PBA][R1];  // Gbar of this column, rows j + q*R2
    sep_chain_x<N, R1, R2, T, R1P, R2P, ALIAS, NZ>(
        t, b1 + l * LS1, b2 + l * LS2, tw, twi,
        [&](int, int m, int j) {
          const int i = j + m * R2 - off;
          return (i >= 0 && i < res) ? cmul(yt[i * L], cf[i]) : make_float2(0.f, 0.f);
        },
        [&](int u) { return mf[u]; },
        [&](int p, int j, const float2* v) {
#pragma unroll
          for (int q = 0; q < R1; q++) {
            const float s = w2 * __ldg(fb + ((j + q * R2) / a.bin) * a.cam);
            gb[p][q] = make_float2(s * v[q].x, s * v[q].y);
          }
        },
        [&] {
          if (kk + 1 < kend) issue(kk + 1);
        },
        [] {});
    if (ALIAS) __syncthreads();  // the first chain's last exchange reads are done
    float2* vo = a.v + ((size_t)b * gridDim.y * a.slot_pts + kk) * res * N + c;
    const float2* cfg = a.colfac + (size_t)kk * res;
    sep_chain<N, R1, R2, T, R1P, R2P>(
        t, b1 + l * LS1, b2 + l * LS2, tw, twi,
        [&](int p, int m, int) { return gb[p][m]; },
        [&](int u) { return cconj(mf[u]); },
        [&](int, int j, const float2* v) {
#pragma unroll
          for (int q = 0; q < R1; q++) {
            const int i = j + q * R2 - off;
            if (i >= 0 && i < res) vo[(size_t)i * N] = cmul(v[q], cconj(__ldg(cfg + i)));
          }
        },
        [] {});
  }
}

template <int N, int R1, int R2, int T, int L>
__global__ void __maxnreg__(128) pwfs_srows_adj(SepAdjArgs a) {
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr int LS1 = xchg_stride(R2 * R1P, T, L, R1P, R2, R1);
  constexpr int LS2 = xchg_stride(R1 * R2P, T, L, R2P, R1, R2);
  constexpr bool ALIAS = (R1 + T - 1) / T == 1;
  constexpr int PBA = (R2 + T - 1) / T;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* twi = sm + N;
  float2* mf = sm + 2 * N;
  float2* b1 = sm + 3 * N;
  float2* b2 = ALIAS ? b1 : b1 + L * LS1;
  const int tid = threadIdx.x;
  const int l = tid / T, t = tid - (tid / T) * T;
  for (int i = tid; i < N; i += T * L) {
    tw[i] = a.tw[(i % R1) * (i / R1)];
    const float2 w = a.tw[(i % R2) * (i / R2)];
    twi[i] = make_float2(w.x, -w.y);
    mf[i] = cconj(a.mrow[i]);
  }
  __syncthreads();
  const int res = a.res, off = a.off;
  const int b = blockIdx.z, slot = blockIdx.y, row = blockIdx.x * L + l;
  const bool active = row < res;
  const int K = gridDim.y * a.slot_pts;
  const int kbeg = slot * a.slot_pts, kend = kbeg + a.slot_pts;
  const float2* fld = a.field + ((size_t)b * res + (active ? row : 0)) * res;
  float acc[PBA][R1];
#pragma unroll
  for (int p = 0; p < PBA; p++)
#pragma unroll
    for (int q = 0; q < R1; q++) acc[p][q] = 0.f;
  for (int kk = kbeg; kk < kend; kk++) {
    if (ALIAS && kk > kbeg) __syncthreads();  // the previous point's exchange reads are done
    const float2* vr = a.v + (((size_t)b * K + kk) * res + (active ? row : 0)) * N;
    const float2* rf = a.rowfac + (size_t)a.group[kk] * res;
    // an offset the compiler cannot see is zero keeps the field loads inside
    // the loop instead of hoisted into registers across points
    int zero;
    asm volatile("mov.b32 %0, 0;" : "=r"(zero));
    const float2* fr = fld + zero;
    sep_chain<N, R1, R2, T, R1P, R2P>(
        t, b1 + l * LS1, b2 + l * LS2, tw, twi,
        [&](int, int m, int j) { return active ? vr[j + m * R2] : make_float2(0.f, 0.f); },
        [&](int u) { return mf[u]; },
        [&](int p, int j, const float2* v) {
          if (active) {
#pragma unroll
            for (int q = 0; q < R1; q++) {
              const int jc = j + q * R2 - off;
              if (jc >= 0 && jc < res) {
                const float2 e = cmul(fr[jc], __ldg(rf + jc));
                acc[p][q] += v[q].y * e.x - v[q].x * e.y;
              }
            }
          }
        },
        [] {});
  }
  if (!active) return;
  float* out = a.phibar + (((size_t)b * a.ksplit + slot) * res + row) * res;
#pragma unroll
  for (int p = 0; p < PBA; p++) {
    const int j = t + p * T;
    if (j < R2) {
#pragma unroll
      for (int q = 0; q < R1; q++) {
        const int jc = j + q * R2 - off;
        if (jc >= 0 && jc < res) out[jc] = acc[p][q];
      }
    }
  }
}

struct SepPasses {
  int n, r1, r2, t, l_rows, l_cols;
  int nz;  // stage-A inputs read per butterfly: the pupil must satisfy res <= nz * r2
  void (*rows)(SepRowsArgs);
  void (*rows_int)(SepRowsIntArgs);  // the one-axis path's row pass (filtered-line intensity over groups)
  void (*cols[3])(SepColsArgs);  // indexed by kSepIntensity / kSepTangent / kSepStore
  void (*cols_adj)(SepAdjArgs);
  void (*rows_adj)(SepAdjArgs);
  size_t smem_rows;
  size_t (*smem_cols)(int res);
};

// MAXREG caps the column pass's registers per thread (its occupancy).
// NZ: non-zero inputs per stage-A butterfly (the pupil occupies at most half
// of a line, res <= N/2, so at most ceil(R1/2) of the R1 inputs j + m*R2
// fall inside it).
template <int N, int R1, int R2, int T, int LR, int LC, int MAXREG, bool SHARE = (R1 + T - 1) / T == 1,
          int NZ = (R1 + 1) / 2>
SepPasses make_sep() {
  static_assert(N % LC == 0, "column blocks must tile N");
  constexpr int R1P = pad_odd(R1), R2P = pad_odd(R2);
  constexpr bool ALIAS = (R1 + T - 1) / T == 1;
  constexpr int LSR1 = xchg_stride(R2 * R1P, T, LR, R1P, R2, R1);
  constexpr int LSR2 = xchg_stride(R1 * R2P, T, LR, R2P, R1, R2);
  constexpr int LSR = ALIAS ? imax(LSR1, LSR2) : LSR1 + LSR2;
  constexpr int LSC1 = cols_layout(R1, R2, T, LC) & 0xFFFF, LSC2 = cols_layout(R2, R1, T, LC) & 0xFFFF;
  constexpr int LSC = SHARE ? imax(LSC1, LSC2) : LSC1 + LSC2;
  // the binning epilogue reuses the exchange as [LC][N] floats
  static_assert((size_t)LC * LSC * 2 >= (size_t)LC * N, "exchange too small for the binning rows");
  SepPasses s;
  s.n = N; s.r1 = R1; s.r2 = R2; s.t = T; s.l_rows = LR; s.l_cols = LC;
  s.nz = NZ;
  s.rows = pwfs_srows<N, R1, R2, T, LR, NZ>;
  s.rows_int = pwfs_srows_int<N, R1, R2, T, LR, NZ>;
  s.cols[kSepIntensity] = pwfs_scols<N, R1, R2, T, LC, kSepIntensity, MAXREG, SHARE, NZ>;
  s.cols[kSepTangent] = pwfs_scols<N, R1, R2, T, LC, kSepTangent, MAXREG, SHARE, NZ>;
  s.cols[kSepStore] = pwfs_scols<N, R1, R2, T, LC, kSepStore, MAXREG, SHARE, NZ>;
  s.cols_adj = pwfs_scols_adj<N, R1, R2, T, LC, NZ>;
  s.rows_adj = pwfs_srows_adj<N, R1, R2, T, LR>;
  s.smem_rows = sizeof(float2) * (3 * (size_t)N + (size_t)LR * LSR);
  s.smem_cols = &SepColsSmem<N, R1, R2, T, LC, SHARE>::bytes;
  return s;
}

// Compile-time two-pass plans for an FFT size (pwfs_sep.cu); 0 when none.
int sep_candidates(int n, const SepPasses** out);
