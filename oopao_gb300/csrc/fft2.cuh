// Register-resident two-stage FFTs of length N = R1*R2 (compile-time plans).
//
// Forward transform (Stockham, two stages):
//   stage A: R2 butterflies of radix R1, span 1:  inputs  x[j + m*R2]  (m < R1)
//            outputs  t[j*R1 + q]                                       (q < R1)
//   stage B: R1 butterflies of radix R2, span R1: inputs  t[j + m*R1] * W_N^{j*m}
//            outputs  X[j + q*R1]                                       (q < R2)
// The inverse uses the reversed order (radix R2 first, then R1) so that the
// registers a thread holds after a forward stage B (X[j + q*R1], j < R1) are
// exactly the inputs of the inverse stage A (x[j + m*R1]) — a focal-plane mask
// can be applied in between without a shared-memory round trip.
//
// Each thread owns butterflies j = t, t+T, ... of a line; loads of stage A
// and stores of stage B touch consecutive addresses for consecutive j, so the
// caller feeds and drains them straight from/to global memory.  The single
// exchange between the stages goes through shared memory with rows padded to
// an odd length (conflict-free strided writes).
//
// Radix-R DFTs are fully unrolled in registers; composite R are split
// R = A*B (decimation in time) with compile-time twiddles.
#pragma once
#include "fft.cuh"

__host__ __device__ constexpr int pad_odd(int r) { return (r % 2 == 0) ? r + 1 : r; }

template <int R>
struct DftSplit { static constexpr int A = 0, B = 0; };
template <> struct DftSplit<6> { static constexpr int A = 2, B = 3; };
template <> struct DftSplit<10> { static constexpr int A = 2, B = 5; };
template <> struct DftSplit<12> { static constexpr int A = 4, B = 3; };
template <> struct DftSplit<14> { static constexpr int A = 2, B = 7; };
template <> struct DftSplit<15> { static constexpr int A = 5, B = 3; };
template <> struct DftSplit<18> { static constexpr int A = 2, B = 9; };
template <> struct DftSplit<20> { static constexpr int A = 4, B = 5; };
template <> struct DftSplit<21> { static constexpr int A = 7, B = 3; };
template <> struct DftSplit<22> { static constexpr int A = 2, B = 11; };
template <> struct DftSplit<24> { static constexpr int A = 8, B = 3; };
template <> struct DftSplit<27> { static constexpr int A = 9, B = 3; };
template <> struct DftSplit<28> { static constexpr int A = 4, B = 7; };
template <> struct DftSplit<30> { static constexpr int A = 2, B = 15; };
template <> struct DftSplit<32> { static constexpr int A = 8, B = 4; };
template <> struct DftSplit<33> { static constexpr int A = 11, B = 3; };
template <> struct DftSplit<35> { static constexpr int A = 7, B = 5; };
template <> struct DftSplit<36> { static constexpr int A = 4, B = 9; };
template <> struct DftSplit<40> { static constexpr int A = 8, B = 5; };
template <> struct DftSplit<42> { static constexpr int A = 2, B = 21; };
template <> struct DftSplit<44> { static constexpr int A = 4, B = 11; };
template <> struct DftSplit<45> { static constexpr int A = 9, B = 5; };
template <> struct DftSplit<48> { static constexpr int A = 16, B = 3; };
template <> struct DftSplit<56> { static constexpr int A = 8, B = 7; };
template <> struct DftSplit<60> { static constexpr int A = 4, B = 15; };
template <> struct DftSplit<63> { static constexpr int A = 9, B = 7; };
template <> struct DftSplit<64> { static constexpr int A = 16, B = 4; };

template <int R>
__host__ __device__ constexpr bool dft_direct() {
  return R == 2 || R == 4 || R == 8 || R == 16 || (R % 2 == 1 && R <= 13);
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2* v);

// R = A*B, n = a*B + b, k = k1 + A*k2:
// X[k1 + A k2] = sum_b W_B^{b k2} W_R^{b k1} sum_a x[aB + b] W_A^{a k1}
template <int R, bool INV>
__device__ __forceinline__ void dft_composite(float2* v) {
  constexpr int A = DftSplit<R>::A, B = DftSplit<R>::B;
  static_assert(A * B == R, "missing DftSplit specialisation");
  float2 y[R];
#pragma unroll
  for (int b = 0; b < B; b++) {
    float2 u[A];
#pragma unroll
    for (int a = 0; a < A; a++) u[a] = v[a * B + b];
    dft<A, INV>(u);
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) {
      const int t = (b * k1) % R;
      if (t == 0) {
        y[k1 * B + b] = u[k1];
      } else if (4 * t == R) {  // W_R^{R/4}: -i forward, +i inverse
        y[k1 * B + b] = mul_mi<INV>(u[k1]);
      } else if (2 * t == R) {
        y[k1 * B + b] = make_float2(-u[k1].x, -u[k1].y);
      } else if (4 * t == 3 * R) {
        y[k1 * B + b] = mul_mi<!INV>(u[k1]);
      } else {
        const float c = rad_cos(R, t), s = INV ? rad_sin(R, t) : -rad_sin(R, t);
        y[k1 * B + b] = cmul(u[k1], make_float2(c, s));
      }
    }
  }
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) {
    float2 w[B];
#pragma unroll
    for (int b = 0; b < B; b++) w[b] = y[k1 * B + b];
    dft<B, INV>(w);
#pragma unroll
    for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = w[k2];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2* v) {
  if constexpr (R == 1) {
    return;
  } else if constexpr (dft_direct<R>()) {
    Dft<R, INV>::run(v);
  } else {
    dft_composite<R, INV>(v);
  }
}

// ---- transforms of lines whose inputs are zero past the first NZ ----
// Split R = A*B used on the input side (u[a] = v[a*B + b]): B large, so that
// most of the A-point sub-transforms see at most one non-zero input.
template <int R>
struct PruneSplit { static constexpr int A = 0, B = 0; };
template <> struct PruneSplit<8> { static constexpr int A = 2, B = 4; };
template <> struct PruneSplit<12> { static constexpr int A = 3, B = 4; };
template <> struct PruneSplit<16> { static constexpr int A = 2, B = 8; };
template <> struct PruneSplit<24> { static constexpr int A = 3, B = 8; };
template <> struct PruneSplit<48> { static constexpr int A = 4, B = 12; };

// A-point DFT of u whose entries past the first NZ are zero (not read).
template <int A, int NZ, bool INV>
__device__ __forceinline__ void dft_lead(float2* u) {
  if constexpr (NZ >= A) {
    dft<A, INV>(u);
  } else if constexpr (NZ == 1) {
#pragma unroll
    for (int k = 1; k < A; k++) u[k] = u[0];
  } else {
    float2 y[A];
#pragma unroll
    for (int k = 0; k < A; k++) {
      float2 acc = u[0];
#pragma unroll
      for (int a = 1; a < NZ; a++) {
        const int t = (a * k) % A;
        if (t == 0) {
          acc = cadd(acc, u[a]);
        } else {
          const float c = rad_cos(A, t), sn = INV ? rad_sin(A, t) : -rad_sin(A, t);
          acc.x = fmaf(u[a].x, c, fmaf(-u[a].y, sn, acc.x));
          acc.y = fmaf(u[a].x, sn, fmaf(u[a].y, c, acc.y));
        }
      }
      y[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < A; k++) u[k] = y[k];
  }
}

template <int R, int NZ, bool INV, int b>
__device__ __forceinline__ void prune_front_stage(const float2* v, float2* y) {
  constexpr int A = PruneSplit<R>::A, B = PruneSplit<R>::B;
  if constexpr (b < B) {
    constexpr int nz = NZ > b ? (NZ - b + B - 1) / B : 0;  // inputs a*B + b < NZ
    if constexpr (nz == 0) {
#pragma unroll
      for (int k1 = 0; k1 < A; k1++) y[k1 * B + b] = make_float2(0.f, 0.f);
    } else {
      float2 u[A];
#pragma unroll
      for (int a = 0; a < nz; a++) u[a] = v[a * B + b];
      dft_lead<A, nz, INV>(u);
#pragma unroll
      for (int k1 = 0; k1 < A; k1++) {
        const int t = (b * k1) % R;
        if (t == 0) {
          y[k1 * B + b] = u[k1];
        } else if (4 * t == R) {
          y[k1 * B + b] = mul_mi<INV>(u[k1]);
        } else if (2 * t == R) {
          y[k1 * B + b] = make_float2(-u[k1].x, -u[k1].y);
        } else if (4 * t == 3 * R) {
          y[k1 * B + b] = mul_mi<!INV>(u[k1]);
        } else {
          const float c = rad_cos(R, t), sn = INV ? rad_sin(R, t) : -rad_sin(R, t);
          y[k1 * B + b] = cmul(u[k1], make_float2(c, sn));
        }
      }
    }
    prune_front_stage<R, NZ, INV, b + 1>(v, y);
  }
}

// R-point DFT of v whose entries v[m], m >= NZ, are zero (only the first NZ
// are read).  Same result as dft<R> on the zero-padded line.
template <int R, int NZ, bool INV>
__device__ __forceinline__ void dft_front(float2* v) {
  constexpr int A = PruneSplit<R>::A, B = PruneSplit<R>::B;
  static_assert(NZ >= R || A * B == R, "no pruning split for this radix");
  if constexpr (NZ >= R) {
    dft<R, INV>(v);
  } else {
    float2 y[R];
    prune_front_stage<R, NZ, INV, 0>(v, y);
#pragma unroll
    for (int k1 = 0; k1 < A; k1++) {
      float2 w[B];
#pragma unroll
      for (int b = 0; b < B; b++) w[b] = y[k1 * B + b];
      dft<B, INV>(w);
#pragma unroll
      for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = w[k2];
    }
  }
}

// Exchange-buffer slot of stage-A output index p (radix RA first stage).
template <int RA>
__device__ __forceinline__ int xslot(int p) {
  return (p / RA) * pad_odd(RA) + (p % RA);
}
