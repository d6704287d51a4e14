// Compile-time layout search for the shared-memory exchange between the two
// stages of the register-resident line FFTs (fft2.cuh): line strides and
// row paddings with the fewest bank conflicts for a pass's thread mapping.
#pragma once
#include "fft2.cuh"

__host__ __device__ constexpr int odd_up(int v) { return (v % 2 == 0) ? v + 1 : v; }
__host__ __device__ constexpr int imax(int a, int b) { return a > b ? a : b; }

// Shared-memory bank conflicts of the exchange buffer of a j-fastest pass
// (thread tid -> line tid/T, butterfly tid%T): stage-A writes at
// line*LS + j*RP (j < nw) and stage-B reads at line*LS + j (j < nr), 8-byte
// words, counted per 16-thread phase.  Used at compile time to pick the line
// stride.
__host__ __device__ constexpr int xchg_conflicts(int LS, int T, int L, int RP, int nw, int nr) {
  int total = 0;
  for (int pat = 0; pat < 2; pat++) {
    const int nj = pat == 0 ? nw : nr, stride = pat == 0 ? RP : 1;
    for (int base = 0; base < T * L; base += 16) {
      int cnt[16] = {};
      for (int u = 0; u < 16 && base + u < T * L; u++) {
        const int tid = base + u, l = tid / T, t = tid % T;
        if (t >= nj) continue;
        cnt[(l * LS + t * stride) % 16]++;
      }
      int mx = 0;
      for (int i = 0; i < 16; i++) mx = cnt[i] > mx ? cnt[i] : mx;
      total += mx > 0 ? mx - 1 : 0;
    }
  }
  return total;
}

__host__ __device__ constexpr int xchg_stride(int min_ls, int T, int L, int RP, int nw, int nr) {
  int best = min_ls, best_c = 1 << 30;
  for (int ls = min_ls; ls < min_ls + 16; ls++) {
    const int c = xchg_conflicts(ls, T, L, RP, nw, nr);
    if (c < best_c) {
      best_c = c;
      best = ls;
    }
  }
  return best;
}

// Same count for an l-fastest pass (thread tid -> line tid % L, butterfly
// tid / L), as the column pass maps its threads.
__host__ __device__ constexpr int xchg_conflicts_lf(int LS, int T, int L, int RP, int nw, int nr) {
  int total = 0;
  for (int pat = 0; pat < 2; pat++) {
    const int nj = pat == 0 ? nw : nr, stride = pat == 0 ? RP : 1;
    for (int base = 0; base < T * L; base += 16) {
      int cnt[16] = {};
      for (int u = 0; u < 16 && base + u < T * L; u++) {
        const int tid = base + u, l = tid % L, t = tid / L;
        if (t >= nj) continue;
        cnt[(l * LS + t * stride) % 16]++;
      }
      int mx = 0;
      for (int i = 0; i < 16; i++) mx = cnt[i] > mx ? cnt[i] : mx;
      total += mx > 0 ? mx - 1 : 0;
    }
  }
  return total;
}

// Exchange layout of one column-pass buffer: radix-R butterflies write
// R values at j*RP (j < NW) and are read back at m*RP + j (j < R); RP >= R
// and the line stride LS >= NW*RP are searched for the fewest conflicts
// (ties: least shared memory).  Returns RP * 65536 + LS.
__host__ __device__ constexpr int cols_layout(int R, int NW, int T, int L) {
  int best = 0, best_c = 1 << 30, best_sz = 1 << 30;
  for (int rp = R; rp < R + 4; rp++) {
    for (int ls = NW * rp; ls < NW * rp + 16; ls++) {
      const int c = xchg_conflicts_lf(ls, T, L, rp, NW, R);
      if (c < best_c || (c == best_c && ls < best_sz)) {
        best_c = c;
        best_sz = ls;
        best = rp * 65536 + ls;
      }
    }
  }
  return best;
}
