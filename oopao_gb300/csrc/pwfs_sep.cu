// Compile-time two-pass (separable-mask) plans, see pwfs_sep.cuh.
// Parameters per FFT size N = R1*R2: T threads per line, LR rows per CTA of
// the row pass, LC columns per CTA of the column pass (a multiple of the
// usual detector binning of 6, so that the binning fuses into the column
// pass; N must be a multiple of LC), and the column pass's register cap.
// Measured on GB300 (20x20 at batch 1-100, 40x40 at batch 1-16): the first
// entry of each size is the fastest or within 1%; register caps of 72-80
// (more resident CTAs, with spills), the other radix orders, and separate
// forward/inverse exchange buffers where one could be shared (two barriers
// fewer per point, but a third fewer resident warps: 3-17% slower) were
// slower.
#include "common.cuh"
#include "pwfs_sep.cuh"

int sep_candidates(int n, const SepPasses** out) {
  static const SepPasses s72[] = {make_sep<72, 8, 9, 9, 8, 12, 96>()};
  static const SepPasses s96[] = {make_sep<96, 8, 12, 12, 8, 12, 96>()};
  static const SepPasses s112[] = {make_sep<112, 16, 7, 8, 16, 16, 96>()};
  static const SepPasses s128[] = {make_sep<128, 16, 8, 8, 16, 16, 96>()};
  static const SepPasses s240[] = {make_sep<240, 16, 15, 16, 8, 12, 96>()};
  static const SepPasses s264[] = {make_sep<264, 12, 22, 12, 16, 12, 96>(), make_sep<264, 24, 11, 12, 16, 12, 96>()};
  static const SepPasses s480[] = {make_sep<480, 24, 20, 24, 8, 12, 96>()};
  static const SepPasses s504[] = {make_sep<504, 24, 21, 24, 8, 12, 96>(), make_sep<504, 24, 21, 24, 8, 6, 96>()};
  static const SepPasses s1920[] = {make_sep<1920, 48, 40, 48, 2, 6, 168>()};
#define OOPAO_SEP(arr) (*out = arr, (int)(sizeof(arr) / sizeof(arr[0])))
  switch (n) {
    case 72: return OOPAO_SEP(s72);
    case 96: return OOPAO_SEP(s96);
    case 112: return OOPAO_SEP(s112);
    case 128: return OOPAO_SEP(s128);
    case 240: return OOPAO_SEP(s240);
    case 264: return OOPAO_SEP(s264);
    case 480: return OOPAO_SEP(s480);
    case 504: return OOPAO_SEP(s504);
    case 1920: return OOPAO_SEP(s1920);
    default: *out = nullptr; return 0;
  }
#undef OOPAO_SEP
}
