// Detector readout stages that need no random numbers: full-well saturation,
// and the tail of the readout (CCD/CMOS gain, ADC digitisation, log scale,
// the cast to the output precision, background-map removal).  One CTA per
// frame: the ADC needs the frame's maximum, so each CTA reduces its frame in
// shared memory and then rewrites it in place.  Frames are small (at most a
// few hundred pixels a side), so the work is a few reads of each pixel.
#include "common.cuh"

namespace {

constexpr int kDetThreads = 512;

__device__ __forceinline__ float block_max(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : -INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[32] = v;
  }
  __syncthreads();
  const float r = red[32];
  __syncthreads();
  return r;
}

// Frame maximum (before clipping) into max_out, then clip to [0, fwc].
__global__ void __launch_bounds__(kDetThreads) det_saturate(float* frames, int npix, float fwc, float* max_out) {
  __shared__ float red[33];
  float* f = frames + (size_t)blockIdx.x * npix;
  float m = -INFINITY;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) m = fmaxf(m, f[i]);
  m = block_max(m, red);
  if (threadIdx.x == 0) max_out[blockIdx.x] = m;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) f[i] = fminf(fmaxf(f[i], 0.f), fwc);
}

struct DetTail {
  float gain;      // applied first (1 for an EMCCD, whose gain acts before binning)
  int bits;        // ADC bits, 0: no digitisation
  float fwc;       // full well, <= 0: none (the ADC then scales by the frame maximum)
  int clip_zero;   // the ADC clips at 0 (unsigned output)
  int log_scale;
  int out_bits;    // 8/16/32/64: unsigned output of that width, 0: floating point
  const float* bg; // [npix] background map subtracted last, or null
};

__global__ void __launch_bounds__(kDetThreads) det_tail(float* frames, int npix, DetTail p, float* max_out) {
  __shared__ float red[33];
  float* f = frames + (size_t)blockIdx.x * npix;
  float m = -INFINITY;
  if (p.bits > 0 || max_out) {
    for (int i = threadIdx.x; i < npix; i += blockDim.x) m = fmaxf(m, f[i] * p.gain);
    m = block_max(m, red);
    if (max_out && threadIdx.x == 0) max_out[blockIdx.x] = m;
  }
  // the ADC levels and the integer conversion in double: 2^bits - 1 is not
  // a float for bits > 24, and a float top level would wrap to 0 in the
  // unsigned conversion
  const double levels = exp2((double)p.bits);
  for (int i = threadIdx.x; i < npix; i += blockDim.x) {
    double v = (double)(f[i] * p.gain);
    if (p.bits > 0) {
      if (p.fwc <= 0.f) {
        v = v / (double)m * levels;
      } else {
        v = v / (double)p.fwc * (levels - 1.0);
        if (p.clip_zero) v = fmax(v, 0.0);
        v = fmin(v, levels - 1.0);
      }
    }
    if (p.log_scale) v = log10(v);
    if (p.out_bits > 0) {
      // conversion to an unsigned integer: truncation toward zero; values
      // outside the type's range wrap modulo 2^bits
      v = trunc(v);
      if (p.out_bits < 64) {
        const double span = exp2((double)p.out_bits);
        v = fmod(v, span);
        if (v < 0) v += span;
      }
    }
    if (p.bg) v -= (double)p.bg[i];
    f[i] = (float)v;
  }
}

}  // namespace

extern "C" int oopao_det_saturate(float* frames, int nframes, int npix, float fwc, float* max_out, void* stream) {
  OOPAO_CHECK_ARG(frames && max_out, "NULL argument");
  OOPAO_CHECK_ARG(nframes >= 1 && npix >= 1 && fwc > 0.f, "bad size or full-well capacity");
  det_saturate<<<nframes, kDetThreads, 0, (cudaStream_t)stream>>>(frames, npix, fwc, max_out);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_det_readout_tail(float* frames, int nframes, int npix, float gain, int bits, float fwc,
                                      int clip_zero, int log_scale, int out_bits, const float* bg_map,
                                      float* max_out, void* stream) {
  OOPAO_CHECK_ARG(frames, "NULL frames");
  OOPAO_CHECK_ARG(nframes >= 1 && npix >= 1, "bad size");
  OOPAO_CHECK_ARG(bits >= 0 && bits <= 64, "bits must be 0 (none) to 64");
  OOPAO_CHECK_ARG(out_bits == 0 || out_bits == 8 || out_bits == 16 || out_bits == 32 || out_bits == 64,
                  "output width must be 0 (floating point), 8, 16, 32 or 64");
  DetTail p{gain, bits, fwc, clip_zero, log_scale, out_bits, bg_map};
  det_tail<<<nframes, kDetThreads, 0, (cudaStream_t)stream>>>(frames, npix, p, max_out);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
