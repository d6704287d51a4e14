// BF16 tensor-core influence-function projection on sm_103a (tcgen05 + TMA).
//
// opd[b][p] = scale * sum_a modes[p][a] * coefs[a][b] (+ base[b][p])
// (dm.coefs setter, OOPAO/DeformableMirror.py:651-686), as a GEMM
//   D[M = pixels][N = batch] = A[M][K = actuators] * B[N][K]^T
// with A = the IF matrix in BF16, K-major ([n_pix][n_act_pad]), B = the
// coefficients transposed to BF16 K-major and split into two BF16 terms,
// hi = bf16(c) and lo = bf16(c - hi) ([2][batch_pad][n_act_pad]).  Both terms
// accumulate into the same FP32 tile, so the coefficients keep ~16
// significant bits and the only BF16 rounding left is the IF storage.
//
// A persistent CTA per SM walks the 128 x BN output tiles.  One thread
// streams 128x64 A and two BNx64 B tiles (hi, then lo; 128-byte swizzle)
// through a 4-stage mbarrier ring; one thread issues tcgen05.mma (kind::f16,
// M=128, K=16) with N = 2*BN, so each instruction multiplies the A tile by the
// hi and the lo coefficients at once (A is read from shared memory once for
// both) into a 2*BN-column TMEM accumulator; four epilogue warps read the
// accumulator back with tcgen05.ld (32 lanes x 16 columns per load), add the
// hi and lo halves and store FP32, coalesced along pixels.  Two accumulators
// (4*BN of the 512 TMEM columns) let the epilogue of one tile overlap the
// MMAs of the next.  Every mbarrier wait is bounded, and every role gives up
// as soon as another has recorded an error: the CTA then drains its loads in
// flight, still frees its TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "tma.cuh"

namespace {

constexpr int kBM = 128;     // pixels per tile = TMEM lanes
constexpr int kBK = 64;      // BF16 actuators per stage (n_act_pad granularity of the BF16 IFs)
constexpr int kEpiWarps = 4;                 // one per quarter of the TMEM lanes
constexpr int kThreads = 64 + 32 * kEpiWarps;  // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

struct TcParams {
  int n_pix, batch;
  int nk;         // K tiles
  int batch_pad;  // row offset of the lo coefficients
  int tiles_n;    // batch tiles per pixel tile
  int tiles;      // all tiles
  float scale;
  const float* base;
  float* out;
  int* err;
};

using tma::mbar_expect_tx;
using tma::mbar_init;
using tma::smem_u32;

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  tma::load_2d(dst, map, bar, x, y);
}

// Bounded wait for phase `parity` that also gives up once any role of the
// launch has recorded an error (checked every 1024 polls); false then, and
// `code` in *err on a time-out of its own.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, int* err, int code) {
  const long long t0 = clock64();
  for (unsigned i = 1;; i++) {
    if (tma::mbar_try_wait(bar, parity)) return true;
    if ((i & 1023u) == 0) {
      if (*(volatile int*)err != 0) return false;
      if (clock64() - t0 > tma::kWaitCycles) {
        atomicExch(err, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;             // leading byte offset (16 B; unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;             // version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// The two operand forms of the GEMM.  BF16: the IFs in BF16, the
// coefficients as hi + lo BF16 terms, one product (kind::f16).  TF32: the IFs
// and the coefficients each as a TF32 value plus its FP32 remainder, three
// products (kind::tf32), FP32 accuracy.  Both stage 128-byte swizzled rows.
template <bool TF32>
struct TcKind {
  static constexpr int kElem = TF32 ? 4 : 2;     // bytes per operand element
  static constexpr int kBK = 128 / kElem;       // K per stage: one 128-byte swizzle row
  static constexpr int kUK = TF32 ? 8 : 16;      // K of one MMA
  static constexpr int kStages = TF32 ? 3 : 4;
  static constexpr int kAPlanes = TF32 ? 2 : 1;  // A: values (then remainders)
  // instruction descriptor: F32 accumulator, A and B of format BF16 (1) or
  // TF32 (2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  static __host__ __device__ constexpr uint32_t idesc(int m, int n) {
    return (1u << 4) | ((TF32 ? 2u : 1u) << 7) | ((TF32 ? 2u : 1u) << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
  }
};

template <bool TF32>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    uint32_t accumulate) {
  if constexpr (TF32) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

template <int BN, bool TF32>
constexpr size_t tc_smem_bytes() {
  using K = TcKind<TF32>;
  return 1024 + (size_t)K::kStages * (K::kAPlanes * kBM + 2 * BN) * K::kBK * K::kElem + 256;
}

// Persistent GEMM over the 128 x BN output tiles; tma_a_lo is read by the
// TF32 form only (the BF16 form is given tma_a twice).
template <int BN, bool TF32>
__global__ void __launch_bounds__(kThreads, 1)
    dm_tc_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_a_lo,
                 const __grid_constant__ CUtensorMap tma_b, TcParams p) {
  using K = TcKind<TF32>;
  constexpr int NC = 2 * BN;                     // accumulator columns of a tile: hi products, then lo products
  constexpr uint32_t kTmemCols = 2 * NC;         // two accumulators (a power of two, <= 512)
  constexpr int A_BYTES = kBM * K::kBK * K::kElem;
  constexpr int B_BYTES = 2 * BN * K::kBK * K::kElem;  // hi rows, then lo rows: one 2*BN-row operand
  constexpr int B_HALF = BN * K::kBK * K::kElem;
  constexpr int S_BYTES = K::kAPlanes * A_BYTES + B_BYTES;
  constexpr int kStages = K::kStages;
  static_assert(NC <= 256 && kTmemCols <= 512, "tile too wide for one MMA or for TMEM");
  static_assert(S_BYTES % 1024 == 0, "stages must keep the 1024-byte swizzle alignment");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * S_BYTES);
  uint64_t* empty = full + kStages;
  uint64_t* tfull = empty + kStages;   // [2] accumulator ready for the epilogue
  uint64_t* tempty = tfull + 2;        // [2] accumulator read back, free for the next tile
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // Tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...; t = pixel tile * tiles_n
  // + batch tile, so the CTAs that share one 128-pixel IF tile run together
  // and the tile is read from HBM once, then from L2.
  int issued = 0;  // loads issued by the producer (warp 0, lane 0)
  if (warp == 0 && lane == 0) {
    // TMA producer, one ring over all tiles of the CTA
    int it = 0;
    for (int t = blockIdx.x; t < p.tiles; t += gridDim.x) {
      const int m0 = (t / p.tiles_n) * kBM, n0 = (t % p.tiles_n) * BN;
      bool ok = true;
      for (int kb = 0; kb < p.nk; kb++, it++) {
        const int s = it % kStages;
        if (!wait_or_abort(&empty[s], ((it / kStages) & 1) ^ 1, p.err, 1)) {
          ok = false;
          break;
        }
        issued = it + 1;
        unsigned char* st = smem + s * S_BYTES;
        mbar_expect_tx(&full[s], S_BYTES);
        tma_load_2d(st, &tma_a, &full[s], kb * K::kBK, m0);
        if constexpr (TF32) tma_load_2d(st + A_BYTES, &tma_a_lo, &full[s], kb * K::kBK, m0);
        unsigned char* sb = st + K::kAPlanes * A_BYTES;
        tma_load_2d(sb, &tma_b, &full[s], kb * K::kBK, n0);
        tma_load_2d(sb + B_HALF, &tma_b, &full[s], kb * K::kBK, p.batch_pad + n0);
      }
      if (!ok) break;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: per K step one MMA of N = 2*BN (A times the hi and the lo
    // coefficient rows); the TF32 form adds the remainder of A times the hi
    // rows (N = BN) into the first half
    constexpr uint32_t idesc2 = K::idesc(kBM, NC), idesc1 = K::idesc(kBM, BN);
    int it = 0, local = 0;
    for (int t = blockIdx.x; t < p.tiles; t += gridDim.x, local++) {
      const int acc = local & 1;
      if (!wait_or_abort(&tempty[acc], ((local >> 1) & 1) ^ 1, p.err, 2)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + (uint32_t)(acc * NC);
      bool ok = true;
      for (int kb = 0; kb < p.nk; kb++, it++) {
        const int s = it % kStages;
        if (!wait_or_abort(&full[s], (it / kStages) & 1, p.err, 3)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(smem + s * S_BYTES), b0 = a0 + K::kAPlanes * A_BYTES;
#pragma unroll
        for (int k = 0; k < K::kBK / K::kUK; k++) {
          const uint64_t bd = sw128_desc(b0 + k * K::kUK * K::kElem);
          mma<TF32>(d, sw128_desc(a0 + k * K::kUK * K::kElem), bd, idesc2, (kb | k) ? 1u : 0u);
          if constexpr (TF32) mma<TF32>(d, sw128_desc(a0 + A_BYTES + k * K::kUK * K::kElem), bd, idesc1, 1u);
        }
        mma_commit(&empty[s]);
      }
      if (!ok) break;
      mma_commit(&tfull[acc]);
    }
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes (pixels) 32 (w % 4) .. 32 (w % 4) + 31
    const int q = warp & 3;
    int local = 0;
    for (int t = blockIdx.x; t < p.tiles; t += gridDim.x, local++) {
      const int acc = local & 1;
      const bool ok = wait_or_abort(&tfull[acc], (local >> 1) & 1, p.err, 4);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int m0 = (t / p.tiles_n) * kBM, n0 = (t % p.tiles_n) * BN;
      const int pix = m0 + q * 32 + lane;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * NC);
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 16) {
        uint32_t hi[16], lo[16];
        tmem_ld16(taddr + (uint32_t)c0, hi);
        tmem_ld16(taddr + (uint32_t)(BN + c0), lo);
        tmem_ld_wait();
        if (pix < p.n_pix) {
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const int b = n0 + c0 + j;
            if (b < p.batch) {
              const size_t o = (size_t)b * p.n_pix + pix;
              const float v = __uint_as_float(hi[j]) + __uint_as_float(lo[j]);
              p.out[o] = v * p.scale + (p.base ? p.base[o] : 0.f);
            }
          }
        }
      }
      // this warp's reads of the accumulator are done: the MMA may overwrite it
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
  }
  __syncwarp();
  if (warp == 0 && lane == 0 && *(volatile int*)p.err != 0) {
    // an error stopped the CTA: give each stage's last issued load a
    // bounded chance to land before the CTA's shared memory is released
    for (int kb = issued - 1; kb >= 0 && kb >= issued - kStages; kb--)
      tma::mbar_wait(&full[kb % kStages], (kb / kStages) & 1, nullptr, 0);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// coefs [n_act][batch] f32 -> [2][batch_pad][n_act_pad] bf16 (hi, lo), zero padded
__global__ void dm_coefs_to_bf16(const float* __restrict__ coefs, int n_act, int batch, int n_act_pad,
                                 int batch_pad, __nv_bfloat16* __restrict__ out) {
  const size_t plane = (size_t)batch_pad * n_act_pad;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const int b = (int)(i / n_act_pad), a = (int)(i % n_act_pad);
  const float c = (a < n_act && b < batch) ? coefs[(size_t)a * batch + b] : 0.f;
  const __nv_bfloat16 hi = __float2bfloat16_rn(c);
  out[i] = hi;
  out[plane + i] = __float2bfloat16_rn(c - __bfloat162float(hi));
}

// Small batches (a closed-loop step): the tensor-core tile would be mostly
// padding, so the projection is a streaming GEMV over the BF16 IF rows with
// the FP32 coefficients held in shared memory.  One warp per pixel row at a
// time (8 rows per warp, two in flight); each lane loads 16 bytes (8 BF16) per
// step.  Bound by the HBM read of the IF matrix.
constexpr int kGemvMaxBatch = 4;
constexpr int kGemvRowsPerWarp = 8;

template <int B>
__global__ void __launch_bounds__(256) dm_gemv_bf16(const __nv_bfloat16* __restrict__ modes, int n_act_pad,
                                                    const float* __restrict__ coefs, int n_act, int n_pix,
                                                    float scale, const float* __restrict__ base,
                                                    float* __restrict__ opd) {
  extern __shared__ float cs[];  // [B][n_act_pad], zero padded
  for (int i = threadIdx.x; i < B * n_act_pad; i += blockDim.x) {
    const int b = i / n_act_pad, a = i - (i / n_act_pad) * n_act_pad;
    cs[i] = a < n_act ? coefs[(size_t)a * B + b] : 0.f;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = (blockIdx.x * (blockDim.x >> 5) + warp) * kGemvRowsPerWarp;
  const int steps = n_act_pad / 256;  // n_act_pad is a multiple of 64; the tail is handled below
  for (int rr = 0; rr < kGemvRowsPerWarp; rr += 2) {
    const int p0 = row0 + rr, p1 = row0 + rr + 1;
    if (p0 >= n_pix) break;
    const bool has1 = p1 < n_pix;
    const uint4* m0 = reinterpret_cast<const uint4*>(modes + (size_t)p0 * n_act_pad);
    const uint4* m1 = reinterpret_cast<const uint4*>(modes + (size_t)(has1 ? p1 : p0) * n_act_pad);
    float acc0[B], acc1[B];
#pragma unroll
    for (int b = 0; b < B; b++) acc0[b] = acc1[b] = 0.f;
    auto accumulate = [&](uint4 w0, uint4 w1, int a0) {
      const __nv_bfloat162* h0 = reinterpret_cast<const __nv_bfloat162*>(&w0);
      const __nv_bfloat162* h1 = reinterpret_cast<const __nv_bfloat162*>(&w1);
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const float2 f0 = __bfloat1622float2(h0[e]);
        const float2 f1 = __bfloat1622float2(h1[e]);
#pragma unroll
        for (int b = 0; b < B; b++) {
          const float c0 = cs[b * n_act_pad + a0 + 2 * e], c1 = cs[b * n_act_pad + a0 + 2 * e + 1];
          acc0[b] = fmaf(f0.x, c0, fmaf(f0.y, c1, acc0[b]));
          acc1[b] = fmaf(f1.x, c0, fmaf(f1.y, c1, acc1[b]));
        }
      }
    };
    for (int st = 0; st < steps; st++) {
      const int q = st * 32 + lane;  // 16-byte chunk index
      accumulate(m0[q], m1[q], q * 8);
    }
    {
      const int q = steps * 32 + lane;
      if (q * 8 < n_act_pad) accumulate(m0[q], m1[q], q * 8);
    }
#pragma unroll
    for (int b = 0; b < B; b++) {
      float v0 = acc0[b], v1 = acc1[b];
      for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_xor_sync(0xffffffffu, v0, o);
        v1 += __shfl_xor_sync(0xffffffffu, v1, o);
      }
      if (lane == 0) {
        const size_t o0 = (size_t)b * n_pix + p0;
        opd[o0] = scale * v0 + (base ? base[o0] : 0.f);
        if (has1) {
          const size_t o1 = (size_t)b * n_pix + p1;
          opd[o1] = scale * v1 + (base ? base[o1] : 0.f);
        }
      }
    }
  }
}

template <int B>
cudaError_t launch_gemv(const void* modes, int n_act_pad, const float* coefs, int n_act, int n_pix, float scale,
                        const float* base, float* opd, cudaStream_t st) {
  const size_t smem = sizeof(float) * B * (size_t)n_act_pad;
  cudaError_t e = cudaFuncSetAttribute(dm_gemv_bf16<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int rows_per_cta = 8 * kGemvRowsPerWarp;
  dm_gemv_bf16<B><<<ceil_div(n_pix, rows_per_cta), 256, smem, st>>>(
      reinterpret_cast<const __nv_bfloat16*>(modes), n_act_pad, coefs, n_act, n_pix, scale, base, opd);
  return cudaGetLastError();
}

// modes_t [n_act][n_pix] f32 -> modes [n_pix][n_act_pad] bf16, zero padded
__global__ void dm_modes_to_bf16(const float* __restrict__ modes_t, int n_act, int n_pix, int n_act_pad,
                                 __nv_bfloat16* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n_pix * n_act_pad) return;
  const int p = (int)(i / n_act_pad), a = (int)(i % n_act_pad);
  out[i] = __float2bfloat16_rn(a < n_act ? modes_t[(size_t)a * n_pix + p] : 0.f);
}

int encode_2d(CUtensorMap* map, const void* base, uint64_t inner, uint64_t rows, uint32_t box_inner,
              uint32_t box_rows, CUtensorMapDataType dtype = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, uint64_t elem = 2) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tma::encode_fn();
  if (!fn) {
    oopao_set_last_error("cuTensorMapEncodeTiled is not available from the driver", __FILE__, __LINE__);
    return OOPAO_ERR_CUDA;
  }
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {inner * elem};
  const cuuint32_t box[2] = {box_inner, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    oopao_set_last_error("cuTensorMapEncodeTiled rejected the tensor map", __FILE__, __LINE__);
    return OOPAO_ERR_INVALID;
  }
  return OOPAO_OK;
}

template <int BN>
int launch_tc(const void* modes, const void* coefs_t, int n_pix, int n_act_pad, int batch, int batch_pad,
              float scale, const float* base, float* out, int* err, cudaStream_t st) {
  CUtensorMap ta, tb;
  int s = encode_2d(&ta, modes, (uint64_t)n_act_pad, (uint64_t)n_pix, kBK, kBM);
  if (s) return s;
  s = encode_2d(&tb, coefs_t, (uint64_t)n_act_pad, (uint64_t)(2 * batch_pad), kBK, BN);
  if (s) return s;
  const size_t smem = tc_smem_bytes<BN, false>();
  OOPAO_CUDA_TRY(cudaFuncSetAttribute(dm_tc_kernel<BN, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const int tiles_n = batch_pad / BN, tiles = tiles_n * ceil_div(n_pix, kBM);
  int dev = 0, sms = 0;
  OOPAO_CUDA_TRY(cudaGetDevice(&dev));
  OOPAO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  TcParams p{n_pix, batch, n_act_pad / kBK, batch_pad, tiles_n, tiles, scale, base, out, err};
  dm_tc_kernel<BN, false><<<std::min(tiles, sms), kThreads, smem, st>>>(ta, ta, tb, p);
  return OOPAO_OK;
}


// ---- FP32-accuracy projection on the tensor cores: kind::tf32, three products ----
// The IFs and the coefficients are each split into a TF32 part and its FP32
// remainder, x = hi + lo with hi = tf32(x) (round to nearest) and lo = x - hi
// (exact).  A*B = Ahi*Bhi + Ahi*Blo + Alo*Bhi + Alo*Blo; the last term is
// ~2^-22 of the product and is dropped, the other three accumulate in FP32,
// and lo itself enters the MMA at TF32 precision, another ~2^-22.  Per K step
// one MMA of N = 2*BN multiplies Ahi by [Bhi; Blo] into both halves of the
// accumulator and a second of N = BN adds Alo*Bhi to the hi half; the rest is
// the persistent pipeline of dm_tc_kernel with FP32 tiles (32 per 128-byte row).
constexpr int kBK3 = TcKind<true>::kBK;  // FP32 actuators per stage (n_act_pad granularity)

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// modes_t [n_act][n_pix] f32 -> [2][n_pix][n_act_pad] f32 (tf32 hi, remainder), zero padded
__global__ void dm_modes_to_tf32x2(const float* __restrict__ modes_t, int n_act, int n_pix, int n_act_pad,
                                   float* __restrict__ out) {
  const size_t plane = (size_t)n_pix * n_act_pad;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const int px = (int)(i / n_act_pad), a = (int)(i % n_act_pad);
  const float x = a < n_act ? modes_t[(size_t)a * n_pix + px] : 0.f;
  const float h = to_tf32(x);
  out[i] = h;
  out[plane + i] = x - h;
}

// coefs [n_act][batch] f32 -> [2][batch_pad][n_act_pad] f32 (tf32 hi, remainder), zero padded
__global__ void dm_coefs_to_tf32x2(const float* __restrict__ coefs, int n_act, int batch, int n_act_pad,
                                   int batch_pad, float* __restrict__ out) {
  const size_t plane = (size_t)batch_pad * n_act_pad;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const int b = (int)(i / n_act_pad), a = (int)(i % n_act_pad);
  const float c = (a < n_act && b < batch) ? coefs[(size_t)a * batch + b] : 0.f;
  const float h = to_tf32(c);
  out[i] = h;
  out[plane + i] = c - h;
}

template <int BN>
int launch_tc3(const float* modes2, const float* coefs2, int n_pix, int n_act_pad, int batch, int batch_pad,
               float scale, const float* base, float* out, int* err, cudaStream_t st) {
  CUtensorMap tah, tal, tb;
  const size_t plane = (size_t)n_pix * n_act_pad;
  int s = encode_2d(&tah, modes2, (uint64_t)n_act_pad, (uint64_t)n_pix, kBK3, kBM, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4);
  if (s) return s;
  s = encode_2d(&tal, modes2 + plane, (uint64_t)n_act_pad, (uint64_t)n_pix, kBK3, kBM, CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                4);
  if (s) return s;
  s = encode_2d(&tb, coefs2, (uint64_t)n_act_pad, (uint64_t)(2 * batch_pad), kBK3, BN, CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                4);
  if (s) return s;
  const size_t smem = tc_smem_bytes<BN, true>();
  OOPAO_CUDA_TRY(cudaFuncSetAttribute(dm_tc_kernel<BN, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  const int tiles_n = batch_pad / BN, tiles = tiles_n * ceil_div(n_pix, kBM);
  int dev = 0, sms = 0;
  OOPAO_CUDA_TRY(cudaGetDevice(&dev));
  OOPAO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  TcParams p{n_pix, batch, n_act_pad / kBK3, batch_pad, tiles_n, tiles, scale, base, out, err};
  dm_tc_kernel<BN, true><<<std::min(tiles, sms), kThreads, smem, st>>>(tah, tal, tb, p);
  return OOPAO_OK;
}

}  // namespace

extern "C" int oopao_dm_modes_bf16(const float* modes_t, int n_act, int n_pix, int n_act_pad, void* out,
                                   void* stream) {
  OOPAO_CHECK_ARG(modes_t && out, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && n_act_pad >= n_act && n_act_pad % kBK == 0,
                  "n_act_pad must be a multiple of 64 and >= n_act");
  const size_t total = (size_t)n_pix * n_act_pad;
  dm_modes_to_bf16<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      modes_t, n_act, n_pix, n_act_pad, reinterpret_cast<__nv_bfloat16*>(out));
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" size_t oopao_dm_bf16_workspace_bytes(int n_act_pad, int batch) {
  if (n_act_pad <= 0 || batch <= 0) return 0;
  // padded to the larger tile, so that either tile width fits
  const size_t batch_pad = (size_t)ceil_div(batch, 128) * 128;
  return 256 + 2 * batch_pad * n_act_pad * 2;
}

extern "C" int oopao_dm_opd_bf16(const void* modes, int n_act_pad, const float* coefs, int n_act, int n_pix,
                                 int batch, float scale, const float* base, float* opd, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  return oopao_dm_opd_bf16_tiled(modes, n_act_pad, coefs, n_act, n_pix, batch, scale, base, opd, workspace,
                                 workspace_bytes, 0, stream);
}

extern "C" int oopao_dm_opd_bf16_tiled(const void* modes, int n_act_pad, const float* coefs, int n_act, int n_pix,
                                       int batch, float scale, const float* base, float* opd, void* workspace,
                                       size_t workspace_bytes, int tile_n, void* stream) {
  OOPAO_CHECK_ARG(tile_n == 0 || tile_n == 64 || tile_n == 128, "tile_n must be 0 (automatic), 64 or 128");
  OOPAO_CHECK_ARG(modes && coefs && opd && workspace, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && batch > 0, "sizes must be positive");
  OOPAO_CHECK_ARG(n_act_pad >= n_act && n_act_pad % kBK == 0, "n_act_pad must be a multiple of 64 and >= n_act");
  OOPAO_CHECK_ARG(((uintptr_t)modes & 15) == 0 && ((uintptr_t)workspace & 255) == 0,
                  "modes must be 16-byte and the workspace 256-byte aligned");
  OOPAO_CHECK_ARG(workspace_bytes >= oopao_dm_bf16_workspace_bytes(n_act_pad, batch), "workspace too small");
  OOPAO_CHECK_ARG(ceil_div(n_pix, kBM) <= 65535, "n_pix above 65535 * 128");
  cudaStream_t st = (cudaStream_t)stream;
  if (batch <= kGemvMaxBatch && tile_n == 0) {
    OOPAO_CHECK_ARG((size_t)batch * n_act_pad * sizeof(float) <= 200 * 1024, "n_act_pad too large for the GEMV form");
    OOPAO_CUDA_TRY(cudaMemsetAsync(workspace, 0, sizeof(int), st));
    cudaError_t e = cudaSuccess;
    switch (batch) {
      case 1: e = launch_gemv<1>(modes, n_act_pad, coefs, n_act, n_pix, scale, base, opd, st); break;
      case 2: e = launch_gemv<2>(modes, n_act_pad, coefs, n_act, n_pix, scale, base, opd, st); break;
      case 3: e = launch_gemv<3>(modes, n_act_pad, coefs, n_act, n_pix, scale, base, opd, st); break;
      default: e = launch_gemv<4>(modes, n_act_pad, coefs, n_act, n_pix, scale, base, opd, st); break;
    }
    if (e != cudaSuccess) {
      oopao_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
      return OOPAO_ERR_CUDA;
    }
    oopao_count_launches(1);
    return OOPAO_OK;
  }
  const int bn = tile_n ? tile_n : (batch <= 64 ? 64 : 128);
  const int batch_pad = ceil_div(batch, bn) * bn;
  int* err = reinterpret_cast<int*>(workspace);
  __nv_bfloat16* ct = reinterpret_cast<__nv_bfloat16*>((char*)workspace + 256);
  OOPAO_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  const size_t total = (size_t)batch_pad * n_act_pad;
  dm_coefs_to_bf16<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(coefs, n_act, batch, n_act_pad, batch_pad, ct);
  const int s = bn == 64 ? launch_tc<64>(modes, ct, n_pix, n_act_pad, batch, batch_pad, scale, base, opd, err, st)
                         : launch_tc<128>(modes, ct, n_pix, n_act_pad, batch, batch_pad, scale, base, opd, err, st);
  if (s) return s;
  oopao_count_launches(2);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" int oopao_dm_modes_tf32x2(const float* modes_t, int n_act, int n_pix, int n_act_pad, float* out,
                                     void* stream) {
  OOPAO_CHECK_ARG(modes_t && out, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && n_act_pad >= n_act && n_act_pad % kBK3 == 0,
                  "n_act_pad must be a multiple of 32 and >= n_act");
  const size_t total = (size_t)n_pix * n_act_pad;
  dm_modes_to_tf32x2<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(modes_t, n_act, n_pix,
                                                                                           n_act_pad, out);
  oopao_count_launches(1);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}

extern "C" size_t oopao_dm_tf32_workspace_bytes(int n_act_pad, int batch) {
  if (n_act_pad <= 0 || batch <= 0) return 0;
  const size_t batch_pad = (size_t)ceil_div(batch, 128) * 128;
  return 256 + 2 * batch_pad * n_act_pad * 4;
}

extern "C" int oopao_dm_opd_tf32x3(const float* modes2, int n_act_pad, const float* coefs, int n_act, int n_pix,
                                   int batch, float scale, const float* base, float* opd, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  OOPAO_CHECK_ARG(modes2 && coefs && opd && workspace, "NULL argument");
  OOPAO_CHECK_ARG(n_act > 0 && n_pix > 0 && batch > 0, "sizes must be positive");
  OOPAO_CHECK_ARG(n_act_pad >= n_act && n_act_pad % kBK3 == 0, "n_act_pad must be a multiple of 32 and >= n_act");
  OOPAO_CHECK_ARG(((uintptr_t)modes2 & 15) == 0 && ((uintptr_t)workspace & 255) == 0,
                  "modes must be 16-byte and the workspace 256-byte aligned");
  OOPAO_CHECK_ARG(workspace_bytes >= oopao_dm_tf32_workspace_bytes(n_act_pad, batch), "workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  const int bn = batch <= 64 ? 64 : 128;
  const int batch_pad = ceil_div(batch, bn) * bn;
  int* err = reinterpret_cast<int*>(workspace);
  float* ct = reinterpret_cast<float*>((char*)workspace + 256);
  OOPAO_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  const size_t total = (size_t)batch_pad * n_act_pad;
  dm_coefs_to_tf32x2<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(coefs, n_act, batch, n_act_pad, batch_pad, ct);
  const int s = bn == 64 ? launch_tc3<64>(modes2, ct, n_pix, n_act_pad, batch, batch_pad, scale, base, opd, err, st)
                         : launch_tc3<128>(modes2, ct, n_pix, n_act_pad, batch, batch_pad, scale, base, opd, err, st);
  if (s) return s;
  oopao_count_launches(2);
  OOPAO_CUDA_TRY(cudaGetLastError());
  return OOPAO_OK;
}
