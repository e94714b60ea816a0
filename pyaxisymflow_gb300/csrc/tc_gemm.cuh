// tcgen05 (5th-generation tensor core) GEMM with FP32-accurate 3xTF32 products.
//
//   C[M, N] = A[M, K] * B[N, K]^T        (both operands K-major, FP32 in HBM)
//
// Each operand is stored as a TF32 "hi" part (x rounded to TF32) and the
// TF32-rounded remainder "lo"; the tensor core accumulates
// hi*hi + hi*lo + lo*hi in FP32 in tensor memory, which restores close to
// FP32 accuracy (the dropped lo*lo term is near FP32 rounding).
//
// Persistent CTAs (one per SM) walk a list of 128 x 128 output tiles:
//   warp 0, one thread   TMA producer: cp.async.bulk.tensor tiles (128 rows x
//                        32 floats, 128-byte swizzle) of A_hi, A_lo, B_hi, B_lo
//                        into a 3-stage shared-memory ring (mbarrier complete_tx),
//                        continuous across tiles
//   warp 1, one thread   MMA issuer: 3 x 4 tcgen05.mma.kind::tf32 per stage into
//                        one of two 128-lane x 128-column FP32 accumulators in
//                        TMEM; tcgen05.commit releases stages and accumulators
//   warps 2-9            epilogue: tcgen05.ld (warp w reads TMEM lanes
//                        32 (w % 4) .., warps 2-5 columns 0-63, warps 6-9
//                        columns 64-127); plain outputs go out as one TMA store
//                        per 32 x 32 block (128-byte swizzled shared-memory
//                        box), the split and scaled forms through a per-warp
//                        shared-memory transpose and row-contiguous stores; it
//                        drains one accumulator while the MMAs fill the other
// Every mbarrier wait is bounded by a 1 s wall-clock limit; on expiry the
// kernel records an error code, drains its outstanding copies (bounded),
// frees its TMEM and returns.
#pragma once

#include <cuda.h>
#include <cstdint>

#include "axi_common.cuh"
#include "tma.cuh"


namespace axi_tc {

constexpr int BM = 128;
constexpr int BN = 128;
// 128 x 128 tiles, 32 K floats (128-byte rows, 128-byte swizzle) per stage,
// 3 stages. Measured alternatives, both slower on the spectral products:
// 16-float stages with a 6-deep ring (64-byte swizzle; twice the barrier and
// copy count per FLOP: 8 tiles of K = 512 per CTA take 107 us against 92 us,
// so the main loop pays a fixed cost per stage rather than waiting on the
// ring) and 128 x 256 tiles with two 96 KB stages (the ring too shallow to
// cover the operand loads).
constexpr int BKF = 32;                         // K floats per stage
constexpr int ROW_BYTES = BKF * 4;              // swizzle span of a tile row
constexpr int NSTAGE = 3;
constexpr int TILE_BYTES = BM * BKF * 4;        // 16 KB per operand tile
constexpr int STAGE_BYTES = 4 * TILE_BYTES;     // A_hi, A_lo, B_hi, B_lo
constexpr int EPI_WARPS = 8;                    // two per TMEM lane quarter
constexpr int THREADS = 32 * (2 + EPI_WARPS);   // TMA warp, MMA warp, 8 epilogue warps
// epilogue staging: a 32 x 33-float transpose per warp, or (TMA stores) a
// 32 x 32-float 128-byte-swizzled box per warp at 4 KB strides
constexpr int EPI_STAGE_BYTES = EPI_WARPS * 32 * 33 * 4;
static_assert(EPI_WARPS * 4096 <= EPI_STAGE_BYTES, "TMA store boxes fit the staging region");
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 1024 + EPI_STAGE_BYTES + 256;

// MODE_PAIR_ADD: the output is the float pair (c, c_lo) holding c + c_lo;
// the product is added to it and the pair renormalised (c the rounded sum,
// c_lo the exact remainder), so repeated additions keep about 48 bits.
enum { MODE_PLAIN = 0, MODE_SPLIT = 1, MODE_SCALE_SPLIT = 2, MODE_SCALE = 3, MODE_PAIR_ADD = 4 };
enum { ERR_PRODUCER = 1, ERR_MMA = 2, ERR_EPILOGUE = 3, ERR_DRAIN = 4 };

// One GEMM problem. Tensor maps are encoded on the host (cuTensorMapEncodeTiled)
// and live in global memory next to the job.
struct TcJob {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;
  CUtensorMap c_map;   // MODE_PLAIN with c_tma: the output in 32 x 32 boxes for TMA stores
  float* c;            // output (MODE_PLAIN) or its hi part
  float* c_lo;         // lo part (split modes; MODE_PAIR_ADD: low part of the pair)
  const float* scale;  // elementwise factor, row-major (M, N) (MODE_SCALE*)
  int M, N, K, ldc;
  int mode;
  int c_tma;           // 1: the epilogue stores tiles through c_map. Every job of
                       // one launch must agree (the two store paths lay out the
                       // epilogue's shared memory differently).
};

// Nearest TF32 value of x (10 explicit mantissa bits, ties away from zero):
// the tensor core ignores the low 13 bits of an operand, so operands are
// rounded before they are stored.
__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// TF32 split: hi = nearest TF32 of x, lo = nearest TF32 of the exact
// remainder x - hi. hi + lo carries about 23 significant bits (truncating
// either part would lose two of them).
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = tf32_round(x);
  lo = tf32_round(x - hi);
}

// Host: encode a 2-D K-major FP32 operand (rows x K, row stride ld floats)
// for 128-row x BKF-float boxes with the ROW_BYTES swizzle. Returns AXI status.
int encode_operand(CUtensorMap* map, const float* base, int rows, int K, int ld);

// Host: encode the output of a MODE_PLAIN job (rows x cols, row stride ld
// floats) for 32 x 32-float TMA stores with the 128-byte swizzle; sets
// job->c_tma. False (job untouched) when the output cannot be stored that way
// (base not 16-byte aligned or ld not a multiple of 4).
bool encode_output(TcJob* job);

// Host: complete a tile table (job, m0, n0, -) with each tile's k-block
// count (w = ceil(K / BKF), which the kernel reads instead of the job) and
// (with `sort`) order it longest main loop (largest K) first, stable within
// equal K. The persistent CTAs take tiles with a fixed stride, so the long
// tiles are spread over all SMs before the short ones.
void order_tiles_by_k(int4* tiles, int n, const TcJob* jobs, bool sort = true);

// Host: launch the grouped kernel over `n_tiles` (job, m0, n0, k-blocks) tiles
// with `ctas_percent` of the SMs as persistent CTAs (0: all of them).
int launch(const TcJob* jobs_dev, const int4* tiles_dev, int n_tiles, int* err_dev,
           cudaStream_t s, int ctas_percent = 0);

}  // namespace axi_tc
