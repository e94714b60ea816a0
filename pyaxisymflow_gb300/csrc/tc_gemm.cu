// tcgen05 3xTF32 GEMM: kernel and host helpers (see tc_gemm.cuh).
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "tc_gemm.cuh"

namespace axi_tc {
namespace {

using axi_tma::globaltimer;
using axi_tma::mbar_expect_tx;
using axi_tma::mbar_init;
using axi_tma::mbar_try_wait;
using axi_tma::mbar_wait;
using axi_tma::smem_u32;
using axi_tma::tma_load_2d;

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D(tmem) (+)= A(smem desc) * B(smem desc), kind::tf32, FP32 accumulate.
__device__ __forceinline__ void umma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with ROW_BYTES-wide rows
// and the matching swizzle (8-row atoms of 8 x ROW_BYTES bytes, consecutive
// atoms 8 x ROW_BYTES apart); layout codes 2 = 128-byte, 4 = 64-byte swizzle.
static_assert(ROW_BYTES == 64 || ROW_BYTES == 128, "tile rows must be 64 or 128 bytes");
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);        // start address >> 4
  d |= static_cast<uint64_t>(1) << 16;                         // leading byte offset (unused)
  d |= static_cast<uint64_t>((8 * ROW_BYTES) >> 4) << 32;      // stride byte offset: 8 rows
  d |= static_cast<uint64_t>(1) << 46;                         // descriptor version
  d |= static_cast<uint64_t>(ROW_BYTES == 128 ? 2 : 4) << 61;  // swizzle mode
  return d;
}

// Instruction descriptor: D = F32, A = B = TF32, both K-major, M = 128, N = 128.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

// TMA store of a 2-D box from shared memory (c0: innermost coordinate,
// 128-byte aligned here) in this thread's bulk group, then committed.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, uint32_t src, int c0,
                                             int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n\t"
      "cp.async.bulk.commit_group;" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(src)
      : "memory");
}
// this thread's bulk stores have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// this thread's bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* m) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Persistent, warp-specialised kernel (one CTA per SM, tiles strided over the
// grid): warp 0 issues TMA, warp 1 issues MMAs into one of two TMEM
// accumulators (2 x 128 columns), warps 2-9 drain the other accumulator, so
// the epilogue of a tile overlaps the main loop of the next one.
__global__ void __launch_bounds__(THREADS, 1)
    tf32x3_gemm_kernel(const TcJob* __restrict__ jobs, const int4* __restrict__ tiles,
                       int n_tiles, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  // epilogue staging first (1024-byte aligned, as the swizzled store boxes
  // need), then the barriers
  float* stage_out = reinterpret_cast<float*>(smem + NSTAGE * STAGE_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * STAGE_BYTES + EPI_STAGE_BYTES);
  // full[NSTAGE], empty[NSTAGE], acc_full[2], acc_empty[2], quiet
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * NSTAGE + 5);
  int* progress = reinterpret_cast<int*>(tmem_slot + 1);  // [0] loads issued, [1] consumed
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + NSTAGE);
  const uint32_t accf0 = smem_u32(bars + 2 * NSTAGE), acce0 = smem_u32(bars + 2 * NSTAGE + 2);
  const uint32_t quiet = smem_u32(bars + 2 * NSTAGE + 4);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, EPI_WARPS);
    }
    mbar_init(quiet, 1);
    progress[0] = 0;
    progress[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(tmem_slot), 2 * BN);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: one continuous ring over all tiles of this CTA ----
      int g = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const int4 tr = tiles[t];
        const TcJob& job = jobs[tr.x];  // only the tensor maps' addresses are used
        const int nk = tr.w;
        if (t + (int)gridDim.x < n_tiles) {
          // the next tile's four tensor maps, fetched while this tile loads
          const TcJob& nj = jobs[tiles[t + gridDim.x].x];
          prefetch_tensormap(&nj.a_hi);
          prefetch_tensormap(&nj.a_lo);
          prefetch_tensormap(&nj.b_hi);
          prefetch_tensormap(&nj.b_lo);
        }
        for (int kb = 0; kb < nk; ++kb, ++g) {
          const int s = g % NSTAGE, use = g / NSTAGE;
          if (use > 0 && !mbar_wait(empty0 + 8 * s, (use - 1) & 1, err, ERR_PRODUCER)) {
            ok = false;
            break;
          }
          const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t fb = full0 + 8 * s;
          mbar_expect_tx(fb, STAGE_BYTES);
          const int kx = kb * BKF;
          tma_load_2d(st + 0 * TILE_BYTES, &job.a_hi, kx, tr.y, fb);
          tma_load_2d(st + 1 * TILE_BYTES, &job.a_lo, kx, tr.y, fb);
          tma_load_2d(st + 2 * TILE_BYTES, &job.b_hi, kx, tr.z, fb);
          tma_load_2d(st + 3 * TILE_BYTES, &job.b_lo, kx, tr.z, fb);
        }
      }
      progress[0] = g;
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      constexpr uint32_t idesc = idesc_tf32(BM, BN);
      int g = 0, it = 0;
      bool ok = true;
      // k-block count of the next tile, loaded one tile ahead (its latency
      // would otherwise sit between two tiles' MMAs)
      int nk_next = blockIdx.x < n_tiles ? tiles[blockIdx.x].w : 0;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++it) {
        const int nk = nk_next;
        if (t + (int)gridDim.x < n_tiles) nk_next = tiles[t + gridDim.x].w;
        const int buf = it & 1, ause = it >> 1;
        if (ause > 0 && !mbar_wait(acce0 + 8 * buf, (ause - 1) & 1, err, ERR_MMA)) break;
        tc_fence_after();
        const uint32_t d = tmem + buf * BN;
        for (int kb = 0; kb < nk; ++kb, ++g) {
          const int s = g % NSTAGE, use = g / NSTAGE;
          if (!mbar_wait(full0 + 8 * s, use & 1, err, ERR_MMA)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
          const uint64_t ah = sw_desc(st), al = sw_desc(st + TILE_BYTES);
          const uint64_t bh = sw_desc(st + 2 * TILE_BYTES), bl = sw_desc(st + 3 * TILE_BYTES);
#pragma unroll
          for (int kk = 0; kk < BKF / 8; ++kk) {
            const uint64_t o = static_cast<uint64_t>(kk * 32) >> 4;  // 8 TF32 = 32 bytes
            umma_tf32(d, ah + o, bh + o, idesc, (kb | kk) != 0 ? 1u : 0u);
            umma_tf32(d, ah + o, bl + o, idesc, 1u);
            umma_tf32(d, al + o, bh + o, idesc, 1u);
          }
          umma_commit(empty0 + 8 * s);
        }
        if (ok) umma_commit(accf0 + 8 * buf);
      }
      progress[1] = g;
      // every MMA of this CTA has completed once `quiet` fires
      umma_commit(quiet);
      mbar_wait(quiet, 0, err, ERR_MMA);
    }
    __syncwarp();
  } else {
    // ---- epilogue warps 2..9: TMEM lane quarter = warp % 4, column half ----
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    constexpr int CHUNKS = BN / 32 / 2;  // 32-column chunks per warp
    float* stg = stage_out + (warp - 2) * 32 * 33;
    int it = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++it) {
      const int4 tr = tiles[t];
      const TcJob& job = jobs[tr.x];
      // the job's fields in registers for the whole tile, loaded while the
      // accumulator is still being computed (read through the reference
      // inside the store loop, each store could alias them and forced a
      // reload per row)
      float* const c = job.c;
      float* const c_lo = job.c_lo;
      const float* const scl = job.scale;
      const int M = job.M, Nc = job.N, ldc = job.ldc, mode = job.mode;
      const bool tma_out = job.c_tma != 0;
      const CUtensorMap* const cmap = &job.c_map;
      const int buf = it & 1;
      const bool ok = mbar_wait(accf0 + 8 * buf, (it >> 1) & 1, err, ERR_EPILOGUE);
      // all lanes leave together; a failure elsewhere in the grid surfaces at
      // the next wait (the error word is read there) and on the host
      if (!__all_sync(0xffffffffu, ok)) break;
      tc_fence_after();
      const int row0 = tr.y + 32 * q;
      const bool scaled = mode == MODE_SCALE_SPLIT || mode == MODE_SCALE;
      const bool split = mode == MODE_SPLIT || mode == MODE_SCALE_SPLIT;
      const bool pair = mode == MODE_PAIR_ADD;
#pragma unroll 1
      for (int cc = half * CHUNKS; cc < (half + 1) * CHUNKS; ++cc) {
        const int col = tr.z + cc * 32 + lane;
        // the elementwise factors of this 32 x 32 block are fetched before the
        // accumulator is read, all 32 loads in flight at once (one load per
        // row in the store loop left the epilogue waiting on L2 latency)
        float sv[32];
        if (scaled) {
#pragma unroll
          for (int rr = 0; rr < 32; ++rr) {
            const int row = row0 + rr;
            sv[rr] = (col < Nc && row < M) ? __ldg(scl + (long long)row * Nc + col) : 0.0f;
          }
        }
        // the pair the product is added to, likewise in flight before the read
        float ph[32], pl[32];
        if (pair) {
#pragma unroll
          for (int rr = 0; rr < 32; ++rr) {
            const int row = row0 + rr;
            const bool in = col < Nc && row < M;
            const long long idx = (long long)row * ldc + col;
            ph[rr] = in ? c[idx] : 0.0f;
            pl[rr] = in ? c_lo[idx] : 0.0f;
          }
        }
        uint32_t r[32];
        tmem_ld32(tmem + buf * BN + (static_cast<uint32_t>(32 * q) << 16) + cc * 32, r);
        if (tma_out) {
          // the warp's 32 x 32 block as one TMA store: row `lane` of the box,
          // 16-byte chunk c at position c ^ (lane % 8) (128-byte swizzle,
          // conflict-free), after the warp's previous store has read the box
          char* box = reinterpret_cast<char*>(stage_out) + (warp - 2) * 4096;
          if (lane == 0) bulk_wait_read();
          __syncwarp();
#pragma unroll
          for (int c = 0; c < 8; ++c)
            *reinterpret_cast<float4*>(box + lane * 128 + ((c ^ (lane & 7)) << 4)) =
                make_float4(__uint_as_float(r[4 * c]), __uint_as_float(r[4 * c + 1]),
                            __uint_as_float(r[4 * c + 2]), __uint_as_float(r[4 * c + 3]));
          axi_tma::fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) tma_store_2d(cmap, smem_u32(box), tr.z + cc * 32, row0);
          continue;
        }
        // transpose the warp's 32 x 32 block so each store instruction writes
        // 32 consecutive columns of one row
#pragma unroll
        for (int j = 0; j < 32; ++j) stg[lane * 33 + j] = __uint_as_float(r[j]);
        __syncwarp();
        if (col < Nc) {
#pragma unroll
          for (int rr = 0; rr < 32; ++rr) {
            const int row = row0 + rr;
            float v = stg[rr * 33 + lane];
            if (scaled) v *= sv[rr];
            if (row < M) {
              const long long idx = (long long)row * ldc + col;
              if (pair) {
                float hi = ph[rr], lo = pl[rr];
                axi_eft::pair_add(hi, lo, v);
                c[idx] = hi;
                c_lo[idx] = lo;
              } else if (split) {
                float hi, lo;
                tf32_split(v, hi, lo);
                c[idx] = hi;
                c_lo[idx] = lo;
              } else {
                c[idx] = v;
              }
            }
          }
        }
        __syncwarp();
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acce0 + 8 * buf)
                                  : "memory");
    }
    // every TMA store of this warp complete before the block's shared
    // memory goes away
    if (lane == 0) bulk_wait_all();
    __syncwarp();
  }
  __syncthreads();
  if (threadIdx.x == 0 && progress[1] < progress[0]) {
    // a failure left copies in flight: wait for them (bounded) before exiting
    for (int g = progress[1]; g < progress[0]; ++g)
      if (!axi_tma::mbar_wait_drain(full0 + 8 * (g % NSTAGE), (g / NSTAGE) & 1))
        atomicCAS(err, 0, ERR_DRAIN);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, 2 * BN);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(axi_tma::encode_tiled_fn());
}

}  // namespace

int encode_operand(CUtensorMap* map, const float* base, int rows, int K, int ld) {
  auto fn = encode_fn();
  if (!fn) {
    axi::set_error("tensor core GEMM: cuTensorMapEncodeTiled unavailable");
    return AXI_ERR_CUDA;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (ld * 4) % 16 != 0 || ld < K) {
    axi::set_error("tensor core GEMM: operand not 16-byte aligned (ld = %d)", ld);
    return AXI_ERR_INVALID;
  }
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 4};
  const cuuint32_t box[2] = {BKF, BM};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  ROW_BYTES == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    axi::set_error("tensor core GEMM: cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
    return AXI_ERR_CUDA;
  }
  return AXI_OK;
}

bool encode_output(TcJob* job) {
  auto fn = encode_fn();
  if (!fn || job->mode != MODE_PLAIN || (reinterpret_cast<uintptr_t>(job->c) & 15) != 0 ||
      job->ldc % 4 != 0 || job->ldc < job->N)
    return false;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(job->N), static_cast<cuuint64_t>(job->M)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(job->ldc) * 4};
  const cuuint32_t box[2] = {32, 32};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(&job->c_map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, job->c, dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  job->c_tma = 1;
  return true;
}

void order_tiles_by_k(int4* tiles, int n, const TcJob* jobs, bool sort) {
  for (int i = 0; i < n; ++i) tiles[i].w = (jobs[tiles[i].x].K + BKF - 1) / BKF;
  if (!sort) return;
  std::stable_sort(tiles, tiles + n,
                   [jobs](const int4& a, const int4& b) { return jobs[a.x].K > jobs[b.x].K; });
}

int launch(const TcJob* jobs_dev, const int4* tiles_dev, int n_tiles, int* err_dev,
           cudaStream_t s, int ctas_percent) {
  static std::once_flag once;
  static cudaError_t attr_status = cudaSuccess;
  std::call_once(once, [] {
    attr_status = cudaFuncSetAttribute(tf32x3_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  if (attr_status != cudaSuccess) {
    axi::set_error("tensor core GEMM: cannot reserve %d bytes of shared memory", SMEM_BYTES);
    return AXI_ERR_CUDA;
  }
  if (n_tiles <= 0) return AXI_OK;
  int ctas = axi::sm_count();
  if (ctas_percent > 0 && ctas_percent < 100) ctas = ctas * ctas_percent / 100 > 0 ? ctas * ctas_percent / 100 : 1;
  const int grid = n_tiles < ctas ? n_tiles : ctas;
  tf32x3_gemm_kernel<<<grid, THREADS, SMEM_BYTES, s>>>(jobs_dev, tiles_dev, n_tiles, err_dev);
  return axi::launch_status("tf32x3_gemm");
}

}  // namespace axi_tc

namespace axi_tma {

void* encode_tiled_fn() {
  static void* fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = p;
  });
  return fn;
}

int encode_box(CUtensorMap* map, const void* base, int elem_bytes, int rows, int cols,
               int box_rows, int box_cols) {
  auto fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(encode_tiled_fn());
  if (!fn) {
    axi::set_error("tensor map: cuTensorMapEncodeTiled unavailable");
    return AXI_ERR_CUDA;
  }
  if ((elem_bytes != 4 && elem_bytes != 8) || (reinterpret_cast<uintptr_t>(base) & 15) != 0 ||
      ((int64_t)cols * elem_bytes) % 16 != 0 || (box_cols * elem_bytes) % 16 != 0 ||
      box_rows < 1 || box_rows > 256 || box_cols < 1 || box_cols > 256) {
    axi::set_error("tensor map: %d x %d array (box %d x %d) breaks the 16-byte rules", rows, cols,
                   box_rows, box_cols);
    return AXI_ERR_INVALID;
  }
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(cols) * elem_bytes};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_cols), static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                  2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    axi::set_error("tensor map: cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
    return AXI_ERR_CUDA;
  }
  return AXI_OK;
}

}  // namespace axi_tma

// ---------------------------------------------------------------------------
// Standalone entry: C (M, N) = A (M, K) * B (N, K)^T in FP32 via 3xTF32.
// ---------------------------------------------------------------------------
namespace {

__global__ void split_kernel(const float* __restrict__ x, float* __restrict__ hi,
                             float* __restrict__ lo, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) axi_tc::tf32_split(x[k], hi[k], lo[k]);
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct TestLayout {
  size_t a_hi, a_lo, b_hi, b_lo, job, tiles, err, total;
};

TestLayout test_layout(int M, int N, int K) {
  TestLayout L;
  size_t o = 0;
  L.a_hi = o; o = align_up(o + (size_t)M * K * 4, 256);
  L.a_lo = o; o = align_up(o + (size_t)M * K * 4, 256);
  L.b_hi = o; o = align_up(o + (size_t)N * K * 4, 256);
  L.b_lo = o; o = align_up(o + (size_t)N * K * 4, 256);
  L.job = o; o = align_up(o + sizeof(axi_tc::TcJob), 256);
  const size_t nt = (size_t)((M + axi_tc::BM - 1) / axi_tc::BM) * ((N + axi_tc::BN - 1) / axi_tc::BN);
  L.tiles = o; o = align_up(o + nt * sizeof(int4), 256);
  L.err = o; o = align_up(o + 16, 256);
  L.total = o;
  return L;
}

}  // namespace

extern "C" int64_t axi_tf32x3_gemm_work_bytes(int M, int N, int K) {
  return (int64_t)test_layout(M, N, K).total;
}

extern "C" int axi_tf32x3_gemm(float* C, const float* A, const float* B, int M, int N, int K,
                               void* work, void* stream) {
  axi::clear_error();
  const char* what = "tf32x3_gemm";
  if (M <= 0 || N <= 0 || K <= 0 || (K % 4) != 0) {
    axi::set_error("%s: invalid shape M=%d N=%d K=%d (K must be a multiple of 4)", what, M, N, K);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptr(what, work, "work"));
  cudaStream_t s = axi::as_stream(stream);
  const TestLayout L = test_layout(M, N, K);
  char* w = static_cast<char*>(work);
  float* ahi = reinterpret_cast<float*>(w + L.a_hi);
  float* alo = reinterpret_cast<float*>(w + L.a_lo);
  float* bhi = reinterpret_cast<float*>(w + L.b_hi);
  float* blo = reinterpret_cast<float*>(w + L.b_lo);
  split_kernel<<<axi::ceil_div((long long)M * K, 256), 256, 0, s>>>(A, ahi, alo, (long long)M * K);
  split_kernel<<<axi::ceil_div((long long)N * K, 256), 256, 0, s>>>(B, bhi, blo, (long long)N * K);
  AXI_TRY(axi::launch_status(what));
  axi_tc::TcJob job;
  memset(&job, 0, sizeof(job));
  AXI_TRY(axi_tc::encode_operand(&job.a_hi, ahi, M, K, K));
  AXI_TRY(axi_tc::encode_operand(&job.a_lo, alo, M, K, K));
  AXI_TRY(axi_tc::encode_operand(&job.b_hi, bhi, N, K, K));
  AXI_TRY(axi_tc::encode_operand(&job.b_lo, blo, N, K, K));
  job.c = C;
  job.c_lo = nullptr;
  job.scale = nullptr;
  job.M = M;
  job.N = N;
  job.K = K;
  job.ldc = N;
  job.mode = axi_tc::MODE_PLAIN;
  axi_tc::encode_output(&job);  // TMA stores where the output allows them
  std::string tiles;
  for (int m0 = 0; m0 < M; m0 += axi_tc::BM)
    for (int n0 = 0; n0 < N; n0 += axi_tc::BN) {
      int4 t = make_int4(0, m0, n0, (K + axi_tc::BKF - 1) / axi_tc::BKF);
      tiles.append(reinterpret_cast<const char*>(&t), sizeof(t));
    }
  const int n_tiles = (int)(tiles.size() / sizeof(int4));
  if (cudaMemcpyAsync(w + L.job, &job, sizeof(job), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(w + L.tiles, tiles.data(), tiles.size(), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemsetAsync(w + L.err, 0, 16, s) != cudaSuccess)
    return axi::launch_status(what);
  AXI_TRY(axi_tc::launch(reinterpret_cast<const axi_tc::TcJob*>(w + L.job),
                         reinterpret_cast<const int4*>(w + L.tiles), n_tiles,
                         reinterpret_cast<int*>(w + L.err), s));
  int err = 0;
  if (cudaMemcpyAsync(&err, w + L.err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status(what);
  if (err != 0) {
    axi::set_error("%s: a pipeline wait timed out (code %d)", what, err);
    return AXI_ERR_CUDA;
  }
  return AXI_OK;
}
