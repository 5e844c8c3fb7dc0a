// Tensor-core contraction on sm_103a: D = A B^T (+ bias) with tcgen05.mma
// kind::tf32 in 3xTF32 form.
//
//   A [M x K], B [N x K] row-major FP32 (K-major operands), each given as a
//   pair (hi, lo) of TF32-representable arrays with x ~= hi + lo;
//   D [M x N] FP32 = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T  (+ bias[n])
// so every product carries ~22 significant bits, accumulated in FP32 in
// tensor memory.  K is consumed in slices of 32 (128 bytes, SWIZZLE_128B)
// through a 3-stage TMA pipeline guarded by mbarriers.
// Every wait is bounded; on timeout the kernel records an error code, skips
// the epilogue, drains its own copies (bounded) and frees tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "tc_util.cuh"

namespace {

constexpr int kBM = 128;
// K slice of one stage: kRowBytes per operand row (the TMA swizzle span), i.e.
// kBK fp32 (2 kBK bf16) elements; smaller slices give more pipeline stages in
// the same shared memory (more copies in flight against the L2 latency).
constexpr int kRowBytes = 128;
constexpr int kBK = kRowBytes / 4;
using namespace smx::tc;

// K-major operand descriptor of this kernel's slices (kRowBytes swizzle)
__device__ __forceinline__ uint64_t make_desc_k(uint32_t saddr) { return make_desc_sw(saddr, kRowBytes); }

// Tiles: 128 x BN outputs per CTA (BN = 128, or 256 for wide products: A is
// then read once per 256 columns and B streams past L2 half as often).  The
// FP32 accumulator of the tensor cores truncates when it adds, so one
// accumulator must not run over long stretches of K: the MMA thread
// alternates between two accumulators in tensor memory (columns [0, BN) and
// [BN, 2 BN)) every few K-tiles, and the drain warps add each finished
// accumulator into FP32 registers, then release it.  Drain warp w reads the
// TMEM lane quadrant w % 4 (rows 32 (w % 4) .. +31) and columns 128 (w / 4) ..
// +127: one row of 128 outputs per thread.
// K-tiles per accumulator use: 64 products for the 3xTF32 form (its error
// bound), 256 for the split-BF16 form, whose error the 16-bit split sets
constexpr int kChunkTf32 = 64 / kBK;
constexpr int kChunkBf16 = 256 / (2 * kBK);

template <int BN>
struct Tile {
  static constexpr int kN = BN;
  static constexpr int kDrainWarps = 4 * (BN / 128);
  static constexpr int kWarpTMA = kDrainWarps, kWarpMMA = kDrainWarps + 1;
  static constexpr int kThreads = 32 * (kDrainWarps + 2);
  static constexpr int kStages = BN == 128 ? 3 : 2;  // 64 KB or 96 KB stages in ~192 KB
  static constexpr int kA = kBM * kBK * 4;
  static constexpr int kB = BN * kBK * 4;
  static constexpr int kStage = 2 * kA + 2 * kB;
  static constexpr int kTiles = kStages * kStage;
  static constexpr int kTotal = kTiles + 1024 /*align*/ + 256 /*barriers*/;
};

struct GemmArgs {
  int M, N, K;
  float* D;
  int64_t ldd;
  const float* bias;
  int* err;
  int accumulate;   // D += A B^T instead of D = A B^T
  int kt_per_z;     // split-K: K-tiles per blockIdx.z slice (0: one slice)
  int64_t zstride;  // split-K: floats between the slices' outputs
  uint64_t wait_ns; // bound on each pipeline wait (kWaitNs; shorter only in the self-test)
  int no_loads;     // self-test only: the producer issues no copies, so the first wait must time out
};

constexpr int kEpiLd = 132;  // epilogue staging row stride (floats): 16-byte rows, conflict-free
static_assert(Tile<128>::kDrainWarps * 32 * kEpiLd * 4 <= Tile<128>::kTiles, "epilogue staging must fit");
static_assert(Tile<256>::kDrainWarps * 32 * kEpiLd * 4 <= Tile<256>::kTiles, "epilogue staging must fit");

// BF16 = false: kind::tf32 on FP32 operands (32 per 128-byte slice); true:
// kind::f16 on BF16 operands (64 per slice).  Same slices, stages and MMAs.
template <bool BF16, int BN>
__global__ void __launch_bounds__(Tile<BN>::kThreads, 1)
    gemm_tf32x3_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                       const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl, GemmArgs g) {
  constexpr int EK = BF16 ? 2 * kBK : kBK;  // elements per K-tile
  constexpr int kChunk = BF16 ? kChunkBf16 : kChunkTf32;
  using L = Tile<BN>;
  constexpr int kBN = BN;
  constexpr int kStages = L::kStages;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + L::kTiles);
  uint64_t* empty = full + kStages;
  uint64_t* acc_full = empty + kStages;  // [2] MMA -> drain
  uint64_t* acc_empty = acc_full + 2;    // [2] drain -> MMA
  uint64_t* flush = acc_empty + 2;       // MMA thread, on failure: its own MMAs complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(flush + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* armed_slot = abort_flag + 1;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int KT_all = (g.K + EK - 1) / EK;
  const int kt_base = g.kt_per_z ? int(blockIdx.z) * g.kt_per_z : 0;
  const int KT = g.kt_per_z ? min(KT_all - kt_base, g.kt_per_z) : KT_all;  // >= 1 (host)
  const int NCH = (KT + kChunk - 1) / kChunk;
  float* const D = g.D + int64_t(blockIdx.z) * g.zstride;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], L::kDrainWarps);  // one arrival per drain warp
    }
    mbar_init(flush, 1);
    *abort_flag = 0;
    *armed_slot = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // tensor memory: two accumulators of 128 fp32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * kBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == L::kWarpTMA) {
    if (lane == 0) {  // ---- TMA producer
      int armed_upto = 0;
      for (int kt = 0; kt < (g.no_loads ? 0 : KT); ++kt) {
        const int s = kt % kStages;
        const uint32_t ph = (kt / kStages) & 1;
        if (kt >= kStages && !mbar_wait(&empty[s], ph ^ 1, abort_flag, g.wait_ns)) {
          atomicExch(g.err, 1);
          *abort_flag = 1;
          break;
        }
        uint8_t* st = base + s * L::kStage;
        mbar_expect_tx(&full[s], L::kStage);
        const int k = (kt_base + kt) * EK;
        tma_load_2d(st, &tmAh, k, m0, &full[s]);
        tma_load_2d(st + L::kA, &tmAl, k, m0, &full[s]);
        tma_load_2d(st + 2 * L::kA, &tmBh, k, n0, &full[s]);
        tma_load_2d(st + 2 * L::kA + L::kB, &tmBl, k, n0, &full[s]);
        armed_upto = kt + 1;
      }
      *armed_slot = armed_upto;
    }
    __syncwarp();
  } else if (warp == L::kWarpMMA) {
    if (lane == 0) {  // ---- MMA issuer
      constexpr uint32_t idesc = idesc_mma(kBM, kBN, BF16);
      bool ok = true;
      int kt = 0;
      for (int c = 0; c < NCH && ok; ++c) {
        const int b = c & 1;
        if (c >= 2 && !mbar_wait(&acc_empty[b], ((c >> 1) & 1) ^ 1, abort_flag, g.wait_ns)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t acc = tmem + uint32_t(b * kBN);
        const int kt_end = min(KT, kt + kChunk);
        bool first = true;
        for (; kt < kt_end; ++kt) {
          const int s = kt % kStages;
          const uint32_t ph = (kt / kStages) & 1;
          if (!mbar_wait(&full[s], ph, abort_flag, g.wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a_hi = smem_u32(base + s * L::kStage);
          const uint32_t a_lo = a_hi + L::kA;
          const uint32_t b_hi = a_hi + 2 * L::kA;
          const uint32_t b_lo = b_hi + L::kB;
#pragma unroll
          for (int k8 = 0; k8 < kRowBytes / 32; ++k8) {  // 32 bytes (8 tf32 or 16 bf16) of K per MMA
            const uint32_t off = k8 * 32;
            const uint64_t dah = make_desc_k(a_hi + off), dal = make_desc_k(a_lo + off);
            const uint64_t dbh = make_desc_k(b_hi + off), dbl = make_desc_k(b_lo + off);
            mma_op<BF16>(acc, dah, dbh, idesc, first ? 0u : 1u);
            first = false;
            mma_op<BF16>(acc, dah, dbl, idesc, 1u);
            mma_op<BF16>(acc, dal, dbh, idesc, 1u);
          }
          mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
        }
        if (ok) mma_commit(&acc_full[b]);  // accumulator b complete
      }
      if (!ok) {
        // A wait ran out (or the producer gave up): the abandoned accumulator
        // is never signalled, so no drain warp reads it; this thread waits
        // (bounded) until its own MMAs have completed, then raises the abort
        // flag, on which the other warps stop waiting, skip the epilogue and
        // the block frees its tensor memory.
        mma_commit(flush);
        mbar_wait(flush, 0, nullptr);
        atomicExch(g.err, 2);
        *abort_flag = 1;
      }
    }
    __syncwarp();
  } else {
    // ---- drain warps: warp w owns TMEM lanes 32 (w % 4) .. +31 (rows m0 + 32 (w % 4) + lane)
    // and the 128 columns cw .. cw + 127 of the tile
    const int quad = warp & 3, cw = (warp >> 2) * 128;
    float acc[128];
#pragma unroll
    for (int j = 0; j < 128; ++j) acc[j] = 0.f;
    bool ok = true;
    const uint32_t lane_base = tmem + (uint32_t(quad * 32) << 16);
    for (int c = 0; c < NCH; ++c) {
      const int b = c & 1;
      ok = __all_sync(0xffffffffu,
                      ok && mbar_wait(&acc_full[b], (c >> 1) & 1, abort_flag, g.wait_ns) && !*abort_flag);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int q = 0; q < 128; q += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(lane_base + uint32_t(b * kBN + cw + q)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[q + j] += __uint_as_float(r[j]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b])) : "memory");
    }
    if (ok) {
      // The last accumulator has been read, so every MMA and every copy into the
      // pipeline stages is complete: the warp stages its 32 rows there
      // (T[row][col], stride kEpiLd) and writes them back row by row, 512
      // contiguous bytes per store instruction.
      float* T = reinterpret_cast<float*>(base) + warp * (32 * kEpiLd);
#pragma unroll
      for (int q = 0; q < 128; q += 4)
        *reinterpret_cast<float4*>(T + lane * kEpiLd + q) = make_float4(acc[q], acc[q + 1], acc[q + 2], acc[q + 3]);
      __syncwarp();
      const int c0 = n0 + cw + 4 * lane;
      const bool vec = (g.ldd % 4) == 0 && (reinterpret_cast<uintptr_t>(D) & 15) == 0 && c0 + 3 < g.N;
      float bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) bv[i] = g.bias && c0 + i < g.N ? g.bias[c0 + i] : 0.f;
      for (int r = 0; r < 32; ++r) {
        const int row = m0 + quad * 32 + r;
        if (row >= g.M) break;
        const float4 t = *reinterpret_cast<const float4*>(T + r * kEpiLd + 4 * lane);
        float v[4] = {t.x + bv[0], t.y + bv[1], t.z + bv[2], t.w + bv[3]};
        float* dr = D + int64_t(row) * g.ldd + c0;
        if (vec) {
          if (g.accumulate) {
            const float4 o = *reinterpret_cast<const float4*>(dr);
            v[0] += o.x, v[1] += o.y, v[2] += o.z, v[3] += o.w;
          }
          *reinterpret_cast<float4*>(dr) = make_float4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (c0 + i < g.N) dr[i] = v[i] + (g.accumulate ? dr[i] : 0.f);
        }
      }
    }
  }
  // after an abort, wait (bounded) for the last copy armed on every stage
  if (warp == L::kWarpTMA && lane == 0 && *abort_flag) {
    const int armed = *armed_slot;
    for (int kt = max(0, armed - kStages); kt < armed; ++kt)
      mbar_wait(&full[kt % kStages], (kt / kStages) & 1, nullptr);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kBN));
  }
}

// ---- TF32 split: hi = x rounded to TF32 (10-bit mantissa, round to nearest), lo = TF32(x - hi)
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__global__ void split_tf32_kernel(const float* __restrict__ src, int64_t rows, int64_t cols, int64_t lds,
                                  float* __restrict__ hi, float* __restrict__ lo, int64_t ldo) {
  const int64_t n = rows * cols;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols, c = i - r * cols;
    const float v = src[r * lds + c];
    const float h = to_tf32(v);
    hi[r * ldo + c] = h;
    lo[r * ldo + c] = to_tf32(v - h);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

int get_encode() {
  std::lock_guard<std::mutex> lock(g_encode_mu);
  if (g_encode) return SMX_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return smx::set_error(SMX_ERR_CUDA, "cuTensorMapEncodeTiled entry point not available");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return SMX_OK;
}

int make_map(CUtensorMap* tm, const void* ptr, int64_t rows, int64_t cols, int64_t ld, int box_rows, bool bf16 = false) {
  const int es = bf16 ? 2 : 4;
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (ld * es) % 16)
    return smx::set_error(SMX_ERR_ARG, "tensor map: base must be 16-byte aligned and the row pitch a multiple of 16");
  cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
  cuuint64_t strides[1] = {cuuint64_t(ld * es)};
  cuuint32_t box[2] = {cuuint32_t(bf16 ? 2 * kBK : kBK), cuuint32_t(box_rows)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(tm, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                        const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        kRowBytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return smx::set_error(SMX_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return SMX_OK;
}

template <bool BF16, int BN>
int launch_tile(const CUtensorMap& tAh, const CUtensorMap& tAl, const void* Bh, const void* Bl, int64_t ldb, int M,
                int N, int K, float* D, int64_t ldd, const float* bias, int* err, int accumulate, cudaStream_t st,
                int splits, uint64_t wait_ns, int no_loads) {
  using L = Tile<BN>;
  CUtensorMap tBh, tBl;
  int rc;
  if ((rc = make_map(&tBh, Bh, N, K, ldb, BN, BF16)) || (rc = make_map(&tBl, Bl, N, K, ldb, BN, BF16))) return rc;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(gemm_tf32x3_kernel<BF16, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::kTotal);
    attr = true;
  }
  // split-K: slice z runs K-tiles [z * kt_per_z, ...) into D + z * zstride
  const int EK = BF16 ? 2 * kBK : kBK;
  const int KT = (K + EK - 1) / EK;
  const int kt_per_z = splits > 1 ? (KT + splits - 1) / splits : 0;
  const int nz = splits > 1 ? (KT + kt_per_z - 1) / kt_per_z : 1;
  GemmArgs g{M, N, K, D, ldd, bias, err, accumulate, kt_per_z, int64_t(M) * ldd, wait_ns, no_loads};
  dim3 grid((N + BN - 1) / BN, (M + kBM - 1) / kBM, nz);
  gemm_tf32x3_kernel<BF16, BN><<<grid, L::kThreads, L::kTotal, st>>>(tAh, tAl, tBh, tBl, g);
  SMX_LAUNCH_CHECK(BF16 ? "smx_gemm_bf16x3" : "smx_gemm_tf32x3");
  return SMX_OK;
}

// Products wider than 192 columns use 128 x 256 tiles, the others 128 x 128.
template <bool BF16>
int launch(const void* Ah, const void* Al, int64_t lda, const void* Bh, const void* Bl, int64_t ldb, int M, int N,
           int K, float* D, int64_t ldd, const float* bias, int* err, int accumulate, cudaStream_t st,
           int splits = 1, uint64_t wait_ns = kWaitNs, int no_loads = 0) {
  CUtensorMap tAh, tAl;
  int rc;
  if ((rc = make_map(&tAh, Ah, M, K, lda, kBM, BF16)) || (rc = make_map(&tAl, Al, M, K, lda, kBM, BF16))) return rc;
  if (N > 192)
    return launch_tile<BF16, 256>(tAh, tAl, Bh, Bl, ldb, M, N, K, D, ldd, bias, err, accumulate, st, splits, wait_ns,
                                  no_loads);
  return launch_tile<BF16, 128>(tAh, tAl, Bh, Bl, ldb, M, N, K, D, ldd, bias, err, accumulate, st, splits, wait_ns,
                                no_loads);
}

// ---- BF16 split: hi = x rounded to BF16 (round to nearest even), lo = BF16(x - hi)
__global__ void split_bf16_kernel(const float* __restrict__ src, int64_t rows, int64_t cols, int64_t lds,
                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t ldo) {
  const int64_t n = rows * cols;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols, c = i - r * cols;
    const float v = src[r * lds + c];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[r * ldo + c] = h;
    lo[r * ldo + c] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

}  // namespace

int smx::tc::tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000* fn) {
  const int rc = get_encode();
  if (rc == SMX_OK) *fn = g_encode;
  return rc;
}

extern "C" int smx_split_tf32(const float* src, int64_t rows, int64_t cols, int64_t lds, float* hi, float* lo,
                              int64_t ldo, void* stream) {
  SMX_REQUIRE(rows >= 0 && cols >= 0 && lds >= cols && ldo >= cols, "smx_split_tf32: bad sizes");
  if (rows * cols == 0) return SMX_OK;
  SMX_REQUIRE(src && hi && lo, "smx_split_tf32: null pointer");
  split_tf32_kernel<<<smx::grid_for(rows * cols, 256), 256, 0, smx::as_stream(stream)>>>(src, rows, cols, lds, hi, lo,
                                                                                        ldo);
  SMX_LAUNCH_CHECK("smx_split_tf32");
  return SMX_OK;
}

extern "C" int smx_gemm_tf32x3(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi, const float* B_lo,
                               int64_t ldb, int M, int N, int K, float* D, int64_t ldd, const float* bias, int accumulate,
                               int* err, void* stream) {
  SMX_REQUIRE(M >= 0 && N >= 0 && K >= 0 && lda >= K && ldb >= K && ldd >= N, "smx_gemm_tf32x3: bad sizes");
  if (M == 0 || N == 0) return SMX_OK;
  SMX_REQUIRE(K >= 1 && A_hi && A_lo && B_hi && B_lo && D && err, "smx_gemm_tf32x3: null pointer");
  int rc = get_encode();
  if (rc) return rc;
  return launch<false>(A_hi, A_lo, lda, B_hi, B_lo, ldb, M, N, K, D, ldd, bias, err, accumulate,
                       smx::as_stream(stream));
}

// Self-test of the timeout path: the same kernel with its producer issuing no
// copies, so the MMA thread's first wait cannot complete; after `wait_ns` it
// records error code 2 in *err, raises the abort flag, the drain warps skip
// the epilogue and the block frees its tensor memory.  Nothing is in flight
// when it gives up (no copy, no MMA), and D is not written.
extern "C" int smx_gemm_tf32x3_timeout_selftest(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi,
                                                const float* B_lo, int64_t ldb, int M, int N, int K, float* D,
                                                int64_t ldd, int* err, uint64_t wait_ns, void* stream) {
  SMX_REQUIRE(M >= 1 && N >= 1 && K >= 1 && lda >= K && ldb >= K && ldd >= N,
              "smx_gemm_tf32x3_timeout_selftest: bad sizes");
  SMX_REQUIRE(A_hi && A_lo && B_hi && B_lo && D && err, "smx_gemm_tf32x3_timeout_selftest: null pointer");
  SMX_REQUIRE(wait_ns <= kWaitNs, "smx_gemm_tf32x3_timeout_selftest: wait bound above the default");
  int rc = get_encode();
  if (rc) return rc;
  return launch<false>(A_hi, A_lo, lda, B_hi, B_lo, ldb, M, N, K, D, ldd, nullptr, err, 0, smx::as_stream(stream), 1,
                       wait_ns, 1);
}

extern "C" int smx_gemm_bf16x3(const uint16_t* A_hi, const uint16_t* A_lo, int64_t lda, const uint16_t* B_hi,
                               const uint16_t* B_lo, int64_t ldb, int M, int N, int K, float* D, int64_t ldd,
                               const float* bias, int accumulate, int* err, void* stream) {
  SMX_REQUIRE(M >= 0 && N >= 0 && K >= 0 && lda >= K && ldb >= K && ldd >= N, "smx_gemm_bf16x3: bad sizes");
  if (M == 0 || N == 0) return SMX_OK;
  SMX_REQUIRE(K >= 1 && A_hi && A_lo && B_hi && B_lo && D && err, "smx_gemm_bf16x3: null pointer");
  int rc = get_encode();
  if (rc) return rc;
  return launch<true>(A_hi, A_lo, lda, B_hi, B_lo, ldb, M, N, K, D, ldd, bias, err, accumulate,
                      smx::as_stream(stream));
}

namespace {
// D = sum over z of the split-K slices (fixed order) + bias (+ D)
__global__ void splitk_reduce_kernel(const float* __restrict__ part, int nz, int M, int N, float* __restrict__ D,
                                     int64_t ldd, const float* __restrict__ bias, int accumulate) {
  const int64_t n = int64_t(M) * N;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = i / N, c = i - r * N;
    float v = 0.f;
    for (int z = 0; z < nz; ++z) v += part[z * n + r * N + c];
    if (bias) v += bias[c];
    float* d = D + r * ldd + c;
    *d = v + (accumulate ? *d : 0.f);
  }
}

int splitk_slices(int K, int splits) {
  const int KT = (K + kBK - 1) / kBK;
  const int per = (KT + splits - 1) / splits;
  return (KT + per - 1) / per;
}
}  // namespace

extern "C" int smx_gemm_tf32x3_splits(int64_t M, int N, int K) {
  if (M <= 0 || N <= 0 || K <= 0) return 1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  const int64_t ctas = (M + kBM - 1) / kBM * (N > 192 ? (N + 255) / 256 : (N + 127) / 128);
  const int64_t k_tiles = (int64_t(K) + kBK - 1) / kBK;
  const int64_t s = std::min<int64_t>(std::min<int64_t>(8, sms / ctas), k_tiles / 64);
  return int(std::max<int64_t>(1, s));
}

extern "C" size_t smx_gemm_tf32x3_splitk_workspace(int M, int N, int K, int splits) {
  if (M <= 0 || N <= 0 || K <= 0 || splits < 1) return 0;
  return size_t(splitk_slices(K, splits)) * size_t(M) * size_t(N) * sizeof(float);
}

extern "C" int smx_gemm_tf32x3_splitk(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi,
                                      const float* B_lo, int64_t ldb, int M, int N, int K, float* D, int64_t ldd,
                                      const float* bias, int accumulate, int splits, void* ws, size_t ws_bytes,
                                      int* err, void* stream) {
  SMX_REQUIRE(M >= 0 && N >= 0 && K >= 0 && lda >= K && ldb >= K && ldd >= N && splits >= 1 && splits <= 65535,
              "smx_gemm_tf32x3_splitk: bad sizes");
  if (M == 0 || N == 0) return SMX_OK;
  SMX_REQUIRE(K >= 1 && A_hi && A_lo && B_hi && B_lo && D && err, "smx_gemm_tf32x3_splitk: null pointer");
  if (splits == 1 || splitk_slices(K, splits) == 1)
    return smx_gemm_tf32x3(A_hi, A_lo, lda, B_hi, B_lo, ldb, M, N, K, D, ldd, bias, accumulate, err, stream);
  SMX_REQUIRE(ws && ws_bytes >= smx_gemm_tf32x3_splitk_workspace(M, N, K, splits),
              "smx_gemm_tf32x3_splitk: workspace too small");
  int rc = get_encode();
  if (rc) return rc;
  cudaStream_t st = smx::as_stream(stream);
  float* part = static_cast<float*>(ws);
  rc = launch<false>(A_hi, A_lo, lda, B_hi, B_lo, ldb, M, N, K, part, N, nullptr, err, 0, st, splits);
  if (rc) return rc;
  splitk_reduce_kernel<<<smx::grid_for(int64_t(M) * N, 256), 256, 0, st>>>(part, splitk_slices(K, splits), M, N, D,
                                                                          ldd, bias, accumulate);
  SMX_LAUNCH_CHECK("smx_gemm_tf32x3_splitk");
  return SMX_OK;
}

extern "C" int smx_split_bf16(const float* src, int64_t rows, int64_t cols, int64_t lds, uint16_t* hi, uint16_t* lo,
                              int64_t ldo, void* stream) {
  SMX_REQUIRE(rows >= 0 && cols >= 0 && lds >= cols && ldo >= cols, "smx_split_bf16: bad sizes");
  if (rows * cols == 0) return SMX_OK;
  SMX_REQUIRE(src && hi && lo, "smx_split_bf16: null pointer");
  split_bf16_kernel<<<smx::grid_for(rows * cols, 256), 256, 0, smx::as_stream(stream)>>>(
      src, rows, cols, lds, reinterpret_cast<__nv_bfloat16*>(hi), reinterpret_cast<__nv_bfloat16*>(lo), ldo);
  SMX_LAUNCH_CHECK("smx_split_bf16");
  return SMX_OK;
}
