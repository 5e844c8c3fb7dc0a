// Shapes shared by the tensor-core blocked evaluator (blocked_tc.cu) and its
// host table builder (layout.cu build_blocked_tc).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SMX_BTC_HD __host__ __device__
#else
#define SMX_BTC_HD
#endif

namespace smx {
namespace btc {

constexpr int kTile = 128;        // points per tile = MMA M = tensor-memory lanes
constexpr int kStep = 16;         // node rows per K step (one bf16 MMA)
constexpr int kMaxN = 64;         // columns per chunk (MMA N, one accumulator)
constexpr int kMaxPhi = 128;      // basis slots of the table dimensions (with the constant slot)
constexpr int kMaxChunks = 64;    // chunks per plan (kernel argument array)
constexpr int kBox = 8;           // dimensions per x box (8 FP64 = one 64-byte swizzle row)
constexpr int kSplits = 3;        // bf16 hi / mid / lo
// tensor memory (512 columns): two accumulators of kMaxN columns, then A:
// K step kk, part s in the 8 columns kAcol + 24 kk + 8 s (two bf16 per column)
constexpr int kAcol = 2 * kMaxN;
constexpr int kMaxSteps = (512 - kAcol) / (kSplits * 8);  // 16 K steps = 256 rows
constexpr int kBStages = 8;       // coefficient stages in shared memory
constexpr int kBStageMax = kSplits * kMaxN * 32;  // one coefficient stage at N = 64: 6 KB
constexpr int kBoxBytes = kBox * kTile * 8;       // one x box: 8 KB
constexpr int kXMin = 6, kXMax = 16;              // x boxes in shared memory (as many as fit)
constexpr int kComputeWarps = 16;
constexpr int kThreads = 32 * (kComputeWarps + 2);  // + producer warp + MMA warp
constexpr int64_t kSmemLimit = 225 * 1024;

SMX_BTC_HD inline int64_t align1k(int64_t v) { return (v + 1023) / 1024 * 1024; }

// Shared-memory layout of one block (byte offsets from a 1024-aligned base):
// basis values Phi [n_phi_pad][128] FP32, coefficient stages, x boxes, the
// per-point partial sums, barriers.  n_x = 0 when not even kXMin boxes fit.
struct Smem {
  int64_t phi, b, x, rs, bar, total;
  int n_x;
};

SMX_BTC_HD inline Smem smem_layout(int64_t n_phi_pad) {
  Smem s;
  s.phi = 0;
  s.b = align1k(n_phi_pad * kTile * 4);
  s.x = s.b + kBStages * kBStageMax;
  const int64_t rest = 4 * kTile * 2 * 4 + 512 + 1024;  // partial sums, barriers, base alignment slack
  int64_t n = (kSmemLimit - s.x - rest) / kBoxBytes;
  n = n > kXMax ? kXMax : n;
  s.n_x = n < kXMin ? 0 : int(n);
  s.rs = s.x + int64_t(s.n_x) * kBoxBytes;
  s.bar = s.rs + 4 * kTile * 2 * 4;
  s.total = s.bar + 512 + 1024;
  return s;
}

}  // namespace btc
}  // namespace smx
