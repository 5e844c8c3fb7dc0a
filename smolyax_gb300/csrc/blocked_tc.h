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
constexpr int kBox = 8;           // linear columns per unit of the contraction (8 FP64 = 64 bytes of x)
constexpr int kSplits = 3;        // bf16 hi / mid / lo
// tensor memory (512 columns): nbuf accumulators of kMaxN columns (3 when A
// leaves room, else 2), then A: K step kk, part s in the 8 columns
// acol + 24 kk + 8 s, acol = nbuf * kMaxN (two bf16 per column)
constexpr int kMaxSteps = (512 - 2 * kMaxN) / (kSplits * 8);  // 16 K steps = 256 rows
SMX_BTC_HD inline int acc_buffers(int n_agen) { return 3 * kMaxN + kSplits * 8 * n_agen <= 512 ? 3 : 2; }
constexpr int kBStages = 12;      // coefficient stages in shared memory
constexpr int kBStageMax = kSplits * kMaxN * 32;  // one coefficient stage at N = 64: 6 KB
constexpr int kComputeWarps = 16;
constexpr int kThreads = 32 * (kComputeWarps + 2);  // + producer warp + MMA warp
constexpr int64_t kSmemLimit = 225 * 1024;

SMX_BTC_HD inline int64_t align1k(int64_t v) { return (v + 1023) / 1024 * 1024; }

// Shared-memory layout of one block (byte offsets from a 1024-aligned base):
// basis values Phi [n_phi_pad][128] FP32, the node rows' paths, coefficient
// stages, the per-point partial sums, barriers.
struct Smem {
  int64_t phi, row, b, rs, bar, total;
};

SMX_BTC_HD inline Smem smem_layout(int64_t n_phi_pad) {
  Smem s;
  s.phi = 0;
  s.row = n_phi_pad * kTile * 4;
  s.b = align1k(s.row + int64_t(kMaxSteps) * kStep * 16);
  s.rs = s.b + int64_t(kBStages) * kBStageMax;
  s.bar = s.rs + 4 * kTile * 2 * 4;
  s.total = s.bar + 512 + 1024;  // barriers and flags; alignment slack of the dynamic base
  return s;
}

}  // namespace btc
}  // namespace smx
