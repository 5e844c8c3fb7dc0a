// Tensor-core blocked evaluator of the orthogonal-polynomial form, one output
// (tables: layout.cu build_blocked_tc).
//
//   I(x) = c_0 + sum_a V_a(x) [ sum_s B_t[a][s] Phi_s(x) + sum_j B_l[a][j] x_j ]
//
// over the nodes a of the index set (rows, by remaining budget), the basis
// slots s of the table dimensions (slot 0 = 1) and the linear dimensions j.
// One persistent block per SM walks 128-point tiles; per tile
//   compute warps (16)  Phi (basis values of the table dimensions, shared
//                       memory) and the rows V_a of A = [128 points x rows],
//                       split into three bf16 parts (hi + mid + lo = the FP32
//                       value), written to tensor memory (thread = point = lane);
//   MMA thread          T = A B for every chunk of <= 64 columns on the tensor
//                       cores (kind::f16, A from tensor memory, B from shared
//                       memory, six part products per 16-row K step, FP32
//                       accumulation in tensor memory, two accumulators);
//   producer thread     the chunks' coefficient stages (bulk copies from the
//                       L2-resident image) and L2 prefetches of the x rows a
//                       few chunks ahead of their use (bulk prefetch of each
//                       point's row segment);
//   compute warps       y_p += sum_j T[p][j] x_pj -- x read once, straight
//                       from global memory (32-byte streaming loads, two units
//                       of 8 coordinates ahead in registers), converted to FP32
//                       on the integer pipes -- and sum_s T[p][s] Phi_s,
//                       Kahan-compensated, then a fixed-order sum over the 4
//                       column groups.
// (Measured and replaced: a TMA tile stream of the x rows, 8 coordinates x
// 128 points per box, reached at most ~2.45 TB/s however many boxes were in
// flight; per-row bulk L2 prefetches through the TMA unit delayed the
// coefficient stages queued behind them.)  Every wait is bounded: on a timeout the block records
// an error, stops waiting and finishes its loops without work, so that every
// barrier is still reached.
#include <cuda_bf16.h>

#include <mutex>
#include <string>

#include "blocked_tc.h"
#include "common.cuh"
#include "fp_convert.cuh"
#include "tc_util.cuh"

namespace {

using namespace smx::tc;
using namespace smx::btc;
using smx::f64_to_f32;
using smx::kahan_add;

constexpr int kRec = 512;
constexpr int kPfChunks = 4;  // linear chunks of x prefetched to L2 ahead of the producer (64 KB each per block)
constexpr int kWarpProducer = kComputeWarps, kWarpMMA = kComputeWarps + 1;

__constant__ float t_alpha[2][kRec];
__constant__ float t_beta[2][kRec];

struct TcArgs {
  int64_t P, ldx;
  const double* x;
  float* y;
  int n_td, n_phi, n_phi_pad, n_rows, max_depth, n_agen, n_chunks, n_tchunks, n_boxes, lin0, stages;
  int nbuf, acol;  // accumulators in tensor memory, first column of A
  int8_t lin_idx[kMaxChunks];  // the linear chunks' positions in the chunk order
  int td_col, td_bytes;  // x row segment of the table dimensions (L2 prefetch)
  float c0;
  const int4* td;
  const float2* tdab;
  const int4* row;
  const uint8_t* bimg;
  const int32_t* box;
  int* err;
  uint64_t wait_ns;
  int4 chunk[kMaxChunks];  // {N | table << 16, K steps, stage image offset / 16, first slot or unit}
};

struct Bars {
  uint64_t b_full[kBStages], b_empty[kBStages];
  uint64_t acc_full[3], acc_empty[3];
  uint64_t a_full, flush;
  uint32_t tmem;
  int abort_flag;
};
static_assert(sizeof(Bars) <= 512, "barrier block");

__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kComputeWarps * 32) : "memory"); }

// D (tensor memory) += A (tensor memory) B (shared memory), kind::f16.
__device__ __forceinline__ void mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tmem_st4(uint32_t taddr, const uint32_t (&v)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "r"(v[0]), "r"(v[1]),
               "r"(v[2]), "r"(v[3])
               : "memory");
}

// Packs the bf16 parts (hi, mid, lo) of two FP32 values: word s of the result
// holds part s of (a, b) (a in the low half).
__device__ __forceinline__ void split3(float a, float b, uint32_t (&w)[3]) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  float2 fh = __bfloat1622float2(h);
  const float ra = a - fh.x, rb = b - fh.y;
  __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
  float2 fm = __bfloat1622float2(m);
  __nv_bfloat162 l = __floats2bfloat162_rn(ra - fm.x, rb - fm.y);
  w[0] = *reinterpret_cast<uint32_t*>(&h);
  w[1] = *reinterpret_cast<uint32_t*>(&m);
  w[2] = *reinterpret_cast<uint32_t*>(&l);
}

// x loads of one unit (8 coordinates of one point): 32-byte (X32) or 16-byte
// streaming loads, or guarded scalar loads when some coordinates are masked.
template <bool X32>
__device__ __forceinline__ void load_unit(const double* __restrict__ p, int mask, double (&v)[8]) {
  if (mask == 0) {
    if constexpr (X32) {
      asm volatile("ld.global.nc.L1::no_allocate.v4.f64 {%0, %1, %2, %3}, [%4];"
                   : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
                   : "l"(p));
      asm volatile("ld.global.nc.L1::no_allocate.v4.f64 {%0, %1, %2, %3}, [%4];"
                   : "=d"(v[4]), "=d"(v[5]), "=d"(v[6]), "=d"(v[7])
                   : "l"(p + 4));
    } else {
#pragma unroll
      for (int j = 0; j < 8; j += 2)
        asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v[j]), "=d"(v[j + 1]) : "l"(p + j));
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = ((mask >> j) & 1) ? 0.0 : __ldg(p + j);
  }
}

template <bool X32>
__global__ void __launch_bounds__(kThreads, 1) blocked_tc_kernel(const __grid_constant__ TcArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const Smem L = smem_layout(g.n_phi_pad);
  float* phi = reinterpret_cast<float*>(base + L.phi);
  int4* rowtab = reinterpret_cast<int4*>(base + L.row);
  uint8_t* bst = base + L.b;
  float* rs = reinterpret_cast<float*>(base + L.rs);
  Bars* bars = reinterpret_cast<Bars*>(base + L.bar);
  volatile int* abort_flag = &bars->abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n_tiles = (g.P + kTile - 1) / kTile;
  const int64_t G = gridDim.x;
  const int nt = blockIdx.x < n_tiles ? int((n_tiles - blockIdx.x + G - 1) / G) : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kBStages; ++s) {
      mbar_init(&bars->b_full[s], 1);
      mbar_init(&bars->b_empty[s], 1);
    }
    for (int b = 0; b < 3; ++b) {
      mbar_init(&bars->acc_full[b], 1);
      mbar_init(&bars->acc_empty[b], kComputeWarps);
    }
    mbar_init(&bars->a_full, 1);
    mbar_init(&bars->flush, 1);
    bars->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // constant slot 0 and the padding slots of Phi (never rewritten); the rows' paths
  for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
    phi[i] = 1.f;
    for (int s = g.n_phi; s < g.n_phi_pad; ++s) phi[s * kTile + i] = 0.f;
  }
  for (int r = threadIdx.x; r < g.n_agen * kStep; r += blockDim.x)
    rowtab[r] = r < g.n_rows ? __ldg(&g.row[r]) : make_int4(0, 0, 0, 0);
  if (warp == kWarpMMA) {  // all of tensor memory: accumulators and A
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = bars->tmem;

  if (warp == kWarpProducer) {
    // ---- producer warp: coefficient stages by bulk copies (lane 0; the TMA
    // unit carries nothing else), and L2 prefetches of the x row segments of
    // the table dimensions (one tile ahead) and of the linear chunks
    // (kPfChunks chunks ahead) by all lanes, one per 128-byte line
    const int n_lin = g.n_chunks - g.n_tchunks;
    auto prefetch_rows = [&](int64_t tile, int64_t col, int bytes) {  // within each row: [col, ldx)
      const int64_t room = (g.ldx - col) * 8;
      bytes = int(room < bytes ? room : int64_t(bytes));
      if (bytes <= 0) return;
      const int64_t p0 = tile * kTile;
      const int rows = int(g.P - p0 < kTile ? g.P - p0 : int64_t(kTile));
      const double* xp = g.x + p0 * g.ldx + col;
      // one prefetch per 128-byte line of every row segment (all inside the row),
      // lanes over (row, line)
      const int lmax = (bytes + 127) / 128 + 1;
      for (int q = lane; q < rows * lmax; q += 32) {
        const int r = q / lmax, l = q - r * lmax;
        const uintptr_t a = reinterpret_cast<uintptr_t>(xp + r * g.ldx);
        const uintptr_t first = a & ~uintptr_t(127), last = (a + bytes - 1) & ~uintptr_t(127);
        if (first + 128 * uintptr_t(l) <= last)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(first + 128 * uintptr_t(l)));
      }
    };
    auto prefetch_lin = [&](int64_t k) {  // the k-th linear chunk of this block's sequence
      const int i = int(k / n_lin), c = g.lin_idx[k % n_lin];
      if (i >= nt) return;
      const int4 ch = g.chunk[c];
      prefetch_rows(blockIdx.x + int64_t(i) * G, g.lin0 + int64_t(kBox) * ch.w, (ch.x & 0xFFFF) * 8);
    };
    int64_t pf = 0;
    if (nt > 0 && g.td_bytes > 0) prefetch_rows(blockIdx.x, g.td_col, g.td_bytes);
    for (; n_lin > 0 && pf < kPfChunks; ++pf) prefetch_lin(pf);
    uint64_t ib = 0;
    bool ok = true;
    for (int i = 0; i < nt && ok; ++i) {
      if (i + 1 < nt && g.td_bytes > 0) prefetch_rows(blockIdx.x + int64_t(i + 1) * G, g.td_col, g.td_bytes);
      for (int c = 0; c < g.n_chunks && ok; ++c) {
        const int4 ch = g.chunk[c];
        if (ch.x >> 16 == 0 && n_lin > 0) prefetch_lin(pf++);
        const uint32_t bytes = uint32_t(ch.x & 0xFFFF) * (kSplits * 32);
        for (int jb = 0; jb < ch.y; ++jb, ++ib) {
          const int s = int(ib % kBStages);
          bool got = true;
          if (lane == 0) {
            if (ib >= kBStages)
              got = mbar_wait(&bars->b_empty[s], uint32_t((ib / kBStages) & 1) ^ 1u, abort_flag, g.wait_ns);
            if (got) {
              mbar_expect_tx(&bars->b_full[s], bytes);
              bulk_load(bst + s * kBStageMax, g.bimg + int64_t(ch.z) * 16 + int64_t(jb) * bytes, bytes,
                        &bars->b_full[s]);
            } else {
              atomicExch(g.err, 1);
              *abort_flag = 1;
            }
          }
          if (!__shfl_sync(0xffffffffu, got ? 1 : 0, 0)) {
            ok = false;
            break;
          }
        }
      }
    }
    if (!ok && lane == 0) {
      // wait (bounded) until the copies already issued have landed
      for (uint64_t u = ib > kBStages ? ib - kBStages : 0; u < ib; ++u)
        mbar_wait(&bars->b_full[u % kBStages], uint32_t((u / kBStages) & 1), nullptr, g.wait_ns);
    }
    __syncwarp();
  } else if (warp == kWarpMMA) {
    if (lane == 0) {
      // ---- MMA issuer
      uint64_t ib = 0, gc = 0;
      bool ok = true;
      for (int i = 0; i < nt && ok; ++i) {
        if (!mbar_wait(&bars->a_full, uint32_t(i & 1), abort_flag, g.wait_ns)) {
          ok = false;
          break;
        }
        for (int c = 0; c < g.n_chunks && ok; ++c, ++gc) {
          const int4 ch = g.chunk[c];
          const int N = ch.x & 0xFFFF, nk = ch.y;
          const int b = int(gc % g.nbuf);
          if (gc >= uint64_t(g.nbuf) &&
              !mbar_wait(&bars->acc_empty[b], uint32_t((gc / g.nbuf) & 1) ^ 1u, abort_flag, g.wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t d_tmem = tmem + uint32_t(b * kMaxN);
          const uint32_t idesc = idesc_mma(kTile, N, true);
          for (int j = 0; j < nk && ok; ++j) {
            const int kk = nk - 1 - j;  // the last rows (small terms) first
            const int bs = int(ib % kBStages);
            if (!mbar_wait(&bars->b_full[bs], uint32_t((ib / kBStages) & 1), abort_flag, g.wait_ns)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t b_addr = smem_u32(bst + bs * kBStageMax);
            const uint32_t bsz = uint32_t(N) * 32;
            const uint32_t a0 = tmem + uint32_t(g.acol + kSplits * 8 * kk);
            uint64_t db[3];
#pragma unroll
            for (int s = 0; s < 3; ++s) db[s] = make_desc_sw(b_addr + s * bsz, 32);
            // part products from the smallest to the largest (the accumulator
            // truncates: the large terms are added last, once)
            mma_ts(d_tmem, a0 + 16, db[0], idesc, j > 0 ? 1u : 0u);
            mma_ts(d_tmem, a0 + 8, db[1], idesc, 1u);
            mma_ts(d_tmem, a0, db[2], idesc, 1u);
            mma_ts(d_tmem, a0 + 8, db[0], idesc, 1u);
            mma_ts(d_tmem, a0, db[1], idesc, 1u);
            mma_ts(d_tmem, a0, db[0], idesc, 1u);
            mma_commit(&bars->b_empty[bs]);
            ++ib;
          }
          if (ok) mma_commit(&bars->acc_full[b]);
        }
      }
      if (!ok) {
        // the abandoned accumulator is never signalled; wait (bounded) for this
        // thread's own MMAs, then raise the abort flag
        mma_commit(&bars->flush);
        mbar_wait(&bars->flush, 0, nullptr, g.wait_ns);
        atomicExch(g.err, 2);
        *abort_flag = 1;
      }
    }
    __syncwarp();
  } else {
    // ---- compute warps: warp (quadrant qd = warp % 4: points 32 qd .. +31 =
    // tensor-memory lanes, column group grp = warp / 4: units grp, grp + 4, ...)
    const int tid = threadIdx.x;
    const int qd = warp & 3, grp = warp >> 2, pt = 32 * qd + lane;
    const uint32_t lane_base = tmem + (uint32_t(32 * qd) << 16);
    uint64_t gc = 0;
    bool ok = true;
    auto wait_ok = [&](uint64_t* bar, uint32_t parity) {
      if (!ok || *abort_flag) {
        ok = false;
        return;
      }
      if (!mbar_wait(bar, parity, abort_flag, g.wait_ns)) {
        atomicExch(g.err, 3);
        *abort_flag = 1;
        ok = false;
      }
    };
    for (int i = 0; i < nt; ++i) {
      const int64_t p0 = (blockIdx.x + int64_t(i) * G) * kTile;
      const double* xrow = g.x + min(p0 + pt, g.P - 1) * g.ldx + g.lin0;

      // phase 0: basis values of the table dimensions (thread: point q, dimensions hb, hb + 4, ...)
      {
        const int q = tid & (kTile - 1), hb = tid >> 7;
        const double* xp = g.x + min(p0 + q, g.P - 1) * g.ldx;
        for (int h0 = hb; h0 < g.n_td; h0 += 4 * 16) {
          double xh[16];
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const int h = h0 + 4 * r;
            xh[r] = h < g.n_td ? __ldg(xp + __ldg(&g.td[h].x)) : 0.0;
          }
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const int h = h0 + 4 * r;
            if (h >= g.n_td) break;
            const int4 t4 = __ldg(&g.td[h]);
            const float2 ab = __ldg(&g.tdab[h]);
            const float z = fmaf(ab.x, f64_to_f32(xh[r]), ab.y);
            float pm1 = 0.f, pc = 1.f;
            for (int n = 0; n < t4.y; ++n) {
              const float pn = t_alpha[t4.w][n] * z * pc - t_beta[t4.w][n] * pm1;
              pm1 = pc;
              pc = pn;
              phi[(t4.z + n) * kTile + q] = pc;
            }
          }
        }
      }
      // the first two units of x of this warp's column group, in flight during A
      double xn0[8], xn1[8];
      if (grp < g.n_boxes) load_unit<X32>(xrow + kBox * grp, __ldg(g.box + grp), xn0);
      if (grp + 4 < g.n_boxes) load_unit<X32>(xrow + kBox * (grp + 4), __ldg(g.box + grp + 4), xn1);
      compute_sync();

      // A = V in tensor memory: warp (qd, grp) writes the half steps (8 rows)
      // grp, grp + 4, ... of its 32 points (lanes), three bf16 parts each
      for (int hs = grp; hs < 2 * g.n_agen; hs += 4) {
        const int kk = hs >> 1, half = hs & 1;
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int r = kk * kStep + 8 * half + j;
          const int4 rw = rowtab[r];
          const unsigned wv[4] = {unsigned(rw.x), unsigned(rw.y), unsigned(rw.z), unsigned(rw.w)};
          float pv = 1.f;
#pragma unroll
          for (int qq = 0; qq < 8; ++qq)
            if (qq < g.max_depth) pv *= phi[((wv[qq >> 1] >> (16 * (qq & 1))) & 0xFFFFu) * kTile + pt];
          v[j] = r < g.n_rows ? pv : 0.f;
        }
        uint32_t w[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint32_t t3[3];
          split3(v[2 * j], v[2 * j + 1], t3);
          w[0][j] = t3[0];
          w[1][j] = t3[1];
          w[2][j] = t3[2];
        }
#pragma unroll
        for (int s = 0; s < 3; ++s) tmem_st4(lane_base + uint32_t(g.acol + kSplits * 8 * kk + 8 * s + 4 * half), w[s]);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      compute_sync();
      if (tid == 0) mbar_arrive(&bars->a_full);

      // contraction of the accumulators: units of 8 columns (u = grp, grp + 4, ...)
      float s_acc = 0.f, c_acc = 0.f;
      for (int c = 0; c < g.n_chunks; ++c, ++gc) {
        const int4 ch = g.chunk[c];
        const int N = ch.x & 0xFFFF, table = ch.x >> 16;
        const int b = int(gc % g.nbuf);
        wait_ok(&bars->acc_full[b], uint32_t((gc / g.nbuf) & 1));
        ok = __all_sync(0xffffffffu, ok);
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (int u = grp; u < N / 8; u += 4) {
          uint32_t T[8];
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                       : "=r"(T[0]), "=r"(T[1]), "=r"(T[2]), "=r"(T[3]), "=r"(T[4]), "=r"(T[5]), "=r"(T[6]),
                         "=r"(T[7])
                       : "r"(lane_base + uint32_t(b * kMaxN + 8 * u)));
          float v;
          if (table) {
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const float* ph = phi + (ch.w + 8 * u) * kTile + pt;
            v = __uint_as_float(T[0]) * ph[0];
#pragma unroll
            for (int j = 1; j < 8; ++j) v = fmaf(__uint_as_float(T[j]), ph[j * kTile], v);
          } else {
            // this unit's x arrived in xn0; the unit two ahead in the group is loaded now
            double xv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              xv[j] = xn0[j];
              xn0[j] = xn1[j];
            }
            const int nb = ch.w + u + 8;
            if (nb < g.n_boxes) load_unit<X32>(xrow + kBox * nb, __ldg(g.box + nb), xn1);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            v = __uint_as_float(T[0]) * f64_to_f32(xv[0]);
#pragma unroll
            for (int j = 1; j < 8; ++j) v = fmaf(__uint_as_float(T[j]), f64_to_f32(xv[j]), v);
          }
          kahan_add(s_acc, c_acc, v);
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars->acc_empty[b]);
      }
      // per-point sum over the 4 column groups, in a fixed order
      rs[grp * kTile + pt] = s_acc;
      rs[(4 + grp) * kTile + pt] = c_acc;
      compute_sync();
      if (tid < kTile) {
        float s = 0.f, cc = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          kahan_add(s, cc, rs[q * kTile + tid]);
          kahan_add(s, cc, -rs[(4 + q) * kTile + tid]);
        }
        if (p0 + tid < g.P) g.y[p0 + tid] = g.c0 + (s - cc);
      }
      compute_sync();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == kWarpMMA) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

std::mutex g_mu;
bool g_ready[64] = {};
int g_sms[64] = {};

int prepare(int* sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return smx::set_error(SMX_ERR_CUDA, "smx_blocked_tc_eval: no current device");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ready[dev]) {
    static float al[2][kRec], be[2][kRec];
    for (int f = 0; f < 2; ++f)
      for (int n = 0; n < kRec; ++n) {
        // phi_{n+1} = alpha_n z phi_n - beta_n phi_{n-1}: Legendre, normalised Hermite
        al[f][n] = f == 0 ? float(double(2 * n + 1) / double(n + 1)) : float(sqrt(2.0 / double(n + 1)));
        be[f][n] = f == 0 ? float(double(n) / double(n + 1)) : float(sqrt(double(n) / double(n + 1)));
      }
    if (cudaMemcpyToSymbol(t_alpha, al, sizeof(al)) != cudaSuccess ||
        cudaMemcpyToSymbol(t_beta, be, sizeof(be)) != cudaSuccess ||
        cudaFuncSetAttribute(blocked_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemLimit)) !=
            cudaSuccess ||
        cudaFuncSetAttribute(blocked_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(kSmemLimit)) != cudaSuccess ||
        cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_blocked_tc_eval: device set-up failed");
    g_ready[dev] = true;
  }
  *sms = g_sms[dev];
  return SMX_OK;
}

int check_plan(const smx_blocked_tc* b) {
  if (!b || b->d_in < 1 || b->n_td < 0 || b->n_phi < 1 || b->n_phi > b->n_phi_pad || b->n_phi_pad > kMaxPhi ||
      b->n_phi_pad % 16 || b->n_rows < 1 || b->max_depth < 0 || b->max_depth > 8 || b->n_agen < 1 ||
      b->n_agen > kMaxSteps || b->n_chunks < 1 || b->n_chunks > kMaxChunks || b->n_boxes < 0 || b->lin0 < 0 ||
      b->lin0 % 2 || b->stages < 1 || !b->row || !b->chunk || !b->bimg || !b->err ||
      (b->n_td > 0 && !(b->td && b->tdab)) || (b->n_boxes > 0 && !b->box) ||
      (reinterpret_cast<uintptr_t>(b->bimg) & 15))
    return smx::set_error(SMX_ERR_ARG, "smx_blocked_tc_eval: bad plan");
  int stages = 0;
  for (int c = 0; c < b->n_chunks; ++c) {
    const int32_t* ch = b->chunk + 4 * c;
    const int N = ch[0] & 0xFFFF, table = ch[0] >> 16, nk = ch[1];
    if (N < 16 || N > kMaxN || N % 16 || nk < 1 || nk > b->n_agen || ch[2] < 0 || ch[3] < 0 ||
        (table && ch[3] + N > b->n_phi_pad) || (!table && ch[3] + N / kBox > b->n_boxes))
      return smx::set_error(SMX_ERR_ARG, "smx_blocked_tc_eval: bad chunk table");
    stages += nk;
  }
  if (stages != b->stages) return smx::set_error(SMX_ERR_ARG, "smx_blocked_tc_eval: stage count");
  if (acc_buffers(b->n_agen) * kMaxN + kSplits * 8 * b->n_agen > 512)
    return smx::set_error(SMX_ERR_ARG, "smx_blocked_tc_eval: A does not fit tensor memory");
  if (smem_layout(b->n_phi_pad).total > kSmemLimit)
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_blocked_tc_eval: shared memory");
  if (b->td_col < 0 || b->td_col % 2 || b->td_bytes < 0 || b->td_bytes % 16)
    return smx::set_error(SMX_ERR_ARG, "smx_blocked_tc_eval: bad table-dimension segment");
  return SMX_OK;
}

}  // namespace

extern "C" int smx_blocked_tc_supported(const smx_blocked_tc* b, const double* x, int64_t ldx) {
  if (!b || !x) return 0;
  return (reinterpret_cast<uintptr_t>(x) & 15) == 0 && ldx % 2 == 0 && ldx >= b->d_in ? 1 : 0;
}

extern "C" int smx_blocked_tc_eval(const smx_blocked_tc* b, const double* x, int64_t P, int64_t ldx, float* y,
                                   void* stream) {
  int rc = check_plan(b);
  if (rc) return rc;
  SMX_REQUIRE(P >= 0 && ldx >= b->d_in, "smx_blocked_tc_eval: bad sizes");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y, "smx_blocked_tc_eval: null pointer");
  if (!smx_blocked_tc_supported(b, x, ldx))
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_blocked_tc_eval: x must be 16-byte aligned with an even row pitch");
  SMX_REQUIRE(P <= (int64_t(1) << 31) - kTile, "smx_blocked_tc_eval: too many points");
  int sms = 0;
  if ((rc = prepare(&sms))) return rc;
  TcArgs a{};
  a.P = P;
  a.ldx = ldx;
  a.x = x;
  a.y = y;
  a.n_td = b->n_td;
  a.n_phi = b->n_phi;
  a.n_phi_pad = b->n_phi_pad;
  a.n_rows = b->n_rows;
  a.max_depth = b->max_depth;
  a.n_agen = b->n_agen;
  a.n_chunks = b->n_chunks;
  a.n_boxes = b->n_boxes;
  a.lin0 = b->lin0;
  a.stages = b->stages;
  a.n_tchunks = 0;
  for (int c = 0, k = 0; c < b->n_chunks; ++c) {
    if (b->chunk[4 * c] >> 16)
      ++a.n_tchunks;
    else
      a.lin_idx[k++] = int8_t(c);
  }
  a.nbuf = acc_buffers(b->n_agen);
  a.acol = a.nbuf * kMaxN;
  a.td_col = b->td_col;
  a.td_bytes = b->td_bytes;
  a.c0 = b->c0;
  a.td = reinterpret_cast<const int4*>(b->td);
  a.tdab = reinterpret_cast<const float2*>(b->tdab);
  a.row = reinterpret_cast<const int4*>(b->row);
  a.bimg = static_cast<const uint8_t*>(b->bimg);
  a.box = b->box;
  a.err = b->err;
  a.wait_ns = kWaitNs;
  for (int c = 0; c < b->n_chunks; ++c)
    a.chunk[c] = make_int4(b->chunk[4 * c], b->chunk[4 * c + 1], b->chunk[4 * c + 2], b->chunk[4 * c + 3]);
  const int64_t tiles = (P + kTile - 1) / kTile;
  const unsigned grid = unsigned(tiles < sms ? tiles : sms);
  const size_t smem = size_t(smem_layout(b->n_phi_pad).total);
  const bool x32 = (reinterpret_cast<uintptr_t>(x) & 31) == 0 && ldx % 4 == 0;
  if (x32)
    blocked_tc_kernel<true><<<grid, kThreads, smem, smx::as_stream(stream)>>>(a);
  else
    blocked_tc_kernel<false><<<grid, kThreads, smem, smx::as_stream(stream)>>>(a);
  SMX_LAUNCH_CHECK("smx_blocked_tc_eval");
  return SMX_OK;
}
