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
//   producer thread     x boxes (8 dimensions x 128 points, FP64) by TMA, with
//                       L2 prefetch ahead, and the chunks' coefficient stages
//                       (bulk copies from the L2-resident image);
//   compute warps       y_p += sum_j T[p][j] x_pj (x converted to FP32 as it
//                       leaves shared memory) and sum_s T[p][s] Phi_s, Kahan-
//                       compensated, then a fixed-order sum over the 4 column
//                       groups.
// The x stream is read once; everything else stays on chip or in L2.  Every
// wait is bounded: on a timeout the block records an error, stops waiting and
// finishes its loops without work, so that every barrier is still reached.
#include <cuda.h>
#include <cudaTypedefs.h>
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
constexpr int kPrefetch = 16;  // x boxes prefetched to L2 ahead of the loads (128 KB per block)
constexpr int kWarpProducer = kComputeWarps, kWarpMMA = kComputeWarps + 1;

__constant__ float t_alpha[2][kRec];
__constant__ float t_beta[2][kRec];

struct TcArgs {
  int64_t P, ldx;
  const double* x;
  float* y;
  int n_td, n_phi, n_phi_pad, n_rows, max_depth, n_agen, n_chunks, n_boxes, lin0, stages, n_x;
  float c0;
  const int4* td;
  const float2* tdab;
  const int4* row;
  const uint8_t* bimg;
  const int32_t* box;
  int* err;
  uint64_t wait_ns;
  int4 chunk[kMaxChunks];  // {N | table << 16, K steps, stage image offset / 16, first slot or x box}
};

struct Bars {
  uint64_t x_full[kXMax], x_empty[kXMax];
  uint64_t b_full[kBStages], b_empty[kBStages];
  uint64_t acc_full[2], acc_empty[2];
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

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
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

__global__ void __launch_bounds__(kThreads, 1)
    blocked_tc_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ TcArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const Smem L = smem_layout(g.n_phi_pad);
  float* phi = reinterpret_cast<float*>(base + L.phi);
  uint8_t* bst = base + L.b;
  uint8_t* xst = base + L.x;
  float* rs = reinterpret_cast<float*>(base + L.rs);
  Bars* bars = reinterpret_cast<Bars*>(base + L.bar);
  volatile int* abort_flag = &bars->abort_flag;
  const int n_x = g.n_x;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n_tiles = (g.P + kTile - 1) / kTile;
  const int64_t G = gridDim.x;
  const int nt = blockIdx.x < n_tiles ? int((n_tiles - blockIdx.x + G - 1) / G) : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < n_x; ++s) {
      mbar_init(&bars->x_full[s], 1);
      mbar_init(&bars->x_empty[s], 4);  // the 4 warps of the column group that reads the box
    }
    for (int s = 0; s < kBStages; ++s) {
      mbar_init(&bars->b_full[s], 1);
      mbar_init(&bars->b_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bars->acc_full[b], 1);
      mbar_init(&bars->acc_empty[b], kComputeWarps);
    }
    mbar_init(&bars->a_full, 1);
    mbar_init(&bars->flush, 1);
    bars->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // constant slot 0 and the padding slots of Phi (never rewritten)
  for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
    phi[i] = 1.f;
    for (int s = g.n_phi; s < g.n_phi_pad; ++s) phi[s * kTile + i] = 0.f;
  }
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
    if (lane == 0) {
      // ---- producer: x boxes and coefficient stages, two independent queues
      const uint64_t total_x = uint64_t(nt) * g.n_boxes, total_b = uint64_t(nt) * g.stages;
      uint64_t ix = 0, ib = 0, pf = 0;
      int cb = 0, jb = 0;
      uint64_t t_last = global_ns();
      while ((ix < total_x || ib < total_b) && !*abort_flag) {
        for (; pf < total_x && pf < ix + kPrefetch; ++pf) {
          const int64_t tile = blockIdx.x + int64_t(pf / g.n_boxes) * G;
          tma_prefetch_2d(&tmx, g.lin0 + kBox * int(pf % g.n_boxes), int(tile * kTile));
        }
        bool prog = false;
        if (ix < total_x) {
          const int s = int(ix % n_x);
          if (ix < uint64_t(n_x) || mbar_test(&bars->x_empty[s], uint32_t((ix / n_x) & 1) ^ 1u)) {
            const int64_t tile = blockIdx.x + int64_t(ix / g.n_boxes) * G;
            mbar_expect_tx(&bars->x_full[s], kBoxBytes);
            tma_load_2d(xst + s * kBoxBytes, &tmx, g.lin0 + kBox * int(ix % g.n_boxes), int(tile * kTile),
                        &bars->x_full[s]);
            ++ix;
            prog = true;
          }
        }
        if (ib < total_b) {
          const int s = int(ib % kBStages);
          if (ib < kBStages || mbar_test(&bars->b_empty[s], uint32_t((ib / kBStages) & 1) ^ 1u)) {
            const int4 ch = g.chunk[cb];
            const uint32_t bytes = uint32_t(ch.x & 0xFFFF) * (kSplits * 32);
            mbar_expect_tx(&bars->b_full[s], bytes);
            bulk_load(bst + s * kBStageMax, g.bimg + int64_t(ch.z) * 16 + int64_t(jb) * bytes, bytes,
                      &bars->b_full[s]);
            ++ib;
            if (++jb == ch.y) {
              jb = 0;
              if (++cb == g.n_chunks) cb = 0;
            }
            prog = true;
          }
        }
        if (prog) {
          t_last = global_ns();
        } else if (global_ns() - t_last > g.wait_ns) {
          atomicExch(g.err, 1);
          *abort_flag = 1;
        }
      }
      if (*abort_flag) {
        // wait (bounded) until the copies already issued have landed
        for (uint64_t u = ix > uint64_t(n_x) ? ix - n_x : 0; u < ix; ++u)
          mbar_wait(&bars->x_full[u % n_x], uint32_t((u / n_x) & 1), nullptr, g.wait_ns);
        for (uint64_t u = ib > kBStages ? ib - kBStages : 0; u < ib; ++u)
          mbar_wait(&bars->b_full[u % kBStages], uint32_t((u / kBStages) & 1), nullptr, g.wait_ns);
      }
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
          const int b = int(gc & 1);
          if (gc >= 2 && !mbar_wait(&bars->acc_empty[b], uint32_t((gc >> 1) & 1) ^ 1u, abort_flag, g.wait_ns)) {
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
            const uint32_t a0 = tmem + uint32_t(kAcol + kSplits * 8 * kk);
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
    // tensor-memory lanes, column group grp = warp / 4)
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
      compute_sync();

      // A = V in tensor memory: warp (qd, grp) writes the K steps grp, grp + 4, ...
      // of its 32 points (lanes), 16 rows per step, three bf16 parts
      for (int kk = grp; kk < g.n_agen; kk += 4) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int r = kk * kStep + j;
          float pv = 0.f;
          if (r < g.n_rows) {
            const int4 rw = __ldg(&g.row[r]);
            const int wv[4] = {rw.x, rw.y, rw.z, rw.w};
            pv = 1.f;
            for (int qq = 0; qq < g.max_depth; ++qq) {
              const int slot = (unsigned(wv[qq >> 1]) >> (16 * (qq & 1))) & 0xFFFF;
              pv *= phi[slot * kTile + pt];
            }
          }
          v[j] = pv;
        }
        uint32_t w[3][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          uint32_t t3[3];
          split3(v[2 * j], v[2 * j + 1], t3);
          w[0][j] = t3[0];
          w[1][j] = t3[1];
          w[2][j] = t3[2];
        }
#pragma unroll
        for (int s = 0; s < 3; ++s) tmem_st8(lane_base + uint32_t(kAcol + kSplits * 8 * kk + 8 * s), w[s]);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      compute_sync();
      if (tid == 0) mbar_arrive(&bars->a_full);

      // contraction of the accumulators: column units of 8 (u = grp, grp + 4, ...)
      float s_acc = 0.f, c_acc = 0.f;
      for (int c = 0; c < g.n_chunks; ++c, ++gc) {
        const int4 ch = g.chunk[c];
        const int N = ch.x & 0xFFFF, table = ch.x >> 16;
        const int b = int(gc & 1);
        wait_ok(&bars->acc_full[b], uint32_t((gc >> 1) & 1));
        ok = __all_sync(0xffffffffu, ok);
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (int u = grp; u < N / 8; u += 4) {
          uint32_t T[8];
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                       : "=r"(T[0]), "=r"(T[1]), "=r"(T[2]), "=r"(T[3]), "=r"(T[4]), "=r"(T[5]), "=r"(T[6]),
                         "=r"(T[7])
                       : "r"(lane_base + uint32_t(b * kMaxN + 8 * u)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          float v;
          if (table) {
            const float* ph = phi + (ch.w + 8 * u) * kTile + pt;
            v = __uint_as_float(T[0]) * ph[0];
#pragma unroll
            for (int j = 1; j < 8; ++j) v = fmaf(__uint_as_float(T[j]), ph[j * kTile], v);
          } else {
            const int box = ch.w + u;
            const uint64_t gb = uint64_t(i) * g.n_boxes + box;
            const int s = int(gb % n_x);
            wait_ok(&bars->x_full[s], uint32_t((gb / n_x) & 1));
            const uint8_t* row = xst + s * kBoxBytes + pt * 64;
            double xv[8];
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              const double2 d2 = *reinterpret_cast<const double2*>(row + ((c4 ^ ((pt >> 1) & 3)) << 4));
              xv[2 * c4] = d2.x;
              xv[2 * c4 + 1] = d2.y;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&bars->x_empty[s]);
            const int mask = __ldg(g.box + box);
            if (mask) {
#pragma unroll
              for (int j = 0; j < 8; ++j)
                if ((mask >> j) & 1) xv[j] = 0.0;
            }
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
        cudaFuncSetAttribute(blocked_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemLimit)) !=
            cudaSuccess ||
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
  if (smem_layout(b->n_phi_pad).n_x == 0)
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_blocked_tc_eval: shared memory");
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
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if ((rc = smx::tc::tensor_map_encoder(&encode))) return rc;
  CUtensorMap tmx;
  cuuint64_t dims[2] = {cuuint64_t(b->d_in), cuuint64_t(P)};
  cuuint64_t strides[1] = {cuuint64_t(ldx) * 8};
  cuuint32_t box[2] = {cuuint32_t(kBox), cuuint32_t(kTile)};
  cuuint32_t estr[2] = {1, 1};
  if (encode(&tmx, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(x), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return smx::set_error(SMX_ERR_CUDA, "smx_blocked_tc_eval: tensor map encoding failed");
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
  a.n_x = smem_layout(b->n_phi_pad).n_x;
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
  blocked_tc_kernel<<<grid, kThreads, smem, smx::as_stream(stream)>>>(tmx, a);
  SMX_LAUNCH_CHECK("smx_blocked_tc_eval");
  return SMX_OK;
}
