// Blocked FP32 evaluator of the orthogonal-polynomial form, one output.
//
// One persistent block of 16 warps per SM walks 128-point tiles.  Per tile:
//   phase 0  Phi[s][.]  basis values of the hot slots            (shared memory)
//   phase 1  Vc[k][.]   values of the prefixes of cold entries   (shared memory)
//   phase 2  every warp runs its own list of work items over all 128 points
//            (lane l holds points l, l+32, l+64, l+96):
//            hot node a:  y += V_a * sum_{(a,s)} c * Phi[s]        (gather form)
//            cold group:  T[4 pts][4 slots] = sum_{k<K} Vc[k] W[k] (staircase
//                         block, 16 FFMA per shared load), then
//                         y += sum_s T[.][s] * phi_s(x)            (x read once)
//   phase 3  per-point sum over the warps in a fixed order, y = c_0 + sum.
// Coefficients and descriptors are read with warp-uniform loads: from the
// block's own copy of the tables in shared memory when they fit beside the
// tile arrays (copied once per launch), else from global memory through L1.
// The lane's 4 points are processed as two FP32 pairs (packed FFMA2/FMUL2).
// x is streamed with L1-bypassing loads (a software L2 prefetch measured slower:
// its per-row requests load the L1 pipeline more than the latency it hides).
// The cancellation-free orthogonal form is summed with Kahan compensation per
// warp and in the final reduction.
#include <math.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "fp_convert.cuh"

namespace {

using smx::f64_to_f32;
using smx::kahan_add;

constexpr int kW = 16;           // warps per block
constexpr int kT = 128;          // points per tile
constexpr int kThr = kW * 32;
constexpr int kHB = kThr / kT;   // thread groups of 128 in phase 0 (one hot dimension each)
constexpr int kRec = 512;        // recurrence table length
constexpr int kColdBit = 1 << 30;
constexpr int kHotPass = 16;     // hot dimensions per thread and pass of phase 0
constexpr int kMaxSplit = 16;    // blocks sharing one tile of the last round

__constant__ float b_alpha[2][kRec];
__constant__ float b_beta[2][kRec];

struct BArgs {
  int n_hs, k_c, n_hot_dims;
  float c0;
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int4* node;      // [n_nodes][3]: {entry offset, entry count, depth, 0}, path[0..3], path[4..7]
  const int4* vc;        // [k_c][3] same format (path only)
  const int4* hot_ent;   // pairs {smem offset, coefficient bits} x 2
  const int4* grp;       // [G][3]: {K, W offset, fast (2: unit maps), slots}, dims, degrees
  const float4* grp_ab;  // [G][2]: affine maps (a, b) of the 4 slots
  const float4* W;       // staircase coefficients, one float4 per prefix row
  const int32_t* warp_off;
  const int32_t* items;
  const float* fa;
  const float* fb;
  const int32_t* fam;
  const int4* hd;     // per hot dimension {dim, degree, slot offset, family} (shared-memory tables only)
  const float2* hab;  // per hot dimension affine map {a, b}                  (shared-memory tables only)
};

__device__ __forceinline__ void ld2_stream(const double* p, double& a, double& b) {
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(a), "=d"(b) : "l"(p));
}

__device__ __forceinline__ void ld4_stream(const double* p, double& a, double& b, double& c, double& d) {
  asm volatile("ld.global.nc.L1::no_allocate.v4.f64 {%0, %1, %2, %3}, [%4];"
               : "=d"(a), "=d"(b), "=d"(c), "=d"(d)
               : "l"(p));
}

__device__ __forceinline__ double ld1_stream(const double* p) {
  double a;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(a) : "l"(p));
  return a;
}

// Table load: shared memory when the block holds its own copy of the tables
// (TS), else a read-only global load.
template <bool TS, typename T>
__device__ __forceinline__ T tl(const T* p) {
  if constexpr (TS)
    return *p;
  else
    return __ldg(p);
}


__device__ __forceinline__ float phi_rec(int fm, float z, int g) {
  float pm1 = 0.f, pc = 1.f;
  for (int n = 0; n < g; ++n) {
    const float pn = b_alpha[fm][n] * z * pc - b_beta[fm][n] * pm1;
    pm1 = pc;
    pc = pn;
  }
  return pc;
}

// Tile point of shared-memory position q: rows are stored as lane-major quads,
// point l + 32 i (lane l) at position 4 l + i.
__device__ __forceinline__ int quad_point(int q) { return 32 * (q & 3) + (q >> 2); }

// Packed FP32 pairs (two lanes of one FFMA2/FMUL2 instruction); each element
// is rounded as the scalar operation would be.
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// Product of the path's basis values for the lane's 4 points, as pairs (0,1), (2,3).
__device__ __forceinline__ void path_value(const float* __restrict__ PH, int4 h0, int4 pa, int4 pb, int q0,
                                           float2& v01, float2& v23) {
  v01 = v23 = make_float2(1.f, 1.f);
  const int path[8] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (q < h0.z) {
      const float4 f = *reinterpret_cast<const float4*>(PH + path[q] + q0);
      v01 = __fmul2_rn(v01, lo2(f));
      v23 = __fmul2_rn(v23, hi2(f));
    }
  }
}

// x values of a cold group's 4 dimensions for the lane's NP points.
template <int NP>
__device__ __forceinline__ void load_x(const double* __restrict__ x, const int64_t (&prow)[NP], int fastx, int4 gd,
                                       int4 gdim, double (&xv)[NP][4]) {
  if (gd.z && fastx == 2) {  // rows 32-byte aligned: one 32-byte load per point
#pragma unroll
    for (int i = 0; i < NP; ++i) ld4_stream(x + prow[i] + gdim.x, xv[i][0], xv[i][1], xv[i][2], xv[i][3]);
  } else if (gd.z && fastx) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      ld2_stream(x + prow[i] + gdim.x, xv[i][0], xv[i][1]);
      ld2_stream(x + prow[i] + gdim.x + 2, xv[i][2], xv[i][3]);
    }
  } else {
    const int dd[4] = {gdim.x, gdim.y, gdim.z, gdim.w};
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) xv[i][j] = ld1_stream(x + prow[i] + dd[j]);
  }
}

// One tile of 32 * NP points of one plan (lane l: points l + 32 i, i < NP),
// shared by the single-plan kernel and the multi-plan batch kernel.
// With split_S > 1 the block runs every split_S-th item (from split_c) of each
// warp's list and leaves its per-point partial sums in part[split_c]; the last
// of the split_S blocks of the tile (counted in *ctr) adds them in order.
//
// Hot-dimension x values of the first phase-0 pass travel between tiles: once
// a warp has finished phase 2 of one tile it issues the loads of the block's
// next tile (xpre, have = true), which then arrive during the other warps'
// phase 2 and the reduction.
template <int NP, bool TS>
__device__ __forceinline__ void blocked_tile(const BArgs& a, const double* __restrict__ x, int64_t P, int64_t ldx,
                                             float* __restrict__ y, int fastx, int64_t tile, float* sm,
                                             double (&xpre)[kHotPass], bool& have, int64_t next,
                                             int split_c = 0, int split_S = 1, float* part = nullptr,
                                             unsigned int* ctr = nullptr) {
  static_assert(NP == 4, "points are processed as two pairs per lane");
  float* PH = sm;
  float* VC = sm + size_t(a.n_hs) * kT;
  float* RS = VC + size_t(a.k_c) * kT;
  float* RC = RS + kW * kT;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q0 = lane * 4;
  const int it0 = tl<TS>(a.warp_off + warp), it1 = tl<TS>(a.warp_off + warp + 1);
  {
    const int64_t p0 = tile * (32 * NP);
    int64_t prow[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) prow[i] = min(p0 + lane + 32 * i, P - 1) * ldx;

    // phase 0: basis values of the hot slots.  Thread (q, hb) handles the hot
    // dimensions hb, hb + kHB, ... of tile point q; its x loads (up to 16 per
    // pass) are all issued before the first is used.
    {
      const int q = threadIdx.x & (kT - 1), hb = threadIdx.x >> 7;
      const double* xp = x + min(p0 + quad_point(q), P - 1) * ldx;
      for (int h0 = 0; h0 < a.n_hot_dims; h0 += kHB * kHotPass) {
        double xh[kHotPass];
        if (h0 == 0 && have) {
#pragma unroll
          for (int r = 0; r < kHotPass; ++r) xh[r] = xpre[r];
        } else {
#pragma unroll
          for (int r = 0; r < kHotPass; ++r) {
            const int h = h0 + hb + kHB * r;
            xh[r] = h < a.n_hot_dims ? __ldg(xp + (TS ? a.hd[h].x : __ldg(a.hot_dim + h))) : 0.0;
          }
        }
#pragma unroll
        for (int r = 0; r < kHotPass; ++r) {
          const int h = h0 + hb + kHB * r;
          if (h >= a.n_hot_dims) break;
          int g, so, fm;
          float fa, fb;
          if constexpr (TS) {
            const int4 d4 = a.hd[h];
            const float2 ab = a.hab[h];
            g = d4.y, so = d4.z, fm = d4.w, fa = ab.x, fb = ab.y;
          } else {
            const int dim = __ldg(a.hot_dim + h);
            g = __ldg(a.hot_deg + h), so = __ldg(a.hot_soff + h), fm = __ldg(a.fam + dim);
            fa = __ldg(a.fa + dim), fb = __ldg(a.fb + dim);
          }
          const float z = fmaf(fa, f64_to_f32(xh[r]), fb);
          float pm1 = 0.f, pc = 1.f;
          for (int n = 0; n < g; ++n) {
            const float pn = b_alpha[fm][n] * z * pc - b_beta[fm][n] * pm1;
            pm1 = pc;
            pc = pn;
            PH[(so + n) * kT + q] = pc;
          }
        }
      }
    }
    __syncthreads();

    // phase 1: prefix rows of the cold entries
    for (int i = threadIdx.x; i < a.k_c * kT; i += kThr) {
      const int k = i >> 7, q = i & (kT - 1);
      const int4 h0 = tl<TS>(a.vc + 3 * k), pa = tl<TS>(a.vc + 3 * k + 1), pb = tl<TS>(a.vc + 3 * k + 2);
      const int path[8] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
      float v = 1.f;
#pragma unroll
      for (int s = 0; s < 8; ++s)
        if (s < h0.z) v *= PH[path[s] + q];
      VC[k * kT + q] = v;
    }
    __syncthreads();

    // phase 2: this warp's items
    float ys[NP], yc[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) ys[i] = yc[i] = 0.f;
    // hot items come first in every warp's list, cold groups after them
    int it = it0 + split_c;
    for (; it < it1; it += split_S) {
      const int code = tl<TS>(a.items + it);
      if (code & kColdBit) break;
        // hot node: gather over its hot entries, times the path product
        const int4 h0 = tl<TS>(a.node + 3 * code), pa = tl<TS>(a.node + 3 * code + 1),
                   pb = tl<TS>(a.node + 3 * code + 2);
        const int4* E = a.hot_ent + (h0.x >> 1);
        const int ne = h0.y >> 1;
        float2 a01 = make_float2(0.f, 0.f), a23 = a01;
#pragma unroll 4
        for (int e = 0; e < ne; ++e) {
          const int4 ee = tl<TS>(E + e);
          const float4 f0 = *reinterpret_cast<const float4*>(PH + ee.x + q0);
          const float4 f1 = *reinterpret_cast<const float4*>(PH + ee.z + q0);
          const float2 c0 = dup2(__int_as_float(ee.y)), c1 = dup2(__int_as_float(ee.w));
          a01 = __ffma2_rn(c0, lo2(f0), a01);
          a23 = __ffma2_rn(c0, hi2(f0), a23);
          a01 = __ffma2_rn(c1, lo2(f1), a01);
          a23 = __ffma2_rn(c1, hi2(f1), a23);
        }
        float2 v01, v23;
        path_value(PH, h0, pa, pb, q0, v01, v23);
        const float2 p01 = __fmul2_rn(v01, a01), p23 = __fmul2_rn(v23, a23);
        const float va[4] = {p01.x, p01.y, p23.x, p23.y};
#pragma unroll
        for (int i = 0; i < NP; ++i) kahan_add(ys[i], yc[i], va[i]);
    }

    // cold groups, software-pipelined: the x values of group n + 1 are loaded
    // while group n is contracted; they are turned into basis values at the
    // start of the next iteration.
    if (it < it1) {
      int g = tl<TS>(a.items + it) & (kColdBit - 1);
      int4 gd = tl<TS>(a.grp + 3 * g), gdim = tl<TS>(a.grp + 3 * g + 1);
      double xv[NP][4];
      load_x<NP>(x, prow, fastx, gd, gdim, xv);
      for (; it < it1; it += split_S) {
        // basis values of this group from the x values that have arrived
        // (ph2[h][j]: slot j of points 2h, 2h + 1)
        float2 ph2[2][4];
        {
          const float4 A = tl<TS>(a.grp_ab + 2 * g), B = tl<TS>(a.grp_ab + 2 * g + 1);
          const float Aa[4] = {A.x, A.y, A.z, A.w}, Bb[4] = {B.x, B.y, B.z, B.w};
          if (gd.z == 2) {  // unit maps (phi_1 = x): the converted coordinates themselves
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
              for (int j = 0; j < 4; ++j)
                ph2[h][j] = make_float2(f64_to_f32(xv[2 * h][j]), f64_to_f32(xv[2 * h + 1][j]));
          } else if (gd.z) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
              for (int j = 0; j < 4; ++j)
                ph2[h][j] = __ffma2_rn(dup2(Aa[j]), make_float2(f64_to_f32(xv[2 * h][j]), f64_to_f32(xv[2 * h + 1][j])),
                                       dup2(Bb[j]));
          } else {
            float ph[NP][4];
            const int4 gdeg = tl<TS>(a.grp + 3 * g + 2);
            const int dd[4] = {gdim.x, gdim.y, gdim.z, gdim.w};
            const int gg[4] = {gdeg.x, gdeg.y, gdeg.z, gdeg.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int fm = gg[j] ? __ldg(a.fam + dd[j]) : 0;
#pragma unroll
              for (int i = 0; i < NP; ++i)
                ph[i][j] = gg[j] ? phi_rec(fm, fmaf(Aa[j], f64_to_f32(xv[i][j]), Bb[j]), gg[j]) : 0.f;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
              for (int j = 0; j < 4; ++j) ph2[h][j] = make_float2(ph[2 * h][j], ph[2 * h + 1][j]);
          }
        }
        // next group: descriptors and x loads in flight during this contraction
        const int4 gdc = gd;
        if (it + split_S < it1) {
          g = tl<TS>(a.items + it + split_S) & (kColdBit - 1);
          gd = tl<TS>(a.grp + 3 * g);
          gdim = tl<TS>(a.grp + 3 * g + 1);
          load_x<NP>(x, prow, fastx, gd, gdim, xv);
        }
        // staircase block T[i][j] = sum_k Vc[k][i] W[k][j], as pairs of points
        // (T2[h][j] = T[2h][j], T[2h + 1][j])
        float2 T2[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int j = 0; j < 4; ++j) T2[h][j] = make_float2(0.f, 0.f);
        const float4* Wg = a.W + (gdc.y >> 2);
        const float* Vk = VC + q0;
#pragma unroll 4
        for (int k = 0; k < gdc.x; ++k) {
          const float4 v = *reinterpret_cast<const float4*>(Vk + k * kT);
          const float4 w = tl<TS>(Wg + k);
          const float ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            T2[0][j] = __ffma2_rn(lo2(v), dup2(ww[j]), T2[0][j]);
            T2[1][j] = __ffma2_rn(hi2(v), dup2(ww[j]), T2[1][j]);
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float2 sacc = make_float2(0.f, 0.f);
#pragma unroll
          for (int j = 0; j < 4; ++j) sacc = __ffma2_rn(T2[h][j], ph2[h][j], sacc);
          kahan_add(ys[2 * h], yc[2 * h], sacc.x);
          kahan_add(ys[2 * h + 1], yc[2 * h + 1], sacc.y);
        }
      }
    }

    // first phase-0 pass of the next tile: its x loads fly during the reduction
    // (written on every path, so that xpre is dead between phase 0 and here)
    have = next >= 0;
    {
      const int q = threadIdx.x & (kT - 1), hb = threadIdx.x >> 7;
      const double* xp = x + min((have ? next : tile) * kT + quad_point(q), P - 1) * ldx;
#pragma unroll
      for (int r = 0; r < kHotPass; ++r) {
        const int h = hb + kHB * r;
        xpre[r] = have && h < a.n_hot_dims ? __ldg(xp + (TS ? a.hd[h].x : __ldg(a.hot_dim + h))) : 0.0;
      }
    }

    // phase 3: per-point sum over the warps, fixed order
    *reinterpret_cast<float4*>(RS + warp * kT + q0) =
        make_float4(ys[0], NP > 1 ? ys[1 % NP] : 0.f, NP > 2 ? ys[2 % NP] : 0.f, NP > 3 ? ys[3 % NP] : 0.f);
    *reinterpret_cast<float4*>(RC + warp * kT + q0) =
        make_float4(yc[0], NP > 1 ? yc[1 % NP] : 0.f, NP > 2 ? yc[2 % NP] : 0.f, NP > 3 ? yc[3 % NP] : 0.f);
    __syncthreads();
    if (threadIdx.x < kT && (threadIdx.x & 3) < NP) {
      const int q = threadIdx.x;
      float s = 0.f, c = 0.f;
      for (int w = 0; w < kW; ++w) {
        kahan_add(s, c, RS[w * kT + q]);
        kahan_add(s, c, -RC[w * kT + q]);
      }
      const int64_t p = p0 + quad_point(q);
      if (split_S == 1) {
        if (p < P) y[p] = a.c0 + (s - c);
      } else {
        part[(2 * split_c) * kT + q] = s;
        part[(2 * split_c + 1) * kT + q] = c;
        __threadfence();
      }
    }
    if (split_S > 1) {
      __shared__ unsigned int s_last;
      __syncthreads();
      if (threadIdx.x == 0) s_last = atomicAdd(ctr, 1u) == unsigned(split_S - 1);
      __syncthreads();
      if (s_last && threadIdx.x < kT && (threadIdx.x & 3) < NP) {
        __threadfence();
        const int q = threadIdx.x;
        float s = 0.f, c = 0.f;
        for (int cc = 0; cc < split_S; ++cc) {
          kahan_add(s, c, __ldcg(part + (2 * cc) * kT + q));
          kahan_add(s, c, -__ldcg(part + (2 * cc + 1) * kT + q));
        }
        const int64_t p = p0 + quad_point(q);
        if (p < P) y[p] = a.c0 + (s - c);
      }
    }
    __syncthreads();
  }
}

// Byte offsets of the tables copied into shared memory (TS), after the tile
// arrays; every table starts on a 16-byte boundary.
struct TabOff {
  int node, vc, hot_ent, grp, grp_ab, W, items, warp_off, hd, hab, end;
  int n_ent16, n_w, n_items;  // 16-byte words of hot_ent, rows of W, work items
};

template <typename T>
__device__ __forceinline__ const T* tab_copy(uint8_t* base, int off, const T* src, int n16) {
  int4* d = reinterpret_cast<int4*>(base + off);
  const int4* s = reinterpret_cast<const int4*>(src);
  for (int i = threadIdx.x; i < n16; i += kThr) d[i] = __ldg(s + i);
  return reinterpret_cast<const T*>(base + off);
}

template <int NP, bool TS>
__global__ void __launch_bounds__(kThr, 1)
    blocked_eval_kernel(BArgs a, TabOff to, const double* __restrict__ x, int64_t P, int64_t ldx,
                        float* __restrict__ y, int fastx, float* __restrict__ part, unsigned int* __restrict__ ctr) {
  extern __shared__ __align__(16) float sm[];
  if constexpr (TS) {
    // the block's own copy of the warp-uniform tables, read once
    uint8_t* tb = reinterpret_cast<uint8_t*>(sm + (size_t(a.n_hs) + a.k_c + 2 * kW) * kT);
    // node, vc and grp rows are 48 bytes, grp_ab rows 32: their spans are exact
    a.node = tab_copy(tb, to.node, a.node, (to.vc - to.node) / 16);
    a.vc = tab_copy(tb, to.vc, a.vc, (to.hot_ent - to.vc) / 16);
    a.hot_ent = tab_copy(tb, to.hot_ent, a.hot_ent, to.n_ent16);
    a.grp = tab_copy(tb, to.grp, a.grp, (to.grp_ab - to.grp) / 16);
    a.grp_ab = tab_copy(tb, to.grp_ab, a.grp_ab, (to.W - to.grp_ab) / 16);
    a.W = tab_copy(tb, to.W, a.W, to.n_w);
    {
      int32_t* d = reinterpret_cast<int32_t*>(tb + to.items);
      for (int i = threadIdx.x; i < to.n_items; i += kThr) d[i] = __ldg(a.items + i);
      a.items = d;
      int32_t* w = reinterpret_cast<int32_t*>(tb + to.warp_off);
      if (threadIdx.x <= kW) w[threadIdx.x] = __ldg(a.warp_off + threadIdx.x);
      a.warp_off = w;
      int4* hd = reinterpret_cast<int4*>(tb + to.hd);
      float2* hab = reinterpret_cast<float2*>(tb + to.hab);
      for (int h = threadIdx.x; h < a.n_hot_dims; h += kThr) {
        const int dim = __ldg(a.hot_dim + h);
        hd[h] = make_int4(dim, __ldg(a.hot_deg + h), __ldg(a.hot_soff + h), __ldg(a.fam + dim));
        hab[h] = make_float2(__ldg(a.fa + dim), __ldg(a.fb + dim));
      }
      a.hd = hd;
      a.hab = hab;
    }
    __syncthreads();
  }
  const int64_t n_tiles = (P + 32 * NP - 1) / (32 * NP);
  const int64_t G = gridDim.x, rounds = n_tiles / G, rem = n_tiles - rounds * G;
  // last round: each remaining tile is shared by S blocks (S = 1 without a full round before it)
  const int S = rounds > 0 && part != nullptr ? int(G / rem < kMaxSplit ? G / rem : kMaxSplit) : 1;
  const int64_t t = rem > 0 ? blockIdx.x / S : rem;
  const int64_t last = t < rem ? rounds * G + t : -1;  // this block's share of the last round
  double xpre[kHotPass];
  bool have = false;
  for (int64_t r = 0; r < rounds; ++r)
    blocked_tile<NP, TS>(a, x, P, ldx, y, fastx, blockIdx.x + r * G, sm, xpre, have,
                         r + 1 < rounds ? blockIdx.x + (r + 1) * G : last);
  if (last < 0) return;
  const int c = int(blockIdx.x - t * S);
  blocked_tile<NP, TS>(a, x, P, ldx, y, fastx, last, sm, xpre, have, -1, c, S, part + t * (2 * kMaxSplit * kT),
                       ctr + t);
}

struct BWork {
  int plan, fastx;
  int64_t tile0, P, ldx;
  const double* x;
  float* y;
};

// Persistent multi-plan launch: blocks take tiles of any work item from a
// shared counter.
__global__ void __launch_bounds__(kThr, 1)
    blocked_eval_batch_kernel(const BArgs* __restrict__ plans, const BWork* __restrict__ items, int n_items,
                              int64_t total_tiles, unsigned long long* counter) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int64_t s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = int64_t(atomicAdd(counter, 1ull));
    __syncthreads();
    const int64_t t = s_tile;
    __syncthreads();
    if (t >= total_tiles) break;
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (items[mid].tile0 <= t) lo = mid; else hi = mid - 1;
    }
    const BWork it = items[lo];
    double xpre[kHotPass];
    bool have = false;
    blocked_tile<4, false>(plans[it.plan], it.x, it.P, it.ldx, it.y, it.fastx, t - it.tile0, sm, xpre, have, -1);
  }
}

std::mutex g_mu;
bool g_ready[64] = {};
int g_sms[64] = {};

int prepare(int* sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return smx::set_error(SMX_ERR_CUDA, "smx_blocked_eval: no current device");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ready[dev]) {
    static float al[2][kRec], be[2][kRec];
    for (int f = 0; f < 2; ++f)
      for (int n = 0; n < kRec; ++n) {
        // phi_{n+1} = alpha_n z phi_n - beta_n phi_{n-1}: Legendre, normalised Hermite
        al[f][n] = f == 0 ? float(double(2 * n + 1) / double(n + 1)) : float(sqrt(2.0 / double(n + 1)));
        be[f][n] = f == 0 ? float(double(n) / double(n + 1)) : float(sqrt(double(n) / double(n + 1)));
      }
    if (cudaMemcpyToSymbol(b_alpha, al, sizeof(al)) != cudaSuccess ||
        cudaMemcpyToSymbol(b_beta, be, sizeof(be)) != cudaSuccess ||
        cudaFuncSetAttribute(blocked_eval_kernel<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024) != cudaSuccess ||
        cudaFuncSetAttribute(blocked_eval_kernel<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024) != cudaSuccess ||
        cudaFuncSetAttribute(blocked_eval_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_blocked_eval: device set-up failed");
    g_ready[dev] = true;
  }
  *sms = g_sms[dev];
  return SMX_OK;
}

size_t smem_of(const smx_blocked* b) {
  return (size_t(b->n_hs) + size_t(b->k_c)) * kT * sizeof(float) + 2 * size_t(kW) * kT * sizeof(float);
}

// Layout of the tables in shared memory (after the tile arrays); end = bytes.
TabOff tab_offsets(const smx_blocked* b) {
  auto up = [](int64_t v) { return int((v + 15) / 16 * 16); };
  TabOff t;
  t.node = 0;
  t.vc = t.node + up(int64_t(b->n_nodes) * 48);
  t.hot_ent = t.vc + up(int64_t(b->k_c) * 48);
  t.grp = t.hot_ent + up(int64_t(b->n_ent) * 4);
  t.grp_ab = t.grp + up(int64_t(b->n_groups) * 48);
  t.W = t.grp_ab + up(int64_t(b->n_groups) * 32);
  t.items = t.W + up(int64_t(b->n_w) * 16);
  t.warp_off = t.items + up(int64_t(b->n_items) * 4);
  t.hd = t.warp_off + up(int64_t(kW + 1) * 4);
  t.hab = t.hd + up(int64_t(b->n_hot_dims) * 16);
  t.end = t.hab + up(int64_t(b->n_hot_dims) * 8);
  t.n_ent16 = b->n_ent / 4;
  t.n_w = b->n_w;
  t.n_items = b->n_items;
  return t;
}

// The tables' sizes are given and they fit beside the tile arrays.
bool tables_in_smem(const smx_blocked* b) {
  if (b->n_ent <= 0 || b->n_w <= 0 || b->n_ent % 4 || !b->node || !b->hot_ent || !b->grp || !b->grp_ab || !b->W ||
      (b->k_c > 0 && !b->vc))
    return false;
  return smem_of(b) + size_t(tab_offsets(b).end) <= 220 * 1024;
}

int check_plan(const smx_blocked* b, const char* what) {
  if (!b || b->d_in <= 0 || b->n_hs < 0 || b->k_c < 0 || b->n_hot_dims < 0 || b->n_items < 0 || !b->warp_off ||
      !b->items || !b->fa || !b->fb || !b->fam ||
      (b->n_hot_dims > 0 && !(b->hot_dim && b->hot_deg && b->hot_soff)) || (b->k_c > 0 && !b->vc) ||
      (b->n_groups > 0 && !(b->grp && b->grp_ab && b->W)))
    return smx::set_error(SMX_ERR_ARG, std::string(what) + ": bad plan");
  if (smem_of(b) > 220 * 1024)
    return smx::set_error(SMX_ERR_UNSUPPORTED, std::string(what) + ": tables exceed shared memory");
  return SMX_OK;
}

BArgs to_args(const smx_blocked* b) {
  BArgs a;
  a.n_hs = b->n_hs;
  a.k_c = b->k_c;
  a.n_hot_dims = b->n_hot_dims;
  a.c0 = b->c0;
  a.hot_dim = b->hot_dim;
  a.hot_deg = b->hot_deg;
  a.hot_soff = b->hot_soff;
  a.node = reinterpret_cast<const int4*>(b->node);
  a.vc = reinterpret_cast<const int4*>(b->vc);
  a.hot_ent = reinterpret_cast<const int4*>(b->hot_ent);
  a.grp = reinterpret_cast<const int4*>(b->grp);
  a.grp_ab = reinterpret_cast<const float4*>(b->grp_ab);
  a.W = reinterpret_cast<const float4*>(b->W);
  a.warp_off = b->warp_off;
  a.items = b->items;
  a.fa = b->fa;
  a.fb = b->fb;
  a.fam = b->fam;
  a.hd = nullptr;
  a.hab = nullptr;
  return a;
}

// 2: rows 32-byte aligned (4 dimensions per load), 1: 16-byte aligned, 0: scalar loads
int fast_x(const double* x, int64_t ldx) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(x);
  if (ldx % 4 == 0 && a % 32 == 0) return 2;
  return (ldx % 2 == 0) && (a % 16 == 0) ? 1 : 0;
}

}  // namespace

extern "C" size_t smx_blocked_smem(const smx_blocked* b) { return b ? smem_of(b) : 0; }

extern "C" size_t smx_blocked_eval_workspace(const smx_blocked* b, int64_t P) {
  (void)b;
  (void)P;
  int sms = 0;
  if (prepare(&sms) != SMX_OK) return 0;
  return size_t(sms) * (2 * kMaxSplit * kT * sizeof(float) + sizeof(unsigned int));
}

extern "C" int smx_blocked_eval(const smx_blocked* b, const double* x, int64_t P, int64_t ldx, float* y, void* ws,
                                size_t ws_bytes, void* stream) {
  int rc = check_plan(b, "smx_blocked_eval");
  if (rc) return rc;
  SMX_REQUIRE(P >= 0 && ldx >= b->d_in, "smx_blocked_eval: bad sizes");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y, "smx_blocked_eval: null pointer");
  int sms = 0;
  rc = prepare(&sms);
  if (rc) return rc;
  // 128-point tiles (96-point tiles measured slower even where they cut the
  // last round of blocks: most per-item work does not scale with the points)
  const int64_t tiles = (P + 127) / 128;
  const unsigned grid = static_cast<unsigned>(tiles < sms ? tiles : sms);
  // scratch of the last-round tile split: partial sums and counters.  (Launches
  // with fewer tiles than SMs are not split: their results must equal the
  // multi-plan batch kernel's, which gives every tile to one block.)
  float* part = nullptr;
  unsigned int* ctr = nullptr;
  if (ws && ws_bytes >= smx_blocked_eval_workspace(b, P) && tiles > sms) {
    part = static_cast<float*>(ws);
    ctr = reinterpret_cast<unsigned int*>(static_cast<char*>(ws) + size_t(sms) * 2 * kMaxSplit * kT * sizeof(float));
    if (cudaMemsetAsync(ctr, 0, size_t(sms) * sizeof(unsigned int), smx::as_stream(stream)) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_blocked_eval: counter reset failed");
  }
  if (tables_in_smem(b)) {
    const TabOff to = tab_offsets(b);
    blocked_eval_kernel<4, true><<<grid, kThr, smem_of(b) + to.end, smx::as_stream(stream)>>>(
        to_args(b), to, x, P, ldx, y, fast_x(x, ldx), part, ctr);
  } else {
    blocked_eval_kernel<4, false><<<grid, kThr, smem_of(b), smx::as_stream(stream)>>>(
        to_args(b), TabOff{}, x, P, ldx, y, fast_x(x, ldx), part, ctr);
  }
  SMX_LAUNCH_CHECK("smx_blocked_eval");
  return SMX_OK;
}

extern "C" size_t smx_blocked_eval_batch_workspace(int n_plans, int n_items) {
  if (n_plans < 0 || n_items < 0) return 0;
  return 256 + (size_t(n_plans) * sizeof(BArgs) + 255) / 256 * 256 + size_t(n_items) * sizeof(BWork);
}

extern "C" int smx_blocked_eval_batch(const smx_blocked* plans, int n_plans, const smx_work* items, int n_items,
                                      void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(n_plans >= 1 && n_items >= 0 && plans && (n_items == 0 || items) && ws,
              "smx_blocked_eval_batch: bad arguments");
  if (n_items == 0) return SMX_OK;
  SMX_REQUIRE(ws_bytes >= smx_blocked_eval_batch_workspace(n_plans, n_items),
              "smx_blocked_eval_batch: workspace too small");
  std::vector<BArgs> args(n_plans);
  size_t smem = 0;
  for (int i = 0; i < n_plans; ++i) {
    int rc = check_plan(&plans[i], "smx_blocked_eval_batch");
    if (rc) return rc;
    args[i] = to_args(&plans[i]);
    smem = std::max(smem, smem_of(&plans[i]));
  }
  std::vector<BWork> work;
  int64_t tiles = 0;
  for (int j = 0; j < n_items; ++j) {
    const smx_work& w = items[j];
    SMX_REQUIRE(w.plan >= 0 && w.plan < n_plans && w.P >= 0 && w.ldx >= plans[w.plan].d_in,
                "smx_blocked_eval_batch: bad work item");
    if (w.P == 0) continue;
    SMX_REQUIRE(w.x && w.y, "smx_blocked_eval_batch: null work pointers");
    BWork it;
    it.plan = w.plan;
    it.fastx = fast_x(w.x, w.ldx);
    it.tile0 = tiles;
    it.P = w.P;
    it.ldx = w.ldx;
    it.x = w.x;
    it.y = w.y;
    work.push_back(it);
    tiles += (w.P + kT - 1) / kT;
  }
  if (work.empty()) return SMX_OK;
  int sms = 0;
  int rc = prepare(&sms);
  if (rc) return rc;
  uint8_t* wsb = static_cast<uint8_t*>(ws);
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(wsb);
  BArgs* d_args = reinterpret_cast<BArgs*>(wsb + 256);
  BWork* d_items = reinterpret_cast<BWork*>(wsb + 256 + (size_t(n_plans) * sizeof(BArgs) + 255) / 256 * 256);
  cudaStream_t st = smx::as_stream(stream);
  cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  cudaMemcpyAsync(d_args, args.data(), args.size() * sizeof(BArgs), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_items, work.data(), work.size() * sizeof(BWork), cudaMemcpyHostToDevice, st);
  SMX_LAUNCH_CHECK("smx_blocked_eval_batch copies");
  const int64_t grid = std::min<int64_t>(tiles, int64_t(std::max(1, sms)));
  blocked_eval_batch_kernel<<<unsigned(grid), kThr, smem, st>>>(d_args, d_items, int(work.size()), tiles, counter);
  SMX_LAUNCH_CHECK("smx_blocked_eval_batch");
  return SMX_OK;
}
