// Mixed-precision path: the interpolant in an orthogonal polynomial basis.
//
// Every tensor-product interpolant I^nu[f] of the combination sum is a
// polynomial whose degree in dimension j is at most nu_j, so the whole sum is
// a polynomial over Lambda:  I(x) = sum_{m in Lambda} c_m prod_j phi_{m_j}(z_j),
// with phi the Legendre polynomials (Leja rules, z in [-1, 1]) or the
// normalised Hermite polynomials (Gauss-Hermite rules).  The coefficients are
// computed once, in FP64, from the nodal values: per pair the Lagrange basis
// is expanded in phi (inverse of the Vandermonde matrix V[j][m] = phi_m(z_j)),
// each summand's tensor of nodal values is transformed mode by mode, and the
// result is scattered into the entries of Lambda.  The cancellation of the
// combination sum (terms ~1e4 times the result) thus happens once in FP64; the
// evaluation sums terms of the size of the result and runs in FP32.
#include <math.h>

#include <algorithm>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "recurrence.cuh"

namespace {

constexpr int kMaxG = 24;     // max degree + 1 handled by the on-device basis-change inversion
constexpr int kMaxRec = 512;  // max degree of the three-term recurrence tables and mode products

using smx::rec_coeffs;

// --- per pair: A = V^{-1}, V[j][m] = phi_m(z_j) --------------------------------------------
__global__ void spectral_pairs_kernel(int n_pairs, const int32_t* __restrict__ pdim, const int32_t* __restrict__ pdeg,
                                      const int32_t* __restrict__ pvoff, const int64_t* __restrict__ aoff,
                                      const double* __restrict__ node, const int32_t* __restrict__ fam,
                                      const double* __restrict__ fa, const double* __restrict__ fb,
                                      double* __restrict__ A, int32_t* __restrict__ flag) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n_pairs) return;
  const int g = pdeg[u], dim = pdim[u], o = pvoff[u];
  const int m = g + 1;
  if (m > kMaxG) {
    atomicExch(flag, 2);
    return;
  }
  double M[kMaxG][2 * kMaxG];
  const int fm = fam[dim];
  for (int j = 0; j < m; ++j) {
    const double z = fa[dim] * node[o + j] + fb[dim];
    double pm1 = 0.0, p = 1.0;
    for (int c = 0; c < m; ++c) {
      M[j][c] = p;
      double al, be;
      rec_coeffs(fm, c, &al, &be);
      const double pn = al * z * p - be * pm1;
      pm1 = p;
      p = pn;
      M[j][m + c] = (j == c) ? 1.0 : 0.0;
    }
  }
  // Gauss-Jordan with partial pivoting on [V | I]
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int r = c + 1; r < m; ++r)
      if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
    if (M[piv][c] == 0.0) {
      atomicExch(flag, 3);
      return;
    }
    if (piv != c)
      for (int q = 0; q < 2 * m; ++q) {
        const double tmp = M[c][q];
        M[c][q] = M[piv][q];
        M[piv][q] = tmp;
      }
    const double inv = 1.0 / M[c][c];
    for (int q = 0; q < 2 * m; ++q) M[c][q] *= inv;
    for (int r = 0; r < m; ++r) {
      if (r == c) continue;
      const double fct = M[r][c];
      if (fct != 0.0)
        for (int q = 0; q < 2 * m; ++q) M[r][q] -= fct * M[c][q];
    }
  }
  double* Au = A + aoff[u];  // A[mm][j] row-major
  for (int mm = 0; mm < m; ++mm)
    for (int j = 0; j < m; ++j) Au[mm * m + j] = M[mm][m + j];
}

// --- per (summand, output): mode products G = (A_1 x ... x A_n) F ---------------------
__global__ void spectral_transform_kernel(int n_sum, const int32_t* __restrict__ poff,
                                          const int32_t* __restrict__ pairs, const int64_t* __restrict__ eoff,
                                          const int32_t* __restrict__ pdeg, const int64_t* __restrict__ aoff,
                                          const double* __restrict__ A, int dout, double* __restrict__ G) {
  const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (tid >= int64_t(n_sum) * dout) return;
  const int s = int(tid / dout);
  const int o = int(tid - int64_t(s) * dout);
  const int q0 = poff[s], n = poff[s + 1] - q0;
  const int64_t e0 = eoff[s], K = eoff[s + 1] - e0;
  double* Gs = G + e0 * dout + o;
  // stride of mode i (last mode fastest)
  int64_t stride = 1;
  for (int i = n - 1; i >= 0; --i) {
    const int u = pairs[q0 + i];
    const int m = pdeg[u] + 1;
    const double* Au = A + aoff[u];
    const int64_t outer = K / (stride * m);
    for (int64_t a = 0; a < outer; ++a) {
      for (int64_t b = 0; b < stride; ++b) {
        const int64_t base = a * stride * m + b;
        double v[kMaxRec];
        for (int j = 0; j < m; ++j) v[j] = Gs[(base + j * stride) * dout];
        for (int mm = 0; mm < m; ++mm) {
          double acc = 0.0;
          for (int j = 0; j < m; ++j) acc = fma(Au[mm * m + j], v[j], acc);
          Gs[(base + mm * stride) * dout] = acc;
        }
      }
    }
    stride *= m;
  }
}

// --- per (summand, entry): id of the multi-index m in Lambda -------------------------------
// Children of a tree entry are sorted by (dim, deg); the entry of m is found by
// descending from the root along m's non-zero components (ascending dim).
__global__ void spectral_ids_kernel(int n_sum, const int32_t* __restrict__ poff, const int32_t* __restrict__ pairs,
                                    const int64_t* __restrict__ eoff, const int32_t* __restrict__ pdim,
                                    const int32_t* __restrict__ pdeg, const int64_t* __restrict__ first_child,
                                    const int64_t* __restrict__ n_child, const int32_t* __restrict__ tdim,
                                    const int32_t* __restrict__ tdeg, int32_t* __restrict__ ids,
                                    int32_t* __restrict__ flag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sum) return;
  const int q0 = poff[s], n = poff[s + 1] - q0;
  const int64_t e0 = eoff[s], K = eoff[s + 1] - e0;
  int mu[SMX_MAX_DEPTH];
  for (int i = 0; i < n; ++i) mu[i] = 0;
  for (int64_t r = 0; r < K; ++r) {
    int64_t cur = 0;
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
      if (mu[i] == 0) continue;
      const int u = pairs[q0 + i];
      const int dd = pdim[u], gg = mu[i];
      int64_t lo = first_child[cur], hi = lo + n_child[cur] - 1;
      int64_t hit = -1;
      while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        const int md = tdim[mid], mg = tdeg[mid];
        if (md == dd && mg == gg) {
          hit = mid;
          break;
        }
        if (md < dd || (md == dd && mg < gg)) lo = mid + 1; else hi = mid - 1;
      }
      if (hit < 0) ok = false; else cur = hit;
    }
    if (!ok) {
      atomicExch(flag, 4);
      ids[e0 + r] = 0;
    } else {
      ids[e0 + r] = int32_t(cur);
    }
    for (int i = n - 1; i >= 0; --i) {
      if (++mu[i] <= pdeg[pairs[q0 + i]]) break;
      mu[i] = 0;
    }
  }
}

// --- deterministic scatter: rows sorted by target entry (stable LSD radix
// sort, 8-bit digits), then one thread per (entry, output) sums its rows in
// row order.  The sum is the same on every run and for every caller.
constexpr int kSortThreads = 256, kSortPer = 8, kSortTile = kSortThreads * kSortPer;

__global__ void sort_hist_kernel(int64_t R, const int32_t* __restrict__ keys, int shift, int nblk,
                                 int32_t* __restrict__ hist) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
  for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
    const int64_t r = base + i;
    if (r < R) atomicAdd(&cnt[(keys[r] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[int64_t(threadIdx.x) * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of hist in (digit, block) order: the first destination of
// every digit of every tile.  One block of 256 threads (thread = digit).
__global__ void sort_scan_kernel(int nblk, int32_t* __restrict__ hist) {
  __shared__ int tot[256];
  const int d = threadIdx.x;
  int s = 0;
  for (int b = 0; b < nblk; ++b) s += hist[int64_t(d) * nblk + b];
  tot[d] = s;
  __syncthreads();
  if (d == 0) {
    int run = 0;
    for (int i = 0; i < 256; ++i) {
      const int t = tot[i];
      tot[i] = run;
      run += t;
    }
  }
  __syncthreads();
  int run = tot[d];
  for (int b = 0; b < nblk; ++b) {
    const int t = hist[int64_t(d) * nblk + b];
    hist[int64_t(d) * nblk + b] = run;
    run += t;
  }
}

// Stable scatter of one tile: the rows are taken in order (rounds of 256,
// warps in order, lanes in order), each placed after the earlier rows of its
// digit.  vin == nullptr: the values are the row indices.
__global__ void sort_scatter_kernel(int64_t R, const int32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                                    int shift, int nblk, const int32_t* __restrict__ off, int32_t* __restrict__ kout,
                                    int32_t* __restrict__ vout) {
  constexpr int kW = kSortThreads / 32;
  __shared__ int cnt[256];
  __shared__ int wcnt[kW][256];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  cnt[t] = off[int64_t(t) * nblk + blockIdx.x];
  for (int i = 0; i < kW; ++i) wcnt[i][t] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
  for (int j = 0; j < kSortPer; ++j) {
    const int64_t r = base + int64_t(j) * kSortThreads + t;
    const bool valid = r < R;
    const int key = valid ? kin[r] : 0;
    const int val = valid ? (vin ? vin[r] : int(r)) : 0;
    const int d = (key >> shift) & 255;
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    unsigned peers = 0;
    if (valid) peers = __match_any_sync(vmask, d);
    const int rank_w = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank_w == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pos = cnt[d] + rank_w;
      for (int w2 = 0; w2 < w; ++w2) pos += wcnt[w2][d];
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    int add = 0;
    for (int w2 = 0; w2 < kW; ++w2) {
      add += wcnt[w2][t];
      wcnt[w2][t] = 0;
    }
    cnt[t] += add;
    __syncthreads();
  }
}

// C[key][o] += sum of G[row][o] over the run of rows of each key (row order).
__global__ void run_sum_kernel(int64_t R, int dout, const int32_t* __restrict__ skeys,
                               const int32_t* __restrict__ srows, const double* __restrict__ G, double* __restrict__ C) {
  const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (idx >= R * dout) return;
  const int64_t i = idx / dout;
  const int o = int(idx - i * dout);
  const int key = skeys[i];
  if (i > 0 && skeys[i - 1] == key) return;
  // The rows of one entry cancel (zeta up to ~2e3, their sum ~1e4 times the
  // coefficient), so they are summed with an error-free transformation
  // (Knuth's TwoSum) and the rounding errors added at the end: the
  // coefficients are then accurate to a few units in the last place, which
  // the FP64 evaluation of the orthogonal form needs.
  double s = C[int64_t(key) * dout + o], e = 0.0;
  for (int64_t j = i; j < R && skeys[j] == key; ++j) {
    const double v = G[int64_t(srows[j]) * dout + o];
    const double t = s + v;
    const double bp = t - s;
    e += (s - (t - bp)) + (v - bp);
    s = t;
  }
  C[int64_t(key) * dout + o] = s + e;
}

// --- FP32 evaluation -----------------------------------------------------------------------
// A CTA evaluates 128 points with 512 threads: warp w serves the 32 points of
// point group w % 4 and work segment w / 4.  Each point owns a row of shared
// memory (stride `row` floats, row = 4 mod 32 so 128-bit loads of 8
// consecutive threads hit distinct banks):
//   [0, n_hb)           phi_g(z_d) of the hot dimensions d, g = 1..maxdeg(d)
//   [n_hb, n_hb + n_vp) products of the hot nodes that cold entries extend
//                       (slot n_hb is the empty prefix, = 1)
// The sum over Lambda is organised as
//   hot nodes (pre-order, the path products on a register stack):
//       v_P * (c_P + sum over runs of hot leaf children c * phi)
//   cold groups (one cold dimension d, its column of x read once):
//       sum over runs (degree g) of phi_g(z_d) * (sum of c * prefix product)
// where every run is a 4-aligned range of row slots with its coefficients
// stored contiguously: one LDS.128 and one warp-uniform LDG.128 feed 4 FMAs.
constexpr int kSeg = 4;
constexpr int kTP = 128;
constexpr int kThreads = kSeg * kTP;

struct SpecArgs {
  int d_in, dout, dstride, row, n_hb, n_vp, n_hot_dims, n_nodes, n_cold_groups;
  int node_seg[kSeg + 1];
  int cold_seg[kSeg + 1];
  int block_seg[kSeg + 1];
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int4* node;
  const float* node_c;
  const int4* cold;
  const float2* cold_ab;
  const int4* blk_dims;
  const int4* blk_run;
  const float4* blk_ab;
  const int4* run;
  const float* coef;
  const float* fam_a;
  const float* fam_b;
  const int32_t* fam;
  const float* c0;
};

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// x coordinate in FP32; infinities become NaN, so that a non-finite
// coordinate makes the point's value NaN as in the FP64 path (whose
// barycentric weights 1/(x - node) then vanish and normalise to 0/0).
__device__ __forceinline__ float x32(double v) {
  const float f = static_cast<float>(v);
  return fabsf(f) == __int_as_float(0x7f800000) ? __int_as_float(0x7fc00000) : f;
}

__constant__ float c_alpha[2][kMaxRec];
__constant__ float c_beta[2][kMaxRec];

// s[q] = sum over the run's slots of coef * row value (runs are at most 32
// slots long, so each is a short FP32 chain; callers add the run sums with
// compensation).
template <int DO>
__device__ __forceinline__ void dot_run(const float* __restrict__ Rw, const float* __restrict__ coef, int4 r,
                                        int dstride, int o0, float (&s)[DO]) {
  const float4* T = reinterpret_cast<const float4*>(Rw + r.x);
  const int n4 = r.y >> 2;
  if constexpr (DO == 1) {
    const float4* Cq = reinterpret_cast<const float4*>(coef + r.z);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll 2
    for (int k = 0; k < n4; ++k) {
      const float4 t = T[k];
      const float4 c = __ldg(Cq + k);
      s0 = fmaf(c.x, t.x, s0);
      s1 = fmaf(c.y, t.y, s1);
      s0 = fmaf(c.z, t.z, s0);
      s1 = fmaf(c.w, t.w, s1);
    }
    s[0] = s0 + s1;
  } else {
#pragma unroll
    for (int q = 0; q < DO; ++q) s[q] = 0.f;
    const float* Cb = coef + r.z + o0;
    for (int k = 0; k < n4; ++k) {
      const float4 t = T[k];
      const float4 c0 = __ldg(reinterpret_cast<const float4*>(Cb + (4 * k + 0) * dstride));
      const float4 c1 = __ldg(reinterpret_cast<const float4*>(Cb + (4 * k + 1) * dstride));
      const float4 c2 = __ldg(reinterpret_cast<const float4*>(Cb + (4 * k + 2) * dstride));
      const float4 c3 = __ldg(reinterpret_cast<const float4*>(Cb + (4 * k + 3) * dstride));
      const float cs[4][4] = {{c0.x, c0.y, c0.z, c0.w}, {c1.x, c1.y, c1.z, c1.w},
                              {c2.x, c2.y, c2.z, c2.w}, {c3.x, c3.y, c3.z, c3.w}};
      const float ts[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
      for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int q = 0; q < DO; ++q) s[q] = fmaf(cs[l][q], ts[l], s[q]);
    }
  }
}

// One tile of 128 points of one plan (body shared by the single-plan kernel
// and the multi-plan batch kernel of the serving loop).
template <int DO>
__device__ __forceinline__ void spectral_eval_tile(const SpecArgs& a, const double* __restrict__ x, int64_t P,
                                                   int64_t ldx, float* __restrict__ y, int o0, int64_t tile,
                                                   float* sm) {
  float* RED = sm + size_t(a.row) * kTP;  // [kSeg][DO][2][kTP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int seg = warp / (kTP / 32);
  const int pl = (warp % (kTP / 32)) * 32 + lane;
  const int64_t p = tile * int64_t(kTP) + pl;
  const bool live = p < P;
  const double* __restrict__ xp = x + (live ? p : 0) * ldx;
  float* Rw = sm + size_t(pl) * a.row;

  // phase 0: hot basis values; constant and padding slots
  for (int h = seg; h < a.n_hot_dims; h += kSeg) {
    const int dim = a.hot_dim[h], g = a.hot_deg[h], so = a.hot_soff[h];
    const int fm = a.fam[dim];
    const float z = fmaf(a.fam_a[dim], x32(xp[dim]), a.fam_b[dim]);
    float pm1 = 0.f, pc = 1.f;
    for (int n = 0; n < g; ++n) {
      const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
      pm1 = pc;
      pc = pn;
      Rw[so + n] = pc;
    }
  }
  if (seg == 0) {
    // the prefix slots start at 0 (phase 1 writes them): the last run of hot
    // leaves may extend past n_hb with zero coefficients and must not meet
    // stale shared memory (a NaN pattern there would survive the zero)
    Rw[a.n_hb] = 1.f;
    for (int i = a.n_hb + 1; i < a.row; ++i) Rw[i] = 0.f;
  }
  __syncthreads();

  float acc[DO], comp[DO];
#pragma unroll
  for (int q = 0; q < DO; ++q) acc[q] = comp[q] = 0.f;

  // phase 1: hot nodes of this segment
  {
    float st1 = 1.f, st2 = 1.f, st3 = 1.f, st4 = 1.f, st5 = 1.f, st6 = 1.f, st7 = 1.f, st8 = 1.f;
    for (int i = a.node_seg[seg]; i < a.node_seg[seg + 1]; ++i) {
      const int4 nd = __ldg(a.node + i);
      const int slot = nd.x & 0xffff;
      const int depth = nd.x >> 16;
      float v;
      if (depth == 0) {
        v = 1.f;
      } else {
        const float b = Rw[slot];
        switch (depth) {
          case 1: st1 = b; v = st1; break;
          case 2: st2 = st1 * b; v = st2; break;
          case 3: st3 = st2 * b; v = st3; break;
          case 4: st4 = st3 * b; v = st4; break;
          case 5: st5 = st4 * b; v = st5; break;
          case 6: st6 = st5 * b; v = st6; break;
          case 7: st7 = st6 * b; v = st7; break;
          default: st8 = st7 * b; v = st8; break;
        }
      }
      if (nd.y >= 0) Rw[nd.y] = v;
      float s[DO], sc[DO];
#pragma unroll
      for (int q = 0; q < DO; ++q) {
        s[q] = (q < a.dout - o0) ? __ldg(a.node_c + size_t(i) * a.dstride + o0 + q) : 0.f;
        sc[q] = 0.f;
      }
      for (int r = nd.z; r < nd.w; ++r) {
        float t[DO];
        dot_run<DO>(Rw, a.coef, __ldg(a.run + r), a.dstride, o0, t);
#pragma unroll
        for (int q = 0; q < DO; ++q) kahan_add(s[q], sc[q], t[q]);
      }
#pragma unroll
      for (int q = 0; q < DO; ++q) kahan_add(acc[q], comp[q], v * (s[q] - sc[q]));
    }
  }
  __syncthreads();  // prefix products complete

  // phase 2a: cold blocks of this segment (d_out = 1).  A block is 4 cold
  // dimensions whose entries all have degree 1, so their contribution is
  //   sum_j phi_1(z_j) * sum_s c[s][j] * prefix[s]
  // over one common run of prefix slots: one LDS.128 of prefix products and 4
  // warp-uniform LDG.128 of coefficients feed 16 FMAs.
  if constexpr (DO == 1) {
    const int b0 = a.block_seg[seg], b1 = a.block_seg[seg + 1];
    float bsum = 0.f;
    int4 dn = b0 < b1 ? __ldg(a.blk_dims + b0) : make_int4(0, 0, 0, 0);
    double xn0 = xp[dn.x], xn1 = xp[dn.y], xn2 = xp[dn.z], xn3 = xp[dn.w];
    for (int bi = b0; bi < b1; ++bi) {
      const double x0 = xn0, x1 = xn1, x2 = xn2, x3 = xn3;
      if (bi + 8 < b1) {
        const int4 pd = __ldg(a.blk_dims + bi + 8);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(xp + pd.x));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(xp + pd.w));
      }
      if (bi + 1 < b1) {
        dn = __ldg(a.blk_dims + bi + 1);
        xn0 = xp[dn.x];
        xn1 = xp[dn.y];
        xn2 = xp[dn.z];
        xn3 = xp[dn.w];
      }
      const float4 ca = __ldg(a.blk_ab + 2 * bi), cb = __ldg(a.blk_ab + 2 * bi + 1);
      const int4 rr = __ldg(a.blk_run + bi);
      const float4* T = reinterpret_cast<const float4*>(Rw + rr.x);
      const float4* Cq = reinterpret_cast<const float4*>(a.coef + rr.z);
      float u0 = 0.f, u1 = 0.f, u2 = 0.f, u3 = 0.f;
      for (int k = 0; k < rr.y; ++k) {
        const float4 t = T[k];
        const float4 c0 = __ldg(Cq + 4 * k + 0), c1 = __ldg(Cq + 4 * k + 1);
        const float4 c2 = __ldg(Cq + 4 * k + 2), c3 = __ldg(Cq + 4 * k + 3);
        u0 = fmaf(c0.x, t.x, u0); u1 = fmaf(c0.y, t.x, u1); u2 = fmaf(c0.z, t.x, u2); u3 = fmaf(c0.w, t.x, u3);
        u0 = fmaf(c1.x, t.y, u0); u1 = fmaf(c1.y, t.y, u1); u2 = fmaf(c1.z, t.y, u2); u3 = fmaf(c1.w, t.y, u3);
        u0 = fmaf(c2.x, t.z, u0); u1 = fmaf(c2.y, t.z, u1); u2 = fmaf(c2.z, t.z, u2); u3 = fmaf(c2.w, t.z, u3);
        u0 = fmaf(c3.x, t.w, u0); u1 = fmaf(c3.y, t.w, u1); u2 = fmaf(c3.z, t.w, u2); u3 = fmaf(c3.w, t.w, u3);
      }
      float v = fmaf(ca.x, x32(x0), cb.x) * u0;
      v = fmaf(fmaf(ca.y, x32(x1), cb.y), u1, v);
      v = fmaf(fmaf(ca.z, x32(x2), cb.z), u2, v);
      v = fmaf(fmaf(ca.w, x32(x3), cb.w), u3, v);
      bsum += v;
      if (((bi - b0) & 3) == 3) {
        kahan_add(acc[0], comp[0], bsum);
        bsum = 0.f;
      }
    }
    kahan_add(acc[0], comp[0], bsum);
  }

  // phase 2: cold groups of this segment.  Group descriptor: (dim, first
  // run, end run, max degree | family << 16), affine map (a, b); runs carry
  // their degree in .w and are sorted by it.  The x column of group gi + 16
  // is prefetched into L2, the one of group gi + 1 into registers.
  {
    const int g0 = a.cold_seg[seg], g1 = a.cold_seg[seg + 1];
    int4 cg = g0 < g1 ? __ldg(a.cold + g0) : make_int4(0, 0, 0, 0);
    double xn = g0 < g1 ? xp[cg.x] : 0.0;
    float blk[DO];
#pragma unroll
    for (int q = 0; q < DO; ++q) blk[q] = 0.f;
    for (int gi = g0; gi < g1; ++gi) {
      const int4 cur = cg;
      const double xv = xn;
      const float2 ab = __ldg(a.cold_ab + gi);
      if (gi + 16 < g1) {
        const double* pf = xp + __ldg(&a.cold[gi + 16].x);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pf));
      }
      if (gi + 1 < g1) {
        cg = __ldg(a.cold + gi + 1);
        xn = xp[cg.x];
      }
      const int fm = cur.w >> 16;
      const float z = fmaf(ab.x, x32(xv), ab.y);
      float pm1 = 0.f, pc = 1.f;
      int gcur = 0;
      for (int r = cur.y; r < cur.z; ++r) {
        const int4 rr = __ldg(a.run + r);
        while (gcur < rr.w) {
          const float pn = c_alpha[fm][gcur] * z * pc - c_beta[fm][gcur] * pm1;
          pm1 = pc;
          pc = pn;
          ++gcur;
        }
        float s[DO];
        dot_run<DO>(Rw, a.coef, rr, a.dstride, o0, s);
#pragma unroll
        for (int q = 0; q < DO; ++q) blk[q] = fmaf(pc, s[q], blk[q]);
      }
      if (((gi - g0) & 3) == 3) {
#pragma unroll
        for (int q = 0; q < DO; ++q) {
          kahan_add(acc[q], comp[q], blk[q]);
          blk[q] = 0.f;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < DO; ++q) kahan_add(acc[q], comp[q], blk[q]);
  }

  // phase 3: combine the segments
#pragma unroll
  for (int q = 0; q < DO; ++q) {
    RED[((seg * DO + q) * 2 + 0) * kTP + pl] = acc[q];
    RED[((seg * DO + q) * 2 + 1) * kTP + pl] = comp[q];
  }
  __syncthreads();
  if (seg == 0 && live) {
#pragma unroll
    for (int q = 0; q < DO; ++q) {
      if (q >= a.dout - o0) continue;
      float s = 0.f, cp = 0.f;
      for (int r = 0; r < kSeg; ++r) {
        kahan_add(s, cp, RED[((r * DO + q) * 2 + 0) * kTP + pl]);
        kahan_add(s, cp, -RED[((r * DO + q) * 2 + 1) * kTP + pl]);
      }
      y[p * a.dout + o0 + q] = a.c0[o0 + q] + (s - cp);
    }
  }
}

template <int DO>
__global__ void __launch_bounds__(kThreads, 2) spectral_eval_kernel(SpecArgs a, const double* __restrict__ x,
                                                                     int64_t P, int64_t ldx, float* __restrict__ y,
                                                                     int o0) {
  extern __shared__ __align__(16) float sm[];
  spectral_eval_tile<DO>(a, x, P, ldx, y, o0, blockIdx.x, sm);
}

// Serving: one persistent launch over a table of work items (plan, inputs,
// outputs, output chunk) of different interpolants and batch sizes.  CTAs take
// 128-point tiles from an atomic counter; the tile's item is found by binary
// search over the items' first tiles.
struct WorkItem {
  int plan, o0;
  int64_t tile0, P, ldx;
  const double* x;
  float* y;
};

__global__ void __launch_bounds__(kThreads, 1) spectral_eval_batch_kernel(const SpecArgs* __restrict__ plans,
                                                                           const WorkItem* __restrict__ items,
                                                                           int n_items, int64_t total_tiles,
                                                                           unsigned long long* counter) {
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
    const WorkItem it = items[lo];
    const SpecArgs& a = plans[it.plan];
    if (a.dout == 1)
      spectral_eval_tile<1>(a, it.x, it.P, it.ldx, it.y, it.o0, t - it.tile0, sm);
    else
      spectral_eval_tile<4>(a, it.x, it.P, it.ldx, it.y, it.o0, t - it.tile0, sm);
    __syncthreads();
  }
}

bool g_consts_ready = false;

int upload_consts() {
  if (g_consts_ready) return SMX_OK;
  static float al[2][kMaxRec], be[2][kMaxRec];
  for (int f = 0; f < 2; ++f)
    for (int n = 0; n < kMaxRec; ++n) {
      double a, b;
      rec_coeffs(f, n, &a, &b);
      al[f][n] = float(a);
      be[f][n] = float(b);
    }
  if (cudaMemcpyToSymbol(c_alpha, al, sizeof(al)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_beta, be, sizeof(be)) != cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "spectral: constant upload failed");
  g_consts_ready = true;
  return SMX_OK;
}

}  // namespace

extern "C" int smx_spectral_pairs(int n_pairs, const int32_t* pair_dim, const int32_t* pair_deg,
                                  const int32_t* pair_voff, const int64_t* aoff, const double* node,
                                  const int32_t* fam, const double* fam_a, const double* fam_b, double* A,
                                  int32_t* flag, void* stream) {
  SMX_REQUIRE(n_pairs >= 0, "smx_spectral_pairs: negative size");
  if (n_pairs == 0) return SMX_OK;
  SMX_REQUIRE(pair_dim && pair_deg && pair_voff && aoff && node && fam && fam_a && fam_b && A && flag,
              "smx_spectral_pairs: null pointer");
  spectral_pairs_kernel<<<smx::grid_for(n_pairs, 64), 64, 0, smx::as_stream(stream)>>>(
      n_pairs, pair_dim, pair_deg, pair_voff, aoff, node, fam, fam_a, fam_b, A, flag);
  SMX_LAUNCH_CHECK("smx_spectral_pairs");
  return SMX_OK;
}

namespace {

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

int sort_blocks(int64_t R) { return int((R + kSortTile - 1) / kSortTile); }

}  // namespace

extern "C" size_t smx_spectral_coefficients_workspace(const smx_plan* pl) {
  if (!pl) return 0;
  const int64_t R = std::max<int64_t>(pl->n_entries, 1);
  return 4 * up256(size_t(R) * sizeof(int32_t)) + up256(size_t(256) * sort_blocks(R) * sizeof(int32_t));
}

extern "C" int smx_spectral_coefficients(const smx_plan* pl, const int64_t* aoff, const double* A,
                                         const int64_t* first_child, const int64_t* n_child, const int32_t* tdim,
                                         const int32_t* tdeg, int64_t n_lambda, double* G, int32_t* ids, double* C,
                                         int32_t* flag, void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(pl != nullptr, "smx_spectral_coefficients: null plan");
  SMX_REQUIRE(C && flag && n_lambda >= 1 && n_lambda < (int64_t(1) << 31), "smx_spectral_coefficients: bad arguments");
  cudaStream_t st = smx::as_stream(stream);
  const int dout = pl->d_out;
  const int64_t R = pl->n_entries;
  cudaMemsetAsync(C, 0, size_t(n_lambda) * dout * sizeof(double), st);
  // C[root] = offset
  cudaMemcpyAsync(C, pl->offset, size_t(dout) * sizeof(double), cudaMemcpyDeviceToDevice, st);
  SMX_LAUNCH_CHECK("smx_spectral_coefficients init");
  if (pl->n_summands == 0 || R == 0) return SMX_OK;
  SMX_REQUIRE(aoff && A && first_child && n_child && tdim && tdeg && G && ids, "smx_spectral_coefficients: null");
  SMX_REQUIRE(ws && ws_bytes >= smx_spectral_coefficients_workspace(pl), "smx_spectral_coefficients: workspace");
  SMX_REQUIRE(R < (int64_t(1) << 31), "smx_spectral_coefficients: too many rows");
  cudaMemcpyAsync(G, pl->F64, size_t(R) * dout * sizeof(double), cudaMemcpyDeviceToDevice, st);
  const int64_t nt = int64_t(pl->n_summands) * dout;
  spectral_transform_kernel<<<smx::grid_for(nt, 128), 128, 0, st>>>(pl->n_summands, pl->sum_poff, pl->sum_pairs,
                                                                     pl->sum_eoff, pl->pair_deg, aoff, A, dout, G);
  spectral_ids_kernel<<<smx::grid_for(pl->n_summands, 128), 128, 0, st>>>(
      pl->n_summands, pl->sum_poff, pl->sum_pairs, pl->sum_eoff, pl->pair_dim, pl->pair_deg, first_child, n_child,
      tdim, tdeg, ids, flag);
  // rows sorted by entry (stable), ping-ponging between two key/row buffers
  uint8_t* w = static_cast<uint8_t*>(ws);
  const size_t rb = up256(size_t(R) * sizeof(int32_t));
  int32_t* k0 = reinterpret_cast<int32_t*>(w);
  int32_t* v0 = reinterpret_cast<int32_t*>(w + rb);
  int32_t* k1 = reinterpret_cast<int32_t*>(w + 2 * rb);
  int32_t* v1 = reinterpret_cast<int32_t*>(w + 3 * rb);
  int32_t* hist = reinterpret_cast<int32_t*>(w + 4 * rb);
  const int nblk = sort_blocks(R);
  int bits = 1;
  while (bits < 31 && (int64_t(1) << bits) < n_lambda) ++bits;
  const int passes = (bits + 7) / 8;
  const int32_t* kin = ids;
  const int32_t* vin = nullptr;
  for (int ps = 0; ps < passes; ++ps) {
    int32_t* ko = (ps & 1) ? k1 : k0;
    int32_t* vo = (ps & 1) ? v1 : v0;
    sort_hist_kernel<<<nblk, kSortThreads, 0, st>>>(R, kin, 8 * ps, nblk, hist);
    sort_scan_kernel<<<1, 256, 0, st>>>(nblk, hist);
    sort_scatter_kernel<<<nblk, kSortThreads, 0, st>>>(R, kin, vin, 8 * ps, nblk, hist, ko, vo);
    kin = ko;
    vin = vo;
  }
  run_sum_kernel<<<smx::grid_for(R * dout, 256), 256, 0, st>>>(R, dout, kin, vin, G, C);
  SMX_LAUNCH_CHECK("smx_spectral_coefficients");
  return SMX_OK;
}

namespace {

int check_spec(const smx_spectral* sp, const char* who) {
  if (!sp) return smx::set_error(SMX_ERR_ARG, std::string(who) + ": null plan");
  if (sp->d_out < 1 || !sp->c0 || !sp->fam || !sp->fam_a || !sp->fam_b || !sp->node || !sp->node_c)
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": incomplete plan");
  if (sp->max_depth > 8) return smx::set_error(SMX_ERR_UNSUPPORTED, std::string(who) + ": hot nodes deeper than 8");
  if (sp->row % 4 != 0 || sp->row < sp->n_hb + sp->n_vp || sp->n_vp < 1)
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": bad row");
  if (sp->d_out != 1 && sp->dstride % 4 != 0)
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": coefficient stride not 4-aligned");
  for (int i = 0; i < kSeg; ++i)
    if (sp->node_seg[i] > sp->node_seg[i + 1] || sp->cold_seg[i] > sp->cold_seg[i + 1] ||
        sp->block_seg[i] > sp->block_seg[i + 1])
      return smx::set_error(SMX_ERR_ARG, std::string(who) + ": segments not ordered");
  if (sp->node_seg[0] != 0 || sp->node_seg[kSeg] != sp->n_nodes || sp->cold_seg[0] != 0 ||
      sp->cold_seg[kSeg] != sp->n_cold_groups || sp->block_seg[0] != 0 || sp->block_seg[kSeg] != sp->n_cold_blocks)
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": segments do not cover the plan");
  if (sp->n_cold_blocks && (sp->d_out != 1 || !sp->blk_dims || !sp->blk_run || !sp->blk_ab))
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": cold blocks need d_out = 1");
  return SMX_OK;
}

SpecArgs to_args(const smx_spectral* sp) {
  SpecArgs a;
  a.d_in = sp->d_in;
  a.dout = sp->d_out;
  a.dstride = sp->dstride;
  a.row = sp->row;
  a.n_hb = sp->n_hb;
  a.n_vp = sp->n_vp;
  a.n_hot_dims = sp->n_hot_dims;
  a.n_nodes = sp->n_nodes;
  a.n_cold_groups = sp->n_cold_groups;
  for (int i = 0; i <= kSeg; ++i) {
    a.node_seg[i] = sp->node_seg[i];
    a.cold_seg[i] = sp->cold_seg[i];
    a.block_seg[i] = sp->block_seg[i];
  }
  a.hot_dim = sp->hot_dim;
  a.hot_deg = sp->hot_deg;
  a.hot_soff = sp->hot_soff;
  a.node = reinterpret_cast<const int4*>(sp->node);
  a.node_c = sp->node_c;
  a.cold = reinterpret_cast<const int4*>(sp->cold);
  a.cold_ab = reinterpret_cast<const float2*>(sp->cold_ab);
  a.blk_dims = reinterpret_cast<const int4*>(sp->blk_dims);
  a.blk_run = reinterpret_cast<const int4*>(sp->blk_run);
  a.blk_ab = reinterpret_cast<const float4*>(sp->blk_ab);
  a.run = reinterpret_cast<const int4*>(sp->run);
  a.coef = sp->coef;
  a.fam_a = sp->fam_a;
  a.fam_b = sp->fam_b;
  a.fam = sp->fam;
  a.c0 = sp->c0;
  return a;
}

size_t spec_smem(const smx_spectral* sp) {
  const int DO = sp->d_out == 1 ? 1 : 4;
  return (size_t(sp->row) + size_t(kSeg) * DO * 2) * kTP * sizeof(float);
}

}  // namespace

extern "C" int smx_spectral_eval(const smx_spectral* sp, const double* x, int64_t P, int64_t ldx, float* y,
                                 void* stream) {
  int rc = check_spec(sp, "smx_spectral_eval");
  if (rc) return rc;
  SMX_REQUIRE(P >= 0 && ldx >= sp->d_in, "smx_spectral_eval: bad sizes");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y, "smx_spectral_eval: null pointer");
  rc = upload_consts();
  if (rc) return rc;
  const SpecArgs a = to_args(sp);
  const int DO = sp->d_out == 1 ? 1 : 4;
  const size_t smem = spec_smem(sp);
  SMX_REQUIRE(smem <= 220 * 1024, "smx_spectral_eval: per-point row too large for shared memory");
  cudaStream_t st = smx::as_stream(stream);
  static bool attr_set[2] = {false, false};
  for (int o0 = 0; o0 < sp->d_out; o0 += DO) {
    if (DO == 1) {
      if (!attr_set[0]) {
        cudaFuncSetAttribute(spectral_eval_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr_set[0] = true;
      }
      spectral_eval_kernel<1><<<smx::grid_for(P, kTP), kThreads, smem, st>>>(a, x, P, ldx, y, o0);
    } else {
      if (!attr_set[1]) {
        cudaFuncSetAttribute(spectral_eval_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr_set[1] = true;
      }
      spectral_eval_kernel<4><<<smx::grid_for(P, kTP), kThreads, smem, st>>>(a, x, P, ldx, y, o0);
    }
    SMX_LAUNCH_CHECK("smx_spectral_eval");
  }
  return SMX_OK;
}

extern "C" size_t smx_spectral_eval_batch_workspace(int n_plans, int n_items, int max_d_out) {
  const int chunks = max_d_out <= 1 ? 1 : (max_d_out + 3) / 4;
  return size_t(n_plans) * sizeof(SpecArgs) + size_t(n_items) * chunks * sizeof(WorkItem) + 1024;
}

extern "C" int smx_spectral_eval_batch(const smx_spectral* plans, int n_plans, const smx_work* items, int n_items,
                                       void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(n_plans >= 1 && n_items >= 0 && plans && (n_items == 0 || items) && ws,
              "smx_spectral_eval_batch: bad arguments");
  if (n_items == 0) return SMX_OK;
  int max_dout = 1;
  size_t smem = 0;
  std::vector<SpecArgs> args(n_plans);
  for (int i = 0; i < n_plans; ++i) {
    int rc = check_spec(&plans[i], "smx_spectral_eval_batch");
    if (rc) return rc;
    args[i] = to_args(&plans[i]);
    max_dout = std::max(max_dout, plans[i].d_out);
    smem = std::max(smem, spec_smem(&plans[i]));
  }
  SMX_REQUIRE(smem <= 220 * 1024, "smx_spectral_eval_batch: per-point row too large for shared memory");
  std::vector<WorkItem> work;
  int64_t tiles = 0;
  for (int j = 0; j < n_items; ++j) {
    const smx_work& w = items[j];
    SMX_REQUIRE(w.plan >= 0 && w.plan < n_plans && w.P >= 0 && w.ldx >= plans[w.plan].d_in,
                "smx_spectral_eval_batch: bad work item");
    if (w.P == 0) continue;
    SMX_REQUIRE(w.x && w.y, "smx_spectral_eval_batch: null work pointers");
    const int dout = plans[w.plan].d_out;
    const int DO = dout == 1 ? 1 : 4;
    for (int o0 = 0; o0 < dout; o0 += DO) {
      WorkItem it;
      it.plan = w.plan;
      it.o0 = o0;
      it.tile0 = tiles;
      it.P = w.P;
      it.ldx = w.ldx;
      it.x = w.x;
      it.y = w.y;
      work.push_back(it);
      tiles += (w.P + kTP - 1) / kTP;
    }
  }
  if (work.empty()) return SMX_OK;
  SMX_REQUIRE(ws_bytes >= smx_spectral_eval_batch_workspace(n_plans, n_items, max_dout),
              "smx_spectral_eval_batch: workspace too small");
  int rc = upload_consts();
  if (rc) return rc;
  uint8_t* wsb = static_cast<uint8_t*>(ws);
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(wsb);
  SpecArgs* d_args = reinterpret_cast<SpecArgs*>(wsb + 256);
  WorkItem* d_items = reinterpret_cast<WorkItem*>(wsb + 256 + ((n_plans * sizeof(SpecArgs) + 255) / 256) * 256);
  cudaStream_t st = smx::as_stream(stream);
  cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  cudaMemcpyAsync(d_args, args.data(), n_plans * sizeof(SpecArgs), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(d_items, work.data(), work.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, st);
  SMX_LAUNCH_CHECK("smx_spectral_eval_batch copies");
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(spectral_eval_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  int dev = 0, sms = 0, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spectral_eval_batch_kernel, kThreads, smem);
  const int64_t grid = std::min<int64_t>(tiles, int64_t(std::max(1, sms) * std::max(1, per_sm)));
  spectral_eval_batch_kernel<<<unsigned(grid), kThreads, smem, st>>>(d_args, d_items, int(work.size()), tiles, counter);
  SMX_LAUNCH_CHECK("smx_spectral_eval_batch");
  return SMX_OK;
}

// --- basis-product panel for the tensor-core contraction ------------------------------------
// A[p][j] = prod over the pairs of entry j of phi_g(z_d), for the non-root
// entries of Lambda in DFS pre-order (tape word: basis slot | depth << 16).
// One thread per point and tape segment (blockIdx.y): the per-point basis
// values of all pairs sit in shared memory ([slot][point]) or, for large plans,
// in a global scratch written by panel_basis_kernel; the path products sit on a
// register stack; blocks of 32 columns go through a shared tile so that the
// hi/lo rows are written with coalesced 128-byte stores.  Every segment starts
// at a depth-1 entry: in DFS pre-order it then holds whole subtrees, so its
// stack starts fresh and the segments of one point are independent.
namespace {

// Basis rows grow[slot][p] (stride rstride) of the listed dimensions, one
// thread per point.
__global__ void __launch_bounds__(128) panel_basis_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                          const int32_t* __restrict__ dmax,
                                                          const int32_t* __restrict__ dsoff,
                                                          const float* __restrict__ fam_a,
                                                          const float* __restrict__ fam_b,
                                                          const int32_t* __restrict__ fam,
                                                          const double* __restrict__ x, int64_t P, int64_t ldx,
                                                          float* __restrict__ grow, int64_t rstride) {
  const int64_t p = blockIdx.x * int64_t(128) + threadIdx.x;
  const double* xp = x + (p < P ? p : 0) * ldx;
  for (int h = 0; h < n_dims; ++h) {
    const int dim = dims[h], g = dmax[h], so = dsoff[h];
    const int fm = fam[dim];
    const float z = fmaf(fam_a[dim], x32(xp[dim]), fam_b[dim]);
    float pm1 = 0.f, pc = 1.f;
    for (int n = 0; n < g; ++n) {
      const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
      pm1 = pc;
      pc = pn;
      grow[(so + n) * rstride + p] = pc;
    }
  }
}

// BF16 = true: the hi/lo pair is written as BF16 (round to nearest even) for
// the kind::f16 contraction.
template <bool BF16>
__global__ void __launch_bounds__(128) panel_tf32_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                         const int32_t* __restrict__ dmax,
                                                         const int32_t* __restrict__ dsoff, int n_slots,
                                                         const int32_t* __restrict__ tape, int K,
                                                         const int32_t* __restrict__ seg,
                                                         const float* __restrict__ fam_a,
                                                         const float* __restrict__ fam_b,
                                                         const int32_t* __restrict__ fam, const double* __restrict__ x,
                                                         int64_t P, int64_t ldx, void* __restrict__ Ahi,
                                                         void* __restrict__ Alo, int64_t lda,
                                                         const float* __restrict__ grow, int64_t gstride) {
  extern __shared__ __align__(16) float sm[];
  // basis row: shared memory [n_slots][128], or (large plans) the global
  // scratch [n_slots][gstride] read through L1
  const int64_t rstride = grow ? gstride : 128;
  float* tile = grow ? sm : sm + size_t(n_slots) * 128;  // [32][129]
  float* stk = tile + 32 * 129;                          // [9][128] path products by depth
  const int tid = threadIdx.x;
  // blockIdx.x = segment (the segments of one block of points run side by side
  // and share its basis rows in cache), blockIdx.y strides over point blocks
  const int64_t n_pb = (P + 127) / 128;
  for (int64_t pb = blockIdx.y; pb < n_pb; pb += gridDim.y) {
  const int64_t p0 = pb * 128;
  const float* row = grow ? grow + p0 : sm;
  if (!grow) {
    const int64_t p = p0 + tid;
    const double* xp = x + (p < P ? p : 0) * ldx;
    for (int h = 0; h < n_dims; ++h) {
      const int dim = dims[h], g = dmax[h], so = dsoff[h];
      const int fm = fam[dim];
      const float z = fmaf(fam_a[dim], x32(xp[dim]), fam_b[dim]);
      float pm1 = 0.f, pc = 1.f;
      for (int n = 0; n < g; ++n) {
        const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
        pm1 = pc;
        pc = pn;
        sm[(so + n) * 128 + tid] = pc;
      }
    }
  }
  const int jbeg = seg ? seg[blockIdx.x] : 0, jend = seg ? seg[blockIdx.x + 1] : K;
  // path products by depth: stk[d][tid] = product of the path's first d factors
  // (stk[0] = 1), so an entry of depth d is stk[d - 1] * its basis value with no
  // branch on d
  stk[tid] = 1.f;
  // tiles of up to 32 entries, cut so that each covers one aligned group of 32
  // output columns (column K-1-j): full 128-byte lines of the FP32 rows
  for (int jb = jbeg, jn = 0; jb < jend; jb += jn) {
    jn = min(jend - jb, ((K - jb - 1) & 31) + 1);
    // 8 tape entries at a time: their basis values are loaded together (the
    // loads are independent; only the path products are sequential)
    for (int j = 0; j < jn; j += 8) {
      int w[8];
      float b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) w[u] = j + u < jn ? __ldg(tape + jb + j + u) : 0;
#pragma unroll
      for (int u = 0; u < 8; ++u) b[u] = row[(w[u] & 0xffff) * rstride + tid];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (j + u < jn) {
          const int d = min(max(w[u] >> 16, 1), 8);
          const float v = stk[(d - 1) * 128 + tid] * b[u];
          stk[d * 128 + tid] = v;
          tile[(j + u) * 129 + tid] = v;
        }
      }
    }
    __syncthreads();
    // write-out: thread t -> 4 adjacent columns (quad t % 8 of the tile's
    // 32-column group) of rows t / 8, t / 8 + 16, ...: a warp stores four whole
    // 128-byte FP32 lines (four 64-byte BF16 half lines) per instruction
    {
      const int hi = (K - 1 - jb) & 31;  // group position of the tile's entry c = 0 (column K-1-jb)
      const int lo = hi - jn + 1;        // ... and of its last entry
      const int64_t colbase = int64_t(K - 1 - jb) - hi;
      const int k0 = 4 * (tid & 7);
      if (k0 + 3 >= lo && k0 <= hi) {
        const bool full = k0 >= lo && k0 + 3 <= hi;
        for (int r = tid >> 3; r < 128; r += 16) {
          if (p0 + r >= P) break;
          float v[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int c = hi - (k0 + k);  // tile entry of group column k0 + k
            v[k] = (c >= 0 && c < jn) ? tile[c * 129 + r] : 0.f;
          }
          // reversed column order: descendants (small coefficients) precede their
          // ancestors, so the tensor-memory accumulator grows from small to large
          const int64_t off = (p0 + r) * lda + colbase + k0;
          if constexpr (BF16) {
            __nv_bfloat16 h[4], l[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              h[k] = __float2bfloat16_rn(v[k]);
              l[k] = __float2bfloat16_rn(v[k] - __bfloat162float(h[k]));
            }
            __nv_bfloat16* H = static_cast<__nv_bfloat16*>(Ahi) + off;
            __nv_bfloat16* L = static_cast<__nv_bfloat16*>(Alo) + off;
            if (full) {
              uint2 hp, lp;
              hp.x = uint32_t(__bfloat16_as_ushort(h[0])) | (uint32_t(__bfloat16_as_ushort(h[1])) << 16);
              hp.y = uint32_t(__bfloat16_as_ushort(h[2])) | (uint32_t(__bfloat16_as_ushort(h[3])) << 16);
              lp.x = uint32_t(__bfloat16_as_ushort(l[0])) | (uint32_t(__bfloat16_as_ushort(l[1])) << 16);
              lp.y = uint32_t(__bfloat16_as_ushort(l[2])) | (uint32_t(__bfloat16_as_ushort(l[3])) << 16);
              *reinterpret_cast<uint2*>(H) = hp;
              *reinterpret_cast<uint2*>(L) = lp;
            } else {
#pragma unroll
              for (int k = 0; k < 4; ++k)
                if (k0 + k >= lo && k0 + k <= hi) {
                  H[k] = h[k];
                  L[k] = l[k];
                }
            }
          } else {
            float h[4], l[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              uint32_t hb, lb;
              asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(v[k]));
              h[k] = __uint_as_float(hb);
              asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lb) : "f"(v[k] - h[k]));
              l[k] = __uint_as_float(lb);
            }
            float* H = static_cast<float*>(Ahi) + off;
            float* L = static_cast<float*>(Alo) + off;
            if (full) {
              *reinterpret_cast<float4*>(H) = make_float4(h[0], h[1], h[2], h[3]);
              *reinterpret_cast<float4*>(L) = make_float4(l[0], l[1], l[2], l[3]);
            } else {
#pragma unroll
              for (int k = 0; k < 4; ++k)
                if (k0 + k >= lo && k0 + k <= hi) {
                  H[k] = h[k];
                  L[k] = l[k];
                }
            }
          }
        }
      }
    }
    __syncthreads();
  }
  }
}

}  // namespace

// Basis rows stay in shared memory only while that leaves room for several
// blocks per SM (the tape walk is latency-bound); otherwise they go to a
// point-contiguous global scratch that is read coalesced through L1/L2.
constexpr size_t kPanelSmemRows = 24 * 1024;

extern "C" size_t smx_spectral_panel_workspace(int n_slots, int64_t P) {
  const size_t smem = (size_t(n_slots) * 128 + 32 * 129 + 9 * 128) * sizeof(float);
  if (smem <= kPanelSmemRows) return 0;
  return size_t(n_slots) * size_t((P + 127) / 128 * 128) * sizeof(float);
}

namespace {
template <bool BF16>
int panel_launch(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff, int n_slots,
                 const int32_t* tape, int K, const int32_t* seg, int n_seg, const float* fam_a, const float* fam_b,
                 const int32_t* fam, const double* x, int64_t P, int64_t ldx, void* A_hi, void* A_lo, int64_t lda,
                 void* ws, size_t ws_bytes, void* stream, const char* what) {
  SMX_REQUIRE(n_dims >= 0 && n_slots >= 0 && K >= 0 && P >= 0 && lda >= K && n_seg >= 1 && n_seg <= 65535 &&
                  (n_seg == 1 || seg),
              what);
  if (P == 0 || K == 0) return SMX_OK;
  SMX_REQUIRE(dims && dmax && dsoff && tape && fam_a && fam_b && fam && x && A_hi && A_lo, what);
  const size_t need = smx_spectral_panel_workspace(n_slots, P);
  SMX_REQUIRE(ws_bytes >= need && (need == 0 || ws), what);
  float* grow = need ? static_cast<float*>(ws) : nullptr;
  const int64_t gstride = (P + 127) / 128 * 128;
  const size_t smem = (grow ? size_t(32 * 129 + 9 * 128) : size_t(n_slots) * 128 + 32 * 129 + 9 * 128) * sizeof(float);
  int rc = upload_consts();
  if (rc) return rc;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(panel_tf32_kernel<BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  cudaStream_t st = smx::as_stream(stream);
  if (grow)
    panel_basis_kernel<<<smx::grid_for(P, 128), 128, 0, st>>>(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, x, P,
                                                              ldx, grow, gstride);
  const int64_t n_pb = (P + 127) / 128;
  const dim3 grid(n_seg, unsigned(n_pb < 65535 ? n_pb : 65535));
  panel_tf32_kernel<BF16><<<grid, 128, smem, st>>>(n_dims, dims, dmax, dsoff, n_slots, tape, K,
                                                   n_seg > 1 ? seg : nullptr, fam_a, fam_b, fam, x, P, ldx, A_hi,
                                                   A_lo, lda, grow, gstride);
  SMX_LAUNCH_CHECK(what);
  return SMX_OK;
}
}  // namespace

extern "C" int smx_spectral_panel_tf32(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff,
                                       int n_slots, const int32_t* tape, int K, const int32_t* seg, int n_seg,
                                       const float* fam_a, const float* fam_b, const int32_t* fam, const double* x,
                                       int64_t P, int64_t ldx, float* A_hi, float* A_lo, int64_t lda, void* ws,
                                       size_t ws_bytes, void* stream) {
  return panel_launch<false>(n_dims, dims, dmax, dsoff, n_slots, tape, K, seg, n_seg, fam_a, fam_b, fam, x, P, ldx,
                             A_hi, A_lo, lda, ws, ws_bytes, stream, "smx_spectral_panel_tf32");
}

extern "C" int smx_spectral_panel_bf16(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff,
                                       int n_slots, const int32_t* tape, int K, const int32_t* seg, int n_seg,
                                       const float* fam_a, const float* fam_b, const int32_t* fam, const double* x,
                                       int64_t P, int64_t ldx, uint16_t* A_hi, uint16_t* A_lo, int64_t lda, void* ws,
                                       size_t ws_bytes, void* stream) {
  return panel_launch<true>(n_dims, dims, dmax, dsoff, n_slots, tape, K, seg, n_seg, fam_a, fam_b, fam, x, P, ldx,
                            A_hi, A_lo, lda, ws, ws_bytes, stream, "smx_spectral_panel_bf16");
}

// --- backward ---------------------------------------------------------------------------------
namespace {

// Basis values of all listed dimensions for one point into row[slot * stride + t].
__device__ __forceinline__ void basis_row(int n_dims, const int32_t* __restrict__ dims,
                                          const int32_t* __restrict__ dmax, const int32_t* __restrict__ dsoff,
                                          const float* __restrict__ fam_a, const float* __restrict__ fam_b,
                                          const int32_t* __restrict__ fam, const double* __restrict__ xp, float* row,
                                          int64_t stride, int t) {
  for (int h = 0; h < n_dims; ++h) {
    const int dim = dims[h], g = dmax[h], so = dsoff[h];
    const int fm = fam[dim];
    const float z = fmaf(fam_a[dim], x32(xp[dim]), fam_b[dim]);
    float pm1 = 0.f, pc = 1.f;
    for (int n = 0; n < g; ++n) {
      const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
      pm1 = pc;
      pc = pn;
      row[(so + n) * stride + t] = pc;
    }
  }
}

// A^T panel: AT[K-1-j][p] (same reversed column order as the forward panel),
// one thread per point, coalesced along points.  Basis values in the
// point-contiguous global scratch rowg[slot][p]; the tape is read 8 entries
// at a time so that their basis values load together.
__global__ void __launch_bounds__(128) panel_t_tf32_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                           const int32_t* __restrict__ dmax,
                                                           const int32_t* __restrict__ dsoff, int n_slots,
                                                           const int32_t* __restrict__ tape, int K,
                                                           const float* __restrict__ fam_a,
                                                           const float* __restrict__ fam_b,
                                                           const int32_t* __restrict__ fam,
                                                           const double* __restrict__ x, int64_t P, int64_t ldx,
                                                           float* __restrict__ ATh, float* __restrict__ ATl,
                                                           int64_t ldp, float* __restrict__ rowg, int64_t rstride) {
  const int tid = threadIdx.x;
  const int64_t p = blockIdx.x * int64_t(128) + tid;
  const double* xp = x + (p < P ? p : 0) * ldx;
  float* row = rowg + blockIdx.x * int64_t(128) + tid;
  basis_row(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, xp, row, rstride, 0);
  if (p >= P) return;
  // path products by depth (stk[d][tid], stk[0] = 1): an entry of depth d is
  // stk[d - 1] * its basis value, with no branch on d
  __shared__ float stk[9 * 128];
  stk[tid] = 1.f;
  for (int j = 0; j < K; j += 8) {
    int w[8];
    float bb[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) w[u] = j + u < K ? __ldg(tape + j + u) : (1 << 16);
#pragma unroll
    for (int u = 0; u < 8; ++u) bb[u] = row[int64_t(w[u] & 0xffff) * rstride];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int d = min(max(w[u] >> 16, 1), 8);
      const float v = stk[(d - 1) * 128 + tid] * bb[u];
      stk[d * 128 + tid] = v;
      if (j + u < K) {
        uint32_t h, l;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(v - __uint_as_float(h)));
        const int64_t col = K - 1 - (j + u);
        ATh[col * ldp + p] = __uint_as_float(h);
        ATl[col * ldp + p] = __uint_as_float(l);
      }
    }
  }
}

// dL/dx[p][d] = a_d * sum_g phibar(d, g) phi'_g(z_d) with
// phibar(pair) = sum over entries e containing the pair of G[p][e] * (product
// of e's other basis values).  One thread per point, 32 per block: the basis
// values sit in a point-contiguous global scratch (rowg[slot][p], written by
// this kernel and read back coalesced), the adjoints of the block's points in
// shared memory ([n_slots][32]), G in tiles of 32 columns (reversed
// pre-order).  The path of the current entry (depth <= 8) is kept in
// registers: slots s_i, basis values f_i and prefix products q_i; the tape is
// read 8 entries at a time so their basis values load together.
constexpr int kVjpTP = 32;

// GB = false: the adjoints bar[slot][point] of the block's 32 points sit in
// shared memory; GB = true (many basis slots, where that shared memory would
// leave room for only a few warps per SM): they sit in a global scratch
// [n_slots][rstride] beside the basis rows, read and updated through L1/L2.
// The reverse walk over the tape entries [j0, j1) for the 32 points of a
// warp: every entry's G value times the products of the other factors of its
// path goes to the adjoint of each factor's basis slot, bar[slot * BS + tid].
// j0 must be the tape position of a depth-1 entry (or 0): the path state
// starts empty there.
__device__ __forceinline__ void vjp_walk(int j0, int j1, int K, const int32_t* __restrict__ tape,
                                         const float* __restrict__ row, int64_t rstride, const float* __restrict__ G,
                                         int64_t ldg, int64_t p0, int64_t P, float* tile, float* bar, int64_t BS,
                                         int tid) {
  constexpr int TP = kVjpTP;
  int64_t s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, s6 = 0, s7 = 0, s8 = 0;
  float f1 = 1.f, f2 = 1.f, f3 = 1.f, f4 = 1.f, f5 = 1.f, f6 = 1.f, f7 = 1.f, f8 = 1.f;
  float q1 = 1.f, q2 = 1.f, q3 = 1.f, q4 = 1.f, q5 = 1.f, q6 = 1.f, q7 = 1.f;
  for (int jb = j0; jb < j1; jb += 32) {
    const int jn = min(32, j1 - jb);
    __syncthreads();
    // tile[c][r] = G[p0 + r][K - 1 - (jb + c)]: coalesced over the 32 columns
    for (int idx = tid; idx < 32 * TP; idx += TP) {
      const int c = idx & 31, r = idx >> 5;
      tile[c * (TP + 1) + r] = (c < jn && p0 + r < P) ? G[(p0 + r) * ldg + (K - 1 - (jb + c))] : 0.f;
    }
    __syncthreads();
    for (int j = 0; j < jn; j += 8) {
      int w[8];
      float b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) w[u] = j + u < jn ? __ldg(tape + jb + j + u) : 0;
#pragma unroll
      for (int u = 0; u < 8; ++u) b[u] = row[int64_t(w[u] & 0xffff) * rstride];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = min(8, w[u] >> 16);  // 0: padding past the end of the range
        const int64_t sl = (w[u] & 0xffff) * BS + tid;
        switch (k) {
          case 1: s1 = sl; f1 = b[u]; q1 = b[u]; break;
          case 2: s2 = sl; f2 = b[u]; q2 = q1 * b[u]; break;
          case 3: s3 = sl; f3 = b[u]; q3 = q2 * b[u]; break;
          case 4: s4 = sl; f4 = b[u]; q4 = q3 * b[u]; break;
          case 5: s5 = sl; f5 = b[u]; q5 = q4 * b[u]; break;
          case 6: s6 = sl; f6 = b[u]; q6 = q5 * b[u]; break;
          case 7: s7 = sl; f7 = b[u]; q7 = q6 * b[u]; break;
          case 8: s8 = sl; f8 = b[u]; break;
          default: break;
        }
        // adjoints of the path's factors: bar(s_i) += G * prod_{i' != i} f_i'
        float suf = k ? tile[(j + u) * (TP + 1) + tid] : 0.f;
        switch (k) {
          case 8: bar[s8] += q7 * suf; suf *= f8; [[fallthrough]];
          case 7: bar[s7] += q6 * suf; suf *= f7; [[fallthrough]];
          case 6: bar[s6] += q5 * suf; suf *= f6; [[fallthrough]];
          case 5: bar[s5] += q4 * suf; suf *= f5; [[fallthrough]];
          case 4: bar[s4] += q3 * suf; suf *= f4; [[fallthrough]];
          case 3: bar[s3] += q2 * suf; suf *= f3; [[fallthrough]];
          case 2: bar[s2] += q1 * suf; suf *= f2; [[fallthrough]];
          case 1: bar[s1] += suf; break;
          default: break;
        }
      }
    }
  }
}

// dL/dx[p][dim] = a_dim * sum_n bar(slot n of dim) * phi_n'(z) for the point
// of thread tid, the adjoints summed over `nb` copies nbs floats apart.
__device__ __forceinline__ void vjp_dx(int n_dims, const int32_t* __restrict__ dims,
                                       const int32_t* __restrict__ dmax, const int32_t* __restrict__ dsoff,
                                       const float* __restrict__ fam_a, const float* __restrict__ fam_b,
                                       const int32_t* __restrict__ fam, const double* __restrict__ xp,
                                       const float* bar, int64_t BS, int nb, int64_t nbs, int tid,
                                       double* __restrict__ dxp) {
  for (int h = 0; h < n_dims; ++h) {
    const int dim = dims[h], g = dmax[h], so = dsoff[h];
    const int fm = fam[dim];
    const float z = fmaf(fam_a[dim], x32(xp[dim]), fam_b[dim]);
    float pm1 = 0.f, pc = 1.f, dm1 = 0.f, dc = 0.f, acc = 0.f;
    for (int n = 0; n < g; ++n) {
      const float al = c_alpha[fm][n], be = c_beta[fm][n];
      const float pn = al * z * pc - be * pm1;
      const float dn = al * (pc + z * dc) - be * dm1;
      pm1 = pc;
      pc = pn;
      dm1 = dc;
      dc = dn;
      float b = 0.f;
      for (int q = 0; q < nb; ++q) b += bar[q * nbs + (so + n) * BS + tid];
      acc = fmaf(b, dc, acc);
    }
    dxp[dim] = double(fam_a[dim]) * double(acc);
  }
}

template <bool GB>
__global__ void __launch_bounds__(kVjpTP) vjp_x_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                       const int32_t* __restrict__ dmax,
                                                       const int32_t* __restrict__ dsoff, int n_slots,
                                                       const int32_t* __restrict__ tape, int K,
                                                       const float* __restrict__ fam_a,
                                                       const float* __restrict__ fam_b,
                                                       const int32_t* __restrict__ fam, const double* __restrict__ x,
                                                       int64_t P, int64_t ldx, const float* __restrict__ G,
                                                       int64_t ldg, double* __restrict__ dx, int64_t lddx,
                                                       float* __restrict__ rowg, int64_t rstride,
                                                       float* __restrict__ barg) {
  extern __shared__ __align__(16) float sm[];
  constexpr int TP = kVjpTP;
  const int64_t BS = GB ? rstride : TP;              // slot stride of the adjoints
  float* tile = GB ? sm : sm + size_t(n_slots) * TP;  // [32][TP + 1]
  const int tid = threadIdx.x;
  const int64_t p0 = blockIdx.x * int64_t(TP);
  const int64_t p = p0 + tid;
  float* bar = GB ? barg + p0 : sm;                  // bar[slot * BS + tid]
  const double* xp = x + (p < P ? p : 0) * ldx;
  float* row = rowg + p;
  basis_row(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, xp, row, rstride, 0);
  for (int s = 0; s < n_slots; ++s) bar[s * BS + tid] = 0.f;
  vjp_walk(0, K, K, tape, row, rstride, G, ldg, p0, P, tile, bar, BS, tid);
  if (p >= P) return;
  vjp_dx(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, xp, bar, BS, 1, 0, tid, dx + p * lddx);
}

// Tape split into segments (each starting at a depth-1 entry) for more
// parallelism when few points are walked: basis rows first (one thread per
// point), then one warp per (32 points, segment) with its own adjoint copy in
// global memory, then the sum over the copies.
__global__ void __launch_bounds__(128) vjp_rows_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                       const int32_t* __restrict__ dmax,
                                                       const int32_t* __restrict__ dsoff,
                                                       const float* __restrict__ fam_a,
                                                       const float* __restrict__ fam_b,
                                                       const int32_t* __restrict__ fam, const double* __restrict__ x,
                                                       int64_t P, int64_t ldx, float* __restrict__ rowg,
                                                       int64_t rstride) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= rstride) return;
  basis_row(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, x + (p < P ? p : 0) * ldx, rowg + p, rstride, 0);
}

__global__ void __launch_bounds__(kVjpTP) vjp_seg_kernel(int n_slots, const int32_t* __restrict__ tape, int K,
                                                         const int32_t* __restrict__ seg, int64_t P,
                                                         const float* __restrict__ G, int64_t ldg,
                                                         const float* __restrict__ rowg, int64_t rstride,
                                                         float* __restrict__ barg) {
  __shared__ float tile[32 * (kVjpTP + 1)];
  const int tid = threadIdx.x;
  const int64_t p0 = blockIdx.x * int64_t(kVjpTP);
  float* bar = barg + int64_t(blockIdx.y) * n_slots * rstride + p0;
  for (int s = 0; s < n_slots; ++s) bar[s * rstride + tid] = 0.f;
  vjp_walk(seg[blockIdx.y], seg[blockIdx.y + 1], K, tape, rowg + p0 + tid, rstride, G, ldg, p0, P, tile, bar, rstride,
           tid);
}

__global__ void __launch_bounds__(128) vjp_sum_kernel(int n_dims, const int32_t* __restrict__ dims,
                                                      const int32_t* __restrict__ dmax,
                                                      const int32_t* __restrict__ dsoff,
                                                      const float* __restrict__ fam_a,
                                                      const float* __restrict__ fam_b,
                                                      const int32_t* __restrict__ fam, const double* __restrict__ x,
                                                      int64_t P, int64_t ldx, int n_slots, int n_seg,
                                                      const float* __restrict__ barg, int64_t rstride,
                                                      double* __restrict__ dx, int64_t lddx) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= P) return;
  vjp_dx(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, x + p * ldx, barg + p, rstride, n_seg,
         int64_t(n_slots) * rstride, 0, dx + p * lddx);
}

__global__ void coeff_adjoint_kernel(int n_sum, const int32_t* __restrict__ poff, const int32_t* __restrict__ pairs,
                                     const int64_t* __restrict__ eoff, const int32_t* __restrict__ pdeg,
                                     const int64_t* __restrict__ aoff, const double* __restrict__ A,
                                     const int32_t* __restrict__ ids, const double* __restrict__ Cbar, int dout,
                                     double* __restrict__ Fbar) {
  const int64_t tid = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (tid >= int64_t(n_sum) * dout) return;
  const int s = int(tid / dout);
  const int o = int(tid - int64_t(s) * dout);
  const int q0 = poff[s], n = poff[s + 1] - q0;
  const int64_t e0 = eoff[s], K = eoff[s + 1] - e0;
  double* Fs = Fbar + e0 * dout + o;
  for (int64_t r = 0; r < K; ++r) Fs[r * dout] = Cbar[int64_t(ids[e0 + r]) * dout + o];
  int64_t stride = 1;
  for (int i = n - 1; i >= 0; --i) {
    const int u = pairs[q0 + i];
    const int m = pdeg[u] + 1;
    const double* Au = A + aoff[u];
    const int64_t outer = K / (stride * m);
    for (int64_t a = 0; a < outer; ++a) {
      for (int64_t b = 0; b < stride; ++b) {
        const int64_t base = a * stride * m + b;
        double v[kMaxRec];
        for (int mm = 0; mm < m; ++mm) v[mm] = Fs[(base + mm * stride) * dout];
        for (int j = 0; j < m; ++j) {
          double acc = 0.0;
          for (int mm = 0; mm < m; ++mm) acc = fma(Au[mm * m + j], v[mm], acc);
          Fs[(base + j * stride) * dout] = acc;
        }
      }
    }
    stride *= m;
  }
}

}  // namespace

extern "C" size_t smx_spectral_panel_t_workspace(int n_slots, int64_t P) {
  if (n_slots < 0 || P < 0) return 0;
  return size_t(n_slots) * size_t((P + 127) / 128 * 128) * sizeof(float);
}

extern "C" int smx_spectral_panel_t_tf32(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff,
                                         int n_slots, const int32_t* tape, int K, const float* fam_a,
                                         const float* fam_b, const int32_t* fam, const double* x, int64_t P,
                                         int64_t ldx, float* AT_hi, float* AT_lo, int64_t ldp, void* ws,
                                         size_t ws_bytes, void* stream) {
  SMX_REQUIRE(n_dims >= 0 && n_slots >= 0 && K >= 0 && P >= 0 && ldp >= P, "smx_spectral_panel_t_tf32: bad sizes");
  if (P == 0 || K == 0) return SMX_OK;
  SMX_REQUIRE(dims && dmax && dsoff && tape && fam_a && fam_b && fam && x && AT_hi && AT_lo,
              "smx_spectral_panel_t_tf32: null pointer");
  SMX_REQUIRE(ws && ws_bytes >= smx_spectral_panel_t_workspace(n_slots, P),
              "smx_spectral_panel_t_tf32: workspace too small");
  int rc = upload_consts();
  if (rc) return rc;
  const int64_t rstride = (P + 127) / 128 * 128;
  panel_t_tf32_kernel<<<smx::grid_for(P, 128), 128, 0, smx::as_stream(stream)>>>(
      n_dims, dims, dmax, dsoff, n_slots, tape, K, fam_a, fam_b, fam, x, P, ldx, AT_hi, AT_lo, ldp,
      static_cast<float*>(ws), rstride);
  SMX_LAUNCH_CHECK("smx_spectral_panel_t_tf32");
  return SMX_OK;
}

// Adjoints in global scratch once their shared memory would exceed 24 KB per
// 32-point block (fewer than ~8 warps per SM).
static bool vjp_global_bar(int n_slots) { return (size_t(n_slots) * kVjpTP + 32 * (kVjpTP + 1)) * 4 > 24 * 1024; }

extern "C" size_t smx_spectral_vjp_x_workspace(int n_slots, int n_seg, int64_t P) {
  if (n_slots < 0 || P < 0 || n_seg < 0) return 0;
  const size_t rows = size_t(n_slots) * size_t((P + kVjpTP - 1) / kVjpTP * kVjpTP) * sizeof(float);
  if (n_seg > 1) return (1 + size_t(n_seg)) * rows;
  return vjp_global_bar(n_slots) ? 2 * rows : rows;
}

extern "C" int smx_spectral_vjp_x(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff,
                                  int n_slots, const int32_t* tape, int K, const int32_t* seg, int n_seg,
                                  const float* fam_a, const float* fam_b, const int32_t* fam, const double* x,
                                  int64_t P, int64_t ldx, const float* G, int64_t ldg, double* dx, int64_t lddx,
                                  void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(n_dims >= 0 && n_slots >= 0 && K >= 0 && P >= 0 && ldg >= K, "smx_spectral_vjp_x: bad sizes");
  if (n_seg < 1 || !seg) n_seg = 1;
  SMX_REQUIRE(n_seg <= 65535, "smx_spectral_vjp_x: too many segments");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(dims && dmax && dsoff && tape && fam_a && fam_b && fam && x && G && dx, "smx_spectral_vjp_x: null");
  SMX_REQUIRE(ws && ws_bytes >= smx_spectral_vjp_x_workspace(n_slots, n_seg, P),
              "smx_spectral_vjp_x: workspace too small");
  int rc = upload_consts();
  if (rc) return rc;
  const int64_t rstride = (P + kVjpTP - 1) / kVjpTP * kVjpTP;
  float* rowg = static_cast<float*>(ws);
  cudaStream_t st = smx::as_stream(stream);
  if (n_seg > 1) {
    float* barg = rowg + size_t(n_slots) * rstride;
    vjp_rows_kernel<<<smx::grid_for(rstride, 128), 128, 0, st>>>(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, x, P,
                                                                 ldx, rowg, rstride);
    vjp_seg_kernel<<<dim3(unsigned(rstride / kVjpTP), unsigned(n_seg)), kVjpTP, 0, st>>>(n_slots, tape, K, seg, P, G,
                                                                                         ldg, rowg, rstride, barg);
    vjp_sum_kernel<<<smx::grid_for(P, 128), 128, 0, st>>>(n_dims, dims, dmax, dsoff, fam_a, fam_b, fam, x, P, ldx,
                                                          n_slots, n_seg, barg, rstride, dx, lddx);
    SMX_LAUNCH_CHECK("smx_spectral_vjp_x");
    return SMX_OK;
  }
  const bool gb = vjp_global_bar(n_slots);
  const size_t smem = ((gb ? 0 : size_t(n_slots) * kVjpTP) + 32 * (kVjpTP + 1)) * sizeof(float);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(vjp_x_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  if (gb)
    vjp_x_kernel<true><<<smx::grid_for(P, kVjpTP), kVjpTP, smem, st>>>(
        n_dims, dims, dmax, dsoff, n_slots, tape, K, fam_a, fam_b, fam, x, P, ldx, G, ldg, dx, lddx, rowg, rstride,
        rowg + size_t(n_slots) * rstride);
  else
    vjp_x_kernel<false><<<smx::grid_for(P, kVjpTP), kVjpTP, smem, st>>>(
        n_dims, dims, dmax, dsoff, n_slots, tape, K, fam_a, fam_b, fam, x, P, ldx, G, ldg, dx, lddx, rowg, rstride,
        nullptr);
  SMX_LAUNCH_CHECK("smx_spectral_vjp_x");
  return SMX_OK;
}

extern "C" int smx_spectral_coefficients_adjoint(const smx_plan* pl, const int64_t* aoff, const double* A,
                                                 const int32_t* ids, const double* Cbar, double* Fbar,
                                                 void* stream) {
  SMX_REQUIRE(pl != nullptr, "smx_spectral_coefficients_adjoint: null plan");
  if (pl->n_summands == 0 || pl->n_entries == 0) return SMX_OK;
  SMX_REQUIRE(aoff && A && ids && Cbar && Fbar, "smx_spectral_coefficients_adjoint: null pointer");
  const int64_t nt = int64_t(pl->n_summands) * pl->d_out;
  coeff_adjoint_kernel<<<smx::grid_for(nt, 128), 128, 0, smx::as_stream(stream)>>>(
      pl->n_summands, pl->sum_poff, pl->sum_pairs, pl->sum_eoff, pl->pair_deg, aoff, A, ids, Cbar, pl->d_out, Fbar);
  SMX_LAUNCH_CHECK("smx_spectral_coefficients_adjoint");
  return SMX_OK;
}
