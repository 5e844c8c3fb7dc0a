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

#include "common.cuh"

namespace {

constexpr int kMaxG = 24;  // max degree of a pair handled by the set-up kernels

// phi_{n+1} = alpha_n z phi_n - beta_n phi_{n-1}, phi_0 = 1, phi_{-1} = 0.
__host__ __device__ inline void rec_coeffs(int fam, int n, double* a, double* b) {
  if (fam == 0) {  // Legendre: P_{n+1} = ((2n+1) z P_n - n P_{n-1}) / (n+1)
    *a = double(2 * n + 1) / double(n + 1);
    *b = double(n) / double(n + 1);
  } else {  // Hermite, psi_n = H_n / sqrt(2^n n!)
    *a = sqrt(2.0 / double(n + 1));
    *b = sqrt(double(n) / double(n + 1));
  }
}

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
        double v[kMaxG];
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

__global__ void spectral_scatter_kernel(int64_t R, int dout, const int32_t* __restrict__ ids,
                                        const double* __restrict__ G, double* __restrict__ C) {
  const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (idx >= R * dout) return;
  const int64_t r = idx / dout;
  const int o = int(idx - r * dout);
  atomicAdd(&C[int64_t(ids[r]) * dout + o], G[idx]);
}

// --- FP32 evaluation -----------------------------------------------------------------------
// One thread per point.  Shared memory: hot basis table HB[slot][TP] and the
// prefix products VP[slot][TP] of the hot entries that cold entries extend.
// Hot entries are visited in DFS pre-order; the running products of the
// current path live in registers st1..st8 (depth is warp-uniform).
// Cold entries are grouped by their cold (last) dimension, whose x column is
// streamed once; contribution c * VP[prefix] * phi_g(z).
struct SpecArgs {
  int d_in, dout, n_hot_slots, n_vp, n_hot_dims, n_tape, n_cold_groups, n_cold, max_depth;
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int32_t* tape;
  const float* tape_c;
  const int32_t* cold_dim;
  const int32_t* cold_gmax;
  const int32_t* cold_off;
  const int32_t* cold_ent;
  const float* cold_c;
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

__constant__ float c_alpha[2][kMaxG];
__constant__ float c_beta[2][kMaxG];

template <int DO>
__global__ void __launch_bounds__(128) spectral_eval_kernel(SpecArgs a, const double* __restrict__ x, int64_t P,
                                                            int64_t ldx, float* __restrict__ y, int o0) {
  extern __shared__ float sm[];
  const int TP = blockDim.x;
  float* HB = sm;                              // [n_hot_slots][TP]
  float* VP = sm + size_t(a.n_hot_slots) * TP; // [n_vp][TP]
  const int tid = threadIdx.x;
  const int64_t p = blockIdx.x * int64_t(TP) + tid;
  const bool live = p < P;
  const double* xp = x + (live ? p : 0) * ldx;

  // hot basis table
  for (int h = 0; h < a.n_hot_dims; ++h) {
    const int dim = a.hot_dim[h], g = a.hot_deg[h], so = a.hot_soff[h];
    const int fm = a.fam[dim];
    const float z = fmaf(a.fam_a[dim], float(xp[dim]), a.fam_b[dim]);
    float pm1 = 0.f, pc = 1.f;
    for (int n = 0; n < g; ++n) {
      const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
      pm1 = pc;
      pc = pn;
      HB[(so + n) * TP + tid] = pc;
    }
  }
  VP[tid] = 1.f;  // slot 0: empty prefix
  __syncthreads();

  // Accumulation: terms go into `blk` with plain FMAs; every 16 hot entries
  // and after every cold group `blk` is added to (acc, comp) by compensated
  // (Kahan) summation, so the rounding of ~1e4 terms stays near 1 ulp.
  float acc[DO], comp[DO], blk[DO];
#pragma unroll
  for (int q = 0; q < DO; ++q) acc[q] = comp[q] = blk[q] = 0.f;
  const int nout = min(DO, a.dout - o0);

  // hot entries, DFS pre-order
  float st1 = 1.f, st2 = 1.f, st3 = 1.f, st4 = 1.f, st5 = 1.f, st6 = 1.f, st7 = 1.f, st8 = 1.f;
  for (int e = 0; e < a.n_tape; ++e) {
    const int w = a.tape[e];
    const int slot = w & 0xffff;
    const int depth = (w >> 16) & 0xf;
    const int vp = w >> 20;
    const float b = HB[slot * TP + tid];
    float pr;
    switch (depth) {
      case 1: st1 = b; pr = st1; break;
      case 2: st2 = st1 * b; pr = st2; break;
      case 3: st3 = st2 * b; pr = st3; break;
      case 4: st4 = st3 * b; pr = st4; break;
      case 5: st5 = st4 * b; pr = st5; break;
      case 6: st6 = st5 * b; pr = st6; break;
      case 7: st7 = st6 * b; pr = st7; break;
      default: st8 = st7 * b; pr = st8; break;
    }
    if (vp) VP[vp * TP + tid] = pr;
    const float* c = a.tape_c + size_t(e) * a.dout + o0;
#pragma unroll
    for (int q = 0; q < DO; ++q)
      if (q < nout) blk[q] = fmaf(c[q], pr, blk[q]);
    if ((e & 15) == 15) {
#pragma unroll
      for (int q = 0; q < DO; ++q) {
        kahan_add(acc[q], comp[q], blk[q]);
        blk[q] = 0.f;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < DO; ++q) {
    kahan_add(acc[q], comp[q], blk[q]);
    blk[q] = 0.f;
  }
  // VP entries are written and read by the same thread only: no barrier needed.

  // cold entries, grouped by cold dimension
  for (int gi = 0; gi < a.n_cold_groups; ++gi) {
    const int dim = a.cold_dim[gi], gmax = a.cold_gmax[gi];
    const int fm = a.fam[dim];
    const float z = fmaf(a.fam_a[dim], float(xp[dim]), a.fam_b[dim]);
    float phi[kMaxG];
    float pm1 = 0.f, pc = 1.f;
#pragma unroll 4
    for (int n = 0; n < gmax; ++n) {
      const float pn = c_alpha[fm][n] * z * pc - c_beta[fm][n] * pm1;
      pm1 = pc;
      pc = pn;
      phi[n] = pc;
    }
    for (int c = a.cold_off[gi]; c < a.cold_off[gi + 1]; ++c) {
      const int w = a.cold_ent[c];
      const int vp = w & 0xffffff;
      const int g = w >> 24;
      const float t = VP[vp * TP + tid] * phi[g - 1];
      const float* cc = a.cold_c + size_t(c) * a.dout + o0;
#pragma unroll
      for (int q = 0; q < DO; ++q)
        if (q < nout) blk[q] = fmaf(cc[q], t, blk[q]);
    }
#pragma unroll
    for (int q = 0; q < DO; ++q) {
      kahan_add(acc[q], comp[q], blk[q]);
      blk[q] = 0.f;
    }
  }
  if (live) {
#pragma unroll
    for (int q = 0; q < DO; ++q)
      if (q < nout) y[p * a.dout + o0 + q] = a.c0[o0 + q] + (acc[q] - comp[q]);
  }
}

bool g_consts_ready = false;

int upload_consts() {
  if (g_consts_ready) return SMX_OK;
  float al[2][kMaxG], be[2][kMaxG];
  for (int f = 0; f < 2; ++f)
    for (int n = 0; n < kMaxG; ++n) {
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

extern "C" int smx_spectral_coefficients(const smx_plan* pl, const int64_t* aoff, const double* A,
                                         const int64_t* first_child, const int64_t* n_child, const int32_t* tdim,
                                         const int32_t* tdeg, int64_t n_lambda, double* G, int32_t* ids, double* C,
                                         int32_t* flag, void* stream) {
  SMX_REQUIRE(pl != nullptr, "smx_spectral_coefficients: null plan");
  SMX_REQUIRE(C && flag && n_lambda >= 1, "smx_spectral_coefficients: bad arguments");
  cudaStream_t st = smx::as_stream(stream);
  const int dout = pl->d_out;
  const int64_t R = pl->n_entries;
  cudaMemsetAsync(C, 0, size_t(n_lambda) * dout * sizeof(double), st);
  // C[root] = offset
  cudaMemcpyAsync(C, pl->offset, size_t(dout) * sizeof(double), cudaMemcpyDeviceToDevice, st);
  SMX_LAUNCH_CHECK("smx_spectral_coefficients init");
  if (pl->n_summands == 0 || R == 0) return SMX_OK;
  SMX_REQUIRE(aoff && A && first_child && n_child && tdim && tdeg && G && ids, "smx_spectral_coefficients: null");
  cudaMemcpyAsync(G, pl->F64, size_t(R) * dout * sizeof(double), cudaMemcpyDeviceToDevice, st);
  const int64_t nt = int64_t(pl->n_summands) * dout;
  spectral_transform_kernel<<<smx::grid_for(nt, 128), 128, 0, st>>>(pl->n_summands, pl->sum_poff, pl->sum_pairs,
                                                                     pl->sum_eoff, pl->pair_deg, aoff, A, dout, G);
  spectral_ids_kernel<<<smx::grid_for(pl->n_summands, 128), 128, 0, st>>>(
      pl->n_summands, pl->sum_poff, pl->sum_pairs, pl->sum_eoff, pl->pair_dim, pl->pair_deg, first_child, n_child,
      tdim, tdeg, ids, flag);
  spectral_scatter_kernel<<<smx::grid_for(R * dout, 256), 256, 0, st>>>(R, dout, ids, G, C);
  SMX_LAUNCH_CHECK("smx_spectral_coefficients");
  return SMX_OK;
}

extern "C" int smx_spectral_eval(const smx_spectral* sp, const double* x, int64_t P, int64_t ldx, float* y,
                                 void* stream) {
  SMX_REQUIRE(sp != nullptr, "smx_spectral_eval: null plan");
  SMX_REQUIRE(P >= 0 && ldx >= sp->d_in && sp->d_out >= 1, "smx_spectral_eval: bad sizes");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y && sp->c0 && sp->fam && sp->fam_a && sp->fam_b, "smx_spectral_eval: null pointer");
  SMX_REQUIRE(sp->max_depth <= 8, "smx_spectral_eval: hot entries deeper than 8 are not supported");
  int rc = upload_consts();
  if (rc) return rc;
  SpecArgs a;
  a.d_in = sp->d_in;
  a.dout = sp->d_out;
  a.n_hot_slots = sp->n_hot_slots;
  a.n_vp = sp->n_vp;
  a.n_hot_dims = sp->n_hot_dims;
  a.n_tape = sp->n_tape;
  a.n_cold_groups = sp->n_cold_groups;
  a.n_cold = sp->n_cold;
  a.max_depth = sp->max_depth;
  a.hot_dim = sp->hot_dim;
  a.hot_deg = sp->hot_deg;
  a.hot_soff = sp->hot_soff;
  a.tape = sp->tape;
  a.tape_c = sp->tape_c;
  a.cold_dim = sp->cold_dim;
  a.cold_gmax = sp->cold_gmax;
  a.cold_off = sp->cold_off;
  a.cold_ent = sp->cold_ent;
  a.cold_c = sp->cold_c;
  a.fam_a = sp->fam_a;
  a.fam_b = sp->fam_b;
  a.fam = sp->fam;
  a.c0 = sp->c0;
  const int TP = 128;
  const size_t smem = size_t(sp->n_hot_slots + sp->n_vp) * TP * sizeof(float);
  SMX_REQUIRE(smem <= 220 * 1024, "smx_spectral_eval: hot table too large for shared memory");
  cudaStream_t st = smx::as_stream(stream);
  static bool attr_set[2] = {false, false};
  for (int o0 = 0; o0 < sp->d_out; o0 += 4) {
    if (sp->d_out == 1) {
      if (!attr_set[0]) {
        cudaFuncSetAttribute(spectral_eval_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr_set[0] = true;
      }
      spectral_eval_kernel<1><<<smx::grid_for(P, TP), TP, smem, st>>>(a, x, P, ldx, y, o0);
    } else {
      if (!attr_set[1]) {
        cudaFuncSetAttribute(spectral_eval_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr_set[1] = true;
      }
      spectral_eval_kernel<4><<<smx::grid_for(P, TP), TP, smem, st>>>(a, x, P, ldx, y, o0);
    }
    SMX_LAUNCH_CHECK("smx_spectral_eval");
  }
  return SMX_OK;
}
