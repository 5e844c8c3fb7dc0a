// FP64 evaluation path: the reference's combination technique, evaluated
// with the barycentric basis (src/smolyax/barycentric.py) over an unpadded,
// ragged summand layout.
//
//   basis   : Lt[v][p]   normalised barycentric basis value of slot v at point p
//   contract: y[p][o]    offset[o] + sum_s sum_mu F_s[mu][o] prod_i Lt[pair_i, mu_i][p]
//   jacobian: J[p][o][j] derivative of the same sum (one factor replaced by dLt)
//   integral: Q[o]       offset[o] + sum_r qw(r) F[r][o]
#include <math.h>

#include <algorithm>

#include "common.cuh"

namespace {

constexpr int kMaxN = 4;   // summands with more active dimensions use the generic path
constexpr int kOC = 4;     // outputs accumulated per pass
constexpr int kMaxGridY = 65535;

// --- barycentric weights (barycentric.py:13-31) ---------------------------------------
__global__ void bary_weights_kernel(int n_pairs, const int32_t* __restrict__ deg, const int32_t* __restrict__ voff,
                                    const double* __restrict__ node, double* __restrict__ w) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n_pairs) return;
  const int g = deg[u], o = voff[u];
  for (int b = 0; b <= g; ++b) {
    double acc = 1.0;
    for (int a = 0; a <= g; ++a) {
      double df = __dsub_rn(node[o + a], node[o + b]);
      if (df == 0.0) df = 1.0;
      acc = __dmul_rn(acc, __ddiv_rn(1.0, df));
    }
    w[o + b] = acc;
  }
}

// Normalised barycentric basis of one pair of degree G (no node hit): one
// reciprocal per node difference and one per row sum, kept in registers (FP64
// division is the expensive operation of this kernel on the FP64 pipe).
template <int G>
__device__ __forceinline__ void basis_pair(double xv, const double* __restrict__ nd, const double* __restrict__ bw,
                                           double* __restrict__ Lt, double* __restrict__ dLt, int o, int64_t P,
                                           int64_t p) {
  double r[G + 1], b[G + 1];
  double S = 0.0, Sd = 0.0;
#pragma unroll
  for (int j = 0; j <= G; ++j) {
    r[j] = 1.0 / __dsub_rn(xv, nd[j]);
    b[j] = bw[j] * r[j];
    S += b[j];
    Sd -= b[j] * r[j];
  }
  const double iS = 1.0 / S;
#pragma unroll
  for (int j = 0; j <= G; ++j) {
    const double l = b[j] * iS;
    Lt[int64_t(o + j) * P + p] = l;
    if (dLt) dLt[int64_t(o + j) * P + p] = (-b[j] * r[j]) * iS - l * Sd * iS;
  }
}

// --- basis table (barycentric.py:34-66, normalisation :117; derivative :126-155, :213-219)
__global__ void basis64_kernel(int n_pairs, const int32_t* __restrict__ pdim, const int32_t* __restrict__ pdeg,
                               const int32_t* __restrict__ pvoff, const double* __restrict__ node,
                               const double* __restrict__ bw, const double* __restrict__ x, int64_t P, int64_t ldx,
                               double* __restrict__ Lt, double* __restrict__ dLt, int pairs_per_block) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= P) return;
  const int u0 = blockIdx.y * pairs_per_block;
  const int u1 = min(n_pairs, u0 + pairs_per_block);
  const double* xp = x + p * ldx;
  const double qnan = __longlong_as_double(0x7ff8000000000000LL);
  for (int u = u0; u < u1; ++u) {
    const int g = pdeg[u], o = pvoff[u];
    const double xv = xp[pdim[u]];
    int hits = 0;
    for (int j = 0; j <= g; ++j) hits += (__dsub_rn(xv, node[o + j]) == 0.0);
    if (hits) {
      // one-hot rule: b_j = [x == xi_j], normalised by the number of hits
      for (int j = 0; j <= g; ++j) {
        const double bj = (__dsub_rn(xv, node[o + j]) == 0.0) ? 1.0 : 0.0;
        Lt[int64_t(o + j) * P + p] = bj / double(hits);
        if (dLt) dLt[int64_t(o + j) * P + p] = qnan;
      }
      continue;
    }
    switch (g) {
      case 0: basis_pair<0>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 1: basis_pair<1>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 2: basis_pair<2>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 3: basis_pair<3>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 4: basis_pair<4>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 5: basis_pair<5>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 6: basis_pair<6>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 7: basis_pair<7>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      case 8: basis_pair<8>(xv, node + o, bw + o, Lt, dLt, o, P, p); break;
      default: {
        double S = 0.0, Sd = 0.0;
        for (int j = 0; j <= g; ++j) {
          const double r = 1.0 / __dsub_rn(xv, node[o + j]);
          const double b = bw[o + j] * r;
          S += b;
          Sd -= b * r;
        }
        const double iS = 1.0 / S;
        for (int j = 0; j <= g; ++j) {
          const double r = 1.0 / __dsub_rn(xv, node[o + j]);
          const double b = bw[o + j] * r;
          const double l = b * iS;
          Lt[int64_t(o + j) * P + p] = l;
          if (dLt) dLt[int64_t(o + j) * P + p] = (-b * r) * iS - l * Sd * iS;
        }
      }
    }
  }
}

// --- contraction --------------------------------------------------------------------------
// Level L of a summand with N active pairs: sum over mu_L of l_L[mu_L] * (inner).
// The innermost level reads rows of F.  `dslot` selects a pair whose basis is
// replaced by its derivative table (jacobian); -1 for evaluation.
template <int OC, int L, int N>
__device__ inline void clevel(const double* __restrict__ Lt, const double* __restrict__ dLt, int dslot, int64_t P,
                              int64_t p, const int (&voff)[kMaxN], const int (&deg)[kMaxN],
                              const double* __restrict__ Fs, int dout, int o0, int nout, int64_t row,
                              double (&acc)[OC]) {
  const int g = deg[L];
  const double* lt = (dslot == L ? dLt : Lt) + int64_t(voff[L]) * P + p;
  if constexpr (L == N - 1 && OC == 1) {
    // innermost level of one output: a dot product with the rows of F, as two
    // interleaved chains (even and odd nodes) so that the FP64 FMA latency overlaps
    const double* fr = Fs + row * (g + 1) * dout + o0;
    double a0[OC], a1[OC];
#pragma unroll
    for (int q = 0; q < OC; ++q) a0[q] = a1[q] = 0.0;
    int j = 0;
    for (; j < g; j += 2) {
      const double l0 = lt[int64_t(j) * P], l1 = lt[int64_t(j + 1) * P];
#pragma unroll
      for (int q = 0; q < OC; ++q) {
        if (q < nout) {
          a0[q] = fma(l0, fr[j * dout + q], a0[q]);
          a1[q] = fma(l1, fr[(j + 1) * dout + q], a1[q]);
        }
      }
    }
    if (j == g) {
      const double l0 = lt[int64_t(j) * P];
#pragma unroll
      for (int q = 0; q < OC; ++q)
        if (q < nout) a0[q] = fma(l0, fr[j * dout + q], a0[q]);
    }
#pragma unroll
    for (int q = 0; q < OC; ++q) acc[q] += a0[q] + a1[q];
  } else {
    for (int j = 0; j <= g; ++j) {
      const double l = lt[int64_t(j) * P];
      double sub[OC];
      if constexpr (L == N - 1) {
        const double* fr = Fs + (row * (g + 1) + j) * dout + o0;
#pragma unroll
        for (int q = 0; q < OC; ++q) sub[q] = q < nout ? fr[q] : 0.0;
      } else {
#pragma unroll
        for (int q = 0; q < OC; ++q) sub[q] = 0.0;
        clevel<OC, L + 1, N>(Lt, dLt, dslot, P, p, voff, deg, Fs, dout, o0, nout, row * (g + 1) + j, sub);
      }
#pragma unroll
      for (int q = 0; q < OC; ++q) acc[q] = fma(l, sub[q], acc[q]);
    }
  }
}

// Generic path (any number of pairs): full product per entry.
template <int OC>
__device__ inline void cgeneric(const double* __restrict__ Lt, const double* __restrict__ dLt, int dslot, int64_t P,
                                int64_t p, const int32_t* __restrict__ pairs, int n,
                                const int32_t* __restrict__ pvoff, const int32_t* __restrict__ pdeg,
                                const double* __restrict__ Fs, int64_t K, int dout, int o0, int nout,
                                double (&acc)[OC]) {
  int mu[SMX_MAX_DEPTH];
  for (int i = 0; i < n; ++i) mu[i] = 0;
  for (int64_t r = 0; r < K; ++r) {
    double w = 1.0;
    for (int i = 0; i < n; ++i) {
      const double* t = (i == dslot ? dLt : Lt);
      w *= t[int64_t(pvoff[pairs[i]] + mu[i]) * P + p];
    }
    const double* fr = Fs + r * dout + o0;
#pragma unroll
    for (int q = 0; q < OC; ++q)
      if (q < nout) acc[q] = fma(w, fr[q], acc[q]);
    for (int i = n - 1; i >= 0; --i) {  // row-major increment, last pair fastest
      if (++mu[i] <= pdeg[pairs[i]]) break;
      mu[i] = 0;
    }
  }
}

template <int OC>
__device__ inline void contract_summand(const double* __restrict__ Lt, const double* __restrict__ dLt, int dslot,
                                        int64_t P, int64_t p, const int32_t* __restrict__ pairs, int n,
                                        const int32_t* __restrict__ pvoff, const int32_t* __restrict__ pdeg,
                                        const double* __restrict__ Fs, int64_t K, int dout, int o0, int nout,
                                        double (&acc)[OC]) {
  if (n > kMaxN) {
    cgeneric<OC>(Lt, dLt, dslot, P, p, pairs, n, pvoff, pdeg, Fs, K, dout, o0, nout, acc);
    return;
  }
  int voff[kMaxN], deg[kMaxN];
#pragma unroll
  for (int i = 0; i < kMaxN; ++i) {
    voff[i] = i < n ? pvoff[pairs[i]] : 0;
    deg[i] = i < n ? pdeg[pairs[i]] : 0;
  }
  switch (n) {
    case 1: clevel<OC, 0, 1>(Lt, dLt, dslot, P, p, voff, deg, Fs, dout, o0, nout, 0, acc); break;
    case 2: clevel<OC, 0, 2>(Lt, dLt, dslot, P, p, voff, deg, Fs, dout, o0, nout, 0, acc); break;
    case 3: clevel<OC, 0, 3>(Lt, dLt, dslot, P, p, voff, deg, Fs, dout, o0, nout, 0, acc); break;
    default: clevel<OC, 0, 4>(Lt, dLt, dslot, P, p, voff, deg, Fs, dout, o0, nout, 0, acc); break;
  }
}

struct PlanArgs {
  int n_sum, dout, d_in;
  const int32_t* poff;
  const int32_t* pairs;
  const int64_t* eoff;
  const int32_t* pvoff;
  const int32_t* pdeg;
  const int32_t* pdim;
  const double* F;
  const double* offset;
};

// Grid: points along x, chunks of OC outputs along y (from output o_base).
template <int OC>
__global__ void __launch_bounds__(128, OC == 1 ? 8 : 5) contract64_kernel(PlanArgs a, const double* __restrict__ Lt,
                                                                          int64_t P, double* __restrict__ y,
                                                                          int o_base) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int o0 = o_base + int(blockIdx.y) * OC;
  if (p >= P || o0 >= a.dout) return;
  const int nout = min(OC, a.dout - o0);
  // Two-level sum: summands accumulate into `blk`, which is folded into `acc`
  // every 32 summands, so rounding grows with 32 + n_sum/32 instead of n_sum.
  double acc[OC], blk[OC];
#pragma unroll
  for (int q = 0; q < OC; ++q) acc[q] = blk[q] = 0.0;
  for (int s = 0; s < a.n_sum; ++s) {
    const int q0 = a.poff[s], n = a.poff[s + 1] - q0;
    const int64_t e0 = a.eoff[s], K = a.eoff[s + 1] - e0;
    double one[OC];
#pragma unroll
    for (int q = 0; q < OC; ++q) one[q] = 0.0;
    contract_summand<OC>(Lt, nullptr, -1, P, p, a.pairs + q0, n, a.pvoff, a.pdeg, a.F + e0 * a.dout, K, a.dout, o0, nout,
                     one);
#pragma unroll
    for (int q = 0; q < OC; ++q) blk[q] += one[q];
    if ((s & 31) == 31) {
#pragma unroll
      for (int q = 0; q < OC; ++q) {
        acc[q] += blk[q];
        blk[q] = 0.0;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < OC; ++q)
    if (q < nout) y[p * a.dout + o0 + q] = a.offset[o0 + q] + (acc[q] + blk[q]);
}

// Jacobian: J[p][o][dim] += derivative contraction of every summand and every
// active slot.  Each thread owns one point, so the read-modify-writes of its
// row of J never race.
template <int OC>
__global__ void jacobian64_kernel(PlanArgs a, const double* __restrict__ Lt, const double* __restrict__ dLt, int64_t P,
                                  double* __restrict__ J, int o_base) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int o0 = o_base + int(blockIdx.y) * OC;
  if (p >= P || o0 >= a.dout) return;
  const int nout = min(OC, a.dout - o0);
  double* Jp = J + p * int64_t(a.dout) * a.d_in;
  for (int s = 0; s < a.n_sum; ++s) {
    const int q0 = a.poff[s], n = a.poff[s + 1] - q0;
    const int64_t e0 = a.eoff[s], K = a.eoff[s + 1] - e0;
    for (int i = 0; i < n; ++i) {
      double acc[OC];
#pragma unroll
      for (int q = 0; q < OC; ++q) acc[q] = 0.0;
      contract_summand<OC>(Lt, dLt, i, P, p, a.pairs + q0, n, a.pvoff, a.pdeg, a.F + e0 * a.dout, K, a.dout, o0, nout,
                       acc);
      const int dim = a.pdim[a.pairs[q0 + i]];
#pragma unroll
      for (int q = 0; q < OC; ++q)
        if (q < nout) Jp[int64_t(o0 + q) * a.d_in + dim] += acc[q];
    }
  }
}

// Integral, step 1: product of quadrature weights for every entry.
__global__ void quad_rows_kernel(PlanArgs a, const double* __restrict__ qnode, double* __restrict__ qw) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n_sum) return;
  const int q0 = a.poff[s], n = a.poff[s + 1] - q0;
  const int64_t e0 = a.eoff[s], K = a.eoff[s + 1] - e0;
  int mu[SMX_MAX_DEPTH];
  for (int i = 0; i < n; ++i) mu[i] = 0;
  for (int64_t r = 0; r < K; ++r) {
    double w = 1.0;
    for (int i = 0; i < n; ++i) w *= qnode[a.pvoff[a.pairs[q0 + i]] + mu[i]];
    qw[e0 + r] = w;
    for (int i = n - 1; i >= 0; --i) {
      if (++mu[i] <= a.pdeg[a.pairs[q0 + i]]) break;
      mu[i] = 0;
    }
  }
}

// Integral, step 2: partial sums over row chunks (deterministic split-K GEMV).
__global__ void quad_partial_kernel(const double* __restrict__ qw, const double* __restrict__ F, int64_t R, int dout,
                                    int64_t rows_per_chunk, double* __restrict__ part) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= dout) return;
  const int64_t r0 = int64_t(blockIdx.y) * rows_per_chunk;
  const int64_t r1 = min(R, r0 + rows_per_chunk);
  double acc = 0.0;
  for (int64_t r = r0; r < r1; ++r) acc = fma(qw[r], F[r * dout + o], acc);
  part[int64_t(blockIdx.y) * dout + o] = acc;
}

__global__ void quad_reduce_kernel(const double* __restrict__ part, int nchunks, int dout,
                                   const double* __restrict__ offset, double* __restrict__ Q) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= dout) return;
  double acc = offset[o];
  for (int c = 0; c < nchunks; ++c) acc += part[int64_t(c) * dout + o];
  Q[o] = acc;
}

// F rows from unique function values, zeta folded in.
__global__ void assemble_kernel(int n_sum, const int64_t* __restrict__ eoff, const int64_t* __restrict__ zeta,
                                const double* __restrict__ fu, const int64_t* __restrict__ umap,
                                const double* __restrict__ center, int dout, int64_t R, double* __restrict__ F64,
                                float* __restrict__ F32) {
  const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (idx >= R * dout) return;
  const int64_t r = idx / dout;
  const int o = int(idx - r * dout);
  int lo = 0, hi = n_sum - 1;  // summand s with eoff[s] <= r < eoff[s+1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (eoff[mid] <= r) lo = mid; else hi = mid - 1;
  }
  const double v = double(zeta[lo]) * (fu[umap[r] * dout + o] - (center ? center[o] : 0.0));
  F64[idx] = v;
  if (F32) F32[idx] = float(v);
}

PlanArgs args_of(const smx_plan* pl, const double* F) {
  PlanArgs a;
  a.n_sum = pl->n_summands;
  a.dout = pl->d_out;
  a.d_in = pl->d_in;
  a.poff = pl->sum_poff;
  a.pairs = pl->sum_pairs;
  a.eoff = pl->sum_eoff;
  a.pvoff = pl->pair_voff;
  a.pdeg = pl->pair_deg;
  a.pdim = pl->pair_dim;
  a.F = F;
  a.offset = pl->offset;
  return a;
}

int check_plan(const smx_plan* pl, const char* who) {
  if (!pl) return smx::set_error(SMX_ERR_ARG, std::string(who) + ": null plan");
  if (pl->d_out < 1 || pl->d_in < 1 || pl->n_summands < 0 || pl->n_values < 0 || pl->n_pairs < 0)
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": bad plan sizes");
  if (pl->n_summands > 0 && (!pl->sum_poff || !pl->sum_pairs || !pl->sum_eoff || !pl->pair_voff || !pl->pair_deg ||
                             !pl->pair_dim || !pl->F64))
    return smx::set_error(SMX_ERR_ARG, std::string(who) + ": null plan array");
  if (!pl->offset) return smx::set_error(SMX_ERR_ARG, std::string(who) + ": null offset");
  return SMX_OK;
}

constexpr int kPairsPerBlock = 64;

}  // namespace

extern "C" int smx_bary_weights(int n_pairs, const int32_t* pair_deg, const int32_t* pair_voff, const double* node,
                                double* bweight, void* stream) {
  SMX_REQUIRE(n_pairs >= 0, "smx_bary_weights: negative size");
  if (n_pairs == 0) return SMX_OK;
  SMX_REQUIRE(pair_deg && pair_voff && node && bweight, "smx_bary_weights: null pointer");
  bary_weights_kernel<<<smx::grid_for(n_pairs, 128), 128, 0, smx::as_stream(stream)>>>(n_pairs, pair_deg, pair_voff,
                                                                                         node, bweight);
  SMX_LAUNCH_CHECK("smx_bary_weights");
  return SMX_OK;
}

extern "C" int smx_basis_f64(const smx_plan* pl, const double* x, int64_t P, int64_t ldx, double* Lt, double* dLt,
                             void* stream) {
  int rc = check_plan(pl, "smx_basis_f64");
  if (rc) return rc;
  SMX_REQUIRE(P >= 0 && ldx >= pl->d_in, "smx_basis_f64: bad sizes");
  if (P == 0 || pl->n_pairs == 0) return SMX_OK;
  SMX_REQUIRE(x && Lt && pl->node && pl->bweight, "smx_basis_f64: null pointer");
  dim3 grid(smx::grid_for(P, 128), (pl->n_pairs + kPairsPerBlock - 1) / kPairsPerBlock);
  basis64_kernel<<<grid, 128, 0, smx::as_stream(stream)>>>(pl->n_pairs, pl->pair_dim, pl->pair_deg, pl->pair_voff,
                                                           pl->node, pl->bweight, x, P, ldx, Lt, dLt, kPairsPerBlock);
  SMX_LAUNCH_CHECK("smx_basis_f64");
  return SMX_OK;
}

extern "C" int smx_contract_f64(const smx_plan* pl, const double* Lt, int64_t P, double* y, void* stream) {
  int rc = check_plan(pl, "smx_contract_f64");
  if (rc) return rc;
  SMX_REQUIRE(P >= 0, "smx_contract_f64: negative P");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(y && (pl->n_summands == 0 || Lt), "smx_contract_f64: null pointer");
  PlanArgs a = args_of(pl, pl->F64);
  // all output chunks in one launch (blockIdx.y), so few points still fill the GPU
  // one output: one accumulator per entry (the FP64 pipe is the bound)
  const int oc = pl->d_out == 1 ? 1 : kOC;
  const int chunks = (pl->d_out + oc - 1) / oc;
  for (int c0 = 0; c0 < chunks; c0 += kMaxGridY) {
    const dim3 grid(smx::grid_for(P, 128), unsigned(std::min(kMaxGridY, chunks - c0)));
    if (oc == 1)
      contract64_kernel<1><<<grid, 128, 0, smx::as_stream(stream)>>>(a, Lt, P, y, c0);
    else
      contract64_kernel<kOC><<<grid, 128, 0, smx::as_stream(stream)>>>(a, Lt, P, y, c0 * kOC);
    SMX_LAUNCH_CHECK("smx_contract_f64");
  }
  return SMX_OK;
}

extern "C" size_t smx_eval_workspace(const smx_plan* pl, int64_t P, int precision) {
  if (!pl || P < 0) return 0;
  if (precision == 32) return pl->fp32 ? smx_fp32_workspace(pl->fp32, P) : 0;
  return size_t(pl->n_values) * size_t(P) * sizeof(double) + 256;
}

extern "C" int smx_eval(const smx_plan* pl, int precision, const double* x, int64_t P, int64_t ldx, void* y, void* ws,
                        size_t ws_bytes, void* stream) {
  int rc = check_plan(pl, "smx_eval");
  if (rc) return rc;
  SMX_REQUIRE(precision == 64 || precision == 32, "smx_eval: precision must be 64 or 32");
  if (precision == 32) {
    if (!pl->fp32)
      return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_eval: precision 32 needs the plan's FP32 form (plan->fp32, "
                                                 "built by smx_fp32_plan_create)");
    return smx_fp32_eval(pl->fp32, x, P, ldx, static_cast<float*>(y), ws, ws_bytes, stream);
  }
  if (pl->fp32 && smx_fp32_plan_has_fp64(pl->fp32))
    return smx_fp32_eval64(pl->fp32, x, P, ldx, static_cast<double*>(y), stream);
  SMX_REQUIRE(ws_bytes >= smx_eval_workspace(pl, P, precision), "smx_eval: workspace too small");
  double* Lt = static_cast<double*>(ws);
  rc = smx_basis_f64(pl, x, P, ldx, Lt, nullptr, stream);
  if (rc) return rc;
  return smx_contract_f64(pl, Lt, P, static_cast<double*>(y), stream);
}

extern "C" size_t smx_jacobian_workspace(const smx_plan* pl, int64_t P) {
  if (!pl || P < 0) return 0;
  return 2 * size_t(pl->n_values) * size_t(P) * sizeof(double) + 256;
}

extern "C" int smx_jacobian(const smx_plan* pl, const double* x, int64_t P, int64_t ldx, double* J, void* ws,
                            size_t ws_bytes, void* stream) {
  int rc = check_plan(pl, "smx_jacobian");
  if (rc) return rc;
  SMX_REQUIRE(P >= 0 && J, "smx_jacobian: bad arguments");
  SMX_REQUIRE(ws_bytes >= smx_jacobian_workspace(pl, P), "smx_jacobian: workspace too small");
  if (P == 0) return SMX_OK;
  cudaStream_t st = smx::as_stream(stream);
  cudaMemsetAsync(J, 0, size_t(P) * pl->d_out * pl->d_in * sizeof(double), st);
  SMX_LAUNCH_CHECK("smx_jacobian memset");
  if (pl->n_summands == 0) return SMX_OK;
  double* Lt = static_cast<double*>(ws);
  double* dLt = Lt + size_t(pl->n_values) * size_t(P);
  rc = smx_basis_f64(pl, x, P, ldx, Lt, dLt, stream);
  if (rc) return rc;
  PlanArgs a = args_of(pl, pl->F64);
  const int oc = pl->d_out == 1 ? 1 : kOC;
  const int chunks = (pl->d_out + oc - 1) / oc;
  for (int c0 = 0; c0 < chunks; c0 += kMaxGridY) {
    const dim3 grid(smx::grid_for(P, 128), unsigned(std::min(kMaxGridY, chunks - c0)));
    if (oc == 1)
      jacobian64_kernel<1><<<grid, 128, 0, st>>>(a, Lt, dLt, P, J, c0);
    else
      jacobian64_kernel<kOC><<<grid, 128, 0, st>>>(a, Lt, dLt, P, J, c0 * kOC);
    SMX_LAUNCH_CHECK("smx_jacobian");
  }
  return SMX_OK;
}

namespace {
constexpr int64_t kQuadRows = 4096;
}

extern "C" size_t smx_integral_workspace(const smx_plan* pl) {
  if (!pl) return 0;
  int64_t nch = (pl->n_entries + kQuadRows - 1) / kQuadRows;
  if (nch < 1) nch = 1;
  return size_t(pl->n_entries) * sizeof(double) + size_t(nch) * pl->d_out * sizeof(double) + 512;
}

extern "C" int smx_integral(const smx_plan* pl, const double* qnode, double* Q, void* ws, size_t ws_bytes,
                            void* stream) {
  int rc = check_plan(pl, "smx_integral");
  if (rc) return rc;
  SMX_REQUIRE(Q && (pl->n_summands == 0 || qnode), "smx_integral: null pointer");
  SMX_REQUIRE(ws_bytes >= smx_integral_workspace(pl), "smx_integral: workspace too small");
  cudaStream_t st = smx::as_stream(stream);
  int64_t nch = (pl->n_entries + kQuadRows - 1) / kQuadRows;
  if (nch < 1) nch = 1;
  double* qw = static_cast<double*>(ws);
  double* part = qw + ((pl->n_entries + 31) / 32) * 32;
  PlanArgs a = args_of(pl, pl->F64);
  if (pl->n_summands > 0) {
    quad_rows_kernel<<<smx::grid_for(pl->n_summands, 128), 128, 0, st>>>(a, qnode, qw);
    dim3 g(smx::grid_for(pl->d_out, 128), (unsigned)nch);
    quad_partial_kernel<<<g, 128, 0, st>>>(qw, pl->F64, pl->n_entries, pl->d_out, kQuadRows, part);
  } else {
    cudaMemsetAsync(part, 0, sizeof(double) * pl->d_out, st);
    nch = 1;
  }
  quad_reduce_kernel<<<smx::grid_for(pl->d_out, 128), 128, 0, st>>>(part, int(nch), pl->d_out, pl->offset, Q);
  SMX_LAUNCH_CHECK("smx_integral");
  return SMX_OK;
}

extern "C" int smx_assemble_F(const smx_plan* pl, const int64_t* sum_zeta, const double* fu, const int64_t* umap,
                              const double* center, double* F64, float* F32, void* stream) {
  SMX_REQUIRE(pl != nullptr, "smx_assemble_F: null plan");
  const int64_t total = pl->n_entries * int64_t(pl->d_out);
  if (total == 0) return SMX_OK;
  SMX_REQUIRE(sum_zeta && fu && umap && F64 && pl->sum_eoff, "smx_assemble_F: null pointer");
  assemble_kernel<<<smx::grid_for(total, 256), 256, 0, smx::as_stream(stream)>>>(
      pl->n_summands, pl->sum_eoff, sum_zeta, fu, umap, center, pl->d_out, pl->n_entries, F64, F32);
  SMX_LAUNCH_CHECK("smx_assemble_F");
  return SMX_OK;
}
