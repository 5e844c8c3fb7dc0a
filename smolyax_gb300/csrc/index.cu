// Anisotropic multi-index set Lambda_{k,t}, Smolyak coefficients and DFS order.
//
// Bit-exactness: every budget update and comparison is done with explicitly
// rounded IEEE operations (__dmul_rn, __dsub_rn, __dadd_rn) in the same form
// and order as the reference's Python/numba code (src/smolyax/indices.py), so
// no fused multiply-add can change a boundary decision.
#include "common.cuh"

namespace {

// Number of j >= 1 admitted at dimension i (and, with emit, the children).
__device__ inline int64_t includes_at(const double* k, int i, double rem, double used, double t, int mode) {
  const double ki = k[i];
  int64_t c = 0;
  for (int64_t j = 1;; ++j) {
    const double jk = __dmul_rn(double(j), ki);
    const bool ok = (mode == SMX_MODE_ADDITIVE) ? (__dadd_rn(used, jk) < t) : (jk < rem);
    if (!ok) break;
    ++c;
    if (c > (int64_t(1) << 40)) break;  // guards k[i] <= 0 from looping forever
  }
  return c;
}

// Walks the continuation chain of an entry.  For every node i of the chain it
// calls visit(i); returns the chain end (node at which the entry is emitted).
template <typename Visit>
__device__ inline int walk_chain(const double* k, int d, double t, int mode, double rem_or_used, int start,
                                 Visit visit) {
  int i = start;
  if (mode == SMX_MODE_INDEXSET) {
    // indices.py:49-67: node i is final when i >= d or k[i] >= rem; otherwise
    // includes at i and an unconditional step to i + 1.
    while (i < d && k[i] < rem_or_used) {
      visit(i);
      ++i;
    }
    return i;
  }
  // indices.py:242-258 (and :98-116 with rem = t - used): includes at every
  // node; step to i + 1 only while k[i+1] < rem.
  const double rem = (mode == SMX_MODE_ADDITIVE) ? __dsub_rn(t, rem_or_used) : rem_or_used;
  if (i >= d) return i;
  for (;;) {
    visit(i);
    if (i + 1 < d && k[i + 1] < rem) {
      ++i;
    } else {
      return i;
    }
  }
}

__global__ void lambda_count_kernel(const double* __restrict__ k, int d, double t, int mode,
                                    const double* __restrict__ rem, const int32_t* __restrict__ start, int64_t n,
                                    int64_t* __restrict__ count, int32_t* __restrict__ term) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    const double r = rem[e];
    int64_t c = 0;
    const double rr = (mode == SMX_MODE_ADDITIVE) ? 0.0 : r;
    const double used = (mode == SMX_MODE_ADDITIVE) ? r : 0.0;
    int end = walk_chain(k, d, t, mode, r, start[e], [&](int i) { c += includes_at(k, i, rr, used, t, mode); });
    count[e] = c;
    if (term) term[e] = end;
  }
}

__global__ void lambda_expand_kernel(const double* __restrict__ k, int d, double t, int mode,
                                     const double* __restrict__ rem, const int32_t* __restrict__ start, int64_t n,
                                     const int64_t* __restrict__ offs, int64_t parent_base, double* __restrict__ c_rem,
                                     int32_t* __restrict__ c_start, int32_t* __restrict__ c_parent,
                                     int32_t* __restrict__ c_dim, int32_t* __restrict__ c_deg) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    const double r = rem[e];
    int64_t o = offs[e];
    walk_chain(k, d, t, mode, r, start[e], [&](int i) {
      const double ki = k[i];
      for (int64_t j = 1;; ++j) {
        const double jk = __dmul_rn(double(j), ki);
        double child;
        if (mode == SMX_MODE_ADDITIVE) {
          const double u = __dadd_rn(r, jk);
          if (!(u < t)) break;
          child = u;
        } else {
          if (!(jk < r)) break;
          child = __dsub_rn(r, jk);
        }
        c_rem[o] = child;
        c_start[o] = i + 1;
        c_parent[o] = int32_t(parent_base + e);
        c_dim[o] = i;
        c_deg[o] = int32_t(j);
        ++o;
      }
    });
  }
}

// Smolyak coefficient by the reference's DFS over e in {0,1}^d
// (indices.py:121-168), with an explicit path stack: frame = (node i, budget,
// sign, phase).  Phase 0: arriving at node i (include child first);
// phase 1: include subtree done, take the skip step or terminate.
__device__ int64_t zeta_of(const double* __restrict__ k, int d, double rem, int* overflow) {
  int fi[SMX_MAX_DEPTH + 1];
  double fr[SMX_MAX_DEPTH + 1];
  int8_t fs[SMX_MAX_DEPTH + 1];
  int8_t fp[SMX_MAX_DEPTH + 1];
  int sp = 0;
  fi[0] = 0;
  fr[0] = rem;
  fs[0] = 1;
  fp[0] = 0;
  int64_t total = 0;
  while (sp >= 0) {
    const int i = fi[sp];
    const double rt = fr[sp];
    if (fp[sp] == 0) {
      if (i >= d) {
        total += fs[sp];
        --sp;
        continue;
      }
      fp[sp] = 1;
      if (k[i] < rt) {
        if (sp == SMX_MAX_DEPTH) {
          *overflow = 1;
          return 0;
        }
        ++sp;
        fi[sp] = i + 1;
        fr[sp] = __dsub_rn(rt, k[i]);
        fs[sp] = int8_t(-fs[sp - 1]);
        fp[sp] = 0;
        continue;
      }
    }
    // phase 1: skip step
    if (i + 1 < d && k[i + 1] < rt) {
      fi[sp] = i + 1;
      fp[sp] = 0;
    } else {
      total += fs[sp];
      --sp;
    }
  }
  return total;
}

__global__ void zeta_kernel(const double* __restrict__ k, int d, const double* __restrict__ rem,
                            const int32_t* __restrict__ parity, int64_t n, int64_t* __restrict__ zeta,
                            int32_t* __restrict__ flag) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    int ovf = 0;
    int64_t z = zeta_of(k, d, rem[e], &ovf);
    if (ovf && flag) atomicExch(flag, 1);
    if (parity && (parity[e] & 1)) z = -z;
    zeta[e] = z;
  }
}

__global__ void subtree_size_kernel(const int64_t* __restrict__ first_child, const int64_t* __restrict__ n_child,
                                    int64_t b, int64_t e_end, int64_t* __restrict__ size) {
  for (int64_t e = b + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < e_end;
       e += int64_t(gridDim.x) * blockDim.x) {
    int64_t s = 1;
    const int64_t c0 = first_child[e], nc = n_child[e];
    for (int64_t c = 0; c < nc; ++c) s += size[c0 + c];
    size[e] = s;
  }
}

// Children of an entry are stored by chain dimension ascending, j ascending
// within a dimension.  The reference's LIFO stack visits them by dimension
// ascending and j DESCENDING; the entry itself is emitted before the
// children at its chain end (non-zero mode) or after all children (indexset
// mode, where the emitting node is the step past the chain end).
__global__ void rank_kernel(int mode, const int32_t* __restrict__ term, const int32_t* __restrict__ dim,
                            const int64_t* __restrict__ first_child, const int64_t* __restrict__ n_child,
                            const int64_t* __restrict__ size, int64_t b, int64_t e_end, int64_t* __restrict__ base,
                            int64_t* __restrict__ rank) {
  for (int64_t e = b + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < e_end;
       e += int64_t(gridDim.x) * blockDim.x) {
    int64_t cur = base[e];
    const int64_t c0 = first_child[e], nc = n_child[e];
    const int td = (mode == SMX_MODE_NONZERO) ? term[e] : (mode == SMX_MODE_PREORDER ? -1 : 0x7fffffff);
    bool placed = false;
    int64_t c = 0;
    while (c < nc) {
      const int dd = dim[c0 + c];
      int64_t c1 = c;
      while (c1 < nc && dim[c0 + c1] == dd) ++c1;
      if (!placed && dd >= td) {
        rank[e] = cur++;
        placed = true;
      }
      for (int64_t q = c1 - 1; q >= c; --q) {
        base[c0 + q] = cur;
        cur += size[c0 + q];
      }
      c = c1;
    }
    if (!placed) rank[e] = cur++;
  }
}

__global__ void max_degree_kernel(int64_t n, const int32_t* __restrict__ dim, const int32_t* __restrict__ deg,
                                  int32_t* __restrict__ maxdeg) {
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
    if (dim[e] >= 0) atomicMax(&maxdeg[dim[e]], deg[e]);
  }
}

__global__ void plan_summands_kernel(int64_t n_sum, const int64_t* __restrict__ ent, const int32_t* __restrict__ parent,
                                     const int32_t* __restrict__ dim, const int32_t* __restrict__ deg,
                                     const int32_t* __restrict__ pair_base, const int32_t* __restrict__ sum_poff,
                                     int32_t* __restrict__ sum_pairs, int64_t* __restrict__ n_ent) {
  for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n_sum; s += int64_t(gridDim.x) * blockDim.x) {
    const int p0 = sum_poff[s], p1 = sum_poff[s + 1];
    int64_t e = ent[s];
    int64_t K = 1;
    // parent chain yields pairs in DESCENDING dim order; write from the back
    for (int q = p1 - 1; q >= p0; --q) {
      const int dd = dim[e], g = deg[e];
      sum_pairs[q] = pair_base[dd] + g - 1;
      K *= (g + 1);
      e = parent[e];
    }
    n_ent[s] = K;
  }
}

}  // namespace

extern "C" int smx_lambda_count(const double* k, int d, double t, int mode, const double* rem, const int32_t* start,
                                int64_t n, int64_t* count, int32_t* term, void* stream) {
  SMX_REQUIRE(d >= 0 && n >= 0, "smx_lambda_count: negative size");
  SMX_REQUIRE(mode >= 0 && mode <= 2, "smx_lambda_count: bad mode");
  if (n == 0) return SMX_OK;
  SMX_REQUIRE(rem && start && count && (d == 0 || k), "smx_lambda_count: null pointer");
  lambda_count_kernel<<<smx::grid_for(n, 128), 128, 0, smx::as_stream(stream)>>>(k, d, t, mode, rem, start, n, count,
                                                                                   term);
  SMX_LAUNCH_CHECK("smx_lambda_count");
  return SMX_OK;
}

extern "C" int smx_lambda_expand(const double* k, int d, double t, int mode, const double* rem, const int32_t* start,
                                 int64_t n, const int64_t* offs, int64_t parent_base, double* c_rem, int32_t* c_start,
                                 int32_t* c_parent, int32_t* c_dim, int32_t* c_deg, void* stream) {
  SMX_REQUIRE(d >= 0 && n >= 0, "smx_lambda_expand: negative size");
  SMX_REQUIRE(mode >= 0 && mode <= 2, "smx_lambda_expand: bad mode");
  if (n == 0) return SMX_OK;
  SMX_REQUIRE(rem && start && offs && c_rem && c_start && c_parent && c_dim && c_deg, "smx_lambda_expand: null");
  lambda_expand_kernel<<<smx::grid_for(n, 128), 128, 0, smx::as_stream(stream)>>>(
      k, d, t, mode, rem, start, n, offs, parent_base, c_rem, c_start, c_parent, c_dim, c_deg);
  SMX_LAUNCH_CHECK("smx_lambda_expand");
  return SMX_OK;
}

extern "C" int smx_zeta(const double* k, int d, const double* rem, const int32_t* parity, int64_t n, int64_t* zeta,
                        int32_t* flag, void* stream) {
  SMX_REQUIRE(d >= 0 && n >= 0, "smx_zeta: negative size");
  if (n == 0) return SMX_OK;
  SMX_REQUIRE(rem && zeta && (d == 0 || k), "smx_zeta: null pointer");
  zeta_kernel<<<smx::grid_for(n, 64), 64, 0, smx::as_stream(stream)>>>(k, d, rem, parity, n, zeta, flag);
  SMX_LAUNCH_CHECK("smx_zeta");
  return SMX_OK;
}

extern "C" int smx_lambda_subtree_sizes(const int64_t* first_child, const int64_t* n_child, int64_t lvl_begin,
                                        int64_t lvl_end, int64_t* size, void* stream) {
  SMX_REQUIRE(lvl_begin >= 0 && lvl_end >= lvl_begin, "smx_lambda_subtree_sizes: bad range");
  if (lvl_end == lvl_begin) return SMX_OK;
  SMX_REQUIRE(first_child && n_child && size, "smx_lambda_subtree_sizes: null pointer");
  subtree_size_kernel<<<smx::grid_for(lvl_end - lvl_begin, 128), 128, 0, smx::as_stream(stream)>>>(
      first_child, n_child, lvl_begin, lvl_end, size);
  SMX_LAUNCH_CHECK("smx_lambda_subtree_sizes");
  return SMX_OK;
}

extern "C" int smx_lambda_ranks(int mode, const int32_t* term, const int32_t* dim, const int64_t* first_child,
                                const int64_t* n_child, const int64_t* size, int64_t lvl_begin, int64_t lvl_end,
                                int64_t* base, int64_t* rank, void* stream) {
  SMX_REQUIRE(mode == SMX_MODE_NONZERO || mode == SMX_MODE_INDEXSET || mode == SMX_MODE_PREORDER,
              "smx_lambda_ranks: bad mode");
  SMX_REQUIRE(lvl_begin >= 0 && lvl_end >= lvl_begin, "smx_lambda_ranks: bad range");
  if (lvl_end == lvl_begin) return SMX_OK;
  SMX_REQUIRE(dim && first_child && n_child && size && base && rank, "smx_lambda_ranks: null pointer");
  SMX_REQUIRE(mode != SMX_MODE_NONZERO || term, "smx_lambda_ranks: term needed");
  rank_kernel<<<smx::grid_for(lvl_end - lvl_begin, 128), 128, 0, smx::as_stream(stream)>>>(
      mode, term, dim, first_child, n_child, size, lvl_begin, lvl_end, base, rank);
  SMX_LAUNCH_CHECK("smx_lambda_ranks");
  return SMX_OK;
}

extern "C" int smx_max_degree(int64_t n, const int32_t* dim, const int32_t* deg, int32_t* maxdeg, void* stream) {
  SMX_REQUIRE(n >= 0, "smx_max_degree: negative size");
  if (n == 0) return SMX_OK;
  SMX_REQUIRE(dim && deg && maxdeg, "smx_max_degree: null pointer");
  max_degree_kernel<<<smx::grid_for(n, 256), 256, 0, smx::as_stream(stream)>>>(n, dim, deg, maxdeg);
  SMX_LAUNCH_CHECK("smx_max_degree");
  return SMX_OK;
}

extern "C" int smx_plan_summands(int64_t n_sum, const int64_t* ent, const int32_t* parent, const int32_t* dim,
                                 const int32_t* deg, const int32_t* pair_base, const int32_t* sum_poff,
                                 int32_t* sum_pairs, int64_t* n_ent, void* stream) {
  SMX_REQUIRE(n_sum >= 0, "smx_plan_summands: negative size");
  if (n_sum == 0) return SMX_OK;
  SMX_REQUIRE(ent && parent && dim && deg && pair_base && sum_poff && sum_pairs && n_ent, "smx_plan_summands: null");
  plan_summands_kernel<<<smx::grid_for(n_sum, 128), 128, 0, smx::as_stream(stream)>>>(
      n_sum, ent, parent, dim, deg, pair_base, sum_poff, sum_pairs, n_ent);
  SMX_LAUNCH_CHECK("smx_plan_summands");
  return SMX_OK;
}
