/*
 * smolyax_gb300 -- C ABI of the GB300 (sm_103a) evaluation path of the
 * barycentric Smolyak interpolant.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer owned by the caller unless the
 *    comment says "host".  Scratch space is passed in by the caller (`ws`,
 *    `ws_bytes`); the only entry point that allocates device memory is
 *    smx_fp32_plan_create (the FP32 plan's tables, released by
 *    smx_fp32_plan_destroy).
 *  - `stream` is a cudaStream_t passed as void*; all work is stream-ordered and
 *    asynchronous unless the comment says the call synchronises.
 *  - Every entry point returns SMX_OK (0) or one of the negative SMX_ERR_*
 *    codes below; smx_last_error_string() describes the most recent failure of
 *    the calling thread.
 *  - Reference citations are paths inside JoWestermann/smolyax.
 */
#ifndef SMOLYAX_GB300_H
#define SMOLYAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SMX_OK = 0,
  SMX_ERR_ARG = -1,        /* invalid argument (null pointer, bad size)            */
  SMX_ERR_WORKSPACE = -2,  /* workspace too small                                   */
  SMX_ERR_CUDA = -3,       /* a CUDA runtime call or launch failed                  */
  SMX_ERR_DEPTH = -4,      /* enumeration deeper than SMX_MAX_DEPTH                 */
  SMX_ERR_UNSUPPORTED = -5 /* configuration outside what the kernels support       */
};

#define SMX_MAX_DEPTH 64 /* max number of included dimensions in one DFS path */

/* ---- anisotropic multi-index set Lambda_{k,t} -----------------------------------
 * The set is built level by level, level n holding the multi-indices with n
 * non-zero entries.  An entry of a level is (rem, start, parent, dim, deg): the
 * remaining budget after its last inclusion, the first dimension of its
 * continuation chain, its parent in level n-1, and its last non-zero entry
 * (dim, deg).  `mode` selects the arithmetic and chain rule of the reference
 * function being replaced:
 *   SMX_MODE_NONZERO  -- subtractive budget, chain continues while k[i+1] < rem
 *                        (indices.py:214-259 non_zero_indices_and_zetas and
 *                        indices.py:175-211 __nodeset_cardinality_non_nested);
 *   SMX_MODE_INDEXSET -- subtractive budget, chain continues while k[i] < rem
 *                        (indices.py:20-69 indexset);
 *   SMX_MODE_ADDITIVE -- `rem` holds the USED budget, inclusion test
 *                        used + j*k[i] < t (indices.py:72-118 indexset_cardinality).
 */
#define SMX_MODE_NONZERO 0
#define SMX_MODE_INDEXSET 1
#define SMX_MODE_ADDITIVE 2
#define SMX_MODE_PREORDER 3 /* ranks only: every entry before its children */

/* Per entry: number of children (written to `count`) and the chain end
 * (`term`).  Replaces the inner expansion loops of indices.py:49-67,
 * indices.py:98-116 and indices.py:242-258. */
int smx_lambda_count(const double* k, int d, double t, int mode, const double* rem, const int32_t* start,
                     int64_t n, int64_t* count, int32_t* term, void* stream);

/* Writes the children of every entry at offsets `offs` (exclusive scan of
 * `count`); c_parent receives parent_base + the parent's index (global id).
 * Same reference lines as smx_lambda_count. */
int smx_lambda_expand(const double* k, int d, double t, int mode, const double* rem, const int32_t* start,
                      int64_t n, const int64_t* offs, int64_t parent_base, double* c_rem, int32_t* c_start,
                      int32_t* c_parent, int32_t* c_dim, int32_t* c_deg, void* stream);

/* zeta[i] = smolyak_coefficient(k, d, rem[i], parity[i] or 0): signed count of
 * e in {0,1}^d with nu+e in Lambda (indices.py:121-168).  `parity` may be NULL.
 * On an enumeration deeper than SMX_MAX_DEPTH the entry's zeta is set to 0 and
 * *flag (device int, may be NULL) is set to 1. */
int smx_zeta(const double* k, int d, const double* rem, const int32_t* parity, int64_t n, int64_t* zeta,
             int32_t* flag, void* stream);

/* Inclusive/exclusive scan of int64 values; out[n] receives the total when
 * `out` has n+1 slots (exclusive form).  ws >= smx_scan_workspace(n) bytes. */
size_t smx_scan_workspace(int64_t n);
int smx_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* ws, size_t ws_bytes, void* stream);

/* DFS-order ranks of all entries of a level set, i.e. the order of the
 * reference's stack-based enumeration (indices.py:46-67, indices.py:241-258).
 * Entries of all levels are concatenated (global ids); `first_child` and
 * `n_child` give each entry's children range (children are written by
 * smx_lambda_expand in dimension-ascending, degree-ascending order).
 * smx_lambda_subtree_sizes is called level by level from the deepest level up;
 * smx_lambda_ranks level by level from the root down, with base[root] = 0: it
 * writes rank[e] and the first rank base[c] of every child subtree.  In
 * SMX_MODE_NONZERO an entry precedes the children at its chain-end dimension
 * `term`; in SMX_MODE_INDEXSET it follows all its children; SMX_MODE_PREORDER
 * places it before all its children (the order used by the FP32 evaluator). */
int smx_lambda_subtree_sizes(const int64_t* first_child, const int64_t* n_child, int64_t lvl_begin, int64_t lvl_end,
                             int64_t* size, void* stream);
int smx_lambda_ranks(int mode, const int32_t* term, const int32_t* dim, const int64_t* first_child,
                     const int64_t* n_child, const int64_t* size, int64_t lvl_begin, int64_t lvl_end, int64_t* base,
                     int64_t* rank, void* stream);

/* ---- interpolation plan ------------------------------------------------------------
 * Summands are the multi-indices with zeta != 0 and n >= 1; each summand's
 * tensor of nodal values is stored unpadded, its active (dim, deg) pairs in
 * ascending dim order, the last pair varying fastest; rows hold d_out values
 * with zeta folded in.  Pairs are unique (dim, deg) combinations, deg >= 1;
 * each owns deg+1 consecutive "value slots" (node, weight, basis value).
 */
typedef struct smx_plan {
  int32_t d_in, d_out;
  int32_t n_pairs;     /* unique (dim, deg) pairs                                  */
  int32_t n_values;    /* V = sum over pairs of (deg + 1)                          */
  int32_t n_summands;  /* summands with n >= 1                                     */
  int32_t max_n;       /* max active dimensions of a summand                       */
  int64_t n_entries;   /* R = sum over summands of prod(deg + 1)                   */
  const int32_t* pair_dim;     /* [n_pairs]                                        */
  const int32_t* pair_deg;     /* [n_pairs]                                        */
  const int32_t* pair_voff;    /* [n_pairs] first value slot of the pair           */
  const double* node;          /* [n_values] nodes of every pair                   */
  const double* bweight;       /* [n_values] barycentric weights                   */
  const int32_t* sum_poff;     /* [n_summands+1] offsets into sum_pairs            */
  const int32_t* sum_pairs;    /* pair ids of each summand, ascending dim          */
  const int64_t* sum_eoff;     /* [n_summands+1] first entry (row) of each summand */
  const double* F64;           /* [n_entries * d_out] zeta * f(node)               */
  const float* F32;            /* [n_entries * d_out] FP32 rounding of F64 (or NULL)*/
  const double* offset;        /* [d_out] zeta_0 * f(zero point)                   */
  const struct smx_fp32_plan* fp32; /* orthogonal form (smx_fp32_plan_create), or NULL:
                                       smx_eval(plan, 32, ...) evaluates through it,
                                       smx_eval(plan, 64, ...) too when it has FP64
                                       tables (one output) */
} smx_plan;

/* Barycentric weights of every pair: w_b = prod_a 1/(xi_a - xi_b) with zero
 * differences replaced by 1 (barycentric.py:13-31). */
int smx_bary_weights(int n_pairs, const int32_t* pair_deg, const int32_t* pair_voff, const double* node,
                     double* bweight, void* stream);

/* Summand pairs and entry counts from the zeta != 0 entries: walks the parent
 * chain of entry `ent[s]` (global ids), writes its pair ids in ascending dim
 * order at sum_poff[s] and prod(deg+1) into n_ent[s] (replaces the block
 * assembly of interpolation.py:168-199 with an unpadded layout). */
int smx_plan_summands(int64_t n_sum, const int64_t* ent, const int32_t* parent, const int32_t* dim,
                      const int32_t* deg, const int32_t* pair_base, const int32_t* sum_poff, int32_t* sum_pairs,
                      int64_t* n_ent, void* stream);

/* Per-dimension maximal degree over a set of entries (atomicMax). */
int smx_max_degree(int64_t n, const int32_t* dim, const int32_t* deg, int32_t* maxdeg, void* stream);

/* F64/F32 rows from unique function values:
 *   F64[r] = zeta(r) * (fu[umap[r]] - center)
 * (interpolation.py:201-235, with the reference's cached f evaluations
 * gathered on the device).  `center` (d_out values, may be NULL for zero) is
 * a constant subtracted from every nodal value; since every tensor-product
 * interpolant reproduces constants, the caller adds center * sum(zeta) to the
 * offset.  Centering shrinks the summands that cancel in the combination
 * sum and so the rounding error of the FP64 result. */
int smx_assemble_F(const smx_plan* plan_host, const int64_t* sum_zeta, const double* fu, const int64_t* umap,
                   const double* center, double* F64, float* F32, void* stream);

/* ---- evaluation -------------------------------------------------------------------
 * Basis table: Lt[v*P + p] = normalised barycentric basis value of slot v at
 * point p, with the one-hot rule at exact nodes (barycentric.py:34-66 and the
 * normalisation at barycentric.py:117).  dLt (nullable) receives the
 * derivative of the normalised basis, NaN at exact nodes (barycentric.py:126-155,
 * :213-219).  x is row-major [P, ldx] FP64. */
int smx_basis_f64(const smx_plan* plan_host, const double* x, int64_t P, int64_t ldx, double* Lt, double* dLt,
                  void* stream);

/* y[p*d_out + o] = offset[o] + sum over summands of the tensor-product
 * contraction of the summand's rows with the basis values of point p
 * (barycentric.py:69-123, interpolation.py:264-304). */
int smx_contract_f64(const smx_plan* plan_host, const double* Lt, int64_t P, double* y, void* stream);

/* One evaluation call (interpolation.py:264-304).  precision 64: the FP64
 * path -- the orthogonal form in FP64 when plan->fp32 is set and has FP64
 * tables (smx_fp32_plan_has_fp64: one output), else the combination sum
 * (basis table into `ws`, then the contraction); y is FP64 [P, d_out].
 * precision 32: the FP32 form plan->fp32 (SMX_ERR_UNSUPPORTED if NULL; y is
 * FP32 [P, d_out]), as smx_fp32_eval.  ws_bytes >= smx_eval_workspace(plan,
 * P, precision). */
size_t smx_eval_workspace(const smx_plan* plan_host, int64_t P, int precision);
int smx_eval(const smx_plan* plan_host, int precision, const double* x, int64_t P, int64_t ldx, void* y, void* ws,
             size_t ws_bytes, void* stream);

/* Full Jacobian J[(p*d_out + o)*d_in + j] (dense, zero outside active
 * dimensions), FP64 (barycentric.py:158-229, interpolation.py:306-345). */
size_t smx_jacobian_workspace(const smx_plan* plan_host, int64_t P);
int smx_jacobian(const smx_plan* plan_host, const double* x, int64_t P, int64_t ldx, double* J, void* ws,
                 size_t ws_bytes, void* stream);

/* Integral: Q[o] = offset[o] + sum_r qw(r) F64[r, o] with qw the product of
 * the pairs' quadrature weights `qnode` ([n_values], host-computed rule
 * weights) (interpolation.py:347-390). */
size_t smx_integral_workspace(const smx_plan* plan_host);
int smx_integral(const smx_plan* plan_host, const double* qnode, double* Q, void* ws, size_t ws_bytes, void* stream);

/* ---- mixed-precision path: orthogonal-polynomial form --------------------------------
 * The interpolant is re-expressed as sum_{m in Lambda} c_m prod_j phi_{m_j}(z_j)
 * with phi_n the Legendre polynomials (fam 0) or the normalised Hermite
 * polynomials H_n / sqrt(2^n n!) (fam 1) of z_j = fam_a[j] * x_j + fam_b[j].
 * This re-expression of the reference's combination sum (interpolation.py:
 * 264-304 over barycentric.py:69-123) is exact in exact arithmetic; it moves
 * the cancellation of the combination sum into an FP64 set-up step so that
 * the evaluation can run in FP32. */

/* Per pair: A = V^{-1} with V[j][m] = phi_m(z(node_j)) (FP64, row-major
 * [m][j] at aoff[pair]); *flag != 0 on failure (degree > 23 or singular V). */
int smx_spectral_pairs(int n_pairs, const int32_t* pair_dim, const int32_t* pair_deg, const int32_t* pair_voff,
                       const int64_t* aoff, const double* node, const int32_t* fam, const double* fam_a,
                       const double* fam_b, double* A, int32_t* flag, void* stream);

/* Coefficients C[n_lambda * d_out] (FP64) of every entry of the index set
 * (tree arrays of smx_lambda_*, NONZERO mode): mode products of each summand's
 * rows with its pairs' A matrices (scratch G: n_entries * d_out doubles, ids:
 * n_entries int32 = the entry of every row) summed into the entries in row
 * order (rows sorted by entry on the device: the same result on every call);
 * C[root] also receives the plan's offset.  Scratch ws of
 * smx_spectral_coefficients_workspace bytes (device).  *flag = 4 if a
 * multi-index is missing from the tree. */
size_t smx_spectral_coefficients_workspace(const smx_plan* plan_host);
int smx_spectral_coefficients(const smx_plan* plan_host, const int64_t* aoff, const double* A,
                              const int64_t* first_child, const int64_t* n_child, const int32_t* tdim,
                              const int32_t* tdeg, int64_t n_lambda, double* G, int32_t* ids, double* C,
                              int32_t* flag, void* ws, size_t ws_bytes, void* stream);

/* Evaluation layout of the orthogonal form.  "Hot" dimensions are those that
 * occur before another dimension in some multi-index; every entry of Lambda
 * is either hot (all its dimensions hot) or cold (hot prefix + one cold last
 * pair).  Per point, a row of `row` floats holds phi_g(z_d) of the hot
 * dimensions ([0, n_hb)) and the products of the hot nodes that cold entries
 * extend ([n_hb, n_hb + n_vp), slot n_hb = empty prefix = 1).  Sums are over
 * runs: int4 (start slot, length, coefficient offset, degree), start and
 * length multiples of 4, coefficients [length][dstride] contiguous; the runs
 * of a cold group are sorted by degree. */
typedef struct smx_spectral {
  int32_t d_in, d_out;
  int32_t dstride;       /* coefficient stride per leaf (1, or d_out rounded up to 4) */
  int32_t row;           /* floats per point row (multiple of 4, = 4 mod 32 ideally) */
  int32_t n_hb;          /* hot basis slots                                       */
  int32_t n_vp;          /* prefix-product slots                                  */
  int32_t n_hot_dims;
  int32_t n_nodes;       /* hot nodes with children, root first, DFS pre-order    */
  int32_t n_cold_groups; /* cold dimensions                                       */
  int32_t max_depth;     /* deepest node (<= 8)                                   */
  int32_t n_cold_blocks; /* blocks of 4 degree-1 cold dimensions (d_out = 1)    */
  int32_t node_seg[5];   /* the evaluator's 4 work segments over the nodes,     */
  int32_t cold_seg[5];   /* the cold groups                                      */
  int32_t block_seg[5];  /* and the cold blocks (host values)                    */
  const int32_t* hot_dim;   /* [n_hot_dims]                                       */
  const int32_t* hot_deg;   /* [n_hot_dims] max degree                            */
  const int32_t* hot_soff;  /* [n_hot_dims] first basis slot                      */
  const int32_t* node;      /* [n_nodes][4] slot | depth << 16, prefix slot or -1, run range */
  const float* node_c;      /* [n_nodes][dstride] own coefficient                  */
  const int32_t* cold;      /* [n_cold_groups][4] dim, run range, max degree | fam << 16 */
  const float* cold_ab;     /* [n_cold_groups][2] affine map z = a x + b of the group */
  const int32_t* blk_dims;  /* [n_cold_blocks][4] the block's dimensions                */
  const int32_t* blk_run;   /* [n_cold_blocks][4] first slot, slot quads, coefficient offset, 0;
                               coefficients [quad][slot][dimension] */
  const float* blk_ab;      /* [n_cold_blocks][2][4] phi_1 = a x + b per dimension      */
  const int32_t* run;       /* [n_runs][4] start, length, coefficient offset, degree */
  const float* coef;        /* run coefficients                                    */
  const float* fam_a;       /* [d_in]                                             */
  const float* fam_b;       /* [d_in]                                             */
  const int32_t* fam;       /* [d_in] 0 Legendre, 1 Hermite                       */
  const float* c0;          /* [d_out] coefficient of the constant                */
} smx_spectral;

/* FP32 evaluation y[P, d_out] (x FP64 row-major, leading dimension ldx). */
int smx_spectral_eval(const smx_spectral* plan_host, const double* x, int64_t P, int64_t ldx, float* y,
                      void* stream);

/* FP64 evaluation of the orthogonal form (the FP64 counterpart of
 * interpolation.py:264-304).  The per-point structure of smx_spectral -- hot
 * basis values and the prefix products of the cold entries' parents in a row
 * of `row` doubles per point (row >= n_hb + n_vp; odd keeps 8-byte reads of
 * consecutive points on distinct banks; a block of B points needs (row + 4 *
 * (d_out == 1 ? 1 : 4)) * B * 8 bytes of shared memory, <= 227 KB, with B =
 * 64, 96 or 128 chosen per call for the fewest idle SM slots in the last
 * wave) -- but
 * every entry of Lambda is exactly one term (row slot, coefficients), without
 * padding: at GB300's FP64 rate each term is a multiply-add that counts.  One
 * output per pass (d_out = 1), else four (outputs o0..o0+3 per block row).
 *   node[n_nodes][4]  slot | depth << 16, prefix slot or -1, term range of the
 *                     hot leaf children (hot nodes in DFS pre-order, root first)
 *   cold[G][4]        dimension, run range, max degree | family << 16 | unit << 20
 *                     (unit: the map z = a x + b is the identity)
 *   run[R][4]         term range, degree, 0 (runs of a group by degree)
 *   terms[T][2]       slot (integer bits of the first double), coefficient (d_out = 1)
 *   coef[T][dstride]  coefficients (d_out > 1; dstride = d_out rounded up to 4)
 * With coefficients from smx_spectral_coefficients (compensated sums) the
 * result is within ~1e-14 relative of the exact value of the interpolant,
 * where the barycentric combination sum in FP64 cancels to 1e-13 .. 1e-10.
 * Non-finite coordinates of active dimensions give NaN. */
typedef struct smx_spectral64 {
  int32_t d_in, d_out;
  int32_t dstride;       /* 1 (d_out = 1) or d_out rounded up to 4                 */
  int32_t row;           /* doubles per point row                                  */
  int32_t n_hb, n_vp, n_hot_dims, n_nodes, n_cold_groups, max_depth, n_terms;
  int32_t node_seg[5], cold_seg[5];  /* the 4 work segments over nodes and cold groups */
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int32_t* node;
  const double* node_c;     /* [n_nodes][dstride] own coefficients (0 for the root)  */
  const int32_t* cold;
  const double* cold_ab;    /* [G][2] a, b                                          */
  const int32_t* run;
  const double* terms;      /* [n_terms][2]                                         */
  const double* coef;       /* [n_terms][dstride] (d_out > 1), else NULL            */
  const double* fam_a;      /* [d_in]                                               */
  const double* fam_b;      /* [d_in]                                               */
  const int32_t* fam;       /* [d_in]                                               */
  const double* c0;         /* [d_out] coefficients of the constant                 */
} smx_spectral64;

/* y[P, d_out] (FP64) = the interpolant at the P rows of x (FP64, leading dimension ldx). */
int smx_spectral_eval64(const smx_spectral64* plan_host, const double* x, int64_t P, int64_t ldx, double* y,
                        void* stream);

/* Blocked FP32 evaluator of the orthogonal form for one output (d_out = 1):
 * the same polynomial as smx_spectral_eval, summed as
 *   y = c0 + sum over hot nodes a of V_a(x) * sum_{(a,s)} c * Phi_s(x)
 *          + sum over cold groups of sum_s (sum_{k<K} Vc_k(x) W[k][s]) * phi_s(x)
 * where hot slots/nodes are those of dimensions with children in the index
 * set, Vc_k the values of the prefixes of cold entries ordered by remaining
 * budget (the admissible prefixes of a cold slot are then a leading range, so
 * W is a staircase), and every group holds 4 cold slots.  Tables (host
 * struct of device pointers; int32 / float32):
 *   node[n_nodes][12]  entry offset, entry count (even), path depth, 0, path slots * 128 (8)
 *   vc[k_c][12]        same format, prefixes of cold entries
 *   hot_ent[2 * n]     (slot * 128, coefficient bits) pairs
 *   grp[G][12]         K, W offset, fast flag, slots, dims[4], degrees[4] (0 = unused)
 *   grp_ab[G][8]       a[4], b[4]: phi = a x + b (fast groups, degree 1) or z = a x + b
 *   W[sum 4 K]         staircase coefficients, [K][4] per group
 *   warp_off[17], items[n_items]: work list of each of the 16 warps of a block
 *                      (hot node index, or 2^30 | group index)
 * This re-expresses the reference's evaluation (interpolation.py:264-304) the
 * same way smx_spectral_eval does. */
typedef struct smx_blocked {
  int32_t d_in;
  int32_t n_hs;       /* hot basis slots                          */
  int32_t k_c;        /* prefix rows of cold entries              */
  int32_t n_hot_dims;
  int32_t n_nodes;
  int32_t n_groups;
  int32_t n_items;
  float c0;           /* coefficient of the constant              */
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int32_t* node;
  const int32_t* vc;
  const int32_t* hot_ent;
  const int32_t* grp;
  const float* grp_ab;
  const float* W;
  const int32_t* warp_off;
  const int32_t* items;
  const float* fa;    /* [d_in] affine map z = fa x + fb of every dimension */
  const float* fb;
  const int32_t* fam; /* [d_in] 0 Legendre, 1 Hermite                       */
  int32_t n_ent;      /* int32 words of hot_ent (a multiple of 4)          */
  int32_t n_w;        /* float4 rows of W                                  */
} smx_blocked;

/* Shared memory of one block's tile arrays: (n_hs + k_c) * 512 + 16384 bytes
 * (<= 220 KiB).  When n_ent and n_w are given and the tables fit beside the
 * tile arrays, smx_blocked_eval also keeps a copy of the tables (node, vc,
 * hot_ent, grp, grp_ab, W, items, warp_off) in each block's shared memory. */
size_t smx_blocked_smem(const smx_blocked* plan_host);
/* y[P] (FP32) at x[P, ldx] (FP64); one persistent block per SM.  When the
 * tiles leave a partial last round, its tiles are shared by several blocks
 * (fixed-order sum of their partial results). */
int smx_blocked_eval(const smx_blocked* plan_host, const double* x, int64_t P, int64_t ldx, float* y, void* ws,
                     size_t ws_bytes, void* stream);
/* Scratch for the split of the last round of tiles across blocks (partial
 * sums and counters); without it (ws = NULL) every tile is one block's work. */
size_t smx_blocked_eval_workspace(const smx_blocked* plan_host, int64_t P);

/* Tensor-core blocked evaluator (one output): an alternative to
 * smx_blocked_eval with ~2.5x smaller rounding error (max element-wise
 * 1.5e-7 against 3.9e-7 at d_in = 1000, |Lambda| = 9999) at ~1.6x its time;
 * no evaluation path selects it by itself.  The same sum split by the kind
 * of each entry's last factor: I(x) = c_0 + sum_a V_a(x) [ sum_s Bt[a][s]
 * Phi_s(x) + sum_j Bl[a][j] x_j ] over the nodes a (entries with children,
 * by remaining budget: the rows), the basis slots s of the table dimensions
 * (hot ones and cold ones of degree >= 2; slot 0 = 1) and the linear
 * dimensions j (cold, degree 1; phi_1(z_j) = alpha0 (fa x + fb) folded into
 * Bl and column 0 of Bt).  Per 128-point tile, T = A B runs on the tensor
 * cores in chunks of <= 64 columns (A = V in three bf16 parts built on chip
 * in tensor memory, B = the coefficients in three bf16 parts, six part
 * products per 16-row K step, FP32 accumulation) and y = c_0 + sum T x +
 * sum T Phi is summed in FP32 (Kahan) as x streams in (read once, units of 8
 * coordinates per point, prefetched to L2 chunks ahead).  Tables from
 * smx_layout_build (SMX_LAYOUT_BLOCKED_TC; names "tc_*").  Device pointers
 * unless noted:
 *   td[n_td][4]        dimension, degree, first basis slot, family
 *   tdab[n_td][2]      affine map a, b (z = a x + b)
 *   row[n_rows][4]     the 8 basis slots (16 bits each, 0 = the constant) of the node's path
 *   chunk[n_chunks][4] HOST: N | table << 16, K steps, stage offset / 16 bytes,
 *                      first basis slot (table chunks) or x box (linear chunks)
 *   bimg               coefficient stages in the order the kernel consumes them (16-byte aligned)
 *   box[n_boxes]       per unit of 8 linear columns: bit i set = dimension lin0 + 8 unit + i is
 *                      inactive or past d_in (masked: never read)
 *   err                int, 0 = ok; set when a pipeline wait ran out */
typedef struct smx_blocked_tc {
  int32_t d_in;
  int32_t n_td, n_phi, n_phi_pad, n_rows, max_depth;
  int32_t n_agen;     /* K steps of A built per tile (the chunks' largest; <= 16) */
  int32_t n_chunks, n_boxes, lin0, stages;
  int32_t td_col, td_bytes; /* x row segment of the table dimensions: first column, bytes (L2 prefetch) */
  float c0;
  const int32_t* td;
  const float* tdab;
  const int32_t* row;
  const int32_t* chunk;
  const void* bimg;
  const int32_t* box;
  int32_t* err;
} smx_blocked_tc;

/* 1 if smx_blocked_tc_eval serves x (16-byte aligned, even row pitch >= d_in;
 * 32-byte loads when x is 32-byte aligned and the pitch a multiple of 4). */
int smx_blocked_tc_supported(const smx_blocked_tc* plan_host, const double* x, int64_t ldx);
/* y[P] (FP32) at x[P, ldx] (FP64); one persistent block per SM (~140 KiB of
 * shared memory, all 512 tensor-memory columns); SMX_ERR_UNSUPPORTED for an
 * x it does not serve. */
int smx_blocked_tc_eval(const smx_blocked_tc* plan_host, const double* x, int64_t P, int64_t ldx, float* y,
                        void* stream);

/* Basis-product panel of the orthogonal form for the tensor-core contraction:
 * A[p][j] = prod over the pairs of entry j of phi_g(z_d) for the K non-root
 * entries of Lambda in DFS pre-order (tape word: basis slot | depth << 16,
 * depth <= 8), written as TF32 hi/lo pairs [P x lda] in REVERSED order (entry j
 * of the tape goes to column K-1-j: summing from small to large terms limits
 * the truncation of the tensor cores' FP32 accumulation).  Basis slots: for each
 * listed dimension dims[h], degrees 1..dmax[h] at dsoff[h].  The tape is walked
 * in n_seg independent segments [seg[s], seg[s+1]) (seg[0] = 0, seg[n_seg] = K,
 * every seg[s] the position of a depth-1 entry; seg may be NULL for n_seg = 1),
 * one block of points per segment. */
size_t smx_spectral_panel_workspace(int n_slots, int64_t P);
int smx_spectral_panel_tf32(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff, int n_slots,
                            const int32_t* tape, int K, const int32_t* seg, int n_seg, const float* fam_a,
                            const float* fam_b, const int32_t* fam, const double* x, int64_t P, int64_t ldx,
                            float* A_hi, float* A_lo, int64_t lda, void* ws, size_t ws_bytes, void* stream);
/* Same panel as BF16 hi/lo pairs (hi = BF16 rounded to nearest, lo = BF16 of
 * the remainder; bit patterns, 2 bytes each) for smx_gemm_bf16x3. */
int smx_spectral_panel_bf16(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff, int n_slots,
                            const int32_t* tape, int K, const int32_t* seg, int n_seg, const float* fam_a,
                            const float* fam_b, const int32_t* fam, const double* x, int64_t P, int64_t ldx,
                            uint16_t* A_hi, uint16_t* A_lo, int64_t lda, void* ws, size_t ws_bytes, void* stream);

/* Backward of the orthogonal form (no counterpart in the reference, whose
 * derivative is the dense Jacobian of interpolation.py:306-345):
 *  - smx_spectral_panel_t_tf32: the transposed panel AT[K-1-j][p] (point-
 *    contiguous, same columns as smx_spectral_panel_tf32) for dL/dC = A^T g;
 *    the basis values go through `ws` (smx_spectral_panel_t_workspace bytes);
 *  - smx_spectral_vjp_x: dL/dx[p][d] from G = g C^T ([P x ldg], columns in the
 *    panel's reversed order): reverse pass through the basis products, one
 *    warp per 32 points; with n_seg > 1 the tape is walked in the segments
 *    seg[0..n_seg] (device int32 bounds, each but the last at a depth-1 entry,
 *    as for smx_spectral_panel_tf32) by separate warps with their own
 *    adjoint copies, which a last kernel sums (more parallelism for long
 *    tapes; the result does not depend on the number of points); basis values
 *    and adjoints in `ws` (smx_spectral_vjp_x_workspace bytes);
 *  - smx_spectral_coefficients_adjoint: adjoint of smx_spectral_coefficients,
 *    Fbar[r] = (A_1^T x ... x A_n^T) Cbar[ids] per summand (FP64). */
size_t smx_spectral_panel_t_workspace(int n_slots, int64_t P);
int smx_spectral_panel_t_tf32(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff,
                              int n_slots, const int32_t* tape, int K, const float* fam_a, const float* fam_b,
                              const int32_t* fam, const double* x, int64_t P, int64_t ldx, float* AT_hi, float* AT_lo,
                              int64_t ldp, void* ws, size_t ws_bytes, void* stream);
size_t smx_spectral_vjp_x_workspace(int n_slots, int n_seg, int64_t P);
int smx_spectral_vjp_x(int n_dims, const int32_t* dims, const int32_t* dmax, const int32_t* dsoff, int n_slots,
                       const int32_t* tape, int K, const int32_t* seg, int n_seg, const float* fam_a,
                       const float* fam_b, const int32_t* fam, const double* x, int64_t P, int64_t ldx, const float* G,
                       int64_t ldg, double* dx, int64_t lddx, void* ws, size_t ws_bytes, void* stream);
int smx_spectral_coefficients_adjoint(const smx_plan* plan_host, const int64_t* aoff, const double* A,
                                      const int32_t* ids, const double* Cbar, double* Fbar, void* stream);

/* Serving: one persistent launch evaluating many work items (interpolant,
 * inputs, outputs) of different plans and batch sizes; CTAs take 128-point
 * tiles from a shared counter.  `plans` and `items` are HOST arrays (copied
 * into the workspace); ws >= smx_spectral_eval_batch_workspace(n_plans,
 * n_items, largest d_out).  Results equal those of smx_spectral_eval. */
typedef struct smx_work {
  int32_t plan;     /* index into plans                                          */
  int32_t reserved;
  const double* x;  /* [P, ldx] FP64 inputs (device)                             */
  int64_t P, ldx;
  float* y;         /* [P, d_out] FP32 outputs (device)                          */
} smx_work;
size_t smx_spectral_eval_batch_workspace(int n_plans, int n_items, int max_d_out);
int smx_spectral_eval_batch(const smx_spectral* plans, int n_plans, const smx_work* items, int n_items, void* ws,
                            size_t ws_bytes, void* stream);

/* Serving: one persistent launch over the 128-point tiles of many work items
 * (struct smx_work, `plan` indexing `plans`), each of a blocked plan; every
 * tile is evaluated exactly as by smx_blocked_eval.  Workspace:
 * smx_blocked_eval_batch_workspace bytes (device). */
size_t smx_blocked_eval_batch_workspace(int n_plans, int n_items);
int smx_blocked_eval_batch(const smx_blocked* plans_host, int n_plans, const smx_work* items_host, int n_items,
                           void* ws, size_t ws_bytes, void* stream);

/* Serving queue: submit FP32 evaluation requests (plan, inputs, outputs) and
 * poll for their completion, the continuous-batching loop of the serving path
 * without a host runtime.  smx_serve_flush launches everything queued as one
 * smx_blocked_eval_batch launch (blocked plans) and one
 * smx_spectral_eval_batch launch (per-point plans, d_out <= 16) on the
 * server's stream and records an event; a submit that finds its kind's queue
 * full (max_items requests, or a new plan beyond max_plans distinct ones)
 * flushes first.  Up to max_inflight flushes are outstanding; the next one
 * waits for the oldest.  Results equal those of smx_blocked_eval /
 * smx_spectral_eval on the same request.
 *  - smx_serve_create: allocates the workspaces of max_inflight flushes (the
 *    only allocation; submit / flush / poll allocate nothing);
 *  - smx_serve_submit: `plan_host` is a host smx_blocked (kind
 *    SMX_SERVE_BLOCKED) or smx_spectral (SMX_SERVE_SPECTRAL), identified by
 *    its address until the request is flushed; x / y device, as for the batch
 *    entry points.  Returns the ticket (>= 0, in submission order) or an
 *    SMX_ERR_* code;
 *  - smx_serve_flush: a flush whose launch is refused (e.g. a per-point plan
 *    beyond shared memory) or fails returns the error and fails all its
 *    requests; the queue is then empty and takes new requests;
 *  - smx_serve_poll: 1 if the ticket's outputs are written, 0 if it is queued
 *    or running, or the SMX_ERR_* code of its failed flush;
 *  - smx_serve_destroy: waits for the flushes in flight and frees the server.
 * A server is used by one host thread at a time. */
#define SMX_SERVE_BLOCKED 0
#define SMX_SERVE_SPECTRAL 1
typedef struct smx_server smx_server;
int smx_serve_create(int max_items, int max_plans, int max_inflight, void* stream, smx_server** out);
int64_t smx_serve_submit(smx_server* server, int kind, const void* plan_host, const double* x, int64_t P, int64_t ldx,
                         float* y);
int smx_serve_flush(smx_server* server);
int smx_serve_poll(smx_server* server, int64_t ticket);
void smx_serve_destroy(smx_server* server);


/* ---- tensor-core contraction ---------------------------------------------------------
 * D[M x N] = A B^T (+ bias[n]) with tcgen05.mma kind::tf32 in 3xTF32 form:
 * A = A_hi + A_lo, B = B_hi + B_lo (row-major [M x K] and [N x K], leading
 * dimensions multiples of 4, 16-byte aligned), D = A_hi B_hi^T + A_hi B_lo^T +
 * A_lo B_hi^T accumulated in FP32 in tensor memory (accumulate != 0: added to
 * the existing D).  *err (device int) is set
 * non-zero if a pipeline wait timed out.  Used for the orthogonal-form
 * contraction when d_out is large (the dense [points x Lambda] x [Lambda x
 * d_out] product of interpolation.py:264-304 in orthogonal form) and for the
 * backward products. */
int smx_gemm_tf32x3(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi, const float* B_lo,
                    int64_t ldb, int M, int N, int K, float* D, int64_t ldd, const float* bias, int accumulate, int* err,
                    void* stream);
/* Same product with the K range split into up to `splits` slices that run side
 * by side (for small M x N with long K, e.g. the backward's dL/dC over all
 * points); the slices' FP32 results go to `ws` and are added in slice order
 * (deterministic).  ws: smx_gemm_tf32x3_splitk_workspace bytes. */
size_t smx_gemm_tf32x3_splitk_workspace(int M, int N, int K, int splits);
/* Split count for the forward contraction of a plan whose panel chunks hold M
 * points: enough K slices that the CTAs of one full chunk (128 x 128 tiles, or
 * 128 x 256 for N > 192) fill the SMs once, at most 8 slices and at least 64
 * K-tiles (2048 products) per slice; 1 where the tiles alone fill the GPU.  A
 * function of (M, N, K) and the SM count only, so that for a fixed chunk size
 * a point's result does not depend on the batch it is evaluated in. */
int smx_gemm_tf32x3_splits(int64_t M, int N, int K);
int smx_gemm_tf32x3_splitk(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi, const float* B_lo,
                           int64_t ldb, int M, int N, int K, float* D, int64_t ldd, const float* bias, int accumulate,
                           int splits, void* ws, size_t ws_bytes, int* err, void* stream);

/* Test of the contraction's failure detection (no counterpart in the
 * reference): runs smx_gemm_tf32x3's kernel with its copy producer switched
 * off, so the first pipeline wait times out after wait_ns (<= 2 s); the
 * kernel then sets *err = 2 and returns without writing D.  Every other
 * entry point uses the 2 s bound. */
int smx_gemm_tf32x3_timeout_selftest(const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi,
                                     const float* B_lo, int64_t ldb, int M, int N, int K, float* D, int64_t ldd,
                                     int* err, uint64_t wait_ns, void* stream);

/* Split-BF16 form of the same contraction (kind::f16, both operands BF16,
 * FP32 accumulation): D = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T with
 * A = A_hi + A_lo, B = B_hi + B_lo in BF16 (2-byte bit patterns; leading
 * dimensions multiples of 8).  About 16 significant bits per product: an
 * option for d_out >= 16 when ~1e-5 relative error is acceptable. */
int smx_gemm_bf16x3(const uint16_t* A_hi, const uint16_t* A_lo, int64_t lda, const uint16_t* B_hi,
                    const uint16_t* B_lo, int64_t ldb, int M, int N, int K, float* D, int64_t ldd, const float* bias,
                    int accumulate, int* err, void* stream);
/* hi = BF16(src), lo = BF16(src - hi) for a [rows x cols] block (2-byte outputs). */
int smx_split_bf16(const float* src, int64_t rows, int64_t cols, int64_t lds, uint16_t* hi, uint16_t* lo,
                   int64_t ldo, void* stream);

/* hi = TF32(src), lo = TF32(src - hi) for a [rows x cols] block. */
int smx_split_tf32(const float* src, int64_t rows, int64_t cols, int64_t lds, float* hi, float* lo, int64_t ldo,
                   void* stream);

/* ---- host-side layout builders of the FP32 evaluators ------------------------------
 * The tables of the blocked one-output evaluator (smx_blocked), of the
 * per-point evaluator (smx_spectral) and the entry tape of the tensor-core
 * panel, built on the host from host copies of the index-set tree (entry 0 =
 * root, parent[0] = -1; level = number of non-zero entries; rank = DFS
 * pre-order rank, as smx_lambda_ranks writes it in SMX_MODE_PREORDER) and the
 * FP32 coefficients C[n][d_out] of every entry.  They re-express the
 * reference's evaluation (interpolation.py:264-304) as the smx_spectral /
 * smx_blocked comments describe; smx_fp32_plan_create uses them.  Tables are
 * read back by name (the field names of smx_blocked / smx_spectral, plus
 * "dims", "dmax", "dsoff", "tape", "ent", "lvl1" of the tape). */
#define SMX_LAYOUT_BLOCKED 0
#define SMX_LAYOUT_PERPOINT 1
#define SMX_LAYOUT_TAPE 2
#define SMX_LAYOUT_BLOCKED_TC 3
typedef struct smx_host_tables smx_host_tables;
int smx_layout_build(int kind, int64_t n, const int32_t* parent_host, const int32_t* dim_host,
                     const int32_t* deg_host, const int32_t* level_host, const int64_t* rank_host,
                     const double* rem_host, const float* C_host, int d_out, const int64_t* maxdeg_host, int d,
                     const int32_t* fam_host, const double* fam_a_host, const double* fam_b_host,
                     smx_host_tables** out);
/* The layout of the FP64 evaluator (smx_spectral64) from FP64 coefficients
 * C[n][d_out]: kind SMX_LAYOUT_PERPOINT only (its FP64 form); tables
 * "node_c", "cold_ab", "terms", "coef" are read with smx_layout_f64, the others
 * with smx_layout_i32 and smx_layout_scalar. */
int smx_layout_build_f64(int kind, int64_t n, const int32_t* parent_host, const int32_t* dim_host,
                         const int32_t* deg_host, const int32_t* level_host, const int64_t* rank_host,
                         const double* rem_host, const double* C_host, int d_out, const int64_t* maxdeg_host, int d,
                         const int32_t* fam_host, const double* fam_a_host, const double* fam_b_host,
                         smx_host_tables** out);
int smx_layout_i32(const smx_host_tables* tables, const char* name, const int32_t** data_host, int64_t* count);
int smx_layout_f32(const smx_host_tables* tables, const char* name, const float** data_host, int64_t* count);
int smx_layout_f64(const smx_host_tables* tables, const char* name, const double** data_host, int64_t* count);
int smx_layout_scalar(const smx_host_tables* tables, const char* name, double* value);
void smx_layout_free(smx_host_tables* tables);

/* ---- FP32 form of a plan behind the C ABI -------------------------------------------
 * smx_fp32_plan_create builds the orthogonal-polynomial form of an FP64 plan
 * (coefficients in FP64 on the device: smx_spectral_pairs and
 * smx_spectral_coefficients; pair degrees up to 23) and the tables of the
 * evaluator that serves it: the blocked evaluator for one output, the
 * per-point evaluator for 2..15 outputs, the tcgen05 3xTF32 contraction for
 * 16 or more outputs (or rows too large for the per-point evaluator).  It is
 * what the Python package builds for precision="fp32" (the same host layout
 * builders), replacing interpolation.py:264-304 in FP32.  The tree is the
 * index set built by smx_lambda_* in SMX_MODE_NONZERO (device arrays); fam /
 * fam_a / fam_b (host, [d_in]) are each dimension's polynomial family (0
 * Legendre, 1 Hermite) and affine map z = a x + b of its node rule.  The
 * handle keeps `plan_host` (which must outlive it) and owns device memory for
 * its tables (allocated here, released by smx_fp32_plan_destroy);
 * memory_limit_gib bounds the points per tensor-core chunk.  The call
 * synchronises `stream`. */
typedef struct smx_tree {
  int64_t n;                  /* entries, root first                            */
  const int32_t* parent;      /* [n] (-1 for the root)                          */
  const int32_t* dim;         /* [n] last non-zero entry (dim, deg)             */
  const int32_t* deg;         /* [n]                                            */
  const double* rem;          /* [n] remaining budget                           */
  const int64_t* first_child; /* [n] children range (smx_lambda_expand order)  */
  const int64_t* n_child;     /* [n]                                            */
} smx_tree;
typedef struct smx_fp32_plan smx_fp32_plan;
#define SMX_FP32_BLOCKED 0
#define SMX_FP32_PERPOINT 1
#define SMX_FP32_TENSOR 2
int smx_fp32_plan_create(const smx_plan* plan_host, const smx_tree* tree_host, const int32_t* fam_host,
                         const double* fam_a_host, const double* fam_b_host, double memory_limit_gib,
                         smx_fp32_plan** out, void* stream);
void smx_fp32_plan_destroy(smx_fp32_plan* fp32);
/* Evaluator (SMX_FP32_*), |Lambda| and the device FP64 coefficients [n_lambda][d_out]. */
int smx_fp32_plan_info(const smx_fp32_plan* fp32, int* evaluator, int64_t* n_lambda, const double** coef);
/* y[P, d_out] (FP32) at x[P, ldx] (FP64). */
size_t smx_fp32_workspace(const smx_fp32_plan* fp32, int64_t P);
int smx_fp32_eval(const smx_fp32_plan* fp32, const double* x, int64_t P, int64_t ldx, float* y, void* ws,
                  size_t ws_bytes, void* stream);
/* SMX_OK, or SMX_ERR_CUDA if a tensor-core pipeline wait of an earlier call
 * timed out (those results are invalid); resets the flag; synchronises. */
int smx_fp32_plan_check(const smx_fp32_plan* fp32, void* stream);
/* FP64 evaluation of the orthogonal form, y[P, d_out] (FP64), for plans whose
 * per-point row fits the FP64 evaluator (smx_spectral64; the handle builds
 * those tables when it can): SMX_ERR_UNSUPPORTED otherwise.
 * smx_eval(plan, 64, ...) evaluates through it when plan->fp32 is set and has
 * them, as the Python package does for precision "fp64". */
int smx_fp32_plan_has_fp64(const smx_fp32_plan* fp32);
int smx_fp32_eval64(const smx_fp32_plan* fp32, const double* x, int64_t P, int64_t ldx, double* y, void* stream);
/* Vector-Jacobian products of y = I(x) (the FP32 form) at the cotangent
 * g[P, ldg] (FP32): dx[P, lddx] = dL/dx (FP64; NULL to skip) and
 * dF[n_entries, d_out] = dL/d(plan rows F64) (FP64; NULL to skip).  The
 * reference has no hand-written derivative w.r.t. the nodal values; dL/dx is
 * the transpose of its Jacobian (barycentric.py:126-229,
 * interpolation.py:306-345) applied to g.  Needs index-set depth <= 8. */
size_t smx_vjp_workspace(const smx_fp32_plan* fp32, int64_t P);
int smx_vjp(const smx_fp32_plan* fp32, const double* x, int64_t P, int64_t ldx, const float* g, int64_t ldg,
            double* dx, int64_t lddx, double* dF, void* ws, size_t ws_bytes, void* stream);

/* ---- allocation-free FP64 evaluation -------------------------------------------------
 * No counterpart in the reference: an added entry point for callers that
 * cannot allocate device memory while evaluating (FFI hosts without a CUDA
 * allocator, services whose device memory belongs to a pool, code that must
 * not call cudaMalloc because it synchronises the device).  Same result as
 * smx_eval(plan, 64, ...), but the basis table lives in a library-owned
 * device array of SMX_STATIC_SCRATCH_BYTES (held by every GPU that loads the
 * library until the process exits); nothing is allocated.  Calls whose table
 * (n_values * P doubles) does not fit return SMX_ERR_WORKSPACE: split the
 * points.  The first call on a device looks up the array's address with that
 * device current -- make it before any stream capture; the address is looked
 * up again when the device's context changes (after a device reset).  All
 * calls share the array, so calls that overlap on the GPU race: serialise them. */
#define SMX_STATIC_SCRATCH_BYTES (32u << 20)
int smx_eval_f64_noalloc(const smx_plan* plan_host, const double* x, int64_t P, int64_t ldx, double* y,
                         void* stream);

/* Device address of page-locked (pinned) host memory, for kernels that read
 * host inputs directly over the host link instead of copying them first;
 * SMX_ERR_ARG if `host` is not page-locked host memory, SMX_ERR_UNSUPPORTED
 * if it is not mapped for the current device.  (No counterpart in the
 * reference: its inputs are copied to the device by JAX, interpolation.py:257.) */
int smx_host_device_pointer(const void* host, void** dev);

/* Human-readable description of the last error on this thread (host string). */
const char* smx_last_error_string(void);

/* Library version string (host). */
const char* smx_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SMOLYAX_GB300_H */
