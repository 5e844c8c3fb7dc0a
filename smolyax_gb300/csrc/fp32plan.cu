// The FP32 (orthogonal-polynomial) form of a plan behind the C ABI: built from
// the FP64 plan and the index-set tree, evaluated by the evaluator that serves
// it (blocked one-output evaluator, per-point evaluator, or the tcgen05
// contraction), and differentiated (dL/dx and dL/d rows of F64).
//
// The build runs the same steps as the Python package (spectral.py
// SpectralPlan): coefficients in FP64 on the device, host layout of the
// chosen evaluator (layout.cu, identical tables), upload.  The handle owns
// the device memory of its tables (allocated at creation, freed by
// smx_fp32_plan_destroy); evaluation and the VJP take caller scratch.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "layout.h"

namespace {

constexpr int kTcMinDout = 16;  // from this many outputs on, the tensor-core contraction
constexpr int kMaxPairDegree = 23;
constexpr size_t kAlign = 256;

size_t up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
int64_t round4(int64_t v) { return (v + 3) / 4 * 4; }
int64_t round32(int64_t v) { return (v + 31) / 32 * 32; }

// dst[o][r] (row pitch ldd) = src[r][o] for o < cols, 0 for cols <= o < ldo; r < rows
__global__ void transpose_pad_kernel(const float* __restrict__ src, int64_t lds, int rows, int cols, int ldo,
                                     float* __restrict__ dst, int64_t ldd) {
  const int64_t n = int64_t(rows) * ldo;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t o = i / rows, r = i - o * rows;
    dst[o * ldd + r] = o < cols ? src[r * lds + o] : 0.f;
  }
}

// dst[p][o] = src[p][o] for o < cols, 0 for cols <= o < ldo
__global__ void pad_rows_kernel(const float* __restrict__ src, int64_t lds, int64_t rows, int cols, int ldo,
                                float* __restrict__ dst) {
  const int64_t n = rows * ldo;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t p = i / ldo, o = i - p * ldo;
    dst[i] = o < cols ? src[p * lds + o] : 0.f;
  }
}

// dC[ent[K-1-j]][o] = dCrev[j][o] (FP64); dC[0][o] = sum_p g[p][o] (fixed order)
__global__ void scatter_dc_kernel(const float* __restrict__ dCrev, const int32_t* __restrict__ ent, int K, int dout,
                                  const float* __restrict__ g, int64_t ldg, int64_t P, double* __restrict__ dC) {
  const int64_t n = int64_t(K) * dout;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n + dout;
       i += int64_t(gridDim.x) * blockDim.x) {
    if (i < n) {
      const int64_t j = i / dout, o = i - j * dout;
      dC[int64_t(ent[K - 1 - j]) * dout + o] = double(dCrev[i]);
    } else {
      const int o = int(i - n);
      double s = 0.0;
      for (int64_t p = 0; p < P; ++p) s += double(g[p * ldg + o]);
      dC[o] = s;
    }
  }
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t count) {
    n = count;
    if (count == 0) return SMX_OK;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) {
      p = nullptr;
      return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: device allocation failed");
    }
    return SMX_OK;
  }
  int upload(const std::vector<T>& v, cudaStream_t st) {
    int rc = alloc(v.size());
    if (rc || v.empty()) return rc;
    if (cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: upload failed");
    return SMX_OK;
  }
};

template <typename T>
int download(std::vector<T>& out, const T* src, size_t n, cudaStream_t st) {
  out.resize(n);
  if (n && cudaMemcpyAsync(out.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: download failed");
  return SMX_OK;
}

}  // namespace

struct smx_fp32_plan {
  int evaluator = -1;  // SMX_FP32_BLOCKED / SMX_FP32_PERPOINT / SMX_FP32_TENSOR
  const smx_plan* plan = nullptr;
  int d_in = 0, d_out = 0, sms = 0;
  int64_t n_lambda = 0;
  double memory_limit = 4.0;
  // coefficients and the adjoint's operands
  DevBuf<double> C64, A;
  DevBuf<int64_t> aoff;
  DevBuf<int32_t> ids;
  // per-dimension family and affine map (FP32, as the kernels read them)
  DevBuf<float> fam_a, fam_b;
  DevBuf<int32_t> fam;
  // blocked / per-point tables: one int32 and one float blob
  DevBuf<int32_t> ti;
  DevBuf<float> tf;
  smx_blocked blocked{};
  smx_spectral spectral{};
  // tape of the tensor-core panel (forward on the tensor cores, and the VJP of every evaluator)
  bool have_tape = false;
  int K = 0, ldk = 0, ldo = 0, n_slots = 0, n_dims = 0;
  DevBuf<int32_t> dims, dmax, dsoff, tape, ent, segs, err;
  DevBuf<float> Bh, Bl, bias, Rh, Rl;
  std::vector<int32_t> lvl1;
  std::vector<int> seg_off, seg_n;  // per wanted segment count: offset into segs, number of segments
  int vjp_want = 1;                 // tape segments of the gradient walk (fixed per plan)
  // FP64 per-point tables of the orthogonal form (one output), when they fit
  bool have64 = false;
  DevBuf<int32_t> ti64;
  DevBuf<double> tf64, fa64, fb64;
  smx_spectral64 spectral64{};
};

namespace {

// Named tables packed into one int32 and one float blob (16-byte aligned each).
struct Blobs {
  std::vector<int32_t> i;
  std::vector<float> f;
  std::vector<std::pair<std::string, size_t>> io, fo;
  void add(const smx::layout::Tables& t, const char* name) {
    auto it = t.i32.find(name);
    if (it != t.i32.end()) {
      io.push_back({name, i.size()});
      i.insert(i.end(), it->second.begin(), it->second.end());
      i.resize(round4(int64_t(i.size())), 0);
      return;
    }
    auto jt = t.f32.find(name);
    fo.push_back({name, f.size()});
    f.insert(f.end(), jt->second.begin(), jt->second.end());
    f.resize(round4(int64_t(f.size())), 0.f);
  }
  const int32_t* ip(const smx_fp32_plan* h, const char* name) const {
    for (const auto& kv : io)
      if (kv.first == name) return h->ti.p + kv.second;
    return nullptr;
  }
  const float* fp(const smx_fp32_plan* h, const char* name) const {
    for (const auto& kv : fo)
      if (kv.first == name) return h->tf.p + kv.second;
    return nullptr;
  }
};

// Named tables of one type packed into one blob, each 4-element aligned.
template <typename T>
struct Pack {
  std::vector<T> v;
  std::vector<std::pair<std::string, size_t>> off;
  void add(const char* name, const std::vector<T>& src) {
    off.push_back({name, v.size()});
    v.insert(v.end(), src.begin(), src.end());
    v.resize(size_t(round4(int64_t(v.size()))), T(0));
  }
  // device address of a table in the uploaded blob, NULL for an empty table
  const T* at(const T* base, const char* name, const std::vector<T>& src) const {
    if (src.empty()) return nullptr;
    for (const auto& kv : off)
      if (kv.first == name) return base + kv.second;
    return nullptr;
  }
};

size_t size_of(const smx::layout::Tables& t, const char* name) {
  auto it = t.i32.find(name);
  if (it != t.i32.end()) return it->second.size();
  auto jt = t.f32.find(name);
  return jt == t.f32.end() ? 0 : jt->second.size();
}

// Points per tensor-core chunk (the TF32 hi/lo panel of one chunk fits the memory limit).
int64_t tc_step(const smx_fp32_plan* h, int64_t P) {
  const int64_t per = 8 * round32(std::max(h->K, 1));
  int64_t step = int64_t(h->memory_limit * 1073741824.0 / double(per)) / 128 * 128;
  step = std::max<int64_t>(128, step);
  return std::max<int64_t>(1, std::min(step, P));
}

// K slices of the forward contraction: fixed per plan (from its full chunk),
// as in the package, so that both give the same values.
int tc_splits(const smx_fp32_plan* h) {
  return smx_gemm_tf32x3_splits(tc_step(h, int64_t(1) << 40), h->d_out, h->K);
}

// Segments of one panel launch over n points (spectral.py segment_count).
int seg_want(const smx_fp32_plan* h, int64_t n) {
  const int64_t n_pb = std::max<int64_t>((n + 127) / 128, 1);
  int64_t want = std::min<int64_t>(32, (12 * int64_t(h->sms) + n_pb - 1) / n_pb);
  want = std::min<int64_t>(want, h->K / 256);
  want = std::min<int64_t>(want, int64_t(h->lvl1.size()));
  return int(std::max<int64_t>(1, want));
}

}  // namespace

extern "C" int smx_fp32_plan_create(const smx_plan* pl, const smx_tree* tree, const int32_t* fam_h, const double* fa_h,
                                    const double* fb_h, double memory_limit_gib, smx_fp32_plan** out, void* stream) {
  SMX_REQUIRE(out && pl && tree && fam_h && fa_h && fb_h && memory_limit_gib > 0,
              "smx_fp32_plan_create: bad arguments");
  SMX_REQUIRE(tree->n >= 1 && tree->parent && tree->dim && tree->deg && tree->rem && tree->first_child &&
                  tree->n_child && pl->d_in >= 1 && pl->d_out >= 1,
              "smx_fp32_plan_create: bad tree or plan");
  *out = nullptr;
  cudaStream_t st = smx::as_stream(stream);
  auto h = std::make_unique<smx_fp32_plan>();
  h->plan = pl;
  h->d_in = pl->d_in;
  h->d_out = pl->d_out;
  h->n_lambda = tree->n;
  h->memory_limit = memory_limit_gib;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: no device");
  const int d = pl->d_in, dout = pl->d_out;
  const int64_t n = tree->n;
  int rc;

  // tree on the host; levels (parents precede children) and pre-order ranks
  std::vector<int32_t> parent, tdim, tdeg, pdeg_h;
  std::vector<double> rem;
  std::vector<int64_t> first_child, n_child;
  if ((rc = download(parent, tree->parent, n, st)) || (rc = download(tdim, tree->dim, n, st)) ||
      (rc = download(tdeg, tree->deg, n, st)) || (rc = download(rem, tree->rem, n, st)) ||
      (rc = download(first_child, tree->first_child, n, st)) || (rc = download(n_child, tree->n_child, n, st)) ||
      (rc = download(pdeg_h, pl->pair_deg, size_t(pl->n_pairs), st)))
    return rc;
  if (cudaStreamSynchronize(st) != cudaSuccess) return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: sync failed");
  std::vector<int32_t> level(n, 0);
  for (int64_t e = 1; e < n; ++e) level[e] = level[parent[e]] + 1;
  // pre-order ranks as smx_lambda_ranks writes them in SMX_MODE_PREORDER (the
  // order the package builds its tables in): an entry before its children,
  // the children by dimension ascending and, within a dimension, by degree
  // descending (children are stored dimension- then degree-ascending)
  std::vector<int64_t> rank(n, 0);
  {
    std::vector<int64_t> stack{0}, visit;
    int64_t r = 0;
    while (!stack.empty()) {
      const int64_t e = stack.back();
      stack.pop_back();
      rank[e] = r++;
      visit.clear();
      const int64_t c0 = first_child[e], nc = n_child[e];
      for (int64_t c = 0; c < nc;) {
        int64_t c1 = c;
        while (c1 < nc && tdim[c0 + c1] == tdim[c0 + c]) ++c1;
        for (int64_t q = c1 - 1; q >= c; --q) visit.push_back(c0 + q);
        c = c1;
      }
      for (auto it = visit.rbegin(); it != visit.rend(); ++it) stack.push_back(*it);
    }
  }
  std::vector<int64_t> maxdeg(d, 0);
  for (int64_t e = 1; e < n; ++e) maxdeg[tdim[e]] = std::max<int64_t>(maxdeg[tdim[e]], tdeg[e]);

  // coefficients over Lambda (FP64): per pair A = V^-1, then the summands' mode products
  int max_pdeg = 0;
  std::vector<int64_t> aoff_h(size_t(std::max(pl->n_pairs, 1)), 0);
  int64_t a_total = 0;
  for (int u = 0; u < pl->n_pairs; ++u) {
    aoff_h[u] = a_total;
    a_total += int64_t(pdeg_h[u] + 1) * (pdeg_h[u] + 1);
    max_pdeg = std::max(max_pdeg, pdeg_h[u]);
  }
  if (max_pdeg > kMaxPairDegree)
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_fp32_plan_create: pair degree " + std::to_string(max_pdeg) +
                                                   " above " + std::to_string(kMaxPairDegree));
  std::vector<int32_t> fam_v(fam_h, fam_h + d);
  std::vector<double> fa_v(fa_h, fa_h + d), fb_v(fb_h, fb_h + d);
  DevBuf<double> fa64, fb64, G;
  DevBuf<int32_t> flag;
  if ((rc = h->aoff.upload(aoff_h, st)) || (rc = h->A.alloc(size_t(std::max<int64_t>(a_total, 1)))) ||
      (rc = fa64.upload(fa_v, st)) || (rc = fb64.upload(fb_v, st)) || (rc = h->fam.upload(fam_v, st)) ||
      (rc = flag.upload(std::vector<int32_t>{0}, st)))
    return rc;
  if ((rc = smx_spectral_pairs(pl->n_pairs, pl->pair_dim, pl->pair_deg, pl->pair_voff, h->aoff.p, pl->node, h->fam.p,
                               fa64.p, fb64.p, h->A.p, flag.p, stream)))
    return rc;
  const int64_t R = pl->n_entries;
  if ((rc = G.alloc(size_t(std::max<int64_t>(R * dout, 1)))) || (rc = h->ids.alloc(size_t(std::max<int64_t>(R, 1)))) ||
      (rc = h->C64.alloc(size_t(n * dout))))
    return rc;
  DevBuf<uint8_t> cws;
  if ((rc = cws.alloc(std::max<size_t>(smx_spectral_coefficients_workspace(pl), 1)))) return rc;
  if ((rc = smx_spectral_coefficients(pl, h->aoff.p, h->A.p, tree->first_child, tree->n_child, tree->dim, tree->deg, n,
                                      G.p, h->ids.p, h->C64.p, flag.p, cws.p, cws.n, stream)))
    return rc;
  std::vector<double> C64_h;
  std::vector<int32_t> flag_h;
  if ((rc = download(C64_h, h->C64.p, size_t(n * dout), st)) || (rc = download(flag_h, flag.p, 1, st))) return rc;
  if (cudaStreamSynchronize(st) != cudaSuccess) return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: sync failed");
  if (flag_h[0]) return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_fp32_plan_create: orthogonal-basis set-up failed");
  std::vector<float> C32(C64_h.begin(), C64_h.end());
  std::vector<float> fa32(fa_v.begin(), fa_v.end()), fb32(fb_v.begin(), fb_v.end());
  if ((rc = h->fam_a.upload(fa32, st)) || (rc = h->fam_b.upload(fb32, st))) return rc;

  // evaluator: tensor core for many outputs or rows too large for the per-point
  // evaluator's shared memory; blocked for one output when its tables fit
  smx::layout::Tree tr{n, parent.data(), tdim.data(), tdeg.data(), level.data(), rank.data(), rem.data()};
  smx::layout::Tables pp, bl, tp;
  smx::layout::build_perpoint(tr, C32.data(), dout, maxdeg.data(), d, fam_v.data(), fa_v.data(), fb_v.data(), pp);
  const int64_t row = int64_t(pp.scalar["row"]);
  const bool stream_fits = (row + 4 * (dout == 1 ? 1 : 4) * 2) * 128 * 4 <= 220 * 1024;
  h->have_tape = smx::layout::build_tape(tr, maxdeg.data(), d, tp);
  const bool use_tc = (dout >= kTcMinDout || !stream_fits) && h->have_tape;
  bool use_blocked = false;
  if (!use_tc && dout == 1)
    use_blocked = smx::layout::build_blocked(tr, C32.data(), maxdeg.data(), d, fam_v.data(), fa_v.data(), fb_v.data(), bl);
  if (!use_tc && !stream_fits)
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_fp32_plan_create: no FP32 evaluator serves this plan");
  if ((rc = h->err.upload(std::vector<int32_t>{0}, st))) return rc;

  if (h->have_tape) {
    h->K = int(tp.scalar["K"]);
    h->ldk = int(round32(std::max(h->K, 1)));
    h->ldo = int(round4(dout));
    h->n_slots = int(tp.scalar["n_slots"]);
    h->n_dims = int(tp.i32["dims"].size());
    h->lvl1 = tp.i32["lvl1"];
    const std::vector<int32_t>& ent = tp.i32["ent"];
    // B[o][j] = C32[ent[K-1-j]][o] (the panel stores the entries in reversed
    // pre-order) for the forward; rows R[j][o] in the same order for the VJP
    std::vector<float> B(use_tc ? size_t(dout) * h->ldk : 0, 0.f), Rrows(size_t(std::max(h->K, 1)) * h->ldo, 0.f);
    std::vector<float> c0(dout);
    for (int j = 0; j < h->K; ++j)
      for (int o = 0; o < dout; ++o) {
        const float v = C32[size_t(ent[h->K - 1 - j]) * dout + o];
        if (use_tc) B[size_t(o) * h->ldk + j] = v;
        Rrows[size_t(j) * h->ldo + o] = v;
      }
    for (int o = 0; o < dout; ++o) c0[o] = C32[o];
    DevBuf<float> Bd, Rd;
    if ((rc = h->dims.upload(tp.i32["dims"], st)) || (rc = h->dmax.upload(tp.i32["dmax"], st)) ||
        (rc = h->dsoff.upload(tp.i32["dsoff"], st)) || (rc = h->tape.upload(tp.i32["tape"], st)) ||
        (rc = h->ent.upload(ent, st)) || (rc = h->bias.upload(c0, st)) || (rc = Rd.upload(Rrows, st)) ||
        (rc = h->Rh.alloc(Rrows.size())) || (rc = h->Rl.alloc(Rrows.size())))
      return rc;
    if ((rc = smx_split_tf32(Rd.p, std::max(h->K, 1), h->ldo, h->ldo, h->Rh.p, h->Rl.p, h->ldo, stream))) return rc;
    if (use_tc) {
      if ((rc = Bd.upload(B, st)) || (rc = h->Bh.alloc(B.size())) || (rc = h->Bl.alloc(B.size())) ||
          (rc = smx_split_tf32(Bd.p, dout, h->ldk, h->ldk, h->Bh.p, h->Bl.p, h->ldk, stream)))
        return rc;
    }
    // segment bounds of the panel for every wanted count (spectral.py segment_bounds):
    // near-equal splits of the tape, every bound but the last at a depth-1 entry
    std::vector<int32_t> segs;
    h->seg_off.assign(33, 0);
    h->seg_n.assign(33, 1);
    for (int want = 2; want <= 32; ++want) {
      std::vector<int32_t> b{0};
      if (!h->lvl1.empty()) {
        for (int i = 1; i < want; ++i) {
          const int64_t target = int64_t(i) * h->K / want;
          size_t q = size_t(std::lower_bound(h->lvl1.begin(), h->lvl1.end(), int32_t(target)) - h->lvl1.begin());
          q = std::min(q, h->lvl1.size() - 1);
          b.push_back(h->lvl1[q]);
        }
      }
      b.push_back(h->K);
      std::sort(b.begin(), b.end());
      b.erase(std::unique(b.begin(), b.end()), b.end());
      h->seg_off[want] = int(segs.size());
      h->seg_n[want] = int(b.size()) - 1;
      segs.insert(segs.end(), b.begin(), b.end());
    }
    if ((rc = h->segs.upload(segs, st))) return rc;
    // gradient walk: one segment per 4096 tape entries, at most 32 and the
    // depth-1 entries (spectral.py vjp_segment_count)
    h->vjp_want = int(std::max<int64_t>(1, std::min<int64_t>({32, int64_t(h->K) / 4096, int64_t(h->lvl1.size())})));
    if (cudaStreamSynchronize(st) != cudaSuccess)  // the staging buffers go out of scope
      return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: sync failed");
  }
  // FP64 tables: the FP64 evaluator of the orthogonal form
  {
    smx::layout::Tables p64;
    const int64_t do_pass = dout == 1 ? 1 : 4;
    if (smx::layout::build_perpoint64(tr, C64_h.data(), dout, maxdeg.data(), d, fam_v.data(), fa_v.data(),
                                      fb_v.data(), p64) &&
        (int64_t(p64.scalar["row"]) + 4 * do_pass) * 64 * 8 <= 227 * 1024 && p64.scalar["max_depth"] <= 8) {
      Pack<int32_t> pi;
      Pack<double> pf;
      const char* names_i[] = {"hot_dim", "hot_deg", "hot_soff", "node", "cold", "run"};
      const char* names_f[] = {"node_c", "cold_ab", "terms", "coef"};
      for (const char* nm : names_i) pi.add(nm, p64.i32[nm]);
      for (const char* nm : names_f) pf.add(nm, p64.f64[nm]);
      if ((rc = h->ti64.upload(pi.v, st)) || (rc = h->tf64.upload(pf.v, st)) || (rc = h->fa64.upload(fa_v, st)) ||
          (rc = h->fb64.upload(fb_v, st)))
        return rc;
      smx_spectral64& s = h->spectral64;
      s.d_in = d;
      s.d_out = dout;
      s.dstride = int(p64.scalar["dstride"]);
      s.row = int(p64.scalar["row"]);
      s.n_hb = int(p64.scalar["n_hb"]);
      s.n_vp = int(p64.scalar["n_vp"]);
      s.n_hot_dims = int(p64.scalar["n_hot_dims"]);
      s.n_nodes = int(p64.scalar["n_nodes"]);
      s.n_cold_groups = int(p64.scalar["n_cold_groups"]);
      s.max_depth = int(p64.scalar["max_depth"]);
      s.n_terms = int(p64.scalar["n_terms"]);
      for (int i = 0; i < 5; ++i) {
        s.node_seg[i] = p64.i32["node_seg"][i];
        s.cold_seg[i] = p64.i32["cold_seg"][i];
      }
      auto ia = [&](const char* nm) { return pi.at(h->ti64.p, nm, p64.i32[nm]); };
      auto fa = [&](const char* nm) { return pf.at(h->tf64.p, nm, p64.f64[nm]); };
      s.hot_dim = ia("hot_dim");
      s.hot_deg = ia("hot_deg");
      s.hot_soff = ia("hot_soff");
      s.node = ia("node");
      s.cold = ia("cold");
      s.run = ia("run");
      s.node_c = fa("node_c");
      s.cold_ab = fa("cold_ab");
      s.terms = fa("terms");
      s.coef = fa("coef");
      s.fam_a = h->fa64.p;
      s.fam_b = h->fb64.p;
      s.fam = h->fam.p;
      s.c0 = h->C64.p;  // row 0: the root's coefficients
      h->have64 = true;
      if (cudaStreamSynchronize(st) != cudaSuccess)  // the host blobs go out of scope
        return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: sync failed");
    }
  }

  if (use_tc) {
    h->evaluator = SMX_FP32_TENSOR;
  } else {
    smx::layout::Tables& t = use_blocked ? bl : pp;
    Blobs b;
    const char* names_bl[] = {"hot_dim", "hot_deg", "hot_soff", "node", "vc", "hot_ent", "grp", "grp_ab", "W",
                              "warp_off", "items"};
    const char* names_pp[] = {"hot_dim", "hot_deg", "hot_soff", "node", "node_c", "cold", "cold_ab", "run", "coef",
                              "blk_dims", "blk_run", "blk_ab"};
    if (use_blocked)
      for (const char* nm : names_bl) b.add(t, nm);
    else
      for (const char* nm : names_pp) b.add(t, nm);
    b.fo.push_back({"c0", b.f.size()});
    for (int o = 0; o < dout; ++o) b.f.push_back(C32[o]);
    if ((rc = h->ti.upload(b.i, st)) || (rc = h->tf.upload(b.f, st))) return rc;
    if (use_blocked) {
      h->evaluator = SMX_FP32_BLOCKED;
      smx_blocked& s = h->blocked;
      s.d_in = d;
      s.n_hs = int(t.scalar["n_hs"]);
      s.k_c = int(t.scalar["k_c"]);
      s.n_hot_dims = int(t.scalar["n_hot_dims"]);
      s.n_nodes = int(t.scalar["n_nodes"]);
      s.n_groups = int(t.scalar["n_groups"]);
      s.n_items = int(t.scalar["n_items"]);
      s.c0 = float(t.scalar["c0"]);
      s.hot_dim = b.ip(h.get(), "hot_dim");
      s.hot_deg = b.ip(h.get(), "hot_deg");
      s.hot_soff = b.ip(h.get(), "hot_soff");
      s.node = b.ip(h.get(), "node");
      s.vc = s.k_c ? b.ip(h.get(), "vc") : nullptr;
      s.hot_ent = b.ip(h.get(), "hot_ent");
      s.grp = b.ip(h.get(), "grp");
      s.grp_ab = b.fp(h.get(), "grp_ab");
      s.W = b.fp(h.get(), "W");
      s.warp_off = b.ip(h.get(), "warp_off");
      s.items = b.ip(h.get(), "items");
      s.fa = h->fam_a.p;
      s.fb = h->fam_b.p;
      s.fam = h->fam.p;
      s.n_ent = int(size_of(t, "hot_ent"));
      s.n_w = int(size_of(t, "W") / 4);
    } else {
      h->evaluator = SMX_FP32_PERPOINT;
      smx_spectral& s = h->spectral;
      s.d_in = d;
      s.d_out = dout;
      s.dstride = int(t.scalar["dstride"]);
      s.row = int(t.scalar["row"]);
      s.n_hb = int(t.scalar["n_hb"]);
      s.n_vp = int(t.scalar["n_vp"]);
      s.n_hot_dims = int(t.scalar["n_hot_dims"]);
      s.n_nodes = int(t.scalar["n_nodes"]);
      s.n_cold_groups = int(t.scalar["n_cold_groups"]);
      s.max_depth = int(t.scalar["max_depth"]);
      s.n_cold_blocks = int(t.scalar["n_cold_blocks"]);
      for (int i = 0; i < 5; ++i) {
        s.node_seg[i] = t.i32["node_seg"][i];
        s.cold_seg[i] = t.i32["cold_seg"][i];
        s.block_seg[i] = t.i32["block_seg"][i];
      }
      auto ipn = [&](const char* nm) { return size_of(t, nm) ? b.ip(h.get(), nm) : nullptr; };
      auto fpn = [&](const char* nm) { return size_of(t, nm) ? b.fp(h.get(), nm) : nullptr; };
      s.hot_dim = ipn("hot_dim");
      s.hot_deg = ipn("hot_deg");
      s.hot_soff = ipn("hot_soff");
      s.node = ipn("node");
      s.node_c = fpn("node_c");
      s.cold = ipn("cold");
      s.cold_ab = fpn("cold_ab");
      s.blk_dims = ipn("blk_dims");
      s.blk_run = ipn("blk_run");
      s.blk_ab = fpn("blk_ab");
      s.run = ipn("run");
      s.coef = fpn("coef");
      s.fam_a = h->fam_a.p;
      s.fam_b = h->fam_b.p;
      s.fam = h->fam.p;
      s.c0 = b.fp(h.get(), "c0");
    }
    if (cudaStreamSynchronize(st) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_create: sync failed");
  }
  *out = h.release();
  return SMX_OK;
}

extern "C" void smx_fp32_plan_destroy(smx_fp32_plan* h) { delete h; }

extern "C" int smx_fp32_plan_info(const smx_fp32_plan* h, int* evaluator, int64_t* n_lambda, const double** coef) {
  SMX_REQUIRE(h, "smx_fp32_plan_info: null plan");
  if (evaluator) *evaluator = h->evaluator;
  if (n_lambda) *n_lambda = h->n_lambda;
  if (coef) *coef = h->C64.p;
  return SMX_OK;
}

extern "C" int smx_fp32_plan_has_fp64(const smx_fp32_plan* h) { return h && h->have64 ? 1 : 0; }

extern "C" int smx_fp32_eval64(const smx_fp32_plan* h, const double* x, int64_t P, int64_t ldx, double* y,
                               void* stream) {
  SMX_REQUIRE(h, "smx_fp32_eval64: null plan");
  if (!h->have64)
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_fp32_eval64: the plan has no FP64 tables (one output, per-point "
                                               "row within shared memory)");
  return smx_spectral_eval64(&h->spectral64, x, P, ldx, y, stream);
}

extern "C" size_t smx_fp32_workspace(const smx_fp32_plan* h, int64_t P) {
  if (!h || P < 0) return 0;
  if (h->evaluator == SMX_FP32_BLOCKED) return smx_blocked_eval_workspace(&h->blocked, P);
  if (h->evaluator != SMX_FP32_TENSOR) return 0;
  const int64_t step = tc_step(h, std::max<int64_t>(P, 1));
  const size_t lda = size_t(round32(std::max(h->K, 1)));
  return 2 * up(size_t(step) * lda * sizeof(float)) + up(smx_spectral_panel_workspace(h->n_slots, step)) +
         (tc_splits(h) > 1 ? up(smx_gemm_tf32x3_splitk_workspace(int(step), h->d_out, h->K, tc_splits(h))) : 0);
}

extern "C" int smx_fp32_eval(const smx_fp32_plan* h, const double* x, int64_t P, int64_t ldx, float* y, void* ws,
                             size_t ws_bytes, void* stream) {
  SMX_REQUIRE(h && P >= 0 && ldx >= h->d_in, "smx_fp32_eval: bad arguments");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y, "smx_fp32_eval: null pointer");
  const size_t need = smx_fp32_workspace(h, P);
  SMX_REQUIRE(ws_bytes >= need && (ws || need == 0), "smx_fp32_eval: workspace too small");
  if (h->evaluator == SMX_FP32_BLOCKED) return smx_blocked_eval(&h->blocked, x, P, ldx, y, ws, ws_bytes, stream);
  if (h->evaluator == SMX_FP32_PERPOINT) return smx_spectral_eval(&h->spectral, x, P, ldx, y, stream);
  // tensor core: per chunk of points a basis-product panel (TF32 hi/lo) and the contraction
  const int64_t step = tc_step(h, P);
  const int64_t lda = round32(std::max(h->K, 1));
  uint8_t* w = static_cast<uint8_t*>(ws);
  const size_t panel_bytes = up(size_t(step) * lda * sizeof(float));
  float* Ah = reinterpret_cast<float*>(w);
  float* Al = reinterpret_cast<float*>(w + panel_bytes);
  const int splits = tc_splits(h);
  const size_t sk_bytes = splits > 1 ? up(smx_gemm_tf32x3_splitk_workspace(int(step), h->d_out, h->K, splits)) : 0;
  void* skws = w + 2 * panel_bytes;
  void* pws = w + 2 * panel_bytes + sk_bytes;
  const size_t pws_bytes = ws_bytes - 2 * panel_bytes - sk_bytes;
  int rc;
  for (int64_t p0 = 0; p0 < P; p0 += step) {
    const int64_t m = std::min(step, P - p0);
    const int want = seg_want(h, m);
    const int n_seg = want <= 1 ? 1 : h->seg_n[want];
    const int32_t* seg = want <= 1 ? nullptr : h->segs.p + h->seg_off[want];
    if ((rc = smx_spectral_panel_tf32(h->n_dims, h->dims.p, h->dmax.p, h->dsoff.p, h->n_slots, h->tape.p, h->K, seg,
                                      n_seg, h->fam_a.p, h->fam_b.p, h->fam.p, x + p0 * ldx, m, ldx, Ah, Al, lda, pws,
                                      pws_bytes, stream)) ||
        (rc = smx_gemm_tf32x3_splitk(Ah, Al, lda, h->Bh.p, h->Bl.p, h->ldk, int(m), h->d_out, h->K,
                                     y + p0 * h->d_out, h->d_out, h->bias.p, 0, splits, skws, sk_bytes, h->err.p,
                                     stream)))
      return rc;
  }
  return SMX_OK;
}

extern "C" int smx_fp32_plan_check(const smx_fp32_plan* h, void* stream) {
  SMX_REQUIRE(h, "smx_fp32_plan_check: null plan");
  int32_t e = 0;
  cudaStream_t st = smx::as_stream(stream);
  if (cudaMemcpyAsync(&e, h->err.p, sizeof(e), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "smx_fp32_plan_check: read failed");
  if (e == 0) return SMX_OK;
  cudaMemsetAsync(h->err.p, 0, sizeof(int32_t), st);
  return smx::set_error(SMX_ERR_CUDA, "tensor-core contraction: a pipeline wait timed out (code " + std::to_string(e) +
                                          "); its results are invalid");
}

namespace {
// Scratch of one VJP call (byte offsets into the caller's workspace).
struct VjpLayout {
  int64_t step, ldp, ldg;
  size_t g32, gh, gl, G, xws, ATh, ATl, gT, gTh, gTl, dCrev, skws, ptws, dC, total;
  size_t n_xws, n_skws, n_ptws;
  int splits;
};

VjpLayout vjp_layout(const smx_fp32_plan* h, int64_t P) {
  VjpLayout L{};
  L.step = std::max<int64_t>(128, int64_t(h->memory_limit * 1073741824.0 / double(8 * int64_t(h->ldk))) / 128 * 128);
  const int64_t m = std::max<int64_t>(1, std::min(L.step, P));
  L.ldp = round32(m);
  L.ldg = round32(std::max(h->K, 1));
  // the [K x d_out] product has few tiles and a long contraction over the points: split it over the SMs
  const int64_t tiles = ((h->K + 127) / 128) * ((h->d_out + 127) / 128);
  L.splits = int(std::max<int64_t>(1, std::min<int64_t>(64, (2 * int64_t(h->sms)) / std::max<int64_t>(tiles, 1))));
  L.n_xws = smx_spectral_vjp_x_workspace(h->n_slots, h->vjp_want <= 1 ? 1 : h->seg_n[h->vjp_want], m);
  L.n_skws = smx_gemm_tf32x3_splitk_workspace(std::max(h->K, 1), h->d_out, int(m), L.splits);
  L.n_ptws = smx_spectral_panel_t_workspace(h->n_slots, m);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += up(std::max<size_t>(bytes, 1));
    return at;
  };
  L.g32 = take(size_t(P) * h->ldo * 4);
  L.gh = take(size_t(P) * h->ldo * 4);
  L.gl = take(size_t(P) * h->ldo * 4);
  L.G = take(size_t(m) * L.ldg * 4);
  L.xws = take(L.n_xws);
  L.ATh = take(size_t(std::max(h->K, 1)) * L.ldp * 4);
  L.ATl = take(size_t(std::max(h->K, 1)) * L.ldp * 4);
  L.gT = take(size_t(h->ldo) * L.ldp * 4);
  L.gTh = take(size_t(h->ldo) * L.ldp * 4);
  L.gTl = take(size_t(h->ldo) * L.ldp * 4);
  L.dCrev = take(size_t(std::max(h->K, 1)) * h->d_out * 4);
  L.skws = take(L.n_skws);
  L.ptws = take(L.n_ptws);
  L.dC = take(size_t(h->n_lambda) * h->d_out * 8);
  L.total = o;
  return L;
}
}  // namespace

extern "C" size_t smx_vjp_workspace(const smx_fp32_plan* h, int64_t P) {
  if (!h || P < 0 || !h->have_tape) return 0;
  return vjp_layout(h, std::max<int64_t>(P, 1)).total;
}

extern "C" int smx_vjp(const smx_fp32_plan* h, const double* x, int64_t P, int64_t ldx, const float* g, int64_t ldg,
                       double* dx, int64_t lddx, double* dF, void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(h && P >= 0 && ldx >= h->d_in && ldg >= h->d_out && (!dx || lddx >= h->d_in), "smx_vjp: bad arguments");
  SMX_REQUIRE(h->have_tape, "smx_vjp: the backward needs index-set depth <= 8");
  cudaStream_t st = smx::as_stream(stream);
  if (P == 0) {  // no points: dL/dF = 0
    if (dF && cudaMemsetAsync(dF, 0, size_t(h->plan->n_entries) * h->d_out * 8, st) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_vjp: memset failed");
    return SMX_OK;
  }
  SMX_REQUIRE(x && g && (dx || dF), "smx_vjp: null pointer");
  const VjpLayout L = vjp_layout(h, P);
  SMX_REQUIRE(ws && ws_bytes >= L.total, "smx_vjp: workspace too small");
  uint8_t* w = static_cast<uint8_t*>(ws);
  auto F = [&](size_t off) { return reinterpret_cast<float*>(w + off); };
  int rc;
  // cotangent padded to ldo columns, split into TF32 hi/lo
  pad_rows_kernel<<<smx::grid_for(P * h->ldo, 256), 256, 0, st>>>(g, ldg, P, h->d_out, h->ldo, F(L.g32));
  SMX_LAUNCH_CHECK("smx_vjp");
  if ((rc = smx_split_tf32(F(L.g32), P, h->ldo, h->ldo, F(L.gh), F(L.gl), h->ldo, stream))) return rc;
  if (dx) {
    // dL/dx: G = g R^T (the adjoints of the entries' basis products), then the chain rule per dimension
    if (cudaMemset2DAsync(dx, size_t(lddx) * 8, 0, size_t(h->d_in) * 8, size_t(P), st) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_vjp: memset failed");
    for (int64_t p0 = 0; p0 < P; p0 += L.step) {
      const int64_t m = std::min(L.step, P - p0);
      if ((rc = smx_gemm_tf32x3(F(L.gh) + p0 * h->ldo, F(L.gl) + p0 * h->ldo, h->ldo, h->Rh.p, h->Rl.p, h->ldo,
                                int(m), h->K, h->ldo, F(L.G), L.ldg, nullptr, 0, h->err.p, stream)) ||
          (rc = smx_spectral_vjp_x(h->n_dims, h->dims.p, h->dmax.p, h->dsoff.p, h->n_slots, h->tape.p, h->K,
                                   h->vjp_want <= 1 ? nullptr : h->segs.p + h->seg_off[h->vjp_want],
                                   h->vjp_want <= 1 ? 1 : h->seg_n[h->vjp_want], h->fam_a.p, h->fam_b.p, h->fam.p,
                                   x + p0 * ldx, m, ldx, F(L.G), L.ldg, dx + p0 * lddx, lddx, w + L.xws, L.n_xws,
                                   stream)))
        return rc;
    }
  }
  if (dF) {
    // dL/dC = A(x)^T g over the points (split-K), then the adjoint of the coefficient transform
    float* dCrev = F(L.dCrev);
    for (int64_t i = 0, p0 = 0; p0 < P; p0 += L.step, ++i) {
      const int64_t m = std::min(L.step, P - p0);
      if ((rc = smx_spectral_panel_t_tf32(h->n_dims, h->dims.p, h->dmax.p, h->dsoff.p, h->n_slots, h->tape.p, h->K,
                                          h->fam_a.p, h->fam_b.p, h->fam.p, x + p0 * ldx, m, ldx, F(L.ATh), F(L.ATl),
                                          L.ldp, w + L.ptws, L.n_ptws, stream)))
        return rc;
      transpose_pad_kernel<<<smx::grid_for(m * h->ldo, 256), 256, 0, st>>>(F(L.g32) + p0 * h->ldo, h->ldo, int(m),
                                                                          h->d_out, h->ldo, F(L.gT), L.ldp);
      SMX_LAUNCH_CHECK("smx_vjp");
      if ((rc = smx_split_tf32(F(L.gT), h->ldo, m, L.ldp, F(L.gTh), F(L.gTl), L.ldp, stream)) ||
          (rc = smx_gemm_tf32x3_splitk(F(L.ATh), F(L.ATl), L.ldp, F(L.gTh), F(L.gTl), L.ldp, h->K, h->d_out, int(m),
                                       dCrev, h->d_out, nullptr, i ? 1 : 0, L.splits, w + L.skws, L.n_skws, h->err.p,
                                       stream)))
        return rc;
    }
    double* dC = reinterpret_cast<double*>(w + L.dC);
    if (cudaMemsetAsync(dC, 0, size_t(h->n_lambda) * h->d_out * 8, st) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_vjp: memset failed");
    scatter_dc_kernel<<<smx::grid_for(int64_t(h->K) * h->d_out + h->d_out, 256), 256, 0, st>>>(
        dCrev, h->ent.p, h->K, h->d_out, F(L.g32), h->ldo, P, dC);
    SMX_LAUNCH_CHECK("smx_vjp");
    if ((rc = smx_spectral_coefficients_adjoint(h->plan, h->aoff.p, h->A.p, h->ids.p, dC, dF, stream))) return rc;
  }
  return SMX_OK;
}
