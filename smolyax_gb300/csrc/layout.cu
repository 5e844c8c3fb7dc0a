// Host-side builders of the FP32 evaluators' tables (no device work).
//
// The same tables as the package's Python builders (``blocked.py``
// build_blocked, ``spectral.py`` build_layout and build_tape), so that a C
// host can build the FP32 form of a plan without Python; CPU tests check that
// both produce identical tables.  Inputs are host arrays of the index-set
// tree (entry 0 = root): parent, dim, deg, level, pre-order rank, remaining
// budget, and the FP32 coefficients of every entry.
#include <math.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "blocked_tc.h"
#include "layout.h"

namespace smx {
namespace layout {

namespace {

constexpr int kWarps = 16;
constexpr int kTile = 128;
constexpr int kMaxPath = 8;
constexpr int64_t kSmemLimit = 220 * 1024;

int32_t f2bits(float v) {
  int32_t b;
  std::memcpy(&b, &v, 4);
  return b;
}

int64_t round4(int64_t v) { return (v + 3) / 4 * 4; }
int64_t round32(int64_t v) { return (v + 31) / 32 * 32; }

// indices 0..n-1 sorted by key (stable)
template <typename Key>
std::vector<int64_t> stable_order(int64_t n, Key key) {
  std::vector<int64_t> o(n);
  std::iota(o.begin(), o.end(), 0);
  std::stable_sort(o.begin(), o.end(), [&](int64_t a, int64_t b) { return key(a) < key(b); });
  return o;
}

int argmin(const double* v, int n) {
  int w = 0;
  for (int i = 1; i < n; ++i)
    if (v[i] < v[w]) w = i;
  return w;
}

// Runs of the per-point evaluator (spectral.py _Runs): 4-aligned slot ranges
// of at most 32 slots, gaps of at most 4, coefficients [length][dstride].
struct Runs {
  int64_t dstride;
  std::vector<int32_t> tab;  // [n][4] start, length, coefficient offset, degree
  std::vector<float> coef;
  struct Range {
    int64_t first, second;
  };
  int64_t n() const { return int64_t(tab.size() / 4); }
  // slots increasing; coefs(i, o) = coefficient o of slot i
  Range add(const std::vector<int64_t>& slots, const std::function<float(size_t, int)>& coefs, int d_out, int degree) {
    const int64_t r0 = n();
    const size_t N = slots.size();
    for (size_t i = 0; i < N;) {
      size_t j = i + 1;
      const int64_t a0 = slots[i] & ~int64_t(3);
      while (j < N && slots[j] - slots[j - 1] <= 4 && slots[j] - a0 < 32) ++j;
      const int64_t length = round4(slots[j - 1] + 1 - a0);
      const size_t base = coef.size();
      coef.resize(base + size_t(length * dstride), 0.f);
      for (size_t q = i; q < j; ++q)
        for (int o = 0; o < d_out; ++o) coef[base + size_t((slots[q] - a0) * dstride + o)] = coefs(q, o);
      tab.insert(tab.end(), {int32_t(a0), int32_t(length), int32_t(base), int32_t(degree)});
      i = j;
    }
    return {r0, n()};
  }
};

// Segment cuts of the per-point evaluator (spectral.py build_layout.cuts):
// boundary k is the allowed index whose cumulative cost is nearest k/nseg of
// the total (the first such, not before the previous boundary).
std::vector<int32_t> cuts(const std::vector<double>& cost, const std::vector<int64_t>& allowed, int nseg) {
  std::vector<double> cum{0.0};
  for (double c : cost) cum.push_back(cum.back() + c);
  const double tot = cum.back();
  std::vector<int32_t> out{0};
  for (int k = 1; k < nseg; ++k) {
    const double want = tot * k / nseg;
    int64_t best = -1;
    double bd = 0;
    for (int64_t a : allowed)
      if (a >= out.back()) {
        const double dd = fabs(cum[a] - want);
        if (best < 0 || dd < bd) best = a, bd = dd;
      }
    out.push_back(best < 0 ? out.back() : int32_t(best));
  }
  out.push_back(int32_t(cost.size()));
  return out;
}

}  // namespace

int64_t blocked_smem_bytes(int64_t n_hs, int64_t k_c) { return (n_hs + k_c) * kTile * 4 + 2 * kWarps * kTile * 4; }

// Port of blocked.py build_blocked.
bool build_blocked(const Tree& tr, const float* C, const int64_t* maxdeg, int d, const int32_t* fam, const double* fa,
                   const double* fb, Tables& out) {
  const int64_t n = tr.n;
  std::vector<char> hot(d, 0);
  for (int64_t e = 1; e < n; ++e)
    if (tr.parent[e] > 0) hot[tr.dim[tr.parent[e]]] = 1;
  std::vector<int32_t> hot_dims, hot_deg, hot_soff;
  std::vector<int64_t> hidx(d, -1);
  int64_t n_hs = 0;
  for (int j = 0; j < d; ++j)
    if (hot[j]) {
      hidx[j] = int64_t(hot_dims.size());
      hot_dims.push_back(j);
      hot_deg.push_back(int32_t(maxdeg[j]));
      hot_soff.push_back(int32_t(n_hs));
      n_hs += maxdeg[j];
    }
  std::vector<int64_t> hot_e, cold_e;
  for (int64_t e = 1; e < n; ++e) (hot[tr.dim[e]] ? hot_e : cold_e).push_back(e);
  std::vector<int64_t> hslot(n, -1);
  for (int64_t e : hot_e) hslot[e] = hot_soff[hidx[tr.dim[e]]] + tr.deg[e] - 1;
  std::vector<char> has_kid(n, 0);
  for (int64_t e = 1; e < n; ++e) has_kid[tr.parent[e]] = 1;
  std::vector<int64_t> nodes{0};
  for (int64_t e = 1; e < n; ++e)
    if (has_kid[e]) nodes.push_back(e);
  const int64_t NN = int64_t(nodes.size());
  std::vector<int64_t> depth(n, 0), nidx(n, -1);
  std::vector<std::vector<int64_t>> paths(NN);
  for (int64_t i = 1; i < NN; ++i) {
    const int64_t a = nodes[i];
    std::vector<int64_t> p;
    for (int64_t v = a; v != 0; v = tr.parent[v]) p.push_back(hslot[v]);
    if (int(p.size()) > kMaxPath || *std::min_element(p.begin(), p.end()) < 0) return false;
    std::reverse(p.begin(), p.end());
    paths[i] = p;
    depth[a] = int64_t(p.size());
  }
  for (int64_t i = 0; i < NN; ++i) nidx[nodes[i]] = i;

  // hot entries grouped by parent node (then slot), two per 16 bytes
  std::vector<int64_t> ord = stable_order(int64_t(hot_e.size()), [&](int64_t i) {
    return std::make_pair(nidx[tr.parent[hot_e[i]]], hslot[hot_e[i]]);
  });
  std::vector<int64_t> cnt(NN, 0);
  for (int64_t e : hot_e) cnt[nidx[tr.parent[e]]] += 1;
  std::vector<int32_t> node_tab(NN * 12, 0);
  std::vector<std::pair<int32_t, float>> ent;
  int64_t pos = 0;
  for (int64_t i = 0; i < NN; ++i) {
    node_tab[i * 12 + 0] = int32_t(ent.size());
    for (int64_t q = 0; q < cnt[i]; ++q) {
      const int64_t v = hot_e[ord[pos + q]];
      ent.push_back({int32_t(hslot[v] * kTile), C[v]});
    }
    if (cnt[i] % 2) ent.push_back({0, 0.f});
    pos += cnt[i];
    node_tab[i * 12 + 1] = int32_t(ent.size()) - node_tab[i * 12 + 0];
    node_tab[i * 12 + 2] = int32_t(depth[nodes[i]]);
    for (size_t q = 0; q < paths[i].size(); ++q) node_tab[i * 12 + 4 + q] = int32_t(paths[i][q] * kTile);
  }
  std::vector<int32_t> hot_ent(2 * ent.size());
  for (size_t i = 0; i < ent.size(); ++i) {
    hot_ent[2 * i] = ent[i].first;
    hot_ent[2 * i + 1] = f2bits(ent[i].second);
  }

  // prefix rows of the cold entries, by remaining budget (descending)
  std::vector<int64_t> pref;
  {
    std::vector<char> isp(n, 0);
    for (int64_t e : cold_e) isp[tr.parent[e]] = 1;
    for (int64_t e = 0; e < n; ++e)
      if (isp[e]) pref.push_back(e);
    std::vector<int64_t> o = stable_order(int64_t(pref.size()), [&](int64_t i) {
      return std::make_pair(-tr.rem[pref[i]], pref[i]);
    });
    std::vector<int64_t> p2;
    for (int64_t i : o) p2.push_back(pref[i]);
    pref.swap(p2);
  }
  const int64_t k_c = int64_t(pref.size());
  std::vector<int64_t> kc(n, -1);
  for (int64_t i = 0; i < k_c; ++i) kc[pref[i]] = i;
  std::vector<int32_t> vc_tab(k_c * 12);
  for (int64_t i = 0; i < k_c; ++i)
    std::copy(node_tab.begin() + nidx[pref[i]] * 12, node_tab.begin() + nidx[pref[i]] * 12 + 12,
              vc_tab.begin() + i * 12);
  if (blocked_smem_bytes(n_hs, k_c) > kSmemLimit) return false;

  // cold slots (dim, deg): staircase check, then groups over windows of 4 dimensions
  std::map<std::pair<int64_t, std::pair<int, int>>, float> coef_of;
  std::map<std::pair<int, int>, int64_t> L;
  for (int64_t v : cold_e) {
    const std::pair<int, int> s{tr.dim[v], tr.deg[v]};
    coef_of[{kc[tr.parent[v]], s}] = C[v];
    L[s] += 1;
  }
  for (const auto& kv : coef_of)
    if (kv.first.first >= L[kv.first.second]) return false;
  std::vector<std::pair<int, int>> slots;
  for (const auto& kv : L) slots.push_back(kv.first);
  struct Group {
    std::vector<std::pair<int, int>> sl;
    bool fast;
  };
  std::vector<Group> groups;
  for (size_t i = 0; i < slots.size();) {
    const int w = slots[i].first / 4;
    size_t j = i;
    while (j < slots.size() && slots[j].first / 4 == w) ++j;
    bool fast = j - i == 4;
    for (size_t q = i; q < j && fast; ++q) fast = slots[q].second == 1 && slots[q].first == 4 * w + int(q - i);
    for (size_t q = i; q < j; q += 4)
      groups.push_back({std::vector<std::pair<int, int>>(slots.begin() + q, slots.begin() + std::min(j, q + 4)), fast});
    i = j;
  }
  const int64_t G = int64_t(groups.size());
  std::vector<int32_t> grp(G * 12, 0);
  std::vector<float> grp_ab(G * 8, 0.f), W;
  for (int64_t g = 0; g < G; ++g) {
    const auto& sl = groups[g].sl;
    int64_t K = 0;
    for (const auto& s : sl) K = std::max(K, L[s]);
    int32_t* gr = &grp[g * 12];
    gr[0] = int32_t(K);
    gr[1] = int32_t(W.size());
    gr[2] = groups[g].fast ? 1 : 0;
    gr[3] = int32_t(sl.size());
    for (int q = 0; q < 4; ++q) {
      if (q < int(sl.size())) {
        const int j_ = sl[q].first;
        gr[4 + q] = j_;
        gr[8 + q] = sl[q].second;
        if (groups[g].fast) {
          const double a0 = fam[j_] == 0 ? 1.0 : sqrt(2.0);
          grp_ab[g * 8 + q] = float(a0 * fa[j_]);
          grp_ab[g * 8 + 4 + q] = float(a0 * fb[j_]);
        } else {
          grp_ab[g * 8 + q] = float(fa[j_]);
          grp_ab[g * 8 + 4 + q] = float(fb[j_]);
        }
      } else {
        gr[4 + q] = sl[0].first;
        gr[8 + q] = 0;
      }
    }
    if (groups[g].fast) {
      bool unit = true;
      for (int q = 0; q < 4; ++q) unit = unit && grp_ab[g * 8 + q] == 1.0f && grp_ab[g * 8 + 4 + q] == 0.0f;
      if (unit) gr[2] = 2;  // unit maps: phi_1 = x
    }
    for (int64_t k = 0; k < K; ++k)
      for (int q = 0; q < 4; ++q) {
        float c = 0.f;
        if (q < int(sl.size())) {
          auto it = coef_of.find({k, sl[q]});
          if (it != coef_of.end()) c = it->second;
        }
        W.push_back(c);
      }
  }

  // items and their balance over the warps
  std::vector<int64_t> hot_items;
  std::vector<double> cost_hot(NN, 0.0);
  for (int64_t i = 0; i < NN; ++i)
    if (node_tab[i * 12 + 1] > 0) {
      hot_items.push_back(i);
      cost_hot[i] = 12 + 6.5 * node_tab[i * 12 + 1] + 3 * node_tab[i * 12 + 2];
    }
  std::stable_sort(hot_items.begin(), hot_items.end(),
                   [&](int64_t a, int64_t b) { return -cost_hot[a] < -cost_hot[b]; });
  double load[kWarps] = {0};
  std::vector<std::vector<int32_t>> lists(kWarps);
  for (int64_t i : hot_items) {
    const int w = argmin(load, kWarps);
    lists[w].push_back(int32_t(i));
    load[w] += cost_hot[i];
  }
  for (int64_t g = 0; g < G; ++g) {
    const int64_t K = grp[g * 12];
    const double c = 24 + 18 * double(K) +
                     (grp[g * 12 + 2] ? 40.0
                                      : 100.0 + 20.0 * (grp[g * 12 + 8] + grp[g * 12 + 9] + grp[g * 12 + 10] +
                                                        grp[g * 12 + 11]));
    const int w = argmin(load, kWarps);
    lists[w].push_back(int32_t((1 << 30) | g));
    load[w] += c;
  }
  std::vector<int32_t> warp_off(kWarps + 1, 0), items;
  for (int w = 0; w < kWarps; ++w) {
    warp_off[w + 1] = warp_off[w] + int32_t(lists[w].size());
    items.insert(items.end(), lists[w].begin(), lists[w].end());
  }
  out.i32["hot_dim"] = hot_dims;
  out.i32["hot_deg"] = hot_deg;
  out.i32["hot_soff"] = hot_soff;
  out.i32["node"] = node_tab;
  out.i32["vc"] = vc_tab;
  out.i32["hot_ent"] = hot_ent;
  out.i32["grp"] = grp;
  out.f32["grp_ab"] = grp_ab;
  out.f32["W"] = W;
  out.i32["warp_off"] = warp_off;
  out.i32["items"] = items;
  out.scalar["n_hs"] = double(n_hs);
  out.scalar["k_c"] = double(k_c);
  out.scalar["n_hot_dims"] = double(hot_dims.size());
  out.scalar["n_nodes"] = double(NN);
  out.scalar["n_groups"] = double(G);
  out.scalar["n_items"] = double(items.size());
  out.scalar["c0"] = double(C[0]);
  return true;
}

namespace {

// bf16 of an FP32 value, rounded to nearest even (NaN stays NaN).
uint16_t bf16_rn(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}

float bf16_value(uint16_t h) {
  const uint32_t u = uint32_t(h) << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

}  // namespace

// Tables of the tensor-core blocked evaluator (blocked_tc.cu), one output.
//
// Every entry e != root extends a node a (an entry with children) by one
// factor: I(x) = c_0 + sum_a V_a(x) [ sum_{table slots s} B_t[a][s] Phi_s(x)
//                                    + sum_{linear dims j} B_l[a][j] x_j ].
// Table dimensions are the hot ones (those with children) and the cold ones
// of degree >= 2; their basis values Phi_s (slot 0 = the constant 1) are
// computed per point.  Linear dimensions (cold, degree 1) enter through
// phi_1(z_j) = alpha0 (fa_j x_j + fb_j): B_l = C alpha0 fa_j, and the constant
// part C alpha0 fb_j is summed into B_t[a][0].  The nodes, sorted by remaining
// budget (descending), are the rows of A = V (per point, computed on chip) and
// of the coefficient matrices, so that a dimension j of weight k_j only uses
// the first rows (a node admits j iff its remaining budget exceeds k_j): the
// table and linear columns are cut into chunks of 64, each with its own
// number of 16-row K steps (at most 16: A lives in tensor memory).
// Coefficients are stored as three bf16 parts (hi + mid + lo = the FP32
// value) in the shared-memory image of the MMA's B operand (K-major, 32-byte
// swizzle: 16-byte half h of row n at (h ^ (n >> 2 & 1))), chunk by chunk,
// each chunk's K steps from the last to the first.
bool build_blocked_tc(const Tree& tr, const float* C, const int64_t* maxdeg, int d, const int32_t* fam,
                      const double* fa, const double* fb, Tables& out) {
  using namespace smx::btc;
  const int64_t n = tr.n;
  if (n < 2) return false;
  std::vector<char> hot(d, 0);
  for (int64_t e = 1; e < n; ++e)
    if (tr.parent[e] > 0) hot[tr.dim[tr.parent[e]]] = 1;
  // table dimensions and their basis slots (slot 0: the constant 1)
  std::vector<int64_t> soff(d, -1);
  std::vector<int32_t> td;
  std::vector<float> tdab;
  int64_t n_phi = 1;
  for (int j = 0; j < d; ++j)
    if (hot[j] || maxdeg[j] >= 2) {
      soff[j] = n_phi;
      td.insert(td.end(), {int32_t(j), int32_t(maxdeg[j]), int32_t(n_phi), fam[j]});
      tdab.insert(tdab.end(), {float(fa[j]), float(fb[j])});
      n_phi += maxdeg[j];
    }
  if (n_phi > kMaxPhi) return false;
  const int64_t n_phi_pad = (n_phi + 15) / 16 * 16;

  // rows: the nodes, by remaining budget (descending), then entry
  std::vector<char> has_kid(n, 0);
  for (int64_t e = 1; e < n; ++e) has_kid[tr.parent[e]] = 1;
  std::vector<int64_t> nodes;
  for (int64_t e = 0; e < n; ++e)
    if (has_kid[e]) nodes.push_back(e);
  {
    std::vector<int64_t> o = stable_order(int64_t(nodes.size()), [&](int64_t i) {
      return std::make_pair(-tr.rem[nodes[i]], nodes[i]);
    });
    std::vector<int64_t> s2;
    for (int64_t i : o) s2.push_back(nodes[i]);
    nodes.swap(s2);
  }
  const int64_t n_rows = int64_t(nodes.size());
  std::vector<int64_t> row_of(n, -1);
  for (int64_t r = 0; r < n_rows; ++r) row_of[nodes[r]] = r;
  std::vector<int32_t> rows(n_rows * 4, 0);
  int max_depth = 0;
  for (int64_t r = 0; r < n_rows; ++r) {
    std::vector<int64_t> p;
    for (int64_t v = nodes[r]; v != 0; v = tr.parent[v]) {
      const int64_t s = soff[tr.dim[v]];
      if (s < 0) return false;  // a node's factor must be a table slot
      p.push_back(s + tr.deg[v] - 1);
    }
    if (int(p.size()) > 8) return false;
    std::reverse(p.begin(), p.end());
    max_depth = std::max(max_depth, int(p.size()));
    for (size_t q = 0; q < p.size(); ++q) rows[r * 4 + q / 2] |= int32_t(uint32_t(p[q]) << (16 * (q % 2)));
  }

  // coefficients
  std::vector<int64_t> lin_dims;
  for (int j = 0; j < d; ++j)
    if (soff[j] < 0 && maxdeg[j] == 1) lin_dims.push_back(j);
  const int64_t lin0 = lin_dims.empty() ? 0 : lin_dims.front() / kBox * kBox;
  const int64_t n_cols = lin_dims.empty() ? 0 : (lin_dims.back() + 1 - lin0 + 15) / 16 * 16;
  std::vector<double> Bt(size_t(n_rows * n_phi_pad), 0.0), Bl(size_t(n_rows * n_cols), 0.0);
  std::vector<int64_t> t_rows(1, 0);  // K extent of the table chunk
  std::vector<int64_t> col_rows(n_cols, 0);
  bool any_table = false;
  for (int64_t e = 1; e < n; ++e) {
    const int64_t r = row_of[tr.parent[e]];
    const int j = tr.dim[e];
    if (soff[j] >= 0) {
      Bt[r * n_phi_pad + soff[j] + tr.deg[e] - 1] = double(C[e]);
      t_rows[0] = std::max(t_rows[0], r + 1);
      any_table = true;
    } else {
      if (tr.deg[e] != 1) return false;
      const double a0 = fam[j] == 0 ? 1.0 : sqrt(2.0);
      Bl[r * n_cols + (j - lin0)] = double(C[e]) * a0 * fa[j];
      col_rows[j - lin0] = std::max(col_rows[j - lin0], r + 1);
      if (fb[j] != 0.0) {
        Bt[r * n_phi_pad] += double(C[e]) * a0 * fb[j];
        t_rows[0] = std::max(t_rows[0], r + 1);
        any_table = true;
      }
    }
  }
  const int64_t kt_t = any_table ? (t_rows[0] + kStep - 1) / kStep : 0;
  struct Chunk {
    int64_t N, nk, table, col0;
  };
  // chunk order: linear chunks (their contraction starts the x stream) with
  // the table chunks spread among them, so that the table chunks' longer
  // products run while earlier linear chunks are summed
  std::vector<Chunk> lin, tab, chunks;
  int64_t n_agen = kt_t;
  for (int64_t c0 = 0; c0 < n_cols; c0 += kMaxN) {
    const int64_t N = std::min<int64_t>(kMaxN, n_cols - c0);
    int64_t rmax = 1;
    for (int64_t c = c0; c < c0 + N; ++c) rmax = std::max(rmax, col_rows[c]);
    const int64_t nk = (rmax + kStep - 1) / kStep;
    n_agen = std::max(n_agen, nk);
    lin.push_back({N, nk, 0, c0});
  }
  for (int64_t c0 = 0; any_table && c0 < n_phi_pad; c0 += kMaxN)
    tab.push_back({std::min<int64_t>(kMaxN, n_phi_pad - c0), kt_t, 1, c0});
  for (size_t q = 0, t = 0; q <= lin.size(); ++q) {
    // table chunk t goes after (t + 1) * n_lin / (n_tab + 1) linear chunks
    while (t < tab.size() && q == (t + 1) * lin.size() / (tab.size() + 1)) chunks.push_back(tab[t++]);
    if (q < lin.size()) chunks.push_back(lin[q]);
  }
  if (chunks.empty() || int(chunks.size()) > kMaxChunks || n_agen > kMaxSteps) return false;
  if (smem_layout(n_phi_pad).total > kSmemLimit) return false;

  // coefficient stages in the order the MMA thread consumes them: per chunk
  // its K steps from the last (small terms) to the first
  std::vector<uint16_t> img;
  std::vector<int32_t> chunk_tab;
  int64_t stages = 0;
  for (const Chunk& ch : chunks) {
    chunk_tab.insert(chunk_tab.end(), {int32_t(ch.N | (ch.table << 16)), int32_t(ch.nk), int32_t(img.size() * 2 / 16),
                                       int32_t(ch.table ? ch.col0 : ch.col0 / kBox)});
    for (int64_t kk = ch.nk - 1; kk >= 0; --kk) {
      const size_t base = img.size();
      img.resize(base + size_t(kSplits * ch.N * 16), 0);
      for (int64_t nn = 0; nn < ch.N; ++nn)
        for (int k = 0; k < kStep; ++k) {
          const int64_t r = kk * kStep + k;
          double v = 0.0;
          if (r < n_rows) v = ch.table ? Bt[r * n_phi_pad + ch.col0 + nn] : Bl[r * n_cols + ch.col0 + nn];
          const float f = float(v);
          const uint16_t h = bf16_rn(f);
          const float r1 = f - bf16_value(h);
          const uint16_t m = bf16_rn(r1);
          const uint16_t l = bf16_rn(r1 - bf16_value(m));
          const uint16_t parts[3] = {h, m, l};
          const size_t off = size_t(nn * 16 + (((k >> 3) ^ ((nn >> 2) & 1)) << 3) + (k & 7));
          for (int sp = 0; sp < kSplits; ++sp) img[base + size_t(sp * ch.N * 16) + off] = parts[sp];
        }
      ++stages;
    }
  }
  std::vector<int32_t> img32((img.size() + 1) / 2, 0);
  std::memcpy(img32.data(), img.data(), img.size() * 2);

  // units of 8 linear columns: inactive dimensions and those past d are
  // masked (never read; their coordinates do not enter the interpolant)
  const int64_t n_boxes = n_cols / kBox;
  std::vector<int32_t> box(n_boxes, 0);
  for (int64_t b = 0; b < n_boxes; ++b)
    for (int i = 0; i < kBox; ++i) {
      const int64_t j = lin0 + b * kBox + i;
      if (j >= d || maxdeg[j] == 0) box[b] |= 1 << i;
    }

  out.i32["tc_td"] = td;
  out.f32["tc_tdab"] = tdab;
  out.i32["tc_row"] = rows;
  out.i32["tc_chunk"] = chunk_tab;
  out.i32["tc_b"] = img32;
  out.i32["tc_box"] = box;
  out.scalar["tc_n_td"] = double(td.size() / 4);
  out.scalar["tc_n_phi"] = double(n_phi);
  out.scalar["tc_n_phi_pad"] = double(n_phi_pad);
  out.scalar["tc_n_rows"] = double(n_rows);
  out.scalar["tc_max_depth"] = double(max_depth);
  out.scalar["tc_n_agen"] = double(n_agen);
  out.scalar["tc_kt_table"] = double(kt_t);
  out.scalar["tc_n_chunks"] = double(chunks.size());
  out.scalar["tc_n_boxes"] = double(n_boxes);
  out.scalar["tc_lin0"] = double(lin0);
  {
    int64_t lo = d, hi = 0;
    for (size_t q = 0; q < td.size(); q += 4) lo = std::min<int64_t>(lo, td[q]), hi = std::max<int64_t>(hi, td[q] + 1);
    lo = lo / 2 * 2;
    out.scalar["tc_td_col"] = double(td.empty() ? 0 : lo);
    out.scalar["tc_td_bytes"] = double(td.empty() ? 0 : ((hi - lo) * 8 + 15) / 16 * 16);
  }
  out.scalar["tc_stages"] = double(stages);
  out.scalar["tc_smem"] = double(smem_layout(n_phi_pad).total);
  out.scalar["c0"] = double(C[0]);
  return true;
}

// The structure shared by the per-point layouts (spectral.py _layout_front):
// hot dimensions and basis slots, hot nodes in DFS pre-order, prefix slots of
// the cold entries' parents by remaining budget (descending), hot leaves
// sorted by (parent, slot) with each node's range.
struct Front {
  std::vector<int32_t> hot_dims, hot_deg, hot_soff;
  int64_t n_hb = 0, n_vp = 0;
  int max_depth = 0;
  std::vector<int64_t> slot, vp_row, nodes, leaf, cold, starts, ends;
};

Front front(const Tree& tr, const int64_t* maxdeg, int d) {
  Front f;
  const int64_t n = tr.n;
  std::vector<char> hot(d, 0);
  for (int64_t e = 1; e < n; ++e)
    if (tr.parent[e] > 0) hot[tr.dim[tr.parent[e]]] = 1;
  std::vector<int64_t> hidx(d, -1);
  for (int j = 0; j < d; ++j)
    if (hot[j]) {
      hidx[j] = int64_t(f.hot_dims.size());
      f.hot_dims.push_back(j);
      f.hot_deg.push_back(int32_t(maxdeg[j]));
      f.hot_soff.push_back(int32_t(f.n_hb));
      f.n_hb += maxdeg[j];
    }
  std::vector<char> is_hot(n, 0);
  is_hot[0] = 1;
  std::vector<int64_t> hot_e;
  for (int64_t e = 1; e < n; ++e) {
    is_hot[e] = hot[tr.dim[e]];
    (is_hot[e] ? hot_e : f.cold).push_back(e);
  }
  f.slot.assign(n, -1);
  for (int64_t e : hot_e) f.slot[e] = f.hot_soff[hidx[tr.dim[e]]] + tr.deg[e] - 1;
  std::vector<char> hhc(n, 0), hcc(n, 0);
  for (int64_t e : hot_e) hhc[tr.parent[e]] = 1;
  for (int64_t e : f.cold) hcc[tr.parent[e]] = 1;
  std::vector<char> node_mask(n, 0);
  for (int64_t e = 0; e < n; ++e) node_mask[e] = is_hot[e] && (hhc[e] || hcc[e]);
  node_mask[0] = 1;
  for (int64_t e = 0; e < n; ++e)
    if (node_mask[e]) f.nodes.push_back(e);
  std::stable_sort(f.nodes.begin(), f.nodes.end(), [&](int64_t a, int64_t b) { return tr.rank[a] < tr.rank[b]; });
  std::vector<int64_t> S;
  for (int64_t e = 1; e < n; ++e)
    if (hcc[e]) S.push_back(e);
  std::stable_sort(S.begin(), S.end(), [&](int64_t a, int64_t b) { return -tr.rem[a] < -tr.rem[b]; });
  f.vp_row.assign(n, -1);
  f.vp_row[0] = f.n_hb;
  for (size_t i = 0; i < S.size(); ++i) f.vp_row[S[i]] = f.n_hb + 1 + int64_t(i);
  f.n_vp = 1 + int64_t(S.size());
  for (int64_t e : hot_e)
    if (!node_mask[e]) f.leaf.push_back(e);
  const std::vector<int64_t>& sl = f.slot;
  std::stable_sort(f.leaf.begin(), f.leaf.end(), [&](int64_t a, int64_t b) {
    return std::make_pair(tr.parent[a], sl[a]) < std::make_pair(tr.parent[b], sl[b]);
  });
  for (int64_t e : f.nodes) {
    f.max_depth = std::max(f.max_depth, int(tr.level[e]));
    auto lo = std::lower_bound(f.leaf.begin(), f.leaf.end(), e, [&](int64_t v, int64_t key) { return tr.parent[v] < key; });
    auto hi = std::upper_bound(f.leaf.begin(), f.leaf.end(), e, [&](int64_t key, int64_t v) { return key < tr.parent[v]; });
    f.starts.push_back(int64_t(lo - f.leaf.begin()));
    f.ends.push_back(int64_t(hi - f.leaf.begin()));
  }
  return f;
}

// Port of spectral.py build_layout (4 segments).
bool build_perpoint(const Tree& tr, const float* C, int d_out, const int64_t* maxdeg, int d, const int32_t* fam,
                    const double* fa, const double* fb, Tables& out) {
  constexpr int nseg = 4;
  const int64_t dstride = d_out == 1 ? 1 : round4(d_out);
  auto Cv = [&](int64_t e, int o) { return C[e * d_out + o]; };
  Front f = front(tr, maxdeg, d);
  const std::vector<int32_t>& hot_dims = f.hot_dims;
  const std::vector<int32_t>& hot_deg = f.hot_deg;
  const std::vector<int32_t>& hot_soff = f.hot_soff;
  const std::vector<int64_t>& slot = f.slot;
  const std::vector<int64_t>& vp_row = f.vp_row;
  const std::vector<int64_t>& nodes = f.nodes;
  const std::vector<int64_t>& cold_e = f.cold;
  const int64_t n_hb = f.n_hb, n_vp = f.n_vp;
  const int max_depth = f.max_depth;
  int64_t row = round4(n_hb + n_vp);
  while (row % 32 != 4) row += 4;
  Runs runs{dstride, {}, {}};
  const int64_t NN = int64_t(nodes.size());
  std::vector<int32_t> node_tab(NN * 4);
  std::vector<float> node_c(NN * dstride, 0.f);
  std::vector<double> cost_nodes(NN);
  for (int64_t i = 0; i < NN; ++i) {
    const int64_t e = nodes[i];
    std::vector<int64_t> le(f.leaf.begin() + f.starts[i], f.leaf.begin() + f.ends[i]), sl;
    for (int64_t v : le) sl.push_back(slot[v]);
    const auto rr = runs.add(sl, [&](size_t q, int o) { return Cv(le[q], o); }, d_out, 0);
    const int64_t s0 = e != 0 ? slot[e] : 0;
    node_tab[i * 4 + 0] = int32_t(s0 | (int64_t(tr.level[e]) << 16));
    node_tab[i * 4 + 1] = int32_t(e != 0 && vp_row[e] >= 0 ? vp_row[e] : -1);
    node_tab[i * 4 + 2] = int32_t(rr.first);
    node_tab[i * 4 + 3] = int32_t(rr.second);
    if (e != 0)
      for (int o = 0; o < d_out; ++o) node_c[i * dstride + o] = Cv(e, o);
    double len = 0;
    for (int64_t r = rr.first; r < rr.second; ++r) len += runs.tab[r * 4 + 1];
    cost_nodes[i] = 12 + len / 4.0 * (1 + d_out);
  }
  // cold entries sorted by (dim, deg, prefix row)
  std::vector<int64_t> ce = cold_e;
  std::stable_sort(ce.begin(), ce.end(), [&](int64_t a, int64_t b) {
    return std::make_tuple(tr.dim[a], tr.deg[a], vp_row[tr.parent[a]]) <
           std::make_tuple(tr.dim[b], tr.deg[b], vp_row[tr.parent[b]]);
  });
  std::vector<std::pair<size_t, size_t>> bounds, simple, general;
  for (size_t i = 0; i < ce.size();) {
    size_t j = i;
    while (j < ce.size() && tr.dim[ce[j]] == tr.dim[ce[i]]) ++j;
    bounds.push_back({i, j});
    i = j;
  }
  for (const auto& b : bounds) {
    bool all1 = true;
    for (size_t q = b.first; q < b.second; ++q) all1 = all1 && tr.deg[ce[q]] == 1;
    (d_out == 1 && all1 ? simple : general).push_back(b);
  }
  auto alpha0 = [&](int dd) { return fam[dd] == 0 ? 1.0 : sqrt(2.0); };
  std::vector<int32_t> blk_dims, blk_run;
  std::vector<float> blk_ab;
  std::vector<double> cost_blk;
  for (size_t q = 0; q < simple.size(); q += 4) {
    const size_t np = std::min<size_t>(4, simple.size() - q);
    std::vector<int32_t> dims4;
    std::vector<int64_t> sl;
    for (size_t jj = 0; jj < np; ++jj) {
      dims4.push_back(tr.dim[ce[simple[q + jj].first]]);
      for (size_t r = simple[q + jj].first; r < simple[q + jj].second; ++r) sl.push_back(vp_row[tr.parent[ce[r]]]);
    }
    std::sort(sl.begin(), sl.end());
    sl.erase(std::unique(sl.begin(), sl.end()), sl.end());
    const int64_t a0 = sl.front() & ~int64_t(3);
    const int64_t n4 = (round4(sl.back() + 1) - a0) / 4;
    std::vector<float> blk(size_t(n4 * 16), 0.f);  // [slot][dimension]
    for (size_t jj = 0; jj < np; ++jj)
      for (size_t r = simple[q + jj].first; r < simple[q + jj].second; ++r) {
        const int64_t v = ce[r];
        blk[size_t((vp_row[tr.parent[v]] - a0) * 4 + int64_t(jj))] = Cv(v, 0);
      }
    float ab[8] = {0};
    for (size_t jj = 0; jj < np; ++jj) {
      const int dd = dims4[jj];
      ab[jj] = float(alpha0(dd) * fa[dd]);
      ab[4 + jj] = float(alpha0(dd) * fb[dd]);
    }
    while (dims4.size() < 4) dims4.push_back(dims4[0]);
    blk_dims.insert(blk_dims.end(), dims4.begin(), dims4.end());
    blk_run.insert(blk_run.end(), {int32_t(a0), int32_t(n4), int32_t(runs.coef.size()), 0});
    runs.coef.insert(runs.coef.end(), blk.begin(), blk.end());
    blk_ab.insert(blk_ab.end(), ab, ab + 8);
    cost_blk.push_back(16.0 + 9.0 * double(n4));
  }
  std::vector<int32_t> cold_tab;
  std::vector<float> cold_ab;
  std::vector<double> cost_cold;
  for (const auto& b : general) {
    const int dd = tr.dim[ce[b.first]];
    const int64_t r_first = runs.n();
    double c = 8.0;
    int gmax = 0;
    for (size_t q = b.first; q < b.second;) {
      const int g = tr.deg[ce[q]];
      size_t q2 = q;
      while (q2 < b.second && tr.deg[ce[q2]] == g) ++q2;
      std::vector<int64_t> grp(ce.begin() + q, ce.begin() + q2), sl;
      for (int64_t v : grp) sl.push_back(vp_row[tr.parent[v]]);
      const auto rr = runs.add(sl, [&](size_t k, int o) { return Cv(grp[k], o); }, d_out, g);
      for (int64_t r = rr.first; r < rr.second; ++r) c += 3 + runs.tab[r * 4 + 1] / 4.0 * (1 + d_out);
      gmax = std::max(gmax, g);
      q = q2;
    }
    cold_tab.insert(cold_tab.end(), {dd, int32_t(r_first), int32_t(runs.n()), int32_t(gmax | (fam[dd] << 16))});
    cold_ab.push_back(float(fa[dd]));
    cold_ab.push_back(float(fb[dd]));
    cost_cold.push_back(c);
  }
  std::vector<int64_t> allowed_nodes, all_cold, all_blk;
  for (int64_t i = 0; i <= NN; ++i)
    if (i == NN || tr.level[nodes[i]] <= 1) allowed_nodes.push_back(i);
  for (int64_t i = 0; i <= int64_t(cost_cold.size()); ++i) all_cold.push_back(i);
  for (int64_t i = 0; i <= int64_t(cost_blk.size()); ++i) all_blk.push_back(i);
  out.i32["node_seg"] = cuts(cost_nodes, allowed_nodes, nseg);
  out.i32["cold_seg"] = cuts(cost_cold, all_cold, nseg);
  out.i32["block_seg"] = cuts(cost_blk, all_blk, nseg);
  out.i32["blk_dims"] = blk_dims;
  out.i32["blk_run"] = blk_run;
  out.f32["blk_ab"] = blk_ab;
  out.f32["cold_ab"] = cold_ab;
  out.i32["hot_dim"] = hot_dims;
  out.i32["hot_deg"] = hot_deg;
  out.i32["hot_soff"] = hot_soff;
  out.i32["node"] = node_tab;
  out.f32["node_c"] = node_c;
  out.i32["cold"] = cold_tab;
  out.i32["run"] = runs.tab;
  if (runs.coef.empty()) runs.coef.assign(4, 0.f);
  out.f32["coef"] = runs.coef;
  out.scalar["dstride"] = double(dstride);
  out.scalar["row"] = double(row);
  out.scalar["n_hb"] = double(n_hb);
  out.scalar["n_vp"] = double(n_vp);
  out.scalar["n_hot_dims"] = double(hot_dims.size());
  out.scalar["n_nodes"] = double(NN);
  out.scalar["n_cold_groups"] = double(cost_cold.size());
  out.scalar["max_depth"] = double(max_depth);
  out.scalar["n_cold_blocks"] = double(cost_blk.size());
  return true;
}

// Port of spectral.py build_layout64: the FP64 evaluator's layout, every
// entry of Lambda one term (slot, coefficient), no padding.
bool build_perpoint64(const Tree& tr, const double* C, int d_out, const int64_t* maxdeg, int d, const int32_t* fam,
                      const double* fa, const double* fb, Tables& out) {
  constexpr int nseg = 4;
  const int64_t dstride = d_out == 1 ? 1 : round4(d_out);
  Front f = front(tr, maxdeg, d);
  const int64_t row = (f.n_hb + f.n_vp) | 1;  // odd: 8-byte row reads of 16 consecutive points on distinct banks
  std::vector<int64_t> t_slot, t_ent;
  const int64_t NN = int64_t(f.nodes.size());
  std::vector<int32_t> node_tab(NN * 4);
  std::vector<double> node_c(size_t(NN * dstride), 0.0), cost_nodes(NN);
  for (int64_t i = 0; i < NN; ++i) {
    const int64_t e = f.nodes[i];
    const int64_t t0 = int64_t(t_slot.size());
    for (int64_t q = f.starts[i]; q < f.ends[i]; ++q) {
      t_slot.push_back(f.slot[f.leaf[q]]);
      t_ent.push_back(f.leaf[q]);
    }
    node_tab[i * 4 + 0] = int32_t((e != 0 ? f.slot[e] : 0) | (int64_t(tr.level[e]) << 16));
    node_tab[i * 4 + 1] = int32_t(e != 0 && f.vp_row[e] >= 0 ? f.vp_row[e] : -1);
    node_tab[i * 4 + 2] = int32_t(t0);
    node_tab[i * 4 + 3] = int32_t(t_slot.size());
    if (e != 0)
      for (int o = 0; o < d_out; ++o) node_c[size_t(i * dstride + o)] = C[e * d_out + o];
    cost_nodes[i] = 4.0 + double(f.ends[i] - f.starts[i]);
  }
  std::vector<int64_t> ce = f.cold;
  std::stable_sort(ce.begin(), ce.end(), [&](int64_t a, int64_t b) {
    return std::make_tuple(tr.dim[a], tr.deg[a], f.vp_row[tr.parent[a]]) <
           std::make_tuple(tr.dim[b], tr.deg[b], f.vp_row[tr.parent[b]]);
  });
  std::vector<int32_t> cold_tab, runs;
  std::vector<double> cold_ab, cost_cold;
  for (size_t i = 0; i < ce.size();) {
    size_t j = i;
    while (j < ce.size() && tr.dim[ce[j]] == tr.dim[ce[i]]) ++j;
    const int dd = tr.dim[ce[i]];
    const int32_t r_first = int32_t(runs.size() / 4);
    int gmax = 0;
    for (size_t q = i; q < j;) {
      const int g = tr.deg[ce[q]];
      size_t q2 = q;
      while (q2 < j && tr.deg[ce[q2]] == g) ++q2;
      const int64_t t0 = int64_t(t_slot.size());
      for (size_t r = q; r < q2; ++r) {
        t_slot.push_back(f.vp_row[tr.parent[ce[r]]]);
        t_ent.push_back(ce[r]);
      }
      runs.insert(runs.end(), {int32_t(t0), int32_t(t_slot.size()), g, 0});
      gmax = std::max(gmax, g);
      q = q2;
    }
    const int unit = fa[dd] == 1.0 && fb[dd] == 0.0 ? 1 : 0;
    cold_tab.insert(cold_tab.end(), {dd, r_first, int32_t(runs.size() / 4), gmax | (fam[dd] << 16) | (unit << 20)});
    cold_ab.push_back(fa[dd]);
    cold_ab.push_back(fb[dd]);
    cost_cold.push_back(3.0 + double(j - i) + 3.0 * gmax);
    i = j;
  }
  std::vector<int64_t> allowed_nodes, all_cold;
  for (int64_t i = 0; i <= NN; ++i)
    if (i == NN || tr.level[f.nodes[i]] <= 1) allowed_nodes.push_back(i);
  for (int64_t i = 0; i <= int64_t(cost_cold.size()); ++i) all_cold.push_back(i);
  const size_t T = t_slot.size();
  std::vector<double> terms(std::max<size_t>(T, 1) * 2, 0.0), coef;
  if (d_out > 1) coef.assign(std::max<size_t>(T, 1) * size_t(dstride), 0.0);
  for (size_t q = 0; q < T; ++q) {
    const int64_t bits = t_slot[q];
    memcpy(&terms[2 * q], &bits, sizeof(bits));
    if (d_out == 1)
      terms[2 * q + 1] = C[t_ent[q]];
    else
      for (int o = 0; o < d_out; ++o) coef[q * size_t(dstride) + o] = C[t_ent[q] * d_out + o];
  }
  out.i32["node_seg"] = cuts(cost_nodes, allowed_nodes, nseg);
  out.i32["cold_seg"] = cuts(cost_cold, all_cold, nseg);
  out.i32["hot_dim"] = f.hot_dims;
  out.i32["hot_deg"] = f.hot_deg;
  out.i32["hot_soff"] = f.hot_soff;
  out.i32["node"] = node_tab;
  out.i32["cold"] = cold_tab;
  out.i32["run"] = runs;
  out.f64["node_c"] = node_c;
  out.f64["cold_ab"] = cold_ab;
  out.f64["terms"] = terms;
  out.f64["coef"] = coef;
  out.scalar["d_out"] = double(d_out);
  out.scalar["dstride"] = double(dstride);
  out.scalar["row"] = double(row);
  out.scalar["n_hb"] = double(f.n_hb);
  out.scalar["n_vp"] = double(f.n_vp);
  out.scalar["n_hot_dims"] = double(f.hot_dims.size());
  out.scalar["n_nodes"] = double(NN);
  out.scalar["n_cold_groups"] = double(cost_cold.size());
  out.scalar["max_depth"] = double(f.max_depth);
  out.scalar["n_terms"] = double(T);
  return true;
}

// Tape of the tensor-core panel (spectral.py build_tape): non-root entries in
// DFS pre-order; word = basis slot | depth << 16; slots of dimension j with
// max degree m_j > 0 are dsoff[j] .. dsoff[j] + m_j - 1.
bool build_tape(const Tree& tr, const int64_t* maxdeg, int d, Tables& out) {
  int max_level = 0;
  for (int64_t e = 0; e < tr.n; ++e) max_level = std::max(max_level, int(tr.level[e]));
  if (max_level > 8) return false;
  std::vector<int32_t> dims, dmax, dsoff;
  std::vector<int64_t> idx(d, -1);
  int64_t n_slots = 0;
  for (int j = 0; j < d; ++j)
    if (maxdeg[j] > 0) {
      idx[j] = int64_t(dims.size());
      dims.push_back(j);
      dmax.push_back(int32_t(maxdeg[j]));
      dsoff.push_back(int32_t(n_slots));
      n_slots += maxdeg[j];
    }
  std::vector<int64_t> ent;
  for (int64_t e = 1; e < tr.n; ++e) ent.push_back(e);
  std::stable_sort(ent.begin(), ent.end(), [&](int64_t a, int64_t b) { return tr.rank[a] < tr.rank[b]; });
  std::vector<int32_t> tape, ent32, lvl1;
  for (size_t i = 0; i < ent.size(); ++i) {
    const int64_t e = ent[i];
    const int64_t slot = dsoff[idx[tr.dim[e]]] + tr.deg[e] - 1;
    tape.push_back(int32_t(slot | (int64_t(tr.level[e]) << 16)));
    ent32.push_back(int32_t(e));
    if (tr.level[e] == 1) lvl1.push_back(int32_t(i));
  }
  out.i32["dims"] = dims;
  out.i32["dmax"] = dmax;
  out.i32["dsoff"] = dsoff;
  out.i32["tape"] = tape;
  out.i32["ent"] = ent32;
  out.i32["lvl1"] = lvl1;
  out.scalar["n_slots"] = double(n_slots);
  out.scalar["K"] = double(ent.size());
  out.scalar["ldk"] = double(round32(std::max<int64_t>(int64_t(ent.size()), 1)));
  return true;
}

}  // namespace layout
}  // namespace smx

// ---- C ABI of the host builders (inspection and tests) -----------------------------

struct smx_host_tables {
  smx::layout::Tables t;
};

extern "C" int smx_layout_build(int kind, int64_t n, const int32_t* parent, const int32_t* dim, const int32_t* deg,
                                const int32_t* level, const int64_t* rank, const double* rem, const float* C,
                                int d_out, const int64_t* maxdeg, int d, const int32_t* fam, const double* fa,
                                const double* fb, smx_host_tables** out) {
  SMX_REQUIRE(out && n >= 1 && d >= 1 && d_out >= 1 && parent && dim && deg && level && rank && rem && maxdeg && fam &&
                  fa && fb && (kind == SMX_LAYOUT_TAPE || C),
              "smx_layout_build: bad arguments");
  *out = nullptr;
  smx::layout::Tree tr{n, parent, dim, deg, level, rank, rem};
  auto h = std::make_unique<smx_host_tables>();
  bool ok = false;
  if (kind == SMX_LAYOUT_BLOCKED) {
    SMX_REQUIRE(d_out == 1, "smx_layout_build: the blocked evaluator has one output");
    ok = smx::layout::build_blocked(tr, C, maxdeg, d, fam, fa, fb, h->t);
  } else if (kind == SMX_LAYOUT_PERPOINT) {
    ok = smx::layout::build_perpoint(tr, C, d_out, maxdeg, d, fam, fa, fb, h->t);
  } else if (kind == SMX_LAYOUT_TAPE) {
    ok = smx::layout::build_tape(tr, maxdeg, d, h->t);
  } else if (kind == SMX_LAYOUT_BLOCKED_TC) {
    SMX_REQUIRE(d_out == 1, "smx_layout_build: the blocked evaluator has one output");
    ok = smx::layout::build_blocked_tc(tr, C, maxdeg, d, fam, fa, fb, h->t);
  } else {
    return smx::set_error(SMX_ERR_ARG, "smx_layout_build: unknown layout kind");
  }
  if (!ok) return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_layout_build: the plan is outside this evaluator's limits");
  *out = h.release();
  return SMX_OK;
}

extern "C" int smx_layout_build_f64(int kind, int64_t n, const int32_t* parent, const int32_t* dim,
                                    const int32_t* deg, const int32_t* level, const int64_t* rank, const double* rem,
                                    const double* C, int d_out, const int64_t* maxdeg, int d, const int32_t* fam,
                                    const double* fa, const double* fb, smx_host_tables** out) {
  SMX_REQUIRE(out && n >= 1 && d >= 1 && d_out >= 1 && parent && dim && deg && level && rank && rem && maxdeg && fam &&
                  fa && fb && C,
              "smx_layout_build_f64: bad arguments");
  SMX_REQUIRE(kind == SMX_LAYOUT_PERPOINT, "smx_layout_build_f64: only the per-point layout has an FP64 form");
  *out = nullptr;
  smx::layout::Tree tr{n, parent, dim, deg, level, rank, rem};
  auto h = std::make_unique<smx_host_tables>();
  if (!smx::layout::build_perpoint64(tr, C, d_out, maxdeg, d, fam, fa, fb, h->t))
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_layout_build_f64: the plan is outside this evaluator's limits");
  *out = h.release();
  return SMX_OK;
}

extern "C" int smx_layout_f64(const smx_host_tables* h, const char* name, const double** data, int64_t* count) {
  SMX_REQUIRE(h && name && data && count, "smx_layout_f64: null argument");
  auto it = h->t.f64.find(name);
  SMX_REQUIRE(it != h->t.f64.end(), std::string("smx_layout_f64: no double table ") + name);
  *data = it->second.data();
  *count = int64_t(it->second.size());
  return SMX_OK;
}

extern "C" int smx_layout_i32(const smx_host_tables* h, const char* name, const int32_t** data, int64_t* count) {
  SMX_REQUIRE(h && name && data && count, "smx_layout_i32: null argument");
  auto it = h->t.i32.find(name);
  SMX_REQUIRE(it != h->t.i32.end(), std::string("smx_layout_i32: no int32 table ") + name);
  *data = it->second.data();
  *count = int64_t(it->second.size());
  return SMX_OK;
}

extern "C" int smx_layout_f32(const smx_host_tables* h, const char* name, const float** data, int64_t* count) {
  SMX_REQUIRE(h && name && data && count, "smx_layout_f32: null argument");
  auto it = h->t.f32.find(name);
  SMX_REQUIRE(it != h->t.f32.end(), std::string("smx_layout_f32: no float table ") + name);
  *data = it->second.data();
  *count = int64_t(it->second.size());
  return SMX_OK;
}

extern "C" int smx_layout_scalar(const smx_host_tables* h, const char* name, double* value) {
  SMX_REQUIRE(h && name && value, "smx_layout_scalar: null argument");
  auto it = h->t.scalar.find(name);
  SMX_REQUIRE(it != h->t.scalar.end(), std::string("smx_layout_scalar: no scalar ") + name);
  *value = it->second;
  return SMX_OK;
}

extern "C" void smx_layout_free(smx_host_tables* h) { delete h; }
