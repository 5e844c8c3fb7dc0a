// FP64 evaluation of the orthogonal form (one output per pass, or four).
//
// The interpolant's combination sum (interpolation.py:264-304 over
// barycentric.py:69-123) visits every tensor-product summand: ~6.6e4 FP64
// multiply-adds per point at d_in = 1000, |Lambda| = 9999, and it cancels
// (terms ~1e4 times the result), which leaves 1e-13 .. 1e-10 of rounding
// error in any FP64 evaluation of it.  The orthogonal form sums one term per
// entry of Lambda (9999 per point), with coefficients whose cancellation was
// done once, by compensated sums, when they were computed; its terms are of
// the size of the result (sum |term| / |y| ~ 2.4 at that workload), so plain
// FP64 sums leave ~1e-14.  On GB300, whose FP64 rate is 2 multiply-adds per
// SM clock, the work per point is the bound: this evaluator does one DFMA per
// term and output, plus a few per hot basis value, hot node and cold
// dimension.
//
// Organisation as the FP32 per-point evaluator (spectral.cu), with 64 points
// per block: 8 warps = 2 point groups x 4 work segments; a row of `row` doubles
// per point holds the hot basis values and the products of the hot prefixes
// that cold entries extend; hot nodes are visited in DFS pre-order with the
// path products on a register stack; each cold dimension reads its x column
// once.  Unlike the FP32 layout, every entry of Lambda is exactly one term
// (slot, coefficients) with no padding: per entry and output one multiply-add,
// the slot read from the term (a uniform 16-byte load), then the row value.
// With several outputs, block row blockIdx.y evaluates outputs 4y .. 4y+3.
#include <math.h>

#include <cmath>

#include "common.cuh"
#include "recurrence.cuh"

namespace {

constexpr int kSeg = 4;
// Points per block: 64, 96 or 128, picked per launch for the fewest idle SM
// slots in the last wave (a point's arithmetic does not depend on the choice).
// With 64, two blocks fit an SM when the row is <= ~215 doubles, so one
// block's load-bound basis phase overlaps the other's multiply-adds.
constexpr int kMaxRec = 512;
constexpr size_t kSmemMax = 227 * 1024;

struct Spec64Args {
  int d_in, d_out, dstride, row, n_hb, n_vp, n_hot_dims;
  int node_seg[kSeg + 1];
  int cold_seg[kSeg + 1];
  const int32_t* hot_dim;
  const int32_t* hot_deg;
  const int32_t* hot_soff;
  const int4* node;
  const double* node_c;  // [n_nodes][dstride]
  const int4* cold;
  const double2* cold_ab;
  const int4* run;
  const double2* terms;  // (slot bits, coefficient when d_out = 1)
  const double* coef;    // [n_terms][dstride] when d_out > 1
  const double* fam_a;
  const double* fam_b;
  const int32_t* fam;
  const double* c0;      // [d_out]
};

__constant__ double c_alpha64[2][kMaxRec];
__constant__ double c_beta64[2][kMaxRec];

// Infinite coordinates become NaN, as in the barycentric evaluation, whose
// weights w/(x - node) vanish and normalise to 0/0 there.
__device__ __forceinline__ double xin(double v) {
  const long long b = __double_as_longlong(v);
  return (b & 0x7fffffffffffffffll) == 0x7ff0000000000000ll ? __longlong_as_double(0x7ff8000000000000ll) : v;
}

// s[q] += sum over the terms [t0, t1) of coefficient (output o0 + q) * row
// value: one output from the packed terms, or four from the coefficient rows.
template <int DO>
__device__ __forceinline__ void sum_terms(const double* __restrict__ Rw, const Spec64Args& a, int o0, int t0, int t1,
                                          double (&s)[DO]) {
  if constexpr (DO == 1) {
#pragma unroll 4
    for (int t = t0; t < t1; ++t) {
      const double2 tc = __ldg(a.terms + t);
      s[0] = fma(tc.y, Rw[__double2loint(tc.x)], s[0]);
    }
  } else {
#pragma unroll 2
    for (int t = t0; t < t1; ++t) {
      const double r = Rw[__double2loint(__ldg(&a.terms[t].x))];
      const double2* c = reinterpret_cast<const double2*>(a.coef + int64_t(t) * a.dstride + o0);
      const double2 c01 = __ldg(c), c23 = __ldg(c + 1);
      s[0] = fma(c01.x, r, s[0]);
      s[1] = fma(c01.y, r, s[1]);
      s[2] = fma(c23.x, r, s[2]);
      s[3] = fma(c23.y, r, s[3]);
    }
  }
}

template <int DO, int kTP>
__global__ void __launch_bounds__(kSeg * kTP, kTP == 64 ? 2 : 1)
    spectral_eval64_kernel(Spec64Args a, const double* __restrict__ x, int64_t P, int64_t ldx,
                           double* __restrict__ y) {
  extern __shared__ __align__(16) double sm64[];
  double* RED = sm64 + size_t(a.row) * kTP;  // [kSeg][DO][kTP]
  const int o0 = blockIdx.y * DO;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int seg = warp / (kTP / 32);
  const int pl = (warp % (kTP / 32)) * 32 + lane;
  const int64_t p = blockIdx.x * int64_t(kTP) + pl;
  const bool live = p < P;
  const double* __restrict__ xp = x + (live ? p : 0) * ldx;
  double* Rw = sm64 + size_t(pl) * a.row;

  // phase 0: hot basis values phi_1..phi_g of every hot dimension; the empty
  // prefix (= 1); zeros in the other prefix slots and the padding
  for (int h = seg; h < a.n_hot_dims; h += kSeg) {
    const int dim = __ldg(a.hot_dim + h), g = __ldg(a.hot_deg + h), so = __ldg(a.hot_soff + h);
    const int fm = __ldg(a.fam + dim);
    const double z = fma(__ldg(a.fam_a + dim), xin(xp[dim]), __ldg(a.fam_b + dim));
    double pm1 = 0.0, pc = 1.0;
    for (int n = 0; n < g; ++n) {
      const double pn = fma(c_alpha64[fm][n] * z, pc, -c_beta64[fm][n] * pm1);
      pm1 = pc;
      pc = pn;
      Rw[so + n] = pc;
    }
  }
  if (seg == 0) {
    Rw[a.n_hb] = 1.0;
    for (int i = a.n_hb + 1; i < a.row; ++i) Rw[i] = 0.0;
  }
  __syncthreads();

  double acc[DO];
#pragma unroll
  for (int q = 0; q < DO; ++q) acc[q] = 0.0;

  // phase 1: hot nodes of this segment: v_node * (c_node + sum of the terms of
  // its leaf children); the node's product is stored for the cold entries
  {
    double st1 = 1.0, st2 = 1.0, st3 = 1.0, st4 = 1.0, st5 = 1.0, st6 = 1.0, st7 = 1.0, st8 = 1.0;
    for (int i = a.node_seg[seg]; i < a.node_seg[seg + 1]; ++i) {
      const int4 nd = __ldg(a.node + i);
      const int slot = nd.x & 0xffff;
      const int depth = nd.x >> 16;
      double v;
      if (depth == 0) {
        v = 1.0;
      } else {
        const double b = Rw[slot];
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
      double sv[DO];
#pragma unroll
      for (int q = 0; q < DO; ++q) sv[q] = __ldg(a.node_c + int64_t(i) * a.dstride + o0 + q);
      sum_terms<DO>(Rw, a, o0, nd.z, nd.w, sv);
#pragma unroll
      for (int q = 0; q < DO; ++q) acc[q] = fma(v, sv[q], acc[q]);
    }
  }
  __syncthreads();  // prefix products complete

  // phase 2: cold dimensions of this segment: per degree g (runs sorted by
  // degree) phi_g(z) * sum of the terms over the prefix slots; the x column
  // of group gi + 16 is prefetched into L2, the one of group gi + 1 into
  // registers
  {
    const int g0 = a.cold_seg[seg], g1 = a.cold_seg[seg + 1];
    int4 cg = g0 < g1 ? __ldg(a.cold + g0) : make_int4(0, 0, 0, 0);
    double xn = g0 < g1 ? xp[cg.x] : 0.0;
    for (int gi = g0; gi < g1; ++gi) {
      const int4 cur = cg;
      const double xv = xin(xn);
      if (gi + 16 < g1) {
        const double* pf = xp + __ldg(&a.cold[gi + 16].x);
        asm volatile("prefetch.global.L2 [%0];" ::"l"(pf));
      }
      if (gi + 1 < g1) {
        cg = __ldg(a.cold + gi + 1);
        xn = xp[cg.x];
      }
      const int fm = (cur.w >> 16) & 0xf;
      double z = xv;
      if (!((cur.w >> 20) & 1)) {
        const double2 ab = __ldg(a.cold_ab + gi);
        z = fma(ab.x, xv, ab.y);
      }
      // phi_1 = alpha_0 z (alpha_0 = 1 for Legendre), then the recurrence
      double pm1 = 1.0, pc = fm == 0 ? z : c_alpha64[fm][0] * z;
      int gcur = 1;
      for (int r = cur.y; r < cur.z; ++r) {
        const int4 rr = __ldg(a.run + r);
        while (gcur < rr.z) {
          const double pn = fma(c_alpha64[fm][gcur] * z, pc, -c_beta64[fm][gcur] * pm1);
          pm1 = pc;
          pc = pn;
          ++gcur;
        }
        double sv[DO];
#pragma unroll
        for (int q = 0; q < DO; ++q) sv[q] = 0.0;
        sum_terms<DO>(Rw, a, o0, rr.x, rr.y, sv);
#pragma unroll
        for (int q = 0; q < DO; ++q) acc[q] = fma(pc, sv[q], acc[q]);
      }
    }
  }

  // phase 3: the segments' sums, in a fixed order
#pragma unroll
  for (int q = 0; q < DO; ++q) RED[(seg * DO + q) * kTP + pl] = acc[q];
  __syncthreads();
  if (seg == 0 && live) {
#pragma unroll
    for (int q = 0; q < DO; ++q) {
      if (o0 + q >= a.d_out) continue;
      double s = __ldg(a.c0 + o0 + q);
#pragma unroll
      for (int r = 0; r < kSeg; ++r) s += RED[(r * DO + q) * kTP + pl];
      y[p * a.d_out + o0 + q] = s;
    }
  }
}

bool g_consts64_ready = false;

int upload_consts64() {
  if (g_consts64_ready) return SMX_OK;
  static double al[2][kMaxRec], be[2][kMaxRec];
  for (int f = 0; f < 2; ++f)
    for (int n = 0; n < kMaxRec; ++n) smx::rec_coeffs(f, n, &al[f][n], &be[f][n]);
  if (cudaMemcpyToSymbol(c_alpha64, al, sizeof(al)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_beta64, be, sizeof(be)) != cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "smx_spectral_eval64: constant upload failed");
  g_consts64_ready = true;
  return SMX_OK;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

// Launch with the block size of the fewest idle SM slots in the last wave:
// cost = waves * (resident blocks per SM * points per block), the points an SM
// could have evaluated in that time, 15 % dearer with a single resident block
// (measured at d_in = 1000: two blocks per SM overlap one block's load-bound
// basis phase with the other's multiply-adds).
template <int DO, int TP>
int occupancy64(size_t smem, int* occ) {
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(spectral_eval64_kernel<DO, TP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(kSmemMax)) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_spectral_eval64: shared-memory attribute");
    attr_set = true;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, spectral_eval64_kernel<DO, TP>, kSeg * TP, smem) !=
      cudaSuccess)
    return smx::set_error(SMX_ERR_CUDA, "smx_spectral_eval64: occupancy query");
  return SMX_OK;
}

template <int DO>
int launch64(const Spec64Args& a, const double* x, int64_t P, int64_t ldx, double* y, unsigned chunks,
             size_t row_bytes, void* stream) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_spectral_eval64: no device");
  }
  const int tps[3] = {64, 96, 128};
  int best = -1;
  double best_cost = 0.0;
  for (int i = 0; i < 3; ++i) {
    const size_t smem = row_bytes * tps[i];
    if (smem > kSmemMax) continue;
    int occ = 0, rc;
    if (i == 0) rc = occupancy64<DO, 64>(smem, &occ);
    else if (i == 1) rc = occupancy64<DO, 96>(smem, &occ);
    else rc = occupancy64<DO, 128>(smem, &occ);
    if (rc) return rc;
    if (occ < 1) continue;
    const double blocks = double((P + tps[i] - 1) / tps[i]) * chunks;
    const double slots = double(sms) * occ;
    const double cost = std::ceil(blocks / slots) * occ * tps[i] * (occ >= 2 ? 1.0 : 1.15);
    if (best < 0 || cost < best_cost) best = i, best_cost = cost;
  }
  if (best < 0) return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_spectral_eval64: no block size fits");
  cudaStream_t st = smx::as_stream(stream);
  const int tp = tps[best];
  const dim3 grid(smx::grid_for(P, tp), chunks);
  const size_t smem = row_bytes * tp;
  if (tp == 64)
    spectral_eval64_kernel<DO, 64><<<grid, kSeg * 64, smem, st>>>(a, x, P, ldx, y);
  else if (tp == 96)
    spectral_eval64_kernel<DO, 96><<<grid, kSeg * 96, smem, st>>>(a, x, P, ldx, y);
  else
    spectral_eval64_kernel<DO, 128><<<grid, kSeg * 128, smem, st>>>(a, x, P, ldx, y);
  SMX_LAUNCH_CHECK("smx_spectral_eval64");
  return SMX_OK;
}

}  // namespace


extern "C" int smx_spectral_eval64(const smx_spectral64* sp, const double* x, int64_t P, int64_t ldx, double* y,
                                   void* stream) {
  const char* who = "smx_spectral_eval64";
  SMX_REQUIRE(sp != nullptr, "smx_spectral_eval64: null plan");
  SMX_REQUIRE(sp->d_out >= 1 && (sp->d_out == 1 ? sp->dstride == 1 : sp->dstride % 4 == 0 && sp->dstride >= sp->d_out),
              "smx_spectral_eval64: bad output stride");
  SMX_REQUIRE(sp->fam && sp->fam_a && sp->fam_b && sp->node && sp->node_c && sp->c0 && sp->n_nodes >= 1 &&
                  (sp->n_hot_dims == 0 || (sp->hot_dim && sp->hot_deg && sp->hot_soff)) &&
                  (sp->n_terms == 0 || (sp->terms && (sp->d_out == 1 || sp->coef))) &&
                  (sp->n_cold_groups == 0 || (sp->cold && sp->cold_ab && sp->run)),
              "smx_spectral_eval64: incomplete plan");
  if (sp->max_depth > 8) return smx::set_error(SMX_ERR_UNSUPPORTED, std::string(who) + ": hot nodes deeper than 8");
  SMX_REQUIRE(sp->n_vp >= 1 && sp->row >= sp->n_hb + sp->n_vp, "smx_spectral_eval64: bad row");
  for (int i = 0; i < kSeg; ++i)
    SMX_REQUIRE(sp->node_seg[i] <= sp->node_seg[i + 1] && sp->cold_seg[i] <= sp->cold_seg[i + 1],
                "smx_spectral_eval64: segments not ordered");
  SMX_REQUIRE(sp->node_seg[0] == 0 && sp->node_seg[kSeg] == sp->n_nodes && sp->cold_seg[0] == 0 &&
                  sp->cold_seg[kSeg] == sp->n_cold_groups,
              "smx_spectral_eval64: segments do not cover the plan");
  SMX_REQUIRE((!sp->terms || aligned(sp->terms, 16)) && (!sp->coef || aligned(sp->coef, 32)) &&
                  (sp->d_out == 1 || aligned(sp->node_c, 32)),
              "smx_spectral_eval64: tables not aligned");
  SMX_REQUIRE(P >= 0 && ldx >= sp->d_in, "smx_spectral_eval64: bad sizes");
  const int DO = sp->d_out == 1 ? 1 : 4;
  const size_t row_bytes = (size_t(sp->row) + size_t(kSeg) * DO) * sizeof(double);  // per point of a block
  if (row_bytes * 64 > kSmemMax)
    return smx::set_error(SMX_ERR_UNSUPPORTED, std::string(who) + ": per-point row too large for shared memory");
  if (P == 0) return SMX_OK;
  SMX_REQUIRE(x && y, "smx_spectral_eval64: null pointer");
  int rc = upload_consts64();
  if (rc) return rc;
  Spec64Args a;
  a.d_in = sp->d_in;
  a.d_out = sp->d_out;
  a.dstride = sp->dstride;
  a.row = sp->row;
  a.n_hb = sp->n_hb;
  a.n_vp = sp->n_vp;
  a.n_hot_dims = sp->n_hot_dims;
  for (int i = 0; i <= kSeg; ++i) {
    a.node_seg[i] = sp->node_seg[i];
    a.cold_seg[i] = sp->cold_seg[i];
  }
  a.hot_dim = sp->hot_dim;
  a.hot_deg = sp->hot_deg;
  a.hot_soff = sp->hot_soff;
  a.node = reinterpret_cast<const int4*>(sp->node);
  a.node_c = sp->node_c;
  a.cold = reinterpret_cast<const int4*>(sp->cold);
  a.cold_ab = reinterpret_cast<const double2*>(sp->cold_ab);
  a.run = reinterpret_cast<const int4*>(sp->run);
  a.terms = reinterpret_cast<const double2*>(sp->terms);
  a.coef = sp->coef;
  a.fam_a = sp->fam_a;
  a.fam_b = sp->fam_b;
  a.fam = sp->fam;
  a.c0 = sp->c0;
  const unsigned chunks = unsigned((sp->d_out + DO - 1) / DO);
  SMX_REQUIRE(chunks <= 65535, "smx_spectral_eval64: too many outputs");
  return DO == 1 ? launch64<1>(a, x, P, ldx, y, chunks, row_bytes, stream)
                 : launch64<4>(a, x, P, ldx, y, chunks, row_bytes, stream);
}
