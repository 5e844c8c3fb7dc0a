// Host-side table builders of the FP32 evaluators (see layout.cu).
#pragma once

#include <stdint.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

#include "common.cuh"

namespace smx {
namespace layout {

// Index-set tree on the host (entry 0 = root, parent[0] = -1).
struct Tree {
  int64_t n;
  const int32_t* parent;
  const int32_t* dim;
  const int32_t* deg;
  const int32_t* level;
  const int64_t* rank;  // DFS pre-order rank
  const double* rem;
};

// Named host tables of one layout.
struct Tables {
  std::map<std::string, std::vector<int32_t>> i32;
  std::map<std::string, std::vector<float>> f32;
  std::map<std::string, std::vector<double>> f64;
  std::map<std::string, double> scalar;
};

int64_t blocked_smem_bytes(int64_t n_hs, int64_t k_c);
// Each returns false when the plan is outside the evaluator's limits.
bool build_blocked(const Tree& tr, const float* C, const int64_t* maxdeg, int d, const int32_t* fam, const double* fa,
                   const double* fb, Tables& out);
bool build_perpoint(const Tree& tr, const float* C, int d_out, const int64_t* maxdeg, int d, const int32_t* fam,
                    const double* fa, const double* fb, Tables& out);
// The FP64 evaluator's layout (FP64 coefficients C[n][d_out]): every entry
// one term (slot, coefficients); FP64 tables in Tables::f64.
bool build_perpoint64(const Tree& tr, const double* C, int d_out, const int64_t* maxdeg, int d, const int32_t* fam,
                      const double* fa, const double* fb, Tables& out);
bool build_tape(const Tree& tr, const int64_t* maxdeg, int d, Tables& out);
bool build_blocked_tc(const Tree& tr, const float* C, const int64_t* maxdeg, int d, const int32_t* fam,
                      const double* fa, const double* fb, Tables& out);

}  // namespace layout
}  // namespace smx
