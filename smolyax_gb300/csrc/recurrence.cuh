// Three-term recurrence of the orthogonal polynomial families of the
// orthogonal form: phi_{n+1} = alpha_n z phi_n - beta_n phi_{n-1}, phi_0 = 1,
// phi_{-1} = 0.  Family 0: Legendre P_n (Leja rules, z in [-1, 1]); family 1:
// normalised Hermite psi_n = H_n / sqrt(2^n n!) (Gauss-Hermite rules).
#pragma once

#include <math.h>

namespace smx {

__host__ __device__ inline void rec_coeffs(int fam, int n, double* a, double* b) {
  if (fam == 0) {  // Legendre: P_{n+1} = ((2n+1) z P_n - n P_{n-1}) / (n+1)
    *a = double(2 * n + 1) / double(n + 1);
    *b = double(n) / double(n + 1);
  } else {  // Hermite: psi_{n+1} = sqrt(2/(n+1)) z psi_n - sqrt(n/(n+1)) psi_{n-1}
    *a = sqrt(2.0 / double(n + 1));
    *b = sqrt(double(n) / double(n + 1));
  }
}

}  // namespace smx
