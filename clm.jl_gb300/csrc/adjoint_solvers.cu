// adjoint_solvers.cu — reverse-mode rules of the batched linear solves.
//
// enzyme_rules.jl gives the reference's custom adjoints of its two solves:
//   band_solve!        (:80-107)   A x = r  ->  A^T lambda = xbar, rbar += lambda,
//                                  Abar -= lambda x^T on the band (LAPACK gbtrf/gbtrs 'T');
//   tridiagonal_solve! (:160-201)  the same with A^T tridiagonal (sub = c[j-1],
//                                  super = a[j+1]) solved by the same Thomas sweep.
// Here both run one system per thread over the batched layouts of batched_band_solve!
// (band_diagonal.jl:179) and tridiagonal_multi! (tridiagonal.jl:129).  The band rule
// reuses the factorisation that k_band_factor_solve stored during the forward solve
// (multipliers and row exchanges, LAPACK's product form), so the reverse pass never
// factorises again.  The operation order equals the oracle's restatement bit for bit.
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr int ADJ_BLOCK = 128;
constexpr int MAXTRI_ADJ = 64;

static inline unsigned int grid_of(int64_t n) { return (unsigned int)((n + ADJ_BLOCK - 1) / ADJ_BLOCK); }

// Forward band solve that also stores its factorisation.  Same eliminations, in the
// same order, as band_lu_solve (so x is bit-identical to k_band_solve); in addition
// each multiplier f_ik is kept in the slot of the entry it eliminated and the pivot
// row of step k is kept as the offset piv(k) - k.  lu is [ldc, W, nlev] with
// W = 2*kl+ku+1 (row i of the system at level jt+i: lu[d] = AB(i, i-kl+d)); piv is
// [ldc, nlev] bytes.
template <int KL, int KU>
__global__ void __launch_bounds__(ADJ_BLOCK)
k_band_factor_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* __restrict__ bmatrix,
                    const double* __restrict__ rvector, const int64_t* jtop, const int64_t* jbot,
                    const uint8_t* mask, int nlevsno_off, double* lu, uint8_t* piv) {
  constexpr int W = 2 * KL + KU + 1;
  constexpr int NB = KL + KU + 1;
  const int64_t c = (int64_t)blockIdx.x * ADJ_BLOCK + threadIdx.x;
  if (c >= nc || !mask[c]) return;
  const int64_t jt = jtop[c] + nlevsno_off + 1;
  const int64_t n64 = jbot[c] - jtop[c] + 1;
  if (n64 <= 0 || jt < 1 || jt + n64 - 1 > nlev || n64 > MAXROWS + 1) return;
  const int n = (int)n64;
  double ab[(MAXROWS + 1) * W];
  double x[MAXROWS + 1];
  for (int k = 0; k < n * W; k++) ab[k] = 0.0;
  for (int i = 0; i < n; i++) {
    const int64_t lev = jt + i;
    for (int j = max(0, i - KL); j <= min(n - 1, i + KU); j++)
      ab[i * W + (j - i + KL)] = bmatrix[c + (int64_t)((i - j) + KL) * ldc + (lev - 1) * ldc * NB];
    x[i] = rvector[c + (lev - 1) * ldc];
  }
  uint8_t pv[MAXROWS + 1];
  band_lu_factor_solve<KL, KU>(ab, x, pv, n);
  for (int k = 0; k < n; k++) piv[c + (jt + k - 1) * ldc] = pv[k];
  for (int i = 0; i < n; i++) {
    tvector[c + (jt + i - 1) * ldc] = x[i];
    for (int d = 0; d < W; d++) lu[c + (int64_t)d * ldc + (jt + i - 1) * ldc * W] = ab[i * W + d];
  }
}

// band_solve! reverse rule from the stored factors: U^T w = xbar (forward
// substitution, j ascending), then for k = n-2..0: w_k -= sum_i f_ik w_i (i
// ascending) and the row exchange of step k; rbar += lambda, bmatrix_bar -= lambda_i
// x_j on the band entries the forward read, xbar consumed.
template <int KL, int KU>
__global__ void __launch_bounds__(ADJ_BLOCK)
k_band_solve_adjoint(int64_t nc, int64_t ldc, int nlev, const double* __restrict__ tvector, double* tbar,
                     const double* __restrict__ lu, const uint8_t* __restrict__ piv, double* bbar, double* rbar,
                     const int64_t* jtop, const int64_t* jbot, const uint8_t* mask, int nlevsno_off) {
  constexpr int W = 2 * KL + KU + 1;
  constexpr int NB = KL + KU + 1;
  const int64_t c = (int64_t)blockIdx.x * ADJ_BLOCK + threadIdx.x;
  if (c >= nc || !mask[c]) return;
  const int64_t jt = jtop[c] + nlevsno_off + 1;
  const int64_t n64 = jbot[c] - jtop[c] + 1;
  if (n64 <= 0 || jt < 1 || jt + n64 - 1 > nlev || n64 > MAXROWS + 1) return;
  const int n = (int)n64;
  double ab[(MAXROWS + 1) * W];
  double w[MAXROWS + 1];
  for (int i = 0; i < n; i++)
    for (int d = 0; d < W; d++) ab[i * W + d] = lu[c + (int64_t)d * ldc + (jt + i - 1) * ldc * W];
  uint8_t pv[MAXROWS + 1];
  for (int i = 0; i < n; i++) {
    w[i] = tbar[c + (jt + i - 1) * ldc];
    pv[i] = piv[c + (jt + i - 1) * ldc];
  }
  band_lu_transpose_solve<KL, KU>(ab, pv, w, n);
  for (int i = 0; i < n; i++) {
    const int64_t lev = jt + i;
    if (rbar) rbar[c + (lev - 1) * ldc] += w[i];
    tbar[c + (lev - 1) * ldc] = 0.0;
  }
  if (bbar) {
    for (int j = 0; j < n; j++) {
      const double xj = tvector[c + (jt + j - 1) * ldc];
      for (int i = max(0, j - KL); i <= min(n - 1, j + KU); i++) {
        double& e = bbar[c + (int64_t)((i - j) + KL) * ldc + (jt + i - 1) * ldc * NB];
        e -= w[i] * xj;
      }
    }
  }
}

// tridiagonal_solve! reverse rule over the [ld, nlevs] layout: the transposed
// system solved by the same (unguarded) Thomas sweep as tridiagonal_solve!
// (tridiagonal.jl:35-63), then the band gradients.
__global__ void __launch_bounds__(ADJ_BLOCK)
k_tridiagonal_adjoint(int64_t ncols, int64_t ld, int nlevs, const double* __restrict__ u,
                      const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ cc,
                      double* ubar, double* abar, double* bbar, double* cbar, double* rbar, const int64_t* jtop,
                      const uint8_t* mask) {
  const int64_t col = (int64_t)blockIdx.x * ADJ_BLOCK + threadIdx.x;
  if (col >= ncols || !mask[col]) return;
  const int64_t j64 = jtop[col];
  if (j64 < 1 || j64 > nlevs) return;
  const int j0 = (int)j64, n = nlevs;
  double cp[MAXTRI_ADJ + 1], dp[MAXTRI_ADJ + 1], lam[MAXTRI_ADJ + 1];
  // transposed bands: aT[j] = c[j-1] (j > j0), bT = b, cT[j] = a[j+1] (j < n), rT = ubar
  {
    const double bT = LVc(b, col, j0, ld);
    const double cT = j0 < n ? LVc(a, col, j0 + 1, ld) : 0.0;
    cp[j0] = cT / bT;
    dp[j0] = LV(ubar, col, j0, ld) / bT;
  }
  for (int jj = j0 + 1; jj <= n; jj++) {
    const double aT = LVc(cc, col, jj - 1, ld);
    const double cT = jj < n ? LVc(a, col, jj + 1, ld) : 0.0;
    const double denom = LVc(b, col, jj, ld) - aT * cp[jj - 1];
    cp[jj] = cT / denom;
    dp[jj] = (LV(ubar, col, jj, ld) - aT * dp[jj - 1]) / denom;
  }
  lam[n] = dp[n];
  for (int jj = n - 1; jj >= j0; jj--) lam[jj] = dp[jj] - cp[jj] * lam[jj + 1];
  if (rbar)
    for (int j = j0; j <= n; j++) LV(rbar, col, j, ld) += lam[j];
  if (bbar)
    for (int j = j0; j <= n; j++) LV(bbar, col, j, ld) -= lam[j] * LVc(u, col, j, ld);
  if (abar)
    for (int j = j0 + 1; j <= n; j++) LV(abar, col, j, ld) -= lam[j] * LVc(u, col, j - 1, ld);
  if (cbar)
    for (int j = j0; j <= n - 1; j++) LV(cbar, col, j, ld) -= lam[j] * LVc(u, col, j + 1, ld);
  for (int j = j0; j <= n; j++) LV(ubar, col, j, ld) = 0.0;
}

cudaError_t launch_band_factor_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* bmatrix,
                                     const double* rvector, const int64_t* jtop, const int64_t* jbot,
                                     const uint8_t* mask, int kl, int ku, int nlevsno_off, double* lu, uint8_t* piv,
                                     cudaStream_t s) {
  if (kl == 2 && ku == 2)
    k_band_factor_solve<2, 2><<<grid_of(nc), ADJ_BLOCK, 0, s>>>(nc, ldc, nlev, tvector, bmatrix, rvector, jtop,
                                                                jbot, mask, nlevsno_off, lu, piv);
  else
    k_band_factor_solve<1, 1><<<grid_of(nc), ADJ_BLOCK, 0, s>>>(nc, ldc, nlev, tvector, bmatrix, rvector, jtop,
                                                                jbot, mask, nlevsno_off, lu, piv);
  return cudaGetLastError();
}

cudaError_t launch_band_solve_adjoint(int64_t nc, int64_t ldc, int nlev, const double* tvector, double* tbar,
                                      const double* lu, const uint8_t* piv, double* bbar, double* rbar,
                                      const int64_t* jtop, const int64_t* jbot, const uint8_t* mask, int kl, int ku,
                                      int nlevsno_off, cudaStream_t s) {
  if (kl == 2 && ku == 2)
    k_band_solve_adjoint<2, 2><<<grid_of(nc), ADJ_BLOCK, 0, s>>>(nc, ldc, nlev, tvector, tbar, lu, piv, bbar,
                                                                 rbar, jtop, jbot, mask, nlevsno_off);
  else
    k_band_solve_adjoint<1, 1><<<grid_of(nc), ADJ_BLOCK, 0, s>>>(nc, ldc, nlev, tvector, tbar, lu, piv, bbar,
                                                                 rbar, jtop, jbot, mask, nlevsno_off);
  return cudaGetLastError();
}

cudaError_t launch_tridiagonal_adjoint(int64_t ncols, int64_t ldc, int nlevs, const double* u, const double* a,
                                       const double* b, const double* c, double* ubar, double* abar, double* bbar,
                                       double* cbar, double* rbar, const int64_t* jtop, const uint8_t* mask,
                                       cudaStream_t s) {
  k_tridiagonal_adjoint<<<grid_of(ncols), ADJ_BLOCK, 0, s>>>(ncols, ldc, nlevs, u, a, b, c, ubar, abar, bbar, cbar,
                                                             rbar, jtop, mask);
  return cudaGetLastError();
}

}  // namespace clmgb
