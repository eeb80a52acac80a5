// adjoint_step.cu — reverse mode through one whole column step.
//
// The reference differentiates a timestep by running Enzyme over the production
// physics (driver_reverse.jl:177-615 for soil_temperature!/soil_water!, reversed one
// step at a time by _reverse_step_into!, canopy_fluxes_reverse.jl:447-465).  Here one
// thread owns one column and replays the step through the SAME device code the
// production kernels run (clmgb_device.cuh, instantiated with a recording scalar
// instead of double): every FP64 operation on a quantity that depends on the step's
// inputs appends one entry (parent indices, partial derivatives) to the thread's
// tape, and the accept/reject, phase-change and pivot decisions are taken on the
// same values as in the forward run, so the replay is the forward run.  The reverse
// sweep then walks the tape backwards, accumulating adjoints, and the thread
// moves to its next column.  Two parts are not recorded operation by operation:
//  * the banded solve of soil_temperature! is one tape node that keeps the LU
//    factors and pivots and, in the reverse sweep, solves the transposed system
//    with them (the band_solve! rule);
//  * the Richards substep loop runs once on values only, keeping the liquid water
//    at the start of every accepted substep (rejected attempts leave no trace in the
//    result); the reverse pass then takes the accepted substeps last to first, each
//    reversed in closed form (mf_substep_reverse) or, with
//    CLMGB_ADJ_RICHARDS_RECORDED, replayed recorded from its checkpoint, swept and
//    rewound.  Either way the tape holds soil temperature plus at most one substep.
//
// Active quantities (differentiated): t_soisno, h2osoi_liq and h2osoi_ice on the
// active levels, t_grnd, t_h2osfc, and the hydraulic parameters watsat, bsw, sucsat,
// hksat on levels 1..nlevsoi.  Everything else is a constant of the step.  State
// that the step changes but that is not active (surface water h2osfc with
// frac_h2osfc > 0, excess ice, snow without layers) would carry sensitivity into
// the next step; columns holding any of it are flagged CLMGB_COL_ADJ_UNSUPPORTED.
//
// Tape layout: [warp][entry][lane] (int2 parent indices, double2 partials, double
// adjoint), see tape_off.
#include "adjoint_richards.cuh"
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr int VJP_BLOCK = 64;

struct TapeView {
  int2* idx;
  double2* par;
  double* adj;
  double* sub;   // per-substep checkpoints [maxsub][SUB_REC][slots]
  int64_t ld;    // slots
  int cap;       // entries per slot
  int maxsub;    // accepted substeps a column can checkpoint
  int richards_mode;  // CLMGB_ADJ_RICHARDS_*
};

__shared__ TapeView s_tape;
__shared__ int s_cur[VJP_BLOCK];
__shared__ int s_ovf[VJP_BLOCK];

__device__ __forceinline__ int64_t vjp_slot() { return (int64_t)blockIdx.x * VJP_BLOCK + threadIdx.x; }

// Offset of record k of this thread: [warp][k][lane].  A warp's tape is one
// contiguous range (few pages, so address translation stays cached while the lanes
// walk their tapes at different positions), and lanes at the same position share
// one 256-byte line.
__device__ __forceinline__ int64_t tape_off(int64_t k) {
  const int64_t slot = vjp_slot();
  return ((slot >> 5) * s_tape.cap + k) * 32 + (slot & 31);
}

// append one entry; returns its index, or -1 once the tape is full
__device__ __forceinline__ int ad_rec(int a, double pa, int b, double pb) {
  const int k = s_cur[threadIdx.x];
  if (k >= s_tape.cap) {
    s_ovf[threadIdx.x] = 1;
    return -1;
  }
  s_cur[threadIdx.x] = k + 1;
  const int64_t o = tape_off(k);
  s_tape.idx[o] = make_int2(a, b);
  s_tape.par[o] = make_double2(pa, pb);
  s_tape.adj[o] = 0.0;
  return k;
}

// The recording scalar: value and tape index (-1: a constant of the step).
struct AD {
  double v;
  int i;
  AD() = default;
  __device__ __forceinline__ AD(double x) : v(x), i(-1) {}
  __device__ __forceinline__ AD(double x, int k) : v(x), i(k) {}
};

__device__ __forceinline__ double VAL(const AD& a) { return a.v; }

__device__ __forceinline__ AD ad_unary(double v, const AD& a, double pa) {
  return a.i < 0 ? AD(v) : AD(v, ad_rec(a.i, pa, -1, 0.0));
}
__device__ __forceinline__ AD ad_binary(double v, const AD& a, double pa, const AD& b, double pb) {
  if (a.i < 0) return b.i < 0 ? AD(v) : AD(v, ad_rec(b.i, pb, -1, 0.0));
  if (b.i < 0) return AD(v, ad_rec(a.i, pa, -1, 0.0));
  return AD(v, ad_rec(a.i, pa, b.i, pb));
}

__device__ __forceinline__ AD operator-(const AD& a) { return ad_unary(-a.v, a, -1.0); }
__device__ __forceinline__ AD operator+(const AD& a, const AD& b) {
  const double v = a.v + b.v;
  if (a.i < 0) return AD(v, b.i);   // d/db = 1: the result shares b's adjoint
  if (b.i < 0) return AD(v, a.i);
  return AD(v, ad_rec(a.i, 1.0, b.i, 1.0));
}
__device__ __forceinline__ AD operator-(const AD& a, const AD& b) {
  const double v = a.v - b.v;
  if (b.i < 0) return AD(v, a.i);
  return ad_binary(v, a, 1.0, b, -1.0);
}
__device__ __forceinline__ AD operator*(const AD& a, const AD& b) { return ad_binary(a.v * b.v, a, b.v, b, a.v); }
__device__ __forceinline__ AD operator/(const AD& a, const AD& b) {
  const double v = a.v / b.v;
  if (a.i < 0 && b.i < 0) return AD(v);
  const double rb = 1.0 / b.v;
  return ad_binary(v, a, rb, b, -v * rb);
}
__device__ __forceinline__ AD& operator+=(AD& a, const AD& b) { a = a + b; return a; }
__device__ __forceinline__ AD& operator-=(AD& a, const AD& b) { a = a - b; return a; }
__device__ __forceinline__ AD& operator*=(AD& a, const AD& b) { a = a * b; return a; }
__device__ __forceinline__ AD& operator/=(AD& a, const AD& b) { a = a / b; return a; }
__device__ __forceinline__ bool operator<(const AD& a, const AD& b) { return a.v < b.v; }
__device__ __forceinline__ bool operator<=(const AD& a, const AD& b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>(const AD& a, const AD& b) { return a.v > b.v; }
__device__ __forceinline__ bool operator>=(const AD& a, const AD& b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(const AD& a, const AD& b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(const AD& a, const AD& b) { return a.v != b.v; }

// Julia max/min select one argument: the result is that argument (its adjoint).
__device__ __forceinline__ AD jl_max(const AD& x, const AD& y) {
  const double r = jl_max(x.v, y.v);
  return __double_as_longlong(r) == __double_as_longlong(x.v) ? x : y;
}
__device__ __forceinline__ AD jl_min(const AD& x, const AD& y) {
  const double r = jl_min(x.v, y.v);
  return __double_as_longlong(r) == __double_as_longlong(x.v) ? x : y;
}
__device__ __forceinline__ AD fabs(const AD& x) { return x.v < 0.0 ? -x : x; }
// x^y: d/dx = y x^(y-1) = y r / x, d/dy = r log x
__device__ __forceinline__ AD cm_pow(const AD& x, const AD& y) {
  const double r = ::cm_pow(x.v, y.v);
  if (x.i < 0 && y.i < 0) return AD(r);
  const double px = x.v != 0.0 ? y.v * r / x.v : 0.0;
  const double py = (y.i >= 0 && x.v > 0.0) ? r * ::cm_log(x.v) : 0.0;
  return ad_binary(r, x, px, y, py);
}
// x^y for a constant base x with log x = lx + lxl formed by the caller (a pair that is
// not renormalised: lx alone can be off by 2^-20): d/dy = r log x
__device__ __forceinline__ AD cm_pow_lx(double x, double lx, double lxl, const AD& y) {
  const double r = ::cm_pow_lx(x, lx, lxl, y.v);
  return ad_unary(r, y, r * (lx + lxl));
}
__device__ __forceinline__ AD cm_log10(const AD& x) {
  return ad_unary(::cm_log10(x.v), x, 0.43429448190325182765 / x.v);
}
__device__ __forceinline__ AD jl_pow4(const AD& x) { return ad_unary(jl_pow4(x.v), x, 4.0 * (x.v * x.v * x.v)); }

// The column's active state for one replayed step, with input registration.
struct AdState {
  typedef AD S;
  AD t[MAXL + 2], liq[MAXL + 2], ice[MAXL + 2], fact[MAXL + 2];
  AD icefrac[MAXSOI + 2];
  AD tg, th, qc, forc;
  AD watsat[MAXGRND + 2], bsw[MAXGRND + 2], sucsat[MAXGRND + 2], hksat[MAXGRND + 2];
  __device__ __forceinline__ AD& T(int jj) { return t[jj]; }
  __device__ __forceinline__ AD& Liq(int jj) { return liq[jj]; }
  __device__ __forceinline__ AD& Ice(int jj) { return ice[jj]; }
  __device__ __forceinline__ AD& Fact(int jj) { return fact[jj]; }
  __device__ __forceinline__ AD& Icefrac(int j) { return icefrac[j]; }
  __device__ __forceinline__ AD& Tgrnd() { return tg; }
  __device__ __forceinline__ AD& Th2osfc() { return th; }
  __device__ __forceinline__ AD& Qcharge() { return qc; }
  __device__ __forceinline__ AD ForcLwrad() const { return forc; }
  __device__ __forceinline__ AD Watsat(int j) const { return watsat[j]; }
  __device__ __forceinline__ AD Bsw(int j) const { return bsw[j]; }
  __device__ __forceinline__ AD Sucsat(int j) const { return sucsat[j]; }
  __device__ __forceinline__ AD Hksat(int j) const { return hksat[j]; }
  __device__ void band_solve(AD* ab, AD* x, int n) const;   // a band node on the tape, below
};

// The values of an AdState's parameters, for the substep loop run without recording.
struct AdValues {
  typedef double S;
  const AdState& A;
  __device__ __forceinline__ double Watsat(int j) const { return A.watsat[j].v; }
  __device__ __forceinline__ double Bsw(int j) const { return A.bsw[j].v; }
  __device__ __forceinline__ double Sucsat(int j) const { return A.sucsat[j].v; }
  __device__ __forceinline__ double Hksat(int j) const { return A.hksat[j].v; }
};

__device__ __forceinline__ AD ad_input(double v) { return AD(v, ad_rec(-1, 0.0, -1, 0.0)); }

// adjoint accumulate into the tape's adjoint of variable k
__device__ __forceinline__ void adj_add(int k, double g) {
  if (k >= 0) s_tape.adj[tape_off(k)] += g;
}
__device__ __forceinline__ double adj_get(int k) {
  return k >= 0 ? s_tape.adj[tape_off(k)] : 0.0;
}

// ---------------------------------------------------------------------------
// The banded solve as one tape node (the band_solve! rule, enzyme_rules.jl:80-107):
// the forward factorises on values and keeps the factors, the pivots, the solution
// and the tape indices of the matrix entries and right-hand side; the solution rows
// enter the tape as fresh variables after a marker entry.  When the reverse sweep
// reaches the marker, lambda = A^-T xbar comes from the stored factors, and
// rbar += lambda, Abar -= lambda x^T go to the recorded indices.
// ---------------------------------------------------------------------------
constexpr int MARK_BAND = -2;

struct BandNode {
  int n, first;
  double lu[MAXROWS * 7];
  double x[MAXROWS];
  int aidx[MAXROWS * 5];
  int ridx[MAXROWS];
  uint8_t piv[MAXROWS];
};
__shared__ BandNode* s_band[VJP_BLOCK];

template <int KL, int KU>
__device__ __forceinline__ void band_lu_solve(AD* ab, AD* x, int n) {
  static_assert(KL == 2 && KU == 2, "the column step solves a pentadiagonal system");
  constexpr int W = 2 * KL + KU + 1;
  BandNode& B = *s_band[threadIdx.x];
  B.n = n;
  for (int r = 0; r < n; r++) {
    for (int d = 0; d < KL + KU + 1; d++) B.aidx[r * 5 + d] = ab[r * W + d].i;
    for (int d = 0; d < W; d++) B.lu[r * W + d] = ab[r * W + d].v;
    B.ridx[r] = x[r].i;
    B.x[r] = x[r].v;
  }
  band_lu_factor_solve<KL, KU>(B.lu, B.x, B.piv, n);
  ad_rec(MARK_BAND, 0.0, -1, 0.0);
  B.first = s_cur[threadIdx.x];
  for (int r = 0; r < n; r++) x[r] = ad_input(B.x[r]);
}

// Reverse sweep over entries hi..lo (descending).  Most operations read values
// computed a few entries earlier, so the adjoints of the newest SWEEP_WIN entries
// below the current one live in shared memory (s_win, one column per thread) and
// only contributions to older entries go to the tape's adjoint array in global
// memory.  An entry's global part is final SWEEP_WIN iterations before the sweep
// reaches it, so the records and global parts of the next entries are loaded ahead
// of the dependent work.  Each entry's total adjoint is written back to the tape
// (tape nodes read their outputs' adjoints from there), and on return the window's
// partial sums below `lo` are added to the tape, so adj_get sees complete values.
constexpr int SWEEP_WIN = 32;
__shared__ double s_win[SWEEP_WIN * VJP_BLOCK];

__device__ __forceinline__ double& win_at(int k) { return s_win[(k & (SWEEP_WIN - 1)) * VJP_BLOCK + threadIdx.x]; }

// adds v to the adjoint of entry p while the sweep is at entry k (p < k)
__device__ __forceinline__ void sweep_add(int p, int k, double v) {
  if (p < 0) return;
  if (p > k - SWEEP_WIN) win_at(p) += v;
  else s_tape.adj[tape_off(p)] += v;
}

// the band node's reverse, at its marker entry k: the solution rows' adjoints are
// complete on the tape (they sit above the marker)
__device__ __forceinline__ void band_node_reverse(const BandNode& B, int k) {
  double w[MAXROWS];
  const int n = B.n;
  for (int r = 0; r < n; r++) w[r] = adj_get(B.first + r);
  band_lu_transpose_solve<2, 2>(B.lu, B.piv, w, n);
  for (int r = 0; r < n; r++) {
    sweep_add(B.ridx[r], k, w[r]);
    for (int d = 0; d < 5; d++) {
      const int col = r - 2 + d;
      if (col >= 0 && col < n) sweep_add(B.aidx[r * 5 + d], k, -w[r] * B.x[col]);
    }
  }
}

__device__ __forceinline__ void AdState::band_solve(AD* ab, AD* x, int n) const { band_lu_solve<2, 2>(ab, x, n); }

__device__ void sweep(int hi, int lo) {
  if (hi < lo) return;
  for (int m = hi; m > hi - SWEEP_WIN; m--) win_at(m) = 0.0;
  // two-deep prefetch of the records and the global adjoint parts
  int64_t o = tape_off(hi);
  int2 e0 = s_tape.idx[o];
  double2 p0 = s_tape.par[o];
  double g0 = s_tape.adj[o];
  int2 e1 = make_int2(-1, -1);
  double2 p1 = make_double2(0.0, 0.0);
  double g1 = 0.0;
  if (hi - 1 >= lo) {
    const int64_t o1 = o - 32;
    e1 = s_tape.idx[o1];
    p1 = s_tape.par[o1];
    g1 = s_tape.adj[o1];
  }
  for (int k = hi; k >= lo; k--, o -= 32) {
    int2 e2 = make_int2(-1, -1);
    double2 p2 = make_double2(0.0, 0.0);
    double g2 = 0.0;
    if (k - 2 >= lo) {
      const int64_t o2 = o - 64;
      e2 = s_tape.idx[o2];
      p2 = s_tape.par[o2];
      g2 = s_tape.adj[o2];
    }
    double& wk = win_at(k);
    const double g = wk + g0;
    wk = 0.0;                                  // the slot now holds entry k - SWEEP_WIN
    s_tape.adj[o] = g;
    if (e0.x == MARK_BAND) {
      band_node_reverse(*s_band[threadIdx.x], k);
    } else if (g != 0.0) {
      if (e0.x >= 0) sweep_add(e0.x, k, p0.x * g);
      if (e0.y >= 0) sweep_add(e0.y, k, p0.y * g);
    }
    e0 = e1; p0 = p1; g0 = g1;
    e1 = e2; p1 = p2; g1 = g2;
  }
  for (int m = lo - 1; m > lo - SWEEP_WIN && m >= 0; m--) {
    double& wm = win_at(m);
    s_tape.adj[tape_off(m)] += wm;
    wm = 0.0;
  }
}

__device__ __forceinline__ double& sub_at(int sidx, int j) {
  const int64_t slot = vjp_slot();
  return s_tape.sub[((slot >> 5) * ((int64_t)s_tape.maxsub * SUB_REC) + (int64_t)sidx * SUB_REC + j) * 32 +
                    (slot & 31)];
}

__global__ void __launch_bounds__(VJP_BLOCK)
k_column_step_vjp(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, clmgb_swm_config cfg,
                  double dtime, int snow_method, double* t_ssbef, double* t_h2osfc_bef, clmgb_step_adjoint adj,
                  TapeView tape, uint32_t* col_status, uint32_t* dev_status, unsigned int* max_entries) {
  if (threadIdx.x == 0) s_tape = tape;
  __syncthreads();
  const int64_t ld = D.ldc;
  const int nlevsno = D.nlevsno, nlevgrnd = D.nlevgrnd, nlevsoi = D.nlevsoi;
  const int nlev = nlevsno + D.nlevmax;
  const int nw = nlevsno + nlevgrnd;
  const int64_t nslots = (int64_t)gridDim.x * VJP_BLOCK;
  BandNode bnode;
  s_band[threadIdx.x] = &bnode;
  for (int64_t c = vjp_slot(); c < nc; c += nslots) {
    const bool do_t = ft.mask_nolakec[c] != 0, do_w = fw.mask_hydrology[c] != 0;
    if (!do_t && !do_w) continue;    // the step leaves the column alone: identity
    s_cur[threadIdx.x] = 0;
    s_ovf[threadIdx.x] = 0;
    uint32_t st = 0;
    const int64_t snl = ft.col_snl[c];
    if (snl > 0 || snl < -nlevsno) {
      st = CLMGB_COL_LEVEL_RANGE;
    } else {
      const int jjtop = (int)snl + 1 + nlevsno;
      const int joff = nlevsno;
      if (ft.frac_h2osfc[c] > 0.0 || ft.h2osno_no_layers[c] > 0.0) st |= CLMGB_COL_ADJ_UNSUPPORTED;
      for (int j = 1; j <= nlevgrnd; j++)
        if (LV(ft.excess_ice, c, j, ld) != 0.0) st |= CLMGB_COL_ADJ_UNSUPPORTED;
      // ---- load the state; register the inputs in a fixed order ----
      AdState X;
      for (int jj = 1; jj <= nlev; jj++) {
        const double v = LV(ft.t_soisno, c, jj, ld);
        X.t[jj] = jj >= jjtop ? ad_input(v) : AD(v);
      }
      for (int jj = 1; jj <= nlev; jj++) {
        const double v = LV(ft.h2osoi_liq, c, jj, ld);
        X.liq[jj] = (jj >= jjtop && jj <= nw) ? ad_input(v) : AD(v);
      }
      for (int jj = 1; jj <= nlev; jj++) {
        const double v = LV(ft.h2osoi_ice, c, jj, ld);
        X.ice[jj] = (jj >= jjtop && jj <= nw) ? ad_input(v) : AD(v);
      }
      X.tg = ad_input(ft.t_grnd[c]);
      X.th = ad_input(ft.t_h2osfc[c]);
      X.forc = ad_input(ft.forc_lwrad[c]);
      for (int j = 1; j <= nlevgrnd; j++) {
        const double v = LV(fw.watsat, c, j, ld);
        X.watsat[j] = j <= nlevsoi ? ad_input(v) : AD(v);
      }
      for (int j = 1; j <= nlevgrnd; j++) {
        const double v = LV(fw.bsw, c, j, ld);
        X.bsw[j] = j <= nlevsoi ? ad_input(v) : AD(v);
      }
      for (int j = 1; j <= nlevgrnd; j++) {
        const double v = LV(fw.sucsat, c, j, ld);
        X.sucsat[j] = j <= nlevsoi ? ad_input(v) : AD(v);
      }
      for (int j = 1; j <= nlevsoi; j++) X.hksat[j] = ad_input(LV(fw.hksat, c, j, ld));
      for (int jj = 1; jj <= nw; jj++) X.fact[jj] = AD(LV(ft.fact, c, jj, ld));
      for (int j = 1; j <= nlevsoi; j++) X.icefrac[j] = AD(LV(fw.icefrac, c, j, ld));
      X.qc = AD(fw.qcharge[c]);
      // input indices follow from the registration order
      const int nT = nlev - jjtop + 1, nW = nw - jjtop + 1;
      const int kT = 0, kL = nT, kI = nT + nW, kTg = nT + 2 * nW, kTh = kTg + 1, kF = kTh + 1, kP = kF + 1;
      const int nin = kP + 4 * nlevsoi;

      // ---- soil_temperature! and set_soil_water_fractions!, recorded ----
      if (do_t) {
        if (t_ssbef)
          for (int jj = 1; jj <= nlev; jj++) LV(t_ssbef, c, jj, ld) = X.t[jj].v;
        if (t_h2osfc_bef) t_h2osfc_bef[c] = X.th.v;
        st |= soil_temperature_col(D, ft, c, dtime, snow_method, X);
      }
      // ---- soil_water!: impedances recorded, the substep loop run on values with the
      //      state at the start of every accepted substep kept for the reverse pass ----
      MfLaneT<AD> LA;
      bool rich = false;
      int nacc = 0;
      double smp_save[MAXSOI + 1], hk_save[MAXSOI + 1];
      if (do_w) {
        water_fractions_col(D, fw, c, X);
        rich = mf_begin(LA, D, fw, cfg, dtime, c, X);
        if (!rich) {
          st |= LA.status;
        } else {
          MfLane L;
          L.c = c;
          L.nlayers = LA.nlayers;
          L.status = 0;
          L.nsub = 0;
          L.dtsub = dtime;
          L.dtdone = 0.0;
          L.qc = 0.0;
          L.fresh = true;
          L.dt_cur = -1.0;
          for (int j = 1; j <= LA.nlayers; j++) {
            L.liq[j] = LA.liq[j].v;
            L.dzv[j] = LA.dzv[j];
            L.imp[j] = LA.imp[j].v;
          }
          const AdValues XV{X};
          bool done = false;
          while (!done) {
            if (L.fresh && nacc < s_tape.maxsub)
              for (int j = 1; j <= L.nlayers; j++) sub_at(nacc, j - 1) = L.liq[j];
            const double dts = L.dtsub, dtd = L.dtdone;
            done = mf_attempt(L, D, fw, cfg, dtime, XV);
            if (L.dtdone != dtd) {     // accepted
              if (nacc < s_tape.maxsub) {
                sub_at(nacc, MAXSOI) = dts;
                sub_at(nacc, MAXSOI + 1) = dtd;
              }
              nacc++;
            }
          }
          uint32_t rs = L.status;
          for (int j = 1; j <= L.nlayers; j++) {
            X.liq[joff + j] = AD(L.liq[j]);
            if (!isfinite(L.liq[j])) rs |= CLMGB_COL_NONFINITE;
            smp_save[j] = LV(fw.smp_l, c, j, ld);
            hk_save[j] = LV(fw.hk_l, c, j, ld);
          }
          X.qc = AD(L.qc);
          fw.num_substeps[c] = (double)L.nsub;
          st |= rs;
          if (nacc > s_tape.maxsub) st |= CLMGB_COL_TAPE_FULL;
        }
      }
      // ---- the final forward state, as the production step leaves it ----
      for (int jj = jjtop; jj <= nlev; jj++) LV(ft.t_soisno, c, jj, ld) = X.t[jj].v;
      for (int jj = jjtop; jj <= nw; jj++) {
        LV(ft.h2osoi_liq, c, jj, ld) = X.liq[jj].v;
        LV(ft.h2osoi_ice, c, jj, ld) = X.ice[jj].v;
        if (do_t) LV(ft.fact, c, jj, ld) = X.fact[jj].v;
      }
      if (do_w)
        for (int j = 1; j <= nlevsoi; j++) LV(fw.icefrac, c, j, ld) = X.icefrac[j].v;
      ft.t_grnd[c] = X.tg.v;
      ft.t_h2osfc[c] = X.th.v;
      if (do_w) fw.qcharge[c] = X.qc.v;

      unsigned int used = (unsigned int)s_cur[threadIdx.x];
      if (s_ovf[threadIdx.x]) st |= CLMGB_COL_TAPE_FULL;
      if (!(st & CLMGB_COL_TAPE_FULL)) {
        const int nphase1 = s_cur[threadIdx.x];
        // ---- seed with the adjoints of the step's outputs (the Richards outputs
        //      are seeded in its own reverse below) ----
        const int rlo = rich ? joff + 1 : 1, rhi = rich ? joff + LA.nlayers : 0;
        for (int jj = jjtop; jj <= nlev; jj++) adj_add(X.t[jj].i, LV(adj.lam_t_soisno, c, jj, ld));
        for (int jj = jjtop; jj <= nw; jj++) {
          if (jj < rlo || jj > rhi) adj_add(X.liq[jj].i, LV(adj.lam_h2osoi_liq, c, jj, ld));
          adj_add(X.ice[jj].i, LV(adj.lam_h2osoi_ice, c, jj, ld));
        }
        adj_add(X.tg.i, adj.lam_t_grnd[c]);
        adj_add(X.th.i, adj.lam_t_h2osfc[c]);
        // ---- the substep loop in reverse: replay each accepted substep from its
        //      checkpoint, recorded, sweep it, rewind ----
        if (rich) {
          double lamL[MAXSOI + 1];
          for (int j = 1; j <= LA.nlayers; j++) lamL[j] = LV(adj.lam_h2osoi_liq, c, joff + j, ld);
          const double lamQ = adj.lam_qcharge && !qcharge_replaced(D, fw, cfg, c) ? adj.lam_qcharge[c] : 0.0;
          if (s_tape.richards_mode == CLMGB_ADJ_RICHARDS_CLOSED_FORM) {
            RichardsBar RB;
            double impv[MAXSOI + 1], liqs[MAXSOI + 1];
            double wsv[MAXSOI + 2], bbv[MAXSOI + 2], sucv[MAXSOI + 2], ksv[MAXSOI + 2];
            for (int j = 1; j <= LA.nlayers; j++) {
              RB.ws[j] = 0.0; RB.b[j] = 0.0; RB.suc[j] = 0.0; RB.ks[j] = 0.0; RB.imp[j] = 0.0;
              impv[j] = LA.imp[j].v;
              wsv[j] = X.watsat[j].v;
              bbv[j] = X.bsw[j].v;
              sucv[j] = X.sucsat[j].v;
              ksv[j] = X.hksat[j].v;
            }
            for (int sidx = nacc - 1; sidx >= 0; sidx--) {
              for (int j = 1; j <= LA.nlayers; j++) liqs[j] = sub_at(sidx, j - 1);
              mf_substep_reverse(D, fw, cfg, dtime, c, LA.nlayers, LA.dzv, impv, wsv, bbv, sucv, ksv,
                                 sub_at(sidx, MAXSOI), liqs, lamL, lamQ, RB);
            }
            for (int j = 1; j <= LA.nlayers; j++) {
              adj_add(X.watsat[j].i, RB.ws[j]);
              adj_add(X.bsw[j].i, RB.b[j]);
              adj_add(X.sucsat[j].i, RB.suc[j]);
              adj_add(X.hksat[j].i, RB.ks[j]);
              adj_add(LA.imp[j].i, RB.imp[j]);
            }
          } else {
            for (int sidx = nacc - 1; sidx >= 0; sidx--) {
              const int mark = s_cur[threadIdx.x];
              MfLaneT<AD> R;
              R.c = c;
              R.nlayers = LA.nlayers;
              R.status = 0;
              R.nsub = 0;
              R.fresh = true;
              R.dt_cur = -1.0;
              R.dtsub = sub_at(sidx, MAXSOI);
              R.dtdone = sub_at(sidx, MAXSOI + 1);
              R.qc = AD(0.0);
              for (int j = 1; j <= R.nlayers; j++) {
                R.liq[j] = ad_input(sub_at(sidx, j - 1));
                R.dzv[j] = LA.dzv[j];
                R.imp[j] = LA.imp[j];
              }
              const double dtd0 = R.dtdone;
              mf_attempt(R, D, fw, cfg, dtime, X);
              if (R.dtdone == dtd0) st |= CLMGB_COL_ADJ_REPLAY;
              if (s_ovf[threadIdx.x]) {
                st |= CLMGB_COL_TAPE_FULL;
                break;
              }
              used = max(used, (unsigned int)s_cur[threadIdx.x]);
              for (int j = 1; j <= R.nlayers; j++) adj_add(R.liq[j].i, lamL[j]);
              adj_add(R.qc.i, lamQ);
              sweep(s_cur[threadIdx.x] - 1, mark + R.nlayers);
              for (int j = 1; j <= R.nlayers; j++) lamL[j] = adj_get(mark + j - 1);
              s_cur[threadIdx.x] = mark;
            }
          }
          for (int j = 1; j <= LA.nlayers; j++) {
            adj_add(LA.liq[j].i, lamL[j]);
            LV(fw.smp_l, c, j, ld) = smp_save[j];
            LV(fw.hk_l, c, j, ld) = hk_save[j];
          }
        }
        if (!(st & CLMGB_COL_TAPE_FULL)) {
          // ---- reverse sweep of soil temperature, fractions and impedances ----
          sweep(nphase1 - 1, nin);
          // ---- adjoints of the step's inputs ----
          for (int jj = jjtop; jj <= nlev; jj++) LV(adj.lam_t_soisno, c, jj, ld) = adj_get(kT + jj - jjtop);
          for (int jj = jjtop; jj <= nw; jj++) {
            LV(adj.lam_h2osoi_liq, c, jj, ld) = adj_get(kL + jj - jjtop);
            LV(adj.lam_h2osoi_ice, c, jj, ld) = adj_get(kI + jj - jjtop);
          }
          adj.lam_t_grnd[c] = adj_get(kTg);
          adj.lam_t_h2osfc[c] = adj_get(kTh);
          if (adj.lam_forc_lwrad) adj.lam_forc_lwrad[c] = adj_get(kF);
          for (int j = 1; j <= nlevsoi; j++) {
            if (adj.grad_watsat) LV(adj.grad_watsat, c, j, ld) += adj_get(kP + j - 1);
            if (adj.grad_bsw) LV(adj.grad_bsw, c, j, ld) += adj_get(kP + nlevsoi + j - 1);
            if (adj.grad_sucsat) LV(adj.grad_sucsat, c, j, ld) += adj_get(kP + 2 * nlevsoi + j - 1);
            if (adj.grad_hksat) LV(adj.grad_hksat, c, j, ld) += adj_get(kP + 3 * nlevsoi + j - 1);
          }
        }
      }
      if (max_entries) atomicMax(max_entries, used);
    }
    if (col_status) col_status[c] = st;
    if (st && dev_status) atomicOr(dev_status, st);
  }
}

cudaError_t launch_column_step_vjp(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                   const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                                   int snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                   const clmgb_step_adjoint& adj, const AdjTape& tp, uint32_t* col_status,
                                   uint32_t* dev_status, cudaStream_t s) {
  TapeView tv{tp.idx, tp.par, tp.adj, tp.sub, tp.slots, (int)tp.entries, (int)tp.maxsub, tp.richards_mode};
  int64_t blocks = (nc + VJP_BLOCK - 1) / VJP_BLOCK;
  const int64_t max_blocks = tp.slots / VJP_BLOCK;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) return cudaErrorInvalidValue;
  k_column_step_vjp<<<(unsigned int)blocks, VJP_BLOCK, 0, s>>>(D, nc, ft, fw, cfg, dtime, snow_method, t_ssbef,
                                                               t_h2osfc_bef, adj, tv, col_status, dev_status,
                                                               tp.max_used);
  return cudaGetLastError();
}

}  // namespace clmgb
