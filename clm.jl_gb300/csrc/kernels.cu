// kernels.cu — CUDA kernels of the soil/snow column solve (one thread per column).
#include "clmgb_device.cuh"
#include "launch.h"
#include "richards_coop.cuh"

namespace clmgb {

constexpr int BLOCK = 128;

static inline unsigned grid_for(int64_t n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }

__device__ __forceinline__ void report(uint32_t st, uint32_t* col_status, uint32_t* dev_status, int64_t c) {
  if (col_status) col_status[c] = st;
  if (st && dev_status) atomicOr(dev_status, st);
}

// The column of this thread in the soil-temperature kernels: the block's NB
// consecutive columns, reordered by snow-layer count (a counting sort in shared
// memory), so the lanes of a warp run level loops and band solves of about the same
// length.  Accesses stay inside the block's columns; each column's arithmetic is
// unchanged, so results do not depend on the order.  Every thread of the block must
// call it; returns -1 past the last column.
template <int NB>
__device__ __forceinline__ int64_t snl_sorted_column(int64_t nc, const int64_t* col_snl, int nlevsno) {
  __shared__ unsigned int s_cnt[16];
  __shared__ unsigned short s_perm[NB];
  const int64_t base = (int64_t)blockIdx.x * NB;
  if (threadIdx.x < 16) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t c0 = base + threadIdx.x;
  int key = 15;
  if (c0 < nc) {
    const int64_t s = -col_snl[c0];
    key = (s < 0 || s > nlevsno || s > 13) ? 14 : (int)s;
  }
  const unsigned int r = atomicAdd(&s_cnt[key], 1u);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int run = 0;
    for (int k = 0; k < 16; k++) {
      const unsigned int t = s_cnt[k];
      s_cnt[k] = run;
      run += t;
    }
  }
  __syncthreads();
  s_perm[s_cnt[key] + r] = (unsigned short)threadIdx.x;
  __syncthreads();
  const int64_t c = base + s_perm[threadIdx.x];
  return c < nc ? c : -1;
}

// NB threads per block, sorted together; 640 / NB resident blocks (20 warps per SM)
template <int NB>
__global__ void __launch_bounds__(NB, 640 / NB)
k_soil_temperature(Dims D, int64_t nc, clmgb_soiltemp_fields f, double dtime, int snow_method,
                   uint32_t* col_status, uint32_t* dev_status) {
  const int64_t c = snl_sorted_column<NB>(nc, f.col_snl, D.nlevsno);
  if (c < 0) return;
  uint32_t st = 0;
  if (f.mask_nolakec[c]) st = soil_temperature_col(D, f, c, dtime, snow_method);
  report(st, col_status, dev_status, c);
}

__global__ void __launch_bounds__(BLOCK)
k_water_fractions(Dims D, int64_t nc, clmgb_soilwater_fields f) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc) return;
  if (f.mask_hydrology[c]) water_fractions_col(D, f, c);
}

__global__ void __launch_bounds__(BLOCK)
k_moisture_form(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                uint32_t* col_status, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc) return;
  uint32_t st = 0;
  if (f.mask_hydrology[c]) st = moisture_form_col(D, f, cfg, dtime, c);
  report(st, col_status, dev_status, c);
}

// soil_temperature! -> set_soil_water_fractions! -> soil_water! for one column, one launch.
__global__ void __launch_bounds__(BLOCK)
k_column_step(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, clmgb_swm_config cfg,
              double dtime, int snow_method, double* t_ssbef, double* t_h2osfc_bef,
              uint32_t* col_status, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc) return;
  uint32_t st = 0;
  if (ft.mask_nolakec[c]) {
    if (t_ssbef) {
      const int L = D.nlevsno + D.nlevmax;
      for (int jj = 1; jj <= L; jj++) LV(t_ssbef, c, jj, D.ldc) = LV(ft.t_soisno, c, jj, D.ldc);
    }
    if (t_h2osfc_bef) t_h2osfc_bef[c] = ft.t_h2osfc[c];
    st |= soil_temperature_col(D, ft, c, dtime, snow_method);
  }
  if (fw.mask_hydrology[c]) {
    water_fractions_col(D, fw, c);
    st |= moisture_form_col(D, fw, cfg, dtime, c);
  }
  report(st, col_status, dev_status, c);
}

// The production state accessor whose band solve also keeps the factorisation in the
// column's soil_temperature! record (StLog); the solution is band_lu_solve's bits.
struct FieldStateStLog : FieldState<clmgb_soiltemp_fields> {
  double* rec;
  __device__ __forceinline__ FieldStateStLog(const clmgb_soiltemp_fields& ff, int64_t cc, int64_t l, double* r)
      : FieldState<clmgb_soiltemp_fields>(ff, cc, l), rec(r) {}
  __device__ __forceinline__ void band_solve(double* ab, double* x, int n) const {
    uint8_t piv[MAXROWS];
    band_lu_factor_solve<2, 2>(ab, x, piv, n);
    rec[ST_N] = (double)n;
    for (int k = 0; k < n * 7; k++) rec[ST_LU + k] = ab[k];
    for (int r = 0; r < n; r++) rec[ST_X + r] = x[r];
    uint8_t* pv = reinterpret_cast<uint8_t*>(rec + ST_PIV);
    for (int r = 0; r < n; r++) pv[r] = piv[r];
  }
};

// soil_temperature! then set_soil_water_fractions! for one column per thread (the
// first half of a column step; the Richards solve follows in k_moisture_form_queue).
// With LOG every column soil_temperature! runs on also gets its record in st_log.
template <bool LOG, int NB>
__global__ void __launch_bounds__(NB, 640 / NB)
k_soil_temperature_fractions(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw,
                             double dtime, int snow_method, double* t_ssbef, double* t_h2osfc_bef,
                             uint32_t* col_status, uint32_t* dev_status, double* st_log) {
  const int64_t c = snl_sorted_column<NB>(nc, ft.col_snl, D.nlevsno);
  if (c < 0) return;
  uint32_t st = 0;
  if (ft.mask_nolakec[c]) {
    if (t_ssbef) {
      const int L = D.nlevsno + D.nlevmax;
      for (int jj = 1; jj <= L; jj++) LV(t_ssbef, c, jj, D.ldc) = LV(ft.t_soisno, c, jj, D.ldc);
    }
    if (t_h2osfc_bef) t_h2osfc_bef[c] = ft.t_h2osfc[c];
    if (LOG) {
      double* rec = st_log + c * (int64_t)CLMGB_LOG_ST_STRIDE;
      rec[ST_N] = 0.0;
      FieldStateStLog X(ft, c, D.ldc, rec);
      const uint32_t s1 = soil_temperature_col(D, ft, c, dtime, snow_method, X);
      st |= s1;
      rec[ST_STATUS] = (double)s1;
      const int64_t snl = ft.col_snl[c];
      if (snl <= 0 && snl >= -D.nlevsno) {     // the levels the call may have changed
        const int jjtop = (int)snl + 1 + D.nlevsno;
        const int nw = D.nlevsno + D.nlevgrnd, nlev = D.nlevsno + D.nlevmax;
        for (int jj = jjtop; jj <= nlev; jj++) rec[ST_T + jj - 1] = LV(ft.t_soisno, c, jj, D.ldc);
        for (int jj = jjtop; jj <= nw; jj++) {
          rec[ST_LIQ + jj - 1] = LV(ft.h2osoi_liq, c, jj, D.ldc);
          rec[ST_ICE + jj - 1] = LV(ft.h2osoi_ice, c, jj, D.ldc);
          rec[ST_FACT + jj - 1] = LV(ft.fact, c, jj, D.ldc);
        }
      }
      rec[ST_TG] = ft.t_grnd[c];
      rec[ST_TH] = ft.t_h2osfc[c];
    } else {
      st |= soil_temperature_col(D, ft, c, dtime, snow_method);
    }
  }
  if (fw.mask_hydrology[c]) water_fractions_col(D, fw, c);
  report(st, col_status, dev_status, c);
}

// soilwm_moisture_form_solve! as a persistent kernel fed by a device work queue.
// Each lane owns one column at a time and advances it one substep attempt per loop
// trip; when its column finishes it takes the next column index from the queue
// (one atomicAdd per warp for all lanes that need work).  Columns need from 1 to
// ~70 attempts, so lanes stay busy instead of waiting for the slowest column of
// the warp.  With `order` the queue hands out columns in that order (longest
// expected first) and the impedances come precomputed in imp_cache.  The
// per-column arithmetic is unchanged, so results do not depend on the schedule.
// `queue` must be zero at launch.
// With LOG the kernel also writes the substep log of every column it solves (the
// starting water of each accepted substep and the solve's outputs), for the step
// adjoint; the solve itself is unchanged.
// With qs.defer > 0 (never with LOG) a column that has made qs.defer attempts and
// is not done leaves the lane at its next accepted substep: the lane stores the
// column's state and takes new work, and warps that run out of queued columns
// finish the deferred ones one warp per column (coop_drain, richards_coop.cuh), so
// the few columns that need several times the mean number of attempts no longer
// hold the kernel's end with one useful lane per warp.
template <bool LOG>
__global__ void __launch_bounds__(BLOCK)
k_moisture_form_queue(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                      uint32_t* col_status, int or_status, uint32_t* dev_status, unsigned long long* queue,
                      const uint32_t* order, const unsigned int* nlisted_ptr, const double* imp_cache,
                      int64_t ld_imp, const double* dt_init, SubstepLogView lg, int fresh_batch, QueueScratch qs) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned long long nq = order ? (unsigned long long)(*(volatile const unsigned int*)nlisted_ptr)
                                      : (unsigned long long)nc;
  MfLane L;
  int nacc = 0;
  bool active = false, exhausted = false, kept = false;
  for (;;) {
    const bool need = !active && !exhausted;
    const unsigned m = __ballot_sync(FULL, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        const unsigned long long k = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
        if (k >= nq) {
          exhausted = true;
        } else {
          const int64_t c = order ? (int64_t)order[k] : (int64_t)k;
          if (order || f.mask_hydrology[c]) {
            if (mf_begin(L, D, f, cfg, dtime, c, imp_cache, ld_imp, dt_init)) {
              active = true;
              nacc = 0;
              kept = false;
            } else {
              const uint32_t st = L.status;
              if (col_status) col_status[c] = or_status ? (col_status[c] | st) : st;
              if (st && dev_status) atomicOr(dev_status, st);
            }
          } else if (col_status && !or_status) {
            col_status[c] = 0;
          }
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (__all_sync(FULL, exhausted)) {
        // no queued column left for this warp: finish deferred ones, one warp each
        if (!LOG && qs.defer > 0) coop_drain(D, f, cfg, dtime, col_status, or_status, dev_status, qs);
        break;
      }
      continue;
    }
    // Batched refresh.  A lane whose substep was just accepted needs the hydraulic
    // block (mf_refresh, about 2.7 attempts' worth of FP64 work) before its next
    // attempt.  Run at once, it idles the other lanes of the warp; with
    // fresh_batch > 0 such lanes wait while the others attempt, until fresh_batch of
    // them need it or no lane can attempt, and then run it together.  Each column's
    // operations and their order are unchanged.
    bool can_try = active;
    if (fresh_batch > 0) {
      const bool want = active && L.fresh && L.nsub < D.attempt_cap;
      const unsigned wm = __ballot_sync(FULL, want);
      const unsigned tm = __ballot_sync(FULL, active && !want);
      if (wm && (__popc(wm) >= fresh_batch || tm == 0) && want) {
        if (LOG && nacc < lg.cap) {
          double* r0 = lg.rec + L.c * lg.stride + (int64_t)nacc * SUB_REC;
          for (int j = 1; j <= L.nlayers; j++) r0[j - 1] = L.liq[j];
        }
        FieldState<clmgb_soilwater_fields> X(f, L.c, D.ldc);
        mf_refresh(L, D, f, cfg, X);
      }
      can_try = active && !(L.fresh && L.nsub < D.attempt_cap);
    }
    if (!can_try) continue;
    double* rec = nullptr;
    double dts = 0.0, dtd = 0.0;
    if (LOG) {
      rec = lg.rec + L.c * lg.stride;
      if (L.fresh && nacc < lg.cap)
        for (int j = 1; j <= L.nlayers; j++) rec[(int64_t)nacc * SUB_REC + j - 1] = L.liq[j];
      dts = L.dtsub;
      dtd = L.dtdone;
    }
    const bool fin = mf_attempt(L, D, f, cfg, dtime);
    if (LOG && L.dtdone != dtd) {
      if (nacc < lg.cap) {
        rec[(int64_t)nacc * SUB_REC + MAXSOI] = dts;
        rec[(int64_t)nacc * SUB_REC + MAXSOI + 1] = dtd;
      }
      nacc++;
    }
    if (!LOG && !fin && qs.defer > 0 && L.fresh && L.nsub >= qs.defer && !kept) {
      // hand the column over; a slot the drain gave back leaves it with this lane
      if (coop_defer(L, qs)) {
        active = false;
        continue;
      }
      kept = true;
    }
    if (fin) {
      const uint32_t st = mf_end(L, D, f);
      if (LOG) {
        double* out = rec + (int64_t)lg.cap * SUB_REC;
        for (int j = 1; j <= L.nlayers; j++) {
          out[j - 1] = L.liq[j];
          out[MAXSOI + j - 1] = LV(f.smp_l, L.c, j, D.ldc);
          out[2 * MAXSOI + j - 1] = LV(f.hk_l, L.c, j, D.ldc);
        }
        out[3 * MAXSOI] = L.qc;
        out[3 * MAXSOI + 1] = (double)L.nsub;
        out[3 * MAXSOI + 2] = (double)st;
        lg.count[L.c] = nacc;
      }
      if (col_status) col_status[L.c] = or_status ? (col_status[L.c] | st) : st;
      if (st && dev_status) atomicOr(dev_status, st);
      active = false;
    }
  }
}

// ---------------------------------------------------------------------------
// The work-queue kernel with a packed hydraulic refresh.  A refresh (the hydraulic
// properties, fluxes and flux derivatives of an accepted substep's water, mf_refresh)
// costs about three attempts and runs for the lanes whose substep was just accepted;
// run lane by lane it leaves the warp's other lanes idle.  Here the warp runs the
// refresh of all its fresh lanes' columns together: the (column, level) pairs are
// spread over the 32 lanes, in four passes over the levels (saturation, hydraulic
// properties, fluxes, net flux), each reading what the pass before wrote.  The
// arrays other lanes read or write live in the warp's shared memory, laid out
// [array][level][lane]; within a pass every lane reads its inputs, the warp syncs,
// then the lanes write, so no level is overwritten before its neighbour has read it.
// Every value is formed by mf_refresh's expression and the attempts are mf_attempt,
// so the results are the per-lane kernel's bits.

// level j (1-based) of one lane's array in the warp's shared memory
struct LevelView {
  double* p;
  __device__ __forceinline__ double& operator[](int j) const { return p[(j - 1) * 32]; }
};

struct MfLaneP {
  static constexpr bool kRefreshInline = false;   // refreshed by mfp_refresh
  static constexpr bool kDzw = true;              // dzv holds 1000*dz (the record's PC_DZW)
  int64_t c;
  int nlayers;
  int nsub;
  bool fresh;
  uint32_t status;
  double dtsub, dtdone, dt_cur;
  double qc, qin1, hk_bot, dhkdw_bot;
  double dzv[MAXSOI + 1], dt_dz[MAXSOI + 1];
  double liq[MAXSOI + 1], gam[MAXSOI + 1], dwat[MAXSOI + 1];
  LevelView qout, dqodw1, dqodw2, fnet1;
};

// mf_end's destination in the packed kernel: the column's water goes to its record
// (the post-pass k_column_outputs moves it to the state), qcharge to the state
struct RecordOut {
  double* rec;
  int joff, nls;
  double* qc;
  __device__ __forceinline__ double& Liq(int jj) const { return rec[PC_LIQ * nls + (jj - joff) - 1]; }
  __device__ __forceinline__ double& Qcharge() const { return *qc; }
};

// shared-memory doubles per warp: 4 level arrays and the bottom conductivity pair
__host__ __device__ constexpr int64_t packed_warp_doubles(int nlevsoi) { return (4LL * nlevsoi + 2) * 32; }
// threads per block of k_moisture_form_packed: 5 warps at 21 KB of shared memory each
// (20 levels) put 2 blocks, 10 warps, on an SM
constexpr int PBLOCK = 160;

// mf_begin for the packed lane (the impedances stay in the cache the refresh reads;
// the water and 1000*dz come from the column's record)
__device__ __forceinline__ bool mfp_begin(MfLaneP& L, const Dims& D, const clmgb_soilwater_fields& f,
                                          const clmgb_swm_config& cfg, double dtime, int64_t c,
                                          const double* dt_init, const double* pcache) {
  const int nls = D.nlevsoi;
  L.c = c;
  L.status = 0;
  const int64_t nl = f.col_nbedrock[c];
  if (nl < 1 || nl > D.nlevsoi) {
    L.status = CLMGB_COL_LEVEL_RANGE;
    return false;
  }
  const int nlayers = (int)nl;
  L.nlayers = nlayers;
  const double* rec = pcache + c * (int64_t)(PC_ALL * nls);
  for (int j = 1; j <= nlayers; j++) {
    L.liq[j] = rec[PC_LIQ * nls + j - 1];
    L.dzv[j] = rec[PC_DZW * nls + j - 1];
  }
  L.nsub = 0;
  L.dtsub = dtime;
  if (dt_init) {
    const double d = dt_init[c];
    if (d == d) L.dtsub = jl_min(jl_max(d, cfg.dtmin), dtime);   // NaN keeps dtime
  }
  L.dtdone = 0.0;
  L.qc = 0.0;
  L.fresh = true;
  L.dt_cur = -1.0;
  return true;
}

// The refresh of the lanes in `mask`, called by all 32 lanes of the warp.  wsm: the
// warp's shared block; nls: D.nlevsoi; pcache: the columns' input records
// ([column][PC_FIELDS][nls], k_impedance).
__device__ __forceinline__ void mfp_refresh(MfLaneP& L, unsigned mask, const Dims& D,
                                            const clmgb_soilwater_fields& f, const clmgb_swm_config& cfg,
                                            double* pcache, double* wsm, int nls) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1, nlevsoi = D.nlevsoi;
  const int lower_bc = cfg.lower_boundary_condition;
  const bool mine = (mask >> lane) & 1u;
  // (column, level) items: lane k's levels are items off_k .. off_k + nl_k - 1
  const int nl_own = mine ? L.nlayers : 0;
  int incl = nl_own;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += v;
  }
  const int off_own = incl - nl_own;
  const int T = __shfl_sync(FULL, incl, 31);
  const int64_t c_own = mine ? L.c : 0;
  double* const sb = wsm + 4LL * nls * 32;                       // hk, dhkdw of the bottom level
  auto A = [&](int a, int k, int j) -> double& { return wsm[((int64_t)a * nls + (j - 1)) * 32 + k]; };
  // input `fld` of level j of column c
  auto P = [&](int64_t c, int fld, int j) -> double {
    return pcache[c * (int64_t)(PC_ALL * nls) + (int64_t)fld * nls + (j - 1)];
  };
  enum { QOUT = 0, D1 = 1, D2 = 2, FN = 3 };
  struct Item { int k, j, nl; int64_t c; bool ok; };
  auto item = [&](int base) -> Item {
    const int t = base + lane;
    int k = 0;                                     // the last lane whose first item is <= t
    for (int step = 16; step > 0; step >>= 1) {
      const int oc = __shfl_sync(FULL, off_own, k + step);
      if (oc <= t) k += step;
    }
    Item it;
    it.k = k;
    it.c = __shfl_sync(FULL, c_own, k);
    it.nl = __shfl_sync(FULL, nl_own, k);
    it.j = t - __shfl_sync(FULL, off_own, k) + 1;
    it.ok = t < T;
    return it;
  };
  // the refreshed lanes' water (kept in their local memory) into FN, where the other
  // lanes of the warp can read it; their net fluxes there are about to be re-formed
  if (mine)
    for (int j = 1; j <= L.nlayers; j++) A(FN, lane, j) = L.liq[j];
  __syncwarp();
  // pass 1: saturation of every level (:1283-1287), kept in FN
  for (int base = 0; base < T; base += 32) {
    const Item it = item(base);
    if (it.ok) {
      const double vwc = jl_div(jl_max(A(FN, it.k, it.j), 1.0e-6), P(it.c, PC_DZW, it.j));
      double s = jl_div(vwc, P(it.c, PC_WS, it.j));
      s = jl_min(s, 1.0);
      A(FN, it.k, it.j) = jl_max(0.01, s);
    }
  }
  __syncwarp();
  // pass 2: hydraulic properties (:1288-1308): hk, dhkdw, smp, dsmpdw into QOUT, D1, D2, FN
  for (int base = 0; base < T; base += 32) {
    const Item it = item(base);
    double hkv = 0.0, dhkds = 0.0, smpv = 0.0, dsmpdw = 0.0;
    if (it.ok) {
      const int j = it.j;
      const int64_t c = it.c;
      const double sj = A(FN, it.k, j);
      const double sn = (j < it.nl) ? A(FN, it.k, j + 1) : sj;
      double s1 = (j == it.nl) ? sj : 0.5 * (sj + sn);
      s1 = jl_min(s1, 1.0);
      s1 = jl_max(0.01, s1);
      const double b = P(c, PC_BSW, j);
      hkv = P(c, PC_IMP, j) * P(c, PC_KS, j) * cm_pow(s1, 2.0 * b + 3.0);
      dhkds = jl_div((2.0 * b + 3.0) * hkv, s1);
      smpv = -P(c, PC_SUC, j) * cm_pow(sj, -b);
      const double dsmpds = jl_div(-b * smpv, sj);
      dsmpdw = jl_div(dsmpds, P(c, PC_WS, j));
      double* rec = pcache + c * (int64_t)(PC_ALL * nls);
      rec[PC_SMP * nls + j - 1] = smpv;
      rec[PC_HK * nls + j - 1] = hkv;
    }
    __syncwarp();
    if (it.ok) {
      A(QOUT, it.k, it.j) = hkv;
      A(D1, it.k, it.j) = dhkds;
      A(D2, it.k, it.j) = smpv;
      A(FN, it.k, it.j) = dsmpdw;
    }
    __syncwarp();
  }
  // pass 3: fluxes and derivatives between levels (:1310-1345) and at the bottom
  // (:1347-1370), over the properties into QOUT, D1, D2
  for (int base = 0; base < T; base += 32) {
    const Item it = item(base);
    double qo = 0.0, d1 = 0.0, d2 = 0.0;
    if (it.ok) {
      const int j = it.j;
      const int64_t c = it.c;
      const double hk = A(QOUT, it.k, j), dhkdw = A(D1, it.k, j), smp = A(D2, it.k, j), dsmpdw = A(FN, it.k, j);
      if (j < it.nl) {
        const double dhkds1 = jl_div(0.5 * dhkdw, P(c, PC_WS, j));
        const double dhkds2 = jl_div(0.5 * dhkdw, P(c, PC_WS, j + 1));
        const double num = A(D2, it.k, j + 1) - smp;
        const double den = P(c, PC_DEN, j);
        qo = jl_div(-hk * num, den) + hk;
        d1 = jl_div(hk * dsmpdw - dhkds1 * num, den) + dhkds1;
        d2 = jl_div(-hk * A(FN, it.k, j + 1) - dhkds2 * num, den) + dhkds2;
      } else {
        sb[it.k] = hk;
        sb[32 + it.k] = dhkdw;
        if (lower_bc == CLMGB_BC_WATERTABLE) {
          int jwt = nlevsoi;
          for (int jj = 1; jj <= nlevsoi; jj++) {
            if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
          }
          if (j <= jwt) {
            const double dhkds1l = dhkdw / P(c, PC_WS, j);
            const double num = -smp;
            const double den = M_TO_MM * (f.zwt[c] - LVc(f.z, c, joff + j, ld));
            qo = jl_div(-hk * num, den) + hk;
            d1 = (hk * dsmpdw - dhkds1l * num) / den + dhkds1l;
          }
        } else if (lower_bc == CLMGB_BC_FLUX) {
          qo = hk;
          d1 = dhkdw / P(c, PC_WS, j);
        }
      }
    }
    __syncwarp();
    if (it.ok) {
      A(QOUT, it.k, it.j) = qo;
      A(D1, it.k, it.j) = d1;
      A(D2, it.k, it.j) = d2;
    }
    __syncwarp();
  }
  // pass 4: net flux of every level (:1372-1378); the inflow of level j > 1 is the
  // outflow of level j-1
  for (int base = 0; base < T; base += 32) {
    const Item it = item(base);
    if (it.ok) {
      const double qin = (it.j == 1) ? f.qflx_infl[it.c] : A(QOUT, it.k, it.j - 1);
      A(FN, it.k, it.j) = qin - A(QOUT, it.k, it.j) - P(it.c, PC_ROOT, it.j);
    }
  }
  __syncwarp();
  if (mine) {
    L.qin1 = f.qflx_infl[L.c];
    L.hk_bot = sb[lane];
    L.dhkdw_bot = sb[32 + lane];
    L.fresh = false;
  }
  __syncwarp();
}

// k_moisture_form_queue with the packed refresh; reads the column records
// (QueueScratch::pcache) k_column_records (records.cu) wrote before it.  With
// LOG it writes the same substep log (the starting water of each accepted substep,
// its dtsub and the time done before it, then the solve's outputs).  Dynamic shared
// memory: packed_warp_doubles(nlevsoi) doubles per warp.
template <bool LOG>
__global__ void __launch_bounds__(PBLOCK)
k_moisture_form_packed(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                       uint32_t* col_status, int or_status, uint32_t* dev_status, unsigned long long* queue,
                       const uint32_t* order, const unsigned int* nlisted_ptr, const double* dt_init,
                       SubstepLogView lg, int fresh_batch, QueueScratch qs) {
  extern __shared__ double smem_packed[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nls = D.nlevsoi;
  double* const wsm = smem_packed + (int64_t)(threadIdx.x >> 5) * packed_warp_doubles(nls);
  const unsigned long long nq = order ? (unsigned long long)(*(volatile const unsigned int*)nlisted_ptr)
                                      : (unsigned long long)nc;
  const int batch = fresh_batch > 0 ? fresh_batch : 1;
  MfLaneP L;
  L.qout.p = wsm + (0LL * nls) * 32 + lane;
  L.dqodw1.p = wsm + (1LL * nls) * 32 + lane;
  L.dqodw2.p = wsm + (2LL * nls) * 32 + lane;
  L.fnet1.p = wsm + (3LL * nls) * 32 + lane;
  int nacc = 0;
  bool active = false, exhausted = false, kept = false;
  for (;;) {
    const bool need = !active && !exhausted;
    const unsigned m = __ballot_sync(FULL, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        const unsigned long long k = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
        if (k >= nq) {
          exhausted = true;
        } else {
          const int64_t c = order ? (int64_t)order[k] : (int64_t)k;
          if (order || f.mask_hydrology[c]) {
            if (mfp_begin(L, D, f, cfg, dtime, c, dt_init, qs.pcache)) {
              active = true;
              nacc = 0;
              kept = false;
            } else {
              const uint32_t st = L.status;
              if (col_status) col_status[c] = or_status ? (col_status[c] | st) : st;
              if (st && dev_status) atomicOr(dev_status, st);
            }
          } else if (col_status && !or_status) {
            col_status[c] = 0;
          }
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (__all_sync(FULL, exhausted)) {
        if (!LOG && qs.defer > 0) coop_drain(D, f, cfg, dtime, col_status, or_status, dev_status, qs);
        break;
      }
      continue;
    }
    // lanes whose substep was accepted wait for the packed refresh until `batch` of
    // them need it or no lane can attempt
    const bool want = active && L.fresh && L.nsub < D.attempt_cap;
    const unsigned wm = __ballot_sync(FULL, want);
    const unsigned tm = __ballot_sync(FULL, active && !want);
    if (wm && (__popc(wm) >= batch || tm == 0)) {
      if (LOG && want && nacc < lg.cap) {
        double* r0 = lg.rec + L.c * lg.stride + (int64_t)nacc * SUB_REC;
        for (int j = 1; j <= L.nlayers; j++) r0[j - 1] = L.liq[j];
      }
      if (qs.work) {
        const unsigned lv = __reduce_add_sync(FULL, want ? (unsigned)L.nlayers : 0u);
        if (lane == 0) atomicAdd(qs.work + 1, (unsigned long long)lv);
      }
      mfp_refresh(L, wm, D, f, cfg, qs.pcache, wsm, nls);
    }
    const bool can_try = active && !(L.fresh && L.nsub < D.attempt_cap);
    if (qs.work) {
      const unsigned lv = __reduce_add_sync(FULL, can_try ? (unsigned)L.nlayers : 0u);
      if (lane == 0) atomicAdd(qs.work, (unsigned long long)lv);
    }
    if (!can_try) continue;
    double* rec = nullptr;
    double dts = 0.0, dtd = 0.0;
    if (LOG) {
      rec = lg.rec + L.c * lg.stride;
      if (L.fresh && nacc < lg.cap)
        for (int j = 1; j <= L.nlayers; j++) rec[(int64_t)nacc * SUB_REC + j - 1] = L.liq[j];
      dts = L.dtsub;
      dtd = L.dtdone;
    }
    FieldState<clmgb_soilwater_fields> X(f, L.c, D.ldc);
    const bool fin = mf_attempt(L, D, f, cfg, dtime, X);
    if (LOG && L.dtdone != dtd) {
      if (nacc < lg.cap) {
        rec[(int64_t)nacc * SUB_REC + MAXSOI] = dts;
        rec[(int64_t)nacc * SUB_REC + MAXSOI + 1] = dtd;
      }
      nacc++;
    }
    if (!LOG && !fin && qs.defer > 0 && L.fresh && L.nsub >= qs.defer && !kept) {
      // hand the column over; a slot the drain gave back leaves it with this lane
      if (coop_defer(L, qs)) {
        active = false;
        continue;
      }
      kept = true;
    }
    if (fin) {
      RecordOut RO{qs.pcache + L.c * (int64_t)(PC_ALL * nls), D.nlevsno, nls, f.qcharge + L.c};
      const uint32_t st = mf_end(L, D, f, RO);
      if (LOG) {
        double* out = rec + (int64_t)lg.cap * SUB_REC;
        for (int j = 1; j <= L.nlayers; j++) {
          out[j - 1] = L.liq[j];
          out[MAXSOI + j - 1] = RO.rec[PC_SMP * nls + j - 1];
          out[2 * MAXSOI + j - 1] = RO.rec[PC_HK * nls + j - 1];
        }
        out[3 * MAXSOI] = L.qc;
        out[3 * MAXSOI + 1] = (double)L.nsub;
        out[3 * MAXSOI + 2] = (double)st;
        lg.count[L.c] = nacc;
      }
      if (col_status) col_status[L.c] = or_status ? (col_status[L.c] | st) : st;
      if (st && dev_status) atomicOr(dev_status, st);
      active = false;
    }
  }
}

// compute_qcharge! after a moisture-form solve with the water-table lower boundary
// (soil_water_movement.jl:1575-1598): one thread per hydrology column the solve
// could take (nbedrock in range).
__global__ void __launch_bounds__(BLOCK)
k_compute_qcharge(Dims D, int64_t nc, clmgb_soilwater_fields f, double dtime) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_hydrology[c]) return;
  const int64_t nl = f.col_nbedrock[c];
  if (nl < 1 || nl > D.nlevsoi) return;
  compute_qcharge_col(D, f, dtime, c);
}

// The use_flexibleCN branch of soil_water! (soil_water_movement.jl:1812-1843) for one
// column: smooth_ifelse on Float64 is the exact branch x >= 0 ? a : b (smooth_ad.jl:253-257).
__global__ void __launch_bounds__(BLOCK)
k_flexible_cn(Dims D, int64_t nc, clmgb_flexcn_fields f) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_hydrology[c]) return;
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno, nlevsoi = D.nlevsoi;
  const double watmin = 0.001;
  for (int j = 1; j <= nlevsoi - 1; j++) {
    double& lj = LV(f.h2osoi_liq, c, joff + j, ld);
    const double xs = lj >= 0.0 ? 0.0 : watmin - lj;
    lj = lj + xs;
    double& ln = LV(f.h2osoi_liq, c, joff + j + 1, ld);
    ln = ln - xs;
  }
  {
    double& lj = LV(f.h2osoi_liq, c, joff + nlevsoi, ld);
    const double xs = (lj - watmin) >= 0.0 ? 0.0 : watmin - lj;
    lj = lj + xs;
    f.wa[c] = f.wa[c] - xs;
  }
  for (int j = 1; j <= nlevsoi; j++) {
    const double dzv = LVc(f.dz, c, joff + j, ld);
    LV(f.h2osoi_vol, c, j, ld) =
        jl_div(LV(f.h2osoi_liq, c, joff + j, ld), dzv * DENH2O) + jl_div(LVc(f.h2osoi_ice, c, joff + j, ld), dzv * DENICE);
  }
}

// Ice impedances of every hydrology column, one thread per column, into imp_cache
// [nlevsoi][ld_imp] (uniform work: no lane waits on another column).
__global__ void __launch_bounds__(BLOCK)
k_impedance(Dims D, int64_t nc, clmgb_soilwater_fields f, double e_ice, double* imp_cache, int64_t ld_imp) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_hydrology[c]) return;
  const int64_t nl = f.col_nbedrock[c];
  if (nl < 1 || nl > D.nlevsoi) return;
  const int nlayers = (int)nl;
  for (int j = 1; j <= nlayers; j++) imp_cache[(int64_t)(j - 1) * ld_imp + c] = mf_impedance(D, f, e_ice, c, j, nlayers);
}

// Longest-expected-first order of the hydrology columns: counting sort on the
// previous call's substep count (num_substeps, the state field), descending.
// Bins 0..63; NaN or non-positive counts go to bin 0.  The order within a bin is
// arbitrary and does not affect any result.
constexpr int ORDER_BINS = 64;
__device__ __forceinline__ int order_bin(double ns) {
  if (!(ns > 0.0)) return 0;
  return ns >= (double)(ORDER_BINS - 1) ? ORDER_BINS - 1 : (int)ns;
}
__global__ void __launch_bounds__(BLOCK)
k_order_hist(int64_t nc, const uint8_t* mask, const double* num_substeps, unsigned int* bins) {
  __shared__ unsigned int sh[ORDER_BINS];
  for (int i = threadIdx.x; i < ORDER_BINS; i += BLOCK) sh[i] = 0;
  __syncthreads();
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c < nc && mask[c]) atomicAdd(&sh[order_bin(num_substeps[c])], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < ORDER_BINS; i += BLOCK)
    if (sh[i]) atomicAdd(&bins[i], sh[i]);
}
// bins[0..63] counts -> bins[64+b] start offset of bin b (descending bins first),
// bins[128] = total listed
__global__ void k_order_scan(unsigned int* bins) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned int run = 0;
  for (int b = ORDER_BINS - 1; b >= 0; b--) {
    bins[ORDER_BINS + b] = run;
    run += bins[b];
  }
  bins[2 * ORDER_BINS] = run;
}
__global__ void __launch_bounds__(BLOCK)
k_order_scatter(int64_t nc, const uint8_t* mask, const double* num_substeps, unsigned int* bins, uint32_t* order,
                uint32_t* col_status, int or_status) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc) return;
  if (!mask[c]) {
    if (col_status && !or_status) col_status[c] = 0;
    return;
  }
  const unsigned int slot = atomicAdd(&bins[ORDER_BINS + order_bin(num_substeps[c])], 1u);
  order[slot] = (uint32_t)c;
}

// Evaluates the shared transcendentals (clm_math.h) elementwise; op 0 log, 1 exp,
// 2 pow, 3 log10.  Used to check that GPU and CPU builds return identical bits.
__global__ void __launch_bounds__(BLOCK)
k_math_eval(int op, int64_t n, const double* x, const double* y, double* out) {
  const int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= n) return;
  const double a = x[i];
  double r;
  if (op == 0) r = cm_log(a);
  else if (op == 1) r = cm_exp(a);
  else if (op == 2) r = cm_pow(a, y[i]);
  else if (op == 3) r = cm_log10(a);
  else if (op == 4) r = cm_sin(a);
  else if (op == 5) r = cm_acos(a);
  else r = jl_div(a, y[i]);
  out[i] = r;
}

__global__ void __launch_bounds__(BLOCK)
k_phase_change(Dims D, int64_t nc, clmgb_soiltemp_fields f, double dtime, const double* dhsdT, int which) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_nolakec[c]) return;
  if (which == 0) phase_change_h2osfc_col(D, f, c, dtime, dhsdT[c]);
  else phase_change_beta_col(D, f, c, dtime, dhsdT[c]);
}

template <int KL, int KU>
__global__ void __launch_bounds__(BLOCK)
k_band_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* __restrict__ bmatrix,
             const double* __restrict__ rvector, const int64_t* jtop, const int64_t* jbot,
             const uint8_t* mask, int nlevsno_off) {
  constexpr int W = 2 * KL + KU + 1;
  constexpr int NB = KL + KU + 1;
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !mask[c]) return;
  const int64_t jt = jtop[c] + nlevsno_off + 1;
  const int64_t n64 = jbot[c] - jtop[c] + 1;
  if (n64 <= 0 || jt < 1 || jt + n64 - 1 > nlev || n64 > MAXROWS + 1) return;
  const int n = (int)n64;
  double ab[(MAXROWS + 1) * W];
  double x[MAXROWS + 1];
  for (int k = 0; k < n * W; k++) ab[k] = 0.0;
  for (int i = 0; i < n; i++) {
    const int64_t lev = jt + i;   // 1-based level of row i
    for (int j = max(0, i - KL); j <= min(n - 1, i + KU); j++) {
      const int band = (i - j) + KL;   // 0-based band
      ab[i * W + (j - i + KL)] = bmatrix[c + (int64_t)band * ldc + (lev - 1) * ldc * NB];
    }
    x[i] = rvector[c + (lev - 1) * ldc];
  }
  band_lu_solve<KL, KU>(ab, x, n);
  for (int i = 0; i < n; i++) tvector[c + (jt + i - 1) * ldc] = x[i];
}

constexpr int MAXTRI = 64;

__global__ void __launch_bounds__(BLOCK)
k_tridiagonal_multi(int64_t ncols, int64_t ld, int nlevs, double* u, const double* __restrict__ a,
                    const double* __restrict__ b, const double* __restrict__ cc, const double* __restrict__ r,
                    const int64_t* jtop, const uint8_t* mask) {
  const int64_t col = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (col >= ncols || !mask[col]) return;
  const int64_t j64 = jtop[col];
  if (j64 < 1 || j64 > nlevs) return;
  const int j = (int)j64;
  double cpv[MAXTRI + 1], dpv[MAXTRI + 1];
  const double tiny = 1e-30;
  double bet = LVc(b, col, j, ld);
  if (fabs(bet) < tiny) bet = tiny;
  double cp_prev = LVc(cc, col, j, ld) / bet;
  double dp_prev = LVc(r, col, j, ld) / bet;
  cpv[j] = cp_prev;
  dpv[j] = dp_prev;
  for (int jj = j + 1; jj <= nlevs; jj++) {
    double denom = LVc(b, col, jj, ld) - LVc(a, col, jj, ld) * cp_prev;
    if (fabs(denom) < tiny) denom = copysign(tiny, denom == 0.0 ? 1.0 : denom);
    cp_prev = LVc(cc, col, jj, ld) / denom;
    dp_prev = (LVc(r, col, jj, ld) - LVc(a, col, jj, ld) * dp_prev) / denom;
    cpv[jj] = cp_prev;
    dpv[jj] = dp_prev;
  }
  double u_next = dp_prev;
  LV(u, col, nlevs, ld) = u_next;
  for (int jj = nlevs - 1; jj >= j; jj--) {
    u_next = dpv[jj] - cpv[jj] * u_next;
    LV(u, col, jj, ld) = u_next;
  }
}

// The same systems by parallel cyclic reduction, one warp per column (CLMGB_TRIDIAG_PCR):
// lane l holds rows l and l+32 of the column's n = nlevs - jtop + 1 <= 64 unknowns in
// registers.  Each round with stride k eliminates the couplings to rows i-k and i+k
// (rows outside the system act as identity rows), so after ceil(log2 n) rounds every
// row stands alone and x_i = r_i / b_i.  The divisors get the reference's 1e-30
// pivot guard.  Without pivoting it is meant for the diagonally dominant systems of the
// soil-water and lake solves; its rounding differs from the sequential elimination's.
constexpr int PCR_WARPS = 4;
// row t (0..32*NH-1) of a value held as v[h] for rows lane + 32h
template <int NH>
__device__ __forceinline__ double pcr_row(const double* v, int t) {
  const double x0 = __shfl_sync(0xffffffffu, v[0], t & 31);
  if (NH == 1) return x0;
  const double x1 = __shfl_sync(0xffffffffu, v[NH - 1], t & 31);
  return (t >> 5) ? x1 : x0;
}
__device__ __forceinline__ double pcr_guard(double d) {
  return fabs(d) < 1e-30 ? copysign(1e-30, d == 0.0 ? 1.0 : d) : d;
}
// the system of one column, n <= 32*NH unknowns, rows lane + 32h of this lane
template <int NH>
__device__ __forceinline__ void pcr_solve(int64_t col, int64_t ld, int j0, int n, double* u,
                                          const double* __restrict__ a, const double* __restrict__ b,
                                          const double* __restrict__ cc, const double* __restrict__ r) {
  const int lane = threadIdx.x & 31;
  double A[NH], B[NH], C[NH], R[NH];
#pragma unroll
  for (int h = 0; h < NH; h++) {
    const int i = lane + 32 * h;
    if (i < n) {
      const int lev = j0 + i;
      A[h] = i == 0 ? 0.0 : LVc(a, col, lev, ld);
      B[h] = LVc(b, col, lev, ld);
      C[h] = i == n - 1 ? 0.0 : LVc(cc, col, lev, ld);
      R[h] = LVc(r, col, lev, ld);
    } else {
      A[h] = 0.0; B[h] = 1.0; C[h] = 0.0; R[h] = 0.0;
    }
  }
  for (int k = 1; k < n; k <<= 1) {
    double An[NH], Bn[NH], Cn[NH], Rn[NH];
#pragma unroll
    for (int h = 0; h < NH; h++) {
      const int i = lane + 32 * h;
      const int lo = i - k, hi = i + k;
      // rows i-k and i+k (identity rows outside 0..n-1); every lane joins every shuffle
      const int tl = lo < 0 ? 0 : lo, th = hi > 32 * NH - 1 ? 32 * NH - 1 : hi;
      double al = pcr_row<NH>(A, tl), bl = pcr_row<NH>(B, tl), cl = pcr_row<NH>(C, tl), rl = pcr_row<NH>(R, tl);
      double ah = pcr_row<NH>(A, th), bh = pcr_row<NH>(B, th), ch = pcr_row<NH>(C, th), rh = pcr_row<NH>(R, th);
      if (lo < 0) { al = 0.0; bl = 1.0; cl = 0.0; rl = 0.0; }
      if (hi >= n) { ah = 0.0; bh = 1.0; ch = 0.0; rh = 0.0; }
      const double alpha = -A[h] / pcr_guard(bl);
      const double gamma = -C[h] / pcr_guard(bh);
      An[h] = alpha * al;
      Cn[h] = gamma * ch;
      Bn[h] = B[h] + alpha * cl + gamma * ah;
      Rn[h] = R[h] + alpha * rl + gamma * rh;
    }
#pragma unroll
    for (int h = 0; h < NH; h++) {
      A[h] = An[h]; B[h] = Bn[h]; C[h] = Cn[h]; R[h] = Rn[h];
    }
  }
#pragma unroll
  for (int h = 0; h < NH; h++) {
    const int i = lane + 32 * h;
    if (i < n) LV(u, col, j0 + i, ld) = R[h] / pcr_guard(B[h]);
  }
}
__global__ void __launch_bounds__(32 * PCR_WARPS)
k_tridiagonal_multi_pcr(int64_t ncols, int64_t ld, int nlevs, double* u, const double* __restrict__ a,
                        const double* __restrict__ b, const double* __restrict__ cc,
                        const double* __restrict__ r, const int64_t* jtop, const uint8_t* mask) {
  const int64_t col = (int64_t)blockIdx.x * PCR_WARPS + (threadIdx.x >> 5);
  if (col >= ncols || !mask[col]) return;             // the whole warp leaves together
  const int64_t j64 = jtop[col];
  if (j64 < 1 || j64 > nlevs) return;
  const int j0 = (int)j64, n = nlevs - j0 + 1;
  if (n <= 32) pcr_solve<1>(col, ld, j0, n, u, a, b, cc, r);
  else pcr_solve<2>(col, ld, j0, n, u, a, b, cc, r);
}

// Synthetic per-step forcing (the upstream radiation / infiltration modules are out
// of scope): sabg = sabg_soil = sabg_snow = G, sabg_lyr = G on the top active layer
// and 0 elsewhere, forc_lwrad = SB*t_grnd^4, qflx_infl = I.
__global__ void __launch_bounds__(BLOCK)
k_synth_forcing(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw, const double* G,
                const double* I) {
  const int64_t c = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (c >= nc || !ft.mask_nolakec[c]) return;
  const double g = G[c];
  const int64_t snl = ft.col_snl[c];
  for (int64_t p1 = ft.col_patchi[c]; p1 <= ft.col_patchf[c]; p1++) {
    if (p1 < 1 || p1 > D.np) break;
    const int64_t p = p1 - 1;
    ((double*)ft.sabg)[p] = g;
    ((double*)ft.sabg_soil)[p] = g;
    ((double*)ft.sabg_snow)[p] = g;
    for (int k = 1; k <= D.nlevsno + 1; k++) LV((double*)ft.sabg_lyr, p, k, D.ldp) = 0.0;
    if (snl <= 0 && snl >= -D.nlevsno) LV((double*)ft.sabg_lyr, p, (int)snl + 1 + D.nlevsno, D.ldp) = g;
  }
  ((double*)ft.forc_lwrad)[c] = SB * jl_pow4(ft.t_grnd[c]);
  ((double*)fw.qflx_infl)[c] = I[c];
}

// ---------------------------------------------------------------------------
cudaError_t launch_soil_temperature(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double dtime,
                                    int snow_method, uint32_t* col_status, uint32_t* dev_status,
                                    cudaStream_t s) {
  const unsigned g = (unsigned)((nc + D.st_block - 1) / D.st_block);
  if (D.st_block == 640)
    k_soil_temperature<640><<<g, 640, 0, s>>>(D, nc, f, dtime, snow_method, col_status, dev_status);
  else if (D.st_block == 320)
    k_soil_temperature<320><<<g, 320, 0, s>>>(D, nc, f, dtime, snow_method, col_status, dev_status);
  else
    k_soil_temperature<128><<<g, 128, 0, s>>>(D, nc, f, dtime, snow_method, col_status, dev_status);
  return cudaGetLastError();
}
cudaError_t launch_water_fractions(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, cudaStream_t s) {
  k_water_fractions<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f);
  return cudaGetLastError();
}
cudaError_t launch_moisture_form(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                 const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                 uint32_t* dev_status, cudaStream_t s) {
  k_moisture_form<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f, cfg, dtime, col_status, dev_status);
  return cudaGetLastError();
}
cudaError_t launch_column_step(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                               const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                               int snow_method, double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                               uint32_t* dev_status, cudaStream_t s) {
  k_column_step<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, ft, fw, cfg, dtime, snow_method, t_ssbef, t_h2osfc_bef,
                                               col_status, dev_status);
  return cudaGetLastError();
}
cudaError_t launch_soiltemp_fractions(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                      const clmgb_soilwater_fields& fw, double dtime, int snow_method,
                                      double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                                      uint32_t* dev_status, cudaStream_t s, double* st_log) {
  const int nb = (D.st_block == 640 || D.st_block == 320) ? D.st_block : 128;
  const unsigned g = (unsigned)((nc + nb - 1) / nb);
#define CLMGB_STF(L, NB) \
  k_soil_temperature_fractions<L, NB><<<g, NB, 0, s>>>(D, nc, ft, fw, dtime, snow_method, t_ssbef, t_h2osfc_bef, \
                                                      col_status, dev_status, st_log)
  if (st_log) {
    if (nb == 640) CLMGB_STF(true, 640);
    else if (nb == 320) CLMGB_STF(true, 320);
    else CLMGB_STF(true, 128);
  } else {
    if (nb == 640) CLMGB_STF(false, 640);
    else if (nb == 320) CLMGB_STF(false, 320);
    else CLMGB_STF(false, 128);
  }
#undef CLMGB_STF
  return cudaGetLastError();
}
int queue_blocks_per_sm() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_moisture_form_queue<false>, BLOCK, 0) != cudaSuccess)
    nb = 1;
  return nb > 0 ? nb : 1;
}
cudaError_t launch_moisture_form_queue(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                       const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                       int or_status, uint32_t* dev_status, unsigned long long* queue,
                                       int grid_blocks, const QueueScratch& qs, cudaStream_t s,
                                       const double* dt_init, const SubstepLogView* log) {
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (log && (e = cudaMemsetAsync(log->count, 0xff, (size_t)nc * sizeof(int32_t), s)) != cudaSuccess) return e;
  const bool use = qs.capacity >= nc && qs.order && qs.bins && qs.imp;
  if (use) {
    if (qs.packed && qs.pcache) {
      if ((e = launch_column_records(D, nc, f, cfg.e_ice, qs.imp, qs.capacity, qs.pcache, qs.records_tma != 0,
                                     dev_status, s, qs.records_tma_used)) != cudaSuccess)
        return e;
    } else {
      k_impedance<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f, cfg.e_ice, qs.imp, qs.capacity);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (qs.longest_first) {
      if ((e = cudaMemsetAsync(qs.bins, 0, (2 * ORDER_BINS + 1) * sizeof(unsigned int), s)) != cudaSuccess) return e;
      k_order_hist<<<grid_for(nc), BLOCK, 0, s>>>(nc, f.mask_hydrology, f.num_substeps, qs.bins);
      k_order_scan<<<1, 32, 0, s>>>(qs.bins);
      k_order_scatter<<<grid_for(nc), BLOCK, 0, s>>>(nc, f.mask_hydrology, f.num_substeps, qs.bins, qs.order,
                                                     col_status, or_status);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  const int64_t need = (nc + BLOCK - 1) / BLOCK;
  const int grid = (int)(need < grid_blocks ? need : grid_blocks);
  const bool listed = use && qs.longest_first;
  const uint32_t* ord = listed ? qs.order : nullptr;
  const unsigned int* nl = listed ? qs.bins + 2 * ORDER_BINS : nullptr;
  const double* imp = use ? qs.imp : nullptr;
  const int64_t ldi = use ? qs.capacity : 0;
  QueueScratch q = qs;
  if (!use || log || !q.d_count) q.defer = 0;              // deferral needs the reserved scratch
  if (q.defer > 0) {                                       // empty list, zero claim/publish/consume counts
    if ((e = cudaMemsetAsync(q.d_count, 0, 3 * sizeof(unsigned long long), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(q.d_list, 0xff, (size_t)nc * sizeof(uint32_t), s)) != cudaSuccess) return e;
  }
  if (use && qs.packed && qs.pcache) {
    const size_t smem = (size_t)(PBLOCK / 32) * (size_t)packed_warp_doubles(D.nlevsoi) * sizeof(double);
    auto kern = log ? k_moisture_form_packed<true> : k_moisture_form_packed<false>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
      return e;
    // the blocks that fit on the GPU at once (the kernel's warps wait on one another
    // only through the bounded waits of the deferred-column list)
    int dev = 0, nsm = 0, nb = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, PBLOCK, smem)) != cudaSuccess) return e;
    if (nb < 1) return cudaErrorInvalidConfiguration;
    int gp = grid > 0 ? grid : 1;
    if (gp > nb * nsm) gp = nb * nsm;
    q.out_records = 1;
    kern<<<gp, PBLOCK, smem, s>>>(D, nc, f, cfg, dtime, col_status, or_status, dev_status, queue, ord, nl, dt_init,
                                 log ? *log : SubstepLogView{nullptr, nullptr, 0, 0}, qs.fresh_batch, q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // the solved columns' water, smp_l and hk_l from their records to the state
    if ((e = launch_column_outputs(D, nc, f, qs.pcache, s)) != cudaSuccess) return e;
  } else if (log)
    k_moisture_form_queue<true><<<grid > 0 ? grid : 1, BLOCK, 0, s>>>(D, nc, f, cfg, dtime, col_status, or_status,
                                                                      dev_status, queue, ord, nl, imp, ldi, dt_init,
                                                                      *log, qs.fresh_batch, q);
  else
    k_moisture_form_queue<false><<<grid > 0 ? grid : 1, BLOCK, 0, s>>>(D, nc, f, cfg, dtime, col_status, or_status,
                                                                       dev_status, queue, ord, nl, imp, ldi, dt_init,
                                                                       SubstepLogView{nullptr, nullptr, 0, 0},
                                                                       qs.fresh_batch, q);
  return cudaGetLastError();
}
cudaError_t launch_compute_qcharge(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                  const clmgb_swm_config& cfg, double dtime, cudaStream_t s) {
  if (cfg.lower_boundary_condition != CLMGB_BC_WATERTABLE || nc <= 0) return cudaSuccess;
  k_compute_qcharge<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f, dtime);
  return cudaGetLastError();
}
cudaError_t launch_flexible_cn(const Dims& D, int64_t nc, const clmgb_flexcn_fields& f, cudaStream_t s) {
  k_flexible_cn<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f);
  return cudaGetLastError();
}
cudaError_t launch_math_eval(int op, int64_t n, const double* x, const double* y, double* out, cudaStream_t s) {
  k_math_eval<<<grid_for(n), BLOCK, 0, s>>>(op, n, x, y, out);
  return cudaGetLastError();
}
cudaError_t launch_phase_change(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double dtime,
                                const double* dhsdT, int which, cudaStream_t s) {
  k_phase_change<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, f, dtime, dhsdT, which);
  return cudaGetLastError();
}
cudaError_t launch_band_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* bmatrix,
                              const double* rvector, const int64_t* jtop, const int64_t* jbot,
                              const uint8_t* mask, int kl, int ku, int nlevsno_off, cudaStream_t s) {
  if (kl == 2 && ku == 2)
    k_band_solve<2, 2><<<grid_for(nc), BLOCK, 0, s>>>(nc, ldc, nlev, tvector, bmatrix, rvector, jtop, jbot, mask,
                                                      nlevsno_off);
  else if (kl == 1 && ku == 1)
    k_band_solve<1, 1><<<grid_for(nc), BLOCK, 0, s>>>(nc, ldc, nlev, tvector, bmatrix, rvector, jtop, jbot, mask,
                                                      nlevsno_off);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}
cudaError_t launch_tridiagonal_multi(int64_t ncols, int64_t ldc, int nlevs, double* u, const double* a,
                                     const double* b, const double* c, const double* r, const int64_t* jtop,
                                     const uint8_t* mask, cudaStream_t s, int method) {
  if (nlevs > MAXTRI) return cudaErrorInvalidValue;
  if (method == CLMGB_TRIDIAG_PCR)
    k_tridiagonal_multi_pcr<<<(unsigned)((ncols + PCR_WARPS - 1) / PCR_WARPS), 32 * PCR_WARPS, 0, s>>>(
        ncols, ldc, nlevs, u, a, b, c, r, jtop, mask);
  else
    k_tridiagonal_multi<<<grid_for(ncols), BLOCK, 0, s>>>(ncols, ldc, nlevs, u, a, b, c, r, jtop, mask);
  return cudaGetLastError();
}
cudaError_t launch_synth_forcing(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                 const clmgb_soilwater_fields& fw, const double* G, const double* I,
                                 cudaStream_t s) {
  k_synth_forcing<<<grid_for(nc), BLOCK, 0, s>>>(D, nc, ft, fw, G, I);
  return cudaGetLastError();
}

}  // namespace clmgb
