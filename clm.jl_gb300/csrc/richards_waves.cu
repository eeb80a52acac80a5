// richards_waves.cu — the moisture-form Richards solve in synchronous waves.
//
// soilwm_moisture_form_solve! (soil_water_movement.jl:1250-1489) gives every column
// its own adaptive substep loop: an attempt (tridiagonal solve and error estimate)
// that is accepted or rejected, and after every accepted substep a fresh evaluation
// of the hydraulic properties and fluxes.  Run one column per thread, the lanes of a
// warp disagree about which of the two they need and idle through the other.
//
// Here one cooperative persistent kernel advances all columns together in rounds
// separated by grid-wide barriers.  In a round every unfinished column makes one
// attempt; the columns that start a new substep (all in round 0, then those that
// accepted in the previous round) first evaluate the hydraulic properties, fluxes
// and flux derivatives.  The round's work list holds those columns first and the
// rejected ones after them, and warps take 32 consecutive entries at a time, so the
// lanes of a warp run the same code.  Outcomes are appended to the next round's
// two lists with one atomic per warp.
// The per-column state between phases lives in the handle's reserved scratch,
// level-major ([level][column]) for coalesced access.  The arithmetic is the same
// expressions in the same order as the one-column-per-thread form (clmgb_device.cuh),
// so the results are identical bit for bit.
//
// Data written by one SM and read by another after a barrier is accessed with
// __ldcg/__stcg (cached in L2 only, never in a possibly stale L1).
#include <cooperative_groups.h>
#include "clmgb_device.cuh"
#include "launch.h"

namespace cg = cooperative_groups;

namespace clmgb {

constexpr int WAVE_BLOCK = 128;

// one attempt result
enum : int { WAVE_REJECT = 0, WAVE_ACCEPT = 1, WAVE_DONE = 2 };

__device__ __forceinline__ void append(uint32_t* list, unsigned int* count, bool want, uint32_t c) {
  const unsigned FULL = __activemask();
  const unsigned m = __ballot_sync(FULL, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  unsigned int base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(m));
  base = __shfl_sync(FULL, base, leader);
  if (want) __stcg(list + base + __popc(m & ((1u << lane) - 1u)), c);
}

#define W(arr, j, c) (arr)[(int64_t)((j) - 1) * w.cap + (c)]

// H phase for column c: soil_water_movement.jl:1274-1378 (hydraulics and fluxes).
__device__ __forceinline__ void wave_hydraulics(const Dims& D, const clmgb_soilwater_fields& f,
                                                const clmgb_swm_config& cfg, const WaveScratch& w, int64_t c) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1, nlevsoi = D.nlevsoi;
  const int nlayers = (int)f.col_nbedrock[c];
  const int lower_bc = cfg.lower_boundary_condition;
  double s2[MAXSOI + 2], smp[MAXSOI + 1], dsmpdw[MAXSOI + 1], hk[MAXSOI + 1], dhkdw[MAXSOI + 1];
  for (int j = 1; j <= nlayers; j++) {
    const double liq = __ldcg(&LV(f.h2osoi_liq, c, joff + j, ld));
    const double vwc = jl_max(liq, 1.0e-6) / (LVc(f.dz, c, joff + j, ld) * DENH2O);
    double s = vwc / LVc(f.watsat, c, j, ld);
    s = jl_min(s, 1.0);
    s = jl_max(0.01, s);
    s2[j] = s;
  }
  for (int j = 1; j <= nlayers; j++) {
    double s1 = (j == nlayers) ? s2[j] : 0.5 * (s2[j] + s2[j + 1]);
    s1 = jl_min(s1, 1.0);
    s1 = jl_max(0.01, s1);
    const double b = LVc(f.bsw, c, j, ld);
    const double hkv = W(w.imp, j, c) * LVc(f.hksat, c, j, ld) * cm_pow(s1, 2.0 * b + 3.0);
    const double dhkds = (2.0 * b + 3.0) * hkv / s1;
    const double sn = s2[j];
    const double smpv = -LVc(f.sucsat, c, j, ld) * cm_pow(sn, -b);
    const double dsmpds = -b * smpv / sn;
    hk[j] = hkv;
    smp[j] = smpv;
    dhkdw[j] = dhkds;
    dsmpdw[j] = dsmpds / LVc(f.watsat, c, j, ld);
    LV(f.smp_l, c, j, ld) = smpv;
    LV(f.hk_l, c, j, ld) = hkv;
  }
  for (int j = 1; j <= nlayers - 1; j++) {
    const double dhkds1 = 0.5 * dhkdw[j] / LVc(f.watsat, c, j, ld);
    const double dhkds2 = 0.5 * dhkdw[j] / LVc(f.watsat, c, j + 1, ld);
    const double num = smp[j + 1] - smp[j];
    const double den = M_TO_MM * (LVc(f.z, c, joff + j + 1, ld) - LVc(f.z, c, joff + j, ld));
    __stcg(&W(w.qout, j, c), -hk[j] * num / den + hk[j]);
    __stcg(&W(w.dqodw1, j, c), (hk[j] * dsmpdw[j] - dhkds1 * num) / den + dhkds1);
    __stcg(&W(w.dqodw2, j, c), (-hk[j] * dsmpdw[j + 1] - dhkds2 * num) / den + dhkds2);
  }
  {
    const int j = nlayers;
    double qo = 0.0, d1 = 0.0;
    if (lower_bc == CLMGB_BC_WATERTABLE) {
      int jwt = nlevsoi;
      for (int jj = 1; jj <= nlevsoi; jj++) {
        if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) { jwt = jj - 1; break; }
      }
      if (j <= jwt) {
        const double dhkds1l = dhkdw[j] / LVc(f.watsat, c, j, ld);
        const double num = -smp[j];
        const double den = M_TO_MM * (f.zwt[c] - LVc(f.z, c, joff + j, ld));
        qo = -hk[j] * num / den + hk[j];
        d1 = (hk[j] * dsmpdw[j] - dhkds1l * num) / den + dhkds1l;
      }
    } else if (lower_bc == CLMGB_BC_FLUX) {
      qo = hk[j];
      d1 = dhkdw[j] / LVc(f.watsat, c, j, ld);
    }
    __stcg(&W(w.qout, j, c), qo);
    __stcg(&W(w.dqodw1, j, c), d1);
    __stcg(&W(w.dqodw2, j, c), 0.0);
    __stcg(&w.hk_bot[c], hk[j]);
    __stcg(&w.dhkdw_bot[c], dhkdw[j]);
  }
  const double qinfl = f.qflx_infl[c];
  for (int j = 1; j <= nlayers; j++) {
    const double qin = j == 1 ? qinfl : __ldcg(&W(w.qout, j - 1, c));
    __stcg(&W(w.fnet1, j, c), qin - __ldcg(&W(w.qout, j, c)) - LVc(f.qflx_rootsoi, c, j, ld));
  }
}

// A phase for column c: one attempt (soil_water_movement.jl:1380-1483).
__device__ __forceinline__ int wave_attempt(const Dims& D, const clmgb_soilwater_fields& f,
                                            const clmgb_swm_config& cfg, double dtime, const WaveScratch& w,
                                            int64_t c) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  const int nlayers = (int)f.col_nbedrock[c];
  const int lower_bc = cfg.lower_boundary_condition;
  int nsub = __ldcg(&w.nsub[c]) + 1;
  __stcg(&w.nsub[c], nsub);
  if (nsub > D.attempt_cap) {
    __stcg(&w.status[c], __ldcg(&w.status[c]) | CLMGB_COL_SUBSTEP_CAP);
    return WAVE_DONE;
  }
  const double dtsub = __ldcg(&w.dtsub[c]);
  const double dt_cur = __ldcg(&w.dtcur[c]);
  double dt_dz[MAXSOI + 1];
  // dt_dz = dtsub / (1000*dz), rescaled exactly by a power of two when dtsub only halved/doubled
  if (dtsub != dt_cur) {
    const uint64_t a = (uint64_t)__double_as_longlong(dtsub), b = (uint64_t)__double_as_longlong(dt_cur);
    const uint64_t MANT = 0x000fffffffffffffULL;
    const int ea = (int)((a >> 52) & 0x7ff), eb = (int)((b >> 52) & 0x7ff);
    const bool pow2 = dt_cur > 0.0 && (a & MANT) == (b & MANT) && ea > 0 && eb > 0 && ea < 2047 && eb < 2047;
    for (int j = 1; j <= nlayers; j++) {
      double v;
      if (pow2) {
        const long long old = __double_as_longlong(__ldcg(&W(w.dtdz, j, c)));
        const int ev = (int)((old >> 52) & 0x7ff);
        if (ev > 0 && ev + (ea - eb) > 0 && ev + (ea - eb) < 2047)
          v = __longlong_as_double(old + ((long long)(ea - eb) << 52));
        else
          v = dtsub / (M_TO_MM * LVc(f.dz, c, joff + j, ld));
      } else {
        v = dtsub / (M_TO_MM * LVc(f.dz, c, joff + j, ld));
      }
      dt_dz[j] = v;
      __stcg(&W(w.dtdz, j, c), v);
    }
    __stcg(&w.dtcur[c], dtsub);
  } else {
    for (int j = 1; j <= nlayers; j++) dt_dz[j] = __ldcg(&W(w.dtdz, j, c));
  }
  // ---- RHS / LHS fused into the Thomas forward sweep ----
  double gam[MAXSOI + 1], dwat[MAXSOI + 1];
  double bet, dwat_prev;
  {
    const double fn1 = __ldcg(&W(w.fnet1, 1, c));
    const double d1 = __ldcg(&W(w.dqodw1, 1, c));
    const double rmx = -fn1 * dt_dz[1];
    const double bmx = -1.0 - (-0.0 + d1) * dt_dz[1];
    bet = bmx;
    if (abs_lt(bet, 1.0e-30)) bet = 1.0e-30;
    dwat_prev = rmx / bet;
    dwat[1] = dwat_prev;
  }
  double cmx_prev = -__ldcg(&W(w.dqodw2, 1, c)) * dt_dz[1];
  double dqodw1_prev = __ldcg(&W(w.dqodw1, 1, c)), dqodw2_prev = __ldcg(&W(w.dqodw2, 1, c));
  for (int j = 2; j <= nlayers; j++) {
    const double dqidw0 = dqodw1_prev, dqidw1 = dqodw2_prev;
    const double dqodw1 = __ldcg(&W(w.dqodw1, j, c));
    const double dqodw2 = __ldcg(&W(w.dqodw2, j, c));
    const double fn1 = __ldcg(&W(w.fnet1, j, c));
    const double amx = dqidw0 * dt_dz[j];
    const double bmx = -1.0 - (-dqidw1 + dqodw1) * dt_dz[j];
    const double cmx = (j == nlayers) ? 0.0 : -dqodw2 * dt_dz[j];
    const double rmx = -fn1 * dt_dz[j];
    gam[j] = cmx_prev / bet;
    bet = bmx - amx * gam[j];
    if (abs_lt(bet, 1.0e-30)) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
    dwat_prev = (rmx - amx * dwat_prev) / bet;
    dwat[j] = dwat_prev;
    cmx_prev = cmx;
    dqodw1_prev = dqodw1;
    dqodw2_prev = dqodw2;
  }
  {
    double dwat_next = dwat_prev;
    for (int j = nlayers - 1; j >= 1; j--) {
      dwat_next = dwat[j] - gam[j + 1] * dwat_next;
      dwat[j] = dwat_next;
    }
  }
  // ---- error estimate ----
  const bool expensive = (cfg.flux_calculation == 42);
  double errorMax = 0.0;
  for (int j = 1; j <= nlayers; j++) {
    const double fn1 = __ldcg(&W(w.fnet1, j, c));
    double fnet0;
    if (expensive) {
      const double qin = j == 1 ? f.qflx_infl[c] : __ldcg(&W(w.qout, j - 1, c));
      const double qout = __ldcg(&W(w.qout, j, c));
      const double dqidw1 = j == 1 ? 0.0 : __ldcg(&W(w.dqodw2, j - 1, c));
      const double dqodw1 = __ldcg(&W(w.dqodw1, j, c));
      const double qin_test = j == 1 ? qin + dqidw1 * dwat[j]
                                     : qin + __ldcg(&W(w.dqodw1, j - 1, c)) * dwat[j - 1] + dqidw1 * dwat[j];
      const double qout_test = j == nlayers ? qout + dqodw1 * dwat[j]
                                            : qout + dqodw1 * dwat[j] + __ldcg(&W(w.dqodw2, j, c)) * dwat[j + 1];
      fnet0 = qin_test - qout_test - LVc(f.qflx_rootsoi, c, j, ld);
    } else {
      fnet0 = dwat[j] / dt_dz[j];
    }
    const double ev = fabs(fn1 - fnet0) * dtsub * 0.5;
    errorMax = jl_max(errorMax, ev);
  }
  if (errorMax > cfg.xTolerUpper && dtsub > cfg.dtmin) {
    __stcg(&w.dtsub[c], jl_max(dtsub / 2.0, cfg.dtmin));
    return WAVE_REJECT;
  }
  for (int j = 1; j <= nlayers; j++) {
    double* p = &LV(f.h2osoi_liq, c, joff + j, ld);
    __stcg(p, __ldcg(p) + dwat[j] * (M_TO_MM * LVc(f.dz, c, joff + j, ld)));
  }
  double qcTemp;
  if (lower_bc == CLMGB_BC_FLUX) qcTemp = __ldcg(&w.hk_bot[c]) + __ldcg(&w.dhkdw_bot[c]) * dwat[nlayers];
  else if (lower_bc == CLMGB_BC_ZERO_FLUX) qcTemp = 0.0;
  else qcTemp = __ldcg(&W(w.qout, nlayers, c)) + __ldcg(&W(w.dqodw1, nlayers, c)) * dwat[nlayers];
  const double qc = __ldcg(&w.qc[c]) + qcTemp * (dtsub / dtime);
  __stcg(&w.qc[c], qc);
  const double dtdone = __ldcg(&w.dtdone[c]) + dtsub;
  __stcg(&w.dtdone[c], dtdone);
  if (fabs(dtime - dtdone) < cfg.verySmall) return WAVE_DONE;
  double nd = dtsub;
  if (errorMax < cfg.xTolerLower) nd = dtsub * 2.0;
  __stcg(&w.dtsub[c], jl_min(nd, dtime - dtdone));
  return WAVE_ACCEPT;
}

// writes qcharge, num_substeps and the status of a finished column
__device__ __forceinline__ uint32_t wave_finish(const Dims& D, const clmgb_soilwater_fields& f, const WaveScratch& w,
                                                int64_t c) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  const int nlayers = (int)f.col_nbedrock[c];
  uint32_t st = __ldcg(&w.status[c]);
  for (int j = 1; j <= nlayers; j++)
    if (!isfinite(__ldcg(&LV(f.h2osoi_liq, c, joff + j, ld)))) st |= CLMGB_COL_NONFINITE;
  f.qcharge[c] = __ldcg(&w.qc[c]);
  f.num_substeps[c] = (double)__ldcg(&w.nsub[c]);
  return st;
}

// counters: three sets of {length of the "hydraulics then attempt" list, length of the
// "attempt only" list, chunk counter}.  Round r reads set r%3, appends into set
// (r+1)%3 and clears set (r+2)%3, which no thread touches during round r (it was
// last read before the barrier that ended round r-1).  The lists are double buffered.
__global__ void __launch_bounds__(WAVE_BLOCK)
k_moisture_form_waves(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                      uint32_t* col_status, int or_status, uint32_t* dev_status, WaveScratch w) {
  cg::grid_group grid = cg::this_grid();
  const int64_t nthr = (int64_t)gridDim.x * WAVE_BLOCK;
  const int64_t tid = (int64_t)blockIdx.x * WAVE_BLOCK + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  volatile unsigned int* cnt = w.counters;
  // set-up: impedances, per-column scalars; every column starts with hydraulics
  for (int64_t base = 0; base < nc; base += nthr) {
    const int64_t c = base + tid;
    bool take = false;
    if (c < nc) {
      if (!f.mask_hydrology[c]) {
        if (col_status && !or_status) col_status[c] = 0;
      } else {
        const int64_t nl = f.col_nbedrock[c];
        if (nl < 1 || nl > D.nlevsoi) {
          const uint32_t st = CLMGB_COL_LEVEL_RANGE;
          if (col_status) col_status[c] = or_status ? (col_status[c] | st) : st;
          if (dev_status) atomicOr(dev_status, st);
        } else {
          const int nlayers = (int)nl;
          for (int j = 1; j <= nlayers; j++) __stcg(&W(w.imp, j, c), mf_impedance(D, f, cfg.e_ice, c, j, nlayers));
          __stcg(&w.nsub[c], 0);
          __stcg(&w.dtsub[c], dtime);
          __stcg(&w.dtdone[c], 0.0);
          __stcg(&w.qc[c], 0.0);
          __stcg(&w.dtcur[c], -1.0);
          __stcg(&w.status[c], 0u);
          take = true;
        }
      }
    }
    append(w.listH[0], w.counters + 0, take, (uint32_t)c);  // set 0, list 0
  }
  grid.sync();
  int cur = 0;  // list buffer
  int cs = 0;   // counter set
  for (int round = 0; round <= D.attempt_cap + 1; round++) {
    const unsigned int nHA = cnt[3 * cs], nA = cnt[3 * cs + 1];
    const unsigned int total = nHA + nA;
    if (total == 0) break;
    const int nxt = cur ^ 1;
    const int cn = cs == 2 ? 0 : cs + 1;
    const int cc = cn == 2 ? 0 : cn + 1;
    if (tid == 0) {
      cnt[3 * cc] = 0;
      cnt[3 * cc + 1] = 0;
      cnt[3 * cc + 2] = 0;
    }
    // warps take 32 consecutive items: first the columns that need hydraulics, then
    // the rest, so all lanes of a warp (but one) run the same code
    for (;;) {
      unsigned int base = 0;
      if (lane == 0) base = atomicAdd(&w.counters[3 * cs + 2], 32u);
      base = __shfl_sync(FULL, base, 0);
      if (base >= total) break;
      const unsigned int i = base + (unsigned int)lane;
      int r = -1;
      int64_t c = 0;
      if (i < total) {
        const bool needH = i < nHA;
        c = (int64_t)(needH ? __ldcg(&w.listH[cur][i]) : __ldcg(&w.listA[cur][i - nHA]));
        if (needH) wave_hydraulics(D, f, cfg, w, c);
        r = wave_attempt(D, f, cfg, dtime, w, c);
        if (r == WAVE_DONE) {
          const uint32_t st = wave_finish(D, f, w, c);
          if (col_status) col_status[c] = or_status ? (col_status[c] | st) : st;
          if (st && dev_status) atomicOr(dev_status, st);
        }
      }
      append(w.listH[nxt], w.counters + 3 * cn, r == WAVE_ACCEPT, (uint32_t)c);
      append(w.listA[nxt], w.counters + 3 * cn + 1, r == WAVE_REJECT, (uint32_t)c);
    }
    grid.sync();
    cur = nxt;
    cs = cn;
  }
}

#undef W

int waves_blocks_per_sm() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_moisture_form_waves, WAVE_BLOCK, 0) != cudaSuccess) nb = 0;
  return nb;
}

cudaError_t launch_moisture_form_waves(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                       const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                       int or_status, uint32_t* dev_status, const WaveScratch& w, int grid_blocks,
                                       cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(w.counters, 0, 9 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  Dims d = D;
  int64_t n = nc;
  clmgb_soilwater_fields ff = f;
  clmgb_swm_config cc = cfg;
  double dt = dtime;
  uint32_t* cs = col_status;
  int ors = or_status;
  uint32_t* ds = dev_status;
  WaveScratch ww = w;
  void* args[] = {&d, &n, &ff, &cc, &dt, &cs, &ors, &ds, &ww};
  return cudaLaunchCooperativeKernel((const void*)k_moisture_form_waves, dim3(grid_blocks), dim3(WAVE_BLOCK), args,
                                     0, s);
}

}  // namespace clmgb
