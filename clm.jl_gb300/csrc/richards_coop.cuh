// richards_coop.cuh — the warp-per-column finish of the moisture-form Richards solve
// (soilwm_moisture_form_solve!, soil_water_movement.jl:1250-1489) for the columns the
// work-queue kernel defers (QueueScratch::defer).
//
// On GB300 an FP64 warp instruction occupies the SM's FP64 pipe for about 17 cycles
// whether 1 or 32 lanes are active, so a column that needs many more substep attempts
// than the rest (up to ~70 against a mean of ~5) crawls at the end of the work queue
// with one useful lane per warp.  Such a column leaves the queue at an accepted
// substep, and a warp whose lanes have run out of work finishes it with lane j-1 on
// level j: the hydraulic properties, fluxes, matrix entries, the error estimate and
// the update are formed by all levels at once, and the Thomas recurrences run level
// by level with the carried values broadcast from the level's lane.  Every level's
// operations and their order are those of mf_refresh and mf_attempt
// (clmgb_device.cuh), so the results are the work-queue kernel's bits.
#pragma once
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr unsigned COOP_FULL = 0xffffffffu;
constexpr uint32_t DEFER_EMPTY = 0xffffffffu;     // a list slot not written yet
constexpr uint32_t DEFER_GIVEN_BACK = 0xfffffffeu; // a slot the drain stopped waiting for

// The deferring lane's half of a hand-over: claim a list slot, store the column's state,
// then write the column's index into the slot and count it published.  Returns false
// when the drain has already given the slot back (its bounded wait for the index ran
// out, coop_drain): the lane then keeps the column and finishes it itself, so no column
// is ever left unfinished.  Each column is handed over at most once, so at most nc
// slots are claimed.
template <class LT>
__device__ __forceinline__ bool coop_defer(const LT& L, const QueueScratch& qs) {
  const int64_t c = L.c, cap = qs.capacity;
  const unsigned long long slot = atomicAdd(qs.d_count, 1ULL);
  for (int j = 1; j <= L.nlayers; j++) qs.d_liq[(int64_t)(j - 1) * cap + c] = L.liq[j];
  qs.d_dtsub[c] = L.dtsub;
  qs.d_dtdone[c] = L.dtdone;
  qs.d_qc[c] = L.qc;
  qs.d_nsub[c] = L.nsub;
  qs.d_status[c] = L.status;
  __threadfence();
  // test hook (CLMGB_OPT_QUEUE_PUBLISH_DELAY): an even slot is counted published before
  // its index is written; the lane then sleeps until a finishing warp has taken the slot
  // (or publish_delay ns have passed, <= 10 ms) and 2 us more, so that warp finds the
  // slot empty
  const bool late = qs.publish_delay > 0 && (slot & 1ULL) == 0;
  if (late) {
    atomicAdd(qs.d_count + 1, 1ULL);
    for (int t = 0; t < qs.publish_delay; t += 500) {
      if (*(volatile unsigned long long*)(qs.d_count + 2) > slot) {
        __nanosleep(2000);
        break;
      }
      __nanosleep(500);
    }
  }
  const uint32_t prev = atomicCAS(qs.d_list + slot, DEFER_EMPTY, (uint32_t)c);
  __threadfence();
  if (!late) atomicAdd(qs.d_count + 1, 1ULL);   // published (a slot given back counts too)
  return prev == DEFER_EMPTY;
}

__device__ __forceinline__ double coop_bcast(double v, int src) { return __shfl_sync(COOP_FULL, v, src); }

// Julia's max over the lanes' non-negative values (NaN wins, as the sequential jl_max)
__device__ __forceinline__ double coop_jl_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = jl_max(v, __shfl_xor_sync(COOP_FULL, v, o));
  return v;
}

// Finishes deferred column c; called by all 32 lanes of a warp with the same c.
__device__ __noinline__ void coop_finish_column(const Dims& D, const clmgb_soilwater_fields& f,
                                                const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                                int or_status, uint32_t* dev_status, const QueueScratch& qs,
                                                int64_t c) {
  const int lane = threadIdx.x & 31;
  const int64_t ld = D.ldc, cap = qs.capacity;
  const int joff = D.nlevsno, joff_zi = D.nlevsno + 1, nlevsoi = D.nlevsoi;
  const int lower_bc = cfg.lower_boundary_condition;
  const bool expensive = (cfg.flux_calculation == 42);
  const int n = (int)f.col_nbedrock[c];       // validated when the column was begun
  const int j = lane + 1;                     // this lane's level
  const bool lv = j <= n;
  // where the water, smp_l and hk_l go: the column's record (packed kernel) or the state
  double* const orec = qs.out_records ? qs.pcache + c * (int64_t)(PC_ALL * nlevsoi) : nullptr;
  // the column's state at its last accepted substep
  double liq = 0.0, dzv = 1.0, imp = 0.0, ws = 1.0, bsw = 0.0, hksat = 0.0, sucsat = 0.0, zj = 0.0, zj1 = 0.0;
  double root = 0.0;
  if (lv) {
    liq = __ldcg(qs.d_liq + (int64_t)(j - 1) * cap + c);
    dzv = LVc(f.dz, c, joff + j, ld);
    imp = qs.imp[(int64_t)(j - 1) * cap + c];
    ws = LVc(f.watsat, c, j, ld);
    bsw = LVc(f.bsw, c, j, ld);
    hksat = LVc(f.hksat, c, j, ld);
    sucsat = LVc(f.sucsat, c, j, ld);
    zj = LVc(f.z, c, joff + j, ld);
    if (j < n) zj1 = LVc(f.z, c, joff + j + 1, ld);
    root = LVc(f.qflx_rootsoi, c, j, ld);
  }
  double dtsub = __ldcg(qs.d_dtsub + c), dtdone = __ldcg(qs.d_dtdone + c), qc = __ldcg(qs.d_qc + c);
  int nsub = __ldcg(qs.d_nsub + c);
  uint32_t status = __ldcg(qs.d_status + c);
  double dt_cur = -1.0, dt_dz = 0.0;
  double hk = 0.0, dhkdw = 0.0, qin = 0.0, qout = 0.0, dqidw0 = 0.0, dqidw1 = 0.0, dqodw1 = 0.0, dqodw2 = 0.0;
  double fnet1 = 0.0, gam = 0.0, dwat = 0.0;
  bool fresh = true;
  for (;;) {
    nsub += 1;
    if (nsub > D.attempt_cap) {
      status |= CLMGB_COL_SUBSTEP_CAP;
      break;
    }
    // dt_dz = dtsub / (1000 dz); the work-queue kernel's exponent rescaling of it
    // gives this quotient's bits, so it is divided afresh here
    if (dtsub != dt_cur) {
      dt_dz = jl_div(dtsub, M_TO_MM * dzv);
      dt_cur = dtsub;
    }
    if (qs.work && lane == 0) atomicAdd(qs.work, (unsigned long long)n);   // an attempt over n levels
    if (fresh) {
      if (qs.work && lane == 0) atomicAdd(qs.work + 1, (unsigned long long)n);
      // hydraulic properties (mf_refresh, :1280-1308)
      double s2 = 0.0;
      if (lv) {
        const double vwc = jl_div(jl_max(liq, 1.0e-6), dzv * DENH2O);
        s2 = jl_div(vwc, ws);
        s2 = jl_min(s2, 1.0);
        s2 = jl_max(0.01, s2);
      }
      const double s2n = __shfl_down_sync(COOP_FULL, s2, 1);
      double smp = 0.0, dsmpdw = 0.0;
      if (lv) {
        double s1 = (j == n) ? s2 : 0.5 * (s2 + s2n);
        s1 = jl_min(s1, 1.0);
        s1 = jl_max(0.01, s1);
        const double hkv = imp * hksat * cm_pow(s1, 2.0 * bsw + 3.0);
        const double dhkds = jl_div((2.0 * bsw + 3.0) * hkv, s1);
        const double smpv = -sucsat * cm_pow(s2, -bsw);
        const double dsmpds = jl_div(-bsw * smpv, s2);
        hk = hkv;
        smp = smpv;
        dhkdw = dhkds;
        dsmpdw = jl_div(dsmpds, ws);
        if (orec) {
          orec[PC_SMP * nlevsoi + j - 1] = smpv;
          orec[PC_HK * nlevsoi + j - 1] = hkv;
        } else {
          LV(f.smp_l, c, j, ld) = smpv;
          LV(f.hk_l, c, j, ld) = hkv;
        }
      }
      // fluxes and derivatives (:1310-1378)
      const double smpn = __shfl_down_sync(COOP_FULL, smp, 1);
      const double wsn = __shfl_down_sync(COOP_FULL, ws, 1);
      const double dsmpdwn = __shfl_down_sync(COOP_FULL, dsmpdw, 1);
      qin = qout = dqidw0 = dqidw1 = dqodw1 = dqodw2 = 0.0;
      if (lv && j <= n - 1) {
        const double dhkds1 = jl_div(0.5 * dhkdw, ws);
        const double dhkds2 = jl_div(0.5 * dhkdw, wsn);
        const double num = smpn - smp;
        const double den = M_TO_MM * (zj1 - zj);
        qout = jl_div(-hk * num, den) + hk;
        dqodw1 = jl_div(hk * dsmpdw - dhkds1 * num, den) + dhkds1;
        dqodw2 = jl_div(-hk * dsmpdwn - dhkds2 * num, den) + dhkds2;
      } else if (lv && j == n) {
        if (lower_bc == CLMGB_BC_WATERTABLE) {
          int jwt = nlevsoi;
          for (int jj = 1; jj <= nlevsoi; jj++) {
            if (f.zwt[c] <= LVc(f.zi, c, joff_zi + jj, ld)) {
              jwt = jj - 1;
              break;
            }
          }
          if (j > jwt) {
            qout = 0.0;
            dqodw1 = 0.0;
            dqodw2 = 0.0;
          } else {
            const double dhkds1l = jl_div(dhkdw, ws);
            const double num = -smp;
            const double den = M_TO_MM * (f.zwt[c] - zj);
            qout = jl_div(-hk * num, den) + hk;
            dqodw1 = jl_div(hk * dsmpdw - dhkds1l * num, den) + dhkds1l;
            dqodw2 = 0.0;
          }
        } else if (lower_bc == CLMGB_BC_FLUX) {
          qout = hk;
          dqodw1 = jl_div(dhkdw, ws);
        } else {
          qout = 0.0;
          dqodw1 = 0.0;
        }
      }
      const double qoutp = __shfl_up_sync(COOP_FULL, qout, 1);
      const double dqodw1p = __shfl_up_sync(COOP_FULL, dqodw1, 1);
      const double dqodw2p = __shfl_up_sync(COOP_FULL, dqodw2, 1);
      if (lv && j >= 2) {
        qin = qoutp;
        dqidw0 = dqodw1p;
        dqidw1 = dqodw2p;
      }
      if (j == 1) {
        qin = f.qflx_infl[c];
        dqidw1 = 0.0;
      }
      fnet1 = lv ? qin - qout - root : 0.0;
      fresh = false;
    }
    // matrix entries (:1380-1397) and the Thomas sweeps (:1421-1438), level by level
    const double amx = dqidw0 * dt_dz;
    const double bmx = -1.0 - (-dqidw1 + dqodw1) * dt_dz;
    const double cmx = (j != n) ? -dqodw2 * dt_dz : 0.0;
    const double rmx = -fnet1 * dt_dz;
    double bet = coop_bcast(bmx, 0);
    if (abs_lt(bet, 1.0e-30)) bet = 1.0e-30;
    double dwat_prev = jl_div(coop_bcast(rmx, 0), bet);
    if (lane == 0) dwat = dwat_prev;
    double cmx_prev = coop_bcast(-dqodw2 * dt_dz, 0);
    for (int i = 2; i <= n; i++) {
      const double a_i = coop_bcast(amx, i - 1), b_i = coop_bcast(bmx, i - 1), c_i = coop_bcast(cmx, i - 1);
      const double r_i = coop_bcast(rmx, i - 1);
      const double g = jl_div(cmx_prev, bet);
      bet = b_i - a_i * g;
      if (abs_lt(bet, 1.0e-30)) bet = copysign(1.0e-30, bet == 0.0 ? 1.0 : bet);
      dwat_prev = jl_div(r_i - a_i * dwat_prev, bet);
      if (lane == i - 1) {
        gam = g;
        dwat = dwat_prev;
      }
      cmx_prev = c_i;
    }
    {
      double dwat_next = dwat_prev;
      for (int i = n - 1; i >= 1; i--) {
        const double gn = coop_bcast(gam, i);          // gam of level i+1
        const double di = coop_bcast(dwat, i - 1);
        dwat_next = di - gn * dwat_next;
        if (lane == i - 1) dwat = dwat_next;
      }
    }
    // error estimate (:1440-1457)
    double ev = 0.0;
    {
      const double dwp = __shfl_up_sync(COOP_FULL, dwat, 1);
      const double dwn = __shfl_down_sync(COOP_FULL, dwat, 1);
      if (lv) {
        double fnet0;
        if (expensive) {
          const double qin_test = j == 1 ? qin + dqidw1 * dwat : qin + dqidw0 * dwp + dqidw1 * dwat;
          const double qout_test = j == n ? qout + dqodw1 * dwat : qout + dqodw1 * dwat + dqodw2 * dwn;
          fnet0 = qin_test - qout_test - root;
        } else {
          fnet0 = jl_div(dwat, dt_dz);
        }
        ev = fabs(fnet1 - fnet0) * dtsub * 0.5;
      }
    }
    const double errorMax = coop_jl_max(ev);
    // reject (:1460-1463)
    if (errorMax > cfg.xTolerUpper && dtsub > cfg.dtmin) {
      dtsub = jl_max(dtsub / 2.0, cfg.dtmin);
      continue;
    }
    // accept (:1466-1483)
    if (lv) liq = liq + dwat * (M_TO_MM * dzv);
    fresh = true;
    double qcTemp;
    if (lower_bc == CLMGB_BC_FLUX) qcTemp = coop_bcast(hk, n - 1) + coop_bcast(dhkdw, n - 1) * coop_bcast(dwat, n - 1);
    else if (lower_bc == CLMGB_BC_ZERO_FLUX) qcTemp = 0.0;
    else qcTemp = coop_bcast(qout, n - 1) + coop_bcast(dqodw1, n - 1) * coop_bcast(dwat, n - 1);
    qc += qcTemp * (dtsub / dtime);
    dtdone += dtsub;
    if (fabs(dtime - dtdone) < cfg.verySmall) break;
    double nd = dtsub;
    if (errorMax < cfg.xTolerLower) nd = dtsub * 2.0;
    dtsub = jl_min(nd, dtime - dtdone);
  }
  // mf_end
  if (lv) {
    if (orec) orec[PC_LIQ * nlevsoi + j - 1] = liq;
    else LV(f.h2osoi_liq, c, joff + j, ld) = liq;
  }
  if (__any_sync(COOP_FULL, lv && !isfinite(liq))) status |= CLMGB_COL_NONFINITE;
  if (lane == 0) {
    f.qcharge[c] = qc;
    f.num_substeps[c] = (double)nsub;
    if (col_status) col_status[c] = or_status ? (col_status[c] | status) : status;
    if (status && dev_status) atomicOr(dev_status, status);
  }
}

// Takes deferred columns until none is published and unclaimed, and finishes each;
// called by a whole warp whose lanes have no work left.  A slot is claimed only
// below the published count; its column index may still be in flight from the
// lane that deferred it (which has already claimed the slot and stores it next), so
// the wait for it is short, and bounded (qs.poll_limit polls): past the limit the
// drain gives the slot back with an atomic exchange, the deferring lane then finds it
// given back and finishes the column itself (coop_defer), and CLMGB_COL_QUEUE_WAIT is
// raised in the device status to record that the slow path ran.  Results do not
// depend on which warp finishes a column.
__device__ __forceinline__ void coop_drain(const Dims& D, const clmgb_soilwater_fields& f, const clmgb_swm_config& cfg,
                                           double dtime, uint32_t* col_status, int or_status, uint32_t* dev_status,
                                           const QueueScratch& qs) {
  const int lane = threadIdx.x & 31;
  unsigned long long* published = qs.d_count + 1;
  unsigned long long* consumed = qs.d_count + 2;
  // test hook (CLMGB_OPT_QUEUE_PUBLISH_DELAY > 0): a warp with nothing to take keeps
  // looking for up to that many ns, so that it is there to take a slot published before
  // its index; 0 in production (the warp leaves at once)
  int linger = qs.publish_delay;
  for (;;) {
    long long got = -1;
    int pending = 0;
    if (lane == 0) {
      unsigned long long k = *(volatile unsigned long long*)consumed;
      for (;;) {
        const unsigned long long p = *(volatile unsigned long long*)published;
        if (k >= p) break;
        const unsigned long long old = atomicCAS(consumed, k, k + 1);
        if (old == k) {
          got = (long long)k;
          break;
        }
        k = old;
      }
      if (got < 0 && linger > 0) pending = 1;
    }
    got = __shfl_sync(COOP_FULL, got, 0);
    pending = __shfl_sync(COOP_FULL, pending, 0);
    if (got < 0) {
      if (!pending) return;
      __nanosleep(500);
      linger -= 500;
      continue;
    }
    uint32_t cidx = DEFER_EMPTY;
    if (lane == 0) {
      for (int it = 0; it < qs.poll_limit; it++) {
        cidx = *(volatile uint32_t*)(qs.d_list + got);
        if (cidx != DEFER_EMPTY) break;
        __nanosleep(64);
      }
      if (cidx == DEFER_EMPTY) {
        // give the slot back, unless the index arrived meanwhile
        cidx = atomicExch(qs.d_list + got, DEFER_GIVEN_BACK);
        if (cidx == DEFER_EMPTY && dev_status) atomicOr(dev_status, CLMGB_COL_QUEUE_WAIT);
      }
      __threadfence();
    }
    cidx = __shfl_sync(COOP_FULL, cidx, 0);
    if (cidx == DEFER_EMPTY) continue;
    coop_finish_column(D, f, cfg, dtime, col_status, or_status, dev_status, qs, (int64_t)cidx);
  }
}

}  // namespace clmgb
