// surface_hydrology.cu — the surface hydrology clm_drv_core! runs between
// set_soil_water_fractions! and the root sink (clm_driver.jl:1938-2007): flood water,
// saturated-excess runoff, the split of surface inputs, infiltration-excess runoff,
// its routing, the surface-water store, infiltration, total surface runoff and urban
// ponding.  Their output qflx_infl is the upper boundary flux of soil_water!.
//
// Every one of those routines is a per-column update with no coupling between
// columns, so one thread per column runs the selected ones in the driver's order,
// each over its own filter.  A value a stage needs comes from a register when an
// earlier selected stage produced it for this column, otherwise from memory (the
// array the reference reads), so any subset of stages gives the bits of the
// reference's calls one after another.  The per-column footprint is ~40 words of
// [nc] vectors and 6 level values, read and written once: the kernel is bound by HBM.
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int SH_BLOCK = 128;
constexpr int64_t ISPVAL = -9999;               // varcon.jl:85
constexpr double QINMAX_UNLIMITED = 1.0e200;    // infilt_excess_runoff.jl:37

// A column value that an earlier stage may have produced in this launch.
struct Lazy {
  double v;
  bool ok;
  __device__ __forceinline__ double get(const double* p, int64_t c) {
    if (!ok) {
      v = p[c];
      ok = true;
    }
    return v;
  }
  __device__ __forceinline__ void set(double x) {
    v = x;
    ok = true;
  }
};

__global__ void __launch_bounds__(SH_BLOCK)
k_surface_hydrology(int64_t nc, int64_t nl, int nlevsno, int64_t ld, clmgb_surfhyd_fields f, clmgb_surfhyd_config P,
                    uint32_t stages, double dtime, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * SH_BLOCK + threadIdx.x;
  if (c >= nc) return;
  constexpr uint32_t HYD = CLMGB_SH_SAT_EXCESS | CLMGB_SH_QFLX_INPUTS | CLMGB_SH_INFL_EXCESS | CLMGB_SH_ROUTE |
                           CLMGB_SH_UPDATE_H2OSFC | CLMGB_SH_INFILTRATION | CLMGB_SH_TOTAL_RUNOFF;
  const bool nolake = (stages & CLMGB_SH_FLOODC) && f.mask_nolakec[c];
  const bool hyd = (stages & HYD) && f.mask_hydrology[c];
  const bool urb = (stages & (CLMGB_SH_TOTAL_RUNOFF | CLMGB_SH_URBAN_PONDING)) && f.mask_urban[c];
  if (!nolake && !hyd && !urb) return;

  // topology indices the selected stages dereference
  int64_t g = 0, l = 0;
  if (nolake) {
    g = f.col_gridcell[c];
    if (g < 1 || g > P.ng) {
      if (dev_status) atomicOr(dev_status, CLMGB_COL_PATCH_RANGE);
      return;
    }
  }
  if (hyd && (((stages & CLMGB_SH_SAT_EXCESS) && P.crop_fsat_equals_zero) || (stages & CLMGB_SH_ROUTE))) {
    l = f.col_landunit[c];
    if (l < 1 || l > nl) {
      if (dev_status) atomicOr(dev_status, CLMGB_COL_PATCH_RANGE);
      return;
    }
  }

  Lazy floodc{0.0, false}, fsat{0.0, false}, sat_surf{0.0, false}, in_soil{0.0, false}, to_h2osfc{0.0, false};
  Lazy qinmax{0.0, false}, infl_excess{0.0, false}, limited{0.0, false}, in_h2osfc{0.0, false};
  Lazy excess_surf{0.0, false}, h2osfc_surf{0.0, false}, h2osfc_drain{0.0, false}, xs_urban{0.0, false};

  // set_floodc! (soil_hydrology.jl:139-152): walls take no flood water
  if (nolake) {
    const int64_t it = f.col_itype[c];
    const double q = (it != ICOL_SUNWALL && it != ICOL_SHADEWALL) ? f.qflx_floodg[g - 1] : 0.0;
    f.qflx_floodc[c] = q;
    floodc.set(q);
  }

  // saturated_excess_runoff! (sat_excess_runoff.jl:246-300)
  if (hyd && (stages & CLMGB_SH_SAT_EXCESS)) {
    double fs;
    if (P.fsat_method == CLMGB_FSAT_TOPMODEL) {
      const double ft = f.frost_table[c], zw = f.zwt[c], zwp = f.zwt_perched[c], wt = f.wtfact[c];
      if (ft > zwp && ft <= zw) fs = wt * cm_exp(-0.5 * P.fff * zwp);     // perched water table
      else fs = wt * cm_exp(-0.5 * P.fff * zw);
    } else {                                                             // VIC (Wood et al. 1992)
      const double bi = f.b_infil[c];
      const double ex = bi / (1.0 + bi);
      fs = 1.0 - cm_pow(1.0 - f.top_moist_limited[c] / f.top_max_moist[c], ex);
    }
    if (P.crop_fsat_equals_zero && f.lun_itype[l - 1] == ISTCROP) fs = 0.0;
    if (P.hillslope_fsat_equals_zero && f.col_is_hillslope[c] && f.col_active[c] && f.col_cold[c] != ISPVAL)
      fs = 0.0;
    f.fsat[c] = fs;
    fsat.set(fs);
    double q = fs * f.qflx_rain_plus_snomelt[c];
    f.fcov[c] = fs;
    if (f.col_urbpoi[c]) q = q + floodc.get(f.qflx_floodc, c);
    f.qflx_sat_excess_surf[c] = q;
    sat_surf.set(q);
  }

  // set_qflx_inputs! (soil_hydrology.jl:160-187)
  if (hyd && (stages & CLMGB_SH_QFLX_INPUTS)) {
    const double top = f.qflx_rain_plus_snomelt[c] + f.qflx_snow_h2osfc[c] + floodc.get(f.qflx_floodc, c);
    f.qflx_top_soil[c] = top;
    double fsno, evap;
    if (f.col_snl[c] >= 0) {
      fsno = 0.0;
      evap = f.qflx_liqevap_from_top_layer[c];
    } else {
      fsno = f.frac_sno_eff[c];
      evap = f.qflx_ev_soil[c];
    }
    const double fh = f.frac_h2osfc[c];
    const double ss = sat_surf.get(f.qflx_sat_excess_surf, c);
    double qs = (1.0 - fh) * (top - ss);
    double qh = fh * (top - ss);
    qs = qs - (1.0 - fsno - fh) * evap;
    qh = qh - fh * f.qflx_ev_h2osfc[c];
    f.qflx_in_soil[c] = qs;
    f.qflx_top_soil_to_h2osfc[c] = qh;
    in_soil.set(qs);
    to_h2osfc.set(qh);
  }

  // infiltration_excess_runoff! (infilt_excess_runoff.jl:142-211) with
  // compute_qinmax_hksat! (:241-274): the smallest ice-impeded hksat of soil levels 1-3
  if (hyd && (stages & CLMGB_SH_INFL_EXCESS)) {
    double qu;
    if (P.qinmax_method == CLMGB_QINMAX_NONE) {
      qu = QINMAX_UNLIMITED;
    } else {
      qu = CM_INF;
      for (int j = 1; j <= 3; j++) {
        const double val = cm_pow(10.0, -P.e_ice * LVc(f.icefrac, c, j, ld)) * LVc(f.hksat, c, j, ld);
        if (val < qu) qu = val;
      }
    }
    const double qm = (1.0 - fsat.get(f.fsat, c)) * qu;
    const double ex = jl_max(0.0, in_soil.get(f.qflx_in_soil, c) - (1.0 - f.frac_h2osfc[c]) * qm);
    f.qinmax[c] = qm;
    f.qflx_infl_excess[c] = ex;
    qinmax.set(qm);
    infl_excess.set(ex);
  }

  // route_infiltration_excess! (soil_hydrology.jl:199-225)
  if (hyd && (stages & CLMGB_SH_ROUTE)) {
    const int64_t lt = f.lun_itype[l - 1];
    double lim, inh, exs;
    if (lt == ISTSOIL || lt == ISTCROP) {
      lim = in_soil.get(f.qflx_in_soil, c) - infl_excess.get(f.qflx_infl_excess, c);
      if (P.h2osfcflag != 0) {
        inh = to_h2osfc.get(f.qflx_top_soil_to_h2osfc, c) + infl_excess.get(f.qflx_infl_excess, c);
        exs = 0.0;
      } else {
        inh = to_h2osfc.get(f.qflx_top_soil_to_h2osfc, c);
        exs = infl_excess.get(f.qflx_infl_excess, c);
      }
    } else {
      lim = in_soil.get(f.qflx_in_soil, c);
      inh = 0.0;
      exs = 0.0;
    }
    f.qflx_in_soil_limited[c] = lim;
    f.qflx_in_h2osfc[c] = inh;
    f.qflx_infl_excess_surf[c] = exs;
    limited.set(lim);
    in_h2osfc.set(inh);
    excess_surf.set(exs);
  }

  // update_h2osfc! (surface_water.jl:462-520): runoff from the store above its
  // fill-and-spill threshold (:279-316), the inflow (:400-414), drainage into the soil
  // (:357-374) and the final state (:426-443); residuals below 1e-13 of the previous
  // storage are truncated to zero
  if (hyd && (stages & CLMGB_SH_UPDATE_H2OSFC)) {
    const double h0 = f.h2osfc[c];
    double qs = 0.0;
    if (P.update_h2osfcflag == 1) {
      const double fn = f.frac_h2osfc_nosnow[c];
      const double fic = fn <= P.pc ? 0.0 : cm_pow(fn - P.pc, P.mu);
      const double thr = f.h2osfc_thresh[c];
      double q = 0.0;
      if (h0 > thr) {
        const double k_wet = 1.0e-4 * cm_sin(CM_DEG2RAD * f.topo_slope[c]);
        q = k_wet * fic * (h0 - thr);
        q = jl_min(q, (h0 - thr) / dtime);
      }
      if (q < 1.0e-8) q = 0.0;
      qs = q;
    }
    double h1 = h0 + (in_h2osfc.get(f.qflx_in_h2osfc, c) - qs) * dtime;
    if (fabs(h1) < 1.0e-13 * fabs(h0)) h1 = 0.0;
    double qd;
    if (h1 < 0.0) {
      qd = h1 / dtime;
    } else {
      qd = jl_min(f.frac_h2osfc[c] * qinmax.get(f.qinmax, c), h1 / dtime);
      if (P.update_h2osfcflag == 0) qd = jl_max(0.0, h1 / dtime);
    }
    double h2 = h1 - qd * dtime;
    if (fabs(h2) < 1.0e-13 * fabs(h1)) h2 = 0.0;
    f.h2osfc[c] = h2;
    f.qflx_h2osfc_surf[c] = qs;
    f.qflx_h2osfc_drain[c] = qd;
    h2osfc_surf.set(qs);
    h2osfc_drain.set(qd);
  }

  // infiltration! (soil_hydrology.jl:236-243)
  if (hyd && (stages & CLMGB_SH_INFILTRATION))
    f.qflx_infl[c] = limited.get(f.qflx_in_soil_limited, c) + h2osfc_drain.get(f.qflx_h2osfc_drain, c);

  // total_surface_runoff! (soil_hydrology.jl:250-301): hydrologically active columns,
  // then the urban columns that are not (roof and impervious road pond in the top soil
  // level; walls shed nothing)
  const int topsoil = nlevsno + 1;
  if (stages & CLMGB_SH_TOTAL_RUNOFF) {
    if (hyd)
      f.qflx_surf[c] = sat_surf.get(f.qflx_sat_excess_surf, c) + excess_surf.get(f.qflx_infl_excess_surf, c) +
                       h2osfc_surf.get(f.qflx_h2osfc_surf, c);
    if (urb) {
      const int64_t it = f.col_itype[c];
      if (it == ICOL_ROOF || it == ICOL_ROAD_IMPERV) {
        double q;
        if (f.col_snl[c] < 0) {
          q = jl_max(0.0, f.qflx_rain_plus_snomelt[c]);
        } else {
          const double xs = jl_max(0.0, LV(f.h2osoi_liq, c, topsoil, ld) / dtime + f.qflx_rain_plus_snomelt[c] -
                                            f.qflx_liqevap_from_top_layer[c] - P.pondmx_urban / dtime);
          f.xs_urban[c] = xs;
          xs_urban.set(xs);
          q = xs;
        }
        f.qflx_surf[c] = q + floodc.get(f.qflx_floodc, c);
      } else if (it == ICOL_SUNWALL || it == ICOL_SHADEWALL) {
        f.qflx_surf[c] = 0.0;
      }
    }
  }

  // update_urban_ponding! (soil_hydrology.jl:316-338)
  if (urb && (stages & CLMGB_SH_URBAN_PONDING)) {
    const int64_t it = f.col_itype[c];
    if ((it == ICOL_ROOF || it == ICOL_ROAD_IMPERV) && f.col_snl[c] >= 0) {
      double& liq = LV(f.h2osoi_liq, c, topsoil, ld);
      if (xs_urban.get(f.xs_urban, c) > 0.0)
        liq = P.pondmx_urban;
      else
        liq = jl_max(0.0, liq + (f.qflx_rain_plus_snomelt[c] - f.qflx_liqevap_from_top_layer[c]) * dtime);
    }
  }
}

}  // namespace

cudaError_t launch_surface_hydrology(const Dims& D, int64_t nc, int64_t nl, const clmgb_surfhyd_fields& f,
                                     const clmgb_surfhyd_config& P, uint32_t stages, double dtime, uint32_t* dev_status,
                                     cudaStream_t s) {
  k_surface_hydrology<<<(unsigned int)((nc + SH_BLOCK - 1) / SH_BLOCK), SH_BLOCK, 0, s>>>(
      nc, nl, D.nlevsno, D.ldc, f, P, stages, dtime, dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
