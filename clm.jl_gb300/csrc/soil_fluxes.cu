// soil_fluxes.cu — soil_fluxes! (soil_fluxes.jl:553-697): surface fluxes corrected to
// the ground temperature the soil/snow solve produced, the partition and limit of
// evaporation from the top layer, flux totals, outgoing longwave and the soil energy
// balance error errsoi.
//
// Every loop of the reference but the patch-to-column average touches one patch and
// reads its column, so one thread per patch runs them in the reference's order:
// soilflux_correct! (:51-76), partition (:181-240), evaporation limit (:242-300),
// totals (:303-378), errsoi base and layers (:380-453), longwave (:455-497) and the
// urban t_skin (:526-534).  The column quantities t_grnd0 and tinc (:19-41) are formed
// by each patch from its column (the same operations, so the same bits), which needs
// no scratch.  A second launch forms errsoi_col as the wtcol-weighted sum of the
// column's patches in ascending patch order (the reference's p2c, :499-524, whose CPU
// backend adds in that order).
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int SF_BLOCK = 128;
constexpr double HVAP = 2.501e6;

// t_grnd0 and tinc of column c (_soilflux_tinc_kernel!, :19-41); zero outside the mask
__device__ __forceinline__ void column_tinc(const clmgb_soilflux_fields& f, int64_t c, int nlevsno, int64_t ld,
                                            double& tinc, double& tg0) {
  tinc = 0.0;
  tg0 = 0.0;
  if (!f.mask_nolakec[c]) return;
  const int64_t snl = f.col_snl[c];
  const double fse = f.frac_sno_eff[c], fh = f.frac_h2osfc[c];
  if (snl < 0)
    tg0 = fse * LVc(f.t_ssbef, c, (int)snl + 1 + nlevsno, ld) + (1.0 - fse - fh) * LVc(f.t_ssbef, c, 1 + nlevsno, ld) +
          fh * f.t_h2osfc_bef[c];
  else
    tg0 = (1.0 - fh) * LVc(f.t_ssbef, c, 1 + nlevsno, ld) + fh * f.t_h2osfc_bef[c];
  tinc = f.t_grnd[c] - tg0;
}

__global__ void __launch_bounds__(SF_BLOCK)
k_soil_fluxes_patch(Dims D, int64_t nc, int64_t np, int64_t nl, clmgb_soilflux_fields f, double dtime,
                    uint32_t* dev_status) {
  const int64_t p = (int64_t)blockIdx.x * SF_BLOCK + threadIdx.x;
  if (p >= np) return;
  if (!f.mask_nolakep[p] && !f.mask_urbanp[p]) return;
  const int64_t ld = D.ldc;
  const int nlevsno = D.nlevsno;
  const int64_t c = f.patch_column[p] - 1, l = f.patch_landunit[p] - 1;
  if (c < 0 || c >= nc || l < 0 || l >= nl) {
    if (dev_status) atomicOr(dev_status, CLMGB_COL_PATCH_RANGE);
    return;
  }
  const int64_t snl = f.col_snl[c];
  if (snl > 0 || snl < -nlevsno) {
    if (dev_status) atomicOr(dev_status, CLMGB_COL_LEVEL_RANGE);
    return;
  }
  double tinc, tg0;
  column_tinc(f, c, nlevsno, ld, tinc, tg0);
  const bool urb = f.lun_urbpoi[l] != 0;
  const int64_t lit = f.lun_itype[l];
  const int64_t it = f.col_itype[c];
  const bool wallroof = is_wallroof(it);
  const double fse = f.frac_sno_eff[c], fh = f.frac_h2osfc[c];
  const double htvp = f.htvp[c];
  const int j = (int)snl + 1;
  const int jj = j + nlevsno;
  double eflx_lwrad_del = 0.0;
  if (f.mask_nolakep[p]) {
    // ---- Loop 2: correct the fluxes to the present soil temperature (:51-76) ----
    f.eflx_sh_grnd[p] += tinc * f.cgrnds[p];
    f.qflx_evap_soi[p] += tinc * f.cgrndl[p];
    if (urb) {
      f.qflx_ev_soil[p] = 0.0;
      f.qflx_ev_h2osfc[p] = 0.0;
      f.qflx_ev_snow[p] = f.qflx_evap_soi[p];
    } else {
      f.qflx_ev_snow[p] += tinc * f.cgrndl[p];
      f.qflx_ev_soil[p] += tinc * f.cgrndl[p];
      f.qflx_ev_h2osfc[p] += tinc * f.cgrndl[p];
    }
    // ---- Loop 3: partition evaporation into liquid and solid (:181-240) ----
    f.qflx_liqevap_from_top_layer[p] = 0.0;
    f.qflx_solidevap_from_top_layer[p] = 0.0;
    f.qflx_soliddew_to_top_layer[p] = 0.0;
    f.qflx_liqdew_to_top_layer[p] = 0.0;
    const double h2o_liq = LVc(f.h2osoi_liq, c, jj, ld);
    const double h2o_ice = LVc(f.h2osoi_ice, c, jj, ld);
    {
      const double ev = urb ? f.qflx_evap_soi[p] : f.qflx_ev_snow[p];
      if (ev >= 0.0) {
        if ((h2o_liq + h2o_ice) > 0.0)
          f.qflx_liqevap_from_top_layer[p] = jl_max(ev * (h2o_liq / (h2o_liq + h2o_ice)), 0.0);
        else
          f.qflx_liqevap_from_top_layer[p] = 0.0;
        f.qflx_solidevap_from_top_layer[p] = ev - f.qflx_liqevap_from_top_layer[p];
      } else {
        if (f.t_grnd[c] < TFRZ) f.qflx_soliddew_to_top_layer[p] = fabs(ev);
        else f.qflx_liqdew_to_top_layer[p] = fabs(ev);
      }
    }
    // ---- Loop 4: evaporation from snow limited to the available water (:242-300) ----
    if (j < 1) {
      const double evaporation_limit = (h2o_ice + h2o_liq) / (fse * dtime);
      if (f.qflx_ev_snow[p] > evaporation_limit) {
        const double evaporation_demand = f.qflx_ev_snow[p];
        f.qflx_ev_snow[p] = evaporation_limit;
        f.qflx_evap_soi[p] -= fse * (evaporation_demand - evaporation_limit);
        f.qflx_liqevap_from_top_layer[p] = jl_max(h2o_liq / (fse * dtime), 0.0);
        f.qflx_solidevap_from_top_layer[p] = jl_max(h2o_ice / (fse * dtime), 0.0);
        f.eflx_sh_grnd[p] += fse * (evaporation_demand - evaporation_limit) * htvp;
      }
    }
    if (urb && it != ICOL_ROAD_PERV && j == 1) {
      const double evaporation_limit = (h2o_ice + h2o_liq) / dtime;
      if (f.qflx_evap_soi[p] > evaporation_limit) {
        const double evaporation_demand = f.qflx_evap_soi[p];
        f.qflx_evap_soi[p] = evaporation_limit;
        f.qflx_ev_snow[p] = f.qflx_evap_soi[p];
        f.qflx_liqevap_from_top_layer[p] = jl_max(h2o_liq / dtime, 0.0);
        f.qflx_solidevap_from_top_layer[p] = jl_max(h2o_ice / dtime, 0.0);
        f.eflx_sh_grnd[p] += (evaporation_demand - evaporation_limit) * htvp;
      }
    }
    if (j == 1 && fh < 1.0) {
      const double evaporation_limit = h2o_ice / (dtime * (1.0 - fh));
      if (f.qflx_solidevap_from_top_layer[p] >= evaporation_limit) {
        const double evaporation_demand = f.qflx_solidevap_from_top_layer[p];
        f.qflx_solidevap_from_top_layer[p] = evaporation_limit;
        f.qflx_liqevap_from_top_layer[p] += (evaporation_demand - evaporation_limit);
      }
    }
    // ---- Loop 5: ground heat flux and totals (:303-378) ----
    const double emg = f.emg[c];
    const double fvn = (double)f.frac_veg_nosno[p];
    if (!urb) {
      const double lw_grnd = fse * jl_pow4(LVc(f.t_ssbef, c, jj, ld)) +
                             (1.0 - fse - fh) * jl_pow4(LVc(f.t_ssbef, c, 1 + nlevsno, ld)) +
                             fh * jl_pow4(f.t_h2osfc_bef[c]);
      f.eflx_soil_grnd[p] = ((1.0 - fse) * f.sabg_soil[p] + fse * f.sabg_snow[p]) + f.dlrad[p] +
                            (1.0 - fvn) * emg * f.forc_lwrad[c] - emg * SB * lw_grnd -
                            emg * SB * (tg0 * tg0 * tg0) * (4.0 * tinc) -
                            (f.eflx_sh_grnd[p] + f.qflx_evap_soi[p] * htvp);
      if (lit == ISTSOIL || lit == ISTCROP) f.eflx_soil_grnd_r[p] = f.eflx_soil_grnd[p];
    } else {
      eflx_lwrad_del = 4.0 * emg * SB * (tg0 * tg0 * tg0) * tinc;
      f.eflx_soil_grnd[p] = f.sabg[p] + f.dlrad[p] - f.eflx_lwrad_net[p] - eflx_lwrad_del -
                            (f.eflx_sh_grnd[p] + f.qflx_evap_soi[p] * htvp + f.qflx_tran_veg[p] * HVAP) +
                            f.eflx_wasteheat[p] + f.eflx_heat_from_ac[p] + f.eflx_traffic[p] + f.eflx_ventilation[p];
      f.eflx_soil_grnd_u[p] = f.eflx_soil_grnd[p];
    }
    f.eflx_sh_tot[p] = f.eflx_sh_veg[p] + f.eflx_sh_grnd[p];
    if (!urb) f.eflx_sh_tot[p] += f.eflx_sh_stem[p];
    f.qflx_evap_tot[p] = f.qflx_evap_veg[p] + f.qflx_evap_soi[p];
    f.eflx_lh_tot[p] = HVAP * f.qflx_evap_veg[p] + htvp * f.qflx_evap_soi[p];
    if (lit == ISTSOIL || lit == ISTCROP) {
      f.eflx_lh_tot_r[p] = f.eflx_lh_tot[p];
      f.eflx_sh_tot_r[p] = f.eflx_sh_tot[p];
    } else if (urb) {
      f.eflx_lh_tot_u[p] = f.eflx_lh_tot[p];
      f.eflx_sh_tot_u[p] = f.eflx_sh_tot[p];
    }
    f.qflx_evap_can[p] = f.qflx_evap_veg[p] - f.qflx_tran_veg[p];
    f.eflx_lh_vege[p] = (f.qflx_evap_veg[p] - f.qflx_tran_veg[p]) * HVAP;
    f.eflx_lh_vegt[p] = f.qflx_tran_veg[p] * HVAP;
    f.eflx_lh_grnd[p] = f.qflx_evap_soi[p] * htvp;
    // ---- Loop 6: soil energy balance error, base (:380-407) ----
    double e = f.eflx_soil_grnd[p] - f.xmf[c] - f.xmf_h2osfc[c] -
               fh * (f.t_h2osfc[c] - f.t_h2osfc_bef[c]) * (f.c_h2osfc[c] / dtime);
    e += f.eflx_h2osfc_to_snow[c];
    if (wallroof) e += f.eflx_building_heat_errsoi[c];
    // layers of non-urban columns (:425-453 with is_urban = false, up to nlevgrnd)
    if (!wallroof) {
      for (int jf = -nlevsno + 1; jf <= D.nlevgrnd; jf++) {
        const int jl = jf + nlevsno;
        if (jf >= snl + 1 && jf < 1)
          e -= fse * (LVc(f.t_soisno, c, jl, ld) - LVc(f.t_ssbef, c, jl, ld)) / LVc(f.fact, c, jl, ld);
        if (jf >= 1) e -= (LVc(f.t_soisno, c, jl, ld) - LVc(f.t_ssbef, c, jl, ld)) / LVc(f.fact, c, jl, ld);
      }
    }
    f.errsoi_patch[p] = e;
  }
  // layers of urban wall and roof columns (mask_urbanp, up to nlevurb)
  if (f.mask_urbanp[p] && wallroof) {
    double e = f.errsoi_patch[p];
    for (int jf = -nlevsno + 1; jf <= D.nlevurb; jf++) {
      const int jl = jf + nlevsno;
      if (jf >= snl + 1 && jf < 1)
        e -= fse * (LVc(f.t_soisno, c, jl, ld) - LVc(f.t_ssbef, c, jl, ld)) / LVc(f.fact, c, jl, ld);
      if (jf >= 1) e -= (LVc(f.t_soisno, c, jl, ld) - LVc(f.t_ssbef, c, jl, ld)) / LVc(f.fact, c, jl, ld);
    }
    f.errsoi_patch[p] = e;
  }
  // ---- Loop 7: outgoing longwave from vegetation and ground (:455-497) ----
  if (f.mask_nolakep[p]) {
    if (!urb) {
      const double emg = f.emg[c];
      const double fvn = (double)f.frac_veg_nosno[p];
      const double lw_grnd = fse * jl_pow4(LVc(f.t_ssbef, c, jj, ld)) +
                             (1.0 - fse - fh) * jl_pow4(LVc(f.t_ssbef, c, 1 + nlevsno, ld)) +
                             fh * jl_pow4(f.t_h2osfc_bef[c]);
      f.eflx_lwrad_out[p] = f.ulrad[p] + (1.0 - fvn) * (1.0 - emg) * f.forc_lwrad[c] +
                            (1.0 - fvn) * emg * SB * lw_grnd + 4.0 * emg * SB * (tg0 * tg0 * tg0) * tinc;
      if (fvn == 0.0) f.t_skin[p] = sqrt(sqrt(lw_grnd));
      f.eflx_lwrad_net[p] = f.eflx_lwrad_out[p] - f.forc_lwrad[c];
      if (lit == ISTSOIL || lit == ISTCROP) {
        f.eflx_lwrad_net_r[p] = f.eflx_lwrad_out[p] - f.forc_lwrad[c];
        f.eflx_lwrad_out_r[p] = f.eflx_lwrad_out[p];
      }
    } else {
      f.eflx_lwrad_out[p] += eflx_lwrad_del;
      f.eflx_lwrad_net[p] += eflx_lwrad_del;
      f.eflx_lwrad_net_u[p] += eflx_lwrad_del;
      f.eflx_lwrad_out_u[p] = f.eflx_lwrad_out[p];
    }
  }
  // ---- urban t_skin from the top active layer (:526-534) ----
  if (f.mask_urbanp[p]) f.t_skin[p] = LVc(f.t_soisno, c, jj, ld);
}

// errsoi_col: wtcol-weighted sum over the column's patch range, ascending (:499-524)
__global__ void __launch_bounds__(SF_BLOCK)
k_soil_fluxes_p2c(int64_t nc, int64_t np, clmgb_soilflux_fields f, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * SF_BLOCK + threadIdx.x;
  if (c >= nc || !f.mask_nolakec[c]) return;
  const int64_t pi = f.col_patchi[c], pf = f.col_patchf[c];
  if (pi < 1 || pf > np) {
    if (dev_status) atomicOr(dev_status, CLMGB_COL_PATCH_RANGE);
    return;
  }
  double s = 0.0;
  for (int64_t p1 = pi; p1 <= pf; p1++) {
    const int64_t p = p1 - 1;
    if (f.patch_column[p] == c + 1) s += f.errsoi_patch[p] * f.patch_wtcol[p];
  }
  f.errsoi_col[c] = s;
}

}  // namespace

cudaError_t launch_soil_fluxes(const Dims& D, int64_t nc, int64_t nl, const clmgb_soilflux_fields& f, double dtime,
                               uint32_t* dev_status, cudaStream_t s) {
  if (D.np > 0) {
    k_soil_fluxes_patch<<<(unsigned int)((D.np + SF_BLOCK - 1) / SF_BLOCK), SF_BLOCK, 0, s>>>(D, nc, D.np, nl, f, dtime,
                                                                                               dev_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_soil_fluxes_p2c<<<(unsigned int)((nc + SF_BLOCK - 1) / SF_BLOCK), SF_BLOCK, 0, s>>>(nc, D.np, f, dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
