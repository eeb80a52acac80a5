// balance.cu — energy and water balance residuals of a column step.
//
// The reference checks every step (balance_check.jl) that the soil/snow column
// conserves energy and water.  For the quantities this path changes:
//
//   energy (soil_fluxes.jl:321-328 eflx_soil_grnd, :380-447 errsoi):
//     eflx_soil_grnd = (1-fsno) sabg_soil + fsno sabg_snow + dlrad
//                      + (1-frac_veg_nosno) emg forc_lwrad - emg SB lw_grnd
//                      - emg SB t_grnd0^3 (4 tinc) - (eflx_sh_grnd + qflx_evap_soi htvp)
//       lw_grnd = fsno t_ssbef[top]^4 + (1-fsno-fh) t_ssbef[1]^4 + fh t_h2osfc_bef^4,
//       tinc = t_grnd - t_grnd0 (ground temperature after minus before the step)
//     errsoi = sum over the column's patches (weight wtcol) of
//              eflx_soil_grnd - xmf - xmf_h2osfc - fh (t_h2osfc - t_h2osfc_bef) c_h2osfc/dtime
//              + eflx_h2osfc_to_snow - sum_snow fsno (T - t_ssbef)/fact - sum_soil (T - t_ssbef)/fact
//
//   water (balance_check.jl:741-768, errh2o, restricted to this path's fluxes):
//     errh2o = storage_end - storage_begin - (qflx_infl - sum_j qflx_rootsoi_j - qcharge) dtime
//     storage = liquid + ice of the active snow and ground levels + h2osfc +
//               h2osno_no_layers (phase change moves water between these)
//
// k_balance_begin records t_grnd0 and the storage before the step; the step itself
// records t_ssbef and t_h2osfc_bef.  x^4 is Julia's Float64 power (jl_pow4), x^3
// the product x*x*x, as Julia lowers these literal powers.
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

__device__ __forceinline__ double column_storage(const Dims& D, const clmgb_soiltemp_fields& f, int64_t c) {
  const int64_t ld = D.ldc;
  const int64_t snl = f.col_snl[c];
  double w = 0.0;
  for (int jj = (int)snl + 1 + D.nlevsno; jj <= D.nlevsno + D.nlevgrnd; jj++)
    w += LV(f.h2osoi_liq, c, jj, ld) + LV(f.h2osoi_ice, c, jj, ld);
  return w + f.h2osfc[c] + f.h2osno_no_layers[c];
}

__global__ void k_balance_begin(Dims D, int64_t nc, clmgb_soiltemp_fields f, double* t_grnd0, double* begwb) {
  const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
  if (c >= nc) return;
  t_grnd0[c] = f.t_grnd[c];
  const int64_t snl = f.col_snl[c];
  begwb[c] = (snl > 0 || snl < -D.nlevsno) ? 0.0 : column_storage(D, f, c);
}

__global__ void k_balance_residuals(Dims D, int64_t nc, clmgb_soiltemp_fields ft, clmgb_soilwater_fields fw,
                                    double dtime, const double* t_ssbef, const double* t_h2osfc_bef,
                                    const double* t_grnd0, const double* begwb, double* errsoi, double* errh2o) {
  const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
  if (c >= nc) return;
  const int64_t ld = D.ldc;
  const int nlevsno = D.nlevsno;
  const int64_t snl = ft.col_snl[c];
  double es = 0.0, eh = 0.0;
  if (snl <= 0 && snl >= -nlevsno) {
    const int64_t l = ft.col_landunit[c] - 1;
    const int64_t it = ft.col_itype[c];
    const bool urban = ft.lun_urbpoi[l] || is_wallroof(it) || it == ICOL_ROAD_IMPERV || it == ICOL_ROAD_PERV;
    if (ft.mask_nolakec[c] && !urban) {
      const double fsno = ft.frac_sno_eff[c], fh = ft.frac_h2osfc[c];
      const double eg = ft.emg[c];
      const double tg0 = t_grnd0[c];
      const double tinc = ft.t_grnd[c] - tg0;
      const double lw_grnd = fsno * jl_pow4(LVc(t_ssbef, c, (int)snl + 1 + nlevsno, ld)) +
                             (1.0 - fsno - fh) * jl_pow4(LVc(t_ssbef, c, 1 + nlevsno, ld)) +
                             fh * jl_pow4(t_h2osfc_bef[c]);
      for (int64_t p1 = ft.col_patchi[c]; p1 <= ft.col_patchf[c]; p1++) {
        const int64_t p = p1 - 1;
        if (p < 0 || p >= D.np || ft.patch_column[p] != c + 1 + D.c0 || !ft.mask_nolakep[p]) continue;
        const double gs = ((1.0 - fsno) * ft.sabg_soil[p] + fsno * ft.sabg_snow[p]) + ft.dlrad[p] +
                          (1.0 - (double)ft.frac_veg_nosno[p]) * eg * ft.forc_lwrad[c] - eg * SB * lw_grnd -
                          eg * SB * (tg0 * tg0 * tg0) * (4.0 * tinc) -
                          (ft.eflx_sh_grnd[p] + ft.qflx_evap_soi[p] * ft.htvp[c]);
        double e = gs - ft.xmf[c] - ft.xmf_h2osfc[c] -
                   fh * (ft.t_h2osfc[c] - t_h2osfc_bef[c]) * (ft.c_h2osfc[c] / dtime);
        e += ft.eflx_h2osfc_to_snow[c];
        for (int j = (int)snl + 1; j <= D.nlevgrnd; j++) {
          const int jj = j + nlevsno;
          const double d = (LV(ft.t_soisno, c, jj, ld) - LVc(t_ssbef, c, jj, ld)) / LV(ft.fact, c, jj, ld);
          if (j < 1) e -= fsno * d;
          else e -= d;
        }
        es += e * ft.patch_wtcol[p];
      }
    }
    if (fw.mask_hydrology[c]) {
      double sink = 0.0;
      const int64_t nl = fw.col_nbedrock[c];
      for (int j = 1; j <= nl && j <= D.nlevsoi; j++) sink += LVc(fw.qflx_rootsoi, c, j, ld);
      eh = column_storage(D, ft, c) - begwb[c] - (fw.qflx_infl[c] - sink - fw.qcharge[c]) * dtime;
    }
  }
  errsoi[c] = es;
  errh2o[c] = eh;
}

cudaError_t launch_balance_begin(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double* t_grnd0,
                                 double* begwb, cudaStream_t s) {
  k_balance_begin<<<(unsigned int)((nc + 127) / 128), 128, 0, s>>>(D, nc, f, t_grnd0, begwb);
  return cudaGetLastError();
}

cudaError_t launch_balance_residuals(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                     const clmgb_soilwater_fields& fw, double dtime, const double* t_ssbef,
                                     const double* t_h2osfc_bef, const double* t_grnd0, const double* begwb,
                                     double* errsoi, double* errh2o, cudaStream_t s) {
  k_balance_residuals<<<(unsigned int)((nc + 127) / 128), 128, 0, s>>>(D, nc, ft, fw, dtime, t_ssbef, t_h2osfc_bef,
                                                                      t_grnd0, begwb, errsoi, errh2o);
  return cudaGetLastError();
}

// ---- balance_check!'s column checks (balance_check.jl:723-770, 1124-1160, 1347-1365) ----
// Maxima of |x| are reduced with integer atomics on the bits of |x| (non-negative doubles
// order as their bit patterns; NaN is canonicalised above +Inf, as Julia's findmax ranks
// it), then a second pass takes the first column holding the maximum.
namespace {

constexpr int CB_BLOCK = 256;
constexpr int64_t ICOL_SUNWALL_ = 72, ICOL_SHADEWALL_ = 73;

__device__ __forceinline__ unsigned long long abs_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  return b > 0x7ff0000000000000ULL ? 0x7ff8000000000000ULL : b;
}

__global__ void k_colbalance_init(unsigned long long* r) {
  if (threadIdx.x < 5) r[threadIdx.x] = (threadIdx.x == 0 || threadIdx.x == 3) ? 0ULL : ~0ULL;
}

__global__ void __launch_bounds__(CB_BLOCK)
k_colbalance(int64_t nc, clmgb_colbalance_fields f, double dtime, unsigned long long* r) {
  const int64_t c = (int64_t)blockIdx.x * CB_BLOCK + threadIdx.x;
  if (c >= nc) return;
  double e = 0.0;
  if (f.col_active[c]) {
    const bool wall = f.col_itype[c] == ICOL_SUNWALL_ || f.col_itype[c] == ICOL_SHADEWALL_;
    const double rain = wall ? 0.0 : f.forc_rain[c], snow = wall ? 0.0 : f.forc_snow[c];
    e = f.endwb[c] - f.begwb[c] -
        (rain + snow + f.qflx_flood[c] + f.qflx_sfc_irrig[c] + f.qflx_glcice_dyn_water_flux[c] -
         f.qflx_evap_tot[c] - f.qflx_surf[c] - f.qflx_qrgwl[c] - f.qflx_drain[c] - f.qflx_drain_perched[c] -
         f.qflx_ice_runoff[c] - f.qflx_snwcp_discarded_liq[c] - f.qflx_snwcp_discarded_ice[c]) *
            dtime;
  }
  f.errh2o[c] = e;
  atomicMax(&r[0], abs_key(e));
  if (!isfinite(e)) atomicMin(&r[2], (unsigned long long)(c + 1));
  if (f.errsoi) atomicMax(&r[3], f.col_active[c] ? abs_key(f.errsoi[c]) : 0ULL);
}

__global__ void __launch_bounds__(CB_BLOCK)
k_colbalance_index(int64_t nc, clmgb_colbalance_fields f, unsigned long long* r) {
  const int64_t c = (int64_t)blockIdx.x * CB_BLOCK + threadIdx.x;
  if (c >= nc) return;
  if (abs_key(f.errh2o[c]) == r[0]) atomicMin(&r[1], (unsigned long long)(c + 1));
  if (f.errsoi && (f.col_active[c] ? abs_key(f.errsoi[c]) : 0ULL) == r[3]) atomicMin(&r[4], (unsigned long long)(c + 1));
}

}  // namespace

cudaError_t launch_colbalance(int64_t nc, const clmgb_colbalance_fields& f, double dtime, unsigned long long* r,
                              cudaStream_t s) {
  // r: max key, first index, first non-finite index, errsoi max key, errsoi first index
  k_colbalance_init<<<1, 32, 0, s>>>(r);
  const unsigned int grid = (unsigned int)((nc + CB_BLOCK - 1) / CB_BLOCK);
  k_colbalance<<<grid, CB_BLOCK, 0, s>>>(nc, f, dtime, r);
  k_colbalance_index<<<grid, CB_BLOCK, 0, s>>>(nc, f, r);
  return cudaGetLastError();
}

}  // namespace clmgb
