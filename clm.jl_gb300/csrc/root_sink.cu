// root_sink.cu — compute_effec_rootfrac_and_vert_tran_sink! (soil_water_plant_sink.jl),
// the transpiration sink qflx_rootsoi that the Richards solve reads.
//
// One thread per hydrology column; a column owns a contiguous patch range
// [patchi, patchi + npatches - 1], so the patch sums are sequential per thread in
// patch order, as in the reference kernels (no atomics), and the results are the
// reference's bits.  The three filters of the wrapper (:341-451) become a per-column
// choice of method, in the wrapper's order: pervious roads, then non-natural
// columns, then natural vegetation.
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int RS_BLOCK = 128;
constexpr int VEGWP_ROOT = 4;    // root segment of vegwp (soil_water_plant_sink.jl:277)

// _plantsink_default_kernel! (:48-78): transpiration-weighted column root fraction
// and the vertical sink
__device__ void rootsink_default(const clmgb_rootsink_fields& f, int64_t c, int nlevsoi, int64_t ldc, int64_t ldp) {
  const int64_t p_lo = f.col_patchi[c] - 1;
  const int64_t p_hi = p_lo + f.col_npatches[c] - 1;
  double temp_c = 0.0;
  for (int64_t p = p_lo; p <= p_hi; p++)
    if (f.patch_active[p]) temp_c += f.qflx_tran_veg_patch[p] * f.patch_wtcol[p];
  for (int j = 1; j <= nlevsoi; j++) {
    double acc = 0.0;
    for (int64_t p = p_lo; p <= p_hi; p++)
      if (f.patch_active[p]) acc += LVc(f.rootr_patch, p, j, ldp) * f.qflx_tran_veg_patch[p] * f.patch_wtcol[p];
    if (temp_c != 0.0) acc /= temp_c;
    LV(f.rootr_col, c, j, ldc) = acc;
    LV(f.qflx_rootsoi_col, c, j, ldc) = acc * f.qflx_tran_veg_col[c];
  }
}

// _plantsink_hydstress_kernel! (:210-245): flux from the soil-root conductance and the
// water-potential difference; the negative part is hydraulic redistribution
__device__ void rootsink_hydstress(const clmgb_rootsink_fields& f, int64_t c, int nlevsno, int nlevsoi, int64_t ldc,
                                   int64_t ldp) {
  const int64_t p_lo = f.col_patchi[c] - 1;
  const int64_t p_hi = p_lo + f.col_npatches[c] - 1;
  double phs_neg = 0.0;
  for (int j = 1; j <= nlevsoi; j++) {
    const double grav2 = LVc(f.z, c, j + nlevsno, ldc) * 1000.0;
    double temp_c = 0.0;
    for (int64_t p = p_lo; p <= p_hi; p++) {
      if (j == 1) f.qflx_hydr_redist_patch[p] = 0.0;
      if (f.patch_active[p] && f.frac_veg_nosno[p] > 0) {
        const double wt = f.patch_wtcol[p];
        if (wt > 0.0) {
          const double patchflux = LVc(f.k_soil_root_patch, p, j, ldp) *
                                   (LVc(f.smp_l, c, j, ldc) - LVc(f.vegwp_patch, p, VEGWP_ROOT, ldp) - grav2);
          if (patchflux < 0.0) f.qflx_hydr_redist_patch[p] += patchflux;
          temp_c += patchflux * wt;
        }
      }
    }
    LV(f.qflx_rootsoi_col, c, j, ldc) = temp_c;
    if (temp_c < 0.0) phs_neg += temp_c;
  }
  f.qflx_phs_neg_col[c] = phs_neg;
}

__global__ void __launch_bounds__(RS_BLOCK)
k_rootsink(int64_t nc, int64_t np, int64_t nl, int nlevsno, int nlevsoi, int64_t ldc, int64_t ldp,
           clmgb_rootsink_fields f, int hydrstress, uint32_t* col_status, uint32_t* dev_status) {
  const int64_t c = (int64_t)blockIdx.x * RS_BLOCK + threadIdx.x;
  if (c >= nc) return;
  uint32_t st = 0;
  if (f.mask_hydrology[c]) {
    const int64_t pi = f.col_patchi[c], npc = f.col_npatches[c], l = f.col_landunit[c];
    if (pi < 1 || npc < 0 || pi - 1 + npc > np || l < 1 || l > nl) st = CLMGB_COL_PATCH_RANGE;
  }
  if (f.mask_hydrology[c] && !st) {
    const bool road = f.col_itype[c] == ICOL_ROAD_PERV;
    const bool natveg = f.lun_itype[f.col_landunit[c] - 1] == ISTSOIL;
    // 1) pervious roads: the default algorithm under either method
    if (road) rootsink_default(f, c, nlevsoi, ldc, ldp);
    // 2) neither pervious road nor natural vegetation; 3) natural vegetation
    if ((!road && !natveg) || natveg) {
      if (hydrstress) rootsink_hydstress(f, c, nlevsno, nlevsoi, ldc, ldp);
      else rootsink_default(f, c, nlevsoi, ldc, ldp);
    }
    if (road && natveg) st = CLMGB_COL_FILTER;
  }
  if (col_status) col_status[c] = st;
  if (st && dev_status) atomicOr(dev_status, st);
}

}  // namespace

cudaError_t launch_rootsink(const Dims& D, int64_t nc, int64_t nl, const clmgb_rootsink_fields& f, int hydrstress,
                            uint32_t* col_status, uint32_t* dev_status, cudaStream_t s) {
  k_rootsink<<<(unsigned int)((nc + RS_BLOCK - 1) / RS_BLOCK), RS_BLOCK, 0, s>>>(
      nc, D.np, nl, D.nlevsno, D.nlevsoi, D.ldc, D.ldp, f, hydrstress, col_status, dev_status);
  return cudaGetLastError();
}

}  // namespace clmgb
