// api.cu — the C ABI (include/clmgb.h): argument validation, handle, launches.
//
// Invalid arguments and configurations the reference rejects with error() are
// reported as negative return codes before anything is enqueued; there is no CPU
// fallback.  Device-side per-column conditions are OR-ed into the handle's status
// word, read back with clmgb_device_status().
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>
#include <initializer_list>
#include "clmgb_device.cuh"
#include "launch.h"
#include <nvtx3/nvToolsExt.h>

// An NVTX range around each compute entry point, so a profiler's timeline shows the
// drop-in calls by name (no cost when no tool is attached).
struct ClmgbRange {
  explicit ClmgbRange(const char* name) { nvtxRangePushA(name); }
  ~ClmgbRange() { nvtxRangePop(); }
  ClmgbRange(const ClmgbRange&) = delete;
  ClmgbRange& operator=(const ClmgbRange&) = delete;
};

#ifndef CLMGB_GIT_DESC
#define CLMGB_GIT_DESC "dev"
#endif
#define CLMGB_STR_(x) #x
#define CLMGB_XSTR(x) CLMGB_STR_(x)

struct clmgb_handle_s {
  uint32_t magic;
  int device;
  int num_sms;
  clmgb_varpar vp;
  // device scratch owned by the handle (one allocation of 12 words): the status word
  // (OR of CLMGB_COL_* bits), the Richards work-queue counter, 5 words for the
  // reductions of clmgb_balance_check_columns, 3 counters of deferred columns
  unsigned long long* scratch;
  uint32_t* dev_status;
  unsigned long long* queue;
  int64_t column_base;          // CLMGB_OPT_COLUMN_BASE
  int64_t defer;                // CLMGB_OPT_QUEUE_DEFER
  int64_t packed;               // CLMGB_OPT_QUEUE_PACKED_REFRESH
  int64_t step_schedule;        // CLMGB_OPT_STEP_SCHEDULE
  int64_t queue_blocks_per_sm;  // CLMGB_OPT_QUEUE_BLOCKS_PER_SM (0 = occupancy limit)
  int occupancy_blocks;         // occupancy limit of the queue kernel
  int64_t queue_order;          // CLMGB_OPT_QUEUE_ORDER
  // per-column scratch from clmgb_reserve (one allocation)
  void* reserve_block;
  clmgb::QueueScratch qs;
  clmgb::WaveScratch ws;
  int waves_blocks;             // co-resident blocks per SM of the wave kernel (0 = cannot launch)
  int64_t waves_blocks_per_sm;  // CLMGB_OPT_WAVES_BLOCKS_PER_SM (0 = all co-resident)
  // tape of the column-step adjoint (clmgb_reserve_adjoint, one allocation)
  void* tape_block;
  clmgb::AdjTape tape;
  int64_t adj_st_mode;          // CLMGB_OPT_ADJ_SOIL_TEMPERATURE
  int64_t fresh_batch;          // CLMGB_OPT_QUEUE_FRESH_BATCH
  int64_t attempt_cap;          // CLMGB_OPT_ATTEMPT_CAP
  int64_t poll_limit;           // CLMGB_OPT_QUEUE_POLL_LIMIT
  int64_t publish_delay;        // CLMGB_OPT_QUEUE_PUBLISH_DELAY
  int64_t count_work;           // CLMGB_OPT_COUNT_WORK (counters in scratch words 10, 11)
  int64_t records_tma;          // CLMGB_OPT_RECORDS_TMA
  int records_tma_used;         // CLMGB_OPT_RECORDS_TMA_USED
  int64_t tridiag_method;       // CLMGB_OPT_TRIDIAG_METHOD
  int64_t st_block;             // CLMGB_OPT_ST_BLOCK
  cudaError_t last_error;
};

static const uint32_t HANDLE_MAGIC = 0xC1A9B300u;
// Resident 128-thread blocks per SM of the work-queue kernel when not tuned: fewer
// resident warps give every lane more columns to balance over, and the FP64 pipe
// (about 1.9 FMA/clk/SM) stays busy with a handful of warps.  Measured on GB300 at
// 262,144 columns: 1 -> 6.8, 2 -> 7.9, 3 -> 7.5, 4 -> 7.2, occupancy limit -> 5.2
// M column-steps/s.
static const int64_t CLMGB_DEFAULT_QUEUE_BLOCKS_PER_SM = 2;
// Lanes of the work-queue kernel that batch the hydraulic block (CLMGB_OPT_QUEUE_FRESH_BATCH).
// Measured on GB300 at 262,144 columns (2 blocks/SM), Richards ms per call with the
// packed refresh: 1 -> 12.73, 2 -> 12.73, 4 -> 12.71, 8 -> 12.77, 12 -> 12.84, 20 -> 13.00
// (the per-lane refresh: 14.82 at 20, its best; 0 -> 10.16, 8 -> 10.36, 16 -> 10.47,
// 20 -> 10.54, 24 -> 10.51 M column-steps/s when it was the default).
static const int64_t CLMGB_DEFAULT_FRESH_BATCH = 4;
// Attempts after which the work-queue kernel hands a column to the warp-per-column
// finish (CLMGB_OPT_QUEUE_DEFER).  Measured on GB300 over the 100 timed steps of the
// scale workload (262,144 columns), ms per step with the packed refresh: 12 -> 29.3,
// 16 -> 19.9, 18 -> 18.6, 20 -> 17.37, 22 -> 17.23, 24 -> 17.56, 28 -> 18.93,
// 32 -> 20.5.  (Over steps 3-12 alone 28 was best: the later steps hold more long
// columns.)  Below ~20 the deferred backlog, finished at a few times the cost per
// attempt, outweighs the shorter end of the queue.
static const int64_t CLMGB_DEFAULT_QUEUE_DEFER = 22;

using clmgb::Dims;

static bool handle_ok(clmgb_handle h) { return h && h->magic == HANDLE_MAGIC; }

static int32_t cuda_fail(clmgb_handle h, cudaError_t e) {
  if (h) h->last_error = e;
  return CLMGB_ERR_CUDA;
}

static int32_t check_varpar(const clmgb_varpar* vp) {
  if (!vp) return CLMGB_ERR_NULL_ARG;
  if (vp->nlevsno < 1 || vp->nlevsno > CLMGB_MAX_NLEVSNO) return CLMGB_ERR_DIMS;
  if (vp->nlevgrnd < 2 || vp->nlevgrnd > CLMGB_MAX_NLEVGRND) return CLMGB_ERR_DIMS;
  if (vp->nlevsoi < 1 || vp->nlevsoi > vp->nlevgrnd || vp->nlevsoi > CLMGB_MAX_NLEVSOI) return CLMGB_ERR_DIMS;
  if (vp->nlevurb < 0 || vp->nlevurb > vp->nlevgrnd) return CLMGB_ERR_DIMS;
  if (vp->nlevmaxurbgrnd != vp->nlevgrnd) return CLMGB_ERR_DIMS;
  return CLMGB_OK;
}

static int32_t check_bounds(const clmgb_bounds* b, bool need_patches) {
  if (!b) return CLMGB_ERR_NULL_ARG;
  if (b->nc < 0 || b->ldc < b->nc || b->np < 0 || b->ldp < b->np || b->nl < 0) return CLMGB_ERR_DIMS;
  if (need_patches && b->nc > 0 && (b->np < 1 || b->nl < 1)) return CLMGB_ERR_DIMS;
  return CLMGB_OK;
}

static Dims make_dims(const clmgb_varpar& vp, const clmgb_bounds& b, int64_t c0 = 0, int attempt_cap = clmgb::MF_ATTEMPT_CAP) {
  Dims D;
  D.c0 = c0;
  D.attempt_cap = attempt_cap;
  D.nlevsno = vp.nlevsno;
  D.nlevgrnd = vp.nlevgrnd;
  D.nlevsoi = vp.nlevsoi;
  D.nlevurb = vp.nlevurb;
  D.nlevmax = vp.nlevmaxurbgrnd;
  D.ldc = b.ldc;
  D.ldp = b.ldp;
  D.np = b.np;
  return D;
}

static Dims hdims(clmgb_handle h, const clmgb_bounds& b) {
  Dims D = make_dims(h->vp, b, h->column_base, (int)h->attempt_cap);
  D.st_block = (int)h->st_block;
  return D;
}

// every pointer member after struct_size must be non-NULL
template <typename S>
static int32_t check_fields(const S* f) {
  if (!f) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(S)) return CLMGB_ERR_ABI;
  const char* base = reinterpret_cast<const char*>(f) + sizeof(int64_t);
  const size_t nptr = (sizeof(S) - sizeof(int64_t)) / sizeof(void*);
  for (size_t i = 0; i < nptr; i++) {
    const void* p;
    memcpy(&p, base + i * sizeof(void*), sizeof(void*));
    if (!p) return CLMGB_ERR_NULL_ARG;
  }
  return CLMGB_OK;
}

static int32_t check_cfg(const clmgb_swm_config* cfg) {
  if (!cfg) return CLMGB_ERR_NULL_ARG;
  if (cfg->soilwater_movement_method == CLMGB_ZENGDECKER_2009) return CLMGB_ERR_UNSUPPORTED;
  if (cfg->soilwater_movement_method != CLMGB_MOISTURE_FORM) return CLMGB_ERR_CONFIG;
  if (cfg->upper_boundary_condition != CLMGB_BC_FLUX) return CLMGB_ERR_CONFIG;
  // soilwm_moisture_form_solve!'s error() for any other lower boundary, BC_AQUIFER included
  // (soil_water_movement.jl:1502-1505)
  const int lb = cfg->lower_boundary_condition;
  if (!(lb == CLMGB_BC_WATERTABLE || lb == CLMGB_BC_FLUX || lb == CLMGB_BC_ZERO_FLUX)) return CLMGB_ERR_CONFIG;
  if (cfg->flux_calculation != 1 && cfg->flux_calculation != 42) return CLMGB_ERR_CONFIG;
  if (!(cfg->dtmin > 0.0)) return CLMGB_ERR_CONFIG;
  return CLMGB_OK;
}

static clmgb::QueueScratch queue_scratch(clmgb_handle h) {
  clmgb::QueueScratch q = h->qs;
  q.longest_first = h->queue_order == 1 ? 1 : 0;
  q.fresh_batch = (int)h->fresh_batch;
  // deferred columns keep their state in the wave scratch of the same reservation
  const bool have = h->ws.cap == h->qs.capacity && h->ws.cap > 0;
  q.defer = have ? (int)h->defer : 0;
  q.packed = (int)h->packed;
  q.d_liq = have ? h->ws.qout : nullptr;
  q.d_dtsub = have ? h->ws.dtsub : nullptr;
  q.d_dtdone = have ? h->ws.dtdone : nullptr;
  q.d_qc = have ? h->ws.qc : nullptr;
  q.d_nsub = have ? h->ws.nsub : nullptr;
  q.d_status = have ? h->ws.status : nullptr;
  q.d_list = have ? h->ws.listA[0] : nullptr;
  q.d_count = have ? h->scratch + 7 : nullptr;
  q.poll_limit = (int)h->poll_limit;
  q.publish_delay = (int)h->publish_delay;
  q.work = h->count_work ? h->scratch + 10 : nullptr;
  q.records_tma = (int)h->records_tma;
  q.records_tma_used = &h->records_tma_used;
  return q;
}

static bool use_waves(clmgb_handle h, int64_t nc) {
  return h->step_schedule == CLMGB_SCHEDULE_WAVES && h->waves_blocks > 0 && h->ws.cap >= nc;
}
static int waves_grid(clmgb_handle h) {
  int per_sm = h->waves_blocks_per_sm > 0 ? (int)h->waves_blocks_per_sm : h->waves_blocks;
  if (per_sm > h->waves_blocks) per_sm = h->waves_blocks;
  return per_sm * h->num_sms;
}

static int queue_grid(clmgb_handle h) {
  int per_sm = h->queue_blocks_per_sm > 0 ? (int)h->queue_blocks_per_sm : h->occupancy_blocks;
  if (per_sm > h->occupancy_blocks) per_sm = h->occupancy_blocks;
  return per_sm * h->num_sms;
}

// resident blocks of the hand-written step adjoint over the device
static int vjp_grid(clmgb_handle h) { return clmgb::vjp_cf_blocks_per_sm() * h->num_sms; }

extern "C" {

int32_t clmgb_abi_version(void) { return CLMGB_ABI_VERSION; }

const char* clmgb_build_info(void) {
  return "clmgb " CLMGB_GIT_DESC " sm_103a fp64 fmad=off (CUDA runtime " CLMGB_XSTR(CUDART_VERSION) ")";
}

const char* clmgb_strerror(int32_t code) {
  switch (code) {
    case CLMGB_OK: return "ok";
    case CLMGB_ERR_NULL_ARG: return "a required pointer is NULL";
    case CLMGB_ERR_DIMS: return "level counts or column/patch dimensions out of the supported range";
    case CLMGB_ERR_CONFIG: return "configuration rejected (the reference raises error() for it)";
    case CLMGB_ERR_UNSUPPORTED: return "configuration not implemented by this library";
    case CLMGB_ERR_CUDA: return "CUDA launch or copy failed";
    case CLMGB_ERR_ABI: return "struct size / ABI version mismatch";
    case CLMGB_ERR_HANDLE: return "invalid handle";
    default: return "unknown error";
  }
}

int32_t clmgb_create(const clmgb_varpar* vp, clmgb_handle* out) {
  if (!out) return CLMGB_ERR_NULL_ARG;
  *out = nullptr;
  int32_t e = check_varpar(vp);
  if (e) return e;
  clmgb_handle h = new clmgb_handle_s();
  h->magic = HANDLE_MAGIC;
  h->vp = *vp;
  h->last_error = cudaSuccess;
  h->column_base = 0;
  h->defer = CLMGB_DEFAULT_QUEUE_DEFER;
  h->packed = 1;
  h->records_tma = 1;
  h->st_block = 320;
  h->step_schedule = CLMGB_SCHEDULE_QUEUE;
  h->queue_blocks_per_sm = CLMGB_DEFAULT_QUEUE_BLOCKS_PER_SM;
  h->scratch = nullptr;
  h->queue_order = 1;
  h->reserve_block = nullptr;
  h->qs.capacity = 0;
  h->qs.imp = nullptr;
  h->qs.order = nullptr;
  h->qs.bins = nullptr;
  h->qs.pcache = nullptr;
  h->qs.longest_first = 1;
  h->fresh_batch = CLMGB_DEFAULT_FRESH_BATCH;
  h->attempt_cap = clmgb::MF_ATTEMPT_CAP;
  h->poll_limit = clmgb::DEFER_POLL_LIMIT;
  h->publish_delay = 0;
  h->count_work = 0;
  memset(&h->ws, 0, sizeof(h->ws));
  h->waves_blocks = 0;
  h->waves_blocks_per_sm = 0;
  cudaError_t ce = cudaGetDevice(&h->device);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (ce == cudaSuccess) ce = cudaMalloc(&h->scratch, 12 * sizeof(unsigned long long));
  if (ce == cudaSuccess) ce = cudaMemset(h->scratch, 0, 12 * sizeof(unsigned long long));
  if (ce == cudaSuccess) {
    h->dev_status = reinterpret_cast<uint32_t*>(h->scratch);
    h->queue = h->scratch + 1;
    h->occupancy_blocks = clmgb::queue_blocks_per_sm();
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device);
    h->waves_blocks = coop ? clmgb::waves_blocks_per_sm() : 0;
  }
  if (ce != cudaSuccess) {
    h->magic = 0;
    delete h;
    return CLMGB_ERR_CUDA;
  }
  *out = h;
  return CLMGB_OK;
}

int32_t clmgb_destroy(clmgb_handle h) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  cudaFree(h->scratch);
  if (h->reserve_block) cudaFree(h->reserve_block);
  if (h->tape_block) cudaFree(h->tape_block);
  h->magic = 0;
  delete h;
  return CLMGB_OK;
}

int32_t clmgb_device_status(clmgb_handle h, void* stream, uint32_t* status, int32_t reset) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!status) return CLMGB_ERR_NULL_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t v = 0;
  cudaError_t ce = cudaMemcpyAsync(&v, h->dev_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess && reset) ce = cudaMemsetAsync(h->dev_status, 0, sizeof(uint32_t), s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return cuda_fail(h, ce);
  *status = v;
  return CLMGB_OK;
}

int32_t clmgb_last_cuda_error(clmgb_handle h) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  return (int32_t)h->last_error;
}

int32_t clmgb_soil_temperature(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* f,
                               double dtime, int32_t snow_method, int32_t use_excess_ice,
                               uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_soil_temperature");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (snow_method != CLMGB_SNOW_JORDAN1991 && snow_method != CLMGB_SNOW_STURM1997) return CLMGB_ERR_CONFIG;
  if (use_excess_ice) return CLMGB_ERR_UNSUPPORTED;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce = clmgb::launch_soil_temperature(hdims(h, *b), b->nc, *f, dtime, snow_method, col_status,
                                                  h->dev_status, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_fluxes(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilflux_fields* f, double dtime,
                          void* stream) {
  const ClmgbRange range_("clmgb_soil_fluxes");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0 && b->np == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce = clmgb::launch_soil_fluxes(hdims(h, *b), b->nc, b->nl, *f, dtime, h->dev_status,
                                             (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_water_zd09(clmgb_handle h, const clmgb_bounds* b, const clmgb_zd09_fields* f,
                              const clmgb_swm_config* cfg, double dtime, void* stream) {
  const ClmgbRange range_("clmgb_soil_water_zd09");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!cfg) return CLMGB_ERR_NULL_ARG;
  // init_soilwater_movement (soil_water_movement.jl:681-698): ZD09 with the aquifer
  // lower boundary only
  if (cfg->soilwater_movement_method != CLMGB_ZENGDECKER_2009) return CLMGB_ERR_CONFIG;
  if (cfg->lower_boundary_condition != CLMGB_BC_AQUIFER) return CLMGB_ERR_CONFIG;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce = clmgb::launch_zd09(hdims(h, *b), b->nc, *f, cfg->e_ice, dtime, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_effec_rootfrac_vert_tran_sink(clmgb_handle h, const clmgb_bounds* b,
                                            const clmgb_rootsink_fields* f, int32_t use_hydrstress,
                                            uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_effec_rootfrac_vert_tran_sink");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if (!f) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(clmgb_rootsink_fields)) return CLMGB_ERR_ABI;
  // the default method's 13 pointers always, the hydraulic-stress method's 7 with it
  const void* need[] = {f->mask_hydrology, f->col_itype, f->col_landunit, f->lun_itype, f->col_patchi,
                        f->col_npatches, f->patch_active, f->patch_wtcol, f->rootr_patch, f->qflx_tran_veg_patch,
                        f->qflx_tran_veg_col, f->rootr_col, f->qflx_rootsoi_col};
  for (const void* p : need)
    if (!p) return CLMGB_ERR_NULL_ARG;
  if (use_hydrstress) {
    const void* hs[] = {f->k_soil_root_patch, f->smp_l, f->vegwp_patch, f->frac_veg_nosno, f->z,
                        f->qflx_phs_neg_col, f->qflx_hydr_redist_patch};
    for (const void* p : hs)
      if (!p) return CLMGB_ERR_NULL_ARG;
  }
  cudaError_t ce = clmgb::launch_rootsink(hdims(h, *b), b->nc, b->nl, *f, use_hydrstress ? 1 : 0,
                                          col_status, h->dev_status, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

// the pointers the selected stages read or write (clmgb_surface_hydrology)
static bool surfhyd_pointers_ok(const clmgb_surfhyd_fields* f, const clmgb_surfhyd_config* cfg, uint32_t st) {
  auto all = [](std::initializer_list<const void*> ps) {
    for (const void* p : ps)
      if (!p) return false;
    return true;
  };
  if ((st & CLMGB_SH_FLOODC) && !all({f->mask_nolakec, f->col_gridcell, f->col_itype, f->qflx_floodg, f->qflx_floodc}))
    return false;
  if (st & CLMGB_SH_SAT_EXCESS) {
    if (!all({f->mask_hydrology, f->col_urbpoi, f->qflx_floodc, f->qflx_rain_plus_snomelt, f->fsat, f->fcov,
              f->qflx_sat_excess_surf}))
      return false;
    if (cfg->fsat_method == CLMGB_FSAT_TOPMODEL ? !all({f->frost_table, f->zwt, f->zwt_perched, f->wtfact})
                                                : !all({f->b_infil, f->top_max_moist, f->top_moist_limited}))
      return false;
    if (cfg->crop_fsat_equals_zero && !all({f->col_landunit, f->lun_itype})) return false;
    if (cfg->hillslope_fsat_equals_zero && !all({f->col_is_hillslope, f->col_active, f->col_cold})) return false;
  }
  if ((st & CLMGB_SH_QFLX_INPUTS) &&
      !all({f->mask_hydrology, f->col_snl, f->qflx_rain_plus_snomelt, f->qflx_snow_h2osfc, f->qflx_floodc,
            f->qflx_liqevap_from_top_layer, f->qflx_ev_soil, f->qflx_ev_h2osfc, f->qflx_sat_excess_surf,
            f->frac_sno_eff, f->frac_h2osfc, f->qflx_top_soil, f->qflx_in_soil, f->qflx_top_soil_to_h2osfc}))
    return false;
  if (st & CLMGB_SH_INFL_EXCESS) {
    if (!all({f->mask_hydrology, f->fsat, f->qflx_in_soil, f->frac_h2osfc, f->qinmax, f->qflx_infl_excess}))
      return false;
    if (cfg->qinmax_method == CLMGB_QINMAX_HKSAT && !all({f->icefrac, f->hksat})) return false;
  }
  if ((st & CLMGB_SH_ROUTE) &&
      !all({f->mask_hydrology, f->col_landunit, f->lun_itype, f->qflx_in_soil, f->qflx_top_soil_to_h2osfc,
            f->qflx_infl_excess, f->qflx_in_soil_limited, f->qflx_in_h2osfc, f->qflx_infl_excess_surf}))
    return false;
  if ((st & CLMGB_SH_UPDATE_H2OSFC) &&
      !all({f->mask_hydrology, f->h2osfc, f->h2osfc_thresh, f->frac_h2osfc_nosnow, f->topo_slope, f->qflx_in_h2osfc,
            f->frac_h2osfc, f->qinmax, f->qflx_h2osfc_surf, f->qflx_h2osfc_drain}))
    return false;
  if ((st & CLMGB_SH_INFILTRATION) &&
      !all({f->mask_hydrology, f->qflx_in_soil_limited, f->qflx_h2osfc_drain, f->qflx_infl}))
    return false;
  if ((st & CLMGB_SH_TOTAL_RUNOFF) &&
      !all({f->mask_hydrology, f->qflx_sat_excess_surf, f->qflx_infl_excess_surf, f->qflx_h2osfc_surf, f->qflx_surf,
            f->mask_urban, f->col_itype, f->col_snl, f->qflx_rain_plus_snomelt, f->h2osoi_liq,
            f->qflx_liqevap_from_top_layer, f->qflx_floodc, f->xs_urban}))
    return false;
  if ((st & CLMGB_SH_URBAN_PONDING) &&
      !all({f->mask_urban, f->col_itype, f->col_snl, f->xs_urban, f->qflx_rain_plus_snomelt,
            f->qflx_liqevap_from_top_layer, f->h2osoi_liq}))
    return false;
  return true;
}

int32_t clmgb_surface_hydrology(clmgb_handle h, const clmgb_bounds* b, const clmgb_surfhyd_fields* f,
                                const clmgb_surfhyd_config* cfg, uint32_t stages, double dtime, void* stream) {
  const ClmgbRange range_("clmgb_surface_hydrology");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!f || !cfg) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(clmgb_surfhyd_fields) ||
      cfg->struct_size != (int64_t)sizeof(clmgb_surfhyd_config))
    return CLMGB_ERR_ABI;
  if (stages & ~CLMGB_SH_ALL) return CLMGB_ERR_CONFIG;
  // the reference's error() on an unknown method (sat_excess_runoff.jl:347-349,
  // infilt_excess_runoff.jl:185-187), raised whenever that routine is called
  if ((stages & CLMGB_SH_SAT_EXCESS) && cfg->fsat_method != CLMGB_FSAT_TOPMODEL && cfg->fsat_method != CLMGB_FSAT_VIC)
    return CLMGB_ERR_CONFIG;
  if ((stages & CLMGB_SH_INFL_EXCESS) && cfg->qinmax_method != CLMGB_QINMAX_NONE &&
      cfg->qinmax_method != CLMGB_QINMAX_HKSAT)
    return CLMGB_ERR_CONFIG;
  if ((stages & CLMGB_SH_FLOODC) && cfg->ng < 0) return CLMGB_ERR_CONFIG;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0 || stages == 0) return CLMGB_OK;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  if (!surfhyd_pointers_ok(f, cfg, stages)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_surface_hydrology(hdims(h, *b), b->nc, b->nl, *f, *cfg, stages, dtime,
                                                   h->dev_status, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_balance_check_columns(clmgb_handle h, const clmgb_bounds* b, const clmgb_colbalance_fields* f,
                                    double dtime, clmgb_balance_report* report, void* stream) {
  const ClmgbRange range_("clmgb_balance_check_columns");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!f || !report) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(clmgb_colbalance_fields)) return CLMGB_ERR_ABI;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  memset(report, 0, sizeof(*report));
  if (b->nc == 0) return CLMGB_OK;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  // every member but errsoi (NULL: no soil energy scan)
  const void* need[] = {f->col_itype, f->col_active, f->forc_rain, f->forc_snow, f->begwb, f->endwb, f->qflx_flood,
                        f->qflx_sfc_irrig, f->qflx_glcice_dyn_water_flux, f->qflx_evap_tot, f->qflx_surf,
                        f->qflx_qrgwl, f->qflx_drain, f->qflx_drain_perched, f->qflx_ice_runoff,
                        f->qflx_snwcp_discarded_liq, f->qflx_snwcp_discarded_ice, f->errh2o};
  for (const void* p : need)
    if (!p) return CLMGB_ERR_NULL_ARG;
  const cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* r = h->scratch + 2;
  cudaError_t ce = clmgb::launch_colbalance(b->nc, *f, dtime, r, s);
  unsigned long long v[5];
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(v, r, sizeof(v), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return cuda_fail(h, ce);
  double m, ms;
  memcpy(&m, &v[0], sizeof(double));
  memcpy(&ms, &v[3], sizeof(double));
  report->errh2o_max = m;
  report->errh2o_index = (int64_t)v[1];
  report->errh2o_nonfinite = v[2] == ~0ULL ? 0 : (int64_t)v[2];
  report->errsoi_max = f->errsoi ? ms : 0.0;
  report->errsoi_index = f->errsoi ? (int64_t)v[4] : 0;
  // the scans' thresholds (balance_check.jl:711-713, 1352, 1356); NaN compares false
  if (m > 1.0e-9) report->flags |= CLMGB_BAL_H2O_WARN;
  if (m > 1.0e-5) report->flags |= CLMGB_BAL_H2O_ERROR;
  if (report->errh2o_nonfinite) report->flags |= CLMGB_BAL_H2O_NONFINITE;
  if (f->errsoi && ms > 1.0e-5) report->flags |= CLMGB_BAL_SOI_WARN;
  if (f->errsoi && ms > 1.0e-4) report->flags |= CLMGB_BAL_SOI_ERROR;
  return CLMGB_OK;
}

int32_t clmgb_lake_temperature(clmgb_handle h, const clmgb_bounds* b, const clmgb_lake_fields* f,
                               const clmgb_lake_config* cfg, double dtime, void* stream) {
  const ClmgbRange range_("clmgb_lake_temperature");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!f || !cfg) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(clmgb_lake_fields) || cfg->struct_size != (int64_t)sizeof(clmgb_lake_config))
    return CLMGB_ERR_ABI;
  if (cfg->nlevlak < 2 || cfg->nlevlak > CLMGB_MAX_NLEVLAK) return CLMGB_ERR_DIMS;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  // every member but the two CH4 outputs, which only use_lch4 writes
  const char* base = reinterpret_cast<const char*>(f) + sizeof(int64_t);
  const size_t nptr = (sizeof(clmgb_lake_fields) - sizeof(int64_t)) / sizeof(void*);
  for (size_t i = 0; i < nptr; i++) {
    const void* q;
    memcpy(&q, base + i * sizeof(void*), sizeof(void*));
    const void* member = base + i * sizeof(void*);
    const bool ch4 = member == (const void*)&f->lakeresist || member == (const void*)&f->grnd_ch4_cond;
    if (!q && !(ch4 && !cfg->use_lch4)) return CLMGB_ERR_NULL_ARG;
  }
  cudaError_t ce = clmgb::launch_lake_temperature(hdims(h, *b), b->nc, *f, *cfg, dtime, h->dev_status,
                                                  (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

// the pointers the selected stages read or write (clmgb_snow_layers)
static bool snowlayer_pointers_ok(const clmgb_snowlayer_fields* f, const clmgb_snowlayer_config* cfg, uint32_t st) {
  auto all = [](std::initializer_list<const void*> ps) {
    for (const void* p : ps)
      if (!p) return false;
    return true;
  };
  const bool layers = st & (CLMGB_SL_COMPACTION | CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE | CLMGB_SL_ZERO_EMPTY);
  if (layers && !all({f->mask_snow, f->col_snl, f->dz, f->t_soisno, f->h2osoi_ice, f->h2osoi_liq})) return false;
  if ((st & CLMGB_SL_COMPACTION) &&
      !all({f->col_landunit, f->lun_lakpoi, f->lun_urbpoi, f->n_melt, f->frac_h2osfc, f->frac_sno, f->int_snow,
            f->imelt, f->swe_old, f->frac_iceold}))
    return false;
  if ((st & CLMGB_SL_COMPACTION) && cfg->wind_dependent_snow_density && !all({f->col_gridcell, f->forc_wind}))
    return false;
  if ((st & (CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE | CLMGB_SL_ZERO_EMPTY)) && !all({f->z, f->zi})) return false;
  if ((st & (CLMGB_SL_COMBINE | CLMGB_SL_DIVIDE)) &&
      !all({f->frac_sno, f->snw_rds, f->mss_bcphi, f->mss_bcpho, f->mss_ocphi, f->mss_ocpho, f->mss_dst1, f->mss_dst2,
            f->mss_dst3, f->mss_dst4}))
    return false;
  if ((st & CLMGB_SL_COMBINE) &&
      !all({f->col_landunit, f->lun_itype, f->lun_urbpoi, f->frac_sno_eff, f->int_snow, f->h2osno_no_layers,
            f->snow_depth, f->qflx_sl_top_soil}))
    return false;
  if ((st & CLMGB_SL_FILTER) && !all({f->mask_snow, f->mask_nosnow, f->mask_nolakec, f->col_snl})) return false;
  return true;
}

int32_t clmgb_snow_layers(clmgb_handle h, const clmgb_bounds* b, const clmgb_snowlayer_fields* f,
                          const clmgb_snowlayer_config* cfg, uint32_t stages, double dtime, void* stream) {
  const ClmgbRange range_("clmgb_snow_layers");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!cfg) return CLMGB_ERR_NULL_ARG;
  if (cfg->struct_size != (int64_t)sizeof(clmgb_snowlayer_config)) return CLMGB_ERR_ABI;
  if (stages & ~CLMGB_SL_ALL) return CLMGB_ERR_CONFIG;
  // snow_compaction!'s error() on an unknown overburden method (snow_hydrology.jl:1373-1377)
  if ((stages & CLMGB_SL_COMPACTION) && cfg->overburden_method != CLMGB_OVERBURDEN_ANDERSON1976 &&
      cfg->overburden_method != CLMGB_OVERBURDEN_VIONNET2012)
    return CLMGB_ERR_CONFIG;
  if (cfg->ng < 0) return CLMGB_ERR_CONFIG;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0 || stages == 0) return CLMGB_OK;
  if (!f) return CLMGB_ERR_NULL_ARG;
  if (f->struct_size != (int64_t)sizeof(clmgb_snowlayer_fields)) return CLMGB_ERR_ABI;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  if (!snowlayer_pointers_ok(f, cfg, stages)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_snow_layers(hdims(h, *b), b->nc, b->nl, *f, *cfg, stages, dtime,
                                             h->dev_status, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_water_fractions(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                                   void* stream) {
  const ClmgbRange range_("clmgb_soil_water_fractions");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  cudaError_t ce = clmgb::launch_water_fractions(hdims(h, *b), b->nc, *f, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_water(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                         const clmgb_swm_config* cfg, double dtime, uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_soil_water");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, false))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce;
  if (h->step_schedule == CLMGB_SCHEDULE_FUSED)
    ce = clmgb::launch_moisture_form(hdims(h, *b), b->nc, *f, *cfg, dtime, col_status, h->dev_status,
                                     (cudaStream_t)stream);
  else if (use_waves(h, b->nc))
    ce = clmgb::launch_moisture_form_waves(hdims(h, *b), b->nc, *f, *cfg, dtime, col_status, 0,
                                           h->dev_status, h->ws, waves_grid(h), (cudaStream_t)stream);
  else
    ce = clmgb::launch_moisture_form_queue(hdims(h, *b), b->nc, *f, *cfg, dtime, col_status, 0,
                                           h->dev_status, h->queue, queue_grid(h), queue_scratch(h),
                                           (cudaStream_t)stream);
  if (ce == cudaSuccess)
    ce = clmgb::launch_compute_qcharge(hdims(h, *b), b->nc, *f, *cfg, dtime,
                                       (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_water_flexible_cn(clmgb_handle h, const clmgb_bounds* b, const clmgb_flexcn_fields* f,
                                     void* stream) {
  const ClmgbRange range_("clmgb_soil_water_flexible_cn");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, false);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (h->vp.nlevsoi < 1) return CLMGB_ERR_DIMS;
  const cudaError_t ce = clmgb::launch_flexible_cn(hdims(h, *b), b->nc, *f, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_column_step(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                          const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                          int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                          void* stream) {
  const ClmgbRange range_("clmgb_column_step");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, true))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if ((e = check_fields(fw))) return e;
  if (snow_method != CLMGB_SNOW_JORDAN1991 && snow_method != CLMGB_SNOW_STURM1997) return CLMGB_ERR_CONFIG;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  const Dims D = hdims(h, *b);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  if (h->step_schedule == CLMGB_SCHEDULE_FUSED) {
    ce = clmgb::launch_column_step(D, b->nc, *ft, *fw, *cfg, dtime, snow_method, t_ssbef, t_h2osfc_bef,
                                   col_status, h->dev_status, s);
  } else {
    ce = clmgb::launch_soiltemp_fractions(D, b->nc, *ft, *fw, dtime, snow_method, t_ssbef, t_h2osfc_bef,
                                          col_status, h->dev_status, s);
    if (ce == cudaSuccess) {
      if (use_waves(h, b->nc))
        ce = clmgb::launch_moisture_form_waves(D, b->nc, *fw, *cfg, dtime, col_status, 1, h->dev_status, h->ws,
                                               waves_grid(h), s);
      else
        ce = clmgb::launch_moisture_form_queue(D, b->nc, *fw, *cfg, dtime, col_status, 1, h->dev_status, h->queue,
                                               queue_grid(h), queue_scratch(h), s);
    }
  }
  if (ce == cudaSuccess) ce = clmgb::launch_compute_qcharge(D, b->nc, *fw, *cfg, dtime, s);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

static int32_t phase_change_common(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* f,
                                   double dtime, const double* dhsdT, int which, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!dhsdT) return CLMGB_ERR_NULL_ARG;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce = clmgb::launch_phase_change(hdims(h, *b), b->nc, *f, dtime, dhsdT, which,
                                              (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_phase_change_h2osfc(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* f,
                                  double dtime, const double* dhsdT, void* stream) {
  const ClmgbRange range_("clmgb_phase_change_h2osfc");
  return phase_change_common(h, b, f, dtime, dhsdT, 0, stream);
}

int32_t clmgb_phase_change_beta(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* f,
                                double dtime, const double* dhsdT, void* stream) {
  const ClmgbRange range_("clmgb_phase_change_beta");
  return phase_change_common(h, b, f, dtime, dhsdT, 1, stream);
}

int32_t clmgb_synth_forcing(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                            const clmgb_soilwater_fields* fw, const double* G, const double* I, void* stream) {
  const ClmgbRange range_("clmgb_synth_forcing");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if ((e = check_fields(fw))) return e;
  if (!G || !I) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_synth_forcing(hdims(h, *b), b->nc, *ft, *fw, G, I, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_batched_band_solve(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev, double* tvector,
                                 const double* bmatrix, const double* rvector, const int64_t* jtop,
                                 const int64_t* jbot, const uint8_t* mask, int32_t kl, int32_t ku,
                                 int32_t nlevsno_off, void* stream) {
  const ClmgbRange range_("clmgb_batched_band_solve");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (nc < 0 || ldc < nc || nlev < 1 || nlev > clmgb::MAXROWS + 1) return CLMGB_ERR_DIMS;
  if (!((kl == 2 && ku == 2) || (kl == 1 && ku == 1))) return CLMGB_ERR_UNSUPPORTED;
  if (nc == 0) return CLMGB_OK;
  if (!tvector || !bmatrix || !rvector || !jtop || !jbot || !mask) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_band_solve(nc, ldc, nlev, tvector, bmatrix, rvector, jtop, jbot, mask, kl, ku,
                                            nlevsno_off, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_reserve(clmgb_handle h, int64_t max_nc) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (max_nc < 0 || max_nc > 0xffffffffLL) return CLMGB_ERR_DIMS;
  if (max_nc <= h->qs.capacity) return CLMGB_OK;
  const size_t n = (size_t)max_nc;
  const size_t nsoi = (size_t)h->vp.nlevsoi;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t lev = al(nsoi * n * sizeof(double));   // one [nlevsoi][n] array
  const size_t col8 = al(n * 8), col4 = al(n * 4);
  // imp + 5 wave level arrays, the column records (PC_ALL level arrays),
  // 6 per-column doubles, nsub + status, order + 4 lists, bins
  const size_t total = (6 + clmgb::PC_ALL) * lev + 6 * col8 + 2 * col4 + 5 * col4 + al(256 * sizeof(unsigned int));
  void* blk = nullptr;
  cudaError_t ce = cudaDeviceSynchronize();
  if (ce == cudaSuccess) ce = cudaMalloc(&blk, total);
  if (ce != cudaSuccess) return cuda_fail(h, ce);
  if (h->reserve_block) cudaFree(h->reserve_block);
  h->reserve_block = blk;
  char* p = static_cast<char*>(blk);
  auto take = [&p](size_t b) { char* q = p; p += b; return q; };
  clmgb::WaveScratch& w = h->ws;
  w.cap = max_nc;
  w.imp = reinterpret_cast<double*>(take(lev));
  w.qout = reinterpret_cast<double*>(take(lev));
  w.dqodw1 = reinterpret_cast<double*>(take(lev));
  w.dqodw2 = reinterpret_cast<double*>(take(lev));
  w.fnet1 = reinterpret_cast<double*>(take(lev));
  w.dtdz = reinterpret_cast<double*>(take(lev));
  w.dtsub = reinterpret_cast<double*>(take(col8));
  w.dtdone = reinterpret_cast<double*>(take(col8));
  w.qc = reinterpret_cast<double*>(take(col8));
  w.dtcur = reinterpret_cast<double*>(take(col8));
  w.hk_bot = reinterpret_cast<double*>(take(col8));
  w.dhkdw_bot = reinterpret_cast<double*>(take(col8));
  w.nsub = reinterpret_cast<int*>(take(col4));
  w.status = reinterpret_cast<uint32_t*>(take(col4));
  h->qs.order = reinterpret_cast<uint32_t*>(take(col4));
  w.listA[0] = reinterpret_cast<uint32_t*>(take(col4));
  w.listA[1] = reinterpret_cast<uint32_t*>(take(col4));
  w.listH[0] = reinterpret_cast<uint32_t*>(take(col4));
  w.listH[1] = reinterpret_cast<uint32_t*>(take(col4));
  h->qs.bins = reinterpret_cast<unsigned int*>(take(al(256 * sizeof(unsigned int))));
  w.counters = h->qs.bins + 192;   // bins use words 0..128
  h->qs.imp = w.imp;
  h->qs.pcache = reinterpret_cast<double*>(take(clmgb::PC_ALL * lev));
  h->qs.capacity = max_nc;
  return CLMGB_OK;
}

int32_t clmgb_set_option(clmgb_handle h, int32_t key, int64_t value) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  switch (key) {
    case CLMGB_OPT_STEP_SCHEDULE:
      if (value != CLMGB_SCHEDULE_FUSED && value != CLMGB_SCHEDULE_QUEUE && value != CLMGB_SCHEDULE_WAVES)
        return CLMGB_ERR_CONFIG;
      h->step_schedule = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_BLOCKS_PER_SM:
      if (value < 0) return CLMGB_ERR_CONFIG;
      h->queue_blocks_per_sm = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_ORDER:
      if (value != 0 && value != 1) return CLMGB_ERR_CONFIG;
      h->queue_order = value;
      return CLMGB_OK;
    case CLMGB_OPT_WAVES_BLOCKS_PER_SM:
      if (value < 0) return CLMGB_ERR_CONFIG;
      h->waves_blocks_per_sm = value;
      return CLMGB_OK;
    case CLMGB_OPT_ADJ_RICHARDS:
      if (value != CLMGB_ADJ_RICHARDS_CLOSED_FORM && value != CLMGB_ADJ_RICHARDS_RECORDED) return CLMGB_ERR_CONFIG;
      h->tape.richards_mode = (int)value;
      return CLMGB_OK;
    case CLMGB_OPT_ADJ_SOIL_TEMPERATURE:
      if (value != CLMGB_ADJ_ST_CLOSED_FORM && value != CLMGB_ADJ_ST_RECORDED) return CLMGB_ERR_CONFIG;
      h->adj_st_mode = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_FRESH_BATCH:
      if (value < 0 || value > 32) return CLMGB_ERR_CONFIG;
      h->fresh_batch = value;
      return CLMGB_OK;
    case CLMGB_OPT_COLUMN_BASE:
      if (value < 0) return CLMGB_ERR_CONFIG;
      h->column_base = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_DEFER:
      if (value < 0 || value > clmgb::MF_ATTEMPT_CAP) return CLMGB_ERR_CONFIG;
      h->defer = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_PACKED_REFRESH:
      if (value != 0 && value != 1) return CLMGB_ERR_CONFIG;
      h->packed = value;
      return CLMGB_OK;
    case CLMGB_OPT_ATTEMPT_CAP:
      if (value < 1 || value > clmgb::MF_ATTEMPT_CAP) return CLMGB_ERR_CONFIG;
      h->attempt_cap = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_POLL_LIMIT:
      if (value < 0 || value > clmgb::DEFER_POLL_LIMIT) return CLMGB_ERR_CONFIG;
      h->poll_limit = value;
      return CLMGB_OK;
    case CLMGB_OPT_QUEUE_PUBLISH_DELAY:
      if (value < 0 || value > 10000000) return CLMGB_ERR_CONFIG;
      h->publish_delay = value;
      return CLMGB_OK;
    case CLMGB_OPT_RECORDS_TMA:
      if (value != 0 && value != 1) return CLMGB_ERR_CONFIG;
      h->records_tma = value;
      return CLMGB_OK;
    case CLMGB_OPT_TRIDIAG_METHOD:
      if (value != CLMGB_TRIDIAG_THOMAS && value != CLMGB_TRIDIAG_PCR) return CLMGB_ERR_CONFIG;
      h->tridiag_method = value;
      return CLMGB_OK;
    case CLMGB_OPT_ST_BLOCK:
      if (value != 128 && value != 320 && value != 640) return CLMGB_ERR_CONFIG;
      h->st_block = value;
      return CLMGB_OK;
    case CLMGB_OPT_COUNT_WORK: {
      if (value != 0 && value != 1) return CLMGB_ERR_CONFIG;
      if (value && !h->count_work) {    // counting starts from zero
        const cudaError_t ce = cudaMemset(h->scratch + 10, 0, 2 * sizeof(unsigned long long));
        if (ce != cudaSuccess) return cuda_fail(h, ce);
      }
      h->count_work = value;
      return CLMGB_OK;
    }
    default:
      return CLMGB_ERR_CONFIG;
  }
}

int32_t clmgb_get_option(clmgb_handle h, int32_t key, int64_t* value) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (!value) return CLMGB_ERR_NULL_ARG;
  switch (key) {
    case CLMGB_OPT_STEP_SCHEDULE: *value = h->step_schedule; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_BLOCKS_PER_SM: *value = h->queue_blocks_per_sm; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_OCCUPANCY: *value = h->occupancy_blocks; return CLMGB_OK;
    case CLMGB_OPT_NUM_SMS: *value = h->num_sms; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_ORDER: *value = h->queue_order; return CLMGB_OK;
    case CLMGB_OPT_RESERVED_COLUMNS: *value = h->qs.capacity; return CLMGB_OK;
    case CLMGB_OPT_WAVES_BLOCKS_PER_SM: *value = h->waves_blocks_per_sm; return CLMGB_OK;
    case CLMGB_OPT_WAVES_OCCUPANCY: *value = h->waves_blocks; return CLMGB_OK;
    case CLMGB_OPT_ADJ_TAPE_SLOTS: *value = h->tape.slots; return CLMGB_OK;
    case CLMGB_OPT_ADJ_RICHARDS: *value = h->tape.richards_mode; return CLMGB_OK;
    case CLMGB_OPT_ADJ_SOIL_TEMPERATURE: *value = h->adj_st_mode; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_FRESH_BATCH: *value = h->fresh_batch; return CLMGB_OK;
    case CLMGB_OPT_COLUMN_BASE: *value = h->column_base; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_DEFER: *value = h->defer; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_PACKED_REFRESH: *value = h->packed; return CLMGB_OK;
    case CLMGB_OPT_ATTEMPT_CAP: *value = h->attempt_cap; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_POLL_LIMIT: *value = h->poll_limit; return CLMGB_OK;
    case CLMGB_OPT_QUEUE_PUBLISH_DELAY: *value = h->publish_delay; return CLMGB_OK;
    case CLMGB_OPT_COUNT_WORK: *value = h->count_work; return CLMGB_OK;
    case CLMGB_OPT_RECORDS_TMA: *value = h->records_tma; return CLMGB_OK;
    case CLMGB_OPT_RECORDS_TMA_USED: *value = h->records_tma_used; return CLMGB_OK;
    case CLMGB_OPT_TRIDIAG_METHOD: *value = h->tridiag_method; return CLMGB_OK;
    case CLMGB_OPT_ST_BLOCK: *value = h->st_block; return CLMGB_OK;
    case CLMGB_OPT_WORK_LEVEL_ATTEMPTS:
    case CLMGB_OPT_WORK_LEVEL_REFRESHES: {
      unsigned long long w[2];
      const cudaError_t ce = cudaMemcpy(w, h->scratch + 10, sizeof(w), cudaMemcpyDeviceToHost);
      if (ce != cudaSuccess) return cuda_fail(h, ce);
      *value = (int64_t)w[key == CLMGB_OPT_WORK_LEVEL_ATTEMPTS ? 0 : 1];
      return CLMGB_OK;
    }
    case CLMGB_OPT_ADJ_TAPE_ENTRIES: *value = h->tape.entries; return CLMGB_OK;
    case CLMGB_OPT_ADJ_TAPE_USED: {
      unsigned int used = 0;
      if (h->tape.max_used) {
        cudaError_t ce = cudaMemcpy(&used, h->tape.max_used, sizeof(used), cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) return cuda_fail(h, ce);
      }
      *value = used;
      return CLMGB_OK;
    }
    default: return CLMGB_ERR_CONFIG;
  }
}

int32_t clmgb_math_eval(clmgb_handle h, int32_t op, int64_t n, const double* x, const double* y, double* out,
                        void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (op < 0 || op > 6 || n < 0) return CLMGB_ERR_CONFIG;
  if (n == 0) return CLMGB_OK;
  if (!x || !out || ((op == 2 || op == 6) && !y)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_math_eval(op, n, x, y, out, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_tridiagonal_multi(clmgb_handle h, int64_t ncols, int64_t ldc, int32_t nlevs, double* u,
                                const double* a, const double* b, const double* c, const double* r,
                                const int64_t* jtop, const uint8_t* mask, void* stream) {
  const ClmgbRange range_("clmgb_tridiagonal_multi");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (ncols < 0 || ldc < ncols || nlevs < 1 || nlevs > 64) return CLMGB_ERR_DIMS;
  if (ncols == 0) return CLMGB_OK;
  if (!u || !a || !b || !c || !r || !jtop || !mask) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_tridiagonal_multi(ncols, ldc, nlevs, u, a, b, c, r, jtop, mask,
                                                   (cudaStream_t)stream, (int)h->tridiag_method);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_batched_band_solve_factor(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev, double* tvector,
                                        const double* bmatrix, const double* rvector, const int64_t* jtop,
                                        const int64_t* jbot, const uint8_t* mask, int32_t kl, int32_t ku,
                                        int32_t nlevsno_off, double* lu, uint8_t* piv, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (nc < 0 || ldc < nc || nlev < 1 || nlev > clmgb::MAXROWS + 1) return CLMGB_ERR_DIMS;
  if (!((kl == 2 && ku == 2) || (kl == 1 && ku == 1))) return CLMGB_ERR_UNSUPPORTED;
  if (nc == 0) return CLMGB_OK;
  if (!tvector || !bmatrix || !rvector || !jtop || !jbot || !mask || !lu || !piv) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_band_factor_solve(nc, ldc, nlev, tvector, bmatrix, rvector, jtop, jbot, mask, kl,
                                                   ku, nlevsno_off, lu, piv, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_batched_band_solve_adjoint(clmgb_handle h, int64_t nc, int64_t ldc, int32_t nlev,
                                         const double* tvector, double* tvector_bar, const double* lu,
                                         const uint8_t* piv, double* bmatrix_bar, double* rvector_bar,
                                         const int64_t* jtop, const int64_t* jbot, const uint8_t* mask, int32_t kl,
                                         int32_t ku, int32_t nlevsno_off, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (nc < 0 || ldc < nc || nlev < 1 || nlev > clmgb::MAXROWS + 1) return CLMGB_ERR_DIMS;
  if (!((kl == 2 && ku == 2) || (kl == 1 && ku == 1))) return CLMGB_ERR_UNSUPPORTED;
  if (nc == 0) return CLMGB_OK;
  if (!tvector || !tvector_bar || !lu || !piv || !jtop || !jbot || !mask) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_band_solve_adjoint(nc, ldc, nlev, tvector, tvector_bar, lu, piv, bmatrix_bar,
                                                    rvector_bar, jtop, jbot, mask, kl, ku, nlevsno_off,
                                                    (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_tridiagonal_adjoint(clmgb_handle h, int64_t ncols, int64_t ldc, int32_t nlevs, const double* u,
                                  const double* a, const double* b, const double* c, double* u_bar, double* a_bar,
                                  double* b_bar, double* c_bar, double* r_bar, const int64_t* jtop,
                                  const uint8_t* mask, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (ncols < 0 || ldc < ncols || nlevs < 1 || nlevs > 64) return CLMGB_ERR_DIMS;
  if (ncols == 0) return CLMGB_OK;
  if (!u || !a || !b || !c || !u_bar || !jtop || !mask) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_tridiagonal_adjoint(ncols, ldc, nlevs, u, a, b, c, u_bar, a_bar, b_bar, c_bar,
                                                     r_bar, jtop, mask, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_reserve_adjoint(clmgb_handle h, int64_t slots, int64_t entries) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (slots < 1 || slots > (1LL << 24) || entries < 256 || entries > (1LL << 30)) return CLMGB_ERR_DIMS;
  slots = (slots + 63) / 64 * 64;
  const size_t n = (size_t)slots * (size_t)entries;
  const size_t nsub = (size_t)slots * CLMGB_ADJ_MAX_SUBSTEPS * (CLMGB_MAX_NLEVSOI + 2);
  const size_t total = n * (sizeof(int2) + sizeof(double2) + sizeof(double)) + nsub * sizeof(double) + 256;
  cudaError_t ce = cudaDeviceSynchronize();
  if (ce != cudaSuccess) return cuda_fail(h, ce);
  if (h->tape_block) {
    cudaFree(h->tape_block);
    h->tape_block = nullptr;
    const int mode = h->tape.richards_mode;
    h->tape = clmgb::AdjTape{};
    h->tape.richards_mode = mode;
  }
  void* blk = nullptr;
  ce = cudaMalloc(&blk, total);
  if (ce != cudaSuccess) return cuda_fail(h, ce);
  char* p = (char*)blk;
  h->tape.par = (double2*)p;
  p += n * sizeof(double2);
  h->tape.adj = (double*)p;
  p += n * sizeof(double);
  h->tape.sub = (double*)p;
  p += nsub * sizeof(double);
  h->tape.idx = (int2*)p;
  p += n * sizeof(int2);
  h->tape.max_used = (unsigned int*)p;
  h->tape.slots = slots;
  h->tape.entries = entries;
  h->tape.maxsub = CLMGB_ADJ_MAX_SUBSTEPS;
  h->tape_block = blk;
  ce = cudaMemset(h->tape.max_used, 0, sizeof(unsigned int));
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

// the size of clmgb_substep_log before st_rec was appended
static constexpr int64_t LOG_SIZE_NO_ST = (int64_t)offsetof(clmgb_substep_log, st_rec);

static int32_t check_log(const clmgb_substep_log* log) {
  if (!log) return CLMGB_OK;
  if (log->struct_size != (int64_t)sizeof(clmgb_substep_log) && log->struct_size != LOG_SIZE_NO_ST)
    return CLMGB_ERR_ABI;
  if (!log->rec || !log->count) return CLMGB_ERR_NULL_ARG;
  if (log->cap < 1 || log->cap > CLMGB_ADJ_MAX_SUBSTEPS) return CLMGB_ERR_CONFIG;
  return CLMGB_OK;
}

static double* log_st(const clmgb_substep_log* log) {
  return (log && log->struct_size >= (int64_t)sizeof(clmgb_substep_log)) ? log->st_rec : nullptr;
}

static clmgb::SubstepLogView log_view(const clmgb_substep_log* log) {
  if (!log) return clmgb::SubstepLogView{nullptr, nullptr, 0, 0, nullptr};
  return clmgb::SubstepLogView{log->rec, log->count, (int)log->cap, CLMGB_LOG_STRIDE(log->cap), log_st(log)};
}

int32_t clmgb_column_step_logged(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                 const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                                 int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                 const clmgb_substep_log* log, uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_column_step_logged");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, true))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if ((e = check_fields(fw))) return e;
  if (!log) return CLMGB_ERR_NULL_ARG;
  if ((e = check_log(log))) return e;
  if (snow_method != CLMGB_SNOW_JORDAN1991 && snow_method != CLMGB_SNOW_STURM1997) return CLMGB_ERR_CONFIG;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  const Dims D = hdims(h, *b);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce = clmgb::launch_soiltemp_fractions(D, b->nc, *ft, *fw, dtime, snow_method, t_ssbef, t_h2osfc_bef,
                                                    col_status, h->dev_status, s, log_st(log));
  if (ce == cudaSuccess) {
    const clmgb::SubstepLogView lv = log_view(log);
    ce = clmgb::launch_moisture_form_queue(D, b->nc, *fw, *cfg, dtime, col_status, 1, h->dev_status, h->queue,
                                           queue_grid(h), queue_scratch(h), s, nullptr, &lv);
  }
  if (ce == cudaSuccess) ce = clmgb::launch_compute_qcharge(D, b->nc, *fw, *cfg, dtime, s);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_column_step_vjp(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                              const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                              int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef,
                              const clmgb_step_adjoint* adj, uint32_t* col_status, void* stream) {
  return clmgb_column_step_vjp_logged(h, b, ft, fw, cfg, dtime, snow_method, t_ssbef, t_h2osfc_bef, adj, nullptr,
                                      col_status, stream);
}

int32_t clmgb_column_step_vjp_logged(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                     const clmgb_soilwater_fields* fw, const clmgb_swm_config* cfg, double dtime,
                                     int32_t snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                     const clmgb_step_adjoint* adj, const clmgb_substep_log* log,
                                     uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_column_step_vjp_logged");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, true))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if ((e = check_fields(fw))) return e;
  if (!adj) return CLMGB_ERR_NULL_ARG;
  if (adj->struct_size != (int64_t)sizeof(clmgb_step_adjoint)) return CLMGB_ERR_ABI;
  if (!adj->lam_t_soisno || !adj->lam_h2osoi_liq || !adj->lam_h2osoi_ice || !adj->lam_t_grnd ||
      !adj->lam_t_h2osfc)
    return CLMGB_ERR_NULL_ARG;
  if (snow_method != CLMGB_SNOW_JORDAN1991 && snow_method != CLMGB_SNOW_STURM1997) return CLMGB_ERR_CONFIG;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  if (!h->tape_block) return CLMGB_ERR_CONFIG;
  const Dims D = hdims(h, *b);
  if ((e = check_log(log))) return e;
  cudaError_t ce;
  if (h->adj_st_mode == CLMGB_ADJ_ST_CLOSED_FORM && h->tape.richards_mode == CLMGB_ADJ_RICHARDS_CLOSED_FORM)
    ce = clmgb::launch_column_step_vjp_cf(D, b->nc, *ft, *fw, *cfg, dtime, snow_method, t_ssbef, t_h2osfc_bef, *adj,
                                          h->tape, log_view(log), h->qs, h->queue, vjp_grid(h), col_status,
                                          h->dev_status, (cudaStream_t)stream);
  else
    ce = clmgb::launch_column_step_vjp(D, b->nc, *ft, *fw, *cfg, dtime, snow_method, t_ssbef, t_h2osfc_bef, *adj,
                                       h->tape, col_status, h->dev_status, (cudaStream_t)stream);
  // the replayed step leaves the forward's state, compute_qcharge! included
  if (ce == cudaSuccess) ce = clmgb::launch_compute_qcharge(D, b->nc, *fw, *cfg, dtime, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_soil_water_warm(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                              const clmgb_swm_config* cfg, double dtime, const double* dt_first,
                              uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_soil_water_warm");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, false))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  cudaError_t ce = clmgb::launch_moisture_form_queue(hdims(h, *b), b->nc, *f, *cfg, dtime, col_status, 0,
                                                     h->dev_status, h->queue, queue_grid(h), queue_scratch(h),
                                                     (cudaStream_t)stream, dt_first);
  if (ce == cudaSuccess)
    ce = clmgb::launch_compute_qcharge(hdims(h, *b), b->nc, *f, *cfg, dtime,
                                       (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_samples(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                          const clmgb_swm_config* cfg, double dtime, int32_t per_column, float* features,
                          float* targets, uint32_t* count, int64_t capacity, uint32_t* col_status, void* stream) {
  const ClmgbRange range_("clmgb_mlp_samples");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, false))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!(dtime > 0.0) || per_column < 0) return CLMGB_ERR_CONFIG;
  if (!features || !targets || !count || capacity < 0) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_richards_samples(hdims(h, *b), b->nc, *f, *cfg, dtime, per_column, features,
                                                  targets, count, capacity, col_status, (cudaStream_t)stream);
  if (ce == cudaSuccess)
    ce = clmgb::launch_compute_qcharge(hdims(h, *b), b->nc, *f, *cfg, dtime,
                                       (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_linear(clmgb_handle h, int64_t M, int32_t N, int32_t K, const uint16_t* X, int64_t ldx,
                         const uint16_t* W, const float* bias, int32_t act, float* Z, int64_t ldz, uint16_t* Y,
                         int64_t ldy, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (M < 0 || ldx < K || (Z && ldz < N) || (Y && ldy < N)) return CLMGB_ERR_DIMS;
  if (!X || !W) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_linear(M, N, K, X, ldx, W, bias, act, Z, ldz, Y, ldy, (cudaStream_t)stream);
  if (ce == cudaErrorInvalidValue) return CLMGB_ERR_UNSUPPORTED;
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_linear_dw(clmgb_handle h, int64_t M, int32_t N, int32_t K, const uint16_t* dZ, int64_t lddz,
                            const uint16_t* X, int64_t ldx, float* dW, float* db, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (M < 0 || lddz < N || ldx < K) return CLMGB_ERR_DIMS;
  if (!dZ || !X || !dW) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_linear_dw(M, N, K, dZ, lddz, X, ldx, dW, db, (cudaStream_t)stream);
  if (ce == cudaErrorInvalidValue) return CLMGB_ERR_UNSUPPORTED;
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_silu_backward(clmgb_handle h, int64_t n, const float* Z, const uint16_t* dY, uint16_t* dZ,
                                void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (n < 0) return CLMGB_ERR_DIMS;
  if (n && (!Z || !dY || !dZ)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_silu_backward(n, Z, dY, dZ, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_loss(clmgb_handle h, int64_t M, const float* Y, const float* T, float w_dt, float w_incr,
                       float* loss, uint16_t* dY, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (M < 0) return CLMGB_ERR_DIMS;
  if (M && (!Y || !T || !loss || !dY)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_loss(M, Y, T, w_dt, w_incr, loss, dY, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_adam(clmgb_handle h, int64_t rows, int64_t cols, float* w, const float* grad, float* m, float* v,
                       float lr, float beta1, float beta2, float eps, int32_t step, uint16_t* w_bf16,
                       uint16_t* wt_bf16, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (rows < 0 || cols < 0 || step < 1) return CLMGB_ERR_DIMS;
  if (rows * cols && (!w || !grad || !m || !v)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_adam(rows, cols, w, grad, m, v, lr, beta1, beta2, eps, step, w_bf16, wt_bf16,
                                          (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_features(clmgb_handle h, const clmgb_bounds* b, const clmgb_soilwater_fields* f,
                           const clmgb_swm_config* cfg, double dtime, const float* mean, const float* istd,
                           uint16_t* X, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_cfg(cfg);
  if (e) return e;
  if ((e = check_bounds(b, false))) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(f))) return e;
  if (!mean || !istd || !X) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_features(hdims(h, *b), b->nc, *f, *cfg, dtime, mean, istd, X,
                                              (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_mlp_first_dt(clmgb_handle h, int64_t nc, const float* Y, double dtime, float margin, int32_t kmax,
                           double* dt_first, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  if (nc < 0 || kmax < 0) return CLMGB_ERR_DIMS;
  if (nc && (!Y || !dt_first)) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_mlp_first_dt(nc, Y, dtime, margin, kmax, dt_first, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_balance_begin(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft, double* t_grnd0,
                            double* begwb, void* stream) {
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if (!t_grnd0 || !begwb) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_balance_begin(hdims(h, *b), b->nc, *ft, t_grnd0, begwb, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

int32_t clmgb_balance_residuals(clmgb_handle h, const clmgb_bounds* b, const clmgb_soiltemp_fields* ft,
                                const clmgb_soilwater_fields* fw, double dtime, const double* t_ssbef,
                                const double* t_h2osfc_bef, const double* t_grnd0, const double* begwb,
                                double* errsoi, double* errh2o, void* stream) {
  const ClmgbRange range_("clmgb_balance_residuals");
  if (!handle_ok(h)) return CLMGB_ERR_HANDLE;
  int32_t e = check_bounds(b, true);
  if (e) return e;
  if (b->nc == 0) return CLMGB_OK;
  if ((e = check_fields(ft))) return e;
  if ((e = check_fields(fw))) return e;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  if (!t_ssbef || !t_h2osfc_bef || !t_grnd0 || !begwb || !errsoi || !errh2o) return CLMGB_ERR_NULL_ARG;
  cudaError_t ce = clmgb::launch_balance_residuals(hdims(h, *b), b->nc, *ft, *fw, dtime, t_ssbef, t_h2osfc_bef,
                                                   t_grnd0, begwb, errsoi, errh2o, (cudaStream_t)stream);
  return ce == cudaSuccess ? CLMGB_OK : cuda_fail(h, ce);
}

}  // extern "C"
