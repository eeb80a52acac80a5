// launch.h — internal launchers shared by the host API (api.cu) and the kernel
// translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/clmgb.h"

namespace clmgb {

struct Dims;

// Per-column scratch of a handle reserved with clmgb_reserve (capacity columns):
// precomputed ice impedances [nlevsoi, capacity], the work-queue order and its
// counting-sort bins (2*64+1 words).
struct QueueScratch {
  int64_t capacity;
  double* imp;
  uint32_t* order;
  unsigned int* bins;
  int longest_first;
  int fresh_batch;   // CLMGB_OPT_QUEUE_FRESH_BATCH (0: refresh at once)
  // CLMGB_OPT_QUEUE_PACKED_REFRESH: the warp refreshes its fresh lanes' columns
  // together, (column, level) pairs spread over the 32 lanes (k_moisture_form_packed)
  int packed;
  // one record per column, contiguous: [capacity][PC_ALL][nlevsoi] (PcField): the
  // packed refresh's inputs (the pre-pass k_column_records fills them), so that a pass
  // over one column's levels reads consecutive addresses and the resident columns'
  // inputs stay in L2, and the column's water, smp_l and hk_l during the solve
  double* pcache;
  // 1 while the solve keeps a column's water, smp_l and hk_l in its record (the packed
  // kernel); the post-pass k_column_outputs writes them to the state at the end
  int out_records = 0;
  // CLMGB_OPT_QUEUE_DEFER: a column still unfinished after `defer` attempts leaves the
  // work queue at its next accepted substep; its state (water [nlevsoi][capacity],
  // dtsub, dtdone, qcharge so far, attempts, status at index c) and its index (list)
  // are kept for the warp-per-column finish (richards_coop.cuh).  d_count: the
  // claimed, published and consumed list slots.  0: off.
  int defer;
  double *d_liq, *d_dtsub, *d_dtdone, *d_qc;
  int* d_nsub;
  uint32_t* d_status;
  uint32_t* d_list;
  unsigned long long* d_count;
  // polls of a list slot whose index is still on its way before the drain gives the
  // slot back (CLMGB_OPT_QUEUE_POLL_LIMIT), and a delay in ns between the publication
  // of an even slot and the write of its index (CLMGB_OPT_QUEUE_PUBLISH_DELAY, 0 in
  // production: it lets a test make that wait run out)
  int poll_limit = DEFER_POLL_LIMIT;
  int publish_delay = 0;
  // CLMGB_OPT_COUNT_WORK: when set, the packed kernel and the warp-per-column finish add
  // the levels of every substep attempt to work[0] and of every hydraulic refresh to
  // work[1] (the FP64 work model of the solve, clmgb/flops_model.py); NULL otherwise
  unsigned long long* work = nullptr;
  // CLMGB_OPT_RECORDS_TMA: the column-record pre-pass stages its tiles with tensor copies
  int records_tma = 1;
  int* records_tma_used = nullptr;   // set to 1 when the last pre-pass used tensor copies
};

// Per-column state of the wave-synchronous Richards solve (richards_waves.cu), from
// the same reserved block: level arrays are [nlevsoi][cap], the rest [cap].
struct WaveScratch {
  int64_t cap;
  double *imp, *qout, *dqodw1, *dqodw2, *fnet1, *dtdz;
  double *dtsub, *dtdone, *qc, *dtcur, *hk_bot, *dhkdw_bot;
  int* nsub;
  uint32_t* status;
  uint32_t* listA[2];
  uint32_t* listH[2];
  unsigned int* counters;
};

// Tape of the column-step adjoint (adjoint_step.cu): slots x entries records.
struct AdjTape {
  int2* idx;
  double2* par;
  double* adj;
  double* sub;
  int64_t slots, entries, maxsub;
  unsigned int* max_used;
  int richards_mode;
};

// A substep log of the moisture-form solve (clmgb_substep_log): per column a region
// of `stride` doubles at rec + c*stride holding up to `cap` records of SUB_REC
// doubles (the liquid water at the start of an accepted substep, its dtsub and the
// time done before it) followed by the solve's outputs; count[c] = accepted
// substeps (-1: the column was not solved).  rec == nullptr: no log.  st, when not
// null, holds per column CLMGB_LOG_ST_STRIDE doubles of soil_temperature! (StLog).
struct SubstepLogView {
  double* rec;
  int32_t* count;
  int cap;
  int64_t stride;
  double* st;
};

// The soil_temperature! record of a column (clmgb_substep_log::st_rec): the band
// system's size n, the status of the call, t_grnd and t_h2osfc after it, then
// temperature, liquid water, ice and fact after it (index jj-1 of level jj), the
// solution x, the factors (n rows of 7, band_lu_factor_solve's layout) and the row
// exchanges (one byte each).
enum StLog {
  ST_N = 0, ST_STATUS = 1, ST_TG = 2, ST_TH = 3,
  ST_T = 4,
  ST_LIQ = ST_T + CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND,
  ST_ICE = ST_LIQ + CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND,
  ST_FACT = ST_ICE + CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND,
  ST_X = ST_FACT + CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND,
  ST_LU = ST_X + CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND + 1,
  ST_PIV = ST_LU + 7 * (CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND + 1),
  ST_END = ST_PIV + (CLMGB_MAX_NLEVSNO + CLMGB_MAX_NLEVGRND + 1 + 7) / 8
};
static_assert(ST_END <= CLMGB_LOG_ST_STRIDE, "soil_temperature! record exceeds CLMGB_LOG_ST_STRIDE");

// fields of a column record (QueueScratch::pcache): the inputs dz*1000, watsat, bsw,
// hksat, sucsat, the ice impedance, 1000*(z[j+1]-z[j]) (levels below the bottom one)
// and qflx_rootsoi; then the column's liquid water (the state's at the start, the
// solve's at its end), smp_l and hk_l (written at every hydraulic refresh)
enum PcField { PC_DZW = 0, PC_WS, PC_BSW, PC_KS, PC_SUC, PC_IMP, PC_DEN, PC_ROOT, PC_FIELDS,
               PC_LIQ = PC_FIELDS, PC_SMP, PC_HK, PC_ALL };

// All launchers return the cudaError_t of the launch (cudaGetLastError()).
cudaError_t launch_soil_temperature(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double dtime,
                                    int snow_method, uint32_t* col_status, uint32_t* dev_status,
                                    cudaStream_t s);
cudaError_t launch_water_fractions(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, cudaStream_t s);
cudaError_t launch_moisture_form(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                 const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                 uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_column_step(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                               const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                               int snow_method, double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                               uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_phase_change(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double dtime,
                                const double* dhsdT, int which, cudaStream_t s);
cudaError_t launch_band_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* bmatrix,
                              const double* rvector, const int64_t* jtop, const int64_t* jbot,
                              const uint8_t* mask, int kl, int ku, int nlevsno_off, cudaStream_t s);
cudaError_t launch_tridiagonal_multi(int64_t ncols, int64_t ldc, int nlevs, double* u, const double* a,
                                     const double* b, const double* c, const double* r, const int64_t* jtop,
                                     const uint8_t* mask, cudaStream_t s,
                                     int method = CLMGB_TRIDIAG_THOMAS);
cudaError_t launch_synth_forcing(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                 const clmgb_soilwater_fields& fw, const double* G, const double* I,
                                 cudaStream_t s);

// The column-record pre-pass of the work-queue Richards solve (records.cu)
size_t column_records_smem(int nlevsoi);
cudaError_t launch_column_records(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, double e_ice,
                                  double* imp_cache, int64_t ld_imp, double* pcache, bool tma, uint32_t* dev_status,
                                  cudaStream_t s, int* tma_used = nullptr);
bool column_records_tma_available();
// writes the solved columns' water, smp_l and hk_l from their records to the state
cudaError_t launch_column_outputs(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, const double* pcache,
                                  cudaStream_t s);

// st_log (optional): the soil_temperature! records of a substep log (StLog)
cudaError_t launch_soiltemp_fractions(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                      const clmgb_soilwater_fields& fw, double dtime, int snow_method,
                                      double* t_ssbef, double* t_h2osfc_bef, uint32_t* col_status,
                                      uint32_t* dev_status, cudaStream_t s, double* st_log = nullptr);
int queue_blocks_per_sm();
cudaError_t launch_moisture_form_queue(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                       const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                       int or_status, uint32_t* dev_status, unsigned long long* queue,
                                       int grid_blocks, const QueueScratch& qs, cudaStream_t s,
                                       const double* dt_init = nullptr, const SubstepLogView* log = nullptr);
// compute_qcharge! over the solved state when cfg's lower boundary is the water table
// (a no-op otherwise); every moisture-form entry point runs it after its solve.
cudaError_t launch_compute_qcharge(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                  const clmgb_swm_config& cfg, double dtime, cudaStream_t s);
cudaError_t launch_flexible_cn(const Dims& D, int64_t nc, const clmgb_flexcn_fields& f, cudaStream_t s);
cudaError_t launch_noalloc_soil_water(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                      const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                      cudaStream_t s);
int waves_blocks_per_sm();
cudaError_t launch_moisture_form_waves(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                       const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                       int or_status, uint32_t* dev_status, const WaveScratch& w, int grid_blocks,
                                       cudaStream_t s);
cudaError_t launch_math_eval(int op, int64_t n, const double* x, const double* y, double* out, cudaStream_t s);
cudaError_t launch_column_step_vjp(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                   const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                                   int snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                   const clmgb_step_adjoint& adj, const AdjTape& tp, uint32_t* col_status,
                                   uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_rootsink(const Dims& D, int64_t nc, int64_t nl, const clmgb_rootsink_fields& f, int hydrstress,
                            uint32_t* col_status, uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_zd09(const Dims& D, int64_t nc, const clmgb_zd09_fields& f, double e_ice, double dtime,
                        cudaStream_t s);
cudaError_t launch_surface_hydrology(const Dims& D, int64_t nc, int64_t nl, const clmgb_surfhyd_fields& f,
                                     const clmgb_surfhyd_config& P, uint32_t stages, double dtime, uint32_t* dev_status,
                                     cudaStream_t s);
cudaError_t launch_snow_layers(const Dims& D, int64_t nc, int64_t nl, const clmgb_snowlayer_fields& f,
                               const clmgb_snowlayer_config& P, uint32_t stages, double dtime, uint32_t* dev_status,
                               cudaStream_t s);
cudaError_t launch_lake_temperature(const Dims& D, int64_t nc, const clmgb_lake_fields& f, const clmgb_lake_config& P,
                                    double dtime, uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_colbalance(int64_t nc, const clmgb_colbalance_fields& f, double dtime, unsigned long long* r,
                              cudaStream_t s);
cudaError_t launch_soil_fluxes(const Dims& D, int64_t nc, int64_t nl, const clmgb_soilflux_fields& f, double dtime,
                               uint32_t* dev_status, cudaStream_t s);
int vjp_cf_blocks_per_sm();
cudaError_t launch_column_step_vjp_cf(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                      const clmgb_soilwater_fields& fw, const clmgb_swm_config& cfg, double dtime,
                                      int snow_method, double* t_ssbef, double* t_h2osfc_bef,
                                      const clmgb_step_adjoint& adj, const AdjTape& tp, const SubstepLogView& lg,
                                      const QueueScratch& qs, unsigned long long* queue, int grid_blocks,
                                      uint32_t* col_status, uint32_t* dev_status, cudaStream_t s);
cudaError_t launch_band_factor_solve(int64_t nc, int64_t ldc, int nlev, double* tvector, const double* bmatrix,
                                     const double* rvector, const int64_t* jtop, const int64_t* jbot,
                                     const uint8_t* mask, int kl, int ku, int nlevsno_off, double* lu, uint8_t* piv,
                                     cudaStream_t s);
cudaError_t launch_band_solve_adjoint(int64_t nc, int64_t ldc, int nlev, const double* tvector, double* tbar,
                                      const double* lu, const uint8_t* piv, double* bbar, double* rbar,
                                      const int64_t* jtop, const int64_t* jbot, const uint8_t* mask, int kl, int ku,
                                      int nlevsno_off, cudaStream_t s);
cudaError_t launch_tridiagonal_adjoint(int64_t ncols, int64_t ldc, int nlevs, const double* u, const double* a,
                                       const double* b, const double* c, double* ubar, double* abar, double* bbar,
                                       double* cbar, double* rbar, const int64_t* jtop, const uint8_t* mask,
                                       cudaStream_t s);

cudaError_t launch_mlp_linear(int64_t M, int N, int K, const void* X, int64_t ldx, const void* W, const float* b,
                              int act, float* Z, int64_t ldz, void* Y, int64_t ldy, cudaStream_t s);
cudaError_t launch_mlp_linear_dw(int64_t M, int N, int K, const void* dZ, int64_t lddz, const void* X, int64_t ldx,
                                 float* dW, float* db, cudaStream_t s);
cudaError_t launch_mlp_silu_backward(int64_t n, const float* Z, const void* dY, void* dZ, cudaStream_t s);
cudaError_t launch_mlp_loss(int64_t M, const float* Y, const float* T, float w0, float w1, float* loss, void* dY,
                            cudaStream_t s);
cudaError_t launch_mlp_adam(int64_t rows, int64_t cols, float* w, const float* g, float* m, float* v, float lr,
                            float b1, float b2, float eps, int step, void* wb, void* wbt, cudaStream_t s);
cudaError_t launch_richards_samples(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                    const clmgb_swm_config& cfg, double dtime, int rmax, float* feat, float* targ,
                                    unsigned int* count, int64_t capacity, uint32_t* col_status, cudaStream_t s);
cudaError_t launch_mlp_features(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                const clmgb_swm_config& cfg, double dtime, const float* mean, const float* istd,
                                void* X, cudaStream_t s);
cudaError_t launch_mlp_first_dt(int64_t nc, const float* Y, double dtime, float margin, int kmax, double* dt_first,
                                cudaStream_t s);

cudaError_t launch_balance_begin(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& f, double* t_grnd0,
                                 double* begwb, cudaStream_t s);
cudaError_t launch_balance_residuals(const Dims& D, int64_t nc, const clmgb_soiltemp_fields& ft,
                                     const clmgb_soilwater_fields& fw, double dtime, const double* t_ssbef,
                                     const double* t_h2osfc_bef, const double* t_grnd0, const double* begwb,
                                     double* errsoi, double* errh2o, cudaStream_t s);

}  // namespace clmgb
