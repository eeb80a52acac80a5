// noalloc.cu — soil_water! (moisture form) for callers that cannot allocate GPU memory.
//
// The handle API (clmgb_create) obtains its scratch with cudaMalloc.  Some callers
// cannot do that: a host runtime that owns the device memory pool and forbids
// foreign allocations, a caller inside stream capture (cudaMalloc is not a
// capturable operation), or embedded code built without an allocator.
// clmgb_soil_water_noalloc serves them: it allocates nothing and keeps its scratch
// in the file-scope device array below, which every GPU that loads this library
// holds until the process exits.
//
// The scratch is 16 bytes of counters plus a list of the columns to solve (one
// 32-bit index per column), so one call accepts at most CLMGB_NOALLOC_MAX_COLUMNS
// columns (4 MiB of list); larger calls are rejected with CLMGB_ERR_DIMS.  Every
// call shares the array and it keeps the last call's contents: each call zeroes
// its counters first.  Two calls whose work overlaps on the GPU (different streams
// or devices sharing a context without ordering) race on the array and must not be
// issued; serialise them on one stream.
//
// Every call looks up the array's device address in the current context with
// cudaGetSymbolAddress, with that device current.  The first call on a device loads
// the library's module there, which stream capture does not allow: make that first
// call before any stream capture.
#include <atomic>
#include <string.h>
#include <cuda_runtime.h>
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr int NOALLOC_BLOCK = 128;
constexpr int NOALLOC_MAX_DEVICES = 64;

// [0] queue counter, [1] number of listed columns, then the column list (uint32)
static __device__ __align__(256) unsigned long long g_noalloc_scratch[2 + CLMGB_NOALLOC_MAX_COLUMNS / 2];

static std::atomic<int> g_noalloc_grid[NOALLOC_MAX_DEVICES];

// Lists the columns with mask[c] set (order irrelevant: columns are independent).
__global__ void __launch_bounds__(NOALLOC_BLOCK)
k_noalloc_list_columns(int64_t nc, const uint8_t* mask, uint32_t* col_status, unsigned long long* scratch) {
  const int64_t c = (int64_t)blockIdx.x * NOALLOC_BLOCK + threadIdx.x;
  if (c >= nc) return;
  if (!mask[c]) {
    if (col_status) col_status[c] = 0;
    return;
  }
  uint32_t* list = reinterpret_cast<uint32_t*>(scratch + 2);
  const unsigned long long slot = atomicAdd(scratch + 1, 1ull);
  list[slot] = (uint32_t)c;
}

// The work-queue Richards kernel over the listed columns; same per-column device
// functions (mf_begin / mf_attempt / mf_end) as the handle path.
__global__ void __launch_bounds__(NOALLOC_BLOCK)
k_noalloc_moisture_form(Dims D, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                        uint32_t* col_status, unsigned long long* scratch) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t* list = reinterpret_cast<const uint32_t*>(scratch + 2);
  const unsigned long long nlisted = *(volatile unsigned long long*)(scratch + 1);
  MfLane L;
  bool active = false, exhausted = false;
  for (;;) {
    const bool need = !active && !exhausted;
    const unsigned m = __ballot_sync(FULL, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(scratch, (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        const unsigned long long k = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
        if (k >= nlisted) {
          exhausted = true;
        } else {
          const int64_t c = (int64_t)list[k];
          if (mf_begin(L, D, f, cfg, dtime, c)) active = true;
          else if (col_status) col_status[c] = L.status;
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (__all_sync(FULL, exhausted)) break;
      continue;
    }
    if (active && mf_attempt(L, D, f, cfg, dtime)) {
      const uint32_t st = mf_end(L, D, f);
      if (col_status) col_status[L.c] = st;
      active = false;
    }
  }
}

// Device address of the scratch array in the current context, and the grid of the
// solve kernel on the current device.  The address is looked up on every call: a
// __device__ array's address belongs to a CUDA context, so a pointer kept from an
// earlier call would dangle after cudaDeviceReset or under another context on the
// same device.  Once the library's module is loaded (by the first call) the lookup
// neither allocates nor synchronises, so later calls may run under stream capture.
// The occupancy-derived grid depends on the device only and is kept per device.
static cudaError_t noalloc_setup(unsigned long long** out, int* grid) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  void* sym = nullptr;
  e = cudaGetSymbolAddress(&sym, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  int g = g_noalloc_grid[dev].load();
  if (g <= 0) {
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_moisture_form, NOALLOC_BLOCK, 0);
    if (e != cudaSuccess) return e;
    g = sms * (per_sm > 0 ? per_sm : 1);
    g_noalloc_grid[dev].store(g);
  }
  *out = static_cast<unsigned long long*>(sym);
  *grid = g;
  return cudaSuccess;
}

cudaError_t launch_noalloc_soil_water(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                      const clmgb_swm_config& cfg, double dtime, uint32_t* col_status,
                                      cudaStream_t s) {
  unsigned long long* scratch = nullptr;
  int grid = 0;
  cudaError_t e = noalloc_setup(&scratch, &grid);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned long long), s);   // queue counter, list length
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((nc + NOALLOC_BLOCK - 1) / NOALLOC_BLOCK);
  k_noalloc_list_columns<<<blocks, NOALLOC_BLOCK, 0, s>>>(nc, f.mask_hydrology, col_status, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int g = (int)((int64_t)blocks < grid ? blocks : grid);
  k_noalloc_moisture_form<<<g > 0 ? g : 1, NOALLOC_BLOCK, 0, s>>>(D, f, cfg, dtime, col_status, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_compute_qcharge(D, nc, f, cfg, dtime, s);
}

}  // namespace clmgb

extern "C" int32_t clmgb_soil_water_noalloc(const clmgb_varpar* vp, const clmgb_bounds* b,
                                            const clmgb_soilwater_fields* f, const clmgb_swm_config* cfg,
                                            double dtime, uint32_t* col_status, void* stream) {
  if (!vp || !b || !f || !cfg) return CLMGB_ERR_NULL_ARG;
  if (vp->nlevsno < 1 || vp->nlevsno > CLMGB_MAX_NLEVSNO || vp->nlevgrnd < 2 || vp->nlevgrnd > CLMGB_MAX_NLEVGRND ||
      vp->nlevsoi < 1 || vp->nlevsoi > vp->nlevgrnd || vp->nlevsoi > CLMGB_MAX_NLEVSOI ||
      vp->nlevurb < 0 || vp->nlevurb > vp->nlevgrnd || vp->nlevmaxurbgrnd != vp->nlevgrnd)
    return CLMGB_ERR_DIMS;
  if (b->nc < 0 || b->ldc < b->nc) return CLMGB_ERR_DIMS;
  if (b->nc > CLMGB_NOALLOC_MAX_COLUMNS) return CLMGB_ERR_DIMS;     // beyond the static scratch
  if (cfg->soilwater_movement_method == CLMGB_ZENGDECKER_2009) return CLMGB_ERR_UNSUPPORTED;
  if (cfg->soilwater_movement_method != CLMGB_MOISTURE_FORM || cfg->upper_boundary_condition != CLMGB_BC_FLUX)
    return CLMGB_ERR_CONFIG;
  if (!(cfg->lower_boundary_condition == CLMGB_BC_WATERTABLE || cfg->lower_boundary_condition == CLMGB_BC_FLUX ||
        cfg->lower_boundary_condition == CLMGB_BC_ZERO_FLUX))
    return CLMGB_ERR_CONFIG;
  if ((cfg->flux_calculation != 1 && cfg->flux_calculation != 42) || !(cfg->dtmin > 0.0)) return CLMGB_ERR_CONFIG;
  if (!(dtime > 0.0)) return CLMGB_ERR_CONFIG;
  if (b->nc == 0) return CLMGB_OK;
  if (f->struct_size != (int64_t)sizeof(clmgb_soilwater_fields)) return CLMGB_ERR_ABI;
  const char* base = reinterpret_cast<const char*>(f) + sizeof(int64_t);
  for (size_t i = 0; i < (sizeof(clmgb_soilwater_fields) - sizeof(int64_t)) / sizeof(void*); i++) {
    const void* p;
    memcpy(&p, base + i * sizeof(void*), sizeof(void*));
    if (!p) return CLMGB_ERR_NULL_ARG;
  }
  clmgb::Dims D;
  D.nlevsno = vp->nlevsno;
  D.nlevgrnd = vp->nlevgrnd;
  D.nlevsoi = vp->nlevsoi;
  D.nlevurb = vp->nlevurb;
  D.nlevmax = vp->nlevmaxurbgrnd;
  D.ldc = b->ldc;
  D.ldp = b->ldp;
  D.np = b->np;
  const cudaError_t e = clmgb::launch_noalloc_soil_water(D, b->nc, *f, *cfg, dtime, col_status, (cudaStream_t)stream);
  return e == cudaSuccess ? CLMGB_OK : CLMGB_ERR_CUDA;
}
