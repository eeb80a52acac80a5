// records.cu — the pre-pass and the post-pass of the work-queue Richards solve.
//
// Pre-pass (k_column_records): every hydrology column's ice impedances (imp_cache,
// [nlevsoi][ld_imp]) and its record (QueueScratch::pcache, [column][PC_ALL][nlevsoi]):
// the packed refresh's inputs and the column's liquid water, by tiles of 32 columns.
// A block stages the tile's levels of the nine fields it reads (dz, z, watsat, bsw,
// hksat, sucsat, qflx_rootsoi, icefrac, h2osoi_liq: [level][column] arrays, columns
// fastest) in shared memory, forms the record values of every (level, column) pair,
// and writes the 32 records as contiguous ranges.  Two ways to stage the tile:
//   * plain loads: the block's threads read the tile row by row (coalesced);
//   * TMA (cp.async.bulk.tensor.2d): one thread issues a 2-D tensor copy of each
//     field's [nlevsoi x 32] box, completing on an mbarrier the block waits on.  The
//     tensor maps cover this GPU's own arrays; no multicast, no cluster.
// Both give the same bits (every value is the expression of the per-column pass).
// Entries of columns the solve skips, and levels below a column's bottom, are zero.
//
// Shared memory: the nine input tiles [9][nlevsoi][32], then the same bytes reused
// as the output tile [32][9*nlevsoi + 1] (the +1 keeps the transposed reads and writes
// free of bank conflicts).
//
// Post-pass (k_column_outputs): the solve keeps each column's water, smp_l and hk_l in
// its record (contiguous, so that the many refreshes of a column write whole sectors);
// the post-pass moves them to the [level][column] state arrays a tile at a time, rows
// coalesced, for the columns the solve ran on.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <string.h>
#include <mutex>
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

namespace {

constexpr int RC_COLS = 32, RC_THREADS = 256, RC_FIELDS_IN = 9;
constexpr int RC_PER_THREAD = (MAXSOI * RC_COLS + RC_THREADS - 1) / RC_THREADS;   // (level, column) pairs
constexpr int RC_OUT = PC_LIQ + 1;                  // record fields the pre-pass writes
enum RcIn { RI_DZ = 0, RI_Z, RI_WS, RI_BSW, RI_KS, RI_SUC, RI_ROOT, RI_ICEF, RI_LIQ };

// upper bound of the TMA wait (ns of %globaltimer): a tile copy takes microseconds
constexpr unsigned long long RC_WAIT_NS = 200000000ull;

struct RecordMaps {
  CUtensorMap m[RC_FIELDS_IN];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}
// waits for phase `phase` of the barrier for at most RC_WAIT_NS; false on expiry
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) {
  if (mbar_try_wait(bar, phase)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, phase))
    if (globaltimer_ns() - t0 > RC_WAIT_NS) return false;
  return true;
}

template <bool TMA>
__global__ void __launch_bounds__(RC_THREADS)
k_column_records(Dims D, int64_t nc, clmgb_soilwater_fields f, double e_ice, double* imp_cache, int64_t ld_imp,
                 double* pcache, const __grid_constant__ RecordMaps maps, uint32_t* dev_status) {
  extern __shared__ __align__(128) unsigned char rc_smem[];
  __shared__ __align__(8) unsigned long long bar;
  double* tile = reinterpret_cast<double*>(rc_smem);            // [RC_FIELDS_IN][nls][RC_COLS]
  const int nls = D.nlevsoi, joff = D.nlevsno;
  const int64_t ld = D.ldc;
  const int64_t c0 = (int64_t)blockIdx.x * RC_COLS;
  const int tid = threadIdx.x;
  const int box = nls * RC_COLS;
#define TL(k, j, cl) tile[((k) * nls + ((j) - 1)) * RC_COLS + (cl)]
  if (TMA) {
    const uint32_t b = smem_u32(&bar);
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
      const uint32_t bytes = (uint32_t)(RC_FIELDS_IN * box * sizeof(double));
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
      for (int k = 0; k < RC_FIELDS_IN; k++) {
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
            ::"r"(smem_u32(tile + (size_t)k * box)), "l"(reinterpret_cast<uint64_t>(&maps.m[k])),
              "r"((int)c0), "r"(0), "r"(b)
            : "memory");
      }
    }
    const bool ok = mbar_wait_bounded(b, 0);
    if (__syncthreads_or(!ok)) {
      // the tile never arrived: record it, give the copies one more bounded wait, and
      // leave this tile's records unwritten (the whole block returns together)
      if (tid == 0 && dev_status) atomicOr(dev_status, CLMGB_COL_COPY_WAIT);
      if (!ok) mbar_wait_bounded(b, 0);
      return;
    }
  } else {
    for (int idx = tid; idx < box; idx += RC_THREADS) {
      const int j = idx / RC_COLS + 1, cl = idx % RC_COLS;
      const int64_t c = c0 + cl;
      const bool in = c < nc;
      TL(RI_DZ, j, cl) = in ? LVc(f.dz, c, joff + j, ld) : 0.0;
      TL(RI_Z, j, cl) = in ? LVc(f.z, c, joff + j, ld) : 0.0;
      TL(RI_WS, j, cl) = in ? LVc(f.watsat, c, j, ld) : 0.0;
      TL(RI_BSW, j, cl) = in ? LVc(f.bsw, c, j, ld) : 0.0;
      TL(RI_KS, j, cl) = in ? LVc(f.hksat, c, j, ld) : 0.0;
      TL(RI_SUC, j, cl) = in ? LVc(f.sucsat, c, j, ld) : 0.0;
      TL(RI_ROOT, j, cl) = in ? LVc(f.qflx_rootsoi, c, j, ld) : 0.0;
      TL(RI_ICEF, j, cl) = in ? LV(f.icefrac, c, j, ld) : 0.0;
      TL(RI_LIQ, j, cl) = in ? LV(f.h2osoi_liq, c, joff + j, ld) : 0.0;
    }
    __syncthreads();
  }
  // ---- the record values of this thread's (level, column) pairs, in registers ----
  double v[RC_PER_THREAD][RC_OUT];
  double ln10_lo;
  const double ln10 = cm_log_dd(10.0, &ln10_lo);
#pragma unroll
  for (int e = 0; e < RC_PER_THREAD; e++) {
    const int idx = tid + e * RC_THREADS;
#pragma unroll
    for (int k = 0; k < RC_OUT; k++) v[e][k] = 0.0;
    if (idx >= box) continue;
    const int j = idx / RC_COLS + 1, cl = idx % RC_COLS;
    const int64_t c = c0 + cl;
    if (c >= nc || !f.mask_hydrology[c]) continue;
    const int64_t nl = f.col_nbedrock[c];
    if (nl < 1 || nl > nls || j > nl) continue;
    const int nlayers = (int)nl;
    // mf_impedance (soil_water_movement.jl:1287-1293)
    const double icef = (j == nlayers) ? TL(RI_ICEF, j, cl) : 0.5 * (TL(RI_ICEF, j, cl) + TL(RI_ICEF, j + 1, cl));
    const double imp = cm_pow_lx(10.0, ln10, ln10_lo, -e_ice * icef);
    imp_cache[(int64_t)(j - 1) * ld_imp + c] = imp;
    v[e][PC_DZW] = TL(RI_DZ, j, cl) * DENH2O;
    v[e][PC_WS] = TL(RI_WS, j, cl);
    v[e][PC_BSW] = TL(RI_BSW, j, cl);
    v[e][PC_KS] = TL(RI_KS, j, cl);
    v[e][PC_SUC] = TL(RI_SUC, j, cl);
    v[e][PC_IMP] = imp;
    if (j < nlayers) v[e][PC_DEN] = M_TO_MM * (TL(RI_Z, j + 1, cl) - TL(RI_Z, j, cl));
    v[e][PC_ROOT] = TL(RI_ROOT, j, cl);
    v[e][PC_LIQ] = TL(RI_LIQ, j, cl);
  }
#undef TL
  __syncthreads();   // every input read: the output tile reuses the bytes
  const int rec = RC_OUT * nls, pitch = rec + 1, stride = PC_ALL * nls;
  double* out_t = tile;                                          // [RC_COLS][pitch]
#pragma unroll
  for (int e = 0; e < RC_PER_THREAD; e++) {
    const int idx = tid + e * RC_THREADS;
    if (idx >= box) continue;
    const int j = idx / RC_COLS + 1, cl = idx % RC_COLS;
#pragma unroll
    for (int k = 0; k < RC_OUT; k++) out_t[cl * pitch + k * nls + (j - 1)] = v[e][k];
  }
  __syncthreads();
  const int64_t ncols = (nc - c0) < RC_COLS ? (nc - c0) : RC_COLS;
  double* out = pcache + c0 * stride;
  for (int idx = tid; idx < ncols * rec; idx += RC_THREADS) {
    const int cl = idx / rec, r = idx % rec;
    out[(int64_t)cl * stride + r] = out_t[cl * pitch + r];
  }
}

// The post-pass: water, smp_l and hk_l of levels 1..nbedrock of every column the solve
// ran on (mask_hydrology set, nbedrock within 1..nlevsoi), from the records.
constexpr int RO_FIELDS = PC_ALL - PC_LIQ;
__global__ void __launch_bounds__(RC_THREADS)
k_column_outputs(Dims D, int64_t nc, clmgb_soilwater_fields f, const double* pcache) {
  extern __shared__ __align__(128) unsigned char ro_smem[];
  double* t = reinterpret_cast<double*>(ro_smem);                 // [RC_COLS][RO_FIELDS*nls + 1]
  const int nls = D.nlevsoi, joff = D.nlevsno;
  const int64_t ld = D.ldc;
  const int64_t c0 = (int64_t)blockIdx.x * RC_COLS;
  const int tid = threadIdx.x;
  const int part = RO_FIELDS * nls, pitch = part + 1, stride = PC_ALL * nls;
  const int64_t ncols = (nc - c0) < RC_COLS ? (nc - c0) : RC_COLS;
  const double* in = pcache + c0 * stride + PC_LIQ * nls;
  for (int idx = tid; idx < ncols * part; idx += RC_THREADS) {
    const int cl = idx / part, r = idx % part;
    t[cl * pitch + r] = in[(int64_t)cl * stride + r];
  }
  __syncthreads();
  for (int idx = tid; idx < RO_FIELDS * nls * RC_COLS; idx += RC_THREADS) {
    const int k = idx / (nls * RC_COLS), rem = idx % (nls * RC_COLS);
    const int j = rem / RC_COLS + 1, cl = rem % RC_COLS;
    const int64_t c = c0 + cl;
    if (c >= nc || !f.mask_hydrology[c]) continue;
    const int64_t nl = f.col_nbedrock[c];
    if (nl < 1 || nl > nls || j > nl) continue;
    const double v = t[cl * pitch + k * nls + (j - 1)];
    if (k == 0) LV(f.h2osoi_liq, c, joff + j, ld) = v;
    else if (k == 1) LV(f.smp_l, c, j, ld) = v;
    else LV(f.hk_l, c, j, ld) = v;
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// A [rows x nc] float64 array with row stride ld (elements), box nls x 32; false
// when the array does not meet the tensor copy's alignment rules.
bool encode_map(CUtensorMap* m, const double* base, int64_t nc, int rows, int64_t ld, int nls) {
  auto fn = encode_fn();
  if (!fn || !base) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * (int64_t)sizeof(double)) & 15)) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nc, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)(ld * (int64_t)sizeof(double))};
  const cuuint32_t boxd[2] = {(cuuint32_t)RC_COLS, (cuuint32_t)nls};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(base), dims, strides, boxd, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t column_records_smem(int nlevsoi) {
  const size_t in = (size_t)RC_FIELDS_IN * nlevsoi * RC_COLS * sizeof(double);
  const size_t out = (size_t)RC_COLS * (RC_OUT * nlevsoi + 1) * sizeof(double);
  return in > out ? in : out;
}

cudaError_t launch_column_records(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, double e_ice,
                                  double* imp_cache, int64_t ld_imp, double* pcache, bool tma, uint32_t* dev_status,
                                  cudaStream_t s, int* tma_used) {
  const int nls = D.nlevsoi;
  const size_t smem = column_records_smem(nls);
  RecordMaps maps;
  memset(&maps, 0, sizeof(maps));
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  bool use_tma = tma && nc < ((int64_t)1 << 31) && nls <= 256 &&
                 encode_map(&maps.m[RI_DZ], f.dz + (int64_t)joff * ld, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_Z], f.z + (int64_t)joff * ld, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_WS], f.watsat, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_BSW], f.bsw, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_KS], f.hksat, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_SUC], f.sucsat, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_ROOT], f.qflx_rootsoi, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_ICEF], f.icefrac, nc, nls, ld, nls) &&
                 encode_map(&maps.m[RI_LIQ], f.h2osoi_liq + (int64_t)joff * ld, nc, nls, ld, nls);
  if (tma_used) *tma_used = use_tma ? 1 : 0;
  auto kern = use_tma ? k_column_records<true> : k_column_records<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)((nc + RC_COLS - 1) / RC_COLS), RC_THREADS, smem, s>>>(D, nc, f, e_ice, imp_cache, ld_imp, pcache,
                                                                          maps, dev_status);
  return cudaGetLastError();
}

bool column_records_tma_available() { return encode_fn() != nullptr; }

cudaError_t launch_column_outputs(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f, const double* pcache,
                                  cudaStream_t s) {
  const size_t smem = (size_t)RC_COLS * (RO_FIELDS * D.nlevsoi + 1) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_column_outputs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_column_outputs<<<(unsigned)((nc + RC_COLS - 1) / RC_COLS), RC_THREADS, smem, s>>>(D, nc, f, pcache);
  return cudaGetLastError();
}

}  // namespace clmgb
