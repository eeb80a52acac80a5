// fp64_probe.cu — measures the FP64 throughput the roofline of the column solve is
// judged against: DFMA instructions per second on the whole device, and the rates of
// a correctly rounded division and of the library's pow and log10 (clm_math.h), whose
// ratios to the DFMA rate convert the solve's operation counts into DFMA-equivalent
// FP64 pipe work (clmgb/flops_model.py).  A measurement utility loaded by bench.py
// from its own library (libclmgb_probe.so); the solver never calls it.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../csrc/clm_math.h"

namespace {

constexpr int THREADS = 256;
constexpr int CHAINS = 8;

// CHAINS independent FMA chains per thread, n rounds each
__global__ void __launch_bounds__(THREADS) k_dfma(int n, double b, double c, double* out) {
  double a[CHAINS];
  for (int k = 0; k < CHAINS; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < n; i++) {
#pragma unroll
    for (int k = 0; k < CHAINS; k++) a[k] = __fma_rn(a[k], b, c);
  }
  double s = 0.0;
  for (int k = 0; k < CHAINS; k++) s += a[k];
  if (s == 12345.678) out[0] = s;   // keeps the chains alive, never true
}

// correctly rounded divisions: 4 independent chains a <- d / a (stays near sqrt(d))
__global__ void __launch_bounds__(THREADS) k_ddiv(int n, double d, double* out) {
  double a[4];
  for (int k = 0; k < 4; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < n; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++) a[k] = __ddiv_rn(d, a[k]);
  }
  double s = a[0] + a[1] + a[2] + a[3];
  if (s == 12345.678) out[0] = s;
}

// the integer-pipe division the kernels use (cm_div): 4 independent chains a <- d / a
__global__ void __launch_bounds__(THREADS) k_idiv(int n, double d, double* out) {
  double a[4];
  for (int k = 0; k < 4; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < n; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++) a[k] = cm_div(d, a[k]);
  }
  double s = a[0] + a[1] + a[2] + a[3];
  if (s == 12345.678) out[0] = s;
}

// cm_pow(x, y) on x in [0.5, 1.5), y non-integral: 4 independent chains
__global__ void __launch_bounds__(THREADS) k_pow(int n, double y, double* out) {
  double a[4];
  for (int k = 0; k < 4; k++) a[k] = 0.6 + 1e-4 * (threadIdx.x + k);
  for (int i = 0; i < n; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++) a[k] = cm_pow(a[k], y) + 0.5;
  }
  double s = a[0] + a[1] + a[2] + a[3];
  if (s == 12345.678) out[0] = s;
}

__global__ void __launch_bounds__(THREADS) k_log10(int n, double* out) {
  double a[4];
  for (int k = 0; k < 4; k++) a[k] = 2.0 + 1e-4 * (threadIdx.x + k);
  for (int i = 0; i < n; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++) a[k] = cm_log10(a[k]) + 2.0;
  }
  double s = a[0] + a[1] + a[2] + a[3];
  if (s == 12345.678) out[0] = s;
}

template <class F>
static double time_ms(F launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();   // warm-up
  cudaEventRecord(e0);
  launch();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return (double)ms;
}

}  // namespace

// out[0] DFMA instructions per second (the device), out[1] divisions per second,
// out[2] cm_pow calls per second, out[3] cm_log10 calls per second, out[4] integer-pipe
// divisions (cm_div) per second.  blocks_per_sm
// resident 256-thread blocks on every SM.  Returns 0, or the CUDA error code.
extern "C" int clmgb_probe_fp64(int blocks_per_sm, double* out) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return (int)e;
  double* sink = nullptr;
  if ((e = cudaMalloc(&sink, sizeof(double))) != cudaSuccess) return (int)e;
  const int grid = sms * (blocks_per_sm > 0 ? blocks_per_sm : 4);
  const double threads = (double)grid * THREADS;
  const int nf = 4096, nd = 512, np = 128, nl = 128;
  const double t_fma = time_ms([&] { k_dfma<<<grid, THREADS>>>(nf, 0.999999, 1e-6, sink); });
  const double t_div = time_ms([&] { k_ddiv<<<grid, THREADS>>>(nd, 1.0000001, sink); });
  const double t_pow = time_ms([&] { k_pow<<<grid, THREADS>>>(np, 0.9, sink); });
  const double t_l10 = time_ms([&] { k_log10<<<grid, THREADS>>>(nl, sink); });
  const double t_idiv = time_ms([&] { k_idiv<<<grid, THREADS>>>(nd, 1.0000001, sink); });
  e = cudaGetLastError();
  cudaFree(sink);
  if (e != cudaSuccess) return (int)e;
  out[0] = threads * CHAINS * nf / (t_fma * 1e-3);
  out[1] = threads * 4 * nd / (t_div * 1e-3);
  out[2] = threads * 4 * np / (t_pow * 1e-3);
  out[3] = threads * 4 * nl / (t_l10 * 1e-3);
  out[4] = threads * 4 * nd / (t_idiv * 1e-3);
  return 0;
}
