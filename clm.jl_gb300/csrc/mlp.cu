// mlp.cu — the learned warm start of the moisture-form Richards solve.
//
// A 64 -> 128 -> 128 -> 21 multilayer perceptron (SiLU hidden layers, BF16 weights
// and activations, FP32 accumulation) proposes, for a column about to start a
// substep, how many times the remaining time must be halved before the solver's
// error test accepts the substep (output 0), together with the saturation increment
// of that substep on each of the 20 soil levels (outputs 1..20).  The solver takes
// the proposal as the size of its first attempt; its own accept/reject test
// (soil_water_movement.jl:1460-1463) still judges it and halves it if needed, so a
// result meets the same tolerance with or without the network.
//
// Kernels:
//   k_richards_samples    the plain solver, recording training pairs at the first R
//                         substep starts of every column: features, and the label
//                         found by trial attempts at remaining/2^k, k = 0, 1, ...
//   k_linear<K, N>        Y = act(X W^T + b) with mma.sync m16n8k16 (bf16 x bf16 ->
//                         fp32); one warp owns 16 rows and all N outputs
//   k_linear_dw<N, K>     dW += dZ^T X, db += sum dZ over a chunk of rows (CUDA cores,
//                         fp32 accumulation, one atomic add per element per chunk)
//   k_silu_backward, k_mlp_loss, k_adam
//   k_mlp_features        the 64 inputs of every column at the start of a call
//   k_mlp_first_dt        proposal -> first substep size
#include <cuda_bf16.h>
#include "clmgb_device.cuh"
#include "launch.h"

namespace clmgb {

constexpr int MLP_IN = 64, MLP_HID = 128, MLP_OUT = 21, MLP_OUTP = 32;
constexpr int FEAT_LEVELS = 20;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }

// ---------------------------------------------------------------------------
// Features of a column about to start a substep, in single precision (they are
// inputs to the network, not part of the solve):
//   0..19  saturation liq / (1000 dz watsat) of soil levels 1..20 (0 below the column)
//   20..39 ice fraction of the level (icefrac, set by set_soil_water_fractions!)
//   40..59 log10 of the hydraulic conductivity (mm/s): log10 ksat + (2b+3) log10 s1
//          - e_ice icefrac_interface, the logarithm of imp * ksat * s1^(2b+3)
//   60     infiltration into the top layer (1e3 mm/s units)
//   61     total transpiration sink (1e3 mm/s units)
//   62     remaining time of the step / dtime
//   63     log2(dtime / 60 s) / 6
// liq(j) gives the liquid water of soil level j.
// ---------------------------------------------------------------------------
template <class LiqF>
__device__ __forceinline__ void column_features(const Dims& D, const clmgb_soilwater_fields& f,
                                                const clmgb_swm_config& cfg, int64_t c, int nlayers, LiqF liq,
                                                double rem, double dtime, float* x) {
  const int64_t ld = D.ldc;
  const int joff = D.nlevsno;
  float s[FEAT_LEVELS + 2];
  float sink = 0.0f;
  for (int j = 1; j <= FEAT_LEVELS; j++) {
    const bool in = j <= nlayers;
    float sv = 0.0f;
    if (in) {
      const float dz = (float)LVc(f.dz, c, joff + j, ld);
      const float ws = (float)LVc(f.watsat, c, j, ld);
      sv = (float)liq(j) / (1000.0f * dz * ws);
      sink += (float)LVc(f.qflx_rootsoi, c, j, ld);
    }
    s[j] = sv;
    x[j - 1] = sv;
    x[19 + j] = in ? (float)LV(f.icefrac, c, j, ld) : 0.0f;
  }
  for (int j = 1; j <= FEAT_LEVELS; j++) {
    if (j > nlayers) {
      x[39 + j] = -30.0f;
      continue;
    }
    float s1 = (j == nlayers) ? s[j] : 0.5f * (s[j] + s[j + 1]);
    s1 = fminf(fmaxf(s1, 0.01f), 1.0f);
    const float fi = (j == nlayers) ? (float)LV(f.icefrac, c, j, ld)
                                    : 0.5f * (float)(LV(f.icefrac, c, j, ld) + LV(f.icefrac, c, j + 1, ld));
    const float b = (float)LVc(f.bsw, c, j, ld);
    x[39 + j] = log10f((float)LVc(f.hksat, c, j, ld)) + (2.0f * b + 3.0f) * log10f(s1) - (float)cfg.e_ice * fi;
  }
  x[60] = (float)(f.qflx_infl[c] * 1.0e3);
  x[61] = sink * 1.0e3f;
  x[62] = (float)(rem / dtime);
  x[63] = log2f((float)(dtime / 60.0)) / 6.0f;
}

// The plain solve of one column, recording up to rmax training pairs (one per
// substep start).  The label of a substep start is the smallest k for which an
// attempt at remaining/2^k (at least dtmin) is accepted; the trials run on a copy of
// the lane and do not change the solve.
__global__ void __launch_bounds__(64)
k_richards_samples(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime, int rmax,
                   float* feat, float* targ, unsigned int* count, int64_t capacity, uint32_t* col_status) {
  const int64_t c = (int64_t)blockIdx.x * 64 + threadIdx.x;
  if (c >= nc) return;
  if (!f.mask_hydrology[c]) return;
  MfLane L;
  if (!mf_begin(L, D, f, cfg, dtime, c)) {
    if (col_status) col_status[c] |= L.status;
    return;
  }
  const int64_t ld = D.ldc;
  int recorded = 0;
  bool done = false;
  while (!done) {
    if (L.fresh && recorded < rmax) {
      const double rem = dtime - L.dtdone;
      float x[MLP_IN];
      column_features(D, f, cfg, c, L.nlayers, [&](int j) { return L.liq[j]; }, rem, dtime, x);
      int k = 0;
      double incr[MAXSOI + 1];
      for (;; k++) {
        MfLane T = L;
        double dt = rem;
        for (int i = 0; i < k; i++) dt = jl_max(dt / 2.0, cfg.dtmin);
        T.dtsub = dt;
        const double before = T.dtdone;
        FieldState<clmgb_soilwater_fields> XT(f, c, ld);
        mf_attempt(T, D, f, cfg, dtime, XT);
        if (T.dtdone != before || dt <= cfg.dtmin || k >= 12) {
          for (int j = 1; j <= L.nlayers; j++)
            incr[j] = (T.liq[j] - L.liq[j]) / (M_TO_MM * L.dzv[j] * LVc(f.watsat, c, j, ld));
          break;
        }
      }
      const unsigned int slot = atomicAdd(count, 1u);
      if (slot < capacity) {
        for (int i = 0; i < MLP_IN; i++) feat[(int64_t)slot * MLP_IN + i] = x[i];
        float* t = targ + (int64_t)slot * MLP_OUTP;
        t[0] = (float)k;
        for (int j = 1; j <= FEAT_LEVELS; j++) t[j] = j <= L.nlayers ? (float)incr[j] : 0.0f;
        for (int j = FEAT_LEVELS + 1; j < MLP_OUTP; j++) t[j] = 0.0f;
      }
      recorded++;
    }
    FieldState<clmgb_soilwater_fields> X(f, c, ld);
    done = mf_attempt(L, D, f, cfg, dtime, X);
  }
  FieldState<clmgb_soilwater_fields> X(f, c, ld);
  const uint32_t st = mf_end(L, D, f, X);
  if (col_status) col_status[c] |= st;
}

// ---------------------------------------------------------------------------
// Y = act(X W^T + b): X [M x K] bf16 (row stride ldx), W [N x K] bf16, b [N] fp32;
// Z [M x N] fp32 pre-activation (optional), Y [M x N] bf16 (optional, row stride
// ldy).  64 rows per block of 4 warps.  mma.sync m16n8k16 fragments (PTX ISA):
// with g = lane/4 and t = lane%4, A regs hold rows g and g+8 at columns 2t, 2t+1
// and 2t+8, 2t+9; B regs hold columns 2t, 2t+1 and 2t+8, 2t+9 of row g of W (one
// output); C holds rows g, g+8 at outputs 2t, 2t+1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int K, int N>
__global__ void __launch_bounds__(128)
k_linear(int64_t M, const __nv_bfloat16* __restrict__ X, int64_t ldx, const __nv_bfloat16* __restrict__ W,
         const float* __restrict__ bias, int act, float* Z, int64_t ldz, __nv_bfloat16* Y, int64_t ldy) {
  constexpr int KP = K + 8;   // padded smem row (bank spread)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sW = (__nv_bfloat16*)smem_raw;
  __nv_bfloat16* sX = sW + N * KP;
  const int64_t row0 = (int64_t)blockIdx.x * 64;
  for (int i = threadIdx.x; i < N * K; i += 128) sW[(i / K) * KP + (i % K)] = W[i];
  for (int i = threadIdx.x; i < 64 * K; i += 128) {
    const int r = i / K, k = i % K;
    const int64_t gr = row0 + r;
    sX[r * KP + k] = gr < M ? X[gr * ldx + k] : __float2bfloat16(0.0f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int r0 = warp * 16;
  float acc[N / 8][4];
#pragma unroll
  for (int n = 0; n < N / 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
#pragma unroll
  for (int kk = 0; kk < K; kk += 16) {
    uint32_t a[4];
    a[0] = *(const uint32_t*)&sX[(r0 + g) * KP + kk + 2 * t];
    a[1] = *(const uint32_t*)&sX[(r0 + g + 8) * KP + kk + 2 * t];
    a[2] = *(const uint32_t*)&sX[(r0 + g) * KP + kk + 8 + 2 * t];
    a[3] = *(const uint32_t*)&sX[(r0 + g + 8) * KP + kk + 8 + 2 * t];
#pragma unroll
    for (int n = 0; n < N / 8; n++) {
      uint32_t b[2];
      b[0] = *(const uint32_t*)&sW[(n * 8 + g) * KP + kk + 2 * t];
      b[1] = *(const uint32_t*)&sW[(n * 8 + g) * KP + kk + 8 + 2 * t];
      mma_bf16(acc[n], a, b);
    }
  }
#pragma unroll
  for (int n = 0; n < N / 8; n++) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int64_t gr = row0 + r0 + g + 8 * h;
      if (gr >= M) continue;
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int col = n * 8 + 2 * t + e;
        const float z = acc[n][2 * h + e] + (bias ? bias[col] : 0.0f);
        if (Z) Z[gr * ldz + col] = z;
        if (Y) Y[gr * ldy + col] = __float2bfloat16(act ? silu(z) : z);
      }
    }
  }
}

// dW [N x K] += dZ^T X, db [N] += column sums of dZ, over rows [chunk*128, +128)
template <int N, int K>
__global__ void __launch_bounds__(256)
k_linear_dw(int64_t M, const __nv_bfloat16* __restrict__ dZ, int64_t lddz, const __nv_bfloat16* __restrict__ X,
            int64_t ldx, float* dW, float* db) {
  constexpr int CH = 128;
  constexpr int TN = (N >= 128) ? 8 : 2, TK = (N >= 128) ? ((K >= 128) ? 8 : 4) : 8;
  static_assert((N / TN) * (K / TK) == 256, "one tile per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sZ = (float*)smem_raw;            // [CH x N]
  float* sX = sZ + CH * N;                 // [CH x K]
  const int64_t r0 = (int64_t)blockIdx.x * CH;
  for (int i = threadIdx.x; i < CH * N; i += 256) {
    const int64_t r = r0 + i / N;
    sZ[i] = r < M ? __bfloat162float(dZ[r * lddz + i % N]) : 0.0f;
  }
  for (int i = threadIdx.x; i < CH * K; i += 256) {
    const int64_t r = r0 + i / K;
    sX[i] = r < M ? __bfloat162float(X[r * ldx + i % K]) : 0.0f;
  }
  __syncthreads();
  const int tn = threadIdx.x / (K / TK), tk = threadIdx.x % (K / TK);
  float acc[TN][TK];
  for (int a = 0; a < TN; a++)
    for (int b = 0; b < TK; b++) acc[a][b] = 0.0f;
  for (int m = 0; m < CH; m++) {
    float zn[TN], xk[TK];
    for (int a = 0; a < TN; a++) zn[a] = sZ[m * N + tn * TN + a];
    for (int b = 0; b < TK; b++) xk[b] = sX[m * K + tk * TK + b];
    for (int a = 0; a < TN; a++)
      for (int b = 0; b < TK; b++) acc[a][b] = fmaf(zn[a], xk[b], acc[a][b]);
  }
  for (int a = 0; a < TN; a++)
    for (int b = 0; b < TK; b++) atomicAdd(&dW[(tn * TN + a) * K + tk * TK + b], acc[a][b]);
  if (db && threadIdx.x < N) {
    float s = 0.0f;
    for (int m = 0; m < CH; m++) s += sZ[m * N + threadIdx.x];
    atomicAdd(&db[threadIdx.x], s);
  }
}

// dZ = dY * silu'(Z), silu'(z) = s (1 + z (1 - s)), s = 1/(1+e^-z); bf16 out
__global__ void k_silu_backward(int64_t n, const float* Z, const __nv_bfloat16* dY, __nv_bfloat16* dZ) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float z = Z[i];
  const float s = 1.0f / (1.0f + expf(-z));
  dZ[i] = __float2bfloat16(__bfloat162float(dY[i]) * s * (1.0f + z * (1.0f - s)));
}

// loss = sum_m [w0 (y0 - t0)^2 + w1/20 sum_{j=1..20} (yj - tj)^2] / M ; dY bf16 [M x 32]
__global__ void k_mlp_loss(int64_t M, const float* Y, const float* T, float w0, float w1, float* loss,
                           __nv_bfloat16* dY) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const float* y = Y + m * MLP_OUTP;
  const float* t = T + m * MLP_OUTP;
  float l = 0.0f;
  const float inv = 1.0f / (float)M;
  for (int j = 0; j < MLP_OUTP; j++) {
    float d = 0.0f;
    if (j == 0) {
      const float e = y[0] - t[0];
      l += w0 * e * e;
      d = 2.0f * w0 * e * inv;
    } else if (j <= FEAT_LEVELS) {
      const float e = y[j] - t[j];
      l += (w1 / FEAT_LEVELS) * e * e;
      d = 2.0f * (w1 / FEAT_LEVELS) * e * inv;
    }
    dY[m * MLP_OUTP + j] = __float2bfloat16(d);
  }
  atomicAdd(loss, l * inv);
}

// Adam on fp32 master weights [rows x cols]; writes the bf16 copy and its transpose
__global__ void k_adam(int64_t rows, int64_t cols, float* w, const float* g, float* m, float* v, float lr,
                       float b1, float b2, float eps, float c1, float c2, __nv_bfloat16* wb, __nv_bfloat16* wbt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
  if (wbt) wbt[(i % cols) * rows + i / cols] = __float2bfloat16(wi);
}

// normalised bf16 features of every column at the start of a solve (first substep)
__global__ void k_mlp_features(Dims D, int64_t nc, clmgb_soilwater_fields f, clmgb_swm_config cfg, double dtime,
                               const float* mean, const float* istd, __nv_bfloat16* X) {
  const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
  if (c >= nc) return;
  float x[MLP_IN];
  const int64_t nl = f.col_nbedrock[c];
  if (f.mask_hydrology[c] && nl >= 1 && nl <= D.nlevsoi) {
    const int64_t ld = D.ldc;
    const int joff = D.nlevsno;
    column_features(D, f, cfg, c, (int)nl, [&](int j) { return LV(f.h2osoi_liq, c, joff + j, ld); }, dtime,
                    dtime, x);
  } else {
    for (int i = 0; i < MLP_IN; i++) x[i] = 0.0f;
  }
  for (int i = 0; i < MLP_IN; i++) X[c * MLP_IN + i] = __float2bfloat16((x[i] - mean[i]) * istd[i]);
}

// first substep = dtime / 2^k, k = clamp(ceil(y0 - margin), 0, kmax)
__global__ void k_mlp_first_dt(int64_t nc, const float* Y, double dtime, float margin, int kmax, double* dt_first) {
  const int64_t c = (int64_t)blockIdx.x * 128 + threadIdx.x;
  if (c >= nc) return;
  const float y = Y[c * MLP_OUTP];
  int k = (int)ceilf(y - margin);
  if (!(y == y)) k = 0;
  k = k < 0 ? 0 : (k > kmax ? kmax : k);
  double dt = dtime;
  for (int i = 0; i < k; i++) dt = dt / 2.0;
  dt_first[c] = dt;
}

// ---------------------------------------------------------------------------
template <int K, int N>
static cudaError_t linear_launch(int64_t M, const void* X, int64_t ldx, const void* W, const float* b, int act,
                                 float* Z, int64_t ldz, void* Y, int64_t ldy, cudaStream_t s) {
  const size_t smem = (size_t)(N + 64) * (K + 8) * sizeof(__nv_bfloat16);
  cudaError_t e = cudaFuncSetAttribute(k_linear<K, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned int grid = (unsigned int)((M + 63) / 64);
  if (grid == 0) return cudaSuccess;
  k_linear<K, N><<<grid, 128, smem, s>>>(M, (const __nv_bfloat16*)X, ldx, (const __nv_bfloat16*)W, b, act, Z, ldz,
                                         (__nv_bfloat16*)Y, ldy);
  return cudaGetLastError();
}

cudaError_t launch_mlp_linear(int64_t M, int N, int K, const void* X, int64_t ldx, const void* W, const float* b,
                              int act, float* Z, int64_t ldz, void* Y, int64_t ldy, cudaStream_t s) {
  if (K == 64 && N == 128) return linear_launch<64, 128>(M, X, ldx, W, b, act, Z, ldz, Y, ldy, s);
  if (K == 128 && N == 128) return linear_launch<128, 128>(M, X, ldx, W, b, act, Z, ldz, Y, ldy, s);
  if (K == 128 && N == 32) return linear_launch<128, 32>(M, X, ldx, W, b, act, Z, ldz, Y, ldy, s);
  if (K == 32 && N == 128) return linear_launch<32, 128>(M, X, ldx, W, b, act, Z, ldz, Y, ldy, s);
  return cudaErrorInvalidValue;
}

template <int N, int K>
static cudaError_t dw_launch(int64_t M, const void* dZ, int64_t lddz, const void* X, int64_t ldx, float* dW,
                             float* db, cudaStream_t s) {
  const size_t smem = (size_t)128 * (N + K) * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_linear_dw<N, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned int grid = (unsigned int)((M + 127) / 128);
  if (grid == 0) return cudaSuccess;
  k_linear_dw<N, K><<<grid, 256, smem, s>>>(M, (const __nv_bfloat16*)dZ, lddz, (const __nv_bfloat16*)X, ldx, dW,
                                            db);
  return cudaGetLastError();
}

cudaError_t launch_mlp_linear_dw(int64_t M, int N, int K, const void* dZ, int64_t lddz, const void* X, int64_t ldx,
                                 float* dW, float* db, cudaStream_t s) {
  if (N == 128 && K == 64) return dw_launch<128, 64>(M, dZ, lddz, X, ldx, dW, db, s);
  if (N == 128 && K == 128) return dw_launch<128, 128>(M, dZ, lddz, X, ldx, dW, db, s);
  if (N == 32 && K == 128) return dw_launch<32, 128>(M, dZ, lddz, X, ldx, dW, db, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_mlp_silu_backward(int64_t n, const float* Z, const void* dY, void* dZ, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_silu_backward<<<(unsigned int)((n + 255) / 256), 256, 0, s>>>(n, Z, (const __nv_bfloat16*)dY,
                                                                 (__nv_bfloat16*)dZ);
  return cudaGetLastError();
}

cudaError_t launch_mlp_loss(int64_t M, const float* Y, const float* T, float w0, float w1, float* loss, void* dY,
                            cudaStream_t s) {
  if (M <= 0) return cudaSuccess;
  k_mlp_loss<<<(unsigned int)((M + 127) / 128), 128, 0, s>>>(M, Y, T, w0, w1, loss, (__nv_bfloat16*)dY);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(int64_t rows, int64_t cols, float* w, const float* g, float* m, float* v, float lr,
                            float b1, float b2, float eps, int step, void* wb, void* wbt, cudaStream_t s) {
  const int64_t n = rows * cols;
  if (n <= 0) return cudaSuccess;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<(unsigned int)((n + 255) / 256), 256, 0, s>>>(rows, cols, w, g, m, v, lr, b1, b2, eps, c1, c2,
                                                        (__nv_bfloat16*)wb, (__nv_bfloat16*)wbt);
  return cudaGetLastError();
}

cudaError_t launch_richards_samples(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                    const clmgb_swm_config& cfg, double dtime, int rmax, float* feat, float* targ,
                                    unsigned int* count, int64_t capacity, uint32_t* col_status, cudaStream_t s) {
  k_richards_samples<<<(unsigned int)((nc + 63) / 64), 64, 0, s>>>(D, nc, f, cfg, dtime, rmax, feat, targ, count,
                                                                   capacity, col_status);
  return cudaGetLastError();
}

cudaError_t launch_mlp_features(const Dims& D, int64_t nc, const clmgb_soilwater_fields& f,
                                const clmgb_swm_config& cfg, double dtime, const float* mean, const float* istd,
                                void* X, cudaStream_t s) {
  k_mlp_features<<<(unsigned int)((nc + 127) / 128), 128, 0, s>>>(D, nc, f, cfg, dtime, mean, istd,
                                                                  (__nv_bfloat16*)X);
  return cudaGetLastError();
}

cudaError_t launch_mlp_first_dt(int64_t nc, const float* Y, double dtime, float margin, int kmax, double* dt_first,
                                cudaStream_t s) {
  k_mlp_first_dt<<<(unsigned int)((nc + 127) / 128), 128, 0, s>>>(nc, Y, dtime, margin, kmax, dt_first);
  return cudaGetLastError();
}

}  // namespace clmgb
