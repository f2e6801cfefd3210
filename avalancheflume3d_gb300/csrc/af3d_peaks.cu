// af3d_peaks.cu -- FP64 throughput microbenchmark: the denominator of the FP64 roofline.
//
// GB300's FP64 rate is a small fraction of its FP32 rate, and the contact law is FP64 by
// contract, so the step kernels are bounded by DFMA issue rather than by HBM.  This kernel
// measures that bound on the device at hand: 8 independent DFMA chains per thread, 8 resident
// blocks per SM, a fixed iteration count (no data-dependent loop), one store per thread.
#include "af3d_internal.h"
#include "af3d_physics.cuh"

namespace af3d {

namespace {

constexpr int kIters = 4096;

__global__ void k_dfma(double *out, double s) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
         a6 = a0 + 6, a7 = a0 + 7;
#pragma unroll 4
  for (int i = 0; i < kIters; i++) {
    a0 = fma(a0, s, 0.5); a1 = fma(a1, s, 0.5); a2 = fma(a2, s, 0.5); a3 = fma(a3, s, 0.5);
    a4 = fma(a4, s, 0.5); a5 = fma(a5, s, 0.5); a6 = fma(a6, s, 0.5); a7 = fma(a7, s, 0.5);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace

cudaError_t measure_dfma(int sms, double *tflops) {
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  k_dfma<<<blocks, threads>>>(out, 0.999);   // warm-up
  cudaEventRecord(t0);
  k_dfma<<<blocks, threads>>>(out, 0.999);
  cudaEventRecord(t1);
  e = cudaEventSynchronize(t1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  *tflops = ms > 0 ? 2.0 * 8.0 * kIters * (double)blocks * threads / (ms * 1e-3) / 1e12 : 0.0;
  return e;
}

namespace {

// The integer-pipe helpers of af3d_physics.cuh against the hardware instructions they replace:
// per element, one bit per helper that disagreed.
__global__ void k_check_bits(const double *x, int *bad, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  int b = 0;
  if (__float_as_uint(to_float_rn(v)) != __float_as_uint((float)v)) b |= 1;
  if (__float_as_uint(to_float_ru(v)) != __float_as_uint(__double2float_ru(v))) b |= 2;
  if (isfinite(v) && fabs(v) < 9.2e18 && trunc_to_ll(v) != (long long)v) b |= 4;
  if (finite_bits(v) != (bool)isfinite(v)) b |= 8;
  if (nonzero_bits(v) != (v != 0.0)) b |= 16;
  const double lo = 1.0 - 1.4901161193847656e-08, hi = 1.0 + 1.4901161193847656e-08;
  if (!(v < 0.0) && in_open_range_bits(v, lo, hi) != (fabs(v - 1.0) < 1.4901161193847656e-08)) b |= 32;
  if (!(v < 0.0) && in_open_range_bits(v, 0.0, 9.765625e-04) != (v > 0.0 && v < 9.765625e-04)) b |= 64;
  bad[i] = b;
}

}  // namespace

cudaError_t check_fp64_bits(const double *x, long n, int *bad) {
  if (n <= 0) return cudaSuccess;
  double *dx = nullptr;
  int *db = nullptr;
  cudaError_t e = cudaMalloc(&dx, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&db, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_check_bits<<<(unsigned)((n + 255) / 256), 256>>>(dx, db, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(bad, db, sizeof(int) * n, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(db);
  return e;
}

}  // namespace af3d
