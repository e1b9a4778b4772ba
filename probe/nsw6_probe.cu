// Throughput probes for the FP64 roofline of the NSW6 kernels.
//
// Measures, on the current device, the sustained rate of FP64 FMA (the FP64
// pipe peak), FP64 add and multiply, FP32 FMA, and of CUDA's own FP64 divide,
// sqrt, exp, log and pow.  The function rates divided into the FMA rate give
// the op weights (FP64 operations per call) used to express the NSW6 step's
// algorithmic work in FP64-operation units.  Every kernel runs a fixed number
// of iterations over independent dependency chains per thread; all loops are
// bounded.
#include <cuda_runtime.h>

#include <cmath>

namespace {

constexpr int CHAINS = 8;

template <int OP>
__global__ void probe_kernel(double* out, int iters, double seed) {
  double v[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) v[c] = seed + 1.0e-3 * (threadIdx.x + c);
  const double a = 1.0000001, b = 1.0e-9;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) {
      if (OP == 0) v[c] = __fma_rn(v[c], a, b);
      else if (OP == 1) v[c] = __dadd_rn(v[c], b);
      else if (OP == 2) v[c] = __dmul_rn(v[c], a);
      else if (OP == 3) v[c] = a / v[c];
      else if (OP == 4) v[c] = sqrt(v[c]) + 1.0;
      else if (OP == 5) v[c] = exp(v[c] * 1.0e-3) + 0.5;
      else if (OP == 6) v[c] = log(v[c]) + 2.0;
      else if (OP == 7) v[c] = pow(v[c], 1.33) * 0.75 + 0.5;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += v[c];
  if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_ffma(float* out, int iters, float seed) {
  float v[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) v[c] = seed + 1.0e-3f * (threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = __fmaf_rn(v[c], 1.0000001f, 1.0e-9f);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += v[c];
  if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Issue cost of one FP64-pipe form for a few warps of one CTA per SM: OP 0
// DFMA, 1 DSETP (the compare feeds an integer chain), 2 F2F double -> float
// (likewise); `active` lanes of each warp execute, the rest wait.  Four
// independent chains per thread; cycles of the CTA's longest warp.
template <int OP>
__global__ void issue_kernel(long long* cyc, double* out, int iters, int active) {
  const int lane = threadIdx.x & 31;
  double a[4];
  long long iv[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    a[c] = 1.0 + 1.0e-3 * (threadIdx.x + c);
    iv[c] = threadIdx.x + c;
  }
  __syncthreads();
  const long long t0 = clock64();
  if (lane < active) {
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (OP == 0) {
          a[c] = __fma_rn(a[c], 0.999999, 1.0e-7);
        } else if (OP == 1) {
          iv[c] += (a[c] < 1.25) ? 3 : 1;
          a[c] = __longlong_as_double(0x3FF0000000000000ll + (iv[c] & 0xFFFFF));
        } else {
          const float f = (float)a[c];
          iv[c] += __float_as_int(f) & 7;
          a[c] = __longlong_as_double(0x3FF0000000000000ll + (iv[c] & 0xFFFFF));
        }
      }
    }
  }
  __syncthreads();
  const long long t1 = clock64();
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 4; ++c) s += a[c] + (double)iv[c];
  if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

}  // namespace

extern "C" {

// Cycles per instruction of one warp for issue_kernel<op> (op 0 DFMA, 1 DSETP,
// 2 F2F) run by `warps` warps (1..32) of one CTA on every SM, `active` lanes
// (1..32) each; the SM's cost per instruction is this over `warps`.  Negative
// on error.
double nsw6_probe_issue(int op, int warps, int active, int iters) {
  if (warps < 1 || warps > 32 || active < 1 || active > 32 || iters < 1) return -4.0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 32 * warps;
  double* out = nullptr;
  long long* cyc = nullptr;
  if (cudaMalloc(&out, sizeof(double) * sms * threads) != cudaSuccess) return -2.0;
  if (cudaMalloc(&cyc, sizeof(long long) * sms) != cudaSuccess) {
    cudaFree(out);
    return -2.0;
  }
  auto launch = [&](int n) {
    if (op == 0) issue_kernel<0><<<sms, threads>>>(cyc, out, n, active);
    else if (op == 1) issue_kernel<1><<<sms, threads>>>(cyc, out, n, active);
    else issue_kernel<2><<<sms, threads>>>(cyc, out, n, active);
  };
  launch(iters / 10 + 1);  // warm-up
  launch(iters);
  long long* h = new long long[sms];
  const cudaError_t e1 = cudaMemcpy(h, cyc, sizeof(long long) * sms, cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  long long mx = 0;
  for (int i = 0; i < sms; ++i) mx = h[i] > mx ? h[i] : mx;
  delete[] h;
  cudaFree(out);
  cudaFree(cyc);
  if (e1 != cudaSuccess || err != cudaSuccess || mx <= 0) return -3.0;
  return (double)mx / (4.0 * iters);
}


// op: 0 dfma, 1 dadd, 2 dmul, 3 ddiv, 4 dsqrt, 5 exp, 6 log, 7 pow, 8 ffma.
// Returns operations per second (one FMA counted as one operation) or a
// negative value on error.
double nsw6_probe_rate(int op, int iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -2.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](int n) {
    switch (op) {
      case 0: probe_kernel<0><<<blocks, threads>>>(out, n, 1.0); break;
      case 1: probe_kernel<1><<<blocks, threads>>>(out, n, 1.0); break;
      case 2: probe_kernel<2><<<blocks, threads>>>(out, n, 1.0); break;
      case 3: probe_kernel<3><<<blocks, threads>>>(out, n, 1.5); break;
      case 4: probe_kernel<4><<<blocks, threads>>>(out, n, 2.0); break;
      case 5: probe_kernel<5><<<blocks, threads>>>(out, n, 0.5); break;
      case 6: probe_kernel<6><<<blocks, threads>>>(out, n, 3.0); break;
      case 7: probe_kernel<7><<<blocks, threads>>>(out, n, 2.0); break;
      default: probe_ffma<<<blocks, threads>>>((float*)out, n, 1.0f); break;
    }
  };
  launch(iters / 10 + 1);  // warm-up
  cudaEventRecord(e0);
  launch(iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return -3.0;
  return (double)blocks * threads * CHAINS * (double)iters / (ms * 1.0e-3);
}

}  // extern "C"
