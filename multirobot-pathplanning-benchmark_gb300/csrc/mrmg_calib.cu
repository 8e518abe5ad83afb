// mrmg_calib.cu -- measured FP32 / FP64 fused-multiply-add peaks of the
// device, the denominators of the roofline fractions reported for the
// collision (FP32 pipe) and distance (FP64 pipe) kernels.
#include "mrmg_internal.cuh"

namespace mrmg {
namespace {

template <typename T>
__global__ void fma_chains(T* out, long long iters, T a, T b) {
  // 8 independent dependency chains per thread: enough ILP to fill the pipe
  T x0 = (T)(threadIdx.x & 7) * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (long long i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)-12345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;   // never true; keeps the chains live
}

// MUFU (special-function unit) throughput: 8 chains of x <- 2^x - 1 per
// thread (x stays in [-1/2, 0]); the FP32 subtraction issues on the FMA pipe,
// which is wider, so the chains are bound by ex2.approx
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void mufu_chains(float* out, long long iters) {
  float x0 = -(float)(threadIdx.x & 7) * 1e-3f, x1 = x0 - 0.01f, x2 = x0 - 0.02f, x3 = x0 - 0.03f;
  float x4 = x0 - 0.04f, x5 = x0 - 0.05f, x6 = x0 - 0.06f, x7 = x0 - 0.07f;
  for (long long i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      x0 = ex2_approx(x0) - 1.f; x1 = ex2_approx(x1) - 1.f; x2 = ex2_approx(x2) - 1.f; x3 = ex2_approx(x3) - 1.f;
      x4 = ex2_approx(x4) - 1.f; x5 = ex2_approx(x5) - 1.f; x6 = ex2_approx(x6) - 1.f; x7 = ex2_approx(x7) - 1.f;
    }
  }
  float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == -12345.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace mrmg

extern "C" int mrmg_microbench_fma(int32_t precision, int64_t iters, double* out_tflops, void* stream) {
  using namespace mrmg;
  if (!out_tflops || iters < 1 || precision < 0 || precision > 2) return MRMG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  void* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * threads * blocks) != cudaSuccess) return MRMG_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](long long it) {
    if (precision == 2)
      mufu_chains<<<blocks, threads, 0, st>>>((float*)buf, it);
    else if (precision == 0)
      fma_chains<float><<<blocks, threads, 0, st>>>((float*)buf, it, 0.9999999f, 1e-7f);
    else
      fma_chains<double><<<blocks, threads, 0, st>>>((double*)buf, it, 0.9999999999, 1e-12);
  };
  launch(iters / 8 + 1);   // warm-up
  cudaEventRecord(e0, st);
  launch(iters);
  cudaEventRecord(e1, st);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return MRMG_ERR_CUDA;
  // FMA: 2 flops per lane-op; MUFU: 1 operation per lane-op
  const double flops = (precision == 2 ? 1.0 : 2.0) * 32.0 * (double)iters * threads * blocks;
  *out_tflops = flops / (ms * 1e-3) / 1e12;
  return MRMG_OK;
}
