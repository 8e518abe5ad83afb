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

}  // namespace
}  // namespace mrmg

extern "C" int mrmg_microbench_fma(int32_t precision, int64_t iters, double* out_tflops, void* stream) {
  using namespace mrmg;
  if (!out_tflops || iters < 1 || (precision != 0 && precision != 1)) return MRMG_ERR_ARG;
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
    if (precision == 0)
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
  const double flops = 2.0 * 32.0 * (double)iters * threads * blocks;
  *out_tflops = flops / (ms * 1e-3) / 1e12;
  return MRMG_OK;
}
