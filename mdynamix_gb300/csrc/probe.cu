// probe.cu -- measured CUDA-core FMA throughput (FP64 and FP32) of the
// device, used as the roofline denominator of the FP64 / FP32 pipe-bound
// kernels.  Eight independent FMA chains per thread, all SMs busy, timed with
// CUDA events; results are written out so nothing is optimised away.
#include "mdx_internal.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma(int iters, T b, T c, T *out) {
  T a0 = (T)threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  for (int i = 0; i < iters; ++i) {
    a0 = a0 * b + c; a1 = a1 * b + c; a2 = a2 * b + c; a3 = a3 * b + c;
    a4 = a4 * b + c; a5 = a5 * b + c; a6 = a6 * b + c; a7 = a7 * b + c;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

template <typename T>
double run(int iters) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma<T><<<blocks, threads>>>(iters / 8, (T)0.999999, (T)1e-7, out);  // warm up
  cudaEventRecord(a);
  k_fma<T><<<blocks, threads>>>(iters, (T)0.999999, (T)1e-7, out);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int mdx_probe_fma_peak(int fp64, double *tflops) {
  if (!tflops) return MDX_ERR_ARG;
  *tflops = fp64 ? run<double>(1 << 12) : run<float>(1 << 16);
  return *tflops > 0 ? MDX_OK : MDX_ERR_CUDA;
}
