// probe.cu -- measured CUDA-core FMA throughput (FP64 and FP32) of the
// device, used as the roofline denominator of the FP64 / FP32 pipe-bound
// kernels.  Independent FMA chains per thread (8 or 16), 2 to 8 blocks of 256
// threads per SM, each configuration timed with CUDA events (best of three
// launches of roughly 10-20 ms); the best configuration is reported.  Results
// are written out so nothing is optimised away.
#include "mdx_internal.cuh"
#include "pair_math.cuh"

namespace {

template <typename T, int NCH>
__global__ void __launch_bounds__(256) k_fma(int iters, T b, T c, T *out) {
  T a[NCH];
#pragma unroll
  for (int k = 0; k < NCH; ++k) a[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < NCH; ++k) a[k] = fma(a[k], b, c);
  }
  T s = T(0);
#pragma unroll
  for (int k = 0; k < NCH; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// One configuration (NCH chains per thread, bps blocks of 256 per SM), best
// of three timed launches.
template <typename T, int NCH>
double run_cfg(int iters, int bps) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * bps, threads = 256;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma<T, NCH><<<blocks, threads>>>(iters / 8, (T)0.999999, (T)1e-7, out);  // warm up
  float ms = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(a);
    k_fma<T, NCH><<<blocks, threads>>>(iters, (T)0.999999, (T)1e-7, out);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    ms = t < ms ? t : ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double flops = 2.0 * NCH * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

// The best of a few occupancy / chain-count configurations.
template <typename T>
double run(int iters) {
  double best = -1.0;
  const int bps[3] = {2, 4, 8};
  for (int k = 0; k < 3; ++k) {
    best = fmax(best, run_cfg<T, 8>(iters * 8 / bps[k], bps[k]));
    best = fmax(best, run_cfg<T, 16>(iters * 4 / bps[k], bps[k]));
  }
  return best;
}

__global__ void k_pair_math(int n, const double *y, const double *d, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = exp_neg(y[i]);
  out[n + i] = exp(-y[i]);
  out[2 * n + i] = rcp_nr(d[i]);
  out[3 * n + i] = 1.0 / d[i];
}

}  // namespace

extern "C" int mdx_probe_pair_math(int n, const double *y, const double *d, double *own_exp,
                                   double *lib_exp, double *own_rcp, double *lib_rcp) {
  if (n <= 0 || !y || !d || !own_exp || !lib_exp || !own_rcp || !lib_rcp) return MDX_ERR_ARG;
  double *buf = nullptr;
  const size_t nb = sizeof(double) * (size_t)n;
  if (cudaMalloc(&buf, 6 * nb) != cudaSuccess) return MDX_ERR_NOMEM;
  int rc = MDX_OK;
  double *dy = buf, *dd = buf + n, *out = buf + 2 * (size_t)n;
  if (cudaMemcpy(dy, y, nb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dd, d, nb, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = MDX_ERR_CUDA;
  } else {
    k_pair_math<<<(n + 255) / 256, 256>>>(n, dy, dd, out);
    double *dst[4] = {own_exp, lib_exp, own_rcp, lib_rcp};
    for (int k = 0; k < 4 && rc == MDX_OK; ++k)
      if (cudaMemcpy(dst[k], out + (size_t)k * n, nb, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = MDX_ERR_CUDA;
  }
  cudaFree(buf);
  return rc;
}

extern "C" int mdx_probe_fma_peak(int fp64, double *tflops) {
  if (!tflops) return MDX_ERR_ARG;
  *tflops = fp64 ? run<double>(1 << 12) : run<float>(1 << 16);
  return *tflops > 0 ? MDX_OK : MDX_ERR_CUDA;
}
