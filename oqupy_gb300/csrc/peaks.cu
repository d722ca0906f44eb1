// FMA-pipe throughput microbenchmark (FP64 DFMA / FP32 FFMA).  The Jacobi
// bond splits run on these pipes, so their measured peaks are the roofline
// denominators of the TEMPO kernels.
#include "../../include/oqupy_gb300.h"
#include "capi_util.h"

namespace otb {

template <typename T>
__global__ void __launch_bounds__(256) fma_loop(T* out, int iters, T seed) {
  T a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  T a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      a0 = fma(a0, m, c);
      a1 = fma(a1, m, c);
      a2 = fma(a2, m, c);
      a3 = fma(a3, m, c);
      a4 = fma(a4, m, c);
      a5 = fma(a5, m, c);
      a6 = fma(a6, m, c);
      a7 = fma(a7, m, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

template <typename T>
static otb_status run_peak(double* tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8, block = 256;
  const int iters = sizeof(T) == 8 ? 256 : 8192;
  DevBuf out;
  if (!out.alloc(sizeof(T) * grid * block)) return OTB_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_loop<T><<<grid, block>>>((T*)out.p, iters, (T)1);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    fma_loop<T><<<grid, block>>>((T*)out.p, iters, (T)1);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!check_cuda(cudaGetLastError(), "fma peak")) return OTB_ERR_CUDA;
  const double flops = 2.0 * 64.0 * iters * (double)grid * block;
  *tflops = flops / (best * 1e-3) / 1e12;
  return OTB_OK;
}

}  // namespace otb

extern "C" otb_status otb_measure_fma_peak(int32_t precision, double* tflops) {
  if (!tflops || (precision != 0 && precision != 1))
    return otb::set_error(OTB_ERR_INVALID_ARG, "precision must be 0 (FP64) or 1 (FP32)");
  return precision == 0 ? otb::run_peak<double>(tflops) : otb::run_peak<float>(tflops);
}
