// Device probe: the FP64 FMA issue rate, the compute roofline that bounds the
// dense FP64 gate kernels on this device (GB300 issues ~2 DFMA/clk/SM, far
// below its HBM bandwidth in FP64 operands).
#include "common.cuh"

namespace spz {

__global__ void fma_chain_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = dfma(x0, a, b); x1 = dfma(x1, a, b); x2 = dfma(x2, a, b); x3 = dfma(x3, a, b);
    x4 = dfma(x4, a, b); x5 = dfma(x5, a, b); x6 = dfma(x6, a, b); x7 = dfma(x7, a, b);
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[0] = s;  // keeps the chain alive; never true in practice
}

}  // namespace spz

using namespace spz;

extern "C" int spz_probe_fp64_fma_rate(double* fma_per_s) {
  if (!fma_per_s) return fail(SPZ_ERR_NULL, "NULL argument");
  int dev, sms;
  SPZ_CUDA(cudaGetDevice(&dev));
  SPZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* d;
  SPZ_CUDA(dev_alloc(&d, 64));
  cudaEvent_t e0, e1;
  SPZ_CUDA(cudaEventCreate(&e0));
  SPZ_CUDA(cudaEventCreate(&e1));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    SPZ_CUDA(cudaEventRecord(e0, 0));
    fma_chain_kernel<<<blocks, threads>>>(d, iters, 0.999, 1e-3);
    SPZ_CUDA(cudaEventRecord(e1, 0));
    SPZ_CUDA(cudaEventSynchronize(e1));
    float ms;
    SPZ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  *fma_per_s = (double)blocks * threads * iters * 8 / (best * 1e-3);
  return SPZ_OK;
}
