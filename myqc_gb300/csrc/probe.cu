// probe.cu -- the FP64 multiply-add rate of the context's device.
//
// No counterpart in the reference.  The integral kernels and the Fock
// digestion are bound by the FP64 pipe, whose rate is not among the copy and
// BF16 peaks measured for this GPU model; bench.py reports their achieved
// FP64 rate against this number.  Each thread runs eight independent chains
// of dependent FP64 fma, enough in flight per SM to keep the pipe busy.
#include "internal.h"

namespace mq {

__global__ void fp64_fma_chain_kernel(double *__restrict__ out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

}  // namespace mq

using namespace mq;

extern "C" int mq_probe_fp64(mq_ctx *c, double *tflops) {
  if (!c || !tflops) return MQ_EINVAL;
  cudaSetDevice(c->device);
  int sms = 0;
  MQ_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const int blocks = 4 * sms, threads = 256, iters = 1 << 13;
  double *out = (double *)buf(c, "probe_fp64", sizeof(double) * (size_t)blocks * threads);
  if (!out) return MQ_ENOMEM;
  cudaEvent_t e0, e1;
  MQ_CUDA(c, cudaEventCreate(&e0));
  MQ_CUDA(c, cudaEventCreate(&e1));
  fp64_fma_chain_kernel<<<blocks, threads, 0, c->stream>>>(out, iters, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0, c->stream);
  fp64_fma_chain_kernel<<<blocks, threads, 0, c->stream>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, c->stream);
  c->stats.launches += 2;
  const cudaError_t le = cudaGetLastError();
  const cudaError_t se = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (se == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MQ_CUDA(c, le);
  MQ_CUDA(c, se);
  *tflops = ms > 0.f ? 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12 : 0.0;
  return MQ_OK;
}
