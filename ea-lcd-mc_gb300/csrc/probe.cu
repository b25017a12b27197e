// probe.cu -- measured peak rate of 32-bit integer instructions on the
// current GPU: the denominator of the integer-pipe roofline of the sweep
// kernels (which are bound by integer issue, not by HBM).
//
// Every thread runs 8 independent chains of alternating xor and add with
// run-time operands, so each counted operation is one integer instruction
// that nothing can fold away (an xor followed by an add has no fused form),
// and 8 chains per thread keep the pipe busy despite each chain's latency.
// A second form runs multiply-add chains (the integer multiplier used by the
// Philox rounds).  Rates are thread-operations per second over all SMs,
// timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "eagb.h"

namespace eagb {
void set_last_error(const char *msg);

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) k_probe_alu(uint32_t a, uint32_t b, int iters, uint32_t *out) {
  uint32_t x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * (2 * c + 1) + blockIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = (x[c] ^ a) + b;
  }
  uint32_t s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s ^= x[c];
  if (s == 0x9E3779B9u) out[0] = s;  // keeps the chains alive; practically never stored
}

__global__ void __launch_bounds__(256) k_probe_imad(uint32_t a, uint32_t b, int iters, uint32_t *out) {
  uint32_t x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * (2 * c + 1) + blockIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = x[c] * a + b;
  }
  uint32_t s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s ^= x[c];
  if (s == 0x9E3779B9u) out[0] = s;
}

}  // namespace
}  // namespace eagb

using namespace eagb;

extern "C" int ea_probe_int32_rate(int32_t device, double *alu_ops_per_s, double *imad_ops_per_s) {
  if (!alu_ops_per_s && !imad_ops_per_s) {
    set_last_error("ea_probe_int32_rate: no output");
    return EA_ERR_ARG;
  }
  cudaDeviceProp prop;
  if (cudaSetDevice(device) != cudaSuccess || cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    set_last_error("ea_probe_int32_rate: no such device");
    return EA_ERR_CUDA;
  }
  uint32_t *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc(&out, 4);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  // 8 blocks of 256 threads per SM (64 warps: every scheduler always has work)
  const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
  const double ops = (double)blocks * threads * iters * kUnroll * kChains;
  for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
    double *dst = kind == 0 ? alu_ops_per_s : imad_ops_per_s;
    if (!dst) continue;
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch warms up
      e = cudaEventRecord(e0, st);
      if (kind == 0) k_probe_alu<<<blocks, threads, 0, st>>>(0x5bd1e995u, 0x68e31da4u, iters, out);
      else k_probe_imad<<<blocks, threads, 0, st>>>(0x5bd1e995u, 0x68e31da4u, iters, out);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e == cudaSuccess) *dst = ops / (best * 1e-3);
  }
  if (st) cudaStreamDestroy(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return EA_ERR_CUDA;
  }
  return EA_OK;
}
