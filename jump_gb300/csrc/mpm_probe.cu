// mpm_probe.cu -- mpm_probe_rates: throughput of the operations the step
// kernels are bound by, measured on the device the library runs on: FP64
// fused multiply-adds, FP64 divisions and FP64 atomic additions executed in
// L2 (RED.ADD at distinct, coalesced addresses).  A measurement aid for the
// FP64 roofline that bench.py reports beside the HBM one.  mpm_probe_dw: the
// double-word operations of mpm_dw.cuh on given operands, for tests of their
// error bounds against exact rational arithmetic.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/jump_mpm.h"
#include "mpm_dw.cuh"

namespace jmpm {
int set_last_error(int code, const std::string& msg);  // mpm_capi.cu
}

namespace {

constexpr int kChains = 8;  // independent FMA chains per thread (hides the pipe latency)

__global__ void fma_probe_kernel(int iters, double a, double b, double* out) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = double(threadIdx.x + c);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

__global__ void div_probe_kernel(int iters, double b, double* out) {
  double x[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) x[c] = 1.0 + double(threadIdx.x + c);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = b / x[c] + 1.0;
  if (x[0] + x[1] + x[2] + x[3] == 12345.678) out[0] = x[0];
}

__global__ void atomic_probe_kernel(int iters, double* buf, int64_t mask) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = int64_t(gridDim.x) * blockDim.x;
  for (int i = 0; i < iters; ++i) atomicAdd(buf + ((t + int64_t(i) * n) & mask), 1.0);
}

// ms of one launch of f, timed with events after one untimed launch
template <class F>
int time_launch(cudaStream_t s, F&& f, float* ms) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return 1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return 1;
  }
  f();
  cudaEventRecord(e0, s);
  f();
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e == cudaSuccess ? 0 : 1;
}

// result i of double-word operation op on operands a[i], b[i], c[i] (each
// converted FP64 -> DW by dw_from): out[2i] = hi, out[2i + 1] = lo
__global__ void dw_probe_kernel(int op, int64_t n, const double* a, const double* b, const double* c, double* out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  using namespace jmpm;
  const dw x = dw_from(a[i]), y = dw_from(b[i]), z = dw_from(c[i]);
  dw r = x;
  switch (op) {
    case MPM_DW_OP_ADD: r = x + y; break;
    case MPM_DW_OP_SUB: r = x - y; break;
    case MPM_DW_OP_MUL: r = x * y; break;
    case MPM_DW_OP_MUL_FLOAT: r = x * y.hi; break;
    case MPM_DW_OP_FMA: r = dw_fma(x, y, z); break;
    case MPM_DW_OP_SQR: r = dw_sqr(x); break;
    case MPM_DW_OP_SQRT: r = dw_sqrt(x); break;
    case MPM_DW_OP_RECIP: r = dw_recip(x); break;
    case MPM_DW_OP_ONE_MINUS: r = dw_one_minus(x); break;
    case MPM_DW_OP_TO_F64: r = dw_make(float(0), float(0)); break;
    default: break;  // MPM_DW_OP_FROM_F64: the conversion itself
  }
  if (op == MPM_DW_OP_TO_F64) {
    out[2 * i] = dw_to_f64(x + y);
    out[2 * i + 1] = 0.0;
    return;
  }
  out[2 * i] = double(r.hi);
  out[2 * i + 1] = double(r.lo);
}

}  // namespace

extern "C" int mpm_probe_dw(int32_t op, int64_t n, const double* a, const double* b, const double* c, double* out) {
  if (op < MPM_DW_OP_FROM_F64 || op > MPM_DW_OP_TO_F64 || n < 0 || (n > 0 && (!a || !b || !c || !out)))
    return jmpm::set_last_error(MPM_ERR_ARG, "mpm_probe_dw: bad operation or arrays");
  if (n == 0) return MPM_OK;
  double* d = nullptr;
  const size_t bytes = size_t(n) * sizeof(double);
  if (cudaMalloc(&d, bytes * 5) != cudaSuccess) return jmpm::set_last_error(MPM_ERR_CUDA, "mpm_probe_dw: allocation");
  cudaError_t e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + 2 * n, c, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    dw_probe_kernel<<<unsigned((n + 255) / 256), 256>>>(op, n, d, d + n, d + 2 * n, d + 3 * n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + 3 * n, 2 * bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return jmpm::set_last_error(MPM_ERR_CUDA, std::string("mpm_probe_dw: ") + cudaGetErrorString(e));
  return MPM_OK;
}

extern "C" int mpm_probe_rates(double* fp64_fma_per_s, double* fp64_div_per_s, double* fp64_atomics_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess)
    return jmpm::set_last_error(MPM_ERR_CUDA, "mpm_probe_rates: no device");
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return jmpm::set_last_error(MPM_ERR_CUDA, "mpm_probe_rates: stream");
  const int64_t nbuf = int64_t(1) << 24;  // 128 MiB of doubles: larger than L2 in footprint
  double* buf = nullptr;
  if (cudaMalloc(&buf, size_t(nbuf) * sizeof(double)) != cudaSuccess) {
    cudaStreamDestroy(s);
    return jmpm::set_last_error(MPM_ERR_CUDA, "mpm_probe_rates: allocation");
  }
  cudaMemsetAsync(buf, 0, size_t(nbuf) * sizeof(double), s);
  const unsigned blocks = unsigned(sms) * 8, threads = 256;
  const double nthreads = double(blocks) * threads;
  int bad = 0;
  float ms = 0.f;
  const int fma_iters = 4096, div_iters = 256, atom_iters = 1024;
  // only the rates asked for (non-NULL outputs) are measured
  if (fp64_fma_per_s) {
    bad |= time_launch(s, [&] { fma_probe_kernel<<<blocks, threads, 0, s>>>(fma_iters, 0.999999, 1e-9, buf); }, &ms);
    if (!bad) *fp64_fma_per_s = nthreads * fma_iters * kChains / (ms * 1e-3);
  }
  if (fp64_div_per_s && !bad) {
    bad |= time_launch(s, [&] { div_probe_kernel<<<blocks, threads, 0, s>>>(div_iters, 3.0, buf); }, &ms);
    if (!bad) *fp64_div_per_s = nthreads * div_iters * 4 / (ms * 1e-3);
  }
  if (fp64_atomics_per_s && !bad) {
    bad |= time_launch(s, [&] { atomic_probe_kernel<<<blocks, threads, 0, s>>>(atom_iters, buf, nbuf - 1); }, &ms);
    if (!bad) *fp64_atomics_per_s = nthreads * atom_iters / (ms * 1e-3);
  }
  cudaStreamSynchronize(s);
  cudaFree(buf);
  cudaStreamDestroy(s);
  if (bad) return jmpm::set_last_error(MPM_ERR_CUDA, "mpm_probe_rates: a probe launch failed");
  return MPM_OK;
}
