// mpm_static.cu -- mpm_energies_static: the EnergiesFix sums over particle
// arrays that already live in the caller's device memory, computed without
// allocating anything.
//
// Who needs it: code that cannot call cudaMalloc at the point where it wants
// the energies -- for example a time loop recorded with CUDA stream capture
// (allocation is not permitted while a stream is being captured), or a host
// application whose device memory is owned by another allocator and which
// only hands out pointers.  mpm_energies allocates nothing per call either,
// but it needs a context (mpm_create allocates); this entry point needs none.
//
// The reduction's scratch (one partial sum per block) is the file-scope
// __device__ array below, of a fixed size: every GPU that loads the library
// holds it until the process exits.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/jump_mpm.h"
#include "mpm_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 4;
constexpr int64_t kPerBlock = int64_t(kThreads) * kPerThread;      // particles per block
constexpr int kMaxBlocks = MPM_STATIC_MAX_PARTICLES / (kThreads * kPerThread);
constexpr int kMaxQ = 5;  // KE, SE, momentum (up to 3)

static_assert(MPM_STATIC_MAX_PARTICLES % (kThreads * kPerThread) == 0, "limit must be whole blocks");

// kMaxBlocks * kMaxQ doubles = 160 KiB
__device__ __align__(256) double g_static_partials[kMaxBlocks * kMaxQ];

int fail(int code, const std::string& msg) { return jmpm::set_last_error(code, msg); }

// Device address of g_static_partials in the calling thread's current CUDA
// context.  A module's device symbols live in one context: a non-primary
// context made current by the caller, or the primary context re-created after
// cudaDeviceReset, loads the module again at another address.  So the cache is
// keyed by the context's unique id (cuCtxGetId, never reused within a process),
// not by the device ordinal.  The two driver calls are fetched through the
// runtime (cudaGetDriverEntryPointByVersion), so the library still links
// against nothing but the driver the runtime loads.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

constexpr int kCacheEntries = 64;
struct ScratchEntry {
  unsigned long long ctx_id;
  double* ptr;
};
std::mutex g_mu;
ScratchEntry g_cache[kCacheEntries] = {};
int g_cache_next = 0;  // round-robin replacement once all entries are used
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;

// the id of the current context, or 0 when none is current (lock held)
int current_context_id(unsigned long long* id) {
  if (!g_get_current || !g_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return fail(MPM_ERR_CUDA, "mpm_energies_static: cuCtxGetCurrent/cuCtxGetId not available from the driver");
    g_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (g_get_current(&ctx) != CUDA_SUCCESS)
    return fail(MPM_ERR_CUDA, "mpm_energies_static: cuCtxGetCurrent failed");
  *id = 0;
  if (ctx && g_get_id(ctx, id) != CUDA_SUCCESS) return fail(MPM_ERR_CUDA, "mpm_energies_static: cuCtxGetId failed");
  return MPM_OK;
}

int scratch_for_current_context(double** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  unsigned long long id = 0;
  int rc = current_context_id(&id);
  if (rc != MPM_OK) return rc;
  if (id != 0)
    for (const ScratchEntry& e : g_cache)
      if (e.ctx_id == id) {
        *out = e.ptr;
        return MPM_OK;
      }
  // first call in this context: look the address up with it current (this also
  // makes the device's primary context current when no context was)
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_partials);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  if (id == 0) {
    rc = current_context_id(&id);
    if (rc != MPM_OK) return rc;
  }
  if (id != 0) {
    g_cache[g_cache_next] = ScratchEntry{id, static_cast<double*>(p)};
    g_cache_next = (g_cache_next + 1) % kCacheEntries;
  }
  *out = static_cast<double*>(p);
  return MPM_OK;
}

// Each block sums kPerBlock particles and writes its partial [KE, SE, P_0..P_{D-1}].
// Symmetric tensors: 2D (xx, yy, xy), 3D (xx, yy, zz, xy, yz, xz), component-major.
template <int D>
__global__ void __launch_bounds__(kThreads) energies_static_kernel(int64_t n, const double* __restrict__ mass,
                                                                   const double* __restrict__ vel,
                                                                   const double* __restrict__ vol,
                                                                   const double* __restrict__ sig,
                                                                   const double* __restrict__ eps,
                                                                   double* partials) {
  constexpr int S = (D == 2) ? 3 : 6;
  constexpr int NQ = 2 + D;
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = 0.0;
  const int64_t b0 = int64_t(blockIdx.x) * kPerBlock;
#pragma unroll
  for (int r = 0; r < kPerThread; ++r) {
    int64_t p = b0 + int64_t(r) * kThreads + threadIdx.x;
    if (p < n) {
      double m = mass[p];
      double vv = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        double va = vel[int64_t(a) * n + p];
        vv += va * va;
        q[2 + a] += m * va;
      }
      q[0] += 0.5 * m * vv;
      double se = 0.0;
#pragma unroll
      for (int c = 0; c < S; ++c) se += (c < D ? 1.0 : 2.0) * sig[int64_t(c) * n + p] * eps[int64_t(c) * n + p];
      q[1] += 0.5 * vol[p] * se;
    }
  }
  __shared__ double sh[NQ][kThreads];
#pragma unroll
  for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NQ; ++k) partials[int64_t(blockIdx.x) * kMaxQ + k] = sh[k][0];
}

// One warp folds the partials of this call (slots [0, nblocks)) in a fixed order.
template <int D>
__global__ void energies_static_fold(const double* partials, int nblocks, double* out) {
  constexpr int NQ = 2 + D;
  int lane = threadIdx.x;
  double acc[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) acc[k] = 0.0;
  for (int b = lane; b < nblocks; b += 32)
#pragma unroll
    for (int k = 0; k < NQ; ++k) acc[k] += partials[int64_t(b) * kMaxQ + k];
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NQ; ++k) out[k] = acc[k];
}

}  // namespace

extern "C" {

int mpm_energies_static(int32_t dim, int64_t count, const double* mass, const double* velocity,
                        const double* volume, const double* stress, const double* strain, double* out,
                        void* stream) {
  if (dim != 2 && dim != 3) return fail(MPM_ERR_ARG, "mpm_energies_static: dim must be 2 or 3");
  if (count < 0) return fail(MPM_ERR_ARG, "mpm_energies_static: negative particle count");
  if (count > MPM_STATIC_MAX_PARTICLES)
    return fail(MPM_ERR_ARG, "mpm_energies_static: count exceeds MPM_STATIC_MAX_PARTICLES (" +
                                 std::to_string(MPM_STATIC_MAX_PARTICLES) + "), the size of its static scratch");
  if (!out || (count > 0 && (!mass || !velocity || !volume || !stress || !strain)))
    return fail(MPM_ERR_ARG, "mpm_energies_static: null array");
  double* scratch = nullptr;
  int rc = scratch_for_current_context(&scratch);
  if (rc != MPM_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int nblocks = int((count + kPerBlock - 1) / kPerBlock);
  if (nblocks > 0) {
    if (dim == 2)
      energies_static_kernel<2><<<nblocks, kThreads, 0, s>>>(count, mass, velocity, volume, stress, strain, scratch);
    else
      energies_static_kernel<3><<<nblocks, kThreads, 0, s>>>(count, mass, velocity, volume, stress, strain, scratch);
  }
  // with no particles the fold reads no slot and writes zeros
  if (dim == 2) energies_static_fold<2><<<1, 32, 0, s>>>(scratch, nblocks, out);
  else energies_static_fold<3><<<1, 32, 0, s>>>(scratch, nblocks, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_energies_static: ") + cudaGetErrorString(e));
  return MPM_OK;
}

}  // extern "C"
