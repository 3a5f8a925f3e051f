// mpm_batch.cu -- batched ensembles: many independent USL problems advance
// together, by one of two strategies.
//
// PERSISTENT (small problems, one material model, no contact).  Layout: the particles of every problem (and of every body inside a
// problem) are contiguous ranges of one SoA allocation; node arrays of every
// problem are packed one after another; InstanceP is the per-problem offset
// table.  A CTA takes a problem from a work queue (problems ordered by
// particle count, largest first), runs all requested steps of it -- reset,
// P2G, grid update, G2P + stress, with __syncthreads between the stages --
// and takes the next one.  Nothing but the queue counter is shared between
// CTAs, and there is one launch for all problems and all steps.  Node data a
// stage reads was written earlier in the same launch, so it is loaded through
// L2 (__ldcg), never through the read-only path.
//
// WIDE (large problems, mixed materials, contact).  One launch per stage for
// all problems (mpm_wide.cuh), the step captured once as a CUDA graph and
// replayed.  It shares the particle SoA and, without contact, the node fields
// of the persistent layout; contact problems get one node field per body.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/jump_mpm.h"
#include "mpm_internal.h"
#include "mpm_kernels.cuh"
#include "mpm_wide.cuh"
#include "mpm_tangent.cuh"

using namespace jmpm;

namespace {

int fail(int code, const std::string& msg) { return set_last_error(code, msg); }

#define BATCH_TRY(x)                                                                 \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess)                                                           \
      return fail(MPM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));    \
  } while (0)

struct InstanceP {
  GridP g;
  NodeP nd;
  int64_t pbegin, pcount;  // all particles of the problem
  int nb;
  int64_t bbeg[MPM_BATCH_MAX_BODIES], bcnt[MPM_BATCH_MAX_BODIES];
  MatParams mp[MPM_BATCH_MAX_BODIES];
  double dt, tol, grav[3];
};

template <int D, class R, int MAT, bool GRAV>
__global__ void batch_kernel(const InstanceP* __restrict__ inst, const int* __restrict__ order, int ninst,
                             int* next, int64_t nsteps, void* P, int64_t pitch, unsigned* status, int32_t* hat_c,
                             void* hat_nl) {
  __shared__ int sh_q;
  constexpr bool F32 = sizeof(R) == 4;
  for (;;) {
    if (threadIdx.x == 0) sh_q = atomicAdd(next, 1);
    __syncthreads();
    const int q = sh_q;
    __syncthreads();  // every thread has read sh_q before thread 0 overwrites it
    if (q >= ninst) return;
    const int id = order[q];
    const InstanceP& I = inst[id];
    const PartP all{P, pitch, I.pbegin, I.pcount, hat_c, hat_nl};
    unsigned* st = status + id;
    const int64_t Nn = I.nd.nodeCount;
    for (int64_t s = 0; s < nsteps; ++s) {
      // reset (:381-385)
      for (int64_t i = threadIdx.x; i < Nn; i += blockDim.x) {
        I.nd.m[i] = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          I.nd.p0[a * Nn + i] = 0.0;
          I.nd.f[a * Nn + i] = 0.0;
        }
      }
      __syncthreads();
      // P2G; every thread runs the same number of iterations (warp-synchronous FP32 path)
      for (int64_t base = 0; base < I.pcount; base += blockDim.x)
        p2g_particle<D, R, GRAV>(I.g, I.nd, all, base + threadIdx.x, I.grav[0], I.grav[1], I.grav[2], st);
      __syncthreads();
      for (int64_t i = threadIdx.x; i < Nn; i += blockDim.x) grid_node<D, F32, true>(I.nd, i, I.dt, I.tol);
      __syncthreads();
      for (int b = 0; b < I.nb; ++b) {
        const PartP pb{P, pitch, I.bbeg[b], I.bcnt[b], hat_c, hat_nl};
        for (int64_t t = threadIdx.x; t < pb.count; t += blockDim.x)
          g2p_particle<D, R, MAT, true>(I.g, I.nd, pb, t, I.mp[b], I.dt, st);
      }
      __syncthreads();
    }
  }
}

// EnergiesFix sums of every problem: one CTA per problem, fixed reduction order
template <int D, class R>
__global__ void __launch_bounds__(256) batch_energies_kernel(const InstanceP* __restrict__ inst, void* P,
                                                             int64_t pitch, double* out) {
  using L = Layout<D>;
  constexpr int NQ = 2 + D;
  const InstanceP& I = inst[blockIdx.x];
  const PartP pp{P, pitch, I.pbegin, I.pcount};
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = 0.0;
  for (int64_t t = threadIdx.x; t < pp.count; t += blockDim.x) {
    int64_t p = pp.begin + t;
    double m = double(*field<R>(pp, L::M, p)), vv = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double va = double(*field<R>(pp, L::V + a, p));
      vv += va * va;
      q[2 + a] += m * va;
    }
    q[0] += 0.5 * m * vv;
    double se = 0.0;
#pragma unroll
    for (int c = 0; c < L::S; ++c)
      se += (c < D ? 1.0 : 2.0) * double(*field<R>(pp, L::SIG + c, p)) * double(*field<R>(pp, L::EPS + c, p));
    q[1] += 0.5 * double(*field<R>(pp, L::VOL, p)) * se;
  }
  __shared__ double sh[NQ][256];
#pragma unroll
  for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NQ; ++k) out[int64_t(blockIdx.x) * NQ + k] = sh[k][0];
}

int sym_slot(int dim, int i, int j) {
  if (i == j) return i;
  if (dim == 2) return 2;
  int a = i < j ? i : j, b = i < j ? j : i;
  return (a == 0 && b == 1) ? 3 : ((a == 1 && b == 2) ? 4 : 5);
}

CompMapH ident(int n) {
  CompMapH m{};
  m.n = n;
  for (int i = 0; i < n; ++i) m.src[i] = i;
  return m;
}

// upload of a symmetric matrix; mirrored entries that differ set `bit` in *flag
CompMapH sym_from_full(int dim, unsigned* flag = nullptr, unsigned bit = 0) {
  CompMapH m{};
  m.n = dim == 2 ? 3 : 6;
  for (int j = 0; j < dim; ++j)
    for (int i = j; i < dim; ++i) m.src[sym_slot(dim, i, j)] = i + dim * j;
  for (int j = 0; j < dim; ++j)
    for (int i = j + 1; i < dim; ++i) {
      m.ca[m.nchk] = i + dim * j;
      m.cb[m.nchk] = j + dim * i;
      ++m.nchk;
    }
  m.flag = flag;
  m.bit = bit;
  return m;
}

CompMapH full_from_sym(int dim) {
  CompMapH m{};
  m.n = dim * dim;
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) m.src[i + dim * j] = sym_slot(dim, i, j);
  return m;
}

}  // namespace

struct mpm_batch {
  int dim = 2;
  bool f32 = false;
  int mat = MPM_MAT_ELASTIC;
  bool grav = false;
  int ninst = 0;
  int64_t np = 0;
  int NF = 0;
  size_t esz = 8;
  void* P = nullptr;
  // hat cache of the persistent kernel's FP64 steps (PartP::hat_c / hat_nl), or null
  int32_t* hat_c = nullptr;
  void* hat_nl = nullptr;
  double* nodebuf = nullptr;
  float* nodebuf_f = nullptr;
  uint8_t* fixed = nullptr;
  double* coords = nullptr;
  std::vector<InstanceP> inst;
  InstanceP* d_inst = nullptr;
  int* d_order = nullptr;
  int* d_next = nullptr;
  unsigned* d_status = nullptr;
  double* d_energy = nullptr;
  double* staging = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
  int threads = 256;
  int ctas_per_sm = 0;  // 0: as many as fit
  int sms = 1;

  // strategy
  bool persistent_ok = true;  // one material model type and no contact
  int strategy = MPM_BATCH_PERSISTENT;
  // WIDE strategy tables and node bookkeeping
  std::vector<WideBody> wbody;
  std::vector<int> wbody_k;       // index of each table body within its problem
  std::vector<double> wbody_nu;   // its Poisson ratio
  std::vector<WideInst> winst;
  std::vector<WideTile> tiles;
  WideBody* d_wbody = nullptr;
  WideInst* d_winst = nullptr;
  WideTile* d_tiles = nullptr;
  int* d_blk_inst = nullptr;
  uint32_t* d_blk = nullptr;  // flags (nblk) | list (nblk) | count (1)
  int64_t nblk = 0;
  double* cnodebuf = nullptr;  // contact problems: one field per body
  float* cnodebuf_f = nullptr;
  cudaGraph_t wgraph = nullptr;
  cudaGraphExec_t wexec = nullptr;
  bool nodes_dirty = false;  // the persistent kernel left node data the WIDE list does not cover
  // forward-mode derivatives (mpm_batch_jvp): tangent particle fields and node fields
  double* tpart = nullptr;
  double* tnodebuf = nullptr;
  size_t tnode_doubles = 0;
  std::vector<TanBody> tbody;
  std::vector<TanInst> tinst;
  TanBody* d_tbody = nullptr;
  TanInst* d_tinst = nullptr;
  cudaGraph_t jgraph = nullptr;
  cudaGraphExec_t jexec = nullptr;

  PartP body(int i, int b) const { return PartP{P, np, inst[i].bbeg[b], inst[i].bcnt[b]}; }
  uint32_t* flags() const { return d_blk; }
  uint32_t* list() const { return d_blk + nblk; }
  uint32_t* count() const { return d_blk + 2 * nblk; }
};

namespace {

void destroy_batch(mpm_batch* b) {
  if (!b) return;
  cudaFree(b->P);
  cudaFree(b->hat_c);
  cudaFree(b->nodebuf);
  cudaFree(b->nodebuf_f);
  cudaFree(b->fixed);
  cudaFree(b->coords);
  cudaFree(b->d_inst);
  cudaFree(b->d_order);
  cudaFree(b->d_next);
  cudaFree(b->d_status);
  cudaFree(b->d_energy);
  cudaFree(b->staging);
  cudaFree(b->d_wbody);
  cudaFree(b->d_winst);
  cudaFree(b->d_tiles);
  cudaFree(b->d_blk_inst);
  cudaFree(b->d_blk);
  cudaFree(b->cnodebuf);
  cudaFree(b->cnodebuf_f);
  if (b->wexec) cudaGraphExecDestroy(b->wexec);
  if (b->wgraph) cudaGraphDestroy(b->wgraph);
  cudaFree(b->tpart);
  cudaFree(b->tnodebuf);
  cudaFree(b->d_tbody);
  cudaFree(b->d_tinst);
  if (b->jexec) cudaGraphExecDestroy(b->jexec);
  if (b->jgraph) cudaGraphDestroy(b->jgraph);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <int D, class R, int MAT, bool GRAV>
int launch_t(mpm_batch* b, void* P, int64_t nsteps, int threads, int per_sm) {
  auto kern = batch_kernel<D, R, MAT, GRAV>;
  cudaFuncAttributes attr;
  BATCH_TRY(cudaFuncGetAttributes(&attr, kern));
  if (threads > attr.maxThreadsPerBlock)
    return fail(MPM_ERR_ARG, "mpm_batch: " + std::to_string(threads) + " threads per CTA exceed this kernel's limit " +
                                 std::to_string(attr.maxThreadsPerBlock));
  int occ = 0;
  BATCH_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0));
  if (occ < 1) return fail(MPM_ERR_ARG, "mpm_batch: launch shape does not fit on an SM");
  int per = per_sm > 0 ? std::min(per_sm, occ) : occ;
  BATCH_TRY(cudaMemsetAsync(b->d_next, 0, sizeof(int), b->stream));
  kern<<<b->sms * per, threads, 0, b->stream>>>(b->d_inst, b->d_order, b->ninst, b->d_next, nsteps, P, b->np,
                                                b->d_status, b->hat_c, b->hat_nl);
  BATCH_TRY(cudaGetLastError());
  return MPM_OK;
}

template <int D, class R>
int launch_m(mpm_batch* b, void* P, int64_t n, int th, int per) {
  switch (b->mat) {
    case MPM_MAT_ELASTIC:
      return b->grav ? launch_t<D, R, MPM_MAT_ELASTIC, true>(b, P, n, th, per)
                     : launch_t<D, R, MPM_MAT_ELASTIC, false>(b, P, n, th, per);
    case MPM_MAT_NEOHOOKEAN:
      return b->grav ? launch_t<D, R, MPM_MAT_NEOHOOKEAN, true>(b, P, n, th, per)
                     : launch_t<D, R, MPM_MAT_NEOHOOKEAN, false>(b, P, n, th, per);
    case MPM_MAT_JOHNSON_COOK:
      if constexpr (D == 3)
        return b->grav ? launch_t<D, R, MPM_MAT_JOHNSON_COOK, true>(b, P, n, th, per)
                       : launch_t<D, R, MPM_MAT_JOHNSON_COOK, false>(b, P, n, th, per);
      return fail(MPM_ERR_ARG, "mpm_batch: Johnson-Cook is a 3D material");
    case MPM_MAT_VOCE:
      if constexpr (D == 3)
        return b->grav ? launch_t<D, R, MPM_MAT_VOCE, true>(b, P, n, th, per)
                       : launch_t<D, R, MPM_MAT_VOCE, false>(b, P, n, th, per);
      return fail(MPM_ERR_ARG, "mpm_batch: Voce is a 3D material");
    case MPM_MAT_JOHNSON_COOK_DAMAGE:
      if constexpr (D == 3)
        return b->grav ? launch_t<D, R, MPM_MAT_JOHNSON_COOK_DAMAGE, true>(b, P, n, th, per)
                       : launch_t<D, R, MPM_MAT_JOHNSON_COOK_DAMAGE, false>(b, P, n, th, per);
      return fail(MPM_ERR_ARG, "mpm_batch: Johnson-Cook with damage is a 3D material");
    default:
      return b->grav ? launch_t<D, R, MPM_MAT_J2, true>(b, P, n, th, per)
                     : launch_t<D, R, MPM_MAT_J2, false>(b, P, n, th, per);
  }
}

int launch(mpm_batch* b, void* P, int64_t nsteps, int threads, int per_sm) {
  if (b->dim == 2)
    return b->f32 ? launch_m<2, float>(b, P, nsteps, threads, per_sm)
                  : launch_m<2, double>(b, P, nsteps, threads, per_sm);
  return b->f32 ? launch_m<3, float>(b, P, nsteps, threads, per_sm)
                : launch_m<3, double>(b, P, nsteps, threads, per_sm);
}

// ---- WIDE strategy ----------------------------------------------------------
template <int D>
void wide_enqueue(mpm_batch* b) {
  cudaStream_t s = b->stream;
  const unsigned nt = unsigned(b->tiles.size());
  const int64_t most = (b->nblk * 64 + 255) / 256;
  const unsigned gctas = unsigned(std::max<int64_t>(1, std::min<int64_t>(most, int64_t(b->sms) * 8)));
  // reset (:381-385) of the blocks the previous step touched
  wide_clear_kernel<D><<<gctas, 256, 0, s>>>(b->d_winst, b->d_blk_inst, b->list(), b->count());
  cudaMemsetAsync(b->count(), 0, sizeof(uint32_t), s);
  if (nt) {
    if (b->f32) wide_p2g_kernel<D, float><<<nt, 256, 0, s>>>(b->d_wbody, b->d_winst, b->d_tiles, b->d_status);
    else wide_p2g_kernel<D, double><<<nt, 256, 0, s>>>(b->d_wbody, b->d_winst, b->d_tiles, b->d_status);
  }
  NodeP all{};
  all.bflag = b->flags();
  all.blist = b->list();
  all.bcount = b->count();
  all.nblk = b->nblk;
  compact_blocks_kernel<<<unsigned((b->nblk + 255) / 256), 256, 0, s>>>(all);
  if (b->f32) wide_grid_kernel<D, true><<<gctas, 256, 0, s>>>(b->d_winst, b->d_blk_inst, b->list(), b->count());
  else wide_grid_kernel<D, false><<<gctas, 256, 0, s>>>(b->d_winst, b->d_blk_inst, b->list(), b->count());
  if (nt) {
    if (b->f32) wide_g2p_kernel<D, float><<<nt, 256, 0, s>>>(b->d_wbody, b->d_winst, b->d_tiles, b->d_status);
    else wide_g2p_kernel<D, double><<<nt, 256, 0, s>>>(b->d_wbody, b->d_winst, b->d_tiles, b->d_status);
  }
}

// zero every node field and the block list (after the persistent kernel, or
// to drop the node state a timing run left)
int wide_clean(mpm_batch* b) {
  const int D = b->dim;
  int64_t plain = 0, contact = 0;
  for (const WideInst& W : b->winst) {
    if (W.contact) contact += W.g.nodeCount * W.cp.nb;
    else plain += W.g.nodeCount;
  }
  if (plain) BATCH_TRY(cudaMemsetAsync(b->nodebuf, 0, size_t(plain) * (1 + 4 * D) * sizeof(double), b->stream));
  if (contact) BATCH_TRY(cudaMemsetAsync(b->cnodebuf, 0, size_t(contact) * (1 + 5 * D) * sizeof(double), b->stream));
  BATCH_TRY(cudaMemsetAsync(b->d_blk, 0, size_t(2 * b->nblk + 1) * sizeof(uint32_t), b->stream));
  b->nodes_dirty = false;
  return MPM_OK;
}

int wide_run(mpm_batch* b, int64_t nsteps) {
  if (b->nodes_dirty) {
    int r = wide_clean(b);
    if (r) return r;
  }
  if (!b->wexec) {
    BATCH_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    if (b->dim == 2) wide_enqueue<2>(b);
    else wide_enqueue<3>(b);
    cudaError_t le = cudaGetLastError();
    cudaError_t ee = cudaStreamEndCapture(b->stream, &b->wgraph);
    if (le != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_batch: kernel launch: ") + cudaGetErrorString(le));
    if (ee != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_batch: graph capture: ") + cudaGetErrorString(ee));
    BATCH_TRY(cudaGraphInstantiate(&b->wexec, b->wgraph, 0));
  }
  for (int64_t k = 0; k < nsteps; ++k) BATCH_TRY(cudaGraphLaunch(b->wexec, b->stream));
  return MPM_OK;
}

// ---- forward-mode derivatives -------------------------------------------------
template <int D>
void jvp_enqueue(mpm_batch* b) {
  cudaStream_t s = b->stream;
  const unsigned nt = unsigned(b->tiles.size());
  const int64_t most = (b->nblk * 64 + 255) / 256;
  const unsigned gctas = unsigned(std::max<int64_t>(1, std::min<int64_t>(most, int64_t(b->sms) * 8)));
  wide_clear_kernel<D><<<gctas, 256, 0, s>>>(b->d_winst, b->d_blk_inst, b->list(), b->count());
  tan_clear_kernel<D><<<gctas, 256, 0, s>>>(b->d_winst, b->d_tinst, b->d_blk_inst, b->list(), b->count());
  cudaMemsetAsync(b->count(), 0, sizeof(uint32_t), s);
  if (nt) tan_p2g_kernel<D><<<nt, 256, 0, s>>>(b->d_wbody, b->d_tbody, b->d_winst, b->d_tiles, b->d_status);
  NodeP all{};
  all.bflag = b->flags();
  all.blist = b->list();
  all.bcount = b->count();
  all.nblk = b->nblk;
  compact_blocks_kernel<<<unsigned((b->nblk + 255) / 256), 256, 0, s>>>(all);
  wide_grid_kernel<D, false><<<gctas, 256, 0, s>>>(b->d_winst, b->d_blk_inst, b->list(), b->count());
  tan_grid_kernel<D><<<gctas, 256, 0, s>>>(b->d_winst, b->d_tinst, b->d_blk_inst, b->list(), b->count());
  // per particle: the tangent G2P reads the state the primal G2P then overwrites
  if (nt) tan_g2p_kernel<D><<<nt, 256, 0, s>>>(b->d_wbody, b->d_tbody, b->d_winst, b->d_tiles, b->d_status);
}

// tangent buffers and tables (first call), seeds (every call)
int jvp_setup(mpm_batch* b, const double* dE) {
  const int D = b->dim;
  const int NT = D == 2 ? TanLayout<2>::NT : TanLayout<3>::NT;
  if (!b->tpart) {
    BATCH_TRY(cudaMalloc(&b->tpart, size_t(NT) * size_t(b->np > 0 ? b->np : 1) * sizeof(double)));
    size_t nd = 0;
    for (const WideInst& W : b->winst)
      nd += size_t(W.g.nodeCount) * (W.contact ? size_t(W.cp.nb) * (1 + 5 * D) : size_t(1 + 4 * D));
    b->tnode_doubles = nd;
    BATCH_TRY(cudaMalloc(&b->tnodebuf, (nd > 0 ? nd : 1) * sizeof(double)));
    b->tinst.resize(b->winst.size());
    size_t off = 0;
    for (size_t i = 0; i < b->winst.size(); ++i) {
      const WideInst& W = b->winst[i];
      TanInst& T = b->tinst[i];
      T.tcp = W.cp;
      const int64_t Nn = W.g.nodeCount;
      const int nf = W.contact ? W.cp.nb : 1;
      const int per = W.contact ? 1 + 5 * D : 1 + 4 * D;
      for (int k = 0; k < nf; ++k) {
        NodeP f = W.cp.body[k];
        double* base = b->tnodebuf + off;
        f.m = base;
        f.p0 = base + Nn;
        f.f = base + Nn * (1 + D);
        f.nrm = W.contact ? base + Nn * (1 + 2 * D) : nullptr;
        f.vdt = base + Nn * (W.contact ? 1 + 3 * D : 1 + 2 * D);
        f.dv = base + Nn * (W.contact ? 1 + 4 * D : 1 + 3 * D);
        f.vdt_f = f.dv_f = nullptr;
        f.bflag = nullptr;
        T.tcp.body[k] = f;
        off += size_t(Nn) * per;
      }
    }
    BATCH_TRY(cudaMalloc(&b->d_tinst, b->tinst.size() * sizeof(TanInst)));
    BATCH_TRY(cudaMemcpy(b->d_tinst, b->tinst.data(), b->tinst.size() * sizeof(TanInst), cudaMemcpyHostToDevice));
    BATCH_TRY(cudaMalloc(&b->d_tbody, b->wbody.size() * sizeof(TanBody) + sizeof(TanBody)));
  }
  b->tbody.resize(b->wbody.size());
  for (size_t q = 0; q < b->wbody.size(); ++q) {
    const WideBody& wb = b->wbody[q];
    TanBody& tb = b->tbody[q];
    tb.tp = wb.pp;
    tb.tp.base = b->tpart;
    const WideInst& W = b->winst[wb.inst];
    const int k = b->wbody_k[q];
    tb.tnd = b->tinst[wb.inst].tcp.body[W.contact ? k : 0];
    const double nu = b->wbody_nu[q];
    const double e = dE ? dE[size_t(wb.inst) * MPM_BATCH_MAX_BODIES + k] : 0.0;
    tb.dlam = e * nu / (1 + nu) / (1 - 2 * nu);  // d lambda / dE times dE (Material.jl:54)
    tb.dmu = e / 2 / (1 + nu);                   // d mu / dE times dE (Material.jl:55)
  }
  BATCH_TRY(cudaMemcpyAsync(b->d_tbody, b->tbody.data(), b->tbody.size() * sizeof(TanBody), cudaMemcpyHostToDevice,
                            b->stream));
  // tangents start at zero: the state at the call does not depend on the scalar
  BATCH_TRY(cudaMemsetAsync(b->tpart, 0, size_t(NT) * size_t(b->np > 0 ? b->np : 1) * sizeof(double), b->stream));
  BATCH_TRY(cudaMemsetAsync(b->tnodebuf, 0, (b->tnode_doubles > 0 ? b->tnode_doubles : 1) * sizeof(double),
                            b->stream));
  return MPM_OK;
}

int jvp_run(mpm_batch* b, int64_t nsteps) {
  if (b->nodes_dirty) {
    int r = wide_clean(b);
    if (r) return r;
  }
  if (!b->jexec) {
    BATCH_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    if (b->dim == 2) jvp_enqueue<2>(b);
    else jvp_enqueue<3>(b);
    cudaError_t le = cudaGetLastError();
    cudaError_t ee = cudaStreamEndCapture(b->stream, &b->jgraph);
    if (le != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_batch_jvp: kernel launch: ") + cudaGetErrorString(le));
    if (ee != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_batch_jvp: graph capture: ") + cudaGetErrorString(ee));
    BATCH_TRY(cudaGraphInstantiate(&b->jexec, b->jgraph, 0));
  }
  for (int64_t k = 0; k < nsteps; ++k) BATCH_TRY(cudaGraphLaunch(b->jexec, b->stream));
  return MPM_OK;
}

int run_steps(mpm_batch* b, int64_t nsteps) {
  if (nsteps <= 0) return MPM_OK;
  if (b->strategy == MPM_BATCH_WIDE) return wide_run(b, nsteps);
  b->nodes_dirty = true;
  return launch(b, b->P, nsteps, b->threads, b->ctas_per_sm);
}

// stream-ordered (the next copy into staging waits for this transpose); the
// create synchronises once after the last upload
int upload(mpm_batch* b, const PartP& pp, const double* host, int per, int f0, const CompMapH& cm) {
  size_t n = size_t(pp.count) * per;
  if (n == 0 || !host) return MPM_OK;
  BATCH_TRY(cudaMemcpyAsync(b->staging, host, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  if (b->dim == 2) Launchers<2>::aos_to_soa(b->stream, pp, b->f32, b->staging, per, f0, cm);
  else Launchers<3>::aos_to_soa(b->stream, pp, b->f32, b->staging, per, f0, cm);
  BATCH_TRY(cudaGetLastError());
  return MPM_OK;
}

int download(mpm_batch* b, const PartP& pp, double* host, int per, int f0, const CompMapH& cm) {
  size_t n = size_t(pp.count) * per;
  if (n == 0 || !host) return MPM_OK;
  if (b->dim == 2) Launchers<2>::soa_to_aos(b->stream, pp, b->f32, b->staging, per, f0, cm);
  else Launchers<3>::soa_to_aos(b->stream, pp, b->f32, b->staging, per, f0, cm);
  BATCH_TRY(cudaGetLastError());
  BATCH_TRY(cudaMemcpyAsync(host, b->staging, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

template <int D>
int create_t(const mpm_instance_desc* in, int32_t n, mpm_batch* b) {
  using L = Layout<D>;
  b->NF = L::NF;
  int64_t maxbody = 1, nodes = 0, ncoord = 0, plain_nodes = 0, contact_nodes = 0;
  for (int i = 0; i < n; ++i) {
    int64_t nn = 1;
    for (int a = 0; a < D; ++a) {
      nn *= in[i].grid.nodes[a];
      ncoord += in[i].grid.nodes[a];
    }
    nodes += nn;
    if (in[i].contact) contact_nodes += nn * in[i].nbodies;
    else plain_nodes += nn;
    for (int k = 0; k < in[i].nbodies; ++k) {
      b->np += in[i].bodies[k].count;
      maxbody = std::max(maxbody, in[i].bodies[k].count);
    }
  }
  const size_t ptot = size_t(b->NF) * size_t(b->np > 0 ? b->np : 1);
  BATCH_TRY(cudaMalloc(&b->P, ptot * b->esz));
  BATCH_TRY(cudaMemset(b->P, 0, ptot * b->esz));
  if (!b->f32 && b->np > 0) {
    // hat cache: int32 codes, then the lower hat values (every axis has at most
    // 2^20 nodes, so a cell fits the code's 27 bits)
    const size_t nc = size_t(D) * size_t(b->np);
    const size_t cbytes = (nc * sizeof(int32_t) + 15) / 16 * 16;
    char* hb = nullptr;
    BATCH_TRY(cudaMalloc(&hb, cbytes + nc * sizeof(double)));
    b->hat_c = reinterpret_cast<int32_t*>(hb);
    b->hat_nl = hb + cbytes;
  }
  // per node: m | p0 (D) | f (D) | vdt (D) | dv (D); contact fields add the normals (D)
  if (plain_nodes > 0) {
    BATCH_TRY(cudaMalloc(&b->nodebuf, size_t(plain_nodes) * (1 + 4 * D) * sizeof(double)));
    BATCH_TRY(cudaMemset(b->nodebuf, 0, size_t(plain_nodes) * (1 + 4 * D) * sizeof(double)));
    if (b->f32) BATCH_TRY(cudaMalloc(&b->nodebuf_f, size_t(plain_nodes) * 2 * D * sizeof(float)));
  }
  if (contact_nodes > 0) {
    BATCH_TRY(cudaMalloc(&b->cnodebuf, size_t(contact_nodes) * (1 + 5 * D) * sizeof(double)));
    BATCH_TRY(cudaMemset(b->cnodebuf, 0, size_t(contact_nodes) * (1 + 5 * D) * sizeof(double)));
    if (b->f32) BATCH_TRY(cudaMalloc(&b->cnodebuf_f, size_t(contact_nodes) * 2 * D * sizeof(float)));
  }
  BATCH_TRY(cudaMalloc(&b->fixed, size_t(nodes)));
  BATCH_TRY(cudaMalloc(&b->coords, size_t(ncoord) * sizeof(double)));
  BATCH_TRY(cudaMalloc(&b->staging, size_t(maxbody) * 9 * sizeof(double)));
  BATCH_TRY(cudaMalloc(&b->d_status, size_t(n) * sizeof(unsigned)));
  BATCH_TRY(cudaMemset(b->d_status, 0, size_t(n) * sizeof(unsigned)));
  BATCH_TRY(cudaMalloc(&b->d_energy, size_t(n) * (2 + D) * sizeof(double)));
  BATCH_TRY(cudaMalloc(&b->d_next, sizeof(int)));
  std::vector<uint8_t> fixed_h(static_cast<size_t>(nodes), 0);
  std::vector<double> coords_h;
  int64_t noff = 0, poff = 0, pnoff = 0, cnoff = 0;
  b->inst.resize(n);
  b->winst.resize(n);
  for (int i = 0; i < n; ++i) {
    const mpm_instance_desc& d = in[i];
    InstanceP I{};
    int64_t nn[3] = {1, 1, 1};
    double dx[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) {
      nn[a] = d.grid.nodes[a];
      dx[a] = (d.grid.xmax[a] - d.grid.xmin[a]) / (double(d.grid.nodes[a]) - 1.0);  // Grid.jl:105
      I.g.xmin[a] = d.grid.xmin[a];
      I.g.dxI[a] = 1.0 / dx[a];
      I.g.dx[a] = dx[a];
      I.g.xminf[a] = float(I.g.xmin[a]);  // the FP32 estimate of hat()'s base node
      I.g.dxIf[a] = float(I.g.dxI[a]);
      I.g.nn[a] = nn[a];
    }
    I.g.nx = nn[0];
    I.g.nxy = nn[0] * nn[1];
    I.g.nodeCount = I.g.nxy * nn[2];
    for (int a = 0; a < 3; ++a) {
      I.g.coord[a] = b->coords + coords_h.size();
      if (a < D)
        for (int64_t k = 0; k < nn[a]; ++k) coords_h.push_back(d.grid.xmin[a] + double(k) * dx[a]);
    }
    const int64_t Nn = I.g.nodeCount;
    if (d.grid.fixed_nodes)
      for (int64_t k = 0; k < Nn; ++k)
        for (int a = 0; a < D; ++a)
          if (d.grid.fixed_nodes[a + D * k] == 1) fixed_h[size_t(noff + k)] |= uint8_t(1u << a);
    NodeP& nd = I.nd;
    nd.nodeCount = Nn;
    nd.fixed = b->fixed + noff;
    for (int a = 0; a < 3; ++a) nd.nn[a] = nn[a];
    // node blocks of the WIDE strategy (global ids blk0 ..)
    WideInst& W = b->winst[i];
    W.blk0 = b->nblk;
    {
      const int B = BlockShape<D>::B;
      nd.nblk = 1;
      for (int a = 0; a < 3; ++a) {
        nd.nb[a] = a < D ? (nn[a] + B - 1) / B : 1;
        nd.nblk *= nd.nb[a];
      }
      b->nblk += nd.nblk;
    }
    if (!d.contact) {
      double* base = b->nodebuf + size_t(pnoff) * (1 + 4 * D);
      nd.m = base;
      nd.p0 = base + Nn;
      nd.f = base + Nn * (1 + D);
      nd.vdt = base + Nn * (1 + 2 * D);
      nd.dv = base + Nn * (1 + 3 * D);
      if (b->f32) {
        nd.vdt_f = b->nodebuf_f + size_t(pnoff) * 2 * D;
        nd.dv_f = nd.vdt_f + Nn * D;
      }
      pnoff += Nn;
      W.contact = 0;
      W.cp.nb = 1;
      W.cp.body[0] = nd;
    } else {
      W.contact = 1;
      W.cp.nb = d.nbodies;
      W.cp.friction = d.friction;
      for (int k = 0; k < d.nbodies; ++k) {
        NodeP f = nd;
        double* base = b->cnodebuf + size_t(cnoff) * (1 + 5 * D);
        f.m = base;
        f.p0 = base + Nn;
        f.f = base + Nn * (1 + D);
        f.nrm = base + Nn * (1 + 2 * D);
        f.vdt = base + Nn * (1 + 3 * D);
        f.dv = base + Nn * (1 + 4 * D);
        if (b->f32) {
          f.vdt_f = b->cnodebuf_f + size_t(cnoff) * 2 * D;
          f.dv_f = f.vdt_f + Nn * D;
        }
        W.cp.body[k] = f;
        cnoff += Nn;
      }
    }
    I.pbegin = poff;
    I.nb = d.nbodies;
    for (int k = 0; k < d.nbodies; ++k) {
      const mpm_material_desc& m = d.bodies[k].mat;
      I.bbeg[k] = poff;
      I.bcnt[k] = d.bodies[k].count;
      poff += d.bodies[k].count;
      I.mp[k] = make_mat_params(m, d.bodies[k].youngs != nullptr, d.dt);
    }
    I.pcount = poff - I.pbegin;
    I.dt = d.dt;
    I.tol = d.tolerance;
    for (int a = 0; a < 3; ++a) I.grav[a] = a < D ? d.body_force[a] : 0.0;
    b->inst[i] = I;
    W.g = I.g;
    W.dt = I.dt;
    W.tol = I.tol;
    for (int a = 0; a < 3; ++a) W.grav[a] = I.grav[a];
    noff += Nn;
  }
  // WIDE tables: block flags/list/count, block -> problem, bodies, particle tiles
  BATCH_TRY(cudaMalloc(&b->d_blk, size_t(2 * b->nblk + 1) * sizeof(uint32_t)));
  BATCH_TRY(cudaMemset(b->d_blk, 0, size_t(2 * b->nblk + 1) * sizeof(uint32_t)));
  {
    std::vector<int> blk_inst(static_cast<size_t>(b->nblk));
    for (int i = 0; i < n; ++i) {
      WideInst& W = b->winst[i];
      const int nf = W.contact ? W.cp.nb : 1;
      for (int k = 0; k < nf; ++k) W.cp.body[k].bflag = b->flags() + W.blk0;
      for (int64_t q = 0; q < b->inst[i].nd.nblk; ++q) blk_inst[size_t(W.blk0 + q)] = i;
      for (int k = 0; k < b->inst[i].nb; ++k) {
        WideBody wb{};
        wb.pp = b->body(i, k);
        wb.pp.hat_c = b->hat_c;  // the wide P2G caches each hat for the wide G2P of the step
        wb.pp.hat_nl = b->hat_nl;
        wb.nd = W.cp.body[W.contact ? k : 0];
        wb.mp = b->inst[i].mp[k];
        wb.inst = i;
        const int body = int(b->wbody.size());
        for (int64_t t = 0; t < wb.pp.count; t += 256) b->tiles.push_back(WideTile{body, t});
        b->wbody.push_back(wb);
        b->wbody_k.push_back(k);
        b->wbody_nu.push_back(in[i].bodies[k].mat.nu);
      }
    }
    BATCH_TRY(cudaMalloc(&b->d_blk_inst, blk_inst.size() * sizeof(int) + sizeof(int)));
    BATCH_TRY(cudaMemcpy(b->d_blk_inst, blk_inst.data(), blk_inst.size() * sizeof(int), cudaMemcpyHostToDevice));
    BATCH_TRY(cudaMalloc(&b->d_winst, b->winst.size() * sizeof(WideInst)));
    BATCH_TRY(cudaMemcpy(b->d_winst, b->winst.data(), b->winst.size() * sizeof(WideInst), cudaMemcpyHostToDevice));
    BATCH_TRY(cudaMalloc(&b->d_wbody, b->wbody.size() * sizeof(WideBody) + sizeof(WideBody)));
    BATCH_TRY(cudaMemcpy(b->d_wbody, b->wbody.data(), b->wbody.size() * sizeof(WideBody), cudaMemcpyHostToDevice));
    BATCH_TRY(cudaMalloc(&b->d_tiles, b->tiles.size() * sizeof(WideTile) + sizeof(WideTile)));
    BATCH_TRY(cudaMemcpy(b->d_tiles, b->tiles.data(), b->tiles.size() * sizeof(WideTile), cudaMemcpyHostToDevice));
  }
  BATCH_TRY(cudaMemcpy(b->fixed, fixed_h.data(), fixed_h.size(), cudaMemcpyHostToDevice));
  BATCH_TRY(cudaMemcpy(b->coords, coords_h.data(), coords_h.size() * sizeof(double), cudaMemcpyHostToDevice));
  BATCH_TRY(cudaMalloc(&b->d_inst, size_t(n) * sizeof(InstanceP)));
  BATCH_TRY(cudaMemcpy(b->d_inst, b->inst.data(), size_t(n) * sizeof(InstanceP), cudaMemcpyHostToDevice));
  // work queue order: largest problem first
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->inst[x].pcount > b->inst[y].pcount; });
  BATCH_TRY(cudaMalloc(&b->d_order, size_t(n) * sizeof(int)));
  BATCH_TRY(cudaMemcpy(b->d_order, order.data(), size_t(n) * sizeof(int), cudaMemcpyHostToDevice));
  // particles
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < in[i].nbodies; ++k) {
      const mpm_body_desc& d = in[i].bodies[k];
      const PartP pp = b->body(i, k);
      if (d.count == 0) continue;
      int r;
      if ((r = upload(b, pp, d.pos, D, L::X, ident(D)))) return r;
      if ((r = upload(b, pp, d.velocity, D, L::V, ident(D)))) return r;
      if ((r = upload(b, pp, d.mass, 1, L::M, ident(1)))) return r;
      if ((r = upload(b, pp, d.volume, 1, L::VOL, ident(1)))) return r;
      if ((r = upload(b, pp, d.volume_initial, 1, L::VOL0, ident(1)))) return r;
      if (d.F) {
        if ((r = upload(b, pp, d.F, D * D, L::F, ident(D * D)))) return r;
      } else {
        std::vector<double> I(size_t(d.count) * D * D, 0.0);
        for (int64_t p = 0; p < d.count; ++p)
          for (int a = 0; a < D; ++a) I[p * D * D + a * (D + 1)] = 1.0;
        if ((r = upload(b, pp, I.data(), D * D, L::F, ident(D * D)))) return r;
      }
      if ((r = upload(b, pp, d.strain, D * D, L::EPS, sym_from_full(D, b->d_status, ST_ASYM_STRESS)))) return r;
      if ((r = upload(b, pp, d.stress, D * D, L::SIG, sym_from_full(D, b->d_status, ST_ASYM_STRESS)))) return r;
      if ((r = upload(b, pp, d.alpha, 1, L::ALPHA, ident(1)))) return r;
      if ((r = upload(b, pp, d.alphadot, 1, L::ALPHAD, ident(1)))) return r;
      if ((r = upload(b, pp, d.vmstr, 1, L::VM, ident(1)))) return r;
      if (D == 3 && d.mat.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
        // damage state in the plastic strain slots; temperatures start at Tr (Material.jl:507)
        if ((r = upload(b, pp, d.damage_init, 1, L::EP, ident(1)))) return r;
        if ((r = upload(b, pp, d.damage, 1, L::EP + 1, ident(1)))) return r;
        std::vector<double> Tr;
        const double* T = d.temperature;
        if (!T) {
          Tr.assign(size_t(d.count), d.mat.Tr);
          T = Tr.data();
        }
        if ((r = upload(b, pp, T, 1, L::EP + 2, ident(1)))) return r;
      } else if (d.pstrain) {
        r = D == 2 ? upload(b, pp, d.pstrain, 3, L::EP, ident(3)) : upload(b, pp, d.pstrain, 9, L::EP, sym_from_full(3, b->d_status, ST_ASYM_PSTRAIN));
        if (r) return r;
      }
      if (d.youngs) {
        std::vector<double> lm(size_t(d.count) * 2);
        double nu = d.mat.nu;
        for (int64_t p = 0; p < d.count; ++p) {
          double E = d.youngs[p];
          lm[2 * p] = E * nu / (1 + nu) / (1 - 2 * nu);
          lm[2 * p + 1] = E / 2 / (1 + nu);
        }
        if ((r = upload(b, pp, lm.data(), 2, L::LAM, ident(2)))) return r;
      }
    }
  }
  // the uploads compared the mirrored entries of every symmetric input (flag: problem 0's status word)
  unsigned st = 0;
  BATCH_TRY(cudaMemcpyAsync(&st, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  if (st & ST_ASYM_STRESS) return fail(MPM_ERR_ARG, "mpm_batch_create: strain and stress must be symmetric");
  if (st & ST_ASYM_PSTRAIN) return fail(MPM_ERR_ARG, "mpm_batch_create: pstrain must be symmetric");
  BATCH_TRY(cudaMemset(b->d_status, 0, sizeof(unsigned)));
  return MPM_OK;
}

template <int D>
int energies_t(mpm_batch* b, double* out) {
  if (b->f32) batch_energies_kernel<D, float><<<b->ninst, 256, 0, b->stream>>>(b->d_inst, b->P, b->np, b->d_energy);
  else batch_energies_kernel<D, double><<<b->ninst, 256, 0, b->stream>>>(b->d_inst, b->P, b->np, b->d_energy);
  BATCH_TRY(cudaGetLastError());
  BATCH_TRY(cudaMemcpyAsync(out, b->d_energy, size_t(b->ninst) * (2 + D) * sizeof(double), cudaMemcpyDeviceToHost,
                            b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

int status_code(unsigned st) {
  if (st & ST_OUT_OF_GRID) return MPM_ERR_OUT_OF_GRID;
  if (st & ST_NONFINITE) return MPM_ERR_NONFINITE;
  if (st & ST_NEGATIVE_J) return MPM_ERR_NEGATIVE_J;
  return MPM_OK;
}

}  // namespace

namespace jmpm {

// MPM_P2G_FUSED: nsteps USL steps of one small FP64 problem of a context in a
// single cooperative launch.  Per step: P2G, grid update, G2P (with the reset
// of the node accumulators for the next step), separated by grid barriers
// (grid_barrier: bounded waits that set q.bar[2] and end the kernel).  Thread
// t handles particles t, t + nthreads, ... in both particle stages, so a
// particle's fields, and the hat its P2G caches for the G2P of the same step,
// are only ever read by the thread that wrote them; node values
// written in the launch by other CTAs are read through L2 (grid_node and
// g2p_particle with CG, P2G through atomics).
struct FusedP {
  GridP g;
  NodeP nd;
  void* P;
  int64_t pitch, np;
  int nb;
  int64_t bbeg[MPM_BATCH_MAX_BODIES];
  MatParams mp[MPM_BATCH_MAX_BODIES];
  double dt, tol, grav[3];
  unsigned* status;
  unsigned* bar;  // [0] arrivals, [1] generation, [2] a barrier wait gave up
  // the second set of node accumulators (m, p0 (D), f (D)): steps alternate
  // between it and nd's, ending on nd's
  double *m2, *p02, *f2;
  // the hat cache (PartP::hat_c / hat_nl; null: the G2P recomputes each hat)
  int32_t* hat_c;
  void* hat_nl;
  // EnergiesFix records after steps first, first + every, ... (rec non-null):
  // per-CTA partial sums, folded by CTA 0 in a fixed order into rec->base[rec->idx++]
  EnRec* rec;
  int64_t first, every;
  double* partial;  // (2 + D) doubles per CTA
};

template <int D, int MAT, bool GRAV>
__global__ void __launch_bounds__(128) fused_steps_kernel(FusedP q, int64_t nsteps) {
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nth = int64_t(gridDim.x) * blockDim.x;
  unsigned* err = q.bar + 2;
  if (*reinterpret_cast<volatile unsigned*>(err)) return;  // an earlier wait gave up
  const PartP all{q.P, q.pitch, 0, q.np, q.hat_c, q.hat_nl};
  const int64_t Nn = q.nd.nodeCount;
  // two sets of accumulators, A (the context's) and B: step s sums into A when
  // nsteps - 1 - s is even, so the last step's sums are the context's; while
  // the grid update of a step reads its set, the other is zeroed for the next
  // step, so no barrier separates a step's G2P from the next step's P2G (a
  // thread's P2G reads only the particles its own G2P updated)
  NodeP nA = q.nd, nB = q.nd;
  nB.m = q.m2;
  nB.p0 = q.p02;
  nB.f = q.f2;
  auto reset = [&](const NodeP& n) {
    for (int64_t i = tid; i < Nn; i += nth) {
      n.m[i] = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        n.p0[a * Nn + i] = 0.0;
        n.f[a * Nn + i] = 0.0;
      }
    }
  };
  reset(nA);
  reset(nB);
  if (!grid_barrier(q.bar, err)) return;
  for (int64_t s = 0; s < nsteps; ++s) {
    const bool onA = ((nsteps - 1 - s) & 1) == 0;
    const NodeP& cur = onA ? nA : nB;
    // P2G: every lane of a warp calls it the same number of times
    for (int64_t base = 0; base < q.np; base += nth)
      p2g_particle<D, double, GRAV, false>(q.g, cur, all, base + tid, q.grav[0], q.grav[1], q.grav[2], q.status);
    if (!grid_barrier(q.bar, err)) return;
    for (int64_t i = tid; i < Nn; i += nth) grid_node<D, false, true>(cur, i, q.dt, q.tol);
    // the other set was last read by the previous step's grid update, before
    // the barrier above; the next step sums into it after the barrier below
    if (s + 1 < nsteps) reset(onA ? nB : nA);
    if (!grid_barrier(q.bar, err)) return;
    for (int64_t p = tid; p < q.np; p += nth) {
      int b = 0;
      while (b + 1 < q.nb && p >= q.bbeg[b + 1]) ++b;
      const PartP pb{q.P, q.pitch, q.bbeg[b], q.np - q.bbeg[b], q.hat_c, q.hat_nl};
      g2p_particle<D, double, MAT, true>(q.g, cur, pb, p - q.bbeg[b], q.mp[b], q.dt, q.status);
    }
    if (q.rec && s >= q.first && (s - q.first) % q.every == 0) {
      // EnergiesFix sums of the particles this thread updated (Fix.jl:248-270;
      // the G2P's mapping, so they need no barrier first): m v.v, V sigma:eps
      // (diagonal + 2 off-diagonal), m v; a fixed CTA tree, a barrier, then
      // CTA 0 folds the CTAs' sums in block order
      constexpr int NQ = 2 + D;
      using L = Layout<D>;
      double e[NQ];
#pragma unroll
      for (int k = 0; k < NQ; ++k) e[k] = 0.0;
      for (int64_t p = tid; p < q.np; p += nth) {
        const double m = *field<double>(all, L::M, p);
        double vv = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const double v = *field<double>(all, L::V + a, p);
          vv += v * v;
          e[2 + a] += m * v;
        }
        e[0] += m * vv;
        double sd = 0.0, so = 0.0;
#pragma unroll
        for (int c = 0; c < L::S; ++c) {
          const double x = *field<double>(all, L::SIG + c, p) * *field<double>(all, L::EPS + c, p);
          if (c < D) sd += x;
          else so += x;
        }
        e[1] += *field<double>(all, L::VOL, p) * (sd + 2.0 * so);
      }
      __shared__ double sh[NQ][128];
#pragma unroll
      for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] = e[k];
      __syncthreads();
      for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
          for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NQ; ++k) q.partial[int64_t(blockIdx.x) * NQ + k] = sh[k][0];
      if (!grid_barrier(q.bar, err)) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        double t[NQ];
#pragma unroll
        for (int k = 0; k < NQ; ++k) t[k] = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b)
#pragma unroll
          for (int k = 0; k < NQ; ++k) t[k] += __ldcg(q.partial + int64_t(b) * NQ + k);
        double* out = q.rec->base + q.rec->idx * NQ;
        out[0] = 0.5 * t[0];
        out[1] = 0.5 * t[1];
#pragma unroll
        for (int k = 2; k < NQ; ++k) out[k] = t[k];
        q.rec->idx += 1;
      }
    }
  }
}

template <int D, int MAT, bool GRAV>
static const void* fused_fn() {
  return reinterpret_cast<const void*>(fused_steps_kernel<D, MAT, GRAV>);
}

static const void* fused_kernel_for(int dim, int mat, bool grav) {
#define JMPM_FK(D)                                                                                   \
  (mat == MPM_MAT_ELASTIC ? (grav ? fused_fn<D, MPM_MAT_ELASTIC, true>() : fused_fn<D, MPM_MAT_ELASTIC, false>()) \
   : mat == MPM_MAT_NEOHOOKEAN                                                                       \
       ? (grav ? fused_fn<D, MPM_MAT_NEOHOOKEAN, true>() : fused_fn<D, MPM_MAT_NEOHOOKEAN, false>())   \
       : (grav ? fused_fn<D, MPM_MAT_J2, true>() : fused_fn<D, MPM_MAT_J2, false>()))
  return dim == 2 ? JMPM_FK(2) : JMPM_FK(3);
#undef JMPM_FK
}

// barrier words, the partial sums of up to 152 CTAs (5 doubles each), then
// the second set of node accumulators (1 + 2 dim doubles per node)
size_t fused_bytes(int dim, int64_t nodes) {
  return 4 * sizeof(unsigned) + 152 * 5 * sizeof(double) + size_t(1 + 2 * dim) * size_t(nodes) * sizeof(double);
}

int fused_steps(int dim, cudaStream_t s, void* dev, const GridP& g, const NodeP& nd, void* P, int64_t pitch,
                int nb, const int64_t* bbeg, const int64_t* bcnt, const MatParams* mp, double dt, double tol,
                const double* grav, int64_t nsteps, unsigned* status, EnRec* rec, int64_t first, int64_t every,
                int32_t* hat_c, void* hat_nl) {
  if (nb < 1 || nb > MPM_BATCH_MAX_BODIES) return fail(MPM_ERR_ARG, "fused_steps: body count");
  FusedP q{};
  q.g = g;
  q.nd = nd;
  q.nd.bflag = nullptr;  // the dense reset of every step needs no block list
  q.nd.rmask = nullptr;
  q.P = P;
  q.pitch = pitch;
  q.np = 0;
  q.nb = nb;
  for (int b = 0; b < nb; ++b) {
    q.bbeg[b] = bbeg[b];
    q.mp[b] = mp[b];
    q.np += bcnt[b];
  }
  q.dt = dt;
  q.tol = tol;
  for (int a = 0; a < 3; ++a) q.grav[a] = grav[a];
  q.status = status;
  q.hat_c = hat_c;
  q.hat_nl = hat_nl;
  q.bar = static_cast<unsigned*>(dev);
  q.rec = rec;
  q.first = first;
  q.every = every > 0 ? every : 1;
  q.partial = reinterpret_cast<double*>(static_cast<char*>(dev) + 4 * sizeof(unsigned));
  const int64_t Nn = nd.nodeCount;
  q.m2 = q.partial + 152 * 5;
  q.p02 = q.m2 + Nn;
  q.f2 = q.p02 + int64_t(dim) * Nn;
  const bool gr = grav[0] != 0.0 || grav[1] != 0.0 || (dim == 3 && grav[2] != 0.0);
  const void* fn = fused_kernel_for(dim, mp[0].type, gr);
  // kFusedThreads-thread CTAs, one per SM at most, no more than the particles need
  constexpr int kFusedThreads = 64;
  int devid = 0, sms = 0, per = 0;
  BATCH_TRY(cudaGetDevice(&devid));
  BATCH_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, devid));
  BATCH_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kFusedThreads, 0));
  if (per < 1) return fail(MPM_ERR_CUDA, "fused_steps: the kernel does not fit on an SM");
  const int64_t want = std::max<int64_t>(1, (q.np + kFusedThreads - 1) / kFusedThreads);
  const unsigned nblk = unsigned(std::min<int64_t>(std::min<int64_t>(want, int64_t(sms)), 152));
  BATCH_TRY(cudaMemsetAsync(q.bar, 0, 3 * sizeof(unsigned), s));
  void* args[] = {&q, &nsteps};
  BATCH_TRY(cudaLaunchCooperativeKernel(fn, dim3(nblk), dim3(kFusedThreads), args, 0, s));
  return MPM_OK;
}

}  // namespace jmpm

extern "C" {

int mpm_batch_create(const mpm_instance_desc* instances, int32_t n, int32_t precision, mpm_batch** out) {
  if (!instances || !out || n < 1) return fail(MPM_ERR_ARG, "mpm_batch_create: need at least one problem");
  *out = nullptr;
  if (precision == MPM_PREC_DW) return fail(MPM_ERR_UNSUPPORTED, "mpm_batch_create: MPM_PREC_DW is for contexts");
  if (precision != MPM_PREC_F64 && precision != MPM_PREC_F32)
    return fail(MPM_ERR_ARG, "mpm_batch_create: unknown precision");
  const int D = instances[0].grid.dim;
  if (D != 2 && D != 3) return fail(MPM_ERR_ARG, "mpm_batch_create: dim must be 2 or 3");
  int mat = -1;
  bool grav = false, mixed = false, any_contact = false;
  for (int i = 0; i < n; ++i) {
    const mpm_instance_desc& d = instances[i];
    if (d.grid.dim != D) return fail(MPM_ERR_ARG, "mpm_batch_create: all problems must share the dimension");
    for (int a = 0; a < D; ++a) {
      if (d.grid.nodes[a] < 2 || d.grid.nodes[a] > (1 << 20))
        return fail(MPM_ERR_ARG, "mpm_batch_create: bad node count");
      if (!(d.grid.xmax[a] > d.grid.xmin[a])) return fail(MPM_ERR_ARG, "mpm_batch_create: need xmax > xmin");
    }
    if (!(d.dt > 0.0)) return fail(MPM_ERR_ARG, "mpm_batch_create: dt must be > 0");
    if (d.nbodies < 1 || d.nbodies > MPM_BATCH_MAX_BODIES || !d.bodies)
      return fail(MPM_ERR_ARG, "mpm_batch_create: 1 to MPM_BATCH_MAX_BODIES bodies per problem");
    if (d.contact != 0 && d.contact != 1) return fail(MPM_ERR_ARG, "mpm_batch_create: contact must be 0 or 1");
    if (d.contact && d.nbodies > kMaxContactBodies)
      return fail(MPM_ERR_ARG, "mpm_batch_create: contact mode supports at most " +
                                   std::to_string(kMaxContactBodies) + " bodies");
    if (d.contact && !(d.friction >= 0.0)) return fail(MPM_ERR_ARG, "mpm_batch_create: friction < 0");
    any_contact = any_contact || d.contact;
    for (int a = 0; a < D; ++a) grav = grav || d.body_force[a] != 0.0;
    for (int k = 0; k < d.nbodies; ++k) {
      const mpm_body_desc& bd = d.bodies[k];
      if (bd.count < 0) return fail(MPM_ERR_ARG, "mpm_batch_create: negative particle count");
      if (bd.count > 0 && (!bd.pos || !bd.velocity || !bd.mass || !bd.volume || !bd.volume_initial))
        return fail(MPM_ERR_ARG, "mpm_batch_create: pos, velocity, mass, volume and volume_initial are required");
      if (bd.mat.type == MPM_MAT_RIGID)
        return fail(MPM_ERR_UNSUPPORTED, "mpm_batch_create: rigid solids run in single contexts only");
      if (!material_ok(bd.mat.type, D))
        return fail(MPM_ERR_ARG, "mpm_batch_create: unknown material type");
      if (!material_params_ok(bd.mat))
        return fail(MPM_ERR_ARG, "mpm_batch_create: Johnson-Cook with damage needs density > 0 and Cp > 0");
      mixed = mixed || (mat >= 0 && bd.mat.type != mat);
      mat = bd.mat.type;
    }
  }
  mpm_batch* b = new mpm_batch();
  b->dim = D;
  b->f32 = precision == MPM_PREC_F32;
  b->esz = b->f32 ? sizeof(float) : sizeof(double);
  b->mat = mat < 0 ? MPM_MAT_ELASTIC : mat;
  b->grav = grav;
  b->ninst = n;
  b->persistent_ok = !mixed && !any_contact;
  b->strategy = b->persistent_ok ? MPM_BATCH_PERSISTENT : MPM_BATCH_WIDE;
  int dev = 0, r = MPM_OK;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->e1);
  if (e != cudaSuccess) r = fail(MPM_ERR_CUDA, std::string("mpm_batch_create: ") + cudaGetErrorString(e));
  if (r == MPM_OK) r = D == 2 ? create_t<2>(instances, n, b) : create_t<3>(instances, n, b);
  if (r != MPM_OK) {
    std::string msg = mpm_last_error();
    destroy_batch(b);
    set_last_error(r, msg);
    return r;
  }
  *out = b;
  return MPM_OK;
}

int mpm_batch_step(mpm_batch* b, int64_t nsteps) {
  if (!b || nsteps < 0) return fail(MPM_ERR_ARG, "mpm_batch_step: bad argument");
  BATCH_TRY(cudaMemsetAsync(b->d_status, 0, size_t(b->ninst) * sizeof(unsigned), b->stream));
  BATCH_TRY(cudaEventRecord(b->e0, b->stream));
  int r = run_steps(b, nsteps);
  if (r) return r;
  BATCH_TRY(cudaEventRecord(b->e1, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  float ms = 0.f;
  BATCH_TRY(cudaEventElapsedTime(&ms, b->e0, b->e1));
  b->last_ms = ms;
  std::vector<unsigned> st(static_cast<size_t>(b->ninst));
  BATCH_TRY(cudaMemcpy(st.data(), b->d_status, st.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
  unsigned all = 0;
  for (unsigned s : st) all |= s;
  r = status_code(all);
  if (r != MPM_OK) return fail(r, "mpm_batch_step: a problem reported a failure (see mpm_batch_status)");
  return MPM_OK;
}

int mpm_batch_status(mpm_batch* b, int32_t* status) {
  if (!b || !status) return fail(MPM_ERR_ARG, "mpm_batch_status: null argument");
  std::vector<unsigned> st(static_cast<size_t>(b->ninst));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  BATCH_TRY(cudaMemcpy(st.data(), b->d_status, st.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
  for (int i = 0; i < b->ninst; ++i) status[i] = status_code(st[i]);
  return MPM_OK;
}

int mpm_batch_download(mpm_batch* b, int32_t instance, int32_t body, const mpm_body_view* v) {
  if (!b || !v) return fail(MPM_ERR_ARG, "mpm_batch_download: null argument");
  if (instance < 0 || instance >= b->ninst || body < 0 || body >= b->inst[instance].nb)
    return fail(MPM_ERR_ARG, "mpm_batch_download: index out of range");
  const int D = b->dim;
  const PartP pp = b->body(instance, body);
  const int X = 0, V = D, VOL = 2 * D + 1, F = 2 * D + 3, EPS = F + D * D, S = D == 2 ? 3 : 6;
  const int SIG = EPS + S, VM = SIG + S, ALPHA = VM + 1, EP = ALPHA + 1;
  int r;
  if ((r = download(b, pp, v->pos, D, X, ident(D)))) return r;
  if ((r = download(b, pp, v->velocity, D, V, ident(D)))) return r;
  if ((r = download(b, pp, v->volume, 1, VOL, ident(1)))) return r;
  if ((r = download(b, pp, v->F, D * D, F, ident(D * D)))) return r;
  if ((r = download(b, pp, v->strain, D * D, EPS, full_from_sym(D)))) return r;
  if ((r = download(b, pp, v->stress, D * D, SIG, full_from_sym(D)))) return r;
  if ((r = download(b, pp, v->alpha, 1, ALPHA, ident(1)))) return r;
  if ((r = download(b, pp, v->alphadot, 1, D == 2 ? Layout<2>::ALPHAD : Layout<3>::ALPHAD, ident(1)))) return r;
  if (D == 3 && b->inst[instance].mp[body].type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    if ((r = download(b, pp, v->damage_init, 1, EP, ident(1)))) return r;
    if ((r = download(b, pp, v->damage, 1, EP + 1, ident(1)))) return r;
    if ((r = download(b, pp, v->temperature, 1, EP + 2, ident(1)))) return r;
  } else if ((r = D == 2 ? download(b, pp, v->pstrain, 3, EP, ident(3))
                        : download(b, pp, v->pstrain, 9, EP, full_from_sym(3)))) {
    return r;
  }
  if (v->vmstr && pp.count > 0) {
    if (b->inst[instance].mp[body].type == MPM_MAT_J2) {
      if (D == 2) Launchers<2>::j2_vm(b->stream, pp, b->f32, b->staging);
      else Launchers<3>::j2_vm(b->stream, pp, b->f32, b->staging);
      BATCH_TRY(cudaGetLastError());
      BATCH_TRY(cudaMemcpyAsync(v->vmstr, b->staging, size_t(pp.count) * sizeof(double), cudaMemcpyDeviceToHost,
                                b->stream));
      BATCH_TRY(cudaStreamSynchronize(b->stream));
    } else if ((r = download(b, pp, v->vmstr, 1, VM, ident(1)))) {
      return r;
    }
  }
  return MPM_OK;
}

int mpm_batch_energies(mpm_batch* b, double* out) {
  if (!b || !out) return fail(MPM_ERR_ARG, "mpm_batch_energies: null argument");
  return b->dim == 2 ? energies_t<2>(b, out) : energies_t<3>(b, out);
}

int mpm_batch_set_launch(mpm_batch* b, int32_t threads, int32_t ctas_per_sm) {
  if (!b || threads < 32 || threads > 1024 || threads % 32 != 0 || ctas_per_sm < 0)
    return fail(MPM_ERR_ARG, "mpm_batch_set_launch: threads must be a multiple of 32 in [32, 1024]");
  b->threads = threads;
  b->ctas_per_sm = ctas_per_sm;
  return MPM_OK;
}

int mpm_batch_tune(mpm_batch* b, int64_t probe_steps, int32_t* threads, int32_t* ctas_per_sm, double* ms_per_step) {
  if (!b || probe_steps < 1) return fail(MPM_ERR_ARG, "mpm_batch_tune: bad argument");
  const size_t bytes = size_t(b->NF) * size_t(b->np > 0 ? b->np : 1) * b->esz;
  void* scratch = nullptr;
  BATCH_TRY(cudaMalloc(&scratch, bytes));
  const int th_list[] = {64, 128, 256, 512, 1024};
  const int cta_list[] = {1, 2, 4, 8, 16};
  double best = 1e300;
  int bt = b->threads, bc = b->ctas_per_sm;
  int rc = MPM_OK;
  for (int th : th_list) {
    if (!b->persistent_ok) break;
    for (int cps : cta_list) {
      cudaMemcpyAsync(scratch, b->P, bytes, cudaMemcpyDeviceToDevice, b->stream);
      cudaEventRecord(b->e0, b->stream);
      int r = launch(b, scratch, probe_steps, th, cps);
      cudaEventRecord(b->e1, b->stream);
      cudaError_t e = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess) {
        rc = fail(MPM_ERR_CUDA, std::string("mpm_batch_tune: ") + cudaGetErrorString(e));
        break;
      }
      if (r != MPM_OK) continue;  // shape does not fit this kernel
      float ms = 0.f;
      cudaEventElapsedTime(&ms, b->e0, b->e1);
      if (ms < best) {
        best = ms;
        bt = th;
        bc = cps;
      }
    }
    if (rc != MPM_OK) break;
  }
  int bs = MPM_BATCH_PERSISTENT;
  if (rc == MPM_OK) {
    // WIDE: probe_steps on the batch itself, particles saved before and put back after
    b->nodes_dirty = true;  // the persistent probes above used the node arrays
    BATCH_TRY(cudaMemcpyAsync(scratch, b->P, bytes, cudaMemcpyDeviceToDevice, b->stream));
    const int saved = b->strategy;
    b->strategy = MPM_BATCH_WIDE;
    int r = wide_run(b, 1);  // builds the step graph outside the timed region
    if (r == MPM_OK) {
      cudaEventRecord(b->e0, b->stream);
      r = wide_run(b, probe_steps - 1 > 0 ? probe_steps - 1 : 1);
      cudaEventRecord(b->e1, b->stream);
    }
    b->strategy = saved;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) rc = fail(MPM_ERR_CUDA, std::string("mpm_batch_tune: ") + cudaGetErrorString(e));
    else if (r != MPM_OK) rc = r;
    if (rc == MPM_OK) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, b->e0, b->e1);
      const double per = ms * double(probe_steps) / double(probe_steps - 1 > 0 ? probe_steps - 1 : 1);
      if (per < best) {
        best = per;
        bs = MPM_BATCH_WIDE;
      }
      cudaMemcpyAsync(b->P, scratch, bytes, cudaMemcpyDeviceToDevice, b->stream);
      rc = wide_clean(b);
      if (rc == MPM_OK) {
        e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) rc = fail(MPM_ERR_CUDA, std::string("mpm_batch_tune: ") + cudaGetErrorString(e));
      }
    }
  }
  cudaFree(scratch);
  if (rc != MPM_OK) return rc;
  b->strategy = bs;
  b->threads = bt;
  b->ctas_per_sm = bc;
  if (threads) *threads = bt;
  if (ctas_per_sm) *ctas_per_sm = bc;
  if (ms_per_step) *ms_per_step = best / double(probe_steps);
  BATCH_TRY(cudaMemsetAsync(b->d_status, 0, size_t(b->ninst) * sizeof(unsigned), b->stream));
  return MPM_OK;
}

int mpm_batch_jvp(mpm_batch* b, int64_t nsteps, const double* dE, double* x_dot) {
  if (!b || nsteps < 0) return fail(MPM_ERR_ARG, "mpm_batch_jvp: bad argument");
  if (b->f32) return fail(MPM_ERR_UNSUPPORTED, "mpm_batch_jvp: needs an FP64 batch");
  for (size_t q = 0; q < b->wbody.size(); ++q) {
    const int t = b->wbody[q].mp.type;
    if (t != MPM_MAT_ELASTIC && t != MPM_MAT_NEOHOOKEAN)
      return fail(MPM_ERR_UNSUPPORTED, "mpm_batch_jvp: elastic and neo-Hookean bodies only");
  }
  for (const WideInst& W : b->winst)
    if (W.contact && b->dim == 2 && W.cp.friction > 0.0)
      return fail(MPM_ERR_UNSUPPORTED, "mpm_batch_jvp: frictionless contact only");
  int r = jvp_setup(b, dE);
  if (r) return r;
  BATCH_TRY(cudaMemsetAsync(b->d_status, 0, size_t(b->ninst) * sizeof(unsigned), b->stream));
  BATCH_TRY(cudaEventRecord(b->e0, b->stream));
  if ((r = jvp_run(b, nsteps))) return r;
  BATCH_TRY(cudaEventRecord(b->e1, b->stream));
  BATCH_TRY(cudaStreamSynchronize(b->stream));
  float ms = 0.f;
  BATCH_TRY(cudaEventElapsedTime(&ms, b->e0, b->e1));
  b->last_ms = ms;
  if (x_dot) {
    const int D = b->dim;
    size_t off = 0;
    for (int i = 0; i < b->ninst; ++i)
      for (int k = 0; k < b->inst[i].nb; ++k) {
        PartP tp = b->body(i, k);
        tp.base = b->tpart;
        if (D == 2) Launchers<2>::soa_to_aos(b->stream, tp, false, b->staging, D, TanLayout<2>::XD, ident(D));
        else Launchers<3>::soa_to_aos(b->stream, tp, false, b->staging, D, TanLayout<3>::XD, ident(D));
        BATCH_TRY(cudaGetLastError());
        BATCH_TRY(cudaMemcpyAsync(x_dot + off, b->staging, size_t(tp.count) * D * sizeof(double),
                                  cudaMemcpyDeviceToHost, b->stream));
        BATCH_TRY(cudaStreamSynchronize(b->stream));
        off += size_t(tp.count) * D;
      }
  }
  std::vector<unsigned> st(static_cast<size_t>(b->ninst));
  BATCH_TRY(cudaMemcpy(st.data(), b->d_status, st.size() * sizeof(unsigned), cudaMemcpyDeviceToHost));
  unsigned all = 0;
  for (unsigned v : st) all |= v;
  r = status_code(all);
  if (r != MPM_OK) return fail(r, "mpm_batch_jvp: a problem reported a failure (see mpm_batch_status)");
  return MPM_OK;
}

int mpm_batch_set_strategy(mpm_batch* b, int32_t strategy) {
  if (!b || (strategy != MPM_BATCH_PERSISTENT && strategy != MPM_BATCH_WIDE))
    return fail(MPM_ERR_ARG, "mpm_batch_set_strategy: unknown strategy");
  if (strategy == MPM_BATCH_PERSISTENT && !b->persistent_ok)
    return fail(MPM_ERR_ARG, "mpm_batch_set_strategy: the persistent kernel needs one material model type and no "
                             "contact");
  b->strategy = strategy;
  return MPM_OK;
}

int mpm_batch_strategy(mpm_batch* b, int32_t* strategy) {
  if (!b || !strategy) return fail(MPM_ERR_ARG, "mpm_batch_strategy: null argument");
  *strategy = b->strategy;
  return MPM_OK;
}

int mpm_batch_last_ms(mpm_batch* b, double* ms) {
  if (!b || !ms) return fail(MPM_ERR_ARG, "mpm_batch_last_ms: null argument");
  *ms = b->last_ms;
  return MPM_OK;
}

int mpm_batch_destroy(mpm_batch* b) {
  if (b) {
    cudaStreamSynchronize(b->stream);
    destroy_batch(b);
  }
  return MPM_OK;
}

}  // extern "C"
