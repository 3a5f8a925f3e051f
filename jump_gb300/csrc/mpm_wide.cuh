// mpm_wide.cuh -- the wide batch strategy: every stage of a USL step is one
// launch over all problems of a batch.
//
//   particles  a tile table maps each CTA to 256 consecutive particles of one
//              body (WideTile); the body table (WideBody) gives the body's
//              particle range, its node field and its material, and the
//              problem table (WideInst) the grid, dt, tolerance, body force
//              and, in contact mode, every node field of the problem;
//   nodes      each problem's node blocks (64 nodes, mpm_sparse.cuh) get
//              global ids blk0 .. blk0 + nblk - 1; P2G flags them through
//              the problem's NodeP, one compaction pass lists the flagged
//              blocks of all problems, and the clear and grid stages walk
//              that list, finding a block's problem in blk_inst.
// A CTA copies the tables it uses into shared memory first, so the device
// functions of the single-problem kernels run unchanged on them.
#pragma once

#include "mpm_kernels.cuh"

namespace jmpm {

struct WideBody {
  PartP pp;
  NodeP nd;       // the field this body scatters to and gathers from
  MatParams mp;
  int inst;
};

struct WideInst {
  GridP g;
  ContactP cp;    // contact: one field per body; otherwise cp.body[0] is the problem's field
  int contact;
  double dt, tol, grav[3];
  int64_t blk0;
};

struct WideTile {
  int body;
  int64_t start;  // first particle (within the body) of this CTA's 256
};

// cooperative copy of a table entry into shared memory
template <class T>
__device__ __forceinline__ void stage(T* dst, const T* src) {
  static_assert(sizeof(T) % 4 == 0, "tables are 4-byte multiples");
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int k = threadIdx.x; k < int(sizeof(T) / 4); k += blockDim.x) d[k] = s[k];
}

template <int D, class R>
__global__ void __launch_bounds__(256) wide_p2g_kernel(const WideBody* __restrict__ bodies,
                                                       const WideInst* __restrict__ inst,
                                                       const WideTile* __restrict__ tiles, unsigned* status) {
  __shared__ WideBody sB;
  __shared__ GridP sG;
  __shared__ double sGrav[3];
  const WideTile tl = tiles[blockIdx.x];
  stage(&sB, bodies + tl.body);
  __syncthreads();
  const WideInst* I = inst + sB.inst;
  stage(&sG, &I->g);
  if (threadIdx.x < 3) sGrav[threadIdx.x] = I->grav[threadIdx.x];
  __syncthreads();
  const int64_t t = tl.start + threadIdx.x;
  unsigned* st = status + sB.inst;
  if (sGrav[0] != 0.0 || sGrav[1] != 0.0 || sGrav[2] != 0.0)
    p2g_particle<D, R, true>(sG, sB.nd, sB.pp, t, sGrav[0], sGrav[1], sGrav[2], st);
  else
    p2g_particle<D, R, false>(sG, sB.nd, sB.pp, t, 0.0, 0.0, 0.0, st);
}

template <int D, class R>
__global__ void __launch_bounds__(256) wide_g2p_kernel(const WideBody* __restrict__ bodies,
                                                       const WideInst* __restrict__ inst,
                                                       const WideTile* __restrict__ tiles, unsigned* status) {
  __shared__ WideBody sB;
  __shared__ GridP sG;
  __shared__ double sDt;
  const WideTile tl = tiles[blockIdx.x];
  stage(&sB, bodies + tl.body);
  __syncthreads();
  const WideInst* I = inst + sB.inst;
  stage(&sG, &I->g);
  if (threadIdx.x == 0) sDt = I->dt;
  __syncthreads();
  const int64_t t = tl.start + threadIdx.x;
  if (t >= sB.pp.count) return;
  unsigned* st = status + sB.inst;
  switch (sB.mp.type) {
    case MPM_MAT_ELASTIC: g2p_particle<D, R, MPM_MAT_ELASTIC>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st); break;
    case MPM_MAT_NEOHOOKEAN: g2p_particle<D, R, MPM_MAT_NEOHOOKEAN>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st); break;
    case MPM_MAT_JOHNSON_COOK:
      if constexpr (D == 3) g2p_particle<D, R, MPM_MAT_JOHNSON_COOK>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st);
      break;
    case MPM_MAT_VOCE:
      if constexpr (D == 3) g2p_particle<D, R, MPM_MAT_VOCE>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st);
      break;
    case MPM_MAT_JOHNSON_COOK_DAMAGE:
      if constexpr (D == 3) g2p_particle<D, R, MPM_MAT_JOHNSON_COOK_DAMAGE>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st);
      break;
    default: g2p_particle<D, R, MPM_MAT_J2>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st); break;
  }
}

// listed block w >> 6, local node w & 63 -> (problem, node index) or node -1
template <int D>
__device__ __forceinline__ int64_t wide_node(const WideInst* inst, const int* blk_inst, const uint32_t* list,
                                             int64_t w, const WideInst*& I) {
  const uint32_t gb = list[w >> 6];
  I = inst + blk_inst[gb];
  return block_node<D>(I->cp.body[0], uint32_t(gb - I->blk0), int(w & 63));
}

template <int D, bool F32COPY>
__global__ void __launch_bounds__(256) wide_grid_kernel(const WideInst* __restrict__ inst,
                                                        const int* __restrict__ blk_inst,
                                                        const uint32_t* __restrict__ list,
                                                        const uint32_t* __restrict__ count) {
  const int64_t work = int64_t(*count) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const WideInst* I;
    const int64_t i = wide_node<D>(inst, blk_inst, list, w, I);
    if (i < 0) continue;
    if (I->contact) contact_node<D, F32COPY>(I->cp, i, I->dt, I->tol);
    else grid_node<D, F32COPY>(I->cp.body[0], i, I->dt, I->tol);
  }
}

// zero the accumulators of the listed blocks of every field (before P2G)
template <int D>
__global__ void __launch_bounds__(256) wide_clear_kernel(const WideInst* __restrict__ inst,
                                                         const int* __restrict__ blk_inst,
                                                         const uint32_t* __restrict__ list,
                                                         const uint32_t* __restrict__ count) {
  const int64_t work = int64_t(*count) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const WideInst* I;
    const int64_t i = wide_node<D>(inst, blk_inst, list, w, I);
    if (i < 0) continue;
    const int nf = I->contact ? I->cp.nb : 1;
    for (int b = 0; b < nf; ++b) {
      const NodeP& nd = I->cp.body[b];
      const int64_t Nn = nd.nodeCount;
      nd.m[i] = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        nd.p0[a * Nn + i] = 0.0;
        nd.f[a * Nn + i] = 0.0;
        if (nd.nrm) nd.nrm[a * Nn + i] = 0.0;
      }
    }
  }
}

}  // namespace jmpm
