// mpm_sparse.cuh -- the grid stages over the node blocks particles touch.
//
// Nodes are grouped in blocks of 64 (4x4x4 in 3D, 8x8 in 2D).  P2G sets a
// flag for every block holding one of a particle's stencil nodes; a
// compaction pass turns the flags into a list (and clears them); the grid
// update runs over the listed blocks only, and the next step clears the
// accumulators of the same blocks before its P2G.  Nodes outside the list
// keep zero accumulators and are never read by G2P, so a mostly empty grid
// (the Taylor bar fills ~10% of its cells) costs nothing per step.
#pragma once

#include "mpm_common.cuh"

namespace jmpm {

template <int D>
struct BlockShape {
  static constexpr int B = (D == 2) ? 8 : 4;   // nodes per block edge
  static constexpr int NODES = (D == 2) ? 64 : 64;
};

// Flag the blocks of the stencil nodes of a particle whose base cell is c.
template <int D>
__device__ __forceinline__ void mark_blocks(const NodeP& nd, const int* c) {
  constexpr int B = BlockShape<D>::B;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    lo[a] = c[a] / B;
    hi[a] = (c[a] + 1) / B;
  }
  for (int bz = lo[2]; bz <= hi[2]; ++bz)
    for (int by = lo[1]; by <= hi[1]; ++by)
      for (int bx = lo[0]; bx <= hi[0]; ++bx) {
        int64_t blk = bx + int64_t(nd.nb[0]) * (by + int64_t(nd.nb[1]) * bz);
        if (nd.bflag[blk] == 0u) nd.bflag[blk] = 1u;
      }
}

// flags -> list (warp-aggregated append), flags cleared
static __global__ void __launch_bounds__(256) compact_blocks_kernel(NodeP nd) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  bool on = i < nd.nblk && nd.bflag[i] != 0u;
  unsigned m = __ballot_sync(0xffffffffu, on);
  if (m == 0u) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(nd.bcount, uint32_t(__popc(m)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (on) {
    nd.blist[base + __popc(m & ((1u << lane) - 1u))] = uint32_t(i);
    nd.bflag[i] = 0u;
  }
}

// node index of local node `l` of listed block `blk`, or -1 outside the grid
template <int D>
__device__ __forceinline__ int64_t block_node(const NodeP& nd, uint32_t blk, int l) {
  constexpr int B = BlockShape<D>::B;
  int64_t bx = blk % uint32_t(nd.nb[0]);
  int64_t rest = blk / uint32_t(nd.nb[0]);
  int64_t by = rest % nd.nb[1];
  int64_t bz = rest / nd.nb[1];
  int64_t ix = bx * B + (l % B);
  int64_t iy = by * B + ((l / B) % B);
  int64_t iz = (D == 3) ? bz * B + l / (B * B) : 0;
  if (ix >= nd.nn[0] || iy >= nd.nn[1] || iz >= nd.nn[2]) return -1;
  return ix + nd.nn[0] * (iy + nd.nn[1] * iz);
}

// zero the accumulators (m, p0, f and, where present, normals, MUSL p2, mass
// stencil and rigid-body node marks) of the listed blocks before the next P2G
template <int D>
__global__ void __launch_bounds__(256) clear_blocks_kernel(NodeP nd) {
  const int64_t Nn = nd.nodeCount;
  const int64_t work = int64_t(*nd.bcount) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = block_node<D>(nd, nd.blist[w >> 6], int(w & 63));
    if (i < 0) continue;
    nd.m[i] = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      nd.p0[a * Nn + i] = 0.0;
      nd.f[a * Nn + i] = 0.0;
      if (nd.nrm) nd.nrm[a * Nn + i] = 0.0;
      if (nd.p2) nd.p2[a * Nn + i] = 0.0;
    }
    if (nd.mc)
      for (int o = 0; o < nd.nmc; ++o) nd.mc[o * Nn + i] = 0.0;
    if (nd.rmask) nd.rmask[i] = 0u;
  }
}

}  // namespace jmpm
