// mpm_musl.cuh -- MUSL (modified update stress last) with the FLIP/PIC blend
// alpha, FP64, one velocity field.
//
// 3D, lumped mass (SolveExplicitSolidMechanics3D.jl:14-223):
//   P2G (no body force in this solver) -> grid: p = p0 + f dt, fixed dofs of
//   p0 and p zeroed, dv = (p - alpha p0)/m, vdt = (p/m) dt where m > 0 ->
//   G2P-1: v = alpha v + sum N dv, then P2G-2: p2 += N m v ->
//   vg = (p2/m) dt where m > 0 (p2 carries no Dirichlet condition) ->
//   G2P-2: x += sum N vdt, (L dt)_ij = sum dN_i vg_j (the solver builds the
//   velocity gradient transposed, :187-189), F, J, V, strain, stress.
// 2D, blended consistent mass (SolveExplicitSolidMechanics2D.jl:24-329):
//   P2G with body force plus the consistent mass stencil M_ij = sum m N_i N_j
//   (9 entries per node for the linear basis, (2K-1)^2 for K nodes per axis) -> v0 = B \ p0 and dv = B \ (dt f) per component with
//   B = 0.1 diag(m) + 0.9 M (massless rows: 1 on the diagonal), by Jacobi-
//   preconditioned conjugate gradients, one CTA per right-hand side ->
//   gv = v0 + dv; dv_node = gv - alpha v0, vdt = vg = gv dt where m > 0 ->
//   G2P-1 -> G2P-2 with (L dt)_ij = sum vg_i dN_j.  The solver's Dirichlet
//   update of nodalMomentum is never read by the particle updates, so fixed
//   nodes do not constrain it; as written.
#pragma once

#include "mpm_kernels.cuh"

namespace jmpm {

// ---- 3D lumped-mass grid update -----------------------------------------
template <int D>
__global__ void __launch_bounds__(256) musl_lumped_grid_kernel(NodeP nd, double dt, double alpha) {
  const int64_t Nn = nd.nodeCount;
  const int64_t work = int64_t(*nd.bcount) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = block_node<D>(nd, nd.blist[w >> 6], int(w & 63));
    if (i < 0) continue;
    const double m = nd.m[i];
    const unsigned fx = nd.fixed[i];
    const bool live = m > 0.0;
    const double invM = live ? 1.0 / m : 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double p0 = nd.p0[a * Nn + i];
      double p = __dadd_rn(p0, __dmul_rn(nd.f[a * Nn + i], dt));  // p = p0 + f*dt
      if (fx & (1u << a)) p0 = p = 0.0;
      nd.dv[a * Nn + i] = live ? (p - alpha * p0) * invM : 0.0;
      nd.vdt[a * Nn + i] = live ? (p * invM) * dt : 0.0;
    }
  }
}

// ---- G2P-1: velocity blend; P2: also P2G-2 of the new velocity ------------
template <int D, bool P2>
__global__ void __launch_bounds__(256) musl_g2p1_kernel(GridP g, NodeP nd, PartP pp, double alpha,
                                                        unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<double>(pp, L::X + a, p);
  Hat<D, double> h;
  if (!hat<D, double>(g, x, h)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  Corners<D, double> cr;
  corners<D, double>(g, h, cr);
  const int64_t Nn = nd.nodeCount;
  double vacc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) vacc[a] = 0.0;
#pragma unroll
  for (int k = 0; k < (1 << D); ++k)
#pragma unroll
    for (int a = 0; a < D; ++a) vacc[a] += cr.N[k] * __ldg(nd.dv + a * Nn + cr.node[k]);
  double v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    v[a] = alpha * *field<double>(pp, L::V + a, p) + vacc[a];
    *field<double>(pp, L::V + a, p) = v[a];
  }
  if (P2) {
    const double mp = *field<double>(pp, L::M, p);
#pragma unroll
    for (int k = 0; k < (1 << D); ++k) {
      const double Nm = cr.N[k] * mp;
#pragma unroll
      for (int a = 0; a < D; ++a) atomicAdd(nd.p2 + a * Nn + cr.node[k], Nm * v[a]);
    }
  }
}

// ---- 3D: vg = (p2/m) dt where m > 0 ----------------------------------------
template <int D>
__global__ void __launch_bounds__(256) musl_vg_kernel(NodeP nd, double dt) {
  const int64_t Nn = nd.nodeCount;
  const int64_t work = int64_t(*nd.bcount) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = block_node<D>(nd, nd.blist[w >> 6], int(w & 63));
    if (i < 0) continue;
    const double m = nd.m[i];
    const double mii = m > 0.0 ? 1.0 / m : 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) nd.vg[a * Nn + i] = (mii * nd.p2[a * Nn + i]) * dt;
  }
}

// ---- G2P-2: positions, velocity gradient, F, J, V, strain, stress ----------
template <int D, int MAT, bool TRANSPOSED>
__global__ void __launch_bounds__(256) musl_g2p2_kernel(GridP g, NodeP nd, PartP pp, MatParams mp,
                                                        unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<double>(pp, L::X + a, p);
  Hat<D, double> h;
  if (!hat<D, double>(g, x, h)) return;  // reported by G2P-1
  Corners<D, double> cr;
  corners<D, double>(g, h, cr);
  const int64_t Nn = nd.nodeCount;
  double Ldt[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int j = 0; j < D; ++j) Ldt[a][j] = 0.0;
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    const int64_t n = cr.node[k];
    double vg[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      x[a] += cr.N[k] * __ldg(nd.vdt + a * Nn + n);
      vg[a] = __ldg(nd.vg + a * Nn + n);
    }
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int j = 0; j < D; ++j) Ldt[a][j] += TRANSPOSED ? cr.dN[k][a] * vg[j] : vg[a] * cr.dN[k][j];
  }
  bool fin = true;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    *field<double>(pp, L::X + a, p) = x[a];
    fin &= finite_bits(x[a]) & finite_bits(*field<double>(pp, L::V + a, p));
  }
  kinematics_stress<D, double, MAT>(pp, p, Ldt, mp, fin, status);
}

// ---- 2D: P2G plus the consistent mass stencil -------------------------------
// mc[o * Nn + i] += (N_i m) N_j for the node pairs (i, j) of the particle's
// cell, o = (dx + 1) + 3 (dy + 1) the offset of j from i
template <bool GRAV>
__global__ void __launch_bounds__(256) musl2d_p2g_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy,
                                                         unsigned* status) {
  using L = Layout<2>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  p2g_particle<2, double, GRAV>(g, nd, pp, t, gx, gy, 0.0, status);
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[2] = {*field<double>(pp, L::X, p), *field<double>(pp, L::X + 1, p)};
  Hat<2, double> h;
  if (!hat<2, double>(g, x, h)) return;
  Corners<2, double> cr;
  corners<2, double>(g, h, cr);
  const double m = *field<double>(pp, L::M, p);
  const int64_t Nn = nd.nodeCount;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const double Nim = cr.N[a] * m;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int o = ((b & 1) - (a & 1) + 1) + 3 * ((b >> 1) - (a >> 1) + 1);
      atomicAdd(nd.mc + o * Nn + cr.node[a], Nim * cr.N[b]);
    }
  }
}

constexpr int kCgMaxIt = 1000;
constexpr double kCgTol = 1e-13;  // relative residual

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();  // sh is free (the previous sum has been read)
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  const int nw = int(blockDim.x + 31) >> 5;
  for (int k = 0; k < nw; ++k) s += sh[k];  // every thread, same order: same value everywhere
  return s;
}

// (B v)_i with B = 0.1 diag(m) + 0.9 M, massless rows the identity.  K nodes per
// axis in a particle's support: M couples nodes up to K-1 apart per axis, so
// its stencil has W x W entries, W = 2K - 1 (o = (dx + K - 1) + W (dy + K - 1)).
template <int K>
__device__ __forceinline__ double musl2d_apply(const NodeP& nd, const double* v, int64_t i) {
  constexpr int W = 2 * K - 1;
  const int64_t Nn = nd.nodeCount, nx = nd.nn[0], ny = nd.nn[1];
  const double m = nd.m[i];
  if (!(m != 0.0)) return v[i];
  const int64_t ix = i % nx, iy = i / nx;
  double s = (0.1 * m) * v[i];
#pragma unroll
  for (int o = 0; o < W * W; ++o) {
    const double c = nd.mc[o * Nn + i];
    const int64_t jx = ix + (o % W) - (K - 1), jy = iy + (o / W) - (K - 1);
    if (c != 0.0 && jx >= 0 && jx < nx && jy >= 0 && jy < ny) s += (0.9 * c) * v[jx + nx * jy];
  }
  return s;
}

template <int K>
__device__ __forceinline__ double musl2d_diag(const NodeP& nd, int64_t i) {
  constexpr int W = 2 * K - 1;
  const double m = nd.m[i];
  return m != 0.0 ? 0.1 * m + 0.9 * nd.mc[((K - 1) * (W + 1)) * nd.nodeCount + i] : 1.0;
}

// One CTA per right-hand side over the nodes of the listed blocks; bounded by
// kCgMaxIt iterations, after which ST_SOLVER is set.
template <int K>
__global__ void __launch_bounds__(1024) musl2d_cg_kernel(NodeP nd, CgP cg, double dt, unsigned* status) {
  __shared__ double sh[32];
  const int rhs = blockIdx.x;
  const int64_t Nn = nd.nodeCount;
  const int64_t work = int64_t(*nd.bcount) * 64;
  double* x = cg.x[rhs];
  double* r = cg.r[rhs];
  double* p = cg.p[rhs];
  double* q = cg.q[rhs];
  const double* bsrc = rhs < 2 ? nd.p0 + rhs * Nn : nd.f + (rhs - 2) * Nn;
  const double bscale = rhs < 2 ? 1.0 : dt;
  double rz = 0.0, bb = 0.0;
  for (int64_t w = threadIdx.x; w < work; w += blockDim.x) {
    const int64_t i = block_node<2>(nd, nd.blist[w >> 6], int(w & 63));
    if (i < 0) continue;
    const double b = bscale * bsrc[i];
    const double z = b / musl2d_diag<K>(nd, i);
    x[i] = 0.0;
    r[i] = b;
    p[i] = z;
    rz += b * z;
    bb += b * b;
  }
  rz = block_sum(rz, sh);
  bb = block_sum(bb, sh);
  double rr = bb;
  bool done = bb == 0.0;
  for (int it = 0; it < kCgMaxIt && !done; ++it) {
    if (rr <= (kCgTol * kCgTol) * bb) {
      done = true;
      break;
    }
    __syncthreads();  // p of every node written
    double pq = 0.0;
    for (int64_t w = threadIdx.x; w < work; w += blockDim.x) {
      const int64_t i = block_node<2>(nd, nd.blist[w >> 6], int(w & 63));
      if (i < 0) continue;
      q[i] = musl2d_apply<K>(nd, p, i);
      pq += p[i] * q[i];
    }
    pq = block_sum(pq, sh);
    const double alpha = rz / pq;
    double rzn = 0.0, rrn = 0.0;
    for (int64_t w = threadIdx.x; w < work; w += blockDim.x) {
      const int64_t i = block_node<2>(nd, nd.blist[w >> 6], int(w & 63));
      if (i < 0) continue;
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      const double z = r[i] / musl2d_diag<K>(nd, i);
      rzn += r[i] * z;
      rrn += r[i] * r[i];
    }
    rzn = block_sum(rzn, sh);
    rrn = block_sum(rrn, sh);
    const double beta = rzn / rz;
    rz = rzn;
    rr = rrn;
    __syncthreads();  // every thread has finished reading p of the SpMV above
    for (int64_t w = threadIdx.x; w < work; w += blockDim.x) {
      const int64_t i = block_node<2>(nd, nd.blist[w >> 6], int(w & 63));
      if (i < 0) continue;
      p[i] = r[i] / musl2d_diag<K>(nd, i) + beta * p[i];
    }
  }
  if (!done && !(rr <= (kCgTol * kCgTol) * bb) && threadIdx.x == 0) atomicOr(status, ST_SOLVER);
}

// gv = v0 + dv; node outputs of the 2D MUSL where m > 0
static __global__ void __launch_bounds__(256) musl2d_node_kernel(NodeP nd, CgP cg, double dt, double alpha) {
  const int64_t Nn = nd.nodeCount;
  const int64_t work = int64_t(*nd.bcount) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = block_node<2>(nd, nd.blist[w >> 6], int(w & 63));
    if (i < 0) continue;
    const bool live = nd.m[i] > 0.0;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const double v0 = cg.x[a][i], gv = v0 + cg.x[2 + a][i];
      nd.dv[a * Nn + i] = live ? gv - alpha * v0 : 0.0;
      nd.vdt[a * Nn + i] = live ? gv * dt : 0.0;
      nd.vg[a * Nn + i] = live ? gv * dt : 0.0;
    }
  }
}

}  // namespace jmpm
