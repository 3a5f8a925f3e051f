// mpm_bspline.cuh -- the quadratic and cubic B-spline bases
// (QuadBsplineBasis / CubicBsplineBasis, Basis.jl:374-820, Bsplines.jl:18-172).
//
// A particle's support is K consecutive nodes per axis (K = 3 quadratic,
// K = 4 cubic), chosen as the reference chooses them, with the 1D spline of
// each node typed by its position on the axis (first/last, second, second
// last, interior).  Kernels keep the K values and derivatives per axis
// (BsAxis) and walk the K^D tensor product in the reference's i, j(, k) order
// without storing it.  Weights are FP64 for both particle precisions and the
// node arrays are read in FP64.  As written in the reference: the 3D
// quadratic basis measures the particle from the origin (numx = xp*dxI), and
// both bases measure y and z from (id-1)*dy, (id-1)*dz rather than from the
// grid's minimum.
#pragma once

#include "mpm_kernels.cuh"

namespace jmpm {

template <int K>
struct BsAxis {
  int64_t first;    // 0-based index of the first support node on this axis
  double N[K];      // 1D values
  double G[K];      // 1D derivatives along the axis: dN/dr x dxI
};

// Bsplines.jl:18-80 (t = 1..4)
__device__ __forceinline__ void quad_bs(int t, double r, double& N, double& dN) {
  N = 0.0;
  dN = 0.0;
  if (t == 1) {
    if (r < -1.5 || r > 1.5) return;
    if (r >= -1.5 && r <= -0.5) { N = 0.5 * r * r + 1.5 * r + 1.125; dN = r + 1.5; }
    else if (r <= 0.) { N = 1. + r; dN = 1.; }
    else if (r <= 0.5) { N = 1. - r; dN = -1.; }
    else { N = 0.5 * r * r - 1.5 * r + 1.125; dN = r - 1.5; }
  } else if (t == 2) {
    if (r < -1.0 || r > 1.5) return;
    if (r >= -1. && r <= -0.5) { N = 1. + r; dN = 1.; }
    else if (r <= 0.5) { N = -r * r + 0.75; dN = -2 * r; }
    else { N = 0.5 * r * r - 1.5 * r + 1.125; dN = r - 1.5; }
  } else if (t == 3) {
    if (r < -1.5 || r > 1.5) return;
    if (r >= -1.5 && r <= -0.5) { N = 0.5 * r * r + 1.5 * r + 1.125; dN = r + 1.5; }
    else if (r <= 0.5) { N = -r * r + 0.75; dN = -2 * r; }
    else { N = 0.5 * r * r - 1.5 * r + 1.125; dN = r - 1.5; }
  } else {
    if (r < -1.5 || r > 1.) return;
    if (r >= -1.5 && r <= -0.5) { N = 0.5 * r * r + 1.5 * r + 1.125; dN = r + 1.5; }
    else if (r <= 0.5) { N = -r * r + 0.75; dN = -2 * r; }
    else { N = 1. - r; dN = -1.; }
  }
}

// Bsplines.jl:86-172 (t = 1..4; type 4 keeps the reference's 0.6666666667)
__device__ __forceinline__ void cubic_bs(int t, double r, double& N, double& dN) {
  N = 0.0;
  dN = 0.0;
  const double r2 = r * r;
  const double c6 = 0.16666666666666666, c3 = 0.3333333333333333, t3 = 0.6666666666666666;
  const double f3 = 1.3333333333333333;
  if (t == 1) {
    if (r < -2. || r > 2.) return;
    if (r >= -2.0 && r <= -1.0) { N = c6 * r * r2 + r2 + 2 * r + f3; dN = 0.5 * r2 + 2 * r + 2.; }
    else if (-1 <= r && r <= 0.) { N = -c6 * r * r2 + r + 1; dN = -0.5 * r2 + 1.; }
    else if (0 <= r && r <= 1.0) { N = c6 * r * r2 - r + 1; dN = 0.5 * r2 - 1.0; }
    else { N = -c6 * r * r2 + r2 - 2 * r + f3; dN = -0.5 * r2 + 2 * r - 2.; }
  } else if (t == 2) {
    if (r < -1. || r > 2.) return;
    if (r >= -1.0 && r <= 0.) { N = -c3 * r * r2 - r2 + t3; dN = -r2 - 2 * r; }
    else if (0. <= r && r <= 1.) { N = 0.5 * r * r2 - r2 + t3; dN = 1.5 * r2 - 2 * r; }
    else if (1 <= r && r <= 2.0) { N = -c6 * r * r2 + r2 - 2 * r + f3; dN = -0.5 * r2 + 2 * r - 2; }
  } else if (t == 3) {
    if (r < -2. || r > 2.) return;
    if (r >= -2.0 && r <= -1.0) { N = c6 * r * r2 + r2 + 2 * r + f3; dN = 0.5 * r2 + 2 * r + 2; }
    else if (-1. <= r && r <= 0.) { N = -0.5 * r * r2 - r2 + t3; dN = -1.5 * r2 - 2 * r; }
    else if (0 <= r && r <= 1.0) { N = 0.5 * r * r2 - r2 + t3; dN = 1.5 * r2 - 2 * r; }
    else if (1. <= r && r <= 2.0) { N = -c6 * r * r2 + r2 - 2 * r + f3; dN = -0.5 * r2 + 2 * r - 2; }
  } else {
    if (r < -2. || r > 1.) return;
    if (r >= -2.0 && r <= -1.0) { N = c6 * r * r2 + r2 + 2 * r + f3; dN = 0.5 * r2 + 2 * r + 2; }
    else if (-1. <= r && r <= 0.) { N = -0.5 * r * r2 - r2 + t3; dN = -1.5 * r2 - 2 * r; }
    else if (0 <= r && r <= 1.0) { N = c3 * r * r2 - r2 + 0.6666666667; dN = r2 - 2 * r; }
  }
}

// Support of a particle at x: per axis the first node and the K 1D values;
// false if its cell lies outside the grid.  The distances that select
// nodes and spline pieces are formed with explicit rounding so that they
// match the reference's to the bit.
template <int D, int K>
__device__ __forceinline__ bool bs_axes(const GridP& g, const double* x, BsAxis<K>* ax) {
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int64_t nn = g.nn[a];
    const double num = (K == 3 && D == 3) ? __dmul_rn(x[a], g.dxI[a]) : __dmul_rn(__dsub_rn(x[a], g.xmin[a]), g.dxI[a]);
    const double rem = __dsub_rn(num, floor(num));
    const double fb = floor(__dadd_rn(num, 1.0));
    if (!(fb >= 1.0) || !(fb <= double(nn - 1))) return false;
    const int64_t ib = int64_t(fb);
    int64_t f1;
    if (K == 3) f1 = ib == 1 ? ib : (ib == nn - 1 ? ib - 1 : (rem < 0.5 ? ib - 1 : ib));
    else f1 = ib == 1 ? 1 : (ib == nn - 1 ? ib - 2 : ib - 1);
    ax[a].first = f1 - 1;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int64_t id = f1 + i;
      const double r = a == 0 ? __dmul_rn(__dsub_rn(x[0], g.coord[0][id - 1]), g.dxI[0])
                              : __dmul_rn(__dsub_rn(x[a], __dmul_rn(double(id - 1), g.dx[a])), g.dxI[a]);
      const int t = (id == 1 || id == nn) ? 1 : (id == 2 ? 2 : (id == nn - 1 ? 4 : 3));
      double dNr;
      if (K == 3) quad_bs(t, r, ax[a].N[i], dNr);
      else cubic_bs(t, r, ax[a].N[i], dNr);
      ax[a].G[i] = dNr * g.dxI[a];
    }
  }
  return true;
}

// node index, value and gradient of support entry (i, j, k): N = Nx Ny (Nz),
// grad N = (Gx Ny (Nz), Nx Gy (Nz), Nx Ny Gz)
template <int D, int K>
__device__ __forceinline__ int64_t bs_entry(const GridP& g, const BsAxis<K>* ax, int i, int j, int k, double& N,
                                           double* dN) {
  if constexpr (D == 2) {
    N = ax[0].N[i] * ax[1].N[j];
    dN[0] = ax[0].G[i] * ax[1].N[j];
    dN[1] = ax[0].N[i] * ax[1].G[j];
    return (ax[0].first + i) + g.nx * (ax[1].first + j);
  } else {
    const double nxy = ax[0].N[i] * ax[1].N[j];
    N = nxy * ax[2].N[k];
    dN[0] = (ax[0].G[i] * ax[1].N[j]) * ax[2].N[k];
    dN[1] = (ax[0].N[i] * ax[1].G[j]) * ax[2].N[k];
    dN[2] = nxy * ax[2].G[k];
    return (ax[0].first + i) + g.nx * (ax[1].first + j) + g.nxy * (ax[2].first + k);
  }
}

// flag the node blocks of the support (nodes first .. first+K-1 per axis)
template <int D, int K>
__device__ __forceinline__ void bs_mark(const NodeP& nd, const BsAxis<K>* ax) {
  constexpr int B = BlockShape<D>::B;
  int64_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    lo[a] = ax[a].first / B;
    hi[a] = (ax[a].first + K - 1) / B;
  }
  for (int64_t bz = lo[2]; bz <= hi[2]; ++bz)
    for (int64_t by = lo[1]; by <= hi[1]; ++by)
      for (int64_t bx = lo[0]; bx <= hi[0]; ++bx) {
        const int64_t blk = bx + nd.nb[0] * (by + nd.nb[1] * bz);
        if (nd.bflag[blk] == 0u) nd.bflag[blk] = 1u;
      }
}

// ---- USL ---------------------------------------------------------------------
// P2G over the support (SolveExplicitSolidMechanics2D.jl:391-423): m, p0, f
// (+ body force), and the contact normals where the field has them.  In 3D the
// per-node work is factored along z: with Nxy = Nx Ny, the force of node
// (i, j, k) is f_a = Nz_k P_a(i,j) + Gz_k Q_a(i,j), where
// P_a = s_a0 Gx Ny + s_a1 Nx Gy (+ m g_a Nxy) and Q_a = s_a2 Nxy with s = -V sigma,
// and its mass m Nxy Nz_k -- about ten FP64 operations per node.
template <int D, class R, int K, bool GRAV>
__global__ void __launch_bounds__(256) bs_p2g_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy, double gz,
                                                     unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = double(*field<R>(pp, L::X + a, p));
  BsAxis<K> ax[D];
  if (!bs_axes<D, K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  if (nd.bflag) bs_mark<D, K>(nd, ax);
  const double m = double(*field<R>(pp, L::M, p)), V = double(*field<R>(pp, L::VOL, p));
  double v[D], ms[L::S], mg[D];
  const double grav[3] = {gx, gy, gz};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    v[a] = double(*field<R>(pp, L::V + a, p));
    mg[a] = m * grav[a];
  }
#pragma unroll
  for (int c = 0; c < L::S; ++c) ms[c] = -V * double(*field<R>(pp, L::SIG + c, p));
  const int64_t Nn = nd.nodeCount;
  const bool NRM = nd.nrm != nullptr;
  if constexpr (D == 2) {
#pragma unroll 1
    for (int i = 0; i < K; ++i)
#pragma unroll
      for (int j = 0; j < K; ++j) {
        double N, dN[2];
        const int64_t n = bs_entry<2, K>(g, ax, i, j, 0, N, dN);
        const double Nm = N * m;
        atomicAdd(nd.m + n, Nm);
#pragma unroll
        for (int a = 0; a < 2; ++a) atomicAdd(nd.p0 + a * Nn + n, Nm * v[a]);
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          double fa = ms[sym<2>(a, 0)] * dN[0] + ms[sym<2>(a, 1)] * dN[1];
          if (GRAV) fa += mg[a] * N;
          atomicAdd(nd.f + a * Nn + n, fa);
        }
        if (NRM)
#pragma unroll
          for (int a = 0; a < 2; ++a) atomicAdd(nd.nrm + a * Nn + n, m * dN[a]);
      }
  } else {
    double mNz[K];
#pragma unroll
    for (int k = 0; k < K; ++k) mNz[k] = m * ax[2].N[k];
    // outer (i, j) loops rolled: unrolling them lets the compiler hold every
    // node's values at once and spill
#pragma unroll 1
    for (int i = 0; i < K; ++i)
#pragma unroll 1
      for (int j = 0; j < K; ++j) {
        const double Nxy = ax[0].N[i] * ax[1].N[j];
        const double GxNy = ax[0].G[i] * ax[1].N[j];
        const double NxGy = ax[0].N[i] * ax[1].G[j];
        double P[3], Q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          P[a] = ms[sym<3>(a, 0)] * GxNy + ms[sym<3>(a, 1)] * NxGy;
          if (GRAV) P[a] += mg[a] * Nxy;
          Q[a] = ms[sym<3>(a, 2)] * Nxy;
        }
        const int64_t nij = (ax[0].first + i) + g.nx * (ax[1].first + j) + g.nxy * ax[2].first;
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const int64_t n = nij + g.nxy * k;
          const double Nm = Nxy * mNz[k];
          atomicAdd(nd.m + n, Nm);
#pragma unroll
          for (int a = 0; a < 3; ++a) atomicAdd(nd.p0 + a * Nn + n, Nm * v[a]);
#pragma unroll
          for (int a = 0; a < 3; ++a) atomicAdd(nd.f + a * Nn + n, P[a] * ax[2].N[k] + Q[a] * ax[2].G[k]);
          if (NRM) {
            // m grad N (SolveExplicitFEMP3DContact.jl)
            atomicAdd(nd.nrm + n, GxNy * mNz[k]);
            atomicAdd(nd.nrm + Nn + n, NxGy * mNz[k]);
            atomicAdd(nd.nrm + 2 * Nn + n, (m * Nxy) * ax[2].G[k]);
          }
        }
      }
  }
}

// G2P over the support (:485-532): v += N dv, x += N vdt, L dt += vdt (x) grad N,
// then the shared kinematics and constitutive update.  The sums are factored
// along the last axis: per (i(, j)) the node values are first contracted with
// that axis's N and G (Z0 = sum Nz vdt, Z1 = sum Gz vdt, W = sum Nz dv), then
// x += Nxy Z0, v += Nxy W, L dt += (Gx Ny Z0, Nx Gy Z0, Nxy Z1).
template <int D, class R, int K, int MAT>
__global__ void __launch_bounds__(256) bs_g2p_kernel(GridP g, NodeP nd, PartP pp, MatParams mp, unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D], v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    x[a] = double(*field<R>(pp, L::X + a, p));
    v[a] = double(*field<R>(pp, L::V + a, p));
  }
  BsAxis<K> ax[D];
  if (!bs_axes<D, K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  const int64_t Nn = nd.nodeCount;
  double Ld[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) Ld[a][b] = 0.0;
  constexpr int NO = D == 3 ? K * K : K;  // outer entries (i, j) in 3D, i in 2D
#pragma unroll 1
  for (int o = 0; o < NO; ++o) {
    const int i = D == 3 ? o / K : o, j = D == 3 ? o % K : 0;
    // outer weights: value and the in-plane gradient factors
    const double No = D == 3 ? ax[0].N[i] * ax[1].N[j] : ax[0].N[i];
    const double Go0 = D == 3 ? ax[0].G[i] * ax[1].N[j] : ax[0].G[i];
    const double Go1 = D == 3 ? ax[0].N[i] * ax[1].G[j] : 0.0;
    const BsAxis<K>& in = ax[D - 1];
    const int64_t no = D == 3 ? (ax[0].first + i) + g.nx * (ax[1].first + j) + g.nxy * in.first
                              : (ax[0].first + i) + g.nx * in.first;
    const int64_t stride = D == 3 ? g.nxy : g.nx;
    double Z0[D], Z1[D], W[D];
#pragma unroll
    for (int a = 0; a < D; ++a) Z0[a] = Z1[a] = W[a] = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int64_t n = no + stride * k;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const double vd = __ldg(nd.vdt + a * Nn + n);
        Z0[a] += in.N[k] * vd;
        Z1[a] += in.G[k] * vd;
        W[a] += in.N[k] * __ldg(nd.dv + a * Nn + n);
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      x[a] += No * Z0[a];
      v[a] += No * W[a];
      Ld[a][0] += Go0 * Z0[a];
      if (D == 3) Ld[a][1] += Go1 * Z0[a];
      Ld[a][D - 1] += No * Z1[a];
    }
  }
  R Ldt[D][D];
  bool fin = true;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    *field<R>(pp, L::X + a, p) = R(x[a]);
    *field<R>(pp, L::V + a, p) = R(v[a]);
    fin &= finite_bits(x[a]) & finite_bits(v[a]);
#pragma unroll
    for (int b = 0; b < D; ++b) Ldt[a][b] = R(Ld[a][b]);
  }
  kinematics_stress<D, R, MAT>(pp, p, Ldt, mp, fin, status);
}

// ---- MUSL (FP64 particles) ------------------------------------------------------
// G2P-1: v = alpha v + sum N dv; P2: P2G-2 of the new velocity into p2 (3D)
template <int D, int K, bool P2>
__global__ void __launch_bounds__(256) bs_musl_g2p1_kernel(GridP g, NodeP nd, PartP pp, double alpha,
                                                           unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<double>(pp, L::X + a, p);
  BsAxis<K> ax[D];
  if (!bs_axes<D, K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  const int64_t Nn = nd.nodeCount;
  double vacc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) vacc[a] = 0.0;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j)
      for (int k = 0; k < (D == 3 ? K : 1); ++k) {
        double N, dN[D];
        const int64_t n = bs_entry<D, K>(g, ax, i, j, k, N, dN);
#pragma unroll
        for (int a = 0; a < D; ++a) vacc[a] += N * __ldg(nd.dv + a * Nn + n);
      }
  double v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    v[a] = alpha * *field<double>(pp, L::V + a, p) + vacc[a];
    *field<double>(pp, L::V + a, p) = v[a];
  }
  if (P2) {
    const double mp = *field<double>(pp, L::M, p);
    for (int i = 0; i < K; ++i)
      for (int j = 0; j < K; ++j)
        for (int k = 0; k < (D == 3 ? K : 1); ++k) {
          double N, dN[D];
          const int64_t n = bs_entry<D, K>(g, ax, i, j, k, N, dN);
          const double Nm = N * mp;
#pragma unroll
          for (int a = 0; a < D; ++a) atomicAdd(nd.p2 + a * Nn + n, Nm * v[a]);
        }
  }
}

// G2P-2: x += sum N vdt, velocity gradient from vg (transposed in 3D), kinematics
template <int D, int K, int MAT, bool TRANSPOSED>
__global__ void __launch_bounds__(256) bs_musl_g2p2_kernel(GridP g, NodeP nd, PartP pp, MatParams mp,
                                                           unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<double>(pp, L::X + a, p);
  BsAxis<K> ax[D];
  if (!bs_axes<D, K>(g, x, ax)) return;  // reported by G2P-1
  const int64_t Nn = nd.nodeCount;
  double Ldt[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) Ldt[a][b] = 0.0;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j)
      for (int k = 0; k < (D == 3 ? K : 1); ++k) {
        double N, dN[D], vg[D];
        const int64_t n = bs_entry<D, K>(g, ax, i, j, k, N, dN);
#pragma unroll
        for (int a = 0; a < D; ++a) {
          x[a] += N * __ldg(nd.vdt + a * Nn + n);
          vg[a] = __ldg(nd.vg + a * Nn + n);
        }
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
          for (int b = 0; b < D; ++b) Ldt[a][b] += TRANSPOSED ? dN[a] * vg[b] : vg[a] * dN[b];
      }
  bool fin = true;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    *field<double>(pp, L::X + a, p) = x[a];
    fin &= finite_bits(x[a]) & finite_bits(*field<double>(pp, L::V + a, p));
  }
  kinematics_stress<D, double, MAT>(pp, p, Ldt, mp, fin, status);
}

// 2D: P2G plus the consistent mass stencil of the support: mc[o * Nn + n_a] +=
// (N_a m) N_b, o = (dx + K - 1) + (2K - 1)(dy + K - 1) the offset of node b from a
template <int K, bool GRAV>
__global__ void __launch_bounds__(256) bs_musl2d_p2g_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy,
                                                            unsigned* status) {
  using L = Layout<2>;
  constexpr int W = 2 * K - 1;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[2] = {*field<double>(pp, L::X, p), *field<double>(pp, L::X + 1, p)};
  BsAxis<K> ax[2];
  if (!bs_axes<2, K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  if (nd.bflag) bs_mark<2, K>(nd, ax);
  const double m = *field<double>(pp, L::M, p), V = *field<double>(pp, L::VOL, p);
  double mv[2], ms[3];
  for (int a = 0; a < 2; ++a) mv[a] = m * *field<double>(pp, L::V + a, p);
  for (int c = 0; c < 3; ++c) ms[c] = -V * *field<double>(pp, L::SIG + c, p);
  const int64_t Nn = nd.nodeCount;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j) {
      double N, dN[2];
      const int64_t n = bs_entry<2, K>(g, ax, i, j, 0, N, dN);
      const double Nim = N * m;
      atomicAdd(nd.m + n, Nim);
      for (int a = 0; a < 2; ++a) atomicAdd(nd.p0 + a * Nn + n, N * mv[a]);
      for (int a = 0; a < 2; ++a) {
        double fa = ms[sym<2>(a, 0)] * dN[0] + ms[sym<2>(a, 1)] * dN[1];
        if (GRAV) fa += (m * (a == 0 ? gx : gy)) * N;
        atomicAdd(nd.f + a * Nn + n, fa);
      }
      for (int i2 = 0; i2 < K; ++i2)
        for (int j2 = 0; j2 < K; ++j2) {
          const double Nb = ax[0].N[i2] * ax[1].N[j2];
          const int o = (i2 - i + K - 1) + W * (j2 - j + K - 1);
          atomicAdd(nd.mc + int64_t(o) * Nn + n, Nim * Nb);
        }
    }
}

}  // namespace jmpm
