// mpm_kernels.cuh -- kernels of one USL step (SolveExplicitSolidMechanics2D.jl:381-534,
// 3D lifted the same way) for D = 2, 3 and particle precision R = double | float.
//
//   p2g        P2G: nodal mass, momentum and force (:391-423), FP64 atomics at L2
//   grid       grid update + Dirichlet mask (:429-442), and the nodal velocities
//              the G2P needs, computed once per node instead of per particle
//   g2p        G2P + velocity gradient + F/J/volume + update_stress! (:485-533)
//              fused in one per-particle pass
//   energies   EnergiesFix sums (Fix.jl:248-270)
#pragma once

#include <climits>
#include <type_traits>

#include "mpm_common.cuh"
#include "mpm_dw.cuh"
#include "mpm_sparse.cuh"
#include "../../include/jump_mpm.h"

namespace jmpm {

template <class R>
__device__ __forceinline__ R* field(const PartP& pp, int f, int64_t p) {
  return static_cast<R*>(pp.base) + int64_t(f) * pp.pitch + p;
}

// ---------------------------------------------------------------------------
// P2G values of particle p (SolveExplicitSolidMechanics2D.jl:391-423) at its
// 2^D stencil corners, handed to put(k, val) (k: corner index, bit 0 +x,
// bit 1 +y, bit 2 +z; val: m N, m N v (D), f (D) and, in contact mode, the
// normal sum m grad N (D)) on the lanes that issue them, and the node blocks
// of the stencil flagged.  All lanes in `mask` call it together with t
// consecutive across the warp; lanes with ok == false add nothing.
// WARP_SUM: lanes with the same base node first add their values by a
// shuffle reduction over the group __match_any_sync finds, and only the
// group's lowest lane calls put; otherwise every lane with ok calls put.
template <int D, class R, bool GRAV, bool WARP_SUM, class Put>
__device__ __forceinline__ void p2g_corner_values(const GridP& g, const NodeP& nd, const PartP& pp, int64_t p,
                                                  bool ok, const Hat<D, R>& h, unsigned mask, double gx,
                                                  double gy, double gz, Put&& put) {
  using L = Layout<D>;
  constexpr int NV = 1 + 3 * D;  // per node: m, p0 (D), f (D), normal (D, contact mode)
  const bool NRM = nd.nrm != nullptr;
  Corners<D, R> cr;
  R m = R(0), V = R(0), v[D], ms[L::S];
  if (ok) {
    if (D == 2) corners<D, R>(g, h, cr);  // in 3D N and grad N are formed per z pair below
    m = *field<R>(pp, L::M, p);
    V = *field<R>(pp, L::VOL, p);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = ok ? *field<R>(pp, L::V + a, p) : R(0);
#pragma unroll
  for (int c = 0; c < L::S; ++c) ms[c] = ok ? -V * *field<R>(pp, L::SIG + c, p) : R(0);  // -V sigma
  R mg[3] = {R(0), R(0), R(0)};
  if (GRAV) {
    mg[0] = m * R(gx);
    mg[1] = m * R(gy);
    if (D == 3) mg[2] = m * R(gz);
  }
  // WARP_SUM: the lanes with the same base node, wherever they sit in the warp
  // (__match_any_sync), add their contributions by a tree reduction over the
  // group's members in lane order, and only the group's lowest lane issues
  // them.  At level l the member of group rank r (r a multiple of 2^(l+1))
  // adds the partial sum held by the member of rank r + 2^l, whose lane is
  // src[l]; take bit l says whether this lane has such a partner.
  const int lane = threadIdx.x & 31;
  bool head = true;
  int levels = 0, src[5];
  unsigned take = 0;
  if (WARP_SUM) {
    long long key = ok ? (long long)(int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + (D == 3 ? g.nxy * int64_t(h.c[D - 1]) : 0))
                       : -1ll - lane;
    const unsigned grp = __match_any_sync(mask, key);
    const int r = __popc(grp & ((1u << lane) - 1u));  // rank in the group
    head = r == 0;
    const unsigned nmax = __reduce_max_sync(mask, unsigned(__popc(grp)));
    while ((1u << levels) < nmax) ++levels;
    unsigned after = grp & ~((2u << lane) - 1u);  // members of higher rank, lowest bit = rank r + 1
#pragma unroll
    for (int l = 0; l < 5; ++l) {
      src[l] = after ? __ffs(after) - 1 : lane;
      if (after && (r & ((2 << l) - 1)) == 0) take |= 1u << l;
      if (l < 4) {  // drop 2^l members: the lowest bit becomes rank r + 2^(l+1)
#pragma unroll
        for (int s = 0; s < (1 << l); ++s) after &= after - 1u;
      }
    }
  }
  auto emit = [&](int k, R* val) {
    if (WARP_SUM) {
      const int nv = NRM ? NV : 1 + 2 * D;
#pragma unroll
      for (int l = 0; l < 5; ++l) {
        if (l >= levels) break;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          if (q >= nv) break;
          R o = __shfl_sync(mask, val[q], src[l]);
          if ((take >> l) & 1u) val[q] += o;
        }
      }
    }
    if (ok && head) put(k, val);
  };
  if (ok && head && nd.bflag) mark_blocks<D>(nd, h.c);
  if constexpr (D == 3) {
    // factored along z: per (x, y) corner pair the force coefficients
    // P_a = s_a0 Gx Ny + s_a1 Nx Gy (+ m g_a Nx Ny) and Q_a = s_a2 Nx Ny (s = -V sigma)
    // give f_a = Nz P_a + Gz Q_a at both z corners.
    // FAST (every lane of the warp strictly inside its cell, hat_interior): the
    // gradients are -dxI and +dxI, so s is scaled by dxI
    // once per particle (c_ab = s_ab dxI_b), P_a = +-c_a0 Ny +- c_a1 Nx and
    // Q_a = c_a2 Nx Ny, and each corner's force is the one FMA Nz P_a +- Q_a.
    // The branch is uniform over the warp, so the shuffles of emit stay in step.
    const R mNz[2] = {m * h.Nl[2], m * h.Nh[2]};
    auto corners3 = [&](auto fast_c) {
      constexpr bool FAST = decltype(fast_c)::value;
      R cs[3][3];
      if constexpr (FAST) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) cs[a][b] = ms[sym<3>(a, b)] * h.gh[b];  // gh = +dxI here
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int bx = q & 1, by = q >> 1;
        const R Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1];
        const R Gx = bx ? h.gh[0] : h.gl[0], Gy = by ? h.gh[1] : h.gl[1];
        const R Nxy = Nx * Ny;
        R P[3], Q[3], GxNy = R(0), NxGy = R(0);
        if constexpr (FAST) {
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            P[a] = (bx ? cs[a][0] : -cs[a][0]) * Ny + (by ? cs[a][1] : -cs[a][1]) * Nx;
            if (GRAV) P[a] += mg[a] * Nxy;
            Q[a] = cs[a][2] * Nxy;
          }
          if (NRM) {  // the contact normals still take the gradient products
            GxNy = Gx * Ny;
            NxGy = Nx * Gy;
          }
        } else {
          GxNy = Gx * Ny;
          NxGy = Nx * Gy;
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            P[a] = ms[sym<3>(a, 0)] * GxNy + ms[sym<3>(a, 1)] * NxGy;
            if (GRAV) P[a] += mg[a] * Nxy;
            Q[a] = ms[sym<3>(a, 2)] * Nxy;
          }
        }
#pragma unroll
        for (int bz = 0; bz < 2; ++bz) {
          const R Nz = bz ? h.Nh[2] : h.Nl[2], Gz = bz ? h.gh[2] : h.gl[2];
          R val[NV];
          const R Nm = Nxy * mNz[bz];
          val[0] = Nm;
#pragma unroll
          for (int a = 0; a < 3; ++a) val[1 + a] = Nm * v[a];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            if constexpr (FAST) val[4 + a] = P[a] * Nz + (bz ? Q[a] : -Q[a]);
            else val[4 + a] = P[a] * Nz + Q[a] * Gz;
          }
          // normals of the contact correction: sum m_p grad N (SolveExplicitFEMP3DContact.jl)
          if (NRM) {
            val[7] = GxNy * mNz[bz];
            val[8] = NxGy * mNz[bz];
            val[9] = (m * Nxy) * Gz;
          }
          emit(q + 4 * bz, val);
        }
      }
    };
    if (__all_sync(mask, hat_interior<3, R>(h))) corners3(std::true_type{});
    else corners3(std::false_type{});
  } else {
#pragma unroll
    for (int k = 0; k < (1 << D); ++k) {
      R val[NV];
      R N = ok ? cr.N[k] : R(0);
      R Nm = N * m;
      val[0] = Nm;
#pragma unroll
      for (int a = 0; a < D; ++a) val[1 + a] = Nm * v[a];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        R fa = ok ? ms[sym<D>(a, 0)] * cr.dN[k][0] : R(0);
#pragma unroll
        for (int j = 1; j < D; ++j) fa += ok ? ms[sym<D>(a, j)] * cr.dN[k][j] : R(0);
        if (GRAV) fa += mg[a] * N;
        val[1 + D + a] = fa;
      }
      // normals of the contact correction: sum m_p grad N (SolveExplicitFEMP2DContact.jl:237)
      if (NRM)
#pragma unroll
        for (int a = 0; a < D; ++a) val[1 + 2 * D + a] = ok ? m * cr.dN[k][a] : R(0);
      emit(k, val);
    }
  }
}

// node value q of node n: m (q = 0), p0 (1 .. D), f (D+1 .. 2D), normal (2D+1 .. 3D)
template <int D>
__device__ __forceinline__ double* node_value(const NodeP& nd, int q, int64_t n) {
  const int64_t Nn = nd.nodeCount;
  if (q == 0) return nd.m + n;
  if (q <= D) return nd.p0 + (q - 1) * Nn + n;
  if (q <= 2 * D) return nd.f + (q - 1 - D) * Nn + n;
  return nd.nrm + (q - 1 - 2 * D) * Nn + n;
}

// FP64 atomics of one corner's values at global node n
template <int D, class R>
__device__ __forceinline__ void add_node_values(const NodeP& nd, int64_t n, const R* val) {
  const int64_t Nn = nd.nodeCount;
  atomicAdd(nd.m + n, to_f64(val[0]));
#pragma unroll
  for (int a = 0; a < D; ++a) atomicAdd(nd.p0 + a * Nn + n, to_f64(val[1 + a]));
#pragma unroll
  for (int a = 0; a < D; ++a) atomicAdd(nd.f + a * Nn + n, to_f64(val[1 + D + a]));
  if (nd.nrm)
#pragma unroll
    for (int a = 0; a < D; ++a) atomicAdd(nd.nrm + a * Nn + n, to_f64(val[1 + 2 * D + a]));
}

// global node index of corner k of base node `base`
template <int D>
__device__ __forceinline__ int64_t corner_node(const GridP& g, int64_t base, int k) {
  return base + (k & 1) + g.nx * ((k >> 1) & 1) + (D == 3 ? g.nxy * (k >> 2) : 0);
}

// P2G of particle pp.begin + t with FP64 atomics at L2: one per lane and node
// value (MPM_P2G_ATOMIC) or one per group of lanes sharing a base node
// (WARP_SUM, MPM_P2G_WARP).  All 32 lanes of a warp call it together
// (t consecutive across the warp); lanes with t >= pp.count do nothing.
template <int D, class R, bool GRAV, bool WARP_SUM = (sizeof(R) == 4)>
__device__ __forceinline__ void p2g_particle(const GridP& g, const NodeP& nd, const PartP& pp, int64_t t,
                                             double gx, double gy, double gz, unsigned* status) {
  using L = Layout<D>;
  // lanes of this warp holding a particle (a contiguous low range)
  const unsigned mask = __ballot_sync(0xffffffffu, t < pp.count);
  if (t >= pp.count) return;
  int64_t p = pp.begin + t;
  R x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<R>(pp, L::X + a, p);
  Hat<D, R> h{};  // zeros on lanes whose cell lies outside (they add nothing)
  const bool ok = hat<D, R>(g, x, h);
  if (!ok) {
    hat_put<D, R>(pp, p, false, h);  // the G2P of this step skips it too
    atomicOr(status, ST_OUT_OF_GRID);
    if (!WARP_SUM) return;
  }
  const int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + (D == 3 ? g.nxy * int64_t(h.c[D - 1]) : 0);
  p2g_corner_values<D, R, GRAV, WARP_SUM>(g, nd, pp, p, ok, h, mask, gx, gy, gz, [&](int k, const R* val) {
    add_node_values<D, R>(nd, corner_node<D>(g, base, k), val);
  });
  if (ok) hat_put<D, R>(pp, p, true, h);  // for the G2P of this step
}

// three CTAs of 256 threads per SM (at most 80 registers): the FP64 P2G's
// latency is hidden better than at two CTAs of 128 registers, despite ~70 B
// of spills (0.1655 -> 0.1595 ms on the Taylor bar at 128 threads)
template <int D, class R, bool GRAV, bool WARP_SUM = (sizeof(R) == 4)>
__global__ void __launch_bounds__(256, 3) p2g_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy,
                                                  double gz, unsigned* status) {
  p2g_particle<D, R, GRAV, WARP_SUM>(g, nd, pp, int64_t(blockIdx.x) * blockDim.x + threadIdx.x, gx, gy, gz,
                                     status);
}

// ---------------------------------------------------------------------------
// P2G staged in a shared-memory grid tile (MPM_P2G_TILE, MPM_P2G_TILE_WARP).
// The CTA finds the box of nodes its particles' stencils cover (min/max base
// cell per axis); if the box holds at most `cap` nodes, the particles add their
// corner values into an FP64 tile of the box in shared memory (shared atomics;
// after the warp-segmented sum under WARP_SUM) and the CTA then adds each
// non-zero tile value to its node with one global FP64 atomic, so a node gets
// one L2 atomic per value and CTA instead of one per particle.  A CTA whose box
// is larger (particles far apart, as without the cell sort) falls back to the
// per-particle global atomics.  Adding a zero is skipped: node accumulators
// start at +0 and x + 0 == x, so the sums are those of the other strategies up
// to summation order.  Dynamic shared memory: cap * (1 + 2D, or 1 + 3D in
// contact mode) doubles.  blockDim.x is a multiple of 32 and at most 256.
template <int D, class R, bool GRAV, bool WARP_SUM>
__global__ void __launch_bounds__(256) p2g_tile_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy,
                                                       double gz, unsigned* status, int cap) {
  using L = Layout<D>;
  extern __shared__ double tile[];
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t p = pp.begin + t;
  Hat<D, R> h{};
  bool ok = false;
  if (t < pp.count) {
    R x[D];
#pragma unroll
    for (int a = 0; a < D; ++a) x[a] = *field<R>(pp, L::X + a, p);
    ok = hat<D, R>(g, x, h);
    hat_put<D, R>(pp, p, ok, h);
    if (!ok) atomicOr(status, ST_OUT_OF_GRID);
  }
  int lo[3], hi[3];
  cta_cell_box<D>(ok, h.c, lo, hi);
  if (lo[0] > hi[0]) return;  // no particle of this CTA inside the grid (uniform)
  const int e0 = hi[0] - lo[0] + 2, e1 = hi[1] - lo[1] + 2, e2 = D == 3 ? hi[2] - lo[2] + 2 : 1;
  // box volume in 64 bits: a spread-out CTA can cover most of a large grid
  const int64_t vol64 = int64_t(e0) * e1 * e2;
  const bool use = vol64 <= int64_t(cap);  // uniform over the CTA
  const int vol = use ? int(vol64) : 0;
  const int nv = nd.nrm ? 1 + 3 * D : 1 + 2 * D;
  if (use) {
    for (int i = threadIdx.x; i < vol * nv; i += blockDim.x) tile[i] = 0.0;
    __syncthreads();
  }
  const int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + (D == 3 ? g.nxy * int64_t(h.c[D - 1]) : 0);
  const int lbase = use ? (h.c[0] - lo[0]) + e0 * ((h.c[1] - lo[1]) + (D == 3 ? e1 * (h.c[D - 1] - lo[D - 1]) : 0)) : 0;
  p2g_corner_values<D, R, GRAV, WARP_SUM>(g, nd, pp, p, ok, h, 0xffffffffu, gx, gy, gz, [&](int k, const R* val) {
    if (use) {
      // ok lanes only: lo <= c <= hi per axis, so 0 <= l < vol
      const int l = lbase + (k & 1) + e0 * ((k >> 1) & 1) + (D == 3 ? e0 * e1 * (k >> 2) : 0);
      for (int q = 0; q < nv; ++q) atomicAdd(tile + q * vol + l, to_f64(val[q]));
    } else {
      add_node_values<D, R>(nd, corner_node<D>(g, base, k), val);
    }
  });
  if (!use) return;  // uniform
  __syncthreads();
  for (int l = threadIdx.x; l < vol; l += blockDim.x) {
    const int ix = l % e0, iy = (l / e0) % e1, iz = l / (e0 * e1);
    const int64_t n = int64_t(lo[0] + ix) + g.nx * int64_t(lo[1] + iy) + (D == 3 ? g.nxy * int64_t(lo[2] + iz) : 0);
    for (int q = 0; q < nv; ++q) {
      const double s = tile[q * vol + l];
      if (s != 0.0) atomicAdd(node_value<D>(nd, q, n), s);
    }
  }
}

// ---------------------------------------------------------------------------
// Contact mode grid update: one field per body, system sums, and the
// multi-body correction at nodes two bodies share
// (SolveExplicitFEMP2DContact.jl:248-266, 305-387; SolveExplicitFEMP3DContact.jl:424-517).
template <int D, bool F32COPY>
__device__ __forceinline__ void contact_node(const ContactP& cp, int64_t i, double dt, double tol) {
  const int64_t Nn = cp.body[0].nodeCount;
  const unsigned fx = cp.body[0].fixed[i];
  double mb[kMaxContactBodies], v[kMaxContactBodies][D], v0[kMaxContactBodies][D];
  double mS = 0.0, pS[D];
#pragma unroll
  for (int a = 0; a < D; ++a) pS[a] = 0.0;
  int s1 = -1, s2 = -1;
#pragma unroll
  for (int b = 0; b < kMaxContactBodies; ++b) {
    if (b >= cp.nb) break;
    const NodeP& nd = cp.body[b];
    double m = nd.m[i];
    mb[b] = m;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double p0 = nd.p0[a * Nn + i];
      double p = __dadd_rn(p0, __dmul_rn(nd.f[a * Nn + i], dt));  // p = p0 + f*dt
      pS[a] += p;                                                // system momentum, before BCs
      v0[b][a] = p0;
      v[b][a] = p;
    }
    mS += m;
    if (m > 0.0) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        v0[b][a] = v0[b][a] / m;
        v[b][a] = v[b][a] / m;
      }
      if (s1 < 0) s1 = b;
      else if (s2 < 0) s2 = b;
    }
#pragma unroll
    for (int a = 0; a < D; ++a)
      if (fx & (1u << a)) {
        v0[b][a] = 0.0;
        v[b][a] = 0.0;
      }
  }
  if (s2 >= 0) {
    // common normal n = (n1 - n2)/|n1 - n2|; body 1 uses n, body 2 uses -n
    double n[D], nn = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      n[a] = cp.body[s1].nrm[a * Nn + i] - cp.body[s2].nrm[a * Nn + i];
      nn += n[a] * n[a];
    }
    nn = sqrt(nn);
#pragma unroll
    for (int a = 0; a < D; ++a) n[a] = n[a] / nn;
#pragma unroll
    for (int is = 0; is < 2; ++is) {
      const int s = is == 0 ? s1 : s2;
      double nI[D], dvv[D], D1 = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        nI[a] = is == 0 ? n[a] : -n[a];
        dvv[a] = v[s][a] - pS[a] / mS;
        D1 += dvv[a] * nI[a];
      }
      if (D1 > 0.0) {  // approaching
        // Coulomb branch; with no tangential slip (C1 == 0) the reference's
        // (muPrime/|C1|) is 0/0, whose limit is the normal-only update below
        if (D == 2 && cp.friction > 0.0 && (dvv[0] * nI[1] - dvv[1] * nI[0]) != 0.0) {
          double C1 = dvv[0] * nI[1] - dvv[1] * nI[0];
          double absC1 = fabs(C1);
          double mup = fmin(cp.friction, absC1 / D1);
          double t0 = nI[0] + (mup / absC1) * (nI[1] * C1);
          double t1 = nI[D - 1] + (mup / absC1) * (-nI[0] * C1);
          v[s][0] = v[s][0] - D1 * t0;
          v[s][D - 1] = v[s][D - 1] - D1 * t1;
        } else {
#pragma unroll
          for (int a = 0; a < D; ++a) v[s][a] = v[s][a] - D1 * nI[a];
        }
      }
    }
  }
#pragma unroll
  for (int b = 0; b < kMaxContactBodies; ++b) {
    if (b >= cp.nb) break;
    const NodeP& nd = cp.body[b];
    const bool live = mb[b] > tol;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double vd = live ? v[b][a] * dt : 0.0;
      double dd = live ? v[b][a] - v0[b][a] : 0.0;
      nd.vdt[a * Nn + i] = vd;
      nd.dv[a * Nn + i] = dd;
      if (F32COPY) {
        nd.vdt_f[a * Nn + i] = float(vd);
        nd.dv_f[a * Nn + i] = float(dd);
      }
    }
  }
}

template <int D, bool F32COPY>
__global__ void __launch_bounds__(256) contact_grid_kernel(NodeP nd, ContactP cp, double dt, double tol) {
  const int64_t work = int64_t(*nd.bcount) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    int64_t i = block_node<D>(nd, nd.blist[w >> 6], int(w & 63));
    if (i >= 0) contact_node<D, F32COPY>(cp, i, dt, tol);
  }
}

// ---------------------------------------------------------------------------
// Grid update (:429-442) + nodal velocities for G2P, for node i.
// Node data written earlier in the same kernel (the persistent batch kernel)
// must be read through L2 (CG); data from an earlier launch may use the
// read-only path.
template <bool CG, class T>
__device__ __forceinline__ T nload(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return __ldg(p);
}

// Rigid bodies after the grid update and its Dirichlet mask
// (SolveExplicitSolidMechanics2D.jl:448-479): for every rigid body marked at
// node i, in body order, both momenta become m v_rigid in the components where
// v_rigid is non-zero, or zero in every component for a fixed body.
template <int D>
__device__ __forceinline__ void rigid_override(const NodeP& nd, int64_t i, double m, double* p0, double* p) {
  unsigned bits = nd.rmask[i];
  while (bits) {
    const int k = __ffs(bits) - 1;
    bits &= bits - 1u;
    const double* rt = nd.rtab + 4 * k;
    const bool fixed = rt[0] != 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (fixed) {
        p0[a] = 0.0;
        p[a] = 0.0;
      } else if (rt[1 + a] != 0.0) {
        const double q = m * rt[1 + a];
        p0[a] = q;
        p[a] = q;
      }
    }
  }
}

template <int D, bool F32COPY, bool CG = false>
__device__ __forceinline__ void grid_node(const NodeP& nd, int64_t i, double dt, double tol) {
  const int64_t Nn = nd.nodeCount;
  double m = CG ? __ldcg(nd.m + i) : nd.m[i];
  if (!(m > tol)) {
    // empty or near-empty node: G2P skips it (:510); no FP64 work here
#pragma unroll
    for (int a = 0; a < D; ++a) {
      nd.vdt[a * Nn + i] = 0.0;
      nd.dv[a * Nn + i] = 0.0;
      if (F32COPY && !nd.nf4) {
        nd.vdt_f[a * Nn + i] = 0.f;
        nd.dv_f[a * Nn + i] = 0.f;
      }
    }
    if (F32COPY && nd.nf4) {
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      nd.nf4[(D == 2 ? 1 : 2) * i] = z;
      if (D == 3) nd.nf4[2 * i + 1] = z;
    }
    if (D == 3 && !F32COPY && nd.dw4) put_node_dw(nd.dw4, i, nullptr, nullptr);
    return;
  }
  const unsigned fx = nd.fixed[i];
  double vdt[D], dv[D], p0[D], p[D];
  double invM = 1.0 / m;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    p0[a] = CG ? __ldcg(nd.p0 + a * Nn + i) : nd.p0[a * Nn + i];
    double fa = CG ? __ldcg(nd.f + a * Nn + i) : nd.f[a * Nn + i];
    p[a] = __dadd_rn(p0[a], __dmul_rn(fa, dt));  // p = p0 + f*dt
    if (fx & (1u << a)) {
      p0[a] = 0.0;
      p[a] = 0.0;
    }
  }
  if (nd.rmask) rigid_override<D>(nd, i, m, p0, p);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    vdt[a] = (p[a] * invM) * dt;
    dv[a] = (p[a] - p0[a]) * invM;
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    nd.vdt[a * Nn + i] = vdt[a];
    nd.dv[a * Nn + i] = dv[a];
    if (F32COPY && !nd.nf4) {
      nd.vdt_f[a * Nn + i] = float(vdt[a]);
      nd.dv_f[a * Nn + i] = float(dv[a]);
    }
  }
  if (D == 3 && !F32COPY && nd.dw4) put_node_dw(nd.dw4, i, vdt, dv);
  if (F32COPY && nd.nf4) {
    if (D == 2) {
      nd.nf4[i] = make_float4(float(vdt[0]), float(vdt[1]), float(dv[0]), float(dv[D - 1]));
    } else {
      nd.nf4[2 * i] = make_float4(float(vdt[0]), float(vdt[1]), float(vdt[D - 1]), 0.f);
      nd.nf4[2 * i + 1] = make_float4(float(dv[0]), float(dv[1]), float(dv[D - 1]), 0.f);
    }
  }
}

// The list compaction and the grid update of the plain step in one launch:
// CTAs of 256 threads stride over all node blocks, four at a time (64 threads
// per block).  A flagged block goes on the list (which the next step's clear
// reads), its flag is reset, and its nodes are updated (grid_node).
// Saves the compact_blocks launch; the list order is immaterial (as with the
// warp-aggregated appends of compact_blocks).  blockDim.x must be 256.
template <int D, bool F32COPY>
__global__ void __launch_bounds__(256) grid_scan_kernel(NodeP nd, double dt, double tol) {
  const int sub = threadIdx.x >> 6, l = threadIdx.x & 63;
  const int64_t stride = int64_t(gridDim.x) * 4;
  for (int64_t b0 = int64_t(blockIdx.x) * 4; b0 < nd.nblk; b0 += stride) {  // same trip count CTA-wide
    const int64_t blk = b0 + sub;
    const bool on = blk < nd.nblk && nd.bflag[blk] != 0u;
    __syncthreads();  // the block's 64 threads have read its flag before it is reset
    if (on && l == 0) {
      nd.bflag[blk] = 0u;
      nd.blist[atomicAdd(nd.bcount, 1u)] = uint32_t(blk);
    }
    if (on) {
      const int64_t i = block_node<D>(nd, uint32_t(blk), l);
      if (i >= 0) grid_node<D, F32COPY>(nd, i, dt, tol);
    }
  }
}

// ---------------------------------------------------------------------------
// Constitutive updates (update_stress!, Material.jl).  eps/sig symmetric storage.
template <int D, class R>
__device__ __forceinline__ void elastic(R lam, R mu, const R* eps, R* sig) {
  // lambda*(tr eps)*I + 2.0*mu*eps   (Material.jl:68-72, 80)
  R tr = (D == 2) ? eps[0] + eps[1] : (eps[0] + eps[1]) + eps[2];
  R lt = lam * tr;
  R tmu = R(2) * mu;
#pragma unroll
  for (int c = 0; c < Layout<D>::S; ++c) sig[c] = tmu * eps[c] + (c < D ? lt : R(0));
}

template <int D, class R>
__device__ __forceinline__ void neohookean(R lam, R mu, const R* F, double J, R* sig) {
  // (1/J)*( mu*(F*F' - I) + lambda*log(J)*I )   (Material.jl:119-122)
  R ll, iJ;
  if constexpr (sizeof(R) == 8) {
    ll = lam * log(J);
    iJ = 1.0 / J;
  } else {
    // FP32 particles: J - 1 taken in FP64 keeps log(J) accurate near J = 1
    ll = lam * log1pf(float(J - 1.0));
    iJ = 1.0f / float(J);
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      R s = F[i] * F[j];
#pragma unroll
      for (int k = 1; k < D; ++k) s += F[i + D * k] * F[j + D * k];
      R v = (i == j) ? mu * (s - R(1)) + ll : mu * s;
      sig[sym<D>(i, j)] = iJ * v;
    }
}

template <class R>
__device__ __forceinline__ R sqr(R a) {
  return a * a;
}

// J2 radial return, 3D (Material.jl:228-275)
template <class R>
__device__ __forceinline__ void j2_3d(R lam, R mu, R kappa, R fy, R k1, const R* eps, R* sig,
                                      R* alpha, R* ep, R* vm, R rtmuk1 = R(0)) {
  (void)lam;
  R tr = (eps[0] + eps[1]) + eps[2];
  R tt = R(0.333333333) * tr;
  R tmu = R(2) * mu;
  R s[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) s[c] = tmu * ((c < 3 ? eps[c] - tt : eps[c]) - ep[c]);
  // sqrt(s11^2 + s22^2 + s33^2 + 2.0*(s12^2 + s23^2 + s13^2))
  // |s| and 1/|s| from one reciprocal square root (|s| = 0: no plastic flow)
  const R q = ((sqr(s[0]) + sqr(s[1])) + sqr(s[2])) + R(2) * ((sqr(s[3]) + sqr(s[4])) + sqr(s[5]));
  const R rq = rsqrt(q);
  R ns = q > R(0) ? q * rq : R(0);
  R kt = kappa * tr;
  R a0 = *alpha;
  R f_trial = ns - (k1 * a0 + fy);
  R sg[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) sg[c] = c < 3 ? s[c] + kt : s[c];  // sigma_trial
  if (!(f_trial <= R(0))) {
    R inv = rq;
    R lamp = rtmuk1 != R(0) ? ((ns - k1 * a0) - fy) * rtmuk1 : ((ns - k1 * a0) - fy) / (tmu + k1);
    a0 += lamp;
    R cc = tmu * lamp;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      R nrm = inv * s[c];
      ep[c] += lamp * nrm;
      sg[c] -= cc * nrm;
    }
    *alpha = a0;
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) sig[c] = sg[c];
  (void)vm;  // von Mises stress is a function of sigma alone: computed at download (j2_vm)
}

// vmStr of the J2 updates from the stored stress (Material.jl:223-224, 273-274)
template <int D, class R>
__device__ __forceinline__ R j2_vm(const R* sg) {
  if constexpr (D == 3) {
    R ts = R(0.333333333) * ((sg[0] + sg[1]) + sg[2]);
    R d0 = sg[0] - ts, d1 = sg[1] - ts, d2 = sg[2] - ts;
    // sqrt(d11^2 + d22^2 + d33^2 + 2*(d12^2 + d13^2 + d23^2))
    return sqrt(((sqr(d0) + sqr(d1)) + sqr(d2)) + R(2) * ((sqr(sg[3]) + sqr(sg[5])) + sqr(sg[4])));
  } else {
    // devSig = I_dev * sigma (Voigt), sqrt(d1^2 + d2^2 + 2*d3^2)
    R d0 = R(0.5) * sg[0] + R(-0.5) * sg[1];
    R d1 = R(-0.5) * sg[0] + R(0.5) * sg[1];
    return sqrt((sqr(d0) + sqr(d1)) + R(2) * sqr(sg[2]));
  }
}

// J2 radial return, 2D Voigt [xx, yy, 2xy] (Material.jl:174-225)
template <class R>
__device__ __forceinline__ void j2_2d(R lam, R mu, R kappa, R fy, R k1, const R* eps, R* sig,
                                      R* alpha, R* ep, R* vm) {
  (void)lam;
  R e0 = eps[0], e1 = eps[1], e2 = R(2) * eps[2];
  // epsilon_dev = I_dev * epsilon, I_dev = [.5 -.5 0; -.5 .5 0; 0 0 1]
  R ed0 = R(0.5) * e0 + R(-0.5) * e1;
  R ed1 = R(-0.5) * e0 + R(0.5) * e1;
  R ed2 = e2;
  R tmu = R(2) * mu;
  // s_trial = diag(1,1,.5) * 2mu*(ed - ep)
  R s0 = tmu * (ed0 - ep[0]);
  R s1 = tmu * (ed1 - ep[1]);
  R s2 = R(0.5) * (tmu * (ed2 - ep[2]));
  R ns = sqrt((sqr(s0) + sqr(s1)) + R(2) * sqr(s2));
  R kt = kappa * (e0 + e1);
  R a0 = *alpha;
  R f_trial = ns - (k1 * a0 + fy);
  R g0 = kt + s0, g1 = kt + s1, g2 = s2;
  if (!(f_trial <= R(0))) {
    R inv = R(1) / ns;
    R n0 = inv * s0, n1 = inv * s1, n2 = inv * s2;
    R lamp = ((ns - k1 * a0) - fy) / (tmu + k1);
    a0 += lamp;
    ep[0] += lamp * n0;
    ep[1] += lamp * n1;
    ep[2] += lamp * (R(2) * n2);  // Iinv = diag(1,1,2)
    R cc = tmu * lamp;
    g0 -= cc * n0;
    g1 -= cc * n1;
    g2 -= cc * n2;
    *alpha = a0;
  }
  sig[0] = g0;
  sig[1] = g1;
  sig[2] = g2;
  (void)vm;  // computed at download (j2_vm)
}

template <int D>
__device__ __forceinline__ double det_d(const double* A) {
  if (D == 2) return A[0] * A[3] - A[2] * A[1];
  const double* x0 = A;
  const double* x1 = A + 3;
  const double* x2 = A + 6;
  double c0 = x1[1] * x2[2] - x1[2] * x2[1];
  double c1 = x1[2] * x2[0] - x1[0] * x2[2];
  double c2 = x1[0] * x2[1] - x1[1] * x2[0];
  return (x0[0] * c0 + x0[1] * c1) + x0[2] * c2;
}

// Johnson-Cook / Voce update_stress! (Material.jl:386-443, 445-493), 3D: trial
// stress sig + 2 mu deps, deviator with the reference's 0.333333333, radial
// return to the yield stress of the equivalent plastic strain (and, for
// Johnson-Cook, of the filtered plastic strain rate), that rate's update, and
// the returned stress deviator + kappa tr(eps) I.  Symmetric storage (xx, yy,
// zz, xy, yz, xz).
template <class R, int MAT>
__device__ __forceinline__ void jc_voce_3d(const MatParams& mp, R mu, R kappa, const R* sig_old, const R* deps,
                                           const R* eps, R* sig, R* alpha, R* alphad, R* vm) {
  const R ep = *alpha;
  R yieldS;
  if (ep < R(1.0e-10)) {
    yieldS = R(mp.A);
  } else if (MAT == MPM_MAT_JOHNSON_COOK) {
    const R ratio = fmax(*alphad / R(mp.epsdot0), R(1));
    const R base = R(mp.A) + R(mp.B) * pow(ep, R(mp.n));
    yieldS = mp.C != 0.0 ? base * pow(R(1) + ratio, R(mp.C)) : base;
  } else {
    yieldS = R(mp.A) - R(mp.B) * exp(-R(mp.C) * ep);
  }
  const R Gd = mu;
  R d[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) d[c] = sig_old[c] + R(2) * Gd * deps[c];
  const R third = R(0.333333333) * ((d[0] + d[1]) + d[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) d[c] = d[c] - third;
  const R J2 = R(1.224744871391589) *
               sqrt(((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + R(2) * ((d[3] * d[3] + d[5] * d[5]) + d[4] * d[4]));
  R dp = R(0);
  if (!(J2 < yieldS)) {
    dp = (J2 - yieldS) / (R(3) * Gd);
    const R sc = yieldS / J2;
#pragma unroll
    for (int c = 0; c < 6; ++c) d[c] = d[c] * sc;
  }
  *alpha = ep + dp;
  const R tav = R(mp.tav);
  R ad = *alphad;
  ad = ad - ad * R(mp.dtime) / tav;
  ad = ad + dp / tav;
  *alphad = fmax(R(0), ad);
  *vm = sqrt(((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + R(2) * ((d[3] * d[3] + d[5] * d[5]) + d[4] * d[4]));
  const R p = kappa * ((eps[0] + eps[1]) + eps[2]);
#pragma unroll
  for (int c = 0; c < 6; ++c) sig[c] = c < 3 ? d[c] + p : d[c];
}

// Johnson-Cook with damage, 3D (Material.jl:566-646 with compute_damage,
// :511-549).  A fully damaged particle (damage >= 1) carries the pressure
// kappa tr(eps) only and keeps its state.  Otherwise: Johnson-Cook yield of the
// equivalent plastic strain, its filtered rate and the temperature (thermal
// softening for Tr <= T < Tm, zero at and above Tm), shear modulus and yield
// scaled by (1 - damage), radial return as in jc_voce_3d, then the failure
// strain of the returned stress's triaxiality, rate and temperature, the
// damage_init / damage update, and the temperature rise delta x flow x dp.
// The reference method reads mat.damage and mat.strength, fields its type
// names damage_part and strength_part; this is what those lines compute on
// the fields they evidently mean.
template <class R>
__device__ __forceinline__ void jc_damage_3d(const MatParams& mp, R mu, R kappa, const R* sig_old, const R* deps,
                                             const R* eps, R* sig, R* alpha, R* alphad, R* vm, R* dinit, R* dam,
                                             R* temp) {
  const R damage = *dam;
  const R pH = kappa * ((eps[0] + eps[1]) + eps[2]);
  if (damage >= R(1)) {  // Material.jl:572-576
#pragma unroll
    for (int c = 0; c < 6; ++c) sig[c] = c < 3 ? pH : R(0);
    return;
  }
  const R ep = *alpha;
  R T = *temp;
  R yieldS;
  if (ep < R(1.0e-10)) {
    yieldS = R(mp.A);
  } else if (T < R(mp.Tm)) {
    const R ratio = fmax(*alphad / R(mp.epsdot0), R(1));
    const R base = R(mp.A) + R(mp.B) * pow(ep, R(mp.n));
    yieldS = mp.C != 0.0 ? base * pow(R(1) + ratio, R(mp.C)) : base;
    if (mp.m != 0.0 && T >= R(mp.Tr)) yieldS *= R(1) - pow((T - R(mp.Tr)) / R(mp.Tmr), R(mp.m));
  } else {
    yieldS = R(0);
  }
  R Gd = mu;
  if (damage > R(0)) {
    Gd *= (R(1) - damage);
    yieldS *= (R(1) - damage);
  }
  R d[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) d[c] = sig_old[c] + R(2) * Gd * deps[c];
  const R third = R(0.333333333) * ((d[0] + d[1]) + d[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) d[c] = d[c] - third;
  const R q0 = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + R(2) * ((d[3] * d[3] + d[5] * d[5]) + d[4] * d[4]);
  const R J2 = R(1.224744871391589) * sqrt(q0);
  R dp = R(0);
  if (!(J2 < yieldS)) {
    dp = (J2 - yieldS) / (R(3) * Gd);
    const R sc = yieldS / J2;
#pragma unroll
    for (int c = 0; c < 6; ++c) d[c] = d[c] * sc;
  }
  *alpha = ep + dp;
#pragma unroll
  for (int c = 0; c < 6; ++c) sig[c] = c < 3 ? d[c] + pH : d[c];
  const R tav = R(mp.tav);
  R ad = *alphad;
  ad = ad - ad * R(mp.dtime) / tav;
  ad = ad + dp / tav;
  ad = fmax(R(0), ad);
  *alphad = ad;
  const R q = ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + R(2) * ((d[3] * d[3] + d[5] * d[5]) + d[4] * d[4]);
  const R flow = R(1.224744871391589) * sqrt(q);
  *vm = flow;
  // compute_damage (Material.jl:511-549), with its own 1.224744871
  const R vmd = R(1.224744871) * sqrt(q);
  R triax = R(0);
  if (pH != R(0) && vmd != R(0)) triax = -pH / (vmd + R(0.01) * fabs(pH));
  if (triax > R(3)) triax = R(3);
  R fs = R(mp.d1) + R(mp.d2) * exp(R(mp.d3) * triax);
  if (mp.d4 > 0.0 && ad > R(mp.depsdot0)) fs *= (R(1) + R(mp.d4) * log(ad / R(mp.depsdot0)));
  if (mp.d5 > 0.0 && T >= R(mp.Tr)) fs *= R(1) + R(mp.d5) * (T - R(mp.Tr)) / R(mp.Tmr);
  R di = *dinit + dp / fs;
  *dinit = di;
  if (di >= R(1)) *dam = fmin((di - R(1)) * R(10), R(1));
  T += R(mp.delta) * flow * dp;
  *temp = T;
}

// F <- F (I + L dt), J, V = J V0, strain += sym(L dt), update_stress! of particle p
// (:520-532), given L dt; fin: the particle's new x and v are finite.
// pre (J2 only, may be null): this thread's prefetched inputs in shared
// memory, slot k at pre[k * blockDim.x]: F (D*D), strain (S), plastic strain
// (PS), alpha, V0 (g2p_prefetch)
template <int D, class R, int MAT>
__device__ __forceinline__ void kinematics_stress(const PartP& pp, int64_t p, const R (&Ldt)[D][D],
                                                  const MatParams& mp, bool fin, unsigned* status,
                                                  const R* pre = nullptr) {
  using L = Layout<D>;
  const int bs = blockDim.x;
  constexpr int PF = 0, PE = D * D, PP = D * D + L::S, PA = D * D + L::S + L::PS, PV = PA + 1;
  // F <- F (I + L dt)   (:523)
  R F[D * D], Fn[D * D];
#pragma unroll
  for (int c = 0; c < D * D; ++c) F[c] = pre ? pre[(PF + c) * bs] : *field<R>(pp, L::F + c, p);
  // F (I + L dt) = F + F (L dt)
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      R s = F[i + D * j];
#pragma unroll
      for (int k = 0; k < D; ++k) s += F[i + D * k] * Ldt[k][j];
      Fn[i + D * j] = s;
    }
  double Fd[D * D];
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    Fd[c] = to_f64(Fn[c]);
    *field<R>(pp, L::F + c, p) = Fn[c];
  }
  double J = det_d<D>(Fd);  // det F in FP64 for both precisions
  *field<R>(pp, L::VOL, p) = R(J * to_f64(pre ? pre[PV * bs] : *field<R>(pp, L::VOL0, p)));
  // strain += dt * 0.5*(L + L')
  R eps[L::S], deps[L::S];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      int c = sym<D>(i, j);
      R e = pre ? pre[(PE + c) * bs] : *field<R>(pp, L::EPS + c, p);
      deps[c] = (i == j) ? Ldt[i][i] : R(0.5) * (Ldt[i][j] + Ldt[j][i]);
      e += deps[c];
      eps[c] = e;
      *field<R>(pp, L::EPS + c, p) = e;
    }
  R lam = mat_const<R>(mp.lambda, mp.f_lambda), mu = mat_const<R>(mp.mu, mp.f_mu);
  R kappa = mat_const<R>(mp.kappa, mp.f_kappa);
  if (mp.per_particle) {
    lam = *field<R>(pp, L::LAM, p);
    mu = *field<R>(pp, L::MU, p);
    kappa = lam + mu;
  }
  R sig[L::S];
  if (MAT == MPM_MAT_ELASTIC) {
    if (D == 3) {
      // vmStr of the incoming stress (Material.jl:78-79)
      R so[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) so[c] = *field<R>(pp, L::SIG + c, p);
      *field<R>(pp, L::VM, p) =
          sqrt(((sqr(so[0]) + sqr(so[1])) + sqr(so[2])) + R(2) * ((sqr(so[3]) + sqr(so[5])) + sqr(so[4])));
    }
    elastic<D, R>(lam, mu, eps, sig);
  } else if (MAT == MPM_MAT_NEOHOOKEAN) {
    neohookean<D, R>(lam, mu, Fn, J, sig);
  } else if (MAT == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    if constexpr (D == 3) {
      R so[6], alpha = *field<R>(pp, L::ALPHA, p), ad = *field<R>(pp, L::ALPHAD, p), vm = *field<R>(pp, L::VM, p);
      R di = *field<R>(pp, L::DINIT, p), dm = *field<R>(pp, L::DAM, p), T = *field<R>(pp, L::TEMP, p);
#pragma unroll
      for (int c = 0; c < 6; ++c) so[c] = *field<R>(pp, L::SIG + c, p);
      jc_damage_3d<R>(mp, mu, kappa, so, deps, eps, sig, &alpha, &ad, &vm, &di, &dm, &T);
      *field<R>(pp, L::ALPHA, p) = alpha;
      *field<R>(pp, L::ALPHAD, p) = ad;
      *field<R>(pp, L::VM, p) = vm;
      *field<R>(pp, L::DINIT, p) = di;
      *field<R>(pp, L::DAM, p) = dm;
      *field<R>(pp, L::TEMP, p) = T;
    }
  } else if (MAT == MPM_MAT_JOHNSON_COOK || MAT == MPM_MAT_VOCE) {
    if constexpr (D == 3) {
      R so[6], alpha = *field<R>(pp, L::ALPHA, p), ad = *field<R>(pp, L::ALPHAD, p), vm;
#pragma unroll
      for (int c = 0; c < 6; ++c) so[c] = *field<R>(pp, L::SIG + c, p);
      jc_voce_3d<R, MAT>(mp, mu, kappa, so, deps, eps, sig, &alpha, &ad, &vm);
      *field<R>(pp, L::ALPHA, p) = alpha;
      *field<R>(pp, L::ALPHAD, p) = ad;
      *field<R>(pp, L::VM, p) = vm;
    }
  } else {
    R alpha = pre ? pre[PA * bs] : *field<R>(pp, L::ALPHA, p);
    R ep[L::PS];
#pragma unroll
    for (int c = 0; c < L::PS; ++c) ep[c] = pre ? pre[(PP + c) * bs] : *field<R>(pp, L::EP + c, p);
    R vm;
    if (D == 3)
      j2_3d<R>(lam, mu, kappa, mat_const<R>(mp.fy, mp.f_fy), mat_const<R>(mp.k1, mp.f_k1), eps, sig, &alpha, ep,
               &vm, mat_const<R>(mp.rtmuk1, mp.f_rtmuk1));
    else
      j2_2d<R>(lam, mu, kappa, mat_const<R>(mp.fy, mp.f_fy), mat_const<R>(mp.k1, mp.f_k1), eps, sig, &alpha, ep,
               &vm);
    *field<R>(pp, L::ALPHA, p) = alpha;
#pragma unroll
    for (int c = 0; c < L::PS; ++c) *field<R>(pp, L::EP + c, p) = ep[c];
  }
#pragma unroll
  for (int c = 0; c < L::S; ++c) {
    *field<R>(pp, L::SIG + c, p) = sig[c];
    fin &= finite_bits(sig[c]);
  }
  unsigned st = (positive_bits(J) ? 0u : ST_NEGATIVE_J) | (fin ? 0u : ST_NONFINITE);
  if (st) atomicOr(status, st);
}

// One 4-byte asynchronous copy global -> shared (cp.async, this thread's own
// slot), and the wait for all of this thread's copies.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// G2P + kinematics + stress of particle pp.begin + t (t < pp.count).
// pre (J2 only, may be null): this thread's shared-memory slots (stride
// blockDim.x) into which the constitutive inputs are copied asynchronously
// at the start, so that their loads overlap the node gather without holding
// registers (the layout of kinematics_stress's pre).
template <int D, class R, int MAT, bool CG = false>
__device__ __forceinline__ void g2p_particle(const GridP& g, const NodeP& nd, const PartP& pp, int64_t t,
                                             const MatParams& mp, double dt, unsigned* status, R* pre = nullptr) {
  using L = Layout<D>;
  int64_t p = pp.begin + t;
  if constexpr (MAT == MPM_MAT_J2) {
    if (pre) {
      const int bs = blockDim.x;
      int k = 0;
#pragma unroll
      for (int c = 0; c < D * D; ++c) cp_async4(pre + (k++) * bs, field<R>(pp, L::F + c, p));
#pragma unroll
      for (int c = 0; c < L::S; ++c) cp_async4(pre + (k++) * bs, field<R>(pp, L::EPS + c, p));
#pragma unroll
      for (int c = 0; c < L::PS; ++c) cp_async4(pre + (k++) * bs, field<R>(pp, L::EP + c, p));
      cp_async4(pre + (k++) * bs, field<R>(pp, L::ALPHA, p));
      cp_async4(pre + (k++) * bs, field<R>(pp, L::VOL0, p));
    }
  }
  R x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<R>(pp, L::X + a, p);
  Hat<D, R> h;
  // the hat the P2G of this step stored (same positions), else computed here
  const bool ok = (sizeof(R) == 8 && pp.hat_c) ? hat_get<D, R>(g, pp, p, h) : hat<D, R>(g, x, h);
  if (!ok) {
    if (pre) cp_async_wait_all();  // no copy into this CTA's shared memory outlives the thread
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  Corners<D, R> cr;
  if (D == 3) corner_nodes<D, R>(g, h, cr);
  else corners<D, R>(g, h, cr);
  R v[D];
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = *field<R>(pp, L::V + a, p);
  R Ldt[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int j = 0; j < D; ++j) Ldt[a][j] = R(0);
  const R* vdt_n = sizeof(R) == 8 ? reinterpret_cast<const R*>(nd.vdt) : reinterpret_cast<const R*>(nd.vdt_f);
  const R* dv_n = sizeof(R) == 8 ? reinterpret_cast<const R*>(nd.dv) : reinterpret_cast<const R*>(nd.dv_f);
  const int64_t Nn = nd.nodeCount;
  if (sizeof(R) == 4 && !CG && nd.nf4) {
    // FP32 particles, interleaved node records: all corner loads issued first
    // (two 16-byte loads per corner in 3D, one in 2D), then the same sums
    constexpr int NC = 1 << D;
    float4 rv[NC], rd[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      if (D == 3) {
        rv[k] = __ldg(nd.nf4 + 2 * cr.node[k]);
        rd[k] = __ldg(nd.nf4 + 2 * cr.node[k] + 1);
      } else {
        rv[k] = __ldg(nd.nf4 + cr.node[k]);
      }
    }
    if constexpr (D == 3) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int bx = q & 1, by = q >> 1;
        const R Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1];
        const R Gx = bx ? h.gh[0] : h.gl[0], Gy = by ? h.gh[1] : h.gl[1];
        const R Nxy = Nx * Ny, GxNy = Gx * Ny, NxGy = Nx * Gy;
        const float4 a0 = rv[q], a1 = rv[q + 4], b0 = rd[q], b1 = rd[q + 4];
        const R vd0[3] = {R(a0.x), R(a0.y), R(a0.z)}, vd1[3] = {R(a1.x), R(a1.y), R(a1.z)};
        const R dv0[3] = {R(b0.x), R(b0.y), R(b0.z)}, dv1[3] = {R(b1.x), R(b1.y), R(b1.z)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const R Z0 = h.Nl[2] * vd0[a] + h.Nh[2] * vd1[a];
          const R Z1 = h.gl[2] * vd0[a] + h.gh[2] * vd1[a];
          const R W = h.Nl[2] * dv0[a] + h.Nh[2] * dv1[a];
          x[a] += Nxy * Z0;
          v[a] += Nxy * W;
          Ldt[a][0] += GxNy * Z0;
          Ldt[a][1] += NxGy * Z0;
          Ldt[a][2] += Nxy * Z1;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        const R N = cr.N[k];
        const R vd[2] = {R(rv[k].x), R(rv[k].y)}, dvv[2] = {R(rv[k].z), R(rv[k].w)};
#pragma unroll
        for (int a = 0; a < D; ++a) {
          v[a] += N * dvv[a];
          x[a] += N * vd[a];
#pragma unroll
          for (int j = 0; j < D; ++j) Ldt[a][j] += vd[a] * cr.dN[k][j];
        }
      }
    }
  } else if constexpr (D == 3) {
    // factored along z: per (x, y) corner pair, Z0 = sum Nz vdt, Z1 = sum Gz vdt,
    // W = sum Nz dv over the two z corners, then x += Nx Ny Z0, v += Nx Ny W,
    // L dt += (Gx Ny Z0, Nx Gy Z0, Nx Ny Z1).
    // Strictly inside the cell (hat_interior: gl = -dxI, gh = +dxI per axis):
    // Z0 = vd0 + Nh_z (vd1 - vd0), Z1 = dxI_z (vd1 - vd0), and the gradient
    // sums are signed sums of Ny Z0, Nx Z0 and Nx Ny (vd1 - vd0), each scaled by
    // its dxI once after the corners.
    if (hat_interior<3, R>(h)) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int bx = q & 1, by = q >> 1;
        const R Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1];
        const R Nxy = Nx * Ny;
        const int64_t n0 = cr.node[q], n1 = cr.node[q + 4];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const R vd0 = nload<CG>(vdt_n + a * Nn + n0), vd1 = nload<CG>(vdt_n + a * Nn + n1);
          const R dv0 = nload<CG>(dv_n + a * Nn + n0), dv1 = nload<CG>(dv_n + a * Nn + n1);
          const R dz = vd1 - vd0;
          const R Z0 = vd0 + h.Nh[2] * dz;
          const R W = h.Nl[2] * dv0 + h.Nh[2] * dv1;
          x[a] += Nxy * Z0;
          v[a] += Nxy * W;
          Ldt[a][0] += (bx ? Ny : -Ny) * Z0;
          Ldt[a][1] += (by ? Nx : -Nx) * Z0;
          Ldt[a][2] += Nxy * dz;
        }
      }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ldt[a][j] *= h.gh[j];
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int bx = q & 1, by = q >> 1;
        const R Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1];
        const R Gx = bx ? h.gh[0] : h.gl[0], Gy = by ? h.gh[1] : h.gl[1];
        const R Nxy = Nx * Ny, GxNy = Gx * Ny, NxGy = Nx * Gy;
        const int64_t n0 = cr.node[q], n1 = cr.node[q + 4];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const R vd0 = nload<CG>(vdt_n + a * Nn + n0), vd1 = nload<CG>(vdt_n + a * Nn + n1);
          const R dv0 = nload<CG>(dv_n + a * Nn + n0), dv1 = nload<CG>(dv_n + a * Nn + n1);
          const R Z0 = h.Nl[2] * vd0 + h.Nh[2] * vd1;
          const R Z1 = h.gl[2] * vd0 + h.gh[2] * vd1;
          const R W = h.Nl[2] * dv0 + h.Nh[2] * dv1;
          x[a] += Nxy * Z0;
          v[a] += Nxy * W;
          Ldt[a][0] += GxNy * Z0;
          Ldt[a][1] += NxGy * Z0;
          Ldt[a][2] += Nxy * Z1;
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < (1 << D); ++k) {
      int64_t n = cr.node[k];
      R N = cr.N[k];
      R vd[D], dvv[D];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        vd[a] = nload<CG>(vdt_n + a * Nn + n);
        dvv[a] = nload<CG>(dv_n + a * Nn + n);
      }
#pragma unroll
      for (int a = 0; a < D; ++a) {
        v[a] += N * dvv[a];
        x[a] += N * vd[a];
#pragma unroll
        for (int j = 0; j < D; ++j) Ldt[a][j] += vd[a] * cr.dN[k][j];
      }
    }
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    *field<R>(pp, L::X + a, p) = x[a];
    *field<R>(pp, L::V + a, p) = v[a];
  }
  bool fin = true;
#pragma unroll
  for (int a = 0; a < D; ++a) fin &= finite_bits(x[a]) & finite_bits(v[a]);
  if (MAT == MPM_MAT_J2 && pre) {
    cp_async_wait_all();
    kinematics_stress<D, R, MAT>(pp, p, Ldt, mp, fin, status, pre);
  } else {
    kinematics_stress<D, R, MAT>(pp, p, Ldt, mp, fin, status);
  }
}

// FP32 particles: at most 48 registers (five 256-thread CTAs per SM); the
// latency-bound FP32 G2P gains more from the extra resident warps than it
// loses to 16-20 bytes of spills (43.0 -> 39.9 us on the Taylor bar).  The
// FP64 kernel keeps its natural register count.
template <int D, class R, int MAT>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 5 : 0) g2p_kernel(GridP g, NodeP nd, PartP pp, MatParams mp, double dt,
                                                  unsigned* status) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < pp.count) g2p_particle<D, R, MAT>(g, nd, pp, t, mp, dt, status);
}

// The J2 G2P with its constitutive inputs (F, strain, plastic strain, alpha,
// V0) prefetched into shared memory by cp.async: dynamic shared memory of
// g2p_prefetch_slots<D>() x blockDim.x particle values.
template <int D>
constexpr int g2p_prefetch_slots() {
  return D * D + Layout<D>::S + Layout<D>::PS + 2;
}

template <int D, class R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 5 : 0) g2p_prefetch_kernel(GridP g, NodeP nd, PartP pp,
                                                                                  MatParams mp, double dt,
                                                                                  unsigned* status) {
  extern __shared__ __align__(16) unsigned char g2p_pre_smem[];
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < pp.count)
    g2p_particle<D, R, MPM_MAT_J2>(g, nd, pp, t, mp, dt, status, reinterpret_cast<R*>(g2p_pre_smem) + threadIdx.x);
}

// ---------------------------------------------------------------------------
// Rigid body `bit` (in body order among the rigid bodies) of one step: every
// particle marks the nodes of its linear cell (getAdjacentGridPoints with the
// linear basis, SolveExplicitSolidMechanics2D.jl:456) and their blocks for the
// grid update's override, then moves by dt v_rigid (:539-551).  The reference
// moves rigid particles after G2P; nothing between this launch (after P2G)
// and the end of the step reads their positions, so marking with the old
// position and moving here is the same.  A particle outside the grid is
// reported and frozen.
template <int D, class R>
__global__ void __launch_bounds__(256) rigid_kernel(GridP g, NodeP nd, PartP pp, int bit, double vx, double vy,
                                                    double vz, double dt, unsigned* status) {
  using L = Layout<D>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  R x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<R>(pp, L::X + a, p);
  Hat<D, R> h;
  if (!hat<D, R>(g, x, h)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  const int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + (D == 3 ? g.nxy * int64_t(h.c[D - 1]) : 0);
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) atomicOr(nd.rmask + corner_node<D>(g, base, k), 1u << bit);
  mark_blocks<D>(nd, h.c);
  const double v[3] = {vx, vy, vz};
#pragma unroll
  for (int a = 0; a < D; ++a) *field<R>(pp, L::X + a, p) = R(to_f64(x[a]) + dt * v[a]);
}

// ---------------------------------------------------------------------------
// EnergiesFix sums (Fix.jl:248-270): kinetic energy, strain energy and
// momentum (D) over the particles, in one launch.  Each CTA writes its sums
// to partial[block]; the CTA that finishes last (a ticket counter after a
// fence) folds the partials into out in a fixed order -- lane l of its first
// warp adds blocks l, l + 32, ..., then a fixed shuffle tree -- so the result
// does not depend on which CTA finishes last, and resets the ticket to zero
// for the next launch.  The 1/2 factors are applied once to the folded sums
// (a power-of-two scaling, exact).  With a record cursor rec the sums go to
// rec->base[rec->idx] and the cursor advances (a captured step graph fills
// successive records); else to out.  kEnergyBlocks CTAs: one wave at the two
// CTAs per SM its registers allow.
template <int D, class R>
__global__ void __launch_bounds__(256) energies_kernel(PartP pp, double* partial, unsigned* ticket, double* out,
                                                       EnRec* rec) {
  using L = Layout<D>;
  constexpr int NQ = 2 + D;
  double q[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) q[k] = 0.0;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < pp.count;
       t += int64_t(gridDim.x) * blockDim.x) {
    int64_t p = pp.begin + t;
    double m = *field<R>(pp, L::M, p);
    double vv = 0.0;
    double v[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      v[a] = *field<R>(pp, L::V + a, p);
      vv += v[a] * v[a];
    }
    q[0] += m * vv;
    // sigma:eps with the off-diagonal entries twice: diagonal + 2 off-diagonal
    double sd = 0.0, so = 0.0;
#pragma unroll
    for (int c = 0; c < L::S; ++c) {
      const double e = double(*field<R>(pp, L::SIG + c, p)) * double(*field<R>(pp, L::EPS + c, p));
      if (c < D) sd += e;
      else so += e;
    }
    q[1] += double(*field<R>(pp, L::VOL, p)) * (sd + 2.0 * so);
#pragma unroll
    for (int a = 0; a < D; ++a) q[2 + a] += m * v[a];
  }
  __shared__ double sh[NQ][256];
  __shared__ bool last;
#pragma unroll
  for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int k = 0; k < NQ; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NQ; ++k) partial[int64_t(blockIdx.x) * NQ + k] = sh[k][0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  const int lane = threadIdx.x;
  double acc[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) acc[k] = 0.0;
  for (int b = lane; b < int(gridDim.x); b += 32)
#pragma unroll
    for (int k = 0; k < NQ; ++k) acc[k] += __ldcg(partial + int64_t(b) * NQ + k);
#pragma unroll
  for (int k = 0; k < NQ; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
  if (lane == 0) {
    if (rec) {  // the record cursor of a captured step: the next record slot
      out = rec->base + rec->idx * NQ;
      rec->idx += 1;
    }
    out[0] = 0.5 * acc[0];
    out[1] = 0.5 * acc[1];
#pragma unroll
    for (int k = 2; k < NQ; ++k) out[k] = acc[k];
    *ticket = 0u;
  }
}

// ---------------------------------------------------------------------------
// AoS (host layout, FP64) <-> SoA (device fields, precision R).
struct CompMap {
  int n;          // components moved per particle
  int src[9];     // AoS component for each SoA field (upload) / SoA field for each AoS entry
  // upload only: pairs of AoS components that must be equal (the mirrored
  // entries of a symmetric matrix); any pair that differs sets `bit` in *flag
  int nchk;
  int ca[3], cb[3];
  unsigned bit;
  unsigned* flag;
};

template <class R>
__global__ void aos_to_soa_kernel(PartP pp, const double* src, int per, int f0, CompMap cm) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  for (int c = 0; c < cm.n; ++c)
    *field<R>(pp, f0 + c, pp.begin + t) = R(src[t * per + cm.src[c]]);
  bool asym = false;
  for (int k = 0; k < cm.nchk; ++k) asym |= src[t * per + cm.ca[k]] != src[t * per + cm.cb[k]];
  if (asym && cm.flag) atomicOr(cm.flag, cm.bit);
}

// vmStr of J2 particles, from the stored stress, into a dense FP64 array
template <int D, class R>
__global__ void j2_vm_kernel(PartP pp, double* dst) {
  using L = Layout<D>;
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  R sg[L::S];
#pragma unroll
  for (int c = 0; c < L::S; ++c) sg[c] = *field<R>(pp, L::SIG + c, pp.begin + t);
  dst[t] = double(j2_vm<D, R>(sg));
}

template <class R>
__global__ void soa_to_aos_kernel(PartP pp, double* dst, int per, int f0, CompMap cm) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  for (int c = 0; c < cm.n; ++c) dst[t * per + c] = double(*field<R>(pp, f0 + cm.src[c], pp.begin + t));
}

}  // namespace jmpm

// ---------------------------------------------------------------------------
// Counting sort of particles by (body, cell).  key = body * ncells + cell
// (cell linear index x-fastest; a particle outside the grid gets its body's
// last bucket, ncells).  Order inside a cell is the atomic arrival order.
namespace jmpm {

template <int D, class R>
__global__ void __launch_bounds__(256) sort_keys_kernel(GridP g, PartP pp, uint32_t body_base, uint32_t ncells,
                                                        SortP sp) {
  using L = Layout<D>;
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  int64_t p = pp.begin + t;
  uint32_t cell = 0;
  bool inside = true;
  int64_t stride = 1;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    R xa = *field<R>(pp, L::X + a, p);
    R tt = add_rn(mul_rn(sub_rn(xa, R(g.xmin[a])), R(g.dxI[a])), R(1));
    int i1 = floor_to_int(tt);
    if (i1 < 1 || i1 > int(g.nn[a] - 1)) inside = false;
    cell += uint32_t(int64_t(i1 - 1) * stride);
    stride *= (g.nn[a] - 1);
  }
  uint32_t key = body_base + (inside ? cell : ncells);
  sp.key[p] = key;
  sp.rank[p] = atomicAdd(sp.count + key, 1u);
}

// exclusive scan, three passes: per-1024 block scan, scan of block sums, add
static __global__ void __launch_bounds__(1024) scan_blocks_kernel(const uint32_t* in, uint32_t* out, uint32_t* blocksum,
                                                           int64_t n) {
  __shared__ uint32_t sh[1024];
  int64_t i = int64_t(blockIdx.x) * 1024 + threadIdx.x;
  uint32_t v = i < n ? in[i] : 0u;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t add = threadIdx.x >= off ? sh[threadIdx.x - off] : 0u;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  if (i < n) out[i] = sh[threadIdx.x] - v;
  if (threadIdx.x == 1023) blocksum[blockIdx.x] = sh[1023];
}

static __global__ void __launch_bounds__(1024) scan_sums_kernel(uint32_t* blocksum, int64_t nb) {
  __shared__ uint32_t sh[1024];
  uint32_t carry = 0;
  for (int64_t base = 0; base < nb; base += 1024) {
    int64_t i = base + threadIdx.x;
    uint32_t v = i < nb ? blocksum[i] : 0u;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      uint32_t add = threadIdx.x >= off ? sh[threadIdx.x - off] : 0u;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nb) blocksum[i] = carry + sh[threadIdx.x] - v;
    uint32_t tot = sh[1023];
    __syncthreads();
    carry += tot;
  }
}

static __global__ void __launch_bounds__(1024) scan_add_kernel(uint32_t* out, const uint32_t* blocksum, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * 1024 + threadIdx.x;
  if (i < n) out[i] += blocksum[blockIdx.x];
}

// move every field of particle p to slot offset[key] + rank, and carry its original index
template <class R>
__global__ void __launch_bounds__(256) sort_scatter_kernel(const R* __restrict__ src, R* __restrict__ dst,
                                                           int64_t pitch, int nf, SortP sp,
                                                           const int64_t* __restrict__ orig_src,
                                                           int64_t* __restrict__ orig_dst) {
  int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= pitch) return;
  int64_t d = int64_t(sp.offset[sp.key[p]]) + sp.rank[p];
  for (int f = 0; f < nf; ++f) dst[int64_t(f) * pitch + d] = src[int64_t(f) * pitch + p];
  orig_dst[d] = orig_src[p];
}

// download in original order: dst[(orig[slot] - first) * per + c] = field[slot]
template <class R>
__global__ void soa_to_aos_perm_kernel(PartP pp, const int64_t* __restrict__ orig, double* dst, int per, int f0,
                                       CompMap cm) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  int64_t o = orig[pp.begin + t] - pp.begin;
  for (int c = 0; c < cm.n; ++c) dst[o * per + c] = double(*field<R>(pp, f0 + cm.src[c], pp.begin + t));
}

template <int D, class R>
__global__ void j2_vm_perm_kernel(PartP pp, const int64_t* __restrict__ orig, double* dst) {
  using L = Layout<D>;
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  R sg[L::S];
#pragma unroll
  for (int c = 0; c < L::S; ++c) sg[c] = *field<R>(pp, L::SIG + c, pp.begin + t);
  dst[orig[pp.begin + t] - pp.begin] = double(j2_vm<D, R>(sg));
}

}  // namespace jmpm
