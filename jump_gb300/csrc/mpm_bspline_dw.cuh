// mpm_bspline_dw.cuh -- the quadratic and cubic B-spline USL step of an
// MPM_PREC_DW context (3D; QuadBsplineBasis / CubicBsplineBasis,
// Basis.jl:374-820, Bsplines.jl:18-172): the P2G and G2P of mpm_bspline.cuh
// with their sums, weights and node values in double-word FP32 (mpm_dw.cuh).
//
// The support -- each axis's first node, the spline type of each node and the
// distance r = (x - x_node) dxI -- is formed in FP64 exactly as bs_axes forms
// it, so the nodes are the FP64 step's; r is then taken to double-word (the
// conversion keeps the sign of r - c for every breakpoint c, so each spline
// piece is the one the FP64 step picks) and the pieces' polynomials are
// evaluated in double-word by Horner's rule.  The G2P's tail is dw_finish,
// shared with the linear basis.
#pragma once

#include "mpm_bspline.cuh"
#include "mpm_step_dw.cuh"

namespace jmpm {

template <int K>
struct BsAxisDW {
  int64_t first;  // 0-based index of the first support node on this axis
  dw N[K];        // 1D values
  dw G[K];        // 1D derivatives along the axis: dN/dr x dxI
};

// an FP64 constant split into a double-word pair at compile time
struct dwc {
  float hi, lo;
};
constexpr dwc dw_split(double d) { return dwc{float(d), float(d - double(float(d)))}; }
__device__ __forceinline__ dw dwk(dwc c) { return dw_make(c.hi, c.lo); }

// x + c for an exact float c (TwoSum of the high parts, then one Fast2Sum)
__device__ __forceinline__ dw add_f(dw x, float c) {
  float s, e, zh, zl;
  two_sum(x.hi, c, s, e);
  fast_two_sum(s, __fadd_rn(e, x.lo), zh, zl);
  return dw_make(zh, zl);
}

// x < c and x <= c for an exact float c (a renormalised pair: hi is x rounded
// to nearest, so when hi == c the sign of lo decides)
__device__ __forceinline__ bool dw_lt(dw x, float c) { return x.hi < c || (x.hi == c && x.lo < 0.f); }
__device__ __forceinline__ bool dw_le(dw x, float c) { return x.hi < c || (x.hi == c && x.lo <= 0.f); }

// quad_bs in double-word (Bsplines.jl:18-80)
__device__ __forceinline__ void quad_bs_dw(int t, dw r, dw& N, dw& dN) {
  const dw z = dw_make(0.f, 0.f);
  N = dN = z;
  // 0.5 r^2 + 1.5 r + 1.125, 0.5 r^2 - 1.5 r + 1.125, 0.75 - r^2
  auto left = [&] { N = add_f(add_f(dw_scale(r, 0.5f), 1.5f) * r, 1.125f); dN = add_f(r, 1.5f); };
  auto right = [&] { N = add_f(add_f(dw_scale(r, 0.5f), -1.5f) * r, 1.125f); dN = add_f(r, -1.5f); };
  auto mid = [&] { N = add_f(-dw_sqr(r), 0.75f); dN = dw_scale(r, -2.f); };
  if (t == 1) {
    if (dw_lt(r, -1.5f) || !dw_le(r, 1.5f)) return;
    if (dw_le(r, -0.5f)) left();
    else if (dw_le(r, 0.f)) { N = add_f(r, 1.f); dN = dw_make(1.f, 0.f); }
    else if (dw_le(r, 0.5f)) { N = add_f(-r, 1.f); dN = dw_make(-1.f, 0.f); }
    else right();
  } else if (t == 2) {
    if (dw_lt(r, -1.f) || !dw_le(r, 1.5f)) return;
    if (dw_le(r, -0.5f)) { N = add_f(r, 1.f); dN = dw_make(1.f, 0.f); }
    else if (dw_le(r, 0.5f)) mid();
    else right();
  } else if (t == 3) {
    if (dw_lt(r, -1.5f) || !dw_le(r, 1.5f)) return;
    if (dw_le(r, -0.5f)) left();
    else if (dw_le(r, 0.5f)) mid();
    else right();
  } else {
    if (dw_lt(r, -1.5f) || !dw_le(r, 1.f)) return;
    if (dw_le(r, -0.5f)) left();
    else if (dw_le(r, 0.5f)) mid();
    else { N = add_f(-r, 1.f); dN = dw_make(-1.f, 0.f); }
  }
}

// cubic_bs in double-word (Bsplines.jl:86-172), with the reference's
// constants (1/6, 1/3, 2/3, 4/3 as FP64 values; type 4's 0.6666666667)
__device__ __forceinline__ void cubic_bs_dw(int t, dw r, dw& N, dw& dN) {
  constexpr dwc C6 = dw_split(0.16666666666666666), C3 = dw_split(0.3333333333333333);
  constexpr dwc T3 = dw_split(0.6666666666666666), F3 = dw_split(1.3333333333333333);
  constexpr dwc T4 = dw_split(0.6666666667);
  const dw z = dw_make(0.f, 0.f);
  N = dN = z;
  const dw r2 = dw_sqr(r);
  // the pieces, by Horner's rule
  auto outer_l = [&] {  // c6 r^3 + r^2 + 2 r + 4/3;  0.5 r^2 + 2 r + 2
    N = ((dwk(C6) * r + dw_make(1.f, 0.f)) * r + dw_make(2.f, 0.f)) * r + dwk(F3);
    dN = add_f(add_f(dw_scale(r, 0.5f), 2.f) * r, 2.f);
  };
  auto outer_r = [&] {  // -c6 r^3 + r^2 - 2 r + 4/3;  -0.5 r^2 + 2 r - 2
    N = ((add_f(-(dwk(C6) * r), 1.f)) * r + dw_make(-2.f, 0.f)) * r + dwk(F3);
    dN = add_f(add_f(dw_scale(r, -0.5f), 2.f) * r, -2.f);
  };
  if (t == 1) {
    if (dw_lt(r, -2.f) || !dw_le(r, 2.f)) return;
    if (dw_le(r, -1.f)) outer_l();
    else if (dw_le(r, 0.f)) {  // -c6 r^3 + r + 1;  -0.5 r^2 + 1
      N = add_f(add_f(-(dwk(C6) * r2), 1.f) * r, 1.f);
      dN = add_f(dw_scale(r2, -0.5f), 1.f);
    } else if (dw_le(r, 1.f)) {  // c6 r^3 - r + 1;  0.5 r^2 - 1
      N = add_f(add_f(dwk(C6) * r2, -1.f) * r, 1.f);
      dN = add_f(dw_scale(r2, 0.5f), -1.f);
    } else {
      outer_r();
    }
  } else if (t == 2) {
    if (dw_lt(r, -1.f) || !dw_le(r, 2.f)) return;
    if (dw_le(r, 0.f)) {  // -c3 r^3 - r^2 + t3;  -r^2 - 2 r
      N = (add_f(-(dwk(C3) * r), -1.f) * r2) + dwk(T3);
      dN = add_f(-r, -2.f) * r;
    } else if (dw_le(r, 1.f)) {  // 0.5 r^3 - r^2 + t3;  1.5 r^2 - 2 r
      N = (add_f(dw_scale(r, 0.5f), -1.f) * r2) + dwk(T3);
      dN = add_f(r * 1.5f, -2.f) * r;
    } else {
      outer_r();
    }
  } else if (t == 3) {
    if (dw_lt(r, -2.f) || !dw_le(r, 2.f)) return;
    if (dw_le(r, -1.f)) outer_l();
    else if (dw_le(r, 0.f)) {  // -0.5 r^3 - r^2 + t3;  -1.5 r^2 - 2 r
      N = (add_f(dw_scale(r, -0.5f), -1.f) * r2) + dwk(T3);
      dN = add_f(r * -1.5f, -2.f) * r;
    } else if (dw_le(r, 1.f)) {
      N = (add_f(dw_scale(r, 0.5f), -1.f) * r2) + dwk(T3);
      dN = add_f(r * 1.5f, -2.f) * r;
    } else {
      outer_r();
    }
  } else {
    if (dw_lt(r, -2.f) || !dw_le(r, 1.f)) return;
    if (dw_le(r, -1.f)) outer_l();
    else if (dw_le(r, 0.f)) {
      N = (add_f(dw_scale(r, -0.5f), -1.f) * r2) + dwk(T3);
      dN = add_f(r * -1.5f, -2.f) * r;
    } else {  // c3 r^3 - r^2 + 0.6666666667;  r^2 - 2 r
      N = (add_f(dwk(C3) * r, -1.f) * r2) + dwk(T4);
      dN = add_f(r, -2.f) * r;
    }
  }
}

// bs_axes<3, K> with double-word values: the same first node, spline types
// and FP64 distances, the values and derivatives in double-word
template <int K>
__device__ __forceinline__ bool bs_axes_dw(const GridP& g, const double* x, BsAxisDW<K>* ax) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int64_t nn = g.nn[a];
    const double num = K == 3 ? __dmul_rn(x[a], g.dxI[a]) : __dmul_rn(__dsub_rn(x[a], g.xmin[a]), g.dxI[a]);
    const double rem = __dsub_rn(num, floor(num));
    const double fb = floor(__dadd_rn(num, 1.0));
    if (!(fb >= 1.0) || !(fb <= double(nn - 1))) return false;
    const int64_t ib = int64_t(fb);
    int64_t f1;
    if (K == 3) f1 = ib == 1 ? ib : (ib == nn - 1 ? ib - 1 : (rem < 0.5 ? ib - 1 : ib));
    else f1 = ib == 1 ? 1 : (ib == nn - 1 ? ib - 2 : ib - 1);
    ax[a].first = f1 - 1;
    const dw dxI = dw_c(g.w_dxI[a]);
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int64_t id = f1 + i;
      const double r = a == 0 ? __dmul_rn(__dsub_rn(x[0], g.coord[0][id - 1]), g.dxI[0])
                              : __dmul_rn(__dsub_rn(x[a], __dmul_rn(double(id - 1), g.dx[a])), g.dxI[a]);
      const int t = (id == 1 || id == nn) ? 1 : (id == 2 ? 2 : (id == nn - 1 ? 4 : 3));
      dw dNr;
      if (K == 3) quad_bs_dw(t, dw_from(r), ax[a].N[i], dNr);
      else cubic_bs_dw(t, dw_from(r), ax[a].N[i], dNr);
      ax[a].G[i] = dNr * dxI;
    }
  }
  return true;
}

// P2G over the support, as bs_p2g_kernel in 3D (per (i, j) the force
// coefficients P_a = s_a0 Gx Ny + s_a1 Nx Gy (+ m g_a Nxy), Q_a = s_a2 Nxy with
// s = -V sigma, and f_a = Nz P_a + Gz Q_a at each k), in double-word; each node
// value rounded to FP64 by one FP64 add and added by one FP64 atomic at L2
template <int K, bool GRAV>
__global__ void __launch_bounds__(256) bs_p2g_dw_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy, double gz,
                                                        unsigned* status) {
  using L = Layout<3>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) x[a] = *field<double>(pp, L::X + a, p);
  BsAxisDW<K> ax[3];
  if (!bs_axes_dw<K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  if (nd.bflag) {
    BsAxis<K> ab[3];  // the support's first nodes, for the block flags
#pragma unroll
    for (int a = 0; a < 3; ++a) ab[a].first = ax[a].first;
    bs_mark<3, K>(nd, ab);
  }
  const dw m = get_dw(pp, L::M, p), V = get_dw(pp, L::VOL, p);
  const double grav[3] = {gx, gy, gz};
  dw v[3], mg[3], ms[6];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    v[a] = get_dw(pp, L::V + a, p);
    if (GRAV) mg[a] = m * dw_from(grav[a]);
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) ms[c] = -(V * get_dw(pp, L::SIG + c, p));
  dw mNz[K];
#pragma unroll
  for (int k = 0; k < K; ++k) mNz[k] = m * ax[2].N[k];
  const int64_t Nn = nd.nodeCount;
#pragma unroll 1
  for (int i = 0; i < K; ++i)
#pragma unroll 1
    for (int j = 0; j < K; ++j) {
      const dw Nxy = ax[0].N[i] * ax[1].N[j];
      const dw GxNy = ax[0].G[i] * ax[1].N[j];
      const dw NxGy = ax[0].N[i] * ax[1].G[j];
      dw P[3], Q[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        P[a] = dw_fma(ms[sym<3>(a, 1)], NxGy, ms[sym<3>(a, 0)] * GxNy);
        if (GRAV) P[a] = dw_fma(mg[a], Nxy, P[a]);
        Q[a] = ms[sym<3>(a, 2)] * Nxy;
      }
      const int64_t nij = (ax[0].first + i) + g.nx * (ax[1].first + j) + g.nxy * ax[2].first;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int64_t n = nij + g.nxy * k;
        const dw Nm = Nxy * mNz[k];
        atomicAdd(nd.m + n, dw_to_f64(Nm));
#pragma unroll
        for (int a = 0; a < 3; ++a) atomicAdd(nd.p0 + a * Nn + n, dw_to_f64(Nm * v[a]));
#pragma unroll
        for (int a = 0; a < 3; ++a)
          atomicAdd(nd.f + a * Nn + n, dw_to_f64(dw_fma(P[a], ax[2].N[k], Q[a] * ax[2].G[k])));
      }
    }
}

// the particle field of DwSlots slot k (MAT's fifth group: plastic strain for
// J2, stress for linear elastic)
template <int MAT>
__device__ __forceinline__ int dw_slot_field(int k) {
  using L = Layout<3>;
  using S = DwSlots;
  return k < S::V ? L::X + k
                  : (k < S::F ? L::V + (k - S::V)
                              : (k < S::EPS ? L::F + (k - S::F)
                                            : (k < S::EP ? L::EPS + (k - S::EPS)
                                                         : (k < S::ALPHA ? (MAT == MPM_MAT_J2 ? L::EP : L::SIG) +
                                                                               (k - S::EP)
                                                                         : L::ALPHA))));
}

// G2P over the support, as bs_g2p_kernel in 3D (per (i, j) the node values
// contracted along z with Nz and Gz first), in double-word, then dw_finish
template <int K, int MAT>
__global__ void __launch_bounds__(256) bs_g2p_dw_kernel(GridP g, NodeP nd, PartP pp, MatParams mp, unsigned* status) {
  using L = Layout<3>;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= pp.count) return;
  const int64_t p = pp.begin + t;
  double x[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) x[a] = *field<double>(pp, L::X + a, p);
  BsAxisDW<K> ax[3];
  if (!bs_axes_dw<K>(g, x, ax)) {
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  dw_acc dx[3], dvp[3], Ld[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dx[a] = dvp[a] = dw_acc{0.f, 0.f};
#pragma unroll
    for (int b = 0; b < 3; ++b) Ld[a][b] = dw_acc{0.f, 0.f};
  }
#pragma unroll 1
  for (int o = 0; o < K * K; ++o) {
    const int i = o / K, j = o % K;
    const dw No = ax[0].N[i] * ax[1].N[j];
    const dw Go0 = ax[0].G[i] * ax[1].N[j];
    const dw Go1 = ax[0].N[i] * ax[1].G[j];
    const int64_t no = (ax[0].first + i) + g.nx * (ax[1].first + j) + g.nxy * ax[2].first;
    dw_acc Z0[3], Z1[3], W[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) Z0[a] = Z1[a] = W[a] = dw_acc{0.f, 0.f};
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const NodeDW r = node_dw(nd.dw4, no + g.nxy * k);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        acc_fma(Z0[a], ax[2].N[k], r.vd[a]);
        acc_fma(Z1[a], ax[2].G[k], r.vd[a]);
        acc_fma(W[a], ax[2].N[k], r.dv[a]);
      }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const dw z0 = acc_value(Z0[a]);
      acc_fma(dx[a], No, z0);
      acc_fma(dvp[a], No, acc_value(W[a]));
      acc_fma(Ld[a][0], Go0, z0);
      acc_fma(Ld[a][1], Go1, z0);
      acc_fma(Ld[a][2], No, acc_value(Z1[a]));
    }
  }
  dw dxv[3], dvv[3], Ldt[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dxv[a] = acc_value(dx[a]);
    dvv[a] = acc_value(dvp[a]);
#pragma unroll
    for (int b = 0; b < 3; ++b) Ldt[a][b] = acc_value(Ld[a][b]);
  }
  dw_finish<MAT>(pp, p, mp, status, [&](int k) -> double { return *field<double>(pp, dw_slot_field<MAT>(k), p); },
                 dxv, dvv, Ldt);
}

}  // namespace jmpm
