// mpm_step_dw.cuh -- the P2G and G2P of an MPM_PREC_DW context in
// double-word FP32 arithmetic (mpm_dw.cuh), for 3D bodies on the linear hat
// basis: the P2G of SolveExplicitSolidMechanics3D.jl:230-378 (the 2D lines
// SolveExplicitSolidMechanics2D.jl:391-423 it follows), the G2P with the
// velocity-gradient, F, volume and strain updates (:485-530) and the
// constitutive update of Material.jl (linear elastic :68-81, J2 :228-275).
//
// The particle fields stay FP64 in HBM.  A field the step accumulates
// (position, velocity, F, strain, plastic strain, alpha) is stored as its FP64
// value plus the step's DW increment rounded to FP64, so the state keeps its
// 53 bits and only the increment carries the DW rounding; the stress is the
// FP64 value of its DW result, and V = J V0 that of J V0 with det F in DW.
// Loads convert FP64 -> DW on the integer pipe.  The P2G's hat has the FP64
// hat's cell and zero gradient factors bit for bit and its weights in DW
// (hat_dw, stored for the G2P in the hat cache as DW pairs); its node values
// are DW, each added to its FP64 node accumulator as an FP64 value.  The grid
// update writes each node's vdt and dv as DW records (NodeP::dw4, three float4
// per node), so the G2P's corner gathers need no conversion.  The G2P's
// particle inputs are copied into the thread's shared-memory slots by cp.async
// at the start, so their loads overlap the gather; its tail (dw_finish) is
// shared with the B-spline G2P of mpm_bspline_dw.cuh.
#pragma once

#include "mpm_kernels.cuh"

namespace jmpm {

// The hat of particle p from the cache the P2G of this step stored (hat_dw):
// base cells, hat values at the lower and upper node, and the gradient factors
// as signs (gl = sl dxI, gh = sh dxI with sl, sh in {-1, 0, +1}).  False when
// the P2G found the particle outside.
struct HatDW {
  int c[3];
  dw Nl[3], Nh[3];
  float sl[3], sh[3];
};

// the sign of an FP64 gradient factor or coordinate difference as a float
__device__ __forceinline__ float sign_of(double gfac) {
  return is_zero_bits(gfac) ? 0.f : (is_neg_bits(gfac) ? -1.f : 1.f);
}

// The hat of particle p at position x (FP64) for the DW step: the cell the
// FP64 hat() chooses, bit for bit (base_node_estimate, else the FP64
// expression, as hat() decides it) -- the differences
// dl = x - x_lower, dh = x - x_upper in FP64 (exact, as in hat()), their signs
// for the gradient factors, and Nl = 1 - |dl| dxI, Nh = 1 - Nl in DW.
// The cache (PartP::hat_c codes, hat_nl as DW pairs) is written for the G2P.
__device__ __forceinline__ bool hat_dw(const GridP& g, const PartP& pp, int64_t p, const double* x, HatDW& h) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int i1;
    if (!base_node_estimate(x[a], g.xminf[a], g.dxIf[a], i1)) i1 = base_node_f64(x[a], g.xmin[a], g.dxI[a]);
    if (i1 < 1 || i1 > int(g.nn[a] - 1)) {
      if (pp.hat_c)
#pragma unroll
        for (int b = 0; b < 3; ++b) pp.hat_c[b * pp.pitch + p] = -1;
      return false;
    }
    const int c = i1 - 1;
    h.c[a] = c;
    const double dl = sub_rn(x[a], g.coord[a][c]), dh = sub_rn(x[a], g.coord[a][c + 1]);
    h.sl[a] = -sign_of(dl);
    h.sh[a] = -sign_of(dh);
    h.Nl[a] = dw_one_minus(dw_from(fabs(dl)) * dw_c(g.w_dxI[a]));
    h.Nh[a] = dw_one_minus(h.Nl[a]);
  }
  if (pp.hat_c) {
    float2* nl = static_cast<float2*>(pp.hat_nl);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      pp.hat_c[a * pp.pitch + p] = h.c[a] | (int32_t(h.sl[a] == 0.f) << 27) | (int32_t(h.sl[a] < 0.f) << 28) |
                                   (int32_t(h.sh[a] == 0.f) << 29) | (int32_t(h.sh[a] < 0.f) << 30);
      nl[a * pp.pitch + p] = make_float2(h.Nl[a].hi, h.Nl[a].lo);
    }
  }
  return true;
}

// The hat the P2G of this step cached (hat_dw), or, without a cache, hat_dw
// of the position.  False when the particle is outside.
__device__ __forceinline__ bool hat_get_dw(const GridP& g, const PartP& pp, int64_t p, HatDW& h) {
  if (!pp.hat_c) {
    double x[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) x[a] = *field<double>(pp, Layout<3>::X + a, p);
    return hat_dw(g, pp, p, x, h);
  }
  const float2* nl = static_cast<const float2*>(pp.hat_nl);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int32_t code = pp.hat_c[a * pp.pitch + p];
    if (code < 0) return false;
    h.c[a] = code & ((1 << 27) - 1);
    const float2 w = nl[a * pp.pitch + p];
    h.Nl[a] = dw_make(w.x, w.y);
    h.Nh[a] = dw_one_minus(h.Nl[a]);
    h.sl[a] = ((code >> 27) & 1) ? 0.f : (((code >> 28) & 1) ? -1.f : 1.f);
    h.sh[a] = ((code >> 29) & 1) ? 0.f : (((code >> 30) & 1) ? -1.f : 1.f);
  }
  return true;
}

// one corner's DW record: vdt (3) and dv (3)
struct NodeDW {
  dw vd[3], dv[3];
};

__device__ __forceinline__ NodeDW node_dw(const float4* r, int64_t n) {
  const float4 a = __ldg(r + 3 * n), b = __ldg(r + 3 * n + 1), c = __ldg(r + 3 * n + 2);
  NodeDW o;
  o.vd[0] = dw_make(a.x, a.y);
  o.vd[1] = dw_make(a.z, a.w);
  o.vd[2] = dw_make(b.x, b.y);
  o.dv[0] = dw_make(b.z, b.w);
  o.dv[1] = dw_make(c.x, c.y);
  o.dv[2] = dw_make(c.z, c.w);
  return o;
}

__device__ __forceinline__ void put_f64(const PartP& pp, int f, int64_t p, double v) { *field<double>(pp, f, p) = v; }
__device__ __forceinline__ dw get_dw(const PartP& pp, int f, int64_t p) { return dw_from(*field<double>(pp, f, p)); }

// ---------------------------------------------------------------------------
// P2G of particle pp.begin + t: mass m N, momentum m N v and force
// -V sigma grad N + m g N at its 8 corners, one FP64 atomic per value at L2.
// Factored along z as p2g_corner_values: per (x, y) corner pair
// P_a = c_a0 sx Ny + c_a1 sy Nx (+ m g_a Nx Ny) and Q_a = c_a2 Nx Ny, with
// c_ab = -V sigma_ab dxI_b and the gradient signs s in {-1, 0, +1}, give the
// force f_a = Nz P_a + sz Q_a at both z corners.
template <bool GRAV>
__device__ __forceinline__ void p2g_dw_particle(const GridP& g, const NodeP& nd, const PartP& pp, int64_t t,
                                                const dw (&grav)[3], unsigned* status) {
  using L = Layout<3>;
  const int64_t p = pp.begin + t;
  double xd[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) xd[a] = *field<double>(pp, L::X + a, p);
  HatDW h;
  if (!hat_dw(g, pp, p, xd, h)) {  // cached for the G2P of this step
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  if (nd.bflag) mark_blocks<3>(nd, h.c);
  const dw(&Nl)[3] = h.Nl, (&Nh)[3] = h.Nh;
  const float(&sl)[3] = h.sl, (&sh)[3] = h.sh;
  const dw m = dw_from(*field<double>(pp, L::M, p)), V = dw_from(*field<double>(pp, L::VOL, p));
  dw v[3], cs[3][3], mg[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    v[a] = dw_from(*field<double>(pp, L::V + a, p));
    if (GRAV) mg[a] = m * grav[a];
  }
  {
    dw ms[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) ms[c] = -(V * dw_from(*field<double>(pp, L::SIG + c, p)));  // -V sigma
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) cs[a][b] = ms[sym<3>(a, b)] * dw_c(g.w_dxI[b]);
  }
  const dw mNz[2] = {m * Nl[2], m * Nh[2]};
  const int64_t Nn = nd.nodeCount;
  const int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + g.nxy * int64_t(h.c[2]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int bx = q & 1, by = q >> 1;
    const dw Nx = bx ? Nh[0] : Nl[0], Ny = by ? Nh[1] : Nl[1];
    const dw Nxy = Nx * Ny;
    const dw sNy = dw_scale(Ny, bx ? sh[0] : sl[0]), sNx = dw_scale(Nx, by ? sh[1] : sl[1]);
    dw P[3], Q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      P[a] = dw_fma(cs[a][1], sNx, cs[a][0] * sNy);
      if (GRAV) P[a] = dw_fma(mg[a], Nxy, P[a]);
      Q[a] = cs[a][2] * Nxy;
    }
#pragma unroll
    for (int bz = 0; bz < 2; ++bz) {
      const dw Nz = bz ? Nh[2] : Nl[2];
      const float sz = bz ? sh[2] : sl[2];
      const int64_t n = base + bx + g.nx * by + g.nxy * bz;
      const dw Nm = Nxy * mNz[bz];
      atomicAdd(nd.m + n, dw_to_f64(Nm));
#pragma unroll
      for (int a = 0; a < 3; ++a) atomicAdd(nd.p0 + a * Nn + n, dw_to_f64(Nm * v[a]));
#pragma unroll
      for (int a = 0; a < 3; ++a)
        atomicAdd(nd.f + a * Nn + n, dw_to_f64(dw_fma(P[a], Nz, dw_scale(Q[a], sz))));
    }
  }
}

// three CTAs of 256 threads per SM (80 registers, ~100 B of spills): 0.120 ->
// 0.114 ms on the Taylor bar
template <bool GRAV>
__global__ void __launch_bounds__(256, 3) p2g_dw_kernel(GridP g, NodeP nd, PartP pp, double gx, double gy, double gz,
                                                     unsigned* status) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const dw grav[3] = {dw_from(gx), dw_from(gy), dw_from(gz)};
  if (t < pp.count) p2g_dw_particle<GRAV>(g, nd, pp, t, grav, status);
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

// shared-memory slots of a particle's inputs (stride blockDim.x doubles):
// x (3), v (3), F (9), strain (6), J2: plastic strain (6) and alpha / linear
// elastic: stress (6)
struct DwSlots {
  static constexpr int X = 0, V = 3, F = 6, EPS = 15, EP = 21, SIG = 21, ALPHA = 27, N = 28;
};

// The G2P after the gather, shared by the bases: x and v (their FP64 values
// plus the DW increments dx, dv), F <- F + F (L dt) (:523), J = det F and
// V = J V0 (:525-526), the strain and the constitutive update.  in(k) is the
// particle's FP64 input of DwSlots slot k.
template <int MAT, class In>
__device__ __forceinline__ void dw_finish(const PartP& pp, int64_t p, const MatParams& mp, unsigned* status, In&& in,
                                          const dw (&dx)[3], const dw (&dvp)[3], const dw (&Ldt)[3][3]) {
  using L = Layout<3>;
  using S = DwSlots;
  bool fin = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double xd = f64_plus_dw(in(S::X + a), dx[a]), vd = f64_plus_dw(in(S::V + a), dvp[a]);
    put_f64(pp, L::X + a, p, xd);
    put_f64(pp, L::V + a, p, vd);
    fin &= finite_bits(xd) & finite_bits(vd);
  }
  // F <- F + F (L dt) (:523), J = det F and V = J V0 (:525-526)
  dw J;
  {
    dw F[9], Fn[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) F[c] = dw_from(in(S::F + c));
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        dw s = F[i] * Ldt[0][j];
#pragma unroll
        for (int k = 1; k < 3; ++k) s = dw_fma(F[i + 3 * k], Ldt[k][j], s);
        put_f64(pp, L::F + i + 3 * j, p, f64_plus_dw(in(S::F + i + 3 * j), s));
        Fn[i + 3 * j] = F[i + 3 * j] + s;
      }
    // det = col0 . (col1 x col2), as det_d (column-major F)
    const dw c0 = dw_fma(Fn[4], Fn[8], -(Fn[5] * Fn[7]));
    const dw c1 = dw_fma(Fn[5], Fn[6], -(Fn[3] * Fn[8]));
    const dw c2 = dw_fma(Fn[3], Fn[7], -(Fn[4] * Fn[6]));
    J = dw_fma(Fn[2], c2, dw_fma(Fn[1], c1, Fn[0] * c0));
  }
  put_f64(pp, L::VOL, p, dw_to_f64(J * dw_from(*field<double>(pp, L::VOL0, p))));
  // strain += dt * 0.5 (L + L')
  dw eps[6];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      const int c = sym<3>(i, j);
      const dw de = (i == j) ? Ldt[i][i] : dw_scale(Ldt[i][j] + Ldt[j][i], 0.5f);
      const double e0 = in(S::EPS + c);
      eps[c] = dw_from(e0) + de;
      put_f64(pp, L::EPS + c, p, f64_plus_dw(e0, de));
    }
  dw lam = dw_c(mp.w_lambda), mu = dw_c(mp.w_mu), kappa = dw_c(mp.w_kappa);
  if (mp.per_particle) {
    lam = dw_from(*field<double>(pp, L::LAM, p));
    mu = dw_from(*field<double>(pp, L::MU, p));
    kappa = lam + mu;
  }
  const dw tmu = dw_scale(mu, 2.f);
  const dw tr = (eps[0] + eps[1]) + eps[2];
  dw sig[6];
  if (MAT == MPM_MAT_ELASTIC) {
    // vmStr of the incoming stress (Material.jl:78-79), then
    // lambda (tr eps) I + 2 mu eps (:68-72, 80)
    dw so[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) so[c] = dw_from(in(S::SIG + c));
    const dw qv = ((dw_sqr(so[0]) + dw_sqr(so[1])) + dw_sqr(so[2])) +
                  dw_scale((dw_sqr(so[3]) + dw_sqr(so[5])) + dw_sqr(so[4]), 2.f);
    put_f64(pp, L::VM, p, dw_to_f64(dw_sqrt(qv)));
    const dw lt = lam * tr;
#pragma unroll
    for (int c = 0; c < 6; ++c) sig[c] = c < 3 ? dw_fma(tmu, eps[c], lt) : tmu * eps[c];
  } else {
    // J2 radial return (Material.jl:228-275), as j2_3d
    dw ep[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) ep[c] = dw_from(in(S::EP + c));
    const dw tt = tr * dw_c(mp.w_third);
    dw s[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) s[c] = tmu * ((c < 3 ? eps[c] - tt : eps[c]) - ep[c]);
    const dw qv = ((dw_sqr(s[0]) + dw_sqr(s[1])) + dw_sqr(s[2])) +
                  dw_scale((dw_sqr(s[3]) + dw_sqr(s[4])) + dw_sqr(s[5]), 2.f);
    const dw ns = dw_sqrt(qv);
    const dw kt = kappa * tr;
    const dw k1 = dw_c(mp.w_k1);
    const double a0d = in(S::ALPHA);
    const dw a0 = dw_from(a0d);
    const dw f_trial = ns - dw_fma(k1, a0, dw_c(mp.w_fy));
#pragma unroll
    for (int c = 0; c < 6; ++c) sig[c] = c < 3 ? s[c] + kt : s[c];
    if (dw_pos(f_trial)) {
      // plastic: the increments of alpha and the plastic strain go to their FP64 values
      const dw inv = dw_recip(ns);
      const dw lamp = mp.per_particle ? f_trial * dw_recip(tmu + k1) : f_trial * dw_c(mp.w_rtmuk1);
      const dw cc = tmu * lamp;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const dw nrm = inv * s[c];
        put_f64(pp, L::EP + c, p, f64_plus_dw(in(S::EP + c), lamp * nrm));
        sig[c] = dw_fma(-cc, nrm, sig[c]);
      }
      put_f64(pp, L::ALPHA, p, f64_plus_dw(a0d, lamp));
    }
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const double sd = dw_to_f64(sig[c]);
    put_f64(pp, L::SIG + c, p, sd);
    fin &= finite_bits(sd);
  }
  const unsigned st = (dw_pos(J) ? 0u : ST_NEGATIVE_J) | (fin ? 0u : ST_NONFINITE);
  if (st) atomicOr(status, st);
}

// MAT: MPM_MAT_J2 or MPM_MAT_ELASTIC; pre: this thread's first slot
template <int MAT>
__device__ __forceinline__ void g2p_dw_particle(const GridP& g, const NodeP& nd, const PartP& pp, int64_t t,
                                                const MatParams& mp, unsigned* status, double* pre) {
  using L = Layout<3>;
  using S = DwSlots;
  const int bs = blockDim.x;
  const int64_t p = pp.begin + t;
  auto slot = [&](int k) -> double& { return pre[k * bs]; };
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    cp_async8(&slot(S::X + a), field<double>(pp, L::X + a, p));
    cp_async8(&slot(S::V + a), field<double>(pp, L::V + a, p));
  }
#pragma unroll
  for (int c = 0; c < 9; ++c) cp_async8(&slot(S::F + c), field<double>(pp, L::F + c, p));
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    cp_async8(&slot(S::EPS + c), field<double>(pp, L::EPS + c, p));
    cp_async8(&slot(S::EP + c), field<double>(pp, (MAT == MPM_MAT_J2 ? L::EP : L::SIG) + c, p));
  }
  if (MAT == MPM_MAT_J2) cp_async8(&slot(S::ALPHA), field<double>(pp, L::ALPHA, p));
  HatDW h;
  if (!hat_get_dw(g, pp, p, h)) {
    cp_async_wait_all();  // no copy into this CTA's shared memory outlives the thread
    atomicOr(status, ST_OUT_OF_GRID);
    return;
  }
  const int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]) + g.nxy * int64_t(h.c[2]);
  // increments of x and v, and the gradient sums
  dw_acc dx[3], dvp[3], Ls[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dx[a] = dvp[a] = dw_acc{0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 3; ++j) Ls[a][j] = dw_acc{0.f, 0.f};
  }
  // factored along z as in g2p_particle: per (x, y) corner pair
  // Z0 = vd0 + Nh_z (vd1 - vd0), Z1 = sl_z vd0 + sh_z vd1 (= vd1 - vd0 strictly
  // inside the cell), W = Nl_z dv0 + Nh_z dv1; then x += Nx Ny Z0,
  // v += Nx Ny W and the gradient sums in units of dxI:
  // (sx Ny Z0, sy Nx Z0, Nx Ny Z1), scaled by dxI once at the end
  const bool inz = h.sl[2] < 0.f && h.sh[2] > 0.f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int bx = q & 1, by = q >> 1;
    const int64_t n0 = base + bx + g.nx * by;
    const NodeDW r0 = node_dw(nd.dw4, n0), r1 = node_dw(nd.dw4, n0 + g.nxy);
    const dw Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1];
    const dw Nxy = Nx * Ny;
    const dw sNy = dw_scale(Ny, bx ? h.sh[0] : h.sl[0]), sNx = dw_scale(Nx, by ? h.sh[1] : h.sl[1]);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const dw dz = r1.vd[a] - r0.vd[a];
      const dw Z0 = dw_fma(h.Nh[2], dz, r0.vd[a]);
      dw Z1 = dz;
      if (!inz) Z1 = dw_scale(r0.vd[a], h.sl[2]) + dw_scale(r1.vd[a], h.sh[2]);
      const dw W = dw_fma(h.Nh[2], r1.dv[a], h.Nl[2] * r0.dv[a]);
      acc_fma(dx[a], Nxy, Z0);
      acc_fma(dvp[a], Nxy, W);
      acc_fma(Ls[a][0], sNy, Z0);
      acc_fma(Ls[a][1], sNx, Z0);
      acc_fma(Ls[a][2], Nxy, Z1);
    }
  }
  cp_async_wait_all();
  dw dxv[3], dvv[3], Ldt[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dxv[a] = acc_value(dx[a]);
    dvv[a] = acc_value(dvp[a]);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const dw s = dw_c(g.w_dxI[j]);
#pragma unroll
    for (int a = 0; a < 3; ++a) Ldt[a][j] = acc_value(Ls[a][j]) * s;
  }
  dw_finish<MAT>(pp, p, mp, status, slot, dxv, dvv, Ldt);
}

// dynamic shared memory: DwSlots::N doubles per thread
template <int MAT>
__global__ void __launch_bounds__(256, 2) g2p_dw_kernel(GridP g, NodeP nd, PartP pp, MatParams mp, unsigned* status) {
  extern __shared__ __align__(16) unsigned char g2p_dw_smem[];
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < pp.count)
    g2p_dw_particle<MAT>(g, nd, pp, t, mp, status, reinterpret_cast<double*>(g2p_dw_smem) + threadIdx.x);
}

}  // namespace jmpm
