// mpm_adjoint.cuh -- reverse-mode (adjoint) kernels of one USL step, FP64,
// single velocity field, neo-Hookean, linear elastic and J2 bodies, D = 2, 3.
// The neo-Hookean stress is a function of F, so its P2G adjoint maps the
// stress adjoint onto F directly (below).  The elastic and J2 stresses are
// particle state formed by the previous G2P's update_stress!: the P2G adjoint
// stores the stress adjoint, and the previous step's G2P adjoint runs it back
// through the constitutive update (stress_adj) onto the strain, the plastic
// state and the moduli.
//
// State of a step n: (x, v, F) per particle, with sigma = NH(F; lambda_p,
// mu_p) and V = det(F) V0 derived from F.  The forward step (mpm_kernels.cuh)
//   P2G   m_I = sum w m_p,  p0_I = sum w m_p v_p,  f_I = sum (-V sigma g + m_p b w)
//   grid  vdt = dt (p0 + dt f)/m,  dv = dt f/m   (free dofs of nodes with m > tol)
//   G2P   v' = v + sum w dv,  x' = x + sum w vdt,  Ldt = sum vdt (x) g,
//         F' = F (I + Ldt)
// is differentiated exactly within the particles' current cells: w = N(x),
// g = grad N(x), H = grad grad N(x) (zero diagonal for the hat product).
// Reverse of step n, given the adjoints (x', v', F') of step n + 1:
//   g2p_adj   F_ = F' (I + Ldt)^T,  Abar = F^T F',  scatter vdt_I += w x' + Abar g,
//             dv_I += w v',  x_ = x' + sum (w_ g + H g_)   (w_ = x'.vdt + v'.dv,
//             g_ = Abar^T vdt)
//   grid_adj  p0_ = dt vdt_/m,  f_ = dt (dt vdt_ + dv_)/m,  m_ = -sum (vdt_ vdt + dv_ dv)/m
//   p2g_adj   w_ = m_p (m_ + v.p0_ + b.f_),  v_ += m_p sum w p0_,  g_ = -V sigma^T f_,
//             sigma_ = -V sum f_ (x) g,  V_ = -sum f_.(sigma g);  then
//             F_ += dNH/dF^T sigma_ + V_ V0 J F^-T,  E_ += c1 lambda_ + c2 mu_
// (c1 = dlambda/dE, c2 = dmu/dE).  Trailing underscore = adjoint.
#pragma once

#include "mpm_common.cuh"

namespace jmpm {

// particle adjoints, SoA (component-major) with pitch = particle count:
// x_ (D) | v_ (D) | F_ (D*D, column-major) | E_ (1), and for the materials whose
// stress is state (linear elastic, J2): strain_ (S) | sigma_ (S) | pstrain_ (S)
// | alpha_ (1), adjoints of the stored symmetric components
template <int D>
struct AdjLayout {
  static constexpr int S = (D == 2) ? 3 : 6;
  static constexpr int XB = 0, VB = D, FB = 2 * D, EB = 2 * D + D * D;
  static constexpr int EPSB = EB + 1, SIGB = EPSB + S, EPB = SIGB + S, ALB = EPB + S;
  static constexpr int NF = ALB + 1;
};

struct AdjP {
  double* base;
  int64_t pitch;
};

// node adjoints: vdt_ (D) | dv_ (D) accumulated by g2p_adj; m_ | p0_ (D) | f_ (D) from grid_adj
struct NodeAdjP {
  double* vdtb;
  double* dvb;
  double* mb;
  double* p0b;
  double* fb;
  int64_t nodeCount;
};

// forward grid outputs recorded for step n: m | vdt (D) | dv (D), component-major
struct GridRec {
  const double* m;
  const double* vdt;
  const double* dv;
};

template <int D>
struct CornersFull {
  int64_t node[1 << D];
  double N[1 << D];
  double g[1 << D][D];
  double H[1 << D][3];  // xy, xz, yz
};

template <int D>
__device__ __forceinline__ void corners_full(const GridP& gp, const Hat<D, double>& h, CornersFull<D>& c) {
  int64_t base = int64_t(h.c[0]) + gp.nx * int64_t(h.c[1]);
  if constexpr (D == 3) base += gp.nxy * int64_t(h.c[2]);
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    const double Nx = bx ? h.Nh[0] : h.Nl[0], gx = bx ? h.gh[0] : h.gl[0];
    const double Ny = by ? h.Nh[1] : h.Nl[1], gy = by ? h.gh[1] : h.gl[1];
    if constexpr (D == 2) {
      c.N[k] = Nx * Ny;
      c.g[k][0] = gx * Ny;
      c.g[k][1] = Nx * gy;
      c.H[k][0] = gx * gy;
      c.H[k][1] = c.H[k][2] = 0.0;
      c.node[k] = base + bx + gp.nx * by;
    } else {
      const double Nz = bz ? h.Nh[2] : h.Nl[2], gz = bz ? h.gh[2] : h.gl[2];
      c.N[k] = Nx * Ny * Nz;
      c.g[k][0] = gx * Ny * Nz;
      c.g[k][1] = Nx * gy * Nz;
      c.g[k][2] = Nx * Ny * gz;
      c.H[k][0] = gx * gy * Nz;
      c.H[k][1] = gx * Ny * gz;
      c.H[k][2] = Nx * gy * gz;
      c.node[k] = base + bx + gp.nx * by + gp.nxy * bz;
    }
  }
}

// x_ += w_ g + H g_
template <int D>
__device__ __forceinline__ void add_shape_adj(double* xb, const CornersFull<D>& c, int k, double wb, const double* gb) {
#pragma unroll
  for (int a = 0; a < D; ++a) xb[a] += wb * c.g[k][a];
  xb[0] += c.H[k][0] * gb[1];
  xb[1] += c.H[k][0] * gb[0];
  if constexpr (D == 3) {
    xb[0] += c.H[k][1] * gb[2];
    xb[2] += c.H[k][1] * gb[0];
    xb[1] += c.H[k][2] * gb[2];
    xb[2] += c.H[k][2] * gb[1];
  }
}

template <int D>
__device__ __forceinline__ double* adj(const AdjP& ad, int f, int64_t p) {
  return ad.base + int64_t(f) * ad.pitch + p;
}

// ---------------------------------------------------------------------------
// Reverse of update_stress! for the materials whose stress is particle state
// (linear elastic, Material.jl:68-81; J2 radial return, :174-275), at the
// strain eps' = eps + sym(L dt) the forward G2P formed.  In: the adjoints of its
// outputs sigma' (sb), alpha' (ab), pstrain' (pb) in stored symmetric
// components; out: the adjoint of eps' (added to eb), of the incoming pstrain
// and alpha (written to pb, ab), and of the moduli (G = 2 mu, lambda, kappa)
// as dL/dmu and dL/dlambda.  Forward as in mpm_kernels.cuh (j2_3d: deviator
// with 0.333333333, |s| = sqrt(sum w s^2) with w = 2 off the diagonal,
// kappa = lambda + mu, linear hardening k1; j2_2d: the Voigt form).
template <int D, int MAT>
__device__ __forceinline__ void stress_adj(const double* eps, double lam, double mu, const MatParams& mp,
                                           const double* ep_in, double alpha_in, const double* sb, double* eb,
                                           double* pb, double& ab, double& mub, double& lamb) {
  constexpr int S = Layout<D>::S;
  const double G = 2.0 * mu;
  if (MAT == MPM_MAT_ELASTIC) {
    // sigma_c = G eps_c + lambda tr (c < D)
    double tr = 0.0, strb = 0.0, Gb = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      tr += eps[c];
      strb += sb[c];
    }
#pragma unroll
    for (int c = 0; c < S; ++c) {
      eb[c] += G * sb[c] + (c < D ? lam * strb : 0.0);
      Gb += sb[c] * eps[c];
    }
    mub += 2.0 * Gb;
    lamb += tr * strb;
    return;
  }
  const double kappa = lam + mu, k1 = mp.k1, fy = mp.fy;
  double d[S], s[S], w[S], sv[S];
  double tr;
  if constexpr (D == 3) {
    tr = (eps[0] + eps[1]) + eps[2];
    const double tt = 0.333333333 * tr;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      d[c] = c < 3 ? eps[c] - tt : eps[c];
      s[c] = G * (d[c] - ep_in[c]);
      w[c] = c < 3 ? 1.0 : 2.0;
      sv[c] = 1.0;  // sigma_c = s_c (+ kt) - G lamp n_c
    }
  } else {
    // Voigt: e = (xx, yy, 2 xy), deviator (e0 - e1)/2, (e1 - e0)/2, e2
    const double e0 = eps[0], e1 = eps[1], e2 = 2.0 * eps[2];
    tr = e0 + e1;
    d[0] = 0.5 * e0 + (-0.5) * e1;
    d[1] = -0.5 * e0 + 0.5 * e1;
    d[2] = e2;
    s[0] = G * (d[0] - ep_in[0]);
    s[1] = G * (d[1] - ep_in[1]);
    s[2] = 0.5 * (G * (d[2] - ep_in[2]));
    w[0] = w[1] = 1.0;
    w[2] = 2.0;
    sv[0] = sv[1] = sv[2] = 1.0;
  }
  double q = 0.0;
#pragma unroll
  for (int c = 0; c < S; ++c) q += w[c] * s[c] * s[c];
  const double ns = sqrt(q);
  double sbar[S], kt_b = 0.0, Gb = 0.0;
#pragma unroll
  for (int c = 0; c < S; ++c) sbar[c] = sb[c];
#pragma unroll
  for (int c = 0; c < D; ++c) kt_b += sb[c];
  double alpha_b = ab;  // alpha' = alpha (+ lamp)
  double epb_pass[S];   // pstrain' = pstrain (+ lamp n, times 2 for the 2D shear)
#pragma unroll
  for (int c = 0; c < S; ++c) epb_pass[c] = pb[c];
  const double ftrial = ns - (k1 * alpha_in + fy);
  if (!(ftrial <= 0.0) && ns > 0.0) {
    const double r = 1.0 / (G + k1);
    const double lamp = ((ns - k1 * alpha_in) - fy) * r;
    const double ins = 1.0 / ns;
    double n[S], lampb = ab, nsb = 0.0;
#pragma unroll
    for (int c = 0; c < S; ++c) {
      n[c] = s[c] * ins;
      const double ew = (D == 2 && c == 2) ? 2.0 : 1.0;  // 2D pstrain shear takes 2 n (Iinv)
      lampb += pb[c] * ew * n[c] - G * sb[c] * n[c];
      Gb -= lamp * sb[c] * n[c];
    }
    Gb -= lampb * lamp * r;  // lamp = (ns - k1 alpha - fy) / (G + k1)
    double nb[S];
#pragma unroll
    for (int c = 0; c < S; ++c) {
      const double ew = (D == 2 && c == 2) ? 2.0 : 1.0;
      nb[c] = lamp * pb[c] * ew - G * lamp * sb[c];
      nsb -= nb[c] * s[c] * ins * ins;
    }
    nsb += lampb * r;
#pragma unroll
    for (int c = 0; c < S; ++c) sbar[c] += nb[c] * ins + nsb * w[c] * s[c] * ins;
    alpha_b -= k1 * r * lampb;
  }
  (void)sv;
  // s_c = G (d_c - ep_c)  (2D shear: 0.5 G (d_2 - ep_2))
  double db[S];
#pragma unroll
  for (int c = 0; c < S; ++c) {
    const double h = (D == 2 && c == 2) ? 0.5 : 1.0;
    db[c] = h * G * sbar[c];
    epb_pass[c] -= h * G * sbar[c];
    Gb += h * sbar[c] * (d[c] - ep_in[c]);
  }
  const double kappab = kt_b * tr;
  if constexpr (D == 3) {
    const double ttb = -((db[0] + db[1]) + db[2]);
    const double trb = 0.333333333 * ttb + kappa * kt_b;
#pragma unroll
    for (int c = 0; c < 6; ++c) eb[c] += db[c] + (c < 3 ? trb : 0.0);
  } else {
    double e0b = 0.5 * db[0] - 0.5 * db[1] + kappa * kt_b;
    double e1b = -0.5 * db[0] + 0.5 * db[1] + kappa * kt_b;
    eb[0] += e0b;
    eb[1] += e1b;
    eb[2] += 2.0 * db[2];
  }
#pragma unroll
  for (int c = 0; c < S; ++c) pb[c] = epb_pass[c];
  ab = alpha_b;
  // G = 2 mu, kappa = lambda + mu
  mub += 2.0 * Gb + kappab;
  lamb += kappab;
}

// G2P adjoint of particle p inside the grid (hat h): reads its adjoints,
// writes x_, F_ (and the constitutive adjoints, with E_ += dL/dE), and hands
// each corner k's node adjoints (vdt_ (D), dv_ (D)) to put(k, node, val).
template <int D, int MAT, class Put>
__device__ __forceinline__ void g2p_adj_particle(const GridP& gp, const GridRec& gr, const PartP& pp, const AdjP& ad,
                                                 const NodeAdjP& na, const MatParams& mp, double c1, double c2,
                                                 int64_t p, const Hat<D, double>& h, Put&& put) {
  using L = Layout<D>;
  using A = AdjLayout<D>;
  const double* P = static_cast<const double*>(pp.base);
  CornersFull<D> c;
  corners_full<D>(gp, h, c);
  const int64_t Nn = na.nodeCount;
  double vdt[1 << D][D], dv[1 << D][D];
  double Ldt[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) Ldt[a][b] = 0.0;
#pragma unroll
  for (int k = 0; k < (1 << D); ++k)
#pragma unroll
    for (int a = 0; a < D; ++a) {
      vdt[k][a] = gr.vdt[a * Nn + c.node[k]];
      dv[k][a] = gr.dv[a * Nn + c.node[k]];
#pragma unroll
      for (int b = 0; b < D; ++b) Ldt[a][b] += vdt[k][a] * c.g[k][b];
    }
  double F[D * D], Fb[D * D], xb[D], vb[D];
#pragma unroll
  for (int q = 0; q < D * D; ++q) {
    F[q] = P[int64_t(L::F + q) * pp.pitch + p];
    Fb[q] = *adj<D>(ad, A::FB + q, p);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    xb[a] = *adj<D>(ad, A::XB + a, p);
    vb[a] = *adj<D>(ad, A::VB + a, p);
  }
  // Abar = F^T F', F_ = F' A^T with A = I + Ldt (column-major F[i + D j])
  double Ab[D][D], Fn[D * D];
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) s += F[i + D * k] * Fb[i + D * j];
      Ab[k][j] = s;
    }
  if constexpr (MAT != MPM_MAT_NEOHOOKEAN) {
    // the strain and stress update of this G2P: eps' = eps + sym(Ldt), then
    // update_stress! at eps' (its adjoint from the next step's P2G and G2P)
    constexpr int S = Layout<D>::S;
    double eps[S], ep_in[S], sb[S], eb[S], pb[S];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = i; j < D; ++j) {
        const int c = sym<D>(i, j);
        const double de = i == j ? Ldt[i][i] : 0.5 * (Ldt[i][j] + Ldt[j][i]);
        eps[c] = P[int64_t(L::EPS + c) * pp.pitch + p] + de;
      }
#pragma unroll
    for (int c = 0; c < S; ++c) {
      ep_in[c] = MAT == MPM_MAT_J2 ? P[int64_t(L::EP + c) * pp.pitch + p] : 0.0;
      sb[c] = *adj<D>(ad, A::SIGB + c, p);
      eb[c] = *adj<D>(ad, A::EPSB + c, p);
      pb[c] = *adj<D>(ad, A::EPB + c, p);
    }
    double ab = *adj<D>(ad, A::ALB, p);
    const double alpha_in = MAT == MPM_MAT_J2 ? P[int64_t(L::ALPHA) * pp.pitch + p] : 0.0;
    double lam = mp.lambda, mu = mp.mu;
    if (mp.per_particle) {
      lam = P[int64_t(L::LAM) * pp.pitch + p];
      mu = P[int64_t(L::MU) * pp.pitch + p];
    }
    double mub = 0.0, lamb = 0.0;
    stress_adj<D, MAT>(eps, lam, mu, mp, ep_in, alpha_in, sb, eb, pb, ab, mub, lamb);
    // eps' = eps + sym(Ldt): eps_ passes through, Ldt_ += the symmetric part
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = i; j < D; ++j) {
        const int c = sym<D>(i, j);
        if (i == j) {
          Ab[i][i] += eb[c];
        } else {
          Ab[i][j] += 0.5 * eb[c];
          Ab[j][i] += 0.5 * eb[c];
        }
      }
#pragma unroll
    for (int c = 0; c < S; ++c) {
      *adj<D>(ad, A::EPSB + c, p) = eb[c];
      *adj<D>(ad, A::EPB + c, p) = pb[c];
    }
    *adj<D>(ad, A::ALB, p) = ab;
    *adj<D>(ad, A::EB, p) += c1 * lamb + c2 * mub;
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int k = 0; k < D; ++k) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) s += Fb[i + D * j] * ((k == j ? 1.0 : 0.0) + Ldt[k][j]);
      Fn[i + D * k] = s;
    }
  double xn[D];
#pragma unroll
  for (int a = 0; a < D; ++a) xn[a] = xb[a];
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    double wb = 0.0, gb[D];
#pragma unroll
    for (int a = 0; a < D; ++a) wb += xb[a] * vdt[k][a] + vb[a] * dv[k][a];
#pragma unroll
    for (int b = 0; b < D; ++b) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) s += Ab[a][b] * vdt[k][a];
      gb[b] = s;
    }
    double val[2 * D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double s = c.N[k] * xb[a];
#pragma unroll
      for (int b = 0; b < D; ++b) s += Ab[a][b] * c.g[k][b];
      val[a] = s;
      val[D + a] = c.N[k] * vb[a];
    }
    put(k, c.node[k], val);
    add_shape_adj<D>(xn, c, k, wb, gb);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) *adj<D>(ad, A::XB + a, p) = xn[a];
#pragma unroll
  for (int q = 0; q < D * D; ++q) *adj<D>(ad, A::FB + q, p) = Fn[q];
}


// G2P adjoint of particle pp.begin + t (t < pp.count) with its node adjoints
// added by FP64 atomics per corner and value at L2
template <int D, int MAT>
__device__ __forceinline__ void g2p_adj_atomic(const GridP& gp, const GridRec& gr, const PartP& pp, const AdjP& ad,
                                               const NodeAdjP& na, const MatParams& mp, double c1, double c2,
                                               int64_t t) {
  using L = Layout<D>;
  const int64_t p = pp.begin + t, Nn = na.nodeCount;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = static_cast<const double*>(pp.base)[int64_t(L::X + a) * pp.pitch + p];
  Hat<D, double> h;
  if (!hat<D, double>(gp, x, h)) return;  // frozen particle: its adjoints pass through unchanged
  g2p_adj_particle<D, MAT>(gp, gr, pp, ad, na, mp, c1, c2, p, h, [&](int, int64_t n, const double* val) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      atomicAdd(na.vdtb + a * Nn + n, val[a]);
      atomicAdd(na.dvb + a * Nn + n, val[D + a]);
    }
  });
}

// The G2P adjoint.  Its scatter of the node adjoints vdt_ and dv_:
// TILE = false: FP64 atomics per particle, corner and value at L2;
// TILE = true: staged in a shared-memory tile of the node box the CTA's
//   particles cover (the box as in the P2G tile kernel): shared FP64 atomics
//   per particle and corner, then one global atomic per non-zero node value and
//   CTA; a CTA whose box holds more than cap nodes adds per particle to global
//   memory.  Dynamic shared memory: cap * 2D doubles.
// blockDim.x is a multiple of 32 and at most 256.
template <int D, int MAT, bool TILE>
__global__ void __launch_bounds__(256) g2p_adj_kernel(GridP gp, GridRec gr, PartP pp, AdjP ad, NodeAdjP na,
                                                      MatParams mp, double c1, double c2, int cap) {
  using L = Layout<D>;
  constexpr int NV = 2 * D;
  extern __shared__ double tile[];
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t p = pp.begin + t;
  const int64_t Nn = na.nodeCount;
  if constexpr (!TILE) {
    if (t < pp.count) g2p_adj_atomic<D, MAT>(gp, gr, pp, ad, na, mp, c1, c2, t);
    return;
  }
  Hat<D, double> h{};
  bool ok = false;  // false: outside the grid, a frozen particle whose adjoints pass through unchanged
  if (t < pp.count) {
    double x[D];
#pragma unroll
    for (int a = 0; a < D; ++a) x[a] = static_cast<const double*>(pp.base)[int64_t(L::X + a) * pp.pitch + p];
    ok = hat<D, double>(gp, x, h);
  }
  int lo[3], hi[3];
  cta_cell_box<D>(ok, h.c, lo, hi);
  if (lo[0] > hi[0]) return;  // uniform
  const int e0 = hi[0] - lo[0] + 2, e1 = hi[1] - lo[1] + 2, e2 = D == 3 ? hi[2] - lo[2] + 2 : 1;
  const int64_t vol64 = int64_t(e0) * e1 * e2;
  const bool use = vol64 <= int64_t(cap);  // uniform
  const int vol = use ? int(vol64) : 0;
  if (use) {
    for (int i = threadIdx.x; i < vol * NV; i += blockDim.x) tile[i] = 0.0;
    __syncthreads();
  }
  if (ok) {
    const int lbase = use ? (h.c[0] - lo[0]) + e0 * ((h.c[1] - lo[1]) + (D == 3 ? e1 * (h.c[D - 1] - lo[D - 1]) : 0)) : 0;
    g2p_adj_particle<D, MAT>(gp, gr, pp, ad, na, mp, c1, c2, p, h, [&](int k, int64_t n, const double* val) {
      if (use) {
        // lo <= c <= hi per axis, so 0 <= l < vol
        const int l = lbase + (k & 1) + e0 * ((k >> 1) & 1) + (D == 3 ? e0 * e1 * (k >> 2) : 0);
#pragma unroll
        for (int q = 0; q < NV; ++q) atomicAdd(tile + q * vol + l, val[q]);
      } else {
#pragma unroll
        for (int a = 0; a < D; ++a) {
          atomicAdd(na.vdtb + a * Nn + n, val[a]);
          atomicAdd(na.dvb + a * Nn + n, val[D + a]);
        }
      }
    });
  }
  if (!use) return;  // uniform
  __syncthreads();
  for (int l = threadIdx.x; l < vol; l += blockDim.x) {
    const int ix = l % e0, iy = (l / e0) % e1, iz = l / (e0 * e1);
    const int64_t n = int64_t(lo[0] + ix) + gp.nx * int64_t(lo[1] + iy) + (D == 3 ? gp.nxy * int64_t(lo[2] + iz) : 0);
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double v = tile[q * vol + l];
      if (v != 0.0) atomicAdd((q < D ? na.vdtb + q * Nn : na.dvb + (q - D) * Nn) + n, v);
    }
  }
}

// grid adjoint of node i (see the header)
template <int D>
__device__ __forceinline__ void grid_adj_node(const GridRec& gr, const NodeAdjP& na, const uint8_t* fixed, double dt,
                                              double tol, int64_t i) {
  const int64_t Nn = na.nodeCount;
  const double m = gr.m[i];
  double mb = 0.0;
  const unsigned fx = fixed[i];
  const double im = m > tol ? 1.0 / m : 0.0;  // one FP64 division per node
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double p0b = 0.0, fb = 0.0;
    const double vdtb = __ldcg(na.vdtb + a * Nn + i), dvb = __ldcg(na.dvb + a * Nn + i);
    if (m > tol && !(fx & (1u << a))) {
      p0b = (dt * vdtb) * im;
      fb = (dt * dt * vdtb + dt * dvb) * im;
      mb -= (vdtb * gr.vdt[a * Nn + i] + dvb * gr.dv[a * Nn + i]) * im;
    }
    na.p0b[a * Nn + i] = p0b;
    na.fb[a * Nn + i] = fb;
    // consumed: zero for the previous step's G2P adjoint, which accumulates into them
    na.vdtb[a * Nn + i] = 0.0;
    na.dvb[a * Nn + i] = 0.0;
  }
  na.mb[i] = mb;
}

template <int D>
__global__ void __launch_bounds__(256) grid_adj_kernel(GridRec gr, NodeAdjP na, const uint8_t* fixed, double dt,
                                                       double tol) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < na.nodeCount) grid_adj_node<D>(gr, na, fixed, dt, tol, i);
}

template <int D>
__device__ __forceinline__ void inv_det(const double* F, double* Fi, double& J, double& iJ) {
  if constexpr (D == 2) {
    J = F[0] * F[3] - F[2] * F[1];
    iJ = 1.0 / J;
    Fi[0] = F[3] * iJ;
    Fi[3] = F[0] * iJ;
    Fi[2] = -F[2] * iJ;
    Fi[1] = -F[1] * iJ;
  } else {
    const double c00 = F[4] * F[8] - F[7] * F[5], c02 = F[1] * F[5] - F[4] * F[2];
    J = F[0] * c00 - F[3] * (F[1] * F[8] - F[2] * F[7]) + F[6] * c02;
    iJ = 1.0 / J;
    // inverse via the adjugate (column-major: Fi[i + 3 j] = (F^-1)_ij)
    Fi[0] = c00 * iJ;
    Fi[1] = -(F[1] * F[8] - F[2] * F[7]) * iJ;
    Fi[2] = c02 * iJ;
    Fi[3] = -(F[3] * F[8] - F[5] * F[6]) * iJ;
    Fi[4] = (F[0] * F[8] - F[2] * F[6]) * iJ;
    Fi[5] = -(F[0] * F[5] - F[2] * F[3]) * iJ;
    Fi[6] = (F[3] * F[7] - F[4] * F[6]) * iJ;
    Fi[7] = -(F[0] * F[7] - F[1] * F[6]) * iJ;
    Fi[8] = (F[0] * F[4] - F[1] * F[3]) * iJ;
  }
}

// P2G adjoint of particle pp.begin + t (t < pp.count; see the header)
template <int D, int MAT>
__device__ __forceinline__ void p2g_adj_particle(const GridP& gp, const PartP& pp, const AdjP& ad, const NodeAdjP& na,
                                                 const MatParams& mp, double c1, double c2, double bx, double by,
                                                 double bz, int64_t t) {
  using L = Layout<D>;
  using A = AdjLayout<D>;
  const int64_t p = pp.begin + t;
  const double* P = static_cast<const double*>(pp.base);
  auto fld = [&](int f) { return P[int64_t(f) * pp.pitch + p]; };
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = fld(L::X + a);
  Hat<D, double> h;
  if (!hat<D, double>(gp, x, h)) return;
  CornersFull<D> c;
  corners_full<D>(gp, h, c);
  const double mpart = fld(L::M), V = fld(L::VOL), V0 = fld(L::VOL0);
  double v[D], sig[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a) v[a] = fld(L::V + a);
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) sig[a][b] = fld(L::SIG + sym<D>(a, b));
  const double grav[3] = {bx, by, bz};
  // per particle once: -V sigma, m v, m g; per corner the sum T = sum_k f_ (x) grad N_k,
  // from which sigma_ = -V T and V_ = -sigma : T after the corners
  double sV[D][D], mv[D], mg[D], T[D][D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    mv[a] = mpart * v[a];
    mg[a] = mpart * grav[a];
#pragma unroll
    for (int b = 0; b < D; ++b) {
      sV[a][b] = -V * sig[a][b];
      T[a][b] = 0.0;
    }
  }
  double xb[D], vb[D], sb[D][D], Vb = 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    xb[a] = *adj<D>(ad, A::XB + a, p);
    vb[a] = *adj<D>(ad, A::VB + a, p);
  }
  const int64_t Nn = na.nodeCount;
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    const int64_t n = c.node[k];
    // node adjoints through L2 (__ldcg): in the fused reverse step other CTAs
    // wrote them in this launch
    const double mb = __ldcg(na.mb + n);
    double p0b[D], fb[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      p0b[a] = __ldcg(na.p0b + a * Nn + n);
      fb[a] = __ldcg(na.fb + a * Nn + n);
    }
    double wb = mpart * mb, gb[D];
    const double mN = mpart * c.N[k];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      wb += mv[a] * p0b[a] + mg[a] * fb[a];
      vb[a] += mN * p0b[a];
    }
#pragma unroll
    for (int b = 0; b < D; ++b) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) s += sV[a][b] * fb[a];
      gb[b] = s;
    }
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = 0; b < D; ++b) T[a][b] += fb[a] * c.g[k][b];
    add_shape_adj<D>(xb, c, k, wb, gb);
  }
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < D; ++b) {
      sb[a][b] = -V * T[a][b];
      Vb -= sig[a][b] * T[a][b];
    }
  double F[D * D], Fi[D * D], J, iJ;
#pragma unroll
  for (int q = 0; q < D * D; ++q) F[q] = fld(L::F + q);
  inv_det<D>(F, Fi, J, iJ);
  if constexpr (MAT != MPM_MAT_NEOHOOKEAN) {
    // the stress is particle state: its adjoint (stored symmetric components)
    // goes to the G2P adjoint of the previous step, which formed it; V = J V0
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = i; j < D; ++j)
        *adj<D>(ad, A::SIGB + sym<D>(i, j), p) = i == j ? sb[i][i] : sb[i][j] + sb[j][i];
    const double cV = Vb * V0 * J;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int q = 0; q < D; ++q) *adj<D>(ad, A::FB + a + D * q, p) += cV * Fi[q + D * a];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      *adj<D>(ad, A::XB + a, p) = xb[a];
      *adj<D>(ad, A::VB + a, p) = vb[a];
    }
    return;
  }
  // sigma = NH(F) = (mu (F F^T - I) + lambda ln J I) / J ;  V = J V0
  double lam = mp.lambda, mu = mp.mu;
  if (mp.per_particle) {
    lam = fld(L::LAM);
    mu = fld(L::MU);
  }
  const double lnJ = log(J);
  double trS = 0.0, SB = 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    trS += sb[a][a];
#pragma unroll
    for (int b = 0; b < D; ++b) {
      double Bab = 0.0;
#pragma unroll
      for (int q = 0; q < D; ++q) Bab += F[a + D * q] * F[b + D * q];
      SB += sb[a][b] * (Bab - (a == b ? 1.0 : 0.0));
    }
  }
  // F_ += (mu/J)[(S + S^T) F - (S:(B - I)) F^-T] + lambda trS (1 - ln J)/J F^-T + V_ V0 J F^-T
  const double cinvT = -mu * iJ * SB + lam * trS * (1.0 - lnJ) * iJ + Vb * V0 * J;
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int q = 0; q < D; ++q) {
      double s = 0.0;
#pragma unroll
      for (int b = 0; b < D; ++b) s += (sb[a][b] + sb[b][a]) * F[b + D * q];
      *adj<D>(ad, A::FB + a + D * q, p) += mu * iJ * s + cinvT * Fi[q + D * a];
    }
  *adj<D>(ad, A::EB, p) += c1 * (trS * lnJ * iJ) + c2 * (SB * iJ);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    *adj<D>(ad, A::XB + a, p) = xb[a];
    *adj<D>(ad, A::VB + a, p) = vb[a];
  }
}

template <int D, int MAT>
__global__ void __launch_bounds__(256) p2g_adj_kernel(GridP gp, PartP pp, AdjP ad, NodeAdjP na, MatParams mp,
                                                      double c1, double c2, double bx, double by, double bz) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < pp.count) p2g_adj_particle<D, MAT>(gp, pp, ad, na, mp, c1, c2, bx, by, bz, t);
}

// ---------------------------------------------------------------------------
// One reversed step of a single-body context in one cooperative launch: the G2P
// adjoint (per-particle atomics), a grid barrier, the grid adjoint of every
// node, a grid barrier, the P2G adjoint -- the three kernels above without two
// launches and the grid adjoint's own launch latency.  Thread t handles
// particle t in the particle stages and nodes t, t + gridDim.x blockDim.x, ...
// in the grid stage, so no thread leaves before a barrier.
struct RevStepP {
  GridP gp;
  GridRec gr;
  PartP pp;
  AdjP ad;
  NodeAdjP na;
  MatParams mp;
  double c1, c2, dt, tol;
  double grav[3];
  const uint8_t* fixed;
  unsigned* bar;  // [0] arrivals, [1] generation: zero before the first launch, left consistent by each
  unsigned* err;  // bit 0: a barrier wait gave up
};

// Grid-wide barrier of a cooperative launch (every CTA resident).  Thread 0 of
// each CTA arrives on bar[0]; the last to arrive resets it and advances the
// generation bar[1]; the others wait for the generation to change, at most
// about one second (globaltimer), after which the wait sets err bit 0 and
// returns false and the kernel ends without its remaining stages.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;  // read before arriving: it cannot advance until this CTA has arrived
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x * gridDim.y * gridDim.z - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      // spin on the generation; the clock is read every 16 polls
      unsigned long long t0, t1;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      unsigned polls = 0;
      while (*gen == g) {
        if ((++polls & 15u) == 0u) {
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
          if (t1 - t0 > 1000000000ull) {
            atomicOr(err, 1u);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <int D, int MAT>
__global__ void __launch_bounds__(256) reverse_step_kernel(RevStepP r) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nth = int64_t(gridDim.x) * blockDim.x;
  if (*reinterpret_cast<volatile unsigned*>(r.err)) return;  // an earlier barrier gave up: the sweep is void
  if (t < r.pp.count) g2p_adj_atomic<D, MAT>(r.gp, r.gr, r.pp, r.ad, r.na, r.mp, r.c1, r.c2, t);
  if (!grid_barrier(r.bar, r.err)) return;
  for (int64_t i = t; i < r.na.nodeCount; i += nth) grid_adj_node<D>(r.gr, r.na, r.fixed, r.dt, r.tol, i);
  if (!grid_barrier(r.bar, r.err)) return;
  if (t < r.pp.count)
    p2g_adj_particle<D, MAT>(r.gp, r.pp, r.ad, r.na, r.mp, r.c1, r.c2, r.grav[0], r.grav[1], r.grav[2], t);
}

}  // namespace jmpm
