// mpm_dual.cpp -- forward-mode derivatives of jump's explicit USL step through
// a restatement templated on the scalar type.
//
// TEST INFRASTRUCTURE ONLY.  This is the gradient oracle the GPU adjoint is
// checked against; nothing in the product library links, loads or calls it.
// It stands in for running ForwardDiff through the reference Julia code (not
// possible here: Julia is not installed): the USL step with the linear hat
// basis and one velocity field -- P2G, grid update with the Dirichlet mask,
// G2P with the F, J, V and strain updates, update_stress! of the linear
// elastic, neo-Hookean and J2 materials with per-particle Young's modulus --
// written once as a template over a scalar T and run with T = Dual<N>, a
// forward-mode dual number written for this file (value + N directional
// derivatives, seeded on N chosen parameters at a time).
//
// Follows, statement by statement and in the same operation order as
// oracle/mpm_oracle.cpp (so that with T = double it reproduces that oracle bit
// for bit, which tests/test_dual_oracle.py checks):
//   time loop body, P2G, grid update, G2P     SolveExplicitSolidMechanics2D.jl:381-534
//   3D (the 2D USL lifted to three components, as the main oracle)
//   hat basis                                  Basis.jl:63-78, 104-137, 219-251, 292-332
//   materials                                  Material.jl:37-81 (elastic), 100-122
//                                              (neo-Hookean), 128-275 (J2)
// The cell of a particle and the sign factors of the hat gradient are
// piecewise constant in x, so they take the value part; everything else is
// differentiated: the derivative is that of the discrete map inside the
// particles' current cells, like the GPU adjoint's.
#include "../include/jump_mpm.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

template <int N>
struct Dual {
  double v = 0.0;
  double d[N] = {};
  Dual() = default;
  Dual(double x) : v(x) {}  // NOLINT: constants promote implicitly, as in the templated code
};

template <int N>
inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N>
inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v / b.v);
  const double ib = 1.0 / b.v;
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { return a * Dual<N>(b); }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return Dual<N>(a) * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { return a = a + b; }

template <int N>
inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r(std::sqrt(a.v));
  const double h = r.v > 0 ? 0.5 / r.v : 0.0;
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int N>
inline Dual<N> log(const Dual<N>& a) {
  Dual<N> r(std::log(a.v));
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / a.v;
  return r;
}
template <int N>
inline Dual<N> fabs(const Dual<N>& a) {
  return a.v < 0 ? -a : a;
}

inline double val(double x) { return x; }
template <int N> inline double val(const Dual<N>& x) { return x.v; }
inline double sqrt(double x) { return std::sqrt(x); }
inline double log(double x) { return std::log(x); }
inline double fabs(double x) { return std::fabs(x); }

template <class T>
inline double sign_of(const T& x) {
  const double v = val(x);
  return (v > 0) ? 1.0 : ((v < 0) ? -1.0 : 0.0);
}

template <int D>
struct Grid {
  double xmin[3] = {0, 0, 0}, dx[3] = {0, 0, 0}, dxI[3] = {0, 0, 0};
  int64_t nn[3] = {1, 1, 1};
  int64_t nodeCount = 0, nodeCountXY = 0;
  std::vector<double> pos;
  std::vector<int64_t> fixed;
};

template <class T, int D>
struct Body {
  int64_t n = 0;
  int type = MPM_MAT_ELASTIC;
  double nu = 0, fy = 0, k1 = 0;
  std::vector<double> mass, vol0;
  std::vector<T> pos, vel, vol, F, strain, stress, alpha, pstrain, youngs;
};

// getAdjacentGridPoints + getShapeAndGradient, as oracle/mpm_oracle.cpp's shape()
template <class T, int D>
bool shape(const Grid<D>& g, const T* xp, int64_t* near, T* N, T* dN) {
  int64_t b[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    const double t = (val(xp[a]) - g.xmin[a]) * g.dxI[a] + 1.0;
    const double f = std::floor(t);
    if (!(f >= 1.0) || !(f <= double(g.nn[a] - 1))) return false;
    b[a] = int64_t(f);
  }
  if (D == 2) {
    const int64_t I = g.nn[0] * (b[1] - 1) + b[0], nx = g.nn[0];
    const int64_t ids[4] = {I, I + 1, I + nx, I + 1 + nx};
    for (int i = 0; i < 4; ++i) {
      near[i] = ids[i] - 1;
      const double* xi = &g.pos[2 * near[i]];
      T xip = xp[0] - xi[0];
      T yip = xp[1] - xi[1];
      T Nx = 1.0 - fabs(xip) * g.dxI[0];
      T Ny = 1.0 - fabs(yip) * g.dxI[1];
      N[i] = Nx * Ny;
      dN[2 * i + 0] = -Ny * sign_of(xip) * g.dxI[0];
      dN[2 * i + 1] = -Nx * sign_of(yip) * g.dxI[1];
    }
  } else {
    const int64_t I = g.nodeCountXY * (b[2] - 1) + g.nn[0] * (b[1] - 1) + b[0];
    const int64_t nx = g.nn[0], nxy = g.nodeCountXY;
    const int64_t ids[8] = {I, I + 1, I + nx, I + nx + 1, I + nxy, I + 1 + nxy, I + nx + nxy, I + nx + 1 + nxy};
    for (int i = 0; i < 8; ++i) {
      near[i] = ids[i] - 1;
      const double* xI = &g.pos[3 * near[i]];
      T xip = xp[0] - xI[0];
      T yip = xp[1] - xI[1];
      T zip = xp[2] - xI[2];
      T Nx = 1.0 - fabs(xip) * g.dxI[0];
      T Ny = 1.0 - fabs(yip) * g.dxI[1];
      T Nz = 1.0 - fabs(zip) * g.dxI[2];
      N[i] = Nx * Ny * Nz;
      dN[3 * i + 0] = -Ny * Nz * sign_of(xip) * g.dxI[0];
      dN[3 * i + 1] = -Nx * Nz * sign_of(yip) * g.dxI[1];
      dN[3 * i + 2] = -Nx * Ny * sign_of(zip) * g.dxI[2];
    }
  }
  return true;
}

template <class T, int D>
inline T det(const T* A) {
  if (D == 2) return A[0] * A[3] - A[2] * A[1];
  const T* x0 = A;
  const T* x1 = A + 3;
  const T* x2 = A + 6;
  T c0 = x1[1] * x2[2] - x1[2] * x2[1];
  T c1 = x1[2] * x2[0] - x1[0] * x2[2];
  T c2 = x1[0] * x2[1] - x1[1] * x2[0];
  return x0[0] * c0 + x0[1] * c1 + x0[2] * c2;
}

// update_stress! of the elastic, neo-Hookean and J2 materials, as the main
// oracle's update_stress (column-major D x D tensors, J2 state per particle)
template <class T, int D>
void update_stress(const Body<T, D>& b, T lambda, T mu, T kappa, T* sig, const T* eps, const T* F, const T& J,
                   T* alpha, T* pstrain) {
  if (b.type == MPM_MAT_ELASTIC) {
    T tr = (D == 2) ? (eps[0] + eps[3]) : (eps[0] + eps[4] + eps[8]);
    T lt = lambda * tr;
    T tmu = 2.0 * mu;
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        T v = tmu * eps[i + D * j];
        if (i == j) v = v + lt;
        sig[i + D * j] = v;
      }
    return;
  }
  if (b.type == MPM_MAT_NEOHOOKEAN) {
    T FFt[9];
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        T s = F[i] * F[j];
        for (int k = 1; k < D; ++k) s = s + F[i + D * k] * F[j + D * k];
        FFt[i + D * j] = s;
      }
    T ll = lambda * log(J);
    T iJ = 1.0 / J;
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        T a = FFt[i + D * j];
        if (i == j) a = a - 1.0;
        T v = mu * a;
        if (i == j) v = v + ll;
        sig[i + D * j] = iJ * v;
      }
    return;
  }
  // J2 (ElastoPlasticMaterial), Material.jl:174-275
  if (D == 3) {
    T tr = eps[0] + eps[4] + eps[8];
    T tt = 0.333333333 * tr;
    T ed[9], s[9];
    for (int k = 0; k < 9; ++k) ed[k] = eps[k];
    ed[0] = ed[0] - tt;
    ed[4] = ed[4] - tt;
    ed[8] = ed[8] - tt;
    T tmu = 2 * mu;
    for (int k = 0; k < 9; ++k) s[k] = tmu * (ed[k] - pstrain[k]);
    T ns = sqrt(s[0] * s[0] + s[4] * s[4] + s[8] * s[8] + 2.0 * (s[3] * s[3] + s[7] * s[7] + s[6] * s[6]));
    T kt = kappa * tr;
    T st[9];
    for (int k = 0; k < 9; ++k) st[k] = s[k];
    st[0] = kt + st[0];
    st[4] = kt + st[4];
    st[8] = kt + st[8];
    T a0 = *alpha;
    T f_trial = ns - (b.k1 * a0 + b.fy);
    T sg[9];
    if (val(f_trial) <= 0.) {
      for (int k = 0; k < 9; ++k) sg[k] = st[k];
    } else {
      T inv = 1.0 / ns;
      T nrm[9];
      for (int k = 0; k < 9; ++k) nrm[k] = inv * s[k];
      T lam = (ns - b.k1 * a0 - b.fy) / (2 * mu + b.k1);
      a0 = a0 + lam;
      for (int k = 0; k < 9; ++k) pstrain[k] = pstrain[k] + lam * nrm[k];
      T c = 2 * mu * lam;
      for (int k = 0; k < 9; ++k) sg[k] = st[k] - c * nrm[k];
    }
    *alpha = a0;
    for (int k = 0; k < 9; ++k) sig[k] = sg[k];
    return;
  }
  const double Idev[9] = {0.5, -0.5, 0.0, -0.5, 0.5, 0.0, 0.0, 0.0, 1.0};
  const double Im[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.5};
  const double Iinv[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 2.0};
  T e[3] = {eps[0], eps[3], 2 * eps[2]};
  T edv[3], a[3], st_[3];
  for (int i = 0; i < 3; ++i) edv[i] = (Idev[i] * e[0] + Idev[i + 3] * e[1]) + Idev[i + 6] * e[2];
  for (int i = 0; i < 3; ++i) a[i] = 2 * mu * (edv[i] - pstrain[i]);
  for (int i = 0; i < 3; ++i) st_[i] = (Im[i] * a[0] + Im[i + 3] * a[1]) + Im[i + 6] * a[2];
  T ns = sqrt(st_[0] * st_[0] + st_[1] * st_[1] + 2 * (st_[2] * st_[2]));
  T kt = kappa * (e[0] + e[1]);
  const double eye2[3] = {1., 1., 0.};
  T sg[3];
  for (int i = 0; i < 3; ++i) sg[i] = kt * eye2[i] + st_[i];
  T a0 = *alpha;
  T f_trial = ns - (b.k1 * a0 + b.fy);
  if (!(val(f_trial) <= 0.)) {
    T inv = 1.0 / ns;
    T nrm[3] = {inv * st_[0], inv * st_[1], inv * st_[2]};
    T lam = (ns - b.k1 * a0 - b.fy) / (2 * mu + b.k1);
    a0 = a0 + lam;
    for (int i = 0; i < 3; ++i) {
      T q = (Iinv[i] * nrm[0] + Iinv[i + 3] * nrm[1]) + Iinv[i + 6] * nrm[2];
      pstrain[i] = pstrain[i] + lam * q;
    }
    for (int i = 0; i < 3; ++i) sg[i] = (kt * eye2[i] + st_[i]) - 2 * mu * lam * nrm[i];
  }
  sig[0] = sg[0];
  sig[3] = sg[1];
  sig[2] = sg[2];
  sig[1] = sg[2];
  *alpha = a0;
}

template <class T, int D>
struct Ctx {
  Grid<D> g;
  std::vector<Body<T, D>> bodies;
  double dt = 0, tol = 0, bf[3] = {0, 0, 0};
  std::vector<T> mass, mom0, mom, force;
  int status = MPM_OK;
};

// one USL step: reset, P2G (:391-423), grid update + Dirichlet (:429-442),
// G2P + kinematics + update_stress! (:485-532)
template <class T, int D>
void step(Ctx<T, D>& c) {
  Grid<D>& g = c.g;
  const size_t Nn = size_t(g.nodeCount);
  for (size_t i = 0; i < Nn; ++i) c.mass[i] = 0.0;
  for (size_t i = 0; i < D * Nn; ++i) {
    c.mom0[i] = 0.0;
    c.force[i] = 0.0;
  }
  int64_t near[8];
  T N[8], dN[8 * D];
  for (const Body<T, D>& b : c.bodies) {
    for (int64_t ip = 0; ip < b.n; ++ip) {
      if (!shape<T, D>(g, &b.pos[D * ip], near, N, dN)) {
        c.status = MPM_ERR_OUT_OF_GRID;
        continue;
      }
      const T fVolume = b.vol[ip];
      const double fMass = b.mass[ip];
      const T* vp = &b.vel[D * ip];
      const T* sigma = &b.stress[D * D * ip];
      for (int i = 0; i < (1 << D); ++i) {
        const int64_t in = near[i];
        const T Ni = N[i];
        const T* dNi = &dN[D * i];
        const T Nim = Ni * fMass;
        c.mass[in] = c.mass[in] + Nim;
        for (int a = 0; a < D; ++a) c.mom0[D * in + a] = c.mom0[D * in + a] + Nim * vp[a];
        for (int a = 0; a < D; ++a) {
          T s = sigma[a] * dNi[0] + sigma[a + D] * dNi[1];
          if (D == 3) s = s + sigma[a + 2 * D] * dNi[2];
          T fa = -fVolume * s + fMass * c.bf[a] * Ni;
          c.force[D * in + a] = c.force[D * in + a] + fa;
        }
      }
    }
  }
  for (int64_t i = 0; i < g.nodeCount; ++i) {
    for (int a = 0; a < D; ++a) c.mom[D * i + a] = c.mom0[D * i + a] + c.force[D * i + a] * c.dt;
    for (int a = 0; a < D; ++a)
      if (g.fixed[D * i + a] == 1) {
        c.mom0[D * i + a] = 0.;
        c.mom[D * i + a] = 0.;
      }
  }
  for (Body<T, D>& b : c.bodies) {
    for (int64_t ip = 0; ip < b.n; ++ip) {
      if (!shape<T, D>(g, &b.pos[D * ip], near, N, dN)) {
        c.status = MPM_ERR_OUT_OF_GRID;
        continue;
      }
      T L[D * D];
      for (int k = 0; k < D * D; ++k) L[k] = 0.;
      T vvp[D], xxp[D];
      for (int a = 0; a < D; ++a) {
        vvp[a] = b.vel[D * ip + a];
        xxp[a] = b.pos[D * ip + a];
      }
      for (int i = 0; i < (1 << D); ++i) {
        const int64_t in = near[i];
        const T Ni = N[i];
        const T* dNi = &dN[D * i];
        const T mI = c.mass[in];
        if (val(mI) > c.tol) {
          T vI[D];
          T invM = 1.0 / mI;
          for (int a = 0; a < D; ++a) vI[a] = c.mom[D * in + a] * invM;
          for (int a = 0; a < D; ++a) vvp[a] = vvp[a] + Ni * (c.mom[D * in + a] - c.mom0[D * in + a]) * invM;
          for (int a = 0; a < D; ++a) xxp[a] = xxp[a] + Ni * vI[a] * c.dt;
          for (int j = 0; j < D; ++j)
            for (int a = 0; a < D; ++a) L[a + D * j] = L[a + D * j] + dNi[j] * vI[a];
        }
      }
      for (int a = 0; a < D; ++a) {
        b.vel[D * ip + a] = vvp[a];
        b.pos[D * ip + a] = xxp[a];
      }
      // strain += dt D, F *= (I + L dt), J, V = J V0, update_stress! (:520-532)
      T Dm[D * D];
      for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) Dm[i + D * j] = 0.5 * (L[i + D * j] + L[j + D * i]);
      T* eps = &b.strain[D * D * ip];
      for (int k = 0; k < D * D; ++k) eps[k] = eps[k] + c.dt * Dm[k];
      T A[D * D];
      for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
          T v = L[i + D * j] * c.dt;
          if (i == j) v = v + 1.0;
          A[i + D * j] = v;
        }
      T* F = &b.F[D * D * ip];
      T Fn[D * D];
      for (int j = 0; j < D; ++j)
        for (int i = 0; i < D; ++i) {
          T s = F[i] * A[D * j];
          for (int k = 1; k < D; ++k) s = s + F[i + D * k] * A[k + D * j];
          Fn[i + D * j] = s;
        }
      for (int k = 0; k < D * D; ++k) F[k] = Fn[k];
      T J = det<T, D>(F);
      b.vol[ip] = J * b.vol0[ip];
      const T E = b.youngs[ip];
      const double nu = b.nu;
      T lambda = E * nu / (1 + nu) / (1 - 2 * nu);
      T mu = E / 2 / (1 + nu);
      T kappa = lambda + mu;
      constexpr int PS = (D == 2) ? 3 : 9;
      update_stress<T, D>(b, lambda, mu, kappa, &b.stress[D * D * ip], eps, F, J, &b.alpha[ip],
                          &b.pstrain[PS * ip]);
      if (!(val(J) > 0.0) && c.status == MPM_OK) c.status = MPM_ERR_NEGATIVE_J;
    }
  }
}

constexpr int kSeeds = 8;  // directional derivatives per pass
using D8 = Dual<kSeeds>;

template <class T, int D>
int build(const mpm_grid_desc* gd, const mpm_body_desc* bd, int nb, const mpm_params* p, Ctx<T, D>& c) {
  if (p->algorithm != MPM_ALG_USL || p->basis != MPM_BASIS_LINEAR || p->contact)
    return MPM_ERR_UNSUPPORTED;
  Grid<D>& g = c.g;
  for (int a = 0; a < D; ++a) {
    g.xmin[a] = gd->xmin[a];
    g.nn[a] = gd->nodes[a];
    g.dx[a] = (gd->xmax[a] - gd->xmin[a]) / (double(gd->nodes[a]) - 1.0);
    g.dxI[a] = 1.0 / g.dx[a];
  }
  g.nodeCountXY = g.nn[0] * g.nn[1];
  g.nodeCount = g.nodeCountXY * (D == 3 ? g.nn[2] : 1);
  g.pos.assign(size_t(D) * g.nodeCount, 0.0);
  for (int64_t k = 0; k < (D == 3 ? g.nn[2] : 1); ++k)
    for (int64_t j = 0; j < g.nn[1]; ++j)
      for (int64_t i = 0; i < g.nn[0]; ++i) {
        const int64_t idx = g.nodeCountXY * k + g.nn[0] * j + i;
        g.pos[D * idx + 0] = g.xmin[0] + double(i) * g.dx[0];
        g.pos[D * idx + 1] = g.xmin[1] + double(j) * g.dx[1];
        if (D == 3) g.pos[D * idx + 2] = g.xmin[2] + double(k) * g.dx[2];
      }
  g.fixed.assign(size_t(D) * g.nodeCount, 0);
  if (gd->fixed_nodes) std::memcpy(g.fixed.data(), gd->fixed_nodes, sizeof(int64_t) * D * g.nodeCount);
  c.mass.assign(g.nodeCount, 0.0);
  c.mom0.assign(size_t(D) * g.nodeCount, 0.0);
  c.mom.assign(size_t(D) * g.nodeCount, 0.0);
  c.force.assign(size_t(D) * g.nodeCount, 0.0);
  c.dt = p->dt;
  c.tol = p->tolerance;
  for (int a = 0; a < 3; ++a) c.bf[a] = p->body_force[a];
  constexpr int PS = (D == 2) ? 3 : 9;
  for (int s = 0; s < nb; ++s) {
    const mpm_body_desc& d = bd[s];
    if (d.mat.type != MPM_MAT_ELASTIC && d.mat.type != MPM_MAT_NEOHOOKEAN && d.mat.type != MPM_MAT_J2)
      return MPM_ERR_UNSUPPORTED;
    Body<T, D> b;
    b.n = d.count;
    b.type = d.mat.type;
    b.nu = d.mat.nu;
    b.fy = d.mat.fy;
    b.k1 = d.mat.k1;
    auto cpd = [&](std::vector<double>& v, const double* src) {
      v.assign(size_t(b.n), 0.0);
      if (src) std::memcpy(v.data(), src, sizeof(double) * b.n);
    };
    auto cpt = [&](std::vector<T>& v, const double* src, size_t per, double fillv) {
      v.assign(per * size_t(b.n), T(fillv));
      if (src)
        for (size_t k = 0; k < per * size_t(b.n); ++k) v[k] = T(src[k]);
    };
    cpd(b.mass, d.mass);
    cpd(b.vol0, d.volume_initial);
    cpt(b.pos, d.pos, D, 0.0);
    cpt(b.vel, d.velocity, D, 0.0);
    cpt(b.vol, d.volume, 1, 0.0);
    cpt(b.F, d.F, D * D, 0.0);
    if (!d.F)
      for (int64_t ip = 0; ip < b.n; ++ip)
        for (int a = 0; a < D; ++a) b.F[D * D * ip + a * (D + 1)] = T(1.0);
    cpt(b.strain, d.strain, D * D, 0.0);
    cpt(b.stress, d.stress, D * D, 0.0);
    cpt(b.alpha, d.alpha, 1, 0.0);
    cpt(b.pstrain, d.pstrain, PS, 0.0);
    cpt(b.youngs, d.youngs, 1, d.mat.E);
    c.bodies.push_back(std::move(b));
  }
  return MPM_OK;
}

// Gradient of L = xbar . x_final (all bodies in order, dim per particle) with
// respect to nseeds parameters after nsteps steps, kSeeds at a time.
// kind 0: the Young's modulus of particle ids[k] (global index over bodies);
// kind 1: component ids[k] % dim of the initial velocity of particle ids[k] / dim.
template <int D>
int grad_impl(const mpm_grid_desc* gd, const mpm_body_desc* bd, int nb, const mpm_params* p, int64_t nsteps,
              int kind, const int64_t* ids, int nseeds, const double* xbar, double* grad) {
  for (int k0 = 0; k0 < nseeds; k0 += kSeeds) {
    Ctx<D8, D> c;
    int rc = build<D8, D>(gd, bd, nb, p, c);
    if (rc != MPM_OK) return rc;
    for (int k = 0; k < kSeeds && k0 + k < nseeds; ++k) {
      int64_t id = ids[k0 + k];
      const int64_t part = kind == 0 ? id : id / D;
      int64_t off = 0;
      for (Body<D8, D>& b : c.bodies) {
        if (part < off + b.n) {
          if (kind == 0) b.youngs[part - off].d[k] = 1.0;
          else b.vel[D * (part - off) + id % D].d[k] = 1.0;
          break;
        }
        off += b.n;
      }
    }
    for (int64_t s = 0; s < nsteps; ++s) step<D8, D>(c);
    if (c.status != MPM_OK && c.status != MPM_ERR_NEGATIVE_J) return c.status;
    for (int k = 0; k < kSeeds && k0 + k < nseeds; ++k) {
      double acc = 0.0;
      int64_t off = 0;
      for (const Body<D8, D>& b : c.bodies) {
        for (int64_t q = 0; q < D * b.n; ++q) acc += xbar[D * off + q] * b.pos[q].d[k];
        off += b.n;
      }
      grad[k0 + k] = acc;
    }
  }
  return MPM_OK;
}

// The value run (T = double) for the bit-for-bit check against the main oracle.
template <int D>
int run_impl(const mpm_grid_desc* gd, const mpm_body_desc* bd, int nb, const mpm_params* p, int64_t nsteps,
             double* pos, double* stress) {
  Ctx<double, D> c;
  int rc = build<double, D>(gd, bd, nb, p, c);
  if (rc != MPM_OK) return rc;
  for (int64_t s = 0; s < nsteps; ++s) step<double, D>(c);
  int64_t off = 0;
  for (const Body<double, D>& b : c.bodies) {
    std::memcpy(pos + D * off, b.pos.data(), sizeof(double) * D * b.n);
    std::memcpy(stress + D * D * off, b.stress.data(), sizeof(double) * D * D * b.n);
    off += b.n;
  }
  return c.status;
}

}  // namespace

extern "C" {

int dual_grad(const mpm_grid_desc* grid, const mpm_body_desc* bodies, int32_t nbodies, const mpm_params* params,
              int64_t nsteps, int32_t kind, const int64_t* ids, int32_t nseeds, const double* xbar, double* grad) {
  if (!grid || !bodies || !params || !ids || !xbar || !grad || nseeds < 0 || (kind != 0 && kind != 1))
    return MPM_ERR_ARG;
  if (grid->dim == 2) return grad_impl<2>(grid, bodies, nbodies, params, nsteps, kind, ids, nseeds, xbar, grad);
  if (grid->dim == 3) return grad_impl<3>(grid, bodies, nbodies, params, nsteps, kind, ids, nseeds, xbar, grad);
  return MPM_ERR_ARG;
}

int dual_run(const mpm_grid_desc* grid, const mpm_body_desc* bodies, int32_t nbodies, const mpm_params* params,
             int64_t nsteps, double* pos, double* stress) {
  if (!grid || !bodies || !params || !pos || !stress) return MPM_ERR_ARG;
  if (grid->dim == 2) return run_impl<2>(grid, bodies, nbodies, params, nsteps, pos, stress);
  if (grid->dim == 3) return run_impl<3>(grid, bodies, nbodies, params, nsteps, pos, stress);
  return MPM_ERR_ARG;
}

}  // extern "C"
