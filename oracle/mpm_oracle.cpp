// mpm_oracle.cpp -- CPU restatement of jump's explicit USL step (linear hat basis).
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA path is checked
// against; it is never linked into, loaded by or called from the product
// library.  Only tests/, the smoke check and bench.py's CPU-baseline leg use it.
//
// PARITY STATUS: not pinned to reference outputs.  The reference is Julia and
// cannot run in this environment (no Julia toolchain), and it ships no golden
// vectors or tests.  This restatement is checked against an independent
// pure-Python restatement (tests/golden/make_golden.py, bit for bit) and against
// known answers that come from no restatement (tests/test_oracle_pins.py): the
// hat basis's partition of unity, zero gradient sum, linear reproduction and
// sign(0) gradient on node lines; B-spline partition of unity; elastic,
// neo-Hookean (uniaxial stretch) and J2 (monotonic shear, linear hardening)
// closed forms of one material point; mass and momentum conservation on the
// free two-disk collision; second-order convergence of a standing-wave
// manufactured solution.
//
// It follows the reference loops statement by statement, in the same loop and
// summation order (solids, then particles, then the nodes of a particle in
// nearPoints order), with FP64 arithmetic and no contraction (built with
// -ffp-contract=off), so that with one thread its sums are the reference's:
//   time loop, reset, P2G, grid update, G2P   SolveExplicitSolidMechanics2D.jl:335-585
//   3D USL (lifted from the 2D USL, see below) SolveExplicitSolidMechanics3D.jl:230-378
//   node lookup and hat functions             Basis.jl:63-78, 104-137, 219-251, 292-332
//   grid geometry                             Grid.jl:104-158, 198-267, 275-291
//   constitutive updates                      Material.jl:37-81, 100-122, 128-275, 279-493
//   energies                                  Fix.jl:248-270
//   multi-body contact correction             SolveExplicitFEMP2DContact.jl:189-387,
//                                             SolveExplicitFEMP3DContact.jl:388-519
//   MUSL, 2D blended consistent mass          SolveExplicitSolidMechanics2D.jl:24-329
//   MUSL, 3D lumped mass                      SolveExplicitSolidMechanics3D.jl:14-223
//
// Documented decisions where the reference cannot be followed literally:
//  * 3D USL reads the undefined `nodalMomentum0` and `counter`
//    (SolveExplicitSolidMechanics3D.jl:309-318,368), so 3D uses the 2D USL
//    step lifted to three components: momentum0 and momentum zeroed at fixed
//    dofs, v += N (p - p0)/m, body force included in the nodal force.
//  * ElastoPlasticMaterial dispatches on MMatrix stress (Material.jl:174,228)
//    and so is unreachable from the solvers; the same arithmetic is applied
//    here and its stress returned.  Plastic state is kept per particle.
//  * det of a 3x3 matrix is the column triple product x0 . (x1 x x2), the
//    published StaticArrays formula; 2x2 is a11 a22 - a12 a21.
//  * A particle whose cell lies outside the grid (undefined behaviour in the
//    reference, Basis.jl:71-74) is skipped and reported as an error.
//  * The 2D MUSL solves its blended mass matrix with a banded Cholesky where the
//    reference calls a dense `\`: the same solution up to rounding.  The MUSL
//    steps run single-threaded.
//  * With more than one thread, P2G runs slab-coloured (even then odd slabs
//    of two cells along the last axis) so the node sums are re-associated;
//    G2P results are identical for any thread count.

#include "../include/jump_mpm.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <type_traits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

struct Material {
  int type = MPM_MAT_ELASTIC;
  double E = 0, nu = 0, density = 0, lambda = 0, mu = 0, kappa = 0, fy = 0, k1 = 0;
  // Johnson-Cook / Voce (Material.jl:279-383): hardening constants, cellsize and
  // the signal velocity sqrt((lambda + 2 mu)/density) of the rate filter
  double A = 0, B = 0, C = 0, n = 0, epsdot0 = 0, cellsize = 0, velo = 0;
  // JohnsonCookMaterialWithDamage (Material.jl:495-564): the strength part's m
  // and delta = chi/(density*Cp), and the JohnsonCookDamage constants
  double m = 0, delta = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, d5 = 0, depsdot0 = 0, Tr = 0, Tm = 0, Tmr = 0;
};

Material make_material(const mpm_material_desc& d) {
  Material m;
  m.type = d.type;
  m.E = d.E;
  m.nu = d.nu;
  m.density = d.density;
  // lambda = E*nu/(1+nu)/(1-2*nu); mu = E/2/(1+nu)   Material.jl:54-55,112-113,159-161
  m.lambda = d.E * d.nu / (1 + d.nu) / (1 - 2 * d.nu);
  m.mu = d.E / 2 / (1 + d.nu);
  m.kappa = m.lambda + m.mu;
  m.fy = d.fy;
  m.k1 = d.k1;
  m.A = d.A;
  m.B = d.B;
  m.C = d.C;
  m.n = d.n;
  m.epsdot0 = d.epsdot0;
  m.cellsize = d.cellsize;
  m.velo = std::sqrt((m.lambda + 2 * m.mu) / m.density);  // Material.jl:317
  m.m = d.m;
  m.delta = d.chi / (d.density * d.Cp);  // Material.jl:323
  m.d1 = d.d1;
  m.d2 = d.d2;
  m.d3 = d.d3;
  m.d4 = d.d4;
  m.d5 = d.d5;
  m.depsdot0 = d.depsdot0;
  m.Tr = d.Tr;
  m.Tm = d.Tm;
  m.Tmr = d.Tm - d.Tr;  // Material.jl:507
  return m;
}

template <int D>
struct Body {
  int64_t n = 0;
  Material mat;
  std::vector<double> mass, vol0, vol, pos, vel, F, strain, stress;
  std::vector<double> alpha, pstrain, vmstr, youngs, alphadot;
  std::vector<double> damage_init, dam, temp;  // JohnsonCookMaterialWithDamage state
  bool has_youngs = false;
  // RigidMaterial as the USL solver reads it (SolveExplicitSolidMechanics2D.jl:453-461)
  bool rigid = false, rigid_fixed = false;
  double vr[3] = {0, 0, 0};
};

template <int D>
struct Grid {
  double xmin[3] = {0, 0, 0};
  double dx[3] = {0, 0, 0}, dxI[3] = {0, 0, 0};
  int64_t nn[3] = {1, 1, 1};
  int64_t nodeCount = 0, nodeCountXY = 0;
  std::vector<double> pos;          // D per node (Grid.jl:147-154, 253-264)
  std::vector<double> mass;         // 1 per node
  std::vector<double> momentum0, momentum, force;  // D per node
  std::vector<int64_t> fixed;       // D per node
  int basis = MPM_BASIS_LINEAR;
};

template <int D>
struct Ctx {
  Grid<D> g;
  std::vector<Body<D>> bodies;
  mpm_params p{};
  int threads = 1;
  int status = MPM_OK;
  // contact mode: per-body node fields (velocities after the grid update)
  std::vector<std::vector<double>> bm, bv0, bv, bnormal;
  std::vector<double> sysp;  // system momentum, D per node
  // MUSL: nodalMomentum2 (lumped), solved velocities v0 and v (2D consistent)
  std::vector<double> mom2, v0, gv;
};

inline double sign_of(double x) { return (x > 0) ? 1.0 : ((x < 0) ? -1.0 : 0.0); }

// getAdjacentGridPoints + getShapeAndGradient (Basis.jl:63-78, 219-251, 104-137, 292-332).
// Returns false if the particle's base cell is outside the grid.
template <int D>
bool shape(const Grid<D>& g, const double* xp, int64_t* near, double* N, double* dN) {
  int64_t b[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    double t = (xp[a] - g.xmin[a]) * g.dxI[a] + 1.0;  // floor(Int64,(x-xmin)*dxI + 1.)
    double f = std::floor(t);
    if (!(f >= 1.0) || !(f <= double(g.nn[a] - 1))) return false;
    b[a] = int64_t(f);
  }
  if (D == 2) {
    int64_t I = g.nn[0] * (b[1] - 1) + b[0];  // to_1D_index, Grid.jl:275-281 (1-based)
    int64_t nx = g.nn[0];
    int64_t ids[4] = {I, I + 1, I + nx, I + 1 + nx};
    for (int i = 0; i < 4; ++i) {
      near[i] = ids[i] - 1;
      const double* xi = &g.pos[2 * near[i]];
      double xip = xp[0] - xi[0];
      double yip = xp[1] - xi[1];
      double Nx = 1.0 - std::fabs(xip) * g.dxI[0];
      double Ny = 1.0 - std::fabs(yip) * g.dxI[1];
      N[i] = Nx * Ny;
      dN[2 * i + 0] = -Ny * sign_of(xip) * g.dxI[0];
      dN[2 * i + 1] = -Nx * sign_of(yip) * g.dxI[1];
    }
  } else {
    int64_t I = g.nodeCountXY * (b[2] - 1) + g.nn[0] * (b[1] - 1) + b[0];  // Grid.jl:283-291
    int64_t nx = g.nn[0], nxy = g.nodeCountXY;
    int64_t ids[8] = {I,       I + 1,       I + nx,       I + nx + 1,
                      I + nxy, I + 1 + nxy, I + nx + nxy, I + nx + 1 + nxy};
    for (int i = 0; i < 8; ++i) {
      near[i] = ids[i] - 1;
      const double* xI = &g.pos[3 * near[i]];
      double xip = xp[0] - xI[0];
      double yip = xp[1] - xI[1];
      double zip = xp[2] - xI[2];
      double Nx = 1.0 - std::fabs(xip) * g.dxI[0];
      double Ny = 1.0 - std::fabs(yip) * g.dxI[1];
      double Nz = 1.0 - std::fabs(zip) * g.dxI[2];
      N[i] = Nx * Ny * Nz;
      dN[3 * i + 0] = -Ny * Nz * sign_of(xip) * g.dxI[0];
      dN[3 * i + 1] = -Nx * Nz * sign_of(yip) * g.dxI[1];
      dN[3 * i + 2] = -Nx * Ny * sign_of(zip) * g.dxI[2];
    }
  }
  return true;
}

// Modified quadratic and cubic B-splines of the normalised distance r and
// their derivatives in r (Bsplines.jl:18-172): type 1 at the first and last
// node of an axis, 2 at the second, 4 at the second last, 3 elsewhere.
inline void quad_bspline(int type, double r, double& N, double& dN) {
  N = 0.;
  dN = 0.;
  if (type == 1) {
    if (r < -1.5 || r > 1.5) return;
    if (r >= -1.5 && r <= -0.5) { N = 0.5 * r * r + 1.5 * r + 1.125; dN = r + 1.5; }
    else if (r <= 0.) { N = 1. + r; dN = 1.; }
    else if (r <= 0.5) { N = 1. - r; dN = -1.; }
    else { N = 0.5 * r * r - 1.5 * r + 1.125; dN = r - 1.5; }
  } else if (type == 2) {
    if (r < -1.0 || r > 1.5) return;
    if (r >= -1. && r <= -0.5) { N = 1. + r; dN = 1.; }
    else if (r <= 0.5) { N = -r * r + 0.75; dN = -2 * r; }
    else { N = 0.5 * r * r - 1.5 * r + 1.125; dN = r - 1.5; }
  } else if (type == 3) {
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

inline void cubic_bspline(int type, double r, double& N, double& dN) {
  N = 0.;
  dN = 0.;
  const double r2 = r * r;
  if (type == 1) {
    if (r < -2. || r > 2.) return;
    if (r >= -2.0 && r <= -1.0) { N = 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333; dN = 0.5 * r2 + 2 * r + 2.; }
    else if (-1 <= r && r <= 0.) { N = -0.16666666666666666 * r * r2 + r + 1; dN = -0.5 * r2 + 1.; }
    else if (0 <= r && r <= 1.0) { N = 0.16666666666666666 * r * r2 - r + 1; dN = 0.5 * r2 - 1.0; }
    else { N = -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333; dN = -0.5 * r2 + 2 * r - 2.; }
  } else if (type == 2) {
    if (r < -1. || r > 2.) return;
    if (r >= -1.0 && r <= 0.) { N = -0.3333333333333333 * r * r2 - r2 + 0.6666666666666666; dN = -r2 - 2 * r; }
    else if (0. <= r && r <= 1.) { N = 0.5 * r * r2 - r2 + 0.6666666666666666; dN = 1.5 * r2 - 2 * r; }
    else if (1 <= r && r <= 2.0) { N = -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333; dN = -0.5 * r2 + 2 * r - 2; }
  } else if (type == 3) {
    if (r < -2. || r > 2.) return;
    if (r >= -2.0 && r <= -1.0) { N = 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333; dN = 0.5 * r2 + 2 * r + 2; }
    else if (-1. <= r && r <= 0.) { N = -0.5 * r * r2 - r2 + 0.6666666666666666; dN = -1.5 * r2 - 2 * r; }
    else if (0 <= r && r <= 1.0) { N = 0.5 * r * r2 - r2 + 0.6666666666666666; dN = 1.5 * r2 - 2 * r; }
    else if (1. <= r && r <= 2.0) { N = -0.16666666666666666 * r * r2 + r2 - 2 * r + 1.3333333333333333; dN = -0.5 * r2 + 2 * r - 2; }
  } else {
    if (r < -2. || r > 1.) return;
    if (r >= -2.0 && r <= -1.0) { N = 0.16666666666666666 * r * r2 + r2 + 2 * r + 1.3333333333333333; dN = 0.5 * r2 + 2 * r + 2; }
    else if (-1. <= r && r <= 0.) { N = -0.5 * r * r2 - r2 + 0.6666666666666666; dN = -1.5 * r2 - 2 * r; }
    else if (0 <= r && r <= 1.0) { N = 0.3333333333333333 * r * r2 - r2 + 0.6666666667; dN = r2 - 2 * r; }
  }
}

constexpr int kMaxSupport = 64;

// getShapeAndGradient for the B-spline bases (Basis.jl:374-592 quadratic,
// 594-820 cubic): per axis the near nodes, then the tensor product in the
// reference's loop order.  As written: the 3D quadratic basis measures the
// particle from the origin (numx = xp*dxI), and every B-spline basis measures
// y and z from (jd-1)*dy, (kd-1)*dz rather than from the grid's minimum.
template <int D>
int bspline_support(const Grid<D>& g, const double* xp, int64_t* near, double* N, double* dN) {
  const int K = g.basis == MPM_BASIS_QUAD_BSPLINE ? 3 : 4;
  int64_t f1[3];
  double Nv[3][4], dNv[3][4];
  for (int a = 0; a < D; ++a) {
    const int64_t nn = g.nn[a];
    const double num = (K == 3 && D == 3) ? xp[a] * g.dxI[a] : (xp[a] - g.xmin[a]) * g.dxI[a];
    const double rem = num - std::floor(num);
    const double fb = std::floor(num + 1.);
    if (!(fb >= 1.0) || !(fb <= double(nn - 1))) return 0;
    const int64_t ib = int64_t(fb);
    if (K == 3) f1[a] = ib == 1 ? ib : (ib == nn - 1 ? ib - 1 : (rem < 0.5 ? ib - 1 : ib));
    else f1[a] = ib == 1 ? 1 : (ib == nn - 1 ? ib - 2 : ib - 1);
    for (int i = 0; i < K; ++i) {
      const int64_t id = f1[a] + i;
      const double r = a == 0 ? (xp[0] - g.pos[D * (id - 1)]) * g.dxI[0] : (xp[a] - double(id - 1) * g.dx[a]) * g.dxI[a];
      const int type = (id == 1 || id == nn) ? 1 : (id == 2 ? 2 : (id == nn - 1 ? 4 : 3));
      if (K == 3) quad_bspline(type, r, Nv[a][i], dNv[a][i]);
      else cubic_bspline(type, r, Nv[a][i], dNv[a][i]);
    }
  }
  int q = 0;
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j) {
      if (D == 2) {
        near[q] = (f1[0] + i - 1) + g.nn[0] * (f1[1] + j - 1);
        N[q] = Nv[0][i] * Nv[1][j];
        dN[D * q] = dNv[0][i] * g.dxI[0] * Nv[1][j];
        dN[D * q + 1] = dNv[1][j] * g.dxI[1] * Nv[0][i];
        ++q;
      } else {
        for (int k = 0; k < K; ++k) {
          near[q] = (f1[0] + i - 1) + g.nn[0] * (f1[1] + j - 1) + g.nodeCountXY * (f1[D - 1] + k - 1);
          N[q] = Nv[0][i] * Nv[1][j] * Nv[D - 1][k];
          dN[D * q] = dNv[0][i] * g.dxI[0] * Nv[1][j] * Nv[D - 1][k];
          dN[D * q + 1] = dNv[1][j] * g.dxI[1] * Nv[0][i] * Nv[D - 1][k];
          dN[D * q + D - 1] = dNv[D - 1][k] * g.dxI[D - 1] * Nv[0][i] * Nv[1][j];
          ++q;
        }
      }
    }
  return q;
}

// nodes, values and gradients of particle position xp for the grid's basis;
// 0 when its cell lies outside the grid
template <int D>
int support(const Grid<D>& g, const double* xp, int64_t* near, double* N, double* dN) {
  if (g.basis != MPM_BASIS_LINEAR) return bspline_support<D>(g, xp, near, N, dN);
  return shape<D>(g, xp, near, N, dN) ? (D == 2 ? 4 : 8) : 0;
}

// 2x2 / 3x3 helpers on column-major storage: M[i + D*j] = M_ij (0-based).
template <int D>
inline double det(const double* A) {
  if (D == 2) return A[0] * A[3] - A[2] * A[1];
  // x0 = col 1, x1 = col 2, x2 = col 3; det = x0 . (x1 x x2)
  const double* x0 = A;
  const double* x1 = A + 3;
  const double* x2 = A + 6;
  double c0 = x1[1] * x2[2] - x1[2] * x2[1];
  double c1 = x1[2] * x2[0] - x1[0] * x2[2];
  double c2 = x1[0] * x2[1] - x1[1] * x2[0];
  return x0[0] * c0 + x0[1] * c1 + x0[2] * c2;
}

// C = A * B, sum in k order (StaticArrays unrolled product).
template <int D>
inline void matmul(const double* A, const double* B, double* C) {
  for (int j = 0; j < D; ++j)
    for (int i = 0; i < D; ++i) {
      double s = A[i] * B[D * j];
      for (int k = 1; k < D; ++k) s = s + A[i + D * k] * B[k + D * j];
      C[i + D * j] = s;
    }
}

// compute_damage (Material.jl:511-549): damage_init and damage after a plastic
// strain increment dp, given the pressure pH, the returned stress deviator Sdev
// (column-major 3x3), the plastic strain rate and the temperature.
inline void compute_damage(double* damage_init, double* damage, double pH, const double* Sdev, double epsdot,
                           double dp, double T, const Material& mat) {
  auto sq = [](double x) { return x * x; };
  const double vm = 1.224744871 * std::sqrt(sq(Sdev[0]) + sq(Sdev[4]) + sq(Sdev[8]) +
                                            2 * (sq(Sdev[3]) + sq(Sdev[6]) + sq(Sdev[7])));
  double triax = 0.0;
  if (pH != 0.0 && vm != 0.0) triax = -pH / (vm + 0.01 * std::fabs(pH));
  if (triax > 3.0) triax = 3.0;
  double jc_failure_strain = mat.d1 + mat.d2 * std::exp(mat.d3 * triax);
  if (mat.d4 > 0.0) {
    if (epsdot > mat.depsdot0) {
      const double epdot_ratio = epsdot / mat.depsdot0;
      jc_failure_strain *= (1.0 + mat.d4 * std::log(epdot_ratio));
    }
  }
  if (mat.d5 > 0.0 && T >= mat.Tr) jc_failure_strain *= 1. + mat.d5 * (T - mat.Tr) / mat.Tmr;
  *damage_init += dp / jc_failure_strain;
  if (*damage_init >= 1.0) *damage = std::min((*damage_init - 1.0) * 10, 1.0);
}

// update_stress! of JohnsonCookMaterialWithDamage (Material.jl:566-646), 3D,
// column-major; sig holds the old stress on entry and the new one on exit.
// The reference method reads mat.damage.Tm, mat.damage.temp (the type's field
// is damage_part) and dispatches on MMatrix while the solvers pass SMatrix and
// assign its return value: restated on the fields it evidently means, with
// the stress returned.
inline void jc_damage_update(const Material& mat, double mu, double kappa, double* sig, const double* eps0,
                             const double* strain_increment, double dtime, double* alpha, double* alphadot,
                             double* vmstr, double* damage_init, double* dam, double* temp) {
  const double damage = *dam;
  if (damage >= 1.0) {
    const double pH = kappa * (eps0[0] + eps0[4] + eps0[8]);
    for (int k = 0; k < 9; ++k) sig[k] = 0.0;
    sig[0] = sig[4] = sig[8] = pH;
    return;
  }
  const double eff_plastic_strain = *alpha;
  double epsdot_ratio = *alphadot / mat.epsdot0;
  epsdot_ratio = std::max(epsdot_ratio, 1.0);
  double T = *temp;
  double yieldStress;
  if (eff_plastic_strain < 1.0e-10) {
    yieldStress = mat.A;
  } else if (T < mat.Tm) {
    if (mat.C != 0)
      yieldStress = (mat.A + mat.B * std::pow(eff_plastic_strain, mat.n)) * std::pow(1.0 + epsdot_ratio, mat.C);
    else
      yieldStress = mat.A + mat.B * std::pow(eff_plastic_strain, mat.n);
    if (mat.m != 0 && T >= mat.Tr) yieldStress *= 1.0 - std::pow((T - mat.Tr) / mat.Tmr, mat.m);
  } else {
    yieldStress = 0.;
  }
  double Gd = mu;
  if (damage > 0) {
    Gd *= (1 - damage);
    yieldStress *= (1 - damage);
  }
  double dev[9];
  for (int k = 0; k < 9; ++k) dev[k] = sig[k] + 2.0 * Gd * strain_increment[k];
  const double tr = 0.333333333 * (dev[0] + dev[4] + dev[8]);
  dev[0] -= tr;
  dev[4] -= tr;
  dev[8] -= tr;
  auto sq = [](double x) { return x * x; };
  const double J2 = 1.224744871391589 * std::sqrt(sq(dev[0]) + sq(dev[4]) + sq(dev[8]) +
                                                  2 * (sq(dev[3]) + sq(dev[6]) + sq(dev[7])));
  double dp;
  if (J2 < yieldStress) {
    dp = 0.0;
  } else {
    dp = (J2 - yieldStress) / (3.0 * Gd);
    for (int k = 0; k < 9; ++k) dev[k] *= (yieldStress / J2);
  }
  *alpha = eff_plastic_strain + dp;
  const double pH = kappa * (eps0[0] + eps0[4] + eps0[8]);
  for (int k = 0; k < 9; ++k) sig[k] = dev[k];
  sig[0] += pH;
  sig[4] += pH;
  sig[8] += pH;
  const double tav = 1000 * mat.cellsize / mat.velo;
  *alphadot -= *alphadot * dtime / tav;
  *alphadot += dp / tav;
  *alphadot = std::max(0.0, *alphadot);
  const double flow_stress = 1.224744871391589 * std::sqrt(sq(dev[0]) + sq(dev[4]) + sq(dev[8]) +
                                                          2 * (sq(dev[3]) + sq(dev[6]) + sq(dev[7])));
  *vmstr = flow_stress;
  compute_damage(damage_init, dam, pH, dev, *alphadot, dp, T, mat);
  T += mat.delta * flow_stress * dp;
  *temp = T;
}

// update_stress!: returns the new stress in sig (column-major D*D).
template <int D>
void update_stress(const Material& mat, double lambda, double mu, double kappa, double* sig,
                   const double* eps, const double* F, double J, double* alpha,
                   double* pstrain, double* vmstr, const double* deps, double dtime, double* alphadot,
                   double* damage_init, double* dam, double* temp) {
  if (D == 3 && mat.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    jc_damage_update(mat, mu, kappa, sig, eps, deps, dtime, alpha, alphadot, vmstr, damage_init, dam, temp);
    return;
  }
  if (D == 3 && (mat.type == MPM_MAT_JOHNSON_COOK || mat.type == MPM_MAT_VOCE)) {
    // Material.jl:386-443 (Johnson-Cook), 445-493 (Voce); column-major 3x3
    const double ep = *alpha;
    double yieldStress;
    if (ep < 1.0e-10) {
      yieldStress = mat.A;
    } else if (mat.type == MPM_MAT_JOHNSON_COOK) {
      double epsdot_ratio = *alphadot / mat.epsdot0;
      epsdot_ratio = std::max(epsdot_ratio, 1.0);
      if (mat.C != 0) yieldStress = (mat.A + mat.B * std::pow(ep, mat.n)) * std::pow(1.0 + epsdot_ratio, mat.C);
      else yieldStress = mat.A + mat.B * std::pow(ep, mat.n);
    } else {
      yieldStress = mat.A - mat.B * std::exp(-mat.C * ep);
    }
    const double Gd = mu;
    double dev[9];
    for (int k = 0; k < 9; ++k) dev[k] = sig[k] + 2.0 * Gd * deps[k];
    const double tr = 0.333333333 * (dev[0] + dev[4] + dev[8]);
    dev[0] -= tr;
    dev[4] -= tr;
    dev[8] -= tr;
    auto sq = [](double x) { return x * x; };
    const double J2 = 1.224744871391589 * std::sqrt(sq(dev[0]) + sq(dev[4]) + sq(dev[8]) +
                                                    2 * (sq(dev[3]) + sq(dev[6]) + sq(dev[7])));
    double dp = 0.0;
    if (!(J2 < yieldStress)) {
      dp = (J2 - yieldStress) / (3.0 * Gd);
      for (int k = 0; k < 9; ++k) dev[k] *= (yieldStress / J2);
    }
    *alpha = ep + dp;
    const double tav = 1000 * mat.cellsize / mat.velo;
    *alphadot -= *alphadot * dtime / tav;
    *alphadot += dp / tav;
    *alphadot = std::max(0.0, *alphadot);
    *vmstr = std::sqrt(sq(dev[0]) + sq(dev[4]) + sq(dev[8]) + 2 * (sq(dev[3]) + sq(dev[6]) + sq(dev[7])));
    const double pr = kappa * (eps[0] + eps[4] + eps[8]);
    for (int k = 0; k < 9; ++k) sig[k] = dev[k];
    sig[0] += pr;
    sig[4] += pr;
    sig[8] += pr;
    return;
  }
  if (mat.type == MPM_MAT_ELASTIC) {
    if (D == 3) {
      // vmStr from the incoming stress (Material.jl:78-79)
      const double* s = sig;
      *vmstr = std::sqrt(s[0] * s[0] + s[4] * s[4] + s[8] * s[8] +
                         2 * (s[3] * s[3] + s[6] * s[6] + s[7] * s[7]));
    }
    // lambda*(tr eps)*I + 2.0*mu*eps   (Material.jl:68-72, 80)
    double tr = (D == 2) ? (eps[0] + eps[3]) : (eps[0] + eps[4] + eps[8]);
    double lt = lambda * tr;
    double tmu = 2.0 * mu;
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        double v = tmu * eps[i + D * j];
        if (i == j) v = v + lt;
        sig[i + D * j] = v;
      }
    return;
  }
  if (mat.type == MPM_MAT_NEOHOOKEAN) {
    // (1.0/J)*( mu*(F*F' - I) + lambda*log(J)*I )   Material.jl:119-122
    double FFt[9];
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        double s = F[i] * F[j];
        for (int k = 1; k < D; ++k) s = s + F[i + D * k] * F[j + D * k];
        FFt[i + D * j] = s;
      }
    double ll = lambda * std::log(J);
    double iJ = 1.0 / J;
    for (int j = 0; j < D; ++j)
      for (int i = 0; i < D; ++i) {
        double a = FFt[i + D * j];
        if (i == j) a = a - 1.0;
        double v = mu * a;
        if (i == j) v = v + ll;
        sig[i + D * j] = iJ * v;
      }
    return;
  }
  // J2 (ElastoPlasticMaterial)
  if (D == 3) {
    // Material.jl:228-275
    double tr = eps[0] + eps[4] + eps[8];
    double tt = 0.333333333 * tr;
    double ed[9], s[9];
    for (int k = 0; k < 9; ++k) ed[k] = eps[k];
    ed[0] = ed[0] - tt;
    ed[4] = ed[4] - tt;
    ed[8] = ed[8] - tt;
    double tmu = 2 * mu;
    for (int k = 0; k < 9; ++k) s[k] = tmu * (ed[k] - pstrain[k]);
    double ns = std::sqrt(s[0] * s[0] + s[4] * s[4] + s[8] * s[8] +
                          2.0 * (s[3] * s[3] + s[7] * s[7] + s[6] * s[6]));
    double kt = kappa * tr;
    double st[9];
    for (int k = 0; k < 9; ++k) st[k] = s[k];
    st[0] = kt + st[0];
    st[4] = kt + st[4];
    st[8] = kt + st[8];
    double a0 = *alpha;
    double f_trial = ns - (mat.k1 * a0 + mat.fy);
    double sg[9];
    if (f_trial <= 0.) {
      for (int k = 0; k < 9; ++k) sg[k] = st[k];
    } else {
      double inv = 1.0 / ns;
      double nrm[9];
      for (int k = 0; k < 9; ++k) nrm[k] = inv * s[k];
      double lam = (ns - mat.k1 * a0 - mat.fy) / (2 * mu + mat.k1);
      a0 = a0 + lam;
      for (int k = 0; k < 9; ++k) pstrain[k] = pstrain[k] + lam * nrm[k];
      double c = 2 * mu * lam;
      for (int k = 0; k < 9; ++k) sg[k] = st[k] - c * nrm[k];
    }
    *alpha = a0;
    for (int k = 0; k < 9; ++k) sig[k] = sg[k];
    double trs = sg[0] + sg[4] + sg[8];
    double ts = 0.333333333 * trs;
    double d[9];
    for (int k = 0; k < 9; ++k) d[k] = sg[k];
    d[0] = d[0] - ts;
    d[4] = d[4] - ts;
    d[8] = d[8] - ts;
    *vmstr = std::sqrt(d[0] * d[0] + d[4] * d[4] + d[8] * d[8] +
                       2 * (d[3] * d[3] + d[6] * d[6] + d[7] * d[7]));
    return;
  }
  // 2D J2, Material.jl:174-225 (Voigt [xx, yy, 2xy])
  const double Idev[9] = {0.5, -0.5, 0.0, -0.5, 0.5, 0.0, 0.0, 0.0, 1.0};  // column-major
  const double Im[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.5};
  const double Iinv[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 2.0};
  double e[3] = {eps[0], eps[3], 2 * eps[2]};
  double edv[3], a[3], st_[3];
  for (int i = 0; i < 3; ++i)
    edv[i] = (Idev[i] * e[0] + Idev[i + 3] * e[1]) + Idev[i + 6] * e[2];
  for (int i = 0; i < 3; ++i) a[i] = 2 * mu * (edv[i] - pstrain[i]);
  for (int i = 0; i < 3; ++i) st_[i] = (Im[i] * a[0] + Im[i + 3] * a[1]) + Im[i + 6] * a[2];
  double ns = std::sqrt(st_[0] * st_[0] + st_[1] * st_[1] + 2 * (st_[2] * st_[2]));
  double kt = kappa * (e[0] + e[1]);
  const double eye2[3] = {1., 1., 0.};
  double sg[3];
  for (int i = 0; i < 3; ++i) sg[i] = kt * eye2[i] + st_[i];
  double a0 = *alpha;
  double f_trial = ns - (mat.k1 * a0 + mat.fy);
  if (!(f_trial <= 0.)) {
    double inv = 1.0 / ns;
    double nrm[3] = {inv * st_[0], inv * st_[1], inv * st_[2]};
    double lam = (ns - mat.k1 * a0 - mat.fy) / (2 * mu + mat.k1);
    a0 = a0 + lam;
    for (int i = 0; i < 3; ++i) {
      double q = (Iinv[i] * nrm[0] + Iinv[i + 3] * nrm[1]) + Iinv[i + 6] * nrm[2];
      pstrain[i] = pstrain[i] + lam * q;
    }
    for (int i = 0; i < 3; ++i) sg[i] = (kt * eye2[i] + st_[i]) - 2 * mu * lam * nrm[i];
  }
  sig[0] = sg[0];
  sig[3] = sg[1];
  sig[2] = sg[2];
  sig[1] = sg[2];
  *alpha = a0;
  double dv[3];
  for (int i = 0; i < 3; ++i) dv[i] = (Idev[i] * sg[0] + Idev[i + 3] * sg[1]) + Idev[i + 6] * sg[2];
  *vmstr = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + 2 * (dv[2] * dv[2]));
}

// ---------------------------------------------------------------------------
// P2G of one particle into (mass, momentum0, force) arrays, plus optional normals
template <int D>
inline void p2g_particle(const Grid<D>& g, const Body<D>& b, int64_t ip, const double* body,
                         double* mass, double* mom0, double* force, double* normal, int* status) {
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
  if (S == 0) {
    *status = MPM_ERR_OUT_OF_GRID;
    return;
  }
  double fVolume = b.vol[ip];
  double fMass = b.mass[ip];
  const double* vp = &b.vel[D * ip];
  const double* sigma = &b.stress[D * D * ip];
  for (int i = 0; i < S; ++i) {
    int64_t in = near[i];
    double Ni = N[i];
    const double* dNi = &dN[D * i];
    double Nim = Ni * fMass;
    mass[in] += Nim;
    for (int a = 0; a < D; ++a) mom0[D * in + a] += Nim * vp[a];
    for (int a = 0; a < D; ++a) {
      // sigma[a,1]*dNi[1] + sigma[a,2]*dNi[2] (+ sigma[a,3]*dNi[3])   (:419-420)
      double s = sigma[a] * dNi[0] + sigma[a + D] * dNi[1];
      if (D == 3) s = s + sigma[a + 2 * D] * dNi[2];
      double fa = -fVolume * s + fMass * body[a] * Ni;
      force[D * in + a] += fa;
    }
    if (normal)
      for (int a = 0; a < D; ++a) normal[D * in + a] += fMass * dNi[a];
  }
}

template <int D>
inline void kin_stress(Body<D>& b, int64_t ip, const double* L, double dt, int* status);

// G2P of one particle (:500-532).  vfield/v0field given as momenta (mode 0: reference
// form (p - p0)/m) or as velocities (mode 1: contact fields, SolveExplicitFEMP2DContact.jl:415-426).
template <int D>
inline void g2p_particle(const Grid<D>& g, Body<D>& b, int64_t ip, double dt, double tol,
                         const double* mass, const double* mom0, const double* mom, int velmode,
                         int* status) {
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
  if (S == 0) {
    *status = MPM_ERR_OUT_OF_GRID;
    return;
  }
  double L[D * D];
  for (int k = 0; k < D * D; ++k) L[k] = 0.;
  double vvp[D], xxp[D];
  for (int a = 0; a < D; ++a) {
    vvp[a] = b.vel[D * ip + a];
    xxp[a] = b.pos[D * ip + a];
  }
  for (int i = 0; i < S; ++i) {
    int64_t in = near[i];
    double Ni = N[i];
    const double* dNi = &dN[D * i];
    double mI = mass[in];
    if (mI > tol) {
      double vI[D];
      if (velmode == 0) {
        double invM = 1.0 / mI;
        for (int a = 0; a < D; ++a) vI[a] = mom[D * in + a] * invM;
        for (int a = 0; a < D; ++a) vvp[a] += Ni * (mom[D * in + a] - mom0[D * in + a]) * invM;
      } else {
        for (int a = 0; a < D; ++a) vI[a] = mom[D * in + a];
        for (int a = 0; a < D; ++a) vvp[a] += Ni * (mom[D * in + a] - mom0[D * in + a]);
      }
      for (int a = 0; a < D; ++a) xxp[a] += Ni * vI[a] * dt;
      // L[i,j] += dN_j * vI_i   (:515-516; 3D USL :354 vI*dNi')
      for (int j = 0; j < D; ++j)
        for (int a = 0; a < D; ++a) L[a + D * j] += dNi[j] * vI[a];
    }
  }
  for (int a = 0; a < D; ++a) {
    b.vel[D * ip + a] = vvp[a];
    b.pos[D * ip + a] = xxp[a];
  }
  kin_stress<D>(b, ip, L, dt, status);
}

// strain += dt D, F *= (I + L dt), J, V = J V0, update_stress! (:520-532)
template <int D>
inline void kin_stress(Body<D>& b, int64_t ip, const double* L, double dt, int* status) {
  double Dm[D * D];
  for (int j = 0; j < D; ++j)
    for (int i = 0; i < D; ++i) Dm[i + D * j] = 0.5 * (L[i + D * j] + L[j + D * i]);
  double* eps = &b.strain[D * D * ip];
  for (int k = 0; k < D * D; ++k) eps[k] += dt * Dm[k];
  double A[D * D];
  for (int j = 0; j < D; ++j)
    for (int i = 0; i < D; ++i) {
      double v = L[i + D * j] * dt;
      if (i == j) v = v + 1.0;  // Identity + vel_grad*dtime
      A[i + D * j] = v;
    }
  double* F = &b.F[D * D * ip];
  double Fn[D * D];
  matmul<D>(F, A, Fn);
  for (int k = 0; k < D * D; ++k) F[k] = Fn[k];
  double J = det<D>(F);
  b.vol[ip] = J * b.vol0[ip];
  double lambda = b.mat.lambda, mu = b.mat.mu, kappa = b.mat.kappa;
  if (b.has_youngs) {
    double E = b.youngs[ip], nu = b.mat.nu;
    lambda = E * nu / (1 + nu) / (1 - 2 * nu);
    mu = E / 2 / (1 + nu);
    kappa = lambda + mu;
  }
  constexpr int PS = (D == 2) ? 3 : 9;
  double deps[D * D];  // strain_increment = dtime*D (SolveExplicitSolidMechanics3D.jl:208, 363)
  for (int k = 0; k < D * D; ++k) deps[k] = dt * Dm[k];
  update_stress<D>(b.mat, lambda, mu, kappa, &b.stress[D * D * ip], eps, F, J, &b.alpha[ip],
                   &b.pstrain[PS * ip], &b.vmstr[ip], deps, dt, &b.alphadot[ip], &b.damage_init[ip], &b.dam[ip],
                   &b.temp[ip]);
  if (!(J > 0.0) && *status == MPM_OK) *status = MPM_ERR_NEGATIVE_J;
}

template <int D>
void zero(std::vector<double>& v) {
  std::fill(v.begin(), v.end(), 0.0);
}

// P2G over every body into the given arrays; sequential or slab-coloured.
template <int D>
void p2g_bodies(Ctx<D>& c, const std::vector<int>& which, double* mass, double* mom0, double* force,
                double* normal, const double* bf = nullptr) {
  if (!bf) bf = c.p.body_force;
  if (c.threads <= 1) {
    for (int s : which) {
      const Body<D>& b = c.bodies[s];
      for (int64_t ip = 0; ip < b.n; ++ip)
        p2g_particle<D>(c.g, b, ip, bf, mass, mom0, force, normal, &c.status);
    }
    return;
  }
#ifdef _OPENMP
  // slabs of K cells along the last axis (K nodes per axis in a particle's
  // support), keyed by the support's first node; even slabs, then odd slabs,
  // so that no two particles of one pass share a node
  const int ax = D - 1;
  const int64_t K = c.g.basis == MPM_BASIS_LINEAR ? 2 : (c.g.basis == MPM_BASIS_QUAD_BSPLINE ? 3 : 4);
  const int64_t stride = D == 3 ? c.g.nodeCountXY : c.g.nn[0];
  int64_t nslab = (c.g.nn[ax] + K - 1) / K;
  std::vector<std::vector<std::pair<int, int64_t>>> slabs(nslab);
  int64_t near[kMaxSupport];
  double Nw[kMaxSupport], dNw[kMaxSupport * D];
  for (int s : which) {
    const Body<D>& b = c.bodies[s];
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(c.g, &b.pos[D * ip], near, Nw, dNw);
      const int64_t k = S > 0 ? near[0] / stride : 0;
      slabs[k / K].push_back({s, ip});
    }
  }
  int st = MPM_OK;
  for (int parity = 0; parity < 2; ++parity) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(c.threads) reduction(max : st)
    for (int64_t sl = parity; sl < nslab; sl += 2) {
      int lst = MPM_OK;
      for (auto& pr : slabs[sl])
        p2g_particle<D>(c.g, c.bodies[pr.first], pr.second, bf, mass, mom0, force, normal, &lst);
      st = std::max(st, lst);
    }
  }
  if (st != MPM_OK && c.status == MPM_OK) c.status = st;
#endif
}

template <int D>
void g2p_body(Ctx<D>& c, int s, const double* mass, const double* mom0, const double* mom,
              int velmode) {
  Body<D>& b = c.bodies[s];
  double dt = c.p.dt, tol = c.p.tolerance;
  if (c.threads <= 1) {
    for (int64_t ip = 0; ip < b.n; ++ip)
      g2p_particle<D>(c.g, b, ip, dt, tol, mass, mom0, mom, velmode, &c.status);
    return;
  }
#ifdef _OPENMP
  int st = MPM_OK;
#pragma omp parallel for schedule(static) num_threads(c.threads) reduction(max : st)
  for (int64_t ip = 0; ip < b.n; ++ip) {
    int lst = MPM_OK;
    g2p_particle<D>(c.g, b, ip, dt, tol, mass, mom0, mom, velmode, &lst);
    st = std::max(st, lst);
  }
  if (st != MPM_OK && (c.status == MPM_OK || st == MPM_ERR_OUT_OF_GRID)) c.status = st;
#endif
}

// Rigid solids after the grid update (SolveExplicitSolidMechanics2D.jl:448-479):
// for every rigid particle, in body and particle order, the nodes of its cell
// found with the linear basis (getAdjacentGridPoints with linBasis, :456)
// get momentum and momentum0 m_I v in each component with v != 0, or zero in
// every component for a fixed body (the field RigidMaterial lacks, see the
// header).  A particle outside the grid is reported and skipped.
template <int D>
void rigid_override(Ctx<D>& c) {
  Grid<D>& g = c.g;
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  for (Body<D>& b : c.bodies) {
    if (!b.rigid) continue;
    for (int64_t ip = 0; ip < b.n; ++ip) {
      if (shape<D>(g, &b.pos[D * ip], near, N, dN) == false) {
        c.status = MPM_ERR_OUT_OF_GRID;
        continue;
      }
      for (int i = 0; i < (1 << D); ++i) {
        const int64_t id = near[i];
        const double mi = g.mass[id];
        for (int a = 0; a < D; ++a) {
          if (b.rigid_fixed) {
            g.momentum[D * id + a] = 0.;
            g.momentum0[D * id + a] = 0.;
          } else if (b.vr[a] != 0.) {
            g.momentum[D * id + a] = mi * b.vr[a];
            g.momentum0[D * id + a] = mi * b.vr[a];
          }
        }
      }
    }
  }
}

// xx[ip] += dtime * v (:539-551); particles outside the grid stay where they are
template <int D>
void rigid_advance(Ctx<D>& c) {
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  for (Body<D>& b : c.bodies) {
    if (!b.rigid) continue;
    for (int64_t ip = 0; ip < b.n; ++ip) {
      // the position the override saw, before this step's move
      if (!shape<D>(c.g, &b.pos[D * ip], near, N, dN)) continue;
      for (int a = 0; a < D; ++a) b.pos[D * ip + a] += c.p.dt * b.vr[a];
    }
  }
}

// One USL step with a single velocity field (the reference).
template <int D>
void step_single(Ctx<D>& c) {
  Grid<D>& g = c.g;
  zero<D>(g.mass);
  zero<D>(g.momentum0);
  zero<D>(g.force);
  std::vector<int> deformable;
  bool any_rigid = false;
  for (size_t s = 0; s < c.bodies.size(); ++s) {
    if (c.bodies[s].rigid) any_rigid = true;  // rigid solids take no P2G (:394) and no G2P (:488)
    else deformable.push_back(int(s));
  }
  p2g_bodies<D>(c, deformable, g.mass.data(), g.momentum0.data(), g.force.data(), nullptr);
  double dt = c.p.dt;
  for (int64_t i = 0; i < g.nodeCount; ++i) {
    for (int a = 0; a < D; ++a)
      g.momentum[D * i + a] = g.momentum0[D * i + a] + g.force[D * i + a] * dt;
    for (int a = 0; a < D; ++a)
      if (g.fixed[D * i + a] == 1) {
        g.momentum0[D * i + a] = 0.;
        g.momentum[D * i + a] = 0.;
      }
  }
  if (any_rigid) rigid_override<D>(c);
  for (int s : deformable) g2p_body<D>(c, s, g.mass.data(), g.momentum0.data(), g.momentum.data(), 0);
  if (any_rigid) rigid_advance<D>(c);
}

// ---------------------------------------------------------------------------
// MUSL with lumped mass, SolveExplicitSolidMechanics3D.jl:14-223.  The 3D solver
// applies no body force, builds the velocity gradient as L_ij = dN_i vI_j
// (SMatrix{3,3}(dNix*vIx, dNiy*vIx, dNiz*vIx, ...), :187-189), updates positions
// with nodalMomentum and the gradient with nodalMomentum2, which carries no
// Dirichlet condition; all as written.
template <int D>
void step_musl_lumped(Ctx<D>& c) {
  Grid<D>& g = c.g;
  const double dt = c.p.dt, alpha = c.p.alpha;
  zero<D>(g.mass);
  zero<D>(g.momentum0);
  zero<D>(c.mom2);
  zero<D>(g.force);
  std::vector<int> all(c.bodies.size());
  for (size_t s = 0; s < all.size(); ++s) all[s] = int(s);
  const double nobf[3] = {0.0, 0.0, 0.0};
  p2g_bodies<D>(c, all, g.mass.data(), g.momentum0.data(), g.force.data(), nullptr, nobf);
  auto bcs = [&]() {
    for (int64_t i = 0; i < g.nodeCount; ++i)
      for (int a = 0; a < D; ++a)
        if (g.fixed[D * i + a] == 1) {
          g.momentum0[D * i + a] = 0.;
          g.momentum[D * i + a] = 0.;
        }
  };
  for (int64_t i = 0; i < g.nodeCount; ++i)
    for (int a = 0; a < D; ++a) g.momentum[D * i + a] = g.momentum0[D * i + a] + g.force[D * i + a] * dt;
  bcs();
  // grid to particle 1 and particle to grid 2 (:113-139), in particle order
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  for (auto& b : c.bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
      if (S == 0) {
        c.status = MPM_ERR_OUT_OF_GRID;
        continue;
      }
      double vacc[D];
      for (int a = 0; a < D; ++a) vacc[a] = 0.;
      for (int i = 0; i < S; ++i) {
        const int64_t in = near[i];
        const double mI = g.mass[in];
        if (mI > 0) {
          const double mii = (1 / mI) * N[i];
          for (int a = 0; a < D; ++a)
            vacc[a] += (g.momentum[D * in + a] - alpha * g.momentum0[D * in + a]) * mii;
        }
      }
      double* vp = &b.vel[D * ip];
      for (int a = 0; a < D; ++a) vp[a] = alpha * vp[a] + vacc[a];
      const double mp = b.mass[ip];
      for (int i = 0; i < S; ++i)
        for (int a = 0; a < D; ++a) c.mom2[D * near[i] + a] += N[i] * mp * vp[a];
    }
  bcs();
  // particle to grid 2 / kinematics (:162-204)
  for (auto& b : c.bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
      if (S == 0) continue;
      double L[D * D], xxp[D];
      for (int q = 0; q < D * D; ++q) L[q] = 0.;
      for (int a = 0; a < D; ++a) xxp[a] = b.pos[D * ip + a];
      for (int i = 0; i < S; ++i) {
        const int64_t in = near[i];
        const double m = g.mass[in];
        if (m > 0.) {
          const double mii = 1 / m;
          double vI[D];
          for (int a = 0; a < D; ++a) vI[a] = mii * c.mom2[D * in + a];
          for (int a = 0; a < D; ++a) xxp[a] += N[i] * mii * dt * g.momentum[D * in + a];
          for (int j = 0; j < D; ++j)
            for (int r = 0; r < D; ++r) L[r + D * j] += dN[D * i + r] * vI[j];
        }
      }
      for (int a = 0; a < D; ++a) b.pos[D * ip + a] = xxp[a];
      kin_stress<D>(b, ip, L, dt, &c.status);
    }
}

// Banded Cholesky of the symmetric positive definite matrix whose lower band
// (half-bandwidth w) is A[i*(w+1) + (i-j)], j = i-w .. i; in place.  The 2D MUSL's
// blended mass matrix couples nodes at most nx+1 apart in index.
inline bool band_cholesky(std::vector<double>& A, int64_t n, int64_t w) {
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = std::max<int64_t>(0, i - w); j <= i; ++j) {
      double sum = A[i * (w + 1) + (i - j)];
      for (int64_t k = std::max<int64_t>(std::max<int64_t>(0, i - w), j - w); k < j; ++k)
        sum -= A[i * (w + 1) + (i - k)] * A[j * (w + 1) + (j - k)];
      if (i == j) {
        if (!(sum > 0.0)) return false;
        A[i * (w + 1)] = std::sqrt(sum);
      } else {
        A[i * (w + 1) + (i - j)] = sum / A[j * (w + 1)];
      }
    }
  return true;
}

inline void band_solve(const std::vector<double>& Lb, int64_t n, int64_t w, const double* b, double* x) {
  std::vector<double> y(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    double sum = b[i];
    for (int64_t k = std::max<int64_t>(0, i - w); k < i; ++k) sum -= Lb[i * (w + 1) + (i - k)] * y[k];
    y[i] = sum / Lb[i * (w + 1)];
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double sum = y[i];
    for (int64_t k = i + 1; k <= std::min<int64_t>(n - 1, i + w); ++k) sum -= Lb[k * (w + 1) + (k - i)] * x[k];
    x[i] = sum / Lb[i * (w + 1)];
  }
}

// MUSL with the blended consistent mass matrix, SolveExplicitSolidMechanics2D.jl:24-329:
// bmassMat = 0.1 Diagonal(m) + 0.9 M (M_ij = sum_p m_p N_i N_j, rows of massless nodes
// set to 1 on the diagonal), v0 = bmassMat \ p0 and v = v0 + bmassMat \ (dt f) per
// component (the reference's dense solve is a banded Cholesky here: same solution up to
// rounding).  The Dirichlet update of nodalMomentum that follows is never read by the
// particle updates, so fixed nodes do not constrain this solver; as written.
void step_musl_consistent(Ctx<2>& c) {
  constexpr int D = 2;
  Grid<2>& g = c.g;
  const double dt = c.p.dt, alpha = c.p.alpha;
  // nodes of one particle's support differ by at most K-1 per axis
  const int64_t K = g.basis == MPM_BASIS_LINEAR ? 2 : (g.basis == MPM_BASIS_QUAD_BSPLINE ? 3 : 4);
  const int64_t n = g.nodeCount, w = (K - 1) * (g.nn[0] + 1);
  zero<D>(g.mass);
  zero<D>(g.momentum0);
  zero<D>(g.force);
  std::vector<double> Mb(static_cast<size_t>(n * (w + 1)), 0.0);
  int64_t near[kMaxSupport];
  double N[kMaxSupport], dN[kMaxSupport * D];
  const double* body = c.p.body_force;
  for (auto& b : c.bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
      if (S == 0) {
        c.status = MPM_ERR_OUT_OF_GRID;
        continue;
      }
      const double fVolume = b.vol[ip], fMass = b.mass[ip];
      const double* vp = &b.vel[D * ip];
      const double* sigma = &b.stress[D * D * ip];
      for (int i = 0; i < S; ++i) {
        const int64_t id = near[i];
        const double Ni = N[i], Nim = Ni * fMass;
        g.mass[id] += Nim;
        for (int j = 0; j < S; ++j)
          if (near[j] <= id) Mb[id * (w + 1) + (id - near[j])] += Nim * N[j];
        for (int a = 0; a < D; ++a) g.momentum0[D * id + a] += Nim * vp[a];
        for (int a = 0; a < D; ++a) {
          double sa = sigma[a] * dN[D * i] + sigma[a + D] * dN[D * i + 1];
          g.force[D * id + a] += -fVolume * sa + fMass * body[a] * Ni;
        }
      }
    }
  const double eps = 0.1;
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t k = 0; k <= w; ++k) Mb[i * (w + 1) + k] *= (1 - eps);
    Mb[i * (w + 1)] += eps * g.mass[i];
    if (g.mass[i] == 0.) Mb[i * (w + 1)] = 1.0;
  }
  if (!band_cholesky(Mb, n, w)) {
    c.status = MPM_ERR_SOLVER;
    return;
  }
  std::vector<double> rhs(static_cast<size_t>(n)), sol(static_cast<size_t>(n));
  for (int a = 0; a < D; ++a) {
    for (int64_t i = 0; i < n; ++i) rhs[i] = g.momentum0[D * i + a];
    band_solve(Mb, n, w, rhs.data(), sol.data());
    for (int64_t i = 0; i < n; ++i) c.v0[D * i + a] = sol[i];
    for (int64_t i = 0; i < n; ++i) rhs[i] = dt * g.force[D * i + a];
    band_solve(Mb, n, w, rhs.data(), sol.data());
    for (int64_t i = 0; i < n; ++i) c.gv[D * i + a] = c.v0[D * i + a] + sol[i];
  }
  // update grid (:168-186): nodalMomentum and the Dirichlet conditions, which no
  // particle update below reads
  for (int64_t i = 0; i < n; ++i) {
    for (int a = 0; a < D; ++a) g.momentum[D * i + a] = g.momentum0[D * i + a] + g.force[D * i + a] * dt;
    for (int a = 0; a < D; ++a)
      if (g.fixed[D * i + a] == 1) {
        g.momentum0[D * i + a] = 0.;
        g.momentum[D * i + a] = 0.;
      }
  }
  // grid to particle 1: velocities (:198-224)
  for (auto& b : c.bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
      if (S == 0) continue;
      double vacc[D] = {0., 0.};
      for (int i = 0; i < S; ++i) {
        const int64_t in = near[i];
        if (g.mass[in] > 0)
          for (int a = 0; a < D; ++a) vacc[a] += N[i] * (c.gv[D * in + a] - alpha * c.v0[D * in + a]);
      }
      double* vp = &b.vel[D * ip];
      for (int a = 0; a < D; ++a) vp[a] = alpha * vp[a] + vacc[a];
    }
  // particle update 2: positions, gradient, F, stress (:245-290)
  for (auto& b : c.bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const int S = support<D>(g, &b.pos[D * ip], near, N, dN);
      if (S == 0) continue;
      double L[D * D] = {0., 0., 0., 0.}, xxp[D];
      for (int a = 0; a < D; ++a) xxp[a] = b.pos[D * ip + a];
      for (int i = 0; i < S; ++i) {
        const int64_t in = near[i];
        if (g.mass[in] > 0.) {
          const double* vI = &c.gv[D * in];
          for (int a = 0; a < D; ++a) xxp[a] += (N[i] * vI[a]) * dt;
          for (int j = 0; j < D; ++j)
            for (int a = 0; a < D; ++a) L[a + D * j] += dN[D * i + j] * vI[a];
        }
      }
      for (int a = 0; a < D; ++a) b.pos[D * ip + a] = xxp[a];
      kin_stress<D>(b, ip, L, dt, &c.status);
    }
}

// One USL step with one velocity field per body and the contact correction.
template <int D>
void step_contact(Ctx<D>& c) {
  Grid<D>& g = c.g;
  size_t nb = c.bodies.size();
  double dt = c.p.dt;
  zero<D>(g.mass);
  std::fill(c.sysp.begin(), c.sysp.end(), 0.0);
  for (size_t s = 0; s < nb; ++s) {
    std::vector<double>& m = c.bm[s];
    std::vector<double>& v0 = c.bv0[s];
    std::vector<double>& v = c.bv[s];
    std::vector<double>& nrm = c.bnormal[s];
    std::fill(m.begin(), m.end(), 0.0);
    std::fill(v0.begin(), v0.end(), 0.0);
    std::fill(nrm.begin(), nrm.end(), 0.0);
    std::vector<double> f(static_cast<size_t>(D) * g.nodeCount, 0.0);
    std::vector<int> one(1, int(s));
    p2g_bodies<D>(c, one, m.data(), v0.data(), f.data(), nrm.data());
    // SolveExplicitFEMP2DContact.jl:248-266: p = p0 + f dt, system sums, velocities, BCs
    for (int64_t i = 0; i < g.nodeCount; ++i) {
      for (int a = 0; a < D; ++a) v[D * i + a] = v0[D * i + a] + f[D * i + a] * dt;
      g.mass[i] += m[i];
      for (int a = 0; a < D; ++a) c.sysp[D * i + a] += v[D * i + a];
      if (m[i] > 0.0) {
        for (int a = 0; a < D; ++a) {
          v0[D * i + a] /= m[i];
          v[D * i + a] /= m[i];
        }
      }
      for (int a = 0; a < D; ++a)
        if (g.fixed[D * i + a] == 1) {
          v0[D * i + a] = 0.;
          v[D * i + a] = 0.;
        }
    }
  }
  // contact correction at nodes touched by two bodies (:311-387)
  double fric = c.p.friction;
  for (int64_t i = 0; i < g.nodeCount; ++i) {
    int s1 = -1, s2 = -1;
    for (size_t s = 0; s < nb; ++s)
      if (c.bm[s][i] > 0.0) {
        if (s1 < 0) s1 = int(s);
        else if (s2 < 0) s2 = int(s);
      }
    if (s2 < 0) continue;
    double n[D], nn = 0;
    for (int a = 0; a < D; ++a) n[a] = c.bnormal[s1][D * i + a] - c.bnormal[s2][D * i + a];
    for (int a = 0; a < D; ++a) nn += n[a] * n[a];
    nn = std::sqrt(nn);
    for (int a = 0; a < D; ++a) n[a] = n[a] / nn;
    int ss[2] = {s1, s2};
    for (int is = 0; is < 2; ++is) {
      int s = ss[is];
      double nI[D];
      for (int a = 0; a < D; ++a) nI[a] = is == 0 ? n[a] : -n[a];
      double* velo1 = &c.bv[s][D * i];
      double dv[D], D1 = 0;
      for (int a = 0; a < D; ++a) dv[a] = velo1[a] - c.sysp[D * i + a] / g.mass[i];
      for (int a = 0; a < D; ++a) D1 += dv[a] * nI[a];
      if (D1 > 0) {
        // Coulomb branch (:376-380); with no tangential slip (C1 == 0) its
        // (muPrime/|C1|) is 0/0 in the reference, whose limit is the normal-only update
        if (D == 2 && fric > 0 && (dv[0] * nI[1] - dv[1] * nI[0]) != 0.0) {
          double C1 = dv[0] * nI[1] - dv[1] * nI[0];
          double absC1 = std::fabs(C1);
          double mup = std::min(fric, absC1 / D1);
          double t0 = nI[0] + (mup / absC1) * (nI[1] * C1);
          double t1 = nI[1] + (mup / absC1) * (-nI[0] * C1);
          velo1[0] = velo1[0] - D1 * t0;
          velo1[1] = velo1[1] - D1 * t1;
        } else {
          for (int a = 0; a < D; ++a) velo1[a] = velo1[a] - D1 * nI[a];
        }
      }
    }
  }
  for (size_t s = 0; s < nb; ++s)
    g2p_body<D>(c, int(s), c.bm[s].data(), c.bv0[s].data(), c.bv[s].data(), 1);
}

template <int D>
int create(const mpm_grid_desc* gd, const mpm_body_desc* bd, int nb, const mpm_params* p,
           Ctx<D>** out) {
  Ctx<D>* c = new Ctx<D>();
  c->p = *p;
  Grid<D>& g = c->g;
  g.basis = p->basis;
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
        int64_t idx = g.nodeCountXY * k + g.nn[0] * j + i;
        g.pos[D * idx + 0] = g.xmin[0] + double(i) * g.dx[0];
        g.pos[D * idx + 1] = g.xmin[1] + double(j) * g.dx[1];
        if (D == 3) g.pos[D * idx + 2] = g.xmin[2] + double(k) * g.dx[2];
      }
  g.mass.assign(g.nodeCount, 0.0);
  g.momentum0.assign(size_t(D) * g.nodeCount, 0.0);
  g.momentum.assign(size_t(D) * g.nodeCount, 0.0);
  g.force.assign(size_t(D) * g.nodeCount, 0.0);
  g.fixed.assign(size_t(D) * g.nodeCount, 0);
  if (gd->fixed_nodes)
    std::memcpy(g.fixed.data(), gd->fixed_nodes, sizeof(int64_t) * D * g.nodeCount);
  constexpr int PS = (D == 2) ? 3 : 9;
  for (int s = 0; s < nb; ++s) {
    Body<D> b;
    const mpm_body_desc& d = bd[s];
    b.n = d.count;
    b.mat = make_material(d.mat);
    auto cp = [&](std::vector<double>& v, const double* src, size_t per, double fillv) {
      v.assign(per * size_t(b.n), fillv);
      if (src) std::memcpy(v.data(), src, sizeof(double) * per * b.n);
    };
    cp(b.pos, d.pos, D, 0.0);
    cp(b.vel, d.velocity, D, 0.0);
    cp(b.mass, d.mass, 1, 0.0);
    cp(b.vol, d.volume, 1, 0.0);
    cp(b.vol0, d.volume_initial, 1, 0.0);
    cp(b.F, d.F, D * D, 0.0);
    if (!d.F)
      for (int64_t ip = 0; ip < b.n; ++ip)
        for (int a = 0; a < D; ++a) b.F[D * D * ip + a * (D + 1)] = 1.0;
    cp(b.strain, d.strain, D * D, 0.0);
    cp(b.stress, d.stress, D * D, 0.0);
    cp(b.alpha, d.alpha, 1, 0.0);
    cp(b.alphadot, d.alphadot, 1, 0.0);
    const bool dmg = D == 3 && d.mat.type == MPM_MAT_JOHNSON_COOK_DAMAGE;
    cp(b.pstrain, dmg ? nullptr : d.pstrain, PS, 0.0);
    // JohnsonCookDamage starts every particle at Tr (Material.jl:507)
    cp(b.damage_init, dmg ? d.damage_init : nullptr, 1, 0.0);
    cp(b.dam, dmg ? d.damage : nullptr, 1, 0.0);
    cp(b.temp, dmg ? d.temperature : nullptr, 1, dmg ? d.mat.Tr : 0.0);
    cp(b.vmstr, d.vmstr, 1, 0.0);
    b.has_youngs = d.youngs != nullptr;
    if (b.has_youngs) cp(b.youngs, d.youngs, 1, 0.0);
    if (d.mat.type == MPM_MAT_RIGID) {
      b.rigid = true;
      b.rigid_fixed = d.mat.fixed != 0;
      for (int a = 0; a < D; ++a) b.vr[a] = d.mat.v_rigid[a];
    }
    c->bodies.push_back(std::move(b));
  }
  if (p->algorithm == MPM_ALG_MUSL) {
    c->mom2.assign(size_t(D) * g.nodeCount, 0.0);
    c->v0.assign(size_t(D) * g.nodeCount, 0.0);
    c->gv.assign(size_t(D) * g.nodeCount, 0.0);
  }
  if (p->contact) {
    c->bm.assign(nb, std::vector<double>(g.nodeCount, 0.0));
    c->bv0.assign(nb, std::vector<double>(size_t(D) * g.nodeCount, 0.0));
    c->bv.assign(nb, std::vector<double>(size_t(D) * g.nodeCount, 0.0));
    c->bnormal.assign(nb, std::vector<double>(size_t(D) * g.nodeCount, 0.0));
    c->sysp.assign(size_t(D) * g.nodeCount, 0.0);
  }
  *out = c;
  return MPM_OK;
}

struct Handle {
  int dim;
  void* ctx;
};

}  // namespace

namespace {
template <int D>
static int step_impl(Ctx<D>* c, int64_t nsteps, double* t) {
  c->status = MPM_OK;
  for (int64_t k = 0; k < nsteps; ++k) {
    if (c->p.algorithm == MPM_ALG_MUSL) {
      if constexpr (D == 2) step_musl_consistent(*c);
      else step_musl_lumped<D>(*c);
    } else if (c->p.contact) {
      step_contact<D>(*c);
    } else {
      step_single<D>(*c);
    }
    if (t) *t += c->p.dt;
  }
  if (c->status == MPM_ERR_OUT_OF_GRID) return fail(c->status, "particle outside the grid");
  if (c->status == MPM_ERR_NEGATIVE_J) return fail(c->status, "det F <= 0 at a particle");
  if (c->status == MPM_ERR_SOLVER) return fail(c->status, "MUSL mass matrix not positive definite");
  return c->status;
}

template <int D>
static int download_impl(Ctx<D>* c, int body, const mpm_body_view* v) {
  if (body < 0 || body >= int(c->bodies.size())) return fail(MPM_ERR_ARG, "bad body index");
  Body<D>& b = c->bodies[body];
  constexpr int PS = (D == 2) ? 3 : 9;
  auto put = [&](double* dst, const std::vector<double>& src, size_t per) {
    if (dst) std::memcpy(dst, src.data(), sizeof(double) * per * b.n);
  };
  put(v->pos, b.pos, D);
  put(v->velocity, b.vel, D);
  put(v->volume, b.vol, 1);
  put(v->F, b.F, D * D);
  put(v->strain, b.strain, D * D);
  put(v->stress, b.stress, D * D);
  put(v->alpha, b.alpha, 1);
  if (D == 3 && b.mat.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    put(v->damage_init, b.damage_init, 1);
    put(v->damage, b.dam, 1);
    put(v->temperature, b.temp, 1);
  } else {
    put(v->pstrain, b.pstrain, PS);
  }
  put(v->vmstr, b.vmstr, 1);
  put(v->alphadot, b.alphadot, 1);
  return MPM_OK;
}

template <int D>
static int grid_impl(Ctx<D>* c, double* m, double* p0, double* p, double* f) {
  Grid<D>& g = c->g;
  if (m) std::memcpy(m, g.mass.data(), sizeof(double) * g.nodeCount);
  if (p0) std::memcpy(p0, g.momentum0.data(), sizeof(double) * D * g.nodeCount);
  if (p) std::memcpy(p, g.momentum.data(), sizeof(double) * D * g.nodeCount);
  if (f) std::memcpy(f, g.force.data(), sizeof(double) * D * g.nodeCount);
  return MPM_OK;
}

template <int D>
static int energies_impl(Ctx<D>* c, double* ke, double* se, double* mom) {
  double KE = 0., SE = 0.;
  double P[3] = {0, 0, 0};
  for (auto& b : c->bodies)
    for (int64_t ip = 0; ip < b.n; ++ip) {
      const double* v = &b.vel[D * ip];
      double vv = v[0] * v[0] + v[1] * v[1];
      if (D == 3) vv = vv + v[2] * v[2];
      KE += 0.5 * b.mass[ip] * vv;
      const double* s = &b.stress[D * D * ip];
      const double* e = &b.strain[D * D * ip];
      double se_ = s[0] * e[0];
      for (int k = 1; k < D * D; ++k) se_ = se_ + s[k] * e[k];
      SE += 0.5 * b.vol[ip] * se_;
      for (int a = 0; a < D; ++a) P[a] += b.mass[ip] * v[a];
    }
  if (ke) *ke = KE;
  if (se) *se = SE;
  if (mom)
    for (int a = 0; a < D; ++a) mom[a] = P[a];
  return MPM_OK;
}
}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_create(const mpm_grid_desc* grid, const mpm_body_desc* bodies, int32_t nbodies,
                  const mpm_params* params, void** out) {
  if (!grid || !params || !out || nbodies < 0 || (nbodies > 0 && !bodies))
    return fail(MPM_ERR_ARG, "oracle_create: null argument");
  if (grid->dim != 2 && grid->dim != 3) return fail(MPM_ERR_ARG, "oracle_create: dim must be 2 or 3");
  for (int a = 0; a < grid->dim; ++a)
    if (grid->nodes[a] < 2) return fail(MPM_ERR_ARG, "oracle_create: need >= 2 nodes per axis");
  if (params && params->basis != MPM_BASIS_LINEAR && params->basis != MPM_BASIS_QUAD_BSPLINE &&
      params->basis != MPM_BASIS_CUBIC_BSPLINE)
    return fail(MPM_ERR_ARG, "oracle_create: unknown basis");
  for (int a = 0; params && a < grid->dim; ++a)
    if (grid->nodes[a] < (params->basis == MPM_BASIS_CUBIC_BSPLINE ? 4 : 3) && params->basis != MPM_BASIS_LINEAR)
      return fail(MPM_ERR_ARG, "oracle_create: B-spline bases need 3 (quadratic) or 4 (cubic) nodes per axis");
  for (int s = 0; s < nbodies; ++s)
    if (bodies[s].mat.type == MPM_MAT_RIGID && (params->algorithm != MPM_ALG_USL || params->contact))
      return fail(MPM_ERR_UNSUPPORTED, "oracle_create: rigid solids need USL with one velocity field");
  Handle* h = new Handle{grid->dim, nullptr};
  if (grid->dim == 2) {
    Ctx<2>* c;
    create<2>(grid, bodies, nbodies, params, &c);
    h->ctx = c;
  } else {
    Ctx<3>* c;
    create<3>(grid, bodies, nbodies, params, &c);
    h->ctx = c;
  }
  *out = h;
  return MPM_OK;
}

int oracle_set_threads(void* hv, int32_t threads) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return fail(MPM_ERR_ARG, "null handle");
#ifndef _OPENMP
  threads = 1;
#endif
  if (threads < 1) threads = 1;
  if (h->dim == 2) static_cast<Ctx<2>*>(h->ctx)->threads = threads;
  else static_cast<Ctx<3>*>(h->ctx)->threads = threads;
  return MPM_OK;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// The shape functions of one point (getShapeAndGradient, Basis.jl:219-251,
// 292-332 and the B-spline forms :374-820) on the grid a descriptor describes:
// fills near[] (0-based node ids), N[] and dN[] (dim per node) and returns the
// support size, 0 when the point's cell lies outside the grid.  For the
// known-answer tests of the basis.
int oracle_shape(const mpm_grid_desc* gd, int32_t basis, const double* x, int64_t* near, double* N, double* dN) {
  if (!gd || !x || !near || !N || !dN || (gd->dim != 2 && gd->dim != 3)) return -1;
  auto run = [&](auto dimtag) -> int {
    constexpr int D = decltype(dimtag)::value;
    Grid<D> g;
    g.basis = basis;
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
          int64_t idx = g.nodeCountXY * k + g.nn[0] * j + i;
          g.pos[D * idx + 0] = g.xmin[0] + double(i) * g.dx[0];
          g.pos[D * idx + 1] = g.xmin[1] + double(j) * g.dx[1];
          if (D == 3) g.pos[D * idx + 2] = g.xmin[2] + double(k) * g.dx[2];
        }
    return support<D>(g, x, near, N, dN);
  };
  if (gd->dim == 2) return run(std::integral_constant<int, 2>{});
  return run(std::integral_constant<int, 3>{});
}


int oracle_step(void* hv, int64_t nsteps, double* t_inout) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return fail(MPM_ERR_ARG, "null handle");
  if (h->dim == 2) return step_impl<2>(static_cast<Ctx<2>*>(h->ctx), nsteps, t_inout);
  return step_impl<3>(static_cast<Ctx<3>*>(h->ctx), nsteps, t_inout);
}


int oracle_download(void* hv, int32_t body, const mpm_body_view* out) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h || !out) return fail(MPM_ERR_ARG, "null argument");
  if (h->dim == 2) return download_impl<2>(static_cast<Ctx<2>*>(h->ctx), body, out);
  return download_impl<3>(static_cast<Ctx<3>*>(h->ctx), body, out);
}


int oracle_download_grid(void* hv, double* mass, double* momentum0, double* momentum,
                         double* force) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return fail(MPM_ERR_ARG, "null handle");
  if (h->dim == 2) return grid_impl<2>(static_cast<Ctx<2>*>(h->ctx), mass, momentum0, momentum, force);
  return grid_impl<3>(static_cast<Ctx<3>*>(h->ctx), mass, momentum0, momentum, force);
}


int oracle_energies(void* hv, double* ke, double* se, double* momentum) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return fail(MPM_ERR_ARG, "null handle");
  if (h->dim == 2) return energies_impl<2>(static_cast<Ctx<2>*>(h->ctx), ke, se, momentum);
  return energies_impl<3>(static_cast<Ctx<3>*>(h->ctx), ke, se, momentum);
}

int oracle_destroy(void* hv) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return MPM_OK;
  if (h->dim == 2) delete static_cast<Ctx<2>*>(h->ctx);
  else delete static_cast<Ctx<3>*>(h->ctx);
  delete h;
  return MPM_OK;
}

}  // extern "C"
