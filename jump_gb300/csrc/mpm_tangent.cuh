// mpm_tangent.cuh -- forward-mode derivatives (tangents) of the USL step, for
// batched problems that each depend on one scalar (e.g. a Young's modulus).
//
// Every primal quantity q of a step gets a tangent q' = dq/ds.  The primal
// device functions run unchanged inside these kernels (same thread, same
// particle), and the tangent code recomputes the primal intermediate values
// it needs:
//
//   tan_p2g    the primal P2G of the particle, then (P2G does not change
//              particles) its tangent scatter:
//                m'_I  += m N'                        N'  = grad N . x'
//                p0'_I += m (N' v + N v')
//                f'_I  += -(V' sig + V sig') grad N - V sig (grad N)' + m b N'
//                n'_I  += m (grad N)'                 (grad N)' = H x'
//              H is the Hessian of the multilinear hat (off-diagonal only).
//   tan_grid   after the primal grid update (own launch): the tangents of
//              p = p0 + f dt, the Dirichlet mask, vdt = p/m dt,
//              dv = (p - p0)/m, and of the frictionless contact correction
//              (system velocity, common normal, approach rate D1 > 0).
//   tan_g2p    the tangent G2P from the state before the step, then the
//              primal G2P of the same particle, which overwrites that state:
//                x' += N' vdt + N vdt',  v' += N' dv + N dv'
//                (L dt)' = vdt' (x) grad N + vdt (x) (grad N)'
//                F_new' = F' (I + L dt) + F (L dt)',  J' = cof(F_new) : F_new'
//                V' = J' V0,  eps' += sym((L dt)'),  sig' from the material
//              with lambda' and mu' the body's seeds.
// The derivative is that of the discrete map within the current cells and
// branches (the hat basis has kinks at nodes and cell faces, the contact
// correction switches on D1 > 0).  FP64 only.
#pragma once

#include "mpm_wide.cuh"

namespace jmpm {

// tangent particle fields: x' (D) v' (D) F' (D*D) eps' (S) sig' (S) V'
template <int D>
struct TanLayout {
  static constexpr int S = (D == 2) ? 3 : 6;
  static constexpr int XD = 0, VD = D, FD = 2 * D, ED = 2 * D + D * D, SD = ED + S, VOLD = SD + S;
  static constexpr int NT = VOLD + 1;
};

struct TanBody {
  PartP tp;       // tangent particle fields (same begin/count/pitch as the body's PartP)
  NodeP tnd;      // tangent node field: m' p0' f' n' vdt' dv'
  double dlam, dmu;
};

struct TanInst {
  ContactP tcp;   // tangent fields of the problem's node fields (one per body in contact mode)
};

// off-diagonal second derivatives of hat corner k: xy, xz, yz
template <int D>
__device__ __forceinline__ void hat_hessian(const Hat<D, double>& h, int k, double* Hk) {
  const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
  const double gx = bx ? h.gh[0] : h.gl[0], gy = by ? h.gh[1] : h.gl[1];
  if constexpr (D == 2) {
    Hk[0] = gx * gy;
    Hk[1] = Hk[2] = 0.0;
  } else {
    const double Nx = bx ? h.Nh[0] : h.Nl[0], Ny = by ? h.Nh[1] : h.Nl[1], Nz = bz ? h.Nh[2] : h.Nl[2];
    const double gz = bz ? h.gh[2] : h.gl[2];
    Hk[0] = gx * gy * Nz;
    Hk[1] = gx * Ny * gz;
    Hk[2] = Nx * gy * gz;
  }
}

// (grad N)' = H x'
template <int D>
__device__ __forceinline__ void grad_tangent(const double* Hk, const double* xd, double* gd) {
  if constexpr (D == 2) {
    gd[0] = Hk[0] * xd[1];
    gd[1] = Hk[0] * xd[0];
  } else {
    gd[0] = Hk[0] * xd[1] + Hk[1] * xd[2];
    gd[1] = Hk[0] * xd[0] + Hk[2] * xd[2];
    gd[2] = Hk[1] * xd[0] + Hk[2] * xd[1];
  }
}

template <int D>
__device__ __forceinline__ double& tf(const PartP& tp, int f, int64_t p) {
  return static_cast<double*>(tp.base)[int64_t(f) * tp.pitch + p];
}

// primal P2G of the particle (p2g_particle, unchanged) followed by its tangent scatter
template <int D>
__global__ void __launch_bounds__(256) tan_p2g_kernel(const WideBody* __restrict__ bodies,
                                                      const TanBody* __restrict__ tbodies,
                                                      const WideInst* __restrict__ inst,
                                                      const WideTile* __restrict__ tiles, unsigned* status) {
  using L = Layout<D>;
  using T = TanLayout<D>;
  __shared__ WideBody sB;
  __shared__ TanBody sT;
  __shared__ GridP sG;
  __shared__ double sGrav[3];
  const WideTile tl = tiles[blockIdx.x];
  stage(&sB, bodies + tl.body);
  stage(&sT, tbodies + tl.body);
  __syncthreads();
  const WideInst* I = inst + sB.inst;
  stage(&sG, &I->g);
  if (threadIdx.x < 3) sGrav[threadIdx.x] = I->grav[threadIdx.x];
  __syncthreads();
  const int64_t t = tl.start + threadIdx.x;
  if (sGrav[0] != 0.0 || sGrav[1] != 0.0 || sGrav[2] != 0.0)
    p2g_particle<D, double, true>(sG, sB.nd, sB.pp, t, sGrav[0], sGrav[1], sGrav[2], status + sB.inst);
  else
    p2g_particle<D, double, false>(sG, sB.nd, sB.pp, t, 0.0, 0.0, 0.0, status + sB.inst);
  if (t >= sB.pp.count) return;
  const int64_t p = sB.pp.begin + t;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) x[a] = *field<double>(sB.pp, L::X + a, p);
  Hat<D, double> h;
  if (!hat<D, double>(sG, x, h)) return;  // reported by the primal P2G
  Corners<D, double> cr;
  corners<D, double>(sG, h, cr);
  const double m = *field<double>(sB.pp, L::M, p), V = *field<double>(sB.pp, L::VOL, p);
  const double Vd = tf<D>(sT.tp, T::VOLD, p);
  double v[D], vd[D], xd[D], sg[L::S], sd[L::S];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    v[a] = *field<double>(sB.pp, L::V + a, p);
    vd[a] = tf<D>(sT.tp, T::VD + a, p);
    xd[a] = tf<D>(sT.tp, T::XD + a, p);
  }
#pragma unroll
  for (int c = 0; c < L::S; ++c) {
    sg[c] = *field<double>(sB.pp, L::SIG + c, p);
    sd[c] = tf<D>(sT.tp, T::SD + c, p);
  }
  // per particle: -(V' sig + V sig') and -V sig, so each corner costs two dot products
  double A[L::S], B[L::S], mg[D], mv[D], mvd[D];
#pragma unroll
  for (int c = 0; c < L::S; ++c) {
    A[c] = -(Vd * sg[c] + V * sd[c]);
    B[c] = -V * sg[c];
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    mg[a] = m * sGrav[a];
    mv[a] = m * v[a];
    mvd[a] = m * vd[a];
  }
  const NodeP& tn = sT.tnd;
  const int64_t Nn = tn.nodeCount;
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    double Hk[3], gd[D];
    hat_hessian<D>(h, k, Hk);
    grad_tangent<D>(Hk, xd, gd);
    const double N = cr.N[k];
    double Nd = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) Nd += cr.dN[k][a] * xd[a];
    const int64_t n = cr.node[k];
    atomicAdd(tn.m + n, m * Nd);
#pragma unroll
    for (int a = 0; a < D; ++a) atomicAdd(tn.p0 + a * Nn + n, Nd * mv[a] + N * mvd[a]);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double fa = mg[a] * Nd;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const int c = sym<D>(a, j);
        fa += A[c] * cr.dN[k][j] + B[c] * gd[j];
      }
      atomicAdd(tn.f + a * Nn + n, fa);
    }
    if (tn.nrm)
#pragma unroll
      for (int a = 0; a < D; ++a) atomicAdd(tn.nrm + a * Nn + n, m * gd[a]);
  }
}

// tangent of grid_node (single velocity field)
template <int D>
__device__ __forceinline__ void tan_grid_node(const NodeP& nd, const NodeP& td, int64_t i, double dt, double tol) {
  const int64_t Nn = nd.nodeCount;
  const double m = nd.m[i];
  if (!(m > tol)) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      td.vdt[a * Nn + i] = 0.0;
      td.dv[a * Nn + i] = 0.0;
    }
    return;
  }
  const double md = td.m[i];
  const unsigned fx = nd.fixed[i];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double p0 = nd.p0[a * Nn + i], p = __dadd_rn(p0, __dmul_rn(nd.f[a * Nn + i], dt));
    double p0d = td.p0[a * Nn + i], pd = p0d + td.f[a * Nn + i] * dt;
    if (fx & (1u << a)) p0 = p = p0d = pd = 0.0;
    td.vdt[a * Nn + i] = (pd - p * md / m) / m * dt;
    td.dv[a * Nn + i] = ((pd - p0d) - (p - p0) * md / m) / m;
  }
}

// tangent of contact_node, frictionless correction
template <int D>
__device__ __forceinline__ void tan_contact_node(const ContactP& cp, const ContactP& tcp, int64_t i, double dt,
                                                 double tol) {
  const int64_t Nn = cp.body[0].nodeCount;
  const unsigned fx = cp.body[0].fixed[i];
  double mb[kMaxContactBodies], v[kMaxContactBodies][D], v0[kMaxContactBodies][D];
  double vd[kMaxContactBodies][D], v0d[kMaxContactBodies][D];
  double mS = 0.0, mSd = 0.0, pS[D], pSd[D];
#pragma unroll
  for (int a = 0; a < D; ++a) pS[a] = pSd[a] = 0.0;
  int s1 = -1, s2 = -1;
#pragma unroll
  for (int b = 0; b < kMaxContactBodies; ++b) {
    if (b >= cp.nb) break;
    const NodeP& nd = cp.body[b];
    const NodeP& td = tcp.body[b];
    const double m = nd.m[i], md = td.m[i];
    mb[b] = m;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      // the primal statements with the primal's rounding, so the branches match
      const double p0 = nd.p0[a * Nn + i], p = __dadd_rn(p0, __dmul_rn(nd.f[a * Nn + i], dt));
      const double p0d = td.p0[a * Nn + i], pd = p0d + td.f[a * Nn + i] * dt;
      pS[a] += p;
      pSd[a] += pd;
      v0[b][a] = p0;
      v[b][a] = p;
      v0d[b][a] = p0d;
      vd[b][a] = pd;
    }
    mS += m;
    mSd += md;
    if (m > 0.0) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        v0[b][a] = v0[b][a] / m;
        v[b][a] = v[b][a] / m;
        v0d[b][a] = (v0d[b][a] - v0[b][a] * md) / m;
        vd[b][a] = (vd[b][a] - v[b][a] * md) / m;
      }
      if (s1 < 0) s1 = b;
      else if (s2 < 0) s2 = b;
    }
#pragma unroll
    for (int a = 0; a < D; ++a)
      if (fx & (1u << a)) v0[b][a] = v[b][a] = v0d[b][a] = vd[b][a] = 0.0;
  }
  if (s2 >= 0) {
    double n[D], ndt[D], nn = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      n[a] = cp.body[s1].nrm[a * Nn + i] - cp.body[s2].nrm[a * Nn + i];
      ndt[a] = tcp.body[s1].nrm[a * Nn + i] - tcp.body[s2].nrm[a * Nn + i];
      nn += n[a] * n[a];
    }
    nn = sqrt(nn);
    double dot = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      n[a] = n[a] / nn;
      dot += n[a] * ndt[a];
    }
#pragma unroll
    for (int a = 0; a < D; ++a) ndt[a] = (ndt[a] - n[a] * dot) / nn;
#pragma unroll
    for (int is = 0; is < 2; ++is) {
      const int s = is == 0 ? s1 : s2;
      const double sgn = is == 0 ? 1.0 : -1.0;
      double D1 = 0.0, D1d = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const double vcm = pS[a] / mS, vcmd = (pSd[a] - vcm * mSd) / mS;
        D1 += (v[s][a] - vcm) * (sgn * n[a]);  // the primal's expression, so the branch matches
        D1d += (vd[s][a] - vcmd) * (sgn * n[a]) + (v[s][a] - vcm) * (sgn * ndt[a]);
      }
      if (D1 > 0.0) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
          v[s][a] -= D1 * (sgn * n[a]);
          vd[s][a] -= D1d * (sgn * n[a]) + D1 * (sgn * ndt[a]);
        }
      }
    }
  }
#pragma unroll
  for (int b = 0; b < kMaxContactBodies; ++b) {
    if (b >= cp.nb) break;
    const NodeP& td = tcp.body[b];
    const bool live = mb[b] > tol;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      td.vdt[a * Nn + i] = live ? vd[b][a] * dt : 0.0;
      td.dv[a * Nn + i] = live ? vd[b][a] - v0d[b][a] : 0.0;
    }
  }
}

template <int D>
__global__ void __launch_bounds__(256) tan_grid_kernel(const WideInst* __restrict__ inst,
                                                       const TanInst* __restrict__ tinst,
                                                       const int* __restrict__ blk_inst,
                                                       const uint32_t* __restrict__ list,
                                                       const uint32_t* __restrict__ count) {
  const int64_t work = int64_t(*count) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const WideInst* I;
    const int64_t i = wide_node<D>(inst, blk_inst, list, w, I);
    if (i < 0) continue;
    const TanInst& TI = tinst[I - inst];
    if (I->contact) tan_contact_node<D>(I->cp, TI.tcp, i, I->dt, I->tol);
    else tan_grid_node<D>(I->cp.body[0], TI.tcp.body[0], i, I->dt, I->tol);
  }
}

// zero the tangent accumulators of the listed blocks
template <int D>
__global__ void __launch_bounds__(256) tan_clear_kernel(const WideInst* __restrict__ inst,
                                                        const TanInst* __restrict__ tinst,
                                                        const int* __restrict__ blk_inst,
                                                        const uint32_t* __restrict__ list,
                                                        const uint32_t* __restrict__ count) {
  const int64_t work = int64_t(*count) * 64;
  for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < work; w += int64_t(gridDim.x) * blockDim.x) {
    const WideInst* I;
    const int64_t i = wide_node<D>(inst, blk_inst, list, w, I);
    if (i < 0) continue;
    const TanInst& TI = tinst[I - inst];
    const int nf = I->contact ? I->cp.nb : 1;
    for (int b = 0; b < nf; ++b) {
      const NodeP& td = TI.tcp.body[b];
      const int64_t Nn = td.nodeCount;
      td.m[i] = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        td.p0[a * Nn + i] = 0.0;
        td.f[a * Nn + i] = 0.0;
        if (td.nrm) td.nrm[a * Nn + i] = 0.0;
      }
    }
  }
}

// cofactor matrix of a column-major D x D matrix (C[i + D j] = d det / d A_ij)
template <int D>
__device__ __forceinline__ void cofactor(const double* A, double* C) {
  if constexpr (D == 2) {
    C[0] = A[3];
    C[1] = -A[2];
    C[2] = -A[1];
    C[3] = A[0];
  } else {
    auto a = [&](int i, int j) { return A[i + 3 * j]; };
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        C[i + 3 * j] = a(i1, j1) * a(i2, j2) - a(i1, j2) * a(i2, j1);
      }
  }
}

// tangent G2P of the particle from the state before the step
template <int D>
__device__ __forceinline__ void tan_g2p_particle(const WideBody& sB, const TanBody& sT, const GridP& sG, int64_t t);

// tangent G2P, then the primal G2P (g2p_particle, unchanged) of the same particle
template <int D>
__global__ void __launch_bounds__(256) tan_g2p_kernel(const WideBody* __restrict__ bodies,
                                                      const TanBody* __restrict__ tbodies,
                                                      const WideInst* __restrict__ inst,
                                                      const WideTile* __restrict__ tiles, unsigned* status) {
  __shared__ WideBody sB;
  __shared__ TanBody sT;
  __shared__ GridP sG;
  __shared__ double sDt;
  const WideTile tl = tiles[blockIdx.x];
  stage(&sB, bodies + tl.body);
  stage(&sT, tbodies + tl.body);
  __syncthreads();
  stage(&sG, &inst[sB.inst].g);
  if (threadIdx.x == 0) sDt = inst[sB.inst].dt;
  __syncthreads();
  const int64_t t = tl.start + threadIdx.x;
  if (t >= sB.pp.count) return;
  tan_g2p_particle<D>(sB, sT, sG, t);
  unsigned* st = status + sB.inst;
  if (sB.mp.type == MPM_MAT_ELASTIC) g2p_particle<D, double, MPM_MAT_ELASTIC>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st);
  else g2p_particle<D, double, MPM_MAT_NEOHOOKEAN>(sG, sB.nd, sB.pp, t, sB.mp, sDt, st);
}

template <int D>
__device__ __forceinline__ void tan_g2p_particle(const WideBody& sB, const TanBody& sT, const GridP& sG, int64_t t) {
  using L = Layout<D>;
  using T = TanLayout<D>;
  const int64_t p = sB.pp.begin + t;
  const PartP& pp = sB.pp;
  const PartP& tp = sT.tp;
  double x[D], xd[D], vd[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    x[a] = *field<double>(pp, L::X + a, p);
    xd[a] = tf<D>(tp, T::XD + a, p);
    vd[a] = tf<D>(tp, T::VD + a, p);
  }
  Hat<D, double> h;
  if (!hat<D, double>(sG, x, h)) return;  // the primal G2P reports it and freezes the particle
  Corners<D, double> cr;
  corners<D, double>(sG, h, cr);
  const NodeP& nd = sB.nd;
  const NodeP& tn = sT.tnd;
  const int64_t Nn = nd.nodeCount;
  double Ldt[D][D], Ld[D][D], xn[D], vn[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    xn[a] = xd[a];
    vn[a] = vd[a];
#pragma unroll
    for (int j = 0; j < D; ++j) Ldt[a][j] = Ld[a][j] = 0.0;
  }
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    double Hk[3], gd[D];
    hat_hessian<D>(h, k, Hk);
    grad_tangent<D>(Hk, xd, gd);
    const double N = cr.N[k];
    double Nd = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) Nd += cr.dN[k][a] * xd[a];
    const int64_t n = cr.node[k];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double vdt = nd.vdt[a * Nn + n], dv = nd.dv[a * Nn + n];
      const double vdtd = tn.vdt[a * Nn + n], dvd = tn.dv[a * Nn + n];
      xn[a] += Nd * vdt + N * vdtd;
      vn[a] += Nd * dv + N * dvd;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        Ldt[a][j] += vdt * cr.dN[k][j];
        Ld[a][j] += vdtd * cr.dN[k][j] + vdt * gd[j];
      }
    }
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    tf<D>(tp, T::XD + a, p) = xn[a];
    tf<D>(tp, T::VD + a, p) = vn[a];
  }
  // F_new = F A, F_new' = F' A + F (L dt)',  A = I + L dt
  double F[D * D], Fdt[D * D], Fn[D * D], Fnd[D * D];
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    F[c] = *field<double>(pp, L::F + c, p);
    Fdt[c] = tf<D>(tp, T::FD + c, p);
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double s = 0.0, sd = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const double A = (k == j ? 1.0 : 0.0) + Ldt[k][j];
        s += F[i + D * k] * A;
        sd += Fdt[i + D * k] * A + F[i + D * k] * Ld[k][j];
      }
      Fn[i + D * j] = s;
      Fnd[i + D * j] = sd;
    }
#pragma unroll
  for (int c = 0; c < D * D; ++c) tf<D>(tp, T::FD + c, p) = Fnd[c];
  double C[D * D];
  cofactor<D>(Fn, C);
  double J = 0.0, Jd = 0.0;
#pragma unroll
  for (int q = 0; q < D; ++q) J += Fn[q] * C[q];  // expansion along the first column
#pragma unroll
  for (int c = 0; c < D * D; ++c) Jd += C[c] * Fnd[c];
  tf<D>(tp, T::VOLD, p) = Jd * *field<double>(pp, L::VOL0, p);
  // eps_new = eps + sym(L dt), eps_new' = eps' + sym((L dt)')
  double e[L::S], ed[L::S];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = i; j < D; ++j) {
      const int c = sym<D>(i, j);
      e[c] = *field<double>(pp, L::EPS + c, p) + (i == j ? Ldt[i][i] : 0.5 * (Ldt[i][j] + Ldt[j][i]));
      ed[c] = tf<D>(tp, T::ED + c, p) + (i == j ? Ld[i][i] : 0.5 * (Ld[i][j] + Ld[j][i]));
      tf<D>(tp, T::ED + c, p) = ed[c];
    }
  double lam = sB.mp.lambda, mu = sB.mp.mu;
  if (sB.mp.per_particle) {
    lam = *field<double>(pp, L::LAM, p);
    mu = *field<double>(pp, L::MU, p);
  }
  const double dlam = sT.dlam, dmu = sT.dmu;
  double sd[L::S];
  if (sB.mp.type == MPM_MAT_ELASTIC) {
    double tr = 0.0, trd = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      tr += e[a];
      trd += ed[a];
    }
#pragma unroll
    for (int c = 0; c < L::S; ++c)
      sd[c] = 2.0 * (dmu * e[c] + mu * ed[c]) + (c < D ? dlam * tr + lam * trd : 0.0);
  } else {
    // sig = (mu (B - I) + lam ln J I) / J, B = F F^T
    const double lnJ = log(J), iJ = 1.0 / J;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = i; j < D; ++j) {
        double B = 0.0, Bd = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          B += Fn[i + D * k] * Fn[j + D * k];
          Bd += Fnd[i + D * k] * Fn[j + D * k] + Fn[i + D * k] * Fnd[j + D * k];
        }
        const double I = (i == j) ? 1.0 : 0.0;
        const double sig = (mu * (B - I) + lam * lnJ * I) * iJ;
        sd[sym<D>(i, j)] = (dmu * (B - I) + mu * Bd + (dlam * lnJ + lam * Jd * iJ) * I) * iJ - sig * Jd * iJ;
      }
  }
#pragma unroll
  for (int c = 0; c < L::S; ++c) tf<D>(tp, T::SD + c, p) = sd[c];
}

}  // namespace jmpm
