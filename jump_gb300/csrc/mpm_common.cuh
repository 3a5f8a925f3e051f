// mpm_common.cuh -- device data layout and shared device helpers of the
// GB300 explicit-MPM step (USL, linear hat basis).
//
// Particle state is one SoA allocation of NF fields x pitch elements
// (field-major), in the particle precision R (double or float).  Bodies
// occupy contiguous particle ranges.  Node state is FP64 SoA over a dense
// grid (nodeCount = nx*ny*nz, node index i + nx*j + nx*ny*k, 0-based).
#pragma once

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace jmpm {

// status bits raised by kernels (atomicOr), mapped to MPM_ERR_* by the host
enum : unsigned { ST_OUT_OF_GRID = 1u, ST_NEGATIVE_J = 2u, ST_NONFINITE = 4u,
                  // set only while uploading: a strain/stress or 3D plastic strain input
                  // whose mirrored entries differ
                  ST_ASYM_STRESS = 8u, ST_ASYM_PSTRAIN = 16u,
                  // the 2D MUSL mass solve reached its iteration cap
                  ST_SOLVER = 32u };

// Field indices of the particle SoA.  Symmetric tensors are stored as
// 2D: (xx, yy, xy); 3D: (xx, yy, zz, xy, yz, xz).
template <int D>
struct Layout {
  static constexpr int S = (D == 2) ? 3 : 6;   // symmetric tensor components
  static constexpr int PS = (D == 2) ? 3 : 6;  // plastic strain components
  static constexpr int X = 0;
  static constexpr int V = D;
  static constexpr int M = 2 * D;
  static constexpr int VOL = 2 * D + 1;
  static constexpr int VOL0 = 2 * D + 2;
  static constexpr int F = 2 * D + 3;          // D*D, column-major
  static constexpr int EPS = F + D * D;
  static constexpr int SIG = EPS + S;
  static constexpr int VM = SIG + S;
  static constexpr int ALPHA = VM + 1;
  static constexpr int EP = ALPHA + 1;
  static constexpr int LAM = EP + PS;          // per-particle Lame constants (optional)
  static constexpr int MU = LAM + 1;
  static constexpr int ALPHAD = MU + 1;        // Johnson-Cook/Voce plastic strain rate
  static constexpr int NF = ALPHAD + 1;
  // Johnson-Cook with damage (3D) keeps its state in the plastic strain slots,
  // which only J2 uses: damage_init, damage, temperature
  static constexpr int DINIT = EP;
  static constexpr int DAM = EP + 1;
  static constexpr int TEMP = EP + 2;
};

// symmetric index (i, j) -> storage slot
template <int D>
__host__ __device__ constexpr int sym(int i, int j) {
  if (i == j) return i;
  if (D == 2) return 2;
  int a = i < j ? i : j, b = i < j ? j : i;
  return (a == 0 && b == 1) ? 3 : ((a == 1 && b == 2) ? 4 : 5);
}

struct MatParams {
  int type;        // MPM_MAT_*
  int per_particle;  // 1: use the LAM/MU particle fields
  double lambda, mu, kappa, fy, k1;
  // Johnson-Cook / Voce: hardening constants, rate filter time 1000 cellsize /
  // signal velocity, and the step dt it is applied with
  double A, B, C, n, epsdot0, tav, dtime;
  // J2: 1 / (2 mu + k1) of the material (0 with per-particle Lame constants)
  double rtmuk1;
  // Johnson-Cook with damage: thermal softening exponent, temperature rise per
  // unit plastic work chi/(density Cp), damage constants, Tm - Tr
  double m, delta, d1, d2, d3, d4, d5, depsdot0, Tr, Tm, Tmr;
  // FP32 particles: lambda, mu, kappa, fy, k1 and rtmuk1 rounded to float once
  // on the host (a per-particle conversion is FP64-pipe work)
  float f_lambda, f_mu, f_kappa, f_fy, f_k1, f_rtmuk1;
  // double-word G2P (MPM_PREC_DW): lambda, mu, kappa, fy, k1, rtmuk1 and the
  // deviator's 0.333333333 as {hi, lo} float pairs split once on the host
  float w_lambda[2], w_mu[2], w_kappa[2], w_fy[2], w_k1[2], w_rtmuk1[2], w_third[2];
};

// a material constant in the particle precision: the FP64 value, or its float copy
template <class R>
__device__ __forceinline__ R mat_const(double d, float f) {
  if constexpr (sizeof(R) == 4) return f;
  else return d;
}

// Grid description shared by all kernels.
struct GridP {
  double xmin[3];
  double dxI[3];
  double dx[3];        // node spacing (xmax - xmin)/(n - 1), Grid.jl:105-107
  int64_t nn[3];       // nodes per axis
  int64_t nx, nxy, nodeCount;
  const double* coord[3];  // node coordinate per axis (xmin + i*dx, Grid.jl:149-152)
  // FP32 particles: the same constants rounded to float once (the hat of an FP32
  // particle needs them in float; converting per particle costs FP64-pipe work);
  // coordf null: convert on the fly
  float xminf[3], dxIf[3];
  const float* coordf[3];
  float w_dxI[3][2];   // dxI as {hi, lo} float pairs (double-word G2P)
};

// Node arrays (FP64).  Accumulators m, p0 (D), f (D); grid-update outputs
// vdt = (p/m)*dt and dv = (p - p0)/m (D each, zero where m <= tolerance).
struct NodeP {
  double* m;
  double* p0;   // D * nodeCount, component-major
  double* f;
  double* vdt;
  double* dv;
  float* vdt_f;  // FP32 copies for the FP32 particle path
  float* dv_f;
  // or, for the linear-basis USL G2P of a single context, one interleaved FP32
  // record per node (2D: vdt x y, dv x y = one float4; 3D: vdt x y z 0, dv x y z 0
  // = two float4), so that a corner's six values come in two 16-byte loads
  float4* nf4;
  // or, for the double-word G2P (MPM_PREC_DW), three float4 per node:
  // {vdt x hi, lo, vdt y hi, lo}, {vdt z hi, lo, dv x hi, lo}, {dv y hi, lo, dv z hi, lo};
  // null otherwise (every NodeP, and every struct holding one, is
  // value-initialised on the host; the grid update writes it when non-null)
  float4* dw4;
  const uint8_t* fixed;  // bit a set: dof a is fixed (grid.fixedNodes)
  int64_t nodeCount;
  int64_t nn[3];         // nodes per axis (1 for the unused axis in 2D)
  // active node blocks (64 nodes each, see mpm_sparse.cuh)
  uint32_t* bflag;       // per block, set by P2G
  uint32_t* blist;       // listed blocks of the current step
  uint32_t* bcount;      // length of blist (device)
  int64_t nb[3];         // blocks per axis
  int64_t nblk;
  double* nrm;           // contact mode: per-body normals sum m_p grad N (D), else nullptr
  // MUSL: second momentum sum (D, lumped), velocity x dt for the velocity
  // gradient (D), consistent-mass stencil (9 per node, 2D)
  double* p2;
  double* vg;
  double* mc;
  int nmc;               // entries of the mass stencil per node ((2K - 1)^2 for K support nodes per axis)
  // rigid bodies (MPM_MAT_RIGID): per node, bit k set when a particle of rigid
  // body k (in body order) has the node in its linear cell this step; zeroed
  // with the accumulators of the listed blocks.  rtab: per rigid body
  // {fixed, vx, vy, vz}.  Both null without rigid bodies.
  uint32_t* rmask;
  const double* rtab;
};

// 2D MUSL mass solve: CG vectors of the four right-hand sides (p0_x, p0_y,
// dt f_x, dt f_y), nodeCount doubles each; x holds v0_x, v0_y, dv_x, dv_y.
struct CgP {
  double* x[4];
  double* r[4];
  double* p[4];
  double* q[4];
};

// Contact mode: one node field per body (SolveExplicitFEMP2DContact.jl:33-52).
constexpr int kMaxContactBodies = 4;
struct ContactP {
  int nb;
  double friction;
  NodeP body[kMaxContactBodies];
};

struct PartP {
  void* base;      // R*, NF * pitch
  int64_t pitch;   // elements per field
  int64_t begin;   // first particle of this launch
  int64_t count;   // particles of this launch
  // Optional hat cache (hat_put / hat_get): the linear P2G stores each
  // particle's hat and the G2P of the same step reads it back, since both see
  // the positions before the G2P moves them.  Null: the G2P recomputes it
  // (every PartP, and every struct holding one, is value-initialised on the
  // host, so both are null unless set).
  int32_t* hat_c;  // D * pitch: cell | bit 27 gl == 0 | bit 28 gl < 0 | bit 29 gh == 0 | bit 30 gh < 0; -1 outside
  void* hat_nl;    // D * pitch values of the particle type: the hat value at the lower node
};

// Record cursor of the EnergiesFix sums of captured steps (energies_kernel):
// the records' base and the next record's index, in device memory.
struct EnRec {
  double* base;
  long long idx;
};

// Buffers of the counting sort by (body, cell).
struct SortP {
  uint32_t* key;       // per particle
  uint32_t* rank;      // per particle: arrival rank inside its key
  uint32_t* count;     // per key, zeroed before the key pass
  uint32_t* offset;    // per key, exclusive scan of count
  uint32_t* blocksum;  // per 1024-key scan block
  int64_t nkeys;
};

__device__ __forceinline__ bool is_zero_bits(double x) {
  return (__double_as_longlong(x) << 1) == 0;
}
__device__ __forceinline__ bool is_zero_bits(float x) {
  return (__float_as_uint(x) << 1) == 0;
}
__device__ __forceinline__ bool is_neg_bits(double x) { return __double_as_longlong(x) < 0; }
__device__ __forceinline__ bool is_neg_bits(float x) { return int(__float_as_uint(x)) < 0; }
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}
__device__ __forceinline__ bool finite_bits(float x) {
  return ((__float_as_uint(x) >> 23) & 0xff) != 0xff;
}

// Exact float -> double on the integer pipe (the hardware conversion issues on
// the FP64 pipe, which runs at 1/64 of the FP32 rate on this GPU).  Normal
// numbers and zeros are repacked bit for bit; subnormals, Inf and NaN take the
// hardware conversion.
__device__ __forceinline__ double to_f64(float f) {
  unsigned u = __float_as_uint(f);
  unsigned e = u & 0x7f800000u;
  if (e == 0u || e == 0x7f800000u) {
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double(int(u & 0x80000000u), 0);
    return double(f);
  }
  unsigned hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + 0x38000000u);
  return __hiloint2double(int(hi), int(u << 29));
}
__device__ __forceinline__ double to_f64(double d) { return d; }

// x > 0 for a double, decided on the integer pipe
__device__ __forceinline__ bool positive_bits(double x) {
  long long b = __double_as_longlong(x);
  return b > 0 && ((b >> 52) & 0x7ff) != 0x7ff;
}

// -sign(delta) * dxI, selected with integer ops (Basis.jl:247-248, sign(0) = 0)
template <class R>
__device__ __forceinline__ R neg_sign_scale(R delta, R dxI) {
  if (is_zero_bits(delta)) return R(0);
  return is_neg_bits(delta) ? dxI : -dxI;
}

// exact-rounding helpers (no contraction) for the shape functions, so the
// hat values are bit-identical to the reference's `1.0 - abs(x)*dxI`
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ int floor_to_int(double t) { return __double2int_rd(t); }
__device__ __forceinline__ int floor_to_int(float t) { return __float2int_rd(t); }

// FP64 -> float by truncation on the integer pipe, for magnitudes in
// [2^-126, 2^128) (relative error below 2^-23); NaN for any other value,
// zero included
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned bh = unsigned(__double2hiint(x)), bl = unsigned(__double2loint(x));
  const unsigned ex = (bh >> 20) & 0x7ffu;
  if (ex - 897u > 253u) return __uint_as_float(0x7fc00000u);
  return __uint_as_float((__funnelshift_l(bl, bh, 3) - (0x180u << 23)) | (bh & 0x80000000u));
}

// hat()'s 1-based base node in FP64, floor((x - xmin) dxI + 1) with the
// reference's roundings; not inlined, so that the compiler cannot evaluate it
// beside the FP32 estimate on the path where the estimate decides
static __device__ __noinline__ int base_node_f64(double x, double xmin, double dxI) {
  return __double2int_rd(__dadd_rn(__dmul_rn(__dsub_rn(x, xmin), dxI), 1.0));
}

// The 1-based base node i1 = floor((x - xmin) dxI + 1) of hat(), decided by an
// FP32 estimate (from the host-rounded float grid constants) when the
// estimate lies farther from an integer than its error bound
// |t32 - t| <= 2^-24 (4 (|x| + |xmin|) dxI + |t|): the FP64 expression, whose
// own error is some 10^8 times smaller, then has the same floor.  False when
// the caller must form it in FP64 (near a node line, outside the float range,
// or without float constants: dxIf == 0).
__device__ __forceinline__ bool base_node_estimate(double x, float xminf, float dxIf, int& i1) {
  if (!(dxIf > 0.f)) return false;
  const float xf = f32_trunc(x);
  const float t32 = __fmaf_rn(__fsub_rn(xf, xminf), dxIf, 1.0f);
  const float bound = 0x1p-21f * __fmaf_rn(__fadd_rn(fabsf(xf), fabsf(xminf)), dxIf, fabsf(t32) + 1.0f);
  const float fl = floorf(t32);
  if (!(t32 - fl > bound && fl + 1.0f - t32 > bound && fabsf(fl) < 1e9f)) return false;
  i1 = int(fl);
  return true;
}

// Per-axis linear hat values and gradient factors of one particle.
template <int D, class R>
struct Hat {
  int c[D];      // 0-based cell per axis
  R Nl[D], Nh[D];  // hat value at the lower / upper node
  R gl[D], gh[D];  // -sign(x - x_node) * dxI
};

// getAdjacentGridPoints + 1D factors of getShapeAndGradient
// (Basis.jl:63-78, 104-137, 219-251, 292-332).  False if outside the grid.
template <int D, class R>
__device__ __forceinline__ bool hat(const GridP& g, const R* x, Hat<D, R>& h) {
  const bool fc = sizeof(R) == 4 && g.coordf[0] != nullptr;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    R xmin = fc ? R(g.xminf[a]) : R(g.xmin[a]), dxI = fc ? R(g.dxIf[a]) : R(g.dxI[a]);
    int i1;  // 1-based base node
    // FP64 particles: the FP32 estimate where it decides the floor (saves
    // FP64-pipe work), else the FP64 expression
    if constexpr (sizeof(R) == 8) {
      if (!base_node_estimate(x[a], g.xminf[a], g.dxIf[a], i1)) i1 = base_node_f64(x[a], g.xmin[a], g.dxI[a]);
    } else {
      i1 = floor_to_int(add_rn(mul_rn(sub_rn(x[a], xmin), dxI), R(1)));
    }
    if (i1 < 1 || i1 > int(g.nn[a] - 1)) return false;
    int c = i1 - 1;
    h.c[a] = c;
    R xl = fc ? R(g.coordf[a][c]) : R(g.coord[a][c]), xh = fc ? R(g.coordf[a][c + 1]) : R(g.coord[a][c + 1]);
    R dl = sub_rn(x[a], xl), dh = sub_rn(x[a], xh);
    h.Nl[a] = sub_rn(R(1), mul_rn(fabs(dl), dxI));
    h.Nh[a] = sub_rn(R(1), h.Nl[a]);  // 1 - |x - xh| dxI for xl <= x <= xh
    h.gl[a] = neg_sign_scale(dl, dxI);
    h.gh[a] = neg_sign_scale(dh, dxI);
  }
  return true;
}

// True when every axis has gl = -dxI and gh = +dxI exactly: the particle lies
// strictly inside its cell (neither on a node line nor rounded past one), so
// sums over the two nodes of an axis weighted by the gradient are dxI times a
// difference.  Integer tests of the sign and zero bits.
template <int D, class R>
__device__ __forceinline__ bool hat_interior(const Hat<D, R>& h) {
  bool in = true;
#pragma unroll
  for (int a = 0; a < D; ++a)
    in = in && is_neg_bits(h.gl[a]) && !is_zero_bits(h.gl[a]) && !is_neg_bits(h.gh[a]) && !is_zero_bits(h.gh[a]);
  return in;
}

// Hat cache of particle p (PartP::hat_c / hat_nl).  The gradient factors are
// 0 or -+dxI (neg_sign_scale), so two bits each restore them exactly, and the
// upper value is recomputed with hat()'s rounding: hat_get gives bit for bit
// the Hat that hat() computes from the same position, without its FP64 work.
template <int D, class R>
__device__ __forceinline__ void hat_put(const PartP& pp, int64_t p, bool ok, const Hat<D, R>& h) {
  if constexpr (sizeof(R) != 8) return;  // FP64 particles only: an FP32 hat is cheaper to recompute
  if (!pp.hat_c) return;
  R* nl = static_cast<R*>(pp.hat_nl);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    int32_t code = -1;
    if (ok) {
      code = h.c[a] | (int32_t(is_zero_bits(h.gl[a])) << 27) | (int32_t(is_neg_bits(h.gl[a])) << 28) |
             (int32_t(is_zero_bits(h.gh[a])) << 29) | (int32_t(is_neg_bits(h.gh[a])) << 30);
      nl[a * pp.pitch + p] = h.Nl[a];
    }
    pp.hat_c[a * pp.pitch + p] = code;
  }
}

template <int D, class R>
__device__ __forceinline__ bool hat_get(const GridP& g, const PartP& pp, int64_t p, Hat<D, R>& h) {
  const R* nl = static_cast<const R*>(pp.hat_nl);
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int32_t code = pp.hat_c[a * pp.pitch + p];
    if (code < 0) return false;
    const R dxI = R(g.dxI[a]);
    h.c[a] = code & ((1 << 27) - 1);
    h.Nl[a] = nl[a * pp.pitch + p];
    h.Nh[a] = sub_rn(R(1), h.Nl[a]);
    h.gl[a] = ((code >> 27) & 1) ? R(0) : (((code >> 28) & 1) ? -dxI : dxI);
    h.gh[a] = ((code >> 29) & 1) ? R(0) : (((code >> 30) & 1) ? -dxI : dxI);
  }
  return true;
}

// Corner k of the stencil in the reference's nearPoints order:
// bit 0 -> +x, bit 1 -> +y, bit 2 -> +z.  N and grad N with the reference's
// products: N = (Nx*Ny)*Nz, dN/dx = (Ny*Nz)*(-sign*dxI), ...
template <int D, class R>
struct Corners {
  R N[1 << D];
  R dN[1 << D][D];
  int64_t node[1 << D];
};

template <int D, class R>
__device__ __forceinline__ void corners(const GridP& g, const Hat<D, R>& h, Corners<D, R>& cr) {
  int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]);
  if (D == 3) base += g.nxy * int64_t(h.c[D == 3 ? 2 : 0]);
  if (D == 2) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int bx = k & 1, by = (k >> 1) & 1;
      R Nx = bx ? h.Nh[0] : h.Nl[0];
      R Ny = by ? h.Nh[1] : h.Nl[1];
      R gx = bx ? h.gh[0] : h.gl[0];
      R gy = by ? h.gh[1] : h.gl[1];
      cr.N[k] = mul_rn(Nx, Ny);
      cr.dN[k][0] = mul_rn(Ny, gx);
      cr.dN[k][1] = mul_rn(Nx, gy);
      cr.node[k] = base + bx + g.nx * by;
    }
  } else {
    R NxNy[4], NyNz[4], NxNz[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int b0 = q & 1, b1 = (q >> 1) & 1;
      NxNy[q] = mul_rn(b0 ? h.Nh[0] : h.Nl[0], b1 ? h.Nh[1] : h.Nl[1]);
      NyNz[q] = mul_rn(b0 ? h.Nh[1] : h.Nl[1], b1 ? h.Nh[D - 1] : h.Nl[D - 1]);
      NxNz[q] = mul_rn(b0 ? h.Nh[0] : h.Nl[0], b1 ? h.Nh[D - 1] : h.Nl[D - 1]);
    }
#pragma unroll
    for (int k = 0; k < (1 << D); ++k) {
      int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
      R Nz = bz ? h.Nh[D - 1] : h.Nl[D - 1];
      R gx = bx ? h.gh[0] : h.gl[0];
      R gy = by ? h.gh[1] : h.gl[1];
      R gz = bz ? h.gh[D - 1] : h.gl[D - 1];
      R nxny = NxNy[bx + 2 * by];
      cr.N[k] = mul_rn(nxny, Nz);
      cr.dN[k][0] = mul_rn(NyNz[by + 2 * bz], gx);
      cr.dN[k][1] = mul_rn(NxNz[bx + 2 * bz], gy);
      cr.dN[k][D - 1] = mul_rn(nxny, gz);
      cr.node[k] = base + bx + g.nx * by + g.nxy * bz;
    }
  }
}

// node indices of the corners only (for kernels that form N and grad N from
// the per-axis factors themselves)
template <int D, class R>
__device__ __forceinline__ void corner_nodes(const GridP& g, const Hat<D, R>& h, Corners<D, R>& cr) {
  int64_t base = int64_t(h.c[0]) + g.nx * int64_t(h.c[1]);
  if (D == 3) base += g.nxy * int64_t(h.c[D == 3 ? 2 : 0]);
#pragma unroll
  for (int k = 0; k < (1 << D); ++k) {
    const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    cr.node[k] = base + bx + g.nx * by + (D == 3 ? g.nxy * bz : 0);
  }
}

// The box [lo, hi] (per axis) of the base cells of the CTA's lanes with ok,
// for the shared-memory node tiles of the P2G and of the G2P adjoint: a
// reduction per warp, then over the CTA's warps.  Every thread of the CTA
// calls it once per launch (it synchronises the CTA); lo[0] > hi[0] when no
// lane has ok; axis 2 stays [0, 0] in 2D.  blockDim.x is a multiple of 32 and
// at most 256.
template <int D>
__device__ __forceinline__ void cta_cell_box(bool ok, const int* c, int (&lo)[3], int (&hi)[3]) {
  __shared__ int wlo[8][3], whi[8][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int wl = __reduce_min_sync(0xffffffffu, ok ? c[a] : INT_MAX);
    const int wh = __reduce_max_sync(0xffffffffu, ok ? c[a] : INT_MIN);
    if (lane == 0) {
      wlo[warp][a] = wl;
      whi[warp][a] = wh;
    }
  }
  __syncthreads();
  lo[2] = hi[2] = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    lo[a] = INT_MAX;
    hi[a] = INT_MIN;
    for (int w = 0; w < nwarps; ++w) {
      lo[a] = min(lo[a], wlo[w][a]);
      hi[a] = max(hi[a], whi[w][a]);
    }
  }
}

}  // namespace jmpm
