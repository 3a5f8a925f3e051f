// mpm_internal.h -- host-side launchers of the step kernels (explicitly
// instantiated per dimension in mpm_k2d.cu / mpm_k3d.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include <cmath>

#include "../../include/jump_mpm.h"
#include "mpm_common.cuh"
#include "mpm_adjoint.cuh"

namespace jmpm {

// Kernel parameters of a material (Material.jl:37-172, 279-383): Lame constants
// as the constructors compute them; for Johnson-Cook/Voce the rate filter time
// 1000 cellsize / sqrt((lambda + 2 mu)/density) and the step dt.
// d as a double-word pair: hi = float(d), lo = float(d - hi)
inline void split_dw(double d, float (&w)[2]) {
  w[0] = float(d);
  w[1] = float(d - double(w[0]));
}

inline MatParams make_mat_params(const mpm_material_desc& m, bool per_particle, double dt) {
  MatParams mp{};
  mp.type = m.type;
  mp.per_particle = per_particle;
  mp.lambda = m.E * m.nu / (1 + m.nu) / (1 - 2 * m.nu);  // Material.jl:54-55
  mp.mu = m.E / 2 / (1 + m.nu);
  mp.kappa = mp.lambda + mp.mu;  // Material.jl:161, 315
  mp.fy = m.fy;
  mp.k1 = m.k1;
  mp.rtmuk1 = per_particle ? 0.0 : 1.0 / (2 * mp.mu + m.k1);
  mp.A = m.A;
  mp.B = m.B;
  mp.C = m.C;
  mp.n = m.n;
  mp.epsdot0 = m.epsdot0;
  if (m.type == MPM_MAT_JOHNSON_COOK || m.type == MPM_MAT_VOCE || m.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    const double velo = std::sqrt((mp.lambda + 2 * mp.mu) / m.density);  // Material.jl:317
    mp.tav = 1000 * m.cellsize / velo;                                   // Material.jl:428
  }
  if (m.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    mp.m = m.m;
    mp.delta = m.chi / (m.density * m.Cp);  // Material.jl:323
    mp.d1 = m.d1;
    mp.d2 = m.d2;
    mp.d3 = m.d3;
    mp.d4 = m.d4;
    mp.d5 = m.d5;
    mp.depsdot0 = m.depsdot0;
    mp.Tr = m.Tr;
    mp.Tm = m.Tm;
    mp.Tmr = m.Tm - m.Tr;  // Material.jl:507
  }
  mp.dtime = dt;
  mp.f_lambda = float(mp.lambda);
  mp.f_mu = float(mp.mu);
  mp.f_kappa = float(mp.kappa);
  mp.f_fy = float(mp.fy);
  mp.f_k1 = float(mp.k1);
  mp.f_rtmuk1 = float(mp.rtmuk1);
  split_dw(mp.lambda, mp.w_lambda);
  split_dw(mp.mu, mp.w_mu);
  split_dw(mp.kappa, mp.w_kappa);
  split_dw(mp.fy, mp.w_fy);
  split_dw(mp.k1, mp.w_k1);
  split_dw(mp.rtmuk1, mp.w_rtmuk1);
  split_dw(0.333333333, mp.w_third);  // the deviator's constant (Material.jl:246)
  return mp;
}

// CTA size for n independent threads: 256, halved (down to 64) while that
// leaves fewer than two CTAs per SM, so small problems spread over the GPU
inline int spread_threads(int64_t n) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) ==
                                                  cudaSuccess && v > 0)
      sms = v;
    else
      sms = 152;
  }
  int th = 256;
  while (th > 64 && (n + th - 1) / th < 2 * int64_t(sms)) th /= 2;
  return th;
}

// MPM_P2G_FUSED (mpm_batch.cu): nsteps USL steps of one FP64 problem of a
// context in one cooperative launch, stages separated by bounded grid
// barriers: linear basis, one velocity field, no rigid bodies, every body
// linear elastic, neo-Hookean or J2 of one type, at most MPM_BATCH_MAX_BODIES
// bodies.  dev: device scratch of fused_bytes() bytes, whose third word is set
// when a barrier wait gave up (read it after the stream synchronises).
size_t fused_bytes(int dim, int64_t nodes);
// rec (may be null): the EnergiesFix record cursor, one record after local
// steps first, first + every, ... of the call
int fused_steps(int dim, cudaStream_t s, void* dev, const GridP& g, const NodeP& nd, void* P, int64_t pitch,
                int nb, const int64_t* bbeg, const int64_t* bcnt, const MatParams* mp, double dt, double tol,
                const double* grav, int64_t nsteps, unsigned* status, EnRec* rec = nullptr, int64_t first = 0,
                int64_t every = 1, int32_t* hat_c = nullptr, void* hat_nl = nullptr);

// deformable material model types a context or batch accepts in dimension dim
// (rigid bodies, MPM_MAT_RIGID, are checked separately: contexts only)
inline bool material_ok(int type, int dim) {
  if (type == MPM_MAT_ELASTIC || type == MPM_MAT_NEOHOOKEAN || type == MPM_MAT_J2) return true;
  return dim == 3 && (type == MPM_MAT_JOHNSON_COOK || type == MPM_MAT_VOCE || type == MPM_MAT_JOHNSON_COOK_DAMAGE);
}

// material parameters a context or batch accepts: the damage model's
// temperature rise chi/(density Cp) needs density Cp > 0
inline bool material_params_ok(const mpm_material_desc& m) {
  if (m.type != MPM_MAT_JOHNSON_COOK_DAMAGE) return true;
  return m.density > 0 && m.Cp > 0;
}

struct CompMapH {
  int n;
  int src[9];
  int nchk;         // upload: mirrored pairs (ca[k], cb[k]) that must be equal
  int ca[3], cb[3];
  unsigned bit;     // set in *flag when a pair differs
  unsigned* flag;
};

template <int D>
struct Launchers {
  // strategy: MPM_P2G_ATOMIC / MPM_P2G_WARP, or -1 for the precision's default
  // (FP64: atomic, FP32: warp); threads per CTA (<= 256), 0 for 256
  static void p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                  const double* grav, unsigned* status, int strategy = -1, int threads = 0);
  // rigid body `bit`: mark its particles' linear-cell nodes and move them by dt v (v: 3 doubles)
  static void rigid(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32, int bit,
                    const double* v, double dt, unsigned* status);
  // compaction of the flagged node blocks + grid update over them
  static void grid(cudaStream_t s, const NodeP& nd, double dt, double tol, bool f32copy);
  // zero the accumulators of the blocks listed by the previous grid stage
  static void clear(cudaStream_t s, const NodeP& nd);
  // adjoint of one step (mpm_adjoint.cuh), FP64 particles; mp.type selects the
  // material (neo-Hookean, linear elastic, J2); c1, c2 = dlambda/dE, dmu/dE
  // tile: the node adjoints scattered through a shared-memory node tile (the
  // contexts whose P2G strategy is a tile one), else per particle at L2
  static void g2p_adj(cudaStream_t s, const GridP& g, const GridRec& gr, const PartP& pp, const AdjP& ad,
                      const NodeAdjP& na, const MatParams& mp, double c1, double c2, bool tile);
  // one reversed step of a single-body context in one cooperative launch
  // (reverse_step_kernel); reverse_step_fits: the device takes cooperative
  // launches and every CTA of count particles' launch can be resident at once
  static bool reverse_step_fits(int64_t count, int mat);
  static cudaError_t reverse_step(cudaStream_t s, const RevStepP& r);
  static void grid_adj(cudaStream_t s, const GridRec& gr, const NodeAdjP& na, const uint8_t* fixed, double dt,
                       double tol);
  static void p2g_adj(cudaStream_t s, const GridP& g, const PartP& pp, const AdjP& ad, const NodeAdjP& na,
                      const MatParams& mp, double c1, double c2, const double* grav);
  // contact mode: compaction + per-node grid update of every body field + correction
  static void contact_grid(cudaStream_t s, const NodeP& nd, const ContactP& cp, double dt, double tol,
                           bool f32copy);
  static void g2p(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                  const MatParams& mp, double dt, unsigned* status, int threads = 0);
  // raises the dynamic shared-memory limit of the double-word G2P (3D), once
  // per context before its first step (outside any stream capture)
  static cudaError_t dw_setup();
  // EnergiesFix sums into out[0 .. 2 + D), or with a record cursor rec into
  // rec->base[rec->idx] (the cursor advances): partial holds nblocks x 5
  // doubles and one more slot, the fold's ticket, zero before the first
  // launch (each launch leaves it zero)
  static void energies(cudaStream_t s, const PartP& pp, bool f32, double* partial, int nblocks,
                       double* out, EnRec* rec = nullptr);
  static void aos_to_soa(cudaStream_t s, const PartP& pp, bool f32, const double* src, int per, int f0,
                         const CompMapH& cm);
  static void soa_to_aos(cudaStream_t s, const PartP& pp, bool f32, double* dst, int per, int f0,
                         const CompMapH& cm);
  static void j2_vm(cudaStream_t s, const PartP& pp, bool f32, double* dst);
  // downloads in original particle order through the permutation orig[slot]
  static void soa_to_aos_perm(cudaStream_t s, const PartP& pp, bool f32, const int64_t* orig, double* dst,
                              int per, int f0, const CompMapH& cm);
  static void j2_vm_perm(cudaStream_t s, const PartP& pp, bool f32, const int64_t* orig, double* dst);
  // counting sort by (body, cell)
  static void sort_keys(cudaStream_t s, const GridP& g, const PartP& pp, bool f32, uint32_t body_base,
                        uint32_t ncells, const SortP& sp);
  static void scan(cudaStream_t s, const uint32_t* in, uint32_t* out, uint32_t* blocksum, int64_t n);
  static void sort_scatter(cudaStream_t s, bool f32, const void* src, void* dst, int64_t pitch, int nf,
                           const SortP& sp, const int64_t* orig_src, int64_t* orig_dst);
  // MUSL (mpm_musl.cuh), FP64 particles.  musl_p2g: P2G (2D: with body force and
  // the consistent mass stencil; 3D: no body force); musl_grid: compaction + grid
  // update (3D lumped) or mass solve + node outputs (2D); musl_g2p1: velocity
  // blend (3D: + P2G-2); musl_vg: 3D gradient velocities; musl_g2p2: kinematics.
  // basis: MPM_BASIS_* of the context (the 2D solve's stencil grows with it)
  static void musl_p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, const double* grav,
                       unsigned* status, int basis);
  static void musl_grid(cudaStream_t s, const NodeP& nd, const CgP& cg, double dt, double alpha, unsigned* status,
                        int basis);
  static void musl_g2p1(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, double alpha,
                        unsigned* status, int basis);
  static void musl_vg(cudaStream_t s, const NodeP& nd, double dt);
  static void musl_g2p2(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, const MatParams& mp,
                        unsigned* status, int basis);
  // USL over the quadratic / cubic B-spline bases (mpm_bspline.cuh)
  static void bs_p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32, const double* grav,
                     unsigned* status, int basis);
  static void bs_g2p(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32, const MatParams& mp,
                     unsigned* status, int basis);
};

// nodes per axis of a particle's support
inline int basis_nodes(int basis) {
  return basis == MPM_BASIS_QUAD_BSPLINE ? 3 : (basis == MPM_BASIS_CUBIC_BSPLINE ? 4 : 2);
}

constexpr int kEnergyBlocks = 304;  // 2 x 152 SMs

// Records msg as the calling thread's mpm_last_error() text; returns code.
int set_last_error(int code, const std::string& msg);

}  // namespace jmpm
