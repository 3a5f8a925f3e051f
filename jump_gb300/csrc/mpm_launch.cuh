// mpm_launch.cuh -- definitions of Launchers<D>; included once per dimension.
#pragma once

#include "mpm_internal.h"
#include "mpm_kernels.cuh"
#include "mpm_musl.cuh"
#include "mpm_bspline.cuh"
#include "mpm_step_dw.cuh"
#include "mpm_bspline_dw.cuh"

#include <type_traits>

namespace jmpm {

static inline unsigned blocks_for(int64_t n, int threads) {
  return unsigned((n + threads - 1) / threads);
}

static inline CompMap to_dev(const CompMapH& h) {
  CompMap c;
  c.n = h.n;
  for (int i = 0; i < 9; ++i) c.src[i] = h.src[i];
  c.nchk = h.nchk;
  for (int i = 0; i < 3; ++i) {
    c.ca[i] = h.ca[i];
    c.cb[i] = h.cb[i];
  }
  c.bit = h.bit;
  c.flag = h.flag;
  return c;
}

template <int D>
void Launchers<D>::p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                       const double* grav, unsigned* status, int strategy, int threads) {
  if (pp.count <= 0) return;
  bool has_g = grav[0] != 0.0 || grav[1] != 0.0 || (D == 3 && grav[2] != 0.0);
  if (!f32 && nd.dw4) {
    // double-word P2G (MPM_PREC_DW contexts, 3D): per-lane FP64 atomics
    if constexpr (D == 3) {
      const int th = threads > 0 ? threads : 256;
      if (has_g) p2g_dw_kernel<true><<<blocks_for(pp.count, th), th, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status);
      else p2g_dw_kernel<false><<<blocks_for(pp.count, th), th, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status);
    }
    return;
  }
  if (strategy < 0) strategy = f32 ? MPM_P2G_WARP : MPM_P2G_ATOMIC;
  const int th = threads > 0 ? threads : 256;
  unsigned nb = blocks_for(pp.count, th);
  const bool w = strategy == MPM_P2G_WARP || strategy == MPM_P2G_TILE_WARP;
  if (strategy == MPM_P2G_TILE || strategy == MPM_P2G_TILE_WARP) {
    // tile of at most cap nodes: 40 KB at most (512 nodes x 10 values), under
    // the default 48 KB of dynamic shared memory
    const int cap = th <= 64 ? 256 : 512;
    const size_t smem = size_t(cap) * size_t(nd.nrm ? 1 + 3 * D : 1 + 2 * D) * sizeof(double);
#define JMPM_P2GT(R, G, W) \
  p2g_tile_kernel<D, R, G, W><<<nb, th, smem, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status, cap)
    if (f32) {
      if (has_g) { if (w) JMPM_P2GT(float, true, true); else JMPM_P2GT(float, true, false); }
      else { if (w) JMPM_P2GT(float, false, true); else JMPM_P2GT(float, false, false); }
    } else {
      if (has_g) { if (w) JMPM_P2GT(double, true, true); else JMPM_P2GT(double, true, false); }
      else { if (w) JMPM_P2GT(double, false, true); else JMPM_P2GT(double, false, false); }
    }
#undef JMPM_P2GT
    return;
  }
#define JMPM_P2G(R, G, W) p2g_kernel<D, R, G, W><<<nb, th, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status)
  if (f32) {
    if (has_g) { if (w) JMPM_P2G(float, true, true); else JMPM_P2G(float, true, false); }
    else { if (w) JMPM_P2G(float, false, true); else JMPM_P2G(float, false, false); }
  } else {
    if (has_g) { if (w) JMPM_P2G(double, true, true); else JMPM_P2G(double, true, false); }
    else { if (w) JMPM_P2G(double, false, true); else JMPM_P2G(double, false, false); }
  }
#undef JMPM_P2G
}

// sparse grid stages: a fixed grid of CTAs strides over the listed blocks
static inline unsigned sparse_ctas(const NodeP& nd) {
  int64_t most = (nd.nblk * 64 + 255) / 256;
  return unsigned(most < 152 * 8 ? (most > 0 ? most : 1) : 152 * 8);
}

template <int D>
void Launchers<D>::grid(cudaStream_t s, const NodeP& nd, double dt, double tol, bool f32copy) {
  // list compaction and grid update in one launch (grid_scan_kernel)
  const int64_t quads = (nd.nblk + 3) / 4;
  const unsigned ctas = unsigned(quads < 152 * 8 ? (quads > 0 ? quads : 1) : 152 * 8);
  if (f32copy) grid_scan_kernel<D, true><<<ctas, 256, 0, s>>>(nd, dt, tol);
  else grid_scan_kernel<D, false><<<ctas, 256, 0, s>>>(nd, dt, tol);
}

template <int D>
void Launchers<D>::contact_grid(cudaStream_t s, const NodeP& nd, const ContactP& cp, double dt, double tol,
                                bool f32copy) {
  compact_blocks_kernel<<<blocks_for(nd.nblk, 256), 256, 0, s>>>(nd);
  if (f32copy) contact_grid_kernel<D, true><<<sparse_ctas(nd), 256, 0, s>>>(nd, cp, dt, tol);
  else contact_grid_kernel<D, false><<<sparse_ctas(nd), 256, 0, s>>>(nd, cp, dt, tol);
}

template <int D>
void Launchers<D>::g2p_adj(cudaStream_t s, const GridP& g, const GridRec& gr, const PartP& pp, const AdjP& ad,
                           const NodeAdjP& na, const MatParams& mp, double c1, double c2, bool tile) {
  if (pp.count <= 0) return;
  const int th = spread_threads(pp.count);
  const unsigned nb = blocks_for(pp.count, th);
  // node tile of the scatter: at most 512 nodes x 2D doubles (24 KB in 3D)
  const int cap = tile ? (th <= 64 ? 256 : 512) : 0;
  const size_t smem = size_t(cap) * 2 * D * sizeof(double);
#define JMPM_G2PA(MAT)                                                                       \
  do {                                                                                       \
    if (tile) g2p_adj_kernel<D, MAT, true><<<nb, th, smem, s>>>(g, gr, pp, ad, na, mp, c1, c2, cap); \
    else g2p_adj_kernel<D, MAT, false><<<nb, th, 0, s>>>(g, gr, pp, ad, na, mp, c1, c2, 0);         \
  } while (0)
  if (mp.type == MPM_MAT_ELASTIC) JMPM_G2PA(MPM_MAT_ELASTIC);
  else if (mp.type == MPM_MAT_J2) JMPM_G2PA(MPM_MAT_J2);
  else JMPM_G2PA(MPM_MAT_NEOHOOKEAN);
#undef JMPM_G2PA
}

template <int D>
static const void* reverse_step_fn(int mat) {
  if (mat == MPM_MAT_ELASTIC) return reinterpret_cast<const void*>(reverse_step_kernel<D, MPM_MAT_ELASTIC>);
  if (mat == MPM_MAT_J2) return reinterpret_cast<const void*>(reverse_step_kernel<D, MPM_MAT_J2>);
  return reinterpret_cast<const void*>(reverse_step_kernel<D, MPM_MAT_NEOHOOKEAN>);
}

template <int D>
bool Launchers<D>::reverse_step_fits(int64_t count, int mat) {
  int dev = 0, coop = 0, sms = 0, per = 0;
  if (count <= 0 || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || !coop)
    return false;
  const int th = spread_threads(count);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, reverse_step_fn<D>(mat), th, 0) != cudaSuccess) return false;
  return int64_t(per) * sms >= int64_t(blocks_for(count, th));
}

template <int D>
cudaError_t Launchers<D>::reverse_step(cudaStream_t s, const RevStepP& r) {
  const int th = spread_threads(r.pp.count);
  RevStepP a = r;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel(reverse_step_fn<D>(r.mp.type), dim3(blocks_for(r.pp.count, th)), dim3(th), args,
                                     0, s);
}

template <int D>
void Launchers<D>::grid_adj(cudaStream_t s, const GridRec& gr, const NodeAdjP& na, const uint8_t* fixed, double dt,
                            double tol) {
  const int th = spread_threads(na.nodeCount);
  grid_adj_kernel<D><<<blocks_for(na.nodeCount, th), th, 0, s>>>(gr, na, fixed, dt, tol);
}

template <int D>
void Launchers<D>::p2g_adj(cudaStream_t s, const GridP& g, const PartP& pp, const AdjP& ad, const NodeAdjP& na,
                           const MatParams& mp, double c1, double c2, const double* grav) {
  if (pp.count <= 0) return;
  const int th = spread_threads(pp.count);
  const unsigned nb = blocks_for(pp.count, th);
  const double gz = D == 3 ? grav[2] : 0.0;
  if (mp.type == MPM_MAT_ELASTIC)
    p2g_adj_kernel<D, MPM_MAT_ELASTIC><<<nb, th, 0, s>>>(g, pp, ad, na, mp, c1, c2, grav[0], grav[1], gz);
  else if (mp.type == MPM_MAT_J2)
    p2g_adj_kernel<D, MPM_MAT_J2><<<nb, th, 0, s>>>(g, pp, ad, na, mp, c1, c2, grav[0], grav[1], gz);
  else
    p2g_adj_kernel<D, MPM_MAT_NEOHOOKEAN><<<nb, th, 0, s>>>(g, pp, ad, na, mp, c1, c2, grav[0], grav[1], gz);
}

template <int D>
void Launchers<D>::rigid(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32, int bit,
                         const double* v, double dt, unsigned* status) {
  if (pp.count <= 0) return;
  if (f32) rigid_kernel<D, float><<<blocks_for(pp.count, 256), 256, 0, s>>>(g, nd, pp, bit, v[0], v[1], v[2], dt, status);
  else rigid_kernel<D, double><<<blocks_for(pp.count, 256), 256, 0, s>>>(g, nd, pp, bit, v[0], v[1], v[2], dt, status);
}

template <int D>
void Launchers<D>::clear(cudaStream_t s, const NodeP& nd) {
  clear_blocks_kernel<D><<<sparse_ctas(nd), 256, 0, s>>>(nd);
}

// f(std::integral_constant<int, MAT>) for a material type (Johnson-Cook and Voce in 3D only)
template <int D, class Fn>
static inline void with_material(int type, Fn&& f) {
  switch (type) {
    case MPM_MAT_ELASTIC: f(std::integral_constant<int, MPM_MAT_ELASTIC>{}); break;
    case MPM_MAT_NEOHOOKEAN: f(std::integral_constant<int, MPM_MAT_NEOHOOKEAN>{}); break;
    case MPM_MAT_JOHNSON_COOK:
      if constexpr (D == 3) f(std::integral_constant<int, MPM_MAT_JOHNSON_COOK>{});
      break;
    case MPM_MAT_VOCE:
      if constexpr (D == 3) f(std::integral_constant<int, MPM_MAT_VOCE>{});
      break;
    case MPM_MAT_JOHNSON_COOK_DAMAGE:
      if constexpr (D == 3) f(std::integral_constant<int, MPM_MAT_JOHNSON_COOK_DAMAGE>{});
      break;
    default: f(std::integral_constant<int, MPM_MAT_J2>{}); break;
  }
}

// f(std::integral_constant<int, K>) for a B-spline basis (K = 3 or 4 nodes per axis)
template <class Fn>
static inline void with_bspline(int basis, Fn&& f) {
  if (basis == MPM_BASIS_QUAD_BSPLINE) f(std::integral_constant<int, 3>{});
  else f(std::integral_constant<int, 4>{});
}

template <int D>
void Launchers<D>::musl_p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, const double* grav,
                            unsigned* status, int basis) {
  if (pp.count <= 0) return;
  const unsigned nb = blocks_for(pp.count, 256);
  const bool gr = grav[0] != 0.0 || grav[1] != 0.0;
  if constexpr (D == 2) {
    if (basis == MPM_BASIS_LINEAR) {
      if (gr) musl2d_p2g_kernel<true><<<nb, 256, 0, s>>>(g, nd, pp, grav[0], grav[1], status);
      else musl2d_p2g_kernel<false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, status);
    } else {
      with_bspline(basis, [&](auto Kc) {
        constexpr int K = decltype(Kc)::value;
        if (gr) bs_musl2d_p2g_kernel<K, true><<<nb, 256, 0, s>>>(g, nd, pp, grav[0], grav[1], status);
        else bs_musl2d_p2g_kernel<K, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, status);
      });
    }
  } else {
    // the 3D MUSL applies no body force
    if (basis == MPM_BASIS_LINEAR) {
      p2g_kernel<D, double, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, 0.0, status);
    } else {
      with_bspline(basis, [&](auto Kc) {
        bs_p2g_kernel<D, double, decltype(Kc)::value, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, 0.0, status);
      });
    }
  }
}

template <int D>
void Launchers<D>::musl_grid(cudaStream_t s, const NodeP& nd, const CgP& cg, double dt, double alpha,
                             unsigned* status, int basis) {
  compact_blocks_kernel<<<blocks_for(nd.nblk, 256), 256, 0, s>>>(nd);
  if constexpr (D == 2) {
    const int K = basis_nodes(basis);
    if (K == 2) musl2d_cg_kernel<2><<<4, 1024, 0, s>>>(nd, cg, dt, status);
    else if (K == 3) musl2d_cg_kernel<3><<<4, 1024, 0, s>>>(nd, cg, dt, status);
    else musl2d_cg_kernel<4><<<4, 1024, 0, s>>>(nd, cg, dt, status);
    musl2d_node_kernel<<<sparse_ctas(nd), 256, 0, s>>>(nd, cg, dt, alpha);
  } else {
    musl_lumped_grid_kernel<D><<<sparse_ctas(nd), 256, 0, s>>>(nd, dt, alpha);
  }
}

template <int D>
void Launchers<D>::musl_g2p1(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, double alpha,
                             unsigned* status, int basis) {
  if (pp.count <= 0) return;
  const unsigned nb = blocks_for(pp.count, 256);
  if (basis == MPM_BASIS_LINEAR) {
    musl_g2p1_kernel<D, D == 3><<<nb, 256, 0, s>>>(g, nd, pp, alpha, status);
  } else {
    with_bspline(basis, [&](auto Kc) {
      bs_musl_g2p1_kernel<D, decltype(Kc)::value, D == 3><<<nb, 256, 0, s>>>(g, nd, pp, alpha, status);
    });
  }
}

template <int D>
void Launchers<D>::musl_vg(cudaStream_t s, const NodeP& nd, double dt) {
  if constexpr (D == 3) musl_vg_kernel<D><<<sparse_ctas(nd), 256, 0, s>>>(nd, dt);
}

template <int D>
void Launchers<D>::musl_g2p2(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, const MatParams& mp,
                             unsigned* status, int basis) {
  if (pp.count <= 0) return;
  const unsigned nb = blocks_for(pp.count, 256);
  with_material<D>(mp.type, [&](auto Mc) {
    constexpr int M = decltype(Mc)::value;
    if (basis == MPM_BASIS_LINEAR) {
      musl_g2p2_kernel<D, M, D == 3><<<nb, 256, 0, s>>>(g, nd, pp, mp, status);
    } else {
      with_bspline(basis, [&](auto Kc) {
        bs_musl_g2p2_kernel<D, decltype(Kc)::value, M, D == 3><<<nb, 256, 0, s>>>(g, nd, pp, mp, status);
      });
    }
  });
}

template <int D>
void Launchers<D>::bs_p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                          const double* grav, unsigned* status, int basis) {
  if (pp.count <= 0) return;
  const unsigned nb = blocks_for(pp.count, 256);
  const bool gr = grav[0] != 0.0 || grav[1] != 0.0 || (D == 3 && grav[2] != 0.0);
  with_bspline(basis, [&](auto Kc) {
    constexpr int K = decltype(Kc)::value;
    if (!f32 && nd.dw4) {
      // double-word P2G (MPM_PREC_DW contexts, 3D)
      if constexpr (D == 3) {
        if (gr) bs_p2g_dw_kernel<K, true><<<nb, 256, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status);
        else bs_p2g_dw_kernel<K, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, 0.0, status);
      }
      return;
    }
    if (f32) {
      if (gr) bs_p2g_kernel<D, float, K, true><<<nb, 256, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status);
      else bs_p2g_kernel<D, float, K, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, 0.0, status);
    } else {
      if (gr) bs_p2g_kernel<D, double, K, true><<<nb, 256, 0, s>>>(g, nd, pp, grav[0], grav[1], grav[2], status);
      else bs_p2g_kernel<D, double, K, false><<<nb, 256, 0, s>>>(g, nd, pp, 0.0, 0.0, 0.0, status);
    }
  });
}

template <int D>
void Launchers<D>::bs_g2p(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                          const MatParams& mp, unsigned* status, int basis) {
  if (pp.count <= 0) return;
  const unsigned nb = blocks_for(pp.count, 256);
  with_material<D>(mp.type, [&](auto Mc) {
    constexpr int M = decltype(Mc)::value;
    with_bspline(basis, [&](auto Kc) {
      constexpr int K = decltype(Kc)::value;
      if (!f32 && nd.dw4) {
        // double-word G2P (MPM_PREC_DW contexts: 3D, linear elastic or J2 bodies)
        if constexpr (D == 3 && (M == MPM_MAT_ELASTIC || M == MPM_MAT_J2))
          bs_g2p_dw_kernel<K, M><<<nb, 256, 0, s>>>(g, nd, pp, mp, status);
        return;
      }
      if (f32) bs_g2p_kernel<D, float, K, M><<<nb, 256, 0, s>>>(g, nd, pp, mp, status);
      else bs_g2p_kernel<D, double, K, M><<<nb, 256, 0, s>>>(g, nd, pp, mp, status);
    });
  });
}

template <int D>
void Launchers<D>::g2p(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                       const MatParams& mp, double dt, unsigned* status, int threads) {
  if (pp.count <= 0) return;
  const int th = threads > 0 ? threads : 256;
  unsigned nb = blocks_for(pp.count, th);
#define JMPM_G2P(R, M) g2p_kernel<D, R, M><<<nb, th, 0, s>>>(g, nd, pp, mp, dt, status)
  if (!f32 && nd.dw4) {
    // double-word G2P (MPM_PREC_DW contexts: 3D, linear elastic or J2 bodies)
    if constexpr (D == 3) {
      // the inputs' shared-memory slots: 28 doubles per thread (57 KB at 256
      // threads; dw_setup raised the kernels' limit)
      const size_t smem = size_t(DwSlots::N) * size_t(th) * sizeof(double);
      if (mp.type == MPM_MAT_ELASTIC) g2p_dw_kernel<MPM_MAT_ELASTIC><<<nb, th, smem, s>>>(g, nd, pp, mp, status);
      else g2p_dw_kernel<MPM_MAT_J2><<<nb, th, smem, s>>>(g, nd, pp, mp, status);
    }
    return;
  }
  if (f32 && nd.nf4 && mp.type == MPM_MAT_J2 && D == 3) {
    // FP32 J2 with interleaved node records: the constitutive inputs prefetched
    const size_t smem = size_t(g2p_prefetch_slots<D>()) * size_t(th) * sizeof(float);
    g2p_prefetch_kernel<D, float><<<nb, th, smem, s>>>(g, nd, pp, mp, dt, status);
    return;
  }
  if (f32) {
    switch (mp.type) {
      case MPM_MAT_ELASTIC: JMPM_G2P(float, MPM_MAT_ELASTIC); break;
      case MPM_MAT_NEOHOOKEAN: JMPM_G2P(float, MPM_MAT_NEOHOOKEAN); break;
      case MPM_MAT_JOHNSON_COOK: if constexpr (D == 3) JMPM_G2P(float, MPM_MAT_JOHNSON_COOK); break;
      case MPM_MAT_VOCE: if constexpr (D == 3) JMPM_G2P(float, MPM_MAT_VOCE); break;
      case MPM_MAT_JOHNSON_COOK_DAMAGE: if constexpr (D == 3) JMPM_G2P(float, MPM_MAT_JOHNSON_COOK_DAMAGE); break;
      default: JMPM_G2P(float, MPM_MAT_J2); break;
    }
  } else {
    switch (mp.type) {
      case MPM_MAT_ELASTIC: JMPM_G2P(double, MPM_MAT_ELASTIC); break;
      case MPM_MAT_NEOHOOKEAN: JMPM_G2P(double, MPM_MAT_NEOHOOKEAN); break;
      case MPM_MAT_JOHNSON_COOK: if constexpr (D == 3) JMPM_G2P(double, MPM_MAT_JOHNSON_COOK); break;
      case MPM_MAT_VOCE: if constexpr (D == 3) JMPM_G2P(double, MPM_MAT_VOCE); break;
      case MPM_MAT_JOHNSON_COOK_DAMAGE: if constexpr (D == 3) JMPM_G2P(double, MPM_MAT_JOHNSON_COOK_DAMAGE); break;
      default: JMPM_G2P(double, MPM_MAT_J2); break;
    }
  }
#undef JMPM_G2P
}

template <int D>
cudaError_t Launchers<D>::dw_setup() {
  if constexpr (D == 3) {
    const int most = int(DwSlots::N * 256 * sizeof(double));
    cudaError_t e = cudaFuncSetAttribute(g2p_dw_kernel<MPM_MAT_ELASTIC>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(g2p_dw_kernel<MPM_MAT_J2>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    return e;
  }
  return cudaSuccess;
}

template <int D>
void Launchers<D>::energies(cudaStream_t s, const PartP& pp, bool f32, double* partial, int nblocks,
                            double* out, EnRec* rec) {
  // the ticket of the last-CTA fold sits after the nblocks x 5 partial sums
  unsigned* ticket = reinterpret_cast<unsigned*>(partial + size_t(nblocks) * 5);
  if (f32) energies_kernel<D, float><<<nblocks, 256, 0, s>>>(pp, partial, ticket, out, rec);
  else energies_kernel<D, double><<<nblocks, 256, 0, s>>>(pp, partial, ticket, out, rec);
}

template <int D>
void Launchers<D>::aos_to_soa(cudaStream_t s, const PartP& pp, bool f32, const double* src, int per,
                              int f0, const CompMapH& cm) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) aos_to_soa_kernel<float><<<nb, 256, 0, s>>>(pp, src, per, f0, to_dev(cm));
  else aos_to_soa_kernel<double><<<nb, 256, 0, s>>>(pp, src, per, f0, to_dev(cm));
}

template <int D>
void Launchers<D>::soa_to_aos(cudaStream_t s, const PartP& pp, bool f32, double* dst, int per, int f0,
                              const CompMapH& cm) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) soa_to_aos_kernel<float><<<nb, 256, 0, s>>>(pp, dst, per, f0, to_dev(cm));
  else soa_to_aos_kernel<double><<<nb, 256, 0, s>>>(pp, dst, per, f0, to_dev(cm));
}

template <int D>
void Launchers<D>::soa_to_aos_perm(cudaStream_t s, const PartP& pp, bool f32, const int64_t* orig, double* dst,
                                   int per, int f0, const CompMapH& cm) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) soa_to_aos_perm_kernel<float><<<nb, 256, 0, s>>>(pp, orig, dst, per, f0, to_dev(cm));
  else soa_to_aos_perm_kernel<double><<<nb, 256, 0, s>>>(pp, orig, dst, per, f0, to_dev(cm));
}

template <int D>
void Launchers<D>::j2_vm_perm(cudaStream_t s, const PartP& pp, bool f32, const int64_t* orig, double* dst) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) j2_vm_perm_kernel<D, float><<<nb, 256, 0, s>>>(pp, orig, dst);
  else j2_vm_perm_kernel<D, double><<<nb, 256, 0, s>>>(pp, orig, dst);
}

template <int D>
void Launchers<D>::sort_keys(cudaStream_t s, const GridP& g, const PartP& pp, bool f32, uint32_t body_base,
                             uint32_t ncells, const SortP& sp) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) sort_keys_kernel<D, float><<<nb, 256, 0, s>>>(g, pp, body_base, ncells, sp);
  else sort_keys_kernel<D, double><<<nb, 256, 0, s>>>(g, pp, body_base, ncells, sp);
}

template <int D>
void Launchers<D>::scan(cudaStream_t s, const uint32_t* in, uint32_t* out, uint32_t* blocksum, int64_t n) {
  if (n <= 0) return;
  unsigned nb = blocks_for(n, 1024);
  scan_blocks_kernel<<<nb, 1024, 0, s>>>(in, out, blocksum, n);
  scan_sums_kernel<<<1, 1024, 0, s>>>(blocksum, nb);
  scan_add_kernel<<<nb, 1024, 0, s>>>(out, blocksum, n);
}

template <int D>
void Launchers<D>::sort_scatter(cudaStream_t s, bool f32, const void* src, void* dst, int64_t pitch, int nf,
                                const SortP& sp, const int64_t* orig_src, int64_t* orig_dst) {
  if (pitch <= 0) return;
  unsigned nb = blocks_for(pitch, 256);
  if (f32)
    sort_scatter_kernel<float><<<nb, 256, 0, s>>>(static_cast<const float*>(src), static_cast<float*>(dst), pitch,
                                                  nf, sp, orig_src, orig_dst);
  else
    sort_scatter_kernel<double><<<nb, 256, 0, s>>>(static_cast<const double*>(src), static_cast<double*>(dst),
                                                   pitch, nf, sp, orig_src, orig_dst);
}

template <int D>
void Launchers<D>::j2_vm(cudaStream_t s, const PartP& pp, bool f32, double* dst) {
  if (pp.count <= 0) return;
  unsigned nb = blocks_for(pp.count, 256);
  if (f32) j2_vm_kernel<D, float><<<nb, 256, 0, s>>>(pp, dst);
  else j2_vm_kernel<D, double><<<nb, 256, 0, s>>>(pp, dst);
}

}  // namespace jmpm
