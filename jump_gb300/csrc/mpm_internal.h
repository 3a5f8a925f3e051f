// mpm_internal.h -- host-side launchers of the step kernels (explicitly
// instantiated per dimension in mpm_k2d.cu / mpm_k3d.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "mpm_common.cuh"

namespace jmpm {

struct CompMapH {
  int n;
  int src[9];
};

template <int D>
struct Launchers {
  static void p2g(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                  const double* grav, unsigned* status);
  static void grid(cudaStream_t s, const NodeP& nd, double dt, double tol, bool f32copy);
  static void g2p(cudaStream_t s, const GridP& g, const NodeP& nd, const PartP& pp, bool f32,
                  const MatParams& mp, double dt, unsigned* status);
  static void energies(cudaStream_t s, const PartP& pp, bool f32, double* partial, int nblocks,
                       double* out);
  static void aos_to_soa(cudaStream_t s, const PartP& pp, bool f32, const double* src, int per, int f0,
                         const CompMapH& cm);
  static void soa_to_aos(cudaStream_t s, const PartP& pp, bool f32, double* dst, int per, int f0,
                         const CompMapH& cm);
  static void j2_vm(cudaStream_t s, const PartP& pp, bool f32, double* dst);
};

constexpr int kEnergyBlocks = 304;  // 2 x 152 SMs

// Records msg as the calling thread's mpm_last_error() text; returns code.
int set_last_error(int code, const std::string& msg);

}  // namespace jmpm
