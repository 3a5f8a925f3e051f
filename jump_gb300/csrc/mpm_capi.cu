// mpm_capi.cu -- the C ABI of include/jump_mpm.h: context lifetime, host <->
// device layout conversion and the step loop (one captured CUDA graph per
// USL step, replayed nsteps times on the context's stream).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jump_mpm.h"
#include "mpm_internal.h"

using namespace jmpm;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(x)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess)                                                           \
      return fail(MPM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));    \
  } while (0)

int sym_slot(int dim, int i, int j) {
  if (i == j) return i;
  if (dim == 2) return 2;
  int a = i < j ? i : j, b = i < j ? j : i;
  return (a == 0 && b == 1) ? 3 : ((a == 1 && b == 2) ? 4 : 5);
}

int num_fields(int dim) { return dim == 2 ? Layout<2>::NF : Layout<3>::NF; }

struct FieldIdx {
  int X, V, M, VOL, VOL0, F, EPS, SIG, VM, ALPHA, EP, LAM, MU, ALPHAD, S, PS;
};

template <int D>
FieldIdx make_idx() {
  using L = Layout<D>;
  return FieldIdx{L::X, L::V, L::M, L::VOL, L::VOL0, L::F, L::EPS, L::SIG,
                  L::VM, L::ALPHA, L::EP, L::LAM, L::MU, L::ALPHAD, L::S, L::PS};
}

}  // namespace

int jmpm::set_last_error(int code, const std::string& msg) { return fail(code, msg); }

struct mpm_ctx {
  int dim = 2;
  bool f32 = false;
  bool dw = false;            // MPM_PREC_DW: FP64 particles, double-word FP32 G2P
  mpm_params prm{};
  int nb = 0;
  std::vector<int64_t> off, cnt;
  std::vector<MatParams> mats;
  int64_t np = 0;
  int NF = 0;
  size_t esz = 8;
  FieldIdx fi{};
  void* P = nullptr;          // particle SoA in use
  void* Palt = nullptr;       // the other buffer of the counting sort (sort_interval > 0)
  int32_t* hat_c = nullptr;   // hat cache of the linear USL step (PartP::hat_c), dim * np
  void* hat_nl = nullptr;     // and its lower hat values (particle type), dim * np
  int64_t* orig = nullptr;    // orig[slot]: original (creation-order) index of the particle in slot
  int64_t* orig_alt = nullptr;
  int cur = 0;                // which physical buffer P is (selects the captured graph)
  SortP sp{};
  uint32_t ncells = 0;
  int64_t since_sort = 0;
  GridP g{};
  NodeP nd{};
  double* coords = nullptr;
  uint8_t* fixed = nullptr;
  uint32_t* blockbuf = nullptr;  // node-block flags | list | count
  std::vector<double> nus;       // Poisson ratio per body (dlambda/dE, dmu/dE of the adjoint)
  // reverse mode: checkpoints of mpm_fwd_checkpointed and the adjoint work buffers
  char* ckpt = nullptr;
  int64_t ckpt_slots = 0, adj_nsteps = -1;
  int32_t adj_every = 0;
  char* segbuf = nullptr;
  int32_t segbuf_slots = 0;
  // captured reverse-mode segments: [kind: 0 recompute, 1 reverse sweep][segment
  // buffer][full or last (shorter) segment length]
  cudaGraph_t seg_graph[2][2][2] = {};
  cudaGraphExec_t seg_exec[2][2][2] = {};
  int seg_len[2][2][2] = {};
  double* gridrec = nullptr;
  double* adjbuf = nullptr;
  double* nodeadj = nullptr;
  unsigned* revbar = nullptr;  // fused reverse step: barrier arrivals, generation, error flag
  void* fused = nullptr;       // barrier words of the fused steps (MPM_P2G_FUSED)
  bool full_clear = false;     // the node accumulators need a dense clear before the next graph step
  bool coop_off = false;       // the fused reverse step could not be captured: three kernels per step
  ContactP cp{};                 // contact mode: per-body node fields
  double* contactbuf = nullptr;
  float* contactbuf_f = nullptr;
  double* nodebuf = nullptr;
  double* fullrec = nullptr;  // reverse mode, checkpoint every step: every step's node buffer
  int64_t fullrec_steps = 0;
  double* muslbuf = nullptr;  // MUSL: 3D p2 | vg; 2D mass stencil (9) | vg | CG vectors (16)
  CgP cg{};
  float* nodebuf_f = nullptr;
  float4* nodebuf_dw = nullptr;  // MPM_PREC_DW: the grid update's double-word node records (NodeP::dw4)
  std::vector<uint8_t> fixed_h;
  // rigid bodies (MPM_MAT_RIGID): rigid ordinal of each body (-1: deformable),
  // the per-node marks and the {fixed, vx, vy, vz} table (device and host)
  std::vector<int> rigid_bit;
  uint32_t* rmask = nullptr;
  double* rtab = nullptr;
  std::vector<double> rtab_h;
  bool rigid(int b) const { return rigid_bit[b] >= 0; }
  unsigned* status = nullptr;
  double* partial = nullptr;
  double* red = nullptr;
  double* staging = nullptr;
  size_t staging_n = 0;
  int p2g_strategy = MPM_P2G_ATOMIC;  // linear-basis USL P2G (mpm_set_launch)
  int threads = 256;                  // CTA size of the linear-basis P2G and G2P
  double* rec_host = nullptr;   // pinned EnergiesFix records of mpm_step_energies
  double* rec_dev = nullptr;    // the same records as the steps form them, on the device
  int64_t rec_cap = 0;          // records each holds
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // reverse mode: the second stream the reverse sweep runs on while the first
  // recomputes the next segment, and the events that order the two
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_adj[2] = {nullptr, nullptr}, ev_sync = nullptr;
  cudaGraph_t graph[2] = {nullptr, nullptr};       // one step, per physical buffer
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  // the same step followed by its EnergiesFix sums, written through the
  // device record cursor en_rec (mpm_step_energies)
  cudaGraph_t graph_en[2] = {nullptr, nullptr};
  cudaGraphExec_t exec_en[2] = {nullptr, nullptr};
  EnRec* en_rec = nullptr;    // device record cursor of the captured energies
  EnRec* en_rec_h = nullptr;  // pinned host copy it is set from
  double last_ms = 0.0;

  PartP part(int b) const {
    PartP pp{};
    pp.base = P;
    pp.pitch = np;
    pp.begin = off[b];
    pp.count = cnt[b];
    return pp;
  }
  // the linear USL step's P2G and G2P: part(b) with the hat cache, for FP64
  // particles (the G2P saves the FP64 work of the hat: 0.270 -> 0.238 ms per
  // step on the Taylor bar, net 0.464 -> 0.438 ms; with FP32 particles the hat
  // is FP32 work and reading it back was slower than recomputing it)
  PartP step_part(int b) const {
    PartP pp = part(b);
    if (!f32) {
      pp.hat_c = hat_c;
      pp.hat_nl = hat_nl;
    }
    return pp;
  }
  PartP all() const {
    PartP pp{};
    pp.base = P;
    pp.pitch = np;
    pp.begin = 0;
    pp.count = np;
    return pp;
  }
};

namespace {

// orig[i] = i
__global__ void iota_kernel(int64_t* p, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    p[i] = i;
}

// drop the captured reverse-mode segment graphs (their buffers changed)
void drop_seg_graphs(mpm_ctx* c) {
  for (int k = 0; k < 2; ++k)
    for (int b = 0; b < 2; ++b)
      for (int l = 0; l < 2; ++l) {
        if (c->seg_exec[k][b][l]) cudaGraphExecDestroy(c->seg_exec[k][b][l]);
        if (c->seg_graph[k][b][l]) cudaGraphDestroy(c->seg_graph[k][b][l]);
        c->seg_exec[k][b][l] = nullptr;
        c->seg_graph[k][b][l] = nullptr;
        c->seg_len[k][b][l] = 0;
      }
}

void destroy_ctx(mpm_ctx* c) {
  if (!c) return;
  cudaFreeHost(c->rec_host);
  cudaFree(c->rec_dev);
  for (int i = 0; i < 2; ++i) {
    if (c->exec[i]) cudaGraphExecDestroy(c->exec[i]);
    if (c->graph[i]) cudaGraphDestroy(c->graph[i]);
    if (c->exec_en[i]) cudaGraphExecDestroy(c->exec_en[i]);
    if (c->graph_en[i]) cudaGraphDestroy(c->graph_en[i]);
  }
  cudaFree(c->en_rec);
  cudaFreeHost(c->en_rec_h);
  cudaFree(c->P);
  cudaFree(c->Palt);
  cudaFree(c->hat_c);
  cudaFree(c->orig);
  cudaFree(c->orig_alt);
  cudaFree(c->sp.key);
  cudaFree(c->sp.rank);
  cudaFree(c->sp.count);
  cudaFree(c->sp.offset);
  cudaFree(c->sp.blocksum);
  cudaFree(c->coords);
  cudaFree(c->fixed);
  cudaFree(c->nodebuf);
  cudaFree(c->fullrec);
  cudaFree(c->muslbuf);
  cudaFree(c->nodebuf_f);
  cudaFree(c->nodebuf_dw);
  cudaFree(c->blockbuf);
  cudaFree(c->rmask);
  cudaFree(c->rtab);
  drop_seg_graphs(c);
  cudaFree(c->ckpt);
  cudaFree(c->segbuf);
  cudaFree(c->gridrec);
  cudaFree(c->adjbuf);
  cudaFree(c->nodeadj);
  cudaFree(c->revbar);
  cudaFree(c->fused);
  cudaFree(c->contactbuf);
  cudaFree(c->contactbuf_f);
  cudaFree(c->status);
  cudaFree(c->partial);
  cudaFree(c->red);
  cudaFree(c->staging);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  for (int i = 0; i < 2; ++i) {
    if (c->ev_rec[i]) cudaEventDestroy(c->ev_rec[i]);
    if (c->ev_adj[i]) cudaEventDestroy(c->ev_adj[i]);
  }
  if (c->ev_sync) cudaEventDestroy(c->ev_sync);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

void launch_aos_to_soa(mpm_ctx* c, const PartP& pp, const double* src, int per, int f0,
                       const CompMapH& cm) {
  if (c->dim == 2) Launchers<2>::aos_to_soa(c->stream, pp, c->f32, src, per, f0, cm);
  else Launchers<3>::aos_to_soa(c->stream, pp, c->f32, src, per, f0, cm);
}

// device SoA -> host AoS in original particle order (through orig[])
void launch_soa_to_aos(mpm_ctx* c, const PartP& pp, double* dst, int per, int f0, const CompMapH& cm) {
  if (c->dim == 2) Launchers<2>::soa_to_aos_perm(c->stream, pp, c->f32, c->orig, dst, per, f0, cm);
  else Launchers<3>::soa_to_aos_perm(c->stream, pp, c->f32, c->orig, dst, per, f0, cm);
}

// second particle buffer + key/rank/count arrays of the counting sort
int alloc_sort(mpm_ctx* c) {
  if (c->Palt || c->np == 0) return MPM_OK;
  if (int64_t(c->nb) * (int64_t(c->ncells) + 1) >= (int64_t(1) << 32))
    return fail(MPM_ERR_ARG, "too many (body, cell) keys for the particle sort");
  CUDA_TRY(cudaMalloc(&c->Palt, size_t(c->NF) * size_t(c->np) * c->esz));
  CUDA_TRY(cudaMalloc(&c->orig_alt, size_t(c->np) * sizeof(int64_t)));
  c->sp.nkeys = int64_t(c->nb) * (int64_t(c->ncells) + 1);
  CUDA_TRY(cudaMalloc(&c->sp.key, size_t(c->np) * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->sp.rank, size_t(c->np) * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->sp.count, size_t(c->sp.nkeys) * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->sp.offset, size_t(c->sp.nkeys) * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->sp.blocksum, size_t((c->sp.nkeys + 1023) / 1024) * sizeof(uint32_t)));
  return MPM_OK;
}

// drop the captured step graphs (the launch configuration changed)
void invalidate_graphs(mpm_ctx* c) {
  for (int i = 0; i < 2; ++i) {
    if (c->exec[i]) cudaGraphExecDestroy(c->exec[i]);
    if (c->graph[i]) cudaGraphDestroy(c->graph[i]);
    if (c->exec_en[i]) cudaGraphExecDestroy(c->exec_en[i]);
    if (c->graph_en[i]) cudaGraphDestroy(c->graph_en[i]);
    c->exec[i] = c->exec_en[i] = nullptr;
    c->graph[i] = c->graph_en[i] = nullptr;
  }
  drop_seg_graphs(c);
}

// Counting sort of all particles by (body, cell) into the other buffer; swaps buffers.
int enqueue_sort(mpm_ctx* c) {
  if (!c->Palt || c->np == 0) return MPM_OK;
  CUDA_TRY(cudaMemsetAsync(c->sp.count, 0, size_t(c->sp.nkeys) * sizeof(uint32_t), c->stream));
  for (int b = 0; b < c->nb; ++b) {
    uint32_t base = uint32_t(b) * (c->ncells + 1);
    if (c->dim == 2) Launchers<2>::sort_keys(c->stream, c->g, c->part(b), c->f32, base, c->ncells, c->sp);
    else Launchers<3>::sort_keys(c->stream, c->g, c->part(b), c->f32, base, c->ncells, c->sp);
  }
  Launchers<2>::scan(c->stream, c->sp.count, c->sp.offset, c->sp.blocksum, c->sp.nkeys);
  Launchers<2>::sort_scatter(c->stream, c->f32, c->P, c->Palt, c->np, c->NF, c->sp, c->orig, c->orig_alt);
  CUDA_TRY(cudaGetLastError());
  std::swap(c->P, c->Palt);
  std::swap(c->orig, c->orig_alt);
  c->cur ^= 1;
  c->since_sort = 0;
  return MPM_OK;
}

// host AoS array -> staging -> SoA fields [f0, f0 + cm.n)
// host AoS array -> staging -> SoA fields [f0, f0 + cm.n).  Stream-ordered:
// the next copy into staging waits for this transpose; the caller
// synchronises once after the last upload, before its host arrays go.  (A
// transpose reading page-locked host arrays in place was slower: its strided
// accesses cross the host link in partial lines.)
int upload(mpm_ctx* c, int b, const double* host, int per, int f0, const CompMapH& cm) {
  size_t n = size_t(c->cnt[b]) * per;
  if (n == 0) return MPM_OK;
  CUDA_TRY(cudaMemcpyAsync(c->staging, host, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_aos_to_soa(c, c->part(b), c->staging, per, f0, cm);
  CUDA_TRY(cudaGetLastError());
  return MPM_OK;
}

// SoA fields -> staging (creation order) -> host AoS array.  Stream-ordered
// like upload; mpm_download synchronises once at its end.
int download(mpm_ctx* c, int b, double* host, int per, int f0, const CompMapH& cm) {
  size_t n = size_t(c->cnt[b]) * per;
  if (n == 0 || !host) return MPM_OK;
  launch_soa_to_aos(c, c->part(b), c->staging, per, f0, cm);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(host, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return MPM_OK;
}

CompMapH ident(int n) {
  CompMapH m{};
  m.n = n;
  for (int i = 0; i < n; ++i) m.src[i] = i;
  return m;
}

// upload: symmetric slot s <- column-major entry; with a flag, entries (i, j)
// and (j, i) are compared on the device and `bit` is set when they differ
CompMapH sym_from_full(int dim, unsigned* flag = nullptr, unsigned bit = 0) {
  CompMapH m{};
  m.n = dim == 2 ? 3 : 6;
  for (int j = 0; j < dim; ++j)
    for (int i = j; i < dim; ++i) m.src[sym_slot(dim, i, j)] = i + dim * j;
  for (int j = 0; j < dim; ++j)
    for (int i = j + 1; i < dim; ++i) {
      m.ca[m.nchk] = i + dim * j;
      m.cb[m.nchk] = j + dim * i;
      ++m.nchk;
    }
  m.flag = flag;
  m.bit = bit;
  return m;
}

// download: column-major entry <- symmetric slot
CompMapH full_from_sym(int dim) {
  CompMapH m{};
  m.n = dim * dim;
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) m.src[i + dim * j] = sym_slot(dim, i, j);
  return m;
}

// The launches of one USL step; ev (optional) gets an event recorded after each stage.
// rec (optional): receives this step's node buffer m | p0 | f | vdt | dv for the adjoint
// One MUSL step (mpm_musl.cuh); ev as enqueue_step.
void enqueue_musl(mpm_ctx* c, cudaEvent_t* ev) {
  const int D = c->dim;
  if (D == 2) Launchers<2>::clear(c->stream, c->nd);
  else Launchers<3>::clear(c->stream, c->nd);
  cudaMemsetAsync(c->nd.bcount, 0, sizeof(uint32_t), c->stream);
  if (ev) cudaEventRecord(ev[0], c->stream);
  const int basis = c->prm.basis;
  for (int b = 0; b < c->nb; ++b) {
    if (D == 2) Launchers<2>::musl_p2g(c->stream, c->g, c->nd, c->part(b), c->prm.body_force, c->status, basis);
    else Launchers<3>::musl_p2g(c->stream, c->g, c->nd, c->part(b), c->prm.body_force, c->status, basis);
  }
  if (ev) cudaEventRecord(ev[1], c->stream);
  if (D == 2) Launchers<2>::musl_grid(c->stream, c->nd, c->cg, c->prm.dt, c->prm.alpha, c->status, basis);
  else Launchers<3>::musl_grid(c->stream, c->nd, c->cg, c->prm.dt, c->prm.alpha, c->status, basis);
  if (ev) cudaEventRecord(ev[2], c->stream);
  for (int b = 0; b < c->nb; ++b) {
    if (D == 2) Launchers<2>::musl_g2p1(c->stream, c->g, c->nd, c->part(b), c->prm.alpha, c->status, basis);
    else Launchers<3>::musl_g2p1(c->stream, c->g, c->nd, c->part(b), c->prm.alpha, c->status, basis);
  }
  if (D == 3) Launchers<3>::musl_vg(c->stream, c->nd, c->prm.dt);
  for (int b = 0; b < c->nb; ++b) {
    if (D == 2) Launchers<2>::musl_g2p2(c->stream, c->g, c->nd, c->part(b), c->mats[b], c->status, basis);
    else Launchers<3>::musl_g2p2(c->stream, c->g, c->nd, c->part(b), c->mats[b], c->status, basis);
  }
  if (ev) cudaEventRecord(ev[3], c->stream);
}

// P2G strategy of the per-stage launches: MPM_P2G_FUSED contexts that take
// the per-stage path (checkpointed forward, stage profiling, the reverse
// sweep's recompute) use per-particle atomics there
static int graph_strategy(const mpm_ctx* c) {
  return c->p2g_strategy == MPM_P2G_FUSED ? MPM_P2G_ATOMIC : c->p2g_strategy;
}

// The launches of one step's kernels (enqueue_step).
static void enqueue_step_kernels(mpm_ctx* c, cudaEvent_t* ev, double* rec) {
  if (c->prm.algorithm == MPM_ALG_MUSL) {
    enqueue_musl(c, ev);
    return;
  }
  const int D = c->dim;
  const bool contact = c->prm.contact != 0;
  // node field of body b: its own in contact mode, else the shared one
  auto field_of = [&](int b) -> const NodeP& { return contact ? c->cp.body[b] : c->nd; };
  // reset (:381-385): only the blocks the previous step touched hold non-zeros
  for (int b = 0; b < (contact ? c->nb : 1); ++b) {
    if (D == 2) Launchers<2>::clear(c->stream, field_of(b));
    else Launchers<3>::clear(c->stream, field_of(b));
  }
  cudaMemsetAsync(c->nd.bcount, 0, sizeof(uint32_t), c->stream);
  if (ev) cudaEventRecord(ev[0], c->stream);
  const int basis = c->prm.basis;
  for (int b = 0; b < c->nb; ++b) {
    if (c->rigid(b)) continue;  // rigid solids add nothing (:394)
    if (basis != MPM_BASIS_LINEAR) {
      if (D == 2) Launchers<2>::bs_p2g(c->stream, c->g, field_of(b), c->part(b), c->f32, c->prm.body_force, c->status, basis);
      else Launchers<3>::bs_p2g(c->stream, c->g, field_of(b), c->part(b), c->f32, c->prm.body_force, c->status, basis);
    } else if (D == 2) {
      Launchers<2>::p2g(c->stream, c->g, field_of(b), c->step_part(b), c->f32, c->prm.body_force, c->status,
                        graph_strategy(c), c->threads);
    } else {
      Launchers<3>::p2g(c->stream, c->g, field_of(b), c->step_part(b), c->f32, c->prm.body_force, c->status,
                        graph_strategy(c), c->threads);
    }
  }
  // rigid solids: mark the nodes the grid update overrides, then move them
  for (int b = 0; b < c->nb; ++b) {
    if (!c->rigid(b)) continue;
    const double* v = c->rtab_h.data() + 4 * c->rigid_bit[b] + 1;
    if (D == 2) Launchers<2>::rigid(c->stream, c->g, c->nd, c->part(b), c->f32, c->rigid_bit[b], v, c->prm.dt, c->status);
    else Launchers<3>::rigid(c->stream, c->g, c->nd, c->part(b), c->f32, c->rigid_bit[b], v, c->prm.dt, c->status);
  }
  if (ev) cudaEventRecord(ev[1], c->stream);
  if (contact) {
    if (D == 2) Launchers<2>::contact_grid(c->stream, c->nd, c->cp, c->prm.dt, c->prm.tolerance, c->f32);
    else Launchers<3>::contact_grid(c->stream, c->nd, c->cp, c->prm.dt, c->prm.tolerance, c->f32);
  } else {
    if (D == 2) Launchers<2>::grid(c->stream, c->nd, c->prm.dt, c->prm.tolerance, c->f32);
    else Launchers<3>::grid(c->stream, c->nd, c->prm.dt, c->prm.tolerance, c->f32);
  }
  if (rec) {
    // the node buffer m | p0 | f | vdt | dv in one copy (the adjoint reads m, vdt, dv)
    const size_t Nn = size_t(c->nd.nodeCount);
    cudaMemcpyAsync(rec, c->nodebuf, Nn * (1 + 4 * D) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  }
  if (ev) cudaEventRecord(ev[2], c->stream);
  for (int b = 0; b < c->nb; ++b) {
    if (c->rigid(b)) continue;  // rigid solids take no G2P (:488)
    if (basis != MPM_BASIS_LINEAR) {
      if (D == 2) Launchers<2>::bs_g2p(c->stream, c->g, field_of(b), c->part(b), c->f32, c->mats[b], c->status, basis);
      else Launchers<3>::bs_g2p(c->stream, c->g, field_of(b), c->part(b), c->f32, c->mats[b], c->status, basis);
    } else if (D == 2) {
      Launchers<2>::g2p(c->stream, c->g, field_of(b), c->step_part(b), c->f32, c->mats[b], c->prm.dt, c->status,
                        c->threads);
    } else {
      Launchers<3>::g2p(c->stream, c->g, field_of(b), c->step_part(b), c->f32, c->mats[b], c->prm.dt, c->status,
                        c->threads);
    }
  }
  if (ev) cudaEventRecord(ev[3], c->stream);
}

// en: the step's EnergiesFix sums follow it, written through the record cursor
// c->en_rec (a captured step fills successive records)
void enqueue_step(mpm_ctx* c, cudaEvent_t* ev, double* rec = nullptr, bool en = false) {
  enqueue_step_kernels(c, ev, rec);
  if (!en || c->np == 0) return;
  if (c->dim == 2) Launchers<2>::energies(c->stream, c->all(), c->f32, c->partial, kEnergyBlocks, nullptr, c->en_rec);
  else Launchers<3>::energies(c->stream, c->all(), c->f32, c->partial, kEnergyBlocks, nullptr, c->en_rec);
}

// The step graph of the buffer currently in use (captured on first use); en:
// the step followed by its EnergiesFix record.
int build_step_graph(mpm_ctx* c, bool en = false) {
  const int k = c->cur;
  cudaGraphExec_t& ex = en ? c->exec_en[k] : c->exec[k];
  cudaGraph_t& gr = en ? c->graph_en[k] : c->graph[k];
  if (ex) return MPM_OK;
  CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step(c, nullptr, nullptr, en);
  cudaError_t le = cudaGetLastError();
  cudaError_t ee = cudaStreamEndCapture(c->stream, &gr);
  if (le != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(le));
  if (ee != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
  CUDA_TRY(cudaGraphInstantiate(&ex, gr, 0));
  return MPM_OK;
}

int status_to_code(unsigned st) {
  if (st & ST_OUT_OF_GRID) return fail(MPM_ERR_OUT_OF_GRID, "a particle left the grid; it was frozen in place");
  if (st & ST_NONFINITE) return fail(MPM_ERR_NONFINITE, "non-finite particle velocity, position or stress");
  if (st & ST_NEGATIVE_J) return fail(MPM_ERR_NEGATIVE_J, "det F <= 0 at a particle");
  if (st & ST_SOLVER) return fail(MPM_ERR_SOLVER, "the MUSL mass solve did not converge");
  return MPM_OK;
}

int create_impl(const mpm_grid_desc* gd, const mpm_body_desc* bd, int32_t nbodies, const mpm_params* prm,
                mpm_ctx* c) {
  const int D = gd->dim;
  c->dim = D;
  c->prm = *prm;
  c->f32 = prm->precision == MPM_PREC_F32;
  c->dw = prm->precision == MPM_PREC_DW;
  c->esz = c->f32 ? sizeof(float) : sizeof(double);
  c->NF = num_fields(D);
  c->fi = D == 2 ? make_idx<2>() : make_idx<3>();
  c->nb = nbodies;
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&c->e0));
  CUDA_TRY(cudaEventCreate(&c->e1));

  // grid geometry, exactly as Grid2D/Grid3D build it (Grid.jl:105-107, 149-152, 199-204, 256-261)
  int64_t nn[3] = {1, 1, 1};
  double dx[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    nn[a] = gd->nodes[a];
    dx[a] = (gd->xmax[a] - gd->xmin[a]) / (double(gd->nodes[a]) - 1.0);
    c->g.xmin[a] = gd->xmin[a];
    c->g.dxI[a] = 1.0 / dx[a];
    c->g.dx[a] = dx[a];
    c->g.nn[a] = nn[a];
  }
  c->g.nx = nn[0];
  c->g.nxy = nn[0] * nn[1];
  c->g.nodeCount = c->g.nxy * nn[2];
  const int64_t Nn = c->g.nodeCount;
  std::vector<double> coords_h;
  for (int a = 0; a < D; ++a)
    for (int64_t i = 0; i < nn[a]; ++i) coords_h.push_back(gd->xmin[a] + double(i) * dx[a]);
  // node coordinates in FP64, then the same rounded to float for FP32 particles
  const size_t ncoord = coords_h.size();
  std::vector<float> coords_f(ncoord);
  for (size_t i = 0; i < ncoord; ++i) coords_f[i] = float(coords_h[i]);
  CUDA_TRY(cudaMalloc(&c->coords, ncoord * (sizeof(double) + sizeof(float))));
  CUDA_TRY(cudaMemcpy(c->coords, coords_h.data(), ncoord * sizeof(double), cudaMemcpyHostToDevice));
  float* coordf = reinterpret_cast<float*>(c->coords + ncoord);
  CUDA_TRY(cudaMemcpy(coordf, coords_f.data(), ncoord * sizeof(float), cudaMemcpyHostToDevice));
  int64_t o = 0;
  for (int a = 0; a < 3; ++a) {
    c->g.coord[a] = a < D ? c->coords + o : c->coords;
    c->g.coordf[a] = a < D ? coordf + o : coordf;
    c->g.xminf[a] = float(c->g.xmin[a]);
    c->g.dxIf[a] = float(c->g.dxI[a]);
    split_dw(c->g.dxI[a], c->g.w_dxI[a]);
    if (a < D) o += nn[a];
  }

  // Dirichlet mask (grid.fixedNodes, set by fix_Dirichlet_grid, Dirichlet.jl:28-78)
  c->fixed_h.assign(Nn, 0);
  if (gd->fixed_nodes) {
    const int64_t* f = gd->fixed_nodes;
    uint8_t* mk = c->fixed_h.data();
    if (D == 3)
      for (int64_t i = 0; i < Nn; ++i)
        mk[i] = uint8_t(int(f[3 * i] == 1) | (int(f[3 * i + 1] == 1) << 1) | (int(f[3 * i + 2] == 1) << 2));
    else
      for (int64_t i = 0; i < Nn; ++i) mk[i] = uint8_t(int(f[2 * i] == 1) | (int(f[2 * i + 1] == 1) << 1));
  }
  CUDA_TRY(cudaMalloc(&c->fixed, Nn));
  CUDA_TRY(cudaMemcpy(c->fixed, c->fixed_h.data(), Nn, cudaMemcpyHostToDevice));

  // node buffers: m | p0 (D) | f (D) | vdt (D) | dv (D)
  CUDA_TRY(cudaMalloc(&c->nodebuf, size_t(Nn) * (1 + 4 * D) * sizeof(double)));
  CUDA_TRY(cudaMemset(c->nodebuf, 0, size_t(Nn) * (1 + 4 * D) * sizeof(double)));
  c->nd.nodeCount = Nn;
  c->nd.m = c->nodebuf;
  c->nd.p0 = c->nodebuf + Nn;
  c->nd.f = c->nodebuf + Nn * (1 + D);
  c->nd.vdt = c->nodebuf + Nn * (1 + 2 * D);
  c->nd.dv = c->nodebuf + Nn * (1 + 3 * D);
  c->nd.fixed = c->fixed;
  {
    // node blocks of 64 (4x4x4 / 8x8) and their flag/list arrays
    const int B = D == 2 ? 8 : 4;
    c->nd.nblk = 1;
    for (int a = 0; a < 3; ++a) {
      c->nd.nn[a] = nn[a];
      c->nd.nb[a] = a < D ? (nn[a] + B - 1) / B : 1;
      c->nd.nblk *= c->nd.nb[a];
    }
    CUDA_TRY(cudaMalloc(&c->blockbuf, size_t(2 * c->nd.nblk + 1) * sizeof(uint32_t)));
    CUDA_TRY(cudaMemset(c->blockbuf, 0, size_t(2 * c->nd.nblk + 1) * sizeof(uint32_t)));
    c->nd.bflag = c->blockbuf;
    c->nd.blist = c->blockbuf + c->nd.nblk;
    c->nd.bcount = c->blockbuf + 2 * c->nd.nblk;
  }
  {
    // rigid bodies: their ordinal among the rigid bodies, node marks and velocity table
    int nr = 0;
    for (int b = 0; b < nbodies; ++b) {
      const bool r = bd[b].mat.type == MPM_MAT_RIGID;
      c->rigid_bit.push_back(r ? nr : -1);
      if (r) {
        const mpm_material_desc& m = bd[b].mat;
        c->rtab_h.insert(c->rtab_h.end(), {m.fixed != 0 ? 1.0 : 0.0, m.v_rigid[0], m.v_rigid[1],
                                           D == 3 ? m.v_rigid[2] : 0.0});
        ++nr;
      }
    }
    if (nr > 0) {
      CUDA_TRY(cudaMalloc(&c->rmask, size_t(Nn) * sizeof(uint32_t)));
      CUDA_TRY(cudaMemset(c->rmask, 0, size_t(Nn) * sizeof(uint32_t)));
      CUDA_TRY(cudaMalloc(&c->rtab, c->rtab_h.size() * sizeof(double)));
      CUDA_TRY(cudaMemcpy(c->rtab, c->rtab_h.data(), c->rtab_h.size() * sizeof(double), cudaMemcpyHostToDevice));
      c->nd.rmask = c->rmask;
      c->nd.rtab = c->rtab;
    }
  }
  if (prm->contact) {
    // per body: m | p0 (D) | f (D) | normal (D) | vdt (D) | dv (D), sharing mask and block list
    const size_t per = size_t(1 + 5 * D);
    CUDA_TRY(cudaMalloc(&c->contactbuf, size_t(Nn) * per * nbodies * sizeof(double)));
    CUDA_TRY(cudaMemset(c->contactbuf, 0, size_t(Nn) * per * nbodies * sizeof(double)));
    if (c->f32) {
      CUDA_TRY(cudaMalloc(&c->contactbuf_f, size_t(Nn) * 2 * D * nbodies * sizeof(float)));
      CUDA_TRY(cudaMemset(c->contactbuf_f, 0, size_t(Nn) * 2 * D * nbodies * sizeof(float)));
    }
    c->cp.nb = nbodies;
    c->cp.friction = prm->friction;
    for (int b = 0; b < nbodies; ++b) {
      NodeP f = c->nd;
      double* base = c->contactbuf + size_t(Nn) * per * b;
      f.m = base;
      f.p0 = base + Nn;
      f.f = base + Nn * (1 + D);
      f.nrm = base + Nn * (1 + 2 * D);
      f.vdt = base + Nn * (1 + 3 * D);
      f.dv = base + Nn * (1 + 4 * D);
      if (c->f32) {
        f.vdt_f = c->contactbuf_f + size_t(Nn) * 2 * D * b;
        f.dv_f = f.vdt_f + Nn * D;
      }
      c->cp.body[b] = f;
    }
  }
  if (prm->algorithm == MPM_ALG_MUSL) {
    // 3D: p2 (D) | vg (D); 2D: mass stencil (W*W, W = 2K - 1 for K support nodes per axis) | vg (D) |
    // CG x, r, p, q of four right-hand sides
    const int W = 2 * basis_nodes(prm->basis) - 1;
    const size_t per = D == 3 ? size_t(2 * D) : size_t(W * W + D + 16);
    CUDA_TRY(cudaMalloc(&c->muslbuf, size_t(Nn) * per * sizeof(double)));
    CUDA_TRY(cudaMemset(c->muslbuf, 0, size_t(Nn) * per * sizeof(double)));
    if (D == 3) {
      c->nd.p2 = c->muslbuf;
      c->nd.vg = c->muslbuf + Nn * D;
    } else {
      c->nd.mc = c->muslbuf;
      c->nd.nmc = W * W;
      c->nd.vg = c->muslbuf + Nn * (W * W);
      double* v = c->muslbuf + Nn * (W * W + D);
      for (int k = 0; k < 4; ++k) {
        c->cg.x[k] = v + Nn * (0 + k);
        c->cg.r[k] = v + Nn * (4 + k);
        c->cg.p[k] = v + Nn * (8 + k);
        c->cg.q[k] = v + Nn * (12 + k);
      }
    }
  }
  if (c->f32) {
    // the linear-basis USL G2P reads interleaved per-node records (NodeP::nf4);
    // the B-spline G2P the component-major copies
    const bool inter = prm->basis == MPM_BASIS_LINEAR && !prm->contact && prm->algorithm == MPM_ALG_USL;
    const size_t per = inter ? size_t(D == 2 ? 4 : 8) : size_t(2 * D);
    CUDA_TRY(cudaMalloc(&c->nodebuf_f, size_t(Nn) * per * sizeof(float)));
    CUDA_TRY(cudaMemset(c->nodebuf_f, 0, size_t(Nn) * per * sizeof(float)));
    c->nd.vdt_f = c->nodebuf_f;
    c->nd.dv_f = c->nodebuf_f + Nn * D;
    c->nd.nf4 = inter ? reinterpret_cast<float4*>(c->nodebuf_f) : nullptr;
  }

  if (c->dw) {
    // three float4 per node (NodeP::dw4), written by every grid update
    CUDA_TRY(cudaMalloc(&c->nodebuf_dw, size_t(Nn) * 3 * sizeof(float4)));
    CUDA_TRY(cudaMemset(c->nodebuf_dw, 0, size_t(Nn) * 3 * sizeof(float4)));
    c->nd.dw4 = c->nodebuf_dw;
    CUDA_TRY(Launchers<3>::dw_setup());
  }

  // particles
  int64_t maxn = 0;
  for (int b = 0; b < nbodies; ++b) {
    c->off.push_back(c->np);
    c->cnt.push_back(bd[b].count);
    c->np += bd[b].count;
    maxn = bd[b].count > maxn ? bd[b].count : maxn;
    const mpm_material_desc& m = bd[b].mat;
    c->mats.push_back(make_mat_params(m, bd[b].youngs != nullptr, prm->dt));
    c->nus.push_back(m.nu);
  }
  size_t ptot = size_t(c->NF) * size_t(c->np > 0 ? c->np : 1);
  CUDA_TRY(cudaMalloc(&c->P, ptot * c->esz));
  CUDA_TRY(cudaMemset(c->P, 0, ptot * c->esz));
  if (!c->f32 && c->np > 0 && c->g.nn[0] < (1 << 27) && c->g.nn[1] < (1 << 27) && c->g.nn[2] < (1 << 27)) {
    // hat cache: int32 codes, then the lower hat values (one allocation)
    const size_t nc = size_t(c->dim) * size_t(c->np);
    const size_t cbytes = (nc * sizeof(int32_t) + 15) / 16 * 16;
    char* hb = nullptr;
    CUDA_TRY(cudaMalloc(&hb, cbytes + nc * c->esz));
    c->hat_c = reinterpret_cast<int32_t*>(hb);
    c->hat_nl = hb + cbytes;
  }
  {
    // identity permutation: slot i holds particle i until the first sort
    const int64_t n = c->np > 0 ? c->np : 1;
    CUDA_TRY(cudaMalloc(&c->orig, size_t(n) * sizeof(int64_t)));
    iota_kernel<<<unsigned((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, c->stream>>>(c->orig, n);
    CUDA_TRY(cudaGetLastError());
  }
  c->ncells = 1;
  for (int a = 0; a < D; ++a) c->ncells *= uint32_t(nn[a] - 1);
  c->p2g_strategy = c->f32 ? MPM_P2G_WARP : MPM_P2G_ATOMIC;  // MPM_P2G_FUSED where it fits: set at the end
  c->threads = spread_threads(maxn);  // small bodies: smaller CTAs, spread over the SMs
  if (prm->sort_interval > 0 && c->np > 0) {
    int r = alloc_sort(c);
    if (r != MPM_OK) return r;
    c->since_sort = prm->sort_interval;  // sort before the first step
  }
  c->staging_n = size_t(maxn > 0 ? maxn : 1) * 9;
  CUDA_TRY(cudaMalloc(&c->staging, c->staging_n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&c->status, sizeof(unsigned)));
  CUDA_TRY(cudaMemset(c->status, 0, sizeof(unsigned)));
  // the energies' partial sums and, after them, the zeroed ticket of their fold
  CUDA_TRY(cudaMalloc(&c->partial, (size_t(kEnergyBlocks) * 5 + 1) * sizeof(double)));
  CUDA_TRY(cudaMemsetAsync(c->partial + size_t(kEnergyBlocks) * 5, 0, sizeof(double), c->stream));
  CUDA_TRY(cudaMalloc(&c->red, 8 * sizeof(double)));

  const FieldIdx& fi = c->fi;
  for (int b = 0; b < nbodies; ++b) {
    const mpm_body_desc& d = bd[b];
    int64_t n = d.count;
    if (n == 0) continue;
    int r;
    if ((r = upload(c, b, d.pos, D, fi.X, ident(D)))) return r;
    if ((r = upload(c, b, d.velocity, D, fi.V, ident(D)))) return r;
    if ((r = upload(c, b, d.mass, 1, fi.M, ident(1)))) return r;
    if ((r = upload(c, b, d.volume, 1, fi.VOL, ident(1)))) return r;
    if ((r = upload(c, b, d.volume_initial, 1, fi.VOL0, ident(1)))) return r;
    if (d.F) {
      if ((r = upload(c, b, d.F, D * D, fi.F, ident(D * D)))) return r;
    } else {
      std::vector<double> I(size_t(n) * D * D, 0.0);
      for (int64_t p = 0; p < n; ++p)
        for (int a = 0; a < D; ++a) I[p * D * D + a * (D + 1)] = 1.0;
      if ((r = upload(c, b, I.data(), D * D, fi.F, ident(D * D)))) return r;
    }
    if (d.strain && (r = upload(c, b, d.strain, D * D, fi.EPS, sym_from_full(D, c->status, ST_ASYM_STRESS))))
      return r;
    if (d.stress && (r = upload(c, b, d.stress, D * D, fi.SIG, sym_from_full(D, c->status, ST_ASYM_STRESS))))
      return r;
    if (d.alpha && (r = upload(c, b, d.alpha, 1, fi.ALPHA, ident(1)))) return r;
    if (d.alphadot && (r = upload(c, b, d.alphadot, 1, fi.ALPHAD, ident(1)))) return r;
    if (d.vmstr && (r = upload(c, b, d.vmstr, 1, fi.VM, ident(1)))) return r;
    if (D == 3 && d.mat.type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
      // damage state in the plastic strain slots; temperatures start at Tr (Material.jl:507)
      if (d.damage_init && (r = upload(c, b, d.damage_init, 1, fi.EP, ident(1)))) return r;
      if (d.damage && (r = upload(c, b, d.damage, 1, fi.EP + 1, ident(1)))) return r;
      std::vector<double> Tr;
      const double* T = d.temperature;
      if (!T) {
        Tr.assign(size_t(n), d.mat.Tr);
        T = Tr.data();
      }
      if ((r = upload(c, b, T, 1, fi.EP + 2, ident(1)))) return r;
    } else if (d.pstrain) {
      if (D == 2) r = upload(c, b, d.pstrain, 3, fi.EP, ident(3));
      else r = upload(c, b, d.pstrain, 9, fi.EP, sym_from_full(3, c->status, ST_ASYM_PSTRAIN));
      if (r) return r;
    }
    if (d.youngs) {
      std::vector<double> lm(size_t(n) * 2);
      double nu = d.mat.nu;
      for (int64_t p = 0; p < n; ++p) {
        double E = d.youngs[p];
        lm[2 * p] = E * nu / (1 + nu) / (1 - 2 * nu);
        lm[2 * p + 1] = E / 2 / (1 + nu);
      }
      if ((r = upload(c, b, lm.data(), 2, fi.LAM, ident(2)))) return r;
    }
  }
  // the uploads compared the mirrored entries of every symmetric input
  unsigned st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (st & ST_ASYM_STRESS) return fail(MPM_ERR_ARG, "mpm_create: strain and stress must be symmetric");
  if (st & ST_ASYM_PSTRAIN) return fail(MPM_ERR_ARG, "mpm_create: pstrain must be symmetric");
  CUDA_TRY(cudaMemset(c->status, 0, sizeof(unsigned)));
  return MPM_OK;
}

}  // namespace

extern "C" {

int mpm_abi_version(void) { return JUMP_MPM_ABI_VERSION; }

const char* mpm_last_error(void) { return g_err.c_str(); }

static bool fused_fits(const mpm_ctx* c, int sort_interval);

int mpm_create(const mpm_grid_desc* grid, const mpm_body_desc* bodies, int32_t nbodies,
               const mpm_params* params, mpm_ctx** out) {
  if (!grid || !params || !out) return fail(MPM_ERR_ARG, "mpm_create: null argument");
  *out = nullptr;
  if (grid->dim != 2 && grid->dim != 3) return fail(MPM_ERR_ARG, "mpm_create: dim must be 2 or 3");
  if (nbodies < 0 || (nbodies > 0 && !bodies)) return fail(MPM_ERR_ARG, "mpm_create: bad body list");
  for (int a = 0; a < grid->dim; ++a) {
    if (grid->nodes[a] < 2) return fail(MPM_ERR_ARG, "mpm_create: a grid axis needs at least 2 nodes");
    if (!(grid->xmax[a] > grid->xmin[a])) return fail(MPM_ERR_ARG, "mpm_create: need xmax > xmin");
    if (grid->nodes[a] > (int64_t(1) << 30)) return fail(MPM_ERR_ARG, "mpm_create: grid axis too large");
  }
  {
    int64_t cells = 1;
    for (int a = 0; a < grid->dim; ++a) cells *= grid->nodes[a] - 1;
    if (params->sort_interval > 0 && int64_t(nbodies) * (cells + 1) >= (int64_t(1) << 32))
      return fail(MPM_ERR_ARG, "mpm_create: too many (body, cell) keys for the particle sort");
  }
  if (params->sort_interval < 0) return fail(MPM_ERR_ARG, "mpm_create: sort_interval < 0");
  if (params->algorithm != MPM_ALG_USL && params->algorithm != MPM_ALG_MUSL)
    return fail(MPM_ERR_ARG, "mpm_create: unknown algorithm");
  if (params->basis != MPM_BASIS_LINEAR && params->basis != MPM_BASIS_QUAD_BSPLINE &&
      params->basis != MPM_BASIS_CUBIC_BSPLINE)
    return fail(MPM_ERR_ARG, "mpm_create: unknown basis");
  for (int a = 0; a < grid->dim; ++a)
    if (params->basis != MPM_BASIS_LINEAR && grid->nodes[a] < basis_nodes(params->basis))
      return fail(MPM_ERR_ARG, "mpm_create: B-spline bases need 3 (quadratic) or 4 (cubic) nodes per axis");
  if (params->algorithm == MPM_ALG_MUSL && (params->precision != MPM_PREC_F64 || params->contact))
    return fail(MPM_ERR_UNSUPPORTED, "mpm_create: MUSL runs FP64 with one velocity field");
  if (!(params->dt > 0.0) || !std::isfinite(params->dt)) return fail(MPM_ERR_ARG, "mpm_create: dt must be > 0");
  if (params->precision != MPM_PREC_F64 && params->precision != MPM_PREC_F32 && params->precision != MPM_PREC_DW)
    return fail(MPM_ERR_ARG, "mpm_create: unknown precision");
  if (params->precision == MPM_PREC_DW) {
    bool ok = grid->dim == 3 && params->algorithm == MPM_ALG_USL && !params->contact;
    for (int b = 0; ok && b < nbodies; ++b) {
      const int t = bodies[b].mat.type;
      ok = t == MPM_MAT_RIGID || t == MPM_MAT_ELASTIC || t == MPM_MAT_J2;
    }
    if (!ok)
      return fail(MPM_ERR_UNSUPPORTED, "mpm_create: MPM_PREC_DW runs 3D USL with one velocity field and linear "
                                       "elastic, J2 or rigid bodies");
  }
  if (params->contact && nbodies > kMaxContactBodies)
    return fail(MPM_ERR_ARG, "mpm_create: contact mode supports at most " + std::to_string(kMaxContactBodies) +
                                 " bodies");
  if (params->contact && !(params->friction >= 0.0)) return fail(MPM_ERR_ARG, "mpm_create: friction < 0");
  const int D = grid->dim;
  int nrigid = 0;
  for (int b = 0; b < nbodies; ++b) {
    const mpm_body_desc& d = bodies[b];
    if (d.count < 0) return fail(MPM_ERR_ARG, "mpm_create: negative particle count");
    if (d.count > 0 && (!d.pos || !d.velocity || !d.mass || !d.volume || !d.volume_initial))
      return fail(MPM_ERR_ARG, "mpm_create: pos, velocity, mass, volume and volume_initial are required");
    if (d.mat.type == MPM_MAT_RIGID) {
      if (params->algorithm != MPM_ALG_USL || params->contact)
        return fail(MPM_ERR_UNSUPPORTED, "mpm_create: rigid solids need USL with one velocity field");
      if (++nrigid > MPM_MAX_RIGID_BODIES)
        return fail(MPM_ERR_ARG, "mpm_create: more than MPM_MAX_RIGID_BODIES rigid solids");
      for (int a = 0; a < D; ++a)
        if (!std::isfinite(d.mat.v_rigid[a])) return fail(MPM_ERR_ARG, "mpm_create: non-finite rigid velocity");
      continue;
    }
    if (!material_ok(d.mat.type, D))
      return fail(MPM_ERR_ARG, "mpm_create: unknown material type (Johnson-Cook, Voce and Johnson-Cook with "
                               "damage are 3D)");
    if (!material_params_ok(d.mat))
      return fail(MPM_ERR_ARG, "mpm_create: Johnson-Cook with damage needs density > 0 and Cp > 0");
  }
  mpm_ctx* c = new mpm_ctx();
  int r = create_impl(grid, bodies, nbodies, params, c);
  if (r != MPM_OK) {
    std::string msg = g_err;
    destroy_ctx(c);
    g_err = msg;
    return r;
  }
  if (fused_fits(c, c->prm.sort_interval)) c->p2g_strategy = MPM_P2G_FUSED;
  *out = c;
  return MPM_OK;
}

// MPM_P2G_FUSED applies to small FP64 problems whose whole step costs less
// than its four launches: linear-basis USL, one velocity field, no rigid
// bodies, no cell sort (sort_interval as given), at most MPM_BATCH_MAX_BODIES
// bodies of one material type (linear elastic, neo-Hookean or J2), at most
// MPM_FUSED_MAX_PARTICLES particles.  mpm_step and mpm_step_energies then run
// their steps in one cooperative launch (fused_steps), whose reset of every
// step is dense.
static bool fused_fits(const mpm_ctx* c, int sort_interval) {
  if (c->f32 || c->dw || c->np == 0 || c->np > MPM_FUSED_MAX_PARTICLES || c->prm.algorithm != MPM_ALG_USL ||
      c->prm.basis != MPM_BASIS_LINEAR || c->prm.contact || sort_interval > 0 || c->nb > MPM_BATCH_MAX_BODIES)
    return false;
  const int t0 = c->mats[0].type;
  for (int b = 0; b < c->nb; ++b) {
    const int t = c->mats[b].type;
    if (c->rigid(b) || t != t0 || (t != MPM_MAT_ELASTIC && t != MPM_MAT_NEOHOOKEAN && t != MPM_MAT_J2)) return false;
  }
  return true;
}

// n steps on the fused path, with the EnergiesFix records of local steps
// first, first + every, ... through c->en_rec when rec; the next per-stage
// step clears every node first
static int fused_run(mpm_ctx* c, int64_t n, bool rec = false, int64_t first = 0, int64_t every = 1) {
  if (n <= 0) return MPM_OK;
  if (!c->fused) CUDA_TRY(cudaMalloc(&c->fused, fused_bytes(c->dim, c->nd.nodeCount)));
  int r = fused_steps(c->dim, c->stream, c->fused, c->g, c->nd, c->P, c->np, c->nb, c->off.data(), c->cnt.data(),
                      c->mats.data(), c->prm.dt, c->prm.tolerance, c->prm.body_force, n, c->status,
                      rec ? c->en_rec : nullptr, first, every, c->hat_c, c->hat_nl);
  c->full_clear = true;
  return r;
}

// after the fused steps' barrier words: MPM_ERR_CUDA if a wait gave up (the
// stream has synchronised)
static int fused_check(mpm_ctx* c) {
  if (!c->fused) return MPM_OK;
  unsigned w[3] = {0, 0, 0};
  CUDA_TRY(cudaMemcpy(w, c->fused, sizeof(w), cudaMemcpyDeviceToHost));
  if (w[2]) return fail(MPM_ERR_CUDA, "a grid barrier of the fused steps gave up after one second");
  return MPM_OK;
}

// after fused steps the block list of the sparse clear is stale: clear
// m, p0 and f of every node before the next step that uses it
static int clear_if_stale(mpm_ctx* c) {
  if (!c->full_clear) return MPM_OK;
  CUDA_TRY(cudaMemsetAsync(c->nodebuf, 0, size_t(c->nd.nodeCount) * (1 + 2 * c->dim) * sizeof(double), c->stream));
  c->full_clear = false;
  return MPM_OK;
}

// enqueue one step: the cell sort when it is due, then the step graph of the
// buffer in use (captured on first use)
static int launch_one_step(mpm_ctx* c, bool en = false) {
  int r;
  if ((r = clear_if_stale(c))) return r;
  if (c->Palt && c->prm.sort_interval > 0 && c->since_sort >= c->prm.sort_interval && (r = enqueue_sort(c)))
    return r;
  if ((r = build_step_graph(c, en))) return r;
  CUDA_TRY(cudaGraphLaunch(en ? c->exec_en[c->cur] : c->exec[c->cur], c->stream));
  ++c->since_sort;
  return MPM_OK;
}

int mpm_step(mpm_ctx* c, int64_t nsteps, double* t_inout) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_step: null context");
  if (nsteps < 0) return fail(MPM_ERR_ARG, "mpm_step: nsteps < 0");
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  CUDA_TRY(cudaEventRecord(c->e0, c->stream));
  if (c->p2g_strategy == MPM_P2G_FUSED) {
    int r;
    if ((r = fused_run(c, nsteps))) return r;
    if (t_inout)
      for (int64_t k = 0; k < nsteps; ++k) *t_inout += c->prm.dt;
  } else {
    for (int64_t k = 0; k < nsteps; ++k) {
      int r;
      if ((r = launch_one_step(c))) return r;
      if (t_inout) *t_inout += c->prm.dt;
    }
  }
  CUDA_TRY(cudaEventRecord(c->e1, c->stream));
  unsigned st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, c->e0, c->e1));
  c->last_ms = ms;
  if (c->p2g_strategy == MPM_P2G_FUSED) {
    int r = fused_check(c);
    if (r) return r;
  }
  return status_to_code(st);
}

int mpm_step_energies(mpm_ctx* c, int64_t nsteps, int64_t every, int64_t first, double* t_inout, double* out) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_step_energies: null context");
  if (nsteps < 0 || every < 1 || first < 0)
    return fail(MPM_ERR_ARG, "mpm_step_energies: nsteps < 0, every < 1 or first < 0");
  const int D = c->dim;
  const int64_t nrec = nsteps > first ? (nsteps - 1 - first) / every + 1 : 0;
  if (nrec > 0 && !out) return fail(MPM_ERR_ARG, "mpm_step_energies: null output");
  if (nrec > c->rec_cap) {
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    CUDA_TRY(cudaFreeHost(c->rec_host));
    CUDA_TRY(cudaFree(c->rec_dev));
    c->rec_host = nullptr;
    c->rec_dev = nullptr;
    c->rec_cap = 0;
    CUDA_TRY(cudaHostAlloc(&c->rec_host, size_t(nrec) * (2 + D) * sizeof(double), cudaHostAllocDefault));
    CUDA_TRY(cudaMalloc(&c->rec_dev, size_t(nrec) * (2 + D) * sizeof(double)));
    c->rec_cap = nrec;
  }
  // a recording step is one graph: the step, then its sums written through
  // the record cursor (set here to the first record slot)
  const bool in_graph = nrec > 0 && c->np > 0;
  if (in_graph) {
    if (!c->en_rec) {
      CUDA_TRY(cudaMalloc(&c->en_rec, sizeof(EnRec)));
      CUDA_TRY(cudaHostAlloc(&c->en_rec_h, sizeof(EnRec), cudaHostAllocDefault));
    }
    c->en_rec_h->base = c->rec_dev;
    c->en_rec_h->idx = 0;
    CUDA_TRY(cudaMemcpyAsync(c->en_rec, c->en_rec_h, sizeof(EnRec), cudaMemcpyHostToDevice, c->stream));
  }
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  CUDA_TRY(cudaEventRecord(c->e0, c->stream));
  int64_t j = 0;
  const bool one = c->p2g_strategy == MPM_P2G_FUSED;
  if (one) {
    // every step and every record of the call in one cooperative launch
    int r;
    if ((r = fused_run(c, nsteps, in_graph, first, every))) return r;
    if (t_inout)
      for (int64_t k = 0; k < nsteps; ++k) *t_inout += c->prm.dt;
  }
  for (int64_t k = 0; k < nsteps && !one; ++k) {
    int r;
    const bool recd = k >= first && (k - first) % every == 0;
    if ((r = launch_one_step(c, in_graph && recd))) return r;
    if (t_inout) *t_inout += c->prm.dt;
    if (recd && !in_graph)  // no particles: zero sums
      CUDA_TRY(cudaMemsetAsync(c->rec_dev + size_t(j) * (2 + D), 0, (2 + D) * sizeof(double), c->stream));
    if (recd) ++j;
  }
  if (nrec > 0)
    CUDA_TRY(cudaMemcpyAsync(c->rec_host, c->rec_dev, size_t(nrec) * (2 + D) * sizeof(double),
                             cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaEventRecord(c->e1, c->stream));
  unsigned st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, c->e0, c->e1));
  c->last_ms = ms;
  if (one) {
    int r = fused_check(c);
    if (r) return r;
  }
  if (nrec > 0) std::memcpy(out, c->rec_host, size_t(nrec) * (2 + D) * sizeof(double));
  return status_to_code(st);
}

int mpm_set_launch(mpm_ctx* c, int32_t p2g_strategy, int32_t threads, int32_t sort_interval) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_set_launch: null context");
  if (p2g_strategy > MPM_P2G_FUSED)
    return fail(MPM_ERR_ARG, "mpm_set_launch: unknown P2G strategy");
  if (threads >= 0 && (threads < 32 || threads > 256 || threads % 32 != 0))
    return fail(MPM_ERR_ARG, "mpm_set_launch: threads must be a multiple of 32 in 32 .. 256");
  const int new_sort = sort_interval >= 0 ? sort_interval : c->prm.sort_interval;
  if (c->dw && p2g_strategy > MPM_P2G_ATOMIC)
    return fail(MPM_ERR_ARG, "mpm_set_launch: MPM_PREC_DW contexts take MPM_P2G_ATOMIC");
  if (p2g_strategy == MPM_P2G_FUSED && !fused_fits(c, new_sort))
    return fail(MPM_ERR_ARG, "mpm_set_launch: MPM_P2G_FUSED needs an FP64 linear-basis USL problem of at most "
                             "MPM_FUSED_MAX_PARTICLES particles, one velocity field, no rigid bodies, no sort and "
                             "one material type (linear elastic, neo-Hookean or J2)");
  if (sort_interval > 0 && !c->Palt) {
    int r = alloc_sort(c);
    if (r != MPM_OK) return r;
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));  // captured graphs may still run
  if (p2g_strategy >= 0) c->p2g_strategy = p2g_strategy;
  // a sort switched on under the default fused strategy: per-stage launches
  if (c->p2g_strategy == MPM_P2G_FUSED && !fused_fits(c, new_sort)) c->p2g_strategy = MPM_P2G_ATOMIC;
  if (threads >= 0) c->threads = threads;
  if (sort_interval >= 0) {
    if (sort_interval > 0 && c->prm.sort_interval != sort_interval) c->since_sort = sort_interval;  // sort next step
    c->prm.sort_interval = sort_interval;
  }
  invalidate_graphs(c);
  return MPM_OK;
}

int mpm_get_launch(mpm_ctx* c, int32_t* p2g_strategy, int32_t* threads, int32_t* sort_interval) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_get_launch: null context");
  if (p2g_strategy) *p2g_strategy = c->p2g_strategy;
  if (threads) *threads = c->threads;
  if (sort_interval) *sort_interval = c->prm.sort_interval;
  return MPM_OK;
}

int mpm_tune(mpm_ctx* c, int64_t probe_steps, int32_t* p2g_strategy, int32_t* threads, int32_t* sort_interval,
             double* ms_per_step, double* all_ms) {
  if (!c || probe_steps < 1) return fail(MPM_ERR_ARG, "mpm_tune: null context or probe_steps < 1");
  if (c->np == 0) return fail(MPM_ERR_ARG, "mpm_tune: no particles");
  // the particle state (and its slot -> particle map) every probe starts from
  const size_t pbytes = size_t(c->NF) * size_t(c->np) * c->esz, obytes = size_t(c->np) * sizeof(int64_t);
  void* snap = nullptr;
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cudaMalloc(&snap, pbytes + obytes));
  struct FreeOnExit {
    void* p;
    ~FreeOnExit() { cudaFree(p); }  // every return path, after the stream's work on it
  } guard{snap};
  char* sp = static_cast<char*>(snap);
  int rc = MPM_OK;
  auto restore = [&]() -> int {
    CUDA_TRY(cudaMemcpyAsync(c->P, sp, pbytes, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->orig, sp + pbytes, obytes, cudaMemcpyDeviceToDevice, c->stream));
    return MPM_OK;
  };
  const int saved_s = c->p2g_strategy, saved_t = c->threads, saved_i = c->prm.sort_interval;
  const int64_t saved_since = c->since_sort;
  if (cudaMemcpyAsync(sp, c->P, pbytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(sp + pbytes, c->orig, obytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
    rc = fail(MPM_ERR_CUDA, "mpm_tune: snapshot copy failed");
  const bool can_sort = rc == MPM_OK && alloc_sort(c) == MPM_OK;
  const int strategies[] = {MPM_P2G_ATOMIC, MPM_P2G_WARP, MPM_P2G_TILE, MPM_P2G_TILE_WARP};
  const int thread_list[] = {64, 128, 256};
  const int sort_list[] = {0, 1, 4, 16};
  double best = 1e300;
  int bs = saved_s, bt = saved_t, bi = saved_i;
  if (all_ms)
    for (int q = 0; q < MPM_TUNE_CANDIDATES; ++q) all_ms[q] = -1.0;
  int idx = -1;
  for (int s : strategies) {
    for (int th : thread_list) {
      for (int si : sort_list) {
        ++idx;
        if (rc != MPM_OK) break;
        if ((si > 0 && !can_sort) || (c->dw && s != MPM_P2G_ATOMIC)) continue;
        c->p2g_strategy = s;
        c->threads = th;
        c->prm.sort_interval = si;
        c->since_sort = si;  // a probe with sorting starts sorted
        invalidate_graphs(c);
        if ((rc = restore())) break;
        if ((rc = launch_one_step(c))) break;  // captures the graphs outside the timed region
        // a whole number of sort intervals, so that each probe pays its share of
        // sorts (the warm-up step above sorted: the window's sorts fall on its
        // steps si, 2 si, ...)
        const int64_t nprobe = si > 0 ? (probe_steps + si - 1) / si * si : probe_steps;
        CUDA_TRY(cudaEventRecord(c->e0, c->stream));
        for (int64_t k = 0; k < nprobe && rc == MPM_OK; ++k) rc = launch_one_step(c);
        CUDA_TRY(cudaEventRecord(c->e1, c->stream));
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc = fail(MPM_ERR_CUDA, std::string("mpm_tune: ") + cudaGetErrorString(e));
        if (rc != MPM_OK) break;
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, c->e0, c->e1));
        const double per = double(ms) / double(nprobe);
        if (all_ms) all_ms[idx] = per;
        if (per < best) {
          best = per;
          bs = s;
          bt = th;
          bi = si;
        }
      }
    }
  }
  // MPM_P2G_FUSED where it fits (candidate 48), from the same saved state
  if (rc == MPM_OK && fused_fits(c, 0)) {
    c->prm.sort_interval = 0;
    if ((rc = restore()) == MPM_OK) rc = fused_run(c, 1);  // allocates its scratch outside the clock
    if (rc == MPM_OK) {
      CUDA_TRY(cudaEventRecord(c->e0, c->stream));
      rc = fused_run(c, probe_steps);
      CUDA_TRY(cudaEventRecord(c->e1, c->stream));
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) rc = fail(MPM_ERR_CUDA, std::string("mpm_tune: ") + cudaGetErrorString(e));
      if (rc == MPM_OK) rc = fused_check(c);
    }
    if (rc == MPM_OK) {
      float ms = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&ms, c->e0, c->e1));
      const double per = double(ms) / double(probe_steps);
      if (all_ms) all_ms[48] = per;
      if (per < best) {
        best = per;
        bs = MPM_P2G_FUSED;
        bt = saved_t;
        bi = 0;
      }
    }
  }
  // the chosen configuration, on the state the call started from
  c->p2g_strategy = rc == MPM_OK ? bs : saved_s;
  c->threads = rc == MPM_OK ? bt : saved_t;
  c->prm.sort_interval = rc == MPM_OK ? bi : saved_i;
  c->since_sort = c->prm.sort_interval > 0 ? c->prm.sort_interval : saved_since;
  invalidate_graphs(c);
  int r2 = restore();
  cudaError_t e = cudaStreamSynchronize(c->stream);
  cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream);
  if (rc != MPM_OK) return rc;
  if (r2 != MPM_OK) return r2;
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_tune: ") + cudaGetErrorString(e));
  if (p2g_strategy) *p2g_strategy = c->p2g_strategy;
  if (threads) *threads = c->threads;
  if (sort_interval) *sort_interval = c->prm.sort_interval;
  if (ms_per_step) *ms_per_step = best;
  return MPM_OK;
}

int mpm_download(mpm_ctx* c, int32_t body, const mpm_body_view* v) {
  if (!c || !v) return fail(MPM_ERR_ARG, "mpm_download: null argument");
  if (body < 0 || body >= c->nb) return fail(MPM_ERR_ARG, "mpm_download: body index out of range");
  const int D = c->dim;
  const FieldIdx& fi = c->fi;
  int r;
  if ((r = download(c, body, v->pos, D, fi.X, ident(D)))) return r;
  if ((r = download(c, body, v->velocity, D, fi.V, ident(D)))) return r;
  if ((r = download(c, body, v->volume, 1, fi.VOL, ident(1)))) return r;
  if ((r = download(c, body, v->F, D * D, fi.F, ident(D * D)))) return r;
  if ((r = download(c, body, v->strain, D * D, fi.EPS, full_from_sym(D)))) return r;
  if ((r = download(c, body, v->stress, D * D, fi.SIG, full_from_sym(D)))) return r;
  if ((r = download(c, body, v->alpha, 1, fi.ALPHA, ident(1)))) return r;
  if ((r = download(c, body, v->alphadot, 1, fi.ALPHAD, ident(1)))) return r;
  if (D == 3 && c->mats[body].type == MPM_MAT_JOHNSON_COOK_DAMAGE) {
    if ((r = download(c, body, v->damage_init, 1, fi.EP, ident(1)))) return r;
    if ((r = download(c, body, v->damage, 1, fi.EP + 1, ident(1)))) return r;
    if ((r = download(c, body, v->temperature, 1, fi.EP + 2, ident(1)))) return r;
  } else {
    if (D == 2) r = download(c, body, v->pstrain, 3, fi.EP, ident(3));
    else r = download(c, body, v->pstrain, 9, fi.EP, full_from_sym(3));
    if (r) return r;
  }
  if (v->vmstr && c->cnt[body] > 0) {
    if (c->mats[body].type == MPM_MAT_J2) {
      // J2 vmStr is a function of the stored stress (Material.jl:223-224, 273-274)
      if (D == 2) Launchers<2>::j2_vm_perm(c->stream, c->part(body), c->f32, c->orig, c->staging);
      else Launchers<3>::j2_vm_perm(c->stream, c->part(body), c->f32, c->orig, c->staging);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(v->vmstr, c->staging, size_t(c->cnt[body]) * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
    } else if ((r = download(c, body, v->vmstr, 1, fi.VM, ident(1)))) {
      return r;
    }
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));  // every copy into the caller's arrays has landed
  return MPM_OK;
}

int mpm_download_grid(mpm_ctx* c, double* mass, double* momentum0, double* momentum, double* force) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_download_grid: null context");
  const int D = c->dim;
  const int64_t Nn = c->g.nodeCount;
  std::vector<double> h(size_t(Nn) * (1 + 2 * D));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (c->prm.contact) {
    // contact mode: the grid holds the system mass sum_b m_b; the single-field
    // momentum and force arrays are not formed (zeros), as in the FEMP solvers
    std::vector<double> mb(static_cast<size_t>(Nn));
    for (int64_t i = 0; i < Nn; ++i) h[i] = 0.0;
    for (int b = 0; b < c->nb; ++b) {
      CUDA_TRY(cudaMemcpy(mb.data(), c->cp.body[b].m, size_t(Nn) * sizeof(double), cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < Nn; ++i) h[i] += mb[i];
    }
    for (int64_t i = 0; i < Nn; ++i) {
      if (mass) mass[i] = h[i];
      for (int a = 0; a < D; ++a) {
        if (momentum0) momentum0[D * i + a] = 0.0;
        if (momentum) momentum[D * i + a] = 0.0;
        if (force) force[D * i + a] = 0.0;
      }
    }
    return MPM_OK;
  }
  CUDA_TRY(cudaMemcpy(h.data(), c->nodebuf, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<uint32_t> rm;
  if (c->rmask) {
    rm.resize(size_t(Nn));
    CUDA_TRY(cudaMemcpy(rm.data(), c->rmask, size_t(Nn) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  }
  const double* m = h.data();
  const double* p0 = m + Nn;
  const double* f = p0 + Nn * D;
  const double dt = c->prm.dt;
  for (int64_t i = 0; i < Nn; ++i) {
    if (mass) mass[i] = m[i];
    double q0[3], q[3];
    for (int a = 0; a < D; ++a) {
      q0[a] = p0[a * Nn + i];
      q[a] = q0[a] + f[a * Nn + i] * dt;  // grid update (:430), then the Dirichlet mask (:433-441)
      if (c->fixed_h[i] & (1u << a)) {
        q0[a] = 0.0;
        q[a] = 0.0;
      }
    }
    // the rigid-body override of the last step (:448-479), in body order
    for (uint32_t bits = rm.empty() ? 0u : rm[size_t(i)]; bits; bits &= bits - 1u) {
      int k = 0;
      while (!((bits >> k) & 1u)) ++k;
      const double* rt = c->rtab_h.data() + 4 * k;
      for (int a = 0; a < D; ++a) {
        if (rt[0] != 0.0) {
          q0[a] = 0.0;
          q[a] = 0.0;
        } else if (rt[1 + a] != 0.0) {
          q0[a] = m[i] * rt[1 + a];
          q[a] = q0[a];
        }
      }
    }
    for (int a = 0; a < D; ++a) {
      if (momentum0) momentum0[D * i + a] = q0[a];
      if (momentum) momentum[D * i + a] = q[a];
      if (force) force[D * i + a] = f[a * Nn + i];
    }
  }
  return MPM_OK;
}

int mpm_energies(mpm_ctx* c, double* ke, double* se, double* momentum) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_energies: null context");
  const int D = c->dim;
  double out[5] = {0, 0, 0, 0, 0};
  if (c->np > 0) {
    if (D == 2) Launchers<2>::energies(c->stream, c->all(), c->f32, c->partial, kEnergyBlocks, c->red);
    else Launchers<3>::energies(c->stream, c->all(), c->f32, c->partial, kEnergyBlocks, c->red);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, c->red, (2 + D) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  if (ke) *ke = out[0];
  if (se) *se = out[1];
  if (momentum)
    for (int a = 0; a < D; ++a) momentum[a] = out[2 + a];
  return MPM_OK;
}

// snapshot layout: 4 x int64 header (magic, dim, precision, particle count),
// the particle SoA in slot order, then orig[slot] (the slot -> particle map)
static const int64_t kMagic = 0x4d504d4a554d5033LL;  // "3": particle records with the JC/Voce rate field

int mpm_save(mpm_ctx* c, void* buf, size_t* nbytes) {
  if (!c || !nbytes) return fail(MPM_ERR_ARG, "mpm_save: null argument");
  size_t body = size_t(c->NF) * size_t(c->np) * c->esz;
  size_t perm = size_t(c->np) * sizeof(int64_t);
  size_t need = 4 * sizeof(int64_t) + body + perm;
  if (!buf) {
    *nbytes = need;
    return MPM_OK;
  }
  if (*nbytes < need) return fail(MPM_ERR_ARG, "mpm_save: buffer too small");
  int64_t hdr[4] = {kMagic, c->dim, c->f32 ? 1 : 0, c->np};
  std::memcpy(buf, hdr, sizeof(hdr));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  char* p = static_cast<char*>(buf) + sizeof(hdr);
  if (body) CUDA_TRY(cudaMemcpy(p, c->P, body, cudaMemcpyDeviceToHost));
  if (perm) CUDA_TRY(cudaMemcpy(p + body, c->orig, perm, cudaMemcpyDeviceToHost));
  *nbytes = need;
  return MPM_OK;
}

int mpm_load(mpm_ctx* c, const void* buf, size_t nbytes) {
  if (!c || !buf) return fail(MPM_ERR_ARG, "mpm_load: null argument");
  size_t body = size_t(c->NF) * size_t(c->np) * c->esz;
  size_t perm = size_t(c->np) * sizeof(int64_t);
  int64_t hdr[4];
  if (nbytes != sizeof(hdr) + body + perm) return fail(MPM_ERR_ARG, "mpm_load: size does not match this context");
  std::memcpy(hdr, buf, sizeof(hdr));
  if (hdr[0] != kMagic || hdr[1] != c->dim || hdr[2] != (c->f32 ? 1 : 0) || hdr[3] != c->np)
    return fail(MPM_ERR_ARG, "mpm_load: snapshot belongs to a different configuration");
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  const char* p = static_cast<const char*>(buf) + sizeof(hdr);
  if (body) CUDA_TRY(cudaMemcpy(c->P, p, body, cudaMemcpyHostToDevice));
  if (perm) CUDA_TRY(cudaMemcpy(c->orig, p + body, perm, cudaMemcpyHostToDevice));
  return MPM_OK;
}

int mpm_last_step_ms(mpm_ctx* c, double* ms) {
  if (!c || !ms) return fail(MPM_ERR_ARG, "mpm_last_step_ms: null argument");
  *ms = c->last_ms;
  return MPM_OK;
}

int mpm_profile_stages(mpm_ctx* c, int64_t nsteps, double* stage_ms) {
  if (!c || !stage_ms || nsteps < 0) return fail(MPM_ERR_ARG, "mpm_profile_stages: bad argument");
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; ++i) CUDA_TRY(cudaEventCreate(&ev[i]));
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  int rc = clear_if_stale(c);
  for (int64_t k = 0; k < nsteps && rc == MPM_OK; ++k) {
    cudaEventRecord(ev[4], c->stream);
    enqueue_step(c, ev);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      rc = fail(MPM_ERR_CUDA, std::string("mpm_profile_stages: ") + cudaGetErrorString(e));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[4], ev[0]);
    stage_ms[MPM_STAGE_RESET] += ms;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    stage_ms[MPM_STAGE_P2G] += ms;
    cudaEventElapsedTime(&ms, ev[1], ev[2]);
    stage_ms[MPM_STAGE_GRID] += ms;
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    stage_ms[MPM_STAGE_G2P] += ms;
  }
  for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  if (rc != MPM_OK) return rc;
  unsigned st = 0;
  CUDA_TRY(cudaMemcpy(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return status_to_code(st);
}

int mpm_fwd_checkpointed(mpm_ctx* c, int64_t nsteps, int32_t every) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_fwd_checkpointed: null context");
  if (nsteps < 1 || every < 1) return fail(MPM_ERR_ARG, "mpm_fwd_checkpointed: need nsteps >= 1, every >= 1");
  if (c->f32 || c->dw || c->prm.contact || c->prm.sort_interval > 0 || c->prm.algorithm != MPM_ALG_USL ||
      c->prm.basis != MPM_BASIS_LINEAR)
    return fail(MPM_ERR_UNSUPPORTED, "mpm_fwd_checkpointed: reverse mode needs USL with the linear basis, FP64 "
                                     "particles and arithmetic, one velocity field and no sorting");
  for (const MatParams& m : c->mats)
    if (m.type != MPM_MAT_NEOHOOKEAN && m.type != MPM_MAT_ELASTIC && m.type != MPM_MAT_J2)
      return fail(MPM_ERR_UNSUPPORTED, "mpm_fwd_checkpointed: reverse mode is built for neo-Hookean, linear "
                                       "elastic and J2 bodies");
  const size_t bytes = size_t(c->NF) * size_t(c->np > 0 ? c->np : 1) * c->esz;
  const int64_t slots = (nsteps + every - 1) / every + 1;  // steps 0, every, ... and the final state
  if (slots != c->ckpt_slots) {
    cudaFree(c->ckpt);
    c->ckpt = nullptr;
    c->ckpt_slots = 0;
    CUDA_TRY(cudaMalloc(&c->ckpt, bytes * size_t(slots)));
    c->ckpt_slots = slots;
  }
  // every == 1: every state is kept anyway, so each step's node buffer is kept
  // too and the reverse sweep recomputes nothing
  const int64_t Nn = c->nd.nodeCount;
  const size_t recbytes = size_t(Nn) * (1 + 4 * c->dim) * sizeof(double);
  if (every == 1) {
    if (c->fullrec_steps != nsteps) {
      cudaFree(c->fullrec);
      c->fullrec = nullptr;
      c->fullrec_steps = 0;
      CUDA_TRY(cudaMalloc(&c->fullrec, recbytes * size_t(nsteps)));
      c->fullrec_steps = nsteps;
    }
  } else if (c->fullrec) {
    cudaFree(c->fullrec);
    c->fullrec = nullptr;
    c->fullrec_steps = 0;
  }
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  CUDA_TRY(cudaMemcpyAsync(c->ckpt, c->P, bytes, cudaMemcpyDeviceToDevice, c->stream));
  int r;
  if ((r = clear_if_stale(c))) return r;
  if ((r = build_step_graph(c))) return r;
  for (int64_t k = 1; k <= nsteps; ++k) {
    CUDA_TRY(cudaGraphLaunch(c->exec[c->cur], c->stream));
    if (every == 1)
      CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(c->fullrec) + recbytes * size_t(k - 1), c->nodebuf, recbytes,
                               cudaMemcpyDeviceToDevice, c->stream));
    if (k % every == 0 && k < nsteps)
      CUDA_TRY(cudaMemcpyAsync(c->ckpt + bytes * size_t(k / every), c->P, bytes, cudaMemcpyDeviceToDevice,
                               c->stream));
  }
  CUDA_TRY(cudaMemcpyAsync(c->ckpt + bytes * size_t(slots - 1), c->P, bytes, cudaMemcpyDeviceToDevice, c->stream));
  unsigned st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->adj_nsteps = nsteps;
  c->adj_every = every;
  return status_to_code(st);
}

int mpm_bwd(mpm_ctx* c, const double* x_bar, const double* v_bar, double* E_bar, double* v0_bar, double* x0_bar) {
  if (!c) return fail(MPM_ERR_ARG, "mpm_bwd: null context");
  if (c->adj_nsteps < 1) return fail(MPM_ERR_ARG, "mpm_bwd: run mpm_fwd_checkpointed first");
  const int D = c->dim;
  const int every = c->adj_every;
  const int64_t nsteps = c->adj_nsteps;
  const int64_t Nn = c->nd.nodeCount;
  const size_t bytes = size_t(c->NF) * size_t(c->np > 0 ? c->np : 1) * c->esz;
  const int ANF = D == 2 ? AdjLayout<2>::NF : AdjLayout<3>::NF;
  const int XB = 0, VB = D, EB = 2 * D + D * D;
  // two segment buffers: the reverse sweep reads one while the next segment is
  // recomputed into the other
  if (c->segbuf_slots < every) {
    drop_seg_graphs(c);  // captured segments point into the old buffers
    cudaFree(c->segbuf);
    cudaFree(c->gridrec);
    c->segbuf = nullptr;
    c->gridrec = nullptr;
    c->segbuf_slots = 0;
    CUDA_TRY(cudaMalloc(&c->segbuf, bytes * size_t(2 * every)));
    CUDA_TRY(cudaMalloc(&c->gridrec, size_t(Nn) * (1 + 4 * D) * sizeof(double) * size_t(2 * every)));
    c->segbuf_slots = every;
  }
  if (!c->stream2) {
    CUDA_TRY(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      CUDA_TRY(cudaEventCreateWithFlags(&c->ev_rec[i], cudaEventDisableTiming));
      CUDA_TRY(cudaEventCreateWithFlags(&c->ev_adj[i], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaEventCreateWithFlags(&c->ev_sync, cudaEventDisableTiming));
  }
  if (!c->adjbuf) {
    CUDA_TRY(cudaMalloc(&c->adjbuf, size_t(ANF) * size_t(c->np > 0 ? c->np : 1) * sizeof(double)));
    CUDA_TRY(cudaMalloc(&c->nodeadj, size_t(Nn) * (1 + 4 * D) * sizeof(double)));
  }
  CUDA_TRY(cudaMemsetAsync(c->adjbuf, 0, size_t(ANF) * size_t(c->np > 0 ? c->np : 1) * sizeof(double), c->stream));
  // adjoints at the final step, per body AoS -> component-major SoA
  auto adj_part = [&](int b) { return PartP{c->adjbuf, c->np, c->off[b], c->cnt[b]}; };
  int64_t base = 0;
  for (int b = 0; b < c->nb; ++b) {
    const size_t n = size_t(c->cnt[b]) * D;
    for (int which = 0; which < 2; ++which) {
      const double* src = which == 0 ? x_bar : v_bar;
      if (!src || n == 0) continue;
      CUDA_TRY(cudaMemcpyAsync(c->staging, src + base * D, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      if (D == 2) Launchers<2>::aos_to_soa(c->stream, adj_part(b), false, c->staging, D, which == 0 ? XB : VB, ident(D));
      else Launchers<3>::aos_to_soa(c->stream, adj_part(b), false, c->staging, D, which == 0 ? XB : VB, ident(D));
      CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    base += c->cnt[b];
  }
  const AdjP ad{c->adjbuf, c->np};
  NodeAdjP na;
  na.nodeCount = Nn;
  na.vdtb = c->nodeadj;
  na.dvb = c->nodeadj + Nn * D;
  na.mb = c->nodeadj + Nn * 2 * D;
  na.p0b = c->nodeadj + Nn * (1 + 2 * D);
  na.fb = c->nodeadj + Nn * (1 + 3 * D);
  const int64_t nseg = c->ckpt_slots - 1;
  void* Pwork = c->P;
  // a tile P2G strategy selects the G2P adjoint's tiled scatter too
  const bool adj_tile = c->p2g_strategy == MPM_P2G_TILE || c->p2g_strategy == MPM_P2G_TILE_WARP;
  CUDA_TRY(cudaMemsetAsync(c->nodeadj, 0, size_t(Nn) * 2 * D * sizeof(double), c->stream));
  // Segment buffer X (0, 1) holds `every` particle states and node records.
  // Recompute: `len` steps from the state in P, recording each step's particle
  // state and grid outputs in buffer X.  Reverse: the adjoint of those steps,
  // last first, from buffer X.
  const size_t recd = size_t(Nn) * (1 + 4 * D);
  auto seg_state = [&](int X, int j) { return c->segbuf + bytes * size_t(X * every + j); };
  auto seg_rec = [&](int X, int j) { return c->gridrec + recd * size_t(X * every + j); };
  auto enqueue_recompute = [&](int X, int len) {
    for (int j = 0; j < len; ++j) {
      cudaMemcpyAsync(seg_state(X, j), Pwork, bytes, cudaMemcpyDeviceToDevice, c->stream);
      enqueue_step(c, nullptr, seg_rec(X, j));
    }
  };
  // One reversed step from a particle state and its node record, on the
  // context's stream.  A single body with the per-particle scatter runs it as
  // one cooperative launch (reverse_step_kernel), else three kernels.  The
  // node adjoints vdt_bar, dv_bar are zero on entry: set once below, then
  // zeroed by the grid adjoint as it consumes them.
  bool coop = c->nb == 1 && !adj_tile && !c->coop_off &&
              (D == 2 ? Launchers<2>::reverse_step_fits(c->cnt[0], c->mats[0].type)
                      : Launchers<3>::reverse_step_fits(c->cnt[0], c->mats[0].type));
  if (coop) {
    if (!c->revbar) CUDA_TRY(cudaMalloc(&c->revbar, 4 * sizeof(unsigned)));
    CUDA_TRY(cudaMemsetAsync(c->revbar, 0, 4 * sizeof(unsigned), c->stream));
  }
  auto reverse_one = [&](const GridRec& gr, void* state) {
    if (coop) {
      const double nu = c->nus[0];
      RevStepP r{};
      r.gp = c->g;
      r.gr = gr;
      r.pp = PartP{state, c->np, c->off[0], c->cnt[0]};
      r.ad = ad;
      r.na = na;
      r.mp = c->mats[0];
      r.c1 = nu / (1 + nu) / (1 - 2 * nu);  // dlambda/dE
      r.c2 = 1.0 / 2.0 / (1 + nu);          // dmu/dE
      r.dt = c->prm.dt;
      r.tol = c->prm.tolerance;
      for (int a = 0; a < 3; ++a) r.grav[a] = (a < D) ? c->prm.body_force[a] : 0.0;
      r.fixed = c->fixed;
      r.bar = c->revbar;
      r.err = c->revbar + 2;
      if (D == 2) Launchers<2>::reverse_step(c->stream, r);
      else Launchers<3>::reverse_step(c->stream, r);
      return;
    }
    for (int b = 0; b < c->nb; ++b) {
      const PartP ps{state, c->np, c->off[b], c->cnt[b]};
      const double nu = c->nus[b];
      const double c1 = nu / (1 + nu) / (1 - 2 * nu), c2 = 1.0 / 2.0 / (1 + nu);  // dlambda/dE, dmu/dE
      if (D == 2) Launchers<2>::g2p_adj(c->stream, c->g, gr, ps, ad, na, c->mats[b], c1, c2, adj_tile);
      else Launchers<3>::g2p_adj(c->stream, c->g, gr, ps, ad, na, c->mats[b], c1, c2, adj_tile);
    }
    if (D == 2) Launchers<2>::grid_adj(c->stream, gr, na, c->fixed, c->prm.dt, c->prm.tolerance);
    else Launchers<3>::grid_adj(c->stream, gr, na, c->fixed, c->prm.dt, c->prm.tolerance);
    for (int b = 0; b < c->nb; ++b) {
      const PartP ps{state, c->np, c->off[b], c->cnt[b]};
      const double nu = c->nus[b];
      const double c1 = nu / (1 + nu) / (1 - 2 * nu), c2 = 1.0 / 2.0 / (1 + nu);
      if (D == 2) Launchers<2>::p2g_adj(c->stream, c->g, ps, ad, na, c->mats[b], c1, c2, c->prm.body_force);
      else Launchers<3>::p2g_adj(c->stream, c->g, ps, ad, na, c->mats[b], c1, c2, c->prm.body_force);
    }
  };
  auto enqueue_reverse = [&](int X, int len) {
    for (int j = len - 1; j >= 0; --j) {
      const double* rec = seg_rec(X, j);
      reverse_one(GridRec{rec, rec + Nn * (1 + 2 * D), rec + Nn * (1 + 3 * D)}, seg_state(X, j));
    }
  };
  // captured once per (kind, buffer, segment length: full or the shorter last one),
  // on the context's stream; launched on either stream
  auto segment_exec = [&](int kind, int X, int len, cudaGraphExec_t* out) -> int {
    for (int l = 0; l < 2; ++l)
      if (c->seg_exec[kind][X][l] && c->seg_len[kind][X][l] == len) {
        *out = c->seg_exec[kind][X][l];
        return MPM_OK;
      }
    const int l = c->seg_exec[kind][X][0] ? 1 : 0;
    if (c->seg_exec[kind][X][l]) {
      cudaGraphExecDestroy(c->seg_exec[kind][X][l]);
      cudaGraphDestroy(c->seg_graph[kind][X][l]);
      c->seg_exec[kind][X][l] = nullptr;
      c->seg_graph[kind][X][l] = nullptr;
    }
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    if (kind == 0) enqueue_recompute(X, len);
    else enqueue_reverse(X, len);
    cudaError_t le = cudaGetLastError();
    cudaError_t ee = cudaStreamEndCapture(c->stream, &c->seg_graph[kind][X][l]);
    if (kind == 1 && coop && (le != cudaSuccess || ee != cudaSuccess)) {
      // the cooperative launch was not captured: three kernels per step from now on
      if (c->seg_graph[kind][X][l]) cudaGraphDestroy(c->seg_graph[kind][X][l]);
      c->seg_graph[kind][X][l] = nullptr;
      cudaGetLastError();
      coop = false;
      c->coop_off = true;
      CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_reverse(X, len);
      le = cudaGetLastError();
      ee = cudaStreamEndCapture(c->stream, &c->seg_graph[kind][X][l]);
    }
    if (le != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_bwd launch: ") + cudaGetErrorString(le));
    if (ee != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("mpm_bwd capture: ") + cudaGetErrorString(ee));
    CUDA_TRY(cudaGraphInstantiate(&c->seg_exec[kind][X][l], c->seg_graph[kind][X][l], 0));
    c->seg_len[kind][X][l] = len;
    *out = c->seg_exec[kind][X][l];
    return MPM_OK;
  };
  if (every == 1 && c->fullrec) {
    // every state and node buffer of the forward run is stored: the reverse
    // sweep is three kernels per step
    const size_t recd = size_t(Nn) * (1 + 4 * D);
    for (int64_t k = nsteps; k >= 1; --k) {
      const double* rec = c->fullrec + recd * size_t(k - 1);
      reverse_one(GridRec{rec, rec + Nn * (1 + 2 * D), rec + Nn * (1 + 3 * D)},
                  reinterpret_cast<char*>(c->ckpt) + bytes * size_t(k - 1));
    }
  }
  if (!(every == 1 && c->fullrec) && nseg > 0) {
    // Checkpointed: segment seg - 1 is recomputed on the context's stream while
    // the reverse sweep of segment seg runs on the second stream, in the other
    // segment buffer.  A small problem (the 16,384-particle cantilever fills 5%
    // of the warp slots) leaves most SMs idle in either pass, so the two
    // overlap.  Stream order: recompute X -> ev_rec[X] -> reverse X ->
    // ev_adj[X] -> the next recompute into X.
    auto seg_len_of = [&](int64_t seg) { return int(std::min<int64_t>(every, nsteps - seg * every)); };
    CUDA_TRY(cudaEventRecord(c->ev_sync, c->stream));  // adjoint inputs are set
    CUDA_TRY(cudaStreamWaitEvent(c->stream2, c->ev_sync, 0));
    bool used[2] = {false, false};
    auto recompute = [&](int64_t seg, int X) -> int {
      if (used[X]) CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_adj[X], 0));
      CUDA_TRY(cudaMemcpyAsync(Pwork, c->ckpt + bytes * size_t(seg), bytes, cudaMemcpyDeviceToDevice, c->stream));
      cudaGraphExec_t ex = nullptr;
      int r = segment_exec(0, X, seg_len_of(seg), &ex);
      if (r) return r;
      CUDA_TRY(cudaGraphLaunch(ex, c->stream));
      CUDA_TRY(cudaEventRecord(c->ev_rec[X], c->stream));
      used[X] = true;
      return MPM_OK;
    };
    int X = 0, r;
    if ((r = recompute(nseg - 1, X))) return r;
    for (int64_t seg = nseg - 1; seg >= 0; --seg) {
      if (seg > 0 && (r = recompute(seg - 1, 1 - X))) return r;
      cudaGraphExec_t ex = nullptr;
      if ((r = segment_exec(1, X, seg_len_of(seg), &ex))) return r;
      CUDA_TRY(cudaStreamWaitEvent(c->stream2, c->ev_rec[X], 0));
      CUDA_TRY(cudaGraphLaunch(ex, c->stream2));
      CUDA_TRY(cudaEventRecord(c->ev_adj[X], c->stream2));
      X = 1 - X;
    }
    CUDA_TRY(cudaEventRecord(c->ev_sync, c->stream2));  // the context's stream waits for the sweep
    CUDA_TRY(cudaStreamWaitEvent(c->stream, c->ev_sync, 0));
  }
  CUDA_TRY(cudaGetLastError());
  if (coop) {
    unsigned err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, c->revbar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) return fail(MPM_ERR_CUDA, "mpm_bwd: a grid barrier of the fused reverse step gave up after one second");
  }
  // gradients in original particle order (no sorting in reverse mode)
  base = 0;
  for (int b = 0; b < c->nb; ++b) {
    const int64_t n = c->cnt[b];
    struct Out {
      double* dst;
      int per, f0;
    } outs[3] = {{E_bar ? E_bar + base : nullptr, 1, EB},
                 {v0_bar ? v0_bar + base * D : nullptr, D, VB},
                 {x0_bar ? x0_bar + base * D : nullptr, D, XB}};
    for (const Out& o : outs) {
      if (!o.dst || n == 0) continue;
      if (D == 2) Launchers<2>::soa_to_aos(c->stream, adj_part(b), false, c->staging, o.per, o.f0, ident(o.per));
      else Launchers<3>::soa_to_aos(c->stream, adj_part(b), false, c->staging, o.per, o.f0, ident(o.per));
      CUDA_TRY(cudaMemcpyAsync(o.dst, c->staging, size_t(n) * o.per * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
      CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    base += n;
  }
  // leave the context at the final state of the forward run
  CUDA_TRY(cudaMemcpyAsync(c->P, c->ckpt + bytes * size_t(c->ckpt_slots - 1), bytes, cudaMemcpyDeviceToDevice,
                           c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int mpm_destroy(mpm_ctx* c) {
  if (c) {
    cudaStreamSynchronize(c->stream);
    destroy_ctx(c);
  }
  return MPM_OK;
}

}  // extern "C"
