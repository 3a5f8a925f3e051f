/*
 * jump_mpm.h -- C ABI of the GB300 explicit-MPM step (USL, linear hat basis).
 *
 * This is the drop-in boundary for jump's explicit solid-mechanics solvers:
 *
 *   solve_explicit_dynamics_2D(grid::Grid2D, solids::Vector{Solid2D}, basis::LinearBasis,
 *                              alg::USL, output, fixes, data)
 *       SolveExplicitSolidMechanics2D.jl:335-585
 *   solve_explicit_dynamics_3D(grid::Grid3D, solids::Vector{Solid3D}, basis::LinearBasis,
 *                              alg::USL, output, fixes, data)
 *       SolveExplicitSolidMechanics3D.jl:230-378
 *
 * A host binding (Julia ccall, Python ctypes) builds one context from the
 * Grid/Solid/Material arrays, advances it some steps, downloads the particle
 * state before each output/fix hook and at the end, then destroys it.
 * Every array crossing this boundary is plain host memory owned by the
 * caller; the library never retains a caller pointer after a call returns.
 *
 * Layouts follow Julia's memory layout of the reference types, so a Julia
 * binding can pass `reinterpret`ed arrays without copies:
 *   - Vector{SVector{d,Float64}}      -> d doubles per particle/node, AoS
 *   - Vector{SMatrix{d,d,Float64}}    -> d*d doubles per particle, column-major
 *   - grid.fixedNodes::Array{Int64,2} -> (d, nodeCount), column-major
 * Node and particle indices in this ABI are 0-based; node I (1-based in the
 * reference, Grid.jl:151,259) is element I-1 here.
 *
 * Every function returns an int status: MPM_OK (0) or one of MPM_ERR_*.
 * mpm_last_error() returns a message for the last failing call of the
 * calling thread.  A context may be used from one host thread at a time.
 */
#ifndef JUMP_MPM_H
#define JUMP_MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JUMP_MPM_ABI_VERSION 10

/* status codes */
#define MPM_OK               0
#define MPM_ERR_ARG          1  /* invalid argument or descriptor */
#define MPM_ERR_CUDA         2  /* a CUDA runtime call failed */
#define MPM_ERR_NEGATIVE_J   3  /* det F <= 0 at some particle (state still advanced) */
#define MPM_ERR_NONFINITE    4  /* NaN/Inf in a particle's velocity, position or stress */
#define MPM_ERR_OUT_OF_GRID  5  /* a particle's cell lies outside the grid; it was frozen */
/* 6 is not used: no kernel of this library waits on another, so no wait can time out */
#define MPM_ERR_UNSUPPORTED  7  /* feature not available in this build */
#define MPM_ERR_SOLVER       8  /* the 2D MUSL mass solve did not converge in its iteration cap */

/* material models (Material.jl) */
#define MPM_MAT_ELASTIC     0   /* ElasticMaterial, Material.jl:37-81 */
#define MPM_MAT_NEOHOOKEAN  1   /* NeoHookeanMaterial, Material.jl:100-122 */
#define MPM_MAT_J2          2   /* ElastoPlasticMaterial, Material.jl:128-275 */
#define MPM_MAT_JOHNSON_COOK 3  /* JohnsonCookMaterial, Material.jl:279-330, 386-443 (3D) */
#define MPM_MAT_VOCE        4   /* VoceMaterial, Material.jl:336-383, 445-493 (3D) */
#define MPM_MAT_JOHNSON_COOK_DAMAGE 5  /* JohnsonCookMaterialWithDamage, Material.jl:495-646 (3D) */
/* Rigid body (RigidMaterial, Material.jl:29-31, with the fields the USL solver
   reads from it, SolveExplicitSolidMechanics2D.jl:448-479, 539-551: vx, vy and
   fixed; vz in 3D).  Its particles add nothing in P2G.  After the grid update
   and its Dirichlet conditions, every node of a rigid particle's linear-basis
   cell gets nodal momentum and old momentum m_I v_rigid in each component
   where v_rigid is non-zero (m_I: the deformable bodies' nodal mass), or zero
   in every component when `fixed`; rigid bodies later in the body list
   override earlier ones at shared nodes.  After G2P the rigid particles move
   by dt v_rigid; their other fields are never updated.  USL with one velocity
   field only (MUSL, contact, batches and the reverse mode reject it); at most
   MPM_MAX_RIGID_BODIES per context. */
#define MPM_MAT_RIGID       6
#define MPM_MAX_RIGID_BODIES 32

/* particle precision (grid accumulation is always FP64) */
#define MPM_PREC_F64        0   /* every particle field and every operation in FP64 */
#define MPM_PREC_F32        1   /* FP32 particle fields and arithmetic; FP64 nodes, det F, energies */
/* FP64 particle fields and FP64 node accumulators; the arithmetic of the P2G
   and the G2P with its constitutive update (linear elastic, J2) in
   double-word FP32: each value a pair of floats hi + lo, about 48 significant
   bits (2^-49 relative per rounding against FP64's 2^-53), from error-free
   transforms on the FP32 pipe, which issues 64 times as many operations per
   clock as the FP64 pipe on GB300.  Every accumulated particle field is its
   FP64 value plus the step's increment rounded to FP64, and the hat (cell and
   weights) is the FP64 one, so the results follow the FP64 step to within the
   FP64 step's own rounding differences.  3D USL (linear, quadratic or cubic
   B-spline basis) with one velocity field and the P2G strategy MPM_P2G_ATOMIC;
   other configurations: MPM_ERR_UNSUPPORTED (MPM_ERR_ARG for another
   strategy).  The reverse mode
   and MPM_P2G_FUSED take FP64 contexts only. */
#define MPM_PREC_DW         2

/* Shape functions (the `basis` argument of solve_explicit_dynamics_2D/3D) */
#define MPM_BASIS_LINEAR        0  /* LinearBasis: hat functions, 2^dim nodes (Basis.jl:219-251, 292-332) */
#define MPM_BASIS_QUAD_BSPLINE  1  /* QuadBsplineBasis: modified quadratic B-splines, 3^dim nodes
                                      (Basis.jl:374-592, Bsplines.jl:18-80); grids of >= 3 nodes per axis */
#define MPM_BASIS_CUBIC_BSPLINE 2  /* CubicBsplineBasis: modified cubic B-splines, 4^dim nodes
                                      (Basis.jl:594-820, Bsplines.jl:86-172); grids of >= 4 nodes per axis */

/* Update scheme (the `alg` argument of solve_explicit_dynamics_2D/3D) */
#define MPM_ALG_USL         0   /* USL(tolerance), SolveExplicitSolidMechanics2D.jl:335-585 */
#define MPM_ALG_MUSL        1   /* MUSL(alpha): 2D SolveExplicitSolidMechanics2D.jl:24-329 (blended
                                   consistent mass), 3D SolveExplicitSolidMechanics3D.jl:14-223
                                   (lumped mass); FP64, one velocity field */

typedef struct mpm_grid_desc {
  int32_t dim;                 /* 2 (Grid2D) or 3 (Grid3D) */
  int32_t reserved;
  double  xmin[3];             /* Grid2D(xmin,xmax,ymin,ymax,nx,ny), Grid.jl:104 */
  double  xmax[3];             /* Grid3D(xmin,xmax,ymin,ymax,zmin,zmax,nx,ny,nz), Grid.jl:198 */
  int64_t nodes[3];            /* iN_x, iN_y(, iN_z): nodes per axis, >= 2 */
  const int64_t* fixed_nodes;  /* grid.fixedNodes (dim x nodeCount, column-major), or NULL */
} mpm_grid_desc;

typedef struct mpm_material_desc {
  int32_t type;                /* MPM_MAT_* */
  int32_t reserved;
  double  E, nu, density;      /* constructor arguments */
  double  fy, k1;              /* J2 yield stress and linear hardening modulus */
  /* Johnson-Cook: yield (A + B ep^n)(1 + epdot/epsdot0)^C (C != 0) or A + B ep^n;
     Voce: A - B exp(-C ep) (n, epsdot0 unused); both: plastic strain rate filter
     time 1000 cellsize / sqrt((lambda + 2 mu)/density) */
  double  A, B, C, n, epsdot0, cellsize;
  /* Johnson-Cook with damage only: thermal softening exponent m, Taylor-Quinney
     coefficient chi and specific heat Cp of the strength part (temperature rise
     chi/(density Cp) x flow stress x plastic strain increment; Cp > 0), and the
     damage part JohnsonCookDamage(d1..d5, epsdot0, Tr, Tm): failure strain
     (d1 + d2 exp(d3 triaxiality))(1 + d4 ln(epdot/depsdot0))(1 + d5 (T - Tr)/(Tm - Tr)) */
  double  m, chi, Cp;
  double  d1, d2, d3, d4, d5, depsdot0, Tr, Tm;
  /* MPM_MAT_RIGID only: the body's prescribed velocity (vx, vy, vz; vz unused
     in 2D) and `fixed` (non-zero: every nodal momentum component under the
     body is zeroed instead) */
  double  v_rigid[3];
  int32_t fixed;
  int32_t reserved2;
} mpm_material_desc;

/* Particle arrays of one Solid2D/Solid3D (Solid.jl:67-125, 267-297), read at create time. */
typedef struct mpm_body_desc {
  int64_t count;                    /* parCount */
  mpm_material_desc mat;
  const double* pos;                /* dim   per particle */
  const double* velocity;           /* dim   per particle */
  const double* mass;               /* 1 */
  const double* volume;             /* 1 */
  const double* volume_initial;     /* 1 */
  const double* F;                  /* dim*dim, column-major */
  const double* strain;             /* dim*dim */
  const double* stress;             /* dim*dim */
  const double* alpha;              /* J2: equivalent plastic strain, or NULL (zeros) */
  const double* pstrain;            /* J2: 3 (2D Voigt) or 9 (3D) per particle, or NULL */
  const double* youngs;             /* optional per-particle Young's modulus, or NULL */
  const double* alphadot;           /* Johnson-Cook/Voce: plastic strain rate, or NULL (zeros) */
  const double* damage_init;        /* Johnson-Cook with damage: damage_init, or NULL (zeros) */
  const double* damage;             /*   dam, or NULL (zeros) */
  const double* temperature;        /*   damage_part.temp, or NULL (Tr) */
  const double* vmstr;              /* the material's vmStr, or NULL (zeros): state for Johnson-Cook with
                                       damage, whose failed particles keep it; recomputed by the others */
} mpm_body_desc;

/* Writable views for mpm_download; any pointer may be NULL to skip that field. */
typedef struct mpm_body_view {
  double* pos;
  double* velocity;
  double* volume;
  double* F;
  double* strain;
  double* stress;
  double* alpha;
  double* pstrain;
  double* vmstr;                    /* von Mises stress written by Elastic-3D and J2 updates */
  double* alphadot;                 /* Johnson-Cook/Voce plastic strain rate, or NULL */
  double* damage_init;              /* Johnson-Cook with damage state, or NULL */
  double* damage;
  double* temperature;
} mpm_body_view;

typedef struct mpm_params {
  double  dt;                  /* data["dt"] */
  double  tolerance;           /* USL.tolerance: nodal mass cutoff in G2P, Algorithm.jl:16-18 */
  double  body_force[3];       /* ConstantBodyForce2D/3D.g, BodyForce.jl:56-62,85-91 */
  int32_t precision;           /* MPM_PREC_F64, MPM_PREC_F32 or MPM_PREC_DW */
  int32_t contact;             /* 0: one velocity field (the reference USL); 1: one field per body
                                  with the multi-body contact correction */
  double  friction;            /* Coulomb coefficient for contact (2D only; 0 = frictionless) */
  int32_t sort_interval;       /* re-sort particles by cell every N steps (0 = never) */
  int32_t flags;               /* reserved, 0 */
  int32_t algorithm;           /* MPM_ALG_USL or MPM_ALG_MUSL */
  int32_t basis;               /* MPM_BASIS_LINEAR, _QUAD_BSPLINE or _CUBIC_BSPLINE */
  double  alpha;               /* MUSL.alpha: FLIP/PIC blend, Algorithm.jl:38-40 (MUSL only) */
} mpm_params;

typedef struct mpm_ctx mpm_ctx;

/* Library identity. */
int         mpm_abi_version(void);
const char* mpm_last_error(void);

/* Build a context: copies grid + particle arrays to device memory. */
int mpm_create(const mpm_grid_desc* grid, const mpm_body_desc* bodies, int32_t nbodies,
               const mpm_params* params, mpm_ctx** out);

/* Advance nsteps USL steps (the body of the `while t < Tf` loop,
   SolveExplicitSolidMechanics2D.jl:381-534).  If t_inout is not NULL,
   *t_inout += dt once per step, in FP64, exactly like `t += dtime` (:580). */
int mpm_step(mpm_ctx* ctx, int64_t nsteps, double* t_inout);

/* nsteps steps as mpm_step, with the EnergiesFix sums (Fix.jl:248-270;
   mpm_energies) taken after local steps first, first + every, first + 2 every,
   ... < nsteps -- the hook schedule `counter % interval == 0` of
   SolveExplicitSolidMechanics2D.jl:574-578 when first = (-counter0) mod every.
   Record r goes to out[(2 + dim) r ...]: kinetic energy, strain energy, momentum
   (dim).  Each record is formed on the device in its own slot, with no host
   synchronisation between steps (under MPM_P2G_FUSED every step and record of
   the call in one launch), and all of them are copied to the host in one
   transfer after the last step; the call returns then, like mpm_step.  out may be any host memory
   ((nsteps - 1 - first)/every + 1 records when nsteps > first). */
int mpm_step_energies(mpm_ctx* ctx, int64_t nsteps, int64_t every, int64_t first, double* t_inout, double* out);

/* Copy one body's particle state back into caller-owned host arrays
   (original particle order, the layouts of mpm_body_desc). */
int mpm_download(mpm_ctx* ctx, int32_t body, const mpm_body_view* out);

/* Grid state after the last step: grid.mass, grid.momentum0, grid.momentum
   and grid.force (the reference's arrays after its grid update, :429-442).
   Each pointer may be NULL; sizes nodeCount and dim*nodeCount. */
int mpm_download_grid(mpm_ctx* ctx, double* mass, double* momentum0, double* momentum,
                      double* force);

/* EnergiesFix quantities (Fix.jl:248-270) reduced on the device in FP64:
   KE = sum 1/2 m v.v, SE = sum 1/2 V sigma:eps, and total momentum (dim). */
int mpm_energies(mpm_ctx* ctx, double* ke, double* se, double* momentum);

/* Snapshot / restore of the full particle state (checkpoint/resume).  With
   buf == NULL, mpm_save stores the byte size it needs in *nbytes. */
int mpm_save(mpm_ctx* ctx, void* buf, size_t* nbytes);
int mpm_load(mpm_ctx* ctx, const void* buf, size_t nbytes);

/* Device time of the kernels of the last mpm_step call, in milliseconds,
   measured with CUDA events on the context's stream. */
int mpm_last_step_ms(mpm_ctx* ctx, double* ms);

/* Measurement aid (no counterpart in the reference): run nsteps steps as
   individual launches with CUDA events between the stages and add each
   stage's device time, in milliseconds, to stage_ms[MPM_STAGE_*]. */
#define MPM_STAGE_RESET 0
#define MPM_STAGE_P2G   1
#define MPM_STAGE_GRID  2
#define MPM_STAGE_G2P   3
#define MPM_NUM_STAGES  4
int mpm_profile_stages(mpm_ctx* ctx, int64_t nsteps, double* stage_ms);

/* Launch configuration and its autotuner (no counterpart in the reference).
   P2G strategy of the linear basis: every particle issues its own FP64 atomics
   (MPM_P2G_ATOMIC, the FP64 default), or lanes of a warp that share a base
   node (the group __match_any_sync finds) first add their values with a
   shuffle reduction and one lane per group issues them (MPM_P2G_WARP, the
   FP32 default); MPM_P2G_TILE and
   MPM_P2G_TILE_WARP stage those two forms in a shared-memory tile of the node
   box a CTA's particles cover and issue one FP64 atomic per node value and CTA
   (a CTA whose box exceeds the tile, 256 nodes for CTAs of 64 threads, else
   512, falls back to per-particle atomics).  threads: CTA size of
   the P2G and G2P launches (32 .. 256, a multiple of 32; default 256, halved
   down to 64 while the largest body would fill fewer than two CTAs per SM).  sort_interval: the
   counting sort by cell every that many steps (0: never); its second particle
   buffer is allocated on first use.  A negative argument keeps that setting.
   MPM_P2G_FUSED runs every stage of every step of an mpm_step call in one
   cooperative launch, the stages separated by grid barriers (each wait
   bounded at about one second, after which the call returns MPM_ERR_CUDA),
   with a dense reset of all nodes each step; it is for small problems, where a
   step's four launches cost more than its work, and the default where it
   applies: FP64, linear basis, USL, one velocity field, no rigid bodies, no
   sort, at most MPM_BATCH_MAX_BODIES bodies of one type (linear elastic,
   neo-Hookean or J2), at most MPM_FUSED_MAX_PARTICLES particles (elsewhere
   MPM_ERR_ARG).
   Results differ between settings only by the summation order of node sums. */
#define MPM_P2G_ATOMIC 0
#define MPM_P2G_WARP   1
#define MPM_P2G_TILE   2
#define MPM_P2G_TILE_WARP 3
#define MPM_P2G_FUSED 4
#define MPM_FUSED_MAX_PARTICLES 2048
int mpm_set_launch(mpm_ctx* ctx, int32_t p2g_strategy, int32_t threads, int32_t sort_interval);
int mpm_get_launch(mpm_ctx* ctx, int32_t* p2g_strategy, int32_t* threads, int32_t* sort_interval);
/* Times probe_steps steps (rounded up to whole sort intervals, so that every
   probe pays its share of sorts) of every combination of P2G strategy
   {atomic, warp, tile, tile_warp} (and MPM_P2G_FUSED where it applies),
   threads {64, 128, 256} and sort interval {0, 1, 4, 16}, each from the same saved
   particle state, keeps the fastest (reported through the non-NULL pointers,
   with its ms per step) and puts the particle state back: the simulation does
   not advance.  Uses a temporary device copy of the particle state.  If
   all_ms is not NULL it receives the ms per step of all MPM_TUNE_CANDIDATES
   combinations, index (strategy * 3 + threads index) * 4 + sort index (a
   negative value: not probed), and at index 48 that of MPM_P2G_FUSED
   where it applies.  The reverse mode needs sort_interval 0. */
#define MPM_TUNE_CANDIDATES 49
int mpm_tune(mpm_ctx* ctx, int64_t probe_steps, int32_t* p2g_strategy, int32_t* threads, int32_t* sort_interval,
             double* ms_per_step, double* all_ms);

int mpm_destroy(mpm_ctx* ctx);

/* Measurement aid (no counterpart in the reference): throughput of FP64 fused
   multiply-adds, FP64 divisions and FP64 atomic additions (executed in L2, at
   distinct coalesced addresses) on the current device, per second; the FP64
   roofline of the step kernels.  Only the rates whose output pointer is not
   NULL are measured. */
int mpm_probe_rates(double* fp64_fma_per_s, double* fp64_div_per_s, double* fp64_atomics_per_s);

/* Test aid (no counterpart in the reference): the double-word operation op of
   the MPM_PREC_DW arithmetic on n operand triples (a[i], b[i], c[i]), each
   first converted FP64 -> double-word; out[2i] and out[2i + 1] receive the
   result's float parts (hi, lo) as doubles (MPM_DW_OP_TO_F64: the double-word
   sum a[i] + b[i] rounded to FP64 by an FP64 add of its exact parts, and 0).  MPM_DW_OP_MUL_FLOAT
   multiplies by the high part of b[i]; MPM_DW_OP_FMA is a[i] b[i] + c[i]. */
#define MPM_DW_OP_FROM_F64  0
#define MPM_DW_OP_ADD       1
#define MPM_DW_OP_SUB       2
#define MPM_DW_OP_MUL       3
#define MPM_DW_OP_MUL_FLOAT 4
#define MPM_DW_OP_FMA       5
#define MPM_DW_OP_SQR       6
#define MPM_DW_OP_SQRT      7
#define MPM_DW_OP_RECIP     8
#define MPM_DW_OP_ONE_MINUS 9
#define MPM_DW_OP_TO_F64    10
int mpm_probe_dw(int32_t op, int64_t n, const double* a, const double* b, const double* c, double* out);

/* ---------------------------------------------------------------------------
 * Reverse mode (no counterpart in the reference): gradients of a loss on the
 * final particle state with respect to the initial velocities and positions
 * and to a per-particle Young's modulus, through hand-written adjoint
 * kernels of every stage.  Built for FP64 contexts with one velocity field,
 * no sorting and neo-Hookean, linear elastic or J2 bodies; otherwise
 * MPM_ERR_UNSUPPORTED.  The backward pass recomputes one checkpoint segment
 * on the context's stream while it differentiates the next on a second one.
 * The derivative is that of the discrete map inside the particles' current
 * cells (the hat basis has kinks at nodes and cell faces).
 * ------------------------------------------------------------------------- */
/* Advance nsteps steps keeping a snapshot of the particle state every
   `checkpoint_every` steps (and the final state) in device memory.  With
   checkpoint_every = 1 every step's state and node buffer are kept
   (nsteps x (state + node buffer) bytes of device memory) and mpm_bwd
   recomputes nothing. */
int mpm_fwd_checkpointed(mpm_ctx* ctx, int64_t nsteps, int32_t checkpoint_every);
/* Reverse sweep over the last mpm_fwd_checkpointed run: each segment is
   recomputed from its snapshot, then differentiated step by step.
     x_bar, v_bar  dL/dx and dL/dv at the final step (v_bar may be NULL),
                   all bodies in order, dim doubles per particle
     E_bar         out: dL/dE per particle (count doubles), or NULL
     v0_bar, x0_bar out: dL/dv, dL/dx at the initial step, or NULL
   The G2P adjoint scatters its node adjoints with FP64 atomics per particle
   at L2, or, when the context's P2G strategy is MPM_P2G_TILE or
   MPM_P2G_TILE_WARP, through a shared-memory tile of each CTA's node box.
   A single-body context with the per-particle scatter runs each reversed step
   as one cooperative launch whose grid barriers wait at most about one second
   each; a wait that gives up makes the call return MPM_ERR_CUDA.
   The context is left at the final state of the forward run. */
int mpm_bwd(mpm_ctx* ctx, const double* x_bar, const double* v_bar, double* E_bar, double* v0_bar,
            double* x0_bar);

/* ---------------------------------------------------------------------------
 * Batched ensembles (no counterpart in the reference, which solves one
 * problem per call): many independent problems -- each what one
 * solve_explicit_dynamics_2D/3D call would take -- advance together.  All
 * problems share the dimension and the precision; sorting is not available.
 * Two execution strategies:
 *   MPM_BATCH_PERSISTENT  one persistent launch for all problems and all
 *                         steps; each CTA takes problems from a work queue
 *                         (largest first) and runs all steps of a problem.
 *                         Needs one material model type for every body and
 *                         no contact: the fit for many small problems.
 *   MPM_BATCH_WIDE        one launch per stage for all problems (clear, P2G,
 *                         block compaction, grid update, G2P) through
 *                         per-problem and per-body offset tables, the step
 *                         captured in a CUDA graph: the fit for problems too
 *                         large for one CTA, problems mixing material models,
 *                         and contact (one node field per body).
 * mpm_batch_create picks PERSISTENT where it is allowed; mpm_batch_tune
 * times both where both are allowed and keeps the faster.
 * ------------------------------------------------------------------------- */
#define MPM_BATCH_MAX_BODIES 4
#define MPM_BATCH_PERSISTENT 0
#define MPM_BATCH_WIDE 1

typedef struct mpm_instance_desc {
  mpm_grid_desc grid;
  const mpm_body_desc* bodies;  /* 1 .. MPM_BATCH_MAX_BODIES */
  int32_t nbodies;
  int32_t contact;              /* 1: one velocity field per body + contact correction */
  double dt;
  double tolerance;
  double body_force[3];
  double friction;              /* contact: Coulomb coefficient (0: frictionless, 2D only above 0) */
} mpm_instance_desc;

typedef struct mpm_batch mpm_batch;

int mpm_batch_create(const mpm_instance_desc* instances, int32_t ninstances, int32_t precision,
                     mpm_batch** out);
/* every problem advances nsteps steps (one launch) */
int mpm_batch_step(mpm_batch* batch, int64_t nsteps);
/* per problem MPM_OK or MPM_ERR_* of the last mpm_batch_step */
int mpm_batch_status(mpm_batch* batch, int32_t* status);
int mpm_batch_download(mpm_batch* batch, int32_t instance, int32_t body, const mpm_body_view* out);
/* EnergiesFix sums per problem: out[i*(2+dim) + {0: KE, 1: SE, 2..: momentum}] */
int mpm_batch_energies(mpm_batch* batch, double* out);
/* launch shape: threads per CTA (multiple of 32, <= 1024) and CTAs per SM */
int mpm_batch_set_launch(mpm_batch* batch, int32_t threads, int32_t ctas_per_sm);
/* Autotuner: times probe_steps steps of every launch shape that fits (on a
   scratch copy of the particles, the batch state is not advanced), keeps the
   fastest and returns it and its device time per step. */
int mpm_batch_tune(mpm_batch* batch, int64_t probe_steps, int32_t* threads, int32_t* ctas_per_sm,
                   double* ms_per_step);
/* Forward-mode derivative (no counterpart in the reference).  Advances every
   problem nsteps steps exactly as mpm_batch_step (WIDE strategy) while
   carrying, for each problem, the derivative of its state with respect to
   one scalar s of that problem: a change of the Young's modulus of its
   bodies, dE[i * MPM_BATCH_MAX_BODIES + k] = dE_k/ds for body k of problem
   i (0 for bodies that do not depend on s; NULL: all 0).  Derivatives start
   at zero at the call.  On return x_dot (or NULL) holds dx/ds of every
   particle, problems and bodies in order, dim doubles per particle.  FP64
   batches with elastic and neo-Hookean bodies and frictionless contact;
   otherwise MPM_ERR_UNSUPPORTED.  The derivative is that of the discrete
   map within the current cells and contact branches. */
int mpm_batch_jvp(mpm_batch* batch, int64_t nsteps, const double* dE, double* x_dot);
/* MPM_BATCH_PERSISTENT or MPM_BATCH_WIDE (MPM_ERR_ARG where not allowed) */
int mpm_batch_set_strategy(mpm_batch* batch, int32_t strategy);
int mpm_batch_strategy(mpm_batch* batch, int32_t* strategy);
/* device time of the last mpm_batch_step, milliseconds */
int mpm_batch_last_ms(mpm_batch* batch, double* ms);
int mpm_batch_destroy(mpm_batch* batch);

/* No counterpart in the reference.  EnergiesFix sums (as mpm_energies) for
   callers that cannot call cudaMalloc where they need them -- e.g. inside a
   CUDA stream capture, where allocation is not permitted, or in a host
   program whose device memory belongs to another allocator -- and that hold
   the particle arrays in their own device memory.  It allocates nothing: its
   scratch (one partial sum per 1024 particles) is a fixed static device array
   that every GPU loading this library keeps until the process exits.
     count     particles, 0 .. MPM_STATIC_MAX_PARTICLES (larger: MPM_ERR_ARG)
     mass, volume          device arrays of count doubles
     velocity              device, dim*count doubles, component-major (v_a at a*count)
     stress, strain        device, symmetric components, component-major:
                           2D (xx, yy, xy), 3D (xx, yy, zz, xy, yz, xz)
     out       device, 2+dim doubles: KE, SE, momentum
     stream    a cudaStream_t of this process, or NULL for the default stream
   The work is enqueued on `stream` and the call returns without waiting.
   The scratch array's device address belongs to a CUDA context: the first
   call in each context (the device's primary context, a context the caller
   made current, or the primary context re-created after cudaDeviceReset)
   looks it up (cudaGetSymbolAddress) with that context current and caches it
   under the context's unique id, so make the first call in a context before
   any stream capture in it.  Calls share the one scratch array of their
   context: calls that overlap on the GPU (other streams, other threads) race
   and must be serialised by the caller. */
#define MPM_STATIC_MAX_PARTICLES 4194304
int mpm_energies_static(int32_t dim, int64_t count, const double* mass, const double* velocity,
                        const double* volume, const double* stress, const double* strain, double* out,
                        void* stream);

#ifdef __cplusplus
}
#endif
#endif /* JUMP_MPM_H */
