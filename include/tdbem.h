/*
 * tdbem.h -- C ABI of tdbem-gb300, the GB300 (sm_103a) implementation of the
 * TD-BEM time-domain elastodynamic boundary-element hot path:
 *
 *   (a) assembly of the G^k / H^k influence-matrix levels (collocation node x
 *       element x time level quadrature of the time-integrated Stokes kernel
 *       with linear temporal shape functions, Duffy-transformed singular
 *       elements, Kelvin-traction regularisation), and
 *   (b) time marching: the history convolution sum_k (G^k t^{n-k} - H^k u^{n-k})
 *       followed by the H^0 solve, with the reference's weighted collocation
 *       (alpha_1, alpha_2).
 *
 * Plain pointers and sizes only.  Every call returns a status (0 = OK, < 0 =
 * error kind below); tdbem_last_error() gives the message of the last failure
 * on the calling thread.  A context is bound to one CUDA device and one
 * stream; calls on one context must not overlap (the host API is not
 * re-entrant per context), different contexts may be used from different
 * threads.  There is no CPU fallback: without a usable CUDA device
 * tdbem_ctx_create fails with TDBEM_ERR_CUDA.
 *
 * Index conventions follow the reference: node ids and dof ids are 0-based,
 * dof = 3*node + direction, matrices are row-major with row = collocation dof
 * and column = field dof (ElastoDynamicsT.cpp:235-259).
 */
#ifndef TDBEM_H
#define TDBEM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
#define TDBEM_OK 0
#define TDBEM_ERR_ARG (-1)         /* invalid argument (size, index, range)   */
#define TDBEM_ERR_CUDA (-2)        /* CUDA runtime failure / no device        */
#define TDBEM_ERR_NOMEM (-3)       /* device or host allocation failed         */
#define TDBEM_ERR_SINGULAR (-4)    /* zero pivot in the H^0 factorisation      */
#define TDBEM_ERR_UNSUPPORTED (-5) /* valid input this build does not support  */
#define TDBEM_ERR_STATE (-6)       /* call out of order (e.g. march before assembly) */

/* ---- precision of the assembled levels and of the marching ---------- */
#define TDBEM_FP64 0  /* the reference's method in FP64 (plain form)         */
#define TDBEM_MIXED 1 /* FP32 far field / FP32 levels, FP64 near field + solve */

typedef struct tdbem_ctx tdbem_ctx;

/* Surface mesh; arrays are copied at tdbem_ctx_create.
 * Replaces ModelManagerT::GetNND/GetNEL/GetElementType/GetIEN/GetCoords
 * (ModelManagerT.h:46-68). */
typedef struct {
    int nnd;              /* number of nodes                                  */
    int nel;              /* number of elements                               */
    int etype;            /* 1 = 4-node bilinear quad, 2 = 8-node serendipity */
    const double* coords; /* nnd x 3                                          */
    const int* ien;       /* nel x 4 (etype 1) or nel x 8 (etype 2), 0-based  */
} tdbem_mesh;

/* Replaces ModelManagerT::GetMaterialConstants (ModelManagerT.h:92). */
typedef struct {
    double E;   /* Young's modulus  */
    double nu;  /* Poisson's ratio  */
    double rho; /* density          */
} tdbem_material;

/* Message of the last failed call on this thread ("" if none). */
const char* tdbem_last_error(void);

/* Library version string. */
const char* tdbem_version(void);

/* Create a context on the current CUDA device: copies the mesh, computes
 * MaxStep exactly as SolverT::ComputeMaxStep (SolverT.cpp:211-250), colours
 * the elements for deterministic assembly.  nq = Gauss points per direction
 * (6, 10, 20 or 40; ShapeFunctionT.cpp:71-169); if_ext != 0 adds the exterior
 * free term 0.5*dt at the first step (ElastoDynamicsT.cpp:212-225).
 * Replaces the constructors of ModelManagerT / ElastoDynamicsT / SolverT
 * (main.cpp:43-57). */
int tdbem_ctx_create(const tdbem_mesh* mesh, const tdbem_material* mat, double dt, int nq,
                     int if_ext, tdbem_ctx** out);
int tdbem_ctx_destroy(tdbem_ctx* ctx);

/* MaxStep M (SolverT::GetMaxStep, SolverT.cpp:252-255); levels are 0..M. */
int tdbem_max_step(const tdbem_ctx* ctx, int* M);
/* Number of dofs D = 3*nnd. */
int tdbem_num_dof(const tdbem_ctx* ctx, int* D);
/* The CUDA stream (cudaStream_t) all work of this context is ordered on. */
int tdbem_get_stream(const tdbem_ctx* ctx, void** stream);

/* ---- (a) assembly --------------------------------------------------- */

/* One call of ElastoDynamicsT::G_H_Driver(t = step*dt, t_1 = dt) followed by
 * GetGHLinear (ElastoDynamicsT.cpp:108-231, 283-289) for collocation rows
 * node_lo..node_hi (inclusive; the reference's SetLowerUpper range).
 * G_I/G_J/H_I/H_J are host buffers of (3*(node_hi-node_lo+1)) x D doubles:
 * the I part (fG_1/fH_1) and J part (fG_2/fH_2) of the step response at that
 * time, C term and exterior free term included at step 1.  FP64. */
int tdbem_gh_driver(tdbem_ctx* ctx, int step, int node_lo, int node_hi, double* G_I,
                    double* G_J, double* H_I, double* H_J);

/* Allocation-free variant of tdbem_gh_driver for callers that cannot allocate
 * device memory (applications that reserve all device memory at start-up and
 * forbid later cudaMalloc/cudaFree, or latency-critical loops that cannot take
 * their implicit synchronisation).  No counterpart in the reference.  Same
 * result as tdbem_gh_driver, written into caller-owned DEVICE buffers
 * (3*(node_hi-node_lo+1) x D doubles each, zeroed by the call), with work
 * ordered on `stream` (a cudaStream_t; NULL = the context's stream); the call
 * never waits for the device.  Its kernels' scratch is one fixed 8 MiB array in
 * device memory that every GPU loading the library holds until exit; meshes whose
 * largest element colour exceeds 262144 elements are rejected
 * (TDBEM_ERR_UNSUPPORTED).  All calls share that array: calls that overlap on the
 * GPU race, so serialise them.  The array's device address is looked up on every
 * call made outside a stream capture, with the context's device current (it must
 * be); the first call on a device must come before any stream capture.  Calls no
 * cudaMalloc, cudaFree or allocating library routine. */
int tdbem_gh_driver_noalloc(const tdbem_ctx* ctx, int step, int node_lo, int node_hi,
                            double* d_G_I, double* d_G_J, double* d_H_I, double* d_H_J,
                            void* stream);

/* Element interface: TDElementStepLinearT::FormGH_Regular (singular[i] = -1) or
 * FormGH_Singular(singular[i]) followed by GetGHLinear (TDElementT.h:16-115,
 * TDElementStepLinearT.cpp:28-626, TDElementT.cpp:148-157) for n independent
 * (collocation point, element) pairs, evaluated together in one launch on the
 * current device.  etype 1 (4 nodes) or 2 (8 nodes), nq Gauss points per direction,
 * material (E, nu, rho) and t_1 (TDElementT::SetTime's second argument, the time
 * step) are shared by the batch; per pair: colloc[i] (3 doubles, SetCollocation),
 * coords[i] (ennd x 3 doubles, SetCoords), t[i] (SetTime's t) and singular[i] (the
 * element's local node at the collocation point, or -1).  Outputs (host buffers):
 * GE_1, GE_2, HE_1, HE_2 of n x 3 x 3*ennd doubles ([i][3a + j] of each pair's
 * block, the reference's fGE_1 ... layout) and C_1, C_2 of n x 9 doubles (the
 * Kelvin term at t[i] == t_1, zeros otherwise).  FP64, with exact zeros where both
 * wave fronts have passed a quadrature point at both evaluation times. */
int tdbem_element_gh(int etype, int nq, double E, double nu, double rho, double t_1, int n,
                     const double* colloc, const double* coords, const double* t,
                     const int* singular, double* GE_1, double* GE_2, double* HE_1,
                     double* HE_2, double* C_1, double* C_2);

/* Assemble the device-resident level store G^k, H^k for k = 0..M: the result
 * of main()'s steps 1..min(M, nsteps) of G_H_Driver + UpdateGHLinear
 * (main.cpp:89-121, SolverStepLinearT.cpp:58-97): level 0 = J(dt), level k =
 * I(k dt) + J((k+1) dt), level M = I(M dt).  precision: TDBEM_FP64 or
 * TDBEM_MIXED. */
int tdbem_assemble_levels(tdbem_ctx* ctx, int nsteps, int precision);

/* Copy level k of G (which = 0) or H (which = 1) to host (D x D doubles).
 * FP32 levels are widened to double. */
int tdbem_get_level(tdbem_ctx* ctx, int k, int which, double* host_out);

/* ---- (b) marching --------------------------------------------------- */

/* Boundary conditions (ModelManagerT::SetBCs, ModelManagerT.cpp:337-354):
 * prescribed displacement values on ubc dofs, traction values on fbc dofs. */
int tdbem_set_bc(tdbem_ctx* ctx, const int* ubc_dofs, const double* ubc_vals, int n_u,
                 const int* fbc_dofs, const double* fbc_vals, int n_f);

/* Weighted-collocation weights (alpha.txt, main.cpp:78-81); range checked as
 * SolverStepLinearT::Solve_Averaging (SolverStepLinearT.cpp:317-322). */
int tdbem_set_alpha(tdbem_ctx* ctx, double a1, double a2);

/* Load amplitude per step: amp[s] multiplies the traction values at step s
 * (time s*dt).  Without a call the reference's Heaviside amp = 1 is used
 * (SolverT::LoadTimeVariation, SolverT.cpp:379-394).  nsteps values. */
int tdbem_set_load_history(tdbem_ctx* ctx, const double* amp, int nsteps);

/* March numstep steps of main()'s loop (SetLoad + Solve(a1,a2),
 * SolverT.cpp:344-377, SolverStepLinearT.cpp:314-544) on the assembled
 * levels.  u_hist / t_hist: host buffers of (numstep+1) x D doubles receiving
 * fDis_DB / fTrac_DB[0..numstep] (entry numstep stays 0 as in the reference),
 * or NULL to keep the histories on the device only. */
int tdbem_march(tdbem_ctx* ctx, int numstep, double* u_hist, double* t_hist);

/* ---- stepwise form of main()'s loop (the C++ host classes use these) ---- */

/* SolverStepLinearT::UpdateGHLinear (SolverStepLinearT.cpp:58-175) for host row
 * blocks of one step, rows 3*node_lo .. 3*node_hi+2 of D columns, row-major:
 * G_I / H_I (ElastoDynamicsT's fG_1 / fH_1, the I part) go to level `step`,
 * G_J / H_J (fG_2 / fH_2, the J part) to level step-1 (inserted at step 1,
 * added after).  Steps beyond MaxStep are ignored, as in the reference.  Builds
 * the FP64 level store that tdbem_march and tdbem_march_step read. */
int tdbem_update_gh_linear(tdbem_ctx* ctx, int step, int node_lo, int node_hi, const double* G_I,
                           const double* G_J, const double* H_I, const double* H_J);

/* Stepwise marching on FP64 levels.  tdbem_march_begin allocates and zeroes the
 * histories of numstep steps (SolverT::Initialize, SolverT::SetTimeControl);
 * tdbem_march_step runs SetLoad + Solve(a1, a2) of main()'s step curr_step
 * (1..numstep; step 1 does nothing, step n >= 2 solves history n-1 as
 * Solve_Averaging, SolverStepLinearT.cpp:314-544) on the levels present and
 * copies history curr_step-1 to u / t (D doubles each, or NULL), the vectors
 * RecordResult prints (SolverStepLinearT.cpp:549-603). */
int tdbem_march_begin(tdbem_ctx* ctx, int numstep);
int tdbem_march_step(tdbem_ctx* ctx, int curr_step, double* u, double* t);

/* ---- many meshes at once --------------------------------------------- */

/* Assemble the levels of n contexts (different meshes) together.  TDBEM_FP64:
 * one pair window, scan and quadrature launch per colour index for all meshes and
 * one C-term launch for all nodes, instead of a sequence per mesh; TDBEM_MIXED:
 * each mesh's near/far assembly from its own host thread on its own stream, the
 * meshes overlapping on the GPU.  Levels hold steps 1..min(MaxStep, nsteps[i]) of
 * context i, as tdbem_assemble_levels(ctx, nsteps[i], precision) gives them.
 * The reference assembles one mesh per run. */
int tdbem_assemble_group(tdbem_ctx* const* ctxs, int n, const int* nsteps, int precision);

/* March n contexts (each with its own boundary conditions, weights and load
 * history; all FP64 or all TDBEM_MIXED levels) for numsteps[i] steps each in ONE
 * persistent cooperative launch: every step of every mesh in grid-wide phases
 * (history vectors, convolution, solve + update; mixed: FP32 levels and inverse
 * with one FP64 refinement sweep when tdbem_set_march_options asks for one).  The
 * launch shape (lanes per row, threads per block, blocks per SM) is picked the
 * first time a group size is seen by timing the candidates on the first steps.
 * u_hist[i] / t_hist[i]: host buffers of (numsteps[i]+1) x D_i doubles, or NULL
 * (arrays or entries). */
int tdbem_march_group(tdbem_ctx* const* ctxs, int n, const int* numsteps, double* const* u_hist,
                      double* const* t_hist);

/* The launch shape the last grouped march used. */
int tdbem_group_shape(int* lanes, int* block, int* blocks_per_sm);

/* Batched marching of nrhs load cases on this context's mesh, boundary
 * conditions, weights and (TDBEM_MIXED) levels: tdbem_march run for every case
 * at once.  Case c's known traction at step s is amp[c*numstep + s] *
 * traction[c*D + d] at every dof d that is not a prescribed-displacement dof
 * (amp NULL: 1 at every step).  Replaces running SolverStepLinearT::
 * Solve_Averaging (SolverStepLinearT.cpp:314-544) once per load case with
 * SolverT::SetLoad (SolverT.cpp:344-377) per case; the reference has no batched
 * form.  Each step's convolution of all cases is one tensor-core GEMM (split
 * BF16 products, FP32 accumulation, compensated sum over levels); the solve
 * applies the FP32 inverse with tdbem_set_batch_options' refinement sweeps
 * (residual in FP32 double-word arithmetic against the FP64 LHS).
 * u_hist / t_hist: host buffers of (numstep+1) x nrhs x D doubles,
 * [step][case][dof], or NULL. */
int tdbem_march_batch(tdbem_ctx* ctx, int numstep, int nrhs, const double* traction,
                      const double* amp, double* u_hist, double* t_hist);

/* Options of tdbem_march_batch.  engine: TDBEM_ENGINE_TCGEN05 (default;
 * tcgen05.mma with TMEM accumulators over the merged levels of the mixed march
 * (BF16 hi/lo planes, half the size of the FP32 levels, shared with tdbem_march)
 * and, per case, its known tractions times every level in FP32) or
 * TDBEM_ENGINE_MMA_SYNC (warp-level mma.sync on G and H, splitting the FP32 levels
 * on the fly, no extra memory).  refine_sweeps (0..4, default 0): refinement sweeps
 * of the batched solve; the split-BF16 convolution, not the FP32 inverse, sets the
 * batched form's error, so the default skips them. */
#define TDBEM_ENGINE_TCGEN05 0
#define TDBEM_ENGINE_MMA_SYNC 1
int tdbem_set_batch_options(tdbem_ctx* ctx, int engine, int refine_sweeps);

/* tdbem_march replays its per-step loop (every kernel of every step) as a CUDA
 * graph, captured on the context's stream the first time and again whenever the
 * step count, block size, refinement, weights, load history or buffers change
 * (on by default; off with on = 0, and off while profiling is on). */
int tdbem_set_graphs(tdbem_ctx* ctx, int on);

/* Engine of the TDBEM_MIXED march's history convolution: TDBEM_ENGINE_TCGEN05
 * (default; per level one merged matrix, each column the unknown's column of G or -H,
 * as BF16 hi/lo planes, with the prescribed values' part from three vectors per level;
 * three BF16 tensor-core products per FP32 product, FP32 accumulation and compensated
 * sums across levels: HBM-bound, history error ~1e-5 of FP64) or TDBEM_ENGINE_FP32
 * (G and H with FP32 products on the CUDA cores: error ~2e-7 of FP64, slower).  The
 * tcgen05 engine keeps the merged planes beside the FP32 levels: half their size. */
#define TDBEM_ENGINE_FP32 2
int tdbem_set_march_engine(tdbem_ctx* ctx, int engine);

/* Options of the TDBEM_MIXED marching: block_steps = time steps per block of the
 * history convolution (1, 4, 6, 8, 12 or 16, and 24 or 32 with the tcgen05 engine;
 * 0 = each engine's default, the fastest on GB300 for the 4614-DOF sphere: 32 with
 * tcgen05, 8 with FP32), refine_sweeps = FP64 residual-refinement sweeps per solve
 * (0..4; default 0: on the 4614-DOF sphere the FP32 inverse alone is within
 * 2.4e-7 of FP64, below the tcgen05 engine's convolution error of ~1e-5; the
 * sweeps are for LHS matrices whose FP32 inverse is less accurate). */
int tdbem_set_march_options(tdbem_ctx* ctx, int block_steps, int refine_sweeps);

/* Limit of each pipeline wait (an mbarrier wait for a TMA copy, an MMA or the
 * epilogue) in the tcgen05 convolution kernel, in seconds of the GPU's global
 * timer (0 = the default, 2 s; at most 60).  A wait that runs out makes the kernel
 * stop its producer, MMA and epilogue roles, wait (2 s at most) for its copies and
 * MMAs in flight, free its tensor memory and return; the march then fails with
 * TDBEM_ERR_CUDA naming the wait, and the context stays usable.  The reference has
 * no device code; this bounds the wait a GPU kernel of this library may spend on a
 * pipeline stage. */
int tdbem_set_pipeline_wait(tdbem_ctx* ctx, double seconds);

/* The FP32 inverses of the TDBEM_MIXED march's LHS (the step-2 LHS and the later
 * one): probe[v] = max |A (X v) - v| / max |v| of inverse X of A (v a fixed vector)
 * and full_search[v] = 1 when the pivot search of the panels left their diagonal
 * blocks (a zero pivot there or a probe above 1e-5 made the inversion start again
 * with the full partial-pivoting search).  *step2_sweeps (may be NULL) > 0 when the
 * step-2 LHS, which serves a single solve, gets no inverse of its own: that solve
 * then runs this many Richardson sweeps x <- x + X (b - A x) with the later LHS's
 * inverse X against its FP64 LHS A (chosen when they reach 1e-7 on a probe problem;
 * entry 0 of probe / full_search then repeats entry 1). */
int tdbem_inverse_report(const tdbem_ctx* ctx, double probe[2], int full_search[2],
                         int* step2_sweeps);

/* The H^0 inverse alone, on the current device: X = A^-1 for a row-major n x n
 * host matrix A (blocked Gauss-Jordan with partial pivoting; precision TDBEM_FP64,
 * or TDBEM_MIXED for the FP32 inverse the mixed march uses, widened to double in
 * X), with the FP32 inverse's probe residual and pivot-search fallback (probe 0 and
 * full_search 1 for FP64).  Replaces the factorisation inside KSPSolve
 * (SolverStepLinearT.cpp:503-504) for callers that solve with the inverse; a zero
 * pivot gives TDBEM_ERR_SINGULAR. */
int tdbem_invert(int n, const double* A, int precision, double* X, double* probe,
                 int* full_search);

/* Device memory the library keeps for reuse.  Buffers a destroyed context releases
 * stay allocated, keyed by device and size (at most half of the device's memory),
 * and the next allocation of the same size takes them: creating a context for a mesh
 * of the same size again allocates and frees nothing.  An allocation that fails
 * releases the device's kept buffers and tries again.  device -1: all devices.
 * tdbem_cached_memory reports the kept bytes; tdbem_release_cached_memory frees
 * them (*released, may be NULL: the bytes freed). */
int tdbem_cached_memory(int device, size_t* bytes);
int tdbem_release_cached_memory(int device, size_t* released);

/* Device pointers of the histories of the last tdbem_march (FP64,
 * (numstep+1) x D each); valid until the next march or destroy. */
int tdbem_history_device(const tdbem_ctx* ctx, const double** u_hist, const double** t_hist);

/* ---- level store export / import (checkpoint) ----------------------- */

/* Device bytes the level store of this context takes at a precision. */
int tdbem_level_bytes(const tdbem_ctx* ctx, int precision, size_t* bytes);

/* Binary checkpoint of the level store: a 64-byte header (magic "TDBEMLVL",
 * version 1, D, MaxStep, precision, levels held, row stride) and the raw levels
 * (FP64: G then H, (M+1) x D x D; TDBEM_MIXED: FP32 G then H, (M+1) x D x ld,
 * then the FP64 levels 0-1 of G and H).  Import needs a context of the same
 * mesh size (D and MaxStep) and replaces its levels.  The reference keeps its
 * levels in memory only; this is the resume point that saves the assembly. */
int tdbem_export_levels(tdbem_ctx* ctx, const char* path);
int tdbem_import_levels(tdbem_ctx* ctx, const char* path);

/* SolverT::WriteGH (SolverT.cpp:670-732) on one rank: writes
 * <name_prefix><step>.txt with num_row lines of num_column values (row stride
 * num_column), each "%15.5e", the file the reference's FE-BE coupling reads
 * (FE-BE Matlab/BE_Matrices/ReadGH.m). */
int tdbem_write_gh(const char* name_prefix, int step, int num_row, int num_column,
                   const double* data);

/* Timing of the phases of the last assemble / march, in milliseconds of
 * device time (CUDA events on the context stream): [0] assembly,
 * [1] H^0 factorisation, [2] marching steps.  */
int tdbem_last_timings(const tdbem_ctx* ctx, double* ms3);

/* ---- profiling ------------------------------------------------------ */

/* Kernel classes for tdbem_kernel_stats. */
#define TDBEM_K_ASSEMBLE 0     /* FP64 level quadrature items (all pairs, or near pairs) */
#define TDBEM_K_CONV 1         /* per-step history convolution (HBM)                 */
#define TDBEM_K_FACTOR 2       /* H^0 inverse (Gauss-Jordan)                         */
#define TDBEM_K_SOLVE 3        /* per-step solve and state update                    */
#define TDBEM_K_ASSEMBLE_F32 4 /* FP32 far-field quadrature items (mixed)            */
#define TDBEM_K_CONV_BLOCK 5   /* time-block history convolution, NB columns (mixed) */
#define TDBEM_K_AUX 6          /* window/scan, C term, LHS build, W vectors          */
#define TDBEM_K_CONV_BATCH 7   /* batched convolution GEMM on the tensor cores       */
#define TDBEM_K_SOLVE_BATCH 8  /* batched inverse product, refinement, state update  */
#define TDBEM_K_COUNT 9

/* With on != 0, every launch of the kernel classes above is bracketed by CUDA
 * events on the context stream and its algorithmic bytes / flops are counted
 * (adds event overhead; off by default).  Resets the counters. */
int tdbem_set_profiling(tdbem_ctx* ctx, int on);

/* Accumulated launches, device milliseconds, algorithmic bytes moved and
 * algorithmic floating-point operations of one kernel class since profiling
 * was switched on. */
int tdbem_kernel_stats(const tdbem_ctx* ctx, int kclass, long long* launches, double* ms,
                       double* bytes, double* flops);

/* Number of CUDA kernels this context has launched so far. */
int tdbem_launch_count(const tdbem_ctx* ctx, long long* n);

/* ---- serving: continuous batching of transient solves ---------------- */
/* The reference runs one solve per process (main.cpp); it has no server.  The
 * server below accepts whole solves as they arrive and admits them by device
 * footprint into a fixed number of slots.  A slot assembles its solve's levels
 * and prepares its march on the solve's own stream; the time steps of all
 * prepared solves are then batched: one march thread advances every resident
 * solve by a time block of steps in ONE persistent launch (each solve at its own
 * step), retires finished solves and lets newly prepared ones join at the next
 * block boundary.  Levels and histories stay on the device until a solve
 * completes; a result is bitwise the same served alone and in any mix. */

/* Device bytes a solve needs: the level store (levels x D x D x bytes x 2)
 * plus the assembly and marching state of tdbem_assemble_levels + tdbem_march
 * at this precision. */
int tdbem_footprint(const tdbem_mesh* mesh, const tdbem_material* mat, double dt, int nq,
                    int numstep, int precision, size_t* bytes);

typedef struct tdbem_server tdbem_server;

/* One transient solve: the inputs of tdbem_ctx_create, tdbem_set_bc,
 * tdbem_set_alpha, tdbem_set_load_history (amp: numstep values or NULL) and
 * tdbem_assemble_levels / tdbem_march.  The server copies every array. */
typedef struct tdbem_request {
    tdbem_mesh mesh;
    tdbem_material mat;
    double dt;
    int nq;
    int if_ext;
    const int* ubc_dofs;
    const double* ubc_vals;
    int n_u;
    const int* fbc_dofs;
    const double* fbc_vals;
    int n_f;
    double alpha1, alpha2;
    const double* amp;
    int numstep;
    int precision;
} tdbem_request;

#define TDBEM_REQ_QUEUED 0
#define TDBEM_REQ_RUNNING 1
#define TDBEM_REQ_DONE 2
#define TDBEM_REQ_FAILED 3

/* Server on a device with an HBM budget in bytes (0: 90% of the free memory at
 * creation) and `slots` concurrently resident solves (1..64). */
int tdbem_server_create(int device, size_t hbm_budget, int slots, tdbem_server** out);
/* Queue a solve; fails with TDBEM_ERR_NOMEM when it can never fit the budget. */
int tdbem_server_submit(tdbem_server* srv, const tdbem_request* req, long long* id);
/* Wait until the request is done or failed, or timeout_s passes (< 0: no
 * limit); *state is its TDBEM_REQ_* state. */
int tdbem_server_wait(tdbem_server* srv, long long id, double timeout_s, int* state);
/* Histories of a finished request ((numstep+1) x D doubles each, or NULL) and
 * times[3] = {seconds queued, seconds running, latency}; releases the request.
 * A failed request returns its error code and message. */
int tdbem_server_result(tdbem_server* srv, long long id, double* u_hist, double* t_hist,
                        double* times);
int tdbem_server_stats(tdbem_server* srv, size_t* used_bytes, size_t* budget_bytes, int* active,
                       int* queued, long long* completed);
/* The batched march so far: grouped launches (time blocks), solve-steps they
 * advanced (each resident solve's steps summed) and the mean number of resident
 * solves per launch. */
int tdbem_server_march_stats(tdbem_server* srv, long long* launches, long long* solve_steps,
                             double* mean_resident);
/* Finish every queued and running request, then stop. */
int tdbem_server_destroy(tdbem_server* srv);

/* ---------------------------------------------------------------------------
 * Two-region solver: SolverMRT (SolverMRT.h:25-226, SolverMRT.cpp:22-1467).
 *
 * Two regions, each a context (its own mesh and material; its FBC list from
 * tdbem_set_bc gives its loads; UBC lists are not used, as in the reference),
 * joined at n_iface interface nodes: iface1 / iface2 are the 0-based node ids of
 * each region's interface list (ModelManagerT::GetInterface).  Region 2's
 * interface node i is paired with the region-1 interface node at the same
 * coordinates (within 1e-10, the first such; InterfaceIndexing,
 * SolverMRT.cpp:458-494); a node without a partner, or two on one partner, is
 * TDBEM_ERR_ARG.  The combined unknowns (N = D1 + D2, LocalIndexing /
 * InterfaceIndexing, SolverMRT.cpp:158-566) are the interior displacements of
 * region 1 and of region 2 (interior nodes in ascending order), then the
 * interface displacements and the interface tractions of region 1 (its interface
 * order); region 2 sees the interface traction with the opposite sign.
 * max_step is SolverMRT's level count (SetMaxStep; the reference's default is
 * 10).  Both contexts need the same dt and device; the solver uses their FP64
 * level stores (assemble them through tdbem_mrt_assemble only).
 * ------------------------------------------------------------------------- */
typedef struct tdbem_mrt tdbem_mrt;
int tdbem_mrt_create(tdbem_ctx* region1, tdbem_ctx* region2, const int* iface1,
                     const int* iface2, int n_iface, int max_step, tdbem_mrt** out);
int tdbem_mrt_destroy(tdbem_mrt* m);
/* N combined unknowns, NG interior traction dofs (the known vector). */
int tdbem_mrt_size(const tdbem_mrt* m, int* N, int* NG);
/* Combined column of each dof of region 1 or 2: its displacement (ucol) and, on
 * interface dofs, its traction (tcol; -1 elsewhere).  Arrays of 3*nnd ints. */
int tdbem_mrt_columns(const tdbem_mrt* m, int region, int* ucol, int* tcol);
/* SetLoad's amplitude (SolverMRT.cpp:867-966): amp[k] at time k dt (k < n; 0
 * beyond).  n = 0 restores the reference's pulse 5.46366e9 t exp(-2000 t). */
int tdbem_mrt_set_load_history(tdbem_mrt* m, const double* amp, int n);
/* FP64 refinement steps of each solve (0..8, default 1). */
int tdbem_mrt_set_refine(tdbem_mrt* m, int refine);
/* Levels of both regions for a run of numstep steps (G_H_Driver for the steps
 * 1..min(max_step, numstep), as the per-step loop calls it; FP64) and the
 * inverse of the combined H^0 (TDBEM_ERR_SINGULAR on a zero pivot). */
int tdbem_mrt_assemble(tdbem_mrt* m, int numstep);
/* Solve_Direct (SolverMRT.cpp:1028-1097) for steps 1..numstep.  Each output has
 * numstep + 1 rows (row 0 = the zero initial state) and may be NULL: x_hist the
 * N combined unknowns; u1/t1 region 1's displacements / tractions (3*nnd1 per
 * row); u2/t2 region 2's.  Row n of u1 / u2 is what ExtractField stores for step
 * n (the reference stores it one step later, while solving step n + 1). */
int tdbem_mrt_march(tdbem_mrt* m, int numstep, double* x_hist, double* u1_hist,
                    double* t1_hist, double* u2_hist, double* t2_hist);
/* Stepwise form for a per-step driver (SolverMRT::UpdateGHLinear / Solve per
 * step): the caller places each region's step blocks with tdbem_update_gh_linear
 * (steps <= max_step), then tdbem_mrt_step solves step curr_step (the first call
 * forms and inverts H_DB^0 from level 0) and copies that step's x, u1, t1, u2, t2
 * (each may be NULL).  tdbem_mrt_begin zeroes the state for numstep steps. */
int tdbem_mrt_begin(tdbem_mrt* m, int numstep);
int tdbem_mrt_step(tdbem_mrt* m, int curr_step, double* x, double* u1, double* t1, double* u2,
                   double* t2);

#ifdef __cplusplus
}
#endif

#endif /* TDBEM_H */
