// Internal declarations shared by the tdbem-gb300 translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tdbem.h"

namespace tdbem {

// Material / time constants every quadrature kernel needs, passed by value.
struct Phys {
    double dt, inv_dt;           // time step T1 and 1/T1
    double cp, cs;               // wave speeds (GreenFunctionT::WaveSpeed, GreenFunctionT.cpp:76-84)
    double inv_cp, inv_cs;       // 1/cp, 1/cs
    double inv_cp2, inv_cs2;     // 1/cp^2, 1/cs^2
    double cs2;                  // cs^2
    double ratio2, ratio3;       // (cs/cp)^2, (cs/cp)^3
    double inv_4pi_rho;          // 1/(4 pi rho)
    double inv_4pi;              // 1/(4 pi)
    double nu;                   // Poisson ratio (Kelvin traction)
};

// Level-window bounds of one (collocation node, element) pair.
// An element's node centroid and largest node distance from it (launch_element_box).
struct alignas(32) ElemBox {
    double x, y, z, rad;
};

struct PairInfo {
    int klo;    // first level with a possibly non-zero contribution
    int cnt;    // number of levels (0 = pair contributes nothing)
    int sing;   // singular corner (last element node within r^2 < 1e-9), -1 if regular
};

// Which pairs a window pass selects (mixed precision integrates well-separated
// pairs in FP32 and the rest in FP64).
enum PairSelect : int {
    SEL_ALL = 0,   // every pair
    SEL_NEAR = 1,  // singular pairs and pairs within kFarRatio element radii
    SEL_FAR = 2,   // the others
};
// far: a non-singular pair whose node lies outside the element's bounding sphere
// (the FP32 form keeps level entries within ~1e-6 of FP64 down to that distance)
constexpr double kFarRatio = 0.0;

// Assembly output selection.
enum AsmMode : int {
    ASM_LEVELS = 0,  // level k <- I(k dt) + J((k+1) dt)  (UpdateGHLinear placement)
    ASM_STEP = 1,    // one time n: I part -> out0, J part -> out1 (G_H_Driver outputs)
};

struct AsmOut {
    double* G0;   // ASM_LEVELS: G level store; ASM_STEP: G_I rows
    double* H0;   // ASM_LEVELS: H level store; ASM_STEP: H_I rows
    double* G1;   // ASM_STEP: G_J rows
    double* H1;   // ASM_STEP: H_J rows
    float* G0f;   // FP32 level store (mixed precision), or null
    float* H0f;
    size_t level_stride;  // entries per level in ASM_LEVELS (D * ld)
    int D;
    int ld;               // row stride of the store written (D, or D padded for FP32)
    int row_node_lo;      // first collocation node of the row block
};

// Launch helpers (assemble.cu).
// ennd: nodes per element (4 or 8).  8-node elements keep a wider geometry
// table (kGeomStride8 doubles per Gauss point, no FP32 copy) and take the FP64
// quadrature only.
cudaError_t launch_gauss_geom(const double* coords, const int* ien, int nel, int ennd, int nq,
                              const double* gx, const double* gw, double* geom, float* geomf,
                              cudaStream_t s);
// Per element: node centroid and largest node distance from it (x, y, z, radius).
cudaError_t launch_element_box(const double* coords, const int* ien, int ennd, int nel,
                               ElemBox* ebox, cudaStream_t s);
// ebox: launch_element_box's table of the mesh (or null: computed per pair).
cudaError_t launch_pair_window(const double* coords, const int* ien, int ennd, const int* elems,
                               int nelem_color, int node_lo, int nnodes, const Phys& ph,
                               int mode, int level_last, int level_cap, int step_n, int select,
                               PairInfo* pairs, unsigned* counts, cudaStream_t s,
                               const ElemBox* ebox = nullptr);
cudaError_t launch_assemble_items(const double* coords, const int* ien, int ennd,
                                  const int* elems, int nelem_color, int node_lo, int nq,
                                  const double* gx, const double* gw, const double* geom,
                                  const Phys& ph, int mode, int level_last, int step_n,
                                  const PairInfo* pairs, const unsigned* offsets,
                                  unsigned npairs, unsigned nitems, const AsmOut& out,
                                  cudaStream_t s, const double* duffy = nullptr);
// The Duffy points of every (element, corner) of a 4-node mesh (kGeomStride doubles
// each): duffy_table_elems doubles.  duffy (may be null) in the item and C-term
// launches: the singular pairs read their points from it.
size_t duffy_table_elems(int nel, int nq);
cudaError_t launch_duffy_table(const double* coords, const int* ien, int nel, int nq,
                               const double* gx, const double* gw, double* duffy,
                               cudaStream_t s);
// Element interface: n independent (collocation point, element) pairs, element
// node coordinates ecoords[n][ennd][3], time times[n], singular local node sing[n]
// (-1: FormGH_Regular); GE1/HE1 (I part), GE2/HE2 (J part) [n][3][3 ennd] and C1 / C2
// [n][9] (the Kelvin part when times[i] == ph.dt, zeros otherwise).
cudaError_t launch_element_gh(int ennd, int n, int nq, const double* gx, const double* gw,
                              const Phys& ph, const double* colloc, const double* ecoords,
                              const double* times, const int* sing, double* GE1, double* GE2,
                              double* HE1, double* HE2, double* C1, double* C2, cudaStream_t s);
// Material and time-step constants of the kernels (GreenFunctionT::WaveSpeed,
// GreenFunctionT.cpp:76-84).
Phys make_phys(double E, double nu, double rho, double dt);
// One step (ASM_STEP) over the pairs of a window pass without compaction: one thread
// per pair (two for 8-node elements), no scan and no item total on the host.
cudaError_t launch_assemble_step_pairs(const double* coords, const int* ien, int ennd,
                                       const int* elems, int nelem_color, int node_lo, int nq,
                                       const double* gx, const double* gw, const double* geom,
                                       const Phys& ph, int step_n, const PairInfo* pairs,
                                       unsigned npairs, const AsmOut& out, cudaStream_t s);
// Far (well-separated) items of every node in FP32, ASM_LEVELS, into the FP32 store:
// one launch over (node, chunk of levels) blocks, colours walked inside each block.
// pairs holds nnd x nel windows (SEL_FAR), elements in colour order; nitems[0..2]
// (if not null) receive the counts of items through the quadrature, of settled jobs
// and of settled levels.  4-node elements only.
cudaError_t launch_assemble_far_rows(const double* coords, const int* ien,
                                     const int* color_elems, const int* color_start, int ncolor,
                                     int nnd, int nel, int nq, const float* geomf,
                                     const double* geom, const float* coordf, const Phys& ph,
                                     int level_last, const PairInfo* pairs, const AsmOut& out,
                                     unsigned long long* nitems, cudaStream_t s,
                                     int level_cap = 1 << 30, bool fp64_out = false);
cudaError_t launch_cterm(const double* coords, const int* ien, int ennd, int nel, int node_lo,
                         int nnodes, int nq, const double* gx, const double* gw,
                         const double* geom, const Phys& ph, double* cbuf, cudaStream_t s,
                         bool fast = false, const float* geomf = nullptr,
                         const float* coordf = nullptr, const ElemBox* ebox = nullptr,
                         const double* duffy = nullptr);
cudaError_t launch_cast_levels01(const double* G01, const double* H01, int D, int ldf, float* Gf,
                                 float* Hf, cudaStream_t s);
cudaError_t launch_cterm_apply(const double* cbuf, int node_lo, int nnodes, double dt,
                               int if_ext, int mode, const AsmOut& out, cudaStream_t s);
size_t scan_temp_bytes(unsigned n);

// One mesh of a grouped assembly launch (many meshes in one launch; assemble.cu).
struct GroupAsm {
    const double* coords;
    const int* ien;
    const int* elems;      // this launch's colour of the mesh
    int ne;                // elements of that colour
    int nnd, nel, nq;
    const double* gx;
    const double* gw;
    const double* geom;
    Phys ph;
    int level_last;        // levels hold steps 1..level_last
    int level_cap;
    int if_ext;
    AsmOut out;            // FP64 level store of the mesh
    unsigned pair_begin;   // first pair of the mesh in the launch's pair list
    unsigned node_begin;   // first node of the mesh in the C-term launches
    double* cbuf;          // nnd x 9 C term of the mesh
};
cudaError_t launch_pair_window_group(const GroupAsm* gm, int nmesh, unsigned npairs,
                                     PairInfo* pairs, unsigned* counts, cudaStream_t s);
cudaError_t launch_assemble_group(const GroupAsm* gm, int nmesh, const PairInfo* pairs,
                                  const unsigned* offsets, unsigned npairs, unsigned nitems,
                                  cudaStream_t s);
cudaError_t launch_cterm_group(const GroupAsm* gm, int nmesh, unsigned nnodes, cudaStream_t s);

// One mesh of a persistent grouped march (group_march.cu): FP64 levels and inverses.
struct GroupMarch {
    int D, M, numstep;
    int off;               // the mesh's step s runs at the launch's global step s + off
    const double* G;       // (M+1) x D x D
    const double* H;
    const double* Ainv0;   // inverse of step 2's LHS
    const double* Ainv1;   // inverse of the LHS of steps >= 3
    double* u;             // (numstep+1) x D histories
    double* t;
    const unsigned char* is_u;
    const unsigned char* is_f;
    const double* ubc;
    const double* fbc;
    const double* load_t;
    const double* load_u;
    const double* amp;     // numstep values, or null (unit step)
    double a1, a2, a3, c0, c1;  // weights; LHS weights of steps >= 3
    double* Wt;            // (M+1) x D
    double* Wu;
    double* rhs;           // D
    unsigned row_begin;    // first row of the mesh in the grid's row list
    unsigned w_begin;      // first (level, dof) entry of the mesh in the W list
    // mixed precision (TDBEM_MIXED levels): FP32 levels and inverses, FP64 LHS
    const float* Gf;       // (M+1) x D x ldf
    const float* Hf;
    int ldf;
    const float* inv32_0;  // FP32 inverses of the two LHS
    const float* inv32_1;
    const double* Hc0;     // FP64 column-exchanged LHS (refinement residual)
    const double* Hc1;
    float* Wtf;            // (M+1) x D FP32 history vectors (group scratch)
    float* Wuf;
    double* x;             // D: first solution, then the refined one
    double* r;             // D: residual
    int refine;            // refinement sweeps (0 or 1)
    int step2_sweeps;      // > 0: step 1's solve by this many Richardson sweeps (inv32_0 =
                           // inv32_1, Hc0 the step's own FP64 LHS)
    // time blocks of kGroupNB steps (mixed): old-history vectors and their product
    float* Wold_t;         // (M+1) x kGroupNB x ldf
    float* Wold_u;
    double* Yold;          // kGroupNB x D
    unsigned quad_begin;   // first 4-row block of the mesh in the grid's list
    unsigned wold_begin;   // first (level, column, dof) entry in the old-W list
};
constexpr int kGroupNB = 12;  // steps per time block of the mixed grouped march
struct GroupShape {
    int lanes;             // lanes per row: 8, 16 or 32
    int block;             // threads per block
    int blocks_per_sm;     // at most the occupancy limit
};
// nquads / nwold: 4-row blocks and old-W entries of all meshes (mixed form only).
// st_lo..st_hi: global steps; mesh i runs its own steps st - gm[i].off (only those
// in 1..numstep-1).  has_offsets: some mesh has off != 0 (they join at block starts
// of the mixed form's time blocks: off is a multiple of kGroupNB).
cudaError_t launch_march_group(const GroupMarch* gm, int nmesh, unsigned nrows, unsigned nw,
                               unsigned nquads, unsigned nwold, int st_lo, int st_hi,
                               const GroupShape& shape, bool mixed, cudaStream_t s,
                               bool has_offsets = false);
cudaError_t exclusive_scan(const unsigned* in, unsigned* out, unsigned n, void* tmp,
                           size_t tmp_bytes, cudaStream_t s);

// Marching helpers (march.cu).
struct MarchDev {
    int D, M;
    const double* G;   // FP64 level store (M+1) x D x D, or null
    const double* H;
    const float* Gf;   // FP32 level store, or null
    const float* Hf;
};
cudaError_t launch_build_lhs(const double* G, const double* H, const float* Gf,
                             const float* Hf, size_t level_stride, int D, double c0,
                             double c1, const unsigned char* is_ubc, double* A,
                             cudaStream_t s);
constexpr int kPermuteBlocks = 152;  // scratch rows the final column permutation may use
// Blocked Gauss-Jordan inverse (inverse.cu); scratch holds inverse_scratch_elems(n)
// elements, perm has n + 2 * kMaxPivotBlocks ints.
constexpr int kMaxPivotBlocks = 32;
size_t inverse_scratch_elems(int n);
// *singular is set (and cudaSuccess returned) when a pivot is exactly zero.
cudaError_t invert_f64(double* A, int n, int* perm, int* d_status, double* scratch,
                       long long* nlaunch, bool* singular, cudaStream_t s);
// Outcome of an FP32 inverse: the probe's relative residual max |A (X v) - v| /
// max |v| and whether the pivot search fell back from the panels' diagonal blocks
// to the full panel (a zero pivot there, or a probe above kInverseProbeBar).
struct InverseReport {
    float probe_rel = 0;
    int full_search = 0;
};
constexpr float kInverseProbeBar = 1e-5f;
// Sweeps of the Richardson iteration x <- x + X (b - A x) (x0 = X b, FP64 residual,
// FP32 X) that bring the probe problem b = A v within tol (max |x - v| / max |v|);
// *sweeps = 0 when max_sweeps do not.  work: 3 n + max_sweeps + 2 doubles of scratch.
cudaError_t richardson_probe(const double* A, const float* X, int n, double* work, int max_sweeps,
                             double tol, int* sweeps, long long* nlaunch, cudaStream_t s);
// The step-2 solve by Richardson sweeps with the later steps' inverse: the iteration's
// tolerance on the probe problem, the most sweeps tried, and the margin added.
constexpr double kStep2Tol = 1e-7;
constexpr int kStep2MaxSweeps = 48, kStep2Margin = 2;
cudaError_t invert_f32(const double* A64, float* A, int n, int* perm, int* d_status,
                       float* scratch, long long* nlaunch, bool* singular, cudaStream_t s,
                       InverseReport* report = nullptr);
cudaError_t launch_history_combine(const double* u_hist, const double* t_hist, int D, int s,
                                   int L, double a1, double a2, double a3, double c0,
                                   double c1, double amp, const double* load_t,
                                   const double* load_u,
                                   double* Wt, double* Wu, cudaStream_t st);
cudaError_t launch_conv(const MarchDev& md, int L, const double* Wt, const double* Wu,
                        double* partial, int nchunks, cudaStream_t s);
cudaError_t launch_reduce_solve(const double* partial, int nchunks, int D,
                                const double* Ainv, double* rhs, double* x, cudaStream_t s);
cudaError_t launch_add_inplace(double* y, const double* x, size_t n, cudaStream_t s);
// rhs[i] = sum over chunks of partial[chunk][i]; x = A v for a D x D row-major A.
cudaError_t launch_reduce_partial(const double* partial, int nchunks, int D, double* rhs,
                                  cudaStream_t s);
cudaError_t launch_gemv(const double* A, int D, const double* v, double* x, cudaStream_t s);
// Level chunks of the convolution over levels 0..L of a D-row store (march.cu).
int conv_chunks(int L, int D);
cudaError_t launch_update_state(const double* x, int D, int s, const unsigned char* is_u,
                                const double* ubc_val, const unsigned char* is_f,
                                const double* fbc_val, double amp, double* u_hist,
                                double* t_hist, cudaStream_t st);
int conv_chunks(int L, int D);

// Per-column load terms of a time block's old pass (steps S + j, j < nload <= 16).
struct BlockLoads {
    int nload;
    double amp[16], c0[16], c1[16];
    const double* load_t;
    const double* load_u;
};

// Batched convolution on tcgen05 tensor cores (conv_tc.cu).
constexpr int kTensorMapBytes = 128;
struct TcMaps {
    alignas(64) unsigned char a[kTensorMapBytes];  // BF16 level planes
    alignas(64) unsigned char b[kTensorMapBytes];  // BF16 history-vector planes
};
int tc_ldb(int D);
int tc_cases_pad(int C);
// Grid splits of a k_conv_tc launch (each writes its own partial sums: at most
// max_splits of them fit the caller's buffer).
// nmat: matrices per level in the planes (1: the merged level matrix of the single
// and batched marches, march_tc.cu; 2: a G and an H plane pair per level).
int tc_conv_splits(int nlev, int D, int C, int max_splits = 1 << 30, int nmat = 1);
size_t tc_plane_bytes(int D, int L, int nmat = 1);
size_t tc_w_bytes(int D, int C, int Lw, int nmat = 1);
bool make_tc_maps(void* planes, int D, int L, void* W, int C, int Lw, TcMaps* out,
                  int nmat = 1);
// Default limit of each pipeline wait of k_conv_tc (2 s of %globaltimer).
constexpr unsigned long long kTcWaitNsDefault = 2000000000ull;
// The product reads level slabs lev0 .. lev0 + nlev - 1 of the planes (L slabs per
// plane) with the vector slabs 0 .. nlev - 1.
// occ (optional, nmat == 1): the tile occupancy of the planes' slabs (tc_occ_bytes);
// all-zero tiles are skipped.
cudaError_t launch_conv_tc(const TcMaps& maps, int D, int L, int Lw, int nlev, int C,
                           double* partial, int splits, int* d_err, cudaStream_t s, int nmat = 1,
                           unsigned long long wait_ns = kTcWaitNsDefault, int lev0 = 0,
                           const unsigned char* occ = nullptr);
// Tile occupancy of the merged planes' slabs [slab_lo, slab_hi) (one byte per
// 128-row x 64-column tile of each slab; tc_occ_bytes(D, slabs) for all slabs).
size_t tc_occ_bytes(int D, int slabs);
cudaError_t launch_tile_occupancy(const void* planes, int D, int slab_lo, int slab_hi,
                                  unsigned char* occ, cudaStream_t s);

// Mixed march with merged levels on tcgen05 (march_tc.cu).
// The merged planes hold, per plane, the M + 1 level matrices A^f and after them the
// kStepMats step-distance matrices B_d (d = 1 .. kStepMats): the weight of the
// history of step m in the right-hand side of step m + d,
//   B_1 = (a2 - a1) A^0 + a3 A^1 + a1 A^2,   B_d = a2 A^(d-1) + a3 A^d + a1 A^(d+1),
// which the in-block cross terms of time blocks of up to kStepMats + 1 steps read
// instead of the levels (two matrices fewer per cross term).
constexpr int kStepMats = 31;
inline int mtc_slabs(int M) { return M + 1 + kStepMats; }
cudaError_t launch_merge_levels(const float* Gf, const float* Hf, int ldf, int D, int L,
                                int slabs, const unsigned char* is_u, const float* kt,
                                const float* lt, const float* lu, void* planes, double* known,
                                cudaStream_t s);
// B_1 .. B_kStepMats from the FP32 levels into slabs M + 1 .. of the planes.
cudaError_t launch_step_mats(const float* Gf, const float* Hf, int ldf, int D, int M, int slabs,
                             const unsigned char* is_u, double a1, double a2, double a3,
                             void* planes, cudaStream_t s);
// History planes of B_1 .. B_nmats for the steps b .. b + ncol - 1 from the history
// steps [a, b): slab d - 1, column j holds x_(b + j - d) where a <= b + j - d < b.
cudaError_t launch_build_w_steps(const double* u_hist, const double* t_hist,
                                 const unsigned char* is_u, int D, int a, int b, int ncol,
                                 int Cmax, int nmats, int Lw, void* W, cudaStream_t st);
cudaError_t launch_build_w_merged(const double* u_hist, const double* t_hist,
                                  const unsigned char* is_u, int D, int s0, int ncol, int Cmax,
                                  int lo, int hi, int nlev, int Lw, double a1, double a2,
                                  double a3, void* W, cudaStream_t st);
// Known part of the right-hand sides of the solve steps 1..last into Yk[step][D].
cudaError_t launch_known_terms(const double* known, const void* coef, int D, int L, int last,
                               double* Yk, cudaStream_t s);
// Batched form of the merged march: history planes of all cases, the cases' known
// tractions as FP32 columns, and the known part of step s added into Y[c][D].
cudaError_t launch_build_w_batch_merged(const double* u_hist, const double* t_hist,
                                        const unsigned char* is_u, int D, int C, int s,
                                        int nlev, int Lw, double a1, double a2, double a3,
                                        void* W, cudaStream_t st);
cudaError_t launch_batch_known_tractions(const double* trac, const unsigned char* is_u, int D,
                                         int C, float* kt, float* lt, cudaStream_t s);
cudaError_t launch_known_batch(const float* GK, const float* GL, const double* HU, int D, int C,
                               int L, int s, double a1, double a2, double a3, double c0,
                               double c1, const double* amp, int numstep, double* Y,
                               cudaStream_t st);
// G^f K for levels f < nlev (FP32 levels, ld ldf) and the columns K [c][D]: out
// [f][c][D], FP32 (k_levels_times_columns, inverse.cu).
cudaError_t levels_times_columns(const float* Gf, int ldf, int D, int nlev, const float* K,
                                 int C, float* out, cudaStream_t s);
void known_coefficients(int numstep, int L, double a1, double a2, double a3,
                        const std::vector<double>& amp, double c0, double c1,
                        std::vector<double>& out);


// Sets the calling thread's tdbem_last_error() message (capi.cu).
void note_error(const char* msg);

// Mixed-precision marching (march_mixed.cu).
int mixed_ldw(int D);
int mixed_ld(int D);
int mixed_chunks(int nlev, int D);
// Column splits for a convolution of nchunks level chunks, at most cap partials.
int mixed_ksplit(int nchunks, int D, int cap);
// *nparts receives the number of partial sums written (level chunks x column splits).
cudaError_t launch_conv_f32(const float* G, const float* H, size_t lstride, int ld, int D,
                            int f_lo, int f_hi, int nb, const float* Wt, const float* Wu,
                            int ldw, double* partial, int nchunks, int ksplit, int* nparts,
                            cudaStream_t s);
cudaError_t launch_build_w_old(const double* u_hist, const double* t_hist, int D, int S, int nb,
                               int nlev, double a1, double a2, double a3, const BlockLoads& bl,
                               int ldw, float* Wt, float* Wu, cudaStream_t s);
// History of steps [a, b) into the steps b .. b+ncol-1 (nbp >= ncol padded columns).
cudaError_t launch_build_w_cross(const double* u_hist, const double* t_hist, int D, int a, int b,
                                 int ncol, int nbp, int nlev, double a1, double a2, double a3,
                                 int ldw, float* Wt, float* Wu, cudaStream_t s);
// The first ncol of nb partial columns (out and add have ncol columns).
// v32 (optional): column 0 of out also in FP32 (the vector the next solve multiplies).
cudaError_t launch_reduce_cols_n(const double* partial, int nchunks, int nb, int ncol, int D,
                                 const double* add, double* out, cudaStream_t s,
                                 float* v32 = nullptr);
cudaError_t launch_reduce_cols(const double* partial, int nchunks, int nb, int D,
                               const double* add, double* out, cudaStream_t s);
// The histories' update of solve step s from its unknowns (state_update.cuh); a null
// u_hist means none.
struct StateUpdate {
    const unsigned char* is_u = nullptr;
    const double* ubc = nullptr;
    const unsigned char* is_f = nullptr;
    const double* fbc = nullptr;
    double amp = 1.0;
    double* u_hist = nullptr;
    double* t_hist = nullptr;
    int s = 0;
};
// v32_ready: v32 already holds rhs in FP32 (the reduction that finished rhs wrote it);
// upd (if its u_hist is set): the step's state update, done by the last product.
cudaError_t launch_solve_mixed(const float* inv32, const double* A64, int D, const double* rhs,
                               double* x, double* r, float* v32, int n_refine, cudaStream_t s,
                               bool v32_ready = false, const StateUpdate& upd = StateUpdate());

// Batched marching of many load cases (batch.cu).
int batch_block_cases();            // cases per tensor-core column block
int batch_ldw(int D);               // row stride of the batched history vectors
int batch_conv_splits(int nlev, int D, int C);
int batch_apply_splits(int D, int C);
cudaError_t launch_conv_mma(const float* G, const float* H, size_t lstride, int ld, int D,
                            int nlev, const float* Wt, const float* Wu, int ldw, int C,
                            double* partial, int splits, cudaStream_t s);
cudaError_t launch_apply_cols(const void* A, int fp64_residual, int D, const double* X, int C,
                              double* partial, int splits, cudaStream_t s);
cudaError_t launch_build_w_batch(const double* u_hist, const double* t_hist, int D, int C, int s,
                                 int nlev, double a1, double a2, double a3, double c0, double c1,
                                 const double* amp, int numstep, const double* traction,
                                 const unsigned char* is_u, const double* ubc_val, int ldw,
                                 float* Wt, float* Wu, cudaStream_t st);
cudaError_t launch_update_batch(const double* x, int D, int C, int s, const unsigned char* is_u,
                                const double* ubc_val, const double* traction,
                                const double* amp, int numstep, double* u_hist, double* t_hist,
                                cudaStream_t st);

}  // namespace tdbem

// A captured marching loop and the values its kernel arguments were captured
// with (a change of any of them means a new capture).
struct MarchGraph {
    cudaGraphExec_t exec = nullptr;
    int kind = -1, numstep = 0, nb = 0, refine = 0;
    double a1 = 0, a2 = 0;
    std::vector<double> amp;
    std::vector<const void*> ptrs;
    unsigned long long wait_ns = 0;  // pipeline wait limit of the tcgen05 kernels
    int step2_sweeps = 0;            // Richardson sweeps of the step-2 solve
    long long launches = 0;  // kernels in the graph
};

// The context (capi.cu owns its lifetime).
struct tdbem_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int nnd = 0, nel = 0, D = 0, M = 0, nq = 6, if_ext = 0;
    int ennd = 4;                    // nodes per element: 4 (EType 1) or 8 (EType 2)
    double E = 0, nu = 0, rho = 0, dt = 0;
    tdbem::Phys ph{};
    std::vector<double> h_coords;
    std::vector<int> h_ien;
    // device mesh and quadrature tables
    double* d_coords = nullptr;
    int* d_ien = nullptr;
    double* d_gx = nullptr;
    double* d_gw = nullptr;
    double* d_geom = nullptr;        // regular Gauss-point geometry, nel x nq^2 x 12
    double* d_cterm = nullptr;       // C term of every node, nnd x 9
    float* d_geomf = nullptr;        // FP32 copy of the geometry (element-relative points)
    float* d_coordf = nullptr;       // node coordinates as FP32 pairs: hi[3], 0, lo[3], 0
    tdbem::ElemBox* d_ebox = nullptr;      // per element: node centroid, node radius (launch_element_box)
    double* d_duffy = nullptr;       // 4-node meshes: the Duffy points of every (element, corner)
    // element colouring: elements of colour c are color_elems[color_start[c] .. color_start[c+1])
    std::vector<int> color_start;
    int* d_color_elems = nullptr;
    int* d_color_start = nullptr;    // color_start on the device
    tdbem::PairInfo* d_far_pairs = nullptr;  // mixed: windows of all nnd x nel pairs (SEL_FAR)
    size_t far_pairs_cap = 0;
    unsigned long long* d_far_items = nullptr;  // far items, settled jobs, settled levels (profiling)
    // pair/item scratch
    tdbem::PairInfo* d_pairs = nullptr;
    unsigned* d_counts = nullptr;
    unsigned* d_offsets = nullptr;
    void* d_scan_tmp = nullptr;
    size_t scan_tmp_bytes = 0;
    size_t pair_cap = 0;
    // level store
    int level_precision = -1;
    int levels_last = 0;             // levels hold steps 1..levels_last
    double* d_G = nullptr;
    double* d_H = nullptr;
    float* d_Gf = nullptr;          // mixed: FP32 levels 0..M, row stride ldf
    float* d_Hf = nullptr;
    int ldf = 0;
    double* d_G01 = nullptr;        // mixed: levels 0 and 1 in FP64 (the LHS)
    double* d_H01 = nullptr;
    // mixed marching
    int nb = 0;                     // steps per time block (0: the engine's default)
    int nb_eff = 0;                 // the block of the last mixed march
    int nb_alloc = 0;               // the block its scratch is sized for
    int n_refine = 0;               // FP64 refinement sweeps per solve
    float* d_inv32[2] = {nullptr, nullptr};
    double* d_Hc64[2] = {nullptr, nullptr};
    float* d_Wt_old = nullptr;
    float* d_Wu_old = nullptr;
    double* d_Yold = nullptr;
    double* d_pmix = nullptr;       // conv partials, chunks x nb x D
    double* d_res = nullptr;
    double* d_dx = nullptr;
    // batched marching (tdbem_march_batch): C cases, histories [step][case][dof]
    int batch_C = 0, batch_steps = -1;
    double* d_bu = nullptr;
    double* d_bt = nullptr;
    double* d_btrac = nullptr;      // C x D traction vectors
    double* d_bamp = nullptr;       // C x numstep amplitudes
    float* d_bWt = nullptr;         // (M+1) x C x ldw history vectors
    float* d_bWu = nullptr;
    double* d_bpart = nullptr;      // split partial sums
    size_t bpart_cap = 0;
    double* d_brhs = nullptr;       // C x D
    double* d_bx = nullptr;
    double* d_br = nullptr;
    int batch_engine = TDBEM_ENGINE_TCGEN05;
    int batch_refine = 0;           // refinement sweeps of the batched solve
    void* d_tc_W = nullptr;         // BF16 hi/lo planes of the batched history vectors
    float* d_bkt = nullptr;         // batched known tractions as FP32 columns: kt, lt (2 C D)
    float* d_bGK = nullptr;         // G^f kt of every level and case [f][c][D]
    float* d_bGL = nullptr;         // G^f lt of levels 0/1 [f][c][D]
    size_t tc_W_bytes = 0;
    int* d_tc_err = nullptr;        // tcgen05 kernel: [0] wait time-out code, [1] CTAs holding TMEM
    unsigned long long tc_wait_ns = tdbem::kTcWaitNsDefault;  // its pipeline wait limit
    tdbem::InverseReport inv_report[2];  // probe and pivot search of the FP32 inverses
    // mixed form: > 0 when step 2's LHS is solved by this many Richardson sweeps with the
    // later steps' FP32 inverse (d_inv32[0] then aliases d_inv32[1]), 0 with its own
    int step2_sweeps = 0;
    // grouped marching: the load history on the device, the FP32 time-block scratch
    double* d_group_amp = nullptr;
    float* d_group_wf = nullptr;
    double* d_group_yold = nullptr;
    tdbem::TcMaps tc_maps{};
    // mixed march: engine of the time blocks' old-history pass, its BF16 vector planes
    // and tensor maps (encoded for d_mtc_W and the level planes)
    int march_engine = TDBEM_ENGINE_TCGEN05;
    void* d_mtc_W = nullptr;
    size_t mtc_W_bytes = 0;
    tdbem::TcMaps mtc_maps{};
    const void* mtc_maps_for[2] = {nullptr, nullptr};
    int mtc_nb = 0;
    // merged level planes of the tcgen05 march (march_tc.cu), the known part's
    // vectors (pt, pl, pu per level), the BC vectors they come from (kt, lt, lu)
    // and the per-step coefficients with the key they were built for
    void* d_mtc_planes = nullptr;
    double* d_mtc_known = nullptr;
    bool mtc_planes_valid = false;
    double mtc_step_key[2] = {-1.0, -1.0};  // (a1, a2) of the planes' step matrices
    bool mtc_steps_valid = false;
    unsigned char* d_mtc_occ = nullptr;  // tile occupancy of the planes' slabs
    // profiling: live 128 x 64 tiles per slab (summed over the row tiles), so that the
    // convolution's bytes count the tiles it reads
    std::vector<long long> h_occ_live;
    float* d_mtc_bc = nullptr;
    double* d_mtc_coef = nullptr;
    size_t mtc_coef_cap = 0;
    double* d_mtc_yk = nullptr;      // known part of every step's right-hand side
    size_t mtc_yk_cap = 0;
    std::vector<double> mtc_coef_key;
    // stepwise marching (tdbem_march_begin / tdbem_march_step) and host-block levels
    bool use_graphs = true;         // replay the marching loop as a CUDA graph
    MarchGraph graph;
    int step_numstep = -1;
    bool step_inv_ready[2] = {false, false};
    double* d_upd_tmp = nullptr;    // one row block of tdbem_update_gh_linear
    size_t upd_tmp_cap = 0;

    // boundary conditions and marching parameters
    std::vector<int> ubc, fbc;
    std::vector<double> ubc_v, fbc_v;
    double a1 = 0, a2 = 0;
    std::vector<double> amp;
    // marching buffers
    int hist_steps = -1;
    double* d_u = nullptr;
    double* d_t = nullptr;
    double* d_Ainv[2] = {nullptr, nullptr};
    double* d_ubc_map = nullptr;     // per-dof prescribed displacement
    double* d_fbc_map = nullptr;     // per-dof traction value
    unsigned char* d_is_ubc = nullptr;
    unsigned char* d_is_fbc = nullptr;
    double* d_inv_scratch = nullptr;  // blocked inverse scratch (FP64)
    float* d_inv_scratch32 = nullptr;
    // mixed: side streams of the FP32 inverses (the two run concurrently, and next to
    // the far-field assembly when it makes them), the second inverse's scratch, and
    // the key of the inverses held (alpha, UBC dofs, count; levels 0/1 unchanged)
    cudaStream_t stream2 = nullptr;
    cudaStream_t stream3 = nullptr;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_fork2 = nullptr;
    bool inv_valid = false;
    int inv_n = 0;
    double inv_a1 = 0, inv_a2 = 0;
    std::vector<int> inv_ubc;
    float* d_inv_scratch32b = nullptr;
    int* d_perm2 = nullptr;
    int* d_status2 = nullptr;
    double* d_load_t = nullptr;
    double* d_load_u = nullptr;
    double* d_Wt = nullptr;
    double* d_Wu = nullptr;
    double* d_partial = nullptr;
    double* d_rhs = nullptr;
    double* d_x = nullptr;
    int* d_perm = nullptr;
    int* d_status = nullptr;
    size_t partial_cap = 0;
    double timings[3] = {0, 0, 0};
    // profiling (tdbem_set_profiling): pending event pairs and per-class totals
    struct ProfEvent {
        int cls;
        cudaEvent_t a, b;
        double bytes, flops;
    };
    long long launches = 0;          // kernels this context has launched (tdbem_launch_count)
    bool prof = false;
    std::vector<ProfEvent> prof_pending;
    long long prof_launches[TDBEM_K_COUNT] = {};
    double prof_ms[TDBEM_K_COUNT] = {};
    double prof_bytes[TDBEM_K_COUNT] = {};
    double prof_flops[TDBEM_K_COUNT] = {};
};
