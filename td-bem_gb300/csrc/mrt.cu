// Two-region solver: SolverMRT (SolverMRT.cpp) on one GB300.
//
// The reference joins two regions at an interface and solves the combined
// system in the unknowns x = [u_r1, u_r2, u_z, t_z]: the interior displacements
// of region 1 and 2, the interface displacements and the interface tractions of
// region 1 (LocalIndexing / InterfaceIndexing, SolverMRT.cpp:158-566).  Its level
// store holds combined (D1 + D2)-row matrices (Assemble_GH_R1/R2, 663-847), and
// each step of Solve_Direct (1028-1097) is
//     x^n = (H_DB^0)^-1 (G_DB^0 tg^n + sum_{f=1}^{min(n,L)} (G_DB^f tg^{n-f} - H_DB^f x^{n-f})).
// On region r's rows the combined products are the region's own:
//     G_DB^f tg^m - H_DB^f x^m = G_r^f t_r^m - H_r^f u_r^m,
// with u_r, t_r the region's displacement and traction rebuilt from x (region 2
// takes the interface traction with the opposite sign) and its interior loads.
// So the level stores stay per region (D1^2 + D2^2 entries per level instead of
// (D1 + D2)^2, and no zero blocks), the history sum is the single-region
// convolution kernel run on each region, and only H_DB^0 is formed, once, for
// its inverse.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "tdbem_internal.cuh"

using namespace tdbem;

namespace {

int mfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    tdbem::note_error(buf);
    return code;
}

#define MRT_TRY(expr)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return mfail(e_ == cudaErrorMemoryAllocation ? TDBEM_ERR_NOMEM : TDBEM_ERR_CUDA, \
                         "%s: %s", #expr, cudaGetErrorString(e_));                       \
    } while (0)

template <typename T>
cudaError_t alloc(T** p, size_t count) {
    *p = nullptr;
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(count, 1));
}

template <typename T>
void release(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// SetLoad's amplitude (SolverMRT.cpp:881-887).
double reference_pulse(int n, double dt) {
    const double p0 = 5.46366e9;
    const double t = n * dt;
    return p0 * t * std::exp(-2000 * t);
}

// Row block of region r in H_DB^0: A[row_lo + i][ucol[j]] = H^0[i][j] and, for
// interface dofs, A[row_lo + i][tcol[j]] = -tsign G^0[i][j] (Assemble_GH_R1 moves
// -G_z to the left, Assemble_GH_R2 +G_z).  The columns of one region are distinct,
// so every entry is written once.
__global__ void k_mrt_lhs(const double* __restrict__ H0, const double* __restrict__ G0, int D,
                          const int* __restrict__ ucol, const int* __restrict__ tcol,
                          double tsign, int row_lo, int N, double* __restrict__ A) {
    const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= (size_t)D * D) return;
    const int i = (int)(idx / D), j = (int)(idx % D);
    double* row = A + (size_t)(row_lo + i) * N;
    row[ucol[j]] = H0[idx];
    if (tcol[j] >= 0) row[tcol[j]] = -tsign * G0[idx];
}

// The convolution vectors of region r at step n: level 0 takes the step's load
// (interior FBC values x amplitude) against G^0 and nothing against H^0; level f
// takes the region's traction / displacement of step n - f.
__global__ void k_mrt_w(const double* __restrict__ u_hist, const double* __restrict__ t_hist,
                        const double* __restrict__ fl, int D, int n, int L, double amp,
                        double* __restrict__ Wt, double* __restrict__ Wu) {
    const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= (size_t)(L + 1) * D) return;
    const int f = (int)(idx / D), j = (int)(idx % D);
    if (f == 0) {
        Wt[idx] = fl[j] * amp;
        Wu[idx] = 0.0;
    } else {
        const size_t m = (size_t)(n - f) * D + j;
        Wt[idx] = t_hist[m];
        Wu[idx] = u_hist[m];
    }
}

// Region r's state of step n from the combined unknowns (ExtractField,
// SolverMRT.cpp:1261-1309, without its one-step lag): u = x[ucol]; t = tsign
// x[tcol] on interface dofs, the load elsewhere.
__global__ void k_mrt_state(const double* __restrict__ x, const int* __restrict__ ucol,
                            const int* __restrict__ tcol, double tsign,
                            const double* __restrict__ fl, double amp, int D, int n,
                            double* __restrict__ u_hist, double* __restrict__ t_hist) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= D) return;
    u_hist[(size_t)n * D + j] = x[ucol[j]];
    t_hist[(size_t)n * D + j] = tcol[j] >= 0 ? tsign * x[tcol[j]] : fl[j] * amp;
}

// r = b - A x, warp per row (FP64 residual of the refinement step).
__global__ void __launch_bounds__(256) k_mrt_residual(const double* __restrict__ A, int N,
                                                      const double* __restrict__ x,
                                                      const double* __restrict__ b,
                                                      double* __restrict__ r) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= N) return;
    const double* row = A + (size_t)warp * N;
    double acc = 0;
    for (int j = lane; j < N; j += 32) acc += row[j] * x[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) r[warp] = b[warp] - acc;
}

}  // namespace

struct tdbem_mrt {
    tdbem_ctx* reg[2] = {nullptr, nullptr};
    int L = 10, refine = 1;
    int N = 0, NG = 0, NZ = 0, D[2] = {0, 0}, NI[2] = {0, 0}, row_lo[2] = {0, 0};
    double tsign[2] = {1.0, -1.0};
    std::vector<int> ucol[2], tcol[2];
    std::vector<double> fl[2];   // FBC value of each interior dof (0 elsewhere)
    std::vector<double> amp;     // amplitude at k dt; empty: the reference's pulse
    int assembled = -1;          // min(L, numstep) of the last assembly
    int lev[2] = {0, 0};         // region levels usable by the convolution
    cudaStream_t stream = nullptr;
    // device
    int* d_ucol[2] = {nullptr, nullptr};
    int* d_tcol[2] = {nullptr, nullptr};
    double* d_fl[2] = {nullptr, nullptr};
    double* d_A = nullptr;       // H_DB^0
    double* d_Ainv = nullptr;
    int* d_perm = nullptr;
    int* d_status = nullptr;
    double* d_scratch = nullptr;
    double* d_Wt[2] = {nullptr, nullptr};
    double* d_Wu[2] = {nullptr, nullptr};
    double* d_partial[2] = {nullptr, nullptr};
    int nch_cap[2] = {0, 0};
    double *d_rhs = nullptr, *d_x = nullptr, *d_r = nullptr, *d_dx = nullptr;
    double* d_X = nullptr;       // (steps + 1) x N
    double* d_u[2] = {nullptr, nullptr};
    double* d_t[2] = {nullptr, nullptr};
    int hist_cap = -1;
    int step_numstep = 0;        // stepwise path: tdbem_mrt_begin's step count
    bool step_ready = false;     // stepwise path: H_DB^0 inverted
    long long launches = 0;

    double amplitude(int n) const {
        if (amp.empty()) return reference_pulse(n, reg[0]->dt);
        return n < (int)amp.size() ? amp[n] : 0.0;
    }
};

namespace {

void free_mrt(tdbem_mrt* m) {
    for (int r = 0; r < 2; r++) {
        release(m->d_ucol[r]);
        release(m->d_tcol[r]);
        release(m->d_fl[r]);
        release(m->d_Wt[r]);
        release(m->d_Wu[r]);
        release(m->d_partial[r]);
        release(m->d_u[r]);
        release(m->d_t[r]);
    }
    release(m->d_A);
    release(m->d_Ainv);
    release(m->d_perm);
    release(m->d_status);
    release(m->d_scratch);
    release(m->d_rhs);
    release(m->d_x);
    release(m->d_r);
    release(m->d_dx);
    release(m->d_X);
}

// The node-by-node interface match of InterfaceIndexing (SolverMRT.cpp:458-494):
// region 2's interface node i -> index of the region-1 interface node within
// 1e-10 (the first such).  -1 if none.
std::vector<int> match_interface(const tdbem_ctx* c1, const tdbem_ctx* c2, const int* if1,
                                 const int* if2, int nz) {
    std::vector<int> match(nz, -1);
    const double* x1 = c1->h_coords.data();
    const double* x2 = c2->h_coords.data();
    for (int ni = 0; ni < nz; ni++) {
        const double* p = x2 + 3 * (size_t)if2[ni];
        for (int nj = 0; nj < nz; nj++) {
            const double* q = x1 + 3 * (size_t)if1[nj];
            const double r = std::sqrt((q[0] - p[0]) * (q[0] - p[0]) + (q[1] - p[1]) * (q[1] - p[1]) +
                                       (q[2] - p[2]) * (q[2] - p[2]));
            if (r < 1e-10) {
                match[ni] = nj;
                break;
            }
        }
    }
    return match;
}

// H_DB^0 from the regions' level 0, its inverse, and the convolution buffers for
// levels up to min(steps, MaxStep of the region).
int prepare_solve(tdbem_mrt* m, int steps) {
    cudaStream_t s = m->stream;
    const size_t NN = (size_t)m->N * m->N;
    MRT_TRY(cudaMemsetAsync(m->d_A, 0, sizeof(double) * NN, s));
    for (int r = 0; r < 2; r++) {
        const tdbem_ctx* c = m->reg[r];
        const size_t DD = (size_t)c->D * c->D;
        k_mrt_lhs<<<(unsigned)((DD + 255) / 256), 256, 0, s>>>(
            c->d_H, c->d_G, c->D, m->d_ucol[r], m->d_tcol[r], m->tsign[r], m->row_lo[r], m->N,
            m->d_A);
        MRT_TRY(cudaGetLastError());
        m->launches++;
        // levels past the region's MaxStep are exactly zero: the convolution stops there
        m->lev[r] = std::min(steps, c->M);
        const int nch = conv_chunks(m->lev[r], c->D);
        if (nch > m->nch_cap[r]) {
            release(m->d_partial[r]);
            MRT_TRY(alloc(&m->d_partial[r], (size_t)nch * c->D));
            m->nch_cap[r] = nch;
        }
        release(m->d_Wt[r]);
        release(m->d_Wu[r]);
        MRT_TRY(alloc(&m->d_Wt[r], (size_t)(m->lev[r] + 1) * c->D));
        MRT_TRY(alloc(&m->d_Wu[r], (size_t)(m->lev[r] + 1) * c->D));
    }
    MRT_TRY(cudaMemcpyAsync(m->d_Ainv, m->d_A, sizeof(double) * NN, cudaMemcpyDeviceToDevice, s));
    bool singular = false;
    MRT_TRY(invert_f64(m->d_Ainv, m->N, m->d_perm, m->d_status, m->d_scratch, &m->launches,
                       &singular, s));
    MRT_TRY(cudaStreamSynchronize(s));
    if (singular) return mfail(TDBEM_ERR_SINGULAR, "zero pivot in the combined H^0");
    return TDBEM_OK;
}

// Histories for numstep steps, row 0 (the initial state) zeroed.
int ensure_history(tdbem_mrt* m, int numstep) {
    cudaStream_t s = m->stream;
    const int N = m->N;
    if (numstep > m->hist_cap) {
        release(m->d_X);
        for (int r = 0; r < 2; r++) {
            release(m->d_u[r]);
            release(m->d_t[r]);
        }
        m->hist_cap = -1;
        MRT_TRY(alloc(&m->d_X, (size_t)(numstep + 1) * N));
        for (int r = 0; r < 2; r++) {
            MRT_TRY(alloc(&m->d_u[r], (size_t)(numstep + 1) * m->D[r]));
            MRT_TRY(alloc(&m->d_t[r], (size_t)(numstep + 1) * m->D[r]));
        }
        m->hist_cap = numstep;
    }
    MRT_TRY(cudaMemsetAsync(m->d_X, 0, sizeof(double) * N, s));
    for (int r = 0; r < 2; r++) {
        MRT_TRY(cudaMemsetAsync(m->d_u[r], 0, sizeof(double) * m->D[r], s));
        MRT_TRY(cudaMemsetAsync(m->d_t[r], 0, sizeof(double) * m->D[r], s));
    }
    return TDBEM_OK;
}

// One step of Solve_Direct: the regions' history sums into the two row blocks
// of the right-hand side, x = (H_DB^0)^-1 rhs with FP64 refinement, the regions'
// states of step n.
int mrt_step(tdbem_mrt* m, int n) {
    cudaStream_t s = m->stream;
    const int N = m->N;
    const double amp = m->amplitude(n);
    for (int r = 0; r < 2; r++) {
        const tdbem_ctx* c = m->reg[r];
        const int D = c->D;
        const int L = std::min(n, m->lev[r]);
        const size_t nw = (size_t)(L + 1) * D;
        k_mrt_w<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(m->d_u[r], m->d_t[r], m->d_fl[r], D,
                                                             n, L, amp, m->d_Wt[r], m->d_Wu[r]);
        MRT_TRY(cudaGetLastError());
        const MarchDev md{D, c->M, c->d_G, c->d_H, nullptr, nullptr};
        const int nch = conv_chunks(L, D);
        MRT_TRY(launch_conv(md, L, m->d_Wt[r], m->d_Wu[r], m->d_partial[r], nch, s));
        MRT_TRY(launch_reduce_partial(m->d_partial[r], nch, D, m->d_rhs + m->row_lo[r], s));
        m->launches += 3;
    }
    MRT_TRY(launch_gemv(m->d_Ainv, N, m->d_rhs, m->d_x, s));
    m->launches++;
    for (int it = 0; it < m->refine; it++) {
        k_mrt_residual<<<(N * 32 + 255) / 256, 256, 0, s>>>(m->d_A, N, m->d_x, m->d_rhs, m->d_r);
        MRT_TRY(cudaGetLastError());
        MRT_TRY(launch_gemv(m->d_Ainv, N, m->d_r, m->d_dx, s));
        MRT_TRY(launch_add_inplace(m->d_x, m->d_dx, N, s));
        m->launches += 3;
    }
    MRT_TRY(cudaMemcpyAsync(m->d_X + (size_t)n * N, m->d_x, sizeof(double) * N,
                            cudaMemcpyDeviceToDevice, s));
    for (int r = 0; r < 2; r++) {
        k_mrt_state<<<(m->D[r] + 255) / 256, 256, 0, s>>>(m->d_x, m->d_ucol[r], m->d_tcol[r],
                                                          m->tsign[r], m->d_fl[r], amp, m->D[r],
                                                          n, m->d_u[r], m->d_t[r]);
        MRT_TRY(cudaGetLastError());
        m->launches++;
    }
    return TDBEM_OK;
}

// Rows [row0, row0 + rows) of the histories to the host (null outputs skipped).
int copy_out(tdbem_mrt* m, int row0, int rows, double* x, double* u1, double* t1, double* u2,
             double* t2) {
    cudaStream_t s = m->stream;
    double* outs[5] = {x, u1, t1, u2, t2};
    const double* srcs[5] = {m->d_X, m->d_u[0], m->d_t[0], m->d_u[1], m->d_t[1]};
    const int widths[5] = {m->N, m->D[0], m->D[0], m->D[1], m->D[1]};
    for (int k = 0; k < 5; k++)
        if (outs[k])
            MRT_TRY(cudaMemcpyAsync(outs[k], srcs[k] + (size_t)row0 * widths[k],
                                    sizeof(double) * (size_t)rows * widths[k],
                                    cudaMemcpyDeviceToHost, s));
    MRT_TRY(cudaStreamSynchronize(s));
    return TDBEM_OK;
}

}  // namespace

extern "C" {

int tdbem_mrt_create(tdbem_ctx* region1, tdbem_ctx* region2, const int* iface1,
                     const int* iface2, int n_iface, int max_step, tdbem_mrt** out) {
    if (!out) return mfail(TDBEM_ERR_ARG, "out is null");
    *out = nullptr;
    if (!region1 || !region2 || region1 == region2)
        return mfail(TDBEM_ERR_ARG, "two distinct region contexts are needed");
    if (n_iface < 0 || (n_iface && (!iface1 || !iface2)))
        return mfail(TDBEM_ERR_ARG, "invalid interface lists");
    if (max_step < 0) return mfail(TDBEM_ERR_ARG, "max_step must be >= 0");
    if (region1->dt != region2->dt)
        return mfail(TDBEM_ERR_ARG, "the regions' time steps differ (%g, %g)", region1->dt,
                     region2->dt);
    if (region1->device != region2->device)
        return mfail(TDBEM_ERR_ARG, "the regions' contexts are on different devices");
    tdbem_ctx* c[2] = {region1, region2};
    const int* ifl[2] = {iface1, iface2};
    std::vector<char> on_if[2];
    for (int r = 0; r < 2; r++) {
        on_if[r].assign(c[r]->nnd, 0);
        for (int i = 0; i < n_iface; i++) {
            const int nd = ifl[r][i];
            if (nd < 0 || nd >= c[r]->nnd)
                return mfail(TDBEM_ERR_ARG, "interface node %d of region %d out of range", nd,
                             r + 1);
            if (on_if[r][nd])
                return mfail(TDBEM_ERR_ARG, "interface node %d of region %d listed twice", nd,
                             r + 1);
            on_if[r][nd] = 1;
        }
    }
    const std::vector<int> match = match_interface(c[0], c[1], iface1, iface2, n_iface);
    std::vector<char> taken(n_iface, 0);
    for (int i = 0; i < n_iface; i++) {
        if (match[i] < 0)
            return mfail(TDBEM_ERR_ARG,
                         "interface mismatch: node %d of region 2 has no region-1 partner",
                         iface2[i]);
        if (taken[match[i]])
            return mfail(TDBEM_ERR_ARG, "interface mismatch: two region-2 nodes on node %d",
                         iface1[match[i]]);
        taken[match[i]] = 1;
    }
    tdbem_mrt* m = new (std::nothrow) tdbem_mrt;
    if (!m) return mfail(TDBEM_ERR_NOMEM, "host allocation failed");
    m->reg[0] = region1;
    m->reg[1] = region2;
    m->L = max_step;
    m->stream = region1->stream;
    m->NZ = 3 * n_iface;
    for (int r = 0; r < 2; r++) {
        m->D[r] = c[r]->D;
        m->NI[r] = m->D[r] - m->NZ;
    }
    m->N = m->D[0] + m->D[1];
    m->NG = m->NI[0] + m->NI[1];
    m->row_lo[1] = m->D[0];
    // columns: interior dofs of region r in ascending node order, then the interface
    // displacements (region 1's order) and tractions
    const int base_z = m->NI[0] + m->NI[1], base_t = base_z + m->NZ;
    int next_int[2] = {0, m->NI[0]};
    for (int r = 0; r < 2; r++) {
        m->ucol[r].assign(m->D[r], -1);
        m->tcol[r].assign(m->D[r], -1);
        for (int nd = 0; nd < c[r]->nnd; nd++)
            if (!on_if[r][nd])
                for (int d = 0; d < 3; d++) m->ucol[r][3 * nd + d] = next_int[r]++;
        for (int i = 0; i < n_iface; i++) {
            const int k = r == 0 ? i : match[i];  // region-1 interface index
            for (int d = 0; d < 3; d++) {
                m->ucol[r][3 * ifl[r][i] + d] = base_z + 3 * k + d;
                m->tcol[r][3 * ifl[r][i] + d] = base_t + 3 * k + d;
            }
        }
        // SetLoad (SolverMRT.cpp:889-958): FBC values, the last entry of a dof
        // winning, kept at interior dofs only
        m->fl[r].assign(m->D[r], 0.0);
        for (size_t i = 0; i < c[r]->fbc.size(); i++) m->fl[r][c[r]->fbc[i]] = c[r]->fbc_v[i];
        for (int j = 0; j < m->D[r]; j++)
            if (m->tcol[r][j] >= 0) m->fl[r][j] = 0.0;
    }
    auto fail_free = [&](cudaError_t e) {
        const int code = mfail(e == cudaErrorMemoryAllocation ? TDBEM_ERR_NOMEM : TDBEM_ERR_CUDA,
                               "tdbem_mrt_create: %s", cudaGetErrorString(e));
        free_mrt(m);
        delete m;
        return code;
    };
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < 2 && e == cudaSuccess; r++) {
        if (e == cudaSuccess) e = alloc(&m->d_ucol[r], m->D[r]);
        if (e == cudaSuccess) e = alloc(&m->d_tcol[r], m->D[r]);
        if (e == cudaSuccess) e = alloc(&m->d_fl[r], m->D[r]);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m->d_ucol[r], m->ucol[r].data(), sizeof(int) * m->D[r],
                                cudaMemcpyHostToDevice, m->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m->d_tcol[r], m->tcol[r].data(), sizeof(int) * m->D[r],
                                cudaMemcpyHostToDevice, m->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(m->d_fl[r], m->fl[r].data(), sizeof(double) * m->D[r],
                                cudaMemcpyHostToDevice, m->stream);
    }
    const size_t NN = (size_t)m->N * m->N;
    if (e == cudaSuccess) e = alloc(&m->d_A, NN);
    if (e == cudaSuccess) e = alloc(&m->d_Ainv, NN);
    if (e == cudaSuccess) e = alloc(&m->d_perm, m->N + 2 * kMaxPivotBlocks);
    if (e == cudaSuccess) e = alloc(&m->d_status, 1);
    if (e == cudaSuccess) e = alloc(&m->d_scratch, inverse_scratch_elems(m->N));
    if (e == cudaSuccess) e = alloc(&m->d_rhs, m->N);
    if (e == cudaSuccess) e = alloc(&m->d_x, m->N);
    if (e == cudaSuccess) e = alloc(&m->d_r, m->N);
    if (e == cudaSuccess) e = alloc(&m->d_dx, m->N);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) return fail_free(e);
    *out = m;
    return TDBEM_OK;
}

int tdbem_mrt_destroy(tdbem_mrt* m) {
    if (!m) return TDBEM_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    free_mrt(m);
    delete m;
    return TDBEM_OK;
}

int tdbem_mrt_size(const tdbem_mrt* m, int* N, int* NG) {
    if (!m || !N || !NG) return mfail(TDBEM_ERR_ARG, "null argument");
    *N = m->N;
    *NG = m->NG;
    return TDBEM_OK;
}

int tdbem_mrt_columns(const tdbem_mrt* m, int region, int* ucol, int* tcol) {
    if (!m || !ucol || !tcol || (region != 1 && region != 2))
        return mfail(TDBEM_ERR_ARG, "invalid argument");
    const int r = region - 1;
    std::copy(m->ucol[r].begin(), m->ucol[r].end(), ucol);
    std::copy(m->tcol[r].begin(), m->tcol[r].end(), tcol);
    return TDBEM_OK;
}

int tdbem_mrt_set_load_history(tdbem_mrt* m, const double* amp, int n) {
    if (!m || n < 0 || (n && !amp)) return mfail(TDBEM_ERR_ARG, "invalid load history");
    m->amp.assign(amp, amp + n);
    return TDBEM_OK;
}

int tdbem_mrt_set_refine(tdbem_mrt* m, int refine) {
    if (!m || refine < 0 || refine > 8) return mfail(TDBEM_ERR_ARG, "refine must be in 0..8");
    m->refine = refine;
    return TDBEM_OK;
}

int tdbem_mrt_assemble(tdbem_mrt* m, int numstep) {
    if (!m) return mfail(TDBEM_ERR_ARG, "null solver");
    if (numstep < 1) return mfail(TDBEM_ERR_ARG, "numstep must be >= 1");
    // G_H_Driver runs for the steps 1..min(max_step, numstep) of the loop (the
    // reference's driver pattern, main.cpp:89-126); both regions side by side
    const int steps = std::max(1, std::min(m->L, numstep));
    int rc[2] = {TDBEM_OK, TDBEM_OK};
    std::string msg[2];
    std::thread t2([&] {
        cudaSetDevice(m->reg[1]->device);
        rc[1] = tdbem_assemble_levels(m->reg[1], steps, TDBEM_FP64);
        if (rc[1] != TDBEM_OK) msg[1] = tdbem_last_error();
    });
    rc[0] = tdbem_assemble_levels(m->reg[0], steps, TDBEM_FP64);
    if (rc[0] != TDBEM_OK) msg[0] = tdbem_last_error();
    t2.join();
    for (int r = 0; r < 2; r++)
        if (rc[r] != TDBEM_OK) return mfail(rc[r], "region %d: %s", r + 1, msg[r].c_str());
    MRT_TRY(cudaStreamSynchronize(m->reg[1]->stream));
    const int rc2 = prepare_solve(m, steps);
    if (rc2 != TDBEM_OK) return rc2;
    m->assembled = steps;
    return TDBEM_OK;
}

int tdbem_mrt_march(tdbem_mrt* m, int numstep, double* x_hist, double* u1_hist,
                    double* t1_hist, double* u2_hist, double* t2_hist) {
    if (!m) return mfail(TDBEM_ERR_ARG, "null solver");
    if (numstep < 1) return mfail(TDBEM_ERR_ARG, "numstep must be >= 1");
    if (m->assembled < 0) return mfail(TDBEM_ERR_STATE, "levels not assembled");
    // levels f >= numstep only ever meet the zero initial state
    if (std::min(m->L, numstep) > m->assembled)
        return mfail(TDBEM_ERR_STATE, "levels assembled for %d steps, %d needed", m->assembled,
                     std::min(m->L, numstep));
    int rc = ensure_history(m, numstep);
    for (int n = 1; rc == TDBEM_OK && n <= numstep; n++) rc = mrt_step(m, n);
    if (rc != TDBEM_OK) return rc;
    return copy_out(m, 0, numstep + 1, x_hist, u1_hist, t1_hist, u2_hist, t2_hist);
}

int tdbem_mrt_begin(tdbem_mrt* m, int numstep) {
    if (!m) return mfail(TDBEM_ERR_ARG, "null solver");
    if (numstep < 1) return mfail(TDBEM_ERR_ARG, "numstep must be >= 1");
    const int rc = ensure_history(m, numstep);
    if (rc != TDBEM_OK) return rc;
    m->step_numstep = numstep;
    m->step_ready = false;
    m->assembled = -1;  // the levels now come from tdbem_update_gh_linear
    return TDBEM_OK;
}

int tdbem_mrt_step(tdbem_mrt* m, int curr_step, double* x, double* u1, double* t1, double* u2,
                   double* t2) {
    if (!m) return mfail(TDBEM_ERR_ARG, "null solver");
    if (m->step_numstep < 1) return mfail(TDBEM_ERR_STATE, "tdbem_mrt_begin has not run");
    if (curr_step < 1 || curr_step > m->step_numstep)
        return mfail(TDBEM_ERR_ARG, "step %d outside 1..%d", curr_step, m->step_numstep);
    for (int r = 0; r < 2; r++)
        if (m->reg[r]->level_precision != TDBEM_FP64 || m->reg[r]->levels_last < 1)
            return mfail(TDBEM_ERR_STATE, "region %d has no level 0 (UpdateGHLinear of step 1)",
                         r + 1);
    if (!m->step_ready) {
        // H_DB^0 is final once step 1 is placed (level 0 holds only J(1)); the
        // convolution reads levels up to the loop's last placed step
        const int rc = prepare_solve(m, std::max(1, std::min(m->L, m->step_numstep)));
        if (rc != TDBEM_OK) return rc;
        m->step_ready = true;
    }
    const int rc = mrt_step(m, curr_step);
    if (rc != TDBEM_OK) return rc;
    return copy_out(m, curr_step, 1, x, u1, t1, u2, t2);
}

}  // extern "C"
