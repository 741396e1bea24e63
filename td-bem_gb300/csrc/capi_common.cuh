// Host-side helpers shared by the translation units of the C ABI (capi*.cu):
// error reporting, device allocation, profiling events, the colour-chunked
// assembly launches, the graph-replayed march loop and the march engines' set-up.
// Internal to the library; not part of include/tdbem.h.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "tdbem_internal.cuh"

namespace tdbem {

// Device buffers of the library (devmem.cu): freed blocks are kept and handed to the
// next allocation of the same rounded size on the same device.
cudaError_t mem_alloc(void** p, size_t bytes);
void mem_free(void* p);
size_t mem_release(int device);       // the kept blocks of a device (all: -1); bytes
size_t mem_cached_bytes(int device);  // bytes kept (all devices: -1)

namespace capi {

// Records the message of a failed call (tdbem_last_error) and returns code.
int fail(int code, const char* fmt, ...);

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            const int code_ = (e_ == cudaErrorMemoryAllocation) ? TDBEM_ERR_NOMEM        \
                                                                : TDBEM_ERR_CUDA;        \
            return fail(code_, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                       \
        }                                                                                \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return mem_alloc(reinterpret_cast<void**>(p), sizeof(T) * count);
}

template <typename T>
void dfree(T*& p) {
    if (p) mem_free(p);
    p = nullptr;
}

bool gauss_table(int nq, std::vector<double>& x, std::vector<double>& w);
int compute_max_step(const std::vector<double>& x, int nnd, double E, double nu, double rho,
                     double dt);
void color_elements(const std::vector<int>& ien, int nel, int ennd, int nnd,
                    std::vector<int>& order, std::vector<int>& start);
void free_levels(tdbem_ctx* c);
void free_batch(tdbem_ctx* c);
void free_march(tdbem_ctx* c);

// Algorithmic FP64 operations of one (item, Gauss point) of the level quadrature
// with both the I and the J part (FMA = 2): geometry 22, four I-part and four
// J-part wave integrals with their differences 150, kernel scalars 37, the two
// 3x3 kernels 65, accumulation into the 4 node blocks 124.
constexpr double kFlopsPerItemPoint = 398.0;
// The FP32 far-field form (tau variables): geometry 20, wave polynomials and
// differences 176, scalars 40, kernels 65, accumulation 124.
constexpr double kFlopsPerItemPointF32 = 425.0;
// A settled job's point (the quasi-static kernel): geometry 18, scalars 8, kernels
// 51, accumulation 124; a settled level: a scaled add per entry of the 4 node blocks.
constexpr double kFlopsSettledPoint = 201.0;
constexpr double kFlopsSettledLevel = 144.0;

int prof_begin_on(tdbem_ctx* c, int cls, cudaStream_t s);
int prof_begin(tdbem_ctx* c, int cls);
void prof_end_on(tdbem_ctx* c, int idx, double bytes, double flops, cudaStream_t s);
void prof_end(tdbem_ctx* c, int idx, double bytes, double flops);
void prof_flush(tdbem_ctx* c);
int assemble_color(tdbem_ctx* c, int color, int node_lo, int nnodes, int mode, int level_last,
                   int level_cap, int step_n, int select, const AsmOut& out);

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start(cudaStream_t s) { cudaEventRecord(a, s); }
    double stop_ms(cudaStream_t s) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
};


// Runs a marching loop (kernel launches only, no host synchronisation) through a
// CUDA graph: captured on the context's stream the first time and whenever a
// captured value changes (kind of loop, step count, block size, refinement
// sweeps, weights, load history, buffer addresses), replayed otherwise.  With
// profiling on (per-launch events) or graphs off the loop runs directly.
template <typename F>
int run_march_loop(tdbem_ctx* c, int kind, int numstep, const std::vector<const void*>& ptrs,
                   F loop) {
    if (c->prof || !c->use_graphs) return loop();
    MarchGraph& g = c->graph;
    cudaStream_t s = c->stream;
    const bool same = g.exec && g.kind == kind && g.numstep == numstep && g.nb == c->nb_eff &&
                      g.refine == c->n_refine && g.a1 == c->a1 && g.a2 == c->a2 &&
                      g.amp == c->amp && g.ptrs == ptrs && g.wait_ns == c->tc_wait_ns &&
                      g.step2_sweeps == c->step2_sweeps;
    if (!same) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        const long long l0 = c->launches;
        CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = loop();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (rc != TDBEM_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CUDA_TRY(e);
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        CUDA_TRY(ei);
        g.launches = c->launches - l0;
        c->launches = l0;
        g.kind = kind;
        g.numstep = numstep;
        g.nb = c->nb_eff;
        g.refine = c->n_refine;
        g.a1 = c->a1;
        g.a2 = c->a2;
        g.amp = c->amp;
        g.ptrs = ptrs;
        g.wait_ns = c->tc_wait_ns;
        g.step2_sweeps = c->step2_sweeps;
    }
    CUDA_TRY(cudaGraphLaunch(g.exec, s));
    c->launches += g.launches;
    return TDBEM_OK;
}

// ---- march engines (capi_march.cu)

int mixed_ninv(int numstep, const double lhs_c[2][2]);
bool inverses_current(const tdbem_ctx* c, int ninv);
int prepare_inverses(tdbem_ctx* c, int ninv);

struct InvResult {
    cudaError_t e[2] = {cudaSuccess, cudaSuccess};
    bool singular[2] = {false, false};
    long long launches[2] = {0, 0};
    InverseReport report[2];
    int step2_sweeps = 0;  // > 0: step 2 by Richardson sweeps with the later inverse
};

void run_inverses(tdbem_ctx* c, int ninv, const double lhs_c[2][2], cudaStream_t s0,
                  cudaStream_t s1, InvResult& r);
int finish_inverses(tdbem_ctx* c, int ninv, const InvResult& r);
int mixed_inverses(tdbem_ctx* c, int numstep, const double lhs_c[2][2]);
int ensure_merged_levels(tdbem_ctx* c);
// Profiling: the live tiles of every slab from the occupancy map (one copy to the
// host), and the merged-plane bytes a convolution over slabs [lev0, lev0 + nlev) reads.
int count_live_tiles(tdbem_ctx* c);
double conv_plane_bytes(const tdbem_ctx* c, int lev0, int nlev);
int march_mixed(tdbem_ctx* c, int numstep, const double lhs_c[2][2]);
int upload_bc(tdbem_ctx* c);
int fp64_inverse(tdbem_ctx* c, int v, const double lhs_c[2][2]);
int fp64_step(tdbem_ctx* c, int st, const double lhs_c[2][2]);
int march_fp64(tdbem_ctx* c, int numstep, const double lhs_c[2][2], double* u_hist,
               double* t_hist);
int ensure_fp64_store(tdbem_ctx* c);

// ---- grouped marching (capi_group.cu)

// Per-mesh preparation of a grouped march of ns steps: boundary conditions, zeroed
// histories, the LHS inverses (FP64, or the mixed form's FP32 pair), the load
// history and the FP32 block scratch on the device (owned by the context), and the
// mesh's GroupMarch entry with off = 0 (the list offsets are group_layout's).
// Synchronises the context's stream.
int group_prepare(tdbem_ctx* c, int ns, bool mixed, GroupMarch& g);
// Row / W / quad / old-W list offsets of the meshes in order, and the totals.
void group_layout(GroupMarch* gm, int n, unsigned* nrows, unsigned* nw, unsigned* nquads,
                  unsigned* nwold);

// Error of the tcgen05 convolution launches since d_tc_err was cleared (the stream
// synchronised by the caller's copy): TDBEM_OK, or TDBEM_ERR_CUDA naming the wait
// that ran out and the CTAs still holding TMEM.
int tc_status(const int err[2], const char* what);

}  // namespace capi
}  // namespace tdbem
