// C ABI of tdbem-gb300 (include/tdbem.h): context lifetime, element colouring,
// and the host-side sequencing of the assembly and marching kernels.
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

using namespace tdbem;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

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
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * count);
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Gauss tables of ShapeFunctionT::SetNQ (ShapeFunctionT.cpp:71-169); the
// 20-point abscissae keep the reference's unsigned entry 19 (ShapeFunctionT.cpp:121).
bool gauss_table(int nq, std::vector<double>& x, std::vector<double>& w) {
    static const double x6[] = {0.6612093864662645, -0.6612093864662645, -0.2386191860831969,
                                0.2386191860831969, -0.9324695142031521, 0.9324695142031521};
    static const double w6[] = {0.3607615730481386, 0.3607615730481386, 0.4679139345726910,
                                0.4679139345726910, 0.1713244923791704, 0.1713244923791704};
    static const double x10[] = {-0.148874339, 0.148874339, -0.433395394, 0.433395394,
                                 -0.679409568, 0.679409568, -0.865063367, 0.865063367,
                                 -0.973906529, 0.973906529};
    static const double w10[] = {0.295524225, 0.295524225, 0.269266719, 0.269266719,
                                 0.219086363, 0.219086363, 0.149451349, 0.149451349,
                                 0.066671344, 0.066671344};
    static const double x20[] = {-0.076526521, 0.076526521, -0.227785851, 0.227785851,
                                 -0.373706089, 0.373706089, -0.510867002, 0.510867002,
                                 -0.636053681, 0.636053681, -0.746331906, 0.746331906,
                                 -0.839116972, 0.839116972, -0.912234428, 0.912234428,
                                 -0.963971927, 0.963971927, 0.993128599, 0.993128599};
    static const double w20[] = {0.152753387, 0.152753387, 0.149172986, 0.149172986,
                                 0.142096109, 0.142096109, 0.131688638, 0.131688638,
                                 0.118194532, 0.118194532, 0.10193012,  0.10193012,
                                 0.083276742, 0.083276742, 0.062672048, 0.062672048,
                                 0.04060143,  0.04060143,  0.017614007, 0.017614007};
    static const double x40[] = {
        -0.0387724175060508, 0.0387724175060508, -0.1160840706752552, 0.1160840706752552,
        -0.1926975807013711, 0.1926975807013711, -0.2681521850072537, 0.2681521850072537,
        -0.3419940908257585, 0.3419940908257585, -0.4137792043716050, 0.4137792043716050,
        -0.4830758016861787, 0.4830758016861787, -0.5494671250951282, 0.5494671250951282,
        -0.6125538896679802, 0.6125538896679802, -0.6719566846141796, 0.6719566846141796,
        -0.7273182551899271, 0.7273182551899271, -0.7783056514265194, 0.7783056514265194,
        -0.8246122308333117, 0.8246122308333117, -0.8659595032122595, 0.8659595032122595,
        -0.9020988069688743, 0.9020988069688743, -0.9328128082786765, 0.9328128082786765,
        -0.9579168192137917, 0.9579168192137917, -0.9772599499837743, 0.9772599499837743,
        -0.9907262386994570, 0.9907262386994570, -0.9982377097105593, 0.9982377097105593};
    static const double w40[] = {
        0.0775059479784248, 0.0775059479784248, 0.0770398181642480, 0.0770398181642480,
        0.0761103619006262, 0.0761103619006262, 0.0747231690579683, 0.0747231690579683,
        0.0728865823958041, 0.0728865823958041, 0.0706116473912868, 0.0706116473912868,
        0.0679120458152339, 0.0679120458152339, 0.0648040134566010, 0.0648040134566010,
        0.0613062424929289, 0.0613062424929289, 0.0574397690993916, 0.0574397690993916,
        0.0532278469839368, 0.0532278469839368, 0.0486958076350722, 0.0486958076350722,
        0.0438709081856733, 0.0438709081856733, 0.0387821679744720, 0.0387821679744720,
        0.0334601952825478, 0.0334601952825478, 0.0279370069800234, 0.0279370069800234,
        0.0222458491941670, 0.0222458491941670, 0.0164210583819079, 0.0164210583819079,
        0.0104982845311528, 0.0104982845311528, 0.0045212770985332, 0.0045212770985332};
    const double *px, *pw;
    switch (nq) {
    case 6: px = x6; pw = w6; break;
    case 10: px = x10; pw = w10; break;
    case 20: px = x20; pw = w20; break;
    case 40: px = x40; pw = w40; break;
    default: return false;
    }
    x.assign(px, px + nq);
    w.assign(pw, pw + nq);
    return true;
}

// SolverT::ComputeMaxStep (SolverT.cpp:211-250), same arithmetic.
int compute_max_step(const std::vector<double>& x, int nnd, double E, double nu, double rho,
                     double dt) {
    const double Mu = E / (2.0 * (1.0 + nu));
    const double Cs = std::sqrt(Mu / rho);
    double max_dis = 0;
    for (int i = 0; i < nnd - 1; i++)
        for (int j = i + 1; j < nnd; j++) {
            double t = 0;
            for (int d = 0; d < 3; d++) {
                const double v = x[i * 3 + d] - x[j * 3 + d];
                t += v * v;
            }
            t = std::sqrt(t);
            if (t > max_dis) max_dis = t;
        }
    return (int)(std::ceil(max_dis / (Cs * dt)) + 1);
}

// Greedy colouring: no two elements of one colour share a node.
void color_elements(const std::vector<int>& ien, int nel, int ennd, int nnd,
                    std::vector<int>& order, std::vector<int>& start) {
    std::vector<std::vector<int>> node_elems(nnd);
    for (int e = 0; e < nel; e++)
        for (int a = 0; a < ennd; a++) node_elems[ien[e * ennd + a]].push_back(e);
    std::vector<int> color(nel, -1);
    int ncolor = 0;
    std::vector<int> used;
    for (int e = 0; e < nel; e++) {
        used.assign(ncolor + 1, 0);
        for (int a = 0; a < ennd; a++)
            for (int o : node_elems[ien[e * ennd + a]])
                if (color[o] >= 0) used[color[o]] = 1;
        int c = 0;
        while (c < ncolor && used[c]) c++;
        color[e] = c;
        if (c == ncolor) ncolor++;
    }
    start.assign(ncolor + 1, 0);
    for (int e = 0; e < nel; e++) start[color[e] + 1]++;
    for (int c = 0; c < ncolor; c++) start[c + 1] += start[c];
    order.assign(nel, 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int e = 0; e < nel; e++) order[fill[color[e]]++] = e;
}

void free_levels(tdbem_ctx* c) {
    c->inv_valid = false;
    dfree(c->d_G);
    dfree(c->d_H);
    dfree(c->d_Gf);
    dfree(c->d_Hf);
    dfree(c->d_G01);
    dfree(c->d_H01);
    c->level_precision = -1;
    c->levels_last = 0;
    if (c->d_mtc_planes) cudaFree(c->d_mtc_planes);
    c->d_mtc_planes = nullptr;
    dfree(c->d_mtc_known);
    dfree(c->d_mtc_bc);
    c->mtc_planes_valid = false;
}

void free_batch(tdbem_ctx* c) {
    dfree(c->d_bu);
    dfree(c->d_bt);
    dfree(c->d_btrac);
    dfree(c->d_bamp);
    dfree(c->d_bWt);
    dfree(c->d_bWu);
    dfree(c->d_bpart);
    dfree(c->d_brhs);
    dfree(c->d_bx);
    dfree(c->d_br);
    c->bpart_cap = 0;
    c->batch_C = 0;
    c->batch_steps = -1;
    if (c->d_tc_W) cudaFree(c->d_tc_W);
    c->d_tc_W = nullptr;
    c->tc_W_bytes = 0;
    dfree(c->d_tc_err);
    dfree(c->d_bkt);
    dfree(c->d_bGK);
    dfree(c->d_bGL);
}

void free_march(tdbem_ctx* c) {
    dfree(c->d_u);
    dfree(c->d_t);
    // one LHS: slot 1 aliases slot 0 (dropped before slot 0 is freed)
    if (c->d_inv32[1] == c->d_inv32[0]) c->d_inv32[1] = nullptr;
    if (c->d_Hc64[1] == c->d_Hc64[0]) c->d_Hc64[1] = nullptr;
    for (int v = 0; v < 2; v++) {
        dfree(c->d_inv32[v]);
        dfree(c->d_Hc64[v]);
    }
    dfree(c->d_Wt_old);
    dfree(c->d_Wu_old);
    dfree(c->d_Yold);
    dfree(c->d_pmix);
    dfree(c->d_res);
    dfree(c->d_dx);
    if (c->d_mtc_W) cudaFree(c->d_mtc_W);
    c->d_mtc_W = nullptr;
    c->mtc_W_bytes = 0;
    c->mtc_maps_for[0] = c->mtc_maps_for[1] = nullptr;
    dfree(c->d_mtc_coef);
    c->mtc_coef_cap = 0;
    c->mtc_coef_key.clear();
    dfree(c->d_mtc_yk);
    c->mtc_yk_cap = 0;

    if (c->d_Ainv[1] == c->d_Ainv[0]) c->d_Ainv[1] = nullptr;
    dfree(c->d_Ainv[0]);
    dfree(c->d_Ainv[1]);
    c->hist_steps = -1;
    dfree(c->d_upd_tmp);
    c->upd_tmp_cap = 0;
    free_batch(c);
}

// Algorithmic FP64 operations of one (item, Gauss point) of the level quadrature
// with both the I and the J part (FMA = 2): geometry 22, four I-part and four
// J-part wave integrals with their differences 150, kernel scalars 37, the two
// 3x3 kernels 65, accumulation into the 4 node blocks 124.
constexpr double kFlopsPerItemPoint = 398.0;
// The FP32 far-field form (tau variables): geometry 20, wave polynomials and
// differences 176, scalars 40, kernels 65, accumulation 124.
constexpr double kFlopsPerItemPointF32 = 425.0;

int prof_begin_on(tdbem_ctx* c, int cls, cudaStream_t s) {
    if (!c->prof) return -1;
    tdbem_ctx::ProfEvent ev{cls, nullptr, nullptr, 0, 0};
    cudaEventCreate(&ev.a);
    cudaEventCreate(&ev.b);
    cudaEventRecord(ev.a, s);
    c->prof_pending.push_back(ev);
    return (int)c->prof_pending.size() - 1;
}

int prof_begin(tdbem_ctx* c, int cls) { return prof_begin_on(c, cls, c->stream); }

void prof_end_on(tdbem_ctx* c, int idx, double bytes, double flops, cudaStream_t s) {
    if (idx < 0) return;
    auto& ev = c->prof_pending[idx];
    cudaEventRecord(ev.b, s);
    ev.bytes = bytes;
    ev.flops = flops;
}

void prof_end(tdbem_ctx* c, int idx, double bytes, double flops) {
    prof_end_on(c, idx, bytes, flops, c->stream);
}

// Resolve pending event pairs (the stream must have been synchronised).
void prof_flush(tdbem_ctx* c) {
    for (auto& ev : c->prof_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ev.a, ev.b) == cudaSuccess) {
            c->prof_launches[ev.cls]++;
            c->prof_ms[ev.cls] += ms;
            c->prof_bytes[ev.cls] += ev.bytes;
            c->prof_flops[ev.cls] += ev.flops;
        }
        cudaEventDestroy(ev.a);
        cudaEventDestroy(ev.b);
    }
    c->prof_pending.clear();
    cudaGetLastError();
}

// Run the window / scan / item kernels of one colour over collocation nodes
// [node_lo, node_lo + nnodes), chunked so that item indices fit in 32 bits.
int assemble_color(tdbem_ctx* c, int color, int node_lo, int nnodes, int mode, int level_last,
                   int level_cap, int step_n, int select, const AsmOut& out) {
    const int e0 = c->color_start[color], ne = c->color_start[color + 1] - e0;
    if (ne == 0 || nnodes == 0) return TDBEM_OK;
    const int* elems = c->d_color_elems + e0;
    const long long per_node_items = (long long)ne * (mode == ASM_LEVELS ? level_last + 1 : 1);
    // item threads (one per item, two for an 8-node element) stay below 2^31
    const long long max_nodes_items =
        (1LL << (c->ennd == 8 ? 30 : 31)) / std::max(1LL, per_node_items);
    const long long max_nodes_pairs = (long long)c->pair_cap / ne;
    const int chunk = (int)std::max(1LL, std::min(max_nodes_items, max_nodes_pairs));
    for (int n0 = node_lo; n0 < node_lo + nnodes; n0 += chunk) {
        const int nn = std::min(chunk, node_lo + nnodes - n0);
        const unsigned npairs = (unsigned)((long long)nn * ne);
        const int pw = prof_begin(c, TDBEM_K_AUX);
        CUDA_TRY(launch_pair_window(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, nn, c->ph, mode,
                                    level_last, level_cap, step_n, select, c->d_pairs,
                                    c->d_counts, c->stream));
        CUDA_TRY(exclusive_scan(c->d_counts, c->d_offsets, npairs, c->d_scan_tmp,
                                c->scan_tmp_bytes, c->stream));
        prof_end(c, pw, 0, 0);
        c->launches += 3;  // window + the scan's init and scan kernels
        unsigned last[2];
        CUDA_TRY(cudaMemcpyAsync(&last[0], c->d_offsets + npairs - 1, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaMemcpyAsync(&last[1], c->d_counts + npairs - 1, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        const unsigned nitems = last[0] + last[1];
        const int pe = prof_begin(c, TDBEM_K_ASSEMBLE);
        CUDA_TRY(launch_assemble_items(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, c->nq,
                                       c->d_gx, c->d_gw, c->d_geom, c->ph, mode, level_last,
                                       step_n, c->d_pairs, c->d_offsets, npairs, nitems, out,
                                       c->stream));
        if (nitems) c->launches += (mode == ASM_STEP ? 2 : 1);
        const double pts = (double)c->nq * c->nq;
        const double items = (double)nitems * (mode == ASM_STEP ? 2.0 : 1.0);
        prof_end(c, pe, items * 4 * 45 * (out.G0f ? 4.0 : 8.0) * 2,
                 items * pts * kFlopsPerItemPoint * (mode == ASM_STEP ? 0.5 : 1.0));
    }
    return TDBEM_OK;
}

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
                      g.amp == c->amp && g.ptrs == ptrs;
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
    }
    CUDA_TRY(cudaGraphLaunch(g.exec, s));
    c->launches += g.launches;
    return TDBEM_OK;
}

// FP64 column-exchanged LHS and its FP32 inverse for each distinct LHS of the
// mixed form (step 2 and steps >= 3).  The inverses depend on alpha, the UBC dofs
// (the column exchange) and levels 0/1; they are kept with that key and reused
// while it holds (an assembly may have made them already, next to its far field).
int mixed_ninv(int numstep, const double lhs_c[2][2]) {
    const bool same = (lhs_c[1][0] == 1.0 && lhs_c[1][1] == 0.0);
    return (numstep >= 3 && !same) ? 2 : 1;
}

bool inverses_current(const tdbem_ctx* c, int ninv) {
    return c->inv_valid && c->inv_n == ninv && c->inv_a1 == c->a1 && c->inv_a2 == c->a2 &&
           c->inv_ubc == c->ubc;
}

int prepare_inverses(tdbem_ctx* c, int ninv) {
    const size_t DD = (size_t)c->D * c->D;
    for (int v = 0; v < 2; v++) {
        if (c->d_inv32[1] == c->d_inv32[0]) c->d_inv32[1] = nullptr;
        if (c->d_Hc64[1] == c->d_Hc64[0]) c->d_Hc64[1] = nullptr;
    }
    for (int v = 0; v < ninv; v++) {
        if (!c->d_Hc64[v]) CUDA_TRY(dalloc(&c->d_Hc64[v], DD));
        if (!c->d_inv32[v]) CUDA_TRY(dalloc(&c->d_inv32[v], DD));
    }
    if (!c->d_inv_scratch32) CUDA_TRY(dalloc(&c->d_inv_scratch32, inverse_scratch_elems(c->D)));
    for (cudaStream_t* st : {&c->stream2, &c->stream3})
        if (!*st) CUDA_TRY(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    if (!c->ev_fork) CUDA_TRY(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    if (!c->ev_fork2) CUDA_TRY(cudaEventCreateWithFlags(&c->ev_fork2, cudaEventDisableTiming));
    if (ninv == 2) {
        if (!c->d_inv_scratch32b)
            CUDA_TRY(dalloc(&c->d_inv_scratch32b, inverse_scratch_elems(c->D)));
        if (!c->d_perm2) CUDA_TRY(dalloc(&c->d_perm2, (size_t)c->D + 2 * kMaxPivotBlocks));
        if (!c->d_status2) CUDA_TRY(dalloc(&c->d_status2, 1));
    }
    return TDBEM_OK;
}

struct InvResult {
    cudaError_t e[2] = {cudaSuccess, cudaSuccess};
    bool singular[2] = {false, false};
    long long launches[2] = {0, 0};
};

// The inverses on streams s0 and s1 (s1 after s0's prior work): the second from a
// second host thread, as each inverse leaves most SMs idle during its pivot
// searches (one cluster of 16 CTAs) and the two overlap.  Touches no profiling
// state or shared counter, so it may run on a helper thread; returns after both
// streams have finished.
void run_inverses(tdbem_ctx* c, int ninv, const double lhs_c[2][2], cudaStream_t s0,
                  cudaStream_t s1, InvResult& r) {
    const int D = c->D;
    const size_t DD = (size_t)D * D;
    auto invert = [&](int v, cudaStream_t st, int* perm, int* status, float* scratch) {
        // a cuBLAS handle of the device's pool for the trailing updates (without one
        // the inverse uses its own update kernel)
        void* blas = blas_checkout(c->device);
        r.e[v] = launch_build_lhs(c->d_G01, c->d_H01, nullptr, nullptr, DD, D, lhs_c[v][0],
                                  lhs_c[v][1], c->d_is_ubc, c->d_Hc64[v], st);
        if (r.e[v] == cudaSuccess)
            r.e[v] = invert_f32(c->d_Hc64[v], c->d_inv32[v], D, perm, status, scratch,
                                &r.launches[v], &r.singular[v], st, blas);
        blas_return(c->device, blas);  // invert_f32 synchronises its stream before returning
        r.launches[v] += 1;
    };
    if (ninv == 2) {
        r.e[1] = cudaEventRecord(c->ev_fork2, s0);  // levels 0/1 and the maps are ready
        if (r.e[1] == cudaSuccess) r.e[1] = cudaStreamWaitEvent(s1, c->ev_fork2, 0);
        if (r.e[1] != cudaSuccess) return;
        std::thread second([&] {
            cudaSetDevice(c->device);
            invert(1, s1, c->d_perm2, c->d_status2, c->d_inv_scratch32b);
        });
        invert(0, s0, c->d_perm, c->d_status, c->d_inv_scratch32);
        second.join();  // both inverses end with a synchronisation of their stream
    } else {
        invert(0, s0, c->d_perm, c->d_status, c->d_inv_scratch32);
    }
}

int finish_inverses(tdbem_ctx* c, int ninv, const InvResult& r) {
    for (int v = 0; v < ninv; v++) {
        c->launches += r.launches[v];
        CUDA_TRY(r.e[v]);
        if (r.singular[v])
            return fail(TDBEM_ERR_SINGULAR, "zero pivot in the H^0 factorisation (LHS %d)", v);
    }
    if (ninv == 1) {
        if (c->d_inv32[1] && c->d_inv32[1] != c->d_inv32[0]) dfree(c->d_inv32[1]);
        if (c->d_Hc64[1] && c->d_Hc64[1] != c->d_Hc64[0]) dfree(c->d_Hc64[1]);
        c->d_inv32[1] = c->d_inv32[0];
        c->d_Hc64[1] = c->d_Hc64[0];
    }
    c->inv_valid = true;
    c->inv_n = ninv;
    c->inv_a1 = c->a1;
    c->inv_a2 = c->a2;
    c->inv_ubc = c->ubc;
    return TDBEM_OK;
}

// The inverses for a march of numstep steps, unless current; c->timings[1] gets
// the time taken (left as it is when they are reused).
int mixed_inverses(tdbem_ctx* c, int numstep, const double lhs_c[2][2]) {
    const int ninv = mixed_ninv(numstep, lhs_c);
    if (inverses_current(c, ninv)) return TDBEM_OK;
    const int rc = prepare_inverses(c, ninv);
    if (rc != TDBEM_OK) return rc;
    cudaStream_t s = c->stream;
    EventTimer tf;
    tf.start(s);
    const int pe = prof_begin(c, TDBEM_K_FACTOR);
    InvResult r;
    run_inverses(c, ninv, lhs_c, s, c->stream2, r);
    const double DD = (double)c->D * c->D;
    prof_end(c, pe, ninv * 2.0 * 4 * DD, ninv * 2.0 * DD * c->D);
    const int rc2 = finish_inverses(c, ninv, r);
    c->timings[1] = tf.stop_ms(s);
    return rc2;
}

// The merged level planes of the tcgen05 march and the known part's vectors (once
// per assembly and boundary conditions; march_tc.cu), from the FP32 levels.
int ensure_merged_levels(tdbem_ctx* c) {
    const int D = c->D, M = c->M;
    cudaStream_t s = c->stream;
    if (c->mtc_planes_valid) return TDBEM_OK;
    if (!c->d_mtc_planes)
        CUDA_TRY(cudaMalloc(&c->d_mtc_planes, tc_plane_bytes(D, M + 1, 1)));
    if (!c->d_mtc_known) CUDA_TRY(dalloc(&c->d_mtc_known, (size_t)3 * (M + 1) * D));
    if (!c->d_mtc_bc) CUDA_TRY(dalloc(&c->d_mtc_bc, (size_t)3 * D));
    // kt, lt, lu (the last list entry of a dof wins, as in upload_bc)
    std::vector<unsigned char> is_u(D, 0), is_f(D, 0);
    std::vector<double> umap(D, 0.0), fmap(D, 0.0);
    for (size_t i = 0; i < c->ubc.size(); i++) {
        is_u[c->ubc[i]] = 1;
        umap[c->ubc[i]] = c->ubc_v[i];
    }
    for (size_t i = 0; i < c->fbc.size(); i++) {
        is_f[c->fbc[i]] = 1;
        fmap[c->fbc[i]] = c->fbc_v[i];
    }
    std::vector<float> bcv((size_t)3 * D, 0.f);
    for (int j = 0; j < D; j++) {
        if (is_f[j] && (!is_u[j] || j == D - 1)) bcv[j] = (float)fmap[j];
        if (is_f[j] && !is_u[j]) bcv[D + j] = (float)fmap[j];
        if (is_u[j]) bcv[2 * D + j] = (float)umap[j];
    }
    CUDA_TRY(cudaMemcpyAsync(c->d_mtc_bc, bcv.data(), sizeof(float) * bcv.size(),
                             cudaMemcpyHostToDevice, s));
    const int pe = prof_begin(c, TDBEM_K_AUX);
    CUDA_TRY(launch_merge_levels(c->d_Gf, c->d_Hf, c->ldf, D, M + 1, c->d_is_ubc,
                                 c->d_mtc_bc, c->d_mtc_bc + D, c->d_mtc_bc + 2 * D,
                                 c->d_mtc_planes, c->d_mtc_known, s));
    prof_end(c, pe, (M + 1) * (double)D * (2.0 * c->ldf + tc_ldb(D)) * 4, 0);
    c->launches += 1;
    c->mtc_planes_valid = true;
    return TDBEM_OK;
}

// Mixed-precision marching: FP32 levels with time blocks of c->nb steps, FP32
// inverse of each distinct LHS, FP64 residual refinement against the FP64 LHS.
int march_mixed(tdbem_ctx* c, int numstep, const double lhs_c[2][2]) {
    // block steps: the setting, or each engine's measured optimum on the 4614-DOF sphere
    const int nb = c->nb ? c->nb : (c->march_engine == TDBEM_ENGINE_TCGEN05 ? 32 : 8);
    const int D = c->D, M = c->M;
    const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
    const size_t DD = (size_t)D * D;
    const int ldw = mixed_ldw(D);
    cudaStream_t s = c->stream;
    if (nb > 16 && c->march_engine != TDBEM_ENGINE_TCGEN05)
        return fail(TDBEM_ERR_ARG, "block_steps %d needs the tcgen05 march engine (FP32: <= 16)",
                    nb);
    c->nb_eff = nb;
    if (c->d_Wt_old && c->nb_alloc != nb) {  // scratch sized by the block
        dfree(c->d_Wt_old);
        dfree(c->d_Wu_old);
        dfree(c->d_Yold);
        dfree(c->d_pmix);
        dfree(c->d_res);
        dfree(c->d_dx);
    }
    if (!c->d_Wt_old) {
        c->nb_alloc = nb;
        CUDA_TRY(dalloc(&c->d_Wt_old, (size_t)(M + 1) * nb * ldw));
        CUDA_TRY(dalloc(&c->d_Wu_old, (size_t)(M + 1) * nb * ldw));
        CUDA_TRY(dalloc(&c->d_Yold, (size_t)nb * D));
        CUDA_TRY(dalloc(&c->d_pmix, (size_t)(M + 1) * nb * D));
        CUDA_TRY(dalloc(&c->d_res, D));
        CUDA_TRY(dalloc(&c->d_dx, D));
    }
    const int rc = mixed_inverses(c, numstep, lhs_c);
    if (rc != TDBEM_OK) return rc;
    // tcgen05 engine: the merged level matrix as BF16 hi/lo planes and the known
    // part's vectors (once per assembly and boundary conditions), the known part's
    // coefficients (once per load history, weights and step count), the history
    // vectors' planes and the tensor maps
    const bool tc = c->march_engine == TDBEM_ENGINE_TCGEN05;
    const int Lw = M + 1;
    if (tc) {
        const int rm = ensure_merged_levels(c);
        if (rm != TDBEM_OK) return rm;
        std::vector<double> key = {(double)numstep, (double)(M + 1), a1, a2,
                                   lhs_c[1][0], lhs_c[1][1]};
        key.insert(key.end(), c->amp.begin(), c->amp.end());
        if (key != c->mtc_coef_key) {
            std::vector<double> tab;
            known_coefficients(numstep, M + 1, a1, a2, a3, c->amp, lhs_c[1][0], lhs_c[1][1], tab);
            if (c->mtc_coef_cap < tab.size()) {
                dfree(c->d_mtc_coef);
                c->mtc_coef_cap = 0;
                CUDA_TRY(dalloc(&c->d_mtc_coef, tab.size()));
                c->mtc_coef_cap = tab.size();
            }
            CUDA_TRY(cudaMemcpyAsync(c->d_mtc_coef, tab.data(), sizeof(double) * tab.size(),
                                     cudaMemcpyHostToDevice, s));
            c->mtc_coef_key = key;
        }
        const size_t yk = (size_t)(numstep + 1) * D;
        if (c->mtc_yk_cap < yk) {
            dfree(c->d_mtc_yk);
            c->mtc_yk_cap = 0;
            CUDA_TRY(dalloc(&c->d_mtc_yk, yk));
            c->mtc_yk_cap = yk;
        }
        const size_t wb = tc_w_bytes(D, nb, Lw, 1);
        if (c->mtc_W_bytes < wb) {
            if (c->d_mtc_W) cudaFree(c->d_mtc_W);
            c->d_mtc_W = nullptr;
            c->mtc_W_bytes = 0;
            c->mtc_maps_for[0] = c->mtc_maps_for[1] = nullptr;
            CUDA_TRY(cudaMalloc(&c->d_mtc_W, wb));
            c->mtc_W_bytes = wb;
        }
        if (c->mtc_maps_for[0] != c->d_mtc_planes || c->mtc_maps_for[1] != c->d_mtc_W ||
            c->mtc_nb != nb) {
            if (!make_tc_maps(c->d_mtc_planes, D, M + 1, c->d_mtc_W, nb, Lw, &c->mtc_maps, 1))
                return fail(TDBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed for the march planes");
            c->mtc_maps_for[0] = c->d_mtc_planes;
            c->mtc_maps_for[1] = c->d_mtc_W;
            c->mtc_nb = nb;
        }
        if (!c->d_tc_err) CUDA_TRY(dalloc(&c->d_tc_err, 1));
        CUDA_TRY(cudaMemsetAsync(c->d_tc_err, 0, sizeof(int), s));
    }

    EventTimer tmr;
    tmr.start(s);
    const size_t lstride = (size_t)D * c->ldf;
    const int last_s = numstep - 1;  // solve steps 1..numstep-1
    const std::vector<const void*> ptrs = {
        c->d_u,       c->d_t,       c->d_Gf,      c->d_Hf,      c->d_inv32[0], c->d_inv32[1],
        c->d_Hc64[0], c->d_Hc64[1], c->d_Wt_old,  c->d_Wu_old,  c->d_Yold,     c->d_pmix,
        c->d_x,       c->d_res,     c->d_dx,      c->d_load_t,  c->d_load_u,   c->d_is_ubc,
        c->d_ubc_map, c->d_is_fbc,  c->d_fbc_map, tc ? c->d_mtc_planes : nullptr,
        tc ? c->d_mtc_W : nullptr,  tc ? c->d_tc_err : nullptr,  tc ? c->d_mtc_known : nullptr,
        tc ? c->d_mtc_coef : nullptr, tc ? c->d_mtc_yk : nullptr};
    // d_Yold[j] accumulates the right-hand side of step S + j of the current block.
    // Old pass: history before the block and the steps' known-load terms.
    auto old_pass = [&](int S, int nbe) -> int {
        const int nlev = (S > 1 ? std::min(M, S + nbe - 1) : std::min(M, 1)) + 1;
        BlockLoads bl{};  // the FP32 engine's known-load terms (its blocks: <= 16 steps)
        bl.nload = tc ? 0 : nbe;
        bl.load_t = c->d_load_t;
        bl.load_u = c->d_load_u;
        for (int j = 0; j < bl.nload; j++) {
            const int st = S + j;
            bl.amp[j] = c->amp.empty() ? 1.0 : c->amp[st];
            bl.c0[j] = st == 1 ? 1.0 : lhs_c[1][0];
            bl.c1[j] = st == 1 ? 0.0 : lhs_c[1][1];
        }
        if (tc) {  // merged levels, split-BF16 products on the tensor cores
            double* Y = c->d_Yold;
            const double* yk = c->d_mtc_yk + (size_t)S * D;  // the steps' known part
            if (S == 1) {  // no unknown history before the first block
                CUDA_TRY(cudaMemcpyAsync(Y, yk, sizeof(double) * nbe * D,
                                         cudaMemcpyDeviceToDevice, s));
            } else {
                CUDA_TRY(launch_build_w_merged(c->d_u, c->d_t, c->d_is_ubc, D, S, nbe, nb, 1, S,
                                               nlev, Lw, a1, a2, a3, c->d_mtc_W, s));
                // d_pmix holds (M+1) x nb x D partial sums
                const int splits = tc_conv_splits(nlev, D, nbe, (M + 1) * nb / nbe, 1);
                const int pe = prof_begin(c, TDBEM_K_CONV_BLOCK);
                CUDA_TRY(launch_conv_tc(c->mtc_maps, D, M + 1, Lw, nlev, nbe, c->d_pmix, splits,
                                        c->d_tc_err, s, 1));
                prof_end(c, pe, nlev * (double)D * tc_ldb(D) * 4 +
                                    nlev * (double)tc_cases_pad(nb) * tc_ldb(D) * 4,
                         nlev * 2.0 * nbe * (double)DD);
                CUDA_TRY(launch_reduce_cols_n(c->d_pmix, splits, nbe, nbe, D, yk, Y, s));
                c->launches += 3;
            }
            return TDBEM_OK;
        }
        CUDA_TRY(launch_build_w_old(c->d_u, c->d_t, D, S, nb, nlev, a1, a2, a3, bl, ldw,
                                    c->d_Wt_old, c->d_Wu_old, s));
        const int nch = mixed_chunks(nlev, D);
        int nparts = 0;
        const int pe = prof_begin(c, TDBEM_K_CONV_BLOCK);
        CUDA_TRY(launch_conv_f32(c->d_Gf, c->d_Hf, lstride, c->ldf, D, 0, nlev - 1, nb,
                                 c->d_Wt_old, c->d_Wu_old, ldw, c->d_pmix, nch,
                                 mixed_ksplit(nch, D, M + 1), &nparts, s));
        prof_end(c, pe, nlev * 2.0 * (double)lstride * 4 + nlev * 2.0 * nb * ldw * 4,
                 nlev * 4.0 * nb * (double)DD);
        CUDA_TRY(launch_reduce_cols(c->d_pmix, nparts, nb, D, nullptr, c->d_Yold, s));
        c->launches += 3;
        return TDBEM_OK;
    };
    // The history of steps [a, b) into the right-hand sides of steps [b, e): levels
    // 0..e-a, e-b columns (padded to a kernel width).
    auto cross = [&](int S, int a, int b, int e) -> int {
        const int ncol = e - b;
        const int nbp = ncol <= 1 ? 1 : ncol <= 2 ? 2 : ncol <= 4 ? 4 : ncol <= 8 ? 8 : 16;
        const int nlev = std::min(M, e - a) + 1;
        double* y = c->d_Yold + (size_t)(b - S) * D;
        if (tc) {
            CUDA_TRY(launch_build_w_merged(c->d_u, c->d_t, c->d_is_ubc, D, b, ncol, nb, a, b,
                                           nlev, Lw, a1, a2, a3, c->d_mtc_W, s));
            const int splits = tc_conv_splits(nlev, D, ncol, (M + 1) * nb / ncol, 1);
            const int pe = prof_begin(c, TDBEM_K_CONV);
            CUDA_TRY(launch_conv_tc(c->mtc_maps, D, M + 1, Lw, nlev, ncol, c->d_pmix, splits,
                                    c->d_tc_err, s, 1));
            prof_end(c, pe, nlev * (double)D * tc_ldb(D) * 4 +
                                nlev * (double)tc_cases_pad(nb) * tc_ldb(D) * 4,
                     nlev * 2.0 * ncol * (double)DD);
            CUDA_TRY(launch_reduce_cols_n(c->d_pmix, splits, ncol, ncol, D, y, y, s));
            c->launches += 3;
            return TDBEM_OK;
        }
        CUDA_TRY(launch_build_w_cross(c->d_u, c->d_t, D, a, b, ncol, nbp, nlev, a1, a2, a3, ldw,
                                      c->d_Wt_old, c->d_Wu_old, s));
        const int nch = mixed_chunks(nlev, D);
        int nparts = 0;
        const int pe = prof_begin(c, TDBEM_K_CONV);
        CUDA_TRY(launch_conv_f32(c->d_Gf, c->d_Hf, lstride, c->ldf, D, 0, nlev - 1, nbp,
                                 c->d_Wt_old, c->d_Wu_old, ldw, c->d_pmix, nch,
                                 mixed_ksplit(nch, D, (M + 1) * nb / nbp), &nparts, s));
        prof_end(c, pe, nlev * 2.0 * (double)lstride * 4 + nlev * 2.0 * nbp * ldw * 4,
                 nlev * 4.0 * ncol * (double)DD);
        CUDA_TRY(launch_reduce_cols_n(c->d_pmix, nparts, nbp, ncol, D, y, y, s));
        c->launches += 3;
        return TDBEM_OK;
    };
    // Step st from its accumulated right-hand side.
    auto solve = [&](int S, int st) -> int {
        const int pe = prof_begin(c, TDBEM_K_SOLVE);
        const int v = st == 1 ? 0 : 1;
        const double amp = c->amp.empty() ? 1.0 : c->amp[st];
        // d_dx (D doubles) holds the D-float FP32 vector of the solve's products
        CUDA_TRY(launch_solve_mixed(c->d_inv32[v], c->d_Hc64[v], D, c->d_Yold + (size_t)(st - S) * D,
                                    c->d_x, c->d_res, reinterpret_cast<float*>(c->d_dx),
                                    c->n_refine, s));
        CUDA_TRY(launch_update_state(c->d_x, D, st, c->d_is_ubc, c->d_ubc_map, c->d_is_fbc,
                                     c->d_fbc_map, amp, c->d_u, c->d_t, s));
        prof_end(c, pe, 4.0 * (double)DD * (1 + 2 * c->n_refine),
                 2.0 * (double)DD * (1 + 2 * c->n_refine));
        c->launches += 4 + 2LL * c->n_refine;  // cast, gemv(s), residual(s), update
        return TDBEM_OK;
    };
    // Steps [s0, s0 + n) of the block starting at S: first half, its history into
    // the second half, second half.
    std::function<int(int, int, int)> rec = [&](int S, int s0, int n) -> int {
        if (n == 1) return solve(S, s0);
        const int h = n / 2;
        int r = rec(S, s0, h);
        if (r == TDBEM_OK) r = cross(S, s0, s0 + h, s0 + n);
        if (r == TDBEM_OK) r = rec(S, s0 + h, n - h);
        return r;
    };
    const int lrc = run_march_loop(c, 1, numstep, ptrs, [&]() -> int {
        if (tc) {  // the known part of every step's right-hand side
            const int pk = prof_begin(c, TDBEM_K_AUX);
            CUDA_TRY(launch_known_terms(c->d_mtc_known, c->d_mtc_coef, D, M + 1, last_s,
                                        c->d_mtc_yk, s));
            prof_end(c, pk, 3.0 * (M + 1) * D * 8 * ((last_s + 15) / 16) + 8.0 * last_s * D, 0);
            c->launches += 1;
        }
        for (int S = 1; S <= last_s; S += nb) {
            const int nbe = std::min(nb, last_s - S + 1);
            int r = old_pass(S, nbe);
            if (r == TDBEM_OK) r = rec(S, S, nbe);
            if (r != TDBEM_OK) return r;
        }
        return TDBEM_OK;
    });
    if (lrc != TDBEM_OK) return lrc;
    if (tc) {  // a bounded pipeline wait of the tcgen05 kernel that ran out
        int err = 0;
        CUDA_TRY(cudaMemcpyAsync(&err, c->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        if (err)
            return fail(TDBEM_ERR_CUDA, "tcgen05 convolution: pipeline wait timed out (code %d)",
                        err);
    }
    c->timings[2] = tmr.stop_ms(s);
    return TDBEM_OK;
}


// Per-dof boundary-condition maps and the marching scratch shared by every
// marching form.
int upload_bc(tdbem_ctx* c) {
    const int D = c->D;
    // per-dof boundary-condition maps; the last list entry of a dof wins (VecSetValues)
    std::vector<unsigned char> is_u(D, 0), is_f(D, 0);
    std::vector<double> umap(D, 0.0), fmap(D, 0.0), load_t(D, 0.0), load_u(D, 0.0);
    for (size_t i = 0; i < c->ubc.size(); i++) {
        is_u[c->ubc[i]] = 1;
        umap[c->ubc[i]] = c->ubc_v[i];
    }
    for (size_t i = 0; i < c->fbc.size(); i++) {
        is_f[c->fbc[i]] = 1;
        fmap[c->fbc[i]] = c->fbc_v[i];
    }
    for (int j = 0; j < D; j++) {
        if (is_u[j]) load_u[j] = umap[j];
        else if (is_f[j]) load_t[j] = fmap[j];
    }
    if (!c->d_ubc_map) {
        CUDA_TRY(dalloc(&c->d_ubc_map, D));
        CUDA_TRY(dalloc(&c->d_fbc_map, D));
        CUDA_TRY(dalloc(&c->d_is_ubc, D));
        CUDA_TRY(dalloc(&c->d_is_fbc, D));
        CUDA_TRY(dalloc(&c->d_load_t, D));
        CUDA_TRY(dalloc(&c->d_load_u, D));
        CUDA_TRY(dalloc(&c->d_Wt, (size_t)(c->M + 1) * D));
        CUDA_TRY(dalloc(&c->d_Wu, (size_t)(c->M + 1) * D));
        CUDA_TRY(dalloc(&c->d_rhs, D));
        CUDA_TRY(dalloc(&c->d_x, D));
        CUDA_TRY(dalloc(&c->d_perm, D + 2 * kMaxPivotBlocks));
        CUDA_TRY(dalloc(&c->d_status, 1));
        c->partial_cap = (size_t)(c->M + 1) * D;
        CUDA_TRY(dalloc(&c->d_partial, c->partial_cap));
    }
    cudaStream_t s = c->stream;
    CUDA_TRY(cudaMemcpyAsync(c->d_ubc_map, umap.data(), sizeof(double) * D,
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->d_fbc_map, fmap.data(), sizeof(double) * D,
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->d_is_ubc, is_u.data(), D, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->d_is_fbc, is_f.data(), D, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->d_load_t, load_t.data(), sizeof(double) * D,
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(c->d_load_u, load_u.data(), sizeof(double) * D,
                             cudaMemcpyHostToDevice, s));
    // the host vectors above are pageable: finish the copies before they go
    CUDA_TRY(cudaStreamSynchronize(s));
    return TDBEM_OK;
}

// FP64 inverse of the column-exchanged LHS v (0: step 2's, 1: steps >= 3) into
// c->d_Ainv[v] (SolverStepLinearT.cpp:357-393, KSPSolve as an explicit inverse).
int fp64_inverse(tdbem_ctx* c, int v, const double lhs_c[2][2]) {
    const int D = c->D;
    const size_t stride = (size_t)D * D;
    cudaStream_t s = c->stream;
    if (c->d_Ainv[1 - v] == c->d_Ainv[v]) c->d_Ainv[v] = nullptr;  // was an alias of the other
    if (!c->d_Ainv[v]) CUDA_TRY(dalloc(&c->d_Ainv[v], stride));
    CUDA_TRY(launch_build_lhs(c->d_G, c->d_H, c->d_Gf, c->d_Hf, stride, D, lhs_c[v][0],
                              lhs_c[v][1], c->d_is_ubc, c->d_Ainv[v], s));
    if (!c->d_inv_scratch) CUDA_TRY(dalloc(&c->d_inv_scratch, inverse_scratch_elems(D)));
    const int pe = prof_begin(c, TDBEM_K_FACTOR);
    bool singular = false;
    cudaError_t e = invert_f64(c->d_Ainv[v], D, c->d_perm, c->d_status, c->d_inv_scratch,
                               &c->launches, &singular, s);
    prof_end(c, pe, 2.0 * 8 * stride, 2.0 * (double)D * D * D);
    c->launches += 1;  // LHS build
    CUDA_TRY(e);
    if (singular)
        return fail(TDBEM_ERR_SINGULAR, "zero pivot in the H^0 factorisation (LHS %d)", v);
    return TDBEM_OK;
}

// One FP64 Solve_Averaging step: solve step st (history st) from histories < st.
int fp64_step(tdbem_ctx* c, int st, const double lhs_c[2][2]) {
    const int D = c->D;
    const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
    const size_t stride = (size_t)D * D;
    cudaStream_t s = c->stream;
    MarchDev md{D, c->M, c->d_G, c->d_H, c->d_Gf, c->d_Hf};
    const int L = std::min(std::max(st, 1), c->M);
    const double c0 = st == 1 ? 1.0 : lhs_c[1][0];
    const double c1 = st == 1 ? 0.0 : lhs_c[1][1];
    const double amp = c->amp.empty() ? 1.0 : c->amp[st];
    CUDA_TRY(launch_history_combine(c->d_u, c->d_t, D, st, L, a1, a2, a3, c0, c1, amp,
                                    c->d_load_t, c->d_load_u, c->d_Wt, c->d_Wu, s));
    const int nch = conv_chunks(L, D);
    const double esz = c->d_G ? 8.0 : 4.0;
    int pe = prof_begin(c, TDBEM_K_CONV);
    CUDA_TRY(launch_conv(md, L, c->d_Wt, c->d_Wu, c->d_partial, nch, s));
    prof_end(c, pe, (L + 1) * 2.0 * (double)stride * esz + (L + 1) * 2.0 * D * 8,
             (L + 1) * 4.0 * (double)stride);
    pe = prof_begin(c, TDBEM_K_SOLVE);
    CUDA_TRY(launch_reduce_solve(c->d_partial, nch, D, c->d_Ainv[st == 1 ? 0 : 1], c->d_rhs,
                                 c->d_x, s));
    CUDA_TRY(launch_update_state(c->d_x, D, st, c->d_is_ubc, c->d_ubc_map, c->d_is_fbc,
                                 c->d_fbc_map, amp, c->d_u, c->d_t, s));
    prof_end(c, pe, 8.0 * (double)stride, 2.0 * (double)stride);
    c->launches += 5;  // combine, conv, reduce, gemv, update
    return TDBEM_OK;
}

// Plain FP64 marching: one level-streamed convolution and one FP64 inverse
// product per step.
int march_fp64(tdbem_ctx* c, int numstep, const double lhs_c[2][2], double* u_hist,
               double* t_hist) {
    const int D = c->D;
    cudaStream_t s = c->stream;
    const bool same = (lhs_c[1][0] == 1.0 && lhs_c[1][1] == 0.0);
    EventTimer tf;
    tf.start(s);
    const int ninv = (numstep >= 3 && !same) ? 2 : 1;
    for (int v = 0; v < ninv; v++) {
        const int rc = fp64_inverse(c, v, lhs_c);
        if (rc != TDBEM_OK) return rc;
    }
    if (ninv == 1) {
        if (c->d_Ainv[1] && c->d_Ainv[1] != c->d_Ainv[0]) dfree(c->d_Ainv[1]);
        c->d_Ainv[1] = c->d_Ainv[0];
    }
    c->timings[1] = tf.stop_ms(s);

    EventTimer tmr;
    tmr.start(s);
    const std::vector<const void*> ptrs = {
        c->d_u,     c->d_t,   c->d_G,       c->d_H,      c->d_Gf,       c->d_Hf,
        c->d_Ainv[0], c->d_Ainv[1], c->d_Wt, c->d_Wu,    c->d_partial,  c->d_rhs,
        c->d_x,     c->d_load_t, c->d_load_u, c->d_is_ubc, c->d_ubc_map, c->d_is_fbc,
        c->d_fbc_map};
    const int lrc = run_march_loop(c, 0, numstep, ptrs, [&]() -> int {
        for (int st = 1; st <= numstep - 1; st++) {
            const int rc = fp64_step(c, st, lhs_c);
            if (rc != TDBEM_OK) return rc;
        }
        return TDBEM_OK;
    });
    if (lrc != TDBEM_OK) return lrc;
    c->timings[2] = tmr.stop_ms(s);
    if (u_hist)
        CUDA_TRY(cudaMemcpyAsync(u_hist, c->d_u, sizeof(double) * (numstep + 1) * D,
                                 cudaMemcpyDeviceToHost, s));
    if (t_hist)
        CUDA_TRY(cudaMemcpyAsync(t_hist, c->d_t, sizeof(double) * (numstep + 1) * D,
                                 cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    prof_flush(c);
    return TDBEM_OK;
}

// FP64 level store of (M+1) levels, zeroed, for levels fed from host row blocks
// or a checkpoint.
int ensure_fp64_store(tdbem_ctx* c) {
    if (c->level_precision == TDBEM_FP64 && c->d_G) return TDBEM_OK;
    free_levels(c);
    const size_t n = (size_t)(c->M + 1) * c->D * c->D;
    CUDA_TRY(dalloc(&c->d_G, n));
    CUDA_TRY(dalloc(&c->d_H, n));
    CUDA_TRY(cudaMemsetAsync(c->d_G, 0, sizeof(double) * n, c->stream));
    CUDA_TRY(cudaMemsetAsync(c->d_H, 0, sizeof(double) * n, c->stream));
    c->level_precision = TDBEM_FP64;
    c->levels_last = 0;
    return TDBEM_OK;
}

}  // namespace

void tdbem::note_error(const char* msg) { g_last_error = msg; }

extern "C" {

const char* tdbem_last_error(void) { return g_last_error.c_str(); }

const char* tdbem_version(void) { return "tdbem-gb300 0.1 (sm_103a)"; }

int tdbem_ctx_create(const tdbem_mesh* mesh, const tdbem_material* mat, double dt, int nq,
                     int if_ext, tdbem_ctx** out) {
    if (!out) return fail(TDBEM_ERR_ARG, "out is null");
    *out = nullptr;
    if (!mesh || !mat || !mesh->coords || !mesh->ien)
        return fail(TDBEM_ERR_ARG, "mesh/material pointers are null");
    if (mesh->etype != 1 && mesh->etype != 2)
        return fail(TDBEM_ERR_UNSUPPORTED,
                    "element type %d: 4-node (EType=1) or 8-node (EType=2) quads only",
                    mesh->etype);
    const int ennd = mesh->etype == 2 ? 8 : 4;
    if (mesh->nnd < 2 || mesh->nel < 1) return fail(TDBEM_ERR_ARG, "empty mesh");
    if (!(dt > 0) || !(mat->rho > 0) || !(mat->E > 0) || !(mat->nu > -1 && mat->nu < 0.5))
        return fail(TDBEM_ERR_ARG, "invalid dt or material");
    std::vector<double> gx, gw;
    if (!gauss_table(nq, gx, gw))
        return fail(TDBEM_ERR_ARG, "unsupported number of Gauss points %d", nq);
    for (long long i = 0; i < (long long)ennd * mesh->nel; i++)
        if (mesh->ien[i] < 0 || mesh->ien[i] >= mesh->nnd)
            return fail(TDBEM_ERR_ARG, "IEN entry %lld = %d out of range", i, mesh->ien[i]);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(TDBEM_ERR_CUDA, "no CUDA device available (tdbem has no CPU path)");
    }
    tdbem_ctx* c = new (std::nothrow) tdbem_ctx;
    if (!c) return fail(TDBEM_ERR_NOMEM, "host allocation failed");
    cudaGetDevice(&c->device);
    c->nnd = mesh->nnd;
    c->nel = mesh->nel;
    c->ennd = ennd;
    c->D = 3 * mesh->nnd;
    c->nq = nq;
    c->if_ext = if_ext ? 1 : 0;
    c->E = mat->E;
    c->nu = mat->nu;
    c->rho = mat->rho;
    c->dt = dt;
    c->h_coords.assign(mesh->coords, mesh->coords + 3 * (size_t)mesh->nnd);
    c->h_ien.assign(mesh->ien, mesh->ien + ennd * (size_t)mesh->nel);
    c->M = compute_max_step(c->h_coords, c->nnd, c->E, c->nu, c->rho, dt);
    // GreenFunctionT::WaveSpeed (GreenFunctionT.cpp:76-84)
    const double mu = c->E / (2 * (1 + c->nu));
    const double lam = c->E * c->nu / ((1 + c->nu) * (1 - 2 * c->nu));
    Phys& ph = c->ph;
    ph.dt = dt;
    ph.inv_dt = 1.0 / dt;
    ph.cp = std::sqrt((lam + 2 * mu) / c->rho);
    ph.cs = std::sqrt(mu / c->rho);
    ph.inv_cp = 1.0 / ph.cp;
    ph.inv_cs = 1.0 / ph.cs;
    ph.inv_cp2 = 1.0 / (ph.cp * ph.cp);
    ph.inv_cs2 = 1.0 / (ph.cs * ph.cs);
    ph.cs2 = ph.cs * ph.cs;
    ph.ratio2 = (ph.cs / ph.cp) * (ph.cs / ph.cp);
    ph.ratio3 = ph.ratio2 * (ph.cs / ph.cp);
    ph.inv_4pi_rho = 1.0 / (4 * M_PI * c->rho);
    ph.inv_4pi = 1.0 / (4 * M_PI);
    ph.nu = c->nu;
    std::vector<int> order;
    color_elements(c->h_ien, c->nel, c->ennd, c->nnd, order, c->color_start);
    int max_color = 0;
    for (size_t k = 0; k + 1 < c->color_start.size(); k++)
        max_color = std::max(max_color, c->color_start[k + 1] - c->color_start[k]);
    auto cleanup_fail = [&](int code) {
        tdbem_ctx_destroy(c);
        return code;
    };
#define CTX_TRY(expr)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            fail(e_ == cudaErrorMemoryAllocation ? TDBEM_ERR_NOMEM : TDBEM_ERR_CUDA, "%s: %s", \
                 #expr, cudaGetErrorString(e_));                                             \
            return cleanup_fail(e_ == cudaErrorMemoryAllocation ? TDBEM_ERR_NOMEM           \
                                                                : TDBEM_ERR_CUDA);          \
        }                                                                                    \
    } while (0)
    CTX_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    blas_pool_init(c->device);  // before any march of this device can capture a graph
    CTX_TRY(dalloc(&c->d_coords, c->h_coords.size()));
    CTX_TRY(dalloc(&c->d_ien, c->h_ien.size()));
    CTX_TRY(dalloc(&c->d_gx, nq));
    CTX_TRY(dalloc(&c->d_gw, nq));
    CTX_TRY(dalloc(&c->d_geom, (size_t)c->nel * nq * nq * (ennd == 8 ? 16 : 12)));
    CTX_TRY(dalloc(&c->d_cterm, (size_t)c->nnd * 9));
    if (ennd == 4) CTX_TRY(dalloc(&c->d_geomf, (size_t)c->nel * nq * nq * 12));
    CTX_TRY(dalloc(&c->d_color_elems, order.size()));
    CTX_TRY(dalloc(&c->d_color_start, c->color_start.size()));
    CTX_TRY(dalloc(&c->d_far_items, 1));
    CTX_TRY(cudaMemcpyAsync(c->d_coords, c->h_coords.data(), sizeof(double) * c->h_coords.size(),
                            cudaMemcpyHostToDevice, c->stream));
    {  // node coordinates as FP32 pairs x = hi + lo for the FP32 far form
        std::vector<float> cf((size_t)8 * c->nnd, 0.f);
        for (int i = 0; i < c->nnd; i++)
            for (int d = 0; d < 3; d++) {
                const double x = c->h_coords[(size_t)3 * i + d];
                const float hi = (float)x;
                cf[(size_t)8 * i + d] = hi;
                cf[(size_t)8 * i + 4 + d] = (float)(x - (double)hi);
            }
        CTX_TRY(dalloc(&c->d_coordf, cf.size()));
        CTX_TRY(cudaMemcpyAsync(c->d_coordf, cf.data(), sizeof(float) * cf.size(),
                                cudaMemcpyHostToDevice, c->stream));
    }
    CTX_TRY(cudaMemcpyAsync(c->d_ien, c->h_ien.data(), sizeof(int) * c->h_ien.size(),
                            cudaMemcpyHostToDevice, c->stream));
    CTX_TRY(cudaMemcpyAsync(c->d_gx, gx.data(), sizeof(double) * nq, cudaMemcpyHostToDevice,
                            c->stream));
    CTX_TRY(cudaMemcpyAsync(c->d_gw, gw.data(), sizeof(double) * nq, cudaMemcpyHostToDevice,
                            c->stream));
    CTX_TRY(cudaMemcpyAsync(c->d_color_start, c->color_start.data(),
                            sizeof(int) * c->color_start.size(), cudaMemcpyHostToDevice,
                            c->stream));
    CTX_TRY(cudaMemcpyAsync(c->d_color_elems, order.data(), sizeof(int) * order.size(),
                            cudaMemcpyHostToDevice, c->stream));
    CTX_TRY(launch_gauss_geom(c->d_coords, c->d_ien, c->nel, ennd, nq, c->d_gx, c->d_gw,
                              c->d_geom, c->d_geomf, c->stream));
    c->pair_cap = std::min<size_t>((size_t)c->nnd * max_color, (size_t)1 << 26);
    c->pair_cap = std::max<size_t>(c->pair_cap, (size_t)max_color);
    CTX_TRY(dalloc(&c->d_pairs, c->pair_cap));
    CTX_TRY(dalloc(&c->d_counts, c->pair_cap));
    CTX_TRY(dalloc(&c->d_offsets, c->pair_cap));
    c->scan_tmp_bytes = scan_temp_bytes((unsigned)c->pair_cap);
    CTX_TRY(cudaMalloc(&c->d_scan_tmp, std::max<size_t>(c->scan_tmp_bytes, 16)));
    CTX_TRY(cudaStreamSynchronize(c->stream));
#undef CTX_TRY
    *out = c;
    return TDBEM_OK;
}

int tdbem_ctx_destroy(tdbem_ctx* c) {
    if (!c) return TDBEM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph.exec) {
        cudaGraphExecDestroy(c->graph.exec);
        c->graph.exec = nullptr;
    }
    free_levels(c);
    free_march(c);
    c->inv_valid = false;
    dfree(c->d_coords);
    dfree(c->d_ien);
    dfree(c->d_gx);
    dfree(c->d_gw);
    dfree(c->d_geom);
    dfree(c->d_cterm);
    dfree(c->d_geomf);
    dfree(c->d_coordf);
    dfree(c->d_color_elems);
    dfree(c->d_color_start);
    dfree(c->d_far_items);
    dfree(c->d_far_pairs);
    dfree(c->d_pairs);
    dfree(c->d_counts);
    dfree(c->d_offsets);
    if (c->d_scan_tmp) cudaFree(c->d_scan_tmp);
    dfree(c->d_ubc_map);
    dfree(c->d_fbc_map);
    dfree(c->d_is_ubc);
    dfree(c->d_is_fbc);
    dfree(c->d_inv_scratch);
    dfree(c->d_inv_scratch32);
    dfree(c->d_load_t);
    dfree(c->d_load_u);
    dfree(c->d_Wt);
    dfree(c->d_Wu);
    dfree(c->d_partial);
    dfree(c->d_rhs);
    dfree(c->d_x);
    dfree(c->d_perm);
    dfree(c->d_status);
    dfree(c->d_inv_scratch32b);
    dfree(c->d_perm2);
    dfree(c->d_status2);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_fork2) cudaEventDestroy(c->ev_fork2);
    if (c->stream3) cudaStreamDestroy(c->stream3);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TDBEM_OK;
}

int tdbem_max_step(const tdbem_ctx* c, int* M) {
    if (!c || !M) return fail(TDBEM_ERR_ARG, "null argument");
    *M = c->M;
    return TDBEM_OK;
}

int tdbem_num_dof(const tdbem_ctx* c, int* D) {
    if (!c || !D) return fail(TDBEM_ERR_ARG, "null argument");
    *D = c->D;
    return TDBEM_OK;
}

int tdbem_get_stream(const tdbem_ctx* c, void** stream) {
    if (!c || !stream) return fail(TDBEM_ERR_ARG, "null argument");
    *stream = (void*)c->stream;
    return TDBEM_OK;
}

int tdbem_level_bytes(const tdbem_ctx* c, int precision, size_t* bytes) {
    if (!c || !bytes) return fail(TDBEM_ERR_ARG, "null argument");
    const size_t D = c->D;
    if (precision == TDBEM_FP64) *bytes = 2 * (size_t)(c->M + 1) * D * D * 8;
    else *bytes = 2 * (size_t)(c->M + 1) * D * mixed_ld(c->D) * 4 + 4 * D * D * 8;
    return TDBEM_OK;
}

int tdbem_gh_driver(tdbem_ctx* c, int step, int node_lo, int node_hi, double* G_I, double* G_J,
                    double* H_I, double* H_J) {
    if (!c || !G_I || !G_J || !H_I || !H_J) return fail(TDBEM_ERR_ARG, "null argument");
    if (step < 1) return fail(TDBEM_ERR_ARG, "step must be >= 1");
    if (node_lo < 0 || node_hi >= c->nnd || node_lo > node_hi)
        return fail(TDBEM_ERR_ARG, "node range [%d, %d] invalid", node_lo, node_hi);
    const int nn = node_hi - node_lo + 1;
    const size_t n = (size_t)3 * nn * c->D;
    double* buf = nullptr;
    CUDA_TRY(dalloc(&buf, 4 * n));
    AsmOut out{};
    out.G0 = buf;
    out.H0 = buf + n;
    out.G1 = buf + 2 * n;
    out.H1 = buf + 3 * n;
    out.D = c->D;
    out.ld = c->D;
    out.row_node_lo = node_lo;
    int rc = TDBEM_OK;
    cudaError_t e = cudaMemsetAsync(buf, 0, sizeof(double) * 4 * n, c->stream);
    if (e != cudaSuccess) rc = fail(TDBEM_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    for (size_t col = 0; rc == TDBEM_OK && col + 1 < c->color_start.size(); col++)
        rc = assemble_color(c, (int)col, node_lo, nn, ASM_STEP, step, 1 << 30, step, SEL_ALL, out);
    if (rc == TDBEM_OK && step == 1) {
        e = launch_cterm(c->d_coords, c->d_ien, c->ennd, c->nel, node_lo, nn, c->nq, c->d_gx, c->d_gw,
                         c->d_geom, c->ph, c->d_cterm, c->stream);
        if (e == cudaSuccess)
            e = launch_cterm_apply(c->d_cterm, node_lo, nn, c->dt, c->if_ext, ASM_STEP, out,
                                   c->stream);
        if (e != cudaSuccess) rc = fail(TDBEM_ERR_CUDA, "cterm: %s", cudaGetErrorString(e));
    }
    double* hosts[4] = {G_I, H_I, G_J, H_J};
    for (int k = 0; rc == TDBEM_OK && k < 4; k++) {
        e = cudaMemcpyAsync(hosts[k], buf + k * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                            c->stream);
        if (e != cudaSuccess) rc = fail(TDBEM_ERR_CUDA, "copy: %s", cudaGetErrorString(e));
    }
    e = cudaStreamSynchronize(c->stream);
    if (rc == TDBEM_OK && e != cudaSuccess)
        rc = fail(TDBEM_ERR_CUDA, "gh_driver: %s", cudaGetErrorString(e));
    cudaFree(buf);
    return rc;
}

int tdbem_assemble_levels(tdbem_ctx* c, int nsteps, int precision) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (nsteps < 1) return fail(TDBEM_ERR_ARG, "nsteps must be >= 1");
    if (precision != TDBEM_FP64 && precision != TDBEM_MIXED)
        return fail(TDBEM_ERR_ARG, "unknown precision %d", precision);
    const size_t D = c->D;
    const int ldf = mixed_ld(c->D);
    if (c->level_precision != precision) {
        free_levels(c);
        if (precision == TDBEM_FP64) {
            CUDA_TRY(dalloc(&c->d_G, (size_t)(c->M + 1) * D * D));
            CUDA_TRY(dalloc(&c->d_H, (size_t)(c->M + 1) * D * D));
        } else {
            CUDA_TRY(dalloc(&c->d_Gf, (size_t)(c->M + 1) * D * ldf));
            CUDA_TRY(dalloc(&c->d_Hf, (size_t)(c->M + 1) * D * ldf));
            CUDA_TRY(dalloc(&c->d_G01, 2 * D * D));
            CUDA_TRY(dalloc(&c->d_H01, 2 * D * D));
        }
        c->level_precision = precision;
        c->ldf = ldf;
    }
    c->inv_valid = false;  // levels 0/1 change
    EventTimer tm;
    tm.start(c->stream);
    const int last = std::min(c->M, nsteps);
    const int ncol = (int)c->color_start.size() - 1;
    if (precision == TDBEM_FP64) {
        const size_t total = (size_t)(c->M + 1) * D * D;
        CUDA_TRY(cudaMemsetAsync(c->d_G, 0, 8 * total, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_H, 0, 8 * total, c->stream));
        AsmOut out{};
        out.G0 = c->d_G;
        out.H0 = c->d_H;
        out.level_stride = D * D;
        out.D = c->D;
        out.ld = c->D;
        for (int col = 0; col < ncol; col++) {
            const int rc = assemble_color(c, col, 0, c->nnd, ASM_LEVELS, last, c->M, 0, SEL_ALL,
                                          out);
            if (rc != TDBEM_OK) return rc;
        }
        const int pc = prof_begin(c, TDBEM_K_AUX);
        CUDA_TRY(launch_cterm(c->d_coords, c->d_ien, c->ennd, c->nel, 0, c->nnd, c->nq, c->d_gx, c->d_gw,
                              c->d_geom, c->ph, c->d_cterm, c->stream));
        CUDA_TRY(launch_cterm_apply(c->d_cterm, 0, c->nnd, c->dt, c->if_ext, ASM_LEVELS, out,
                                    c->stream));
        prof_end(c, pc, 0, 0);
        c->launches += 2;
    } else {
        // FP32 store for all levels: near pairs with the FP64 quadrature, far pairs with
        // the FP32 tau form; levels 0 and 1 again in FP64 for the LHS of the solve.
        const size_t total = (size_t)(c->M + 1) * D * ldf;
        CUDA_TRY(cudaMemsetAsync(c->d_Gf, 0, 4 * total, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_Hf, 0, 4 * total, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_G01, 0, 16 * D * D, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_H01, 0, 16 * D * D, c->stream));
        AsmOut o32{};
        o32.G0f = c->d_Gf;
        o32.H0f = c->d_Hf;
        o32.level_stride = D * ldf;
        o32.D = c->D;
        o32.ld = ldf;
        AsmOut o64{};
        o64.G0 = c->d_G01;
        o64.H0 = c->d_H01;
        o64.level_stride = D * D;
        o64.D = c->D;
        o64.ld = c->D;
        // 8-node elements: every pair through the FP64 quadrature (the FP32 far form
        // is written for 4-node elements)
        const bool split = c->ennd == 4;
        // FP64 levels 0/1 first: with the C term they are final, and the inverses can
        // start next to the rest of the assembly.  Singular pairs through the FP64
        // quadrature, the others through the FP32 far form (FP64 sums): the store's
        // FP32 inverses and levels carry FP32 accuracy either way.
        const size_t np = (size_t)c->nnd * c->nel;
        if (split && c->far_pairs_cap < np) {
            dfree(c->d_far_pairs);
            c->far_pairs_cap = 0;
            CUDA_TRY(dalloc(&c->d_far_pairs, np));
            c->far_pairs_cap = np;
        }
        for (int col = 0; col < ncol; col++) {
            const int rc = assemble_color(c, col, 0, c->nnd, ASM_LEVELS, last, 1, 0,
                                          split ? SEL_NEAR : SEL_ALL, o64);
            if (rc != TDBEM_OK) return rc;
        }
        const bool count = c->prof;  // the far item count feeds the profile's byte/flop totals
        if (count)
            CUDA_TRY(cudaMemsetAsync(c->d_far_items, 0, sizeof(unsigned long long), c->stream));
        if (split) {
            const int pw = prof_begin(c, TDBEM_K_AUX);
            CUDA_TRY(launch_pair_window(c->d_coords, c->d_ien, 4, c->d_color_elems, c->nel, 0,
                                        c->nnd, c->ph, ASM_LEVELS, last, 1, 0, SEL_FAR,
                                        c->d_far_pairs, nullptr, c->stream));
            prof_end(c, pw, 0, 0);
            const int pe = prof_begin(c, TDBEM_K_ASSEMBLE_F32);
            CUDA_TRY(launch_assemble_far_rows(c->d_coords, c->d_ien, c->d_color_elems,
                                              c->d_color_start, ncol, c->nnd, c->nel, c->nq,
                                              c->d_geomf, c->d_geom, c->d_coordf, c->ph, last,
                                              c->d_far_pairs, o64,
                                              count ? c->d_far_items : nullptr, c->stream, 1,
                                              true));
            prof_end(c, pe, 0, 0);
            c->launches += 2;
        }
        // the C term, regular elements in FP32 (the FP32 store gets it with levels 0/1)
        const int pc = prof_begin(c, TDBEM_K_AUX);
        CUDA_TRY(launch_cterm(c->d_coords, c->d_ien, c->ennd, c->nel, 0, c->nnd, c->nq, c->d_gx,
                              c->d_gw, c->d_geom, c->ph, c->d_cterm, c->stream, true,
                              c->d_geomf));
        CUDA_TRY(launch_cterm_apply(c->d_cterm, 0, c->nnd, c->dt, c->if_ext, ASM_LEVELS, o64,
                                    c->stream));
        prof_end(c, pc, 0, 0);
        c->launches += 2;
        // The march's FP32 inverses need only levels 0/1, alpha and the UBC dofs: made
        // here on the side streams while the near and far fields run (the march reuses
        // them while alpha, the UBC dofs and the levels stay as they are).
        const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
        const double lhs_c[2][2] = {{1.0, 0.0}, {2 * a1 + a3, a1}};
        const int ninv = mixed_ninv(nsteps, lhs_c);
        InvResult ir;  // written by the helper thread: declared before its joiner
        EventTimer tf;
        std::thread inv_thread;
        struct Joiner {
            std::thread& t;
            ~Joiner() {
                if (t.joinable()) t.join();
            }
        } joiner{inv_thread};
        int pf = -1;
        if (split) {
            int rc = upload_bc(c);
            if (rc == TDBEM_OK) rc = prepare_inverses(c, ninv);
            if (rc != TDBEM_OK) return rc;
            CUDA_TRY(cudaEventRecord(c->ev_fork, c->stream));
            CUDA_TRY(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
            tf.start(c->stream2);
            pf = prof_begin_on(c, TDBEM_K_FACTOR, c->stream2);
            inv_thread = std::thread([&] {
                cudaSetDevice(c->device);
                run_inverses(c, ninv, lhs_c, c->stream2, c->stream3, ir);
            });
        }
        // near pairs (FP64 quadrature into the FP32 store), colour by colour, from level
        // 2 on: levels 0/1 are the FP64 ones, cast at the end
        for (int col = 0; col < ncol; col++) {
            const int rc = assemble_color(c, col, 0, c->nnd, ASM_LEVELS, last, c->M, 2,
                                          split ? SEL_NEAR : SEL_ALL, o32);
            if (rc != TDBEM_OK) return rc;
        }
        if (split) {
            // far pairs: windows of every (node, element) pair, elements in colour order,
            // then one row-local FP32 launch
            const int pw = prof_begin(c, TDBEM_K_AUX);
            CUDA_TRY(launch_pair_window(c->d_coords, c->d_ien, 4, c->d_color_elems, c->nel, 0,
                                        c->nnd, c->ph, ASM_LEVELS, last, c->M, 2, SEL_FAR,
                                        c->d_far_pairs, nullptr, c->stream));
            prof_end(c, pw, 0, 0);
            const int pe = prof_begin(c, TDBEM_K_ASSEMBLE_F32);
            CUDA_TRY(launch_assemble_far_rows(c->d_coords, c->d_ien, c->d_color_elems,
                                              c->d_color_start, ncol, c->nnd, c->nel, c->nq,
                                              c->d_geomf, c->d_geom, c->d_coordf, c->ph, last,
                                              c->d_far_pairs, o32,
                                              count ? c->d_far_items : nullptr, c->stream));
            prof_end(c, pe, 0, 0);
            c->launches += 2;
            if (count && pe >= 0) {
                unsigned long long n = 0;
                CUDA_TRY(cudaMemcpyAsync(&n, c->d_far_items, sizeof(n), cudaMemcpyDeviceToHost,
                                         c->stream));
                CUDA_TRY(cudaStreamSynchronize(c->stream));
                c->prof_pending[pe].bytes = (double)n * 4 * 45 * 4.0 * 2;
                c->prof_pending[pe].flops = (double)n * c->nq * c->nq * kFlopsPerItemPointF32;
            }
        }
        // levels 0/1 (with the C term) from the FP64 pair
        CUDA_TRY(launch_cast_levels01(c->d_G01, c->d_H01, D, (int)ldf, c->d_Gf, c->d_Hf,
                                      c->stream));
        c->launches += 1;
        if (split) {
            inv_thread.join();  // its streams are synchronised when it returns
            const double DD = (double)D * D;
            prof_end_on(c, pf, ninv * 2.0 * 4 * DD, ninv * 2.0 * DD * D, c->stream2);
            c->timings[1] = tf.stop_ms(c->stream2);
            const int rc = finish_inverses(c, ninv, ir);
            if (rc != TDBEM_OK) return rc;
        }
    }
    c->timings[0] = tm.stop_ms(c->stream);
    CUDA_TRY(cudaGetLastError());
    prof_flush(c);
    c->levels_last = last;
    c->mtc_planes_valid = false;  // the merged planes follow the levels
    return TDBEM_OK;
}

int tdbem_get_level(tdbem_ctx* c, int k, int which, double* host_out) {
    if (!c || !host_out) return fail(TDBEM_ERR_ARG, "null argument");
    if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "levels not assembled");
    if (k < 0 || k > c->M || (which != 0 && which != 1))
        return fail(TDBEM_ERR_ARG, "level %d / which %d out of range", k, which);
    const size_t stride = (size_t)c->D * c->D;
    if (c->level_precision == TDBEM_FP64) {
        const double* src = (which == 0 ? c->d_G : c->d_H) + k * stride;
        CUDA_TRY(cudaMemcpyAsync(host_out, src, sizeof(double) * stride, cudaMemcpyDeviceToHost,
                                 c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else {
        std::vector<float> tmp(stride);
        const float* src = (which == 0 ? c->d_Gf : c->d_Hf) + (size_t)k * c->D * c->ldf;
        CUDA_TRY(cudaMemcpy2DAsync(tmp.data(), sizeof(float) * c->D, src, sizeof(float) * c->ldf,
                                   sizeof(float) * c->D, c->D, cudaMemcpyDeviceToHost,
                                   c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < stride; i++) host_out[i] = tmp[i];
    }
    return TDBEM_OK;
}

int tdbem_set_bc(tdbem_ctx* c, const int* ubc_dofs, const double* ubc_vals, int n_u,
                 const int* fbc_dofs, const double* fbc_vals, int n_f) {
    if (!c || n_u < 0 || n_f < 0 || (n_u && (!ubc_dofs || !ubc_vals)) ||
        (n_f && (!fbc_dofs || !fbc_vals)))
        return fail(TDBEM_ERR_ARG, "invalid boundary-condition arrays");
    for (int i = 0; i < n_u; i++)
        if (ubc_dofs[i] < 0 || ubc_dofs[i] >= c->D)
            return fail(TDBEM_ERR_ARG, "UBC dof %d out of range", ubc_dofs[i]);
    for (int i = 0; i < n_f; i++)
        if (fbc_dofs[i] < 0 || fbc_dofs[i] >= c->D)
            return fail(TDBEM_ERR_ARG, "FBC dof %d out of range", fbc_dofs[i]);
    c->ubc.assign(ubc_dofs, ubc_dofs + n_u);
    c->ubc_v.assign(ubc_vals, ubc_vals + n_u);
    c->fbc.assign(fbc_dofs, fbc_dofs + n_f);
    c->fbc_v.assign(fbc_vals, fbc_vals + n_f);
    c->mtc_planes_valid = false;  // the merged levels follow the BC types and values
    return TDBEM_OK;
}

int tdbem_set_alpha(tdbem_ctx* c, double a1, double a2) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    // SolverStepLinearT::Solve_Averaging range check (SolverStepLinearT.cpp:317-322)
    if (!(a1 >= 0 && a1 <= 1 && a2 >= 0 && a2 < 1 && a1 + a2 <= 1))
        return fail(TDBEM_ERR_ARG, "Alpha is out of range (alpha_1=%g alpha_2=%g)", a1, a2);
    c->a1 = a1;
    c->a2 = a2;
    return TDBEM_OK;
}

int tdbem_set_load_history(tdbem_ctx* c, const double* amp, int nsteps) {
    if (!c || nsteps < 0 || (nsteps && !amp)) return fail(TDBEM_ERR_ARG, "invalid load history");
    c->amp.assign(amp, amp + nsteps);
    return TDBEM_OK;
}

int tdbem_march(tdbem_ctx* c, int numstep, double* u_hist, double* t_hist) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (numstep < 1) return fail(TDBEM_ERR_ARG, "numstep must be >= 1");
    if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "levels not assembled");
    if (c->levels_last < std::min(c->M, numstep))
        return fail(TDBEM_ERR_STATE, "levels assembled for %d steps, %d needed", c->levels_last,
                    std::min(c->M, numstep));
    if (!c->amp.empty() && (int)c->amp.size() < numstep)
        return fail(TDBEM_ERR_ARG, "load history has %zu values, %d steps", c->amp.size(),
                    numstep);
    const int D = c->D;
    const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
    const int rc0 = upload_bc(c);
    if (rc0 != TDBEM_OK) return rc0;
    cudaStream_t s = c->stream;
    if (c->hist_steps != numstep) {
        dfree(c->d_u);
        dfree(c->d_t);
        CUDA_TRY(dalloc(&c->d_u, (size_t)(numstep + 1) * D));
        CUDA_TRY(dalloc(&c->d_t, (size_t)(numstep + 1) * D));
        c->hist_steps = numstep;
    }
    CUDA_TRY(cudaMemsetAsync(c->d_u, 0, sizeof(double) * (numstep + 1) * D, s));
    CUDA_TRY(cudaMemsetAsync(c->d_t, 0, sizeof(double) * (numstep + 1) * D, s));

    // LHS of step 2 (SolverStepLinearT.cpp:357-371) and of steps >= 3 (381-393)
    const double lhs_c[2][2] = {{1.0, 0.0}, {2 * a1 + a3, a1}};
    if (c->level_precision == TDBEM_MIXED) {
        const int rc = march_mixed(c, numstep, lhs_c);
        if (rc != TDBEM_OK) return rc;
        if (u_hist)
            CUDA_TRY(cudaMemcpyAsync(u_hist, c->d_u, sizeof(double) * (numstep + 1) * D,
                                     cudaMemcpyDeviceToHost, s));
        if (t_hist)
            CUDA_TRY(cudaMemcpyAsync(t_hist, c->d_t, sizeof(double) * (numstep + 1) * D,
                                     cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        prof_flush(c);
        return TDBEM_OK;
    }
    return march_fp64(c, numstep, lhs_c, u_hist, t_hist);
}

int tdbem_march_batch(tdbem_ctx* c, int numstep, int nrhs, const double* traction,
                      const double* amp, double* u_hist, double* t_hist) {
    if (!c || !traction) return fail(TDBEM_ERR_ARG, "null argument");
    if (numstep < 1 || nrhs < 1) return fail(TDBEM_ERR_ARG, "numstep and nrhs must be >= 1");
    if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "levels not assembled");
    if (c->level_precision != TDBEM_MIXED)
        return fail(TDBEM_ERR_UNSUPPORTED,
                    "batched marching runs on FP32 levels: assemble with TDBEM_MIXED");
    if (c->levels_last < std::min(c->M, numstep))
        return fail(TDBEM_ERR_STATE, "levels assembled for %d steps, %d needed", c->levels_last,
                    std::min(c->M, numstep));
    const int D = c->D, M = c->M, C = nrhs;
    if ((size_t)C * D > (size_t)INT32_MAX / 2)
        return fail(TDBEM_ERR_ARG, "nrhs x D = %zu is too large", (size_t)C * D);
    const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
    const int rc0 = upload_bc(c);
    if (rc0 != TDBEM_OK) return rc0;
    cudaStream_t s = c->stream;
    const size_t CD = (size_t)C * D;
    const int ldw = batch_ldw(D);
    if (c->batch_C != C || c->batch_steps != numstep) {
        free_batch(c);
        CUDA_TRY(dalloc(&c->d_bu, (size_t)(numstep + 1) * CD));
        CUDA_TRY(dalloc(&c->d_bt, (size_t)(numstep + 1) * CD));
        CUDA_TRY(dalloc(&c->d_btrac, CD));
        CUDA_TRY(dalloc(&c->d_bamp, (size_t)C * numstep));
        CUDA_TRY(dalloc(&c->d_bWt, (size_t)(M + 1) * C * ldw));
        CUDA_TRY(dalloc(&c->d_bWu, (size_t)(M + 1) * C * ldw));
        int smax = batch_apply_splits(D, C);
        for (int nlev = 2; nlev <= M + 1; nlev++)
            smax = std::max({smax, batch_conv_splits(nlev, D, C),
                             tc_conv_splits(nlev, D, C, 1 << 30, 1)});
        c->bpart_cap = (size_t)smax * CD;
        CUDA_TRY(dalloc(&c->d_bpart, c->bpart_cap));
        CUDA_TRY(dalloc(&c->d_brhs, CD));
        CUDA_TRY(dalloc(&c->d_bx, CD));
        CUDA_TRY(dalloc(&c->d_br, CD));
        c->batch_C = C;
        c->batch_steps = numstep;
    }
    CUDA_TRY(cudaMemcpyAsync(c->d_btrac, traction, sizeof(double) * CD, cudaMemcpyHostToDevice, s));
    if (amp)
        CUDA_TRY(cudaMemcpyAsync(c->d_bamp, amp, sizeof(double) * C * numstep,
                                 cudaMemcpyHostToDevice, s));
    const double* d_amp = amp ? c->d_bamp : nullptr;
    CUDA_TRY(cudaMemsetAsync(c->d_bu, 0, sizeof(double) * (numstep + 1) * CD, s));
    CUDA_TRY(cudaMemsetAsync(c->d_bt, 0, sizeof(double) * (numstep + 1) * CD, s));
    c->launches += 0;

    const double lhs_c[2][2] = {{1.0, 0.0}, {2 * a1 + a3, a1}};
    const int rc = mixed_inverses(c, numstep, lhs_c);
    if (rc != TDBEM_OK) return rc;

    // tcgen05 engine: the merged level planes of the single march (the cases share the
    // boundary-condition types) and, per case, its known tractions times every level
    const bool tc = c->batch_engine == TDBEM_ENGINE_TCGEN05;
    const int Lw = M + 1;
    if (tc) {
        if (!c->d_tc_err) CUDA_TRY(dalloc(&c->d_tc_err, 1));
        CUDA_TRY(cudaMemsetAsync(c->d_tc_err, 0, sizeof(int), s));
        const int rm = ensure_merged_levels(c);
        if (rm != TDBEM_OK) return rm;
        const size_t wb = tc_w_bytes(D, C, Lw, 1);
        if (c->tc_W_bytes < wb) {
            if (c->d_tc_W) cudaFree(c->d_tc_W);
            c->d_tc_W = nullptr;
            c->tc_W_bytes = 0;
            CUDA_TRY(cudaMalloc(&c->d_tc_W, wb));
            c->tc_W_bytes = wb;
        }
        if (!make_tc_maps(c->d_mtc_planes, D, M + 1, c->d_tc_W, C, Lw, &c->tc_maps, 1))
            return fail(TDBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed for the batched planes");
        if (!c->d_bkt) {
            CUDA_TRY(dalloc(&c->d_bkt, 2 * CD));
            CUDA_TRY(dalloc(&c->d_bGK, (size_t)(M + 1) * CD));
            CUDA_TRY(dalloc(&c->d_bGL, 2 * CD));
        }
        const int pk = prof_begin(c, TDBEM_K_AUX);
        CUDA_TRY(launch_batch_known_tractions(c->d_btrac, c->d_is_ubc, D, C, c->d_bkt,
                                              c->d_bkt + CD, s));
        CUDA_TRY(levels_times_columns(c->d_Gf, c->ldf, D, M + 1, c->d_bkt, C, c->d_bGK,
                                      c->device, s));
        CUDA_TRY(levels_times_columns(c->d_Gf, c->ldf, D, std::min(2, M + 1), c->d_bkt + CD, C,
                                      c->d_bGL, c->device, s));
        prof_end(c, pk, (M + 3) * (double)D * c->ldf * 4, 2.0 * (M + 3) * (double)D * D * C);
        c->launches += 3;
    }

    EventTimer tmr;
    tmr.start(s);
    const size_t lstride = (size_t)D * c->ldf;
    const double DD = (double)D * D;
    const int sp = batch_apply_splits(D, C);
    for (int st = 1; st <= numstep - 1; st++) {
        const int L = std::min(M, std::max(1, st));
        const int nlev = L + 1;
        const double c0 = st == 1 ? 1.0 : lhs_c[1][0];
        const double c1 = st == 1 ? 0.0 : lhs_c[1][1];
        int pe;
        if (tc) {  // merged levels: the unknowns' history, then the known values' part
            CUDA_TRY(launch_build_w_batch_merged(c->d_bu, c->d_bt, c->d_is_ubc, D, C, st, nlev,
                                                 Lw, a1, a2, a3, c->d_tc_W, s));
            const int splits = tc_conv_splits(nlev, D, C, 1 << 30, 1);
            const double ldb = tc_ldb(D), cp = tc_cases_pad(C);
            pe = prof_begin(c, TDBEM_K_CONV_BATCH);
            CUDA_TRY(launch_conv_tc(c->tc_maps, D, M + 1, Lw, nlev, C, c->d_bpart, splits,
                                    c->d_tc_err, s, 1));
            prof_end(c, pe, nlev * (double)D * ldb * 4 + nlev * cp * ldb * 4,
                     nlev * 2.0 * DD * C);
            CUDA_TRY(launch_reduce_cols(c->d_bpart, splits, C, D, nullptr, c->d_brhs, s));
            const double* hu = c->d_mtc_known + (size_t)2 * (M + 1) * D;  // H^f ubc
            CUDA_TRY(launch_known_batch(c->d_bGK, c->d_bGL, hu, D, C, M + 1, st, a1, a2, a3, c0,
                                        c1, d_amp, numstep, c->d_brhs, s));
            c->launches += 1;
        } else {
            CUDA_TRY(launch_build_w_batch(c->d_bu, c->d_bt, D, C, st, nlev, a1, a2, a3, c0, c1,
                                          d_amp, numstep, c->d_btrac, c->d_is_ubc, c->d_ubc_map,
                                          ldw, c->d_bWt, c->d_bWu, s));
            const int splits = batch_conv_splits(nlev, D, C);
            pe = prof_begin(c, TDBEM_K_CONV_BATCH);
            CUDA_TRY(launch_conv_mma(c->d_Gf, c->d_Hf, lstride, c->ldf, D, nlev, c->d_bWt,
                                     c->d_bWu, ldw, C, c->d_bpart, splits, s));
            prof_end(c, pe, nlev * 2.0 * (double)lstride * 4 + nlev * 2.0 * C * ldw * 4,
                     nlev * 4.0 * DD * C);
            CUDA_TRY(launch_reduce_cols(c->d_bpart, splits, C, D, nullptr, c->d_brhs, s));
        }
        pe = prof_begin(c, TDBEM_K_SOLVE_BATCH);
        const int v = st == 1 ? 0 : 1;
        CUDA_TRY(launch_apply_cols(c->d_inv32[v], 0, D, c->d_brhs, C, c->d_bpart, sp, s));
        CUDA_TRY(launch_reduce_cols(c->d_bpart, sp, C, D, nullptr, c->d_bx, s));
        for (int it = 0; it < c->batch_refine; it++) {
            CUDA_TRY(launch_apply_cols(c->d_Hc64[v], 1, D, c->d_bx, C, c->d_bpart, sp, s));
            CUDA_TRY(launch_reduce_cols(c->d_bpart, sp, C, D, c->d_brhs, c->d_br, s));
            CUDA_TRY(launch_apply_cols(c->d_inv32[v], 0, D, c->d_br, C, c->d_bpart, sp, s));
            CUDA_TRY(launch_reduce_cols(c->d_bpart, sp, C, D, c->d_bx, c->d_bx, s));
        }
        CUDA_TRY(launch_update_batch(c->d_bx, D, C, st, c->d_is_ubc, c->d_ubc_map, c->d_btrac,
                                     d_amp, numstep, c->d_bu, c->d_bt, s));
        prof_end(c, pe, DD * 4 * (1 + c->batch_refine) + DD * 8 * c->batch_refine,
                 2.0 * DD * C * (1 + 2 * c->batch_refine));
        c->launches += 6 + 4LL * c->batch_refine;
    }
    c->timings[2] = tmr.stop_ms(s);
    if (tc) {
        int code = 0;
        CUDA_TRY(cudaMemcpyAsync(&code, c->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        if (code)
            return fail(TDBEM_ERR_CUDA,
                        "tensor-core convolution: a pipeline wait timed out (code %d)", code);
    }
    if (u_hist)
        CUDA_TRY(cudaMemcpyAsync(u_hist, c->d_bu, sizeof(double) * (numstep + 1) * CD,
                                 cudaMemcpyDeviceToHost, s));
    if (t_hist)
        CUDA_TRY(cudaMemcpyAsync(t_hist, c->d_bt, sizeof(double) * (numstep + 1) * CD,
                                 cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    prof_flush(c);
    return TDBEM_OK;
}

int tdbem_update_gh_linear(tdbem_ctx* c, int step, int node_lo, int node_hi, const double* G_I,
                           const double* G_J, const double* H_I, const double* H_J) {
    if (!c || !G_I || !G_J || !H_I || !H_J) return fail(TDBEM_ERR_ARG, "null argument");
    if (step < 1) return fail(TDBEM_ERR_ARG, "step must be >= 1");
    if (node_lo < 0 || node_hi >= c->nnd || node_lo > node_hi)
        return fail(TDBEM_ERR_ARG, "node range [%d, %d] invalid", node_lo, node_hi);
    if (step > c->M) return TDBEM_OK;  // SolverStepLinearT.cpp:66: only steps <= MaxStep
    const int rc = ensure_fp64_store(c);
    if (rc != TDBEM_OK) return rc;
    const int D = c->D;
    const size_t rows = 3 * (size_t)(node_hi - node_lo + 1), n = rows * D;
    const size_t off = 3 * (size_t)node_lo * D, lev = (size_t)D * D;
    cudaStream_t s = c->stream;
    if (c->upd_tmp_cap < n) {
        dfree(c->d_upd_tmp);
        c->upd_tmp_cap = 0;
        CUDA_TRY(dalloc(&c->d_upd_tmp, n));
        c->upd_tmp_cap = n;
    }
    const double* J[2] = {G_J, H_J};
    const double* I[2] = {G_I, H_I};
    double* store[2] = {c->d_G, c->d_H};
    for (int m = 0; m < 2; m++) {
        double* lvl_prev = store[m] + (size_t)(step - 1) * lev + off;  // level step-1 <- J part
        double* lvl_cur = store[m] + (size_t)step * lev + off;         // level step   <- I part
        if (step == 1) {
            CUDA_TRY(cudaMemcpyAsync(lvl_prev, J[m], sizeof(double) * n, cudaMemcpyHostToDevice, s));
        } else {
            CUDA_TRY(cudaMemcpyAsync(c->d_upd_tmp, J[m], sizeof(double) * n,
                                     cudaMemcpyHostToDevice, s));
            CUDA_TRY(launch_add_inplace(lvl_prev, c->d_upd_tmp, n, s));
            c->launches += 1;
        }
        CUDA_TRY(cudaMemcpyAsync(lvl_cur, I[m], sizeof(double) * n, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaStreamSynchronize(s));  // the temporary is reused for H
    }
    c->levels_last = std::max(c->levels_last, step);
    c->mtc_planes_valid = false;
    c->step_inv_ready[0] = c->step_inv_ready[1] = false;
    return TDBEM_OK;
}

int tdbem_march_begin(tdbem_ctx* c, int numstep) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (numstep < 1) return fail(TDBEM_ERR_ARG, "numstep must be >= 1");
    if (!c->amp.empty() && (int)c->amp.size() < numstep)
        return fail(TDBEM_ERR_ARG, "load history has %zu values, %d steps", c->amp.size(),
                    numstep);
    const int rc = upload_bc(c);
    if (rc != TDBEM_OK) return rc;
    const int D = c->D;
    cudaStream_t s = c->stream;
    if (c->hist_steps != numstep) {
        dfree(c->d_u);
        dfree(c->d_t);
        CUDA_TRY(dalloc(&c->d_u, (size_t)(numstep + 1) * D));
        CUDA_TRY(dalloc(&c->d_t, (size_t)(numstep + 1) * D));
        c->hist_steps = numstep;
    }
    CUDA_TRY(cudaMemsetAsync(c->d_u, 0, sizeof(double) * (numstep + 1) * D, s));
    CUDA_TRY(cudaMemsetAsync(c->d_t, 0, sizeof(double) * (numstep + 1) * D, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    c->step_numstep = numstep;
    c->step_inv_ready[0] = c->step_inv_ready[1] = false;
    return TDBEM_OK;
}

int tdbem_march_step(tdbem_ctx* c, int curr_step, double* u, double* t) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (c->step_numstep < 1) return fail(TDBEM_ERR_STATE, "tdbem_march_begin has not run");
    if (curr_step < 1 || curr_step > c->step_numstep)
        return fail(TDBEM_ERR_ARG, "step %d outside 1..%d", curr_step, c->step_numstep);
    const int D = c->D, st = curr_step - 1;
    cudaStream_t s = c->stream;
    if (st >= 1) {
        if (c->level_precision != TDBEM_FP64)
            return fail(TDBEM_ERR_UNSUPPORTED, "stepwise marching runs on FP64 levels");
        if (c->levels_last < std::min(c->M, curr_step))
            return fail(TDBEM_ERR_STATE, "levels hold %d steps, step %d needs %d", c->levels_last,
                        curr_step, std::min(c->M, curr_step));
        const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
        const double lhs_c[2][2] = {{1.0, 0.0}, {2 * a1 + a3, a1}};
        const int v = st == 1 ? 0 : 1;
        if (!c->step_inv_ready[v]) {
            const int rc = fp64_inverse(c, v, lhs_c);
            if (rc != TDBEM_OK) return rc;
            c->step_inv_ready[v] = true;
        }
        const int rc = fp64_step(c, st, lhs_c);
        if (rc != TDBEM_OK) return rc;
    }
    if (u)
        CUDA_TRY(cudaMemcpyAsync(u, c->d_u + (size_t)st * D, sizeof(double) * D,
                                 cudaMemcpyDeviceToHost, s));
    if (t)
        CUDA_TRY(cudaMemcpyAsync(t, c->d_t + (size_t)st * D, sizeof(double) * D,
                                 cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    prof_flush(c);
    return TDBEM_OK;
}

// Level checkpoint: a 64-byte header (magic, version, D, M, precision, levels held,
// row stride) followed by the raw level store (FP64: G then H, (M+1) x D x D;
// mixed: FP32 G then H, (M+1) x D x ld, then FP64 levels 0-1 of G and H).
namespace {
constexpr char kCkptMagic[8] = {'T', 'D', 'B', 'E', 'M', 'L', 'V', 'L'};
struct CkptHeader {
    char magic[8];
    int32_t version, D, M, precision, levels_last, ld;
    int32_t pad[8];
};
static_assert(sizeof(CkptHeader) == 64, "checkpoint header is 64 bytes");

struct LevelArrays {
    void* dev[4];
    size_t bytes[4];
    int n;
};

LevelArrays level_arrays(tdbem_ctx* c) {
    LevelArrays a{};
    const size_t L = (size_t)c->M + 1, D = c->D;
    if (c->level_precision == TDBEM_FP64) {
        a.n = 2;
        a.dev[0] = c->d_G;
        a.dev[1] = c->d_H;
        a.bytes[0] = a.bytes[1] = L * D * D * 8;
    } else {
        a.n = 4;
        a.dev[0] = c->d_Gf;
        a.dev[1] = c->d_Hf;
        a.bytes[0] = a.bytes[1] = L * D * c->ldf * 4;
        a.dev[2] = c->d_G01;
        a.dev[3] = c->d_H01;
        a.bytes[2] = a.bytes[3] = 2 * D * D * 8;
    }
    return a;
}
}  // namespace

int tdbem_export_levels(tdbem_ctx* c, const char* path) {
    if (!c || !path) return fail(TDBEM_ERR_ARG, "null argument");
    if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "levels not assembled");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s for writing", path);
    CkptHeader h{};
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.D = c->D;
    h.M = c->M;
    h.precision = c->level_precision;
    h.levels_last = c->levels_last;
    h.ld = c->level_precision == TDBEM_FP64 ? c->D : c->ldf;
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    const LevelArrays a = level_arrays(c);
    std::vector<unsigned char> buf;
    const size_t chunk = (size_t)64 << 20;
    for (int k = 0; k < a.n && ok; k++)
        for (size_t o = 0; o < a.bytes[k] && ok; o += chunk) {
            const size_t b = std::min(chunk, a.bytes[k] - o);
            buf.resize(b);
            if (cudaMemcpy(buf.data(), static_cast<unsigned char*>(a.dev[k]) + o, b,
                           cudaMemcpyDeviceToHost) != cudaSuccess) {
                std::fclose(f);
                return fail(TDBEM_ERR_CUDA, "level copy to host failed");
            }
            ok = std::fwrite(buf.data(), 1, b, f) == b;
        }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(TDBEM_ERR_ARG, "write to %s failed", path);
    return TDBEM_OK;
}

int tdbem_import_levels(tdbem_ctx* c, const char* path) {
    if (!c || !path) return fail(TDBEM_ERR_ARG, "null argument");
    c->inv_valid = false;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s", path);
    CkptHeader h{};
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 ||
        h.version != 1) {
        std::fclose(f);
        return fail(TDBEM_ERR_ARG, "%s is not a level checkpoint", path);
    }
    if (h.D != c->D || h.M != c->M) {
        std::fclose(f);
        return fail(TDBEM_ERR_ARG, "checkpoint is for D=%d, M=%d; this mesh has D=%d, M=%d", h.D,
                    h.M, c->D, c->M);
    }
    int rc = TDBEM_OK;
    if (h.precision == TDBEM_FP64) {
        rc = ensure_fp64_store(c);
    } else if (h.precision == TDBEM_MIXED && h.ld == mixed_ld(c->D)) {
        if (c->level_precision != TDBEM_MIXED || !c->d_Gf) {
            free_levels(c);
            const size_t n = (size_t)(c->M + 1) * c->D * mixed_ld(c->D);
            cudaError_t e = dalloc(&c->d_Gf, n);
            if (e == cudaSuccess) e = dalloc(&c->d_Hf, n);
            if (e == cudaSuccess) e = dalloc(&c->d_G01, 2 * (size_t)c->D * c->D);
            if (e == cudaSuccess) e = dalloc(&c->d_H01, 2 * (size_t)c->D * c->D);
            if (e != cudaSuccess) rc = fail(TDBEM_ERR_NOMEM, "level allocation failed");
            c->ldf = mixed_ld(c->D);
            c->level_precision = TDBEM_MIXED;
        }
    } else {
        rc = fail(TDBEM_ERR_ARG, "checkpoint precision %d / row stride %d not supported",
                  h.precision, h.ld);
    }
    if (rc != TDBEM_OK) {
        std::fclose(f);
        return rc;
    }
    const LevelArrays a = level_arrays(c);
    std::vector<unsigned char> buf;
    const size_t chunk = (size_t)64 << 20;
    bool ok = true;
    for (int k = 0; k < a.n && ok; k++)
        for (size_t o = 0; o < a.bytes[k] && ok; o += chunk) {
            const size_t b = std::min(chunk, a.bytes[k] - o);
            buf.resize(b);
            ok = std::fread(buf.data(), 1, b, f) == b &&
                 cudaMemcpy(static_cast<unsigned char*>(a.dev[k]) + o, buf.data(), b,
                            cudaMemcpyHostToDevice) == cudaSuccess;
        }
    std::fclose(f);
    if (!ok) {
        free_levels(c);
        return fail(TDBEM_ERR_ARG, "%s is truncated or the copy failed", path);
    }
    c->levels_last = h.levels_last;
    c->mtc_planes_valid = false;
    c->step_inv_ready[0] = c->step_inv_ready[1] = false;
    return TDBEM_OK;
}

int tdbem_write_gh(const char* name_prefix, int step, int num_row, int num_column,
                   const double* data) {
    if (!name_prefix || !data || num_row < 0 || num_column < 0)
        return fail(TDBEM_ERR_ARG, "invalid arguments");
    char path[4096];
    std::snprintf(path, sizeof(path), "%s%d.txt", name_prefix, step);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s", path);
    bool ok = true;
    for (int i = 0; i < num_row && ok; i++) {
        for (int j = 0; j < num_column && ok; j++)
            ok = std::fprintf(f, "%15.5e", data[(size_t)i * num_column + j]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TDBEM_OK : fail(TDBEM_ERR_ARG, "write to %s failed", path);
}

}  // extern "C"

namespace {
// Runs fn(i) for i < n on n host threads (each sets the context's device) and
// returns the first failure with its message.
template <typename F>
int parallel_contexts(tdbem_ctx* const* ctxs, int n, F fn) {
    std::vector<int> rc(n, TDBEM_OK);
    std::vector<std::string> msg(n);
    std::vector<std::thread> th;
    th.reserve(n);
    for (int i = 0; i < n; i++)
        th.emplace_back([&, i] {
            cudaSetDevice(ctxs[i]->device);
            rc[i] = fn(i);
            if (rc[i] != TDBEM_OK) msg[i] = tdbem_last_error();
        });
    for (auto& t : th) t.join();
    for (int i = 0; i < n; i++)
        if (rc[i] != TDBEM_OK) return fail(rc[i], "mesh %d: %s", i, msg[i].c_str());
    return TDBEM_OK;
}
}  // namespace

extern "C" {

int tdbem_assemble_group(tdbem_ctx* const* ctxs, int n, const int* nsteps, int precision) {
    if (!ctxs || !nsteps || n < 1) return fail(TDBEM_ERR_ARG, "invalid group");
    if (precision != TDBEM_FP64 && precision != TDBEM_MIXED)
        return fail(TDBEM_ERR_ARG, "unknown precision %d", precision);
    for (int i = 0; i < n; i++) {
        if (!ctxs[i]) return fail(TDBEM_ERR_ARG, "null context %d", i);
        if (ctxs[i]->device != ctxs[0]->device)
            return fail(TDBEM_ERR_ARG, "the group's contexts are on different devices");
        if (nsteps[i] < 1) return fail(TDBEM_ERR_ARG, "nsteps[%d] must be >= 1", i);
        for (int j = 0; j < i; j++)
            if (ctxs[j] == ctxs[i]) return fail(TDBEM_ERR_ARG, "context %d appears twice", i);
    }
    bool any_q8 = false;
    for (int i = 0; i < n; i++) any_q8 = any_q8 || ctxs[i]->ennd == 8;
    // mixed: near/far split per mesh; 8-node meshes: the single-mesh launches (the
    // grouped kernels are written for 4-node elements).  The meshes' streams overlap.
    if (precision == TDBEM_MIXED || any_q8)
        return parallel_contexts(ctxs, n, [&](int i) {
            return tdbem_assemble_levels(ctxs[i], nsteps[i], precision);
        });
    tdbem_ctx* c0 = ctxs[0];
    cudaStream_t s = c0->stream;
    EventTimer tm;
    int ncol = 0;
    for (int i = 0; i < n; i++) {
        tdbem_ctx* c = ctxs[i];
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        if (c->level_precision != TDBEM_FP64 || !c->d_G) {
            free_levels(c);
            const size_t nn = (size_t)(c->M + 1) * c->D * c->D;
            CUDA_TRY(dalloc(&c->d_G, nn));
            CUDA_TRY(dalloc(&c->d_H, nn));
            c->level_precision = TDBEM_FP64;
        }
        const size_t total = (size_t)(c->M + 1) * c->D * c->D;
        CUDA_TRY(cudaMemsetAsync(c->d_G, 0, 8 * total, s));
        CUDA_TRY(cudaMemsetAsync(c->d_H, 0, 8 * total, s));
        ncol = std::max(ncol, (int)c->color_start.size() - 1);
    }
    tm.start(s);
    // descriptors of every mesh; per colour only the meshes that have it
    std::vector<GroupAsm> all(n);
    unsigned node_total = 0;
    size_t pair_max = 0;
    for (int i = 0; i < n; i++) {
        tdbem_ctx* c = ctxs[i];
        GroupAsm& g = all[i];
        g = GroupAsm{};
        g.coords = c->d_coords;
        g.ien = c->d_ien;
        g.nnd = c->nnd;
        g.nel = c->nel;
        g.nq = c->nq;
        g.gx = c->d_gx;
        g.gw = c->d_gw;
        g.geom = c->d_geom;
        g.ph = c->ph;
        g.level_last = std::min(c->M, nsteps[i]);
        g.level_cap = c->M;
        g.if_ext = c->if_ext;
        g.out.G0 = c->d_G;
        g.out.H0 = c->d_H;
        g.out.level_stride = (size_t)c->D * c->D;
        g.out.D = c->D;
        g.out.ld = c->D;
        g.node_begin = node_total;
        g.cbuf = c->d_cterm;
        node_total += (unsigned)c->nnd;
    }
    for (int col = 0; col < ncol; col++) {
        size_t np = 0;
        for (int i = 0; i < n; i++) {
            const tdbem_ctx* c = ctxs[i];
            if (col + 1 < (int)c->color_start.size())
                np += (size_t)c->nnd * (c->color_start[col + 1] - c->color_start[col]);
        }
        pair_max = std::max(pair_max, np);
    }
    if (pair_max >= ((size_t)1 << 31)) return fail(TDBEM_ERR_UNSUPPORTED, "group too large");
    PairInfo* d_pairs = nullptr;
    unsigned *d_counts = nullptr, *d_offsets = nullptr;
    GroupAsm* d_gm = nullptr;
    void* d_tmp = nullptr;
    const size_t tmp_bytes = std::max<size_t>(scan_temp_bytes((unsigned)std::max<size_t>(pair_max, 1)), 16);
    struct Free {
        PairInfo*& a;
        unsigned*& b;
        unsigned*& c;
        GroupAsm*& d;
        void*& e;
        ~Free() {
            dfree(a);
            dfree(b);
            dfree(c);
            dfree(d);
            if (e) cudaFree(e);
        }
    } guard{d_pairs, d_counts, d_offsets, d_gm, d_tmp};
    CUDA_TRY(dalloc(&d_pairs, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_counts, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_offsets, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_gm, (size_t)n));
    CUDA_TRY(cudaMalloc(&d_tmp, tmp_bytes));
    long long launches = 0;
    for (int col = 0; col < ncol; col++) {
        std::vector<GroupAsm> gl;
        unsigned np = 0;
        for (int i = 0; i < n; i++) {
            const tdbem_ctx* c = ctxs[i];
            if (col + 1 >= (int)c->color_start.size()) continue;
            const int e0 = c->color_start[col], ne = c->color_start[col + 1] - e0;
            if (ne == 0) continue;
            GroupAsm g = all[i];
            g.elems = c->d_color_elems + e0;
            g.ne = ne;
            g.pair_begin = np;
            np += (unsigned)(c->nnd * ne);
            gl.push_back(g);
        }
        if (gl.empty()) continue;
        CUDA_TRY(cudaMemcpyAsync(d_gm, gl.data(), sizeof(GroupAsm) * gl.size(),
                                 cudaMemcpyHostToDevice, s));
        CUDA_TRY(launch_pair_window_group(d_gm, (int)gl.size(), np, d_pairs, d_counts, s));
        CUDA_TRY(exclusive_scan(d_counts, d_offsets, np, d_tmp, tmp_bytes, s));
        unsigned last[2];
        CUDA_TRY(cudaMemcpyAsync(&last[0], d_offsets + np - 1, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaMemcpyAsync(&last[1], d_counts + np - 1, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));  // also keeps d_gm alive until its launches ran
        const unsigned nitems = last[0] + last[1];
        CUDA_TRY(launch_assemble_group(d_gm, (int)gl.size(), d_pairs, d_offsets, np, nitems, s));
        CUDA_TRY(cudaStreamSynchronize(s));  // d_gm is rewritten for the next colour
        launches += 4;
    }
    CUDA_TRY(cudaMemcpyAsync(d_gm, all.data(), sizeof(GroupAsm) * n, cudaMemcpyHostToDevice, s));
    CUDA_TRY(launch_cterm_group(d_gm, n, node_total, s));
    launches += 1;
    const double ms = tm.stop_ms(s);
    for (int i = 0; i < n; i++) {
        tdbem_ctx* c = ctxs[i];
        c->levels_last = std::min(c->M, nsteps[i]);
        c->mtc_planes_valid = false;
        c->step_inv_ready[0] = c->step_inv_ready[1] = false;
        c->timings[0] = ms;
    }
    c0->launches += launches;
    return TDBEM_OK;
}

namespace {
struct ShapeKey {
    int nmesh;
    unsigned nrows, nw;
    bool operator==(const ShapeKey& o) const {
        return nmesh == o.nmesh && nrows == o.nrows && nw == o.nw;
    }
};
std::mutex g_shape_mu;
std::vector<std::pair<ShapeKey, GroupShape>> g_shapes;  // autotuned launch shapes
}  // namespace

int tdbem_march_group(tdbem_ctx* const* ctxs, int n, const int* numsteps, double* const* u_hist,
                      double* const* t_hist) {
    if (!ctxs || !numsteps || n < 1) return fail(TDBEM_ERR_ARG, "invalid group");
    int max_steps = 0;
    for (int i = 0; i < n; i++) {
        tdbem_ctx* c = ctxs[i];
        if (!c) return fail(TDBEM_ERR_ARG, "null context %d", i);
        if (c->device != ctxs[0]->device)
            return fail(TDBEM_ERR_ARG, "the group's contexts are on different devices");
        for (int j = 0; j < i; j++)
            if (ctxs[j] == c) return fail(TDBEM_ERR_ARG, "context %d appears twice", i);
        if (numsteps[i] < 1) return fail(TDBEM_ERR_ARG, "numsteps[%d] must be >= 1", i);
        if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "mesh %d: levels not assembled", i);
        if (c->level_precision != ctxs[0]->level_precision)
            return fail(TDBEM_ERR_UNSUPPORTED,
                        "a group marches FP64 levels or TDBEM_MIXED levels, not both (mesh %d)", i);
        if (c->levels_last < std::min(c->M, numsteps[i]))
            return fail(TDBEM_ERR_STATE, "mesh %d: levels hold %d steps, %d needed", i,
                        c->levels_last, std::min(c->M, numsteps[i]));
        if (!c->amp.empty() && (int)c->amp.size() < numsteps[i])
            return fail(TDBEM_ERR_ARG, "mesh %d: load history shorter than its steps", i);
        max_steps = std::max(max_steps, numsteps[i]);
    }
    const bool mixed = ctxs[0]->level_precision == TDBEM_MIXED;
    cudaStream_t s = ctxs[0]->stream;
    std::vector<GroupMarch> gm(n);
    std::vector<double*> d_amp(n, nullptr);
    struct FreeAmp {
        std::vector<double*>& v;
        ~FreeAmp() {
            for (auto& p : v) dfree(p);
        }
    } amp_guard{d_amp};
    unsigned nrows = 0, nw = 0;
    EventTimer tf;
    tf.start(s);
    // per mesh: boundary conditions, histories, inverses, load history -- on the
    // mesh's own stream from its own host thread, so the meshes overlap
    int rc = parallel_contexts(ctxs, n, [&](int i) -> int {
        tdbem_ctx* c = ctxs[i];
        const int D = c->D, ns = numsteps[i];
        int r = upload_bc(c);
        if (r != TDBEM_OK) return r;
        if (c->hist_steps != ns) {
            dfree(c->d_u);
            dfree(c->d_t);
            CUDA_TRY(dalloc(&c->d_u, (size_t)(ns + 1) * D));
            CUDA_TRY(dalloc(&c->d_t, (size_t)(ns + 1) * D));
            c->hist_steps = ns;
        }
        CUDA_TRY(cudaMemsetAsync(c->d_u, 0, sizeof(double) * (ns + 1) * D, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_t, 0, sizeof(double) * (ns + 1) * D, c->stream));
        const double a1 = c->a1, a2 = c->a2, a3 = 1 - a1 - a2;
        const double lhs_c[2][2] = {{1.0, 0.0}, {2 * a1 + a3, a1}};
        if (mixed) {
            if (!c->d_res) CUDA_TRY(dalloc(&c->d_res, D));
            r = mixed_inverses(c, ns, lhs_c);
            if (r != TDBEM_OK) return r;
        } else {
            const bool same = (lhs_c[1][0] == 1.0 && lhs_c[1][1] == 0.0);
            const int ninv = (ns >= 3 && !same) ? 2 : 1;
            for (int v = 0; v < ninv; v++) {
                r = fp64_inverse(c, v, lhs_c);
                if (r != TDBEM_OK) return r;
            }
            if (ninv == 1) {
                if (c->d_Ainv[1] && c->d_Ainv[1] != c->d_Ainv[0]) dfree(c->d_Ainv[1]);
                c->d_Ainv[1] = c->d_Ainv[0];
            }
        }
        if (!c->amp.empty()) {
            CUDA_TRY(dalloc(&d_amp[i], (size_t)ns));
            CUDA_TRY(cudaMemcpyAsync(d_amp[i], c->amp.data(), sizeof(double) * ns,
                                     cudaMemcpyHostToDevice, c->stream));
        }
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        GroupMarch& g = gm[i];
        g = GroupMarch{};
        g.D = D;
        g.M = c->M;
        g.numstep = ns;
        g.G = c->d_G;
        g.H = c->d_H;
        g.Ainv0 = c->d_Ainv[0];
        g.Ainv1 = c->d_Ainv[1];
        g.u = c->d_u;
        g.t = c->d_t;
        g.is_u = c->d_is_ubc;
        g.is_f = c->d_is_fbc;
        g.ubc = c->d_ubc_map;
        g.fbc = c->d_fbc_map;
        g.load_t = c->d_load_t;
        g.load_u = c->d_load_u;
        g.amp = d_amp[i];
        g.a1 = a1;
        g.a2 = a2;
        g.a3 = a3;
        g.c0 = lhs_c[1][0];
        g.c1 = lhs_c[1][1];
        g.Wt = c->d_Wt;
        g.Wu = c->d_Wu;
        g.rhs = c->d_rhs;
        g.Gf = c->d_Gf;
        g.Hf = c->d_Hf;
        g.ldf = c->ldf;
        g.inv32_0 = c->d_inv32[0];
        g.inv32_1 = c->d_inv32[1];
        g.Hc0 = c->d_Hc64[0];
        g.Hc1 = c->d_Hc64[1];
        g.x = c->d_x;
        g.r = c->d_res;
        g.refine = c->n_refine > 0 ? 1 : 0;
        return TDBEM_OK;
    });
    if (rc != TDBEM_OK) return rc;
    unsigned nquads = 0, nwold = 0;
    size_t nwf = 0, nwoldf = 0, nyold = 0;  // FP32 scratch (row stride ldf) and Y_old sizes
    for (int i = 0; i < n; i++) {
        const tdbem_ctx* c = ctxs[i];
        gm[i].row_begin = nrows;
        gm[i].w_begin = nw;
        gm[i].quad_begin = nquads;
        gm[i].wold_begin = nwold;
        nrows += (unsigned)c->D;
        nw += (unsigned)((c->M + 1) * c->D);
        nquads += (unsigned)((c->D + 3) / 4);
        nwold += (unsigned)((c->M + 1) * kGroupNB * c->D);
        nwf += (size_t)(c->M + 1) * c->ldf;
        nwoldf += (size_t)(c->M + 1) * kGroupNB * c->ldf;
        nyold += (size_t)kGroupNB * c->D;
    }
    float* d_wf = nullptr;    // FP32 history vectors of every mesh (mixed)
    double* d_yold = nullptr;
    struct FreeWf {
        float*& p;
        double*& q;
        ~FreeWf() {
            dfree(p);
            dfree(q);
        }
    } wf_guard{d_wf, d_yold};
    if (mixed) {
        // new-W (2 x nwf) and old-W (2 x nwoldf) planes, zeroed: the padding columns
        // ldf > D are read by the 16-byte loads and must stay zero
        const size_t tot = 2 * nwf + 2 * nwoldf;
        CUDA_TRY(dalloc(&d_wf, tot));
        CUDA_TRY(cudaMemsetAsync(d_wf, 0, sizeof(float) * tot, s));
        CUDA_TRY(dalloc(&d_yold, nyold));
        size_t ow = 0, oo = 0, oy = 0;
        for (int i = 0; i < n; i++) {
            const tdbem_ctx* c = ctxs[i];
            gm[i].Wtf = d_wf + ow;
            gm[i].Wuf = d_wf + nwf + ow;
            gm[i].Wold_t = d_wf + 2 * nwf + oo;
            gm[i].Wold_u = d_wf + 2 * nwf + nwoldf + oo;
            gm[i].Yold = d_yold + oy;
            ow += (size_t)(c->M + 1) * c->ldf;
            oo += (size_t)(c->M + 1) * kGroupNB * c->ldf;
            oy += (size_t)kGroupNB * c->D;
        }
    }
    const double factor_ms = tf.stop_ms(s);
    GroupMarch* d_gm = nullptr;
    CUDA_TRY(dalloc(&d_gm, (size_t)n));
    struct FreeGm {
        GroupMarch*& p;
        ~FreeGm() { dfree(p); }
    } gm_guard{d_gm};
    CUDA_TRY(cudaMemcpyAsync(d_gm, gm.data(), sizeof(GroupMarch) * n, cudaMemcpyHostToDevice, s));

    // launch shape: the fastest of the candidates on the first steps, remembered per
    // group size (the march is deterministic: every step is recomputed by the full run)
    const ShapeKey key{n * (mixed ? -1 : 1), nrows, nw};
    GroupShape shape{0, 0, 0};
    {
        std::lock_guard<std::mutex> lock(g_shape_mu);
        for (auto& kv : g_shapes)
            if (kv.first == key) shape = kv.second;
    }
    if (shape.lanes == 0) {
        // the probe covers one old-history pass of the time-blocked form
        const int probe_hi = std::min(max_steps, mixed ? 2 * kGroupNB + 1 : 8);
        float best = 1e30f;
        GroupShape best_shape{32, 256, 1};
        for (int lanes : {8, 16, 32})
            for (int block : {128, 256, 512})
                for (int bps : {1, 2, 4}) {
                    if (block * bps > 2048) continue;
                    const GroupShape cand{lanes, block, bps};
                    if (probe_hi <= 1) break;
                    EventTimer t;
                    t.start(s);
                    const cudaError_t e = launch_march_group(d_gm, n, nrows, nw, nquads, nwold, 1,
                                                             probe_hi, cand, mixed, s);
                    if (e == cudaErrorInvalidConfiguration || e == cudaErrorCooperativeLaunchTooLarge) {
                        cudaGetLastError();
                        t.stop_ms(s);
                        continue;
                    }
                    CUDA_TRY(e);
                    const float ms = (float)t.stop_ms(s);
                    if (ms < best) {
                        best = ms;
                        best_shape = cand;
                    }
                }
        shape = best_shape;
        std::lock_guard<std::mutex> lock(g_shape_mu);
        g_shapes.push_back({key, shape});
    }
    EventTimer tmr;
    tmr.start(s);
    CUDA_TRY(launch_march_group(d_gm, n, nrows, nw, nquads, nwold, 1, max_steps, shape, mixed, s));
    ctxs[0]->launches += 1;
    const double march_ms = tmr.stop_ms(s);
    for (int i = 0; i < n; i++) {
        tdbem_ctx* c = ctxs[i];
        const size_t bytes = sizeof(double) * (numsteps[i] + 1) * c->D;
        if (u_hist && u_hist[i])
            CUDA_TRY(cudaMemcpyAsync(u_hist[i], c->d_u, bytes, cudaMemcpyDeviceToHost, s));
        if (t_hist && t_hist[i])
            CUDA_TRY(cudaMemcpyAsync(t_hist[i], c->d_t, bytes, cudaMemcpyDeviceToHost, s));
        c->timings[1] = factor_ms;
        c->timings[2] = march_ms;
    }
    CUDA_TRY(cudaStreamSynchronize(s));
    return TDBEM_OK;
}

int tdbem_group_shape(int* lanes, int* block, int* blocks_per_sm) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    if (g_shapes.empty()) return fail(TDBEM_ERR_STATE, "no grouped march has run");
    const GroupShape& sh = g_shapes.back().second;
    if (lanes) *lanes = sh.lanes;
    if (block) *block = sh.block;
    if (blocks_per_sm) *blocks_per_sm = sh.blocks_per_sm;
    return TDBEM_OK;
}

int tdbem_set_graphs(tdbem_ctx* c, int on) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    c->use_graphs = on != 0;
    if (!c->use_graphs && c->graph.exec) {
        cudaStreamSynchronize(c->stream);
        cudaGraphExecDestroy(c->graph.exec);
        c->graph.exec = nullptr;
    }
    return TDBEM_OK;
}

int tdbem_set_batch_options(tdbem_ctx* c, int engine, int refine_sweeps) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (engine != TDBEM_ENGINE_TCGEN05 && engine != TDBEM_ENGINE_MMA_SYNC)
        return fail(TDBEM_ERR_ARG, "unknown batch engine %d", engine);
    if (refine_sweeps < 0 || refine_sweeps > 4)
        return fail(TDBEM_ERR_ARG, "refine_sweeps must be in 0..4");
    c->batch_engine = engine;
    c->batch_refine = refine_sweeps;
    return TDBEM_OK;
}

int tdbem_set_march_engine(tdbem_ctx* c, int engine) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (engine != TDBEM_ENGINE_TCGEN05 && engine != TDBEM_ENGINE_FP32)
        return fail(TDBEM_ERR_ARG, "engine must be TDBEM_ENGINE_TCGEN05 or TDBEM_ENGINE_FP32");
    c->march_engine = engine;
    return TDBEM_OK;
}

int tdbem_set_march_options(tdbem_ctx* c, int block_steps, int refine_sweeps) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (block_steps != 0 && block_steps != 1 && block_steps != 4 && block_steps != 6 &&
        block_steps != 8 && block_steps != 12 && block_steps != 16 && block_steps != 24 &&
        block_steps != 32)
        return fail(TDBEM_ERR_ARG, "block_steps must be 0 (auto), 1, 4, 6, 8, 12, 16, 24 or 32");
    if (refine_sweeps < 0 || refine_sweeps > 4)
        return fail(TDBEM_ERR_ARG, "refine_sweeps must be in 0..4");
    c->nb = block_steps;  // the march resizes its scratch when the block changes
    c->n_refine = refine_sweeps;
    return TDBEM_OK;
}

int tdbem_history_device(const tdbem_ctx* c, const double** u_hist, const double** t_hist) {
    if (!c || !u_hist || !t_hist) return fail(TDBEM_ERR_ARG, "null argument");
    if (c->hist_steps < 0) return fail(TDBEM_ERR_STATE, "no march has run");
    *u_hist = c->d_u;
    *t_hist = c->d_t;
    return TDBEM_OK;
}

int tdbem_set_profiling(tdbem_ctx* c, int on) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (c->stream) cudaStreamSynchronize(c->stream);
    prof_flush(c);
    c->prof = on != 0;
    for (int k = 0; k < TDBEM_K_COUNT; k++) {
        c->prof_launches[k] = 0;
        c->prof_ms[k] = c->prof_bytes[k] = c->prof_flops[k] = 0;
    }
    (void)0;
    return TDBEM_OK;
}

int tdbem_kernel_stats(const tdbem_ctx* c, int k, long long* launches, double* ms,
                       double* bytes, double* flops) {
    if (!c || k < 0 || k >= TDBEM_K_COUNT) return fail(TDBEM_ERR_ARG, "bad kernel class");
    if (launches) *launches = c->prof_launches[k];
    if (ms) *ms = c->prof_ms[k];
    if (bytes) *bytes = c->prof_bytes[k];
    if (flops) *flops = c->prof_flops[k];
    return TDBEM_OK;
}

int tdbem_launch_count(const tdbem_ctx* c, long long* n) {
    if (!c || !n) return fail(TDBEM_ERR_ARG, "null argument");
    *n = c->launches;
    return TDBEM_OK;
}

int tdbem_footprint(const tdbem_mesh* mesh, const tdbem_material* mat, double dt, int nq,
                    int numstep, int precision, size_t* bytes) {
    if (!mesh || !mat || !bytes || !mesh->coords || !mesh->ien)
        return fail(TDBEM_ERR_ARG, "null argument");
    if (mesh->nnd < 2 || mesh->nel < 1 || !(dt > 0) || numstep < 1 || !(mat->rho > 0) ||
        !(mat->E > 0) || !(mat->nu > -1 && mat->nu < 0.5) ||
        (mesh->etype != 1 && mesh->etype != 2))
        return fail(TDBEM_ERR_ARG, "invalid mesh, material, time step or step count");
    const int ennd = mesh->etype == 2 ? 8 : 4;
    if (precision != TDBEM_FP64 && precision != TDBEM_MIXED)
        return fail(TDBEM_ERR_ARG, "precision must be TDBEM_FP64 or TDBEM_MIXED");
    std::vector<double> x(mesh->coords, mesh->coords + 3 * (size_t)mesh->nnd);
    std::vector<int> ien(mesh->ien, mesh->ien + ennd * (size_t)mesh->nel);
    for (int v : ien)
        if (v < 0 || v >= mesh->nnd) return fail(TDBEM_ERR_ARG, "element node out of range");
    const int M = compute_max_step(x, mesh->nnd, mat->E, mat->nu, mat->rho, dt);
    std::vector<int> order, start;
    color_elements(ien, mesh->nel, ennd, mesh->nnd, order, start);
    size_t max_color = 0;
    for (size_t k = 0; k + 1 < start.size(); k++)
        max_color = std::max<size_t>(max_color, (size_t)(start[k + 1] - start[k]));
    const size_t D = 3 * (size_t)mesh->nnd, DD = D * D, L = (size_t)M + 1;
    const size_t nel = mesh->nel, q2 = (size_t)nq * nq;
    size_t pair_cap = std::min<size_t>((size_t)mesh->nnd * max_color, (size_t)1 << 26);
    pair_cap = std::max(pair_cap, max_color);
    // tdbem_ctx_create: mesh, Gauss geometry (FP64 + FP32 for 4-node elements, FP64
    // only, 16 per point, for 8-node ones), C term, colours, pair scratch
    size_t b = 24 * (size_t)mesh->nnd + 4 * (ennd + 1) * nel + q2 * nel * 16 * 8 +
               72 * (size_t)mesh->nnd +
               pair_cap * (sizeof(PairInfo) + 8) + pair_cap / 8 + ((size_t)1 << 16);  // + scan
    // marching state common to both forms: maps, W vectors, partials, histories
    b += 8 * D * 8 + 3 * L * D * 8 + 2 * ((size_t)numstep + 1) * D * 8 + 4 * (D + 64);
    if (precision == TDBEM_FP64) {
        b += 2 * L * DD * 8;                    // levels
        b += 2 * DD * 8 + inverse_scratch_elems((int)D) * 8;  // inverses
    } else {
        const size_t ld = mixed_ld((int)D), ldw = mixed_ldw((int)D), nb = 32;
        b += 2 * L * D * ld * 4 + 4 * DD * 8;   // FP32 levels, FP64 levels 0 and 1
        b += 2 * DD * 8 + 2 * DD * 4 + inverse_scratch_elems((int)D) * 4;  // LHS, inverses
        b += 2 * L * (nb + 1) * ldw * 4 + L * nb * D * 8 + (nb + 2) * D * 8;  // time blocks
        // tcgen05 march: merged planes, history planes, known part and its coefficients
        b += tc_plane_bytes((int)D, (int)L, 1) + tc_w_bytes((int)D, 32, (int)L, 1) +
             3 * L * D * 8 + (numstep + 1) * (L * 3 + D) * 8 + 3 * D * 4;
    }
    *bytes = b;
    return TDBEM_OK;
}

int tdbem_last_timings(const tdbem_ctx* c, double* ms3) {
    if (!c || !ms3) return fail(TDBEM_ERR_ARG, "null argument");
    for (int i = 0; i < 3; i++) ms3[i] = c->timings[i];
    return TDBEM_OK;
}

}  // extern "C"
