// C ABI of tdbem-gb300 (include/tdbem.h), context and levels: context lifetime,
// element colouring, the single-step driver, the level assembly, boundary
// conditions and weights, the stepwise level placement, profiling counters.
// The march engines are in capi_march.cu, the batched march in capi_batch.cu,
// checkpoints in capi_ckpt.cu and the many-mesh calls in capi_group.cu.
#include <system_error>

#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace tdbem {
namespace capi {

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
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

// SolverT::ComputeMaxStep (SolverT.cpp:211-250), same arithmetic.  The largest node
// distance is the square root of the largest squared distance (a correctly rounded
// square root is monotonic: the same value bit for bit), and the pairs are split over
// a few host threads (the maximum does not depend on the order): at 1538 nodes,
// 1.2 M pairs.
int compute_max_step(const std::vector<double>& x, int nnd, double E, double nu, double rho,
                     double dt) {
    const double Mu = E / (2.0 * (1.0 + nu));
    const double Cs = std::sqrt(Mu / rho);
    std::vector<double> px(nnd), py(nnd), pz(nnd);
    for (int i = 0; i < nnd; i++) {
        px[i] = x[i * 3];
        py[i] = x[i * 3 + 1];
        pz[i] = x[i * 3 + 2];
    }
    // rows [lo, hi) of the pair triangle (row i: the pairs (i, j > i))
    auto rows = [&](int lo, int hi) {
        double m2 = 0;
        for (int i = lo; i < hi; i++) {
            const double xi = px[i], yi = py[i], zi = pz[i];
            double mi = 0;
            for (int j = i + 1; j < nnd; j++) {
                const double v0 = xi - px[j], v1 = yi - py[j], v2 = zi - pz[j];
                double t = 0;
                t += v0 * v0;
                t += v1 * v1;
                t += v2 * v2;
                mi = t > mi ? t : mi;
            }
            m2 = mi > m2 ? mi : m2;
        }
        return m2;
    };
    const long long pairs = (long long)nnd * (nnd - 1) / 2;
    const int nt = (int)std::max(1LL, std::min<long long>(
                                          {8LL, (long long)std::thread::hardware_concurrency(),
                                           pairs / 200000}));
    std::vector<double> part(nt, 0.0);
    std::vector<std::thread> th;
    int lo = 0;
    long long done = 0;
    for (int t = 0; t < nt; t++) {
        // equal pair counts per thread
        int hi = lo;
        const long long want = pairs * (t + 1) / nt;
        while (hi < nnd && done < want) done += nnd - 1 - hi++;
        if (t == nt - 1) hi = nnd;
        bool started = false;
        if (t < nt - 1) {
            try {
                th.emplace_back([&, t, lo, hi] { part[t] = rows(lo, hi); });
                started = true;
            } catch (const std::system_error&) {  // no thread to be had: this share here
            }
        }
        if (!started) part[t] = rows(lo, hi);
        lo = hi;
    }
    for (auto& t : th) t.join();
    double m2 = 0;
    for (double v : part) m2 = v > m2 ? v : m2;
    const double max_dis = std::sqrt(m2);
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
    mem_free(c->d_mtc_planes);
    c->d_mtc_planes = nullptr;
    dfree(c->d_mtc_occ);
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
    mem_free(c->d_tc_W);
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
    mem_free(c->d_mtc_W);
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
    dfree(c->d_group_amp);
    dfree(c->d_group_wf);
    dfree(c->d_group_yold);
    free_batch(c);
}

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
                                    c->d_counts, c->stream, c->d_ebox));
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
                                       c->stream, c->d_duffy));
        if (nitems) c->launches += (mode == ASM_STEP ? 2 : 1);
        const double pts = (double)c->nq * c->nq;
        const double items = (double)nitems * (mode == ASM_STEP ? 2.0 : 1.0);
        prof_end(c, pe, items * 4 * 45 * (out.G0f ? 4.0 : 8.0) * 2,
                 items * pts * kFlopsPerItemPoint * (mode == ASM_STEP ? 0.5 : 1.0));
    }
    return TDBEM_OK;
}

}  // namespace capi
}  // namespace tdbem

void tdbem::note_error(const char* msg) { g_last_error = msg; }

tdbem::Phys tdbem::make_phys(double E, double nu, double rho, double dt) {
    // GreenFunctionT::WaveSpeed (GreenFunctionT.cpp:76-84)
    const double mu = E / (2 * (1 + nu));
    const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    Phys ph;
    ph.dt = dt;
    ph.inv_dt = 1.0 / dt;
    ph.cp = std::sqrt((lam + 2 * mu) / rho);
    ph.cs = std::sqrt(mu / rho);
    ph.inv_cp = 1.0 / ph.cp;
    ph.inv_cs = 1.0 / ph.cs;
    ph.inv_cp2 = 1.0 / (ph.cp * ph.cp);
    ph.inv_cs2 = 1.0 / (ph.cs * ph.cs);
    ph.cs2 = ph.cs * ph.cs;
    ph.ratio2 = (ph.cs / ph.cp) * (ph.cs / ph.cp);
    ph.ratio3 = ph.ratio2 * (ph.cs / ph.cp);
    ph.inv_4pi_rho = 1.0 / (4 * M_PI * rho);
    ph.inv_4pi = 1.0 / (4 * M_PI);
    ph.nu = nu;
    return ph;
}

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
    c->ph = make_phys(c->E, c->nu, c->rho, dt);
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
    CTX_TRY(dalloc(&c->d_coords, c->h_coords.size()));
    CTX_TRY(dalloc(&c->d_ien, c->h_ien.size()));
    CTX_TRY(dalloc(&c->d_gx, nq));
    CTX_TRY(dalloc(&c->d_gw, nq));
    CTX_TRY(dalloc(&c->d_geom, (size_t)c->nel * nq * nq * (ennd == 8 ? 16 : 12)));
    CTX_TRY(dalloc(&c->d_cterm, (size_t)c->nnd * 9));
    if (ennd == 4) CTX_TRY(dalloc(&c->d_geomf, (size_t)c->nel * nq * nq * 12));
    CTX_TRY(dalloc(&c->d_color_elems, order.size()));
    CTX_TRY(dalloc(&c->d_color_start, c->color_start.size()));
    CTX_TRY(dalloc(&c->d_far_items, 3));
    CTX_TRY(dalloc(&c->d_ebox, c->nel));
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
    CTX_TRY(launch_element_box(c->d_coords, c->d_ien, ennd, c->nel, c->d_ebox, c->stream));
    // 4-node meshes: the singular pairs' Duffy points, once (skipped above 512 MB: the
    // kernels then map each point themselves)
    if (ennd == 4 && duffy_table_elems(c->nel, nq) * sizeof(double) <= (size_t(512) << 20)) {
        CTX_TRY(dalloc(&c->d_duffy, duffy_table_elems(c->nel, nq)));
        CTX_TRY(launch_duffy_table(c->d_coords, c->d_ien, c->nel, nq, c->d_gx, c->d_gw,
                                   c->d_duffy, c->stream));
    }
    c->pair_cap = std::min<size_t>((size_t)c->nnd * max_color, (size_t)1 << 26);
    c->pair_cap = std::max<size_t>(c->pair_cap, (size_t)max_color);
    CTX_TRY(dalloc(&c->d_pairs, c->pair_cap));
    CTX_TRY(dalloc(&c->d_counts, c->pair_cap));
    CTX_TRY(dalloc(&c->d_offsets, c->pair_cap));
    c->scan_tmp_bytes = scan_temp_bytes((unsigned)c->pair_cap);
    CTX_TRY(mem_alloc(&c->d_scan_tmp, std::max<size_t>(c->scan_tmp_bytes, 16)));
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
    dfree(c->d_ebox);
    dfree(c->d_duffy);
    dfree(c->d_color_elems);
    dfree(c->d_color_start);
    dfree(c->d_far_items);
    dfree(c->d_far_pairs);
    dfree(c->d_pairs);
    dfree(c->d_counts);
    dfree(c->d_offsets);
    mem_free(c->d_scan_tmp);
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
                         c->d_geom, c->ph, c->d_cterm, c->stream, false, nullptr, nullptr,
                         c->d_ebox, c->d_duffy);
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
    mem_free(buf);
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
                              c->d_geom, c->ph, c->d_cterm, c->stream, false, nullptr, nullptr,
                              c->d_ebox, c->d_duffy));
        CUDA_TRY(launch_cterm_apply(c->d_cterm, 0, c->nnd, c->dt, c->if_ext, ASM_LEVELS, out,
                                    c->stream));
        prof_end(c, pc, 0, 0);
        c->launches += 2;
    } else {
        // FP32 store for all levels: near pairs with the FP64 quadrature, far pairs with
        // the FP32 tau form; levels 0 and 1 again in FP64 for the LHS of the solve.
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
            CUDA_TRY(cudaMemsetAsync(c->d_far_items, 0, 3 * sizeof(unsigned long long), c->stream));
        if (split) {
            const int pw = prof_begin(c, TDBEM_K_AUX);
            CUDA_TRY(launch_pair_window(c->d_coords, c->d_ien, 4, c->d_color_elems, c->nel, 0,
                                        c->nnd, c->ph, ASM_LEVELS, last, 1, 0, SEL_FAR,
                                        c->d_far_pairs, nullptr, c->stream, c->d_ebox));
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
                              c->d_geomf, c->d_coordf, c->d_ebox, c->d_duffy));
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
        // The FP32 store's zero fill (10 GB on the 4614-DOF sphere, ~2 ms) after the
        // fork: nothing before it writes the store, and the inverses bound the
        // assembly's time.
        const size_t total = (size_t)(c->M + 1) * D * ldf;
        CUDA_TRY(cudaMemsetAsync(c->d_Gf, 0, 4 * total, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->d_Hf, 0, 4 * total, c->stream));
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
                                        c->d_far_pairs, nullptr, c->stream, c->d_ebox));
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
                unsigned long long n[3] = {0, 0, 0};
                CUDA_TRY(cudaMemcpyAsync(n, c->d_far_items, sizeof(n), cudaMemcpyDeviceToHost,
                                         c->stream));
                CUDA_TRY(cudaStreamSynchronize(c->stream));
                c->prof_pending[pe].bytes = (double)(n[0] + n[2]) * 4 * 45 * 4.0 * 2;
                // algorithmic flops: every far (node, element, level) item's Gauss points at
                // the per-point count, settled levels included (a settled job produces
                // them from one quasi-static pass per pair: kFlopsSettledPoint per point
                // and kFlopsSettledLevel per level executed)
                c->prof_pending[pe].flops =
                    (double)(n[0] + n[2]) * c->nq * c->nq * kFlopsPerItemPointF32;
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
    // element boxes; the Duffy table of a 4-node mesh (when made: up to 512 MB)
    b += sizeof(ElemBox) * nel;
    if (ennd == 4 && duffy_table_elems((int)nel, nq) * sizeof(double) <= (size_t(512) << 20))
        b += duffy_table_elems((int)nel, nq) * sizeof(double);
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
        b += tc_plane_bytes((int)D, (int)L + kStepMats, 1) + tc_w_bytes((int)D, 32, (int)L, 1) +
             tc_occ_bytes((int)D, (int)L + kStepMats) +
             3 * L * D * 8 + (numstep + 1) * (L * 3 + D) * 8 + 3 * D * 4;
        // grouped march (the server's batched steps): FP32 time-block vectors
        b += (2 + 2 * (size_t)kGroupNB) * L * ld * 4 + (size_t)kGroupNB * D * 8;
    }
    b += (size_t)numstep * 8;  // the load history on the device
    *bytes = b;
    return TDBEM_OK;
}

int tdbem_last_timings(const tdbem_ctx* c, double* ms3) {
    if (!c || !ms3) return fail(TDBEM_ERR_ARG, "null argument");
    for (int i = 0; i < 3; i++) ms3[i] = c->timings[i];
    return TDBEM_OK;
}

}  // extern "C"
