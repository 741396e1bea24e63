// C ABI of tdbem-gb300, many meshes at once: grouped assembly and the persistent
// grouped march with its autotuned launch shape.
#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

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

namespace tdbem {
namespace capi {

int group_prepare(tdbem_ctx* c, int ns, bool mixed, GroupMarch& g) {
    const int D = c->D;
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
        // FP32 history vectors of the time blocks: new W (2 x (M+1) x ldf), old W
        // (2 x (M+1) x kGroupNB x ldf), zeroed once (the padding columns ldf > D are
        // read by 16-byte loads and never written), and Y_old (kGroupNB x D)
        const size_t nwf = (size_t)(c->M + 1) * c->ldf, nwold = nwf * kGroupNB;
        if (!c->d_group_wf) {
            CUDA_TRY(dalloc(&c->d_group_wf, 2 * nwf + 2 * nwold));
            CUDA_TRY(cudaMemsetAsync(c->d_group_wf, 0, sizeof(float) * (2 * nwf + 2 * nwold),
                                     c->stream));
            CUDA_TRY(dalloc(&c->d_group_yold, (size_t)kGroupNB * D));
        }
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
    dfree(c->d_group_amp);
    if (!c->amp.empty()) {
        CUDA_TRY(dalloc(&c->d_group_amp, (size_t)ns));
        CUDA_TRY(cudaMemcpyAsync(c->d_group_amp, c->amp.data(), sizeof(double) * ns,
                                 cudaMemcpyHostToDevice, c->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
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
    g.amp = c->d_group_amp;
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
    g.step2_sweeps = mixed ? c->step2_sweeps : 0;
    if (mixed) {
        const size_t nwf = (size_t)(c->M + 1) * c->ldf, nwold = nwf * kGroupNB;
        g.Wtf = c->d_group_wf;
        g.Wuf = c->d_group_wf + nwf;
        g.Wold_t = c->d_group_wf + 2 * nwf;
        g.Wold_u = c->d_group_wf + 2 * nwf + nwold;
        g.Yold = c->d_group_yold;
    }
    return TDBEM_OK;
}

void group_layout(GroupMarch* gm, int n, unsigned* nrows, unsigned* nw, unsigned* nquads,
                  unsigned* nwold) {
    unsigned r = 0, w = 0, q = 0, wo = 0;
    for (int i = 0; i < n; i++) {
        gm[i].row_begin = r;
        gm[i].w_begin = w;
        gm[i].quad_begin = q;
        gm[i].wold_begin = wo;
        r += (unsigned)gm[i].D;
        w += (unsigned)((gm[i].M + 1) * gm[i].D);
        q += (unsigned)((gm[i].D + 3) / 4);
        wo += (unsigned)((gm[i].M + 1) * kGroupNB * gm[i].D);
    }
    *nrows = r;
    *nw = w;
    *nquads = q;
    *nwold = wo;
}

}  // namespace capi
}  // namespace tdbem

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
            mem_free(e);
        }
    } guard{d_pairs, d_counts, d_offsets, d_gm, d_tmp};
    CUDA_TRY(dalloc(&d_pairs, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_counts, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_offsets, std::max<size_t>(pair_max, 1)));
    CUDA_TRY(dalloc(&d_gm, (size_t)n));
    CUDA_TRY(mem_alloc(&d_tmp, tmp_bytes));
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
    EventTimer tf;
    tf.start(s);
    // per mesh: boundary conditions, histories, inverses, load history -- on the
    // mesh's own stream from its own host thread, so the meshes overlap
    int rc = parallel_contexts(ctxs, n, [&](int i) -> int {
        return group_prepare(ctxs[i], numsteps[i], mixed, gm[i]);
    });
    if (rc != TDBEM_OK) return rc;
    unsigned nrows = 0, nw = 0, nquads = 0, nwold = 0;
    group_layout(gm.data(), n, &nrows, &nw, &nquads, &nwold);
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

}  // extern "C"
