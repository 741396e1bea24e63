// C ABI of tdbem-gb300, marching: the FP64 and mixed march engines (inverses of
// the column-exchanged LHS, merged level planes, graph-replayed step loops),
// tdbem_march, its stepwise form and the march options.
#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

namespace tdbem {
namespace capi {

int tc_status(const int err[2], const char* what) {
    if (err[0] == 0 && err[1] == 0) return TDBEM_OK;
    static const char* const wait_name[] = {"",
                                            "producer waiting for a free stage",
                                            "MMA issuer waiting for a free accumulator",
                                            "MMA issuer waiting for a loaded stage",
                                            "epilogue waiting for a finished level",
                                            "producer draining its copies",
                                            "MMA issuer draining its MMAs"};
    const int code = err[0];
    return fail(TDBEM_ERR_CUDA,
                "tcgen05 convolution (%s): a pipeline wait timed out (code %d: %s); CTAs "
                "still holding TMEM: %d",
                what, code, (code >= 1 && code <= 6) ? wait_name[code] : "none", err[1]);
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
    // The inverses are chains of short dependent launches that run beside the
    // assembly's long quadrature launches: their streams take the device's highest
    // priority, so each of their blocks is scheduled as soon as an SM has room
    // instead of queueing behind the quadrature's pending blocks.
    int prio_least = 0, prio_greatest = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    for (cudaStream_t* st : {&c->stream2, &c->stream3})
        if (!*st)
            CUDA_TRY(cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, prio_greatest));
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
        r.e[v] = launch_build_lhs(c->d_G01, c->d_H01, nullptr, nullptr, DD, D, lhs_c[v][0],
                                  lhs_c[v][1], c->d_is_ubc, c->d_Hc64[v], st);
        if (r.e[v] == cudaSuccess)
            r.e[v] = invert_f32(c->d_Hc64[v], c->d_inv32[v], D, perm, status, scratch,
                                &r.launches[v], &r.singular[v], st, &r.report[v]);
        r.launches[v] += 1;  // invert_f32 synchronises its stream before returning
    };
    if (ninv == 2) {
        // The step-2 LHS serves one solve: it is solved by Richardson sweeps
        // x <- x + X (b - A2 x) with the later steps' inverse X and the FP64 step-2 LHS
        // A2 when they converge on a probe problem (their contraction is ~0.35 on the
        // sphere, ~0.6 on a bar with a fixed end), which spares its own inverse; it
        // gets its own inverse otherwise.
        invert(1, s0, c->d_perm, c->d_status, c->d_inv_scratch32);
        if (r.e[1] != cudaSuccess || r.singular[1]) return;
        r.e[0] = launch_build_lhs(c->d_G01, c->d_H01, nullptr, nullptr, DD, D, lhs_c[0][0],
                                  lhs_c[0][1], c->d_is_ubc, c->d_Hc64[0], s0);
        int k = 0;
        if (r.e[0] == cudaSuccess)
            r.e[0] = richardson_probe(c->d_Hc64[0], c->d_inv32[1], D,
                                      reinterpret_cast<double*>(c->d_inv_scratch32),
                                      kStep2MaxSweeps, kStep2Tol, &k, &r.launches[0], s0);
        r.launches[0] += 1;
        if (r.e[0] != cudaSuccess) return;
        if (k > 0) {
            r.step2_sweeps = k + kStep2Margin;
            r.report[0] = r.report[1];
        } else {
            invert(0, s0, c->d_perm, c->d_status, c->d_inv_scratch32);
        }
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
    // the step-2 solve by Richardson sweeps: its inverse slot is the later LHS's inverse
    if (ninv == 2 && r.step2_sweeps > 0 && c->d_inv32[0] != c->d_inv32[1]) {
        dfree(c->d_inv32[0]);
        c->d_inv32[0] = c->d_inv32[1];
    }
    c->step2_sweeps = ninv == 2 ? r.step2_sweeps : 0;
    for (int v = 0; v < 2; v++) c->inv_report[v] = r.report[v < ninv ? v : 0];
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
        CUDA_TRY(mem_alloc(&c->d_mtc_planes, tc_plane_bytes(D, mtc_slabs(M), 1)));
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
    CUDA_TRY(launch_merge_levels(c->d_Gf, c->d_Hf, c->ldf, D, M + 1, mtc_slabs(M),
                                 c->d_is_ubc, c->d_mtc_bc, c->d_mtc_bc + D, c->d_mtc_bc + 2 * D,
                                 c->d_mtc_planes, c->d_mtc_known, s));
    // which 128 x 64 tiles of the levels are all zero (the convolution skips them)
    if (!c->d_mtc_occ) CUDA_TRY(dalloc(&c->d_mtc_occ, tc_occ_bytes(D, mtc_slabs(M))));
    CUDA_TRY(launch_tile_occupancy(c->d_mtc_planes, D, 0, M + 1, c->d_mtc_occ, s));
    prof_end(c, pe, (M + 1) * (double)D * (2.0 * c->ldf + tc_ldb(D)) * 4 +
                        (M + 1) * (double)D * tc_ldb(D) * 2,
             0);
    c->launches += 2;
    c->mtc_planes_valid = true;
    c->mtc_steps_valid = false;  // the step-distance matrices follow the levels
    return TDBEM_OK;
}

int count_live_tiles(tdbem_ctx* c) {
    const int D = c->D, slabs = mtc_slabs(c->M);
    const size_t n = tc_occ_bytes(D, slabs);
    std::vector<unsigned char> occ(n);
    CUDA_TRY(cudaMemcpyAsync(occ.data(), c->d_mtc_occ, n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    const size_t per_slab = n / slabs;
    c->h_occ_live.assign(slabs, 0);
    for (int sl = 0; sl < slabs; sl++)
        for (size_t i = 0; i < per_slab; i++) c->h_occ_live[sl] += occ[sl * per_slab + i] != 0;
    return TDBEM_OK;
}

double conv_plane_bytes(const tdbem_ctx* c, int lev0, int nlev) {
    const double tile = 128.0 * 64 * 2 * 2;  // hi + lo BF16
    if ((int)c->h_occ_live.size() < lev0 + nlev)  // not counted: every tile
        return nlev * (double)c->D * tc_ldb(c->D) * 4;
    double live = 0;
    for (int sl = lev0; sl < lev0 + nlev; sl++) live += (double)c->h_occ_live[sl];
    return live * tile;
}

// The planes' step-distance matrices B_1 .. B_kStepMats for the weights (a1, a2):
// after every merge and when the weights change.
int ensure_step_mats(tdbem_ctx* c, double a1, double a2) {
    if (c->mtc_steps_valid && c->mtc_step_key[0] == a1 && c->mtc_step_key[1] == a2)
        return TDBEM_OK;
    const int pe = prof_begin(c, TDBEM_K_AUX);
    CUDA_TRY(launch_step_mats(c->d_Gf, c->d_Hf, c->ldf, c->D, c->M, mtc_slabs(c->M), c->d_is_ubc,
                              a1, a2, 1 - a1 - a2, c->d_mtc_planes, c->stream));
    CUDA_TRY(launch_tile_occupancy(c->d_mtc_planes, c->D, c->M + 1, mtc_slabs(c->M), c->d_mtc_occ,
                                   c->stream));
    prof_end(c, pe,
             std::min(c->M + 1, kStepMats + 2) * (double)c->D * 2.0 * c->ldf * 4 +
                 kStepMats * (double)c->D * tc_ldb(c->D) * 6,
             0);
    c->launches += 2;
    c->mtc_step_key[0] = a1;
    c->mtc_step_key[1] = a2;
    c->mtc_steps_valid = true;
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
        int rm = ensure_merged_levels(c);
        if (rm == TDBEM_OK) rm = ensure_step_mats(c, a1, a2);
        if (rm == TDBEM_OK && c->prof) rm = count_live_tiles(c);
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
            mem_free(c->d_mtc_W);
            c->d_mtc_W = nullptr;
            c->mtc_W_bytes = 0;
            c->mtc_maps_for[0] = c->mtc_maps_for[1] = nullptr;
            CUDA_TRY(mem_alloc(&c->d_mtc_W, wb));
            c->mtc_W_bytes = wb;
        }
        if (c->mtc_maps_for[0] != c->d_mtc_planes || c->mtc_maps_for[1] != c->d_mtc_W ||
            c->mtc_nb != nb) {
            if (!make_tc_maps(c->d_mtc_planes, D, mtc_slabs(M), c->d_mtc_W, nb, Lw, &c->mtc_maps,
                              1))
                return fail(TDBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed for the march planes");
            c->mtc_maps_for[0] = c->d_mtc_planes;
            c->mtc_maps_for[1] = c->d_mtc_W;
            c->mtc_nb = nb;
        }
        if (!c->d_tc_err) CUDA_TRY(dalloc(&c->d_tc_err, 2));
        CUDA_TRY(cudaMemsetAsync(c->d_tc_err, 0, 2 * sizeof(int), s));
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
    // set when the reduction that finished the right-hand side of the step solved next
    // also wrote its FP32 copy (the solve's first product reads it)
    bool v32_ready = false;
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
                CUDA_TRY(launch_conv_tc(c->mtc_maps, D, mtc_slabs(M), Lw, nlev, nbe, c->d_pmix,
                                        splits, c->d_tc_err, s, 1, c->tc_wait_ns, 0,
                                        c->d_mtc_occ));
                const double pb = conv_plane_bytes(c, 0, nlev);
                prof_end(c, pe, pb + nlev * (double)tc_cases_pad(nb) * tc_ldb(D) * 4,
                         pb / 4 * 2.0 * nbe);
                // column 0 (step S, solved next) also in FP32 for its solve
                CUDA_TRY(launch_reduce_cols_n(c->d_pmix, splits, nbe, nbe, D, yk, Y, s,
                                              reinterpret_cast<float*>(c->d_dx)));
                v32_ready = true;
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
        const int nm = e - a - 1;  // step-distance matrices B_1 .. B_(e-a-1)
        if (tc && nm <= std::min(kStepMats, Lw)) {
            CUDA_TRY(launch_build_w_steps(c->d_u, c->d_t, c->d_is_ubc, D, a, b, ncol, nb, nm, Lw,
                                          c->d_mtc_W, s));
            const int splits = tc_conv_splits(nm, D, ncol, (M + 1) * nb / ncol, 1);
            const int pe = prof_begin(c, TDBEM_K_CONV);
            CUDA_TRY(launch_conv_tc(c->mtc_maps, D, mtc_slabs(M), Lw, nm, ncol, c->d_pmix, splits,
                                    c->d_tc_err, s, 1, c->tc_wait_ns, M + 1, c->d_mtc_occ));
            const double pb = conv_plane_bytes(c, M + 1, nm);
            prof_end(c, pe, pb + nm * (double)tc_cases_pad(nb) * tc_ldb(D) * 4,
                     pb / 4 * 2.0 * ncol);
            // column 0 (step b, solved next) also in FP32 for its solve
            CUDA_TRY(launch_reduce_cols_n(c->d_pmix, splits, ncol, ncol, D, y, y, s,
                                          reinterpret_cast<float*>(c->d_dx)));
            v32_ready = true;
            c->launches += 3;
            return TDBEM_OK;
        }
        if (tc) {
            CUDA_TRY(launch_build_w_merged(c->d_u, c->d_t, c->d_is_ubc, D, b, ncol, nb, a, b,
                                           nlev, Lw, a1, a2, a3, c->d_mtc_W, s));
            const int splits = tc_conv_splits(nlev, D, ncol, (M + 1) * nb / ncol, 1);
            const int pe = prof_begin(c, TDBEM_K_CONV);
            CUDA_TRY(launch_conv_tc(c->mtc_maps, D, mtc_slabs(M), Lw, nlev, ncol, c->d_pmix,
                                    splits, c->d_tc_err, s, 1, c->tc_wait_ns, 0, c->d_mtc_occ));
            const double pb = conv_plane_bytes(c, 0, nlev);
            prof_end(c, pe, pb + nlev * (double)tc_cases_pad(nb) * tc_ldb(D) * 4,
                     pb / 4 * 2.0 * ncol);
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
        const int sweeps = (st == 1 && c->step2_sweeps > 0) ? std::max(c->step2_sweeps, c->n_refine)
                                                            : c->n_refine;
        // the step's state update rides on its last product
        StateUpdate upd;
        upd.is_u = c->d_is_ubc;
        upd.ubc = c->d_ubc_map;
        upd.is_f = c->d_is_fbc;
        upd.fbc = c->d_fbc_map;
        upd.amp = amp;
        upd.u_hist = c->d_u;
        upd.t_hist = c->d_t;
        upd.s = st;
        CUDA_TRY(launch_solve_mixed(c->d_inv32[v], c->d_Hc64[v], D, c->d_Yold + (size_t)(st - S) * D,
                                    c->d_x, c->d_res, reinterpret_cast<float*>(c->d_dx),
                                    sweeps, s, v32_ready, upd));
        prof_end(c, pe, 4.0 * (double)DD * (1 + 2 * sweeps), 2.0 * (double)DD * (1 + 2 * sweeps));
        c->launches += (v32_ready ? 1 : 2) + 2LL * sweeps;  // cast, gemv(s), residual(s)
        v32_ready = false;
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
        int err[2] = {0, 0};
        CUDA_TRY(cudaMemcpyAsync(err, c->d_tc_err, sizeof(err), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        const int rc = tc_status(err, "march");
        if (rc != TDBEM_OK) return rc;
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

}  // namespace capi
}  // namespace tdbem

extern "C" {

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

int tdbem_set_pipeline_wait(tdbem_ctx* c, double seconds) {
    if (!c) return fail(TDBEM_ERR_ARG, "null context");
    if (!(seconds >= 0) || seconds > 60) return fail(TDBEM_ERR_ARG, "wait limit %g s", seconds);
    const unsigned long long ns = (unsigned long long)(seconds * 1e9);
    c->tc_wait_ns = seconds == 0 ? kTcWaitNsDefault : std::max(1ull, ns);
    return TDBEM_OK;
}

int tdbem_inverse_report(const tdbem_ctx* c, double probe[2], int full_search[2],
                         int* step2_sweeps) {
    if (!c || !probe || !full_search) return fail(TDBEM_ERR_ARG, "null argument");
    if (!c->inv_valid) return fail(TDBEM_ERR_STATE, "no FP32 inverse made yet");
    for (int v = 0; v < 2; v++) {
        probe[v] = c->inv_report[v].probe_rel;
        full_search[v] = c->inv_report[v].full_search;
    }
    if (step2_sweeps) *step2_sweeps = c->step2_sweeps;
    return TDBEM_OK;
}

int tdbem_invert(int n, const double* A, int precision, double* X, double* probe,
                 int* full_search) {
    if (n < 1 || !A || !X) return fail(TDBEM_ERR_ARG, "invalid matrix");
    if (precision != TDBEM_FP64 && precision != TDBEM_MIXED)
        return fail(TDBEM_ERR_ARG, "unknown precision %d", precision);
    const size_t nn = (size_t)n * n;
    cudaStream_t s = cudaStreamPerThread;
    double* dA = nullptr;
    double* dA64 = nullptr;
    float* dX = nullptr;
    int* perm = nullptr;
    int* status = nullptr;
    void* scratch = nullptr;
    auto release = [&] {
        dfree(dA);
        dfree(dA64);
        dfree(dX);
        dfree(perm);
        dfree(status);
        mem_free(scratch);
    };
    const size_t scratch_bytes = inverse_scratch_elems(n) * sizeof(double);
    cudaError_t e = dalloc(&dA, nn);
    if (e == cudaSuccess) e = dalloc(&perm, (size_t)n + 2 * kMaxPivotBlocks);
    if (e == cudaSuccess) e = dalloc(&status, 1);
    if (e == cudaSuccess) e = mem_alloc(&scratch, scratch_bytes);
    if (e == cudaSuccess && precision == TDBEM_MIXED) e = dalloc(&dX, nn);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dA, A, sizeof(double) * nn, cudaMemcpyHostToDevice, s);
    long long nl = 0;
    bool singular = false;
    InverseReport rep;
    if (e == cudaSuccess) {
        if (precision == TDBEM_FP64)
            e = invert_f64(dA, n, perm, status, static_cast<double*>(scratch), &nl, &singular, s);
        else
            e = invert_f32(dA, dX, n, perm, status, static_cast<float*>(scratch), &nl, &singular,
                           s, &rep);
    }
    std::vector<float> hx;
    if (e == cudaSuccess && !singular) {
        if (precision == TDBEM_FP64) {
            e = cudaMemcpyAsync(X, dA, sizeof(double) * nn, cudaMemcpyDeviceToHost, s);
        } else {
            hx.resize(nn);
            e = cudaMemcpyAsync(hx.data(), dX, sizeof(float) * nn, cudaMemcpyDeviceToHost, s);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    release();
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? TDBEM_ERR_NOMEM : TDBEM_ERR_CUDA,
                    "tdbem_invert: %s", cudaGetErrorString(e));
    if (singular) return fail(TDBEM_ERR_SINGULAR, "zero pivot in the inversion");
    for (size_t i = 0; i < hx.size(); i++) X[i] = hx[i];
    if (probe) *probe = precision == TDBEM_MIXED ? rep.probe_rel : 0.0;
    if (full_search) *full_search = precision == TDBEM_MIXED ? rep.full_search : 1;
    return TDBEM_OK;
}

int tdbem_history_device(const tdbem_ctx* c, const double** u_hist, const double** t_hist) {
    if (!c || !u_hist || !t_hist) return fail(TDBEM_ERR_ARG, "null argument");
    if (c->hist_steps < 0) return fail(TDBEM_ERR_STATE, "no march has run");
    *u_hist = c->d_u;
    *t_hist = c->d_t;
    return TDBEM_OK;
}

}  // extern "C"
