// C ABI of tdbem-gb300, batched marching of many load cases on one mesh
// (tdbem_march_batch) and its options.
#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

extern "C" {

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
        if (!c->d_tc_err) CUDA_TRY(dalloc(&c->d_tc_err, 2));
        CUDA_TRY(cudaMemsetAsync(c->d_tc_err, 0, 2 * sizeof(int), s));
        int rm = ensure_merged_levels(c);
        // profiling: the level slabs' live tiles (the product's bytes)
        if (rm == TDBEM_OK && c->prof) rm = count_live_tiles(c);
        if (rm != TDBEM_OK) return rm;
        const size_t wb = tc_w_bytes(D, C, Lw, 1);
        if (c->tc_W_bytes < wb) {
            mem_free(c->d_tc_W);
            c->d_tc_W = nullptr;
            c->tc_W_bytes = 0;
            CUDA_TRY(mem_alloc(&c->d_tc_W, wb));
            c->tc_W_bytes = wb;
        }
        if (!make_tc_maps(c->d_mtc_planes, D, mtc_slabs(M), c->d_tc_W, C, Lw, &c->tc_maps, 1))
            return fail(TDBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed for the batched planes");
        if (!c->d_bkt) {
            CUDA_TRY(dalloc(&c->d_bkt, 2 * CD));
            CUDA_TRY(dalloc(&c->d_bGK, (size_t)(M + 1) * CD));
            CUDA_TRY(dalloc(&c->d_bGL, 2 * CD));
        }
        const int pk = prof_begin(c, TDBEM_K_AUX);
        CUDA_TRY(launch_batch_known_tractions(c->d_btrac, c->d_is_ubc, D, C, c->d_bkt,
                                              c->d_bkt + CD, s));
        CUDA_TRY(levels_times_columns(c->d_Gf, c->ldf, D, M + 1, c->d_bkt, C, c->d_bGK, s));
        CUDA_TRY(levels_times_columns(c->d_Gf, c->ldf, D, std::min(2, M + 1), c->d_bkt + CD, C,
                                      c->d_bGL, s));
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
            CUDA_TRY(launch_conv_tc(c->tc_maps, D, mtc_slabs(M), Lw, nlev, C, c->d_bpart, splits,
                                    c->d_tc_err, s, 1, c->tc_wait_ns, 0, c->d_mtc_occ));
            const double pb = conv_plane_bytes(c, 0, nlev);
            prof_end(c, pe, pb + nlev * cp * ldb * 4, pb / 4 * 2.0 * C);
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
        const int sweeps =
            (st == 1 && c->step2_sweeps > 0) ? std::max(c->step2_sweeps, c->batch_refine)
                                             : c->batch_refine;
        for (int it = 0; it < sweeps; it++) {
            CUDA_TRY(launch_apply_cols(c->d_Hc64[v], 1, D, c->d_bx, C, c->d_bpart, sp, s));
            CUDA_TRY(launch_reduce_cols(c->d_bpart, sp, C, D, c->d_brhs, c->d_br, s));
            CUDA_TRY(launch_apply_cols(c->d_inv32[v], 0, D, c->d_br, C, c->d_bpart, sp, s));
            CUDA_TRY(launch_reduce_cols(c->d_bpart, sp, C, D, c->d_bx, c->d_bx, s));
        }
        CUDA_TRY(launch_update_batch(c->d_bx, D, C, st, c->d_is_ubc, c->d_ubc_map, c->d_btrac,
                                     d_amp, numstep, c->d_bu, c->d_bt, s));
        prof_end(c, pe, DD * 4 * (1 + sweeps) + DD * 8 * sweeps, 2.0 * DD * C * (1 + 2 * sweeps));
        c->launches += 6 + 4LL * sweeps;
    }
    c->timings[2] = tmr.stop_ms(s);
    if (tc) {
        int code[2] = {0, 0};
        CUDA_TRY(cudaMemcpyAsync(code, c->d_tc_err, sizeof(code), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        const int rc = tc_status(code, "batched march");
        if (rc != TDBEM_OK) return rc;
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

}  // extern "C"
