// Serving: a request loop for transient solves with continuous batching.
//
// A request is a whole transient solve (mesh, material, time step, boundary
// conditions, weights, load history, step count, precision).  The server keeps
// a queue in arrival order and a fixed number of slots.  A free slot admits the
// oldest queued request whose device footprint (tdbem_footprint: levels x D^2 x
// bytes x 2 plus the marching state) fits in what is left of the HBM budget; a
// request may overtake an older one that does not fit, at most kMaxBypass times,
// after which the server waits for memory to free up for the older one (no
// starvation).  An admitted solve owns a context with its own CUDA stream: its
// slot's thread assembles the levels and prepares the march (inverses, histories)
// there, concurrently with the other slots.
//
// The time steps of the resident solves are batched: one march thread advances
// every prepared solve of a precision by a time block of kGroupNB steps in ONE
// persistent cooperative launch (group_march.cu), each solve at its own step (a
// per-solve step offset), and repeats.  A solve that finishes its steps is
// retired at the block boundary (histories copied to the host, slot released);
// one that finishes its preparation joins at the next block boundary, so requests
// that arrive while others march are admitted into the running batch.  The
// grouped kernels compute each solve's rows with a fixed lane count and a fixed
// reduction order whatever the other solves are, so a result is bitwise the same
// served alone and in any mix.
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "capi_common.cuh"

namespace {

constexpr int kMaxBypass = 8;

int sfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    tdbem::note_error(buf);
    return code;
}

struct Request {
    long long id = 0;
    std::vector<double> coords;
    std::vector<int> ien;
    int nnd = 0, nel = 0, etype = 1;
    tdbem_material mat{};
    double dt = 0;
    int nq = 6, if_ext = 0;
    std::vector<int> ubc, fbc;
    std::vector<double> ubc_v, fbc_v;
    double a1 = 0, a2 = 0;
    std::vector<double> amp;
    int numstep = 0, precision = TDBEM_MIXED;
    size_t footprint = 0;
    int state = TDBEM_REQ_QUEUED;
    int rc = TDBEM_OK;
    std::string error;
    std::vector<double> u, t;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int bypassed = 0;
    // batched marching
    tdbem_ctx* ctx = nullptr;
    tdbem::GroupMarch gm{};
    bool marched = false;  // the march thread has retired it
};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct tdbem_server {
    int device = 0;
    size_t budget = 0;
    int slots = 1;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_march;
    std::deque<Request*> queue;
    std::unordered_map<long long, std::unique_ptr<Request>> reqs;
    long long next_id = 1;
    size_t used = 0;
    int active = 0;
    bool stop = false;
    long long completed = 0;
    double dof_steps_done = 0;
    std::vector<std::thread> workers;
    // batched marching: prepared solves wait in `ready` for the next block boundary;
    // `resident` are marching, per precision (0: FP64, 1: TDBEM_MIXED)
    std::vector<Request*> ready;
    std::vector<Request*> resident[2];
    long long global_step[2] = {1, 1};  // start of the next block, per precision
    long long rounds = 0, solve_steps = 0, resident_sum = 0;
    std::thread marcher;
    cudaStream_t mstream = nullptr;
    tdbem::GroupMarch* d_gm = nullptr;
    size_t d_gm_cap = 0;

    // Oldest queued request that fits; called with mu held.
    Request* pick() {
        for (size_t i = 0; i < queue.size(); i++) {
            Request* r = queue[i];
            if (used + r->footprint <= budget) {
                for (size_t j = 0; j < i; j++) queue[j]->bypassed++;
                queue.erase(queue.begin() + (long)i);
                return r;
            }
            if (r->bypassed >= kMaxBypass) return nullptr;  // the older one goes first
        }
        return nullptr;
    }

    // A slot's part: the solve's context, levels and march preparation (on the
    // context's own stream).
    void prepare(Request* r) {
        cudaSetDevice(device);
        tdbem_mesh mesh{r->nnd, r->nel, r->etype, r->coords.data(), r->ien.data()};
        tdbem_ctx* ctx = nullptr;
        int rc = tdbem_ctx_create(&mesh, &r->mat, r->dt, r->nq, r->if_ext, &ctx);
        if (rc == TDBEM_OK)
            rc = tdbem_set_bc(ctx, r->ubc.data(), r->ubc_v.data(), (int)r->ubc.size(),
                              r->fbc.data(), r->fbc_v.data(), (int)r->fbc.size());
        if (rc == TDBEM_OK) rc = tdbem_set_alpha(ctx, r->a1, r->a2);
        if (rc == TDBEM_OK && !r->amp.empty())
            rc = tdbem_set_load_history(ctx, r->amp.data(), (int)r->amp.size());
        if (rc == TDBEM_OK) rc = tdbem_assemble_levels(ctx, r->numstep, r->precision);
        if (rc == TDBEM_OK)
            rc = tdbem::capi::group_prepare(ctx, r->numstep, r->precision == TDBEM_MIXED,
                                            r->gm);
        if (rc != TDBEM_OK) {
            r->error = tdbem_last_error();
            if (ctx) tdbem_ctx_destroy(ctx);
            ctx = nullptr;
        }
        r->rc = rc;
        r->ctx = ctx;
    }

    void worker() {
        std::unique_lock<std::mutex> lock(mu);
        while (true) {
            Request* r = nullptr;
            cv_work.wait(lock, [&] { return stop || (r = pick()) != nullptr; });
            if (!r) return;  // stopping with nothing admissible
            used += r->footprint;
            active++;
            r->state = TDBEM_REQ_RUNNING;
            r->t_admit = now_s(t0);
            lock.unlock();
            prepare(r);
            lock.lock();
            if (r->rc == TDBEM_OK) {  // hand over to the march thread and hold the slot
                ready.push_back(r);
                cv_march.notify_one();
                cv_done.wait(lock, [&] { return r->marched; });
            }
            if (r->ctx) {
                lock.unlock();
                tdbem_ctx_destroy(r->ctx);
                lock.lock();
                r->ctx = nullptr;
            }
            used -= r->footprint;
            active--;
            r->t_done = now_s(t0);
            r->state = r->rc == TDBEM_OK ? TDBEM_REQ_DONE : TDBEM_REQ_FAILED;
            completed++;
            if (r->rc == TDBEM_OK) dof_steps_done += 3.0 * r->nnd * r->numstep;
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }

    // One time block of every resident solve of one precision, in one launch.
    int march_block(int prec) {
        std::vector<Request*>& res = resident[prec];
        const int n = (int)res.size();
        std::vector<tdbem::GroupMarch> gm(n);
        for (int i = 0; i < n; i++) gm[i] = res[i]->gm;
        unsigned nrows = 0, nw = 0, nquads = 0, nwold = 0;
        tdbem::capi::group_layout(gm.data(), n, &nrows, &nw, &nquads, &nwold);
        if ((size_t)n > d_gm_cap) {
            if (d_gm) cudaFree(d_gm);
            d_gm = nullptr;
            d_gm_cap = 0;
            if (cudaMalloc(&d_gm, sizeof(tdbem::GroupMarch) * (size_t)n * 2) != cudaSuccess)
                return sfail(TDBEM_ERR_NOMEM, "server: group descriptors");
            d_gm_cap = (size_t)n * 2;
        }
        cudaError_t e = cudaMemcpyAsync(d_gm, gm.data(), sizeof(tdbem::GroupMarch) * n,
                                        cudaMemcpyHostToDevice, mstream);
        const long long S = global_step[prec];
        // a fixed shape: the lane count fixes every row's reduction order, so a
        // result does not depend on the other resident solves
        const tdbem::GroupShape shape{16, 256, 2};
        const int step_hi = (int)S + tdbem::kGroupNB;
        if (e == cudaSuccess)
            e = tdbem::launch_march_group(d_gm, n, nrows, nw, nquads, nwold, (int)S, step_hi,
                                          shape, prec == 1, mstream, true);
        if (e == cudaSuccess) e = cudaStreamSynchronize(mstream);
        if (e != cudaSuccess)
            return sfail(TDBEM_ERR_CUDA, "server: grouped march: %s", cudaGetErrorString(e));
        global_step[prec] = step_hi;
        rounds++;
        resident_sum += n;
        for (auto* r : res) {
            const long long lo = std::max<long long>(1, S - r->gm.off);
            const long long hi = std::min<long long>(r->numstep, step_hi - r->gm.off);
            if (hi > lo) solve_steps += hi - lo;
        }
        return TDBEM_OK;
    }

    // Histories of a finished solve to the host.
    int collect(Request* r) {
        const size_t n = (size_t)(r->numstep + 1) * 3 * r->nnd;
        r->u.assign(n, 0.0);
        r->t.assign(n, 0.0);
        cudaError_t e = cudaMemcpyAsync(r->u.data(), r->gm.u, sizeof(double) * n,
                                        cudaMemcpyDeviceToHost, mstream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(r->t.data(), r->gm.t, sizeof(double) * n,
                                cudaMemcpyDeviceToHost, mstream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(mstream);
        if (e != cudaSuccess)
            return sfail(TDBEM_ERR_CUDA, "server: histories: %s", cudaGetErrorString(e));
        return TDBEM_OK;
    }

    void march_loop() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lock(mu);
        while (true) {
            cv_march.wait(lock, [&] {
                return stop || !ready.empty() || !resident[0].empty() || !resident[1].empty();
            });
            if (stop && ready.empty() && resident[0].empty() && resident[1].empty()) return;
            // solves prepared since the last boundary join at this one
            for (Request* r : ready) {
                const int prec = r->precision == TDBEM_MIXED ? 1 : 0;
                r->gm.off = (int)(global_step[prec] - 1);
                resident[prec].push_back(r);
            }
            ready.clear();
            lock.unlock();
            int rcs[2] = {TDBEM_OK, TDBEM_OK};
            std::string msg[2];
            for (int prec = 0; prec < 2; prec++) {
                bool any = false;  // solves of one step have nothing to march
                for (auto* r : resident[prec]) any = any || r->numstep >= 2;
                if (!any) continue;
                rcs[prec] = march_block(prec);
                if (rcs[prec] != TDBEM_OK) msg[prec] = tdbem_last_error();
            }
            lock.lock();
            for (int prec = 0; prec < 2; prec++) {
                std::vector<Request*> keep;
                for (Request* r : resident[prec]) {
                    // done once the launches have passed its last step (numstep - 1)
                    const bool done =
                        rcs[prec] != TDBEM_OK || global_step[prec] - r->gm.off >= r->numstep;
                    if (!done) {
                        keep.push_back(r);
                        continue;
                    }
                    if (rcs[prec] != TDBEM_OK) {
                        r->rc = rcs[prec];
                        r->error = msg[prec];
                    } else {
                        lock.unlock();
                        const int rc = collect(r);
                        lock.lock();
                        if (rc != TDBEM_OK) {
                            r->rc = rc;
                            r->error = tdbem_last_error();
                        }
                    }
                    r->marched = true;
                }
                resident[prec].swap(keep);
            }
            cv_done.notify_all();
        }
    }
};

extern "C" {

int tdbem_server_create(int device, size_t hbm_budget, int slots, tdbem_server** out) {
    if (!out) return sfail(TDBEM_ERR_ARG, "out is null");
    *out = nullptr;
    if (slots < 1 || slots > 64) return sfail(TDBEM_ERR_ARG, "slots must be in 1..64");
    if (cudaSetDevice(device) != cudaSuccess) return sfail(TDBEM_ERR_CUDA, "device %d", device);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess)
        return sfail(TDBEM_ERR_CUDA, "cudaMemGetInfo failed");
    auto* s = new (std::nothrow) tdbem_server();
    if (!s) return sfail(TDBEM_ERR_NOMEM, "server allocation");
    s->device = device;
    // memory the library keeps for reuse counts as free: contexts take it first
    size_t kept = 0;
    tdbem_cached_memory(device, &kept);
    s->budget = hbm_budget ? hbm_budget : (free_b + kept) / 10 * 9;
    s->slots = slots;
    s->t0 = std::chrono::steady_clock::now();
    if (cudaStreamCreateWithFlags(&s->mstream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return sfail(TDBEM_ERR_CUDA, "server stream");
    }
    s->marcher = std::thread([s] { s->march_loop(); });
    for (int i = 0; i < slots; i++) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return TDBEM_OK;
}

int tdbem_server_submit(tdbem_server* s, const tdbem_request* q, long long* id) {
    if (!s || !q || !id) return sfail(TDBEM_ERR_ARG, "null argument");
    const tdbem_mesh& m = q->mesh;
    if (!m.coords || !m.ien || m.nnd < 2 || m.nel < 1 || q->numstep < 1)
        return sfail(TDBEM_ERR_ARG, "invalid request");
    if ((q->n_u && (!q->ubc_dofs || !q->ubc_vals)) || (q->n_f && (!q->fbc_dofs || !q->fbc_vals)))
        return sfail(TDBEM_ERR_ARG, "boundary-condition arrays are null");
    size_t fp = 0;
    const int rc = tdbem_footprint(&q->mesh, &q->mat, q->dt, q->nq, q->numstep, q->precision, &fp);
    if (rc != TDBEM_OK) return rc;
    if (fp > s->budget)
        return sfail(TDBEM_ERR_NOMEM, "request needs %zu bytes, the budget is %zu", fp, s->budget);
    auto r = std::make_unique<Request>();
    r->coords.assign(m.coords, m.coords + 3 * (size_t)m.nnd);
    r->ien.assign(m.ien, m.ien + (m.etype == 2 ? 8 : 4) * (size_t)m.nel);
    r->nnd = m.nnd;
    r->nel = m.nel;
    r->etype = m.etype;
    r->mat = q->mat;
    r->dt = q->dt;
    r->nq = q->nq;
    r->if_ext = q->if_ext;
    r->ubc.assign(q->ubc_dofs, q->ubc_dofs + q->n_u);
    r->ubc_v.assign(q->ubc_vals, q->ubc_vals + q->n_u);
    r->fbc.assign(q->fbc_dofs, q->fbc_dofs + q->n_f);
    r->fbc_v.assign(q->fbc_vals, q->fbc_vals + q->n_f);
    r->a1 = q->alpha1;
    r->a2 = q->alpha2;
    if (q->amp) r->amp.assign(q->amp, q->amp + q->numstep);
    r->numstep = q->numstep;
    r->precision = q->precision;
    r->footprint = fp;
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return sfail(TDBEM_ERR_STATE, "server is stopping");
    r->id = s->next_id++;
    r->t_submit = now_s(s->t0);
    *id = r->id;
    s->queue.push_back(r.get());
    s->reqs.emplace(r->id, std::move(r));
    s->cv_work.notify_one();
    return TDBEM_OK;
}

int tdbem_server_wait(tdbem_server* s, long long id, double timeout_s, int* state) {
    if (!s || !state) return sfail(TDBEM_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(TDBEM_ERR_ARG, "unknown request %lld", id);
    Request* r = it->second.get();
    auto done = [&] { return r->state == TDBEM_REQ_DONE || r->state == TDBEM_REQ_FAILED; };
    if (timeout_s < 0) s->cv_done.wait(lock, done);
    else s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), done);
    *state = r->state;
    return TDBEM_OK;
}

int tdbem_server_result(tdbem_server* s, long long id, double* u_hist, double* t_hist,
                        double* times) {
    if (!s) return sfail(TDBEM_ERR_ARG, "null server");
    std::unique_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) return sfail(TDBEM_ERR_ARG, "unknown request %lld", id);
        const int st = it->second->state;
        if (st != TDBEM_REQ_DONE && st != TDBEM_REQ_FAILED)
            return sfail(TDBEM_ERR_STATE, "request %lld has not finished", id);
        r = std::move(it->second);
        s->reqs.erase(it);
    }
    if (times) {
        times[0] = r->t_admit - r->t_submit;  // queued
        times[1] = r->t_done - r->t_admit;    // on the GPU
        times[2] = r->t_done - r->t_submit;   // latency
    }
    if (r->state == TDBEM_REQ_FAILED)
        return sfail(r->rc, "request %lld failed: %s", id, r->error.c_str());
    if (u_hist) std::memcpy(u_hist, r->u.data(), sizeof(double) * r->u.size());
    if (t_hist) std::memcpy(t_hist, r->t.data(), sizeof(double) * r->t.size());
    return TDBEM_OK;
}

int tdbem_server_stats(tdbem_server* s, size_t* used_bytes, size_t* budget_bytes, int* active,
                       int* queued, long long* completed) {
    if (!s) return sfail(TDBEM_ERR_ARG, "null server");
    std::lock_guard<std::mutex> lock(s->mu);
    if (used_bytes) *used_bytes = s->used;
    if (budget_bytes) *budget_bytes = s->budget;
    if (active) *active = s->active;
    if (queued) *queued = (int)s->queue.size();
    if (completed) *completed = s->completed;
    return TDBEM_OK;
}

int tdbem_server_march_stats(tdbem_server* s, long long* launches, long long* solve_steps,
                             double* mean_resident) {
    if (!s) return sfail(TDBEM_ERR_ARG, "null server");
    std::lock_guard<std::mutex> lock(s->mu);
    if (launches) *launches = s->rounds;
    if (solve_steps) *solve_steps = s->solve_steps;
    if (mean_resident) *mean_resident = s->rounds ? (double)s->resident_sum / s->rounds : 0.0;
    return TDBEM_OK;
}

int tdbem_server_destroy(tdbem_server* s) {
    if (!s) return TDBEM_OK;
    {
        // finish what is queued or running, then stop the workers
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv_done.wait(lock, [&] { return s->queue.empty() && s->active == 0; });
        s->stop = true;
        s->cv_work.notify_all();
    }
    for (auto& w : s->workers) w.join();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->cv_march.notify_all();
    }
    s->marcher.join();
    if (s->d_gm) cudaFree(s->d_gm);
    cudaStreamDestroy(s->mstream);
    delete s;
    return TDBEM_OK;
}

}  // extern "C"
