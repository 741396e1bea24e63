// Persistent marching of many meshes: every step of every mesh in one
// cooperative launch.
//
// Each mesh is a Solve_Averaging march (SolverStepLinearT.cpp:314-544).
//
// FP64 levels (k_march_group, as march.cu's per-step kernels), per step three
// phases separated by grid-wide barriers:
//   A  combined history vectors W_f of every mesh (march.cu: k_history_combine);
//   B  rhs = sum_f (G^f W_t[f] - H^f W_u[f]): one group of LANES lanes per row
//      of every mesh, FP64 partial sums per lane, fixed-order shuffle reduction;
//   C  x = inv(LHS) rhs with the mesh's FP64 inverse, one lane group per row,
//      and the state update of that dof (march.cu: k_update_state).
//
// Mixed levels (k_march_group_tb, as march_mixed.cu): FP32 levels, time blocks of
// kGroupNB steps.  At the start of a block, the part of the next kGroupNB
// right-hand sides that only needs history from before the block is one pass
// over the levels with kGroupNB columns (old-W build | product, each lane group
// four rows of one mesh so that every 16-byte load of W serves four rows); then
// per step the new-history part over levels f <= s - S + 1 (new-W build |
// product), x0 = inv32 rhs | r = rhs - A64 x0 (FP64) | x = x0 + inv32 r with the
// state update.
//
// Meshes with fewer steps idle once done.  The row loops are uniform across
// each warp and every lane joins the shuffle reductions (rows past the end or of
// a finished mesh contribute zero).  The lane count per row and the launch shape
// are picked by timing (capi.cu: the group autotuner).
#include <cooperative_groups.h>

#include <algorithm>

#include "tdbem_internal.cuh"

namespace cg = cooperative_groups;

namespace tdbem {

namespace {

// Last mesh whose first entry of the given list is <= x.
template <typename F>
__device__ __forceinline__ int mesh_of(const GroupMarch* __restrict__ gm, int nmesh, unsigned x,
                                       F begin) {
    int lo = 0, hi = nmesh - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (begin(gm[mid]) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct RowBegin {
    __device__ unsigned operator()(const GroupMarch& g) const { return g.row_begin; }
};
struct WBegin {
    __device__ unsigned operator()(const GroupMarch& g) const { return g.w_begin; }
};
struct QuadBegin {
    __device__ unsigned operator()(const GroupMarch& g) const { return g.quad_begin; }
};
struct WoldBegin {
    __device__ unsigned operator()(const GroupMarch& g) const { return g.wold_begin; }
};

template <int LANES>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, LANES);
    return v;
}

__device__ __forceinline__ float dot4(const float4 a, const float4 b) {
    return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}

// The history combination of k_history_combine / k_build_w_old / k_build_w_new:
// histories m with lo <= m < hi (and m >= 1) enter; loads only when with_load.
__device__ __forceinline__ void combine(const GroupMarch& g, int s, int f, int j, int lo, int hi,
                                        bool with_load, double& wt, double& wu) {
    const double* th = g.t;
    const double* uh = g.u;
    const int D = g.D;
    wt = 0;
    wu = 0;
    const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
    auto in = [&](int m) { return m >= 1 && m >= lo && m < hi; };
    if (f >= 2 && in(m1)) {
        wt += g.a1 * th[(size_t)m1 * D + j];
        wu += g.a1 * uh[(size_t)m1 * D + j];
    }
    if (f >= 1 && in(m3)) {
        wt += g.a3 * th[(size_t)m3 * D + j];
        wu += g.a3 * uh[(size_t)m3 * D + j];
    }
    if (in(m2)) {
        wt += g.a2 * th[(size_t)m2 * D + j];
        wu += g.a2 * uh[(size_t)m2 * D + j];
    }
    if (f == 0 && in(s - 1)) {
        wt -= g.a1 * th[(size_t)(s - 1) * D + j];
        wu -= g.a1 * uh[(size_t)(s - 1) * D + j];
    }
    if (with_load && f <= 1) {
        const double c0 = s == 1 ? 1.0 : g.c0, c1 = s == 1 ? 0.0 : g.c1;
        const double cf = f == 0 ? c0 : c1;
        const double amp = g.amp ? g.amp[s] : 1.0;
        wt += cf * (amp * g.load_t[j]);
        wu += cf * g.load_u[j];
    }
}

// State update of dof j at step s (march.cu: k_update_state).
__device__ __forceinline__ void update_dof(const GroupMarch& g, int s, int j, double x) {
    const int D = g.D;
    const double amp = g.amp ? g.amp[s] : 1.0;
    const bool u = g.is_u[j] != 0, f = g.is_f[j] != 0;
    g.u[(size_t)s * D + j] = u ? g.ubc[j] : x;
    double tv = f ? g.fbc[j] * amp : 0.0;
    if (u && j < D - 1) tv = x;
    g.t[(size_t)s * D + j] = tv;
}

// ---------------------------------------------------------------- FP64 levels
template <int LANES>
__global__ void __launch_bounds__(512) k_march_group(const GroupMarch* __restrict__ gm, int nmesh,
                                                     unsigned nrows, unsigned nw, int st_lo,
                                                     int st_hi) {
    cg::grid_group grid = cg::this_grid();
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x % LANES;
    const unsigned ngroups = nthreads / LANES;
    const unsigned warp_group0 = (tid / 32) * (32 / LANES);  // the warp's first lane group
    const unsigned sub = (threadIdx.x % 32) / LANES;          // this lane's group in the warp
    for (int st = st_lo; st < st_hi; st++) {
        // ---- A: combined history vectors (levels f <= L of each mesh)
        for (unsigned idx = tid; idx < nw; idx += nthreads) {
            const GroupMarch& g = gm[mesh_of(gm, nmesh, idx, WBegin{})];
            const int ls = st - g.off;  // the mesh's own step
            if (ls < 1 || ls >= g.numstep) continue;
            const unsigned loc = idx - g.w_begin;
            const int f = (int)(loc / g.D), j = (int)(loc % g.D);
            if (f > min(max(ls, 1), g.M)) continue;
            double wt, wu;
            combine(g, ls, f, j, 1, ls, true, wt, wu);
            g.Wt[loc] = wt;
            g.Wu[loc] = wu;
        }
        grid.sync();
        // ---- B: history convolution, one lane group per row
        for (unsigned base = warp_group0; base < nrows; base += ngroups) {
            const unsigned r = base + sub;
            const GroupMarch* g = r < nrows ? &gm[mesh_of(gm, nmesh, r, RowBegin{})] : nullptr;
            const int ls = g ? st - g->off : 0;
            const bool live = g && ls >= 1 && ls < g->numstep;
            double acc = 0;
            if (live) {
                const int row = (int)(r - g->row_begin), D = g->D;
                const int L = min(max(ls, 1), g->M);
                for (int f = 0; f <= L; f++) {
                    const double* Gr = g->G + ((size_t)f * D + row) * D;
                    const double* Hr = g->H + ((size_t)f * D + row) * D;
                    const double* wt = g->Wt + (size_t)f * D;
                    const double* wu = g->Wu + (size_t)f * D;
                    for (int k = lane; k < D; k += LANES)
                        acc += __ldcs(Gr + k) * wt[k] - __ldcs(Hr + k) * wu[k];
                }
            }
            acc = group_sum<LANES>(acc);
            if (live && lane == 0) g->rhs[r - g->row_begin] = acc;
        }
        grid.sync();
        // ---- C: solve with the inverse, state update of the row's dof
        for (unsigned base = warp_group0; base < nrows; base += ngroups) {
            const unsigned r = base + sub;
            const GroupMarch* g = r < nrows ? &gm[mesh_of(gm, nmesh, r, RowBegin{})] : nullptr;
            const int ls = g ? st - g->off : 0;
            const bool live = g && ls >= 1 && ls < g->numstep;
            double acc = 0;
            int j = 0;
            if (live) {
                j = (int)(r - g->row_begin);
                const double* Ar = (ls == 1 ? g->Ainv0 : g->Ainv1) + (size_t)j * g->D;
                for (int k = lane; k < g->D; k += LANES) acc += Ar[k] * g->rhs[k];
            }
            acc = group_sum<LANES>(acc);
            if (live && lane == 0) update_dof(*g, ls, j, acc);
        }
        grid.sync();
    }
}

// ---------------------------------------------------------------- mixed levels
template <int LANES>
__global__ void __launch_bounds__(512) k_march_group_tb(const GroupMarch* __restrict__ gm,
                                                        int nmesh, unsigned nrows, unsigned nw,
                                                        unsigned nquads, unsigned nwold,
                                                        int st_lo, int st_hi, int has_offsets) {
    constexpr int NB = kGroupNB, RQ = 4;
    cg::grid_group grid = cg::this_grid();
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x % LANES;
    const unsigned ngroups = nthreads / LANES;
    const unsigned warp_group0 = (tid / 32) * (32 / LANES);
    const unsigned sub = (threadIdx.x % 32) / LANES;
    for (int S = st_lo; S < st_hi; S += NB) {
        // meshes join at block starts: a mesh's own block start lS = S - off is 1 or a
        // later block start of its march
        if (S > 1 || has_offsets) {
            // ---- old-history vectors of the block: W_f^old[:, j], s = lS + j, m < lS
            for (unsigned idx = tid; idx < nwold; idx += nthreads) {
                const GroupMarch& g = gm[mesh_of(gm, nmesh, idx, WoldBegin{})];
                const int lS = S - g.off;
                if (lS <= 1 || lS >= g.numstep) continue;
                const unsigned loc = idx - g.wold_begin;
                const int k = (int)(loc % g.D);
                const int j = (int)((loc / g.D) % NB);
                const int f = (int)(loc / ((unsigned)g.D * NB));
                const int nbe = min(NB, g.numstep - lS);
                if (f > min(g.M, lS + nbe - 1)) continue;
                double wt, wu;
                combine(g, lS + j, f, k, 1, lS, false, wt, wu);
                const size_t o = ((size_t)f * NB + j) * g.ldf + k;
                g.Wold_t[o] = (float)wt;
                g.Wold_u[o] = (float)wu;
            }
            grid.sync();
            // ---- Y_old[j][row] = sum_f X^f[row] . W_f^old[j], four rows per lane group
            for (unsigned base = warp_group0; base < nquads; base += ngroups) {
                const unsigned q = base + sub;
                const GroupMarch* g =
                    q < nquads ? &gm[mesh_of(gm, nmesh, q, QuadBegin{})] : nullptr;
                const int lS = g ? S - g->off : 0;
                const bool live = g && lS > 1 && lS < g->numstep;
                float acc[RQ][NB];
#pragma unroll
                for (int r = 0; r < RQ; r++)
#pragma unroll
                    for (int j = 0; j < NB; j++) acc[r][j] = 0.f;
                int row0 = 0;
                if (live) {
                    const int D = g->D, ld4 = g->ldf / 4;
                    row0 = (int)(q - g->quad_begin) * RQ;
                    const int nbe = min(NB, g->numstep - lS);
                    const int nlev = min(g->M, lS + nbe - 1) + 1;
                    size_t rowoff[RQ];
#pragma unroll
                    for (int r = 0; r < RQ; r++) rowoff[r] = (size_t)min(row0 + r, D - 1) * ld4;
                    for (int f = 0; f < nlev; f++) {
                        const float4* G4 =
                            reinterpret_cast<const float4*>(g->Gf) + (size_t)f * D * ld4;
                        const float4* H4 =
                            reinterpret_cast<const float4*>(g->Hf) + (size_t)f * D * ld4;
                        const float4* wt =
                            reinterpret_cast<const float4*>(g->Wold_t) + (size_t)f * NB * ld4;
                        const float4* wu =
                            reinterpret_cast<const float4*>(g->Wold_u) + (size_t)f * NB * ld4;
                        for (int k4 = lane; k4 < ld4; k4 += LANES) {
                            float4 a[RQ], b[RQ];
#pragma unroll
                            for (int r = 0; r < RQ; r++) {
                                a[r] = __ldcs(G4 + rowoff[r] + k4);
                                b[r] = __ldcs(H4 + rowoff[r] + k4);
                            }
#pragma unroll
                            for (int j = 0; j < NB; j++) {
                                const float4 x = wt[(size_t)j * ld4 + k4];
                                const float4 y = wu[(size_t)j * ld4 + k4];
#pragma unroll
                                for (int r = 0; r < RQ; r++)
                                    acc[r][j] += dot4(a[r], x) - dot4(b[r], y);
                            }
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < RQ; r++)
#pragma unroll
                    for (int j = 0; j < NB; j++) {
                        const double v = group_sum<LANES>((double)acc[r][j]);
                        if (live && lane == 0 && row0 + r < g->D)
                            g->Yold[(size_t)j * g->D + row0 + r] = v;
                    }
            }
            grid.sync();
        }
        for (int jb = 0; jb < NB && S + jb < st_hi; jb++) {
            const int st = S + jb;
            // ---- new-history vectors: m >= S, and the known loads, levels f <= s - S + 1
            for (unsigned idx = tid; idx < nw; idx += nthreads) {
                const GroupMarch& g = gm[mesh_of(gm, nmesh, idx, WBegin{})];
                const int ls = st - g.off, lS = S - g.off;
                if (ls < 1 || ls >= g.numstep) continue;
                const unsigned loc = idx - g.w_begin;
                const int f = (int)(loc / g.D), k = (int)(loc % g.D);
                if (f > min(g.M, max(1, st + 1 - S))) continue;
                double wt, wu;
                combine(g, ls, f, k, lS, ls, true, wt, wu);
                g.Wtf[(size_t)f * g.ldf + k] = (float)wt;
                g.Wuf[(size_t)f * g.ldf + k] = (float)wu;
            }
            grid.sync();
            // ---- rhs = Y_old[jb] + sum_{f <= L} X^f . W_f^new
            for (unsigned base = warp_group0; base < nrows; base += ngroups) {
                const unsigned r = base + sub;
                const GroupMarch* g = r < nrows ? &gm[mesh_of(gm, nmesh, r, RowBegin{})] : nullptr;
                const int ls = g ? st - g->off : 0, lS = g ? S - g->off : 0;
                const bool live = g && ls >= 1 && ls < g->numstep;
                double acc = 0;
                int row = 0;
                if (live) {
                    row = (int)(r - g->row_begin);
                    const int D = g->D, ld4 = g->ldf / 4;
                    const int L = min(g->M, max(1, st + 1 - S));
                    for (int f = 0; f <= L; f++) {
                        const float4* G4 =
                            reinterpret_cast<const float4*>(g->Gf) + ((size_t)f * D + row) * ld4;
                        const float4* H4 =
                            reinterpret_cast<const float4*>(g->Hf) + ((size_t)f * D + row) * ld4;
                        const float4* wt = reinterpret_cast<const float4*>(g->Wtf) + (size_t)f * ld4;
                        const float4* wu = reinterpret_cast<const float4*>(g->Wuf) + (size_t)f * ld4;
                        float a32 = 0.f;
                        for (int k4 = lane; k4 < ld4; k4 += LANES)
                            a32 += dot4(__ldcs(G4 + k4), wt[k4]) - dot4(__ldcs(H4 + k4), wu[k4]);
                        acc += (double)a32;
                    }
                }
                acc = group_sum<LANES>(acc);
                if (live && lane == 0)
                    g->rhs[row] = acc + (lS > 1 ? g->Yold[(size_t)jb * g->D + row] : 0.0);
            }
            grid.sync();
            // ---- x0 = inv32 rhs | r = rhs - A64 x0 | x = x0 + inv32 r, state update; a mesh
            // at its step 1 whose step-2 LHS has no inverse of its own repeats the last two
            // (Richardson sweeps with the later inverse).  The sweep count is the same for
            // every thread: the largest any mesh needs at this step.
            int nsw = 3;
            for (int i = 0; i < nmesh; i++)
                if (st - gm[i].off == 1 && gm[i].step2_sweeps > 0)
                    nsw = max(nsw, 1 + 2 * gm[i].step2_sweeps);
            for (int sweep = 0; sweep < nsw; sweep++) {
                for (unsigned base = warp_group0; base < nrows; base += ngroups) {
                    const unsigned r = base + sub;
                    const GroupMarch* g =
                        r < nrows ? &gm[mesh_of(gm, nmesh, r, RowBegin{})] : nullptr;
                    const int ls = g ? st - g->off : 0;
                    const int msw = !g ? 0
                                    : (ls == 1 && g->step2_sweeps > 0) ? 1 + 2 * g->step2_sweeps
                                    : g->refine > 0                    ? 3
                                                                       : 1;
                    const bool live = g && ls >= 1 && ls < g->numstep && sweep < msw;
                    double acc = 0;
                    int j = 0;
                    if (live) {
                        j = (int)(r - g->row_begin);
                        const int D = g->D;
                        if (sweep & 1) {
                            const double* Ar = (ls == 1 ? g->Hc0 : g->Hc1) + (size_t)j * D;
                            for (int k = lane; k < D; k += LANES) acc += Ar[k] * g->x[k];
                        } else {
                            const float* Ar = (ls == 1 ? g->inv32_0 : g->inv32_1) + (size_t)j * D;
                            const double* v = sweep == 0 ? g->rhs : g->r;
                            float a32 = 0.f;
                            for (int k = lane; k < D; k += LANES) a32 += Ar[k] * (float)v[k];
                            acc = a32;
                        }
                    }
                    acc = group_sum<LANES>(acc);
                    if (live && lane == 0) {
                        if (sweep == 0) {
                            g->x[j] = acc;
                            if (msw == 1) update_dof(*g, ls, j, acc);
                        } else if (sweep & 1) {
                            g->r[j] = g->rhs[j] - acc;
                        } else {
                            const double xv = g->x[j] + acc;
                            g->x[j] = xv;
                            if (sweep == msw - 1) update_dof(*g, ls, j, xv);
                        }
                    }
                }
                grid.sync();
            }
        }
    }
}

template <int LANES>
cudaError_t launch_lanes(const GroupMarch* gm, int nmesh, unsigned nrows, unsigned nw,
                         unsigned nquads, unsigned nwold, int st_lo, int st_hi, int block,
                         int blocks_per_sm, bool mixed, int has_offsets, cudaStream_t s) {
    int dev = 0, nsm = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const void* fn =
        mixed ? (const void*)k_march_group_tb<LANES> : (const void*)k_march_group<LANES>;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int grid = nsm * std::min(occ, blocks_per_sm);  // every block resident: grid.sync is safe
    if (mixed) {
        void* args[] = {(void*)&gm,     (void*)&nmesh, (void*)&nrows, (void*)&nw,
                        (void*)&nquads, (void*)&nwold, (void*)&st_lo, (void*)&st_hi,
                        (void*)&has_offsets};
        return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, 0, s);
    }
    void* args[] = {(void*)&gm, (void*)&nmesh, (void*)&nrows, (void*)&nw, (void*)&st_lo,
                    (void*)&st_hi};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, 0, s);
}

}  // namespace

cudaError_t launch_march_group(const GroupMarch* gm, int nmesh, unsigned nrows, unsigned nw,
                               unsigned nquads, unsigned nwold, int st_lo, int st_hi,
                               const GroupShape& shape, bool mixed, cudaStream_t s,
                               bool has_offsets) {
    if (shape.block < 32 || shape.block > 512 || shape.block % 32 || shape.blocks_per_sm < 1)
        return cudaErrorInvalidValue;
    switch (shape.lanes) {
    case 8:
        return launch_lanes<8>(gm, nmesh, nrows, nw, nquads, nwold, st_lo, st_hi, shape.block,
                               shape.blocks_per_sm, mixed, has_offsets ? 1 : 0, s);
    case 16:
        return launch_lanes<16>(gm, nmesh, nrows, nw, nquads, nwold, st_lo, st_hi, shape.block,
                                shape.blocks_per_sm, mixed, has_offsets ? 1 : 0, s);
    case 32:
        return launch_lanes<32>(gm, nmesh, nrows, nw, nquads, nwold, st_lo, st_hi, shape.block,
                                shape.blocks_per_sm, mixed, has_offsets ? 1 : 0, s);
    default:
        return cudaErrorInvalidValue;
    }
}

}  // namespace tdbem
