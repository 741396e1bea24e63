// Persistent marching of many meshes: every step of every mesh in one
// cooperative launch.
//
// Each mesh is a plain FP64 solve (SolverStepLinearT::Solve_Averaging,
// SolverStepLinearT.cpp:314-544, as march.cu's per-step kernels).  Per step the
// grid runs three phases separated by grid-wide barriers:
//   A  combined history vectors W_f of every mesh (march.cu: k_history_combine);
//   B  rhs = sum_f (G^f W_t[f] - H^f W_u[f]): one group of LANES lanes per row
//      of every mesh, FP64 partial sums per lane, fixed-order shuffle reduction;
//   C  x = inv(LHS) rhs with the mesh's FP64 inverse, one lane group per row,
//      and the state update of that dof (march.cu: k_update_state).
// Meshes with fewer steps idle once done.  Small meshes (a few hundred DOF)
// would otherwise spend their time in launch latency: five launches per step
// per mesh become three barriers per step for all of them.  The lane count per
// row and the launch shape are picked by timing (capi.cu: the group autotuner).
#include <cooperative_groups.h>

#include <algorithm>

#include "tdbem_internal.cuh"

namespace cg = cooperative_groups;

namespace tdbem {

namespace {

__device__ __forceinline__ int mesh_of_row(const GroupMarch* __restrict__ gm, int nmesh,
                                           unsigned x, bool by_w) {
    int lo = 0, hi = nmesh - 1;  // last mesh whose first row / W entry is <= x
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const unsigned b = by_w ? gm[mid].w_begin : gm[mid].row_begin;
        if (b <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int LANES>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, LANES);
    return v;
}

template <int LANES>
__global__ void __launch_bounds__(512) k_march_group(const GroupMarch* __restrict__ gm, int nmesh,
                                                     unsigned nrows, unsigned nw, int st_lo,
                                                     int st_hi) {
    cg::grid_group grid = cg::this_grid();
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned lane = threadIdx.x % LANES;
    const unsigned ngroups = nthreads / LANES;
    // the warp's first lane group and this lane's group within the warp
    const unsigned warp_group0 = (tid / 32) * (32 / LANES);
    const unsigned sub = (threadIdx.x % 32) / LANES;
    for (int st = st_lo; st < st_hi; st++) {
        // ---- A: combined history vectors (levels f <= L of each mesh)
        for (unsigned idx = tid; idx < nw; idx += nthreads) {
            const GroupMarch& g = gm[mesh_of_row(gm, nmesh, idx, true)];
            if (st >= g.numstep) continue;
            const unsigned loc = idx - g.w_begin;
            const int f = (int)(loc / g.D), j = (int)(loc % g.D);
            const int L = min(max(st, 1), g.M);
            if (f > L) continue;
            const double c0 = st == 1 ? 1.0 : g.c0, c1 = st == 1 ? 0.0 : g.c1;
            const double amp = g.amp ? g.amp[st] : 1.0;
            const double* uh = g.u;
            const double* th = g.t;
            const int D = g.D;
            double wt = 0, wu = 0;
            const int m1 = st + 1 - f, m3 = st - f, m2 = st - 1 - f;
            if (f >= 2 && m1 >= 1) {
                wt += g.a1 * th[(size_t)m1 * D + j];
                wu += g.a1 * uh[(size_t)m1 * D + j];
            }
            if (f >= 1 && m3 >= 1) {
                wt += g.a3 * th[(size_t)m3 * D + j];
                wu += g.a3 * uh[(size_t)m3 * D + j];
            }
            if (m2 >= 1) {
                wt += g.a2 * th[(size_t)m2 * D + j];
                wu += g.a2 * uh[(size_t)m2 * D + j];
            }
            if (f == 0) {
                if (st - 1 >= 1) {
                    wt -= g.a1 * th[(size_t)(st - 1) * D + j];
                    wu -= g.a1 * uh[(size_t)(st - 1) * D + j];
                }
                wt += c0 * (amp * g.load_t[j]);
                wu += c0 * g.load_u[j];
            } else if (f == 1) {
                wt += c1 * (amp * g.load_t[j]);
                wu += c1 * g.load_u[j];
            }
            g.Wt[loc] = wt;
            g.Wu[loc] = wu;
        }
        grid.sync();
        // ---- B: history convolution, one lane group per row.  The row loop is
        // uniform across each warp (stepped by the warp's first group) and every
        // lane joins the shuffle reduction, also for rows past the end or of a
        // finished mesh, which contribute zero.
        for (unsigned base = warp_group0; base < nrows; base += ngroups) {
            const unsigned r = base + sub;
            const GroupMarch* g = r < nrows ? &gm[mesh_of_row(gm, nmesh, r, false)] : nullptr;
            const bool live = g && st < g->numstep;
            double acc = 0;
            if (live) {
                const int row = (int)(r - g->row_begin), D = g->D;
                const int L = min(max(st, 1), g->M);
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
            const GroupMarch* g = r < nrows ? &gm[mesh_of_row(gm, nmesh, r, false)] : nullptr;
            const bool live = g && st < g->numstep;
            double acc = 0;
            int j = 0;
            if (live) {
                j = (int)(r - g->row_begin);
                const int D = g->D;
                const double* Ar = (st == 1 ? g->Ainv0 : g->Ainv1) + (size_t)j * D;
                for (int k = lane; k < D; k += LANES) acc += Ar[k] * g->rhs[k];
            }
            acc = group_sum<LANES>(acc);
            if (live && lane == 0) {
                const int D = g->D;
                const double amp = g->amp ? g->amp[st] : 1.0;
                const bool u = g->is_u[j] != 0, f = g->is_f[j] != 0;
                g->u[(size_t)st * D + j] = u ? g->ubc[j] : acc;
                double tv = f ? g->fbc[j] * amp : 0.0;
                if (u && j < D - 1) tv = acc;
                g->t[(size_t)st * D + j] = tv;
            }
        }
        grid.sync();
    }
}

template <int LANES>
cudaError_t launch_lanes(const GroupMarch* gm, int nmesh, unsigned nrows, unsigned nw, int st_lo,
                         int st_hi, int block, int blocks_per_sm, cudaStream_t s) {
    int dev = 0, nsm = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_march_group<LANES>, block, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int grid = nsm * std::min(occ, blocks_per_sm);  // every block resident: grid.sync is safe
    void* args[] = {(void*)&gm, (void*)&nmesh, (void*)&nrows, (void*)&nw, (void*)&st_lo,
                    (void*)&st_hi};
    return cudaLaunchCooperativeKernel((const void*)k_march_group<LANES>, dim3(grid), dim3(block),
                                       args, 0, s);
}

}  // namespace

cudaError_t launch_march_group(const GroupMarch* gm, int nmesh, unsigned nrows, unsigned nw,
                               int st_lo, int st_hi, const GroupShape& shape, cudaStream_t s) {
    if (shape.block < 32 || shape.block > 512 || shape.block % 32 || shape.blocks_per_sm < 1)
        return cudaErrorInvalidValue;
    switch (shape.lanes) {
    case 8: return launch_lanes<8>(gm, nmesh, nrows, nw, st_lo, st_hi, shape.block,
                                   shape.blocks_per_sm, s);
    case 16: return launch_lanes<16>(gm, nmesh, nrows, nw, st_lo, st_hi, shape.block,
                                     shape.blocks_per_sm, s);
    case 32: return launch_lanes<32>(gm, nmesh, nrows, nw, st_lo, st_hi, shape.block,
                                     shape.blocks_per_sm, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tdbem
