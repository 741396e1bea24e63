// Mixed-precision time marching on sm_103a: FP32 level store, time-blocked
// history convolution, FP32 inverse of the column-exchanged LHS with FP64
// iterative refinement against the FP64 LHS.
//
// Time blocking.  The right-hand side of step s (SolverStepLinearT.cpp:400-482)
// is sum_f X^f w_f(s) with w_f(s) a combination of the history vectors x^m,
// m in {s+1-f, s-f, s-1-f} (and -a1 x^{s-1} on level 0).  For a block of NB steps
// s = S..S+NB-1, the part with m < S (history known when the block starts) is
// one pass over the levels with NB right-hand-side columns,
//     Y_old[:, j] = sum_f X^f W_f^old[:, j],
// so each level is read once per block instead of once per step.  The part with
// S <= m < s (history inside the block) is added by recursive halving: the block's
// first half is solved, then the first half's history enters every step of the
// second half in one multi-column pass over levels 0..n (a history step m reaches
// step s only through levels s-m-1, s-m, s-m+1), then the second half is solved.
// A block of n steps reads n log2(n) + n - 1 levels for its inner part instead of
// n (n+3)/2 step by step; the known-load terms of levels 0/1 join the old pass, and
// the leaves are plain solves.
#include <algorithm>

#include "state_update.cuh"
#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

constexpr int kRowsPerWarp = 4;
constexpr int kWarps = 8;
constexpr int kRows = kRowsPerWarp * kWarps;  // rows per block
constexpr int kKC = 256;                      // columns staged in shared memory per pass

// partial[chunk][j][row] = sum_{f in chunk} (G^f[row,:] . Wt[f][j] - H^f[row,:] . Wu[f][j])
// for NB right-hand-side columns.  Levels are FP32 with row stride ld (a multiple
// of 4, zero-padded); W is FP32 [f][j][ldw] with ldw a multiple of kKC,
// zero-padded; products and per-lane sums are FP32, the cross-lane and
// cross-chunk sums FP64.
template <int NB>
__global__ void __launch_bounds__(256) k_conv_f32(const float* __restrict__ G,
                                                  const float* __restrict__ H, size_t lstride,
                                                  int ld, int D, int f_lo, int f_hi,
                                                  int per_chunk, const float* __restrict__ Wt,
                                                  const float* __restrict__ Wu, int ldw,
                                                  int kspan, double* __restrict__ partial) {
    __shared__ float4 sw[2][NB][kKC / 4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kRows + warp * kRowsPerWarp;
    const int f0 = f_lo + blockIdx.y * per_chunk;
    const int f1 = min(f_hi, f0 + per_chunk - 1);
    float acc[kRowsPerWarp][NB];
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; r++)
#pragma unroll
        for (int j = 0; j < NB; j++) acc[r][j] = 0.f;
    size_t rowoff[kRowsPerWarp];
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; r++) rowoff[r] = (size_t)min(row0 + r, D - 1) * ld;
    for (int f = f0; f <= f1; f++) {
        const float* Gf = G + (size_t)f * lstride;
        const float* Hf = H + (size_t)f * lstride;
        const float4* wt = reinterpret_cast<const float4*>(Wt + (size_t)f * NB * ldw);
        const float4* wu = reinterpret_cast<const float4*>(Wu + (size_t)f * NB * ldw);
        const int kbeg = blockIdx.z * kspan, kend = min(ld, kbeg + kspan);
        for (int k0 = kbeg; k0 < kend; k0 += kKC) {
            __syncthreads();
            for (int i = threadIdx.x; i < NB * (kKC / 4); i += blockDim.x) {
                const int j = i / (kKC / 4), kk = i % (kKC / 4);
                sw[0][j][kk] = wt[(size_t)j * (ldw / 4) + k0 / 4 + kk];
                sw[1][j][kk] = wu[(size_t)j * (ldw / 4) + k0 / 4 + kk];
            }
            __syncthreads();
#pragma unroll 2
            for (int kk = lane; kk < kKC / 4; kk += 32) {
                const int k = k0 + 4 * kk;
                if (k >= kend) break;
                // all rows' G/H segments first, then each W column once from shared
                // memory for the 4 rows (one LDS.128 pair per column, not per row)
                float4 g[kRowsPerWarp], h[kRowsPerWarp];
#pragma unroll
                for (int r = 0; r < kRowsPerWarp; r++) {
                    g[r] = __ldcs(reinterpret_cast<const float4*>(Gf + rowoff[r] + k));
                    h[r] = __ldcs(reinterpret_cast<const float4*>(Hf + rowoff[r] + k));
                }
#pragma unroll
                for (int j = 0; j < NB; j++) {
                    const float4 a = sw[0][j][kk], b = sw[1][j][kk];
#pragma unroll
                    for (int r = 0; r < kRowsPerWarp; r++)
                        acc[r][j] += (g[r].x * a.x + g[r].y * a.y + g[r].z * a.z + g[r].w * a.w) -
                                     (h[r].x * b.x + h[r].y * b.y + h[r].z * b.z + h[r].w * b.w);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kRowsPerWarp; r++)
#pragma unroll
        for (int j = 0; j < NB; j++) {
            double v = acc[r][j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && row0 + r < D)
                partial[((size_t)(blockIdx.z * gridDim.y + blockIdx.y) * NB + j) * D + row0 + r] =
                    v;
        }
}

// W_f^old[:, j] for s = S + j: history indices 1 <= m < S, plus the known-load
// terms of levels 0/1 (c0, c1: the LHS weights of those levels, amp the step's load
// amplitude; columns j < nload).
__global__ void k_build_w_old(const double* __restrict__ u_hist,
                              const double* __restrict__ t_hist, int D, int S, int nb, int nlev,
                              double a1, double a2, double a3, BlockLoads bl, int ldw,
                              float* __restrict__ Wt, float* __restrict__ Wu) {
    const size_t total = (size_t)nlev * nb * ldw;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % ldw);
        const int j = (int)((idx / ldw) % nb);
        const int f = (int)(idx / ((size_t)ldw * nb));
        const int s = S + j;
        double wt = 0, wu = 0;
        if (k < D) {
            const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
            if (f >= 2 && m1 >= 1 && m1 < S) {
                wt += a1 * t_hist[(size_t)m1 * D + k];
                wu += a1 * u_hist[(size_t)m1 * D + k];
            }
            if (f >= 1 && m3 >= 1 && m3 < S) {
                wt += a3 * t_hist[(size_t)m3 * D + k];
                wu += a3 * u_hist[(size_t)m3 * D + k];
            }
            if (m2 >= 1 && m2 < S) {
                wt += a2 * t_hist[(size_t)m2 * D + k];
                wu += a2 * u_hist[(size_t)m2 * D + k];
            }
            if (f == 0 && s - 1 >= 1 && s - 1 < S) {
                wt -= a1 * t_hist[(size_t)(s - 1) * D + k];
                wu -= a1 * u_hist[(size_t)(s - 1) * D + k];
            }
            if (f <= 1 && j < bl.nload) {
                const double cf = f == 0 ? bl.c0[j] : bl.c1[j];
                wt += cf * (bl.amp[j] * bl.load_t[k]);
                wu += cf * bl.load_u[k];
            }
        }
        Wt[idx] = (float)wt;
        Wu[idx] = (float)wu;
    }
}

// W_f[:, j] of the history steps m in [a, b) for the steps s = b + j, j < ncol
// (columns ncol..nbp-1 zero): a1 x^m on level s+1-m (>= 2), a3 x^m on level s-m
// (>= 1), a2 x^m on level s-1-m, and -a1 x^{s-1} on level 0.
__global__ void k_build_w_cross(const double* __restrict__ u_hist,
                                const double* __restrict__ t_hist, int D, int a, int b,
                                int ncol, int nbp, int nlev, double a1, double a2, double a3,
                                int ldw, float* __restrict__ Wt, float* __restrict__ Wu) {
    const size_t total = (size_t)nlev * nbp * ldw;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % ldw);
        const int j = (int)((idx / ldw) % nbp);
        const int f = (int)(idx / ((size_t)ldw * nbp));
        const int s = b + j;
        double wt = 0, wu = 0;
        if (k < D && j < ncol) {
            const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
            if (f >= 2 && m1 >= a && m1 < b) {
                wt += a1 * t_hist[(size_t)m1 * D + k];
                wu += a1 * u_hist[(size_t)m1 * D + k];
            }
            if (f >= 1 && m3 >= a && m3 < b) {
                wt += a3 * t_hist[(size_t)m3 * D + k];
                wu += a3 * u_hist[(size_t)m3 * D + k];
            }
            if (m2 >= a && m2 < b) {
                wt += a2 * t_hist[(size_t)m2 * D + k];
                wu += a2 * u_hist[(size_t)m2 * D + k];
            }
            if (f == 0 && s - 1 >= a && s - 1 < b) {
                wt -= a1 * t_hist[(size_t)(s - 1) * D + k];
                wu -= a1 * u_hist[(size_t)(s - 1) * D + k];
            }
        }
        Wt[idx] = (float)wt;
        Wu[idx] = (float)wu;
    }
}

// out[j][row] = sum over chunks of partial[chunk][j][row] (+ add[j][row] if given),
// for the first ncol of the nb partial columns.
__global__ void k_reduce_cols(const double* __restrict__ partial, int nchunks, int nb, int ncol,
                              int D, const double* __restrict__ add, double* __restrict__ out,
                              float* __restrict__ v32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncol * D) return;
    double s = add ? add[i] : 0.0;
    for (int c = 0; c < nchunks; c++) s += partial[(size_t)c * nb * D + i];
    out[i] = s;
    if (v32 && i < D) v32[i] = (float)s;
}

// A load of the step's FP32 inverse, with an L2 evict-last policy: every step's
// solve reads the whole inverse (85 MB at D = 4614, under GB300's 129 MB L2), and
// streaming loads (evict-first) would give its lines up first.  Measured on the
// 4614-DOF march: 41.3 ms with streaming loads, 41.1 ms with these.
__device__ __forceinline__ float2 ld_keep(const float2* p, unsigned long long pol) {
    float2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                 : "=f"(v.x), "=f"(v.y)
                 : "l"(p), "l"(pol));
    return v;
}

// y = A32 v (+ y if accumulate): FP32 products, FP64 cross-lane sum; warp per
// row, pairs of columns per load when D is even.  v is FP32: converting an FP64
// vector in every row would put D^2 conversions on GB300's narrow FP64 pipe.
// A row's loads go out in batches of kGemvBatch 8-byte loads per lane, all in flight
// together: at D = 4614 (2307 pairs a row) three batches, three round trips to memory
// per warp.  128-thread blocks of at most 64 registers keep 32 warps on every SM: the
// 4614 rows' warps are resident at once.
constexpr int kGemvBatch = 26;
__global__ void __launch_bounds__(128, 8) k_gemv_f32(const float* __restrict__ A, int D,
                                                     const float* __restrict__ v,
                                                     double* __restrict__ y, int accumulate,
                                                     StateUpdate upd) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= D) return;
    const float* a = A + (size_t)row * D;
    float acc = 0.f;
    if ((D & 1) == 0) {
        const float2* a2 = reinterpret_cast<const float2*>(a);
        const float2* v2 = reinterpret_cast<const float2*>(v);
        const int n2 = D / 2;
        unsigned long long pol;
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        for (int base = lane; base < n2; base += 32 * kGemvBatch) {
            float2 x[kGemvBatch];
#pragma unroll
            for (int u = 0; u < kGemvBatch; u++) {
                const int j = base + 32 * u;
                x[u] = j < n2 ? ld_keep(a2 + j, pol) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < kGemvBatch; u++) {
                const int j = base + 32 * u;
                const float2 w = j < n2 ? v2[j] : make_float2(0.f, 0.f);
                c[u & 3] += x[u].x * w.x + x[u].y * w.y;
            }
        }
        acc = (c[0] + c[1]) + (c[2] + c[3]);
    } else {
        for (int j = lane; j < D; j += 32) acc += __ldcs(a + j) * v[j];
    }
    double s = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const double xr = accumulate ? y[row] + s : s;
        y[row] = xr;
        if (upd.u_hist) update_state_dof(upd, D, row, xr);  // the step's last product
    }
}

// r = b - A64 x, FP64, warp per row; also r in FP32 for the correction product.
__global__ void __launch_bounds__(256) k_residual_f64(const double* __restrict__ A, int D,
                                                      const double* __restrict__ x,
                                                      const double* __restrict__ b,
                                                      double* __restrict__ r,
                                                      float* __restrict__ r32) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= D) return;
    const double* a = A + (size_t)row * D;
    double acc = 0;
    for (int j = lane; j < D; j += 32) acc += __ldcs(a + j) * x[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        const double v = b[row] - acc;
        r[row] = v;
        r32[row] = (float)v;
    }
}

__global__ void k_to_f32(const double* __restrict__ v, float* __restrict__ v32, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v32[i] = (float)v[i];
}

}  // namespace

int mixed_ldw(int D) { return (D + kKC - 1) / kKC * kKC; }
int mixed_ld(int D) { return (D + 3) / 4 * 4; }

int mixed_chunks(int nlev, int D) {
    const int tiles = (D + kRows - 1) / kRows;
    const int chunks = (4 * 152 + tiles - 1) / tiles;
    return std::max(1, std::min(chunks, nlev));
}

// Column splits: enough blocks for a full wave (8 per SM) when few levels leave
// the row tiles x level chunks grid short of it; at most cap partial chunks.
int mixed_ksplit(int nchunks, int D, int cap) {
    const int tiles = (D + kRows - 1) / kRows;
    const int want = (8 * 152 + tiles * nchunks - 1) / (tiles * nchunks);
    const int ncol = (mixed_ld(D) + kKC - 1) / kKC;
    return std::max(1, std::min(std::min(want, ncol), cap / std::max(1, nchunks)));
}

cudaError_t launch_conv_f32(const float* G, const float* H, size_t lstride, int ld, int D,
                            int f_lo, int f_hi, int nb, const float* Wt, const float* Wu,
                            int ldw, double* partial, int nchunks, int ksplit, int* nparts,
                            cudaStream_t s) {
    const int nlev = f_hi - f_lo + 1;
    const int per_chunk = (nlev + nchunks - 1) / nchunks;
    // column span of a split: a multiple of the staged chunk, covering ld
    const int nkc = (ld + kKC - 1) / kKC;
    const int kspan = (nkc + ksplit - 1) / ksplit * kKC;
    dim3 grid((D + kRows - 1) / kRows, nchunks, (nkc * kKC + kspan - 1) / kspan);
    *nparts = nchunks * (int)grid.z;  // partial sums the reduction adds
    // W for level f sits at W + (f - f_lo) * nb * ldw: pass shifted base pointers
    const float* wt = Wt - (size_t)f_lo * nb * ldw;
    const float* wu = Wu - (size_t)f_lo * nb * ldw;
    switch (nb) {
    case 1: k_conv_f32<1><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 2: k_conv_f32<2><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 4: k_conv_f32<4><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 6: k_conv_f32<6><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 8: k_conv_f32<8><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 12: k_conv_f32<12><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    case 16: k_conv_f32<16><<<grid, 256, 0, s>>>(G, H, lstride, ld, D, f_lo, f_hi, per_chunk, wt, wu, ldw, kspan, partial); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_build_w_old(const double* u_hist, const double* t_hist, int D, int S, int nb,
                               int nlev, double a1, double a2, double a3, const BlockLoads& bl,
                               int ldw, float* Wt, float* Wu, cudaStream_t s) {
    const size_t total = (size_t)nlev * nb * ldw;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 8192);
    k_build_w_old<<<grid, 256, 0, s>>>(u_hist, t_hist, D, S, nb, nlev, a1, a2, a3, bl, ldw, Wt,
                                       Wu);
    return cudaGetLastError();
}

cudaError_t launch_build_w_cross(const double* u_hist, const double* t_hist, int D, int a, int b,
                                 int ncol, int nbp, int nlev, double a1, double a2, double a3,
                                 int ldw, float* Wt, float* Wu, cudaStream_t s) {
    const size_t total = (size_t)nlev * nbp * ldw;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 8192);
    k_build_w_cross<<<grid, 256, 0, s>>>(u_hist, t_hist, D, a, b, ncol, nbp, nlev, a1, a2, a3,
                                         ldw, Wt, Wu);
    return cudaGetLastError();
}

cudaError_t launch_reduce_cols(const double* partial, int nchunks, int nb, int D,
                               const double* add, double* out, cudaStream_t s) {
    k_reduce_cols<<<(nb * D + 255) / 256, 256, 0, s>>>(partial, nchunks, nb, nb, D, add, out,
                                                       nullptr);
    return cudaGetLastError();
}

cudaError_t launch_reduce_cols_n(const double* partial, int nchunks, int nb, int ncol, int D,
                                 const double* add, double* out, cudaStream_t s, float* v32) {
    k_reduce_cols<<<(ncol * D + 255) / 256, 256, 0, s>>>(partial, nchunks, nb, ncol, D, add,
                                                         out, v32);
    return cudaGetLastError();
}

// x = inv32 rhs, then n_refine times: r = rhs - A64 x; x += inv32 r.  v32 is D
// floats of scratch (the FP32 copy of the vector each product reads).
cudaError_t launch_solve_mixed(const float* inv32, const double* A64, int D, const double* rhs,
                               double* x, double* r, float* v32, int n_refine, cudaStream_t s,
                               bool v32_ready, const StateUpdate& upd) {
    const unsigned g = (D * 32 + 255) / 256, gv = (D * 32 + 127) / 128;
    const StateUpdate none;
    if (!v32_ready) k_to_f32<<<(D + 255) / 256, 256, 0, s>>>(rhs, v32, D);
    k_gemv_f32<<<gv, 128, 0, s>>>(inv32, D, v32, x, 0, n_refine == 0 ? upd : none);
    for (int it = 0; it < n_refine; it++) {
        k_residual_f64<<<g, 256, 0, s>>>(A64, D, x, rhs, r, v32);
        k_gemv_f32<<<gv, 128, 0, s>>>(inv32, D, v32, x, 1, it == n_refine - 1 ? upd : none);
    }
    return cudaGetLastError();
}

}  // namespace tdbem
