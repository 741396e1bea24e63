// Blocked in-place Gauss-Jordan inversion with partial pivoting (FP32 / FP64).
// The pivot search of each panel runs in one thread-block cluster with the panel in
// distributed shared memory (k_panel_pivots_cluster) when the panel fits in 16
// CTAs' shared memory, else on a cooperative grid (k_panel_pivots).
//
// Replaces KSPSolve's factorisation (SolverStepLinearT.cpp:503-504) by an
// explicit inverse of the column-exchanged LHS, computed once per distinct LHS.
// Panel step for columns C1 = [k0, k0+bw):
//   1. LU with partial pivoting of the tall panel A[k0:, C1] (one block; pivots
//      are searched among rows >= the current column, as unblocked GJE does);
//   2. the panel's row swaps applied to all columns;
//   3. Ainv11 = A11^-1 from the panel's L11 U11;
//   4. T12 = Ainv11 A[R1, :]            (R1 = the bw pivot rows);
//   5. A[i, j] -= A[i, C1] T12[:, j]     for rows i not in R1, columns j not in C1;
//   6. A[R1, j] = T12[:, j] (j not in C1), A[R1, C1] = Ainv11,
//      A[i, C1] = -A[i, C1] Ainv11       for rows i not in R1.
// After the last panel the columns are permuted back (reverse order of the
// row swaps).  Step 5 is a rank-bw update with bw-deep dot products, so the
// whole inversion is 2 n^3 flops in GEMM form.  With a cuBLAS handle (the FP32
// inverse) step 5 is two plain GEMMs over the columns left and right of C1 and
// every row: rows R1 are rewritten by step 6 whatever step 5 leaves there, and
// step 6 reads only columns C1, which the GEMMs do not write.
//
// The FP32 inverse (a preconditioner that FP64 refinement corrects) may restrict
// step 1's search to the panel's diagonal block (k_block_pivots, one CTA: no
// cluster-wide reduction per column).  On the boundary-element LHS the column
// maximum lies in that block (diagonal dominance), so the pivots are the same; a
// zero pivot in the block, or a probe ||A (X v) - v|| / ||v|| above 1e-2 of the
// finished inverse, sends the inversion back to the full search.
#include <cooperative_groups.h>
#include <cublas_v2.h>

#include <algorithm>
#include <cstring>
#include <condition_variable>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

template <typename T>
__device__ __forceinline__ T absv(T x) { return x < T(0) ? -x : x; }

// Pivot sequence of the panel: LU with partial pivoting of rows k0..n-1 of
// columns C1, spread over a cooperative grid (all blocks co-resident, so the
// grid barrier always completes).  Each block keeps `rpb` panel rows in shared
// memory.  Per column, each block publishes its best candidate together with
// that candidate's row (and the owner of row c publishes row c); after one grid
// barrier every block picks the same pivot (largest magnitude, lowest row on
// ties), swaps, and updates its own rows.  Publications alternate between two
// buffers by column parity, so a fast block never overwrites what a slow block
// still reads.
template <typename T, int BW>
__global__ void __launch_bounds__(256) k_panel_pivots(const T* __restrict__ A, int n, int k0,
                                                      int bw, int rpb, int* __restrict__ perm,
                                                      int* __restrict__ status,
                                                      T* __restrict__ gval,
                                                      int* __restrict__ gidx,
                                                      T* __restrict__ grows) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    extern __shared__ unsigned char smem_raw[];
    T* ws = reinterpret_cast<T*>(smem_raw);  // rpb x BW
    __shared__ T sv[256];
    __shared__ int si[256];
    __shared__ T su[BW];
    __shared__ int s_p, s_b;
    const int nb = gridDim.x;
    const int rows = n - k0;
    const int r0 = blockIdx.x * rpb, r1 = min(rows, r0 + rpb);
    for (int idx = threadIdx.x; idx < rpb * BW; idx += blockDim.x) {
        const int r = idx / BW, c = idx % BW;
        ws[idx] = (r0 + r < r1 && c < bw) ? A[(size_t)(k0 + r0 + r) * n + k0 + c] : T(0);
    }
    __syncthreads();
    for (int c = 0; c < bw; c++) {
        const int par = c & 1;
        T* cval = gval + par * nb;
        int* cidx = gidx + par * nb;
        T* crows = grows + (size_t)par * (nb + 1) * BW;  // nb candidate rows, then row c
        T best = T(-1);
        int bi = rows;
        for (int r = max(r0, c) + threadIdx.x; r < r1; r += blockDim.x) {
            const T v = absv(ws[(r - r0) * BW + c]);
            if (v > best) { best = v; bi = r; }
        }
        sv[threadIdx.x] = best;
        si[threadIdx.x] = bi;
        __syncthreads();
        for (int st = blockDim.x / 2; st > 0; st >>= 1) {
            if (threadIdx.x < st) {
                const T v2 = sv[threadIdx.x + st];
                const int i2 = si[threadIdx.x + st];
                if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
                    sv[threadIdx.x] = v2;
                    si[threadIdx.x] = i2;
                }
            }
            __syncthreads();
        }
        const int li = si[0];
        if (threadIdx.x == 0) {
            cval[blockIdx.x] = sv[0];
            cidx[blockIdx.x] = li;
        }
        if (threadIdx.x < BW) {
            if (li < r1) crows[(size_t)blockIdx.x * BW + threadIdx.x] = ws[(li - r0) * BW + threadIdx.x];
            if (c >= r0 && c < r1) crows[(size_t)nb * BW + threadIdx.x] = ws[(c - r0) * BW + threadIdx.x];
        }
        grid.sync();
        if (threadIdx.x == 0) {  // every block reduces the same list in the same order
            T bv = T(-1);
            int bp = rows, bb = 0;
            for (int b = 0; b < nb; b++) {
                const T v = cval[b];
                const int i = cidx[b];
                if (v > bv || (v == bv && i < bp)) { bv = v; bp = i; bb = b; }
            }
            s_p = (bp < rows && bv != T(0)) ? bp : -1;
            s_b = bb;
        }
        __syncthreads();
        const int p = s_p;
        if (p < 0) {  // zero pivot: every block sees it and leaves
            if (blockIdx.x == 0 && threadIdx.x == 0) *status = 1;
            return;
        }
        if (threadIdx.x < BW) {
            const T pv = crows[(size_t)s_b * BW + threadIdx.x];  // the pivot row
            su[threadIdx.x] = pv;
            if (c >= r0 && c < r1) ws[(c - r0) * BW + threadIdx.x] = pv;
            if (p != c && p >= r0 && p < r1)
                ws[(p - r0) * BW + threadIdx.x] = crows[(size_t)nb * BW + threadIdx.x];
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) perm[k0 + c] = k0 + p;
        __syncthreads();
        const T inv = T(1) / su[c];
        for (int r = max(r0, c + 1) + threadIdx.x; r < r1; r += blockDim.x) {
            T* wr = ws + (r - r0) * BW;
            const T l = wr[c] * inv;
            wr[c] = l;
            for (int j = c + 1; j < bw; j++) wr[j] -= l * su[j];
        }
        __syncthreads();
    }
}

// The same pivot sequence with the panel held in the distributed shared memory of
// one thread-block cluster (CS CTAs): per column every CTA publishes its best
// candidate (value, row, the row's panel entries) and, if it owns it, row c in
// its own shared memory; after a hardware cluster barrier every CTA reads all
// CTAs' candidates through DSMEM and picks the same pivot as k_panel_pivots.
// Publications alternate between two slots by column parity: a CTA can only
// reuse a slot after the next column's barrier, which every reader passes only
// once it has finished reading.  A final barrier keeps every CTA's shared memory
// alive until no other CTA can read it.
template <typename T, int BW>
__global__ void __launch_bounds__(1024) k_panel_pivots_cluster(const T* __restrict__ A, int n,
                                                               int k0, int bw, int rpb,
                                                               int* __restrict__ perm,
                                                               int* __restrict__ status) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ unsigned char smem_raw[];
    T* ws = reinterpret_cast<T*>(smem_raw);  // rpb x BW
    __shared__ T wv[32];
    __shared__ int wi[32];
    __shared__ T su[BW];
    __shared__ T cand_val[2];
    __shared__ int cand_idx[2];
    __shared__ T cand_row[2][BW];
    __shared__ T row_c[2][BW];
    __shared__ int s_p, s_b;
    const int nb = (int)cluster.num_blocks();
    const int me = (int)cluster.block_rank();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int rows = n - k0;
    const int r0 = me * rpb, r1 = min(rows, r0 + rpb);
    for (int idx = threadIdx.x; idx < rpb * BW; idx += blockDim.x) {
        const int r = idx / BW, c = idx % BW;
        ws[idx] = (r0 + r < r1 && c < bw) ? A[(size_t)(k0 + r0 + r) * n + k0 + c] : T(0);
    }
    __syncthreads();
    // (value, row): larger value wins, then the lower row
    auto better = [](T v2, int i2, T v, int i) { return v2 > v || (v2 == v && i2 < i); };
    for (int c = 0; c < bw; c++) {
        const int par = c & 1;
        // ---- this CTA's candidate: thread, warp, then block arg-max
        T best = T(-1);
        int bi = rows;
        for (int r = max(r0, c) + threadIdx.x; r < r1; r += blockDim.x) {
            const T v = absv(ws[(r - r0) * BW + c]);
            if (better(v, r, best, bi)) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const T v2 = __shfl_xor_sync(0xffffffffu, best, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
            if (better(v2, i2, best, bi)) { best = v2; bi = i2; }
        }
        if (lane == 0) {
            wv[warp] = best;
            wi[warp] = bi;
        }
        __syncthreads();
        if (warp == 0) {
            best = lane < nwarp ? wv[lane] : T(-1);
            bi = lane < nwarp ? wi[lane] : rows;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T v2 = __shfl_xor_sync(0xffffffffu, best, o);
                const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
                if (better(v2, i2, best, bi)) { best = v2; bi = i2; }
            }
            if (lane == 0) {
                cand_val[par] = best;
                cand_idx[par] = bi;
            }
            // the candidate row (and row c, if this CTA owns it) for the other CTAs
            for (int t = lane; t < BW; t += 32) {
                if (bi < r1) cand_row[par][t] = ws[(bi - r0) * BW + t];
                if (c >= r0 && c < r1) row_c[par][t] = ws[(c - r0) * BW + t];
            }
        }
        cluster.sync();
        if (warp == 0) {  // one lane per CTA reads its candidate; the same arg-max in every CTA
            T bv = T(-1);
            int bp = rows, bb = lane;
            if (lane < nb) {
                bv = *cluster.map_shared_rank(&cand_val[par], lane);
                bp = *cluster.map_shared_rank(&cand_idx[par], lane);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T v2 = __shfl_xor_sync(0xffffffffu, bv, o);
                const int i2 = __shfl_xor_sync(0xffffffffu, bp, o);
                const int b2 = __shfl_xor_sync(0xffffffffu, bb, o);
                if (better(v2, i2, bv, bp)) { bv = v2; bp = i2; bb = b2; }
            }
            if (lane == 0) {
                s_p = (bp < rows && bv != T(0)) ? bp : -1;
                s_b = bb;
            }
        }
        __syncthreads();
        const int p = s_p;
        if (p < 0) {  // zero pivot: every CTA sees it; leave together
            if (me == 0 && threadIdx.x == 0) *status = 1;
            cluster.sync();
            return;
        }
        if (threadIdx.x < BW) {
            const T pv = cluster.map_shared_rank(&cand_row[par][0], s_b)[threadIdx.x];
            su[threadIdx.x] = pv;
            if (c >= r0 && c < r1) ws[(c - r0) * BW + threadIdx.x] = pv;
            if (p != c && p >= r0 && p < r1)
                ws[(p - r0) * BW + threadIdx.x] =
                    cluster.map_shared_rank(&row_c[par][0], c / rpb)[threadIdx.x];
        }
        if (me == 0 && threadIdx.x == 0) perm[k0 + c] = k0 + p;
        __syncthreads();
        // ---- eliminate below row c: multipliers, then the (row, column) updates
        const T inv = T(1) / su[c];
        const int rb = max(r0, c + 1);
        for (int r = rb + threadIdx.x; r < r1; r += blockDim.x) ws[(r - r0) * BW + c] *= inv;
        __syncthreads();
        const int w = bw - c - 1;
        if (w > 0) {
            const int cnt = (r1 > rb) ? (r1 - rb) * w : 0;
            for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                const int r = rb + idx / w, j = c + 1 + idx % w;
                T* wr = ws + (r - r0) * BW;
                wr[j] -= wr[c] * su[j];
            }
        }
        __syncthreads();
    }
    cluster.sync();
}

// Row swaps of the panel applied to every column, in pivot order.
template <typename T>
__global__ void k_apply_swaps(T* __restrict__ A, int n, int k0, int bw,
                              const int* __restrict__ perm, const int* __restrict__ status) {
    if (*status) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int c = 0; c < bw; c++) {
        const int p = perm[k0 + c];
        if (p != k0 + c) {
            const T t = A[(size_t)(k0 + c) * n + j];
            A[(size_t)(k0 + c) * n + j] = A[(size_t)p * n + j];
            A[(size_t)p * n + j] = t;
        }
    }
}

// Ainv11 = A11^-1 for the swapped pivot block A[R1, C1]: Gauss-Jordan without
// further pivoting in shared memory (A11 = L11 U11 with the panel's pivots, so
// its pivots are U11's diagonal).  Entries beyond a narrow last panel are zero.
template <typename T, int BW>
__global__ void __launch_bounds__(1024) k_panel_inv(const T* __restrict__ A, int n, int k0,
                                                    int bw, T* __restrict__ Ainv,
                                                    const int* __restrict__ status) {
    if (*status) return;
    __shared__ T m[BW][BW + 1];
    __shared__ T col[BW], row[BW];
    for (int idx = threadIdx.x; idx < BW * BW; idx += blockDim.x) {
        const int i = idx / BW, j = idx % BW;
        m[i][j] = (i < bw && j < bw) ? A[(size_t)(k0 + i) * n + k0 + j] : T(i == j ? 1 : 0);
    }
    __syncthreads();
    for (int c = 0; c < bw; c++) {
        const T inv = T(1) / m[c][c];
        if (threadIdx.x < BW) {
            col[threadIdx.x] = m[threadIdx.x][c];
            row[threadIdx.x] = (threadIdx.x == c ? T(1) : m[c][threadIdx.x]) * inv;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < BW * BW; idx += blockDim.x) {
            const int i = idx / BW, j = idx % BW;
            if (i == c) m[i][j] = row[j];
            else m[i][j] = (j == c ? T(0) : m[i][j]) - col[i] * row[j];
        }
        __syncthreads();
    }
    for (int idx = threadIdx.x; idx < BW * BW; idx += blockDim.x) {
        const int i = idx / BW, j = idx % BW;
        Ainv[idx] = (i < bw && j < bw) ? m[i][j] : T(0);
    }
}

// T12[c][j] = sum_d Ainv11[c][d] A[k0+d][j] for every column j.
template <typename T, int BW>
__global__ void __launch_bounds__(256) k_panel_t12(const T* __restrict__ A, int n, int k0,
                                                   int bw, const T* __restrict__ Ainv,
                                                   T* __restrict__ T12,
                                                   const int* __restrict__ status) {
    if (*status) return;
    __shared__ T sa[BW * BW];
    for (int i = threadIdx.x; i < BW * BW; i += blockDim.x) sa[i] = Ainv[i];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    T a[BW];
#pragma unroll
    for (int d = 0; d < BW; d++) a[d] = d < bw ? A[(size_t)(k0 + d) * n + j] : T(0);
    for (int c = 0; c < bw; c++) {
        T s = T(0);
#pragma unroll
        for (int d = 0; d < BW; d++) s += sa[c * BW + d] * a[d];
        T12[(size_t)c * n + j] = s;
    }
}

// A[i][j] -= sum_c A[i][k0+c] T12[c][j] for i not in R1, j not in C1.  64 x 64 tiles.
template <typename T, int BW>
__global__ void __launch_bounds__(256) k_panel_update(T* __restrict__ A, int n, int k0, int bw,
                                                      const T* __restrict__ T12,
                                                      const int* __restrict__ status) {
    if (*status) return;
    constexpr int TS = 64;
    __shared__ T sp[TS][BW + 1];
    __shared__ T st[BW][TS];
    const int i0 = blockIdx.y * TS, j0 = blockIdx.x * TS;
    for (int idx = threadIdx.x; idx < TS * BW; idx += blockDim.x) {
        const int r = idx / BW, c = idx % BW;
        const int i = i0 + r;
        sp[r][c] = (i < n && c < bw) ? A[(size_t)i * n + k0 + c] : T(0);
    }
    for (int idx = threadIdx.x; idx < TS * BW; idx += blockDim.x) {
        const int c = idx / TS, q = idx % TS;
        const int j = j0 + q;
        st[c][q] = (j < n && c < bw) ? T12[(size_t)c * n + j] : T(0);
    }
    __syncthreads();
    const int tr = (threadIdx.x / 16) * 4, tc = (threadIdx.x % 16) * 4;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = T(0);
#pragma unroll 8
    for (int c = 0; c < BW; c++) {
        T pa[4], tb[4];
#pragma unroll
        for (int a = 0; a < 4; a++) pa[a] = sp[tr + a][c];
#pragma unroll
        for (int b = 0; b < 4; b++) tb[b] = st[c][tc + b];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] += pa[a] * tb[b];
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int i = i0 + tr + a;
        if (i >= n || (i >= k0 && i < k0 + bw)) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int j = j0 + tc + b;
            if (j >= n || (j >= k0 && j < k0 + bw)) continue;
            A[(size_t)i * n + j] -= acc[a][b];
        }
    }
}

// Rows R1 <- [T12 | Ainv11]; other rows' C1 block <- -A[i, C1] Ainv11.
template <typename T, int BW>
__global__ void __launch_bounds__(256) k_panel_finish(T* __restrict__ A, int n, int k0, int bw,
                                                      const T* __restrict__ T12,
                                                      const T* __restrict__ Ainv,
                                                      const int* __restrict__ status) {
    if (*status) return;
    __shared__ T sa[BW * BW];
    for (int i = threadIdx.x; i < BW * BW; i += blockDim.x) sa[i] = Ainv[i];
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {  // row t, columns C1
        const int i = t;
        if (i >= k0 && i < k0 + bw) {
            for (int d = 0; d < bw; d++) A[(size_t)i * n + k0 + d] = sa[(i - k0) * BW + d];
        } else {
            T a[BW];
#pragma unroll
            for (int c = 0; c < BW; c++) a[c] = c < bw ? A[(size_t)i * n + k0 + c] : T(0);
            for (int d = 0; d < bw; d++) {
                T s = T(0);
#pragma unroll
                for (int c = 0; c < BW; c++) s += a[c] * sa[c * BW + d];
                A[(size_t)i * n + k0 + d] = -s;
            }
        }
    }
    // rows R1, columns outside C1 (a grid-stride pass over bw x n)
    for (size_t idx = t; idx < (size_t)bw * n; idx += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(idx / n), j = (int)(idx % n);
        if (j >= k0 && j < k0 + bw) continue;
        A[(size_t)(k0 + c) * n + j] = T12[(size_t)c * n + j];
    }
}

template <typename T>
__global__ void k_permute_cols_t(T* __restrict__ A, int n, const int* __restrict__ cols,
                                 T* __restrict__ tmp) {
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        T* row = A + (size_t)i * n;
        T* t = tmp + (size_t)blockIdx.x * n;
        for (int j = threadIdx.x; j < n; j += blockDim.x) t[j] = row[cols[j]];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) row[j] = t[j];
        __syncthreads();
    }
}

// Pivot sequence of the panel with the search restricted to its diagonal block:
// LU with partial pivoting (largest magnitude, lowest row on ties) of the bw x bw
// block A[k0:k0+bw, k0:k0+bw] in shared memory, one CTA.  Writes perm[k0 + c] as
// the tall-panel kernels do; a zero pivot sets *status = 2 (the caller retries
// with the full search).
template <typename T, int BW>
__global__ void __launch_bounds__(256) k_block_pivots(const T* __restrict__ A, int n, int k0,
                                                      int bw, int* __restrict__ perm,
                                                      int* __restrict__ status) {
    __shared__ T ws[BW][BW + 1];
    __shared__ int s_p;
    for (int idx = threadIdx.x; idx < BW * BW; idx += blockDim.x) {
        const int r = idx / BW, c = idx % BW;
        ws[r][c] = (r < bw && c < bw) ? A[(size_t)(k0 + r) * n + k0 + c] : T(0);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int c = 0; c < bw; c++) {
        if (threadIdx.x < 32) {  // warp 0: argmax of |ws[r][c]|, r in [c, bw)
            T best = T(-1);
            int bi = bw;
            for (int r = c + lane; r < bw; r += 32) {
                const T v = absv(ws[r][c]);
                if (v > best) { best = v; bi = r; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T v2 = __shfl_xor_sync(0xffffffffu, best, o);
                const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
                if (v2 > best || (v2 == best && i2 < bi)) { best = v2; bi = i2; }
            }
            if (lane == 0) s_p = (bi < bw && best != T(0)) ? bi : -1;
        }
        __syncthreads();
        const int p = s_p;
        if (p < 0) {
            if (threadIdx.x == 0) *status = 2;
            return;
        }
        if (p != c)
            for (int j = threadIdx.x; j < BW; j += blockDim.x) {
                const T t = ws[c][j];
                ws[c][j] = ws[p][j];
                ws[p][j] = t;
            }
        if (threadIdx.x == 0) perm[k0 + c] = k0 + p;
        __syncthreads();
        const T inv = T(1) / ws[c][c];
        const int nr = bw - c - 1, nc = bw - c;  // rows c+1.., columns c.. (column c -> l)
        for (int idx = threadIdx.x; idx < nr * nc; idx += blockDim.x) {
            const int r = c + 1 + idx / nc, j = c + idx % nc;
            const T l = ws[r][c] * inv;
            if (j > c) ws[r][j] -= l * ws[c][j];
        }
        __syncthreads();
        for (int r = c + 1 + threadIdx.x; r < bw; r += blockDim.x) ws[r][c] *= inv;
        __syncthreads();
    }
}

// Probe of an FP32 inverse X of A64: y = X v, then err = max_i |(A64 y)_i - v_i|
// (v_i = (i mod 13) - 6.5, max |v| = 6.5), as the float bits of a non-negative
// value (integer max preserves the order).  Warp per row.
__device__ __forceinline__ double probe_v(int i) { return (double)(i % 13) - 6.5; }

__global__ void __launch_bounds__(256) k_probe_xv(const float* __restrict__ X, int n,
                                                  double* __restrict__ y) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    const float* row = X + (size_t)w * n;
    double acc = 0;
    for (int j = lane; j < n; j += 32) acc += (double)row[j] * probe_v(j);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[w] = acc;
}

__global__ void __launch_bounds__(256) k_probe_ay(const double* __restrict__ A, int n,
                                                  const double* __restrict__ y,
                                                  unsigned* __restrict__ err_bits) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    const double* row = A + (size_t)w * n;
    double acc = 0;
    for (int j = lane; j < n; j += 32) acc += row[j] * y[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        const float e = (float)fabs(acc - probe_v(w));
        atomicMax(err_bits, __float_as_uint(e == e ? e : 3.0e38f));  // NaN counts as huge
    }
}

__global__ void k_cast_f64_f32(const double* __restrict__ a, float* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

constexpr size_t kClusterPanelBytes = 200 * 1024;  // panel rows per CTA of a cluster

// Whether a cluster of cs CTAs of the pivot kernel can be resident on this device
// (checked once per size; 16 needs the non-portable cluster size).
bool cluster_probe(int cs) {
    const void* fn8 = (const void*)k_panel_pivots_cluster<float, 64>;
    const void* fn16 = (const void*)k_panel_pivots_cluster<double, 16>;
    for (const void* fn : {fn8, fn16}) {
        if (cs == 16 &&
            cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess)
            return false;
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kClusterPanelBytes) != cudaSuccess)
            return false;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = kClusterPanelBytes;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            return false;
        }
    }
    return true;
}

// Both sizes probed once, before any caller sees an answer (host threads invert
// concurrently: a half-made answer would send one of them to another kernel).
bool cluster_ok(int cs) {
    static const bool ok8 = cluster_probe(8);
    static const bool ok16 = cluster_probe(16);
    return cs == 16 ? ok16 : ok8;
}

// The pivot kernels' dynamic shared-memory limit, raised once per kernel to the
// largest panel any call uses (a per-call setting would race between host threads
// inverting at the same time: one could lower the limit under another's launch).
template <typename T, int BW>
cudaError_t pivot_attributes() {
    static const cudaError_t e = [] {
        cudaError_t r = cudaFuncSetAttribute((const void*)k_panel_pivots<T, BW>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kClusterPanelBytes);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute((const void*)k_panel_pivots_cluster<T, BW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kClusterPanelBytes);
        return r;
    }();
    return e;
}

// FP32 GEMM on the tensor cores with FP32 accuracy (each input as three BF16
// terms), where this cuBLAS offers it.
cublasComputeType_t blas_compute() { return CUBLAS_COMPUTE_32F_EMULATED_16BFX9; }

template <typename T, int BW>
cudaError_t invert_blocked(T* A, int n, int* perm, int* d_status, T* scratch, long long* nlaunch,
                           bool* singular, cudaStream_t s, bool restricted = false,
                           void* blas = nullptr) {
    *singular = false;
    {
        const cudaError_t ea = pivot_attributes<T, BW>();
        if (ea != cudaSuccess) return ea;
    }
    T* W = scratch;                          // 2*BW*n: permutation scratch rows at the end
    T* T12 = W + (size_t)n * BW;             // BW x n
    T* Ainv = T12 + (size_t)n * BW;          // BW x BW
    T* gval = Ainv + BW * BW;                // per-block pivot candidates, 2 buffers
    T* grows = gval + 2 * kMaxPivotBlocks;   // candidate rows + row c, 2 buffers
    int* gidx = perm + n;                    // perm has n + 2*kMaxPivotBlocks ints
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const dim3 ugrid((n + 63) / 64, (n + 63) / 64);
    for (int k0 = 0; k0 < n; k0 += BW) {
        const int bw = std::min(BW, n - k0);
        const int rows = n - k0;
        const int nblk = std::max(1, std::min(kMaxPivotBlocks, (rows + 63) / 64));
        int rpb = (rows + nblk - 1) / nblk;
        size_t smem = (size_t)rpb * BW * sizeof(T);
        if (smem > kClusterPanelBytes) return cudaErrorInvalidConfiguration;  // panel too tall
        int kk0 = k0, kbw = bw, kn = n;
        const T* cA = A;
        bool done = false;
        if (restricted) {
            k_block_pivots<T, BW><<<1, 256, 0, s>>>(A, n, k0, bw, perm, d_status);
            done = true;
        }
        // the panel in one cluster's distributed shared memory when it fits
        for (int cs : {16, 8}) {
            if (done) break;
            const int crpb = (rows + cs - 1) / cs;
            const size_t csmem = (size_t)crpb * BW * sizeof(T);
            if (csmem > kClusterPanelBytes || !cluster_ok(cs)) continue;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(1024);
            cfg.dynamicSmemBytes = csmem;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = cs;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            e = cudaLaunchKernelEx(&cfg, k_panel_pivots_cluster<T, BW>, cA, kn, kk0, kbw, crpb,
                                   perm, d_status);
            if (e != cudaSuccess) return e;
            done = true;
            break;
        }
        if (!done) {
            void* args[] = {&cA, &kn, &kk0, &kbw, &rpb, &perm, &d_status, &gval, &gidx, &grows};
            e = cudaLaunchCooperativeKernel((const void*)k_panel_pivots<T, BW>, dim3(nblk),
                                            dim3(256), args, smem, s);
            if (e != cudaSuccess) return e;
        }
        k_apply_swaps<T><<<(n + 255) / 256, 256, 0, s>>>(A, n, k0, bw, perm, d_status);
        k_panel_inv<T, BW><<<1, 1024, 0, s>>>(A, n, k0, bw, Ainv, d_status);
        k_panel_t12<T, BW><<<(n + 255) / 256, 256, 0, s>>>(A, n, k0, bw, Ainv, T12, d_status);
        bool updated = false;
        if constexpr (std::is_same<T, float>::value) {
            if (blas) {  // A[:, J] -= A[:, C1] T12[:, J] for J left and right of C1
                cublasHandle_t h = static_cast<cublasHandle_t>(blas);
                if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
                const float alpha = -1.f, beta = 1.f;
                const int spans[2][2] = {{0, k0}, {k0 + bw, n - k0 - bw}};
                for (const auto& sp : spans) {
                    if (sp[1] <= 0) continue;
                    // column-major views of the row-major arrays: C^T -= T12_J^T A_C1^T;
                    // plain FP32 where the emulated form does not take the shape
                    // (rows of an odd n are not 16-byte aligned)
                    auto gemm = [&](cublasComputeType_t ct) {
                        return cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, sp[1], n, bw, &alpha,
                                            T12 + sp[0], CUDA_R_32F, n, A + k0, CUDA_R_32F, n,
                                            &beta, A + sp[0], CUDA_R_32F, n, ct,
                                            CUBLAS_GEMM_DEFAULT);
                    };
                    cublasStatus_t st = gemm(blas_compute());
                    if (st == CUBLAS_STATUS_NOT_SUPPORTED) st = gemm(CUBLAS_COMPUTE_32F);
                    if (st != CUBLAS_STATUS_SUCCESS) {
                        note_error(("cuBLAS trailing update: " +
                                    std::string(cublasGetStatusString(st))).c_str());
                        return cudaErrorUnknown;
                    }
                    *nlaunch += 1;
                }
                updated = true;
            }
        }
        if (!updated) {
            k_panel_update<T, BW><<<ugrid, 256, 0, s>>>(A, n, k0, bw, T12, d_status);
            *nlaunch += 1;
        }
        k_panel_finish<T, BW><<<std::max(1, (n + 255) / 256), 256, 0, s>>>(A, n, k0, bw, T12,
                                                                           Ainv, d_status);
        *nlaunch += 5;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int status = 0;
    std::vector<int> hperm(n);
    e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hperm.data(), perm, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    if (status) {  // zero pivot
        *singular = true;
        return cudaSuccess;
    }
    std::vector<int> cols(n);
    for (int j = 0; j < n; j++) cols[j] = j;
    for (int k = n - 1; k >= 0; k--) std::swap(cols[k], cols[hperm[k]]);
    e = cudaMemcpyAsync(perm, cols.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    // column permutation with the panel buffers as scratch rows (needs kPermuteBlocks*n <= 2*BW*n)
    k_permute_cols_t<T><<<std::min(kPermuteBlocks, 2 * BW), 256, 0, s>>>(A, n, perm, W);
    *nlaunch += 1;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

}  // namespace

size_t inverse_scratch_elems(int n) {
    return (size_t)2 * 64 * n + 64 * 64 + 2 * kMaxPivotBlocks + 2 * (kMaxPivotBlocks + 1) * 64;
}

cudaError_t invert_f64(double* A, int n, int* perm, int* d_status, double* scratch,
                       long long* nlaunch, bool* singular, cudaStream_t s) {
    return invert_blocked<double, 16>(A, n, perm, d_status, scratch, nlaunch, singular, s);
}

// cuBLAS handles, a fixed pool per device.  Creating (or destroying) a handle
// invalidates a stream capture that another thread has in progress (measured on
// GB300: a loop creating and destroying handles next to 200 thread-local
// captures broke 45 of them; GEMM calls broke none), so the pool is made when the
// first context of a device is created, before any of its marches can capture,
// and lives as long as the process.
namespace {
constexpr int kBlasPool = 8;
constexpr int kBlasDevices = 64;
struct BlasPool {
    std::mutex m;
    std::condition_variable cv;
    bool made = false;
    int total = 0;
    std::vector<cublasHandle_t> free_handles;
};
BlasPool& blas_pool(int dev) {
    static BlasPool pools[kBlasDevices];
    return pools[dev];
}
}  // namespace

void blas_pool_init(int dev) {
    if (dev < 0 || dev >= kBlasDevices) return;
    BlasPool& p = blas_pool(dev);
    std::lock_guard<std::mutex> lk(p.m);
    if (p.made) return;
    p.made = true;
    for (int i = 0; i < kBlasPool; i++) {
        cublasHandle_t h = nullptr;
        if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) break;
        p.free_handles.push_back(h);
        p.total++;
    }
}

// wait: block until a handle is free (each user returns it once its work on the
// stream has finished); otherwise nullptr when none is free.
void* blas_checkout(int dev, bool wait) {
    if (dev < 0 || dev >= kBlasDevices) return nullptr;
    BlasPool& p = blas_pool(dev);
    std::unique_lock<std::mutex> lk(p.m);
    if (wait && p.total > 0) p.cv.wait(lk, [&] { return !p.free_handles.empty(); });
    if (p.free_handles.empty()) return nullptr;
    cublasHandle_t h = p.free_handles.back();
    p.free_handles.pop_back();
    return h;
}

void blas_return(int dev, void* h) {
    if (!h || dev < 0 || dev >= kBlasDevices) return;
    BlasPool& p = blas_pool(dev);
    {
        std::lock_guard<std::mutex> lk(p.m);
        p.free_handles.push_back(static_cast<cublasHandle_t>(h));
    }
    p.cv.notify_one();
}

cudaError_t levels_times_columns(const float* Gf, int ldf, int D, int nlev, const float* K,
                                 int C, float* out, int device, cudaStream_t s) {
    // column-major views: out_f (D x C, ld D) = G_f (row-major, ld ldf: op T) K (D x C)
    void* h = blas_checkout(device, true);
    if (!h) return cudaErrorNotReady;  // no handle could be made on this device
    cublasHandle_t hb = static_cast<cublasHandle_t>(h);
    const float one = 1.f, zero = 0.f;
    cublasStatus_t st = cublasSetStream(hb, s);
    if (st == CUBLAS_STATUS_SUCCESS)
        st = cublasSgemmStridedBatched(hb, CUBLAS_OP_T, CUBLAS_OP_N, D, C, D, &one, Gf, ldf,
                                       (long long)D * ldf, K, D, 0, &zero, out, D,
                                       (long long)C * D, nlev);
    // the handle (and any workspace of its) goes back only after the products ran
    const cudaError_t e = cudaStreamSynchronize(s);
    blas_return(device, h);
    if (e != cudaSuccess) return e;
    return st == CUBLAS_STATUS_SUCCESS ? cudaSuccess : cudaErrorUnknown;
}

cudaError_t invert_f32(const double* A64, float* A, int n, int* perm, int* d_status,
                       float* scratch, long long* nlaunch, bool* singular, cudaStream_t s,
                       void* blas) {
    k_cast_f64_f32<<<1216, 256, 0, s>>>(A64, A, (size_t)n * n);
    *nlaunch += 1;
    // first with the pivot search in the panels' diagonal blocks, then checked
    cudaError_t e = invert_blocked<float, 64>(A, n, perm, d_status, scratch, nlaunch, singular,
                                              s, true, blas);
    if (e != cudaSuccess) return e;
    bool good = false;
    if (!*singular) {
        // the probe's y (n doubles) and error word fit in the panel scratch rows
        double* y = reinterpret_cast<double*>(scratch);
        unsigned* err = reinterpret_cast<unsigned*>(y + n);
        e = cudaMemsetAsync(err, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        const unsigned g = (unsigned)(((size_t)n * 32 + 255) / 256);
        k_probe_xv<<<g, 256, 0, s>>>(A, n, y);
        k_probe_ay<<<g, 256, 0, s>>>(A64, n, y, err);
        *nlaunch += 2;
        unsigned bits = 0;
        e = cudaMemcpyAsync(&bits, err, sizeof(bits), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        float ef;
        std::memcpy(&ef, &bits, sizeof(ef));
        good = ef <= 1e-2f * 6.5f;
    }
    if (good) return cudaSuccess;
    k_cast_f64_f32<<<1216, 256, 0, s>>>(A64, A, (size_t)n * n);
    *nlaunch += 1;
    return invert_blocked<float, 64>(A, n, perm, d_status, scratch, nlaunch, singular, s, false,
                                     blas);
}

}  // namespace tdbem
