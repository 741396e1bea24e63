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
// whole inversion is 2 n^3 flops in GEMM form; the FP32 inverse runs step 5 on
// 128 x 128 tiles (k_panel_update_f32), the FP64 one on 64 x 64 tiles.
//
// The FP32 inverse (a preconditioner that FP64 refinement corrects) first restricts
// step 1's search to the panel's diagonal block, which needs no row swaps outside the
// panel and fits in three launches per panel (invert_blockpiv_f32).  On the
// boundary-element LHS the column maximum lies in that block (diagonal dominance), so
// the pivots are the same; a zero pivot in the block, or a probe
// max |A (X v) - v| / max |v| of the finished inverse above kInverseProbeBar (1e-5),
// sends the inversion back to the full search.
#include <cooperative_groups.h>

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

// The FP32 inverse's rank-64 trailing update, A[i][j] -= sum_c A[i][k0+c] T12[c][j]
// for i not in R1, j not in C1, on 128 x 128 tiles: the panel columns (transposed)
// and the T12 rows in shared memory, 8 x 8 outputs per thread (two 4-wide groups in
// rows and columns, 64 apart, so that a warp's shared-memory reads are conflict
// free), 64 FMAs per four 16-byte shared loads.  FP32 products and sums, as a
// plain SGEMM; the reads and writes of A are scalar (rows of an n not divisible by
// 4 are not 16-byte aligned).
constexpr int kUpdTile = 128, kUpdBW = 64, kUpdPad = 4;

// 4-byte asynchronous global-to-shared copy (cp.async, completion awaited with
// cp.async.wait_all by the issuing thread).
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
constexpr int kUpdSmem = 2 * kUpdBW * (kUpdTile + kUpdPad) * (int)sizeof(float);

__global__ void __launch_bounds__(256) k_panel_update_f32(float* __restrict__ A, int n, int k0,
                                                          int bw, const float* __restrict__ T12,
                                                          const int* __restrict__ status) {
    if (*status) return;
    extern __shared__ float usm[];
    float* sP = usm;                                 // [c][r], row stride kUpdTile + kUpdPad
    float* sT = usm + kUpdBW * (kUpdTile + kUpdPad);  // [c][q]
    constexpr int LD = kUpdTile + kUpdPad;
    const int i0 = blockIdx.y * kUpdTile, j0 = blockIdx.x * kUpdTile;
    const int tid = threadIdx.x;
    // panel tile sP[c][r] = A[i0 + r][k0 + c] (a warp reads 32 consecutive c of one
    // row) and T12 tile sT[c][q] = T12[c][j0 + q]: every element an asynchronous
    // 4-byte copy, all in flight together; zeros outside the matrix
#pragma unroll
    for (int it = 0; it < kUpdTile * kUpdBW / 256; it++) {
        const int idx = tid + it * 256;
        const int r = idx / kUpdBW, c = idx % kUpdBW;
        const int i = i0 + r;
        float* dst = sP + c * LD + r;
        if (i < n && c < bw) cp_async4(dst, A + (size_t)i * n + k0 + c);
        else *dst = 0.f;
    }
#pragma unroll
    for (int it = 0; it < kUpdTile * kUpdBW / 256; it++) {
        const int idx = tid + it * 256;
        const int c = idx / kUpdTile, q = idx % kUpdTile;
        const int j = j0 + q;
        float* dst = sT + c * LD + q;
        if (j < n && c < bw) cp_async4(dst, T12 + (size_t)c * n + j);
        else *dst = 0.f;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    const int tx = tid % 16, ty = tid / 16;
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[a][b] = 0.f;
#pragma unroll 4
    for (int c = 0; c < kUpdBW; c++) {
        const float4 p0 = *reinterpret_cast<const float4*>(sP + c * LD + ty * 4);
        const float4 p1 = *reinterpret_cast<const float4*>(sP + c * LD + ty * 4 + 64);
        const float4 t0 = *reinterpret_cast<const float4*>(sT + c * LD + tx * 4);
        const float4 t1 = *reinterpret_cast<const float4*>(sT + c * LD + tx * 4 + 64);
        const float pa[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
        const float tb[8] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w};
#pragma unroll
        for (int a = 0; a < 8; a++)
#pragma unroll
            for (int b = 0; b < 8; b++) acc[a][b] = fmaf(pa[a], tb[b], acc[a][b]);
    }
    // read-modify-write of the C tile, two of the thread's rows at a time: their 16
    // reads are issued together before any write (a store to A between two reads
    // of A would otherwise serialise every read's DRAM latency)
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float cv[2][8];
        bool ok[2][8];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int a = 2 * q + h;
            const int i = i0 + ty * 4 + (a & 3) + (a >> 2) * 64;
            const bool row_ok = i < n && !(i >= k0 && i < k0 + bw);
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const int j = j0 + tx * 4 + (b & 3) + (b >> 2) * 64;
                ok[h][b] = row_ok && j < n && !(j >= k0 && j < k0 + bw);
                cv[h][b] = ok[h][b] ? A[(size_t)i * n + j] : 0.f;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int a = 2 * q + h;
            const int i = i0 + ty * 4 + (a & 3) + (a >> 2) * 64;
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const int j = j0 + tx * 4 + (b & 3) + (b >> 2) * 64;
                if (ok[h][b]) A[(size_t)i * n + j] = cv[h][b] - acc[a][b];
            }
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

// Richardson iteration x <- x + X (b - A x) (FP64 residual, FP32 X) on the probe
// problem b = A v: the kernels of richardson_probe.
__global__ void __launch_bounds__(256) k_rich_b(const double* __restrict__ A, int n,
                                                double* __restrict__ b, float* __restrict__ b32) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    const double* row = A + (size_t)w * n;
    double acc = 0;
    for (int j = lane; j < n; j += 32) acc += row[j] * probe_v(j);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
        b[w] = acc;
        b32[w] = (float)acc;
    }
}

// Whether the previous sweep (its error word prev, null for the first) has already
// reached the tolerance: the sweeps after it do nothing.
__device__ __forceinline__ bool rich_done(const unsigned* prev, unsigned tol_bits) {
    return prev && *prev <= tol_bits;
}

// x = X r32 (accumulate = 0) or x += X r32; err_bits (if set) receives
// max_i |x_i - v_i| as float bits.
__global__ void __launch_bounds__(256) k_rich_x(const float* __restrict__ X, int n,
                                                const float* __restrict__ r32,
                                                double* __restrict__ x, int accumulate,
                                                unsigned* __restrict__ err_bits,
                                                const unsigned* __restrict__ prev,
                                                unsigned tol_bits) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n || rich_done(prev, tol_bits)) return;
    const float* row = X + (size_t)w * n;
    float acc = 0.f;
    for (int j = lane; j < n; j += 32) acc += row[j] * r32[j];
    double a = acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) {
        const double xv = accumulate ? x[w] + a : a;
        x[w] = xv;
        if (err_bits) {
            const float e = (float)fabs(xv - probe_v(w));
            atomicMax(err_bits, __float_as_uint(e == e ? e : 3.0e38f));  // NaN counts as huge
        }
    }
}

// r32 = b - A x
__global__ void __launch_bounds__(256) k_rich_r(const double* __restrict__ A, int n,
                                                const double* __restrict__ x,
                                                const double* __restrict__ b,
                                                float* __restrict__ r32,
                                                const unsigned* __restrict__ prev,
                                                unsigned tol_bits) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n || rich_done(prev, tol_bits)) return;
    const double* row = A + (size_t)w * n;
    double acc = 0;
    for (int j = lane; j < n; j += 32) acc += row[j] * x[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) r32[w] = (float)(b[w] - acc);
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
        if (r == cudaSuccess && std::is_same<T, float>::value && BW == kUpdBW)
            r = cudaFuncSetAttribute((const void*)k_panel_update_f32,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, kUpdSmem);
        return r;
    }();
    return e;
}


template <typename T, int BW>
cudaError_t invert_blocked(T* A, int n, int* perm, int* d_status, T* scratch, long long* nlaunch,
                           bool* singular, cudaStream_t s) {
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
        if constexpr (std::is_same<T, float>::value && BW == kUpdBW) {
            const dim3 wgrid((n + kUpdTile - 1) / kUpdTile, (n + kUpdTile - 1) / kUpdTile);
            k_panel_update_f32<<<wgrid, 256, kUpdSmem, s>>>(A, n, k0, bw, T12, d_status);
            *nlaunch += 1;
            updated = true;
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

// ---------------------------------------------------------------------------
// The FP32 inverse with the pivot search restricted to the panels' diagonal blocks,
// in three launches per 64-column panel.  With the swaps confined to the panel's own
// rows R1, and those rows overwritten by the panel step, the step needs only the
// inverse of the unpermuted diagonal block A11 (with P the block's row permutation,
// (P A11)^-1 P A[R1, :] = A11^-1 A[R1, :], and the column exchange the swaps imply
// on A[:, C1] cancels against the permutation of the finished inverse's columns):
//   T12 = A11^-1 A[R1, :],    A[i, j] -= A[i, C1] T12[:, j]   (i not in R1, j not in C1)
//   A[R1, :] = T12 with A[R1, C1] = A11^-1,   A[i, C1] = -A[i, C1] A11^-1  (i not in R1)
// which is block Gauss-Jordan without swaps between panels: the finished matrix is
// A^-1 with no column permutation.  Per panel:
//   k_block_inverse_f32  (one CTA) A11^-1, Gauss-Jordan with partial pivoting;
//   k_panel_b_f32        B = [T12 | A11^-1] (64 x n) and Pc = A[:, C1]^T (64 x n);
//   k_panel_step_f32     every 128 x 64 tile of A from Pc^T B: the trailing update,
//                        the pivot rows and the panel columns in one pass.
// Each block fits in a fourth of an SM (16K registers, <= 34 KB of shared memory), so
// that beside the assembly's kernels it waits for one block of theirs to retire.
// ---------------------------------------------------------------------------
constexpr int kGjThreads = 256;

// A11^-1 of the panel's diagonal block (bw x bw, padded to 64 x 64 with the
// identity) by in-place Gauss-Jordan with partial pivoting among the rows not yet
// pivoted (largest magnitude, lowest row on ties), rows left in place: at step c the
// pivot row p_c is scaled and column c eliminated from every other row, and column
// c's storage then holds the transformed identity column p_c.  The result S gives
// A11^-1[c][j] = S[p_c][q] with p_q = j.  Thread t keeps entries q0 .. q0 + 15 of row
// t / 4 (q0 = 16 (t % 4)) in registers; per column the owners of column c publish it,
// warp 0 picks the pivot, the pivot row's owners publish it scaled, and every thread
// updates its entries (three barriers, 64 + 64 shared values per column).  The column
// loop runs in blocks of 16 so that the owned entry of column c is a fixed register.
// A zero pivot sets *status = 2.
__global__ void __launch_bounds__(kGjThreads) k_block_inverse_f32(const float* __restrict__ A,
                                                                  int n, int k0, int bw,
                                                                  float* __restrict__ Ainv,
                                                                  int* __restrict__ status) {
    if (*status) return;
    __shared__ float s_col[64], s_row[64];
    __shared__ int s_p[64], s_pinv[64], s_used[64];
    __shared__ float s_piv;
    __shared__ int s_pc;
    const int t = threadIdx.x;
    const int r = t >> 2, q0 = (t & 3) * 16;
    float a[16];
#pragma unroll
    for (int jj = 0; jj < 16; jj++) {
        const int j = q0 + jj;
        a[jj] = (r < bw && j < bw) ? A[(size_t)(k0 + r) * n + k0 + j] : (r == j ? 1.f : 0.f);
    }
    if (t < 64) s_used[t] = 0;
    for (int cb = 0; cb < 64; cb += 16) {
        const bool own = q0 == cb;  // this thread holds columns cb .. cb + 15 of its row
#pragma unroll
        for (int ci = 0; ci < 16; ci++) {
            const int c = cb + ci;
            if (own) s_col[r] = a[ci];
            __syncthreads();
            if (t < 32) {
                const float v0 = s_used[t] ? -1.f : fabsf(s_col[t]);
                const float v1 = s_used[t + 32] ? -1.f : fabsf(s_col[t + 32]);
                float best = v0;
                int bi = t;
                if (v1 > best) {
                    best = v1;
                    bi = t + 32;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float v2 = __shfl_xor_sync(0xffffffffu, best, o);
                    const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (v2 > best || (v2 == best && i2 < bi)) {
                        best = v2;
                        bi = i2;
                    }
                }
                if (t == 0) {
                    s_pc = best > 0.f ? bi : -1;
                    s_p[c] = bi;
                    if (best > 0.f) {
                        s_used[bi] = 1;
                        s_piv = 1.f / s_col[bi];
                    }
                }
            }
            __syncthreads();
            const int p = s_pc;
            if (p < 0) {  // the same on every thread
                if (t == 0) *status = 2;
                return;
            }
            const float piv = s_piv;
            if (r == p) {  // the pivot row, scaled (its column c becomes piv)
#pragma unroll
                for (int jj = 0; jj < 16; jj++)
                    s_row[q0 + jj] = (own && jj == ci ? 1.f : a[jj]) * piv;
            }
            const float f = s_col[r];
            __syncthreads();
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
                const float rp = s_row[q0 + jj];
                a[jj] = r == p ? rp : (own && jj == ci ? 0.f : a[jj]) - f * rp;
            }
        }
    }
    __syncthreads();
    if (t < 64) s_pinv[s_p[t]] = t;
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < 16; jj++) Ainv[s_pinv[r] * 64 + s_p[q0 + jj]] = a[jj];
}

// B[c][j] = sum_d Ainv[c][d] A[k0 + d][j] (T12) for j outside the panel columns and
// Ainv[c][j - k0] inside them; Pc[c][i] = A[i][k0 + c].  Thread per column j (and
// per row i = j for Pc); rows c >= bw of B and Pc come out zero (Ainv is the
// identity there and the panel's columns beyond bw are zero).  ld: the leading
// dimension of B and Pc.
__global__ void __launch_bounds__(128) k_panel_b_f32(const float* __restrict__ A, int n, int k0,
                                                     int bw, const float* __restrict__ Ainv,
                                                     float* __restrict__ B,
                                                     float* __restrict__ Pc, int ld,
                                                     const int* __restrict__ status) {
    if (*status) return;
    __shared__ float sa[64 * 64];
    for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) sa[i] = Ainv[i];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
#pragma unroll 16
    for (int c = 0; c < 64; c++) Pc[(size_t)c * ld + j] = c < bw ? A[(size_t)j * n + k0 + c] : 0.f;
    if (j >= k0 && j < k0 + bw) {
        for (int c = 0; c < 64; c++) B[(size_t)c * ld + j] = sa[c * 64 + (j - k0)];
        return;
    }
    float a[64];
#pragma unroll
    for (int d = 0; d < 64; d++) a[d] = d < bw ? A[(size_t)(k0 + d) * n + j] : 0.f;
    for (int c = 0; c < 64; c++) {
        float acc = 0.f;
#pragma unroll
        for (int d = 0; d < 64; d++) acc = fmaf(sa[c * 64 + d], a[d], acc);
        B[(size_t)c * ld + j] = acc;
    }
}

// One tile of the panel step, 128 rows x 64 columns, 128 threads (8 x 8 outputs
// each): acc = Pc[:, i0..]^T B[:, j0..] over the 64 panel columns in two halves of 32
// (25.6 KB of shared memory), then per entry (i, j): a pivot row i takes
// B[i - k0][j]; a panel column j (other rows) takes -acc; the rest A[i][j] - acc
// (their reads issued two rows at a time before the writes).  16K registers and
// 25.6 KB of shared memory per block.
constexpr int kStepTM = 128, kStepTN = 64, kStepKH = 32;
constexpr int kStepLP = kStepTM + 4, kStepLT = kStepTN + 4;
constexpr int kStepSmem = kStepKH * (kStepLP + kStepLT) * (int)sizeof(float);

__global__ void __launch_bounds__(128, 4) k_panel_step_f32(float* __restrict__ A, int n, int k0,
                                                        int bw, const float* __restrict__ B,
                                                        const float* __restrict__ Pc, int ld,
                                                        const int* __restrict__ status) {
    if (*status) return;
    __shared__ __align__(16) float sP[kStepKH * kStepLP];  // [c][r]
    __shared__ __align__(16) float sT[kStepKH * kStepLT];  // [c][q]
    const int i0 = blockIdx.y * kStepTM, j0 = blockIdx.x * kStepTN;
    const int tid = threadIdx.x;
    const int tx = tid % 8, ty = tid / 8;
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[a][b] = 0.f;
    for (int h0 = 0; h0 < 64; h0 += kStepKH) {
        if (h0) __syncthreads();  // the first half's reads are done
#pragma unroll
        for (int it = 0; it < kStepKH * kStepTM / 128; it++) {
            const int idx = tid + it * 128;
            const int c = idx / kStepTM, q = idx % kStepTM;
            if (i0 + q < n) cp_async4(sP + c * kStepLP + q, Pc + (size_t)(h0 + c) * ld + i0 + q);
            else sP[c * kStepLP + q] = 0.f;
        }
#pragma unroll
        for (int it = 0; it < kStepKH * kStepTN / 128; it++) {
            const int idx = tid + it * 128;
            const int c = idx / kStepTN, q = idx % kStepTN;
            if (j0 + q < n) cp_async4(sT + c * kStepLT + q, B + (size_t)(h0 + c) * ld + j0 + q);
            else sT[c * kStepLT + q] = 0.f;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
#pragma unroll 4
        for (int c = 0; c < kStepKH; c++) {
            const float4 p0 = *reinterpret_cast<const float4*>(sP + c * kStepLP + ty * 4);
            const float4 p1 = *reinterpret_cast<const float4*>(sP + c * kStepLP + ty * 4 + 64);
            const float4 t0 = *reinterpret_cast<const float4*>(sT + c * kStepLT + tx * 4);
            const float4 t1 = *reinterpret_cast<const float4*>(sT + c * kStepLT + tx * 4 + 32);
            const float pa[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
            const float tb[8] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w};
#pragma unroll
            for (int a = 0; a < 8; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) acc[a][b] = fmaf(pa[a], tb[b], acc[a][b]);
        }
    }
    // A tile inside the matrix that meets neither the pivot rows nor the pivot columns
    // (most tiles): every entry is A - acc, read and written as float pairs (n even:
    // a row's pairs start on 8-byte boundaries), four rows' reads before their writes.
    const bool interior = (n % 2 == 0) && i0 + kStepTM <= n && j0 + kStepTN <= n &&
                          (i0 >= k0 + bw || i0 + kStepTM <= k0) &&
                          (j0 >= k0 + bw || j0 + kStepTN <= k0);
    if (interior) {
#pragma unroll
        for (int g = 0; g < 2; g++) {
            float2 cv[4][4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const float* row = A + (size_t)(i0 + ty * 4 + r + g * 64) * n + j0 + tx * 4;
#pragma unroll
                for (int h = 0; h < 4; h++)
                    cv[r][h] = *reinterpret_cast<const float2*>(row + (h >> 1) * 32 + (h & 1) * 2);
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int a = r + 4 * g;
                float* row = A + (size_t)(i0 + ty * 4 + r + g * 64) * n + j0 + tx * 4;
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const int b = (h >> 1) * 4 + (h & 1) * 2;
                    *reinterpret_cast<float2*>(row + (h >> 1) * 32 + (h & 1) * 2) =
                        make_float2(cv[r][h].x - acc[a][b], cv[r][h].y - acc[a][b + 1]);
                }
            }
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float cv[2][8];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int a = 2 * q + h;
            const int i = i0 + ty * 4 + (a & 3) + (a >> 2) * 64;
            const bool rest_row = i < n && !(i >= k0 && i < k0 + bw);
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const int j = j0 + tx * 4 + (b & 3) + (b >> 2) * 32;
                const bool rest = rest_row && j < n && !(j >= k0 && j < k0 + bw);
                cv[h][b] = rest ? A[(size_t)i * n + j] : 0.f;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int a = 2 * q + h;
            const int i = i0 + ty * 4 + (a & 3) + (a >> 2) * 64;
            if (i >= n) continue;
            const bool pivot_row = i >= k0 && i < k0 + bw;
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const int j = j0 + tx * 4 + (b & 3) + (b >> 2) * 32;
                if (j >= n) continue;
                float v;
                if (pivot_row) v = B[(size_t)(i - k0) * ld + j];
                else if (j >= k0 && j < k0 + bw) v = -acc[a][b];
                else v = cv[h][b] - acc[a][b];
                A[(size_t)i * n + j] = v;
            }
        }
    }
}

// The three-launch FP32 inversion (above) in place; *singular on a zero pivot in a
// diagonal block.  scratch holds B and Pc (64 x ld each, ld = n rounded up to 4) and
// the block inverse (64 x 64).
cudaError_t invert_blockpiv_f32(float* A, int n, int* d_status, float* scratch,
                                long long* nlaunch, bool* singular, cudaStream_t s) {
    *singular = false;
    const int ld = (n + 3) & ~3;
    float* B = scratch;
    float* Pc = B + (size_t)64 * ld;
    float* Ainv = Pc + (size_t)64 * ld;
    // prefer the largest shared-memory carveout, so that these blocks fit beside the
    // assembly's blocks on an SM
    static const cudaError_t ea = [] {
        const void* fns[3] = {(const void*)k_block_inverse_f32, (const void*)k_panel_b_f32,
                              (const void*)k_panel_step_f32};
        for (const void* fn : fns) {
            const cudaError_t r = cudaFuncSetAttribute(
                fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }();
    if (ea != cudaSuccess) return ea;
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    for (int k0 = 0; k0 < n; k0 += 64) {
        const int bw = std::min(64, n - k0);
        k_block_inverse_f32<<<1, kGjThreads, 0, s>>>(A, n, k0, bw, Ainv, d_status);
        k_panel_b_f32<<<(n + 127) / 128, 128, 0, s>>>(A, n, k0, bw, Ainv, B, Pc, ld, d_status);
        k_panel_step_f32<<<dim3((n + kStepTN - 1) / kStepTN, (n + kStepTM - 1) / kStepTM), 128, 0,
                           s>>>(A, n, k0, bw, B, Pc, ld, d_status);
        *nlaunch += 3;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int status = 0;
    e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    *singular = status != 0;
    return cudaSuccess;
}

}  // namespace

size_t inverse_scratch_elems(int n) {
    // the panel kernels' T12 and permutation rows, the diagonal-block inverse and the
    // pivot candidates; the three-launch FP32 form's B and Pc (64 x ld each, ld = n
    // rounded up to 4) and block inverse
    const size_t blocked =
        (size_t)2 * 64 * n + 64 * 64 + 2 * kMaxPivotBlocks + 2 * (kMaxPivotBlocks + 1) * 64;
    const size_t blockpiv = (size_t)2 * 64 * (size_t)((n + 3) & ~3) + 64 * 64;
    return std::max(blocked, blockpiv);
}

cudaError_t invert_f64(double* A, int n, int* perm, int* d_status, double* scratch,
                       long long* nlaunch, bool* singular, cudaStream_t s) {
    return invert_blocked<double, 16>(A, n, perm, d_status, scratch, nlaunch, singular, s);
}

namespace {

// out[f][c][row] = sum_col Gf[f][row][col] K[c][col] for levels f < nlev: every
// level of the FP32 store times the C columns of K (the batched march's known
// tractions), in FP32 as an SGEMM per level.  A CTA takes 128 rows x 64 columns of
// one level, 32-wide K chunks staged in shared memory (the level rows transposed),
// 8 x 4 outputs per thread.
constexpr int kLtcRows = 128, kLtcCols = 64, kLtcK = 32;

__global__ void __launch_bounds__(256) k_levels_times_columns(const float* __restrict__ Gf,
                                                              int ldf, int D,
                                                              const float* __restrict__ K,
                                                              int C, float* __restrict__ out) {
    __shared__ __align__(16) float sG[kLtcK][kLtcRows + 4];
    __shared__ __align__(16) float sK[kLtcK][kLtcCols + 4];
    const int f = blockIdx.z;
    const int r0 = blockIdx.x * kLtcRows, c0 = blockIdx.y * kLtcCols;
    const float* G = Gf + (size_t)f * D * ldf;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    float acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0.f;
    for (int k0 = 0; k0 < D; k0 += kLtcK) {
#pragma unroll
        for (int it = 0; it < kLtcRows * kLtcK / 256; it++) {
            const int idx = tid + it * 256;
            const int r = idx / kLtcK, k = idx % kLtcK;
            const int row = r0 + r, col = k0 + k;
            if (row < D && col < D) cp_async4(&sG[k][r], G + (size_t)row * ldf + col);
            else sG[k][r] = 0.f;
        }
#pragma unroll
        for (int it = 0; it < kLtcCols * kLtcK / 256; it++) {
            const int idx = tid + it * 256;
            const int c = idx / kLtcK, k = idx % kLtcK;
            const int cc = c0 + c, col = k0 + k;
            if (cc < C && col < D) cp_async4(&sK[k][c], K + (size_t)cc * D + col);
            else sK[k][c] = 0.f;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < kLtcK; k++) {
            const float4 g0 = *reinterpret_cast<const float4*>(&sG[k][ty * 4]);
            const float4 g1 = *reinterpret_cast<const float4*>(&sG[k][ty * 4 + 64]);
            const float4 kv = *reinterpret_cast<const float4*>(&sK[k][tx * 4]);
            const float ga[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
            const float kb[4] = {kv.x, kv.y, kv.z, kv.w};
#pragma unroll
            for (int a = 0; a < 8; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fmaf(ga[a], kb[b], acc[a][b]);
        }
        __syncthreads();
    }
    float* o = out + (size_t)f * C * D;
#pragma unroll
    for (int a = 0; a < 8; a++) {
        const int row = r0 + ty * 4 + (a & 3) + (a >> 2) * 64;
        if (row >= D) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int cc = c0 + tx * 4 + b;
            if (cc < C) o[(size_t)cc * D + row] = acc[a][b];
        }
    }
}

}  // namespace

cudaError_t levels_times_columns(const float* Gf, int ldf, int D, int nlev, const float* K,
                                 int C, float* out, cudaStream_t s) {
    if (nlev <= 0 || C <= 0) return cudaSuccess;
    const dim3 grid((D + kLtcRows - 1) / kLtcRows, (C + kLtcCols - 1) / kLtcCols, nlev);
    k_levels_times_columns<<<grid, 256, 0, s>>>(Gf, ldf, D, K, C, out);
    return cudaGetLastError();
}

// The probe's relative residual max |A64 (X v) - v| / max |v| (max |v| = 6.5).
cudaError_t probe_inverse(const double* A64, const float* X, int n, float* scratch, float* rel,
                          long long* nlaunch, cudaStream_t s) {
    // the probe's y (n doubles) and error word fit in the panel scratch rows
    double* y = reinterpret_cast<double*>(scratch);
    unsigned* err = reinterpret_cast<unsigned*>(y + n);
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)(((size_t)n * 32 + 255) / 256);
    k_probe_xv<<<g, 256, 0, s>>>(X, n, y);
    k_probe_ay<<<g, 256, 0, s>>>(A64, n, y, err);
    *nlaunch += 2;
    unsigned bits = 0;
    e = cudaMemcpyAsync(&bits, err, sizeof(bits), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    float ef;
    std::memcpy(&ef, &bits, sizeof(ef));
    *rel = ef / 6.5f;
    return cudaSuccess;
}

cudaError_t richardson_probe(const double* A, const float* X, int n, double* work, int max_sweeps,
                             double tol, int* sweeps, long long* nlaunch, cudaStream_t s) {
    *sweeps = 0;
    if (max_sweeps < 1) return cudaSuccess;
    double* b = work;
    double* x = work + n;
    float* r32 = reinterpret_cast<float*>(work + 2 * (size_t)n);
    unsigned* err = reinterpret_cast<unsigned*>(r32 + n + (n & 1));  // max_sweeps + 1 words
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned) * (max_sweeps + 1), s);
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)(((size_t)n * 32 + 255) / 256);
    // a sweep after the first that reaches the tolerance returns at once (the count is
    // all that is kept; the later error words stay 0)
    const float tol_err = (float)(tol * 6.5);
    unsigned tol_bits = 0;
    std::memcpy(&tol_bits, &tol_err, sizeof(tol_bits));
    k_rich_b<<<g, 256, 0, s>>>(A, n, b, r32);
    k_rich_x<<<g, 256, 0, s>>>(X, n, r32, x, 0, err, nullptr, tol_bits);
    for (int it = 1; it <= max_sweeps; it++) {
        const unsigned* prev = it >= 2 ? err + it - 1 : nullptr;
        k_rich_r<<<g, 256, 0, s>>>(A, n, x, b, r32, prev, tol_bits);
        k_rich_x<<<g, 256, 0, s>>>(X, n, r32, x, 1, err + it, prev, tol_bits);
    }
    *nlaunch += 2 + 2LL * max_sweeps;
    std::vector<unsigned> bits(max_sweeps + 1);
    e = cudaMemcpyAsync(bits.data(), err, sizeof(unsigned) * bits.size(), cudaMemcpyDeviceToHost,
                        s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    // the test the sweeps applied on the device (max |x - v| <= tol max |v|, as float
    // bits): the first sweep that passes it
    for (int it = 1; it <= max_sweeps; it++) {
        if (bits[it] <= tol_bits) {
            *sweeps = it;
            break;
        }
    }
    return cudaSuccess;
}

cudaError_t invert_f32(const double* A64, float* A, int n, int* perm, int* d_status,
                       float* scratch, long long* nlaunch, bool* singular, cudaStream_t s,
                       InverseReport* report) {
    k_cast_f64_f32<<<1216, 256, 0, s>>>(A64, A, (size_t)n * n);
    *nlaunch += 1;
    // first with the pivot search in the panels' diagonal blocks, then checked
    cudaError_t e = invert_blockpiv_f32(A, n, d_status, scratch, nlaunch, singular, s);
    if (e != cudaSuccess) return e;
    float rel = 3.0e38f;
    if (!*singular) {
        e = probe_inverse(A64, A, n, scratch, &rel, nlaunch, s);
        if (e != cudaSuccess) return e;
    }
    if (report) {
        report->probe_rel = rel;
        report->full_search = 0;
    }
    if (rel <= kInverseProbeBar) return cudaSuccess;
    // a zero pivot in a diagonal block or a residual above the bar: the full search
    k_cast_f64_f32<<<1216, 256, 0, s>>>(A64, A, (size_t)n * n);
    *nlaunch += 1;
    e = invert_blocked<float, 64>(A, n, perm, d_status, scratch, nlaunch, singular, s);
    if (e != cudaSuccess || *singular || !report) return e;
    report->full_search = 1;
    return probe_inverse(A64, A, n, scratch, &report->probe_rel, nlaunch, s);
}

}  // namespace tdbem
