// Batched marching: many load cases on one mesh (same levels, LHS and boundary
// conditions), the per-case loop of SolverStepLinearT::Solve_Averaging
// (SolverStepLinearT.cpp:314-544) run for all cases at once.
//
// Per step the history convolution of all C cases is one GEMM,
//     RHS[c][row] = sum_f ( G^f[row,:] . Wt[f][c] - H^f[row,:] . Wu[f][c] ),
// with M = D rows, N = C cases and K = levels x D.  It runs on the tensor cores
// with warp-level mma.sync m16n8k16 BF16 -> FP32 and a 3-term split of both
// operands (x = hi + lo, hi = bf16(x), lo = bf16(x - hi);
// A B ~ Ahi Bhi + Ahi Blo + Alo Bhi, about 16 significant bits per operand).  The
// MMAs accumulate one level's product in FP32; the levels are added with
// compensated (Kahan) FP32 summation.  The levels are split over blocks
// (split-K) so that the blocks sharing a slice of W run together and W stays in
// L2; the split partial sums are reduced in FP64.
//
// The solve applies the FP32 inverse of the column-exchanged LHS to all
// right-hand sides (FP32 products and sums on the CUDA cores).  A refinement
// sweep computes r = rhs - A64 x with the FP64 LHS and FP64 x, each split into
// two FP32 words, by compensated dot products in FP32 arithmetic (TwoProd and
// TwoSum error terms carried in a second FP32 sum, the Dot2 scheme of Ogita,
// Rump and Oishi, 2005), so the FP64 pipe is not used; dx = inv32 r, x += dx.
#include <cuda_bf16.h>

#include <algorithm>

#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

// ---------------------------------------------------------------------------
// Tensor-core convolution
// ---------------------------------------------------------------------------
constexpr int BM = 128, BN = 64, BK = 32;
constexpr int SPAD = BK + 8;  // bf16 per shared row: 80 B, conflict-free ldmatrix rows

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(__fsub_rn(x, __bfloat162float(hi)));
}

__device__ __forceinline__ void ldmatrix_x4(unsigned r[4], const __nv_bfloat16* p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float d[4], const unsigned a[4], unsigned b0,
                                         unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
        "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void store_split4(__nv_bfloat16* hi, __nv_bfloat16* lo, float4 v,
                                             float sgn) {
    __nv_bfloat16 h, l;
    split_bf16(sgn * v.x, h, l); hi[0] = h; lo[0] = l;
    split_bf16(sgn * v.y, h, l); hi[1] = h; lo[1] = l;
    split_bf16(sgn * v.z, h, l); hi[2] = h; lo[2] = l;
    split_bf16(sgn * v.w, h, l); hi[3] = h; lo[3] = l;
}

// partial[split][c][row] = sum over this split's levels f of
//   G^f[row, :] . Wt[f][c, :]  -  H^f[row, :] . Wu[f][c, :]
// G/H: FP32 levels [f][row][ld] (ld % 4 == 0, zero-padded columns);
// Wt/Wu: FP32 [f][c][ldw] (ldw a multiple of BK >= ld, zero-padded).
// Grid: (row tiles, splits, column blocks of BN cases).  256 threads as 4 x 2
// warps, each warp a 32 x 32 tile of 2 x 4 m16n8 fragments.
__global__ void __launch_bounds__(256) k_conv_mma(const float* __restrict__ G,
                                                  const float* __restrict__ H, size_t lstride,
                                                  int ld, int D, int nlev, int per_split,
                                                  const float* __restrict__ Wt,
                                                  const float* __restrict__ Wu, int ldw, int C,
                                                  double* __restrict__ partial) {
    __shared__ __align__(16) __nv_bfloat16 sAh[BM][SPAD], sAl[BM][SPAD];
    __shared__ __align__(16) __nv_bfloat16 sBh[BN][SPAD], sBl[BN][SPAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp & 3, wn = warp >> 2;
    const int row0 = blockIdx.x * BM;
    const int c0 = blockIdx.z * BN;
    const int Cl = min(BN, C - c0);
    const int f0 = blockIdx.y * per_split;
    const int f1 = min(nlev, f0 + per_split);
    const int nk = (ld + BK - 1) / BK;
    const int per_level = 2 * nk;
    const int total = max(0, f1 - f0) * per_level;

    float acc[2][4][4], sum[2][4][4], cmp[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = sum[i][j][e] = cmp[i][j][e] = 0.f;

    // global -> register prefetch of one (level, matrix, k-tile) iteration
    float4 va[4], vb[2];
    auto load = [&](int it) {
        const int f = f0 + it / per_level;
        const int rem = it % per_level;
        const int mat = rem / nk, k0 = (rem % nk) * BK;
        const float* Am = (mat == 0 ? G : H) + (size_t)f * lstride;
        const float* Bm = (mat == 0 ? Wt : Wu) + ((size_t)f * C + c0) * ldw;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int idx = tid + q * 256;
            const int r = idx >> 3, k = k0 + 4 * (idx & 7);
            const int row = row0 + r;
            va[q] = (row < D && k < ld)
                        ? __ldcs(reinterpret_cast<const float4*>(Am + (size_t)row * ld + k))
                        : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int idx = tid + q * 256;
            const int cc = idx >> 3, k = k0 + 4 * (idx & 7);
            vb[q] = cc < Cl ? *reinterpret_cast<const float4*>(Bm + (size_t)cc * ldw + k)
                            : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };

    if (total > 0) load(0);
    for (int it = 0; it < total; it++) {
        const int rem = it % per_level;
        const float sgn = rem < nk ? 1.f : -1.f;  // H products enter with a minus sign
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int idx = tid + q * 256;
            const int r = idx >> 3, k = 4 * (idx & 7);
            store_split4(&sAh[r][k], &sAl[r][k], va[q], 1.f);
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int idx = tid + q * 256;
            const int cc = idx >> 3, k = 4 * (idx & 7);
            store_split4(&sBh[cc][k], &sBl[cc][k], vb[q], sgn);
        }
        __syncthreads();
        if (it + 1 < total) load(it + 1);
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            unsigned ah[2][4], al[2][4], bh[2][4], bl[2][4];
            // A: lanes 0-15 rows 0-15 at k, lanes 16-31 rows 0-15 at k+8
            const int ar = lane & 15, ac = kk + ((lane >> 4) << 3);
#pragma unroll
            for (int i = 0; i < 2; i++) {
                ldmatrix_x4(ah[i], &sAh[wm * 32 + i * 16 + ar][ac]);
                ldmatrix_x4(al[i], &sAl[wm * 32 + i * 16 + ar][ac]);
            }
            // B ([n][k]): lanes 0-7 n0-7 k, 8-15 n0-7 k+8, 16-23 n8-15 k, 24-31 n8-15 k+8
            const int bn = ((lane >> 4) << 3) + (lane & 7);
            const int bc = kk + (((lane >> 3) & 1) << 3);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                ldmatrix_x4(bh[j], &sBh[wn * 32 + j * 16 + bn][bc]);
                ldmatrix_x4(bl[j], &sBl[wn * 32 + j * 16 + bn][bc]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int jj = j >> 1, o = (j & 1) * 2;
                    mma_bf16(acc[i][j], al[i], bh[jj][o], bh[jj][o + 1]);
                    mma_bf16(acc[i][j], ah[i], bl[jj][o], bl[jj][o + 1]);
                    mma_bf16(acc[i][j], ah[i], bh[jj][o], bh[jj][o + 1]);
                }
        }
        if (rem == per_level - 1) {  // level done: compensated add, restart the level sum
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float y = __fsub_rn(acc[i][j][e], cmp[i][j][e]);
                        const float t = __fadd_rn(sum[i][j][e], y);
                        cmp[i][j][e] = __fsub_rn(__fsub_rn(t, sum[i][j][e]), y);
                        sum[i][j][e] = t;
                        acc[i][j][e] = 0.f;
                    }
        }
    }
    // D fragment of m16n8: e0 (row g, col 2t), e1 (g, 2t+1), e2 (g+8, 2t), e3 (g+8, 2t+1)
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int row = row0 + wm * 32 + i * 16 + g + ((e >> 1) << 3);
                const int cc = wn * 32 + j * 8 + 2 * t4 + (e & 1);
                if (row < D && cc < Cl)
                    partial[((size_t)blockIdx.y * C + c0 + cc) * D + row] =
                        (double)sum[i][j][e] - (double)cmp[i][j][e];
            }
}

// ---------------------------------------------------------------------------
// Inverse application and residual on the CUDA cores
// ---------------------------------------------------------------------------
constexpr int TM = 64, TN = 64, TK = 16, TP = TM + 4;

// MODE 0: partial[z][c][row] =  sum_{k in split z} inv32[row][k] * float(X[c][k])
// MODE 1: partial[z][c][row] = -sum_{k in split z} A64[row][k] * X[c][k], with
//         A64 = Ah + Al and X = Xh + Xl split into FP32 words and each product /
//         sum error carried in a second FP32 accumulator (Dot2).
// Grid: (row tiles, column tiles, K splits); 256 threads, 4 x 4 outputs each.
template <int MODE>
__global__ void __launch_bounds__(256) k_apply_cols(const void* __restrict__ Aptr, int D,
                                                    const double* __restrict__ X, int C,
                                                    int kper, double* __restrict__ partial) {
    __shared__ __align__(16) float sAh[TK][TP], sXh[TK][TP];
    __shared__ __align__(16) float sAl[MODE == 1 ? TK : 1][TP], sXl[MODE == 1 ? TK : 1][TP];
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int row0 = blockIdx.x * TM, c0 = blockIdx.y * TN;
    const int kb = blockIdx.z * kper, ke = min(D, kb + kper);
    float s[4][4], t[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) s[i][j] = t[i][j] = 0.f;
    for (int k0 = kb; k0 < ke; k0 += TK) {
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int idx = tid + q * 256;
            const int r = idx >> 4, k = idx & 15;
            const int row = row0 + r, kk = k0 + k;
            const bool in = row < D && kk < ke;
            if (MODE == 0) {
                const float* A = static_cast<const float*>(Aptr);
                sAh[k][r] = in ? __ldcs(A + (size_t)row * D + kk) : 0.f;
            } else {
                const double* A = static_cast<const double*>(Aptr);
                const double a = in ? __ldcs(A + (size_t)row * D + kk) : 0.0;
                const float ah = (float)a;
                sAh[k][r] = ah;
                sAl[k][r] = (float)(a - (double)ah);
            }
            const int cc = c0 + r;
            const double x = (cc < C && kk < ke) ? X[(size_t)cc * D + kk] : 0.0;
            const float xh = (float)x;
            sXh[k][r] = xh;
            if (MODE == 1) sXl[k][r] = (float)(x - (double)xh);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TK; k++) {
            const float4 a4 = *reinterpret_cast<const float4*>(&sAh[k][ty * 4]);
            const float4 x4 = *reinterpret_cast<const float4*>(&sXh[k][tx * 4]);
            const float a[4] = {a4.x, a4.y, a4.z, a4.w};
            const float x[4] = {x4.x, x4.y, x4.z, x4.w};
            if (MODE == 0) {
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) s[i][j] = fmaf(a[i], x[j], s[i][j]);
            } else {
                const float4 al4 = *reinterpret_cast<const float4*>(&sAl[k][ty * 4]);
                const float4 xl4 = *reinterpret_cast<const float4*>(&sXl[k][tx * 4]);
                const float al[4] = {al4.x, al4.y, al4.z, al4.w};
                const float xl[4] = {xl4.x, xl4.y, xl4.z, xl4.w};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float p = __fmul_rn(a[i], x[j]);
                        const float e = __fmaf_rn(a[i], x[j], -p);  // exact product error
                        const float sn = __fadd_rn(s[i][j], p);
                        const float bp = __fsub_rn(sn, s[i][j]);
                        const float q = __fadd_rn(__fsub_rn(s[i][j], __fsub_rn(sn, bp)),
                                                  __fsub_rn(p, bp));  // exact sum error
                        s[i][j] = sn;
                        float tt = __fadd_rn(t[i][j], __fadd_rn(q, e));
                        tt = __fmaf_rn(a[i], xl[j], tt);
                        t[i][j] = __fmaf_rn(al[i], x[j], tt);
                    }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int row = row0 + ty * 4 + i, cc = c0 + tx * 4 + j;
            if (row < D && cc < C) {
                const double v =
                    MODE == 0 ? (double)s[i][j] : -((double)s[i][j] + (double)t[i][j]);
                partial[((size_t)blockIdx.z * C + cc) * D + row] = v;
            }
        }
}

// ---------------------------------------------------------------------------
// History vectors and state update
// ---------------------------------------------------------------------------

// Combined history vectors of all cases for step s (histories [step][case][dof]):
// W_f[c] = a1 x_c^{s+1-f} [f>=2] + a3 x_c^{s-f} [f>=1] + a2 x_c^{s-1-f} - a1 x_c^{s-1} [f=0]
//          + c0 (f=0) / c1 (f=1) x the known part of case c's load at step s.
__global__ void k_build_w_batch(const double* __restrict__ u_hist,
                                const double* __restrict__ t_hist, int D, int C, int s, int nlev,
                                double a1, double a2, double a3, double c0, double c1,
                                const double* __restrict__ amp, int numstep,
                                const double* __restrict__ traction,
                                const unsigned char* __restrict__ is_u,
                                const double* __restrict__ ubc_val, int ldw,
                                float* __restrict__ Wt, float* __restrict__ Wu) {
    const size_t total = (size_t)nlev * C * ldw;
    const size_t cs = (size_t)C * D;  // one history step of all cases
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % ldw);
        const int c = (int)((idx / ldw) % C);
        const int f = (int)(idx / ((size_t)ldw * C));
        double wt = 0, wu = 0;
        if (k < D) {
            const size_t o = (size_t)c * D + k;
            const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
            if (f >= 2 && m1 >= 1) {
                wt += a1 * t_hist[m1 * cs + o];
                wu += a1 * u_hist[m1 * cs + o];
            }
            if (f >= 1 && m3 >= 1) {
                wt += a3 * t_hist[m3 * cs + o];
                wu += a3 * u_hist[m3 * cs + o];
            }
            if (m2 >= 1) {
                wt += a2 * t_hist[m2 * cs + o];
                wu += a2 * u_hist[m2 * cs + o];
            }
            if (f <= 1) {
                const double cf = f == 0 ? c0 : c1;
                if (f == 0 && s - 1 >= 1) {
                    wt -= a1 * t_hist[(size_t)(s - 1) * cs + o];
                    wu -= a1 * u_hist[(size_t)(s - 1) * cs + o];
                }
                const double a = amp ? amp[(size_t)c * numstep + s] : 1.0;
                if (is_u[k]) wu += cf * ubc_val[k];
                else wt += cf * (a * traction[o]);
            }
        }
        Wt[idx] = (float)wt;
        Wu[idx] = (float)wu;
    }
}

// State update of all cases (SolverStepLinearT.cpp:512-535 per case).
__global__ void k_update_batch(const double* __restrict__ x, int D, int C, int s,
                               const unsigned char* __restrict__ is_u,
                               const double* __restrict__ ubc_val,
                               const double* __restrict__ traction,
                               const double* __restrict__ amp, int numstep,
                               double* __restrict__ u_hist, double* __restrict__ t_hist) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= C * D) return;
    const int c = idx / D, j = idx % D;
    const size_t o = (size_t)s * C * D + idx;
    const bool u = is_u[j] != 0;
    u_hist[o] = u ? ubc_val[j] : x[idx];
    const double a = amp ? amp[(size_t)c * numstep + s] : 1.0;
    double tv = a * traction[idx];
    if (u && j < D - 1) tv = x[idx];
    t_hist[o] = tv;
}

}  // namespace

int batch_block_cases() { return BN; }
int batch_ldw(int D) { return (D + BK - 1) / BK * BK; }

int batch_conv_splits(int nlev, int D, int C) {
    const int tiles = (D + BM - 1) / BM * ((C + BN - 1) / BN);
    const int splits = (2 * 152 + tiles - 1) / tiles;
    return std::max(1, std::min(splits, nlev));
}

int batch_apply_splits(int D, int C) {
    const int tiles = (D + TM - 1) / TM * ((C + TN - 1) / TN);
    const int want = (2 * 152 + tiles - 1) / tiles;
    const int kper = ((D + want - 1) / want + TK - 1) / TK * TK;
    return (D + kper - 1) / kper;  // splits actually used, every one non-empty
}

cudaError_t launch_conv_mma(const float* G, const float* H, size_t lstride, int ld, int D,
                            int nlev, const float* Wt, const float* Wu, int ldw, int C,
                            double* partial, int splits, cudaStream_t s) {
    if (ld % 4 != 0 || ldw % BK != 0 || (ld + BK - 1) / BK * BK > ldw || lstride % 4 != 0 ||
        splits < 1)
        return cudaErrorInvalidValue;
    const int per = (nlev + splits - 1) / splits;
    dim3 grid((D + BM - 1) / BM, splits, (C + BN - 1) / BN);
    k_conv_mma<<<grid, 256, 0, s>>>(G, H, lstride, ld, D, nlev, per, Wt, Wu, ldw, C, partial);
    return cudaGetLastError();
}

cudaError_t launch_apply_cols(const void* A, int fp64_residual, int D, const double* X, int C,
                              double* partial, int splits, cudaStream_t s) {
    if (splits < 1) return cudaErrorInvalidValue;
    const int kper = ((D + splits - 1) / splits + TK - 1) / TK * TK;
    const int nz = (D + kper - 1) / kper;
    if (nz != splits) return cudaErrorInvalidValue;  // splits from batch_apply_splits
    dim3 grid((D + TM - 1) / TM, (C + TN - 1) / TN, nz);
    if (fp64_residual)
        k_apply_cols<1><<<grid, 256, 0, s>>>(A, D, X, C, kper, partial);
    else
        k_apply_cols<0><<<grid, 256, 0, s>>>(A, D, X, C, kper, partial);
    return cudaGetLastError();
}

cudaError_t launch_build_w_batch(const double* u_hist, const double* t_hist, int D, int C, int s,
                                 int nlev, double a1, double a2, double a3, double c0, double c1,
                                 const double* amp, int numstep, const double* traction,
                                 const unsigned char* is_u, const double* ubc_val, int ldw,
                                 float* Wt, float* Wu, cudaStream_t st) {
    const size_t total = (size_t)nlev * C * ldw;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 16384);
    k_build_w_batch<<<grid, 256, 0, st>>>(u_hist, t_hist, D, C, s, nlev, a1, a2, a3, c0, c1, amp,
                                          numstep, traction, is_u, ubc_val, ldw, Wt, Wu);
    return cudaGetLastError();
}

cudaError_t launch_update_batch(const double* x, int D, int C, int s, const unsigned char* is_u,
                                const double* ubc_val, const double* traction,
                                const double* amp, int numstep, double* u_hist, double* t_hist,
                                cudaStream_t st) {
    k_update_batch<<<(C * D + 255) / 256, 256, 0, st>>>(x, D, C, s, is_u, ubc_val, traction, amp,
                                                        numstep, u_hist, t_hist);
    return cudaGetLastError();
}

}  // namespace tdbem
