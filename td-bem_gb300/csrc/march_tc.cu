// Mixed march on the tcgen05 tensor cores: one merged level matrix per level.
//
// At every dof one of (u_j, t_j) is prescribed and the other is the unknown
// x_j of the step's solve; the state update (march.cu: k_update_state) writes
//   u_j = ubc_j,            t_j = x_j                 dof with a prescribed
//                                                      displacement, j < D-1
//   u_j = x_j,              t_j = fbc_j amp(m) or 0   every other dof
// and, for the last dof with a prescribed displacement, u = ubc and t = fbc amp
// or 0 (the reference's ExtractField leaves it out of its loop).  A history term
// G^f wt - H^f wu of the march therefore splits, column by column, into
//   A^f w   with A^f[:, j] = G^f[:, j] (t_j unknown), -H^f[:, j] (u_j unknown),
//           0 (the last dof above), and w the same combination of x's history,
// plus the known values' part, a scalar times one of three vectors per level:
//   pt_f = G^f kt   kt_j = fbc_j where t_j is known and prescribed (history),
//   pl_f = G^f lt   lt_j = fbc_j at the dofs without a prescribed displacement
//                   (the step's own load, the known-load terms of levels 0/1),
//   pu_f = H^f lu   lu_j = ubc_j.
// The convolution streams A^f (BF16 hi/lo planes, half the bytes of G^f and
// H^f); the known part is a sum over levels of those vectors with coefficients
// tabulated per step from the load history.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

// Column selector of A^f: 1 = G (t unknown), 2 = -H (u unknown), 0 = none.
__device__ __forceinline__ int col_sel(const unsigned char* __restrict__ is_u, int k, int D) {
    if (k >= D) return 0;
    if (is_u[k]) return k < D - 1 ? 1 : 0;
    return 2;
}

// FP32 levels [f][row][ldf] -> merged planes [plane*slabs + f][row][ldb] and the
// known part's vectors known[(v*L + f)*D + row], v = 0 pt, 1 pl, 2 pu.  Warp per
// (f, row), 4 columns per lane (16-byte loads of G and H, 8-byte stores per
// plane); FP32 products, FP64 warp sums.
__global__ void __launch_bounds__(256) k_merge_levels(
    const float* __restrict__ Gf, const float* __restrict__ Hf, int ldf, int D, int L, int slabs,
    int ldb, const unsigned char* __restrict__ is_u, const float* __restrict__ kt,
    const float* __restrict__ lt, const float* __restrict__ lu, __nv_bfloat16* __restrict__ P,
    double* __restrict__ known) {
    const size_t rows = (size_t)L * D;
    const size_t plane = (size_t)slabs * D * ldb;
    const int lane = threadIdx.x & 31;
    const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t fr = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); fr < rows;
         fr += nwarps) {
        const float* g = Gf + fr * ldf;
        const float* h = Hf + fr * ldf;
        __nv_bfloat16* hi_row = P + fr * ldb;
        __nv_bfloat16* lo_row = P + plane + fr * ldb;
        float st = 0.f, sl = 0.f, su = 0.f;
        for (int k = 4 * lane; k < ldb; k += 128) {
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f), y = x;
            if (k < ldf) {
                x = __ldcs(reinterpret_cast<const float4*>(g + k));
                y = __ldcs(reinterpret_cast<const float4*>(h + k));
            }
            const float gv[4] = {x.x, x.y, x.z, x.w}, hv[4] = {y.x, y.y, y.z, y.w};
            __align__(8) __nv_bfloat16 hb[4], lb[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int c = k + q;
                const int sel = col_sel(is_u, c, D);
                const float a = sel == 1 ? gv[q] : sel == 2 ? -hv[q] : 0.f;
                hb[q] = __float2bfloat16_rn(a);
                lb[q] = __float2bfloat16_rn(__fsub_rn(a, __bfloat162float(hb[q])));
                if (c < D) {
                    st = fmaf(gv[q], kt[c], st);
                    sl = fmaf(gv[q], lt[c], sl);
                    su = fmaf(hv[q], lu[c], su);
                }
            }
            *reinterpret_cast<uint2*>(hi_row + k) = *reinterpret_cast<const uint2*>(hb);
            *reinterpret_cast<uint2*>(lo_row + k) = *reinterpret_cast<const uint2*>(lb);
        }
        double v[3] = {st, sl, su};
#pragma unroll
        for (int i = 0; i < 3; i++)
            for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
        if (lane < 3) {
            const size_t f = fr / D, row = fr - f * D;
            known[((size_t)lane * L + f) * D + row] = lane == 0 ? v[0] : lane == 1 ? v[1] : v[2];
        }
    }
}

// Step-distance matrices B_d (d = 1 .. kStepMats) into slabs M + d of the planes:
//   B_1 = (a2 - a1) A^0 + a3 A^1 + a1 A^2,   B_d = a2 A^(d-1) + a3 A^d + a1 A^(d+1)
// (A^f = 0 beyond level M), the weights with which w_of combines the history of
// step m into level f of step m + d.  Warp per row, 4 columns per lane: the lane
// walks levels 0 .. kStepMats + 1 with the last two merged values kept, so every
// level is read once; FP32 sums of the FP32 levels, then the BF16 hi/lo split.
__global__ void __launch_bounds__(256) k_step_mats(
    const float* __restrict__ Gf, const float* __restrict__ Hf, int ldf, int D, int M, int slabs,
    int ldb, const unsigned char* __restrict__ is_u, float a1, float a2, float a3,
    __nv_bfloat16* __restrict__ P) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= D) return;
    const size_t plane = (size_t)slabs * D * ldb;
    const size_t lstride = (size_t)D * ldf;
    for (int k = 4 * lane; k < ldb; k += 128) {
        int sel[4];
#pragma unroll
        for (int q = 0; q < 4; q++) sel[q] = col_sel(is_u, k + q, D);
        float am2[4] = {0.f, 0.f, 0.f, 0.f}, am1[4] = {0.f, 0.f, 0.f, 0.f};
        for (int f = 0; f <= kStepMats + 1; f++) {
            float a[4] = {0.f, 0.f, 0.f, 0.f};
            if (f <= M && k < ldf) {
                const float4 x =
                    __ldcs(reinterpret_cast<const float4*>(Gf + f * lstride + (size_t)row * ldf + k));
                const float4 y =
                    __ldcs(reinterpret_cast<const float4*>(Hf + f * lstride + (size_t)row * ldf + k));
                const float gv[4] = {x.x, x.y, x.z, x.w}, hv[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                for (int q = 0; q < 4; q++)
                    a[q] = sel[q] == 1 ? gv[q] : sel[q] == 2 ? -hv[q] : 0.f;
            }
            if (f >= 2) {  // B_(f-1) from levels f - 2, f - 1, f
                const int d = f - 1;
                const float c0 = d == 1 ? a2 - a1 : a2;
                __align__(8) __nv_bfloat16 hb[4], lb[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float b = fmaf(c0, am2[q], fmaf(a3, am1[q], a1 * a[q]));
                    hb[q] = __float2bfloat16_rn(b);
                    lb[q] = __float2bfloat16_rn(__fsub_rn(b, __bfloat162float(hb[q])));
                }
                const size_t off = ((size_t)(M + d) * D + row) * ldb + k;
                *reinterpret_cast<uint2*>(P + off) = *reinterpret_cast<const uint2*>(hb);
                *reinterpret_cast<uint2*>(P + plane + off) = *reinterpret_cast<const uint2*>(lb);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                am2[q] = am1[q];
                am1[q] = a[q];
            }
        }
    }
}

// History planes of the step-distance matrices for the steps b + j (j < ncol) from
// the history steps [a, b): slab d - 1, column j holds the unknowns' history
// x_(b + j - d) (t where t is the unknown, u where u is; zero beyond D and outside
// [a, b)).  Columns ncol..Cpad-1 are left as they are.  Grid (K tiles, ncol, nmats).
__global__ void __launch_bounds__(256) k_build_w_steps(
    const double* __restrict__ u_hist, const double* __restrict__ t_hist,
    const unsigned char* __restrict__ is_u, int D, int a, int b, int Cpad, int Lw, int ldb,
    __nv_bfloat16* __restrict__ W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, d = blockIdx.z + 1;
    if (k >= ldb) return;
    const int m = b + j - d;
    double w = 0;
    const int sel = col_sel(is_u, k, D);
    if (sel && m >= a && m < b) w = (sel == 1 ? t_hist : u_hist)[(size_t)m * D + k];
    const size_t idx = ((size_t)(d - 1) * Cpad + j) * ldb + k;
    const size_t plane = (size_t)Lw * Cpad * ldb;
    const __nv_bfloat16 h = __float2bfloat16_rn((float)w);
    W[idx] = h;
    W[plane + idx] = __float2bfloat16_rn((float)(w - (double)__bfloat162float(h)));
}

// x's history combination of level f for step s over history steps [lo, hi)
// (the W terms of march_mixed.cu's k_build_w_old / k_build_w_cross).
__device__ __forceinline__ double w_of(const double* __restrict__ hist, int D, int k, int s,
                                       int f, int lo, int hi, double a1, double a2, double a3) {
    double w = 0;
    const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
    if (f >= 2 && m1 >= lo && m1 < hi) w += a1 * hist[(size_t)m1 * D + k];
    if (f >= 1 && m3 >= lo && m3 < hi) w += a3 * hist[(size_t)m3 * D + k];
    if (m2 >= lo && m2 < hi) w += a2 * hist[(size_t)m2 * D + k];
    if (f == 0 && s - 1 >= lo && s - 1 < hi) w -= a1 * hist[(size_t)(s - 1) * D + k];
    return w;
}

// Merged history vectors [plane*Lw + f][j][ldb] of the steps s0 + j (j < ncol,
// zero beyond D) over history steps [lo, hi).  Columns ncol..Cpad-1 are left as
// they are: the product's output columns are independent and those are not read.
// Grid (K tiles, ncol, nlev).
__global__ void __launch_bounds__(256) k_build_w_merged(
    const double* __restrict__ u_hist, const double* __restrict__ t_hist,
    const unsigned char* __restrict__ is_u, int D, int s0, int Cpad, int lo, int hi, int Lw,
    double a1, double a2, double a3, int ldb, __nv_bfloat16* __restrict__ W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, f = blockIdx.z;
    if (k >= ldb) return;
    double w = 0;
    const int sel = col_sel(is_u, k, D);
    if (sel) w = w_of(sel == 1 ? t_hist : u_hist, D, k, s0 + j, f, lo, hi, a1, a2, a3);
    const size_t idx = ((size_t)f * Cpad + j) * ldb + k;
    const size_t plane = (size_t)Lw * Cpad * ldb;
    const __nv_bfloat16 h = __float2bfloat16_rn((float)w);
    W[idx] = h;
    W[plane + idx] = __float2bfloat16_rn((float)(w - (double)__bfloat162float(h)));
}

// Known part of the right-hand sides of every solve step, once per march:
// Yk[s][row] = sum_f ( ct pt_f + cl pl_f - cu pu_f )[row] with (ct, cl, cu) =
// coef[s * L + f], for the steps s = 1 + blockIdx.y * nbs + j (j < nbs, s <= last).
// Thread per row.
constexpr int kKnownMaxSteps = 16;
__global__ void __launch_bounds__(128) k_known_terms(const double* __restrict__ known,
                                                     const double3* __restrict__ coef, int D,
                                                     int L, int nbs, int last,
                                                     double* __restrict__ Yk) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int S = 1 + blockIdx.y * nbs;
    const int nbe = min(nbs, last - S + 1);
    if (row >= D || nbe < 1) return;
    double acc[kKnownMaxSteps];
#pragma unroll
    for (int j = 0; j < kKnownMaxSteps; j++) acc[j] = 0;
    const int flast = min(L - 1, S + nbe - 1);
    for (int f = 0; f <= flast; f++) {
        const double pt = known[(size_t)f * D + row];
        const double pl = known[((size_t)L + f) * D + row];
        const double pu = known[((size_t)2 * L + f) * D + row];
#pragma unroll
        for (int j = 0; j < kKnownMaxSteps; j++)
            if (j < nbe) {
                const double3 c = coef[(size_t)(S + j) * L + f];
                acc[j] += c.x * pt + c.y * pl - c.z * pu;
            }
    }
#pragma unroll
    for (int j = 0; j < kKnownMaxSteps; j++)
        if (j < nbe) Yk[(size_t)(S + j) * D + row] = acc[j];
}

// Batched form ([step][case][dof] histories): the merged history vectors of all
// cases for step s over history steps [1, s), planes [plane*Lw + f][c][ldb].
__global__ void __launch_bounds__(256) k_build_w_batch_merged(
    const double* __restrict__ u_hist, const double* __restrict__ t_hist,
    const unsigned char* __restrict__ is_u, int D, int C, int Cpad, int s, int Lw, double a1,
    double a2, double a3, int ldb, __nv_bfloat16* __restrict__ W) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y, f = blockIdx.z;
    if (k >= ldb) return;
    double w = 0;
    const int sel = col_sel(is_u, k, D);
    if (sel) {
        const double* h = (sel == 1 ? t_hist : u_hist) + (size_t)c * D;  // [m][c][k]
        w = w_of(h, C * D, k, s, f, 1, s, a1, a2, a3);
    }
    const size_t idx = ((size_t)f * Cpad + c) * ldb + k;
    const size_t plane = (size_t)Lw * Cpad * ldb;
    const __nv_bfloat16 hb = __float2bfloat16_rn((float)w);
    W[idx] = hb;
    W[plane + idx] = __float2bfloat16_rn((float)(w - (double)__bfloat162float(hb)));
}

// Known tractions of the batched cases as FP32 columns [c][D]: kt (history: every dof
// but a prescribed-displacement dof below D-1) and lt (the step's own load: the dofs
// without a prescribed displacement).
__global__ void k_batch_known_tractions(const double* __restrict__ trac,
                                        const unsigned char* __restrict__ is_u, int D, int C,
                                        float* __restrict__ kt, float* __restrict__ lt) {
    const size_t n = (size_t)C * D;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(i % D);
        const float v = (float)trac[i];
        kt[i] = (is_u[j] && j < D - 1) ? 0.f : v;
        lt[i] = is_u[j] ? 0.f : v;
    }
}

// Batched right-hand sides of step s, Y[c][row] += the known values' part:
// sum_f ( ct_c GK[f][c][row] + cl_c GL[f][c][row] (f <= 1) - cu HU[f][row] ) with the
// coefficients of known_coefficients, case c's amplitude amp[c][m] (or 1).
__global__ void __launch_bounds__(128) k_known_batch(const float* __restrict__ GK,
                                                     const float* __restrict__ GL,
                                                     const double* __restrict__ HU, int D, int C,
                                                     int L, int s, double a1, double a2,
                                                     double a3, double c0, double c1,
                                                     const double* __restrict__ amp,
                                                     int numstep, double* __restrict__ Y) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (row >= D) return;
    auto A = [&](int m) { return amp ? amp[(size_t)c * numstep + m] : 1.0; };
    double acc = 0;
    const int flast = min(L - 1, s);
    for (int f = 0; f <= flast; f++) {
        double ct = 0, cu = 0;
        auto term = [&](int m, double w) {
            if (m >= 1 && m <= s - 1) {
                ct += w * A(m);
                cu += w;
            }
        };
        if (f >= 2) term(s + 1 - f, a1);
        if (f >= 1) term(s - f, a3);
        term(s - 1 - f, a2);
        if (f == 0) term(s - 1, -a1);
        double v = ct * (double)GK[((size_t)f * C + c) * D + row];
        if (f <= 1) {
            const double cf = f == 0 ? c0 : c1;
            v += cf * A(s) * (double)GL[((size_t)f * C + c) * D + row];
            cu += cf;
        }
        acc += v - cu * HU[(size_t)f * D + row];
    }
    Y[(size_t)c * D + row] += acc;
}

}  // namespace

cudaError_t launch_build_w_batch_merged(const double* u_hist, const double* t_hist,
                                        const unsigned char* is_u, int D, int C, int s,
                                        int nlev, int Lw, double a1, double a2, double a3,
                                        void* W, cudaStream_t st) {
    if (C < 1 || nlev < 1 || nlev > Lw) return cudaErrorInvalidValue;
    const int Cpad = tc_cases_pad(C), ldb = tc_ldb(D);
    const dim3 grid((ldb + 255) / 256, C, nlev);
    k_build_w_batch_merged<<<grid, 256, 0, st>>>(u_hist, t_hist, is_u, D, C, Cpad, s, Lw, a1,
                                                 a2, a3, ldb, static_cast<__nv_bfloat16*>(W));
    return cudaGetLastError();
}

cudaError_t launch_batch_known_tractions(const double* trac, const unsigned char* is_u, int D,
                                         int C, float* kt, float* lt, cudaStream_t s) {
    k_batch_known_tractions<<<1216, 256, 0, s>>>(trac, is_u, D, C, kt, lt);
    return cudaGetLastError();
}

cudaError_t launch_known_batch(const float* GK, const float* GL, const double* HU, int D, int C,
                               int L, int s, double a1, double a2, double a3, double c0,
                               double c1, const double* amp, int numstep, double* Y,
                               cudaStream_t st) {
    const dim3 grid((D + 127) / 128, C);
    k_known_batch<<<grid, 128, 0, st>>>(GK, GL, HU, D, C, L, s, a1, a2, a3, c0, c1, amp,
                                        numstep, Y);
    return cudaGetLastError();
}

cudaError_t launch_merge_levels(const float* Gf, const float* Hf, int ldf, int D, int L,
                                int slabs, const unsigned char* is_u, const float* kt,
                                const float* lt, const float* lu, void* planes, double* known,
                                cudaStream_t s) {
    const int ldb = tc_ldb(D);
    if (ldf % 4 != 0 || ldf > ldb || slabs < L) return cudaErrorInvalidValue;
    const size_t rows = (size_t)L * D;
    const unsigned grid = (unsigned)std::min<size_t>((rows + 7) / 8, 152 * 8);
    k_merge_levels<<<grid, 256, 0, s>>>(Gf, Hf, ldf, D, L, slabs, ldb, is_u, kt, lt, lu,
                                        static_cast<__nv_bfloat16*>(planes), known);
    return cudaGetLastError();
}

cudaError_t launch_step_mats(const float* Gf, const float* Hf, int ldf, int D, int M, int slabs,
                             const unsigned char* is_u, double a1, double a2, double a3,
                             void* planes, cudaStream_t s) {
    const int ldb = tc_ldb(D);
    if (ldf % 4 != 0 || ldf > ldb || slabs < M + 1 + kStepMats) return cudaErrorInvalidValue;
    k_step_mats<<<(D + 7) / 8, 256, 0, s>>>(Gf, Hf, ldf, D, M, slabs, ldb, is_u, (float)a1,
                                            (float)a2, (float)a3,
                                            static_cast<__nv_bfloat16*>(planes));
    return cudaGetLastError();
}

cudaError_t launch_build_w_steps(const double* u_hist, const double* t_hist,
                                 const unsigned char* is_u, int D, int a, int b, int ncol,
                                 int Cmax, int nmats, int Lw, void* W, cudaStream_t st) {
    if (ncol < 1 || ncol > Cmax || nmats < 1 || nmats > Lw || nmats > kStepMats)
        return cudaErrorInvalidValue;
    const int Cpad = tc_cases_pad(Cmax), ldb = tc_ldb(D);
    const dim3 grid((ldb + 255) / 256, ncol, nmats);
    k_build_w_steps<<<grid, 256, 0, st>>>(u_hist, t_hist, is_u, D, a, b, Cpad, Lw, ldb,
                                          static_cast<__nv_bfloat16*>(W));
    return cudaGetLastError();
}

cudaError_t launch_build_w_merged(const double* u_hist, const double* t_hist,
                                  const unsigned char* is_u, int D, int s0, int ncol, int Cmax,
                                  int lo, int hi, int nlev, int Lw, double a1, double a2,
                                  double a3, void* W, cudaStream_t st) {
    if (ncol < 1 || ncol > Cmax || nlev < 1 || nlev > Lw) return cudaErrorInvalidValue;
    const int Cpad = tc_cases_pad(Cmax), ldb = tc_ldb(D);
    const dim3 grid((ldb + 255) / 256, ncol, nlev);
    k_build_w_merged<<<grid, 256, 0, st>>>(u_hist, t_hist, is_u, D, s0, Cpad, lo, hi, Lw, a1, a2,
                                           a3, ldb, static_cast<__nv_bfloat16*>(W));
    return cudaGetLastError();
}

cudaError_t launch_known_terms(const double* known, const void* coef, int D, int L, int last,
                               double* Yk, cudaStream_t s) {
    if (last < 1) return cudaSuccess;
    const int nbs = kKnownMaxSteps;
    const dim3 grid((D + 127) / 128, (last + nbs - 1) / nbs);
    k_known_terms<<<grid, 128, 0, s>>>(known, static_cast<const double3*>(coef), D, L, nbs, last,
                                       Yk);
    return cudaGetLastError();
}

// Coefficients (ct, cl, cu) of the known part for the solve steps 1..numstep-1 and
// levels 0..L-1 (zero for step 0 and numstep; see the header): the history terms of
// the W combination with m >= 1, amp(m) on the prescribed tractions, 1 on the
// prescribed displacements, and the step's own load with lhs_c0/lhs_c1 at levels 0/1
// (step 1: 1 and 0).  amp: empty (unit load) or at least numstep values.
void known_coefficients(int numstep, int L, double a1, double a2, double a3,
                        const std::vector<double>& amp, double c0, double c1,
                        std::vector<double>& out) {
    out.assign((size_t)(numstep + 1) * L * 3, 0.0);
    auto A = [&](int m) { return amp.empty() ? 1.0 : amp[m]; };
    for (int s = 1; s <= numstep - 1; s++)
        for (int f = 0; f < L && f <= s; f++) {
            double ct = 0, cu = 0;
            auto term = [&](int m, double w) {
                if (m >= 1 && m <= s - 1) {
                    ct += w * A(m);
                    cu += w;
                }
            };
            if (f >= 2) term(s + 1 - f, a1);
            if (f >= 1) term(s - f, a3);
            term(s - 1 - f, a2);
            if (f == 0) term(s - 1, -a1);
            double cl = 0;
            if (f <= 1) {
                const double cf = f == 0 ? (s == 1 ? 1.0 : c0) : (s == 1 ? 0.0 : c1);
                cl = cf * A(s);
                cu += cf;
            }
            double* o = &out[((size_t)s * L + f) * 3];
            o[0] = ct;
            o[1] = cl;
            o[2] = cu;
        }
}

}  // namespace tdbem
