// Time marching on sm_103a: the history convolution and the H^0 solve of
// SolverStepLinearT::Solve_Averaging (SolverStepLinearT.cpp:314-544).
//
// Per step s the reference forms rhs = G_c load + a sum of level matvecs with
// weights a1, a2, a3 = 1 - a1 - a2 on the histories.  Every level f appears in
// that sum with one combination of history vectors,
//     w_f = a1 x^{s+1-f} [f>=2] + a3 x^{s-f} [f>=1] + a2 x^{s-1-f} - a1 x^{s-1} [f=0]
// (x^m = 0 for m <= 0: the initial state and the fG_DB_bgn terms multiply zero),
// and G_c load = sum over levels 0/1 of the column-exchanged LHS weights times
// the known traction / displacement parts of the load.  So one pass over each
// stored level with its combined vector computes the whole right-hand side:
//     rhs = sum_f (G^f W_t[f] - H^f W_u[f]).
// The solve uses the inverse of the column-exchanged LHS (ExchangeColumns,
// SolverT.cpp:265-342), computed once per distinct LHS (inverse.cu).
#include <algorithm>

#include "state_update.cuh"
#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

__global__ void k_build_lhs(const double* __restrict__ G, const double* __restrict__ H,
                            const float* __restrict__ Gf, const float* __restrict__ Hf,
                            size_t stride, int D, double c0, double c1,
                            const unsigned char* __restrict__ is_ubc, double* __restrict__ A) {
    const size_t n = (size_t)D * D;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % D);
        double g0, g1, h0, h1;
        if (G) {
            g0 = G[idx]; g1 = G[stride + idx]; h0 = H[idx]; h1 = H[stride + idx];
        } else {
            g0 = Gf[idx]; g1 = Gf[stride + idx]; h0 = Hf[idx]; h1 = Hf[stride + idx];
        }
        // (0 + c0 X0) + c1 X1 as MatAXPY on a zeroed matrix; UBC columns swapped and negated
        const double gc = c0 * g0 + c1 * g1;
        const double hc = c0 * h0 + c1 * h1;
        A[idx] = is_ubc[j] ? -1 * gc : hc;
    }
}

__global__ void k_history_combine(const double* __restrict__ u_hist,
                                  const double* __restrict__ t_hist, int D, int s, int L,
                                  double a1, double a2, double a3, double c0, double c1, double amp,
                                  const double* __restrict__ load_t,
                                  const double* __restrict__ load_u, double* __restrict__ Wt,
                                  double* __restrict__ Wu) {
    const size_t total = (size_t)(L + 1) * D;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int f = (int)(idx / D), j = (int)(idx % D);
        double wt = 0, wu = 0;
        const int m1 = s + 1 - f, m3 = s - f, m2 = s - 1 - f;
        if (f >= 2 && m1 >= 1) {
            wt += a1 * t_hist[(size_t)m1 * D + j];
            wu += a1 * u_hist[(size_t)m1 * D + j];
        }
        if (f >= 1 && m3 >= 1) {
            wt += a3 * t_hist[(size_t)m3 * D + j];
            wu += a3 * u_hist[(size_t)m3 * D + j];
        }
        if (m2 >= 1) {
            wt += a2 * t_hist[(size_t)m2 * D + j];
            wu += a2 * u_hist[(size_t)m2 * D + j];
        }
        if (f == 0) {
            if (s - 1 >= 1) {
                wt -= a1 * t_hist[(size_t)(s - 1) * D + j];
                wu -= a1 * u_hist[(size_t)(s - 1) * D + j];
            }
            wt += c0 * (amp * load_t[j]);
            wu += c0 * load_u[j];
        } else if (f == 1) {
            wt += c1 * (amp * load_t[j]);
            wu += c1 * load_u[j];
        }
        Wt[idx] = wt;
        Wu[idx] = wu;
    }
}

constexpr int kConvRowsPerWarp = 4;
constexpr int kConvWarps = 8;
constexpr int kConvRows = kConvRowsPerWarp * kConvWarps;

// partial[chunk][row] = sum_{f in chunk} (G^f[row,:] . Wt[f] - H^f[row,:] . Wu[f]).
// Each warp streams 4 rows of a level with 16-byte loads; the vectors come
// through L1/L2 and are shared by the 4 rows.
template <typename T>
__global__ void __launch_bounds__(256) k_conv(const T* __restrict__ G, const T* __restrict__ H,
                                              size_t stride, int D, int L, int per_chunk,
                                              const double* __restrict__ Wt,
                                              const double* __restrict__ Wu,
                                              double* __restrict__ partial) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kConvRows + warp * kConvRowsPerWarp;
    const int f0 = blockIdx.y * per_chunk;
    const int f1 = min(L, f0 + per_chunk - 1);
    double acc[kConvRowsPerWarp] = {0, 0, 0, 0};
    int rows[kConvRowsPerWarp];
#pragma unroll
    for (int r = 0; r < kConvRowsPerWarp; r++) rows[r] = min(row0 + r, D - 1);
    const bool even = (D % 2) == 0;
    for (int f = f0; f <= f1; f++) {
        const T* Gf = G + (size_t)f * stride;
        const T* Hf = H + (size_t)f * stride;
        const double* wt = Wt + (size_t)f * D;
        const double* wu = Wu + (size_t)f * D;
        if (even && sizeof(T) == 8) {
            for (int j = 2 * lane; j < D; j += 64) {
                const double2 vt = *reinterpret_cast<const double2*>(wt + j);
                const double2 vu = *reinterpret_cast<const double2*>(wu + j);
#pragma unroll
                for (int r = 0; r < kConvRowsPerWarp; r++) {
                    const size_t o = (size_t)rows[r] * D + j;
                    const double2 g = __ldcs(reinterpret_cast<const double2*>(Gf + o));
                    const double2 h = __ldcs(reinterpret_cast<const double2*>(Hf + o));
                    acc[r] += g.x * vt.x + g.y * vt.y - h.x * vu.x - h.y * vu.y;
                }
            }
        } else {
            for (int j = lane; j < D; j += 32) {
                const double vt = wt[j], vu = wu[j];
#pragma unroll
                for (int r = 0; r < kConvRowsPerWarp; r++) {
                    const size_t o = (size_t)rows[r] * D + j;
                    acc[r] += (double)Gf[o] * vt - (double)Hf[o] * vu;
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kConvRowsPerWarp; r++) {
        double v = acc[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && row0 + r < D) partial[(size_t)blockIdx.y * D + row0 + r] = v;
    }
}

__global__ void k_reduce_partial(const double* __restrict__ partial, int nchunks, int D,
                                 double* __restrict__ rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D) return;
    double s = 0;
    for (int c = 0; c < nchunks; c++) s += partial[(size_t)c * D + i];
    rhs[i] = s;
}

// x = Ainv rhs, warp per row.
__global__ void __launch_bounds__(256) k_gemv(const double* __restrict__ A, int D,
                                              const double* __restrict__ v,
                                              double* __restrict__ x) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= D) return;
    const double* row = A + (size_t)warp * D;
    double acc = 0;
    for (int j = lane; j < D; j += 32) acc += __ldcs(row + j) * v[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[warp] = acc;
}

// u^s = x with prescribed values on UBC dofs; t^s = FBC*amp, and x on UBC dofs
// below the last dof (SolverStepLinearT.cpp:512-535).  ubc_val[j] / fbc_val[j] are
// per-dof maps with flags is_u / is_f (the last list entry of a dof wins).
__global__ void k_update_state(const double* __restrict__ x, int D, int s,
                               const unsigned char* __restrict__ is_u,
                               const double* __restrict__ ubc_val,
                               const unsigned char* __restrict__ is_f,
                               const double* __restrict__ fbc_val, double amp,
                               double* __restrict__ u_hist, double* __restrict__ t_hist) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= D) return;
    StateUpdate p;
    p.is_u = is_u;
    p.ubc = ubc_val;
    p.is_f = is_f;
    p.fbc = fbc_val;
    p.amp = amp;
    p.u_hist = u_hist;
    p.t_hist = t_hist;
    p.s = s;
    update_state_dof(p, D, j, x[j]);
}

__global__ void k_add_inplace(double* __restrict__ y, const double* __restrict__ x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        y[i] += x[i];
}

}  // namespace

cudaError_t launch_add_inplace(double* y, const double* x, size_t n, cudaStream_t s) {
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_add_inplace<<<grid, 256, 0, s>>>(y, x, n);
    return cudaGetLastError();
}

cudaError_t launch_build_lhs(const double* G, const double* H, const float* Gf,
                             const float* Hf, size_t level_stride, int D, double c0,
                             double c1, const unsigned char* is_ubc, double* A,
                             cudaStream_t s) {
    k_build_lhs<<<1216, 256, 0, s>>>(G, H, Gf, Hf, level_stride, D, c0, c1, is_ubc, A);
    return cudaGetLastError();
}

cudaError_t launch_history_combine(const double* u_hist, const double* t_hist, int D, int s,
                                   int L, double a1, double a2, double a3, double c0,
                                   double c1, double amp, const double* load_t,
                                   const double* load_u,
                                   double* Wt, double* Wu, cudaStream_t st) {
    const size_t total = (size_t)(L + 1) * D;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 4096);
    k_history_combine<<<grid, 256, 0, st>>>(u_hist, t_hist, D, s, L, a1, a2, a3, c0, c1,
                                            amp, load_t, load_u, Wt, Wu);
    return cudaGetLastError();
}

int conv_chunks(int L, int D) {
    const int tiles = (D + kConvRows - 1) / kConvRows;
    int chunks = (4 * 152 + tiles - 1) / tiles;
    return std::max(1, std::min(chunks, L + 1));
}

cudaError_t launch_conv(const MarchDev& md, int L, const double* Wt, const double* Wu,
                        double* partial, int nchunks, cudaStream_t s) {
    const int D = md.D;
    const int per_chunk = (L + 1 + nchunks - 1) / nchunks;
    dim3 grid((D + kConvRows - 1) / kConvRows, nchunks);
    const size_t stride = (size_t)D * D;
    if (md.G)
        k_conv<double><<<grid, 256, 0, s>>>(md.G, md.H, stride, D, L, per_chunk, Wt, Wu, partial);
    else
        k_conv<float><<<grid, 256, 0, s>>>(md.Gf, md.Hf, stride, D, L, per_chunk, Wt, Wu,
                                           partial);
    return cudaGetLastError();
}

cudaError_t launch_reduce_solve(const double* partial, int nchunks, int D, const double* Ainv,
                                double* rhs, double* x, cudaStream_t s) {
    k_reduce_partial<<<(D + 255) / 256, 256, 0, s>>>(partial, nchunks, D, rhs);
    k_gemv<<<(D * 32 + 255) / 256, 256, 0, s>>>(Ainv, D, rhs, x);
    return cudaGetLastError();
}

cudaError_t launch_reduce_partial(const double* partial, int nchunks, int D, double* rhs,
                                  cudaStream_t s) {
    k_reduce_partial<<<(D + 255) / 256, 256, 0, s>>>(partial, nchunks, D, rhs);
    return cudaGetLastError();
}

cudaError_t launch_gemv(const double* A, int D, const double* v, double* x, cudaStream_t s) {
    k_gemv<<<(D * 32 + 255) / 256, 256, 0, s>>>(A, D, v, x);
    return cudaGetLastError();
}

cudaError_t launch_update_state(const double* x, int D, int s, const unsigned char* is_u,
                                const double* ubc_val, const unsigned char* is_f,
                                const double* fbc_val, double amp, double* u_hist,
                                double* t_hist, cudaStream_t st) {
    k_update_state<<<(D + 255) / 256, 256, 0, st>>>(x, D, s, is_u, ubc_val, is_f, fbc_val, amp,
                                                    u_hist, t_hist);
    return cudaGetLastError();
}

}  // namespace tdbem
