// G^k / H^k level assembly on sm_103a (FP64 plain form and FP32 level store).
//
// Work decomposition.  The unit of work is one (collocation node c, element e,
// time level k) item.  For a pair (c, e) only the levels whose time window
// meets the P- or S-wave front crossing the element can be non-zero: the
// Heaviside response H(T) of GreenFunctionT::Stokes_Heaviside_Linear
// (GreenFunctionT.cpp:241-416) is exactly 0 for T < r/c_p (b = 0 for both waves)
// and constant for T - r/c_s >= dt (b = dt for both waves, I5 = I6 = 0), so the
// step response H(T) - H(T - dt) (Stokes_Step_Linear, GreenFunctionT.cpp:424-446)
// vanishes outside  r/(c_p dt) <= n < r/(c_s dt) + 2.  A window kernel bounds r
// over the element with its bounding sphere, a scan turns the per-pair level
// counts into item offsets, and one thread per item integrates all Gauss points
// of the element for its level.  Levels outside every window stay exactly zero
// (the reference stores round-off noise there).
//
// Level placement follows main.cpp:89-121 + SolverStepLinearT::UpdateGHLinear
// (SolverStepLinearT.cpp:58-97): level k = I(k dt) + J((k+1) dt), so one item
// sums the I part at time k dt and the J part at time (k+1) dt before the
// scatter, halving the scatter traffic.
//
// Determinism.  Elements are coloured so that no two elements of a colour share
// a node; one launch per colour, so every level entry receives at most one
// read-modify-write per launch and the result does not depend on scheduling.
//
// Arithmetic.  The time integrals are the reference's closed forms
// (GreenFunctionT.cpp:251-314) in Horner form; the 3x3 kernels are written as
// DU = A r r^T + B I and DT = alpha rdn r r^T + beta n r^T + gamma (r n^T + rdn I)
// (GreenFunctionT.cpp:332-406 with the s1..s5 terms collected), so an item does
// the per-level work with ~300 FP64 operations per Gauss point.
#include <cub/device/device_scan.cuh>

#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

constexpr int kGeomStride = 12;   // Q4: x[3], n[3], wJ, N[4], pad
constexpr int kGeomStride8 = 16;  // Q8: x[3], n[3], wJ, N[8], pad

// ShapeFunctionT::Evaluate for the 4-node quad (ShapeFunctionT.cpp:241-301).
__device__ __forceinline__ void q4_eval(const double* c, double e1, double e2, double N[4],
                                        double x[3], double n[3], double& J) {
    N[0] = 0.25 * (1 - e1) * (1 - e2);
    N[1] = 0.25 * (1 + e1) * (1 - e2);
    N[2] = 0.25 * (1 + e1) * (1 + e2);
    N[3] = 0.25 * (1 - e1) * (1 + e2);
    const double d1[4] = {-0.25 * (1 - e2), 0.25 * (1 - e2), 0.25 * (1 + e2), -0.25 * (1 + e2)};
    const double d2[4] = {-0.25 * (1 - e1), -0.25 * (1 + e1), 0.25 * (1 + e1), 0.25 * (1 - e1)};
    double dx1[3] = {0, 0, 0}, dx2[3] = {0, 0, 0};
    x[0] = x[1] = x[2] = 0;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            x[d] += N[a] * c[a * 3 + d];
            dx1[d] += d1[a] * c[a * 3 + d];
            dx2[d] += d2[a] * c[a * 3 + d];
        }
    n[0] = dx1[1] * dx2[2] - dx1[2] * dx2[1];
    n[1] = dx1[2] * dx2[0] - dx1[0] * dx2[2];
    n[2] = dx1[0] * dx2[1] - dx1[1] * dx2[0];
    J = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= J;
    n[1] /= J;
    n[2] /= J;
}

// Duffy point of the singular integration (TDElementStepLinearT.cpp:406-590):
// triangle tri of the corner `corner`, tensor Gauss point (et1, et2) of weight w.
__device__ __forceinline__ void duffy_point(const double* c, int corner, int tri, double et1,
                                            double et2, double w, double N[4], double x[3],
                                            double n[3], double& wJ) {
    const double ec0 = (corner == 1 || corner == 2) ? 1.0 : -1.0;
    const double ec1 = (corner >= 2) ? 1.0 : -1.0;
    const double J_tri = 0.5 * (1 - et1);
    double e1, e2;
    if (tri == 0) {
        e1 = ec0 * (1 - 0.5 * (1 - et1) * (1 + ec0 * ec1 * et2));
        e2 = ec1 * et1;
    } else {
        e1 = ec0 * et1;
        e2 = ec1 * (1 - 0.5 * (1 - et1) * (1 - ec0 * ec1 * et2));
    }
    double J;
    q4_eval(c, e1, e2, N, x, n, J);
    wJ = w * J_tri * J;
}

// ShapeFunctionT::Evaluate for the 8-node serendipity quad (ShapeFunctionT.cpp:303-366).
__device__ __forceinline__ void q8_eval(const double* c, double e1, double e2, double N[8],
                                        double x[3], double n[3], double& J) {
    const double e1s = e1 * e1, e2s = e2 * e2;
    N[0] = 0.25 * (1 - e1) * (1 - e2) * (-e1 - e2 - 1);
    N[1] = 0.25 * (1 + e1) * (1 - e2) * (e1 - e2 - 1);
    N[2] = 0.25 * (1 + e1) * (1 + e2) * (e1 + e2 - 1);
    N[3] = 0.25 * (1 - e1) * (1 + e2) * (-e1 + e2 - 1);
    N[4] = 0.5 * (1 - e1s) * (1 - e2);
    N[5] = 0.5 * (1 + e1) * (1 - e2s);
    N[6] = 0.5 * (1 - e1s) * (1 + e2);
    N[7] = 0.5 * (1 - e1) * (1 - e2s);
    const double d1[8] = {-0.25 * (1 - e1) * (1 - e2) - 0.25 * (1 - e2) * (-1 - e1 - e2),
                          0.25 * (1 + e1) * (1 - e2) + 0.25 * (1 - e2) * (-1 + e1 - e2),
                          0.25 * (1 + e1) * (1 + e2) + 0.25 * (1 + e2) * (-1 + e1 + e2),
                          -0.25 * (1 - e1) * (1 + e2) - 0.25 * (1 + e2) * (-1 - e1 + e2),
                          -e1 * (1 - e2),
                          0.5 * (1 - e2s),
                          -e1 * (1 + e2),
                          -0.5 * (1 - e2s)};
    const double d2[8] = {-0.25 * (1 - e1) * (1 - e2) - 0.25 * (1 - e1) * (-1 - e1 - e2),
                          -0.25 * (1 + e1) * (1 - e2) - 0.25 * (1 + e1) * (-1 + e1 - e2),
                          0.25 * (1 + e1) * (1 + e2) + 0.25 * (1 + e1) * (-1 + e1 + e2),
                          0.25 * (1 - e1) * (1 + e2) + 0.25 * (1 - e1) * (-1 - e1 + e2),
                          -0.5 * (1 - e1s),
                          -(1 + e1) * e2,
                          0.5 * (1 - e1s),
                          -(1 - e1) * e2};
    double dx1[3] = {0, 0, 0}, dx2[3] = {0, 0, 0};
    x[0] = x[1] = x[2] = 0;
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            x[d] += N[a] * c[a * 3 + d];
            dx1[d] += d1[a] * c[a * 3 + d];
            dx2[d] += d2[a] * c[a * 3 + d];
        }
    n[0] = dx1[1] * dx2[2] - dx1[2] * dx2[1];
    n[1] = dx1[2] * dx2[0] - dx1[0] * dx2[2];
    n[2] = dx1[0] * dx2[1] - dx1[1] * dx2[0];
    J = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= J;
    n[1] /= J;
    n[2] /= J;
}

// SubElement (TDElementStepLinearT.cpp:192-386): a singular 8-node element is
// integrated as 4-node sub-elements over parent nodes; a singular corner keeps
// the corner quad (its corner singular), a singular midside node splits the
// element into two quads singular at their first corner.
__device__ __forceinline__ int q8_subelements(int singular, int ids[2][4], int cid[2]) {
    constexpr int mid[4][2][4] = {
        {{4, 6, 3, 0}, {4, 1, 2, 6}},
        {{5, 2, 3, 7}, {5, 7, 0, 1}},
        {{6, 3, 0, 4}, {6, 4, 1, 2}},
        {{7, 0, 1, 5}, {7, 5, 2, 3}},
    };
    if (singular < 4) {
#pragma unroll
        for (int i = 0; i < 4; i++) ids[0][i] = i;
        cid[0] = singular;
        return 1;
    }
#pragma unroll
    for (int e = 0; e < 2; e++) {
#pragma unroll
        for (int i = 0; i < 4; i++) ids[e][i] = mid[singular - 4][e][i];
        cid[e] = 0;
    }
    return 2;
}

// I-part time integrals of one wave at time T (GreenFunctionT.cpp:251-279):
// I1 (or I2), I3 (or I4), I5 (or I6).  cA = 8T + 4T1, cB = 6T^2 + 12 T T1,
// cC = 12 T1 T^2 are per-thread constants.
__device__ __forceinline__ void wave_I(double T, double cA, double cB, double cC, double roc,
                                       double inv12R2, double invc2, const Phys& ph,
                                       double& I1, double& I3, double& I5) {
    const double tr = T - roc;
    double b, x5;
    if (ph.dt <= tr) {
        b = ph.dt;
        x5 = 0;
    } else if (0 <= tr) {
        b = tr;
        x5 = (ph.dt - tr) * ph.inv_dt;
    } else {
        b = 0;
        x5 = 0;
    }
    const double poly = b * (cC + b * (-cB + b * (cA - 3 * b)));
    const double q = b * (ph.dt - 0.5 * b);
    I1 = (poly * inv12R2 - q * invc2) * ph.inv_dt;
    I3 = q * ph.inv_dt;
    I5 = x5;
}

// J-part time integrals (GreenFunctionT.cpp:275-280, 309-314): dA = 8T, dB = 6T^2.
__device__ __forceinline__ void wave_J(double T, double dA, double dB, double roc,
                                       double inv12R2, double invc2, const Phys& ph,
                                       double& J1, double& J3, double& J5) {
    const double tr = T - roc;
    double b, x5;
    if (ph.dt <= tr) {
        b = ph.dt;
        x5 = 0;
    } else if (0 <= tr) {
        b = tr;
        x5 = tr * ph.inv_dt;
    } else {
        b = 0;
        x5 = 0;
    }
    const double b2 = b * b;
    const double poly = b2 * (dB + b * (3 * b - dA));
    J1 = (poly * inv12R2 - 0.5 * b2 * invc2) * ph.inv_dt;
    J3 = 0.5 * b2 * ph.inv_dt;
    J5 = x5;
}

struct TimeConsts {
    bool doI, doJ;
    double TI0, TI1, TJ0, TJ1;          // I part at TI0 minus at TI1 = TI0 - dt; same for J
    double cA0, cB0, cC0, cA1, cB1, cC1;
    double dA0, dB0, dA1, dB1;
};

__device__ __forceinline__ void time_consts(TimeConsts& tc, double TI, double TJ, double dt) {
    tc.TI0 = TI;
    tc.TI1 = TI - dt;
    tc.TJ0 = TJ;
    tc.TJ1 = TJ - dt;
    tc.cA0 = 8 * tc.TI0 + 4 * dt;
    tc.cB0 = 6 * tc.TI0 * tc.TI0 + 12 * tc.TI0 * dt;
    tc.cC0 = 12 * dt * tc.TI0 * tc.TI0;
    tc.cA1 = 8 * tc.TI1 + 4 * dt;
    tc.cB1 = 6 * tc.TI1 * tc.TI1 + 12 * tc.TI1 * dt;
    tc.cC1 = 12 * dt * tc.TI1 * tc.TI1;
    tc.dA0 = 8 * tc.TJ0;
    tc.dB0 = 6 * tc.TJ0 * tc.TJ0;
    tc.dA1 = 8 * tc.TJ1;
    tc.dB1 = 6 * tc.TJ1 * tc.TJ1;
}

// Accumulators of one item: the 4 node blocks of G (symmetric, 6 entries)
// and H (9 entries, [i][j] of HE[i][3a+j]).
struct ItemAcc {
    double g[4][6];
    double h[4][9];
};

// One Gauss point of one item: step responses for the item's time(s) and the
// collected 3x3 kernels, sg = DU (symmetric, 6 entries) and th[i][j] = DT[j][i].
// Returns false when both parts are exactly zero at this point.
__device__ __forceinline__ bool point_kernels(const TimeConsts& tc, const Phys& ph,
                                              const double xc[3], const double xq[3],
                                              const double nq[3], double sg[6],
                                              double th[9]) {
    const double d0 = xq[0] - xc[0], d1 = xq[1] - xc[1], d2 = xq[2] - xc[2];
    const double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    const double inv_r = 1.0 / r;
    const double rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
    const double rdn = rv[0] * nq[0] + rv[1] * nq[1] + rv[2] * nq[2];
    const double inv12R2 = inv_r * inv_r * (1.0 / 12.0);
    const double roc_p = r * ph.inv_cp, roc_s = r * ph.inv_cs;

    // Once the S front has passed the point at both evaluation times of a part
    // ((T - dt) - r/c_s >= dt), that part's step response is identically zero
    // (b = dt and I5 = I6 = 0 at both times): skip it instead of summing round-off.
    const bool doI = tc.doI && !(tc.TI1 - roc_s >= ph.dt);
    const bool doJ = tc.doJ && !(tc.TJ1 - roc_s >= ph.dt);
    if (!doI && !doJ) return false;
    double P1 = 0, P3 = 0, P5 = 0, S2 = 0, S4 = 0, S6 = 0;
    if (doI) {
        double a1, a3, a5, b1, b3, b5;
        wave_I(tc.TI0, tc.cA0, tc.cB0, tc.cC0, roc_p, inv12R2, ph.inv_cp2, ph, a1, a3, a5);
        wave_I(tc.TI1, tc.cA1, tc.cB1, tc.cC1, roc_p, inv12R2, ph.inv_cp2, ph, b1, b3, b5);
        P1 = a1 - b1;
        P3 = a3 - b3;
        P5 = a5 - b5;
        wave_I(tc.TI0, tc.cA0, tc.cB0, tc.cC0, roc_s, inv12R2, ph.inv_cs2, ph, a1, a3, a5);
        wave_I(tc.TI1, tc.cA1, tc.cB1, tc.cC1, roc_s, inv12R2, ph.inv_cs2, ph, b1, b3, b5);
        S2 = a1 - b1;
        S4 = a3 - b3;
        S6 = a5 - b5;
    }
    if (doJ) {
        double a1, a3, a5, b1, b3, b5;
        wave_J(tc.TJ0, tc.dA0, tc.dB0, roc_p, inv12R2, ph.inv_cp2, ph, a1, a3, a5);
        wave_J(tc.TJ1, tc.dA1, tc.dB1, roc_p, inv12R2, ph.inv_cp2, ph, b1, b3, b5);
        P1 += a1 - b1;
        P3 += a3 - b3;
        P5 += a5 - b5;
        wave_J(tc.TJ0, tc.dA0, tc.dB0, roc_s, inv12R2, ph.inv_cs2, ph, a1, a3, a5);
        wave_J(tc.TJ1, tc.dA1, tc.dB1, roc_s, inv12R2, ph.inv_cs2, ph, b1, b3, b5);
        S2 += a1 - b1;
        S4 += a3 - b3;
        S6 += a5 - b5;
    }
    // DU (GreenFunctionT.cpp:321-353): A r r^T + B I
    const double It1 = 0.5 * (P1 - S2);
    const double It2u = P3 * ph.inv_cp2 - S4 * ph.inv_cs2;
    const double invDiv = inv_r * ph.inv_4pi_rho;
    const double A = (3 * It1 + It2u) * invDiv;
    const double B = (S4 * ph.inv_cs2 - It1) * invDiv;
    // DT (GreenFunctionT.cpp:360-406): alpha rdn r r^T + beta n r^T + gamma (r n^T + rdn I)
    const double It2t = S4 - ph.ratio2 * P3;
    const double It3t = S6 - ph.ratio3 * P5;
    const double It4 = P3 + roc_p * P5;
    const double It5 = S4 + roc_s * S6;
    const double ir2 = inv_r * inv_r * ph.inv_4pi;
    const double Q = 6 * ph.cs2 * It1 - 2 * It2t;
    const double alpha = ((-30 * ph.cs2) * It1 + 12 * It2t) * ir2 +
                         (2 * ph.inv_cs * ph.inv_4pi) * inv_r * It3t;
    const double beta = (Q - (1 - 2 * ph.ratio2) * It4) * ir2;
    const double gamma = (Q - It5) * ir2;

    const double rr00 = rv[0] * rv[0], rr01 = rv[0] * rv[1], rr02 = rv[0] * rv[2];
    const double rr11 = rv[1] * rv[1], rr12 = rv[1] * rv[2], rr22 = rv[2] * rv[2];
    sg[0] = A * rr00 + B;
    sg[1] = A * rr01;
    sg[2] = A * rr02;
    sg[3] = A * rr11 + B;
    sg[4] = A * rr12;
    sg[5] = A * rr22 + B;
    const double ar = alpha * rdn, gd = gamma * rdn;
    // T[i][j] = DT[j][i] = ar r_i r_j + beta n_j r_i + gamma n_i r_j (+ gamma rdn on i == j)
    const double rrm[9] = {rr00, rr01, rr02, rr01, rr11, rr12, rr02, rr12, rr22};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            th[i * 3 + j] = ar * rrm[i * 3 + j] + beta * (nq[j] * rv[i]) +
                            gamma * (nq[i] * rv[j]) + (i == j ? gd : 0.0);
    return true;
}

// One Gauss point of one Q4 item, accumulated into the 4 node blocks.
__device__ __forceinline__ void gauss_point(ItemAcc& acc, const TimeConsts& tc, const Phys& ph,
                                            const double xc[3], const double xq[3],
                                            const double nq[3], double wJ, const double N[4]) {
    double sg[6], th[9];
    if (!point_kernels(tc, ph, xc, xq, nq, sg, th)) return;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const double w = wJ * N[a];
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] += w * sg[m];
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] += w * th[m];
    }
}

__global__ void k_gauss_geom(const double* __restrict__ coords, const int* __restrict__ ien,
                             int nel, int nq, const double* __restrict__ gx,
                             const double* __restrict__ gw, double* __restrict__ geom,
                             float* __restrict__ geomf) {
    const int nq2 = nq * nq;
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (gid >= (long long)nel * nq2) return;
    const int e = (int)(gid / nq2), q = (int)(gid % nq2);
    double c[12];
    for (int a = 0; a < 4; a++) {
        const int nid = ien[e * 4 + a];
        for (int d = 0; d < 3; d++) c[a * 3 + d] = coords[nid * 3 + d];
    }
    // FormGH_Regular's loop order: q_1 outer, q_2 inner (TDElementStepLinearT.cpp:52-56)
    const int q1 = q / nq, q2 = q % nq;
    double N[4], x[3], n[3], J;
    q4_eval(c, gx[q1], gx[q2], N, x, n, J);
    double* g = geom + gid * kGeomStride;
    g[0] = x[0];
    g[1] = x[1];
    g[2] = x[2];
    g[3] = n[0];
    g[4] = n[1];
    g[5] = n[2];
    g[6] = (gw[q1] * gw[q2]) * J;
    g[7] = N[0];
    g[8] = N[1];
    g[9] = N[2];
    g[10] = N[3];
    g[11] = 0;
    // FP32 copy for the far-field kernel: the point relative to the element's first
    // node (small numbers, so FP32 differences to the collocation point stay
    // accurate), the unit normal, w J and N.
    float* gf = geomf + gid * kGeomStride;
    gf[0] = (float)(x[0] - c[0]);
    gf[1] = (float)(x[1] - c[1]);
    gf[2] = (float)(x[2] - c[2]);
    gf[3] = (float)n[0];
    gf[4] = (float)n[1];
    gf[5] = (float)n[2];
    gf[6] = (float)g[6];
    gf[7] = (float)N[0];
    gf[8] = (float)N[1];
    gf[9] = (float)N[2];
    gf[10] = (float)N[3];
    gf[11] = 0.f;
}

// Gauss-point geometry of 8-node elements: x[3], n[3], w J, N[8] (stride kGeomStride8).
__global__ void k_gauss_geom8(const double* __restrict__ coords, const int* __restrict__ ien,
                              int nel, int nq, const double* __restrict__ gx,
                              const double* __restrict__ gw, double* __restrict__ geom) {
    const int nq2 = nq * nq;
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (gid >= (long long)nel * nq2) return;
    const int e = (int)(gid / nq2), q = (int)(gid % nq2);
    double c[24];
    for (int a = 0; a < 8; a++) {
        const int nid = ien[e * 8 + a];
        for (int d = 0; d < 3; d++) c[a * 3 + d] = coords[nid * 3 + d];
    }
    const int q1 = q / nq, q2 = q % nq;
    double N[8], x[3], n[3], J;
    q8_eval(c, gx[q1], gx[q2], N, x, n, J);
    double* g = geom + gid * kGeomStride8;
    g[0] = x[0];
    g[1] = x[1];
    g[2] = x[2];
    g[3] = n[0];
    g[4] = n[1];
    g[5] = n[2];
    g[6] = (gw[q1] * gw[q2]) * J;
    for (int a = 0; a < 8; a++) g[7 + a] = N[a];
    g[15] = 0;
}

// Last pair p in [lo, hi] with offsets[p] <= gid (the pair owning item gid).
__device__ __forceinline__ unsigned find_pair(const unsigned* __restrict__ offsets, unsigned lo,
                                              unsigned hi, unsigned gid) {
    while (lo < hi) {
        const unsigned mid = (lo + hi + 1) >> 1;
        if (__ldg(offsets + mid) <= gid) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The pair of this thread's item (item = global thread index >> sh): one full
// search per block for its first and last items, then a short search inside that
// range.  Call with all threads of the block (it synchronises); returns false
// for threads past the last item.
__device__ __forceinline__ bool item_pair(const unsigned* __restrict__ offsets, unsigned npairs,
                                          unsigned nitems, unsigned& p, int sh = 0) {
    __shared__ unsigned s_lo, s_hi;
    const unsigned first = (blockIdx.x * blockDim.x) >> sh;
    if (first >= nitems) return false;  // uniform over the block
    const unsigned last = min(first + (blockDim.x >> sh), nitems) - 1;
    if (threadIdx.x == 0) s_lo = find_pair(offsets, 0, npairs - 1, first);
    if (threadIdx.x == 32) s_hi = find_pair(offsets, 0, npairs - 1, last);
    __syncthreads();
    const unsigned item = first + (threadIdx.x >> sh);
    if (item >= nitems) return false;
    p = find_pair(offsets, s_lo, s_hi, item);
    return true;
}

// Singular test of ElastoDynamicsT::G_H_Driver (ElastoDynamicsT.cpp:166-175):
// the last element node with r^2 < 1e-9 (unfused, as the reference's pow sum).
template <int ENND = 4>
__device__ __forceinline__ int singular_corner(const double* c, const double xc[3]) {
    int s = -1;
#pragma unroll
    for (int a = 0; a < ENND; a++) {
        const double dx = c[a * 3] - xc[0], dy = c[a * 3 + 1] - xc[1], dz = c[a * 3 + 2] - xc[2];
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        if (r2 < 1e-9) s = a;
    }
    return s;
}

// Node coordinates (nd), node centroid (ctr) and the largest node distance from it
// (the return value) of element e.
template <int ENND>
__device__ __forceinline__ double element_box(const double* __restrict__ coords,
                                              const int* __restrict__ ien, int e,
                                              double nd[3 * ENND], double ctr[3]) {
    ctr[0] = ctr[1] = ctr[2] = 0;
    for (int a = 0; a < ENND; a++) {
        const int nid = ien[e * ENND + a];
        for (int d = 0; d < 3; d++) {
            nd[a * 3 + d] = coords[nid * 3 + d];
            ctr[d] += (1.0 / ENND) * nd[a * 3 + d];
        }
    }
    double rad = 0;
    for (int a = 0; a < ENND; a++) {
        const double dx = nd[a * 3] - ctr[0], dy = nd[a * 3 + 1] - ctr[1], dz = nd[a * 3 + 2] - ctr[2];
        rad = fmax(rad, sqrt(dx * dx + dy * dy + dz * dz));
    }
    return rad;
}

// Distance from a node beyond which no node of the element passes the singular test
// (r^2 < 1e-9, r < 3.2e-5): every node lies within rad of the centroid.
constexpr double kSingularClear = 1e-4;

// Level window (or step membership) and singular corner of pair p (collocation
// node node_lo + p / ne, element elems[p % ne]).  ebox (may be null): per element
// the centroid and node radius of element_box, made once per mesh (k_element_box);
// with it a pair takes one FP64 square root instead of five, and reads the element's
// nodes only when the node is within kSingularClear of the element's node radius.
template <int ENND = 4>
__device__ __forceinline__ PairInfo pair_window_info(const double* __restrict__ coords,
                                                     const int* __restrict__ ien,
                                                     const int* __restrict__ elems, int ne,
                                                     int node_lo, const Phys& ph, int mode,
                                                     int level_last, int level_cap, int step_n,
                                                     int select, long long p,
                                                     const ElemBox* __restrict__ ebox = nullptr) {
    const int c = node_lo + (int)(p / ne);
    const int e = elems[p % ne];
    const double xc[3] = {coords[c * 3], coords[c * 3 + 1], coords[c * 3 + 2]};
    double nd[3 * ENND];
    double ctr[3];
    double rad;
    if (ebox) {
        const ElemBox b = ebox[e];
        ctr[0] = b.x;
        ctr[1] = b.y;
        ctr[2] = b.z;
        rad = b.rad;
    } else {
        rad = element_box<ENND>(coords, ien, e, nd, ctr);
    }
    const double rad_nodes = rad;
    // An 8-node element's surface x = sum N_a x_a is no convex combination of its
    // nodes; sum |N_a| <= 3 on the reference square (at its centre), so the surface
    // lies within 3 rad of the node centroid.
    if (ENND == 8) rad *= 3.0;
    const double dx = xc[0] - ctr[0], dy = xc[1] - ctr[1], dz = xc[2] - ctr[2];
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    const double margin = 1e-3 * rad + 1e-12;
    const double rmin = fmax(0.0, dist - rad - margin), rmax = dist + rad + margin;
    int sing = -1;
    if (!ebox) {
        sing = singular_corner<ENND>(nd, xc);
    } else if (dist <= rad_nodes + kSingularClear) {
        for (int a = 0; a < ENND; a++) {
            const int nid = ien[e * ENND + a];
            for (int d = 0; d < 3; d++) nd[a * 3 + d] = coords[nid * 3 + d];
        }
        sing = singular_corner<ENND>(nd, xc);
    }
    // The step response at time n dt is exactly zero unless r/c_p <= n dt and
    // n < r/(c_s dt) + 2; level k takes n = k (I part) and n = k + 1 (J part), so it
    // can be non-zero only for r_min/(c_p dt) - 1 <= k < r_max/(c_s dt) + 1 (one level
    // of margin on the low side for rounding).
    int n_lo = (int)floor(rmin * ph.inv_cp * ph.inv_dt) - 1;
    const int n_hi = (int)ceil(rmax * ph.inv_cs * ph.inv_dt) + 2;
    if (sing >= 0) n_lo = 0;
    PairInfo pi;
    pi.sing = sing;
    if (mode == ASM_LEVELS) {  // step_n: the lowest level wanted
        const int klo = max(step_n, n_lo);
        const int khi = min(min(level_last, (int)ceil(rmax * ph.inv_cs * ph.inv_dt) + 1),
                            level_cap);
        pi.klo = klo;
        pi.cnt = max(0, khi - klo + 1);
    } else {
        pi.klo = step_n;
        pi.cnt = (step_n >= n_lo && step_n <= n_hi) ? 1 : 0;
    }
    // FP32 far form: non-singular, and every point at least c_s dt / 8 from the node.
    // Closer, the dynamic kernel nears the static one through the cancellation of
    // terms ~(c_s dt / r)^2 larger, which FP32 would amplify by as much.
    const bool far = sing < 0 && rmin > kFarRatio * rad && 8.0 * rmin * ph.inv_cs >= ph.dt;
    if ((select == SEL_NEAR && far) || (select == SEL_FAR && !far)) pi.cnt = 0;
    return pi;
}

// The Duffy points of every (element, corner) of a 4-node mesh, as duffy_point gives
// them (x, n, wJ, N in the geometry table's layout): t = ((e * 4 + corner) * 2 nq^2 +
// point).  The singular pairs' quadrature (near field at every level, C term) reads
// them instead of mapping each point again in FP64.
__global__ void k_duffy_table(const double* __restrict__ coords, const int* __restrict__ ien,
                              int nel, int nq, const double* __restrict__ gx,
                              const double* __restrict__ gw, double* __restrict__ duffy) {
    const int nq2 = nq * nq, per = 2 * nq2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nel * 4 * per) return;
    const int qq = (int)(t % per);
    const long long ec = t / per;
    const int corner = (int)(ec % 4), e = (int)(ec / 4);
    double cn[12];
    for (int a = 0; a < 4; a++) {
        const int nid = ien[e * 4 + a];
        for (int d = 0; d < 3; d++) cn[a * 3 + d] = coords[nid * 3 + d];
    }
    const int tri = qq / nq2, q = qq % nq2, q1 = q / nq, q2 = q % nq;
    double N[4], xq[3], nv[3], wJ;
    duffy_point(cn, corner, tri, gx[q1], gx[q2], gw[q1] * gw[q2], N, xq, nv, wJ);
    double* g = duffy + t * kGeomStride;
    for (int d = 0; d < 3; d++) {
        g[d] = xq[d];
        g[3 + d] = nv[d];
    }
    g[6] = wJ;
    for (int a = 0; a < 4; a++) g[7 + a] = N[a];
    g[11] = 0;
}

template <int ENND>
__global__ void k_element_box(const double* __restrict__ coords, const int* __restrict__ ien,
                              int nel, ElemBox* __restrict__ ebox) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nel) return;
    double nd[3 * ENND], ctr[3];
    const double rad = element_box<ENND>(coords, ien, e, nd, ctr);
    ebox[e] = ElemBox{ctr[0], ctr[1], ctr[2], rad};
}

template <int ENND>
__global__ void k_pair_window(const double* __restrict__ coords, const int* __restrict__ ien,
                              const int* __restrict__ elems, int ne, int node_lo, int nnodes,
                              Phys ph, int mode, int level_last, int level_cap, int step_n,
                              int select, PairInfo* __restrict__ pairs,
                              unsigned* __restrict__ counts, const ElemBox* __restrict__ ebox) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= (long long)nnodes * ne) return;
    const PairInfo pi = pair_window_info<ENND>(coords, ien, elems, ne, node_lo, ph, mode,
                                               level_last, level_cap, step_n, select, p, ebox);
    pairs[p] = pi;
    if (counts) counts[p] = (unsigned)pi.cnt;
}

// mode ASM_LEVELS: item = (pair, level k), I part at k dt (k >= 1) plus J part at
// (k+1) dt ((k+1) <= level_last), scattered into level k of G0/H0 (or the FP32 store).
// mode ASM_STEP:   item = (pair, step_n), part = 0 -> I part into G0/H0,
//                  part = 1 -> J part into G1/H1 (row block starting at row_node_lo).
// One item: pair p (collocation node node_lo + p / ne, element elems[p % ne]) at
// level (or step) k; accumulates its Gauss points and scatters into out.  An
// 8-node element's item is split over two threads, half 0 holding the blocks of
// nodes 0-3 and half 1 those of nodes 4-7 (each evaluates every point's kernels).
// L > 1 (a power of two, at most 32): L aligned lanes of a warp share the item (or
// half), lane sub taking every L-th Gauss point; an xor butterfly of shuffles then
// gives every lane the item's sums (bitwise the same on all lanes: each addition
// has the same two operands on both lanes of a pair), and the lanes split the
// scatter by node.  L = 1 is one thread's sequential sum.
template <int MODE, int ENND = 4>
__device__ __forceinline__ void assemble_item(
    const double* __restrict__ coords, const int* __restrict__ ien,
    const int* __restrict__ elems, int ne, int node_lo, int nq, const double* __restrict__ gx,
    const double* __restrict__ gw, const double* __restrict__ geom, const Phys& ph,
    int level_last, int step_n, int part, const PairInfo& pi, unsigned p, int k,
    const AsmOut& out, int half = 0, int sub = 0, int L = 1,
    const double* __restrict__ duffy = nullptr) {
    const int c = node_lo + (int)(p / ne);
    const int e = elems[p % ne];
    const double xc[3] = {coords[c * 3], coords[c * 3 + 1], coords[c * 3 + 2]};
    int nid[4];
#pragma unroll
    for (int a = 0; a < 4; a++) nid[a] = ien[e * ENND + 4 * half + a];

    TimeConsts tc;
    if (MODE == ASM_LEVELS) {
        tc.doI = (k >= 1);
        tc.doJ = (k + 1 <= level_last);
        time_consts(tc, k * ph.dt, (k + 1) * ph.dt, ph.dt);
    } else {
        tc.doI = (part == 0);
        tc.doJ = (part == 1);
        time_consts(tc, step_n * ph.dt, step_n * ph.dt, ph.dt);
    }

    ItemAcc acc;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] = 0;
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] = 0;
    }
    const int nq2 = nq * nq;
    constexpr int stride = ENND == 8 ? kGeomStride8 : kGeomStride;
    if (pi.sing < 0) {
        const double* g0 = geom + (size_t)e * nq2 * stride;
        const int n0 = 7 + 4 * half;
        for (int q = sub; q < nq2; q += L) {
            const double* g = g0 + (size_t)q * stride;
            const double xq[3] = {__ldg(g), __ldg(g + 1), __ldg(g + 2)};
            const double nqv[3] = {__ldg(g + 3), __ldg(g + 4), __ldg(g + 5)};
            const double N[4] = {__ldg(g + n0), __ldg(g + n0 + 1), __ldg(g + n0 + 2),
                                 __ldg(g + n0 + 3)};
            gauss_point(acc, tc, ph, xc, xq, nqv, __ldg(g + 6), N);
        }
    } else if (ENND == 8) {
        // 4-node sub-elements over parent nodes, each with the Duffy rule from its
        // singular corner; a sub-element node's shape value goes to its parent node
        // when that node belongs to this half (AssembleSubElement,
        // TDElementStepLinearT.cpp:597-626).
        int ids[2][4], cid[2];
        const int nsub = q8_subelements(pi.sing, ids, cid);
        for (int se = 0; se < nsub; se++) {
            double cn[12];
            int slot[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int id = ids[se][i];
                slot[i] = id - 4 * half;  // in [0, 4) when parent node id is in this half
                const int n = ien[e * 8 + id];
#pragma unroll
                for (int d = 0; d < 3; d++) cn[i * 3 + d] = coords[n * 3 + d];
            }
            for (int qq = sub; qq < 2 * nq2; qq += L) {
                const int tri = qq / nq2, q = qq % nq2, q1 = q / nq, q2 = q % nq;
                double N4[4], xq[3], nqv[3], wJ;
                duffy_point(cn, cid[se], tri, gx[q1], gx[q2], gw[q1] * gw[q2], N4, xq, nqv,
                            wJ);
                double N[4] = {0, 0, 0, 0};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int a = 0; a < 4; a++)
                        if (slot[i] == a) N[a] = N4[i];
                gauss_point(acc, tc, ph, xc, xq, nqv, wJ, N);
            }
        }
    } else if (duffy) {
        // the element's Duffy points from this corner, made once per mesh
        const double* g0 = duffy + ((size_t)e * 4 + pi.sing) * 2 * nq2 * kGeomStride;
        for (int qq = sub; qq < 2 * nq2; qq += L) {
            const double* g = g0 + (size_t)qq * kGeomStride;
            const double xq[3] = {__ldg(g), __ldg(g + 1), __ldg(g + 2)};
            const double nqv[3] = {__ldg(g + 3), __ldg(g + 4), __ldg(g + 5)};
            const double N[4] = {__ldg(g + 7), __ldg(g + 8), __ldg(g + 9), __ldg(g + 10)};
            gauss_point(acc, tc, ph, xc, xq, nqv, __ldg(g + 6), N);
        }
    } else {
        double cn[12];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int d = 0; d < 3; d++) cn[a * 3 + d] = coords[nid[a] * 3 + d];
        for (int qq = sub; qq < 2 * nq2; qq += L) {
            const int tri = qq / nq2, q = qq % nq2, q1 = q / nq, q2 = q % nq;
            double N[4], xq[3], nqv[3], wJ;
            duffy_point(cn, pi.sing, tri, gx[q1], gx[q2], gw[q1] * gw[q2], N, xq, nqv, wJ);
            gauss_point(acc, tc, ph, xc, xq, nqv, wJ, N);
        }
    }

    if (L > 1) {
        const unsigned lane = threadIdx.x & 31;
        const unsigned mask =
            L == 32 ? 0xffffffffu : ((1u << L) - 1) << (lane & ~(unsigned)(L - 1));
        for (int o = 1; o < L; o <<= 1) {
#pragma unroll
            for (int a = 0; a < 4; a++) {
#pragma unroll
                for (int m = 0; m < 6; m++) acc.g[a][m] += __shfl_xor_sync(mask, acc.g[a][m], o);
#pragma unroll
                for (int m = 0; m < 9; m++) acc.h[a][m] += __shfl_xor_sync(mask, acc.h[a][m], o);
            }
        }
    }
    // lane sub writes the blocks of the nodes a with (a & own) == sub
    const int own = min(L, 4) - 1;

    // scatter: rows 3c+i, columns 3*nid[a]+j
    const size_t D = (size_t)out.ld;
    double* G;
    double* H;
    float* Gf = nullptr;
    float* Hf = nullptr;
    size_t rowbase;
    if (MODE == ASM_LEVELS) {
        G = out.G0;
        H = out.H0;
        Gf = out.G0f;
        Hf = out.H0f;
        rowbase = (size_t)k * out.level_stride + (size_t)(3 * c) * D;
    } else {
        G = part == 0 ? out.G0 : out.G1;
        H = part == 0 ? out.H0 : out.H1;
        rowbase = (size_t)(3 * (c - out.row_node_lo)) * D;
    }
    constexpr int sym[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
    // read-modify-write of the item's entries, a node block at a time, reads before
    // writes (as in far_item)
#pragma unroll
    for (int a = 0; a < 4; a++) {
        if ((a & own) != sub) continue;
        if (Gf) {
            float og[9], oh[9];
#pragma unroll
            for (int m = 0; m < 9; m++) {
                const size_t idx = rowbase + (size_t)(m / 3) * D + 3 * (size_t)nid[a] + m % 3;
                og[m] = Gf[idx];
                oh[m] = Hf[idx];
            }
#pragma unroll
            for (int m = 0; m < 9; m++) {
                const size_t idx = rowbase + (size_t)(m / 3) * D + 3 * (size_t)nid[a] + m % 3;
                Gf[idx] = og[m] + (float)acc.g[a][sym[m]];
                Hf[idx] = oh[m] + (float)acc.h[a][m];
            }
        } else {
            double og[9], oh[9];
#pragma unroll
            for (int m = 0; m < 9; m++) {
                const size_t idx = rowbase + (size_t)(m / 3) * D + 3 * (size_t)nid[a] + m % 3;
                og[m] = G[idx];
                oh[m] = H[idx];
            }
#pragma unroll
            for (int m = 0; m < 9; m++) {
                const size_t idx = rowbase + (size_t)(m / 3) * D + 3 * (size_t)nid[a] + m % 3;
                G[idx] = og[m] + acc.g[a][sym[m]];
                H[idx] = oh[m] + acc.h[a][m];
            }
        }
    }
}



// 2^lg adjacent lanes per item (4-node elements) or per half of an item (8-node
// elements, one half per group of the element's nodes).
template <int MODE, int ENND>
__global__ void __launch_bounds__(128) k_assemble_items(
    const double* __restrict__ coords, const int* __restrict__ ien,
    const int* __restrict__ elems, int ne, int node_lo, int nq, const double* __restrict__ gx,
    const double* __restrict__ gw, const double* __restrict__ geom, Phys ph, int level_last,
    int step_n, int part, const PairInfo* __restrict__ pairs,
    const unsigned* __restrict__ offsets, unsigned npairs, unsigned nitems, AsmOut out,
    int lg, const double* __restrict__ duffy) {
    constexpr int SH = ENND == 8 ? 1 : 0;
    unsigned p;
    if (!item_pair(offsets, npairs, nitems, p, SH + lg)) return;
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned unit = gid >> lg;
    const PairInfo pi = pairs[p];
    const int k = pi.klo + (int)((unit >> SH) - __ldg(offsets + p));
    assemble_item<MODE, ENND>(coords, ien, elems, ne, node_lo, nq, gx, gw, geom, ph, level_last,
                              step_n, part, pi, p, k, out, (int)(unit & SH),
                              (int)(gid & ((1u << lg) - 1)), 1 << lg, duffy);
}

// One step (ASM_STEP) without compaction: one thread per pair (two for an 8-node
// element), the pairs outside the step's window returning at once.  A pair holds
// at most one item of a step, so this needs neither a scan of the counts nor the
// item total on the host; the allocation-free driver (noalloc.cu) uses it so that
// a call never waits for the device.  Same items, same arithmetic and the same
// colour-ordered scatter as k_assemble_items with one lane per item, so the same
// results bit for bit as that; where k_assemble_items splits an item's points over
// lanes (launches of few items) its sums are formed in another order (~1e-16
// relative).
template <int ENND>
__global__ void __launch_bounds__(128) k_assemble_step_pairs(
    const double* __restrict__ coords, const int* __restrict__ ien,
    const int* __restrict__ elems, int ne, int node_lo, int nq, const double* __restrict__ gx,
    const double* __restrict__ gw, const double* __restrict__ geom, Phys ph, int step_n,
    int part, const PairInfo* __restrict__ pairs, unsigned npairs, AsmOut out) {
    constexpr int SH = ENND == 8 ? 1 : 0;
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned p = gid >> SH;
    if (p >= npairs) return;
    const PairInfo pi = pairs[p];
    if (pi.cnt == 0) return;
    assemble_item<ASM_STEP, ENND>(coords, ien, elems, ne, node_lo, nq, gx, gw, geom, ph, step_n,
                                  step_n, part, pi, p, pi.klo, out, (int)(gid & SH));
}

// ---------------------------------------------------------------------------
// Element interface (TDElementT / TDElementStepLinearT): a batch of independent
// (collocation point, element) pairs, each with its own node coordinates, time and
// singular node, integrated as FormGH_Regular / FormGH_Singular(singular)
// integrate one element (TDElementStepLinearT.cpp:28-626) and written as the
// element blocks GetGHLinear returns: GE_1/HE_1 (I part) and GE_2/HE_2 (J part),
// 3 x 3 ennd row-major each, [i][3a + j].  The points, Duffy rules, sub-elements
// and kernels are the mesh path's (q4_eval / q8_eval, duffy_point,
// q8_subelements, gauss_point); the geometry is evaluated per point instead of
// read from a per-mesh table.
// ---------------------------------------------------------------------------

// Kelvin part of one element (C_1 = C_2 = -sum wJ DT_Kelvin^T at t == t_1,
// TDElementStepLinearT.cpp:110-116 and its singular counterpart), from the same
// points as the element's quadrature.
template <int ENND>
__device__ void element_cterm(const double* en, const double xc[3], int sing, int nq,
                              const double* __restrict__ gx, const double* __restrict__ gw,
                              const Phys& ph, double acc[9]) {
    const double onem2nu = 1 - 2 * ph.nu;
    const double kscale = (0.5 * ph.dt) / (-(8 * M_PI) * (1 - ph.nu));
    for (int m = 0; m < 9; m++) acc[m] = 0;
    int ids[2][4] = {{0, 1, 2, 3}, {0, 1, 2, 3}}, cid[2] = {sing, sing};
    int nsub = 1;
    if (ENND == 8 && sing >= 0) nsub = q8_subelements(sing, ids, cid);
    const int nq2 = nq * nq;
    const int npts = sing < 0 ? nq2 : nsub * 2 * nq2;
    double cn[12];
    int cur = -1;
    for (int qq = 0; qq < npts; qq++) {
        double xq[3], nv[3], wJ;
        if (sing < 0) {
            const int q1 = qq / nq, q2 = qq % nq;
            double N[ENND], J;
            if constexpr (ENND == 8) q8_eval(en, gx[q1], gx[q2], N, xq, nv, J);
            else q4_eval(en, gx[q1], gx[q2], N, xq, nv, J);
            wJ = (gw[q1] * gw[q2]) * J;
        } else {
            const int se = qq / (2 * nq2), r = qq % (2 * nq2);
            if (se != cur) {
                for (int i = 0; i < 4; i++)
                    for (int d = 0; d < 3; d++) cn[i * 3 + d] = en[ids[se][i] * 3 + d];
                cur = se;
            }
            const int tri = r / nq2, q = r % nq2, q1 = q / nq, q2 = q % nq;
            double N[4];
            duffy_point(cn, cid[se], tri, gx[q1], gx[q2], gw[q1] * gw[q2], N, xq, nv, wJ);
        }
        const double d0 = xq[0] - xc[0], d1 = xq[1] - xc[1], d2 = xq[2] - xc[2];
        const double inv_r = 1.0 / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        const double rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
        const double rdn = rv[0] * nv[0] + rv[1] * nv[1] + rv[2] * nv[2];
        const double w = wJ * (kscale * inv_r * inv_r);
        for (int i = 0; i < 3; i++)
            for (int kk = 0; kk < 3; kk++) {
                const double Kki = ((kk == i ? onem2nu : 0.0) + 3 * rv[kk] * rv[i]) * rdn -
                                   onem2nu * (rv[i] * nv[kk] - rv[kk] * nv[i]);
                acc[i * 3 + kk] -= w * Kki;
            }
    }
}

// One thread per pair (two adjacent threads for an 8-node element, one per half of
// its nodes); part 0 writes GE_1 / HE_1 (and C at t == t_1), part 1 GE_2 / HE_2.
template <int ENND>
__global__ void __launch_bounds__(128) k_element_gh(
    int n, int nq, const double* __restrict__ gx, const double* __restrict__ gw, Phys ph,
    const double* __restrict__ colloc, const double* __restrict__ ecoords,
    const double* __restrict__ times, const int* __restrict__ sing_in, int part,
    double* __restrict__ GE, double* __restrict__ HE, double* __restrict__ C1,
    double* __restrict__ C2) {
    constexpr int SH = ENND == 8 ? 1 : 0;
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned item = gid >> SH;
    const int half = (int)(gid & SH);
    if (item >= (unsigned)n) return;
    const double xc[3] = {colloc[item * 3], colloc[item * 3 + 1], colloc[item * 3 + 2]};
    double en[3 * ENND];
    for (int m = 0; m < 3 * ENND; m++) en[m] = ecoords[(size_t)item * 3 * ENND + m];
    const double t = times[item];
    const int sing = sing_in[item];
    TimeConsts tc;
    tc.doI = (part == 0);
    tc.doJ = (part == 1);
    time_consts(tc, t, t, ph.dt);
    ItemAcc acc;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] = 0;
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] = 0;
    }
    const int nq2 = nq * nq;
    if (sing < 0) {
        for (int q = 0; q < nq2; q++) {
            const int q1 = q / nq, q2 = q % nq;
            double Nf[ENND], xq[3], nqv[3], J;
            if constexpr (ENND == 8) q8_eval(en, gx[q1], gx[q2], Nf, xq, nqv, J);
            else q4_eval(en, gx[q1], gx[q2], Nf, xq, nqv, J);
            const double N[4] = {Nf[4 * half], Nf[4 * half + 1], Nf[4 * half + 2],
                                 Nf[4 * half + 3]};
            gauss_point(acc, tc, ph, xc, xq, nqv, (gw[q1] * gw[q2]) * J, N);
        }
    } else if (ENND == 8) {
        int ids[2][4], cid[2];
        const int nsub = q8_subelements(sing, ids, cid);
        for (int se = 0; se < nsub; se++) {
            double cn[12];
            int slot[4];
            for (int i = 0; i < 4; i++) {
                slot[i] = ids[se][i] - 4 * half;
                for (int d = 0; d < 3; d++) cn[i * 3 + d] = en[ids[se][i] * 3 + d];
            }
            for (int qq = 0; qq < 2 * nq2; qq++) {
                const int tri = qq / nq2, q = qq % nq2, q1 = q / nq, q2 = q % nq;
                double N4[4], xq[3], nqv[3], wJ;
                duffy_point(cn, cid[se], tri, gx[q1], gx[q2], gw[q1] * gw[q2], N4, xq, nqv,
                            wJ);
                double N[4] = {0, 0, 0, 0};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int a = 0; a < 4; a++)
                        if (slot[i] == a) N[a] = N4[i];
                gauss_point(acc, tc, ph, xc, xq, nqv, wJ, N);
            }
        }
    } else {
        for (int qq = 0; qq < 2 * nq2; qq++) {
            const int tri = qq / nq2, q = qq % nq2, q1 = q / nq, q2 = q % nq;
            double N[4], xq[3], nqv[3], wJ;
            duffy_point(en, sing, tri, gx[q1], gx[q2], gw[q1] * gw[q2], N, xq, nqv, wJ);
            gauss_point(acc, tc, ph, xc, xq, nqv, wJ, N);
        }
    }
    constexpr int sym[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
    const size_t row = 3 * (size_t)ENND;  // 3 ennd entries per row of an element block
    double* G = GE + (size_t)item * 3 * row;
    double* H = HE + (size_t)item * 3 * row;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const size_t idx = (size_t)i * row + 3 * (size_t)(a + 4 * half) + j;
                G[idx] = acc.g[a][sym[i * 3 + j]];
                H[idx] = acc.h[a][i * 3 + j];
            }
    if (part == 0 && half == 0) {
        double c[9];
        if (t == ph.dt) {
            element_cterm<ENND>(en, xc, sing, nq, gx, gw, ph, c);
        } else {
            for (int m = 0; m < 9; m++) c[m] = 0;
        }
        for (int m = 0; m < 9; m++) {
            C1[item * 9 + m] = c[m];
            C2[item * 9 + m] = c[m];
        }
    }
}


// ---------------------------------------------------------------------------
// FP32 far-field quadrature (mixed precision).
//
// The reference's time integrals carry the absolute time T through terms like
// T^2 b^2 / (12 r^2) that cancel in the step response; in FP32 that loses
// ~(T/dt)^2 of the 24 mantissa bits.  With tau = T - r/c (time since the front
// passed the point, b = clamp(tau, 0, dt)) and rho = r/c, the rho^2 part of those
// polynomials cancels the -(dt b - b^2/2)/c^2 (and -(b^2/2)/c^2) terms exactly:
//   I1 = (rho Q1 + Q0) / (12 r^2 dt),  J1 = (rho R1 + R0) / (12 r^2 dt)
//   Q1 = 8b^3 - 12 tau b^2 - 12 dt b^2 + 24 dt tau b
//   Q0 = -3b^4 + (8 tau + 4 dt) b^3 - 6 tau^2 b^2 - 12 tau dt b^2 + 12 dt tau^2 b
//   R1 = -8b^3 + 12 tau b^2,   R0 = 3b^4 - 8 tau b^3 + 6 tau^2 b^2
// (GreenFunctionT.cpp:271-277 with T = rho + tau).  Only differences of
// polynomials in tau remain, whose relative error is ~ eps32 * T/dt.
// ---------------------------------------------------------------------------
struct PhysF {
    float dt, inv_dt, inv_cp, inv_cs, inv_cp2, inv_cs2, cs2, ratio2, ratio3, inv_4pi_rho,
        inv_4pi, c4;  // c4 = 1 - 2 (cs/cp)^2
    float dt_below;   // the largest float below dt
};

// A point's FP32 tau = T - r/c is off by at most ~8 eps (T + r/c) (T = k dt and r/c
// each rounded, r from FP32 offsets); within 64 eps (T + dt + r/c_p) of a threshold
// of the time integrals' regimes (tau of some evaluation time at 0 or dt, where the
// step terms I5/J5 jump and the exact-zero skips switch) the regimes are decided in
// FP64 as the FP64 quadrature decides them.
constexpr float kTauMargin = 64.f / 16777216.f;

__host__ __device__ __forceinline__ PhysF to_f(const Phys& p) {
    PhysF f;
    f.dt = (float)p.dt;
    f.inv_dt = (float)p.inv_dt;
    f.inv_cp = (float)p.inv_cp;
    f.inv_cs = (float)p.inv_cs;
    f.inv_cp2 = (float)p.inv_cp2;
    f.inv_cs2 = (float)p.inv_cs2;
    f.cs2 = (float)p.cs2;
    f.ratio2 = (float)p.ratio2;
    f.ratio3 = (float)p.ratio3;
    f.inv_4pi_rho = (float)p.inv_4pi_rho;
    f.inv_4pi = (float)p.inv_4pi;
    f.c4 = (float)(1 - 2 * p.ratio2);
    f.dt_below = nextafterf(f.dt, 0.f);
    return f;
}

// FP32 tau in the regime that FP64 gives tr (wave_I / wave_J: dt <= tr, 0 <= tr < dt,
// tr < 0).
__device__ __forceinline__ float snap_tau(double tr, double dt, const PhysF& f) {
    const float t = (float)tr;
    if (dt <= tr) return fmaxf(t, f.dt);
    if (0 <= tr) return fminf(fmaxf(t, 0.f), f.dt_below);
    return t < 0.f ? t : -1e-30f;
}

struct FrontTaus {
    float p[4], s[4];
};

// The taus of both waves at TI = k dt, TI - dt, TJ = (k+1) dt, TJ - dt from the FP64
// point, node and times of the FP64 quadrature (point_kernels, time_consts), snapped
// into its regimes.  Kept out of line: it runs for the few points near a front, and
// inlined its FP64 temporaries would cost the FP32 point loop registers.
__device__ __noinline__ FrontTaus front_taus(const double* xq64, const double* xc64, int k,
                                             const Phys& ph, const PhysF& f) {
    const double e0 = xq64[0] - xc64[0], e1 = xq64[1] - xc64[1], e2 = xq64[2] - xc64[2];
    const double r64 = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
    const double rp = r64 * ph.inv_cp, rs = r64 * ph.inv_cs;
    const double TI0 = k * ph.dt, TJ0 = (k + 1) * ph.dt;
    const double T4[4] = {TI0, TI0 - ph.dt, TJ0, TJ0 - ph.dt};
    FrontTaus t;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        t.p[i] = snap_tau(T4[i] - rp, ph.dt, f);
        t.s[i] = snap_tau(T4[i] - rs, ph.dt, f);
    }
    return t;
}

// One wave at local time tau: F_I = rho Q1 + Q0, I3, I5 and F_J = rho R1 + R0, J3, J5.
__device__ __forceinline__ void wave_tau_I(float tau, float rho, const PhysF& f, float& FI,
                                           float& I3, float& I5) {
    // b = clamp(tau, 0, dt); the I5 term lives on 0 <= tau < dt (GreenFunctionT.cpp:251-269)
    const float b = fminf(fmaxf(tau, 0.f), f.dt);
    const float x5 = (tau >= 0.f && tau < f.dt) ? (f.dt - tau) * f.inv_dt : 0.f;
    const float b2 = b * b;
    const float q1 = b * (8.f * b2 - 12.f * tau * b - 12.f * f.dt * b + 24.f * f.dt * tau);
    const float q0 = b * (b2 * (-3.f * b + 8.f * tau + 4.f * f.dt) - 6.f * tau * tau * b -
                          12.f * tau * f.dt * b + 12.f * f.dt * tau * tau);
    FI = rho * q1 + q0;
    I3 = b * (f.dt - 0.5f * b) * f.inv_dt;
    I5 = x5;
}

__device__ __forceinline__ void wave_tau_J(float tau, float rho, const PhysF& f, float& FJ,
                                           float& J3, float& J5) {
    const float b = fminf(fmaxf(tau, 0.f), f.dt);
    const float x5 = (tau >= 0.f && tau < f.dt) ? tau * f.inv_dt : 0.f;
    const float b2 = b * b;
    const float r1 = b2 * (-8.f * b + 12.f * tau);
    const float r0 = b2 * (3.f * b2 - 8.f * tau * b + 6.f * tau * tau);
    FJ = rho * r1 + r0;
    J3 = 0.5f * b2 * f.inv_dt;
    J5 = x5;
}

struct ItemAccF {
    float g[4][6];
    float h[4][9];
};

// One Gauss point of a far item in FP32: TI = k dt (I part), TJ = (k+1) dt (J part).
// xq64, xc64, k, ph: the point, the node and the level in FP64, for the regime
// decisions of points near a wave front.
__device__ __forceinline__ void gauss_point_f32(ItemAccF& acc, bool doI0, bool doJ0, float TI,
                                                const PhysF& f, const float xc[3],
                                                const float xq[3], const float nq[3], float wJ,
                                                const float N[4], const double* xq64,
                                                const double* xc64, int k, const Phys& ph) {
    const float d0 = xq[0] - xc[0], d1 = xq[1] - xc[1], d2 = xq[2] - xc[2];
    const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const float inv_r = rsqrtf(r2);
    const float r = r2 * inv_r;
    const float rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
    const float rdn = rv[0] * nq[0] + rv[1] * nq[1] + rv[2] * nq[2];
    const float rho_p = r * f.inv_cp, rho_s = r * f.inv_cs;
    const float tp = TI - rho_p, ts = TI - rho_s;  // tau of each wave at T = TI
    // tau of each wave at the part's times: [0] TI, [1] TI - dt (I part), [2] TI + dt,
    // [3] TI (J part)
    float tP[4] = {tp, tp - f.dt, tp + f.dt, tp}, tS[4] = {ts, ts - f.dt, ts + f.dt, ts};
    {
        const float m = kTauMargin * (TI + f.dt + rho_p);
        auto near = [&](float t) {
            return fminf(fminf(fabsf(t + f.dt), fabsf(t)), fminf(fabsf(t - f.dt),
                                                                 fabsf(t - 2.f * f.dt))) < m;
        };
        if (near(tp) || near(ts)) {  // regimes from FP64, as the FP64 quadrature has them
            const FrontTaus t = front_taus(xq64, xc64, k, ph, f);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                tP[i] = t.p[i];
                tS[i] = t.s[i];
            }
        }
    }
    // exact zero once the S front has passed at both times of a part, and before the
    // P front arrives (b = 0 and no I5/J5 step at both times of the part: every term
    // of the part is then exactly zero)
    const bool doI = doI0 && !(tS[1] >= f.dt) && !(tP[0] < 0.f);
    const bool doJ = doJ0 && !(tS[3] >= f.dt) && !(tP[2] < 0.f);
    if (!doI && !doJ) return;
    float P1 = 0.f, P3 = 0.f, P5 = 0.f, S2 = 0.f, S4 = 0.f, S6 = 0.f;
    float a1, a3, a5, b1, b3, b5;
    if (doI) {
        wave_tau_I(tP[0], rho_p, f, a1, a3, a5);
        wave_tau_I(tP[1], rho_p, f, b1, b3, b5);
        P1 = a1 - b1; P3 = a3 - b3; P5 = a5 - b5;
        wave_tau_I(tS[0], rho_s, f, a1, a3, a5);
        wave_tau_I(tS[1], rho_s, f, b1, b3, b5);
        S2 = a1 - b1; S4 = a3 - b3; S6 = a5 - b5;
    }
    if (doJ) {
        wave_tau_J(tP[2], rho_p, f, a1, a3, a5);
        wave_tau_J(tP[3], rho_p, f, b1, b3, b5);
        P1 += a1 - b1; P3 += a3 - b3; P5 += a5 - b5;
        wave_tau_J(tS[2], rho_s, f, a1, a3, a5);
        wave_tau_J(tS[3], rho_s, f, b1, b3, b5);
        S2 += a1 - b1; S4 += a3 - b3; S6 += a5 - b5;
    }
    const float inv_r2 = inv_r * inv_r;
    const float scale1 = inv_r2 * (1.f / 12.f) * f.inv_dt;  // 1/(12 r^2 dt) of I1/J1
    P1 *= scale1;
    S2 *= scale1;
    const float It1 = 0.5f * (P1 - S2);
    const float It2u = P3 * f.inv_cp2 - S4 * f.inv_cs2;
    const float invDiv = inv_r * f.inv_4pi_rho;
    const float A = (3.f * It1 + It2u) * invDiv;
    const float B = (S4 * f.inv_cs2 - It1) * invDiv;
    const float It2t = S4 - f.ratio2 * P3;
    const float It3t = S6 - f.ratio3 * P5;
    const float It4 = P3 + rho_p * P5;
    const float It5 = S4 + rho_s * S6;
    const float ir2 = inv_r2 * f.inv_4pi;
    const float Q = 6.f * f.cs2 * It1 - 2.f * It2t;
    const float alpha = ((-30.f * f.cs2) * It1 + 12.f * It2t) * ir2 +
                        (2.f * f.inv_cs * f.inv_4pi) * inv_r * It3t;
    const float beta = (Q - f.c4 * It4) * ir2;
    const float gamma = (Q - It5) * ir2;
    const float rr00 = rv[0] * rv[0], rr01 = rv[0] * rv[1], rr02 = rv[0] * rv[2];
    const float rr11 = rv[1] * rv[1], rr12 = rv[1] * rv[2], rr22 = rv[2] * rv[2];
    const float sg[6] = {A * rr00 + B, A * rr01, A * rr02, A * rr11 + B, A * rr12, A * rr22 + B};
    const float ar = alpha * rdn, gd = gamma * rdn;
    const float rrm[9] = {rr00, rr01, rr02, rr01, rr11, rr12, rr02, rr12, rr22};
    float th[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            th[i * 3 + j] = ar * rrm[i * 3 + j] + beta * (nq[j] * rv[i]) +
                            gamma * (nq[i] * rv[j]) + (i == j ? gd : 0.f);
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const float w = wJ * N[a];
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] += w * sg[m];
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] += w * th[m];
    }
}

// One far (well-separated, non-singular) item in FP32: collocation node c,
// element e, level k (I part at k dt, J part at (k+1) dt), added into the FP32
// level store.  Gauss-point geometry comes from the FP32 table (points relative to
// the element's first node); no FP64 arithmetic in the point loop, which on GB300
// would run on the narrow FP64 pipe.
template <typename T>
__device__ __forceinline__ T* far_out(const AsmOut& o, int which);
template <>
__device__ __forceinline__ float* far_out<float>(const AsmOut& o, int which) {
    return which == 0 ? o.G0f : o.H0f;
}
template <>
__device__ __forceinline__ double* far_out<double>(const AsmOut& o, int which) {
    return which == 0 ? o.G0 : o.H0;
}

// Adds s times an item's 4 node blocks (G as symmetric 6-vectors, H as 3x3) into the
// 3 rows at rowbase of a level store with leading dimension D, as reductions
// (red.global.add): none waits for a read of the store, where a read-modify-write
// would wait for every read in turn (as far as the compiler knows G and H, and two
// nodes' columns, may alias).  The order of the adds into one entry is still fixed:
// all of an entry's adds come from one block (the block owns its node's rows), at
// most one per colour, and a barrier separates the colours, so each add is performed
// before the next colour's (bitwise reproducible).  The FP32 reduction flushes
// subnormal values to zero (below 1.2e-38, far under the store's resolution).
template <typename T>
__device__ __forceinline__ void add_node_blocks(T* G, T* H, size_t rowbase, size_t D,
                                                const int nid[4], const ItemAccF& acc,
                                                float s) {
    constexpr int sym[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const size_t col = rowbase + 3 * (size_t)nid[a];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                atomicAdd(G + col + (size_t)i * D + j, (T)(s * acc.g[a][sym[i * 3 + j]]));
                atomicAdd(H + col + (size_t)i * D + j, (T)(s * acc.h[a][i * 3 + j]));
            }
    }
}

template <typename T>
__device__ __forceinline__ void far_item(const double* __restrict__ coords,
                                         const int* __restrict__ ien, int c, int e, int k,
                                         int nq2, const float* __restrict__ geomf,
                                         const double* __restrict__ geom,
                                         const float* __restrict__ coordf, const PhysF& f,
                                         const Phys& ph, float TI, int level_last,
                                         const AsmOut& out) {
    int nid[4];
#pragma unroll
    for (int a = 0; a < 4; a++) nid[a] = ien[e * 4 + a];
    // collocation point relative to the element's first node from the coordinates'
    // FP32 pairs, (hi - hi) + (lo - lo): ~1.5 eps relative, no FP64 arithmetic
    const float4* cf4 = reinterpret_cast<const float4*>(coordf);
    const float4 ch = __ldg(cf4 + 2 * c), cl = __ldg(cf4 + 2 * c + 1);
    const float4 eh = __ldg(cf4 + 2 * nid[0]), el = __ldg(cf4 + 2 * nid[0] + 1);
    const float xc[3] = {(ch.x - eh.x) + (cl.x - el.x), (ch.y - eh.y) + (cl.y - el.y),
                         (ch.z - eh.z) + (cl.z - el.z)};
    const bool doI = (k >= 1), doJ = (k + 1 <= level_last);
    ItemAccF acc;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] = 0.f;
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] = 0.f;
    }
    const float4* g4 = reinterpret_cast<const float4*>(geomf + (size_t)e * nq2 * kGeomStride);
    for (int q = 0; q < nq2; q++) {
        const float4 p0 = __ldg(g4 + 3 * q), p1 = __ldg(g4 + 3 * q + 1), p2 = __ldg(g4 + 3 * q + 2);
        const float xq[3] = {p0.x, p0.y, p0.z};
        const float nqv[3] = {p0.w, p1.x, p1.y};
        const float N[4] = {p1.w, p2.x, p2.y, p2.z};
        gauss_point_f32(acc, doI, doJ, TI, f, xc, xq, nqv, p1.z, N,
                        geom + ((size_t)e * nq2 + q) * kGeomStride, coords + 3 * c, k, ph);
    }
    const size_t D = (size_t)out.ld;
    add_node_blocks<T>(far_out<T>(out, 0), far_out<T>(out, 1),
                       (size_t)k * out.level_stride + (size_t)(3 * c) * D, D, nid, acc, 1.f);
}

// Settled far items.  At level k the P front has passed every Gauss point of the
// element at all four evaluation times of the level (TI - dt - r/c_p >= dt) and the S
// front reaches none of them (TJ - r/c_s < 0, TJ = TI + dt).  Every tau of the P wave
// is then >= dt (b = dt, no I5/J5 step, I3 and J3 constant) and the S wave's terms are
// all zero, so the differences of the tau polynomials reduce to
//   Q1(tau) - Q1(tau - dt) + R1(tau + dt) - R1(tau) = 24 dt^3,
//   Q0(tau) - Q0(tau - dt) + R0(tau + dt) - R0(tau) = 24 tau dt^3 - 12 dt^4,
// and with rho + tau = TI: P1 = 2 dt^2 (TI - dt/2) / r^2, It1 = dt^2 (TI - dt/2) / r^2,
// every other time integral zero.  The level's blocks are (TI - dt/2) times one
// time-independent block of the pair (the quasi-static kernel):
//   G: dt^2 / (4 pi rho r^3) (3 r r^T - I)
//   H: 6 c_s^2 dt^2 / (4 pi r^4) (-5 (r.n) r r^T + r n^T + n r^T + (r.n) I)
// (GreenFunctionT.cpp:241-446 and TDElementStepLinearT.cpp:28-125 evaluated in that
// regime), so a pair's settled levels take one pass over its Gauss points and one
// scaled add per level.  The range is decided from FP32 distances with margins that
// only narrow it (a level at a regime threshold takes the general quadrature).
constexpr float kSettledRel = 1e-5f;  // relative margin on FP32 point distances
constexpr float kSettledAbs = 1e-3f;  // margin in levels

// Levels slo..shi at which pair (c, e) is settled (empty if slo > shi).
__device__ __forceinline__ void settled_range(const int* __restrict__ ien, int c, int e,
                                              int nq2, const float* __restrict__ geomf,
                                              const float* __restrict__ coordf,
                                              const PhysF& f, int& slo, int& shi) {
    const int n0 = ien[e * 4];
    const float4* cf4 = reinterpret_cast<const float4*>(coordf);
    const float4 ch = __ldg(cf4 + 2 * c), cl = __ldg(cf4 + 2 * c + 1);
    const float4 eh = __ldg(cf4 + 2 * n0), el = __ldg(cf4 + 2 * n0 + 1);
    const float x0 = (ch.x - eh.x) + (cl.x - el.x), x1 = (ch.y - eh.y) + (cl.y - el.y),
                x2 = (ch.z - eh.z) + (cl.z - el.z);
    const float4* g4 = reinterpret_cast<const float4*>(geomf + (size_t)e * nq2 * kGeomStride);
    float r2min = 3.4e38f, r2max = 0.f;
#pragma unroll 4
    for (int q = 0; q < nq2; q++) {
        const float4 p = __ldg(g4 + 3 * q);
        const float d0 = p.x - x0, d1 = p.y - x1, d2 = p.z - x2;
        const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
        r2min = fminf(r2min, r2);
        r2max = fmaxf(r2max, r2);
    }
    const float rmax = sqrtf(r2max) * (1.f + kSettledRel);
    const float rmin = sqrtf(r2min) * (1.f - kSettledRel);
    // P passed at TI - dt: k >= 2 + r/(c_p dt) at the farthest point
    slo = (int)ceilf(2.f + rmax * f.inv_cp * f.inv_dt + kSettledAbs);
    // S short of the nearest point at TJ: k + 1 < r/(c_s dt), i.e. k <= ceil(y) - 2
    shi = (int)ceilf(rmin * f.inv_cs * f.inv_dt - kSettledAbs) - 2;
}

// A settled job: pair (c, e) at levels ks .. ks + ns - 1, all settled.
template <typename T>
__device__ __forceinline__ void settled_job(const int* __restrict__ ien, int c, int e, int ks,
                                            int ns, int nq2, const float* __restrict__ geomf,
                                            const float* __restrict__ coordf, const PhysF& f,
                                            const AsmOut& out) {
    int nid[4];
#pragma unroll
    for (int a = 0; a < 4; a++) nid[a] = ien[e * 4 + a];
    const float4* cf4 = reinterpret_cast<const float4*>(coordf);
    const float4 ch = __ldg(cf4 + 2 * c), cl = __ldg(cf4 + 2 * c + 1);
    const float4 eh = __ldg(cf4 + 2 * nid[0]), el = __ldg(cf4 + 2 * nid[0] + 1);
    const float xc[3] = {(ch.x - eh.x) + (cl.x - el.x), (ch.y - eh.y) + (cl.y - el.y),
                         (ch.z - eh.z) + (cl.z - el.z)};
    ItemAccF acc;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int m = 0; m < 6; m++) acc.g[a][m] = 0.f;
#pragma unroll
        for (int m = 0; m < 9; m++) acc.h[a][m] = 0.f;
    }
    const float dt2 = f.dt * f.dt;
    const float h6 = 6.f * f.cs2 * f.inv_4pi;
    const float4* g4 = reinterpret_cast<const float4*>(geomf + (size_t)e * nq2 * kGeomStride);
    for (int q = 0; q < nq2; q++) {
        const float4 p0 = __ldg(g4 + 3 * q), p1 = __ldg(g4 + 3 * q + 1), p2 = __ldg(g4 + 3 * q + 2);
        const float nq[3] = {p0.w, p1.x, p1.y};
        const float N[4] = {p1.w, p2.x, p2.y, p2.z};
        const float d0 = p0.x - xc[0], d1 = p0.y - xc[1], d2 = p0.z - xc[2];
        const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
        const float inv_r = rsqrtf(r2);
        const float rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
        const float rdn = rv[0] * nq[0] + rv[1] * nq[1] + rv[2] * nq[2];
        const float u = dt2 * inv_r * inv_r;       // It1 / (TI - dt/2)
        const float ga = u * inv_r * f.inv_4pi_rho;  // A = 3 ga, B = -ga
        const float hb = h6 * u * inv_r * inv_r;     // beta = gamma = hb, alpha = -5 hb
        const float ga3 = 3.f * ga;
        const float rr00 = rv[0] * rv[0], rr01 = rv[0] * rv[1], rr02 = rv[0] * rv[2];
        const float rr11 = rv[1] * rv[1], rr12 = rv[1] * rv[2], rr22 = rv[2] * rv[2];
        const float sg[6] = {ga3 * rr00 - ga, ga3 * rr01, ga3 * rr02,
                             ga3 * rr11 - ga, ga3 * rr12, ga3 * rr22 - ga};
        const float ar = -5.f * hb * rdn, gd = hb * rdn;
        const float rrm[9] = {rr00, rr01, rr02, rr01, rr11, rr12, rr02, rr12, rr22};
        float th[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
                th[i * 3 + j] = ar * rrm[i * 3 + j] + hb * (nq[j] * rv[i] + nq[i] * rv[j]) +
                                (i == j ? gd : 0.f);
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const float w = p1.z * N[a];
#pragma unroll
            for (int m = 0; m < 6; m++) acc.g[a][m] += w * sg[m];
#pragma unroll
            for (int m = 0; m < 9; m++) acc.h[a][m] += w * th[m];
        }
    }
    const size_t D = (size_t)out.ld;
    for (int k = ks; k < ks + ns; k++)  // scaled by TI - dt/2
        add_node_blocks<T>(far_out<T>(out, 0), far_out<T>(out, 1),
                           (size_t)k * out.level_stride + (size_t)(3 * c) * D, D, nid, acc,
                           ((float)k - 0.5f) * f.dt);
}

constexpr int kFarBlock = 128;  // threads of a far-field block
#ifndef TDBEM_FAR_CHUNK
#define TDBEM_FAR_CHUNK 8
#endif
#ifndef TDBEM_FAR_MIN_BLOCKS
#define TDBEM_FAR_MIN_BLOCKS 4
#endif
constexpr int kFarChunk = TDBEM_FAR_CHUNK;  // levels of a far-field block (at most 256)
constexpr int kFarCodeBits = 8;             // level offset bits of a compacted item code
static_assert(kFarChunk >= 1 && kFarChunk <= (1 << kFarCodeBits), "far-field level chunk");

// Exclusive scan of one value per thread over the block; returns the block total.
__device__ __forceinline__ int far_block_scan(int v, int& excl, int* s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    int before = 0, total = 0;
#pragma unroll
    for (int i = 0; i < kFarBlock / 32; i++) {
        const int t = s_warp[i];
        before += i < w ? t : 0;
        total += t;
    }
    excl = before + x - v;
    __syncthreads();  // s_warp is reused by the next scan
    return total;
}

// Capacity of a far-field block's item and settled-job lists (one colour's worth
// at a time; flushed earlier when a colour's elements hold more).
constexpr int kFarItemCap = 2 * kFarBlock * kFarChunk;
constexpr int kFarJobCap = 4 * kFarBlock;

// All far items of collocation node c = blockIdx.x at levels [k0, k0 + kFarChunk),
// k0 = blockIdx.y * kFarChunk.  The block owns those rows of those levels, so it
// walks the element colours in order (elements of one colour share no node:
// their items write distinct entries) with a barrier between colours: every add
// to a row lands while the rows are resident in L2, in a fixed order (bitwise
// reproducible), and one launch covers all colours.  The candidate items (element,
// level) of a colour's elements, kFarBlock elements at a time, are compacted with
// one block scan per chunk into the colour's list, which the threads then work
// through in one pass (a list about to overflow is worked through first).
// pairs[c * nel + j] is the window of node c and the j-th element in colour order.
// A pair's settled levels (settled_range) leave its item list and go to one settled
// job; the items come first in the thread order and the jobs after them, so most
// warps hold one kind of work.  level_top: the highest level any window reaches.
// f: ph's FP32 constants, converted on the host.  Kernel parameters are operands of
// the FP32 instructions as they stand; converted in the kernel, they were re-derived
// from ph at their uses (one FP64-to-FP32 conversion each, ~14 per Gauss point) to
// save registers, and GB300 runs conversions on its narrow FP64 pipe.
// nitems (if not null) receives the item, job and settled-level counts.
template <typename T>
__global__ void __launch_bounds__(kFarBlock, TDBEM_FAR_MIN_BLOCKS) k_assemble_far_rows(
    const double* __restrict__ coords, const int* __restrict__ ien,
    const int* __restrict__ color_elems, const int* __restrict__ color_start, int ncolor,
    int nel, int nq2, const float* __restrict__ geomf, const double* __restrict__ geom,
    const float* __restrict__ coordf, Phys ph, PhysF f, int level_last, int level_top,
    const PairInfo* __restrict__ pairs, AsmOut out, unsigned long long* __restrict__ nitems) {
    __shared__ int s_warp[kFarBlock / 32];
    __shared__ int s_items[kFarItemCap];          // (element in colour) << bits | level
    __shared__ int s_jobs[kFarJobCap];            // element in colour
    __shared__ unsigned short s_jobl[kFarJobCap];  // first level << 8 | levels - 1
    const int c = blockIdx.x;
    const int k0 = blockIdx.y * kFarChunk;
    const int k1 = min(k0 + kFarChunk, level_top + 1);
    // settled levels need both parts (1 <= k <= level_last - 1) and k >= 2
    const bool settle = k1 - 1 >= 2 && level_last >= 3;
    const PairInfo* pc = pairs + (size_t)c * nel;
    unsigned long long count = 0, njobs = 0, nsettled = 0;
    for (int col = 0; col < ncolor; col++) {
        const int j0 = color_start[col], j1 = color_start[col + 1];
        // work through the list: items [0, ni), then jobs [0, nj)
        auto work = [&](int ni, int nj) {
            for (int i = threadIdx.x; i < ni + nj; i += kFarBlock) {
                if (i < ni) {
                    const int code = s_items[i];
                    const int k = k0 + (code & ((1 << kFarCodeBits) - 1));
                    far_item<T>(coords, ien, c, color_elems[j0 + (code >> kFarCodeBits)], k,
                                nq2, geomf, geom, coordf, f, ph, (float)k * f.dt, level_last,
                                out);
                } else {
                    const int jl = s_jobl[i - ni];
                    settled_job<T>(ien, c, color_elems[j0 + s_jobs[i - ni]], k0 + (jl >> 8),
                                   (jl & 0xff) + 1, nq2, geomf, coordf, f, out);
                }
            }
        };
        int ni = 0, nj = 0;  // the colour's list so far (uniform over the block)
        for (int base = j0; base < j1; base += kFarBlock) {
            const int j = base + (int)threadIdx.x;
            int na = 0, lo = 0, ss = 0, sn = 0;
            if (j < j1) {
                const PairInfo pi = pc[j];
                lo = max(k0, pi.klo);
                na = max(0, min(k1, pi.klo + pi.cnt) - lo);
                if (settle && na > 0) {
                    int slo, shi;
                    settled_range(ien, c, color_elems[j], nq2, geomf, coordf, f, slo, shi);
                    slo = max(slo, lo);
                    shi = min(shi, min(lo + na - 1, level_last - 1));
                    if (shi >= slo) {
                        ss = slo;
                        sn = shi - slo + 1;
                    }
                }
            }
            // items in the low 16 bits, the job in the high ones (chunk totals < 2^16)
            int off;
            const int tot = far_block_scan((na - sn) | ((sn > 0 ? 1 : 0) << 16), off, s_warp);
            const int ti = tot & 0xffff, tj = tot >> 16;
            if (ni + ti > kFarItemCap || nj + tj > kFarJobCap) {
                // the chunks so far are written (the scan's barriers follow them)
                work(ni, nj);
                __syncthreads();  // the list is rewritten next
                ni = nj = 0;
            }
            int oi = ni + (off & 0xffff);
            for (int k = lo; k < lo + na; k++)
                if (k < ss || k >= ss + sn)
                    s_items[oi++] = ((j - j0) << kFarCodeBits) | (k - k0);
            if (sn > 0) {
                const int oj = nj + (off >> 16);
                s_jobs[oj] = j - j0;
                s_jobl[oj] = (unsigned short)(((ss - k0) << 8) | (sn - 1));
            }
            ni += ti;
            nj += tj;
            count += ti;
            njobs += tj;
            nsettled += sn;
        }
        __syncthreads();
        work(ni, nj);
        // the list is rebuilt next; this colour's adds come before the next colour's
        __syncthreads();
    }
    if (nitems) {
        if (threadIdx.x == 0 && count) atomicAdd(nitems, count);
        if (threadIdx.x == 0 && njobs) atomicAdd(nitems + 1, njobs);
        const unsigned w = __reduce_add_sync(0xffffffffu, (unsigned)nsettled);
        if ((threadIdx.x & 31) == 0 && w) atomicAdd(nitems + 2, (unsigned long long)w);
    }
}

// C term (TDElementStepLinearT.cpp:103-109, 501-508, 577-584 with AssembleC,
// ElastoDynamicsT.cpp:261-280): C_c = -sum_e sum_q wJ DT_Kelvin(q)^T over the whole
// surface, with the reference's regular / Duffy quadrature per element.  One
// block per node, fixed-order tree reduction; the result goes to cbuf[c][9].
// C term of node c, computed by the whole block (256 threads), into dst[9].  A
// singular 8-node element contributes through its 4-node sub-elements.  FAST (the
// mixed-precision assembly): a regular element's points in FP32, summed in FP32
// per element and across a thread's elements with a TwoSum compensation term
// (Knuth's error-free addition: the pair (sum, compensation) carries the sum to
// ~1e-14), in FP64 across threads; relative error ~1e-7 of C.  For 4-node elements
// from the FP32 geometry table (points relative to the element's first node) and
// the node's offset to that node from the coordinates' FP32 pairs (coordf), so no
// FP64 arithmetic per regular element but the singular filter; for 8-node elements
// from the FP64 points' offsets to the node.  Singular elements as in the FP64
// form.  ebox (may be null): the mesh's element boxes; an element whose node
// radius the node is kSingularClear beyond skips the singular test (and the loads
// of its nodes).  onem2nu_f, kscale_f: the FAST path's FP32 constants, converted
// on the host.
template <int ENND = 4, bool FAST = false>
__device__ __forceinline__ void cterm_node(const double* __restrict__ coords,
                                           const int* __restrict__ ien, int nel, int c, int nq,
                                           const double* __restrict__ gx,
                                           const double* __restrict__ gw,
                                           const double* __restrict__ geom, const Phys& ph,
                                           double* __restrict__ dst,
                                           const float* __restrict__ geomf = nullptr,
                                           const float* __restrict__ coordf = nullptr,
                                           const ElemBox* __restrict__ ebox = nullptr,
                                           float onem2nu_f = 0.f, float kscale_f = 0.f,
                                           const double* __restrict__ duffy = nullptr) {
    const double xc[3] = {coords[c * 3], coords[c * 3 + 1], coords[c * 3 + 2]};
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float s32[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, e32[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int nq2 = nq * nq;
    const double onem2nu = 1 - 2 * ph.nu;
    // Kelvin_Linear (GreenFunctionT.cpp:205-231): K = [..] / (-8 pi (1-nu) r^2) * 0.5 dt
    const double kscale = (0.5 * ph.dt) / (-(8 * M_PI) * (1 - ph.nu));
    constexpr int stride = ENND == 8 ? kGeomStride8 : kGeomStride;
    const bool pairs4 = FAST && ENND == 4 && geomf && coordf;
    // C[i][k] -= wJ K[k][i] at an FP64 point
    auto kelvin64 = [&](const double xq[3], const double nv[3], double wJ) {
        const double d0 = xq[0] - xc[0], d1 = xq[1] - xc[1], d2 = xq[2] - xc[2];
        const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
        const double inv_r = 1.0 / sqrt(r2);
        const double rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
        const double rdn = rv[0] * nv[0] + rv[1] * nv[1] + rv[2] * nv[2];
        const double w = wJ * (kscale * inv_r * inv_r);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int kk = 0; kk < 3; kk++) {
                const double Kki = ((kk == i ? onem2nu : 0.0) + 3 * rv[kk] * rv[i]) * rdn -
                                   onem2nu * (rv[i] * nv[kk] - rv[kk] * nv[i]);
                acc[i * 3 + kk] -= w * Kki;
            }
    };
    // Rounds of one element per thread (blockDim.x = 256).  A regular element is summed
    // by its thread.  The round's singular elements (the node's few) are listed in
    // thread order and their Duffy points spread over the block: summed by their own
    // threads, 2 nq^2 FP64 points per sub-element would keep single lanes busy on the
    // FP64 pipe while the rest of their warps wait.
    __shared__ int s_sing[256];  // element << 3 | singular corner
    __shared__ int s_wcnt[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int base = 0; base < nel; base += blockDim.x) {
        const int e = base + threadIdx.x;
        int sing = -1;
        if (e < nel) {
            bool near = true;
            if (ebox) {
                const ElemBox b = ebox[e];
                const double dx = xc[0] - b.x, dy = xc[1] - b.y, dz = xc[2] - b.z;
                const double lim = b.rad + kSingularClear;
                near = dx * dx + dy * dy + dz * dz <= lim * lim;
            }
            if (near) {
                double en[3 * ENND];
                for (int a = 0; a < ENND; a++) {
                    const int nid = ien[e * ENND + a];
                    for (int d = 0; d < 3; d++) en[a * 3 + d] = coords[nid * 3 + d];
                }
                sing = singular_corner<ENND>(en, xc);
            }
            if (FAST && sing < 0) {
                float a32[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                // the node relative to the element's first node (4-node FP32 table), from
                // the FP32 pairs (hi - hi) + (lo - lo): ~1.5 eps relative
                float xr[3] = {0.f, 0.f, 0.f};
                if (pairs4) {
                    const float4* cf4 = reinterpret_cast<const float4*>(coordf);
                    const int n0 = ien[e * 4];
                    const float4 ch = __ldg(cf4 + 2 * c), cl = __ldg(cf4 + 2 * c + 1);
                    const float4 eh = __ldg(cf4 + 2 * n0), el = __ldg(cf4 + 2 * n0 + 1);
                    xr[0] = (ch.x - eh.x) + (cl.x - el.x);
                    xr[1] = (ch.y - eh.y) + (cl.y - el.y);
                    xr[2] = (ch.z - eh.z) + (cl.z - el.z);
                }
                for (int qq = 0; qq < nq2; qq++) {
                    float d0, d1, d2, nv[3], wJf;
                    if (pairs4) {
                        const float4* g4 =
                            reinterpret_cast<const float4*>(geomf + ((size_t)e * nq2 + qq) * 12);
                        const float4 p0 = __ldg(g4), p1 = __ldg(g4 + 1);
                        d0 = p0.x - xr[0];
                        d1 = p0.y - xr[1];
                        d2 = p0.z - xr[2];
                        nv[0] = p0.w;
                        nv[1] = p1.x;
                        nv[2] = p1.y;
                        wJf = p1.z;
                    } else {
                        const double* g = geom + ((size_t)e * nq2 + qq) * stride;
                        d0 = (float)(g[0] - xc[0]);
                        d1 = (float)(g[1] - xc[1]);
                        d2 = (float)(g[2] - xc[2]);
                        nv[0] = (float)g[3];
                        nv[1] = (float)g[4];
                        nv[2] = (float)g[5];
                        wJf = (float)g[6];
                    }
                    const float inv_r = rsqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    const float rv[3] = {d0 * inv_r, d1 * inv_r, d2 * inv_r};
                    const float rdn = rv[0] * nv[0] + rv[1] * nv[1] + rv[2] * nv[2];
                    const float w = wJf * (kscale_f * inv_r * inv_r);
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int kk = 0; kk < 3; kk++) {
                            const float Kki = ((kk == i ? onem2nu_f : 0.f) + 3.f * rv[kk] * rv[i]) * rdn -
                                              onem2nu_f * (rv[i] * nv[kk] - rv[kk] * nv[i]);
                            a32[i * 3 + kk] -= w * Kki;
                        }
                }
                // TwoSum: t = s + a exactly as t + err
#pragma unroll
                for (int m = 0; m < 9; m++) {
                    const float t = s32[m] + a32[m];
                    const float z = t - s32[m];
                    e32[m] += (s32[m] - (t - z)) + (a32[m] - z);
                    s32[m] = t;
                }
            } else if (sing < 0) {
                for (int qq = 0; qq < nq2; qq++) {
                    const double* g = geom + ((size_t)e * nq2 + qq) * stride;
                    const double xq[3] = {g[0], g[1], g[2]}, nv[3] = {g[3], g[4], g[5]};
                    kelvin64(xq, nv, g[6]);
                }
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, sing >= 0);
        if (lane == 0) s_wcnt[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < nwarp; w++) {
            const int n = s_wcnt[w];
            before += w < warp ? n : 0;
            total += n;
        }
        if (sing >= 0) s_sing[before + __popc(bal & ((1u << lane) - 1))] = (e << 3) | sing;
        __syncthreads();
        // point slots of a singular element: sub-elements (up to 2 for an 8-node element,
        // the element itself for a 4-node one) x 2 triangles x nq^2
        const int slots = (ENND == 8 ? 4 : 2) * nq2;
        for (int t = threadIdx.x; t < total * slots; t += blockDim.x) {
            const int code = s_sing[t / slots], qq = t % slots;
            const int es = code >> 3, sg = code & 7;
            if (ENND == 4 && duffy) {  // the mesh's Duffy table
                const double* g = duffy + (((size_t)es * 4 + sg) * slots + qq) * kGeomStride;
                const double xq[3] = {__ldg(g), __ldg(g + 1), __ldg(g + 2)};
                const double nv[3] = {__ldg(g + 3), __ldg(g + 4), __ldg(g + 5)};
                kelvin64(xq, nv, __ldg(g + 6));
                continue;
            }
            int ids[2][4] = {{0, 1, 2, 3}, {0, 1, 2, 3}}, cid[2] = {sg, sg};
            int nsub = 1;
            if (ENND == 8) nsub = q8_subelements(sg, ids, cid);
            const int se = qq / (2 * nq2), r = qq % (2 * nq2);
            if (se >= nsub) continue;
            double cn[12];
            for (int i = 0; i < 4; i++) {
                const int nid = ien[es * ENND + ids[se][i]];
                for (int d = 0; d < 3; d++) cn[i * 3 + d] = coords[nid * 3 + d];
            }
            const int tri = r / nq2, q = r % nq2, q1 = q / nq, q2 = q % nq;
            double N[4], xq[3], nv[3], wJ;
            duffy_point(cn, cid[se], tri, gx[q1], gx[q2], gw[q1] * gw[q2], N, xq, nv, wJ);
            kelvin64(xq, nv, wJ);
        }
        __syncthreads();  // s_sing and s_wcnt are rewritten in the next round
    }
    if (FAST) {
#pragma unroll
        for (int m = 0; m < 9; m++) acc[m] += (double)s32[m] + (double)e32[m];
    }
    __shared__ double red[9][256];
    for (int m = 0; m < 9; m++) red[m][threadIdx.x] = acc[m];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int m = 0; m < 9; m++) red[m][threadIdx.x] += red[m][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 9) dst[threadIdx.x] = red[threadIdx.x][0];
}

template <int ENND, bool FAST>
__global__ void __launch_bounds__(256) k_cterm(const double* __restrict__ coords,
                                               const int* __restrict__ ien, int nel,
                                               int node_lo, int nq,
                                               const double* __restrict__ gx,
                                               const double* __restrict__ gw,
                                               const double* __restrict__ geom, Phys ph,
                                               double* __restrict__ cbuf,
                                               const float* __restrict__ geomf,
                                               const float* __restrict__ coordf,
                                               const ElemBox* __restrict__ ebox,
                                               float onem2nu_f, float kscale_f,
                                               const double* __restrict__ duffy) {
    cterm_node<ENND, FAST>(coords, ien, nel, node_lo + blockIdx.x, nq, gx, gw, geom, ph,
                           cbuf + (size_t)blockIdx.x * 9, geomf, coordf, ebox, onem2nu_f,
                           kscale_f, duffy);
}

// Add C (+ the exterior free term 0.5 dt I, ElastoDynamicsT.cpp:212-225) to the
// diagonal blocks of the first step's I and J parts: levels 0 and 1 of a level
// store, or the H_I / H_J row blocks of a single-step call.
__global__ void k_cterm_apply(const double* __restrict__ cbuf, int node_lo, int nnodes,
                              double dt, int if_ext, int mode, AsmOut out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * 9) return;
    const int cl = t / 9, m = t % 9, i = m / 3, j = m % 3, c = node_lo + cl;
    const double v = cbuf[t] + ((if_ext && i == j) ? 0.5 * dt : 0.0);
    const size_t ld = (size_t)out.ld;
    if (mode == ASM_LEVELS) {
        const size_t off = (size_t)(3 * c + i) * ld + 3 * (size_t)c + j;
        if (out.H0f) {
            out.H0f[off] += (float)v;
            out.H0f[out.level_stride + off] += (float)v;
        } else {
            out.H0[off] += v;
            out.H0[out.level_stride + off] += v;
        }
    } else {
        const size_t roff = (size_t)(3 * cl + i) * ld + 3 * (size_t)c + j;
        out.H0[roff] += v;
        out.H1[roff] += v;
    }
}

// ---------------------------------------------------------------------------
// Grouped assembly: the pairs, items and C-term nodes of many meshes in one
// launch each.  gm[] holds one descriptor per mesh; a thread finds its mesh by
// binary search on the first pair (or node) of each mesh.  Meshes share no
// rows, so one launch per colour index stays free of write conflicts.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int group_of(const GroupAsm* __restrict__ gm, int nmesh, unsigned x,
                                        bool by_node) {
    int lo = 0, hi = nmesh - 1;  // last mesh whose first pair / node is <= x
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const unsigned b = by_node ? gm[mid].node_begin : gm[mid].pair_begin;
        if (b <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_pair_window_group(const GroupAsm* __restrict__ gm, int nmesh, unsigned npairs,
                                    PairInfo* __restrict__ pairs,
                                    unsigned* __restrict__ counts) {
    const unsigned p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const GroupAsm& g = gm[group_of(gm, nmesh, p, false)];
    const PairInfo pi = pair_window_info(g.coords, g.ien, g.elems, g.ne, 0, g.ph, ASM_LEVELS,
                                         g.level_last, g.level_cap, 0, SEL_ALL,
                                         (long long)(p - g.pair_begin));
    pairs[p] = pi;
    counts[p] = (unsigned)pi.cnt;
}

__global__ void __launch_bounds__(128) k_assemble_group(const GroupAsm* __restrict__ gm,
                                                        int nmesh,
                                                        const PairInfo* __restrict__ pairs,
                                                        const unsigned* __restrict__ offsets,
                                                        unsigned npairs, unsigned nitems) {
    unsigned p;
    if (!item_pair(offsets, npairs, nitems, p)) return;
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    const GroupAsm& g = gm[group_of(gm, nmesh, p, false)];
    const PairInfo pi = pairs[p];
    const int k = pi.klo + (int)(gid - __ldg(offsets + p));
    assemble_item<ASM_LEVELS>(g.coords, g.ien, g.elems, g.ne, 0, g.nq, g.gx, g.gw, g.geom, g.ph,
                              g.level_last, 0, 0, pi, p - g.pair_begin, k, g.out);
}

// One block per node of every mesh: the C term, then its application to levels 0
// and 1 of the mesh (+ 0.5 dt I for exterior problems), as k_cterm + k_cterm_apply.
__global__ void __launch_bounds__(256) k_cterm_group(const GroupAsm* __restrict__ gm, int nmesh) {
    const GroupAsm& g = gm[group_of(gm, nmesh, blockIdx.x, true)];
    const int c = (int)(blockIdx.x - g.node_begin);
    double* dst = g.cbuf + (size_t)c * 9;
    cterm_node(g.coords, g.ien, g.nel, c, g.nq, g.gx, g.gw, g.geom, g.ph, dst);
    __syncthreads();
    if (threadIdx.x < 9) {
        const int i = threadIdx.x / 3, j = threadIdx.x % 3;
        const double v = dst[threadIdx.x] + ((g.if_ext && i == j) ? 0.5 * g.ph.dt : 0.0);
        const size_t off = (size_t)(3 * c + i) * g.out.ld + 3 * (size_t)c + j;
        g.out.H0[off] += v;
        g.out.H0[g.out.level_stride + off] += v;
    }
}

}  // namespace

cudaError_t launch_gauss_geom(const double* coords, const int* ien, int nel, int ennd, int nq,
                              const double* gx, const double* gw, double* geom, float* geomf,
                              cudaStream_t s) {
    const long long n = (long long)nel * nq * nq;
    const int bs = 128;
    const unsigned grid = (unsigned)((n + bs - 1) / bs);
    if (ennd == 8) k_gauss_geom8<<<grid, bs, 0, s>>>(coords, ien, nel, nq, gx, gw, geom);
    else k_gauss_geom<<<grid, bs, 0, s>>>(coords, ien, nel, nq, gx, gw, geom, geomf);
    return cudaGetLastError();
}

size_t duffy_table_elems(int nel, int nq) {
    return (size_t)nel * 4 * 2 * nq * nq * kGeomStride;
}

cudaError_t launch_duffy_table(const double* coords, const int* ien, int nel, int nq,
                               const double* gx, const double* gw, double* duffy,
                               cudaStream_t s) {
    const long long n = (long long)nel * 4 * 2 * nq * nq;
    if (n == 0) return cudaSuccess;
    k_duffy_table<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(coords, ien, nel, nq, gx, gw,
                                                              duffy);
    return cudaGetLastError();
}

cudaError_t launch_element_box(const double* coords, const int* ien, int ennd, int nel,
                               ElemBox* ebox, cudaStream_t s) {
    if (nel == 0) return cudaSuccess;
    const int bs = 128;
    const unsigned grid = (unsigned)((nel + bs - 1) / bs);
    if (ennd == 8)
        k_element_box<8><<<grid, bs, 0, s>>>(coords, ien, nel, ebox);
    else
        k_element_box<4><<<grid, bs, 0, s>>>(coords, ien, nel, ebox);
    return cudaGetLastError();
}

cudaError_t launch_pair_window(const double* coords, const int* ien, int ennd, const int* elems,
                               int nelem_color, int node_lo, int nnodes, const Phys& ph,
                               int mode, int level_last, int level_cap, int step_n, int select,
                               PairInfo* pairs, unsigned* counts, cudaStream_t s,
                               const ElemBox* ebox) {
    const long long n = (long long)nnodes * nelem_color;
    if (n == 0) return cudaSuccess;
    const int bs = 256;
    const unsigned grid = (unsigned)((n + bs - 1) / bs);
    if (ennd == 8)
        k_pair_window<8><<<grid, bs, 0, s>>>(coords, ien, elems, nelem_color, node_lo, nnodes, ph,
                                             mode, level_last, level_cap, step_n, select, pairs,
                                             counts, ebox);
    else
        k_pair_window<4><<<grid, bs, 0, s>>>(coords, ien, elems, nelem_color, node_lo, nnodes, ph,
                                             mode, level_last, level_cap, step_n, select, pairs,
                                             counts, ebox);
    return cudaGetLastError();
}

template <int ENND>
static void launch_items_fp64(const double* coords, const int* ien, const int* elems,
                              int nelem_color, int node_lo, int nq, const double* gx,
                              const double* gw, const double* geom, const Phys& ph, int mode,
                              int level_last, int step_n, const PairInfo* pairs,
                              const unsigned* offsets, unsigned npairs, unsigned nitems,
                              const AsmOut& out, cudaStream_t s, const double* duffy) {
    const int bs = 128;
    // Lanes per item: a launch of few items (the near field of one colour: a few
    // thousand) would hold a handful of blocks, each thread summing 36-72 FP64 Gauss
    // points in turn on the few SMs it lands on; split the points over up to 32 lanes
    // until the launch fills two residencies of the GPU (two 128-thread blocks of 255
    // registers per SM).
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 1;
    const unsigned long long want = (unsigned long long)sms * 2 * 2 * bs;
    const int sh = ENND == 8 ? 1 : 0;
    int lg = 0;
    while (lg < 5 && ((unsigned long long)nitems << (sh + lg)) < want) lg++;
    const unsigned long long threads = (unsigned long long)nitems << (sh + lg);
    const unsigned grid = (unsigned)((threads + bs - 1) / bs);
    if (mode == ASM_LEVELS) {
        k_assemble_items<ASM_LEVELS, ENND><<<grid, bs, 0, s>>>(
            coords, ien, elems, nelem_color, node_lo, nq, gx, gw, geom, ph, level_last, step_n, 0,
            pairs, offsets, npairs, nitems, out, lg, duffy);
    } else {
        for (int part = 0; part < 2; part++)
            k_assemble_items<ASM_STEP, ENND><<<grid, bs, 0, s>>>(
                coords, ien, elems, nelem_color, node_lo, nq, gx, gw, geom, ph, level_last,
                step_n, part, pairs, offsets, npairs, nitems, out, lg, duffy);
    }
}

cudaError_t launch_assemble_items(const double* coords, const int* ien, int ennd,
                                  const int* elems, int nelem_color, int node_lo, int nq,
                                  const double* gx, const double* gw, const double* geom,
                                  const Phys& ph, int mode, int level_last, int step_n,
                                  const PairInfo* pairs, const unsigned* offsets,
                                  unsigned npairs, unsigned nitems, const AsmOut& out,
                                  cudaStream_t s, const double* duffy) {
    if (nitems == 0) return cudaSuccess;
    if (ennd == 8) {
        launch_items_fp64<8>(coords, ien, elems, nelem_color, node_lo, nq, gx, gw, geom, ph, mode,
                             level_last, step_n, pairs, offsets, npairs, nitems, out, s, nullptr);
    } else {
        launch_items_fp64<4>(coords, ien, elems, nelem_color, node_lo, nq, gx, gw, geom, ph, mode,
                             level_last, step_n, pairs, offsets, npairs, nitems, out, s, duffy);
    }
    return cudaGetLastError();
}

cudaError_t launch_assemble_step_pairs(const double* coords, const int* ien, int ennd,
                                       const int* elems, int nelem_color, int node_lo, int nq,
                                       const double* gx, const double* gw, const double* geom,
                                       const Phys& ph, int step_n, const PairInfo* pairs,
                                       unsigned npairs, const AsmOut& out, cudaStream_t s) {
    if (npairs == 0) return cudaSuccess;
    const int bs = 128;
    const unsigned long long threads = (unsigned long long)npairs << (ennd == 8 ? 1 : 0);
    const unsigned grid = (unsigned)((threads + bs - 1) / bs);
    for (int part = 0; part < 2; part++) {
        if (ennd == 8)
            k_assemble_step_pairs<8><<<grid, bs, 0, s>>>(coords, ien, elems, nelem_color, node_lo,
                                                         nq, gx, gw, geom, ph, step_n, part,
                                                         pairs, npairs, out);
        else
            k_assemble_step_pairs<4><<<grid, bs, 0, s>>>(coords, ien, elems, nelem_color, node_lo,
                                                         nq, gx, gw, geom, ph, step_n, part,
                                                         pairs, npairs, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_element_gh(int ennd, int n, int nq, const double* gx, const double* gw,
                              const Phys& ph, const double* colloc, const double* ecoords,
                              const double* times, const int* sing, double* GE1, double* GE2,
                              double* HE1, double* HE2, double* C1, double* C2, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int bs = 128;
    const unsigned long long threads = (unsigned long long)n << (ennd == 8 ? 1 : 0);
    const unsigned grid = (unsigned)((threads + bs - 1) / bs);
    for (int part = 0; part < 2; part++) {
        double* G = part == 0 ? GE1 : GE2;
        double* H = part == 0 ? HE1 : HE2;
        if (ennd == 8)
            k_element_gh<8><<<grid, bs, 0, s>>>(n, nq, gx, gw, ph, colloc, ecoords, times, sing,
                                                part, G, H, C1, C2);
        else
            k_element_gh<4><<<grid, bs, 0, s>>>(n, nq, gx, gw, ph, colloc, ecoords, times, sing,
                                                part, G, H, C1, C2);
    }
    return cudaGetLastError();
}

cudaError_t launch_assemble_far_rows(const double* coords, const int* ien,
                                     const int* color_elems, const int* color_start, int ncolor,
                                     int nnd, int nel, int nq, const float* geomf,
                                     const double* geom, const float* coordf, const Phys& ph,
                                     int level_last, const PairInfo* pairs, const AsmOut& out,
                                     unsigned long long* nitems, cudaStream_t s, int level_cap,
                                     bool fp64_out) {
    // the pairs' windows are capped at level_cap already; the grid covers its chunks
    const int top = std::min(level_last, level_cap);
    if (top < 0) return cudaSuccess;
    const dim3 grid(nnd, (top + kFarChunk) / kFarChunk);
    const PhysF f = to_f(ph);
    if (fp64_out)
        k_assemble_far_rows<double><<<grid, kFarBlock, 0, s>>>(coords, ien, color_elems,
                                                               color_start, ncolor, nel, nq * nq,
                                                               geomf, geom, coordf, ph, f,
                                                               level_last, top, pairs, out,
                                                               nitems);
    else
        k_assemble_far_rows<float><<<grid, kFarBlock, 0, s>>>(coords, ien, color_elems,
                                                              color_start, ncolor, nel, nq * nq,
                                                              geomf, geom, coordf, ph, f,
                                                              level_last, top, pairs, out,
                                                              nitems);
    return cudaGetLastError();
}

cudaError_t launch_cterm(const double* coords, const int* ien, int ennd, int nel, int node_lo,
                         int nnodes, int nq, const double* gx, const double* gw,
                         const double* geom, const Phys& ph, double* cbuf, cudaStream_t s,
                         bool fast, const float* geomf, const float* coordf,
                         const ElemBox* ebox, const double* duffy) {
    if (nnodes == 0) return cudaSuccess;
    // the FP32 path's constants, as cterm_node's FP64 ones rounded once
    const float onem2nu_f = (float)(1 - 2 * ph.nu);
    const float kscale_f = (float)((0.5 * ph.dt) / (-(8 * M_PI) * (1 - ph.nu)));
    if (ennd == 8) {
        if (fast)
            k_cterm<8, true><<<nnodes, 256, 0, s>>>(coords, ien, nel, node_lo, nq, gx, gw, geom, ph,
                                                    cbuf, nullptr, nullptr, ebox, onem2nu_f,
                                                    kscale_f, nullptr);
        else
            k_cterm<8, false><<<nnodes, 256, 0, s>>>(coords, ien, nel, node_lo, nq, gx, gw, geom,
                                                     ph, cbuf, nullptr, nullptr, ebox, 0.f, 0.f,
                                                     nullptr);
    } else {
        if (fast)
            k_cterm<4, true><<<nnodes, 256, 0, s>>>(coords, ien, nel, node_lo, nq, gx, gw, geom, ph,
                                                    cbuf, geomf, coordf, ebox, onem2nu_f,
                                                    kscale_f, duffy);
        else
            k_cterm<4, false><<<nnodes, 256, 0, s>>>(coords, ien, nel, node_lo, nq, gx, gw, geom,
                                                     ph, cbuf, nullptr, nullptr, ebox, 0.f, 0.f,
                                                     duffy);
    }
    return cudaGetLastError();
}

// FP32 store levels 0/1 from the finished FP64 levels 0/1 (ld D -> ldf).
__global__ void k_cast_levels01(const double* __restrict__ G01, const double* __restrict__ H01,
                                int D, int ldf, float* __restrict__ Gf, float* __restrict__ Hf) {
    const size_t n = (size_t)2 * D * D;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t kr = i / D, col = i - kr * D;  // kr = level * D + row
        Gf[kr * ldf + col] = (float)G01[i];
        Hf[kr * ldf + col] = (float)H01[i];
    }
}

cudaError_t launch_cast_levels01(const double* G01, const double* H01, int D, int ldf, float* Gf,
                                 float* Hf, cudaStream_t s) {
    if (ldf < D) return cudaErrorInvalidValue;
    k_cast_levels01<<<152 * 8, 256, 0, s>>>(G01, H01, D, ldf, Gf, Hf);
    return cudaGetLastError();
}

cudaError_t launch_cterm_apply(const double* cbuf, int node_lo, int nnodes, double dt,
                               int if_ext, int mode, const AsmOut& out, cudaStream_t s) {
    if (nnodes == 0) return cudaSuccess;
    k_cterm_apply<<<(nnodes * 9 + 255) / 256, 256, 0, s>>>(cbuf, node_lo, nnodes, dt, if_ext,
                                                             mode, out);
    return cudaGetLastError();
}

size_t scan_temp_bytes(unsigned n) {
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, (const unsigned*)nullptr, (unsigned*)nullptr,
                                  (int)n);
    return bytes;
}

cudaError_t exclusive_scan(const unsigned* in, unsigned* out, unsigned n, void* tmp,
                           size_t tmp_bytes, cudaStream_t s) {
    return cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, (int)n, s);
}

cudaError_t launch_pair_window_group(const GroupAsm* gm, int nmesh, unsigned npairs,
                                     PairInfo* pairs, unsigned* counts, cudaStream_t s) {
    if (npairs == 0) return cudaSuccess;
    k_pair_window_group<<<(npairs + 255) / 256, 256, 0, s>>>(gm, nmesh, npairs, pairs, counts);
    return cudaGetLastError();
}

cudaError_t launch_assemble_group(const GroupAsm* gm, int nmesh, const PairInfo* pairs,
                                  const unsigned* offsets, unsigned npairs, unsigned nitems,
                                  cudaStream_t s) {
    if (nitems == 0) return cudaSuccess;
    k_assemble_group<<<(nitems + 127) / 128, 128, 0, s>>>(gm, nmesh, pairs, offsets, npairs,
                                                          nitems);
    return cudaGetLastError();
}

cudaError_t launch_cterm_group(const GroupAsm* gm, int nmesh, unsigned nnodes, cudaStream_t s) {
    if (nnodes == 0) return cudaSuccess;
    k_cterm_group<<<nnodes, 256, 0, s>>>(gm, nmesh);
    return cudaGetLastError();
}

}  // namespace tdbem
