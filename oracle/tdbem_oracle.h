/*
 * tdbem_oracle.h -- CPU oracle for the TD-BEM hot path (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference's assembly and marching, function by
 * function, each citing the reference file:line it follows.  Only the tests,
 * the smoke check and the benchmark's CPU-baseline leg may call it, and only
 * as the checker or as the timed CPU baseline; the product never links it.
 *
 * Pinning: its outputs are compared with the reference's own sources built
 * here (oracle/Makefile.ref) through the golden fixtures in tests/golden/.
 * The reference's linear solve is PETSc's default GMRES; here it is an exact
 * dense LU with partial pivoting, so histories are "the reference's
 * discretisation with an exact linear solve".
 */
#ifndef TDBEM_ORACLE_H
#define TDBEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nnd;              /* nodes */
    int nel;              /* elements */
    int etype;            /* 1 = 4-node bilinear, 2 = 8-node serendipity */
    const double* coords; /* nnd x 3 */
    const int* ien;       /* nel x ennd, 0-based */
    double E, nu, rho;
    double dt;
    int nq;               /* Gauss points per direction: 6, 10, 20 or 40 */
    int if_ext;           /* exterior problem: +0.5*dt on the first-step diagonal */
} orc_model;

/* Test hook (0 by default): non-zero makes the oracle return the exact value 0
 * for the step response once both wave fronts have passed a quadrature point at
 * both evaluation times, where the reference's arithmetic leaves round-off
 * (GreenFunctionT.cpp:241-446 evaluated with b = dt and I5 = I6 = 0 at T and at
 * T - dt).  Used to measure the reference's round-off floor. */
extern int orc_clean_passed_waves;

/* SolverT::ComputeMaxStep (SolverT.cpp:211-250). */
int orc_max_step(const orc_model* m);

/* ElastoDynamicsT::G_H_Driver + GetGHLinear (ElastoDynamicsT.cpp:108-231, 283-289)
 * for rows node_lo..node_hi (inclusive) at time t with step t_1.  Outputs are
 * the four row blocks ((node_hi-node_lo+1)*3) x (3*nnd), row-major:
 * G_I = fG_1, G_J = fG_2, H_I = fH_1, H_J = fH_2.  Returns 0 or a negative
 * error code. */
int orc_gh_driver(const orc_model* m, double t, double t_1, int node_lo, int node_hi,
                  double* G_I, double* G_J, double* H_I, double* H_J, int nthreads);

/* Level store after steps 1..min(M, nsteps) of the main loop
 * (main.cpp:89-121 with SolverStepLinearT::UpdateGHLinear,
 * SolverStepLinearT.cpp:58-97): G_levels/H_levels are (M+1) x D x D. */
int orc_assemble_levels(const orc_model* m, int M, int nsteps, double* G_levels,
                        double* H_levels, int nthreads);

/* Marching (SolverT::SetLoad SolverT.cpp:344-377, SolverStepLinearT::Solve_Averaging
 * SolverStepLinearT.cpp:314-544, SolverT::ExchangeColumns SolverT.cpp:265-342) over
 * the given level store.  amp[s] multiplies the traction BC values at step s
 * (time s*dt); NULL means the reference's hard-wired Heaviside amp = 1
 * (SolverT.cpp:379-394).  u_hist/t_hist are (numstep+1) x D.  Returns 0, or a
 * negative error code (-2 alpha out of range, -3 singular operator). */
int orc_march(int D, int M, const double* G_levels, const double* H_levels, int ubc_num,
              const int* ubc_dofs, const double* ubc_vals, int fbc_num, const int* fbc_dofs,
              const double* fbc_vals, const double* amp, double a1, double a2, int numstep,
              double* u_hist, double* t_hist, int nthreads);

/* Marching cost probe for the CPU baseline: runs Solve_Averaging's steps
 * step_lo..step_hi (1-based curr_step) of the above, starting from the given
 * histories, and returns nothing but the histories it wrote. */
int orc_march_range(int D, int M, const double* G_levels, const double* H_levels,
                    int ubc_num, const int* ubc_dofs, const double* ubc_vals, int fbc_num,
                    const int* fbc_dofs, const double* fbc_vals, const double* amp, double a1,
                    double a2, int step_lo, int step_hi, double* u_hist, double* t_hist,
                    int nthreads);

/* Factorize an n x n matrix in place with the LU of the KSPSolve stand-in
 * (used by the CPU baseline to time the solve setup).  Returns 0 or -3. */
int orc_lu_factor(int n, double* A, int nthreads);

/* One Green's function evaluation, GreenFunctionT::Compute(4)
 * (GreenFunctionT.cpp:134-136): direction = x - x_c, normal = unnormalised
 * surface normal.  Outputs are 3x3 row-major [i][k] as the reference stores
 * them: DU_1, DU_2, DT_1, DT_2 (step response, I and J parts) and DT_K
 * (Kelvin_Linear). */
void orc_green_step_linear(double E, double nu, double rho, const double* direction,
                           const double* normal, double t, double t_1, double* DU_1,
                           double* DU_2, double* DT_1, double* DT_2, double* DT_K);

/* One element, TDElementStepLinearT::FormGH_Regular (TDElementStepLinearT.cpp:28-125)
 * if singular < 0, else FormGH_Singular(singular) (128-190).  coords is ennd x 3.
 * Outputs GE_1, GE_2, HE_1, HE_2 are 3 x 3*ennd, C_1, C_2 are 3 x 3. */
int orc_element_gh(int etype, int nq, double E, double nu, double rho, const double* coords,
                   const double* collocation, double t, double t_1, int singular, double* GE_1,
                   double* GE_2, double* HE_1, double* HE_2, double* C_1, double* C_2);

/* Two-region solver, SolverMRT (SolverMRT.cpp).  The index maps and the combined
 * level placement (Assemble_GH_R1/R2, 663-847) are exact copies done by the
 * caller; this is the arithmetic.
 *
 * orc_mrt_amplitude: SetLoad's amplitude p0 t exp(-2000 t) at t = n dt
 * (SolverMRT.cpp:881-887).
 *
 * orc_mrt_march: Solve_Direct (SolverMRT.cpp:1028-1097) on the combined system:
 * per step n, rhs = G^0 load^n + sum_{f=1}^{min(n,L)} (G^f tg^{n-f} - H^f x^{n-f}),
 * x^n = H^0 \ rhs (the KSPSolve stand-in), tg^n = load^n.  GG: (L+1) x N x NG,
 * HH: (L+1) x N x N, load: (numstep+1) x NG with row n = fLoad of step n (row 0
 * unused: tg^0 = 0), X: (numstep+1) x N, row 0 = 0.  Returns 0, -3 (singular H^0)
 * or -4 (no memory). */
double orc_mrt_amplitude(int n, double dt);
int orc_mrt_march(int N, int NG, int L, const double* GG, const double* HH,
                  const double* load, int numstep, double* X, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
