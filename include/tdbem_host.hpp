// C++ host classes of tdbem-gb300 with the reference's interfaces.
//
// They mirror the classes main.cpp drives (src/main.cpp:42-130) so that its
// sequence runs unchanged on the GPU:
//   ModelManagerT        ModelManagerT.h:16-196 (input reading and getters)
//   TDElementGpuT        TDElementT.h:16-115 / TDElementStepLinearT (one element's
//                        G/H blocks: SetCollocation, SetCoords, SetTime, SetNQ,
//                        SetMaterial, FormGH_Regular, FormGH_Singular, GetGHLinear)
//   ElastoDynamicsGpuT   ElastoDynamicsT.h:22-39 (G_H_Driver, GetGHLinear)
//   SolverStepLinearGpuT SolverT.h:22-128 / SolverStepLinearT (SetTimeControl,
//                        Initialize, GetMaxStep, UpdateGHLinear, SetLoad,
//                        Solve, RecordResult, WriteGH)
//   SolverMRGpuT         SolverMRT.h:25-226 (the two-region solver: SetMaxStep,
//                        SetTimeControl, UpdateGHLinear with both regions' blocks,
//                        SetLoad, Solve, RecordResult)
// Names, argument meaning and error behaviour follow the reference: failures
// throw `const char*` (the message stays valid until the next failure on this
// thread), as main.cpp catches.  Everything runs on one GPU through the C ABI of
// tdbem.h; the classes live in namespace tdbem so that they can be linked next
// to the reference's own classes.
//
// G_H_Driver assembles a step's row blocks on the device and GetGHLinear returns
// host copies of them (the reference's pointers, valid until the next
// G_H_Driver); UpdateGHLinear places host row blocks into the solver's device
// level store and Solve marches one step on the device.  An ElastoDynamicsGpuT
// built with a SolverStepLinearGpuT shares its device context (one copy of the
// mesh and quadrature tables).  The whole-run path without per-step host copies
// is tdbem_assemble_levels + tdbem_march (tdbem_run --fast).
#pragma once

#include <string>
#include <vector>

#include "tdbem.h"

namespace tdbem {

class ModelManagerT {
   public:
    ModelManagerT() = default;

    // InputT::ReadInput (InputT.cpp:84-994): the keyword format, tokens split at
    // " \t=;,", integers by atoi and reals by atof, 1-based ids in the file.
    void ReadInput(const char* name);

    int GetFormulation() { return formulation_; }
    int GetNumStep() { return numstep_; }
    void SetNumStep(int n) { numstep_ = n; }
    double GetDT() { return dt_; }
    void SetDT(double dt) { dt_ = dt; }
    int GetTimeInterpolation() { return interpolation_; }
    int GetNQ() { return nq_; }
    int GetSD() { return sd_; }
    int GetIfExt() { return if_ext_; }
    int GetNND() { return nnd_; }
    int GetElementType() { return etype_; }
    int GetENND() { return ennd_; }
    int GetNEL() { return nel_; }
    const int* GetIEN() { return ien_.data(); }
    const double* GetCoords() { return coords_.data(); }
    void GetMaterialConstants(double& E, double& nu, double& rho) {
        E = E_;
        nu = nu_;
        rho = rho_;
    }
    void SetMaterialConstants(double E, double nu, double rho) {
        E_ = E;
        nu_ = nu;
        rho_ = rho;
    }
    void BoundaryCondition_Global(int& UBC_num, int** UBC_DOFs, double** UBC_Values,
                                  int& FBC_num, int** FBC_DOFs, double** FBC_Values);
    void SetBCs(int UBC_num, const int* UBC_DOFs, const double* UBC_values, int FBC_num,
                const int* FBC_DOFs, const double* FBC_values);
    int GetNumInterface() { return (int)interface_.size(); }
    const int* GetInterface() { return interface_.data(); }
    // Auxiliary mesh of a multi-region input (ModelManagerT.cpp:236-304); read, not
    // used by the assembly or the marching.
    int GetNND_Aux() { return nnd_aux_; }
    int GetElementType_Aux() { return etype_aux_; }
    int GetENND_Aux() { return ennd_aux_; }
    int GetNEL_Aux() { return nel_aux_; }
    const int* GetIEN_Aux() { return ien_aux_.data(); }
    const double* GetCoords_Aux() { return coords_aux_.data(); }
    // Single process: every dof is local (ModelManagerT::Distributed_BC keeps all).
    void Distributed_BC(int, int) {}

    // The C-ABI views of the model.
    tdbem_mesh Mesh() const;
    tdbem_material Material() const;

   private:
    int formulation_ = 1, numstep_ = 1, interpolation_ = 1, nq_ = 6, sd_ = 3, if_ext_ = 0;
    int nnd_ = 0, nel_ = 0, etype_ = 1, ennd_ = 4;
    int nnd_aux_ = 0, nel_aux_ = 0, etype_aux_ = 1, ennd_aux_ = 4;
    double dt_ = 0, E_ = 1, nu_ = 0, rho_ = 1;
    std::vector<double> coords_, coords_aux_;
    std::vector<int> ien_, ien_aux_;
    std::vector<int> ubc_dof_, fbc_dof_, interface_;
    std::vector<double> ubc_val_, fbc_val_;
};

// TDElementT / TDElementStepLinearT (TDElementT.h:16-115): the element-level
// quadrature of one (collocation point, element) pair, with the reference's call
// sequence.  FormGH_Regular / FormGH_Singular take a copy of the current
// collocation point, coordinates and time and queue the pair; GetGHLinear
// evaluates every queued pair in one launch (tdbem_element_gh) and returns the
// blocks of the pair formed last, as the reference's element returns its own.
// GetGHLinear(k, ...) returns pair k of that evaluation (0 = the first formed
// since the previous evaluation), so a caller that forms many elements before
// reading them gets one launch for all of them.  Material, quadrature order and
// t_1 are shared by a launch: changing one evaluates the queued pairs first.
// The returned pointers stay valid until the next evaluation.
class TDElementGpuT {
   public:
    // type: 1 = 4-node quad, 2 = 8-node quad (TDElementT(int type)).
    explicit TDElementGpuT(int type);
    void SetCollocation(double* collocation);
    void SetCoords(double* coords);
    virtual void SetTime(double t, double t_1);
    void SetNQ(int nq);
    void SetMaterial(double E, double nu, double density);
    virtual void FormGH_Regular();
    virtual void FormGH_Singular(int singular);
    void GetGHLinear(const double** GE_1, const double** GE_2, const double** HE_1,
                     const double** HE_2, const double** C_1, const double** C_2);
    void GetGHLinear(int k, const double** GE_1, const double** GE_2, const double** HE_1,
                     const double** HE_2, const double** C_1, const double** C_2);
    // Pairs of the last evaluation.
    int NumEvaluated() const { return evaluated_; }
    virtual ~TDElementGpuT() = default;

   private:
    void Queue(int singular);
    void Evaluate();
    int type_, ennd_, nq_ = 6;
    double E_ = 0, nu_ = 0, rho_ = 0, t_ = 0, t_1_ = 0;
    const double* colloc_ = nullptr;
    const double* coords_ = nullptr;
    std::vector<double> q_colloc_, q_coords_, q_t_;
    std::vector<int> q_sing_;
    std::vector<double> ge1_, ge2_, he1_, he2_, c1_, c2_;
    int evaluated_ = 0;
};

class SolverStepLinearGpuT;
class SolverMRGpuT;

class ElastoDynamicsGpuT {
   public:
    // Own device context for the model.
    explicit ElastoDynamicsGpuT(ModelManagerT* model);
    // Shares the solver's device context.
    ElastoDynamicsGpuT(ModelManagerT* model, SolverStepLinearGpuT* solver);
    // Shares the device context of region 1 or 2 of a two-region solver.
    ElastoDynamicsGpuT(ModelManagerT* model, SolverMRGpuT* solver, int region);
    ~ElastoDynamicsGpuT();
    ElastoDynamicsGpuT(const ElastoDynamicsGpuT&) = delete;
    ElastoDynamicsGpuT& operator=(const ElastoDynamicsGpuT&) = delete;

    void SetLowerUpper(int lower, int upper);
    // G_H_Driver (ElastoDynamicsT.cpp:108-231) at time t = n * t_1.
    void G_H_Driver(double t, double t_1);
    // The step's I parts (G_1, H_1) and J parts (G_2, H_2), rows of the node range.
    void GetGHLinear(double** G_1, double** G_2, double** H_1, double** H_2);

    int Step() const { return step_; }
    tdbem_ctx* Context() const { return ctx_; }

   private:
    ModelManagerT* model_;
    tdbem_ctx* ctx_ = nullptr;
    bool own_ctx_ = false;
    int lo_ = 0, hi_ = -1, step_ = 0;
    std::vector<double> G1_, G2_, H1_, H2_;
};

class SolverStepLinearGpuT {
   public:
    explicit SolverStepLinearGpuT(ModelManagerT* model);
    ~SolverStepLinearGpuT();
    SolverStepLinearGpuT(const SolverStepLinearGpuT&) = delete;
    SolverStepLinearGpuT& operator=(const SolverStepLinearGpuT&) = delete;

    void GetNodeLowHigh(int* low, int* high);
    void GetDofLowHigh(int* low, int* high);
    void SetTimeControl(double dt, int num_steps);
    void Initialize();
    int GetMaxStep();
    void SetCurrStep(int curr_step);
    // Row blocks of the current step (SolverStepLinearT.cpp:58-175): G_0 / H_0 the
    // I parts, G_1 / H_1 the J parts, as main.cpp passes GetGHLinear's outputs.
    void UpdateGHLinear(const double* G_0, const double* G_1, const double* H_0,
                        const double* H_1);
    void SetLoad();
    void Solve(double a1, double a2);
    // One line per step to displacement.txt (SolverStepLinearT.cpp:549-603):
    // time, load amplitude, displacement and traction of dof 2.
    void RecordResult();
    // SolverT::LoadTimeVariation (SolverT.cpp:379-394): amp[s] at step s when a
    // load history is set, else the reference's unit step.
    double LoadTimeVariation(double t);
    void SetLoadHistory(const std::vector<double>& amp);
    void SetResultFile(const std::string& path) { result_file_ = path; }
    // SolverT::WriteGH (SolverT.cpp:670-732) on one process.
    void WriteGH(const char* name_prefix, int step, int num_row, int num_column, double* data,
                 int comm_size = 1, int comm_rank = 0);

    // Histories so far: step s of u / t is Displacement(s) / Traction(s).
    const std::vector<double>& Displacement(int s) const { return u_[s]; }
    const std::vector<double>& Traction(int s) const { return t_[s]; }
    tdbem_ctx* Context() const { return ctx_; }

   private:
    ModelManagerT* model_;
    tdbem_ctx* ctx_ = nullptr;
    double dt_ = 0;
    int num_steps_ = 0, curr_ = 0, max_step_ = 0;
    bool begun_ = false;
    std::vector<double> amp_;
    std::vector<std::vector<double>> u_, t_;
    std::string result_file_ = "displacement.txt";
};

// SolverMRT (SolverMRT.cpp): two regions joined at the nodes of their interface
// lists (ModelManagerT::GetInterface), marched with Solve_Direct.  One device
// context per region (its FBC list gives its loads; UBC lists are not used, as
// in the reference); the combined system runs on the device (tdbem_mrt_*).
class SolverMRGpuT {
   public:
    // SolverMRT(model_1, model_2) (SolverMRT.cpp:22-64); LocalIndexing and
    // InterfaceIndexing happen here, as in the reference's constructor.
    SolverMRGpuT(ModelManagerT* model_1, ModelManagerT* model_2);
    ~SolverMRGpuT();
    SolverMRGpuT(const SolverMRGpuT&) = delete;
    SolverMRGpuT& operator=(const SolverMRGpuT&) = delete;

    void LocalIndexing() {}
    void InterfaceIndexing() {}
    // Level count (default 10, SolverMRT.cpp:35); set it before SetTimeControl as
    // the reference sizes its level store there.
    void SetMaxStep(int MaxStep);
    int GetMaxStep() const { return max_step_; }
    void SetTimeControl(double dt, int Numsteps);
    void SetCurrStep(int curr_step) { curr_ = curr_step; }
    // Both regions' blocks of the current step (SolverMRT.cpp:850-949): G_0 / H_0 /
    // g_0 / h_0 the I parts, G_1 / H_1 / g_1 / h_1 the J parts; steps past MaxStep
    // are ignored.
    void UpdateGHLinear(const double* G_0, const double* G_1, const double* H_0,
                        const double* H_1, const double* g_0, const double* g_1,
                        const double* h_0, const double* h_1);
    // The load (interior FBC values x amplitude) is formed on the device in Solve.
    void SetLoad() {}
    void Solve();
    void ExtractField() {}
    void GetNodeLowHigh(int* low_1, int* high_1, int* low_2, int* high_2);
    void GetDofLowHigh(int* low_1, int* high_1, int* low_2, int* high_2);
    // One line per step (SolverMRT.cpp:1337-1388): the time (curr - 1) dt and the
    // displacement of region 2's record dof at that step.  The reference prints
    // dof 137 (46*3-1) of its test mesh; here that dof when region 2 has it, else
    // dof 2, or the dof set by SetRecordDof.  VTK output is not written.
    void RecordResult();
    void SetRecordDof(int dof) { record_dof_ = dof; }
    void SetResultFile(const std::string& path) { result_file_ = path; }
    // amp[n] at time n dt in place of the built-in pulse 5.46366e9 t exp(-2000 t).
    void SetLoadHistory(const std::vector<double>& amp);

    // Combined unknowns x of step s (the reference's fDis_DB_Global[s]) and the
    // regions' displacements / tractions of step s.
    const std::vector<double>& Unknowns(int s) const { return x_[s]; }
    const std::vector<double>& Displacement(int region, int s) const { return u_[region - 1][s]; }
    const std::vector<double>& Traction(int region, int s) const { return t_[region - 1][s]; }
    int NumUnknowns() const { return N_; }
    tdbem_ctx* Context(int region) const { return ctx_[region - 1]; }

   private:
    void make_solver();
    ModelManagerT* model_[2];
    tdbem_ctx* ctx_[2] = {nullptr, nullptr};
    tdbem_mrt* mrt_ = nullptr;
    int max_step_ = 10, num_steps_ = 0, curr_ = 0, N_ = 0, record_dof_ = -1;
    double dt_ = 0;
    bool begun_ = false;
    std::vector<double> amp_;
    std::vector<std::vector<double>> x_, u_[2], t_[2];
    std::string result_file_ = "displacement.txt";
};

}  // namespace tdbem
