// ElastoDynamicsGpuT and SolverStepLinearGpuT: the reference's per-step driver
// interfaces over the C ABI (tdbem.h), one device context per model.
#include <cmath>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "../../../include/tdbem_host.hpp"

namespace tdbem {

namespace {

thread_local std::string g_msg;

// Throws the C ABI's message as the reference throws: a const char*.
void check(int rc, const char* what) {
    if (rc == TDBEM_OK) return;
    g_msg = std::string(what) + ": " + tdbem_last_error();
    throw g_msg.c_str();
}

tdbem_ctx* make_ctx(ModelManagerT* model) {
    if (!model) {
        g_msg = "model is null";
        throw g_msg.c_str();
    }
    const tdbem_mesh mesh = model->Mesh();
    const tdbem_material mat = model->Material();
    tdbem_ctx* ctx = nullptr;
    check(tdbem_ctx_create(&mesh, &mat, model->GetDT(), model->GetNQ(), model->GetIfExt(), &ctx),
          "tdbem_ctx_create");
    return ctx;
}

}  // namespace

// ---------------------------------------------------------------- ElastoDynamicsGpuT

ElastoDynamicsGpuT::ElastoDynamicsGpuT(ModelManagerT* model)
    : model_(model), ctx_(make_ctx(model)), own_ctx_(true) {
    SetLowerUpper(0, model->GetNND() - 1);
}

ElastoDynamicsGpuT::ElastoDynamicsGpuT(ModelManagerT* model, SolverStepLinearGpuT* solver)
    : model_(model), ctx_(solver ? solver->Context() : nullptr), own_ctx_(false) {
    if (!ctx_) {
        g_msg = "solver has no device context";
        throw g_msg.c_str();
    }
    SetLowerUpper(0, model->GetNND() - 1);
}

ElastoDynamicsGpuT::ElastoDynamicsGpuT(ModelManagerT* model, SolverMRGpuT* solver, int region)
    : model_(model),
      ctx_(solver && (region == 1 || region == 2) ? solver->Context(region) : nullptr),
      own_ctx_(false) {
    if (!ctx_) {
        g_msg = "solver has no device context for that region";
        throw g_msg.c_str();
    }
    SetLowerUpper(0, model->GetNND() - 1);
}

ElastoDynamicsGpuT::~ElastoDynamicsGpuT() {
    if (own_ctx_) tdbem_ctx_destroy(ctx_);
}

void ElastoDynamicsGpuT::SetLowerUpper(int lower, int upper) {
    if (lower < 0 || upper >= model_->GetNND() || lower > upper) {
        g_msg = "node range out of the mesh";
        throw g_msg.c_str();
    }
    lo_ = lower;
    hi_ = upper;
    // ElastoDynamicsT keeps four zeroed row blocks of the node range
    const size_t n = 3 * (size_t)(hi_ - lo_ + 1) * 3 * (size_t)model_->GetNND();
    G1_.assign(n, 0.0);
    G2_.assign(n, 0.0);
    H1_.assign(n, 0.0);
    H2_.assign(n, 0.0);
}

void ElastoDynamicsGpuT::G_H_Driver(double t, double t_1) {
    if (!(t_1 > 0)) {
        g_msg = "time step must be positive";
        throw g_msg.c_str();
    }
    step_ = (int)std::lround(t / t_1);
    check(tdbem_gh_driver(ctx_, step_, lo_, hi_, G1_.data(), G2_.data(), H1_.data(), H2_.data()),
          "G_H_Driver");
}

void ElastoDynamicsGpuT::GetGHLinear(double** G_1, double** G_2, double** H_1, double** H_2) {
    *G_1 = G1_.data();
    *G_2 = G2_.data();
    *H_1 = H1_.data();
    *H_2 = H2_.data();
}

// ---------------------------------------------------------------- SolverStepLinearGpuT

SolverStepLinearGpuT::SolverStepLinearGpuT(ModelManagerT* model)
    : model_(model), ctx_(make_ctx(model)) {
    int nu = 0, nf = 0;
    int *ud = nullptr, *fd = nullptr;
    double *uv = nullptr, *fv = nullptr;
    model->BoundaryCondition_Global(nu, &ud, &uv, nf, &fd, &fv);
    check(tdbem_set_bc(ctx_, ud, uv, nu, fd, fv, nf), "boundary conditions");
    check(tdbem_max_step(ctx_, &max_step_), "ComputeMaxStep");
    dt_ = model->GetDT();
    num_steps_ = model->GetNumStep();
}

SolverStepLinearGpuT::~SolverStepLinearGpuT() { tdbem_ctx_destroy(ctx_); }

void SolverStepLinearGpuT::GetNodeLowHigh(int* low, int* high) {
    *low = 0;
    *high = model_->GetNND() - 1;
}

void SolverStepLinearGpuT::GetDofLowHigh(int* low, int* high) {
    *low = 0;
    *high = 3 * model_->GetNND() - 1;
}

void SolverStepLinearGpuT::SetTimeControl(double dt, int num_steps) {
    if (dt != model_->GetDT()) {
        g_msg = "the time step differs from the model's (the levels depend on it)";
        throw g_msg.c_str();
    }
    dt_ = dt;
    num_steps_ = num_steps;
}

void SolverStepLinearGpuT::Initialize() {
    // zero displacement and traction at step 0 (SolverT::Initialize)
    const size_t D = 3 * (size_t)model_->GetNND();
    u_.assign(num_steps_ + 1, std::vector<double>(D, 0.0));
    t_.assign(num_steps_ + 1, std::vector<double>(D, 0.0));
    check(tdbem_march_begin(ctx_, num_steps_), "Initialize");
    begun_ = true;
}

int SolverStepLinearGpuT::GetMaxStep() { return max_step_; }

void SolverStepLinearGpuT::SetCurrStep(int curr_step) { curr_ = curr_step; }

void SolverStepLinearGpuT::UpdateGHLinear(const double* G_0, const double* G_1,
                                          const double* H_0, const double* H_1) {
    if (curr_ < 1 || curr_ > max_step_) return;  // SolverStepLinearT.cpp:66
    check(tdbem_update_gh_linear(ctx_, curr_, 0, model_->GetNND() - 1, G_0, G_1, H_0, H_1),
          "UpdateGHLinear");
}

void SolverStepLinearGpuT::SetLoad() {
    // The load of each step (prescribed values x LoadTimeVariation) is formed on
    // the device inside Solve from the boundary conditions and the load history.
}

void SolverStepLinearGpuT::Solve(double a1, double a2) {
    if (!(a1 >= 0 && a1 <= 1 && a2 >= 0 && a2 < 1 && a1 + a2 <= 1)) {
        g_msg = "Alpha is out of range";  // SolverStepLinearT.cpp:317-322
        throw g_msg.c_str();
    }
    if (!begun_) Initialize();
    check(tdbem_set_alpha(ctx_, a1, a2), "Solve");
    if (curr_ < 1 || curr_ > num_steps_) {
        g_msg = "current step outside 1..num_steps";
        throw g_msg.c_str();
    }
    check(tdbem_march_step(ctx_, curr_, u_[curr_ - 1].data(), t_[curr_ - 1].data()), "Solve");
}

double SolverStepLinearGpuT::LoadTimeVariation(double t) {
    if (amp_.empty()) return 1.0;  // Heaviside (SolverT.cpp:379-394)
    const long s = std::lround(t / dt_);
    return (s >= 0 && s < (long)amp_.size()) ? amp_[s] : 0.0;
}

void SolverStepLinearGpuT::SetLoadHistory(const std::vector<double>& amp) {
    amp_ = amp;
    check(tdbem_set_load_history(ctx_, amp_.data(), (int)amp_.size()), "SetLoadHistory");
}

void SolverStepLinearGpuT::RecordResult() {
    if (curr_ < 1) return;
    std::ofstream f;
    if (curr_ == 1) {
        f.open(result_file_, std::fstream::out | std::fstream::trunc);
        f << std::setw(10) << "%time" << std::setw(15) << "load" << std::setw(15)
          << "displacement" << std::setw(15) << "traction" << std::endl;
    } else {
        f.open(result_file_, std::fstream::out | std::fstream::app);
    }
    if (!f) {
        g_msg = "cannot open " + result_file_;
        throw g_msg.c_str();
    }
    f << std::setprecision(6);
    const double time = dt_ * (curr_ - 1);
    const double amp = LoadTimeVariation(time);
    const std::vector<double>& u = u_[curr_ - 1];
    const std::vector<double>& t = t_[curr_ - 1];
    f << std::setw(10) << time << std::setw(15) << amp << std::setw(15) << u[2] << std::setw(15)
      << t[2] << std::endl;
}

void SolverStepLinearGpuT::WriteGH(const char* name_prefix, int step, int num_row,
                                   int num_column, double* data, int, int) {
    check(tdbem_write_gh(name_prefix, step, num_row, num_column, data), "WriteGH");
}

}  // namespace tdbem
