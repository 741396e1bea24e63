// SolverMRGpuT: the reference's two-region solver interface (SolverMRT.h:25-226)
// over the C ABI (tdbem_mrt_* in tdbem.h), one device context per region.
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "../../../include/tdbem_host.hpp"

namespace tdbem {

namespace {

thread_local std::string g_msg;

void check(int rc, const char* what) {
    if (rc == TDBEM_OK) return;
    g_msg = std::string(what) + ": " + tdbem_last_error();
    throw g_msg.c_str();
}

[[noreturn]] void raise(const std::string& msg) {
    g_msg = msg;
    throw g_msg.c_str();
}

tdbem_ctx* region_ctx(ModelManagerT* m) {
    if (!m) raise("model is null");
    const tdbem_mesh mesh = m->Mesh();
    const tdbem_material mat = m->Material();
    tdbem_ctx* ctx = nullptr;
    check(tdbem_ctx_create(&mesh, &mat, m->GetDT(), m->GetNQ(), m->GetIfExt(), &ctx),
          "tdbem_ctx_create");
    int nu = 0, nf = 0;
    int *ud = nullptr, *fd = nullptr;
    double *uv = nullptr, *fv = nullptr;
    m->BoundaryCondition_Global(nu, &ud, &uv, nf, &fd, &fv);
    const int rc = tdbem_set_bc(ctx, ud, uv, nu, fd, fv, nf);
    if (rc != TDBEM_OK) {
        tdbem_ctx_destroy(ctx);
        check(rc, "boundary conditions");
    }
    return ctx;
}

}  // namespace

SolverMRGpuT::SolverMRGpuT(ModelManagerT* model_1, ModelManagerT* model_2)
    : model_{model_1, model_2} {
    if (!model_1 || !model_2) raise("model is null");
    if (model_1->GetNumInterface() != model_2->GetNumInterface())
        raise("Interface mismatch, interface nodes must match one-to-one");
    ctx_[0] = region_ctx(model_1);
    try {
        ctx_[1] = region_ctx(model_2);
        // SolverMRT.cpp:35-37: MaxStep 10, time control of model 1
        dt_ = model_1->GetDT();
        num_steps_ = model_1->GetNumStep();
        make_solver();
    } catch (...) {
        if (mrt_) tdbem_mrt_destroy(mrt_);
        if (ctx_[1]) tdbem_ctx_destroy(ctx_[1]);
        tdbem_ctx_destroy(ctx_[0]);
        throw;
    }
}

SolverMRGpuT::~SolverMRGpuT() {
    if (mrt_) tdbem_mrt_destroy(mrt_);
    tdbem_ctx_destroy(ctx_[1]);
    tdbem_ctx_destroy(ctx_[0]);
}

void SolverMRGpuT::make_solver() {
    if (mrt_) tdbem_mrt_destroy(mrt_);
    mrt_ = nullptr;
    check(tdbem_mrt_create(ctx_[0], ctx_[1], model_[0]->GetInterface(), model_[1]->GetInterface(),
                           model_[0]->GetNumInterface(), max_step_, &mrt_),
          "SolverMRT");
    int ng = 0;
    check(tdbem_mrt_size(mrt_, &N_, &ng), "SolverMRT");
    if (!amp_.empty())
        check(tdbem_mrt_set_load_history(mrt_, amp_.data(), (int)amp_.size()), "SetLoadHistory");
    begun_ = false;
}

void SolverMRGpuT::SetMaxStep(int MaxStep) {
    if (MaxStep < 0) raise("MaxStep must be >= 0");
    max_step_ = MaxStep;
    make_solver();
}

void SolverMRGpuT::SetTimeControl(double dt, int Numsteps) {
    if (dt != model_[0]->GetDT() || dt != model_[1]->GetDT())
        raise("the time step differs from the models' (the levels depend on it)");
    if (Numsteps < 1) raise("number of steps must be >= 1");
    dt_ = dt;
    num_steps_ = Numsteps;
    begun_ = false;
}

void SolverMRGpuT::SetLoadHistory(const std::vector<double>& amp) {
    amp_ = amp;
    check(tdbem_mrt_set_load_history(mrt_, amp_.data(), (int)amp_.size()), "SetLoadHistory");
}

void SolverMRGpuT::GetNodeLowHigh(int* low_1, int* high_1, int* low_2, int* high_2) {
    *low_1 = 0;
    *high_1 = model_[0]->GetNND() - 1;
    *low_2 = 0;
    *high_2 = model_[1]->GetNND() - 1;
}

void SolverMRGpuT::GetDofLowHigh(int* low_1, int* high_1, int* low_2, int* high_2) {
    *low_1 = 0;
    *high_1 = 3 * model_[0]->GetNND() - 1;
    *low_2 = 0;
    *high_2 = 3 * model_[1]->GetNND() - 1;
}

void SolverMRGpuT::UpdateGHLinear(const double* G_0, const double* G_1, const double* H_0,
                                  const double* H_1, const double* g_0, const double* g_1,
                                  const double* h_0, const double* h_1) {
    if (curr_ < 1 || curr_ > max_step_) return;  // SolverMRT.cpp:857
    check(tdbem_update_gh_linear(ctx_[0], curr_, 0, model_[0]->GetNND() - 1, G_0, G_1, H_0, H_1),
          "UpdateGHLinear (region 1)");
    check(tdbem_update_gh_linear(ctx_[1], curr_, 0, model_[1]->GetNND() - 1, g_0, g_1, h_0, h_1),
          "UpdateGHLinear (region 2)");
}

void SolverMRGpuT::Solve() {
    if (curr_ < 1 || curr_ > num_steps_) raise("current step outside 1..num_steps");
    if (!begun_) {
        check(tdbem_mrt_begin(mrt_, num_steps_), "Solve");
        x_.assign(num_steps_ + 1, std::vector<double>(N_, 0.0));
        for (int r = 0; r < 2; r++) {
            const size_t D = 3 * (size_t)model_[r]->GetNND();
            u_[r].assign(num_steps_ + 1, std::vector<double>(D, 0.0));
            t_[r].assign(num_steps_ + 1, std::vector<double>(D, 0.0));
        }
        begun_ = true;
    }
    check(tdbem_mrt_step(mrt_, curr_, x_[curr_].data(), u_[0][curr_].data(), t_[0][curr_].data(),
                         u_[1][curr_].data(), t_[1][curr_].data()),
          "Solve");
}

void SolverMRGpuT::RecordResult() {
    if (curr_ < 1 || !begun_) return;
    const int D2 = 3 * model_[1]->GetNND();
    int dof = record_dof_;
    if (dof < 0) dof = D2 > 137 ? 137 : 2;
    if (dof >= D2) raise("record dof outside region 2");
    std::ofstream f;
    if (curr_ == 1) f.open(result_file_, std::fstream::out | std::fstream::trunc);
    else f.open(result_file_, std::fstream::out | std::fstream::app);
    if (!f) raise("cannot open " + result_file_);
    f << std::setprecision(6);
    f << std::setw(10) << dt_ * (curr_ - 1) << std::setw(15) << u_[1][curr_ - 1][dof]
      << std::endl;
}

}  // namespace tdbem
