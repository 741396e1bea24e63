// TDElementGpuT: the reference's element interface (TDElementT.h:16-115,
// TDElementStepLinearT) over the batched element call of the C ABI
// (tdbem_element_gh).  Pairs formed between two reads are evaluated together.
#include <string>
#include <vector>

#include "../../../include/tdbem_host.hpp"

namespace tdbem {

namespace {

thread_local std::string g_emsg;

[[noreturn]] void throw_msg(const std::string& m) {
    g_emsg = m;
    throw g_emsg.c_str();
}

}  // namespace

TDElementGpuT::TDElementGpuT(int type) : type_(type) {
    // TDElementT::TDElementT (TDElementT.cpp:17-56) throws for other types
    if (type != 1 && type != 2)
        throw_msg("TDElementGpuT::TDElementGpuT, unsupported element type");
    ennd_ = type == 1 ? 4 : 8;
}

void TDElementGpuT::SetCollocation(double* collocation) { colloc_ = collocation; }

void TDElementGpuT::SetCoords(double* coords) { coords_ = coords; }

void TDElementGpuT::SetTime(double t, double t_1) {
    if (t_1 != t_1_ && !q_sing_.empty()) Evaluate();
    t_ = t;
    t_1_ = t_1;
}

void TDElementGpuT::SetNQ(int nq) {
    if (nq != nq_ && !q_sing_.empty()) Evaluate();
    nq_ = nq;
}

void TDElementGpuT::SetMaterial(double E, double nu, double density) {
    if ((E != E_ || nu != nu_ || density != rho_) && !q_sing_.empty()) Evaluate();
    E_ = E;
    nu_ = nu;
    rho_ = density;
}

void TDElementGpuT::FormGH_Regular() { Queue(-1); }

void TDElementGpuT::FormGH_Singular(int singular) {
    // FormGH_Singular_1 / SubElement accept the element's local nodes only
    // (TDElementStepLinearT.cpp:407-427, 192-386)
    if (singular < 0 || singular >= ennd_)
        throw_msg("TDElementGpuT::FormGH_Singular, collocation id is out of range");
    Queue(singular);
}

void TDElementGpuT::Queue(int singular) {
    if (!colloc_ || !coords_)
        throw_msg("TDElementGpuT: SetCollocation and SetCoords before FormGH");
    if (q_sing_.empty()) evaluated_ = 0;  // the previous evaluation's blocks are released
    q_colloc_.insert(q_colloc_.end(), colloc_, colloc_ + 3);
    q_coords_.insert(q_coords_.end(), coords_, coords_ + 3 * ennd_);
    q_t_.push_back(t_);
    q_sing_.push_back(singular);
}

void TDElementGpuT::Evaluate() {
    const int n = (int)q_sing_.size();
    if (n == 0) return;
    const size_t blk = 9 * (size_t)ennd_;
    ge1_.assign(blk * n, 0);
    ge2_.assign(blk * n, 0);
    he1_.assign(blk * n, 0);
    he2_.assign(blk * n, 0);
    c1_.assign(9 * (size_t)n, 0);
    c2_.assign(9 * (size_t)n, 0);
    const int rc = tdbem_element_gh(type_, nq_, E_, nu_, rho_, t_1_, n, q_colloc_.data(),
                                    q_coords_.data(), q_t_.data(), q_sing_.data(), ge1_.data(),
                                    ge2_.data(), he1_.data(), he2_.data(), c1_.data(),
                                    c2_.data());
    q_colloc_.clear();
    q_coords_.clear();
    q_t_.clear();
    q_sing_.clear();
    if (rc != TDBEM_OK)
        throw_msg(std::string("TDElementGpuT: tdbem_element_gh: ") + tdbem_last_error());
    evaluated_ = n;
}

void TDElementGpuT::GetGHLinear(const double** GE_1, const double** GE_2, const double** HE_1,
                                const double** HE_2, const double** C_1, const double** C_2) {
    Evaluate();
    if (evaluated_ == 0) throw_msg("TDElementGpuT::GetGHLinear before FormGH");
    GetGHLinear(evaluated_ - 1, GE_1, GE_2, HE_1, HE_2, C_1, C_2);
}

void TDElementGpuT::GetGHLinear(int k, const double** GE_1, const double** GE_2,
                                const double** HE_1, const double** HE_2, const double** C_1,
                                const double** C_2) {
    Evaluate();
    if (k < 0 || k >= evaluated_) throw_msg("TDElementGpuT::GetGHLinear, pair out of range");
    const size_t blk = 9 * (size_t)ennd_;
    *GE_1 = ge1_.data() + blk * k;
    *GE_2 = ge2_.data() + blk * k;
    *HE_1 = he1_.data() + blk * k;
    *HE_2 = he2_.data() + blk * k;
    *C_1 = c1_.data() + 9 * (size_t)k;
    *C_2 = c2_.data() + 9 * (size_t)k;
}

}  // namespace tdbem
