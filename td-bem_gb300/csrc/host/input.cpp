// ModelManagerT::ReadInput: the reference's keyword input format.
//
// Follows InputT::ReadInput (InputT.cpp:84-144) and its per-keyword readers
// (InputT.cpp:146-994): one keyword per line; tokens separated by any of
// " \t=;," (InputT.cpp:21); integers converted with atoi and reals with atof;
// "nodes" and "IEN" are followed by nnd / nel lines; UBC_dof, UBC_values,
// FBC_dof, FBC_values and interface read further lines until their count is
// reached; node and dof ids are 1-based in the file and 0-based in memory
// (InputT.cpp:529, 747, 856); an unknown keyword is an error (InputT.cpp:130-136).
// With formulation = 3 the auxiliary-mesh keywords nnd_aux, etype_aux, nel_aux,
// nodes_aux and IEN_aux are read too (InputT::ReadGeometry_Aux, InputT.cpp:548-693).
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../../include/tdbem_host.hpp"

namespace tdbem {

namespace {

thread_local std::string g_msg;

[[noreturn]] void raise(const std::string& msg) {
    g_msg = msg;
    throw g_msg.c_str();
}

std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> out;
    std::string cur;
    for (char ch : line) {
        if (ch == ' ' || ch == '\t' || ch == '=' || ch == ';' || ch == ',' || ch == '\r' ||
            ch == '\n') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

}  // namespace

void ModelManagerT::ReadInput(const char* name) {
    std::ifstream in(name);
    if (!in) raise(std::string("cannot open input file ") + (name ? name : "(null)"));
    std::vector<std::string> lines;
    for (std::string l; std::getline(in, l);) lines.push_back(l);

    int ubc_num = 0, fbc_num = 0, num_if = 0;
    bool have_nodes = false, have_ien = false;
    auto need = [&](const std::vector<std::string>& t, size_t i) {
        if (t.size() < 2) raise("line " + std::to_string(i + 1) + ": " + t[0] + " is not set properly");
        return t[1].c_str();
    };
    // Reads `count` values from the lines after i (the list readers of InputT).
    auto read_list = [&](size_t& i, int count, auto conv) {
        using V = decltype(conv(""));
        std::vector<V> out;
        while ((int)out.size() < count) {
            if (++i >= lines.size()) raise("unexpected end of file in a dof/value list");
            const auto t = tokens(lines[i]);
            if (t.empty()) raise("line " + std::to_string(i + 1) + ": empty line inside a list");
            for (const auto& s : t)
                if ((int)out.size() < count) out.push_back(conv(s.c_str()));
        }
        return out;
    };
    for (size_t i = 0; i < lines.size(); i++) {
        const auto t = tokens(lines[i]);
        if (t.empty()) continue;
        const std::string& k = t[0];
        if (k == "formulation") formulation_ = std::atoi(need(t, i));
        else if (k == "numstep") numstep_ = std::atoi(need(t, i));
        else if (k == "sd") sd_ = std::atoi(need(t, i));
        else if (k == "if_ext") if_ext_ = std::atoi(need(t, i));
        else if (k == "nnd") nnd_ = std::atoi(need(t, i));
        else if (k == "nel") nel_ = std::atoi(need(t, i));
        else if (k == "dt") dt_ = std::atof(need(t, i));
        else if (k == "E") E_ = std::atof(need(t, i));
        else if (k == "nu") nu_ = std::atof(need(t, i));
        else if (k == "density") rho_ = std::atof(need(t, i));
        else if (k == "interpolation") interpolation_ = (int)std::atof(need(t, i));
        else if (k == "nq") nq_ = (int)std::atof(need(t, i));
        else if (k == "EType") {
            etype_ = std::atoi(need(t, i));
            if (etype_ == 1) ennd_ = 4;
            else if (etype_ == 2) ennd_ = 8;
            else raise("unsupported element type");
        } else if (k == "nodes") {
            coords_.assign(3 * (size_t)nnd_, 0.0);
            for (int n = 0; n < nnd_; n++) {
                if (++i >= lines.size()) raise("unexpected end of file in nodes");
                const auto c = tokens(lines[i]);
                if (c.size() < 3)
                    raise("line " + std::to_string(i + 1) + ": node " + std::to_string(n + 1) +
                          " needs 3 coordinates");
                for (int d = 0; d < 3; d++) coords_[3 * (size_t)n + d] = std::atof(c[d].c_str());
            }
            have_nodes = true;
        } else if (k == "IEN") {
            ien_.assign((size_t)ennd_ * nel_, 0);
            for (int e = 0; e < nel_; e++) {
                if (++i >= lines.size()) raise("unexpected end of file in IEN");
                const auto c = tokens(lines[i]);
                if ((int)c.size() < ennd_)
                    raise("line " + std::to_string(i + 1) + ": element " + std::to_string(e + 1) +
                          " needs " + std::to_string(ennd_) + " nodes");
                for (int a = 0; a < ennd_; a++)
                    ien_[(size_t)e * ennd_ + a] = std::atoi(c[a].c_str()) - 1;
            }
            have_ien = true;
        } else if (k == "UBC_num") ubc_num = std::atoi(need(t, i));
        else if (k == "UBC_dof")
            ubc_dof_ = read_list(i, ubc_num, [](const char* s) { return std::atoi(s) - 1; });
        else if (k == "UBC_values")
            ubc_val_ = read_list(i, ubc_num, [](const char* s) { return std::atof(s); });
        else if (k == "FBC_num") fbc_num = std::atoi(need(t, i));
        else if (k == "FBC_dof")
            fbc_dof_ = read_list(i, fbc_num, [](const char* s) { return std::atoi(s) - 1; });
        else if (k == "FBC_values")
            fbc_val_ = read_list(i, fbc_num, [](const char* s) { return std::atof(s); });
        else if (k == "num_interface") num_if = std::atoi(need(t, i));
        else if (k == "interface")
            interface_ = read_list(i, num_if, [](const char* s) { return std::atoi(s) - 1; });
        else if (formulation_ == 3 && k == "nnd_aux") nnd_aux_ = std::atoi(need(t, i));
        else if (formulation_ == 3 && k == "nel_aux") nel_aux_ = std::atoi(need(t, i));
        else if (formulation_ == 3 && k == "etype_aux") {
            etype_aux_ = std::atoi(need(t, i));
            if (etype_aux_ == 1) ennd_aux_ = 4;
            else if (etype_ == 2) ennd_aux_ = 8;  // the reference tests the main EType (:599)
            else raise("unsupported element type");
        } else if (formulation_ == 3 && k == "nodes_aux") {
            coords_aux_.assign(3 * (size_t)nnd_aux_, 0.0);
            for (int n = 0; n < nnd_aux_; n++) {
                if (++i >= lines.size()) raise("unexpected end of file in nodes_aux");
                const auto c = tokens(lines[i]);
                if (c.size() < 3)
                    raise("line " + std::to_string(i + 1) + ": aux node " + std::to_string(n + 1) +
                          " needs 3 coordinates");
                for (int d = 0; d < 3; d++)
                    coords_aux_[3 * (size_t)n + d] = std::atof(c[d].c_str());
            }
        } else if (formulation_ == 3 && k == "IEN_aux") {
            ien_aux_.assign((size_t)ennd_aux_ * nel_aux_, 0);
            for (int e = 0; e < nel_aux_; e++) {
                if (++i >= lines.size()) raise("unexpected end of file in IEN_aux");
                const auto c = tokens(lines[i]);
                if ((int)c.size() < ennd_aux_)
                    raise("line " + std::to_string(i + 1) + ": aux element " +
                          std::to_string(e + 1) + " needs " + std::to_string(ennd_aux_) +
                          " nodes");
                for (int a = 0; a < ennd_aux_; a++)
                    ien_aux_[(size_t)e * ennd_aux_ + a] = std::atoi(c[a].c_str()) - 1;
            }
        } else
            raise("line " + std::to_string(i + 1) + ": unaccepted key word " + k);
    }
    if (!have_nodes || !have_ien) raise("input has no nodes or no IEN block");
    if ((int)ubc_dof_.size() != ubc_num || (int)ubc_val_.size() != ubc_num)
        raise("UBC_dof / UBC_values do not match UBC_num");
    if ((int)fbc_dof_.size() != fbc_num || (int)fbc_val_.size() != fbc_num)
        raise("FBC_dof / FBC_values do not match FBC_num");
}

void ModelManagerT::BoundaryCondition_Global(int& UBC_num, int** UBC_DOFs, double** UBC_Values,
                                             int& FBC_num, int** FBC_DOFs,
                                             double** FBC_Values) {
    UBC_num = (int)ubc_dof_.size();
    FBC_num = (int)fbc_dof_.size();
    *UBC_DOFs = ubc_dof_.data();
    *UBC_Values = ubc_val_.data();
    *FBC_DOFs = fbc_dof_.data();
    *FBC_Values = fbc_val_.data();
}

void ModelManagerT::SetBCs(int UBC_num, const int* UBC_DOFs, const double* UBC_values,
                           int FBC_num, const int* FBC_DOFs, const double* FBC_values) {
    ubc_dof_.assign(UBC_DOFs, UBC_DOFs + UBC_num);
    ubc_val_.assign(UBC_values, UBC_values + UBC_num);
    fbc_dof_.assign(FBC_DOFs, FBC_DOFs + FBC_num);
    fbc_val_.assign(FBC_values, FBC_values + FBC_num);
}

tdbem_mesh ModelManagerT::Mesh() const {
    return tdbem_mesh{nnd_, nel_, etype_, coords_.data(), ien_.data()};
}

tdbem_material ModelManagerT::Material() const { return tdbem_material{E_, nu_, rho_}; }

}  // namespace tdbem
