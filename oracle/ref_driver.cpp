/*
 * Dump driver for the TD-BEM reference, compiled against the reference's own
 * unmodified sources and the single-rank stand-in in ref_shim/.
 *
 * It runs the call sequence of the reference's main() (main.cpp:43-128:
 * ReadInput -> SolverStepLinearT -> Distributed_BC -> SetTimeControl ->
 * Initialize -> per step G_H_Driver / GetGHLinear / SetCurrStep /
 * UpdateGHLinear / SetLoad / Solve(a1,a2) / RecordResult), with alpha passed
 * on the command line instead of alpha.txt (main.cpp:78-81), and at the end
 * writes the reference's level store fG_DB/fH_DB[0..MaxStep] and histories
 * fDis_DB/fTrac_DB[0..numstep] as raw little-endian float64 files.
 *
 * Test infrastructure only (generates the golden fixtures that pin the
 * oracle); never part of the product.
 *
 *   ref_driver <input.txt> <a1> <a2> <out_prefix> [nolevels]
 *   ref_driver <input.txt> --assemble <node_lo> <node_hi> <nsteps>
 *       (times G_H_Driver alone on a node range, the reference's MPI row split)
 *   ref_driver <input.txt> --rows <node_lo> <node_hi> <step> <out_prefix>
 *       (one G_H_Driver(step*dt, dt) on a node range; writes the four row blocks
 *       GetGHLinear returns, G_1 G_2 H_1 H_2, as <out_prefix>.rows: 4 x
 *       3*(node_hi-node_lo+1) x 3*nnd float64)
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include "ElastoDynamicsT.h"
#include "ModelManagerT.h"
#include "SolverStepLinearT.h"
#include "shim_access.h"

using namespace TD_BEM;

class DumpSolver : public SolverStepLinearT {
public:
    explicit DumpSolver(ModelManagerT* m) : SolverStepLinearT(m) {}

    void Dump(const char* prefix, int numstep, bool levels) {
        const int D = fGblNumDof;
        std::string p(prefix);
        FILE* meta = std::fopen((p + ".meta").c_str(), "w");
        std::fprintf(meta, "%d %d %d\n", D, fMaxStep, numstep);
        std::fclose(meta);
        write_vecs(p + ".u", fDis_DB, numstep + 1);
        write_vecs(p + ".t", fTrac_DB, numstep + 1);
        if (levels) {
            write_mats(p + ".G", fG_DB, fMaxStep + 1);
            write_mats(p + ".H", fH_DB, fMaxStep + 1);
        }
    }

private:
    static void write_vecs(const std::string& path, Vec* v, int count) {
        FILE* f = std::fopen(path.c_str(), "wb");
        for (int i = 0; i < count; i++) {
            int n;
            const double* a = shim_vec_data(v[i], &n);
            std::fwrite(a, sizeof(double), n, f);
        }
        std::fclose(f);
    }
    static void write_mats(const std::string& path, Mat* m, int count) {
        FILE* f = std::fopen(path.c_str(), "wb");
        for (int i = 0; i < count; i++) {
            int r, c;
            const double* a = shim_mat_data(m[i], &r, &c);
            std::fwrite(a, sizeof(double), (size_t)r * c, f);
        }
        std::fclose(f);
    }
};

static int run_full(const char* input, double a1, double a2, const char* prefix, bool levels) {
    ModelManagerT* model = new ModelManagerT;
    model->ReadInput(input);
    DumpSolver* solver = new DumpSolver(model);
    int dof_low, dof_high;
    solver->GetDofLowHigh(&dof_low, &dof_high);
    model->Distributed_BC(dof_low, dof_high);
    const int num_step = model->GetNumStep();
    const double time_step = model->GetDT();
    solver->SetTimeControl(time_step, num_step);
    solver->Initialize();

    ElastoDynamicsT* ED = new ElastoDynamicsT(model);
    int node_low, node_high;
    solver->GetNodeLowHigh(&node_low, &node_high);
    ED->SetLowerUpper(node_low, node_high);
    for (int curr_step = 1; curr_step <= num_step; curr_step++) {
        const double t_curr = curr_step * time_step;
        const double t_1 = time_step;
        const int MaxStep = solver->GetMaxStep();
        if (curr_step <= MaxStep) ED->G_H_Driver(t_curr, t_1);
        double *G_0, *G_1, *H_0, *H_1;
        ED->GetGHLinear(&G_0, &G_1, &H_0, &H_1);
        solver->SetCurrStep(curr_step);
        solver->UpdateGHLinear(G_0, G_1, H_0, H_1);
        solver->SetLoad();
        solver->Solve(a1, a2);
        solver->RecordResult();
    }
    solver->Dump(prefix, num_step, levels);
    std::fprintf(stderr, "ref_driver: %ld LU factorizations\n", shim_ksp_factorizations());
    delete ED;
    delete solver;
    delete model;
    return 0;
}

static int run_assemble(const char* input, int lo, int hi, int nsteps) {
    ModelManagerT* model = new ModelManagerT;
    model->ReadInput(input);
    ElastoDynamicsT* ED = new ElastoDynamicsT(model);
    ED->SetLowerUpper(lo, hi);
    const double dt = model->GetDT();
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 1; s <= nsteps; s++) ED->G_H_Driver(s * dt, dt);
    auto t1 = std::chrono::steady_clock::now();
    std::printf("ASSEMBLE_SECONDS %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    delete ED;
    delete model;
    return 0;
}

static int run_rows(const char* input, int lo, int hi, int step, const char* prefix) {
    ModelManagerT* model = new ModelManagerT;
    model->ReadInput(input);
    ElastoDynamicsT* ED = new ElastoDynamicsT(model);
    ED->SetLowerUpper(lo, hi);
    const double dt = model->GetDT();
    ED->G_H_Driver(step * dt, dt);
    double* blocks[4];
    ED->GetGHLinear(&blocks[0], &blocks[1], &blocks[2], &blocks[3]);
    const size_t n = (size_t)3 * (hi - lo + 1) * 3 * model->GetNND();
    FILE* f = std::fopen((std::string(prefix) + ".rows").c_str(), "wb");
    for (int b = 0; b < 4; b++) std::fwrite(blocks[b], sizeof(double), n, f);
    std::fclose(f);
    delete ED;
    delete model;
    return 0;
}

int main(int argc, char** argv) {
    try {
        if (argc >= 7 && std::strcmp(argv[2], "--rows") == 0)
            return run_rows(argv[1], std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]),
                            argv[6]);
        if (argc >= 6 && std::strcmp(argv[2], "--assemble") == 0)
            return run_assemble(argv[1], std::atoi(argv[3]), std::atoi(argv[4]),
                                std::atoi(argv[5]));
        if (argc < 5) {
            std::fprintf(stderr, "usage: ref_driver input a1 a2 out_prefix [nolevels]\n");
            return 2;
        }
        const bool levels = !(argc >= 6 && std::strcmp(argv[5], "nolevels") == 0);
        return run_full(argv[1], std::atof(argv[2]), std::atof(argv[3]), argv[4], levels);
    } catch (const char* msg) {
        std::fprintf(stderr, "reference threw: %s\n", msg);
        return 3;
    }
}
