/*
 * Dump driver for the TD-BEM reference's two-region solver (SolverMRT), compiled
 * against the reference's own unmodified sources and the single-rank stand-in in
 * ref_shim/.
 *
 * The reference's main() never instantiates SolverMRT; this driver runs it with
 * main()'s per-step pattern (main.cpp:89-126) applied to two models:
 *   ReadInput x2 -> SolverMRT(model_1, model_2) -> SetMaxStep -> SetTimeControl ->
 *   ElastoDynamicsT x2 with SetLowerUpper(GetNodeLowHigh) -> per step n:
 *   G_H_Driver(n dt, dt) on both regions while n <= MaxStep, GetGHLinear x2,
 *   SetCurrStep, UpdateGHLinear(8 blocks), SetLoad, Solve.
 * RecordResult is not called (it writes VTK files and prints a hard-coded dof of
 * one particular mesh, SolverMRT.cpp:1337-1388).
 *
 * At the end it writes the combined level store fG_DB/fH_DB[0..MaxStep], the
 * combined histories fDis_DB_Global/fTrac_DB_Global[0..numstep] and the region
 * displacement histories fDis_DB_1/fDis_DB_2[0..numstep] as raw little-endian
 * float64 files, and a .meta line "N NG D1 D2 MaxStep numstep".
 *
 * Test infrastructure only (generates golden fixtures that pin the oracle's
 * multi-region restatement); never part of the product.
 *
 *   ref_mrt_driver <region1.txt> <region2.txt> <max_step> <out_prefix>
 */
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "ElastoDynamicsT.h"
#include "ModelManagerT.h"
#include "SolverMRT.h"
#include "shim_access.h"

using namespace TD_BEM;

class DumpMRT : public SolverMRT {
public:
    DumpMRT(ModelManagerT* m1, ModelManagerT* m2) : SolverMRT(m1, m2) {}

    void Dump(const char* prefix) {
        std::string p(prefix);
        FILE* meta = std::fopen((p + ".meta").c_str(), "w");
        std::fprintf(meta, "%d %d %d %d %d %d\n", fNumRow_H, fNumCol_G, fNumDofs_1, fNumDofs_2,
                     fMaxStep, fNumStep);
        std::fclose(meta);
        write_vecs(p + ".x", fDis_DB_Global, fNumStep + 1);
        write_vecs(p + ".tg", fTrac_DB_Global, fNumStep + 1);
        write_vecs(p + ".u1", fDis_DB_1, fNumStep + 1);
        write_vecs(p + ".u2", fDis_DB_2, fNumStep + 1);
        write_mats(p + ".G", fG_DB, fMaxStep + 1);
        write_mats(p + ".H", fH_DB, fMaxStep + 1);
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

int main(int argc, char** argv) {
    if (argc != 5) {
        std::cerr << "usage: ref_mrt_driver region1.txt region2.txt max_step out_prefix\n";
        return 2;
    }
    try {
        ModelManagerT* m1 = new ModelManagerT;
        ModelManagerT* m2 = new ModelManagerT;
        m1->ReadInput(argv[1]);
        m2->ReadInput(argv[2]);
        DumpMRT* solver = new DumpMRT(m1, m2);
        const int max_step = std::atoi(argv[3]);
        solver->SetMaxStep(max_step);
        const int num_step = m1->GetNumStep();
        const double dt = m1->GetDT();
        solver->SetTimeControl(dt, num_step);
        ElastoDynamicsT* ed1 = new ElastoDynamicsT(m1);
        ElastoDynamicsT* ed2 = new ElastoDynamicsT(m2);
        int l1, h1, l2, h2;
        solver->GetNodeLowHigh(&l1, &h1, &l2, &h2);
        ed1->SetLowerUpper(l1, h1);
        ed2->SetLowerUpper(l2, h2);
        for (int n = 1; n <= num_step; n++) {
            if (n <= max_step) {
                ed1->G_H_Driver(n * dt, dt);
                ed2->G_H_Driver(n * dt, dt);
            }
            double *G_0, *G_1, *H_0, *H_1, *g_0, *g_1, *h_0, *h_1;
            ed1->GetGHLinear(&G_0, &G_1, &H_0, &H_1);
            ed2->GetGHLinear(&g_0, &g_1, &h_0, &h_1);
            solver->SetCurrStep(n);
            solver->UpdateGHLinear(G_0, G_1, H_0, H_1, g_0, g_1, h_0, h_1);
            solver->SetLoad();
            solver->Solve();
        }
        solver->Dump(argv[4]);
        delete ed1;
        delete ed2;
        delete solver;
        delete m1;
        delete m2;
    } catch (const char* msg) {
        std::cerr << msg << std::endl;
        return 1;
    }
    return 0;
}
