// tdbem_run: main.cpp's transient solve on one GB300.
//
//   tdbem_run input.txt [options]
//
// Default: the reference's sequence (src/main.cpp:42-130) with the GPU host
// classes: read the input file and alpha.txt, then for every step
// G_H_Driver (steps <= MaxStep), GetGHLinear, SetCurrStep, UpdateGHLinear,
// SetLoad, Solve(a1, a2), RecordResult -> displacement.txt.
//
// Options:
//   --fast                whole-run path: tdbem_assemble_levels + tdbem_march
//                         (no per-step host copies of the G/H blocks); writes
//                         the same displacement.txt
//   --mixed               with --fast: mixed precision (FP32 far field and
//                         levels, FP64 LHS and refinement)
//   --alpha a1 a2         weights instead of alpha.txt
//   --load-history file   per-step load amplitudes (one value per step)
//   --result file         instead of displacement.txt
//   --dump file           binary histories: int32 numstep, int32 D, then
//                         (numstep+1) x D doubles of u, then of t
//   --write-gh prefix     stepwise path: the step matrices main.cpp's commented
//                         block writes (prefix G1_step / G2_step / H1_step /
//                         H2_step, SolverT::WriteGH format)
//   --export-levels file  --fast: write the level store after assembly
//   --import-levels file  --fast: read the level store instead of assembling
//   --region2 file        two-region run (SolverMRT, formulation = 3): input.txt
//                         is region 1, file region 2; per step G_H_Driver on both
//                         regions while step <= MaxStep, UpdateGHLinear with both
//                         regions' blocks, SetLoad, Solve, RecordResult; --fast
//                         assembles both regions' levels and marches in one call.
//                         --dump writes int32 numstep, int32 N, then (numstep+1) x N
//                         doubles of the combined unknowns
//   --max-step L          two-region run: SolverMRT's level count (default 10)
//   --parse-only          print the model summary and exit (no GPU needed)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "../../../include/tdbem_host.hpp"

namespace {

struct Options {
    const char* input = nullptr;
    bool fast = false, mixed = false, parse_only = false, have_alpha = false;
    double a1 = 0, a2 = 0;
    std::string load_history, result = "displacement.txt", dump, write_gh, export_levels,
                import_levels, region2;
    int max_step = 10;
};

void usage() {
    std::cerr << "usage: tdbem_run input.txt [--fast] [--mixed] [--alpha a1 a2] "
                 "[--load-history file] [--result file] [--dump file] [--write-gh prefix] "
                 "[--export-levels file] [--import-levels file] [--region2 file] "
                 "[--max-step L] [--parse-only]\n";
}

bool parse_args(int argc, char** argv, Options& o) {
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
        if (a == "--fast") o.fast = true;
        else if (a == "--mixed") o.mixed = true;
        else if (a == "--parse-only") o.parse_only = true;
        else if (a == "--alpha") {
            const char* x = next();
            const char* y = next();
            if (!x || !y) return false;
            o.a1 = std::atof(x);
            o.a2 = std::atof(y);
            o.have_alpha = true;
        } else if (a == "--max-step") {
            const char* v = next();
            if (!v) return false;
            o.max_step = std::atoi(v);
        } else if (a == "--load-history" || a == "--result" || a == "--dump" ||
                   a == "--write-gh" || a == "--export-levels" || a == "--import-levels" ||
                   a == "--region2") {
            const char* v = next();
            if (!v) return false;
            if (a == "--load-history") o.load_history = v;
            else if (a == "--result") o.result = v;
            else if (a == "--dump") o.dump = v;
            else if (a == "--write-gh") o.write_gh = v;
            else if (a == "--export-levels") o.export_levels = v;
            else if (a == "--region2") o.region2 = v;
            else o.import_levels = v;
        } else if (!a.empty() && a[0] == '-') return false;
        else if (!o.input) o.input = argv[i];
        else return false;
    }
    return o.input != nullptr;
}

std::vector<double> read_values(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw "cannot open the load history file";
    std::vector<double> v;
    for (std::string tok; in >> tok;) v.push_back(std::atof(tok.c_str()));
    return v;
}

void write_line(std::ofstream& f, double time, double amp, double u2, double t2) {
    f << std::setprecision(6) << std::setw(10) << time << std::setw(15) << amp << std::setw(15)
      << u2 << std::setw(15) << t2 << std::endl;
}

void dump(const std::string& path, int numstep, int D, const std::vector<double>& u,
          const std::vector<double>& t) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw "cannot open the dump file";
    const int32_t hdr[2] = {numstep, D};
    f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    f.write(reinterpret_cast<const char*>(u.data()), sizeof(double) * u.size());
    f.write(reinterpret_cast<const char*>(t.data()), sizeof(double) * t.size());
    if (!f) throw "writing the dump file failed";
}

void tcheck(int rc) {
    static std::string msg;
    if (rc != TDBEM_OK) {
        msg = tdbem_last_error();
        throw msg.c_str();
    }
}

// The reference's loop with the GPU host classes.
void run_stepwise(tdbem::ModelManagerT& model, const Options& o, double a1, double a2,
                  const std::vector<double>& amp) {
    tdbem::SolverStepLinearGpuT solver(&model);
    solver.SetResultFile(o.result);
    int dof_low, dof_high;
    solver.GetDofLowHigh(&dof_low, &dof_high);
    model.Distributed_BC(dof_low, dof_high);
    const int num_step = model.GetNumStep();
    const double time_step = model.GetDT();
    solver.SetTimeControl(time_step, num_step);
    if (!amp.empty()) solver.SetLoadHistory(amp);
    solver.Initialize();
    tdbem::ElastoDynamicsGpuT ED(&model, &solver);
    int node_low, node_high;
    solver.GetNodeLowHigh(&node_low, &node_high);
    ED.SetLowerUpper(node_low, node_high);
    const int MaxStep = solver.GetMaxStep();
    for (int curr_step = 1; curr_step <= num_step; curr_step++) {
        const double t_curr = curr_step * time_step, t_1 = time_step;
        if (curr_step <= MaxStep) ED.G_H_Driver(t_curr, t_1);
        double *G_0, *G_1, *H_0, *H_1;
        ED.GetGHLinear(&G_0, &G_1, &H_0, &H_1);
        if (!o.write_gh.empty() && curr_step <= MaxStep) {
            const int rows = dof_high - dof_low + 1, cols = 3 * model.GetNND();
            solver.WriteGH((o.write_gh + "G1_step").c_str(), curr_step - 1, rows, cols, G_1);
            solver.WriteGH((o.write_gh + "G2_step").c_str(), curr_step - 1, rows, cols, G_0);
            solver.WriteGH((o.write_gh + "H1_step").c_str(), curr_step - 1, rows, cols, H_1);
            solver.WriteGH((o.write_gh + "H2_step").c_str(), curr_step - 1, rows, cols, H_0);
        }
        solver.SetCurrStep(curr_step);
        solver.UpdateGHLinear(G_0, G_1, H_0, H_1);
        solver.SetLoad();
        solver.Solve(a1, a2);
        solver.RecordResult();
    }
    if (!o.dump.empty()) {
        const int D = 3 * model.GetNND();
        std::vector<double> u((size_t)(num_step + 1) * D, 0.0), t(u.size(), 0.0);
        for (int s = 0; s < num_step; s++) {
            std::copy(solver.Displacement(s).begin(), solver.Displacement(s).end(),
                      u.begin() + (size_t)s * D);
            std::copy(solver.Traction(s).begin(), solver.Traction(s).end(),
                      t.begin() + (size_t)s * D);
        }
        dump(o.dump, num_step, D, u, t);
    }
}

// Whole run on the device: every level, then every step.
void run_fast(tdbem::ModelManagerT& model, const Options& o, double a1, double a2,
              const std::vector<double>& amp) {
    const tdbem_mesh mesh = model.Mesh();
    const tdbem_material mat = model.Material();
    tdbem_ctx* ctx = nullptr;
    tcheck(tdbem_ctx_create(&mesh, &mat, model.GetDT(), model.GetNQ(), model.GetIfExt(), &ctx));
    struct Guard {
        tdbem_ctx* c;
        ~Guard() { tdbem_ctx_destroy(c); }
    } guard{ctx};
    int nu = 0, nf = 0;
    int *ud, *fd;
    double *uv, *fv;
    model.BoundaryCondition_Global(nu, &ud, &uv, nf, &fd, &fv);
    tcheck(tdbem_set_bc(ctx, ud, uv, nu, fd, fv, nf));
    tcheck(tdbem_set_alpha(ctx, a1, a2));
    if (!amp.empty()) tcheck(tdbem_set_load_history(ctx, amp.data(), (int)amp.size()));
    const int n = model.GetNumStep(), D = 3 * model.GetNND();
    if (!o.import_levels.empty()) tcheck(tdbem_import_levels(ctx, o.import_levels.c_str()));
    else tcheck(tdbem_assemble_levels(ctx, n, o.mixed ? TDBEM_MIXED : TDBEM_FP64));
    if (!o.export_levels.empty()) tcheck(tdbem_export_levels(ctx, o.export_levels.c_str()));
    std::vector<double> u((size_t)(n + 1) * D), t(u.size());
    tcheck(tdbem_march(ctx, n, u.data(), t.data()));
    std::ofstream f(o.result, std::fstream::out | std::fstream::trunc);
    if (!f) throw "cannot open the result file";
    f << std::setw(10) << "%time" << std::setw(15) << "load" << std::setw(15) << "displacement"
      << std::setw(15) << "traction" << std::endl;
    for (int s = 0; s < n; s++) {
        const double time = model.GetDT() * s;
        const double a = amp.empty() ? 1.0 : amp[s];
        write_line(f, time, a, u[(size_t)s * D + 2], t[(size_t)s * D + 2]);
    }
    if (!o.dump.empty()) dump(o.dump, n, D, u, t);
}

void dump_x(const std::string& path, int numstep, int N, const std::vector<double>& x) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw "cannot open the dump file";
    const int32_t hdr[2] = {numstep, N};
    f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    f.write(reinterpret_cast<const char*>(x.data()), sizeof(double) * x.size());
    if (!f) throw "writing the dump file failed";
}

// The two-region solver with the per-step pattern of main.cpp (89-126) applied to
// both regions, or (--fast) the whole run on the device.
void run_mrt(tdbem::ModelManagerT& m1, tdbem::ModelManagerT& m2, const Options& o,
             const std::vector<double>& amp) {
    const int num_step = m1.GetNumStep();
    const double dt = m1.GetDT();
    tdbem::SolverMRGpuT solver(&m1, &m2);
    solver.SetResultFile(o.result);
    solver.SetMaxStep(o.max_step);
    solver.SetTimeControl(dt, num_step);
    if (!amp.empty()) solver.SetLoadHistory(amp);
    const int N = solver.NumUnknowns();
    std::vector<double> x((size_t)(num_step + 1) * N, 0.0);
    if (o.fast) {
        tdbem_mrt* mrt = nullptr;
        tcheck(tdbem_mrt_create(solver.Context(1), solver.Context(2), m1.GetInterface(),
                                m2.GetInterface(), m1.GetNumInterface(), o.max_step, &mrt));
        struct Guard {
            tdbem_mrt* m;
            ~Guard() { tdbem_mrt_destroy(m); }
        } guard{mrt};
        if (!amp.empty()) tcheck(tdbem_mrt_set_load_history(mrt, amp.data(), (int)amp.size()));
        tcheck(tdbem_mrt_assemble(mrt, num_step));
        const int D2 = 3 * m2.GetNND();
        std::vector<double> u2((size_t)(num_step + 1) * D2);
        tcheck(tdbem_mrt_march(mrt, num_step, x.data(), nullptr, nullptr, u2.data(), nullptr));
        std::ofstream f(o.result, std::fstream::out | std::fstream::trunc);
        if (!f) throw "cannot open the result file";
        const int dof = D2 > 137 ? 137 : 2;  // SolverMRGpuT::RecordResult's default
        f << std::setprecision(6);
        for (int s = 0; s < num_step; s++)
            f << std::setw(10) << dt * s << std::setw(15) << u2[(size_t)s * D2 + dof]
              << std::endl;
    } else {
        tdbem::ElastoDynamicsGpuT ed1(&m1, &solver, 1), ed2(&m2, &solver, 2);
        int l1, h1, l2, h2;
        solver.GetNodeLowHigh(&l1, &h1, &l2, &h2);
        ed1.SetLowerUpper(l1, h1);
        ed2.SetLowerUpper(l2, h2);
        const int max_step = solver.GetMaxStep();
        for (int n = 1; n <= num_step; n++) {
            if (n <= max_step) {
                ed1.G_H_Driver(n * dt, dt);
                ed2.G_H_Driver(n * dt, dt);
            }
            double *G_0, *G_1, *H_0, *H_1, *g_0, *g_1, *h_0, *h_1;
            ed1.GetGHLinear(&G_0, &G_1, &H_0, &H_1);
            ed2.GetGHLinear(&g_0, &g_1, &h_0, &h_1);
            solver.SetCurrStep(n);
            solver.UpdateGHLinear(G_0, G_1, H_0, H_1, g_0, g_1, h_0, h_1);
            solver.SetLoad();
            solver.Solve();
            solver.RecordResult();
        }
        for (int n = 1; n <= num_step; n++)
            std::copy(solver.Unknowns(n).begin(), solver.Unknowns(n).end(),
                      x.begin() + (size_t)n * N);
    }
    if (!o.dump.empty()) dump_x(o.dump, num_step, N, x);
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    if (!parse_args(argc, argv, o)) {
        usage();
        return 2;
    }
    try {
        tdbem::ModelManagerT model;
        model.ReadInput(o.input);
        if (o.parse_only) {
            int nu, nf;
            int *ud, *fd;
            double *uv, *fv;
            model.BoundaryCondition_Global(nu, &ud, &uv, nf, &fd, &fv);
            double E, nuv, rho;
            model.GetMaterialConstants(E, nuv, rho);
            double csum = 0, bsum = 0;
            long isum = 0;
            for (int i = 0; i < 3 * model.GetNND(); i++) csum += model.GetCoords()[i] * (1 + i % 7);
            for (int i = 0; i < model.GetENND() * model.GetNEL(); i++)
                isum += (long)model.GetIEN()[i] * (1 + i % 5);
            for (int i = 0; i < nu; i++) bsum += (ud[i] + 1) * uv[i];
            for (int i = 0; i < nf; i++) bsum += (fd[i] + 1) * fv[i];
            long ifsum = 0, auxsum = 0;
            for (int i = 0; i < model.GetNumInterface(); i++)
                ifsum += (long)(model.GetInterface()[i] + 1) * (1 + i % 3);
            for (int i = 0; i < model.GetENND_Aux() * model.GetNEL_Aux(); i++)
                auxsum += (long)model.GetIEN_Aux()[i] * (1 + i % 5);
            std::printf(
                "nnd %d nel %d etype %d numstep %d dt %.17g nq %d if_ext %d E %.17g nu %.17g "
                "rho %.17g ubc %d fbc %d coordsum %.17g iensum %ld bcsum %.17g formulation %d "
                "ninterface %d ifsum %ld nnd_aux %d nel_aux %d auxsum %ld\n",
                model.GetNND(), model.GetNEL(), model.GetElementType(), model.GetNumStep(),
                model.GetDT(), model.GetNQ(), model.GetIfExt(), E, nuv, rho, nu, nf, csum, isum,
                bsum, model.GetFormulation(), model.GetNumInterface(), ifsum, model.GetNND_Aux(),
                model.GetNEL_Aux(), auxsum);
            return 0;
        }
        if (!o.region2.empty()) {
            tdbem::ModelManagerT model2;
            model2.ReadInput(o.region2.c_str());
            std::vector<double> amp;
            if (!o.load_history.empty()) {
                amp = read_values(o.load_history);
                if ((int)amp.size() < model.GetNumStep() + 1)
                    throw "load history shorter than numstep + 1 (amp[n] at n dt)";
            }
            run_mrt(model, model2, o, amp);
            return 0;
        }
        double a1 = o.a1, a2 = o.a2;
        if (!o.have_alpha) {
            std::ifstream alpha_reader("alpha.txt");  // main.cpp:78-81
            if (alpha_reader) alpha_reader >> a1 >> a2;
        }
        std::cout << "***********************************\n"
                  << "alpha_1=" << a1 << "  alpha_2=" << a2 << "\n"
                  << "***********************************" << std::endl;
        std::vector<double> amp;
        if (!o.load_history.empty()) {
            amp = read_values(o.load_history);
            if ((int)amp.size() < model.GetNumStep()) throw "load history shorter than numstep";
            amp.resize(model.GetNumStep());
        }
        if (o.fast) run_fast(model, o, a1, a2, amp);
        else run_stepwise(model, o, a1, a2, amp);
    } catch (const char* msg) {
        std::cerr << msg << std::endl;
        return 1;
    }
    return 0;
}
