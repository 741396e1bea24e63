// Test driver of TDElementGpuT (include/tdbem_host.hpp) with the reference's
// element call sequence (ElastoDynamicsT.cpp:108-231: SetNQ, SetMaterial, then per
// element SetCollocation, SetCoords, SetTime, FormGH_Regular or
// FormGH_Singular(node), GetGHLinear).
//
// stdin:  etype nq E nu rho mode      (mode 0: read each element after forming it;
//         n                            mode 1: form all, then read pair by pair)
//         n lines: t t_1 singular x y z c_0 ... c_{3 ennd - 1}
// stdout: per pair six lines, GE_1 GE_2 HE_1 HE_2 (3 x 3 ennd) and C_1 C_2 (9), %.17g
#include <cstdio>
#include <vector>

#include "tdbem_host.hpp"

int main() {
    int etype, nq, mode, n;
    double E, nu, rho;
    if (std::scanf("%d %d %lf %lf %lf %d %d", &etype, &nq, &E, &nu, &rho, &mode, &n) != 7)
        return 2;
    const int ennd = etype == 1 ? 4 : 8;
    std::vector<double> t(n), t1(n), xc(3 * n), en(3 * ennd * n);
    std::vector<int> sing(n);
    for (int i = 0; i < n; i++) {
        if (std::scanf("%lf %lf %d", &t[i], &t1[i], &sing[i]) != 3) return 2;
        for (int d = 0; d < 3; d++)
            if (std::scanf("%lf", &xc[3 * i + d]) != 1) return 2;
        for (int m = 0; m < 3 * ennd; m++)
            if (std::scanf("%lf", &en[3 * ennd * i + m]) != 1) return 2;
    }
    auto print = [&](const double* const* b) {
        for (int k = 0; k < 6; k++) {
            const int len = k < 4 ? 9 * ennd : 9;
            for (int m = 0; m < len; m++) std::printf("%.17g ", b[k][m]);
            std::printf("\n");
        }
    };
    try {
        tdbem::TDElementGpuT el(etype);
        el.SetNQ(nq);
        el.SetMaterial(E, nu, rho);
        for (int i = 0; i < n; i++) {
            el.SetCollocation(&xc[3 * i]);
            el.SetCoords(&en[3 * ennd * i]);
            el.SetTime(t[i], t1[i]);
            if (sing[i] < 0) el.FormGH_Regular();
            else el.FormGH_Singular(sing[i]);
            if (mode == 0) {
                const double* b[6];
                el.GetGHLinear(&b[0], &b[1], &b[2], &b[3], &b[4], &b[5]);
                print(b);
            }
        }
        if (mode == 1) {
            const double* b[6];
            el.GetGHLinear(&b[0], &b[1], &b[2], &b[3], &b[4], &b[5]);  // evaluates the queue
            for (int k = 0; k < el.NumEvaluated(); k++) {
                el.GetGHLinear(k, &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]);
                print(b);
            }
        }
    } catch (const char* msg) {
        std::fprintf(stderr, "%s\n", msg);
        return 3;
    }
    return 0;
}
