// C ABI of tdbem-gb300, the element interface: TDElementStepLinearT's element-level
// quadrature (FormGH_Regular / FormGH_Singular + GetGHLinear,
// TDElementStepLinearT.cpp:28-626) for a batch of independent (collocation point,
// element) pairs in one launch.  The C++ class TDElementGpuT (element_host.cpp)
// queues the pairs of the reference's per-element calls and evaluates them here.
#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

namespace {

// Device copies of one call's inputs and outputs, freed on every return path.
struct ElementBuffers {
    double *colloc = nullptr, *coords = nullptr, *t = nullptr, *gx = nullptr, *gw = nullptr;
    double *out = nullptr;
    int* sing = nullptr;
    ~ElementBuffers() {
        dfree(colloc);
        dfree(coords);
        dfree(t);
        dfree(gx);
        dfree(gw);
        dfree(out);
        dfree(sing);
    }
};

}  // namespace

extern "C" {

int tdbem_element_gh(int etype, int nq, double E, double nu, double rho, double t_1, int n,
                     const double* colloc, const double* coords, const double* t,
                     const int* singular, double* GE_1, double* GE_2, double* HE_1,
                     double* HE_2, double* C_1, double* C_2) {
    if (etype != 1 && etype != 2) return fail(TDBEM_ERR_ARG, "element type %d", etype);
    std::vector<double> hx, hw;
    if (!gauss_table(nq, hx, hw)) return fail(TDBEM_ERR_ARG, "nq = %d has no Gauss table", nq);
    if (!(E > 0) || !(nu > -1 && nu < 0.5) || !(rho > 0) || !(t_1 > 0))
        return fail(TDBEM_ERR_ARG, "material (%g, %g, %g) or t_1 = %g out of range", E, nu, rho,
                    t_1);
    if (n < 0) return fail(TDBEM_ERR_ARG, "n = %d", n);
    if (n == 0) return TDBEM_OK;
    if (!colloc || !coords || !t || !singular || !GE_1 || !GE_2 || !HE_1 || !HE_2 || !C_1 ||
        !C_2)
        return fail(TDBEM_ERR_ARG, "null argument");
    const int ennd = etype == 1 ? 4 : 8;
    for (int i = 0; i < n; i++)
        if (singular[i] < -1 || singular[i] >= ennd)
            return fail(TDBEM_ERR_ARG, "pair %d: singular node %d of a %d-node element", i,
                        singular[i], ennd);
    const size_t nn = (size_t)n, blk = 9 * (size_t)ennd;
    cudaStream_t s = cudaStreamPerThread;
    ElementBuffers b;
    CUDA_TRY(dalloc(&b.colloc, 3 * nn));
    CUDA_TRY(dalloc(&b.coords, 3 * ennd * nn));
    CUDA_TRY(dalloc(&b.t, nn));
    CUDA_TRY(dalloc(&b.sing, nn));
    CUDA_TRY(dalloc(&b.gx, hx.size()));
    CUDA_TRY(dalloc(&b.gw, hw.size()));
    CUDA_TRY(dalloc(&b.out, (4 * blk + 18) * nn));
    CUDA_TRY(cudaMemcpyAsync(b.colloc, colloc, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(b.coords, coords, sizeof(double) * 3 * ennd * nn,
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(b.t, t, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(b.sing, singular, sizeof(int) * nn, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(b.gx, hx.data(), sizeof(double) * hx.size(), cudaMemcpyHostToDevice,
                             s));
    CUDA_TRY(cudaMemcpyAsync(b.gw, hw.data(), sizeof(double) * hw.size(), cudaMemcpyHostToDevice,
                             s));
    double* d_out[6] = {b.out, b.out + blk * nn, b.out + 2 * blk * nn, b.out + 3 * blk * nn,
                        b.out + 4 * blk * nn, b.out + 4 * blk * nn + 9 * nn};
    const Phys ph = make_phys(E, nu, rho, t_1);
    CUDA_TRY(launch_element_gh(ennd, n, nq, b.gx, b.gw, ph, b.colloc, b.coords, b.t, b.sing,
                               d_out[0], d_out[1], d_out[2], d_out[3], d_out[4], d_out[5], s));
    double* h_out[6] = {GE_1, GE_2, HE_1, HE_2, C_1, C_2};
    for (int k = 0; k < 6; k++)
        CUDA_TRY(cudaMemcpyAsync(h_out[k], d_out[k], sizeof(double) * (k < 4 ? blk : 9) * nn,
                                 cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    return TDBEM_OK;
}

}  // extern "C"
