// tdbem_gh_driver_noalloc: the single-step assembly of tdbem_gh_driver for
// callers that cannot allocate device memory.
//
// Some host applications own every byte of device memory: they reserve their
// pools when they start and forbid libraries to call cudaMalloc / cudaFree later
// (a serving process with a fixed memory budget, or a latency-critical loop where
// the implicit device synchronisation of cudaMalloc / cudaFree is not
// acceptable).  tdbem_gh_driver allocates a device staging buffer on every call;
// this variant writes into device buffers the caller already owns and keeps the
// per-call scratch of the kernels (pair windows, the C term) in one fixed-size
// array in device memory that is part of the library image (kNoAllocScratchBytes;
// every GPU that loads the library holds it until the process exits).  The call
// never waits for the device: a step has at most one item per (node, element)
// pair, so the quadrature runs one thread per pair of a window pass
// (k_assemble_step_pairs) instead of compacting the items with a scan whose total
// the host would have to read back.
//
// Every call shares that array and it keeps the last call's contents; each call
// overwrites what it reads (windows and the C term are recomputed, outputs are
// zeroed first), but calls whose work overlaps on the GPU (other streams, other
// host threads) race on it and must be serialised by the caller.  The array's
// device address is looked up with the context's device current on every call made
// outside a stream capture (so a device reset that reloads the module is seen) and
// taken from the last lookup during a capture; make the first call on a device
// before any capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "tdbem_internal.cuh"

using namespace tdbem;

namespace {

constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB
constexpr size_t kMaxPairs = 1u << 18;             // pairs per launch chunk
constexpr size_t kMaxNodes = 1u << 14;             // collocation nodes per chunk (C term)
constexpr int kMaxDevices = 64;

// Layout: PairInfo[kMaxPairs] | C term[kMaxNodes * 9].
constexpr size_t kOffPairs = 0;
constexpr size_t kOffCterm = kOffPairs + kMaxPairs * sizeof(PairInfo);
static_assert(kOffCterm + kMaxNodes * 9 * sizeof(double) <= kNoAllocScratchBytes,
              "scratch layout exceeds the array");
static_assert(kOffCterm % 256 == 0, "scratch regions stay 256-byte aligned");

// Per-launch chunk limits: the maxima above, or smaller ones from the environment
// (TDBEM_NOALLOC_CHUNK_PAIRS / TDBEM_NOALLOC_CHUNK_NODES) so that a test can make a
// small mesh run several chunks.
size_t chunk_limit(const char* name, size_t max) {
    const char* v = std::getenv(name);
    if (!v || !*v) return max;
    const long long n = std::atoll(v);
    return n >= 1 ? std::min<size_t>((size_t)n, max) : max;
}

std::mutex g_mu;
void* g_scratch[kMaxDevices] = {};

int nfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    tdbem::note_error(buf);  // becomes tdbem_last_error() of this thread
    return code;
}

}  // namespace

// The scratch array itself: a file-scope device symbol, not a host address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of the scratch array on the current device: looked up with that
// device current whenever the stream is not being captured (a reset device may have
// reloaded the module at another address), the last lookup otherwise.
int scratch_address(int dev, cudaStream_t s, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) return nfail(TDBEM_ERR_UNSUPPORTED, "device %d", dev);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t ec = cudaStreamIsCapturing(s, &cap);
    if (ec != cudaSuccess)
        return nfail(TDBEM_ERR_CUDA, "cudaStreamIsCapturing: %s", cudaGetErrorString(ec));
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev] && cap != cudaStreamCaptureStatusNone)
        return nfail(TDBEM_ERR_STATE,
                     "first allocation-free call on device %d made during a stream capture", dev);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return nfail(TDBEM_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s",
                         cudaGetErrorString(e));
        g_scratch[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch[dev]);
    return TDBEM_OK;
}

#define NA_TRY(expr)                                                                        \
    do {                                                                                    \
        const cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess)                                                              \
            return nfail(TDBEM_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_));          \
    } while (0)

}  // namespace

extern "C" int tdbem_gh_driver_noalloc(const tdbem_ctx* c, int step, int node_lo, int node_hi,
                                       double* d_G_I, double* d_G_J, double* d_H_I,
                                       double* d_H_J, void* stream) {
    if (!c || !d_G_I || !d_G_J || !d_H_I || !d_H_J)
        return nfail(TDBEM_ERR_ARG, "null argument");
    if (step < 1) return nfail(TDBEM_ERR_ARG, "step must be >= 1");
    if (node_lo < 0 || node_hi >= c->nnd || node_lo > node_hi)
        return nfail(TDBEM_ERR_ARG, "node range [%d, %d] invalid", node_lo, node_hi);
    int dev = -1;
    NA_TRY(cudaGetDevice(&dev));
    if (dev != c->device)
        return nfail(TDBEM_ERR_ARG, "current device %d is not the context's device %d", dev,
                     c->device);
    int max_color = 0;
    for (size_t k = 0; k + 1 < c->color_start.size(); k++)
        max_color = std::max(max_color, c->color_start[k + 1] - c->color_start[k]);
    if ((size_t)max_color > kMaxPairs)
        return nfail(TDBEM_ERR_UNSUPPORTED,
                     "an element colour of %d elements exceeds the allocation-free maximum of "
                     "%zu pairs per launch (8 MiB scratch)",
                     max_color, kMaxPairs);
    const size_t max_pairs = chunk_limit("TDBEM_NOALLOC_CHUNK_PAIRS", kMaxPairs);
    const int max_nodes = (int)chunk_limit("TDBEM_NOALLOC_CHUNK_NODES", kMaxNodes);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    unsigned char* base = nullptr;
    const int rc0 = scratch_address(dev, s, &base);
    if (rc0 != TDBEM_OK) return rc0;
    PairInfo* pairs = reinterpret_cast<PairInfo*>(base + kOffPairs);
    double* cbuf = reinterpret_cast<double*>(base + kOffCterm);

    const int nn = node_hi - node_lo + 1;
    const size_t n = (size_t)3 * nn * c->D;
    NA_TRY(cudaMemsetAsync(d_G_I, 0, sizeof(double) * n, s));
    NA_TRY(cudaMemsetAsync(d_G_J, 0, sizeof(double) * n, s));
    NA_TRY(cudaMemsetAsync(d_H_I, 0, sizeof(double) * n, s));
    NA_TRY(cudaMemsetAsync(d_H_J, 0, sizeof(double) * n, s));
    AsmOut out{};
    out.G0 = d_G_I;
    out.H0 = d_H_I;
    out.G1 = d_G_J;
    out.H1 = d_H_J;
    out.D = c->D;
    out.ld = c->D;
    out.row_node_lo = node_lo;
    // The pair windows of tdbem_gh_driver, colour by colour in node chunks that fit
    // the fixed scratch, each followed by the uncompacted step kernel.
    for (size_t col = 0; col + 1 < c->color_start.size(); col++) {
        const int e0 = c->color_start[col], ne = c->color_start[col + 1] - e0;
        if (ne == 0) continue;
        const int* elems = c->d_color_elems + e0;
        const int chunk = (int)std::max<size_t>(1, max_pairs / (size_t)ne);
        for (int n0 = node_lo; n0 <= node_hi; n0 += chunk) {
            const int cn = std::min(chunk, node_hi - n0 + 1);
            const unsigned npairs = (unsigned)((size_t)cn * ne);
            NA_TRY(launch_pair_window(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, cn, c->ph,
                                      ASM_STEP, step, 1 << 30, step, SEL_ALL, pairs, nullptr, s,
                                      c->d_ebox));
            NA_TRY(launch_assemble_step_pairs(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, c->nq,
                                              c->d_gx, c->d_gw, c->d_geom, c->ph, step, pairs,
                                              npairs, out, s));
        }
    }
    if (step == 1) {
        for (int n0 = node_lo; n0 <= node_hi; n0 += max_nodes) {
            const int cn = std::min(max_nodes, node_hi - n0 + 1);
            NA_TRY(launch_cterm(c->d_coords, c->d_ien, c->ennd, c->nel, n0, cn, c->nq, c->d_gx, c->d_gw,
                                c->d_geom, c->ph, cbuf, s, false, nullptr, nullptr, c->d_ebox));
            AsmOut o2 = out;
            // rows of this chunk inside the caller's row block
            const size_t shift = (size_t)3 * (n0 - node_lo) * c->D;
            o2.H0 = d_H_I + shift;
            o2.H1 = d_H_J + shift;
            o2.row_node_lo = n0;
            NA_TRY(launch_cterm_apply(cbuf, n0, cn, c->dt, c->if_ext, ASM_STEP, o2, s));
        }
    }
    NA_TRY(cudaGetLastError());
    return TDBEM_OK;
}
