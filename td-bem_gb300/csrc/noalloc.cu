// tdbem_gh_driver_noalloc: the single-step assembly of tdbem_gh_driver for
// callers that cannot allocate device memory.
//
// Some host applications own every byte of device memory: they reserve their
// pools when they start and forbid libraries to call cudaMalloc / cudaFree later
// (a serving process with a fixed memory budget, or a latency-critical loop where
// the implicit device synchronisation of cudaMalloc / cudaFree is not
// acceptable).  tdbem_gh_driver allocates a device staging buffer on every call;
// this variant writes into device buffers the caller already owns and keeps the
// per-call scratch of the kernels (pair windows, item counts and offsets, the
// scan's temporaries, the C term) in one fixed-size array in device memory that
// is part of the library image (kNoAllocScratchBytes; every GPU that loads the
// library holds it until the process exits).
//
// Every call shares that array and it keeps the last call's contents; each call
// overwrites what it reads (counts, offsets and the C term are recomputed,
// outputs are zeroed first), but calls whose work overlaps on the GPU (other
// streams, other host threads) race on it and must be serialised by the caller.
// The first call on a device looks up the array's device address with that
// device current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "tdbem_internal.cuh"

using namespace tdbem;

namespace {

constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB
constexpr size_t kMaxPairs = 1u << 18;             // pairs per launch chunk
constexpr size_t kMaxNodes = 1u << 14;             // collocation nodes per chunk (C term)
constexpr size_t kScanBytes = 64u << 10;           // scan temporaries
constexpr int kMaxDevices = 64;

// Layout: PairInfo[kMaxPairs] | counts[kMaxPairs] | offsets[kMaxPairs] |
//         C term[kMaxNodes * 9] | scan temporaries.
constexpr size_t kOffPairs = 0;
constexpr size_t kOffCounts = kOffPairs + kMaxPairs * sizeof(PairInfo);
constexpr size_t kOffOffsets = kOffCounts + kMaxPairs * sizeof(unsigned);
constexpr size_t kOffCterm = kOffOffsets + kMaxPairs * sizeof(unsigned);
constexpr size_t kOffScan = kOffCterm + kMaxNodes * 9 * sizeof(double);
static_assert(kOffScan + kScanBytes <= kNoAllocScratchBytes, "scratch layout exceeds the array");
static_assert(kOffCterm % 256 == 0 && kOffScan % 256 == 0, "scratch regions stay 256-byte aligned");

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

// Device address of the scratch array on the current device, looked up once per
// device with that device current.
int scratch_address(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) return nfail(TDBEM_ERR_UNSUPPORTED, "device %d", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev]) {
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
    if (scan_temp_bytes((unsigned)kMaxPairs) > kScanBytes)
        return nfail(TDBEM_ERR_UNSUPPORTED, "scan temporaries exceed the scratch reserve");
    unsigned char* base = nullptr;
    const int rc0 = scratch_address(dev, &base);
    if (rc0 != TDBEM_OK) return rc0;
    PairInfo* pairs = reinterpret_cast<PairInfo*>(base + kOffPairs);
    unsigned* counts = reinterpret_cast<unsigned*>(base + kOffCounts);
    unsigned* offsets = reinterpret_cast<unsigned*>(base + kOffOffsets);
    double* cbuf = reinterpret_cast<double*>(base + kOffCterm);
    void* scan_tmp = base + kOffScan;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;

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
    // Same window / scan / item sequence as tdbem_gh_driver, in node chunks that
    // fit the fixed scratch.
    for (size_t col = 0; col + 1 < c->color_start.size(); col++) {
        const int e0 = c->color_start[col], ne = c->color_start[col + 1] - e0;
        if (ne == 0) continue;
        const int* elems = c->d_color_elems + e0;
        const int chunk = (int)std::max<size_t>(1, kMaxPairs / (size_t)ne);
        for (int n0 = node_lo; n0 <= node_hi; n0 += chunk) {
            const int cn = std::min(chunk, node_hi - n0 + 1);
            const unsigned npairs = (unsigned)((size_t)cn * ne);
            NA_TRY(launch_pair_window(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, cn, c->ph, ASM_STEP,
                                      step, 1 << 30, step, SEL_ALL, pairs, counts, s));
            NA_TRY(exclusive_scan(counts, offsets, npairs, scan_tmp, kScanBytes, s));
            unsigned last[2];
            NA_TRY(cudaMemcpyAsync(&last[0], offsets + npairs - 1, sizeof(unsigned),
                                   cudaMemcpyDeviceToHost, s));
            NA_TRY(cudaMemcpyAsync(&last[1], counts + npairs - 1, sizeof(unsigned),
                                   cudaMemcpyDeviceToHost, s));
            NA_TRY(cudaStreamSynchronize(s));
            NA_TRY(launch_assemble_items(c->d_coords, c->d_ien, c->ennd, elems, ne, n0, c->nq,
                                         c->d_gx, c->d_gw, c->d_geom, c->ph, ASM_STEP, step,
                                         step, pairs, offsets, npairs, last[0] + last[1], out,
                                         s));
        }
    }
    if (step == 1) {
        for (int n0 = node_lo; n0 <= node_hi; n0 += (int)kMaxNodes) {
            const int cn = std::min((int)kMaxNodes, node_hi - n0 + 1);
            NA_TRY(launch_cterm(c->d_coords, c->d_ien, c->ennd, c->nel, n0, cn, c->nq, c->d_gx, c->d_gw,
                                c->d_geom, c->ph, cbuf, s));
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
