// History convolution on the 5th-generation tensor cores (tcgen05), for the single
// and the batched mixed marches:
//     partial[split][c][row] = sum_f sum_mat A_mat^f[row,:] . W_mat[f][c]
// over nmat matrices per level (1: the merged level matrix of march_tc.cu; 2: a G
// and an H plane pair, W_1 holding -Wu, as k_conv_mma of batch.cu multiplies them),
// with both operands pre-split into BF16 planes (x = hi + lo, hi = bf16(x),
// lo = bf16(x - hi)) so that no conversion runs in the product kernel:
//   level planes  [(mat*2 + plane)*L  + f][row][ldb]
//   vector planes [(mat*2 + plane)*Lw + f][column][ldb]
// with ldb = D rounded up to 64 (zero-padded K).
//
// One CTA owns a 128-row tile of (<= 64) columns and an equal share of the tile's
// (level, matrix, 64-wide K chunk) iterations, taken in that order, so a share may
// start and end inside a level (every CTA of the grid streams the same number of
// level bytes, whatever the level count):
//   warp 0      TMA producer: per stage a 128 x 64 tile of the hi and lo level
//               planes and a 64 x 64 tile of the hi and lo vector planes
//               (128-byte swizzle), completion counted on an mbarrier;
//   warp 1      allocates 128 TMEM columns and issues tcgen05.mma
//               (kind::f16, BF16 x BF16 -> FP32, M = 128, N = 64, K = 16):
//               lo*hi + hi*lo + hi*hi per K step into the accumulator of the
//               current level; tcgen05.commit frees the stage / hands the
//               finished level (its part in this share) to the epilogue;
//   warps 2..5  epilogue: tcgen05.ld of a finished level's accumulator (double
//               buffered in TMEM, columns 0-63 / 64-127), compensated (Kahan)
//               FP32 sum over the levels, FP64 partial sums at the end.
// Every mbarrier wait is bounded (%globaltimer); a wait of the pipeline that runs
// out of its limit (a kernel argument, 2 s by default) sets an error code and
// makes every role stop; the CTA then still waits (2 s at most per wait) for its
// copies in flight and its MMAs before it frees TMEM.  err[1] counts the CTAs
// holding TMEM: +1 after the allocation, -1 after the release, so it returns to 0
// once every CTA has freed its columns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "tdbem_internal.cuh"

namespace tdbem {

namespace {

constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 64, TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;                      // 16 KiB
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;                      // 8 KiB
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;    // 48 KiB
constexpr int TC_THREADS = 192;
constexpr int TC_TMEM_COLS = 128;
constexpr int TC_NBAR = 2 * TC_STAGES + 5;  // full, empty, tmem full x2, tmem empty x2, done
constexpr int TC_SMEM = 1024 + TC_STAGES * TC_STAGE_BYTES + TC_NBAR * 8 + 16;
constexpr unsigned long long kDrainWaitNs = 2000000000ull;  // 2 s per drain wait

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            ((uint32_t)(TC_BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of `parity`: false when it runs out of limit_ns
// (error code recorded, every role told to stop) or when another role has stopped
// (honour_abort).
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                          int code, unsigned long long limit_ns, bool honour_abort = true) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    while (true) {
        if (honour_abort && *abort_flag) return false;
        if (mbar_try(bar, parity)) return true;
        if (gtimer() - t0 > limit_ns) {
            *abort_flag = 1;
            atomicExch(err, code);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset 16 B (unused for this
// layout), stride byte offset 1024 B between 8-row groups (bits 32-45),
// descriptor version 1 (bits 46-47), swizzle mode 128 B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) |
           ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::
                     "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Tile occupancy (optional, one matrix per level): occ[(slab * nrt + rt) * nk + kc] is
// zero where the 128-row x 64-column tile (row tile rt, K chunk kc) of level slab
// `slab` holds only zeros.  Such an iteration adds nothing to the product: every role
// skips it (the producer loads no stage, the MMA thread issues nothing, and a level
// whose tiles in the share are all zero hands no accumulator to the epilogue), each
// role evaluating the same predicate.
__device__ __forceinline__ bool tile_live(const unsigned char* __restrict__ occ, int slab,
                                          int nrt, int rt, int nk, int kc) {
    return !occ || occ[((size_t)slab * nrt + rt) * nk + kc] != 0;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              int D, int L, int Lw, int nlev, int nk, int nmat, int C,
              double* __restrict__ partial, int* __restrict__ err, unsigned long long wait_ns,
              int lev0, const unsigned char* __restrict__ occ, int nrt) {
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* base = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sbase = smem_u32(base);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + TC_STAGES * TC_STAGE_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + TC_NBAR);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    auto bar = [&](int i) { return smem_u32(bars + i); };
    const int FULL = 0, EMPTY = TC_STAGES, TFULL = 2 * TC_STAGES, TEMPTY = 2 * TC_STAGES + 2,
              DONE = 2 * TC_STAGES + 4;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * TC_BM;
    const int c0 = blockIdx.z * TC_BN;
    // this CTA's iterations [i0, i1) of nlev x nmat x nk; level f = i / per_lev
    const int per_lev = nmat * nk;
    const long long T = (long long)nlev * per_lev;
    const int i0 = (int)(T * blockIdx.y / gridDim.y), i1 = (int)(T * (blockIdx.y + 1) / gridDim.y);
    const int f0 = i0 / per_lev;
    const int nseg = i1 > i0 ? (i1 - 1) / per_lev - f0 + 1 : 0;  // levels touched
    // iteration i reads a nonzero tile (occupancy maps come with nmat == 1)
    auto live = [&](int i) {
        const int f = i / per_lev;
        return tile_live(occ, lev0 + f, nrt, blockIdx.x, nk, i - f * per_lev);
    };
    // level segment j of the share: iterations [ia, ib), and whether any is live
    auto seg_live = [&](int j, int& ia, int& ib) {
        const int f = f0 + j;
        ia = max(i0, f * per_lev);
        ib = min(i1, (f + 1) * per_lev);
        if (!occ) return ia < ib;
        for (int i = ia; i < ib; i++)
            if (live(i)) return true;
        return false;
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(bar(FULL + s), 1);
            mbar_init(bar(EMPTY + s), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(bar(TFULL + b), 1);
            mbar_init(bar(TEMPTY + b), 128);
        }
        mbar_init(bar(DONE), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    if (threadIdx.x == 0) atomicAdd(err + 1, 1);  // this CTA holds TMEM

    if (warp == 0) {
        if (lane == 0) {  // ---------------- TMA producer
            int it = 0;
            for (int i = i0; i < i1; i++) {
                if (!live(i)) continue;
                const int f = i / per_lev, r = i - f * per_lev;
                const int mat = r / nk, kc = r - mat * nk;
                const int s = it % TC_STAGES, n = it / TC_STAGES;
                if (n >= 1 && !mbar_wait(bar(EMPTY + s), (n - 1) & 1, abort_flag, err, 1, wait_ns))
                    break;
                const uint32_t st = sbase + s * TC_STAGE_BYTES;
                mbar_expect_tx(bar(FULL + s), TC_STAGE_BYTES);
                const int x = kc * TC_BK;
                tma_load_3d(st, &tmA, x, row0, (mat * 2 + 0) * L + lev0 + f, bar(FULL + s));
                tma_load_3d(st + TC_A_BYTES, &tmA, x, row0, (mat * 2 + 1) * L + lev0 + f,
                            bar(FULL + s));
                tma_load_3d(st + 2 * TC_A_BYTES, &tmB, x, c0, (mat * 2 + 0) * Lw + f,
                            bar(FULL + s));
                tma_load_3d(st + 2 * TC_A_BYTES + TC_B_BYTES, &tmB, x, c0, (mat * 2 + 1) * Lw + f,
                            bar(FULL + s));
                it++;  // issued (the drain below waits for exactly these)
            }
            // every issued copy has landed before the CTA can exit
            for (int k = std::max(0, it - TC_STAGES); k < it; k++)
                mbar_wait(bar(FULL + k % TC_STAGES), (k / TC_STAGES) & 1, abort_flag, err, 5,
                          kDrainWaitNs, false);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---------------- MMA issuer
            int it = 0, jj = 0;  // stages used, levels handed over
            bool ok = true;
            for (int j = 0; j < nseg && ok; j++) {
                int ia, ib;
                if (!seg_live(j, ia, ib)) continue;
                const int b = jj & 1, u = jj >> 1;
                jj++;
                if (u >= 1 && !mbar_wait(bar(TEMPTY + b), (u - 1) & 1, abort_flag, err, 2, wait_ns))
                    break;
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(b * TC_BN);
                uint32_t acc = 0;
                for (int i = ia; i < ib; i++) {
                    if (!live(i)) continue;
                    const int s = it % TC_STAGES, n = it / TC_STAGES;
                    if (!mbar_wait(bar(FULL + s), n & 1, abort_flag, err, 3, wait_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t ah = sbase + s * TC_STAGE_BYTES, al = ah + TC_A_BYTES;
                    const uint32_t bh = ah + 2 * TC_A_BYTES, bl = bh + TC_B_BYTES;
#pragma unroll
                    for (int kk = 0; kk < TC_BK / 16; kk++) {
                        const uint32_t o = kk * 32;  // 16 BF16 along K inside the swizzle atom
                        umma_bf16(d_tmem, sw128_desc(al + o), sw128_desc(bh + o), acc);
                        umma_bf16(d_tmem, sw128_desc(ah + o), sw128_desc(bl + o), 1);
                        umma_bf16(d_tmem, sw128_desc(ah + o), sw128_desc(bh + o), 1);
                        acc = 1;
                    }
                    umma_commit(bar(EMPTY + s));
                    it++;
                }
                if (ok) umma_commit(bar(TFULL + b));
            }
            // all MMAs of this thread complete before TMEM is released
            umma_commit(bar(DONE));
            mbar_wait(bar(DONE), 0, abort_flag, err, 6, kDrainWaitNs, false);
        }
    } else {  // ---------------- epilogue, warps 2..5 -> TMEM lanes 32 * (warp % 4)
        const int q = warp & 3;
        float sum[TC_BN], cmp[TC_BN];
#pragma unroll
        for (int i = 0; i < TC_BN; i++) sum[i] = cmp[i] = 0.f;
        int jj = 0;
        for (int j = 0; j < nseg; j++) {
            int ia, ib;
            if (!seg_live(j, ia, ib)) continue;
            const int b = jj & 1, u = jj >> 1;
            jj++;
            if (!mbar_wait(bar(TFULL + b), u & 1, abort_flag, err, 4, wait_ns)) break;
            tc_fence_after();
#pragma unroll
            for (int ch = 0; ch < TC_BN / 16; ch++) {
                float v[16];
                tmem_ld16(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * TC_BN + ch * 16),
                          v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int k = ch * 16 + i;
                    const float y = __fsub_rn(v[i], cmp[k]);
                    const float t = __fadd_rn(sum[k], y);
                    cmp[k] = __fsub_rn(__fsub_rn(t, sum[k]), y);
                    sum[k] = t;
                }
            }
            tc_fence_before();
            mbar_arrive(bar(TEMPTY + b));
        }
        const int row = row0 + q * 32 + lane;
        const int Cl = min(TC_BN, C - c0);
        if (row < D) {
#pragma unroll
            for (int k = 0; k < TC_BN; k++)
                if (k < Cl)
                    partial[((size_t)blockIdx.y * C + c0 + k) * D + row] =
                        (double)sum[k] - (double)cmp[k];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        if (lane == 0) atomicSub(err + 1, 1);  // released
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 3-D BF16 tensor [slabs][rows][ldb] with a 64 x box_rows x 1 box, 128-byte swizzle.
bool encode_map(void* map, void* gaddr, int ldb, int rows, int slabs, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)ldb, (cuuint64_t)rows, (cuuint64_t)slabs};
    const cuuint64_t strides[2] = {(cuuint64_t)ldb * 2, (cuuint64_t)rows * ldb * 2};
    const cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, gaddr, dims,
              strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

}  // namespace

static_assert(sizeof(CUtensorMap) == kTensorMapBytes, "tensor map size");

int tc_ldb(int D) { return (D + TC_BK - 1) / TC_BK * TC_BK; }
int tc_cases_pad(int C) { return (C + TC_BN - 1) / TC_BN * TC_BN; }

int tc_conv_splits(int nlev, int D, int C, int max_splits, int nmat) {
    // One CTA per SM (197 KB of shared memory each) and at least 16 iterations
    // (16 x 48 KB) per CTA so the pipeline's fill and drain stay small.  The split
    // count fills the waves best: tiles x splits CTAs in ceil(tiles x splits / 152)
    // waves of 152 (37 row tiles: 4 splits, 148 CTAs; 82: 11 splits, 902 CTAs in 6
    // waves), the smallest count within 3 % of the best fill.
    const int tiles = std::max(1, (D + TC_BM - 1) / TC_BM * ((C + TC_BN - 1) / TC_BN));
    const long long iters = (long long)nlev * nmat * (tc_ldb(D) / TC_BK);
    const long long smax =
        std::max<long long>(1, std::min<long long>({(long long)max_splits, iters / 16, 64}));
    auto fill = [&](long long s) {
        const long long ctas = tiles * s, waves = (ctas + 151) / 152;
        return (double)ctas / (double)(waves * 152);
    };
    double best = 0;
    for (long long s = 1; s <= smax; s++) best = std::max(best, fill(s));
    for (long long s = 1; s <= smax; s++)
        if (fill(s) >= best - 0.03) return (int)s;
    return 1;
}

bool make_tc_maps(void* planes, int D, int L, void* W, int C, int Lw, TcMaps* out, int nmat) {
    const int ldb = tc_ldb(D);
    return encode_map(out->a, planes, ldb, D, 2 * nmat * L, TC_BM) &&
           encode_map(out->b, W, ldb, tc_cases_pad(C), 2 * nmat * Lw, TC_BN);
}

cudaError_t launch_conv_tc(const TcMaps& maps, int D, int L, int Lw, int nlev, int C,
                           double* partial, int splits, int* d_err, cudaStream_t s, int nmat,
                           unsigned long long wait_ns, int lev0, const unsigned char* occ) {
    static unsigned long long attr_set = 0;  // devices with the shared-memory attribute set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!(attr_set & (1ull << dev))) {
        e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
        if (e != cudaSuccess) return e;
        attr_set |= 1ull << dev;
    }
    if (splits < 1 || nlev < 1 || lev0 < 0 || lev0 + nlev > L || nlev > Lw ||
        (nmat != 1 && nmat != 2) || wait_ns == 0 || (occ && nmat != 1))
        return cudaErrorInvalidValue;
    CUtensorMap ma, mb;
    std::memcpy(&ma, maps.a, sizeof(ma));
    std::memcpy(&mb, maps.b, sizeof(mb));
    dim3 grid((D + TC_BM - 1) / TC_BM, splits, (C + TC_BN - 1) / TC_BN);
    k_conv_tc<<<grid, TC_THREADS, TC_SMEM, s>>>(ma, mb, D, L, Lw, nlev, tc_ldb(D) / TC_BK, nmat,
                                                C, partial, d_err, wait_ns, lev0, occ,
                                                (D + TC_BM - 1) / TC_BM);
    return cudaGetLastError();
}

namespace {

// occ[(slab * nrt + rt) * nk + kc] = 1 where the hi plane's tile (rows rt*128..,
// columns kc*64..) of a slab in [slab_lo, slab_hi) holds a nonzero: warp per tile,
// 16-byte loads (a zero hi part means a zero lo part: hi = bf16(a) is zero only for
// |a| below half the smallest BF16 subnormal, and lo = bf16(a - hi) is then zero).
__global__ void __launch_bounds__(256) k_tile_occupancy(const __nv_bfloat16* __restrict__ hi,
                                                        int D, int ldb, int slab_lo,
                                                        int slab_hi, unsigned char* occ) {
    const int nrt = (D + TC_BM - 1) / TC_BM, nk = ldb / TC_BK;
    const long long tiles = (long long)(slab_hi - slab_lo) * nrt * nk;
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= tiles) return;
    const int kc = (int)(t % nk);
    const int rt = (int)((t / nk) % nrt);
    const int slab = slab_lo + (int)(t / ((long long)nk * nrt));
    unsigned any = 0;
    // 128 rows x 8 16-byte pieces: lane takes piece lane % 8 of rows lane / 8 + 4 q
    for (int q = 0; q < TC_BM / 4; q++) {
        const int r = rt * TC_BM + lane / 8 + 4 * q;
        if (r >= D) break;
        const uint4 v = __ldcs(reinterpret_cast<const uint4*>(
            hi + ((size_t)slab * D + r) * ldb + (size_t)kc * TC_BK) + (lane & 7));
        any |= v.x | v.y | v.z | v.w;
    }
    // BF16 -0 is 0x8000: not a nonzero value
    any &= 0x7fff7fffu;
    const unsigned w = __ballot_sync(0xffffffffu, any != 0);
    if (lane == 0) occ[((size_t)slab * nrt + rt) * nk + kc] = w != 0;
}

}  // namespace

size_t tc_occ_bytes(int D, int slabs) {
    return (size_t)slabs * ((D + TC_BM - 1) / TC_BM) * (tc_ldb(D) / TC_BK);
}

cudaError_t launch_tile_occupancy(const void* planes, int D, int slab_lo, int slab_hi,
                                  unsigned char* occ, cudaStream_t s) {
    const int ldb = tc_ldb(D);
    const long long tiles =
        (long long)(slab_hi - slab_lo) * ((D + TC_BM - 1) / TC_BM) * (ldb / TC_BK);
    if (tiles <= 0) return cudaSuccess;
    k_tile_occupancy<<<(unsigned)((tiles * 32 + 255) / 256), 256, 0, s>>>(
        static_cast<const __nv_bfloat16*>(planes), D, ldb, slab_lo, slab_hi, occ);
    return cudaGetLastError();
}

size_t tc_plane_bytes(int D, int L, int nmat) { return 2 * nmat * (size_t)L * D * tc_ldb(D) * 2; }
size_t tc_w_bytes(int D, int C, int Lw, int nmat) {
    return 2 * nmat * (size_t)Lw * tc_cases_pad(C) * tc_ldb(D) * 2;
}

}  // namespace tdbem
