// C ABI of tdbem-gb300, level-store checkpoints (binary export / import) and
// the reference's WriteGH text file.
#include "capi_common.cuh"

using namespace tdbem;
using namespace tdbem::capi;

extern "C" {

// Level checkpoint: a 64-byte header (magic, version, D, M, precision, levels held,
// row stride) followed by the raw level store (FP64: G then H, (M+1) x D x D;
// mixed: FP32 G then H, (M+1) x D x ld, then FP64 levels 0-1 of G and H).
namespace {
constexpr char kCkptMagic[8] = {'T', 'D', 'B', 'E', 'M', 'L', 'V', 'L'};
struct CkptHeader {
    char magic[8];
    int32_t version, D, M, precision, levels_last, ld;
    int32_t pad[8];
};
static_assert(sizeof(CkptHeader) == 64, "checkpoint header is 64 bytes");

struct LevelArrays {
    void* dev[4];
    size_t bytes[4];
    int n;
};

LevelArrays level_arrays(tdbem_ctx* c) {
    LevelArrays a{};
    const size_t L = (size_t)c->M + 1, D = c->D;
    if (c->level_precision == TDBEM_FP64) {
        a.n = 2;
        a.dev[0] = c->d_G;
        a.dev[1] = c->d_H;
        a.bytes[0] = a.bytes[1] = L * D * D * 8;
    } else {
        a.n = 4;
        a.dev[0] = c->d_Gf;
        a.dev[1] = c->d_Hf;
        a.bytes[0] = a.bytes[1] = L * D * c->ldf * 4;
        a.dev[2] = c->d_G01;
        a.dev[3] = c->d_H01;
        a.bytes[2] = a.bytes[3] = 2 * D * D * 8;
    }
    return a;
}
}  // namespace

int tdbem_export_levels(tdbem_ctx* c, const char* path) {
    if (!c || !path) return fail(TDBEM_ERR_ARG, "null argument");
    if (c->level_precision < 0) return fail(TDBEM_ERR_STATE, "levels not assembled");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s for writing", path);
    CkptHeader h{};
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.D = c->D;
    h.M = c->M;
    h.precision = c->level_precision;
    h.levels_last = c->levels_last;
    h.ld = c->level_precision == TDBEM_FP64 ? c->D : c->ldf;
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    const LevelArrays a = level_arrays(c);
    std::vector<unsigned char> buf;
    const size_t chunk = (size_t)64 << 20;
    for (int k = 0; k < a.n && ok; k++)
        for (size_t o = 0; o < a.bytes[k] && ok; o += chunk) {
            const size_t b = std::min(chunk, a.bytes[k] - o);
            buf.resize(b);
            if (cudaMemcpy(buf.data(), static_cast<unsigned char*>(a.dev[k]) + o, b,
                           cudaMemcpyDeviceToHost) != cudaSuccess) {
                std::fclose(f);
                return fail(TDBEM_ERR_CUDA, "level copy to host failed");
            }
            ok = std::fwrite(buf.data(), 1, b, f) == b;
        }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(TDBEM_ERR_ARG, "write to %s failed", path);
    return TDBEM_OK;
}

int tdbem_import_levels(tdbem_ctx* c, const char* path) {
    if (!c || !path) return fail(TDBEM_ERR_ARG, "null argument");
    c->inv_valid = false;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s", path);
    CkptHeader h{};
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kCkptMagic, 8) != 0 ||
        h.version != 1) {
        std::fclose(f);
        return fail(TDBEM_ERR_ARG, "%s is not a level checkpoint", path);
    }
    if (h.D != c->D || h.M != c->M) {
        std::fclose(f);
        return fail(TDBEM_ERR_ARG, "checkpoint is for D=%d, M=%d; this mesh has D=%d, M=%d", h.D,
                    h.M, c->D, c->M);
    }
    int rc = TDBEM_OK;
    if (h.precision == TDBEM_FP64) {
        rc = ensure_fp64_store(c);
    } else if (h.precision == TDBEM_MIXED && h.ld == mixed_ld(c->D)) {
        if (c->level_precision != TDBEM_MIXED || !c->d_Gf) {
            free_levels(c);
            const size_t n = (size_t)(c->M + 1) * c->D * mixed_ld(c->D);
            cudaError_t e = dalloc(&c->d_Gf, n);
            if (e == cudaSuccess) e = dalloc(&c->d_Hf, n);
            if (e == cudaSuccess) e = dalloc(&c->d_G01, 2 * (size_t)c->D * c->D);
            if (e == cudaSuccess) e = dalloc(&c->d_H01, 2 * (size_t)c->D * c->D);
            if (e != cudaSuccess) rc = fail(TDBEM_ERR_NOMEM, "level allocation failed");
            c->ldf = mixed_ld(c->D);
            c->level_precision = TDBEM_MIXED;
        }
    } else {
        rc = fail(TDBEM_ERR_ARG, "checkpoint precision %d / row stride %d not supported",
                  h.precision, h.ld);
    }
    if (rc != TDBEM_OK) {
        std::fclose(f);
        return rc;
    }
    const LevelArrays a = level_arrays(c);
    std::vector<unsigned char> buf;
    const size_t chunk = (size_t)64 << 20;
    bool ok = true;
    for (int k = 0; k < a.n && ok; k++)
        for (size_t o = 0; o < a.bytes[k] && ok; o += chunk) {
            const size_t b = std::min(chunk, a.bytes[k] - o);
            buf.resize(b);
            ok = std::fread(buf.data(), 1, b, f) == b &&
                 cudaMemcpy(static_cast<unsigned char*>(a.dev[k]) + o, buf.data(), b,
                            cudaMemcpyHostToDevice) == cudaSuccess;
        }
    std::fclose(f);
    if (!ok) {
        free_levels(c);
        return fail(TDBEM_ERR_ARG, "%s is truncated or the copy failed", path);
    }
    c->levels_last = h.levels_last;
    c->mtc_planes_valid = false;
    c->step_inv_ready[0] = c->step_inv_ready[1] = false;
    return TDBEM_OK;
}

int tdbem_write_gh(const char* name_prefix, int step, int num_row, int num_column,
                   const double* data) {
    if (!name_prefix || !data || num_row < 0 || num_column < 0)
        return fail(TDBEM_ERR_ARG, "invalid arguments");
    char path[4096];
    std::snprintf(path, sizeof(path), "%s%d.txt", name_prefix, step);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(TDBEM_ERR_ARG, "cannot open %s", path);
    bool ok = true;
    for (int i = 0; i < num_row && ok; i++) {
        for (int j = 0; j < num_column && ok; j++)
            ok = std::fprintf(f, "%15.5e", data[(size_t)i * num_column + j]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TDBEM_OK : fail(TDBEM_ERR_ARG, "write to %s failed", path);
}

}  // extern "C"
