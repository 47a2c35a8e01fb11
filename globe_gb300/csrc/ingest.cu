// ingest.cu -- streaming PLINK .bed ingest.
//
// globe_load_bed_file reads <prefix>.bed in chunks of whole SNP rows into two
// pinned host buffers taken in turn.  Each chunk goes to the device with one
// 2-D asynchronous copy (file rows of ceil(N/4) bytes -> device rows of the
// padded stride) while the next chunk is read from the file, so file I/O and
// the host-to-device copy overlap and host memory stays at two chunks.  The
// rows then go through the same statistics, filter and compaction as
// globe_load_bed_dev (prepGenotypeInput, PCGsolver.cpp:615-763, which reads
// the whole file serially).  The tile-blocked layout is built after the file's
// device copy is released.
#include <cstdio>
#include <string>

#include "internal.cuh"

using namespace globe;

extern "C" int globe_load_bed_file(globe_ctx* ctx, const char* prefix, float min_maf, float max_miss,
                                   int64_t chunk_bytes, int64_t* alt_count, int64_t* miss_count, float* maf,
                                   float* miss_rate, uint8_t* keep, globe_bed_info* info) {
    if (!ctx || !prefix) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int32_t N = ctx->coh.N;
    if (N < 1) return set_err(ctx, GLOBE_ERR_STATE, "load the record table first (N comes from it)");
    if (chunk_bytes < 0) return set_err(ctx, GLOBE_ERR_ARG, "chunk_bytes must be >= 0");
    char err[512] = {0};
    int64_t M = 0;
    int rc = globe_bed_dims(prefix, N, &M, err, sizeof err);   // .bim lines, magic, size
    if (rc != GLOBE_OK) return set_err(ctx, rc, "%s", err);
    const int64_t bps = ((int64_t)N + 3) / 4;
    const int64_t stride = (bps + 15) / 16 * 16;
    const int64_t want = chunk_bytes > 0 ? chunk_bytes : ((int64_t)256 << 20);
    const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(M, want / bps));

    const std::string path = std::string(prefix) + ".bed";
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return set_err(ctx, GLOBE_ERR_IO, "Error opening .bed file: %s", path.c_str());
    uint8_t* d_bed = nullptr;
    int64_t* d_alt = nullptr;
    int64_t* d_miss = nullptr;
    float* d_maf = nullptr;
    float* d_mr = nullptr;
    uint8_t* d_keep = nullptr;
    uint8_t* host[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    if (std::fseek(f, 3, SEEK_SET) != 0) {
        rc = set_err(ctx, GLOBE_ERR_IO, "cannot seek in %s", path.c_str());
        goto done;
    }
    if ((rc = dalloc(ctx, &d_bed, (size_t)std::max<int64_t>(M, 1) * stride)) ||
        (rc = dalloc(ctx, &d_alt, (size_t)std::max<int64_t>(M, 1))) ||
        (rc = dalloc(ctx, &d_miss, (size_t)std::max<int64_t>(M, 1))) ||
        (rc = dalloc(ctx, &d_maf, (size_t)std::max<int64_t>(M, 1))) ||
        (rc = dalloc(ctx, &d_mr, (size_t)std::max<int64_t>(M, 1))) ||
        (rc = dalloc(ctx, &d_keep, (size_t)std::max<int64_t>(M, 1))))
        goto done;
    for (int b = 0; b < 2; ++b) {
        cudaError_t e = cudaHostAlloc((void**)&host[b], (size_t)(rows * bps), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
        if (e != cudaSuccess) {
            rc = cuda_err(ctx, e, "pinned chunk buffers");
            goto done;
        }
    }
    for (int64_t s0 = 0, ci = 0; s0 < M; s0 += rows, ++ci) {
        const int b = (int)(ci & 1);
        const int64_t r = std::min<int64_t>(rows, M - s0);
        if (used[b]) {   // the copy out of this buffer must have finished before it is refilled
            cudaError_t e = cudaEventSynchronize(ev[b]);
            if (e != cudaSuccess) {
                rc = cuda_err(ctx, e, "chunk copy");
                goto done;
            }
        }
        const size_t got = std::fread(host[b], 1, (size_t)(r * bps), f);
        if (got != (size_t)(r * bps)) {
            rc = set_err(ctx, GLOBE_ERR_FORMAT, "%s: short read at SNP %lld", path.c_str(), (long long)s0);
            goto done;
        }
        cudaError_t e = cudaMemcpy2DAsync(d_bed + s0 * stride, (size_t)stride, host[b], (size_t)bps, (size_t)bps,
                                          (size_t)r, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], ctx->stream);
        if (e != cudaSuccess) {
            rc = cuda_err(ctx, e, "chunk copy");
            goto done;
        }
        used[b] = true;
    }
    rc = load_bed_rows(ctx, d_bed, M, stride, min_maf, max_miss, d_alt, d_miss, d_maf, d_mr, d_keep, info);
    if (rc == GLOBE_OK && M > 0) {
        cudaError_t e = cudaSuccess;
        if (alt_count && e == cudaSuccess) e = cudaMemcpyAsync(alt_count, d_alt, 8 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (miss_count && e == cudaSuccess) e = cudaMemcpyAsync(miss_count, d_miss, 8 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (maf && e == cudaSuccess) e = cudaMemcpyAsync(maf, d_maf, 4 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (miss_rate && e == cudaSuccess) e = cudaMemcpyAsync(miss_rate, d_mr, 4 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (keep && e == cudaSuccess) e = cudaMemcpyAsync(keep, d_keep, M, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "copy SNP statistics");
    }
done:
    std::fclose(f);
    cudaStreamSynchronize(ctx->stream);
    for (int b = 0; b < 2; ++b) {
        if (ev[b]) cudaEventDestroy(ev[b]);
        if (host[b]) cudaFreeHost(host[b]);
    }
    for (void* p : {(void*)d_bed, (void*)d_alt, (void*)d_miss, (void*)d_maf, (void*)d_mr, (void*)d_keep}) dfree(ctx, p);
    // tile-blocked layout once the file's device copy is gone
    if (rc == GLOBE_OK && ctx->gen.Mk > 0) rc = ensure_blk1(ctx);
    return rc;
}
