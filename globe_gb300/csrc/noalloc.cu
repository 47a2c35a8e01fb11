// noalloc.cu -- an entry point that allocates no device memory.
//
// globe_precond_apply_dev_noalloc applies the block preconditioner (the same
// kernels as globe_precond_apply) to device buffers and returns the per-column
// r'z.  The only scratch, the per-CTA r'z partials, lives in a file-scope
// __device__ array of fixed size.  Its address is looked up once per device
// (cudaGetSymbolAddress, with that device current) and cached.  Sizes that
// need more partials than the array holds are rejected before any launch.
#include <mutex>

#include "internal.cuh"

namespace globe {

constexpr size_t NOALLOC_PART_DOUBLES = (size_t)1 << 18;   // 2 MiB of r'z partials
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_part[NOALLOC_PART_DOUBLES];

static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[NOALLOC_MAX_DEVICES];

// address of the static scratch on ctx->device (the current device)
static int noalloc_scratch(globe_ctx* ctx, double** out) {
    if (ctx->device < 0 || ctx->device >= NOALLOC_MAX_DEVICES)
        return set_err(ctx, GLOBE_ERR_ARG, "device %d beyond the %d devices the static scratch table covers",
                       ctx->device, NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[ctx->device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
        if (e != cudaSuccess) return set_err(ctx, GLOBE_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_noalloc_ptr[ctx->device] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[ctx->device];
    return GLOBE_OK;
}

}  // namespace globe

using namespace globe;

extern "C" int globe_precond_apply_dev_noalloc(globe_ctx* ctx, const double* d_r, double* d_z, int k,
                                               double* d_rz) {
    if (!ctx || !d_r || !d_z || k < 1) return GLOBE_ERR_ARG;
    const cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return set_err(ctx, GLOBE_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    if (ctx->coh.Nrec < 1) return set_err(ctx, GLOBE_ERR_STATE, "no records loaded");
    if (!ctx->precond_ok)
        return set_err(ctx, GLOBE_ERR_STATE,
                       "preconditioner not built at the current components: call globe_precond_apply or globe_pcg "
                       "once first (building it allocates)");
    double* part = nullptr;
    GLOBE_RET(noalloc_scratch(ctx, &part));
    return precond_apply_scratch(ctx, static_cast<const double*>(ctx->ws[WS_H].p), d_r, d_z, k, part,
                                 NOALLOC_PART_DOUBLES, d_rz);
}
