// Fused persistent band-detection kernel (one launch per chunk).  Placeholder until the
// fused kernel lands: reports every plan as unsupported.
#include "ebsd_internal.cuh"

namespace ebsd {

int fused_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d) {
    (void)d;
    p->fg = FusedGeom{};
    return EBSD_OK;
}

void fused_release(ebsd_plan_s* p) { (void)p; }

int fused_supported(const ebsd_plan_s* p, int method) {
    (void)p;
    (void)method;
    return 0;
}

size_t fused_workspace_bytes(const ebsd_plan_s* p, int method, int64_t chunk) {
    (void)p;
    (void)method;
    (void)chunk;
    return 0;
}

int fused_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches) {
    (void)p; (void)method; (void)dtype; (void)d_pats; (void)n; (void)out; (void)out_offset; (void)st;
    (void)launches;
    return EBSD_E_UNSUPPORTED;
}

}  // namespace ebsd
