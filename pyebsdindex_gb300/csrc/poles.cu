// Band (theta, rho) -> unit plane normal on the device: the radon2pole epilogue
// (radon_fast.py:314-397, Krieger Lassen 1994 eq. 3.1.6), so that band normals can feed
// indexing without a host round trip.  float32 arithmetic in the reference's order; sin/cos
// are CUDA's (within an ulp or two of numpy's float32 functions).
#include "ebsd_internal.cuh"

namespace ebsd {
namespace {

// pattern-centre vector t (detector frame, origin at the bottom-left pixel) for one pattern
__device__ __forceinline__ void source_point(const float* pc, int vendor, float W, float H, float t[3]) {
    float x = pc[0], y = pc[1], z = pc[2];
    switch (vendor) {
        case EBSD_VENDOR_OXFORD:
            t[0] = __fmul_rn(x, W); t[1] = __fmul_rn(y, W); t[2] = __fmul_rn(z, -W);
            break;
        case EBSD_VENDOR_EMSOFT: {
            z = __fdiv_rn(z, pc[3]);  // normalise by the pixel size
            t[0] = __fadd_rn(-x, W * 0.5f);
            t[1] = __fadd_rn(y, H * 0.5f);
            t[2] = -z;
            break;
        }
        case EBSD_VENDOR_KIKUCHIPY:
        case EBSD_VENDOR_BRUKER:
            t[0] = __fmul_rn(x, W); t[1] = __fsub_rn(H, __fmul_rn(y, H)); t[2] = __fmul_rn(z, -H);
            break;
        default:  // EDAX
            t[0] = __fmul_rn(x, W); t[1] = __fmul_rn(y, H); t[2] = __fmul_rn(z, -fminf(W, H));
            break;
    }
}

__global__ void k_radon2pole(const float* __restrict__ theta, const float* __restrict__ rho, int64_t npat,
                             int nB, float W, float H, int vendor, const float* __restrict__ pc,
                             int pc_stride, float* __restrict__ normals) {
    const int64_t total = npat * nB;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
         o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = o / nB;
        float t[3];
        source_point(pc + (pc_stride > 0 ? q * pc_stride : 0), vendor, W, H, t);
        const float th = theta[o], r = rho[o];
        const float st = sinf(th), ct = cosf(th);
        // r_v = (-sin, cos, 0); p = rho (cos, sin) + centre; n = r_v x (p - t)
        const float a0 = -st, a1 = ct;
        const float b0 = __fsub_rn(__fadd_rn(__fmul_rn(r, ct), W * 0.5f), t[0]);
        const float b1 = __fsub_rn(__fadd_rn(__fmul_rn(r, st), H * 0.5f), t[1]);
        const float b2 = -t[2];
        const float n0 = __fsub_rn(__fmul_rn(a1, b2), 0.0f * b1);
        const float n1 = __fsub_rn(0.0f * b0, __fmul_rn(a0, b2));
        const float n2 = __fsub_rn(__fmul_rn(a0, b1), __fmul_rn(a1, b0));
        float nrm = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(n0, n0), __fmul_rn(n1, n1)), __fmul_rn(n2, n2)));
        nrm = fmaxf(nrm, 1e-12f);
        normals[3 * o + 0] = __fdiv_rn(n0, nrm);
        normals[3 * o + 1] = __fdiv_rn(n1, nrm);
        normals[3 * o + 2] = __fdiv_rn(n2, nrm);
    }
}

}  // namespace
}  // namespace ebsd

using namespace ebsd;

extern "C" int ebsd_radon2pole(const float* d_theta, const float* d_rho, int64_t npat, int32_t nBands,
                               int32_t H, int32_t W, int32_t vendor, const float* d_pc, int32_t pc_stride,
                               float* d_normals, void* stream) {
    if (npat < 0 || nBands <= 0 || H <= 0 || W <= 0 || pc_stride < 0) return EBSD_E_ARG;
    if (vendor < EBSD_VENDOR_EDAX || vendor > EBSD_VENDOR_BRUKER) return EBSD_E_ARG;
    if (npat == 0) return EBSD_OK;
    if (!d_theta || !d_rho || !d_pc || !d_normals) return EBSD_E_ARG;
    if (vendor == EBSD_VENDOR_EMSOFT ? (pc_stride != 0 && pc_stride < 4) : (pc_stride != 0 && pc_stride < 3))
        return EBSD_E_ARG;
    const int64_t total = npat * nBands;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
    k_radon2pole<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_theta, d_rho, npat, nBands, (float)W, (float)H,
                                                          vendor, d_pc, pc_stride, d_normals);
    return launch_status();
}
