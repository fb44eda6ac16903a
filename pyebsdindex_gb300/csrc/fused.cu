// Fused persistent band-detection kernel: one launch per chunk, one CTA per SM, each CTA
// looping over patterns.  Everything between the pattern bytes in HBM and the band fields
// in HBM stays in shared memory:
//
//   1. load      pattern -> FP32 tile (background subtracted as radon_fast.py:255-259 does)
//   2. radon     thread per ray, sequential FP32 sum over the ray's LUT entries in the
//                reference's order (rdn_loops, radon_fast.py:299-305), mean -> Radon tile
//                (stored FP32, or FP16 for EBSD_FUSED_F16)
//   3. pad       theta mirror with rho flip + rho edge rows + zero rows below the array
//                (band_detect.py:573-580; the FFT convolution's zero extension)
//   4. conv      register-blocked LoG convolution into an FP32 conv tile (separable: theta
//                taps per row, then rho taps), in the same multiply-add order as the per-stage
//                kernel; min/sum for normmax on the fly
//   5. peaks     separable max filter: theta max per row into the dead Radon tile, then
//                rho max per column in registers, exact equality + rdnmask
//                (band_detect.py:639-664); candidates go into a warp top-N list ordered
//                by (value desc, position asc)
//   6. merge     threshold = nB-th best warp-list head; rank the survivors among themselves
//   7. label     lanes 0..nB-1 of warp 0 fit their band (band_detect.py:691-809) and write
//                the record fields, normmax, theta and rho (band_detect.py:457-460, :521-524)
//
// Shared-memory footprint decides which plans the fused path takes (fused_supported()).
#include "ebsd_internal.cuh"
#include "label.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cfloat>
#include <cstring>

namespace ebsd {
namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kRowBlock = 8;
constexpr int kRing = 2;  // LUT chunks in flight per warp (deeper rings cost registers, not latency)
// packed modes: per CTA, per (pattern of the unit, band): the 3x3 conv block around the peak and
// its position; then per pattern the conv minimum and mean
constexpr int kCapBand = 10;
constexpr int kCapFloats = 8 * kMaxBands * kCapBand + 8 * 2;

struct FusedArgs {
    const void* pats;
    int64_t n;
    int H, W, nPx, pitch;      // pattern tile pitch (W + 1); zero word at H*pitch
    const uint4* lut;          // per-warp LUT streams: 8 u16 byte offsets per lane per chunk
    const uint4* lut8;         // the same for the 8-byte pixel elements of the 4-pattern tile
    const int32_t* count;      // [nRaysPad] entries per ray (group-major, lane-minor)
    const float* rcount;       // [nRaysPad] RN(1 / count) (0 for empty rays)
    const uint32_t* gstream;   // [nGroups] per-warp stream order: group id | chunks << 16
    const uint32_t* gtile;     // [nGroups] same order: Radon tile offset of lane 0 | rays << 16
    const int32_t* wofs;       // [2*(kWarps+1)]: per-warp first group index, first chunk
    const unsigned* padlist;   // [npad] (source tile cell << 16) | destination tile cell
    int npad;
    float* pack_scratch;       // packed modes: [gridDim.x][kPack-1][nRaysPad] parked ray means
    unsigned one;              // 1, as a runtime value: ray-sum adds become multiply-adds (below)
    float* cap;                // packed modes: [gridDim.x][kCapFloats] captured band fits (below)
    int nRays, nRaysPad, nGroups, gpt, nRho, nTheta;  // gpt: 32-ray groups per theta column
    int p0, p1, R, Tp;
    int row0, col0, TR, TC;    // Radon tile origin (padded frame) and extent
    int crow0, ccol0, CR, CC;  // conv tile origin and extent
    int statR1;                // end row of the statistics slice (padded frame)
    float taps[81];            // LoG taps [K0*K1] (parameter space: FMA operands, no loads)
    float ku[9], kw[9];        // separable factors: taps[a][b] = ku[a] * kw[b] (when sep)
    int sep;
    float ksum;                // sum of the kernel taps (FP16 centring correction)
    const float* wimg;         // [nPx] pixel weights whose dot product is the Radon mean
    const uint8_t* rdnmask;    // [nRho][nTheta]
    const uint32_t* rdnbits;   // [nTheta][rdnw] the same as bit columns
    int rdnw;
    int bg_mode;
    const double* bg;
    const float* bgf;
    LabelConsts kc;
    ebsd_bands out;
    int64_t out_offset;
};

template <typename S> __device__ __forceinline__ S to_store(float v);
template <> __device__ __forceinline__ float to_store<float>(float v) { return v; }
template <> __device__ __forceinline__ __half to_store<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }

// RN(s / c) for integers 0 <= s < 2^16 and 1 <= c <= 257, given r = RN(1 / c): one
// correction step of Markstein's division (P. Markstein, IBM J. Res. Dev. 34(1), 1990):
// q0 = RN(s r), the remainder s - q0 c is exact in one FMA, q = RN(q0 + rem r).  Checked
// exhaustively over that domain against the correctly rounded quotient.
__device__ __forceinline__ float div_int_exact(unsigned s, float c, float r) {
    const float fs = (float)s;
    const float q0 = __fmul_rn(fs, r);
    const float rem = __fmaf_rn(-q0, c, fs);
    return __fmaf_rn(rem, r, q0);
}

// L2 eviction-priority hints (createpolicy + cache_hint, sm_80+): the packed modes' parked
// ray means are written once and read once a few patterns later, so they are stored
// "evict last" and read back "evict first"; the streamed input patterns are loaded "evict
// first" (ld.global.cs), so that the parked rows rather than the input stay in L2.
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void st_keep(float* addr, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(addr), "f"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ float4 ld_once(const float* addr, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(addr), "l"(pol));
    return v;
}

// (hi, lo) += (bh, bl) for unevaluated float pairs: two-sum of the high parts (Knuth, TAOCP
// vol. 2, 4.2.2), the low parts added to the error term, then renormalised.
__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float bh, float bl) {
    const float s = __fadd_rn(hi, bh);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    const float e = __fadd_rn(err, __fadd_rn(lo, bl));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}

__device__ __forceinline__ bool beats(float v, int p, float w, int q) {
    return v > w || (v == w && p < q);
}

// Insert (v, pos) into a warp list ordered by (value desc, position asc).
__device__ __forceinline__ void list_insert(float v, int pos, float& lv, int& lp, int nB, int lane) {
    unsigned ahead = __ballot_sync(0xffffffffu, lane < nB && lp >= 0 && beats(lv, lp, v, pos));
    int ins = __popc(ahead);
    if (ins < nB) {
        float uv = __shfl_up_sync(0xffffffffu, lv, 1);
        int up = __shfl_up_sync(0xffffffffu, lp, 1);
        if (lane > ins && lane < nB) { lv = uv; lp = up; }
        if (lane == ins) { lv = v; lp = pos; }
    }
}

struct SmemConv {
    const float* c;
    int crow0, ccol0, CC;
    __device__ __forceinline__ float operator()(int r, int col) const {
        return c[(r - crow0) * CC + (col - ccol0)];
    }
};

template <typename InT>
__device__ __forceinline__ float load_pixel(const InT* p, int idx, int bg_mode, const double* bg, const float* bgf) {
    if (bg_mode == 1) return (float)((double)p[idx] - bg[idx]);
    if (bg_mode == 2) return __fsub_rn((float)p[idx], bgf[idx]);
    return (float)p[idx];
}

// The float64 epilogue of band_fit_write<float, false> for bands [0, nbands) of `out`:
// width from the stored log-curvature, theta/rho from the stored aveloc.
__global__ void __launch_bounds__(256) k_band_epilogue(ebsd_bands out, int64_t nbands, LabelConsts k) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nbands; o += (int64_t)gridDim.x * blockDim.x) {
        out.width[o] = band_width(out.width[o]);
        band_theta_rho(out.aveloc[2 * o], out.aveloc[2 * o + 1], k, out.theta + o, out.rho + o);
    }
}

// kPack = 2, 4 or 8: that many uint8 patterns per pass (no background).  Pattern pixels are
// packed -- as 16-bit lanes two per shared word (kPack 2) or four per 8-byte element
// (kPack 4), or as bytes eight per 8-byte element (kPack 8, spread to 16-bit lanes by byte
// permutes before the adds) -- so one shared load gathers a slot for all of them and one
// integer add accumulates two; a ray sum of at most 257 uint8 values fits a 16-bit lane, and
// integer sums are exact, so the means equal the float sequential sums of the single-pattern
// pass.  The other patterns' ray means are parked in a per-CTA global scratch
// (L2-resident) and reloaded once the pattern before them is finished.
// kNT > 0: nTheta fixed at compile time, so every tile pitch is a constant (0: runtime).
template <typename InT, typename S, int K0, int K1, int kPack, int kNT>
__global__ void __launch_bounds__(kThreads, 1) k_fused(FusedArgs a) {
    static_assert(kPack == 1 || sizeof(InT) == 1, "packed modes: uint8 input");
    static_assert(kPack == 1 || kPack == 2 || kPack == 4 || kPack == 8, "1, 2, 4 or 8 patterns per pass");
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int D0 = K0;  // rho half-window of the max filter (peakPad = 2*ksz + 1)
    constexpr int D1 = K1;  // theta half-window
    constexpr int WIN = 2 * D1 + 1;  // theta window of the max filter
    constexpr int H0 = K0 / 2, H1 = K1 / 2;
    constexpr int NV = kRowBlock + 2 * D0;  // theta-max rows a peak task reads

    constexpr bool kHalf = sizeof(S) == 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // geometry: conv tile = padded rows [p0 - D0, ..) x columns [p1 - D1, p1 + nTheta + D1),
    // Radon tile = the conv tile grown by the kernel half-widths (H0, H1) on each side
    const int nT = kNT > 0 ? kNT : a.nTheta;
    const int CC = kNT > 0 ? kNT + 2 * D1 : a.CC;
    const int TC = kNT > 0 ? kNT + 2 * D1 + 2 * H1 : a.TC;
    // row pitches of the conv tile, the Radon tile and the theta-max rows: odd, so that a warp
    // walking down a column touches 32 different banks
    const int CP = CC | 1, TP = TC | 1, MP = nT | 1;
    size_t off = 0;
    // the conv tile comes first so that the pattern tile aliased into it starts at shared
    // offset 0: the LUT then holds byte offsets usable directly as load addresses
    float* conv = (float*)(smem + off);
    float* pat = conv;  // aliased: the pattern tile is dead once the Radon is built
    off += ((size_t)(a.CR + 2 * H0) * (a.CC | 1) * sizeof(float) + 15) & ~(size_t)15;  // two-pass conv
    S* tile = (S*)(smem + off);
    {
        // the Radon tile region also holds the peaks' theta-max rows once the tile is dead
        const size_t tb = (size_t)a.TR * (a.TC | 1) * sizeof(S), mb = (size_t)(a.nRho + 2 * D0) * (a.nTheta | 1) * sizeof(float);
        off += ((tb > mb ? tb : mb) + 15) & ~(size_t)15;
    }
    float* lv_s = (float*)(smem + off);
    off += kWarps * kMaxBands * sizeof(float);
    int* lp_s = (int*)(smem + off);
    off += kWarps * kMaxBands * sizeof(int);
    double* red_d = (double*)(smem + off);
    off += 32 * sizeof(double);
    float* red_f = (float*)(smem + off);  // 66 floats
    off += 80 * sizeof(float);
    unsigned* gst_s = (unsigned*)(smem + off);  // nGroups: group id | chunks << 16, stream order
    off += (size_t)a.nGroups * sizeof(unsigned);
    unsigned* gtb_s = (unsigned*)(smem + off);  // nGroups: tile offset | valid rays << 16
    off += (size_t)a.nGroups * sizeof(unsigned);
    int* wofs_s = (int*)(smem + off);     // 2 * (kWarps + 1) ints: per-warp group / chunk offsets

    for (int i = tid; i < a.nGroups; i += kThreads) {
        gst_s[i] = a.gstream[i];
        gtb_s[i] = a.gtile[i];
    }
    for (int i = tid; i < 2 * (kWarps + 1); i += kThreads) wofs_s[i] = a.wofs[i];
    for (int i = tid; i < kWarps * kMaxBands; i += kThreads) lp_s[i] = -1;  // empty warp lists
    __syncthreads();
    const int nB = a.kc.nB;
    const int stat_r0 = a.p0, stat_r1 = a.statR1, stat_c0 = a.p1, stat_c1 = a.p1 + a.nTheta;
    const int stat_count = (stat_r1 - stat_r0) * (stat_c1 - stat_c0);

    const int64_t nunits = (a.n + kPack - 1) / kPack;
    float* scratch = kPack > 1 ? a.pack_scratch + (size_t)blockIdx.x * (kPack - 1) * a.nRaysPad : nullptr;
    for (int64_t u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int64_t q0 = u * kPack;
        const int npk = (int)(a.n - q0 < kPack ? a.n - q0 : kPack);  // patterns in this unit
        // ---- 1. load the pattern into the FP32 tile (pitch W+1, zero word after it) ----
        const InT* gp = (const InT*)a.pats + q0 * (int64_t)a.nPx;
        float wsum = 0.0f, pmin = -1.0f, pmax = -1.0f;  // -1: value of an empty ray
        for (int y = warp; y < a.H; y += kWarps) {
            for (int x = lane; x < a.W; x += 32) {
                const int i = y * a.W + x;
                float v;
                if (kPack == 2) {
                    const unsigned lo = (unsigned)gp[i], hi = npk > 1 ? (unsigned)gp[a.nPx + i] : 0u;
                    ((unsigned*)pat)[y * a.pitch + x] = lo | (hi << 16);
                    v = 0.0f;
                } else if (kPack == 8) {
                    // eight uint8 pixels in one 8-byte element, one byte per pattern
                    unsigned w[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) w[j] = j < npk ? (unsigned)__ldcs(gp + (size_t)j * a.nPx + i) : 0u;
                    ((uint2*)pat)[y * a.pitch + x] = make_uint2(w[0] | (w[1] << 8) | (w[2] << 16) | (w[3] << 24),
                                                                w[4] | (w[5] << 8) | (w[6] << 16) | (w[7] << 24));
                    v = 0.0f;
                } else if (kPack == 4) {
                    unsigned w[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) w[j] = j < npk ? (unsigned)__ldcs(gp + (size_t)j * a.nPx + i) : 0u;
                    ((uint2*)pat)[y * a.pitch + x] = make_uint2(w[0] | (w[1] << 16), w[2] | (w[3] << 16));
                    v = 0.0f;
                } else {
                    v = load_pixel<InT>(gp, i, a.bg_mode, a.bg, a.bgf);
                    pat[y * a.pitch + x] = v;
                }
                if (kHalf && kPack == 1) {
                    wsum = fmaf(a.wimg[i], v, wsum);
                    pmin = fminf(pmin, v);
                    pmax = fmaxf(pmax, v);
                }
            }
        }
        if (tid == 0) {
            if (kPack >= 4) ((uint2*)pat)[a.H * a.pitch] = make_uint2(0u, 0u);
            else pat[a.H * a.pitch] = 0.0f;
        }
        // FP16 storage keeps (value - m) * s: m = mean of the Radon interior (exact by
        // linearity: sum_px w[px] * p[px]), s = power of two keeping |value - m| * s < 2^14.
        // Pattern k of the unit keeps its m and s in red_f[64 + 2k], red_f[65 + 2k] (the conv
        // statistics use red_f[0..63] only).
        auto centre_scale = [&](float ws, float mn, float mx, int slot) {
            double dw = (double)ws;
            for (int o = 16; o > 0; o >>= 1) {
                dw += __shfl_down_sync(0xffffffffu, dw, o);
                mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
                mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
            }
            if (lane == 0) { red_d[warp] = dw; red_f[warp] = mn; red_f[32 + warp] = mx; }
            __syncthreads();
            if (warp == 0) {
                dw = red_d[lane];
                mn = red_f[lane];
                mx = red_f[32 + lane];
                for (int o = 16; o > 0; o >>= 1) {
                    dw += __shfl_down_sync(0xffffffffu, dw, o);
                    mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
                    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
                }
                if (lane == 0) {
                    float m = (float)dw;
                    float amax = fmaxf(fabsf(mx - m), fabsf(mn - m));
                    int e = 0;
                    frexpf(fmaxf(amax, 1e-30f), &e);  // amax < 2^e
                    red_f[64 + 2 * slot] = m;
                    red_f[65 + 2 * slot] = ldexpf(1.0f, 14 - e);
                }
            }
            __syncthreads();
        };
        float cen = 0.0f, scl = 1.0f, inv_scl = 1.0f;
        if (kHalf && kPack == 1) {
            centre_scale(wsum, pmin, pmax, 0);
        } else if (kHalf) {
            // packed units: each pattern's weighted sum, minimum and maximum from the packed
            // tile, with the thread-to-pixel order and multiply-adds of the one-pattern pass
            __syncthreads();
            for (int k = 0; k < npk; ++k) {
                float ws = 0.0f, mn = -1.0f, mx = -1.0f;
                for (int y = warp; y < a.H; y += kWarps) {
                    for (int x = lane; x < a.W; x += 32) {
                        unsigned b;
                        if (kPack == 8) {
                            const uint2 w = ((const uint2*)pat)[y * a.pitch + x];
                            b = ((k < 4 ? w.x : w.y) >> (8 * (k & 3))) & 0xFFu;
                        } else if (kPack == 4) {
                            const uint2 w = ((const uint2*)pat)[y * a.pitch + x];
                            b = ((k < 2 ? w.x : w.y) >> (16 * (k & 1))) & 0xFFFFu;
                        } else {
                            b = (((const unsigned*)pat)[y * a.pitch + x] >> (16 * k)) & 0xFFFFu;
                        }
                        const float v = (float)b;
                        ws = fmaf(a.wimg[y * a.W + x], v, ws);
                        mn = fminf(mn, v);
                        mx = fmaxf(mx, v);
                    }
                }
                centre_scale(ws, mn, mx, k);
            }
        } else {
            __syncthreads();
        }
        if (kHalf) {
            cen = red_f[64];
            scl = red_f[65];
            inv_scl = 1.0f / scl;  // exact: scl is a power of two
        }

        // ---- 2. Radon: one ray per lane ----
        // Each warp walks its own stream of LUT chunks: the chunks of its groups (32
        // neighbouring rho at one theta, one ray per lane) back to back, 16 B per lane per
        // chunk, groups balanced across warps on the host.  The next kRing chunks are kept in
        // flight in a register ring.  A chunk holds 8 byte offsets into the pattern tile;
        // short rays are padded with the zero word (adding +0.0 leaves a sum as it is).
        {
            const int g0 = wofs_s[warp], g1 = wofs_s[warp + 1];
            // each warp stream ends with kRing zero chunks, so the ring loads unconditionally
            const uint4* ip = (kPack >= 4 ? a.lut8 : a.lut) + ((size_t)wofs_s[kWarps + 1 + warp] * 32 + lane);
            const unsigned char* pb = (const unsigned char*)pat;
            uint4 ring[kRing];
#pragma unroll
            for (int k = 0; k < kRing; ++k) ring[k] = __ldg(ip + (size_t)k * 32);
            ip += (size_t)kRing * 32;
            int gi = g0, pc = 0;
            unsigned gs = gi < g1 ? gst_s[gi] : 0u;
            int t = (int)(gs & 0xFFFFu) * 32 + lane;  // ray slot: group * 32 + lane
            int cnt = gi < g1 ? __ldg(a.count + t) : 0;
            float rc = gi < g1 ? __ldg(a.rcount + t) : 0.0f;
            float sum = 0.0f;
            const uint64_t keep = kPack > 1 ? l2_evict_last_policy() : 0ull;
            // packed modes: 16-bit lane sums, two patterns per register.  The adds are written
            // as multiply-adds by a runtime 1, which run on the FMA pipe and leave the ALU pipe
            // (the gather's bottleneck) to the offset extraction and the byte permutes.
            unsigned isum = 0u, isum2 = 0u, isum3 = 0u, isum4 = 0u;
            const unsigned one = a.one;
            while (gi < g1) {
#pragma unroll
                for (int k = 0; k < kRing; ++k) {
                    if (gi < g1) {
                        const uint4 e = ring[k];
                        ring[k] = __ldg(ip);
                        ip += 32;
                        if (kPack == 8) {
                            const unsigned o[8] = {e.x & 0xFFFF, e.x >> 16, e.y & 0xFFFF, e.y >> 16,
                                                   e.z & 0xFFFF, e.z >> 16, e.w & 0xFFFF, e.w >> 16};
#pragma unroll
                            for (int k8 = 0; k8 < 8; ++k8) {
                                // spread the byte lanes to 16-bit lanes: (b0, b1) and (b2, b3)
                                const uint2 w = *(const uint2*)(pb + o[k8]);
                                isum = __byte_perm(w.x, 0u, 0x4140) * one + isum;
                                isum2 = __byte_perm(w.x, 0u, 0x4342) * one + isum2;
                                isum3 = __byte_perm(w.y, 0u, 0x4140) * one + isum3;
                                isum4 = __byte_perm(w.y, 0u, 0x4342) * one + isum4;
                            }
                        } else if (kPack == 4) {
                            const unsigned o[8] = {e.x & 0xFFFF, e.x >> 16, e.y & 0xFFFF, e.y >> 16,
                                                   e.z & 0xFFFF, e.z >> 16, e.w & 0xFFFF, e.w >> 16};
#pragma unroll
                            for (int k8 = 0; k8 < 8; ++k8) {
                                const uint2 w = *(const uint2*)(pb + o[k8]);
                                isum = w.x * one + isum;
                                isum2 = w.y * one + isum2;
                            }
                        } else if (kPack == 2) {
                            isum += *(const unsigned*)(pb + (e.x & 0xFFFF));
                            isum += *(const unsigned*)(pb + (e.x >> 16));
                            isum += *(const unsigned*)(pb + (e.y & 0xFFFF));
                            isum += *(const unsigned*)(pb + (e.y >> 16));
                            isum += *(const unsigned*)(pb + (e.z & 0xFFFF));
                            isum += *(const unsigned*)(pb + (e.z >> 16));
                            isum += *(const unsigned*)(pb + (e.w & 0xFFFF));
                            isum += *(const unsigned*)(pb + (e.w >> 16));
                        } else {
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.x & 0xFFFF)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.x >> 16)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.y & 0xFFFF)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.y >> 16)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.z & 0xFFFF)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.z >> 16)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.w & 0xFFFF)));
                            sum = __fadd_rn(sum, *(const float*)(pb + (e.w >> 16)));
                        }
                        if (++pc == (int)(gs >> 16)) {
                            // ray ends: the mean of an empty ray is -1 (radon_fast.py:265)
                            float v;
                            if (kPack > 1) {
                                const float fc = (float)cnt;
                                v = cnt > 0 ? div_int_exact(isum & 0xFFFFu, fc, rc) : -1.0f;
                                if (kHalf) v = (v - cen) * scl;
                                st_keep(scratch + t, cnt > 0 ? div_int_exact(isum >> 16, fc, rc) : -1.0f, keep);
                                if (kPack >= 4) {
                                    st_keep(scratch + a.nRaysPad + t, cnt > 0 ? div_int_exact(isum2 & 0xFFFFu, fc, rc) : -1.0f, keep);
                                    st_keep(scratch + 2 * a.nRaysPad + t, cnt > 0 ? div_int_exact(isum2 >> 16, fc, rc) : -1.0f, keep);
                                }
                                if (kPack == 8) {
                                    st_keep(scratch + 3 * a.nRaysPad + t, cnt > 0 ? div_int_exact(isum3 & 0xFFFFu, fc, rc) : -1.0f, keep);
                                    st_keep(scratch + 4 * a.nRaysPad + t, cnt > 0 ? div_int_exact(isum3 >> 16, fc, rc) : -1.0f, keep);
                                    st_keep(scratch + 5 * a.nRaysPad + t, cnt > 0 ? div_int_exact(isum4 & 0xFFFFu, fc, rc) : -1.0f, keep);
                                    st_keep(scratch + 6 * a.nRaysPad + t, cnt > 0 ? div_int_exact(isum4 >> 16, fc, rc) : -1.0f, keep);
                                }
                            } else {
                                v = cnt > 0 ? __fdiv_rn(sum, (float)cnt) : -1.0f;
                                if (kHalf) v = (v - cen) * scl;
                            }
                            const unsigned tb = gtb_s[gi];
                            if (lane < (int)(tb >> 16)) tile[(tb & 0xFFFFu) + lane * TP] = to_store<S>(v);
                            ++gi;
                            pc = 0;
                            sum = 0.0f;
                            isum = 0u;
                            isum2 = 0u;
                            isum3 = 0u;
                            isum4 = 0u;
                            if (gi < g1) {
                                gs = gst_s[gi];
                                t = (int)(gs & 0xFFFFu) * 32 + lane;
                                cnt = __ldg(a.count + t);
                                rc = __ldg(a.rcount + t);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();

        // ---- 6. merge + 7. label (warp 0), for pattern qq: a k-way merge of the sorted
        //      warp lists -- lane l holds the head of warp l's list; each round the best head
        //      under (value desc, position asc), a strict total order on which every lane of
        //      the xor butterfly agrees, goes to lane k and its list advances -- then lanes
        //      0..nB-1 fit their band (band_detect.py:691-809).  Reads the warp lists, the conv
        //      tile and the conv statistics of qq only.
        // k-way merge of the sorted warp lists by warp 0: lane l holds the head of warp l's list;
        // each round the best head under (value desc, position asc) -- a strict total order --
        // is found with two warp reductions (largest value key, then smallest position among
        // the heads holding it), goes to lane k, and its list advances.  Returns, in lanes
        // 0..nB-1, the position of band `lane` (-1: none).  -0 is folded into +0 first, as the
        // value comparison of the reference's sort treats them alike.
        auto tournament = [&]() -> int {
            int ptr = 0;
            float hv = lane < kWarps ? lv_s[lane * kMaxBands] : -INFINITY;
            int hp = lane < kWarps ? lp_s[lane * kMaxBands] : -1;
            int mypos = -1;
            for (int k = 0; k < nB; ++k) {
                const unsigned u = __float_as_uint(hv + 0.0f);
                const unsigned key = hp < 0 ? 0u : ((u & 0x80000000u) ? ~u : (u | 0x80000000u));
                const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
                if (kmax == 0u) break;  // every list is exhausted
                const unsigned pmin = __reduce_min_sync(0xffffffffu, key == kmax ? (unsigned)hp : 0xffffffffu);
                const unsigned win = __ballot_sync(0xffffffffu, key == kmax && (unsigned)hp == pmin);
                if (lane == k) mypos = (int)pmin;
                if (lane == __ffs(win) - 1) {
                    ++ptr;
                    hp = ptr < nB ? lp_s[lane * kMaxBands + ptr] : -1;
                    hv = ptr < nB ? lv_s[lane * kMaxBands + ptr] : -INFINITY;
                }
            }
            return mypos;
        };
        // ---- 6. merge + 7. label (warp 0), one pattern per pass: the band fit
        //      (band_detect.py:691-809) straight from the conv tile
        auto merge_label = [&](int64_t qq) {
            const int mypos = tournament();
            if (lane < nB) {
                const bool has = mypos >= 0;
                int r = 0, c = 0;
                if (has) {
                    const int i = mypos / nT;
                    r = i + a.p0;
                    c = (mypos - i * nT) + a.p1;
                }
                const float mn = red_f[0];
                const float mean = (float)(red_d[0] / (double)stat_count);
                SmemConv acc{conv, a.p0 - D0, a.p1 - D1, CP};
                band_fit_write<float, false>(has, r, c, acc, mn, mean, a.kc, a.out, (a.out_offset + qq) * nB + lane);
            }
        };
        // ---- 6. merge (warp 0), packed modes: the bands' 3x3 blocks, positions and the conv
        //      statistics of pattern `sb` of the unit go to the CTA's capture scratch; the fits
        //      run for the whole unit at once after its last pattern (label_unit)
        float* cap = kPack > 1 ? a.cap + (size_t)blockIdx.x * kCapFloats : nullptr;
        auto merge_capture = [&](int sb) {
            const int mypos = tournament();
            if (lane < nB) {
                float* cb = cap + (sb * nB + lane) * kCapBand;
                if (mypos >= 0) {
                    const int i = mypos / nT, j = mypos - (mypos / nT) * nT;
                    const float* c0 = conv + (i + D0 - 1) * CP + (j + D1 - 1);
#pragma unroll
                    for (int r3 = 0; r3 < 3; ++r3)
#pragma unroll
                        for (int c3 = 0; c3 < 3; ++c3) cb[r3 * 3 + c3] = c0[r3 * CP + c3];
                }
                cb[9] = __int_as_float(mypos);
            }
            if (lane == 0) {
                cap[8 * kMaxBands * kCapBand + 2 * sb] = red_f[0];
                cap[8 * kMaxBands * kCapBand + 2 * sb + 1] = (float)(red_d[0] / (double)stat_count);
            }
        };
        // ---- 7. label, packed modes: every band of the unit, one thread each
        auto label_unit = [&](int npat) {
            for (int t = tid; t < npat * nB; t += kThreads) {
                const int sb = t / nB, b = t - (t / nB) * nB;
                const float* cb = cap + (sb * nB + b) * kCapBand;
                const int pos = __float_as_int(cb[9]);
                const bool has = pos >= 0;
                float nn[9];
#pragma unroll
                for (int k9 = 0; k9 < 9; ++k9) nn[k9] = has ? cb[k9] : 0.0f;
                int r = 0, c = 0;
                if (has) {
                    const int i = pos / nT;
                    r = i + a.p0;
                    c = (pos - i * nT) + a.p1;
                }
                const float mn = cap[8 * kMaxBands * kCapBand + 2 * sb];
                const float mean = cap[8 * kMaxBands * kCapBand + 2 * sb + 1];
                band_fit_block<float, false>(has, r, c, nn, mn, mean, a.kc, a.out, (a.out_offset + q0 + sb) * nB + b);
            }
        };

        // the padding cells of the Radon tile from the plan's cell list (sources are interior
        // cells only, so the copies are independent): four list entries in flight per thread
        auto pad_cells = [&](int first, int stride, S zero) {
            for (int k = first; k < a.npad; k += 4 * stride) {
                unsigned e[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) e[u] = k + u * stride < a.npad ? __ldg(a.padlist + k + u * stride) : 0xFFFFFFFFu;
                S v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = (e[u] >> 16) == 0xFFFFu ? zero : tile[e[u] >> 16];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (k + u * stride < a.npad) tile[e[u] & 0xFFFF] = v[u];
            }
        };

        for (int sub = 0; sub < npk; ++sub) {
        const int64_t q = q0 + sub;
        if (kHalf && kPack > 1 && sub > 0) {  // this pattern's FP16 centre and scale
            cen = red_f[64 + 2 * sub];
            scl = red_f[65 + 2 * sub];
            inv_scl = 1.0f / scl;
        }
        // ---- 3. pad the tile around the interior ----
        // padding cell list (plan table): low half = destination tile cell, high half = source
        // tile cell, 0xFFFF = zero (rows below the padded array, the convolution's zero fill).
        // After the first pattern of a packed unit, warp 0 merges and labels the previous
        // pattern while warps 1.. reload this pattern's parked ray means and pad the tile.
        if (kPack > 1 && sub > 0) {
            if (warp == 0) {
                merge_capture(sub - 1);
            } else {
                // parked ray means back into the tile: eight threads per 32-ray group, each
                // moving four neighbouring rays with one 16-byte load (the scratch row is mostly
                // outside L2, so bytes in flight set the pace); four groups in flight per thread
                const float* src = scratch + (size_t)(sub - 1) * a.nRaysPad;
                const uint64_t once = l2_evict_first_policy();
                constexpr int kRel = kThreads - 32;
                const int ntask = a.nGroups * 8;
                for (int it = tid - 32; it < ntask; it += 4 * kRel) {
                    float4 v[4];
                    unsigned tb[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int task = it + u * kRel;
                        const int gi = task >> 3;
                        tb[u] = task < ntask ? gtb_s[gi] : 0u;
                        v[u] = task < ntask ? ld_once(src + (gst_s[gi] & 0xFFFFu) * 32 + (task & 7) * 4, once)
                                            : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int j4 = ((it + u * kRel) & 7) * 4;
                        const int nval = (int)(tb[u] >> 16);
                        S* dst = tile + (tb[u] & 0xFFFFu) + j4 * TP;
                        if (kHalf) {
                            v[u].x = (v[u].x - cen) * scl;
                            v[u].y = (v[u].y - cen) * scl;
                            v[u].z = (v[u].z - cen) * scl;
                            v[u].w = (v[u].w - cen) * scl;
                        }
                        if (j4 + 0 < nval) dst[0] = to_store<S>(v[u].x);
                        if (j4 + 1 < nval) dst[TP] = to_store<S>(v[u].y);
                        if (j4 + 2 < nval) dst[2 * TP] = to_store<S>(v[u].z);
                        if (j4 + 3 < nval) dst[3 * TP] = to_store<S>(v[u].w);
                    }
                }
                asm volatile("bar.sync 1, %0;" ::"r"(kThreads - 32) : "memory");  // warps 1.. only
                pad_cells(tid - 32, kThreads - 32, to_store<S>(kHalf ? -cen * scl : 0.0f));
            }
        } else {
            pad_cells(tid, kThreads, to_store<S>(kHalf ? -cen * scl : 0.0f));
        }
        __syncthreads();

        // the parked ray means of the next pattern of this unit are read back in the next pass;
        // start moving them into L2 now (the scratch does not stay in L2 between the gather and
        // the last patterns of a unit)
        if (kPack > 1 && tid == 0 && sub + 1 < npk) {
            const float* nxt = scratch + (size_t)sub * a.nRaysPad;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt), "r"(a.nRaysPad * 4) : "memory");
        }

        // ---- 4. LoG convolution: conv[cr][cc] = sum_a sum_b tap[a][b] tile[cr+2H0-a][cc+2H1-b]
        //      with the statistics slice's min and sum on the fly (padded rows [stat_r0,
        //      stat_r1) x columns [stat_c0, stat_c1), i.e. conv rows from D0 and conv columns
        //      [D1, D1 + nTheta)).
        float smin = INFINITY, ssum = 0.0f;
        const unsigned stat_rows = (unsigned)(stat_r1 - stat_r0);
        if (a.sep) {
            // Separable taps (the reference's LoG is a Gaussian second derivative along rho
            // times a Gaussian along theta), in two passes through the conv region, which holds
            // TR rows: (a) theta taps along every Radon tile row, h[r][cc] = sum_b kw[b]
            // tile[r][cc + 2H1 - b] (ascending b), 16 outputs per thread from a sliding row of
            // 16 + K1 - 1 loads, lanes on neighbouring rows; (b) rho taps down each column,
            // conv[cr][cc] = sum_a ku[a] h[cr + 2H0 - a][cc] (ascending a), in place: each
            // thread walks a strip of rows of one column with a register window of K0 h rows
            // and writes each output over its own h row as soon as it is computed (later
            // outputs of the strip read only later rows).  The strip above reads this strip's
            // first 2H0 h rows, so those outputs are held in registers and written after a
            // barrier.  The multiply-add order is the per-stage FP32 kernel's.
            constexpr int kSegA = 16;
            const int TR = a.CR + 2 * H0;
            {
                const int nseg = (CC + kSegA - 1) / kSegA;
                for (int task = tid; task < TR * nseg; task += kThreads) {
                    const int sg = task / TR, r = task - sg * TR;
                    const int c0 = sg * kSegA < CC - kSegA ? sg * kSegA : CC - kSegA;
                    const S* trow = tile + r * TP + c0;
                    float x[kSegA + K1 - 1];
#pragma unroll
                    for (int k = 0; k < kSegA + K1 - 1; ++k) x[k] = to_f(trow[k]);
                    float* hrow = conv + r * CP + c0;
#pragma unroll
                    for (int j = 0; j < kSegA; ++j) {
                        float hv = 0.0f;
#pragma unroll
                        for (int b = 0; b < K1; ++b) hv = fmaf(a.kw[b], x[j + 2 * H1 - b], hv);
                        hrow[j] = hv;
                    }
                }
            }
            __syncthreads();
            {
                const int CR = a.CR;
                // strips per column: as many as fit one task per thread (at least 8 rows each)
                const int nstrip = CC >= kThreads ? 1 : (kThreads / CC < (CR + 7) / 8 ? kThreads / CC : (CR + 7) / 8);
                const int L = (CR + nstrip - 1) / nstrip;
                const int ntask = nstrip * CC;
                // more than one round only with one strip per column (no strip boundaries)
                const int rounds = (ntask + kThreads - 1) / kThreads;
                for (int rd = 0; rd < rounds; ++rd) {
                    const int task = rd * kThreads + tid;
                    const int st = task < ntask ? task / CC : 0, cc = task < ntask ? task - st * CC : 0;
                    const int o0 = st * L, o1 = task < ntask ? (o0 + L < CR ? o0 + L : CR) : 0;
                    float* hcol = conv + cc;
                    const bool colstat = (unsigned)(cc - D1) < (unsigned)nT;
                    float w[K0], held[K0 - 1];
#pragma unroll
                    for (int k = 0; k < K0 - 1; ++k) {
                        w[k] = o0 < o1 ? hcol[(o0 + k) * CP] : 0.0f;
                        held[k] = 0.0f;
                    }
                    // window slot of h row (o0 + m): m mod K0; K0 outputs per step keep every
                    // slot index a constant
                    for (int o = o0; o < o1; o += K0) {
#pragma unroll
                        for (int j = 0; j < K0; ++j) {
                            const int oj = o + j;
                            if (oj < o1) {
                                w[(j + K0 - 1) % K0] = hcol[(oj + K0 - 1) * CP];
                                float acc = 0.0f;
#pragma unroll
                                for (int ka = 0; ka < K0; ++ka) acc = fmaf(a.ku[ka], w[(j + K0 - 1 - ka) % K0], acc);
                                if (kHalf) acc = fmaf(a.ksum, cen, acc * inv_scl);
                                if (j < K0 - 1 && o == o0) held[j < K0 - 1 ? j : 0] = acc;
                                else hcol[oj * CP] = acc;
                                if (colstat && (unsigned)(oj - D0) < stat_rows) {
                                    smin = fminf(smin, acc);
                                    ssum += acc;
                                }
                            }
                        }
                    }
                    __syncthreads();
#pragma unroll
                    for (int k = 0; k < K0 - 1; ++k)
                        if (o0 + k < o1) hcol[(o0 + k) * CP] = held[k];
                }
            }
        } else {
            // 2-D taps: kRowBlock outputs per thread down one column.  The last row block is
            // moved up to end at CR, so no load leaves the tile; rows it shares with the block
            // above are neither stored again nor counted twice.
            const int CR = a.CR;
            const int nrb = (CR + kRowBlock - 1) / kRowBlock;
            const int ntask = nrb * CC;
            // task = rb * CC + cc, advanced by kThreads without a division per task
            int cc = tid % CC, rb = tid / CC;
            const int dcc = kThreads % CC, drb = kThreads / CC;
            for (int task = tid; task < ntask; task += kThreads) {
                const int cr_first = rb * kRowBlock;
                const int cr0 = cr_first < CR - kRowBlock ? cr_first : CR - kRowBlock;
                float acc[kRowBlock];
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) acc[o] = 0.0f;
                // tile row (cr0 + t) feeds output o through kernel row a = o + 2*H0 - t;
                // descending t keeps each output's multiply-add order = ascending a.
                const S* tcol = tile + cr0 * TP + cc + 2 * H1;
#pragma unroll
                for (int t = kRowBlock + 2 * H0 - 1; t >= 0; --t) {
                    float v[K1];
#pragma unroll
                    for (int b = 0; b < K1; ++b) v[b] = to_f(tcol[t * TP - b]);
#pragma unroll
                    for (int o = 0; o < kRowBlock; ++o) {
                        const int ka = o + 2 * H0 - t;
                        if (ka >= 0 && ka < K0) {
#pragma unroll
                            for (int b = 0; b < K1; ++b) acc[o] = fmaf(a.taps[ka * K1 + b], v[b], acc[o]);
                        }
                    }
                }
                const bool colstat = (unsigned)(cc - D1) < (unsigned)nT;
                float* ccol = conv + cr0 * CP + cc;
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) {
                    if (kHalf) acc[o] = fmaf(a.ksum, cen, acc[o] * inv_scl);
                    if (cr0 + o >= cr_first) {
                        ccol[o * CP] = acc[o];
                        if (colstat && (unsigned)(cr0 + o - D0) < stat_rows) {
                            smin = fminf(smin, acc[o]);
                            ssum += acc[o];
                        }
                    }
                }
                cc += dcc;
                rb += drb;
                if (cc >= CC) {
                    cc -= CC;
                    ++rb;
                }
            }
        }
        // block reduction of min / sum: the per-thread float sums are combined as unevaluated
        // float pairs (Knuth's two-sum, exact to about 2^-48), which keeps the slow float64
        // pipe out of the 32-warp reduction; warp 0 turns the pair into a double at the end
        {
            float hi = ssum, lo = 0.0f;
            float m = smin;
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, hi, o);
                const float ol = __shfl_down_sync(0xffffffffu, lo, o);
                two_sum_add(hi, lo, oh, ol);
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            if (lane == 0) { red_f[warp] = m; red_f[32 + warp] = hi; red_d[warp] = (double)lo; }
        }
        __syncthreads();
        if (warp == 0) {
            float hi = red_f[32 + lane], lo = (float)red_d[lane];
            float m = red_f[lane];
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, hi, o);
                const float ol = __shfl_down_sync(0xffffffffu, lo, o);
                two_sum_add(hi, lo, oh, ol);
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            if (lane == 0) { red_d[0] = (double)hi + (double)lo; red_f[0] = m; }
        }
        // (red_d[0] / red_f[0] are read after the next barrier)

        // ---- 5. peaks: separable max filter (band_detect.py:639-664, :811-843) ----
        // 5a. theta max of every conv row the rho window needs, into the dead Radon tile:
        //     tm[rr][j] = max(conv[rr][j .. j + 2*D1]) for rr < nRho + 2*D0, j < nTheta (conv
        //     row rr = padded row p0 - D0 + rr, conv column j = padded column p1 + j - D1).
        //     One thread per WIN consecutive outputs: suffix maxima of the first WIN inputs and
        //     running prefix maxima of the next WIN - 1 give every window with two max
        //     operations.  The last segment is moved left to end at nTheta (its overlap is
        //     written twice with the same values).
        float* tm = (float*)tile;
        {
            const int NR = a.nRho + 2 * D0;
            constexpr int kSeg = (kNT + WIN - 1) / WIN;  // segments per row when nTheta is fixed
            const int nseg = kNT > 0 ? kSeg : (nT + WIN - 1) / WIN;
            for (int task = tid; task < NR * nseg; task += kThreads) {
                // neighbouring lanes take neighbouring rows (odd pitches: no bank conflicts)
                const int sg = task / NR, rr = task - sg * NR;
                const int j0 = sg * WIN < nT - WIN ? sg * WIN : nT - WIN;
                const float* x = conv + rr * CP + j0;
                float* out = tm + rr * MP + j0;
                float xv[2 * WIN - 1];
#pragma unroll
                for (int k = 0; k < 2 * WIN - 1; ++k) xv[k] = x[k];
#pragma unroll
                for (int k = WIN - 2; k >= 0; --k) xv[k] = fmaxf(xv[k], xv[k + 1]);  // suffix maxima
                float pm = -INFINITY;
#pragma unroll
                for (int t = 0; t < WIN; ++t) {
                    if (t > 0) pm = fmaxf(pm, xv[WIN - 1 + t]);
                    out[t] = fmaxf(xv[t], pm);
                }
            }
        }
        __syncthreads();

        // 5b. rho max of tm over [i - D0, i + D0], exact equality with the conv value and the
        //     Radon mask; warp task = kRowBlock output rows x 32 columns (one per lane).  The
        //     last row block is moved up to end at nRho and the last strip's spare lanes
        //     repeat column nTheta - 1; only rows and columns a task owns can flag.  Flagged
        //     peaks go into the warp's top-N list ordered by (value desc, position asc).
        float lv = -INFINITY;
        int lp = -1;
        {
            const int nrho = a.nRho;
            constexpr int kStrip = (kNT + 31) / 32;
            const int nstrip = kNT > 0 ? kStrip : (nT + 31) / 32;
            const int nrowb = (nrho + kRowBlock - 1) / kRowBlock;
            for (int task = warp; task < nstrip * nrowb; task += kWarps) {
                const int rb = task / nstrip, st = task - rb * nstrip;
                const int jl = 32 * st + lane;
                const bool colok = jl < nT;
                const int j = colok ? jl : nT - 1;
                const int i_first = rb * kRowBlock;
                const int i0 = i_first < nrho - kRowBlock ? i_first : nrho - kRowBlock;
                // Radon-mask bits of rows i0 .. i0 + kRowBlock - 1 (issued before the tile loads)
                const uint32_t* mb = a.rdnbits + (size_t)j * a.rdnw + (i0 >> 5);
                const unsigned mbits = __funnelshift_r(__ldg(mb), __ldg(mb + 1), i0 & 31);
                const float* tcol = tm + i0 * MP + j;
                float v[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) v[k] = tcol[k * MP];
                // rho max over [o, o + 2*D0] for o = 0..kRowBlock-1: suffix / core / prefix maxima
                float suf[kRowBlock], pre[kRowBlock], core = -INFINITY;
                suf[kRowBlock - 1] = -INFINITY;
#pragma unroll
                for (int o = kRowBlock - 2; o >= 0; --o) suf[o] = fmaxf(v[o], o + 1 <= kRowBlock - 2 ? suf[o + 1] : -INFINITY);
#pragma unroll
                for (int k = kRowBlock - 1; k <= 2 * D0; ++k) core = fmaxf(core, v[k]);
                pre[0] = -INFINITY;
#pragma unroll
                for (int o = 1; o < kRowBlock; ++o) pre[o] = fmaxf(pre[o - 1], v[2 * D0 + o]);
                const float* crow = conv + (i0 + D0) * CP + j + D1;
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) {
                    const float m = fmaxf(fmaxf(suf[o], core), pre[o]);
                    const int i = i0 + o;
                    const float val = crow[o * CP];
                    const bool f = colok && i >= i_first && val == m && ((mbits >> o) & 1u);
                    unsigned bal = __ballot_sync(0xffffffffu, f);
                    while (bal) {
                        const int b = __ffs(bal) - 1;
                        bal &= bal - 1;
                        const float cv = __shfl_sync(0xffffffffu, val, b);
                        list_insert(cv, i * nT + 32 * st + b, lv, lp, nB, lane);
                    }
                }
            }
        }
        if (lane < nB) {
            lv_s[warp * kMaxBands + lane] = lv;
            lp_s[warp * kMaxBands + lane] = lp;
        }
        __syncthreads();

        // the last pattern of a unit is merged before the next unit's load overwrites the conv
        // tile; packed units are then labelled from the capture scratch (only global memory:
        // the next unit's load runs on beside it)
        if (kPack == 1) {
            if (warp == 0) merge_label(q);
            __syncthreads();
        } else if (sub == npk - 1) {
            if (warp == 0) merge_capture(sub);
            __syncthreads();
            label_unit(npk);
        }
        }  // sub
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
size_t smem_bytes(const FusedGeom& g, size_t store, int ngroups, size_t tm_bytes) {
    // odd row pitches, as the kernel lays the tiles out
    size_t b = (std::max((size_t)(g.row1 - g.row0) * ((g.col1 - g.col0) | 1) * store, tm_bytes) + 15) & ~(size_t)15;
    b += ((size_t)(g.row1 - g.row0) * ((g.ccol1 - g.ccol0) | 1) * 4 + 15) & ~(size_t)15;
    b += (size_t)kWarps * kMaxBands * 8 + 32 * 8 + 80 * 4;
    b += (size_t)ngroups * 8 + 2 * (kWarps + 1) * 4;
    return b;
}

template <typename InT, typename S, int P>
void* kernel_ptr(int k0, int k1, int nTheta) {
    // the common geometry (5x5 LoG, 180 theta samples) gets constant tile pitches
    if (k0 == 5 && k1 == 5 && nTheta == 180) return (void*)k_fused<InT, S, 5, 5, P, 180>;
    if (k0 == 5 && k1 == 5) return (void*)k_fused<InT, S, 5, 5, P, 0>;
    if (k0 == 7 && k1 == 7) return (void*)k_fused<InT, S, 7, 7, P, 0>;
    if (k0 == 9 && k1 == 9) return (void*)k_fused<InT, S, 9, 9, P, 0>;
    if (k0 == 5 && k1 == 7) return (void*)k_fused<InT, S, 5, 7, P, 0>;
    if (k0 == 7 && k1 == 5) return (void*)k_fused<InT, S, 7, 5, P, 0>;
    return nullptr;
}

// FP16 storage, packed uint8 units: the 5x5 LoG only (other kernel shapes run one pattern per pass)
template <int P>
void* kernel_ptr_half_packed(int k0, int k1, int nTheta) {
    if (k0 == 5 && k1 == 5 && nTheta == 180) return (void*)k_fused<uint8_t, __half, 5, 5, P, 180>;
    if (k0 == 5 && k1 == 5) return (void*)k_fused<uint8_t, __half, 5, 5, P, 0>;
    return nullptr;
}

void* pick_kernel(int method, int dtype, int k0, int k1, int pack, int nTheta) {
    bool h = method == EBSD_FUSED_F16;
    switch (dtype) {
        case EBSD_U8:
            if (pack == 8) return h ? kernel_ptr_half_packed<8>(k0, k1, nTheta) : kernel_ptr<uint8_t, float, 8>(k0, k1, nTheta);
            if (pack == 4) return h ? kernel_ptr_half_packed<4>(k0, k1, nTheta) : kernel_ptr<uint8_t, float, 4>(k0, k1, nTheta);
            if (pack == 2) return h ? kernel_ptr_half_packed<2>(k0, k1, nTheta) : kernel_ptr<uint8_t, float, 2>(k0, k1, nTheta);
            return h ? kernel_ptr<uint8_t, __half, 1>(k0, k1, nTheta) : kernel_ptr<uint8_t, float, 1>(k0, k1, nTheta);
        case EBSD_U16:
            return h ? kernel_ptr<uint16_t, __half, 1>(k0, k1, nTheta) : kernel_ptr<uint16_t, float, 1>(k0, k1, nTheta);
        case EBSD_F32:
            return h ? kernel_ptr<float, __half, 1>(k0, k1, nTheta) : kernel_ptr<float, float, 1>(k0, k1, nTheta);
    }
    return nullptr;
}

// Packed modes apply to uint8 patterns without a background, FP32 tile, rays of <= 257
// pixels; four or eight per pass also need the 8-byte-element tile and its LUT (fg.quad).
// Returns the largest patterns-per-pass the call may use (1, 2 or 8).
int max_pack(const ebsd_plan_s* p, int method, int dtype, int64_t n) {
    const bool tile_ok = (method == EBSD_FUSED_F32 && p->fg.ok_f32) ||
                         // FP16 storage: packed kernels are built for the 5x5 LoG only
                         (method == EBSD_FUSED_F16 && p->fg.ok && p->k0 == 5 && p->k1 == 5);
    if (!(dtype == EBSD_U8 && tile_ok && p->bg_mode == 0 && p->maxCount <= 257 && n >= 2)) return 1;
    return p->fg.quad && p->d_flut8 ? 8 : 2;
}

// Launch facts, set up on first use so that later launches -- also inside a CUDA-graph
// capture -- issue nothing but the launch itself.  The opt-in shared-memory attribute is per
// (kernel, device) and only ever raised (plans of different sizes share a kernel); resident
// CTAs per SM are kept per (kernel, device, shared-memory size).
struct SmemAttr {
    const void* fn;
    int device, smem_max;
};
struct LaunchCfg {
    const void* fn;
    int device, smem, sms, per_sm;
};
std::mutex g_cfg_mtx;
std::vector<SmemAttr> g_attr;
std::vector<LaunchCfg> g_cfg;

int launch_config(const void* fn, int device, int smem, int* sms, int* per_sm) {
    std::lock_guard<std::mutex> lk(g_cfg_mtx);
    SmemAttr* attr = nullptr;
    for (SmemAttr& s : g_attr)
        if (s.fn == fn && s.device == device) attr = &s;
    if (!attr) {
        g_attr.push_back(SmemAttr{fn, device, 0});
        attr = &g_attr.back();
    }
    if (smem > attr->smem_max) {
        EBSD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr->smem_max = smem;
    }
    for (const LaunchCfg& c : g_cfg)
        if (c.fn == fn && c.device == device && c.smem == smem) {
            *sms = c.sms;
            *per_sm = c.per_sm;
            return EBSD_OK;
        }
    LaunchCfg c{fn, device, smem, 0, 0};
    EBSD_CUDA_TRY(cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, device));
    EBSD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_sm, fn, kThreads, smem));
    g_cfg.push_back(c);
    *sms = c.sms;
    *per_sm = c.per_sm;
    return EBSD_OK;
}

}  // namespace

int fused_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d) {
    FusedGeom g;
    const int K0 = p->k0, K1 = p->k1;
    // the fused kernel assumes the standard windows: peakPad = 2*ksz + 1 (half-window = ksz)
    bool shape_ok = p->pk0 == 2 * K0 + 1 && p->pk1 == 2 * K1 + 1 && 2 * K1 < 32 &&
                    pick_kernel(EBSD_FUSED_F32, EBSD_U8, K0, K1, 1, p->nTheta) != nullptr &&
                    p->nRho >= kRowBlock && p->nTheta >= 2 * K1 + 1 &&
                    p->p0 >= K0 + K0 / 2 && p->p1 >= K1 + K1 / 2;
    int pitch = p->W + 1;
    if (((int64_t)p->H * pitch + 1) * 4 >= 65535) shape_ok = false;  // byte offsets in 16 bits
    if (shape_ok) {
        const int D0 = K0, D1 = K1, H0 = K0 / 2, H1 = K1 / 2;
        int statR1 = std::min(p->R, p->Tp - p->p0);
        g.crow0 = p->p0 - D0;
        g.crow1 = std::max(p->p0 + p->nRho + D0, statR1);
        g.ccol0 = p->p1 - D1;
        g.ccol1 = p->p1 + p->nTheta + D1;
        g.row0 = g.crow0 - H0;
        g.row1 = g.crow1 + H0;
        g.col0 = g.ccol0 - H1;
        g.col1 = g.ccol1 + H1;
        g.tile_pitch = pitch;
        g.threads = kThreads;
        int ngroups = p->nTheta * ((p->nRho + 31) / 32);  // 32-ray groups of the fused LUT
        const size_t tm_bytes = (size_t)(p->nRho + 2 * D0) * (p->nTheta | 1) * sizeof(float);
        g.smem_f32 = (int)smem_bytes(g, 4, ngroups, tm_bytes);
        g.smem_f16 = (int)smem_bytes(g, 2, ngroups, tm_bytes);
        size_t conv_cells = (size_t)(g.crow1 - g.crow0) * ((g.ccol1 - g.ccol0) | 1);
        int dev_smem = 0;
        cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
        g.ok = conv_cells >= (size_t)p->H * pitch + 1 && g.smem_f16 <= dev_smem && g.row0 >= 0 &&
               (size_t)(g.row1 - g.row0) * ((g.col1 - g.col0) | 1) < 65535;
        g.ok_f32 = g.ok && g.smem_f32 <= dev_smem;
        // four patterns per pass: 8-byte pixel elements, byte offsets still in 16 bits
        const size_t quad_bytes = ((size_t)p->H * pitch + 1) * 8;
        g.quad = g.ok_f32 && quad_bytes < 65535 && conv_cells * 4 >= quad_bytes;
    }
    p->fg = g;
    if (!g.ok) return EBSD_OK;

    // LUT: groups of 32 consecutive rho at one theta (rho padded to a multiple of 32).  When
    // every ray of a group has at most one pixel per image column (the sampling of rays with
    // |sin theta| >= sqrt(2)/2, radon_fast.py:113-133), slot s of every lane is column
    // base + s: a warp then reads one column at distinct rows of the odd-pitch tile, free of
    // bank conflicts.  Likewise per row for the other family (radon_fast.py:134-158); a group
    // that fits neither (a custom maskindex) keeps each ray's own sorted order.  Entries are
    // tile offsets y*pitch + x; empty slots point at the zero word after the pattern.  Integer
    // pixel sums are exact in float32 whatever the order; for background-subtracted or float
    // patterns the slot order changes the ray sums at rounding level only.
    const int L = d->lut_len;
    const int gpt = (p->nRho + 31) / 32;  // groups per theta column
    const int nGroups = p->nTheta * gpt;
    const int nRaysPad = nGroups * 32;
    if (nGroups > 65535) {  // group ids are packed into 16 bits
        p->fg.ok = p->fg.ok_f32 = p->fg.quad = 0;
        return EBSD_OK;
    }
    const uint16_t zero = (uint16_t)(p->H * pitch);
    std::vector<int32_t> cnt(nRaysPad, 0), gch(nGroups, 1), gaxis(nGroups, 2), gbase(nGroups, 0);
    std::vector<char> seen((size_t)std::max(p->W, p->H));
    int nch = 1;
    for (int g = 0; g < nGroups; ++g) {
        int j = g / gpt, i0 = (g % gpt) * 32;
        bool colok = true, rowok = true;
        int xmin = 1 << 30, xmax = -1, ymin = 1 << 30, ymax = -1, maxc = 0;
        for (int l = 0; l < 32; ++l) {
            int i = i0 + l;
            if (i >= p->nRho) continue;
            const int64_t* ray = d->lut + ((size_t)i * p->nTheta + j) * L;
            int c = 0;
            while (c < L && ray[c] >= 0 && ray[c] < p->nPx) ++c;
            cnt[g * 32 + l] = c;
            maxc = std::max(maxc, c);
            std::fill(seen.begin(), seen.end(), 0);
            for (int k = 0; k < c; ++k) {
                int x = (int)(ray[k] % p->W);
                if (seen[x]) colok = false;
                seen[x] = 1;
                xmin = std::min(xmin, x);
                xmax = std::max(xmax, x);
            }
            std::fill(seen.begin(), seen.end(), 0);
            for (int k = 0; k < c; ++k) {
                int y = (int)(ray[k] / p->W);
                if (seen[y]) rowok = false;
                seen[y] = 1;
                ymin = std::min(ymin, y);
                ymax = std::max(ymax, y);
            }
        }
        int nslot;
        if (maxc == 0) {
            nslot = 0;
        } else if (colok) {
            gaxis[g] = 0;
            gbase[g] = xmin;
            nslot = xmax - xmin + 1;
        } else if (rowok) {
            gaxis[g] = 1;
            gbase[g] = ymin;
            nslot = ymax - ymin + 1;
        } else {
            nslot = maxc;
        }
        gch[g] = std::max(1, (nslot + 7) / 8);
        nch = std::max(nch, gch[g]);
    }
    // assign groups to warps, longest first, each to the warp with the fewest chunks so far
    std::vector<int> order(nGroups);
    for (int g = 0; g < nGroups; ++g) order[g] = g;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return gch[x] > gch[y]; });
    std::vector<std::vector<int>> wg(kWarps);
    std::vector<long> wload(kWarps, 0);
    for (int g : order) {
        int w = (int)(std::min_element(wload.begin(), wload.end()) - wload.begin());
        wg[w].push_back(g);
        wload[w] += gch[g];
    }
    // per-warp stream order: group id | chunks << 16, and the Radon tile offset of the
    // group's lane 0 | rays inside nRho << 16; each warp's chunk stream is followed by kRing
    // zero chunks so that the kernel's ring of prefetched chunks loads unconditionally
    std::vector<uint32_t> gst, gtb;
    std::vector<int32_t> wofs(2 * (kWarps + 1), 0);
    const int TP = (g.col1 - g.col0) | 1;  // Radon tile row pitch (odd, as in the kernel)
    for (int w = 0; w < kWarps; ++w) {
        std::sort(wg[w].begin(), wg[w].end());
        wofs[w + 1] = wofs[w] + (int)wg[w].size();
        wofs[kWarps + 1 + w + 1] = wofs[kWarps + 1 + w] + (int)wload[w] + kRing;
        for (int gg : wg[w]) {
            const int j = gg / gpt, i0 = (gg % gpt) * 32;
            gst.push_back((uint32_t)gg | ((uint32_t)gch[gg] << 16));
            const int base = (i0 + p->p0 - g.row0) * TP + (j + p->p1 - g.col0);
            gtb.push_back((uint32_t)base | ((uint32_t)std::min(32, p->nRho - i0) << 16));
        }
    }
    const long total_chunks = wofs[2 * kWarps + 1];
    // stream layout: [chunk of the warp's stream][lane][8 entries], entry = byte offset
    std::vector<uint16_t> lut((size_t)total_chunks * 32 * 8, (uint16_t)(zero * 4));
    std::vector<long> gstart(nGroups, 0);
    for (int w = 0; w < kWarps; ++w) {
        long f = wofs[kWarps + 1 + w];
        for (int g : wg[w]) {
            gstart[g] = f;
            f += gch[g];
        }
    }
    for (int g = 0; g < nGroups; ++g) {
        int j = g / gpt, i0 = (g % gpt) * 32;
        for (int l = 0; l < 32; ++l) {
            int i = i0 + l;
            if (i >= p->nRho) continue;
            int t = g * 32 + l;
            const int64_t* ray = d->lut + ((size_t)i * p->nTheta + j) * L;
            for (int k = 0; k < cnt[t]; ++k) {
                int idx = (int)ray[k];
                int y = idx / p->W, x = idx - (idx / p->W) * p->W;
                int slot = gaxis[g] == 0 ? x - gbase[g] : (gaxis[g] == 1 ? y - gbase[g] : k);
                lut[((size_t)(gstart[g] + slot / 8) * 32 + l) * 8 + (slot % 8)] = (uint16_t)((y * pitch + x) * 4);
            }
        }
    }
    // padding cells of the Radon tile and where each copies from (band_detect.py:573-580):
    // theta padding = theta-wrapped interior column with rho flipped, rho padding = first /
    // last interior row, rows at or below R = zero (the convolution's zero extension)
    std::vector<unsigned> padlist;
    {
        const int TR = g.row1 - g.row0, TC = g.col1 - g.col0, TPp = TC | 1;
        for (int tr = 0; tr < TR; ++tr)
            for (int tc = 0; tc < TC; ++tc) {
                int r = tr + g.row0, i = r - p->p0, j = tc + g.col0 - p->p1;
                if (i >= 0 && i < p->nRho && j >= 0 && j < p->nTheta) continue;
                unsigned src = 0xFFFFu;
                if (r >= 0 && r < p->R) {
                    int ic = i < 0 ? 0 : (i >= p->nRho ? p->nRho - 1 : i);
                    int si = ic, sj = j;
                    if (j < 0) { si = p->nRho - 1 - ic; sj = p->nTheta + j; }
                    else if (j >= p->nTheta) { si = p->nRho - 1 - ic; sj = j - p->nTheta; }
                    src = (unsigned)((si + p->p0 - g.row0) * TPp + (sj + p->p1 - g.col0));
                }
                padlist.push_back((src << 16) | (unsigned)(tr * TPp + tc));
            }
    }
    EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_fpad, padlist.size() * sizeof(unsigned)));
    EBSD_CUDA_TRY(cudaMemcpy(p->d_fpad, padlist.data(), padlist.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
    p->fg.npad = (int)padlist.size();
    p->fg.nGroups = nGroups;
    p->fg.nRaysPad = nRaysPad;
    p->fg.gpt = gpt;
    // weight image: mean over non-empty rays of the ray means = sum_px w[px] * value[px]
    {
        std::vector<double> w(p->nPx, 0.0);
        int nonempty = 0;
        for (int t = 0; t < nRaysPad; ++t) nonempty += cnt[t] > 0;
        for (int g = 0; g < nGroups; ++g) {
            int j = g / gpt, i0 = (g % gpt) * 32;
            for (int l = 0; l < 32; ++l) {
                int i = i0 + l, t = g * 32 + l;
                if (i >= p->nRho || !cnt[t]) continue;
                const int64_t* ray = d->lut + ((size_t)i * p->nTheta + j) * L;
                double f = 1.0 / ((double)cnt[t] * std::max(nonempty, 1));
                for (int k = 0; k < cnt[t]; ++k) w[ray[k]] += f;
            }
        }
        std::vector<float> wf(w.begin(), w.end());
        EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_fray, wf.size() * sizeof(float)));
        EBSD_CUDA_TRY(cudaMemcpy(p->d_fray, wf.data(), wf.size() * sizeof(float), cudaMemcpyHostToDevice));
        double ks = 0.0;
        for (int k = 0; k < K0 * K1; ++k) ks += d->kernel[k];
        p->fg.ksum = (float)ks;
    }
    EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_flut, lut.size() * sizeof(uint16_t)));
    EBSD_CUDA_TRY(cudaMemcpy(p->d_flut, lut.data(), lut.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    if (p->fg.quad) {
        // 8-byte tile elements: every byte offset (cell * 4) doubles; fg.quad guarantees
        // the doubled offsets, zero element included, stay below 65535
        for (uint16_t& e : lut) e = (uint16_t)(e * 2);
        EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_flut8, lut.size() * sizeof(uint16_t)));
        EBSD_CUDA_TRY(cudaMemcpy(p->d_flut8, lut.data(), lut.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    // device tables: [count][RN(1/count)][stream group ids][stream tile offsets][wofs]
    std::vector<int32_t> tables(cnt);
    for (int t = 0; t < nRaysPad; ++t) {
        const float r = cnt[t] > 0 ? 1.0f / (float)cnt[t] : 0.0f;
        int32_t bits;
        std::memcpy(&bits, &r, sizeof(bits));
        tables.push_back(bits);
    }
    tables.insert(tables.end(), gst.begin(), gst.end());
    tables.insert(tables.end(), gtb.begin(), gtb.end());
    tables.insert(tables.end(), wofs.begin(), wofs.end());
    EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_fgroup, tables.size() * sizeof(int32_t)));
    EBSD_CUDA_TRY(cudaMemcpy(p->d_fgroup, tables.data(), tables.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    p->flut_entries = (int64_t)lut.size();
    return EBSD_OK;
}

void fused_release(ebsd_plan_s* p) {
    cudaFree(p->d_flut);
    cudaFree(p->d_flut8);
    p->d_flut8 = nullptr;
    cudaFree(p->d_fgroup);
    cudaFree(p->d_fray);
    cudaFree(p->d_fpad);
    p->d_fpad = nullptr;
    p->d_flut = nullptr;
    p->d_fgroup = nullptr;
    p->d_fray = nullptr;
}

int fused_supported(const ebsd_plan_s* p, int method) {
    // plans too large for the single tile run the FP32 method in theta slabs (slab.cu), and FP16
    // storage there when the FP16 slab tile fits (integer patterns)
    if (method == EBSD_FUSED_F32 && !p->fg.ok_f32 && p->sg.ok) return 1;
    if (method == EBSD_FUSED_F16 && !p->fg.ok && p->sg.ok && p->sg.ok16) return 1;
    if (!p->fg.ok) return 0;
    if (method == EBSD_FUSED_F32) return p->fg.ok_f32;
    return method == EBSD_FUSED_F16;
}

void band_epilogue_launch(const ebsd_bands& out, int64_t out_offset, int64_t n, int nB, const LabelConsts& kc,
                          int sms, cudaStream_t st) {
    const int64_t nbands = n * nB;
    ebsd_bands ob = out;
    const int64_t o0 = out_offset * nB;
    ob.max += o0; ob.normmax += o0; ob.maxloc += 2 * o0; ob.avemax += o0; ob.aveloc += 2 * o0;
    ob.width += o0; ob.theta += o0; ob.rho += o0; ob.valid += o0;
    const int eblocks = (int)std::min<int64_t>((nbands + 255) / 256, (int64_t)sms * 8);
    if (eblocks > 0) k_band_epilogue<<<eblocks, 256, 0, st>>>(ob, nbands, kc);
}

// packed-mode scratch: (patterns per pass - 1) rows of parked ray means per resident CTA
size_t fused_workspace_bytes(const ebsd_plan_s* p, int method, int64_t) {
    if (!((method == EBSD_FUSED_F32 && p->fg.ok_f32) || (method == EBSD_FUSED_F16 && p->fg.ok))) return 0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    const int rows = p->fg.quad ? 7 : 1;
    return (size_t)std::max(sms, 1) * ((size_t)rows * p->fg.nRaysPad + kCapFloats) * sizeof(float);
}

int fused_patterns_per_pass(const ebsd_plan_s* p, int method, int dtype, int64_t n) {
    int pack = max_pack(p, method, dtype, n);
    if (pack == 1 || p->ws.ptr == nullptr || p->ws.bytes < fused_workspace_bytes(p, method, n)) return 1;
    if (p->fused_ppp >= 1 && p->fused_ppp < pack) pack = p->fused_ppp;
    return pack;
}

int fused_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches) {
    if (n <= 0) return EBSD_OK;
    if (slab_serves(p, method, dtype)) return slab_run_chunk(p, method, dtype, d_pats, n, out, out_offset, st, launches);
    if ((method == EBSD_FUSED_F32 && !p->fg.ok_f32) || !p->fg.ok) return EBSD_E_UNSUPPORTED;
    const int pack = fused_patterns_per_pass(p, method, dtype, n);
    void* fn = pick_kernel(method, dtype, p->k0, p->k1, pack, p->nTheta);
    if (!fn) return EBSD_E_UNSUPPORTED;
    const FusedGeom& g = p->fg;
    int smem = method == EBSD_FUSED_F16 ? g.smem_f16 : g.smem_f32;
    int sms = 0, per_sm = 0;
    int rc = launch_config(fn, p->device, smem, &sms, &per_sm);
    if (rc != EBSD_OK) return rc;
    if (per_sm < 1) return EBSD_E_UNSUPPORTED;
    int64_t units = (n + pack - 1) / pack;
    int64_t grid = std::min<int64_t>(units, (int64_t)sms * per_sm);
    if (pack > 1 && grid > sms) grid = sms;  // the scratch holds one set of rows per SM

    FusedArgs a;
    a.pats = d_pats;
    a.n = n;
    a.H = p->H;
    a.W = p->W;
    a.nPx = p->nPx;
    a.pitch = g.tile_pitch;
    a.lut = (const uint4*)p->d_flut;
    a.lut8 = (const uint4*)p->d_flut8;
    a.count = p->d_fgroup;
    a.rcount = (const float*)(p->d_fgroup + g.nRaysPad);
    a.gstream = (const uint32_t*)(p->d_fgroup + 2 * g.nRaysPad);
    a.gtile = a.gstream + g.nGroups;
    a.wofs = (const int32_t*)(a.gtile + g.nGroups);
    a.padlist = p->d_fpad;
    a.npad = g.npad;
    a.pack_scratch = pack > 1 ? (float*)p->ws.ptr : nullptr;
    a.one = 1u;
    {
        // capture scratch after the parked-row scratch of every CTA
        const int rows = p->fg.quad ? 7 : 1;
        a.cap = pack > 1 ? (float*)p->ws.ptr + (size_t)sms * rows * g.nRaysPad : nullptr;
    }
    a.gpt = g.gpt;
    a.nRays = p->nRays;
    a.nRaysPad = g.nRaysPad;
    a.nGroups = g.nGroups;
    a.nRho = p->nRho;
    a.nTheta = p->nTheta;
    a.p0 = p->p0;
    a.p1 = p->p1;
    a.R = p->R;
    a.Tp = p->Tp;
    a.row0 = g.row0;
    a.col0 = g.col0;
    a.TR = g.row1 - g.row0;
    a.TC = g.col1 - g.col0;
    a.crow0 = g.crow0;
    a.ccol0 = g.ccol0;
    a.CR = g.crow1 - g.crow0;
    a.CC = g.ccol1 - g.ccol0;
    a.statR1 = std::min(p->R, p->Tp - p->p0);
    for (int k = 0; k < p->k0 * p->k1 && k < 81; ++k) a.taps[k] = p->h_kernel[k];
    a.sep = p->sep && p->k0 <= 9 && p->k1 <= 9;
    for (int k = 0; k < 9; ++k) {
        a.ku[k] = k < p->k0 && a.sep ? p->h_ku[k] : 0.0f;
        a.kw[k] = k < p->k1 && a.sep ? p->h_kw[k] : 0.0f;
    }
    a.ksum = g.ksum;
    if (a.sep) {  // FP16 centring: the separable form's tap sum
        double su = 0.0, sw = 0.0;
        for (int k = 0; k < p->k0; ++k) su += p->h_ku[k];
        for (int k = 0; k < p->k1; ++k) sw += p->h_kw[k];
        a.ksum = (float)(su * sw);
    }
    a.wimg = p->d_fray;
    a.rdnmask = p->d_rdnmask;
    a.rdnbits = p->d_rdnbits;
    a.rdnw = p->rdn_words;
    a.bg_mode = p->bg_mode;
    a.bg = p->d_bg;
    a.bgf = p->d_bgf;
    a.kc = LabelConsts{p->p0, p->p1, p->nTheta, p->nRho, p->nB, p->d_theta, p->d_rho};
    a.out = *out;
    a.out_offset = out_offset;
    void* args[] = {&a};
    EBSD_CUDA_TRY(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kThreads), args, (size_t)smem, st));
    // the float64 part of the band fit (width, theta, rho) as a separate elementwise pass, so
    // that the fused kernel's label warp is not held up by float64 latency
    band_epilogue_launch(*out, out_offset, n, p->nB, a.kc, sms, st);
    *launches += 2;
    return launch_status();
}

}  // namespace ebsd

