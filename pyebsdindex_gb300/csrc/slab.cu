// Fused band detection in theta slabs, for plans whose padded Radon image does not fit in
// shared memory next to its LoG image (120x120 and 240x240 patterns with nRho = 1.5 * size).
//
// One persistent CTA per SM, one pattern at a time.  The pattern stays in shared memory
// (uint8 / uint16 / float32 elements as stored) while the theta range is processed in slabs
// of Ts output columns.  For each slab:
//   1. radon   the rays of the slab's Ts columns plus D1 + H1 columns on either side (the max
//              filter's and the LoG's theta reach), one ray per lane as in the single-tile
//              kernel: per-warp streams of 32-ray groups (32 neighbouring rho at one theta),
//              8 pattern-element offsets per lane per 16-byte LUT load, sums in the LUT's
//              column (or row) order -- exact integers for uint8/uint16 patterns -- and the
//              mean as a correctly rounded quotient (rdn_loops, radon_fast.py:281-310).
//              Columns beyond theta 0 / 180 deg are the theta-wrapped rays written rho-flipped,
//              as band_detect.py:573-575 pads the Radon image.  Neighbouring slabs share
//              2 * (D1 + H1) Radon columns: they move to the front of the tile after the conv's
//              theta pass, and every slab but the first computes only the columns after them.
//   2. pad     rho padding rows: the first / last interior row, zero from row R on
//              (band_detect.py:578-580 and the FFT convolution's zero extension).
//   3. conv    two-pass separable LoG (theta taps along rows, rho taps down columns in place)
//              with the multiply-add order of the per-stage kernels; the statistics slice's
//              min and sum accumulate over the slabs' own columns.
//   4. peaks   theta max of the conv rows, rho max, exact equality with the conv value and
//              the Radon mask (band_detect.py:639-664); warp top-N lists ordered by (value
//              desc, position asc) with positions i * nTheta + j of the whole image.
//   5. merge   warp 0 takes the slab's best nB peaks (k-way tournament over the warp lists)
//              with their 3x3 conv blocks and merges them into the pattern's running top-N,
//              while the other warps start the next slab.  Under one strict total order the
//              top-N of the union equals the top-N of the slabs' top-N lists, so the bands equal
//              those of the single-tile kernel.
// After the last slab: the min / mean reduction and the band fits (band_detect.py:691-809)
// from the captured blocks; width, theta and rho in float64 by the shared epilogue pass.
#include "ebsd_internal.cuh"
#include "label.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cfloat>
#include <cstring>

namespace ebsd {

void band_epilogue_launch(const ebsd_bands& out, int64_t out_offset, int64_t n, int nB, const LabelConsts& kc,
                          int sms, cudaStream_t st);

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kRowBlock = 8;
constexpr int kRing = 2;
constexpr int kBlk = 12;  // running top-N entry: value, position, 9 conv values, pad

struct SlabArgs {
    const void* pats;
    int64_t n;
    int H, W, pitch;           // pattern tile: H rows of pitch W + 1 elements, then one zero element
    const uint4* lut;          // per-slab, per-warp streams of 8 element offsets per lane per chunk
    const uint32_t* gst;       // [all slabs' groups] source group id | chunks << 16
    const uint32_t* gtb;       // same order: tile offset of lane 0 | rays << 16 | rho-flipped << 22
    const int32_t* slab_g;     // [nslab + 1] first group of each slab
    const int32_t* slab_j;     // [nslab + 1] first output theta column of each slab
    const int32_t* wofs;       // [nslab][2 * (kWarps + 1)] per-warp first group (slab-relative), first chunk
    const int32_t* count;      // [nTheta * gpt * 32] in-mask pixels of each ray (source group * 32 + lane)
    int nslab, maxg;
    int nRho, nTheta, nB;
    int p0, p1;
    int TR, TBP, CCP, MP;      // Radon tile rows, Radon / conv / theta-max pitches (FP32 tile: MP = TBP)
    int regb, tmb;             // bytes of the Radon-tile region; FP16 tile: theta-max rows first (tmb bytes)
    const float* wimg;         // FP16 tile: [H * W] pixel weights whose dot product is the Radon mean
    float ksum;                // FP16 tile: sum of the LoG taps (the centring correction)
    int rho0;                  // tile row of interior row 0 (p0 - row0)
    int rpad_end;              // tile rows from here on are zero (padded row R)
    int CR;                    // conv rows
    int statR;                 // statistics rows (conv rows [D0, D0 + statR))
    float ku[9], kw[9];
    const uint8_t* rdnmask;
    const uint32_t* rdnbits;   // [nTheta][rdnw] the Radon mask as bit columns
    int rdnw;
    LabelConsts kc;
    ebsd_bands out;
    int64_t out_offset;
};

// One launch serves up to kMaxPlans plans of one input type and LoG size (mixed pattern sizes):
// plan k's patterns are indices [start[k], start[k + 1]) of the launch, which the persistent
// CTAs stride over, so every CTA takes patterns of every plan.  The arguments travel by value
// in the launch parameters.
constexpr int kMaxPlans = 8;
struct MultiArgs {
    SlabArgs plan[kMaxPlans];
    int64_t start[kMaxPlans + 1];
    int nplans;
};

template <typename S> __device__ __forceinline__ S slab_store(float v);
template <> __device__ __forceinline__ float slab_store<float>(float v) { return v; }
template <> __device__ __forceinline__ __half slab_store<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float slab_load(float v) { return v; }
__device__ __forceinline__ float slab_load(__half v) { return __half2float(v); }

__device__ __forceinline__ bool beats(float v, int p, float w, int q) {
    return v > w || (v == w && p < q);
}

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

// S: Radon tile storage -- float, or __half holding (value - m) * s with m the pattern's Radon
// mean and s a power of two (FP16 storage, as the single-tile kernel's; FP32 conv and fit).
template <typename InT, typename S, int K0, int K1>
__global__ void __launch_bounds__(kThreads, 1) k_slab(const __grid_constant__ MultiArgs ma) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int D0 = K0, D1 = K1;          // max-filter half windows (peakPad = 2*ksz + 1)
    constexpr int H1 = K1 / 2;               // LoG half width along theta
    constexpr int WIN = 2 * D1 + 1;
    constexpr int NV = kRowBlock + 2 * D0;
    constexpr int kCarry = 2 * (D1 + H1);    // Radon columns shared by neighbouring slabs
    constexpr bool kInt = sizeof(InT) < 4;
    constexpr bool kHalf = sizeof(S) == 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int64_t qq = blockIdx.x; qq < ma.start[ma.nplans]; qq += gridDim.x) {
    int pid = 0;
    while (pid + 1 < ma.nplans && qq >= ma.start[pid + 1]) ++pid;
    const SlabArgs& a = ma.plan[pid];
    const int64_t q = qq - ma.start[pid];
    const int nB = a.nB, TBP = a.TBP, CCP = a.CCP, MP = a.MP;

    size_t off = 0;
    InT* pat = (InT*)(smem + off);
    off += ((size_t)(a.H * a.pitch + 1) * sizeof(InT) + 15) & ~(size_t)15;
    // Radon slab; the theta-max rows sit after the carried columns of its rows (FP32), or
    // before the tile (FP16: tmb bytes)
    S* tile = (S*)(smem + off + (kHalf ? a.tmb : 0));
    float* tm = kHalf ? (float*)(smem + off) : (float*)tile + kCarry;
    off += (size_t)a.regb;
    float* conv = (float*)(smem + off);  // TR rows: the two-pass convolution's theta pass
    off += ((size_t)a.TR * CCP * sizeof(float) + 15) & ~(size_t)15;
    float* lv_s = (float*)(smem + off);
    off += kWarps * kMaxBands * sizeof(float);
    int* lp_s = (int*)(smem + off);
    off += kWarps * kMaxBands * sizeof(int);
    float* run = (float*)(smem + off);   // running top-N: [kMaxBands][kBlk], ping-pong
    off += 2 * kMaxBands * kBlk * sizeof(float);
    float* red_f = (float*)(smem + off);
    off += 80 * sizeof(float);
    double* red_d = (double*)(smem + off);
    off += 32 * sizeof(double);
    int* wofs_s = (int*)(smem + off);
    off += 2 * (kWarps + 1) * sizeof(int);
    unsigned* gst_s = (unsigned*)(smem + off);
    off += (size_t)a.maxg * sizeof(unsigned);
    unsigned* gtb_s = (unsigned*)(smem + off);

    const int stat_rows = a.statR;
    {
        // ---- the pattern into shared memory; one zero element after it (the LUT's pad slot)
        {
            const InT* gp = (const InT*)a.pats + q * (int64_t)a.H * a.W;
            for (int y = warp; y < a.H; y += kWarps)
                for (int x = lane; x < a.W; x += 32) pat[y * a.pitch + x] = gp[y * a.W + x];
            if (tid == 0) pat[a.H * a.pitch] = (InT)0;
        }
        // FP16 tile: the pattern's Radon mean m (by linearity, sum_px w[px] p[px]) and a power
        // of two s keeping |value - m| s < 2^14, as the single-tile kernel computes them
        float cen = 0.0f, scl = 1.0f, inv_scl = 1.0f;
        if (kHalf) {
            float ws = 0.0f, mn = -1.0f, mx = -1.0f;  // -1: value of an empty ray
            for (int y = warp; y < a.H; y += kWarps)
                for (int x = lane; x < a.W; x += 32) {
                    const float v = (float)pat[y * a.pitch + x];
                    ws = fmaf(a.wimg[y * a.W + x], v, ws);
                    mn = fminf(mn, v);
                    mx = fmaxf(mx, v);
                }
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
                    const float m = (float)dw;
                    int e = 0;
                    frexpf(fmaxf(fmaxf(fabsf(mx - m), fabsf(mn - m)), 1e-30f), &e);
                    red_f[64] = m;
                    red_f[65] = ldexpf(1.0f, 14 - e);
                }
            }
            __syncthreads();
            cen = red_f[64];
            scl = red_f[65];
            inv_scl = 1.0f / scl;  // exact: scl is a power of two
        }
        float smin = INFINITY, ssum = 0.0f;
        int cur = 0;  // running list buffer
        if (tid < kMaxBands) {
            run[tid * kBlk + 1] = __int_as_float(-1);
            run[kMaxBands * kBlk + tid * kBlk + 1] = __int_as_float(-1);
        }

        // slab merge (warp 0): the slab's nB best peaks from the warp lists, their 3x3 conv
        // blocks from the conv region, merged into the running list by rank
        auto slab_merge = [&](int j0) {
            int ptr = 0;
            float hv = lane < kWarps ? lv_s[lane * kMaxBands] : -INFINITY;
            int hp = lane < kWarps ? lp_s[lane * kMaxBands] : -1;
            int mypos = -1;
            float myval = 0.0f;
            for (int k = 0; k < nB; ++k) {
                const unsigned u = __float_as_uint(hv + 0.0f);
                const unsigned key = hp < 0 ? 0u : ((u & 0x80000000u) ? ~u : (u | 0x80000000u));
                const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
                if (kmax == 0u) break;
                const unsigned pmin = __reduce_min_sync(0xffffffffu, key == kmax ? (unsigned)hp : 0xffffffffu);
                const unsigned win = __ballot_sync(0xffffffffu, key == kmax && (unsigned)hp == pmin);
                const float wv = __shfl_sync(0xffffffffu, hv, __ffs(win) - 1);
                if (lane == k) { mypos = (int)pmin; myval = wv; }
                if (lane == __ffs(win) - 1) {
                    ++ptr;
                    hp = ptr < nB ? lp_s[lane * kMaxBands + ptr] : -1;
                    hv = ptr < nB ? lv_s[lane * kMaxBands + ptr] : -INFINITY;
                }
            }
            float blk[9];
#pragma unroll
            for (int k9 = 0; k9 < 9; ++k9) blk[k9] = 0.0f;
            if (mypos >= 0) {
                const int i = mypos / a.nTheta, j = mypos - i * a.nTheta - j0;
                const float* c0 = conv + (i + D0 - 1) * CCP + (j + D1 - 1);
#pragma unroll
                for (int r3 = 0; r3 < 3; ++r3)
#pragma unroll
                    for (int c3 = 0; c3 < 3; ++c3) blk[r3 * 3 + c3] = c0[r3 * CCP + c3];
            }
            // ranks: a slab entry counts the running entries ahead of it, a running entry the
            // slab entries ahead of it; positions are unique, so the ranks are distinct
            const float* ro = run + cur * kMaxBands * kBlk;
            float* rn = run + (cur ^ 1) * kMaxBands * kBlk;
            const float rv = lane < nB ? ro[lane * kBlk] : 0.0f;
            const int rp = lane < nB ? __float_as_int(ro[lane * kBlk + 1]) : -1;
            int rank_s = lane, rank_r = lane;
            for (int k = 0; k < nB; ++k) {
                const float ov = __shfl_sync(0xffffffffu, rv, k);
                const int op = __shfl_sync(0xffffffffu, rp, k);
                const float sv = __shfl_sync(0xffffffffu, myval, k);
                const int sp = __shfl_sync(0xffffffffu, mypos, k);
                if (op >= 0 && beats(ov, op, myval, mypos)) ++rank_s;
                if (sp >= 0 && beats(sv, sp, rv, rp)) ++rank_r;
            }
            if (lane < nB && mypos >= 0 && rank_s < nB) {
                float* d = rn + rank_s * kBlk;
                d[0] = myval;
                d[1] = __int_as_float(mypos);
#pragma unroll
                for (int k9 = 0; k9 < 9; ++k9) d[2 + k9] = blk[k9];
            }
            if (lane < nB && rp >= 0 && rank_r < nB) {
                float* d = rn + rank_r * kBlk;
                const float* s = ro + lane * kBlk;
#pragma unroll
                for (int k = 0; k < 11; ++k) d[k] = s[k];
            }
            // slots past the merged entries stay empty
            const int nsl = __popc(__ballot_sync(0xffffffffu, lane < nB && mypos >= 0));
            const int nrn = __popc(__ballot_sync(0xffffffffu, lane < nB && rp >= 0));
            if (lane < nB && lane >= nsl + nrn) rn[lane * kBlk + 1] = __int_as_float(-1);
            __syncwarp();
        };

        for (int s = 0; s < a.nslab; ++s) {
            const int j0 = __ldg(a.slab_j + s), Ts = __ldg(a.slab_j + s + 1) - j0;
            const int gbeg = __ldg(a.slab_g + s), ng = __ldg(a.slab_g + s + 1) - gbeg;
            // (the previous slab's merge, below, reads only the warp lists and the conv region)
            for (int i = tid; i < ng; i += kThreads) {
                gst_s[i] = __ldg(a.gst + gbeg + i);
                gtb_s[i] = __ldg(a.gtb + gbeg + i);
            }
            for (int i = tid; i < 2 * (kWarps + 1); i += kThreads) wofs_s[i] = __ldg(a.wofs + s * 2 * (kWarps + 1) + i);
            __syncthreads();
            if (s > 0 && warp == 0) {
                slab_merge(__ldg(a.slab_j + s - 1));
                cur ^= 1;
            }

            // ---- 1. Radon of the slab's columns, one ray per lane
            {
                const int g0 = wofs_s[warp], g1 = wofs_s[warp + 1];
                const uint4* ip = a.lut + ((size_t)wofs_s[kWarps + 1 + warp] * 32 + lane);
                uint4 ring[kRing];
#pragma unroll
                for (int k = 0; k < kRing; ++k) ring[k] = __ldg(ip + (size_t)k * 32);
                ip += (size_t)kRing * 32;
                int gi = g0, pc = 0;
                unsigned gs = gi < g1 ? gst_s[gi] : 0u;
                int t = (int)(gs & 0xFFFFu) * 32 + lane;
                int cnt = gi < g1 ? __ldg(a.count + t) : 0;
                unsigned isum = 0u;
                float fsum = 0.0f;
                while (gi < g1) {
#pragma unroll
                    for (int k = 0; k < kRing; ++k) {
                        if (gi < g1) {
                            const uint4 e = ring[k];
                            ring[k] = __ldg(ip);
                            ip += 32;
                            const unsigned o[8] = {e.x & 0xFFFF, e.x >> 16, e.y & 0xFFFF, e.y >> 16,
                                                   e.z & 0xFFFF, e.z >> 16, e.w & 0xFFFF, e.w >> 16};
#pragma unroll
                            for (int k8 = 0; k8 < 8; ++k8) {
                                if (kInt) isum += (unsigned)pat[o[k8]];
                                else fsum = __fadd_rn(fsum, (float)pat[o[k8]]);
                            }
                            if (++pc == (int)(gs >> 16)) {
                                // ray ends: the mean of an empty ray is -1 (radon_fast.py:265)
                                float v = cnt > 0 ? __fdiv_rn(kInt ? (float)isum : fsum, (float)cnt) : -1.0f;
                                if (kHalf) v = (v - cen) * scl;
                                const unsigned tb = gtb_s[gi];
                                const int stride = (tb >> 22) & 1 ? -TBP : TBP;
                                if (lane < (int)((tb >> 16) & 63)) tile[(int)(tb & 0xFFFFu) + lane * stride] = slab_store<S>(v);
                                ++gi;
                                pc = 0;
                                isum = 0u;
                                fsum = 0.0f;
                                if (gi < g1) {
                                    gs = gst_s[gi];
                                    t = (int)(gs & 0xFFFFu) * 32 + lane;
                                    cnt = __ldg(a.count + t);
                                }
                            }
                        }
                    }
                }
            }
            __syncthreads();

            // ---- 2. rho padding rows of every buffer column
            {
                const int TB = Ts + 2 * (D1 + H1);
                const int top = a.rho0, bot = a.rho0 + a.nRho;  // interior tile rows [top, bot)
                const int npadrow = top + (a.TR - bot);
                for (int k = tid; k < npadrow * TB; k += kThreads) {
                    const int pr = k / TB, c = k - pr * TB;
                    const int r = pr < top ? pr : bot + (pr - top);
                    S v;
                    if (r >= a.rpad_end) v = slab_store<S>(kHalf ? -cen * scl : 0.0f);
                    else v = tile[(r < top ? top : bot - 1) * TBP + c];
                    tile[r * TBP + c] = v;
                }
            }
            __syncthreads();

            // ---- 3. LoG convolution, two separable passes (as the single-tile kernel)
            const int CCs = Ts + 2 * D1;
            {
                constexpr int kSegA = 16;
                const int nseg = (CCs + kSegA - 1) / kSegA;
                for (int task = tid; task < a.TR * nseg; task += kThreads) {
                    const int sg = task / a.TR, r = task - sg * a.TR;
                    const int c0 = sg * kSegA < CCs - kSegA ? sg * kSegA : CCs - kSegA;
                    const S* trow = tile + r * TBP + c0;
                    float x[kSegA + K1 - 1];
#pragma unroll
                    for (int k = 0; k < kSegA + K1 - 1; ++k) x[k] = slab_load(trow[k]);
                    float* hrow = conv + r * CCP + c0;
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
            // the Radon columns the next slab shares with this one (its left halo and the first
            // halo-width of its own columns) move to the front of the tile; the next slab's
            // Radon phase computes only the columns after them
            if (s + 1 < a.nslab) {
                for (int k = tid; k < a.TR * kCarry; k += kThreads) {
                    const int r = k / kCarry, c = k - r * kCarry;
                    tile[r * TBP + c] = tile[r * TBP + Ts + c];
                }
            }
            {
                const int CR = a.CR;
                const int nstrip = CCs >= kThreads ? 1 : (kThreads / CCs < (CR + 7) / 8 ? kThreads / CCs : (CR + 7) / 8);
                const int L = (CR + nstrip - 1) / nstrip;
                const int ntask = nstrip * CCs;
                const int rounds = (ntask + kThreads - 1) / kThreads;
                for (int rd = 0; rd < rounds; ++rd) {
                    const int task = rd * kThreads + tid;
                    const int st = task < ntask ? task / CCs : 0, cc = task < ntask ? task - st * CCs : 0;
                    const int o0 = st * L, o1 = task < ntask ? (o0 + L < CR ? o0 + L : CR) : 0;
                    float* hcol = conv + cc;
                    // statistics columns: this slab's own theta columns
                    const bool colstat = (unsigned)(cc - D1) < (unsigned)Ts;
                    float w[K0], held[K0 - 1];
#pragma unroll
                    for (int k = 0; k < K0 - 1; ++k) {
                        w[k] = o0 < o1 ? hcol[(o0 + k) * CCP] : 0.0f;
                        held[k] = 0.0f;
                    }
                    for (int o = o0; o < o1; o += K0) {
#pragma unroll
                        for (int j = 0; j < K0; ++j) {
                            const int oj = o + j;
                            if (oj < o1) {
                                w[(j + K0 - 1) % K0] = hcol[(oj + K0 - 1) * CCP];
                                float acc = 0.0f;
#pragma unroll
                                for (int ka = 0; ka < K0; ++ka) acc = fmaf(a.ku[ka], w[(j + K0 - 1 - ka) % K0], acc);
                                if (kHalf) acc = fmaf(a.ksum, cen, acc * inv_scl);
                                if (j < K0 - 1 && o == o0) held[j < K0 - 1 ? j : 0] = acc;
                                else hcol[oj * CCP] = acc;
                                if (colstat && (unsigned)(oj - D0) < (unsigned)stat_rows) {
                                    smin = fminf(smin, acc);
                                    ssum += acc;
                                }
                            }
                        }
                    }
                    __syncthreads();
#pragma unroll
                    for (int k = 0; k < K0 - 1; ++k)
                        if (o0 + k < o1) hcol[(o0 + k) * CCP] = held[k];
                }
            }
            __syncthreads();

            // ---- 4a. theta max of the conv rows the rho window needs (into the dead Radon tile,
            // after the carried columns; FP16 tile: into the rows before it)
            {
                const int NR = a.nRho + 2 * D0;
                const int nseg = (Ts + WIN - 1) / WIN;
                for (int task = tid; task < NR * nseg; task += kThreads) {
                    const int sg = task / NR, rr = task - sg * NR;
                    const int jj = sg * WIN < Ts - WIN ? sg * WIN : Ts - WIN;
                    const float* x = conv + rr * CCP + jj;
                    float* o = tm + rr * MP + jj;
                    float xv[2 * WIN - 1];
#pragma unroll
                    for (int k = 0; k < 2 * WIN - 1; ++k) xv[k] = x[k];
#pragma unroll
                    for (int k = WIN - 2; k >= 0; --k) xv[k] = fmaxf(xv[k], xv[k + 1]);
                    float pm = -INFINITY;
#pragma unroll
                    for (int tt = 0; tt < WIN; ++tt) {
                        if (tt > 0) pm = fmaxf(pm, xv[WIN - 1 + tt]);
                        o[tt] = fmaxf(xv[tt], pm);
                    }
                }
            }
            __syncthreads();

            // ---- 4b. rho max, exact equality, Radon mask; warp top-N lists
            float lv = -INFINITY;
            int lp = -1;
            {
                const int nrho = a.nRho;
                const int nstrip = (Ts + 31) / 32;
                const int nrowb = (nrho + kRowBlock - 1) / kRowBlock;
                for (int task = warp; task < nstrip * nrowb; task += kWarps) {
                    const int rb = task / nstrip, st = task - rb * nstrip;
                    const int jl = 32 * st + lane;
                    const bool colok = jl < Ts;
                    const int j = colok ? jl : Ts - 1;
                    const int i_first = rb * kRowBlock;
                    const int i0 = i_first < nrho - kRowBlock ? i_first : nrho - kRowBlock;
                    // Radon-mask bits of rows i0 .. i0 + kRowBlock - 1 (issued before the tile loads)
                    const uint32_t* mb = a.rdnbits + (size_t)(j0 + j) * a.rdnw + (i0 >> 5);
                    const unsigned mbits = __funnelshift_r(__ldg(mb), __ldg(mb + 1), i0 & 31);
                    const float* tcol = tm + i0 * MP + j;
                    float v[NV];
#pragma unroll
                    for (int k = 0; k < NV; ++k) v[k] = tcol[k * MP];
                    float suf[kRowBlock], pre[kRowBlock], core = -INFINITY;
                    suf[kRowBlock - 1] = -INFINITY;
#pragma unroll
                    for (int o = kRowBlock - 2; o >= 0; --o) suf[o] = fmaxf(v[o], o + 1 <= kRowBlock - 2 ? suf[o + 1] : -INFINITY);
#pragma unroll
                    for (int k = kRowBlock - 1; k <= 2 * D0; ++k) core = fmaxf(core, v[k]);
                    pre[0] = -INFINITY;
#pragma unroll
                    for (int o = 1; o < kRowBlock; ++o) pre[o] = fmaxf(pre[o - 1], v[2 * D0 + o]);
                    const float* crow = conv + (i0 + D0) * CCP + j + D1;
#pragma unroll
                    for (int o = 0; o < kRowBlock; ++o) {
                        const float m = fmaxf(fmaxf(suf[o], core), pre[o]);
                        const int i = i0 + o;
                        const float val = crow[o * CCP];
                        const bool f = colok && i >= i_first && val == m && ((mbits >> o) & 1u);
                        unsigned bal = __ballot_sync(0xffffffffu, f);
                        while (bal) {
                            const int b = __ffs(bal) - 1;
                            bal &= bal - 1;
                            const float cv = __shfl_sync(0xffffffffu, val, b);
                            list_insert(cv, i * a.nTheta + j0 + 32 * st + b, lv, lp, nB, lane);
                        }
                    }
                }
            }
            if (lane < nB) {
                lv_s[warp * kMaxBands + lane] = lv;
                lp_s[warp * kMaxBands + lane] = lp;
            }
            __syncthreads();
        }
        // the last slab's peaks, then the statistics and the band fits
        if (warp == 0) {
            slab_merge(__ldg(a.slab_j + a.nslab - 1));
            cur ^= 1;
        }
        {
            float hi = ssum, lo = 0.0f, m = smin;
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, hi, o);
                const float ol = __shfl_down_sync(0xffffffffu, lo, o);
                const float s2 = __fadd_rn(hi, oh);
                const float bb = __fsub_rn(s2, hi);
                const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s2, bb)), __fsub_rn(oh, bb));
                const float e2 = __fadd_rn(err, __fadd_rn(lo, ol));
                hi = __fadd_rn(s2, e2);
                lo = __fsub_rn(e2, __fsub_rn(hi, s2));
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            if (lane == 0) { red_f[warp] = m; red_f[32 + warp] = hi; red_d[warp] = (double)lo; }
        }
        __syncthreads();
        if (warp == 0) {
            double sd = (double)red_f[32 + lane] + red_d[lane];
            float m = red_f[lane];
            for (int o = 16; o > 0; o >>= 1) {
                sd += __shfl_down_sync(0xffffffffu, sd, o);
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            sd = __shfl_sync(0xffffffffu, sd, 0);
            m = __shfl_sync(0xffffffffu, m, 0);
            const int stat_count = stat_rows * a.nTheta;
            const float mean = (float)(sd / (double)stat_count);
            if (lane < nB) {
                const float* e = run + cur * kMaxBands * kBlk + lane * kBlk;
                const int pos = __float_as_int(e[1]);
                const bool has = pos >= 0;
                int r = 0, c = 0;
                float nn[9];
#pragma unroll
                for (int k9 = 0; k9 < 9; ++k9) nn[k9] = has ? e[2 + k9] : 0.0f;
                if (has) {
                    const int i = pos / a.nTheta;
                    r = i + a.p0;
                    c = (pos - i * a.nTheta) + a.p1;
                }
                band_fit_block<float, false>(has, r, c, nn, m, mean, a.kc, a.out, (a.out_offset + q) * nB + lane);
            }
        }
        __syncthreads();
    }
    }  // patterns
}

}  // namespace
}  // namespace ebsd

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
namespace ebsd {
namespace {

template <typename InT>
void* slab_kernel(int k0, int k1) {
    if (k0 == 5 && k1 == 5) return (void*)k_slab<InT, float, 5, 5>;
    if (k0 == 7 && k1 == 7) return (void*)k_slab<InT, float, 7, 7>;
    if (k0 == 9 && k1 == 9) return (void*)k_slab<InT, float, 9, 9>;
    return nullptr;
}

void* pick_slab_kernel(int dtype, int k0, int k1, bool half = false) {
    // FP16 Radon storage: integer patterns and the 5x5 LoG
    if (half) {
        if (k0 != 5 || k1 != 5) return nullptr;
        if (dtype == EBSD_U8) return (void*)k_slab<uint8_t, __half, 5, 5>;
        if (dtype == EBSD_U16) return (void*)k_slab<uint16_t, __half, 5, 5>;
        return nullptr;
    }
    switch (dtype) {
        case EBSD_U8: return slab_kernel<uint8_t>(k0, k1);
        case EBSD_U16: return slab_kernel<uint16_t>(k0, k1);
        case EBSD_F32: return slab_kernel<float>(k0, k1);
    }
    return nullptr;
}

size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// dynamic shared memory of k_slab, as the kernel carves it (regb: the Radon-tile region)
size_t slab_smem(size_t pat_elems, size_t esize, size_t regb, int TR, int CCP, int maxg) {
    size_t b = align16(pat_elems * esize);
    b += regb;
    b += align16((size_t)TR * CCP * 4);
    b += (size_t)kWarps * kMaxBands * 8 + 2 * kMaxBands * kBlk * 4 + 80 * 4 + 32 * 8 + 2 * (kWarps + 1) * 4;
    b += (size_t)maxg * 8;
    return b;
}

std::mutex g_slab_mtx;
struct SlabAttr {
    const void* fn;
    int device, smem;
};
std::vector<SlabAttr> g_slab_attr;

int slab_attr(const void* fn, int device, int smem) {
    std::lock_guard<std::mutex> lk(g_slab_mtx);
    for (SlabAttr& s : g_slab_attr)
        if (s.fn == fn && s.device == device) {
            if (smem > s.smem) {
                EBSD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
                s.smem = smem;
            }
            return EBSD_OK;
        }
    EBSD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    g_slab_attr.push_back(SlabAttr{fn, device, smem});
    return EBSD_OK;
}

}  // namespace

namespace {

// Slab geometry for nslab slabs of the plan's theta range, or false when the slabs are too
// narrow for the filters' reach or their tiles do not fit (uint16 pattern tile).
bool slab_geom_for(const ebsd_plan_s* p, const SlabSource& src, int nslab, int dev_smem, SlabGeom* out) {
    const int D1 = p->k1, H1 = p->k1 / 2, halo = D1 + H1;
    if (nslab < 1 || nslab > p->nTheta) return false;
    const int ts = (p->nTheta + nslab - 1) / nslab;
    // every slab (widths differ by at most one column) must hold the filters' reach
    const int tmin = p->nTheta / nslab;
    if (tmin < 2 * D1 + 1 || tmin < 16 || tmin < 2 * halo) return false;
    SlabGeom g;
    g.nslab = nslab;
    g.Ts = ts;
    g.TR = src.TR;
    g.TBP = (ts + 2 * halo) | 1;
    g.CCP = (ts + 2 * D1) | 1;
    if ((size_t)g.TR * g.TBP >= 65536) return false;
    g.MP = g.TBP;  // the theta-max rows sit in the Radon tile after the carried columns
    g.rho0 = src.rho0;
    g.rpad_end = src.rpad_end;
    g.CR = src.CR;
    g.statR = src.statR;
    g.pitch = src.pitch;
    g.maxg = (ts + 2 * halo) * src.gpt;
    g.regb = (int)align16((size_t)g.TR * g.TBP * 4);
    g.smem[0] = (int)slab_smem(src.pat_elems, 1, g.regb, g.TR, g.CCP, g.maxg);
    g.smem[1] = (int)slab_smem(src.pat_elems, 2, g.regb, g.TR, g.CCP, g.maxg);
    g.smem[2] = (int)slab_smem(src.pat_elems, 4, g.regb, g.TR, g.CCP, g.maxg);
    if (g.smem[1] > dev_smem) return false;
    g.ok = 1;
    g.ok_f32 = g.smem[2] <= dev_smem;
    // FP16 tile (5x5 LoG): the theta-max rows (nRho + 2 D0 rows of an odd pitch >= Ts) first,
    // then the 16-bit Radon tile
    if (p->k0 == 5 && p->k1 == 5) {
        g.MP16 = ts | 1;
        g.tmb16 = (int)align16((size_t)(p->nRho + 2 * p->k0) * g.MP16 * 4);
        g.regb16 = g.tmb16 + (int)align16((size_t)g.TR * g.TBP * 2);
        g.smem16[0] = (int)slab_smem(src.pat_elems, 1, g.regb16, g.TR, g.CCP, g.maxg);
        g.smem16[1] = (int)slab_smem(src.pat_elems, 2, g.regb16, g.TR, g.CCP, g.maxg);
        g.ok16 = g.smem16[1] <= dev_smem;
    }
    *out = g;
    return true;
}

// Device tables of the geometry g: per slab, buffer columns [j0 - halo, j0 + ts + halo), the
// slab's 32-ray groups balanced over the warps (longest first, each to the least-loaded warp).
int slab_upload(ebsd_plan_s* p, const SlabSource& src, SlabGeom g) {
    const int D1 = p->k1, H1 = p->k1 / 2, halo = D1 + H1;
    const int nslab = g.nslab, gpt = src.gpt;
    std::vector<int32_t> slab_j(nslab + 1), slab_g(nslab + 1, 0), wofs;
    std::vector<uint32_t> gst, gtb;
    std::vector<uint16_t> lut;
    for (int s = 0; s <= nslab; ++s) slab_j[s] = (int)((int64_t)p->nTheta * s / nslab);
    int maxg = 0;
    for (int s = 0; s < nslab; ++s) {
        const int j0 = slab_j[s], ts = slab_j[s + 1] - j0, TB = ts + 2 * halo;
        if (ts < 2 * D1 + 1 || ts < 2 * halo) return EBSD_E_UNSUPPORTED;
        struct Grp {
            int src;
            uint32_t tb;
        };
        std::vector<Grp> grps;
        // slabs after the first take their first 2 * halo columns from the previous slab
        for (int jb = s > 0 ? 2 * halo : 0; jb < TB; ++jb) {
            const int jc = j0 - halo + jb;
            const bool flip = jc < 0 || jc >= p->nTheta;
            const int js = ((jc % p->nTheta) + p->nTheta) % p->nTheta;
            for (int b = 0; b < gpt; ++b) {
                const int nval = std::min(32, p->nRho - 32 * b);
                const int row = g.rho0 + (flip ? p->nRho - 1 - 32 * b : 32 * b);
                const uint32_t offs = (uint32_t)(row * g.TBP + jb);
                grps.push_back(Grp{js * gpt + b, offs | ((uint32_t)nval << 16) | ((flip ? 1u : 0u) << 22)});
            }
        }
        maxg = std::max(maxg, (int)grps.size());
        std::vector<int> order(grps.size());
        for (size_t k = 0; k < grps.size(); ++k) order[k] = (int)k;
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return src.gch[grps[x].src] > src.gch[grps[y].src]; });
        std::vector<std::vector<int>> wg(kWarps);
        std::vector<long> wload(kWarps, 0);
        for (int k : order) {
            const int w = (int)(std::min_element(wload.begin(), wload.end()) - wload.begin());
            wg[w].push_back(k);
            wload[w] += src.gch[grps[k].src];
        }
        std::vector<int32_t> wo(2 * (kWarps + 1), 0);
        int gcount = 0;
        for (int w = 0; w < kWarps; ++w) {
            wo[w] = gcount;
            wo[kWarps + 1 + w] = (int32_t)(lut.size() / (32 * 8));
            for (int k : wg[w]) {
                const Grp& gr = grps[k];
                gst.push_back((uint32_t)gr.src | ((uint32_t)src.gch[gr.src] << 16));
                gtb.push_back(gr.tb);
                const uint16_t* sl = src.slots.data() + src.goff[gr.src];
                lut.insert(lut.end(), sl, sl + (size_t)src.gch[gr.src] * 32 * 8);
                ++gcount;
            }
            lut.insert(lut.end(), (size_t)kRing * 32 * 8, src.zero);  // the ring's unconditional loads
        }
        wo[kWarps] = gcount;
        wo[2 * kWarps + 1] = (int32_t)(lut.size() / (32 * 8));
        wofs.insert(wofs.end(), wo.begin(), wo.end());
        slab_g[s + 1] = slab_g[s] + gcount;
    }
    if (maxg > g.maxg) return EBSD_E_UNSUPPORTED;
    // device tables: [gst][gtb][slab_g][slab_j][wofs][count], each part 16-byte aligned
    std::vector<int32_t> tab;
    auto part = [&](const int32_t* a, size_t cnt) {
        const int32_t at = (int32_t)tab.size();
        tab.insert(tab.end(), a, a + cnt);
        while (tab.size() % 4) tab.push_back(0);
        return at;
    };
    const int32_t o_gst = part((const int32_t*)gst.data(), gst.size());
    const int32_t o_gtb = part((const int32_t*)gtb.data(), gtb.size());
    const int32_t o_slabg = part(slab_g.data(), slab_g.size());
    const int32_t o_slabj = part(slab_j.data(), slab_j.size());
    const int32_t o_wofs = part(wofs.data(), wofs.size());
    const int32_t o_count = part(src.count.data(), src.count.size());
    int32_t* d_tab = nullptr;
    uint16_t* d_lut = nullptr;
    EBSD_CUDA_TRY(cudaMalloc((void**)&d_tab, tab.size() * sizeof(int32_t)));
    if (cudaMalloc((void**)&d_lut, lut.size() * sizeof(uint16_t)) != cudaSuccess ||
        cudaMemcpy(d_tab, tab.data(), tab.size() * sizeof(int32_t), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_lut, lut.data(), lut.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d_tab);
        cudaFree(d_lut);
        return EBSD_E_NOMEM;
    }
    // launches already queued may still read the old tables
    if (p->d_stab || p->d_slut) {
        EBSD_CUDA_TRY(cudaDeviceSynchronize());
        cudaFree(p->d_slut);
        cudaFree(p->d_stab);
    }
    p->d_stab = d_tab;
    p->d_slut = d_lut;
    p->s_gst = o_gst;
    p->s_gtb = o_gtb;
    p->s_slabg = o_slabg;
    p->s_slabj = o_slabj;
    p->s_wofs = o_wofs;
    p->s_count = o_count;
    p->sg = g;
    return EBSD_OK;
}

int device_smem_optin(int device) {
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    return dev_smem;
}

}  // namespace

// Plan-time tables for the slab kernel.  The LUT groups are those of the single-tile kernel:
// 32 neighbouring rho at one theta, slot s of every lane at image column (or row) base + s when
// each ray of the group has at most one pixel per column (row), as the reference's sampling
// gives (radon_fast.py:113-158); a group that fits neither keeps each ray's sorted order.
// Built for every plan whose geometry qualifies: the single-plan path uses it when the single
// tile does not fit (or the plan is set to slabs), the mixed-size launch
// (ebsd_find_bands_mixed) for every plan.  The widest slabs that fit are laid out first.
int slab_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d) {
    p->sg = SlabGeom{};
    const int K0 = p->k0, K1 = p->k1;
    const int D0 = K0, D1 = K1, H0 = K0 / 2, H1 = K1 / 2;
    if (!(p->pk0 == 2 * K0 + 1 && p->pk1 == 2 * K1 + 1 && K0 == K1 && pick_slab_kernel(EBSD_U16, K0, K1) &&
          p->sep && p->bg_mode == 0 && p->nRho >= kRowBlock && p->nTheta >= 4 * (D1 + H1) &&
          p->p0 >= D0 + H0 && p->maxCount <= 255 && p->H <= 255 && p->W <= 255))
        return EBSD_OK;
    SlabSource* src = new SlabSource;
    src->pitch = p->W + 1;
    src->pat_elems = (size_t)p->H * src->pitch + 1;
    if (src->pat_elems > 65535) {  // element offsets in 16 bits
        delete src;
        return EBSD_OK;
    }
    // padded-frame rows as the single-tile kernel: tile rows [row0, row1), conv rows [crow0, crow1)
    const int statR1 = std::min(p->R, p->Tp - p->p0);
    const int crow0 = p->p0 - D0, crow1 = std::max(p->p0 + p->nRho + D0, statR1);
    const int row0 = crow0 - H0, row1 = crow1 + H0;
    src->TR = row1 - row0;
    src->CR = crow1 - crow0;
    src->rho0 = p->p0 - row0;
    src->rpad_end = p->R - row0;
    src->statR = statR1 - p->p0;
    src->gpt = (p->nRho + 31) / 32;
    const int gpt = src->gpt;

    // the slab counts whose tiles fit
    const int dev_smem = device_smem_optin(p->device);
    SlabGeom g;
    int nmin = 0, nmax = 0;
    for (int ns = 1; ns <= p->nTheta; ++ns) {
        SlabGeom t;
        if (!slab_geom_for(p, *src, ns, dev_smem, &t)) {
            if (nmin) break;
            continue;
        }
        if (!nmin) {
            nmin = ns;
            g = t;
        }
        nmax = ns;
    }
    if (!nmin) {
        delete src;
        return EBSD_OK;
    }

    // per source group (theta j, rho block b): chunks, and each lane's slot -> element offset
    const int L = d->lut_len;
    const int nsrc = p->nTheta * gpt;
    src->nsrc = nsrc;
    src->zero = (uint16_t)(p->H * src->pitch);
    src->gch.assign(nsrc, 1);
    src->goff.assign(nsrc, 0);
    src->count.assign((size_t)nsrc * 32, 0);
    std::vector<char> seen((size_t)std::max(p->W, p->H));
    for (int gs = 0; gs < nsrc; ++gs) {
        const int j = gs / gpt, i0 = (gs % gpt) * 32;
        bool colok = true, rowok = true;
        int xmin = 1 << 30, xmax = -1, ymin = 1 << 30, ymax = -1, maxc = 0;
        for (int l = 0; l < 32 && i0 + l < p->nRho; ++l) {
            const int64_t* ray = d->lut + ((size_t)(i0 + l) * p->nTheta + j) * L;
            int c = 0;
            while (c < L && ray[c] >= 0 && ray[c] < p->nPx) ++c;
            src->count[(size_t)gs * 32 + l] = c;
            maxc = std::max(maxc, c);
            std::fill(seen.begin(), seen.end(), 0);
            for (int k = 0; k < c; ++k) {
                const int x = (int)(ray[k] % p->W);
                if (seen[x]) colok = false;
                seen[x] = 1;
                xmin = std::min(xmin, x);
                xmax = std::max(xmax, x);
            }
            std::fill(seen.begin(), seen.end(), 0);
            for (int k = 0; k < c; ++k) {
                const int y = (int)(ray[k] / p->W);
                if (seen[y]) rowok = false;
                seen[y] = 1;
                ymin = std::min(ymin, y);
                ymax = std::max(ymax, y);
            }
        }
        int axis = 2, base = 0, nslot = maxc;
        if (maxc == 0) {
            nslot = 0;
        } else if (colok) {
            axis = 0;
            base = xmin;
            nslot = xmax - xmin + 1;
        } else if (rowok) {
            axis = 1;
            base = ymin;
            nslot = ymax - ymin + 1;
        }
        src->gch[gs] = std::max(1, (nslot + 7) / 8);
        src->goff[gs] = src->slots.size();
        src->slots.resize(src->slots.size() + (size_t)src->gch[gs] * 32 * 8, src->zero);
        uint16_t* sl = src->slots.data() + src->goff[gs];
        for (int l = 0; l < 32 && i0 + l < p->nRho; ++l) {
            const int64_t* ray = d->lut + ((size_t)(i0 + l) * p->nTheta + j) * L;
            for (int k = 0; k < src->count[(size_t)gs * 32 + l]; ++k) {
                const int idx = (int)ray[k], y = idx / p->W, x = idx - y * p->W;
                const int slot = axis == 0 ? x - base : (axis == 1 ? y - base : k);
                sl[((size_t)(slot / 8) * 32 + l) * 8 + slot % 8] = (uint16_t)(y * src->pitch + x);
            }
        }
    }
    g.nslab_min = nmin;
    g.nslab_max = nmax;
    if (p->k0 == 5 && p->k1 == 5) {
        // pixel weights of the FP16 centring (built for every slab count: the widest slabs may
        // leave no room for an FP16 tile, narrower ones do): the mean over non-empty rays of the ray means is
        // sum_px w[px] * pixel[px] with w[px] = sum over the rays through px of 1 / (count * rays)
        int nonempty = 0;
        for (int32_t c : src->count) nonempty += c > 0;
        std::vector<double> w(p->nPx, 0.0);
        for (int gs = 0; gs < nsrc; ++gs)
            for (int l = 0; l < 32; ++l) {
                const int c = src->count[(size_t)gs * 32 + l];
                if (c <= 0) continue;
                const double f = 1.0 / ((double)c * nonempty);
                for (int ch = 0; ch < src->gch[gs]; ++ch)
                    for (int k = 0; k < 8; ++k) {
                        const uint16_t o = src->slots[src->goff[gs] + ((size_t)ch * 32 + l) * 8 + k];
                        if (o == src->zero) continue;
                        w[(size_t)(o / src->pitch) * p->W + o % src->pitch] += f;
                    }
            }
        std::vector<float> wf(w.begin(), w.end());
        if (cudaMalloc((void**)&p->d_swimg, wf.size() * sizeof(float)) != cudaSuccess ||
            cudaMemcpy(p->d_swimg, wf.data(), wf.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(p->d_swimg);
            p->d_swimg = nullptr;
            delete src;
            return EBSD_E_NOMEM;
        }
    }
    const int rc = slab_upload(p, *src, g);
    if (rc != EBSD_OK) {
        delete src;
        p->sg = SlabGeom{};
        // a plan whose slab layout cannot be built keeps the other paths
        return rc == EBSD_E_UNSUPPORTED ? EBSD_OK : rc;
    }
    p->ssrc = src;
    return EBSD_OK;
}

int slab_relayout(ebsd_plan_s* p, int nslab) {
    if (!p->ssrc || !p->sg.ok) return EBSD_E_UNSUPPORTED;
    const int nmin = p->sg.nslab_min, nmax = p->sg.nslab_max;
    if (nslab == 0) nslab = nmin;
    if (nslab < nmin || nslab > nmax) return EBSD_E_UNSUPPORTED;
    if (nslab == p->sg.nslab) return EBSD_OK;
    SlabGeom g;
    if (!slab_geom_for(p, *p->ssrc, nslab, device_smem_optin(p->device), &g)) return EBSD_E_UNSUPPORTED;
    g.nslab_min = nmin;
    g.nslab_max = nmax;
    return slab_upload(p, *p->ssrc, g);
}

void slab_release(ebsd_plan_s* p) {
    cudaFree(p->d_slut);
    cudaFree(p->d_stab);
    cudaFree(p->d_swimg);
    p->d_swimg = nullptr;
    p->d_slut = nullptr;
    p->d_stab = nullptr;
    p->sg = SlabGeom{};
    delete p->ssrc;
    p->ssrc = nullptr;
}

bool slab_serves(const ebsd_plan_s* p, int method, int dtype) {
    if (!p->sg.ok) return false;
    if (method == EBSD_FUSED_F16)  // FP16 storage: plans the single FP16 tile cannot take
        return !p->fg.ok && p->sg.ok16 && p->d_swimg && (dtype == EBSD_U8 || dtype == EBSD_U16);
    if (method != EBSD_FUSED_F32) return false;
    if (dtype == EBSD_F32 && !p->sg.ok_f32) return false;
    return !p->fg.ok_f32 || p->tile_mode == 2;
}

namespace {

SlabArgs slab_args(const ebsd_plan_s* p, const void* d_pats, int64_t n, const ebsd_bands& out, int64_t out_offset,
                   bool half) {
    const SlabGeom& g = p->sg;
    SlabArgs a;
    a.regb = half ? g.regb16 : g.regb;
    a.tmb = half ? g.tmb16 : 0;
    a.wimg = p->d_swimg;
    {
        double su = 0.0, sw = 0.0;
        for (float v : p->h_ku) su += v;
        for (float v : p->h_kw) sw += v;
        a.ksum = (float)(su * sw);
    }
    a.pats = d_pats;
    a.n = n;
    a.H = p->H;
    a.W = p->W;
    a.pitch = g.pitch;
    a.lut = (const uint4*)p->d_slut;
    a.gst = (const uint32_t*)(p->d_stab + p->s_gst);
    a.gtb = (const uint32_t*)(p->d_stab + p->s_gtb);
    a.slab_g = p->d_stab + p->s_slabg;
    a.slab_j = p->d_stab + p->s_slabj;
    a.wofs = p->d_stab + p->s_wofs;
    a.count = p->d_stab + p->s_count;
    a.nslab = g.nslab;
    a.maxg = g.maxg;
    a.nRho = p->nRho;
    a.nTheta = p->nTheta;
    a.nB = p->nB;
    a.p0 = p->p0;
    a.p1 = p->p1;
    a.TR = g.TR;
    a.TBP = g.TBP;
    a.CCP = g.CCP;
    a.MP = half ? g.MP16 : g.MP;
    a.rho0 = g.rho0;
    a.rpad_end = g.rpad_end;
    a.CR = g.CR;
    a.statR = g.statR;
    for (int k = 0; k < 9; ++k) {
        a.ku[k] = k < p->k0 ? p->h_ku[k] : 0.0f;
        a.kw[k] = k < p->k1 ? p->h_kw[k] : 0.0f;
    }
    a.rdnmask = p->d_rdnmask;
    a.rdnbits = p->d_rdnbits;
    a.rdnw = p->rdn_words;
    a.kc = LabelConsts{p->p0, p->p1, p->nTheta, p->nRho, p->nB, p->d_theta, p->d_rho};
    a.out = out;
    a.out_offset = out_offset;
    return a;
}

int smem_index(int dtype) { return dtype == EBSD_U8 ? 0 : (dtype == EBSD_U16 ? 1 : 2); }

int slab_smem_for(const ebsd_plan_s* p, int dtype, bool half) {
    return half ? p->sg.smem16[dtype == EBSD_U8 ? 0 : 1] : p->sg.smem[smem_index(dtype)];
}

// One persistent launch over the plans' patterns, then each plan's float64 epilogue pass.
int slab_launch(ebsd_plan_s* const* plans, int nplans, int dtype, const void* const* d_pats, const int64_t* n,
                const ebsd_bands* out, const int64_t* out_offset, cudaStream_t st, int64_t* launches,
                bool half = false) {
    const ebsd_plan_s* p0 = plans[0];
    void* fn = pick_slab_kernel(dtype, p0->k0, p0->k1, half);
    if (!fn) return EBSD_E_UNSUPPORTED;
    MultiArgs ma;
    std::memset(&ma, 0, sizeof(ma));
    ma.nplans = nplans;
    int smem = 0;
    int64_t total = 0;
    for (int k = 0; k < nplans; ++k) {
        ma.start[k] = total;
        ma.plan[k] = slab_args(plans[k], d_pats[k], n[k], out[k], out_offset[k], half);
        smem = std::max(smem, slab_smem_for(plans[k], dtype, half));
        total += n[k];
    }
    ma.start[nplans] = total;
    if (total == 0) return EBSD_OK;
    int rc = slab_attr(fn, p0->device, smem);
    if (rc != EBSD_OK) return rc;
    int sms = 0;
    EBSD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p0->device));
    void* args[] = {&ma};
    const int64_t grid = std::min<int64_t>(total, sms);
    EBSD_CUDA_TRY(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kThreads), args, (size_t)smem, st));
    *launches += 1;
    for (int k = 0; k < nplans; ++k) {
        if (n[k] <= 0) continue;
        const SlabArgs& a = ma.plan[k];
        band_epilogue_launch(out[k], out_offset[k], n[k], plans[k]->nB, a.kc, sms, st);
        *launches += 1;
    }
    return launch_status();
}

}  // namespace

int slab_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n, const ebsd_bands* out,
                   int64_t out_offset, cudaStream_t st, int64_t* launches) {
    if (n <= 0) return EBSD_OK;
    if (!slab_serves(p, method, dtype)) return EBSD_E_UNSUPPORTED;
    ebsd_plan_s* plans[1] = {p};
    const void* pats[1] = {d_pats};
    return slab_launch(plans, 1, dtype, pats, &n, out, &out_offset, st, launches, method == EBSD_FUSED_F16);
}

bool slab_mixable(const ebsd_plan_s* p, int dtype) {
    return p->sg.ok && (dtype != EBSD_F32 || p->sg.ok_f32);
}

int slab_run_mixed(ebsd_plan_s* const* plans, int nplans, int dtype, const void* const* d_pats, const int64_t* n,
                   const ebsd_bands* out, cudaStream_t st, int64_t* launches) {
    if (nplans < 1 || nplans > kMaxPlans) return EBSD_E_ARG;
    int64_t offs[kMaxPlans] = {};
    return slab_launch(plans, nplans, dtype, d_pats, n, out, offs, st, launches);
}

}  // namespace ebsd
