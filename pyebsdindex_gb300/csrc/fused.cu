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
//   4. conv      register-blocked direct LoG convolution into an FP32 conv tile, in the same
//                multiply-add order as the per-stage kernel; min/sum for normmax on the fly
//   5. peaks     per warp: 32-column strip x 8 rows; rho max in registers, theta max by warp
//                shuffles, exact equality + rdnmask (band_detect.py:639-664); candidates go
//                into a warp top-N list ordered by (value desc, position asc)
//   6. merge     tree merge of the 32 warp lists
//   7. label     lanes 0..nB-1 of warp 0 fit their band (band_detect.py:691-809) and write
//                the record fields, normmax, theta and rho (band_detect.py:457-460, :521-524)
//
// Shared-memory footprint decides which plans the fused path takes (fused_supported()).
#include "ebsd_internal.cuh"
#include "label.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cfloat>

namespace ebsd {
namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kRowBlock = 8;

struct FusedArgs {
    const void* pats;
    int64_t n;
    int H, W, nPx, pitch;      // pattern tile pitch (W + 1); zero word at H*pitch
    const uint4* lut;          // [chunks][nRaysPad][8] u16 tile offsets, ray order theta-major
    const int32_t* count;      // [nRaysPad] entries per ray (group-major, lane-minor)
    const int32_t* gchunks;    // [nGroups] chunks walked by each 32-ray group
    const int32_t* gids;       // [nGroups] group ids in per-warp stream order
    const int32_t* wofs;       // [2*(kWarps+1)]: per-warp first group index, first chunk
    const unsigned* padlist;   // [npad] (source tile cell << 16) | destination tile cell
    int npad;
    int nRays, nRaysPad, nGroups, gpt, nRho, nTheta;  // gpt: 32-ray groups per theta column
    int p0, p1, R, Tp;
    int row0, col0, TR, TC;    // Radon tile origin (padded frame) and extent
    int crow0, ccol0, CR, CC;  // conv tile origin and extent
    int statR1;                // end row of the statistics slice (padded frame)
    float taps[81];            // LoG taps [K0*K1] (parameter space: FMA operands, no loads)
    float ksum;                // sum of the kernel taps (FP16 centring correction)
    const float* wimg;         // [nPx] pixel weights whose dot product is the Radon mean
    const uint8_t* rdnmask;    // [nRho][nTheta]
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

template <typename InT, typename S, int K0, int K1>
__global__ void __launch_bounds__(kThreads, 1) k_fused(FusedArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int D0 = K0;  // rho half-window of the max filter (peakPad = 2*ksz + 1)
    constexpr int D1 = K1;  // theta half-window
    constexpr int SW = 32 - 2 * D1;  // output columns per warp strip
    constexpr int H0 = K0 / 2, H1 = K1 / 2;
    constexpr int NV = kRowBlock + 2 * D0;  // conv rows a strip block reads

    constexpr bool kHalf = sizeof(S) == 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    size_t off = 0;
    // the conv tile comes first so that the pattern tile aliased into it starts at shared
    // offset 0: the LUT then holds byte offsets usable directly as load addresses
    float* conv = (float*)(smem + off);
    float* pat = conv;  // aliased: the pattern tile is dead once the Radon is built
    off += ((size_t)a.CR * a.CC * sizeof(float) + 15) & ~(size_t)15;
    S* tile = (S*)(smem + off);
    off += ((size_t)a.TR * a.TC * sizeof(S) + 15) & ~(size_t)15;
    float* lv_s = (float*)(smem + off);
    off += kWarps * kMaxBands * sizeof(float);
    int* lp_s = (int*)(smem + off);
    off += kWarps * kMaxBands * sizeof(int);
    double* red_d = (double*)(smem + off);
    off += 32 * sizeof(double);
    float* red_f = (float*)(smem + off);  // 66 floats
    off += 80 * sizeof(float);
    int* gch_s = (int*)(smem + off);      // nGroups ints: chunks of each group
    off += (size_t)a.nGroups * sizeof(int);
    int* gid_s = (int*)(smem + off);      // nGroups ints: group ids, warp after warp
    off += (size_t)a.nGroups * sizeof(int);
    int* wofs_s = (int*)(smem + off);     // 2 * (kWarps + 1) ints: per-warp group / chunk offsets
    off += 2 * (kWarps + 1) * sizeof(int);
    int* rank_s = (int*)(smem + off);     // kThreads ints: candidate ranks
    off += kThreads * sizeof(int);
    float* fin_v = (float*)(smem + off);  // final top-N list
    off += kMaxBands * sizeof(float);
    int* fin_p = (int*)(smem + off);

    for (int i = tid; i < a.nGroups; i += kThreads) {
        gch_s[i] = a.gchunks[i];
        gid_s[i] = a.gids[i];
    }
    for (int i = tid; i < 2 * (kWarps + 1); i += kThreads) wofs_s[i] = a.wofs[i];
    __syncthreads();
    const int nB = a.kc.nB;
    const int stat_r0 = a.p0, stat_r1 = a.statR1, stat_c0 = a.p1, stat_c1 = a.p1 + a.nTheta;
    const int stat_count = (stat_r1 - stat_r0) * (stat_c1 - stat_c0);

    for (int64_t q = blockIdx.x; q < a.n; q += gridDim.x) {
        // ---- 1. load the pattern into the FP32 tile (pitch W+1, zero word after it) ----
        const InT* gp = (const InT*)a.pats + q * (int64_t)a.nPx;
        float wsum = 0.0f, pmin = -1.0f, pmax = -1.0f;  // -1: value of an empty ray
        for (int y = warp; y < a.H; y += kWarps) {
            for (int x = lane; x < a.W; x += 32) {
                const int i = y * a.W + x;
                float v = load_pixel<InT>(gp, i, a.bg_mode, a.bg, a.bgf);
                pat[y * a.pitch + x] = v;
                if (kHalf) {
                    wsum = fmaf(a.wimg[i], v, wsum);
                    pmin = fminf(pmin, v);
                    pmax = fmaxf(pmax, v);
                }
            }
        }
        if (tid == 0) pat[a.H * a.pitch] = 0.0f;
        // FP16 storage keeps (value - m) * s: m = mean of the Radon interior (exact by
        // linearity: sum_px w[px] * p[px]), s = power of two keeping |value - m| * s < 2^14.
        float cen = 0.0f, scl = 1.0f, inv_scl = 1.0f;
        if (kHalf) {
            double dw = (double)wsum;
            for (int o = 16; o > 0; o >>= 1) {
                dw += __shfl_down_sync(0xffffffffu, dw, o);
                pmin = fminf(pmin, __shfl_down_sync(0xffffffffu, pmin, o));
                pmax = fmaxf(pmax, __shfl_down_sync(0xffffffffu, pmax, o));
            }
            if (lane == 0) { red_d[warp] = dw; red_f[warp] = pmin; red_f[32 + warp] = pmax; }
            __syncthreads();
            if (warp == 0) {
                dw = red_d[lane];
                pmin = red_f[lane];
                pmax = red_f[32 + lane];
                for (int o = 16; o > 0; o >>= 1) {
                    dw += __shfl_down_sync(0xffffffffu, dw, o);
                    pmin = fminf(pmin, __shfl_down_sync(0xffffffffu, pmin, o));
                    pmax = fmaxf(pmax, __shfl_down_sync(0xffffffffu, pmax, o));
                }
                if (lane == 0) {
                    float m = (float)dw;
                    float amax = fmaxf(fabsf(pmax - m), fabsf(pmin - m));
                    int e = 0;
                    frexpf(fmaxf(amax, 1e-30f), &e);  // amax < 2^e
                    red_f[64] = m;
                    red_f[65] = ldexpf(1.0f, 14 - e);
                }
            }
        }
        __syncthreads();
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
            constexpr int kRing = 2;  // deeper rings cost registers without hiding more latency
            const unsigned zw = (unsigned)(a.H * a.pitch * 4) * 0x10001u;
            const uint4 zero4 = make_uint4(zw, zw, zw, zw);
            const int g0 = wofs_s[warp], g1 = wofs_s[warp + 1];
            const int nchunk = wofs_s[kWarps + 1 + warp + 1] - wofs_s[kWarps + 1 + warp];
            const uint4* ip = a.lut + ((size_t)wofs_s[kWarps + 1 + warp] * 32 + lane);
            const unsigned char* pb = (const unsigned char*)pat;
            uint4 ring[kRing];
#pragma unroll
            for (int k = 0; k < kRing; ++k) ring[k] = k < nchunk ? __ldg(ip + (size_t)k * 32) : zero4;
            ip += (size_t)kRing * 32;
            int left = nchunk - kRing;  // chunks not yet issued
            int gi = g0, pc = 0;
            int grp = gi < g1 ? gid_s[gi] : 0;
            int pnch = gi < g1 ? gch_s[grp] : 0;
            int cnt = gi < g1 ? __ldg(a.count + grp * 32 + lane) : 0;
            float sum = 0.0f;
            while (gi < g1) {
#pragma unroll
                for (int k = 0; k < kRing; ++k) {
                    if (gi < g1) {
                        const uint4 e = ring[k];
                        ring[k] = left > 0 ? __ldg(ip) : zero4;
                        ip += 32;
                        --left;
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.x & 0xFFFF)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.x >> 16)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.y & 0xFFFF)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.y >> 16)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.z & 0xFFFF)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.z >> 16)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.w & 0xFFFF)));
                        sum = __fadd_rn(sum, *(const float*)(pb + (e.w >> 16)));
                        if (++pc == pnch) {
                            const int j = grp / a.gpt, i = (grp - j * a.gpt) * 32 + lane;
                            if (i < a.nRho) {
                                float v = cnt > 0 ? __fdiv_rn(sum, (float)cnt) : -1.0f;
                                if (kHalf) v = (v - cen) * scl;
                                tile[(i + a.p0 - a.row0) * a.TC + (j + a.p1 - a.col0)] = to_store<S>(v);
                            }
                            ++gi;
                            pc = 0;
                            sum = 0.0f;
                            if (gi < g1) {
                                grp = gid_s[gi];
                                pnch = gch_s[grp];
                                cnt = __ldg(a.count + grp * 32 + lane);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();

        // ---- 3. pad the tile around the interior ----
        // padding cell list (plan table): low half = destination tile cell, high half = source
        // tile cell, 0xFFFF = zero (rows below the padded array, the convolution's zero fill)
        for (int k = tid; k < a.npad; k += kThreads) {
            const unsigned e = __ldg(a.padlist + k);
            const unsigned src = e >> 16;
            tile[e & 0xFFFF] = src == 0xFFFFu ? to_store<S>(kHalf ? -cen * scl : 0.0f) : tile[src];
        }
        __syncthreads();

        // ---- 4. LoG convolution, kRowBlock outputs per thread down one column ----
        float smin = INFINITY, ssum = 0.0f;
        {
            const int nrb = (a.CR + kRowBlock - 1) / kRowBlock;
            for (int task = tid; task < nrb * a.CC; task += kThreads) {
                int cc = task % a.CC, rb = task / a.CC;
                int cr0 = rb * kRowBlock;
                float acc[kRowBlock];
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) acc[o] = 0.0f;
                // tile row (cr0 + t) feeds output o through kernel row a = o + 2*H0 - t;
                // descending t keeps each output's multiply-add order = ascending a.
#pragma unroll
                for (int t = kRowBlock + 2 * H0 - 1; t >= 0; --t) {
                    int tr = cr0 + t;
                    float v[K1];
                    if (tr < a.TR) {
#pragma unroll
                        for (int b = 0; b < K1; ++b) v[b] = to_f(tile[tr * a.TC + cc + 2 * H1 - b]);
                    } else {
#pragma unroll
                        for (int b = 0; b < K1; ++b) v[b] = 0.0f;
                    }
#pragma unroll
                    for (int o = 0; o < kRowBlock; ++o) {
                        int ka = o + 2 * H0 - t;
                        if (ka >= 0 && ka < K0) {
#pragma unroll
                            for (int b = 0; b < K1; ++b) acc[o] = fmaf(a.taps[ka * K1 + b], v[b], acc[o]);
                        }
                    }
                }
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) {
                    int cr = cr0 + o;
                    if (kHalf) acc[o] = fmaf(a.ksum, cen, acc[o] * inv_scl);
                    if (cr < a.CR) {
                        conv[cr * a.CC + cc] = acc[o];
                        int r = cr + a.crow0, col = cc + a.ccol0;
                        if (r >= stat_r0 && r < stat_r1 && col >= stat_c0 && col < stat_c1) {
                            smin = fminf(smin, acc[o]);
                            ssum += acc[o];
                        }
                    }
                }
            }
        }
        // block reduction of min / sum (sum in FP64 across threads)
        {
            double dsum = (double)ssum;
            float m = smin;
            for (int o = 16; o > 0; o >>= 1) {
                dsum += __shfl_down_sync(0xffffffffu, dsum, o);
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            if (lane == 0) { red_d[warp] = dsum; red_f[warp] = m; }
        }
        __syncthreads();
        if (warp == 0) {
            double dsum = red_d[lane];
            float m = red_f[lane];
            for (int o = 16; o > 0; o >>= 1) {
                dsum += __shfl_down_sync(0xffffffffu, dsum, o);
                m = fminf(m, __shfl_down_sync(0xffffffffu, m, o));
            }
            if (lane == 0) { red_d[0] = dsum; red_f[0] = m; }
        }
        // (red_d[0] / red_f[0] are read after the next barrier)

        // ---- 5. peaks: strips of SW output columns x kRowBlock rows per warp task ----
        float lv = -INFINITY;
        int lp = -1;
        {
            const int nstrip = (a.nTheta + SW - 1) / SW;
            const int nrowb = (a.nRho + kRowBlock - 1) / kRowBlock;
            for (int task = warp; task < nstrip * nrowb; task += kWarps) {
                int s = task % nstrip, rb = task / nstrip;
                // lane column in the conv tile: output column p1 + SW*s + (lane - D1)
                int cc = SW * s + lane + (a.p1 - D1 - a.ccol0);
                int cr0 = rb * kRowBlock + (a.p0 - D0 - a.crow0);
                bool colok = cc >= 0 && cc < a.CC;
                float v[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    int cr = cr0 + k;
                    v[k] = (colok && cr < a.CR) ? conv[cr * a.CC + cc] : -INFINITY;
                }
                // rho max over [o, o + 2*D0] for o = 0..7: suffix / core / prefix maxima
                float suf[kRowBlock], pre[kRowBlock], core = -INFINITY;
                suf[kRowBlock - 1] = -INFINITY;
#pragma unroll
                for (int o = kRowBlock - 2; o >= 0; --o) suf[o] = fmaxf(v[o], o + 1 <= kRowBlock - 2 ? suf[o + 1] : -INFINITY);
#pragma unroll
                for (int k = kRowBlock - 1; k <= 2 * D0; ++k) core = fmaxf(core, v[k]);
                pre[0] = -INFINITY;
#pragma unroll
                for (int o = 1; o < kRowBlock; ++o) pre[o] = fmaxf(pre[o - 1], v[2 * D0 + o]);
                int ocol = a.p1 + SW * s + (lane - D1);  // output column (padded frame)
                bool lane_out = lane >= D1 && lane < 32 - D1 && ocol < a.p1 + a.nTheta;
#pragma unroll
                for (int o = 0; o < kRowBlock; ++o) {
                    float m = fmaxf(fmaxf(suf[o], core), pre[o]);
                    float mt = m;
#pragma unroll
                    for (int d = 1; d <= D1; ++d) {
                        mt = fmaxf(mt, __shfl_up_sync(0xffffffffu, m, d));
                        mt = fmaxf(mt, __shfl_down_sync(0xffffffffu, m, d));
                    }
                    int orow = a.p0 + rb * kRowBlock + o;
                    float val = v[o + D0];
                    bool f = lane_out && orow < a.p0 + a.nRho && val == mt &&
                             a.rdnmask[(orow - a.p0) * a.nTheta + (ocol - a.p1)];
                    unsigned bal = __ballot_sync(0xffffffffu, f);
                    while (bal) {
                        int b = __ffs(bal) - 1;
                        bal &= bal - 1;
                        float cv = __shfl_sync(0xffffffffu, val, b);
                        int pos = (orow - a.p0) * a.nTheta + (a.p1 + SW * s + (b - D1) - a.p1);
                        list_insert(cv, pos, lv, lp, nB, lane);
                    }
                }
            }
        }
        if (lane < nB) {
            lv_s[warp * kMaxBands + lane] = lv;
            lp_s[warp * kMaxBands + lane] = lp;
        }
        rank_s[tid] = 0;
        if (tid < kMaxBands) fin_p[tid] = -1;
        __syncthreads();

        // ---- 6. merge the warp lists: rank of a candidate = candidates ahead of it ----
        // (value desc, position asc is a strict total order: positions are unique).  Each
        // candidate's rank is counted over `parts` disjoint sets of warp lists by different
        // threads, combined with shared-memory atomics; the candidates of rank < nB form the
        // final list.
        {
            const int ncand = kWarps * nB;
            const int parts = kThreads / ncand;  // >= 1 since nB <= 32
            const int c = tid % ncand, part = tid / ncand;
            if (part < parts) {
                const int cw = c / nB, ck = c - (c / nB) * nB;
                const float cv = lv_s[cw * kMaxBands + ck];
                const int cp = lp_s[cw * kMaxBands + ck];
                if (cp >= 0) {
                    int rank = 0;
                    for (int w = part; w < kWarps; w += parts) {
                        const float* vw = lv_s + w * kMaxBands;
                        const int* pw = lp_s + w * kMaxBands;
                        for (int k = 0; k < nB; ++k) {
                            const int op = pw[k];
                            if (op < 0) break;
                            rank += beats(vw[k], op, cv, cp);
                        }
                    }
                    if (rank) atomicAdd(rank_s + c, rank);
                }
            }
            __syncthreads();
            if (part == 0) {
                const int cw = c / nB, ck = c - (c / nB) * nB;
                const float cv = lv_s[cw * kMaxBands + ck];
                const int cp = lp_s[cw * kMaxBands + ck];
                const int rank = rank_s[c];
                if (cp >= 0 && rank < nB) {
                    fin_v[rank] = cv;
                    fin_p[rank] = cp;
                }
            }
            __syncthreads();
        }

        // ---- 7. label: warp 0, one lane per band ----
        if (warp == 0 && lane < nB) {
            int pos = fin_p[lane];
            bool has = pos >= 0;
            int r = 0, c = 0;
            if (has) {
                int i = pos / a.nTheta;
                r = i + a.p0;
                c = (pos - i * a.nTheta) + a.p1;
            }
            float mn = red_f[0];
            float mean = (float)(red_d[0] / (double)stat_count);
            SmemConv acc{conv, a.crow0, a.ccol0, a.CC};
            band_fit_write<float>(has, r, c, acc, mn, mean, a.kc, a.out, (a.out_offset + q) * nB + lane);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
size_t smem_bytes(const FusedGeom& g, size_t store, int k0, int k1, int ngroups) {
    size_t b = ((size_t)(g.row1 - g.row0) * (g.col1 - g.col0) * store + 15) & ~(size_t)15;
    b += ((size_t)(g.crow1 - g.crow0) * (g.ccol1 - g.ccol0) * 4 + 15) & ~(size_t)15;
    b += (size_t)kWarps * kMaxBands * 8 + 32 * 8 + 80 * 4;
    b += (size_t)ngroups * 8 + 2 * (kWarps + 1) * 4;
    b += (size_t)kThreads * 4 + kMaxBands * 8;
    return b;
}

template <typename InT, typename S>
void* kernel_ptr(int k0, int k1) {
    if (k0 == 5 && k1 == 5) return (void*)k_fused<InT, S, 5, 5>;
    if (k0 == 7 && k1 == 7) return (void*)k_fused<InT, S, 7, 7>;
    if (k0 == 9 && k1 == 9) return (void*)k_fused<InT, S, 9, 9>;
    if (k0 == 5 && k1 == 7) return (void*)k_fused<InT, S, 5, 7>;
    if (k0 == 7 && k1 == 5) return (void*)k_fused<InT, S, 7, 5>;
    return nullptr;
}

void* pick_kernel(int method, int dtype, int k0, int k1) {
    bool h = method == EBSD_FUSED_F16;
    switch (dtype) {
        case EBSD_U8: return h ? kernel_ptr<uint8_t, __half>(k0, k1) : kernel_ptr<uint8_t, float>(k0, k1);
        case EBSD_U16: return h ? kernel_ptr<uint16_t, __half>(k0, k1) : kernel_ptr<uint16_t, float>(k0, k1);
        case EBSD_F32: return h ? kernel_ptr<float, __half>(k0, k1) : kernel_ptr<float, float>(k0, k1);
    }
    return nullptr;
}

}  // namespace

int fused_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d) {
    FusedGeom g;
    const int K0 = p->k0, K1 = p->k1;
    // the fused kernel assumes the standard windows: peakPad = 2*ksz + 1 (half-window = ksz)
    bool shape_ok = p->pk0 == 2 * K0 + 1 && p->pk1 == 2 * K1 + 1 && 2 * K1 < 32 &&
                    pick_kernel(EBSD_FUSED_F32, EBSD_U8, K0, K1) != nullptr &&
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
        g.smem_f32 = (int)smem_bytes(g, 4, K0, K1, ngroups);
        g.smem_f16 = (int)smem_bytes(g, 2, K0, K1, ngroups);
        size_t conv_cells = (size_t)(g.crow1 - g.crow0) * (g.ccol1 - g.ccol0);
        int dev_smem = 0;
        cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
        g.ok = conv_cells >= (size_t)p->H * pitch + 1 && g.smem_f16 <= dev_smem && g.row0 >= 0 &&
               (size_t)(g.row1 - g.row0) * (g.col1 - g.col0) < 65535;
        g.ok_f32 = g.ok && g.smem_f32 <= dev_smem;
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
    std::vector<int32_t> gids, wofs(2 * (kWarps + 1), 0);
    for (int w = 0; w < kWarps; ++w) {
        std::sort(wg[w].begin(), wg[w].end());
        wofs[w + 1] = wofs[w] + (int)wg[w].size();
        wofs[kWarps + 1 + w + 1] = wofs[kWarps + 1 + w] + (int)wload[w];
        for (int g : wg[w]) gids.push_back(g);
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
        const int TR = g.row1 - g.row0, TC = g.col1 - g.col0;
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
                    src = (unsigned)((si + p->p0 - g.row0) * TC + (sj + p->p1 - g.col0));
                }
                padlist.push_back((src << 16) | (unsigned)(tr * TC + tc));
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
    std::vector<int32_t> tables(cnt);
    tables.insert(tables.end(), gch.begin(), gch.end());
    tables.insert(tables.end(), gids.begin(), gids.end());
    tables.insert(tables.end(), wofs.begin(), wofs.end());
    EBSD_CUDA_TRY(cudaMalloc((void**)&p->d_fgroup, tables.size() * sizeof(int32_t)));
    EBSD_CUDA_TRY(cudaMemcpy(p->d_fgroup, tables.data(), tables.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    p->flut_entries = (int64_t)lut.size();
    return EBSD_OK;
}

void fused_release(ebsd_plan_s* p) {
    cudaFree(p->d_flut);
    cudaFree(p->d_fgroup);
    cudaFree(p->d_fray);
    cudaFree(p->d_fpad);
    p->d_fpad = nullptr;
    p->d_flut = nullptr;
    p->d_fgroup = nullptr;
    p->d_fray = nullptr;
}

int fused_supported(const ebsd_plan_s* p, int method) {
    if (!p->fg.ok) return 0;
    if (method == EBSD_FUSED_F32) return p->fg.ok_f32;
    return method == EBSD_FUSED_F16;
}

size_t fused_workspace_bytes(const ebsd_plan_s*, int, int64_t) { return 0; }

int fused_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches) {
    if (n <= 0) return EBSD_OK;
    void* fn = pick_kernel(method, dtype, p->k0, p->k1);
    if (!fn) return EBSD_E_UNSUPPORTED;
    const FusedGeom& g = p->fg;
    int smem = method == EBSD_FUSED_F16 ? g.smem_f16 : g.smem_f32;
    EBSD_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int sms = 0, per_sm = 0;
    EBSD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device));
    EBSD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem));
    if (per_sm < 1) return EBSD_E_UNSUPPORTED;
    int64_t grid = std::min<int64_t>(n, (int64_t)sms * per_sm);

    FusedArgs a;
    a.pats = d_pats;
    a.n = n;
    a.H = p->H;
    a.W = p->W;
    a.nPx = p->nPx;
    a.pitch = g.tile_pitch;
    a.lut = (const uint4*)p->d_flut;
    a.count = p->d_fgroup;
    a.gchunks = p->d_fgroup + g.nRaysPad;
    a.gids = a.gchunks + g.nGroups;
    a.wofs = a.gids + g.nGroups;
    a.padlist = p->d_fpad;
    a.npad = g.npad;
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
    a.ksum = g.ksum;
    a.wimg = p->d_fray;
    a.rdnmask = p->d_rdnmask;
    a.bg_mode = p->bg_mode;
    a.bg = p->d_bg;
    a.bgf = p->d_bgf;
    a.kc = LabelConsts{p->p0, p->p1, p->nTheta, p->nRho, p->nB, p->d_theta, p->d_rho};
    a.out = *out;
    a.out_offset = out_offset;
    void* args[] = {&a};
    EBSD_CUDA_TRY(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kThreads), args, (size_t)smem, st));
    *launches += 1;
    return launch_status();
}

}  // namespace ebsd
