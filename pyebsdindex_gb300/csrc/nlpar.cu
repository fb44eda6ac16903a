// NLPAR (non-local pattern averaging) on the device: the noise estimate and the weighted
// neighbour average that run in front of band detection.
//
//   k_nlpar_sigma    NLPAR.sigma_numba, nlpar_cpu.py:753-796 (nn = 1): min over the clipped
//                    3x3 scan neighbourhood of SSD / (2 n), then sqrt
//   k_nlpar_weights  NLPAR.nlpar_nb, nlpar_cpu.py:866-927: normalised pair distance to each
//                    pattern of the (2 sr + 1)^2 window (shifted inward at the scan edges),
//                    weight exp(-max(d - dthresh, 0) / lam^2), centre weight 1, normalised
//   k_nlpar_average  nlpar_cpu.py:929-934: weighted sum over the window for every pixel
//   *_tiled          the same two for 32 neighbouring scan pixels per block, with the patterns
//                    their windows touch staged in shared memory (used for sr <= 3)
//
// The float32 arithmetic keeps the reference's order: squared differences accumulate
// sequentially over the masked-pixel list, window weights are summed and applied in window
// order, and every add/mul is an explicitly rounded intrinsic (no contracted FMAs).
#include "ebsd_internal.cuh"

#include <algorithm>

namespace ebsd {
namespace {

__device__ __forceinline__ void window(int i, int sr, int n, int& start, int& end) {
    int a = i - sr > 0 ? i - sr : 0;
    int b = i + sr - (n - 1) > 0 ? i + sr - (n - 1) : 0;
    start = a - b;
    int c = i + sr < n - 1 ? i + sr : n - 1;
    int e = sr - i > 0 ? sr - i : 0;
    end = c + e + 1;
}

// Sequential float32 SSD over the masked pixels where both values are below mxval.
__device__ __forceinline__ void pair_ssd(const float* __restrict__ a, const float* __restrict__ b,
                                         const int32_t* __restrict__ ind, int nind, float mxval,
                                         float n_init, float& d2, float& n2) {
    float d = 0.0f, n = n_init;
    for (int q = 0; q < nind; ++q) {
        int k = __ldg(ind + q);
        float x = __ldg(a + k), y = __ldg(b + k);
        if (y < mxval && x < mxval) {
            n = __fadd_rn(n, 1.0f);
            float t = __fsub_rn(x, y);
            d = __fadd_rn(d, __fmul_rn(t, t));
        }
    }
    d2 = d;
    n2 = n;
}

// One warp per 4 scan pixels, 8 lanes per pixel (one neighbour each), min over the lanes.
__global__ void k_nlpar_sigma(const float* __restrict__ data, int nrows, int ncols, int npx,
                              const int32_t* __restrict__ ind, int nind, float mxval,
                              float* __restrict__ sigma) {
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int pix = gt >> 3, slot = gt & 7;
    int npix = nrows * ncols;
    float s0 = 1e24f;
    if (pix < npix) {
        int j = pix / ncols, i = pix - (pix / ncols) * ncols;
        int k = slot < 4 ? slot : slot + 1;  // skip the centre of the 3x3 block
        int jn = j + k / 3 - 1, inn = i + k % 3 - 1;
        if (jn >= 0 && jn < nrows && inn >= 0 && inn < ncols) {
            float d2, n2;
            pair_ssd(data + (int64_t)pix * npx, data + (int64_t)(inn + ncols * jn) * npx, ind, nind, mxval,
                     1.0e-12f, d2, n2);
            if (d2 >= 1.e-3f) s0 = __fdiv_rn(d2, __fmul_rn(n2, 2.0f));
        }
    }
    for (int o = 4; o > 0; o >>= 1) s0 = fminf(s0, __shfl_down_sync(0xffffffffu, s0, o, 8));
    if (slot == 0 && pix < npix) sigma[pix] = sqrtf(s0);
}

// One block per scan pixel, one thread per window slot.
__global__ void k_nlpar_weights(const float* __restrict__ data, int nrows, int ncols, int npx,
                                const int32_t* __restrict__ ind, int nind, float mxval,
                                const float* __restrict__ sigma, float lam2, float dthresh, int sr,
                                float* __restrict__ wout, const float* __restrict__ coff = nullptr) {
    extern __shared__ float w_s[];
    __shared__ float tot_s;
    int pix = blockIdx.x;
    int j = pix / ncols, i = pix - (pix / ncols) * ncols;
    int xs, xe, ys, ye;
    window(i, sr, ncols, xs, xe);
    window(j, sr, nrows, ys, ye);
    int wx = xe - xs, winsz = (2 * sr + 1) * (2 * sr + 1);
    int c = threadIdx.x;
    if (c < winsz) {
        int jn = ys + c / wx, inn = xs + c % wx;
        int nb = inn + ncols * jn;
        float w;
        if (nb == pix) {
            w = -1.0e6f;
        } else {
            float s0 = sigma[pix], s1 = sigma[nb];
            s0 = __fmul_rn(s0, s0);
            s1 = __fmul_rn(s1, s1);
            float d2, n2;
            pair_ssd(data + (int64_t)pix * npx, data + (int64_t)nb * npx, ind, nind, mxval, 0.0f, d2, n2);
            float ss = __fadd_rn(s0, s1);
            d2 = __fsub_rn(d2, __fmul_rn(n2, ss));
            float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, n2)));
            w = dnorm > 1.e-8f ? __fdiv_rn(d2, dnorm) : __fmul_rn(1e6f, n2);
        }
        w = fmaxf(__fsub_rn(w, dthresh), 0.0f);
        w = expf(__fmul_rn(__fmul_rn(-1.0f, w), lam2));
        if (coff && nb == pix) w = __fadd_rn(w, coff[pix]);  // diff_offset's centre addition
        w_s[c] = w;
    }
    __syncthreads();
    if (c == 0) {
        float t = 0.0f;
        for (int k = 0; k < winsz; ++k) t = __fadd_rn(t, w_s[k]);
        tot_s = t;
    }
    __syncthreads();
    if (c < winsz) wout[(int64_t)pix * winsz + c] = __fdiv_rn(w_s[c], tot_s);
}

__device__ __forceinline__ float wadd(float acc, float x, float w) { return __fadd_rn(acc, __fmul_rn(x, w)); }
__device__ __forceinline__ double wadd(double acc, double x, double w) { return __dadd_rn(acc, __dmul_rn(x, w)); }

// The averaged value as stored: float as is; an unsigned integer type as the reference's pattern
// writer stores it (pat_flt2int with method 'clip', ebsd_pattern.py:118-182: clipped to the
// type's range, then truncated toward zero by astype).
template <typename O> __device__ __forceinline__ O store_as(float v);
template <> __device__ __forceinline__ float store_as<float>(float v) { return v; }
template <> __device__ __forceinline__ double store_as<double>(float v) { return (double)v; }
template <> __device__ __forceinline__ uint8_t store_as<uint8_t>(float v) {
    return (uint8_t)fminf(fmaxf(v, 0.0f), 255.0f);
}
template <> __device__ __forceinline__ uint16_t store_as<uint16_t>(float v) {
    return (uint16_t)fminf(fmaxf(v, 0.0f), 65535.0f);
}

// out[pix][k] = sum over the window, in window order, of data[nb][k] * w[pix][c].
template <typename T>
__global__ void k_nlpar_average(const T* __restrict__ data, int nrows, int ncols, int npx,
                                const T* __restrict__ w, int sr, T* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int pix = blockIdx.y;
    if (k >= npx) return;
    int j = pix / ncols, i = pix - (pix / ncols) * ncols;
    int xs, xe, ys, ye;
    window(i, sr, ncols, xs, xe);
    window(j, sr, nrows, ys, ye);
    int winsz = (2 * sr + 1) * (2 * sr + 1);
    const T* wp = w + (int64_t)pix * winsz;
    T acc = (T)0;
    int c = 0;
    for (int jn = ys; jn < ye; ++jn)
        for (int inn = xs; inn < xe; ++inn, ++c)
            acc = wadd(acc, __ldg(data + (int64_t)(inn + ncols * jn) * npx + k), __ldg(wp + c));
    out[(int64_t)pix * npx + k] = acc;
}

// The same, stored as O.
template <typename O>
__global__ void k_nlpar_average_to(const float* __restrict__ data, int nrows, int ncols, int npx,
                                   const float* __restrict__ w, int sr, O* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int pix = blockIdx.y;
    if (k >= npx) return;
    int j = pix / ncols, i = pix - (pix / ncols) * ncols;
    int xs, xe, ys, ye;
    window(i, sr, ncols, xs, xe);
    window(j, sr, nrows, ys, ye);
    int winsz = (2 * sr + 1) * (2 * sr + 1);
    const float* wp = w + (int64_t)pix * winsz;
    float acc = 0.0f;
    int c = 0;
    for (int jn = ys; jn < ye; ++jn)
        for (int inn = xs; inn < xe; ++inn, ++c)
            acc = wadd(acc, __ldg(data + (int64_t)(inn + ncols * jn) * npx + k), __ldg(wp + c));
    out[(int64_t)pix * npx + k] = store_as<O>(acc);
}

// ---- tiled kernels: one block per 32 neighbouring scan pixels of one scan row ------------
// The block stages, for a chunk of pixels, the values of every pattern its windows touch
// (2 sr + 1 rows x up to 32 + 4 sr columns of the scan) in shared memory, so that each pattern
// is read from memory once per block instead of once per (pixel, window slot); the per-pair
// and per-output arithmetic is the untiled kernels', in the same order.
constexpr int kTileX = 32;  // scan pixels per block
constexpr int kChunk = 32;  // pixel values per staged pattern per step
constexpr int kSP = kChunk + 1;  // staged row pitch (odd: lanes on different patterns, no conflicts)
constexpr int kTy = 16;     // threadIdx.y extent (blockDim = 32 x 16)

// Scan rows whose windows are shifted inward (rows within sr of the top or bottom edge), and
// columns likewise: their windows reach past +-sr.
__device__ __forceinline__ bool edge_row(int y, int sr, int nrows) { return y < sr || y >= nrows - sr; }
__device__ __forceinline__ bool edge_col(int x, int sr, int ncols) { return x < sr || x >= ncols - sr; }

// Distance weights of NLPAR.nlpar_nb (nlpar_cpu.py:866-927) for window slots c = ty + 16 j.
template <int MP>
__global__ void __launch_bounds__(kTileX * kTy) k_nlpar_weights_tiled(
        const float* __restrict__ data, int nrows, int ncols, int npx, const int32_t* __restrict__ ind,
        int nind, float mxval, const float* __restrict__ sigma, float lam2, float dthresh, int sr,
        float* __restrict__ wout, const float* __restrict__ coff) {
    extern __shared__ float sm[];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTileX + tx;
    const int y = blockIdx.y, x0 = blockIdx.x * kTileX;
    const int wn = 2 * sr + 1, winsz = wn * wn;
    int ys, ye;
    window(y, sr, nrows, ys, ye);
    const int cx0 = x0 - 2 * sr > 0 ? x0 - 2 * sr : 0;
    const int cx1 = x0 + kTileX + 2 * sr < ncols ? x0 + kTileX + 2 * sr : ncols;
    const int ncx = cx1 - cx0, nstage = wn * ncx;
    float* S = sm;                    // [nstage][kSP]
    float* W = sm + nstage * kSP;     // [kTileX][winsz], then [kTileX] totals
    float* T = W + kTileX * winsz;
    const int x = x0 + tx;
    const bool px_ok = x < ncols;
    int xs, xe;
    window(px_ok ? x : ncols - 1, sr, ncols, xs, xe);
    const int pix = y * ncols + (px_ok ? x : ncols - 1);
    const int cslot = (y - ys) * ncx + ((px_ok ? x : ncols - 1) - cx0);
    float d[MP], n[MP];
    int nbs[MP];
#pragma unroll
    for (int j = 0; j < MP; ++j) {
        const int c = ty + kTy * j;
        d[j] = 0.0f;
        n[j] = 0.0f;
        nbs[j] = c < winsz ? (c / wn) * ncx + (xs + c % wn - cx0) : cslot;
    }
    for (int q0 = 0; q0 < nind; q0 += kChunk) {
        const int qn = nind - q0 < kChunk ? nind - q0 : kChunk;
        const int k = tx < qn ? __ldg(ind + q0 + tx) : 0;
        __syncthreads();  // the previous chunk has been consumed
        for (int st = ty; st < nstage; st += kTy) {
            const int r = st / ncx, cc = st - r * ncx;
            const int64_t pat = (int64_t)(ys + r) * ncols + (cx0 + cc);
            S[st * kSP + tx] = tx < qn ? __ldg(data + pat * npx + k) : 0.0f;
        }
        __syncthreads();
        for (int qq = 0; qq < qn; ++qq) {
            const float xv = S[cslot * kSP + qq];
#pragma unroll
            for (int j = 0; j < MP; ++j) {
                const float yv = S[nbs[j] * kSP + qq];
                if (yv < mxval && xv < mxval) {  // pair_ssd's order: count, difference, square
                    n[j] = __fadd_rn(n[j], 1.0f);
                    const float t = __fsub_rn(xv, yv);
                    d[j] = __fadd_rn(d[j], __fmul_rn(t, t));
                }
            }
        }
    }
    // weights (k_nlpar_weights' arithmetic), then the window-order normalisation
#pragma unroll
    for (int j = 0; j < MP; ++j) {
        const int c = ty + kTy * j;
        if (c < winsz && px_ok) {
            const int jn = ys + c / wn, inn = xs + c % wn;
            const int nb = inn + ncols * jn;
            float w;
            if (nb == pix) {
                w = -1.0e6f;
            } else {
                float s0 = sigma[pix], s1 = sigma[nb];
                s0 = __fmul_rn(s0, s0);
                s1 = __fmul_rn(s1, s1);
                const float ss = __fadd_rn(s0, s1);
                const float d2 = __fsub_rn(d[j], __fmul_rn(n[j], ss));
                const float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, n[j])));
                w = dnorm > 1.e-8f ? __fdiv_rn(d2, dnorm) : __fmul_rn(1e6f, n[j]);
            }
            w = fmaxf(__fsub_rn(w, dthresh), 0.0f);
            w = expf(__fmul_rn(__fmul_rn(-1.0f, w), lam2));
            if (coff && nb == pix) w = __fadd_rn(w, coff[pix]);  // diff_offset's centre addition
            W[tx * winsz + c] = w;
        }
    }
    __syncthreads();
    if (ty == 0 && px_ok) {
        float t = 0.0f;
        for (int c = 0; c < winsz; ++c) t = __fadd_rn(t, W[tx * winsz + c]);
        T[tx] = t;
    }
    __syncthreads();
    for (int i = tid; i < kTileX * winsz; i += kTileX * kTy) {
        const int px = i / winsz, c = i - px * winsz;
        if (x0 + px < ncols) wout[(int64_t)(y * ncols + x0 + px) * winsz + c] = __fdiv_rn(W[px * winsz + c], T[px]);
    }
}

// Weighted window sum (k_nlpar_average's order) for 32 scan pixels x 32 pattern pixels per step,
// stored as O (float, or clipped and truncated to uint8 / uint16 -- the detection input).
// SR > 0 fixes the search radius at compile time (unrolled window loops); 0 reads sr.
template <typename T, typename O, int SR>
__global__ void __launch_bounds__(kTileX * kTy) k_nlpar_average_tiled(
        const T* __restrict__ data, int nrows, int ncols, int npx, const T* __restrict__ w, int sr_arg,
        O* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sm = (T*)smraw;
    const int sr = SR > 0 ? SR : sr_arg;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTileX + tx;
    const int y = blockIdx.y, x0 = blockIdx.x * kTileX;
    const int wn = 2 * sr + 1, winsz = wn * wn;
    int ys, ye;
    window(y, sr, nrows, ys, ye);
    const int cx0 = x0 - 2 * sr > 0 ? x0 - 2 * sr : 0;
    const int cx1 = x0 + kTileX + 2 * sr < ncols ? x0 + kTileX + 2 * sr : ncols;
    const int ncx = cx1 - cx0;
    T* S = sm;                      // [wn rows][ncx][kSP]
    // [kTileX][WP]: each pixel's weights at a 16-byte aligned row of WP = winsz rounded up to 4,
    // read four at a time (one broadcast load for four window slots)
    const int WP = (winsz + 3) & ~3;
    T* Wt = sm + ((wn * ncx * kSP + 3) & ~3);
    const int npix_tile = ncols - x0 < kTileX ? ncols - x0 : kTileX;
    for (int i = tid; i < npix_tile * winsz; i += kTileX * kTy)
        Wt[(i / winsz) * WP + i % winsz] = w[(int64_t)(y * ncols + x0) * winsz + i];
    // this thread's scan pixels: the neighbours px = 2 ty + m (kTileX = 2 kTy), and their
    // windows' first staged column
    constexpr int kPx = kTileX / kTy;
    int xsc[kPx];
#pragma unroll
    for (int m = 0; m < kPx; ++m) {
        const int px = kPx * ty + m;
        int xs, xe;
        window(px < npix_tile ? x0 + px : x0, sr, ncols, xs, xe);
        xsc[m] = xs - cx0;
    }
    // neighbouring windows one column apart share all but one column of staged values
    const bool shared_cols = SR > 0 && kPx == 2 && kPx * ty + 1 < npix_tile && xsc[1] == xsc[0] + 1;
    for (int k0 = 0; k0 < npx; k0 += kChunk) {
        const int kn = npx - k0 < kChunk ? npx - k0 : kChunk;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < (SR > 0 ? 2 * SR + 1 : 1); ++r) {
            const int rr0 = SR > 0 ? r : 0, rr1 = SR > 0 ? r + 1 : wn;
            for (int rr = rr0; rr < rr1; ++rr) {
                const int64_t prow = (int64_t)(ys + rr) * ncols + cx0;
                for (int cc = ty; cc < ncx; cc += kTy)
                    S[(rr * ncx + cc) * kSP + tx] = tx < kn ? data[(prow + cc) * npx + k0 + tx] : (T)0;
            }
        }
        __syncthreads();
        if (tx >= kn) continue;
        if (SR > 0 && shared_cols) {
            // both pixels at once: each staged value loaded once for the two sums
            constexpr int WN = 2 * SR + 1, WS = WN * WN;
            const T* s0 = S + xsc[0] * kSP + tx;
            const T* wpa = Wt + (kPx * ty) * WP;
            const T* wpb = wpa + WP;
            T acc0 = (T)0, acc1 = (T)0;
#pragma unroll
            for (int c4 = 0; c4 < WS; c4 += 4) {
                T wa[4], wb[4];
                if (sizeof(T) == 4) {
                    const float4 a4 = *(const float4*)(wpa + c4), b4 = *(const float4*)(wpb + c4);
                    wa[0] = a4.x; wa[1] = a4.y; wa[2] = a4.z; wa[3] = a4.w;
                    wb[0] = b4.x; wb[1] = b4.y; wb[2] = b4.z; wb[3] = b4.w;
                } else {
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        wa[t] = c4 + t < WS ? wpa[c4 + t] : (T)0;
                        wb[t] = c4 + t < WS ? wpb[c4 + t] : (T)0;
                    }
                }
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int c = c4 + t;
                    if (c < WS) {
                        const int r = c / WN, cc = c % WN;
                        acc0 = wadd(acc0, s0[(r * ncx + cc) * kSP], wa[t]);
                        acc1 = wadd(acc1, s0[(r * ncx + cc + 1) * kSP], wb[t]);
                    }
                }
            }
            const int64_t o = (int64_t)(y * ncols + x0 + kPx * ty) * npx + k0 + tx;
            out[o] = store_as<O>(acc0);
            out[o + npx] = store_as<O>(acc1);
            continue;
        }
#pragma unroll
        for (int m = 0; m < kPx; ++m) {
            const int px = kPx * ty + m;
            if (px < npix_tile) {
                const T* wp = Wt + px * WP;
                T acc = (T)0;
                int c = 0;
                for (int r = 0; r < wn; ++r) {
                    const T* srow = S + (r * ncx + xsc[m]) * kSP + tx;
                    for (int cc = 0; cc < wn; ++cc, ++c) acc = wadd(acc, srow[cc * kSP], wp[c]);
                }
                out[(int64_t)(y * ncols + x0 + px) * npx + k0 + tx] = store_as<O>(acc);
            }
        }
    }
}

template <typename T, typename O>
void launch_average_tiled(dim3 grid, dim3 block, size_t smem, cudaStream_t st, const T* data, int nrows, int ncols,
                          int npx, const T* w, int sr, O* out) {
    switch (sr) {
        case 1: k_nlpar_average_tiled<T, O, 1><<<grid, block, smem, st>>>(data, nrows, ncols, npx, w, sr, out); break;
        case 2: k_nlpar_average_tiled<T, O, 2><<<grid, block, smem, st>>>(data, nrows, ncols, npx, w, sr, out); break;
        case 3: k_nlpar_average_tiled<T, O, 3><<<grid, block, smem, st>>>(data, nrows, ncols, npx, w, sr, out); break;
        default: k_nlpar_average_tiled<T, O, 0><<<grid, block, smem, st>>>(data, nrows, ncols, npx, w, sr, out);
    }
}

// Weighted window sum, register-blocked along the scan row (search radius SR fixed).  A block
// takes RP neighbouring scan pixels of one row and 4 * kRbThreads pattern values; each thread
// holds the RP pixels' sums for four consecutive pattern values and streams the window rows'
// RP + 2 SR columns once: a loaded value feeds every pixel whose window holds its column, and a
// broadcast weight feeds the four values.  Each sum adds its window slots in window order
// (rows, then columns) as fadd(acc, fmul(value, weight)) from zero -- the order and rounding of
// k_nlpar_average -- so the result equals the tiled kernel's bit for bit.  Needs npx % 4 == 0
// and 16-byte aligned data.
constexpr int kRbThreads = 128;
constexpr int kRbPix = 8;

template <typename O> __device__ __forceinline__ void store4(O* dst, const float* v);
template <> __device__ __forceinline__ void store4<float>(float* dst, const float* v) {
    *(float4*)dst = make_float4(v[0], v[1], v[2], v[3]);
}
template <> __device__ __forceinline__ void store4<uint8_t>(uint8_t* dst, const float* v) {
    *(uint32_t*)dst = (uint32_t)store_as<uint8_t>(v[0]) | ((uint32_t)store_as<uint8_t>(v[1]) << 8) |
                      ((uint32_t)store_as<uint8_t>(v[2]) << 16) | ((uint32_t)store_as<uint8_t>(v[3]) << 24);
}
template <> __device__ __forceinline__ void store4<uint16_t>(uint16_t* dst, const float* v) {
    *(uint2*)dst = make_uint2((uint32_t)store_as<uint16_t>(v[0]) | ((uint32_t)store_as<uint16_t>(v[1]) << 16),
                              (uint32_t)store_as<uint16_t>(v[2]) | ((uint32_t)store_as<uint16_t>(v[3]) << 16));
}

template <typename O, int SR>
__global__ void __launch_bounds__(kRbThreads) k_nlpar_average_rb(const float* __restrict__ data, int nrows, int ncols,
                                                                  int npx, const float* __restrict__ w,
                                                                  O* __restrict__ out) {
    constexpr int WN = 2 * SR + 1, WS = WN * WN, RP = kRbPix, NC = RP + 2 * SR;
    __shared__ float ws[RP * WS];
    const int y = blockIdx.z, p0 = blockIdx.y * RP;
    const int np = ncols - p0 < RP ? ncols - p0 : RP;
    for (int i = threadIdx.x; i < np * WS; i += kRbThreads) ws[i] = w[(int64_t)(y * ncols + p0) * WS + i];
    __syncthreads();
    const int k = (blockIdx.x * kRbThreads + threadIdx.x) * 4;
    if (k >= npx) return;
    int ys, ye;
    window(y, SR, nrows, ys, ye);
    float acc[RP][4];
#pragma unroll
    for (int m = 0; m < RP; ++m)
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[m][t] = 0.0f;
    if (p0 >= SR && p0 + RP + SR <= ncols) {
        // every window of the block is centred: column j of the strip is slot j - m of pixel m
#pragma unroll
        for (int r = 0; r < WN; ++r) {
            const float* src = data + ((int64_t)(ys + r) * ncols + (p0 - SR)) * npx + k;
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                const float4 v = __ldg((const float4*)(src + (int64_t)j * npx));
#pragma unroll
                for (int m = 0; m < RP; ++m) {
                    if (j - m >= 0 && j - m < WN) {
                        const float wv = ws[m * WS + r * WN + (j - m)];
                        acc[m][0] = wadd(acc[m][0], v.x, wv);
                        acc[m][1] = wadd(acc[m][1], v.y, wv);
                        acc[m][2] = wadd(acc[m][2], v.z, wv);
                        acc[m][3] = wadd(acc[m][3], v.w, wv);
                    }
                }
            }
        }
    } else {
        // windows shifted inward at the scan's left / right edge: window starts from window()
        int xs[RP];
#pragma unroll
        for (int m = 0; m < RP; ++m) {
            int xe;
            window(m < np ? p0 + m : p0 + np - 1, SR, ncols, xs[m], xe);
        }
        const int c0 = xs[0], c1 = xs[np - 1] + 2 * SR;  // window starts do not decrease with m
#pragma unroll
        for (int r = 0; r < WN; ++r) {
            const float* src = data + (int64_t)(ys + r) * ncols * npx + k;
            for (int c = c0; c <= c1; ++c) {
                const float4 v = __ldg((const float4*)(src + (int64_t)c * npx));
#pragma unroll
                for (int m = 0; m < RP; ++m) {
                    const int d = c - xs[m];
                    if (m < np && d >= 0 && d < WN) {
                        const float wv = ws[m * WS + r * WN + d];
                        acc[m][0] = wadd(acc[m][0], v.x, wv);
                        acc[m][1] = wadd(acc[m][1], v.y, wv);
                        acc[m][2] = wadd(acc[m][2], v.z, wv);
                        acc[m][3] = wadd(acc[m][3], v.w, wv);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int m = 0; m < RP; ++m)
        if (m < np) store4<O>(out + (int64_t)(y * ncols + p0 + m) * npx + k, acc[m]);
}

// The weighted window sum of the pair path: the register-blocked kernel where it applies
// (radius 1-3, npx a multiple of 4, 16-byte aligned buffers), else the tiled kernel.
template <typename O>
void launch_average(dim3 tgrid, dim3 tblock, size_t tsmem, cudaStream_t st, const float* data, int nrows, int ncols,
                    int npx, const float* w, int sr, O* out) {
    const bool rb = sr >= 1 && sr <= 3 && npx % 4 == 0 && (uintptr_t)data % 16 == 0 && (uintptr_t)out % 16 == 0 &&
                    nrows <= 65535 && (ncols + kRbPix - 1) / kRbPix <= 65535;  // grid y / z limits
    if (!rb) {
        launch_average_tiled<float, O>(tgrid, tblock, tsmem, st, data, nrows, ncols, npx, w, sr, out);
        return;
    }
    const dim3 grid((unsigned)((npx / 4 + kRbThreads - 1) / kRbThreads), (unsigned)((ncols + kRbPix - 1) / kRbPix),
                    (unsigned)nrows);
    switch (sr) {
        case 1: k_nlpar_average_rb<O, 1><<<grid, kRbThreads, 0, st>>>(data, nrows, ncols, npx, w, out); break;
        case 2: k_nlpar_average_rb<O, 2><<<grid, kRbThreads, 0, st>>>(data, nrows, ncols, npx, w, out); break;
        default: k_nlpar_average_rb<O, 3><<<grid, kRbThreads, 0, st>>>(data, nrows, ncols, npx, w, out); break;
    }
}

// ---- pair kernels: each unordered pair's distance computed once ---------------------------
// The squared difference of a pair is symmetric bit for bit ((a - b)^2 == (b - a)^2 in float,
// and the saturation test is symmetric), so pixel p's distance to neighbour q is the same
// float sum whichever of the two computes it.  k_nlpar_pairs computes, for every scan pixel,
// the sums of the nF = sr (2 sr + 1) + sr "forward" offsets (dy, dx) -- dy > 0, or dy == 0 and
// dx > 0, |dy|, |dx| <= sr -- in the reference's pixel order; a pixel's window slot at offset
// -o reads the sum its neighbour computed for o.  Slots beyond +-sr, which only the windows
// shifted inward at the scan edges have, are summed directly from memory.  With kSig the
// kernel also sums the four forward 3x3 neighbours under sigma_numba's saturation level, from
// which k_nlpar_sigma_pairs takes the noise sigma without another pass over the patterns.
constexpr int kPairTy = 8;  // threadIdx.y extent of k_nlpar_pairs (blockDim = 32 x 8)

__device__ __forceinline__ int fwd_count(int sr) { return sr * (2 * sr + 1) + sr; }
__device__ __forceinline__ void fwd_offset(int f, int sr, int& dy, int& dx) {
    if (f < sr) {
        dy = 0;
        dx = f + 1;
    } else {
        const int g = f - sr, w = 2 * sr + 1;
        dy = 1 + g / w;
        dx = g - (dy - 1) * w - sr;
    }
}
__device__ __forceinline__ int fwd_index(int dy, int dx, int sr) {
    return dy == 0 ? dx - 1 : sr + (dy - 1) * (2 * sr + 1) + (dx + sr);
}

template <int MPF, bool kSig>
__global__ void __launch_bounds__(kTileX * kPairTy) k_nlpar_pairs(
        const float* __restrict__ data, int nrows, int ncols, int npx, const int32_t* __restrict__ ind,
        int nind, float mxval, float mxsig, int sr, float2* __restrict__ pairs, float2* __restrict__ sigp) {
    extern __shared__ float sm[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int y = blockIdx.y, x0 = blockIdx.x * kTileX;
    const int nF = fwd_count(sr);
    const int nr = (y + sr < nrows ? y + sr : nrows - 1) - y + 1;  // staged scan rows y .. y + nr - 1
    const int cx0 = x0 - sr > 0 ? x0 - sr : 0;
    const int cx1 = x0 + kTileX + sr < ncols ? x0 + kTileX + sr : ncols;
    const int ncx = cx1 - cx0;
    float* S = sm;  // [nr][ncx][kSP]
    const int x = x0 + tx;
    const bool px_ok = x < ncols;
    const int self = (px_ok ? x : ncols - 1) - cx0;
    int slot[MPF];
    bool ok[MPF];
#pragma unroll
    for (int j = 0; j < MPF; ++j) {
        const int f = ty + kPairTy * j;
        int dy = 0, dx = 0;
        if (f < nF) fwd_offset(f, sr, dy, dx);
        ok[j] = px_ok && f < nF && x + dx >= 0 && x + dx < ncols && y + dy < nrows;
        slot[j] = ok[j] ? dy * ncx + (x + dx - cx0) : self;
    }
    // sigma's four forward 3x3 neighbours sit at f = 0, 2 sr - 1, 2 sr, 2 sr + 1 (warp-uniform ty)
    const int sk = ty == 0 ? 0 : (ty == 2 * sr - 1 ? 1 : (ty == 2 * sr ? 2 : (ty == 2 * sr + 1 ? 3 : -1)));
    const bool near = kSig && sk >= 0 && ok[0];
    float d[MPF], n[MPF], ds = 0.0f, ns = 0.0f;
#pragma unroll
    for (int j = 0; j < MPF; ++j) {
        d[j] = 0.0f;
        n[j] = 0.0f;
    }
    for (int q0 = 0; q0 < nind; q0 += kChunk) {
        const int qn = nind - q0 < kChunk ? nind - q0 : kChunk;
        const int k = tx < qn ? __ldg(ind + q0 + tx) : 0;
        __syncthreads();  // the previous chunk has been consumed
        int bad = 0, bad_sig = 0;  // a staged value at or above a saturation level
        for (int r = 0; r < nr; ++r) {
            const float* prow = data + ((int64_t)(y + r) * ncols + cx0) * npx + k;
            float* srow = S + r * ncx * kSP + tx;
            for (int cc = ty; cc < ncx; cc += kPairTy) {
                const float v = tx < qn ? __ldg(prow + (int64_t)cc * npx) : 0.0f;
                bad |= !(v < mxval);
                if (kSig) bad_sig |= !(v < mxsig);
                srow[cc * kSP] = v;
            }
        }
        const int any_bad = __syncthreads_or(bad);
        const int any_bad_sig = kSig ? __syncthreads_or(bad_sig) : 0;
        if (any_bad == 0 && any_bad_sig == 0) {
            // every term of the chunk counts: the squares added without the tests, the chunk
            // counted whole (the counts are exact integers either way)
            for (int qq = 0; qq < qn; ++qq) {
                const float xv = S[self * kSP + qq];
#pragma unroll
                for (int j = 0; j < MPF; ++j) {
                    const float t = __fsub_rn(xv, S[slot[j] * kSP + qq]);
                    const float tt = __fmul_rn(t, t);
                    d[j] = __fadd_rn(d[j], tt);
                    if (kSig && j == 0 && near) ds = __fadd_rn(ds, tt);
                }
            }
#pragma unroll
            for (int j = 0; j < MPF; ++j) n[j] = __fadd_rn(n[j], (float)qn);
            if (kSig && near) ns = __fadd_rn(ns, (float)qn);
            continue;
        }
        for (int qq = 0; qq < qn; ++qq) {
            const float xv = S[self * kSP + qq];
#pragma unroll
            for (int j = 0; j < MPF; ++j) {
                const float yv = S[slot[j] * kSP + qq];
                if (yv < mxval && xv < mxval) {  // pair_ssd's order: count, difference, square
                    n[j] = __fadd_rn(n[j], 1.0f);
                    const float t = __fsub_rn(xv, yv);
                    d[j] = __fadd_rn(d[j], __fmul_rn(t, t));
                }
                if (kSig && j == 0 && near && yv < mxsig && xv < mxsig) {
                    ns = __fadd_rn(ns, 1.0f);
                    const float t = __fsub_rn(xv, yv);
                    ds = __fadd_rn(ds, __fmul_rn(t, t));
                }
            }
        }
    }
    const int64_t pix = (int64_t)y * ncols + x;
#pragma unroll
    for (int j = 0; j < MPF; ++j)
        if (ok[j]) pairs[pix * nF + ty + kPairTy * j] = make_float2(d[j], n[j]);
    if (near) sigp[pix * 4 + sk] = make_float2(ds, ns);
}

// sigma_numba (nn = 1) from the pair sums: min over the clipped 3x3 neighbourhood of
// SSD / (2 n) for SSD >= 1e-3 (the count starts at 1e-12, which the first add absorbs).
__global__ void k_nlpar_sigma_pairs(const float2* __restrict__ sigp, int nrows, int ncols, float* __restrict__ sigma) {
    const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (int64_t)nrows * ncols) return;
    const int j = (int)(pix / ncols), i = (int)(pix - (int64_t)j * ncols);
    // forward 3x3 offsets in sigp order, and their mirrors
    const int fdy[4] = {0, 1, 1, 1}, fdx[4] = {1, -1, 0, 1};
    float s0 = 1e24f;
    for (int k = 0; k < 8; ++k) {
        const int kk = k & 3;
        const int dy = k < 4 ? fdy[kk] : -fdy[kk], dx = k < 4 ? fdx[kk] : -fdx[kk];
        const int jn = j + dy, inn = i + dx;
        if (jn < 0 || jn >= nrows || inn < 0 || inn >= ncols) continue;
        const float2 e = k < 4 ? sigp[pix * 4 + kk] : sigp[((int64_t)jn * ncols + inn) * 4 + kk];
        const float n2 = e.y > 0.0f ? e.y : 1.0e-12f;
        if (e.x >= 1.e-3f) s0 = fminf(s0, __fdiv_rn(e.x, __fmul_rn(n2, 2.0f)));
    }
    sigma[pix] = sqrtf(s0);
}

// The window weights of k_nlpar_weights_tiled from the pair sums (slots c = ty + 16 j), for the
// pixels whose windows are centred; the edge pixels take k_nlpar_weights_edge.
template <int MP>
__global__ void __launch_bounds__(kTileX * kTy) k_nlpar_weights_pairs(
        const float* __restrict__ data, int nrows, int ncols, int npx, const int32_t* __restrict__ ind,
        int nind, float mxval, const float2* __restrict__ pairs, const float* __restrict__ sigma, float lam2,
        float dthresh, int sr, float* __restrict__ wout, const float* __restrict__ coff) {
    __shared__ float W[kTileX * 49];
    __shared__ float T[kTileX];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTileX + tx;
    const int y = blockIdx.y, x0 = blockIdx.x * kTileX;
    if (edge_row(y, sr, nrows)) return;
    const int wn = 2 * sr + 1, winsz = wn * wn, nF = fwd_count(sr);
    int ys, ye;
    window(y, sr, nrows, ys, ye);
    const int x = x0 + tx;
    const bool px_ok = x < ncols && !edge_col(x, sr, ncols);
    int xs, xe;
    window(x < ncols ? x : ncols - 1, sr, ncols, xs, xe);
    const int64_t pix = (int64_t)y * ncols + (x < ncols ? x : ncols - 1);
#pragma unroll
    for (int j = 0; j < MP; ++j) {
        const int c = ty + kTy * j;
        if (c < winsz && px_ok) {
            const int jn = ys + c / wn, inn = xs + c % wn;
            const int64_t nb = (int64_t)jn * ncols + inn;
            const int dy = jn - y, dx = inn - x;
            float w;
            if (nb == pix) {
                w = -1.0e6f;
            } else {
                float d2, n2;
                if (dy >= -sr && dy <= sr && dx >= -sr && dx <= sr) {
                    const float2 e = (dy > 0 || (dy == 0 && dx > 0)) ? pairs[pix * nF + fwd_index(dy, dx, sr)]
                                                                    : pairs[nb * nF + fwd_index(-dy, -dx, sr)];
                    d2 = e.x;
                    n2 = e.y;
                } else {  // (not reached: the windows of these blocks are centred)
                    pair_ssd(data + pix * npx, data + nb * npx, ind, nind, mxval, 0.0f, d2, n2);
                }
                float s0 = sigma[pix], s1 = sigma[nb];
                s0 = __fmul_rn(s0, s0);
                s1 = __fmul_rn(s1, s1);
                const float ss = __fadd_rn(s0, s1);
                d2 = __fsub_rn(d2, __fmul_rn(n2, ss));
                const float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, n2)));
                w = dnorm > 1.e-8f ? __fdiv_rn(d2, dnorm) : __fmul_rn(1e6f, n2);
            }
            w = fmaxf(__fsub_rn(w, dthresh), 0.0f);
            w = expf(__fmul_rn(__fmul_rn(-1.0f, w), lam2));
            if (coff && nb == pix) w = __fadd_rn(w, coff[pix]);  // diff_offset's centre addition
            W[tx * winsz + c] = w;
        }
    }
    __syncthreads();
    if (ty == 0 && px_ok) {
        float t = 0.0f;
        for (int c = 0; c < winsz; ++c) t = __fadd_rn(t, W[tx * winsz + c]);
        T[tx] = t;
    }
    __syncthreads();
    for (int i = tid; i < kTileX * winsz; i += kTileX * kTy) {
        const int px = i / winsz, c = i - px * winsz;
        if (x0 + px < ncols && !edge_col(x0 + px, sr, ncols))
            wout[((int64_t)y * ncols + x0 + px) * winsz + c] = __fdiv_rn(W[px * winsz + c], T[px]);
    }
}

// ---- edge pixels: windows shifted inward, reaching past +-sr ----------------------------------
// Edge pixels are those of the sr top and bottom rows, and the sr left and right columns of the
// other rows; index: top rows, bottom rows, then per middle row its 2 sr edge columns.  Their
// raw window sums (SSD, count per slot, in the reference's pixel order) are computed by two
// kernels that split the slots over many blocks, then k_nlpar_weights_edge turns them into
// normalised weights, one block per edge pixel.
__device__ __forceinline__ int64_t edge_index(int y, int x, int sr, int nrows, int ncols) {
    if (y < sr) return (int64_t)y * ncols + x;
    if (y >= nrows - sr) return (int64_t)(sr + y - (nrows - sr)) * ncols + x;
    return (int64_t)2 * sr * ncols + (int64_t)(y - sr) * 2 * sr + (x < sr ? x : sr + x - (ncols - sr));
}

// Edge rows: blockIdx.y picks the row (the sr top rows, then the sr bottom rows), blockIdx.x 32
// neighbouring pixels (one per lane), blockIdx.z a range of kTy window slots (one per thread row).
// All pixels of the row share the window rows; the patterns of those rows in the columns the
// block's windows touch are staged.
__global__ void __launch_bounds__(kTileX * kTy) k_nlpar_edge_rows(
        const float* __restrict__ data, int nrows, int ncols, int npx, const int32_t* __restrict__ ind, int nind,
        float mxval, int sr, float2* __restrict__ raw) {
    extern __shared__ float sm[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int wn = 2 * sr + 1, winsz = wn * wn;
    const int y = blockIdx.y < sr ? blockIdx.y : nrows - 2 * sr + blockIdx.y;
    const int x0 = blockIdx.x * kTileX;
    int ys, ye;
    window(y, sr, nrows, ys, ye);
    const int cx0 = x0 - 2 * sr > 0 ? x0 - 2 * sr : 0;
    const int cx1 = x0 + kTileX + 2 * sr < ncols ? x0 + kTileX + 2 * sr : ncols;
    const int ncx = cx1 - cx0;
    float* S = sm;  // [wn][ncx][kSP]
    const int x = x0 + tx;
    const int c = blockIdx.z * kTy + ty;
    const bool ok = x < ncols && c < winsz;
    int xs, xe;
    window(x < ncols ? x : ncols - 1, sr, ncols, xs, xe);
    const int self = (y - ys) * ncx + ((x < ncols ? x : ncols - 1) - cx0);
    const int nbs = ok ? (c / wn) * ncx + (xs + c % wn - cx0) : self;
    float d = 0.0f, n = 0.0f;
    for (int q0 = 0; q0 < nind; q0 += kChunk) {
        const int qn = nind - q0 < kChunk ? nind - q0 : kChunk;
        const int k = tx < qn ? __ldg(ind + q0 + tx) : 0;
        __syncthreads();
        for (int r = 0; r < wn; ++r) {
            const float* prow = data + ((int64_t)(ys + r) * ncols + cx0) * npx + k;
            float* srow = S + r * ncx * kSP + tx;
            for (int cc = ty; cc < ncx; cc += kTy) srow[cc * kSP] = tx < qn ? __ldg(prow + (int64_t)cc * npx) : 0.0f;
        }
        __syncthreads();
        for (int qq = 0; qq < qn; ++qq) {
            const float xv = S[self * kSP + qq], yv = S[nbs * kSP + qq];
            if (yv < mxval && xv < mxval) {  // pair_ssd's order: count, difference, square
                n = __fadd_rn(n, 1.0f);
                const float t = __fsub_rn(xv, yv);
                d = __fadd_rn(d, __fmul_rn(t, t));
            }
        }
    }
    if (ok) raw[edge_index(y, x, sr, nrows, ncols) * winsz + c] = make_float2(d, n);
}

// Edge columns of the middle rows: blockIdx.y the side, blockIdx.x 32 neighbouring rows (one per
// lane), blockIdx.z a range of kTy (edge column, window slot) combinations.  All edge pixels of
// one side share the window columns [0, 2 sr] (or the last 2 sr + 1).
__global__ void __launch_bounds__(kTileX * kTy) k_nlpar_edge_cols(
        const float* __restrict__ data, int nrows, int ncols, int npx, const int32_t* __restrict__ ind, int nind,
        float mxval, int sr, float2* __restrict__ raw) {
    extern __shared__ float sm[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int wn = 2 * sr + 1, winsz = wn * wn;
    const int nri = nrows - 2 * sr;
    const int y0 = sr + blockIdx.x * kTileX;
    const int nrow = nri - blockIdx.x * kTileX < kTileX ? nri - blockIdx.x * kTileX : kTileX;
    const int side = blockIdx.y;
    const int colbase = side ? ncols - wn : 0;
    const int xe0 = side ? ncols - sr : 0;
    const int nrs = nrow + 2 * sr;
    float* S = sm;  // [nrs][wn][kSP]
    const int idx = blockIdx.z * kTy + ty;
    const bool ok = tx < nrow && idx < sr * winsz;
    const int e = ok ? idx / winsz : 0, c = ok ? idx - e * winsz : 0;
    const int self = ((ok ? tx : 0) + sr) * wn + (xe0 + e - colbase);
    const int nbs = ok ? (tx + c / wn) * wn + c % wn : self;
    float d = 0.0f, n = 0.0f;
    for (int q0 = 0; q0 < nind; q0 += kChunk) {
        const int qn = nind - q0 < kChunk ? nind - q0 : kChunk;
        const int k = tx < qn ? __ldg(ind + q0 + tx) : 0;
        __syncthreads();
        for (int r = ty; r < nrs; r += kTy) {
            const float* prow = data + ((int64_t)(y0 - sr + r) * ncols + colbase) * npx + k;
            float* srow = S + r * wn * kSP + tx;
            for (int cc = 0; cc < wn; ++cc) srow[cc * kSP] = tx < qn ? __ldg(prow + (int64_t)cc * npx) : 0.0f;
        }
        __syncthreads();
        for (int qq = 0; qq < qn; ++qq) {
            const float xv = S[self * kSP + qq], yv = S[nbs * kSP + qq];
            if (yv < mxval && xv < mxval) {  // pair_ssd's order: count, difference, square
                n = __fadd_rn(n, 1.0f);
                const float t = __fsub_rn(xv, yv);
                d = __fadd_rn(d, __fmul_rn(t, t));
            }
        }
    }
    if (ok) raw[edge_index(y0 + tx, xe0 + e, sr, nrows, ncols) * winsz + c] = make_float2(d, n);
}

// Normalised window weights of the edge pixels from their raw sums: one block (64 threads) per
// edge pixel, the arithmetic of k_nlpar_weights_tiled.
__global__ void k_nlpar_weights_edge(const float2* __restrict__ raw, int nrows, int ncols, int sr,
                                     const float* __restrict__ sigma, float lam2, float dthresh,
                                     float* __restrict__ wout, const float* __restrict__ coff) {
    __shared__ float W[64];
    __shared__ float T;
    const int wn = 2 * sr + 1, winsz = wn * wn;
    const int64_t b = blockIdx.x;
    // edge index -> pixel
    int y, x;
    const int64_t top = (int64_t)sr * ncols;
    if (b < 2 * top) {
        const int64_t r = b / ncols;
        y = (int)(r < sr ? r : nrows - 2 * sr + r);
        x = (int)(b - r * ncols);
    } else {
        const int64_t m = b - 2 * top;
        y = sr + (int)(m / (2 * sr));
        const int e = (int)(m - (int64_t)(y - sr) * 2 * sr);
        x = e < sr ? e : ncols - 2 * sr + e;
    }
    int ys, ye, xs, xe;
    window(y, sr, nrows, ys, ye);
    window(x, sr, ncols, xs, xe);
    const int64_t pix = (int64_t)y * ncols + x;
    const int c = threadIdx.x;
    if (c < winsz) {
        const int64_t nb = (int64_t)(ys + c / wn) * ncols + (xs + c % wn);
        float w;
        if (nb == pix) {
            w = -1.0e6f;
        } else {
            const float2 e2 = raw[b * winsz + c];
            float s0 = sigma[pix], s1 = sigma[nb];
            s0 = __fmul_rn(s0, s0);
            s1 = __fmul_rn(s1, s1);
            const float ss = __fadd_rn(s0, s1);
            const float d2 = __fsub_rn(e2.x, __fmul_rn(e2.y, ss));
            const float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, e2.y)));
            w = dnorm > 1.e-8f ? __fdiv_rn(d2, dnorm) : __fmul_rn(1e6f, e2.y);
        }
        w = fmaxf(__fsub_rn(w, dthresh), 0.0f);
        w = expf(__fmul_rn(__fmul_rn(-1.0f, w), lam2));
        if (coff && nb == pix) w = __fadd_rn(w, coff[pix]);  // diff_offset's centre addition
        W[c] = w;
    }
    __syncthreads();
    if (c == 0) {
        float t = 0.0f;
        for (int k = 0; k < winsz; ++k) t = __fadd_rn(t, W[k]);
        T = t;
    }
    __syncthreads();
    if (c < winsz) wout[pix * winsz + c] = __fdiv_rn(W[c], T);
}

size_t edge_rows_smem(int sr, int ncols) {
    const int ncx = std::min(ncols, kTileX + 4 * sr);
    return (size_t)(2 * sr + 1) * ncx * kSP * sizeof(float);
}
size_t edge_cols_smem(int sr) { return (size_t)(kTileX + 2 * sr) * (2 * sr + 1) * kSP * sizeof(float); }

size_t pairs_smem(int sr, int ncols) {
    const int ncx = std::min(ncols, kTileX + 2 * sr);
    return (size_t)(sr + 1) * ncx * kSP * sizeof(float);
}

size_t tiled_smem(int sr, int ncols, size_t elem, bool weights) {
    const int wn = 2 * sr + 1;
    const int ncx = std::min(ncols, kTileX + 4 * sr);
    // staged rows (rounded up to 4 elements), then the pixels' weights at rows of winsz
    // rounded up to 4
    size_t b = (((size_t)wn * ncx * kSP + 3) & ~(size_t)3) * elem + (size_t)kTileX * ((wn * wn + 3) & ~3) * elem;
    if (weights) b += kTileX * sizeof(float);
    return b;
}


// ---- lambda optimisation (NLPAR.opt_lambda_cpu, nlpar_cpu.py:94-155) -------------------
// calcsigma_cpu (nlpar_cpu.py:157-264) runs sigma_numba per scan tile with nn and the tile's
// start/count arrays as uint64, so `j - nn` wraps for the tile's first row and first column:
// those pixels get an empty window (sigma sqrt(1e24), no distances).  Every other pixel gets
// its clipped 3x3 window in row-major slot order (centre: count = pattern length, distance 0);
// the distances are normalised with the tile's own sigma (nlpar_cpu.py:805-817), then merged
// into the scan: sigma = min over tiles, a slot's distance and count replaced where the tile's
// count is positive.

__device__ __forceinline__ uint32_t fmax_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fmax_unkey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// largest value of the tile's patterns (np.max(data) of the tile)
__global__ void k_tile_max(const float* __restrict__ data, int ncols, int npx, int r0, int c0, int tr, int tc,
                           uint32_t* __restrict__ key) {
    const int64_t total = (int64_t)tr * tc * npx;
    float m = -INFINITY;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pix = t / npx;
        const int q = (int)(t - pix * npx);
        const int j = (int)(pix / tc), i = (int)(pix - (int64_t)j * tc);
        m = fmaxf(m, __ldg(data + ((int64_t)(r0 + j) * ncols + (c0 + i)) * npx + q));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(key, fmax_key(m));
}

// raw distances and counts per slot, and the tile sigma; 8 lanes per pixel (the neighbours)
__global__ void k_tile_dist(const float* __restrict__ data, int ncols, int npx, int r0, int c0, int tr, int tc,
                            const int32_t* __restrict__ ind, int nind, int satp, const uint32_t* __restrict__ key,
                            float* __restrict__ sig_t, float* __restrict__ d2_t, float* __restrict__ n2_t) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int pix = gt >> 3, lane8 = gt & 7;
    const float m = fmax_unkey(*key);
    const float mxval = satp ? __fmul_rn(m, 0.9961f) : __fadd_rn(m, 1.0f);
    float s0 = 1e24f;
    if (pix < tr * tc) {
        const int j = pix / tc, i = pix - (pix / tc) * tc;
        if (j >= 1 && i >= 1) {  // the first row and column of a tile have empty windows
            const int cstart = i - 1, cend = min(i + 1, tc - 1) + 1, width = cend - cstart;
            const int k = lane8 < 4 ? lane8 : lane8 + 1;
            const int jn = j + k / 3 - 1, inn = i + k % 3 - 1;
            if (lane8 == 0) {
                const int cslot = width + 1;  // (j - rstart) * width + (i - cstart)
                n2_t[(int64_t)pix * 9 + cslot] = (float)npx;
                d2_t[(int64_t)pix * 9 + cslot] = 0.0f;
            }
            if (jn < tr && inn < tc) {
                const int slot = (jn - (j - 1)) * width + (inn - cstart);
                float d2, n2;
                pair_ssd(data + ((int64_t)(r0 + j) * ncols + (c0 + i)) * npx,
                         data + ((int64_t)(r0 + jn) * ncols + (c0 + inn)) * npx, ind, nind, mxval, 1.0e-12f, d2, n2);
                n2_t[(int64_t)pix * 9 + slot] = n2;
                d2_t[(int64_t)pix * 9 + slot] = d2;
                if (d2 >= 1.e-3f) s0 = __fdiv_rn(d2, __fmul_rn(n2, 2.0f));
            }
        }
    }
    for (int o = 4; o > 0; o >>= 1) s0 = fminf(s0, __shfl_down_sync(0xffffffffu, s0, o, 8));
    if (lane8 == 0 && pix < tr * tc) sig_t[pix] = __fsqrt_rn(s0);
}

// normalise with the tile sigma and merge into the scan arrays (one thread per pixel and slot)
__global__ void k_tile_merge(int ncols, int r0, int c0, int tr, int tc, const float* __restrict__ sig_t,
                             const float* __restrict__ d2_t, const float* __restrict__ n2_t,
                             float* __restrict__ sigma, float* __restrict__ d2, float* __restrict__ n2) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)tr * tc * 9) return;
    const int pix = (int)(t / 9), q = (int)(t - (int64_t)pix * 9);
    const int j = pix / tc, i = pix - (pix / tc) * tc;
    const int64_t g = (int64_t)(r0 + j) * ncols + (c0 + i);
    if (q == 0) sigma[g] = fminf(sigma[g], sig_t[pix]);
    const float n = n2_t[t];
    if (n > 0.0f) {
        const int cstart = i - 1, cend = min(i + 1, tc - 1) + 1, width = cend - cstart;
        const int jj = j - 1 + q / width, ii = cstart + q % width;
        const float sa = sig_t[pix], sb = sig_t[jj * tc + ii];
        const float s12 = __fadd_rn(__fmul_rn(sa, sa), __fmul_rn(sb, sb));
        float v = __fsub_rn(d2_t[t], __fmul_rn(n, s12));
        v = __fdiv_rn(v, __fmul_rn(s12, __fsqrt_rn(__fmul_rn(2.0f, n))));
        d2[g * 9 + q] = v;
        n2[g * 9 + q] = n;
    }
}

// the objective mean |tw - 1 / (sum_q exp(-max(d2, dthresh) / lam^2) + 1e-12)| over the pixels
// (rows and columns stepped by `stride`), float64; per-block sums, then one block in order
constexpr int kLamBlocks = 256;

__global__ void k_lam_partial(const float* __restrict__ d2, int nrows, int ncols, int stride, float dthresh,
                              double lam2, double tw, double* __restrict__ part) {
    __shared__ double red[256];
    const int sr = (nrows + stride - 1) / stride, sc = (ncols + stride - 1) / stride;
    const int64_t total = (int64_t)sr * sc;
    double acc = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(t / sc), b = (int)(t - (int64_t)a * sc);
        const float* v = d2 + ((int64_t)(a * stride) * ncols + b * stride) * 9;
        double e[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float m = fmaxf(v[q], dthresh);  // np.maximum (no NaN in the distances)
            e[q] = exp(__ddiv_rn((double)(-m), lam2));
        }
        // numpy's pairwise order for nine terms
        double w = __dadd_rn(__dadd_rn(__dadd_rn(e[0], e[1]), __dadd_rn(e[2], e[3])),
                             __dadd_rn(__dadd_rn(e[4], e[5]), __dadd_rn(e[6], e[7])));
        w = __dadd_rn(__dadd_rn(w, e[8]), 1e-12);
        acc = __dadd_rn(acc, fabs(__dsub_rn(tw, __ddiv_rn(1.0, w))));
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_lam_final(const double* __restrict__ part, int nparts, double count, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nparts; ++b) s = __dadd_rn(s, part[b]);
        *out = __ddiv_rn(s, count);
    }
}

}  // namespace
}  // namespace ebsd

using namespace ebsd;

extern "C" {

int ebsd_nlpar_sigma(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                     int32_t nind, float datamax, int saturation_protect, float* d_sigma, void* stream) {
    if (!d_data || !d_indices || !d_sigma || nrows <= 0 || ncols <= 0 || npx <= 0 || nind < 0 || nind > npx)
        return EBSD_E_ARG;
    float mxval = saturation_protect ? datamax * 0.9961f : datamax + 1.0f;
    int64_t threads = (int64_t)nrows * ncols * 8;
    k_nlpar_sigma<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        d_data, nrows, ncols, npx, d_indices, nind, mxval, d_sigma);
    return launch_status();
}

int ebsd_nlpar_sigma_tile(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, int32_t r0, int32_t r1,
                          int32_t c0, int32_t c1, const int32_t* d_indices, int32_t nind, int saturation_protect,
                          float* d_sigma, float* d_d2, float* d_n2, float* d_work, void* stream) {
    if (!d_data || !d_indices || !d_sigma || !d_d2 || !d_n2 || !d_work || nrows <= 0 || ncols <= 0 || npx <= 0 ||
        nind < 0 || nind > npx)
        return EBSD_E_ARG;
    if (r0 < 0 || c0 < 0 || r1 > nrows || c1 > ncols || r1 <= r0 || c1 <= c0) return EBSD_E_ARG;
    const int tr = r1 - r0, tc = c1 - c0;
    const int64_t tp = (int64_t)tr * tc;
    cudaStream_t st = (cudaStream_t)stream;
    float* sig_t = d_work;
    float* d2_t = sig_t + tp;
    float* n2_t = d2_t + tp * 9;
    uint32_t* key = (uint32_t*)(n2_t + tp * 9);
    EBSD_CUDA_TRY(cudaMemsetAsync(d2_t, 0, (size_t)tp * 18 * sizeof(float) + sizeof(uint32_t), st));
    const int64_t elems = tp * npx;
    const int mb = (int)std::min<int64_t>((elems + 255) / 256, 152 * 8);
    k_tile_max<<<mb, 256, 0, st>>>(d_data, ncols, npx, r0, c0, tr, tc, key);
    int rc = launch_status();
    if (rc != EBSD_OK) return rc;
    const int64_t th = tp * 8;
    k_tile_dist<<<(unsigned)((th + 255) / 256), 256, 0, st>>>(d_data, ncols, npx, r0, c0, tr, tc, d_indices, nind,
                                                             saturation_protect, key, sig_t, d2_t, n2_t);
    rc = launch_status();
    if (rc != EBSD_OK) return rc;
    const int64_t tm = tp * 9;
    k_tile_merge<<<(unsigned)((tm + 255) / 256), 256, 0, st>>>(ncols, r0, c0, tr, tc, sig_t, d2_t, n2_t, d_sigma,
                                                              d_d2, d_n2);
    return launch_status();
}

int ebsd_nlpar_lambda_metric(const float* d_d2, int32_t nrows, int32_t ncols, int32_t stride, float dthresh,
                             double lam, double tw, double* d_work, double* d_out, void* stream) {
    if (!d_d2 || !d_work || !d_out || nrows <= 0 || ncols <= 0 || stride < 1) return EBSD_E_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t sr = (nrows + stride - 1) / stride, sc = (ncols + stride - 1) / stride;
    k_lam_partial<<<kLamBlocks, 256, 0, st>>>(d_d2, nrows, ncols, stride, dthresh, lam * lam, tw, d_work);
    int rc = launch_status();
    if (rc != EBSD_OK) return rc;
    k_lam_final<<<1, 32, 0, st>>>(d_work, kLamBlocks, (double)(sr * sc), d_out);
    return launch_status();
}

int ebsd_nlpar(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
               int32_t nind, float datamax, float lam, int32_t sr, float dthresh, const float* d_sigma,
               int saturation_protect, float* d_work, float* d_out, void* stream) {
    return ebsd_nlpar_out(d_data, nrows, ncols, npx, d_indices, nind, datamax, lam, sr, dthresh, d_sigma,
                          saturation_protect, d_work, EBSD_F32, d_out, nullptr, stream);
}

int ebsd_nlpar_out(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                   int32_t nind, float datamax, float lam, int32_t sr, float dthresh, const float* d_sigma,
                   int saturation_protect, float* d_work, int out_dtype, void* d_out,
                   const float* d_centre_offset, void* stream) {
    if (out_dtype != EBSD_F32 && out_dtype != EBSD_U8 && out_dtype != EBSD_U16) return EBSD_E_DTYPE;
    if (!d_data || !d_indices || !d_sigma || !d_work || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 ||
        nind < 0 || nind > npx || sr < 0 || sr > 10 || !(lam > 0.0f))
        return EBSD_E_ARG;
    if (2 * sr + 1 > nrows || 2 * sr + 1 > ncols) return EBSD_E_ARG;  // window must fit the scan
    float mxval = saturation_protect ? datamax * 0.999f : datamax + 1.0f;
    float lam2 = 1.0f / (lam * lam);
    int winsz = (2 * sr + 1) * (2 * sr + 1);
    int bs = ((winsz + 31) / 32) * 32;
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 tgrid((unsigned)((ncols + kTileX - 1) / kTileX), (unsigned)nrows), tblock(kTileX, kTy);
    const size_t wsm = tiled_smem(sr, ncols, sizeof(float), true), asm_ = tiled_smem(sr, ncols, sizeof(float), false);
    if (sr <= 3 && wsm <= 48 * 1024 && asm_ <= 48 * 1024) {
        k_nlpar_weights_tiled<4><<<tgrid, tblock, wsm, st>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval,
                                                             d_sigma, lam2, dthresh, sr, d_work, d_centre_offset);
        int rc = launch_status();
        if (rc != EBSD_OK) return rc;
        if (out_dtype == EBSD_U8)
            launch_average_tiled<float, uint8_t>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, d_work, sr,
                                                 (uint8_t*)d_out);
        else if (out_dtype == EBSD_U16)
            launch_average_tiled<float, uint16_t>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, d_work, sr,
                                                  (uint16_t*)d_out);
        else
            launch_average_tiled<float, float>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, d_work, sr,
                                               (float*)d_out);
        return launch_status();
    }
    k_nlpar_weights<<<(unsigned)(nrows * ncols), bs, winsz * sizeof(float), st>>>(
        d_data, nrows, ncols, npx, d_indices, nind, mxval, d_sigma, lam2, dthresh, sr, d_work, d_centre_offset);
    int rc = launch_status();
    if (rc != EBSD_OK) return rc;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    if (out_dtype == EBSD_U8)
        k_nlpar_average_to<uint8_t><<<grid, 256, 0, st>>>(d_data, nrows, ncols, npx, d_work, sr, (uint8_t*)d_out);
    else if (out_dtype == EBSD_U16)
        k_nlpar_average_to<uint16_t><<<grid, 256, 0, st>>>(d_data, nrows, ncols, npx, d_work, sr, (uint16_t*)d_out);
    else
        k_nlpar_average<float><<<grid, 256, 0, st>>>(d_data, nrows, ncols, npx, d_work, sr, (float*)d_out);
    return launch_status();
}

int ebsd_nlpar_pairs_out(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                         int32_t nind, float datamax, float lam, int32_t sr, float dthresh, float* d_sigma,
                         int compute_sigma, int saturation_protect, float* d_work, int out_dtype, void* d_out,
                         const float* d_centre_offset, void* stream) {
    if (out_dtype != EBSD_F32 && out_dtype != EBSD_U8 && out_dtype != EBSD_U16) return EBSD_E_DTYPE;
    if (!d_data || !d_indices || !d_sigma || !d_work || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 ||
        nind < 0 || nind > npx || sr < 1 || sr > 3 || !(lam > 0.0f))
        return EBSD_E_ARG;
    if (2 * sr + 1 > nrows || 2 * sr + 1 > ncols) return EBSD_E_ARG;  // window must fit the scan
    const size_t psm = pairs_smem(sr, ncols), asm_ = tiled_smem(sr, ncols, sizeof(float), false);
    if (psm > 48 * 1024 || asm_ > 48 * 1024 || edge_rows_smem(sr, ncols) > 48 * 1024 || edge_cols_smem(sr) > 48 * 1024)
        return EBSD_E_UNSUPPORTED;
    const float mxval = saturation_protect ? datamax * 0.999f : datamax + 1.0f;
    const float mxsig = saturation_protect ? datamax * 0.9961f : datamax + 1.0f;
    const float lam2 = 1.0f / (lam * lam);
    const int64_t npix = (int64_t)nrows * ncols;
    const int winsz = (2 * sr + 1) * (2 * sr + 1), nF = sr * (2 * sr + 1) + sr;
    float* w = d_work;
    // the pair sums start at the next even float after the weights (8-byte aligned float2;
    // d_work itself is at least 8-byte aligned)
    if ((uintptr_t)d_work % 8 != 0) return EBSD_E_ARG;
    float2* pairs = (float2*)(d_work + ((npix * winsz + 1) & ~(int64_t)1));
    float2* sigp = pairs + npix * nF;
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 pgrid((unsigned)((ncols + kTileX - 1) / kTileX), (unsigned)nrows), pblock(kTileX, kPairTy);
    const int mpf = (nF + kPairTy - 1) / kPairTy;
#define EBSD_PAIRS(M, SG)                                                                                     \
    k_nlpar_pairs<M, SG><<<pgrid, pblock, psm, st>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval, mxsig, sr, \
                                                     pairs, sigp)
    if (compute_sigma) {
        if (mpf == 1) EBSD_PAIRS(1, true);
        else if (mpf == 2) EBSD_PAIRS(2, true);
        else EBSD_PAIRS(3, true);
    } else {
        if (mpf == 1) EBSD_PAIRS(1, false);
        else if (mpf == 2) EBSD_PAIRS(2, false);
        else EBSD_PAIRS(3, false);
    }
#undef EBSD_PAIRS
    int rc = launch_status();
    if (rc != EBSD_OK) return rc;
    if (compute_sigma) {
        k_nlpar_sigma_pairs<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(sigp, nrows, ncols, d_sigma);
        if ((rc = launch_status()) != EBSD_OK) return rc;
    }
    const dim3 tgrid((unsigned)((ncols + kTileX - 1) / kTileX), (unsigned)nrows), tblock(kTileX, kTy);
    k_nlpar_weights_pairs<4><<<tgrid, tblock, 0, st>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval, pairs,
                                                       d_sigma, lam2, dthresh, sr, w, d_centre_offset);
    if ((rc = launch_status()) != EBSD_OK) return rc;
    {
        // edge pixels: raw window sums (rows, then the middle rows' columns), then their weights
        float2* raw = sigp + npix * 4;
        const int nri = nrows - 2 * sr;
        const unsigned zr = (unsigned)((winsz + kTy - 1) / kTy), zc = (unsigned)((sr * winsz + kTy - 1) / kTy);
        k_nlpar_edge_rows<<<dim3((unsigned)((ncols + kTileX - 1) / kTileX), (unsigned)(2 * sr), zr), tblock,
                            edge_rows_smem(sr, ncols), st>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval, sr, raw);
        if ((rc = launch_status()) != EBSD_OK) return rc;
        if (nri > 0) {
            k_nlpar_edge_cols<<<dim3((unsigned)((nri + kTileX - 1) / kTileX), 2u, zc), tblock, edge_cols_smem(sr), st>>>(
                d_data, nrows, ncols, npx, d_indices, nind, mxval, sr, raw);
            if ((rc = launch_status()) != EBSD_OK) return rc;
        }
        const int64_t nedge = (int64_t)2 * sr * ncols + (int64_t)nri * 2 * sr;
        k_nlpar_weights_edge<<<(unsigned)nedge, 64, 0, st>>>(raw, nrows, ncols, sr, d_sigma, lam2, dthresh, w,
                                                             d_centre_offset);
        if ((rc = launch_status()) != EBSD_OK) return rc;
    }
    if (out_dtype == EBSD_U8)
        launch_average<uint8_t>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, w, sr, (uint8_t*)d_out);
    else if (out_dtype == EBSD_U16)
        launch_average<uint16_t>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, w, sr, (uint16_t*)d_out);
    else
        launch_average<float>(tgrid, tblock, asm_, st, d_data, nrows, ncols, npx, w, sr, (float*)d_out);
    return launch_status();
}

int ebsd_nlpar_apply(const float* d_x, int32_t nrows, int32_t ncols, int32_t npx, const float* d_w, int32_t sr,
                     float* d_out, void* stream) {
    if (!d_x || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10 || 2 * sr + 1 > nrows ||
        2 * sr + 1 > ncols)
        return EBSD_E_ARG;
    const size_t asm_ = tiled_smem(sr, ncols, sizeof(float), false);
    if (asm_ <= 48 * 1024) {
        const dim3 tgrid((unsigned)((ncols + kTileX - 1) / kTileX), (unsigned)nrows), tblock(kTileX, kTy);
        launch_average_tiled<float, float>(tgrid, tblock, asm_, (cudaStream_t)stream, d_x, nrows, ncols, npx, d_w, sr,
                                           d_out);
        return launch_status();
    }
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_average<float><<<grid, 256, 0, (cudaStream_t)stream>>>(d_x, nrows, ncols, npx, d_w, sr, d_out);
    return launch_status();
}

int ebsd_nlpar_apply64(const double* d_x, int32_t nrows, int32_t ncols, int32_t npx, const double* d_w, int32_t sr,
                       double* d_out, void* stream) {
    if (!d_x || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10 || 2 * sr + 1 > nrows ||
        2 * sr + 1 > ncols)
        return EBSD_E_ARG;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_average<double><<<grid, 256, 0, (cudaStream_t)stream>>>(d_x, nrows, ncols, npx, d_w, sr, d_out);
    return launch_status();
}

}  // extern "C"
