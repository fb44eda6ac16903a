// Per-stage ("plain") band-detection path: one kernel per reference stage, intermediates in
// HBM.  Templated on the arithmetic type T: float is the plain FP32 path, double is the
// FP64 GPU oracle of the same pipeline.
//
//   k_radon_plain      radon_fast.py:242-310  (background subtract, ray mean, missing = -1)
//   k_pad_plain        band_detect.py:573-580 (theta mirror with rho flip, rho edge copy)
//   k_conv_plain       band_detect.py:596-606 ('same' convolution, zero extension)
//   k_stats_plain      band_detect.py:627-630 (min / mean over the statistics slice)
//   k_dilate_theta     band_detect.py:646, :811-843 (window clipped at the array edge)
//   k_dilate_rho_flag  band_detect.py:647-663 (second pass, exact equality, Radon mask)
//   k_label_plain      band_detect.py:667-809 + :457-460 + :521-524
#include "ebsd_internal.cuh"
#include "label.cuh"

#include <cfloat>

namespace ebsd {
namespace {

template <typename InT, typename T>
__device__ __forceinline__ T pixel_value(const InT* p, int idx, int bg_mode, const double* bg,
                                         const float* bgf) {
    if (bg_mode == 1) {
        return (T)((double)p[idx] - bg[idx]);
    } else if (bg_mode == 2) {
        if (sizeof(T) == 4) return (T)__fsub_rn((float)p[idx], bgf[idx]);
        return (T)((double)p[idx] - (double)bgf[idx]);
    }
    return (T)p[idx];
}

// One thread per (pattern, ray): sequential sum over the ray's sorted LUT entries, exactly
// the accumulation order of rdn_loops (radon_fast.py:299-305).
template <typename InT, typename T>
__global__ void k_radon_plain(const InT* __restrict__ pats, const uint16_t* __restrict__ lut16,
                              const int32_t* __restrict__ lut32, const int32_t* __restrict__ count,
                              int nRays, int nTheta, int nPx, int bg_mode,
                              const double* __restrict__ bg, const float* __restrict__ bgf,
                              T* __restrict__ radon, int R, int Tp, int p0, int p1) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    int64_t q = blockIdx.y;
    if (r >= nRays) return;
    const InT* p = pats + q * (int64_t)nPx;
    int cnt = count[r];
    T sum = (T)0;
    if (lut16) {
        for (int k = 0; k < cnt; ++k) {
            int idx = lut16[(size_t)k * nRays + r];
            sum = r_add(sum, pixel_value<InT, T>(p, idx, bg_mode, bg, bgf));
        }
    } else {
        for (int k = 0; k < cnt; ++k) {
            int idx = lut32[(size_t)k * nRays + r];
            sum = r_add(sum, pixel_value<InT, T>(p, idx, bg_mode, bg, bgf));
        }
    }
    T val = cnt >= 1 ? r_div(sum, (T)cnt) : (T)-1;
    int i = r / nTheta, j = r - (r / nTheta) * nTheta;
    radon[q * (int64_t)R * Tp + (int64_t)(i + p0) * Tp + (j + p1)] = val;
}

// The same ray means with the patterns staged in shared memory (P patterns per block, the
// threads striding over the rays; each LUT entry read once serves the P patterns): the
// gathers hit shared memory instead of scattered global loads.  Used without a background
// and when the patterns fit; every per-ray sum keeps the sequential LUT order, so the values
// equal k_radon_plain's.
template <typename InT, typename T, int P>
__global__ void __launch_bounds__(1024) k_radon_smem(const InT* __restrict__ pats, const uint16_t* __restrict__ lut16,
                                                    const int32_t* __restrict__ lut32,
                                                    const int32_t* __restrict__ count, int64_t n, int nRays,
                                                    int nTheta, int nPx, T* __restrict__ radon, int R, int Tp, int p0,
                                                    int p1) {
    extern __shared__ __align__(16) unsigned char rsm[];
    InT* px = (InT*)rsm;
    const int64_t q0 = (int64_t)blockIdx.x * P;
    const int np = (int)(n - q0 < P ? n - q0 : P);
    for (int t = threadIdx.x; t < np * nPx; t += blockDim.x) px[t] = pats[q0 * nPx + t];
    __syncthreads();
    for (int r = threadIdx.x; r < nRays; r += blockDim.x) {
        const int cnt = count[r];
        T sum[P];
#pragma unroll
        for (int i = 0; i < P; ++i) sum[i] = (T)0;
        for (int k = 0; k < cnt; ++k) {
            const int idx = lut16 ? (int)lut16[(size_t)k * nRays + r] : lut32[(size_t)k * nRays + r];
#pragma unroll
            for (int i = 0; i < P; ++i) sum[i] = r_add(sum[i], (T)px[i * nPx + idx]);
        }
        const int ri = r / nTheta, rj = r - (r / nTheta) * nTheta;
#pragma unroll
        for (int i = 0; i < P; ++i) {
            if (i < np) {
                const T val = cnt >= 1 ? r_div(sum[i], (T)cnt) : (T)-1;
                radon[(q0 + i) * (int64_t)R * Tp + (int64_t)(ri + p0) * Tp + (rj + p1)] = val;
            }
        }
    }
}

template <typename InT, typename T, int P>
int launch_radon_smem(const ebsd_plan_s* p, const InT* d_pats, int64_t n, T* radon, cudaStream_t st) {
    const size_t bytes = (size_t)P * p->nPx * sizeof(InT);
    static int raised[64] = {};
    if (bytes > 48 * 1024 && raised[p->device] < (int)bytes) {
        EBSD_CUDA_TRY(cudaFuncSetAttribute(k_radon_smem<InT, T, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
        raised[p->device] = (int)bytes;
    }
    k_radon_smem<InT, T, P><<<(unsigned)((n + P - 1) / P), 1024, bytes, st>>>(
        d_pats, p->d_lut16, p->d_lut32, p->d_count, n, p->nRays, p->nTheta, p->nPx, radon, p->R, p->Tp, p->p0, p->p1);
    return launch_status();
}

// Fills every padding cell from the interior: theta padding is the theta-wrapped column
// flipped in rho, rho padding repeats the first/last interior row (after theta padding).
template <typename T>
__global__ void k_pad_plain(T* __restrict__ radon, int64_t n, int R, int Tp, int p0, int p1,
                            int nRho, int nTheta) {
    int64_t per = (int64_t)R * Tp;
    int64_t total = per * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t q = t / per;
        int cell = (int)(t - q * per);
        int r = cell / Tp, c = cell - (cell / Tp) * Tp;
        int i = r - p0, j = c - p1;
        if (i >= 0 && i < nRho && j >= 0 && j < nTheta) continue;
        int ic = i < 0 ? 0 : (i >= nRho ? nRho - 1 : i);
        int si, sj;
        if (j < 0) {
            si = nRho - 1 - ic;
            sj = nTheta + j;
        } else if (j >= nTheta) {
            si = nRho - 1 - ic;
            sj = j - nTheta;
        } else {
            si = ic;
            sj = j;
        }
        T* base = radon + q * per;
        base[cell] = base[(int64_t)(si + p0) * Tp + (sj + p1)];
    }
}

// 'same'-mode 2-D convolution over the whole padded frame, zero outside it.
template <typename T>
__global__ void k_conv_plain(const T* __restrict__ radon, T* __restrict__ conv,
                             const T* __restrict__ kern, const float* __restrict__ ksep, int sep,
                             int k0, int k1, int R, int Tp) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    int64_t q = blockIdx.z;
    if (c >= Tp) return;
    const T* src = radon + q * (int64_t)R * Tp;
    int h0 = k0 / 2, h1 = k1 / 2;
    T acc = (T)0;
    if (sep) {
        // separable taps (FP32): each kernel row's theta convolution, then the rho taps, in
        // ascending order -- the fused kernel's arithmetic
        for (int a = 0; a < k0; ++a) {
            int rr = r + h0 - a;
            if (rr < 0 || rr >= R) continue;
            T h = (T)0;
            for (int b = 0; b < k1; ++b) {
                int cc = c + h1 - b;
                if (cc < 0 || cc >= Tp) continue;
                h = fma((T)ksep[k0 + b], src[(int64_t)rr * Tp + cc], h);
            }
            acc = fma((T)ksep[a], h, acc);
        }
    } else {
        for (int a = 0; a < k0; ++a) {
            int rr = r + h0 - a;
            if (rr < 0 || rr >= R) continue;
            for (int b = 0; b < k1; ++b) {
                int cc = c + h1 - b;
                if (cc < 0 || cc >= Tp) continue;
                acc = fma(kern[a * k1 + b], src[(int64_t)rr * Tp + cc], acc);
            }
        }
    }
    conv[q * (int64_t)R * Tp + (int64_t)r * Tp + c] = acc;
}

// Per-pattern min and mean over rows [p0, min(R, Tp - p0)) x cols [p1, Tp - p1): the slice
// band_detect.py:627-630 takes (its rho bound is the padded theta size, shprdn[1]).
template <typename T>
__global__ void k_stats_plain(const T* __restrict__ conv, T* __restrict__ stats, int R, int Tp,
                              int p0, int p1) {
    int64_t q = blockIdx.x;
    const T* src = conv + q * (int64_t)R * Tp;
    int r1 = Tp - p0 < R ? Tp - p0 : R;
    int c1 = Tp - p1;
    int nr = r1 - p0, nc = c1 - p1;
    int total = nr * nc;
    double s = 0.0;
    T mn = (T)INFINITY;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int rr = p0 + t / nc, cc = p1 + t % nc;
        T v = src[(int64_t)rr * Tp + cc];
        s += (double)v;
        mn = v < mn ? v : mn;
    }
    __shared__ double ss[32];
    __shared__ T sm[32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        T m2 = __shfl_down_sync(0xffffffffu, mn, o);
        mn = m2 < mn ? m2 : mn;
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { ss[w] = s; sm[w] = mn; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        s = l < nw ? ss[l] : 0.0;
        mn = l < nw ? sm[l] : (T)INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_down_sync(0xffffffffu, s, o);
            T m2 = __shfl_down_sync(0xffffffffu, mn, o);
            mn = m2 < mn ? m2 : mn;
        }
        if (l == 0) {
            stats[2 * q] = mn;
            stats[2 * q + 1] = (T)(s / (double)total);
        }
    }
}

// First max-filter pass along theta, window [c-h, c+h] clipped to the array.
template <typename T>
__global__ void k_dilate_theta(const T* __restrict__ conv, T* __restrict__ tmp, int R, int Tp, int h) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    int64_t q = blockIdx.z;
    if (c >= Tp) return;
    const T* src = conv + q * (int64_t)R * Tp + (int64_t)r * Tp;
    int c0 = c - h < 0 ? 0 : c - h;
    int c1 = c + h > Tp - 1 ? Tp - 1 : c + h;
    T m = neg_inf<T>();
    for (int cc = c0; cc <= c1; ++cc) {
        T v = src[cc];
        m = v > m ? v : m;
    }
    tmp[q * (int64_t)R * Tp + (int64_t)r * Tp + c] = m;
}

// Second pass along rho on the interior cells, local-max flag = (max == value) AND rdnmask.
template <typename T>
__global__ void k_dilate_rho_flag(const T* __restrict__ conv, const T* __restrict__ tmp,
                                  const uint8_t* __restrict__ rdnmask, uint8_t* __restrict__ flags,
                                  int R, int Tp, int p0, int p1, int nRho, int nTheta, int h) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    int64_t q = blockIdx.z;
    if (j >= nTheta) return;
    int r = i + p0, c = j + p1;
    const T* t = tmp + q * (int64_t)R * Tp;
    int r0 = r - h < 0 ? 0 : r - h;
    int r1 = r + h > R - 1 ? R - 1 : r + h;
    T m = neg_inf<T>();
    for (int rr = r0; rr <= r1; ++rr) {
        T v = t[(int64_t)rr * Tp + c];
        m = v > m ? v : m;
    }
    T v0 = conv[q * (int64_t)R * Tp + (int64_t)r * Tp + c];
    flags[q * (int64_t)nRho * nTheta + (int64_t)i * nTheta + j] =
        (uint8_t)((m == v0) && rdnmask[i * nTheta + j]);
}

template <typename T>
struct GlobalConv {
    const T* base;
    int Tp;
    __device__ __forceinline__ T operator()(int r, int c) const { return base[(int64_t)r * Tp + c]; }
};

// One warp per pattern: scan the flags in row-major order into a warp top-N list, then
// lanes 0..nB-1 fit their band and write the record fields.
template <typename T>
__global__ void k_label_plain(const T* __restrict__ conv, const uint8_t* __restrict__ flags,
                              const T* __restrict__ stats, int64_t n, int R, int Tp, int nRho,
                              int nTheta, LabelConsts kc, ebsd_bands out, int64_t out_offset) {
    int lane = threadIdx.x & 31;
    int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= n) return;
    const T* cq = conv + q * (int64_t)R * Tp;
    const uint8_t* fq = flags + q * (int64_t)nRho * nTheta;
    int nB = kc.nB;
    T lv = neg_inf<T>();
    int lpos = -1;
    int total = nRho * nTheta;
    for (int base = 0; base < total; base += 32) {
        int t = base + lane;
        bool f = t < total && fq[t];
        unsigned bal = __ballot_sync(0xffffffffu, f);
        T myv = (T)0;
        if (f) {
            int i = t / nTheta, j = t - (t / nTheta) * nTheta;
            myv = cq[(int64_t)(i + kc.p0) * Tp + (j + kc.p1)];
        }
        while (bal) {
            int b = __ffs(bal) - 1;
            bal &= bal - 1;
            T v = __shfl_sync(0xffffffffu, myv, b);
            topn_insert(v, base + b, lv, lpos, nB, lane);
        }
    }
    if (lane < nB) {
        bool has = lpos >= 0;
        int r = 0, c = 0;
        if (has) {
            int i = lpos / nTheta;
            r = i + kc.p0;
            c = (lpos - i * nTheta) + kc.p1;
        }
        GlobalConv<T> acc{cq, Tp};
        band_fit_write<T>(has, r, c, acc, stats[2 * q], stats[2 * q + 1], kc, out,
                          (out_offset + q) * nB + lane);
    }
}

template <typename T>
size_t ws_bytes(const ebsd_plan_s* p, int64_t chunk) {
    size_t cells = (size_t)p->R * p->Tp;
    size_t b = 3 * cells * sizeof(T) * chunk;                 // radon, conv, tmp
    b += (size_t)p->nRays * chunk;                            // flags
    b += 2 * sizeof(T) * chunk;                               // stats
    b += (size_t)p->k0 * p->k1 * sizeof(T) + 1024;            // kernel copy + alignment slack
    return b;
}

template <typename T, typename InT>
int run_chunk_t(ebsd_plan_s* p, const InT* d_pats, int64_t n, const ebsd_bands* out,
                int64_t out_offset, cudaStream_t st, int64_t* launches, char* ws) {
    size_t cells = (size_t)p->R * p->Tp;
    T* radon = (T*)ws;
    T* conv = radon + cells * n;
    T* tmp = conv + cells * n;
    T* stats = tmp + cells * n;
    uint8_t* flags = (uint8_t*)(stats + 2 * n);
    const T* kern = sizeof(T) == 4 ? (const T*)p->d_kernel : (const T*)p->d_kernel64;

    const size_t px_smem = (size_t)p->nPx * sizeof(InT);
    constexpr size_t kRadonSmem = 200 * 1024;
    if (p->bg_mode == 0 && px_smem <= kRadonSmem) {
        const int rrc = (4 * px_smem <= kRadonSmem && n >= 4)   ? launch_radon_smem<InT, T, 4>(p, d_pats, n, radon, st)
                        : (2 * px_smem <= kRadonSmem && n >= 2) ? launch_radon_smem<InT, T, 2>(p, d_pats, n, radon, st)
                                                                : launch_radon_smem<InT, T, 1>(p, d_pats, n, radon, st);
        if (rrc != EBSD_OK) return rrc;
    } else {
        dim3 gr((p->nRays + 127) / 128, (unsigned)n);
        k_radon_plain<InT, T><<<gr, 128, 0, st>>>(d_pats, p->d_lut16, p->d_lut32, p->d_count, p->nRays,
                                                  p->nTheta, p->nPx, p->bg_mode, p->d_bg, p->d_bgf, radon,
                                                  p->R, p->Tp, p->p0, p->p1);
    }
    int64_t padcells = (int64_t)cells * n;
    int pblocks = (int)((padcells + 255) / 256 < 152 * 32 ? (padcells + 255) / 256 : 152 * 32);
    k_pad_plain<T><<<pblocks, 256, 0, st>>>(radon, n, p->R, p->Tp, p->p0, p->p1, p->nRho, p->nTheta);
    dim3 gc((p->Tp + 127) / 128, p->R, (unsigned)n);
    // FP64 keeps the full 2-D taps (the FP64 oracle); FP32 uses the separable form when the
    // plan's kernel is separable, as the fused kernel does
    const int sep = sizeof(T) == 4 ? p->sep : 0;
    k_conv_plain<T><<<gc, 128, 0, st>>>(radon, conv, kern, p->d_ksep, sep, p->k0, p->k1, p->R, p->Tp);
    k_stats_plain<T><<<(unsigned)n, 256, 0, st>>>(conv, stats, p->R, p->Tp, p->p0, p->p1);
    k_dilate_theta<T><<<gc, 128, 0, st>>>(conv, tmp, p->R, p->Tp, p->pk1 / 2);
    dim3 gf((p->nTheta + 127) / 128, p->nRho, (unsigned)n);
    k_dilate_rho_flag<T><<<gf, 128, 0, st>>>(conv, tmp, p->d_rdnmask, flags, p->R, p->Tp, p->p0,
                                             p->p1, p->nRho, p->nTheta, p->pk0 / 2);
    LabelConsts kc{p->p0, p->p1, p->nTheta, p->nRho, p->nB, p->d_theta, p->d_rho};
    k_label_plain<T><<<(unsigned)((n + 3) / 4), 128, 0, st>>>(conv, flags, stats, n, p->R, p->Tp,
                                                              p->nRho, p->nTheta, kc, *out, out_offset);
    *launches += 7;
    return launch_status();
}

}  // namespace

size_t plain_workspace_bytes(const ebsd_plan_s* p, int method, int64_t chunk) {
    return method == EBSD_PLAIN_F64 ? ws_bytes<double>(p, chunk) : ws_bytes<float>(p, chunk);
}

int plain_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches) {
    return plain_run_chunk_ws(p, method, dtype, d_pats, n, out, out_offset, st, launches,
                              p->ws.ptr);
}

int plain_run_chunk_ws(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                       const ebsd_bands* out, int64_t out_offset, cudaStream_t st,
                       int64_t* launches, void* workspace) {
    char* ws = (char*)workspace;
    if (n <= 0) return EBSD_OK;
    if (n > 65535) return EBSD_E_ARG;
    if (method == EBSD_PLAIN_F64) {
        switch (dtype) {
            case EBSD_U8: return run_chunk_t<double>(p, (const uint8_t*)d_pats, n, out, out_offset, st, launches, ws);
            case EBSD_U16: return run_chunk_t<double>(p, (const uint16_t*)d_pats, n, out, out_offset, st, launches, ws);
            case EBSD_F32: return run_chunk_t<double>(p, (const float*)d_pats, n, out, out_offset, st, launches, ws);
        }
    } else {
        switch (dtype) {
            case EBSD_U8: return run_chunk_t<float>(p, (const uint8_t*)d_pats, n, out, out_offset, st, launches, ws);
            case EBSD_U16: return run_chunk_t<float>(p, (const uint16_t*)d_pats, n, out, out_offset, st, launches, ws);
            case EBSD_F32: return run_chunk_t<float>(p, (const float*)d_pats, n, out, out_offset, st, launches, ws);
        }
    }
    return EBSD_E_DTYPE;
}

}  // namespace ebsd
