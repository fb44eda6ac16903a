// Adjoint kernels for the differentiable band-sharpness path.
//
// Linear stages are sparse operators held on the device in CSR form; each is applied by a
// gather (one thread per output row per pattern), so the adjoint needs no atomics:
//   Radon          R[ray][px] = 1/count(ray) for the ray's pixels  (radon_fast.py:281-310)
//   Radon adjoint  R^T: per pixel, the rays through it -- back-projection through the
//                  transposed lookup table
//   LoG            M = conv(kernel) o pad (band_detect.py:573-606) restricted to the interior;
//                  its transpose M^T is the correlation with the kernel folded back through
//                  the padding map
// NLPAR (nlpar_cpu.py:821-936) with weights W(lambda) held fixed in the patterns:
//   k_nlpar_weights2  normalised window weights w and exponent arguments m = max(d - dthresh, 0)
//   k_nlpar_apply_t   W^T g (gather over the windows that contain each scan pixel)
//   k_nlpar_lam_grad  dL/dlambda = sum_p sum_c dw_pc/dlambda (g_p . x_c),
//                     dw_pc/dlambda = w_pc (2 / lambda^3) (m_pc - sum_c' w_pc' m_pc')
#include "ebsd_internal.cuh"

#include <new>

struct ebsd_linop_s {
    int device = 0;
    int64_t nrows = 0, ncols = 0, nnz = 0;
    int64_t* rowptr = nullptr;
    int32_t* col = nullptr;
    float* val = nullptr;
    double* val64 = nullptr;
};

namespace ebsd {
namespace {

template <typename T>
__global__ void k_csr_gather(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y,
                             int64_t nrows, int64_t ncols) {
    int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t b = blockIdx.y;
    if (row >= nrows) return;
    const T* xb = x + b * ncols;
    T acc = (T)0;
    for (int64_t e = rowptr[row]; e < rowptr[row + 1]; ++e) acc = fma(val[e], xb[col[e]], acc);
    y[b * nrows + row] = acc;
}

// The same products with the patterns along the fast axis: x^T [ncols][ldx], y^T [nrows][ldy]
// hold pattern b in column b.  A warp takes one operator row for 32 patterns (lanes): each
// nonzero's column of x^T is one coalesced load, and the row's entries are read once per 32
// patterns.  Each output adds its row's terms in CSR order with fused multiply-adds, as
// k_csr_gather, so the results are the same bit for bit.
template <typename T>
__global__ void __launch_bounds__(256) k_csr_gather_cols(const int64_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ col,
                                                         const T* __restrict__ val, const T* __restrict__ xT,
                                                         int64_t ldx, T* __restrict__ yT, int64_t ldy,
                                                         int64_t nrows, int64_t n) {
    const int64_t row = (int64_t)blockIdx.x * 8 + threadIdx.y;
    const int64_t b = (int64_t)blockIdx.y * 32 + threadIdx.x;
    if (row >= nrows || b >= n) return;
    const int64_t e1 = __ldg(rowptr + row + 1);
    T acc = (T)0;
#pragma unroll 4
    for (int64_t e = __ldg(rowptr + row); e < e1; ++e)
        acc = fma(__ldg(val + e), __ldg(xT + (int64_t)__ldg(col + e) * ldx + b), acc);
    yT[row * ldy + b] = acc;
}

__device__ __forceinline__ void window(int i, int sr, int n, int& start, int& end) {
    int a = i - sr > 0 ? i - sr : 0;
    int b = i + sr - (n - 1) > 0 ? i + sr - (n - 1) : 0;
    start = a - b;
    int c = i + sr < n - 1 ? i + sr : n - 1;
    int e = sr - i > 0 ? sr - i : 0;
    end = c + e + 1;
}

__device__ __forceinline__ void pair_ssd(const float* __restrict__ a, const float* __restrict__ b,
                                         const int32_t* __restrict__ ind, int nind, float mxval,
                                         float& d2, float& n2) {
    float d = 0.0f, n = 0.0f;
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

// Normalised weights w and exponent arguments m of every window slot (one block per pixel).
__global__ void k_nlpar_weights2(const float* __restrict__ data, int nrows, int ncols, int npx,
                                 const int32_t* __restrict__ ind, int nind, float mxval,
                                 const float* __restrict__ sigma, float lam2, float dthresh, int sr,
                                 float* __restrict__ wout, float* __restrict__ mout) {
    extern __shared__ float w_s[];
    __shared__ float tot_s;
    int pix = blockIdx.x;
    int j = pix / ncols, i = pix - (pix / ncols) * ncols;
    int xs, xe, ys, ye;
    window(i, sr, ncols, xs, xe);
    window(j, sr, nrows, ys, ye);
    int wx = xe - xs, winsz = (2 * sr + 1) * (2 * sr + 1);
    int c = threadIdx.x;
    float m = 0.0f;
    if (c < winsz) {
        int nb = (xs + c % wx) + ncols * (ys + c / wx);
        float w;
        if (nb == pix) {
            w = -1.0e6f;
        } else {
            float s0 = sigma[pix], s1 = sigma[nb];
            s0 = __fmul_rn(s0, s0);
            s1 = __fmul_rn(s1, s1);
            float d2, n2;
            pair_ssd(data + (int64_t)pix * npx, data + (int64_t)nb * npx, ind, nind, mxval, d2, n2);
            float ss = __fadd_rn(s0, s1);
            d2 = __fsub_rn(d2, __fmul_rn(n2, ss));
            float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, n2)));
            w = dnorm > 1.e-8f ? __fdiv_rn(d2, dnorm) : __fmul_rn(1e6f, n2);
        }
        m = fmaxf(__fsub_rn(w, dthresh), 0.0f);
        w_s[c] = expf(__fmul_rn(__fmul_rn(-1.0f, m), lam2));
    }
    __syncthreads();
    if (c == 0) {
        float t = 0.0f;
        for (int k = 0; k < winsz; ++k) t = __fadd_rn(t, w_s[k]);
        tot_s = t;
    }
    __syncthreads();
    if (c < winsz) {
        wout[(int64_t)pix * winsz + c] = __fdiv_rn(w_s[c], tot_s);
        mout[(int64_t)pix * winsz + c] = m;
    }
}

// out[q][k] = sum over scan pixels p whose window holds q of w[p][slot] * g[p][k].
template <typename T>
__global__ void __launch_bounds__(256) k_nlpar_apply_t(const T* __restrict__ g, int nrows, int ncols, int npx,
                                                       const T* __restrict__ w, int sr, T* __restrict__ out) {
    // one scan pixel q per blockIdx.y: the windows that hold q (pixel p, slot c) are listed
    // once per block in the scan order of the sum, then each pattern value k adds
    // w[p][c] g[p][k] over the list with fused multiply-adds
    extern __shared__ unsigned char atsm[];
    const int q = blockIdx.y;
    const int winsz = (2 * sr + 1) * (2 * sr + 1), wx = 2 * sr + 1;
    const int maxt = (4 * sr + 1) * (4 * sr + 1);
    T* wt = (T*)atsm;                 // [maxt] weights
    int* pt = (int*)(wt + maxt);      // [maxt] pixels
    __shared__ int nterm;
    if (threadIdx.x == 0) {
        const int jq = q / ncols, iq = q - (q / ncols) * ncols;
        const int j0 = jq - 2 * sr < 0 ? 0 : jq - 2 * sr, j1 = jq + 2 * sr > nrows - 1 ? nrows - 1 : jq + 2 * sr;
        const int i0 = iq - 2 * sr < 0 ? 0 : iq - 2 * sr, i1 = iq + 2 * sr > ncols - 1 ? ncols - 1 : iq + 2 * sr;
        int t = 0;
        for (int jp = j0; jp <= j1; ++jp) {
            int ys, ye;
            window(jp, sr, nrows, ys, ye);
            if (jq < ys || jq >= ye) continue;
            for (int ip = i0; ip <= i1; ++ip) {
                int xs, xe;
                window(ip, sr, ncols, xs, xe);
                if (iq < xs || iq >= xe) continue;
                const int p = ip + ncols * jp;
                wt[t] = w[(int64_t)p * winsz + (jq - ys) * wx + (iq - xs)];
                pt[t++] = p;
            }
        }
        nterm = t;
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npx) return;
    const int nt = nterm;
    T acc = (T)0;
    for (int t = 0; t < nt; ++t) acc = fma(wt[t], __ldg(g + (int64_t)pt[t] * npx + k), acc);
    out[(int64_t)q * npx + k] = acc;
}

// Per scan pixel: sum_c dw_pc/dlambda * (g_p . x_c); block reduction over the pattern pixels.
template <typename T>
__global__ void k_nlpar_lam_grad(const T* __restrict__ g, const T* __restrict__ x, int nrows, int ncols, int npx,
                                 const float* __restrict__ w, const float* __restrict__ m, int sr, float lam,
                                 double* __restrict__ out) {
    __shared__ double red[32];
    int p = blockIdx.x;
    int jp = p / ncols, ip = p - (p / ncols) * ncols;
    int xs, xe, ys, ye;
    window(ip, sr, ncols, xs, xe);
    window(jp, sr, nrows, ys, ye);
    int wx = xe - xs, winsz = (2 * sr + 1) * (2 * sr + 1);
    const float* wp = w + (int64_t)p * winsz;
    const float* mp = m + (int64_t)p * winsz;
    double mbar = 0.0;
    for (int c = 0; c < winsz; ++c) mbar += (double)wp[c] * (double)mp[c];
    const double coef = 2.0 / ((double)lam * lam * lam);
    double acc = 0.0;
    const T* gp = g + (int64_t)p * npx;
    for (int k = threadIdx.x; k < npx; k += blockDim.x) {
        double gk = (double)gp[k], s = 0.0;
        for (int c = 0; c < winsz; ++c) {
            int nb = (xs + c % wx) + ncols * (ys + c / wx);
            s += (double)wp[c] * ((double)mp[c] - mbar) * (double)x[(int64_t)nb * npx + k];
        }
        acc += gk * s;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[p] = acc * coef;
    }
}

// ---- Gaussian background blur: one axis of a separable filter with reflect padding ----------
// Forward along `axis` (0: rows y, 1: columns x) of [n][H][W]:
//   out[o] = sum_{t=-r..r} taps[t + r] in[refl(o + t)],   refl(q) = -q (q < 0), 2(L-1) - q (q >= L)
// (torch's "reflect" padding followed by a correlation), and its adjoint
//   out[i] = sum_o sum_t taps[t + r] v[o] [refl(o + t) == i]
// as a gather: the direct terms o = i - t, the mirror of the low edge (o + t = -i, 1 <= i <= r)
// and of the high edge (o + t = 2(L-1) - i, L-1-r <= i <= L-2).  Requires r < L.
template <typename T>
__global__ void k_blur1d(const T* __restrict__ in, T* __restrict__ out, int64_t total, int H, int W, int axis,
                         const T* __restrict__ taps, int r) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int64_t p = idx / ((int64_t)H * W);
    const int rem = (int)(idx - p * H * W), y = rem / W, x = rem - (rem / W) * W;
    const int L = axis == 0 ? H : W, o = axis == 0 ? y : x, stride = axis == 0 ? W : 1;
    const T* base = in + p * H * W + (axis == 0 ? x : y * W);
    T acc = (T)0;
    if (o >= r && o + r < L) {
        // the window lies inside the line: no reflection (the same taps in the same order)
        const T* b0 = base + (int64_t)(o - r) * stride;
        for (int t = 0; t <= 2 * r; ++t) acc = fma(__ldg(taps + t), __ldg(b0 + (int64_t)t * stride), acc);
    } else {
        for (int t = -r; t <= r; ++t) {
            int q = o + t;
            q = q < 0 ? -q : (q >= L ? 2 * (L - 1) - q : q);
            acc = fma(__ldg(taps + t + r), __ldg(base + (int64_t)q * stride), acc);
        }
    }
    out[idx] = acc;
}

template <typename T>
__global__ void k_blur1d_t(const T* __restrict__ v, T* __restrict__ out, int64_t total, int H, int W, int axis,
                           const T* __restrict__ taps, int r) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int64_t p = idx / ((int64_t)H * W);
    const int rem = (int)(idx - p * H * W), y = rem / W, x = rem - (rem / W) * W;
    const int L = axis == 0 ? H : W, i = axis == 0 ? y : x, stride = axis == 0 ? W : 1;
    const T* base = v + p * H * W + (axis == 0 ? x : y * W);
    T acc = (T)0;
    const int a0 = i - r > 0 ? i - r : 0, a1 = i + r < L - 1 ? i + r : L - 1;
    for (int o = a0; o <= a1; ++o) acc = fma(__ldg(taps + (i - o) + r), __ldg(base + (int64_t)o * stride), acc);
    if (i >= 1 && i <= r)
        for (int o = 0; o <= r - i; ++o) acc = fma(__ldg(taps + (-i - o) + r), __ldg(base + (int64_t)o * stride), acc);
    if (i <= L - 2 && i >= L - 1 - r)
        for (int o = 2 * (L - 1) - i - r; o <= L - 1; ++o)
            acc = fma(__ldg(taps + (2 * (L - 1) - i - o) + r), __ldg(base + (int64_t)o * stride), acc);
    out[idx] = acc;
}

// ---- soft-argmax band sharpness ------------------------------------------------------------
// Per pattern (one block): J_p = sum_i s_i c_i over the Radon-mask cells, s = softmax(c / tau),
// and dJ_p / dc_i = s_i (1 + (c_i - J_p) / tau) (zero off the mask).  Sums in float64.
template <typename T>
__global__ void k_softargmax(const T* __restrict__ c, int64_t ncell, const int32_t* __restrict__ cells, int ncm,
                             double inv_tau, double* __restrict__ Jp, T* __restrict__ grad) {
    // float patterns take the exponentials in float (their arguments formed in double), double
    // patterns in double; the sums are double either way
    __shared__ double red[64];
    const int64_t p = blockIdx.x;
    const T* cp = c + p * ncell;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    double mx = -INFINITY;
    for (int k = tid; k < ncm; k += blockDim.x) mx = fmax(mx, (double)cp[cells[k]] * inv_tau);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if (lane == 0) red[warp] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = red[0];
        for (int w = 1; w < nw; ++w) m = fmax(m, red[w]);
        red[63] = m;
    }
    __syncthreads();
    mx = red[63];
    auto expo = [&](double v) -> double {
        if (sizeof(T) == 4) return (double)expf((float)(v * inv_tau - mx));
        return exp(v * inv_tau - mx);
    };
    double s0 = 0.0, s1 = 0.0;
    for (int k = tid; k < ncm; k += blockDim.x) {
        const double v = (double)cp[cells[k]];
        const double e = expo(v);
        s0 += e;
        s1 += e * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
    }
    __syncthreads();
    if (lane == 0) { red[warp] = s0; red[32 + warp] = s1; }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < nw; ++w) { a += red[w]; b += red[32 + w]; }
        red[62] = a;
        red[61] = b / a;
        Jp[p] = b / a;
    }
    __syncthreads();
    const double S0 = red[62], J = red[61];
    T* gp = grad + p * ncell;
    for (int k = tid; k < ncm; k += blockDim.x) {
        const double v = (double)cp[cells[k]];
        const double si = expo(v) / S0;
        gp[cells[k]] = (T)(si * (1.0 + (v - J) * inv_tau));
    }
}

// ---- NLPAR weights as functions of the patterns ----------------------------------------------
// sigma (nlpar_cpu.py:753-796, nn = 1) with the neighbour that attains the minimum and its pair
// count: sig2 = sigma^2 as the weights use it, arg = that neighbour (-1: none), nsig = its count.
__global__ void k_sigma_arg(const float* __restrict__ data, int nrows, int ncols, int npx,
                            const int32_t* __restrict__ ind, int nind, float mxval, float* __restrict__ sig2,
                            int* __restrict__ arg, float* __restrict__ nsig) {
    // eight lanes per scan pixel, one per neighbour of the 3x3 neighbourhood in raster order
    // (the centre skipped); each lane sums its pair in pair_ssd's order, then the pixel's first
    // lane takes the minimum in raster order (strict <, the first of equal values), as a
    // sequential scan of the eight pairs would
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int pix = t >> 3, slot = t & 7;
    const int npix = nrows * ncols;
    const int kk = slot < 4 ? slot : slot + 1;  // 3x3 index, the centre (4) skipped
    float s0 = 1e24f, n2 = 0.0f;
    int nb = -1;
    if (pix < npix) {
        const int j = pix / ncols, i = pix - (pix / ncols) * ncols;
        const int jn = j + kk / 3 - 1, inn = i + kk % 3 - 1;
        if (jn >= 0 && jn < nrows && inn >= 0 && inn < ncols) {
            nb = inn + ncols * jn;
            float d2;
            pair_ssd(data + (int64_t)pix * npx, data + (int64_t)nb * npx, ind, nind, mxval, d2, n2);
            n2 = __fadd_rn(n2, 1.0e-12f);
            if (d2 >= 1.e-3f) s0 = __fdiv_rn(d2, __fmul_rn(n2, 2.0f));
            else nb = -1;
        }
    }
    const int lane = threadIdx.x & 31, base = lane & ~7;
    float best = 1e24f, bn = 0.0f;
    int ba = -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float v = __shfl_sync(0xffffffffu, s0, base + k);
        const float vn = __shfl_sync(0xffffffffu, n2, base + k);
        const int vb = __shfl_sync(0xffffffffu, nb, base + k);
        if (vb >= 0 && v < best) { best = v; ba = vb; bn = vn; }
    }
    if (pix < npix && slot == 0) {
        const float sg = sqrtf(best);
        sig2[pix] = __fmul_rn(sg, sg);
        arg[pix] = ba;
        nsig[pix] = bn;
    }
}

// Window weights with the pieces of their derivative (one block per scan pixel, one thread per
// slot): w (normalised), m = max(d - dthresh, 0), and for the normalised distance
// d = (S - n s) / (s sqrt(2 n)) (s = sigma_p^2 + sigma_c^2): dS = dd/dS = 1 / (s sqrt(2 n)),
// ds = dd/ds = -S / (s^2 sqrt(2 n)); both 0 at the centre slot and where d is set to 1e6 n.
__global__ void k_nlpar_weights_d(const float* __restrict__ data, int nrows, int ncols, int npx,
                                  const int32_t* __restrict__ ind, int nind, float mxval,
                                  const float* __restrict__ sig2, float lam2, float dthresh, int sr,
                                  float* __restrict__ wout, float* __restrict__ mout, float* __restrict__ dsout,
                                  float* __restrict__ dgout) {
    extern __shared__ float w_s[];
    __shared__ float tot_s;
    const int pix = blockIdx.x;
    const int j = pix / ncols, i = pix - (pix / ncols) * ncols;
    int xs, xe, ys, ye;
    window(i, sr, ncols, xs, xe);
    window(j, sr, nrows, ys, ye);
    const int wx = xe - xs, winsz = (2 * sr + 1) * (2 * sr + 1);
    const int c = threadIdx.x;
    float m = 0.0f, dS = 0.0f, dg = 0.0f;
    if (c < winsz) {
        const int nb = (xs + c % wx) + ncols * (ys + c / wx);
        float w;
        if (nb == pix) {
            w = -1.0e6f;
        } else {
            float d2, n2;
            pair_ssd(data + (int64_t)pix * npx, data + (int64_t)nb * npx, ind, nind, mxval, d2, n2);
            const float ss = __fadd_rn(sig2[pix], sig2[nb]);
            const float S = d2;
            d2 = __fsub_rn(d2, __fmul_rn(n2, ss));
            const float dnorm = __fmul_rn(ss, sqrtf(__fmul_rn(2.0f, n2)));
            if (dnorm > 1.e-8f) {
                w = __fdiv_rn(d2, dnorm);
                dS = 1.0f / dnorm;
                dg = -S / (ss * dnorm);
            } else {
                w = __fmul_rn(1e6f, n2);
            }
        }
        m = fmaxf(__fsub_rn(w, dthresh), 0.0f);
        if (!(w - dthresh > 0.0f)) { dS = 0.0f; dg = 0.0f; }  // clamped: no derivative
        w_s[c] = expf(__fmul_rn(__fmul_rn(-1.0f, m), lam2));
    }
    __syncthreads();
    if (c == 0) {
        float t = 0.0f;
        for (int k = 0; k < winsz; ++k) t = __fadd_rn(t, w_s[k]);
        tot_s = t;
    }
    __syncthreads();
    if (c < winsz) {
        const int64_t o = (int64_t)pix * winsz + c;
        wout[o] = __fdiv_rn(w_s[c], tot_s);
        mout[o] = m;
        dsout[o] = dS;
        dgout[o] = dg;
    }
}

// G[p][c] = g_p . x_c over all pattern pixels (float64 sums); one block per scan pixel, one warp
// per window slot at a time.
template <typename T>
__global__ void k_nlpar_dots(const T* __restrict__ g, const T* __restrict__ x, int nrows, int ncols, int npx, int sr,
                             double* __restrict__ G) {
    const int p = blockIdx.x;
    const int jp = p / ncols, ip = p - (p / ncols) * ncols;
    int xs, xe, ys, ye;
    window(ip, sr, ncols, xs, xe);
    window(jp, sr, nrows, ys, ye);
    const int wx = xe - xs, winsz = (2 * sr + 1) * (2 * sr + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T* gp = g + (int64_t)p * npx;
    for (int c = warp; c < winsz; c += nw) {
        const int nb = (xs + c % wx) + ncols * (ys + c / wx);
        const T* xc = x + (int64_t)nb * npx;
        double acc = 0.0;
        if (sizeof(T) == 4) {
            // float patterns: each lane's products summed in float with Kahan's compensation
            // (off the slow FP64 pipe), the lanes' sums combined in double
            float sum = 0.0f, comp = 0.0f;
            for (int k = lane; k < npx; k += 32) {
                const float y = __fsub_rn(__fmul_rn((float)__ldg(gp + k), (float)__ldg(xc + k)), comp);
                const float t = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(t, sum), y);
                sum = t;
            }
            acc = (double)sum - (double)comp;
        } else {
            for (int k = lane; k < npx; k += 32) acc += (double)__ldg(gp + k) * (double)__ldg(xc + k);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) G[(int64_t)p * winsz + c] = acc;
    }
}

// Per scan pixel p: Gbar = sum_c w_pc G_pc; dJ/dd_pc = -(w_pc / lam^2) (G_pc - Gbar) where the
// weight's exponent is not clamped; alpha = dJ/dd * dd/dS, beta = dJ/dd * dd/ds; and the lambda
// term sum_c w_pc (2 m_pc / lam^3) (G_pc - Gbar).
__global__ void k_nlpar_coef(const double* __restrict__ G, const float* __restrict__ w, const float* __restrict__ m,
                             const float* __restrict__ dS, const float* __restrict__ dg, int npix, int winsz,
                             double lam, double* __restrict__ alpha, double* __restrict__ beta,
                             double* __restrict__ glam) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int64_t o = (int64_t)p * winsz;
    double gbar = 0.0;
    for (int c = 0; c < winsz; ++c) gbar += (double)w[o + c] * G[o + c];
    const double il2 = 1.0 / (lam * lam), c3 = 2.0 / (lam * lam * lam);
    double gl = 0.0;
    for (int c = 0; c < winsz; ++c) {
        const double dg_ = G[o + c] - gbar;
        const double a = -(double)w[o + c] * il2 * dg_;
        alpha[o + c] = a * (double)dS[o + c];
        beta[o + c] = a * (double)dg[o + c];
        gl += (double)w[o + c] * c3 * (double)m[o + c] * dg_;
    }
    glam[p] = gl;
}

// gamma_q = dJ / d sigma_q^2 = sum of beta over the pairs that hold q (as window centre or as
// neighbour); s_pc = sigma_p^2 + sigma_c^2 enters both.
__global__ void k_nlpar_gamma(const double* __restrict__ beta, int nrows, int ncols, int sr,
                              double* __restrict__ gamma) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows * ncols) return;
    const int winsz = (2 * sr + 1) * (2 * sr + 1), wx = 2 * sr + 1;
    const int jq = q / ncols, iq = q - (q / ncols) * ncols;
    double acc = 0.0;
    for (int c = 0; c < winsz; ++c) acc += beta[(int64_t)q * winsz + c];
    const int j0 = jq - 2 * sr < 0 ? 0 : jq - 2 * sr, j1 = jq + 2 * sr > nrows - 1 ? nrows - 1 : jq + 2 * sr;
    const int i0 = iq - 2 * sr < 0 ? 0 : iq - 2 * sr, i1 = iq + 2 * sr > ncols - 1 ? ncols - 1 : iq + 2 * sr;
    for (int jp = j0; jp <= j1; ++jp) {
        int ys, ye;
        window(jp, sr, nrows, ys, ye);
        if (jq < ys || jq >= ye) continue;
        for (int ip = i0; ip <= i1; ++ip) {
            int xs, xe;
            window(ip, sr, ncols, xs, xe);
            if (iq < xs || iq >= xe) continue;
            const int p = ip + ncols * jp;
            if (p == q) continue;
            acc += beta[(int64_t)p * winsz + (jq - ys) * wx + (iq - xs)];
        }
    }
    gamma[q] = acc;
}

// dJ/dx_q[k] from the weights' dependence on the patterns: the pair SSDs of q's own window, of
// the windows that hold q, and the noise sigma's minimising pair (q's own, and those of the
// 3x3 neighbours whose minimum pairs with q).  Masked pixels only, each pair's saturation test.
// d/dx of the weights' pattern dependence, one block per scan pixel q, its threads over the
// pattern values k.  The terms that reach q -- its own window slots (the pair distances it
// enters as the centre), the windows of the pixels whose windows hold q, and the noise sigma
// of q and of the neighbours whose sigma pairs end at q -- are listed once per block with
// their coefficients (2 alpha, gamma / n), then every value k adds coef * (x_q - x_n) for the
// terms whose two values pass the saturation test of their kind.  Sums in the pixel's order;
// float patterns accumulate in float (the coefficients rounded once), double in double.
template <typename T>
__global__ void __launch_bounds__(128) k_nlpar_dx(const T* __restrict__ x, int nrows, int ncols, int npx, int sr,
                                                  const uint8_t* __restrict__ pmask, float mxw, float mxs,
                                                  const double* __restrict__ alpha, const double* __restrict__ gamma,
                                                  const int* __restrict__ arg, const float* __restrict__ nsig,
                                                  T* __restrict__ out) {
    extern __shared__ unsigned char dxsm[];
    const int q = blockIdx.x;
    const int winsz = (2 * sr + 1) * (2 * sr + 1), wx = 2 * sr + 1;
    const int maxt = winsz + (4 * sr + 1) * (4 * sr + 1) + 9;
    T* co = (T*)dxsm;                        // [maxt] coefficients
    int* nbs = (int*)(co + maxt);           // [maxt] the other pixel; bit 31: a sigma term
    __shared__ int nterm;
    if (threadIdx.x == 0) {
        int t = 0;
        const int jq = q / ncols, iq = q - (q / ncols) * ncols;
        {
            int xs, xe, ys, ye;
            window(iq, sr, ncols, xs, xe);
            window(jq, sr, nrows, ys, ye);
            const int wq = xe - xs;
            for (int c = 0; c < winsz; ++c) {
                const int nb = (xs + c % wq) + ncols * (ys + c / wq);
                if (nb == q) continue;
                co[t] = (T)(2.0 * alpha[(int64_t)q * winsz + c]);
                nbs[t++] = nb;
            }
        }
        const int j0 = jq - 2 * sr < 0 ? 0 : jq - 2 * sr, j1 = jq + 2 * sr > nrows - 1 ? nrows - 1 : jq + 2 * sr;
        const int i0 = iq - 2 * sr < 0 ? 0 : iq - 2 * sr, i1 = iq + 2 * sr > ncols - 1 ? ncols - 1 : iq + 2 * sr;
        for (int jp = j0; jp <= j1; ++jp) {
            int ys, ye;
            window(jp, sr, nrows, ys, ye);
            if (jq < ys || jq >= ye) continue;
            for (int ip = i0; ip <= i1; ++ip) {
                int xs, xe;
                window(ip, sr, ncols, xs, xe);
                if (iq < xs || iq >= xe) continue;
                const int p = ip + ncols * jp;
                if (p == q) continue;
                co[t] = (T)(2.0 * alpha[(int64_t)p * winsz + (jq - ys) * wx + (iq - xs)]);
                nbs[t++] = p;
            }
        }
        // noise sigma: sigma_p^2 = SSD(p, arg_p) / (2 n_p)
        const int aq = arg[q];
        if (aq >= 0) {
            co[t] = (T)(gamma[q] / (double)nsig[q]);
            nbs[t++] = aq | (int)0x80000000u;
        }
        for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
                const int jn = jq + dj, in_ = iq + di;
                if ((dj == 0 && di == 0) || jn < 0 || jn >= nrows || in_ < 0 || in_ >= ncols) continue;
                const int p = in_ + ncols * jn;
                if (arg[p] != q) continue;
                co[t] = (T)(gamma[p] / (double)nsig[p]);
                nbs[t++] = p | (int)0x80000000u;
            }
        nterm = t;
    }
    __syncthreads();
    const int nt = nterm;
    const T* xq_row = x + (int64_t)q * npx;
    for (int k = threadIdx.x; k < npx; k += blockDim.x) {
        T acc = (T)0;
        if (pmask[k]) {
            const T xq = xq_row[k];
            const bool qw = xq < (T)mxw, qs = xq < (T)mxs;
            for (int t = 0; t < nt; ++t) {
                const int e = nbs[t];
                const bool sigma_term = e < 0;
                const T xn = x[(int64_t)(e & 0x7fffffff) * npx + k];
                if (sigma_term ? (qs && xn < (T)mxs) : (qw && xn < (T)mxw)) acc += co[t] * (xq - xn);
            }
        }
        out[(int64_t)q * npx + k] = acc;
    }
}

}  // namespace
}  // namespace ebsd

using namespace ebsd;

extern "C" {

int ebsd_linop_create(int64_t nrows, int64_t ncols, const int64_t* rowptr, const int32_t* col, const float* val,
                      int device, ebsd_linop_t* out) {
    if (!out || nrows <= 0 || ncols <= 0 || !rowptr || (!col && rowptr[nrows] > 0) || (!val && rowptr[nrows] > 0))
        return EBSD_E_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return EBSD_E_DEVICE;
    int64_t nnz = rowptr[nrows];
    for (int64_t e = 0; e < nnz; ++e)
        if (col[e] < 0 || col[e] >= ncols) return EBSD_E_ARG;
    ebsd_linop_s* op = new (std::nothrow) ebsd_linop_s();
    if (!op) return EBSD_E_NOMEM;
    op->device = device;
    op->nrows = nrows;
    op->ncols = ncols;
    op->nnz = nnz;
    std::vector<double> v64(val, val + nnz);
    bool ok = cudaMalloc((void**)&op->rowptr, (nrows + 1) * sizeof(int64_t)) == cudaSuccess &&
              cudaMalloc((void**)&op->col, std::max<int64_t>(nnz, 1) * sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc((void**)&op->val, std::max<int64_t>(nnz, 1) * sizeof(float)) == cudaSuccess &&
              cudaMalloc((void**)&op->val64, std::max<int64_t>(nnz, 1) * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMemcpy(op->rowptr, rowptr, (nrows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && nnz > 0) {
        ok = cudaMemcpy(op->col, col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(op->val, val, nnz * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(op->val64, v64.data(), nnz * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        cudaFree(op->rowptr);
        cudaFree(op->col);
        cudaFree(op->val);
        cudaFree(op->val64);
        delete op;
        return EBSD_E_NOMEM;
    }
    *out = op;
    return EBSD_OK;
}

int ebsd_linop_apply(ebsd_linop_t op, int fp64, const void* d_x, int64_t n, void* d_y, void* stream) {
    if (!op || n < 0 || (n > 0 && (!d_x || !d_y)) || n > 65535) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if (cudaSetDevice(op->device) != cudaSuccess) return EBSD_E_DEVICE;
    dim3 grid((unsigned)((op->nrows + 255) / 256), (unsigned)n);
    if (fp64)
        k_csr_gather<double><<<grid, 256, 0, (cudaStream_t)stream>>>(op->rowptr, op->col, op->val64,
                                                                    (const double*)d_x, (double*)d_y,
                                                                    op->nrows, op->ncols);
    else
        k_csr_gather<float><<<grid, 256, 0, (cudaStream_t)stream>>>(op->rowptr, op->col, op->val,
                                                                   (const float*)d_x, (float*)d_y,
                                                                   op->nrows, op->ncols);
    return launch_status();
}

int ebsd_linop_apply_cols(ebsd_linop_t op, int fp64, const void* d_xT, int64_t ldx, int64_t n, void* d_yT,
                          int64_t ldy, void* stream) {
    if (!op || n < 0 || (n > 0 && (!d_xT || !d_yT)) || ldx < n || ldy < n || (n + 31) / 32 > 65535) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if ((op->nrows + 7) / 8 > 0x7fffffff) return EBSD_E_ARG;
    if (cudaSetDevice(op->device) != cudaSuccess) return EBSD_E_DEVICE;
    const dim3 grid((unsigned)((op->nrows + 7) / 8), (unsigned)((n + 31) / 32)), block(32, 8);
    if (fp64)
        k_csr_gather_cols<double><<<grid, block, 0, (cudaStream_t)stream>>>(
            op->rowptr, op->col, op->val64, (const double*)d_xT, ldx, (double*)d_yT, ldy, op->nrows, n);
    else
        k_csr_gather_cols<float><<<grid, block, 0, (cudaStream_t)stream>>>(
            op->rowptr, op->col, op->val, (const float*)d_xT, ldx, (float*)d_yT, ldy, op->nrows, n);
    return launch_status();
}

int ebsd_linop_destroy(ebsd_linop_t op) {
    if (!op) return EBSD_E_ARG;
    cudaSetDevice(op->device);
    cudaFree(op->rowptr);
    cudaFree(op->col);
    cudaFree(op->val);
    cudaFree(op->val64);
    delete op;
    return EBSD_OK;
}

int ebsd_nlpar_weights(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                       int32_t nind, float datamax, float lam, int32_t sr, float dthresh, const float* d_sigma,
                       int saturation_protect, float* d_w, float* d_m, void* stream) {
    if (!d_data || !d_indices || !d_sigma || !d_w || !d_m || nrows <= 0 || ncols <= 0 || npx <= 0 || nind < 0 ||
        nind > npx || sr < 0 || sr > 10 || !(lam > 0.0f) || 2 * sr + 1 > nrows || 2 * sr + 1 > ncols)
        return EBSD_E_ARG;
    float mxval = saturation_protect ? datamax * 0.999f : datamax + 1.0f;
    float lam2 = 1.0f / (lam * lam);
    int winsz = (2 * sr + 1) * (2 * sr + 1);
    k_nlpar_weights2<<<(unsigned)(nrows * ncols), ((winsz + 31) / 32) * 32, winsz * sizeof(float),
                       (cudaStream_t)stream>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval, d_sigma, lam2,
                                               dthresh, sr, d_w, d_m);
    return launch_status();
}

int ebsd_blur1d(int fp64, int adjoint, int axis, const void* d_in, int64_t n, int32_t H, int32_t W,
                const void* d_taps, int32_t r, void* d_out, void* stream) {
    if (!d_in || !d_taps || !d_out || n < 0 || H <= 0 || W <= 0 || r < 0 || (axis != 0 && axis != 1) ||
        r >= (axis == 0 ? H : W))
        return EBSD_E_ARG;
    const int64_t total = n * H * W;
    if (total == 0) return EBSD_OK;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (fp64) {
        if (adjoint) k_blur1d_t<double><<<blocks, 256, 0, st>>>((const double*)d_in, (double*)d_out, total, H, W, axis, (const double*)d_taps, r);
        else k_blur1d<double><<<blocks, 256, 0, st>>>((const double*)d_in, (double*)d_out, total, H, W, axis, (const double*)d_taps, r);
    } else {
        if (adjoint) k_blur1d_t<float><<<blocks, 256, 0, st>>>((const float*)d_in, (float*)d_out, total, H, W, axis, (const float*)d_taps, r);
        else k_blur1d<float><<<blocks, 256, 0, st>>>((const float*)d_in, (float*)d_out, total, H, W, axis, (const float*)d_taps, r);
    }
    return launch_status();
}

int ebsd_softargmax(int fp64, const void* d_c, int64_t n, int64_t ncell, const int32_t* d_cells, int32_t ncm,
                    double tau, double* d_J, void* d_grad, void* stream) {
    if (!d_c || !d_cells || !d_J || !d_grad || n < 0 || ncell <= 0 || ncm <= 0 || ncm > ncell || !(tau > 0.0))
        return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (fp64) k_softargmax<double><<<(unsigned)n, 256, 0, st>>>((const double*)d_c, ncell, d_cells, ncm, 1.0 / tau, d_J, (double*)d_grad);
    else k_softargmax<float><<<(unsigned)n, 256, 0, st>>>((const float*)d_c, ncell, d_cells, ncm, 1.0 / tau, d_J, (float*)d_grad);
    return launch_status();
}

int ebsd_nlpar_sigma_arg(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                         int32_t nind, float datamax, int saturation_protect, float* d_sig2, int32_t* d_arg,
                         float* d_nsig, void* stream) {
    if (!d_data || !d_indices || !d_sig2 || !d_arg || !d_nsig || nrows <= 0 || ncols <= 0 || npx <= 0 || nind < 0 ||
        nind > npx)
        return EBSD_E_ARG;
    const float mxval = saturation_protect ? datamax * 0.9961f : datamax + 1.0f;
    const int npix = nrows * ncols;
    k_sigma_arg<<<(unsigned)(((int64_t)npix * 8 + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        d_data, nrows, ncols, npx, d_indices, nind, mxval, d_sig2, d_arg, d_nsig);
    return launch_status();
}

int ebsd_nlpar_weights_d(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, const int32_t* d_indices,
                         int32_t nind, float datamax, float lam, int32_t sr, float dthresh, const float* d_sig2,
                         int saturation_protect, float* d_w, float* d_m, float* d_dS, float* d_dsig, void* stream) {
    if (!d_data || !d_indices || !d_sig2 || !d_w || !d_m || !d_dS || !d_dsig || nrows <= 0 || ncols <= 0 ||
        npx <= 0 || nind < 0 || nind > npx || sr < 0 || sr > 10 || !(lam > 0.0f) || 2 * sr + 1 > nrows ||
        2 * sr + 1 > ncols)
        return EBSD_E_ARG;
    const float mxval = saturation_protect ? datamax * 0.999f : datamax + 1.0f;
    const int winsz = (2 * sr + 1) * (2 * sr + 1);
    k_nlpar_weights_d<<<(unsigned)(nrows * ncols), ((winsz + 31) / 32) * 32, winsz * sizeof(float),
                        (cudaStream_t)stream>>>(d_data, nrows, ncols, npx, d_indices, nind, mxval, d_sig2,
                                                1.0f / (lam * lam), dthresh, sr, d_w, d_m, d_dS, d_dsig);
    return launch_status();
}

int ebsd_nlpar_weights_grad(int fp64, const void* d_g, const void* d_x, int32_t nrows, int32_t ncols, int32_t npx,
                            int32_t sr, const float* d_w, const float* d_m, const float* d_dS, const float* d_dsig,
                            double lam, const uint8_t* d_pmask, float datamax, int saturation_protect,
                            const int32_t* d_arg, const float* d_nsig, double* d_scratch, double* d_glam,
                            void* d_gx, void* stream) {
    if (!d_g || !d_x || !d_w || !d_m || !d_dS || !d_dsig || !d_pmask || !d_arg || !d_nsig || !d_scratch ||
        !d_glam || !d_gx || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10 || !(lam > 0.0))
        return EBSD_E_ARG;
    const int npix = nrows * ncols, winsz = (2 * sr + 1) * (2 * sr + 1);
    double* G = d_scratch;
    double* alpha = G + (int64_t)npix * winsz;
    double* beta = alpha + (int64_t)npix * winsz;
    double* gamma = beta + (int64_t)npix * winsz;
    cudaStream_t st = (cudaStream_t)stream;
    const float mxw = saturation_protect ? datamax * 0.999f : datamax + 1.0f;
    const float mxs = saturation_protect ? datamax * 0.9961f : datamax + 1.0f;
    if (fp64) k_nlpar_dots<double><<<(unsigned)npix, 256, 0, st>>>((const double*)d_g, (const double*)d_x, nrows, ncols, npx, sr, G);
    else k_nlpar_dots<float><<<(unsigned)npix, 256, 0, st>>>((const float*)d_g, (const float*)d_x, nrows, ncols, npx, sr, G);
    k_nlpar_coef<<<(unsigned)((npix + 127) / 128), 128, 0, st>>>(G, d_w, d_m, d_dS, d_dsig, npix, winsz, lam, alpha,
                                                                 beta, d_glam);
    k_nlpar_gamma<<<(unsigned)((npix + 127) / 128), 128, 0, st>>>(beta, nrows, ncols, sr, gamma);
    const size_t maxt = (size_t)winsz + (size_t)(4 * sr + 1) * (4 * sr + 1) + 9;
    const size_t dsm = maxt * ((fp64 ? sizeof(double) : sizeof(float)) + sizeof(int));
    if (fp64) k_nlpar_dx<double><<<(unsigned)npix, 128, dsm, st>>>((const double*)d_x, nrows, ncols, npx, sr, d_pmask, mxw, mxs, alpha, gamma, d_arg, d_nsig, (double*)d_gx);
    else k_nlpar_dx<float><<<(unsigned)npix, 128, dsm, st>>>((const float*)d_x, nrows, ncols, npx, sr, d_pmask, mxw, mxs, alpha, gamma, d_arg, d_nsig, (float*)d_gx);
    return launch_status();
}

int ebsd_nlpar_apply_t(const float* d_g, int32_t nrows, int32_t ncols, int32_t npx, const float* d_w, int32_t sr,
                       float* d_out, void* stream) {
    if (!d_g || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10) return EBSD_E_ARG;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_apply_t<float><<<grid, 256, (size_t)(4 * sr + 1) * (4 * sr + 1) * (sizeof(float) + sizeof(int)),
                             (cudaStream_t)stream>>>(d_g, nrows, ncols, npx, d_w, sr, d_out);
    return launch_status();
}

int ebsd_nlpar_apply_t64(const double* d_g, int32_t nrows, int32_t ncols, int32_t npx, const double* d_w,
                         int32_t sr, double* d_out, void* stream) {
    if (!d_g || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10) return EBSD_E_ARG;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_apply_t<double><<<grid, 256, (size_t)(4 * sr + 1) * (4 * sr + 1) * (sizeof(double) + sizeof(int)),
                              (cudaStream_t)stream>>>(d_g, nrows, ncols, npx, d_w, sr, d_out);
    return launch_status();
}

int ebsd_nlpar_lambda_grad(const float* d_g, const float* d_x, int32_t nrows, int32_t ncols, int32_t npx,
                           const float* d_w, const float* d_m, int32_t sr, float lam, double* d_out,
                           void* stream) {
    if (!d_g || !d_x || !d_w || !d_m || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10 ||
        !(lam > 0.0f))
        return EBSD_E_ARG;
    k_nlpar_lam_grad<float><<<(unsigned)(nrows * ncols), 256, 0, (cudaStream_t)stream>>>(
        d_g, d_x, nrows, ncols, npx, d_w, d_m, sr, lam, d_out);
    return launch_status();
}

int ebsd_nlpar_lambda_grad64(const double* d_g, const double* d_x, int32_t nrows, int32_t ncols, int32_t npx,
                             const float* d_w, const float* d_m, int32_t sr, float lam, double* d_out,
                             void* stream) {
    if (!d_g || !d_x || !d_w || !d_m || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10 ||
        !(lam > 0.0f))
        return EBSD_E_ARG;
    k_nlpar_lam_grad<double><<<(unsigned)(nrows * ncols), 256, 0, (cudaStream_t)stream>>>(
        d_g, d_x, nrows, ncols, npx, d_w, d_m, sr, lam, d_out);
    return launch_status();
}

}  // extern "C"
