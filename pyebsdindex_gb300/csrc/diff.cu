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
__global__ void k_nlpar_apply_t(const T* __restrict__ g, int nrows, int ncols, int npx,
                                const T* __restrict__ w, int sr, T* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int q = blockIdx.y;
    if (k >= npx) return;
    int jq = q / ncols, iq = q - (q / ncols) * ncols;
    int winsz = (2 * sr + 1) * (2 * sr + 1), wx = 2 * sr + 1;
    T acc = (T)0;
    int j0 = jq - 2 * sr < 0 ? 0 : jq - 2 * sr, j1 = jq + 2 * sr > nrows - 1 ? nrows - 1 : jq + 2 * sr;
    int i0 = iq - 2 * sr < 0 ? 0 : iq - 2 * sr, i1 = iq + 2 * sr > ncols - 1 ? ncols - 1 : iq + 2 * sr;
    for (int jp = j0; jp <= j1; ++jp) {
        int ys, ye;
        window(jp, sr, nrows, ys, ye);
        if (jq < ys || jq >= ye) continue;
        for (int ip = i0; ip <= i1; ++ip) {
            int xs, xe;
            window(ip, sr, ncols, xs, xe);
            if (iq < xs || iq >= xe) continue;
            int p = ip + ncols * jp;
            int c = (jq - ys) * wx + (iq - xs);
            acc = fma(__ldg(w + (int64_t)p * winsz + c), __ldg(g + (int64_t)p * npx + k), acc);
        }
    }
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

int ebsd_nlpar_apply_t(const float* d_g, int32_t nrows, int32_t ncols, int32_t npx, const float* d_w, int32_t sr,
                       float* d_out, void* stream) {
    if (!d_g || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10) return EBSD_E_ARG;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_apply_t<float><<<grid, 256, 0, (cudaStream_t)stream>>>(d_g, nrows, ncols, npx, d_w, sr, d_out);
    return launch_status();
}

int ebsd_nlpar_apply_t64(const double* d_g, int32_t nrows, int32_t ncols, int32_t npx, const double* d_w,
                         int32_t sr, double* d_out, void* stream) {
    if (!d_g || !d_w || !d_out || nrows <= 0 || ncols <= 0 || npx <= 0 || sr < 0 || sr > 10) return EBSD_E_ARG;
    dim3 grid((unsigned)((npx + 255) / 256), (unsigned)(nrows * ncols));
    k_nlpar_apply_t<double><<<grid, 256, 0, (cudaStream_t)stream>>>(d_g, nrows, ncols, npx, d_w, sr, d_out);
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
