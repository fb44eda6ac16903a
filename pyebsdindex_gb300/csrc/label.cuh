// Band labelling device code shared by the per-stage and fused kernels.
//
// Restates band_label_numba (band_detect.py:691-809) and the find_bands epilogue
// (band_detect.py:457-460, :521-524) with the reference's float32 operation order: every
// add/sub/mul/div is an explicitly rounded intrinsic so that the compiler cannot contract a
// multiply-add into an FMA the reference does not perform.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <math.h>

#include "../../include/ebsdgpu.h"

namespace ebsd {

__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float r_log(float a) { return logf(a); }
__device__ __forceinline__ double r_log(double a) { return log(a); }
__device__ __forceinline__ float r_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double r_abs(double a) { return fabs(a); }

template <typename T> __device__ __forceinline__ T neg_inf();
template <> __device__ __forceinline__ float neg_inf<float>() { return -INFINITY; }
template <> __device__ __forceinline__ double neg_inf<double>() { return -INFINITY; }

// np.interp(x, arange(n), fp) in float64 (numpy arr_interp: clamp at both ends, exact hit
// returns the sample, else slope*(x - xj) + yj without a fused multiply-add).
__device__ __forceinline__ double interp_arange(double x, const double* fp, int n) {
    if (x != x) return x;
    if (x < 0.0) return fp[0];
    if (x >= (double)(n - 1)) return fp[n - 1];
    int j = (int)floor(x);
    if ((double)j == x) return fp[j];
    double slope = __dsub_rn(fp[j + 1], fp[j]);  // / (xp[j+1] - xp[j]) = / 1.0, exact
    return __dadd_rn(__dmul_rn(slope, __dsub_rn(x, (double)j)), fp[j]);
}

// Warp-wide top-N list: lanes 0..nB-1 hold (value, position) sorted by value, largest first;
// `pos < 0` marks an empty slot.  Inserting after all entries >= v keeps candidates that
// arrive earlier (row-major scan order) ahead on exact ties.
template <typename T>
__device__ __forceinline__ void topn_insert(T v, int pos, T& lv, int& lpos, int nB, int lane) {
    const unsigned full = 0xffffffffu;
    unsigned ge = __ballot_sync(full, lane < nB && lpos >= 0 && lv >= v);
    int ins = __popc(ge);
    if (ins < nB) {
        T upv = __shfl_up_sync(full, lv, 1);
        int upp = __shfl_up_sync(full, lpos, 1);
        if (lane > ins && lane < nB) { lv = upv; lpos = upp; }
        if (lane == ins) { lv = v; lpos = pos; }
    }
}

// Merge: insert every entry of another sorted list (held by lanes 0..nB-1 as ov/opos).
template <typename T>
__device__ __forceinline__ void topn_merge(T ov, int opos, T& lv, int& lpos, int nB, int lane) {
    for (int k = 0; k < nB; ++k) {
        T v = __shfl_sync(0xffffffffu, ov, k);
        int p = __shfl_sync(0xffffffffu, opos, k);
        if (p < 0) break;
        topn_insert(v, p, lv, lpos, nB, lane);
    }
}

struct LabelConsts {
    int p0, p1, nTheta, nRho, nB;
    const double* theta;  // degrees
    const double* rho;
};

// FWHM width from the peak's log-curvature a (band_detect.py:748-753): 2 sqrt(ln 2 / -a) in
// float64 when a < -1e-8, else 0.
template <typename T>
__device__ __forceinline__ T band_width(T a) {
    return a < (T)-1.e-8 ? (T)(2.0 * sqrt(0.6931471805599453 / (double)(-a))) : (T)0;
}

// theta = pi - interp(aveloc_theta)/RADEG ; rho = -interp(aveloc_rho) in float64
// (band_detect.py:521-522), from the record's aveloc as stored (float32 for T = float).
template <typename T>
__device__ __forceinline__ void band_theta_rho(T ar, T ac, const LabelConsts& k, float* theta, float* rho) {
    double xt = (sizeof(T) == 4) ? (double)(float)ac : (double)ac;
    double xr = (sizeof(T) == 4) ? (double)(float)ar : (double)ar;
    const double RADEG = 180.0 / 3.141592653589793;
    double th = __dsub_rn(3.141592653589793, __ddiv_rn(interp_arange(xt, k.theta, k.nTheta), RADEG));
    double rh = -interp_arange(xr, k.rho, k.nRho);
    *theta = (float)th;
    *rho = (float)rh;
}

// Fit one band (padded-frame peak (r, c)) from its 3x3 block nn of LoG-convolved Radon values
// (nn[i*3 + j] = conv(r - 1 + i, c - 1 + j)) and write its record fields.  kEpilogue = false
// leaves the float64 epilogue to a separate pass: the width field then holds the
// log-curvature a (or 0) and theta/rho are not written.
template <typename T, bool kEpilogue = true>
__device__ void band_fit_block(bool has, int r, int c, const T* nn_in, T mn, T mean,
                               const LabelConsts& k, const ebsd_bands& out, int64_t o) {
    T vmax = (T)-2.0e6, vavemax = (T)-2.0e6, acurv = (T)0;
    T mlr = (T)0, mlc = (T)0, alr = (T)0, alc = (T)0;
    int8_t valid = 0;
    if (has) {
        T v = nn_in[4];
        if (v > (T)0) {
            valid = 1;
            mlr = (T)r;
            mlc = (T)c;
            vmax = v;
            T ym = nn_in[1], yp = nn_in[7];
            T m3 = ym < v ? ym : v;
            m3 = yp < m3 ? yp : m3;
            if (m3 > (T)0) {
                T a = r_sub(r_mul(r_sub(r_log(yp), r_log(ym)), (T)0.5), r_log(v));
                if (a < (T)-1.e-8) acurv = a;
            }
            T nn[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) nn[i] = nn_in[i];
            // numpy float32 sum of 9 contiguous values: 8-way pairwise block, then the tail.
            T s = r_add(r_add(r_add(nn[0], nn[1]), r_add(nn[2], nn[3])),
                        r_add(r_add(nn[4], nn[5]), r_add(nn[6], nn[7])));
            s = r_add(s, nn[8]);
            s = s > (T)1e-12 ? s : (T)1e-12;
#pragma unroll
            for (int i = 0; i < 9; ++i) nn[i] = r_div(nn[i], s);
            vavemax = r_div(s, (T)9);
            T dx = r_mul((T)0.5, r_sub(nn[5], nn[3]));
            T dy = r_mul((T)0.5, r_sub(nn[7], nn[1]));
            T dxx = r_sub(r_add(nn[5], nn[3]), r_mul((T)2, nn[4]));
            T dyy = r_sub(r_add(nn[7], nn[1]), r_mul((T)2, nn[4]));
            T dxy = r_mul((T)0.25, r_add(r_sub(r_sub(nn[8], nn[2]), nn[6]), nn[0]));
            const T big = (T)(1.0 / 1e-12);
            T det = r_sub(r_mul(dxx, dyy), r_mul(dxy, dxy));
            det = r_abs(det) > (T)1e-12 ? r_div((T)1, det) : big;
            T dc = r_mul(r_sub(r_mul(dyy, dx), r_mul(dxy, dy)), det);
            T rc = r_mul(r_sub(r_mul(dxx, dy), r_mul(dxy, dx)), det);
            if (r_abs(dc) > (T)0.875 || r_abs(rc) > (T)0.875) {
                det = r_mul(dxx, dyy);
                det = r_abs(det) > (T)1e-12 ? r_div((T)1, det) : big;
                dc = r_mul(r_mul(dyy, dx), det);
                rc = r_mul(r_mul(dxx, dy), det);
                if (r_abs(dc) > (T)0.875 || r_abs(rc) > (T)0.875) {
                    dc = (T)0;
                    rc = (T)0;
                }
            }
            alr = r_sub((T)r, rc);
            alc = r_sub((T)c, dc);
        }
    }
    // padding removal (band_detect.py:686-687): one rounding of the exact difference
    T ar = r_sub(alr, (T)k.p0), ac = r_sub(alc, (T)k.p1);
    out.max[o] = (float)vmax;
    T nm = r_div(r_sub(vmax, mn), (r_sub(mean, mn) > (T)1e-7f ? r_sub(mean, mn) : (T)1e-7f));
    out.normmax[o] = (float)nm;
    out.maxloc[2 * o] = (float)(mlr - (T)k.p0);
    out.maxloc[2 * o + 1] = (float)(mlc - (T)k.p1);
    out.avemax[o] = (float)vavemax;
    out.aveloc[2 * o] = (float)ar;
    out.aveloc[2 * o + 1] = (float)ac;
    out.valid[o] = valid;
    if (kEpilogue) {
        out.width[o] = (float)band_width(acurv);
        band_theta_rho(ar, ac, k, out.theta + o, out.rho + o);
    } else {
        out.width[o] = (float)acurv;
    }
}

// The same, reading the 3x3 block through C(r, c) (the LoG-convolved Radon value in the
// padded frame as T).
template <typename T, bool kEpilogue = true, typename Acc>
__device__ void band_fit_write(bool has, int r, int c, const Acc& C, T mn, T mean,
                               const LabelConsts& k, const ebsd_bands& out, int64_t o) {
    T nn[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) nn[i] = (T)0;
    if (has) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) nn[i * 3 + j] = C(r - 1 + i, c - 1 + j);
    }
    band_fit_block<T, kEpilogue>(has, r, c, nn, mn, mean, k, out, o);
}

}  // namespace ebsd
