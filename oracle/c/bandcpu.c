/*
 * bandcpu.c -- C/OpenMP restatement of the reference CPU band detection (the timed CPU
 * baseline and a fast oracle).  TEST / BENCHMARK INFRASTRUCTURE ONLY: called from tests/ and
 * from bench.py's CPU-baseline leg, never from the product library.
 *
 * Per pattern (one OpenMP thread each), following the reference step by step:
 *   radon   radon_fast.py:281-310   float32 sequential ray sums / count, missing rays = -1,
 *                                    background subtracted in float64 (radon_fast.py:255-259)
 *   pad     band_detect.py:573-580  theta mirror with rho flip, then rho edge copy
 *   conv    band_detect.py:596-606  'same' 2-D convolution, zero outside (evaluated directly,
 *                                    the reference uses an FFT)
 *   stats   band_detect.py:627-630  min / mean over the slice with the shprdn[1] rho bound
 *   peaks   band_detect.py:639-664  separable clipped max filter, exact equality, rdnmask
 *   label   band_detect.py:691-809  top-N by value, FWHM width, 3x3 Taylor sub-pixel step
 *   epilog  band_detect.py:457-460, :521-524   normmax, theta/rho interpolation
 * Compile with -ffp-contract=off so no multiply-add is fused.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int H, W, nTheta, nRho, nB, p0, p1, pk0, pk1, k0, k1, L;
    const float* kernel;      /* [k0*k1] */
    const int32_t* lut;       /* [nRho*nTheta][L], entries < 0 or >= H*W end the ray */
    const uint8_t* rdnmask;   /* [nRho*nTheta] */
    const double* theta;      /* [nTheta] degrees */
    const double* rho;        /* [nRho] */
    const double* bg;         /* [H*W] or NULL */
} bc_plan;

typedef struct {
    float *max, *normmax, *maxloc, *avemax, *aveloc, *width, *theta, *rho;
    int8_t* valid;
} bc_out;

static double interp_arange(double x, const double* fp, int n) {
    if (x != x) return x;
    if (x < 0.0) return fp[0];
    if (x >= (double)(n - 1)) return fp[n - 1];
    int j = (int)floor(x);
    if ((double)j == x) return fp[j];
    double slope = (fp[j + 1] - fp[j]) / 1.0;
    return slope * (x - (double)j) + fp[j];
}

static void one_pattern(const bc_plan* P, const void* pat, int dtype, float* radon, float* conv, float* tmp,
                        float* cval, int* cpos, const bc_out* o, int64_t q) {
    const int R = P->nRho + 2 * P->p0, Tp = P->nTheta + 2 * P->p1;
    const int nPx = P->H * P->W, nRays = P->nRho * P->nTheta;
    /* radon */
    for (int r = 0; r < nRays; ++r) {
        const int32_t* ray = P->lut + (size_t)r * P->L;
        float sum = 0.0f;
        int cnt = 0;
        for (int k = 0; k < P->L; ++k) {
            int idx = ray[k];
            if (idx < 0 || idx >= nPx) break;
            double v;
            if (dtype == 0) v = ((const uint8_t*)pat)[idx];
            else if (dtype == 1) v = ((const uint16_t*)pat)[idx];
            else v = ((const float*)pat)[idx];
            float fv = P->bg ? (float)(v - P->bg[idx]) : (float)v;
            sum = sum + fv;
            ++cnt;
        }
        int i = r / P->nTheta, j = r % P->nTheta;
        radon[(i + P->p0) * Tp + j + P->p1] = cnt ? sum / (float)cnt : -1.0f;
    }
    /* pad */
    for (int r = 0; r < R; ++r)
        for (int c = 0; c < Tp; ++c) {
            int i = r - P->p0, j = c - P->p1;
            if (i >= 0 && i < P->nRho && j >= 0 && j < P->nTheta) continue;
            int ic = i < 0 ? 0 : (i >= P->nRho ? P->nRho - 1 : i);
            int si = ic, sj = j;
            if (j < 0) { si = P->nRho - 1 - ic; sj = P->nTheta + j; }
            else if (j >= P->nTheta) { si = P->nRho - 1 - ic; sj = j - P->nTheta; }
            radon[r * Tp + c] = radon[(si + P->p0) * Tp + sj + P->p1];
        }
    /* conv */
    const int h0 = P->k0 / 2, h1 = P->k1 / 2;
    for (int r = 0; r < R; ++r)
        for (int c = 0; c < Tp; ++c) {
            float acc = 0.0f;
            for (int a = 0; a < P->k0; ++a) {
                int rr = r + h0 - a;
                if (rr < 0 || rr >= R) continue;
                for (int b = 0; b < P->k1; ++b) {
                    int cc = c + h1 - b;
                    if (cc < 0 || cc >= Tp) continue;
                    acc = fmaf(P->kernel[a * P->k1 + b], radon[rr * Tp + cc], acc);
                }
            }
            conv[r * Tp + c] = acc;
        }
    /* stats */
    int r1 = Tp - P->p0 < R ? Tp - P->p0 : R;
    double s = 0.0;
    float mn = INFINITY;
    int tot = 0;
    for (int r = P->p0; r < r1; ++r)
        for (int c = P->p1; c < Tp - P->p1; ++c) {
            float v = conv[r * Tp + c];
            s += v;
            mn = v < mn ? v : mn;
            ++tot;
        }
    float mean = (float)(s / (double)tot);
    /* dilation along theta then rho, on the rows/cols the interior windows reach */
    const int ht = P->pk1 / 2, hr = P->pk0 / 2;
    for (int r = 0; r < R; ++r)
        for (int c = 0; c < Tp; ++c) {
            int c0 = c - ht < 0 ? 0 : c - ht, c1 = c + ht > Tp - 1 ? Tp - 1 : c + ht;
            float m = -INFINITY;
            for (int cc = c0; cc <= c1; ++cc) m = conv[r * Tp + cc] > m ? conv[r * Tp + cc] : m;
            tmp[r * Tp + c] = m;
        }
    int ncand = 0;
    const int nB = P->nB;
    for (int i = 0; i < P->nRho; ++i)
        for (int j = 0; j < P->nTheta; ++j) {
            if (!P->rdnmask[i * P->nTheta + j]) continue;
            int r = i + P->p0, c = j + P->p1;
            int ra = r - hr < 0 ? 0 : r - hr, rb = r + hr > R - 1 ? R - 1 : r + hr;
            float m = -INFINITY;
            for (int rr = ra; rr <= rb; ++rr) m = tmp[rr * Tp + c] > m ? tmp[rr * Tp + c] : m;
            float v = conv[r * Tp + c];
            if (m != v) continue;
            /* insertion into a sorted top-nB list; earlier (row-major) candidates win ties */
            int pos = ncand < nB ? ncand : nB;
            while (pos > 0 && cval[pos - 1] < v) --pos;
            if (pos >= nB) continue;
            int last = ncand < nB ? ncand : nB - 1;
            for (int k = last; k > pos; --k) { cval[k] = cval[k - 1]; cpos[k] = cpos[k - 1]; }
            cval[pos] = v;
            cpos[pos] = r * Tp + c;
            if (ncand < nB) ++ncand;
        }
    /* label */
    for (int b = 0; b < nB; ++b) {
        int64_t oi = q * nB + b;
        float vmax = -2.0e6f, vavemax = -2.0e6f, w = 0.0f, mlr = 0, mlc = 0, alr = 0, alc = 0;
        int8_t valid = 0;
        if (b < ncand && conv[cpos[b]] > 0.0f) {
            int r = cpos[b] / Tp, c = cpos[b] % Tp;
            float v = conv[cpos[b]];
            valid = 1;
            mlr = (float)r;
            mlc = (float)c;
            vmax = v;
            float ym = conv[(r - 1) * Tp + c], yp = conv[(r + 1) * Tp + c];
            float m3 = ym < v ? ym : v;
            m3 = yp < m3 ? yp : m3;
            if (m3 > 0.0f) {
                float a = (logf(yp) - logf(ym)) * 0.5f - logf(v);
                if (a < -1.e-8f) w = (float)(2.0 * sqrt(0.6931471805599453 / (double)(-a)));
            }
            float nn[9];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) nn[i * 3 + j] = conv[(r - 1 + i) * Tp + c - 1 + j];
            float sm = ((nn[0] + nn[1]) + (nn[2] + nn[3])) + ((nn[4] + nn[5]) + (nn[6] + nn[7]));
            sm = sm + nn[8];
            sm = sm > 1e-12f ? sm : 1e-12f;
            for (int i = 0; i < 9; ++i) nn[i] = nn[i] / sm;
            vavemax = sm / 9.0f;
            float dx = 0.5f * (nn[5] - nn[3]), dy = 0.5f * (nn[7] - nn[1]);
            float dxx = (nn[5] + nn[3]) - 2.0f * nn[4], dyy = (nn[7] + nn[1]) - 2.0f * nn[4];
            float dxy = 0.25f * (((nn[8] - nn[2]) - nn[6]) + nn[0]);
            const float big = (float)(1.0 / 1e-12);
            float det = dxx * dyy - dxy * dxy;
            det = fabsf(det) > 1e-12f ? 1.0f / det : big;
            float dc = (dyy * dx - dxy * dy) * det, rc = (dxx * dy - dxy * dx) * det;
            if (fabsf(dc) > 0.875f || fabsf(rc) > 0.875f) {
                det = dxx * dyy;
                det = fabsf(det) > 1e-12f ? 1.0f / det : big;
                dc = (dyy * dx) * det;
                rc = (dxx * dy) * det;
                if (fabsf(dc) > 0.875f || fabsf(rc) > 0.875f) { dc = 0.0f; rc = 0.0f; }
            }
            alr = (float)r - rc;
            alc = (float)c - dc;
        }
        float ar = alr - (float)P->p0, ac = alc - (float)P->p1;
        o->max[oi] = vmax;
        float den = mean - mn;
        o->normmax[oi] = (vmax - mn) / (den > 1e-7f ? den : 1e-7f);
        o->maxloc[2 * oi] = mlr - (float)P->p0;
        o->maxloc[2 * oi + 1] = mlc - (float)P->p1;
        o->avemax[oi] = vavemax;
        o->aveloc[2 * oi] = ar;
        o->aveloc[2 * oi + 1] = ac;
        o->width[oi] = w;
        o->valid[oi] = valid;
        const double RADEG = 180.0 / 3.141592653589793;
        o->theta[oi] = (float)(3.141592653589793 - interp_arange((double)ac, P->theta, P->nTheta) / RADEG);
        o->rho[oi] = (float)(-interp_arange((double)ar, P->rho, P->nRho));
    }
}

int bandcpu_find_bands(const bc_plan* P, const void* pats, int dtype, int64_t n, const bc_out* o, int threads) {
    const int R = P->nRho + 2 * P->p0, Tp = P->nTheta + 2 * P->p1;
    const size_t esz = dtype == 0 ? 1 : (dtype == 1 ? 2 : 4);
    const size_t nPx = (size_t)P->H * P->W;
    if (P->nB > 64) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    int err = 0;
#pragma omp parallel
    {
        float* radon = (float*)malloc(sizeof(float) * (size_t)R * Tp);
        float* conv = (float*)malloc(sizeof(float) * (size_t)R * Tp);
        float* tmp = (float*)malloc(sizeof(float) * (size_t)R * Tp);
        float cval[64];
        int cpos[64];
        if (!radon || !conv || !tmp) {
#pragma omp atomic write
            err = -2;
        } else {
#pragma omp for schedule(dynamic, 4)
            for (int64_t q = 0; q < n; ++q)
                one_pattern(P, (const char*)pats + (size_t)q * nPx * esz, dtype, radon, conv, tmp, cval, cpos, o, q);
        }
        free(radon);
        free(conv);
        free(tmp);
    }
    return err;
}
