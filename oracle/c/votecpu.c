/*
 * C/OpenMP restatement of the reference's triplet voting, BandIndexer.bandindex
 * (PyEBSDIndex v0.3.10.1 tripletvote.py:492-633, with high_fidelity on).
 *
 * TEST / BENCHMARK INFRASTRUCTURE ONLY: the multi-core CPU baseline of the device band indexer
 * (bench.py's indexing leg) and a second oracle in tests/.  It follows oracle/vote_oracle.py
 * (the numpy restatement, bit-identical to the reference) step by step:
 *   - band-band angles: float32 3-term dot products as BLAS's fused multiply-add chain,
 *     arccos * RADEG in float32 (tripletvote.py:1181-1188);
 *   - the vote over band triplets with the library's float64 angle tests, float32 weights
 *     added in library order (:1023-1135), vote metrics and band rank (:1137-1191);
 *   - the TRIAD search over band pairs in rank order with early exit (:1483-1690);
 *   - QUEST weights (:856-901), the float64 QUEST solve and fits (:903-1020), the vote
 *     confidence (:2057-2075);
 *   - sums in numpy's pairwise order, ties in ranks broken by band order (stable sorts).
 * Built with -ffp-contract=off: every float operation is rounded on its own unless written
 * as fmaf / fma.  arccos is libm's acosf (numpy's float32 arccos may differ by an ulp).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXB 32
#define MAXF 16

typedef struct {
    int nfam, ntrip, npoles, early, simpleq;
    double tol;
    const double* trip_angles; /* [ntrip][3] */
    const int64_t* trip_family; /* [ntrip][3] */
    const int64_t* lut;         /* [3][3][3][3] */
    const double* poles;        /* [npoles][3] */
    const int32_t* pfam;        /* [npoles] */
    const double* angtab;       /* [npoles][npoles] */
    const int32_t* famcnt;      /* [nfam] */
    const int64_t* famidx;      /* [nfam] */
} VoteLib;

static const double RADEG = 57.29577951308232;

static float dot3f(const float* a, const float* b) { return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0])); }

static void cross3f(const float* a, const float* b, float* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static float acos_deg(float x) { return acosf(x) * (float)RADEG; }

/* numpy's pairwise summation of a contiguous run (n <= 512 here) */
static float pw_f(const float* a, int n) {
    if (n < 8) {
        float r = 0.0f;
        for (int i = 0; i < n; ++i) r += a[i];
        return r;
    }
    if (n <= 128) {
        float r[8];
        for (int j = 0; j < 8; ++j) r[j] = a[j];
        int i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; ++j) r[j] += a[i + j];
        float res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) res += a[i];
        return res;
    }
    int h = n / 2;
    h -= h % 8;
    return pw_f(a, h) + pw_f(a + h, n - h);
}

static double pw_d(const double* a, int n) {
    if (n < 8) {
        double r = 0.0;
        for (int i = 0; i < n; ++i) r += a[i];
        return r;
    }
    if (n <= 128) {
        double r[8];
        for (int j = 0; j < 8; ++j) r[j] = a[j];
        int i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; ++j) r[j] += a[i + j];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) res += a[i];
        return res;
    }
    int h = n / 2;
    h -= h % 8;
    return pw_d(a, h) + pw_d(a + h, n - h);
}

static void argsort3f(const float* v, int* s) {
    int t;
    s[0] = 0; s[1] = 1; s[2] = 2;
    if (v[s[0]] > v[s[2]]) { t = s[2]; s[2] = s[0]; s[0] = t; }
    if (v[s[0]] > v[s[1]]) { t = s[1]; s[1] = s[0]; s[0] = t; }
    if (v[s[1]] > v[s[2]]) { t = s[2]; s[2] = s[1]; s[1] = t; }
}

static void argsort3i(const int* v, int* s) {
    int t;
    s[0] = 0; s[1] = 1; s[2] = 2;
    if (v[s[0]] > v[s[2]]) { t = s[2]; s[2] = s[0]; s[0] = t; }
    if (v[s[0]] > v[s[1]]) { t = s[1]; s[1] = s[0]; s[0] = t; }
    if (v[s[1]] > v[s[2]]) { t = s[2]; s[2] = s[1]; s[1] = t; }
}

/* position of each element in a stable ascending order */
static void stable_rank(const float* v, int n, int* order) {
    for (int b = 0; b < n; ++b) {
        int pos = 0;
        for (int c = 0; c < n; ++c) pos += (v[c] < v[b]) || (v[c] == v[b] && c < b);
        order[pos] = b;
    }
}

static void index_one(const VoteLib* L, const float* bn, const float* inten_in, int nb, double* quat, double* fit,
                      float* cm_out, int64_t* pm_out, int64_t* nmatch_out, int64_t* ij_out, int32_t* acc_out,
                      double* bandfit) {
    const int nfam = L->nfam;
    const double tol = L->tol;
    const float tolf = (float)tol;
    float inten[MAXB];
    for (int b = 0; b < nb; ++b) inten[b] = inten_in ? inten_in[b] : 1.0f;
    float ang[MAXB][MAXB];
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
            float d = fabsf(dot3f(bn + 3 * i, bn + 3 * j));
            d = d < -1.0f ? -1.0f : (d > 1.0f ? 1.0f : d);
            ang[i][j] = acos_deg(d);
        }
    for (int q = 0; q < nb; ++q)
        if (inten[q] < 1e-6f)
            for (int t = 0; t < nb; ++t) ang[q][t] = ang[t][q] = 10000.0f;

    /* ---- vote ---- */
    float accw[MAXF][MAXB], accn[MAXF][MAXB];
    memset(accw, 0, sizeof(accw));
    memset(accn, 0, sizeof(accn));
    for (int i = 0; i < nb; ++i)
        for (int j = i + 1; j < nb; ++j)
            for (int k = j + 1; k < nb; ++k) {
                const float x[3] = {ang[i][j], ang[i][k], ang[j][k]};
                int s[3], u[3];
                argsort3f(x, s);
                int r[3];
                for (int m = 0; m < 3; ++m) r[m] = (int)L->lut[((m * 3 + s[0]) * 3 + s[1]) * 3 + s[2]];
                argsort3i(r, u);
                const float a0 = x[s[0]], a1 = x[s[1]], a2 = x[s[2]];
                const int e1 = fabsf(a0 - a1) < tolf, e2 = fabsf(a1 - a2) < tolf, e3 = fabsf(a2 - a0) < tolf;
                for (int q = 0; q < L->ntrip; ++q) {
                    const double* T = L->trip_angles + 3 * (size_t)q;
                    const double d0 = fabs(T[0] - (double)a0);
                    if (d0 > tol) continue;
                    const double d1 = fabs(T[1] - (double)a1);
                    if (d1 > tol) continue;
                    const double d2 = fabs(T[2] - (double)a2);
                    if (d2 > tol) continue;
                    const float t0 = (float)d0, t1 = (float)d1, t2 = (float)d2;
                    const int64_t* F = L->trip_family + 3 * (size_t)q;
                    const int f0 = (int)F[u[0]], f1 = (int)F[u[1]], f2 = (int)F[u[2]];
                    const float w1 = tolf - 0.5f * (t0 + t1), w2 = tolf - 0.5f * (t0 + t2), w3 = tolf - 0.5f * (t1 + t2);
#define VOTE(f, b, w) do { accw[f][b] += (w); accn[f][b] += 1.0f; } while (0)
                    VOTE(f0, i, w1); VOTE(f1, j, w2); VOTE(f2, k, w3);
                    if (e1) { VOTE(f0, j, w1); VOTE(f1, i, w2); VOTE(f2, k, w3); }
                    if (e2) { VOTE(f0, i, w1); VOTE(f1, k, w2); VOTE(f2, j, w3); }
                    if (e3) { VOTE(f0, k, w1); VOTE(f1, j, w2); VOTE(f2, i, w3); }
                    if (e1 && e2 && e3) {
                        VOTE(f0, k, w1); VOTE(f1, i, w2); VOTE(f2, j, w3);
                        VOTE(f0, j, w1); VOTE(f1, k, w2); VOTE(f2, i, w3);
                    }
#undef VOTE
                }
            }
    /* vote metrics and rank */
    float rank[MAXB];
    int bfam[MAXB];
    for (int b = 0; b < nb; ++b) {
        float sum = 0.0f, mx = -1.0e12f, m1 = -INFINITY, m2 = -INFINITY;
        int fam = 0;
        for (int f = 0; f < nfam; ++f) {
            const float v = accw[f][b];
            sum += v;
            if (v > mx) { mx = v; fam = f; }
            if (v > m1) { m2 = m1; m1 = v; } else if (v > m2) { m2 = v; }
        }
        const int mxvote = (int)mx, tvotes = (int)sum;
        const float cmb = tvotes < 1 ? 0.0f : (float)((double)(m1 - m2) / (double)tvotes);
        rank[b] = (float)((double)(nb - b) / (double)nb * (double)cmb * (double)mxvote);
        bfam[b] = fam;
    }
    int rarg[MAXB];
    stable_rank(rank, nb, rarg);

    /* ---- TRIAD assignment ---- */
    int best_n = 0;
    float best_fit = 360.0f;
    int64_t bij[4] = {-1, -1, -1, -1};
    int64_t bpm[MAXB];
    int bpv[MAXB];
    for (int j = 0; j < nb; ++j) { bpm[j] = -1000; bpv[j] = 0; }
    int stop = 0;
    for (int ii = 0; ii < nb - 1 && !stop; ++ii)
        for (int jj = ii + 1; jj < nb; ++jj) {
            const int b1 = rarg[nb - 1 - ii], b2 = rarg[nb - 1 - jj];
            const float* v1 = bn + 3 * b1;
            const float* v2 = bn + 3 * b2;
            const int f1 = bfam[b1], f2 = bfam[b2];
            float c12 = dot3f(v1, v2);
            if (c12 > 1.0f) c12 = 1.0f;
            if (c12 < -1.0f) c12 = -1.0f;
            float afit[MAXB];
            int64_t pm[MAXB];
            int pv[MAXB];
            for (int j = 0; j < nb; ++j) { afit[j] = 0.0f; pm[j] = -1; pv[j] = 0; }
            int ngood = 0;
            if (acos_deg(fabsf(c12)) > tolf) {
                const float a01 = acos_deg(c12);
                const int row = (int)L->famidx[f1], lo = (int)L->famidx[f2], cnt = L->famcnt[f2];
                int any = 0;
                float x[3], y[3];
                cross3f(v1, v2, x);
                const float nx = sqrtf(dot3f(x, x));
                x[0] /= nx; x[1] /= nx; x[2] /= nx;
                cross3f(v1, x, y);
                const float B[3][3] = {{v1[0], v1[1], v1[2]}, {x[0], x[1], x[2]}, {y[0], y[1], y[2]}};
                const float p1[3] = {(float)L->poles[3 * row], (float)L->poles[3 * row + 1], (float)L->poles[3 * row + 2]};
                float score = -1.0f;
                for (int c = lo; c < lo + cnt; ++c) {
                    if (!(fabs(L->angtab[(size_t)row * L->npoles + c] - (double)a01) < tol)) continue;
                    any = 1;
                    float p2[3] = {(float)L->poles[3 * c], (float)L->poles[3 * c + 1], (float)L->poles[3 * c + 2]};
                    const float n2 = sqrtf(dot3f(p2, p2)) + 1.0e-35f;
                    p2[0] /= n2; p2[1] /= n2; p2[2] /= n2;
                    float pc[3], a2[3];
                    cross3f(p1, p2, pc);
                    const float npc = sqrtf(dot3f(pc, pc)) + 1.0e-35f;
                    pc[0] /= npc; pc[1] /= npc; pc[2] /= npc;
                    cross3f(p1, pc, a2);
                    const float A[3][3] = {{p1[0], pc[0], a2[0]}, {p1[1], pc[1], a2[1]}, {p1[2], pc[2], a2[2]}};
                    float AB[3][3];
                    for (int r = 0; r < 3; ++r)
                        for (int cc = 0; cc < 3; ++cc)
                            AB[r][cc] = fmaf(A[r][2], B[2][cc], fmaf(A[r][1], B[1][cc], A[r][0] * B[0][cc]));
                    float ftry[MAXB];
                    int64_t arg[MAXB];
                    int nm = 0;
                    float matched[MAXB];
                    for (int j = 0; j < nb; ++j) {
                        const float* bj = bn + 3 * j;
                        const float t[3] = {dot3f(AB[0], bj), dot3f(AB[1], bj), dot3f(AB[2], bj)};
                        float best = -INFINITY;
                        int a = 0;
                        for (int P = 0; P < L->npoles; ++P) {
                            const float pp[3] = {(float)L->poles[3 * P], (float)L->poles[3 * P + 1], (float)L->poles[3 * P + 2]};
                            const float v = dot3f(pp, t);
                            if (v > best) { best = v; a = P; }
                        }
                        best = best < -1.0f ? -1.0f : best;
                        best = best > 1.0f ? 1.0f : best;
                        ftry[j] = acos_deg(best);
                        arg[j] = a;
                        if (ftry[j] < tolf) matched[nm++] = ftry[j];
                    }
                    const float mean = pw_f(matched, nm) / (float)nm;
                    const float stry = (float)nm / (mean + 1e-6f);
                    if (stry > score) {
                        score = stry;
                        for (int j = 0; j < nb; ++j) { afit[j] = ftry[j]; pm[j] = arg[j]; pv[j] = ftry[j] < tolf; }
                    }
                }
                if (any)
                    for (int j = 0; j < nb; ++j) ngood += afit[j] < tolf;
            }
            if (ngood >= 3) {
                float f = 0.0f;
                for (int j = 0; j < nb; ++j)
                    if (afit[j] < tolf) f += afit[j];
                f /= (float)ngood;
                if (best_n < ngood || (best_n == ngood && best_fit > f)) {
                    best_fit = f;
                    best_n = ngood;
                    for (int j = 0; j < nb; ++j) { bpm[j] = pm[j]; bpv[j] = pv[j]; }
                    bij[0] = ii; bij[1] = jj; bij[2] = b1; bij[3] = b2;
                }
            }
            if (best_n >= L->early) { stop = 1; break; }
        }

    /* ---- outputs of the assignment ---- */
    int ngood = 0, acc = 0;
    for (int j = 0; j < nb; ++j) {
        ngood += bpv[j] != 0;
        const int64_t pmc = bpm[j] > 0 ? bpm[j] : 0;
        acc += bpv[j] != 0 && L->pfam[pmc] == bfam[j];
        pm_out[j] = bpm[j];
    }
    *nmatch_out = best_n;
    for (int t = 0; t < 4; ++t) ij_out[t] = bij[t];
    *acc_out = acc;

    /* ---- QUEST weights ---- */
    float wsel[MAXB];
    for (int j = 0; j < nb; ++j) wsel[j] = 0.0f;
    if (ngood >= 3) {
        float sc[MAXB];
        int q = 0;
        for (int j = 0; j < nb; ++j) {
            sc[j] = -1.0f;
            if (bpv[j]) {
                if (!L->simpleq) {
                    const int a = L->pfam[bpm[j]];
                    sc[j] = accw[a][j] / (accn[a][j] > 0.0f ? accn[a][j] : 1.0e-12f);
                } else {
                    sc[j] = inten[q];
                }
                ++q;
            }
        }
        int ord[MAXB];
        stable_rank(sc, nb, ord);
        const int nfit = ngood < 6 ? ngood : 6;
        double wd[MAXB];
        for (int j = 0; j < nb; ++j) wd[j] = 0.0;
        for (int t = 0; t < nfit; ++t) wd[ord[nb - 1 - t]] = (double)inten[ord[nb - 1 - t]];
        const double tot = pw_d(wd, nb);
        for (int j = 0; j < nb; ++j) wsel[j] = (float)(wd[j] / tot);
    }

    /* ---- QUEST fit ---- */
    double wq[MAXB];
    for (int j = 0; j < nb; ++j) wq[j] = (double)wsel[j];
    double tot = pw_d(wq, nb);
    tot = (tot != tot) ? tot : (tot > 1e-12 ? tot : 1e-12);
    int idx[MAXB], m = 0;
    double wn[MAXB];
    for (int j = 0; j < nb; ++j) {
        const double w = (double)wsel[j] / tot;
        if (w > 1.0e-7) { idx[m] = j; wn[m] = w; ++m; }
    }
    double q4[4] = {1.0, 0.0, 0.0, 0.0};
    double mad = -1.0;
    double bdot[MAXB];
    for (int j = 0; j < nb; ++j) bdot[j] = -1.0;
    if (m >= 3) {
        const double ws = pw_d(wn, m);
        double bq[MAXB][3], pq[MAXB][3];
        for (int k = 0; k < m; ++k) {
            wn[k] /= ws;
            const int64_t pmk = bpm[idx[k]] > 0 ? bpm[idx[k]] : 0;
            for (int c = 0; c < 3; ++c) {
                bq[k][c] = (double)bn[3 * idx[k] + c];
                pq[k][c] = L->poles[3 * pmk + c];
            }
        }
        double S[3][3], Bm[3][3], z[3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double a = (wn[0] * bq[0][r]) * pq[0][c];
                for (int k = 1; k < m; ++k) a = fma(wn[k] * bq[k][r], pq[k][c], a);
                Bm[r][c] = a;
            }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S[r][c] = Bm[r][c] + Bm[c][r];
        for (int c = 0; c < 3; ++c) {
            const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            double zc = 0.0;
            for (int k = 0; k < m; ++k) {
                const double v = wn[k] * (bq[k][c1] * pq[k][c2] - bq[k][c2] * pq[k][c1]);
                zc = k == 0 ? v : zc + v;
            }
            z[c] = zc;
        }
        double S2[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S2[r][c] = fma(S[r][2], S[2][c], fma(S[r][1], S[1][c], S[r][0] * S[0][c]));
        const double det = S[0][0] * (S[1][1] * S[2][2] - S[1][2] * S[2][1]) -
                           S[0][1] * (S[1][0] * S[2][2] - S[1][2] * S[2][0]) +
                           S[0][2] * (S[1][0] * S[2][1] - S[1][1] * S[2][0]);
        const double kk = (S[1][1] * S[2][2] - S[1][2] * S[2][1]) + (S[0][0] * S[2][2] - S[0][2] * S[2][0]) +
                          (S[0][0] * S[1][1] - S[1][0] * S[0][1]);
        const double sig = 0.5 * ((S[0][0] + S[1][1]) + S[2][2]);
        const double sig2 = sig * sig;
        double u[3], v[3];
        for (int c = 0; c < 3; ++c) {
            u[c] = fma(z[2], S2[2][c], fma(z[1], S2[1][c], z[0] * S2[0][c]));
            v[c] = fma(z[2], S[2][c], fma(z[1], S[1][c], z[0] * S[0][c]));
        }
        const double d = fma(u[2], z[2], fma(u[1], z[1], u[0] * z[0]));
        const double cc = det + fma(v[2], z[2], fma(v[1], z[1], v[0] * z[0]));
        const double b = sig2 + fma(z[2], z[2], fma(z[1], z[1], z[0] * z[0]));
        const double a = sig2 - kk;
        double lam = 1.0, dlam = 1e6;
        for (int it = 0; dlam > 1.0e-12 && it < 10; ++it) {
            const double lam0 = lam, l2 = lam * lam;
            lam = lam - (l2 * l2 - (a + b) * l2 - cc * lam + (a * b + cc * sig - d)) /
                            (4.0 * (l2 * lam) - 2.0 * (a + b) * lam - cc);
            dlam = fabs(lam0 - lam);
        }
        const double beta = lam - sig, alpha = lam * lam - sig2 + kk, gamma = (lam + sig) * alpha - det;
        double X[3];
        for (int r = 0; r < 3; ++r) {
            double M[3];
            for (int c = 0; c < 3; ++c) M[c] = ((r == c ? alpha : 0.0) + beta * S[r][c]) + S2[r][c];
            X[r] = fma(M[2], z[2], fma(M[1], z[1], M[0] * z[0]));
        }
        const double qn = sqrt(((gamma * gamma + X[0] * X[0]) + X[1] * X[1]) + X[2] * X[2]);
        q4[0] = gamma / qn; q4[1] = X[0] / qn; q4[2] = X[1] / qn; q4[3] = X[2] / qn;
        if (gamma < 0.0)
            for (int t = 0; t < 4; ++t) q4[t] = -q4[t];
        double dots[MAXB];
        for (int k = 0; k < m; ++k) {
            const double* vv = bq[k];
            const double w0 = q4[0], r0 = q4[1], r1 = q4[2], r2 = q4[3];
            double t[3] = {r1 * vv[2] - r2 * vv[1], r2 * vv[0] - r0 * vv[2], r0 * vv[1] - r1 * vv[0]};
            for (int c = 0; c < 3; ++c) t[c] = t[c] + w0 * vv[c];
            const double t2[3] = {r1 * t[2] - r2 * t[1], r2 * t[0] - r0 * t[2], r0 * t[1] - r1 * t[0]};
            double sd = 0.0;
            for (int c = 0; c < 3; ++c) sd = sd + (2.0 * t2[c] + vv[c]) * pq[k][c];
            dots[k] = sd;
            bdot[idx[k]] = sd;
        }
        mad = pw_d(dots, m) / (double)m;
    }
    for (int t = 0; t < 4; ++t) quat[t] = q4[t];
    const double mc = mad < -1.0 ? -1.0 : (mad > 1.0 ? 1.0 : mad);
    *fit = acos(mc) * RADEG;
    for (int j = 0; j < nb; ++j) {
        const double bc = bdot[j] < -1.0 ? -1.0 : (bdot[j] > 1.0 ? 1.0 : bdot[j]);
        bandfit[j] = acos(bc) * RADEG;
    }

    /* ---- vote confidence ---- */
    float cm2 = -1.0f;
    if (ngood >= 3) {
        float num = 0.0f;
        for (int j = 0; j < nb; ++j)
            if (bpv[j]) num += accw[L->pfam[bpm[j]]][j];
        float clip[MAXF * MAXB];
        for (int f = 0; f < nfam; ++f)
            for (int b = 0; b < nb; ++b) {
                const float v = accw[f][b];
                clip[f * nb + b] = (v != v || v >= 1.0f) ? v : 1.0f;
            }
        cm2 = num / pw_f(clip, nfam * nb);
    }
    *cm_out = cm2;
}

int votecpu_bandindex(const VoteLib* L, const float* norms, const float* inten, int64_t n, int nb, double* quat,
                      double* fit, float* cm, int64_t* polematch, int64_t* nmatch, int64_t* ij, int32_t* acc_correct,
                      double* bandfit, int threads) {
    if (!L || nb < 1 || nb > MAXB || L->nfam < 2 || L->nfam > MAXF) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t p = 0; p < n; ++p)
        index_one(L, norms + p * nb * 3, inten ? inten + p * nb : NULL, nb, quat + 4 * p, fit + p, cm + p,
                  polematch + p * nb, nmatch + p, ij + 4 * p, acc_correct + p, bandfit + p * nb);
    return 0;
}

int votecpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
