// Band indexing by triplet voting on the device: tripletvote.BandIndexer.bandindex
// (tripletvote.py:492-633) with high_fidelity on -- the triplet vote (:1021-1210), the TRIAD
// band assignment over band pairs (:1483-1690), the QUEST band weights and orientation fit
// (:856-1020, rotlib.py:1641-1674) and the vote confidence (:2057-2075) -- plus the indexer's
// band weights and pattern quality (_ebsd_index_single.py:751-763).
//
// One warp indexes one pattern; a block of kWarps warps shares the phase library in shared
// memory.  Arithmetic follows the reference as numpy evaluates it: float32 where the reference
// works on float32 arrays (band angles, votes, the TRIAD fit), float64 for the QUEST fit, every
// add/multiply rounded on its own (no contraction), 3-term dot products as the fused
// multiply-add chain BLAS uses for these shapes, sums in numpy's pairwise order.  arccos is
// CUDA's float32 acosf (within two ulp, as numpy's own float32 arccos is).
//
// Two steps are reorganised for the GPU without changing their result:
//   * the vote's library test |T - a| <= angTol (float64, T a library angle, a a float32 band
//     angle) becomes a <= / >= test against the float32 interval of a that passes it, computed
//     once per library on the host;
//   * the warp tests 32 library triplets at once and applies the matches one by one in library
//     order, so that every float32 vote sum adds in the reference's order.
#include "ebsd_internal.cuh"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>

struct ebsd_vote_plan_s {
    int device = 0;
    int nfam = 0, ntrip = 0, npoles = 0;
    double tol = 0.0;
    int early = 0, simpleq = 0;
    uint8_t lut[27] = {};         // lut[:, s0, s1, s2] as 3 x 2 bits, index s0 * 9 + s1 * 3 + s2
    float* d_iv = nullptr;        // [6][ntrip] acceptance intervals lo0, hi0, lo1, hi1, lo2, hi2, rows sorted by lo0
    uint32_t* d_tfam = nullptr;   // [ntrip] f0 | f1 << 8 | f2 << 16
    double* d_tang = nullptr;     // [ntrip][3]
    float* d_pole = nullptr;      // [3][npoles] float32 poles, component-major
    double* d_pole64 = nullptr;   // [npoles][3]
    int32_t* d_pfam = nullptr;    // [npoles]
    double* d_angtab = nullptr;   // [npoles][npoles]
    int32_t* d_famcnt = nullptr;  // [nfam]
    int32_t* d_famidx = nullptr;  // [nfam]
    float* d_cand = nullptr;      // [nfam][npoles][2] band-pair cosine interval per library column
    float* d_par = nullptr;       // [1] largest |cosine| of a band pair that is not parallel
    float par = -1.0f;            // host copy of *d_par
    int32_t* d_orig = nullptr;    // [ntrip] library index of each interval row (rows sorted by lo0)
    void* d_quest = nullptr;      // QUEST hand-over scratch, quest_cap patterns
    int64_t quest_cap = 0;
    float win = 0.0f;             // widest first-angle interval (hi0 - lo0), plus a margin
};

namespace ebsd {
namespace {

constexpr int kWarps = 8;
constexpr int kList = 96;  // matches of one band triplet held for sorting into library order
constexpr unsigned kFull = 0xffffffffu;
constexpr double kRadeg = 57.29577951308232;  // 180 / pi
constexpr float kRadegF = 57.29577951308232f;

// What the warp hands to the QUEST solve for one pattern: the bands chosen for the weights
// (bit j: band j) and the number of matched bands; k_quest adds the bands in the fit (mask, m;
// m < 3: no fit) for k_quest_fit.
struct QuestInput {
    uint32_t sel;
    int32_t ngood;
    uint32_t mask;
    int32_t m;
};

struct VoteArgs {
    const float* iv;
    const uint32_t* tfam;
    const double* tang;
    const float* pole;
    const double* pole64;
    const int32_t* pfam;
    const double* angtab;
    const int32_t* famcnt;
    const int32_t* famidx;
    const float* cand;
    const int32_t* orig;
    float par, win;
    int nfam, ntrip, npoles, nb;
    float tol_f;
    double tol;
    int early, simpleq;
    uint8_t lut[28];
    const float* norms;
    const float* inten;
    int64_t n;
    ebsd_index_out out;
    QuestInput* quest;  // [n] scratch, device
};

__device__ __forceinline__ float addf(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double addf(double a, double b) { return __dadd_rn(a, b); }

// numpy's pairwise summation (the add reduction of a contiguous float32 / float64 run), over
// get(0 .. n-1): below 8 elements a running sum from 0; up to 128 eight interleaved partial
// sums combined as ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)), then the tail; above
// 128 the two halves (split at a multiple of 8) summed the same way.
template <class T, class G>
__device__ T np_sum_block(G get, int lo, int n) {
    if (n < 8) {
        T r = T(0);
        for (int i = 0; i < n; ++i) r = addf(r, get(lo + i));
        return r;
    }
    T r[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = get(lo + j);
    int i = 8;
    for (; i < n - (n % 8); i += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = addf(r[j], get(lo + i + j));
    }
    T res = addf(addf(addf(r[0], r[1]), addf(r[2], r[3])), addf(addf(r[4], r[5]), addf(r[6], r[7])));
    for (; i < n; ++i) res = addf(res, get(lo + i));
    return res;
}

template <class T, class G>
__device__ T np_sum_half(G get, int lo, int n) {  // n <= 256
    if (n <= 128) return np_sum_block<T>(get, lo, n);
    int h = n / 2;
    h -= h % 8;
    return addf(np_sum_block<T>(get, lo, h), np_sum_block<T>(get, lo + h, n - h));
}

template <class T, class G>
__device__ T np_sum_get(G get, int n) {  // n <= 512
    if (n <= 256) return np_sum_half<T>(get, 0, n);
    int h = n / 2;
    h -= h % 8;
    return addf(np_sum_half<T>(get, 0, h), np_sum_half<T>(get, h, n - h));
}

template <class T>
__device__ T np_sum(const T* a, int n) {
    return np_sum_get<T>([a](int i) { return a[i]; }, n);
}

// float32 3-term dot product as BLAS sgemm forms it: fma(a2, b2, fma(a1, b1, a0 * b0))
__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
    return __fmaf_rn(a2, b2, __fmaf_rn(a1, b1, __fmul_rn(a0, b0)));
}

// numpy.cross of float32 3-vectors: each component a product difference, each op rounded
__device__ __forceinline__ void cross3(const float* a, const float* b, float* c) {
    c[0] = __fsub_rn(__fmul_rn(a[1], b[2]), __fmul_rn(a[2], b[1]));
    c[1] = __fsub_rn(__fmul_rn(a[2], b[0]), __fmul_rn(a[0], b[2]));
    c[2] = __fsub_rn(__fmul_rn(a[0], b[1]), __fmul_rn(a[1], b[0]));
}

__device__ __forceinline__ float norm3(const float* a) {
    return __fsqrt_rn(dot3(a[0], a[1], a[2], a[0], a[1], a[2]));
}

// float32 arccos(x) * RADEG.  The reference's float32 arccos is numpy's (SIMD, not correctly
// rounded: one or two ulp off for about a third of the inputs on x86); CUDA's acosf is within
// two ulp as well, so either may sit an ulp or two from the reference's value.
__device__ __forceinline__ float acos_deg(float x) {
    return __fmul_rn(acosf(x), kRadegF);
}

__device__ __forceinline__ void sort3(const float* v, int& s0, int& s1, int& s2) {
    int s[3] = {0, 1, 2};
    int t;
    if (v[s[0]] > v[s[2]]) { t = s[2]; s[2] = s[0]; s[0] = t; }
    if (v[s[0]] > v[s[1]]) { t = s[1]; s[1] = s[0]; s[0] = t; }
    if (v[s[1]] > v[s[2]]) { t = s[2]; s[2] = s[1]; s[1] = t; }
    s0 = s[0]; s1 = s[1]; s2 = s[2];
}

__device__ __forceinline__ void sort3i(const int* v, int& s0, int& s1, int& s2) {
    int s[3] = {0, 1, 2};
    int t;
    if (v[s[0]] > v[s[2]]) { t = s[2]; s[2] = s[0]; s[0] = t; }
    if (v[s[0]] > v[s[1]]) { t = s[1]; s[1] = s[0]; s[0] = t; }
    if (v[s[1]] > v[s[2]]) { t = s[2]; s[2] = s[1]; s[1] = t; }
    s0 = s[0]; s1 = s[1]; s2 = s[2];
}

__device__ __forceinline__ double np_maximum(double a, double b) {  // NaN-propagating
    if (a != a) return a;
    if (b != b) return b;
    return a > b ? a : b;
}

__host__ __device__ inline size_t align8(size_t words) { return (words + 1) & ~size_t(1); }

// 4-byte words of one warp's region
__host__ __device__ inline size_t warp_words(int nb, int nfam) {
    return align8(3 * size_t(nb) + nb + nb * nb + 2 * size_t(nfam) * nb + nb + nb + 64 + kList);
}

__host__ __device__ inline size_t block_words(int ntrip, int npoles) {
    return align8(6 * size_t(ntrip) + ntrip + 3 * size_t(npoles) + npoles);
}

// Warp-cooperative search on a monotone predicate (true for a leading run of [0, n), then
// false): the length of the run.  32-way: each round samples 32 evenly spaced indices.
template <class P>
__device__ __forceinline__ int warp_count_leading(int n, int lane, P pred) {
    int lo = 0, hi = n;  // the answer lies in [lo, hi]
    while (hi - lo > 32) {
        const int step = (hi - lo + 31) / 32;
        const int idx = lo + lane * step;
        const int c = __popc(__ballot_sync(kFull, idx < hi && pred(idx)));
        if (c == 0) return lo;
        const int nlo = lo + (c - 1) * step + 1;
        hi = min(hi, lo + c * step);
        lo = nlo;
    }
    const int idx = lo + lane;
    return lo + __popc(__ballot_sync(kFull, idx < hi && pred(idx)));
}

// ---------------------------------------------------------------------------------------
__device__ void index_pattern(const VoteArgs& A, int64_t p, int lane, const float* s_iv,
                              const int* s_orig, const float* s_pole, const int* s_pfam,
                              float* w) {
    const int nb = A.nb, nfam = A.nfam, ntrip = A.ntrip, npoles = A.npoles;
    const float tolf = A.tol_f;
    float* bn = w;                       // [nb][3]
    float* inten = bn + 3 * nb;          // [nb]
    float* ang = inten + nb;             // [nb][nb]
    float* accw = ang + nb * nb;          // [nfam][nb]
    float* accn = accw + nfam * nb;      // [nfam][nb]
    int* rarg = (int*)(accn + nfam * nb);  // [nb] band order, ascending rank
    int* bfam = rarg + nb;               // [nb]
    float* fscr = (float*)(bfam + nb);   // [64]
    int* mlist = (int*)(fscr + 64);      // [kList]
    const unsigned lt_mask = (1u << lane) - 1u;

    for (int t = lane; t < 3 * nb; t += 32) bn[t] = A.norms[p * 3 * nb + t];
    for (int t = lane; t < nb; t += 32) inten[t] = A.inten ? A.inten[p * nb + t] : 1.0f;
    for (int t = lane; t < 2 * nfam * nb; t += 32) accw[t] = 0.0f;
    __syncwarp();

    // band-band angles, tripletvote.py:1181-1188 (the vote reads the upper triangle only)
    for (int t = lane; t < nb * (nb - 1) / 2; t += 32) {
        int i = 0, r = t;
        while (r >= nb - 1 - i) {
            r -= nb - 1 - i;
            ++i;
        }
        const int j = i + 1 + r;
        const float* a = bn + 3 * i;
        const float* b = bn + 3 * j;
        float d = fabsf(dot3(a[0], a[1], a[2], b[0], b[1], b[2]));
        d = fminf(fmaxf(d, -1.0f), 1.0f);
        float v = acos_deg(d);
        if (inten[i] < 1e-6f || inten[j] < 1e-6f) v = 10000.0f;
        ang[i * nb + j] = v;
    }
    __syncwarp();

    // ---- triplet vote, tripletvote.py:1023-1135 ----
    for (int i = 0; i < nb; ++i) {
        if (inten[i] < 1e-6f) continue;  // all its angles are 10000: no library triplet matches
        for (int j = i + 1; j < nb; ++j) {
            if (inten[j] < 1e-6f) continue;
            for (int k = j + 1; k < nb; ++k) {
                if (inten[k] < 1e-6f) continue;
                float x[3] = {ang[i * nb + j], ang[i * nb + k], ang[j * nb + k]};
                int s0, s1, s2;
                sort3(x, s0, s1, s2);
                const int code = A.lut[s0 * 9 + s1 * 3 + s2];
                const int r[3] = {code & 3, (code >> 2) & 3, (code >> 4) & 3};
                int u0, u1, u2;
                sort3i(r, u0, u1, u2);
                const float a0 = x[s0], a1 = x[s1], a2 = x[s2];
                const bool e1 = fabsf(__fsub_rn(a0, a1)) < tolf;
                const bool e2 = fabsf(__fsub_rn(a1, a2)) < tolf;
                const bool e3 = fabsf(__fsub_rn(a2, a0)) < tolf;
                // library entries whose first-angle interval can hold a0: sorted by its lower
                // end, so [s, e) with lo0 in [a0 - win, a0]
                const float tgt = a0 - A.win;
                const int e = warp_count_leading(ntrip, lane, [&](int q) { return s_iv[q] <= a0; });
                const int s = warp_count_leading(e, lane, [&](int q) { return s_iv[q] < tgt; });
                auto test = [&](int q) {
                    return a0 >= s_iv[q] && a0 <= s_iv[ntrip + q] && a1 >= s_iv[2 * ntrip + q] &&
                           a1 <= s_iv[3 * ntrip + q] && a2 >= s_iv[4 * ntrip + q] && a2 <= s_iv[5 * ntrip + q];
                };
                // one match, in the reference's library order (lane 0 applies them all)
                auto apply = [&](int q) {
                    const double* T = A.tang + 3 * (size_t)q;
                    const float t0 = __double2float_rn(fabs(__dsub_rn(T[0], (double)a0)));
                    const float t1 = __double2float_rn(fabs(__dsub_rn(T[1], (double)a1)));
                    const float t2 = __double2float_rn(fabs(__dsub_rn(T[2], (double)a2)));
                    const uint32_t fw = A.tfam[q];
                    const int fq[3] = {int(fw & 255u), int((fw >> 8) & 255u), int((fw >> 16) & 255u)};
                    const int f0 = fq[u0], f1 = fq[u1], f2 = fq[u2];
                    const float w1 = __fsub_rn(tolf, __fmul_rn(0.5f, __fadd_rn(t0, t1)));
                    const float w2 = __fsub_rn(tolf, __fmul_rn(0.5f, __fadd_rn(t0, t2)));
                    const float w3 = __fsub_rn(tolf, __fmul_rn(0.5f, __fadd_rn(t1, t2)));
                    auto vote = [&](int f, int b, float wt) {
                        accw[f * nb + b] = __fadd_rn(accw[f * nb + b], wt);
                        accn[f * nb + b] = __fadd_rn(accn[f * nb + b], 1.0f);
                    };
                    vote(f0, i, w1); vote(f1, j, w2); vote(f2, k, w3);
                    if (e1) { vote(f0, j, w1); vote(f1, i, w2); vote(f2, k, w3); }
                    if (e2) { vote(f0, i, w1); vote(f1, k, w2); vote(f2, j, w3); }
                    if (e3) { vote(f0, k, w1); vote(f1, j, w2); vote(f2, i, w3); }
                    if (e1 && e2 && e3) {
                        vote(f0, k, w1); vote(f1, i, w2); vote(f2, j, w3);
                        vote(f0, j, w1); vote(f1, k, w2); vote(f2, i, w3);
                    }
                };
                int cnt = 0;
                for (int base = s; base < e; base += 32) {
                    const int q = base + lane;
                    const bool hit = q < e && test(q);
                    const unsigned m = __ballot_sync(kFull, hit);
                    if (hit && cnt + __popc(m & lt_mask) < kList) mlist[cnt + __popc(m & lt_mask)] = s_orig[q];
                    cnt += __popc(m);
                }
                __syncwarp();
                if (cnt <= kList) {
                    if (lane == 0) {
                        for (int a = 1; a < cnt; ++a) {  // insertion sort into library order
                            const int v = mlist[a];
                            int b = a - 1;
                            while (b >= 0 && mlist[b] > v) {
                                mlist[b + 1] = mlist[b];
                                --b;
                            }
                            mlist[b + 1] = v;
                        }
                        for (int a = 0; a < cnt; ++a) apply(mlist[a]);
                    }
                } else {
                    // more matches than the list holds: take them one at a time, smallest
                    // library index above the last one applied
                    int last = -1;
                    while (true) {
                        int mine = INT_MAX;
                        for (int q = s + lane; q < e; q += 32)
                            if (test(q) && s_orig[q] > last && s_orig[q] < mine) mine = s_orig[q];
                        const int next = __reduce_min_sync(kFull, mine);
                        if (next == INT_MAX) break;
                        if (lane == 0) apply(next);
                        last = next;
                        __syncwarp();
                    }
                }
                __syncwarp();
            }
        }
    }
    __syncwarp();

    // ---- vote metrics per band, tripletvote.py:1137-1171, and rank, :1189-1191 ----
    float rank = 0.0f;
    int fam = 0;
    if (lane < nb) {
        float sum = 0.0f, mx = -1.0e12f, m1 = -INFINITY, m2 = -INFINITY;
        for (int f = 0; f < nfam; ++f) {
            const float v = accw[f * nb + lane];
            sum = __fadd_rn(sum, v);
            if (v > mx) { mx = v; fam = f; }
            if (v > m1) { m2 = m1; m1 = v; } else if (v > m2) { m2 = v; }
        }
        const int mxvote = (int)mx, tvotes = (int)sum;
        const float cm = tvotes < 1 ? 0.0f
                                    : __double2float_rn(__ddiv_rn((double)__fsub_rn(m1, m2), (double)tvotes));
        const double lead = __ddiv_rn((double)(nb - lane), (double)nb);
        rank = __double2float_rn(__dmul_rn(__dmul_rn(lead, (double)cm), (double)mxvote));
        bfam[lane] = fam;
    }
    {
        int pos = 0;
        for (int c = 0; c < nb; ++c) {
            const float rc = __shfl_sync(kFull, rank, c);
            pos += (rc < rank) || (rc == rank && c < lane);
        }
        if (lane < nb) rarg[pos] = lane;
    }
    __syncwarp();

    // ---- TRIAD assignment over band pairs in rank order, tripletvote.py:1600-1690 ----
    int best_n = 0;
    float best_fit = 360.0f;
    int bij[4] = {-1, -1, -1, -1};
    int best_pm = -1000, best_pv = 0;
    bool stop = false;
    for (int ii = 0; ii < nb - 1 && !stop; ++ii) {
        for (int jj = ii + 1; jj < nb; ++jj) {
            const int b1 = rarg[nb - 1 - ii], b2 = rarg[nb - 1 - jj];
            const float* v1 = bn + 3 * b1;
            const float* v2 = bn + 3 * b2;
            const int f1 = bfam[b1], f2 = bfam[b2];
            float c12 = dot3(v1[0], v1[1], v1[2], v2[0], v2[1], v2[2]);
            if (c12 > 1.0f) c12 = 1.0f;
            if (c12 < -1.0f) c12 = -1.0f;
            int ngood = 0;
            float afit = 0.0f;
            int pm = -1, pv = 0;
            // arccos(|c12|) > angTol and |angTable - arccos(c12)| < angTol (tripletvote.py:1517-1524) as
            // cosine intervals precomputed with the same arccos (k_vote_thresholds)
            if (fabsf(c12) <= A.par) {
                const float* cint = A.cand + (size_t)f1 * npoles * 2;
                const int row = A.famidx[f1], lo = A.famidx[f2], cnt = A.famcnt[f2];
                float x[3];
                cross3(v1, v2, x);
                const float nx = norm3(x);
                x[0] = __fdiv_rn(x[0], nx); x[1] = __fdiv_rn(x[1], nx); x[2] = __fdiv_rn(x[2], nx);
                float y[3];
                cross3(v1, x, y);
                const float B[3][3] = {{v1[0], v1[1], v1[2]}, {x[0], x[1], x[2]}, {y[0], y[1], y[2]}};
                const float p1[3] = {s_pole[row], s_pole[npoles + row], s_pole[2 * npoles + row]};
                const float* bj = bn + 3 * (lane < nb ? lane : 0);
                float score = -1.0f;
                bool any = false;
                for (int cb = 0; cb < cnt; cb += 32) {
                    const int col = lo + cb + lane;
                    const bool hit = cb + lane < cnt && c12 >= cint[2 * col] && c12 <= cint[2 * col + 1];
                    unsigned m = __ballot_sync(kFull, hit);
                    any = any || m != 0;
                    while (m) {
                        const int cand = lo + cb + __ffs(m) - 1;
                        m &= m - 1;
                        float p2[3] = {s_pole[cand], s_pole[npoles + cand], s_pole[2 * npoles + cand]};
                        const float n2 = __fadd_rn(norm3(p2), 1.0e-35f);
                        p2[0] = __fdiv_rn(p2[0], n2); p2[1] = __fdiv_rn(p2[1], n2); p2[2] = __fdiv_rn(p2[2], n2);
                        float pc[3];
                        cross3(p1, p2, pc);
                        const float npc = __fadd_rn(norm3(pc), 1.0e-35f);
                        pc[0] = __fdiv_rn(pc[0], npc); pc[1] = __fdiv_rn(pc[1], npc); pc[2] = __fdiv_rn(pc[2], npc);
                        float a2[3];
                        cross3(p1, pc, a2);
                        const float Am[3][3] = {{p1[0], pc[0], a2[0]}, {p1[1], pc[1], a2[1]}, {p1[2], pc[2], a2[2]}};
                        float AB[3][3];
#pragma unroll
                        for (int r = 0; r < 3; ++r)
#pragma unroll
                            for (int c = 0; c < 3; ++c)
                                AB[r][c] = dot3(Am[r][0], Am[r][1], Am[r][2], B[0][c], B[1][c], B[2][c]);
                        // this lane's band: rotated normal, best library pole
                        const float t0 = dot3(AB[0][0], AB[0][1], AB[0][2], bj[0], bj[1], bj[2]);
                        const float t1 = dot3(AB[1][0], AB[1][1], AB[1][2], bj[0], bj[1], bj[2]);
                        const float t2 = dot3(AB[2][0], AB[2][1], AB[2][2], bj[0], bj[1], bj[2]);
                        float best = -INFINITY;
                        int arg = 0;
                        for (int P = 0; P < npoles; ++P) {
                            const float v = dot3(s_pole[P], s_pole[npoles + P], s_pole[2 * npoles + P], t0, t1, t2);
                            if (v > best) { best = v; arg = P; }
                        }
                        best = best < -1.0f ? -1.0f : best;
                        best = best > 1.0f ? 1.0f : best;
                        const float ftry = acos_deg(best);
                        const bool ok = lane < nb && ftry < tolf;
                        const unsigned okm = __ballot_sync(kFull, ok);
                        const int nmatch = __popc(okm);
                        if (ok) fscr[__popc(okm & lt_mask)] = ftry;
                        __syncwarp();
                        float mean = 0.0f;
                        if (lane == 0) mean = __fdiv_rn(np_sum(fscr, nmatch), (float)nmatch);
                        mean = __shfl_sync(kFull, mean, 0);
                        const float stry = __fdiv_rn((float)nmatch, __fadd_rn(mean, 1e-6f));
                        if (stry > score) {
                            score = stry;
                            afit = ftry;
                            pm = arg;
                            pv = ftry < tolf;
                        }
                        __syncwarp();
                    }
                }
                if (any) ngood = __popc(__ballot_sync(kFull, lane < nb && afit < tolf));
            }
            if (ngood >= 3) {
                float fit = 0.0f;
                for (int j = 0; j < nb; ++j) {
                    const float v = __shfl_sync(kFull, afit, j);
                    if (v < tolf) fit = __fadd_rn(fit, v);
                }
                fit = __fdiv_rn(fit, (float)ngood);
                if (best_n < ngood || (best_n == ngood && best_fit > fit)) {
                    best_fit = fit;
                    best_n = ngood;
                    best_pm = pm;
                    best_pv = pv;
                    bij[0] = ii; bij[1] = jj; bij[2] = b1; bij[3] = b2;
                }
            }
            if (best_n >= A.early) {
                stop = true;
                break;
            }
        }
    }

    // ---- QUEST weights, tripletvote.py:856-901: the band selection here (its scores need the
    // votes); the float64 weights, B and z and the solve in k_quest, one thread per pattern ----
    const bool good = lane < nb && best_pv != 0;
    const unsigned goodm = __ballot_sync(kFull, good);
    const int ngood = __popc(goodm);
    unsigned selm = 0;
    if (ngood >= 3) {
        float sc = -1.0f;
        if (!A.simpleq) {
            if (good) {
                const int a = s_pfam[best_pm];
                const float an = accn[a * nb + lane];
                sc = __fdiv_rn(accw[a * nb + lane], an > 0.0f ? an : 1.0e-12f);
            }
        } else if (good) {
            sc = inten[__popc(goodm & lt_mask)];
        }
        int pos = 0;
        for (int c = 0; c < nb; ++c) {
            const float s = __shfl_sync(kFull, sc, c);
            pos += (s < sc) || (s == sc && c < lane);
        }
        const int nfit = ngood < 6 ? ngood : 6;
        selm = __ballot_sync(kFull, lane < nb && (nb - 1 - pos) < nfit);
    }
    if (lane == 0) {
        QuestInput* qi = A.quest + p;
        qi->sel = selm;
        qi->ngood = ngood;
    }

    // ---- vote confidence of the matched bands, tripletvote.py:2057-2075 ----
    float cm2 = -1.0f;
    if (ngood >= 3) {
        float num = 0.0f;
        for (int j = 0; j < nb; ++j) {
            const int pmj = __shfl_sync(kFull, best_pm, j);
            if ((goodm >> j) & 1u) num = __fadd_rn(num, accw[s_pfam[pmj] * nb + j]);
        }
        float den = 0.0f;
        if (lane == 0)  // accumulator.clip(1) summed over all families and bands
            den = np_sum_get<float>([accw](int t) { const float v = accw[t]; return (v != v || v >= 1.0f) ? v : 1.0f; },
                                    nfam * nb);
        den = __shfl_sync(kFull, den, 0);
        cm2 = __fdiv_rn(num, den);
    }

    // ---- outputs ----
    const ebsd_index_out& o = A.out;
    const int accc = __popc(__ballot_sync(kFull, good && s_pfam[best_pm > 0 ? best_pm : 0] == fam));
    if (lane < nb) {
        const int64_t e = p * nb + lane;
        o.polematch[e] = best_pm;
        if (o.bandfam) o.bandfam[e] = fam;
        if (o.bandrank) o.bandrank[e] = rank;
        if (o.polevalid) o.polevalid[e] = (uint8_t)best_pv;
    }
    if (o.accw)
        for (int t = lane; t < nfam * nb; t += 32) o.accw[p * nfam * nb + t] = accw[t];
    if (o.accn)
        for (int t = lane; t < nfam * nb; t += 32) o.accn[p * nfam * nb + t] = accn[t];
    if (lane == 0) {
        o.cm[p] = cm2;
        o.nmatch[p] = best_n;
        for (int t = 0; t < 4; ++t) o.ij[4 * p + t] = bij[t];
        o.acc_correct[p] = accc;
    }
    __syncwarp();
}

// Plan-time thresholds of the TRIAD step, evaluated with the kernel's own arccos so that the
// float comparisons replace the reference's tests exactly (acos_deg is monotone in x):
//   par: the largest y in [0, 1] with acos_deg(y) > angTol, so that the pair test
//        arccos(|c|) * RADEG > angTol (tripletvote.py:1517) is |c| <= par;
//   cand[f][c] = [lo, hi]: the cosines x in [-1, 1] with |angTable[famIndex[f]][c] - acos_deg(x)|
//        < angTol in float64 (tripletvote.py:1521-1522); empty as [+inf, -inf].
__device__ __forceinline__ int64_t okey(float f) {
    const uint32_t u = __float_as_uint(f);
    return (int64_t)((u & 0x80000000u) ? ~u : (u | 0x80000000u));
}
__device__ __forceinline__ float okey_float(int64_t k) {
    const uint32_t v = (uint32_t)k;
    return __uint_as_float((v & 0x80000000u) ? (v & 0x7fffffffu) : ~v);
}

__global__ void k_vote_thresholds(const double* __restrict__ angtab, const int32_t* __restrict__ famidx,
                                  int nfam, int npoles, double tol, float tolf, float* __restrict__ cand,
                                  float* __restrict__ par) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        int64_t a = okey(0.0f), b = okey(1.0f);
        if (!(acos_deg(0.0f) > tolf)) {
            *par = -1.0f;
        } else {
            while (a < b) {  // last key with the test true
                const int64_t mid = a + (b - a + 1) / 2;
                if (acos_deg(okey_float(mid)) > tolf) a = mid; else b = mid - 1;
            }
            *par = okey_float(a);
        }
    }
    if (t >= nfam * npoles) return;
    const int f = t / npoles, c = t - f * npoles;
    const double T = angtab[(size_t)famidx[f] * npoles + c];
    const int64_t k0 = okey(-1.0f), k1 = okey(1.0f);
    // d(x) = T - acos_deg(x) does not decrease with x; the test is -tol < d < tol
    int64_t a = k0, b = k1 + 1;
    while (a < b) {  // first key with d > -tol (k1 + 1: none)
        const int64_t mid = a + (b - a) / 2;
        if (__dsub_rn(T, (double)acos_deg(okey_float(mid))) > -tol) b = mid; else a = mid + 1;
    }
    const int64_t lo = a;
    a = k0 - 1;
    b = k1;
    while (a < b) {  // last key with d < tol (k0 - 1: none)
        const int64_t mid = a + (b - a + 1) / 2;
        if (__dsub_rn(T, (double)acos_deg(okey_float(mid))) < tol) a = mid; else b = mid - 1;
    }
    const int64_t hi = a;
    if (lo > k1 || hi < k0 || lo > hi) {
        cand[2 * t] = INFINITY;
        cand[2 * t + 1] = -INFINITY;
    } else {
        cand[2 * t] = okey_float(lo);
        cand[2 * t + 1] = okey_float(hi);
    }
}


// ---- the scalar QUEST solve (tripletvote.py:955-993), one thread per pattern so that every
// float64 instruction carries a full warp of patterns ----
__global__ void k_quest(QuestInput* __restrict__ qin, int64_t n, int nb, const float* __restrict__ norms,
                        const float* __restrict__ inten, const int64_t* __restrict__ polematch,
                        const double* __restrict__ pole64, double* __restrict__ quat) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        QuestInput& qi = qin[p];
        double qout[4] = {1.0, 0.0, 0.0, 0.0};
        // band weights (tripletvote.py:885-899): the chosen bands' intensities normalised to
        // sum one, stored as float32
        float wsel[32];
        double wq[32];
        for (int j = 0; j < nb; ++j) {
            const float it = inten ? inten[p * nb + j] : 1.0f;
            wq[j] = (qi.ngood >= 3 && ((qi.sel >> j) & 1u)) ? (double)it : 0.0;
        }
        double tot = np_sum(wq, nb);
        for (int j = 0; j < nb; ++j) wsel[j] = qi.ngood >= 3 ? __double2float_rn(__ddiv_rn(wq[j], tot)) : 0.0f;
        // the fit's weights (tripletvote.py:912-914, 940-947)
        for (int j = 0; j < nb; ++j) wq[j] = (double)wsel[j];
        tot = np_maximum(np_sum(wq, nb), 1e-12);
        double wn[32];
        int idx[32];
        int m = 0;
        uint32_t mask = 0;
        for (int j = 0; j < nb; ++j) {
            const double w = __ddiv_rn((double)wsel[j], tot);
            if (w > 1.0e-7) {
                wn[m] = w;
                idx[m] = j;
                mask |= 1u << j;
                ++m;
            }
        }
        qi.mask = m >= 3 ? mask : 0u;
        qi.m = m >= 3 ? m : 0;
        if (m >= 3) {
            const double ws = np_sum(wn, m);
            for (int k = 0; k < m; ++k) wn[k] = __ddiv_rn(wn[k], ws);
            auto bcomp = [&](int k, int c) { return (double)norms[(p * nb + idx[k]) * 3 + c]; };
            auto pcomp = [&](int k, int c) {
                const int64_t pm = polematch[p * nb + idx[k]];
                return pole64[3 * (pm > 0 ? pm : 0) + c];
            };
            // B = (w b)^T p and z = sum_k w_k (b_k x p_k), in the reference's operation order
            double Bm[3][3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    double acc = __dmul_rn(__dmul_rn(wn[0], bcomp(0, r)), pcomp(0, c));
                    for (int k = 1; k < m; ++k) acc = __fma_rn(__dmul_rn(wn[k], bcomp(k, r)), pcomp(k, c), acc);
                    Bm[r][c] = acc;
                }
            double z[3];
            for (int c = 0; c < 3; ++c) {
                const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                double zc = 0.0;
                for (int k = 0; k < m; ++k) {
                    const double cr = __dsub_rn(__dmul_rn(bcomp(k, c1), pcomp(k, c2)), __dmul_rn(bcomp(k, c2), pcomp(k, c1)));
                    const double v = __dmul_rn(wn[k], cr);
                    zc = k == 0 ? v : __dadd_rn(zc, v);
                }
                z[c] = zc;
            }
            double S[3][3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) S[r][c] = __dadd_rn(Bm[r][c], Bm[c][r]);
            double S2[3][3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    S2[r][c] = __fma_rn(S[r][2], S[2][c], __fma_rn(S[r][1], S[1][c], __dmul_rn(S[r][0], S[0][c])));
            const double det =
                __dadd_rn(__dsub_rn(__dmul_rn(S[0][0], __dsub_rn(__dmul_rn(S[1][1], S[2][2]), __dmul_rn(S[1][2], S[2][1]))),
                                    __dmul_rn(S[0][1], __dsub_rn(__dmul_rn(S[1][0], S[2][2]), __dmul_rn(S[1][2], S[2][0])))),
                          __dmul_rn(S[0][2], __dsub_rn(__dmul_rn(S[1][0], S[2][1]), __dmul_rn(S[1][1], S[2][0]))));
            const double kk = __dadd_rn(__dadd_rn(__dsub_rn(__dmul_rn(S[1][1], S[2][2]), __dmul_rn(S[1][2], S[2][1])),
                                                  __dsub_rn(__dmul_rn(S[0][0], S[2][2]), __dmul_rn(S[0][2], S[2][0]))),
                                        __dsub_rn(__dmul_rn(S[0][0], S[1][1]), __dmul_rn(S[1][0], S[0][1])));
            const double sig = __dmul_rn(0.5, __dadd_rn(__dadd_rn(S[0][0], S[1][1]), S[2][2]));
            const double sig2 = __dmul_rn(sig, sig);
            double u[3], v[3];
            for (int c = 0; c < 3; ++c) {
                u[c] = __fma_rn(z[2], S2[2][c], __fma_rn(z[1], S2[1][c], __dmul_rn(z[0], S2[0][c])));
                v[c] = __fma_rn(z[2], S[2][c], __fma_rn(z[1], S[1][c], __dmul_rn(z[0], S[0][c])));
            }
            const double d = __fma_rn(u[2], z[2], __fma_rn(u[1], z[1], __dmul_rn(u[0], z[0])));
            const double c = __dadd_rn(det, __fma_rn(v[2], z[2], __fma_rn(v[1], z[1], __dmul_rn(v[0], z[0]))));
            const double b = __dadd_rn(sig2, __fma_rn(z[2], z[2], __fma_rn(z[1], z[1], __dmul_rn(z[0], z[0]))));
            const double a = __dsub_rn(sig2, kk);
            const double apb = __dadd_rn(a, b);
            const double cst = __dsub_rn(__dadd_rn(__dmul_rn(a, b), __dmul_rn(c, sig)), d);
            double lam = 1.0, dlam = 1e6;
            for (int it = 0; dlam > 1.0e-12 && it < 10; ++it) {
                const double lam0 = lam;
                const double l2 = __dmul_rn(lam, lam);
                const double num = __dadd_rn(__dsub_rn(__dsub_rn(__dmul_rn(l2, l2), __dmul_rn(apb, l2)), __dmul_rn(c, lam)), cst);
                const double den = __dsub_rn(__dsub_rn(__dmul_rn(4.0, __dmul_rn(l2, lam)), __dmul_rn(__dmul_rn(2.0, apb), lam)), c);
                lam = __dsub_rn(lam, __ddiv_rn(num, den));
                dlam = fabs(__dsub_rn(lam0, lam));
            }
            const double beta = __dsub_rn(lam, sig);
            const double alpha = __dadd_rn(__dsub_rn(__dmul_rn(lam, lam), sig2), kk);
            const double gamma = __dsub_rn(__dmul_rn(__dadd_rn(lam, sig), alpha), det);
            double X[3];
            for (int r = 0; r < 3; ++r) {
                double M[3];
                for (int cc = 0; cc < 3; ++cc)
                    M[cc] = __dadd_rn(__dadd_rn(r == cc ? alpha : 0.0, __dmul_rn(beta, S[r][cc])), S2[r][cc]);
                X[r] = __fma_rn(M[2], z[2], __fma_rn(M[1], z[1], __dmul_rn(M[0], z[0])));
            }
            const double qn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(gamma, gamma), __dmul_rn(X[0], X[0])),
                                                             __dmul_rn(X[1], X[1])), __dmul_rn(X[2], X[2])));
            qout[0] = __ddiv_rn(gamma, qn);
            qout[1] = __ddiv_rn(X[0], qn);
            qout[2] = __ddiv_rn(X[1], qn);
            qout[3] = __ddiv_rn(X[2], qn);
            if (gamma < 0.0)
                for (int t = 0; t < 4; ++t) qout[t] = -qout[t];
        }
        for (int t = 0; t < 4; ++t) quat[4 * p + t] = qout[t];
    }
}

// ---- per-band and mean fit (tripletvote.py:994-1018, rotlib.quat_vectorL1N with p = 1, and
// the arccos of bandindex, :601-604), one thread per pattern ----
__global__ void k_quest_fit(const QuestInput* __restrict__ qin, const float* __restrict__ norms,
                            const int64_t* __restrict__ polematch, const double* __restrict__ pole64,
                            const double* __restrict__ quat, int64_t n, int nb, double* __restrict__ fit,
                            double* __restrict__ bandfit) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const QuestInput& qi = qin[p];
        const int m = qi.m >= 3 ? qi.m : 0;
        const double w0 = quat[4 * p], r0 = quat[4 * p + 1], r1 = quat[4 * p + 2], r2 = quat[4 * p + 3];
        double dots[32];
        int k = 0;
        for (int j = 0; j < nb; ++j) {
            double bd = -1.0;
            if (m > 0 && ((qi.mask >> j) & 1u)) {
                const float* f = norms + (p * nb + j) * 3;
                const double vv[3] = {(double)f[0], (double)f[1], (double)f[2]};
                const int64_t pm = polematch[p * nb + j];
                const double* pp = pole64 + 3 * (pm > 0 ? pm : 0);
                double t[3] = {__dsub_rn(__dmul_rn(r1, vv[2]), __dmul_rn(r2, vv[1])),
                               __dsub_rn(__dmul_rn(r2, vv[0]), __dmul_rn(r0, vv[2])),
                               __dsub_rn(__dmul_rn(r0, vv[1]), __dmul_rn(r1, vv[0]))};
                for (int cc = 0; cc < 3; ++cc) t[cc] = __dadd_rn(t[cc], __dmul_rn(w0, vv[cc]));
                const double t2[3] = {__dsub_rn(__dmul_rn(r1, t[2]), __dmul_rn(r2, t[1])),
                                      __dsub_rn(__dmul_rn(r2, t[0]), __dmul_rn(r0, t[2])),
                                      __dsub_rn(__dmul_rn(r0, t[1]), __dmul_rn(r1, t[0]))};
                double sd = 0.0;
                for (int cc = 0; cc < 3; ++cc)
                    sd = __dadd_rn(sd, __dmul_rn(__dadd_rn(__dmul_rn(2.0, t2[cc]), vv[cc]), pp[cc]));
                bd = sd;
                dots[k++] = sd;
            }
            const double bc = bd < -1.0 ? -1.0 : (bd > 1.0 ? 1.0 : bd);
            bandfit[p * nb + j] = __dmul_rn(acos(bc), kRadeg);
        }
        double mad = -1.0;
        if (m > 0) mad = __ddiv_rn(np_sum(dots, m), (double)m);
        const double mc = mad < -1.0 ? -1.0 : (mad > 1.0 ? 1.0 : mad);
        fit[p] = __dmul_rn(acos(mc), kRadeg);
    }
}

__global__ void __launch_bounds__(kWarps * 32, 3) k_band_index(VoteArgs A) {
    extern __shared__ __align__(16) float vsm[];
    float* s_iv = vsm;
    int* s_orig = (int*)(s_iv + 6 * A.ntrip);
    float* s_pole = (float*)(s_orig + A.ntrip);
    int* s_pfam = (int*)(s_pole + 3 * A.npoles);
    for (int t = threadIdx.x; t < 6 * A.ntrip; t += blockDim.x) s_iv[t] = A.iv[t];
    for (int t = threadIdx.x; t < A.ntrip; t += blockDim.x) s_orig[t] = A.orig[t];
    for (int t = threadIdx.x; t < 3 * A.npoles; t += blockDim.x) s_pole[t] = A.pole[t];
    for (int t = threadIdx.x; t < A.npoles; t += blockDim.x) s_pfam[t] = A.pfam[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* w = vsm + block_words(A.ntrip, A.npoles) + warp * warp_words(A.nb, A.nfam);
    const int64_t stride = (int64_t)gridDim.x * kWarps;
    for (int64_t p = (int64_t)blockIdx.x * kWarps + warp; p < A.n; p += stride)
        index_pattern(A, p, lane, s_iv, s_orig, s_pole, s_pfam, w);
}

// ---- band weights and pattern quality, _ebsd_index_single.py:751-763 ----
__global__ void k_band_intensity(const float* __restrict__ mx, const float* __restrict__ nmx,
                                 const float* __restrict__ theta, const float* __restrict__ rho,
                                 const int8_t* __restrict__ valid, int64_t n, int nb, float rhomax,
                                 float* __restrict__ adj, float* __restrict__ pq, float* __restrict__ iq) {
    const float lo = (float)(2.0 * 3.141592653589793 / 180.0);
    const float hi = (float)(178.0 * 3.141592653589793 / 180.0);
    float a[128];
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        for (int b = 0; b < nb; ++b) {
            const int64_t e = p * nb + b;
            const float v = (float)valid[e];
            float t = __fmul_rn(__fmul_rn(-1.0f, fabsf(rho[e])), 0.5f);
            t = __fmul_rn(__fadd_rn(__fdiv_rn(t, rhomax), 1.0f), mx[e]);
            t = __fmul_rn(t, __fdiv_rn(__fadd_rn(theta[e] > lo ? 1.0f : 0.0f, 0.5f), 2.0f));
            t = __fmul_rn(t, __fdiv_rn(__fadd_rn(theta[e] < hi ? 1.0f : 0.0f, 0.5f), 2.0f));
            adj[e] = __fmul_rn(t, v);
        }
        if (pq) {
            for (int b = 0; b < nb; ++b) a[b] = __fmul_rn(mx[p * nb + b], (float)valid[p * nb + b]);
            pq[p] = __fdiv_rn(np_sum(a, nb), (float)nb);
        }
        if (iq) {
            for (int b = 0; b < nb; ++b) a[b] = __fmul_rn(nmx[p * nb + b], (float)valid[p * nb + b]);
            iq[p] = __fdiv_rn(np_sum(a, nb), (float)nb);
        }
    }
}

// ---- host: float32 acceptance interval of |T - a| <= tol (evaluated in float64) ----
inline uint32_t fkey(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
inline float funkey(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline bool within(double T, float a, double tol) { return std::fabs(T - (double)a) <= tol; }

void accept_interval(double T, double tol, float* lo, float* hi) {
    const float fT = (float)T;
    if (!(tol >= 0.0) || !std::isfinite(T) || !within(T, fT, tol)) {
        *lo = INFINITY;
        *hi = -INFINITY;
        return;
    }
    const uint32_t kT = fkey(fT);
    uint32_t a = fkey(-FLT_MAX), b = kT;  // smallest key in [a, b] that passes
    while (a < b) {
        const uint32_t mid = a + (b - a) / 2;
        if (within(T, funkey(mid), tol)) b = mid; else a = mid + 1;
    }
    *lo = funkey(a);
    a = kT;
    b = fkey(FLT_MAX);  // largest key in [a, b] that passes
    while (a < b) {
        const uint32_t mid = a + (b - a + 1) / 2;
        if (within(T, funkey(mid), tol)) a = mid; else b = mid - 1;
    }
    *hi = funkey(a);
}

}  // namespace
}  // namespace ebsd

using namespace ebsd;

extern "C" int ebsd_vote_plan_create(const ebsd_triplib_desc* d, int device, ebsd_vote_plan_t* out) {
    if (!d || !out) return EBSD_E_ARG;
    *out = nullptr;
    if (d->nfam < 2 || d->nfam > 16 || d->ntrip < 1 || d->ntrip > 8192 || d->npoles < 1 || d->npoles > 512)
        return EBSD_E_ARG;
    if (!d->trip_angles || !d->trip_family || !d->lut || !d->poles_cart || !d->pole_family || !d->ang_table ||
        !d->fam_count || !d->fam_index)
        return EBSD_E_ARG;
    const int nt = d->ntrip, np_ = d->npoles, nf = d->nfam;
    for (int i = 0; i < 81; ++i)
        if (d->lut[i] < 0 || d->lut[i] > 2) return EBSD_E_ARG;
    for (int i = 0; i < 3 * nt; ++i)
        if (d->trip_family[i] < 0 || d->trip_family[i] >= nf) return EBSD_E_ARG;
    for (int i = 0; i < np_; ++i)
        if (d->pole_family[i] < 0 || d->pole_family[i] >= nf) return EBSD_E_ARG;
    for (int f = 0; f < nf; ++f)
        if (d->fam_index[f] < 0 || d->fam_count[f] < 0 || d->fam_index[f] + d->fam_count[f] > np_) return EBSD_E_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return EBSD_E_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return EBSD_E_DEVICE;

    auto* p = new ebsd_vote_plan_s();
    p->device = device;
    p->nfam = nf;
    p->ntrip = nt;
    p->npoles = np_;
    p->tol = d->ang_tol;
    p->early = d->nband_earlyexit;
    p->simpleq = d->simple_qweights ? 1 : 0;
    for (int s0 = 0; s0 < 3; ++s0)
        for (int s1 = 0; s1 < 3; ++s1)
            for (int s2 = 0; s2 < 3; ++s2) {
                int code = 0;
                for (int r = 0; r < 3; ++r) code |= int(d->lut[((r * 3 + s0) * 3 + s1) * 3 + s2]) << (2 * r);
                p->lut[s0 * 9 + s1 * 3 + s2] = (uint8_t)code;
            }
    std::vector<float> iv0(6 * (size_t)nt);
    std::vector<uint32_t> tf(nt);
    for (int q = 0; q < nt; ++q) {
        for (int c = 0; c < 3; ++c)
            accept_interval(d->trip_angles[3 * q + c], d->ang_tol, &iv0[(2 * c) * nt + q], &iv0[(2 * c + 1) * nt + q]);
        tf[q] = uint32_t(d->trip_family[3 * q]) | uint32_t(d->trip_family[3 * q + 1]) << 8 |
                uint32_t(d->trip_family[3 * q + 2]) << 16;
    }
    // interval rows sorted by the lower end of the first angle's interval (library order kept
    // in d_orig), so that a band triplet scans only the rows whose first interval can hold it
    std::vector<int32_t> order(nt);
    for (int q = 0; q < nt; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return iv0[a] < iv0[b]; });
    std::vector<float> iv(6 * (size_t)nt);
    double wmax = 0.0;
    for (int r = 0; r < nt; ++r) {
        const int q = order[r];
        for (int c = 0; c < 6; ++c) iv[(size_t)c * nt + r] = iv0[(size_t)c * nt + q];
        if (iv0[q] <= iv0[nt + q]) wmax = std::max(wmax, (double)iv0[nt + q] - (double)iv0[q]);
    }
    p->win = (float)(wmax + 1e-3);
    std::vector<float> pole(3 * (size_t)np_);
    for (int i = 0; i < np_; ++i)
        for (int c = 0; c < 3; ++c) pole[c * np_ + i] = (float)d->poles_cart[3 * i + c];
    std::vector<int32_t> fidx(nf);
    for (int f = 0; f < nf; ++f) fidx[f] = (int32_t)d->fam_index[f];

    auto up = [](void** dst, const void* src, size_t bytes) -> int {
        if (cudaMalloc(dst, bytes) != cudaSuccess) return EBSD_E_NOMEM;
        if (cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return EBSD_E_LAUNCH;
        return EBSD_OK;
    };
    int rc = EBSD_OK;
    if (!rc) rc = up((void**)&p->d_iv, iv.data(), iv.size() * 4);
    if (!rc) rc = up((void**)&p->d_tfam, tf.data(), tf.size() * 4);
    if (!rc) rc = up((void**)&p->d_tang, d->trip_angles, 3 * (size_t)nt * 8);
    if (!rc) rc = up((void**)&p->d_pole, pole.data(), pole.size() * 4);
    if (!rc) rc = up((void**)&p->d_pole64, d->poles_cart, 3 * (size_t)np_ * 8);
    if (!rc) rc = up((void**)&p->d_pfam, d->pole_family, (size_t)np_ * 4);
    if (!rc) rc = up((void**)&p->d_angtab, d->ang_table, (size_t)np_ * np_ * 8);
    if (!rc) rc = up((void**)&p->d_famcnt, d->fam_count, (size_t)nf * 4);
    if (!rc) rc = up((void**)&p->d_famidx, fidx.data(), (size_t)nf * 4);
    if (!rc) rc = up((void**)&p->d_orig, order.data(), (size_t)nt * 4);
    if (!rc && cudaMalloc((void**)&p->d_cand, (size_t)nf * np_ * 2 * 4) != cudaSuccess) rc = EBSD_E_NOMEM;
    if (!rc && cudaMalloc((void**)&p->d_par, 4) != cudaSuccess) rc = EBSD_E_NOMEM;
    if (!rc) {
        const int total = nf * np_;
        k_vote_thresholds<<<(total + 127) / 128, 128>>>(p->d_angtab, p->d_famidx, nf, np_, p->tol, (float)p->tol,
                                                        p->d_cand, p->d_par);
        rc = launch_status();
        if (!rc && cudaMemcpy(&p->par, p->d_par, 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = EBSD_E_LAUNCH;
    }
    if (rc) {
        ebsd_vote_plan_destroy(p);
        return rc;
    }
    *out = p;
    return EBSD_OK;
}

extern "C" int ebsd_vote_plan_destroy(ebsd_vote_plan_t p) {
    if (!p) return EBSD_OK;
    cudaSetDevice(p->device);
    cudaFree(p->d_iv);
    cudaFree(p->d_tfam);
    cudaFree(p->d_tang);
    cudaFree(p->d_pole);
    cudaFree(p->d_pole64);
    cudaFree(p->d_pfam);
    cudaFree(p->d_angtab);
    cudaFree(p->d_famcnt);
    cudaFree(p->d_famidx);
    cudaFree(p->d_cand);
    cudaFree(p->d_par);
    cudaFree(p->d_orig);
    cudaFree(p->d_quest);
    delete p;
    return EBSD_OK;
}

extern "C" int ebsd_band_index(ebsd_vote_plan_t p, const float* d_norms, const float* d_intensity, int64_t n,
                               int32_t nBands, const ebsd_index_out* out, void* stream) {
    if (!p || !out || n < 0 || nBands < 1 || nBands > 32) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if (!d_norms || !out->quat || !out->fit || !out->cm || !out->polematch || !out->nmatch || !out->ij ||
        !out->acc_correct || !out->bandfit)
        return EBSD_E_ARG;
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    const size_t words = block_words(p->ntrip, p->npoles) + kWarps * warp_words(nBands, p->nfam);
    const size_t smem = words * 4;
    int dev_max = 0;
    cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
    if (smem > (size_t)dev_max) return EBSD_E_UNSUPPORTED;
    static int raised[64] = {};
    if (smem > 48 * 1024 && raised[p->device] < (int)smem) {
        EBSD_CUDA_TRY(cudaFuncSetAttribute(k_band_index, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        raised[p->device] = (int)smem;
    }
    VoteArgs A;
    A.iv = p->d_iv;
    A.tfam = p->d_tfam;
    A.tang = p->d_tang;
    A.pole = p->d_pole;
    A.pole64 = p->d_pole64;
    A.pfam = p->d_pfam;
    A.angtab = p->d_angtab;
    A.famcnt = p->d_famcnt;
    A.famidx = p->d_famidx;
    A.cand = p->d_cand;
    A.par = p->par;
    A.orig = p->d_orig;
    A.win = p->win;
    A.nfam = p->nfam;
    A.ntrip = p->ntrip;
    A.npoles = p->npoles;
    A.nb = nBands;
    A.tol_f = (float)p->tol;
    A.tol = p->tol;
    A.early = p->early;
    A.simpleq = p->simpleq;
    std::memcpy(A.lut, p->lut, 27);
    A.lut[27] = 0;
    // patterns go in pieces of at most kQuestChunk; the hand-over scratch is allocated on the
    // first call (make it outside a CUDA-graph capture) and reused
    constexpr int64_t kQuestChunk = 1 << 20;
    const int64_t cap = std::min<int64_t>(n, kQuestChunk);
    if (cap > p->quest_cap) {
        cudaFree(p->d_quest);
        p->d_quest = nullptr;
        p->quest_cap = 0;
        EBSD_CUDA_TRY(cudaMalloc(&p->d_quest, (size_t)cap * sizeof(QuestInput)));
        p->quest_cap = cap;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_band_index, kWarps * 32, smem);
    if (per_sm < 1) per_sm = 1;
    const int nf = p->nfam;
    for (int64_t off = 0; off < n; off += kQuestChunk) {
        const int64_t cnt = std::min<int64_t>(kQuestChunk, n - off);
        A.norms = d_norms + off * nBands * 3;
        A.inten = d_intensity ? d_intensity + off * nBands : nullptr;
        A.n = cnt;
        ebsd_index_out o = *out;
        o.quat += 4 * off;
        o.fit += off;
        o.cm += off;
        o.polematch += off * nBands;
        o.nmatch += off;
        o.ij += 4 * off;
        o.acc_correct += off;
        o.bandfit += off * nBands;
        if (o.accw) o.accw += off * nf * nBands;
        if (o.accn) o.accn += off * nf * nBands;
        if (o.bandfam) o.bandfam += off * nBands;
        if (o.bandrank) o.bandrank += off * nBands;
        if (o.polevalid) o.polevalid += off * nBands;
        A.out = o;
        A.quest = (QuestInput*)p->d_quest;
        const int64_t need = (cnt + kWarps - 1) / kWarps;
        const int blocks = (int)std::min<int64_t>(need, (int64_t)sms * per_sm);
        k_band_index<<<blocks, kWarps * 32, smem, (cudaStream_t)stream>>>(A);
        int rc = launch_status();
        if (rc != EBSD_OK) return rc;
        const int qb = (int)std::min<int64_t>((cnt + 127) / 128, (int64_t)sms * 16);
        k_quest<<<qb, 128, 0, (cudaStream_t)stream>>>(A.quest, cnt, nBands, A.norms, A.inten, o.polematch,
                                                     p->d_pole64, o.quat);
        if ((rc = launch_status()) != EBSD_OK) return rc;
        k_quest_fit<<<qb, 128, 0, (cudaStream_t)stream>>>(A.quest, A.norms, o.polematch, p->d_pole64, o.quat, cnt,
                                                         nBands, o.fit, o.bandfit);
        if ((rc = launch_status()) != EBSD_OK) return rc;
    }
    return EBSD_OK;
}

extern "C" int ebsd_band_intensity(const float* d_max, const float* d_normmax, const float* d_theta,
                                   const float* d_rho, const int8_t* d_valid, int64_t n, int32_t nBands,
                                   float rhomax, float* d_adj, float* d_pq, float* d_iq, void* stream) {
    if (n < 0 || nBands < 1 || nBands > 128) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if (!d_max || !d_theta || !d_rho || !d_valid || !d_adj || (d_iq && !d_normmax)) return EBSD_E_ARG;
    const int blocks = (int)std::min<int64_t>((n + 127) / 128, 152 * 8);
    k_band_intensity<<<blocks, 128, 0, (cudaStream_t)stream>>>(d_max, d_normmax, d_theta, d_rho, d_valid, n,
                                                               nBands, rhomax, d_adj, d_pq, d_iq);
    return launch_status();
}
