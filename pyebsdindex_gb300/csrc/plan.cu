// C-ABI entry points: plan lifetime, method dispatch, chunking and the host-buffer pipeline.
#include "ebsd_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

using namespace ebsd;

namespace {

template <typename T>
int upload(T** dst, const T* src, size_t count) {
    *dst = nullptr;
    if (count == 0) return EBSD_OK;
    EBSD_CUDA_TRY(cudaMalloc((void**)dst, count * sizeof(T)));
    EBSD_CUDA_TRY(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return EBSD_OK;
}

void free_plan_tables(ebsd_plan_s* p) {
    cudaFree(p->d_lut16);
    cudaFree(p->d_lut32);
    cudaFree(p->d_count);
    cudaFree(p->d_rdnmask);
    cudaFree(p->d_kernel);
    cudaFree(p->d_kernel64);
    cudaFree(p->d_ksep);
    cudaFree(p->d_theta);
    cudaFree(p->d_rho);
    cudaFree(p->d_bg);
    cudaFree(p->d_bgf);
    fused_release(p);
    cudaFree(p->ws.ptr);
    p->ws = Workspace{};
    cudaFree(p->stats.ptr);
    p->stats = Workspace{};
    for (int i = 0; i < 2; ++i) {
        if (p->hstream[i]) cudaStreamDestroy(p->hstream[i]);
        if (p->hevent[i]) cudaEventDestroy(p->hevent[i]);
        cudaFree(p->h_in_dev[i]);
        cudaFree(p->h_out_dev[i]);
        p->hstream[i] = nullptr;
        p->hevent[i] = nullptr;
        p->h_in_dev[i] = nullptr;
        p->h_out_dev[i] = nullptr;
    }
}

bool is_plain(int method) { return method == EBSD_PLAIN_F32 || method == EBSD_PLAIN_F64; }
bool is_fused(int method) { return method == EBSD_FUSED_F32 || method == EBSD_FUSED_F16; }

int64_t default_chunk(const ebsd_plan_s* p, int method) {
    if (is_fused(method)) return 1 << 20;
    // per-stage intermediates: keep a chunk's workspace near 2 GB
    size_t per = plain_workspace_bytes(p, method, 1);
    int64_t c = (int64_t)((size_t)2 << 30) / (int64_t)std::max<size_t>(per, 1);
    return std::max<int64_t>(1, std::min<int64_t>(c, 16384));
}

size_t workspace_bytes(const ebsd_plan_s* p, int method, int64_t chunk) {
    return is_plain(method) ? plain_workspace_bytes(p, method, chunk)
                            : fused_workspace_bytes(p, method, chunk);
}

int reserve(ebsd_plan_s* p, int method, int64_t chunk) {
    size_t need = workspace_bytes(p, method, chunk);
    if (need > p->ws.bytes) {
        cudaFree(p->ws.ptr);
        p->ws = Workspace{};
        void* ptr = nullptr;
        EBSD_CUDA_TRY(cudaMalloc(&ptr, need));
        p->ws.ptr = ptr;
        p->ws.bytes = need;
    }
    return EBSD_OK;
}

int check_method(const ebsd_plan_s* p, int method) {
    if (is_plain(method)) return EBSD_OK;
    if (is_fused(method)) return fused_supported(p, method) ? EBSD_OK : EBSD_E_UNSUPPORTED;
    return EBSD_E_ARG;
}

ebsd_bands offset_bands(const ebsd_bands& b, int64_t off, int nB) {
    int64_t o = off * nB;
    ebsd_bands r;
    r.max = b.max + o;
    r.normmax = b.normmax + o;
    r.maxloc = b.maxloc + 2 * o;
    r.avemax = b.avemax + o;
    r.aveloc = b.aveloc + 2 * o;
    r.width = b.width + o;
    r.theta = b.theta + o;
    r.rho = b.rho + o;
    r.valid = b.valid + o;
    return r;
}

int run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
              const ebsd_bands* out, int64_t out_off, cudaStream_t st, int64_t* launches) {
    if (is_plain(method)) return plain_run_chunk(p, method, dtype, d_pats, n, out, out_off, st, launches);
    return fused_run_chunk(p, method, dtype, d_pats, n, out, out_off, st, launches);
}

}  // namespace

extern "C" {

const char* ebsd_version(void) { return "ebsdgpu 0.1 (sm_103a)"; }

const char* ebsd_strerror(int code) {
    switch (code) {
        case EBSD_OK: return "success";
        case EBSD_E_ARG: return "invalid argument";
        case EBSD_E_DTYPE: return "unsupported pattern data type (uint8, uint16, float32 are supported)";
        case EBSD_E_NOMEM: return "out of device or pinned host memory";
        case EBSD_E_LAUNCH: return "CUDA kernel launch or runtime call failed";
        case EBSD_E_UNSUPPORTED: return "plan shape not supported by this method";
        case EBSD_E_DEVICE: return "no usable CUDA device";
        case EBSD_E_TIMEOUT: return "a bounded device-side wait timed out";
        case EBSD_E_SCRATCH: return "request needs more scratch than the library's 64 MiB static device array holds";
        default: return "unknown error";
    }
}

int ebsd_plan_create(const ebsd_plan_desc* d, int device, ebsd_plan_t* out) {
    if (!d || !out) return EBSD_E_ARG;
    *out = nullptr;
    if (d->H <= 0 || d->W <= 0 || d->nTheta <= 0 || d->nRho <= 0) return EBSD_E_ARG;
    if (d->nBands <= 0 || d->nBands > kMaxBands) return EBSD_E_ARG;
    if (d->pad_rho < 0 || d->pad_theta < 0 || d->pad_theta > d->nTheta) return EBSD_E_ARG;
    if (d->peak_rho <= 0 || d->peak_theta <= 0 || d->ksz_rho <= 0 || d->ksz_theta <= 0) return EBSD_E_ARG;
    if (!(d->ksz_rho & 1) || !(d->ksz_theta & 1)) return EBSD_E_ARG;
    if (!d->kernel || !d->lut || !d->rdnmask || !d->theta || !d->rho || d->lut_len <= 0) return EBSD_E_ARG;
    // the band fit reads +-1 around a peak and the max filter +-peak/2: padding must cover it
    if (d->pad_rho < 1 || d->pad_theta < 1) return EBSD_E_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return EBSD_E_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return EBSD_E_DEVICE;

    ebsd_plan_s* p = new (std::nothrow) ebsd_plan_s();
    if (!p) return EBSD_E_NOMEM;
    p->device = device;
    p->H = d->H;
    p->W = d->W;
    p->nPx = d->H * d->W;
    p->nTheta = d->nTheta;
    p->nRho = d->nRho;
    p->nRays = d->nTheta * d->nRho;
    p->nB = d->nBands;
    p->p0 = d->pad_rho;
    p->p1 = d->pad_theta;
    p->pk0 = d->peak_rho;
    p->pk1 = d->peak_theta;
    p->k0 = d->ksz_rho;
    p->k1 = d->ksz_theta;
    p->R = d->nRho + 2 * d->pad_rho;
    p->Tp = d->nTheta + 2 * d->pad_theta;

    // ---- LUT: count the valid prefix of every ray, re-encode entry-major ----
    const int L = d->lut_len;
    const int nRays = p->nRays;
    std::vector<int32_t> count(nRays);
    int maxc = 0;
    for (int r = 0; r < nRays; ++r) {
        const int64_t* ray = d->lut + (size_t)r * L;
        int c = 0;
        while (c < L && ray[c] >= 0 && ray[c] < p->nPx) ++c;
        for (int k = c; k < L; ++k) {
            if (ray[k] >= 0 && ray[k] < p->nPx) {  // valid entry after a sentinel: not sorted
                delete p;
                return EBSD_E_ARG;
            }
        }
        count[r] = c;
        maxc = std::max(maxc, c);
    }
    p->maxCount = maxc;
    int rc = EBSD_OK;
    if (p->nPx < 65535) {
        std::vector<uint16_t> lut((size_t)std::max(maxc, 1) * nRays, 0xFFFF);
        for (int r = 0; r < nRays; ++r)
            for (int k = 0; k < count[r]; ++k) lut[(size_t)k * nRays + r] = (uint16_t)d->lut[(size_t)r * L + k];
        rc = upload(&p->d_lut16, lut.data(), lut.size());
    } else {
        std::vector<int32_t> lut((size_t)std::max(maxc, 1) * nRays, -1);
        for (int r = 0; r < nRays; ++r)
            for (int k = 0; k < count[r]; ++k) lut[(size_t)k * nRays + r] = (int32_t)d->lut[(size_t)r * L + k];
        rc = upload(&p->d_lut32, lut.data(), lut.size());
    }
    if (rc == EBSD_OK) rc = upload(&p->d_count, count.data(), count.size());
    if (rc == EBSD_OK) rc = upload(&p->d_rdnmask, d->rdnmask, (size_t)nRays);
    if (rc == EBSD_OK) rc = upload(&p->d_kernel, d->kernel, (size_t)p->k0 * p->k1);
    p->h_kernel.assign(d->kernel, d->kernel + (size_t)p->k0 * p->k1);
    {
        // rank-1 factors from the centre row and column: ku[a] = K[a][h1],
        // kw[b] = K[h0][b] / K[h0][h1]; separable when every product is within two ulps of
        // the largest tap from the tap it replaces
        const int h0 = p->k0 / 2, h1 = p->k1 / 2;
        const float kc = p->h_kernel[(size_t)h0 * p->k1 + h1];
        float kmax = 0.0f;
        for (float v : p->h_kernel) kmax = std::max(kmax, std::fabs(v));
        p->h_ku.resize(p->k0);
        p->h_kw.resize(p->k1);
        for (int a = 0; a < p->k0; ++a) p->h_ku[a] = p->h_kernel[(size_t)a * p->k1 + h1];
        for (int b = 0; b < p->k1; ++b) p->h_kw[b] = kc != 0.0f ? (float)((double)p->h_kernel[(size_t)h0 * p->k1 + b] / (double)kc) : 0.0f;
        bool sep = kc != 0.0f && kmax > 0.0f;
        for (int a = 0; sep && a < p->k0; ++a)
            for (int b = 0; b < p->k1; ++b)
                if (std::fabs(p->h_ku[a] * p->h_kw[b] - p->h_kernel[(size_t)a * p->k1 + b]) > kmax * 2.4e-7f) sep = false;
        p->sep = sep ? 1 : 0;
        std::vector<float> ks(p->h_ku);
        ks.insert(ks.end(), p->h_kw.begin(), p->h_kw.end());
        if (rc == EBSD_OK) rc = upload(&p->d_ksep, ks.data(), ks.size());
    }
    if (rc == EBSD_OK) {
        std::vector<double> k64(d->kernel, d->kernel + (size_t)p->k0 * p->k1);
        rc = upload(&p->d_kernel64, k64.data(), k64.size());
    }
    if (rc == EBSD_OK) {
        std::vector<double> th(d->theta, d->theta + p->nTheta), rh(d->rho, d->rho + p->nRho);
        rc = upload(&p->d_theta, th.data(), th.size());
        if (rc == EBSD_OK) rc = upload(&p->d_rho, rh.data(), rh.size());
    }
    if (rc == EBSD_OK && d->background) {
        p->bg_mode = d->background_f32 ? 2 : 1;
        rc = upload(&p->d_bg, d->background, (size_t)p->nPx);
        if (rc == EBSD_OK) {
            std::vector<float> bgf(d->background, d->background + p->nPx);
            rc = upload(&p->d_bgf, bgf.data(), bgf.size());
        }
    }
    if (rc == EBSD_OK) rc = fused_prepare(p, d);
    if (rc != EBSD_OK) {
        free_plan_tables(p);
        delete p;
        return rc;
    }
    *out = p;
    return EBSD_OK;
}

int ebsd_plan_destroy(ebsd_plan_t p) {
    if (!p) return EBSD_E_ARG;
    cudaSetDevice(p->device);
    cudaDeviceSynchronize();
    free_plan_tables(p);
    delete p;
    return EBSD_OK;
}

int ebsd_method_supported(ebsd_plan_t p, int method) {
    if (!p) return EBSD_E_ARG;
    if (is_plain(method)) return 1;
    if (is_fused(method)) return fused_supported(p, method) ? 1 : 0;
    return EBSD_E_ARG;
}

int ebsd_plan_reserve(ebsd_plan_t p, int method, int64_t max_chunk) {
    if (!p || max_chunk <= 0) return EBSD_E_ARG;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    return reserve(p, method, is_plain(method) ? std::min<int64_t>(max_chunk, 65535) : max_chunk);
}

int64_t ebsd_last_launch_count(ebsd_plan_t p) { return p ? p->last_launches : -1; }

int ebsd_find_bands(ebsd_plan_t p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* d_out, int64_t chunk, void* stream) {
    if (!p || !d_out || n < 0) return EBSD_E_ARG;
    if (n > 0 && !d_pats) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    if (!d_out->max || !d_out->normmax || !d_out->maxloc || !d_out->avemax || !d_out->aveloc ||
        !d_out->width || !d_out->theta || !d_out->rho || !d_out->valid)
        return EBSD_E_ARG;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    if (chunk <= 0) chunk = default_chunk(p, method);
    if (is_plain(method)) chunk = std::min<int64_t>(chunk, 65535);
    chunk = std::min(chunk, n);
    rc = reserve(p, method, chunk);
    if (rc != EBSD_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    size_t es = elem_size(dtype);
    for (int64_t s = 0; s < n; s += chunk) {
        int64_t m = std::min(chunk, n - s);
        rc = run_chunk(p, method, dtype, (const char*)d_pats + (size_t)s * p->nPx * es, m, d_out, s, st,
                       &p->last_launches);
        if (rc != EBSD_OK) return rc;
    }
    return EBSD_OK;
}

int ebsd_find_bands_host(ebsd_plan_t p, int method, int dtype, const void* h_pats, int64_t n,
                         const ebsd_bands* h_out, int64_t chunk) {
    if (!p || !h_out || n < 0) return EBSD_E_ARG;
    if (n > 0 && !h_pats) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    if (!h_out->max || !h_out->normmax || !h_out->maxloc || !h_out->avemax || !h_out->aveloc ||
        !h_out->width || !h_out->theta || !h_out->rho || !h_out->valid)
        return EBSD_E_ARG;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    if (chunk <= 0) chunk = is_plain(method) ? default_chunk(p, method) : 65536;
    if (is_plain(method)) chunk = std::min<int64_t>(chunk, 65535);
    chunk = std::min(chunk, n);
    rc = reserve(p, method, chunk);
    if (rc != EBSD_OK) return rc;

    const int nB = p->nB;
    size_t es = elem_size(dtype);
    size_t in_bytes = (size_t)chunk * p->nPx * es;
    // nine fields per band: eight float fields of which maxloc/aveloc are pairs (10 floats)
    // plus the int8 'valid' = 41 bytes per band
    size_t out_bytes = (size_t)chunk * nB * (10 * sizeof(float) + 1) + 256;
    for (int i = 0; i < 2; ++i) {
        if (!p->hstream[i]) EBSD_CUDA_TRY(cudaStreamCreateWithFlags(&p->hstream[i], cudaStreamNonBlocking));
        if (!p->hevent[i]) EBSD_CUDA_TRY(cudaEventCreateWithFlags(&p->hevent[i], cudaEventDisableTiming));
    }
    if (in_bytes > p->h_in_bytes) {
        for (int i = 0; i < 2; ++i) {
            cudaFree(p->h_in_dev[i]);
            p->h_in_dev[i] = nullptr;
        }
        p->h_in_bytes = 0;
        for (int i = 0; i < 2; ++i) EBSD_CUDA_TRY(cudaMalloc(&p->h_in_dev[i], in_bytes));
        p->h_in_bytes = in_bytes;
    }
    if (out_bytes > p->h_out_bytes) {
        for (int i = 0; i < 2; ++i) {
            cudaFree(p->h_out_dev[i]);
            p->h_out_dev[i] = nullptr;
        }
        p->h_out_bytes = 0;
        for (int i = 0; i < 2; ++i) EBSD_CUDA_TRY(cudaMalloc(&p->h_out_dev[i], out_bytes));
        p->h_out_bytes = out_bytes;
    }
    // the workspace is shared by both streams: chunk k+1's compute waits for chunk k's
    // compute (event), while its H2D copy overlaps chunk k's compute and D2H copy.
    cudaEvent_t done_compute[2];
    for (int i = 0; i < 2; ++i) EBSD_CUDA_TRY(cudaEventCreateWithFlags(&done_compute[i], cudaEventDisableTiming));
    int slot = 0;
    int64_t prev = -1;
    for (int64_t s = 0; s < n; s += chunk, slot ^= 1) {
        int64_t m = std::min(chunk, n - s);
        cudaStream_t st = p->hstream[slot];
        EBSD_CUDA_TRY(cudaMemcpyAsync(p->h_in_dev[slot], (const char*)h_pats + (size_t)s * p->nPx * es,
                                      (size_t)m * p->nPx * es, cudaMemcpyHostToDevice, st));
        if (prev >= 0) EBSD_CUDA_TRY(cudaStreamWaitEvent(st, done_compute[slot ^ 1], 0));
        char* ob = (char*)p->h_out_dev[slot];
        size_t nb = (size_t)m * nB;
        ebsd_bands dev;
        dev.max = (float*)ob;
        dev.normmax = dev.max + nb;
        dev.maxloc = dev.normmax + nb;
        dev.avemax = dev.maxloc + 2 * nb;
        dev.aveloc = dev.avemax + nb;
        dev.width = dev.aveloc + 2 * nb;
        dev.theta = dev.width + nb;
        dev.rho = dev.theta + nb;
        dev.valid = (int8_t*)(dev.rho + nb);
        rc = run_chunk(p, method, dtype, p->h_in_dev[slot], m, &dev, 0, st, &p->last_launches);
        if (rc != EBSD_OK) break;
        EBSD_CUDA_TRY(cudaEventRecord(done_compute[slot], st));
        ebsd_bands ho = offset_bands(*h_out, s, nB);
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.max, dev.max, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.normmax, dev.normmax, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.maxloc, dev.maxloc, nb * 8, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.avemax, dev.avemax, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.aveloc, dev.aveloc, nb * 8, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.width, dev.width, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.theta, dev.theta, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.rho, dev.rho, nb * 4, cudaMemcpyDeviceToHost, st));
        EBSD_CUDA_TRY(cudaMemcpyAsync(ho.valid, dev.valid, nb, cudaMemcpyDeviceToHost, st));
        // the next use of this slot's buffers (two chunks later) is ordered on this stream
        prev = s;
    }
    cudaError_t e0 = cudaStreamSynchronize(p->hstream[0]);
    cudaError_t e1 = cudaStreamSynchronize(p->hstream[1]);
    for (int i = 0; i < 2; ++i) cudaEventDestroy(done_compute[i]);
    if (rc != EBSD_OK) return rc;
    if (e0 != cudaSuccess || e1 != cudaSuccess) return EBSD_E_LAUNCH;
    return EBSD_OK;
}

int ebsd_plan_set_patterns_per_pass(ebsd_plan_t p, int ppp) {
    if (!p || !(ppp == 0 || ppp == 1 || ppp == 2 || ppp == 4 || ppp == 8)) return EBSD_E_ARG;
    std::lock_guard<std::mutex> lk(p->mtx);
    p->fused_ppp = ppp == 0 ? -1 : ppp;
    return EBSD_OK;
}

int ebsd_plan_autotune(ebsd_plan_t p, int method, int dtype, const void* d_pats, int64_t n,
                       void* stream, int* patterns_per_pass) {
    if (!p || n <= 0 || !d_pats) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    if (!is_fused(method)) {
        if (patterns_per_pass) *patterns_per_pass = 1;
        return EBSD_OK;
    }
    rc = reserve(p, method, n);
    if (rc != EBSD_OK) return rc;
    p->fused_ppp = -1;
    const int maxp = fused_patterns_per_pass(p, method, dtype, n);
    if (maxp == 1) {  // one variant only
        if (patterns_per_pass) *patterns_per_pass = 1;
        return EBSD_OK;
    }
    // time the variants (they give identical records) on the caller's sample
    const size_t nb = (size_t)n * p->nB;
    char* buf = nullptr;
    EBSD_CUDA_TRY(cudaMalloc((void**)&buf, nb * (10 * sizeof(float) + 1) + 256));
    ebsd_bands dev;
    dev.max = (float*)buf;
    dev.normmax = dev.max + nb;
    dev.maxloc = dev.normmax + nb;
    dev.avemax = dev.maxloc + 2 * nb;
    dev.aveloc = dev.avemax + nb;
    dev.width = dev.aveloc + 2 * nb;
    dev.theta = dev.width + nb;
    dev.rho = dev.theta + nb;
    dev.valid = (int8_t*)(dev.rho + nb);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    float best_ms = 0.0f;
    int best = maxp;
    int64_t launches = 0;
    for (int i = 0; i < 2 && rc == EBSD_OK; ++i)
        if (cudaEventCreate(&ev[i]) != cudaSuccess) rc = EBSD_E_LAUNCH;
    for (int ppp = maxp; ppp >= 1 && rc == EBSD_OK; ppp /= 2) {
        p->fused_ppp = ppp;
        float ms_min = 0.0f;
        for (int rep = 0; rep < 3 && rc == EBSD_OK; ++rep) {  // first pass warms up
            if (cudaEventRecord(ev[0], st) != cudaSuccess) { rc = EBSD_E_LAUNCH; break; }
            rc = fused_run_chunk(p, method, dtype, d_pats, n, &dev, 0, st, &launches);
            if (rc != EBSD_OK) break;
            if (cudaEventRecord(ev[1], st) != cudaSuccess || cudaEventSynchronize(ev[1]) != cudaSuccess) {
                rc = EBSD_E_LAUNCH;
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (rep > 0 && (rep == 1 || ms < ms_min)) ms_min = ms;
        }
        if (rc == EBSD_OK && (ppp == maxp || ms_min < best_ms)) {
            best_ms = ms_min;
            best = ppp;
        }
    }
    for (int i = 0; i < 2; ++i)
        if (ev[i]) cudaEventDestroy(ev[i]);
    cudaFree(buf);
    p->fused_ppp = rc == EBSD_OK ? best : -1;
    if (rc == EBSD_OK && patterns_per_pass) *patterns_per_pass = best;
    return rc;
}

}  // extern "C"
