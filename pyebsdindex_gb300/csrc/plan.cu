// C-ABI entry points: plan lifetime, method dispatch, chunking and the host-buffer pipeline.
#include "ebsd_internal.cuh"

#include <condition_variable>
#include <fcntl.h>
#include <thread>
#include <unistd.h>
#include <utility>

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
    cudaFree(p->d_rdnbits);
    cudaFree(p->d_kernel);
    cudaFree(p->d_kernel64);
    cudaFree(p->d_ksep);
    cudaFree(p->d_theta);
    cudaFree(p->d_rho);
    cudaFree(p->d_bg);
    cudaFree(p->d_bgf);
    fused_release(p);
    slab_release(p);
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
    for (int i = 0; i < 3; ++i) {
        if (p->h_pin[i]) cudaFreeHost(p->h_pin[i]);
        p->h_pin[i] = nullptr;
    }
    p->h_pin_bytes = 0;
    for (int i = 0; i < 2; ++i) {
        if (p->h_outpin[i]) cudaFreeHost(p->h_outpin[i]);
        p->h_outpin[i] = nullptr;
    }
    p->h_outpin_bytes = 0;
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


bool all_outputs(const ebsd_bands* b) {
    return b->max && b->normmax && b->maxloc && b->avemax && b->aveloc && b->width && b->theta && b->rho && b->valid;
}

// Page-locked (pinned or registered) host memory: copies from or to it run asynchronously.
bool is_pinned(const void* ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void parallel_copy(void* dst, const void* src, size_t bytes, int threads) {
    threads = (int)std::max<size_t>(1, std::min<size_t>((size_t)threads, bytes >> 22));  // >= 4 MiB each
    if (threads == 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    std::vector<std::thread> pool;
    const size_t part = ((bytes / threads) + 4095) & ~size_t(4095);
    for (int t = 0; t < threads; ++t) {
        const size_t a = std::min(bytes, t * part), b = std::min(bytes, a + part);
        pool.emplace_back([=] { std::memcpy((char*)dst + a, (const char*)src + a, b - a); });
    }
    for (auto& th : pool) th.join();
}

// Where a host pipeline's patterns come from: a host array, or patterns of a UP file, or of
// an EBSP / TFPAT file (pf, with EBSP's record positions).
struct ChunkSource {
    const char* mem = nullptr;
    bool mem_pinned = false;
    int fd = -1;
    const ebsd_up_info* info = nullptr;
    const ebsd_pf_info* pf = nullptr;
    const uint64_t* pos = nullptr;
    int64_t file_start = 0;
    size_t pat_bytes = 0;
};

// Record output: an array of fixed-size records (one per band) with the nine band fields at
// byte offsets (the reference's BandDetect.dataType, band_detect.py:110-115); every other
// byte of a record is zero, as np.zeros leaves it.
struct RecordSink {
    char* base = nullptr;
    int32_t itemsize = 0;
    int32_t off[9] = {};
};

// Staged SoA fields of `nb` bands -> records [first, first + nb), in parallel.
void pack_records(const RecordSink& rs, int64_t first, const ebsd_bands& st, size_t nb, int threads) {
    auto work = [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            char* r = rs.base + (size_t)(first + (int64_t)i) * rs.itemsize;
            std::memset(r, 0, rs.itemsize);
            std::memcpy(r + rs.off[0], st.max + i, 4);
            std::memcpy(r + rs.off[1], st.normmax + i, 4);
            std::memcpy(r + rs.off[2], st.maxloc + 2 * i, 8);
            std::memcpy(r + rs.off[3], st.avemax + i, 4);
            std::memcpy(r + rs.off[4], st.aveloc + 2 * i, 8);
            std::memcpy(r + rs.off[5], st.width + i, 4);
            std::memcpy(r + rs.off[6], st.theta + i, 4);
            std::memcpy(r + rs.off[7], st.rho + i, 4);
            std::memcpy(r + rs.off[8], st.valid + i, 1);
        }
    };
    threads = (int)std::max<size_t>(1, std::min<size_t>((size_t)threads, nb / 4096));
    if (threads == 1) {
        work(0, nb);
        return;
    }
    std::vector<std::thread> pool;
    const size_t part = (nb + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) pool.emplace_back(work, std::min(nb, t * part), std::min(nb, (t + 1) * part));
    for (auto& th : pool) th.join();
}

bool valid_sink(const RecordSink& rs) {
    const int sizes[9] = {4, 4, 8, 4, 8, 4, 4, 4, 1};
    if (!rs.base || rs.itemsize <= 0) return false;
    for (int f = 0; f < 9; ++f)
        if (rs.off[f] < 0 || rs.off[f] + sizes[f] > rs.itemsize) return false;
    return true;
}

// The device layout of one chunk's band fields (nb = patterns x bands).
ebsd_bands chunk_fields(char* base, size_t nb) {
    ebsd_bands d;
    d.max = (float*)base;
    d.normmax = d.max + nb;
    d.maxloc = d.normmax + nb;
    d.avemax = d.maxloc + 2 * nb;
    d.aveloc = d.avemax + nb;
    d.width = d.aveloc + 2 * nb;
    d.theta = d.width + nb;
    d.rho = d.theta + nb;
    d.valid = (int8_t*)(d.rho + nb);
    return d;
}

// Host-buffer pipeline shared by ebsd_find_bands_host and ebsd_find_bands_file.  Two CUDA
// streams alternate chunks: chunk k + 1's upload overlaps chunk k's detection (the shared
// workspace orders the detections through events).  Pageable or file input goes through three
// pinned slots that a filler thread fills ahead (parallel positional reads, or a parallel
// memcpy); pinned input is uploaded directly.  Records go straight to pinned output arrays, or
// through two pinned staging buffers copied out while the next chunk computes.
int host_pipeline(ebsd_plan_s* p, int method, int dtype, const ChunkSource& src, int64_t n, const ebsd_bands* h_out,
                  int64_t chunk, const RecordSink* sink = nullptr) {
    if (chunk <= 0) chunk = is_plain(method) ? default_chunk(p, method) : 65536;
    if (is_plain(method)) chunk = std::min<int64_t>(chunk, 65535);
    chunk = std::min(chunk, n);
    int rc = reserve(p, method, chunk);
    if (rc != EBSD_OK) return rc;
    const int nB = p->nB;
    const size_t in_bytes = (size_t)chunk * src.pat_bytes;
    const size_t out_bytes = (size_t)chunk * nB * (10 * sizeof(float) + 1) + 256;
    for (int i = 0; i < 2; ++i) {
        if (!p->hstream[i]) EBSD_CUDA_TRY(cudaStreamCreateWithFlags(&p->hstream[i], cudaStreamNonBlocking));
        if (!p->hevent[i]) EBSD_CUDA_TRY(cudaEventCreateWithFlags(&p->hevent[i], cudaEventDisableTiming));
    }
    auto regrow = [](void** bufs, int count, size_t* have, size_t want, bool host) -> int {
        if (want <= *have) return EBSD_OK;
        for (int i = 0; i < count; ++i) {
            if (bufs[i]) host ? cudaFreeHost(bufs[i]) : cudaFree(bufs[i]);
            bufs[i] = nullptr;
        }
        *have = 0;
        for (int i = 0; i < count; ++i) {
            const cudaError_t e = host ? cudaHostAlloc(&bufs[i], want, cudaHostAllocDefault) : cudaMalloc(&bufs[i], want);
            if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? EBSD_E_NOMEM : EBSD_E_LAUNCH;
        }
        *have = want;
        return EBSD_OK;
    };
    const bool ring = !(src.mem && src.mem_pinned);
    // pinned input read in place by the kernels over the CPU-GPU link (no staging copy) when
    // the device uses the host page tables (GB300's NVLink-C2C) or the caller asked for it
    const char* in_place = nullptr;
    if (!ring && p->host_input_mode != 0) {
        int coherent = 0;
        cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, p->device);
        cudaPointerAttributes pa;
        if ((p->host_input_mode == 1 || coherent) && cudaPointerGetAttributes(&pa, src.mem) == cudaSuccess &&
            pa.devicePointer)
            in_place = (const char*)pa.devicePointer;
        cudaGetLastError();
    }
    const bool direct_out = !sink && is_pinned(h_out->max) && is_pinned(h_out->normmax) &&
                            is_pinned(h_out->maxloc) && is_pinned(h_out->avemax) && is_pinned(h_out->aveloc) &&
                            is_pinned(h_out->width) && is_pinned(h_out->theta) && is_pinned(h_out->rho) &&
                            is_pinned(h_out->valid);
    if (!in_place && (rc = regrow(p->h_in_dev, 2, &p->h_in_bytes, in_bytes, false)) != EBSD_OK) return rc;
    if ((rc = regrow(p->h_out_dev, 2, &p->h_out_bytes, out_bytes, false)) != EBSD_OK) return rc;
    if (ring && (rc = regrow(p->h_pin, 3, &p->h_pin_bytes, in_bytes, true)) != EBSD_OK) return rc;
    if (!direct_out && (rc = regrow(p->h_outpin, 2, &p->h_outpin_bytes, out_bytes, true)) != EBSD_OK) return rc;
    const int64_t nchunks = (n + chunk - 1) / chunk;
    const int threads = default_read_threads();

    // filler thread: chunk k into pinned slot k % 3 once the slot is free
    std::mutex m;
    std::condition_variable cv;
    int64_t ready[3] = {-1, -1, -1};
    bool free_slot[3] = {true, true, true};
    int fill_err = EBSD_OK;
    bool stop = false;
    std::thread filler;
    if (ring) {
        filler = std::thread([&] {
            for (int64_t k = 0; k < nchunks; ++k) {
                const int sl = (int)(k % 3);
                {
                    std::unique_lock<std::mutex> g(m);
                    cv.wait(g, [&] { return free_slot[sl] || stop; });
                    if (stop) return;
                    free_slot[sl] = false;
                }
                const int64_t s0 = k * chunk, cnt = std::min(chunk, n - s0);
                int r = EBSD_OK;
                if (src.fd >= 0 && src.pf)
                    r = pf_read_range(src.fd, src.pf, src.pos, src.file_start + s0, cnt, p->h_pin[sl], nullptr,
                                      threads);
                else if (src.fd >= 0)
                    r = up_read_range(src.fd, src.info, src.file_start + s0, cnt, p->h_pin[sl], threads);
                else
                    parallel_copy(p->h_pin[sl], src.mem + (size_t)s0 * src.pat_bytes, (size_t)cnt * src.pat_bytes,
                                  threads);
                {
                    std::lock_guard<std::mutex> g(m);
                    if (r != EBSD_OK) fill_err = r;
                    ready[sl] = k;
                }
                cv.notify_all();
                if (r != EBSD_OK) return;
            }
        });
    }

    cudaEvent_t copied[3], done_compute[2], out_done[2];
    for (int i = 0; i < 3; ++i) cudaEventCreateWithFlags(&copied[i], cudaEventDisableTiming);
    for (int i = 0; i < 2; ++i) cudaEventCreateWithFlags(&done_compute[i], cudaEventDisableTiming);
    for (int i = 0; i < 2; ++i) cudaEventCreateWithFlags(&out_done[i], cudaEventDisableTiming);
    int64_t staged_s[2] = {-1, -1}, staged_n[2] = {0, 0};
    auto flush = [&](int ds) {  // staged records of slot ds -> the caller's arrays
        if (staged_s[ds] < 0) return;
        cudaEventSynchronize(out_done[ds]);
        const size_t nb = (size_t)staged_n[ds] * nB;
        const ebsd_bands st = chunk_fields((char*)p->h_outpin[ds], nb);
        if (sink) {
            pack_records(*sink, staged_s[ds] * nB, st, nb, threads);
            staged_s[ds] = -1;
            return;
        }
        const ebsd_bands ho = offset_bands(*h_out, staged_s[ds], nB);
        std::memcpy(ho.max, st.max, nb * 4);
        std::memcpy(ho.normmax, st.normmax, nb * 4);
        std::memcpy(ho.maxloc, st.maxloc, nb * 8);
        std::memcpy(ho.avemax, st.avemax, nb * 4);
        std::memcpy(ho.aveloc, st.aveloc, nb * 8);
        std::memcpy(ho.width, st.width, nb * 4);
        std::memcpy(ho.theta, st.theta, nb * 4);
        std::memcpy(ho.rho, st.rho, nb * 4);
        std::memcpy(ho.valid, st.valid, nb);
        staged_s[ds] = -1;
    };
    for (int64_t k = 0; k < nchunks && rc == EBSD_OK; ++k) {
        const int sl = (int)(k % 3), ds = (int)(k % 2);
        const int64_t s0 = k * chunk, cnt = std::min(chunk, n - s0);
        cudaStream_t st = p->hstream[ds];
        const void* host_in = src.mem + (size_t)s0 * src.pat_bytes;
        if (ring) {
            std::unique_lock<std::mutex> g(m);
            cv.wait(g, [&] { return ready[sl] == k || fill_err != EBSD_OK; });
            if (fill_err != EBSD_OK) {
                rc = fill_err;
                break;
            }
            host_in = p->h_pin[sl];
        }
        const void* kin = p->h_in_dev[ds];
        if (in_place) {
            kin = in_place + (size_t)s0 * src.pat_bytes;
        } else if (cudaMemcpyAsync(p->h_in_dev[ds], host_in, (size_t)cnt * src.pat_bytes, cudaMemcpyHostToDevice,
                                   st) != cudaSuccess ||
                   cudaEventRecord(copied[sl], st) != cudaSuccess) {
            rc = EBSD_E_LAUNCH;
            break;
        }
        if (k > 0 && cudaStreamWaitEvent(st, done_compute[ds ^ 1], 0) != cudaSuccess) {
            rc = EBSD_E_LAUNCH;
            break;
        }
        const size_t nb = (size_t)cnt * nB;
        const ebsd_bands dev = chunk_fields((char*)p->h_out_dev[ds], nb);
        rc = run_chunk(p, method, dtype, kin, cnt, &dev, 0, st, &p->last_launches);
        if (rc != EBSD_OK) break;
        cudaEventRecord(done_compute[ds], st);
        ebsd_bands dst;
        if (direct_out) {
            dst = offset_bands(*h_out, s0, nB);
        } else {
            flush(ds);  // chunk k - 2's records leave the staging buffer first
            dst = chunk_fields((char*)p->h_outpin[ds], nb);
        }
        const std::pair<void*, const void*> parts[9] = {
            {dst.max, dev.max}, {dst.normmax, dev.normmax}, {dst.maxloc, dev.maxloc}, {dst.avemax, dev.avemax},
            {dst.aveloc, dev.aveloc}, {dst.width, dev.width}, {dst.theta, dev.theta}, {dst.rho, dev.rho},
            {dst.valid, dev.valid}};
        const size_t sizes[9] = {nb * 4, nb * 4, nb * 8, nb * 4, nb * 8, nb * 4, nb * 4, nb * 4, nb};
        for (int f = 0; f < 9 && rc == EBSD_OK; ++f)
            if (cudaMemcpyAsync(parts[f].first, parts[f].second, sizes[f], cudaMemcpyDeviceToHost, st) != cudaSuccess)
                rc = EBSD_E_LAUNCH;
        if (!direct_out) {
            cudaEventRecord(out_done[ds], st);
            staged_s[ds] = s0;
            staged_n[ds] = cnt;
        }
        if (k >= 1) {
            if (ring) {  // chunk k - 1's upload was issued an iteration ago; its slot takes chunk k + 2
                const int ps = (int)((k - 1) % 3);
                cudaEventSynchronize(copied[ps]);
                {
                    std::lock_guard<std::mutex> g(m);
                    free_slot[ps] = true;
                }
                cv.notify_all();
            }
            if (!direct_out) flush(ds ^ 1);  // chunk k - 1, while chunk k computes
        }
    }
    if (ring) {
        {
            std::lock_guard<std::mutex> g(m);
            stop = true;
        }
        cv.notify_all();
        filler.join();
    }
    const cudaError_t e0 = cudaStreamSynchronize(p->hstream[0]);
    const cudaError_t e1 = cudaStreamSynchronize(p->hstream[1]);
    if (rc == EBSD_OK && !direct_out) {
        flush(0);
        flush(1);
    }
    for (int i = 0; i < 3; ++i) cudaEventDestroy(copied[i]);
    for (int i = 0; i < 2; ++i) cudaEventDestroy(done_compute[i]);
    for (int i = 0; i < 2; ++i) cudaEventDestroy(out_done[i]);
    if (rc != EBSD_OK) return rc;
    if (e0 != cudaSuccess || e1 != cudaSuccess) return EBSD_E_LAUNCH;
    return EBSD_OK;
}

// A pattern file opened for a host pipeline: its header (UP, or EBSP / TFPAT by extension),
// EBSP's record positions, the descriptor; closed when it goes out of scope.
struct PatternFile {
    ebsd_up_info up{};
    ebsd_pf_info pf{};
    std::vector<uint64_t> pos;
    const char* path = nullptr;
    ChunkSource src;
    int dtype = EBSD_U8;

    int open_file(const ebsd_plan_s* p, const char* file, int bitdepth, int64_t start, int64_t n) {
        path = file;
        int64_t npat = 0;
        int bpp = 0, W = 0, H = 0;
        if (pf_path(file)) {
            int rc = pf_parse_header(file, &pf);
            if (rc != EBSD_OK) return rc;
            npat = pf.n_patterns, bpp = pf.bytes_per_px, W = pf.W, H = pf.H;
            src.pf = &pf;
        } else {
            int rc = up_parse_header(file, bitdepth, &up);
            if (rc != EBSD_OK) return rc;
            npat = up.n_patterns, bpp = up.bytes_per_px, W = up.W, H = up.H;
            src.info = &up;
        }
        if (H != p->H || W != p->W || start + n > npat) return EBSD_E_ARG;
        if (bpp != 1 && bpp != 2) return EBSD_E_DTYPE;
        dtype = bpp == 1 ? EBSD_U8 : EBSD_U16;
        src.file_start = start;
        src.pat_bytes = (size_t)p->nPx * bpp;
        return EBSD_OK;
    }

    int open_data() {
        src.fd = open(path, O_RDONLY);
        if (src.fd < 0) return EBSD_E_IO;
        if (src.pf && pf.format == EBSD_PF_EBSP) {
            pos.resize((size_t)pf.n_patterns);
            int rc = pf_read_positions(src.fd, &pf, pos.data());
            if (rc != EBSD_OK) return rc;
            src.pos = pos.data();
        }
        return EBSD_OK;
    }

    ~PatternFile() {
        if (src.fd >= 0) close(src.fd);
    }
};

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
        case EBSD_E_IO: return "pattern file could not be opened, read or parsed";
        case EBSD_E_FORMAT: return "pattern file format or version not read (compressed or version 0)";
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
    {
        // the Radon mask as bit columns: a peak task reads the mask of its rows with one
        // funnel shift of two words, loaded ahead of its tile loads
        p->rdn_words = (p->nRho + 31) / 32 + 1;
        std::vector<uint32_t> bits((size_t)p->nTheta * p->rdn_words, 0u);
        for (int i = 0; i < p->nRho; ++i)
            for (int j = 0; j < p->nTheta; ++j)
                if (d->rdnmask[(size_t)i * p->nTheta + j]) bits[(size_t)j * p->rdn_words + (i >> 5)] |= 1u << (i & 31);
        if (rc == EBSD_OK) rc = upload(&p->d_rdnbits, bits.data(), bits.size());
    }
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
    if (rc == EBSD_OK) rc = slab_prepare(p, d);
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

int ebsd_method_supported_for(ebsd_plan_t p, int method, int dtype) {
    if (!p) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    if (is_plain(method)) return 1;
    if (!is_fused(method)) return EBSD_E_ARG;
    if (!fused_supported(p, method)) return 0;
    if (slab_serves(p, method, dtype)) return 1;
    if ((method == EBSD_FUSED_F32 && !p->fg.ok_f32) || !p->fg.ok) return 0;
    return 1;
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

int ebsd_find_bands_mixed(const ebsd_plan_t* plans, int nplans, int dtype, const void* const* d_pats,
                          const int64_t* n, const ebsd_bands* d_out, void* stream) {
    if (!plans || !d_pats || !n || !d_out || nplans < 1 || nplans > kMaxMixedPlans) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    for (int k = 0; k < nplans; ++k) {
        const ebsd_plan_s* p = plans[k];
        if (!p || n[k] < 0 || (n[k] > 0 && !d_pats[k]) || !all_outputs(&d_out[k])) return EBSD_E_ARG;
        if (p->device != plans[0]->device || p->k0 != plans[0]->k0 || p->k1 != plans[0]->k1) return EBSD_E_ARG;
        if (!slab_mixable(p, dtype)) return EBSD_E_UNSUPPORTED;
    }
    // one plan's lock at a time would let two mixed calls interleave; lock in address order
    std::vector<ebsd_plan_s*> order(plans, plans + nplans);
    std::sort(order.begin(), order.end());
    order.erase(std::unique(order.begin(), order.end()), order.end());
    std::vector<std::unique_lock<std::mutex>> locks;
    for (ebsd_plan_s* p : order) locks.emplace_back(p->mtx);
    if (cudaSetDevice(plans[0]->device) != cudaSuccess) return EBSD_E_DEVICE;
    std::vector<ebsd_plan_s*> ps(plans, plans + nplans);
    int64_t launches = 0;
    const int rc = slab_run_mixed(ps.data(), nplans, dtype, d_pats, n, d_out, (cudaStream_t)stream, &launches);
    for (ebsd_plan_s* p : order) p->last_launches = launches;
    return rc;
}

int ebsd_find_bands_host(ebsd_plan_t p, int method, int dtype, const void* h_pats, int64_t n,
                         const ebsd_bands* h_out, int64_t chunk) {
    if (!p || !h_out || n < 0) return EBSD_E_ARG;
    if (n > 0 && !h_pats) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    if (!all_outputs(h_out)) return EBSD_E_ARG;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    ChunkSource src;
    src.mem = (const char*)h_pats;
    src.mem_pinned = is_pinned(h_pats);
    src.pat_bytes = (size_t)p->nPx * elem_size(dtype);
    return host_pipeline(p, method, dtype, src, n, h_out, chunk);
}

int ebsd_find_bands_file(ebsd_plan_t p, int method, const char* path, int bitdepth, int64_t pat_start, int64_t n,
                         const ebsd_bands* h_out, int64_t chunk) {
    if (!p || !path || !h_out || n < 0 || pat_start < 0) return EBSD_E_ARG;
    if (!all_outputs(h_out)) return EBSD_E_ARG;
    PatternFile pf;
    int rc = pf.open_file(p, path, bitdepth, pat_start, n);
    if (rc != EBSD_OK) return rc;
    rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    if ((rc = pf.open_data()) != EBSD_OK) return rc;
    return host_pipeline(p, method, pf.dtype, pf.src, n, h_out, chunk);
}

int ebsd_find_bands_host_records(ebsd_plan_t p, int method, int dtype, const void* h_pats, int64_t n,
                                 void* h_records, int32_t itemsize, const int32_t* field_offsets, int64_t chunk) {
    if (!p || n < 0 || !field_offsets) return EBSD_E_ARG;
    if (n > 0 && (!h_pats || !h_records)) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    RecordSink rs;
    rs.base = (char*)h_records;
    rs.itemsize = itemsize;
    for (int f = 0; f < 9; ++f) rs.off[f] = field_offsets[f];
    if (n > 0 && !valid_sink(rs)) return EBSD_E_ARG;
    int rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    ChunkSource src;
    src.mem = (const char*)h_pats;
    src.mem_pinned = is_pinned(h_pats);
    src.pat_bytes = (size_t)p->nPx * elem_size(dtype);
    const ebsd_bands none{};
    return host_pipeline(p, method, dtype, src, n, &none, chunk, &rs);
}

int ebsd_find_bands_file_records(ebsd_plan_t p, int method, const char* path, int bitdepth, int64_t pat_start,
                                 int64_t n, void* h_records, int32_t itemsize, const int32_t* field_offsets,
                                 int64_t chunk) {
    if (!p || !path || n < 0 || pat_start < 0 || !field_offsets) return EBSD_E_ARG;
    if (n > 0 && !h_records) return EBSD_E_ARG;
    RecordSink rs;
    rs.base = (char*)h_records;
    rs.itemsize = itemsize;
    for (int f = 0; f < 9; ++f) rs.off[f] = field_offsets[f];
    if (n > 0 && !valid_sink(rs)) return EBSD_E_ARG;
    PatternFile pf;
    int rc = pf.open_file(p, path, bitdepth, pat_start, n);
    if (rc != EBSD_OK) return rc;
    rc = check_method(p, method);
    if (rc != EBSD_OK) return rc;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
    p->last_launches = 0;
    if (n == 0) return EBSD_OK;
    if ((rc = pf.open_data()) != EBSD_OK) return rc;
    const ebsd_bands none{};
    return host_pipeline(p, method, pf.dtype, pf.src, n, &none, chunk, &rs);
}

int ebsd_plan_set_host_input(ebsd_plan_t p, int mode) {
    if (!p || mode < -1 || mode > 1) return EBSD_E_ARG;
    std::lock_guard<std::mutex> lk(p->mtx);
    p->host_input_mode = mode;
    return EBSD_OK;
}

int ebsd_plan_host_input_in_place(ebsd_plan_t p) {
    if (!p) return EBSD_E_ARG;
    if (p->host_input_mode != -1) return p->host_input_mode;
    int coherent = 0;
    if (cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, p->device) != cudaSuccess)
        return EBSD_E_DEVICE;
    return coherent ? 1 : 0;
}

int ebsd_plan_set_patterns_per_pass(ebsd_plan_t p, int ppp) {
    if (!p || !(ppp == 0 || ppp == 1 || ppp == 2 || ppp == 4 || ppp == 8)) return EBSD_E_ARG;
    std::lock_guard<std::mutex> lk(p->mtx);
    p->fused_ppp = ppp == 0 ? -1 : ppp;
    return EBSD_OK;
}

int ebsd_plan_set_tile(ebsd_plan_t p, int tile, int slabs) {
    if (!p || tile < 0 || tile > 2 || slabs < 0) return EBSD_E_ARG;
    std::lock_guard<std::mutex> lk(p->mtx);
    if (tile == 1 && !p->fg.ok_f32) return EBSD_E_UNSUPPORTED;
    if ((tile == 2 || slabs > 0) && !p->sg.ok) return EBSD_E_UNSUPPORTED;
    if (p->sg.ok) {
        if (cudaSetDevice(p->device) != cudaSuccess) return EBSD_E_DEVICE;
        const int rc = slab_relayout(p, slabs);
        if (rc != EBSD_OK) return rc;
    }
    p->tile_mode = tile;
    return EBSD_OK;
}

int ebsd_plan_get_tile(ebsd_plan_t p, ebsd_tile_info* info) {
    if (!p || !info) return EBSD_E_ARG;
    std::lock_guard<std::mutex> lk(p->mtx);
    ebsd_tile_info t;
    std::memset(&t, 0, sizeof(t));
    t.single_fits = p->fg.ok_f32 ? 1 : 0;
    t.tile = p->fg.ok_f32 ? (p->tile_mode == 2 && p->sg.ok ? 2 : 1) : (p->sg.ok ? 2 : 0);
    t.patterns_per_pass = p->fused_ppp > 0 ? p->fused_ppp : 0;
    t.slabs = p->sg.ok ? p->sg.nslab : 0;
    t.slab_columns = p->sg.ok ? p->sg.Ts : 0;
    t.slabs_min = p->sg.ok ? p->sg.nslab_min : 0;
    t.slabs_max = p->sg.ok ? p->sg.nslab_max : 0;
    t.slabs_fp16 = p->sg.ok && p->sg.ok16 && p->d_swimg ? 1 : 0;
    *info = t;
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
    // the candidates, which give identical records: the single tile with 8, 4, 2 or 1 patterns
    // per block pass, and theta slabs from the widest that fit to three more
    struct Cand {
        int tile, v;  // tile 1: v = patterns per pass; tile 2: v = slab count
    };
    std::vector<Cand> cands;
    const int old_mode = p->tile_mode, old_slabs = p->sg.ok ? p->sg.nslab : 0;
    p->fused_ppp = -1;
    const bool single = method == EBSD_FUSED_F32 ? p->fg.ok_f32 != 0 : p->fg.ok != 0;
    if (single) {
        p->tile_mode = 1;
        const int maxp = fused_patterns_per_pass(p, method, dtype, n);
        for (int ppp = maxp; ppp >= 1; ppp /= 2) cands.push_back(Cand{1, ppp});
    }
    if (method == EBSD_FUSED_F32 && p->sg.ok && (dtype != EBSD_F32 || p->sg.ok_f32))
        for (int ns = p->sg.nslab_min; ns <= std::min(p->sg.nslab_max, p->sg.nslab_min + 3); ++ns)
            cands.push_back(Cand{2, ns});
    auto apply = [&](const Cand& c) -> int {
        if (c.tile == 1) {
            p->tile_mode = 1;
            p->fused_ppp = c.v;
            return EBSD_OK;
        }
        p->tile_mode = 2;
        p->fused_ppp = -1;
        return slab_relayout(p, c.v);
    };
    if (cands.size() <= 1) {  // one variant only
        if (!cands.empty()) rc = apply(cands[0]);
        if (!single || cands.empty()) p->tile_mode = old_mode;
        if (patterns_per_pass) *patterns_per_pass = cands.empty() || cands[0].tile != 1 ? 1 : cands[0].v;
        return rc;
    }
    // time the variants on the caller's sample
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
    size_t best = 0;
    int64_t launches = 0;
    for (int i = 0; i < 2 && rc == EBSD_OK; ++i)
        if (cudaEventCreate(&ev[i]) != cudaSuccess) rc = EBSD_E_LAUNCH;
    for (size_t ci = 0; ci < cands.size() && rc == EBSD_OK; ++ci) {
        rc = apply(cands[ci]);
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
        if (rc == EBSD_OK && (ci == 0 || ms_min < best_ms)) {
            best_ms = ms_min;
            best = ci;
        }
    }
    for (int i = 0; i < 2; ++i)
        if (ev[i]) cudaEventDestroy(ev[i]);
    cudaFree(buf);
    if (rc == EBSD_OK) {
        rc = apply(cands[best]);
        if (rc == EBSD_OK && patterns_per_pass) *patterns_per_pass = cands[best].tile == 1 ? cands[best].v : 1;
    } else {
        // back to the settings before the call
        p->fused_ppp = -1;
        p->tile_mode = old_mode;
        if (old_slabs) slab_relayout(p, old_slabs);
    }
    return rc;
}

}  // extern "C"
