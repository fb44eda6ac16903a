// EDAX UP1 / UP2 pattern files (ebsd_pattern.UPFile, ebsd_pattern.py:435-570): header parsing
// and multi-threaded reads into caller buffers (pinned host memory for the streaming path,
// ebsd_find_bands_file in plan.cu).
//
// Layout (read_header, ebsd_pattern.py:449-513; write_header, :573-620): a uint32 version; for
// version 1 three uint32 (pattern width, height, byte offset of the first pattern) and the
// pattern count implied by the file size (size - 16) / (width * height * bytes); for version
// >= 3 the same three uint32, a uint8 count of extra patterns, uint32 columns and rows, a
// uint8 hex-grid flag and two float64 steps (x, y), packed.  Patterns follow at the offset,
// row-major, uint8 for .up1, uint16 for .up2.
#include "ebsd_internal.cuh"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstring>
#include <fcntl.h>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <unistd.h>

namespace ebsd {

namespace {

bool read_exact(int fd, void* dst, size_t bytes, int64_t offset) {
    char* p = (char*)dst;
    while (bytes > 0) {
        const ssize_t r = pread(fd, p, bytes, (off_t)offset);
        if (r < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        if (r == 0) return false;  // past the end of the file
        p += r;
        bytes -= (size_t)r;
        offset += r;
    }
    return true;
}

template <class T>
T le_get(const unsigned char* b) {
    T v;
    std::memcpy(&v, b, sizeof(T));  // the files are little-endian, as both hosts are
    return v;
}

}  // namespace

int up_parse_header(const char* path, int bitdepth, ebsd_up_info* info) {
    if (!path || !info) return EBSD_E_ARG;
    std::memset(info, 0, sizeof(*info));
    const std::string s(path);
    const size_t dot = s.find_last_of('.');
    std::string ext = dot == std::string::npos ? "" : s.substr(dot);
    for (auto& c : ext) c = (char)std::tolower((unsigned char)c);
    if (ext == ".up1") info->bytes_per_px = 1;
    else if (ext == ".up2") info->bytes_per_px = 2;
    else if (bitdepth == 8) info->bytes_per_px = 1;
    else if (bitdepth == 16) info->bytes_per_px = 2;
    else return EBSD_E_ARG;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return EBSD_E_IO;
    struct stat st {};
    unsigned char h[42];
    std::memset(h, 0, sizeof(h));
    int rc = EBSD_OK;
    if (fstat(fd, &st) != 0 || !read_exact(fd, h, 16, 0)) rc = EBSD_E_IO;
    if (rc == EBSD_OK) {
        info->version = (int32_t)le_get<uint32_t>(h);
        info->W = (int32_t)le_get<uint32_t>(h + 4);
        info->H = (int32_t)le_get<uint32_t>(h + 8);
        info->file_pos = le_get<uint32_t>(h + 12);
        if (info->W <= 0 || info->H <= 0) rc = EBSD_E_IO;
    }
    if (rc == EBSD_OK && info->version == 1) {
        const double per = (double)info->W * info->H * info->bytes_per_px;
        info->n_patterns = (int64_t)((double)(st.st_size - 16) / per);  // np.int64 of the float quotient
        info->n_cols = info->n_patterns;
        info->n_rows = info->n_cols > 0 ? (int64_t)std::floor((double)info->n_patterns / (double)info->n_cols) : 0;
    } else if (rc == EBSD_OK && info->version >= 3) {
        if (!read_exact(fd, h + 16, 26, 16)) {
            rc = EBSD_E_IO;
        } else {
            info->extra_patterns = h[16];
            info->n_cols = le_get<uint32_t>(h + 17);
            info->n_rows = le_get<uint32_t>(h + 21);
            info->n_patterns = info->n_cols * info->n_rows;
            info->hexflag = h[25];
            info->x_step = le_get<double>(h + 26);
            info->y_step = le_get<double>(h + 34);
        }
    } else if (rc == EBSD_OK) {
        rc = EBSD_E_IO;  // versions 0 and 2 are not described
    }
    info->file_bytes = (int64_t)st.st_size;
    close(fd);
    return rc;
}

int up_read_range(int fd, const ebsd_up_info* info, int64_t start, int64_t n, void* dst, int threads) {
    if (n <= 0) return EBSD_OK;
    const int64_t per = (int64_t)info->W * info->H * info->bytes_per_px;
    const int64_t off = info->file_pos + start * per;
    const int64_t bytes = n * per;
    if (off + bytes > info->file_bytes) return EBSD_E_IO;
    threads = std::max(1, std::min(threads, 64));
    if (bytes < (int64_t)threads << 22) threads = (int)std::max<int64_t>(1, bytes >> 22);  // >= 4 MiB a thread
    if (threads == 1) return read_exact(fd, dst, (size_t)bytes, off) ? EBSD_OK : EBSD_E_IO;
    std::vector<std::thread> pool;
    std::vector<int> ok(threads, 0);
    const int64_t part = ((bytes / threads) + 4095) & ~int64_t(4095);
    for (int t = 0; t < threads; ++t) {
        const int64_t a = std::min<int64_t>(t * part, bytes), b = std::min<int64_t>(a + part, bytes);
        pool.emplace_back([&, t, a, b] { ok[t] = read_exact(fd, (char*)dst + a, (size_t)(b - a), off + a) ? 1 : 0; });
    }
    for (auto& th : pool) th.join();
    for (int t = 0; t < threads; ++t)
        if (!ok[t]) return EBSD_E_IO;
    return EBSD_OK;
}

int default_read_threads() {
    const unsigned hc = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(8u, hc ? hc / 2 : 4u));
}

}  // namespace ebsd

using namespace ebsd;

extern "C" int ebsd_up_read_header(const char* path, int bitdepth, ebsd_up_info* info) {
    return up_parse_header(path, bitdepth, info);
}

extern "C" int ebsd_up_read(const char* path, const ebsd_up_info* info, int64_t pat_start, int64_t n, void* h_dst,
                            int threads) {
    if (!path || !info || pat_start < 0 || n < 0 || (n > 0 && !h_dst)) return EBSD_E_ARG;
    if (pat_start + n > info->n_patterns) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return EBSD_E_IO;
    const int rc = up_read_range(fd, info, pat_start, n, h_dst, threads > 0 ? threads : default_read_threads());
    close(fd);
    return rc;
}
