// Pattern files: EDAX UP1 / UP2 (ebsd_pattern.UPFile, ebsd_pattern.py:435-570), Oxford .ebsp
// (EBSPFile, :709-1088) and ThermoFisher .pat (TFPatFile, :1090-1395): header parsing and
// multi-threaded reads into caller buffers (pinned host memory for the streaming path,
// ebsd_find_bands_file in plan.cu).
//
// Layout (read_header, ebsd_pattern.py:449-513; write_header, :573-620): a uint32 version; for
// version 1 three uint32 (pattern width, height, byte offset of the first pattern) and the
// pattern count implied by the file size (size - 16) / (width * height * bytes); for version
// >= 3 the same three uint32, a uint8 count of extra patterns, uint32 columns and rows, a
// uint8 hex-grid flag and two float64 steps (x, y), packed.  Patterns follow at the offset,
// row-major, uint8 for .up1, uint16 for .up2.
//
// Oxford .ebsp (EBSPFile, ebsd_pattern.py:709-1088): an int64 holding minus the version, from
// version 4 one more byte, then a table of uint64 record positions (0: not stored).  A record
// is a header of 4 uint32 (6 from version 5: ..., height, width, pixel bytes; the first word 1
// marks compressed pixels), the pixels, and from version 2 a flag byte that, when set, is
// followed by x (float64), a flag byte and y; version 1 records end in x, y without flags.
// ThermoFisher .pat (TFPatFile, :1090-1395): uint32 version, columns, rows, width, height, an
// int16 scan flag, a uint8 bit depth and an int16 background flag (25 bytes); when the flag is
// negative a uint16 background pattern follows; then one record per pattern: two uint32 pixel
// locations and the uint16 pixels.
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

// ---- Oxford EBSP / ThermoFisher TFPAT ----------------------------------------------------

namespace {

std::string lower_ext(const char* path) {
    const std::string s(path);
    const size_t dot = s.find_last_of('.');
    const size_t slash = s.find_last_of('/');
    std::string ext = (dot == std::string::npos || (slash != std::string::npos && dot < slash)) ? "" : s.substr(dot);
    for (auto& c : ext) c = (char)std::tolower((unsigned char)c);
    return ext;
}

// The uint64 entries from an EBSP file's table start, read forward in blocks of 512 KB so that
// a corrupt first position cannot make the header parse hold the whole file.
struct TableCursor {
    static constexpr int64_t kBlock = 1 << 16;
    int fd;
    int64_t table;  // byte of entry 0
    int64_t avail;  // entries the file holds from there
    std::vector<uint64_t> buf;
    int64_t base = -1;

    bool get(int64_t k, uint64_t* v) {
        if (k < 0 || k >= avail) return false;
        if (base < 0 || k < base || k >= base + (int64_t)buf.size()) {
            const int64_t n = std::min<int64_t>(kBlock, avail - k);
            buf.resize((size_t)n);
            if (!read_exact(fd, buf.data(), (size_t)n * 8, table + 8 * k)) return false;
            base = k;
        }
        *v = buf[(size_t)(k - base)];
        return true;
    }
};

// EBSPFile.read_header, ebsd_pattern.py:724-858: the version, the record-position table (its
// length: version <= 4, the entries in front of the lowest stored position; version 5, the
// first entry that equals height + (width << 32)), the first record's header, the footer flag.
int ebsp_header(int fd, ebsd_pf_info* I) {
    const int64_t fsz = I->file_bytes;
    unsigned char b[8];
    if (!read_exact(fd, b, 8, 0)) return EBSD_E_IO;
    const uint64_t raw = le_get<uint64_t>(b);
    const int64_t v = (int64_t)(0 - raw);  // the file stores minus the version
    if (v <= 0) return EBSD_E_FORMAT;  // version 0: the reference reads no header either
    if (v > (1 << 20)) return EBSD_E_IO;
    I->version = (int32_t)v;
    const int pph = v >= 5 ? 6 : 4;  // uint32 words of a record header
    const int64_t table = v >= 4 ? 9 : 8;
    I->record_head = 4 * pph;
    I->first_record = table;
    TableCursor tab{fd, table, std::max<int64_t>(0, (fsz - table) / 8)};
    // the first stored position (leading entries may be 0)
    uint64_t loc0 = 0;
    for (int64_t k = 0; loc0 == 0; ++k)
        if (!tab.get(k, &loc0)) return EBSD_E_IO;
    // the reference holds the entries from the table start up to loc0 / 8 of them
    const double want = (double)(int64_t)loc0 / 8.0 + 0.001;
    const int64_t nread = std::min<int64_t>(want > 0 ? (int64_t)want : 0, tab.avail);
    tab.avail = nread;
    uint64_t first = 0;
    if (!tab.get(0, &first)) return EBSD_E_IO;
    int64_t npat = 0;
    if (v <= 4) {
        int64_t loc1 = (int64_t)((double)((int64_t)loc0 - table) / 8.0 + 0.001);
        int64_t counter = 0;
        while (loc1 != counter) {
            uint64_t e;
            if (!tab.get(counter, &e)) return EBSD_E_IO;  // the reference indexes past its array
            if (e != 0 && e >= (uint64_t)table) loc1 = std::min(loc1, (int64_t)((double)(e - (uint64_t)table) / 8.0));
            ++counter;
        }
        npat = counter;
    } else {
        uint32_t w[6];
        if (!read_exact(fd, w, sizeof(w), (int64_t)first)) return EBSD_E_IO;
        if (w[0] == 1) return EBSD_E_FORMAT;  // compressed patterns
        const uint64_t magic = (uint64_t)w[3] + ((uint64_t)w[4] << 32);
        npat = -1;
        uint64_t e;
        for (int64_t k = 0; npat < 0 && tab.get(k, &e); ++k)
            if (e == magic) npat = k;
        if (npat < 0) return EBSD_E_IO;
    }
    if (npat <= 0) return EBSD_E_IO;
    I->n_patterns = npat;
    // the first record's header: compressed flag, height, width, pixel bytes
    uint32_t w[6];
    if (!read_exact(fd, w, 4 * (size_t)pph, (int64_t)first)) return EBSD_E_IO;
    if (w[0] == 1) return EBSD_E_FORMAT;
    I->W = (int32_t)w[pph - 2];
    I->H = (int32_t)w[pph - 3];
    const uint32_t nbytes = w[pph - 1];
    if (I->W <= 0 || I->H <= 0) return EBSD_E_IO;
    const double bits = (double)nbytes / (double)((uint32_t)I->W * (uint32_t)I->H) * 8.0;
    if (bits == 8.0) I->bytes_per_px = 1;
    else if (bits == 16.0) I->bytes_per_px = 2;
    else if (bits == 32.0) I->bytes_per_px = 4;
    else return EBSD_E_IO;
    // positions in the footers: always in version 1; later versions flag them per record (the
    // lowest stored record decides)
    if (v == 1) {
        I->has_xy = 1;
        I->xy_flag_bytes = 0;
    } else {
        uint64_t lo = 0, e;
        for (int64_t k = 0; k < npat; ++k) {
            if (!tab.get(k, &e)) return EBSD_E_IO;
            if (e > 0 && (lo == 0 || e < lo)) lo = e;
        }
        if (lo == 0) return EBSD_E_IO;
        unsigned char flag = 0;
        if (read_exact(fd, &flag, 1, (int64_t)lo + 4 * pph + nbytes) && flag > 0) {
            I->has_xy = 1;
            I->xy_flag_bytes = 1;
        }
    }
    return EBSD_OK;
}

// TFPatFile.read_header, ebsd_pattern.py:1113-1167.
int tfpat_header(int fd, ebsd_pf_info* I) {
    unsigned char h[25];
    if (!read_exact(fd, h, 4, 0)) return EBSD_E_IO;
    const uint32_t version = le_get<uint32_t>(h);
    if (version == 0) return EBSD_E_FORMAT;  // no header fields in version 0
    if (!read_exact(fd, h + 4, 21, 4)) return EBSD_E_IO;
    I->version = (int32_t)std::min<uint32_t>(version, 0x7fffffffu);
    const uint32_t ncols = le_get<uint32_t>(h + 4), nrows = le_get<uint32_t>(h + 8);
    const uint32_t W = le_get<uint32_t>(h + 12), H = le_get<uint32_t>(h + 16);
    if (W == 0 || H == 0 || W > 0x7fffffffu || H > 0x7fffffffu) return EBSD_E_IO;
    I->n_cols = ncols;
    I->n_rows = nrows;
    I->W = (int32_t)W;
    I->H = (int32_t)H;
    I->is_scan = le_get<int16_t>(h + 20);
    I->bitdepth = h[22];
    const int16_t back = le_get<int16_t>(h + 23);
    I->has_background = back < 0;
    I->bytes_per_px = 2;  // uint16 pixels whatever the bit depth
    I->record_head = 8;
    // uint32 arithmetic, as numpy does it on the header's uint32 fields
    const uint32_t pat_bytes = W * H * 2u;
    I->first_record = back < 0 ? (int64_t)(uint32_t)(25u + pat_bytes) : 25;
    I->record_bytes = (int64_t)(uint32_t)(pat_bytes + 8u);
    if (I->is_scan < 0) I->n_patterns = (int64_t)ncols * (int64_t)nrows;
    else I->n_patterns = std::max<int64_t>(0, (I->file_bytes - I->first_record) / I->record_bytes);
    return EBSD_OK;
}

bool pf_record(const ebsd_pf_info& I, const uint64_t* pos, int64_t i, int64_t* at) {
    if (I.format == EBSD_PF_EBSP) {
        if (pos[i] == 0) return false;
        *at = (int64_t)pos[i];
        return true;
    }
    *at = I.first_record + i * I.record_bytes;
    return true;
}

// Bytes of a record the read needs, relative to its position: [lo, hi).
struct RecordWindow {
    int64_t lo, hi;
    int64_t px;             // pixel offset
    int64_t pb;             // pixel bytes
    int64_t aux_at = -1;    // EBSP x (y follows after 8 + flag bytes); TFPAT the locations
    int64_t flag = 0;
    int64_t aux_bytes = 0;  // bytes of aux per pattern
};

RecordWindow record_window(const ebsd_pf_info& I, bool pixels, bool aux) {
    RecordWindow w{};
    w.px = I.record_head;
    w.pb = (int64_t)I.W * I.H * I.bytes_per_px;
    int64_t alo = 0, ahi = 0;
    if (I.format == EBSD_PF_EBSP) {
        w.aux_bytes = 16;
        if (aux && I.has_xy) {
            w.flag = I.xy_flag_bytes;
            w.aux_at = w.px + w.pb + w.flag;
            alo = w.px + w.pb;
            ahi = w.aux_at + 8 + w.flag + 8;
        }
    } else {
        w.aux_bytes = 8;
        if (aux) {
            w.aux_at = 0;
            alo = 0;
            ahi = 8;
        }
    }
    const bool has_aux = w.aux_at >= 0;
    if (pixels && has_aux) {
        w.lo = std::min(w.px, alo);
        w.hi = std::max(w.px + w.pb, ahi);
    } else if (pixels) {
        w.lo = w.px;
        w.hi = w.px + w.pb;
    } else {
        w.lo = alo;
        w.hi = ahi;
    }
    return w;
}

void unpack_record(const RecordWindow& w, const char* rec, int64_t k, char* dst, char* aux, int format) {
    // rec points at the record's byte w.lo
    if (dst) std::memcpy(dst + k * w.pb, rec + (w.px - w.lo), (size_t)w.pb);
    if (aux) {
        char* a = aux + k * w.aux_bytes;
        if (w.aux_at < 0) {
            std::memset(a, 0, (size_t)w.aux_bytes);
        } else if (format == EBSD_PF_EBSP) {
            std::memcpy(a, rec + (w.aux_at - w.lo), 8);
            std::memcpy(a + 8, rec + (w.aux_at + 8 + w.flag - w.lo), 8);
        } else {
            std::memcpy(a, rec + (w.aux_at - w.lo), 8);
        }
    }
}

// Patterns [i0, i1) of the read [start, ...): runs of records at one spacing go through a
// bounce buffer in reads of up to kBounce bytes.
int pf_read_part(int fd, const ebsd_pf_info& I, const uint64_t* pos, const RecordWindow& w, int64_t start,
                 int64_t i0, int64_t i1, char* dst, char* aux) {
    constexpr int64_t kBounce = 8 << 20;
    const int64_t one = w.hi - w.lo;
    std::vector<char> buf;
    int64_t i = i0;
    while (i < i1) {
        int64_t a;
        const int64_t k = i - start;
        if (!pf_record(I, pos, i, &a)) {  // not stored: zeros
            if (dst) std::memset(dst + k * w.pb, 0, (size_t)w.pb);
            if (aux) std::memset(aux + k * w.aux_bytes, 0, (size_t)w.aux_bytes);
            ++i;
            continue;
        }
        int64_t j = i + 1, step = 0, b;
        if (dst && j < i1 && pf_record(I, pos, j, &b) && b - a >= one) {
            step = b - a;
            const int64_t maxrun = std::max<int64_t>(1, (kBounce - one) / step + 1);
            ++j;
            int64_t c;
            while (j < i1 && j - i < maxrun && pf_record(I, pos, j, &c) && c == a + (j - i) * step) ++j;
        }
        const int64_t cnt = j - i;
        const int64_t span = (cnt - 1) * step + one;
        if ((size_t)span > buf.size()) buf.resize((size_t)span);
        if (!read_exact(fd, buf.data(), (size_t)span, a + w.lo)) return EBSD_E_IO;
        for (int64_t r = 0; r < cnt; ++r)
            unpack_record(w, buf.data() + r * step, k + r, dst, aux, I.format);
        i = j;
    }
    return EBSD_OK;
}

}  // namespace

bool pf_path(const char* path) {
    if (!path) return false;
    const std::string ext = lower_ext(path);
    return ext == ".ebsp" || ext == ".pat";
}

int pf_parse_header(const char* path, ebsd_pf_info* info) {
    if (!path || !info) return EBSD_E_ARG;
    std::memset(info, 0, sizeof(*info));
    const std::string ext = lower_ext(path);
    if (ext == ".ebsp") info->format = EBSD_PF_EBSP;
    else if (ext == ".pat") info->format = EBSD_PF_TFPAT;
    else return EBSD_E_ARG;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return EBSD_E_IO;
    struct stat st {};
    int rc = fstat(fd, &st) == 0 ? EBSD_OK : EBSD_E_IO;
    info->file_bytes = (int64_t)st.st_size;
    if (rc == EBSD_OK) rc = info->format == EBSD_PF_EBSP ? ebsp_header(fd, info) : tfpat_header(fd, info);
    close(fd);
    return rc;
}

int pf_read_positions(int fd, const ebsd_pf_info* info, uint64_t* pos) {
    if (info->format != EBSD_PF_EBSP) return EBSD_E_ARG;
    if (info->n_patterns <= 0) return EBSD_OK;
    return read_exact(fd, pos, (size_t)info->n_patterns * 8, info->first_record) ? EBSD_OK : EBSD_E_IO;
}

int pf_read_range(int fd, const ebsd_pf_info* info, const uint64_t* pos, int64_t start, int64_t n, void* dst,
                  void* aux, int threads) {
    if (n <= 0) return EBSD_OK;
    if (info->format == EBSD_PF_EBSP && !pos) return EBSD_E_ARG;
    const RecordWindow w = record_window(*info, dst != nullptr, aux != nullptr);
    if (w.hi <= w.lo) {  // nothing to read: aux of a file without footers
        if (aux) std::memset(aux, 0, (size_t)(n * w.aux_bytes));
        return EBSD_OK;
    }
    // about 4 MiB of records per thread at least
    const int64_t per = std::max<int64_t>(1, w.hi - w.lo);
    threads = std::max(1, std::min(threads, 64));
    threads = (int)std::max<int64_t>(1, std::min<int64_t>(threads, (n * per) >> 22));
    threads = (int)std::min<int64_t>(threads, n);
    char* d = (char*)dst;
    char* a = (char*)aux;
    if (threads == 1) return pf_read_part(fd, *info, pos, w, start, start, start + n, d, a);
    std::vector<std::thread> pool;
    std::vector<int> rc(threads, EBSD_OK);
    const int64_t part = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const int64_t i0 = start + std::min<int64_t>(n, t * part), i1 = start + std::min<int64_t>(n, (t + 1) * part);
        pool.emplace_back([&, t, i0, i1] { rc[t] = pf_read_part(fd, *info, pos, w, start, i0, i1, d, a); });
    }
    for (auto& th : pool) th.join();
    for (int t = 0; t < threads; ++t)
        if (rc[t] != EBSD_OK) return rc[t];
    return EBSD_OK;
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

extern "C" int ebsd_pf_read_header(const char* path, ebsd_pf_info* info) { return pf_parse_header(path, info); }

extern "C" int ebsd_pf_read_positions(const char* path, const ebsd_pf_info* info, uint64_t* h_pos) {
    if (!path || !info || (info->n_patterns > 0 && !h_pos)) return EBSD_E_ARG;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return EBSD_E_IO;
    const int rc = pf_read_positions(fd, info, h_pos);
    close(fd);
    return rc;
}

extern "C" int ebsd_pf_read(const char* path, const ebsd_pf_info* info, const uint64_t* h_pos, int64_t pat_start,
                            int64_t n, void* h_dst, void* h_aux, int threads) {
    if (!path || !info || pat_start < 0 || n < 0) return EBSD_E_ARG;
    if (info->format != EBSD_PF_EBSP && info->format != EBSD_PF_TFPAT) return EBSD_E_ARG;
    if (pat_start + n > info->n_patterns) return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if (!h_dst && !h_aux) return EBSD_E_ARG;
    if (info->format == EBSD_PF_EBSP && !h_pos) return EBSD_E_ARG;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return EBSD_E_IO;
    const int rc = pf_read_range(fd, info, h_pos, pat_start, n, h_dst, h_aux,
                                 threads > 0 ? threads : default_read_threads());
    close(fd);
    return rc;
}
