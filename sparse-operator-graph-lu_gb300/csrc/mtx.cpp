// MatrixMarket I/O with the reference reader's acceptance rules
// (mtx.cpp:44-117 coordinate reader, mtx.cpp:145-181 array reader).
#include <omp.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "plan.h"

namespace sog {

namespace {
bool slurp(const std::string& path, std::string& buf) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    buf = ss.str();
    return true;
}
}  // namespace

namespace {

// One coordinate line after the size line, with the reference's rules:
// lines of <= 3 characters or containing '%' are skipped, zero values are
// dropped, entries beyond the size are ignored, indices below 1 are an error.
// Returns 0 = skip, 1 = entry, -1 = error.
int parse_entry(const char* s, size_t len, int rows, int32_t& i, int32_t& j, double& v) {
    if (len <= 3 || memchr(s, '%', len) || len >= 1000) return 0;
    char line[1024];
    memcpy(line, s, len);
    line[len] = 0;
    char *ps, *pe;
    const long r = strtol(line, &ps, 10);
    const long c = strtol(ps, &pe, 10);
    v = strtod(pe, NULL);
    if (v == 0) return 0;
    if (r > rows || c > rows) return 0;
    if (r < 1 || c < 1) return -1;
    i = (int32_t)(r - 1);
    j = (int32_t)(c - 1);
    return 1;
}

}  // namespace

// The size line is found sequentially; the entry lines are parsed in chunks
// split at line ends, in parallel, and concatenated in file order (so a
// repeated entry keeps its position: the last one still wins downstream).
bool read_mtx(const std::string& path, MtxData& out, std::string& err) {
    std::string buf;
    if (!slurp(path, buf)) { err = "can not open file " + path; return false; }
    out = MtxData();
    size_t pos = 0, eol = buf.find('\n');
    std::string first = buf.substr(0, eol);
    if (first.find("symmetric") != std::string::npos) out.symmetric = true;
    int rows = -1;
    long cnt = 0;
    char line[1024];
    while (pos < buf.size() && rows < 0) {
        eol = buf.find('\n', pos);
        if (eol == std::string::npos) eol = buf.size();
        size_t len = eol - pos;
        if (len > 0 && buf[pos + len - 1] == '\r') len--;
        const char* s = buf.data() + pos;
        pos = eol + 1;
        if (len <= 3 || memchr(s, '%', len) || len >= sizeof(line)) continue;
        memcpy(line, s, len);
        line[len] = 0;
        char *ps, *pe;
        rows = (int)strtol(line, &ps, 10);
        const int cols = (int)strtol(ps, &pe, 10);
        cnt = strtol(pe, NULL, 10);
        if (rows != cols && rows > cols) rows = cols;
        if (rows <= 0) { err = "bad size line"; return false; }
        out.n = rows;
    }
    if (rows < 0) { err = "no size line"; return false; }
    const size_t body = std::min(pos, buf.size()), total = buf.size();
    const int nthreads = std::max(1, std::min(omp_get_max_threads(), (int)((total - body) / (1 << 20)) + 1));
    std::vector<size_t> cut(nthreads + 1, total);
    cut[0] = body;
    for (int t = 1; t < nthreads; t++) {
        size_t c = body + (total - body) * t / nthreads;
        const size_t nl = buf.find('\n', c);
        cut[t] = nl == std::string::npos ? total : nl + 1;
        if (cut[t] < cut[t - 1]) cut[t] = cut[t - 1];
    }
    std::vector<MtxData> part(nthreads);
    std::vector<long> bad(nthreads, -1);
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
    for (int t = 0; t < nthreads; t++) {
        MtxData& m = part[t];
        if (nthreads == 1 && cnt > 0) { m.I.reserve(cnt); m.J.reserve(cnt); m.V.reserve(cnt); }
        size_t p = cut[t];
        while (p < cut[t + 1]) {
            size_t e = buf.find('\n', p);
            if (e == std::string::npos || e > cut[t + 1]) e = cut[t + 1];
            size_t len = e - p;
            if (len > 0 && buf[p + len - 1] == '\r') len--;
            int32_t i, j;
            double v;
            const int k = parse_entry(buf.data() + p, len, rows, i, j, v);
            if (k < 0) { bad[t] = (long)p; break; }
            if (k > 0) { m.I.push_back(i); m.J.push_back(j); m.V.push_back(v); }
            p = e + 1;
        }
    }
    for (int t = 0; t < nthreads; t++)
        if (bad[t] >= 0) { err = "index below 1 in " + path; return false; }
    if (nthreads == 1) {
        out.I.swap(part[0].I); out.J.swap(part[0].J); out.V.swap(part[0].V);
    } else {
        size_t nnz = 0;
        for (auto& m : part) nnz += m.I.size();
        out.I.reserve(nnz); out.J.reserve(nnz); out.V.reserve(nnz);
        for (auto& m : part) {
            out.I.insert(out.I.end(), m.I.begin(), m.I.end());
            out.J.insert(out.J.end(), m.J.begin(), m.J.end());
            out.V.insert(out.V.end(), m.V.begin(), m.V.end());
        }
    }
    return true;
}

// Binary cache beside the text file: <path>.sogbin holds the parsed triplets
// and the text file's size and modification time; it is used only while both
// still match.
namespace {
struct CacheHeader {
    char magic[8];
    uint64_t src_size;
    int64_t src_mtime;
    int32_t n, symmetric;
    int64_t nnz;
};
bool src_stamp(const std::string& path, uint64_t& size, int64_t& mtime) {
    struct stat st;
    if (stat(path.c_str(), &st) != 0) return false;
    size = (uint64_t)st.st_size;
    mtime = (int64_t)st.st_mtime;
    return true;
}
}  // namespace

bool read_mtx_cached(const std::string& path, MtxData& out, std::string& err, bool* from_cache) {
    if (from_cache) *from_cache = false;
    uint64_t size = 0;
    int64_t mtime = 0;
    const bool have = src_stamp(path, size, mtime);
    const std::string cpath = path + ".sogbin";
    if (have) {
        FILE* f = fopen(cpath.c_str(), "rb");
        if (f) {
            CacheHeader h;
            bool ok = fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, "SOGMTX1", 8) == 0 && h.src_size == size &&
                      h.src_mtime == mtime && h.nnz >= 0 && h.n > 0;
            if (ok) {
                out = MtxData();
                out.n = h.n;
                out.symmetric = h.symmetric != 0;
                out.I.resize(h.nnz); out.J.resize(h.nnz); out.V.resize(h.nnz);
                ok = fread(out.I.data(), 4, h.nnz, f) == (size_t)h.nnz && fread(out.J.data(), 4, h.nnz, f) == (size_t)h.nnz &&
                     fread(out.V.data(), 8, h.nnz, f) == (size_t)h.nnz;
            }
            fclose(f);
            if (ok) {
                if (from_cache) *from_cache = true;
                return true;
            }
        }
    }
    if (!read_mtx(path, out, err)) return false;
    if (have) {  // best effort: an unwritable directory just means no cache
        const std::string tmp = cpath + ".tmp";
        FILE* f = fopen(tmp.c_str(), "wb");
        if (f) {
            CacheHeader h;
            memset(&h, 0, sizeof(h));
            memcpy(h.magic, "SOGMTX1", 8);
            h.src_size = size;
            h.src_mtime = mtime;
            h.n = out.n;
            h.symmetric = out.symmetric ? 1 : 0;
            h.nnz = (int64_t)out.I.size();
            bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(out.I.data(), 4, out.I.size(), f) == out.I.size() &&
                      fwrite(out.J.data(), 4, out.J.size(), f) == out.J.size() &&
                      fwrite(out.V.data(), 8, out.V.size(), f) == out.V.size();
            ok = (fclose(f) == 0) && ok;
            if (ok) rename(tmp.c_str(), cpath.c_str());
            else remove(tmp.c_str());
        }
    }
    return true;
}

std::vector<double> read_rhs(const std::string& path, int n) {
    std::vector<double> b(n, 1.0);
    std::string buf;
    if (!slurp(path, buf)) return b;
    size_t pos = 0;
    bool header_done = false;
    int count = 0;
    char line[1024];
    while (pos < buf.size() && count < n) {
        size_t eol = buf.find('\n', pos);
        if (eol == std::string::npos) eol = buf.size();
        size_t len = eol - pos;
        const char* s = buf.data() + pos;
        pos = eol + 1;
        if (memchr(s, '%', len)) continue;
        if (!header_done) { header_done = true; continue; }
        if (len >= 1000) continue;
        memcpy(line, s, len); line[len] = 0;
        b[count++] = strtod(line, NULL);
    }
    return b;
}

}  // namespace sog
