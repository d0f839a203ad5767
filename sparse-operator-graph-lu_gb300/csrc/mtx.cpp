// MatrixMarket I/O with the reference reader's acceptance rules
// (mtx.cpp:44-117 coordinate reader, mtx.cpp:145-181 array reader).
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

bool read_mtx(const std::string& path, MtxData& out, std::string& err) {
    std::string buf;
    if (!slurp(path, buf)) { err = "can not open file " + path; return false; }
    out = MtxData();
    size_t pos = 0, eol = buf.find('\n');
    std::string first = buf.substr(0, eol);
    if (first.find("symmetric") != std::string::npos) out.symmetric = true;
    int rows = -1;
    char line[1024];
    while (pos < buf.size()) {
        eol = buf.find('\n', pos);
        if (eol == std::string::npos) eol = buf.size();
        size_t len = eol - pos;
        if (len > 0 && buf[pos + len - 1] == '\r') len--;
        const char* s = buf.data() + pos;
        pos = eol + 1;
        if (len <= 3) continue;
        if (memchr(s, '%', len)) continue;
        if (rows < 0) {  // size line: rows cols count
            if (len >= sizeof(line)) continue;
            memcpy(line, s, len); line[len] = 0;
            char *ps, *pe;
            rows = (int)strtol(line, &ps, 10);
            int cols = (int)strtol(ps, &pe, 10);
            long cnt = strtol(pe, NULL, 10);
            if (rows != cols && rows > cols) rows = cols;
            if (rows <= 0) { err = "bad size line"; return false; }
            out.n = rows;
            if (cnt > 0) { out.I.reserve(cnt); out.J.reserve(cnt); out.V.reserve(cnt); }
            continue;
        }
        if (len >= 1000) continue;
        memcpy(line, s, len); line[len] = 0;
        char *ps, *pe;
        long r = strtol(line, &ps, 10);
        long c = strtol(ps, &pe, 10);
        double v = strtod(pe, NULL);
        if (v == 0) continue;
        if (r > rows || c > rows) continue;
        if (r < 1 || c < 1) { err = "index below 1 in " + path; return false; }
        out.I.push_back((int32_t)(r - 1));
        out.J.push_back((int32_t)(c - 1));
        out.V.push_back(v);
    }
    if (rows < 0) { err = "no size line"; return false; }
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
