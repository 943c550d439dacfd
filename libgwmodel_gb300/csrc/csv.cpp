// csv.cpp -- bulk CSV input for the C ABI (gwgpu_csv_read / gwgpu_table_*).
//
// The reference's callers load their data with Armadillo's csv_name (a header
// row of column names, quoted or not, then numeric rows: test/data/
// londonhp100.cpp:6-26) and pass it cell by cell through IGWRBasicGpuTask.
// This reader takes the file in one read, splits it at line starts and
// parses the rows on all host threads with std::from_chars (locale-free,
// round-trip exact), into column-major doubles that the bulk setters take
// directly.  An empty or non-numeric cell is an error naming its line.
#include "../../include/gwgpu.h"

#include <algorithm>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace gwgpu {
void set_last_error(const char* msg);
}

struct gwgpu_table {
    std::vector<std::string> names;
    std::vector<double> data;  // rows x cols column-major
    int rows = 0, cols = 0;
};

namespace {

std::string unquote(std::string s)
{
    auto ws = [](char c) { return c == ' ' || c == '\t'; };
    while (!s.empty() && ws(s.back())) s.pop_back();
    size_t b = 0;
    while (b < s.size() && ws(s[b])) b++;
    s = s.substr(b);
    if (s.size() >= 2 && s.front() == '"' && s.back() == '"') s = s.substr(1, s.size() - 2);
    return s;
}

// Splits [p, e) at commas (names only: no commas inside quotes are expected in numeric tables,
// but a quoted name may contain one).
std::vector<std::string> split_header(const char* p, const char* e)
{
    std::vector<std::string> out;
    std::string cur;
    bool quoted = false;
    for (; p < e; p++) {
        if (*p == '"') quoted = !quoted;
        if (*p == ',' && !quoted) {
            out.push_back(unquote(cur));
            cur.clear();
        } else {
            cur.push_back(*p);
        }
    }
    out.push_back(unquote(cur));
    return out;
}

// Parses one numeric row [p, e) into cols cells of row r; returns false with a message.
bool parse_row(const char* p, const char* e, int cols, int r, int rows, double* data, std::string& err)
{
    for (int c = 0; c < cols; c++) {
        while (p < e && (*p == ' ' || *p == '\t')) p++;
        const char* q = p;
        while (q < e && *q != ',') q++;
        const char* te = q;
        while (te > p && (te[-1] == ' ' || te[-1] == '\t')) te--;
        if (te == p) {
            err = "empty cell in column " + std::to_string(c + 1);
            return false;
        }
        const char* sp = p;
        if (*sp == '+') sp++;  // from_chars takes no leading '+'
        double v = 0.0;
        auto res = std::from_chars(sp, te, v);
        if (res.ec != std::errc() || res.ptr != te) {
            err = "not a number in column " + std::to_string(c + 1) + ": '" + std::string(p, te) + "'";
            return false;
        }
        data[(size_t)r + (size_t)c * rows] = v;
        if (c + 1 < cols) {
            if (q == e) {
                err = "expected " + std::to_string(cols) + " cells, found " + std::to_string(c + 1);
                return false;
            }
            p = q + 1;
        } else if (q != e) {
            err = "more than " + std::to_string(cols) + " cells";
            return false;
        }
    }
    return true;
}

int fail(int code, const std::string& msg)
{
    gwgpu::set_last_error(msg.c_str());
    return code;
}

}  // namespace

extern "C" {

int gwgpu_csv_read(const char* path, gwgpu_table** out)
{
    if (!path || !out) return fail(GWGPU_ERR_INVALID, "null argument");
    *out = nullptr;
    try {
        FILE* f = std::fopen(path, "rb");
        if (!f) return fail(GWGPU_ERR_INVALID, std::string("cannot open ") + path);
        std::vector<char> buf;
        std::fseek(f, 0, SEEK_END);
        const long size = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf.resize(size > 0 ? (size_t)size : 0);
        const size_t got = buf.empty() ? 0 : std::fread(buf.data(), 1, buf.size(), f);
        std::fclose(f);
        if (got != buf.size()) return fail(GWGPU_ERR_INVALID, std::string("cannot read ") + path);
        // line extents, without the line ending; blank lines skipped
        std::vector<std::pair<size_t, size_t>> lines;
        std::vector<size_t> lineno;
        size_t s = 0, ln = 0;
        const size_t n = buf.size();
        while (s < n) {
            const char* nl = (const char*)std::memchr(buf.data() + s, '\n', n - s);
            size_t e = nl ? (size_t)(nl - buf.data()) : n;
            ln++;
            size_t ee = e;
            if (ee > s && buf[ee - 1] == '\r') ee--;
            bool blank = true;
            for (size_t k = s; k < ee && blank; k++) blank = buf[k] == ' ' || buf[k] == '\t';
            if (!blank) {
                lines.push_back({s, ee});
                lineno.push_back(ln);
            }
            s = e + 1;
        }
        if (lines.empty()) return fail(GWGPU_ERR_INVALID, std::string(path) + ": no header row");
        std::unique_ptr<gwgpu_table> t(new gwgpu_table());
        t->names = split_header(buf.data() + lines[0].first, buf.data() + lines[0].second);
        t->cols = (int)t->names.size();
        t->rows = (int)(lines.size() - 1);
        t->data.assign((size_t)t->rows * t->cols, 0.0);
        const int rows = t->rows, cols = t->cols;
        const int nthreads = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64u));
        const int chunk = (rows + nthreads - 1) / std::max(nthreads, 1);
        std::vector<std::string> errs(nthreads);
        std::vector<long long> err_line(nthreads, -1);
        std::vector<std::thread> pool;
        for (int w = 0; w < nthreads && w * chunk < rows; w++) {
            pool.emplace_back([&, w] {
                const int r0 = w * chunk, r1 = std::min(rows, r0 + chunk);
                for (int r = r0; r < r1; r++) {
                    const auto& L = lines[(size_t)r + 1];
                    std::string err;
                    if (!parse_row(buf.data() + L.first, buf.data() + L.second, cols, r, rows, t->data.data(), err)) {
                        errs[w] = err;
                        err_line[w] = (long long)lineno[(size_t)r + 1];
                        return;
                    }
                }
            });
        }
        for (auto& th : pool) th.join();
        for (int w = 0; w < nthreads; w++)
            if (err_line[w] >= 0)
                return fail(GWGPU_ERR_INVALID,
                            std::string(path) + ":" + std::to_string(err_line[w]) + ": " + errs[w]);
        *out = t.release();
        return GWGPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(GWGPU_ERR_RUNTIME, "out of host memory");
    } catch (const std::exception& e) {
        return fail(GWGPU_ERR_RUNTIME, e.what());
    }
}

int gwgpu_table_shape(const gwgpu_table* t, int* rows, int* cols)
{
    if (!t) return fail(GWGPU_ERR_INVALID, "null table");
    if (rows) *rows = t->rows;
    if (cols) *cols = t->cols;
    return GWGPU_OK;
}

const char* gwgpu_table_column_name(const gwgpu_table* t, int col)
{
    if (!t || col < 0 || col >= t->cols) return nullptr;
    return t->names[(size_t)col].c_str();
}

int gwgpu_table_columns(const gwgpu_table* t, int ncol, const char* const* names, double* out)
{
    if (!t) return fail(GWGPU_ERR_INVALID, "null table");
    if (ncol < 0 || (ncol && (!names || !out))) return fail(GWGPU_ERR_INVALID, "bad arguments");
    for (int k = 0; k < ncol; k++) {
        if (!names[k]) return fail(GWGPU_ERR_INVALID, "null column name");
        auto it = std::find(t->names.begin(), t->names.end(), std::string(names[k]));
        if (it == t->names.end()) return fail(GWGPU_ERR_INVALID, std::string("no column named ") + names[k]);
        const size_t c = (size_t)(it - t->names.begin());
        std::copy(t->data.begin() + c * t->rows, t->data.begin() + (c + 1) * t->rows, out + (size_t)k * t->rows);
    }
    return GWGPU_OK;
}

void gwgpu_table_destroy(gwgpu_table* t) { delete t; }

}  // extern "C"
