// Grid results I/O of libmsl_gb300.so: the `;`-separated text dump of the
// reference's example programs and its reader.
//
// Reference: examples/heatdiffusion.cpp:99-114 (2-D: one line per row, every
// value followed by ';') and :156-170 (3-D: one line per (x, y) column with z
// innermost, index x + cols*y + cols*rows*z). Values are written the way
// `std::ostream << value` writes them by default: %g with 6 significant
// digits for floating point, decimal for integers. Files are appended to, as
// the examples open them with std::ios::app.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "msl_internal.h"

using namespace msl;
using msl::rt::ctx;

namespace {

float bf16_to_f(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
uint16_t f_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// One value as `std::ostream << v` formats it by default.
int format_value(int dtype, const char *p, size_t k, char *buf, size_t cap) {
    switch (dtype) {
        case MSL_F32: {
            float v;
            memcpy(&v, p + 4 * k, 4);
            return snprintf(buf, cap, "%g", (double)v);
        }
        case MSL_F64: {
            double v;
            memcpy(&v, p + 8 * k, 8);
            return snprintf(buf, cap, "%g", v);
        }
        case MSL_I32: {
            int32_t v;
            memcpy(&v, p + 4 * k, 4);
            return snprintf(buf, cap, "%d", (int)v);
        }
        default: {  // MSL_BF16: written as the float it holds
            uint16_t v;
            memcpy(&v, p + 2 * k, 2);
            return snprintf(buf, cap, "%g", (double)bf16_to_f(v));
        }
    }
}

bool dims_ok(int dtype, int depth, int rows, int cols) {
    return rt::dtype_size(dtype) && depth >= 1 && rows >= 1 && cols >= 1 &&
           (long long)depth * rows * cols <= (1LL << 34);
}

// Position in memory of the k-th value in file order.
size_t file_to_memory(size_t k, int depth, int rows, int cols) {
    if (depth == 1) return k;  // rows in order, row-major
    const size_t z = k % depth, xy = k / depth;  // line xy = x * rows + y, z innermost
    const size_t y = xy % rows, x = xy / rows;
    return x + (size_t)cols * y + (size_t)cols * rows * z;
}

}  // namespace

extern "C" {

int msl_grid_dump_text(const char *path, int dtype, const void *grid, int depth, int rows, int cols) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (!path || !grid || !dims_ok(dtype, depth, rows, cols))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_dump_text: bad arguments");
    const size_t n = (size_t)depth * rows * cols, es = rt::dtype_size(dtype);
    std::vector<char> h(n * es);
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_grid_dump_text");
    MSL_TRY_CUDA(cudaMemcpy(h.data(), grid, h.size(), cudaMemcpyDeviceToHost), "msl_grid_dump_text");
    FILE *f = fopen(path, "ab");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_dump_text: cannot open %s", path);
    std::vector<char> line;
    const size_t per_line = depth == 1 ? (size_t)cols : (size_t)depth;
    char buf[64];
    bool ok = true;
    for (size_t k = 0; ok && k < n; k++) {
        const int len = format_value(dtype, h.data(), file_to_memory(k, depth, rows, cols), buf, sizeof buf);
        line.insert(line.end(), buf, buf + len);
        line.push_back(';');
        if ((k + 1) % per_line == 0) {
            line.push_back('\n');
            if (line.size() > (1 << 20) || k + 1 == n) {
                ok = fwrite(line.data(), 1, line.size(), f) == line.size();
                line.clear();
            }
        }
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? MSL_OK : rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_dump_text: write to %s failed", path);
}

int msl_grid_load_text(const char *path, int dtype, void *grid, int depth, int rows, int cols) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (!path || !grid || !dims_ok(dtype, depth, rows, cols))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_load_text: bad arguments");
    FILE *f = fopen(path, "rb");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_load_text: cannot open %s", path);
    std::vector<char> text;
    char chunk[1 << 16];
    size_t got;
    while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) text.insert(text.end(), chunk, chunk + got);
    fclose(f);
    text.push_back('\0');
    const size_t n = (size_t)depth * rows * cols, es = rt::dtype_size(dtype);
    std::vector<char> h(n * es);
    const char *s = text.data();
    size_t k = 0;
    for (;;) {
        while (*s == ';' || *s == '\n' || *s == '\r' || *s == ' ' || *s == '\t') s++;
        if (!*s) break;
        if (k == n) return rt::fail(MSL_ERR_SIZE_MISMATCH, "msl_grid_load_text: %s holds more than %zu values", path, n);
        char *end = nullptr;
        errno = 0;
        const size_t at = file_to_memory(k, depth, rows, cols) * es;
        if (dtype == MSL_I32) {
            const long v = strtol(s, &end, 10);
            const int32_t w = (int32_t)v;
            memcpy(h.data() + at, &w, 4);
        } else {
            const double v = strtod(s, &end);
            if (dtype == MSL_F64) memcpy(h.data() + at, &v, 8);
            else if (dtype == MSL_F32) {
                const float w = (float)v;
                memcpy(h.data() + at, &w, 4);
            } else {
                const uint16_t w = f_to_bf16((float)v);
                memcpy(h.data() + at, &w, 2);
            }
        }
        if (end == s || (*end && *end != ';' && *end != '\n' && *end != '\r' && *end != ' ' && *end != '\t'))
            return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_grid_load_text: value %zu of %s is not a number", k, path);
        s = end;
        k++;
    }
    if (k != n) return rt::fail(MSL_ERR_SIZE_MISMATCH, "msl_grid_load_text: %s holds %zu values, %zu expected", path, k, n);
    MSL_TRY_CUDA(cudaMemcpyAsync(grid, h.data(), h.size(), cudaMemcpyHostToDevice, c.stream), "msl_grid_load_text");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_grid_load_text");
    return MSL_OK;
}

}  // extern "C"
