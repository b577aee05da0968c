// Autotuner for the stencil skeletons: times the candidate launch shapes of
// msl_stencil2d_iterate -- temporal depth (sweeps per launch) and, for depths
// of two and more, the tile height of the temporal-blocking kernel (64 x 16,
// 64 x 32 or 64 x 64 cells on 128, 256 or 512 threads) -- on the caller's
// grid shape and records the fastest per (element type, functor, radius,
// grid-size class). The reference fixes its tiling statically (tile width 16,
// include/muesli.h:195; 1024-thread blocks, src/muesli.cpp:103).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "../include/detail/msl_stencil.cuh"
#include "msl_internal.h"

namespace msl {
namespace rt {

namespace {
using Key = std::tuple<int, int, int, int>;  // dtype, kind, radius, size class
struct Record {
    int depth;
    int tile_rows;
    double rate;
};
std::mutex g_mu;
std::map<Key, Record> &table() {
    static std::map<Key, Record> t;
    return t;
}
// Grid-size class: rounded log2 of the cell count (grids within a factor of
// sqrt(2) share a record).
int size_class(int rows, int cols) { return (int)std::lround(std::log2((double)rows * (double)cols)); }
}  // namespace

int tuned_depth(int dtype, int kind, int rows, int cols, int radius) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = table().find(Key{dtype, kind, radius, size_class(rows, cols)});
    return it == table().end() ? 1 : it->second.depth;
}

int tuned_tile_rows(int dtype, int kind, int rows, int cols, int radius) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = table().find(Key{dtype, kind, radius, size_class(rows, cols)});
    return it == table().end() ? 32 : it->second.tile_rows;
}

// Fill a tuning grid with a pseudo-random 0/1 pattern (a valid input for
// every built-in functor; a constant grid would hide data-dependent branches).
// `one` is the element bit pattern of 1 in the grid's element type.
__global__ void tune_fill_kernel(unsigned char *p, size_t n, int es, unsigned long long one) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned h = (unsigned)i * 2654435761u;
        h ^= h >> 15;
        const unsigned long long v = ((h >> 7) % 10u) < 3u ? one : 0ull;  // about 30 % ones
        for (int k = 0; k < es; k++) p[i * es + k] = (unsigned char)(v >> (8 * k));
    }
}

unsigned long long one_bits(int dtype) {
    switch (dtype) {
        case MSL_F32: return 0x3F800000ull;
        case MSL_F64: return 0x3FF0000000000000ull;
        case MSL_I32: return 1ull;
        default: return 0x3F80ull;  // MSL_BF16
    }
}

}  // namespace rt
}  // namespace msl

using namespace msl;

extern "C" {

int msl_autotune_stencil2d_shape(int dtype, int kind, int rows, int cols, int radius, int iters, int *best_depth,
                                 int *best_tile_rows, double *best_rate) {
    auto &c = rt::ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (rows <= 0 || cols <= 0 || iters < 1)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_stencil2d: bad shape or iteration count");
    const size_t es = rt::dtype_size(dtype);
    if (!es) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_stencil2d: unknown dtype %d", dtype);
    const size_t bytes = (size_t)rows * cols * es;
    void *a = nullptr, *b = nullptr;
    MSL_TRY_CUDA(cudaMalloc(&a, bytes), "msl_autotune_stencil2d");
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaFree(a);
        return rt::fail(MSL_ERR_OUT_OF_MEMORY, "msl_autotune_stencil2d: scratch grids");
    }
    rt::tune_fill_kernel<<<(unsigned)(c.sm_count * 8), 256, 0, c.stream>>>((unsigned char *)a, (size_t)rows * cols,
                                                                            (int)es, rt::one_bits(dtype));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = 1, best_rows = 32;
    double best_r = 0.0;
    int rc = MSL_OK;
    // the caller's settings, put back when the trials end
    const int saved_depth = rt::temporal_depth_setting(), saved_rows = rt::tile_rows_setting();
    // (depth, tile rows); depth 1 is the one-sweep kernel, whose tiles are fixed
    struct Cand {
        int depth, tile_rows;
    };
    Cand candidates[1 + 9 * 3];
    int ncand = 0;
    candidates[ncand++] = Cand{1, 32};
    const bool tiles_vary = dtype != MSL_I32;  // Life's fused generations run on the packed kernel's own tiles
    for (int d : {2, 3, 4, 6, 8, 12, 16, 24, 32})
        for (int t : {16, 32, 64})
            if (tiles_vary || t == 32) candidates[ncand++] = Cand{d, t};
    double rate[1 + 9 * 3] = {};
    bool usable[1 + 9 * 3] = {};
    // Warm every shape up once, then time each five times, interleaved, and
    // keep each shape's best run (clock ramps and other work on the GPU slow
    // single runs down, never speed them up; shapes within a few per cent of
    // each other swap places between single runs).
    for (int round = 0; round < 6 && rc == MSL_OK; round++) {
        for (int k = 0; k < ncand; k++) {
            const int d = candidates[k].depth;
            if (d > iters || (round > 0 && !usable[k])) continue;
            if (msl_set_temporal_depth(d) != MSL_OK || msl_set_tile_rows(candidates[k].tile_rows) != MSL_OK) continue;
            int inb = 0;
            if (round == 0) {
                rc = msl_stencil2d_iterate(dtype, kind, a, b, rows, cols, radius, 0.0, d, nullptr, &inb);
                if (rc != MSL_OK) {
                    if (d == 1) break;  // the functor itself is not available: report it
                    rc = MSL_OK;        // this shape does not fit: skip it
                    continue;
                }
                usable[k] = true;
                continue;
            }
            cudaEventRecord(e0, c.stream);
            rc = msl_stencil2d_iterate(dtype, kind, a, b, rows, cols, radius, 0.0, iters, nullptr, &inb);
            cudaEventRecord(e1, c.stream);
            if (rc != MSL_OK) break;
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            rate[k] = std::max(rate[k], (double)rows * cols * iters / (ms * 1e-3));
        }
    }
    for (int k = 0; k < ncand; k++)
        if (usable[k] && rate[k] > best_r) {
            best_r = rate[k];
            best = candidates[k].depth;
            best_rows = candidates[k].tile_rows;
        }
    msl_set_temporal_depth(saved_depth);
    msl_set_tile_rows(saved_rows);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    if (rc != MSL_OK) return rc;
    {
        std::lock_guard<std::mutex> g2(rt::g_mu);
        rt::table()[rt::Key{dtype, kind, radius, rt::size_class(rows, cols)}] = rt::Record{best, best_rows, best_r};
    }
    if (best_depth) *best_depth = best;
    if (best_tile_rows) *best_tile_rows = best_rows;
    if (best_rate) *best_rate = best_r;
    return rt::check_device_errors("msl_autotune_stencil2d");
}

int msl_autotune_stencil2d(int dtype, int kind, int rows, int cols, int radius, int iters, int *best_depth,
                           double *best_rate) {
    return msl_autotune_stencil2d_shape(dtype, kind, rows, cols, radius, iters, best_depth, nullptr, best_rate);
}

int msl_autotune_save(const char *path) {
    if (!path) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_save: NULL path");
    FILE *f = std::fopen(path, "w");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_save: cannot open %s", path);
    std::lock_guard<std::mutex> g(rt::g_mu);
    std::fprintf(f, "# dtype kind radius size_class depth rate tile_rows\n");
    for (auto &kv : rt::table())
        std::fprintf(f, "%d %d %d %d %d %.6g %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
                     std::get<2>(kv.first), std::get<3>(kv.first), kv.second.depth, kv.second.rate,
                     kv.second.tile_rows);
    std::fclose(f);
    return MSL_OK;
}

int msl_autotune_load(const char *path) {
    if (!path) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_load: NULL path");
    FILE *f = std::fopen(path, "r");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_autotune_load: cannot open %s", path);
    char line[256];
    std::lock_guard<std::mutex> g(rt::g_mu);
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '#') continue;
        int dt, k, r, sc, d, t = 32;
        double rate;
        const int got = std::sscanf(line, "%d %d %d %d %d %lf %d", &dt, &k, &r, &sc, &d, &rate, &t);
        if (got >= 6 && d >= 1 && d <= 32 && msl::gpu::valid_tile_rows(t))  // no tile height recorded: 32 rows
            rt::table()[rt::Key{dt, k, r, sc}] = rt::Record{d, t, rate};
    }
    std::fclose(f);
    return MSL_OK;
}

}  // extern "C"
