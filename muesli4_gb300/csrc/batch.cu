// Batched plain-Jacobi solver of libmsl_gb300.so (msl_batch_*): many grids of
// uneven size iterated to an FP64 residual tolerance together. See
// include/detail/msl_batch.cuh for the kernels.
//
// No reference counterpart: the reference solves one DM at a time
// (examples/jacobisolver.cpp:110-145).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "../include/detail/msl_batch.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

constexpr size_t kResidentSmemMax = 200 * 1024;  // both iterates of a resident grid

struct Batch {
    int storage = MSL_F32;
    bool dc = false;   // MSL_BF16_DC: FP32 solution, BF16 corrections (defect correction)
    size_t es = 4;     // element bytes of the swept arrays (the corrections under defect correction)
    size_t sol_es = 4; // element bytes of the solution the caller sets and gets
    std::vector<int> rows, cols;
    void *pool = nullptr;
    size_t pool_bytes = 0;
    std::vector<BatchGrid> host;
    std::vector<void *> init;  // initial values of each grid (msl_batch_reset restores them)
    BatchGrid *dev = nullptr;
    int *d_lists = nullptr;  // resident list | work list
    int *d_tile_grid = nullptr;  // work-list tile -> position of its grid in the work list
    int *d_active = nullptr;
    int *h_active = nullptr;  // pinned
    std::vector<int> resident, worklist;
    long long total_tiles = 0;
    size_t resident_smem = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

void clear_state(BatchGrid &g) {
    g.cur = 0;
    g.ucur = 0;
    g.done = 0;
    g.iters = 0;
    g.residual = 0.0;
    g.resid_bits = 0ull;
}

constexpr char kCheckpointMagic[8] = {'M', 'S', 'L', 'B', 'A', 'T', '0', '1'};
struct CheckpointGrid {
    int32_t rows, cols;
    int64_t iters;
    double residual;
    int32_t done, pad;
};
static_assert(sizeof(CheckpointGrid) == 32, "checkpoint record layout");

size_t grid_bytes(const Batch &b, int i) { return ((size_t)b.rows[i] * b.cols[i] * b.es + 255) / 256 * 256; }
size_t sol_bytes(const Batch &b, int i) { return ((size_t)b.rows[i] * b.cols[i] * b.sol_es + 255) / 256 * 256; }
// Device bytes of one grid: two iterates and the initial values; under defect
// correction two FP32 solutions, two corrections, the defect and the initial values.
size_t pool_need(const Batch &b, int i) {
    return b.dc ? 3 * sol_bytes(b, i) + 3 * grid_bytes(b, i) : 3 * grid_bytes(b, i);
}
size_t resident_need(const Batch &b, int i) {
    const size_t n = (size_t)b.rows[i] * b.cols[i];
    if (b.dc) return (n * 4 + 127) / 128 * 128 + 3 * ((n * 2 + 127) / 128 * 128);
    return 2 * ((n * b.es + 127) / 128 * 128);
}

template <typename S> size_t round_smem(int depth) {
    return stencil2d_tb_smem<S>(1, depth, batch_tile_rows<S, JacobiSel>());
}
// Tile height of the batch's work-list: that of its plain rounds (defect
// correction keeps 64 x 32 tiles for its defect kernel and correction rounds).
int worklist_tile_rows(const Batch &b) {
    return b.storage == MSL_F32 ? batch_tile_rows<float, JacobiSel>() : kSt2BY;
}

void destroy(Batch *b) {
    if (!b) return;
    if (b->pool) cudaFree(b->pool);
    if (b->dev) cudaFree(b->dev);
    if (b->d_lists) cudaFree(b->d_lists);
    if (b->d_tile_grid) cudaFree(b->d_tile_grid);
    if (b->d_active) cudaFree(b->d_active);
    if (b->h_active) cudaFreeHost(b->h_active);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    delete b;
}

float bf16_bits_to_f(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
uint16_t f_to_bf16_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

template <typename S>
int solve_t(Batch &b, double tol, long long max_iters, int check_every, int depth) {
    auto &c = ctx();
    cudaStream_t st = c.stream;
    // Each grid continues from its own state: a grid set, reset or created
    // starts at sweep 0; a grid that converged or ran out of sweeps in an
    // earlier solve (or in a restored checkpoint) resumes from its sweep count
    // and stops as soon as it is done under this call's tol and max_iters.
    for (auto &g : b.host) {
        if (g.iters % check_every)
            return rt::fail(MSL_ERR_INVALID_ARGUMENT,
                            "msl_batch_solve: a grid stopped after %lld sweeps, not a multiple of check_every %d",
                            g.iters, check_every);
        g.done = g.iters >= max_iters || (g.iters > 0 && !(g.residual > tol));
        g.resid_bits = 0ull;
    }
    MSL_TRY_CUDA(cudaMemcpyAsync(b.dev, b.host.data(), b.host.size() * sizeof(BatchGrid), cudaMemcpyHostToDevice, st),
                 "msl_batch_solve");
    // Resident grids: one launch on the side stream, overlapping the rounds.
    if (!b.resident.empty()) {
        MSL_TRY_CUDA(cudaEventRecord(b.fork, st), "msl_batch_solve");
        MSL_TRY_CUDA(cudaStreamWaitEvent(b.side, b.fork, 0), "msl_batch_solve");
        auto k = batch_resident_kernel<S>;
        MSL_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b.resident_smem),
                     "msl_batch_solve");
        k<<<(unsigned)b.resident.size(), kBatchResidentThreads, b.resident_smem, b.side>>>(b.dev, b.d_lists, tol, max_iters,
                                                                                           check_every, max_iters);
        MSL_TRY_CUDA(cudaGetLastError(), "msl_batch_solve: resident kernel");
        rt::count_launch();
        MSL_TRY_CUDA(cudaEventRecord(b.join, b.side), "msl_batch_solve");
    }
    if (!b.worklist.empty()) {
        const int nlist = (int)b.worklist.size();
        const int *wl = b.d_lists + b.resident.size();
        const size_t smem = round_smem<S>(depth);
        auto rk = batch_round_kernel<S>;
        if (smem > 48 * 1024)
            MSL_TRY_CUDA(cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "msl_batch_solve");
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rk, kSt2Threads, smem);
        const long long grid = std::max(1LL, std::min<long long>(b.total_tiles, (long long)std::max(per_sm, 1) * c.sm_count));
        // Rounds per graph: a whole number of check chunks (and at least 8).
        const int chunk_rounds = check_every / depth;
        int rounds = chunk_rounds % 2 ? 2 * chunk_rounds : chunk_rounds;
        while (rounds < 8) rounds *= 2;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        MSL_TRY_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "msl_batch_solve: capture");
        for (int j = 0; j < rounds; j++) {
            const int check = ((j + 1) % chunk_rounds) == 0;
            rk<<<(unsigned)grid, kSt2Threads, smem, st>>>(b.dev, wl, b.d_tile_grid, b.total_tiles, depth, check,
                                                           nullptr, 0, 0.0, 0, nullptr);
            batch_finalize_kernel<<<1, 256, 0, st>>>(b.dev, wl, nlist, depth, check, tol, max_iters, b.d_active);
        }
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess) return rt::cuda_fail(ce, "msl_batch_solve: capture");
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return rt::cuda_fail(ce, "msl_batch_solve: instantiate");
        const long long max_replays = max_iters / ((long long)rounds * depth) + 2;
        int rc = MSL_OK;
        for (long long rep = 0; rep < max_replays; rep++) {
            ce = cudaGraphLaunch(exec, st);
            if (ce == cudaSuccess) ce = cudaMemcpyAsync(b.h_active, b.d_active, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) {
                rc = rt::cuda_fail(ce, "msl_batch_solve: rounds");
                break;
            }
            rt::count_launch(2 * rounds);
            if (*(volatile int *)b.h_active == 0) break;
        }
        cudaGraphExecDestroy(exec);
        if (rc != MSL_OK) return rc;
    }
    if (!b.resident.empty()) MSL_TRY_CUDA(cudaStreamWaitEvent(st, b.join, 0), "msl_batch_solve");
    MSL_TRY_CUDA(cudaMemcpyAsync(b.host.data(), b.dev, b.host.size() * sizeof(BatchGrid), cudaMemcpyDeviceToHost, st),
                 "msl_batch_solve");
    MSL_TRY_CUDA(cudaStreamSynchronize(st), "msl_batch_solve");
    return rt::check_device_errors("msl_batch_solve");
}

// Defect-correction solve: cycles of `cycle` sweeps (see msl_batch.cuh).
int solve_dc(Batch &b, double tol, long long max_iters, int cycle, int depth) {
    auto &c = ctx();
    cudaStream_t st = c.stream;
    for (auto &g : b.host) {
        if (g.iters % cycle)
            return rt::fail(MSL_ERR_INVALID_ARGUMENT,
                            "msl_batch_solve: a grid stopped after %lld sweeps, not a multiple of the cycle %d", g.iters,
                            cycle);
        g.done = g.iters >= max_iters || (g.iters > 0 && !(g.residual > tol));
        g.resid_bits = 0ull;
    }
    // A solve starts without a pending correction: the first step of a grid
    // re-takes the defect of its solution (the resident kernel clears its own).
    for (int i : b.worklist)
        MSL_TRY_CUDA(cudaMemsetAsync(b.host[i].buf[b.host[i].cur], 0, (size_t)b.rows[i] * b.cols[i] * 2, st),
                     "msl_batch_solve");
    MSL_TRY_CUDA(cudaMemcpyAsync(b.dev, b.host.data(), b.host.size() * sizeof(BatchGrid), cudaMemcpyHostToDevice, st),
                 "msl_batch_solve");
    if (!b.resident.empty()) {
        MSL_TRY_CUDA(cudaEventRecord(b.fork, st), "msl_batch_solve");
        MSL_TRY_CUDA(cudaStreamWaitEvent(b.side, b.fork, 0), "msl_batch_solve");
        auto k = batch_resident_defect_kernel;
        MSL_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b.resident_smem),
                     "msl_batch_solve");
        k<<<(unsigned)b.resident.size(), kBatchResidentThreads, b.resident_smem, b.side>>>(b.dev, b.d_lists, tol,
                                                                                           max_iters, cycle);
        MSL_TRY_CUDA(cudaGetLastError(), "msl_batch_solve: resident kernel");
        rt::count_launch();
        MSL_TRY_CUDA(cudaEventRecord(b.join, b.side), "msl_batch_solve");
    }
    if (!b.worklist.empty()) {
        const int nlist = (int)b.worklist.size();
        const int *wl = b.d_lists + b.resident.size();
        const size_t smem = round_smem<bf16s>(depth);
        auto rk = batch_round_kernel<bf16s, DefectSel>;
        if (smem > 48 * 1024)
            MSL_TRY_CUDA(cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "msl_batch_solve");
        int per_sm = 1, per_sm_d = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rk, kSt2Threads, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_d, batch_defect_kernel, kSt2Threads, 0);
        auto grid_of = [&](int k) {
            return (unsigned)std::max(1LL, std::min<long long>(b.total_tiles, (long long)std::max(k, 1) * c.sm_count));
        };
        // One cycle: the opening step, then the cycle - 1 correction sweeps in
        // rounds of `depth` (the last round takes the remainder).
        std::vector<int> rounds;
        for (int left = cycle - 1; left > 0; left -= depth) rounds.push_back(std::min(depth, left));
        const int cycles_per_graph = 4;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        MSL_TRY_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "msl_batch_solve: capture");
        for (int j = 0; j < cycles_per_graph; j++) {
            batch_defect_kernel<<<grid_of(per_sm_d), kSt2Threads, 0, st>>>(b.dev, wl, b.d_tile_grid, b.total_tiles);
            batch_defect_finalize_kernel<<<1, 256, 0, st>>>(b.dev, wl, nlist, tol, max_iters, b.d_active);
            for (int d : rounds) {
                rk<<<grid_of(per_sm), kSt2Threads, smem, st>>>(b.dev, wl, b.d_tile_grid, b.total_tiles, d, 0, nullptr,
                                                               0, 0.0, 0, nullptr);
                batch_defect_round_finalize_kernel<<<1, 256, 0, st>>>(b.dev, wl, nlist, d);
            }
        }
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess) return rt::cuda_fail(ce, "msl_batch_solve: capture");
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return rt::cuda_fail(ce, "msl_batch_solve: instantiate");
        const long long max_replays = max_iters / ((long long)cycles_per_graph * cycle) + 2;
        int rc = MSL_OK;
        for (long long rep = 0; rep < max_replays; rep++) {
            ce = cudaGraphLaunch(exec, st);
            if (ce == cudaSuccess) ce = cudaMemcpyAsync(b.h_active, b.d_active, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) {
                rc = rt::cuda_fail(ce, "msl_batch_solve: cycles");
                break;
            }
            rt::count_launch(cycles_per_graph * 2 * (1 + (int)rounds.size()));
            if (*(volatile int *)b.h_active == 0) break;
        }
        cudaGraphExecDestroy(exec);
        if (rc != MSL_OK) return rc;
    }
    if (!b.resident.empty()) MSL_TRY_CUDA(cudaStreamWaitEvent(st, b.join, 0), "msl_batch_solve");
    MSL_TRY_CUDA(cudaMemcpyAsync(b.host.data(), b.dev, b.host.size() * sizeof(BatchGrid), cudaMemcpyDeviceToHost, st),
                 "msl_batch_solve");
    MSL_TRY_CUDA(cudaStreamSynchronize(st), "msl_batch_solve");
    return rt::check_device_errors("msl_batch_solve");
}

}  // namespace

extern "C" {

int msl_batch_create(int storage, int count, const int *rows, const int *cols, size_t hbm_budget, void **batch) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (batch) *batch = nullptr;
    if (rt::alloc_fault()) return rt::fail(MSL_ERR_OUT_OF_MEMORY, "msl_batch_create: allocation failure injected");
    if (int e = rt::require_init()) return e;
    if (!batch || !rows || !cols || count <= 0)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_create: bad arguments");
    if (storage != MSL_F32 && storage != MSL_BF16 && storage != MSL_BF16_DC)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT,
                        "msl_batch_create: storage must be MSL_F32, MSL_BF16 or MSL_BF16_DC");
    *batch = nullptr;
    Batch *b = new Batch;
    b->storage = storage;
    b->dc = storage == MSL_BF16_DC;
    b->es = b->dc ? 2 : rt::dtype_size(storage);
    b->sol_es = b->dc ? 4 : b->es;
    b->rows.assign(rows, rows + count);
    b->cols.assign(cols, cols + count);
    for (int i = 0; i < count; i++) {
        if (rows[i] < 1 || cols[i] < 1 || (long long)rows[i] * cols[i] > (1LL << 30)) {
            destroy(b);
            return rt::fail(MSL_ERR_SIZE_MISMATCH, "msl_batch_create: grid %d is %d x %d", i, rows[i], cols[i]);
        }
        b->pool_bytes += pool_need(*b, i);
    }
    const size_t meta = count * sizeof(BatchGrid) + 2 * count * sizeof(int) + 64;
    if (hbm_budget && b->pool_bytes + meta > hbm_budget) {
        size_t need = b->pool_bytes + meta;
        destroy(b);
        return rt::fail(MSL_ERR_BUDGET, "msl_batch_create: %zu bytes needed, budget %zu", need, hbm_budget);
    }
    cudaError_t e = cudaMalloc(&b->pool, b->pool_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->dev, count * sizeof(BatchGrid));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_lists, 2 * count * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_active, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_active, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        destroy(b);
        return rt::cuda_fail(e, "msl_batch_create");
    }
    char *p = (char *)b->pool;
    b->host.resize(count);
    b->init.resize(count);
    for (int i = 0; i < count; i++) {
        BatchGrid &gd = b->host[i];
        memset(&gd, 0, sizeof gd);
        gd.rows = rows[i];
        gd.cols = cols[i];
        gd.buf[0] = p;
        p += grid_bytes(*b, i);
        gd.buf[1] = p;
        p += grid_bytes(*b, i);
        if (b->dc) {
            gd.rhs = p;
            p += grid_bytes(*b, i);
            gd.u[0] = p;
            p += sol_bytes(*b, i);
            gd.u[1] = p;
            p += sol_bytes(*b, i);
        }
        b->init[i] = p;
        p += sol_bytes(*b, i);
        if (resident_need(*b, i) <= kResidentSmemMax) {
            b->resident.push_back(i);
            b->resident_smem = std::max(b->resident_smem, resident_need(*b, i));
        } else {
            b->worklist.push_back(i);
        }
    }
    // Work-list tile prefix (64-column tiles of worklist_tile_rows rows).
    const int ty = worklist_tile_rows(*b);
    for (int i : b->worklist) {
        b->host[i].first_tile = b->total_tiles;
        b->total_tiles += (long long)((cols[i] + kSt2BX - 1) / kSt2BX) * ((rows[i] + ty - 1) / ty);
    }
    std::vector<int> lists(b->resident);
    lists.insert(lists.end(), b->worklist.begin(), b->worklist.end());
    e = cudaMemcpy(b->d_lists, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && b->total_tiles) {
        std::vector<int> tg((size_t)b->total_tiles);
        for (size_t w = 0; w < b->worklist.size(); w++) {
            const BatchGrid &gd = b->host[b->worklist[w]];
            const long long nt = (long long)((gd.cols + kSt2BX - 1) / kSt2BX) * ((gd.rows + ty - 1) / ty);
            for (long long t = 0; t < nt; t++) tg[(size_t)(gd.first_tile + t)] = (int)w;
        }
        e = cudaMalloc(&b->d_tile_grid, tg.size() * sizeof(int));
        if (e == cudaSuccess) e = cudaMemcpy(b->d_tile_grid, tg.data(), tg.size() * sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(b->pool, 0, b->pool_bytes);
    if (e != cudaSuccess) {
        destroy(b);
        return rt::cuda_fail(e, "msl_batch_create");
    }
    *batch = b;
    return MSL_OK;
}

int msl_batch_destroy(void *batch) {
    std::lock_guard<std::recursive_mutex> g(ctx().mu);
    if (batch) {
        cudaStreamSynchronize(ctx().stream);
        destroy((Batch *)batch);
    }
    return MSL_OK;
}

int msl_batch_set_grid(void *batch, int index, const float *host_grid) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    Batch *b = (Batch *)batch;
    if (!b || !host_grid || index < 0 || index >= (int)b->host.size())
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_set_grid: bad arguments");
    const size_t n = (size_t)b->rows[index] * b->cols[index];
    BatchGrid &gd = b->host[index];
    clear_state(gd);
    if (b->dc) {
        MSL_TRY_CUDA(cudaMemcpy(gd.u[0], host_grid, n * 4, cudaMemcpyHostToDevice), "msl_batch_set_grid");
        MSL_TRY_CUDA(cudaMemcpy(b->init[index], host_grid, n * 4, cudaMemcpyHostToDevice), "msl_batch_set_grid");
        return MSL_OK;
    }
    if (b->storage == MSL_F32) {
        MSL_TRY_CUDA(cudaMemcpy(gd.buf[0], host_grid, n * 4, cudaMemcpyHostToDevice), "msl_batch_set_grid");
    } else {
        std::vector<uint16_t> h(n);
        for (size_t i = 0; i < n; i++) h[i] = f_to_bf16_bits(host_grid[i]);
        MSL_TRY_CUDA(cudaMemcpy(gd.buf[0], h.data(), n * 2, cudaMemcpyHostToDevice), "msl_batch_set_grid");
    }
    MSL_TRY_CUDA(cudaMemcpy(b->init[index], gd.buf[0], n * b->es, cudaMemcpyDeviceToDevice), "msl_batch_set_grid");
    return MSL_OK;
}

int msl_batch_get_grid(void *batch, int index, float *host_out, long long *iters, double *residual) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    Batch *b = (Batch *)batch;
    if (!b || !host_out || index < 0 || index >= (int)b->host.size())
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_get_grid: bad arguments");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_batch_get_grid");
    const size_t n = (size_t)b->rows[index] * b->cols[index];
    const BatchGrid &gd = b->host[index];
    if (b->dc) {
        MSL_TRY_CUDA(cudaMemcpy(host_out, gd.u[gd.ucur], n * 4, cudaMemcpyDeviceToHost), "msl_batch_get_grid");
    } else if (b->storage == MSL_F32) {
        MSL_TRY_CUDA(cudaMemcpy(host_out, gd.buf[gd.cur], n * 4, cudaMemcpyDeviceToHost), "msl_batch_get_grid");
    } else {
        std::vector<uint16_t> h(n);
        MSL_TRY_CUDA(cudaMemcpy(h.data(), gd.buf[gd.cur], n * 2, cudaMemcpyDeviceToHost), "msl_batch_get_grid");
        for (size_t i = 0; i < n; i++) host_out[i] = bf16_bits_to_f(h[i]);
    }
    if (iters) *iters = gd.iters;
    if (residual) *residual = gd.residual;
    return MSL_OK;
}

int msl_batch_solve(void *batch, double tol, long long max_iters, int check_every, int depth) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    Batch *b = (Batch *)batch;
    if (!b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_solve: NULL batch");
    if (check_every < 1 || max_iters < 1 || max_iters % check_every)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT,
                        "msl_batch_solve: check_every must be >= 1 and divide max_iters (%lld, %d)", max_iters,
                        check_every);
    if (b->dc) {
        if (check_every < 2 || check_every > kBatchDefectMaxCycle)
            return rt::fail(MSL_ERR_INVALID_ARGUMENT,
                            "msl_batch_solve: the defect-correction cycle (check_every) must be in [2, %d], got %d",
                            kBatchDefectMaxCycle, check_every);
        if (depth <= 0) depth = rt::tuned_depth(MSL_BF16, MSL_ST2_JACOBI5, 1024, 1024, 1);
        if (depth > 8) depth = 8;
        return solve_dc(*b, tol, max_iters, check_every, depth);
    }
    if (depth <= 0) depth = rt::tuned_depth(b->storage, MSL_ST2_JACOBI5, 1024, 1024, 1);
    while (depth > 1 && check_every % depth) depth--;
    if (depth > 8) depth = 8;
    return b->storage == MSL_F32 ? solve_t<float>(*b, tol, max_iters, check_every, depth)
                                 : solve_t<bf16s>(*b, tol, max_iters, check_every, depth);
}

int msl_batch_reset(void *batch) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    Batch *b = (Batch *)batch;
    if (!b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_reset: NULL batch");
    for (size_t i = 0; i < b->host.size(); i++) {
        const size_t n = (size_t)b->rows[i] * b->cols[i];
        void *dst = b->dc ? b->host[i].u[0] : b->host[i].buf[0];
        MSL_TRY_CUDA(cudaMemcpyAsync(dst, b->init[i], n * b->sol_es, cudaMemcpyDeviceToDevice, c.stream),
                     "msl_batch_reset");
        clear_state(b->host[i]);
    }
    return MSL_OK;
}

// Checkpoint file: "MSLBAT01", int32 storage, int32 count, then per grid
// {int32 rows, int32 cols, int64 sweeps, float64 residual, int32 done,
// int32 0}, then per grid the latest iterate and the initial values, each
// rows*cols elements of the storage type (FP32 under MSL_BF16_DC: the
// solution; a resumed solve re-takes its defect). Host byte order.
int msl_batch_checkpoint(void *batch, const char *path) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    Batch *b = (Batch *)batch;
    if (!b || !path) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_checkpoint: bad arguments");
    MSL_TRY_CUDA(cudaStreamSynchronize(c.stream), "msl_batch_checkpoint");
    FILE *f = fopen(path, "wb");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_checkpoint: cannot open %s", path);
    bool ok = fwrite(kCheckpointMagic, 1, 8, f) == 8;
    const int32_t head[2] = {b->storage, (int32_t)b->host.size()};
    ok = ok && fwrite(head, sizeof head, 1, f) == 1;
    for (size_t i = 0; ok && i < b->host.size(); i++) {
        const BatchGrid &gd = b->host[i];
        CheckpointGrid r{b->rows[i], b->cols[i], gd.iters, gd.residual, gd.done, 0};
        ok = fwrite(&r, sizeof r, 1, f) == 1;
    }
    std::vector<char> h;
    for (size_t i = 0; ok && i < b->host.size(); i++) {
        const size_t bytes = (size_t)b->rows[i] * b->cols[i] * b->sol_es;
        h.resize(bytes);
        const BatchGrid &gd = b->host[i];
        const void *src[2] = {b->dc ? gd.u[gd.ucur] : gd.buf[gd.cur], b->init[i]};
        for (int k = 0; ok && k < 2; k++) {
            cudaError_t e = cudaMemcpy(h.data(), src[k], bytes, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                fclose(f);
                return rt::cuda_fail(e, "msl_batch_checkpoint");
            }
            ok = fwrite(h.data(), 1, bytes, f) == bytes;
        }
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? MSL_OK : rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_checkpoint: write to %s failed", path);
}

int msl_batch_restore(const char *path, size_t hbm_budget, void **batch) {
    auto &c = ctx();
    std::lock_guard<std::recursive_mutex> g(c.mu);
    if (int e = rt::require_init()) return e;
    if (!path || !batch) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_restore: bad arguments");
    *batch = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_restore: cannot open %s", path);
    char magic[8];
    int32_t head[2];
    bool ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, kCheckpointMagic, 8) && fread(head, sizeof head, 1, f) == 1 &&
              head[1] > 0 && head[1] <= (1 << 24);
    std::vector<CheckpointGrid> recs;
    if (ok) {
        recs.resize(head[1]);
        ok = fread(recs.data(), sizeof(CheckpointGrid), recs.size(), f) == recs.size();
    }
    std::vector<int> rows, cols;
    for (size_t i = 0; ok && i < recs.size(); i++) {
        ok = recs[i].rows > 0 && recs[i].cols > 0 && recs[i].iters >= 0;
        rows.push_back(recs[i].rows);
        cols.push_back(recs[i].cols);
    }
    if (!ok) {
        fclose(f);
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_restore: %s is not a batch checkpoint", path);
    }
    void *handle = nullptr;
    if (int e = msl_batch_create(head[0], head[1], rows.data(), cols.data(), hbm_budget, &handle)) {
        fclose(f);
        return e;
    }
    Batch *b = (Batch *)handle;
    std::vector<char> h;
    for (size_t i = 0; ok && i < recs.size(); i++) {
        const size_t bytes = (size_t)rows[i] * cols[i] * b->sol_es;
        h.resize(bytes);
        void *dst[2] = {b->dc ? b->host[i].u[0] : b->host[i].buf[0], b->init[i]};
        for (int k = 0; ok && k < 2; k++) {
            ok = fread(h.data(), 1, bytes, f) == bytes;
            if (ok && cudaMemcpy(dst[k], h.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
        }
        BatchGrid &gd = b->host[i];
        clear_state(gd);
        gd.iters = recs[i].iters;
        gd.residual = recs[i].residual;
        gd.done = recs[i].done;
    }
    fclose(f);
    if (!ok) {
        destroy(b);
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_restore: %s is truncated", path);
    }
    *batch = b;
    return MSL_OK;
}

int msl_batch_info(void *batch, int *count, int *resident, long long *tiles, size_t *device_bytes) {
    Batch *b = (Batch *)batch;
    if (!b) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_batch_info: NULL batch");
    if (count) *count = (int)b->host.size();
    if (resident) *resident = (int)b->resident.size();
    if (tiles) *tiles = b->total_tiles;
    if (device_bytes) *device_bytes = b->pool_bytes;
    return MSL_OK;
}

}  // extern "C"
