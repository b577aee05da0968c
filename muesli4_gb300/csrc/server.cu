// Stencil-solve server of libmsl_gb300.so (msl_server_*): continuous batching
// of plain-Jacobi (2-D) and heat3D (3-D) solve requests.
//
// A worker thread owns the device side. Every iteration of its loop it
// (1) admits queued requests in arrival order while their iterates fit in the
//     HBM budget (stream-ordered allocation from the device's memory pool,
//     host-to-device copy of the initial values),
// (2) advances every active request by one check interval of `check_every`
//     sweeps -- all 2-D requests in one tile work-list (batch_round_kernel,
//     `depth` fused sweeps per launch) and all 3-D requests in another
//     (serve3d_round_kernel), on two streams so their work overlaps -- and
//     takes each request's FP64 residual at the end of the interval,
// (3) retires requests whose residual is <= tol or that reached max_iters:
//     copies the result to host memory, frees its iterates, stamps its
//     completion time.
// Requests that arrive while others run join at the next interval, as slots
// and memory free up. Each request's sweeps are exactly those of
// msl_stencil2d_iterate / msl_stencil3d_iterate run on it alone in chunks of
// check_every sweeps, so its result does not depend on what else is served.
//
// No reference counterpart: the reference solves one container at a time.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../include/detail/msl_serve.cuh"
#include "msl_internal.h"

using namespace msl;
using namespace msl::gpu;
using msl::rt::ctx;

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kMaxActive = 4096;  // active requests of each kind
constexpr size_t kResidentSmem = 200 * 1024;  // both iterates of a shared-memory-resident 2-D request
constexpr int kFewRequests = 4;  // at most this many requests of a kind in an interval: one-request kernels

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kFailed = 3, kCancelled = 4 };

struct Request {
    long long id = 0;
    int kind = 0;  // MSL_SERVE_JACOBI2D / MSL_SERVE_HEAT3D
    int depth = 1, rows = 0, cols = 0;
    std::vector<float> init, out;
    Clock::time_point t_submit, t_admit, t_done;
    size_t bytes = 0;  // both iterates
    void *buf[2] = {nullptr, nullptr};
    int cur = 0;
    int launches = 0;  // launches of the last interval on the one-request kernels (buffer flips)
    long long iters = 0;
    double residual = 0.0;
    int waited = 0;          // consecutive intervals this running request was not scheduled
    int state = kQueued;     // read and written under the server lock
    bool finished = false;   // set by the worker when the request converged or ran out of sweeps
    bool cancel = false;     // msl_server_cancel on a running request: retired at the next interval boundary
    int fail_code = 0;       // MSL_ERR_* of a request that failed on its own (kFailed without a server error)
    std::string fail_why;
    size_t cells() const { return (size_t)depth * rows * cols; }
};

struct Server {
    size_t budget = 0, used = 0;
    double tol = 1e-4;
    long long max_iters = 5000;
    int check_every = 100, depth2d = 1;
    int device = 0, sm_count = 152;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::string error;
    long long next_id = 1, completed = 0, intervals = 0;
    std::deque<Request *> queue;
    std::vector<Request *> active;
    std::map<long long, std::unique_ptr<Request>> all;
    cudaStream_t s2 = nullptr, s3 = nullptr, sr = nullptr;  // 2-D rounds, 3-D rounds, resident 2-D grids
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_res_fork = nullptr, ev_res_join = nullptr;
    unsigned *d_ticket = nullptr;  // last-CTA tickets of the 2-D and 3-D round kernels
    unsigned *d_err = nullptr, *h_err = nullptr;  // error word of the one-request kernels (device, pinned host)
    BatchGrid *d2 = nullptr;
    ServeCube *d3 = nullptr;
    int *dlist = nullptr;  // 0..kMaxActive-1
    int *d_active = nullptr;
    int *d_map2 = nullptr, *d_map3 = nullptr;  // tile -> request, block -> request (grown as needed)
    size_t cap_map2 = 0, cap_map3 = 0;
    std::vector<int> map2, map3;
    std::vector<BatchGrid> h2;
    std::vector<ServeCube> h3;
    // checkpoint request: written by the worker between intervals
    std::string ckpt_path;
    bool ckpt_pending = false, ckpt_halt = false, halted = false;
    int ckpt_rc = MSL_OK;
    std::string ckpt_error;
    std::condition_variable cv_ckpt;
};

// Checkpoint file: "MSLSRV01", a CkptHeader, `count` CkptRecords, then per
// record the request's values as FP32 (depth*rows*cols): the initial values
// of a queued request, the latest iterate of a running one, the result of a
// finished one. Host byte order.
constexpr char kServerMagic[8] = {'M', 'S', 'L', 'S', 'R', 'V', '0', '1'};
struct CkptHeader {
    double tol;
    int64_t max_iters;
    int32_t check_every, depth2d;
    uint64_t budget;
    int64_t next_id, count;
};
struct CkptRecord {
    int64_t id;
    int32_t kind, state, depth, rows, cols, pad;
    int64_t iters;
    double residual;
};
static_assert(sizeof(CkptHeader) == 48 && sizeof(CkptRecord) == 48, "checkpoint layout");

double bits_to_double(unsigned long long bits) {
    double d;
    std::memcpy(&d, &bits, sizeof d);
    return d;
}

size_t iterate_bytes(const Request &r) { return 2 * ((r.cells() * sizeof(float) + 255) / 256 * 256); }

void fail_all(Server &s, const std::string &why) {
    std::lock_guard<std::mutex> g(s.mu);
    s.error = why;
    for (auto &kv : s.all)
        if (kv.second->state == kQueued || kv.second->state == kRunning) kv.second->state = kFailed;
    s.queue.clear();
    s.active.clear();
    s.cv_done.notify_all();
}

#define SERVE_TRY(call)                      \
    do {                                     \
        cudaError_t _e = (call);             \
        if (_e != cudaSuccess) return _e;    \
    } while (0)

// Copy an item -> request map to the device, growing its buffer when needed.
// The host vector stays alive until the interval's synchronisation.
cudaError_t upload_map(const std::vector<int> &m, int **d, size_t *cap, cudaStream_t st) {
    if (m.size() > *cap) {
        if (*d) SERVE_TRY(cudaFreeAsync(*d, st));
        const size_t n = std::max(m.size(), 2 * *cap);
        SERVE_TRY(cudaMallocAsync((void **)d, n * sizeof(int), st));
        *cap = n;
    }
    return cudaMemcpyAsync(*d, m.data(), m.size() * sizeof(int), cudaMemcpyHostToDevice, st);
}

// One check interval (check_every sweeps) for every active request.
cudaError_t run_interval(Server &s, const std::vector<Request *> &act) {
    s.h2.clear();
    s.h3.clear();
    s.map2.clear();
    s.map3.clear();
    std::vector<Request *> r2, r3, res2;
    long long tiles = 0, blocks = 0;
    size_t res_smem = 0;
    auto cube3d = [](const Request *r) {
        ServeCube c{};
        c.buf[0] = r->buf[0];
        c.buf[1] = r->buf[1];
        c.depth = r->depth;
        c.rows = r->rows;
        c.cols = r->cols;
        c.cur = r->cur;
        c.iters = r->iters;
        return c;
    };
    auto grid2d = [](const Request *r) {
        BatchGrid g{};
        g.buf[0] = r->buf[0];
        g.buf[1] = r->buf[1];
        g.rows = r->rows;
        g.cols = r->cols;
        g.cur = r->cur;
        g.iters = r->iters;
        return g;
    };
    std::vector<Request *> big2, big3;
    const long long big_items = 2LL * s.sm_count;  // a request this large fills the GPU on its own
    // With only a few requests of a kind in the interval, batching them gains
    // nothing: each runs the one-request kernels, as the plain path would
    // (the resident kernel, one CTA per grid, would leave the GPU idle).
    int count2 = 0, count3 = 0;
    for (Request *r : act) (r->kind == MSL_SERVE_JACOBI2D ? count2 : count3)++;
    const bool alone2 = count2 <= kFewRequests, alone3 = count3 <= kFewRequests;
    for (Request *r : act) {
        if (r->kind == MSL_SERVE_JACOBI2D) {
            if (alone2) {
                big2.push_back(r);
                continue;
            }
            const size_t need = 2 * ((r->cells() * sizeof(float) + 127) / 128 * 128);
            if (need <= kResidentSmem) {  // whole grid in shared memory: one launch per interval
                res2.push_back(r);
                res_smem = std::max(res_smem, need);
                continue;
            }
            const long long nt0 = (long long)((r->cols + kSt2BX - 1) / kSt2BX) * ((r->rows + kSt2BY - 1) / kSt2BY);
            if (nt0 >= big_items) {  // the one-request kernels (TMA, temporal blocking)
                big2.push_back(r);
                continue;
            }
            BatchGrid g = grid2d(r);
            g.first_tile = tiles;
            constexpr int ty = batch_tile_rows<float, JacobiSel>();  // the work-list round's tile height
            const long long nt = (long long)((r->cols + kSt2BX - 1) / kSt2BX) * ((r->rows + ty - 1) / ty);
            tiles += nt;
            s.map2.insert(s.map2.end(), (size_t)nt, (int)s.h2.size());
            s.h2.push_back(g);
            r2.push_back(r);
        } else {
            const long long nb = (long long)((r->cols + kT3BX - 1) / kT3BX) * ((r->rows + kT3BY - 1) / kT3BY) *
                                 ((r->depth + kT3BZ - 1) / kT3BZ);
            if (alone3 || nb >= big_items) {
                big3.push_back(r);
                continue;
            }
            ServeCube c = cube3d(r);
            c.first_block = blocks;
            blocks += nb;
            s.map3.insert(s.map3.end(), (size_t)nb, (int)s.h3.size());
            s.h3.push_back(c);
            r3.push_back(r);
        }
    }
    // descriptor order: batched grids first (the fused finalize covers them),
    // then the resident 2-D grids, then the large requests (their descriptors
    // only carry the residual slot)
    const int nw = (int)s.h2.size(), n3b = (int)s.h3.size();
    for (Request *r : res2) {
        s.h2.push_back(grid2d(r));
        r2.push_back(r);
    }
    const int nres = (int)s.h2.size() - nw;
    for (Request *r : big2) {
        s.h2.push_back(grid2d(r));
        r2.push_back(r);
    }
    for (Request *r : big3) {
        s.h3.push_back(cube3d(r));
        r3.push_back(r);
    }
    const int n2 = (int)s.h2.size(), n3 = (int)s.h3.size();
    SERVE_TRY(cudaEventRecord(s.ev_fork, s.s2));
    SERVE_TRY(cudaStreamWaitEvent(s.s3, s.ev_fork, 0));
    if (n2) {
        SERVE_TRY(cudaMemcpyAsync(s.d2, s.h2.data(), n2 * sizeof(BatchGrid), cudaMemcpyHostToDevice, s.s2));
        if (nres) {  // resident grids on their own stream, overlapping the work-list rounds
            SERVE_TRY(cudaEventRecord(s.ev_res_fork, s.s2));
            SERVE_TRY(cudaStreamWaitEvent(s.sr, s.ev_res_fork, 0));
            auto k = batch_resident_kernel<float>;
            SERVE_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res_smem));
            k<<<(unsigned)nres, kBatchResidentThreads, res_smem, s.sr>>>(s.d2, s.dlist + nw, s.tol, s.max_iters,
                                                                          s.check_every, s.check_every);
            SERVE_TRY(cudaGetLastError());
            rt::count_launch();
            SERVE_TRY(cudaEventRecord(s.ev_res_join, s.sr));
        }
        if (tiles) {
            SERVE_TRY(upload_map(s.map2, &s.d_map2, &s.cap_map2, s.s2));
            const int depth = s.depth2d;
            const size_t smem = stencil2d_tb_smem<float>(1, depth, batch_tile_rows<float, JacobiSel>());
            auto rk = batch_round_kernel<float>;
            if (smem > 48 * 1024)
                SERVE_TRY(cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int per_sm = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rk, kSt2Threads, smem);
            const long long grid =
                std::max(1LL, std::min<long long>(tiles, (long long)std::max(per_sm, 1) * s.sm_count));
            const int launches = s.check_every / depth;
            for (int j = 0; j < launches; j++) {
                const int check = j == launches - 1;
                rk<<<(unsigned)grid, kSt2Threads, smem, s.s2>>>(s.d2, s.dlist, s.d_map2, tiles, depth, check,
                                                                 s.d_ticket, nw, s.tol, s.max_iters, s.d_active);
            }
            SERVE_TRY(cudaGetLastError());
            rt::count_launch(launches);
        }
        for (size_t k = 0; k < big2.size(); k++) {  // as msl_stencil2d_iterate runs a grid alone
            Request *r = big2[k];
            BatchGrid *dg = s.d2 + nw + nres + (int)k;
            const int depth = rt::tuned_depth(MSL_F32, MSL_ST2_JACOBI5, r->rows, r->cols, 1);
            const int tile_rows = rt::tuned_tile_rows(MSL_F32, MSL_ST2_JACOBI5, r->rows, r->cols, 1);
            float *p = (float *)r->buf[r->cur], *q = (float *)r->buf[r->cur ^ 1];
            r->launches = 0;
            for (int i = 0; i < s.check_every;) {
                const int d = std::min(std::max(depth, 1), s.check_every - i);
                unsigned long long *resid = i + d == s.check_every ? &dg->resid_bits : nullptr;
                cudaError_t e = d > 1 ? launch_stencil2d_tb<float>(p, q, r->rows, r->cols, 1, d, 0.0f, JacobiFn{}, resid,
                                                                   s.d_err, s.s2, true, tile_rows)
                                      : launch_stencil2d<float>(p, q, r->rows, r->cols, 1, 0.0f, JacobiFn{}, resid,
                                                                s.d_err, s.s2);
                SERVE_TRY(e);
                rt::count_launch();
                std::swap(p, q);
                i += d;
            }
        }
        if (nres) SERVE_TRY(cudaStreamWaitEvent(s.s2, s.ev_res_join, 0));
        SERVE_TRY(cudaMemcpyAsync(s.h2.data(), s.d2, n2 * sizeof(BatchGrid), cudaMemcpyDeviceToHost, s.s2));
    }
    if (n3) {
        SERVE_TRY(cudaMemcpyAsync(s.d3, s.h3.data(), n3 * sizeof(ServeCube), cudaMemcpyHostToDevice, s.s3));
        if (blocks) {
            SERVE_TRY(upload_map(s.map3, &s.d_map3, &s.cap_map3, s.s3));
            const size_t smem = serve3d_smem();
            SERVE_TRY(cudaFuncSetAttribute(serve3d_round_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int per_sm = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, serve3d_round_kernel, kT3Threads, smem);
            const long long grid =
                std::max(1LL, std::min<long long>(blocks, (long long)std::max(per_sm, 1) * s.sm_count));
            for (int j = 0; j < s.check_every; j++) {
                const int check = j == s.check_every - 1;
                serve3d_round_kernel<<<(unsigned)grid, kT3Threads, smem, s.s3>>>(
                    s.d3, s.dlist, s.d_map3, blocks, check, s.d_ticket + 1, n3b, s.tol, s.max_iters);
            }
            SERVE_TRY(cudaGetLastError());
            rt::count_launch(s.check_every);
        }
        const bool pairs = rt::stencil3d_pair_sweeps() != 0;
        for (size_t k = 0; k < big3.size(); k++) {  // as msl_stencil3d_iterate runs a cube alone
            Request *r = big3[k];
            ServeCube *dc = s.d3 + n3b + (int)k;
            float *p = (float *)r->buf[r->cur], *q = (float *)r->buf[r->cur ^ 1];
            r->launches = 0;
            for (int i = 0; i < s.check_every;) {
                // two sweeps per launch on the z-marching kernel where it applies
                const int n = pairs && i + 2 <= s.check_every ? 2 : 1;
                unsigned long long *resid = i + n == s.check_every ? &dc->resid_bits : nullptr;
                cudaError_t e = cudaErrorNotSupported;
                if (n == 2)
                    e = launch_stencil3d_ztb(p, q, r->depth, r->rows, r->cols, Heat7Fn{}, resid, s.d_err, s.s3,
                                             rt::stencil3d_zchunk());
                if (e == cudaErrorNotSupported) {  // one sweep (a grid TMA cannot address: each sweep alone)
                    for (int j = 0; j < n; j++) {
                        unsigned long long *rj = j + 1 == n ? resid : nullptr;
                        SERVE_TRY(launch_stencil3d<float>(p, q, r->depth, r->rows, r->cols, 1, 0.0f, Heat7Fn{}, rj,
                                                          s.d_err, s.s3, s.sm_count));
                        rt::count_launch();
                        r->launches++;
                        if (j + 1 < n) std::swap(p, q);
                    }
                } else {
                    SERVE_TRY(e);
                    rt::count_launch();
                    r->launches++;
                }
                std::swap(p, q);
                i += n;
            }
        }
        SERVE_TRY(cudaMemcpyAsync(s.h3.data(), s.d3, n3 * sizeof(ServeCube), cudaMemcpyDeviceToHost, s.s3));
    }
    SERVE_TRY(cudaEventRecord(s.ev_join, s.s3));
    SERVE_TRY(cudaStreamWaitEvent(s.s2, s.ev_join, 0));
    if (!big2.empty() || !big3.empty())
        SERVE_TRY(cudaMemcpyAsync(s.h_err, s.d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s.s2));
    SERVE_TRY(cudaStreamSynchronize(s.s2));
    if (*s.h_err) return cudaErrorLaunchTimeout;  // a bounded wait in a stencil kernel gave up
    // large requests: one check interval of sweeps, the residual of its last sweep
    auto advance = [&](Request *r, unsigned long long bits, int flips) {
        r->iters += s.check_every;
        r->cur ^= flips & 1;
        r->residual = bits_to_double(bits);
        r->finished = !(r->residual > s.tol) || r->iters >= s.max_iters;
    };
    for (int i = 0; i < n2; i++) {
        Request *r = r2[i];
        if (i >= nw + nres) {
            const int depth = std::max(1, rt::tuned_depth(MSL_F32, MSL_ST2_JACOBI5, r->rows, r->cols, 1));
            advance(r, s.h2[i].resid_bits, (s.check_every + depth - 1) / depth);
            continue;
        }
        r->cur = s.h2[i].cur;
        r->iters = s.h2[i].iters;
        r->residual = s.h2[i].residual;
        r->finished = s.h2[i].done != 0;
    }
    for (int i = 0; i < n3; i++) {
        Request *r = r3[i];
        if (i >= n3b) {
            advance(r, s.h3[i].resid_bits, r->launches);
            continue;
        }
        r->cur = s.h3[i].cur;
        r->iters = s.h3[i].iters;
        r->residual = s.h3[i].residual;
        r->finished = s.h3[i].done != 0;
    }
    return cudaSuccess;
}

// The running requests one check interval advances. Running every request in
// every interval makes a small request wait for as many intervals as the
// largest one needs, each as long as the sum of all requests' sweeps; so an
// interval takes the requests with the smallest remaining work (cells times
// sweeps left before the cap) until kIntervalCells cells are scheduled --
// several waves of blocks, enough to fill the GPU. A request left out ages:
// its priority is its remaining work halved for every kAgeHalving intervals
// it waited, so large requests keep moving under a steady stream of small
// ones. Which requests share an interval changes only the order in which
// sweeps happen, never a request's own sweeps, so results are unchanged.
constexpr size_t kIntervalCells = 48ull << 20;
constexpr double kAgeHalving = 16.0;

std::vector<Request *> pick_interval(Server &s, const std::vector<Request *> &running) {
    std::vector<std::pair<double, Request *>> order;
    order.reserve(running.size());
    for (Request *r : running) {
        const double rem = (double)r->cells() * (double)std::max(1LL, s.max_iters - r->iters);
        order.emplace_back(rem * std::exp2(-r->waited / kAgeHalving), r);
    }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<double, Request *> &a, const std::pair<double, Request *> &b) {
                         return a.first < b.first;
                     });
    std::vector<Request *> pick;
    size_t cells = 0;
    for (auto &pr : order) {
        Request *r = pr.second;
        if (!pick.empty() && cells >= kIntervalCells) {
            r->waited++;
            continue;
        }
        pick.push_back(r);
        cells += r->cells();
        r->waited = 0;
    }
    return pick;
}

// Called by the worker with the lock held and no device work in flight.
int write_checkpoint(Server &s, const std::string &path, std::string &why) {
    std::vector<Request *> reqs;
    for (Request *r : s.active) reqs.push_back(r);
    for (Request *r : s.queue) reqs.push_back(r);
    for (auto &kv : s.all)
        if (kv.second->state == kDone) reqs.push_back(kv.second.get());
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        why = "cannot open " + path;
        return MSL_ERR_INVALID_ARGUMENT;
    }
    CkptHeader h{s.tol, s.max_iters, s.check_every, s.depth2d, (uint64_t)s.budget, s.next_id, (int64_t)reqs.size()};
    bool ok = fwrite(kServerMagic, 1, 8, f) == 8 && fwrite(&h, sizeof h, 1, f) == 1;
    for (size_t i = 0; ok && i < reqs.size(); i++) {
        const Request *r = reqs[i];
        CkptRecord rec{r->id, r->kind, r->state, r->depth, r->rows, r->cols, 0, r->iters, r->residual};
        ok = fwrite(&rec, sizeof rec, 1, f) == 1;
    }
    std::vector<float> h_buf;
    for (size_t i = 0; ok && i < reqs.size(); i++) {
        Request *r = reqs[i];
        const float *src;
        if (r->state == kRunning) {
            h_buf.resize(r->cells());
            cudaError_t e = cudaMemcpyAsync(h_buf.data(), r->buf[r->cur], r->cells() * sizeof(float),
                                            cudaMemcpyDeviceToHost, s.s2);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s.s2);
            if (e != cudaSuccess) {
                fclose(f);
                why = std::string("checkpoint copy: ") + cudaGetErrorString(e);
                return MSL_ERR_CUDA;
            }
            src = h_buf.data();
        } else {
            src = r->state == kQueued ? r->init.data() : r->out.data();
        }
        ok = fwrite(src, sizeof(float), r->cells(), f) == r->cells();
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        why = "write to " + path + " failed";
        return MSL_ERR_INVALID_ARGUMENT;
    }
    return MSL_OK;
}

void worker_loop(Server *sp) {
    Server &s = *sp;
    cudaSetDevice(s.device);
    std::vector<void *> cancelled_bufs;
    for (;;) {
        std::vector<Request *> act;
        for (void *p : cancelled_bufs) cudaFreeAsync(p, s.s2);
        cancelled_bufs.clear();
        {
            std::unique_lock<std::mutex> g(s.mu);
            if (s.ckpt_pending) {  // no work in flight here: every active request sits at an interval end
                s.ckpt_rc = write_checkpoint(s, s.ckpt_path, s.ckpt_error);
                s.ckpt_pending = false;
                s.halted = s.ckpt_halt && s.ckpt_rc == MSL_OK;
                s.cv_ckpt.notify_all();
                if (s.halted) {
                    s.cv_done.notify_all();
                    return;
                }
            }
            // retire running requests cancelled since the last interval (no
            // device work is in flight here); their iterates are freed below
            for (size_t i = 0; i < s.active.size();) {
                Request *r = s.active[i];
                if (!r->cancel) {
                    i++;
                    continue;
                }
                r->state = kCancelled;
                r->t_done = Clock::now();
                if (r->buf[0]) cancelled_bufs.push_back(r->buf[0]);
                r->buf[0] = r->buf[1] = nullptr;
                r->init.clear();
                r->init.shrink_to_fit();
                s.used -= r->bytes;
                s.active.erase(s.active.begin() + i);
                s.cv_done.notify_all();
            }
            // admit in arrival order while memory and slots allow
            int n2 = 0, n3 = 0;
            for (Request *r : s.active) (r->kind == MSL_SERVE_JACOBI2D ? n2 : n3)++;
            while (!s.queue.empty()) {
                Request *r = s.queue.front();
                int &n = r->kind == MSL_SERVE_JACOBI2D ? n2 : n3;
                if (n >= kMaxActive || (s.budget && s.used + r->bytes > s.budget)) break;
                s.queue.pop_front();
                s.used += r->bytes;
                n++;
                r->state = kRunning;
                r->t_admit = Clock::now();
                s.active.push_back(r);
                // allocation and upload happen below, outside the lock
                r->buf[0] = nullptr;
            }
            if (s.active.empty()) {
                if (s.stop) return;
                s.cv_work.wait(g, [&] { return s.stop || !s.queue.empty() || s.ckpt_pending; });
                continue;
            }
            act = s.active;
        }
        bool ok = true;
        std::string why;
        std::vector<Request *> no_memory;  // admitted requests whose iterates could not be allocated
        for (Request *r : act) {
            if (r->buf[0]) continue;
            const size_t half = r->bytes / 2;
            void *p = nullptr;
            cudaError_t e = rt::alloc_fault() ? cudaErrorMemoryAllocation : cudaMallocAsync(&p, r->bytes, s.s2);
            if (e == cudaErrorMemoryAllocation) {  // this request fails alone; the others go on
                cudaGetLastError();
                no_memory.push_back(r);
                continue;
            }
            if (e == cudaSuccess) {
                r->buf[0] = p;
                r->buf[1] = (char *)p + half;
                r->cur = 0;  // r->iters is 0, or the sweeps of a request resumed from a checkpoint
                e = cudaMemcpyAsync(r->buf[0], r->init.data(), r->cells() * sizeof(float), cudaMemcpyHostToDevice, s.s2);
            }
            if (e != cudaSuccess) {
                ok = false;
                why = std::string("admission: ") + cudaGetErrorString(e);
                break;
            }
        }
        if (ok && !no_memory.empty()) {
            std::lock_guard<std::mutex> g(s.mu);
            for (Request *r : no_memory) {
                r->state = kFailed;
                r->fail_code = MSL_ERR_OUT_OF_MEMORY;
                r->fail_why = "no device memory for the request's iterates";
                r->t_done = Clock::now();
                s.used -= r->bytes;
                s.active.erase(std::find(s.active.begin(), s.active.end(), r));
                act.erase(std::find(act.begin(), act.end(), r));
            }
            s.cv_done.notify_all();
        }
        if (ok && act.empty()) continue;
        if (ok) {
            act = pick_interval(s, act);
            cudaError_t e = run_interval(s, act);
            if (e != cudaSuccess) {
                ok = false;
                why = std::string("interval: ") + cudaGetErrorString(e);
            }
        }
        if (!ok) {
            fail_all(s, why);
            return;
        }
        s.intervals++;
        // retire finished requests
        std::vector<Request *> done;
        for (Request *r : act)
            if (r->finished) done.push_back(r);
        for (Request *r : done) {
            r->out.resize(r->cells());
            cudaError_t e = cudaMemcpyAsync(r->out.data(), r->buf[r->cur], r->cells() * sizeof(float),
                                            cudaMemcpyDeviceToHost, s.s2);
            if (e == cudaSuccess) e = cudaFreeAsync(r->buf[0], s.s2);
            if (e != cudaSuccess) {
                fail_all(s, std::string("retire: ") + cudaGetErrorString(e));
                return;
            }
        }
        if (!done.empty()) {
            cudaStreamSynchronize(s.s2);
            const auto now = Clock::now();
            std::lock_guard<std::mutex> g(s.mu);
            for (Request *r : done) {
                r->state = kDone;
                r->t_done = now;
                r->buf[0] = r->buf[1] = nullptr;
                r->init.clear();
                r->init.shrink_to_fit();
                s.used -= r->bytes;
                s.completed++;
                s.active.erase(std::find(s.active.begin(), s.active.end(), r));
            }
            s.cv_done.notify_all();
        }
    }
}

Server *as_server(void *p) { return (Server *)p; }

}  // namespace

extern "C" {

int msl_server_start(size_t hbm_budget, double tol, long long max_iters, int check_every, int depth, void **server) {
    auto &c = ctx();
    if (int e = rt::require_init()) return e;
    if (!server || check_every < 1 || max_iters < 1 || max_iters % check_every)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_start: check_every must be >= 1 and divide max_iters");
    if (depth <= 0) depth = rt::tuned_depth(MSL_F32, MSL_ST2_JACOBI5, 1024, 1024, 1);
    while (depth > 1 && check_every % depth) depth--;
    auto *s = new Server;
    s->budget = hbm_budget;
    s->tol = tol;
    s->max_iters = max_iters;
    s->check_every = check_every;
    s->depth2d = std::min(depth, 8);
    s->device = c.device;
    s->sm_count = c.sm_count;
    cudaError_t e = cudaStreamCreateWithFlags(&s->s2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s3, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->sr, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_res_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_res_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_ticket, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(s->d_ticket, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_err, 2 * sizeof(unsigned));  // error word, wait limit (0: default)
    if (e == cudaSuccess) e = cudaMemset(s->d_err, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_err, sizeof(unsigned));
    if (e == cudaSuccess) *s->h_err = 0;
    if (e == cudaSuccess) e = cudaMalloc(&s->d2, kMaxActive * sizeof(BatchGrid));
    if (e == cudaSuccess) e = cudaMalloc(&s->d3, kMaxActive * sizeof(ServeCube));
    if (e == cudaSuccess) e = cudaMalloc(&s->dlist, kMaxActive * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_active, sizeof(int));
    if (e == cudaSuccess) {
        std::vector<int> iota(kMaxActive);
        for (int i = 0; i < kMaxActive; i++) iota[i] = i;
        e = cudaMemcpy(s->dlist, iota.data(), kMaxActive * sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        // keep freed iterates in the pool for the next admissions (up to the budget)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, c.device) == cudaSuccess) {
            cuuint64_t keep = hbm_budget ? hbm_budget : ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e != cudaSuccess) {
        delete s;
        return rt::cuda_fail(e, "msl_server_start");
    }
    s->worker = std::thread(worker_loop, s);
    *server = s;
    return MSL_OK;
}

int msl_server_submit(void *server, int kind, int depth, int rows, int cols, const float *init, long long *request) {
    Server *s = as_server(server);
    if (!s || !init || !request) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_submit: NULL argument");
    if (kind != MSL_SERVE_JACOBI2D && kind != MSL_SERVE_HEAT3D)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_submit: unknown kind %d", kind);
    if (kind == MSL_SERVE_JACOBI2D) depth = 1;
    if (depth < 1 || rows < 1 || cols < 1 || (long long)depth * rows * cols > (1LL << 31) - 1)
        return rt::fail(MSL_ERR_SIZE_MISMATCH, "msl_server_submit: bad shape %d x %d x %d", depth, rows, cols);
    auto r = std::make_unique<Request>();
    r->kind = kind;
    r->depth = depth;
    r->rows = rows;
    r->cols = cols;
    r->init.assign(init, init + r->cells());
    r->bytes = iterate_bytes(*r);
    if (s->budget && r->bytes > s->budget)
        return rt::fail(MSL_ERR_BUDGET, "msl_server_submit: request needs %zu bytes, budget %zu", r->bytes, s->budget);
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->error.empty()) return rt::fail(MSL_ERR_CUDA, "msl_server_submit: server failed: %s", s->error.c_str());
    if (s->stop || s->halted) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_submit: server is stopping");
    r->id = s->next_id++;
    r->t_submit = Clock::now();
    *request = r->id;
    s->queue.push_back(r.get());
    s->all[r->id] = std::move(r);
    s->cv_work.notify_one();
    return MSL_OK;
}

int msl_server_wait(void *server, long long request, double timeout_s) {
    Server *s = as_server(server);
    if (!s) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_wait: NULL server");
    std::unique_lock<std::mutex> g(s->mu);
    auto it = s->all.find(request);
    if (it == s->all.end()) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_wait: unknown request %lld", request);
    Request *r = it->second.get();
    auto pred = [&] { return r->state == kDone || r->state == kFailed || r->state == kCancelled || s->halted; };
    if (timeout_s < 0) s->cv_done.wait(g, pred);
    else if (!s->cv_done.wait_for(g, std::chrono::duration<double>(timeout_s), pred))
        return rt::fail(MSL_ERR_TIMEOUT, "msl_server_wait: request %lld not finished", request);
    if (r->state == kCancelled) return rt::fail(MSL_ERR_CANCELLED, "msl_server_wait: request %lld was cancelled", request);
    if (r->state == kFailed && r->fail_code)
        return rt::fail(r->fail_code, "msl_server_wait: request %lld: %s", request, r->fail_why.c_str());
    if (r->state == kFailed) return rt::fail(MSL_ERR_CUDA, "msl_server_wait: %s", s->error.c_str());
    if (r->state != kDone)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_wait: the server halted after a checkpoint");
    return MSL_OK;
}

int msl_server_result(void *server, long long request, float *out, long long *iters, double *residual,
                      double *latency_s, double *queue_s) {
    Server *s = as_server(server);
    if (!s) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_result: NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(request);
    if (it == s->all.end()) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_result: unknown request %lld", request);
    Request *r = it->second.get();
    if (r->state == kCancelled)
        return rt::fail(MSL_ERR_CANCELLED, "msl_server_result: request %lld was cancelled", request);
    if (r->state != kDone) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_result: request %lld not done", request);
    if (out) std::memcpy(out, r->out.data(), r->out.size() * sizeof(float));
    if (iters) *iters = r->iters;
    if (residual) *residual = r->residual;
    if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    if (queue_s) *queue_s = std::chrono::duration<double>(r->t_admit - r->t_submit).count();
    return MSL_OK;
}

int msl_server_cancel(void *server, long long request) {
    Server *s = as_server(server);
    if (!s) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_cancel: NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(request);
    if (it == s->all.end()) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_cancel: unknown request %lld", request);
    Request *r = it->second.get();
    if (r->state == kQueued) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
        r->state = kCancelled;
        r->t_done = Clock::now();
        r->init.clear();
        r->init.shrink_to_fit();
        s->cv_done.notify_all();
        return MSL_OK;
    }
    if (r->state == kRunning) {
        r->cancel = true;  // the worker retires it before its next interval
        s->cv_work.notify_all();
        return MSL_OK;
    }
    return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_cancel: request %lld has already finished", request);
}

int msl_server_release(void *server, long long request) {
    Server *s = as_server(server);
    if (!s) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_release: NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->all.find(request);
    if (it == s->all.end() || (it->second->state != kDone && it->second->state != kCancelled &&
                               !(it->second->state == kFailed && it->second->fail_code)))
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_release: request %lld is not a finished request", request);
    s->all.erase(it);
    return MSL_OK;
}

int msl_server_stats(void *server, long long *completed, long long *active, long long *queued, size_t *device_bytes,
                     long long *intervals) {
    Server *s = as_server(server);
    if (!s) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_stats: NULL server");
    std::lock_guard<std::mutex> g(s->mu);
    if (completed) *completed = s->completed;
    if (active) *active = (long long)s->active.size();
    if (queued) *queued = (long long)s->queue.size();
    if (device_bytes) *device_bytes = s->used;
    if (intervals) *intervals = s->intervals;
    return MSL_OK;
}

int msl_server_checkpoint(void *server, const char *path, int halt) {
    Server *s = as_server(server);
    if (!s || !path) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_checkpoint: NULL argument");
    std::unique_lock<std::mutex> g(s->mu);
    if (!s->error.empty()) return rt::fail(MSL_ERR_CUDA, "msl_server_checkpoint: server failed: %s", s->error.c_str());
    if (s->halted || s->stop || s->ckpt_pending)
        return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_checkpoint: server is stopping or busy");
    s->ckpt_path = path;
    s->ckpt_halt = halt != 0;
    s->ckpt_pending = true;
    s->cv_work.notify_all();
    // the worker takes it between two intervals (one interval at most)
    s->cv_ckpt.wait(g, [&] { return !s->ckpt_pending || !s->error.empty(); });
    if (s->ckpt_pending) return rt::fail(MSL_ERR_CUDA, "msl_server_checkpoint: server failed: %s", s->error.c_str());
    if (s->ckpt_rc != MSL_OK) return rt::fail(s->ckpt_rc, "msl_server_checkpoint: %s", s->ckpt_error.c_str());
    return MSL_OK;
}

int msl_server_restore(const char *path, void **server) {
    if (!path || !server) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_restore: NULL argument");
    *server = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_restore: cannot open %s", path);
    char magic[8];
    CkptHeader h{};
    bool ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, kServerMagic, 8) && fread(&h, sizeof h, 1, f) == 1 &&
              h.count >= 0 && h.count <= (1 << 24) && h.check_every >= 1 && h.max_iters >= 1 &&
              h.max_iters % h.check_every == 0;
    std::vector<CkptRecord> recs;
    if (ok) {
        recs.resize((size_t)h.count);
        ok = fread(recs.data(), sizeof(CkptRecord), recs.size(), f) == recs.size();
    }
    std::vector<std::unique_ptr<Request>> reqs;
    std::set<long long> ids;  // a request id appears once: the server's table is keyed by it
    for (size_t i = 0; ok && i < recs.size(); i++) {
        const CkptRecord &c = recs[i];
        ok = (c.kind == MSL_SERVE_JACOBI2D || c.kind == MSL_SERVE_HEAT3D) &&
             (c.state == kQueued || c.state == kRunning || c.state == kDone) && c.depth >= 1 && c.rows >= 1 &&
             c.cols >= 1 && (long long)c.depth * c.rows * c.cols <= (1LL << 31) - 1 && c.iters >= 0 &&
             c.iters % h.check_every == 0 && c.id > 0 && c.id < h.next_id && ids.insert(c.id).second;
        if (!ok) break;
        auto r = std::make_unique<Request>();
        r->id = c.id;
        r->kind = c.kind;
        r->depth = c.depth;
        r->rows = c.rows;
        r->cols = c.cols;
        r->iters = c.iters;
        r->residual = c.residual;
        r->state = c.state;
        std::vector<float> &dst = c.state == kDone ? r->out : r->init;
        dst.resize(r->cells());
        ok = fread(dst.data(), sizeof(float), dst.size(), f) == dst.size();
        r->bytes = iterate_bytes(*r);
        reqs.push_back(std::move(r));
    }
    fclose(f);
    if (!ok) return rt::fail(MSL_ERR_INVALID_ARGUMENT, "msl_server_restore: %s is not a complete server checkpoint", path);
    void *handle = nullptr;
    if (int e = msl_server_start((size_t)h.budget, h.tol, h.max_iters, h.check_every, h.depth2d, &handle)) return e;
    Server *s = as_server(handle);
    {
        std::lock_guard<std::mutex> g(s->mu);
        const auto now = Clock::now();
        s->next_id = h.next_id;
        // running requests first (they were admitted before the queued ones), then the queue, in file order
        for (int pass = 0; pass < 2; pass++)
            for (auto &r : reqs) {
                if (!r || r->state == kDone || (pass == 0) != (r->state == kRunning)) continue;
                r->state = kQueued;
                r->t_submit = now;
                s->queue.push_back(r.get());
                const long long id = r->id;
                s->all[id] = std::move(r);
            }
        for (auto &r : reqs) {
            if (!r) continue;
            r->t_submit = r->t_admit = r->t_done = now;
            s->completed++;
            const long long id = r->id;
            s->all[id] = std::move(r);
        }
        s->cv_work.notify_one();
    }
    *server = s;
    return MSL_OK;
}

int msl_server_stop(void *server) {
    Server *s = as_server(server);
    if (!s) return MSL_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto &kv : s->all)
        if (kv.second->buf[0]) cudaFreeAsync(kv.second->buf[0], s->s2);
    cudaStreamSynchronize(s->s2);
    cudaFree(s->d2);
    cudaFree(s->d3);
    cudaFree(s->dlist);
    cudaFree(s->d_active);
    if (s->d_map2) cudaFree(s->d_map2);
    if (s->d_map3) cudaFree(s->d_map3);
    cudaFree(s->d_ticket);
    cudaFree(s->d_err);
    cudaFreeHost(s->h_err);
    cudaEventDestroy(s->ev_fork);
    cudaEventDestroy(s->ev_join);
    cudaEventDestroy(s->ev_res_fork);
    cudaEventDestroy(s->ev_res_join);
    cudaStreamDestroy(s->sr);
    cudaStreamDestroy(s->s2);
    cudaStreamDestroy(s->s3);
    std::string err = s->error;
    delete s;
    if (!err.empty()) return rt::fail(MSL_ERR_CUDA, "msl_server_stop: the server had failed: %s", err.c_str());
    return MSL_OK;
}

}  // extern "C"
