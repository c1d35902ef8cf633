// ma_batch.cu -- many independent OT problems at once.
//
// The reference solves one problem per MA::ot_solve call
// (include/MA/optimal_transport.hpp:89-193).  Small problems (a few thousand sites)
// leave most of the 152 SMs idle and spend their time in launch and host round-trip
// latency, so a batch of them is solved by K workers, each a context of its own (one
// CUDA stream, its own scratch) driven by one host thread: the workers take the
// problems in order from a shared counter, and the kernels of K problems run side by
// side on the GPU.  Every problem goes through the same ma_ot_solve as a single call;
// a worker's cooperative CG grid is its share of the GPU, so the CG sums run in
// another order and the result agrees with a sequential loop's to the solver's
// tolerance (not to the last bit).
//
// K is autotuned when the caller passes 0 and the context has no earlier choice: the
// batch's median-sized problem is solved once on every candidate worker (their
// buffers reach that size), then K copies of it are solved concurrently for each
// candidate K = 4, 8, 16, 32, 64, and the K with the most problems per second is kept in
// the context.  The batch then runs largest problem first: every worker's buffers
// reach their size early (device allocations synchronise the whole GPU), and the
// longest solves do not end up last.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "ma_runtime.h"

namespace ma {

static ma_status ensure_workers(Ctx* c, int k)
{
    while ((int)c->workers.size() < k) {
        ma_ctx* w = nullptr;
        ma_status st = ma_ctx_create(c->device, &w);
        if (st != MA_OK) return st;
        c->workers.push_back(w);
    }
    // k problems share the GPU: each cooperative solve takes 1 / k of it
    for (int t = 0; t < k; t++) {
        c->workers[(size_t)t]->grid_share = k;
        c->workers[(size_t)t]->blocking_sync = true;
    }
    return MA_OK;
}

// solve problems order[begin, end) with k workers; returns the first failure status of
// a worker's CUDA or argument errors (per-problem solver outcomes go to the problems)
static ma_status run_chunk(Ctx* c, ma_problem* pb, const std::vector<int64_t>& order, int64_t begin, int64_t end,
                           ma_mem mem, const ma_solve_opts* o, int k)
{
    std::atomic<int64_t> next(begin);
    std::vector<std::thread> th;
    std::vector<ma_status> err((size_t)k, MA_OK);
    for (int t = 0; t < k; t++) {
        th.emplace_back([&, t]() {
            ma_ctx* wc = c->workers[(size_t)t];
            for (;;) {
                const int64_t r = next.fetch_add(1);
                if (r >= end) break;
                ma_problem& p = pb[order[(size_t)r]];
                ma_stats st{};
                p.status = ma_ot_solve(wc, p.mesh, p.n, p.x, p.y, p.nu, p.w, mem, o, &st);
                p.stats = st;
                if (p.status == MA_ERR_CUDA || p.status == MA_ERR_OUT_OF_MEMORY || p.status == MA_ERR_NO_DEVICE) {
                    err[(size_t)t] = p.status;
                    break;
                }
            }
        });
    }
    for (auto& x : th) x.join();
    for (ma_status e : err)
        if (e != MA_OK) return e;
    return MA_OK;
}

// K concurrent copies of problem p on workers 0..K-1: seconds taken
static ma_status solve_copies(Ctx* c, const ma_problem& p, ma_mem mem, const ma_solve_opts* o, int K, double* dt)
{
    const size_t n = (size_t)p.n;
    std::vector<ma_status> err((size_t)K, MA_OK);
    std::vector<std::thread> th;
    const auto t0 = std::chrono::steady_clock::now();
    for (int t = 0; t < K; t++) {
        th.emplace_back([&, t]() {
            ma_ctx* wc = c->workers[(size_t)t];
            double* wp = mem == MA_MEM_DEVICE ? c->tune_w.as<double>() + (size_t)t * n : c->tune_wh.data() + (size_t)t * n;
            if (mem == MA_MEM_DEVICE) {
                if (cudaMemcpyAsync(wp, p.w, sizeof(double) * n, cudaMemcpyDeviceToDevice, wc->stream) != cudaSuccess) {
                    err[(size_t)t] = MA_ERR_CUDA;
                    return;
                }
            } else {
                std::copy(p.w, p.w + n, wp);
            }
            ma_stats st{};
            ma_status r = ma_ot_solve(wc, p.mesh, p.n, p.x, p.y, p.nu, wp, mem, o, &st);
            if (r == MA_ERR_CUDA || r == MA_ERR_OUT_OF_MEMORY || r == MA_ERR_NO_DEVICE) err[(size_t)t] = r;
        });
    }
    for (auto& x : th) x.join();
    *dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (ma_status e : err)
        if (e != MA_OK) return e;
    return MA_OK;
}

static ma_status autotune(Ctx* c, const ma_problem* pb, int64_t count, ma_mem mem, const ma_solve_opts* o, int* best)
{
    const int cand[] = {4, 8, 16, 32, 64};
    const int kmax = 64;
    std::vector<int64_t> idx((size_t)count);
    for (int64_t i = 0; i < count; i++) idx[(size_t)i] = i;
    std::nth_element(idx.begin(), idx.begin() + count / 2, idx.end(),
                     [&](int64_t a, int64_t b) { return pb[a].n < pb[b].n; });
    const ma_problem& p = pb[idx[(size_t)(count / 2)]];
    ma_status st;
    if ((st = ensure_workers(c, kmax)) != MA_OK) return st;
    if (mem == MA_MEM_DEVICE)
        MA_CUDA(c, c->tune_w.ensure(sizeof(double) * (size_t)kmax * (size_t)p.n));
    else
        c->tune_wh.resize((size_t)kmax * (size_t)p.n);
    double dt = 0.0, best_rate = -1.0;
    if ((st = solve_copies(c, p, mem, o, kmax, &dt)) != MA_OK) return st;  // warm-up
    *best = 8;
    for (int K : cand) {
        for (int t = 0; t < kmax; t++) c->workers[(size_t)t]->grid_share = K;
        if ((st = solve_copies(c, p, mem, o, K, &dt)) != MA_OK) return st;
        const double rate = dt > 0 ? K / dt : 0.0;
        if (rate > best_rate) {
            best_rate = rate;
            *best = K;
        }
    }
    return MA_OK;
}

}  // namespace ma

using namespace ma;

extern "C" {

ma_status ma_ot_solve_batch(ma_ctx* cp, ma_problem* problems, int64_t count, ma_mem mem, const ma_solve_opts* opts,
                            int workers, int* workers_used)
{
    Ctx* c = cp;
    if (!c || (!problems && count > 0) || count < 0 || workers < 0 || workers > 64) return MA_ERR_INVALID_ARGUMENT;
    for (int64_t i = 0; i < count; i++) {
        const ma_problem& p = problems[i];
        if (!p.mesh || !p.x || !p.y || !p.nu || !p.w || p.n < 1) return MA_ERR_INVALID_ARGUMENT;
        if (p.mesh->ctx && p.mesh->ctx->device != c->device)
            return fail(c, MA_ERR_INVALID_ARGUMENT, "a problem's mesh lives on another device");
    }
    if (count == 0) return MA_OK;
    cudaSetDevice(c->device);
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    int k = workers > 0 ? workers : c->batch_workers;
    int64_t done = 0;
    ma_status st;
    std::vector<int64_t> order((size_t)count);
    for (int64_t i = 0; i < count; i++) order[(size_t)i] = i;
    if (k <= 0) {
        if ((st = autotune(c, problems, count, mem, opts, &k)) != MA_OK) return st;
        c->batch_workers = k;
    }
    if ((st = ensure_workers(c, k)) != MA_OK) return st;
    std::stable_sort(order.begin() + done, order.end(),
                     [&](int64_t a, int64_t b) { return problems[a].n > problems[b].n; });
    if (done < count && (st = run_chunk(c, problems, order, done, count, mem, opts, k)) != MA_OK) return st;
    if (workers_used) *workers_used = k;
    return MA_OK;
}

}  // extern "C"
