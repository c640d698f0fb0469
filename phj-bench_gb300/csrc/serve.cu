// serve.cu -- a request loop over the join path: admission by estimated HBM
// footprint, a fixed number of execution slots (one stream each), and
// continuous batching of small requests into shared launches.
//
// Requests arrive over time (each carries its arrival offset).  A dispatcher
// thread moves arrived requests into a FIFO ready queue and hands work to
// idle slots: the oldest request alone if it is large, or, if it is small,
// up to `batch_max_joins` small ready requests that fit the budget, run
// through phj_batch_run.  A request is admitted only while the summed
// footprint of the requests in flight stays within `hbm_budget_bytes` (a
// request larger than the whole budget runs when nothing else is in flight).
// Each slot owns a phj_ctx (stream + memory pool) and a worker thread that
// generates the request's inputs on the device, joins, fingerprints the
// output and frees everything, then records the request's times.
//
// With one slot and batching off this is the plain form: one join per call,
// in arrival order.
#include "internal.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

struct phj_server
{
    phj_serve_config cfg{};
    std::mutex mu;
    std::condition_variable cv;      // dispatcher wake-ups
    std::condition_variable done_cv; // waiters for completion
    std::vector<phj_serve_request> reqs;
    std::vector<phj_serve_record> recs;
    std::vector<uint64_t> footprint;
    std::vector<uint64_t> arrival_order; // request ids sorted by arrival
    size_t next_arrival = 0;
    std::deque<uint64_t> ready;
    uint64_t inflight_bytes = 0;
    uint32_t inflight_requests = 0;
    uint64_t completed = 0;
    bool started = false, stop = false;
    std::chrono::steady_clock::time_point t0;
    struct Slot
    {
        phj_ctx * ctx = nullptr;
        std::vector<uint64_t> job;
        bool busy = false;
        std::thread th;
    };
    std::vector<Slot> slots;
    std::thread dispatcher;
    std::string error;

    double now_s() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace phjg
{
namespace
{
uint64_t side_row_bytes(const phj_schema & s)
{
    return 8 + schema_bytes(s);
}

// Estimated device bytes a request holds while it runs: its inputs, the
// table (cells at load <= 1/2 plus the next-chain), the partition buffers of
// a join run alone (both sides' shuffles) or the partitioned copies of a
// batched one, and an output of one row per probe row.
uint64_t estimate_footprint(const phj_serve_request & r, bool batched)
{
    const uint64_t B = r.build.rows, P = r.probe.rows;
    const uint64_t rb = side_row_bytes(r.build.schema), rp = side_row_bytes(r.probe.schema);
    const uint64_t cells = B ? bit_ceil64(2 * B) : 1;
    const uint64_t in = B * rb + P * rp;
    const uint64_t table = cells * 16 + B * 8;
    const uint64_t buffers = batched ? B * rb + P * rp : 2 * B * rb + P * rp + P * 4;
    const uint64_t out = P * (rb + rp - 8);
    return in + table + buffers + out;
}

bool is_small(const phj_server & s, uint64_t id)
{
    return s.cfg.batch_max_build_rows > 0 && s.cfg.batch_max_joins > 1 && s.reqs[id].build.rows <= s.cfg.batch_max_build_rows;
}

void run_job(phj_server & S, uint32_t slot, const std::vector<uint64_t> & job)
{
    phj_ctx * ctx = S.slots[slot].ctx;
    DeviceScope dev(ctx); // this worker thread's CUDA calls go to the slot's device
    const double t_start = S.now_s();
    const size_t n = job.size();
    std::vector<phj_table *> b(n, nullptr), p(n, nullptr);
    std::vector<phj_output *> o(n, nullptr);
    std::vector<int32_t> st(n, PHJ_OK);
    std::vector<std::array<uint64_t, 3>> fp(n, {0, 0, 0});
    phj_status s = PHJ_OK;
    for (size_t i = 0; i < n && s == PHJ_OK; ++i)
    {
        s = phj_table_generate(ctx, &S.reqs[job[i]].build, &b[i]);
        if (s == PHJ_OK)
            s = phj_table_generate(ctx, &S.reqs[job[i]].probe, &p[i]);
    }
    if (s == PHJ_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        s = PHJ_ERR_CUDA;
    const double t_gen = S.now_s();
    double device_ms = 0.0;
    if (s == PHJ_OK)
    {
        if (n == 1)
        {
            uint8_t bits[8];
            uint32_t np = S.cfg.n_passes;
            std::copy(S.cfg.pass_bits, S.cfg.pass_bits + 8, bits);
            if (np == 0)
                phj_autotune_radix(S.reqs[job[0]].build.rows, S.reqs[job[0]].probe.rows, bits, &np);
            phj_phj_result r{};
            s = phj_run_phj_pure(ctx, b[0], p[0], bits, np, &o[0], &r);
            device_ms = r.e2e_wall_ms;
        }
        else
        {
            phj_batch_result r{};
            s = phj_batch_run(ctx, (uint32_t)n, b.data(), p.data(), o.data(), &r);
            device_ms = r.e2e_wall_ms;
        }
    }
    const double t_call = S.now_s();
    const uint64_t job_peak = ctx->peak_bytes; // the scheme run's peak, inputs and outputs included
    for (size_t i = 0; i < n; ++i)
    {
        if (s == PHJ_OK && o[i])
            st[i] = phj_output_fingerprint(ctx, o[i], fp[i].data());
        else
            st[i] = s;
        phj_output_free(ctx, o[i]);
        phj_table_free(ctx, b[i]);
        phj_table_free(ctx, p[i]);
    }
    cudaStreamSynchronize(ctx->stream);
    const double t_done = S.now_s();
    std::lock_guard<std::mutex> lock(S.mu);
    for (size_t i = 0; i < n; ++i)
    {
        phj_serve_record & r = S.recs[job[i]];
        r.start_s = t_start;
        r.done_s = t_done;
        r.status = st[i];
        r.batch_size = (uint32_t)n;
        r.slot = slot;
        for (int k = 0; k < 3; ++k)
            r.fingerprint[k] = fp[i][k];
        r.output_rows = fp[i][0];
        r.job_peak_bytes = job_peak;
        r.gen_s = (t_gen - t_start) / (double)n;
        r.call_s = (t_call - t_gen) / (double)n;
        r.device_ms = device_ms / (double)n;
        S.inflight_bytes -= S.footprint[job[i]];
        S.inflight_requests -= 1;
        ++S.completed;
        if (st[i] != PHJ_OK && S.error.empty())
            S.error = std::string("request ") + std::to_string(job[i]) + ": " + phj_last_error(ctx);
    }
    S.slots[slot].busy = false;
    S.cv.notify_all();
    S.done_cv.notify_all();
}

void worker_loop(phj_server * S, uint32_t slot)
{
    std::unique_lock<std::mutex> lock(S->mu);
    for (;;)
    {
        S->cv.wait(lock, [&] { return S->stop || !S->slots[slot].job.empty(); });
        if (S->slots[slot].job.empty() && S->stop)
            return;
        std::vector<uint64_t> job;
        job.swap(S->slots[slot].job);
        lock.unlock();
        run_job(*S, slot, job);
        lock.lock();
    }
}

// Picks work for an idle slot from the ready queue (lock held).  Returns the
// request ids, empty if nothing can be admitted now.
std::vector<uint64_t> pick(phj_server & S)
{
    std::vector<uint64_t> job;
    if (S.ready.empty())
        return job;
    const uint64_t head = S.ready.front();
    auto fits = [&](uint64_t bytes) { return S.inflight_requests == 0 || S.inflight_bytes + bytes <= S.cfg.hbm_budget_bytes; };
    if (!is_small(S, head))
    {
        if (!fits(S.footprint[head]))
            return job;
        job.push_back(head);
        S.ready.pop_front();
        return job;
    }
    // continuous batching: every small ready request that fits, oldest first
    // (a batch holds fewer than 2^31 rows on each side)
    uint64_t bytes = 0, brows = 0, prows = 0;
    const uint64_t row_cap = 1ull << 31;
    for (auto it = S.ready.begin(); it != S.ready.end() && job.size() < S.cfg.batch_max_joins;)
    {
        const uint64_t id = *it;
        const bool rows_fit = job.empty() || (brows + S.reqs[id].build.rows < row_cap && prows + S.reqs[id].probe.rows < row_cap);
        if (is_small(S, id) && rows_fit &&
            (job.empty() ? fits(S.footprint[id]) : S.inflight_bytes + bytes + S.footprint[id] <= S.cfg.hbm_budget_bytes))
        {
            job.push_back(id);
            bytes += S.footprint[id];
            brows += S.reqs[id].build.rows;
            prows += S.reqs[id].probe.rows;
            it = S.ready.erase(it);
        }
        else if (!is_small(S, id))
            break; // keep arrival order behind a waiting large request
        else
            ++it;
    }
    return job;
}

void dispatcher_loop(phj_server * S)
{
    std::unique_lock<std::mutex> lock(S->mu);
    while (!S->stop)
    {
        const double now = S->now_s();
        while (S->next_arrival < S->arrival_order.size() && S->reqs[S->arrival_order[S->next_arrival]].arrival_s <= now)
        {
            const uint64_t id = S->arrival_order[S->next_arrival++];
            S->ready.push_back(id);
        }
        bool assigned = false;
        for (uint32_t k = 0; k < S->slots.size() && !S->ready.empty(); ++k)
        {
            if (S->slots[k].busy)
                continue;
            std::vector<uint64_t> job = pick(*S);
            if (job.empty())
                break;
            for (uint64_t id : job)
            {
                S->recs[id].admit_s = now;
                S->inflight_bytes += S->footprint[id];
                S->inflight_requests += 1;
            }
            S->slots[k].busy = true;
            S->slots[k].job = std::move(job);
            assigned = true;
        }
        if (assigned)
        {
            S->cv.notify_all();
            continue;
        }
        // sleep until the next arrival or a completion
        if (S->next_arrival < S->arrival_order.size())
        {
            const double dt = S->reqs[S->arrival_order[S->next_arrival]].arrival_s - now;
            S->cv.wait_for(lock, std::chrono::duration<double>(std::max(0.0, std::min(dt, 0.01))));
        }
        else
            S->cv.wait_for(lock, std::chrono::milliseconds(10));
    }
}
} // namespace
} // namespace phjg

using namespace phjg;

extern "C" {

phj_status phj_serve_create(const phj_serve_config * cfg, phj_server ** out)
{
    if (!cfg || !out || cfg->workers == 0 || cfg->workers > 64 || cfg->n_passes > 8)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    phj_server * S = new phj_server();
    S->cfg = *cfg;
    S->slots.resize(cfg->workers);
    for (uint32_t k = 0; k < cfg->workers; ++k)
    {
        const phj_status st = phj_ctx_create(cfg->device, &S->slots[k].ctx);
        if (st != PHJ_OK)
        {
            for (auto & sl : S->slots)
                if (sl.ctx)
                    phj_ctx_destroy(sl.ctx);
            delete S;
            return st;
        }
        phj_ctx_set_int(S->slots[k].ctx, "time_kernels", 0);
    }
    *out = S;
    return PHJ_OK;
}

phj_status phj_serve_submit(phj_server * S, const phj_serve_request * r, uint64_t * id)
{
    if (!S || !r)
        return PHJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->started)
        return PHJ_ERR_INVALID_ARGUMENT; // the trace is fixed before the clock starts
    const uint64_t k = S->reqs.size();
    S->reqs.push_back(*r);
    phj_serve_record rec{};
    rec.id = k;
    rec.arrival_s = r->arrival_s;
    rec.build_rows = r->build.rows;
    rec.probe_rows = r->probe.rows;
    rec.status = -1;
    S->recs.push_back(rec);
    const bool small = S->cfg.batch_max_build_rows > 0 && S->cfg.batch_max_joins > 1 && r->build.rows <= S->cfg.batch_max_build_rows;
    S->footprint.push_back(estimate_footprint(*r, small));
    S->recs.back().footprint_bytes = S->footprint.back();
    if (id)
        *id = k;
    return PHJ_OK;
}

phj_status phj_serve_start(phj_server * S)
{
    if (!S)
        return PHJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->started)
        return PHJ_ERR_INVALID_ARGUMENT;
    S->arrival_order.resize(S->reqs.size());
    for (uint64_t i = 0; i < S->reqs.size(); ++i)
        S->arrival_order[i] = i;
    std::stable_sort(S->arrival_order.begin(), S->arrival_order.end(),
                     [&](uint64_t a, uint64_t b) { return S->reqs[a].arrival_s < S->reqs[b].arrival_s; });
    S->started = true;
    S->t0 = std::chrono::steady_clock::now();
    for (uint32_t k = 0; k < S->slots.size(); ++k)
        S->slots[k].th = std::thread(worker_loop, S, k);
    S->dispatcher = std::thread(dispatcher_loop, S);
    return PHJ_OK;
}

phj_status phj_serve_wait(phj_server * S, double timeout_s)
{
    if (!S)
        return PHJ_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lock(S->mu);
    const bool ok = S->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] { return S->completed == S->reqs.size(); });
    if (!ok)
        return PHJ_ERR_DEVICE_TIMEOUT;
    return S->error.empty() ? PHJ_OK : PHJ_ERR_CUDA;
}

uint32_t phj_serve_records(phj_server * S, phj_serve_record * out, uint32_t cap)
{
    if (!S)
        return 0;
    std::lock_guard<std::mutex> lock(S->mu);
    const uint32_t n = (uint32_t)std::min<size_t>(cap, S->recs.size());
    for (uint32_t i = 0; i < n && out; ++i)
        out[i] = S->recs[i];
    return (uint32_t)S->recs.size();
}

const char * phj_serve_error(const phj_server * S)
{
    return S ? S->error.c_str() : "";
}

void phj_serve_destroy(phj_server * S)
{
    if (!S)
        return;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->dispatcher.joinable())
        S->dispatcher.join();
    for (auto & sl : S->slots)
        if (sl.th.joinable())
            sl.th.join();
    for (auto & sl : S->slots)
        phj_ctx_destroy(sl.ctx);
    delete S;
}

uint64_t phj_serve_footprint(const phj_serve_request * r, int batched)
{
    return r ? estimate_footprint(*r, batched != 0) : 0;
}

} // extern "C"
