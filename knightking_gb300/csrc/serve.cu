/*
 * Serving: continuous batching of walk requests on resident tables.
 *
 * The server prepares once what every request of its app reads (sorted
 * adjacency, vertex type masks, alias tables kept with the engine's
 * alias_cache) and runs `slots` host threads, each driving one BatchSlot (its
 * own CUDA stream and buffers).  A free slot takes the requests queued so far,
 * first come first served, up to max_jobs and slot_bytes of walker paths and
 * state, and runs them as one walk_batch_kernel launch; so requests that
 * arrive while other batches are on the GPU start as soon as a slot frees up,
 * and the slots' kernels overlap on the device.  Each request's walkers are
 * keyed by its own seed and walker ids, so its paths are those of the request
 * run alone.
 */
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "knightking_gb300/engine.cuh"

using namespace kk;

namespace
{
typedef std::chrono::steady_clock Clock;

struct Request
{
    uint64_t ticket;
    kk_walk_opts opts;
    uint64_t bytes;
    Clock::time_point t_submit;
};

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

/* Device bytes of a request in a slot: each walker's path slots and length. */
uint64_t request_bytes(const kk_walk_opts &o)
{
    return (uint64_t)o.walker_num * (((uint64_t)o.walk_length + 1) * 4 + 4);
}

/* One job's paths in a pooled pinned block: lengths and vertices copied
 * straight from the slot's buffers on stream st (asynchronously: the caller
 * waits for st before reading them), offsets i * (walk_length + 1) written
 * here.  total_steps is set once the lengths have arrived (finish_paths). */
kk_paths *job_paths(HostPool *pool, const BatchJob &b, const uint32_t *d_len_all, const uint32_t *d_path,
                    cudaStream_t st)
{
    const uint32_t n = b.walker_num;
    const size_t len_bytes = ((size_t)n * 4 + 15) & ~(size_t)15;
    const size_t off_bytes = ((size_t)n * 8 + 15) & ~(size_t)15;
    const size_t vert_bytes = (size_t)n * b.cap * 4;
    kk_paths *p = (kk_paths *)calloc(1, sizeof(kk_paths));
    PooledPaths *o = new (std::nothrow) PooledPaths();
    size_t cls = 0;
    char *blk = (p && o) ? (char *)pool->get(len_bytes + off_bytes + vert_bytes + 16, &cls) : nullptr;
    if (!blk)
    {
        free(p);
        delete o;
        fail(KK_ERR_OOM, "host allocation failed");
    }
    o->pool = pool;
    o->block = blk;
    o->cls = cls;
    p->owner = o;
    p->walker_num = n;
    p->walker_begin = b.walker_begin;
    p->epoch_walkers = n;
    p->length = (uint32_t *)blk;
    p->offset = (uint64_t *)(blk + len_bytes);
    p->vertices = (uint32_t *)(blk + len_bytes + off_bytes);
    for (uint32_t i = 0; i < n; i++)
        p->offset[i] = (uint64_t)i * b.cap;
    if (n != 0)
    {
        cudaError_t err = cudaMemcpyAsync(p->length, d_len_all + b.first_task, (size_t)n * 4,
                                          cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(p->vertices, d_path + b.path_base, vert_bytes, cudaMemcpyDeviceToHost, st);
        if (err != cudaSuccess)
        {
            kk_paths_free(p);
            fail(KK_ERR_CUDA, std::string("path copy: ") + cudaGetErrorString(err));
        }
    }
    return p;
}

/* A job's paths once their copies are done: the walker-steps from the lengths. */
void finish_paths(kk_paths *p)
{
    uint64_t total = 0;
    for (uint32_t i = 0; i < p->walker_num; i++)
        total += p->length[i];
    p->total_steps = total - p->walker_num;
}

/* The status of a request from its walkers' status word. */
kk_status job_status_of(uint32_t word)
{
    if (word & KK_STATUS_TRIAL_LIMIT)
        return KK_ERR_TRIAL_LIMIT;
    if (word & KK_STATUS_PATH_CAPACITY)
        return KK_ERR_PATH_CAPACITY;
    return word ? KK_ERR_CUDA : KK_OK;
}

} // namespace

struct kk_server
{
    kk_engine *e = nullptr;
    kk_serve_opts o;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::unordered_map<uint64_t, kk_serve_result> done;
    std::unordered_set<uint64_t> pending; /* submitted, result not yet handed out */
    uint64_t next_ticket = 1;
    bool stopping = false;
    int prev_alias_cache = 0;
    std::vector<BatchSlot> slots;
    HostPool *pool = nullptr; /* pinned blocks of the results handed out */
    std::vector<std::thread> threads;
    /* statistics of completed requests */
    std::vector<double> latencies;
    uint64_t completed = 0, failed = 0, batches = 0, steps = 0, batch_jobs_sum = 0;
    double walk_ms = 0.0, copy_ms = 0.0, host_ms = 0.0;
};

namespace
{

/* Hands request j of a batch out (the caller holds s->m). */
void hand_out(kk_server *s, const Request &r, kk_status st, kk_paths *paths, Clock::time_point t_launch,
              Clock::time_point t_done, size_t n)
{
    kk_serve_result res;
    res.status = st;
    res.paths = st == KK_OK ? paths : nullptr;
    res.queue_ms = ms_between(r.t_submit, t_launch);
    res.latency_ms = ms_between(r.t_submit, t_done);
    res.batch_jobs = (uint32_t)n;
    s->done[r.ticket] = res;
    if (st == KK_OK)
    {
        s->completed++;
        s->latencies.push_back(res.latency_ms);
    }
    else
    {
        kk_paths_free(paths);
        s->failed++;
    }
}

/* A request whose paths are on their way to its pinned block. */
struct InFlight
{
    Request r;
    kk_status st;
    kk_paths *paths;
    cudaEvent_t ev; /* recorded on the slot's copy stream after its copies */
    Clock::time_point t_launch;
    size_t n; /* requests in its batch */
};

/* The status of a failure caught in a slot's loop. */
kk_status caught_status()
{
    try
    {
        throw;
    }
    catch (const Error &x)
    {
        return x.status;
    }
    catch (const std::bad_alloc &)
    {
        return KK_ERR_OOM;
    }
    catch (...)
    {
        return KK_ERR_CUDA;
    }
}

/* One slot's loop: take a batch of queued requests, launch it, and hand each
 * request out as soon as its own walkers have ended (its flag, raised by the
 * last of them with the request's status) and its paths have reached pinned
 * host memory, while the rest of the batch is still walking.  Once the last
 * request's copies are issued the slot takes its next batch: that walk waits
 * on the GPU for the copies (an event on the copy stream), and the requests
 * still in flight are handed out while it runs. */
void slot_loop(kk_server *s, int k)
{
    cudaSetDevice(s->e->device);
    BatchSlot &slot = s->slots[k];
    std::deque<InFlight> out;         /* copies issued, in issue order */
    std::vector<cudaEvent_t> free_ev; /* events of requests handed out */
    cudaEvent_t copies_ev = nullptr;  /* after the last copy issued */

    auto new_event = [&]() {
        if (!free_ev.empty())
        {
            cudaEvent_t ev = free_ev.back();
            free_ev.pop_back();
            return ev;
        }
        cudaEvent_t ev = nullptr;
        KK_CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        slot.job_ev.push_back(ev); /* destroyed with the slot */
        return ev;
    };
    /* hands out the requests whose copies are done, in issue order */
    auto hand_out_ready = [&]() {
        size_t ready = 0;
        while (ready < out.size())
        {
            const cudaError_t q = cudaEventQuery(out[ready].ev);
            if (q == cudaErrorNotReady)
                break;
            KK_CUDA_CHECK(q);
            ready++;
        }
        if (ready == 0)
            return false;
        const Clock::time_point t_done = Clock::now();
        for (size_t x = 0; x < ready; x++)
            finish_paths(out[x].paths);
        {
            std::lock_guard<std::mutex> lk(s->m);
            for (size_t x = 0; x < ready; x++)
            {
                InFlight &f = out.front();
                if (f.st == KK_OK)
                    s->steps += f.paths->total_steps;
                hand_out(s, f.r, f.st, f.paths, f.t_launch, t_done, f.n);
                free_ev.push_back(f.ev);
                out.pop_front();
            }
        }
        s->cv_done.notify_all();
        return true;
    };
    /* after a failure: the requests in flight go out once their copies have
     * landed, with their own status if the copies did, else with st */
    auto drain_after_failure = [&](kk_status st) {
        const bool copied = slot.copy == nullptr || cudaStreamSynchronize(slot.copy) == cudaSuccess;
        const Clock::time_point t_done = Clock::now();
        std::lock_guard<std::mutex> lk(s->m);
        for (InFlight &f : out)
        {
            if (copied)
                finish_paths(f.paths);
            hand_out(s, f.r, copied ? f.st : st, f.paths, f.t_launch, t_done, f.n);
            free_ev.push_back(f.ev);
        }
        out.clear();
    };

    for (;;)
    {
        std::vector<Request> batch;
        try
        {
            std::unique_lock<std::mutex> lk(s->m);
            for (;;)
            {
                if (!s->queue.empty())
                    break;
                if (out.empty())
                {
                    s->cv_work.wait(lk, [&] { return s->stopping || !s->queue.empty(); });
                    if (s->queue.empty())
                        return; /* stopping, queue drained, nothing in flight */
                    break;
                }
                /* requests in flight: hand them out while waiting for work */
                lk.unlock();
                if (!hand_out_ready())
                    std::this_thread::yield();
                lk.lock();
            }
            uint64_t bytes = 0;
            while (!s->queue.empty() && batch.size() < s->o.max_jobs)
            {
                const Request &r = s->queue.front();
                if (!batch.empty() && bytes + r.bytes > s->o.slot_bytes)
                    break;
                bytes += r.bytes;
                batch.push_back(r);
                s->queue.pop_front();
            }
        }
        catch (...)
        {
            drain_after_failure(caught_status());
            s->cv_done.notify_all();
            continue;
        }
        const Clock::time_point t_launch = Clock::now();
        const size_t n = batch.size();
        std::vector<kk_walk_opts> jobs(n);
        for (size_t j = 0; j < n; j++)
            jobs[j] = batch[j].opts;
        std::vector<char> issued(n, 0);
        kk_status st = KK_OK;
        Clock::time_point t_walked = t_launch, t_copied = t_launch;
        try
        {
            /* in arrival order: a request is handed out as soon as it ends,
             * and the long ones of the batch need not all start first */
            BatchPlan plan = plan_batch(s->e, jobs.data(), (int)n, false);
            /* every flag of the slot's previous batch has been read: no
             * walker of it writes one any more */
            volatile uint32_t *flag = slot.h_flag;
            for (size_t j = 0; j < n; j++)
                flag[j] = 0;
            /* the walk overwrites the slot's buffers the previous batch's
             * copies read from */
            if (copies_ev != nullptr)
                KK_CUDA_CHECK(cudaStreamWaitEvent(slot.stream, copies_ev, 0));
            batch_launch_async(s->e, plan, slot);
            size_t n_issued = 0;
            bool walked = false;
            while (n_issued < n)
            {
                if (!walked)
                {
                    const cudaError_t q = cudaEventQuery(slot.ev[2]);
                    if (q == cudaSuccess)
                    {
                        walked = true;
                        t_walked = Clock::now();
                    }
                    else if (q != cudaErrorNotReady)
                    {
                        KK_CUDA_CHECK(q);
                    }
                }
                bool any = false;
                for (size_t j = 0; j < n && n_issued < n; j++)
                {
                    if (issued[j])
                        continue;
                    /* a request of no walkers has nothing to walk */
                    const uint32_t f = plan.jobs[j].walker_num == 0 ? 1u : flag[j];
                    if (f == 0)
                    {
                        /* the batch has ended and visibly so: a request whose
                         * walkers never all counted themselves done */
                        if (walked && flag[j] == 0)
                            fail(KK_ERR_CUDA, "a request of the batch did not complete");
                        continue;
                    }
                    kk_paths *pj = job_paths(s->pool, plan.jobs[j], (const uint32_t *)slot.length.p,
                                             (const uint32_t *)slot.path.p, slot.copy);
                    cudaEvent_t ev = nullptr;
                    try
                    {
                        ev = new_event();
                        out.push_back(InFlight{batch[j], job_status_of(f - 1), pj, ev, t_launch, n});
                    }
                    catch (...)
                    {
                        cudaStreamSynchronize(slot.copy);
                        kk_paths_free(pj);
                        throw;
                    }
                    issued[j] = 1;
                    n_issued++;
                    KK_CUDA_CHECK(cudaEventRecord(ev, slot.copy));
                    any = true;
                }
                if (hand_out_ready())
                    any = true;
                if (!any)
                {
                    /* the slot's thread polls while its batch is on the GPU
                     * (a core per busy slot), so a finished request is seen
                     * within microseconds rather than a timer tick */
                    std::this_thread::yield();
                }
            }
            if (copies_ev == nullptr)
                copies_ev = new_event();
            KK_CUDA_CHECK(cudaEventRecord(copies_ev, slot.copy));
            /* nothing of this batch is read back: its last blocks leave the
             * GPU ahead of the slot's next walk on the same stream (a fault
             * would surface at that launch or its event) */
            t_copied = Clock::now();
        }
        catch (...)
        {
            st = caught_status();
        }
        if (st != KK_OK)
        {
            /* copies in flight land in blocks about to go back to the pool */
            drain_after_failure(st);
            cudaStreamSynchronize(slot.stream);
        }
        const Clock::time_point t_done = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->m);
            for (size_t j = 0; j < n; j++)
                if (!issued[j])
                    hand_out(s, batch[j], st, nullptr, t_launch, t_done, n);
            s->batches++;
            s->batch_jobs_sum += n;
            s->walk_ms += ms_between(t_launch, t_walked);
            s->copy_ms += ms_between(t_walked, t_copied);
            s->host_ms += ms_between(t_copied, t_done);
        }
        s->cv_done.notify_all();
    }
}

} // namespace

extern "C" {

kk_status kk_serve_start(kk_engine *e, const kk_serve_opts *opts, kk_server **out)
{
    if (!e || !opts || !out)
        return KK_ERR_INVALID_CONFIG;
    *out = nullptr;
    kk_server *s = new (std::nothrow) kk_server();
    if (!s)
        return KK_ERR_OOM;
    kk_status st = guard(e, [&] {
        require_graph(e);
        kk_serve_opts o = *opts;
        if (o.app != KK_APP_DEEPWALK && o.app != KK_APP_NODE2VEC && o.app != KK_APP_METAPATH)
            fail(KK_ERR_INVALID_CONFIG, "the server runs DeepWalk, node2vec or metapath requests");
        if (o.weighted && e->d_w == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "weighted server on a graph without weights");
        if (o.app == KK_APP_METAPATH && e->d_type == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "metapath needs edge types");
        if (o.slots == 0)
            o.slots = 2;
        if (o.max_jobs == 0)
            o.max_jobs = 256;
        if (o.slot_bytes == 0)
            o.slot_bytes = 1ull << 30;
        if (o.slots < 1 || o.slots > 8 || o.max_jobs > kMaxBatchJobs || o.launch_mode < 0 || o.launch_mode > 1)
            fail(KK_ERR_INVALID_CONFIG, "slots 1..8, max_jobs 1..1024, launch_mode 0 or 1");
        s->e = e;
        s->o = o;
        /* resident tables, built once on the engine's stream */
        s->prev_alias_cache = e->alias_cache;
        e->alias_cache = 1;
        BatchPlan plan;
        plan.app = o.app;
        plan.weighted = o.weighted != 0;
        batch_prepare(e, plan);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        s->slots.resize(o.slots);
        for (int k = 0; k < o.slots; k++)
        {
            KK_CUDA_CHECK(cudaStreamCreateWithFlags(&s->slots[k].stream, cudaStreamNonBlocking));
            if (o.launch_mode == 0)
                batch_slot_graph_mode(e, s->slots[k], (uint32_t)std::min<uint64_t>(o.slot_bytes / 8, 0x80000000ull),
                                      o.slot_bytes / 4);
            batch_slot_notify_mode(s->slots[k]);
        }
        s->pool = new HostPool();
        s->pool->limit = (size_t)o.slots * 2 * o.slot_bytes;
        for (int k = 0; k < o.slots; k++)
            s->threads.emplace_back(slot_loop, s, k);
    });
    if (st != KK_OK)
    {
        if (s->e)
            e->alias_cache = s->prev_alias_cache;
        for (BatchSlot &sl : s->slots)
        {
            if (sl.stream)
                cudaStreamDestroy(sl.stream);
            sl.release();
        }
        if (s->pool)
            s->pool->release();
        delete s;
        return st;
    }
    *out = s;
    return KK_OK;
}

kk_status kk_serve_submit(kk_server *s, const kk_walk_opts *req, uint64_t *ticket)
{
    if (!s || !req || !ticket)
        return KK_ERR_INVALID_CONFIG;
    if (req->app != s->o.app || (req->weighted != 0) != (s->o.weighted != 0))
        return KK_ERR_INVALID_CONFIG;
    if (req->start != nullptr || (req->rate != 0.0 && req->rate != 1.0))
        return KK_ERR_INVALID_CONFIG;
    if ((uint64_t)req->walker_begin + req->walker_num > 0x100000000ULL || req->walker_num > 0x80000000u ||
        req->walk_length >= 0xfffffff0u)
        return KK_ERR_INVALID_CONFIG;
    if (req->app == KK_APP_NODE2VEC && !(req->p > 0.0f && req->q > 0.0f))
        return KK_ERR_INVALID_CONFIG;
    if (req->app == KK_APP_METAPATH)
    {
        if (req->n_schemes < 1 || req->n_schemes > KK_MAX_SCHEMES)
            return KK_ERR_INVALID_CONFIG;
        for (int i = 0; i < req->n_schemes; i++)
            if (req->scheme_len[i] < 1 || req->scheme_len[i] > KK_MAX_SCHEME_LEN)
                return KK_ERR_INVALID_CONFIG;
    }
    Request r;
    r.opts = *req;
    r.bytes = request_bytes(*req);
    if (r.bytes > s->o.slot_bytes)
        return KK_ERR_INVALID_CONFIG;
    r.t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->m);
        if (s->stopping)
            return KK_ERR_INVALID_CONFIG;
        r.ticket = s->next_ticket++;
        s->queue.push_back(r);
        s->pending.insert(r.ticket);
    }
    *ticket = r.ticket;
    s->cv_work.notify_one();
    return KK_OK;
}

kk_status kk_serve_poll(kk_server *s, uint64_t ticket, int timeout_ms, kk_serve_result *out)
{
    if (!s || !out || ticket == 0)
        return KK_ERR_INVALID_CONFIG;
    std::unique_lock<std::mutex> lk(s->m);
    if (s->pending.count(ticket) == 0)
        return KK_ERR_INVALID_CONFIG; /* never submitted, or already handed out */
    auto ready = [&] { return s->done.count(ticket) != 0; };
    if (timeout_ms < 0)
        s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return KK_ERR_TIMEOUT;
    *out = s->done[ticket];
    s->done.erase(ticket);
    s->pending.erase(ticket);
    return KK_OK;
}

kk_status kk_serve_stats_get(kk_server *s, kk_serve_stats *out)
{
    if (!s || !out)
        return KK_ERR_INVALID_CONFIG;
    std::lock_guard<std::mutex> lk(s->m);
    memset(out, 0, sizeof(*out));
    out->completed = s->completed;
    out->failed = s->failed;
    out->batches = s->batches;
    out->walker_steps = s->steps;
    out->mean_batch_jobs = s->batches ? (double)s->batch_jobs_sum / (double)s->batches : 0.0;
    out->walk_ms = s->walk_ms;
    out->copy_ms = s->copy_ms;
    out->host_ms = s->host_ms;
    if (!s->latencies.empty())
    {
        std::vector<double> l = s->latencies;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) {
            size_t i = (size_t)(q * (double)(l.size() - 1) + 0.5);
            return l[i < l.size() ? i : l.size() - 1];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double sum = 0.0;
        for (double x : l)
            sum += x;
        out->mean_ms = sum / (double)l.size();
    }
    return KK_OK;
}

kk_status kk_serve_stats_reset(kk_server *s)
{
    if (!s)
        return KK_ERR_INVALID_CONFIG;
    std::lock_guard<std::mutex> lk(s->m);
    s->latencies.clear();
    s->completed = s->failed = s->batches = s->steps = s->batch_jobs_sum = 0;
    s->walk_ms = s->copy_ms = s->host_ms = 0.0;
    return KK_OK;
}

kk_status kk_serve_replay(kk_server *s, const kk_walk_opts *reqs, const double *arrival_s, uint32_t n,
                          double *latency_ms, uint64_t *total_steps, double *elapsed_s)
{
    if (!s || !reqs || !arrival_s || n == 0)
        return KK_ERR_INVALID_CONFIG;
    for (uint32_t i = 1; i < n; i++)
        if (!(arrival_s[i] >= arrival_s[i - 1]))
            return KK_ERR_INVALID_CONFIG;
    std::vector<uint64_t> tickets(n, 0);
    std::mutex m;
    std::condition_variable cv;
    uint32_t n_sub = 0;      /* tickets[0, n_sub) are valid */
    bool sub_done = false;   /* no more submissions */
    kk_status sub_st = KK_OK, res_st = KK_OK;
    uint64_t steps = 0;
    const Clock::time_point t0 = Clock::now();
    std::thread poller([&] {
        for (uint32_t i = 0;; i++)
        {
            {
                std::unique_lock<std::mutex> lk(m);
                cv.wait(lk, [&] { return i < n_sub || sub_done; });
                if (i >= n_sub)
                    return;
            }
            kk_serve_result r;
            const kk_status st = kk_serve_poll(s, tickets[i], -1, &r);
            if (st != KK_OK || r.status != KK_OK)
            {
                if (res_st == KK_OK)
                    res_st = st != KK_OK ? st : r.status;
                if (latency_ms)
                    latency_ms[i] = -1.0;
            }
            else if (latency_ms)
            {
                latency_ms[i] = r.latency_ms;
            }
            if (st == KK_OK && r.paths)
            {
                steps += r.paths->total_steps;
                kk_paths_free(r.paths);
            }
        }
    });
    for (uint32_t i = 0; i < n; i++)
    {
        /* sleep until shortly before the arrival, then spin to it */
        const Clock::time_point due =
            t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
        if (due - Clock::now() > std::chrono::microseconds(200))
            std::this_thread::sleep_until(due - std::chrono::microseconds(100));
        while (Clock::now() < due)
        {
        }
        const kk_status st = kk_serve_submit(s, &reqs[i], &tickets[i]);
        if (st != KK_OK)
        {
            sub_st = st;
            if (latency_ms)
                for (uint32_t j = i; j < n; j++)
                    latency_ms[j] = -1.0;
            break;
        }
        {
            std::lock_guard<std::mutex> lk(m);
            n_sub = i + 1;
        }
        cv.notify_one();
    }
    {
        std::lock_guard<std::mutex> lk(m);
        sub_done = true;
    }
    cv.notify_one();
    poller.join();
    if (total_steps)
        *total_steps = steps;
    if (elapsed_s)
        *elapsed_s = std::chrono::duration<double>(Clock::now() - t0).count();
    return sub_st != KK_OK ? sub_st : res_st;
}

kk_status kk_serve_stop(kk_server *s)
{
    if (!s)
        return KK_ERR_INVALID_CONFIG;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (std::thread &t : s->threads)
        t.join();
    for (BatchSlot &sl : s->slots)
    {
        if (sl.stream)
        {
            cudaStreamSynchronize(sl.stream);
            cudaStreamDestroy(sl.stream);
        }
        sl.release();
    }
    for (auto &kv : s->done)
        kk_paths_free(kv.second.paths);
    s->pool->release();
    s->e->alias_cache = s->prev_alias_cache;
    delete s;
    return KK_OK;
}

} /* extern "C" */
