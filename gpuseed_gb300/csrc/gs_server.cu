/*
 * gs_server.cu -- serving loop with continuous batching.
 *
 * The reference seeds one file batch after another on the default stream
 * (seed_gen.cu:2910-3790).  Here requests (read sets of any size) arrive at
 * any time; the index stays resident; n_slots worker threads each own a
 * context (stream + workspace).  Whenever a slot is free it takes every
 * pending request that fits -- in arrival order, up to max_batch_reads reads
 * and within the HBM budget -- merges them into one pass, runs it, and hands
 * each request its own seeds back.  Passes of different slots overlap on the
 * device, so a request that arrives while others run is admitted as soon as
 * a slot and memory free up, not after a whole queue drains.
 *
 * Results do not depend on the company a request keeps: every read's seeds
 * depend on that read alone (the per-read semantics of gs_post.cu), and a
 * request's reads come back in its own order.
 */
#include "gs_internal.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string.h>
#include <thread>
#include <unordered_map>
#include <vector>

extern "C" int gs_index_get_info(const gs_index *idx, gs_index_info *out);
int gs_index_device(const gs_index *idx);

namespace {

double now_ms()
{
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Req {
    uint64_t id;
    std::vector<char> seqs;
    const char *ext;            /* gs_server_submit_ref: the caller's bases, in place */
    std::vector<uint64_t> offs;
    std::vector<uint32_t> lens;
    uint64_t bases;
    uint64_t est_bytes;
    double t_submit, t_start, t_done;
    int status;
    bool done;
    std::vector<uint64_t> seed_off, pos_off;
    std::vector<gs_seed_rec> seeds;
    std::vector<uint32_t> pos;
};

/* device bytes one pass needs per base and per read: slots (2 x 16 B per
 * start position) and their record bitmap, the batched search's walker
 * buffer (16 entries of 24 B per work item of 31 start positions, about
 * 25 B per base and 0.8 KB per read), per-read counters, outputs (a few seeds
 * and positions per read) */
inline uint64_t estimate_bytes(uint64_t bases, uint64_t reads)
{
    return bases * 64 + reads * 1024 + (4u << 20);
}

}  // namespace

struct gs_server {
    gs_index *idx;
    gs_server_opts opts;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> pending;
    std::unordered_map<uint64_t, Req *> reqs;
    /* released requests, kept with their buffers' capacity for the next
     * submissions: copying into memory that was written before costs no page
     * faults, which otherwise dominate copying requests in and seeds out */
    std::vector<Req *> spare;
    std::vector<std::thread> workers;
    bool stopping;
    uint64_t next_id;
    uint64_t reserved, budget;
    gs_server_stats stats;
    int start_error;
};

static void fail_request(gs_server *s, Req *r, int code)
{
    r->status = code;
    r->done = true;
    r->t_done = now_ms();
    s->stats.failed++;
}

static void worker_main(gs_server *s, int slot)
{
    (void)slot;
    cudaSetDevice(gs_index_device(s->idx));
    gs_ctx *ctx = NULL;
    int rc = gs_ctx_create(s->idx, NULL, &ctx);
    if (rc) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->start_error = rc;
        s->cv_done.notify_all();
        return;
    }
    /* merged batch in pinned host memory: the H2D copy runs at link speed */
    char *seqs = NULL;
    uint64_t *offs = NULL;
    uint32_t *lens = NULL;
    size_t cap_b = 0, cap_r = 0;
    std::vector<Req *> batch;
    for (;;) {
        uint64_t est = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stopping || !s->pending.empty(); });
            if (s->stopping && s->pending.empty()) break;
            batch.clear();
            uint64_t reads = 0, bases = 0;
            while (!s->pending.empty()) {
                Req *r = s->pending.front();
                uint64_t nr = reads + r->lens.size(), nb = bases + r->bases;
                uint64_t e = estimate_bytes(nb, nr);
                if (!batch.empty() &&
                    (nr > (uint64_t)s->opts.max_batch_reads || s->reserved + e > s->budget))
                    break;
                if (batch.empty() && s->reserved + e > s->budget) {
                    if (s->reserved == 0) {
                        /* cannot fit even alone on an idle device */
                        s->pending.pop_front();
                        fail_request(s, r, GS_ENOMEM);
                        s->cv_done.notify_all();
                        continue;
                    }
                    break;   /* wait for memory to free up */
                }
                s->pending.pop_front();
                batch.push_back(r);
                reads = nr;
                bases = nb;
                est = e;
            }
            if (batch.empty()) {
                /* memory is held by other slots: wait for a completion */
                s->cv_done.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
            s->reserved += est;
        }
        /* merge the requests into one pass */
        uint64_t nb = 0, nr = 0;
        for (Req *r : batch) {
            nb += r->bases;
            nr += r->lens.size();
        }
        rc = GS_OK;
        if (nb + 1 > cap_b) {
            cudaFreeHost(seqs);
            cap_b = nb + nb / 2 + 4096;
            if (cudaMallocHost(&seqs, cap_b) != cudaSuccess) { seqs = NULL; cap_b = 0; rc = GS_ENOMEM; }
        }
        if (nr + 1 > cap_r) {
            cudaFreeHost(offs);
            cudaFreeHost(lens);
            cap_r = nr + nr / 2 + 256;
            if (cudaMallocHost(&offs, cap_r * 8) != cudaSuccess ||
                cudaMallocHost(&lens, cap_r * 4) != cudaSuccess) {
                offs = NULL; lens = NULL; cap_r = 0; rc = GS_ENOMEM;
            }
        }
        double t0 = now_ms();
        uint64_t wb = 0, wr = 0;
        double t_merged = 0, t_seeded = 0, t_split = 0;
        if (rc == GS_OK)
            for (Req *r : batch) {
                r->t_start = t0;
                memcpy(seqs + wb, r->ext ? r->ext : r->seqs.data(), r->bases);
                for (size_t i = 0; i < r->lens.size(); i++) {
                    offs[wr] = wb + r->offs[i];
                    lens[wr] = r->lens[i];
                    wr++;
                }
                wb += r->bases;
            }
        t_merged = now_ms();
        if (rc == GS_OK) rc = gs_seed(ctx, seqs, offs, lens, (uint32_t)nr, &s->opts.params);
        t_seeded = now_ms();
        gs_result_view v;
        if (rc == GS_OK) rc = gs_result_host(ctx, &v);
        /* split */
        uint64_t read0 = 0;
        for (Req *r : batch) {
            if (rc == GS_OK) {
                uint64_t n = r->lens.size();
                uint64_t s0 = v.read_seed_off[read0], s1 = v.read_seed_off[read0 + n];
                uint64_t p0 = v.read_pos_off[read0], p1 = v.read_pos_off[read0 + n];
                r->seed_off.resize(n + 1);
                r->pos_off.resize(n + 1);
                for (uint64_t i = 0; i <= n; i++) {
                    r->seed_off[i] = v.read_seed_off[read0 + i] - s0;
                    r->pos_off[i] = v.read_pos_off[read0 + i] - p0;
                }
                r->seeds.assign(v.seeds + s0, v.seeds + s1);
                r->pos.assign(v.pos + p0, v.pos + p1);
                read0 += n;
            }
        }
        t_split = now_ms();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            double t1 = now_ms();
            s->stats.merge_us += (uint64_t)((t_merged - t0) * 1e3);
            s->stats.seed_us += (uint64_t)((t_seeded - t_merged) * 1e3);
            s->stats.split_us += (uint64_t)((t_split - t_seeded) * 1e3);
            for (Req *r : batch) {
                r->status = rc;
                r->done = true;
                r->t_done = t1;
                r->seqs.clear();
                r->ext = NULL;
                if (rc == GS_OK) s->stats.completed++;
                else s->stats.failed++;
            }
            s->stats.passes++;
            s->stats.reads += nr;
            if (nr > s->stats.max_batch_reads) s->stats.max_batch_reads = nr;
            s->reserved -= est;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
    cudaFreeHost(seqs);
    cudaFreeHost(offs);
    cudaFreeHost(lens);
    gs_ctx_free(ctx);
}

extern "C" int gs_server_start(gs_index *idx, const gs_server_opts *opts, gs_server **out)
{
    if (!idx || !opts || !out) {
        gs_set_error("gs_server_start: null argument");
        return GS_EINVAL;
    }
    *out = NULL;
    if (!opts->params.smem && opts->params.mem_next != GS_MEM_NEXT_READ) {
        gs_set_error("gs_server_start: a request's seeds must not depend on the requests merged "
                     "with it (mem_next must be GS_MEM_NEXT_READ)");
        return GS_EINVAL;
    }
    gs_server *s = new gs_server();
    s->idx = idx;
    s->opts = *opts;
    if (s->opts.n_slots <= 0) s->opts.n_slots = 12;
    if (s->opts.n_slots > 64) s->opts.n_slots = 64;
    if (s->opts.max_batch_reads <= 0) s->opts.max_batch_reads = 1 << 18;
    s->stopping = false;
    s->next_id = 1;
    s->reserved = 0;
    s->start_error = 0;
    memset(&s->stats, 0, sizeof(s->stats));
    GS_ON_DEVICE(gs_index_device(idx));
    size_t free_b = 0, total_b = 0;
    GS_CUDA(cudaMemGetInfo(&free_b, &total_b));
    s->budget = opts->hbm_budget ? opts->hbm_budget : (uint64_t)(free_b * 0.6);
    for (int i = 0; i < s->opts.n_slots; i++) s->workers.emplace_back(worker_main, s, i);
    *out = s;
    return GS_OK;
}

static int submit(gs_server *s, const char *seqs, const uint64_t *offsets,
                  const uint32_t *lengths, uint32_t n_reads, uint64_t *request_id, bool by_ref)
{
    if (!s || !request_id || (n_reads && (!seqs || !offsets || !lengths))) {
        gs_set_error("gs_server_submit: null argument");
        return GS_EINVAL;
    }
    if (s->opts.params.k < GS_K0) {
        gs_set_error("gs_server_submit: server params have k < 13");
        return GS_EINVAL;
    }
    const double t_enter = now_ms();
    Req *r = NULL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->spare.empty()) {
            r = s->spare.back();
            s->spare.pop_back();
        }
    }
    if (!r) r = new Req();
    uint64_t bytes = 0;
    for (uint32_t i = 0; i < n_reads; i++) bytes += lengths[i];
    r->seed_off.clear();
    r->pos_off.clear();
    r->seeds.clear();
    r->pos.clear();
    r->ext = NULL;
    r->offs.resize(n_reads);
    r->lens.assign(lengths, lengths + n_reads);
    /* reads that lie back to back in the caller's buffer (the usual case)
     * are copied in one piece; otherwise read by read */
    bool packed = true;
    for (uint32_t i = 0; i + 1 < n_reads && packed; i++)
        packed = offsets[i + 1] == offsets[i] + lengths[i];
    uint64_t w = 0;
    if (packed && n_reads) {
        /* by reference: the worker copies the bases straight from the
         * caller's buffer when it merges the pass */
        if (by_ref) {
            r->ext = seqs + offsets[0];
            r->seqs.clear();
        } else {
            r->seqs.resize(bytes);
            memcpy(r->seqs.data(), seqs + offsets[0], bytes);
        }
        for (uint32_t i = 0; i < n_reads; i++) {
            r->offs[i] = w;
            w += lengths[i];
        }
    } else {
        r->seqs.resize(bytes);
        for (uint32_t i = 0; i < n_reads; i++) {
            memcpy(r->seqs.data() + w, seqs + offsets[i], lengths[i]);
            r->offs[i] = w;
            w += lengths[i];
        }
    }
    r->bases = bytes;
    r->est_bytes = estimate_bytes(bytes, n_reads);
    r->done = false;
    r->status = 0;
    r->t_submit = now_ms();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.submit_us += (uint64_t)((r->t_submit - t_enter) * 1e3);
        if (s->stopping) {
            delete r;
            gs_set_error("server is stopping");
            return GS_ESTATE;
        }
        r->id = s->next_id++;
        s->reqs[r->id] = r;
        s->pending.push_back(r);
        s->stats.submitted++;
        *request_id = r->id;
    }
    s->cv_work.notify_one();
    return GS_OK;
}

extern "C" int gs_server_submit(gs_server *s, const char *seqs, const uint64_t *offsets,
                                const uint32_t *lengths, uint32_t n_reads, uint64_t *request_id)
{
    return submit(s, seqs, offsets, lengths, n_reads, request_id, false);
}

extern "C" int gs_server_submit_ref(gs_server *s, const char *seqs, const uint64_t *offsets,
                                    const uint32_t *lengths, uint32_t n_reads,
                                    uint64_t *request_id)
{
    return submit(s, seqs, offsets, lengths, n_reads, request_id, true);
}

extern "C" int gs_server_wait(gs_server *s, uint64_t id, int32_t timeout_ms)
{
    if (!s) return GS_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) {
        gs_set_error("unknown request %llu", (unsigned long long)id);
        return GS_EINVAL;
    }
    Req *r = it->second;
    auto pred = [&] { return r->done || s->start_error; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return GS_ETIMEOUT;
    if (!r->done) {
        gs_set_error("server worker failed to start");
        return s->start_error;
    }
    return r->status;
}

extern "C" int gs_server_result(gs_server *s, uint64_t id, gs_result_view *out, double *latency_ms)
{
    if (!s || !out) return GS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second->done) {
        gs_set_error("request %llu unknown or not finished", (unsigned long long)id);
        return GS_ESTATE;
    }
    Req *r = it->second;
    if (r->status) return r->status;
    out->n_reads = (uint32_t)r->lens.size();
    out->n_seeds = r->seeds.size();
    out->n_pos = r->pos.size();
    out->read_seed_off = r->seed_off.data();
    out->read_pos_off = r->pos_off.data();
    out->seeds = r->seeds.data();
    out->pos = r->pos.data();
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    return GS_OK;
}

extern "C" int gs_server_release(gs_server *s, uint64_t id)
{
    if (!s) return GS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second->done) return GS_ESTATE;
    Req *r = it->second;
    s->reqs.erase(it);
    const size_t held = r->seqs.capacity() + r->offs.capacity() * 8 + r->lens.capacity() * 4 +
                        r->seed_off.capacity() * 16 + r->seeds.capacity() * sizeof(gs_seed_rec) +
                        r->pos.capacity() * 4;
    if (s->spare.size() < 1024 && held <= ((size_t)32 << 20)) s->spare.push_back(r);
    else delete r;
    return GS_OK;
}

extern "C" int gs_server_get_stats(gs_server *s, gs_server_stats *out)
{
    if (!s || !out) return GS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->pending = s->pending.size();
    out->reserved_bytes = s->reserved;
    out->budget_bytes = s->budget;
    return GS_OK;
}

extern "C" void gs_server_stop(gs_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (auto &kv : s->reqs) delete kv.second;
    for (Req *r : s->spare) delete r;
    delete s;
}

/* Load generator: submits request i (reads first[i] .. first[i]+count[i]-1 of
 * the pool) gap_ms[i] after request i-1, from this thread, then waits for
 * all; latency_ms[i] gets each request's submit-to-done time and *wall_ms the
 * time from the first submission to the last completion. */
extern "C" int gs_server_replay(gs_server *s, const char *pool_seqs, const uint64_t *pool_offsets,
                                const uint32_t *pool_lengths, uint32_t n_req, const uint32_t *first,
                                const uint32_t *count, const double *gap_ms, double *latency_ms,
                                double *wall_ms, double *submit_ms)
{
    if (!s || !pool_seqs || !pool_offsets || !pool_lengths || !first || !count || !gap_ms ||
        !latency_ms)
        return GS_EINVAL;
    std::vector<uint64_t> ids(n_req);
    std::vector<uint64_t> offs;
    int status = GS_OK;
    uint32_t next_done = 0;
    /* a client that takes each result as it is done (in submission order)
     * and releases it, so the server reuses its buffers */
    auto collect = [&](uint32_t upto, bool block) {
        while (next_done < upto) {
            int rc = gs_server_wait(s, ids[next_done], block ? -1 : 0);
            if (rc == GS_ETIMEOUT) return;
            gs_result_view v;
            if (rc == GS_OK) rc = gs_server_result(s, ids[next_done], &v, &latency_ms[next_done]);
            if (rc && !status) status = rc;
            gs_server_release(s, ids[next_done]);
            next_done++;
        }
    };
    double t0 = now_ms(), due = t0;
    for (uint32_t i = 0; i < n_req; i++) {
        due += gap_ms[i];
        double now;
        while ((now = now_ms()) < due) {
            collect(i, false);
            if (due - now > 0.2) std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
        const uint32_t f = first[i], n = count[i];
        offs.resize(n);
        uint64_t base = pool_offsets[f];
        for (uint32_t j = 0; j < n; j++) offs[j] = pool_offsets[f + j] - base;
        /* the pool outlives every request: submitted by reference */
        int rc = gs_server_submit_ref(s, pool_seqs + base, offs.data(), pool_lengths + f, n,
                                      &ids[i]);
        if (rc) return rc;
    }
    double t_sub = now_ms();
    collect(n_req, true);
    if (wall_ms) *wall_ms = now_ms() - t0;
    if (submit_ms) *submit_ms = t_sub - t0;
    return status;
}
