/*
 * trax_serve.cpp -- continuous-batching request loop over the C-ABI.
 *
 * Requests are single events.  `slots` worker threads each own a trax_ctx
 * (stream, reserved device buffers, captured graph) and pinned staging.  A
 * worker takes every request that has arrived -- up to the slot's event and
 * hit capacity -- into its next batch, runs grid build -> pairs -> predict ->
 * filter as one graph, and hands each event its own tracklets.  Requests that
 * arrive while batches are on the GPU join the next batch of whichever slot
 * frees first, so the slots' batches overlap on the device.
 *
 * Admission by memory budget: the budget is split over the slots and sized
 * into hit / pair / candidate / tracklet capacities.  A worker admits the
 * arrived requests into its batch while they fit the slot's event and hit
 * capacity and -- the pair bound -- while their pair totals fit its pair
 * capacity.  Pair totals come from the device: the grid build and the pair
 * stage's count passes run on the requests not counted yet, as one batch,
 * and the scanned totals come back per event (trax_count_pairs_batch); they
 * are exact, so a batch so admitted never overflows its pairs.  Requests
 * that do not fit go back to the front of the queue with their totals and
 * lead the next batch.  The count costs a pass over the batch, so it runs
 * only when the batch could come near the capacity: the counted events give
 * kappa, the largest pairs / hits^2 seen (pairs grow with the square of an
 * event's hit density), and a batch whose sum of 1.25 kappa hits^2 stays
 * within the pair capacity is admitted without counting.  The candidate and
 * tracklet totals are scanned on the device before anything is stored; when
 * a batch would exceed one of those capacities the device stores nothing
 * beyond it, reports TRAX_ERR_CAPACITY with the true size, and the worker
 * splits the batch in halves and reruns them.
 *
 * Per-event results do not depend on the batch: every stage works inside its
 * (event, layer triplet) group and tracklets are returned as hit positions
 * within the event.
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/trax.h"

namespace {

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

constexpr uint32_t kPairsUnknown = 0xffffffffu;

struct Request {
    uint64_t ticket = 0;
    uint64_t arrival_ns = 0;
    uint32_t n_hits = 0;
    uint32_t pairs = kPairsUnknown;  /* the event's pair total, once counted */
    uint32_t layer_nhits[TRAX_MAX_LAYERS] = {};
    bool borrowed = false;
    /* the columns the batched chain reads (not the detector and hit ids:
     * tracklets come back as positions in the request's own columns) */
    const float *x = nullptr, *y = nullptr, *z = nullptr;
    const uint32_t *layer = nullptr;
    std::vector<float> own_f;      /* x | y | z when copied */
    std::vector<uint32_t> own_u;   /* layer when copied */
};

struct Result {
    uint64_t ticket = 0, arrival_ns = 0, start_ns = 0, done_ns = 0;
    trax_status status = TRAX_OK;
    uint32_t batch_events = 0;
    std::vector<uint32_t> trk;     /* hit1 | hit2 | hit3 */
    uint32_t n_trk = 0;
    uint32_t offsets[TRAX_MAX_LAYER_TRIPLETS + 1] = {};
};

struct Slot {
    trax_ctx *ctx = nullptr;
    uint32_t max_events = 0, max_hits = 0, trk_cap = 0;
    uint64_t pair_cap = 0;
    std::vector<uint32_t> event_pairs;  /* per event of an admission count */
    float *x = nullptr, *y = nullptr, *z = nullptr;
    uint32_t *layer = nullptr, *event = nullptr;
    uint32_t *layer_nhits = nullptr;
    uint32_t *h1 = nullptr, *h2 = nullptr, *h3 = nullptr, *off = nullptr;
};

}  // namespace

struct trax_server {
    int device = 0;
    trax_config cfg{};
    trax_server_opts opts{};
    uint32_t T = 0, L = 0;
    std::vector<Slot> slots;
    std::vector<std::thread> workers;
    std::thread feeder;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::deque<Result *> done;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::vector<uint64_t> latencies_ns;
    double kappa = 0.0;  /* largest pairs / hits^2 of a counted event */
    uint64_t first_arrival = UINT64_MAX, last_done = 0;
    trax_server_stats stats{};
    std::string err;
};

namespace {

/* Copies requests [lo, hi) into the slot's pinned staging as one batch. */
trax_event_batch stage_requests(const trax_server *srv, Slot &slot,
                                const std::vector<Request *> &reqs, size_t lo, size_t hi)
{
    const uint32_t L = srv->L;
    const uint32_t E = (uint32_t)(hi - lo);
    uint32_t n = 0;
    for (size_t i = lo; i < hi; ++i) {
        const Request *r = reqs[i];
        const uint32_t e = (uint32_t)(i - lo);
        std::memcpy(slot.x + n, r->x, r->n_hits * 4ull);
        std::memcpy(slot.y + n, r->y, r->n_hits * 4ull);
        std::memcpy(slot.z + n, r->z, r->n_hits * 4ull);
        std::memcpy(slot.layer + n, r->layer, r->n_hits * 4ull);
        std::fill(slot.event + n, slot.event + n + r->n_hits, e);
        std::memcpy(slot.layer_nhits + (size_t)e * L, r->layer_nhits, L * 4ull);
        n += r->n_hits;
    }
    return trax_event_batch{E, L, n, slot.x, slot.y, slot.z, slot.layer, nullptr, nullptr,
                            slot.event, slot.layer_nhits};
}

/* The pair totals of the requests not counted yet, from one device count
 * pass over them as a batch. */
trax_status count_pairs(trax_server *srv, Slot &slot, const std::vector<Request *> &reqs)
{
    std::vector<Request *> todo;
    for (Request *r : reqs)
        if (r->pairs == kPairsUnknown) todo.push_back(r);
    if (todo.empty()) return TRAX_OK;
    trax_event_batch b = stage_requests(srv, slot, todo, 0, todo.size());
    slot.event_pairs.resize(todo.size());
    const trax_status st = trax_count_pairs_batch(slot.ctx, &b, slot.event_pairs.data());
    if (st != TRAX_OK) return st;
    double kappa = 0.0;
    for (size_t i = 0; i < todo.size(); ++i) {
        todo[i]->pairs = slot.event_pairs[i];
        const double h = (double)todo[i]->n_hits;
        if (h > 0) kappa = std::max(kappa, (double)todo[i]->pairs / (h * h));
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->kappa = std::max(srv->kappa, kappa);
    srv->stats.count_passes += 1;
    return TRAX_OK;
}

void run_batch(trax_server *srv, Slot &slot, std::vector<Request *> &reqs, size_t lo, size_t hi,
               uint64_t start_ns, std::vector<Result *> &out)
{
    const uint32_t T = srv->T;
    const uint32_t E = (uint32_t)(hi - lo);
    trax_event_batch b = stage_requests(srv, slot, reqs, lo, hi);
    trax_batch_result res{};
    res.hit1 = slot.h1; res.hit2 = slot.h2; res.hit3 = slot.h3; res.offsets = slot.off;
    res.capacity = slot.trk_cap;
    res.input_indices = 1;
    trax_status st = trax_seed_batch(slot.ctx, &b, &res);
    if (st == TRAX_ERR_CAPACITY && E > 1) {
        {
            std::lock_guard<std::mutex> lock(srv->mu);
            srv->stats.splits += 1;
        }
        const size_t mid = lo + (hi - lo) / 2;
        run_batch(srv, slot, reqs, lo, mid, start_ns, out);
        run_batch(srv, slot, reqs, mid, hi, start_ns, out);
        return;
    }
    const uint64_t t_done = now_ns();
    uint32_t base = 0;
    for (size_t i = lo; i < hi; ++i) {
        const Request *r = reqs[i];
        const uint32_t e = (uint32_t)(i - lo);
        Result *o = new Result();
        o->ticket = r->ticket;
        o->arrival_ns = r->arrival_ns;
        o->start_ns = start_ns;
        o->done_ns = t_done;
        o->status = st;
        o->batch_events = E;
        if (st == TRAX_OK) {
            const uint32_t a = slot.off[(size_t)e * T], z = slot.off[(size_t)(e + 1) * T];
            o->n_trk = z - a;
            o->trk.resize(3ull * o->n_trk);
            for (uint32_t k = 0; k < o->n_trk; ++k) {
                o->trk[k] = slot.h1[a + k] - base;
                o->trk[o->n_trk + k] = slot.h2[a + k] - base;
                o->trk[2ull * o->n_trk + k] = slot.h3[a + k] - base;
            }
            for (uint32_t t = 0; t <= T; ++t) o->offsets[t] = slot.off[(size_t)e * T + t] - a;
        }
        base += r->n_hits;
        out.push_back(o);
    }
}

void worker_main(trax_server *srv, size_t si)
{
    cudaSetDevice(srv->device);
    Slot &slot = srv->slots[si];
    std::vector<Request *> batch;
    std::vector<Result *> results;
    for (;;) {
        batch.clear();
        results.clear();
        {
            std::unique_lock<std::mutex> lock(srv->mu);
            for (;;) {
                if (srv->stop && srv->pending.empty()) return;
                if (!srv->pending.empty()) {
                    const uint64_t t = now_ns();
                    const uint64_t a = srv->pending.front()->arrival_ns;
                    if (a <= t) break;
                    srv->cv_work.wait_for(lock, std::chrono::nanoseconds(a - t));
                } else {
                    srv->cv_work.wait(lock);
                }
            }
            /* continuous batching: everything that has arrived, up to capacity */
            const uint64_t t = now_ns();
            uint32_t hits = 0;
            while (!srv->pending.empty() && batch.size() < slot.max_events) {
                Request *r = srv->pending.front();
                if (r->arrival_ns > t) break;
                if (!batch.empty() && hits + r->n_hits > slot.max_hits) break;
                srv->pending.pop_front();
                batch.push_back(r);
                hits += r->n_hits;
            }
            if (!srv->pending.empty()) srv->cv_work.notify_one();
        }
        const uint64_t start = now_ns();
        auto refuse = [&](Request *r) {
            Result *o = new Result();
            o->ticket = r->ticket;
            o->arrival_ns = r->arrival_ns;
            o->start_ns = o->done_ns = start;
            o->status = TRAX_ERR_CAPACITY;
            results.push_back(o);
        };
        if (batch.size() == 1 && batch[0]->n_hits > slot.max_hits) {
            refuse(batch[0]);
        } else {
            /* the pair bound: admit the longest prefix whose counted pairs
             * fit the slot; the rest leads the next batch */
            size_t k = batch.size();
            double kappa, est = 0.0;
            {
                std::lock_guard<std::mutex> lock(srv->mu);
                kappa = srv->kappa;
            }
            for (const Request *r : batch)
                est += r->pairs != kPairsUnknown ? (double)r->pairs
                                                 : 1.25 * kappa * (double)r->n_hits * r->n_hits;
            const bool fits = kappa > 0.0 && est <= (double)slot.pair_cap;
            if (!fits && count_pairs(srv, slot, batch) == TRAX_OK) {
                uint64_t pairs = 0;
                k = 0;
                while (k < batch.size() && pairs + batch[k]->pairs <= slot.pair_cap)
                    pairs += batch[k++]->pairs;
                if (k < batch.size()) {
                    std::lock_guard<std::mutex> lock(srv->mu);
                    for (size_t i = batch.size(); i-- > std::max<size_t>(k, 1);)
                        srv->pending.push_front(batch[i]);
                    srv->stats.deferred += batch.size() - std::max<size_t>(k, 1);
                }
                if (k == 0) {  /* one event beyond the pair capacity: never fits */
                    refuse(batch[0]);
                    batch.resize(1);
                } else {
                    batch.resize(k);
                }
                srv->cv_work.notify_one();
            }
            if (k > 0) run_batch(srv, slot, batch, 0, batch.size(), start, results);
        }
        {
            std::lock_guard<std::mutex> lock(srv->mu);
            srv->stats.batches += 1;
            for (Result *o : results) {
                srv->stats.events += 1;
                if (o->status != TRAX_OK) srv->stats.errors += 1;
                srv->latencies_ns.push_back(o->done_ns - o->arrival_ns);
                srv->first_arrival = std::min(srv->first_arrival, o->arrival_ns);
                srv->last_done = std::max(srv->last_done, o->done_ns);
                if (srv->opts.keep_results) srv->done.push_back(o);
                else delete o;
            }
            srv->stats.batched_events += batch.size();
        }
        for (Request *r : batch) delete r;
        srv->cv_done.notify_all();
    }
}

trax_status pinned(trax_ctx *ctx, void **p, size_t bytes) { return trax_host_alloc_pinned(ctx, p, bytes); }

void destroy_slots(trax_server *srv)
{
    for (Slot &s : srv->slots) {
        if (!s.ctx) continue;
        void *bufs[] = {s.x, s.y, s.z, s.layer, s.event, s.layer_nhits, s.h1, s.h2, s.h3, s.off};
        for (void *b : bufs) if (b) trax_host_free_pinned(s.ctx, b);
        trax_ctx_destroy(s.ctx);
        s.ctx = nullptr;
    }
}

Request *make_request(trax_server *srv, const trax_event_batch *ev, uint64_t arrival_ns,
                      int borrow)
{
    Request *r = new Request();
    r->arrival_ns = arrival_ns ? arrival_ns : now_ns();
    r->n_hits = ev->n_hits;
    std::memcpy(r->layer_nhits, ev->layer_nhits, srv->L * 4ull);
    r->borrowed = borrow != 0;
    if (borrow) {
        r->x = ev->x; r->y = ev->y; r->z = ev->z;
        r->layer = ev->layer;
    } else {
        const size_t n = ev->n_hits;
        r->own_f.resize(3 * n);
        r->own_u.resize(n);
        std::memcpy(r->own_f.data(), ev->x, n * 4);
        std::memcpy(r->own_f.data() + n, ev->y, n * 4);
        std::memcpy(r->own_f.data() + 2 * n, ev->z, n * 4);
        std::memcpy(r->own_u.data(), ev->layer, n * 4);
        r->x = r->own_f.data(); r->y = r->own_f.data() + n; r->z = r->own_f.data() + 2 * n;
        r->layer = r->own_u.data();
    }
    return r;
}

}  // namespace

extern "C" {

uint64_t trax_now_ns(void) { return now_ns(); }

trax_status trax_server_create(trax_server **out, int device, const trax_config *cfg,
                               const trax_server_opts *opts)
{
    if (!out || !cfg || !opts) return TRAX_ERR_BAD_ARG;
    *out = nullptr;
    if (opts->slots == 0 || opts->slots > 16 || opts->max_batch_events == 0 ||
        opts->n_layers == 0 || opts->n_layers > TRAX_MAX_LAYERS)
        return TRAX_ERR_BAD_ARG;
    trax_grid_cfg g{opts->max_batch_events, opts->n_layers, opts->n_sectors_z,
                    opts->n_sectors_phi};
    if (trax_config_validate(cfg, &g) != TRAX_OK) return TRAX_ERR_BAD_ARG;
    trax_server *srv = new trax_server();
    srv->device = device;
    srv->cfg = *cfg;
    srv->opts = *opts;
    srv->T = cfg->n_layer_triplets;
    srv->L = opts->n_layers;
    /* Split the budget over the slots.  Bytes per hit of a slot: 28 input +
     * 12 sorted (layer, event, input position) + 26 packed copies (z/phi,
     * half z, x/y/z/phi) + 12 per
     * triplet of outer-slot scratch and 4 per kept pair accept (32) and
     * triplet, plus capacity for the pairs (12 B each with their scratch),
     * candidates (8 B) and tracklets (24 B) allowed per hit. */
    const uint64_t kp = opts->pairs_per_hit ? opts->pairs_per_hit : 24;
    const uint64_t kc = opts->candidates_per_hit ? opts->candidates_per_hit : 12;
    const uint64_t kt = opts->tracklets_per_hit ? opts->tracklets_per_hit : 4;
    const uint64_t cells = (uint64_t)(opts->n_sectors_z + 1) * (opts->n_sectors_phi + 1);
    const uint64_t fixed = (uint64_t)opts->max_batch_events * opts->n_layers * cells * 4 +
                           (uint64_t)opts->max_batch_events * srv->T * 40;
    const uint64_t per_slot = opts->memory_budget_bytes / opts->slots;
    auto per_hit_for = [&](uint64_t keep) {
        return 28 + 12 + 26 + 12ull * srv->T + 4ull * keep * srv->T + kp * 12 + kc * 8 + kt * 24;
    };
    const uint64_t per_hit = per_hit_for(32);
    if (per_slot <= fixed + per_hit * 1024) {
        delete srv;
        return TRAX_ERR_OOM;
    }
    uint64_t H = (per_slot - fixed) / per_hit;
    if (opts->max_batch_hits && opts->max_batch_hits < H) H = opts->max_batch_hits;
    const uint64_t kmax = std::max(kp, std::max(kc, kt));
    if (H > 0x7fffffffull / kmax) H = 0x7fffffffull / kmax;
    if (opts->max_event_hits > H) {
        delete srv;
        return TRAX_ERR_OOM;
    }
    srv->slots.resize(opts->slots);
    for (Slot &s : srv->slots) {
        trax_status st = trax_ctx_create(&s.ctx, device);
        if (st != TRAX_OK) {
            s.ctx = nullptr;
            destroy_slots(srv);
            delete srv;
            return st;
        }
        s.max_events = opts->max_batch_events;
        s.max_hits = (uint32_t)H;
        s.trk_cap = (uint32_t)(kt * H);
        s.pair_cap = kp * H;
        st = trax_configure(s.ctx, cfg);
        const trax_tuning &tn = opts->tuning;
        if (st == TRAX_OK && (tn.run_walk | tn.index_min | tn.pair_record | tn.blocks_per_sm))
            st = trax_set_tuning(s.ctx, &tn);
        if (st == TRAX_OK)
            st = trax_reserve(s.ctx, s.max_events, srv->L, s.max_hits, &g, (uint32_t)(kp * H),
                              (uint32_t)(kc * H), s.trk_cap);
        void **f[] = {(void **)&s.x, (void **)&s.y, (void **)&s.z, (void **)&s.layer,
                      (void **)&s.event};
        for (void **p : f)
            if (st == TRAX_OK) st = pinned(s.ctx, p, H * 4);
        if (st == TRAX_OK) st = pinned(s.ctx, (void **)&s.layer_nhits, (size_t)s.max_events * srv->L * 4);
        void **o[] = {(void **)&s.h1, (void **)&s.h2, (void **)&s.h3};
        for (void **p : o)
            if (st == TRAX_OK) st = pinned(s.ctx, p, (size_t)s.trk_cap * 4);
        if (st == TRAX_OK) st = pinned(s.ctx, (void **)&s.off, ((size_t)s.max_events * srv->T + 1) * 4);
        if (st != TRAX_OK) {
            destroy_slots(srv);
            delete srv;
            return st;
        }
    }
    srv->stats.slot_max_hits = H;
    srv->stats.slot_max_pairs = kp * H;
    for (size_t i = 0; i < srv->slots.size(); ++i) srv->workers.emplace_back(worker_main, srv, i);
    *out = srv;
    return TRAX_OK;
}

trax_status trax_server_submit(trax_server *srv, const trax_event_batch *ev, uint64_t arrival_ns,
                               int borrow, uint64_t *ticket)
{
    if (!srv || !ev || ev->n_events != 1 || ev->n_layers != srv->L || !ev->layer_nhits)
        return TRAX_ERR_BAD_ARG;
    uint64_t sum = 0;
    for (uint32_t l = 0; l < srv->L; ++l) sum += ev->layer_nhits[l];
    if (sum != ev->n_hits) return TRAX_ERR_BAD_INPUT;
    Request *r = make_request(srv, ev, arrival_ns, borrow);
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        r->ticket = srv->next_ticket++;
        srv->pending.push_back(r);
        srv->stats.submitted += 1;
    }
    srv->cv_work.notify_one();
    if (ticket) *ticket = r->ticket;
    return TRAX_OK;
}

trax_status trax_server_replay(trax_server *srv, const trax_event_batch *pool,
                               const uint32_t *order, const uint64_t *arrival_ns, uint32_t n)
{
    if (!srv || !pool || !order || !arrival_ns) return TRAX_ERR_BAD_ARG;
    if (srv->feeder.joinable()) srv->feeder.join();
    srv->feeder = std::thread([=] {
        for (uint32_t i = 0; i < n; ++i) {
            const uint64_t a = arrival_ns[i];
            /* submit shortly before the arrival; the workers admit at `a` */
            for (;;) {
                const uint64_t t = now_ns();
                if (t + 200000 >= a) break;
                std::this_thread::sleep_for(std::chrono::nanoseconds(a - t - 200000));
            }
            trax_server_submit(srv, &pool[order[i]], a, 1, nullptr);
        }
    });
    return TRAX_OK;
}

trax_status trax_server_poll(trax_server *srv, trax_server_result *out, int timeout_ms)
{
    if (!srv || !out) return TRAX_ERR_BAD_ARG;
    Result *o = nullptr;
    {
        std::unique_lock<std::mutex> lock(srv->mu);
        if (srv->done.empty())
            srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                  [&] { return !srv->done.empty(); });
        if (srv->done.empty()) return TRAX_ERR_TIMEOUT;
        o = srv->done.front();
        srv->done.pop_front();
    }
    out->ticket = o->ticket;
    out->status = o->status;
    out->arrival_ns = o->arrival_ns;
    out->start_ns = o->start_ns;
    out->done_ns = o->done_ns;
    out->batch_events = o->batch_events;
    out->n_tracklets = o->n_trk;
    const uint32_t n = std::min(o->n_trk, out->capacity);
    if (n) {
        if (out->hit1) std::memcpy(out->hit1, o->trk.data(), n * 4ull);
        if (out->hit2) std::memcpy(out->hit2, o->trk.data() + o->n_trk, n * 4ull);
        if (out->hit3) std::memcpy(out->hit3, o->trk.data() + 2ull * o->n_trk, n * 4ull);
    }
    std::memcpy(out->offsets, o->offsets, sizeof(out->offsets));
    delete o;
    return n < out->n_tracklets ? TRAX_ERR_CAPACITY : TRAX_OK;
}

trax_status trax_server_drain(trax_server *srv, int timeout_ms)
{
    if (!srv) return TRAX_ERR_BAD_ARG;
    if (srv->feeder.joinable()) srv->feeder.join();
    std::unique_lock<std::mutex> lock(srv->mu);
    const bool ok = srv->cv_done.wait_for(
        lock, std::chrono::milliseconds(timeout_ms), [&] {
            return srv->pending.empty() && srv->stats.events == srv->stats.submitted;
        });
    return ok ? TRAX_OK : TRAX_ERR_TIMEOUT;
}

trax_status trax_server_get_stats(trax_server *srv, trax_server_stats *out)
{
    if (!srv || !out) return TRAX_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lock(srv->mu);
    *out = srv->stats;
    std::vector<uint64_t> l = srv->latencies_ns;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            const size_t i = std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5));
            return l[i];
        };
        out->p50_ns = pct(0.50);
        out->p99_ns = pct(0.99);
        out->max_ns = l.back();
        if (srv->last_done > srv->first_arrival)
            out->sustained_events_per_s =
                (double)l.size() / ((double)(srv->last_done - srv->first_arrival) * 1e-9);
    }
    return TRAX_OK;
}

trax_status trax_server_reset_stats(trax_server *srv)
{
    if (!srv) return TRAX_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lock(srv->mu);
    const uint64_t H = srv->stats.slot_max_hits, PC = srv->stats.slot_max_pairs;
    const uint64_t sub = srv->stats.submitted, ev = srv->stats.events;
    srv->stats = trax_server_stats{};
    srv->stats.slot_max_hits = H;
    srv->stats.slot_max_pairs = PC;
    srv->stats.submitted = sub - ev;
    srv->latencies_ns.clear();
    srv->first_arrival = UINT64_MAX;
    srv->last_done = 0;
    return TRAX_OK;
}

void trax_server_destroy(trax_server *srv)
{
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    if (srv->feeder.joinable()) srv->feeder.join();
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (std::thread &t : srv->workers) t.join();
    for (Request *r : srv->pending) delete r;
    for (Result *o : srv->done) delete o;
    destroy_slots(srv);
    delete srv;
}

}  // extern "C"
