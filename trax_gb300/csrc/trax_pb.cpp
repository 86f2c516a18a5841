/*
 * trax_pb.cpp -- native decoder of the reference's event files.
 *
 * Two layouts (EventLoader.h:15-147):
 *   TRAX_PB_CONTAINER   one PEventContainer message (Event.proto:35-38), as
 *                       EventLoader / RepeatedEventLoader parse it;
 *   TRAX_PB_EVENT_STORE GenericOutputStore's stream (PEventStore.h:25-80):
 *                       little-endian uint32 event count, then per event a
 *                       varint entry type (1 = event), a varint size and the
 *                       PEvent bytes.
 * Messages are protobuf-2 wire format (Event.proto:9-33).  Unknown fields
 * are skipped; a missing required field or a truncated message is an error,
 * as ParseFromCodedStream fails on both.
 *
 * Decoding is two-phase: an index pass finds every event's byte range, then
 * worker threads decode events independently into the caller's arrays at
 * offsets from a prefix sum of per-event hit counts.
 */
#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/trax.h"

namespace {

thread_local std::string g_pb_err;

struct Reader {
    const uint8_t *p, *end;
    bool ok = true;

    bool more() const { return ok && p < end; }

    uint64_t varint()
    {
        uint64_t r = 0;
        for (int s = 0; s < 70; s += 7) {
            if (p >= end) { ok = false; return 0; }
            const uint8_t c = *p++;
            r |= (uint64_t)(c & 0x7f) << s;
            if (!(c & 0x80)) return r;
        }
        ok = false; /* more than 10 bytes */
        return 0;
    }
    uint32_t fixed32()
    {
        if (end - p < 4) { ok = false; p = end; return 0; }
        const uint32_t v = (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 |
                           (uint32_t)p[3] << 24;
        p += 4;
        return v;
    }
    float f32()
    {
        const uint32_t u = fixed32();
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    }
    Reader sub()
    {
        const uint64_t n = varint();
        if (!ok || n > (uint64_t)(end - p)) { ok = false; p = end; return Reader{end, end}; }
        Reader r{p, p + n};
        p += n;
        return r;
    }
    void skip(uint32_t wire)
    {
        switch (wire) {
        case 0: varint(); break;
        case 1: if (end - p < 8) { ok = false; p = end; } else p += 8; break;
        case 2: sub(); break;
        case 5: fixed32(); break;
        default: ok = false; /* groups (3, 4) do not occur in Event.proto */
        }
    }
};

struct EventRange {
    const uint8_t *p, *end;
};

/* PGlobalPoint (Event.proto:9-14). */
bool read_point(Reader r, float *x, float *y, float *z)
{
    int seen = 0;
    while (r.more()) {
        const uint64_t key = r.varint();
        const uint32_t f = (uint32_t)(key >> 3), w = (uint32_t)(key & 7);
        if (f >= 1 && f <= 3 && w == 5) {
            const float v = r.f32();
            (f == 1 ? *x : f == 2 ? *y : *z) = v;
            seen |= 1 << f;
        } else {
            r.skip(w);
        }
    }
    return r.ok && seen == 0xE;
}

/* PHit (Event.proto:16-24).  Fields 2-5 are required, 6-7 optional with
 * default 0. */
bool read_hit(Reader r, trax_pb_events *out, uint64_t h)
{
    int seen = 0;
    float x = 0, y = 0, z = 0;
    uint64_t layer = 0, det = 0, hit_id = 0, track = 0;
    int64_t type = 0;
    float pt = 0.0f;
    while (r.more()) {
        const uint64_t key = r.varint();
        const uint32_t f = (uint32_t)(key >> 3), w = (uint32_t)(key & 7);
        if (f == 1 && w == 2) {
            if (!read_point(r.sub(), &x, &y, &z)) return false;
            seen |= 1 << 1;
        } else if (f >= 2 && f <= 6 && w == 0) {
            const uint64_t v = r.varint();
            if (f == 2) type = (int64_t)v;
            else if (f == 3) layer = v;
            else if (f == 4) det = v;
            else if (f == 5) hit_id = v;
            else track = v;
            seen |= 1 << f;
        } else if (f == 7 && w == 5) {
            pt = r.f32();
        } else {
            r.skip(w);
        }
    }
    if (!r.ok || (seen & 0x3E) != 0x3E) return false;
    if (out) {
        out->x[h] = x; out->y[h] = y; out->z[h] = z;
        out->detector_type[h] = (int32_t)type;
        out->layer[h] = (uint32_t)layer;
        out->detector_id[h] = (uint32_t)det;
        out->hit_id[h] = hit_id;
        out->sim_track_id[h] = (uint32_t)track;
        out->sim_track_pt[h] = pt;
    }
    return true;
}

/* PEvent (Event.proto:26-33): counts hits (out == NULL) or decodes them. */
bool read_event(EventRange ev, trax_pb_events *out, uint32_t e, uint64_t first_hit,
                uint64_t *n_hits)
{
    Reader r{ev.p, ev.end};
    int seen = 0;
    uint64_t h = first_hit;
    uint64_t hdr[3] = {0, 0, 0};
    while (r.more()) {
        const uint64_t key = r.varint();
        const uint32_t f = (uint32_t)(key >> 3), w = (uint32_t)(key & 7);
        if (f >= 1 && f <= 3 && w == 0) {
            hdr[f - 1] = r.varint();
            seen |= 1 << f;
        } else if (f == 4 && w == 2) {
            Reader hr = r.sub();
            if (!r.ok) return false;
            if (out) {
                if (!read_hit(hr, out, h)) return false;
            } else if (!read_hit(hr, nullptr, 0)) {
                return false;
            }
            ++h;
        } else {
            r.skip(w);
        }
    }
    if (!r.ok || seen != 0xE) return false;
    if (out) {
        out->run[e] = hdr[0];
        out->lumi[e] = hdr[1];
        out->event_number[e] = hdr[2];
    }
    *n_hits = h - first_hit;
    return true;
}

trax_status index_events(const uint8_t *buf, size_t len, int format, std::vector<EventRange> &evs)
{
    evs.clear();
    if (!buf && len) { g_pb_err = "NULL buffer"; return TRAX_ERR_BAD_ARG; }
    Reader r{buf, buf + len};
    if (format == TRAX_PB_CONTAINER) {
        while (r.more()) {
            const uint64_t key = r.varint();
            const uint32_t f = (uint32_t)(key >> 3), w = (uint32_t)(key & 7);
            if (f == 1 && w == 2) {
                Reader e = r.sub();
                if (r.ok) evs.push_back({e.p, e.end});
            } else {
                r.skip(w);
            }
        }
    } else if (format == TRAX_PB_EVENT_STORE) {
        const uint32_t n = r.fixed32();
        for (uint32_t i = 0; i < n && r.ok; ++i) {
            const uint64_t type = r.varint();
            if (!r.ok) break;
            if (type != 1) { g_pb_err = "event store entry of unknown type"; return TRAX_ERR_BAD_INPUT; }
            Reader e = r.sub();
            if (r.ok) evs.push_back({e.p, e.end});
        }
    } else {
        g_pb_err = "unknown file layout";
        return TRAX_ERR_BAD_ARG;
    }
    if (!r.ok) {
        g_pb_err = "truncated or malformed message at byte " + std::to_string(r.p - buf);
        return TRAX_ERR_BAD_INPUT;
    }
    if (evs.size() > 0xFFFFFFFEull) { g_pb_err = "too many events"; return TRAX_ERR_BAD_INPUT; }
    return TRAX_OK;
}

/* Runs fn(i) for i in [0, n) on up to n_threads threads; returns the
 * smallest i whose call failed, or n. */
template <class F>
size_t parallel_for(size_t n, int n_threads, F fn)
{
    const size_t workers = std::max<size_t>(1, std::min<size_t>((size_t)std::max(n_threads, 1), n));
    std::atomic<size_t> next{0}, first_bad{n};
    auto body = [&]() {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= n) return;
            if (!fn(i)) {
                size_t cur = first_bad.load();
                while (i < cur && !first_bad.compare_exchange_weak(cur, i)) {}
            }
        }
    };
    if (workers == 1) {
        body();
    } else {
        std::vector<std::thread> ts;
        for (size_t t = 0; t < workers; ++t) ts.emplace_back(body);
        for (auto &t : ts) t.join();
    }
    return first_bad.load();
}

}  // namespace

extern "C" {

const char *trax_pb_error(void) { return g_pb_err.c_str(); }

trax_status trax_pb_scan(const uint8_t *buf, size_t len, int format, uint32_t *n_events,
                         uint64_t *n_hits)
{
    if (!n_events || !n_hits) return TRAX_ERR_BAD_ARG;
    std::vector<EventRange> evs;
    trax_status s = index_events(buf, len, format, evs);
    if (s != TRAX_OK) return s;
    std::vector<uint64_t> cnt(evs.size());
    const size_t bad = parallel_for(evs.size(), (int)std::thread::hardware_concurrency(),
                                    [&](size_t i) { return read_event(evs[i], nullptr, 0, 0, &cnt[i]); });
    if (bad < evs.size()) {
        g_pb_err = "event " + std::to_string(bad) + ": malformed or missing a required field";
        return TRAX_ERR_BAD_INPUT;
    }
    uint64_t total = 0;
    for (uint64_t c : cnt) total += c;
    *n_events = (uint32_t)evs.size();
    *n_hits = total;
    return TRAX_OK;
}

trax_status trax_pb_decode(const uint8_t *buf, size_t len, int format, trax_pb_events *out,
                           int n_threads)
{
    if (!out || !out->hit_offset) return TRAX_ERR_BAD_ARG;
    std::vector<EventRange> evs;
    trax_status s = index_events(buf, len, format, evs);
    if (s != TRAX_OK) return s;
    if (evs.size() != out->n_events) {
        g_pb_err = "event count differs from the arrays' (call trax_pb_scan first)";
        return TRAX_ERR_BAD_ARG;
    }
    if (n_threads <= 0) n_threads = (int)std::thread::hardware_concurrency();
    std::vector<uint64_t> cnt(evs.size());
    size_t bad = parallel_for(evs.size(), n_threads,
                              [&](size_t i) { return read_event(evs[i], nullptr, 0, 0, &cnt[i]); });
    if (bad < evs.size()) {
        g_pb_err = "event " + std::to_string(bad) + ": malformed or missing a required field";
        return TRAX_ERR_BAD_INPUT;
    }
    uint64_t off = 0;
    for (size_t i = 0; i < evs.size(); ++i) {
        out->hit_offset[i] = off;
        off += cnt[i];
    }
    out->hit_offset[evs.size()] = off;
    if (off != out->n_hits) {
        g_pb_err = "hit count differs from the arrays' (call trax_pb_scan first)";
        return TRAX_ERR_BAD_ARG;
    }
    if (evs.size() && (!out->x || !out->y || !out->z || !out->detector_type || !out->layer ||
                       !out->detector_id || !out->hit_id || !out->sim_track_id ||
                       !out->sim_track_pt || !out->run || !out->lumi || !out->event_number))
        return TRAX_ERR_BAD_ARG;
    uint64_t dummy;
    bad = parallel_for(evs.size(), n_threads, [&](size_t i) {
        return read_event(evs[i], out, (uint32_t)i, out->hit_offset[i], &dummy);
    });
    if (bad < evs.size()) {
        g_pb_err = "event " + std::to_string(bad) + ": decode failed";
        return TRAX_ERR_BAD_INPUT;
    }
    return TRAX_OK;
}

}  // extern "C"
