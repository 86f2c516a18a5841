/*
 * trax_ingest.cuh -- HitCollection::addEvent (HitCollection.cpp:20-149) on
 * the GPU, for a batch of decoded events at once.
 *
 * One CTA per event runs the event's whole selection as stable counting
 * sorts in global scratch (L2-resident at event sizes):
 *   0. stable partition of the hits that pass the minPt / track-id filters
 *      (:39-48);
 *   1. LSD radix sort by simTrackID, 8-bit digits, skipping digits that are
 *      constant over the event -- the std::map<uint, ...> iteration order of
 *      the track list, hits of a track in file order (:38-56);
 *   2. track segments (rank of each hit's track, start of each track);
 *   3. the findable rule: a track is findable when it has a hit on every
 *      layer a triplet uses (:66-78);
 *   4. the data.tracks limit: iteration stops at the num_tracks-th findable
 *      track (:61);
 *   5. per findable track its first, middle and last hit in layer order
 *      (what PhysicsRecord.cpp:183-185 reads from the returned track list);
 *   6. a stable counting sort of the selected hits into layer buckets, the
 *      hits of non-findable tracks (kept when onlyTracks is false) before
 *      those of findable tracks, as the two push_back loops order them
 *      (:84-104, :121-146).
 * A second kernel scans the per-event counts and a third gathers the output
 * columns, resolving DetectorId through the geometry table (DetectorGeometry.
 * cpp:4-30).
 *
 * Defined outcomes where the reference is undefined: hits of a track that
 * share a layer keep file order (the reference's std::sort is not stable;
 * for tracks of at most 16 hits libstdc++'s insertion sort is); layers 0 and
 * above max_layer do not count towards coverage (the reference indexes
 * covLayers outside its size); a detId lookup that runs past the table end
 * is "not found".
 */
#ifndef TRAX_INGEST_CUH
#define TRAX_INGEST_CUH

#include "trax_kernels.cuh"

namespace trax {

constexpr int kIngThreads = 256;
constexpr int kIngWarps = kIngThreads / 32;
constexpr uint32_t kIngBins = 256;

struct IngestRaw {
    const float *x, *y, *z;
    const uint32_t *layer, *det, *track;
    const float *pt;
    const uint32_t *event_offset;  /* [n_events + 1] */
    uint32_t n_events;
};

struct IngestCfg {
    float min_pt;
    uint32_t max_layer, used, only_tracks;
    int32_t num_tracks;
};

/* Per-hit scratch, each [n_raw], indexed at the event's raw offset. */
struct IngestScratch {
    uint32_t *ka, *va, *kb, *vb, *rank, *tstart, *tflag, *perm;
    uint32_t *tid, *tin, *tmid, *tout;
    uint32_t *n_out, *n_trk;  /* [n_events] */
};

struct IngShared {
    uint32_t cnt[kIngWarps][kIngBins];
    uint32_t tot[kIngBins];
    uint32_t s_warp[33];
    uint32_t carry, flag, cut;
};

/* Per-warp digit counts over warp-owned contiguous chunks of [0, n). */
template <class Digit>
__device__ void ing_count(IngShared &sh, uint32_t n, Digit digit)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t i = threadIdx.x; i < kIngWarps * kIngBins; i += blockDim.x)
        (&sh.cnt[0][0])[i] = 0;
    __syncthreads();
    const uint32_t chunk = (n + kIngWarps - 1) / kIngWarps;
    const uint32_t lo = min(w * chunk, n), hi = min(lo + chunk, n);
    for (uint32_t b = lo; b < hi; b += 32) {
        const uint32_t i = b + lane;
        const bool v = i < hi;
        const uint32_t d = v ? digit(i) : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(kFull, d);
        if (v && lane == (uint32_t)(__ffs(peers) - 1)) sh.cnt[w][d] += __popc(peers);
    }
    __syncthreads();
}

/* Per-warp counts -> per-warp scatter bases (bin-major, warp-minor: a
 * stable order); sh.tot gets the bin totals.  Returns true when one bin
 * holds all n items (the pass would not move anything). */
__device__ bool ing_bases(IngShared &sh, uint32_t n, uint32_t nbins)
{
    const uint32_t b = threadIdx.x;
    uint32_t s = 0;
    if (b < nbins)
        for (int w = 0; w < kIngWarps; ++w) {
            const uint32_t c = sh.cnt[w][b];
            sh.cnt[w][b] = s;
            s += c;
        }
    if (threadIdx.x == 0) sh.flag = 0;
    __syncthreads();
    if (b < nbins && s == n) sh.flag = 1;
    uint32_t total;
    const uint32_t base = block_exclusive_scan(b < nbins ? s : 0u, sh.s_warp, &total);
    if (b < nbins) {
        for (int w = 0; w < kIngWarps; ++w) sh.cnt[w][b] += base;
        sh.tot[b] = s;
    }
    __syncthreads();
    return sh.flag != 0;
}

/* Stable scatter of [0, n): emit(i, position). */
template <class Digit, class Emit>
__device__ void ing_scatter(IngShared &sh, uint32_t n, Digit digit, Emit emit)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t chunk = (n + kIngWarps - 1) / kIngWarps;
    const uint32_t lo = min(w * chunk, n), hi = min(lo + chunk, n);
    for (uint32_t b = lo; b < hi; b += 32) {
        const uint32_t i = b + lane;
        const bool v = i < hi;
        const uint32_t d = v ? digit(i) : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(kFull, d);
        uint32_t pos = 0;
        if (v) pos = sh.cnt[w][d] + __popc(peers & lt);
        __syncwarp();
        if (v && lane == (uint32_t)(__ffs(peers) - 1)) sh.cnt[w][d] += __popc(peers);
        __syncwarp();
        if (v) emit(i, pos);
    }
    __syncthreads();
}

/* Exclusive prefix of flag(i) over [0, n) in index order; out(i, excl,
 * flag) for each i.  Returns the total. */
template <class Flag, class Out>
__device__ uint32_t ing_scan(IngShared &sh, uint32_t n, Flag flag, Out out)
{
    if (threadIdx.x == 0) sh.carry = 0;
    __syncthreads();
    for (uint32_t b = 0; b < n; b += blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t f = i < n ? flag(i) : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(f, sh.s_warp, &tot);
        const uint32_t c = sh.carry;
        if (i < n) out(i, c + ex, f);
        __syncthreads();
        if (threadIdx.x == 0) sh.carry = c + tot;
        __syncthreads();
    }
    const uint32_t total = sh.carry;
    __syncthreads();
    return total;
}

/* The k-th hit (0-based) of positions [b, e) of a track in stable layer
 * order: distinct layers are visited in ascending order. */
__device__ uint32_t ing_kth_by_layer(const uint32_t *v, const uint32_t *layer, uint32_t b,
                                     uint32_t e, uint32_t k)
{
    long long prev = -1;
    uint32_t cum = 0;
    for (;;) {
        uint32_t L = 0xFFFFFFFFu;
        bool any = false;
        for (uint32_t p = b; p < e; ++p) {
            const uint32_t l = layer[v[p]];
            if ((long long)l > prev && (!any || l < L)) { L = l; any = true; }
        }
        if (!any) return v[b];  /* unreachable for k < e - b */
        uint32_t c = 0;
        for (uint32_t p = b; p < e; ++p) {
            if (layer[v[p]] != L) continue;
            if (cum + c == k) return v[p];
            ++c;
        }
        cum += c;
        prev = L;
    }
}

__global__ void __launch_bounds__(kIngThreads) k_ingest_event(IngestRaw raw, IngestCfg cfg,
                                                              IngestScratch sc,
                                                              uint32_t *layer_nhits)
{
    __shared__ IngShared sh;
    const uint32_t NB = 2 * cfg.max_layer; /* bucket bins; NB = not selected */
    for (uint32_t e = blockIdx.x; e < raw.n_events; e += gridDim.x) {
        const uint32_t o = raw.event_offset[e];
        const uint32_t n = raw.event_offset[e + 1] - o;

        /* 0: filters, kept hits first */
        auto drop = [&](uint32_t i) -> uint32_t {
            const uint32_t r = o + i;
            return ((cfg.only_tracks && raw.track[r] == 0u) || raw.pt[r] < cfg.min_pt) ? 1u : 0u;
        };
        ing_count(sh, n, drop);
        ing_bases(sh, n, 2);
        const uint32_t nk = sh.tot[0];
        {
            uint32_t *ka = sc.ka + o, *va = sc.va + o;
            ing_scatter(sh, n, drop, [&](uint32_t i, uint32_t pos) {
                ka[pos] = raw.track[o + i];
                va[pos] = o + i;
            });
        }

        /* 1: radix sort of the kept hits by track id */
        uint32_t *k0 = sc.ka + o, *v0 = sc.va + o, *k1 = sc.kb + o, *v1 = sc.vb + o;
        for (uint32_t sft = 0; sft < 32; sft += 8) {
            auto dig = [&](uint32_t i) -> uint32_t { return (k0[i] >> sft) & 0xFFu; };
            ing_count(sh, nk, dig);
            if (ing_bases(sh, nk, kIngBins)) continue;
            ing_scatter(sh, nk, dig, [&](uint32_t i, uint32_t pos) {
                k1[pos] = k0[i];
                v1[pos] = v0[i];
            });
            uint32_t *t = k0; k0 = k1; k1 = t;
            t = v0; v0 = v1; v1 = t;
        }

        /* 2: track segments */
        uint32_t *rank = sc.rank + o, *tstart = sc.tstart + o, *tflag = sc.tflag + o;
        const uint32_t ntr = ing_scan(
            sh, nk, [&](uint32_t i) -> uint32_t { return (i == 0 || k0[i] != k0[i - 1]) ? 1u : 0u; },
            [&](uint32_t i, uint32_t ex, uint32_t f) {
                rank[i] = ex + f - 1;
                if (f) tstart[ex] = i;
            });

        /* 3: findable rule */
        for (uint32_t t = threadIdx.x; t < ntr; t += blockDim.x) {
            const uint32_t b = tstart[t], en = t + 1 < ntr ? tstart[t + 1] : nk;
            uint32_t mask = 0;
            for (uint32_t p = b; p < en; ++p) {
                const uint32_t l = raw.layer[v0[p]];
                if (l >= 1 && l <= cfg.max_layer) mask |= 1u << (l - 1);
            }
            tflag[t] = (mask & cfg.used) == cfg.used ? 1u : 0u;
        }
        __syncthreads();

        /* 4: data.tracks limit */
        uint32_t cutoff = ntr;
        if (cfg.num_tracks == 0) {
            cutoff = 0;
        } else if (cfg.num_tracks > 0) {
            if (threadIdx.x == 0) sh.cut = ntr;
            __syncthreads();
            ing_scan(sh, ntr, [&](uint32_t t) -> uint32_t { return tflag[t]; },
                     [&](uint32_t t, uint32_t ex, uint32_t f) {
                         if (f && ex + 1 == (uint32_t)cfg.num_tracks) sh.cut = t + 1;
                     });
            cutoff = sh.cut;
            __syncthreads();
        }

        /* 5: findable track records */
        const uint32_t nf = ing_scan(
            sh, cutoff, [&](uint32_t t) -> uint32_t { return tflag[t]; },
            [&](uint32_t t, uint32_t ex, uint32_t f) {
                if (!f) return;
                const uint32_t b = tstart[t], en = t + 1 < ntr ? tstart[t + 1] : nk;
                const uint32_t cnt = en - b;
                sc.tid[o + ex] = k0[b];
                sc.tin[o + ex] = ing_kth_by_layer(v0, raw.layer, b, en, 0);
                sc.tmid[o + ex] = ing_kth_by_layer(v0, raw.layer, b, en, cnt / 2);
                sc.tout[o + ex] = ing_kth_by_layer(v0, raw.layer, b, en, cnt - 1);
            });

        /* 6: layer buckets */
        auto bucket = [&](uint32_t p) -> uint32_t {
            const uint32_t t = rank[p];
            const uint32_t l = raw.layer[v0[p]];
            const bool in = t < cutoff && l >= 1 && l <= cfg.max_layer && (tflag[t] || !cfg.only_tracks);
            return in ? 2 * (l - 1) + tflag[t] : NB;
        };
        ing_count(sh, nk, bucket);
        ing_bases(sh, nk, NB + 1);
        {
            uint32_t *perm = sc.perm + o;
            ing_scatter(sh, nk, bucket, [&](uint32_t p, uint32_t pos) { perm[pos] = v0[p]; });
        }
        if (threadIdx.x < cfg.max_layer)
            layer_nhits[(size_t)e * cfg.max_layer + threadIdx.x] =
                sh.tot[2 * threadIdx.x] + sh.tot[2 * threadIdx.x + 1];
        if (threadIdx.x == 0) {
            sc.n_out[e] = nk - sh.tot[NB];
            sc.n_trk[e] = nf;
        }
        __syncthreads();
    }
}

/* Exclusive offsets of the per-event output and track counts.  One CTA. */
__global__ void __launch_bounds__(1024) k_ingest_offsets(const uint32_t *n_out, const uint32_t *n_trk,
                                                         uint32_t n_events, uint32_t *out_off,
                                                         uint32_t *trk_off)
{
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_carry[2];
    if (threadIdx.x < 2) s_carry[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t b = 0; b < n_events; b += blockDim.x) {
        const uint32_t e = b + threadIdx.x;
        uint32_t t0, t1;
        const uint32_t x0 = block_exclusive_scan(e < n_events ? n_out[e] : 0u, s_warp, &t0);
        const uint32_t x1 = block_exclusive_scan(e < n_events ? n_trk[e] : 0u, s_warp, &t1);
        if (e < n_events) {
            out_off[e] = s_carry[0] + x0;
            trk_off[e] = s_carry[1] + x1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_carry[0] += t0;
            s_carry[1] += t1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out_off[n_events] = s_carry[0];
        trk_off[n_events] = s_carry[1];
    }
}

/* DetectorGeometry::resolveDetId (DetectorGeometry.cpp:4-30): the same
 * binary search over the geometry's detId column; -1 when absent. */
__device__ __forceinline__ int ing_resolve(const uint32_t *ids, uint32_t n, uint32_t det)
{
    int imin = 0, imax = (int)n;
    while (imin < imax) {
        const int imid = imin + (imax - imin) / 2;
        if (ids[imid] < det) imin = imid + 1;
        else imax = imid;
    }
    return (imax == imin && imin < (int)n && ids[imin] == det) ? imin : -1;
}

struct IngestOut {
    float *x, *y, *z;
    uint32_t *layer, *det, *hitid, *event;
    uint32_t cap;
    uint32_t *tid, *tin, *tmid, *tout;
    uint32_t tcap;
};

/* HitCollection::addWithValue of the bucketed hits (HitCollection.cpp:
 * 121-146) and the track list, at the scanned offsets. */
__global__ void __launch_bounds__(256) k_ingest_gather(IngestRaw raw, IngestScratch sc,
                                                       const uint32_t *out_off,
                                                       const uint32_t *trk_off,
                                                       const uint32_t *det_ids, uint32_t n_det,
                                                       IngestOut out)
{
    for (uint32_t e = blockIdx.x; e < raw.n_events; e += gridDim.x) {
        const uint32_t o = raw.event_offset[e];
        const uint32_t d0 = out_off[e], cnt = out_off[e + 1] - d0;
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
            const uint32_t d = d0 + i;
            if (d >= out.cap) break;
            const uint32_t r = sc.perm[o + i];
            out.x[d] = raw.x[r];
            out.y[d] = raw.y[r];
            out.z[d] = raw.z[r];
            out.layer[d] = raw.layer[r];
            const int idx = ing_resolve(det_ids, n_det, raw.det[r]);
            out.det[d] = idx >= 0 ? (uint32_t)idx : raw.det[r];
            out.hitid[d] = raw.track[r];
            out.event[d] = e;
        }
        if (out.tid) {
            const uint32_t t0 = trk_off[e], tc = trk_off[e + 1] - t0;
            for (uint32_t i = threadIdx.x; i < tc; i += blockDim.x) {
                const uint32_t d = t0 + i;
                if (d >= out.tcap) break;
                out.tid[d] = sc.tid[o + i];
                out.tin[d] = sc.tin[o + i];
                out.tmid[d] = sc.tmid[o + i];
                out.tout[d] = sc.tout[o + i];
            }
        }
    }
}

}  // namespace trax

#endif /* TRAX_INGEST_CUH */
