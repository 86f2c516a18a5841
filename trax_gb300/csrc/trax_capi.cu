/*
 * trax_capi.cu -- the C-ABI of include/trax.h over the sm_103a kernels.
 *
 * The four stage entry points mirror the reference's operator methods
 * (GridBuilder::run, PairGeneratorBeamspot::run, TripletThetaPhiPredictor::run,
 * TripletThetaPhiFilter::run) but never synchronise: every size the
 * reference downloads to the host to allocate the next buffer
 * (PairGeneratorBeamspot.cpp:120, TripletThetaPhiPredictor.cpp:59,
 * TripletThetaPhiFilter.cpp:82) stays on the device, and outputs are bounded
 * by caller capacities.  The batched pipeline runs the same kernels from one
 * CUDA graph.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "trax_kernels.cuh"
#include "trax_ingest.cuh"
#include "trax_physics.cuh"

using namespace trax;

namespace {

constexpr int kTimerSlots = 64;
constexpr int kScanItems = 16;      /* items per thread in k_scan */
constexpr int kScanThreads = 256;
constexpr int kTileItems = 32;      /* items per fused pair / predict tile (one warp) */
constexpr uint32_t kSplitSeedHits = 1u << 20;  /* trax_seed_batch pipelines two halves from here */
/* pair accepts an outer hit keeps for the split store: more than 32 is rare
 * below pile-up (an outer hit with more walks again in the store) */
constexpr uint32_t kPairKeepSplit = 32;
constexpr uint32_t kDefaultRunWalk = 48;  /* see trax_set_tuning */
constexpr uint32_t kDefaultIndexMin = 16;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

/* The input columns (x, y, z, layer, detector id, hit id, event) the batched
 * chain reads: x, y, z, layer and event.  The detector and hit ids stay on
 * the host -- the chain's tracklets come back as input positions and its
 * sorted hits are never returned -- so their buffers are neither allocated
 * nor uploaded. */
constexpr int kChainCols[5] = {0, 1, 2, 3, 6};

/* One of the two batches a context can have in flight
 * (trax_submit_batch / trax_wait_batch): its own inputs, upload staging,
 * graph and result counts. */
struct AsyncSlot {
    DevBuf in_cols[7], seg;
    DevBuf res[3], res_off;       /* the batch's tracklets and offsets, kept until read */
    uint32_t *h_meta = nullptr;   /* pinned: segment starts, counts, (events, hits) */
    DevState *h_snap = nullptr;   /* pinned: the run's counts, written by the device */
    cudaEvent_t h2d_done = nullptr, done = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool busy = false;
    uint32_t ticket = 0, capacity = 0, n_off = 0;
    uint32_t *out[4] = {};        /* the caller's host outputs: hit1..3, offsets */
};

}  // namespace

struct trax_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    bool configured = false;
    int pair_generator = TRAX_PAIRS_BEAMSPOT;  /* used by the batched pipeline */
    trax_config cfg{};
    KParams kp{};
    DevState *d_state = nullptr;
    DevState *h_state = nullptr;          /* pinned mirror */
    uint32_t *h_stage = nullptr;          /* pinned staging for small uploads */
    size_t h_stage_words = 0;
    cudaEvent_t stage_free = nullptr;     /* last upload from h_stage done */
    DevBuf seg, g_start, g_base, slots, pexcl, cexcl, st0, st1, st2, st3, zi, conn_keys, conn_sums;
    DevBuf ing;   /* event ingest scratch */
    DevBuf phys;  /* physics evaluation scratch */
    DevBuf prec;  /* prediction store records */
    DevBuf zp;    /* input position of each z-index entry */
    DevBuf ptile; /* prediction tile totals / prefixes */
    DevBuf fmask; /* filter accept mask words and their positions */
    DevBuf zphi;  /* packed (z, phi) of the sorted hits */
    DevBuf zh;    /* half-precision z of the sorted hits (candidate screen) */
    DevBuf pkeep; /* per outer hit: its first kept pair accepts (split pair stage) */
    DevBuf gscr;  /* grid build: each hit's cell and phi, for segments beyond the registers */
    DevBuf xyzp;  /* packed (x, y, z, phi) of the sorted hits */
    cudaEvent_t timers[kTimerSlots] = {};
    int blk_pair = 0, blk_pair0 = 0, blk_pair_lane = 0, blk_pair_count = 0, blk_pair_store = 0, blk_sector = 0, blk_pred = 0, blk_filter = 0, blk_scan = 0, blk_small = 0;
    /* resident blocks per SM that fit, per candidate kernel (occupancy), and
     * the tuning's cap on them (0: none) */
    int occ_pair = 0, occ_pair0 = 0, occ_pair_lane = 0, occ_pair_count = 0, occ_pair_store = 0,
        occ_sector = 0, occ_pred = 0, occ_filter = 0, occ_pstore = 0, occ_fstore = 0;
    uint32_t blocks_cap = 0;
    int blk_pstore = 0, blk_fstore = 0;  /* the store passes: their own occupancy */

    /* batched pipeline */
    bool reserved = false;
    uint32_t r_events = 0, r_layers = 0, r_hits = 0, r_pairs = 0, r_cands = 0, r_trk = 0;
    trax_grid_cfg r_grid{};
    DevBuf in_cols[7], srt_cols[9], grid_buf, pairs_buf, pair_off, cands_buf, cand_off;
    DevBuf trk_cols[3], trk_off, trk_map[3], r_seg;
    uint32_t gb_C = 0, gb_P1 = 0, gb_avg = 0;  /* cached k_grid_build launch plan */
    int gb_warps = 0, gb_per_sm = 0;
    uint32_t gb_stage = 0;                /* k_grid_build staged-segment capacity */
    uint32_t gb_cells = 0;                /* k_grid_build per-warp table cells */
    /* dense segments on fine grids: k_grid_build_wb with gb_wb_warps warps,
     * bands of gb_R2 z rows, gb_wb_smem bytes of shared memory */
    bool gb_wb = false;
    uint32_t gb_R2 = 0, gb_wb_warps = 0;
    size_t gb_wb_smem = 0;
    cudaGraphExec_t graph = nullptr;
    uint32_t staged_events = 0, staged_hits = 0;
    /* streaming submission: two slots, uploads on their own stream */
    AsyncSlot aslot[2];
    cudaStream_t copy_stream = nullptr;   /* uploads */
    cudaStream_t d2h_stream = nullptr;    /* result downloads */
    uint32_t next_ticket = 0;
    /* per-kernel timing marks (events recorded between launches) */
    bool profiling = false;
    int n_marks = 0;
    const char *mark_names[kTimerSlots] = {};
    int launches = 0;                     /* kernels enqueued by the last pipeline */
};

namespace {

trax_status fail(trax_ctx *c, trax_status s, const std::string &msg)
{
    if (c) c->err = msg;
    return s;
}

/* Executable graphs hold the reserved buffers' addresses; any change of the
 * captured parameters or buffers drops them all (they are re-captured on
 * their next launch). */
bool has_graph(const trax_ctx *ctx)
{
    return ctx->graph || ctx->aslot[0].graph || ctx->aslot[1].graph;
}

void drop_graphs(trax_ctx *ctx)
{
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
    for (auto &a : ctx->aslot) {
        if (a.graph) cudaGraphExecDestroy(a.graph);
        a.graph = nullptr;
    }
}

/* Frees the streaming slots (after their work is done); trax_submit_batch
 * creates them again at the reservation's sizes. */
void free_async(trax_ctx *ctx)
{
    for (auto &a : ctx->aslot) {
        if (a.done) cudaEventSynchronize(a.done);
        if (a.graph) cudaGraphExecDestroy(a.graph);
        for (auto &b : a.in_cols) if (b.p) cudaFree(b.p);
        for (auto &b : a.res) if (b.p) cudaFree(b.p);
        if (a.res_off.p) cudaFree(a.res_off.p);
        if (a.seg.p) cudaFree(a.seg.p);
        if (a.h_meta) cudaFreeHost(a.h_meta);
        if (a.h_snap) cudaFreeHost(a.h_snap);
        if (a.h2d_done) cudaEventDestroy(a.h2d_done);
        if (a.done) cudaEventDestroy(a.done);
        a = AsyncSlot{};
    }
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->d2h_stream) cudaStreamDestroy(ctx->d2h_stream);
    ctx->copy_stream = ctx->d2h_stream = nullptr;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, TRAX_ERR_DEVICE, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

/* in_graph: the buffer may be referenced by a captured graph (every scratch
 * buffer of the chain); st3, used only by the standalone scan, is not. */
trax_status ensure(trax_ctx *ctx, DevBuf &b, size_t bytes, bool in_graph = true)
{
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return TRAX_OK;
    if (in_graph && ctx->reserved && has_graph(ctx)) {
        /* buffers captured in the graph must not move */
        return fail(ctx, TRAX_ERR_OOM, "scratch beyond the reserved size");
    }
    if (b.p) {
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaFree(b.p));
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, TRAX_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.bytes = want;
    return TRAX_OK;
}

trax_status ensure_stage(trax_ctx *ctx, size_t words)
{
    if (ctx->stage_free) CK(cudaEventSynchronize(ctx->stage_free));
    if (ctx->h_stage_words >= words) return TRAX_OK;
    if (ctx->h_stage) CK(cudaFreeHost(ctx->h_stage));
    ctx->h_stage = nullptr;
    size_t want = std::max<size_t>(words + words / 4, 1024);
    CK(cudaMallocHost(&ctx->h_stage, want * 4));
    ctx->h_stage_words = want;
    return TRAX_OK;
}

uint32_t tiles_for(uint32_t n, uint32_t per) { return (n + per - 1) / per + 1; }

void fill_grid_params(KParams &kp, const trax_grid_cfg *g)
{
    kp.n_layers = g->n_layers;
    kp.nz = g->n_sectors_z;
    kp.nphi = g->n_sectors_phi;
    kp.C = (g->n_sectors_z + 1) * (g->n_sectors_phi + 1);
    kp.sz_z = trax_sector_size_z(g->n_sectors_z);
    kp.sz_phi = trax_sector_size_phi(g->n_sectors_phi);
    kp.inv_sz_z = 1.0f / kp.sz_z;
    kp.inv_sz_phi = 1.0f / kp.sz_phi;
}

/* The grid build needs no layer-triplet configuration (GridBuilder::run
 * takes none, GridBuilder.h:42); the later stages do. */
trax_status check_grid(trax_ctx *ctx, const trax_grid_cfg *g, bool need_cfg = true)
{
    if (need_cfg && !ctx->configured) return fail(ctx, TRAX_ERR_BAD_ARG, "trax_configure not called");
    if (!g || g->n_sectors_z == 0 || g->n_sectors_phi == 0 || g->n_layers == 0 ||
        g->n_layers > TRAX_MAX_LAYERS)
        return fail(ctx, TRAX_ERR_BAD_ARG, "bad grid configuration");
    if ((uint64_t)(g->n_sectors_z + 1) * (g->n_sectors_phi + 1) > 65536)
        return fail(ctx, TRAX_ERR_BAD_ARG, "grid has more than 65536 cells per layer");
    for (uint32_t i = 0; i < ctx->cfg.n_layer_triplets; ++i) {
        const trax_layer_triplet &t = ctx->cfg.triplets[i];
        if (t.layer1 > g->n_layers || t.layer2 > g->n_layers || t.layer3 > g->n_layers)
            return fail(ctx, TRAX_ERR_BAD_ARG, "layer triplet uses a layer outside the grid");
    }
    return TRAX_OK;
}

/* Grid sizes of the candidate kernels: the blocks per SM that fit, capped
 * by the tuning's blocks_per_sm. */
void apply_launch_cap(trax_ctx *ctx)
{
    auto grid = [&](int occ) {
        int b = std::max(occ, 1);
        if (ctx->blocks_cap) b = std::min<int>(b, (int)ctx->blocks_cap);
        return ctx->sm_count * b;
    };
    ctx->blk_pair = grid(ctx->occ_pair);
    ctx->blk_pair0 = grid(ctx->occ_pair0);
    ctx->blk_pair_lane = grid(ctx->occ_pair_lane);
    ctx->blk_pair_count = grid(ctx->occ_pair_count);
    ctx->blk_pair_store = grid(ctx->occ_pair_store);
    ctx->blk_sector = grid(ctx->occ_sector);
    ctx->blk_pred = grid(ctx->occ_pred);
    ctx->blk_filter = grid(ctx->occ_filter);
    ctx->blk_pstore = grid(ctx->occ_pstore);
    ctx->blk_fstore = grid(ctx->occ_fstore);
}

/* Launch plan of k_grid_build for C cells of nphi + 1 columns and segments
 * of avg_seg hits on average; computed outside any stream capture and
 * cached.
 *   staging  segments up to 1.5x the average (at least 512 hits) are staged
 *            in shared memory for coalesced column writes, within half of
 *            the shared-memory budget;
 *   warps    enough for 1.5x the average segment at kGridItems * 32 hits a
 *            warp (kGridItemsBanded with bands; at most 32);
 *   tables   per-warp cell tables of Ct cells: the whole grid when it fits,
 *            else whole z rows -- at least min(4, Z + 1) of them, with fewer
 *            warps if need be -- and the kernel works in bands of rows (the
 *            table work of a segment grows with the warps times the cells its
 *            rows occupy, not with the number of bands, so more warps and
 *            narrower bands win: 8 rows 0.75 ms, 4 rows 0.72 ms at 256 x 192). */
/* The grid build's scratch: each hit's (cell, phi), then the warp-band
 * kernel's band list (one word per hit). */
size_t gscr_bytes(size_t n_hits) { return (n_hits + 1) * 8 + n_hits * 4 + 16; }

constexpr uint32_t kWbWarps = 16;  /* k_grid_build_wb: warps per CTA */
constexpr uint32_t kWbRows = 1;    /* k_grid_build_wb: z rows per band */

trax_status grid_plan(trax_ctx *ctx, uint32_t C, uint32_t avg_seg)
{
    const uint32_t P1 = ctx->kp.nphi + 1, rows = C / P1;
    if (ctx->gb_C == C && ctx->gb_P1 == P1 && ctx->gb_avg == avg_seg && ctx->gb_warps > 0)
        return TRAX_OK;
    const size_t budget = std::min<size_t>(ctx->smem_optin, 200 * 1024);
    uint32_t stage = std::max<uint32_t>(512, (3 * avg_seg / 2 + 255) / 256 * 256);
    while (stage > 256 && 8ull * stage > budget / 2) stage -= 256;
    auto table = [&](long w) -> uint64_t { return (budget - 8ull * stage) / (4ull * (w + 1)); };
    auto warps_for = [&](long items) {
        const long per_warp = 32 * items;
        const long w = (long)((3ull * avg_seg / 2 + per_warp - 1) / per_warp);
        return std::min<long>(std::max<long>(w, 1), 32);
    };
    /* the banded instance holds more hits per lane */
    long W = warps_for(kGridItems);
    if (C > table(W)) W = warps_for(kGridItemsBanded);
    const uint64_t want = C <= table(W) ? C : (uint64_t)std::min<uint32_t>(4, rows) * P1;
    while (W > 1 && table(W) < want) --W;
    uint64_t Ct = std::min<uint64_t>(table(W), C);
    if (Ct < C) Ct = Ct / P1 * P1;
    if (Ct < P1) {
        stage = 0;
        W = 1;
        Ct = std::min<uint64_t>(table(1), C);
        if (Ct < C) Ct = Ct / P1 * P1;
    }
    if (Ct < P1) return fail(ctx, TRAX_ERR_BAD_ARG, "grid too large for shared memory");
    int per_sm = 0;
    const size_t smem = ((size_t)(W + 1) * Ct + 2ull * stage) * 4;
    if (Ct < C)
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grid_build<true>, (int)W * 32, smem));
    else
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grid_build<false>, (int)W * 32, smem));
    ctx->gb_stage = stage;
    ctx->gb_C = C;
    ctx->gb_P1 = P1;
    ctx->gb_avg = avg_seg;
    ctx->gb_warps = (int)W;
    ctx->gb_cells = (uint32_t)Ct;
    ctx->gb_per_sm = per_sm < 1 ? 1 : per_sm;
    /* a fine grid (bands) whose average segment is beyond the registers of
     * k_grid_build (each hit's cell would go through the scratch column):
     * warp bands in k_grid_build_wb, two or more CTAs per SM */
    ctx->gb_wb = false;
    if (Ct < C && avg_seg > (uint32_t)W * 32u * (uint32_t)kGridItemsBanded) {
        const uint32_t Wb = kWbWarps, R2 = kWbRows, nbm = (rows + R2 - 1) / R2;
        const uint32_t stage_b = std::max<uint32_t>(512, (3 * avg_seg / 2 + 255) / 256 * 256);
        const size_t tabw = std::max<size_t>((size_t)nbm * Wb, (size_t)Wb * R2 * P1);
        const size_t smem_b = ((size_t)stage_b + tabw + nbm + 1) * 4;
        int per_sm_b = 0;
        if (smem_b <= ctx->smem_optin)
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_b, k_grid_build_wb,
                                                             (int)Wb * 32, smem_b));
        if (per_sm_b >= 2) {
            ctx->gb_wb = true;
            ctx->gb_R2 = R2;
            ctx->gb_wb_warps = Wb;
            ctx->gb_wb_smem = smem_b;
            ctx->gb_stage = stage_b;
            ctx->gb_per_sm = per_sm_b;
        }
    }
    return TRAX_OK;
}

/* Called after every kernel launch: counts it and, when profiling, records
 * a timing event named after it (timer slot 0 is the pipeline start). */
trax_status mark(trax_ctx *ctx, const char *name)
{
    ++ctx->launches;
    if (!ctx->profiling || ctx->n_marks + 1 >= kTimerSlots) return TRAX_OK;
    ++ctx->n_marks;
    ctx->mark_names[ctx->n_marks] = name;
    /* External: inside a stream capture the record becomes a graph node that
     * fires on every replay */
    CK(cudaEventRecordWithFlags(ctx->timers[ctx->n_marks], ctx->stream, cudaEventRecordExternal));
    return TRAX_OK;
}

trax_status begin_marks(trax_ctx *ctx)
{
    ctx->n_marks = 0;
    ctx->launches = 0;
    if (ctx->profiling)
        CK(cudaEventRecordWithFlags(ctx->timers[0], ctx->stream, cudaEventRecordExternal));
    return TRAX_OK;
}

trax_status set_sizes(trax_ctx *ctx, uint32_t n_events, uint32_t n_hits)
{
    trax_status s = ensure_stage(ctx, 2);
    if (s != TRAX_OK) return s;
    ctx->h_stage[0] = n_events;
    ctx->h_stage[1] = n_hits;
    CK(cudaMemcpyAsync(ctx->d_state, ctx->h_stage, 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->stage_free, ctx->stream));
    return TRAX_OK;
}

/* ---------------------------------------------------------------------- */
/* Stage enqueue functions shared by the stage API and the graph pipeline. */

trax_status enqueue_grid(trax_ctx *ctx, const InCols &in, const SortedCols &out,
                         const uint32_t *seg_start, const uint32_t *seg_n, uint32_t *grid,
                         uint32_t max_segs, uint32_t n_hits)
{
    const KParams &kp = ctx->kp;
    trax_status s = grid_plan(ctx, kp.C, max_segs ? n_hits / max_segs : 0);
    if (s != TRAX_OK) return s;
    const int W = ctx->gb_warps, per_sm = ctx->gb_per_sm;
    const size_t smem = ((size_t)(W + 1) * ctx->gb_cells + 2ull * ctx->gb_stage) * 4;
    if ((s = ensure(ctx, ctx->gscr, gscr_bytes(n_hits))) != TRAX_OK) return s;
    uint2 *cscr = (uint2 *)ctx->gscr.p;
    uint32_t blocks = std::min<uint32_t>(max_segs, (uint32_t)(ctx->sm_count * per_sm));
    if (blocks == 0) blocks = 1;
    CK(cudaMemsetAsync(&ctx->d_state->gb_next, 0, 4, ctx->stream));  /* segment counter */
    if (ctx->gb_wb)
        k_grid_build_wb<<<blocks, ctx->gb_wb_warps * 32, ctx->gb_wb_smem, ctx->stream>>>(
            kp, in, out, seg_start, seg_n, grid, ctx->gb_stage, ctx->gb_R2, cscr,
            (uint32_t *)(cscr + (size_t)n_hits + 1), ctx->d_state);
    else if (ctx->gb_cells < kp.C)
        k_grid_build<true><<<blocks, W * 32, smem, ctx->stream>>>(
            kp, in, out, seg_start, seg_n, grid, ctx->gb_stage, ctx->gb_cells, cscr, ctx->d_state);
    else
        k_grid_build<false><<<blocks, W * 32, smem, ctx->stream>>>(
            kp, in, out, seg_start, seg_n, grid, ctx->gb_stage, ctx->gb_cells, cscr, ctx->d_state);
    CK(cudaGetLastError());
    return mark(ctx, "grid_build");
}

/* Pair stage with either generator: TRAX_PAIRS_BEAMSPOT (items are the
 * outer hits, k_pair_fused) or TRAX_PAIRS_SECTOR (items are the inner hits,
 * k_pair_sector).  Both write pairs (inner, outer) and per-group offsets. */
/* The candidate kernels read the packed columns; a stage call without them
 * is a bug of this library, reported instead of faulting on the device. */
trax_status need_packed(trax_ctx *ctx, const SortedCols &h)
{
    if (!h.zphi || !h.zh || !h.xyzp)
        return fail(ctx, TRAX_ERR_BAD_ARG, "packed hit columns missing");
    return TRAX_OK;
}

trax_status enqueue_pairs(trax_ctx *ctx, const SortedCols &h, const uint32_t *grid, uint2 *pairs,
                          uint32_t *pair_offsets, uint32_t pair_cap, uint32_t slot_cap,
                          uint32_t max_groups, int generator)
{
    const bool sector = generator == TRAX_PAIRS_SECTOR;
    const KParams &kp = ctx->kp;
    trax_status s = need_packed(ctx, h);
    if (s != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_start, (size_t)max_groups * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_base, (size_t)(max_groups + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->slots, (size_t)slot_cap * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pexcl, (size_t)(slot_cap + 1) * 4)) != TRAX_OK) return s;
    const uint32_t ntile = tiles_for(slot_cap, kTileItems);
    if ((s = ensure(ctx, ctx->st0, (size_t)ntile * 8)) != TRAX_OK) return s;
    uint32_t *g_start = (uint32_t *)ctx->g_start.p, *g_base = (uint32_t *)ctx->g_base.p;
    uint2 *slots = (uint2 *)ctx->slots.p;
    uint32_t *pexcl = (uint32_t *)ctx->pexcl.p;
    DevState *st = ctx->d_state;

    k_pair_groups<<<1, 1024, 0, ctx->stream>>>(kp, grid, g_start, g_base, st, sector);
    if ((s = mark(ctx, "pair_groups")) != TRAX_OK) return s;
    k_pair_slots<<<ctx->blk_small, 256, 0, ctx->stream>>>(kp, g_start, g_base, slots, slot_cap, st);
    if ((s = mark(ctx, "pair_slots")) != TRAX_OK) return s;
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->st0.p, 0, (size_t)ntile * 8, ctx->stream));
    if (!sector && kp.pair_record == 3) {
        /* split: count -> scan of the counts -> store (no look-back waits) */
        if ((s = ensure(ctx, ctx->pkeep, (size_t)slot_cap * kPairKeepSplit * 4)) != TRAX_OK) return s;
        uint32_t *pkeep = (uint32_t *)ctx->pkeep.p;
        k_pair_count_lane<<<ctx->blk_pair_count, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, pkeep, kPairKeepSplit, st);
        if ((s = mark(ctx, "pair_gen")) != TRAX_OK) return s;
        const uint32_t stile = tiles_for(slot_cap, kScanItems * kScanThreads);
        CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));
        CK(cudaMemsetAsync(ctx->st0.p, 0, (size_t)stile * 8, ctx->stream));
        k_scan<kScanItems><<<std::min<uint32_t>(ctx->blk_scan, stile), kScanThreads, 0, ctx->stream>>>(
            pexcl, pexcl, &st->n_outer, slot_cap, &st->n_pairs, 0,
            (unsigned long long *)ctx->st0.p, st);
        if ((s = mark(ctx, "pair_scan")) != TRAX_OK) return s;
        k_pair_store_lane<<<ctx->blk_pair_store, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, pkeep, kPairKeepSplit, pairs,
            pair_cap, st);
        if ((s = mark(ctx, "pair_store")) != TRAX_OK) return s;
    } else if (sector)
        k_pair_sector<<<ctx->blk_sector, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.zphi, slots, slot_cap, pexcl, pairs, pair_cap,
            (unsigned long long *)ctx->st0.p, st);
    else if (kp.pair_record == 2 || kp.pair_record == 4)
        (kp.pair_record == 2 ? k_pair_lane<kPairKeep> : k_pair_lane<kPairKeepWide>)
            <<<ctx->blk_pair_lane, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, pairs, pair_cap,
            (unsigned long long *)ctx->st0.p, st);
    else if (kp.pair_record)
        k_pair_fused<true><<<ctx->blk_pair, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, pairs, pair_cap,
            (unsigned long long *)ctx->st0.p, st);
    else
        k_pair_fused<false><<<ctx->blk_pair0, kFusedThreads, 0, ctx->stream>>>(
            kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, pairs, pair_cap,
            (unsigned long long *)ctx->st0.p, st);
    if (sector || kp.pair_record != 3)
        if ((s = mark(ctx, "pair_gen")) != TRAX_OK) return s;
    k_group_offsets<<<ctx->blk_small, 256, 0, ctx->stream>>>(g_base, pexcl, pair_offsets, kp.n_lt,
                                                             slot_cap, &st->n_pairs, pair_cap,
                                                             TRAX_DETAIL_PAIR_CAPACITY, st);
    CK(cudaGetLastError());
    return mark(ctx, "pair_offsets");
}

/* The pair stage's count passes alone (beam-spot generator): per outer hit
 * the distinct pairs it makes, their scan, and the per-group offsets --
 * what the chain would store, without storing it. */
trax_status enqueue_pair_count(trax_ctx *ctx, const SortedCols &h, const uint32_t *grid,
                               uint32_t *pair_offsets, uint32_t slot_cap, uint32_t max_groups)
{
    const KParams &kp = ctx->kp;
    trax_status s = need_packed(ctx, h);
    if (s != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_start, (size_t)max_groups * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_base, (size_t)(max_groups + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->slots, (size_t)slot_cap * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pexcl, (size_t)(slot_cap + 1) * 4)) != TRAX_OK) return s;
    const uint32_t stile = tiles_for(slot_cap, kScanItems * kScanThreads);
    if ((s = ensure(ctx, ctx->st0, (size_t)std::max(stile, tiles_for(slot_cap, kTileItems)) * 8)) != TRAX_OK)
        return s;
    uint32_t *g_start = (uint32_t *)ctx->g_start.p, *g_base = (uint32_t *)ctx->g_base.p;
    uint2 *slots = (uint2 *)ctx->slots.p;
    uint32_t *pexcl = (uint32_t *)ctx->pexcl.p;
    DevState *st = ctx->d_state;
    k_pair_groups<<<1, 1024, 0, ctx->stream>>>(kp, grid, g_start, g_base, st, false);
    k_pair_slots<<<ctx->blk_small, 256, 0, ctx->stream>>>(kp, g_start, g_base, slots, slot_cap, st);
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));
    k_pair_count_lane<<<ctx->blk_pair_count, kFusedThreads, 0, ctx->stream>>>(
        kp, grid, h.xyzp, h.zphi, slots, slot_cap, pexcl, nullptr, 0, st);
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->st0.p, 0, (size_t)stile * 8, ctx->stream));
    k_scan<kScanItems><<<std::min<uint32_t>(ctx->blk_scan, stile), kScanThreads, 0, ctx->stream>>>(
        pexcl, pexcl, &st->n_outer, slot_cap, &st->n_pairs, 0, (unsigned long long *)ctx->st0.p, st);
    k_group_offsets<<<ctx->blk_small, 256, 0, ctx->stream>>>(g_base, pexcl, pair_offsets, kp.n_lt,
                                                             slot_cap, &st->n_pairs, 0xffffffffu,
                                                             TRAX_DETAIL_PAIR_CAPACITY, st);
    CK(cudaGetLastError());
    return TRAX_OK;
}

/* Per-cell z index of the sorted hits (k_zindex) into ctx->zi. */
trax_status enqueue_zindex(trax_ctx *ctx, const SortedCols &h, const uint32_t *grid,
                           uint32_t max_hits)
{
    if (ctx->kp.zi_min >= 256) return TRAX_OK; /* no cell is searched: no index */
    trax_status s = ensure(ctx, ctx->zi, (size_t)max_hits * 8 + 8);
    if (s != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->zp, (size_t)max_hits * 4 + 4)) != TRAX_OK) return s;
    k_zindex<<<ctx->blk_small * 4, 256, 0, ctx->stream>>>(
        grid, ctx->kp.n_layers * ctx->kp.C, ctx->kp.zi_min, h.zphi, (float2 *)ctx->zi.p,
        (uint32_t *)ctx->zp.p, ctx->d_state);
    CK(cudaGetLastError());
    return mark(ctx, "zindex");
}

trax_status enqueue_predict(trax_ctx *ctx, const SortedCols &h, const uint32_t *grid,
                            const uint2 *pairs, const uint32_t *pair_offsets, uint32_t pair_cap,
                            uint2 *cands, uint32_t *cand_offsets, uint32_t cand_cap,
                            uint32_t max_groups)
{
    const KParams &kp = ctx->kp;
    trax_status s = need_packed(ctx, h);
    if (s != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->cexcl, (size_t)(pair_cap + 1) * 4)) != TRAX_OK) return s;
    const uint32_t ptiles = tiles_for(pair_cap, 32) + 1;
    const uint32_t ntile = tiles_for(ptiles, kScanItems * kScanThreads);
    if ((s = ensure(ctx, ctx->st1, (size_t)ntile * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->ptile, (size_t)ptiles * 4)) != TRAX_OK) return s;
    /* staged accepts (at most one per candidate), the tiles' stage offsets
     * and the walk records (each stands for more than kPredKeep candidates) */
    const uint32_t stage_cap = cand_cap ? cand_cap : 1;
    const uint32_t walk_cap = stage_cap / (kPredKeep + 1) + 1;
    const size_t stage_off = (size_t)walk_cap * sizeof(PredRec);
    const size_t sbase_off = stage_off + (((size_t)stage_cap * 4 + 255) & ~(size_t)255);
    if ((s = ensure(ctx, ctx->prec, sbase_off + (size_t)ptiles * 4)) != TRAX_OK) return s;
    uint32_t *cexcl = (uint32_t *)ctx->cexcl.p;
    uint32_t *ptile = (uint32_t *)ctx->ptile.p;
    PredRec *walks = (PredRec *)ctx->prec.p;
    uint32_t *stage = (uint32_t *)((char *)ctx->prec.p + stage_off);
    uint32_t *tile_sbase = (uint32_t *)((char *)ctx->prec.p + sbase_off);
    DevState *st = ctx->d_state;
    /* the pair total is st->n_pairs: written by the pair stage, or copied
     * from pair_offsets[G] by trax_triplet_predict */
    CK(cudaMemsetAsync(&st->n_prec, 0, 8, ctx->stream));  /* n_prec, n_pwalk */
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));  /* work tickets */
    (kp.zi_min >= kZiMax ? k_predict_count<true> : k_predict_count<false>)
        <<<ctx->blk_pred, kFusedThreads, 0, ctx->stream>>>(
        kp, grid, h.xyzp, h.zphi, h.zh, h.event, h.layer, (const float2 *)ctx->zi.p,
        (const uint32_t *)ctx->zp.p, pairs, &st->n_pairs, pair_cap, cexcl, ptile, stage, stage_cap,
        tile_sbase, walks, walk_cap, st);
    if ((s = mark(ctx, "predict")) != TRAX_OK) return s;
    CK(cudaMemsetAsync(&st->tile_ctr[1], 0, 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->st1.p, 0, (size_t)ntile * 8, ctx->stream));
    k_scan<kScanItems><<<std::min<uint32_t>(ctx->blk_scan, ntile), kScanThreads, 0, ctx->stream>>>(
        ptile, ptile, &st->n_ptile, ptiles, &st->n_cands, 1, (unsigned long long *)ctx->st1.p, st);
    if ((s = mark(ctx, "predict_scan")) != TRAX_OK) return s;
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));  /* work tickets */
    k_predict_store<<<ctx->blk_pstore, kFusedThreads, 0, ctx->stream>>>(
        kp, grid, h.zphi, h.zh, stage, stage_cap, tile_sbase, walks, walk_cap, cexcl, ptile,
        &st->n_pairs, pair_cap, &st->n_cands, cands, cand_cap, st);
    if ((s = mark(ctx, "predict_store")) != TRAX_OK) return s;
    k_cand_offsets<<<ctx->blk_small, 256, 0, ctx->stream>>>(pair_offsets, cexcl, ptile,
                                                            cand_offsets, kp.n_lt, pair_cap,
                                                            &st->n_cands, cand_cap, st);
    CK(cudaGetLastError());
    return mark(ctx, "predict_offsets");
}

/* cand_offsets: the chain's own candidate offsets (the batched pipeline),
 * which let the tracklet offsets come from the accept mask; null (a stage
 * call with the caller's candidates) derives them from the tracklets' hits
 * as the reference does. */
trax_status enqueue_filter(trax_ctx *ctx, const SortedCols &h, const uint2 *pairs,
                           const uint2 *cands, uint32_t cand_cap, uint32_t *t1, uint32_t *t2,
                           uint32_t *t3, uint32_t *trk_offsets, uint32_t trk_cap,
                           uint32_t max_groups, const uint32_t *cand_offsets)
{
    const KParams &kp = ctx->kp;
    trax_status s = need_packed(ctx, h);
    if (s != TRAX_OK) return s;
    const uint32_t words = tiles_for(cand_cap, 32) + 1;
    const uint32_t ntile = tiles_for(words, kScanItems * kScanThreads);
    if ((s = ensure(ctx, ctx->st2, (size_t)ntile * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->fmask, (size_t)words * 8)) != TRAX_OK) return s;
    uint32_t *mask = (uint32_t *)ctx->fmask.p, *wpos = mask + words;
    DevState *st = ctx->d_state;
    CK(cudaMemsetAsync(trk_offsets, 0, (size_t)(max_groups + 1) * 4, ctx->stream));
    CK(cudaMemsetAsync(&st->tile_ctr[0], 0, 4, ctx->stream));  /* work tickets */
    k_filter_count<<<ctx->blk_filter, 256, 0, ctx->stream>>>(kp, h.xyzp, h.layer, pairs,
                                                             cands, &st->n_cands, cand_cap, mask,
                                                             wpos, st);
    if ((s = mark(ctx, "filter")) != TRAX_OK) return s;
    CK(cudaMemsetAsync(&st->tile_ctr[2], 0, 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->st2.p, 0, (size_t)ntile * 8, ctx->stream));
    k_scan<kScanItems><<<std::min<uint32_t>(ctx->blk_scan, ntile), kScanThreads, 0, ctx->stream>>>(
        wpos, wpos, &st->n_ftile, words, &st->n_trk, 2, (unsigned long long *)ctx->st2.p, st);
    if ((s = mark(ctx, "filter_scan")) != TRAX_OK) return s;
    k_filter_store<<<ctx->blk_fstore, 256, 0, ctx->stream>>>(pairs, cands, mask, wpos, t1, t2, t3,
                                                             trk_cap, st);
    if ((s = mark(ctx, "filter_store")) != TRAX_OK) return s;
    bool by_mask = cand_offsets != nullptr;
    for (uint32_t lt = 0; lt < kp.n_lt; ++lt) by_mask = by_mask && kp.l1[lt] == lt + 1;
    if (by_mask) {
        k_trk_offsets_mask<<<ctx->blk_small, 256, 0, ctx->stream>>>(
            cand_offsets, mask, wpos, trk_offsets, kp.n_lt, cand_cap, trk_cap, st);
        CK(cudaGetLastError());
        return mark(ctx, "filter_offsets");
    }
    k_trk_offsets<<<ctx->blk_small, 256, 0, ctx->stream>>>(t1, h.event, h.layer, trk_offsets,
                                                           kp.n_lt, trk_cap, st);
    if ((s = mark(ctx, "filter_offsets")) != TRAX_OK) return s;
    k_monotonize<<<1, 1024, 0, ctx->stream>>>(trk_offsets, kp.n_lt, st);
    CK(cudaGetLastError());
    return mark(ctx, "filter_monotonize");
}

SortedCols sorted_from(const trax_sorted_hits *o)
{
    SortedCols s;
    s.x = o->x; s.y = o->y; s.z = o->z; s.phi = o->phi;
    s.layer = o->layer; s.det = o->detector_id; s.hitid = o->hit_id; s.event = o->event;
    s.orig = o->orig;
    s.zphi = nullptr;
    s.zh = nullptr;
    s.xyzp = nullptr;
    return s;
}

/* Stage calls get the caller's sorted columns: pack (z, phi) for the
 * candidate loops into context scratch first. */
trax_status with_zphi(trax_ctx *ctx, SortedCols &s, uint32_t n)
{
    trax_status st = ensure(ctx, ctx->zphi, (size_t)n * 8 + 8);
    if (st != TRAX_OK) return st;
    if ((st = ensure(ctx, ctx->zh, (size_t)n * 2 + 32)) != TRAX_OK) return st;
    if ((st = ensure(ctx, ctx->xyzp, (size_t)n * 16 + 16)) != TRAX_OK) return st;
    s.zphi = (float2 *)ctx->zphi.p;
    s.zh = (uint16_t *)ctx->zh.p;
    s.xyzp = (float4 *)ctx->xyzp.p;
    if (n) {
        k_pack_zphi<<<std::min<uint32_t>((n + 255) / 256, ctx->blk_small * 4), 256, 0,
                      ctx->stream>>>(s.x, s.y, s.z, s.phi, n, s.zphi, s.zh, s.xyzp);
        CK(cudaGetLastError());
    }
    return TRAX_OK;
}

trax_status build_segments(trax_ctx *ctx, const trax_layout *lay, uint32_t n_hits,
                           uint32_t **d_start, uint32_t **d_n)
{
    const uint32_t E = lay->n_events, L = lay->n_layers;
    const size_t nseg = (size_t)E * L;
    trax_status s = ensure_stage(ctx, 2 * nseg + 2);
    if (s != TRAX_OK) return s;
    uint32_t *hs = ctx->h_stage, *hn = ctx->h_stage + nseg;
    uint64_t run = 0;
    for (uint32_t e = 0; e < E; ++e) {
        if (lay->event_offset && lay->event_offset[e] != run)
            return fail(ctx, TRAX_ERR_BAD_INPUT, "event offsets are not the running hit count");
        uint64_t in_event = 0;
        for (uint32_t l = 0; l < L; ++l) {
            const uint32_t n = lay->layer_nhits[(size_t)e * L + l];
            if (lay->layer_offset && lay->layer_offset[(size_t)e * L + l] != in_event)
                return fail(ctx, TRAX_ERR_BAD_INPUT, "layer offsets are not the running hit count");
            hs[(size_t)e * L + l] = (uint32_t)run;
            hn[(size_t)e * L + l] = n;
            run += n;
            in_event += n;
        }
        if (lay->event_nhits && lay->event_nhits[e] != in_event)
            return fail(ctx, TRAX_ERR_BAD_INPUT, "event hit count differs from its layers' sum");
    }
    if (run != n_hits) return fail(ctx, TRAX_ERR_BAD_INPUT, "layout does not cover the hits");
    if ((s = ensure(ctx, ctx->seg, nseg * 8 + 8)) != TRAX_OK) return s;
    CK(cudaMemcpyAsync(ctx->seg.p, ctx->h_stage, nseg * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->stage_free, ctx->stream));
    *d_start = (uint32_t *)ctx->seg.p;
    *d_n = (uint32_t *)ctx->seg.p + nseg;
    return TRAX_OK;
}

}  // namespace

/* ====================================================================== */

namespace {

__global__ void k_eval_math(int fn, const float *a, const float *b, float *out, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = fn == 0 ? trax_atan2f(a[i], b[i]) : fn == 1 ? trax_acosf(a[i])
               : fn == 2 ? trax_atanf(a[i]) : fn == 3 ? __uint_as_float(trax_f2u(a[i]))
               : fn == 4 ? __int_as_float(trax_f2i(a[i]))
               : trax_floor_div(a[i], b[i], 1.0f / b[i]);
}

std::string g_create_error;

/* ---- allocation-free prefix sum ------------------------------------------
 * Scratch of trax_prefix_sum_noalloc: a DevState (tile ticket, element count,
 * status word) followed by one look-back status word per tile.  It lives in
 * this file-scope device array, so the entry point never allocates; every
 * GPU that loads the library holds it until the process exits. */
constexpr uint32_t kNoAllocTiles =
    (TRAX_PREFIX_SUM_NOALLOC_MAX + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
constexpr size_t kNoAllocStateWords = (sizeof(DevState) + 7) / 8;
constexpr size_t kNoAllocWords = kNoAllocStateWords + kNoAllocTiles + 1;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};
/* per calling thread: a failure on one thread never overwrites another
 * thread's message, and the pointer trax_prefix_sum_noalloc_error() returns
 * stays valid until this thread's next failing call */
thread_local std::string g_noalloc_error;

__global__ void k_set_u32(uint32_t *dst, uint32_t v) { *dst = v; }

/* Device address of the scratch array on the current device; looked up
 * once per device (the host-side symbol is only a stand-in). */
trax_status noalloc_scratch(int dev, unsigned long long **out)
{
    if (dev < 0 || dev >= kMaxDevices) {
        g_noalloc_error = "trax_prefix_sum_noalloc: device " + std::to_string(dev) +
                          " beyond the " + std::to_string(kMaxDevices) + " devices it serves";
        return TRAX_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            g_noalloc_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            cudaGetLastError();
            return TRAX_ERR_DEVICE;
        }
        g_noalloc_addr[dev] = ptr;
    }
    *out = (unsigned long long *)g_noalloc_addr[dev];
    return TRAX_OK;
}

}  // namespace

extern "C" {

const char *trax_version(void) { return "trax-gb300 1 (sm_103a)"; }

trax_status trax_config_validate(const trax_config *cfg, const trax_grid_cfg *grid)
{
    if (!cfg) return TRAX_ERR_BAD_ARG;
    if (cfg->n_layer_triplets == 0 || cfg->n_layer_triplets > TRAX_MAX_LAYER_TRIPLETS)
        return TRAX_ERR_BAD_ARG;
    if (cfg->n_geom_layers == 0 || cfg->n_geom_layers > TRAX_MAX_LAYERS) return TRAX_ERR_BAD_ARG;
    if (!(cfg->min_pt > 0.0f)) return TRAX_ERR_BAD_ARG;
    for (uint32_t i = 0; i < cfg->n_layer_triplets; ++i) {
        const trax_layer_triplet &t = cfg->triplets[i];
        /* the triplet index is derived from the innermost hit's layer
         * (TripletThetaPhiPredictor.h:79, TripletThetaPhiFilter.h:73) */
        if (t.layer1 != i + 1) return TRAX_ERR_BAD_ARG;
        if (t.layer2 == 0 || t.layer3 == 0 || t.layer2 > cfg->n_geom_layers ||
            t.layer3 > cfg->n_geom_layers || t.layer1 > cfg->n_geom_layers)
            return TRAX_ERR_BAD_ARG;
        if (grid && (t.layer1 > grid->n_layers || t.layer2 > grid->n_layers ||
                     t.layer3 > grid->n_layers))
            return TRAX_ERR_BAD_ARG;
    }
    if (grid) {
        if (grid->n_sectors_z == 0 || grid->n_sectors_phi == 0 || grid->n_layers == 0 ||
            grid->n_layers > TRAX_MAX_LAYERS)
            return TRAX_ERR_BAD_ARG;
        if ((uint64_t)(grid->n_sectors_z + 1) * (grid->n_sectors_phi + 1) > 65536)
            return TRAX_ERR_BAD_ARG;
    }
    return TRAX_OK;
}

trax_status trax_layout_validate(const trax_layout *lay, uint32_t n_hits)
{
    if (!lay || !lay->layer_nhits) return TRAX_ERR_BAD_ARG;
    const uint32_t E = lay->n_events, L = lay->n_layers;
    uint64_t run = 0;
    for (uint32_t e = 0; e < E; ++e) {
        if (lay->event_offset && lay->event_offset[e] != run) return TRAX_ERR_BAD_INPUT;
        uint64_t in_event = 0;
        for (uint32_t l = 0; l < L; ++l) {
            if (lay->layer_offset && lay->layer_offset[(size_t)e * L + l] != in_event)
                return TRAX_ERR_BAD_INPUT;
            in_event += lay->layer_nhits[(size_t)e * L + l];
        }
        if (lay->event_nhits && lay->event_nhits[e] != in_event) return TRAX_ERR_BAD_INPUT;
        run += in_event;
    }
    return run == n_hits ? TRAX_OK : TRAX_ERR_BAD_INPUT;
}

size_t trax_abi_sizeof(const char *name)
{
    if (!name) return 0;
    const struct { const char *n; size_t s; } t[] = {
        {"trax_grid_cfg", sizeof(trax_grid_cfg)}, {"trax_layer_triplet", sizeof(trax_layer_triplet)},
        {"trax_tuning", sizeof(trax_tuning)},
        {"trax_config", sizeof(trax_config)}, {"trax_hits", sizeof(trax_hits)},
        {"trax_sorted_hits", sizeof(trax_sorted_hits)}, {"trax_layout", sizeof(trax_layout)},
        {"trax_pairs", sizeof(trax_pairs)}, {"trax_tracklets", sizeof(trax_tracklets)},
        {"trax_counts", sizeof(trax_counts)}, {"trax_event_batch", sizeof(trax_event_batch)},
        {"trax_batch_result", sizeof(trax_batch_result)},
        {"trax_server_opts", sizeof(trax_server_opts)},
        {"trax_server_result", sizeof(trax_server_result)},
        {"trax_server_stats", sizeof(trax_server_stats)},
        {"trax_pb_events", sizeof(trax_pb_events)}, {"trax_raw_hits", sizeof(trax_raw_hits)},
        {"trax_ingest_cfg", sizeof(trax_ingest_cfg)}, {"trax_hits_out", sizeof(trax_hits_out)},
        {"trax_track_list", sizeof(trax_track_list)},
        {"trax_physics_counts", sizeof(trax_physics_counts)}};
    for (const auto &e : t)
        if (strcmp(e.n, name) == 0) return e.s;
    return 0;
}

trax_status trax_eval_math(trax_ctx *ctx, int fn, const float *d_a, const float *d_b,
                           float *d_out, uint32_t n)
{
    if (!ctx || fn < 0 || fn > 5 || !d_a || !d_out || ((fn == 0 || fn == 5) && !d_b))
        return TRAX_ERR_BAD_ARG;
    if (n == 0) return TRAX_OK;
    k_eval_math<<<ctx->blk_small, 256, 0, ctx->stream>>>(fn, d_a, d_b, d_out, n);
    CK(cudaGetLastError());
    return TRAX_OK;
}

float trax_min_radius_curvature(float min_pt, float bz)
{
    /* TripletConfiguration.cpp:145-152 in double, returned as float. */
    const double Q = 1.602177E-19;
    const double GEV_C = 5.344286E-19;
    if (bz == 0.0f) bz = (float)3.8112;
    return (float)(min_pt * GEV_C / (bz * Q) * 1E2);
}

trax_status trax_ctx_create(trax_ctx **out, int device)
{
    if (!out) {
        g_create_error = "trax_ctx_create: out is NULL";
        return TRAX_ERR_BAD_ARG;
    }
    *out = nullptr;
    int n = 0;
    const cudaError_t ce = cudaGetDeviceCount(&n);
    if (ce != cudaSuccess || n == 0) {
        g_create_error = std::string("trax_ctx_create: no CUDA device (") +
                         (ce != cudaSuccess ? cudaGetErrorString(ce) : "device count 0") + ")";
        cudaGetLastError();
        return TRAX_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) {
        g_create_error = "trax_ctx_create: device " + std::to_string(device) + " of " +
                         std::to_string(n);
        return TRAX_ERR_BAD_ARG;
    }
    trax_ctx *ctx = new trax_ctx();
    ctx->device = device;
    auto bail = [&](cudaError_t e) {
        g_create_error = std::string("trax_ctx_create: ") + cudaGetErrorString(e);
        cudaGetLastError();
        delete ctx;
        return TRAX_ERR_DEVICE;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e);
    if ((e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return bail(e);
    int optin = 0;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device)) != cudaSuccess) return bail(e);
    ctx->smem_optin = (size_t)optin;
    if ((e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    ctx->stream = ctx->own_stream;
    if ((e = cudaMalloc(&ctx->d_state, sizeof(DevState))) != cudaSuccess) return bail(e);
    if ((e = cudaMemset(ctx->d_state, 0, sizeof(DevState))) != cudaSuccess) return bail(e);
    if ((e = cudaMallocHost(&ctx->h_state, sizeof(DevState))) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&ctx->stage_free, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    for (int i = 0; i < kTimerSlots; ++i)
        if ((e = cudaEventCreate(&ctx->timers[i])) != cudaSuccess) return bail(e);
    cudaFuncAttributes fa{};
    if ((e = cudaFuncGetAttributes(&fa, k_grid_build<true>)) != cudaSuccess) return bail(e);
    ctx->smem_optin = (size_t)optin - fa.sharedSizeBytes;
    if ((e = cudaFuncSetAttribute(k_grid_build<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ctx->smem_optin)) != cudaSuccess) return bail(e);
    if ((e = cudaFuncSetAttribute(k_grid_build<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ctx->smem_optin)) != cudaSuccess) return bail(e);
    if ((e = cudaFuncSetAttribute(k_grid_build_wb, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ctx->smem_optin)) != cudaSuccess) return bail(e);
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pair, k_pair_fused<true>, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pair0, k_pair_fused<false>, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pair_lane, k_pair_lane<kPairKeep>, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pair_count, k_pair_count_lane, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pair_store, k_pair_store_lane, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_sector, k_pair_sector, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pred, k_predict_count<false>, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_filter, k_filter_count, 256, 0);
    /* the store passes are bound by load latency and use fewer registers
     * than their count passes: a full complement of their own blocks */
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_pstore, k_predict_store, kFusedThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->occ_fstore, k_filter_store, 256, 0);
    apply_launch_cap(ctx);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_scan<kScanItems>, kScanThreads, 0);
    ctx->blk_scan = ctx->sm_count * std::max(b, 1);
    ctx->blk_small = ctx->sm_count * 2;
    if ((e = cudaGetLastError()) != cudaSuccess) return bail(e);
    *out = ctx;
    return TRAX_OK;
}

void trax_ctx_destroy(trax_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_async(ctx);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    DevBuf *bufs[] = {&ctx->seg, &ctx->g_start, &ctx->g_base, &ctx->slots, &ctx->pexcl,
                      &ctx->cexcl, &ctx->st0, &ctx->st1, &ctx->st2, &ctx->st3, &ctx->zi,
                      &ctx->conn_keys, &ctx->conn_sums, &ctx->grid_buf,
                      &ctx->pairs_buf, &ctx->pair_off, &ctx->cands_buf, &ctx->cand_off, &ctx->trk_off,
                      &ctx->r_seg, &ctx->ing, &ctx->phys, &ctx->prec, &ctx->zp, &ctx->ptile,
                      &ctx->fmask, &ctx->zphi, &ctx->zh, &ctx->xyzp, &ctx->pkeep, &ctx->gscr};
    for (DevBuf *b : bufs) if (b->p) cudaFree(b->p);
    for (auto &b : ctx->in_cols) if (b.p) cudaFree(b.p);
    for (auto &b : ctx->srt_cols) if (b.p) cudaFree(b.p);
    for (auto &b : ctx->trk_cols) if (b.p) cudaFree(b.p);
    for (auto &b : ctx->trk_map) if (b.p) cudaFree(b.p);
    if (ctx->d_state) cudaFree(ctx->d_state);
    if (ctx->h_state) cudaFreeHost(ctx->h_state);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->stage_free) cudaEventDestroy(ctx->stage_free);
    for (auto &t : ctx->timers) if (t) cudaEventDestroy(t);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

trax_status trax_ctx_set_stream(trax_ctx *ctx, void *stream)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    drop_graphs(ctx);
    return TRAX_OK;
}

void *trax_ctx_get_stream(trax_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

const char *trax_ctx_last_error(const trax_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

int trax_ctx_sm_count(const trax_ctx *ctx) { return ctx ? ctx->sm_count : 0; }

trax_status trax_ctx_synchronize(trax_ctx *ctx)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    CK(cudaMemcpyAsync(&ctx->h_state->status, &ctx->d_state->status, 8, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return (trax_status)ctx->h_state->status;
}

trax_status trax_configure(trax_ctx *ctx, const trax_config *cfg)
{
    if (!ctx || !cfg) return TRAX_ERR_BAD_ARG;
    if (trax_config_validate(cfg, nullptr) != TRAX_OK)
        return fail(ctx, TRAX_ERR_BAD_ARG,
                    "invalid configuration: 1..16 layer triplets, triplet i starting on layer "
                    "i+1, geometry for every layer used, min_pt > 0");
    ctx->cfg = *cfg;
    KParams &kp = ctx->kp;
    kp.n_lt = cfg->n_layer_triplets;
    for (uint32_t i = 0; i < kMaxLT; ++i) {
        const trax_layer_triplet &t = cfg->triplets[i < cfg->n_layer_triplets ? i : 0];
        kp.l1[i] = t.layer1; kp.l2[i] = t.layer2; kp.l3[i] = t.layer3;
        kp.dtheta[i] = t.dtheta_cut; kp.sigma_z[i] = t.sigma_z; kp.dphi[i] = t.dphi_cut;
        kp.sigma_phi[i] = t.sigma_phi; kp.tip[i] = t.tip_cut; kp.z0[i] = t.z0;
        kp.spread_z[i] = t.pair_spread_z;
        kp.spread_phi[i] = t.pair_spread_phi;
        trax_dphi_screen_bounds(t.dphi_cut, &kp.dphi_tlo[i], &kp.dphi_thi[i]);
    }
    for (uint32_t l = 0; l < kMaxLayers; ++l) {
        kp.rmin[l] = l < cfg->n_geom_layers ? cfg->min_radius[l] : 0.0f;
        kp.rmax[l] = l < cfg->n_geom_layers ? cfg->max_radius[l] : 0.0f;
    }
    kp.rmin_curv = trax_min_radius_curvature(cfg->min_pt, cfg->bz);
    for (uint32_t l = 0; l < kMaxLayers; ++l) {
        kp.acos_rmin[l] = trax_acosf(kp.rmin[l] / (2 * kp.rmin_curv));
        kp.acos_rmax[l] = trax_acosf(kp.rmax[l] / (2 * kp.rmin_curv));
    }
    if (kp.run_walk == 0 && kp.zi_min == 0) {
        kp.run_walk = kDefaultRunWalk;
        kp.zi_min = kDefaultIndexMin;
        kp.pair_record = 3;
    }
    ctx->configured = true;
    drop_graphs(ctx);
    return TRAX_OK;
}

trax_status trax_set_tuning(trax_ctx *ctx, const trax_tuning *t)
{
    if (!ctx || !t) return TRAX_ERR_BAD_ARG;
    if (t->index_min > 256) return fail(ctx, TRAX_ERR_BAD_ARG, "index_min must be <= 256");
    if (t->pair_record > 4) return fail(ctx, TRAX_ERR_BAD_ARG, "pair_record must be 0 to 4");
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->kp.run_walk = t->run_walk;
    ctx->kp.zi_min = t->index_min;
    ctx->kp.pair_record = t->pair_record;
    ctx->blocks_cap = t->blocks_per_sm;
    apply_launch_cap(ctx);
    drop_graphs(ctx);
    return TRAX_OK;
}

trax_status trax_set_pair_generator(trax_ctx *ctx, int generator)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    if (generator != TRAX_PAIRS_BEAMSPOT && generator != TRAX_PAIRS_SECTOR)
        return fail(ctx, TRAX_ERR_BAD_ARG, "unknown pair generator");
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pair_generator = generator;
    drop_graphs(ctx);
    return TRAX_OK;
}

int trax_get_pair_generator(const trax_ctx *ctx)
{
    return ctx ? ctx->pair_generator : -1;
}

trax_status trax_get_tuning(const trax_ctx *ctx, trax_tuning *t)
{
    if (!ctx || !t) return TRAX_ERR_BAD_ARG;
    t->run_walk = ctx->kp.run_walk;
    t->index_min = ctx->kp.zi_min;
    t->pair_record = ctx->kp.pair_record;
    t->blocks_per_sm = ctx->blocks_cap;
    return TRAX_OK;
}

trax_status trax_dev_alloc(trax_ctx *ctx, void **ptr, size_t bytes)
{
    if (!ctx || !ptr) return TRAX_ERR_BAD_ARG;
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, TRAX_ERR_OOM, cudaGetErrorString(e));
    }
    return TRAX_OK;
}

trax_status trax_dev_free(trax_ctx *ctx, void *ptr)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaFree(ptr));
    return TRAX_OK;
}

trax_status trax_host_alloc_pinned(trax_ctx *ctx, void **ptr, size_t bytes)
{
    if (!ctx || !ptr) return TRAX_ERR_BAD_ARG;
    cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, TRAX_ERR_OOM, cudaGetErrorString(e));
    }
    return TRAX_OK;
}

trax_status trax_host_free_pinned(trax_ctx *ctx, void *ptr)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaFreeHost(ptr));
    return TRAX_OK;
}

trax_status trax_memcpy_h2d(trax_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return TRAX_OK;
}

trax_status trax_memcpy_d2h(trax_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    if (bytes) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return TRAX_OK;
}

trax_status trax_memset_d(trax_ctx *ctx, void *dst, int value, size_t bytes)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    if (bytes) CK(cudaMemsetAsync(dst, value, bytes, ctx->stream));
    return TRAX_OK;
}

trax_status trax_timer_record(trax_ctx *ctx, int slot)
{
    if (!ctx || slot < 0 || slot >= kTimerSlots) return TRAX_ERR_BAD_ARG;
    CK(cudaEventRecord(ctx->timers[slot], ctx->stream));
    return TRAX_OK;
}

trax_status trax_timer_elapsed_ms(trax_ctx *ctx, int a, int b, float *ms)
{
    if (!ctx || !ms || a < 0 || b < 0 || a >= kTimerSlots || b >= kTimerSlots) return TRAX_ERR_BAD_ARG;
    CK(cudaEventSynchronize(ctx->timers[b]));
    CK(cudaEventElapsedTime(ms, ctx->timers[a], ctx->timers[b]));
    return TRAX_OK;
}

trax_status trax_reset_counts(trax_ctx *ctx)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    CK(cudaMemsetAsync(&ctx->d_state->n_outer, 0, sizeof(DevState) - 8, ctx->stream));
    return TRAX_OK;
}

trax_status trax_prefix_sum(trax_ctx *ctx, const uint32_t *d_in, uint32_t *d_out, uint32_t n,
                            uint32_t *d_total)
{
    if (!ctx || (n && (!d_in || !d_out))) return TRAX_ERR_BAD_ARG;
    const uint32_t items = kScanThreads * kScanItems;
    trax_status s = ensure(ctx, ctx->st3, (size_t)tiles_for(n, items) * 8, false);
    if (s != TRAX_OK) return s;
    if ((s = ensure_stage(ctx, 1)) != TRAX_OK) return s;
    ctx->h_stage[0] = n;
    DevState *st = ctx->d_state;
    CK(cudaMemcpyAsync(&st->aux_n, ctx->h_stage, 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->stage_free, ctx->stream));
    CK(cudaMemsetAsync(&st->tile_ctr[3], 0, 4, ctx->stream));
    CK(cudaMemsetAsync(ctx->st3.p, 0, (size_t)tiles_for(n, items) * 8, ctx->stream));
    const uint32_t blocks = std::max(1u, std::min<uint32_t>((n + items - 1) / items,
                                                            (uint32_t)ctx->blk_scan));
    k_scan<kScanItems><<<blocks, kScanThreads, 0, ctx->stream>>>(
        d_in, d_out, &st->aux_n, n, d_total, 3, (unsigned long long *)ctx->st3.p, st);
    CK(cudaGetLastError());
    return TRAX_OK;
}

trax_status trax_prefix_sum_noalloc(const uint32_t *d_in, uint32_t *d_out, uint32_t n,
                                    uint32_t *d_total, void *stream)
{
    if (n && (!d_in || !d_out)) {
        g_noalloc_error = "trax_prefix_sum_noalloc: null input or output";
        return TRAX_ERR_BAD_ARG;
    }
    if (n > TRAX_PREFIX_SUM_NOALLOC_MAX) {
        g_noalloc_error = "trax_prefix_sum_noalloc: n exceeds TRAX_PREFIX_SUM_NOALLOC_MAX (" +
                          std::to_string(TRAX_PREFIX_SUM_NOALLOC_MAX) + " elements)";
        return TRAX_ERR_BAD_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return TRAX_ERR_NO_DEVICE;
    }
    unsigned long long *scratch = nullptr;
    trax_status s = noalloc_scratch(dev, &scratch);
    if (s != TRAX_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    DevState *ds = (DevState *)scratch;
    unsigned long long *status = scratch + kNoAllocStateWords;
    const uint32_t items = kScanThreads * kScanItems;
    const uint32_t tiles = (n + items - 1) / items;
    /* the previous call's tickets, count and tile flags must start at zero */
    e = cudaMemsetAsync(scratch, 0, (kNoAllocStateWords + tiles + 1) * 8, st);
    if (e == cudaSuccess) {
        k_set_u32<<<1, 1, 0, st>>>(&ds->aux_n, n);
        const uint32_t blocks = std::max(1u, std::min(tiles, 4u * kNoAllocTiles));
        k_scan<kScanItems><<<blocks, kScanThreads, 0, st>>>(d_in, d_out, &ds->aux_n, n, d_total,
                                                            0, status, ds);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("trax_prefix_sum_noalloc: ") + cudaGetErrorString(e);
        return TRAX_ERR_DEVICE;
    }
    return TRAX_OK;
}

const char *trax_prefix_sum_noalloc_error(void) { return g_noalloc_error.c_str(); }

trax_status trax_prefix_sum_noalloc_status(void *stream)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return TRAX_ERR_NO_DEVICE;
    }
    unsigned long long *scratch = nullptr;
    trax_status s = noalloc_scratch(dev, &scratch);
    if (s != TRAX_OK) return s;
    uint32_t word[2] = {0, 0};  /* DevState::status, DevState::detail */
    const DevState *ds = (const DevState *)scratch;
    cudaStream_t st = (cudaStream_t)stream;
    e = cudaMemcpyAsync(word, &ds->status, sizeof(word), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("trax_prefix_sum_noalloc_status: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return TRAX_ERR_DEVICE;
    }
    if (word[0] != TRAX_OK) {
        g_noalloc_error = "trax_prefix_sum_noalloc: the look-back wait gave up (detail " +
                          std::to_string(word[1]) + "); that call's output is not a valid scan";
        return (trax_status)word[0];
    }
    return TRAX_OK;
}

trax_status trax_selftest_lookback_timeout(trax_ctx *ctx, const uint32_t *d_in, uint32_t *d_out,
                                           uint32_t n, uint32_t spin_limit)
{
    const uint32_t items = kScanThreads * kScanItems;
    if (!ctx || !d_in || !d_out || n <= items || spin_limit == 0) return TRAX_ERR_BAD_ARG;
    trax_status s = ensure(ctx, ctx->st3, (size_t)tiles_for(n, items) * 8, false);
    if (s != TRAX_OK) return s;
    DevState *st = ctx->d_state;
    CK(cudaMemsetAsync(ctx->st3.p, 0, (size_t)tiles_for(n, items) * 8, ctx->stream));
    k_set_u32<<<1, 1, 0, ctx->stream>>>(&st->aux_n, n);
    k_set_u32<<<1, 1, 0, ctx->stream>>>(&st->spin_limit, spin_limit);
    /* tickets start at 1: no CTA ever takes tile 0, so tile 1 waits for a
     * predecessor that never publishes */
    k_set_u32<<<1, 1, 0, ctx->stream>>>(&st->tile_ctr[3], 1u);
    const uint32_t blocks = std::max(1u, std::min<uint32_t>((n + items - 1) / items,
                                                            (uint32_t)ctx->blk_scan));
    k_scan<kScanItems><<<blocks, kScanThreads, 0, ctx->stream>>>(
        d_in, d_out, &st->aux_n, n, nullptr, 3, (unsigned long long *)ctx->st3.p, st);
    k_set_u32<<<1, 1, 0, ctx->stream>>>(&st->spin_limit, 0u);
    CK(cudaGetLastError());
    return TRAX_OK;
}

trax_status trax_ingest(trax_ctx *ctx, const trax_raw_hits *raw, const trax_ingest_cfg *cfg,
                        const uint32_t *d_det_ids, uint32_t n_det_ids, trax_hits_out *out,
                        uint32_t *d_layer_nhits, trax_track_list *tracks, uint32_t *n_hits_out,
                        uint32_t *n_tracks_out)
{
    if (!ctx || !raw || !cfg || !out || !d_layer_nhits || !n_hits_out) return TRAX_ERR_BAD_ARG;
    if (cfg->max_layer == 0 || cfg->max_layer > TRAX_MAX_LAYERS)
        return fail(ctx, TRAX_ERR_BAD_ARG, "max_layer must be 1..16");
    if (cfg->used_layers == 0 || (cfg->used_layers >> cfg->max_layer) != 0)
        return fail(ctx, TRAX_ERR_BAD_ARG, "used_layers must be a non-empty subset of 1..max_layer");
    if (n_det_ids && !d_det_ids) return TRAX_ERR_BAD_ARG;
    const uint32_t E = raw->n_events, N = raw->n_hits;
    *n_hits_out = 0;
    if (n_tracks_out) *n_tracks_out = 0;
    if (E == 0) {
        if (tracks && tracks->offsets) CK(cudaMemsetAsync(tracks->offsets, 0, 4, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return TRAX_OK;
    }
    if (!raw->event_offset || (N && (!raw->x || !raw->y || !raw->z || !raw->layer ||
                                     !raw->detector_id || !raw->sim_track_id || !raw->sim_track_pt)))
        return TRAX_ERR_BAD_ARG;
    /* the per-event CTAs index scratch by these offsets: check them first */
    std::vector<uint32_t> hoff(E + 1);
    CK(cudaMemcpyAsync(hoff.data(), raw->event_offset, (size_t)(E + 1) * 4, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (hoff[0] != 0 || hoff[E] != N)
        return fail(ctx, TRAX_ERR_BAD_INPUT, "event offsets must start at 0 and end at n_hits");
    for (uint32_t e = 0; e < E; ++e)
        if (hoff[e + 1] < hoff[e]) return fail(ctx, TRAX_ERR_BAD_INPUT, "event offsets decrease");

    const size_t words = 12ull * N + 2ull * E + 2ull * (E + 1) + 64;
    trax_status s = ensure(ctx, ctx->ing, words * 4);
    if (s != TRAX_OK) return s;
    uint32_t *w = (uint32_t *)ctx->ing.p;
    IngestScratch sc;
    uint32_t **cols[12] = {&sc.ka, &sc.va, &sc.kb, &sc.vb, &sc.rank, &sc.tstart,
                           &sc.tflag, &sc.perm, &sc.tid, &sc.tin, &sc.tmid, &sc.tout};
    for (int i = 0; i < 12; ++i) *cols[i] = w + (size_t)i * N;
    sc.n_out = w + 12ull * N;
    sc.n_trk = sc.n_out + E;
    uint32_t *out_off = sc.n_trk + E, *trk_off = out_off + (E + 1);

    IngestRaw r{raw->x, raw->y, raw->z, raw->layer, raw->detector_id, raw->sim_track_id,
                raw->sim_track_pt, raw->event_offset, E};
    IngestCfg c{cfg->min_pt, cfg->max_layer, cfg->used_layers, cfg->only_tracks ? 1u : 0u,
                cfg->num_tracks};
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ingest_event, kIngThreads, 0);
    const uint32_t blocks = std::min<uint32_t>(E, (uint32_t)(ctx->sm_count * std::max(b, 1)));
    k_ingest_event<<<blocks, kIngThreads, 0, ctx->stream>>>(r, c, sc, d_layer_nhits);
    if ((s = mark(ctx, "ingest_event")) != TRAX_OK) return s;
    k_ingest_offsets<<<1, 1024, 0, ctx->stream>>>(sc.n_out, sc.n_trk, E, out_off, trk_off);
    IngestOut o{out->x, out->y, out->z, out->layer, out->detector_id, out->hit_id, out->event,
                out->capacity, nullptr, nullptr, nullptr, nullptr, 0};
    if (tracks && tracks->track_id) {
        o.tid = tracks->track_id; o.tin = tracks->inner; o.tmid = tracks->middle;
        o.tout = tracks->outer; o.tcap = tracks->capacity;
    }
    k_ingest_gather<<<std::min<uint32_t>(E, (uint32_t)ctx->blk_small * 4), 256, 0, ctx->stream>>>(
        r, sc, out_off, trk_off, d_det_ids, n_det_ids, o);
    if ((s = mark(ctx, "ingest_gather")) != TRAX_OK) return s;
    if (tracks && tracks->offsets)
        CK(cudaMemcpyAsync(tracks->offsets, trk_off, (size_t)(E + 1) * 4, cudaMemcpyDeviceToDevice,
                           ctx->stream));
    uint32_t tot[2];
    CK(cudaMemcpyAsync(&tot[0], out_off + E, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&tot[1], trk_off + E, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *n_hits_out = tot[0];
    if (n_tracks_out) *n_tracks_out = tot[1];
    if (tot[0] > out->capacity) return fail(ctx, TRAX_ERR_CAPACITY, "hit output smaller than the selected hits");
    if (tracks && tracks->track_id && tot[1] > tracks->capacity)
        return fail(ctx, TRAX_ERR_CAPACITY, "track list smaller than the findable tracks");
    return TRAX_OK;
}

trax_status trax_physics_eval(trax_ctx *ctx, trax_physics *rec, const trax_sorted_hits *hits,
                              const trax_tracklets *trk, uint32_t n_events, uint32_t n_lt,
                              const trax_track_list *mc, const float *d_raw_x,
                              const float *d_raw_y, const float *d_raw_z,
                              trax_physics_counts *counts, uint8_t *categories)
{
    if (!ctx || !rec || !hits || !trk || !mc || !trk->offsets || !mc->offsets || n_lt == 0)
        return TRAX_ERR_BAD_ARG;
    if (n_events == 0) return TRAX_OK;
    const uint32_t G = n_events * n_lt;
    std::vector<uint32_t> toff(G + 1), moff(n_events + 1);
    CK(cudaMemcpyAsync(toff.data(), trk->offsets, (size_t)(G + 1) * 4, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(moff.data(), mc->offsets, (size_t)(n_events + 1) * 4,
                       cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t g = 0; g < G; ++g)
        if (toff[g + 1] < toff[g] || toff[0] != 0)
            return fail(ctx, TRAX_ERR_BAD_INPUT, "tracklet offsets must rise from 0");
    for (uint32_t e = 0; e < n_events; ++e)
        if (moff[e + 1] < moff[e] || moff[0] != 0)
            return fail(ctx, TRAX_ERR_BAD_INPUT, "track list offsets must rise from 0");
    const uint32_t K = toff[G], M = moff[n_events];
    if (K && (!hits->hit_id || !hits->x || !hits->y || !hits->z || !trk->hit1 || !trk->hit2 || !trk->hit3))
        return TRAX_ERR_BAD_ARG;
    if (M && (!mc->track_id || !mc->inner || !mc->middle || !mc->outer || !d_raw_x || !d_raw_y || !d_raw_z))
        return TRAX_ERR_BAD_ARG;
    const size_t nf = (size_t)n_lt * M;
    /* scratch: first[nf] u32, mc_index[K] u32, counts[G*kPcN] u32, cat[K] u8,
     * eta/pt bins [K] f64, missed bins [nf] f64 */
    const size_t b_u32 = (nf + K + (size_t)G * kPcN) * 4, b_f64 = (2 * (size_t)K + 2 * nf) * 8;
    trax_status s = ensure(ctx, ctx->phys, b_f64 + b_u32 + K + nf + 64);
    if (s != TRAX_OK) return s;
    char *base = (char *)ctx->phys.p;
    PhysOut o;
    o.eta_bin = (double *)base;
    o.pt_bin = o.eta_bin + K;
    o.miss_eta_bin = o.pt_bin + K;
    o.miss_pt_bin = o.miss_eta_bin + nf;
    o.first = (uint32_t *)(o.miss_pt_bin + nf);
    o.mc_index = o.first + nf;
    o.counts = o.mc_index + K;
    o.cat = (uint8_t *)(o.counts + (size_t)G * kPcN);
    o.missed = o.cat + K;
    CK(cudaMemsetAsync(o.first, 0xff, nf * 4, ctx->stream));
    CK(cudaMemsetAsync(o.counts, 0, (size_t)G * kPcN * 4, ctx->stream));
    PhysIn in{hits->hit_id, hits->x, hits->y, hits->z, trk->hit1, trk->hit2, trk->hit3,
              trk->offsets, n_events, n_lt, mc->track_id, mc->inner, mc->middle, mc->outer,
              mc->offsets, d_raw_x, d_raw_y, d_raw_z};
    const uint32_t blocks = std::max(1u, std::min<uint32_t>((K + 255) / 256, ctx->blk_small * 4));
    const uint32_t mblocks = std::max(1u, std::min<uint32_t>((uint32_t)((nf + 255) / 256), ctx->blk_small * 4));
    k_phys_tracklets<<<blocks, 256, 0, ctx->stream>>>(in, o);
    k_phys_classify<<<blocks, 256, 0, ctx->stream>>>(in, o);
    k_phys_missed<<<mblocks, 256, 0, ctx->stream>>>(in, o);
    CK(cudaGetLastError());
    std::vector<uint32_t> hc((size_t)G * kPcN);
    std::vector<uint8_t> hcat(K);
    std::vector<double> heta(K), hpt(K), hmeta(nf), hmpt(nf);
    std::vector<uint8_t> hmiss(nf);
    CK(cudaMemcpyAsync(hc.data(), o.counts, hc.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (K) {
        CK(cudaMemcpyAsync(hcat.data(), o.cat, K, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(heta.data(), o.eta_bin, (size_t)K * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hpt.data(), o.pt_bin, (size_t)K * 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (nf) {
        CK(cudaMemcpyAsync(hmeta.data(), o.miss_eta_bin, nf * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hmpt.data(), o.miss_pt_bin, nf * 8, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(hmiss.data(), o.missed, nf, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    /* records in the reference's order; missed tracks in track-id order */
    std::vector<double> me, mp;
    for (uint32_t e = 0; e < n_events; ++e)
        for (uint32_t lt = 0; lt < n_lt; ++lt) {
            const uint32_t g = e * n_lt + lt;
            trax_physics_counts c;
            const uint32_t *q = &hc[(size_t)g * kPcN];
            c.tracklets = q[kPcTracklets]; c.valid = q[kPcValid]; c.clones = q[kPcClones];
            c.fake = q[kPcFake]; c.misc = q[kPcMisc]; c.missed = q[kPcMissed];
            c.findable = q[kPcFindable];
            if (counts) counts[g] = c;
            me.clear();
            mp.clear();
            for (uint32_t k = moff[e]; k < moff[e + 1]; ++k) {
                const size_t qk = (size_t)lt * M + k;
                if (hmiss[qk]) {
                    me.push_back(hmeta[qk]);
                    mp.push_back(hmpt[qk]);
                }
            }
            const uint32_t t0 = toff[g];
            trax_status r = trax_physics_add_group(rec, e, lt, &c, hcat.data() + t0, heta.data() + t0,
                                                   hpt.data() + t0, toff[g + 1] - t0, me.data(),
                                                   mp.data(), (uint32_t)me.size());
            if (r != TRAX_OK) return r;
        }
    if (categories && K) memcpy(categories, hcat.data(), K);
    return TRAX_OK;
}

trax_status trax_triplet_connectivity(trax_ctx *ctx, const trax_tracklets *base,
                                      uint32_t n_base, const uint32_t *base_con,
                                      const trax_tracklets *following, uint32_t n_following,
                                      uint32_t *following_con, int iterate_backwards,
                                      int tight_packing)
{
    if (!ctx || !base || !following || (n_following && !following_con)) return TRAX_ERR_BAD_ARG;
    if (tight_packing && iterate_backwards)
        return fail(ctx, TRAX_ERR_BAD_ARG, "tight packing runs forward only (TripletConnectivity.cpp:56)");
    if (n_base == 0 || n_following == 0) return TRAX_OK;
    /* keys: wide forward base hit3 / follow hit1; backward base hit1 /
     * follow hit3; tight (base hit2, hit3) / (follow hit1, hit2) */
    const uint32_t *ba, *bb = nullptr, *fa, *fb = nullptr;
    if (tight_packing) {
        ba = base->hit2; bb = base->hit3; fa = following->hit1; fb = following->hit2;
    } else if (!iterate_backwards) {
        ba = base->hit3; fa = following->hit1;
    } else {
        ba = base->hit1; fa = following->hit3;
    }
    uint32_t cap = 1024;
    while (cap < 2ull * n_base) cap <<= 1;
    trax_status s;
    if ((s = ensure(ctx, ctx->conn_keys, (size_t)cap * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->conn_sums, (size_t)cap * 4)) != TRAX_OK) return s;
    CK(cudaMemsetAsync(ctx->conn_keys.p, 0xff, (size_t)cap * 8, ctx->stream));
    CK(cudaMemsetAsync(ctx->conn_sums.p, 0, (size_t)cap * 4, ctx->stream));
    const uint32_t blocks = std::max(1u, std::min((n_base + 255) / 256, (uint32_t)ctx->blk_small * 4));
    k_conn_build<<<blocks, 256, 0, ctx->stream>>>(ba, bb, base_con, n_base,
                                                  (unsigned long long *)ctx->conn_keys.p,
                                                  (uint32_t *)ctx->conn_sums.p, cap - 1,
                                                  ctx->d_state);
    const uint32_t fblocks =
        std::max(1u, std::min((n_following + 255) / 256, (uint32_t)ctx->blk_small * 4));
    k_conn_probe<<<fblocks, 256, 0, ctx->stream>>>(fa, fb, n_following,
                                                   (const unsigned long long *)ctx->conn_keys.p,
                                                   (const uint32_t *)ctx->conn_sums.p, cap - 1,
                                                   following_con);
    CK(cudaGetLastError());
    return TRAX_OK;
}

trax_status trax_read_counts(trax_ctx *ctx, trax_counts *out)
{
    if (!ctx || !out) return TRAX_ERR_BAD_ARG;
    CK(cudaMemcpyAsync(ctx->h_state, ctx->d_state, sizeof(DevState), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const DevState &s = *ctx->h_state;
    out->n_hits = s.n_hits;
    out->n_pairs = s.n_pairs;
    out->pair_slots = s.pair_slots;
    out->n_candidates = s.n_cands;
    out->cand_slots = s.cand_slots;
    out->cand_truncated = s.cand_truncated;
    out->n_tracklets = s.n_trk;
    out->status = s.status;
    out->error_detail = s.detail;
    return TRAX_OK;
}

/* ---------------------------------------------------------------------- */

trax_status trax_grid_build(trax_ctx *ctx, const trax_hits *in, const trax_layout *layout,
                            const trax_grid_cfg *grid, trax_sorted_hits *out, uint32_t *d_grid)
{
    if (!ctx || !in || !layout || !grid || !out || !d_grid) return TRAX_ERR_BAD_ARG;
    trax_status s = check_grid(ctx, grid, false);
    if (s != TRAX_OK) return s;
    if (layout->n_events != grid->n_events || layout->n_layers != grid->n_layers)
        return fail(ctx, TRAX_ERR_BAD_ARG, "layout and grid disagree on events or layers");
    if (out->n < in->n) return fail(ctx, TRAX_ERR_CAPACITY, "sorted output smaller than the input");
    fill_grid_params(ctx->kp, grid);
    uint32_t *d_start = nullptr, *d_n = nullptr;
    if ((s = build_segments(ctx, layout, in->n, &d_start, &d_n)) != TRAX_OK) return s;
    if ((s = set_sizes(ctx, grid->n_events, in->n)) != TRAX_OK) return s;
    if (grid->n_events == 0) return TRAX_OK;
    InCols ic{in->x, in->y, in->z, in->layer, in->detector_id, in->hit_id, in->event};
    return enqueue_grid(ctx, ic, sorted_from(out), d_start, d_n, d_grid,
                        grid->n_events * grid->n_layers, in->n);
}

static trax_status pair_gen(trax_ctx *ctx, const trax_sorted_hits *hits, const uint32_t *d_grid,
                            const trax_grid_cfg *grid, trax_pairs *out, int generator)
{
    if (!ctx || !hits || !d_grid || !grid || !out) return TRAX_ERR_BAD_ARG;
    trax_status s = check_grid(ctx, grid);
    if (s != TRAX_OK) return s;
    fill_grid_params(ctx->kp, grid);
    if ((s = set_sizes(ctx, grid->n_events, hits->n)) != TRAX_OK) return s;
    const uint32_t G = grid->n_events * ctx->kp.n_lt;
    const uint64_t slot_cap = (uint64_t)hits->n * ctx->kp.n_lt + 1;
    if (slot_cap > 0xF0000000ull) return fail(ctx, TRAX_ERR_BAD_ARG, "too many hits");
    SortedCols sc = sorted_from(hits);
    if ((s = with_zphi(ctx, sc, hits->n)) != TRAX_OK) return s;
    return enqueue_pairs(ctx, sc, d_grid, (uint2 *)out->pairs, out->offsets,
                         out->capacity, (uint32_t)slot_cap, G, generator);
}

trax_status trax_pair_gen(trax_ctx *ctx, const trax_sorted_hits *hits, const uint32_t *d_grid,
                          const trax_grid_cfg *grid, trax_pairs *out)
{
    return pair_gen(ctx, hits, d_grid, grid, out, TRAX_PAIRS_BEAMSPOT);
}

trax_status trax_pair_gen_sector(trax_ctx *ctx, const trax_sorted_hits *hits,
                                 const uint32_t *d_grid, const trax_grid_cfg *grid,
                                 trax_pairs *out)
{
    return pair_gen(ctx, hits, d_grid, grid, out, TRAX_PAIRS_SECTOR);
}

trax_status trax_triplet_predict(trax_ctx *ctx, const trax_sorted_hits *hits,
                                 const uint32_t *d_grid, const trax_grid_cfg *grid,
                                 const trax_pairs *pairs, trax_pairs *cands)
{
    if (!ctx || !hits || !d_grid || !grid || !pairs || !cands) return TRAX_ERR_BAD_ARG;
    trax_status s = check_grid(ctx, grid);
    if (s != TRAX_OK) return s;
    fill_grid_params(ctx->kp, grid);
    const uint32_t G = grid->n_events * ctx->kp.n_lt;
    if ((s = set_sizes(ctx, grid->n_events, hits->n)) != TRAX_OK) return s;
    /* the pair total is pairs->offsets[G]; copy it into the state word the
     * kernels read (device to device, stream ordered) */
    CK(cudaMemcpyAsync(&ctx->d_state->n_pairs, pairs->offsets + G, 4, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    SortedCols sc = sorted_from(hits);
    if ((s = with_zphi(ctx, sc, hits->n)) != TRAX_OK) return s;
    if ((s = enqueue_zindex(ctx, sc, d_grid, hits->n)) != TRAX_OK) return s;
    return enqueue_predict(ctx, sc, d_grid, (const uint2 *)pairs->pairs,
                           pairs->offsets, pairs->capacity, (uint2 *)cands->pairs, cands->offsets,
                           cands->capacity, G);
}

trax_status trax_triplet_filter(trax_ctx *ctx, const trax_sorted_hits *hits,
                                const trax_grid_cfg *grid, const trax_pairs *pairs,
                                const trax_pairs *cands, trax_tracklets *out)
{
    if (!ctx || !hits || !grid || !pairs || !cands || !out) return TRAX_ERR_BAD_ARG;
    trax_status s = check_grid(ctx, grid);
    if (s != TRAX_OK) return s;
    fill_grid_params(ctx->kp, grid);
    const uint32_t G = grid->n_events * ctx->kp.n_lt;
    CK(cudaMemcpyAsync(&ctx->d_state->n_cands, cands->offsets + G, 4, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    SortedCols sc = sorted_from(hits);
    if ((s = with_zphi(ctx, sc, hits->n)) != TRAX_OK) return s;
    return enqueue_filter(ctx, sc, (const uint2 *)pairs->pairs,
                          (const uint2 *)cands->pairs, cands->capacity, out->hit1, out->hit2,
                          out->hit3, out->offsets, out->capacity, G, nullptr);
}

/* ---------------------------------------------------------------------- */
/* Batched pipeline                                                        */

trax_status trax_reserve(trax_ctx *ctx, uint32_t max_events, uint32_t max_layers,
                         uint32_t max_hits, const trax_grid_cfg *grid, uint32_t max_pairs,
                         uint32_t max_candidates, uint32_t max_tracklets)
{
    if (!ctx || !grid) return TRAX_ERR_BAD_ARG;
    trax_grid_cfg g = *grid;
    g.n_events = max_events;
    g.n_layers = max_layers;
    trax_status s = check_grid(ctx, &g);
    if (s != TRAX_OK) return s;
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graphs(ctx);
    free_async(ctx);
    ctx->reserved = false;
    const uint32_t T = ctx->kp.n_lt;
    const uint64_t C = (uint64_t)(g.n_sectors_z + 1) * (g.n_sectors_phi + 1);
    const uint64_t G = (uint64_t)max_events * T;
    const uint64_t slot_cap = (uint64_t)max_hits * T + 1;
    if (slot_cap > 0xF0000000ull || (uint64_t)max_events * max_layers * C > 0xF0000000ull)
        return fail(ctx, TRAX_ERR_BAD_ARG, "reservation too large");
    for (int i : kChainCols)
        if ((s = ensure(ctx, ctx->in_cols[i], (size_t)max_hits * 4)) != TRAX_OK) return s;
    /* the chain keeps only layer, event and input position of the sorted
     * hits (plus the packed columns below) */
    for (int i : {4, 7, 8}) if ((s = ensure(ctx, ctx->srt_cols[i], (size_t)max_hits * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->grid_buf, (size_t)(max_events * max_layers * C) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->r_seg, (size_t)max_events * max_layers * 8 + 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pairs_buf, (size_t)max_pairs * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pair_off, (size_t)(G + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->cands_buf, (size_t)max_candidates * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->cand_off, (size_t)(G + 1) * 4)) != TRAX_OK) return s;
    for (int i = 0; i < 3; ++i) if ((s = ensure(ctx, ctx->trk_cols[i], (size_t)max_tracklets * 4)) != TRAX_OK) return s;
    for (int i = 0; i < 3; ++i) if ((s = ensure(ctx, ctx->trk_map[i], (size_t)max_tracklets * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->trk_off, (size_t)(G + 1) * 4)) != TRAX_OK) return s;
    /* scratch at its maximum so the captured graph never reallocates */
    if ((s = ensure(ctx, ctx->zi, (size_t)max_hits * 8 + 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->zp, (size_t)max_hits * 4 + 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->zphi, (size_t)max_hits * 8 + 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->zh, (size_t)max_hits * 2 + 32)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->xyzp, (size_t)max_hits * 16 + 16)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->gscr, gscr_bytes(max_hits))) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_start, G * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->g_base, (G + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->slots, slot_cap * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pexcl, (slot_cap + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->st0, (size_t)tiles_for((uint32_t)slot_cap, kTileItems) * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->pkeep, (size_t)slot_cap * kPairKeepSplit * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->cexcl, (size_t)(max_pairs + 1) * 4)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->st1, (size_t)tiles_for(tiles_for(max_pairs, 32) + 1, kScanItems * kScanThreads) * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->ptile, (size_t)(tiles_for(max_pairs, 32) + 1) * 4)) != TRAX_OK) return s;
    {
        const size_t rc = max_candidates ? max_candidates : 1;
        if ((s = ensure(ctx, ctx->prec, (rc + rc / (kPredKeep + 1) + 1) * sizeof(PredRec))) != TRAX_OK) return s;
    }
    if ((s = ensure(ctx, ctx->st2, (size_t)tiles_for(tiles_for(max_candidates, 32) + 1, kScanItems * kScanThreads) * 8)) != TRAX_OK) return s;
    if ((s = ensure(ctx, ctx->fmask, (size_t)(tiles_for(max_candidates, 32) + 1) * 8)) != TRAX_OK) return s;
    if ((s = ensure_stage(ctx, (size_t)max_events * max_layers * 2 + 4)) != TRAX_OK) return s;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->r_events = max_events;
    ctx->r_layers = max_layers;
    ctx->r_hits = max_hits;
    ctx->r_pairs = max_pairs;
    ctx->r_cands = max_candidates;
    ctx->r_trk = max_tracklets;
    ctx->r_grid = g;
    ctx->reserved = true;
    return TRAX_OK;
}

namespace {

SortedCols reserved_sorted(trax_ctx *ctx)
{
    SortedCols s;
    s.x = s.y = s.z = s.phi = nullptr;  /* not kept by the chain */
    s.det = s.hitid = nullptr;
    s.layer = (uint32_t *)ctx->srt_cols[4].p;
    s.event = (uint32_t *)ctx->srt_cols[7].p;
    s.orig = (uint32_t *)ctx->srt_cols[8].p;
    s.zphi = (float2 *)ctx->zphi.p;
    s.zh = (uint16_t *)ctx->zh.p;
    s.xyzp = (float4 *)ctx->xyzp.p;
    return s;
}

InCols in_cols_of(const DevBuf *c)
{
    return InCols{(const float *)c[0].p, (const float *)c[1].p, (const float *)c[2].p,
                  (const uint32_t *)c[3].p, (const uint32_t *)c[4].p, (const uint32_t *)c[5].p,
                  (const uint32_t *)c[6].p};
}

/* The whole chain on reserved buffers, reading the inputs `ic` and the
 * segment table `seg`; sizes come from DevState. */
trax_status enqueue_pipeline(trax_ctx *ctx, const InCols &ic, const uint32_t *seg)
{
    const uint32_t T = ctx->kp.n_lt;
    const uint32_t G = ctx->r_events * T;
    const uint32_t nseg = ctx->r_events * ctx->r_layers;
    const SortedCols sc = reserved_sorted(ctx);
    uint32_t *grid = (uint32_t *)ctx->grid_buf.p;
    trax_status s = begin_marks(ctx);
    if (s != TRAX_OK) return s;
    CK(cudaMemsetAsync(&ctx->d_state->n_outer, 0, sizeof(DevState) - 8, ctx->stream));
    s = enqueue_grid(ctx, ic, sc, seg, seg + nseg, grid, nseg, ctx->r_hits);
    if (s != TRAX_OK) return s;
    s = enqueue_zindex(ctx, sc, grid, ctx->r_hits);
    if (s != TRAX_OK) return s;
    const uint32_t slot_cap = ctx->r_hits * T + 1;
    s = enqueue_pairs(ctx, sc, grid, (uint2 *)ctx->pairs_buf.p, (uint32_t *)ctx->pair_off.p,
                      ctx->r_pairs, slot_cap, G, ctx->pair_generator);
    if (s != TRAX_OK) return s;
    s = enqueue_predict(ctx, sc, grid, (const uint2 *)ctx->pairs_buf.p,
                        (const uint32_t *)ctx->pair_off.p, ctx->r_pairs, (uint2 *)ctx->cands_buf.p,
                        (uint32_t *)ctx->cand_off.p, ctx->r_cands, G);
    if (s != TRAX_OK) return s;
    return enqueue_filter(ctx, sc, (const uint2 *)ctx->pairs_buf.p,
                          (const uint2 *)ctx->cands_buf.p, ctx->r_cands,
                          (uint32_t *)ctx->trk_cols[0].p, (uint32_t *)ctx->trk_cols[1].p,
                          (uint32_t *)ctx->trk_cols[2].p, (uint32_t *)ctx->trk_off.p, ctx->r_trk,
                          G, (const uint32_t *)ctx->cand_off.p);
}

/* Copies a finished batch's results into the slot's own device buffers (the
 * next batch overwrites the chain's), mapping to input positions on
 * request, and the run's counts into the slot's pinned snapshot; tracklets
 * only when they fit the capacity. */
__global__ void k_emit(const DevState *st, DevState *snap, const uint32_t *orig,
                       const uint32_t *t1, const uint32_t *t2, const uint32_t *t3, uint32_t r_trk,
                       uint32_t *o1, uint32_t *o2, uint32_t *o3, uint32_t cap,
                       const uint32_t *off, uint32_t *o_off, uint32_t n_off, uint32_t index_base)
{
    uint32_t n = st->n_trk;
    if (n > r_trk) n = r_trk;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t stride = gridDim.x * blockDim.x;
    if (n <= cap) {
        for (uint32_t i = tid; i < n; i += stride) {
            const uint32_t a = t1[i], b = t2[i], c = t3[i];
            if (o1) o1[i] = (orig ? orig[a] : a) + index_base;
            if (o2) o2[i] = (orig ? orig[b] : b) + index_base;
            if (o3) o3[i] = (orig ? orig[c] : c) + index_base;
        }
    }
    if (o_off)
        for (uint32_t g = tid; g < n_off; g += stride) o_off[g] = off[g];
    if (tid == 0) *snap = *st;
}

/* Event numbers of a batch's second half, counted from its first event. */
__global__ void k_rebase_events(uint32_t *event, uint32_t n, uint32_t base)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        event[i] -= base;
}

__global__ void k_map_orig(const uint32_t *orig, const uint32_t *t1, const uint32_t *t2,
                           const uint32_t *t3, uint32_t *m1, uint32_t *m2, uint32_t *m3,
                           uint32_t cap, const DevState *st)
{
    uint32_t n = st->n_trk;
    if (n > cap) n = cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        m1[i] = orig[t1[i]];
        m2[i] = orig[t2[i]];
        m3[i] = orig[t3[i]];
    }
}

}  // namespace

/* Segment table of a batch at the reservation's stride: starts in
 * hs[0, nseg_r), counts in hs[nseg_r, 2 nseg_r), then (events, hits). */
static trax_status fill_meta(trax_ctx *ctx, const trax_event_batch *in, uint32_t *hs,
                             size_t nseg_r)
{
    const uint32_t E = in->n_events, L = in->n_layers;
    uint32_t *hn = hs + nseg_r;
    uint64_t run = 0;
    for (uint32_t e = 0; e < E; ++e)
        for (uint32_t l = 0; l < L; ++l) {
            hs[(size_t)e * L + l] = (uint32_t)run;
            hn[(size_t)e * L + l] = in->layer_nhits[(size_t)e * L + l];
            run += in->layer_nhits[(size_t)e * L + l];
        }
    if (run != in->n_hits) return fail(ctx, TRAX_ERR_BAD_INPUT, "layer_nhits do not sum to n_hits");
    hs[2 * nseg_r] = E;
    hs[2 * nseg_r + 1] = in->n_hits;
    return TRAX_OK;
}

trax_status trax_stage_batch(trax_ctx *ctx, const trax_event_batch *in)
{
    if (!ctx || !in) return TRAX_ERR_BAD_ARG;
    if (!ctx->reserved) return fail(ctx, TRAX_ERR_BAD_ARG, "trax_reserve not called");
    if (in->n_events > ctx->r_events || in->n_layers != ctx->r_layers || in->n_hits > ctx->r_hits)
        return fail(ctx, TRAX_ERR_CAPACITY, "batch larger than the reservation");
    /* the reserved segment buffer holds [start | count] at a fixed stride */
    const uint32_t E = in->n_events, L = in->n_layers;
    const size_t nseg_r = (size_t)ctx->r_events * L;
    trax_status s = ensure_stage(ctx, 2 * nseg_r + 4);
    if (s != TRAX_OK) return s;
    uint32_t *hs = ctx->h_stage, *hn = ctx->h_stage + nseg_r;
    if ((s = fill_meta(ctx, in, hs, nseg_r)) != TRAX_OK) return s;
    const size_t nseg = (size_t)E * L;
    CK(cudaMemcpyAsync(ctx->r_seg.p, hs, nseg * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync((uint32_t *)ctx->r_seg.p + nseg_r, hn, nseg * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_state, hs + 2 * nseg_r, 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->stage_free, ctx->stream));
    const void *src[7] = {in->x, in->y, in->z, in->layer, in->detector_id, in->hit_id, in->event};
    for (int i : kChainCols)
        if (in->n_hits) CK(cudaMemcpyAsync(ctx->in_cols[i].p, src[i], (size_t)in->n_hits * 4,
                                           cudaMemcpyHostToDevice, ctx->stream));
    ctx->staged_events = E;
    ctx->staged_hits = in->n_hits;
    return TRAX_OK;
}

trax_status trax_count_pairs_batch(trax_ctx *ctx, const trax_event_batch *in,
                                   uint32_t *event_pairs)
{
    if (!ctx || !in || !event_pairs) return TRAX_ERR_BAD_ARG;
    if (ctx->pair_generator != TRAX_PAIRS_BEAMSPOT)
        return fail(ctx, TRAX_ERR_BAD_ARG, "pair counts need the beam-spot pair generator");
    trax_status s = trax_stage_batch(ctx, in);
    if (s != TRAX_OK) return s;
    fill_grid_params(ctx->kp, &ctx->r_grid);
    const uint32_t T = ctx->kp.n_lt, E = in->n_events;
    const uint32_t nseg = ctx->r_events * ctx->r_layers;
    if ((s = grid_plan(ctx, ctx->kp.C, nseg ? ctx->r_hits / nseg : 0)) != TRAX_OK) return s;
    const SortedCols sc = reserved_sorted(ctx);
    uint32_t *grid = (uint32_t *)ctx->grid_buf.p;
    const uint32_t *seg = (const uint32_t *)ctx->r_seg.p;
    CK(cudaMemsetAsync(&ctx->d_state->n_outer, 0, sizeof(DevState) - 8, ctx->stream));
    if ((s = enqueue_grid(ctx, in_cols_of(ctx->in_cols), sc, seg, seg + nseg, grid, nseg,
                          ctx->r_hits)) != TRAX_OK)
        return s;
    if ((s = enqueue_pair_count(ctx, sc, grid, (uint32_t *)ctx->pair_off.p, ctx->r_hits * T + 1,
                                ctx->r_events * T)) != TRAX_OK)
        return s;
    const size_t n_off = (size_t)E * T + 1;
    if ((s = ensure_stage(ctx, n_off + 2)) != TRAX_OK) return s;
    uint32_t *h = ctx->h_stage;
    CK(cudaMemcpyAsync(h, ctx->pair_off.p, n_off * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&ctx->h_state->status, &ctx->d_state->status, 8, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_state->status != TRAX_OK)
        return fail(ctx, (trax_status)ctx->h_state->status, "device fault in the pair count");
    for (uint32_t e = 0; e < E; ++e) event_pairs[e] = h[(size_t)(e + 1) * T] - h[(size_t)e * T];
    return TRAX_OK;
}

/* Captures the chain over the inputs `ic` / `seg` into *exec. */
trax_status capture_pipeline(trax_ctx *ctx, const InCols &ic, const uint32_t *seg,
                             cudaGraphExec_t *exec)
{
    const uint32_t nseg = ctx->r_events * ctx->r_layers;
    trax_status s0 = grid_plan(ctx, ctx->kp.C, nseg ? ctx->r_hits / nseg : 0);
    if (s0 != TRAX_OK) return s0;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    trax_status s = enqueue_pipeline(ctx, ic, seg);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (s != TRAX_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess) return fail(ctx, TRAX_ERR_DEVICE, cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return fail(ctx, TRAX_ERR_DEVICE, cudaGetErrorString(e));
    }
    return TRAX_OK;
}

trax_status trax_run_staged(trax_ctx *ctx)
{
    if (!ctx || !ctx->reserved) return TRAX_ERR_BAD_ARG;
    fill_grid_params(ctx->kp, &ctx->r_grid);
    if (!ctx->graph) {
        trax_status s = capture_pipeline(ctx, in_cols_of(ctx->in_cols),
                                         (const uint32_t *)ctx->r_seg.p, &ctx->graph);
        if (s != TRAX_OK) return s;
    }
    CK(cudaGraphLaunch(ctx->graph, ctx->stream));
    return TRAX_OK;
}

trax_status trax_run_staged_eager(trax_ctx *ctx)
{
    if (!ctx || !ctx->reserved) return TRAX_ERR_BAD_ARG;
    fill_grid_params(ctx->kp, &ctx->r_grid);
    return enqueue_pipeline(ctx, in_cols_of(ctx->in_cols), (const uint32_t *)ctx->r_seg.p);
}

trax_status trax_set_profiling(trax_ctx *ctx, int on)
{
    if (!ctx) return TRAX_ERR_BAD_ARG;
    if ((bool)on != ctx->profiling && has_graph(ctx)) {
        CK(cudaStreamSynchronize(ctx->stream));
        drop_graphs(ctx);
    }
    ctx->profiling = on != 0;
    return TRAX_OK;
}

int trax_kernel_launches(const trax_ctx *ctx) { return ctx ? ctx->launches : 0; }

trax_status trax_kernel_times(trax_ctx *ctx, float *ms, const char **names, int max_n, int *n)
{
    if (!ctx || !n) return TRAX_ERR_BAD_ARG;
    *n = 0;
    if (!ctx->profiling) return TRAX_OK;
    CK(cudaEventSynchronize(ctx->timers[ctx->n_marks]));
    for (int i = 1; i <= ctx->n_marks && *n < max_n; ++i) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, ctx->timers[i - 1], ctx->timers[i]));
        if (ms) ms[*n] = t;
        if (names) names[*n] = ctx->mark_names[i];
        ++*n;
    }
    return TRAX_OK;
}

/* trax_seed_batch in one piece: upload, graph, download in turn. */
static trax_status seed_whole(trax_ctx *ctx, const trax_event_batch *in, trax_batch_result *out)
{
    trax_status s = trax_stage_batch(ctx, in);
    if (s != TRAX_OK) return s;
    if ((s = trax_run_staged(ctx)) != TRAX_OK) return s;
    if (out->input_indices) {
        k_map_orig<<<ctx->blk_small, 256, 0, ctx->stream>>>(
            (const uint32_t *)ctx->srt_cols[8].p, (const uint32_t *)ctx->trk_cols[0].p,
            (const uint32_t *)ctx->trk_cols[1].p, (const uint32_t *)ctx->trk_cols[2].p,
            (uint32_t *)ctx->trk_map[0].p, (uint32_t *)ctx->trk_map[1].p,
            (uint32_t *)ctx->trk_map[2].p, ctx->r_trk, ctx->d_state);
        CK(cudaGetLastError());
    }
    if ((s = trax_read_counts(ctx, &out->counts)) != TRAX_OK) return s;
    const uint32_t G = in->n_events * ctx->kp.n_lt;
    uint32_t n = (uint32_t)out->counts.n_tracklets;
    out->n_tracklets = n;
    if (n > ctx->r_trk) n = ctx->r_trk;
    const bool fits = n <= out->capacity;
    if (fits && n) {
        DevBuf *cols = out->input_indices ? ctx->trk_map : ctx->trk_cols;
        uint32_t *dst[3] = {out->hit1, out->hit2, out->hit3};
        for (int i = 0; i < 3; ++i)
            if (dst[i]) CK(cudaMemcpyAsync(dst[i], cols[i].p, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (out->offsets)
        CK(cudaMemcpyAsync(out->offsets, ctx->trk_off.p, (size_t)(G + 1) * 4, cudaMemcpyDeviceToHost,
                           ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (out->counts.status != TRAX_OK) {
        char buf[96];
        snprintf(buf, sizeof buf, "device status %u detail %u", out->counts.status,
                 out->counts.error_detail);
        return fail(ctx, (trax_status)out->counts.status, buf);
    }
    if (!fits) return fail(ctx, TRAX_ERR_CAPACITY, "result larger than the output capacity");
    return TRAX_OK;
}

static trax_status submit_slot(trax_ctx *ctx, const trax_event_batch *in,
                               const trax_batch_result *out, uint32_t event_base,
                               uint32_t index_base, uint32_t *ticket);
static trax_status wait_slot(trax_ctx *ctx, uint32_t ticket, trax_batch_result *out,
                             uint32_t trk_shift, uint32_t off_shift, bool download);

/*
 * trax_seed_batch as two halves of its events through the streaming slots:
 * the second half uploads while the first computes, and the first half's
 * results download while the second computes.  Events are independent, so
 * the halves' results, concatenated (the second half's hit indices and
 * offsets shifted), are the whole batch's.
 */
trax_status trax_seed_batch(trax_ctx *ctx, const trax_event_batch *in, trax_batch_result *out)
{
    if (!ctx || !in || !out) return TRAX_ERR_BAD_ARG;
    const uint32_t E = in->n_events, L = in->n_layers;
    /* small batches (a serving slot's) gain nothing from the overlap and
     * keep the one-piece form, without the streaming slots' buffers */
    if (E < 2 || in->n_hits < kSplitSeedHits || !ctx->reserved || ctx->aslot[0].busy ||
        ctx->aslot[1].busy || L != ctx->r_layers || E > ctx->r_events || in->n_hits > ctx->r_hits)
        return seed_whole(ctx, in, out);
    const uint32_t E1 = E / 2;
    uint64_t n1 = 0;
    for (size_t i = 0; i < (size_t)E1 * L; ++i) n1 += in->layer_nhits[i];
    if (n1 > in->n_hits) return fail(ctx, TRAX_ERR_BAD_INPUT, "layer_nhits do not sum to n_hits");
    trax_event_batch b1 = *in, b2 = *in;
    b1.n_events = E1;
    b1.n_hits = (uint32_t)n1;
    b2.n_events = E - E1;
    b2.n_hits = in->n_hits - (uint32_t)n1;
    b2.x += n1; b2.y += n1; b2.z += n1;
    b2.layer += n1; b2.event += n1;  /* the ids are not read (and may be null) */
    b2.layer_nhits += (size_t)E1 * L;
    uint32_t t1 = 0, t2 = 0;
    trax_status s = submit_slot(ctx, &b1, out, 0, 0, &t1);
    if (s != TRAX_OK) return s;
    s = submit_slot(ctx, &b2, out, E1, (uint32_t)n1, &t2);
    if (s != TRAX_OK) {
        trax_batch_result r = *out;
        wait_slot(ctx, t1, &r, 0, 0, false);
        return s;
    }
    trax_batch_result r1 = *out, r2 = *out;
    const trax_status s1 = wait_slot(ctx, t1, &r1, 0, 0, true);
    const trax_status s2 = wait_slot(ctx, t2, &r2, s1 == TRAX_OK ? r1.n_tracklets : 0,
                                     E1 * ctx->kp.n_lt, s1 == TRAX_OK);
    trax_counts &c = out->counts;
    c.n_hits = r1.counts.n_hits + r2.counts.n_hits;
    c.n_pairs = r1.counts.n_pairs + r2.counts.n_pairs;
    c.pair_slots = r1.counts.pair_slots + r2.counts.pair_slots;
    c.n_candidates = r1.counts.n_candidates + r2.counts.n_candidates;
    c.cand_slots = r1.counts.cand_slots + r2.counts.cand_slots;
    c.cand_truncated = r1.counts.cand_truncated + r2.counts.cand_truncated;
    c.n_tracklets = r1.counts.n_tracklets + r2.counts.n_tracklets;
    c.status = r1.counts.status ? r1.counts.status : r2.counts.status;
    c.error_detail = r1.counts.status ? r1.counts.error_detail : r2.counts.error_detail;
    out->n_tracklets = r1.n_tracklets + r2.n_tracklets;
    if (c.status != TRAX_OK) {
        char buf[96];
        snprintf(buf, sizeof buf, "device status %u detail %u", c.status, c.error_detail);
        return fail(ctx, (trax_status)c.status, buf);
    }
    if (s1 != TRAX_OK || s2 != TRAX_OK || out->n_tracklets > out->capacity)
        return fail(ctx, TRAX_ERR_CAPACITY, "result larger than the output capacity");
    return TRAX_OK;
}

/* Creates a streaming slot's buffers at the reservation's sizes. */
static trax_status ensure_slot(trax_ctx *ctx, AsyncSlot &a)
{
    if (!ctx->copy_stream) CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    if (!ctx->d2h_stream) CK(cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking));
    if (a.h_meta) return TRAX_OK;
    const size_t nseg_r = (size_t)ctx->r_events * ctx->r_layers;
    /* plain allocations: the slot's graph is captured after them */
    for (int i : kChainCols) {
        DevBuf &b = a.in_cols[i];
        b.bytes = std::max<size_t>((size_t)ctx->r_hits * 4, 16);
        CK(cudaMalloc(&b.p, b.bytes));
    }
    a.seg.bytes = (2 * nseg_r + 2) * 4;
    CK(cudaMalloc(&a.seg.p, a.seg.bytes));
    for (auto &b : a.res) {
        b.bytes = std::max<size_t>((size_t)ctx->r_trk * 4, 16);
        CK(cudaMalloc(&b.p, b.bytes));
    }
    a.res_off.bytes = ((size_t)ctx->r_events * ctx->kp.n_lt + 1) * 4;
    CK(cudaMalloc(&a.res_off.p, a.res_off.bytes));
    CK(cudaMallocHost(&a.h_meta, (2 * nseg_r + 2) * 4));
    CK(cudaMallocHost(&a.h_snap, sizeof(DevState)));
    CK(cudaEventCreateWithFlags(&a.h2d_done, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
    return TRAX_OK;
}

/* Queues one batch on a free slot.  event_base: the batch's hits carry
 * event numbers from event_base on (rebased on the device); index_base is
 * added to every returned hit index. */
static trax_status submit_slot(trax_ctx *ctx, const trax_event_batch *in,
                               const trax_batch_result *out, uint32_t event_base,
                               uint32_t index_base, uint32_t *ticket)
{
    if (!ctx->reserved) return fail(ctx, TRAX_ERR_BAD_ARG, "trax_reserve not called");
    if (in->n_events > ctx->r_events || in->n_layers != ctx->r_layers || in->n_hits > ctx->r_hits)
        return fail(ctx, TRAX_ERR_CAPACITY, "batch larger than the reservation");
    AsyncSlot &a = ctx->aslot[ctx->next_ticket & 1];
    if (a.busy) return fail(ctx, TRAX_ERR_BAD_ARG, "two batches in flight: wait for the older one first");
    trax_status s = ensure_slot(ctx, a);
    if (s != TRAX_OK) return s;
    const size_t nseg_r = (size_t)ctx->r_events * ctx->r_layers;
    const size_t nseg = (size_t)in->n_events * in->n_layers;
    if ((s = fill_meta(ctx, in, a.h_meta, nseg_r)) != TRAX_OK) return s;
    /* uploads: the slot's previous batch was waited for, so nothing reads
     * its inputs any more */
    uint32_t *seg = (uint32_t *)a.seg.p;
    CK(cudaMemcpyAsync(seg, a.h_meta, nseg * 4, cudaMemcpyHostToDevice, ctx->copy_stream));
    CK(cudaMemcpyAsync(seg + nseg_r, a.h_meta + nseg_r, nseg * 4, cudaMemcpyHostToDevice,
                       ctx->copy_stream));
    CK(cudaMemcpyAsync(seg + 2 * nseg_r, a.h_meta + 2 * nseg_r, 8, cudaMemcpyHostToDevice,
                       ctx->copy_stream));
    const void *src[7] = {in->x, in->y, in->z, in->layer, in->detector_id, in->hit_id, in->event};
    for (int i : kChainCols)
        if (in->n_hits)
            CK(cudaMemcpyAsync(a.in_cols[i].p, src[i], (size_t)in->n_hits * 4,
                               cudaMemcpyHostToDevice, ctx->copy_stream));
    CK(cudaEventRecord(a.h2d_done, ctx->copy_stream));
    /* the chain on the context stream once the upload is in */
    fill_grid_params(ctx->kp, &ctx->r_grid);
    if (!a.graph) {
        if ((s = capture_pipeline(ctx, in_cols_of(a.in_cols), seg, &a.graph)) != TRAX_OK) return s;
    }
    CK(cudaStreamWaitEvent(ctx->stream, a.h2d_done, 0));
    if (event_base && in->n_hits)
        k_rebase_events<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>((uint32_t *)a.in_cols[6].p,
                                                                in->n_hits, event_base);
    CK(cudaMemcpyAsync(ctx->d_state, seg + 2 * nseg_r, 8, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaGraphLaunch(a.graph, ctx->stream));
    const uint32_t n_off = in->n_events * ctx->kp.n_lt + 1;
    /* a full grid: the input-position mapping is a dependent gather per
     * tracklet hit, bound by load latency */
    k_emit<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(
        ctx->d_state, a.h_snap, out->input_indices ? (const uint32_t *)ctx->srt_cols[8].p : nullptr,
        (const uint32_t *)ctx->trk_cols[0].p, (const uint32_t *)ctx->trk_cols[1].p,
        (const uint32_t *)ctx->trk_cols[2].p, ctx->r_trk, (uint32_t *)a.res[0].p,
        (uint32_t *)a.res[1].p, (uint32_t *)a.res[2].p, out->capacity,
        (const uint32_t *)ctx->trk_off.p, (uint32_t *)a.res_off.p, n_off, index_base);
    CK(cudaGetLastError());
    CK(cudaEventRecord(a.done, ctx->stream));
    a.busy = true;
    a.ticket = ctx->next_ticket++;
    a.capacity = out->capacity;
    a.n_off = n_off;
    a.out[0] = out->hit1;
    a.out[1] = out->hit2;
    a.out[2] = out->hit3;
    a.out[3] = out->offsets;
    *ticket = a.ticket;
    return TRAX_OK;
}

trax_status trax_submit_batch(trax_ctx *ctx, const trax_event_batch *in,
                              const trax_batch_result *out, uint32_t *ticket)
{
    if (!ctx || !in || !out || !ticket) return TRAX_ERR_BAD_ARG;
    return submit_slot(ctx, in, out, 0, 0, ticket);
}

/* Waits for a slot's batch and downloads its results to the slot's output
 * pointers shifted by trk_shift tracklets (offsets: by off_shift entries, each
 * plus trk_shift); the capacity counts from the unshifted start. */
static trax_status wait_slot(trax_ctx *ctx, uint32_t ticket, trax_batch_result *out,
                             uint32_t trk_shift, uint32_t off_shift, bool download)
{
    AsyncSlot &a = ctx->aslot[ticket & 1];
    if (!a.busy || a.ticket != ticket) return fail(ctx, TRAX_ERR_BAD_ARG, "no batch in flight with this ticket");
    a.busy = false;
    CK(cudaEventSynchronize(a.done));
    const DevState &st = *a.h_snap;
    out->counts.n_hits = st.n_hits;
    out->counts.n_pairs = st.n_pairs;
    out->counts.pair_slots = st.pair_slots;
    out->counts.n_candidates = st.n_cands;
    out->counts.cand_slots = st.cand_slots;
    out->counts.cand_truncated = st.cand_truncated;
    out->counts.n_tracklets = st.n_trk;
    out->counts.status = st.status;
    out->counts.error_detail = st.detail;
    out->n_tracklets = st.n_trk;
    if (st.status != TRAX_OK) {
        char buf[96];
        snprintf(buf, sizeof buf, "device status %u detail %u", st.status, st.detail);
        return fail(ctx, (trax_status)st.status, buf);
    }
    if (st.n_trk > ctx->r_trk || (uint64_t)trk_shift + st.n_trk > a.capacity)
        return fail(ctx, TRAX_ERR_CAPACITY, "result larger than the output capacity");
    if (!download) return TRAX_OK;
    /* the download, on its own stream: it overlaps the next batch's chain */
    for (int i = 0; i < 3; ++i)
        if (a.out[i] && st.n_trk)
            CK(cudaMemcpyAsync(a.out[i] + trk_shift, a.res[i].p, (size_t)st.n_trk * 4,
                               cudaMemcpyDeviceToHost, ctx->d2h_stream));
    if (a.out[3])
        CK(cudaMemcpyAsync(a.out[3] + off_shift, a.res_off.p, (size_t)a.n_off * 4,
                           cudaMemcpyDeviceToHost, ctx->d2h_stream));
    CK(cudaStreamSynchronize(ctx->d2h_stream));
    if (a.out[3] && trk_shift)
        for (uint32_t g = 0; g < a.n_off; ++g) a.out[3][off_shift + g] += trk_shift;
    return TRAX_OK;
}

trax_status trax_wait_batch(trax_ctx *ctx, uint32_t ticket, trax_batch_result *out)
{
    if (!ctx || !out) return TRAX_ERR_BAD_ARG;
    return wait_slot(ctx, ticket, out, 0, 0, true);
}

}  // extern "C"
