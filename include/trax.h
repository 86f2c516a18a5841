/*
 * trax.h -- C-ABI of the GB300 triplet-seeding path.
 *
 * Replaces the C++ operator surface of trax's seeding chain, which the
 * reference calls in this order from buildTriplets
 * (src/triplet_builder/TripletBuilder.cpp:240-263):
 *
 *   GridBuilder::run              src/algorithms/GridBuilder.h:42, GridBuilder.cpp:6
 *   PairGeneratorBeamspot::run    src/algorithms/PairGeneratorBeamspot.h:40-41, .cpp:5
 *   TripletThetaPhiPredictor::run src/algorithms/TripletThetaPhiPredictor.h:43-44, .cpp:10
 *   TripletThetaPhiFilter::run    src/algorithms/TripletThetaPhiFilter.h:46-48, .cpp:10
 *
 * Conventions
 *  - Plain C types only; every pointer documents whether it is host or device.
 *  - Every call returns a trax_status and never throws.  Kernel-side faults
 *    (hits outside the grid, a bounded wait that gave up, an output larger
 *    than its capacity) are recorded in a device status word that
 *    trax_read_counts() and trax_ctx_synchronize() return.
 *  - Stage calls are asynchronous and stream ordered on the context's stream.
 *    One context per host thread; contexts are independent.
 *  - Output buffers are caller allocated with an explicit capacity.  When a
 *    result does not fit, nothing is written out of bounds and the status
 *    word reports TRAX_ERR_CAPACITY; the true size is still reported.
 *  - Hit indices in pairs, candidates and tracklets are indices into the
 *    cell-sorted hit columns written by trax_grid_build, as in the reference.
 *    The sorted `orig` column maps them back to input positions.
 */
#ifndef TRAX_H
#define TRAX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TRAX_ABI_VERSION 1
#define TRAX_MAX_LAYER_TRIPLETS 16
#define TRAX_MAX_LAYERS 16

typedef enum trax_status {
    TRAX_OK = 0,
    TRAX_ERR_BAD_ARG = 1,   /* invalid argument or configuration */
    TRAX_ERR_OOM = 2,       /* device allocation failed / memory budget exceeded */
    TRAX_ERR_TIMEOUT = 3,   /* a bounded device-side wait gave up */
    TRAX_ERR_DEVICE = 4,    /* CUDA runtime error */
    TRAX_ERR_CAPACITY = 5,  /* an output did not fit its capacity */
    TRAX_ERR_BAD_INPUT = 6, /* hit outside the grid, NaN, or layout mismatch */
    TRAX_ERR_NO_DEVICE = 7  /* no CUDA device / CUDA unavailable */
} trax_status;

typedef struct trax_ctx trax_ctx;

/* GridConfig (src/datastructures/Grid.h:5-39).  The z and phi extents are the
 * reference's fixed -300..300 cm and -pi..pi. */
typedef struct trax_grid_cfg {
    uint32_t n_events;
    uint32_t n_layers;      /* layers 1..n_layers are gridded */
    uint32_t n_sectors_z;
    uint32_t n_sectors_phi;
} trax_grid_cfg;

/* One row of TripletConfigurations
 * (src/datastructures/TripletConfiguration.h:33, values as parsed by
 * TripletConfiguration.cpp:191-207; z0 is parsed as an unsigned integer). */
typedef struct trax_layer_triplet {
    uint32_t layer1, layer2, layer3;
    float dtheta_cut;
    float sigma_z;
    float dphi_cut;
    float sigma_phi;
    float tip_cut;
    uint32_t pair_spread_z;
    float z0;
    uint32_t pair_spread_phi;
    uint32_t n_candidates;
} trax_layer_triplet;

/* Everything on the path that is not per event.
 * Layer triplet i must have layer1 == i + 1: the reference's predictor and
 * filter derive the triplet index from the innermost hit's layer
 * (TripletThetaPhiPredictor.h:79, TripletThetaPhiFilter.h:73). */
typedef struct trax_config {
    uint32_t n_layer_triplets;
    trax_layer_triplet triplets[TRAX_MAX_LAYER_TRIPLETS];
    /* GeometrySupplement (GeometrySupplement.h:21-43), index = layer - 1 */
    uint32_t n_geom_layers;
    float min_radius[TRAX_MAX_LAYERS];
    float max_radius[TRAX_MAX_LAYERS];
    float min_pt;  /* GeV; TripletConfigurations::minPt_ */
    float bz;      /* Tesla; 0 selects the reference's IDEAL_BZ 3.8112 */
} trax_config;

/* HitCollection columns (HitCollection.h:23, HIT_COLLECTION_ITEMS), device
 * pointers.  Input order: event-major, then layer-major, exactly as
 * HitCollection::addEvent produces it (HitCollection.cpp:121-146). */
typedef struct trax_hits {
    const float *x, *y, *z;
    const uint32_t *layer;       /* 1-based detector layer */
    const uint32_t *detector_id;
    const uint32_t *hit_id;      /* the reference stores the sim-track id here */
    const uint32_t *event;       /* event index within the batch */
    uint32_t n;
} trax_hits;

/* Cell-sorted hit columns written by trax_grid_build (device pointers).  The
 * seven reference columns plus `phi` (atan2(y,x), used by the later stages)
 * and `orig` (input position of the hit). */
typedef struct trax_sorted_hits {
    float *x, *y, *z, *phi;
    uint32_t *layer, *detector_id, *hit_id, *event, *orig;
    uint32_t n;
} trax_sorted_hits;

/* EventSupplement / LayerSupplement (EventSupplement.h:8-32,
 * LayerSupplement.h:7-31): host arrays. */
typedef struct trax_layout {
    uint32_t n_events;
    uint32_t n_layers;
    const uint32_t *event_nhits;   /* [n_events] */
    const uint32_t *event_offset;  /* [n_events] */
    const uint32_t *layer_nhits;   /* [n_events * n_layers] */
    const uint32_t *layer_offset;  /* [n_events * n_layers], within the event */
} trax_layout;

/* Pairing (src/datastructures/Pairings.h:9-59): uint2 records plus
 * per-(event, layer triplet) offsets.  Device pointers. */
typedef struct trax_pairs {
    uint32_t *pairs;    /* 2 * capacity uint32: (x, y) records */
    uint32_t *offsets;  /* n_events * n_layer_triplets + 1 */
    uint32_t capacity;  /* records */
} trax_pairs;

/* TrackletCollection (src/datastructures/TrackletCollection.h:32-77):
 * TrackletHit1/2/3 columns plus per-(event, layer triplet) offsets. */
typedef struct trax_tracklets {
    uint32_t *hit1, *hit2, *hit3;
    uint32_t *offsets;  /* n_events * n_layer_triplets + 1 */
    uint32_t capacity;
} trax_tracklets;

/* Device counters accumulated since the last trax_reset_counts(). */
typedef struct trax_counts {
    uint64_t n_hits;
    uint64_t n_pairs;          /* distinct accepted (inner, outer) pairs */
    uint64_t pair_slots;       /* pairCount total: slots the reference allocates */
    uint64_t n_candidates;     /* candidates stored by the predictor */
    uint64_t cand_slots;       /* predictCount total: slots the reference allocates */
    uint64_t cand_truncated;   /* store-window accepts dropped at the count cap */
    uint64_t n_tracklets;
    uint32_t status;           /* trax_status of the first device-side fault */
    uint32_t error_detail;     /* which check raised it (TRAX_DETAIL_*) */
} trax_counts;

#define TRAX_DETAIL_HIT_OUTSIDE_GRID 1u
#define TRAX_DETAIL_HIT_LAYER_MISMATCH 2u
#define TRAX_DETAIL_WINDOW_OUTSIDE_GRID 3u
#define TRAX_DETAIL_PAIR_CAPACITY 4u
#define TRAX_DETAIL_CAND_CAPACITY 5u
#define TRAX_DETAIL_TRACKLET_CAPACITY 6u
#define TRAX_DETAIL_SCAN_TIMEOUT 7u
#define TRAX_DETAIL_BAD_TRIPLET_INDEX 8u

/* ---- context ----------------------------------------------------------
 * Replaces the clever::context the reference's operators take
 * (createContext, TripletBuilder.cpp:52-92): one CUDA device and a stream. */

const char *trax_version(void);
trax_status trax_ctx_create(trax_ctx **out, int device);
void trax_ctx_destroy(trax_ctx *ctx);
/* cudaStream_t passed as void*; NULL selects the context's own stream. */
trax_status trax_ctx_set_stream(trax_ctx *ctx, void *stream);
void *trax_ctx_get_stream(trax_ctx *ctx);
/* Message of the last failed call on ctx; with ctx == NULL, of the last
 * failed trax_ctx_create. */
const char *trax_ctx_last_error(const trax_ctx *ctx);
/* Waits for the stream; returns the device status word (or a CUDA error). */
trax_status trax_ctx_synchronize(trax_ctx *ctx);
/* Number of streaming multiprocessors of the context's device. */
int trax_ctx_sm_count(const trax_ctx *ctx);

/* Host-only checks (no device needed).  trax_config_validate enforces the
 * reference's implicit preconditions: triplet i starts on layer i+1, every
 * layer used has geometry, and (when grid is given) lies inside the grid.
 * trax_layout_validate checks that the supplements describe hits bucketed
 * event-major then layer-major with running offsets covering n_hits. */
trax_status trax_config_validate(const trax_config *cfg, const trax_grid_cfg *grid);
trax_status trax_layout_validate(const trax_layout *layout, uint32_t n_hits);
/* sizeof of an ABI struct by name ("trax_config", ...); 0 if unknown. */
size_t trax_abi_sizeof(const char *type_name);

/* Validates and stores the per-run parameters; computes minRadiusCurvature
 * (TripletConfiguration.cpp:145-152). */
trax_status trax_configure(trax_ctx *ctx, const trax_config *cfg);
/* TripletConfigurations::minRadiusCurvature(minPt, Bz) in cm. */
float trax_min_radius_curvature(float min_pt, float bz);

/* How the pair and prediction kernels visit a window's candidates.  Results
 * never depend on it, only speed: a run of neighbouring cells with at most
 * run_walk hits is walked hit by hit; in larger runs, every cell with more
 * than index_min (<= 256) hits is searched through a per-cell z index.
 * pair_record selects the pair kernels: 3 walks one outer hit per lane in a
 * count pass, scans the counts and copies the kept accepts in a store pass;
 * 2 walks one outer hit per lane with a look-back in one kernel, keeping 16
 * accepts per outer hit for the store (4: the same keeping 48, for outer hits
 * with a few dozen pairs each); 1 and 0
 * sweep each outer hit's candidates with the whole warp, replaying the count
 * sweep's ballots for the store (1) or sweeping twice (0).  Sparse events
 * favour walking and pair_record 3, dense (pile-up) events the index.
 * blocks_per_sm caps the resident blocks per SM of the candidate kernels
 * (pairs, prediction, filter: grid-stride kernels launched one wave deep);
 * 0 launches as many as fit -- the launch shape the reference sweeps as its
 * work-group size (TripletBuilder.cpp:345, configs' `threads`).
 * trax_configure installs run_walk 48, index_min 16, pair_record 3,
 * blocks_per_sm 0. */
typedef struct trax_tuning {
    uint32_t run_walk;
    uint32_t index_min;
    uint32_t pair_record;
    uint32_t blocks_per_sm;
} trax_tuning;
trax_status trax_set_tuning(trax_ctx *ctx, const trax_tuning *t);

/* Which pair generator the batched pipeline (trax_seed_batch,
 * trax_run_staged) runs.  The reference's TripletBuilder runs the beam-spot
 * generator (TripletBuilder.cpp:247-250; the sector one's include is
 * commented out at :32).  Unlike the tuning, this changes results. */
#define TRAX_PAIRS_BEAMSPOT 0
#define TRAX_PAIRS_SECTOR 1
trax_status trax_set_pair_generator(trax_ctx *ctx, int generator);
int trax_get_pair_generator(const trax_ctx *ctx);
trax_status trax_get_tuning(const trax_ctx *ctx, trax_tuning *t);

/* ---- device memory helpers (for hosts without their own CUDA binding) --
 * Stand in for clever::OpenCLTransfer's initBuffers / toDevice / fromDevice
 * on the collections (HitCollection.h:57, TripletBuilder.cpp:225-238). */

trax_status trax_dev_alloc(trax_ctx *ctx, void **ptr, size_t bytes);
trax_status trax_dev_free(trax_ctx *ctx, void *ptr);
trax_status trax_host_alloc_pinned(trax_ctx *ctx, void **ptr, size_t bytes);
trax_status trax_host_free_pinned(trax_ctx *ctx, void *ptr);
trax_status trax_memcpy_h2d(trax_ctx *ctx, void *dst, const void *src, size_t bytes);
trax_status trax_memcpy_d2h(trax_ctx *ctx, void *dst, const void *src, size_t bytes);
trax_status trax_memset_d(trax_ctx *ctx, void *dst, int value, size_t bytes);
/* CUDA-event timing on the context stream: record marks, read elapsed ms
 * (the per-stage times the reference's RuntimeRecord collects from OpenCL
 * events, RuntimeRecord.h:67). */
trax_status trax_timer_record(trax_ctx *ctx, int slot);
trax_status trax_timer_elapsed_ms(trax_ctx *ctx, int slot_begin, int slot_end, float *ms);

/* ---- the four stages -------------------------------------------------- */

/* GridBuilder::run (GridBuilder.cpp:6-160): per (event, layer) counting sort
 * of the hits into (z, phi) cells.  Writes the exclusive-scanned grid
 * (n_events * n_layers * (nZ+1)(nPhi+1) uint32, device) and the sorted hit
 * columns.  Within a cell hits keep their input order (the reference's order
 * there is racy, GridBuilder.h:243-244). */
trax_status trax_grid_build(trax_ctx *ctx, const trax_hits *in, const trax_layout *layout,
                            const trax_grid_cfg *grid, trax_sorted_hits *out,
                            uint32_t *d_grid);

/* PairGeneratorBeamspot::run (PairGeneratorBeamspot.cpp:5-177): for every
 * (event, layer triplet) and every hit on layer2, the beam-spot z/phi window
 * on layer1; writes distinct accepted pairs (inner, outer) ordered by outer
 * hit, then inner hit. */
trax_status trax_pair_gen(trax_ctx *ctx, const trax_sorted_hits *hits, const uint32_t *d_grid,
                          const trax_grid_cfg *grid, trax_pairs *out);

/* PairGeneratorSector::run (PairGeneratorSector.h:38-39, .cpp:5-151): no
 * cut; every layer2 hit in the cells within pairSpreadZ rows and
 * pairSpreadPhi columns of the layer1 hit's own cell (with the reference's
 * unsigned z-underflow and phi wrap arithmetic, PairGeneratorSector.h:96-140).
 * Writes distinct pairs (inner, outer) ordered by inner hit, then outer hit. */
trax_status trax_pair_gen_sector(trax_ctx *ctx, const trax_sorted_hits *hits,
                                 const uint32_t *d_grid, const trax_grid_cfg *grid,
                                 trax_pairs *out);

/* TripletThetaPhiPredictor::run (TripletThetaPhiPredictor.cpp:10-131):
 * per pair, the theta/phi window on layer3; writes candidates
 * (pair index, hit3) with the reference's count/store semantics. */
trax_status trax_triplet_predict(trax_ctx *ctx, const trax_sorted_hits *hits,
                                 const uint32_t *d_grid, const trax_grid_cfg *grid,
                                 const trax_pairs *pairs, trax_pairs *candidates);

/* TripletThetaPhiFilter::run (TripletThetaPhiFilter.cpp:10-164): dTheta,
 * dPhi, circle-fit TIP and minimum-radius cuts; writes tracklets in candidate
 * order. */
trax_status trax_triplet_filter(trax_ctx *ctx, const trax_sorted_hits *hits,
                                const trax_grid_cfg *grid, const trax_pairs *pairs,
                                const trax_pairs *candidates, trax_tracklets *out);

/* PrefixSum::run (src/algorithms/PrefixSum.h:42-43, PrefixSum.cpp:8-30):
 * exclusive scan of n uint32 (device pointers; in place allowed).  One
 * single-pass decoupled-look-back kernel instead of the reference's
 * recursive work-group scans.  The total goes to *d_total when non-NULL. */
trax_status trax_prefix_sum(trax_ctx *ctx, const uint32_t *d_in, uint32_t *d_out, uint32_t n,
                            uint32_t *d_total);

/* Allocation-free exclusive scan.  No counterpart in the reference.  Some
 * callers of this library cannot call cudaMalloc at the point where they
 * need a scan: code that runs inside another framework's memory pool or
 * allocator callback (a cudaMalloc there re-enters that allocator or waits
 * on its lock), code whose device memory a pool has already reserved in
 * full (a cudaMalloc there fails), and latency-critical paths that cannot
 * take cudaMalloc's implicit device synchronisation.  For them this entry
 * point takes no context and allocates nothing: the look-back scratch of its
 * kernel is a file-scope device array of (TRAX_PREFIX_SUM_NOALLOC_MAX / 4096
 * + 1) 8-byte tile words plus about 100 bytes of counters -- 16.5 KB -- that
 * every GPU which loads this library holds until the process exits.  Same
 * result as trax_prefix_sum.  n is limited to TRAX_PREFIX_SUM_NOALLOC_MAX;
 * a larger n returns TRAX_ERR_BAD_ARG, with the message in
 * trax_prefix_sum_noalloc_error().  Runs on the current device and on
 * `stream` (a cudaStream_t, NULL = the legacy default stream).  The first
 * call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and caches it; make that first call before any
 * stream capture.  Every call clears and reuses the same array, so calls
 * that overlap on the GPU (different streams, or threads without ordering)
 * race: serialise them.
 *
 * The kernel's waits are bounded; a wait that gives up is recorded in the
 * array and makes that call's output invalid.  trax_prefix_sum_noalloc_status
 * synchronises `stream` and returns TRAX_OK or the status the last call on
 * the current device recorded (TRAX_ERR_TIMEOUT); the next call clears it.
 * trax_prefix_sum_noalloc_error() returns the calling thread's last message;
 * the pointer stays valid until that thread's next failing call. */
#define TRAX_PREFIX_SUM_NOALLOC_MAX 8388608u
trax_status trax_prefix_sum_noalloc(const uint32_t *d_in, uint32_t *d_out, uint32_t n,
                                    uint32_t *d_total, void *stream);
trax_status trax_prefix_sum_noalloc_status(void *stream);
const char *trax_prefix_sum_noalloc_error(void);

/* Self-test of the bounded waits (no counterpart in the reference: it has no
 * kernel-side error reporting).  Runs trax_prefix_sum's scan kernel over n
 * elements (n > 4096, device pointers) with tile 0 never taken, so the next
 * tile's look-back waits for a predecessor that never publishes, and with a
 * look-back limit of spin_limit polls for this launch only.  The wait gives
 * up, the kernel records TRAX_ERR_TIMEOUT / TRAX_DETAIL_SCAN_TIMEOUT in the
 * context's status (trax_counts) and returns; d_out is then not a scan.  The
 * context stays usable (trax_reset_counts clears the status). */
trax_status trax_selftest_lookback_timeout(trax_ctx *ctx, const uint32_t *d_in, uint32_t *d_out,
                                           uint32_t n, uint32_t spin_limit);

/* TripletConnectivity::run (src/algorithms/TripletConnectivity.h:52-54,
 * .cpp:21-71): following_con[f] += sum over base tracklets b that chain
 * with f of (base_con[b] + 1).  Wide packing shares one hit (forward: base
 * hit3 == follow hit1; iterate_backwards: base hit1 == follow hit3); tight
 * packing shares two (base hit2, hit3 == follow hit1, hit2; forward only).
 * The semantics are those the reference's own tests pin
 * (src/algorithms/test/TripletConnectivityTest.h:147-259); its wide kernel
 * as written swaps the base and following indices (TripletConnectivity.h:71-73)
 * and would fail its multilayer test.  base_con may be NULL (all zero).
 * Device pointers; asynchronous. */
trax_status trax_triplet_connectivity(trax_ctx *ctx, const trax_tracklets *base,
                                      uint32_t n_base, const uint32_t *base_con,
                                      const trax_tracklets *following, uint32_t n_following,
                                      uint32_t *following_con, int iterate_backwards,
                                      int tight_packing);

/* ---- event ingest ------------------------------------------------------
 * The reference reads PEventContainer files (EventLoader.h:15-111) or event
 * stores (PEventStore.h) with protobuf and selects hits with
 * HitCollection::addEvent (HitCollection.cpp:20-149).  Here a native
 * decoder fills flat columns on the host and trax_ingest runs addEvent for a
 * whole batch of events on the GPU. */
#define TRAX_PB_CONTAINER 0    /* one PEventContainer message (Event.proto:35-38) */
#define TRAX_PB_EVENT_STORE 1  /* uint32 count, then (varint 1, varint size, PEvent)* */

/* Decoded PEvent / PHit fields (Event.proto:9-33), host arrays sized by
 * trax_pb_scan.  Integer fields are cut to the widths the reference stores
 * them in (uint layer, detId and simTrackID); absent optional fields are 0. */
typedef struct trax_pb_events {
    uint32_t n_events;
    uint64_t n_hits;
    uint64_t *run, *lumi, *event_number;   /* [n_events] */
    uint64_t *hit_offset;                  /* [n_events + 1] */
    float *x, *y, *z;                      /* [n_hits] ... */
    int32_t *detector_type;
    uint32_t *layer;
    uint32_t *detector_id;
    uint64_t *hit_id;
    uint32_t *sim_track_id;
    float *sim_track_pt;
} trax_pb_events;

/* Counts the events and hits of a file image.  Malformed input or a missing
 * required field returns TRAX_ERR_BAD_INPUT (message in trax_pb_error()). */
trax_status trax_pb_scan(const uint8_t *buf, size_t len, int format, uint32_t *n_events,
                         uint64_t *n_hits);
/* Decodes into the arrays of *out (n_events / n_hits as scanned), on
 * n_threads host threads (<= 0: all cores). */
trax_status trax_pb_decode(const uint8_t *buf, size_t len, int format, trax_pb_events *out,
                           int n_threads);
const char *trax_pb_error(void);  /* last decoder error of the calling thread */

/* Decoded hit columns on the device, event-major; event_offset[n_events]
 * == n_hits. */
typedef struct trax_raw_hits {
    const float *x, *y, *z;
    const uint32_t *layer, *detector_id, *sim_track_id;
    const float *sim_track_pt;
    const uint32_t *event_offset;  /* [n_events + 1], device */
    uint32_t n_events, n_hits;
} trax_raw_hits;

/* addEvent's parameters: TripletConfigurations::minPt_, the layers the
 * triplets use (bit l-1 for layer l) and the largest of them
 * (loader.maxLayer), data.onlyTracks and data.tracks (-1 = all;
 * TripletBuilder.cpp:337-338). */
typedef struct trax_ingest_cfg {
    float min_pt;
    uint32_t max_layer;
    uint32_t used_layers;
    int only_tracks;
    int32_t num_tracks;
} trax_ingest_cfg;

/* HitCollection columns written by trax_ingest (device, capacity hits). */
typedef struct trax_hits_out {
    float *x, *y, *z;
    uint32_t *layer, *detector_id, *hit_id, *event;
    uint32_t capacity;
} trax_hits_out;

/* The findable tracks addEvent returns (HitCollection::tTrackList), by
 * event and ascending track id: per track the raw hit index (into the
 * decoded columns) of its first, middle (index n/2) and last hit in layer
 * order, which PhysicsRecord::fillData reads (PhysicsRecord.cpp:183-185).
 * Device arrays; offsets [n_events + 1]. */
typedef struct trax_track_list {
    uint32_t *track_id, *inner, *middle, *outer;
    uint32_t *offsets;
    uint32_t capacity;
} trax_track_list;

/* HitCollection::addEvent for every event of the batch: drops hits below
 * min_pt (and of track 0 with only_tracks), keeps the findable tracks (a hit
 * on every used layer; with only_tracks 0 also the others), stops at the
 * num_tracks-th findable track, and writes the hits layer-major per event in
 * the reference's order with DetectorId resolved through the sorted detId
 * table (DetectorGeometry.cpp:4-30; unresolved ids stay raw).  Writes
 * d_layer_nhits[n_events * max_layer] (LayerSupplement) and, if tracks is
 * not NULL, the track list.  Synchronous; *n_hits_out / *n_tracks_out get
 * the totals (TRAX_ERR_CAPACITY when they exceed the capacities). */
trax_status trax_ingest(trax_ctx *ctx, const trax_raw_hits *raw, const trax_ingest_cfg *cfg,
                        const uint32_t *d_det_ids, uint32_t n_det_ids, trax_hits_out *out,
                        uint32_t *d_layer_nhits, trax_track_list *tracks, uint32_t *n_hits_out,
                        uint32_t *n_tracks_out);

/* ---- physics evaluation (PhysicsRecord, PhysicsRecord.cpp:81-368) -------
 * Efficiency, fake and clone rates and their eta / pT histograms per
 * (event, layer triplet), merged per layer triplet (PhysicsRecords). */
typedef struct trax_physics trax_physics;

/* Per (event, layer triplet): tracklets; valid (first find of a findable
 * track), clones (later finds), fakes (hits of different tracks), misc
 * (valid but not findable); findable tracks of the event not found
 * (missed); findable tracks of the event. */
typedef struct trax_physics_counts {
    uint32_t tracklets, valid, clones, fake, misc, missed, findable;
} trax_physics_counts;

trax_status trax_physics_create(trax_physics **out);
void trax_physics_destroy(trax_physics *p);
uint32_t trax_physics_n_records(const trax_physics *p);

/* PhysicsRecord::fillData for every (event, layer triplet) of a batch, in
 * the reference's order (events outer, triplets inner; TripletBuilder.cpp:
 * 272-278), merged into rec.  hits: the sorted hit columns the tracklets
 * index (HitId = simulated track); trk: tracklets with offsets
 * [n_events * n_lt + 1]; mc: the findable-track list of trax_ingest with the
 * decoded coordinates it indexes (d_raw_x/y/z).  Device pointers.  counts
 * (host, [n_events * n_lt]) and categories (host, one per tracklet: 0 valid,
 * 1 clone, 2 fake, 3 misc) may be NULL.  Synchronous.  Pseudorapidity uses
 * the project's FP64 asinh (trax_math.h), which agrees with the C library's
 * to an ulp or two; a histogram bin can differ only for a value within that
 * distance of a bin edge. */
trax_status trax_physics_eval(trax_ctx *ctx, trax_physics *rec, const trax_sorted_hits *hits,
                              const trax_tracklets *trk, uint32_t n_events, uint32_t n_lt,
                              const trax_track_list *mc, const float *d_raw_x,
                              const float *d_raw_y, const float *d_raw_z,
                              trax_physics_counts *counts, uint8_t *categories);

/* Adds one (event, layer triplet) record from host arrays: the tracklets'
 * categories and bin numbers floor(eta / 0.1), floor(pT / 0.1), and the
 * missed tracks' bin numbers.  trax_physics_eval calls it per group. */
trax_status trax_physics_add_group(trax_physics *rec, uint32_t event, uint32_t lt,
                                   const trax_physics_counts *c, const uint8_t *cat,
                                   const double *eta_bin, const double *pt_bin, uint32_t n_trk,
                                   const double *miss_eta_bin, const double *miss_pt_bin,
                                   uint32_t n_missed);

/* PhysicsRecords::csvDump text (what 0) or one record's eta (1) / pT (2)
 * histogram file text (tHistogram::csvDump); layer_triplet selects the
 * record, records + 1 the merged total.  *len gets the full length; with
 * buf the text is copied NUL-terminated (TRAX_ERR_CAPACITY if cut). */
trax_status trax_physics_csv(const trax_physics *rec, int what, uint32_t layer_triplet,
                             char *buf, size_t cap, size_t *len);

trax_status trax_read_counts(trax_ctx *ctx, trax_counts *out);  /* synchronises */

/* Diagnostic: evaluates the path's FP32 math on the device for n inputs
 * (fn 0: atan2(a, b), 1: acos(a), 2: atan(a); 3 and 4: the float-to-uint /
 * float-to-int casts of the sector arithmetic, result bits stored in the
 * float output; 5: floor(a / b) in the kernels' reciprocal form); device
 * pointers. */
trax_status trax_eval_math(trax_ctx *ctx, int fn, const float *d_a, const float *d_b,
                           float *d_out, uint32_t n);
trax_status trax_reset_counts(trax_ctx *ctx);

/* ---- batched pipeline -------------------------------------------------
 * The body of the reference's event-group loop (TripletBuilder.cpp:186-263:
 * addEvent, uploads, the four stages, the result downloads) as one call on
 * reserved buffers and one CUDA graph. */

/* Host-side batch of events, bucketed as HitCollection::addEvent does.  The
 * batched calls (trax_stage_batch, trax_seed_batch, trax_submit_batch,
 * trax_count_pairs_batch, the server) upload and read x, y, z, layer and
 * event only: detector_id and hit_id are not used on that path (tracklets
 * come back as input positions, or sorted positions whose hits are never
 * returned) and may be null. */
typedef struct trax_event_batch {
    uint32_t n_events;
    uint32_t n_layers;
    uint32_t n_hits;
    const float *x, *y, *z;
    const uint32_t *layer, *detector_id, *hit_id, *event;
    const uint32_t *layer_nhits;  /* [n_events * n_layers] */
} trax_event_batch;

/* Host-side result.  Tracklet hit indices are input positions of the hits
 * (the reference's sorted indices mapped through `orig`) when
 * `input_indices` is non-zero, else sorted indices. */
typedef struct trax_batch_result {
    uint32_t *hit1, *hit2, *hit3;  /* host, capacity entries */
    uint32_t *offsets;             /* host, n_events * n_layer_triplets + 1 */
    uint32_t capacity;
    int input_indices;
    uint32_t n_tracklets;          /* out */
    trax_counts counts;            /* out */
} trax_batch_result;

/* Pre-sizes every device buffer of the batched pipeline so that later
 * trax_seed_batch calls allocate nothing and replay one CUDA graph. */
trax_status trax_reserve(trax_ctx *ctx, uint32_t max_events, uint32_t max_layers,
                         uint32_t max_hits, const trax_grid_cfg *grid,
                         uint32_t max_pairs, uint32_t max_candidates,
                         uint32_t max_tracklets);

/* Uploads the batch, runs grid build -> pairs -> predict -> filter as one
 * CUDA graph and downloads the tracklets.  Synchronous.  A batch of a million
 * hits or more runs as two halves of its events through the streaming
 * slots below, the second half's upload overlapping the first half's chain;
 * the result is the same. */
trax_status trax_seed_batch(trax_ctx *ctx, const trax_event_batch *in, trax_batch_result *out);

/* Admission bound for serving (no counterpart in the reference, which sizes
 * its Pairing after a blocking download of the scanned pair count,
 * PairGeneratorBeamspot.cpp:117-136).  Stages the batch like
 * trax_stage_batch, runs the grid build and the pair stage's count passes --
 * per outer hit its distinct pairs, their scan, the per-(event, layer
 * triplet) offsets -- and writes each event's pair total to
 * event_pairs[n_events] (host).  Nothing is stored; synchronous.  These are
 * exactly the pairs trax_seed_batch would store for the event, in any batch.
 * Needs the beam-spot pair generator. */
trax_status trax_count_pairs_batch(trax_ctx *ctx, const trax_event_batch *in,
                                   uint32_t *event_pairs);

/* Streaming form of trax_seed_batch (the reference's per-group loop in
 * TripletBuilder.cpp:183-285, with the next group's upload overlapping this
 * group's chain).  trax_submit_batch queues one batch -- its upload on the
 * context's copy stream, then the chain's graph and a copy of the results
 * into the batch's own device buffers -- and returns at once with a ticket;
 * trax_wait_batch waits for that batch, downloads its tracklets and offsets
 * into the output buffers given at submit (on a third stream, while the next
 * batch computes) and fills n_tracklets and counts (status and capacity
 * errors as trax_seed_batch).  Two batches may be in flight; a third submit
 * before a wait returns TRAX_ERR_BAD_ARG.  Pinned host buffers
 * (trax_host_alloc_pinned or cudaHostAlloc) make the copies asynchronous;
 * inputs and outputs must stay in place until the wait returns. */
trax_status trax_submit_batch(trax_ctx *ctx, const trax_event_batch *in,
                              const trax_batch_result *out, uint32_t *ticket);
trax_status trax_wait_batch(trax_ctx *ctx, uint32_t ticket, trax_batch_result *out);

/* Device-resident variant for throughput measurement: the batch was uploaded
 * by trax_stage_batch; runs the graph only (asynchronous). */
trax_status trax_stage_batch(trax_ctx *ctx, const trax_event_batch *in);
trax_status trax_run_staged(trax_ctx *ctx);
/* The same chain launched kernel by kernel, without a graph (the plain form). */
trax_status trax_run_staged_eager(trax_ctx *ctx);

/* Per-kernel timing of the batched chain: when on, CUDA events are recorded
 * between kernels (also inside the graph).  trax_kernel_times returns the
 * durations (ms) and names of the last run's kernels in launch order. */
trax_status trax_set_profiling(trax_ctx *ctx, int on);
trax_status trax_kernel_times(trax_ctx *ctx, float *ms, const char **names, int max_n, int *n);
/* Kernels launched by the last pipeline enqueue (graph capture or eager). */
int trax_kernel_launches(const trax_ctx *ctx);

/* ---- continuous-batching server --------------------------------------
 * No counterpart in the reference, which runs its event groups one after
 * another (TripletBuilder.cpp:186). */

/* Requests are single events.  `slots` worker threads each own a context
 * (stream, reserved buffers, graph); each takes every request that has
 * arrived, up to its capacity, into its next batch, so batches of different
 * slots overlap on the device.  The memory budget is split over the slots;
 * a batch whose scanned pair / candidate / tracklet totals exceed the
 * capacities is split in halves and rerun.  Results are per event and do not
 * depend on the batch (tracklet hit indices are positions within the event). */
typedef struct trax_server trax_server;

typedef struct trax_server_opts {
    uint32_t slots;                /* batches in flight, 1..16 */
    uint32_t max_batch_events;     /* events per batch */
    uint32_t max_event_hits;       /* largest event accepted */
    uint32_t n_layers;             /* per-event grid */
    uint32_t n_sectors_z;
    uint32_t n_sectors_phi;
    uint64_t memory_budget_bytes;  /* device memory for all slots */
    int keep_results;              /* 0: results are only counted (load tests) */
    uint32_t max_batch_hits;       /* hits per batch; 0: as many as the budget allows */
    uint32_t pairs_per_hit;        /* capacity ratios; 0: 24 pairs, 12 candidates, */
    uint32_t candidates_per_hit;   /*   4 tracklets per hit of the batch */
    uint32_t tracklets_per_hit;
    trax_tuning tuning;            /* installed on every slot; all zero: the default */
} trax_server_opts;

typedef struct trax_server_result {
    uint64_t ticket;
    int status;                    /* trax_status of this request */
    uint64_t arrival_ns, start_ns, done_ns;   /* trax_now_ns clock */
    uint32_t batch_events;         /* events in the batch that served it */
    uint32_t *hit1, *hit2, *hit3;  /* caller buffers (host) */
    uint32_t capacity;
    uint32_t n_tracklets;
    uint32_t offsets[TRAX_MAX_LAYER_TRIPLETS + 1];  /* per layer triplet, within the event */
} trax_server_result;

typedef struct trax_server_stats {
    uint64_t submitted, events, batches, batched_events, splits, errors;
    uint64_t slot_max_hits;        /* hit capacity of one slot's batch */
    uint64_t p50_ns, p99_ns, max_ns;   /* arrival -> result latency */
    double sustained_events_per_s;     /* events / (last result - first arrival) */
    uint64_t slot_max_pairs;       /* pair capacity of one slot's batch */
    uint64_t count_passes;         /* admission pair-count passes run */
    uint64_t deferred;             /* requests sent back to the queue by the pair bound */
} trax_server_stats;

uint64_t trax_now_ns(void);  /* monotonic clock used for arrivals and latencies */
trax_status trax_server_create(trax_server **out, int device, const trax_config *cfg,
                               const trax_server_opts *opts);
void trax_server_destroy(trax_server *srv);
/* Queues one event (n_events == 1).  arrival_ns: when the request counts as
 * arrived (0 = now); it is not admitted earlier.  borrow != 0: the host
 * columns are used in place and must stay valid until the result is out. */
trax_status trax_server_submit(trax_server *srv, const trax_event_batch *event,
                               uint64_t arrival_ns, int borrow, uint64_t *ticket);
/* Submits pool[order[i]] at arrival_ns[i] for i < n from a feeder thread
 * (borrowed; the pool, order and arrivals must outlive trax_server_drain). */
trax_status trax_server_replay(trax_server *srv, const trax_event_batch *pool,
                               const uint32_t *order, const uint64_t *arrival_ns, uint32_t n);
/* Next finished request (keep_results != 0), waiting up to timeout_ms. */
trax_status trax_server_poll(trax_server *srv, trax_server_result *out, int timeout_ms);
/* Waits until every submitted request has finished. */
trax_status trax_server_drain(trax_server *srv, int timeout_ms);
trax_status trax_server_get_stats(trax_server *srv, trax_server_stats *out);
trax_status trax_server_reset_stats(trax_server *srv);

#ifdef __cplusplus
}
#endif

#endif /* TRAX_H */
