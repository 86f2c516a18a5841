/*
 * trax_oracle.h -- CPU restatement of trax's triplet-seeding path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library; the product path never
 * calls it.  It follows the reference kernels loop by loop (file:line cited
 * at each function in trax_oracle.c), using the same project FP32 math
 * (trax_gb300/csrc/trax_math.h) as the CUDA kernels.
 *
 * Parity status: pinned to the reference's own kernels.  The reference's host
 * side cannot be built here (empty `clever` submodule, no OpenCL headers or
 * device, no Boost, no protobuf-2.4 runtime), but its OpenCL kernel text can:
 * oracle/ref_build.py compiles it for the host into oracle/_ref, and
 * tests/test_ref_pin.py shows this restatement equal to it element for
 * element (grid, sorted columns, pair and candidate slots, tracklets, every
 * offset array, slot totals) on every workload, at the reference's
 * work-group sizes, for every kernel variant and both pair generators, and on
 * the reference's own ttbar events.  The golden vectors of tests/golden/ are
 * the reference kernels' output.
 */
#ifndef TRAX_ORACLE_H
#define TRAX_ORACLE_H

#include <stdint.h>
#include "../include/trax.h"

#ifdef __cplusplus
extern "C" {
#endif

enum or_item {
    OR_SORTED_X = 0, OR_SORTED_Y, OR_SORTED_Z, OR_SORTED_PHI,
    OR_SORTED_LAYER, OR_SORTED_DET, OR_SORTED_HITID, OR_SORTED_EVENT, OR_SORTED_ORIG,
    OR_GRID,
    OR_PAIRS,          /* uint32[2*slots] in the reference's slot layout */
    OR_PAIR_VALID,     /* uint8[slots]: 0 marks a slot pairStore leaves unwritten */
    OR_PAIR_OFFSETS,   /* uint32[E*T+1] */
    OR_CANDS,
    OR_CAND_VALID,
    OR_CAND_OFFSETS,
    OR_TRK_H1, OR_TRK_H2, OR_TRK_H3,
    OR_TRK_OFFSETS,
    OR_STATS,          /* uint64[OR_NSTATS] */
    OR_NITEMS
};

enum or_stat {
    ORS_STATUS = 0,        /* trax_status of the first fault */
    ORS_DETAIL,            /* TRAX_DETAIL_* */
    ORS_PAIR_SLOTS,        /* pairCount total (reference Pairing size) */
    ORS_PAIRS,             /* distinct pairs written */
    ORS_CAND_SLOTS,        /* predictCount total */
    ORS_CANDS,             /* candidates written */
    ORS_CAND_TRUNCATED,    /* store-window accepts beyond the count */
    ORS_TRACKLETS,
    OR_NSTATS
};

typedef struct or_result or_result;

/*
 * Runs stages 1..n_stages (1 grid, 2 pairs, 3 predict, 4 filter) on host
 * arrays.  n_threads is the reference's work-group size (exec.threads), which
 * fixes the pair slot layout and the scan blocking.  n_omp_threads > 1
 * parallelises over segments, groups and candidates with identical results.
 * Returns NULL only on allocation failure.
 */
or_result *or_run(const trax_config *cfg, const trax_grid_cfg *grid,
                  const float *x, const float *y, const float *z,
                  const uint32_t *layer, const uint32_t *det, const uint32_t *hitid,
                  const uint32_t *event, uint32_t n_hits,
                  const uint32_t *event_offset, const uint32_t *layer_nhits,
                  const uint32_t *layer_offset, int n_stages, uint32_t n_threads,
                  int n_omp_threads);
/* or_run with a choice of pair generator: OR_PAIRS_BEAMSPOT
 * (PairGeneratorBeamspot, the one the reference's TripletBuilder runs) or
 * OR_PAIRS_SECTOR (PairGeneratorSector). */
enum { OR_PAIRS_BEAMSPOT = 0, OR_PAIRS_SECTOR = 1 };
or_result *or_run_ex(const trax_config *cfg, const trax_grid_cfg *grid,
                     const float *x, const float *y, const float *z,
                     const uint32_t *layer, const uint32_t *det, const uint32_t *hitid,
                     const uint32_t *event, uint32_t n_hits,
                     const uint32_t *event_offset, const uint32_t *layer_nhits,
                     const uint32_t *layer_offset, int n_stages, uint32_t n_threads,
                     int n_omp_threads, int pair_generator);
uint64_t or_size(const or_result *r, int item);  /* elements */
const void *or_data(const or_result *r, int item);
void or_free(or_result *r);

/* PrefixSum::run restated (PrefixSum.cpp:35-126, PrefixSum.h:55-245):
 * in-place exclusive scan by recursive work-group scans. */
void or_prefix_sum(uint32_t *data, uint32_t n, uint32_t wg);

/* TripletConnectivity::run (TripletConnectivity.cpp:21-71) with the
 * semantics its tests pin (TripletConnectivityTest.h:147-259):
 * follow_con[f] += sum_b [key(b) == key(f)] * (base_con[b] + 1).
 * or_connectivity_literal_wide restates the wide kernel exactly as written
 * (TripletConnectivity.h:67-75: base indexed by the following id). */
void or_connectivity(const uint32_t *b1, const uint32_t *b2, const uint32_t *b3,
                     const uint32_t *base_con, uint32_t n_base, const uint32_t *f1,
                     const uint32_t *f2, const uint32_t *f3, uint32_t *follow_con,
                     uint32_t n_follow, int iterate_backwards, int tight_packing);
void or_connectivity_literal_wide(const uint32_t *base_hit, const uint32_t *base_con,
                                  uint32_t n_base, const uint32_t *follow_hit,
                                  uint32_t *follow_con, uint32_t n_follow);

/* HitCollection::addEvent (HitCollection.cpp:20-149) on one event of
 * decoded columns [first, first + n): writes the selected hits' indices in
 * the reference's order (layer-major) to out_idx, layer_nhits[max_layer],
 * and per findable track (track id, first, middle, last hit in layer order)
 * to trk (4 words each, may be NULL).  Returns the number of hits. */
uint32_t or_add_event(const uint32_t *layer, const uint32_t *track, const float *pt,
                      uint32_t first, uint32_t n, float min_pt, uint32_t max_layer,
                      uint32_t used_mask, int only_tracks, int32_t num_tracks,
                      uint32_t *out_idx, uint32_t *layer_nhits, uint32_t *trk,
                      uint32_t *n_trk);

/* PhysicsRecord::fillData (PhysicsRecord.cpp:81-218) for every (event,
 * layer triplet): counts[g][7] = tracklets, valid, clones, fake, misc,
 * missed, findable; per tracklet its category (0 valid, 1 clone, 2 fake,
 * 3 misc) and bin numbers floor(eta / 0.1), floor(pT / 0.1); per (layer
 * triplet, findable track) whether it was missed and its bin numbers. */
void or_physics(const uint32_t *hid, const float *x, const float *y, const float *z,
                const uint32_t *h1, const uint32_t *h2, const uint32_t *h3, const uint32_t *toff,
                uint32_t n_events, uint32_t n_lt, const uint32_t *mc_id, const uint32_t *mc_in,
                const uint32_t *mc_mid, const uint32_t *mc_out, const uint32_t *mc_off,
                const float *rx, const float *ry, const float *rz, uint32_t *counts,
                uint8_t *cat, double *eta_bin, double *pt_bin, uint8_t *missed,
                double *miss_eta_bin, double *miss_pt_bin);
double or_asinh(double t);

/* Project math, exported so tests can compare against libm / CUDA. */
float or_atan2f(float y, float x);
float or_acosf(float x);
float or_atanf(float x);
float or_min_radius_curvature(float min_pt, float bz);
uint64_t or_floor_div_mismatches(const float *x, const float *d, uint64_t n);
/* fn 0: atan2(a, b), 1: acos(a), 2: atan(a), 3: trax_f2u(a), 4: trax_f2i(a)
 * (3, 4: the integer's bits in the float output), over n floats. */
void or_math_batch(int fn, const float *a, const float *b, float *out, uint64_t n);

#ifdef __cplusplus
}
#endif

#endif
