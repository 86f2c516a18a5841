/*
 * trax_oracle.c -- CPU restatement of trax's triplet-seeding path.
 *
 * TEST INFRASTRUCTURE ONLY (see trax_oracle.h).  Loop structure, index
 * arithmetic and FP32 operation order follow the reference OpenCL kernels
 * line by line; each block cites the lines it restates.  Where the reference
 * has undefined behaviour the restatement chooses a defined outcome and says
 * so:
 *   - within-cell order of the sorted hits is the input order (the reference
 *     uses a racy atomic_inc, GridBuilder.h:243-244);
 *   - slots that pairStore / predictStore leave unwritten (count > stored)
 *     are marked invalid instead of holding garbage, and later stages skip
 *     them;
 *   - a phi window whose sector index falls outside the grid row (possible
 *     only for windows wider than 2*pi) is skipped and flagged instead of
 *     reading outside the grid;
 *   - a hit outside the grid (|z| > 300 cm, NaN) is clamped to the last cell
 *     and flagged instead of writing outside the grid.
 * Compile with -ffp-contract=off and without -ffast-math.
 */
#include "trax_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../trax_gb300/csrc/trax_math.h"

struct or_result {
    uint64_t size[OR_NITEMS];
    void *data[OR_NITEMS];
    uint64_t stats[OR_NSTATS];
};

typedef struct { uint32_t x, y; } u2;

static void set_fault(or_result *r, uint32_t status, uint32_t detail)
{
    int first = 0;
#pragma omp critical(or_fault)
    {
        if (r->stats[ORS_STATUS] == 0) {
            r->stats[ORS_STATUS] = status;
            r->stats[ORS_DETAIL] = detail;
            first = 1;
        }
    }
    (void)first;
}

static void *alloc_item(or_result *r, int item, uint64_t n, size_t elem)
{
    r->size[item] = n;
    r->data[item] = calloc(n ? n : 1, elem);
    return r->data[item];
}

float or_atan2f(float y, float x) { return trax_atan2f(y, x); }
float or_acosf(float x) { return trax_acosf(x); }
float or_atanf(float x) { return trax_atanf(x); }

/* trax_floor_div(x, d, 1/d) and floorf(x / d) for n pairs: the kernels'
 * reciprocal form must equal the plain division everywhere. */
uint64_t or_floor_div_mismatches(const float *x, const float *d, uint64_t n)
{
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float a = trax_floor_div(x[i], d[i], 1.0f / d[i]);
        const float b = floorf(x[i] / d[i]);
        if (!(a == b || (a != a && b != b))) ++bad;
    }
    return bad;
}

void or_math_batch(int fn, const float *a, const float *b, float *out, uint64_t n)
{
    for (uint64_t i = 0; i < n; ++i)
    {
        if (fn <= 2) {
            out[i] = fn == 0 ? trax_atan2f(a[i], b[i]) : fn == 1 ? trax_acosf(a[i]) : trax_atanf(a[i]);
        } else {
            const uint32_t u = fn == 3 ? trax_f2u(a[i]) : (uint32_t)trax_f2i(a[i]);
            memcpy(&out[i], &u, 4);
        }
    }
}

/* TripletConfigurations::minRadiusCurvature (TripletConfiguration.cpp:145-152),
 * called with IDEAL_BZ = 3.8112 converted to the float parameter Bz
 * (TripletConfiguration.h:60-64,70). */
float or_min_radius_curvature(float min_pt, float bz)
{
    const double Q = 1.602177E-19;
    const double GEV_C = 5.344286E-19;
    if (bz == 0.0f) bz = (float)3.8112;
    return (float)(min_pt * GEV_C / (bz * Q) * 1E2);
}

/* ------------------------------------------------------------------------
 * PrefixSum (PrefixSum.h:55-245, PrefixSum.cpp:35-126).
 * One work-group scans 2*ls elements through a bank-padded local array:
 * up-sweep (:77-93), clear last (:98-104 / :181-188), down-sweep (:107-124).
 * Work-items run in lock step: each barrier-separated phase is a loop over
 * lid.
 * ---------------------------------------------------------------------- */
#define OR_BANK_OFFSET(i) ((i) >> 4)

static void wg_scan(uint32_t *input, uint32_t size, uint32_t gid, uint32_t ls,
                    uint32_t *partial, uint32_t *data)
{
    const uint32_t gOffset = gid * (ls << 1);
    for (uint32_t lid = 0; lid < ls; ++lid) {
        data[lid + OR_BANK_OFFSET(lid)] = (gOffset + lid) < size ? input[gOffset + lid] : 0;
        data[lid + ls + OR_BANK_OFFSET(lid + ls)] =
            (gOffset + lid + ls) < size ? input[gOffset + lid + ls] : 0;
    }
    uint32_t offset = 1;
    for (uint32_t d = ls; d > 0; d >>= 1) {
        for (uint32_t lid = 0; lid < d; ++lid) {
            uint32_t ai = offset * ((lid << 1) + 1) - 1;
            uint32_t bi = offset * ((lid << 1) + 2) - 1;
            ai += OR_BANK_OFFSET(ai);
            bi += OR_BANK_OFFSET(bi);
            data[bi] += data[ai];
        }
        offset <<= 1;
    }
    {
        uint32_t idx = (ls << 1) - 1;
        idx += OR_BANK_OFFSET(idx);
        if (partial) partial[gid] = data[idx];
        data[idx] = 0;
    }
    for (uint32_t d = 1; d <= ls; d <<= 1) {
        offset >>= 1;
        for (uint32_t lid = 0; lid < d; ++lid) {
            uint32_t ai = offset * ((lid << 1) + 1) - 1;
            uint32_t bi = offset * ((lid << 1) + 2) - 1;
            ai += OR_BANK_OFFSET(ai);
            bi += OR_BANK_OFFSET(bi);
            uint32_t t = data[ai];
            data[ai] = data[bi];
            data[bi] += t;
        }
    }
    for (uint32_t lid = 0; lid < ls; ++lid) {
        if (gOffset + lid < size) input[gOffset + lid] = data[lid + OR_BANK_OFFSET(lid)];
        if (gOffset + lid + ls < size) input[gOffset + lid + ls] = data[lid + ls + OR_BANK_OFFSET(lid + ls)];
    }
}

static uint32_t next_pow2(uint32_t n)
{
    n--;
    n |= n >> 1; n |= n >> 2; n |= n >> 4; n |= n >> 8; n |= n >> 16;
    n++;
    return n;
}

/* The group counts are computed through float as in PrefixSum.cpp:35,50,
 * which the reference does for every size; sizes used here stay below 2^24
 * where that is exact. */
static void recursive_scan(uint32_t *input, uint32_t size, uint32_t wg)
{
    float fg = ceilf(((float)size) / (float)(wg << 1));
    uint32_t nGroups = (uint32_t)(fg > 1.0f ? fg : 1.0f);
    uint32_t padding = (wg << 1) / 16;
    if (nGroups == 1) {
        float fl = ceilf(((float)size) / 2);
        uint32_t localSize = (uint32_t)(fl > 1.0f ? fl : 1.0f);
        localSize = next_pow2(localSize);
        uint32_t *data = (uint32_t *)calloc((size_t)(wg << 1) + padding + (localSize << 1) + 64, 4);
        wg_scan(input, size, 0, localSize, NULL, data);
        free(data);
    } else {
        uint32_t *partial = (uint32_t *)calloc(nGroups, 4);
        uint32_t *data = (uint32_t *)calloc((size_t)(wg << 1) + padding + 64, 4);
        for (uint32_t g = 0; g < nGroups; ++g) wg_scan(input, size, g, wg, partial, data);
        free(data);
        recursive_scan(partial, nGroups, wg);
        for (uint32_t g = 0; g < nGroups; ++g) { /* prefixSumUniformAdd, PrefixSum.h:222-243 */
            uint32_t add = partial[g];
            uint32_t gOffset = g * (wg << 1);
            for (uint32_t lid = 0; lid < wg; ++lid) {
                if (gOffset + lid < size) input[gOffset + lid] += add;
                if (gOffset + lid + wg < size) input[gOffset + lid + wg] += add;
            }
        }
        free(partial);
    }
}

void or_prefix_sum(uint32_t *data, uint32_t n, uint32_t wg)
{
    if (n == 0) return;
    if (wg == 0) wg = 1;
    recursive_scan(data, n, wg);
}

/* ------------------------------------------------------------------------
 * Stage 1: GridBuilder (GridBuilder.h:48-115 count, :172-257 store;
 * GridBuilder.cpp:6-160).
 * ---------------------------------------------------------------------- */
static void grid_stage(or_result *r, const trax_grid_cfg *g, const float *x, const float *y,
                       const float *z, const uint32_t *layer, const uint32_t *det,
                       const uint32_t *hitid, const uint32_t *event, uint32_t n_hits,
                       const uint32_t *event_offset, const uint32_t *layer_nhits,
                       const uint32_t *layer_offset, uint32_t n_threads, int omp)
{
    const uint32_t E = g->n_events, L = g->n_layers, Z = g->n_sectors_z, P = g->n_sectors_phi;
    const uint32_t C = (Z + 1) * (P + 1);
    const float szZ = trax_sector_size_z(Z);
    const float szP = trax_sector_size_phi(P);
    const long nseg = (long)E * L;

    uint32_t *grid = (uint32_t *)alloc_item(r, OR_GRID, (uint64_t)E * L * C, 4);
    float *sx = (float *)alloc_item(r, OR_SORTED_X, n_hits, 4);
    float *sy = (float *)alloc_item(r, OR_SORTED_Y, n_hits, 4);
    float *sz = (float *)alloc_item(r, OR_SORTED_Z, n_hits, 4);
    float *sphi = (float *)alloc_item(r, OR_SORTED_PHI, n_hits, 4);
    uint32_t *sl = (uint32_t *)alloc_item(r, OR_SORTED_LAYER, n_hits, 4);
    uint32_t *sd = (uint32_t *)alloc_item(r, OR_SORTED_DET, n_hits, 4);
    uint32_t *sh = (uint32_t *)alloc_item(r, OR_SORTED_HITID, n_hits, 4);
    uint32_t *se = (uint32_t *)alloc_item(r, OR_SORTED_EVENT, n_hits, 4);
    uint32_t *so = (uint32_t *)alloc_item(r, OR_SORTED_ORIG, n_hits, 4);

    /* gridCount (GridBuilder.h:75-94): zSector, phiSector per hit, histogram. */
#pragma omp parallel for schedule(dynamic, 1) if (omp)
    for (long seg = 0; seg < nseg; ++seg) {
        const uint32_t e = (uint32_t)(seg / L), l = (uint32_t)(seg % L);
        const uint32_t hits = layer_nhits[e * L + l];
        const uint32_t offset = event_offset[e] + layer_offset[e * L + l];
        uint32_t *lGrid = grid + (uint64_t)seg * C;
        for (uint32_t i = 0; i < hits; ++i) {
            const uint32_t h = offset + i;
            uint32_t zSector = trax_sector_z(z[h], szZ);
            const float phi = trax_atan2f(y[h], x[h]);
            uint32_t phiSector = trax_sector_phi(phi, szP);
            if (zSector > Z || phiSector > P) {
                set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_OUTSIDE_GRID);
                if (zSector > Z) zSector = Z;
                if (phiSector > P) phiSector = P;
            }
            if (layer[h] != l + 1 || event[h] != e)
                set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH);
            lGrid[zSector * (P + 1) + phiSector] += 1;
        }
    }

    /* PrefixSum over the whole grid (GridBuilder.cpp:58). */
    if (!omp) {
        or_prefix_sum(grid, (uint32_t)((uint64_t)E * L * C), n_threads);
    } else {
        /* Same result: the exclusive prefix before a segment is the number of
         * hits in all earlier segments, i.e. its start in the bucketed input. */
#pragma omp parallel for schedule(static) if (omp)
        for (long seg = 0; seg < nseg; ++seg) {
            const uint32_t e = (uint32_t)(seg / L), l = (uint32_t)(seg % L);
            uint32_t run = event_offset[e] + layer_offset[e * L + l];
            uint32_t *lGrid = grid + (uint64_t)seg * C;
            for (uint32_t c = 0; c < C; ++c) {
                uint32_t t = lGrid[c];
                lGrid[c] = run;
                run += t;
            }
        }
    }

    /* gridStore (GridBuilder.h:238-253) with the within-cell order fixed to
     * the input order. */
#pragma omp parallel for schedule(dynamic, 1) if (omp)
    for (long seg = 0; seg < nseg; ++seg) {
        const uint32_t e = (uint32_t)(seg / L), l = (uint32_t)(seg % L);
        const uint32_t offset = event_offset[e] + layer_offset[e * L + l];
        const uint32_t hits = offset + layer_nhits[e * L + l];
        const uint32_t *lGrid = grid + (uint64_t)seg * C;
        uint32_t *written = (uint32_t *)calloc(C, 4);
        for (uint32_t i = offset; i < hits; ++i) {
            uint32_t zSector = trax_sector_z(z[i], szZ);
            const float phi = trax_atan2f(y[i], x[i]);
            uint32_t phiSector = trax_sector_phi(phi, szP);
            if (zSector > Z) zSector = Z;
            if (phiSector > P) phiSector = P;
            const uint32_t cell = zSector * (P + 1) + phiSector;
            const uint32_t w = lGrid[cell] + written[cell]++;
            if (w >= n_hits) { set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH); continue; }
            sx[w] = x[i]; sy[w] = y[i]; sz[w] = z[i]; sphi[w] = phi;
            sl[w] = layer[i]; sd[w] = det[i]; sh[w] = hitid[i]; se[w] = event[i]; so[w] = i;
        }
        free(written);
    }
}

/* ------------------------------------------------------------------------
 * Stage 2: PairGeneratorBeamspot (pairCount PairGeneratorBeamspot.h:43-246,
 * pairStore :448-525, host PairGeneratorBeamspot.cpp:9-152).
 * ---------------------------------------------------------------------- */
typedef struct {
    uint32_t *bits;   /* oracle bitmap of this (event, layer triplet) */
    uint32_t nHits1, nHits2, offset, layer2Offset;
} pair_group;

static inline float f_as(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static void pair_stage(or_result *res, const trax_config *cfg, const trax_grid_cfg *g,
                       float minRadiusCurvature, uint32_t nThreads, int omp)
{
    const uint32_t E = g->n_events, L = g->n_layers, Z = g->n_sectors_z, P = g->n_sectors_phi;
    const uint32_t T = cfg->n_layer_triplets;
    const uint32_t C = (Z + 1) * (P + 1);
    const float minZ = TRAX_MIN_Z, minPhi = TRAX_MIN_PHI;
    const float sectorSizeZ = trax_sector_size_z(Z), sectorSizePhi = trax_sector_size_phi(P);
    const uint32_t *grid = (const uint32_t *)res->data[OR_GRID];
    const float *hitGlobalX = (const float *)res->data[OR_SORTED_X];
    const float *hitGlobalY = (const float *)res->data[OR_SORTED_Y];
    const float *hitGlobalZ = (const float *)res->data[OR_SORTED_Z];
    const long G = (long)E * T;

    pair_group *pg = (pair_group *)calloc((size_t)(G ? G : 1), sizeof(pair_group));
    uint32_t *prefixSum = (uint32_t *)calloc((size_t)G * nThreads + 1, 4);

    /* pairCount: one work-group of nThreads per (event, layer pair). */
#pragma omp parallel for schedule(dynamic, 1) if (omp)
    for (long gp = 0; gp < G; ++gp) {
        const uint32_t event = (uint32_t)(gp / T), layerPair = (uint32_t)(gp % T);
        const trax_layer_triplet *lt = &cfg->triplets[layerPair];
        uint32_t layer = lt->layer2 - 1; /* outer layer, :68-73 */
        uint32_t offset = event * L * C + layer * C;
        const uint32_t layer2Offset = grid[offset];
        const uint32_t end = grid[offset + C - 1];
        const uint32_t nHits2 = end - layer2Offset;
        layer = lt->layer1 - 1; /* inner layer, :77-86 */
        offset = event * L * C + layer * C;
        const uint32_t *lGrid1 = grid + offset;
        const uint32_t nHits1 = lGrid1[C - 1] - lGrid1[0];
        const uint32_t off1 = lGrid1[0];

        const float z0 = lt->z0;
        const float tip = lt->tip_cut;
        const float sigmaZ = lt->sigma_z;
        /* The host binds the pairSpreadPhi uint buffer as gSigmaPhi
         * (PairGeneratorBeamspot.cpp:55), so the kernel reads its bits. */
        const float sigmaPhi = f_as(lt->pair_spread_phi);
        const float minLayerRadius1 = cfg->min_radius[layer];
        const float maxLayerRadius1 = cfg->max_radius[layer];

        const uint64_t nbits = (uint64_t)nHits1 * nHits2;
        pg[gp].bits = (uint32_t *)calloc((size_t)((nbits + 31) / 32 + 1), 4);
        pg[gp].nHits1 = nHits1; pg[gp].nHits2 = nHits2;
        pg[gp].offset = off1; pg[gp].layer2Offset = layer2Offset;

        for (uint32_t thread = 0; thread < nThreads; ++thread) {
            uint32_t nFound = 0;
            for (uint32_t i = layer2Offset + thread; i < end; i += nThreads) {
                /* :110-130 */
                const float signRadius = trax_signf(hitGlobalY[i]);
                const float r = signRadius * sqrtf(hitGlobalX[i] * hitGlobalX[i] + hitGlobalY[i] * hitGlobalY[i]);
                const float cotThetaHigh = (hitGlobalZ[i] - z0) / r;
                const float cotThetaLow = (hitGlobalZ[i] + z0) / r;
                float tmp = signRadius * maxLayerRadius1 * cotThetaHigh + z0;
                float zHigh = signRadius * minLayerRadius1 * cotThetaHigh + z0;
                zHigh = (float)(tmp < zHigh) * zHigh + (float)(tmp > zHigh) * tmp;
                tmp = signRadius * maxLayerRadius1 * cotThetaLow - z0;
                float zLow = signRadius * minLayerRadius1 * cotThetaLow - z0;
                zLow = (float)(tmp < zLow) * tmp + (float)(tmp > zLow) * zLow;
                zLow -= sigmaZ;
                zHigh += sigmaZ;
                /* :133-134 */
                int32_t zl = trax_f2i(floorf((zLow - minZ) / sectorSizeZ));
                const uint32_t zLowSector = (uint32_t)(zl > 0 ? zl : 0);
                uint32_t zh = trax_f2u(floorf((zHigh - minZ) / sectorSizeZ)) + 1;
                const uint32_t zHighSector = zh < Z ? zh : Z;
                /* :138-162 */
                const float phi = trax_atan2f(hitGlobalY[i], hitGlobalX[i]);
                tmp = fabsf(trax_acosf(r / (2 * minRadiusCurvature)) - trax_acosf(maxLayerRadius1 / (2 * minRadiusCurvature)));
                float dPhi = fabsf(trax_acosf(r / (2 * minRadiusCurvature)) - trax_acosf(minLayerRadius1 / (2 * minRadiusCurvature)));
                dPhi = (float)(tmp < dPhi) * dPhi + (float)(tmp > dPhi) * tmp;
                tmp = trax_atanf(tip * (r - minLayerRadius1)) / (r * minLayerRadius1);
                float phiHigh = trax_atanf(tip * (r - maxLayerRadius1)) / (r * maxLayerRadius1);
                dPhi += tmp > phiHigh ? tmp : phiHigh;
                float phiLow = phi - dPhi - sigmaPhi;
                phiHigh = phi + dPhi + sigmaPhi;
                const int wrapAround = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
                phiLow -= (float)((phiLow > TRAX_PI_F) * 2) * TRAX_PI_F;
                phiLow += (float)((phiLow < -TRAX_PI_F) * 2) * TRAX_PI_F;
                phiHigh -= (float)((phiHigh > TRAX_PI_F) * 2) * TRAX_PI_F;
                phiHigh += (float)((phiHigh < -TRAX_PI_F) * 2) * TRAX_PI_F;
                const uint32_t phiLowSector = trax_f2u(floorf((phiLow - minPhi) / sectorSizePhi));
                const uint32_t phiHighSector = trax_f2u(floorf((phiHigh - minPhi) / sectorSizePhi)) + 1;
                if (phiLowSector > P + 1 || phiHighSector > P + 1) {
                    set_fault(res, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                    continue;
                }
                /* :172-230 */
                for (uint32_t zSector = zLowSector; zSector < zHighSector; ++zSector) {
                    const uint32_t zSectorStart = lGrid1[zSector * (P + 1)];
                    const uint32_t zSectorEnd = lGrid1[(zSector + 1) * (P + 1) - 1];
                    const uint32_t zSectorLength = zSectorEnd - zSectorStart;
                    uint32_t j = lGrid1[zSector * (P + 1) + phiLowSector];
                    const uint32_t end2 = (uint32_t)wrapAround * zSectorEnd
                                        + lGrid1[zSector * (P + 1) + phiHighSector]
                                        - (uint32_t)wrapAround * zSectorStart;
                    for (; j < end2; ++j) {
                        const uint32_t index = j - (uint32_t)(j >= zSectorEnd) * zSectorLength;
                        int valid = zLow <= hitGlobalZ[index] && hitGlobalZ[index] <= zHigh;
                        const float actPhi = trax_atan2f(hitGlobalY[index], hitGlobalX[index]);
                        valid = valid * ((!wrapAround && (phiLow <= actPhi && actPhi <= phiHigh))
                                  || (wrapAround && ((phiLow <= actPhi && actPhi <= TRAX_PI_F) || (-TRAX_PI_F <= actPhi && actPhi <= phiHigh))));
                        nFound += valid;
                        if (valid) {
                            const uint32_t bit = (index - off1) * nHits2 + i - layer2Offset;
                            pg[gp].bits[bit / 32] |= (1u << (bit % 32));
                        }
                    }
                }
            }
            prefixSum[(uint64_t)event * T * nThreads + (uint64_t)layerPair * nThreads + thread] = nFound;
        }
    }

    /* PrefixSum over the per-thread counts and the total
     * (PairGeneratorBeamspot.cpp:117-120). */
    or_prefix_sum(prefixSum, (uint32_t)((uint64_t)G * nThreads + 1), nThreads);
    const uint32_t nFoundPairs = prefixSum[(uint64_t)G * nThreads];

    u2 *pairs = (u2 *)alloc_item(res, OR_PAIRS, (uint64_t)nFoundPairs * 2, 4);
    uint8_t *valid_slot = (uint8_t *)alloc_item(res, OR_PAIR_VALID, nFoundPairs, 1);
    uint32_t *pairOffsets = (uint32_t *)alloc_item(res, OR_PAIR_OFFSETS, (uint64_t)G + 1, 4);
    res->size[OR_PAIRS] = (uint64_t)nFoundPairs * 2;
    uint64_t written_total = 0;

    /* pairStore (:478-521). */
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : written_total) if (omp)
    for (long gp = 0; gp < G; ++gp) {
        const uint32_t event = (uint32_t)(gp / T), layerPair = (uint32_t)(gp % T);
        const pair_group *q = &pg[gp];
        const uint32_t end = q->layer2Offset + q->nHits2;
        for (uint32_t thread = 0; thread < nThreads; ++thread) {
            const uint64_t slot = (uint64_t)event * T * nThreads + (uint64_t)layerPair * nThreads + thread;
            uint32_t pos = prefixSum[slot];
            const uint32_t nextThread = prefixSum[slot + 1];
            for (uint32_t i = q->layer2Offset + thread; i < end; i += nThreads) {
                for (uint32_t j = 0; j < q->nHits1 && pos < nextThread; ++j) {
                    const uint32_t index = j * q->nHits2 + i - q->layer2Offset;
                    const int valid = (q->bits[index / 32] & (1u << (index % 32))) != 0;
                    if (valid) {
                        pairs[pos].x = j + q->offset;
                        pairs[pos].y = i;
                        valid_slot[pos] = 1;
                        written_total += 1;
                    }
                    pos += valid;
                }
            }
            if (thread == nThreads - 1) pairOffsets[(uint64_t)event * T + layerPair + 1] = nextThread;
        }
    }
    for (long gp = 0; gp < G; ++gp) free(pg[gp].bits);
    free(pg);
    free(prefixSum);
    res->stats[ORS_PAIR_SLOTS] = nFoundPairs;
    res->stats[ORS_PAIRS] = written_total;
}

/* ------------------------------------------------------------------------
 * Stage 2, sector variant: PairGeneratorSector (pairCount
 * PairGeneratorSector.h:43-147, pairStore :160-230, host
 * PairGeneratorSector.cpp:5-151).  No cut: every layer-2 hit in the block of
 * cells around the inner hit's own cell (pairSpreadZ rows, pairSpreadPhi
 * columns each side) is paired with it.  Threads stride the INNER hits.
 * ---------------------------------------------------------------------- */
static void pair_stage_sector(or_result *res, const trax_config *cfg, const trax_grid_cfg *g,
                              uint32_t nThreads, int omp)
{
    const uint32_t E = g->n_events, L = g->n_layers, Z = g->n_sectors_z, P = g->n_sectors_phi;
    const uint32_t T = cfg->n_layer_triplets;
    const uint32_t C = (Z + 1) * (P + 1);
    const float minZ = TRAX_MIN_Z, minPhi = TRAX_MIN_PHI;
    const float sectorSizeZ = trax_sector_size_z(Z), sectorSizePhi = trax_sector_size_phi(P);
    const uint32_t *grid = (const uint32_t *)res->data[OR_GRID];
    const float *hitGlobalY = (const float *)res->data[OR_SORTED_Y];
    const float *hitGlobalX = (const float *)res->data[OR_SORTED_X];
    const float *hitGlobalZ = (const float *)res->data[OR_SORTED_Z];
    const long G = (long)E * T;

    pair_group *pg = (pair_group *)calloc((size_t)(G ? G : 1), sizeof(pair_group));
    uint32_t *prefixSum = (uint32_t *)calloc((size_t)G * nThreads + 1, 4);

#pragma omp parallel for schedule(dynamic, 1) if (omp)
    for (long gp = 0; gp < G; ++gp) {
        const uint32_t event = (uint32_t)(gp / T), layerPair = (uint32_t)(gp % T);
        const trax_layer_triplet *lt = &cfg->triplets[layerPair];
        /* :63-67 inner layer range */
        const uint32_t *lGrid1 = grid + (uint64_t)event * L * C + (uint64_t)(lt->layer1 - 1) * C;
        const uint32_t layer1Offset = lGrid1[0];
        const uint32_t end = lGrid1[C - 1];
        /* :71-80 outer layer */
        const uint32_t *lGrid2 = grid + (uint64_t)event * L * C + (uint64_t)(lt->layer2 - 1) * C;
        const uint32_t nHits2 = lGrid2[C - 1] - lGrid2[0];
        const uint32_t offset = lGrid2[0];
        const uint32_t spreadZ = lt->pair_spread_z, spreadPhi = lt->pair_spread_phi;

        const uint32_t nHits1 = end - layer1Offset;
        const uint64_t nbits = (uint64_t)nHits1 * nHits2;
        pg[gp].bits = (uint32_t *)calloc((size_t)((nbits + 31) / 32 + 1), 4);
        pg[gp].nHits1 = nHits1; pg[gp].nHits2 = nHits2;
        pg[gp].offset = layer1Offset; pg[gp].layer2Offset = offset;

        for (uint32_t thread = 0; thread < nThreads; ++thread) {
            uint32_t nFound = 0;
            for (uint32_t i = layer1Offset + thread; i < end; i += nThreads) {
                /* :96-98.  zLowSector is unsigned: max(0u, zLowSector -
                 * spreadZ) is the plain difference, so an inner hit in a z
                 * sector below spreadZ wraps to a huge start and visits no
                 * row. */
                uint32_t zLowSector = trax_f2u(floorf((hitGlobalZ[i] - minZ) / sectorSizeZ));
                const uint32_t zh = zLowSector + spreadZ + 1u;
                const uint32_t zHighSector = zh < Z ? zh : Z;
                zLowSector = zLowSector - spreadZ;
                /* :102-110 */
                const float phi = trax_atan2f(hitGlobalY[i], hitGlobalX[i]);
                int32_t phiLowSector = trax_f2i(floorf((phi - minPhi) / sectorSizePhi) - (float)spreadPhi);
                uint32_t phiHighSector = (uint32_t)phiLowSector + 2u * spreadPhi + 1u;
                const int wrapAround = phiLowSector < 0 || phiHighSector > P + 1;
                phiLowSector = (int32_t)((uint32_t)phiLowSector + (uint32_t)(phiLowSector < 0) * P);
                phiHighSector -= (uint32_t)(phiHighSector > P + 1) * P;
                if (phiLowSector < 0 || (uint32_t)phiLowSector > P + 1 || phiHighSector > P + 1) {
                    /* only for 2*pairSpreadPhi + 1 > nSectorsPhi: the reference
                     * reads outside the grid row */
                    set_fault(res, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                    continue;
                }
                /* :114-142 */
                for (uint32_t zSector = zLowSector; zSector < zHighSector; ++zSector) {
                    const uint32_t zSectorStart = lGrid2[zSector * (P + 1)];
                    const uint32_t zSectorEnd = lGrid2[(zSector + 1) * (P + 1) - 1];
                    const uint32_t zSectorLength = zSectorEnd - zSectorStart;
                    uint32_t j = lGrid2[zSector * (P + 1) + (uint32_t)phiLowSector];
                    const uint32_t end2 = (uint32_t)wrapAround * zSectorEnd
                                        + lGrid2[zSector * (P + 1) + phiHighSector]
                                        - (uint32_t)wrapAround * zSectorStart;
                    for (; j < end2; ++j) {
                        ++nFound;
                        const uint32_t hit2 = j - (uint32_t)(j >= zSectorEnd) * zSectorLength - offset;
                        if (hit2 >= nHits2) { /* not reachable from a valid grid */
                            set_fault(res, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                            continue;
                        }
                        const uint64_t index = (uint64_t)(i - layer1Offset) * nHits2 + hit2;
                        pg[gp].bits[index / 32] |= (1u << (index % 32));
                    }
                }
            }
            prefixSum[(uint64_t)event * T * nThreads + (uint64_t)layerPair * nThreads + thread] = nFound;
        }
    }

    /* PairGeneratorSector.cpp:91-94 */
    or_prefix_sum(prefixSum, (uint32_t)((uint64_t)G * nThreads + 1), nThreads);
    const uint32_t nFoundPairs = prefixSum[(uint64_t)G * nThreads];

    u2 *pairs = (u2 *)alloc_item(res, OR_PAIRS, (uint64_t)nFoundPairs * 2, 4);
    uint8_t *valid_slot = (uint8_t *)alloc_item(res, OR_PAIR_VALID, nFoundPairs, 1);
    uint32_t *pairOffsets = (uint32_t *)alloc_item(res, OR_PAIR_OFFSETS, (uint64_t)G + 1, 4);
    uint64_t written_total = 0;

    /* pairStore (:176-229): per thread, its inner hits in stride order and
     * every outer hit in sorted order, while slots remain. */
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : written_total) if (omp)
    for (long gp = 0; gp < G; ++gp) {
        const uint32_t event = (uint32_t)(gp / T), layerPair = (uint32_t)(gp % T);
        const pair_group *q = &pg[gp];
        const uint32_t end = q->offset + q->nHits1;
        for (uint32_t thread = 0; thread < nThreads; ++thread) {
            const uint64_t slot = (uint64_t)event * T * nThreads + (uint64_t)layerPair * nThreads + thread;
            uint32_t pos = prefixSum[slot];
            const uint32_t nextThread = prefixSum[slot + 1];
            for (uint32_t i = q->offset + thread; i < end; i += nThreads) {
                for (uint32_t j = 0; j < q->nHits2 && pos < nextThread; ++j) {
                    const uint64_t index = (uint64_t)(i - q->offset) * q->nHits2 + j;
                    const int valid = (q->bits[index / 32] & (1u << (index % 32))) != 0;
                    if (valid) {
                        pairs[pos].x = i;
                        pairs[pos].y = q->layer2Offset + j;
                        valid_slot[pos] = 1;
                        written_total += 1;
                    }
                    pos += valid;
                }
            }
            if (thread == nThreads - 1) pairOffsets[(uint64_t)event * T + layerPair + 1] = nextThread;
        }
    }
    for (long gp = 0; gp < G; ++gp) free(pg[gp].bits);
    free(pg);
    free(prefixSum);
    res->stats[ORS_PAIR_SLOTS] = nFoundPairs;
    res->stats[ORS_PAIRS] = written_total;
}

/* ------------------------------------------------------------------------
 * Stage 3: TripletThetaPhiPredictor (predictCount :46-248, predictStore
 * :250-481, predictOffsetMonotonizeStore :483-497; host .cpp:10-131).
 * ---------------------------------------------------------------------- */
typedef struct {
    int ok;
    float zLow, zHigh, phiLow, phiHigh;
    uint32_t zLowSector, zHighSector, phiLowSector, phiHighSector;
    int wrapAround;
    const uint32_t *lGrid3;
} pred_window;

/* `store` selects predictStore's variants: rOrigin through sqrt(r)^2
 * (:326-327 vs :117-118) and zHigh padded by sigmaZ (:339 vs :130). */
static pred_window pred_window_for(const or_result *r, const trax_config *cfg,
                                   const trax_grid_cfg *g, float minRadiusCurvature,
                                   uint32_t firstHit, uint32_t secondHit, int store)
{
    pred_window w;
    memset(&w, 0, sizeof(w));
    const uint32_t L = g->n_layers, Z = g->n_sectors_z, P = g->n_sectors_phi;
    const uint32_t C = (Z + 1) * (P + 1);
    const float minZ = TRAX_MIN_Z, minPhi = TRAX_MIN_PHI;
    const float sectorSizeZ = trax_sector_size_z(Z), sectorSizePhi = trax_sector_size_phi(P);
    const float *X = (const float *)r->data[OR_SORTED_X];
    const float *Y = (const float *)r->data[OR_SORTED_Y];
    const float *Zc = (const float *)r->data[OR_SORTED_Z];
    const uint32_t *hitEvent = (const uint32_t *)r->data[OR_SORTED_EVENT];
    const uint32_t *hitLayer = (const uint32_t *)r->data[OR_SORTED_LAYER];
    const uint32_t *grid = (const uint32_t *)r->data[OR_GRID];

    const uint32_t event = hitEvent[firstHit];
    const uint32_t layerTriplet = hitLayer[firstHit] - 1;
    if (layerTriplet >= cfg->n_layer_triplets || event >= g->n_events) return w;
    const trax_layer_triplet *lt = &cfg->triplets[layerTriplet];
    const uint32_t layer = lt->layer3 - 1;
    w.lGrid3 = grid + (uint64_t)event * L * C + (uint64_t)layer * C;
    const float sigmaZ = lt->sigma_z;
    const float sigmaPhi = lt->sigma_phi;
    const float minLayerRadius = cfg->min_radius[layer];
    const float maxLayerRadius = cfg->max_radius[layer];

    const float p1x = X[firstHit], p1y = Y[firstHit], p1z = Zc[firstHit];
    const float p2x = X[secondHit], p2y = Y[secondHit], p2z = Zc[secondHit];
    /* :111-119 / :320-328 */
    float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
    tip2 *= tip2;
    tip2 /= ((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
    float rOrigin;
    if (!store) {
        rOrigin = p1x * p1x + p1y * p1y;
        rOrigin = sqrtf(rOrigin - tip2);
    } else {
        rOrigin = sqrtf(p1x * p1x + p1y * p1y);
        rOrigin = sqrtf(rOrigin * rOrigin - tip2);
    }
    const float cotTheta = (p2z - p1z) / (sqrtf(p2x * p2x + p2y * p2y - tip2) - rOrigin);
    /* :123-133 / :332-342 */
    float tmp = p1z + (sqrtf(maxLayerRadius * maxLayerRadius - tip2) - rOrigin) * cotTheta;
    float zLow = p1z + (sqrtf(minLayerRadius * minLayerRadius - tip2) - rOrigin) * cotTheta;
    float zHigh = (float)(tmp > zLow) * tmp + (float)(tmp < zLow) * zLow;
    zLow = (float)(tmp > zLow) * zLow + (float)(tmp < zLow) * tmp;
    zLow -= sigmaZ;
    zHigh += store ? sigmaZ : sigmaPhi;
    int32_t zl = trax_f2i(floorf((zLow - minZ) / sectorSizeZ));
    w.zLowSector = (uint32_t)(zl > 0 ? zl : 0);
    uint32_t zh = trax_f2u(floorf((zHigh - minZ) / sectorSizeZ)) + 1;
    w.zHighSector = zh < Z ? zh : Z;
    /* :138-166 / :347-375 */
    const float phi = trax_atan2f(p2y, p2x);
    tmp = trax_atan2f(p1y, p1x);
    float dPhi = phi - tmp;
    dPhi += (dPhi > TRAX_PI_F) ? -2 * TRAX_PI_F : (dPhi < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
    dPhi = fabsf(dPhi);
    const float dHits = sqrtf((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
    tmp = fabsf(trax_acosf(dHits / (2 * minRadiusCurvature)) - trax_acosf(maxLayerRadius / (2 * minRadiusCurvature)));
    float phiLow = fabsf(trax_acosf(dHits / (2 * minRadiusCurvature)) - trax_acosf(minLayerRadius / (2 * minRadiusCurvature)));
    dPhi = trax_maxf(dPhi, trax_maxf(tmp, phiLow));
    float phiHigh = phi + dPhi + sigmaPhi;
    phiLow = phi - dPhi - sigmaPhi;
    w.wrapAround = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
    phiLow -= (float)((phiLow > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiLow += (float)((phiLow < -TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh -= (float)((phiHigh > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh += (float)((phiHigh < -TRAX_PI_F) * 2) * TRAX_PI_F;
    w.phiLowSector = trax_f2u(floorf((phiLow - minPhi) / sectorSizePhi));
    uint32_t ph = trax_f2u(floorf((phiHigh - minPhi) / sectorSizePhi)) + 1;
    w.phiHighSector = ph < P ? ph : P;
    w.zLow = zLow; w.zHigh = zHigh; w.phiLow = phiLow; w.phiHigh = phiHigh;
    w.ok = w.phiLowSector <= P + 1 ? 1 : -1;
    return w;
}

/* Visits the window's candidates in the kernels' order (:170-233 /
 * :379-456).  Returns accepted visits; stores at most `cap` of them. */
static uint32_t pred_visit(const or_result *r, const trax_grid_cfg *g, const pred_window *w,
                           uint32_t gid, u2 *out, uint8_t *out_valid, uint32_t cap)
{
    const uint32_t P = g->n_sectors_phi;
    const float *X = (const float *)r->data[OR_SORTED_X];
    const float *Y = (const float *)r->data[OR_SORTED_Y];
    const float *Zc = (const float *)r->data[OR_SORTED_Z];
    const uint32_t *lGrid3 = w->lGrid3;
    uint32_t nFound = 0;
    for (uint32_t zSector = w->zLowSector; zSector < w->zHighSector; ++zSector) {
        const uint32_t zSectorStart = lGrid3[zSector * (P + 1)];
        const uint32_t zSectorEnd = lGrid3[(zSector + 1) * (P + 1)];
        const uint32_t zSectorLength = zSectorEnd - zSectorStart;
        uint32_t j = lGrid3[zSector * (P + 1) + w->phiLowSector];
        const uint32_t end2 = (uint32_t)w->wrapAround * zSectorEnd
                            + lGrid3[zSector * (P + 1) + w->phiHighSector]
                            - (uint32_t)w->wrapAround * zSectorStart;
        for (; j < end2; ++j) {
            const uint32_t index = j - (uint32_t)(j >= zSectorEnd) * zSectorLength;
            int valid = w->zLow <= Zc[index] && Zc[index] <= w->zHigh;
            const float actPhi = trax_atan2f(Y[index], X[index]);
            valid = valid * ((!w->wrapAround && (w->phiLow <= actPhi && actPhi <= w->phiHigh))
                      || (w->wrapAround && ((w->phiLow <= actPhi && actPhi <= TRAX_PI_F) || (-TRAX_PI_F <= actPhi && actPhi <= w->phiHigh))));
            if (valid && out && nFound < cap) {
                out[nFound].x = gid;
                out[nFound].y = index;
                out_valid[nFound] = 1;
            }
            nFound += valid;
        }
    }
    return nFound;
}

static void predict_stage(or_result *r, const trax_config *cfg, const trax_grid_cfg *g,
                          float minRadiusCurvature, uint32_t nThreads, int omp)
{
    const uint32_t E = g->n_events, T = cfg->n_layer_triplets;
    const u2 *pairs = (const u2 *)r->data[OR_PAIRS];
    const uint8_t *pair_valid = (const uint8_t *)r->data[OR_PAIR_VALID];
    const uint32_t *pairOffsets = (const uint32_t *)r->data[OR_PAIR_OFFSETS];
    const uint32_t nPairs = (uint32_t)r->size[OR_PAIR_VALID];
    uint32_t *prefixSum = (uint32_t *)calloc((size_t)nPairs + 1, 4);

    /* predictCount: one work-item per pair (:71-235). */
#pragma omp parallel for schedule(dynamic, 256) if (omp)
    for (long gid = 0; gid < (long)nPairs; ++gid) {
        if (!pair_valid[gid]) continue;
        pred_window w = pred_window_for(r, cfg, g, minRadiusCurvature, pairs[gid].x, pairs[gid].y, 0);
        if (w.ok == 0) { set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_BAD_TRIPLET_INDEX); continue; }
        if (w.ok < 0) { set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID); continue; }
        prefixSum[gid] = pred_visit(r, g, &w, (uint32_t)gid, NULL, NULL, 0);
    }
    or_prefix_sum(prefixSum, nPairs + 1, nThreads); /* .cpp:56-59 */
    const uint32_t nCand = prefixSum[nPairs];

    u2 *cands = (u2 *)alloc_item(r, OR_CANDS, (uint64_t)nCand * 2, 4);
    uint8_t *cvalid = (uint8_t *)alloc_item(r, OR_CAND_VALID, nCand, 1);
    uint32_t *off = (uint32_t *)alloc_item(r, OR_CAND_OFFSETS, (uint64_t)E * T + 1, 4);
    uint64_t stored = 0, truncated = 0;

    /* predictStore (:289-455): store window, truncated to the count. */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : stored, truncated) if (omp)
    for (long gid = 0; gid < (long)nPairs; ++gid) {
        if (!pair_valid[gid]) continue;
        const uint32_t pos = prefixSum[gid];
        const uint32_t nextThread = prefixSum[gid + 1];
        if (nextThread == pos) {
            /* The kernel stops at pos == nextThread; only the truncation
             * statistic needs the store window here. */
        }
        pred_window w = pred_window_for(r, cfg, g, minRadiusCurvature, pairs[gid].x, pairs[gid].y, 1);
        if (w.ok <= 0) continue;
        const uint32_t cap = nextThread - pos;
        const uint32_t acc = pred_visit(r, g, &w, (uint32_t)gid, cands + pos, cvalid + pos, cap);
        stored += acc < cap ? acc : cap;
        truncated += acc > cap ? acc - cap : 0;
    }

    /* Offsets (:459-469): the last pair of each (event, layer triplet)
     * writes prefixSum[gid+1]; groups are the pair slot ranges, which the
     * reference reads back through hitEvent/hitLayer of the first hit. */
    for (uint64_t gp = 0; gp < (uint64_t)E * T; ++gp) {
        const uint32_t a = pairOffsets[gp], b = pairOffsets[gp + 1];
        if (b > a) off[gp + 1] = prefixSum[b];
    }
    for (uint64_t i = 1; i <= (uint64_t)E * T; ++i) /* :483-497, sequential */
        if (off[i] == 0) off[i] = off[i - 1];
    free(prefixSum);
    r->stats[ORS_CAND_SLOTS] = nCand;
    r->stats[ORS_CANDS] = stored;
    r->stats[ORS_CAND_TRUNCATED] = truncated;
}

/* ------------------------------------------------------------------------
 * Stage 4: TripletThetaPhiFilter (filterCount :50-168, filterPopCount
 * :170-184, filterStore :186-252, filterOffsetStore :254-297,
 * filterOffsetMonotonizeStore :299-313; host .cpp:10-164).
 * ---------------------------------------------------------------------- */
static int filter_cut(const or_result *r, const trax_config *cfg, float minRadius,
                      uint32_t firstHit, uint32_t secondHit, uint32_t thirdHit)
{
    const float *X = (const float *)r->data[OR_SORTED_X];
    const float *Y = (const float *)r->data[OR_SORTED_Y];
    const float *Zc = (const float *)r->data[OR_SORTED_Z];
    const uint32_t *hitLayer = (const uint32_t *)r->data[OR_SORTED_LAYER];
    const uint32_t layerTriplet = hitLayer[firstHit] - 1;
    if (layerTriplet >= cfg->n_layer_triplets) return -1;
    const float dThetaCut = cfg->triplets[layerTriplet].dtheta_cut;
    const float dPhiCut = cfg->triplets[layerTriplet].dphi_cut;
    const float tipCut = cfg->triplets[layerTriplet].tip_cut;

    int valid = 1;
    /* :86-94 */
    float angle1 = trax_atan2f(sqrtf((X[secondHit] - X[firstHit]) * (X[secondHit] - X[firstHit])
                                     + (Y[secondHit] - Y[firstHit]) * (Y[secondHit] - Y[firstHit])),
                               (Zc[secondHit] - Zc[firstHit]));
    float angle2 = trax_atan2f(sqrtf((X[thirdHit] - X[secondHit]) * (X[thirdHit] - X[secondHit])
                                     + (Y[thirdHit] - Y[secondHit]) * (Y[thirdHit] - Y[secondHit])),
                               (Zc[thirdHit] - Zc[secondHit]));
    float delta = fabsf(angle2 / angle1);
    valid = valid * (1 - dThetaCut <= delta && delta <= 1 + dThetaCut);
    /* :97-103 */
    angle1 = trax_atan2f((Y[secondHit] - Y[firstHit]), (X[secondHit] - X[firstHit]));
    angle2 = trax_atan2f((Y[thirdHit] - Y[secondHit]), (X[thirdHit] - X[secondHit]));
    delta = angle2 - angle1;
    delta += (delta > TRAX_PI_F) ? -2 * TRAX_PI_F : (delta < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
    valid = valid * (fabsf(delta) <= dPhiCut);
    /* :107-147; normalize(v) = v / sqrt(dot(v, v)) */
    const float p1x = X[firstHit], p1y = Y[firstHit], p1z = X[firstHit] * X[firstHit] + Y[firstHit] * Y[firstHit];
    const float p2x = X[secondHit], p2y = Y[secondHit], p2z = X[secondHit] * X[secondHit] + Y[secondHit] * Y[secondHit];
    const float p3x = X[thirdHit], p3y = Y[thirdHit], p3z = X[thirdHit] * X[thirdHit] + Y[thirdHit] * Y[thirdHit];
    const float ax = p2x - p1x, ay = p2y - p1y, az = p2z - p1z;
    const float bx = p3x - p1x, by = p3y - p1y, bz = p3z - p1z;
    float nx = ay * bz - az * by;
    float ny = az * bx - ax * bz;
    float nz = ax * by - ay * bx;
    const float nlen = sqrtf(nx * nx + ny * ny + nz * nz);
    nx = nx / nlen; ny = ny / nlen; nz = nz / nlen;
    const float cOx = (-nx) / (2 * nz);
    const float cOy = (-ny) / (2 * nz);
    const float c = -(nx * p1x + ny * p1y + nz * p1z);
    const float cR = sqrtf((1 - nz * nz - 4 * c * nz) / (4 * nz * nz));
    float vx = -cOx, vy = -cOy;
    const float vlen = sqrtf(vx * vx + vy * vy);
    vx = vx / vlen; vy = vy / vlen;
    const float pCAx = cOx + cR * vx;
    const float pCAy = cOy + cR * vy;
    const float tip = pCAx * pCAx + pCAy * pCAy;
    valid = valid * (tip <= (tipCut * tipCut));
    valid = valid * (cR >= minRadius);
    return valid;
}

static uint32_t swar_popcount(uint32_t i) /* :178-181 */
{
    i = i - ((i >> 1) & 0x55555555);
    i = (i & 0x33333333) + ((i >> 2) & 0x33333333);
    return (((i + (i >> 4)) & 0x0F0F0F0F) * 0x01010101) >> 24;
}

static void filter_stage(or_result *r, const trax_config *cfg, const trax_grid_cfg *g,
                         float minRadiusCurvature, uint32_t nThreads, int omp)
{
    const uint32_t E = g->n_events, T = cfg->n_layer_triplets;
    const u2 *pairs = (const u2 *)r->data[OR_PAIRS];
    const u2 *trip = (const u2 *)r->data[OR_CANDS];
    const uint8_t *cvalid = (const uint8_t *)r->data[OR_CAND_VALID];
    const uint32_t nTriplets = (uint32_t)r->size[OR_CAND_VALID];
    const uint32_t *hitEvent = (const uint32_t *)r->data[OR_SORTED_EVENT];
    const uint32_t *hitLayer = (const uint32_t *)r->data[OR_SORTED_LAYER];
    const uint32_t nOracleCount = (nTriplets + 31) / 32;
    uint32_t *oracle = (uint32_t *)calloc((size_t)nOracleCount + 1, 4);
    uint8_t *flag = (uint8_t *)calloc((size_t)nTriplets + 1, 1);

#pragma omp parallel for schedule(dynamic, 1024) if (omp)
    for (long gid = 0; gid < (long)nTriplets; ++gid) {
        if (!cvalid[gid]) continue;
        const uint32_t firstHit = pairs[trip[gid].x].x;
        const uint32_t secondHit = pairs[trip[gid].x].y;
        const uint32_t thirdHit = trip[gid].y;
        int v = filter_cut(r, cfg, minRadiusCurvature, firstHit, secondHit, thirdHit);
        if (v < 0) { set_fault(r, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_BAD_TRIPLET_INDEX); v = 0; }
        flag[gid] = (uint8_t)v;
    }
    for (uint32_t gid = 0; gid < nTriplets; ++gid) /* atomic_or, :156 */
        oracle[gid / 32] |= ((uint32_t)flag[gid] << (gid % 32));
    free(flag);

    uint32_t *prefixSum = (uint32_t *)calloc((size_t)nOracleCount + 1, 4);
    for (uint32_t w = 0; w < nOracleCount; ++w) prefixSum[w] = swar_popcount(oracle[w]);
    or_prefix_sum(prefixSum, nOracleCount + 1, nThreads);
    const uint32_t nFound = prefixSum[nOracleCount];

    uint32_t *h1 = (uint32_t *)alloc_item(r, OR_TRK_H1, nFound, 4);
    uint32_t *h2 = (uint32_t *)alloc_item(r, OR_TRK_H2, nFound, 4);
    uint32_t *h3 = (uint32_t *)alloc_item(r, OR_TRK_H3, nFound, 4);
    uint32_t *off = (uint32_t *)alloc_item(r, OR_TRK_OFFSETS, (uint64_t)E * T + 1, 4);
    for (uint32_t w = 0; w < nOracleCount; ++w) { /* filterStore :203-246 */
        uint32_t pos = prefixSum[w];
        const uint32_t lOracle = oracle[w];
        for (uint32_t i = 0; i < 32; ++i) {
            const int valid = (lOracle & (1u << i)) != 0;
            if (valid) {
                h1[pos] = pairs[trip[w * 32 + i].x].x;
                h2[pos] = pairs[trip[w * 32 + i].x].y;
                h3[pos] = trip[w * 32 + i].y;
            }
            pos += valid;
        }
    }
    for (uint32_t gid = 0; gid < nFound; ++gid) { /* filterOffsetStore :270-292 */
        const uint32_t ev = hitEvent[h1[gid]];
        const uint32_t layerTriplet = hitLayer[h1[gid]] - 1;
        if (gid < nFound - 1) {
            const uint32_t nev = hitEvent[h1[gid + 1]];
            const uint32_t nlt = hitLayer[h1[gid + 1]] - 1;
            if (layerTriplet != nlt || ev != nev) off[(uint64_t)ev * T + layerTriplet + 1] = gid + 1;
        } else {
            off[(uint64_t)ev * T + layerTriplet + 1] = gid + 1;
        }
    }
    for (uint64_t i = 1; i <= (uint64_t)E * T; ++i) /* :309-312, sequential */
        if (off[i] == 0) off[i] = off[i - 1];
    free(prefixSum);
    free(oracle);
    r->stats[ORS_TRACKLETS] = nFound;
}

/* ------------------------------------------------------------------------
 * TripletConnectivity (TripletConnectivity.h:56-108, .cpp:21-71).
 * ---------------------------------------------------------------------- */
void or_connectivity(const uint32_t *b1, const uint32_t *b2, const uint32_t *b3,
                     const uint32_t *base_con, uint32_t n_base, const uint32_t *f1,
                     const uint32_t *f2, const uint32_t *f3, uint32_t *follow_con,
                     uint32_t n_follow, int iterate_backwards, int tight_packing)
{
    for (uint32_t gid = 0; gid < n_follow; ++gid) {
        for (uint32_t i = 0; i < n_base; ++i) {
            int connected;
            if (tight_packing) /* tripletConnectivityTight, :100-101 */
                connected = b2[i] == f1[gid] && b3[i] == f2[gid];
            else if (!iterate_backwards)
                connected = b3[i] == f1[gid];
            else
                connected = b1[i] == f3[gid];
            follow_con[gid] += (uint32_t)connected * ((base_con ? base_con[i] : 0u) + 1u);
        }
    }
}

void or_connectivity_literal_wide(const uint32_t *base_hit, const uint32_t *base_con,
                                  uint32_t n_base, const uint32_t *follow_hit,
                                  uint32_t *follow_con, uint32_t n_follow)
{
    /* :67-75; base_hit is read at the following index, so n_follow must not
     * exceed n_base (the reference reads past the base buffer otherwise) */
    for (uint32_t gid = 0; gid < n_follow && gid < n_base; ++gid)
        for (uint32_t i = 0; i < n_base; ++i) {
            const int connected = base_hit[gid] == follow_hit[i];
            follow_con[gid] += (uint32_t)connected * (base_con[i] + 1u);
        }
}

or_result *or_run(const trax_config *cfg, const trax_grid_cfg *grid, const float *x, const float *y,
                  const float *z, const uint32_t *layer, const uint32_t *det, const uint32_t *hitid,
                  const uint32_t *event, uint32_t n_hits, const uint32_t *event_offset,
                  const uint32_t *layer_nhits, const uint32_t *layer_offset, int n_stages,
                  uint32_t n_threads, int n_omp_threads)
{
    return or_run_ex(cfg, grid, x, y, z, layer, det, hitid, event, n_hits, event_offset,
                     layer_nhits, layer_offset, n_stages, n_threads, n_omp_threads,
                     OR_PAIRS_BEAMSPOT);
}

or_result *or_run_ex(const trax_config *cfg, const trax_grid_cfg *grid, const float *x,
                     const float *y, const float *z, const uint32_t *layer, const uint32_t *det,
                     const uint32_t *hitid, const uint32_t *event, uint32_t n_hits,
                     const uint32_t *event_offset, const uint32_t *layer_nhits,
                     const uint32_t *layer_offset, int n_stages, uint32_t n_threads,
                     int n_omp_threads, int pair_generator)
{
    or_result *r = (or_result *)calloc(1, sizeof(or_result));
    if (!r) return NULL;
    if (n_threads == 0) n_threads = 256;
    int omp = n_omp_threads > 1;
#ifdef _OPENMP
    if (omp) omp_set_num_threads(n_omp_threads);
#else
    omp = 0;
#endif
    const float rmin = or_min_radius_curvature(cfg->min_pt, cfg->bz);
    grid_stage(r, grid, x, y, z, layer, det, hitid, event, n_hits, event_offset, layer_nhits,
               layer_offset, n_threads, omp);
    if (n_stages >= 2) {
        if (pair_generator == OR_PAIRS_SECTOR)
            pair_stage_sector(r, cfg, grid, n_threads, omp);
        else
            pair_stage(r, cfg, grid, rmin, n_threads, omp);
    }
    if (n_stages >= 3) predict_stage(r, cfg, grid, rmin, n_threads, omp);
    if (n_stages >= 4) filter_stage(r, cfg, grid, rmin, n_threads, omp);
    r->size[OR_STATS] = OR_NSTATS;
    r->data[OR_STATS] = r->stats;
    return r;
}

uint64_t or_size(const or_result *r, int item)
{
    return (item >= 0 && item < OR_NITEMS) ? r->size[item] : 0;
}

const void *or_data(const or_result *r, int item)
{
    return (item >= 0 && item < OR_NITEMS) ? r->data[item] : NULL;
}

void or_free(or_result *r)
{
    if (!r) return;
    for (int i = 0; i < OR_NITEMS; ++i)
        if (i != OR_STATS) free(r->data[i]);
    free(r);
}

/* ------------------------------------------------------------------------
 * HitCollection::addEvent (HitCollection.cpp:20-149) for one decoded event.
 * ---------------------------------------------------------------------- */
typedef struct { uint32_t track, idx; } ae_hit;

static int ae_cmp_track(const void *a, const void *b)
{
    const ae_hit *x = (const ae_hit *)a, *y = (const ae_hit *)b;
    if (x->track != y->track) return x->track < y->track ? -1 : 1;
    return x->idx < y->idx ? -1 : x->idx > y->idx;
}

/* Stable sort by layer of one track's hits (insertion sort). */
static void ae_sort_layer(uint32_t *idx, uint32_t n, const uint32_t *layer)
{
    for (uint32_t i = 1; i < n; ++i) {
        const uint32_t v = idx[i];
        uint32_t j = i;
        while (j > 0 && layer[idx[j - 1]] > layer[v]) {
            idx[j] = idx[j - 1];
            --j;
        }
        idx[j] = v;
    }
}

uint32_t or_add_event(const uint32_t *layer, const uint32_t *track, const float *pt,
                      uint32_t first, uint32_t n, float min_pt, uint32_t max_layer,
                      uint32_t used_mask, int only_tracks, int32_t num_tracks,
                      uint32_t *out_idx, uint32_t *layer_nhits, uint32_t *trk,
                      uint32_t *n_trk)
{
    /* :37-48 allTracks[simTrackID] gets every hit passing the filters, in
     * file order; a std::map iterates the ids ascending */
    ae_hit *h = (ae_hit *)malloc((size_t)(n ? n : 1) * sizeof(ae_hit));
    uint32_t nk = 0;
    for (uint32_t i = first; i < first + n; ++i) {
        if (only_tracks && track[i] == 0) continue;
        if (pt[i] < min_pt) continue;
        h[nk].track = track[i];
        h[nk].idx = i;
        ++nk;
    }
    qsort(h, nk, sizeof(ae_hit), ae_cmp_track);
    uint32_t *sorted = (uint32_t *)malloc((size_t)(nk ? nk : 1) * 4);
    for (uint32_t i = 0; i < nk; ++i) sorted[i] = h[i].idx;

    /* layers[l]: bucket lists; built as (track start, count, findable)
     * records replayed below in the reference's push order */
    uint32_t *bucket_of = (uint32_t *)malloc((size_t)(nk ? nk : 1) * 4); /* 0 none, 1 early, 2 late */
    memset(bucket_of, 0, (size_t)(nk ? nk : 1) * 4);
    uint32_t nf = 0;
    int foundTracks = 0;
    uint32_t b = 0;
    while (b < nk && foundTracks != num_tracks) {   /* :61 */
        uint32_t e = b;
        while (e < nk && h[e].track == h[b].track) ++e;
        uint32_t *t = sorted + b;
        const uint32_t cnt = e - b;
        ae_sort_layer(t, cnt, layer); /* :51-56 */
        if (!(only_tracks && h[b].track == 0)) {
            uint32_t cov = 0; /* :66-78 */
            for (uint32_t k = 0; k < cnt; ++k)
                if (layer[t[k]] >= 1 && layer[t[k]] <= max_layer) cov |= 1u << (layer[t[k]] - 1);
            const int missingHits = (cov & used_mask) != used_mask;
            if (!(pt[t[0]] < min_pt)) { /* :81-82 */
                for (uint32_t k = 0; k < cnt; ++k) /* :85-90 */
                    if (!missingHits) bucket_of[b + k] = 2;
                    else if (!only_tracks) bucket_of[b + k] = 1;
                if (!missingHits) {
                    if (trk) {
                        trk[4 * nf + 0] = h[b].track;
                        trk[4 * nf + 1] = t[0];
                        trk[4 * nf + 2] = t[cnt / 2];
                        trk[4 * nf + 3] = t[cnt - 1];
                    }
                    ++nf;
                    ++foundTracks;
                }
            }
        }
        b = e;
    }
    /* :96-146: per layer, the early (non-findable) hits in loop order, then
     * the findable tracks' hits with layer <= maxLayer */
    uint32_t w = 0;
    for (uint32_t l = 1; l <= max_layer; ++l) {
        const uint32_t start = w;
        for (int pass = 1; pass <= 2; ++pass)
            for (uint32_t k = 0; k < nk; ++k)
                if (bucket_of[k] == (uint32_t)pass && layer[sorted[k]] == l) out_idx[w++] = sorted[k];
        layer_nhits[l - 1] = w - start;
    }
    if (n_trk) *n_trk = nf;
    free(bucket_of);
    free(sorted);
    free(h);
    return w;
}

/* ------------------------------------------------------------------------
 * PhysicsRecord::fillData (PhysicsRecord.cpp:81-218) per (event, layer
 * triplet), tracklet by tracklet.
 * ---------------------------------------------------------------------- */
/* PhysicsRecord::getEta(inner, outer), PhysicsRecord.h:147-155 */
static double ph_eta(float x1, float y1, float z1, float x3, float y3, float z3)
{
    const double px = (double)(x3 - x1), py = (double)(y3 - y1), pz = (double)(z3 - z1);
    const double t = pz / sqrt(px * px + py * py);
    return trax_asinh_d(t);
}

/* getPt(getCircleParams(p1, p2, p3)), PhysicsRecord.cpp:41-79 and
 * PhysicsRecord.h:161-167 */
static double ph_pt(float x1, float y1, float x2, float y2, float x3, float y3)
{
    const double p1[3] = {x1, y1, (double)(x1 * x1 + y1 * y1)};
    const double p2[3] = {x2, y2, (double)(x2 * x2 + y2 * y2)};
    const double p3[3] = {x3, y3, (double)(x3 * x3 + y3 * y3)};
    const double a[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const double b[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const double value = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= value;
    n[1] /= value;
    n[2] /= value;
    const double c = -(n[0] * p1[0] + n[1] * p1[1] + n[2] * p1[2]);
    const double radius = sqrt((1 - n[2] * n[2] - 4 * c * n[2]) / (4 * n[2] * n[2]));
    const double Q = 1.602177E-19, BZ = 3.8112, GEV_C = 5.344286E-19;
    return Q * BZ * (radius * 1E-2) / GEV_C;
}

void or_physics(const uint32_t *hid, const float *x, const float *y, const float *z,
                const uint32_t *h1, const uint32_t *h2, const uint32_t *h3, const uint32_t *toff,
                uint32_t n_events, uint32_t n_lt, const uint32_t *mc_id, const uint32_t *mc_in,
                const uint32_t *mc_mid, const uint32_t *mc_out, const uint32_t *mc_off,
                const float *rx, const float *ry, const float *rz, uint32_t *counts,
                uint8_t *cat, double *eta_bin, double *pt_bin, uint8_t *missed,
                double *miss_eta_bin, double *miss_pt_bin)
{
    const uint32_t M = mc_off[n_events];
    uint8_t *found = (uint8_t *)malloc(M ? M : 1);
    for (uint32_t e = 0; e < n_events; ++e)
        for (uint32_t lt = 0; lt < n_lt; ++lt) {
            const uint32_t g = e * n_lt + lt;
            uint32_t *c = counts + (size_t)g * 7;
            memset(c, 0, 7 * 4);
            memset(found, 0, M ? M : 1);
            for (uint32_t i = toff[g]; i < toff[g + 1]; ++i) { /* :97-174 */
                const uint32_t a = h1[i], b = h2[i], d = h3[i];
                eta_bin[i] = floor(ph_eta(x[a], y[a], z[a], x[d], y[d], z[d]) / 0.1);
                pt_bin[i] = floor(ph_pt(x[a], y[a], x[b], y[b], x[d], y[d]) / 0.1);
                if (hid[a] == hid[b] && hid[a] == hid[d]) {
                    uint32_t k = mc_off[e + 1];
                    for (uint32_t j = mc_off[e]; j < mc_off[e + 1]; ++j)
                        if (mc_id[j] == hid[a]) { k = j; break; }
                    if (k < mc_off[e + 1]) {
                        if (!found[k]) { found[k] = 1; cat[i] = 0; c[1]++; }
                        else { cat[i] = 1; c[2]++; }
                    } else {
                        cat[i] = 3; c[4]++;
                    }
                } else {
                    cat[i] = 2; c[3]++;
                }
                c[0]++;
            }
            for (uint32_t k = mc_off[e]; k < mc_off[e + 1]; ++k) { /* :179-202 */
                const size_t q = (size_t)lt * M + k;
                c[6]++;
                missed[q] = !found[k];
                miss_eta_bin[q] = miss_pt_bin[q] = 0.0;
                if (!found[k]) {
                    c[5]++;
                    const uint32_t a = mc_in[k], m = mc_mid[k], d = mc_out[k];
                    miss_eta_bin[q] = floor(ph_eta(rx[a], ry[a], rz[a], rx[d], ry[d], rz[d]) / 0.1);
                    miss_pt_bin[q] = floor(ph_pt(rx[a], ry[a], rx[m], ry[m], rx[d], ry[d]) / 0.1);
                }
            }
        }
    free(found);
}

double or_asinh(double t) { return trax_asinh_d(t); }
