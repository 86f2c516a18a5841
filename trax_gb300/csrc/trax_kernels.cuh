/*
 * trax_kernels.cuh -- sm_103a kernels of the triplet-seeding path.
 *
 * Layout in HBM (all SoA, uint32 / float32):
 *   hits (input)      x y z layer detector_id hit_id event      [N]
 *   sorted hits       x y z phi layer detector_id hit_id event orig [N]
 *   grid              [E][L][(Z+1)(P+1)] global start of each cell
 *   outer slots       (outer hit, group) per (event, layer triplet) layer2 hit
 *   pairs             uint2 (inner, outer)                         [M]
 *   candidates        uint2 (pair index, hit3)                     [K]
 *   tracklets         hit1 hit2 hit3                               [R]
 *
 * Every kernel is persistent (grid = a multiple of the SM count) and reads
 * its problem size from device memory, so one launch sequence serves any
 * batch up to the reserved capacity and can be captured in a CUDA graph.
 *
 * FP32 arithmetic mirrors the reference kernels operation by operation and
 * is compiled with -fmad=false (see trax_math.h).
 */
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "trax_math.h"
#include "../../include/trax.h"

namespace trax {

constexpr int kMaxLT = TRAX_MAX_LAYER_TRIPLETS;
constexpr int kMaxLayers = TRAX_MAX_LAYERS;
constexpr uint32_t kFull = 0xffffffffu;
constexpr int kPairSave = 8;  /* ballot chunks a pair-stage item keeps for its store */
constexpr int kFusedThreads = 256;  /* threads per block of the tiled pair / predict kernels */

/* Per-run constants, passed by value to every kernel. */
struct KParams {
    uint32_t n_layers, nz, nphi, C, n_lt;
    float sz_z, sz_phi, rmin_curv;
    float inv_sz_z, inv_sz_phi;  /* 1.0f / sz_*: trax_floor_div */
    uint32_t l1[kMaxLT], l2[kMaxLT], l3[kMaxLT];
    float dtheta[kMaxLT], sigma_z[kMaxLT], dphi[kMaxLT], sigma_phi[kMaxLT];
    float tip[kMaxLT], z0[kMaxLT];
    /* outward-rounded tan(dphi -/+ margin) of trax_dphi_screen; thi < 0: screen off */
    float dphi_tlo[kMaxLT], dphi_thi[kMaxLT];
    uint32_t spread_z[kMaxLT], spread_phi[kMaxLT];
    float rmin[kMaxLayers], rmax[kMaxLayers];
    /* acos(r / (2 * minRadiusCurvature)) of each layer's min / max radius:
     * loop invariants of the phi windows, evaluated once on the host with the
     * same trax_acosf (host and device agree bit for bit) */
    float acos_rmin[kMaxLayers], acos_rmax[kMaxLayers];
    uint32_t run_walk, zi_min;   /* candidate-walk tuning, see k_zindex */
    uint32_t pair_record;        /* pair stage replays its count ballots (trax_tuning) */
};

/* Device-side sizes, counters and status of one pipeline run. */
struct DevState {
    uint32_t n_events;
    uint32_t n_hits;
    uint32_t n_outer;        /* outer slots (sum of layer2 hits over groups) */
    uint32_t n_pairs;
    uint32_t n_cands;
    uint32_t n_trk;
    uint32_t status;
    uint32_t detail;
    unsigned long long pair_slots;
    unsigned long long cand_slots;
    unsigned long long cand_truncated;
    uint32_t tile_ctr[4];    /* decoupled look-back tile tickets; [0] also the count passes' work tickets */
    uint32_t aux_n;          /* element count of a standalone prefix sum */
    uint32_t n_prec;         /* accepts the prediction count staged for the store pass */
    uint32_t n_pwalk;        /* prediction store records that walk (after them) */
    uint32_t n_ptile;        /* 32-pair tiles of the prediction count pass */
    uint32_t n_ftile;        /* 32-candidate words of the filter's accept mask */
    uint32_t gb_next;        /* grid build: the next segment a CTA takes */
    uint32_t spin_limit;     /* look-back polls before a wait gives up; 0 = kSpinLimit */
};

struct SortedCols {
    /* x, y, z, phi, det and hitid are null in the batched chain, which reads
     * the packed columns and never returns the sorted hits */
    float *x, *y, *z, *phi;
    uint32_t *layer, *det, *hitid, *event, *orig;
    float2 *zphi;  /* (z, phi) packed for the candidate loops; may be null */
    uint16_t *zh;  /* z rounded to half precision (bits), the candidate screen;
                    * null exactly when zphi is; 8 readable slots past the end */
    float4 *xyzp;  /* (x, y, z, phi) of each hit, one load for the window and
                    * cut arithmetic; null exactly when zphi is */
};

struct InCols {
    const float *x, *y, *z;
    const uint32_t *layer, *det, *hitid, *event;
};

__device__ __forceinline__ void set_fault(DevState *st, uint32_t status, uint32_t detail)
{
    if (atomicCAS(&st->status, 0u, status) == 0u) atomicExch(&st->detail, detail);
}

/* A hint to bring the 128-byte line holding `a` into L2; `a` must lie inside
 * an allocation. */
__device__ __forceinline__ void prefetch_l2(const void *a)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" : : "l"(p), "l"(v) : "memory");
}

/* ------------------------------------------------------------------------
 * Block-wide exclusive scan of one value per thread (blockDim <= 1024).
 * ---------------------------------------------------------------------- */
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp,
                                                         uint32_t *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        uint32_t t = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, t, d);
            if (lane >= d) t += y;
        }
        if (lane < nw) s_warp[lane] = t - w;
        if (lane == 31) s_warp[32] = t;
    }
    __syncthreads();
    const uint32_t r = s_warp[wid] + x - v;
    if (total) *total = s_warp[32];
    __syncthreads();
    return r;
}

/* ------------------------------------------------------------------------
 * Decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix Scan
 * with Decoupled Look-back", 2016).  Tile status words pack a 2-bit flag
 * (1 aggregate, 2 inclusive prefix) above a 32-bit value.  Waits are
 * bounded: after kSpinLimit polls (DevState::spin_limit when set) the tile
 * records TRAX_ERR_TIMEOUT and treats the missing predecessor as 0, so the
 * kernel always terminates.
 * ---------------------------------------------------------------------- */
constexpr unsigned long long kFlagAgg = 1ull << 32;
constexpr unsigned long long kFlagInc = 2ull << 32;
constexpr uint32_t kSpinLimit = 1u << 22;

/* Warp-wide decoupled look-back for a tile: lane i inspects predecessor
 * tile - 1 - i, so 32 predecessors are examined per poll.  The prefix is the
 * sum of the aggregates up to and including the nearest inclusive prefix.
 * A predecessor that shows nothing for kSpinLimit polls records
 * TRAX_ERR_TIMEOUT and ends the wait. */
__device__ __forceinline__ uint32_t warp_lookback(unsigned long long *status, uint32_t tile,
                                                  DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t prefix = 0;
    int64_t base = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (base >= 0) {
        const int64_t k = base - lane;
        unsigned long long s = k >= 0 ? ld_relaxed64(status + k) : (kFlagInc | 0ull);
        const unsigned long long flag = s & (3ull << 32);
        const uint32_t inc = __ballot_sync(kFull, flag == kFlagInc);
        const uint32_t zero = __ballot_sync(kFull, flag == 0);
        const uint32_t first_inc = inc ? (uint32_t)(__ffs(inc) - 1) : 32u;
        const uint32_t upto = first_inc < 32 ? ((first_inc == 31) ? kFull : ((2u << first_inc) - 1u)) : kFull;
        if (zero & upto) {
            if (++spins > (st->spin_limit ? st->spin_limit : kSpinLimit)) {
                if (lane == 0) set_fault(st, TRAX_ERR_TIMEOUT, TRAX_DETAIL_SCAN_TIMEOUT);
                break;
            }
            __nanosleep(32);
            continue;
        }
        uint32_t v = ((upto >> lane) & 1u) ? (uint32_t)s : 0u;
#pragma unroll
        for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
        prefix += v;
        if (first_inc < 32) break;
        base -= 32;
    }
    return prefix;
}

/* Warp-sized tile scan: exclusive prefix of v within the warp, the tile's
 * aggregate published and looked back; returns the global exclusive position
 * and (lane-uniform) the inclusive end of the tile. */
__device__ __forceinline__ uint32_t warp_tile_position(uint32_t v, uint32_t tile,
                                                       unsigned long long *status,
                                                       DevState *st, uint32_t *tile_end)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, d);
        if (lane >= (uint32_t)d) x += y;
    }
    const uint32_t agg = __shfl_sync(kFull, x, 31);
    uint32_t prefix = 0;
    if (tile == 0) {
        if (lane == 0) st_relaxed64(status, kFlagInc | agg);
    } else {
        if (lane == 0) st_relaxed64(status + tile, kFlagAgg | agg);
        prefix = warp_lookback(status, tile, st);
        if (lane == 0) st_relaxed64(status + tile, kFlagInc | (uint32_t)(prefix + agg));
    }
    *tile_end = prefix + agg;
    return prefix + x - v;
}

/* Exclusive scan of in[0..n) into out[0..n) (in place allowed); the total
 * goes to *total_out when given. */
template <int ITEMS>
__global__ void __launch_bounds__(256) k_scan(const uint32_t *in, uint32_t *out,
                                              const uint32_t *n_ptr, uint32_t n_cap,
                                              uint32_t *total_out, int ctr_slot,
                                              unsigned long long *status, DevState *st)
{
    uint32_t n = *n_ptr;
    if (n > n_cap) n = n_cap;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && total_out) *total_out = 0;
        return;
    }
    /* full tiles of 16-byte aligned arrays move 4 elements per access */
    const bool vec = ITEMS % 4 == 0 && ((reinterpret_cast<uintptr_t>(in) |
                                         reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_prefix;
    const uint32_t tileItems = blockDim.x * ITEMS;
    const uint32_t ntiles = (n + tileItems - 1) / tileItems;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&st->tile_ctr[ctr_slot], 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * tileItems + threadIdx.x * ITEMS;
        const bool full = vec && (tile + 1) * tileItems <= n;
        uint32_t v[ITEMS];
        if (full) {
#pragma unroll
            for (int k = 0; k < ITEMS; k += 4) {
                const uint4 q = *reinterpret_cast<const uint4 *>(in + base + k);
                v[k] = q.x; v[k + 1] = q.y; v[k + 2] = q.z; v[k + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) v[k] = (base + k < n) ? in[base + k] : 0u;
        }
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) sum += v[k];
        uint32_t agg;
        const uint32_t excl = block_exclusive_scan(sum, s_warp, &agg);
        if (threadIdx.x < 32) {
            /* warp 0 looks back over 32 predecessors per poll */
            uint32_t prefix = 0;
            if (tile == 0) {
                if (threadIdx.x == 0) st_relaxed64(status, kFlagInc | agg);
            } else {
                if (threadIdx.x == 0) st_relaxed64(status + tile, kFlagAgg | agg);
                prefix = warp_lookback(status, tile, st);
                if (threadIdx.x == 0) st_relaxed64(status + tile, kFlagInc | (uint32_t)(prefix + agg));
            }
            if (threadIdx.x == 0) {
                s_prefix = prefix;
                if (tile == ntiles - 1 && total_out) *total_out = prefix + agg;
            }
        }
        __syncthreads();
        uint32_t run = s_prefix + excl;
        uint32_t o[ITEMS];
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            o[k] = run;
            run += v[k];
        }
        if (full) {
#pragma unroll
            for (int k = 0; k < ITEMS; k += 4)
                *reinterpret_cast<uint4 *>(out + base + k) = make_uint4(o[k], o[k + 1], o[k + 2], o[k + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < ITEMS; ++k)
                if (base + k < n) out[base + k] = o[k];
        }
        __syncthreads();
    }
}

/* ------------------------------------------------------------------------
 * Stage 1: grid build.  One CTA per (event, layer) segment (persistent
 * CTAs taking segments from a counter).  Counting sort into (z, phi)
 * cells, stable within a cell:
 *   pass 1  each warp owns a contiguous sub-range of the segment and counts
 *           its cells (warp match + one shared add per distinct cell);
 *   pass 2  per cell, exclusive prefix over warps and an exclusive scan over
 *           cells give every warp's write cursor; the grid row is written;
 *   pass 3  each warp re-walks its sub-range in order and scatters the hit
 *           columns at cursor + rank-in-warp.
 * The segment's first sorted position equals its first input position
 * (the input is event/layer bucketed), so no global scan is needed.
 * Shared memory: (W + 1) * C uint32.
 * ---------------------------------------------------------------------- */
__device__ __forceinline__ uint32_t hit_cell(const KParams &kp, float x, float y, float z,
                                             float *phi_out, bool *bad)
{
    uint32_t zs = trax_f2u(trax_floor_div(z - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z));
    const float phi = trax_atan2f(y, x);
    uint32_t ps = trax_f2u(trax_floor_div(phi - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi));
    *bad = false;
    if (zs > kp.nz) { zs = kp.nz; *bad = true; }
    if (ps > kp.nphi) { ps = kp.nphi; *bad = true; }
    *phi_out = phi;
    return zs * (kp.nphi + 1) + ps;
}

constexpr int kGridItems = 4;        /* hits per lane held in registers across passes */
constexpr int kGridItemsBanded = 4;  /* the same in the banded instance */

/*
 * One CTA per (event, layer) segment; W warps own contiguous sub-ranges.
 *   pass 1  cell of every hit (one atan2), per-warp cell counts via
 *           __match_any_sync into shared memory;
 *   pass 2  prefix over warps per cell, block scan over cells -> the grid;
 *   pass 3  each hit's sorted position: segments of at most `stage` hits
 *           record the inverse permutation (and phi) in shared memory,
 *   pass 4  and write every column out coalesced, reading the inputs
 *           gathered from inside the segment (L1/L2 resident).
 * Larger segments scatter each column directly (4-byte stores to random
 * positions: one L2 sector per store).  Within a cell, hits keep input order.
 *
 * The per-warp cell tables hold Ct cells.  When the grid has more (fine
 * grids: 64 x 128 bins are 8385 cells per layer), passes 1-3 run per band of
 * Ct / (P + 1) z rows, over the rows the segment's hits occupy (pass 0 finds
 * them; a band covers the whole occupied range in one go for hits within a
 * few z rows, as barrel layers give), and the grid rows outside that range
 * get the segment's start or end.  Cells are row-major, so a band's hits are
 * one contiguous part of the sorted segment.  Block-wide bands visit every
 * hit once per band; staged segments whose cells sit in the scratch column
 * (dense layers on fine grids) instead bucket their hits by band once and
 * let each warp sort whole bands (the warp bands below).
 * Dynamic shared memory: (W + 1) * Ct + 2 * stage words.  BANDED is Ct < C
 * (the instance with bands has 64 registers, the other 48).
 */
template <bool BANDED>
__global__ void __maxnreg__(BANDED ? 64 : 48) k_grid_build(KParams kp, InCols in, SortedCols out,
                                                           const uint32_t *seg_start,
                                                           const uint32_t *seg_n, uint32_t *grid,
                                                           uint32_t stage, uint32_t Ct,
                                                           uint2 *cscr, DevState *st)
{
    constexpr int kItems = BANDED ? kGridItemsBanded : kGridItems;
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_warp[33];
    const uint32_t C = kp.C, P1 = kp.nphi + 1;
    const int W = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t *s_cnt = smem;                 /* [W][Ct] */
    uint32_t *s_tot = smem + W * Ct;        /* [Ct] */
    uint32_t *s_src = s_tot + Ct;           /* [stage] segment-relative input index */
    float *s_phi = (float *)(s_src + stage);  /* [stage] */
    const uint32_t nseg = st->n_events * kp.n_layers;
    const uint32_t lt_mask = lanemask_lt();
    /* BANDED: the grid's Z + 1 rows do not fit one table (Ct < C) */
    const uint32_t R = BANDED ? Ct / P1 : kp.nz + 1;  /* z rows per band, >= 1 */
    const bool banded = BANDED;

    /* each CTA takes its next segment from a counter as it finishes one:
     * the layers' segment sizes differ, and a fixed stride by the grid size
     * would pin every CTA to one layer (the grid is a multiple of the layer
     * count).  Every thread reads s_seg (and the row range) before the
     * segment's last barrier, after which thread 0 may overwrite them. */
    __shared__ uint32_t s_seg, s_rlo, s_rhi;
    for (;;) {
        if (threadIdx.x == 0) {
            s_seg = atomicAdd(&st->gb_next, 1u);
            s_rlo = 0xffffffffu;
            s_rhi = 0u;
        }
        __syncthreads();
        const uint32_t seg = s_seg;
        if (seg >= nseg) break;  /* block-uniform */
        const uint32_t e = seg / kp.n_layers, l = seg % kp.n_layers;
        const uint32_t start = seg_start[seg], n = seg_n[seg];
        const uint32_t chunk = (n + W - 1) / W;
        const uint32_t lo = min(n, w * chunk), hi = min(n, lo + chunk);
        /* chunks of at most kItems * 32 hits keep cell, phi and peer mask
         * in registers from pass 1 to pass 3 */
        const bool cached = chunk <= (uint32_t)(kItems * 32);
        const bool staged = n <= stage;
        uint32_t *gseg = grid + (size_t)seg * C;

        /* pass 0: with bands, segments too large for the registers compute
         * every hit's cell and phi once, into cscr (read back by the same
         * thread in passes 1 and 3 of every band, instead of an atan2 per
         * hit per band), and the z rows the segment's hits occupy */
        const bool scratch = BANDED && !cached && cscr != nullptr;
        if (scratch) {
            bool anybad = false;
            for (uint32_t i = lo + lane; i < hi; i += 32) {
                const uint32_t h = start + i;
                float phi;
                bool bad;
                const uint32_t cell = hit_cell(kp, in.x[h], in.y[h], in.z[h], &phi, &bad);
                anybad |= bad;
                cscr[h] = make_uint2(cell, __float_as_uint(phi));
            }
            if (anybad) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_OUTSIDE_GRID);
        }
        uint32_t rlo = 0, rhi = kp.nz;
        if (banded) {
            uint32_t mn = 0xffffffffu, mx = 0u;
            if (scratch) {
                for (uint32_t i = lo + lane; i < hi; i += 32) {
                    const uint32_t zs = cscr[start + i].x / P1;
                    mn = min(mn, zs);
                    mx = max(mx, zs);
                }
            } else {
                for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                    uint32_t zs = trax_f2u(trax_floor_div(in.z[start + i] - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z));
                    if (zs > kp.nz) zs = kp.nz;
                    mn = min(mn, zs);
                    mx = max(mx, zs);
                }
            }
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                mn = min(mn, __shfl_xor_sync(kFull, mn, d));
                mx = max(mx, __shfl_xor_sync(kFull, mx, d));
            }
            if (lane == 0) {
                atomicMin(&s_rlo, mn);
                atomicMax(&s_rhi, mx);
            }
            __syncthreads();
            rlo = s_rlo;
            rhi = s_rhi;
            if (rlo > rhi) rlo = rhi = 0;  /* no hits */
            /* rows below the occupied range start at the segment start */
            for (uint32_t c = threadIdx.x; c < rlo * P1; c += blockDim.x) gseg[c] = start;
            for (uint32_t c = (rhi + 1) * P1 + threadIdx.x; c < C; c += blockDim.x) gseg[c] = start + n;
        }

        float cphi[kItems];
        uint32_t ccell[kItems], cpeers[kItems];
        if (cached) {
            float cx[kItems], cy[kItems], cz[kItems];
#pragma unroll
            for (int j = 0; j < kItems; ++j) {
                const uint32_t i = lo + j * 32 + lane;
                if (i < hi) {
                    const uint32_t h = start + i;
                    cx[j] = in.x[h]; cy[j] = in.y[h]; cz[j] = in.z[h];
                }
            }
            /* independent atan2 chains first (ILP), then the warp votes */
            bool anybad = false;
#pragma unroll
            for (int j = 0; j < kItems; ++j) {
                bool bad = false;
                ccell[j] = 0;
                cphi[j] = 0.f;
                if (lo + j * 32 + lane < hi) ccell[j] = hit_cell(kp, cx[j], cy[j], cz[j], &cphi[j], &bad);
                anybad |= bad;
            }
            if (anybad) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_OUTSIDE_GRID);
            /* the peers of a hit (same cell, same warp step) do not depend on
             * the band: with bands they are found once, here */
            if (BANDED) {
#pragma unroll
                for (int j = 0; j < kItems; ++j) {
                    cpeers[j] = 0;
                    const uint32_t b = lo + j * 32;
                    if (b < hi) {  /* warp-uniform */
                        const bool valid = b + lane < hi;
                        const uint32_t act = __ballot_sync(kFull, valid);
                        if (valid) cpeers[j] = __match_any_sync(act, ccell[j]);
                    }
                }
            }
        }

        /* Warp bands (BANDED, staged, cells in the scratch column): the hits
         * are bucketed once by band of R2 z rows (a stable counting sort over
         * (band, warp)), and each warp then sorts whole bands on its own:
         * count the band's hits per cell in a warp-private table, scan it,
         * write the band's grid rows and place its hits -- every hit is
         * visited a fixed number of times and no band waits for a block
         * barrier.  The band list (one word per hit) takes the last `stage`
         * words of the per-warp tables, and each warp's table the R2 rows
         * that fit in front of it.  Otherwise the block-wide bands below. */
        const uint32_t tab_words = BANDED ? ((uint32_t)W * Ct > stage ? (uint32_t)W * Ct - stage : 0u) : 0u;
        const uint32_t R2 = tab_words / ((uint32_t)W * P1);
        const uint32_t nb2 = R2 ? (rhi - rlo) / R2 + 1 : 0u;
        const bool wband = BANDED && scratch && staged && R2 >= 1 &&
                           nb2 * (uint32_t)W <= tab_words && nb2 + 1 <= Ct;
        if (wband) {
            uint32_t *s_bc = s_cnt;                       /* [nb2][W] hits per band and warp */
            uint32_t *s_bstart = s_tot;                   /* [nb2 + 1] first position of each band */
            uint32_t *s_blist = s_cnt + (uint32_t)W * Ct - stage;  /* [n] hits in band order */
            const uint32_t m = nb2 * (uint32_t)W;
            for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) s_bc[k] = 0;
            __syncthreads();
            /* bucket counts per (band, warp) over each warp's sub-range */
            for (uint32_t b = lo; b < hi; b += 32) {  /* warp-uniform */
                const uint32_t i = b + lane;
                const bool valid = i < hi;
                const uint32_t band = valid ? (cscr[start + i].x / P1 - rlo) / R2 : 0u;
                const uint32_t act = __ballot_sync(kFull, valid);
                if (valid) {
                    const uint32_t peers = __match_any_sync(act, band);
                    if (lane == __ffs(peers) - 1) s_bc[band * W + w] += __popc(peers);
                }
                __syncwarp();
            }
            __syncthreads();
            {
                const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
                const uint32_t c0 = min(m, threadIdx.x * per), c1 = min(m, c0 + per);
                uint32_t sum = 0, total;
                for (uint32_t c = c0; c < c1; ++c) sum += s_bc[c];
                uint32_t run = block_exclusive_scan(sum, s_warp, &total);
                for (uint32_t c = c0; c < c1; ++c) {
                    const uint32_t t = s_bc[c];
                    s_bc[c] = run;
                    run += t;
                }
            }
            __syncthreads();
            for (uint32_t k = threadIdx.x; k <= nb2; k += blockDim.x) s_bstart[k] = k < nb2 ? s_bc[k * W] : n;
            __syncthreads();
            /* the band list, stable: warps in order, each sub-range in order */
            for (uint32_t b = lo; b < hi; b += 32) {  /* warp-uniform */
                const uint32_t i = b + lane;
                const bool valid = i < hi;
                const uint32_t band = valid ? (cscr[start + i].x / P1 - rlo) / R2 : 0u;
                const uint32_t act = __ballot_sync(kFull, valid);
                uint32_t peers = 0, pos = 0;
                if (valid) {
                    peers = __match_any_sync(act, band);
                    pos = s_bc[band * W + w] + __popc(peers & lt_mask);
                }
                __syncwarp();
                if (valid && lane == __ffs(peers) - 1) s_bc[band * W + w] += __popc(peers);
                __syncwarp();
                if (valid) s_blist[pos] = i;
            }
            __syncthreads();
            /* each warp sorts whole bands */
            uint32_t *tab = s_cnt + (uint32_t)w * R2 * P1;
            for (uint32_t bb = w; bb < nb2; bb += W) {  /* warp-uniform */
                const uint32_t rb = rlo + bb * R2;
                const uint32_t cb0 = rb * P1, nb = min(R2, rhi + 1 - rb) * P1;
                const uint32_t bs = s_bstart[bb], be = s_bstart[bb + 1];
                for (uint32_t c = lane; c < nb; c += 32) tab[c] = 0;
                __syncwarp();
                for (uint32_t kb = bs; kb < be; kb += 32) {
                    const uint32_t k = kb + lane;
                    const bool valid = k < be;
                    const uint32_t lc = valid ? cscr[start + s_blist[k]].x - cb0 : 0u;
                    const uint32_t act = __ballot_sync(kFull, valid);
                    if (valid) {
                        const uint32_t peers = __match_any_sync(act, lc);
                        if (lane == __ffs(peers) - 1) tab[lc] += __popc(peers);
                    }
                    __syncwarp();
                }
                /* exclusive scan of the band's cells, lane-contiguous blocks */
                const uint32_t per = (nb + 31) / 32;
                const uint32_t c0 = min(nb, lane * per), c1 = min(nb, c0 + per);
                uint32_t sum = 0;
                for (uint32_t c = c0; c < c1; ++c) sum += tab[c];
                uint32_t incl = sum;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t y = __shfl_up_sync(kFull, incl, d);
                    if (lane >= (uint32_t)d) incl += y;
                }
                uint32_t run = incl - sum;
                for (uint32_t c = c0; c < c1; ++c) {
                    const uint32_t t = tab[c];
                    tab[c] = run;
                    run += t;
                }
                __syncwarp();
                for (uint32_t c = lane; c < nb; c += 32) gseg[cb0 + c] = start + bs + tab[c];
                /* place: the band's hits in list order, cursor per cell */
                for (uint32_t kb = bs; kb < be; kb += 32) {
                    const uint32_t k = kb + lane;
                    const bool valid = k < be;
                    uint32_t i = 0, lc = 0, peers = 0, pos = 0;
                    float phi = 0.f;
                    if (valid) {
                        i = s_blist[k];
                        const uint2 cp = cscr[start + i];
                        lc = cp.x - cb0;
                        phi = __uint_as_float(cp.y);
                    }
                    const uint32_t act = __ballot_sync(kFull, valid);
                    if (valid) {
                        peers = __match_any_sync(act, lc);
                        pos = bs + tab[lc] + __popc(peers & lt_mask);
                    }
                    __syncwarp();
                    if (valid && lane == __ffs(peers) - 1) tab[lc] += __popc(peers);
                    __syncwarp();
                    if (valid) {
                        s_src[pos] = i;
                        s_phi[pos] = phi;
                    }
                }
                __syncwarp();
            }
            __syncthreads();
        }

        uint32_t band_base = 0;  /* hits in the rows below the band */
        for (uint32_t rb = rlo; !wband && rb <= rhi; rb += R) {  /* block-uniform */
            const uint32_t cb0 = BANDED ? rb * P1 : 0u;
            const uint32_t nb = BANDED ? min(R, rhi + 1 - rb) * P1 : C;  /* the band's cells */
            {
                const uint32_t nw = (uint32_t)W * Ct, n4 = nw >> 2;
                for (uint32_t k = threadIdx.x; k < n4; k += blockDim.x)
                    reinterpret_cast<uint4 *>(s_cnt)[k] = make_uint4(0u, 0u, 0u, 0u);
                for (uint32_t k = (n4 << 2) + threadIdx.x; k < nw; k += blockDim.x) s_cnt[k] = 0;
            }
            __syncthreads();

            /* pass 1: per-warp counts of the band's cells */
            if (cached) {
#pragma unroll
                for (int j = 0; j < kItems; ++j) {
                    const uint32_t b = lo + j * 32;
                    if (b < hi) {  /* warp-uniform */
                        const bool valid = b + lane < hi;
                        if (!BANDED) {
                            const uint32_t act = __ballot_sync(kFull, valid);
                            if (valid) cpeers[j] = __match_any_sync(act, ccell[j]);
                        }
                        const uint32_t lc = ccell[j] - cb0;
                        if (valid && lc < nb && lane == __ffs(cpeers[j]) - 1)
                            s_cnt[w * Ct + lc] += __popc(cpeers[j]);
                        __syncwarp();
                    }
                }
            } else {
                for (uint32_t b = lo; b < hi; b += 32) {
                    const uint32_t i = b + lane;
                    bool valid = i < hi;
                    uint32_t cell = 0;
                    if (valid) {
                        const uint32_t h = start + i;
                        if (scratch) {
                            cell = cscr[h].x;
                        } else {
                            float phi;
                            bool bad;
                            cell = hit_cell(kp, in.x[h], in.y[h], in.z[h], &phi, &bad);
                            if (bad && rb == rlo) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_OUTSIDE_GRID);
                        }
                        valid = cell - cb0 < nb;
                    }
                    const uint32_t act = __ballot_sync(kFull, valid);
                    if (valid) {
                        const uint32_t peers = __match_any_sync(act, cell);
                        if (lane == __ffs(peers) - 1) s_cnt[w * Ct + (cell - cb0)] += __popc(peers);
                    }
                    __syncwarp();
                }
            }
            __syncthreads();

            /* pass 2: prefix over warps per cell, then scan over cells */
            for (uint32_t c = threadIdx.x; c < nb; c += blockDim.x) {
                uint32_t run = 0;
                for (int q = 0; q < W; ++q) {
                    const uint32_t t = s_cnt[q * Ct + c];
                    s_cnt[q * Ct + c] = run;
                    run += t;
                }
                s_tot[c] = run;
            }
            __syncthreads();
            uint32_t band_n;
            {
                const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
                const uint32_t c0 = min(nb, threadIdx.x * per), c1 = min(nb, c0 + per);
                uint32_t sum = 0;
                for (uint32_t c = c0; c < c1; ++c) sum += s_tot[c];
                uint32_t run = block_exclusive_scan(sum, s_warp, &band_n);
                for (uint32_t c = c0; c < c1; ++c) {
                    const uint32_t t = s_tot[c];
                    s_tot[c] = run;
                    run += t;
                }
            }
            __syncthreads();
            /* s_tot now holds the band's cell starts and s_cnt each warp's
             * offset inside the cell: a hit's position is band_base plus
             * their sum plus its rank in the warp */
            for (uint32_t c = threadIdx.x; c < nb; c += blockDim.x)
                gseg[cb0 + c] = start + band_base + s_tot[c];

            /* pass 3: positions (segment-relative) */
            if (staged && cached) {
#pragma unroll
                for (int j = 0; j < kItems; ++j) {
                    const uint32_t b = lo + j * 32;
                    if (b < hi) {  /* warp-uniform */
                        const uint32_t lc = ccell[j] - cb0;
                        const bool valid = b + lane < hi && lc < nb;
                        uint32_t pos = 0;
                        if (valid) pos = band_base + s_tot[lc] + s_cnt[w * Ct + lc] + __popc(cpeers[j] & lt_mask);
                        __syncwarp();
                        if (valid && lane == __ffs(cpeers[j]) - 1) s_cnt[w * Ct + lc] += __popc(cpeers[j]);
                        __syncwarp();
                        if (valid) {
                            s_src[pos] = b + lane;
                            s_phi[pos] = cphi[j];
                        }
                    }
                }
            } else {
                for (uint32_t b = lo; b < hi; b += 32) {
                    const uint32_t i = b + lane;
                    bool valid = i < hi;
                    uint32_t pos = 0, peers = 0, cell = 0;
                    float x = 0.f, y = 0.f, z = 0.f, phi = 0.f;
                    uint32_t h = 0;
                    if (valid) {
                        h = start + i;
                        if (!staged) {
                            x = in.x[h]; y = in.y[h]; z = in.z[h];
                        }
                        if (scratch) {
                            const uint2 cp = cscr[h];
                            cell = cp.x;
                            phi = __uint_as_float(cp.y);
                        } else {
                            if (staged) {
                                x = in.x[h]; y = in.y[h]; z = in.z[h];
                            }
                            bool bad;
                            cell = hit_cell(kp, x, y, z, &phi, &bad);
                        }
                        valid = cell - cb0 < nb;
                    }
                    const uint32_t act = __ballot_sync(kFull, valid);
                    if (valid) {
                        peers = __match_any_sync(act, cell);
                        pos = band_base + s_tot[cell - cb0] + s_cnt[w * Ct + (cell - cb0)] +
                              __popc(peers & lt_mask);
                    }
                    __syncwarp();
                    if (valid && lane == __ffs(peers) - 1) s_cnt[w * Ct + (cell - cb0)] += __popc(peers);
                    __syncwarp();
                    if (valid) {
                        if (staged) {
                            s_src[pos] = i;
                            s_phi[pos] = phi;
                        } else {
                            const uint32_t ly = in.layer[h], ev = in.event[h];
                            if (ly != l + 1 || ev != e) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH);
                            const uint32_t d = start + pos;
                            if (out.x) {
                                out.x[d] = x; out.y[d] = y; out.z[d] = z; out.phi[d] = phi;
                                out.det[d] = in.det[h]; out.hitid[d] = in.hitid[h];
                            }
                            out.layer[d] = ly; out.event[d] = ev; out.orig[d] = h;
                            if (out.zphi) {
                                out.zphi[d] = make_float2(z, phi);
                                out.zh[d] = __half_as_ushort(__float2half_rn(z));
                                out.xyzp[d] = make_float4(x, y, z, phi);
                            }
                        }
                    }
                }
            }
            band_base += band_n;
            __syncthreads();
            if (!BANDED) break;
        }

        /* pass 4: coalesced column writes of a staged segment */
        if (staged) {
            bool mismatch = false;
            for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
                const uint32_t h = start + s_src[k];
                const float x = in.x[h], y = in.y[h], z = in.z[h];
                const uint32_t ly = in.layer[h], ev = in.event[h];
                mismatch |= ly != l + 1 || ev != e;
                const uint32_t d = start + k;
                if (out.x) {
                    out.x[d] = x; out.y[d] = y; out.z[d] = z; out.phi[d] = s_phi[k];
                    out.det[d] = in.det[h]; out.hitid[d] = in.hitid[h];
                }
                out.layer[d] = ly; out.event[d] = ev;
                out.orig[d] = h;
                if (out.zphi) {
                    out.zphi[d] = make_float2(z, s_phi[k]);
                    out.zh[d] = __half_as_ushort(__float2half_rn(z));
                    out.xyzp[d] = make_float4(x, y, z, s_phi[k]);
                }
            }
            if (mismatch) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH);
            __syncthreads();
        }
    }
}

/* One sorted hit written to every output column at position d. */
__device__ __forceinline__ void grid_write_hit(const InCols &in, const SortedCols &out, uint32_t h,
                                               uint32_t d, float x, float y, float z, float phi,
                                               uint32_t ly, uint32_t ev)
{
    if (out.x) {
        out.x[d] = x; out.y[d] = y; out.z[d] = z; out.phi[d] = phi;
        out.det[d] = in.det[h]; out.hitid[d] = in.hitid[h];
    }
    out.layer[d] = ly; out.event[d] = ev; out.orig[d] = h;
    if (out.zphi) {
        out.zphi[d] = make_float2(z, phi);
        out.zh[d] = __half_as_ushort(__float2half_rn(z));
        out.xyzp[d] = make_float4(x, y, z, phi);
    }
}

/*
 * Grid build for dense segments on fine grids (the average segment beyond the
 * registers of k_grid_build, its grid beyond one cell table): warp bands,
 * with shared memory small enough for two CTAs per SM, so that one
 * segment's barriers and loads overlap another's.  A CTA takes (event, layer)
 * segments from a device counter:
 *   pass 0  each hit's cell and phi into the scratch column `cscr`, and the
 *           z rows the segment occupies;
 *   pass 1  hits per (band of R2 rows, warp) over each warp's sub-range; an
 *           exclusive scan over (band, warp) gives every band's first
 *           position and every warp's cursor in it;
 *   pass 2  the band list `blist` (segment-relative input indices in band
 *           order; stable: warps in order, each sub-range in order);
 *   pass 3  each warp sorts whole bands: per-cell counts in a warp-private
 *           table, their scan, the band's grid rows, and each hit's position,
 *           recorded in shared memory (segments of at most `stage` hits) or
 *           the columns written there at once;
 *   pass 4  staged segments write every column coalesced.
 * Within a cell hits keep input order, as in k_grid_build.  Dynamic shared
 * memory: stage + tabw + nbm + 1 words (nbm = the bands of Z + 1 rows,
 * tabw = max(nbm * W, W * R2 * (P + 1))).
 */
__global__ void __launch_bounds__(512, 2) k_grid_build_wb(KParams kp, InCols in, SortedCols out,
                                                          const uint32_t *seg_start,
                                                          const uint32_t *seg_n, uint32_t *grid,
                                                          uint32_t stage, uint32_t R2, uint2 *cscr,
                                                          uint32_t *blist, DevState *st)
{
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_seg, s_rlo, s_rhi;
    const uint32_t C = kp.C, P1 = kp.nphi + 1;
    const uint32_t W = blockDim.x >> 5;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt_mask = lanemask_lt();
    const uint32_t nbm = (kp.nz + R2) / R2;  /* bands of the Z + 1 rows */
    const uint32_t tabw = max(nbm * W, W * R2 * P1);
    uint32_t *s_src = smem;              /* [stage] segment-relative input index per position */
    uint32_t *s_tab = smem + stage;      /* [tabw] (band, warp) counts, then the warps' cell tables */
    uint32_t *s_bstart = s_tab + tabw;   /* [nbm + 1] first position of each band */
    const uint32_t nseg = st->n_events * kp.n_layers;
    for (;;) {
        if (threadIdx.x == 0) {
            s_seg = atomicAdd(&st->gb_next, 1u);
            s_rlo = 0xffffffffu;
            s_rhi = 0u;
        }
        __syncthreads();
        const uint32_t seg = s_seg;
        if (seg >= nseg) break;  /* block-uniform */
        const uint32_t e = seg / kp.n_layers, l = seg % kp.n_layers;
        const uint32_t start = seg_start[seg], n = seg_n[seg];
        const uint32_t chunk = (n + W - 1) / W;
        const uint32_t lo = min(n, w * chunk), hi = min(n, lo + chunk);
        const bool staged = n <= stage;
        uint32_t *gseg = grid + (size_t)seg * C;
        uint32_t *bl = blist + start;

        /* pass 0 */
        {
            bool anybad = false;
            uint32_t mn = 0xffffffffu, mx = 0u;
            for (uint32_t i = lo + lane; i < hi; i += 32) {
                const uint32_t h = start + i;
                float phi;
                bool bad;
                const uint32_t cell = hit_cell(kp, in.x[h], in.y[h], in.z[h], &phi, &bad);
                anybad |= bad;
                cscr[h] = make_uint2(cell, __float_as_uint(phi));
                const uint32_t zs = cell / P1;
                mn = min(mn, zs);
                mx = max(mx, zs);
            }
            if (anybad) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_OUTSIDE_GRID);
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                mn = min(mn, __shfl_xor_sync(kFull, mn, d));
                mx = max(mx, __shfl_xor_sync(kFull, mx, d));
            }
            if (lane == 0) {
                atomicMin(&s_rlo, mn);
                atomicMax(&s_rhi, mx);
            }
        }
        __syncthreads();
        uint32_t rlo = s_rlo, rhi = s_rhi;
        if (rlo > rhi) rlo = rhi = 0;  /* no hits */
        /* rows below the occupied range start at the segment start, rows
         * above it at its end */
        for (uint32_t c = threadIdx.x; c < rlo * P1; c += blockDim.x) gseg[c] = start;
        for (uint32_t c = (rhi + 1) * P1 + threadIdx.x; c < C; c += blockDim.x) gseg[c] = start + n;
        const uint32_t nb2 = (rhi - rlo) / R2 + 1;  /* <= nbm */
        const uint32_t m = nb2 * W;
        for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) s_tab[k] = 0;
        __syncthreads();

        /* pass 1 */
        for (uint32_t b = lo; b < hi; b += 32) {  /* warp-uniform */
            const uint32_t i = b + lane;
            const bool valid = i < hi;
            const uint32_t band = valid ? (cscr[start + i].x / P1 - rlo) / R2 : 0u;
            const uint32_t act = __ballot_sync(kFull, valid);
            if (valid) {
                const uint32_t peers = __match_any_sync(act, band);
                if (lane == __ffs(peers) - 1) s_tab[band * W + w] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        {
            const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
            const uint32_t c0 = min(m, threadIdx.x * per), c1 = min(m, c0 + per);
            uint32_t sum = 0, total;
            for (uint32_t c = c0; c < c1; ++c) sum += s_tab[c];
            uint32_t run = block_exclusive_scan(sum, s_warp, &total);
            for (uint32_t c = c0; c < c1; ++c) {
                const uint32_t t = s_tab[c];
                s_tab[c] = run;
                run += t;
            }
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k <= nb2; k += blockDim.x) s_bstart[k] = k < nb2 ? s_tab[k * W] : n;
        __syncthreads();

        /* pass 2 */
        for (uint32_t b = lo; b < hi; b += 32) {  /* warp-uniform */
            const uint32_t i = b + lane;
            const bool valid = i < hi;
            const uint32_t band = valid ? (cscr[start + i].x / P1 - rlo) / R2 : 0u;
            const uint32_t act = __ballot_sync(kFull, valid);
            uint32_t peers = 0, pos = 0;
            if (valid) {
                peers = __match_any_sync(act, band);
                pos = s_tab[band * W + w] + __popc(peers & lt_mask);
            }
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) s_tab[band * W + w] += __popc(peers);
            __syncwarp();
            if (valid) bl[pos] = i;
        }
        __syncthreads();

        /* pass 3 */
        uint32_t *tab = s_tab + w * R2 * P1;
        bool mismatch = false;
        for (uint32_t bb = w; bb < nb2; bb += W) {  /* warp-uniform */
            const uint32_t rb = rlo + bb * R2;
            const uint32_t cb0 = rb * P1, nb = min(R2, rhi + 1 - rb) * P1;
            const uint32_t bs = s_bstart[bb], be = s_bstart[bb + 1];
            for (uint32_t c = lane; c < nb; c += 32) tab[c] = 0;
            __syncwarp();
            for (uint32_t kb = bs; kb < be; kb += 32) {
                const uint32_t k = kb + lane;
                const bool valid = k < be;
                const uint32_t lc = valid ? cscr[start + bl[k]].x - cb0 : 0u;
                const uint32_t act = __ballot_sync(kFull, valid);
                if (valid) {
                    const uint32_t peers = __match_any_sync(act, lc);
                    if (lane == __ffs(peers) - 1) tab[lc] += __popc(peers);
                }
                __syncwarp();
            }
            const uint32_t per = (nb + 31) / 32;
            const uint32_t c0 = min(nb, lane * per), c1 = min(nb, c0 + per);
            uint32_t sum = 0;
            for (uint32_t c = c0; c < c1; ++c) sum += tab[c];
            uint32_t incl = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, incl, d);
                if (lane >= (uint32_t)d) incl += y;
            }
            uint32_t run = incl - sum;
            for (uint32_t c = c0; c < c1; ++c) {
                const uint32_t t = tab[c];
                tab[c] = run;
                run += t;
            }
            __syncwarp();
            for (uint32_t c = lane; c < nb; c += 32) gseg[cb0 + c] = start + bs + tab[c];
            for (uint32_t kb = bs; kb < be; kb += 32) {
                const uint32_t k = kb + lane;
                const bool valid = k < be;
                uint32_t i = 0, lc = 0, peers = 0, pos = 0;
                float phi = 0.f;
                if (valid) {
                    i = bl[k];
                    const uint2 cp = cscr[start + i];
                    lc = cp.x - cb0;
                    phi = __uint_as_float(cp.y);
                }
                const uint32_t act = __ballot_sync(kFull, valid);
                if (valid) {
                    peers = __match_any_sync(act, lc);
                    pos = bs + tab[lc] + __popc(peers & lt_mask);
                }
                __syncwarp();
                if (valid && lane == __ffs(peers) - 1) tab[lc] += __popc(peers);
                __syncwarp();
                if (valid) {
                    if (staged) {
                        s_src[pos] = i;
                    } else {
                        const uint32_t h = start + i;
                        const uint32_t ly = in.layer[h], ev = in.event[h];
                        mismatch |= ly != l + 1 || ev != e;
                        grid_write_hit(in, out, h, start + pos, in.x[h], in.y[h], in.z[h], phi, ly, ev);
                    }
                }
            }
            __syncwarp();
        }
        if (mismatch) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH);
        __syncthreads();

        /* pass 4 */
        if (staged) {
            bool mm = false;
            for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
                const uint32_t h = start + s_src[k];
                const uint32_t ly = in.layer[h], ev = in.event[h];
                mm |= ly != l + 1 || ev != e;
                grid_write_hit(in, out, h, start + k, in.x[h], in.y[h], in.z[h],
                               __uint_as_float(cscr[h].y), ly, ev);
            }
            if (mm) set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_HIT_LAYER_MISMATCH);
            __syncthreads();
        }
    }
}

/* (z, phi) of the sorted hits packed for the candidate loops, z in half
 * precision for the candidate screen, and (x, y, z, phi) packed. */
__global__ void __launch_bounds__(256) k_pack_zphi(const float *X, const float *Y, const float *Z,
                                                   const float *PHI, uint32_t n, float2 *zphi,
                                                   uint16_t *zh, float4 *xyzp)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float z = Z[i], phi = PHI[i];
        zphi[i] = make_float2(z, phi);
        zh[i] = __half_as_ushort(__float2half_rn(z));
        xyzp[i] = make_float4(X[i], Y[i], z, phi);
    }
}

/*
 * Candidate screen on half-precision z.  Rounding to nearest is monotone, so
 * a hit with zLow <= z <= zHigh has RD(zLow) <= RN(z) <= RU(zHigh) in half
 * precision: hits outside that half interval cannot pass the exact test and
 * are skipped without loading their float columns (NaN fails both).  The
 * screen reads 8 halves (16 bytes) per step; `visit(j)` runs, in ascending
 * j, for every hit of [ra, rb) that passes, until it returns false.
 */
struct ZScreen {
    __half2 lo, hi;
};

/* The screen for the union of the active z windows [lo_v, hi_v]; a window
 * that accepts nothing (lo > hi, or NaN) is left out. */
__device__ __forceinline__ ZScreen zscreen_make(bool a, float loA, float hiA, bool b, float loB,
                                                float hiB)
{
    float lo = INFINITY, hi = -INFINITY;
    if (a && loA <= hiA) { lo = loA; hi = hiA; }
    if (b && loB <= hiB) { lo = loB < lo ? loB : lo; hi = hiB > hi ? hiB : hi; }
    ZScreen zs;
    zs.lo = __half2half2(__float2half_rd(lo));
    zs.hi = __half2half2(__float2half_ru(hi));
    return zs;
}

__device__ __forceinline__ uint32_t zscreen_word(uint32_t w, const ZScreen &zs)
{
    const __half2 h = *reinterpret_cast<const __half2 *>(&w);
    return __hge2_mask(h, zs.lo) & __hle2_mask(h, zs.hi);
}

template <class Visit>
__device__ __forceinline__ void zscreen_walk(const uint16_t *ZH, uint32_t ra, uint32_t rb,
                                             const ZScreen &zs, Visit &&visit)
{
    if (ra >= rb) return;
    /* the run's first and last steps keep only the hits inside [ra, rb) */
    const uint32_t first = ra & ~7u, last = (rb - 1) & ~7u;
    const uint32_t first_mask = 0xffu & ~((1u << (ra & 7u)) - 1u);
    const uint32_t last_mask = (2u << ((rb - 1) & 7u)) - 1u;
    for (uint32_t j8 = first; j8 < rb; j8 += 8) {
        const uint4 q = *reinterpret_cast<const uint4 *>(ZH + j8);
        const uint32_t m0 = zscreen_word(q.x, zs), m1 = zscreen_word(q.y, zs);
        const uint32_t m2 = zscreen_word(q.z, zs), m3 = zscreen_word(q.w, zs);
        if ((m0 | m1 | m2 | m3) == 0u) continue;
        /* one bit per half: a byte from each half (0x00 / 0xff), then the
         * bytes' top bits gathered by a multiply that cannot carry */
        const uint32_t t01 = __byte_perm(m0, m1, 0x7531u) & 0x80808080u;
        const uint32_t t23 = __byte_perm(m2, m3, 0x7531u) & 0x80808080u;
        uint32_t bits = ((t01 * 0x00204081u) >> 28) | (((t23 * 0x00204081u) >> 28) << 4);
        if (j8 == first) bits &= first_mask;
        if (j8 == last) bits &= last_mask;
        while (bits) {
            const uint32_t b = __ffs(bits) - 1;
            bits &= bits - 1;
            if (!visit(j8 + b)) return;
        }
    }
}

/* ------------------------------------------------------------------------
 * Stage 2: pair generation.
 * ---------------------------------------------------------------------- */

/* Group table: per (event, layer triplet) the first item hit and the
 * exclusive prefix of item counts.  The items are the layer-2 (outer) hits
 * for the beam-spot generator, which strides them (PairGeneratorBeamspot.h:
 * 68-73), and the layer-1 (inner) hits for the sector generator
 * (PairGeneratorSector.h:63-67).  One CTA. */
__global__ void __launch_bounds__(1024) k_pair_groups(KParams kp, const uint32_t *grid,
                                                      uint32_t *g_outer_start, uint32_t *g_base,
                                                      DevState *st, bool inner_items)
{
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_carry;
    const uint32_t G = st->n_events * kp.n_lt;
    const uint32_t C = kp.C;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t b = 0; b < G; b += blockDim.x) {
        const uint32_t g = b + threadIdx.x;
        uint32_t n2 = 0;
        if (g < G) {
            const uint32_t e = g / kp.n_lt, lt = g % kp.n_lt;
            const uint32_t item_layer = inner_items ? kp.l1[lt] : kp.l2[lt];
            const uint32_t *row = grid + ((size_t)e * kp.n_layers + (item_layer - 1)) * C;
            g_outer_start[g] = row[0];
            n2 = row[C - 1] - row[0];
        }
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(n2, s_warp, &tot);
        if (g < G) g_base[g] = s_carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        g_base[G] = s_carry;
        st->n_outer = s_carry;
    }
}

/* Outer slot s -> (outer sorted hit, group).  One warp per group. */
__global__ void __launch_bounds__(256) k_pair_slots(KParams kp, const uint32_t *g_outer_start,
                                                    const uint32_t *g_base, uint2 *slots,
                                                    uint32_t slot_cap, DevState *st)
{
    const uint32_t G = st->n_events * kp.n_lt;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t g = gw; g < G; g += nw) {
        const uint32_t b0 = g_base[g], b1 = g_base[g + 1], o = g_outer_start[g];
        for (uint32_t s = b0 + lane; s < b1 && s < slot_cap; s += 32) slots[s] = make_uint2(o + (s - b0), g);
    }
}

struct PairWindow {
    float zLow, zHigh, phiLow, phiHigh;
    uint32_t zLowSector, zHighSector, phiLowSector, phiHighSector;
    uint32_t wrap;
    bool ok;
};

/* pairCount's window (PairGeneratorBeamspot.h:110-162), same FP32 order. */
__device__ __forceinline__ PairWindow pair_window(const KParams &kp, uint32_t lt, float hx,
                                                  float hy, float hz, float phi)
{
    PairWindow w;
    const uint32_t layer = kp.l1[lt] - 1;
    const float z0 = kp.z0[lt];
    const float tip = kp.tip[lt];
    const float sigmaZ = kp.sigma_z[lt];
    const float sigmaPhi = __uint_as_float(kp.spread_phi[lt]);
    const float minLayerRadius1 = kp.rmin[layer];
    const float maxLayerRadius1 = kp.rmax[layer];
    const float minRadiusCurvature = kp.rmin_curv;

    const float signRadius = trax_signf(hy);
    const float r = signRadius * sqrtf(hx * hx + hy * hy);
    const float cotThetaHigh = (hz - z0) / r;
    const float cotThetaLow = (hz + z0) / r;
    float tmp = signRadius * maxLayerRadius1 * cotThetaHigh + z0;
    float zHigh = signRadius * minLayerRadius1 * cotThetaHigh + z0;
    zHigh = (float)(tmp < zHigh) * zHigh + (float)(tmp > zHigh) * tmp;
    tmp = signRadius * maxLayerRadius1 * cotThetaLow - z0;
    float zLow = signRadius * minLayerRadius1 * cotThetaLow - z0;
    zLow = (float)(tmp < zLow) * tmp + (float)(tmp > zLow) * zLow;
    zLow -= sigmaZ;
    zHigh += sigmaZ;
    const int32_t zl = trax_f2i(trax_floor_div(zLow - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z));
    w.zLowSector = (uint32_t)(zl > 0 ? zl : 0);
    const uint32_t zh = trax_f2u(trax_floor_div(zHigh - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z)) + 1u;
    w.zHighSector = zh < kp.nz ? zh : kp.nz;

    const float acos_r = trax_acosf(r / (2 * minRadiusCurvature));
    tmp = fabsf(acos_r - kp.acos_rmax[layer]);
    float dPhi = fabsf(acos_r - kp.acos_rmin[layer]);
    dPhi = (float)(tmp < dPhi) * dPhi + (float)(tmp > dPhi) * tmp;
    tmp = trax_atanf(tip * (r - minLayerRadius1)) / (r * minLayerRadius1);
    float phiHigh = trax_atanf(tip * (r - maxLayerRadius1)) / (r * maxLayerRadius1);
    dPhi += tmp > phiHigh ? tmp : phiHigh;
    float phiLow = phi - dPhi - sigmaPhi;
    phiHigh = phi + dPhi + sigmaPhi;
    const bool wrap = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
    phiLow -= (float)((phiLow > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiLow += (float)((phiLow < -TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh -= (float)((phiHigh > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh += (float)((phiHigh < -TRAX_PI_F) * 2) * TRAX_PI_F;
    w.phiLowSector = trax_f2u(trax_floor_div(phiLow - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi));
    w.phiHighSector = trax_f2u(trax_floor_div(phiHigh - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi)) + 1u;
    w.zLow = zLow; w.zHigh = zHigh; w.phiLow = phiLow; w.phiHigh = phiHigh;
    w.wrap = wrap ? 1u : 0u;
    w.ok = w.phiLowSector <= kp.nphi + 1 && w.phiHighSector <= kp.nphi + 1;
    return w;
}

/* The reference's phi acceptance (PairGeneratorBeamspot.h:213-214,
 * TripletThetaPhiPredictor.h:209-210, :420-421).  actPhi is always a sorted hit's phi,
 * trax_atan2f in [-pi, pi] or NaN, so its wrap-around form
 * (lo <= phi <= pi) || (-pi <= phi <= hi) is lo <= phi || phi <= hi. */
__device__ __forceinline__ bool phi_in(float actPhi, float phiLow, float phiHigh, uint32_t wrap)
{
    return wrap ? (phiLow <= actPhi || actPhi <= phiHigh) : (phiLow <= actPhi && actPhi <= phiHigh);
}

/*
 * Store sweep of one outer hit's inner candidates, row by row.  For each row
 * the reference loop walks j in [jlo, end2) and maps j >= rowEnd back by the
 * row length; that is the index range A = [jlo, min(end2, rowEnd)) followed
 * by the wrapped range B = [max(jlo, rowEnd) - len, end2 - len).  The pairs
 * are the union in ascending index order (the reference's bitmap order): B
 * first, then the part of A above B, written from `pos` on.
 */
__device__ __forceinline__ void pair_store_sweep(const KParams &kp, const uint32_t *lGrid1,
                                                 const float2 *ZP, const PairWindow &w,
                                                 uint32_t lane, uint32_t lt_mask, uint32_t outer,
                                                 uint2 *pairs, uint32_t pos, uint32_t cap)
{
    const uint32_t P1 = kp.nphi + 1;
    uint32_t distinct = 0;
    for (uint32_t zs = w.zLowSector; zs < w.zHighSector; ++zs) {
        const uint32_t rowStart = lGrid1[zs * P1];
        const uint32_t rowEnd = lGrid1[(zs + 1) * P1 - 1];
        const uint32_t len = rowEnd - rowStart;
        const uint32_t jlo = lGrid1[zs * P1 + w.phiLowSector];
        const uint32_t end2 = w.wrap * rowEnd + lGrid1[zs * P1 + w.phiHighSector] - w.wrap * rowStart;
        const uint32_t aLo = jlo, aHi = min(end2, rowEnd);
        const uint32_t jb = max(jlo, rowEnd);
        const uint32_t bLo = jb - len;
        const uint32_t bHi = end2 > jb ? end2 - len : bLo;
        const uint32_t a2 = max(aLo, bHi);
        for (int part = 0; part < 2; ++part) {
            const uint32_t lo = part == 0 ? bLo : a2;
            const uint32_t hi = part == 0 ? bHi : aHi;
            for (uint32_t c = lo; c < hi; c += 32) {
                const uint32_t idx = c + lane;
                bool acc = false;
                if (idx < hi) {
                    const float2 v = ZP[idx];
                    acc = w.zLow <= v.x && v.x <= w.zHigh && phi_in(v.y, w.phiLow, w.phiHigh, w.wrap);
                }
                const uint32_t b = __ballot_sync(kFull, acc);
                if (acc) {
                    const uint32_t p = pos + distinct + __popc(b & lt_mask);
                    if (p < cap) pairs[p] = make_uint2(idx, outer);
                }
                distinct += __popc(b);
            }
        }
    }
}

/*
 * Count sweep of one outer hit in the store's order (per row: B, then the part
 * of A above B).  With B's accepts that also lie in A counted twice, the
 * visits equal the reference's (A and B walked in full) and the distinct
 * accepts its bitmap bits.  Every chunk with accepts is recorded as (first
 * index, ballot mask) while `cap` entries last, so that the store replays
 * the ballots instead of sweeping again; *n_save counts all such chunks
 * (> cap: the record is incomplete and the store sweeps again).
 */
__device__ __forceinline__ void pair_count_sweep(const KParams &kp, const uint32_t *lGrid1,
                                                 const float2 *ZP,
                                                 const PairWindow &w, uint32_t lane,
                                                 uint32_t &visits, uint32_t &distinct,
                                                 uint2 *save, uint32_t &n_save, uint32_t cap)
{
    const uint32_t P1 = kp.nphi + 1;
    for (uint32_t zs = w.zLowSector; zs < w.zHighSector; ++zs) {
        const uint32_t rowStart = lGrid1[zs * P1];
        const uint32_t rowEnd = lGrid1[(zs + 1) * P1 - 1];
        const uint32_t len = rowEnd - rowStart;
        const uint32_t jlo = lGrid1[zs * P1 + w.phiLowSector];
        const uint32_t end2 = w.wrap * rowEnd + lGrid1[zs * P1 + w.phiHighSector] - w.wrap * rowStart;
        const uint32_t aLo = jlo, aHi = min(end2, rowEnd);
        const uint32_t jb = max(jlo, rowEnd);
        const uint32_t bLo = jb - len;
        const uint32_t bHi = end2 > jb ? end2 - len : bLo;
        const uint32_t a2 = max(aLo, bHi);
        for (int part = 0; part < 2; ++part) {
            const uint32_t lo = part == 0 ? bLo : a2;
            const uint32_t hi = part == 0 ? bHi : aHi;
            for (uint32_t c = lo; c < hi; c += 32) {
                const uint32_t idx = c + lane;
                bool acc = false;
                if (idx < hi) {
                    const float2 v = ZP[idx];
                    acc = w.zLow <= v.x && v.x <= w.zHigh && phi_in(v.y, w.phiLow, w.phiHigh, w.wrap);
                }
                const uint32_t m = __ballot_sync(kFull, acc);
                const uint32_t nm = __popc(m);
                visits += nm;
                distinct += nm;
                if (part == 0) visits += __popc(__ballot_sync(kFull, acc && idx >= aLo && idx < aHi));
                if (m) {
                    if (lane == 0 && n_save < cap) save[n_save] = make_uint2(c, m);
                    ++n_save;
                }
            }
        }
    }
}

/*
 * Pair stage in one pass.  Warp-sized tiles of 32 outer slots, one per lane:
 * each lane computes its own outer hit's window (no redundant math), then
 * the warp sweeps the candidates of its 32 items one item at a time with all
 * lanes (coalesced loads; ballots keep the inner-hit order).  A warp scan
 * plus warp-wide decoupled look-back turns the distinct counts into positions;
 * with RECORD the store replays the count sweep's ballots (kept per item in
 * shared memory), otherwise -- and for an item whose ballots did not fit --
 * a second sweep on L1-resident hits stores the pairs.
 */
__device__ __forceinline__ PairWindow shfl_window(const PairWindow &w, int k)
{
    PairWindow r;
    r.zLow = __shfl_sync(kFull, w.zLow, k);
    r.zHigh = __shfl_sync(kFull, w.zHigh, k);
    r.phiLow = __shfl_sync(kFull, w.phiLow, k);
    r.phiHigh = __shfl_sync(kFull, w.phiHigh, k);
    r.zLowSector = __shfl_sync(kFull, w.zLowSector, k);
    r.zHighSector = __shfl_sync(kFull, w.zHighSector, k);
    r.phiLowSector = __shfl_sync(kFull, w.phiLowSector, k);
    r.phiHighSector = __shfl_sync(kFull, w.phiHighSector, k);
    r.wrap = __shfl_sync(kFull, w.wrap, k);
    r.ok = true;
    return r;
}

template <bool RECORD>
__global__ void __launch_bounds__(256) k_pair_fused(KParams kp, const uint32_t *grid,
                                                    const float4 *XYZP, const float2 *ZP,
                                                    const uint2 *slots, uint32_t slot_cap,
                                                    uint32_t *pexcl, uint2 *pairs,
                                                    uint32_t pair_cap, unsigned long long *status,
                                                    DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = lanemask_lt();
    /* per warp and item: the count sweep's chunks with accepts (RECORD) */
    __shared__ uint2 s_save[kFusedThreads / 32][32][RECORD ? kPairSave : 1];
    __shared__ uint32_t s_nsave[kFusedThreads / 32][32];
    const uint32_t wib = threadIdx.x >> 5;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            pexcl[0] = 0;
            st->n_pairs = 0;
        }
        return;
    }
    const uint32_t ntiles = (n + 31) / 32;
    unsigned long long my_visits = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(&st->tile_ctr[0], 1u);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= ntiles) break;
        const uint32_t s = tile * 32 + lane;
        bool live = s < n;
        PairWindow w{};
        uint32_t outer = 0, lgoff = 0;
        if (live) {
            const uint2 sl = slots[s];
            outer = sl.x;
            const uint32_t e = sl.y / kp.n_lt, lt = sl.y % kp.n_lt;
            lgoff = (e * kp.n_layers + (kp.l1[lt] - 1)) * kp.C;
            const float4 o = XYZP[outer];
            w = pair_window(kp, lt, o.x, o.y, o.z, o.w);
            if (!w.ok) {
                set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                live = false;
            }
        }
        /* count sweep: the warp walks each live item's candidates */
        uint32_t mine = 0;
        const uint32_t live_mask = __ballot_sync(kFull, live);
        for (uint32_t m = live_mask; m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            const PairWindow wk = shfl_window(w, k);
            const uint32_t lgk = __shfl_sync(kFull, lgoff, k);
            uint32_t visits = 0, distinct = 0, nsave = 0;
            pair_count_sweep(kp, grid + lgk, ZP, wk, lane, visits, distinct,
                             &s_save[wib][k][0], nsave, RECORD ? kPairSave : 0);
            if (lane == (uint32_t)k) mine = distinct;
            if (lane == 0) {
                my_visits += visits;
                s_nsave[wib][k] = nsave;
            }
        }
        __syncwarp();
        uint32_t tile_end;
        const uint32_t pos = warp_tile_position(mine, tile, status, st, &tile_end);
        if (s < n) pexcl[s] = pos;
        if (tile == ntiles - 1 && lane == 0) {
            pexcl[n] = tile_end;
            st->n_pairs = tile_end;
        }
        /* store: replay the recorded ballots (an item whose record
         * overflowed sweeps again) */
        for (uint32_t m = __ballot_sync(kFull, live && mine != 0); m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            const uint32_t pk = __shfl_sync(kFull, pos, k);
            const uint32_t ok = __shfl_sync(kFull, outer, k);
            const uint32_t ns = s_nsave[wib][k];
            if (RECORD && ns <= (uint32_t)kPairSave) {
                uint32_t run = 0;
                for (uint32_t q = 0; q < ns; ++q) {
                    const uint2 e = s_save[wib][k][q];
                    if ((e.y >> lane) & 1u) {
                        const uint32_t p = pk + run + __popc(e.y & lt_mask);
                        if (p < pair_cap) pairs[p] = make_uint2(e.x + lane, ok);
                    }
                    run += __popc(e.y);
                }
            } else {
                const PairWindow wk = shfl_window(w, k);
                const uint32_t lgk = __shfl_sync(kFull, lgoff, k);
                pair_store_sweep(kp, grid + lgk, ZP, wk, lane, lt_mask, ok, pairs, pk, pair_cap);
            }
        }
        __syncwarp();
    }
    if (lane == 0 && my_visits) atomicAdd(&st->pair_slots, my_visits);
}

/*
 * Pair stage with one outer hit per lane.  The lane walks its own window's
 * candidates in the reference's bitmap order (per row: B, then the part of A
 * above B), so a warp handles 32 outer hits at once instead of one; the walk
 * loads kPairUnroll candidates before testing them, so that their loads are
 * in flight together.  The count walk keeps the first kPairKeep accepts; a
 * warp scan plus warp-wide decoupled look-back gives every lane its
 * position, and the lane writes the kept accepts or, when it had more, walks
 * again.  KEEP is kPairKeep, or kPairKeepWide for batches whose outer hits
 * mostly have a few dozen pairs (pile-up 50: 40 % faster; at pile-up 200 the
 * larger local array costs more than the second walks it saves).
 */
constexpr int kPairKeep = 16;
constexpr int kPairKeepWide = 48;
constexpr int kPairUnroll = 8;

/* The walk of one outer hit; visit(j, both) gets every accepted inner hit in
 * ascending order (both: a B accept that also lies in A, which the
 * reference's visit count sees twice) and returns false to stop. */
template <class Visit>
__device__ __forceinline__ void pair_lane_walk(const KParams &kp, const uint32_t *lGrid1,
                                               const float2 *ZP, const PairWindow &w,
                                               Visit &&visit)
{
    const uint32_t P1 = kp.nphi + 1;
    bool go = true;
    for (uint32_t zs = w.zLowSector; zs < w.zHighSector && go; ++zs) {
        const uint32_t rowStart = lGrid1[zs * P1];
        const uint32_t rowEnd = lGrid1[(zs + 1) * P1 - 1];
        const uint32_t len = rowEnd - rowStart;
        const uint32_t jlo = lGrid1[zs * P1 + w.phiLowSector];
        const uint32_t end2 = w.wrap * rowEnd + lGrid1[zs * P1 + w.phiHighSector] - w.wrap * rowStart;
        const uint32_t aLo = jlo, aHi = min(end2, rowEnd);
        const uint32_t jb = max(jlo, rowEnd);
        const uint32_t bLo = jb - len;
        const uint32_t bHi = end2 > jb ? end2 - len : bLo;
        const uint32_t a2 = max(aLo, bHi);
        auto range = [&](uint32_t lo, uint32_t hi, bool inB) {
            for (uint32_t j = lo; j < hi && go; j += kPairUnroll) {
                float2 v[kPairUnroll];
#pragma unroll
                for (int u = 0; u < kPairUnroll; ++u)
                    v[u] = j + u < hi ? ZP[j + u] : make_float2(NAN, NAN);  /* NaN fails */
                /* the tests without branches, then the (few) accepts */
                uint32_t m = 0;
#pragma unroll
                for (int u = 0; u < kPairUnroll; ++u)
                    m |= (w.zLow <= v[u].x && v[u].x <= w.zHigh &&
                          phi_in(v[u].y, w.phiLow, w.phiHigh, w.wrap)) ? 1u << u : 0u;
                while (m && go) {
                    const uint32_t jj = j + __ffs(m) - 1;
                    m &= m - 1;
                    go = visit(jj, inB && jj >= aLo && jj < aHi);
                }
            }
        };
        range(bLo, bHi, true);
        if (go) range(a2, aHi, false);
    }
}

template <int KEEP>
__global__ void __launch_bounds__(256) k_pair_lane(KParams kp, const uint32_t *grid,
                                                   const float4 *XYZP, const float2 *ZP,
                                                   const uint2 *slots, uint32_t slot_cap,
                                                   uint32_t *pexcl, uint2 *pairs,
                                                   uint32_t pair_cap, unsigned long long *status,
                                                   DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            pexcl[0] = 0;
            st->n_pairs = 0;
        }
        return;
    }
    const uint32_t ntiles = (n + 31) / 32;
    unsigned long long my_visits = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(&st->tile_ctr[0], 1u);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= ntiles) break;
        const uint32_t s = tile * 32 + lane;
        bool live = s < n;
        PairWindow w{};
        uint32_t outer = 0;
        const uint32_t *lGrid1 = grid;
        if (live) {
            const uint2 sl = slots[s];
            outer = sl.x;
            const uint32_t e = sl.y / kp.n_lt, lt = sl.y % kp.n_lt;
            lGrid1 = grid + (size_t)(e * kp.n_layers + (kp.l1[lt] - 1)) * kp.C;
            const float4 o = XYZP[outer];
            w = pair_window(kp, lt, o.x, o.y, o.z, o.w);
            if (!w.ok) {
                set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                live = false;
            }
        }
        uint32_t mine = 0;
        uint32_t keep[KEEP];
        if (live) {
            pair_lane_walk(kp, lGrid1, ZP, w, [&](uint32_t j, bool both) {
                my_visits += both ? 2u : 1u;
                if (mine < (uint32_t)KEEP) keep[mine] = j;
                ++mine;
                return true;
            });
        }
        uint32_t tile_end;
        const uint32_t pos = warp_tile_position(mine, tile, status, st, &tile_end);
        if (s < n) pexcl[s] = pos;
        if (tile == ntiles - 1 && lane == 0) {
            pexcl[n] = tile_end;
            st->n_pairs = tile_end;
        }
        if (mine == 0) continue;
        if (mine <= (uint32_t)KEEP) {
            for (uint32_t q = 0; q < mine; ++q)
                if (pos + q < pair_cap) pairs[pos + q] = make_uint2(keep[q], outer);
        } else {
            uint32_t q = pos;
            pair_lane_walk(kp, lGrid1, ZP, w, [&](uint32_t j, bool) {
                if (q < pair_cap) pairs[q] = make_uint2(j, outer);
                ++q;
                return true;
            });
        }
    }
    for (int d = 16; d; d >>= 1) my_visits += __shfl_down_sync(kFull, my_visits, d);
    if (lane == 0 && my_visits) atomicAdd(&st->pair_slots, my_visits);
}

/*
 * The same walk split at the scan, so that no warp waits for another (the
 * look-back above cost a third of that kernel on sparse events):
 *   k_pair_count_lane  one outer hit per lane: its count, and its first
 *                      `keep` accepts in walk order in a per-item scratch row;
 *   k_scan             exclusive scan of the counts (the pair total);
 *   k_pair_store_lane  one outer hit per lane: copies its row to the pairs at
 *                      its position, or (more accepts than kept) recomputes
 *                      the window and walks again.
 */
__global__ void __launch_bounds__(256) k_pair_count_lane(KParams kp, const uint32_t *grid,
                                                         const float4 *XYZP, const float2 *ZP,
                                                         const uint2 *slots, uint32_t slot_cap,
                                                         uint32_t *count, uint32_t *keep,
                                                         uint32_t keep_n, DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    const uint32_t ntiles = (n + 31) / 32;
    uint32_t my_visits = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(&st->tile_ctr[0], 1u);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= ntiles) break;
        const uint32_t s = tile * 32 + lane;
        if (s < n) {
            const uint2 sl = slots[s];
            const uint32_t outer = sl.x;
            const uint32_t e = sl.y / kp.n_lt, lt = sl.y % kp.n_lt;
            const uint32_t *lGrid1 = grid + (size_t)(e * kp.n_layers + (kp.l1[lt] - 1)) * kp.C;
            const float4 o = XYZP[outer];
            const PairWindow w = pair_window(kp, lt, o.x, o.y, o.z, o.w);
            uint32_t mine = 0;
            if (!w.ok) {
                set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
            } else {
                /* accept q of outer hit s at keep[q * slot_cap + s]: the
                 * store pass reads each q across 32 hits in one access */
                pair_lane_walk(kp, lGrid1, ZP, w, [&](uint32_t j, bool both) {
                    my_visits += both ? 2u : 1u;
                    if (mine < keep_n) keep[(size_t)mine * slot_cap + s] = j;
                    ++mine;
                    return true;
                });
            }
            count[s] = mine;
        }
    }
    unsigned long long v = my_visits;
    for (int d = 16; d; d >>= 1) v += __shfl_down_sync(kFull, v, d);
    if (lane == 0 && v) atomicAdd(&st->pair_slots, v);
}

/* 256 outer hits per block: their pairs form one contiguous range, staged
 * in shared memory from the kept accepts and written out coalesced (a range
 * larger than the stage is written directly); outer hits with more accepts
 * than kept walk again. */
constexpr uint32_t kPairStoreStage = 4096;

__global__ void __launch_bounds__(256) k_pair_store_lane(KParams kp, const uint32_t *grid,
                                                         const float4 *XYZP, const float2 *ZP,
                                                         const uint2 *slots, uint32_t slot_cap,
                                                         const uint32_t *excl,
                                                         const uint32_t *keep, uint32_t keep_n,
                                                         uint2 *pairs, uint32_t pair_cap,
                                                         DevState *st)
{
    __shared__ uint2 s_buf[kPairStoreStage];
    __shared__ uint32_t s_lo, s_hi;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    const uint32_t total = st->n_pairs;
    for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < n; b0 += gridDim.x * blockDim.x) {
        const uint32_t s = b0 + threadIdx.x;
        uint32_t pos = 0, cnt = 0, outer = 0;
        if (s < n) {
            pos = excl[s];
            cnt = (s + 1 < n ? excl[s + 1] : total) - pos;
            if (cnt) outer = slots[s].x;
        }
        if (threadIdx.x == 0) s_lo = pos;
        const uint32_t last = min(n, b0 + blockDim.x) - 1;
        if (s == last) s_hi = pos + cnt;
        __syncthreads();
        const uint32_t lo = s_lo, span = s_hi - s_lo;
        const bool staged = span <= kPairStoreStage;
        if (cnt && cnt <= keep_n) {
            for (uint32_t q = 0; q < cnt; ++q) {
                const uint2 v = make_uint2(keep[(size_t)q * slot_cap + s], outer);
                if (staged) s_buf[pos - lo + q] = v;
                else if (pos + q < pair_cap) pairs[pos + q] = v;
            }
        } else if (cnt && staged) {
            /* this outer hit walks again and writes its own range */
            for (uint32_t q = 0; q < cnt; ++q) s_buf[pos - lo + q] = make_uint2(0u, 0xffffffffu);
        }
        __syncthreads();
        if (staged)
            for (uint32_t k = threadIdx.x; k < span; k += blockDim.x) {
                const uint2 v = s_buf[k];
                /* entries of outer hits that walk again are written by them */
                if (lo + k < pair_cap && v.y != 0xffffffffu) pairs[lo + k] = v;
            }
        if (cnt > keep_n) {
            const uint2 sl = slots[s];
            const uint32_t e = sl.y / kp.n_lt, lt = sl.y % kp.n_lt;
            const uint32_t *lGrid1 = grid + (size_t)(e * kp.n_layers + (kp.l1[lt] - 1)) * kp.C;
            const float4 o = XYZP[outer];
            const PairWindow w = pair_window(kp, lt, o.x, o.y, o.z, o.w);
            uint32_t q = pos;
            pair_lane_walk(kp, lGrid1, ZP, w, [&](uint32_t j, bool) {
                if (q < pair_cap) pairs[q] = make_uint2(j, outer);
                ++q;
                return true;
            });
        }
        __syncthreads();
    }
}

/* ------------------------------------------------------------------------
 * Stage 2, sector variant (PairGeneratorSector.h:43-230).  No cut: every
 * layer-2 hit in the block of pairSpreadZ rows and pairSpreadPhi columns on
 * either side of the inner hit's own cell is paired with it.  The window is
 * pure index arithmetic, so counts need no candidate loads and the kernel
 * is bound by the 8-byte pair writes.
 * ---------------------------------------------------------------------- */
struct SectorWindow {
    uint32_t zLowSector, zHighSector, phiLowSector, phiHighSector, wrap;
    bool ok;
};

/* pairCount's cell block (PairGeneratorSector.h:96-110), same arithmetic. */
__device__ __forceinline__ SectorWindow sector_window(const KParams &kp, uint32_t lt, float hz,
                                                      float phi)
{
    SectorWindow w;
    const uint32_t spreadZ = kp.spread_z[lt], spreadPhi = kp.spread_phi[lt];
    const uint32_t zs = trax_f2u(trax_floor_div(hz - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z));
    const uint32_t zh = zs + spreadZ + 1u;
    w.zHighSector = zh < kp.nz ? zh : kp.nz;
    /* max(0u, zLowSector - spreadZ) of unsigned values is the plain
     * difference: below spreadZ it wraps and no row is visited (:98) */
    w.zLowSector = zs - spreadZ;
    int32_t lo = trax_f2i(trax_floor_div(phi - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi) - (float)spreadPhi);
    uint32_t hi = (uint32_t)lo + 2u * spreadPhi + 1u;
    const bool wrap = lo < 0 || hi > kp.nphi + 1;
    lo = (int32_t)((uint32_t)lo + (uint32_t)(lo < 0) * kp.nphi);
    hi -= (uint32_t)(hi > kp.nphi + 1) * kp.nphi;
    w.ok = lo >= 0 && (uint32_t)lo <= kp.nphi + 1 && hi <= kp.nphi + 1;
    w.phiLowSector = (uint32_t)lo;
    w.phiHighSector = hi;
    w.wrap = wrap ? 1u : 0u;
    return w;
}

/* One row of the block (:114-140): the loop visits j in [jlo, end2) and maps
 * j >= rowEnd back by the row length.  As index sets that is
 * A = [jlo, min(end2, rowEnd)) and B = [max(jlo, rowEnd) - len, end2 - len);
 * their union in ascending order is B, then A above B. */
struct RowSpans {
    uint32_t bLo, bHi, aLo, aHi, visits;
};

__device__ __forceinline__ RowSpans sector_row(const uint32_t *lGrid2, uint32_t P1,
                                               const SectorWindow &w, uint32_t zs)
{
    RowSpans r;
    const uint32_t rowStart = lGrid2[zs * P1];
    const uint32_t rowEnd = lGrid2[(zs + 1) * P1 - 1];
    const uint32_t len = rowEnd - rowStart;
    const uint32_t jlo = lGrid2[zs * P1 + w.phiLowSector];
    const uint32_t end2 = w.wrap * rowEnd + lGrid2[zs * P1 + w.phiHighSector] - w.wrap * rowStart;
    const uint32_t jb = max(jlo, rowEnd);
    r.bLo = jb - len;
    r.bHi = end2 > jb ? end2 - len : r.bLo;
    r.aHi = min(end2, rowEnd);
    r.aLo = max(jlo, r.bHi);
    if (r.aHi < r.aLo) r.aHi = r.aLo;
    r.visits = end2 > jlo ? end2 - jlo : 0u;
    return r;
}

/* Warp tiles of 32 inner-hit items: each lane counts its item's block by
 * arithmetic, a warp scan plus look-back places the tile, then the warp
 * writes each item's pairs with all lanes (coalesced 8-byte stores) in
 * ascending outer-hit order -- the order of the reference's bitmap walk. */
__global__ void __launch_bounds__(256) k_pair_sector(KParams kp, const uint32_t *grid,
                                                     const float2 *ZP,
                                                     const uint2 *slots, uint32_t slot_cap,
                                                     uint32_t *pexcl, uint2 *pairs,
                                                     uint32_t pair_cap, unsigned long long *status,
                                                     DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t P1 = kp.nphi + 1;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    if (n == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            pexcl[0] = 0;
            st->n_pairs = 0;
        }
        return;
    }
    const uint32_t ntiles = (n + 31) / 32;
    unsigned long long my_visits = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(&st->tile_ctr[0], 1u);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= ntiles) break;
        const uint32_t s = tile * 32 + lane;
        bool live = s < n;
        SectorWindow w{};
        uint32_t inner = 0, lgoff = 0, mine = 0;
        if (live) {
            const uint2 sl = slots[s];
            inner = sl.x;
            const uint32_t e = sl.y / kp.n_lt, lt = sl.y % kp.n_lt;
            lgoff = (e * kp.n_layers + (kp.l2[lt] - 1)) * kp.C;
            const float2 zp = ZP[inner];
            w = sector_window(kp, lt, zp.x, zp.y);
            if (!w.ok) {
                set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                live = false;
            } else {
                for (uint32_t zs = w.zLowSector; zs < w.zHighSector; ++zs) {
                    const RowSpans r = sector_row(grid + lgoff, P1, w, zs);
                    mine += (r.bHi - r.bLo) + (r.aHi - r.aLo);
                    my_visits += r.visits;
                }
            }
        }
        uint32_t tile_end;
        const uint32_t pos = warp_tile_position(mine, tile, status, st, &tile_end);
        if (s < n) pexcl[s] = pos;
        if (tile == ntiles - 1 && lane == 0) {
            pexcl[n] = tile_end;
            st->n_pairs = tile_end;
        }
        const uint32_t live_mask = __ballot_sync(kFull, live && mine != 0);
        for (uint32_t m = live_mask; m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            SectorWindow wk;
            wk.zLowSector = __shfl_sync(kFull, w.zLowSector, k);
            wk.zHighSector = __shfl_sync(kFull, w.zHighSector, k);
            wk.phiLowSector = __shfl_sync(kFull, w.phiLowSector, k);
            wk.phiHighSector = __shfl_sync(kFull, w.phiHighSector, k);
            wk.wrap = __shfl_sync(kFull, w.wrap, k);
            const uint32_t lgk = __shfl_sync(kFull, lgoff, k);
            const uint32_t ik = __shfl_sync(kFull, inner, k);
            uint32_t p = __shfl_sync(kFull, pos, k);
            for (uint32_t zs = wk.zLowSector; zs < wk.zHighSector; ++zs) {
                const RowSpans r = sector_row(grid + lgk, P1, wk, zs);
                for (int part = 0; part < 2; ++part) {
                    const uint32_t lo = part == 0 ? r.bLo : r.aLo;
                    const uint32_t hi = part == 0 ? r.bHi : r.aHi;
                    for (uint32_t idx = lo + lane; idx < hi; idx += 32) {
                        const uint32_t q = p + (idx - lo);
                        if (q < pair_cap) pairs[q] = make_uint2(ik, idx);
                    }
                    p += hi - lo;
                }
            }
        }
    }
    for (int d = 16; d > 0; d >>= 1) my_visits += __shfl_xor_sync(kFull, my_visits, d);
    if (lane == 0 && my_visits) atomicAdd(&st->pair_slots, my_visits);
}

/* pair_offsets[g+1] = pairs before the first slot of group g+1. */
__global__ void k_group_offsets(const uint32_t *g_base, const uint32_t *excl, uint32_t *offsets,
                                uint32_t n_lt, uint32_t slot_cap, const uint32_t *total,
                                uint32_t cap, uint32_t detail, DevState *st)
{
    const uint32_t G = st->n_events * n_lt;
    uint32_t n = st->n_outer;
    if (n > slot_cap) n = slot_cap;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t q = g_base[g];
        if (q > n) q = n;
        offsets[g] = g == 0 ? 0u : (q >= n ? *total : excl[q]);
        if (g == G && *total > cap) set_fault(st, TRAX_ERR_CAPACITY, detail);
    }
}

/* ------------------------------------------------------------------------
 * Stage 3: triplet prediction.  One warp per pair.
 * ---------------------------------------------------------------------- */
/* ------------------------------------------------------------------------
 * Per-cell z index.  For every cell with zi_min..kZiMax hits, the (z, phi)
 * of its hits sorted by z (ties by sorted position) at the cell's own
 * positions.  The candidate loops binary-search a z window in it instead of
 * walking the cell; each hit found still gets the reference's exact float
 * tests, so accepted counts are unchanged.  Smaller and larger cells are
 * walked.
 * Sort key: float bits made unsigned-orderable, -0 folded onto +0 and every
 * NaN last, so the order is total and agrees with float comparison on all
 * values a window test can accept.
 * ---------------------------------------------------------------------- */
constexpr uint32_t kZiMax = 256;
/* Runtime knobs (KParams::run_walk, KParams::zi_min; they never change a
 * result): runs of cells with at most run_walk hits are walked whole, and
 * only cells with more than zi_min hits are indexed and searched -- a walk
 * pipelines its loads, a search wins once cells are dense. */

__device__ __forceinline__ uint32_t zkey(float z)
{
    const uint32_t b = __float_as_uint(z);
    if ((b & 0x7fffffffu) == 0u) return 0x80000000u;
    if ((b & 0x7f800000u) == 0x7f800000u && (b & 0x007fffffu)) return 0xffffffffu;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* Each lane probes one cell of a 32-cell group; the warp then ranks the
 * hits of every indexable cell of the group together and scatters them. */
__global__ void __launch_bounds__(256) k_zindex(const uint32_t *grid, uint32_t cells_per_event,
                                                uint32_t zi_min, const float2 *ZP,
                                                float2 *zi, uint32_t *zpos, DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t total = st->n_events * cells_per_event;
    const uint32_t n_hits = st->n_hits;
    for (uint32_t q0 = gw * 32; q0 < total; q0 += nw * 32) {
        const uint32_t q = q0 + lane;
        uint32_t my_a = 0, my_cnt = 0;
        if (q < total) {
            my_a = grid[q];
            const uint32_t b = q + 1 < total ? grid[q + 1] : n_hits;
            my_cnt = b > my_a ? b - my_a : 0u;
        }
        uint32_t todo = __ballot_sync(kFull, my_cnt > zi_min && my_cnt <= kZiMax);
        for (; todo; todo &= todo - 1) {
        const int src = __ffs(todo) - 1;
        const uint32_t a = __shfl_sync(kFull, my_a, src);
        const uint32_t cnt = __shfl_sync(kFull, my_cnt, src);
        uint32_t key[8], rank[8];
        float zz[8], pp[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t i = k * 32 + lane;
            key[k] = 0xffffffffu;
            rank[k] = 0;
            zz[k] = 0.f;
            pp[k] = 0.f;
            if (i < cnt) {
                const float2 v = ZP[a + i];
                zz[k] = v.x;
                pp[k] = v.y;
                key[k] = zkey(zz[k]);
            }
        }
#pragma unroll
        for (int ks = 0; ks < 8; ++ks) {
            if ((uint32_t)ks * 32 >= cnt) break;
            for (uint32_t t = 0; t < 32; ++t) {
                const uint32_t s_idx = ks * 32 + t;
                if (s_idx >= cnt) break;
                const uint32_t ksrc = __shfl_sync(kFull, key[ks], t);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const uint32_t i = k * 32 + lane;
                    rank[k] += (ksrc < key[k] || (ksrc == key[k] && s_idx < i)) ? 1u : 0u;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t i = k * 32 + lane;
            if (i < cnt) {
                zi[a + rank[k]] = make_float2(zz[k], pp[k]);
                zpos[a + rank[k]] = a + i;
            }
        }
        }
    }
}

struct PredWindow {
    float zLow[2], zHigh[2];
    uint32_t zLowSector[2], zHighSector[2];
    float phiLow, phiHigh;
    uint32_t phiLowSector, phiHighSector, wrap;
    bool ok;
};

/* predictCount (variant 0, TripletThetaPhiPredictor.h:111-166) and
 * predictStore (variant 1, :320-375): identical except rOrigin
 * (sqrt(r^2 - tip2) vs sqrt(sqrt(r^2)^2 - tip2)) and zHigh padding
 * (sigmaPhi vs sigmaZ). */
__device__ __forceinline__ PredWindow pred_window(const KParams &kp, uint32_t lt, float p1x,
                                                  float p1y, float p1z, float p2x, float p2y,
                                                  float p2z, float phi1, float phi2)
{
    PredWindow w;
    const uint32_t layer = kp.l3[lt] - 1;
    const float sigmaZ = kp.sigma_z[lt];
    const float sigmaPhi = kp.sigma_phi[lt];
    const float minLayerRadius = kp.rmin[layer];
    const float maxLayerRadius = kp.rmax[layer];
    const float minRadiusCurvature = kp.rmin_curv;

    float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
    tip2 *= tip2;
    tip2 /= ((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
#pragma unroll
    for (int v = 0; v < 2; ++v) {
        float rOrigin;
        if (v == 0) {
            rOrigin = p1x * p1x + p1y * p1y;
            rOrigin = sqrtf(rOrigin - tip2);
        } else {
            rOrigin = sqrtf(p1x * p1x + p1y * p1y);
            rOrigin = sqrtf(rOrigin * rOrigin - tip2);
        }
        const float cotTheta = (p2z - p1z) / (sqrtf(p2x * p2x + p2y * p2y - tip2) - rOrigin);
        const float tmp = p1z + (sqrtf(maxLayerRadius * maxLayerRadius - tip2) - rOrigin) * cotTheta;
        float zLow = p1z + (sqrtf(minLayerRadius * minLayerRadius - tip2) - rOrigin) * cotTheta;
        float zHigh = (float)(tmp > zLow) * tmp + (float)(tmp < zLow) * zLow;
        zLow = (float)(tmp > zLow) * zLow + (float)(tmp < zLow) * tmp;
        zLow -= sigmaZ;
        zHigh += v == 0 ? sigmaPhi : sigmaZ;
        const int32_t zl = trax_f2i(trax_floor_div(zLow - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z));
        w.zLowSector[v] = (uint32_t)(zl > 0 ? zl : 0);
        const uint32_t zh = trax_f2u(trax_floor_div(zHigh - TRAX_MIN_Z, kp.sz_z, kp.inv_sz_z)) + 1u;
        w.zHighSector[v] = zh < kp.nz ? zh : kp.nz;
        w.zLow[v] = zLow;
        w.zHigh[v] = zHigh;
    }
    const float phi = phi2;
    float tmp = phi1;
    float dPhi = phi - tmp;
    dPhi += (dPhi > TRAX_PI_F) ? -2 * TRAX_PI_F : (dPhi < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
    dPhi = fabsf(dPhi);
    const float dHits = sqrtf((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
    const float acos_d = trax_acosf(dHits / (2 * minRadiusCurvature));
    tmp = fabsf(acos_d - kp.acos_rmax[layer]);
    float phiLow = fabsf(acos_d - kp.acos_rmin[layer]);
    dPhi = trax_maxf(dPhi, trax_maxf(tmp, phiLow));
    float phiHigh = phi + dPhi + sigmaPhi;
    phiLow = phi - dPhi - sigmaPhi;
    const bool wrap = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
    phiLow -= (float)((phiLow > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiLow += (float)((phiLow < -TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh -= (float)((phiHigh > TRAX_PI_F) * 2) * TRAX_PI_F;
    phiHigh += (float)((phiHigh < -TRAX_PI_F) * 2) * TRAX_PI_F;
    w.phiLowSector = trax_f2u(trax_floor_div(phiLow - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi));
    const uint32_t ph = trax_f2u(trax_floor_div(phiHigh - TRAX_MIN_PHI, kp.sz_phi, kp.inv_sz_phi)) + 1u;
    w.phiHighSector = ph < kp.nphi ? ph : kp.nphi;
    w.phiLow = phiLow;
    w.phiHigh = phiHigh;
    w.wrap = wrap ? 1u : 0u;
    w.ok = w.phiLowSector <= kp.nphi + 1;
    return w;
}

/*
 * Prediction in two passes and a scan, so that no warp waits for another:
 *   k_predict_count   one pair per thread (grid-stride): both windows, the
 *                     count walk over layer-3 cells (window A = the
 *                     reference's predictCount, B = predictStore), the
 *                     emitted count min(A, B) per pair, its exclusive prefix
 *                     within the pair's 32-pair tile and the tile's total;
 *                     the first kPredKeep window-B accepts of each pair that
 *                     emits go to a stage (a tile's together, in candidate
 *                     order, warp-aggregated atomic append), and a pair with
 *                     more accepts leaves a 32-byte record of its store
 *                     window;
 *   k_scan            exclusive scan of the tile totals (pair order);
 *   k_predict_store   one warp per tile copies its staged accepts to their
 *                     positions (tile prefix + in-tile prefix); the records
 *                     walk window B for the accepts after the first
 *                     kPredKeep, in the reference's visit order.
 * Only pairs with more than kPredKeep candidates are walked twice, and no
 * window is recomputed.
 */
constexpr int kPredKeep = 7;  /* window-B accepts staged per pair */
constexpr uint32_t kPredTicket = 4;  /* 32-pair tiles per work ticket of the count pass */

/* 32-byte record of a pair with more than kPredKeep candidates: its store
 * window (window B). */
struct PredRec {
    uint32_t pair;
    uint32_t grid_off;    /* layer-3 grid of the pair's event */
    uint32_t zsec;        /* zLowSector | zHighSector << 16 */
    uint32_t psec;        /* phiLowSector | phiHighSector << 16 | wrap << 31 */
    float zLow, zHigh, phiLow, phiHigh;  /* window B */
};
static_assert(sizeof(PredRec) == 32, "a store record is one 32-byte sector");

/* Adds window-B accept j (the n-th found) to keep[], the first kPredKeep
 * accepts in visit order: position order within a cell, whose accepts begin
 * at keep[cell0].  Accepts of an indexed cell arrive in z order, so a later
 * one with a smaller position still displaces the cell's largest kept one. */
__device__ __forceinline__ void pred_keep(uint32_t *keep, uint32_t n, uint32_t cell0, uint32_t j)
{
    uint32_t k = n;
    if (k >= (uint32_t)kPredKeep) {
        if (cell0 >= (uint32_t)kPredKeep || keep[kPredKeep - 1] < j) return;
        k = kPredKeep - 1;  /* drop the cell's largest kept position */
    }
    while (k > cell0 && keep[k - 1] > j) {
        keep[k] = keep[k - 1];
        --k;
    }
    keep[k] = j;
}

/* Count walk of one pair: accepts of window A (cA) and B (cB), and the first
 * kPredKeep window-B accepts in the reference's visit order. */
template <bool NOINDEX>
__device__ __forceinline__ void pred_count_walk(const KParams &kp, const uint32_t *lGrid3,
                                                const float2 *ZP, const uint16_t *ZH,
                                                const float2 *zi, const uint32_t *zpos,
                                                const PredWindow &w, uint32_t &cA,
                                                uint32_t &cB, uint32_t *keep)
{
    const uint32_t P1 = kp.nphi + 1;
    cA = 0;
    cB = 0;
    const uint32_t zlo = min(w.zLowSector[0], w.zLowSector[1]);
    const uint32_t zhi = max(w.zHighSector[0], w.zHighSector[1]);
    /* one screen for the pair: the union of the two z windows (a row in
     * only one of them screens a little wider; the exact test decides) */
    const ZScreen scr = zscreen_make(true, w.zLow[0], w.zHigh[0], true, w.zLow[1], w.zHigh[1]);
    for (uint32_t zs = zlo; zs < zhi; ++zs) {
        const bool inA = zs >= w.zLowSector[0] && zs < w.zHighSector[0];
        const bool inB = zs >= w.zLowSector[1] && zs < w.zHighSector[1];
        const uint32_t *row = lGrid3 + zs * P1;
        /* the exact test of a hit that passed the screen (walks visit in
         * position order, so accepts append) */
        auto exact = [&](uint32_t j) {
            const float2 v = ZP[j];
            const bool ph = phi_in(v.y, w.phiLow, w.phiHigh, w.wrap);
            cA += (inA && ph && w.zLow[0] <= v.x && v.x <= w.zHigh[0]) ? 1u : 0u;
            if (inB && ph && w.zLow[1] <= v.x && v.x <= w.zHigh[1]) {
                pred_keep(keep, cB, cB, j);
                ++cB;
            }
            return true;
        };
        /* the reference's visits, as runs of whole cells: columns
         * c0..c1-1 (with wrap-around pLow..P, then 0..pHigh-1) */
        auto run = [&](uint32_t c0, uint32_t c1) {
            const uint32_t ra = row[c0], rb = row[c1];
            /* a small run (every run without the index): walk its contiguous hits */
            if (NOINDEX || rb - ra <= kp.run_walk) {
                zscreen_walk(ZH, ra, rb, scr, exact);
                return;
            }
            /* the run's cells one by one; NOINDEX never gets here, and its
             * loop bound of zero keeps the compiler from warning about it */
            const uint32_t cend = NOINDEX ? c0 : c1;
            for (uint32_t c = c0; c < cend; ++c) {
                const uint32_t ca = row[c], cb = row[c + 1];
                if (cb - ca <= kp.zi_min || cb - ca > kZiMax) {
                    zscreen_walk(ZH, ca, cb, scr, exact);
                    continue;
                }
                const uint32_t keyLo = min(inA ? zkey(w.zLow[0]) : 0xffffffffu,
                                           inB ? zkey(w.zLow[1]) : 0xffffffffu);
                const uint32_t keyHi = max(inA ? zkey(w.zHigh[0]) : 0u, inB ? zkey(w.zHigh[1]) : 0u);
                uint32_t lo = ca, hi = cb;
                while (lo < hi) {
                    const uint32_t m = (lo + hi) >> 1;
                    if (zkey(zi[m].x) < keyLo) lo = m + 1; else hi = m;
                }
                const uint32_t cell0 = cB;
                for (; lo < cb; ++lo) {
                    const float2 v = zi[lo];
                    if (zkey(v.x) > keyHi) break;
                    const bool ph = phi_in(v.y, w.phiLow, w.phiHigh, w.wrap);
                    cA += (inA && ph && w.zLow[0] <= v.x && v.x <= w.zHigh[0]) ? 1u : 0u;
                    if (inB && ph && w.zLow[1] <= v.x && v.x <= w.zHigh[1]) {
                        pred_keep(keep, cB, cell0, zpos[lo]);
                        ++cB;
                    }
                }
            }
        };
        const uint32_t c1 = w.wrap ? P1 : w.phiHighSector;
        if (w.phiLowSector < c1) run(w.phiLowSector, c1);
        if (w.wrap && w.phiHighSector > 0) run(0, w.phiHighSector);
    }
}

/* NOINDEX: the tuning never searches a cell's z index (index_min >= kZiMax),
 * so every run is walked and the search code is left out. */
template <bool NOINDEX>
__global__ void __launch_bounds__(256, 5) k_predict_count(
    KParams kp, const uint32_t *grid, const float4 *XYZP, const float2 *ZP,
    const uint16_t *ZH, const uint32_t *EVENT,
    const uint32_t *LAYER, const float2 *zi, const uint32_t *zpos, const uint2 *pairs,
    const uint32_t *n_pairs_ptr,
    uint32_t pair_cap,
    uint32_t *in_tile,
    uint32_t *tile_sum, uint32_t *stage, uint32_t stage_cap, uint32_t *tile_sbase,
    PredRec *walks, uint32_t walk_cap, DevState *st)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = lanemask_lt();
    uint32_t n = *n_pairs_ptr;
    if (n > pair_cap) n = pair_cap;
    const uint32_t E = st->n_events;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->n_ptile = (n + 31) / 32;
    unsigned long long my_slots = 0, my_trunc = 0;
    /* warps take kPredTicket consecutive 32-pair tiles at a time from a device
     * counter: tiles cost very different amounts (dense rows, long walks),
     * and a warp's consecutive tiles share outer hits and layer-3 cells.
     * With each ticket a warp has the pairs of the ticket one round of warps
     * ahead (one 128-byte line per 16) brought into L2: some warp takes that
     * ticket about when this one is done (a warp holding a ticket ahead
     * would stretch the tail of small batches). */
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    uint32_t tile = 0, left = 0;
    for (;;) {
        if (left == 0) {
            if (lane == 0) tile = atomicAdd(&st->tile_ctr[0], 1u);
            tile = __shfl_sync(kFull, tile, 0);
            const unsigned long long q =
                ((unsigned long long)tile + nw) * (kPredTicket * 32) + lane * 16;
            if (lane < kPredTicket * 2 && q < n) prefetch_l2(pairs + q);
            tile *= kPredTicket;
            left = kPredTicket;
        }
        const uint32_t p0 = tile * 32;
        ++tile;
        --left;
        if (p0 >= n) break;
        const uint32_t p = p0 + lane;
        bool live = p < n;
        PredWindow w{};
        uint32_t goff = 0;
        if (live) {
            const uint2 pr = pairs[p];
            const uint32_t h1 = pr.x, h2 = pr.y;
            const uint32_t event = EVENT[h1];
            const uint32_t lt = LAYER[h1] - 1;
            if (lt >= kp.n_lt || event >= E) {
                set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_BAD_TRIPLET_INDEX);
                live = false;
            } else {
                goff = (event * kp.n_layers + (kp.l3[lt] - 1)) * kp.C;
                const float4 a = XYZP[h1], b = XYZP[h2];
                w = pred_window(kp, lt, a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
                if (!w.ok) {
                    set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_WINDOW_OUTSIDE_GRID);
                    live = false;
                }
            }
        }
        uint32_t emitted = 0;
        uint32_t keep[kPredKeep];
        if (live) {
            uint32_t cA, cB;
            pred_count_walk<NOINDEX>(kp, grid + goff, ZP, ZH, zi, zpos, w, cA, cB, keep);
            emitted = cA < cB ? cA : cB;
            my_slots += cA;
            my_trunc += cB - emitted;
        }
        uint32_t incl = emitted;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        if (p < n) in_tile[p] = incl - emitted;
        if (lane == 31) tile_sum[p0 >> 5] = incl;
        /* the first kPredKeep accepts of every pair that emits go to the
         * stage: a tile's together, in candidate order, at tile_sbase */
        const uint32_t kept = emitted < (uint32_t)kPredKeep ? emitted : (uint32_t)kPredKeep;
        uint32_t kincl = kept;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, kincl, d);
            if (lane >= (uint32_t)d) kincl += y;
        }
        const uint32_t ktotal = __shfl_sync(kFull, kincl, 31);
        uint32_t sbase = 0;
        if (lane == 0) {
            if (ktotal) sbase = atomicAdd(&st->n_prec, ktotal);
            tile_sbase[p0 >> 5] = sbase;
        }
        sbase = __shfl_sync(kFull, sbase, 0);
        const uint32_t at = sbase + kincl - kept;
#pragma unroll
        for (uint32_t q = 0; q < (uint32_t)kPredKeep; ++q)
            if (q < kept && at + q < stage_cap) stage[at + q] = keep[q];
        /* a pair with more accepts also leaves its store window, for the
         * store pass to walk on warps of its own */
        const bool walk = emitted > (uint32_t)kPredKeep;
        const uint32_t wwant = __ballot_sync(kFull, walk);
        uint32_t wbase = 0;
        if (lane == 0 && wwant) wbase = atomicAdd(&st->n_pwalk, (uint32_t)__popc(wwant));
        wbase = __shfl_sync(kFull, wbase, 0);
        if (walk) {
            const uint32_t r = wbase + __popc(wwant & lt_mask);
            if (r < walk_cap) {
                PredRec rec;
                rec.pair = p;
                rec.grid_off = goff;
                rec.zsec = w.zLowSector[1] | (w.zHighSector[1] << 16);
                rec.psec = w.phiLowSector | (w.phiHighSector << 16) | (w.wrap << 31);
                rec.zLow = w.zLow[1];
                rec.zHigh = w.zHigh[1];
                rec.phiLow = w.phiLow;
                rec.phiHigh = w.phiHigh;
                walks[r] = rec;
            }
        }
    }
    /* warp-reduce the statistics, one atomic per warp */
    for (int d = 16; d; d >>= 1) {
        my_slots += __shfl_down_sync(kFull, my_slots, d);
        my_trunc += __shfl_down_sync(kFull, my_trunc, d);
    }
    if (lane == 0 && (my_slots | my_trunc)) {
        atomicAdd(&st->cand_slots, my_slots);
        atomicAdd(&st->cand_truncated, my_trunc);
    }
}

__global__ void __launch_bounds__(256) k_predict_store(
    KParams kp, const uint32_t *grid, const float2 *ZP, const uint16_t *ZH,
    const uint32_t *stage, uint32_t stage_cap, const uint32_t *tile_sbase, const PredRec *walks,
    uint32_t walk_cap, const uint32_t *in_tile, const uint32_t *tile_prefix,
    const uint32_t *n_pairs_ptr, uint32_t pair_cap, const uint32_t *total_ptr, uint2 *cands,
    uint32_t cand_cap, DevState *st)
{
    uint32_t nwalk = st->n_pwalk;
    if (nwalk > walk_cap) nwalk = walk_cap;
    uint32_t n = *n_pairs_ptr;
    if (n > pair_cap) n = pair_cap;
    const uint32_t ntiles = (n + 31) / 32;
    const uint32_t total = *total_ptr;
    const uint32_t P1 = kp.nphi + 1;
    const uint32_t lane = threadIdx.x & 31;
    /*
     * A warp takes groups of 32 tiles of 32 pairs from a device counter (the
     * groups' costs differ); lane i reads tile i's prefix, total and stage
     * offset (coalesced), and the warp then copies each non-empty tile: its
     * candidates are one run of positions and its staged accepts one run of
     * the stage in the same order (the first kPredKeep of each pair), so it
     * copies them one candidate per lane with coalesced stage reads and
     * candidate writes.  The stage reads do not wait for the counts: a tile
     * stages at most 32 * kPredKeep accepts, and the first 32 are read ahead.
     */
    for (;;) {
        uint32_t group = 0;
        if (lane == 0) group = atomicAdd(&st->tile_ctr[0], 1u);
        const uint32_t t0 = __shfl_sync(kFull, group, 0) * 32;
        if (t0 >= ntiles) break;
        const uint32_t tt = t0 + lane;
        uint32_t tp = 0, sb = 0;
        if (tt < ntiles) {
            tp = tile_prefix[tt];
            sb = tile_sbase[tt];
        }
        uint32_t tnext = __shfl_down_sync(kFull, tp, 1);
        if (lane == 31 || tt + 1 >= ntiles) tnext = tt + 1 < ntiles ? tile_prefix[tt + 1] : total;
        const uint32_t ttot = tt < ntiles ? tnext - tp : 0u;
        for (uint32_t busy = __ballot_sync(kFull, ttot != 0); busy; busy &= busy - 1) {
            const uint32_t i = __ffs(busy) - 1;
            const uint32_t t = t0 + i;
            const uint32_t tpi = __shfl_sync(kFull, tp, i);
            const uint32_t ttotal = __shfl_sync(kFull, ttot, i);
            const uint32_t sbase = __shfl_sync(kFull, sb, i);
            const uint32_t p = t * 32 + lane;
            const uint32_t ahead = sbase + lane < stage_cap ? stage[sbase + lane] : 0u;
            const uint32_t it = p < n ? in_tile[p] : ttotal;
            uint32_t next = __shfl_down_sync(kFull, it, 1);
            if (lane == 31) next = ttotal;
            const uint32_t emitted = p < n ? next - it : 0u;
            const uint32_t kept = emitted < (uint32_t)kPredKeep ? emitted : (uint32_t)kPredKeep;
            uint32_t kincl = kept;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, kincl, d);
                if (lane >= (uint32_t)d) kincl += y;
            }
            const uint32_t ktotal = __shfl_sync(kFull, kincl, 31);
            for (uint32_t k0 = 0; k0 < ktotal; k0 += 32) {
                const uint32_t k = k0 + lane;
                /* the pair of staged accept k: the lanes whose inclusive
                 * count is <= k come before it */
                uint32_t o = 0;
#pragma unroll
                for (uint32_t step = 16; step; step >>= 1)
                    if (__shfl_sync(kFull, kincl, o + step - 1) <= k) o += step;
                const uint32_t q = k - __shfl_sync(kFull, kincl - kept, o);
                const uint32_t at = tpi + __shfl_sync(kFull, it, o) + q;
                if (k < ktotal && at < cand_cap && sbase + k < stage_cap)
                    cands[at] = make_uint2(t * 32 + o, k0 == 0 ? ahead : stage[sbase + k]);
            }
        }
    }
    /* the pairs with more than kPredKeep accepts, one per thread: accepts
     * kPredKeep .. min(A, B) - 1 of window B in the reference's visit order */
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nwalk;
         r += gridDim.x * blockDim.x) {
        const PredRec rec = walks[r];
        const uint32_t p = rec.pair;
        if (p >= n) continue;
        const uint32_t pos = tile_prefix[p >> 5] + in_tile[p];
        const uint32_t emitted =
            (p + 1 < n ? tile_prefix[(p + 1) >> 5] + in_tile[p + 1] : total) - pos;
        const uint32_t *lGrid3 = grid + rec.grid_off;
        const uint32_t zLowSector = rec.zsec & 0xffffu, zHighSector = rec.zsec >> 16;
        const uint32_t phiLowSector = rec.psec & 0xffffu;
        const uint32_t phiHighSector = (rec.psec >> 16) & 0x7fffu;
        const uint32_t wrap = rec.psec >> 31;
        const ZScreen scr = zscreen_make(false, 0.f, 0.f, true, rec.zLow, rec.zHigh);
        /* cells in run order, hits of a cell by position -- runs of whole
         * cells walked in position order through the z screen (no z index:
         * its accepts would come in z order) */
        uint32_t written = 0;
        /* a hit of a walk that passed the screen: the exact test */
        auto store = [&](uint32_t j) {
            const float2 v = ZP[j];
            if (rec.zLow <= v.x && v.x <= rec.zHigh && phi_in(v.y, rec.phiLow, rec.phiHigh, wrap)) {
                if (written >= (uint32_t)kPredKeep && pos + written < cand_cap)
                    cands[pos + written] = make_uint2(p, j);
                ++written;
            }
            return written < emitted;
        };
        for (uint32_t zs = zLowSector; zs < zHighSector && written < emitted; ++zs) {
            const uint32_t *row = lGrid3 + zs * P1;
            for (int run = 0; run < 2 && written < emitted; ++run) {
                const uint32_t c0 = run == 0 ? phiLowSector : 0u;
                const uint32_t c1 = run == 0 ? (wrap ? P1 : phiHighSector) : (wrap ? phiHighSector : 0u);
                if (c1 <= c0) continue;
                zscreen_walk(ZH, row[c0], row[c1], scr, store);
            }
        }
    }
}

/* cand_offsets[g+1] = candidates before the first pair of group g+1: the
 * pair's tile prefix plus its in-tile prefix (the total past the last pair). */
__global__ void k_cand_offsets(const uint32_t *pair_offsets, const uint32_t *in_tile,
                               const uint32_t *tile_prefix, uint32_t *cand_offsets,
                               uint32_t n_lt, uint32_t pair_cap, const uint32_t *total,
                               uint32_t cap, DevState *st)
{
    const uint32_t G = st->n_events * n_lt;
    uint32_t n = st->n_pairs;
    if (n > pair_cap) n = pair_cap;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t q = pair_offsets[g];
        if (q > n) q = n;
        cand_offsets[g] = g == 0 ? 0u : (q >= n ? *total : tile_prefix[q >> 5] + in_tile[q]);
        if (g == G && *total > cap) set_fault(st, TRAX_ERR_CAPACITY, TRAX_DETAIL_CAND_CAPACITY);
    }
}

/* ------------------------------------------------------------------------
 * Stage 4: triplet filter + stable compaction in one pass.
 * ---------------------------------------------------------------------- */
/* The filter's cuts (TripletThetaPhiFilter.h:86-147) in two parts with
 * the reference's arithmetic: the dphi cut, then the dtheta cut and the
 * circle fit (impact parameter, minimum radius).  A candidate passes when
 * both do -- the reference's conjunction, evaluated in another order. */
__device__ __forceinline__ bool filter_phi_cut(const KParams &kp, uint32_t lt, const float4 h1,
                                               const float4 h2, const float4 h3)
{
    const float dPhiCut = kp.dphi[lt];
    const float x1 = h1.x, y1 = h1.y;
    const float x2 = h2.x, y2 = h2.y;
    const float x3 = h3.x, y3 = h3.y;
    const int screened = trax_dphi_screen(x2 - x1, y2 - y1, x3 - x2, y3 - y2, kp.dphi_tlo[lt],
                                          kp.dphi_thi[lt]);
    if (screened >= 0) return screened != 0;
    const float angle1 = trax_atan2f((y2 - y1), (x2 - x1));
    const float angle2 = trax_atan2f((y3 - y2), (x3 - x2));
    float delta = angle2 - angle1;
    delta += (delta > TRAX_PI_F) ? -2 * TRAX_PI_F : (delta < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
    return fabsf(delta) <= dPhiCut;
}

__device__ __forceinline__ bool filter_theta_fit_cut(const KParams &kp, uint32_t lt,
                                                     const float4 h1, const float4 h2,
                                                     const float4 h3)
{
    const float dThetaCut = kp.dtheta[lt];
    const float tipCut = kp.tip[lt];
    const float minRadius = kp.rmin_curv;
    const float x1 = h1.x, y1 = h1.y, z1 = h1.z;
    const float x2 = h2.x, y2 = h2.y, z2 = h2.z;
    const float x3 = h3.x, y3 = h3.y, z3 = h3.z;
    bool valid = true;
    const float angle1 = trax_atan2f(sqrtf((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)), (z2 - z1));
    const float angle2 = trax_atan2f(sqrtf((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2)), (z3 - z2));
    const float delta = fabsf(angle2 / angle1);
    valid = valid && (1 - dThetaCut <= delta && delta <= 1 + dThetaCut);
    const float p1z = x1 * x1 + y1 * y1;
    const float p2z = x2 * x2 + y2 * y2;
    const float p3z = x3 * x3 + y3 * y3;
    const float ax = x2 - x1, ay = y2 - y1, az = p2z - p1z;
    const float bx = x3 - x1, by = y3 - y1, bz = p3z - p1z;
    float nx = ay * bz - az * by;
    float ny = az * bx - ax * bz;
    float nz = ax * by - ay * bx;
    const float nlen = sqrtf(nx * nx + ny * ny + nz * nz);
    nx = nx / nlen; ny = ny / nlen; nz = nz / nlen;
    const float cOx = (-nx) / (2 * nz);
    const float cOy = (-ny) / (2 * nz);
    const float c = -(nx * x1 + ny * y1 + nz * p1z);
    const float cR = sqrtf((1 - nz * nz - 4 * c * nz) / (4 * nz * nz));
    float vx = -cOx, vy = -cOy;
    const float vlen = sqrtf(vx * vx + vy * vy);
    vx = vx / vlen; vy = vy / vlen;
    const float pCAx = cOx + cR * vx;
    const float pCAy = cOy + cR * vy;
    const float tip = pCAx * pCAx + pCAy * pCAy;
    valid = valid && (tip <= (tipCut * tipCut));
    valid = valid && (cR >= minRadius);
    return valid;
}

/*
 * The filter as the reference structures it (filterCount's accept bitmap,
 * filterPopCount, scan, filterStore; TripletThetaPhiFilter.h:50-252), without
 * any wait between warps: k_filter_count evaluates the cuts one candidate per
 * thread and writes each 32-candidate word of the accept mask and its
 * popcount; k_scan turns the popcounts into positions; k_filter_store writes
 * the accepted candidates' hits at those positions in candidate order.
 */
/* Two phases per warp and 64 candidates: the dphi cut for all of them
 * (most candidates fail it), then the dtheta cut and the circle fit for the
 * survivors only, queued in shared memory and taken 32 at a time so that
 * the expensive part runs on full warps: survivors left over from one chunk
 * wait for the next chunk's, and a chunk's two mask words are written once
 * its last survivor is done (at most kFiltRing chunks wait).  Accept bits
 * land in the mask words by shared-memory atomics. */
constexpr uint32_t kFiltRing = 4;     /* chunks whose survivors may wait in the queue */
constexpr uint32_t kFiltQueue = 96;   /* survivors waiting: < 32 left over + one chunk */

/* 7 blocks per SM (32 registers, a few spilled): the gathers wait on memory, and
 * more resident warps hide it better than the registers saved would. */
__global__ void __launch_bounds__(256, 7) k_filter_count(KParams kp, const float4 *XYZP,
                                                      const uint32_t *LAYER,
                                                      const uint2 *pairs, const uint2 *cands,
                                                      const uint32_t *n_cands_ptr,
                                                      uint32_t cand_cap, uint32_t *mask,
                                                      uint32_t *word_count, DevState *st)
{
    __shared__ uint4 s_q[kFusedThreads / 32][kFiltQueue];
    __shared__ uint32_t s_w[kFusedThreads / 32][kFiltRing][2];
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = lanemask_lt();
    const uint32_t wib = threadIdx.x >> 5;
    uint32_t n = *n_cands_ptr;
    if (n > cand_cap) n = cand_cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->n_ftile = (n + 31) / 32;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    /* warp-uniform bookkeeping: survivors queued [0, qn); chunks in the ring
     * slots [oldest, oldest + pending), each with its first candidate and
     * the running index one past its last survivor; done = survivors
     * finished so far (running index) */
    uint32_t qn = 0, pending = 0, oldest = 0, done = 0, queued = 0;
    uint32_t ring_i0 = 0, ring_end = 0;  /* lane r < kFiltRing holds slot r */
    /* the dtheta cut and circle fit for the first m queued survivors */
    auto round = [&](uint32_t m) {
        if (lane < m) {
            const uint4 e = s_q[wib][lane];
            const uint32_t lt = e.w & 0xffu, slot = (e.w >> 8) & 0xffu, r = e.w >> 16;
            if (filter_theta_fit_cut(kp, lt, XYZP[e.x], XYZP[e.y], XYZP[e.z]))
                atomicOr(&s_w[wib][r][slot >> 5], 1u << (slot & 31));
        }
        __syncwarp();
        /* move the rest to the front */
        const uint32_t rest = qn - m;
        uint4 keep0 = make_uint4(0, 0, 0, 0), keep1 = keep0;
        if (lane < rest) keep0 = s_q[wib][m + lane];
        if (lane + 32 < rest) keep1 = s_q[wib][m + 32 + lane];
        __syncwarp();
        if (lane < rest) s_q[wib][lane] = keep0;
        if (lane + 32 < rest) s_q[wib][32 + lane] = keep1;
        __syncwarp();
        qn = rest;
        done += m;
    };
    /* writes the mask words of the finished chunks, oldest first */
    auto retire = [&]() {
        while (pending) {
            const uint32_t end = __shfl_sync(kFull, ring_end, oldest);
            if (end > done) break;
            const uint32_t i0 = __shfl_sync(kFull, ring_i0, oldest);
            if (lane < 2 && i0 + lane * 32 < n) {
                const uint32_t m = s_w[wib][oldest][lane];
                mask[(i0 >> 5) + lane] = m;
                word_count[(i0 >> 5) + lane] = __popc(m);
            }
            oldest = (oldest + 1) % kFiltRing;
            --pending;
        }
        __syncwarp();
    };
    /* with many chunks per warp, warps take 4 consecutive chunks at a time
     * from a device counter (chunks cost different amounts, and consecutive
     * ones share pairs and hits); with few, a fixed stride spreads them over
     * every warp and spares the counter.  With each ticket a warp has the
     * candidates of the ticket one round of warps ahead (8 bytes each, one
     * 128-byte line per 16) brought into L2 for the warp that takes it. */
    const bool tickets = (n + 63) / 64 >= nw * 64;
    uint32_t ticket = 0, left = 0;
    for (uint32_t i0 = gw * 64;;) {
        if (tickets) {
            if (left == 0) {
                if (lane == 0) ticket = atomicAdd(&st->tile_ctr[0], 1u);
                ticket = __shfl_sync(kFull, ticket, 0);
                const unsigned long long q = ((unsigned long long)ticket + nw) * 256 + lane * 16;
                if (lane < 16 && q < n) prefetch_l2(cands + q);
                ticket *= 4;
                left = 4;
            }
            i0 = ticket * 64;
            ++ticket;
            --left;
        }
        if (i0 >= n) break;
        /* a free ring slot for this chunk: finish queued survivors until the
         * oldest chunk retires */
        while (pending == kFiltRing) {
            round(qn < 32 ? qn : 32);
            retire();
        }
        const uint32_t r = (oldest + pending) % kFiltRing;
        if (lane < 2) s_w[wib][r][lane] = 0;
        __syncwarp();
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const uint32_t i = i0 + half * 32 + lane;
            bool pass = false;
            uint4 e = make_uint4(0, 0, 0, 0);
            if (i < n) {
                const uint2 c = cands[i];
                const uint2 pr = pairs[c.x];
                const uint32_t lt = LAYER[pr.x] - 1;
                if (lt >= kp.n_lt) {
                    set_fault(st, TRAX_ERR_BAD_INPUT, TRAX_DETAIL_BAD_TRIPLET_INDEX);
                } else {
                    pass = filter_phi_cut(kp, lt, XYZP[pr.x], XYZP[pr.y], XYZP[c.y]);
                    e = make_uint4(pr.x, pr.y, c.y,
                                   lt | ((uint32_t)(half * 32) + lane) << 8 | r << 16);
                }
            }
            const uint32_t b = __ballot_sync(kFull, pass);
            if (pass) s_q[wib][qn + __popc(b & lt_mask)] = e;
            qn += __popc(b);
            queued += __popc(b);
        }
        __syncwarp();
        if (lane == r) {
            ring_i0 = i0;
            ring_end = queued;
        }
        ++pending;
        while (qn >= 32) round(32);
        retire();
        if (!tickets) i0 += nw * 64;
    }
    while (pending) {
        round(qn);
        retire();
    }
}

__global__ void __launch_bounds__(256) k_filter_store(const uint2 *pairs, const uint2 *cands,
                                                      const uint32_t *mask,
                                                      const uint32_t *word_pos, uint32_t *t1,
                                                      uint32_t *t2, uint32_t *t3,
                                                      uint32_t trk_cap, DevState *st)
{
    const uint32_t words = st->n_ftile;
    if (blockIdx.x == 0 && threadIdx.x == 0 && st->n_trk > trk_cap)
        set_fault(st, TRAX_ERR_CAPACITY, TRAX_DETAIL_TRACKLET_CAPACITY);
    /* 32 mask words per warp, one per lane; the accepted candidates of the
     * 32 words are then spread over the lanes in candidate order, so the
     * tracklet writes are coalesced however sparse the words are (a few
     * percent of the candidates pass on pile-up events, a quarter on
     * isolated tracks) */
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; t0 < words;
         t0 += nw * 32) {
        const uint32_t t = t0 + lane;
        const uint32_t m = t < words ? mask[t] : 0u;
        const uint32_t base = m ? word_pos[t] : 0u;
        const uint32_t cnt = __popc(m);
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        for (uint32_t k0 = 0; k0 < total; k0 += 32) {
            const uint32_t k = k0 + lane;
            /* the word holding accepted candidate k: the lanes whose
             * inclusive count is <= k come before it */
            uint32_t o = 0;
#pragma unroll
            for (uint32_t step = 16; step; step >>= 1)
                if (__shfl_sync(kFull, incl, o + step - 1) <= k) o += step;
            const uint32_t mo = __shfl_sync(kFull, m, o);
            const uint32_t before = __shfl_sync(kFull, incl - cnt, o);
            const uint32_t pos0 = __shfl_sync(kFull, base, o);
            if (k < total) {
                const uint32_t r = k - before;
                const uint32_t pos = pos0 + r;
                const uint32_t bit = __fns(mo, 0, (int)r + 1);
                if (pos < trk_cap) {
                    const uint2 c = cands[(t0 + o) * 32 + bit];
                    const uint2 pr = pairs[c.x];
                    t1[pos] = pr.x;
                    t2[pos] = pr.y;
                    t3[pos] = c.y;
                }
            }
        }
    }
}

/* filterOffsetStore (TripletThetaPhiFilter.h:270-292): the last tracklet of
 * each (event, layer triplet) writes its end; offsets must start zeroed. */
__global__ void k_trk_offsets(const uint32_t *t1, const uint32_t *EVENT, const uint32_t *LAYER,
                              uint32_t *offsets, uint32_t n_lt, uint32_t trk_cap, DevState *st)
{
    uint32_t n = st->n_trk;
    if (n > trk_cap) n = trk_cap;
    const uint32_t G = st->n_events * n_lt;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t h = t1[i];
        const uint32_t g = EVENT[h] * n_lt + LAYER[h] - 1;
        bool last = i + 1 == n;
        if (!last) {
            const uint32_t hn = t1[i + 1];
            last = (EVENT[hn] * n_lt + LAYER[hn] - 1) != g;
        }
        if (last && g < G) offsets[g + 1] = i + 1;
    }
}

/* The same offsets when every candidate group is its tracklets' group (the
 * chain's own candidates, with each layer triplet starting on layer lt + 1):
 * the tracklets before group g are the accepted candidates before the
 * group's first candidate, read from the accept mask and its scanned word
 * counts -- one thread per group instead of one per tracklet plus the
 * running maximum. */
__global__ void k_trk_offsets_mask(const uint32_t *cand_offsets, const uint32_t *mask,
                                   const uint32_t *word_pos, uint32_t *offsets, uint32_t n_lt,
                                   uint32_t cand_cap, uint32_t trk_cap, DevState *st)
{
    const uint32_t G = st->n_events * n_lt;
    uint32_t n = st->n_cands;
    if (n > cand_cap) n = cand_cap;
    const uint32_t total = st->n_trk;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t q = cand_offsets[g];
        uint32_t v;
        if (q >= n) {
            v = total;
        } else {
            const uint32_t b = q & 31u;
            v = word_pos[q >> 5] + (b ? __popc(mask[q >> 5] & ((1u << b) - 1u)) : 0u);
        }
        offsets[g] = v < trk_cap ? v : trk_cap;
    }
}

/* filterOffsetMonotonizeStore with sequential semantics: a zero entry takes
 * the previous value, i.e. a running maximum.  One CTA. */
__global__ void __launch_bounds__(1024) k_monotonize(uint32_t *offsets, uint32_t n_lt, DevState *st)
{
    __shared__ uint32_t s_carry;
    __shared__ uint32_t s_w[32];
    const uint32_t n = st->n_events * n_lt + 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t b = 0; b < n; b += blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        uint32_t v = i < n ? offsets[i] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, v, d);
            if (lane >= d) v = max(v, y);
        }
        if (lane == 31) s_w[wid] = v;
        __syncthreads();
        if (wid == 0) {
            uint32_t t = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 0u;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, t, d);
                if (lane >= d) t = max(t, y);
            }
            s_w[lane] = t;
        }
        __syncthreads();
        uint32_t r = max(v, s_carry);
        if (wid > 0) r = max(r, s_w[wid - 1]);
        if (i < n) offsets[i] = r;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = r;
        __syncthreads();
    }
}

/* ------------------------------------------------------------------------
 * TripletConnectivity (src/algorithms/TripletConnectivity.h:56-108): each
 * following tracklet gains sum(base connectivity + 1) over the base
 * tracklets it chains with -- wide: one shared hit (base hit3 == follow
 * hit1, or base hit1 == follow hit3 backwards), tight: two (base hit2, hit3
 * == follow hit1, hit2).  A hash join instead of the reference's
 * all-pairs loop: base keys accumulate their weights in an open-addressing
 * table, then every following tracklet probes its key once.  Probes are
 * bounded by the table size (it is never full: capacity >= 2 * n_base).
 * ---------------------------------------------------------------------- */
constexpr unsigned long long kEmptyKey = 0xffffffffffffffffull;

__device__ __forceinline__ uint32_t conn_hash(unsigned long long k, uint32_t mask)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k & mask;
}

__global__ void k_conn_build(const uint32_t *ka, const uint32_t *kb, const uint32_t *con,
                             uint32_t n, unsigned long long *keys, uint32_t *sums, uint32_t mask,
                             DevState *st)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long key = kb ? (((unsigned long long)ka[i] << 32) | kb[i]) : ka[i];
        const uint32_t w = (con ? con[i] : 0u) + 1u;
        uint32_t h = conn_hash(key, mask);
        for (uint32_t probe = 0; probe <= mask; ++probe) {
            const unsigned long long prev = atomicCAS(&keys[h], kEmptyKey, key);
            if (prev == kEmptyKey || prev == key) {
                atomicAdd(&sums[h], w);
                break;
            }
            if (probe == mask) set_fault(st, TRAX_ERR_CAPACITY, TRAX_DETAIL_TRACKLET_CAPACITY);
            h = (h + 1) & mask;
        }
    }
}

__global__ void k_conn_probe(const uint32_t *ka, const uint32_t *kb, uint32_t n,
                             const unsigned long long *keys, const uint32_t *sums, uint32_t mask,
                             uint32_t *con)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long key = kb ? (((unsigned long long)ka[i] << 32) | kb[i]) : ka[i];
        uint32_t h = conn_hash(key, mask);
        for (uint32_t probe = 0; probe <= mask; ++probe) {
            const unsigned long long k = keys[h];
            if (k == key) {
                con[i] += sums[h];
                break;
            }
            if (k == kEmptyKey) break;
            h = (h + 1) & mask;
        }
    }
}

}  // namespace trax
