/*
 * ref_host.cpp -- the reference's host chain around its own kernel text.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/ref_build.py compiles this file together
 * with the reference's OpenCL kernels (lifted unchanged, apart from comments
 * and vector literals, into oracle/_ref/ref_kernels.inc) into
 * oracle/_ref/libtrax_ref.so.  Tests run it next to the CPU restatement in
 * trax_oracle.c to show that the restatement computes what the reference's
 * kernels compute, element for element.
 *
 * This file restates, in its own code, what the reference's host classes do
 * around the kernels: buffer sizes and initial contents, launch shapes, and
 * the order of the launches --
 *   GridBuilder::run            src/algorithms/GridBuilder.cpp:6-160
 *   PrefixSum::run              src/algorithms/PrefixSum.cpp:8-126
 *   PairGeneratorBeamspot::run  src/algorithms/PairGeneratorBeamspot.cpp:5-177
 *   PairGeneratorSector::run    src/algorithms/PairGeneratorSector.cpp:5-151
 *   TripletThetaPhiPredictor::run  src/algorithms/TripletThetaPhiPredictor.cpp:10-131
 *   TripletThetaPhiFilter::run  src/algorithms/TripletThetaPhiFilter.cpp:10-164
 * called in buildTriplets' order (src/triplet_builder/TripletBuilder.cpp:240-263).
 * Blocking scalar downloads become plain reads; every buffer the reference
 * zero-initialises is zeroed here.
 *
 * Where the reference reads memory it never wrote the harness must pick a
 * value.  Pairing buffers are uninitialised in the reference
 * (Pairings.h:24): slots that pairStore / predictStore leave unwritten are
 * marked with 0xFFFFFFFF here.  An unwritten pair slot would send the
 * predictor to an undefined hit, so the chain stops after the pair stage
 * and reports it.  An unwritten candidate slot is given (0, 0), as a
 * zero-filled fresh buffer would hold, and its accept bit is cleared after
 * filterCount: the restatement in trax_oracle.c skips such slots, and this is
 * the same definition of the undefined slot.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#include <ucontext.h>

#include "ref_cl.h"

#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wunused-variable"
#pragma GCC diagnostic ignored "-Wunused-parameter"
#pragma GCC diagnostic ignored "-Wunused-but-set-variable"
#pragma GCC diagnostic ignored "-Wsign-compare"
#pragma GCC diagnostic ignored "-Wparentheses"
#include "ref_kernels.inc"
#pragma GCC diagnostic pop

#include "trax_oracle.h"

typedef uint32_t u32_t;

namespace refcl {

const NDRange *g_range = nullptr;
thread_local const WorkItem *g_item = nullptr;

namespace {

struct Fiber {
    ucontext_t ctx;
    WorkItem wi;
    bool done;
};

/* Fiber state belongs to the OS thread that runs the work-group: a fiber
 * never moves between threads. */
constexpr size_t kFiberStack = 64 * 1024;
thread_local ucontext_t g_sched;
thread_local std::vector<Fiber> g_fibers;
thread_local std::vector<std::unique_ptr<char[]>> g_stacks;
thread_local size_t g_cur = 0;
thread_local bool g_fibered = false;
thread_local const std::function<void()> *g_body = nullptr;
int g_workers = 1;

void fiber_main()
{
    (*g_body)();
    g_fibers[g_cur].done = true;
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

/* One work-group.  A kernel with barriers gets one fiber per work-item; the
 * fibers take turns in local-id order from one barrier to the next.  Returns
 * false when the work-items disagree on the number of barriers. */
bool run_group(const NDRange &r, const size_t grp[3], bool fibered,
               const std::function<void()> &body)
{
    if (!fibered) {
        WorkItem wi;
        for (size_t lz = 0; lz < r.local[2]; ++lz)
            for (size_t ly = 0; ly < r.local[1]; ++ly)
                for (size_t lx = 0; lx < r.local[0]; ++lx) {
                    const size_t lid[3] = {lx, ly, lz};
                    for (int d = 0; d < 3; ++d) {
                        wi.lid[d] = lid[d];
                        wi.grp[d] = grp[d];
                        wi.gid[d] = grp[d] * r.local[d] + lid[d];
                    }
                    g_item = &wi;
                    body();
                }
        return true;
    }
    const size_t n_local = r.local[0] * r.local[1] * r.local[2];
    if (g_fibers.size() < n_local) g_fibers.resize(n_local);
    while (g_stacks.size() < n_local) g_stacks.emplace_back(new char[kFiberStack]);
    g_fibered = true;
    g_body = &body;
    size_t i = 0;
    for (size_t lz = 0; lz < r.local[2]; ++lz)
        for (size_t ly = 0; ly < r.local[1]; ++ly)
            for (size_t lx = 0; lx < r.local[0]; ++lx, ++i) {
                Fiber &f = g_fibers[i];
                const size_t lid[3] = {lx, ly, lz};
                for (int d = 0; d < 3; ++d) {
                    f.wi.lid[d] = lid[d];
                    f.wi.grp[d] = grp[d];
                    f.wi.gid[d] = grp[d] * r.local[d] + lid[d];
                }
                f.done = false;
                getcontext(&f.ctx);
                f.ctx.uc_stack.ss_sp = g_stacks[i].get();
                f.ctx.uc_stack.ss_size = kFiberStack;
                f.ctx.uc_link = nullptr;
                makecontext(&f.ctx, fiber_main, 0);
            }
    bool ok = true;
    for (;;) {
        size_t n_done = 0;
        for (size_t k = 0; k < n_local; ++k) {
            if (g_fibers[k].done) continue;
            g_cur = k;
            g_item = &g_fibers[k].wi;
            swapcontext(&g_sched, &g_fibers[k].ctx);
            n_done += g_fibers[k].done;
        }
        if (n_done == n_local) break;
        if (n_done != 0) {
            ok = false;
            break;
        }
    }
    g_fibered = false;
    return ok;
}

}  // namespace

void barrier(int)
{
    if (!g_fibered) return;
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

/* Runs `body` once per work-item of the NDRange.  With one worker the groups
 * run in group-id order on the calling thread; with more, worker threads
 * take groups from a shared counter.  Returns false when a group's
 * work-items disagree on the number of barriers. */
static bool launch(const NDRange &r, bool barriers, const std::function<void()> &body)
{
    size_t ng[3];
    for (int d = 0; d < 3; ++d) {
        if (r.local[d] == 0 || r.global[d] % r.local[d] != 0) return false;
        ng[d] = r.global[d] / r.local[d];
    }
    g_range = &r;
    const bool fibered = barriers && r.local[0] * r.local[1] * r.local[2] > 1;
    const size_t total = ng[0] * ng[1] * ng[2];
    std::atomic<size_t> next{0};
    std::atomic<bool> ok{true};
    auto work = [&] {
        for (;;) {
            const size_t g = next.fetch_add(1, std::memory_order_relaxed);
            if (g >= total) break;
            const size_t grp[3] = {g % ng[0], (g / ng[0]) % ng[1], g / (ng[0] * ng[1])};
            if (!run_group(r, grp, fibered, body)) ok = false;
        }
    };
    const size_t workers = std::min<size_t>((size_t)std::max(1, g_workers), total);
    std::vector<std::thread> pool;
    for (size_t t = 1; t < workers; ++t) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    return ok;
}

/* __local memory of a kernel argument: one buffer per slot and OS thread,
 * shared by the work-items of the group that thread runs. */
static u32_t *local_buf(int slot, size_t n)
{
    thread_local std::vector<u32_t> bufs[2];
    std::vector<u32_t> &b = bufs[slot];
    if (b.size() < n) b.resize(n);
    return b.data();
}

}  // namespace refcl

using refcl::NDRange;
using refcl::local_buf;
using refcl::uint2;
typedef uint32_t u32;

namespace {

constexpr u32 kUnwritten = 0xFFFFFFFFu;
constexpr size_t kPad = 64;  // elements past every array's end

NDRange range3(size_t g0, size_t g1, size_t g2, size_t l0)
{
    return NDRange{{g0, g1, g2}, {l0, 1, 1}};
}
NDRange range1(size_t g, size_t l) { return NDRange{{g, 1, 1}, {l, 1, 1}}; }

/* (uint) std::max(1.0f, ceil(((float) n) / d)): the reference computes its
 * group counts in float (PrefixSum.cpp:35,65; TripletThetaPhiPredictor.cpp:19). */
u32 groups_f(u32 n, u32 d)
{
    return (u32)std::max(1.0f, std::ceil(((float)n) / d));
}

u32 next_pow2(u32 n)
{
    n--;
    n |= n >> 1;
    n |= n >> 2;
    n |= n >> 4;
    n |= n >> 8;
    n |= n >> 16;
    n++;
    return n;
}

struct Result {
    std::vector<uint8_t> buf[OR_NITEMS];
    uint64_t size[OR_NITEMS] = {};
    uint64_t stats[OR_NSTATS] = {};
    bool ok = true;
};

template <class T> T *put(Result &r, int item, const std::vector<T> &v, size_t n)
{
    r.buf[item].resize(std::max<size_t>(n, 1) * sizeof(T));
    if (n) std::memcpy(r.buf[item].data(), v.data(), n * sizeof(T));
    r.size[item] = n;
    return reinterpret_cast<T *>(r.buf[item].data());
}

/* PrefixSum (PrefixSum.cpp:8-126): exclusive scan in place by recursive
 * work-group scans over partial sums; wg is the caller's nThreads. */
struct PrefixSum {
    u32 wg;
    std::vector<std::vector<u32>> partial;
    bool ok = true;

    void run(u32 *input, u32 size)
    {
        partial.clear();
        u32 n = groups_f(size, wg << 1);
        while (n > 1) { /* createPartialSums, :35-46 */
            partial.emplace_back(n + kPad, 0u);
            n = groups_f(n, wg << 1);
        }
        scan(input, size, 0);
    }

    void scan(u32 *input, u32 size, u32 level)
    {
        using namespace refcl::PrefixSum;
        const u32 nGroups = groups_f(size, wg << 1);
        const u32 padding = (wg << 1) / MEMORY_BANK_COUNT;
        const size_t nlocal = (wg << 1) + padding + kPad;
        if (nGroups == 1) { /* :72-86 */
            u32 localSize = (u32)std::max(1.0f, std::ceil(((float)size) / 2));
            localSize = next_pow2(localSize);
            NDRange r = range1(localSize, localSize);
            ok &= refcl::launch(r, prefixSumWG_barriers,
                                [&] { prefixSumWG(input, size, local_buf(0, nlocal)); });
            return;
        }
        u32 *part = partial[level].data(); /* :87-124 */
        NDRange r = range1((size_t)wg * nGroups, wg);
        ok &= refcl::launch(r, prefixSumPartial_barriers,
                            [&] { prefixSumPartial(input, size, part, local_buf(0, nlocal)); });
        scan(part, nGroups, level + 1);
        ok &= refcl::launch(r, prefixSumUniformAdd_barriers,
                            [&] { prefixSumUniformAdd(input, size, part); });
    }
};

struct Chain {
    const trax_config *cfg;
    const trax_grid_cfg *g;
    u32 E, L, Z, P, T, C;
    float minZ, minPhi, szZ, szP, minRadiusCurvature;
    // TripletConfigurations columns (TripletConfiguration.h:33)
    std::vector<u32> layer1, layer2, layer3, pairSpreadZ, pairSpreadPhi;
    std::vector<float> dThetaCut, sigmaZ, dPhiCut, sigmaPhi, tipCut, z0;
    std::vector<float> minRadius, maxRadius;  // GeometrySupplement, index layer - 1
    // sorted hits (GridBuilder's output buffers)
    std::vector<float> X, Y, Zc;
    std::vector<u32> layer, det, hitid, event;
    std::vector<u32> grid;
    std::vector<uint2> pairs, cands;
    std::vector<u32> pairOffsets, candOffsets;
    u32 nPairs = 0, nCands = 0;
    bool ok = true;

    void setup(const trax_config *c, const trax_grid_cfg *gc)
    {
        cfg = c;
        g = gc;
        E = g->n_events; L = g->n_layers; Z = g->n_sectors_z; P = g->n_sectors_phi;
        T = cfg->n_layer_triplets;
        C = (Z + 1) * (P + 1);
        /* GridConfig (Grid.h:9-15, 33-37): float constants and quotients */
        const float MIN_Z = -300, MAX_Z = 300;
        const float MIN_PHI = -M_PI, MAX_PHI = M_PI;
        minZ = MIN_Z;
        minPhi = MIN_PHI;
        szZ = (MAX_Z - MIN_Z) / Z;
        szP = (MAX_PHI - MIN_PHI) / P;
        /* TripletConfigurations::minRadiusCurvature (TripletConfiguration.cpp:36-43,
         * TripletConfiguration.h:56-64): double arithmetic, float Bz */
        const double Q = 1.602177E-19, GEV_C = 5.344286E-19;
        const float Bz = cfg->bz > 0 ? cfg->bz : (float)3.8112;
        minRadiusCurvature = (float)(cfg->min_pt * GEV_C / (Bz * Q) * 1E2);
        for (u32 t = 0; t < T; ++t) {
            const trax_layer_triplet &lt = cfg->triplets[t];
            layer1.push_back(lt.layer1); layer2.push_back(lt.layer2); layer3.push_back(lt.layer3);
            dThetaCut.push_back(lt.dtheta_cut); sigmaZ.push_back(lt.sigma_z);
            dPhiCut.push_back(lt.dphi_cut); sigmaPhi.push_back(lt.sigma_phi);
            tipCut.push_back(lt.tip_cut); pairSpreadZ.push_back(lt.pair_spread_z);
            z0.push_back(lt.z0); pairSpreadPhi.push_back(lt.pair_spread_phi);
        }
        for (u32 l = 0; l < cfg->n_geom_layers; ++l) {
            minRadius.push_back(cfg->min_radius[l]);
            maxRadius.push_back(cfg->max_radius[l]);
        }
        for (auto *v : {&layer1, &layer2, &layer3, &pairSpreadZ, &pairSpreadPhi}) v->resize(v->size() + kPad);
        for (auto *v : {&dThetaCut, &sigmaZ, &dPhiCut, &sigmaPhi, &tipCut, &z0, &minRadius, &maxRadius})
            v->resize(v->size() + kPad);
    }

    /* GridBuilder::run (GridBuilder.cpp:6-160).  count_variant 0 gridCount,
     * 1 gridNoLocalCount; store_variant 0 gridStore, 1 gridWrittenLocalStore,
     * 2 gridNoLocalStore (the reference picks by local memory size). */
    void grid_stage(const float *x, const float *y, const float *z, const u32 *lay, const u32 *dt,
                    const u32 *hid, const u32 *ev, u32 n, const u32 *eventOffsets,
                    const u32 *layerHits, const u32 *layerOffsets, u32 nThreads,
                    int count_variant, int store_variant)
    {
        using namespace refcl::GridBuilder;
        /* gridCount takes its hit columns without const */
        float *xm = const_cast<float *>(x), *ym = const_cast<float *>(y), *zm = const_cast<float *>(z);
        grid.assign((size_t)E * L * C + kPad, 0u);
        const size_t nlocal = C + kPad;
        NDRange r = range3(nThreads, L, E, nThreads);
        if (count_variant == 0)
            ok &= refcl::launch(r, gridCount_barriers, [&] {
                gridCount(eventOffsets, layerHits, layerOffsets, L, grid.data(), minZ, szZ, Z,
                          minPhi, szP, P, xm, ym, zm, local_buf(0, nlocal));
            });
        else
            ok &= refcl::launch(r, gridNoLocalCount_barriers, [&] {
                gridNoLocalCount(eventOffsets, layerHits, layerOffsets, L, grid.data(), minZ, szZ,
                                 Z, minPhi, szP, P, xm, ym, zm);
            });
        PrefixSum ps{nThreads};
        ps.run(grid.data(), E * L * C);
        ok &= ps.ok;
        X.assign(n + kPad, 0.f); Y.assign(n + kPad, 0.f); Zc.assign(n + kPad, 0.f);
        layer.assign(n + kPad, 0u); det.assign(n + kPad, 0u);
        hitid.assign(n + kPad, 0u); event.assign(n + kPad, 0u);
        if (store_variant == 0)
            ok &= refcl::launch(r, gridStore_barriers, [&] {
                gridStore(eventOffsets, layerHits, layerOffsets, L, grid.data(), minZ, szZ, Z,
                          minPhi, szP, P, x, y, z, lay, dt, hid, ev, X.data(), Y.data(),
                          Zc.data(), layer.data(), det.data(), hitid.data(), event.data(),
                          local_buf(0, nlocal), local_buf(1, nlocal));
            });
        else if (store_variant == 1)
            ok &= refcl::launch(r, gridWrittenLocalStore_barriers, [&] {
                gridWrittenLocalStore(eventOffsets, layerHits, layerOffsets, L, grid.data(), minZ,
                                      szZ, Z, minPhi, szP, P, x, y, z, lay, dt, hid, ev, X.data(),
                                      Y.data(), Zc.data(), layer.data(), det.data(),
                                      hitid.data(), event.data(), local_buf(1, nlocal));
            });
        else {
            std::vector<u32> gWritten((size_t)E * L * C + kPad, 0u);
            ok &= refcl::launch(r, gridNoLocalStore_barriers, [&] {
                gridNoLocalStore(eventOffsets, layerHits, layerOffsets, L, grid.data(), minZ, szZ,
                                 Z, minPhi, szP, P, x, y, z, lay, dt, hid, ev, X.data(), Y.data(),
                                 Zc.data(), layer.data(), det.data(), hitid.data(), event.data(),
                                 gWritten.data());
            });
        }
    }

    /* LayerGrid(grid, layer, e).size() (Grid.h:90-123): the entries pass
     * through GridEntry::idx(), which returns float. */
    u32 layer_size(u32 lay, u32 e) const
    {
        const size_t base = (size_t)e * L * C + (size_t)(lay - 1) * C;
        const u32 last = (u32)(float)grid[base + C - 1];
        const u32 first = (u32)(float)grid[base];
        return last - first;
    }

    /* The oracle bitmap offsets of both pair generators
     * (PairGeneratorBeamspot.cpp:9-27, PairGeneratorSector.cpp:9-27). */
    u32 bitmap_offsets(std::vector<u32> &oracleOffset) const
    {
        u32 totalMaxPairs = 0;
        for (u32 e = 0; e < E; ++e)
            for (u32 p = 0; p < T; ++p) {
                u32 nMaxPairs = layer_size(layer1[p], e) * layer_size(layer2[p], e);
                nMaxPairs = 32 * std::ceil(nMaxPairs / 32.0);
                oracleOffset.push_back(totalMaxPairs);
                totalMaxPairs += nMaxPairs;
            }
        oracleOffset.resize(oracleOffset.size() + kPad);
        return totalMaxPairs;
    }

    /* PairGeneratorBeamspot::run (PairGeneratorBeamspot.cpp:5-177) or
     * PairGeneratorSector::run (PairGeneratorSector.cpp:5-151). */
    void pair_stage(u32 nThreads, bool sector, int count_variant)
    {
        std::vector<u32> oracleOffset;
        const u32 totalMaxPairs = bitmap_offsets(oracleOffset);
        std::vector<u32> oracle((size_t)std::ceil(totalMaxPairs / 32.0) + kPad, 0u);
        std::vector<u32> prefixSum((size_t)E * T * nThreads + 1 + kPad, 0u);
        const size_t nlocal = C + kPad;
        NDRange r = range3(nThreads, T, E, nThreads);
        if (sector) {
            using namespace refcl::PairGeneratorSector;
            ok &= refcl::launch(r, pairCount_barriers, [&] {
                pairCount(layer1.data(), layer2.data(), L, grid.data(), minZ, szZ, Z, minPhi,
                          szP, P, pairSpreadZ.data(), pairSpreadPhi.data(), X.data(), Y.data(),
                          Zc.data(), oracle.data(), oracleOffset.data(), prefixSum.data(),
                          local_buf(0, nlocal));
            });
        } else {
            using namespace refcl::PairGeneratorBeamspot;
            /* gSigmaPhi is bound to the pairSpreadPhi uint buffer
             * (PairGeneratorBeamspot.cpp:55) */
            const float *sigmaPhiBuf = reinterpret_cast<const float *>(pairSpreadPhi.data());
            if (count_variant == 0)
                ok &= refcl::launch(r, pairCount_barriers, [&] {
                    pairCount(minRadius.data(), maxRadius.data(), layer1.data(), layer2.data(), L,
                              grid.data(), minZ, szZ, Z, minPhi, szP, P, z0.data(), sigmaPhiBuf,
                              sigmaZ.data(), tipCut.data(), minRadiusCurvature, X.data(),
                              Y.data(), Zc.data(), oracle.data(), oracleOffset.data(),
                              prefixSum.data(), local_buf(0, nlocal));
                });
            else
                ok &= refcl::launch(r, pairNoLocalCount_barriers, [&] {
                    pairNoLocalCount(minRadius.data(), maxRadius.data(), layer1.data(),
                                     layer2.data(), L, grid.data(), minZ, szZ, Z, minPhi, szP, P,
                                     z0.data(), sigmaPhiBuf, sigmaZ.data(), tipCut.data(),
                                     minRadiusCurvature, X.data(), Y.data(), Zc.data(),
                                     oracle.data(), oracleOffset.data(), prefixSum.data());
                });
        }
        const u32 count = E * T * nThreads + 1;
        PrefixSum ps{nThreads};
        ps.run(prefixSum.data(), count);
        ok &= ps.ok;
        nPairs = prefixSum[count - 1];
        pairs.assign((size_t)nPairs + kPad, uint2{kUnwritten, kUnwritten});
        pairOffsets.assign((size_t)E * T + 1 + kPad, 0u);
        if (sector) {
            using namespace refcl::PairGeneratorSector;
            ok &= refcl::launch(r, pairStore_barriers, [&] {
                pairStore(layer1.data(), layer2.data(), L, grid.data(), Z, P, oracle.data(),
                          oracleOffset.data(), prefixSum.data(), pairs.data(), pairOffsets.data());
            });
        } else {
            using namespace refcl::PairGeneratorBeamspot;
            ok &= refcl::launch(r, pairStore_barriers, [&] {
                pairStore(layer1.data(), layer2.data(), L, grid.data(), Z, P, oracle.data(),
                          oracleOffset.data(), prefixSum.data(), pairs.data(), pairOffsets.data());
            });
        }
    }

    /* TripletThetaPhiPredictor::run (TripletThetaPhiPredictor.cpp:10-131). */
    void predict_stage(u32 nThreads)
    {
        using namespace refcl::TripletThetaPhiPredictor;
        std::vector<u32> prefixSum((size_t)nPairs + 1 + kPad, 0u);
        u32 nGroups = groups_f(nPairs, nThreads);
        NDRange r = range1((size_t)nGroups * nThreads, nThreads);
        const int *hid = reinterpret_cast<const int *>(hitid.data());
        ok &= refcl::launch(r, predictCount_barriers, [&] {
            predictCount(nullptr, nullptr, minRadius.data(), maxRadius.data(), grid.data(),
                         layer3.data(), L, minZ, szZ, Z, minPhi, szP, P, sigmaZ.data(),
                         sigmaPhi.data(), minRadiusCurvature, pairs.data(), nPairs, X.data(),
                         Y.data(), Zc.data(), event.data(), layer.data(), det.data(), hid,
                         prefixSum.data());
        });
        PrefixSum ps{nThreads};
        ps.run(prefixSum.data(), nPairs + 1);
        ok &= ps.ok;
        nCands = prefixSum[nPairs];
        cands.assign((size_t)nCands + kPad, uint2{kUnwritten, kUnwritten});
        candOffsets.assign((size_t)E * T + 1 + kPad, 0u);
        ok &= refcl::launch(r, predictStore_barriers, [&] {
            predictStore(nullptr, nullptr, minRadius.data(), maxRadius.data(), grid.data(),
                         layer3.data(), L, minZ, szZ, Z, minPhi, szP, P, sigmaZ.data(),
                         sigmaPhi.data(), T, minRadiusCurvature, pairs.data(), nPairs, X.data(),
                         Y.data(), Zc.data(), event.data(), layer.data(), det.data(),
                         prefixSum.data(), cands.data(), candOffsets.data());
        });
        const u32 nOffsets = E * T + 1;
        nGroups = groups_f(nOffsets, nThreads);
        NDRange rm = range1((size_t)nGroups * nThreads, nThreads);
        ok &= refcl::launch(rm, predictOffsetMonotonizeStore_barriers, [&] {
            predictOffsetMonotonizeStore(candOffsets.data(), nOffsets);
        });
    }

    /* TripletThetaPhiFilter::run (TripletThetaPhiFilter.cpp:10-164). */
    void filter_stage(Result &res, u32 nThreads, const std::vector<uint8_t> &candWritten)
    {
        using namespace refcl::TripletThetaPhiFilter;
        const u32 nTripletCandidates = nCands;
        const u32 nOracleCount = (u32)std::ceil(nTripletCandidates / 32.0);
        u32 nGroups = groups_f(nTripletCandidates, nThreads);
        std::vector<u32> oracle((size_t)nOracleCount + kPad, 0u);
        NDRange r = range1((size_t)nGroups * nThreads, nThreads);
        ok &= refcl::launch(r, filterCount_barriers, [&] {
            filterCount(dThetaCut.data(), dPhiCut.data(), tipCut.data(), minRadiusCurvature,
                        pairs.data(), cands.data(), nTripletCandidates, X.data(), Y.data(),
                        Zc.data(), event.data(), layer.data(), oracle.data());
        });
        for (u32 i = 0; i < nTripletCandidates; ++i)
            if (!candWritten[i]) oracle[i / 32] &= ~(1u << (i % 32));
        std::vector<u32> prefixSum((size_t)nOracleCount + 1 + kPad, 0u);
        nGroups = groups_f(nOracleCount, nThreads);
        NDRange rp = range1((size_t)nGroups * nThreads, nThreads);
        ok &= refcl::launch(rp, filterPopCount_barriers, [&] {
            filterPopCount(oracle.data(), prefixSum.data(), nOracleCount);
        });
        PrefixSum ps{nThreads};
        ps.run(prefixSum.data(), nOracleCount + 1);
        ok &= ps.ok;
        const u32 nFoundTriplets = prefixSum[nOracleCount];
        std::vector<u32> h1((size_t)nFoundTriplets + kPad, 0u), h2(h1), h3(h1);
        std::vector<u32> trkOffsets((size_t)E * T + 1 + kPad, 0u);
        ok &= refcl::launch(rp, filterStore_barriers, [&] {
            filterStore(pairs.data(), T, cands.data(), nTripletCandidates, oracle.data(),
                        nOracleCount, prefixSum.data(), h1.data(), h2.data(), h3.data(),
                        trkOffsets.data());
        });
        nGroups = groups_f(nFoundTriplets, nThreads);
        NDRange ro = range1((size_t)nGroups * nThreads, nThreads);
        ok &= refcl::launch(ro, filterOffsetStore_barriers, [&] {
            filterOffsetStore(h1.data(), h2.data(), h3.data(), nFoundTriplets, T, event.data(),
                              layer.data(), trkOffsets.data());
        });
        const u32 nOffsets = E * T + 1;
        nGroups = groups_f(nOffsets, nThreads);
        NDRange rm = range1((size_t)nGroups * nThreads, nThreads);
        ok &= refcl::launch(rm, filterOffsetMonotonizeStore_barriers, [&] {
            filterOffsetMonotonizeStore(trkOffsets.data(), nOffsets);
        });
        put(res, OR_TRK_H1, h1, nFoundTriplets);
        put(res, OR_TRK_H2, h2, nFoundTriplets);
        put(res, OR_TRK_H3, h3, nFoundTriplets);
        put(res, OR_TRK_OFFSETS, trkOffsets, nOffsets);
        res.stats[ORS_TRACKLETS] = nFoundTriplets;
    }
};

}  // namespace

extern "C" {

/* Runs stages 1..n_stages of the reference's chain on host arrays, with the
 * same inputs and the same result items as or_run_ex (trax_oracle.h).
 * grid_threads is the work-group size of the grid stage; one work-item per
 * (event, layer) makes gridStore's racy within-cell order the input order.
 * variant: bit 0 gridNoLocalCount, bits 1-2 store (0 gridStore,
 * 1 gridWrittenLocalStore, 2 gridNoLocalStore), bit 3 pairNoLocalCount.
 * workers > 1 spreads the work-groups of every launch over that many threads
 * (for timing: the reference's races then resolve in no fixed order).
 * Stats: ORS_STATUS 0, or 1 when a work-group's barriers disagreed, or 2 when
 * the pair stage left slots unwritten (the chain stops there), or 3 when a
 * work-group size is not a power of two (PrefixSum's tree walks need one);
 * ORS_CAND_TRUNCATED is not measured (UINT64_MAX). */
void *ref_run(const trax_config *cfg, const trax_grid_cfg *grid, const float *x, const float *y,
              const float *z, const uint32_t *layer, const uint32_t *det, const uint32_t *hitid,
              const uint32_t *event, uint32_t n_hits, const uint32_t *event_offset,
              const uint32_t *layer_nhits, const uint32_t *layer_offset, int n_stages,
              uint32_t n_threads, uint32_t grid_threads, int pair_generator, int variant,
              int workers)
{
    refcl::g_workers = workers > 0 ? workers : 1;
    Result *res = new Result();
    res->size[OR_STATS] = OR_NSTATS;
    Chain c;
    c.setup(cfg, grid);
    if (n_threads == 0) n_threads = 256;
    if (grid_threads == 0) grid_threads = n_threads;
    /* PrefixSum's tree walks assume a power-of-two work-group size */
    if ((n_threads & (n_threads - 1)) || (grid_threads & (grid_threads - 1))) {
        res->stats[ORS_STATUS] = 3;
        return res;
    }
    c.grid_stage(x, y, z, layer, det, hitid, event, n_hits, event_offset, layer_nhits,
                 layer_offset, grid_threads, variant & 1, (variant >> 1) & 3);
    put(*res, OR_SORTED_X, c.X, n_hits);
    put(*res, OR_SORTED_Y, c.Y, n_hits);
    put(*res, OR_SORTED_Z, c.Zc, n_hits);
    put(*res, OR_SORTED_LAYER, c.layer, n_hits);
    put(*res, OR_SORTED_DET, c.det, n_hits);
    put(*res, OR_SORTED_HITID, c.hitid, n_hits);
    put(*res, OR_SORTED_EVENT, c.event, n_hits);
    put(*res, OR_GRID, c.grid, (size_t)c.E * c.L * c.C);
    res->stats[ORS_CAND_TRUNCATED] = UINT64_MAX;
    if (n_stages >= 2 && c.ok) {
        c.pair_stage(n_threads, pair_generator == OR_PAIRS_SECTOR, (variant >> 3) & 1);
        std::vector<uint32_t> flat((size_t)c.nPairs * 2);
        std::vector<uint8_t> valid(c.nPairs);
        uint64_t written = 0;
        for (uint32_t i = 0; i < c.nPairs; ++i) {
            flat[2 * i] = c.pairs[i].x;
            flat[2 * i + 1] = c.pairs[i].y;
            valid[i] = c.pairs[i].x != kUnwritten;
            written += valid[i];
        }
        put(*res, OR_PAIRS, flat, flat.size());
        put(*res, OR_PAIR_VALID, valid, valid.size());
        put(*res, OR_PAIR_OFFSETS, c.pairOffsets, (size_t)c.E * c.T + 1);
        res->stats[ORS_PAIR_SLOTS] = c.nPairs;
        res->stats[ORS_PAIRS] = written;
        if (written != c.nPairs) {
            res->stats[ORS_STATUS] = 2;
            n_stages = 2;
        }
    }
    if (n_stages >= 3 && c.ok) {
        c.predict_stage(n_threads);
        std::vector<uint32_t> flat((size_t)c.nCands * 2);
        std::vector<uint8_t> valid(c.nCands);
        uint64_t written = 0;
        for (uint32_t i = 0; i < c.nCands; ++i) {
            valid[i] = c.cands[i].x != kUnwritten;
            written += valid[i];
            flat[2 * i] = c.cands[i].x;
            flat[2 * i + 1] = c.cands[i].y;
            if (!valid[i]) c.cands[i] = uint2{0u, 0u};
        }
        put(*res, OR_CANDS, flat, flat.size());
        put(*res, OR_CAND_VALID, valid, valid.size());
        put(*res, OR_CAND_OFFSETS, c.candOffsets, (size_t)c.E * c.T + 1);
        res->stats[ORS_CAND_SLOTS] = c.nCands;
        res->stats[ORS_CANDS] = written;
        if (n_stages >= 4 && c.ok) c.filter_stage(*res, n_threads, valid);
    }
    if (!c.ok) res->stats[ORS_STATUS] = 1;
    return res;
}

uint64_t ref_size(const void *r, int item)
{
    return (item >= 0 && item < OR_NITEMS) ? static_cast<const Result *>(r)->size[item] : 0;
}

const void *ref_data(const void *r, int item)
{
    const Result *res = static_cast<const Result *>(r);
    if (item == OR_STATS) return res->stats;
    return (item >= 0 && item < OR_NITEMS && res->size[item]) ? res->buf[item].data() : nullptr;
}

void ref_free(void *r) { delete static_cast<Result *>(r); }

}  // extern "C"
