/*
 * trax_ops.hpp -- the reference's C++ operator surface over the C-ABI.
 *
 * Class and method names, argument order and meaning follow the reference
 * (src/algorithms/GridBuilder.h:42, PairGeneratorBeamspot.h:40-41,
 * PairGeneratorSector.h:38-39, TripletThetaPhiPredictor.h:43-44, TripletThetaPhiFilter.h:46-48,
 * PrefixSum.h:42, TripletConnectivity.h:52-54); collections are device
 * resident and the stages that return a collection hand back an owning raw
 * pointer, as the reference does (TripletBuilder.cpp:282-284).  The work
 * group size argument is accepted and ignored (launch shapes are the
 * library's); the reference's DetectorGeometry / Dictionary arguments are
 * accepted as opaque pointers and unused, as in its kernels.
 *
 * Header only; link libtrax_gb300.so.  Errors throw trax::Error (the C-ABI
 * itself never throws).
 */
#ifndef TRAX_OPS_HPP
#define TRAX_OPS_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "trax.h"

namespace trax {

struct Error : std::runtime_error {
    trax_status status;
    Error(trax_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(trax_ctx *ctx, trax_status s, const char *what)
{
    if (s != TRAX_OK)
        throw Error(s, std::string(what) + ": " + trax_ctx_last_error(ctx));
}

/* One device and stream (the reference's clever::context). */
class Context {
public:
    explicit Context(int device = 0)
    {
        trax_status s = trax_ctx_create(&h_, device);
        if (s != TRAX_OK) throw Error(s, std::string("trax_ctx_create: ") + trax_ctx_last_error(nullptr));
    }
    ~Context() { trax_ctx_destroy(h_); }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    trax_ctx *get() const { return h_; }
    void synchronize() { check(h_, trax_ctx_synchronize(h_), "trax_ctx_synchronize"); }
    trax_counts counts()
    {
        trax_counts c{};
        check(h_, trax_read_counts(h_, &c), "trax_read_counts");
        return c;
    }
    /* The configuration an operator last installed on this context (its
     * GeometrySupplement serves operators whose reference signature takes
     * none), or null before the first one. */
    const trax_config *config() const { return has_config_ ? &config_ : nullptr; }
    void remember(const trax_config &c)
    {
        config_ = c;
        has_config_ = true;
    }

private:
    trax_ctx *h_ = nullptr;
    trax_config config_{};
    bool has_config_ = false;
};

/* A device array owned through the context. */
template <class T>
class DeviceArray {
public:
    DeviceArray(Context &ctx, size_t n) : ctx_(&ctx), n_(n)
    {
        check(ctx.get(), trax_dev_alloc(ctx.get(), (void **)&p_, (n ? n : 1) * sizeof(T)),
              "trax_dev_alloc");
    }
    DeviceArray(Context &ctx, const std::vector<T> &host) : DeviceArray(ctx, host.size())
    {
        upload(host);
    }
    ~DeviceArray()
    {
        if (p_) trax_dev_free(ctx_->get(), p_);
    }
    DeviceArray(const DeviceArray &) = delete;
    DeviceArray &operator=(const DeviceArray &) = delete;
    DeviceArray(DeviceArray &&o) noexcept : ctx_(o.ctx_), p_(o.p_), n_(o.n_) { o.p_ = nullptr; }
    T *data() const { return p_; }
    size_t size() const { return n_; }
    void upload(const std::vector<T> &host)
    {
        if (host.size() > n_) throw Error(TRAX_ERR_BAD_ARG, "upload larger than the array");
        check(ctx_->get(), trax_memcpy_h2d(ctx_->get(), p_, host.data(), host.size() * sizeof(T)),
              "trax_memcpy_h2d");
    }
    void zero() { check(ctx_->get(), trax_memset_d(ctx_->get(), p_, 0, n_ * sizeof(T)), "trax_memset_d"); }
    std::vector<T> download(size_t count) const
    {
        std::vector<T> h(count);
        if (count)
            check(ctx_->get(), trax_memcpy_d2h(ctx_->get(), h.data(), p_, count * sizeof(T)),
                  "trax_memcpy_d2h");
        return h;
    }

private:
    Context *ctx_;
    T *p_ = nullptr;
    size_t n_;
};

/* EventSupplement / LayerSupplement (EventSupplement.h, LayerSupplement.h). */
struct EventSupplement {
    std::vector<uint32_t> nHits, offset;
    uint32_t nEvents() const { return (uint32_t)nHits.size(); }
};
struct LayerSupplement {
    uint32_t nLayers = 0;
    std::vector<uint32_t> nHits, offset;  /* [event * nLayers + layer - 1] */
};

/* GeometrySupplement (GeometrySupplement.h:21-43): radii per layer, index
 * layer - 1. */
struct GeometrySupplement {
    std::vector<float> minRadius, maxRadius;
};

/* TripletConfigurations (TripletConfiguration.h:39-72). */
struct TripletConfigurations {
    explicit TripletConfigurations(float minPt) : minPt_(minPt) {}
    void addWithValue(uint32_t l1, uint32_t l2, uint32_t l3, float dThetaCut, float sigmaZ,
                      float dPhiCut, float sigmaPhi, float tipCut, uint32_t pairSpreadZ, float z0,
                      uint32_t pairSpreadPhi, uint32_t nCandidates)
    {
        rows.push_back({l1, l2, l3, dThetaCut, sigmaZ, dPhiCut, sigmaPhi, tipCut, pairSpreadZ,
                        z0, pairSpreadPhi, nCandidates});
    }
    size_t size() const { return rows.size(); }
    float minRadiusCurvature() const { return trax_min_radius_curvature(minPt_, 0.0f); }
    trax_config config(const GeometrySupplement &geom) const
    {
        trax_config c{};
        if (rows.size() > TRAX_MAX_LAYER_TRIPLETS || geom.minRadius.size() > TRAX_MAX_LAYERS)
            throw Error(TRAX_ERR_BAD_ARG, "too many layer triplets or layers");
        c.n_layer_triplets = (uint32_t)rows.size();
        for (size_t i = 0; i < rows.size(); ++i) c.triplets[i] = rows[i];
        c.n_geom_layers = (uint32_t)geom.minRadius.size();
        for (size_t l = 0; l < geom.minRadius.size(); ++l) {
            c.min_radius[l] = geom.minRadius[l];
            c.max_radius[l] = geom.maxRadius[l];
        }
        c.min_pt = minPt_;
        return c;
    }
    std::vector<trax_layer_triplet> rows;
    float minPt_;
};

/* HitCollection (HitCollection.h:23-59): the seven columns on the device;
 * GridBuilder::run replaces them by the cell-sorted columns (plus phi and
 * the input position `orig`). */
class HitCollection {
public:
    HitCollection(Context &ctx, const std::vector<float> &x, const std::vector<float> &y,
                  const std::vector<float> &z, const std::vector<uint32_t> &layer,
                  const std::vector<uint32_t> &detectorId, const std::vector<uint32_t> &hitId,
                  const std::vector<uint32_t> &eventNumber)
        : n_((uint32_t)x.size()), x_(ctx, x), y_(ctx, y), z_(ctx, z), layer_(ctx, layer),
          det_(ctx, detectorId), hitid_(ctx, hitId), event_(ctx, eventNumber),
          sx_(ctx, n_), sy_(ctx, n_), sz_(ctx, n_), sphi_(ctx, n_), slayer_(ctx, n_),
          sdet_(ctx, n_), shitid_(ctx, n_), sevent_(ctx, n_), sorig_(ctx, n_)
    {
    }
    uint32_t size() const { return n_; }
    trax_hits input() const
    {
        return {x_.data(), y_.data(), z_.data(), layer_.data(), det_.data(), hitid_.data(),
                event_.data(), n_};
    }
    trax_sorted_hits sorted() const
    {
        return {sx_.data(), sy_.data(), sz_.data(), sphi_.data(), slayer_.data(), sdet_.data(),
                shitid_.data(), sevent_.data(), sorig_.data(), n_};
    }
    std::vector<uint32_t> inputPositions() const { return sorig_.download(n_); }
    std::vector<uint32_t> hitIds() const { return shitid_.download(n_); }

private:
    uint32_t n_;
    DeviceArray<float> x_, y_, z_;
    DeviceArray<uint32_t> layer_, det_, hitid_, event_;
    DeviceArray<float> sx_, sy_, sz_, sphi_;
    DeviceArray<uint32_t> slayer_, sdet_, shitid_, sevent_, sorig_;
};

/* GridConfig + Grid (Grid.h:5-68). */
struct GridConfig {
    uint32_t nEvents, nLayers, nSectorsZ, nSectorsPhi;
    trax_grid_cfg c() const { return {nEvents, nLayers, nSectorsZ, nSectorsPhi}; }
    uint32_t cells() const { return (nSectorsZ + 1) * (nSectorsPhi + 1); }
};
class Grid {
public:
    Grid(Context &ctx, const GridConfig &cfg)
        : config(cfg), boundary(ctx, (size_t)cfg.nEvents * cfg.nLayers * cfg.cells()) {}
    std::vector<uint32_t> download() const { return boundary.download(boundary.size()); }
    GridConfig config;
    DeviceArray<uint32_t> boundary;
};

/* Pairing (Pairings.h:9-59). */
class Pairing {
public:
    Pairing(Context &ctx, uint32_t capacity, uint32_t nEvents, uint32_t nLayerTriplets)
        : pairing(ctx, 2ull * (capacity ? capacity : 1)), pairingOffsets(ctx, (size_t)nEvents * nLayerTriplets + 1),
          capacity_(capacity ? capacity : 1)
    {
        pairingOffsets.zero();
    }
    trax_pairs c() const { return {pairing.data(), pairingOffsets.data(), capacity_}; }
    std::vector<uint32_t> getPairings() const { return pairing.download(2ull * size()); }
    std::vector<uint32_t> getPairingOffsets() const { return pairingOffsets.download(pairingOffsets.size()); }
    uint32_t size() const { return count < capacity_ ? count : capacity_; }
    DeviceArray<uint32_t> pairing, pairingOffsets;
    uint32_t count = 0;

private:
    uint32_t capacity_;
};

/* TrackletCollection (TrackletCollection.h:32-77). */
class TrackletCollection {
public:
    TrackletCollection(Context &ctx, uint32_t capacity, uint32_t nEvents, uint32_t nLayerTriplets)
        : hit1(ctx, capacity ? capacity : 1), hit2(ctx, capacity ? capacity : 1),
          hit3(ctx, capacity ? capacity : 1), connectivity(ctx, capacity ? capacity : 1),
          trackletOffsets(ctx, (size_t)nEvents * nLayerTriplets + 1), capacity_(capacity ? capacity : 1)
    {
        connectivity.zero();
        trackletOffsets.zero();
    }
    /* From host columns, one layer triplet (the reference's tests build
     * collections this way, TripletConnectivityTest.h:147-259). */
    TrackletCollection(Context &ctx, const std::vector<uint32_t> &h1, const std::vector<uint32_t> &h2,
                       const std::vector<uint32_t> &h3)
        : TrackletCollection(ctx, (uint32_t)h1.size(), 1, 1)
    {
        if (h2.size() != h1.size() || h3.size() != h1.size())
            throw Error(TRAX_ERR_BAD_ARG, "tracklet columns differ in length");
        hit1.upload(h1);
        hit2.upload(h2);
        hit3.upload(h3);
        trackletOffsets.upload({0u, (uint32_t)h1.size()});
        count = (uint32_t)h1.size();
    }
    trax_tracklets c() const
    {
        return {hit1.data(), hit2.data(), hit3.data(), trackletOffsets.data(), capacity_};
    }
    uint32_t size() const { return count < capacity_ ? count : capacity_; }
    std::vector<uint32_t> getTrackletOffsets() const { return trackletOffsets.download(trackletOffsets.size()); }
    DeviceArray<uint32_t> hit1, hit2, hit3, connectivity, trackletOffsets;
    uint32_t count = 0;

private:
    uint32_t capacity_;
};

class KernelWrapper {
public:
    explicit KernelWrapper(Context &ctx) : ctx_(ctx) {}

protected:
    Context &ctx_;
};

class GridBuilder : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    unsigned long run(HitCollection &hits, unsigned nThreads, const EventSupplement &es,
                      const LayerSupplement &ls, Grid &grid)
    {
        (void)nThreads;
        trax_layout lay{es.nEvents(), ls.nLayers, es.nHits.data(), es.offset.data(),
                        ls.nHits.data(), ls.offset.data()};
        trax_hits in = hits.input();
        trax_sorted_hits out = hits.sorted();
        trax_grid_cfg g = grid.config.c();
        check(ctx_.get(), trax_grid_build(ctx_.get(), &in, &lay, &g, &out, grid.boundary.data()),
              "trax_grid_build");
        return 0;
    }
};

namespace detail {
inline void configure(Context &ctx, const TripletConfigurations &lt, const GeometrySupplement &geom)
{
    trax_config c = lt.config(geom);
    check(ctx.get(), trax_configure(ctx.get(), &c), "trax_configure");
    ctx.remember(c);
}

/* The layer triplets of `lt` with the geometry the context was last
 * configured with. */
inline void configure_cuts(Context &ctx, const TripletConfigurations &lt, const char *who)
{
    const trax_config *prev = ctx.config();
    if (!prev)
        throw Error(TRAX_ERR_BAD_ARG, std::string(who) +
                                          ": no GeometrySupplement configured on this context yet");
    GeometrySupplement geom;
    geom.minRadius.assign(prev->min_radius, prev->min_radius + prev->n_geom_layers);
    geom.maxRadius.assign(prev->max_radius, prev->max_radius + prev->n_geom_layers);
    configure(ctx, lt, geom);
}
}  // namespace detail

namespace detail {
typedef trax_status (*pair_fn)(trax_ctx *, const trax_sorted_hits *, const uint32_t *,
                               const trax_grid_cfg *, trax_pairs *);

/* Runs a pair generator; when the pairs overflow the first capacity the
 * device reports the exact count and the stage reruns once at that size. */
inline Pairing *run_pairs(Context &ctx, pair_fn fn, const char *name, HitCollection &hits,
                          const GeometrySupplement &geom, const TripletConfigurations &lt,
                          const Grid &grid, uint32_t cap)
{
    configure(ctx, lt, geom);
    trax_sorted_hits h = hits.sorted();
    trax_grid_cfg g = grid.config.c();
    for (int attempt = 0; attempt < 2; ++attempt) {
        Pairing *p = new Pairing(ctx, cap, grid.config.nEvents, (uint32_t)lt.size());
        check(ctx.get(), trax_reset_counts(ctx.get()), "trax_reset_counts");
        trax_pairs pc = p->c();
        trax_status s = fn(ctx.get(), &h, grid.boundary.data(), &g, &pc);
        if (s != TRAX_OK) { delete p; check(ctx.get(), s, name); }
        trax_counts c = ctx.counts();
        p->count = (uint32_t)c.n_pairs;
        if (c.status == TRAX_OK) return p;
        delete p;
        if (c.status != TRAX_ERR_CAPACITY) throw Error((trax_status)c.status, name);
        cap = (uint32_t)c.n_pairs + 1;
    }
    throw Error(TRAX_ERR_CAPACITY, name);
}
}  // namespace detail

class PairGeneratorBeamspot : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    Pairing *run(HitCollection &hits, const GeometrySupplement &geom, unsigned nThreads,
                 const TripletConfigurations &lt, const Grid &grid)
    {
        (void)nThreads;
        return detail::run_pairs(ctx_, trax_pair_gen, "trax_pair_gen", hits, geom, lt, grid,
                                 64u * hits.size() + 1024u);
    }
};

/* PairGeneratorSector::run (PairGeneratorSector.h:38-39). */
class PairGeneratorSector : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    Pairing *run(HitCollection &hits, const GeometrySupplement &geom, unsigned nThreads,
                 const TripletConfigurations &lt, const Grid &grid)
    {
        (void)nThreads;
        return detail::run_pairs(ctx_, trax_pair_gen_sector, "trax_pair_gen_sector", hits, geom,
                                 lt, grid, 256u * hits.size() + 1024u);
    }
};

class TripletThetaPhiPredictor : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    Pairing *run(HitCollection &hits, const void *geom, const GeometrySupplement &geomSupplement,
                 const void *dict, int nThreads, const TripletConfigurations &lt, const Grid &grid,
                 const Pairing &pairs)
    {
        (void)geom; (void)dict; (void)nThreads;
        detail::configure(ctx_, lt, geomSupplement);
        trax_sorted_hits h = hits.sorted();
        trax_grid_cfg g = grid.config.c();
        uint32_t cap = 4u * pairs.count + 1024u;
        for (int attempt = 0; attempt < 2; ++attempt) {
            Pairing *c = new Pairing(ctx_, cap, grid.config.nEvents, (uint32_t)lt.size());
            check(ctx_.get(), trax_reset_counts(ctx_.get()), "trax_reset_counts");
            trax_pairs pc = pairs.c(), cc = c->c();
            trax_status s = trax_triplet_predict(ctx_.get(), &h, grid.boundary.data(), &g, &pc, &cc);
            if (s != TRAX_OK) { delete c; check(ctx_.get(), s, "trax_triplet_predict"); }
            trax_counts k = ctx_.counts();
            c->count = (uint32_t)k.n_candidates;
            if (k.status == TRAX_OK) return c;
            delete c;
            if (k.status != TRAX_ERR_CAPACITY) throw Error((trax_status)k.status, "triplet prediction");
            cap = (uint32_t)k.n_candidates + 1;
        }
        throw Error(TRAX_ERR_CAPACITY, "triplet prediction");
    }
};

class TripletThetaPhiFilter : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    /* The reference's signature (TripletThetaPhiFilter.h:46-48): the cuts
     * come from `lt`, the layer radii from the GeometrySupplement the
     * context was configured with by the pair generator or predictor. */
    TrackletCollection *run(HitCollection &hits, const Grid &grid, const Pairing &pairs,
                            const Pairing &tripletCandidates, int nThreads,
                            const TripletConfigurations &lt)
    {
        detail::configure_cuts(ctx_, lt, "TripletThetaPhiFilter::run");
        return filter(hits, grid, pairs, tripletCandidates, nThreads, lt);
    }
    /* The same with the geometry given explicitly. */
    TrackletCollection *run(HitCollection &hits, const Grid &grid, const Pairing &pairs,
                            const Pairing &tripletCandidates, int nThreads,
                            const TripletConfigurations &lt, const GeometrySupplement &geom)
    {
        detail::configure(ctx_, lt, geom);
        return filter(hits, grid, pairs, tripletCandidates, nThreads, lt);
    }

private:
    TrackletCollection *filter(HitCollection &hits, const Grid &grid, const Pairing &pairs,
                               const Pairing &tripletCandidates, int nThreads,
                               const TripletConfigurations &lt)
    {
        (void)nThreads;
        trax_sorted_hits h = hits.sorted();
        trax_grid_cfg g = grid.config.c();
        uint32_t cap = tripletCandidates.count + 1024u;
        TrackletCollection *t = new TrackletCollection(ctx_, cap, grid.config.nEvents, (uint32_t)lt.size());
        check(ctx_.get(), trax_reset_counts(ctx_.get()), "trax_reset_counts");
        trax_pairs pc = pairs.c(), cc = tripletCandidates.c();
        trax_tracklets tc = t->c();
        trax_status s = trax_triplet_filter(ctx_.get(), &h, &g, &pc, &cc, &tc);
        if (s != TRAX_OK) { delete t; check(ctx_.get(), s, "trax_triplet_filter"); }
        trax_counts k = ctx_.counts();
        t->count = (uint32_t)k.n_tracklets;
        if (k.status != TRAX_OK) { delete t; throw Error((trax_status)k.status, "triplet filter"); }
        return t;
    }
};

class PrefixSum : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    void run(DeviceArray<uint32_t> &input, uint32_t size, unsigned nThreads)
    {
        (void)nThreads;
        check(ctx_.get(), trax_prefix_sum(ctx_.get(), input.data(), input.data(), size, nullptr),
              "trax_prefix_sum");
    }
};

class TripletConnectivity : public KernelWrapper {
public:
    using KernelWrapper::KernelWrapper;
    void run(const TrackletCollection &base, TrackletCollection &following,
             bool iterateBackwards = false, bool tightPacking = false) const
    {
        trax_tracklets b = base.c(), f = following.c();
        check(ctx_.get(), trax_triplet_connectivity(ctx_.get(), &b, base.size(), base.connectivity.data(), &f,
                                                    following.size(), following.connectivity.data(),
                                                    iterateBackwards ? 1 : 0, tightPacking ? 1 : 0),
              "trax_triplet_connectivity");
    }
};

}  // namespace trax

#endif /* TRAX_OPS_HPP */
