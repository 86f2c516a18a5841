/*
 * trax_physics.cpp -- host side of the physics evaluation: PhysicsRecord /
 * PhysicsRecords (PhysicsRecord.h:46-186, PhysicsRecord.cpp:10-39,81-218,
 * 220-368) fed with the per-tracklet classes and histogram bins the GPU
 * computed (trax_physics.cuh).
 *
 * The arithmetic keeps the reference's types and order: per-record rates in
 * double stored to long double, merges in long double with uint weights,
 * Utils::clamp on int, histograms as std::map<double, tBinnedData> filled in
 * tracklet order then missed-track order (so even NaN keys land where the
 * reference's map puts them).  Two reference behaviours are kept as they
 * are: tBinnedData::operator+= does not add `misc`, and merging a histogram
 * bin into an empty map first default-constructs it with n = 1.
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/trax.h"

namespace {

constexpr char SEP = ' ';

unsigned clamp_n(int n) { return n > 0 ? (unsigned)n : 1u; }  /* Utils::clamp (utils.h:65-67) */

template <class T>
std::string csv(std::initializer_list<T> args)
{
    std::stringstream s;
    for (auto it = args.begin(); it != args.end(); ++it) {
        s << *it;
        if (it + 1 != args.end()) s << SEP;
    }
    return s.str();
}

struct Binned {  /* tBinnedData */
    unsigned valid = 0, clones = 0, fake = 0, missed = 0, misc = 0;
    long double efficiencyMean = 0, efficiencyVar = 0, fakeRateMean = 0, fakeRateVar = 0,
                cloneRateMean = 0, cloneRateVar = 0;
    unsigned n = 1;

    void fill()
    {
        efficiencyMean = ((double)valid) / clamp_n((int)(valid + missed));
        fakeRateMean = ((double)fake / clamp_n((int)(valid + fake + clones + misc)));
        cloneRateMean = ((double)clones / clamp_n((int)(valid + fake + clones + misc)));
        n = valid + fake + clones + misc;
    }
    long double toVar(long double x) const { return n > 1 ? std::sqrt(x / clamp_n((int)(n - 1))) : 0; }
    void add(const Binned &c)
    {
        valid += c.valid;
        clones += c.clones;
        fake += c.fake;
        missed += c.missed;
        n += c.n;
        long double delta = c.efficiencyMean - efficiencyMean;
        efficiencyMean += (c.valid + c.missed) * delta / clamp_n((int)(valid + missed));
        efficiencyVar += (c.valid + c.missed) * delta * (c.efficiencyMean - efficiencyMean) + c.efficiencyVar;
        delta = c.fakeRateMean - fakeRateMean;
        fakeRateMean += c.n * delta / clamp_n((int)n);
        fakeRateVar += c.n * delta * (c.fakeRateMean - fakeRateMean) + c.fakeRateVar;
        delta = c.cloneRateMean - cloneRateMean;
        cloneRateMean += c.n * delta / clamp_n((int)n);
        cloneRateVar += c.n * delta * (c.cloneRateMean - cloneRateMean) + c.cloneRateVar;
    }
    std::string dump() const
    {
        std::stringstream s;
        s << csv<unsigned>({valid, fake, clones, missed, misc}) << SEP
          << csv<long double>({efficiencyMean, toVar(efficiencyVar), fakeRateMean, toVar(fakeRateVar),
                               cloneRateMean, toVar(cloneRateVar)});
        return s.str();
    }
};

struct Histogram {  /* tHistogram */
    double binWidth;
    std::map<double, Binned> bins;
    explicit Histogram(double w) : binWidth(w) {}
    void fill()
    {
        for (auto &t : bins) t.second.fill();
    }
    void merge(const Histogram &t2)  /* mergeHistograms (PhysicsRecord.cpp:220-230) */
    {
        for (const auto &t : t2.bins) {
            if (binWidth == t2.binWidth) {
                bins[t.first].add(t.second);
            } else {
                double bin = t.first * t2.binWidth + t2.binWidth / 2;
                bin = binWidth * std::floor(bin / binWidth);
                bins[bin].add(t.second);
            }
        }
    }
    std::string dump() const
    {
        std::stringstream s;
        s << "bin valid fake clones missed misc efficiencyMean efficiencyVar fakeRateMean "
             "fakeRateVar cloneRateMean cloneRateVar"
          << std::endl;
        for (const auto &b : bins) s << b.first << SEP << b.second.dump() << std::endl;
        return s.str();
    }
};

struct Record {  /* PhysicsRecord */
    unsigned event, layerTriplet;
    long double efficiencyMean = 0, efficiencyVar = 0, fakeRateMean = 0, fakeRateVar = 0,
                cloneRateMean = 0, cloneRateVar = 0;
    unsigned n = 1;
    Histogram pt{0.1}, eta{0.1};

    Record(unsigned e, unsigned lt) : event(e), layerTriplet(lt) {}
    long double toVar(long double x) const { return n > 1 ? std::sqrt(x / clamp_n((int)(n - 1))) : 0; }
    void merge(const Record &c)
    {
        eta.merge(c.eta);
        pt.merge(c.pt);
        n += c.n;
        long double delta = c.efficiencyMean - efficiencyMean;
        efficiencyMean += c.n * delta / clamp_n((int)n);
        efficiencyVar += c.n * delta * (c.efficiencyMean - efficiencyMean) + c.efficiencyVar;
        delta = c.fakeRateMean - fakeRateMean;
        fakeRateMean += c.n * delta / clamp_n((int)n);
        fakeRateVar += c.n * delta * (c.fakeRateMean - fakeRateMean) + c.fakeRateVar;
        delta = c.cloneRateMean - cloneRateMean;
        cloneRateMean += c.n * delta / clamp_n((int)n);
        cloneRateVar += c.n * delta * (c.cloneRateMean - cloneRateMean) + c.cloneRateVar;
    }
    std::string dump() const
    {
        std::stringstream s;
        s << csv<unsigned>({layerTriplet, n}) << SEP
          << csv<long double>({efficiencyMean, toVar(efficiencyVar)}) << SEP
          << csv<long double>({fakeRateMean, toVar(fakeRateVar)}) << SEP
          << csv<long double>({cloneRateMean, toVar(cloneRateVar)});
        return s.str();
    }
};

}  // namespace

struct trax_physics {  /* PhysicsRecords */
    std::vector<Record> records;

    void add(const Record &r)
    {
        for (auto &q : records)
            if (q.layerTriplet == r.layerTriplet) {
                q.merge(r);
                return;
            }
        records.push_back(r);
    }
    /* the merged total csvDump prints last (PhysicsRecord.cpp:336-352) */
    Record total() const
    {
        Record t(records[0]);
        t.layerTriplet = (unsigned)records.size() + 1;
        for (size_t i = 1; i < records.size(); ++i) t.merge(records[i]);
        return t;
    }
    std::string dump() const
    {
        std::stringstream s;
        s << "layerTriplet n eff effVar fr frVar cr crVar" << std::endl;
        if (records.empty()) return s.str();
        for (const auto &r : records) s << r.dump() << std::endl;
        s << total().dump() << std::endl;
        return s.str();
    }
};

extern "C" {

trax_status trax_physics_create(trax_physics **out)
{
    if (!out) return TRAX_ERR_BAD_ARG;
    *out = new (std::nothrow) trax_physics();
    return *out ? TRAX_OK : TRAX_ERR_OOM;
}

void trax_physics_destroy(trax_physics *p) { delete p; }

/* PhysicsRecord::fillData for group (event, lt) from host arrays; called by
 * trax_physics_eval after the GPU pass. */
trax_status trax_physics_add_group(trax_physics *p, uint32_t event, uint32_t lt,
                                   const trax_physics_counts *c, const uint8_t *cat,
                                   const double *eta_bin, const double *pt_bin, uint32_t n_trk,
                                   const double *miss_eta_bin, const double *miss_pt_bin,
                                   uint32_t n_missed)
{
    if (!p || !c) return TRAX_ERR_BAD_ARG;
    Record r(event, lt);
    for (uint32_t i = 0; i < n_trk; ++i) {
        const double ek = r.eta.binWidth * eta_bin[i], pk = r.pt.binWidth * pt_bin[i];
        switch (cat[i]) {
        case 0: r.eta.bins[ek].valid++; r.pt.bins[pk].valid++; break;
        case 1: r.eta.bins[ek].clones++; r.pt.bins[pk].clones++; break;
        case 2: r.eta.bins[ek].fake++; r.pt.bins[pk].fake++; break;
        default: r.eta.bins[ek].misc++; r.pt.bins[pk].misc++; break;
        }
    }
    for (uint32_t i = 0; i < n_missed; ++i) {
        r.eta.bins[r.eta.binWidth * miss_eta_bin[i]].missed++;
        r.pt.bins[r.pt.binWidth * miss_pt_bin[i]].missed++;
    }
    r.efficiencyMean = ((double)c->valid) / clamp_n((int)c->findable);
    r.fakeRateMean = ((double)c->fake) / clamp_n((int)c->tracklets);
    r.cloneRateMean = ((double)c->clones) / clamp_n((int)c->tracklets);
    r.eta.fill();
    r.pt.fill();
    p->add(r);
    return TRAX_OK;
}

uint32_t trax_physics_n_records(const trax_physics *p) { return p ? (uint32_t)p->records.size() : 0; }

trax_status trax_physics_csv(const trax_physics *p, int what, uint32_t layer_triplet, char *buf,
                             size_t cap, size_t *len)
{
    if (!p || !len || what < 0 || what > 2) return TRAX_ERR_BAD_ARG;
    std::string s;
    if (what == 0) {
        s = p->dump();
    } else {
        if (p->records.empty()) return TRAX_ERR_BAD_ARG;
        const Record *r = nullptr;
        Record tot = p->total();
        if (layer_triplet == tot.layerTriplet) r = &tot;
        for (const auto &q : p->records)
            if (!r && q.layerTriplet == layer_triplet) r = &q;
        if (!r) return TRAX_ERR_BAD_ARG;
        s = what == 1 ? r->eta.dump() : r->pt.dump();
    }
    *len = s.size();
    if (buf && cap) {
        const size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(buf, s.data(), n);
        buf[n] = 0;
        if (s.size() >= cap) return TRAX_ERR_CAPACITY;
    }
    return TRAX_OK;
}

}  // extern "C"
