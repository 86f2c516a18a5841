/*
 * Runs the reference's operator chain (TripletBuilder.cpp:234-300: grid
 * build, beam-spot pairs, theta/phi prediction, theta/phi filter, then
 * TripletConnectivity) through include/trax_ops.hpp and writes every
 * collection to a file, for the GPU test that compares them with the golden
 * vectors.
 *
 * usage: ops_chain <input> <output> [beamspot|sector]
 * input  (little-endian): u32 n_hits, n_events, n_layers, n_sectors_z,
 *        n_sectors_phi, n_layer_triplets, n_geom_layers; f32 min_pt;
 *        f32 x, y, z [n_hits]; u32 layer, detector_id, hit_id, event
 *        [n_hits]; u32 layer_nhits [n_events * n_layers];
 *        trax_layer_triplet [n_layer_triplets]; f32 min_radius, max_radius
 *        [n_geom_layers]
 * output: a sequence of (u32 length, u32 words[length]) records: grid,
 *         input positions of the sorted hits, pairs, pair offsets,
 *         candidates, candidate offsets, hit1, hit2, hit3, tracklet offsets,
 *         connectivity of the tracklets following themselves.
 */
#include <cstdio>
#include <cstring>
#include <memory>

#include "trax_ops.hpp"

namespace {

struct Reader {
    FILE *f;
    template <class T>
    std::vector<T> get(size_t n)
    {
        std::vector<T> v(n);
        if (n && fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short input");
        return v;
    }
    uint32_t u32() { return get<uint32_t>(1)[0]; }
};

void put(FILE *f, const std::vector<uint32_t> &v)
{
    uint32_t n = (uint32_t)v.size();
    fwrite(&n, 4, 1, f);
    if (n) fwrite(v.data(), 4, n, f);
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 4) {
        fprintf(stderr, "usage: %s <input> <output> [beamspot|sector]\n", argv[0]);
        return 2;
    }
    const bool sector = argc == 4 && strcmp(argv[3], "sector") == 0;
    try {
        FILE *fi = fopen(argv[1], "rb");
        if (!fi) throw std::runtime_error("cannot open input");
        Reader r{fi};
        uint32_t n = r.u32(), ne = r.u32(), nl = r.u32(), nz = r.u32(), nphi = r.u32(),
                 nlt = r.u32(), ngeom = r.u32();
        float min_pt = r.get<float>(1)[0];
        auto x = r.get<float>(n), y = r.get<float>(n), z = r.get<float>(n);
        auto layer = r.get<uint32_t>(n), det = r.get<uint32_t>(n), hid = r.get<uint32_t>(n),
             ev = r.get<uint32_t>(n);
        auto layer_nhits = r.get<uint32_t>((size_t)ne * nl);
        auto rows = r.get<trax_layer_triplet>(nlt);
        trax::GeometrySupplement geom{r.get<float>(ngeom), r.get<float>(ngeom)};
        fclose(fi);

        trax::EventSupplement es;
        trax::LayerSupplement ls;
        ls.nLayers = nl;
        uint32_t off = 0;
        for (uint32_t e = 0; e < ne; ++e) {
            uint32_t within = 0;
            for (uint32_t l = 0; l < nl; ++l) {
                ls.nHits.push_back(layer_nhits[(size_t)e * nl + l]);
                ls.offset.push_back(within);
                within += layer_nhits[(size_t)e * nl + l];
            }
            es.nHits.push_back(within);
            es.offset.push_back(off);
            off += within;
        }

        trax::TripletConfigurations lt(min_pt);
        lt.rows = rows;

        trax::Context ctx(0);
        trax::HitCollection hits(ctx, x, y, z, layer, det, hid, ev);
        trax::Grid grid(ctx, trax::GridConfig{ne, nl, nz, nphi});
        trax::GridBuilder(ctx).run(hits, 256, es, ls, grid);
        std::unique_ptr<trax::Pairing> pairs(
            sector ? trax::PairGeneratorSector(ctx).run(hits, geom, 256, lt, grid)
                   : trax::PairGeneratorBeamspot(ctx).run(hits, geom, 256, lt, grid));
        std::unique_ptr<trax::Pairing> cands(trax::TripletThetaPhiPredictor(ctx).run(
            hits, nullptr, geom, nullptr, 256, lt, grid, *pairs));
        std::unique_ptr<trax::TrackletCollection> trk(
            trax::TripletThetaPhiFilter(ctx).run(hits, grid, *pairs, *cands, 256, lt));

        std::vector<uint32_t> h1 = trk->hit1.download(trk->size()),
                              h2 = trk->hit2.download(trk->size()),
                              h3 = trk->hit3.download(trk->size());
        trax::TrackletCollection follow(ctx, h1, h2, h3);
        trax::TripletConnectivity(ctx).run(*trk, follow);
        ctx.synchronize();

        FILE *fo = fopen(argv[2], "wb");
        if (!fo) throw std::runtime_error("cannot open output");
        put(fo, grid.download());
        put(fo, hits.inputPositions());
        put(fo, pairs->getPairings());
        put(fo, pairs->getPairingOffsets());
        put(fo, cands->getPairings());
        put(fo, cands->getPairingOffsets());
        put(fo, h1);
        put(fo, h2);
        put(fo, h3);
        put(fo, trk->getTrackletOffsets());
        put(fo, follow.connectivity.download(follow.size()));
        fclose(fo);
    } catch (const std::exception &e) {
        fprintf(stderr, "ops_chain: %s\n", e.what());
        return 1;
    }
    return 0;
}
