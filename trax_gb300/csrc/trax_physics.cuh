/*
 * trax_physics.cuh -- PhysicsRecord::fillData (PhysicsRecord.cpp:81-218) on
 * the GPU for every (event, layer triplet) of a batch.
 *
 * Per tracklet: valid when its three hits carry the same HitId (the
 * simulated track, TrackletCollection.h:121-132); a valid tracklet of a
 * findable track (the event's track list from addEvent) is the track's
 * first find in tracklet order -- "valid" -- or a clone; valid tracklets of
 * other tracks are "misc", the rest fakes.  The first find per (layer
 * triplet, track) is an atomicMin of the tracklet index, so the split
 * matches the reference's std::set insertion in tracklet order.  Each
 * tracklet's pseudorapidity (hits 1, 3) and circle-fit pT (hits 1, 2, 3) are
 * computed in FP64 with the reference's operation order (PhysicsRecord.cpp:
 * 41-79, PhysicsRecord.h:147-171) and returned as histogram bin numbers
 * floor(value / 0.1); findable tracks that no tracklet found ("missed") get
 * theirs from the first, middle and last hit of the track.
 */
#ifndef TRAX_PHYSICS_CUH
#define TRAX_PHYSICS_CUH

#include "trax_kernels.cuh"

namespace trax {

enum : uint8_t { kPhysValid = 0, kPhysClone = 1, kPhysFake = 2, kPhysMisc = 3 };

/* Field order of trax_physics_counts. */
enum { kPcTracklets = 0, kPcValid, kPcClones, kPcFake, kPcMisc, kPcMissed, kPcFindable, kPcN };

/* PhysicsRecord::getEta(inner, outer) (PhysicsRecord.h:147-155): the
 * coordinate differences are float, the rest double. */
__device__ __forceinline__ double phys_eta(float x1, float y1, float z1, float x3, float y3, float z3)
{
    const double px = (double)(x3 - x1), py = (double)(y3 - y1), pz = (double)(z3 - z1);
    const double t = pz / sqrt(px * px + py * py);
    return trax_asinh_d(t);
}

/* getPt(getCircleParams(p1, p2, p3)) (PhysicsRecord.cpp:41-79,
 * PhysicsRecord.h:165-167): paraboloid lift in float, the fit in double. */
__device__ __forceinline__ double phys_pt(float x1, float y1, float x2, float y2, float x3, float y3)
{
    const double P1x = x1, P1y = y1, P1z = (double)(x1 * x1 + y1 * y1);
    const double P2x = x2, P2y = y2, P2z = (double)(x2 * x2 + y2 * y2);
    const double P3x = x3, P3y = y3, P3z = (double)(x3 * x3 + y3 * y3);
    const double ax = P2x - P1x, ay = P2y - P1y, az = P2z - P1z;
    const double bx = P3x - P1x, by = P3y - P1y, bz = P3z - P1z;
    double nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
    const double value = sqrt(nx * nx + ny * ny + nz * nz);
    nx /= value;
    ny /= value;
    nz /= value;
    const double c = -(nx * P1x + ny * P1y + nz * P1z);
    const double radius = sqrt((1 - nz * nz - 4 * c * nz) / (4 * nz * nz));
    const double Q = 1.602177E-19, BZ = 3.8112, GEV_C = 5.344286E-19;
    return Q * BZ * (radius * 1E-2) / GEV_C;
}

__device__ __forceinline__ uint32_t phys_upper(const uint32_t *a, uint32_t n, uint32_t v)
{
    uint32_t lo = 0, hi = n; /* first index with a[i] > v */
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

struct PhysIn {
    const uint32_t *hid;
    const float *x, *y, *z;
    const uint32_t *h1, *h2, *h3, *toff;  /* toff [G + 1] */
    uint32_t n_events, n_lt;
    const uint32_t *mc_id, *mc_in, *mc_mid, *mc_out, *mc_off;  /* mc_off [n_events + 1] */
    const float *rx, *ry, *rz;
};

struct PhysOut {
    uint32_t *first;     /* [n_lt * n_mc] */
    uint32_t *mc_index;  /* [K] */
    uint8_t *cat;        /* [K] */
    double *eta_bin, *pt_bin;          /* [K] */
    double *miss_eta_bin, *miss_pt_bin;  /* [n_lt * n_mc] */
    uint8_t *missed;                     /* [n_lt * n_mc] */
    uint32_t *counts;    /* [G][kPcN] */
};

__global__ void __launch_bounds__(256) k_phys_tracklets(PhysIn in, PhysOut out)
{
    const uint32_t G = in.n_events * in.n_lt;
    const uint32_t K = in.toff[G];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        const uint32_t g = phys_upper(in.toff, G + 1, i) - 1;
        const uint32_t e = g / in.n_lt, lt = g % in.n_lt;
        const uint32_t a = in.h1[i], b = in.h2[i], c = in.h3[i];
        const double eta = phys_eta(in.x[a], in.y[a], in.z[a], in.x[c], in.y[c], in.z[c]);
        const double pt = phys_pt(in.x[a], in.y[a], in.x[b], in.y[b], in.x[c], in.y[c]);
        out.eta_bin[i] = floor(eta / 0.1);
        out.pt_bin[i] = floor(pt / 0.1);
        const uint32_t t = in.hid[a];
        uint32_t k = 0xFFFFFFFFu;
        uint8_t cat = kPhysFake;
        if (t == in.hid[b] && t == in.hid[c]) {
            cat = kPhysMisc;
            const uint32_t lo = in.mc_off[e], hi = in.mc_off[e + 1];
            const uint32_t j = lo + phys_upper(in.mc_id + lo, hi - lo, t);
            if (j > lo && in.mc_id[j - 1] == t) {
                k = j - 1;
                cat = kPhysValid;
                atomicMin(&out.first[(size_t)lt * in.mc_off[in.n_events] + k], i);
            }
        }
        out.mc_index[i] = k;
        out.cat[i] = cat;
    }
}

__global__ void __launch_bounds__(256) k_phys_classify(PhysIn in, PhysOut out)
{
    const uint32_t G = in.n_events * in.n_lt;
    const uint32_t K = in.toff[G];
    const uint32_t n_mc = in.mc_off[in.n_events];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
        const uint32_t g = phys_upper(in.toff, G + 1, i) - 1;
        const uint32_t lt = g % in.n_lt;
        uint8_t cat = out.cat[i];
        const uint32_t k = out.mc_index[i];
        if (k != 0xFFFFFFFFu) {
            cat = out.first[(size_t)lt * n_mc + k] == i ? kPhysValid : kPhysClone;
            out.cat[i] = cat;
        }
        const int field = cat == kPhysValid ? kPcValid : cat == kPhysClone ? kPcClones
                        : cat == kPhysFake ? kPcFake : kPcMisc;
        atomicAdd(&out.counts[(size_t)g * kPcN + field], 1u);
        atomicAdd(&out.counts[(size_t)g * kPcN + kPcTracklets], 1u);
    }
}

__global__ void __launch_bounds__(256) k_phys_missed(PhysIn in, PhysOut out)
{
    const uint32_t n_mc = in.mc_off[in.n_events];
    const uint32_t total = in.n_lt * n_mc;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        const uint32_t lt = q / n_mc, k = q % n_mc;
        const uint32_t e = phys_upper(in.mc_off, in.n_events + 1, k) - 1;
        const uint32_t g = e * in.n_lt + lt;
        atomicAdd(&out.counts[(size_t)g * kPcN + kPcFindable], 1u);
        double eb = 0.0, pb = 0.0;
        const bool miss = out.first[q] == 0xFFFFFFFFu;
        if (miss) {
            atomicAdd(&out.counts[(size_t)g * kPcN + kPcMissed], 1u);
            const uint32_t a = in.mc_in[k], m = in.mc_mid[k], c = in.mc_out[k];
            eb = floor(phys_eta(in.rx[a], in.ry[a], in.rz[a], in.rx[c], in.ry[c], in.rz[c]) / 0.1);
            pb = floor(phys_pt(in.rx[a], in.ry[a], in.rx[m], in.ry[m], in.rx[c], in.ry[c]) / 0.1);
        }
        out.miss_eta_bin[q] = eb;
        out.miss_pt_bin[q] = pb;
        out.missed[q] = miss ? 1 : 0;
    }
}

}  // namespace trax

#endif /* TRAX_PHYSICS_CUH */
