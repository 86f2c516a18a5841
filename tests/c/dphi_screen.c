/*
 * The filter's dphi screen (trax_dphi_screen in trax_math.h) against the
 * cut it stands in for (TripletThetaPhiFilter.h:86-99, evaluated with the
 * same trax_atan2f as the kernels): on every case where the screen decides,
 * its answer must equal the cut's.  Cases: hits on barrel layers at random
 * radii and angles, triplets built to sit within 1e-4 rad of the cut (the
 * screen's undecided band is 2e-5 wide on each side), degenerate and
 * non-finite vectors.  Prints "cases N undecided U mismatches M" and the
 * same for the random triplets under the cuts the screen serves.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#define PI 3.14159265358979323846

#include "trax_math.h"

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;

static uint64_t next_u64(void)
{
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double uniform(double lo, double hi)
{
    return lo + (hi - lo) * (double)(next_u64() >> 11) * 0x1p-53;
}

/* The cut as the kernels evaluate it without the screen. */
static int exact_cut(float x1, float y1, float x2, float y2, float x3, float y3, float cut)
{
    const float angle1 = trax_atan2f((y2 - y1), (x2 - x1));
    const float angle2 = trax_atan2f((y3 - y2), (x3 - x2));
    float delta = angle2 - angle1;
    delta += (delta > TRAX_PI_F) ? -2 * TRAX_PI_F : (delta < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
    return fabsf(delta) <= cut;
}

static long cases, undecided, mismatches;

static int check(float x1, float y1, float x2, float y2, float x3, float y3, float cut)
{
    float tlo, thi;
    trax_dphi_screen_bounds(cut, &tlo, &thi);
    const int s = trax_dphi_screen(x2 - x1, y2 - y1, x3 - x2, y3 - y2, tlo, thi);
    const int e = exact_cut(x1, y1, x2, y2, x3, y3, cut);
    ++cases;
    if (s < 0) {
        ++undecided;
    } else if (s != e) {
        if (mismatches < 10)
            printf("MISMATCH cut %.9g hits (%.9g %.9g) (%.9g %.9g) (%.9g %.9g) screen %d cut %d\n",
                   cut, x1, y1, x2, y2, x3, y3, s, e);
        ++mismatches;
    }
    return s;
}

int main(void)
{
    static const float cuts[] = {0.001f, 0.0035f, 0.01f, 0.03f, 0.05f, 0.1f, 0.3f, 0.7f, 1.0f,
                                 0.00008f, 1.2f, 2.0f};
    const int ncuts = (int)(sizeof cuts / sizeof cuts[0]);
    /* random triplets on three barrel layers */
    long active = 0, active_undecided = 0;
    for (long i = 0; i < 3000000; ++i) {
        const float cut = cuts[i % ncuts];
        const double r1 = uniform(2, 6), r2 = r1 + uniform(1, 5), r3 = r2 + uniform(1, 8);
        const double p1 = uniform(-PI, PI);
        const double p2 = p1 + uniform(-0.3, 0.3), p3 = p2 + uniform(-0.3, 0.3);
        const int d = check((float)(r1 * cos(p1)), (float)(r1 * sin(p1)), (float)(r2 * cos(p2)),
                            (float)(r2 * sin(p2)), (float)(r3 * cos(p3)), (float)(r3 * sin(p3)),
                            cut);
        if (i % ncuts < 9) {  /* cuts the screen serves */
            ++active;
            active_undecided += d < 0;
        }
    }
    /* triplets whose bend sits within 1e-4 rad of the cut, either side */
    for (long i = 0; i < 3000000; ++i) {
        const float cut = cuts[i % 9];
        const double x1 = uniform(-10, 10), y1 = uniform(-10, 10);
        const double a = uniform(-PI, PI), l1 = uniform(0.5, 10), l2 = uniform(0.5, 10);
        const double bend = ((next_u64() & 1) ? 1 : -1) * (cut + uniform(-1e-4, 1e-4));
        const double x2 = x1 + l1 * cos(a), y2 = y1 + l1 * sin(a);
        const double x3 = x2 + l2 * cos(a + bend), y3 = y2 + l2 * sin(a + bend);
        check((float)x1, (float)y1, (float)x2, (float)y2, (float)x3, (float)y3, cut);
    }
    /* bends near +-pi, short and long vectors, huge and tiny coordinates */
    for (long i = 0; i < 1000000; ++i) {
        const float cut = cuts[i % ncuts];
        const double sc = pow(2.0, uniform(-60, 70));
        const double x1 = uniform(-1, 1) * sc, y1 = uniform(-1, 1) * sc;
        const double a = uniform(-PI, PI), bend = uniform(-PI, PI);
        const double l1 = uniform(0, 2) * sc * pow(2.0, uniform(-30, 0)), l2 = uniform(0, 2) * sc;
        const double x2 = x1 + l1 * cos(a), y2 = y1 + l1 * sin(a);
        const double x3 = x2 + l2 * cos(a + bend), y3 = y2 + l2 * sin(a + bend);
        check((float)x1, (float)y1, (float)x2, (float)y2, (float)x3, (float)y3, cut);
    }
    /* coincident hits, collinear, NaN and infinity */
    const float inf = INFINITY, nan = NAN;
    const float special[][6] = {{1, 1, 1, 1, 2, 2},   {1, 1, 2, 2, 2, 2},   {0, 0, 1, 0, 2, 0},
                                {0, 0, 1, 0, 0, 0},   {0, 0, 1, 0, -1, 0},  {nan, 0, 1, 0, 2, 0},
                                {0, 0, inf, 0, 2, 0}, {0, 0, 1, 0, 2, inf}, {0, 0, 1, 1e-30f, 2, 0},
                                {0, 0, 1e-30f, 0, 2e-30f, 1e-31f}};
    for (int k = 0; k < (int)(sizeof special / sizeof special[0]); ++k)
        for (int c = 0; c < ncuts; ++c)
            check(special[k][0], special[k][1], special[k][2], special[k][3], special[k][4],
                  special[k][5], cuts[c]);
    printf("cases %ld undecided %ld mismatches %ld\n", cases, undecided, mismatches);
    printf("served %ld undecided %ld\n", active, active_undecided);
    return mismatches != 0;
}
