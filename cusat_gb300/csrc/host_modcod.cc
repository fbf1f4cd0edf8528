// Constellations, bit interleaver and demapper parameters of the DVB-S2/S2X
// MODCODs, plus the product-side mapper for generated traffic.
//
// The ring ratios, angles and label assignments are those of ETSI EN 302
// 307-1 clause 5.4 and EN 302 307-2 clause 5.4 as the reference builds them
// (lib/cusat_dsp/modulation/constellation.cc); every point is produced with
// the same float/double arithmetic so that the points are bit-identical to
// the reference's (checked against the reference host code in the tests).
#include <stdlib.h>
#include <math.h>

#include <cmath>
#include <string.h>

#include <algorithm>

#include "host.h"

extern "C" {
#include "cusat_data.h"
}

namespace cusat {

namespace {

#include "gen/apsk256_points.inc"

constexpr double kPi = 3.14159265358979323846;

void put(std::vector<float>* p, int label, float re, float im)
{
    (*p)[2 * label] = re;
    (*p)[2 * label + 1] = im;
}

void polar(std::vector<float>* p, int label, double radius, double angle)
{
    put(p, label, (float)(radius * cos(angle)), (float)(radius * sin(angle)));
}

// angle k pi / d evaluated in single precision (S2 16/32APSK)
void s2_point(std::vector<float>* p, int label, float radius, int k, int d)
{
    const float pi = (float)kPi;
    const float angle = (float)(k * (double)pi / d);
    put(p, label, radius * cosf(angle), radius * sinf(angle));
}

float gamma_16apsk(int rate)
{
    switch (rate) {
    case CUSAT_RATE_2_3: return 3.15f;
    case CUSAT_RATE_3_4: return 2.85f;
    case CUSAT_RATE_4_5: return 2.75f;
    case CUSAT_RATE_5_6: return 2.70f;
    case CUSAT_RATE_8_9: return 2.60f;
    case CUSAT_RATE_9_10: return 2.57f;
    case CUSAT_RATE_26_45: return 3.7f;
    case CUSAT_RATE_3_5: return 3.7f;
    case CUSAT_RATE_28_45: return 3.5f;
    case CUSAT_RATE_23_36: return 3.1f;
    case CUSAT_RATE_25_36: return 3.1f;
    case CUSAT_RATE_13_18: return 2.85f;
    case CUSAT_RATE_140_180: return 3.6f;
    case CUSAT_RATE_154_180: return 3.2f;
    case CUSAT_RATE_7_15: return 3.32f;
    case CUSAT_RATE_8_15: return 3.50f;
    default: return 2.85f;
    }
}

struct RingK { int ring, k, d; };

void build_16apsk_4_12(std::vector<float>* p, int rate)
{
    // 4+12APSK: label -> (ring, angle k pi / d)
    static const RingK L[16] = {
        {1, 1, 4}, {1, -1, 4}, {1, 3, 4}, {1, -3, 4}, {1, 1, 12}, {1, -1, 12}, {1, 11, 12}, {1, -11, 12},
        {1, 5, 12}, {1, -5, 12}, {1, 7, 12}, {1, -7, 12}, {0, 1, 4}, {0, -1, 4}, {0, 3, 4}, {0, -3, 4},
    };
    const float g = gamma_16apsk(rate);
    const float r1 = (float)sqrt(16.0 / (4.0 + 12.0 * g * g));
    const float radius[2] = {r1, g * r1};
    for (int l = 0; l < 16; l++)
        s2_point(p, l, radius[L[l].ring], L[l].k, L[l].d);
}

void build_16apsk_8_8(std::vector<float>* p, int rate)
{
    static const double C18[16][2] = {
        {0.4718, 0.2606}, {0.2606, 0.4718}, {-0.4718, 0.2606}, {-0.2606, 0.4718},
        {0.4718, -0.2606}, {0.2606, -0.4718}, {-0.4718, -0.2606}, {-0.2606, -0.4718},
        {1.2088, 0.4984}, {0.4984, 1.2088}, {-1.2088, 0.4984}, {-0.4984, 1.2088},
        {1.2088, -0.4984}, {0.4984, -1.2088}, {-1.2088, -0.4984}, {-0.4984, -1.2088},
    };
    static const double C20[16][2] = {
        {0.5061, 0.2474}, {0.2474, 0.5061}, {-0.5061, 0.2474}, {-0.2474, 0.5061},
        {0.5061, -0.2474}, {0.2474, -0.5061}, {-0.5061, -0.2474}, {-0.2474, -0.5061},
        {1.2007, 0.4909}, {0.4909, 1.2007}, {-1.2007, 0.4909}, {-0.4909, 1.2007},
        {1.2007, -0.4909}, {0.4909, -1.2007}, {-1.2007, -0.4909}, {-0.4909, -1.2007},
    };
    const double(*c)[2] = rate == CUSAT_RATE_18_30 ? C18 : rate == CUSAT_RATE_20_30 ? C20 : nullptr;
    if (c) {
        double e = 0.0;
        for (int i = 0; i < 16; i++)
            e += c[i][0] * c[i][0] + c[i][1] * c[i][1];
        const double s = sqrt(16.0 / e);
        for (int i = 0; i < 16; i++)
            put(p, i, (float)(c[i][0] * s), (float)(c[i][1] * s));
        return;
    }
    const double g = 2.19;
    const double r1 = sqrt(2.0 / (1.0 + g * g));
    static const int NN[2][2][2] = {{{1, 15}, {7, 9}}, {{3, 13}, {5, 11}}};
    for (int l = 0; l < 16; l++) {
        const int ring = (l >> 3) & 1, qq = (l >> 2) & 1, pp = (l >> 1) & 1, b0 = l & 1;
        polar(p, l, ring ? g * r1 : r1, NN[b0][pp][qq] * (kPi / 8.0));
    }
}

void build_32apsk_4_12_16(std::vector<float>* p, int rate)
{
    double g1 = 2.84, g2 = 5.27;
    switch (rate) {
    case CUSAT_RATE_4_5: g1 = 2.72; g2 = 4.87; break;
    case CUSAT_RATE_5_6: g1 = 2.64; g2 = 4.64; break;
    case CUSAT_RATE_8_9: g1 = 2.54; g2 = 4.33; break;
    case CUSAT_RATE_9_10: g1 = 2.53; g2 = 4.30; break;
    default: break;
    }
    const double r1 = sqrt(8.0 / (1.0 + 3.0 * g1 * g1 + 4.0 * g2 * g2));
    const float radius[3] = {(float)r1, (float)(g1 * r1), (float)(g2 * r1)};
    static const RingK L[32] = {
        {1, 1, 4}, {1, 5, 12}, {1, -1, 4}, {1, -5, 12}, {1, 3, 4}, {1, 7, 12}, {1, -3, 4}, {1, -7, 12},
        {2, 1, 8}, {2, 3, 8}, {2, -1, 4}, {2, -1, 2}, {2, 3, 4}, {2, 1, 2}, {2, -7, 8}, {2, -5, 8},
        {1, 1, 12}, {0, 1, 4}, {1, -1, 12}, {0, -1, 4}, {1, 11, 12}, {0, 3, 4}, {1, -11, 12}, {0, -3, 4},
        {2, 0, 1}, {2, 1, 4}, {2, -1, 8}, {2, -3, 8}, {2, 7, 8}, {2, 5, 8}, {2, 1, 1}, {2, -3, 4},
    };
    for (int l = 0; l < 32; l++)
        s2_point(p, l, radius[L[l].ring], L[l].k, L[l].d);
}

void build_32apsk_rb(std::vector<float>* p, int rate, int framesize)
{
    double g1 = 2.85, g2 = 5.55;
    if (rate == CUSAT_RATE_32_45) {
        g1 = 2.839;
        g2 = 5.258;
    } else if (framesize == CUSAT_FECFRAME_SHORT) {
        g1 = 2.84;
        g2 = 5.54;
    }
    const double r1 = sqrt(32.0 / (4.0 + 12.0 * g1 * g1 + 16.0 * g2 * g2));
    const double radius[4] = {0.0, r1, g1 * r1, g2 * r1};
    static const int RING[8] = {3, 3, 2, 2, 3, 3, 2, 1};
    static const double A[8][4] = {
        {11.0 / 16, 5.0 / 16, 21.0 / 16, 27.0 / 16}, {9.0 / 16, 7.0 / 16, 23.0 / 16, 25.0 / 16},
        {3.0 / 4, 1.0 / 4, 5.0 / 4, 7.0 / 4}, {7.0 / 12, 5.0 / 12, 17.0 / 12, 19.0 / 12},
        {13.0 / 16, 3.0 / 16, 19.0 / 16, 29.0 / 16}, {15.0 / 16, 1.0 / 16, 17.0 / 16, 31.0 / 16},
        {11.0 / 12, 1.0 / 12, 13.0 / 12, 23.0 / 12}, {3.0 / 4, 1.0 / 4, 5.0 / 4, 7.0 / 4},
    };
    for (int l = 0; l < 32; l++) {
        const int row = (((l >> 3) & 1) << 2) | (((l >> 2) & 1) << 1) | (l & 1);
        const int col = (((l >> 4) & 1) << 1) | ((l >> 1) & 1);
        polar(p, l, radius[RING[row]], A[row][col] * kPi);
    }
}

void build_32apsk_4_8_4_16(std::vector<float>* p, int rate)
{
    double g1 = 2.6, g2 = 2.99, g3 = 5.6;
    switch (rate) {
    case CUSAT_RATE_132_180: g2 = 2.86; break;
    case CUSAT_RATE_7_9:
    case CUSAT_RATE_140_180: g1 = 2.8; g2 = 3.08; break;
    case CUSAT_RATE_32_45: g1 = 2.84; g2 = 2.84; g3 = 5.26; break;
    default: break;
    }
    const double r1 = sqrt(32.0 / (4.0 + 8.0 * g1 * g1 + 4.0 * g2 * g2 + 16.0 * g3 * g3));
    const double radius[5] = {0.0, r1, g1 * r1, g2 * r1, g3 * r1};
    static const int RING[8] = {1, 4, 2, 4, 2, 4, 3, 4};
    static const double A[8][4] = {
        {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}, {7.0 / 16, 25.0 / 16, 9.0 / 16, 23.0 / 16},
        {1.0 / 12, 23.0 / 12, 11.0 / 12, 13.0 / 12}, {1.0 / 16, 31.0 / 16, 15.0 / 16, 17.0 / 16},
        {5.0 / 12, 19.0 / 12, 7.0 / 12, 17.0 / 12}, {5.0 / 16, 27.0 / 16, 11.0 / 16, 21.0 / 16},
        {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}, {3.0 / 16, 29.0 / 16, 13.0 / 16, 19.0 / 16},
    };
    for (int l = 0; l < 32; l++) {
        const int row = (((l >> 4) & 1) << 2) | (((l >> 3) & 1) << 1) | (l & 1);
        const int col = (((l >> 2) & 1) << 1) | ((l >> 1) & 1);
        polar(p, l, radius[RING[row]], A[row][col] * kPi);
    }
}

struct RingRow { int ring; double a[4]; };

void build_64apsk(std::vector<float>* p, int rate)
{
    static const RingRow RA[16] = {
        {3, {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}}, {3, {13.0 / 28, 43.0 / 28, 15.0 / 28, 41.0 / 28}},
        {3, {1.0 / 28, 55.0 / 28, 27.0 / 28, 29.0 / 28}}, {0, {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}},
        {3, {9.0 / 28, 47.0 / 28, 19.0 / 28, 37.0 / 28}}, {3, {11.0 / 28, 45.0 / 28, 17.0 / 28, 39.0 / 28}},
        {2, {1.0 / 20, 39.0 / 20, 19.0 / 20, 21.0 / 20}}, {1, {1.0 / 12, 23.0 / 12, 11.0 / 12, 13.0 / 12}},
        {3, {5.0 / 28, 51.0 / 28, 23.0 / 28, 33.0 / 28}}, {2, {9.0 / 20, 31.0 / 20, 11.0 / 20, 29.0 / 20}},
        {3, {3.0 / 28, 53.0 / 28, 25.0 / 28, 31.0 / 28}}, {1, {5.0 / 12, 19.0 / 12, 7.0 / 12, 17.0 / 12}},
        {2, {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}}, {2, {7.0 / 20, 33.0 / 20, 13.0 / 20, 27.0 / 20}},
        {2, {3.0 / 20, 37.0 / 20, 17.0 / 20, 23.0 / 20}}, {1, {1.0 / 4, 7.0 / 4, 3.0 / 4, 5.0 / 4}},
    };
    static const RingRow RB[16] = {
        {1, {25.0 / 16, 23.0 / 16, 7.0 / 16, 9.0 / 16}}, {3, {7.0 / 4, 5.0 / 4, 1.0 / 4, 3.0 / 4}},
        {1, {27.0 / 16, 21.0 / 16, 5.0 / 16, 11.0 / 16}}, {2, {7.0 / 4, 5.0 / 4, 1.0 / 4, 3.0 / 4}},
        {3, {31.0 / 20, 29.0 / 20, 9.0 / 20, 11.0 / 20}}, {3, {33.0 / 20, 27.0 / 20, 7.0 / 20, 13.0 / 20}},
        {2, {31.0 / 20, 29.0 / 20, 9.0 / 20, 11.0 / 20}}, {2, {33.0 / 20, 27.0 / 20, 7.0 / 20, 13.0 / 20}},
        {0, {13.0 / 8, 11.0 / 8, 3.0 / 8, 5.0 / 8}}, {3, {37.0 / 20, 23.0 / 20, 3.0 / 20, 17.0 / 20}},
        {1, {29.0 / 16, 19.0 / 16, 3.0 / 16, 13.0 / 16}}, {2, {37.0 / 20, 23.0 / 20, 3.0 / 20, 17.0 / 20}},
        {0, {15.0 / 8, 9.0 / 8, 1.0 / 8, 7.0 / 8}}, {3, {39.0 / 20, 21.0 / 20, 1.0 / 20, 19.0 / 20}},
        {1, {31.0 / 16, 17.0 / 16, 1.0 / 16, 15.0 / 16}}, {2, {39.0 / 20, 21.0 / 20, 1.0 / 20, 19.0 / 20}},
    };
    static const RingRow RC[16] = {
        {0, {1.0 / 16, 31.0 / 16, 15.0 / 16, 17.0 / 16}}, {0, {3.0 / 16, 29.0 / 16, 13.0 / 16, 19.0 / 16}},
        {0, {7.0 / 16, 25.0 / 16, 9.0 / 16, 23.0 / 16}}, {0, {5.0 / 16, 27.0 / 16, 11.0 / 16, 21.0 / 16}},
        {1, {1.0 / 16, 31.0 / 16, 15.0 / 16, 17.0 / 16}}, {1, {3.0 / 16, 29.0 / 16, 13.0 / 16, 19.0 / 16}},
        {1, {7.0 / 16, 25.0 / 16, 9.0 / 16, 23.0 / 16}}, {1, {5.0 / 16, 27.0 / 16, 11.0 / 16, 21.0 / 16}},
        {3, {1.0 / 16, 31.0 / 16, 15.0 / 16, 17.0 / 16}}, {3, {3.0 / 16, 29.0 / 16, 13.0 / 16, 19.0 / 16}},
        {3, {7.0 / 16, 25.0 / 16, 9.0 / 16, 23.0 / 16}}, {3, {5.0 / 16, 27.0 / 16, 11.0 / 16, 21.0 / 16}},
        {2, {1.0 / 16, 31.0 / 16, 15.0 / 16, 17.0 / 16}}, {2, {3.0 / 16, 29.0 / 16, 13.0 / 16, 19.0 / 16}},
        {2, {7.0 / 16, 25.0 / 16, 9.0 / 16, 23.0 / 16}}, {2, {5.0 / 16, 27.0 / 16, 11.0 / 16, 21.0 / 16}},
    };
    int layout = 0;
    double g1 = 2.4, g2 = 4.3, g3 = 7.0;
    switch (rate) {
    case CUSAT_RATE_7_9:
    case CUSAT_RATE_140_180:
    case CUSAT_RATE_4_5: layout = 1; g1 = 2.2; g2 = 3.6; g3 = 5.2; break;
    case CUSAT_RATE_5_6: layout = 1; g1 = 2.2; g2 = 3.5; g3 = 5.0; break;
    case CUSAT_RATE_128_180: layout = 2; g1 = 1.88; g2 = 2.72; g3 = 3.95; break;
    default: break;
    }
    static const int COUNTS[3][4] = {{4, 12, 20, 28}, {8, 16, 20, 20}, {16, 16, 16, 16}};
    const RingRow* rows = layout == 0 ? RA : layout == 1 ? RB : RC;
    const double ratio[4] = {1.0, g1, g2, g3};
    double e = 0.0;
    for (int i = 0; i < 4; i++)
        e += COUNTS[layout][i] * ratio[i] * ratio[i];
    const double scale = sqrt(64.0 / e);
    float radius[4];
    for (int i = 0; i < 4; i++)
        radius[i] = (float)(ratio[i] * scale);
    for (int row = 0; row < 16; row++)
        for (int col = 0; col < 4; col++) {
            const int pp = col >> 1, qq = col & 1;
            int label;
            if (layout == 0)
                label = (row << 2) | (pp << 1) | qq;
            else if (layout == 1)
                label = (pp << 5) | ((row >> 3) << 4) | (qq << 3) | (row & 7);
            else
                label = ((row >> 2) << 4) | (qq << 3) | (pp << 2) | (row & 3);
            polar(p, label, radius[rows[row].ring], rows[row].a[col] * kPi);
        }
}

void build_8apsk(std::vector<float>* p, int rate)
{
    const double g1 = rate == CUSAT_RATE_100_180 ? 5.32 : 6.39;
    const double g2 = rate == CUSAT_RATE_100_180 ? 6.8 : 8.0;
    const double r1 = sqrt(8.0 / (2.0 + 4.0 * g1 * g1 + 2.0 * g2 * g2));
    const double radius[8] = {r1, g1 * r1, g1 * r1, g2 * r1, r1, g1 * r1, g1 * r1, g2 * r1};
    const double angle[8] = {1.0, 1.0 + 0.352, 1.0 - 0.352, 1.0, 0.0, -0.352, 0.352, 0.0};
    for (int l = 0; l < 8; l++)
        polar(p, l, radius[l], angle[l] * kPi);
}

// 128APSK (EN 302 307-2 Tables 14a/14b): six rings; a label is q p r4..r0,
// row r of 32 sits on one ring at first-quadrant angle a/d (units of pi),
// mirrored into the quadrants (p, q) = 00, 01, 10, 11 as a, 2 - a, 1 - a,
// 1 + a.  Each row is stored as {ring, a, d} with integer a, d; the four
// angles are (a, 2d - a, d - a, d + a) / d, the table's own fractions.
// (reference modulation/constellation.cc:347-398)
void build_128apsk(std::vector<float>* p, int rate)
{
    static const int ROWS[32][3] = {
        {0, 83, 1260},  {5, 11, 105},    {5, 37, 1680},  {5, 11, 168},   {1, 121, 2520},  {2, 23, 280},
        {4, 19, 720},   {3, 61, 720},    {0, 103, 560},  {5, 61, 420},   {5, 383, 1680},  {5, 929, 5040},
        {1, 113, 560},  {2, 169, 1008},  {4, 563, 2520}, {3, 139, 840},  {0, 243, 560},   {5, 1993, 5040},
        {5, 43, 90},    {5, 73, 168},    {1, 1139, 2520}, {2, 117, 280}, {4, 341, 720},   {3, 349, 840},
        {0, 177, 560},  {5, 1789, 5040}, {5, 49, 180},   {5, 53, 168},   {1, 167, 560},   {2, 239, 720},
        {4, 199, 720},  {3, 281, 840},
    };
    const double ratio[6] = {1.0, 1.715, 2.118, 2.681, 2.75, rate == CUSAT_RATE_135_180 ? 3.819 : 3.733};
    static const int COUNTS[6] = {16, 16, 16, 16, 16, 48};
    double e = 0.0;
    for (int i = 0; i < 6; i++)
        e += COUNTS[i] * ratio[i] * ratio[i];
    const double scale = sqrt(128.0 / e);
    for (int row = 0; row < 32; row++) {
        const float radius = (float)(ratio[ROWS[row][0]] * scale);
        const int a = ROWS[row][1], d = ROWS[row][2];
        const int num[4] = {a, 2 * d - a, d - a, d + a};
        for (int col = 0; col < 4; col++) {
            const int pp = col >> 1, qq = col & 1;
            polar(p, (qq << 6) | (pp << 5) | row, radius, (double)num[col] / d * kPi);
        }
    }
}

// 256APSK: the rates 20/30 and 22/30 (and 132/180, which shares 22/30's
// points) by the coordinates of EN 302 307-2 Table 15d, renormalised to unit
// energy; the others on eight rings of 32 points (Tables 15a-15c), label
// = x2 x1 x0 q p a2 a1 a0 with ring RING_OF[x] and angle (2 K_OF[a] - 1)
// pi / 32 mirrored by (p, q).  (reference modulation/constellation.cc:400-444)
void build_256apsk(std::vector<float>* p, int rate)
{
    const float* c = rate == CUSAT_RATE_20_30 ? cusat_apsk256_20_30
                     : (rate == CUSAT_RATE_132_180 || rate == CUSAT_RATE_22_30) ? cusat_apsk256_22_30
                                                                              : nullptr;
    if (c) {
        double e = 0.0;
        for (int i = 0; i < 256; i++)
            e += (double)c[2 * i] * c[2 * i] + (double)c[2 * i + 1] * c[2 * i + 1];
        const float s = (float)sqrt(256.0 / e);
        for (int i = 0; i < 256; i++)
            put(p, i, c[2 * i] * s, c[2 * i + 1] * s);
        return;
    }
    double g[7] = {1.791, 2.405, 2.980, 3.569, 4.235, 5.078, 6.536};
    if (rate == CUSAT_RATE_128_180 || rate == CUSAT_RATE_135_180) {
        const double common[5] = {1.794, 2.409, 2.986, 3.579, 4.045};
        for (int i = 0; i < 5; i++)
            g[i] = common[i];
        g[5] = rate == CUSAT_RATE_128_180 ? 4.6 : 4.5;
        g[6] = rate == CUSAT_RATE_128_180 ? 5.4 : 5.2;
    }
    const double ratio[8] = {1.0, g[0], g[1], g[2], g[3], g[4], g[5], g[6]};
    double e = 0.0;
    for (int i = 0; i < 8; i++)
        e += 32.0 * ratio[i] * ratio[i];
    const double scale = sqrt(256.0 / e);
    static const int RING_OF[8] = {0, 1, 3, 2, 7, 6, 4, 5};
    static const int K_OF[8] = {1, 2, 4, 3, 8, 7, 5, 6};
    for (int x = 0; x < 8; x++) {
        const float radius = (float)(ratio[RING_OF[x]] * scale);
        for (int qq = 0; qq < 2; qq++)
            for (int pp = 0; pp < 2; pp++)
                for (int a = 0; a < 8; a++) {
                    const double phi = (2 * K_OF[a] - 1) * kPi / 32.0;
                    const double angle = pp ? (qq ? kPi + phi : kPi - phi) : (qq ? -phi : phi);
                    polar(p, (x << 5) | (qq << 4) | (pp << 3) | a, radius, angle);
                }
    }
}

bool is_16apsk_8_8(int r)
{
    return r == CUSAT_RATE_90_180 || r == CUSAT_RATE_96_180 || r == CUSAT_RATE_100_180 ||
           r == CUSAT_RATE_18_30 || r == CUSAT_RATE_20_30;
}

const char* column_order(int mod, int r)
{
    switch (mod) {
    case CUSAT_MOD_8PSK:
        if (r == CUSAT_RATE_3_5) return "210";
        if (r == CUSAT_RATE_25_36 || r == CUSAT_RATE_13_18 || r == CUSAT_RATE_7_15 ||
            r == CUSAT_RATE_8_15 || r == CUSAT_RATE_26_45)
            return "102";
        return "012";
    case CUSAT_MOD_8APSK: return "012";
    case CUSAT_MOD_16APSK:
        switch (r) {
        case CUSAT_RATE_26_45: return "3201";
        case CUSAT_RATE_3_5: return "3210";
        case CUSAT_RATE_28_45: return "3012";
        case CUSAT_RATE_23_36: return "3021";
        case CUSAT_RATE_25_36: return "2310";
        case CUSAT_RATE_13_18: return "3021";
        case CUSAT_RATE_7_9:
        case CUSAT_RATE_140_180: return "3210";
        case CUSAT_RATE_154_180: return "0321";
        case CUSAT_RATE_90_180: return "3210";
        case CUSAT_RATE_96_180: return "2310";
        case CUSAT_RATE_100_180: return "2301";
        default: return "0123";
        }
    case CUSAT_MOD_32APSK:
        if (r == CUSAT_RATE_2_3 || r == CUSAT_RATE_32_45) return "21430";
        if (r == CUSAT_RATE_128_180 || r == CUSAT_RATE_132_180 || r == CUSAT_RATE_22_30) return "40312";
        if (r == CUSAT_RATE_7_9 || r == CUSAT_RATE_140_180) return "40213";
        return "01234";
    case CUSAT_MOD_64APSK:
        if (r == CUSAT_RATE_7_9 || r == CUSAT_RATE_140_180) return "201543";
        if (r == CUSAT_RATE_4_5) return "124053";
        if (r == CUSAT_RATE_5_6) return "421053";
        if (r == CUSAT_RATE_128_180) return "305214";
        return "520143";
    case CUSAT_MOD_128APSK:
        return (r == CUSAT_RATE_7_9 || r == CUSAT_RATE_140_180) ? "4130256" : "4250316";
    case CUSAT_MOD_256APSK:
        switch (r) {
        case CUSAT_RATE_135_180: return "50743612";
        case CUSAT_RATE_128_180: return "75642301";
        case CUSAT_RATE_116_180: return "40372156";
        case CUSAT_RATE_124_180: return "46320571";
        default: return "01234567";
        }
    default: return nullptr;
    }
}

}  // namespace

int make_constellation(int mod, int rate, int framesize, std::vector<float>* p)
{
    int bits;
    switch (mod) {
    case CUSAT_MOD_QPSK: bits = 2; break;
    case CUSAT_MOD_8PSK:
    case CUSAT_MOD_8APSK: bits = 3; break;
    case CUSAT_MOD_16APSK: bits = 4; break;
    case CUSAT_MOD_32APSK: bits = 5; break;
    case CUSAT_MOD_64APSK: bits = 6; break;
    case CUSAT_MOD_128APSK: bits = 7; break;
    case CUSAT_MOD_256APSK: bits = 8; break;
    default: return -1;
    }
    p->assign(2 << bits, 0.0f);
    switch (mod) {
    case CUSAT_MOD_QPSK: {
        const float a = (float)M_SQRT1_2;
        for (int l = 0; l < 4; l++)
            put(p, l, (l & 2) ? -a : a, (l & 1) ? -a : a);
        break;
    }
    case CUSAT_MOD_8PSK: {
        const float a = (float)M_SQRT1_2;
        const float pts[8][2] = {{a, a}, {1, 0}, {-1, 0}, {-a, -a}, {0, 1}, {a, -a}, {-a, a}, {0, -1}};
        for (int l = 0; l < 8; l++)
            put(p, l, pts[l][0], pts[l][1]);
        break;
    }
    case CUSAT_MOD_8APSK: build_8apsk(p, rate); break;
    case CUSAT_MOD_16APSK:
        if (is_16apsk_8_8(rate))
            build_16apsk_8_8(p, rate);
        else
            build_16apsk_4_12(p, rate);
        break;
    case CUSAT_MOD_32APSK:
        if (rate == CUSAT_RATE_2_3 || rate == CUSAT_RATE_32_45)
            build_32apsk_rb(p, rate, framesize);
        else if (rate == CUSAT_RATE_128_180 || rate == CUSAT_RATE_132_180 || rate == CUSAT_RATE_22_30 ||
                 rate == CUSAT_RATE_140_180 || rate == CUSAT_RATE_7_9)
            build_32apsk_4_8_4_16(p, rate);
        else
            build_32apsk_4_12_16(p, rate);
        break;
    case CUSAT_MOD_64APSK: build_64apsk(p, rate); break;
    case CUSAT_MOD_128APSK: build_128apsk(p, rate); break;
    case CUSAT_MOD_256APSK: build_256apsk(p, rate); break;
    }
    return bits;
}

int make_interleaver(int mod, int rate, int framesize, uint32_t col[8], uint32_t* rows)
{
    for (int i = 0; i < 8; i++)
        col[i] = 0;
    *rows = 0;
    if (mod == CUSAT_MOD_QPSK)
        return 0;
    const char* order = column_order(mod, rate);
    if (!order)
        return -1;
    const int n_cols = (int)strlen(order);
    const unsigned n_fec = (unsigned)cusat_fecframe_bits(framesize);
    const unsigned stuffed = mod == CUSAT_MOD_128APSK ? n_fec + 6 : n_fec;
    *rows = stuffed / n_cols;
    for (int c = 0; c < n_cols; c++)
        col[c] = *rows * (unsigned)(order[c] - '0');
    return n_cols;
}

bool build_modcod_demap(int mod, int rate, int framesize, ModcodDemap* d, std::string* err)
{
    if (framesize < 0 || framesize > 2 || rate < 0 || rate >= CUSAT_RATE_COUNT) {
        if (err) *err = "frame size or rate out of range";
        return false;
    }
    d->modulation = mod;
    d->rate = rate;
    d->framesize = framesize;
    const int bits = make_constellation(mod, rate, framesize, &d->pts);
    if (bits < 0) {
        if (err) *err = "modulation not supported";
        return false;
    }
    d->n_mod = bits;
    d->n_points = 1 << bits;
    d->fec_len = cusat_fecframe_bits(framesize);
    // 128APSK: 6 stuffing bits ahead of the interleaver and 12 padding
    // symbols after it (reference cuda/demapper_kernel.cu:241-247)
    if (mod == CUSAT_MOD_128APSK) {
        d->interleaved_len = (d->fec_len + 6) / bits;
        d->xfec = d->interleaved_len + 12;
    } else {
        d->xfec = d->fec_len / bits;
        d->interleaved_len = d->xfec;
    }
    d->kind = mod == CUSAT_MOD_QPSK ? 0 : mod == CUSAT_MOD_8PSK ? 1 : 2;
    uint32_t rows;
    if (make_interleaver(mod, rate, framesize, d->col, &rows) < 0) {
        if (err) *err = "no interleaver for this modulation";
        return false;
    }
    // loudest-bit distance (reference cuda/demapper_kernel.cu:216-237)
    if (mod == CUSAT_MOD_QPSK) {
        d->dmax = 2.0f;
    } else if (mod == CUSAT_MOD_8PSK) {
        d->dmax = 4.0f;
    } else {
        float dmax = 0.0f;
        for (int i = 0; i < d->n_points; i++)
            for (int b = 0; b < bits; b++) {
                const int mask = 1 << (bits - 1 - b);
                float dmin = 1e30f;
                for (int k = 0; k < d->n_points; k++) {
                    if (((i ^ k) & mask) == 0)
                        continue;
                    const float dr = d->pts[2 * i] - d->pts[2 * k];
                    const float di = d->pts[2 * i + 1] - d->pts[2 * k + 1];
                    const float dd = dr * dr + di * di;
                    if (dd < dmin)
                        dmin = dd;
                }
                if (dmin > dmax)
                    dmax = dmin;
            }
        d->dmax = dmax;
    }
    // LLR target of the gain cap: 320, or CUSAT_DEMAP_LLR_TARGET when set
    // (read at construction, as the reference does: demapper_kernel.cu:238-239)
    const char* tgt = getenv("CUSAT_DEMAP_LLR_TARGET");
    d->llr_target = tgt ? (float)atof(tgt) : 320.0f;
    return true;
}

float capped_llr_gain(const ModcodDemap& d, float llr_gain)
{
    if (d.llr_target <= 0.0f || d.dmax <= 0.0f)
        return llr_gain;
    const float cap = 2.0f * d.llr_target / d.dmax;
    return llr_gain < cap ? llr_gain : cap;
}

void map_frames(const ModcodDemap& d, const uint8_t* cw, int B, float* sym)
{
    const int cw_bytes = d.fec_len / 8;
    const int stride = d.kind == 0 ? 2 : 1;
    uint32_t col[8];
    for (int b = 0; b < 8; b++)
        col[b] = d.kind == 0 ? (uint32_t)b : d.col[b];
    for (int f = 0; f < B; f++) {
        const uint8_t* in = cw + (size_t)f * cw_bytes;
        float* out = sym + (size_t)f * d.xfec * 2;
        for (int j = 0; j < d.xfec; j++) {
            // stuffing bits (positions past the FECFRAME) are 0; padding
            // symbols (128APSK) carry the all-ones label (reference
            // mapper.cc:42-62)
            int label = d.n_points - 1;
            if (j < d.interleaved_len) {
                label = 0;
                for (int b = 0; b < d.n_mod; b++) {
                    const int pos = (int)col[b] + j * stride;
                    if (pos < d.fec_len)
                        label |= ((in[pos >> 3] >> (7 - (pos & 7))) & 1) << (d.n_mod - 1 - b);
                }
            }
            out[2 * j] = d.pts[2 * label];
            out[2 * j + 1] = d.pts[2 * label + 1];
        }
    }
}

// Decision-directed SNR (reference modulation/dd_snr.cc:12-47): each symbol
// is replaced by its nearest constellation point; SNR = energy of the
// decisions / energy of the errors, 1e6 when the errors are that small, 0 for
// non-finite input.  Float accumulation in symbol order, no contraction (this
// file is built with -ffp-contract=off), so the value is the reference's.
static float dd_ratio(float signal, float error)
{
    if (!std::isfinite(signal) || !std::isfinite(error))
        return 0.0f;
    const float cap = 1e6f;
    return error * cap <= signal ? cap : signal / error;
}

float dd_snr_qpsk(const float* sym, int n_sym)
{
    const float a = (float)0.70710678118654752440;
    float signal = 0.0f, error = 0.0f;
    for (int i = 0; i < n_sym; i++) {
        const float re = sym[2 * i], im = sym[2 * i + 1];
        const float dr = re < 0 ? -a : a, di = im < 0 ? -a : a;
        signal += dr * dr + di * di;
        const float er = re - dr, ei = im - di;
        error += er * er;
        error += ei * ei;
    }
    return dd_ratio(signal, error);
}

float dd_snr_points(const std::vector<float>& pts, const float* sym, int n_sym, int stride)
{
    const int n_points = (int)pts.size() / 2;
    float signal = 0.0f, error = 0.0f;
    for (int i = 0; i < n_sym; i += stride) {
        const float re = sym[2 * i], im = sym[2 * i + 1];
        // nearest point, first of equals (reference constellation.cc:495-507)
        int best = 0;
        float best_d = 3.402823466e38f;
        for (int l = 0; l < n_points; l++) {
            const float dr = re - pts[2 * l], di = im - pts[2 * l + 1];
            const float d = dr * dr + di * di;
            if (d < best_d) {
                best_d = d;
                best = l;
            }
        }
        const float pr = pts[2 * best], pi = pts[2 * best + 1];
        signal += pr * pr + pi * pi;
        const float er = re - pr, ei = im - pi;
        error += er * er + ei * ei;
    }
    return dd_ratio(signal, error);
}

}  // namespace cusat
