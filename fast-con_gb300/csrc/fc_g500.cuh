// fc_g500.cuh -- the Graph500 Kronecker generator's arithmetic, as host and
// device functions (the device kernels are in fc_g500.cu; the host copies let
// the host side build the jump tables).
//
// The reference driver generates its graphs with the vendored Graph500
// generator (make_graph, bernaschi/ST_CONN_ONE_ATOMIC/current-st/generator/
// make_graph.c:35-104).  Reproducing its edges bit for bit fixes every step
// below to the generator's own: the same multiple recursive generator and
// jump-ahead rule (splittable_mrg.c), the same recursive quadrant split with
// binomial counts by Hoermann's BTRD method (graph_generator.c,
// btrd_binomial_distribution.c), the same vertex permutation by random keys
// (permutation_gen.c rand_sort_shared) -- written here in this library's own
// code.  All floating-point work is IEEE double without fused multiply-add
// (the unit is compiled with -fmad=false), in the generator's operation
// order; log and sqrt are the CUDA library's.
#pragma once

#include <stdint.h>
#include <cmath>

namespace fc {
namespace g500 {

constexpr uint32_t MRG_P = 0x7FFFFFFFu;  // 2^31 - 1
// x_n = 107374182 x_{n-1} + 104480 x_{n-5} (mod 2^31 - 1), L'Ecuyer's MRG5
constexpr uint32_t MRG_A1 = 107374182u, MRG_A5 = 104480u;
// 1 / (2^31 - 1) and 1 / (2^31 - 1)^2, to 22 significant digits
constexpr double INV_P1 = 4.656612875245796924106e-10;
constexpr double INV_P2 = 2.168404346990492786791e-19;

__host__ __device__ inline uint32_t mod_add(uint32_t a, uint32_t b)
{
    const uint32_t r = a + b;
    return r >= MRG_P ? r - MRG_P : r;
}

__host__ __device__ inline uint32_t mod_mul(uint32_t a, uint32_t b)
{
    const uint64_t t = (uint64_t)a * b;
    const uint32_t r = (uint32_t)(t & MRG_P) + (uint32_t)(t >> 31);
    return r >= MRG_P ? r - MRG_P : r;
}

// State (z1 .. z5), z1 the newest value.
struct Mrg {
    uint32_t z[5];
};

__host__ __device__ inline uint32_t mrg_next(Mrg &s)
{
    const uint32_t n = mod_add(mod_mul(MRG_A1, s.z[0]), mod_mul(MRG_A5, s.z[4]));
    s.z[4] = s.z[3];
    s.z[3] = s.z[2];
    s.z[2] = s.z[1];
    s.z[1] = s.z[0];
    s.z[0] = n;
    return n;
}

// A double in [0, 1) from two consecutive values (the first one weighs 2^-31).
__host__ __device__ inline double mrg_double(Mrg &s)
{
    const double hi = (double)mrg_next(s);
    const double lo = (double)mrg_next(s);
    return hi * INV_P1 + lo * INV_P2;
}

// Seed from two 64-bit user seeds: five values in [1, 2^30], the generator's
// spreading rule (make_mrg_seed, generator/utils.c).
__host__ __device__ inline Mrg mrg_seed(uint64_t s1, uint64_t s2)
{
    Mrg m;
    m.z[0] = (uint32_t)(s1 & 0x3FFFFFFF) + 1;
    m.z[1] = (uint32_t)((s1 >> 30) & 0x3FFFFFFF) + 1;
    m.z[2] = (uint32_t)(s2 & 0x3FFFFFFF) + 1;
    m.z[3] = (uint32_t)((s2 >> 30) & 0x3FFFFFFF) + 1;
    m.z[4] = (uint32_t)(((s2 >> 60) << 4) + (s1 >> 60) + 1);
    return m;
}

// 5 x 5 matrices over GF(2^31 - 1) acting on (z1 .. z5); the jump tables hold
// T[k][b] = A^(b * 256^k), k < 24 (jumps below 2^192).
struct Mat5 {
    uint32_t m[25];
};
constexpr int JUMP_BYTES = 24;

__host__ __device__ inline Mrg mat_apply(const Mat5 &M, const Mrg &s)
{
    Mrg r;
    for (int i = 0; i < 5; ++i) {
        uint32_t acc = 0;
        for (int j = 0; j < 5; ++j) acc = mod_add(acc, mod_mul(M.m[i * 5 + j], s.z[j]));
        r.z[i] = acc;
    }
    return r;
}

inline Mat5 mat_mul(const Mat5 &X, const Mat5 &Y)
{
    Mat5 r;
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            uint32_t acc = 0;
            for (int k = 0; k < 5; ++k) acc = mod_add(acc, mod_mul(X.m[i * 5 + k], Y.m[k * 5 + j]));
            r.m[i * 5 + j] = acc;
        }
    return r;
}

// table[k * 256 + b] = A^(b * 256^k) for k < JUMP_BYTES, b < 256 (host).
inline void build_jump_tables(Mat5 *table)
{
    Mat5 I{}, A{};
    for (int i = 0; i < 5; ++i) I.m[i * 5 + i] = 1;
    A.m[0] = MRG_A1;
    A.m[4] = MRG_A5;
    for (int i = 1; i < 5; ++i) A.m[i * 5 + i - 1] = 1;
    Mat5 base = A;  // A^(256^k)
    for (int k = 0; k < JUMP_BYTES; ++k) {
        table[k * 256] = I;
        for (int b = 1; b < 256; ++b) table[k * 256 + b] = mat_mul(table[k * 256 + b - 1], base);
        base = mat_mul(table[k * 256 + 255], base);  // A^(256^(k+1))
    }
}

// s advanced by hi * 2^128 + mid * 2^64 + lo steps.
__host__ __device__ inline Mrg mrg_jump(const Mat5 *table, Mrg s, uint64_t hi, uint64_t mid,
                                        uint64_t lo)
{
    const uint64_t part[3] = {lo, mid, hi};
    for (int q = 0; q < 3; ++q) {
        uint64_t e = part[q];
        for (int k = 0; e; ++k, e >>= 8) {
            const int b = (int)(e & 0xFF);
            if (b) s = mat_apply(table[(q * 8 + k) * 256 + b], s);
        }
    }
    return s;
}

// Uniform integer in [0, n) by rejection, n <= (2^31 - 1)^2 (random_up_to,
// generator/utils.c).
__host__ __device__ inline uint64_t mrg_below(Mrg &s, uint64_t n)
{
    if (n == 1) return 0;
    if (n <= 0x7FFFFFFFull) {
        const uint64_t limit = (0x7FFFFFFFull / n) * n;
        while (true) {
            const uint64_t x = mrg_next(s);
            if (x < limit) return x % n;
        }
    }
    const uint64_t top = 0x3FFFFFFF00000001ull;  // (2^31 - 1)^2
    const uint64_t limit = (top / n) * n;
    while (true) {
        uint64_t x = (uint64_t)mrg_next(s) * 0x7FFFFFFFull;
        x += mrg_next(s);
        if (x < limit) return x % n;
    }
}

// ---------------------------------------------------------------------------
// Binomial variates: Hoermann's BTRD (transformed rejection with decomposition,
// "The Generation of Binomial Random Variates", J. Statist. Comput. Simul. 46,
// 1993), and for n p < 10 the sum of geometric waiting times (Devroye, "Non-
// Uniform Random Variate Generation", 1986, ch. X.4), ln(1 - p) from the series
// 2 / r (1 + r^-2 / 3 + r^-4 / 5 + r^-6 / 7), r = 1 - 2 / p.
// ---------------------------------------------------------------------------
// Stirling-series remainder f_c(k) = ln k! - (k + 1/2) ln(k + 1) + (k + 1)
// - ln sqrt(2 pi): exact values (correctly rounded) for k < 10, the series
// 1/12 - 1/360 x^2 + 1/1260 x^4 (x = 1 / (k + 1)) times x beyond.
__host__ __device__ inline double stirling_fc(int k)
{
    constexpr double exact[10] = {8.1061466795327258219670e-2, 4.1340695955409294093822e-2,
                                  2.7677925684998339148789e-2, 2.0790672103765093111523e-2,
                                  1.6644691189821192163195e-2, 1.3876128823070747998746e-2,
                                  1.1896709945891770095056e-2, 1.0411265261972096497479e-2,
                                  9.2554621827127329177286e-3, 8.3305634333628712564693e-3};
    if (k <= 9) return exact[k];
    const double x = 1. / (k + 1);
    return (1. / 12 - (1. / 360 - 1. / 1260 * x * x) * x * x) * x;
}

__host__ __device__ inline long long binomial_small_np(long long n, double p, Mrg &s)
{
    const double r = 1. - 2. / p;
    const double ir = 1. / r;
    const double ir2 = ir * ir;
    const double ir4 = ir2 * ir2;
    const double ir6 = ir4 * ir2;
    const double ln1p = 2. * ir * (1 + ir2 / 3. + ir4 / 5. + ir6 / 7.);  // ln(1 - p)
    const double inv = 1. / ln1p;
    int x = 0, sum = 0;
    do {
        sum += (int)ceil(log(mrg_double(s)) * inv);
        ++x;
    } while ((long long)sum <= n);
    return x - 1;
}

__host__ __device__ inline long long binomial_btrd(int n, double p, Mrg &s)
{
    const int m = (int)floor((n + 1) * p);
    const double r = p / (1. - p);
    const double nr = (n + 1) * r;
    const double npq = n * p * (1. - p);
    const double sq = sqrt(npq);
    const double b = 1.15 + 2.53 * sq;
    const double a = -.0873 + .0248 * b + .01 * p;
    const double c = n * p + .5;
    const double alpha = (2.83 + 5.1 / b) * sq;
    const double vr = .92 - 4.2 / b;
    const double urvr = .86 * vr;
    while (true) {
        double v = mrg_double(s);
        if (v <= urvr) {
            const double u = v / vr - .43;
            return (int)floor((2 * a / (.5 + fabs(u)) + b) * u + c);
        }
        const double w = mrg_double(s);
        double u;
        if (v >= vr) {
            u = w - .5;
        } else {
            u = v / vr - .93;
            u = (u > 0. ? 1. : u < 0. ? -1. : 0.) * .5 - u;
            v = vr * w;
        }
        const double us = .5 - fabs(u);
        const int k = (int)floor((2 * a / us + b) * u + c);
        if (k < 0 || k > n) continue;
        v *= alpha / (a / (us * us) + b);
        const int km = k >= m ? k - m : m - k;
        if (km > 15) {
            const double rho = (km / npq) * (((km / 3 + .625) * km + 1. / 6) / npq + .5);
            const double t = -km * km / (2 * npq);
            v = log(v);
            if (v < t - rho) return k;
            if (v > t + rho) continue;
            const int nm = n - m + 1;
            const double h = (m + .5) * log((m + 1) / (r * nm)) + stirling_fc(m) + stirling_fc(n - m);
            const int nk = n - k + 1;
            const double bound = h + (n + 1) * log((double)nm / nk) +
                                 (k + .5) * log(nk * r / (k + 1)) - stirling_fc(k) -
                                 stirling_fc(n - k);
            if (v <= bound) return k;
        } else {
            double f = 1.;
            if (m < k) {
                for (int i = m; i != k; ++i) f *= nr / i - r;
            } else if (m > k) {
                for (int i = k; i != m; ++i) v *= nr / i + r;
            }
            if (v <= f) return k;
        }
    }
}

// Binomial(n, p): p above 1/2 drawn as n - Binomial(n, 1 - p); counts above
// 10^9 in parts of 10^9, the first part first.
__host__ __device__ inline long long binomial(long long n, double p, Mrg &s)
{
    if (p == 0.) return 0;
    bool flip = false;
    if (p > .5) {
        flip = true;
        p = 1. - p;
    }
    long long x = 0, rest = n;
    if (rest * p < 10) {
        x = binomial_small_np(rest, p, s);
    } else {
        while (rest > 1000000000) {
            x += binomial_btrd(1000000000, p, s);
            rest -= 1000000000;
        }
        x += (double)rest * p < 10 ? binomial_small_np(rest, p, s) : binomial_btrd((int)rest, p, s);
    }
    return flip ? n - x : x;
}

// ---------------------------------------------------------------------------
// Kronecker quadrant choices (initiator a, b, c, d: quadrant index = 2 src
// bit + tgt bit).  Undirected form: on the diagonal (src base == tgt base)
// the upper and lower off-diagonal quadrants are folded onto the upper one.
// ---------------------------------------------------------------------------
struct Initiator {
    double q[4];
};

__host__ __device__ inline int quadrant(const Initiator &I, Mrg &s)
{
    double x = mrg_double(s);
    for (int j = 0; j < 3; ++j) {
        if (x < I.q[j]) return j;
        x -= I.q[j];
    }
    return 3;
}

// How many of `ne` edges fall in each quadrant of a node.
__host__ __device__ inline void quadrant_counts(long long ne, const Initiator &I, Mrg &s,
                                                bool diagonal, long long cnt[4])
{
    if (ne <= 20) {
        cnt[0] = cnt[1] = cnt[2] = cnt[3] = 0;
        for (long long e = 0; e < ne; ++e) {
            double x = mrg_double(s);
            for (int j = 0; j < 4; ++j) {
                if (x < I.q[j] || j == 3) {
                    ++cnt[j];
                    break;
                }
                x -= I.q[j];
            }
        }
    } else {
        long long left = ne;
        double div = 1.;
        for (int j = 0; j < 3; ++j) {
            cnt[j] = binomial(left, I.q[j] / div, s);
            left -= cnt[j];
            div -= I.q[j];
        }
        cnt[3] = left;
    }
    if (diagonal) {
        cnt[1] += cnt[2];
        cnt[2] = 0;
    }
}

// A node holding one edge: descend to a single cell.
__host__ __device__ inline void one_edge(long long bs, long long bt, long long nverts,
                                         const Initiator &I, Mrg &s, long long *src,
                                         long long *tgt)
{
    while (nverts > 1) {
        const int q = quadrant(I, s);
        int so = q / 2, to = q % 2;
        if (bs == bt && so > to) {
            const int t = so;
            so = to;
            to = t;
        }
        nverts /= 2;
        bs += nverts * so;
        bt += nverts * to;
    }
    *src = bs;
    *tgt = bt;
}

}  // namespace g500
}  // namespace fc
