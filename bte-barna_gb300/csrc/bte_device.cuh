// bte_device.cuh - arithmetic shared by the host table builder and the
// sm_103a kernels: random streams, uniform mappings, log, fixed-point tally
// quantisation and the 2D geometry primitives of the particle loop.
//
// Every function here is written so that host (g++ -ffp-contract=off) and
// device (nvcc -fmad=false, replay translation unit) evaluate the same
// IEEE-754 operations in the same order: the replay mode reproduces the CPU
// restatement bit for bit.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define BTE_HD __host__ __device__ __forceinline__
#else
#define BTE_HD inline
#endif

namespace bte {

// ------------------------------------------------------------- integer helpers
BTE_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return uint64_t((unsigned __int128)a * b >> 64);
#endif
}

BTE_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return uint32_t((uint64_t(a) * b) >> 32);
#endif
}

BTE_HD double u64_to_double(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __ull2double_rn(x);
#else
    return double(x);
#endif
}

BTE_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return uint64_t(__double_as_longlong(x));
#else
    uint64_t b;
    __builtin_memcpy(&b, &x, 8);
    return b;
#endif
}

BTE_HD double bitsd(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    __builtin_memcpy(&x, &b, 8);
    return x;
#endif
}

// ------------------------------------------------------------- pcg64
// PCG XSL-RR 128/64 with a selectable stream (the reference's pcg64,
// pcg-cpp pcg_random.hpp setseq_xsl_rr_128_64): 128-bit LCG state, output
// xor-fold of the two halves rotated by the top six bits.
struct Pcg64 {
    uint64_t sh, sl, ih, il;
    static constexpr uint64_t MH = 2549297995355413924ULL;
    static constexpr uint64_t ML = 4865540595714422341ULL;

    BTE_HD void step() {
        uint64_t lo = sl * ML;
        uint64_t hi = mulhi64(sl, ML) + sh * ML + sl * MH;
        uint64_t lo2 = lo + il;
        hi = hi + ih + (lo2 < lo ? 1u : 0u);
        sh = hi;
        sl = lo2;
    }
    BTE_HD void seed(uint64_t seed, uint64_t stream) {
        ih = stream >> 63;
        il = (stream << 1) | 1u;
        uint64_t lo = seed + il;
        sh = ih + (lo < seed ? 1u : 0u);
        sl = lo;
        step();
    }
    BTE_HD uint64_t next() {
        step();
        unsigned rot = unsigned(sh >> 58);
        uint64_t x = sh ^ sl;
        return rot ? (x >> rot) | (x << ((64u - rot) & 63u)) : x;
    }
};

// generate_canonical<double, 53> over a 64-bit engine: x / 2^64, moved below
// one when the conversion rounds up (libstdc++ bits/random.tcc).
BTE_HD double canonical_from(uint64_t x) {
    double u = u64_to_double(x) * 0x1p-64;
    if (u >= 1.0) u = 0x1.fffffffffffffp-1;
    return u;
}

// uniform_int_distribution<int>(0, n-1) over a 64-bit engine: Lemire's
// nearly-divisionless reduction as libstdc++ implements it.
template <class G>
BTE_HD int uniform_below(G& g, uint32_t n) {
    const uint64_t range = n;
    uint64_t x = g.next();
    uint64_t lo = x * range;
    uint64_t hi = mulhi64(x, range);
    if (lo < range) {
        const uint64_t threshold = (0 - range) % range;
        while (lo < threshold) {
            x = g.next();
            lo = x * range;
            hi = mulhi64(x, range);
        }
    }
    return int(hi);
}

// ------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror and Shaw (SC'11): ten
// rounds of two 32x32->64 multiplies with a Weyl-sequence key schedule.
struct Philox {
    uint32_t c0, c1, c2, c3;  // counter: draw index (c0,c1), particle (c2,c3)
    uint32_t k0, k1;          // key: master seed
    uint32_t b0, b1, b2, b3;  // unread words of the last block, b0 first
    int avail;

    BTE_HD void init(uint64_t seed, uint64_t particle) {
        c0 = 0;
        c1 = 0;
        c2 = uint32_t(particle);
        c3 = uint32_t(particle >> 32);
        k0 = uint32_t(seed);
        k1 = uint32_t(seed >> 32);
        avail = 0;
        b0 = b1 = b2 = b3 = 0;
    }
    BTE_HD void block() {
        uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3;
        uint32_t a = k0, b = k1;
#if defined(__CUDACC__)
#pragma unroll
#endif
        for (int r = 0; r < 10; ++r) {
            const uint32_t lo0 = 0xD2511F53u * x0, hi0 = mulhi32(0xD2511F53u, x0);
            const uint32_t lo1 = 0xCD9E8D57u * x2, hi1 = mulhi32(0xCD9E8D57u, x2);
            x0 = hi1 ^ x1 ^ a;
            x1 = lo1;
            x2 = hi0 ^ x3 ^ b;
            x3 = lo0;
            a += 0x9E3779B9u;
            b += 0xBB67AE85u;
        }
        b0 = x3;  // words leave in the order x3, x2, x1, x0
        b1 = x2;
        b2 = x1;
        b3 = x0;
    }
    BTE_HD uint32_t next32() {
        if (avail == 0) {
            block();
            if (++c0 == 0) ++c1;
            avail = 4;
        }
        const uint32_t r = b0;  // a register queue: no indexed (local-memory) access
        b0 = b1;
        b1 = b2;
        b2 = b3;
        --avail;
        return r;
    }
    BTE_HD uint64_t next() {
        uint64_t h = next32();
        return (h << 32) | next32();
    }
    // Uniform in [2^-24, 1 - 2^-24] on a 2^-23 lattice, for the
    // single-precision -log(u): (k + 1/2) 2^-23 is exact in FP32 for every
    // 23-bit k, so u never rounds to 0 or 1.
    BTE_HD float uniformf() { return (float(next32() >> 9) + 0.5f) * 0x1p-23f; }
    // Uniform in [0, 1) with 53 bits.
    BTE_HD double uniform() { return u64_to_double(next() >> 11) * 0x1p-53; }
};

// ------------------------------------------------------------- log
// Natural log by Cody-Waite reduction x = 2^e m, m in (1/sqrt2, sqrt2], and
// the series log m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = (m-1)/(m+1),
// summed to s^23 (|s| <= 0.1716, so the next term is below 2^-53).
BTE_HD double bte_log(double x) {
    if (!(x > 0.)) return x == 0. ? -__builtin_huge_val() : __builtin_nan("");
    if (x == __builtin_huge_val()) return x;
    uint64_t bits = dbits(x);
    int e = int((bits >> 52) & 0x7ff);
    if (e == 0) {
        bits = dbits(x * 18014398509481984.0);
        e = int((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double m = bitsd((bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double f = m - 1.0;
    const double s = f / (2.0 + f);
    const double z = s * s;
    double p = 1.0 / 23.0;
    p = p * z + 1.0 / 21.0;
    p = p * z + 1.0 / 19.0;
    p = p * z + 1.0 / 17.0;
    p = p * z + 1.0 / 15.0;
    p = p * z + 1.0 / 13.0;
    p = p * z + 1.0 / 11.0;
    p = p * z + 1.0 / 9.0;
    p = p * z + 1.0 / 7.0;
    p = p * z + 1.0 / 5.0;
    p = p * z + 1.0 / 3.0;
    const double two_s = s + s;
    const double logm = two_s + two_s * z * p;
    const double de = double(e);
    const double LN2_HI = 0.6931471787393093;      // ln 2 with 28 significant bits
    const double LN2_LO = 1.8206359985041462e-09;  // ln 2 - LN2_HI
    return de * LN2_HI + (de * LN2_LO + logm);
}

// ------------------------------------------------------------- comparisons
// alma::almost_equal with its defaults (abs 1e-8, rel 1e-5).
BTE_HD bool almost_equal(double a, double b) {
    const double tol = 1e-8 + __builtin_fabs(1e-5 * b);
    return __builtin_fabs(a - b) < tol;
}

// ------------------------------------------------------------- fixed point
// Replay tallies accumulate contributions as 128-bit integers scaled by 2^44:
// integer addition is associative, so the sum does not depend on the order
// in which threads add.  |contribution| must stay below 2^18.
constexpr double FIX_SCALE = 17592186044416.0;        // 2^44
constexpr double FIX_LIMIT = 4611686018427387904.0;   // 2^62 after scaling

BTE_HD bool quantise(double x, long long& q) {
    const double y = x * FIX_SCALE;
    if (!(__builtin_fabs(y) < FIX_LIMIT)) return false;
#if defined(__CUDA_ARCH__)
    q = __double2ll_rn(y);
#else
    q = __builtin_llrint(y);
#endif
    return true;
}

// ------------------------------------------------------------- 2D geometry
struct V2 {
    double x, y;
};
BTE_HD V2 v2(double x, double y) {
    V2 r;
    r.x = x;
    r.y = y;
    return r;
}
BTE_HD V2 add(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
BTE_HD V2 sub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
BTE_HD V2 scal(double s, V2 a) { return v2(s * a.x, s * a.y); }
BTE_HD V2 divs(V2 a, double s) { return v2(a.x / s, a.y / s); }
BTE_HD double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
BTE_HD double cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
BTE_HD double norm(V2 a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a.x * a.x + a.y * a.y);
#else
    return __builtin_sqrt(a.x * a.x + a.y * a.y);
#endif
}

// Point on segment a-b, end points included; a degenerate segment is a point.
BTE_HD bool on_segment(V2 p, V2 a, V2 b) {
    const V2 d = sub(b, a);
    if (d.x == 0. && d.y == 0.) return p.x == a.x && p.y == a.y;
    if (cross(d, sub(p, a)) != 0.) return false;
    const double t = dot(sub(p, a), d);
    return t >= 0. && t <= dot(d, d);
}

// Segment s0-s1 against l0-l1; the crossing point is taken on l0-l1 so that
// it lies exactly on an axis-aligned border.  Parallel segments never meet.
BTE_HD bool seg_intersect(V2 s0, V2 s1, V2 l0, V2 l1, V2& out) {
    const V2 d1 = sub(s1, s0), d2 = sub(l1, l0);
    const double den = cross(d1, d2);
    if (den == 0.) return false;
    const V2 w = sub(l0, s0);
    const double t = cross(w, d2) / den;
    const double u = cross(w, d1) / den;
    if (!(t >= 0. && t <= 1. && u >= 0. && u <= 1.)) return false;
    out = add(l0, scal(u, d2));
    return true;
}

// boost::geometry::intersects / intersection of two closed segments, as the
// periodic translation uses them: true when s0-s1 and l0-l1 share a point;
// `out` is the first shared point (a crossing is taken on l0-l1; for
// collinear segments, the end of the overlap nearest s0; a degenerate l is
// the point l0).
BTE_HD bool seg_meet(V2 s0, V2 s1, V2 l0, V2 l1, V2& out) {
    const V2 d1 = sub(s1, s0), d2 = sub(l1, l0);
    if (d2.x == 0. && d2.y == 0.) {
        if (!on_segment(l0, s0, s1)) return false;
        out = l0;
        return true;
    }
    const double den = cross(d1, d2);
    const V2 w = sub(l0, s0);
    if (den != 0.) {
        const double t = cross(w, d2) / den;
        const double u = cross(w, d1) / den;
        if (!(t >= 0. && t <= 1. && u >= 0. && u <= 1.)) return false;
        out = add(l0, scal(u, d2));
        return true;
    }
    if (cross(w, d1) != 0.) return false;  // parallel, apart
    const double dd = dot(d1, d1);
    if (dd == 0.) {
        if (!on_segment(s0, l0, l1)) return false;
        out = s0;
        return true;
    }
    // overlap of the parameter ranges along s
    const double a = dot(sub(l0, s0), d1) / dd, b = dot(sub(l1, s0), d1) / dd;
    const double lo = a < b ? a : b, hi = a < b ? b : a;
    if (hi < 0. || lo > 1.) return false;
    if (lo <= 0.) {
        out = s0;
    } else {
        out = a < b ? l0 : l1;
    }
    return true;
}

// Device geometry records (built by the host from the boxes of the XML).
struct GBorder {
    V2 p1, p2, nd, np, la, lb;  // ends, p2-p1, outward normal, lengthened ends
    int ncls;                   // index of np among the distinct wall normals
    int pad;
};
struct GContact {
    int id;     // neighbour box
    int pad;
    V2 np;      // normal of the contact border seen from this box
};
// An interval (lo, hi) of r0.u for the translations out of one periodic box
// in which the translated segment meets contact ci of the target box and
// no other candidate.
struct TransFast {
    double lo, hi;
    int ci, pad;
};
struct GBox {
    V2 center;
    double area;
    int hull_off, nhull;
    int border_off, nborders;
    int contact_off, ncontacts;
    int reservoir;
    int tto;  // periodic box: the box it translates to (<Translate_to id>); -1 otherwise
};

// Inside or on the border of a counter-clockwise convex hull.
BTE_HD bool inside_hull(const V2* hull, int n, V2 p) {
    for (int i = 0; i < n; ++i) {
        const V2 a = hull[i], b = hull[(i + 1 == n) ? 0 : i + 1];
        if (cross(sub(b, a), sub(p, a)) < 0.) return false;
    }
    return true;
}

}  // namespace bte
