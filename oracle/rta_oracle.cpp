// rta_oracle.cpp - CPU restatement of BTE-Barna's RTAMC2D transient particle
// loop.  TEST INFRASTRUCTURE ONLY: it is the checker of the GPU engine and the
// CPU baseline of bench.py; the engine never links or calls it.
//
// Parity status: the reference cannot be built here (Boost, TBB, HDF5, MPI and
// msgpack-c are absent) and its own tests never exercise this path, so the
// restatement is pinned only at its leaves: pcg64 outputs, the libstdc++
// uniform mappings and the time grid are checked against golden vectors made
// by oracle/build_ref.py from the reference's vendored pcg-cpp / Eigen
// headers.  Geometry (restated without Boost.Geometry) and the table
// iteration orders are this restatement's own definitions; parity with the
// reference is unpinned there.
//
// What it follows (file:line of the reference):
//   src/RTA_MC2D.cpp:272-449      generators::Init_generator (isothermal walls)
//   src/RTA_MC2D.cpp:556-678      generators::diffusive_bouncing (table, bounce)
//   src/RTA_MC2D.cpp:133-148      get_bin_index
//   src/RTA_MC2D.cpp:699-769      process_segment (transient)
//   src/RTA_MC2D.cpp:843-856      get_v
//   src/RTA_MC2D.cpp:990-1386     evolparticle (transient, single material)
//   src/RTA_MC2D.cpp:2118-2124    time grid
//   src/RTA_MC2D.cpp:2262-2316    per-particle flight loop
//   src/RTA_MC2D.cpp:2326-2435    merge, scaling, cumulative sum, temperature
//   src/geometry_2d.cpp:51-158    borders (get_sides), hull, inside
//   src/geometry_2d.cpp:160-293   get_inter_side
//   src/geometry_2d.cpp:295-406   calculate_contacts, in_corner3
//   include/geometry_2d.hpp:114-125,524-561  border point, correct_corner_problem
//   include/sampling.hpp:40-114   random_dt, Grid_distribution::sample*
//   src/sampling.cpp:26-68,189-269 fill_cumulative, BE_derivative, isothermal wall
//   include/utilities.hpp:45-49,214-224,385-417  choose, almost_equal, BE functions
//   include/bulk_properties.hpp:32-47  calc_cv
//   src/isotopic_scattering.cpp:31-50  calc_percentiles_log
//
// Replay contract (shared with the GPU replay mode): particle i owns the
// stream pcg64(seed, stream = i); every draw of its life (generation, flight
// times, resampling, bounces, random choices) comes from that stream in the
// reference's order.  Uniforms are libstdc++'s generate_canonical<double,53>
// over a 64-bit engine; integers are libstdc++'s uniform_int_distribution
// (Lemire's nearly-divisionless method).  -log(u) uses bte_log (log_impl 0),
// written identically in the engine, or glibc's log (log_impl 1).

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <tuple>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../include/btegpu.h"

namespace orc {

// ---------------------------------------------------------------- numerics
constexpr double kB = 1.3806488e-23;      // include/constants.hpp:37
constexpr double hbar = 1.054571726e-34;  // include/constants.hpp:47
constexpr double nsigma = 2.828427124746190097603377448419396157138;
constexpr double PI = 3.1415926535897932384626433832795028841953;

struct geometry_error : std::runtime_error { using std::runtime_error::runtime_error; };
struct value_error : std::runtime_error { using std::runtime_error::runtime_error; };
struct input_error : std::runtime_error { using std::runtime_error::runtime_error; };
struct limit_error : std::runtime_error { using std::runtime_error::runtime_error; };

inline bool almost_equal(double a, double b, double abstol = 1e-8,
                         double reltol = 1e-5) {
    const double tol = std::fabs(abstol) + std::fabs(reltol * b);
    return std::fabs(a - b) < tol;
}

inline double bose_einstein(double omega, double T) {
    constexpr double prefactor = 1e12 * hbar / kB;
    return 1. / (std::exp(prefactor * omega / T) - 1.);
}

inline double bose_einstein_kernel(double omega, double T) {
    constexpr double prefactor = 0.5 * 1e12 * hbar / kB;
    double x = prefactor * omega / T;
    if (x < 1e-320) return 1.;
    if (x > 300.) return 0.;
    double s = x / std::sinh(x);
    return s * s;
}

// Natural log by Cody-Waite reduction x = 2^e m, m in (1/sqrt2, sqrt2], and
// the series log m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = (m-1)/(m+1).
// The engine carries the same function operation for operation, so both give
// the same bits when neither contracts a*b+c into an FMA.
inline double bte_log(double x) {
    if (!(x > 0.)) return x == 0. ? -HUGE_VAL : std::nan("");
    if (x == HUGE_VAL) return x;
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    int e = int((bits >> 52) & 0x7ff);
    if (e == 0) {  // subnormal: scale by 2^54
        double y = x * 18014398509481984.0;
        std::memcpy(&bits, &y, 8);
        e = int((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    uint64_t mb = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m;
    std::memcpy(&m, &mb, 8);
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

// ---------------------------------------------------------------- pcg64
// setseq_xsl_rr_128_64 (external/pcg-cpp-0.98/include/pcg_random.hpp:1592,1675)
struct Pcg64 {
    using u128 = unsigned __int128;
    u128 state, inc;
    static u128 mult() {
        return (u128(2549297995355413924ULL) << 64) | u128(4865540595714422341ULL);
    }
    Pcg64(uint64_t seed, uint64_t stream) {
        inc = (u128(stream) << 1) | 1u;
        state = (u128(seed) + inc) * mult() + inc;
    }
    uint64_t operator()() {
        state = state * mult() + inc;
        unsigned rot = unsigned(state >> 122) & 63u;
        uint64_t x = uint64_t(state >> 64) ^ uint64_t(state);
        return rot ? (x >> rot) | (x << ((64 - rot) & 63)) : x;
    }
};

// generate_canonical<double, 53> over a 64-bit engine: one draw, x / 2^64,
// moved below 1 when it rounds up (libstdc++ bits/random.tcc).
inline double canonical(Pcg64& g) {
    double u = double(g()) * 0x1p-64;
    if (u >= 1.0) u = 0x1.fffffffffffffp-1;
    return u;
}

// uniform_int_distribution<int>(a, b) over a 64-bit engine (libstdc++
// bits/uniform_int_dist.h, Lemire 2019).  b < a is an empty range.
inline int uniform_int(Pcg64& g, int a, int b) {
    if (b < a) throw geometry_error("random choice from an empty set");
    using u128 = unsigned __int128;
    const uint64_t range = uint64_t(int64_t(b)) - uint64_t(int64_t(a)) + 1u;
    u128 product = u128(g()) * u128(range);
    uint64_t low = uint64_t(product);
    if (low < range) {
        uint64_t threshold = (0 - range) % range;
        while (low < threshold) {
            product = u128(g()) * u128(range);
            low = uint64_t(product);
        }
    }
    return int(uint64_t(product >> 64) + uint64_t(int64_t(a)));
}

// ---------------------------------------------------------------- geometry
struct V2 {
    double x = 0, y = 0;
};
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator*(double s, V2 a) { return {s * a.x, s * a.y}; }
inline V2 operator/(V2 a, double s) { return {a.x / s, a.y / s}; }
inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
inline double cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
inline double norm(V2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }

struct Border {
    V2 p1, p2, nd, np;  // end points, p2 - p1, outward unit normal
    V2 sa, sb;          // the segment
    V2 la, lb;          // the segment lengthened at both ends (sbl)
};

// Point on a segment, including its end points; a degenerate segment is a point.
inline bool on_segment(V2 p, V2 a, V2 b) {
    V2 d = b - a;
    if (d.x == 0. && d.y == 0.) return p.x == a.x && p.y == a.y;
    if (cross(d, p - a) != 0.) return false;
    double t = dot(p - a, d);
    return t >= 0. && t <= dot(d, d);
}

// Intersection of segments s0-s1 and l0-l1 (parallel segments never meet);
// the point is taken on l0-l1 so that it lies exactly on axis-aligned borders.
inline bool seg_intersect(V2 s0, V2 s1, V2 l0, V2 l1, V2& out) {
    V2 d1 = s1 - s0, d2 = l1 - l0;
    double den = cross(d1, d2);
    if (den == 0.) return false;
    V2 w = l0 - s0;
    double t = cross(w, d2) / den;
    double u = cross(w, d1) / den;
    if (!(t >= 0. && t <= 1. && u >= 0. && u <= 1.)) return false;
    out = l0 + u * d2;
    return true;
}

// boost::geometry::intersects + intersection of two closed segments: true
// when s0-s1 and l0-l1 share a point, `out` = the first shared point (a
// crossing is taken on l0-l1; collinear overlap: the overlap end nearest s0;
// a degenerate l is its point).  Boost's own choice for collinear overlaps is
// not available here; the restatement defines it.
inline bool seg_meet(V2 s0, V2 s1, V2 l0, V2 l1, V2& out) {
    V2 d1 = s1 - s0, d2 = l1 - l0;
    if (d2.x == 0. && d2.y == 0.) {
        if (!on_segment(l0, s0, s1)) return false;
        out = l0;
        return true;
    }
    double den = cross(d1, d2);
    V2 w = l0 - s0;
    if (den != 0.) {
        double t = cross(w, d2) / den;
        double u = cross(w, d1) / den;
        if (!(t >= 0. && t <= 1. && u >= 0. && u <= 1.)) return false;
        out = l0 + u * d2;
        return true;
    }
    if (cross(w, d1) != 0.) return false;
    double dd = dot(d1, d1);
    if (dd == 0.) {
        if (!on_segment(s0, l0, l1)) return false;
        out = s0;
        return true;
    }
    double a = dot(l0 - s0, d1) / dd, b = dot(l1 - s0, d1) / dd;
    double lo = std::min(a, b), hi = std::max(a, b);
    if (hi < 0. || lo > 1.) return false;
    out = lo <= 0. ? s0 : (a < b ? l0 : l1);
    return true;
}

struct Box {
    std::vector<V2> hull;  // counter-clockwise convex hull
    V2 center;
    double area = 0;
    std::vector<Border> borders;
    std::map<std::size_t, std::vector<Border>> contacts;
    double Teq = -1, Treal = -1;
    bool reservoir = false;
    int mat = 0;                 // material (batched sweeps)
    bool periodic = false;       // <Translate_to>
    std::size_t box2translate = 0;
    V2 translation;
    std::size_t id = 0;

    bool inside(V2 p) const {
        const std::size_t n = hull.size();
        for (std::size_t i = 0; i < n; ++i) {
            V2 a = hull[i], b = hull[(i + 1) % n];
            if (cross(b - a, p - a) < 0.) return false;
        }
        return true;
    }
};

inline std::vector<V2> convex_hull(std::vector<V2> pts) {
    std::sort(pts.begin(), pts.end(), [](V2 a, V2 b) {
        return a.x < b.x || (a.x == b.x && a.y < b.y);
    });
    pts.erase(std::unique(pts.begin(), pts.end(),
                          [](V2 a, V2 b) { return a.x == b.x && a.y == b.y; }),
              pts.end());
    if (pts.size() < 3) throw input_error("a box needs three distinct vertices");
    std::vector<V2> h(2 * pts.size());
    std::size_t k = 0;
    for (std::size_t i = 0; i < pts.size(); ++i) {
        while (k >= 2 && cross(h[k - 1] - h[k - 2], pts[i] - h[k - 2]) <= 0.) --k;
        h[k++] = pts[i];
    }
    for (std::size_t i = pts.size() - 1, t = k + 1; i > 0; --i) {
        while (k >= t && cross(h[k - 1] - h[k - 2], pts[i - 1] - h[k - 2]) <= 0.) --k;
        h[k++] = pts[i - 1];
    }
    h.resize(k - 1);
    return h;
}

// Box from vertices: hull, area, area centroid, borders in the order of
// geometry_2d::get_sides (pairs i <= j of the input vertices whose midpoint,
// pushed 1e-4 away from the centre, falls outside the hull).
inline Box make_box(const std::vector<V2>& verts) {
    Box b;
    b.hull = convex_hull(verts);
    const std::size_t n = b.hull.size();
    double a2 = 0, cx = 0, cy = 0;
    V2 o = b.hull[0];
    for (std::size_t i = 0; i < n; ++i) {
        V2 p = b.hull[i] - o, q = b.hull[(i + 1) % n] - o;
        double c = cross(p, q);
        a2 += c;
        cx += (p.x + q.x) * c;
        cy += (p.y + q.y) * c;
    }
    b.area = 0.5 * a2;
    b.center = {o.x + cx / (3. * a2), o.y + cy / (3. * a2)};
    for (std::size_t i = 0; i < verts.size(); ++i) {
        V2 p1 = verts[i];
        for (std::size_t j = i; j < verts.size(); ++j) {
            V2 p2 = verts[j];
            if (norm(p1 - p2) < 1.0e-6) continue;
            V2 sc = {(p1.x + p2.x) / 2., (p1.y + p2.y) / 2.};
            V2 ncsc = sc - b.center;
            if (norm(ncsc) == 0.) continue;
            double nc = 1. / norm(ncsc);
            ncsc.x *= 1.0e-4 * nc;
            ncsc.y *= 1.0e-4 * nc;
            V2 fp = ncsc + sc;
            if (b.inside(fp)) continue;
            Border br;
            br.p1 = p1;
            br.p2 = p2;
            br.nd = p2 - p1;
            V2 npt = {br.nd.y, -br.nd.x};
            if (dot(npt, ncsc) < 0.) npt = -1. * npt;
            br.np = npt / norm(npt);
            br.sa = p1;
            br.sb = p2;
            br.la = p1 - 1.0e-6 * br.nd;
            br.lb = p2 + 1.0e-6 * br.nd;
            bool dup = false;
            for (auto& o2 : b.borders)
                if (norm(o2.np - br.np) < 1.0e-6) dup = true;
            if (!dup) b.borders.push_back(br);
            if (b.borders.size() > verts.size())
                throw geometry_error("To much borders");
        }
    }
    return b;
}

// Shared boundary of two touching convex boxes: the end points of the
// overlap of collinear edges, else a shared point.  Returns 0, 1 or 2 points.
inline std::vector<V2> touching_points(const Box& A, const Box& B) {
    std::vector<V2> pts;
    auto add = [&](V2 p) {
        for (auto& q : pts)
            if (q.x == p.x && q.y == p.y) return;
        pts.push_back(p);
    };
    const std::size_t na = A.hull.size(), nb = B.hull.size();
    for (std::size_t i = 0; i < na; ++i) {
        V2 a0 = A.hull[i], a1 = A.hull[(i + 1) % na];
        for (std::size_t j = 0; j < nb; ++j) {
            V2 b0 = B.hull[j], b1 = B.hull[(j + 1) % nb];
            if (on_segment(b0, a0, a1)) add(b0);
            if (on_segment(b1, a0, a1)) add(b1);
            if (on_segment(a0, b0, b1)) add(a0);
            if (on_segment(a1, b0, b1)) add(a1);
        }
    }
    if (pts.size() > 2) throw geometry_error("overlapping boxes are not supported");
    std::sort(pts.begin(), pts.end(), [](V2 a, V2 b) {
        return a.x < b.x || (a.x == b.x && a.y < b.y);
    });
    return pts;
}

inline bool bboxes_meet(const Box& A, const Box& B) {
    double ax0 = A.hull[0].x, ax1 = ax0, ay0 = A.hull[0].y, ay1 = ay0;
    for (auto& p : A.hull) {
        ax0 = std::min(ax0, p.x); ax1 = std::max(ax1, p.x);
        ay0 = std::min(ay0, p.y); ay1 = std::max(ay1, p.y);
    }
    double bx0 = B.hull[0].x, bx1 = bx0, by0 = B.hull[0].y, by1 = by0;
    for (auto& p : B.hull) {
        bx0 = std::min(bx0, p.x); bx1 = std::max(bx1, p.x);
        by0 = std::min(by0, p.y); by1 = std::max(by1, p.y);
    }
    return !(bx0 > ax1 || ax0 > bx1 || by0 > ay1 || ay0 > by1);
}

inline void calculate_contacts(std::vector<Box>& sys) {
    for (auto& me : sys) {
        for (auto& other : sys) {
            if (other.id == me.id) continue;
            if (!bboxes_meet(me, other)) continue;  // boxes apart cannot touch
            auto pinter = touching_points(me, other);
            if (pinter.empty()) continue;
            Border cb;
            if (pinter.size() == 1 || norm(pinter[1] - pinter[0]) < 1.0e-6) {
                cb.p1 = cb.p2 = pinter[0];
                cb.sa = cb.sb = pinter[0];
                cb.np = (cb.p1 - me.center) / norm(cb.p1 - me.center);
                me.contacts[other.id] = {cb};
                continue;
            }
            cb.p1 = pinter[0];
            cb.p2 = pinter[1];
            cb.nd = cb.p2 - cb.p1;
            V2 sc = {(cb.p1.x + cb.p2.x) / 2., (cb.p1.y + cb.p2.y) / 2.};
            V2 ncsc = sc - me.center;
            V2 npt = {cb.nd.y, -cb.nd.x};
            if (dot(npt, ncsc) < 0.) npt = -1. * npt;
            cb.np = npt / norm(npt);
            cb.sa = cb.p1;
            cb.sb = cb.p2;
            cb.la = cb.p1 - 1.0e-6 * cb.nd / norm(cb.nd);
            cb.lb = cb.p2 + 1.0e-6 * cb.nd / norm(cb.nd);
            me.contacts[other.id] = {cb};
        }
        if (me.contacts.empty() && sys.size() > 1)
            throw geometry_error("There are unconnected boxes");
    }
}

struct Hit {
    double time;
    V2 rf;
    std::vector<int> bids;
};

// geometry_2d::get_inter_side, src/geometry_2d.cpp:160-293.
inline Hit get_inter_side(const Box& box, V2 r0, V2 v, double dt) {
    V2 pf = {r0.x + dt * v.x, r0.y + dt * v.y};
    double time = 1.0e+7;
    V2 rf;
    std::vector<int> bids;
    bool already_there = true;
    int border_id = 0;
    for (auto& b : box.borders) {
        V2 rin;
        if (seg_intersect(r0, pf, b.la, b.lb, rin) && !on_segment(r0, b.la, b.lb)) {
            if (dot(b.np, v) > 0.) {
                double tx = (std::fabs(v.x) < 1.0e-6) ? -1 : (rin.x - r0.x) / v.x;
                double ty = (std::fabs(v.y) < 1.0e-6) ? -1 : (rin.y - r0.y) / v.y;
                double newtime = std::max(tx, ty);
                if (newtime == time) bids.push_back(border_id);
                if (newtime < time) {
                    bids.clear();
                    rf = rin;
                    time = newtime;
                    already_there = false;
                    bids.push_back(border_id);
                }
            }
        }
        border_id++;
    }
    if (already_there) {
        V2 p0p = {r0.x - 1.0e-6 * v.x, r0.y - 1.0e-6 * v.y};
        border_id = 0;
        for (auto& b : box.borders) {
            V2 rin;
            if (seg_intersect(p0p, pf, b.la, b.lb, rin)) {
                if (dot(b.np, v) > 0.) {
                    double tx = (std::fabs(v.x) < 1.0e-6) ? -1.0e+8 : (rin.x - r0.x) / v.x;
                    double ty = (std::fabs(v.y) < 1.0e-6) ? -1.0e+8 : (rin.y - r0.y) / v.y;
                    double newtime = std::max(tx, ty);
                    if (newtime == time) bids.push_back(border_id);
                    if (std::fabs(newtime) < time) {
                        bids.clear();
                        rf = rin;
                        time = newtime;
                        bids.push_back(border_id);
                    }
                }
            }
            border_id++;
        }
        if (time > 1.0e+6) throw geometry_error("Error to huge time");
    }
    if (almost_equal(time, 0.)) time = 0.;
    if (time < 0.) throw geometry_error("Bad time");
    return {time, rf, bids};
}

// ---------------------------------------------------------------- distributions
// Grid_distribution::fill_cumulative, src/sampling.cpp:26-44
inline std::vector<double> fill_cumulative(const std::vector<double>& p) {
    if (*std::min_element(p.begin(), p.end()) < 0.)
        throw value_error("probabilities must be >= 0.");
    std::vector<double> c;
    c.reserve(p.size());
    std::partial_sum(p.begin(), p.end(), std::back_inserter(c));
    double last = c.back();
    for (auto& x : c) x /= last;
    return c;
}

inline std::size_t lower_bound_idx(const std::vector<double>& c, double u) {
    return std::size_t(std::lower_bound(c.begin(), c.end(), u) - c.begin());
}

// random_dt, include/sampling.hpp:40-46: -log(u) / w from one uniform, with
// bte_log (log_impl 0) or glibc's log (log_impl 1).
inline double random_dt(double w, Pcg64& rng, int log_impl) {
    if (w == 0.) throw value_error("invalid scattering rate");
    double u = canonical(rng);
    return -(log_impl == 0 ? bte_log(u) : std::log(u)) / w;
}

struct Modes {
    int nq = 0, nb = 0, grid[3] = {0, 0, 0};
    std::vector<double> omega, vx, vy, vz, w;
    double dq[9] = {0};
    double V = 0, c = 0;
    std::size_t n() const { return std::size_t(nq) * nb; }
};

// BE_derivative_distribution, src/sampling.cpp:47-68: pmf C(omega, T) w,
// zero for omega <= 0.
inline std::vector<double> be_derivative_pmf(const Modes& m, const std::vector<double>& w, double T) {
    std::vector<double> pmf(m.n());
    for (std::size_t k = 0; k < m.n(); ++k)
        pmf[k] = m.omega[k] <= 0. ? 0. : bose_einstein_kernel(m.omega[k], T) * w[k];
    return pmf;
}

// outTref_distribution, src/sampling.cpp:271-330: pmf omega |n(Tinit) -
// n(Tref)|, zero where omega is almost 0; returns cumulsum.
inline double out_tref_pmf(const Modes& m, double Tinit, double Tref, std::vector<double>& pmf) {
    pmf.assign(m.n(), 0.);
    for (std::size_t k = 0; k < m.n(); ++k) {
        const double om = m.omega[k];
        if (almost_equal(om, 0.)) continue;
        pmf[k] = om * std::fabs(bose_einstein(om, Tinit) - bose_einstein(om, Tref));
    }
    return 1.0e+12 * hbar * std::accumulate(pmf.begin(), pmf.end(), 0.);
}

// Nabla_T_distribution, src/sampling.cpp:118-164 (theta = 0): pmf
// |v.gradT C(omega, T)| with the sign of -v.gradT; returns cumulsum.
inline double nabla_t_pmf(const Modes& m, double gx, double gy, double T, std::vector<double>& pmf,
                          std::vector<int>& sign) {
    pmf.assign(m.n(), 0.);
    sign.assign(m.n(), 1);
    for (std::size_t k = 0; k < m.n(); ++k) {
        double vgradT = -(gx * m.vx[k] + gy * m.vy[k] + 0. * m.vz[k]);
        if (m.omega[k] == 0.) {
            pmf[k] = 0.;
        } else {
            pmf[k] = std::fabs(vgradT * bose_einstein_kernel(m.omega[k], T));
            sign[k] = vgradT >= 0 ? 1 : -1;
        }
    }
    return kB * std::accumulate(pmf.begin(), pmf.end(), 0.);
}

// The particle numbers of the distributions' Ntogenerate before stochastic
// rounding: time spf cumulsum / (Eff nq) for walls (src/sampling.cpp:243),
// time vol cumulsum / (Eff nq) for Nabla_T (:166), vol cumulsum / (Eff nq)
// for outTref (:310); get_energy is vol cumulsum / nq (:185, :328) and
// get_flux sign cumulsum / (nq vuc) (:263-269).
inline double gen_scaled(double time, double f, double cumulsum, double Eff, double nq) {
    return time * f * cumulsum / (Eff * nq);
}
inline double gen_plain(double vol, double cumulsum, double Eff, double nq) {
    return vol * cumulsum / (Eff * nq);
}
inline double dist_energy(double vol, double cumulsum, double nq) { return vol * cumulsum / nq; }
inline double wall_flux(int sign, double cumulsum, double nq, double vuc) { return sign * (cumulsum / (nq * vuc)); }

// Isothermal_wall_distribution, src/sampling.cpp:189-269 (theta = 0), for
// the outward normal n of the wall seen from the emitting side; returns
// cumulsum.
inline double wall_pmf(const Modes& m, V2 n, double Tw, double Te, std::vector<double>& pmf) {
    pmf.assign(m.n(), 0.);
    for (std::size_t k = 0; k < m.n(); ++k) {
        const double vn = n.x * m.vx[k] + n.y * m.vy[k] + 0. * m.vz[k];
        if (vn <= 0. || almost_equal(0., m.omega[k]))
            pmf[k] = 0.;
        else
            pmf[k] = vn * m.omega[k] * std::fabs(bose_einstein(m.omega[k], Tw) - bose_einstein(m.omega[k], Te));
    }
    return 1.0e+12 * hbar * std::accumulate(pmf.begin(), pmf.end(), 0.);
}

struct WallGen {
    std::size_t res, box;     // reservoir id, injection box id
    Border b;                 // contact border seen from the reservoir
    std::vector<double> cdf;  // Isothermal_wall_distribution
    int sign;
    double flux;              // J nm^-2 ps^-1 (get_flux)
    double cumulsum;          // 1e12 hbar sum(pmf)
};

struct Sim {
    Modes m;
    std::vector<Box> sys;
    double thickness = 0;
    // first global mode of this material's table (several materials: their
    // tables one after the other, as the spectral tallies index them)
    std::size_t mode_off = 0;
    // run state
    std::vector<double> timegrid;
    std::vector<double> resample_cdf;
    // per-material rates and post-scattering CDFs (material 0 = w and
    // resample_cdf when no materials are given)
    std::vector<std::vector<double>> mat_w, mat_res;
    std::vector<double> mat_T0;
    const std::vector<double>& w_of(int mt) const { return mat_w.empty() ? m.w : mat_w[std::size_t(mt)]; }
    const std::vector<double>& res_of(int mt) const {
        return mat_res.empty() ? resample_cdf : mat_res[std::size_t(mt)];
    }
    std::vector<std::vector<std::pair<std::size_t, double>>> lambert;  // rows by ascending mode
    std::vector<WallGen> gens;
    std::vector<double> gen_cum;  // cumulative generator weights
    double Eeff = 0, energy = 0;
    // initial-deviation source (outTref_distribution per box)
    std::vector<std::size_t> init_box;
    std::vector<int> init_sign;
    std::vector<std::vector<double>> init_cdf;
    std::vector<long long> init_first;
};

// generators::diffusive_bouncing constructor, src/RTA_MC2D.cpp:556-626, with
// trivial q-point symmetry (every q is its own class; class 0 is Gamma).
inline void build_lambert(Sim& S) {
    const Modes& m = S.m;
    const std::size_t nq = m.nq, nb = m.nb;
    std::vector<double> sig(nq * nb);
    for (std::size_t iq = 0; iq < nq; ++iq)
        for (std::size_t im = 0; im < nb; ++im) {
            std::size_t k = iq * nb + im;
            double v[3] = {m.vx[k], m.vy[k], m.vz[k]};
            double r[3];
            for (int j = 0; j < 3; ++j)
                r[j] = v[0] * m.dq[0 + 3 * j] + v[1] * m.dq[1 + 3 * j] + v[2] * m.dq[2 + 3 * j];
            sig[k] = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / std::sqrt(12.);
        }
    // calc_percentiles_log, src/isotopic_scattering.cpp:31-50 (column-major
    // (nb x nq) order, sorted anyway)
    std::vector<double> ls(sig.size());
    for (std::size_t k = 0; k < sig.size(); ++k)
        ls[k] = sig[k] == 0. ? std::numeric_limits<double>::lowest() : std::log(sig[k]);
    std::sort(ls.begin(), ls.end());
    const std::size_t N = ls.size();
    double p25 = ls[25 * N / 100], p75 = ls[75 * N / 100];
    double lbound = std::exp(p25 - 1.5 * (p75 - p25));
    for (auto& s : sig)
        if (s < lbound) s = lbound;
    S.lambert.assign(nq * nb, {});
    const double root_two_pi = std::sqrt(2. * PI);
    // rows are filled in (iq2, im2) order, i.e. by ascending outgoing mode;
    // threads own disjoint ranges of iq1
    auto work = [&](std::size_t q0, std::size_t q1) {
        for (std::size_t iq1 = q0; iq1 < q1; ++iq1)
            for (std::size_t iq2 = 1; iq2 < nq; ++iq2)
                for (std::size_t im1 = 0; im1 < nb; ++im1)
                    for (std::size_t im2 = 0; im2 < nb; ++im2) {
                        std::size_t k1 = iq1 * nb + im1, k2 = iq2 * nb + im2;
                        if (almost_equal(0., m.omega[k1]) || almost_equal(0., m.omega[k2]))
                            continue;
                        double sigma = std::hypot(sig[k1], sig[k2]);
                        double delta = std::fabs(m.omega[k1] - m.omega[k2]);
                        if (delta <= nsigma * sigma) {
                            double e = delta;
                            e *= -e;
                            e /= 2 * sigma * sigma;
                            double pdf = std::exp(e);
                            pdf /= sigma * root_two_pi;
                            S.lambert[k1].push_back({k2, pdf});
                        }
                    }
    };
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back(work, 1 + (nq - 1) * t / nt, 1 + (nq - 1) * (t + 1) / nt);
    for (auto& t : th) t.join();
}

inline V2 get_v(const Modes& m, std::size_t k) {
    V2 v = {m.vx[k], m.vy[k]};
    if (almost_equal(v.x, 0.)) v.x = 0.;
    if (almost_equal(v.y, 0.)) v.y = 0.;
    return v;
}

// diffusive_bouncing::bounce, src/RTA_MC2D.cpp:635-678.  The weights are
// summed in ascending outgoing-mode order; a cumulative value that repeats
// keeps the later mode (std::map assignment); a draw above the last
// cumulative value takes the last mode.
inline std::size_t bounce(const Sim& S, V2 npout, std::size_t imode, Pcg64& rng) {
    const auto& tm = S.lambert[imode];
    std::vector<std::pair<std::size_t, double>> states;
    double cum = 0.;
    for (auto& [imf, econ] : tm) {
        V2 v = get_v(S.m, imf);
        double vn = -(npout.x * v.x + npout.y * v.y);
        if (vn < 0. || almost_equal(vn, 0.)) continue;
        cum += vn * econ;
        states.push_back({imf, vn * econ});
    }
    std::vector<std::pair<double, std::size_t>> st2;
    double cum2 = 0;
    for (auto& [imf, tran] : states) {
        cum2 += tran / cum;
        if (!st2.empty() && st2.back().first == cum2)
            st2.back().second = imf;
        else
            st2.push_back({cum2, imf});
    }
    double s = canonical(rng);
    if (st2.empty()) throw geometry_error("diffuse wall without outgoing states");
    auto it = std::lower_bound(st2.begin(), st2.end(), s,
                               [](const std::pair<double, std::size_t>& a, double x) {
                                   return a.first < x;
                               });
    if (it == st2.end()) --it;
    return it->second;
}

// Generators of Init_generator, src/RTA_MC2D.cpp:289-418, in the order
// (reservoir id, injection box id).
inline void build_generators(Sim& S, double /*T0*/, bool required = true, int only_mat = -1) {
    S.gens.clear();
    const Modes& m = S.m;
    const double vuc = m.V * S.thickness / m.c;
    for (auto& s : S.sys) {
        if (!s.reservoir) continue;
        if (only_mat >= 0 && s.mat != only_mat) continue;  // another material's reservoir
        for (auto& [c, bv] : s.contacts) {
            if (S.sys[c].reservoir || S.sys[c].periodic) continue;
            if (only_mat >= 0 && S.sys[c].mat != s.mat && !almost_equal(norm(bv[0].p2 - bv[0].p1), 0.))
                throw input_error("Injection from material A to B is not allowed");
            const Border& b = bv[0];
            if (almost_equal(norm(b.p2 - b.p1), 0.)) continue;
            if (almost_equal(s.Teq, S.sys[c].Teq)) continue;
            WallGen g;
            g.res = s.id;
            g.box = c;
            g.b = b;
            const double Tw = s.Teq, Te = S.sys[c].Teq;
            std::vector<double> pmf;
            double cumulsum = wall_pmf(m, b.np, Tw, Te, pmf);
            g.sign = (Tw - Te) >= 0 ? 1 : -1;
            g.cdf = fill_cumulative(pmf);
            g.flux = wall_flux(g.sign, cumulsum, double(m.nq), vuc);
            g.cumulsum = cumulsum;
            S.gens.push_back(std::move(g));
        }
    }
    if (S.gens.empty()) {
        if (required) throw input_error("no isothermal wall generator (no reservoir with a different Teq)");
        S.energy = 0.;
        return;
    }
    std::vector<double> ws;
    double total = 0;
    for (auto& g : S.gens) {
        double Lb = norm(g.b.p2 - g.b.p1);
        double e = std::fabs(g.flux) * Lb * S.thickness;
        total += e;
        ws.push_back(e);
    }
    double wnorm = std::accumulate(ws.begin(), ws.end(), 0.);
    double cum = 0;
    S.gen_cum.clear();
    for (double w : ws) {
        cum += w / wnorm;
        S.gen_cum.push_back(cum);
    }
    S.energy = total;
}

struct Particle {
    V2 pos;
    std::size_t q = 0, alpha = 0;
    int sign = 1;
    double t = 0;
    std::size_t box = 0;
    int mat = 0;  // material of the birth box, kept for the particle's life
};

struct Tally {
    std::size_t nboxes = 0, nbins = 0;
    std::vector<double> gz, jx, jy;
    std::vector<__int128> ex;  // [box][bin][3]
    // spectral decomposition: box -> location, per-mode time [loc][bin][mode]
    const std::vector<int>* loc = nullptr;
    std::size_t nmodes = 0;
    std::vector<__int128> spec;
    std::vector<int64_t> scnt;  // steady: signed segments per [loc][mode]
    int64_t events = 0, wall_hits = 0, crossings = 0, absorbed = 0, nudges = 0,
            quirks = 0, specular = 0, translations = 0;
    int64_t interface_hits = 0, interface_transmissions = 0;  // diffuse mismatch
    void init(std::size_t nbx, std::size_t nbn) {
        nboxes = nbx;
        nbins = nbn;
        gz.assign(nbx * nbn, 0.);
        jx = gz;
        jy = gz;
        ex.assign(nbx * nbn * 3, 0);
    }
};

// Fixed-point quantisation of one contribution (scale 2^44, |x| < 2^18).
inline __int128 quant(double x) {
    double y = x * 17592186044416.0;  // 2^44
    if (!(std::fabs(y) < 4611686018427387904.0))  // 2^62
        throw limit_error("tally contribution out of fixed-point range");
    return __int128(std::llrint(y));
}

inline std::size_t bin_index(const std::vector<double>& g, double t) {
    long k = long(std::lower_bound(g.begin(), g.end(), t) - g.begin()) - 1;
    long hi = long(g.size()) - 2;
    return std::size_t(std::clamp(k, 0L, hi));
}

// process_segment (transient), src/RTA_MC2D.cpp:699-769, without the
// spectral decomposition.
inline void process_segment(const Sim& S, Tally& T, std::size_t ibox, double t0,
                            double t1, int sign, V2 v, std::size_t mode = 0) {
    const int lc = T.loc ? (*T.loc)[ibox] : -1;
    const auto& g = S.timegrid;
    std::size_t sb = bin_index(g, t0), eb = bin_index(g, t1);
    double delta_t = t1 - t0;
    for (std::size_t i = sb; i <= eb; ++i) {
        double lo = std::max(g[i] - t0, 0.);
        double hi = std::min(g[i + 1] - t0, delta_t);
        double contr = double(sign) * std::max(hi - lo, 0.);
        std::size_t k = ibox * T.nbins + i;
        T.gz[k] += contr;
        T.jx[k] += v.x * contr;
        T.jy[k] += v.y * contr;
        T.ex[3 * k + 0] += quant(contr);
        T.ex[3 * k + 1] += quant(v.x * contr);
        T.ex[3 * k + 2] += quant(v.y * contr);
        // per-mode time at a spectral location (the gamma weights, v and
        // 1/omega of the reference's sd tallies are linear in it)
        if (lc >= 0) T.spec[(std::size_t(lc) * T.nbins + i) * T.nmodes + S.mode_off + mode] += quant(contr);
    }
}

struct Opts {
    bool ballistic = false;
    int log_impl = 0;
    double specularity = 0.;  // p of void walls (this engine's extension)
};

// Specular image of mode k at a wall of outward normal np on the q grid:
// q mirrored across the wall, same branch; -1 when the wall is not
// axis-aligned or the image does not carry the reflected velocity.
inline long long mirror_mode(const Sim& S, V2 np, std::size_t k) {
    const Modes& m = S.m;
    const int n1 = m.grid[0], n2 = m.grid[1];
    if (n1 < 1 || n2 < 1 || std::size_t(n1) * std::size_t(n2) != std::size_t(m.nq)) return -1;
    const bool ny = (np.x == 0. && std::fabs(np.y) == 1.);
    const bool nx = (np.y == 0. && std::fabs(np.x) == 1.);
    if (!nx && !ny) return -1;
    const int iq = int(k / std::size_t(m.nb)), ib = int(k % std::size_t(m.nb));
    int i = iq / n2, j = iq % n2;
    if (ny) j = (n2 - j) % n2;
    if (nx) i = (n1 - i) % n1;
    const std::size_t k2 = std::size_t(i * n2 + j) * std::size_t(m.nb) + std::size_t(ib);
    const V2 a = get_v(m, k), b = get_v(m, k2);
    const double vn_in = np.x * a.x + np.y * a.y, vn_out = np.x * b.x + np.y * b.y;
    const double vt_in = nx ? a.y : a.x, vt_out = nx ? b.y : b.x;
    if (vn_out == -vn_in && vt_out == vt_in && m.omega[k2] > 0.) return (long long)k2;
    return -1;
}

// correct_corner_problem, include/geometry_2d.hpp:524-561: the winner box.
inline std::size_t correct_corner_problem(const Sim& S, V2 rf, V2 v,
                                          const std::vector<std::size_t>& cand,
                                          Pcg64& rng) {
    std::vector<std::size_t> finalist;
    for (auto c : cand) {
        int nb = 0;
        for (auto& b : S.sys[c].borders)
            if (on_segment(rf, b.la, b.lb) && dot(b.np, v) > 0.) nb++;
        if (nb <= 1) finalist.push_back(c);
    }
    if (finalist.empty()) throw geometry_error("corner without a candidate box");
    return finalist[std::size_t(uniform_int(rng, 0, int(finalist.size()) - 1))];
}

// geometry_2d::translate, include/geometry_2d.hpp:366-493.  The particle in
// periodic box `ib` jumps by 1.0005 x the translation into box2translate and
// from there into the first-level neighbour the jump segment meets.  As in
// the reference, boost's intersection() appends to one point list, so every
// contact met by the segment reports the first contact's point, and with
// several candidates the point is read at the drawn position of the
// filtered list.
inline std::pair<std::size_t, V2> translate(const Sim& S, std::size_t ib, V2 r0, V2 v, Pcg64& rng) {
    const Box& me = S.sys[ib];
    if (!me.periodic) throw geometry_error("Error: this can only be used in periodic cells");
    V2 T = 1.0005 * me.translation;
    std::size_t tib = me.box2translate;
    if (tib >= S.sys.size() || almost_equal(norm(T), 0.))
        throw geometry_error("Error: Bad id for mapping of periodic cells");
    V2 p1 = r0 + T;
    const Box& TB = S.sys[tib];
    V2 tp;
    bool found = false;
    for (auto& b : TB.borders)
        if (seg_meet(r0, p1, b.la, b.lb, tp)) {
            found = true;
            break;
        }
    if (!found) throw geometry_error("Error in translation, no box found");
    V2 tp_T = tp - (1.0e-6 * me.translation) / norm(me.translation);
    V2 tp_v = tp + (1.0e-6 * v) / norm(v);
    std::vector<V2> rf;
    std::vector<std::size_t> pboxes;
    std::vector<V2> rinter;  // boost's output list: appended, never cleared in the loop
    for (auto& [ibc, bv] : TB.contacts) {
        const Border& cb = bv[0];
        bool point = cb.p1.x == cb.p2.x && cb.p1.y == cb.p2.y;
        V2 la = point ? cb.p1 : cb.la, lb = point ? cb.p1 : cb.lb;
        V2 xin;
        bool here_i = seg_meet(r0, p1, la, lb, xin);
        bool here_T = S.sys[ibc].inside(tp);
        bool here_Tv = S.sys[ibc].inside(tp_v);
        bool here_TT = S.sys[ibc].inside(tp_T);
        bool here = here_i || here_T || here_Tv || here_TT;
        if (ibc == tib || !here || S.sys[ibc].periodic || S.sys[ibc].reservoir) continue;
        if (here_i) {
            rinter.push_back(xin);
            rf.push_back(rinter[0]);
        } else if (here_T) {
            rf.push_back(tp);
        } else if (here_Tv) {
            rf.push_back(tp_v);
        } else {
            rf.push_back(tp_T);
        }
        pboxes.push_back(ibc);
    }
    if (pboxes.size() > 1) {
        std::vector<std::size_t> pboxes2;
        for (std::size_t k = 0; k < pboxes.size(); ++k)
            if (S.sys[pboxes[k]].inside(rf[k] + 1.0e-6 * v)) pboxes2.push_back(pboxes[k]);
        if (pboxes2.empty()) throw geometry_error("translation: no candidate box ahead");
        std::size_t pos = std::size_t(uniform_int(rng, 0, int(pboxes2.size()) - 1));
        return {pboxes2[pos], rf[pos]};
    }
    if (pboxes.size() == 1) return {pboxes[0], rf[0]};
    throw geometry_error("Error in Translation");
}

// ---- Diffuse mismatch interfaces between materials
// (Diffuse_mismatch_distribution, src/sampling.cpp:437-880, without the
// layer coupling of LDMM; change_material_diffuse, src/RTA_MC2D.cpp:871-964).

// Gaussian_for_DOS (include/dos.hpp:28-82) of mode k: mu = omega, sigma =
// scalebroad * base_sigma(v) (include/qpoint_grid.hpp:179-181), the
// compatibility window [lbound, ubound] of nsigma sigmas (lbound 0 when it
// would be negative); no distribution when mu or sigma is 0.
struct DosGauss {
    double mu = 0, sigma = 0, lbound = 0, ubound = 0;
    bool has = false;
};
inline DosGauss dos_gauss(const Modes& m, std::size_t k, double scalebroad) {
    const double v[3] = {m.vx[k], m.vy[k], m.vz[k]};
    double r[3];
    for (int j = 0; j < 3; ++j) r[j] = v[0] * m.dq[0 + 3 * j] + v[1] * m.dq[1 + 3 * j] + v[2] * m.dq[2 + 3 * j];
    DosGauss g;
    g.mu = m.omega[k];
    g.sigma = scalebroad * (std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / std::sqrt(12.));
    const bool truncated = g.mu - nsigma * g.sigma < 0.;
    g.lbound = truncated ? 0. : g.mu - nsigma * g.sigma;
    g.ubound = g.mu + nsigma * g.sigma;
    g.has = !(g.mu == 0. || g.sigma == 0.);
    return g;
}
// boost::math::pdf of the normal distribution, in its own order of operations
inline double dos_pdf(const DosGauss& g, double x) {
    if (!g.has) return 0.;
    double e = x - g.mu;
    e *= -e;
    e /= 2 * g.sigma * g.sigma;
    double pdf = std::exp(e);
    pdf /= g.sigma * std::sqrt(2. * PI);
    return pdf;
}

// One interface: per incident mode of side A (0) or B (1), its lookup
// entries (side out, mode index out, cumulative probability), the
// cumulative running over all incident modes of that side.
struct DmmEntry {
    int side;
    std::size_t idx;
    double cum;
};
struct Dmm {
    std::size_t nb[2] = {0, 0};
    std::vector<std::vector<DmmEntry>> in[2];
};

// The Diffuse_mismatch_distribution constructor: normal n points from A to
// B; V[s] are the cells' volumes scaled to the thickness.
inline Dmm build_dmm(const Modes& A, const Modes& B, double VA, double VB, V2 n, double scalebroad, double Tref) {
    const double nn = std::sqrt(n.x * n.x + n.y * n.y);
    if (nn == 0.) throw value_error("invalid normal vector");
    const double ux = n.x / nn, uy = n.y / nn, uz = 0. / nn;
    struct Mode {
        int side;
        std::size_t branch, q;
        double vn, C;
        DosGauss g;
    };
    const Modes* M[2] = {&A, &B};
    const double V[2] = {VA, VB};
    std::vector<Mode> all;
    all.reserve(A.n() + B.n());
    for (int s = 0; s < 2; ++s) {
        const Modes& m = *M[s];
        for (std::size_t q = 0; q < std::size_t(m.nq); ++q)
            for (std::size_t b = 0; b < std::size_t(m.nb); ++b) {
                const std::size_t k = q * std::size_t(m.nb) + b;
                Mode md;
                md.side = s;
                md.branch = b;
                md.q = q;
                md.vn = ux * m.vx[k] + uy * m.vy[k] + uz * m.vz[k];
                md.C = bose_einstein_kernel(m.omega[k], Tref) / (kB * double(m.nq) * V[s]);
                md.g = dos_gauss(m, k, scalebroad);
                all.push_back(md);
            }
    }
    Dmm D;
    D.nb[0] = std::size_t(A.nb);
    D.nb[1] = std::size_t(B.nb);
    D.in[0].assign(A.n(), {});
    D.in[1].assign(B.n(), {});
    std::vector<std::vector<double>> raw[2];
    raw[0].assign(A.n(), {});
    raw[1].assign(B.n(), {});
    auto incident = [](const Mode& md) { return (md.side == 0 && md.vn > 0.) || (md.side == 1 && md.vn < 0.); };
    auto emission = [](const Mode& md) { return (md.side == 0 && md.vn < 0.) || (md.side == 1 && md.vn > 0.); };
    // every allowed transition, per incident mode (independent lists,
    // filled on several threads; the totals are summed below in the
    // reference's order)
    auto work = [&](std::size_t lo, std::size_t hi) {
        for (std::size_t li = lo; li < hi; ++li) {
            const Mode& mi = all[li];
            if (!incident(mi)) continue;
            const std::size_t idx_in = mi.branch + mi.q * D.nb[mi.side];
            const double target = mi.g.mu;
            auto& lst = D.in[mi.side][idx_in];
            auto& rw = raw[mi.side][idx_in];
            for (const Mode& c : all) {
                if (!(emission(c) && target > c.g.lbound && target < c.g.ubound)) continue;
                const double r = c.C * std::fabs(c.vn) * 1.0 * dos_pdf(c.g, target);
                lst.push_back(DmmEntry{c.side, c.branch + c.q * D.nb[c.side], 0.});
                rw.push_back(r);
            }
        }
    };
    {
        const std::size_t nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (std::size_t t = 0; t < nt; ++t)
            th.emplace_back(work, all.size() * t / nt, all.size() * (t + 1) / nt);
        for (auto& t : th) t.join();
    }
    double total[2] = {0., 0.};
    for (const Mode& mi : all) {
        if (!incident(mi)) continue;
        for (double r : raw[mi.side][mi.branch + mi.q * D.nb[mi.side]]) total[mi.side] += r;
    }
    // incident modes without a transition: the reflection of the closest
    // frequency.  The reference records it with the side of the last mode
    // it scanned (its side_out variable is assigned for every candidate),
    // which is always B: an incident mode of A leaves into B with the index
    // of A's reflection read in B's table.  Kept.
    const int fix_side = all.empty() ? 0 : all.back().side;
    for (const Mode& mi : all) {
        if (!incident(mi)) continue;
        const std::size_t idx_in = mi.branch + mi.q * D.nb[mi.side];
        if (!D.in[mi.side][idx_in].empty()) continue;
        const double target = mi.g.mu;
        long long best = -1;
        double dmin = 1e300;
        for (std::size_t ci = 0; ci < all.size(); ++ci) {
            const Mode& c = all[ci];
            if (c.side != mi.side || !emission(c)) continue;
            const double d = std::fabs(c.g.mu - target);
            if (d < dmin) {
                best = (long long)ci;
                dmin = d;
            }
        }
        if (best < 0) throw value_error("no matching mode was found for some incident mode");
        const Mode& c = all[std::size_t(best)];
        const double r = c.C * std::fabs(c.vn) * 1.0;
        const std::size_t io = c.branch + c.q * D.nb[c.side];
        if (io >= (fix_side == 0 ? A.n() : B.n()))
            throw value_error("a reflection index beyond the other material's table");
        D.in[mi.side][idx_in].push_back(DmmEntry{fix_side, io, 0.});
        raw[mi.side][idx_in].push_back(r);
        total[mi.side] += r;
    }
    // cumulative probabilities over the incident modes in index order
    for (int s = 0; s < 2; ++s) {
        double pc = 0.;
        for (std::size_t i = 0; i < D.in[s].size(); ++i)
            for (std::size_t j = 0; j < D.in[s][i].size(); ++j) {
                pc += raw[s][i][j] / total[s];
                D.in[s][i][j].cum = pc;
            }
    }
    return D;
}

// Diffuse_mismatch_distribution::reemit (src/sampling.cpp:831-880): p
// uniform between the first and the last cumulative value of the incident
// mode's entries, the first entry whose value is not below p.  Returns the
// side out (-1: no entry, the reference's 'X').
inline int dmm_reemit(const Dmm& D, int side_in, std::size_t idx_in, Pcg64& rng, std::size_t& idx_out) {
    const auto& L = D.in[side_in][idx_in];
    if (L.empty()) return -1;
    const double lo = L.front().cum, hi = L.back().cum;
    const double p = canonical(rng) * (hi - lo) + lo;
    for (const DmmEntry& e : L)
        if (e.cum >= p) {
            idx_out = e.idx;
            return e.side;
        }
    idx_out = L.back().idx;  // p above the last value by rounding
    return L.back().side;
}

// The interfaces of a multi-material geometry, keyed by (material A,
// material B, contact normal from A to B).
struct DmmSet {
    std::map<std::tuple<int, int, double, double>, Dmm> tab;
    std::vector<const Modes*> modes;  // per material
};

// change_material_diffuse (src/RTA_MC2D.cpp:871-964): the particle meets
// the contact with box inew of another material; the interface of (its
// material, inew's, the contact normal) re-emits it on either side; the
// flight ends there (dt = 0).  An incident mode without entries (the
// reference's 'X') crosses with its mode unchanged, as there.
inline void dmm_cross(const Sim& S, const DmmSet& M, Particle& p, std::size_t inew, double& dt, Pcg64& rng,
                      Tally& T) {
    const Box& a = S.sys[p.box];
    V2 nw = {0., 0.};
    for (auto& [c, bb] : a.contacts)
        if (c == inew) {
            nw.x += bb[0].np.x;
            nw.y += bb[0].np.y;
        }
    const auto it = M.tab.find(std::make_tuple(a.mat, S.sys[inew].mat, nw.x, nw.y));
    if (it == M.tab.end()) throw geometry_error("interface without a mismatch table");
    const Dmm& D = it->second;
    std::size_t idx_out = 0;
    const int side = dmm_reemit(D, 0, p.alpha + p.q * D.nb[0], rng, idx_out);
    if (side >= 0) {
        p.q = idx_out / D.nb[side];
        p.alpha = idx_out % D.nb[side];
    } else {
        T.quirks++;
    }
    T.interface_hits++;
    if (side != 0) {
        p.box = inew;
        T.interface_transmissions++;
    }
    dt = 0.;
}

// evolparticle (transient, one material), src/RTA_MC2D.cpp:990-1386.
inline void evolparticle(const Sim& S, Particle& p, V2 v, double& dt, Pcg64& rng,
                         Tally& T, const Opts& o, const DmmSet* dmm = nullptr) {
    const std::size_t nb = S.m.nb;
    V2 opos = p.pos;
    const Box& box = S.sys[p.box];
    if (box.periodic) {  // Apply PBC, :1034-1042
        auto sol = translate(S, p.box, opos, v, rng);
        p.box = sol.first;
        p.pos = sol.second;
        T.translations++;
        return;
    }
    if (box.reservoir) {
        p.q = 0;
        p.alpha = 0;
        dt = 0.;
        T.absorbed++;
        return;
    }
    V2 rnew = {p.pos.x + dt * v.x, p.pos.y + dt * v.y};
    if (box.inside(rnew)) {
        p.pos = rnew;
        process_segment(S, T, p.box, p.t, p.t + dt, p.sign, v, p.q * nb + p.alpha);
        p.t += dt;
        if (!o.ballistic) {
            double u = canonical(rng);
            std::size_t pos = lower_bound_idx(S.res_of(p.mat), u);
            p.q = pos / nb;
            p.alpha = pos % nb;
        }
        dt = 0.;
        return;
    }
    Hit mru;
    try {
        mru = get_inter_side(box, p.pos, v, dt);
    } catch (const geometry_error&) {
        V2 d = box.center - opos;
        p.pos = p.pos + (1.0e-6 * d) / norm(d);
        T.nudges++;
        return;
    }
    double left_time = dt - mru.time;
    double tf = mru.time;
    if (almost_equal(left_time, 0.)) left_time = 0.;
    dt = left_time;
    rnew = mru.rf;
    V2 reps = rnew + (1.0e-6 * v) / norm(v);
    std::vector<std::size_t> cboxes;
    for (auto& [ibc, bb] : box.contacts) cboxes.push_back(ibc);
    std::vector<std::size_t> pboxes;
    for (auto test : cboxes) {
        if (test == p.box) continue;
        const Border& bc = box.contacts.at(test)[0];
        double npv = dot(bc.np, v);
        bool parallel = almost_equal(npv, 0.);
        bool oriented = npv > 0.;
        if ((S.sys[test].inside(rnew) || S.sys[test].inside(reps)) && !parallel && oriented)
            pboxes.push_back(test);
    }
    if (pboxes.empty()) {
        process_segment(S, T, p.box, p.t, p.t + tf, p.sign, v, p.q * nb + p.alpha);
        p.t += tf;
        // in_corner3, src/geometry_2d.cpp:388-406
        std::vector<std::size_t> ids;
        for (auto& g : S.sys)
            if (g.inside(rnew)) ids.push_back(g.id);
        if (ids.size() > 2) {
            p.box = correct_corner_problem(S, rnew, v, ids, rng);
            V2 corr = S.sys[p.box].center - rnew;
            V2 cpos = rnew + (1.0e-6 * corr) / norm(corr);
            mru = get_inter_side(S.sys[p.box], cpos, v, 1.0e+18);
            rnew = mru.rf;
        }
        const Box& cur = S.sys[p.box];
        std::size_t iborder;
        if (mru.bids.size() > 1) {
            std::vector<std::size_t> voidborders;
            for (int tvb : mru.bids) {
                const Border& mb = cur.borders[std::size_t(tvb)];
                V2 rc = rnew + 1.0e-4 * mb.np;
                bool isvoid = true;
                for (auto cb : cboxes)
                    if (S.sys[cb].inside(rc)) {
                        isvoid = false;
                        break;
                    }
                if (isvoid) voidborders.push_back(std::size_t(tvb));
            }
            if (voidborders.empty()) throw geometry_error("Error in void borders");
            // uniform_int_distribution(0, size) has an inclusive upper bound;
            // the reference then reads one past the end.  Counted and clamped.
            int idx = uniform_int(rng, 0, int(voidborders.size()));
            if (std::size_t(idx) == voidborders.size()) {
                T.quirks++;
                idx--;
            }
            iborder = voidborders[std::size_t(idx)];
        } else {
            iborder = std::size_t(mru.bids.at(0));
        }
        V2 u = cur.borders[iborder].np;
        const std::size_t k0 = p.q * nb + p.alpha;
        long long nmm = -1;
        if (o.specularity > 0.) {
            if (canonical(rng) < o.specularity) {
                nmm = mirror_mode(S, u, k0);
                if (nmm >= 0) T.specular++;
            }
        }
        std::size_t nm = nmm >= 0 ? std::size_t(nmm) : bounce(S, u, k0, rng);
        p.pos = rnew;
        p.q = nm / nb;
        p.alpha = nm % nb;
        dt = 0.;
        T.wall_hits++;
        return;
    } else if (pboxes.size() == 1) {
        p.pos = rnew;
        process_segment(S, T, p.box, p.t, p.t + tf, p.sign, v, p.q * nb + p.alpha);
        p.t += tf;
        if (dmm && S.sys[pboxes[0]].mat != S.sys[p.box].mat) {
            dmm_cross(S, *dmm, p, pboxes[0], dt, rng, T);
            return;
        }
        p.box = pboxes[0];
        T.crossings++;
        return;
    } else {
        process_segment(S, T, p.box, p.t, p.t + tf, p.sign, v, p.q * nb + p.alpha);
        p.t += tf;
        p.pos = rnew;
        std::vector<std::size_t> pbox2;
        V2 rcheck = rnew + 1.0e-6 * v;
        for (auto PB : pboxes)
            if (S.sys[PB].inside(rcheck)) pbox2.push_back(PB);
        std::size_t newid;
        if (pbox2.empty()) {
            newid = pboxes[std::size_t(uniform_int(rng, 0, int(pboxes.size()) - 1))];
            V2 d = S.sys[newid].center - rnew;
            if (!S.sys[newid].periodic) p.pos = p.pos + (1.0e-6 * d) / norm(d);
        } else {
            newid = pbox2[std::size_t(uniform_int(rng, 0, int(pbox2.size()) - 1))];
        }
        if (dmm && S.sys[newid].mat != S.sys[p.box].mat) {
            dmm_cross(S, *dmm, p, newid, dt, rng, T);
            return;
        }
        p.box = newid;
        T.crossings++;
        return;
    }
}

// One particle of Init_generator (walls), src/RTA_MC2D.cpp:421-511.
inline Particle generate_at(const Sim& S, const WallGen& G, Pcg64& rng);
inline Particle generate(const Sim& S, Pcg64& rng) {
    double selectGenR = canonical(rng);
    (void)selectGenR;  // ExGen = {1, 1} without a gradient: always walls
    double whereGenR = canonical(rng);
    auto it = std::lower_bound(S.gen_cum.begin(), S.gen_cum.end(), whereGenR);
    if (it == S.gen_cum.end()) --it;
    return generate_at(S, S.gens[std::size_t(it - S.gen_cum.begin())], rng);
}

// The rest of one particle of Init_generator from wall generator G: a point
// on its border, its mode.
inline Particle generate_at(const Sim& S, const WallGen& G, Pcg64& rng) {
    const std::size_t nb = S.m.nb;
    V2 ppos;
    for (int tries = 0;; ++tries) {
        if (tries > 1000) throw limit_error("border point rejection loop");
        ppos = G.b.p1 + canonical(rng) * G.b.nd;
        if (on_segment(ppos, G.b.sa, G.b.sb)) break;
    }
    const Box& inj = S.sys[G.box];
    if (!inj.inside(ppos)) {
        V2 d = inj.center - ppos;
        ppos = ppos + (1.0e-6 * d) / norm(d);
        if (!inj.inside(ppos)) throw geometry_error("Generated particle out of insertion box");
    }
    double u = canonical(rng);
    std::size_t pos = lower_bound_idx(G.cdf, u);
    Particle p;
    p.pos = ppos;
    p.q = pos / nb;
    p.alpha = pos % nb;
    p.sign = G.sign;
    p.t = 0.;
    p.box = G.box;
    p.mat = S.sys[G.box].mat;
    return p;
}

// Initial deviation Tinit - Teq of each box (init_particles,
// src/beyondRTA_MC2d.cpp:211-269, with outTref_distribution,
// src/sampling.cpp:271-330): particle pid belongs to the box whose prefix
// range holds it; uniform position by bounding-box rejection
// (geometry_2d::get_random_point, include/geometry_2d.hpp:338-356).
inline Particle generate_initial(const Sim& S, std::size_t pid, Pcg64& rng) {
    auto it = std::upper_bound(S.init_first.begin(), S.init_first.end(), (long long)pid);
    const std::size_t g = std::size_t(it - S.init_first.begin()) - 1;
    const Box& B = S.sys[S.init_box[g]];
    double x0 = B.hull[0].x, x1 = B.hull[0].x, y0 = B.hull[0].y, y1 = B.hull[0].y;
    for (auto& h : B.hull) {
        x0 = std::min(x0, h.x);
        x1 = std::max(x1, h.x);
        y0 = std::min(y0, h.y);
        y1 = std::max(y1, h.y);
    }
    V2 r;
    for (int tries = 0;; ++tries) {
        if (tries > 100000) throw limit_error("random point rejection loop");
        r.x = x0 + canonical(rng) * (x1 - x0);
        r.y = y0 + canonical(rng) * (y1 - y0);
        if (B.inside(r)) break;
    }
    const double u = canonical(rng);
    const std::size_t pos = lower_bound_idx(S.init_cdf[g], u);
    Particle p;
    p.pos = r;
    p.q = pos / S.m.nb;
    p.alpha = pos % S.m.nb;
    p.sign = S.init_sign[g];
    p.t = 0.;
    p.box = S.init_box[g];
    p.mat = S.sys[p.box].mat;
    return p;
}

inline void build_initial(Sim& S, int64_t nparticles, uint64_t seed) {
    const Modes& m = S.m;
    const double vuc = m.V * S.thickness / m.c;
    std::vector<double> pmf, energy;
    for (auto& s : S.sys) {
        if (s.reservoir || s.periodic) continue;
        if (almost_equal(s.Teq, s.Treal)) continue;
        if (s.Treal <= 0 || s.Teq <= 0) throw value_error("Invalid temperature value");
        const double cumulsum = out_tref_pmf(m, s.Treal, s.Teq, pmf);
        const double vol = s.area * S.thickness / vuc;
        S.init_box.push_back(s.id);
        S.init_sign.push_back((s.Treal - s.Teq) >= 0 ? 1 : -1);
        S.init_cdf.push_back(fill_cumulative(pmf));
        energy.push_back(dist_energy(vol, cumulsum, double(m.nq)));
    }
    if (S.init_box.empty()) throw input_error("no box with Tinit different from Teq");
    double total = 0;
    for (double e : energy) total += e;
    S.energy = total;
    S.Eeff = total / double(nparticles);
    long long first = 0;
    for (std::size_t b = 0; b < S.init_box.size(); ++b) {
        S.init_first.push_back(first);
        const double gen = energy[b] / S.Eeff;
        long long np = (long long)gen;
        const double rem = gen - std::floor(gen);
        Pcg64 r(seed, (uint64_t(1) << 63) + uint64_t(S.init_box[b]));
        if (canonical(r) <= rem) np++;
        first += np;
    }
    S.init_first.push_back(first);
}

inline void run_particle(const Sim& S, std::size_t pid, uint64_t seed, double maxtime,
                         Tally& T, const Opts& o) {
    Pcg64 rng(seed, pid);
    Particle p = S.init_first.empty() ? generate(S, rng) : generate_initial(S, pid, rng);
    const std::size_t nb = S.m.nb;
    double time = 0.;
    long long nev = 0;
    while (time < maxtime) {
        if (++nev > (1ll << 26)) throw limit_error("free flights per particle cap");
        std::size_t k = p.q * nb + p.alpha;
        V2 v = get_v(S.m, k);
        double dt_ = random_dt(S.w_of(p.mat)[k], rng, o.log_impl);
        T.events++;
        if (time + dt_ > maxtime) dt_ = maxtime - time + 1.0e-8;
        int guard = 0;
        while (!almost_equal(dt_, 0.)) {
            if (++guard > 1000000) throw limit_error("flight step cap");
            evolparticle(S, p, v, dt_, rng, T, o);
        }
        if (p.q == 0 && p.alpha == 0) break;
        time = p.t;
    }
}


// ============================================================ several materials
// Geometries whose boxes hold different crystals (one mode table per
// material, box b in material gm->material[b]), joined by diffuse mismatch
// interfaces.  Each material keeps its own Sim (modes, Lambert rows,
// post-scattering CDF, wall generators) over the shared boxes; a particle
// uses the Sim of its box's material, and its mode indexes that material's
// table.
struct MultiSim {
    std::vector<Sim> mats;
    DmmSet dmm;
    std::vector<std::pair<int, std::size_t>> gref;  // wall generators: (material, index)
    std::vector<double> gcum;
    double energy = 0, Eeff = 0;
    // initial deviation: the boxes in ascending order, their material's CDF
    std::vector<std::size_t> init_box;
    std::vector<int> init_sign;
    std::vector<std::vector<double>> init_cdf;
    std::vector<long long> init_first;
};

// The interface tables of every contact from a box that is neither a
// reservoir nor periodic to a box of another material (a reservoir or a
// periodic box included), each built at the Teq of the first box (in box
// order) that meets it; the reference builds each on first use, at the Teq
// of the box the first particle comes from.
inline void build_interfaces(MultiSim& M, double scalebroad = 0.1) {
    const Sim& S0 = M.mats[0];
    for (auto& a : S0.sys) {
        if (a.reservoir || a.periodic) continue;
        for (auto& [c, bv] : a.contacts) {
            const Box& b = S0.sys[c];
            if (b.mat == a.mat) continue;
            V2 nw = {0., 0.};
            nw.x += bv[0].np.x;
            nw.y += bv[0].np.y;
            const auto key = std::make_tuple(a.mat, b.mat, nw.x, nw.y);
            if (M.dmm.tab.count(key)) continue;
            const Modes& A = M.mats[std::size_t(a.mat)].m;
            const Modes& B = M.mats[std::size_t(b.mat)].m;
            const double VA = A.V * M.mats[std::size_t(a.mat)].thickness / A.c;
            const double VB = B.V * M.mats[std::size_t(b.mat)].thickness / B.c;
            M.dmm.tab.emplace(key, build_dmm(A, B, VA, VB, nw, scalebroad, a.Teq));
        }
    }
}

inline Particle generate_multi(const MultiSim& M, Pcg64& rng) {
    double selectGenR = canonical(rng);
    (void)selectGenR;
    double whereGenR = canonical(rng);
    auto it = std::lower_bound(M.gcum.begin(), M.gcum.end(), whereGenR);
    if (it == M.gcum.end()) --it;
    const auto& gr = M.gref[std::size_t(it - M.gcum.begin())];
    const Sim& S = M.mats[std::size_t(gr.first)];
    Particle p = generate_at(S, S.gens[gr.second], rng);
    p.mat = 0;  // rates and resampling come from the material's own Sim
    return p;
}

inline Particle generate_initial_multi(const MultiSim& M, std::size_t pid, Pcg64& rng) {
    auto it = std::upper_bound(M.init_first.begin(), M.init_first.end(), (long long)pid);
    const std::size_t g = std::size_t(it - M.init_first.begin()) - 1;
    const Sim& S = M.mats[std::size_t(M.mats[0].sys[M.init_box[g]].mat)];
    const Box& B = S.sys[M.init_box[g]];
    double x0 = B.hull[0].x, x1 = B.hull[0].x, y0 = B.hull[0].y, y1 = B.hull[0].y;
    for (auto& h : B.hull) {
        x0 = std::min(x0, h.x);
        x1 = std::max(x1, h.x);
        y0 = std::min(y0, h.y);
        y1 = std::max(y1, h.y);
    }
    V2 r;
    for (int tries = 0;; ++tries) {
        if (tries > 100000) throw limit_error("random point rejection loop");
        r.x = x0 + canonical(rng) * (x1 - x0);
        r.y = y0 + canonical(rng) * (y1 - y0);
        if (B.inside(r)) break;
    }
    const std::size_t pos = lower_bound_idx(M.init_cdf[g], canonical(rng));
    Particle p;
    p.pos = r;
    p.q = pos / S.m.nb;
    p.alpha = pos % S.m.nb;
    p.sign = M.init_sign[g];
    p.t = 0.;
    p.box = M.init_box[g];
    p.mat = 0;
    return p;
}

inline void build_initial_multi(MultiSim& M, int64_t nparticles, uint64_t seed) {
    std::vector<double> pmf, energy;
    for (auto& s : M.mats[0].sys) {
        if (s.reservoir || s.periodic) continue;
        if (almost_equal(s.Teq, s.Treal)) continue;
        if (s.Treal <= 0 || s.Teq <= 0) throw value_error("Invalid temperature value");
        const Sim& S = M.mats[std::size_t(s.mat)];
        const double vuc = S.m.V * S.thickness / S.m.c;
        const double cumulsum = out_tref_pmf(S.m, s.Treal, s.Teq, pmf);
        M.init_box.push_back(s.id);
        M.init_sign.push_back((s.Treal - s.Teq) >= 0 ? 1 : -1);
        M.init_cdf.push_back(fill_cumulative(pmf));
        energy.push_back(dist_energy(s.area * S.thickness / vuc, cumulsum, double(S.m.nq)));
    }
    if (M.init_box.empty()) throw input_error("no box with Tinit different from Teq");
    double total = 0;
    for (double e : energy) total += e;
    M.energy = total;
    M.Eeff = total / double(nparticles);
    long long first = 0;
    for (std::size_t b = 0; b < M.init_box.size(); ++b) {
        M.init_first.push_back(first);
        const double gen = energy[b] / M.Eeff;
        long long np = (long long)gen;
        Pcg64 r(seed, (uint64_t(1) << 63) + uint64_t(M.init_box[b]));
        if (canonical(r) <= gen - std::floor(gen)) np++;
        first += np;
    }
    M.init_first.push_back(first);
}

inline void run_particle_multi(const MultiSim& M, std::size_t pid, uint64_t seed, double maxtime, Tally& T,
                               const Opts& o) {
    Pcg64 rng(seed, pid);
    Particle p = M.init_first.empty() ? generate_multi(M, rng) : generate_initial_multi(M, pid, rng);
    double time = 0.;
    long long nev = 0;
    while (time < maxtime) {
        if (++nev > (1ll << 26)) throw limit_error("free flights per particle cap");
        const Sim& S = M.mats[std::size_t(M.mats[0].sys[p.box].mat)];
        const std::size_t k = p.q * std::size_t(S.m.nb) + p.alpha;
        V2 v = get_v(S.m, k);
        double dt_ = random_dt(S.m.w[k], rng, o.log_impl);
        T.events++;
        if (time + dt_ > maxtime) dt_ = maxtime - time + 1.0e-8;
        int guard = 0;
        while (!almost_equal(dt_, 0.)) {
            if (++guard > 1000000) throw limit_error("flight step cap");
            // a crossing into another material ends the flight, so the Sim
            // stays the particle's material's for the whole loop
            evolparticle(S, p, v, dt_, rng, T, o, &M.dmm);
        }
        if (p.q == 0 && p.alpha == 0) break;
        time = p.t;
    }
}

// ============================================================ steady state
// The periodic / gradient branch of RTAMC2D (src/RTA_MC2D.cpp:2544-2842):
// generations of one free flight per particle.
//
// Draws: slot s of generation g owns pcg64(seed, stream = g * 2^40 + s); the
// reference's thread-local generators and its serial `rng` (used for the
// births) are replaced by these per-slot streams.  Generation 0 is
// Init_generator with a gradient (:443-529); later generations are the
// particles reflected at void walls in the previous one, in slot order, then
// |phi(box)| births per box in ascending box order (:2640-2658).

inline uint64_t steady_stream(uint64_t gen, uint64_t slot) { return (gen << 40) | slot; }

// Nabla_T_distribution, src/sampling.cpp:118-187, per interior box.
struct GradGen {
    std::size_t box;
    int mat = 0;      // the material whose modes cdf runs over
    std::vector<double> cdf;
    std::vector<int> sign;
    double energy;    // get_energy(vol) = vol cumulsum / nq
    double vol;       // box volume in unit cells
    double cumulsum;
};

inline std::vector<GradGen> build_gradient(const Sim& S, double gx, double gy, int only_mat = -1) {
    const Modes& m = S.m;
    const double vuc = m.V * S.thickness / m.c;
    std::vector<GradGen> out;
    for (auto& s : S.sys) {
        if (s.reservoir || s.periodic) continue;
        if (only_mat >= 0 && s.mat != only_mat) continue;  // another material's box
        GradGen G;
        G.box = s.id;
        G.mat = only_mat >= 0 ? only_mat : 0;
        std::vector<double> pmf;
        double cumulsum = nabla_t_pmf(m, gx, gy, s.Teq, pmf, G.sign);
        double vol = s.area * S.thickness / vuc;
        G.energy = dist_energy(vol, cumulsum, double(m.nq));
        G.vol = vol;
        G.cumulsum = cumulsum;
        G.cdf = fill_cumulative(pmf);
        out.push_back(std::move(G));
    }
    return out;
}

// Nabla_T sources with one gradient per box (source_term_gradient,
// src/beyondRTA_MC2d.cpp:626-647): a box whose gradient is zero
// (almost_equal on its norm) has none.
inline std::vector<GradGen> build_gradient_boxes(const Sim& S, const std::vector<V2>& grad) {
    const Modes& m = S.m;
    const double vuc = m.V * S.thickness / m.c;
    std::vector<GradGen> out;
    for (auto& s : S.sys) {
        if (s.reservoir || s.periodic) continue;
        const V2 g = grad[s.id];
        if (almost_equal(std::sqrt(g.x * g.x + g.y * g.y), 0.)) continue;
        GradGen G;
        G.box = s.id;
        std::vector<double> pmf;
        double cumulsum = nabla_t_pmf(m, g.x, g.y, s.Teq, pmf, G.sign);
        double vol = s.area * S.thickness / vuc;
        G.energy = dist_energy(vol, cumulsum, double(m.nq));
        G.vol = vol;
        G.cumulsum = cumulsum;
        G.cdf = fill_cumulative(pmf);
        out.push_back(std::move(G));
    }
    return out;
}

// calculate_gradientT, src/geometry_2d.cpp:524-575: for each box that is
// neither a reservoir nor periodic, the rows h_i = c_i - c_0 and
// d_i = Teq_i - Teq_0 over its contacts of that kind, and the
// minimum-norm least-squares solution of h g = d, which the reference gets
// from Eigen's CompleteOrthogonalDecomposition: Householder QR with column
// pivoting, the rank from |R_ii| > min(rows, 2) eps |R_11|, and, for rank 1,
// the minimum-norm solution along R's first row.
inline V2 cod_solve(std::vector<std::array<double, 2>> h, std::vector<double> d) {
    const std::size_t m = h.size();
    if (m == 0) return V2{0., 0.};
    double nrm[2] = {0., 0.};
    for (auto& r : h) {
        nrm[0] += r[0] * r[0];
        nrm[1] += r[1] * r[1];
    }
    const int p0 = nrm[1] > nrm[0] ? 1 : 0, p1 = 1 - p0;
    // Householder reflection of column p0 onto e1, applied to both columns and d
    auto reflect = [&](std::size_t k, int col) -> double {
        double sig = 0.;
        for (std::size_t i = k; i < m; ++i) sig += h[i][col] * h[i][col];
        const double alpha = -std::copysign(std::sqrt(sig), h[k][col]);
        if (sig == 0.) return 0.;
        std::vector<double> v(m, 0.);
        for (std::size_t i = k; i < m; ++i) v[i] = h[i][col];
        v[k] -= alpha;
        double vv = 0.;
        for (std::size_t i = k; i < m; ++i) vv += v[i] * v[i];
        if (vv == 0.) return alpha;
        for (int c = 0; c < 2; ++c) {
            double t = 0.;
            for (std::size_t i = k; i < m; ++i) t += v[i] * h[i][c];
            t = 2. * t / vv;
            for (std::size_t i = k; i < m; ++i) h[i][c] -= t * v[i];
        }
        double t = 0.;
        for (std::size_t i = k; i < m; ++i) t += v[i] * d[i];
        t = 2. * t / vv;
        for (std::size_t i = k; i < m; ++i) d[i] -= t * v[i];
        return alpha;
    };
    const double r11 = reflect(0, p0);
    if (r11 == 0.) return V2{0., 0.};
    const double r12 = h[0][p1];
    double r22 = 0.;
    if (m >= 2) r22 = reflect(1, p1);
    const double thr = double(std::min<std::size_t>(m, 2)) * std::numeric_limits<double>::epsilon() * std::fabs(r11);
    double x[2];
    if (m >= 2 && std::fabs(r22) > thr) {
        x[p1] = d[1] / r22;
        x[p0] = (d[0] - r12 * x[p1]) / r11;
    } else {
        // rank 1: the solutions of r11 x0 + r12 x1 = d0; the one of least norm
        const double t = d[0] / (r11 * r11 + r12 * r12);
        x[p0] = r11 * t;
        x[p1] = r12 * t;
    }
    return V2{x[0], x[1]};
}

inline std::vector<V2> calculate_gradientT(const Sim& S) {
    std::vector<V2> out(S.sys.size(), V2{0., 0.});
    for (auto& s : S.sys) {
        if (s.reservoir || s.periodic) continue;
        std::vector<std::array<double, 2>> h;
        std::vector<double> d;
        for (auto& [c, b] : s.contacts) {
            const Box& o = S.sys[c];
            if (o.reservoir || o.periodic) continue;
            h.push_back({o.center.x - s.center.x, o.center.y - s.center.y});
            d.push_back(o.Teq - s.Teq);
        }
        out[s.id] = cod_solve(h, d);
    }
    return out;
}

// The sources of generation 0: wall generators (material, index into that
// material's gens) with their cumulative weights, and gradient generators.
struct SteadyGen {
    std::vector<std::pair<int, std::size_t>> wall;
    std::vector<double> wall_cum;
    std::vector<GradGen> grad;
    std::vector<double> grad_cum;
    double exg0 = 0, exg1 = 0;
};

// process_segment (periodic), src/RTA_MC2D.cpp:784-834.
// The three contributions of one periodic segment (gz, gz_jx, gz_jy),
// src/RTA_MC2D.cpp:798-801.
inline void steady_terms(int sign, double dt, V2 vg, double out[3]) {
    double contr = double(sign);
    out[0] = contr * dt;
    out[1] = vg.x * contr * dt;
    out[2] = vg.y * contr * dt;
}

inline void process_segment_steady(Tally& T, std::size_t ibox, int sign, double dt, V2 vg,
                                   std::size_t mode) {
    double contr = double(sign);
    double c[3];
    steady_terms(sign, dt, vg, c);
    T.ex[3 * ibox + 0] += quant(c[0]);
    T.ex[3 * ibox + 1] += quant(c[1]);
    T.ex[3 * ibox + 2] += quant(c[2]);
    // spectral location: the mode's time and, for fd_qmesh (contr / omega
    // once per segment, :829), its signed segment count
    const int lc = T.loc ? (*T.loc)[ibox] : -1;
    if (lc >= 0) {
        T.spec[std::size_t(lc) * T.nmodes + mode] += quant(contr * dt);
        T.scnt[std::size_t(lc) * T.nmodes + mode] += sign;
    }
}

enum Fate { F_LOST = 0, F_SCATTER = 1, F_BOUNCE = 2, F_ABSORBED = 3 };

// evolparticle (periodic), src/RTA_MC2D.cpp:1406-1799, in the material of
// the particle's box (S); with `dmm`, a crossing into a box of another
// material is change_material_diffuse (:1672-1689, :1751-1779): re-emitted
// at the interface and carried into the next generation, as a void-wall
// reflection is.
inline void evolparticle_steady(const Sim& S, Particle& p, V2 v, double& dt, Pcg64& rng, Tally& T,
                                Fate& fate, double specularity = 0., const DmmSet* dmm = nullptr) {
    const std::size_t nb = S.m.nb;
    V2 opos = p.pos;
    const Box& box = S.sys[p.box];
    if (box.periodic) {
        auto sol = translate(S, p.box, opos, v, rng);
        p.box = sol.first;
        p.pos = sol.second;
        T.translations++;
        return;
    }
    if (box.reservoir) {
        p.q = 0;
        p.alpha = 0;
        dt = 0.;
        T.absorbed++;
        fate = F_ABSORBED;
        return;
    }
    V2 rnew = {p.pos.x + dt * v.x, p.pos.y + dt * v.y};
    if (box.inside(rnew)) {
        p.pos = rnew;
        p.t += dt;
        process_segment_steady(T, p.box, p.sign, dt, v, S.mode_off + p.q * nb + p.alpha);  // evalphi: phi += sign
        dt = 0.;
        fate = F_SCATTER;
        return;
    }
    Hit mru;
    try {
        mru = get_inter_side(box, p.pos, v, dt);
    } catch (const geometry_error&) {
        V2 d = box.center - opos;
        p.pos = p.pos + (1.0e-6 * d) / norm(d);
        T.nudges++;
        return;
    }
    double left_time = dt - mru.time;
    double tf = mru.time;
    if (almost_equal(left_time, 0.)) left_time = 0.;
    rnew = mru.rf;
    dt = left_time;
    V2 reps = rnew + (1.0e-6 * v) / norm(v);
    std::vector<std::size_t> cboxes;
    for (auto& [ibc, bb] : box.contacts) cboxes.push_back(ibc);
    std::vector<std::size_t> pboxes;
    for (auto test : cboxes) {
        if (test == p.box) continue;
        const Border& bc = box.contacts.at(test)[0];
        bool parallel = almost_equal(dot(bc.np, v), 0.);
        bool oriented = dot(bc.np, v) > 0.;
        if ((S.sys[test].inside(rnew) || S.sys[test].inside(reps)) && !parallel && oriented)
            pboxes.push_back(test);
    }
    if (pboxes.empty()) {
        process_segment_steady(T, p.box, p.sign, tf, v, S.mode_off + p.q * nb + p.alpha);
        p.t += tf;
        std::vector<std::size_t> ids;
        for (auto& g : S.sys)
            if (g.inside(rnew)) ids.push_back(g.id);
        if (ids.size() > 2) {
            p.box = correct_corner_problem(S, rnew, v, ids, rng);
            V2 corr = S.sys[p.box].center - rnew;
            V2 cpos = rnew + (1.0e-6 * corr) / norm(corr);
            mru = get_inter_side(S.sys[p.box], cpos, v, 1.0e+18);
            rnew = mru.rf;
        }
        const Box& cur = S.sys[p.box];
        std::size_t iborder;
        if (mru.bids.size() > 1) {
            std::vector<std::size_t> voidborders;
            for (int tvb : mru.bids) {
                const Border& mb = cur.borders[std::size_t(tvb)];
                V2 rc = rnew + 1.0e-4 * mb.np;
                bool isvoid = true;
                for (auto cb : cboxes)
                    if (S.sys[cb].inside(rc)) {
                        isvoid = false;
                        break;
                    }
                if (isvoid) voidborders.push_back(std::size_t(tvb));
            }
            if (voidborders.empty()) throw geometry_error("Error in void borders");
            int idx = uniform_int(rng, 0, int(voidborders.size()));
            if (std::size_t(idx) == voidborders.size()) {
                T.quirks++;
                idx--;
            }
            iborder = voidborders[std::size_t(idx)];
        } else {
            iborder = std::size_t(mru.bids.at(0));
        }
        V2 u = cur.borders[iborder].np;
        const std::size_t k0 = p.q * nb + p.alpha;
        long long nmm = -1;
        if (specularity > 0.) {  // this engine's extension, as in the transient flight
            if (canonical(rng) < specularity) {
                nmm = mirror_mode(S, u, k0);
                if (nmm >= 0) T.specular++;
            }
        }
        std::size_t nm = nmm >= 0 ? std::size_t(nmm) : bounce(S, u, k0, rng);
        p.pos = rnew;
        p.q = nm / nb;
        p.alpha = nm % nb;
        dt = 0.;
        T.wall_hits++;
        fate = F_BOUNCE;  // pushed into the next generation
        return;
    } else if (pboxes.size() == 1) {
        p.pos = rnew;
        p.t += tf;
        process_segment_steady(T, p.box, p.sign, tf, v, S.mode_off + p.q * nb + p.alpha);
        if (dmm && S.sys[pboxes[0]].mat != S.sys[p.box].mat) {
            dmm_cross(S, *dmm, p, pboxes[0], dt, rng, T);
            fate = F_BOUNCE;
            return;
        }
        p.box = pboxes[0];
        T.crossings++;
        return;
    } else {
        process_segment_steady(T, p.box, p.sign, tf, v, S.mode_off + p.q * nb + p.alpha);
        p.t += tf;
        p.pos = rnew;
        std::vector<std::size_t> pbox2;
        V2 rcheck = rnew + 1.0e-6 * v;
        for (auto PB : pboxes)
            if (S.sys[PB].inside(rcheck)) pbox2.push_back(PB);
        std::size_t newid;
        if (pbox2.empty()) {
            newid = pboxes[std::size_t(uniform_int(rng, 0, int(pboxes.size()) - 1))];
            V2 d = S.sys[newid].center - rnew;
            if (!S.sys[newid].periodic) p.pos = p.pos + (1.0e-6 * d) / norm(d);
        } else {
            newid = pbox2[std::size_t(uniform_int(rng, 0, int(pbox2.size()) - 1))];
        }
        if (dmm && S.sys[newid].mat != S.sys[p.box].mat) {
            dmm_cross(S, *dmm, p, newid, dt, rng, T);
            fate = F_BOUNCE;
            return;
        }
        p.box = newid;
        T.crossings++;
        return;
    }
}

inline int steady_gen_type(const SteadyGen& SG, double u) {
    int id = u <= SG.exg0 ? 0 : 1;  // lower_bound over ExGen
    if (id == 0 && SG.wall.empty()) id = 1;
    if (id == 1 && SG.grad.empty()) id = 0;
    return id;
}

inline V2 random_point(const Box& B, Pcg64& rng) {
    double x0 = B.hull[0].x, x1 = B.hull[0].x, y0 = B.hull[0].y, y1 = B.hull[0].y;
    for (auto& h : B.hull) {
        x0 = std::min(x0, h.x);
        x1 = std::max(x1, h.x);
        y0 = std::min(y0, h.y);
        y1 = std::max(y1, h.y);
    }
    V2 r;
    for (int tries = 0;; ++tries) {
        if (tries > 100000) throw limit_error("random point rejection loop");
        r.x = x0 + canonical(rng) * (x1 - x0);
        r.y = y0 + canonical(rng) * (y1 - y0);
        if (B.inside(r)) return r;
    }
}

// Generation-0 particle of slot s (Init_generator with a gradient); `rank`
// counts the gradient-generated slots before s (gsign alternates from -).
// mats: one Sim per material; a generator's mode indexes its material's
// table.
inline Particle steady_generate0(const std::vector<Sim>& mats, const SteadyGen& SG, uint64_t rank, Pcg64& rng) {
    double selectGenR = canonical(rng);
    if (steady_gen_type(SG, selectGenR) == 0) {
        // case 0 of Init_generator after the generator-type draw
        double whereGenR = canonical(rng);
        auto it = std::lower_bound(SG.wall_cum.begin(), SG.wall_cum.end(), whereGenR);
        if (it == SG.wall_cum.end()) --it;
        const auto& ref = SG.wall[std::size_t(it - SG.wall_cum.begin())];
        const Sim& S = mats[std::size_t(ref.first)];
        const WallGen& G = S.gens[ref.second];
        V2 ppos;
        for (int tries = 0;; ++tries) {
            if (tries > 1000) throw limit_error("border point rejection loop");
            ppos = G.b.p1 + canonical(rng) * G.b.nd;
            if (on_segment(ppos, G.b.sa, G.b.sb)) break;
        }
        const Box& inj = S.sys[G.box];
        if (!inj.inside(ppos)) {
            V2 d = inj.center - ppos;
            ppos = ppos + (1.0e-6 * d) / norm(d);
            if (!inj.inside(ppos)) throw geometry_error("Generated particle out of insertion box");
        }
        std::size_t pos = lower_bound_idx(G.cdf, canonical(rng));
        Particle p;
        p.pos = ppos;
        p.q = pos / S.m.nb;
        p.alpha = pos % S.m.nb;
        p.sign = G.sign;
        p.box = G.box;
        return p;
    }
    double whereGenR = canonical(rng);
    auto it = std::lower_bound(SG.grad_cum.begin(), SG.grad_cum.end(), whereGenR);
    if (it == SG.grad_cum.end()) --it;
    const GradGen& G = SG.grad[std::size_t(it - SG.grad_cum.begin())];
    const Sim& S = mats[std::size_t(G.mat)];
    V2 ppos = random_point(S.sys[G.box], rng);
    const int want = (rank & 1u) ? 1 : -1;
    std::size_t pos = 0;
    for (int tries = 0;; ++tries) {
        if (tries > 1000000) throw limit_error("gradient sign rejection loop");
        pos = lower_bound_idx(G.cdf, canonical(rng));
        if (G.sign[pos] == want) break;
    }
    Particle p;
    p.pos = ppos;
    p.q = pos / S.m.nb;
    p.alpha = pos % S.m.nb;
    p.sign = want;
    p.box = G.box;
    return p;
}

// ================================================================ beRTAMC2D
// Restatement of the beRTAMC2D step loop (src/beyondRTA_MC2d.cpp:2138-2425):
// ballistic advection with absorbing walls (evolparticle :708-970),
// isothermal-wall injection (Isothermal_walls :446-585), adiabatic diffuse
// re-emission at the spline-interpolated wall temperature
// (adiabatic_diffuse_walls :281-435, CubicSpline1D src/interpolation.cpp),
// propagator scattering with sign branching (Scattering :1073-1210,
// propagator_H src/collision_operator.cpp:857-903), the RTA alternative
// (ScatteringRTA :983-1062), the per-box histogram, cancellation every 4th
// step (:2295-2370) and calculate_prop (:1538-1602).
//
// Draws: the reference's `rng` (generators) is pcg64(seed, 0) and its
// thread-local `rng_` (advection, scattering) is pcg64(seed, 1), consumed in
// the serial order of a one-thread run.  The gradient source term is zero
// here (all interior boxes share Teq), as in the benchmark configurations.

// CubicSpline1D: natural cubic spline (src/interpolation.cpp:20-103).
struct Spline {
    std::vector<double> a, b, c, d, x0, xs;
    void build(const std::vector<double>& X, const std::vector<double>& Y) {
        const int n = int(Y.size()) - 1;
        const std::size_t N = static_cast<std::size_t>(n);
        std::vector<double> A(Y), B(N), D(N), h(N), alpha(N), C(N + 1), l(N + 1), mu(N + 1), z(N + 1);
        for (int i = 0; i < n; i++) h[std::size_t(i)] = X[std::size_t(i) + 1] - X[std::size_t(i)];
        for (int i = 1; i < n; i++)
            alpha[std::size_t(i)] = 3. / h[std::size_t(i)] * (A[std::size_t(i) + 1] - A[std::size_t(i)]) -
                                    3. / h[std::size_t(i) - 1] * (A[std::size_t(i)] - A[std::size_t(i) - 1]);
        l[0] = 1;
        mu[0] = 0;
        z[0] = 0;
        for (int i = 1; i < n; i++) {
            const std::size_t k = std::size_t(i);
            l[k] = 2 * (X[k + 1] - X[k - 1]) - h[k - 1] * mu[k - 1];
            mu[k] = h[k] / l[k];
            z[k] = (alpha[k] - h[k - 1] * z[k - 1]) / l[k];
        }
        l[std::size_t(n)] = 1;
        z[std::size_t(n)] = 0;
        C[std::size_t(n)] = 0;
        for (int j = n - 1; j >= 0; j--) {
            const std::size_t k = std::size_t(j);
            C[k] = z[k] - mu[k] * C[k + 1];
            B[k] = (A[k + 1] - A[k]) / h[k] - h[k] * (C[k + 1] + 2 * C[k]) / 3;
            D[k] = (C[k + 1] - C[k]) / (3 * h[k]);
        }
        a.assign(A.begin(), A.begin() + n);
        b = B;
        c.assign(C.begin(), C.begin() + n);
        d = D;
        x0.assign(X.begin(), X.begin() + n);
        xs.assign(X.begin() + 1, X.end());
    }
    double interp(double x) const {
        std::size_t idx = std::size_t(std::lower_bound(xs.begin(), xs.end(), x) - xs.begin());
        if (idx >= a.size()) idx--;
        const double dx = x - x0[idx];
        return a[idx] + dx * (b[idx] + dx * (c[idx] + d[idx] * dx));
    }
};

struct BeParticle {
    V2 pos;
    std::size_t mode = 0;  // q * nb + alpha; 0 marks a particle to delete
    int sign = 1;
    std::size_t box = 0;
};

struct BeRun {
    Sim S;
    bool rta = false;
    int nm = 0;                       // propagator size (modes minus the 3 Gamma acoustic)
    std::vector<double> cumm;         // signed cumulative per column, column-major
    std::vector<const double*> box_cumm;  // per box: the table it scatters with
    std::vector<std::vector<double>> cumms; // the tables of the boxes' Teq
    std::vector<double> resample_cdf; // RTA resampling at T (BE_derivative_distribution)
    double dt = 0, maxtime = 0, Eeff = 0;
    std::vector<std::vector<int>> Eborder;   // per box, per border
    std::vector<std::vector<Spline>> spl;    // J(T) -> T per box, per border
    std::vector<std::vector<char>> spl_ok;
};

// propagator_H(b): |b| accumulated and signed by the entry, src/collision_operator.cpp:857-870
// Sum of |x| in the order of the reference's b.array().abs().sum()
// (propagator_H, src/collision_operator.cpp:857-870): Eigen's vectorised
// reduction of a 16-byte aligned vector over packets of two doubles, as in
// its redux_impl for LinearVectorizedTraversal: two packet accumulators over
// blocks of four, their lane-wise sum, the last whole packet, then the two
// lanes, then the tail element.
inline double eigen_abs_sum(const double* x, std::size_t n) {
    if (n < 2) return n ? std::fabs(x[0]) : 0.;
    const std::size_t end2 = n / 4 * 4, end = n / 2 * 2;
    double a0 = std::fabs(x[0]), a1 = std::fabs(x[1]);
    if (end > 2) {
        double b0 = std::fabs(x[2]), b1 = std::fabs(x[3]);
        for (std::size_t i = 4; i < end2; i += 4) {
            a0 += std::fabs(x[i]);
            a1 += std::fabs(x[i + 1]);
            b0 += std::fabs(x[i + 2]);
            b1 += std::fabs(x[i + 3]);
        }
        a0 += b0;
        a1 += b1;
        if (end > end2) {
            a0 += std::fabs(x[end2]);
            a1 += std::fabs(x[end2 + 1]);
        }
    }
    double r = a0 + a1;
    for (std::size_t i = end; i < n; ++i) r += std::fabs(x[i]);
    return r;
}

// lirp of two signed CDFs, src/collision_operator.cpp:918-929.
inline double lirp_value(double a, double b, double T1, double T2, double Tx) {
    return a + (Tx - T1) * (b - a) / (T2 - T1);
}

inline void build_cumm(BeRun& R, const double* P) {
    const std::size_t n = std::size_t(R.nm);
    R.cumm.resize(n * n);
    for (std::size_t j = 0; j < n; ++j) {
        const double* col = P + j * n;
        const double abssum = eigen_abs_sum(col, n);
        double acc = 0.;
        for (std::size_t i = 0; i < n; ++i) {
            acc += std::fabs(col[i]);
            R.cumm[j * n + i] = (col[i] < 0.) ? -acc / abssum : acc / abssum;
        }
    }
}

// propagator_H::get: lower_bound on |cumm| (abs_less), sign of the entry,
// index + 3; `tab` is the table (column-major nm x nm signed CDFs).
inline std::pair<int, std::size_t> prop_get_tab(const BeRun& R, const double* tab, std::size_t col, double u) {
    const double* c = tab + col * std::size_t(R.nm);
    const double* it = std::lower_bound(c, c + R.nm, u,
                                        [](double a, double b) { return std::fabs(a) < std::fabs(b); });
    std::size_t im = std::size_t(it - c);
    if (im >= std::size_t(R.nm)) im = std::size_t(R.nm) - 1;
    return {c[im] > 0. ? 1 : -1, im + 3};
}

inline std::pair<int, std::size_t> prop_get(const BeRun& R, std::size_t col, double u) {
    const double* c = &R.cumm[col * std::size_t(R.nm)];
    const double* it = std::lower_bound(c, c + R.nm, u,
                                        [](double a, double b) { return std::fabs(a) < std::fabs(b); });
    std::size_t im = std::size_t(it - c);
    if (im >= std::size_t(R.nm)) im = std::size_t(R.nm) - 1;
    return {c[im] > 0. ? 1 : -1, im + 3};
}

inline void be_kill(BeParticle& p) { p.mode = 0; }

// evolparticle (beyond RTA), src/beyondRTA_MC2d.cpp:708-970, with the
// recursion written as a loop.
inline void be_evolve(BeRun& R, BeParticle& p, V2 v, double dt, Pcg64& rng) {
    const auto& sys = R.S.sys;
    for (int guard = 0;; ++guard) {
        if (guard > 1000000) throw limit_error("advection step cap");
        if (sys[p.box].reservoir) {
            be_kill(p);
            return;
        }
        if (sys[p.box].periodic) {  // Apply PBC and go on with the same time (:728-737)
            auto sol = translate(R.S, p.box, p.pos, v, rng);
            p.box = sol.first;
            p.pos = sol.second;
        }
        const V2 opos = p.pos;
        const Box& box = sys[p.box];
        V2 rnew = {p.pos.x + dt * v.x, p.pos.y + dt * v.y};
        if (box.inside(rnew)) {
            p.pos = rnew;
            return;
        }
        Hit mru;
        try {
            mru = get_inter_side(box, p.pos, v, dt);
        } catch (const geometry_error&) {
            V2 d = box.center - opos;
            p.pos = p.pos + (1.0e-6 * d) / norm(d);
            continue;
        }
        double left_time = dt - mru.time;
        if (almost_equal(left_time, 0.)) left_time = 0.;
        rnew = mru.rf;
        V2 reps = rnew + (1.0e-6 * v) / norm(v);
        std::vector<std::size_t> cboxes, pboxes;
        for (auto& [ibc, bb] : box.contacts) cboxes.push_back(ibc);
        for (auto test : cboxes) {
            if (test == p.box) continue;
            const double npv = dot(box.contacts.at(test)[0].np, v);
            if ((sys[test].inside(rnew) || sys[test].inside(reps)) && !almost_equal(npv, 0.) && npv > 0.)
                pboxes.push_back(test);
        }
        if (pboxes.empty()) {
            std::vector<std::size_t> ids;
            for (auto& g : sys)
                if (g.inside(rnew)) ids.push_back(g.id);
            if (ids.size() > 2) {
                // correct_corner_problem: winner box and its first outgoing border at rnew
                std::vector<std::pair<std::size_t, int>> fin;
                for (auto cnd : ids) {
                    std::vector<int> bids;
                    int k = 0;
                    for (auto& b : sys[cnd].borders) {
                        if (on_segment(rnew, b.la, b.lb) && dot(b.np, v) > 0.) bids.push_back(k);
                        k++;
                    }
                    if (bids.size() <= 1) fin.push_back({cnd, bids.empty() ? -1 : bids[0]});
                }
                if (fin.empty()) throw geometry_error("corner without a candidate box");
                auto w = fin[std::size_t(uniform_int(rng, 0, int(fin.size()) - 1))];
                if (w.second < 0) throw geometry_error("corner box without an outgoing border");
                p.box = w.first;
                p.pos = rnew;
                R.Eborder[w.first][std::size_t(w.second)] += p.sign;
                be_kill(p);
                return;
            }
            std::size_t iborder;
            if (mru.bids.size() > 1) {
                std::vector<std::size_t> voidborders;
                for (int tvb : mru.bids) {
                    const Border& mb = box.borders[std::size_t(tvb)];
                    V2 rc = rnew + 1.0e-4 * mb.np;
                    bool isvoid = true;
                    for (auto cb : cboxes)
                        if (sys[cb].inside(rc)) {
                            isvoid = false;
                            break;
                        }
                    if (isvoid) voidborders.push_back(std::size_t(tvb));
                }
                if (voidborders.empty()) throw geometry_error("Error in void borders");
                iborder = voidborders[std::size_t(uniform_int(rng, 0, int(voidborders.size()) - 1))];
            } else {
                iborder = std::size_t(mru.bids.at(0));
            }
            R.Eborder[p.box][iborder] += p.sign;
            be_kill(p);
            return;
        } else if (pboxes.size() == 1) {
            p.box = pboxes[0];
            p.pos = rnew;
            dt = left_time;
            continue;
        } else {
            std::vector<std::size_t> pbox2;
            double tau = 1.0e-6;
            bool nudged = false;
            while (true) {
                V2 rcheck = rnew + tau * v;
                for (auto PB : pboxes)
                    if (sys[PB].inside(rcheck)) pbox2.push_back(PB);
                if (pbox2.empty()) {
                    tau /= 10.0;
                    if (tau < 1.0e-15) {
                        V2 d = box.center - rnew;
                        p.pos = rnew + (1.0e-6 * d) / norm(d);
                        dt = left_time;
                        nudged = true;
                        break;
                    }
                } else {
                    break;
                }
            }
            if (nudged) continue;
            p.box = pbox2[std::size_t(uniform_int(rng, 0, int(pbox2.size()) - 1))];
            p.pos = rnew;
            dt = left_time;
            continue;
        }
    }
}

// Random point on a border segment (geom2d_border::get_random_point).
inline V2 border_point(const Border& b, Pcg64& rng) {
    for (int tries = 0;; ++tries) {
        if (tries > 1000) throw limit_error("border point rejection loop");
        V2 rp = b.p1 + canonical(rng) * b.nd;
        if (on_segment(rp, b.p1, b.p2)) return rp;
    }
}

// Ntogenerate stochastic rounding (src/sampling.cpp:243-260).
inline std::size_t n_to_generate(double gen, Pcg64& rng) {
    std::size_t np = std::size_t(gen);
    const double rem = gen - std::floor(gen);
    if (canonical(rng) <= rem) np++;
    return np;
}

}  // namespace orc

// ---------------------------------------------------------------- C API
namespace {
thread_local std::string g_err;

int fail(int code, const char* what) {
    g_err = what;
    return code;
}

orc::Modes modes_from(const bte_mode_table* mt) {
    orc::Modes m;
    m.nq = mt->nq;
    m.nb = mt->nb;
    const std::size_t n = std::size_t(mt->nq) * mt->nb;
    m.omega.assign(mt->omega, mt->omega + n);
    m.w.assign(mt->w, mt->w + n);
    m.vx.resize(n);
    m.vy.resize(n);
    m.vz.resize(n);
    for (std::size_t k = 0; k < n; ++k) {
        m.vx[k] = mt->vg[3 * k];
        m.vy[k] = mt->vg[3 * k + 1];
        m.vz[k] = mt->vg[3 * k + 2];
    }
    std::memcpy(m.dq, mt->dq, sizeof(m.dq));
    m.V = mt->V;
    m.c = mt->c_lat;
    for (int i = 0; i < 3; ++i) m.grid[i] = mt->grid[i];
    return m;
}

orc::Sim build_sim(const bte_mode_table* mt, const bte_geometry* gm) {
    orc::Sim S;
    S.m = modes_from(mt);
    S.thickness = gm->thickness;
    std::size_t off = 0;
    for (int i = 0; i < gm->nboxes; ++i) {
        std::vector<orc::V2> verts;
        for (int j = 0; j < gm->npoints[i]; ++j, ++off)
            verts.push_back({gm->vertices[2 * off], gm->vertices[2 * off + 1]});
        orc::Box b = orc::make_box(verts);
        b.Teq = gm->Teq[i];
        b.Treal = gm->Tinit ? gm->Tinit[i] : gm->Teq[i];
        b.reservoir = gm->reservoir[i] != 0;
        b.mat = gm->material ? gm->material[i] : 0;
        if (gm->translate_to && gm->translate_to[i] >= 0) {
            b.periodic = true;
            b.box2translate = std::size_t(gm->translate_to[i]);
            b.translation = {gm->translation[2 * i], gm->translation[2 * i + 1]};
        }
        b.id = std::size_t(i);
        S.sys.push_back(std::move(b));
    }
    orc::calculate_contacts(S.sys);
    return S;
}
}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

// Borders and contacts of every box, for geometry known-answer tests.
// Writes per box: nborders, then (p1x p1y p2x p2y npx npy) per border; then
// ncontacts, then (id npx npy) per contact.  Returns doubles written.
long long oracle_geometry_dump(const bte_mode_table* /*unused*/, const bte_geometry* gm,
                               double* out, long long cap) {
    try {
        bte_mode_table dummy{};
        (void)dummy;
        orc::Sim S;
        std::size_t off = 0;
        for (int i = 0; i < gm->nboxes; ++i) {
            std::vector<orc::V2> verts;
            for (int j = 0; j < gm->npoints[i]; ++j, ++off)
                verts.push_back({gm->vertices[2 * off], gm->vertices[2 * off + 1]});
            orc::Box b = orc::make_box(verts);
            b.id = std::size_t(i);
            b.reservoir = gm->reservoir[i] != 0;
            S.sys.push_back(std::move(b));
        }
        orc::calculate_contacts(S.sys);
        long long k = 0;
        auto put = [&](double x) {
            if (k < cap) out[k] = x;
            k++;
        };
        for (auto& b : S.sys) {
            put(double(b.borders.size()));
            for (auto& br : b.borders) {
                put(br.p1.x); put(br.p1.y); put(br.p2.x); put(br.p2.y);
                put(br.np.x); put(br.np.y);
            }
            put(double(b.contacts.size()));
            for (auto& [id, cv] : b.contacts) {
                put(double(id)); put(cv[0].np.x); put(cv[0].np.y);
            }
            put(b.center.x); put(b.center.y); put(b.area);
        }
        return k;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

// get_inter_side on box `ibox`: writes (time, rx, ry, nbids, bids...).
int oracle_inter_side(const bte_geometry* gm, int ibox, double x, double y, double vx,
                      double vy, double dt, double* out) {
    try {
        std::vector<orc::Box> sys;
        std::size_t off = 0;
        for (int i = 0; i < gm->nboxes; ++i) {
            std::vector<orc::V2> verts;
            for (int j = 0; j < gm->npoints[i]; ++j, ++off)
                verts.push_back({gm->vertices[2 * off], gm->vertices[2 * off + 1]});
            sys.push_back(orc::make_box(verts));
        }
        orc::Hit h = orc::get_inter_side(sys.at(std::size_t(ibox)), {x, y}, {vx, vy}, dt);
        out[0] = h.time;
        out[1] = h.rf.x;
        out[2] = h.rf.y;
        out[3] = double(h.bids.size());
        for (std::size_t i = 0; i < h.bids.size() && i < 8; ++i) out[4 + i] = h.bids[i];
        return 0;
    } catch (const orc::geometry_error& e) {
        g_err = e.what();
        return BTE_ERR_GEOMETRY;
    }
}

// pcg64 outputs and the libstdc++ mappings, for the golden-vector tests.
void oracle_pcg64(uint64_t seed, uint64_t stream, int n, uint64_t* raw, double* canon,
                  int* ints, int int_hi) {
    orc::Pcg64 a(seed, stream), b(seed, stream), c(seed, stream);
    for (int i = 0; i < n; ++i) {
        raw[i] = a();
        canon[i] = orc::canonical(b);
        ints[i] = orc::uniform_int(c, 0, int_hi);
    }
}

// uniform_int_distribution<int>(0, his[i]) for i = 0..n-1, drawn in sequence
// from one pcg64(seed, stream), as one engine shared by successive calls.
void oracle_uniform_int_seq(uint64_t seed, uint64_t stream, const int* his, int n, int* out) {
    orc::Pcg64 g(seed, stream);
    for (int i = 0; i < n; ++i) out[i] = orc::uniform_int(g, 0, his[i]);
}

// The time grid of src/RTA_MC2D.cpp:2118-2124 (Eigen LinSpaced); returns ntime.
int oracle_timegrid(double dt, double maxtime_in, double* out, int cap) {
    std::size_t ntime = std::size_t(std::floor(maxtime_in / dt + 1.0e-6)) + 1;
    double maxtime = double(ntime - 1) * dt;
    double step = (maxtime - 0.0) / double(ntime - 1);
    for (std::size_t i = 0; i < ntime && int(i) < cap; ++i)
        out[i] = (i == ntime - 1) ? maxtime : 0.0 + double(i) * step;
    return int(ntime);
}

void oracle_log(const double* x, double* y, long long n, int impl) {
    for (long long i = 0; i < n; ++i) y[i] = impl == 0 ? orc::bte_log(x[i]) : std::log(x[i]);
}

void oracle_be(const double* omega, long long n, double T, double* be, double* kern) {
    for (long long i = 0; i < n; ++i) {
        be[i] = orc::bose_einstein(omega[i], T);
        kern[i] = orc::bose_einstein_kernel(omega[i], T);
    }
}

// One periodic jump (geometry_2d::translate) of a particle at (x, y) with
// velocity (vx, vy) in periodic box ibox; draws from pcg64(seed, stream).
int oracle_translate(const bte_geometry* gm, int ibox, double x, double y, double vx, double vy,
                     uint64_t seed, uint64_t stream, int* nbox, double* xy) {
    try {
        bte_mode_table mt{};
        orc::Sim S;
        S.thickness = gm->thickness;
        std::size_t off = 0;
        for (int i = 0; i < gm->nboxes; ++i) {
            std::vector<orc::V2> verts;
            for (int j = 0; j < gm->npoints[i]; ++j, ++off)
                verts.push_back({gm->vertices[2 * off], gm->vertices[2 * off + 1]});
            orc::Box b = orc::make_box(verts);
            b.reservoir = gm->reservoir[i] != 0;
            if (gm->translate_to && gm->translate_to[i] >= 0) {
                b.periodic = true;
                b.box2translate = std::size_t(gm->translate_to[i]);
                b.translation = {gm->translation[2 * i], gm->translation[2 * i + 1]};
            }
            b.id = std::size_t(i);
            S.sys.push_back(std::move(b));
        }
        orc::calculate_contacts(S.sys);
        (void)mt;
        orc::Pcg64 rng(seed, stream);
        auto sol = orc::translate(S, std::size_t(ibox), {x, y}, {vx, vy}, rng);
        *nbox = int(sol.first);
        xy[0] = sol.second.x;
        xy[1] = sol.second.y;
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// Lambert table row sizes (for the table-equality tests): nnz per mode.
int oracle_lambert_nnz(const bte_mode_table* mt, const bte_geometry* gm, long long* nnz) {
    try {
        orc::Sim S = build_sim(mt, gm);
        orc::build_lambert(S);
        for (std::size_t k = 0; k < S.lambert.size(); ++k) nnz[k] = (long long)S.lambert[k].size();
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_INPUT, e.what());
    }
}

// One RTA run (walls source) over particles [begin, end) on `nthreads` host
// threads (1 gives the reference's per-particle order of summation).
// counters: events, wall_hits, crossings, absorbed, nudges, quirks.
int oracle_rta_run_mat(const bte_mode_table* mt, const bte_geometry* gm, int nmat, const double* mw,
                       const double* mT0, const double* share, const bte_rta_params* rp, int nthreads,
                       int log_impl, bte_rta_result* out, int64_t* counters);

namespace {
std::vector<int> g_spec_boxes;      // spectral locations of the following runs
std::vector<__int128> g_spec_last;  // the last run's per-mode tally
std::vector<int64_t> g_spec_cnt;     // the last steady run's signed segment counts
}  // namespace

// Known-answer hooks into single pieces of the restatement.
// process_segment's split of [t0, t1] over the time grid: the signed time
// each bin receives, added to bins[ntime - 1].
void oracle_kat_segment(const double* grid, int ntime, double t0, double t1, int sign, double* bins) {
    orc::Sim S;
    S.timegrid.assign(grid, grid + ntime);
    orc::Tally T;
    T.init(1, std::size_t(ntime - 1));
    orc::process_segment(S, T, 0, t0, t1, sign, orc::V2{0., 0.});
    for (int i = 0; i + 1 < ntime; ++i) bins[i] += T.gz[std::size_t(i)];
}

// Grid_distribution::sample: index drawn by u from the pmf's CDF; -1 when
// fill_cumulative rejects the pmf (a negative weight).
long long oracle_kat_cdf_sample(const double* pmf, int n, double u) {
    try {
        const std::vector<double> p(pmf, pmf + n);
        return (long long)orc::lower_bound_idx(orc::fill_cumulative(p), u);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

// propagator_H::get on column `col` of the column-major n x n P: the
// outgoing mode (row + 3) and its sign.
int oracle_kat_propagator(const double* P, int n, int col, double u, int* sign) {
    orc::BeRun R;
    R.nm = n;
    orc::build_cumm(R, P);
    const auto r = orc::prop_get(R, std::size_t(col), u);
    *sign = r.first;
    return int(r.second);
}

// ---- Hooks compared with the reference's own code (tests/golden/
// ref_pins.json, built by oracle/build_ref.py from the cited functions).
// Each calls the helper the runs above use.
int oracle_kat_almost_equal(double a, double b) { return orc::almost_equal(a, b) ? 1 : 0; }

// get_bin_index, src/RTA_MC2D.cpp:140-148.
long long oracle_kat_bin_index(const double* grid, int n, double t) {
    const std::vector<double> g(grid, grid + n);
    return (long long)orc::bin_index(g, t);
}

// process_segment (transient), src/RTA_MC2D.cpp:699-769: the three tallies
// of one segment with velocity (vx, vy), per bin.
void oracle_kat_segment3(const double* grid, int ntime, double t0, double t1, int sign, double vx, double vy,
                         double* gz, double* jx, double* jy) {
    orc::Sim S;
    S.timegrid.assign(grid, grid + ntime);
    orc::Tally T;
    T.init(1, std::size_t(ntime - 1));
    orc::process_segment(S, T, 0, t0, t1, sign, orc::V2{vx, vy});
    for (int i = 0; i + 1 < ntime; ++i) {
        gz[i] = T.gz[std::size_t(i)];
        jx[i] = T.jx[std::size_t(i)];
        jy[i] = T.jy[std::size_t(i)];
    }
}

// process_segment (periodic), src/RTA_MC2D.cpp:784-834: the contributions.
void oracle_kat_steady_terms(int sign, double dt, double vx, double vy, double* out) {
    orc::steady_terms(sign, dt, orc::V2{vx, vy}, out);
}

// get_v, src/RTA_MC2D.cpp:843-856, for every mode.
void oracle_kat_get_v(const bte_mode_table* mt, double* vx, double* vy) {
    const orc::Modes m = modes_from(mt);
    for (std::size_t k = 0; k < m.n(); ++k) {
        const orc::V2 v = orc::get_v(m, k);
        vx[k] = v.x;
        vy[k] = v.y;
    }
}

// random_dt, include/sampling.hpp:40-46: K draws from pcg64(seed, stream)
// with rates w[i % nw].
int oracle_kat_random_dt(uint64_t seed, uint64_t stream, const double* w, int nw, int K, int log_impl,
                         double* out) {
    try {
        orc::Pcg64 rng(seed, stream);
        for (int i = 0; i < K; ++i) out[i] = orc::random_dt(w[i % nw], rng, log_impl);
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_VALUE, e.what());
    }
}

// The distributions of src/sampling.cpp over the mode table: kind 0
// BE_derivative (a = {T}), 1 Isothermal_wall (a = {Tw, Teq, nx, ny, vuc}),
// 2 outTref (a = {Tinit, Tref, vol}), 3 Nabla_T (a = {gx, gy, T, vol}).
// Writes the cumulative distribution, the signs and scal = {cumulsum,
// flux (1) or energy (2, 3)}.
int oracle_kat_distribution(const bte_mode_table* mt, int kind, const double* a, double* cum, int* sign,
                            double* scal) {
    try {
        const orc::Modes m = modes_from(mt);
        const double nq = double(m.nq);
        std::vector<double> pmf;
        std::vector<int> sg(m.n(), 1);
        double cs = 0., extra = 0.;
        if (kind == 0) {
            pmf = orc::be_derivative_pmf(m, m.w, a[0]);
        } else if (kind == 1) {
            cs = orc::wall_pmf(m, orc::V2{a[2], a[3]}, a[0], a[1], pmf);
            const int s = (a[0] - a[1]) >= 0 ? 1 : -1;
            sg.assign(m.n(), s);
            extra = orc::wall_flux(s, cs, nq, a[4]);
        } else if (kind == 2) {
            cs = orc::out_tref_pmf(m, a[0], a[1], pmf);
            sg.assign(m.n(), (a[0] - a[1]) >= 0 ? 1 : -1);
            extra = orc::dist_energy(a[2], cs, nq);
        } else if (kind == 3) {
            cs = orc::nabla_t_pmf(m, a[0], a[1], a[2], pmf, sg);
            extra = orc::dist_energy(a[3], cs, nq);
        } else {
            return fail(BTE_ERR_INPUT, "unknown distribution");
        }
        const std::vector<double> c = orc::fill_cumulative(pmf);
        for (std::size_t k = 0; k < m.n(); ++k) {
            cum[k] = c[k];
            sign[k] = sg[k];
        }
        scal[0] = cs;
        scal[1] = extra;
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_VALUE, e.what());
    }
}

// Ntogenerate with stochastic rounding from one pcg64(seed, stream):
// K calls, kind 1 (wall) and 3 (Nabla_T) with args[i] = {time, spf or vol,
// Eff}, kind 2 (outTref) with args[i] = {vol, Eff, unused}.
void oracle_kat_ntogen(int kind, const double* args, int K, double cumulsum, double nq, uint64_t seed,
                       uint64_t stream, long long* out) {
    orc::Pcg64 rng(seed, stream);
    for (int i = 0; i < K; ++i) {
        const double* q = args + 3 * i;
        const double gen = kind == 2 ? orc::gen_plain(q[0], cumulsum, q[1], nq)
                                     : orc::gen_scaled(q[0], q[1], cumulsum, q[2], nq);
        out[i] = (long long)orc::n_to_generate(gen, rng);
    }
}

// K draws of the BE_derivative distribution at T (Grid_distribution::sample).
void oracle_kat_be_samples(const bte_mode_table* mt, double T, uint64_t seed, uint64_t stream, int K,
                           long long* out) {
    const orc::Modes m = modes_from(mt);
    const std::vector<double> c = orc::fill_cumulative(orc::be_derivative_pmf(m, m.w, T));
    orc::Pcg64 rng(seed, stream);
    for (int i = 0; i < K; ++i) out[i] = (long long)orc::lower_bound_idx(c, orc::canonical(rng));
}

// The Lambert table of diffusive_bouncing (src/RTA_MC2D.cpp:556-626) in
// CSR form: row k holds idx[rowptr[k] .. rowptr[k+1]) with their values.
// Returns the number of entries (written only when it fits `cap`).
long long oracle_kat_lambert(const bte_mode_table* mt, long long* rowptr, long long* idx, double* val,
                             long long cap) {
    orc::Sim S;
    S.m = modes_from(mt);
    orc::build_lambert(S);
    long long nnz = 0;
    for (auto& r : S.lambert) nnz += (long long)r.size();
    if (nnz > cap) return nnz;
    long long o = 0;
    for (std::size_t k = 0; k < S.lambert.size(); ++k) {
        rowptr[k] = o;
        for (auto& [f, v] : S.lambert[k]) {
            idx[o] = (long long)f;
            val[o] = v;
            ++o;
        }
    }
    rowptr[S.lambert.size()] = o;
    return nnz;
}

// K bounces (diffusive_bouncing::bounce, :635-678) of mode imode at a wall
// of outward normal (npx, npy), one pcg64(seed, stream) for all of them.
int oracle_kat_bounce(const bte_mode_table* mt, double npx, double npy, int imode, uint64_t seed,
                      uint64_t stream, int K, long long* out) {
    try {
        orc::Sim S;
        S.m = modes_from(mt);
        orc::build_lambert(S);
        orc::Pcg64 rng(seed, stream);
        for (int i = 0; i < K; ++i) out[i] = (long long)orc::bounce(S, orc::V2{npx, npy}, std::size_t(imode), rng);
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// propagator_H(b) (src/collision_operator.cpp:857-870): the signed
// cumulative distribution of column `col` of the column-major n x n P.
void oracle_kat_prop_cumm(const double* P, int n, int col, double* out) {
    orc::BeRun R;
    R.nm = n;
    orc::build_cumm(R, P);
    for (int i = 0; i < n; ++i) out[i] = R.cumm[std::size_t(col) * std::size_t(n) + std::size_t(i)];
}

// lirp (src/collision_operator.cpp:918-929) of column `col` of P1 (at T1)
// and P2 (at T2), at Tx.
void oracle_kat_lirp(const double* P1, const double* P2, int n, int col, double T1, double T2, double Tx,
                     double* out) {
    orc::BeRun A, B;
    A.nm = B.nm = n;
    orc::build_cumm(A, P1);
    orc::build_cumm(B, P2);
    const std::size_t o = std::size_t(col) * std::size_t(n);
    for (int i = 0; i < n; ++i)
        out[i] = orc::lirp_value(A.cumm[o + std::size_t(i)], B.cumm[o + std::size_t(i)], T1, T2, Tx);
}

// calculate_gradientT (src/geometry_2d.cpp:524-575) of the geometry's
// boxes: out[2 * box + {0, 1}], K/nm.
int oracle_kat_gradientT(const bte_mode_table* mt, const bte_geometry* gm, double* out) {
    try {
        const orc::Sim S = build_sim(mt, gm);
        const auto g = orc::calculate_gradientT(S);
        for (std::size_t i = 0; i < g.size(); ++i) {
            out[2 * i] = g[i].x;
            out[2 * i + 1] = g[i].y;
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// Spectral locations for the following oracle_rta_run calls (nloc = 0: off).
void oracle_set_spectral(int nloc, const int* boxes) {
    g_spec_boxes.assign(boxes, boxes + (nloc > 0 ? nloc : 0));
}

// The last run's per-mode time at the locations, [loc][bin][mode] as
// 128-bit fixed-point (hi, lo) pairs; returns the number of values.
long long oracle_spectral_raw(int64_t* out, long long cap) {
    const long long n = (long long)g_spec_last.size();
    if (out && cap >= n)
        for (long long i = 0; i < n; ++i) {
            unsigned __int128 u = (unsigned __int128)g_spec_last[std::size_t(i)];
            out[2 * i] = int64_t(uint64_t(u >> 64));
            out[2 * i + 1] = int64_t(uint64_t(u));
        }
    return n;
}

// The last steady run's signed segment counts per [loc][mode].
long long oracle_spectral_counts(int64_t* out, long long cap) {
    const long long n = (long long)g_spec_cnt.size();
    if (out && cap >= n)
        for (long long i = 0; i < n; ++i) out[i] = g_spec_cnt[std::size_t(i)];
    return n;
}

int oracle_rta_run(const bte_mode_table* mt, const bte_geometry* gm, const bte_rta_params* rp,
                   int nthreads, int log_impl, bte_rta_result* out, int64_t* counters) {
    return oracle_rta_run_mat(mt, gm, 0, nullptr, nullptr, nullptr, rp, nthreads, log_impl, out, counters);
}

// The same with nmat materials: rates mw[m][mode] at reference temperature
// mT0[m]; box b uses material gm->material[b] (rates, post-scattering
// distribution, temperature conversion).  With share[m] (walls source) the
// wall of material m is drawn with probability share[m] E_w / E_m and the
// particles of material m carry Eeff_m = E_m / (share[m] N).
int oracle_rta_run_mat(const bte_mode_table* mt, const bte_geometry* gm, int nmat, const double* mw,
                       const double* mT0, const double* share, const bte_rta_params* rp, int nthreads,
                       int log_impl, bte_rta_result* out, int64_t* counters) {
    try {
        orc::Sim S = build_sim(mt, gm);
        for (int k = 0; k < nmat; ++k) {
            const std::size_t n = S.m.n();
            S.mat_w.emplace_back(mw + std::size_t(k) * n, mw + std::size_t(k + 1) * n);
            S.mat_res.push_back(orc::fill_cumulative(orc::be_derivative_pmf(S.m, S.mat_w.back(), mT0[k])));
            S.mat_T0.push_back(mT0[k]);
        }
        // time grid (src/RTA_MC2D.cpp:2118-2124), Eigen LinSpaced(low + i*step)
        std::size_t ntime = std::size_t(std::floor(rp->maxtime / rp->dt + 1.0e-6)) + 1;
        double maxtime = double(ntime - 1) * rp->dt;
        S.timegrid.resize(ntime);
        double step = (maxtime - 0.0) / double(ntime - 1);
        for (std::size_t i = 0; i < ntime; ++i)
            S.timegrid[i] = (i == ntime - 1) ? maxtime : 0.0 + double(i) * step;
        // resampling distribution (BE_derivative_distribution)
        S.resample_cdf = orc::fill_cumulative(orc::be_derivative_pmf(S.m, S.m.w, rp->T0));
        orc::build_lambert(S);
        int64_t total_particles = rp->nparticles;
        std::vector<double> Em;  // energy rate per material (with shares)
        if (rp->source == BTE_SOURCE_WALLS) {
            orc::build_generators(S, rp->T0);
            S.Eeff = S.energy / double(rp->nparticles);
            if (share && nmat > 0) {
                Em.assign(std::size_t(nmat), 0.);
                std::vector<double> e;
                for (auto& g : S.gens) {
                    double Lb = orc::norm(g.b.p2 - g.b.p1);
                    e.push_back(std::fabs(g.flux) * Lb * S.thickness);
                    Em[std::size_t(S.sys[g.box].mat)] += e.back();
                }
                double cum = 0.;
                for (std::size_t i = 0; i < S.gens.size(); ++i) {
                    const std::size_t k = std::size_t(S.sys[S.gens[i].box].mat);
                    cum += share[k] * e[i] / Em[k];
                    S.gen_cum[i] = cum;
                }
            }
        } else {
            orc::build_initial(S, rp->nparticles, rp->seed);
            total_particles = S.init_first.back();
        }
        orc::Opts o;
        o.ballistic = rp->ballistic != 0;
        o.log_impl = log_impl;
        o.specularity = rp->specularity;
        const std::size_t nbx = S.sys.size(), nbn = ntime - 1;
        int64_t begin = rp->particle_begin,
                end = rp->particle_end > 0 ? std::min<int64_t>(rp->particle_end, total_particles) : total_particles;
        if (end < begin) end = begin;
        if (nthreads < 1) nthreads = 1;
        std::vector<orc::Tally> tl(static_cast<std::size_t>(nthreads));
        std::vector<std::string> errs(static_cast<std::size_t>(nthreads));
        std::vector<int> codes(static_cast<std::size_t>(nthreads), 0);
        std::vector<int> locs(nbx, -1);
        for (std::size_t i = 0; i < g_spec_boxes.size(); ++i) locs[std::size_t(g_spec_boxes[i])] = int(i);
        auto work = [&](int tid) {
            orc::Tally& T = tl[std::size_t(tid)];
            T.init(nbx, nbn);
            if (!g_spec_boxes.empty()) {
                T.loc = &locs;
                T.nmodes = S.m.n();
                T.spec.assign(g_spec_boxes.size() * nbn * S.m.n(), 0);
            }
            int64_t n = end - begin;
            int64_t lo = begin + n * tid / nthreads, hi = begin + n * (tid + 1) / nthreads;
            try {
                for (int64_t i = lo; i < hi; ++i)
                    orc::run_particle(S, std::size_t(i), rp->seed, maxtime, T, o);
            } catch (const orc::value_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_VALUE;
            } catch (const orc::limit_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_LIMIT;
            } catch (const orc::input_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_INPUT;
            } catch (const std::exception& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_GEOMETRY;
            }
        };
        const auto loop_start = std::chrono::steady_clock::now();
        if (nthreads == 1) {
            work(0);
        } else {
            std::vector<std::thread> th;
            for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
            for (auto& t : th) t.join();
        }
        const double loop_us = std::chrono::duration<double, std::micro>(
                                   std::chrono::steady_clock::now() - loop_start).count();
        for (std::size_t t = 0; t < errs.size(); ++t)
            if (!errs[t].empty()) return fail(codes[t], errs[t].c_str());
        orc::Tally T = std::move(tl[0]);
        for (std::size_t t = 1; t < tl.size(); ++t) {
            for (std::size_t k = 0; k < T.gz.size(); ++k) {
                T.gz[k] += tl[t].gz[k];
                T.jx[k] += tl[t].jx[k];
                T.jy[k] += tl[t].jy[k];
            }
            for (std::size_t k = 0; k < T.ex.size(); ++k) T.ex[k] += tl[t].ex[k];
            T.events += tl[t].events;
            T.wall_hits += tl[t].wall_hits;
            T.crossings += tl[t].crossings;
            T.absorbed += tl[t].absorbed;
            T.nudges += tl[t].nudges;
            T.quirks += tl[t].quirks;
            T.specular += tl[t].specular;
            T.translations += tl[t].translations;
            for (std::size_t k = 0; k < T.spec.size(); ++k) T.spec[k] += tl[t].spec[k];
        }
        g_spec_last = T.spec;
        out->nboxes = int32_t(nbx);
        out->nbins = int32_t(nbn);
        out->Eeff = S.Eeff;
        out->energy_rate = S.energy;
        out->events = T.events;
        out->wall_hits = T.wall_hits;
        out->crossings = T.crossings;
        out->absorbed = T.absorbed;
        out->specular_hits = T.specular;
        out->tally_updates = 0;
        out->translations = T.translations;
        if (counters) {
            counters[0] = T.events; counters[1] = T.wall_hits; counters[2] = T.crossings;
            counters[3] = T.absorbed; counters[4] = T.nudges; counters[5] = T.quirks;
            counters[6] = int64_t(loop_us);  // the particle loop alone (no table set-up)
        }
        const std::size_t nk = nbx * nbn;
        if (out->gz) std::copy(T.gz.begin(), T.gz.end(), out->gz);
        if (out->gz_jx) std::copy(T.jx.begin(), T.jx.end(), out->gz_jx);
        if (out->gz_jy) std::copy(T.jy.begin(), T.jy.end(), out->gz_jy);
        if (out->exact)
            for (std::size_t k = 0; k < nk * 3; ++k) {
                unsigned __int128 u = (unsigned __int128)T.ex[k];
                out->exact[2 * k] = int64_t(uint64_t(u >> 64));
                out->exact[2 * k + 1] = int64_t(uint64_t(u));
            }
        // post-processing, src/RTA_MC2D.cpp:2336-2435
        std::vector<double> gz = T.gz, jx = T.jx, jy = T.jy;
        for (std::size_t ir = 0; ir < nbx; ++ir) {
            double vbox = S.sys[ir].area * S.thickness;
            for (std::size_t i = 0; i < nbn; ++i) {
                gz[ir * nbn + i] /= vbox;
                jx[ir * nbn + i] /= vbox;
                jy[ir * nbn + i] /= vbox;
            }
        }
        if (!Em.empty()) {
            for (std::size_t ir = 0; ir < nbx; ++ir) {
                const std::size_t k = std::size_t(S.sys[ir].mat);
                const double E = share[k] > 0. ? Em[k] / (share[k] * double(rp->nparticles)) : 0.;
                for (std::size_t i = 0; i < nbn; ++i) {
                    gz[ir * nbn + i] *= E;
                    jx[ir * nbn + i] *= E * 1e12 * 1e9 * 1e9;
                    jy[ir * nbn + i] *= E * 1e12 * 1e9 * 1e9;
                }
            }
        } else {
            for (auto& x : gz) x *= S.Eeff;
            for (auto& x : jx) x *= S.Eeff * 1e12 * 1e9 * 1e9;
            for (auto& x : jy) x *= S.Eeff * 1e12 * 1e9 * 1e9;
        }
        if (rp->source == BTE_SOURCE_WALLS) {
            for (std::size_t ir = 0; ir < nbx; ++ir)
                for (std::size_t i = 1; i < nbn; ++i) {
                    gz[ir * nbn + i] += gz[ir * nbn + i - 1];
                    jx[ir * nbn + i] += jx[ir * nbn + i - 1];
                    jy[ir * nbn + i] += jy[ir * nbn + i - 1];
                }
        } else {  // relaxation of an initial deviation: bin averages
            for (std::size_t k = 0; k < nk; ++k) {
                gz[k] /= step;
                jx[k] /= step;
                jy[k] /= step;
            }
        }
        double vcorr = S.thickness / S.m.c;
        auto cv_at = [&](double T) {
            double cv = 0.;
            for (std::size_t k = 0; k < S.m.n(); ++k) cv += orc::bose_einstein_kernel(S.m.omega[k], T);
            return cv * orc::kB / double(S.m.nq) / S.m.V;
        };
        if (out->temperature)
            for (std::size_t ir = 0; ir < nbx; ++ir) {
                const double T0b = nmat > 0 ? S.mat_T0[std::size_t(S.sys[ir].mat)] : rp->T0;
                const double cv = cv_at(T0b);
                for (std::size_t i = 0; i < nbn; ++i)
                    out->temperature[ir * nbn + i] = gz[ir * nbn + i] / (cv / vcorr) + T0b;
            }
        if (out->jx) std::copy(jx.begin(), jx.end(), out->jx);
        if (out->jy) std::copy(jy.begin(), jy.end(), out->jy);
        return 0;
    } catch (const orc::input_error& e) {
        return fail(BTE_ERR_INPUT, e.what());
    } catch (const orc::value_error& e) {
        return fail(BTE_ERR_VALUE, e.what());
    } catch (const orc::limit_error& e) {
        return fail(BTE_ERR_LIMIT, e.what());
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// A transient run of a geometry of nmat materials with their own mode
// tables mts[m] (box b in gm->material[b]), diffuse mismatch at the
// contacts between materials; production semantics (per-particle pcg64
// streams as oracle_rta_run, the interfaces draw from the particle's
// stream).  counters: events, wall_hits, crossings, absorbed, nudges,
// quirks, loop microseconds, interface hits, interface transmissions.
int oracle_rta_run_multi(const bte_mode_table* mts, int nmat, const bte_geometry* gm, const bte_rta_params* rp,
                         int nthreads, bte_rta_result* out, int64_t* counters, const double* thickness) {
    try {
        if (nmat < 1 || !gm->material) return fail(BTE_ERR_INPUT, "materials need mode tables and box materials");
        orc::MultiSim M;
        for (int k = 0; k < nmat; ++k) M.mats.push_back(build_sim(&mts[k], gm));
        if (thickness)  // each material's boxes at its own thickness (thicknesses[box])
            for (int k = 0; k < nmat; ++k) M.mats[std::size_t(k)].thickness = thickness[k];
        for (auto& b : M.mats[0].sys)
            if (b.mat < 0 || b.mat >= nmat) return fail(BTE_ERR_INPUT, "box material out of range");
        std::size_t ntime = std::size_t(std::floor(rp->maxtime / rp->dt + 1.0e-6)) + 1;
        double maxtime = double(ntime - 1) * rp->dt;
        const double step = maxtime / double(ntime - 1);
        for (auto& S : M.mats) {
            S.timegrid.resize(ntime);
            for (std::size_t i = 0; i < ntime; ++i) S.timegrid[i] = (i == ntime - 1) ? maxtime : double(i) * step;
            S.resample_cdf = orc::fill_cumulative(orc::be_derivative_pmf(S.m, S.m.w, rp->T0));
            orc::build_lambert(S);
        }
        orc::build_interfaces(M);
        std::size_t ntot = 0;  // the materials' modes one after the other
        for (auto& S : M.mats) {
            S.mode_off = ntot;
            ntot += S.m.n();
        }
        int64_t total_particles = rp->nparticles;
        if (rp->source == BTE_SOURCE_WALLS) {
            std::vector<double> e;
            for (int k = 0; k < nmat; ++k) {
                orc::Sim& S = M.mats[std::size_t(k)];
                orc::build_generators(S, rp->T0, false, k);
                for (std::size_t i = 0; i < S.gens.size(); ++i) {
                    M.gref.push_back({k, i});
                    e.push_back(std::fabs(S.gens[i].flux) * orc::norm(S.gens[i].b.p2 - S.gens[i].b.p1) * S.thickness);
                }
            }
            if (M.gref.empty()) return fail(BTE_ERR_INPUT, "no isothermal wall generator (no reservoir with a different Teq)");
            double total = 0.;
            for (double x : e) total += x;
            double cum = 0.;
            for (double x : e) {
                cum += x / total;
                M.gcum.push_back(cum);
            }
            M.energy = total;
            M.Eeff = total / double(rp->nparticles);
        } else {
            orc::build_initial_multi(M, rp->nparticles, rp->seed);
            total_particles = M.init_first.back();
        }
        orc::Opts o;
        o.ballistic = rp->ballistic != 0;
        o.specularity = rp->specularity;
        const std::size_t nbx = M.mats[0].sys.size(), nbn = ntime - 1;
        int64_t begin = rp->particle_begin,
                end = rp->particle_end > 0 ? std::min<int64_t>(rp->particle_end, total_particles) : total_particles;
        if (end < begin) end = begin;
        if (nthreads < 1) nthreads = 1;
        std::vector<orc::Tally> tl(static_cast<std::size_t>(nthreads));
        std::vector<std::string> errs(static_cast<std::size_t>(nthreads));
        std::vector<int> codes(static_cast<std::size_t>(nthreads), 0);
        std::vector<int> locs(nbx, -1);
        for (std::size_t q = 0; q < g_spec_boxes.size(); ++q) locs[std::size_t(g_spec_boxes[q])] = int(q);
        auto work = [&](int tid) {
            orc::Tally& T = tl[std::size_t(tid)];
            T.init(nbx, nbn);
            if (!g_spec_boxes.empty()) {
                T.loc = &locs;
                T.nmodes = ntot;
                T.spec.assign(g_spec_boxes.size() * nbn * ntot, 0);
            }
            const int64_t n = end - begin;
            const int64_t lo = begin + n * tid / nthreads, hi = begin + n * (tid + 1) / nthreads;
            try {
                for (int64_t i = lo; i < hi; ++i) orc::run_particle_multi(M, std::size_t(i), rp->seed, maxtime, T, o);
            } catch (const orc::value_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_VALUE;
            } catch (const orc::limit_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_LIMIT;
            } catch (const orc::input_error& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_INPUT;
            } catch (const std::exception& e) {
                errs[std::size_t(tid)] = e.what();
                codes[std::size_t(tid)] = BTE_ERR_GEOMETRY;
            }
        };
        const auto loop_start = std::chrono::steady_clock::now();
        {
            std::vector<std::thread> th;
            for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
            for (auto& t : th) t.join();
        }
        const double loop_us =
            std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - loop_start).count();
        for (std::size_t t = 0; t < errs.size(); ++t)
            if (!errs[t].empty()) return fail(codes[t], errs[t].c_str());
        orc::Tally T = std::move(tl[0]);
        for (std::size_t t = 1; t < tl.size(); ++t) {
            for (std::size_t k = 0; k < T.gz.size(); ++k) {
                T.gz[k] += tl[t].gz[k];
                T.jx[k] += tl[t].jx[k];
                T.jy[k] += tl[t].jy[k];
            }
            for (std::size_t k = 0; k < T.ex.size(); ++k) T.ex[k] += tl[t].ex[k];
            T.events += tl[t].events;
            T.wall_hits += tl[t].wall_hits;
            T.crossings += tl[t].crossings;
            T.absorbed += tl[t].absorbed;
            T.nudges += tl[t].nudges;
            T.quirks += tl[t].quirks;
            T.specular += tl[t].specular;
            T.translations += tl[t].translations;
            T.interface_hits += tl[t].interface_hits;
            T.interface_transmissions += tl[t].interface_transmissions;
            for (std::size_t k = 0; k < T.spec.size(); ++k) T.spec[k] += tl[t].spec[k];
        }
        g_spec_last = T.spec;
        // the exact 128-bit sums, as the replay kernels keep them
        if (out->exact)
            for (std::size_t k = 0; k < T.ex.size(); ++k) {
                unsigned __int128 u = (unsigned __int128)T.ex[k];
                out->exact[2 * k] = int64_t(uint64_t(u >> 64));
                out->exact[2 * k + 1] = int64_t(uint64_t(u));
            }
        out->nboxes = int32_t(nbx);
        out->nbins = int32_t(nbn);
        out->Eeff = M.Eeff;
        out->energy_rate = M.energy;
        out->events = T.events;
        out->wall_hits = T.wall_hits;
        out->crossings = T.crossings;
        out->absorbed = T.absorbed;
        out->specular_hits = T.specular;
        out->tally_updates = 0;
        out->translations = T.translations;
        if (counters) {
            counters[0] = T.events; counters[1] = T.wall_hits; counters[2] = T.crossings;
            counters[3] = T.absorbed; counters[4] = T.nudges; counters[5] = T.quirks;
            counters[6] = int64_t(loop_us);
            counters[7] = T.interface_hits; counters[8] = T.interface_transmissions;
        }
        if (out->gz) std::copy(T.gz.begin(), T.gz.end(), out->gz);
        if (out->gz_jx) std::copy(T.jx.begin(), T.jx.end(), out->gz_jx);
        if (out->gz_jy) std::copy(T.jy.begin(), T.jy.end(), out->gz_jy);
        // post-processing (src/RTA_MC2D.cpp:2336-2435), each box with its
        // material's heat capacity and out-of-plane lattice vector
        const orc::Sim& S0 = M.mats[0];
        std::vector<double> gz = T.gz, jx = T.jx, jy = T.jy;
        for (std::size_t ir = 0; ir < nbx; ++ir) {
            const double vbox = S0.sys[ir].area * M.mats[std::size_t(S0.sys[ir].mat)].thickness;
            for (std::size_t i = 0; i < nbn; ++i) {
                gz[ir * nbn + i] = gz[ir * nbn + i] / vbox * M.Eeff;
                jx[ir * nbn + i] = jx[ir * nbn + i] / vbox * (M.Eeff * 1e12 * 1e9 * 1e9);
                jy[ir * nbn + i] = jy[ir * nbn + i] / vbox * (M.Eeff * 1e12 * 1e9 * 1e9);
            }
        }
        if (rp->source == BTE_SOURCE_WALLS) {
            for (std::size_t ir = 0; ir < nbx; ++ir)
                for (std::size_t i = 1; i < nbn; ++i) {
                    gz[ir * nbn + i] += gz[ir * nbn + i - 1];
                    jx[ir * nbn + i] += jx[ir * nbn + i - 1];
                    jy[ir * nbn + i] += jy[ir * nbn + i - 1];
                }
        } else {
            for (std::size_t k = 0; k < gz.size(); ++k) {
                gz[k] /= step;
                jx[k] /= step;
                jy[k] /= step;
            }
        }
        if (out->temperature)
            for (std::size_t ir = 0; ir < nbx; ++ir) {
                const orc::Modes& m = M.mats[std::size_t(S0.sys[ir].mat)].m;
                double cv = 0.;
                for (std::size_t k = 0; k < m.n(); ++k) cv += orc::bose_einstein_kernel(m.omega[k], rp->T0);
                cv = cv * orc::kB / double(m.nq) / m.V;
                const double vcorr = M.mats[std::size_t(S0.sys[ir].mat)].thickness / m.c;
                for (std::size_t i = 0; i < nbn; ++i)
                    out->temperature[ir * nbn + i] = gz[ir * nbn + i] / (cv / vcorr) + rp->T0;
            }
        if (out->jx) std::copy(jx.begin(), jx.end(), out->jx);
        if (out->jy) std::copy(jy.begin(), jy.end(), out->jy);
        return 0;
    } catch (const orc::input_error& e) {
        return fail(BTE_ERR_INPUT, e.what());
    } catch (const orc::value_error& e) {
        return fail(BTE_ERR_VALUE, e.what());
    } catch (const orc::limit_error& e) {
        return fail(BTE_ERR_LIMIT, e.what());
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// reemit draws of the interface of tables A and B (as oracle_kat_dmm) from
// one pcg64(seed, stream), incident modes idx_in[i] of side A in turn.
int oracle_kat_dmm_reemit(const bte_mode_table* A, const bte_mode_table* B, double nx, double ny, double thickness,
                          double Tref, uint64_t seed, uint64_t stream, int n, const long long* idx_in, int* side_out,
                          long long* idx_out) {
    try {
        const orc::Modes a = modes_from(A), b = modes_from(B);
        const orc::Dmm D = orc::build_dmm(a, b, a.V * thickness / a.c, b.V * thickness / b.c, orc::V2{nx, ny}, 0.1,
                                          Tref);
        orc::Pcg64 rng(seed, stream);
        for (int i = 0; i < n; ++i) {
            std::size_t io = 0;
            side_out[i] = orc::dmm_reemit(D, 0, std::size_t(idx_in[i]), rng, io);
            idx_out[i] = (long long)io;
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(BTE_ERR_INPUT, e.what());
    }
}

// One interface table (the Diffuse_mismatch_distribution of tables A and B,
// normal (nx, ny) from A to B, thickness t, Tref): for incident mode i of
// side s (0 = A, 1 = B) its entries [first[s][i], first[s][i+1]) of
// (side out, mode out, cumulative).  Call with null outputs for the sizes
// (nentries[2]), then with arrays of those sizes.
int oracle_kat_dmm(const bte_mode_table* A, const bte_mode_table* B, double nx, double ny, double thickness,
                   double Tref, long long* nentries, long long* firstA, long long* firstB, int* side, long long* idx,
                   double* cum) {
    try {
        const orc::Modes a = modes_from(A), b = modes_from(B);
        const orc::Dmm D = orc::build_dmm(a, b, a.V * thickness / a.c, b.V * thickness / b.c, orc::V2{nx, ny}, 0.1,
                                          Tref);
        long long k = 0;
        for (int s = 0; s < 2; ++s) {
            long long* first = s == 0 ? firstA : firstB;
            long long cnt = 0;
            for (std::size_t i = 0; i < D.in[s].size(); ++i) {
                if (first) first[i] = cnt;
                for (const auto& e : D.in[s][i]) {
                    if (side) {
                        side[k] = e.side;
                        idx[k] = (long long)e.idx;
                        cum[k] = e.cum;
                    }
                    ++k;
                    ++cnt;
                }
            }
            if (first) first[D.in[s].size()] = cnt;
            nentries[s] = cnt;
        }
        return 0;
    } catch (const orc::value_error& e) {
        return fail(BTE_ERR_VALUE, e.what());
    } catch (const std::exception& e) {
        return fail(BTE_ERR_INPUT, e.what());
    }
}

namespace {
// The steady run over one Sim per material (mats[0] alone: the single
// table, every box in it; several: box b in material sys[b].mat, the
// interfaces in dmm).
int steady_core(std::vector<orc::Sim>& mats, const orc::DmmSet* dmm, const bte_steady_params* sp, int nthreads,
                bte_steady_result* out) {
    try {
        const bool multi = mats.size() > 1;
        const orc::Sim& S = mats[0];  // the boxes (shared by every material's Sim)
        auto mat_of = [&](std::size_t b) -> std::size_t { return multi ? std::size_t(S.sys[b].mat) : 0; };
        const double gx = sp->gradient[0], gy = sp->gradient[1];
        if (orc::almost_equal(std::sqrt(gx * gx + gy * gy), 0.))
            return fail(BTE_ERR_INPUT, "the steady state needs a non-zero temperature gradient");
        const std::size_t nbx = S.sys.size();
        orc::SteadyGen SG;
        double E0 = 0.;
        for (std::size_t k = 0; k < mats.size(); ++k) {
            orc::Sim& Sk = mats[k];
            Sk.resample_cdf = orc::fill_cumulative(orc::be_derivative_pmf(Sk.m, Sk.m.w, sp->T0));
            orc::build_lambert(Sk);
            orc::build_generators(Sk, sp->T0, false, multi ? int(k) : -1);
            if (!multi) {
                E0 = Sk.gens.empty() ? 0. : Sk.energy;
                for (std::size_t i = 0; i < Sk.gens.size(); ++i) SG.wall.push_back({0, i});
                SG.wall_cum = Sk.gen_cum;
            } else {
                for (std::size_t i = 0; i < Sk.gens.size(); ++i) SG.wall.push_back({int(k), i});
            }
            std::vector<orc::GradGen> gk = orc::build_gradient(Sk, gx, gy, multi ? int(k) : -1);
            for (auto& G : gk) SG.grad.push_back(std::move(G));
        }
        if (multi) {
            // wall weights |flux| L thickness over every material's
            // generators; gradient sources in ascending box order
            std::vector<double> e;
            for (auto& r : SG.wall) {
                const orc::Sim& Sr = mats[std::size_t(r.first)];
                const orc::WallGen& G = Sr.gens[r.second];
                e.push_back(std::fabs(G.flux) * orc::norm(G.b.p2 - G.b.p1) * Sr.thickness);
            }
            for (double x : e) E0 += x;
            double c = 0.;
            for (double x : e) {
                c += x / E0;
                SG.wall_cum.push_back(c);
            }
            std::stable_sort(SG.grad.begin(), SG.grad.end(),
                             [](const orc::GradGen& a, const orc::GradGen& b) { return a.box < b.box; });
        }
        std::vector<double> ge;
        for (auto& G : SG.grad) ge.push_back(G.energy);
        const double E1 = std::accumulate(ge.begin(), ge.end(), 0.);
        double cum = 0.;
        for (double w : ge) {
            cum += w / E1;
            SG.grad_cum.push_back(cum);
        }
        const double total = E0 + E1;
        if (!(total > 0.)) return fail(BTE_ERR_INPUT, "the generators inject no energy");
        SG.exg0 = E0 / total;
        SG.exg1 = E1 / total + SG.exg0;
        const int64_t N = sp->nparticles;
        const double Eeff = total / double(N);
        if (nthreads < 1) nthreads = 1;
        const int max_gen = sp->max_generations > 0 ? sp->max_generations : 100000;

        std::vector<__int128> ex(3 * nbx, 0);
        std::vector<double> oldv(3 * nbx, 0.), cur(3 * nbx, 0.);
        // spectral locations: per-mode time and segment counts over all generations
        std::vector<int> locs(nbx, -1);
        for (std::size_t i = 0; i < g_spec_boxes.size(); ++i) locs[std::size_t(g_spec_boxes[i])] = int(i);
        std::size_t ntot = 0;  // the materials' modes one after the other
        for (auto& Sk : mats) {
            Sk.mode_off = ntot;
            ntot += Sk.m.n();
        }
        const std::size_t nspec = g_spec_boxes.size() * ntot;
        std::vector<__int128> spec_tot(nspec, 0);
        std::vector<int64_t> cnt_tot(nspec, 0);
        std::vector<orc::Particle> carry;
        std::vector<std::size_t> bbox;
        std::vector<int> bsign;
        std::vector<int64_t> bfirst;
        int64_t nbirth = 0, births_total = 0;
        int64_t ev = 0, wh = 0, cr = 0, ab = 0, tr = 0, sc = 0, lost = 0, ih = 0, it_ = 0;
        int gen = 0, converged = 0;
        for (;;) {
            const int64_t nin = gen == 0 ? 0 : int64_t(carry.size());
            const int64_t nslots = gen == 0 ? N : nin + nbirth;
            std::vector<uint64_t> rank;
            if (gen == 0) {
                rank.resize(std::size_t(nslots));
                uint64_t c = 0;
                for (int64_t sl = 0; sl < nslots; ++sl) {
                    orc::Pcg64 r(sp->seed, orc::steady_stream(0, uint64_t(sl)));
                    rank[std::size_t(sl)] = c;
                    if (orc::steady_gen_type(SG, orc::canonical(r)) == 1) c++;
                }
            }
            std::vector<orc::Particle> outp(static_cast<std::size_t>(nslots));
            std::vector<char> fate(static_cast<std::size_t>(nslots), 0);
            std::vector<orc::Tally> tl(static_cast<std::size_t>(nthreads));
            std::vector<std::vector<int64_t>> phis(static_cast<std::size_t>(nthreads));
            std::vector<std::string> errs(static_cast<std::size_t>(nthreads));
            std::vector<int> codes(static_cast<std::size_t>(nthreads), 0);
            auto work = [&](int tid) {
                orc::Tally& T = tl[std::size_t(tid)];
                T.init(nbx, 1);
                if (nspec > 0) {
                    T.loc = &locs;
                    T.nmodes = ntot;
                    T.spec.assign(nspec, 0);
                    T.scnt.assign(nspec, 0);
                }
                std::vector<int64_t>& phi = phis[std::size_t(tid)];
                phi.assign(nbx, 0);
                const int64_t lo = nslots * tid / nthreads, hi = nslots * (tid + 1) / nthreads;
                try {
                    for (int64_t sl = lo; sl < hi; ++sl) {
                        orc::Pcg64 rng(sp->seed, orc::steady_stream(uint64_t(gen), uint64_t(sl)));
                        orc::Particle p;
                        if (gen == 0) {
                            p = orc::steady_generate0(mats, SG, rank[std::size_t(sl)], rng);
                        } else if (sl < nin) {
                            p = carry[std::size_t(sl)];
                        } else {
                            const int64_t k = sl - nin;
                            auto it = std::upper_bound(bfirst.begin(), bfirst.end(), k);
                            const std::size_t j = std::size_t(it - bfirst.begin()) - 1;
                            const orc::Sim& Sb = mats[mat_of(bbox[j])];
                            p.pos = orc::random_point(S.sys[bbox[j]], rng);
                            const std::size_t pos = orc::lower_bound_idx(Sb.resample_cdf, orc::canonical(rng));
                            p.q = pos / std::size_t(Sb.m.nb);
                            p.alpha = pos % std::size_t(Sb.m.nb);
                            p.sign = bsign[j];
                            p.box = bbox[j];
                        }
                        p.t = 0.;
                        // the flight in the material of the particle's box
                        // (material_w0[mat], :2580-2595)
                        const orc::Sim& Sp = mats[mat_of(p.box)];
                        const std::size_t k = p.q * std::size_t(Sp.m.nb) + p.alpha;
                        const orc::V2 v = orc::get_v(Sp.m, k);
                        const double w = Sp.m.w[k];
                        if (w == 0.) throw orc::value_error("invalid scattering rate");
                        double dt = -orc::bte_log(orc::canonical(rng)) / w;
                        T.events++;
                        orc::Fate f = orc::F_LOST;
                        int guard = 0;
                        while (!orc::almost_equal(dt, 0.)) {
                            if (++guard > 1000000) throw orc::limit_error("flight step cap");
                            orc::evolparticle_steady(Sp, p, v, dt, rng, T, f, sp->specularity, dmm);
                        }
                        fate[std::size_t(sl)] = char(f);
                        if (f == orc::F_SCATTER) phi[p.box] += p.sign;
                        if (f == orc::F_BOUNCE) outp[std::size_t(sl)] = p;
                    }
                } catch (const orc::value_error& e) {
                    errs[std::size_t(tid)] = e.what();
                    codes[std::size_t(tid)] = BTE_ERR_VALUE;
                } catch (const orc::limit_error& e) {
                    errs[std::size_t(tid)] = e.what();
                    codes[std::size_t(tid)] = BTE_ERR_LIMIT;
                } catch (const std::exception& e) {
                    errs[std::size_t(tid)] = e.what();
                    codes[std::size_t(tid)] = BTE_ERR_GEOMETRY;
                }
            };
            if (nthreads == 1) {
                work(0);
            } else {
                std::vector<std::thread> th;
                for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
                for (auto& t : th) t.join();
            }
            for (std::size_t t = 0; t < errs.size(); ++t)
                if (!errs[t].empty()) return fail(codes[t], errs[t].c_str());
            std::vector<int64_t> phi(nbx, 0);
            for (auto& T : tl) {
                for (std::size_t k = 0; k < 3 * nbx; ++k) ex[k] += T.ex[k];
                for (std::size_t k = 0; k < nspec; ++k) {
                    spec_tot[k] += T.spec[k];
                    cnt_tot[k] += T.scnt[k];
                }
                ev += T.events;
                wh += T.wall_hits;
                cr += T.crossings;
                ab += T.absorbed;
                tr += T.translations;
                ih += T.interface_hits;
                it_ += T.interface_transmissions;
            }
            for (auto& ph : phis)
                for (std::size_t b = 0; b < nbx; ++b) phi[b] += ph[b];
            carry.clear();
            for (int64_t sl = 0; sl < nslots; ++sl) {
                const char f = fate[std::size_t(sl)];
                if (f == orc::F_BOUNCE) carry.push_back(outp[std::size_t(sl)]);
                if (f == orc::F_SCATTER) sc++;
                if (f == orc::F_LOST) lost++;
            }
            bbox.clear();
            bsign.clear();
            bfirst.clear();
            nbirth = 0;
            for (std::size_t b = 0; b < nbx; ++b) {
                if (phi[b] == 0) continue;
                bfirst.push_back(nbirth);
                bbox.push_back(b);
                bsign.push_back(phi[b] >= 0 ? 1 : -1);
                nbirth += phi[b] >= 0 ? phi[b] : -phi[b];
            }
            births_total += nbirth;
            for (std::size_t b = 0; b < nbx; ++b)
                for (int q = 0; q < 3; ++q) cur[std::size_t(q) * nbx + b] = double(ex[3 * b + std::size_t(q)]) / 17592186044416.0;
            auto rel = [&](int q) {
                double a = 0., c = 0.;
                for (std::size_t b = 0; b < nbx; ++b) {
                    const double d = oldv[std::size_t(q) * nbx + b] - cur[std::size_t(q) * nbx + b];
                    a += d * d;
                }
                for (std::size_t b = 0; b < nbx; ++b) c += cur[std::size_t(q) * nbx + b] * cur[std::size_t(q) * nbx + b];
                return std::sqrt(a) / std::sqrt(c);
            };
            const double rgz = rel(0), rjx = rel(1), rjy = rel(2);
            if (orc::almost_equal(gx, 0.))
                converged = rgz < sp->eps_energy && rjy < sp->eps_flux;
            else if (orc::almost_equal(gy, 0.))
                converged = rgz < sp->eps_energy && rjx < sp->eps_flux;
            else
                converged = rgz < sp->eps_energy && rjx < sp->eps_flux && rjy < sp->eps_flux;
            if (out->log && gen < out->log_cap) {
                double* row = out->log + std::size_t(gen) * 4;
                row[0] = double(int64_t(carry.size()) + nbirth);
                row[1] = rgz;
                row[2] = rjx;
                row[3] = rjy;
            }
            oldv = cur;
            gen++;
            if (int64_t(carry.size()) + nbirth == 0 || converged || gen >= max_gen) break;
        }
        out->nboxes = int32_t(nbx);
        out->generations = gen;
        out->converged = converged;
        out->Eeff = Eeff;
        out->energy_rate = total;
        out->events = ev;
        out->wall_hits = wh;
        out->crossings = cr;
        out->absorbed = ab;
        out->translations = tr;
        out->scattered = sc;
        out->births = births_total;
        out->lost = lost;
        out->kernel_ms = 0.;
        g_spec_last = spec_tot;
        g_spec_cnt = cnt_tot;
        if (out->exact)
            for (std::size_t k = 0; k < 3 * nbx; ++k) {
                unsigned __int128 u = (unsigned __int128)ex[k];
                out->exact[2 * k] = int64_t(uint64_t(u >> 64));
                out->exact[2 * k + 1] = int64_t(uint64_t(u));
            }
        out->interface_hits = ih;
        out->interface_transmissions = it_;
        // post-processing, src/RTA_MC2D.cpp:2698-2731: C_v and vcorr of
        // each box's material
        std::vector<double> cvs, vcorrs;
        for (auto& Sk : mats) {
            double cv = 0.;
            for (std::size_t k = 0; k < Sk.m.n(); ++k) cv += orc::bose_einstein_kernel(Sk.m.omega[k], sp->T0);
            cvs.push_back(cv * orc::kB / double(Sk.m.nq) / Sk.m.V);
            vcorrs.push_back(Sk.thickness / Sk.m.c);
        }
        for (std::size_t b = 0; b < nbx; ++b) {
            const double vbox = S.sys[b].area * mats[mat_of(b)].thickness;
            const double z = cur[b], zx = cur[nbx + b], zy = cur[2 * nbx + b];
            if (out->gz) out->gz[b] = z;
            if (out->gz_jx) out->gz_jx[b] = zx;
            if (out->gz_jy) out->gz_jy[b] = zy;
            const double ed = z / vbox * Eeff;
            const std::size_t mk = mat_of(b);
            if (out->temperature) out->temperature[b] = ed / (cvs[mk] / vcorrs[mk]) + sp->T0;
            if (out->jx) out->jx[b] = zx / vbox * (Eeff * 1e12 * 1e9 * 1e9);
            if (out->jy) out->jy[b] = zy / vbox * (Eeff * 1e12 * 1e9 * 1e9);
        }
        return 0;
    } catch (const orc::input_error& e) {
        return fail(BTE_ERR_INPUT, e.what());
    } catch (const orc::value_error& e) {
        return fail(BTE_ERR_VALUE, e.what());
    } catch (const orc::limit_error& e) {
        return fail(BTE_ERR_LIMIT, e.what());
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}
}  // namespace

// One steady-state run of a periodic structure under a gradient (the
// restatement above) on `nthreads` host threads; fills `out` as
// bte_steady_run does.  Tallies are exact 128-bit sums, turned into doubles
// for the convergence test and the outputs.
int oracle_steady_run(const bte_mode_table* mt, const bte_geometry* gm, const bte_steady_params* sp,
                      int nthreads, bte_steady_result* out) {
    try {
        std::vector<orc::Sim> mats;
        mats.push_back(build_sim(mt, gm));
        return steady_core(mats, nullptr, sp, nthreads, out);
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// The steady state of a geometry of nmat crystals with their own mode
// tables mts[m] (box b in gm->material[b]), diffuse mismatch at the contacts
// between them (change_material_diffuse in the periodic evolparticle,
// src/RTA_MC2D.cpp:1672-1689, 1751-1779: the re-emitted particle is carried
// into the next generation).
int oracle_steady_run_multi(const bte_mode_table* mts, int nmat, const bte_geometry* gm,
                            const bte_steady_params* sp, int nthreads, bte_steady_result* out,
                            const double* thickness) {
    try {
        if (nmat < 1 || !gm->material) return fail(BTE_ERR_INPUT, "materials need mode tables and box materials");
        orc::MultiSim M;
        for (int k = 0; k < nmat; ++k) M.mats.push_back(build_sim(&mts[k], gm));
        if (thickness)
            for (int k = 0; k < nmat; ++k) M.mats[std::size_t(k)].thickness = thickness[k];
        for (auto& b : M.mats[0].sys)
            if (b.mat < 0 || b.mat >= nmat) return fail(BTE_ERR_INPUT, "box material out of range");
        orc::build_interfaces(M);
        if (nmat == 1) {
            // one crystal: box materials are all 0, the single-table run
            return steady_core(M.mats, nullptr, sp, nthreads, out);
        }
        return steady_core(M.mats, &M.dmm, sp, nthreads, out);
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

// One beRTAMC2D run (see the restatement above).  P: [nmP*nmP] column-major
// propagator over modes 3..n-1 (ignored when params->rta).  Outputs per step
// s = 0..nsteps: ed[s][box] (J m^-3), flux[s][box][2] (J m^-2 s^-1),
// nparticles[s]; H_out: final histogram [box][mode] (optional).
// beRTA with the propagator tabulated at nprop temperatures Ts (P: the
// nprop column-major nmP x nmP matrices one after the other).  The run at
// Teq = T0 takes the tabulated propagator at T0, or lirp between the first
// tabulated temperature above T0 and the next one (Scattering,
// src/beyondRTA_MC2d.cpp:1130-1165; lirp src/collision_operator.cpp:918-929).
int oracle_berta_run_tab(const bte_mode_table* mt, const bte_geometry* gm, const double* P,
                         const double* Ts, int nprop, int nmP, const bte_berta_params* bp, double* ed_out,
                         double* flux_out, int64_t* np_out, int32_t* H_out, int64_t* counters);

int oracle_berta_run(const bte_mode_table* mt, const bte_geometry* gm, const double* P, int nmP,
                     const bte_berta_params* bp, double* ed_out, double* flux_out,
                     int64_t* np_out, int32_t* H_out, int64_t* counters) {
    const double T0 = bp->T0;
    return oracle_berta_run_tab(mt, gm, P, &T0, 1, nmP, bp, ed_out, flux_out, np_out, H_out, counters);
}

int oracle_berta_run_tab(const bte_mode_table* mt, const bte_geometry* gm, const double* P,
                         const double* Ts, int nprop, int nmP, const bte_berta_params* bp, double* ed_out,
                         double* flux_out, int64_t* np_out, int32_t* H_out, int64_t* counters) {
    try {
        orc::BeRun R;
        R.S = build_sim(mt, gm);
        orc::Sim& S = R.S;
        const orc::Modes& m = S.m;
        const std::size_t n = m.n(), nbx = S.sys.size();
        R.rta = bp->rta != 0;
        R.dt = bp->dt;
        R.maxtime = bp->maxtime;
        R.Eeff = bp->Eeff;
        if (!(R.Eeff > 0.)) return fail(BTE_ERR_INPUT, "Eeff must be positive");
        if (!R.rta) {
            if (nmP != int(n) - 3) return fail(BTE_ERR_INPUT, "propagator size must be nmodes - 3");
            if (nprop < 1) return fail(BTE_ERR_INPUT, "no propagator");
            R.nm = nmP;
            const std::size_t nn = std::size_t(nmP) * std::size_t(nmP);
            std::map<double, const double*> tab;
            for (int i = 0; i < nprop; ++i) tab[Ts[i]] = P + std::size_t(i) * nn;
            // the table of each box's Teq: the tabulated one, or lirp between
            // the first tabulated temperature above Teq and the next one
            std::map<double, std::size_t> of_T;
            for (auto& s : S.sys) {
                if (s.reservoir || s.periodic || of_T.count(s.Teq)) continue;
                orc::BeRun R1;
                R1.nm = nmP;
                const auto hit = tab.find(s.Teq);
                if (hit != tab.end()) {
                    orc::build_cumm(R1, hit->second);
                } else {
                    const auto m1 = tab.lower_bound(s.Teq);
                    if (m1 == tab.end() || std::next(m1) == tab.end() || s.Teq < tab.begin()->first)
                        return fail(BTE_ERR_INPUT, "Extrapolation is not allowed");
                    const auto m2 = std::next(m1);
                    orc::BeRun R2;
                    R2.nm = nmP;
                    orc::build_cumm(R1, m1->second);
                    orc::build_cumm(R2, m2->second);
                    const double T1 = m1->first, T2 = m2->first;
                    for (std::size_t i = 0; i < nn; ++i)
                        R1.cumm[i] = orc::lirp_value(R1.cumm[i], R2.cumm[i], T1, T2, s.Teq);
                }
                of_T[s.Teq] = R.cumms.size();
                R.cumms.push_back(std::move(R1.cumm));
            }
            R.box_cumm.assign(nbx, nullptr);
            for (auto& s : S.sys)
                if (!s.reservoir && !s.periodic) R.box_cumm[s.id] = R.cumms[of_T.at(s.Teq)].data();
        } else {
            // the mode table's rates are given at T0 only
            for (auto& s : S.sys)
                if (!s.reservoir && !s.periodic && s.Teq != bp->T0)
                    return fail(BTE_ERR_INPUT, "RTA scattering needs Teq = T0 in every box");
            R.resample_cdf = orc::fill_cumulative(orc::be_derivative_pmf(m, m.w, bp->T0));
        }
        for (auto& b : S.sys) {
            R.Eborder.push_back(std::vector<int>(b.borders.size(), 0));
            R.spl.push_back(std::vector<orc::Spline>(b.borders.size()));
            R.spl_ok.push_back(std::vector<char>(b.borders.size(), 0));
        }
        orc::build_generators(S, bp->T0, false);
        orc::Pcg64 rng(bp->seed, 0), rng_(bp->seed, 1);
        const double vuc = m.V * S.thickness / m.c;
        std::vector<orc::BeParticle> parts;
        // init_particles (Tinit != Teq), src/beyondRTA_MC2d.cpp:211-269
        std::vector<double> pmf;
        for (auto& s : S.sys) {
            if (s.reservoir || s.periodic || orc::almost_equal(s.Teq, s.Treal)) continue;
            const double cumulsum = orc::out_tref_pmf(m, s.Treal, s.Teq, pmf);
            const int sgn = (s.Treal - s.Teq) >= 0 ? 1 : -1;
            auto cdf = orc::fill_cumulative(pmf);
            const double vol = s.area * S.thickness / vuc;
            const std::size_t ngen = orc::n_to_generate(orc::gen_plain(vol, cumulsum, R.Eeff, double(m.nq)), rng);
            double x0 = s.hull[0].x, x1 = x0, y0 = s.hull[0].y, y1 = y0;
            for (auto& h : s.hull) {
                x0 = std::min(x0, h.x); x1 = std::max(x1, h.x);
                y0 = std::min(y0, h.y); y1 = std::max(y1, h.y);
            }
            for (std::size_t i = 0; i < ngen; ++i) {
                orc::V2 r;
                for (int tries = 0;; ++tries) {
                    if (tries > 100000) throw orc::limit_error("random point rejection loop");
                    r.x = x0 + orc::canonical(rng) * (x1 - x0);
                    r.y = y0 + orc::canonical(rng) * (y1 - y0);
                    if (s.inside(r)) break;
                }
                orc::BeParticle p;
                p.pos = r;
                p.mode = orc::lower_bound_idx(cdf, orc::canonical(rng));
                p.sign = sgn;
                p.box = s.id;
                parts.push_back(p);
            }
        }
        std::vector<double> vol(nbx);
        for (std::size_t i = 0; i < nbx; ++i) vol[i] = S.sys[i].area * S.thickness;
        int64_t step_out = 0, psteps = 0, branches = 0;
        auto emit_props_particles = [&]() {
            std::vector<double> ed(nbx, 0.), fx(nbx, 0.), fy(nbx, 0.);
            for (auto& p : parts) {
                ed[p.box] += p.sign;
                fx[p.box] += p.sign * m.vx[p.mode];
                fy[p.box] += p.sign * m.vy[p.mode];
            }
            for (std::size_t i = 0; i < nbx; ++i) {
                ed_out[step_out * nbx + i] = ed[i] * (R.Eeff / vol[i] * 1.0e+27);
                flux_out[(step_out * nbx + i) * 2] = fx[i] * (R.Eeff / vol[i] * 1e12 * 1e9 * 1e9);
                flux_out[(step_out * nbx + i) * 2 + 1] = fy[i] * (R.Eeff / vol[i] * 1e12 * 1e9 * 1e9);
            }
            np_out[step_out] = int64_t(parts.size());
            step_out++;
        };
        emit_props_particles();
        std::vector<int> H(nbx * n);
        double time = 0.;
        std::size_t istep = 0;
        auto advect_new = [&](std::vector<orc::BeParticle>& np) {
            for (auto& p : np) {
                const double rdt = R.dt * orc::canonical(rng_);
                orc::be_evolve(R, p, orc::get_v(m, p.mode), rdt, rng_);
            }
            parts.insert(parts.end(), np.begin(), np.end());
        };
        // gradient source term (source_term_gradient, src/beyondRTA_MC2d.cpp:
        // 597-676): the homogeneous <gradient> on every box that is neither a
        // reservoir nor periodic, or (the default, :1441-1458) the gradients
        // of the boxes' Teq from calculate_gradientT; the generators are
        // built once
        std::vector<orc::GradGen> grad;
        if (bp->gradient_mode == 1) {
            if (!orc::almost_equal(std::hypot(bp->gradient[0], bp->gradient[1]), 0.))
                grad = orc::build_gradient(S, bp->gradient[0], bp->gradient[1]);
        } else {
            grad = orc::build_gradient_boxes(S, orc::calculate_gradientT(S));
        }
        while (time <= R.maxtime) {
            // 1. advection
            for (auto& p : parts) orc::be_evolve(R, p, orc::get_v(m, p.mode), R.dt, rng_);
            psteps += int64_t(parts.size());
            // 2. gradient source: Ntogenerate(dt, vol, Eeff) particles per box at
            // random points, mode and sign from the Nabla_T distribution
            if (!grad.empty()) {
                std::vector<orc::BeParticle> np;
                for (auto& G : grad) {
                    const std::size_t ngen = orc::n_to_generate(
                        orc::gen_scaled(R.dt, G.vol, G.cumulsum, R.Eeff, double(m.nq)), rng);
                    for (std::size_t i = 0; i < ngen; ++i) {
                        orc::BeParticle p;
                        p.pos = orc::random_point(S.sys[G.box], rng);
                        p.mode = orc::lower_bound_idx(G.cdf, orc::canonical(rng));
                        p.sign = G.sign[std::size_t(p.mode)];
                        p.box = int(G.box);
                        np.push_back(p);
                    }
                }
                advect_new(np);
            }
            // 3. isothermal walls
            {
                std::vector<orc::BeParticle> np;
                for (auto& g : S.gens) {
                    const double Lb = orc::norm(g.b.p2 - g.b.p1);
                    const double spf = Lb * S.thickness / (m.V * S.thickness / m.c);
                    const std::size_t ngen =
                        orc::n_to_generate(orc::gen_scaled(R.dt, spf, g.cumulsum, R.Eeff, double(m.nq)), rng);
                    const orc::Box& inj = S.sys[g.box];
                    for (std::size_t i = 0; i < ngen; ++i) {
                        orc::V2 pp = orc::border_point(g.b, rng);
                        if (!inj.inside(pp)) {
                            orc::V2 d = inj.center - pp;
                            pp = pp + (1.0e-6 * d) / orc::norm(d);
                            if (!inj.inside(pp)) throw orc::geometry_error("Generated particle out of insertion box");
                        }
                        orc::BeParticle p;
                        p.pos = pp;
                        p.mode = orc::lower_bound_idx(g.cdf, orc::canonical(rng));
                        p.sign = g.sign;
                        p.box = g.box;
                        np.push_back(p);
                    }
                }
                advect_new(np);
            }
            // 4. adiabatic diffuse walls
            {
                std::vector<orc::BeParticle> np;
                for (auto& s : S.sys) {
                    if (s.reservoir || s.periodic) continue;
                    for (std::size_t k = 0; k < s.borders.size(); ++k) {
                        const orc::Border& b = s.borders[k];
                        const orc::V2 nwall = {-b.np.x, -b.np.y};
                        if (!R.spl_ok[s.id][k]) {
                            std::vector<double> J(100), Tv(100);
                            for (int t = 0; t < 100; ++t) {
                                const double T = 10.0 + 10.0 * t;
                                Tv[std::size_t(t)] = T;
                                const double cs = orc::wall_pmf(m, nwall, T, s.Teq, pmf);
                                const int sg = (T - s.Teq) >= 0 ? 1 : -1;
                                J[std::size_t(t)] = sg * (cs / (double(m.nq) * vuc));
                            }
                            R.spl[s.id][k].build(J, Tv);
                            R.spl_ok[s.id][k] = 1;
                        }
                        int& E = R.Eborder[s.id][k];
                        if (E != 0) {
                            const double Jb = R.Eeff * E / R.dt / (orc::norm(b.p2 - b.p1) * S.thickness);
                            const double Tb = R.spl[s.id][k].interp(Jb);
                            orc::wall_pmf(m, nwall, Tb, s.Teq, pmf);
                            auto cdf = orc::fill_cumulative(pmf);
                            const int sg = (Tb - s.Teq) >= 0 ? 1 : -1;
                            const std::size_t ng = std::size_t(std::abs(E) + 1.0e-6);
                            for (std::size_t i = 0; i < ng; ++i) {
                                orc::BeParticle p;
                                p.pos = orc::border_point(b, rng);
                                p.mode = orc::lower_bound_idx(cdf, orc::canonical(rng));
                                p.sign = sg;
                                p.box = s.id;
                                np.push_back(p);
                            }
                            E = 0;
                        }
                    }
                }
                advect_new(np);
            }
            // 5. delete
            parts.erase(std::remove_if(parts.begin(), parts.end(),
                                       [](const orc::BeParticle& p) { return p.mode == 0; }),
                        parts.end());
            // 6. scattering
            if (R.rta) {
                for (auto& p : parts) {
                    const double w = m.w[p.mode];
                    const double u = orc::canonical(rng_);
                    if (u < (1 - std::exp(-w * R.dt)))
                        p.mode = orc::lower_bound_idx(R.resample_cdf, orc::canonical(rng_));
                }
            } else {
                std::vector<orc::BeParticle> elements = parts, out;
                int rounds = 0;
                while (!elements.empty()) {
                    if (++rounds > 4096) throw orc::limit_error("branching rounds cap");
                    std::vector<orc::BeParticle> next;
                    for (auto& p : elements) {
                        if (p.mode < 3) throw orc::value_error("Gamma acoustic particle has no propagator column");
                        const double u = orc::canonical(rng_);
                        const double* t = R.box_cumm[p.box];
                        if (!t) throw orc::value_error("particle where nothing scatters");
                        auto sol = orc::prop_get_tab(R, t, p.mode - 3, u);
                        const int newsign = (p.sign * sol.first) < 0 ? -1 : 1;
                        orc::BeParticle s1 = p;
                        s1.mode = sol.second;
                        s1.sign = newsign;
                        out.push_back(s1);
                        if (newsign * p.sign < 0) {
                            next.push_back(p);
                            next.push_back(p);
                            branches++;
                        }
                    }
                    elements.swap(next);
                }
                parts.swap(out);
            }
            // 7. histogram
            std::fill(H.begin(), H.end(), 0);
            for (auto& p : parts) H[p.box * n + p.mode] += p.sign;
            // 8. cancellation every 4th step
            if (istep % 4 == 0) {
                std::vector<int> Hc(H);
                // the reference sorts with tbb::parallel_sort, which leaves the
                // order of equal (box, mode, sign) particles unspecified; the
                // survivors are taken uniformly at random here (a seeded
                // Fisher-Yates shuffle before a stable sort)
                for (std::size_t i = parts.size(); i > 1; --i) {
                    const std::size_t j = std::size_t(orc::uniform_int(rng_, 0, int(i) - 1));
                    std::swap(parts[i - 1], parts[j]);
                }
                std::stable_sort(parts.begin(), parts.end(), [](const orc::BeParticle& a, const orc::BeParticle& b) {
                    return std::make_tuple(a.box, a.mode, a.sign) < std::make_tuple(b.box, b.mode, b.sign);
                });
                std::vector<orc::BeParticle> kept;
                for (auto& p : parts) {
                    if (S.sys[p.box].reservoir) continue;
                    int& h = Hc[p.box * n + p.mode];
                    if (h == 0) continue;
                    if ((p.sign < 0) != (h < 0)) continue;
                    h -= p.sign;
                    kept.push_back(p);
                }
                parts.swap(kept);
            }
            // 9. properties from the histogram
            for (std::size_t i = 0; i < nbx; ++i) {
                double e = 0., fx = 0., fy = 0.;
                for (std::size_t k = 0; k < n; ++k) {
                    const double hk = double(H[i * n + k]);
                    e += hk;
                    fx += hk * m.vx[k];
                    fy += hk * m.vy[k];
                }
                ed_out[step_out * nbx + i] = (R.Eeff / vol[i] * 1.0e+27) * e;
                flux_out[(step_out * nbx + i) * 2] = (R.Eeff / vol[i] * 1.0e+30) * fx;
                flux_out[(step_out * nbx + i) * 2 + 1] = (R.Eeff / vol[i] * 1.0e+30) * fy;
            }
            np_out[step_out] = int64_t(parts.size());
            step_out++;
            istep++;
            time += R.dt;
        }
        if (H_out) std::copy(H.begin(), H.end(), H_out);
        if (counters) {
            counters[0] = psteps;
            counters[1] = branches;
            counters[2] = step_out;
        }
        return 0;
    } catch (const orc::input_error& e) {
        return fail(BTE_ERR_INPUT, e.what());
    } catch (const orc::value_error& e) {
        return fail(BTE_ERR_VALUE, e.what());
    } catch (const orc::limit_error& e) {
        return fail(BTE_ERR_LIMIT, e.what());
    } catch (const std::exception& e) {
        return fail(BTE_ERR_GEOMETRY, e.what());
    }
}

}  // extern "C"
