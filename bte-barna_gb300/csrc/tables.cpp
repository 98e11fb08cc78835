// tables.cpp - host construction of the device tables (see tables.hpp).
//
// The formulas and their operation order follow the reference so that the
// replay mode reproduces the CPU restatement bit for bit:
//   geometry_2d ctor / get_sides      src/geometry_2d.cpp:51-153
//   calculate_contacts                src/geometry_2d.cpp:295-381
//   BE_derivative_distribution        src/sampling.cpp:47-68
//   Isothermal_wall_distribution      src/sampling.cpp:189-269
//   outTref_distribution              src/sampling.cpp:271-330
//   fill_cumulative                   src/sampling.cpp:26-44
//   diffusive_bouncing table + bounce src/RTA_MC2D.cpp:556-678
//   Init_generator weights            src/RTA_MC2D.cpp:289-418
//   calc_cv                           include/bulk_properties.hpp:32-47
#include "tables.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <thread>
#include <tuple>

namespace bte {

namespace {
constexpr double kB = 1.3806488e-23;
constexpr double hbar = 1.054571726e-34;
constexpr double nsigma = 2.828427124746190097603377448419396157138;
constexpr double PI = 3.1415926535897932384626433832795028841953;

V2 vneg(V2 a) { return v2(-1. * a.x, -1. * a.y); }

std::vector<V2> convex_hull(std::vector<V2> pts) {
    std::sort(pts.begin(), pts.end(),
              [](V2 a, V2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); });
    pts.erase(std::unique(pts.begin(), pts.end(),
                          [](V2 a, V2 b) { return a.x == b.x && a.y == b.y; }),
              pts.end());
    if (pts.size() < 3) throw Error(BTE_ERR_INPUT, "a box needs three distinct vertices");
    std::vector<V2> h(2 * pts.size());
    std::size_t k = 0;
    for (std::size_t i = 0; i < pts.size(); ++i) {
        while (k >= 2 && cross(sub(h[k - 1], h[k - 2]), sub(pts[i], h[k - 2])) <= 0.) --k;
        h[k++] = pts[i];
    }
    for (std::size_t i = pts.size() - 1, t = k + 1; i > 0; --i) {
        while (k >= t && cross(sub(h[k - 1], h[k - 2]), sub(pts[i - 1], h[k - 2])) <= 0.) --k;
        h[k++] = pts[i - 1];
    }
    h.resize(k - 1);
    return h;
}

struct BoxBuild {
    std::vector<V2> hull;
    V2 center;
    double area;
    std::vector<GBorder> borders;
    std::map<int, GBorder> contacts;  // neighbour -> contact border (seen from here)
};

BoxBuild make_box(const std::vector<V2>& verts) {
    BoxBuild b;
    b.hull = convex_hull(verts);
    const std::size_t n = b.hull.size();
    double a2 = 0, cx = 0, cy = 0;
    const V2 o = b.hull[0];
    for (std::size_t i = 0; i < n; ++i) {
        V2 p = sub(b.hull[i], o), q = sub(b.hull[(i + 1) % n], o);
        double c = cross(p, q);
        a2 += c;
        cx += (p.x + q.x) * c;
        cy += (p.y + q.y) * c;
    }
    b.area = 0.5 * a2;
    b.center = v2(o.x + cx / (3. * a2), o.y + cy / (3. * a2));
    for (std::size_t i = 0; i < verts.size(); ++i) {
        V2 p1 = verts[i];
        for (std::size_t j = i; j < verts.size(); ++j) {
            V2 p2 = verts[j];
            if (norm(sub(p1, p2)) < 1.0e-6) continue;
            V2 sc = v2((p1.x + p2.x) / 2., (p1.y + p2.y) / 2.);
            V2 ncsc = sub(sc, b.center);
            if (norm(ncsc) == 0.) continue;
            double nc = 1. / norm(ncsc);
            ncsc.x *= 1.0e-4 * nc;
            ncsc.y *= 1.0e-4 * nc;
            V2 fp = add(ncsc, sc);
            if (inside_hull(b.hull.data(), int(b.hull.size()), fp)) continue;
            GBorder br{};
            br.p1 = p1;
            br.p2 = p2;
            br.nd = sub(p2, p1);
            V2 npt = v2(br.nd.y, -br.nd.x);
            if (dot(npt, ncsc) < 0.) npt = vneg(npt);
            br.np = divs(npt, norm(npt));
            br.la = sub(p1, scal(1.0e-6, br.nd));
            br.lb = add(p2, scal(1.0e-6, br.nd));
            bool dup = false;
            for (auto& o2 : b.borders)
                if (norm(sub(o2.np, br.np)) < 1.0e-6) dup = true;
            if (!dup) b.borders.push_back(br);
            if (b.borders.size() > verts.size()) throw Error(BTE_ERR_GEOMETRY, "To much borders");
        }
    }
    return b;
}

std::vector<V2> touching_points(const BoxBuild& A, const BoxBuild& B) {
    std::vector<V2> pts;
    auto addp = [&](V2 p) {
        for (auto& q : pts)
            if (q.x == p.x && q.y == p.y) return;
        pts.push_back(p);
    };
    const std::size_t na = A.hull.size(), nb = B.hull.size();
    for (std::size_t i = 0; i < na; ++i) {
        V2 a0 = A.hull[i], a1 = A.hull[(i + 1) % na];
        for (std::size_t j = 0; j < nb; ++j) {
            V2 b0 = B.hull[j], b1 = B.hull[(j + 1) % nb];
            if (on_segment(b0, a0, a1)) addp(b0);
            if (on_segment(b1, a0, a1)) addp(b1);
            if (on_segment(a0, b0, b1)) addp(a0);
            if (on_segment(a1, b0, b1)) addp(a1);
        }
    }
    if (pts.size() > 2) throw Error(BTE_ERR_GEOMETRY, "overlapping boxes are not supported");
    std::sort(pts.begin(), pts.end(),
              [](V2 a, V2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); });
    return pts;
}

std::vector<double> fill_cumulative(const std::vector<double>& p) {
    if (*std::min_element(p.begin(), p.end()) < 0.)
        throw Error(BTE_ERR_VALUE, "probabilities must be >= 0.");
    std::vector<double> c;
    c.reserve(p.size());
    std::partial_sum(p.begin(), p.end(), std::back_inserter(c));
    const double last = c.back();
    if (!(last > 0.)) throw Error(BTE_ERR_VALUE, "distribution with zero total weight");
    for (auto& x : c) x /= last;
    return c;
}

// Axis-aligned rectangle check: returns true and its bounds.
bool as_rect(const std::vector<V2>& hull, double& x0, double& y0, double& x1, double& y1) {
    if (hull.size() != 4) return false;
    x0 = x1 = hull[0].x;
    y0 = y1 = hull[0].y;
    for (auto& p : hull) {
        x0 = std::min(x0, p.x);
        x1 = std::max(x1, p.x);
        y0 = std::min(y0, p.y);
        y1 = std::max(y1, p.y);
    }
    for (auto& p : hull)
        if (!((p.x == x0 || p.x == x1) && (p.y == y0 || p.y == y1))) return false;
    return true;
}

void detect_grid(HostGeometry& G, const std::vector<BoxBuild>& bb) {
    std::vector<double> xs, ys;
    std::vector<std::array<double, 4>> r(bb.size());
    for (std::size_t i = 0; i < bb.size(); ++i) {
        if (!as_rect(bb[i].hull, r[i][0], r[i][1], r[i][2], r[i][3])) return;
        xs.push_back(r[i][0]);
        xs.push_back(r[i][2]);
        ys.push_back(r[i][1]);
        ys.push_back(r[i][3]);
    }
    std::sort(xs.begin(), xs.end());
    xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
    std::sort(ys.begin(), ys.end());
    ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
    const int nx = int(xs.size()) - 1, ny = int(ys.size()) - 1;
    if (nx < 1 || ny < 1 || double(nx) * ny > 5.0e7) return;
    std::vector<int> cell(std::size_t(nx) * ny, -1);
    for (std::size_t b = 0; b < bb.size(); ++b) {
        int i0 = int(std::lower_bound(xs.begin(), xs.end(), r[b][0]) - xs.begin());
        int i1 = int(std::lower_bound(xs.begin(), xs.end(), r[b][2]) - xs.begin());
        int j0 = int(std::lower_bound(ys.begin(), ys.end(), r[b][1]) - ys.begin());
        int j1 = int(std::lower_bound(ys.begin(), ys.end(), r[b][3]) - ys.begin());
        if (i1 != i0 + 1 || j1 != j0 + 1) return;  // a box spanning several cells
        int& c = cell[std::size_t(i0) * ny + j0];
        if (c != -1) return;
        c = G.reservoir[b] ? -2 - int(b) : int(b);
    }
    G.rect_grid = true;
    G.gnx = nx;
    G.gny = ny;
    G.gx = xs;
    G.gy = ys;
    G.gcell = std::move(cell);
}
}  // namespace

double bose_einstein(double omega, double T) {
    constexpr double prefactor = 1e12 * hbar / kB;
    return 1. / (std::exp(prefactor * omega / T) - 1.);
}

double bose_einstein_kernel(double omega, double T) {
    constexpr double prefactor = 0.5 * 1e12 * hbar / kB;
    double x = prefactor * omega / T;
    if (x < 1e-320) return 1.;
    if (x > 300.) return 0.;
    double s = x / std::sinh(x);
    return s * s;
}

double calc_cv(const HostModes& m, double T) {
    double cv = 0.;
    for (std::size_t k = 0; k < m.n(); ++k) cv += bose_einstein_kernel(m.omega[k], T);
    cv *= kB / double(m.nq) / m.V;
    return cv;
}

HostModes build_modes(const bte_mode_table* mt) {
    if (!mt || mt->nq < 2 || mt->nb < 1 || !mt->omega || !mt->vg || !mt->w || !mt->dq)
        throw Error(BTE_ERR_INPUT, "incomplete mode table");
    if (!(mt->V > 0.) || !(mt->c_lat > 0.)) throw Error(BTE_ERR_INPUT, "bad unit cell");
    HostModes m;
    m.nq = mt->nq;
    m.nb = mt->nb;
    for (int i = 0; i < 3; ++i) m.grid[i] = mt->grid[i];
    const std::size_t n = m.n();
    if (n > (std::size_t(1) << 30)) throw Error(BTE_ERR_INPUT, "too many modes");
    m.omega.assign(mt->omega, mt->omega + n);
    m.w.assign(mt->w, mt->w + n);
    m.vx.resize(n);
    m.vy.resize(n);
    m.vz.resize(n);
    m.vxc.resize(n);
    m.vyc.resize(n);
    for (std::size_t k = 0; k < n; ++k) {
        m.vx[k] = mt->vg[3 * k];
        m.vy[k] = mt->vg[3 * k + 1];
        m.vz[k] = mt->vg[3 * k + 2];
        m.vxc[k] = almost_equal(m.vx[k], 0.) ? 0. : m.vx[k];
        m.vyc[k] = almost_equal(m.vy[k], 0.) ? 0. : m.vy[k];
        if (!std::isfinite(m.omega[k]) || !std::isfinite(m.w[k]) || m.w[k] < 0.)
            throw Error(BTE_ERR_VALUE, "non-finite or negative mode data");
    }
    std::memcpy(m.dq, mt->dq, sizeof(m.dq));
    m.V = mt->V;
    m.c = mt->c_lat;
    return m;
}

HostGeometry build_geometry(const bte_geometry* g) {
    if (!g || g->nboxes < 1 || !g->npoints || !g->vertices || !g->Teq || !g->reservoir)
        throw Error(BTE_ERR_INPUT, "incomplete geometry");
    if (!(g->thickness > 0.)) throw Error(BTE_ERR_INPUT, "material thickness must be > 0");
    HostGeometry G;
    G.thickness = g->thickness;
    std::vector<BoxBuild> bb;
    std::size_t off = 0;
    for (int i = 0; i < g->nboxes; ++i) {
        std::vector<V2> verts;
        if (g->npoints[i] < 3) throw Error(BTE_ERR_INPUT, "a box needs at least three vertices");
        for (int j = 0; j < g->npoints[i]; ++j, ++off)
            verts.push_back(v2(g->vertices[2 * off], g->vertices[2 * off + 1]));
        bb.push_back(make_box(verts));
        G.Teq.push_back(g->Teq[i]);
        G.Tinit.push_back(g->Tinit ? g->Tinit[i] : g->Teq[i]);
        G.reservoir.push_back(g->reservoir[i] != 0);
        const int mt = g->material ? g->material[i] : 0;
        if (mt < 0) throw Error(BTE_ERR_INPUT, "negative material index");
        G.mat.push_back(mt);
        const int to = g->translate_to ? g->translate_to[i] : -1;
        G.tto.push_back(to);
        G.translation.push_back(to >= 0 && g->translation
                                    ? v2(g->translation[2 * i], g->translation[2 * i + 1])
                                    : v2(0., 0.));
        if (to >= 0) {
            if (to >= g->nboxes || to == i)
                throw Error(BTE_ERR_GEOMETRY, "Error: Bad id for mapping of periodic cells");
            if (!g->translation) throw Error(BTE_ERR_INPUT, "periodic box without a translation vector");
            if (g->reservoir[i]) throw Error(BTE_ERR_GEOMETRY, "a box cannot be periodic and a reservoir");
            G.periodic = true;
        }
    }
    const int nbx = g->nboxes;
    std::vector<std::array<double, 4>> bx(static_cast<std::size_t>(nbx));
    for (int a = 0; a < nbx; ++a) {
        const auto& h = bb[std::size_t(a)].hull;
        double x0 = h[0].x, x1 = x0, y0 = h[0].y, y1 = y0;
        for (auto& p : h) {
            x0 = std::min(x0, p.x); x1 = std::max(x1, p.x);
            y0 = std::min(y0, p.y); y1 = std::max(y1, p.y);
        }
        bx[std::size_t(a)] = {x0, y0, x1, y1};
    }
    for (int a = 0; a < nbx; ++a) {
        for (int b = 0; b < nbx; ++b) {
            if (a == b) continue;
            const auto& A = bx[std::size_t(a)];
            const auto& B = bx[std::size_t(b)];
            if (B[0] > A[2] || A[0] > B[2] || B[1] > A[3] || A[1] > B[3]) continue;  // apart
            auto pinter = touching_points(bb[std::size_t(a)], bb[std::size_t(b)]);
            if (pinter.empty()) continue;
            GBorder cb{};
            const BoxBuild& me = bb[std::size_t(a)];
            if (pinter.size() == 1 || norm(sub(pinter[1], pinter[0])) < 1.0e-6) {
                cb.p1 = cb.p2 = pinter[0];
                cb.np = divs(sub(cb.p1, me.center), norm(sub(cb.p1, me.center)));
                bb[std::size_t(a)].contacts[b] = cb;
                continue;
            }
            cb.p1 = pinter[0];
            cb.p2 = pinter[1];
            cb.nd = sub(cb.p2, cb.p1);
            V2 sc = v2((cb.p1.x + cb.p2.x) / 2., (cb.p1.y + cb.p2.y) / 2.);
            V2 ncsc = sub(sc, me.center);
            V2 npt = v2(cb.nd.y, -cb.nd.x);
            if (dot(npt, ncsc) < 0.) npt = vneg(npt);
            cb.np = divs(npt, norm(npt));
            cb.la = sub(cb.p1, divs(scal(1.0e-6, cb.nd), norm(cb.nd)));
            cb.lb = add(cb.p2, divs(scal(1.0e-6, cb.nd), norm(cb.nd)));
            bb[std::size_t(a)].contacts[b] = cb;
        }
        if (bb[std::size_t(a)].contacts.empty() && nbx > 1)
            throw Error(BTE_ERR_GEOMETRY, "There are unconnected boxes");
    }
    for (int a = 0; a < nbx; ++a) {
        const BoxBuild& me = bb[std::size_t(a)];
        GBox box{};
        box.center = me.center;
        box.area = me.area;
        box.hull_off = int(G.hull.size());
        box.nhull = int(me.hull.size());
        for (auto& p : me.hull) G.hull.push_back(p);
        box.border_off = int(G.borders.size());
        box.nborders = int(me.borders.size());
        for (auto br : me.borders) {
            int cls = -1;
            for (std::size_t c = 0; c < G.normals.size(); ++c)
                if (G.normals[c].x == br.np.x && G.normals[c].y == br.np.y) cls = int(c);
            if (cls < 0) {
                cls = int(G.normals.size());
                G.normals.push_back(br.np);
            }
            br.ncls = cls;
            G.borders.push_back(br);
        }
        box.contact_off = int(G.contacts.size());
        box.ncontacts = int(me.contacts.size());
        for (auto& [id, cb] : me.contacts) {
            GContact c{};
            c.id = id;
            c.np = cb.np;
            G.contacts.push_back(c);
            G.contact_borders.push_back(cb);
            const bool point = cb.p1.x == cb.p2.x && cb.p1.y == cb.p2.y;
            G.contact_seg.push_back(point ? cb.p1 : cb.la);
            G.contact_seg.push_back(point ? cb.p1 : cb.lb);
        }
        box.reservoir = G.reservoir[std::size_t(a)];
        box.tto = G.tto[std::size_t(a)];
        G.boxes.push_back(box);
    }
    // periodic jumps leave the cell walk of the grid path: general kernels
    if (!G.periodic) detect_grid(G, bb);
    return G;
}

void alias_table(const double* w, int n, Alias* out) {
    // Vose's alias method on weights scaled to mean 1.
    double sum = 0.;
    for (int i = 0; i < n; ++i) sum += w[i];
    std::vector<double> p(static_cast<std::size_t>(n));
    std::vector<int> small, large;
    for (int i = 0; i < n; ++i) {
        p[std::size_t(i)] = sum > 0. ? w[i] * n / sum : 0.;
        (p[std::size_t(i)] < 1.0 ? small : large).push_back(i);
        out[i].alt = i;
        out[i].prob = 1.0f;
    }
    while (!small.empty() && !large.empty()) {
        int s = small.back(), l = large.back();
        small.pop_back();
        out[s].prob = float(p[std::size_t(s)]);
        out[s].alt = l;
        p[std::size_t(l)] = (p[std::size_t(l)] + p[std::size_t(s)]) - 1.0;
        if (p[std::size_t(l)] < 1.0) {
            large.pop_back();
            small.push_back(l);
        }
    }
    // leftovers (rounding) keep themselves
    for (int s : small) {
        out[s].prob = 1.0f;
        out[s].alt = s;
    }
    for (int l : large) {
        out[l].prob = 1.0f;
        out[l].alt = l;
    }
    // a zero-weight slot must never be kept
    for (int i = 0; i < n; ++i)
        if (w[i] <= 0. && out[i].alt == i) {
            // point it to any positive slot
            for (int j = 0; j < n; ++j)
                if (w[j] > 0.) {
                    out[i].alt = j;
                    out[i].prob = 0.f;
                    break;
                }
        } else if (w[i] <= 0.) {
            out[i].prob = 0.f;
        }
}

void build_resample(const HostModes& m, double T0, std::vector<double>& cdf,
                    std::vector<Alias>& alias) {
    std::vector<double> pmf(m.n());
    for (std::size_t k = 0; k < m.n(); ++k)
        pmf[k] = m.omega[k] <= 0. ? 0. : bose_einstein_kernel(m.omega[k], T0) * m.w[k];
    cdf = fill_cumulative(pmf);
    alias.resize(m.n());
    alias_table(pmf.data(), int(m.n()), alias.data());
}

std::vector<double> mode_sigmas(const HostModes& m) {
    const std::size_t n = m.n();
    // broadening per mode, Gamma_grid::base_sigma (include/qpoint_grid.hpp:179-181)
    std::vector<double> sig(n);
    for (std::size_t k = 0; k < n; ++k) {
        const double v[3] = {m.vx[k], m.vy[k], m.vz[k]};
        double r[3];
        for (int j = 0; j < 3; ++j)
            r[j] = v[0] * m.dq[0 + 3 * j] + v[1] * m.dq[1 + 3 * j] + v[2] * m.dq[2 + 3 * j];
        sig[k] = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / std::sqrt(12.);
    }
    // outliers clipped at exp(p25 - 1.5 (p75 - p25)) of the log-percentiles
    // (calc_percentiles_log, src/RTA_MC2D.cpp:573-576, :2038-2040)
    std::vector<double> ls(n);
    for (std::size_t k = 0; k < n; ++k)
        ls[k] = sig[k] == 0. ? std::numeric_limits<double>::lowest() : std::log(sig[k]);
    std::sort(ls.begin(), ls.end());
    const double p25 = ls[25 * n / 100], p75 = ls[75 * n / 100];
    const double lbound = std::exp(p25 - 1.5 * (p75 - p25));
    for (auto& s : sig)
        if (s < lbound) s = lbound;
    return sig;
}

LambertTable build_lambert(const HostModes& m, const HostGeometry& g, int nthreads) {
    const std::size_t nq = std::size_t(m.nq), nb = std::size_t(m.nb), n = m.n();
    std::vector<double> sig = mode_sigmas(m);
    const double root_two_pi = std::sqrt(2. * PI);
    // candidate modes (not Gamma, omega not ~0), sorted by omega for windows
    std::vector<int> cand;
    double smax = 0.;
    for (std::size_t k = 0; k < n; ++k)
        if (k / nb >= 1 && !almost_equal(0., m.omega[k])) {
            cand.push_back(int(k));
            smax = std::max(smax, sig[k]);
        }
    std::vector<int> byw = cand;
    std::sort(byw.begin(), byw.end(), [&](int a, int b) {
        return m.omega[std::size_t(a)] < m.omega[std::size_t(b)] || (m.omega[std::size_t(a)] == m.omega[std::size_t(b)] && a < b);
    });
    std::vector<double> wsorted(byw.size());
    for (std::size_t i = 0; i < byw.size(); ++i) wsorted[i] = m.omega[std::size_t(byw[i])];
    // rows of (outgoing mode, pdf) for every incoming mode
    std::vector<std::vector<std::pair<int, double>>> rows(n);
    auto work = [&](std::size_t lo, std::size_t hi) {
        std::vector<std::pair<int, double>> tmp;
        for (std::size_t ci = lo; ci < hi; ++ci) {
            const std::size_t k1 = std::size_t(cand[ci]);
            const double w1 = m.omega[k1];
            // hypot(a, b) <= a + b: a window of half-width nsigma (s1 + smax)
            // (with a margin) contains every accepted partner.
            const double half = nsigma * (sig[k1] + smax) * (1.0 + 1e-9) + 1e-300;
            auto a = std::lower_bound(wsorted.begin(), wsorted.end(), w1 - half);
            auto b = std::upper_bound(wsorted.begin(), wsorted.end(), w1 + half);
            tmp.clear();
            for (auto it = a; it != b; ++it) {
                const std::size_t k2 = std::size_t(byw[std::size_t(it - wsorted.begin())]);
                const double sigma = std::hypot(sig[k1], sig[k2]);
                const double delta = std::fabs(m.omega[k1] - m.omega[k2]);
                if (delta <= nsigma * sigma) {
                    double e = delta;
                    e *= -e;
                    e /= 2 * sigma * sigma;
                    double pdf = std::exp(e);
                    pdf /= sigma * root_two_pi;
                    tmp.push_back({int(k2), pdf});
                }
            }
            std::sort(tmp.begin(), tmp.end());
            rows[k1] = tmp;
        }
    };
    if (nthreads < 1) nthreads = 1;
    {
        std::vector<std::thread> th;
        const std::size_t nc = cand.size();
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back(work, nc * std::size_t(t) / std::size_t(nthreads),
                            nc * std::size_t(t + 1) / std::size_t(nthreads));
        for (auto& t : th) t.join();
    }
    (void)nq;
    // per wall-normal class: filter by outgoing direction and build the
    // cumulative values of bounce() and an alias table
    LambertTable L;
    L.nclass = int(g.normals.size());
    L.row_ptr.assign(std::size_t(L.nclass) * (n + 1), 0);
    std::vector<std::vector<int>> ccol(std::size_t(L.nclass));
    std::vector<std::vector<double>> ccdf(std::size_t(L.nclass));
    std::vector<std::vector<AliasRow>> cal(std::size_t(L.nclass));
    auto cwork = [&](int c) {
        const V2 np = g.normals[std::size_t(c)];
        auto& col = ccol[std::size_t(c)];
        auto& cdf = ccdf[std::size_t(c)];
        auto& al = cal[std::size_t(c)];
        long long* rp = &L.row_ptr[std::size_t(c) * (n + 1)];
        std::vector<std::pair<int, double>> states;
        std::vector<double> wts;
        std::vector<Alias> atmp;
        for (std::size_t k = 0; k < n; ++k) {
            rp[k] = (long long)col.size();
            states.clear();
            double cum = 0.;
            for (auto& [imf, econ] : rows[k]) {
                const double vx = m.vxc[std::size_t(imf)], vy = m.vyc[std::size_t(imf)];
                const double vn = -(np.x * vx + np.y * vy);
                if (vn < 0. || almost_equal(vn, 0.)) continue;
                cum += vn * econ;
                states.push_back({imf, vn * econ});
            }
            // std::map<double, size_t> semantics: a repeated key keeps the
            // later mode
            const std::size_t start = col.size();
            double cum2 = 0;
            wts.clear();
            for (auto& [imf, tran] : states) {
                cum2 += tran / cum;
                if (col.size() > start && cdf.back() == cum2) {
                    col.back() = imf;
                    wts.back() += tran;
                } else {
                    col.push_back(imf);
                    cdf.push_back(cum2);
                    wts.push_back(tran);
                }
            }
            const int len = int(col.size() - start);
            atmp.resize(std::size_t(len));
            if (len > 0) alias_table(wts.data(), len, atmp.data());
            for (int j = 0; j < len; ++j) {
                AliasRow r;
                r.prob = atmp[std::size_t(j)].prob;
                r.keep = col[start + std::size_t(j)];
                r.alt = col[start + std::size_t(atmp[std::size_t(j)].alt)];
                r.pad = 0;
                al.push_back(r);
            }
        }
        rp[n] = (long long)col.size();
    };
    {
        std::vector<std::thread> th;
        for (int c = 0; c < L.nclass; ++c) th.emplace_back(cwork, c);
        for (auto& t : th) t.join();
    }
    long long base = 0;
    for (int c = 0; c < L.nclass; ++c) {
        long long* rp = &L.row_ptr[std::size_t(c) * (n + 1)];
        for (std::size_t k = 0; k <= n; ++k) rp[k] += base;
        base += (long long)ccol[std::size_t(c)].size();
        L.col.insert(L.col.end(), ccol[std::size_t(c)].begin(), ccol[std::size_t(c)].end());
        L.cdf.insert(L.cdf.end(), ccdf[std::size_t(c)].begin(), ccdf[std::size_t(c)].end());
        L.alias.insert(L.alias.end(), cal[std::size_t(c)].begin(), cal[std::size_t(c)].end());
    }
    return L;
}

// pmf (the crystal's n modes) placed at e->off in a row of e->n, zeros
// elsewhere; the row itself without an embedding
static const std::vector<double>& embed_row(const std::vector<double>& pmf, const GenEmbed* e,
                                            std::vector<double>& row) {
    if (!e) return pmf;
    row.assign(e->n, 0.);
    std::copy(pmf.begin(), pmf.end(), row.begin() + std::ptrdiff_t(e->off));
    return row;
}

Generators build_wall_generators(const HostModes& m, const HostGeometry& g, bool required, const GenEmbed* e) {
    Generators R;
    const std::size_t n = m.n();
    const double th = e && e->thickness > 0. ? e->thickness : g.thickness;
    const double vuc = m.V * th / m.c;
    const int nbx = int(g.boxes.size());
    std::vector<double> pmf(n), row;
    for (int s = 0; s < nbx; ++s) {
        if (!g.reservoir[std::size_t(s)]) continue;
        if (e && g.mat[std::size_t(s)] != e->mat) continue;  // another crystal's reservoir
        const GBox& rb = g.boxes[std::size_t(s)];
        for (int ci = 0; ci < rb.ncontacts; ++ci) {
            const int c = g.contacts[std::size_t(rb.contact_off + ci)].id;
            if (g.reservoir[std::size_t(c)] || g.tto[std::size_t(c)] >= 0) continue;
            const GBorder& b = g.contact_borders[std::size_t(rb.contact_off + ci)];
            if (almost_equal(norm(sub(b.p2, b.p1)), 0.)) continue;
            // Isothermal_walls, src/beyondRTA_MC2d.cpp:484-487 (and
            // Init_generator): a reservoir injects into its own material only
            if (e && g.mat[std::size_t(c)] != e->mat)
                throw Error(BTE_ERR_INPUT, "Injection from material A to B is not allowed");
            const double Tw = g.Teq[std::size_t(s)], Te = g.Teq[std::size_t(c)];
            if (almost_equal(Tw, Te)) continue;
            for (std::size_t k = 0; k < n; ++k) {
                const double vn = b.np.x * m.vx[k] + b.np.y * m.vy[k] + 0. * m.vz[k];
                if (vn <= 0. || almost_equal(0., m.omega[k]))
                    pmf[k] = 0.;
                else
                    pmf[k] = vn * m.omega[k] *
                             std::fabs(bose_einstein(m.omega[k], Tw) - bose_einstein(m.omega[k], Te));
            }
            const double cumulsum = 1.0e+12 * hbar * std::accumulate(pmf.begin(), pmf.end(), 0.);
            WallGenerator W{};
            W.res = s;
            W.box = c;
            W.sign = (Tw - Te) >= 0 ? 1 : -1;
            W.p1 = b.p1;
            W.nd = b.nd;
            W.sa = b.p1;
            W.sb = b.p2;
            W.flux = W.sign * (cumulsum / (double(m.nq) * vuc));
            const std::vector<double>& rw = embed_row(pmf, e, row);
            auto cdf = fill_cumulative(rw);
            R.cdf.insert(R.cdf.end(), cdf.begin(), cdf.end());
            std::vector<Alias> al(rw.size());
            alias_table(rw.data(), int(rw.size()), al.data());
            R.alias.insert(R.alias.end(), al.begin(), al.end());
            R.walls.push_back(W);
        }
    }
    if (R.walls.empty()) {
        if (!required) return R;
        throw Error(BTE_ERR_INPUT, "no isothermal wall generator (no reservoir with a different Teq)");
    }
    std::vector<double> ws;
    double total = 0;
    for (auto& W : R.walls) {
        const double Lb = norm(sub(W.sb, W.sa));
        W.energy = std::fabs(W.flux) * Lb * th;
        total += W.energy;
        ws.push_back(W.energy);
    }
    const double wnorm = std::accumulate(ws.begin(), ws.end(), 0.);
    double cum = 0;
    for (double w : ws) {
        cum += w / wnorm;
        R.wall_cum.push_back(cum);
    }
    R.total_energy = total;
    return R;
}

GradGenerators build_gradient_generators(const HostModes& m, const HostGeometry& g, double gx,
                                         double gy) {
    return build_gradient_generators_boxes(m, g, std::vector<V2>(g.boxes.size(), v2(gx, gy)));
}

GradGenerators build_gradient_generators_boxes(const HostModes& m, const HostGeometry& g,
                                               const std::vector<V2>& grad, const GenEmbed* e) {
    GradGenerators R;
    const std::size_t n = m.n();
    const double th = e && e->thickness > 0. ? e->thickness : g.thickness;
    const double vuc = m.V * th / m.c;
    std::vector<double> pmf(n), row;
    std::vector<signed char> sg(n);
    for (std::size_t s = 0; s < g.boxes.size(); ++s) {
        if (g.reservoir[s] || g.tto[s] >= 0) continue;
        if (e && g.mat[s] != e->mat) continue;  // another crystal's box
        const double gx = grad[s].x, gy = grad[s].y;
        // a box without a gradient has no source (source_term_gradient,
        // src/beyondRTA_MC2d.cpp:626-628)
        if (almost_equal(std::hypot(gx, gy), 0.)) continue;
        const double T = g.Teq[s];
        for (std::size_t k = 0; k < n; ++k) {
            const double vgradT = -(gx * m.vx[k] + gy * m.vy[k] + 0. * m.vz[k]);
            if (m.omega[k] == 0.) {
                pmf[k] = 0.;
                sg[k] = 1;
            } else {
                pmf[k] = std::fabs(vgradT * bose_einstein_kernel(m.omega[k], T));
                sg[k] = vgradT >= 0 ? 1 : -1;
            }
        }
        const double cumulsum = kB * std::accumulate(pmf.begin(), pmf.end(), 0.);
        const double vol = g.boxes[s].area * th / vuc;
        R.box.push_back(int(s));
        R.energy.push_back(vol * cumulsum / double(m.nq));
        const std::vector<double>& rw = embed_row(pmf, e, row);
        auto cdf = fill_cumulative(rw);
        R.cdf.insert(R.cdf.end(), cdf.begin(), cdf.end());
        std::vector<Alias> al(rw.size());
        alias_table(rw.data(), int(rw.size()), al.data());
        R.alias.insert(R.alias.end(), al.begin(), al.end());
        if (e) {  // modes outside the crystal are never drawn
            std::vector<signed char> srow(e->n, 1);
            std::copy(sg.begin(), sg.end(), srow.begin() + std::ptrdiff_t(e->off));
            R.sign.insert(R.sign.end(), srow.begin(), srow.end());
        } else {
            R.sign.insert(R.sign.end(), sg.begin(), sg.end());
        }
    }
    const double wnorm = std::accumulate(R.energy.begin(), R.energy.end(), 0.);
    double cum = 0;
    for (double w : R.energy) {
        cum += w / wnorm;
        R.cum.push_back(cum);
    }
    R.total_energy = wnorm;
    return R;
}

GradGenerators merge_gradient_generators(const std::vector<GradGenerators>& G) {
    // (box, crystal, index) in ascending box order
    std::vector<std::tuple<int, std::size_t, std::size_t>> order;
    for (std::size_t k = 0; k < G.size(); ++k)
        for (std::size_t i = 0; i < G[k].box.size(); ++i) order.emplace_back(G[k].box[i], k, i);
    std::sort(order.begin(), order.end());
    GradGenerators R;
    for (auto& [b, k, i] : order) {
        const GradGenerators& S = G[k];
        const std::size_t n = S.cdf.size() / S.box.size();
        R.box.push_back(b);
        R.energy.push_back(S.energy[i]);
        R.cdf.insert(R.cdf.end(), S.cdf.begin() + std::ptrdiff_t(i * n), S.cdf.begin() + std::ptrdiff_t((i + 1) * n));
        R.alias.insert(R.alias.end(), S.alias.begin() + std::ptrdiff_t(i * n),
                       S.alias.begin() + std::ptrdiff_t((i + 1) * n));
        R.sign.insert(R.sign.end(), S.sign.begin() + std::ptrdiff_t(i * n), S.sign.begin() + std::ptrdiff_t((i + 1) * n));
    }
    const double wnorm = std::accumulate(R.energy.begin(), R.energy.end(), 0.);
    double cum = 0;
    for (double w : R.energy) {
        cum += w / wnorm;
        R.cum.push_back(cum);
    }
    R.total_energy = wnorm;
    return R;
}

std::vector<V2> calculate_gradientT(const HostGeometry& g) {
    std::vector<V2> out(g.boxes.size(), v2(0., 0.));
    std::vector<double> hx, hy, d;
    for (std::size_t s = 0; s < g.boxes.size(); ++s) {
        if (g.reservoir[s] || g.tto[s] >= 0) continue;
        const GBox& B = g.boxes[s];
        // rows h_i = c_i - c_0, d_i = T_i - T_0 over the neighbours that are
        // neither reservoirs nor periodic (contacts are unique per neighbour)
        hx.clear();
        hy.clear();
        d.clear();
        for (int i = 0; i < B.ncontacts; ++i) {
            const int o = g.contacts[std::size_t(B.contact_off + i)].id;
            if (g.reservoir[std::size_t(o)] || g.tto[std::size_t(o)] >= 0) continue;
            hx.push_back(g.boxes[std::size_t(o)].center.x - B.center.x);
            hy.push_back(g.boxes[std::size_t(o)].center.y - B.center.y);
            d.push_back(g.Teq[std::size_t(o)] - g.Teq[s]);
        }
        out[s] = min_norm_lstsq2(hx, hy, d);
    }
    return out;
}

V2 min_norm_lstsq2(const std::vector<double>& hx, const std::vector<double>& hy, const std::vector<double>& d) {
    // Minimum-norm least squares of [hx hy] g = d, as a complete orthogonal
    // decomposition does it: QR with column pivoting (the column of larger
    // norm first, Gram-Schmidt for the second), the rank from |R_ii| above
    // diag_size * epsilon * |R_11|, and for rank 1 the minimum-norm
    // solution along the first row of R.
    const std::size_t m = hx.size();
    if (m == 0) return v2(0., 0.);
    double n0 = 0., n1 = 0.;
    for (std::size_t i = 0; i < m; ++i) {
        n0 += hx[i] * hx[i];
        n1 += hy[i] * hy[i];
    }
    const bool swap = n1 > n0;
    const std::vector<double>& c1 = swap ? hy : hx;
    const std::vector<double>& c2 = swap ? hx : hy;
    const double r11 = std::sqrt(swap ? n1 : n0);
    if (!(r11 > 0.)) return v2(0., 0.);
    std::vector<double> q1(m), q2(m);
    double r12 = 0., b1 = 0.;
    for (std::size_t i = 0; i < m; ++i) {
        q1[i] = c1[i] / r11;
        r12 += q1[i] * c2[i];
        b1 += q1[i] * d[i];
    }
    double r22s = 0.;
    for (std::size_t i = 0; i < m; ++i) {
        q2[i] = c2[i] - r12 * q1[i];
        r22s += q2[i] * q2[i];
    }
    const double r22 = std::sqrt(r22s);
    const double diag = double(std::min<std::size_t>(m, 2));
    double x1, x2;
    if (m >= 2 && r22 > diag * std::numeric_limits<double>::epsilon() * r11) {
        double b2 = 0.;
        for (std::size_t i = 0; i < m; ++i) b2 += (q2[i] / r22) * d[i];
        x2 = b2 / r22;
        x1 = (b1 - r12 * x2) / r11;
    } else {
        const double t = b1 / (r11 * r11 + r12 * r12);
        x1 = r11 * t;
        x2 = r12 * t;
    }
    return swap ? v2(x2, x1) : v2(x1, x2);
}

TranslationFast build_translation_fast(const HostGeometry& g, double margin) {
    TranslationFast R;
    const std::size_t nbx = g.boxes.size();
    R.rng.assign(nbx, IntPair{0, 0});
    R.u.assign(nbx, v2(0., 0.));
    for (std::size_t P = 0; P < nbx; ++P) {
        const int tb = g.tto[P];
        if (tb < 0) continue;
        const V2 t = g.translation[P];
        const double tn = std::hypot(t.x, t.y);
        if (!(tn > 0.)) continue;
        const V2 u = v2(-t.y / tn, t.x / tn);
        // every candidate contact's interval of r.u, its ends widened by
        // the margin (a point contact is an interval of zero length)
        struct Span {
            double lo, hi;
            int ci;
        };
        std::vector<Span> sp;
        const GBox& TB = g.boxes[std::size_t(tb)];
        for (int i = 0; i < TB.ncontacts; ++i) {
            const int ci = TB.contact_off + i;
            const int id = g.contacts[std::size_t(ci)].id;
            if (id == tb || g.tto[std::size_t(id)] >= 0 || g.reservoir[std::size_t(id)]) continue;
            const V2 a = g.contact_seg[2 * std::size_t(ci)], b = g.contact_seg[2 * std::size_t(ci) + 1];
            const double ua = u.x * a.x + u.y * a.y, ub = u.x * b.x + u.y * b.y;
            sp.push_back(Span{std::min(ua, ub), std::max(ua, ub), ci});
        }
        // the parts of each interval farther than the margin from every
        // candidate's ends and covered by no other candidate
        std::vector<double> cut;
        for (auto& s : sp) {
            cut.push_back(s.lo - margin);
            cut.push_back(s.lo + margin);
            cut.push_back(s.hi - margin);
            cut.push_back(s.hi + margin);
        }
        std::sort(cut.begin(), cut.end());
        R.rng[P].x = int(R.iv.size());
        R.u[P] = u;
        for (std::size_t k = 0; k + 1 < cut.size(); ++k) {
            const double lo = cut[k], hi = cut[k + 1];
            if (!(hi > lo)) continue;
            const double mid = 0.5 * (lo + hi);
            int owner = -1, cover = 0;
            bool near_end = false;
            for (auto& s : sp) {
                if (std::fabs(mid - s.lo) < margin || std::fabs(mid - s.hi) < margin) near_end = true;
                if (mid > s.lo && mid < s.hi) {
                    ++cover;
                    owner = s.ci;
                }
            }
            if (near_end || cover != 1) continue;
            if (!R.iv.empty() && int(R.iv.size()) > R.rng[P].x && R.iv.back().ci == owner &&
                R.iv.back().hi == lo) {
                R.iv.back().hi = hi;  // the same contact on both sides of a cut
                continue;
            }
            R.iv.push_back(TransFast{lo, hi, owner, 0});
        }
        R.rng[P].y = int(R.iv.size()) - R.rng[P].x;
    }
    return R;
}

Generators build_initial_generators(const HostModes& m, const HostGeometry& g, const GenEmbed* e) {
    Generators R;
    const std::size_t n = m.n();
    const double th = e && e->thickness > 0. ? e->thickness : g.thickness;
    const double vuc = m.V * th / m.c;
    std::vector<double> pmf(n), row;
    for (std::size_t s = 0; s < g.boxes.size(); ++s) {
        if (g.reservoir[s] || g.tto[s] >= 0) continue;
        if (e && g.mat[s] != e->mat) continue;
        const double Tr = g.Tinit[s], Te = g.Teq[s];
        if (almost_equal(Te, Tr)) continue;
        if (Tr <= 0 || Te <= 0) throw Error(BTE_ERR_VALUE, "Invalid temperature value");
        for (std::size_t k = 0; k < n; ++k) {
            const double om = m.omega[k];
            pmf[k] = almost_equal(om, 0.)
                         ? 0.
                         : om * std::fabs(bose_einstein(om, Tr) - bose_einstein(om, Te));
        }
        const double cumulsum = 1.0e+12 * hbar * std::accumulate(pmf.begin(), pmf.end(), 0.);
        const double vol = g.boxes[s].area * th / vuc;
        R.init_box.push_back(int(s));
        R.init_sign.push_back((Tr - Te) >= 0 ? 1 : -1);
        R.init_energy.push_back(vol * cumulsum / double(m.nq));
        const std::vector<double>& rw = embed_row(pmf, e, row);
        auto cdf = fill_cumulative(rw);
        R.cdf.insert(R.cdf.end(), cdf.begin(), cdf.end());
        std::vector<Alias> al(rw.size());
        alias_table(rw.data(), int(rw.size()), al.data());
        R.alias.insert(R.alias.end(), al.begin(), al.end());
    }
    if (R.init_box.empty() && !e) throw Error(BTE_ERR_INPUT, "no box with Tinit different from Teq");
    double total = 0;
    for (double x : R.init_energy) total += x;
    R.total_energy = total;
    return R;
}

double initial_counts(Generators& R, int64_t nparticles, uint64_t seed) {
    if (nparticles < 1) throw Error(BTE_ERR_INPUT, "nparticles must be >= 1");
    const double Eeff = R.total_energy / double(nparticles);
    R.init_first.clear();
    // Ntogenerate: floor(E_box / Eeff) plus one with probability equal to the
    // fraction (src/sampling.cpp:310-326), drawn from pcg64(seed, 2^63 + box)
    long long first = 0;
    for (std::size_t b = 0; b < R.init_box.size(); ++b) {
        R.init_first.push_back(first);
        const double gen = R.init_energy[b] / Eeff;
        long long np = (long long)gen;
        const double rem = gen - std::floor(gen);
        Pcg64 r;
        r.seed(seed, (uint64_t(1) << 63) + uint64_t(R.init_box[b]));
        if (canonical_from(r.next()) <= rem) np++;
        first += np;
    }
    R.init_first.push_back(first);
    return Eeff;
}

std::vector<int> build_mirror(const HostModes& m, const HostGeometry& g) {
    const std::size_t n = m.n();
    const int nc = int(g.normals.size());
    std::vector<int> mir(std::size_t(nc) * n, -1);
    const int n1 = m.grid[0], n2 = m.grid[1];
    if (n1 < 1 || n2 < 1 || std::size_t(n1) * std::size_t(n2) != std::size_t(m.nq)) return mir;
    for (int c = 0; c < nc; ++c) {
        const V2 np = g.normals[std::size_t(c)];
        const bool ny = (np.x == 0. && std::fabs(np.y) == 1.);
        const bool nx = (np.y == 0. && std::fabs(np.x) == 1.);
        if (!nx && !ny) continue;
        for (std::size_t k = 0; k < n; ++k) {
            const int iq = int(k / std::size_t(m.nb)), ib = int(k % std::size_t(m.nb));
            int i = iq / n2, j = iq % n2;
            if (ny) j = (n2 - j) % n2;
            if (nx) i = (n1 - i) % n1;
            const std::size_t k2 = std::size_t(i * n2 + j) * std::size_t(m.nb) + std::size_t(ib);
            // the image must carry the reflected velocity
            const double vn_in = np.x * m.vxc[k] + np.y * m.vyc[k];
            const double vn_out = np.x * m.vxc[k2] + np.y * m.vyc[k2];
            const double vt_in = nx ? m.vyc[k] : m.vxc[k];
            const double vt_out = nx ? m.vyc[k2] : m.vxc[k2];
            if (vn_out == -vn_in && vt_out == vt_in && m.omega[k2] > 0.)
                mir[std::size_t(c) * n + k] = int(k2);
        }
    }
    return mir;
}


HostModes concat_modes(const std::vector<HostModes>& crys, std::vector<std::size_t>& off) {
    HostModes all;
    off.clear();
    std::size_t n = 0;
    for (const HostModes& m : crys) {
        off.push_back(n);
        n += m.n();
        using Field = std::vector<double> HostModes::*;
        for (Field pr : {&HostModes::omega, &HostModes::vx, &HostModes::vy, &HostModes::vz, &HostModes::w,
                         &HostModes::vxc, &HostModes::vyc})
            (all.*pr).insert((all.*pr).end(), (m.*pr).begin(), (m.*pr).end());
    }
    // one "q point" per mode: the concatenation has no q grid (no mirror
    // images, no spectral q mesh); the cell of crystal 0 stands in where a
    // per-table constant is read, which the crystal paths never do
    all.nq = int(n);
    all.nb = 1;
    if (!crys.empty()) {
        all.V = crys[0].V;
        all.c = crys[0].c;
    }
    return all;
}

LambertTable merge_lambert(const std::vector<LambertTable>& L, const std::vector<HostModes>& crys,
                           const std::vector<std::size_t>& off) {
    LambertTable R;
    if (L.empty()) return R;
    R.nclass = L[0].nclass;
    std::size_t n = 0;
    for (const HostModes& m : crys) n += m.n();
    R.row_ptr.assign(std::size_t(R.nclass) * (n + 1), 0);
    for (int c = 0; c < R.nclass; ++c) {
        long long* rp = &R.row_ptr[std::size_t(c) * (n + 1)];
        for (std::size_t k = 0; k < crys.size(); ++k) {
            const std::size_t nk = crys[k].n(), o = off[k];
            const long long* lp = &L[k].row_ptr[std::size_t(c) * (nk + 1)];
            for (std::size_t j = 0; j < nk; ++j) {
                rp[o + j] = (long long)R.col.size();
                for (long long e = lp[j]; e < lp[j + 1]; ++e) {
                    R.col.push_back(L[k].col[std::size_t(e)] + int(o));
                    R.cdf.push_back(L[k].cdf[std::size_t(e)]);
                    AliasRow a = L[k].alias[std::size_t(e)];
                    a.keep += int(o);
                    a.alt += int(o);
                    R.alias.push_back(a);
                }
            }
        }
        rp[n] = (long long)R.col.size();
    }
    return R;
}

std::vector<int> merge_mirror(const std::vector<std::vector<int>>& mir, const std::vector<HostModes>& crys,
                              const std::vector<std::size_t>& off, int nclass) {
    std::size_t n = 0;
    for (const HostModes& m : crys) n += m.n();
    std::vector<int> R(std::size_t(nclass) * n, -1);
    for (std::size_t k = 0; k < crys.size(); ++k) {
        const std::size_t nk = crys[k].n();
        for (int c = 0; c < nclass; ++c)
            for (std::size_t j = 0; j < nk; ++j) {
                const int v = mir[k][std::size_t(c) * nk + j];
                R[std::size_t(c) * n + off[k] + j] = v >= 0 ? v + int(off[k]) : -1;
            }
    }
    return R;
}

Generators merge_generators(std::vector<Generators>& G, bool walls, bool required) {
    Generators R;
    for (Generators& g : G) {
        if (walls) R.walls.insert(R.walls.end(), g.walls.begin(), g.walls.end());
        R.init_box.insert(R.init_box.end(), g.init_box.begin(), g.init_box.end());
        R.init_sign.insert(R.init_sign.end(), g.init_sign.begin(), g.init_sign.end());
        R.init_energy.insert(R.init_energy.end(), g.init_energy.begin(), g.init_energy.end());
        R.cdf.insert(R.cdf.end(), g.cdf.begin(), g.cdf.end());
        R.alias.insert(R.alias.end(), g.alias.begin(), g.alias.end());
        R.total_energy += g.total_energy;
    }
    if (walls) {
        if (R.walls.empty() && required)
            throw Error(BTE_ERR_INPUT, "no isothermal wall generator (no reservoir with a different Teq)");
        double total = 0.;
        for (auto& W : R.walls) total += W.energy;
        double cum = 0.;
        for (auto& W : R.walls) {
            cum += W.energy / total;
            R.wall_cum.push_back(cum);
        }
        R.total_energy = total;
    } else if (R.init_box.empty()) {
        throw Error(BTE_ERR_INPUT, "no box with Tinit different from Teq");
    } else {
        // the initial deviation's boxes in ascending box order, as one
        // crystal's are, and their energy summed in that order
        const std::size_t nb = R.init_box.size(), n = R.cdf.size() / nb;
        std::vector<std::size_t> ord(nb);
        std::iota(ord.begin(), ord.end(), std::size_t(0));
        std::stable_sort(ord.begin(), ord.end(),
                         [&](std::size_t a, std::size_t b) { return R.init_box[a] < R.init_box[b]; });
        Generators S;
        S.total_energy = 0.;
        for (std::size_t i : ord) {
            S.init_box.push_back(R.init_box[i]);
            S.init_sign.push_back(R.init_sign[i]);
            S.init_energy.push_back(R.init_energy[i]);
            S.cdf.insert(S.cdf.end(), R.cdf.begin() + std::ptrdiff_t(i * n), R.cdf.begin() + std::ptrdiff_t((i + 1) * n));
            S.alias.insert(S.alias.end(), R.alias.begin() + std::ptrdiff_t(i * n),
                           R.alias.begin() + std::ptrdiff_t((i + 1) * n));
            S.total_energy += R.init_energy[i];
        }
        return S;
    }
    return R;
}

DmmTable build_dmm_table(const HostModes& A, std::size_t offA, const HostModes& B, std::size_t offB,
                         std::size_t n_total, V2 nrm, double VA, double VB, double Tref, int nthreads) {
    const double nn = std::sqrt(nrm.x * nrm.x + nrm.y * nrm.y);
    if (!(nn > 0.)) throw Error(BTE_ERR_VALUE, "invalid normal vector");
    const double ux = nrm.x / nn, uy = nrm.y / nn, uz = 0. / nn;
    constexpr double scalebroad = 0.1;
    // every mode of A then of B, q-major: side, index in its crystal, v.n,
    // C = C(omega, Tref) / (kB nq V), and its Gaussian_for_DOS
    // (include/dos.hpp:49-63): mu, sigma, the window (lbound, ubound)
    struct M {
        int side;
        std::size_t j;
        double vn, C, mu, sigma, lo, hi;
        bool has;
    };
    std::vector<M> all;
    const HostModes* cr[2] = {&A, &B};
    const double V[2] = {VA, VB};
    for (int s = 0; s < 2; ++s) {
        const HostModes& m = *cr[s];
        for (std::size_t k = 0; k < m.n(); ++k) {
            M x;
            x.side = s;
            x.j = k;
            x.vn = ux * m.vx[k] + uy * m.vy[k] + uz * m.vz[k];
            x.C = bose_einstein_kernel(m.omega[k], Tref) / (kB * double(m.nq) * V[s]);
            double r[3];
            for (int a = 0; a < 3; ++a)
                r[a] = m.vx[k] * m.dq[0 + 3 * a] + m.vy[k] * m.dq[1 + 3 * a] + m.vz[k] * m.dq[2 + 3 * a];
            x.mu = m.omega[k];
            x.sigma = scalebroad * (std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / std::sqrt(12.));
            x.lo = x.mu - nsigma * x.sigma < 0. ? 0. : x.mu - nsigma * x.sigma;
            x.hi = x.mu + nsigma * x.sigma;
            x.has = !(x.mu == 0. || x.sigma == 0.);
            all.push_back(x);
        }
    }
    const double root_two_pi = std::sqrt(2. * PI);
    auto pdf = [&](const M& c, double t) {
        if (!c.has) return 0.;
        double e = t - c.mu;
        e *= -e;
        e /= 2 * c.sigma * c.sigma;
        double v = std::exp(e);
        v /= c.sigma * root_two_pi;
        return v;
    };
    auto emission = [](const M& c) { return (c.side == 0 && c.vn < 0.) || (c.side == 1 && c.vn > 0.); };
    // the candidates by mu, for windows: a candidate is compatible with
    // target t when lo < t < hi, and hi - lo <= 2 nsigma sigma_max
    std::vector<int> byw;
    double smax = 0.;
    for (std::size_t i = 0; i < all.size(); ++i)
        if (emission(all[i])) {
            byw.push_back(int(i));
            smax = std::max(smax, all[i].sigma);
        }
    std::sort(byw.begin(), byw.end(), [&](int a, int b) {
        return all[std::size_t(a)].mu < all[std::size_t(b)].mu ||
               (all[std::size_t(a)].mu == all[std::size_t(b)].mu && a < b);
    });
    std::vector<double> mus(byw.size());
    for (std::size_t i = 0; i < byw.size(); ++i) mus[i] = all[std::size_t(byw[i])].mu;
    // side A's incident lists (v.n > 0), entries in the order of `all`
    const std::size_t nA = A.n();
    std::vector<std::vector<int>> lst(nA);
    std::vector<std::vector<double>> raw(nA);
    auto work = [&](std::size_t lo, std::size_t hi) {
        std::vector<int> cand;
        for (std::size_t j = lo; j < hi; ++j) {
            const M& mi = all[j];
            if (!(mi.vn > 0.)) continue;
            const double t = mi.mu;
            const double half = nsigma * smax * (1. + 1e-9) + 1e-300;
            auto a = std::lower_bound(mus.begin(), mus.end(), t - half);
            auto b = std::upper_bound(mus.begin(), mus.end(), t + half);
            cand.clear();
            for (auto it = a; it != b; ++it) {
                const int ci = byw[std::size_t(it - mus.begin())];
                const M& c = all[std::size_t(ci)];
                if (t > c.lo && t < c.hi) cand.push_back(ci);
            }
            std::sort(cand.begin(), cand.end());  // the order of `all`
            for (int ci : cand) {
                const M& c = all[std::size_t(ci)];
                lst[j].push_back(ci);
                raw[j].push_back(c.C * std::fabs(c.vn) * 1.0 * pdf(c, t));
            }
        }
    };
    if (nthreads < 1) nthreads = 1;
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back(work, nA * std::size_t(t) / std::size_t(nthreads),
                            nA * std::size_t(t + 1) / std::size_t(nthreads));
        for (auto& t : th) t.join();
    }
    double total = 0.;
    for (std::size_t j = 0; j < nA; ++j)
        for (double r : raw[j]) total += r;
    // incident modes without a transition: the reflection of the closest
    // frequency, recorded with the side of the last mode scanned (always B,
    // as the reference's side_out variable ends the scan)
    const int fix_side = all.back().side;
    for (std::size_t j = 0; j < nA; ++j) {
        const M& mi = all[j];
        if (!(mi.vn > 0.) || !lst[j].empty()) continue;
        long long best = -1;
        double dmin = 1e300;
        for (std::size_t ci = 0; ci < all.size(); ++ci) {
            const M& c = all[ci];
            if (c.side != 0 || !emission(c)) continue;
            const double d = std::fabs(c.mu - mi.mu);
            if (d < dmin) {
                best = (long long)ci;
                dmin = d;
            }
        }
        if (best < 0) throw Error(BTE_ERR_VALUE, "no matching mode was found for some incident mode");
        const M& c = all[std::size_t(best)];
        if (c.j >= (fix_side == 0 ? A.n() : B.n()))
            throw Error(BTE_ERR_VALUE, "a reflection index beyond the other material's table");
        lst[j].push_back(-1 - int(best));  // marks the side quirk
        const double r = c.C * std::fabs(c.vn) * 1.0;
        raw[j].push_back(r);
        total += r;
    }
    DmmTable T;
    T.row.assign(n_total + 1, 0);
    double pc = 0.;
    for (std::size_t K = 0; K < n_total; ++K) {
        T.row[K] = (long long)T.out.size();
        if (K < offA || K >= offA + nA) continue;
        const std::size_t j = K - offA;
        for (std::size_t e = 0; e < lst[j].size(); ++e) {
            const int ci = lst[j][e];
            const M& c = all[std::size_t(ci >= 0 ? ci : -1 - ci)];
            const int side = ci >= 0 ? c.side : fix_side;
            pc += raw[j][e] / total;
            T.out.push_back(int((side == 0 ? offA : offB) + c.j));
            T.side.push_back(side);
            T.cum.push_back(pc);
        }
    }
    T.row[n_total] = (long long)T.out.size();
    return T;
}

}  // namespace bte
