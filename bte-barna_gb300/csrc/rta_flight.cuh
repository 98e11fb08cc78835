// rta_flight.cuh - the RTA particle life on the device, for general convex
// boxes.  One thread carries one particle from its generation to absorption
// or maxtime.  The logic follows, step for step:
//   per-particle loop     src/RTA_MC2D.cpp:2262-2316
//   evolparticle          src/RTA_MC2D.cpp:990-1386 (transient, one material)
//   get_inter_side        src/geometry_2d.cpp:160-293
//   in_corner3            src/geometry_2d.cpp:388-406
//   correct_corner_problem include/geometry_2d.hpp:524-561
//   translate             include/geometry_2d.hpp:366-493 (periodic boxes)
//   Init_generator        src/RTA_MC2D.cpp:421-511 (walls)
//   init_particles        src/beyondRTA_MC2d.cpp:211-269 (initial deviation)
// The policy P supplies the random draws, the samplers and the tally, so the
// same code serves the bit-exact replay mode and the production mode.
#pragma once

#include "bte_device.cuh"

namespace bte {

constexpr int MAXB = 16;        // borders per box
constexpr int MAXC = 32;        // candidate boxes at one crossing
constexpr int FLIGHT_CAP = 1 << 20;  // evolparticle calls per free flight
constexpr int NUDGE_CAP = 64;   // consecutive geometry nudges
constexpr long long EVENT_CAP = 1ll << 26;  // free flights per particle

// Error codes written to the device error word (bte_status values).
constexpr int E_VALUE = 2, E_GEOM = 3, E_LIMIT = 4, E_CHECK = 7;

struct WallGenDev {
    V2 p1, nd, sa, sb;
    int box, sign;
};

// One entry of a diffuse mismatch table: cumulative probability, global
// mode out, side out (0: back into the incident box, 1: into the other).
struct DmmEnt {
    double cum;
    int out, side;
};

struct DevTables {
    // modes
    int n, nb;
    const double* vxc;
    const double* vyc;
    const double* w;
    const double* tau;
    const int* box_mat;     // [box] material (null: one material)
    const double* resample_cdf;
    const float* resample_prob;
    const int* resample_alt;
    // geometry
    int nboxes;
    const GBox* boxes;
    const V2* hull;
    const GBorder* borders;
    const GContact* contacts;
    const V2* cseg;         // [contact][2]: lengthened contact segment (sbl)
    const V2* translation;  // [box]: <Translate_to> vector of periodic boxes
    // translations that need no search (build_translation_fast): per
    // periodic box, the unit normal u of its translation and the intervals
    // of r0.u in which the translated segment meets exactly one candidate
    // contact; null: none
    const TransFast* tfast;
    const int2* tfast_rng;  // [box]: first interval, count
    const V2* tfast_u;      // [box]
    int nclass;
    // Lambert rows
    const long long* row_ptr;
    const int* lcol;
    const double* lcdf;
    const int4* lalias;   // {prob bits, keep, alt, pad}
    const int* mirror;    // [nclass][n] or null
    // time grid
    int ntime;
    const double* timegrid;   // ntime points, then the ntime - 1 bin widths
    double maxtime;
    double inv_dt;        // 1 / bin width (production)
    // generators
    int source, ngen;
    const double* gen_cdf;
    const float* gen_prob;
    const int* gen_alt;
    const WallGenDev* walls;
    const double* wall_cum;
    const long long* init_first;
    const int* init_box;
    const int* init_sign;
    // run
    unsigned long long seed;
    int ballistic;
    double specularity;
    long long flight_cap;  // free flights per particle (EVENT_CAP unless the run sets one)
    int checks;            // BTE_FLAG_CHECKS: the checked grid-kernel variant
    long long pbegin, pend;
    int nbins;
    // spectral decomposition: box -> location (-1: none, null: off) and the
    // per-mode time tally [location][bin][mode] (FP64; replay: 2 x u64)
    const int* spec_loc;
    double* spec;
    unsigned long long* spec_ex;
    unsigned long long* spec_cnt;  // steady state: signed segments per [loc][mode]
    // replica groups of the grid kernel: particle p tallies into group
    // p mod ngroups, group_stride doubles after the previous group (ngroups
    // <= 1: one tally)
    int ngroups;
    long long group_stride;
    // crystals joined by mismatch interfaces (null: one crystal): per
    // contact the interface table of (its box's crystal, the neighbour's,
    // the contact normal), -1 within a crystal; the tables' rows
    // [table][n + 1] into their entries; each crystal's first global mode
    // (ncrys + 1 values)
    const int* contact_dmm;
    const long long* dmm_row;
    const DmmEnt* dmm_ent;
    const int* crys_off;
};

// One thread's counts over one launch (32 bits: a thread would need over
// 4e9 flight events in a launch to wrap one), warp-reduced into the
// launch's 64-bit counters at its end.
struct Counters {
    unsigned events, wall_hits, crossings, absorbed, specular, nudges, quirks, tallies,
        translations, scattered, lost, ifc_hits, ifc_trans;
};

// How a steady-state flight ends (periodic / gradient branch).
constexpr int FATE_LOST = 0;      // left_time rounded to 0 at a crossing: dropped
constexpr int FATE_SCATTER = 1;   // scattered inside a box: counted in phi
constexpr int FATE_BOUNCE = 2;    // reflected at a void wall: carried to the next generation
constexpr int FATE_ABSORBED = 3;  // reached a reservoir

struct Particle {
    V2 pos;
    int mode;
    int sign;
    double t;
    int box;
    int mo;   // material offset into the per-material tables (material * n)
};

// Offset of box b's material in the [material][mode] tables.
__device__ __forceinline__ int mat_off(const DevTables& T, int b) {
    return T.box_mat ? __ldg(T.box_mat + b) * T.n : 0;
}

// std::lower_bound over a sorted double array: first index with a[i] >= u.
__device__ __forceinline__ int lower_bound_d(const double* a, int n, double u) {
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int step = cnt >> 1;
        const int it = lo + step;
        if (a[it] < u) {
            lo = it + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    return lo;
}

__device__ __forceinline__ bool box_inside(const DevTables& T, int b, V2 p) {
    const GBox& B = T.boxes[b];
    return inside_hull(T.hull + B.hull_off, B.nhull, p);
}

struct HitD {
    double time;
    V2 rf;
    int nb;
    int bids[MAXB];
};

// get_inter_side: returns false on the reference's geometry_error.
static __device__ __noinline__ bool get_inter_side(const DevTables& T, int box, V2 r0, V2 v, double dt, HitD& h) {
    const GBox& B = T.boxes[box];
    const V2 pf = v2(r0.x + dt * v.x, r0.y + dt * v.y);
    double time = 1.0e+7;
    V2 rf = v2(0., 0.);
    h.nb = 0;
    bool already_there = true;
    for (int id = 0; id < B.nborders; ++id) {
        const GBorder& b = T.borders[B.border_off + id];
        V2 rin;
        if (seg_intersect(r0, pf, b.la, b.lb, rin) && !on_segment(r0, b.la, b.lb)) {
            if (dot(b.np, v) > 0.) {
                const double tx = (__builtin_fabs(v.x) < 1.0e-6) ? -1 : (rin.x - r0.x) / v.x;
                const double ty = (__builtin_fabs(v.y) < 1.0e-6) ? -1 : (rin.y - r0.y) / v.y;
                const double newtime = tx > ty ? tx : ty;
                if (newtime == time && h.nb < MAXB) h.bids[h.nb++] = id;
                if (newtime < time) {
                    h.nb = 0;
                    rf = rin;
                    time = newtime;
                    already_there = false;
                    h.bids[h.nb++] = id;
                }
            }
        }
    }
    if (already_there) {
        const V2 p0p = v2(r0.x - 1.0e-6 * v.x, r0.y - 1.0e-6 * v.y);
        for (int id = 0; id < B.nborders; ++id) {
            const GBorder& b = T.borders[B.border_off + id];
            V2 rin;
            if (seg_intersect(p0p, pf, b.la, b.lb, rin)) {
                if (dot(b.np, v) > 0.) {
                    const double tx = (__builtin_fabs(v.x) < 1.0e-6) ? -1.0e+8 : (rin.x - r0.x) / v.x;
                    const double ty = (__builtin_fabs(v.y) < 1.0e-6) ? -1.0e+8 : (rin.y - r0.y) / v.y;
                    const double newtime = tx > ty ? tx : ty;
                    if (newtime == time && h.nb < MAXB) h.bids[h.nb++] = id;
                    if (__builtin_fabs(newtime) < time) {
                        h.nb = 0;
                        rf = rin;
                        time = newtime;
                        h.bids[h.nb++] = id;
                    }
                }
            }
        }
        if (time > 1.0e+6) return false;
    }
    if (almost_equal(time, 0.)) time = 0.;
    if (time < 0.) return false;
    h.time = time;
    h.rf = rf;
    return true;
}

// Contact normal of `box` towards neighbour `test` (contacts sorted by id).
__device__ __forceinline__ int contact_index(const DevTables& T, int box, int test) {
    const GBox& B = T.boxes[box];
    for (int i = 0; i < B.ncontacts; ++i)
        if (T.contacts[B.contact_off + i].id == test) return B.contact_off + i;
    return -1;
}

// The interface table between `box` and its neighbour `inew`, or -1 (one
// crystal, the same crystal, or no contact).
__device__ __forceinline__ int dmm_table(const DevTables& T, int box, int inew) {
    if (!T.contact_dmm) return -1;
    const int ci = contact_index(T, box, inew);
    return ci >= 0 ? T.contact_dmm[ci] : -1;
}

// Mode k of the incident crystal `ma` read in crystal `mb` by its index
// within its crystal (the reference keeps (q, alpha) across an interface
// without a transition), or -1 beyond mb's table.
__device__ __forceinline__ int dmm_same_index(const DevTables& T, int k, int ma, int mb) {
    const int local = k - T.crys_off[ma];
    return local < T.crys_off[mb + 1] - T.crys_off[mb] ? T.crys_off[mb] + local : -1;
}

// change_material_diffuse (src/RTA_MC2D.cpp:871-964): the particle meets
// its box's contact with box `inew` of another crystal; the interface's
// table re-emits it on either side (Diffuse_mismatch_distribution::reemit,
// src/sampling.cpp:831-902: p uniform between the first and the last
// cumulative value of the incident mode's entries, the first entry not
// below p) and the flight ends (dt = 0).  An incident mode without entries
// (the reference's 'X') crosses with its index kept within the crystal.
template <class P>
__device__ int dmm_cross(const DevTables& T, P& pol, Particle& p, int inew, int table, double& dt, Counters& c) {
    const long long* row = T.dmm_row + (long long)table * (T.n + 1);
    const long long e0 = row[p.mode], e1 = row[p.mode + 1];
    c.ifc_hits++;
    if (e1 > e0) {
        const double lo = T.dmm_ent[e0].cum, hi = T.dmm_ent[e1 - 1].cum;
        const double pp = pol.u() * (hi - lo) + lo;
        long long a = e0, b = e1 - 1;
        while (a < b) {
            const long long mid = (a + b) >> 1;
            if (T.dmm_ent[mid].cum >= pp) b = mid;
            else a = mid + 1;
        }
        const DmmEnt en = T.dmm_ent[a];
        p.mode = en.out;
        if (en.side != 0) {
            p.box = inew;
            p.mo = mat_off(T, inew);
            c.ifc_trans++;
        }
    } else {
        c.quirks++;
        const int k = dmm_same_index(T, p.mode, T.box_mat[p.box], T.box_mat[inew]);
        if (k < 0) return E_VALUE;
        p.mode = k;
        p.box = inew;
        p.mo = mat_off(T, inew);
        c.ifc_trans++;
    }
    dt = 0.;
    return 0;
}

template <class P>
__device__ int correct_corner_problem(const DevTables& T, P& pol, V2 rf, V2 v, const int* cand,
                                      int ncand, int& winner) {
    int fin[MAXC];
    int nf = 0;
    for (int i = 0; i < ncand; ++i) {
        const GBox& B = T.boxes[cand[i]];
        int nbrd = 0;
        for (int k = 0; k < B.nborders; ++k) {
            const GBorder& b = T.borders[B.border_off + k];
            if (on_segment(rf, b.la, b.lb) && dot(b.np, v) > 0.) nbrd++;
        }
        if (nbrd <= 1) fin[nf++] = cand[i];
    }
    if (nf == 0) return E_GEOM;
    winner = fin[pol.choose(nf)];
    return 0;
}

// geometry_2d::translate, include/geometry_2d.hpp:366-493: a particle in
// periodic box `box` jumps by 1.0005 x its translation vector into the box
// it maps to and from there into the neighbour that the jump segment meets.
// Two behaviours of the reference are kept: boost's intersection() appends
// to one point list, so every contact met by the segment reports the first
// contact's crossing point; with several candidates the point is taken from
// the candidate list at the position drawn among the filtered candidates.
// Returns 0 or an error code.
// FAST (production kernels): contacts that cannot take part are skipped
// before the segment and hull tests -- the excluded kinds first, then those
// whose contact segment's bounding box is apart from both the jump segment
// (no meet is possible) and the entry point tp (tp, tp + 1e-6 v and
// tp - 1e-6 T lie on this machine's border, so they can be inside the
// neighbour only next to the contact between the two).  A skipped contact
// is one the full tests reject too, so the candidates, their order and the
// draws are unchanged.
template <class P, bool FAST = false>
__device__ int translate(const DevTables& T, P& pol, int box, V2 r0, V2 v, int& nbox, V2& rf) {
    const int tib = T.boxes[box].tto;
    const V2 tv = T.translation[box];
    const V2 tj = scal(1.0005, tv);
    if (tib < 0 || tib >= T.nboxes || almost_equal(norm(tj), 0.)) return E_GEOM;
    const V2 p1 = add(r0, tj);
    const GBox& TB = T.boxes[tib];
    if (FAST && T.tfast) {
        // away from the ends of the contacts' intervals exactly one contact
        // of the target box qualifies, and it is the one the segment
        // crosses: the search below would find it alone and return the
        // crossing point, with no draw
        const int2 rg = T.tfast_rng[box];
        if (rg.y > 0) {
            const V2 uh = T.tfast_u[box];
            const double u = uh.x * r0.x + uh.y * r0.y;
            for (int k = 0; k < rg.y; ++k) {
                const TransFast f = T.tfast[rg.x + k];
                if (u > f.lo && u < f.hi) {
                    V2 xin;
                    if (seg_meet(r0, p1, T.cseg[2 * f.ci], T.cseg[2 * f.ci + 1], xin)) {
                        nbox = T.contacts[f.ci].id;
                        rf = xin;
                        return 0;
                    }
                    break;
                }
            }
        }
    }
    V2 tp;
    bool found = false;
    for (int k = 0; k < TB.nborders && !found; ++k) {
        const GBorder& b = T.borders[TB.border_off + k];
        found = seg_meet(r0, p1, b.la, b.lb, tp);
    }
    if (!found) return E_GEOM;  // "Error in translation, no box found"
    const V2 tp_T = sub(tp, divs(scal(1.0e-6, tv), norm(tv)));
    const V2 tp_v = add(tp, divs(scal(1.0e-6, v), norm(v)));
    int pb[MAXC];
    V2 prf[MAXC];
    int np = 0;
    bool have_first = false;
    V2 first = v2(0., 0.);
    for (int i = 0; i < TB.ncontacts; ++i) {
        const int ci = TB.contact_off + i;
        const int ibc = T.contacts[ci].id;
        if (FAST) {
            if (ibc == tib || T.boxes[ibc].tto >= 0 || T.boxes[ibc].reservoir) continue;
            const V2 a = T.cseg[2 * ci], b = T.cseg[2 * ci + 1];
            const double lox = fmin(a.x, b.x), hix = fmax(a.x, b.x);
            const double loy = fmin(a.y, b.y), hiy = fmax(a.y, b.y);
            const double mp = 1.0e-3, ms = 1.0e-9;  // nm
            const bool near_tp = tp.x >= lox - mp && tp.x <= hix + mp && tp.y >= loy - mp && tp.y <= hiy + mp;
            const bool near_seg = fmax(r0.x, p1.x) >= lox - ms && fmin(r0.x, p1.x) <= hix + ms &&
                                  fmax(r0.y, p1.y) >= loy - ms && fmin(r0.y, p1.y) <= hiy + ms;
            if (!near_tp && !near_seg) continue;
        }
        V2 xin;
        const bool here_i = seg_meet(r0, p1, T.cseg[2 * ci], T.cseg[2 * ci + 1], xin);
        const bool here_T = box_inside(T, ibc, tp);
        const bool here_Tv = box_inside(T, ibc, tp_v);
        const bool here_TT = box_inside(T, ibc, tp_T);
        const bool here = here_i || here_T || here_Tv || here_TT;
        if (ibc == tib || !here || T.boxes[ibc].tto >= 0 || T.boxes[ibc].reservoir) continue;
        V2 r;
        if (here_i) {
            if (!have_first) {
                first = xin;
                have_first = true;
            }
            r = first;
        } else if (here_T) {
            r = tp;
        } else if (here_Tv) {
            r = tp_v;
        } else {
            r = tp_T;
        }
        if (np == MAXC) return E_LIMIT;
        pb[np] = ibc;
        prf[np] = r;
        np++;
    }
    if (np > 1) {
        int p2[MAXC];
        int n2 = 0;
        for (int i = 0; i < np; ++i)
            if (box_inside(T, pb[i], add(prf[i], scal(1.0e-6, v)))) p2[n2++] = i;
        if (n2 == 0) return E_GEOM;  // the reference draws from an empty range here
        const int pos = pol.choose(n2);
        rf = prf[pos];
        nbox = pb[p2[pos]];
    } else if (np == 1) {
        nbox = pb[0];
        rf = prf[0];
    } else {
        return E_GEOM;  // "Error in Translation"
    }
    return 0;
}

// process_segment of a segment of length d starting at the particle:
// transient (time bins, src/RTA_MC2D.cpp:699-769) or steady (one value per
// box, :784-834).
template <bool STEADY, class P>
__device__ __forceinline__ int seg_tally(const DevTables& T, P& pol, const Particle& p, double d, V2 v) {
    if (STEADY) return pol.tally_dt(T, p.box, d, p.sign, v, p.mode);
    return pol.tally(T, p.box, p.t, p.t + d, p.sign, v, p.mode);
}

// evolparticle: transient (src/RTA_MC2D.cpp:990-1386) or, with STEADY, the
// periodic/gradient variant (:1406-1799): the flight ends inside a box with
// phi += sign instead of a resample, and a reflected particle leaves the
// generation (`fate`).  Returns 0 or an error code.
template <class P, bool STEADY = false>
__device__ int evolparticle(const DevTables& T, P& pol, Particle& p, V2 v, double& dt,
                            Counters& c, int& nudges, int& fate) {
    const V2 opos = p.pos;
    const GBox& box = T.boxes[p.box];
    if (box.tto >= 0) {  // periodic box (src/RTA_MC2D.cpp:1034-1042)
        int nb;
        V2 rf;
        const int e = translate(T, pol, p.box, opos, v, nb, rf);
        if (e) return e;
        p.box = nb;
        p.pos = rf;
        c.translations++;
        return 0;
    }
    if (box.reservoir) {
        p.mode = 0;
        dt = 0.;
        c.absorbed++;
        fate = FATE_ABSORBED;
        return 0;
    }
    V2 rnew = v2(p.pos.x + dt * v.x, p.pos.y + dt * v.y);
    if (inside_hull(T.hull + box.hull_off, box.nhull, rnew)) {
        p.pos = rnew;
        int e = seg_tally<STEADY>(T, pol, p, dt, v);
        if (e) return e;
        p.t += dt;
        if (STEADY) {
            fate = FATE_SCATTER;
            c.scattered++;
        } else if (!T.ballistic) {
            p.mode = pol.resample(T, p.mo);
        }
        dt = 0.;
        nudges = 0;
        return 0;
    }
    HitD mru;
    if (!get_inter_side(T, p.box, p.pos, v, dt, mru)) {
        const V2 d = sub(box.center, opos);
        p.pos = add(p.pos, divs(scal(1.0e-6, d), norm(d)));
        c.nudges++;
        if (++nudges > NUDGE_CAP) return E_LIMIT;
        return 0;
    }
    nudges = 0;
    double left_time = dt - mru.time;
    const double tf = mru.time;
    if (almost_equal(left_time, 0.)) left_time = 0.;
    dt = left_time;
    rnew = mru.rf;
    const V2 reps = add(rnew, divs(scal(1.0e-6, v), norm(v)));
    // candidate boxes among the contacts (ascending id)
    int pboxes[MAXC];
    int np = 0;
    for (int i = 0; i < box.ncontacts; ++i) {
        const GContact& gc = T.contacts[box.contact_off + i];
        const int test = gc.id;
        if (test == p.box) continue;
        const double npv = dot(gc.np, v);
        const bool parallel = almost_equal(npv, 0.);
        const bool oriented = npv > 0.;
        if ((box_inside(T, test, rnew) || box_inside(T, test, reps)) && !parallel && oriented) {
            if (np == MAXC) return E_LIMIT;
            pboxes[np++] = test;
        }
    }
    if (np == 0) {
        int e = seg_tally<STEADY>(T, pol, p, tf, v);
        if (e) return e;
        p.t += tf;
        // in_corner3 over the boxes that can cover a border point: this box
        // and its contacts, in ascending id order
        int ids[MAXC + 1];
        int ni = 0;
        {
            const int self = p.box;
            bool self_added = false;
            for (int i = 0; i < box.ncontacts; ++i) {
                const int cand = T.contacts[box.contact_off + i].id;
                if (!self_added && self < cand) {
                    if (box_inside(T, self, rnew)) ids[ni++] = self;
                    self_added = true;
                }
                if (ni >= MAXC) return E_LIMIT;
                if (box_inside(T, cand, rnew)) ids[ni++] = cand;
            }
            if (!self_added && box_inside(T, self, rnew)) ids[ni++] = self;
        }
        if (ni > 2) {
            int winner;
            int e2 = correct_corner_problem(T, pol, rnew, v, ids, ni, winner);
            if (e2) return e2;
            p.box = winner;
            const V2 corr = sub(T.boxes[winner].center, rnew);
            const V2 cpos = add(rnew, divs(scal(1.0e-6, corr), norm(corr)));
            if (!get_inter_side(T, winner, cpos, v, 1.0e+18, mru)) return E_GEOM;
            rnew = mru.rf;
        }
        const GBox& cur = T.boxes[p.box];
        int iborder;
        if (mru.nb > 1) {
            int vb[MAXB];
            int nv = 0;
            for (int i = 0; i < mru.nb; ++i) {
                const GBorder& mb = T.borders[cur.border_off + mru.bids[i]];
                const V2 rc = add(rnew, scal(1.0e-4, mb.np));
                bool isvoid = true;
                for (int j = 0; j < box.ncontacts; ++j)
                    if (box_inside(T, T.contacts[box.contact_off + j].id, rc)) {
                        isvoid = false;
                        break;
                    }
                if (isvoid) vb[nv++] = mru.bids[i];
            }
            if (nv == 0) return E_GEOM;
            // uniform_int_distribution(0, size): inclusive bound of the
            // reference; the out-of-range draw is counted and clamped
            int idx = pol.choose(nv + 1);
            if (idx == nv) {
                c.quirks++;
                idx--;
            }
            iborder = vb[idx];
        } else {
            iborder = mru.bids[0];
        }
        const GBorder& wb = T.borders[cur.border_off + iborder];
        int nm = -1;
        if (T.specularity > 0.) {
            if (pol.u() < T.specularity) {
                const int mm = T.mirror ? T.mirror[wb.ncls * T.n + p.mode] : -1;
                if (mm >= 0) {
                    nm = mm;
                    c.specular++;
                }
            }
        }
        if (nm < 0) {
            nm = pol.bounce(T, wb.ncls, p.mode);
            if (nm < 0) return E_GEOM;
        }
        p.pos = rnew;
        p.mode = nm;
        dt = 0.;
        c.wall_hits++;
        fate = FATE_BOUNCE;
        return 0;
    } else if (np == 1) {
        p.pos = rnew;
        int e = seg_tally<STEADY>(T, pol, p, tf, v);
        if (e) return e;
        p.t += tf;
        const int tab = dmm_table(T, p.box, pboxes[0]);
        if (tab >= 0) {  // another crystal (:1282, :1690)
            e = dmm_cross(T, pol, p, pboxes[0], tab, dt, c);
            if (STEADY) fate = FATE_BOUNCE;  // pushed into the next generation
            return e;
        }
        p.box = pboxes[0];
        c.crossings++;
        return 0;
    } else {
        int e = seg_tally<STEADY>(T, pol, p, tf, v);
        if (e) return e;
        p.t += tf;
        p.pos = rnew;
        int pbox2[MAXC];
        int n2 = 0;
        const V2 rcheck = add(rnew, scal(1.0e-6, v));
        for (int i = 0; i < np; ++i)
            if (box_inside(T, pboxes[i], rcheck)) pbox2[n2++] = pboxes[i];
        int newid;
        if (n2 == 0) {
            newid = pboxes[pol.choose(np)];
            const V2 d = sub(T.boxes[newid].center, rnew);
            if (T.boxes[newid].tto < 0) p.pos = add(p.pos, divs(scal(1.0e-6, d), norm(d)));
        } else {
            newid = pbox2[pol.choose(n2)];
        }
        const int tab = dmm_table(T, p.box, newid);
        if (tab >= 0) {  // another crystal (:1355-1366, :1762-1776)
            e = dmm_cross(T, pol, p, newid, tab, dt, c);
            if (STEADY) fate = FATE_BOUNCE;
            return e;
        }
        p.box = newid;
        c.crossings++;
        return 0;
    }
}

// A wall particle of Init_generator (case 0, src/RTA_MC2D.cpp:453-497),
// after the generator-type draw.
template <class P>
__device__ int generate_wall(const DevTables& T, P& pol, Particle& p) {
    const double whereGenR = pol.u();
    int g = lower_bound_d(T.wall_cum, T.ngen, whereGenR);
    if (g >= T.ngen) g = T.ngen - 1;
    const WallGenDev W = T.walls[g];
    V2 ppos;
    int tries = 0;
    for (;;) {
        if (++tries > 1000) return E_LIMIT;
        ppos = add(W.p1, scal(pol.u(), W.nd));
        if (on_segment(ppos, W.sa, W.sb)) break;
    }
    if (!box_inside(T, W.box, ppos)) {
        const V2 d = sub(T.boxes[W.box].center, ppos);
        ppos = add(ppos, divs(scal(1.0e-6, d), norm(d)));
        if (!box_inside(T, W.box, ppos)) return E_GEOM;
    }
    p.mode = pol.gen_mode(T, g);
    p.pos = ppos;
    p.sign = W.sign;
    p.t = 0.;
    p.box = W.box;
    p.mo = mat_off(T, W.box);
    return 0;
}

// Uniform point of box b by bounding-box rejection
// (geometry_2d::get_random_point, include/geometry_2d.hpp:338-356).
template <class P>
__device__ int random_point(const DevTables& T, P& pol, int b, V2& r) {
    const GBox& B = T.boxes[b];
    const V2* h = T.hull + B.hull_off;
    double x0 = h[0].x, x1 = h[0].x, y0 = h[0].y, y1 = h[0].y;
    for (int i = 1; i < B.nhull; ++i) {
        x0 = fmin(x0, h[i].x);
        x1 = fmax(x1, h[i].x);
        y0 = fmin(y0, h[i].y);
        y1 = fmax(y1, h[i].y);
    }
    int tries = 0;
    for (;;) {
        if (++tries > 100000) return E_LIMIT;
        r.x = x0 + pol.u() * (x1 - x0);
        r.y = y0 + pol.u() * (y1 - y0);
        if (inside_hull(h, B.nhull, r)) return 0;
    }
}

// Particle generation.  Returns 0 or an error code.
template <class P>
__device__ int generate(const DevTables& T, P& pol, long long pid, Particle& p) {
    if (T.source == 0) {
        (void)pol.u();  // generator type: without a gradient every particle comes from a wall
        return generate_wall(T, pol, p);
    }
    // initial deviation: particle -> box by the prefix of generated counts
    int lo = 0, hi = T.ngen;  // find g with init_first[g] <= pid < init_first[g+1]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (T.init_first[mid] <= pid) lo = mid; else hi = mid;
    }
    const int g = lo;
    const int b = T.init_box[g];
    V2 r;
    const int e = random_point(T, pol, b, r);
    if (e) return e;
    p.mode = pol.gen_mode(T, g);
    p.pos = r;
    p.sign = T.init_sign[g];
    p.t = 0.;
    p.box = b;
    p.mo = mat_off(T, b);
    return 0;
}

// A whole particle life.  Returns 0 or an error code.
template <class P>
__device__ int run_particle(const DevTables& T, P& pol, long long pid, Counters& c) {
    Particle p;
    int e = generate(T, pol, pid, p);
    if (e) return e;
    double time = 0.;
    int nudges = 0;
    long long nev = 0;
    while (time < T.maxtime) {
        if (++nev > T.flight_cap) return E_LIMIT;
        const int k = p.mode;
        const V2 v = v2(T.vxc[k], T.vyc[k]);
        const double w = T.w[p.mo + k];
        if (w == 0.) return E_VALUE;
        double dt = pol.flight(T, p.mo + k);
        c.events++;
        if (time + dt > T.maxtime) dt = T.maxtime - time + 1.0e-8;
        int guard = 0, fate = FATE_LOST;
        while (!almost_equal(dt, 0.)) {
            if (++guard > FLIGHT_CAP) return E_LIMIT;
            e = evolparticle(T, pol, p, v, dt, c, nudges, fate);
            if (e) return e;
        }
        if (p.mode == 0) break;
        time = p.t;
    }
    return 0;
}

}  // namespace bte
