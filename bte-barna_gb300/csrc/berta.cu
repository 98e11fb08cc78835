// berta.cu - beyond-RTA deviational MC (beRTAMC2D) on the device.
//
// The step loop of src/beyondRTA_MC2d.cpp:2138-2425, production mode, with
// the particle numbers kept on the device (no host wait inside the loop):
//   1 advection by dt; void walls absorb and count Eborder, reservoirs absorb
//     (evolparticle :708-970), fused with 5-7 for the particles of the last
//     step                                                        be_advance
//   2 gradient source term: Nabla_T particles at random points of every box
//     with a gradient, random sub-step (source_term_gradient :597-676,
//     Nabla_T_distribution src/sampling.cpp:118-187)
//                                           be_plan_sources, be_generate_dev
//   3 isothermal-wall injection, random sub-step (Isothermal_walls :446-585,
//     Ntogenerate src/sampling.cpp:243-260)
//                                           be_plan_sources, be_generate_dev
//   4 adiabatic diffuse re-emission of |Eborder| at the wall temperature from
//     the J(T) cubic spline (adiabatic_diffuse_walls :281-435)
//                  be_plan_adiabatic, be_wall_cdf1/2_dev, be_generate_dev
//   5 deletion of the absorbed particles, 6 propagator scattering with sign
//     branching (Scattering :1073-1210, propagator_H::get
//     src/collision_operator.cpp:892-903), each parent's branching attempts
//     made in place by its thread, or the RTA alternative (ScatteringRTA
//     :983-1062), 7 histogram H[box][mode] += sign: one pass that reads each
//     particle once and writes each outgoing particle once     be_advance
//   8 cancellation every 4th step: keep |H| particles of the majority sign
//     per (box, mode) (:2295-2370), by per-key ranks, no sort
//                                            be_cancel_dev, be_compact_dev
//   9 calculate_prop: ed and flux per box from H (:1538-1602), recorded per
//     step on the device                                          be_props
// Particles live in HBM as structure-of-arrays (x, y FP64; mode, box, sign
// int32).  Draws: Philox4x32-10 keyed by (seed, step, phase), counter =
// particle index.  Geometry: boxes that tile an axis-aligned grid, or any
// convex boxes with periodic boxes (the general advection).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace bte {

struct PArr {
    double* x;
    double* y;
    int* mode;
    int* box;
    int* sign;
};

// A particle source of one step: a border segment (walls) or a box
// rectangle (initial deviation), a sign, a mode distribution (alias table at
// `alias_off` of the step's alias buffer) and its particles [first, first+n).
struct GenDesc {
    double x0, y0, dx, dy;  // border: p1 + u (dx, dy); rectangle: x0 + u dx, y0 + v dy
    int box, sign, rect;
    int cdf;                // >= 0: mode from device CDF row `cdf`; -1: alias row at alias_off
    long long alias_off;
    long long first;
    int msign;              // 1: sign of each mode from the sign row at alias_off
    int pad;
};

// One adiabatic re-emission distribution to build on the device: an
// isothermal wall at Tw facing a box at Te, inward normal (nx, ny).
struct WallReq {
    double nx, ny, Tw, Te;
};

// Propagator alias entry: slot j keeps outgoing mode j+3 with probability
// prob, else takes alt; the two top bits carry the signs of P at the kept
// and alternative slots.
struct PAlias {
    float prob;
    unsigned alt;  // bits 0-29 slot, bit 30 alt negative, bit 31 keep negative
};

// The scattering table of one box (Scattering, src/beyondRTA_MC2d.cpp:
// 1130-1165): the alias table of the propagator tabulated at the box's Teq,
// or the signed CDFs c1, c2 of the two tabulated temperatures T1 < T2 that
// the reference picks for it, interpolated at T = Teq on the fly as lirp
// (src/collision_operator.cpp:918-929) interpolates them; all null for a
// box where nothing scatters (reservoirs, periodic boxes).
struct BoxProp {
    const PAlias* alias;
    const double* c1;
    const double* c2;
    double T, T1, T2;
};

// Page-locked staging for the per-step uploads: a copy from pageable memory
// may wait for the stream's earlier work, a copy from here does not.  Each
// upload site has its own buffer, written again only after a later sync.
template <class T>
void upload_pinned(DBuf& d, Pinned& h, const std::vector<T>& v, cudaStream_t s) {
    const size_t bytes = v.size() * sizeof(T);
    if (bytes == 0) return;
    d.alloc(bytes);
    h.reserve(bytes);
    std::memcpy(h.p, v.data(), bytes);
    ck(cudaMemcpyAsync(d.p, h.p, bytes, cudaMemcpyHostToDevice, s), "h2d");
}

struct BertaState {
    bool have_prop = false;
    int nm = 0;
    double T = 0;
    // propagators tabulated in temperature (one bte_load_propagator call
    // each), host copies kept for the interpolation of lirp
    std::map<double, std::vector<double>> props;
    long long props_version = 0;
    // device tables per tabulated temperature, built when a box asks for
    // them: the alias table (a box at that Teq) and the signed CDF (an end
    // of an interpolation); dropped when the propagators change
    std::map<double, DBuf> dev_alias, dev_cdf;
    long long dev_version = -1;
    DBuf d_boxprop;                         // BoxProp per box
    long long cap = 0;
    DBuf a_x, a_y, a_mode, a_box, a_sign;   // particles
    DBuf b_x, b_y, b_mode, b_box, b_sign;   // compaction / scattering output
    DBuf d_H, d_cnt, d_Eb, d_props, d_boxwall, d_gens, d_alias, d_rvx, d_rvy;
    DBuf d_om, d_vx, d_vy, d_req, d_cdf, d_cdftot, d_isoprob, d_isoalt;
    DBuf d_gprob, d_galt, d_gsign;          // gradient source rows
    DBuf d_ctot;                            // wall-CDF chunk sums
    Pinned h_gens[1];                       // staging: descriptors of the initial particles
    // device-resident step loop: counters, planned sources, per-step records
    DBuf d_dc, d_span, d_gdesc, d_ggenf, d_gcnt, d_idesc, d_igenf, d_icnt, d_adi, d_adesc, d_acnt;
    DBuf d_phist, d_nhist, d_sa, d_sb, d_sc, d_sd, d_sx0, d_sxs;

    std::vector<Spline1D> spl;
    std::vector<char> spl_ok;
    long long spl_version = -1;   // tables the splines were built for
};

void reset_propagators(bte_ctx* c) {
    if (!c->berta) return;
    c->berta->props.clear();
    c->berta->have_prop = false;
    c->berta->props_version++;
}

void destroy_berta(bte_ctx* c) {
    delete c->berta;
    c->berta = nullptr;
}

namespace {

__device__ __forceinline__ long long obits(double x) { return __double_as_longlong(x); }

__device__ __forceinline__ int grid_at(const DevGrid& G, int i, int j) {
    if (i < 0 || j < 0 || i >= G.nx || j >= G.ny) return -1;
    return __ldg(G.cell + i * G.ny + j);
}

// Ballistic advection of one particle for time `dt` on the grid.  Returns
// false when it was absorbed (mode set to -1): at a void wall its signed
// count goes to the wall's Eborder, at a reservoir it is dropped.
__device__ bool advect_one(const DevGrid& G, const int2* boxcell, const ModeVel* mv, const int4* boxwall,
                           int* Eb, double& x, double& y, int& box, int mode, int sign, double dt) {
    const ModeVel v = mv[mode];
    const int2 ij = __ldg(boxcell + box);
    int i = ij.x, j = ij.y;
    for (int guard = 0; guard < (1 << 20); ++guard) {
        const int upx = obits(v.vx) >= 0 ? 1 : 0, upy = obits(v.vy) >= 0 ? 1 : 0;
        const double xw = __ldg(G.gx + i + upx), yw = __ldg(G.gy + j + upy);
        const double tx = (xw - x) * v.ivx, ty = (yw - y) * v.ivy;
        const bool xfirst = obits(tx) <= obits(ty);
        const long long te_b = xfirst ? obits(tx) : obits(ty);
        if (!(obits(dt) > te_b)) {  // stays in the cell
            x = fma(dt, v.vx, x);
            y = fma(dt, v.vy, y);
            return true;
        }
        const double seg = __longlong_as_double(te_b > 0 ? te_b : 0);
        double nx = fma(seg, v.vx, x), ny = fma(seg, v.vy, y);
        int ni = i, nj = j, wall;
        if (xfirst) {
            nx = xw;
            ni = i + (upx ? 1 : -1);
            wall = upx ? 0 : 1;
        } else {
            ny = yw;
            nj = j + (upy ? 1 : -1);
            wall = upy ? 2 : 3;
        }
        x = nx;
        y = ny;
        dt -= seg;
        const int nb = grid_at(G, ni, nj);
        if (nb >= 0) {
            i = ni;
            j = nj;
            box = nb;
            continue;
        }
        if (nb == -1) {  // void wall: absorbed, counted on the wall
            const int4 bw = __ldg(boxwall + box);
            const int gb = wall == 0 ? bw.x : wall == 1 ? bw.y : wall == 2 ? bw.z : bw.w;
            if (gb >= 0) atomicAdd(Eb + gb, sign);
        }
        return false;
    }
    return false;
}

struct AdvectArgs {
    DevGrid G;
    const int2* boxcell;
    const ModeVel* mv;
    const int4* boxwall;
    int* Eb;
    double dt;
    unsigned long long key;  // Philox key of the random sub-steps
    int random_substep;
    // boxes that do not tile a grid (or periodic boxes): the convex-box
    // tables and the key of the geometric choices
    int general;
    unsigned long long gkey;
    int* err;
    DevTables T;
};

// Draws of the geometric choices of one particle's advection.
struct BePol {
    Philox g;
    __device__ double u() { return g.uniform(); }
    __device__ int choose(int n) { return uniform_below(g, uint32_t(n)); }
};

// beRTA evolparticle on convex boxes (src/beyondRTA_MC2d.cpp:708-970):
// ballistic advance by dt; a periodic box translates and the remaining time
// goes on; a void wall absorbs the particle into its border's Eborder (at a
// corner of three or more boxes, into the first border of the chosen box
// that faces the velocity); reservoirs absorb.  Returns false when the
// particle was absorbed; err is set on a geometry failure.
__device__ bool advect_general(const DevTables& T, BePol& pol, int* Eb, double& x, double& y, int& box,
                               int mode, int sign, double dt, int& err) {
    const V2 v = v2(T.vxc[mode], T.vyc[mode]);
    V2 pos = v2(x, y);
    for (int guard = 0; guard < (1 << 16); ++guard) {
        if (T.boxes[box].reservoir) return false;
        if (T.boxes[box].tto >= 0) {
            int nb;
            V2 rf;
            if (translate<BePol, true>(T, pol, box, pos, v, nb, rf)) {
                err = E_GEOM;
                return false;
            }
            box = nb;
            pos = rf;
        }
        const GBox& B = T.boxes[box];
        V2 rnew = v2(pos.x + dt * v.x, pos.y + dt * v.y);
        if (inside_hull(T.hull + B.hull_off, B.nhull, rnew)) {
            x = rnew.x;
            y = rnew.y;
            return true;
        }
        HitD mru;
        if (!get_inter_side(T, box, pos, v, dt, mru)) {
            const V2 d = sub(B.center, pos);
            pos = add(pos, divs(scal(1.0e-6, d), norm(d)));
            continue;
        }
        double left = dt - mru.time;
        if (almost_equal(left, 0.)) left = 0.;
        rnew = mru.rf;
        const V2 reps = add(rnew, divs(scal(1.0e-6, v), norm(v)));
        int pb[MAXC];
        int np = 0;
        for (int i = 0; i < B.ncontacts; ++i) {
            const GContact& gc = T.contacts[B.contact_off + i];
            if (gc.id == box) continue;
            const double npv = dot(gc.np, v);
            if ((box_inside(T, gc.id, rnew) || box_inside(T, gc.id, reps)) && !almost_equal(npv, 0.) && npv > 0.) {
                if (np == MAXC) {
                    err = E_LIMIT;
                    return false;
                }
                pb[np++] = gc.id;
            }
        }
        if (np == 0) {
            // in_corner3 over this box and its contacts
            int ids[MAXC + 1];
            int ni = 0;
            if (box_inside(T, box, rnew)) ids[ni++] = box;
            for (int i = 0; i < B.ncontacts && ni < MAXC; ++i) {
                const int cnd = T.contacts[B.contact_off + i].id;
                if (box_inside(T, cnd, rnew)) ids[ni++] = cnd;
            }
            if (ni > 2) {
                // correct_corner_problem (include/geometry_2d.hpp:524-561):
                // candidates with at most one border at rnew facing v; the
                // particle goes to the first such border of the drawn one
                int fin[MAXC + 1], fb[MAXC + 1];
                int nf = 0;
                for (int i = 0; i < ni; ++i) {
                    const GBox& C = T.boxes[ids[i]];
                    int cnt = 0, first = -1;
                    for (int k = 0; k < C.nborders; ++k) {
                        const GBorder& bb = T.borders[C.border_off + k];
                        if (on_segment(rnew, bb.la, bb.lb) && dot(bb.np, v) > 0.) {
                            if (cnt == 0) first = k;
                            cnt++;
                        }
                    }
                    if (cnt <= 1) {
                        fin[nf] = ids[i];
                        fb[nf] = first;
                        nf++;
                    }
                }
                if (nf == 0) {
                    err = E_GEOM;
                    return false;
                }
                const int w = pol.choose(nf);
                if (fb[w] < 0) {  // the reference reads an empty border list here
                    err = E_GEOM;
                    return false;
                }
                box = fin[w];
                atomicAdd(Eb + T.boxes[box].border_off + fb[w], sign);
                x = rnew.x;
                y = rnew.y;
                return false;
            }
            int ib;
            if (mru.nb > 1) {
                int vb[MAXB];
                int nv = 0;
                for (int i = 0; i < mru.nb; ++i) {
                    const GBorder& mb = T.borders[B.border_off + mru.bids[i]];
                    const V2 rc = add(rnew, scal(1.0e-4, mb.np));
                    bool isvoid = true;
                    for (int j = 0; j < B.ncontacts; ++j)
                        if (box_inside(T, T.contacts[B.contact_off + j].id, rc)) {
                            isvoid = false;
                            break;
                        }
                    if (isvoid) vb[nv++] = mru.bids[i];
                }
                if (nv == 0) {
                    err = E_GEOM;
                    return false;
                }
                ib = vb[pol.choose(nv)];  // alma::choose: uniform over the void borders
            } else {
                ib = mru.bids[0];
            }
            atomicAdd(Eb + B.border_off + ib, sign);
            x = rnew.x;
            y = rnew.y;
            return false;
        }
        if (np == 1) {
            box = pb[0];
            pos = rnew;
            dt = left;
            continue;
        }
        // several candidates: the ones that contain rnew + tau v for the
        // largest tau in 1e-6, 1e-7, ... 1e-15
        int p2[MAXC];
        int n2 = 0;
        for (double tau = 1.0e-6; n2 == 0 && tau >= 1.0e-15; tau /= 10.0) {
            const V2 rc = add(rnew, scal(tau, v));
            for (int i = 0; i < np; ++i)
                if (box_inside(T, pb[i], rc)) p2[n2++] = pb[i];
        }
        if (n2 == 0) {
            const V2 d = sub(B.center, rnew);
            pos = add(rnew, divs(scal(1.0e-6, d), norm(d)));
            dt = left;
            continue;
        }
        box = p2[pol.choose(n2)];
        pos = rnew;
        dt = left;
    }
    err = E_LIMIT;
    return false;
}

// Isothermal_wall_distribution (src/sampling.cpp:189-269) of each request:
// pmf_k = v_n omega_k |n(omega_k, Tw) - n(omega_k, Te)| for v_n > 0, turned
// into a CDF row; tot[r] keeps the sum.  Each request's row is split into
// chunks of WCDF_CHUNK modes, one block each.
//
// The pmf is evaluated in FP32 and summed in FP64: with x = hbar omega / kT,
// n_w - n_e = expm1(x_e - x_w) / (expm1(x_e) (-expm1(-x_w))), which has no
// cancellation when Tw is close to Te; when |x_e - x_w| >= 1/2 the plain
// difference 1/expm1(x_w) - 1/expm1(x_e) loses nothing either.  Entries
// above 1e-6 of the row's largest are within 4e-6 relative of the FP64
// value, all entries above 1e-30 of it within 1e-5 (the rounding of x to
// FP32 at x ~ 60), and the FP64 units do one addition per mode instead of
// two exponentials and two divisions.
constexpr int WCDF_CHUNK = 1024;

__device__ __forceinline__ float wall_pmf_f(float w, float vn, float ce, float q, float rr) {
    const float xe = ce * w;   // x_e
    const float xw = xe * q;   // x_w = x_e Te / Tw
    const float d = xe * rr;   // x_e - x_w = x_e (Tw - Te) / Tw
    float diff;
    if (fabsf(d) < 0.5f)
        diff = xe < 80.f ? expm1f(d) / (expm1f(xe) * -expm1f(-xw)) : 0.f;
    else
        diff = 1.f / expm1f(xw) - 1.f / expm1f(xe);
    return vn * w * fabsf(diff);
}

// pass 1: the chunk's running sums in place and its total
__device__ __forceinline__ void wall_cdf1_body(const float* om, const float* vx, const float* vy, int n,
                                               const WallReq* req, double* cdf, double* chunk_tot) {
    __shared__ double part[256];
    const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
    const int r = blockIdx.x / nch, ch = blockIdx.x % nch;
    const WallReq R = req[r];
    double* row = cdf + (long long)r * n;
    const int c0 = ch * WCDF_CHUNK, c1 = min(n, c0 + WCDF_CHUNK);
    const int seg = (c1 - c0 + blockDim.x - 1) / blockDim.x;
    const int k0 = c0 + threadIdx.x * seg, k1 = min(c1, k0 + seg);
    constexpr double pre = 1e12 * 1.054571726e-34 / 1.3806488e-23;
    const float ce = float(pre / R.Te), q = float(R.Te / R.Tw), rr = float((R.Tw - R.Te) / R.Tw);
    const float nx = float(R.nx), ny = float(R.ny);
    double acc = 0.;
    for (int k = k0; k < k1; ++k) {
        const float w = __ldg(om + k);  // 0 where almost_equal(0, omega)
        const float vn = nx * __ldg(vx + k) + ny * __ldg(vy + k);
        const float p = (vn > 0.f && w != 0.f) ? wall_pmf_f(w, vn, ce, q, rr) : 0.f;
        acc += double(p);
        row[k] = acc;  // running sum within the thread's segment
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive offsets of the segments
        double sum = 0.;
        for (int t = 0; t < blockDim.x; ++t) {
            const double v = part[t];
            part[t] = sum;
            sum += v;
        }
        chunk_tot[blockIdx.x] = sum;
    }
    __syncthreads();
    const double off = part[threadIdx.x];
    for (int k = k0; k < k1; ++k) row[k] += off;
}

// pass 2: offsets of the chunks, normalisation, the request's total
__device__ __forceinline__ void wall_cdf2_body(int n, const double* chunk_tot, double* cdf, double* tot) {
    const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
    const int r = blockIdx.x / nch, ch = blockIdx.x % nch;
    double off = 0., total = 0.;
    for (int c = 0; c < nch; ++c) {
        const double v = chunk_tot[(long long)r * nch + c];
        if (c < ch) off += v;
        total += v;
    }
    if (ch == 0 && threadIdx.x == 0) tot[r] = total;
    if (!(total > 0.)) return;
    double* row = cdf + (long long)r * n;
    const int c0 = ch * WCDF_CHUNK, c1 = min(n, c0 + WCDF_CHUNK);
    for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) row[k] = (row[k] + off) / total;
}

// New particles [base, base + n) from the step's sources.
__global__ void be_generate(PArr P, long long base, long long n, const GenDesc* gens, int ngen,
                            const float* aprob, const int* aalt, const signed char* asign,
                            const double* cdfs, const double* cdftot, int nmodes, unsigned long long key,
                            const GBox* boxes, const V2* hull) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = ngen;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (gens[mid].first <= k) lo = mid; else hi = mid;
        }
        const GenDesc gd = gens[lo];
        Philox g;
        g.init(key, (uint64_t)k);
        double x, y;
        bool placed = true;
        if (gd.rect == 2) {
            // a box that is not a grid cell: bounding box and rejection
            // (geometry_2d::get_random_point, include/geometry_2d.hpp:338-356)
            const GBox& Bx = boxes[gd.box];
            placed = false;
            for (int tries = 0; tries < 100000 && !placed; ++tries) {
                x = gd.x0 + g.uniform() * gd.dx;
                y = gd.y0 + g.uniform() * gd.dy;
                placed = inside_hull(hull + Bx.hull_off, Bx.nhull, v2(x, y));
            }
        } else if (gd.rect) {
            x = gd.x0 + g.uniform() * gd.dx;
            y = gd.y0 + g.uniform() * gd.dy;
        } else {
            const double u = g.uniform();
            x = gd.x0 + u * gd.dx;
            y = gd.y0 + u * gd.dy;
        }
        int mode;
        if (gd.cdf >= 0) {
            // lower_bound over the border's CDF row (Grid_distribution::sample)
            const double* row = cdfs + (long long)gd.cdf * nmodes;
            mode = cdftot[gd.cdf] > 0. ? lower_bound_d(row, nmodes, g.uniform()) : -1;
            if (mode >= nmodes) mode = nmodes - 1;
            if (!placed) mode = -1;
        } else {
            const float* pr = aprob + gd.alias_off;
            const int* al = aalt + gd.alias_off;
            const int j = int(mulhi32(g.next32(), uint32_t(nmodes)));
            const float acc = float(g.next32() >> 8) * 0x1p-24f;
            mode = acc < __ldg(pr + j) ? j : __ldg(al + j);
        }
        const long long i = base + k;
        P.x[i] = x;
        P.y[i] = y;
        P.box[i] = gd.box;
        P.mode[i] = mode;
        P.sign[i] = (gd.msign && mode >= 0) ? int(__ldg(asign + gd.alias_off + mode)) : gd.sign;
    }
}

// Append the live particles of [0, n) to `out` (warp-aggregated).
// Compaction of [0, n): each block takes tiles of 4 x blockDim particles,
// counts its survivors with warp ballots and claims their places with one
// atomic per tile (the order inside a tile is kept).
constexpr int COMPACT_ITEMS = 4;
__device__ __forceinline__ void compact_body(PArr in, long long n, PArr out, unsigned long long* count) {
    __shared__ unsigned wcnt[COMPACT_ITEMS][32];
    __shared__ unsigned long long tile_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long long tile = (long long)COMPACT_ITEMS * blockDim.x;
    for (long long base = blockIdx.x * tile; base < n; base += (long long)gridDim.x * tile) {
        bool live[COMPACT_ITEMS];
        unsigned m[COMPACT_ITEMS];
#pragma unroll
        for (int k = 0; k < COMPACT_ITEMS; ++k) {
            const long long i = base + (long long)k * blockDim.x + threadIdx.x;
            live[k] = i < n && in.mode[i] >= 0;
            m[k] = __ballot_sync(0xffffffffu, live[k]);
            if (lane == 0) wcnt[k][warp] = __popc(m[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // exclusive offsets of (item, warp) in tile order
            unsigned tot = 0;
            for (int k = 0; k < COMPACT_ITEMS; ++k)
                for (int w = 0; w < nw; ++w) {
                    const unsigned c = wcnt[k][w];
                    wcnt[k][w] = tot;
                    tot += c;
                }
            tile_base = tot ? atomicAdd(count, (unsigned long long)tot) : 0ull;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < COMPACT_ITEMS; ++k) {
            if (live[k]) {
                const long long i = base + (long long)k * blockDim.x + threadIdx.x;
                const long long o = (long long)(tile_base + wcnt[k][warp]) + __popc(m[k] & ((1u << lane) - 1u));
                out.x[o] = in.x[i];
                out.y[o] = in.y[i];
                out.mode[o] = in.mode[i];
                out.box[o] = in.box[i];
                out.sign[o] = in.sign[i];
            }
        }
        __syncthreads();
    }
}

// Entry k of the column interpolated at T: c1 + (T - T1) (c2 - c1) / (T2 - T1),
// rounded step by step as the host's interpolation of the whole table is.
__device__ __forceinline__ double lirp_at(const double* c1, const double* c2, int k, double T, double T1, double T2) {
    const double a = __ldg(c1 + k), b = __ldg(c2 + k);
    return __dadd_rn(a, __ddiv_rn(__dmul_rn(__dsub_rn(T, T1), __dsub_rn(b, a)), __dsub_rn(T2, T1)));
}

// propagator_H::lower_bound (include/collision_operator.hpp:263-269) over
// the column interpolated at T: the first entry whose |value| is not below
// u, by std::lower_bound's own probing (each probe interpolated when it is
// read), so that an interpolated column whose |values| are not monotone
// gives the same index as in the reference; clamped to the last entry.
__device__ __forceinline__ int lower_bound_abs_lirp(const double* c1, const double* c2, int n, double u, double T,
                                                    double T1, double T2) {
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int step = cnt >> 1;
        const int it = lo + step;
        if (fabs(lirp_at(c1, c2, it, T, T1, T2)) < fabs(u)) {
            lo = it + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    return lo < n ? lo : n - 1;
}

__global__ void be_hist(PArr P, long long n, int* H, int nmodes) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        atomicAdd(H + (long long)P.box[i] * nmodes + P.mode[i], P.sign[i]);
}

// Cancellation: a particle survives when its sign is the sign of H at its
// (box, mode) and its rank among those particles is below |H|.  Warps visit
// the particles in chunks of 32 consecutive ones: chunk c in the order of a
// random affine permutation w -> (a w + b) mod nchunks (a coprime to
// nchunks), and the lanes the chunk's particles in the order of a random
// XOR mask of the chunk, so the ranks, and with them the survivors, do not
// follow the order of the particle list, while every read stays coalesced.
__device__ __forceinline__ void cancel_body(PArr P, long long n, const int* H, int* cnt, int nmodes,
                                            const int* reservoir, unsigned long long pa, unsigned long long pb,
                                            unsigned mkey) {
    const unsigned long long nch = (unsigned long long)((n + 31) >> 5);
    const int lane = threadIdx.x & 31;
    const unsigned long long gw = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long w = gw; w < nch; w += nwarps) {
        const unsigned long long c = (pa * w + pb) % nch;
        const unsigned mask = ((unsigned)c * 0x9E3779B1u + mkey) >> 27;
        const long long i = (long long)(c << 5) + (long long)((unsigned)lane ^ mask);
        if (i >= n) continue;
        const long long key = (long long)P.box[i] * nmodes + P.mode[i];
        const int h = H[key];
        const int s = P.sign[i];
        bool keep = !reservoir[P.box[i]] && h != 0 && ((s < 0) == (h < 0));
        if (keep) keep = atomicAdd(cnt + key, 1) < (h < 0 ? -h : h);
        if (!keep) P.mode[i] = -1;
    }
}

// ed, flux_x, flux_y sums of one box (raw velocities, as calculate_prop).
__global__ void be_props(const int* H, int nmodes, const double* vx, const double* vy, double* out) {
    const int box = blockIdx.x;
    double e = 0., fx = 0., fy = 0.;
    for (int k = threadIdx.x; k < nmodes; k += blockDim.x) {
        const double h = double(H[(long long)box * nmodes + k]);
        e += h;
        fx += h * vx[k];
        fy += h * vy[k];
    }
    __shared__ double red[3][256];
    red[0][threadIdx.x] = e;
    red[1][threadIdx.x] = fx;
    red[2][threadIdx.x] = fy;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) out[3 * box + q] = red[q][0];
}

// ------------------------------------------------ device-resident step
// Counters of the step loop, kept on the device between kernels.
// DC_IN and DC_OUTT sum the particles read and written by be_advance over
// the run (the algorithmic traffic of its roofline).
enum { DC_NP = 0, DC_NOUT, DC_WORK, DC_FLIPS, DC_PSTEPS, DC_NGEN, DC_IN, DC_OUTT, DC_COUNT = 8 };

// A source planned on the device: where its particles start in the
// particle arrays and how many there are.
struct SrcSpan {
    unsigned long long base, total;
};

// Propagator scattering with sign branching (Scattering,
// src/beyondRTA_MC2d.cpp:1073-1210): every scattering attempt of a parent
// draws its next mode from the parent's column (an alias table over |P|
// with the signs in the alias word, or, for an interpolated propagator, the
// signed CDF probed as propagator_H::lower_bound does) and emits one
// outgoing particle; when the drawn sign differs from the parent's, the
// reference puts two copies of the parent back into the queue, and each
// copy makes an attempt of its own.  The copies are identical to the
// parent, so a thread keeps only the number of attempts its parent still
// owes and makes them in place, with fresh draws.  BRANCH_CAP bounds the
// attempts of one parent (a supercritical propagator never stops).
constexpr unsigned BRANCH_CAP = 1u << 20;

// One step of the particles [0, *n_in) of `in`, fused: advection by the
// step (advect = 1; particles born in this step were advected when they were
// made), then the scattering of the survivors -- RTA (ScatteringRTA,
// src/beyondRTA_MC2d.cpp:983-1062, a resampling with probability
// 1 - exp(-w dt)) or the propagator with sign branching as above -- and the
// histogram H[box][mode] += sign of every outgoing particle, appended to
// `out` warp by warp.  Persistent warps: a lane whose parent owes no more
// attempts takes the next parent from a counter; a parent absorbed during
// its advection owes none.  Each particle is read once and each outgoing
// particle written once.
__global__ void __launch_bounds__(256) be_advance(PArr in, const unsigned long long* n_in, PArr out,
                                                  unsigned long long* dc, long long ocap, int advect,
                                                  AdvectArgs aa, int rta, const PAlias* pal, const BoxProp* bprop,
                                                  int nm, const double* w, const float* rprob, const int* ralt,
                                                  int nmodes, unsigned long long skey, int* H, int* err) {
    const long long n = min((long long)*n_in, ocap);  // places beyond the buffers (an overflow) are not read
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) {
        if (advect) atomicAdd(dc + DC_PSTEPS, (unsigned long long)n);
        atomicAdd(dc + DC_IN, (unsigned long long)n);
    }
    unsigned long long flips = 0;
    int mode = 0, sign = 1, box = 0, col = 0;
    double x = 0., y = 0.;
    unsigned todo = 0, made = 0;
    bool done = false, valid = false;
    Philox g;
    g.init(skey, 0);
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, todo == 0 && !done);
        if (idle) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader) base = atomicAdd(dc + DC_WORK, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (todo == 0 && !done) {
                const long long i = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    mode = in.mode[i];
                    if (mode >= 0) {
                        sign = in.sign[i];
                        box = in.box[i];
                        x = in.x[i];
                        y = in.y[i];
                        bool alive = true;
                        if (advect) {
                            if (aa.general) {
                                BePol pol;
                                pol.g.init(aa.gkey, (uint64_t)i);
                                int e = 0;
                                alive = advect_general(aa.T, pol, aa.Eb, x, y, box, mode, sign, aa.dt, e);
                                if (e && aa.err) atomicCAS(aa.err, 0, e);
                            } else {
                                alive = advect_one(aa.G, aa.boxcell, aa.mv, aa.boxwall, aa.Eb, x, y, box, mode,
                                                   sign, aa.dt);
                            }
                        }
                        if (alive) {
                            col = mode - 3;
                            valid = rta ? true : (col >= 0 && col < nm);
                            if (!valid) atomicCAS(err, 0, E_VALUE);
                            g.init(skey, (uint64_t)i);
                            todo = 1;
                            made = 0;
                        }
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        const bool act = todo > 0;
        // the warp's output places, claimed before the draws so that the
        // atomic's round trip overlaps the propagator read
        const unsigned m1 = __ballot_sync(0xffffffffu, act);
        unsigned long long wo = 0;
        if (lane == 0 && m1) wo = atomicAdd(dc + DC_NOUT, (unsigned long long)__popc(m1));
        int nmode = mode, nsign = sign;
        if (act && rta) {
            const double u = g.uniform();
            if (u < 1. - exp(-__ldg(w + mode) * aa.dt)) {
                const int j = int(mulhi32(g.next32(), uint32_t(nmodes)));
                const float acc = float(g.next32() >> 8) * 0x1p-24f;
                nmode = acc < __ldg(rprob + j) ? j : __ldg(ralt + j);
            }
        } else if (act && valid) {
            // one table for every box (pal), or the box's own
            const PAlias* tab = pal ? pal : bprop[box].alias;
            if (tab) {
                const int j = int(mulhi32(g.next32(), uint32_t(nm)));
                const float acc = float(g.next32() >> 8) * 0x1p-24f;
                const PAlias e = tab[(long long)col * nm + j];
                const bool keep = acc < e.prob;
                const int slot = keep ? j : int(e.alt & 0x3fffffffu);
                const bool neg = keep ? (e.alt >> 31) != 0u : ((e.alt >> 30) & 1u) != 0u;
                nmode = slot + 3;
                nsign = neg ? -sign : sign;
            } else {
                const BoxProp bp = bprop[box];
                if (bp.c1) {
                    const long long off = (long long)col * nm;
                    const int im = lower_bound_abs_lirp(bp.c1 + off, bp.c2 + off, nm, g.uniform(), bp.T, bp.T1, bp.T2);
                    nmode = im + 3;
                    nsign = lirp_at(bp.c1 + off, bp.c2 + off, im, bp.T, bp.T1, bp.T2) > 0. ? sign : -sign;
                } else {
                    atomicCAS(err, 0, E_VALUE);  // a particle where nothing scatters
                }
            }
        }
        wo = __shfl_sync(0xffffffffu, wo, 0);
        if (act) {
            const long long o = (long long)wo + __popc(m1 & ((1u << lane) - 1u));
            if (o < ocap) {
                out.x[o] = x;
                out.y[o] = y;
                out.box[o] = box;
                out.mode[o] = nmode;
                out.sign[o] = nsign;
                atomicAdd(H + (long long)box * nmodes + nmode, nsign);
            } else {
                atomicCAS(err, 0, E_LIMIT);
            }
            --todo;
            if (!rta && nsign != sign) {
                todo += 2;
                ++flips;
            }
            if (++made >= BRANCH_CAP) {
                atomicCAS(err, 0, E_LIMIT);
                todo = 0;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) flips += __shfl_down_sync(0xffffffffu, flips, o);
    if (lane == 0 && flips) atomicAdd(dc + DC_FLIPS, flips);
}

// Exclusive scan of cnt[0..n) into descs[k].first, by one warp; returns the
// total.
__device__ unsigned long long warp_scan_first(const long long* cnt, int n, GenDesc* descs) {
    const int lane = threadIdx.x & 31;
    unsigned long long carry = 0;
    for (int b = 0; b < n; b += 32) {
        const int k = b + lane;
        unsigned long long v = k < n ? (unsigned long long)cnt[k] : 0ull;
        unsigned long long incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (k < n) descs[k].first = (long long)(carry + incl - v);
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    return carry;
}

// Claim `total` slots of the step's new particles at A[DC_NGEN..), within
// the capacity (a source that would overflow it sets BTE_ERR_LIMIT and
// makes nothing).
__device__ void claim_span(unsigned long long total, unsigned long long* dc, SrcSpan* span, long long cap,
                           int* err) {
    const unsigned long long base = dc[DC_NGEN];
    if ((long long)(base + total) > cap) {
        atomicCAS(err, 0, E_LIMIT);
        total = 0;
    }
    span->base = base;
    span->total = total;
    dc[DC_NGEN] = base + total;
}

// Particle numbers of the gradient and isothermal-wall sources of one step:
// Ntogenerate's stochastic rounding (src/sampling.cpp:166-183, :243-260) of
// the expected numbers genf[k], from one Philox block per source.  One warp.
__global__ void be_plan_sources(GenDesc* descs, const double* genf, long long* cnt, int ngen,
                                unsigned long long key, unsigned long long* dc, SrcSpan* span, long long cap,
                                int* err) {
    if (threadIdx.x >= 32) return;
    for (int k = threadIdx.x; k < ngen; k += 32) {
        Philox q;
        q.init(key, (uint64_t)k);
        const double gen = genf[k];
        long long c = (long long)gen;
        if (q.uniform() <= gen - floor(gen)) ++c;
        cnt[k] = c;
    }
    __syncwarp();
    const unsigned long long total = warp_scan_first(cnt, ngen, descs);
    if (threadIdx.x == 0) claim_span(total, dc, span, cap, err);
}

// A void border's adiabatic re-emission, tabulated per run: its segment,
// the inward normal, its box and the box's Teq, its length and the spline
// J(T) -> T of its wall (-1: not re-emitting: reservoirs, periodic boxes).
struct AdiBorder {
    double x0, y0, dx, dy, nx, ny, Teq, len;
    int box, spline, pad0, pad1;
};

// Natural cubic splines on the device (the host's Spline1D, the reference's
// CubicSpline1D src/interpolation.cpp:20-103): per spline `nk` intervals of
// coefficients a, b, c, d from x0, with the right ends xs for the search.
struct SplineDev {
    const double *a, *b, *c, *d, *x0, *xs;
    int nk;
};

__device__ __forceinline__ double spline_eval(const SplineDev& S, int id, double x) {
    const long long o = (long long)id * S.nk;
    int lo = 0, cnt = S.nk;  // lower_bound over xs
    while (cnt > 0) {
        const int st = cnt >> 1;
        if (S.xs[o + lo + st] < x) {
            lo += st + 1;
            cnt -= st + 1;
        } else {
            cnt = st;
        }
    }
    const int idx = lo >= S.nk ? S.nk - 1 : lo;
    const double dx = x - S.x0[o + idx];
    return S.a[o + idx] + dx * (S.b[o + idx] + dx * (S.c[o + idx] + S.d[o + idx] * dx));
}

// The adiabatic walls of one step (src/beyondRTA_MC2d.cpp:294-350): each
// re-emitting border re-emits |Eborder| particles at the temperature whose
// isothermal flux carries its absorbed energy (spline of J), one
// distribution request per border; Eborder starts again from zero.  One
// warp.
__global__ void be_plan_adiabatic(int* Eb, const AdiBorder* ab, int nborders, SplineDev S, double Eeff, double dtstep,
                                  double thickness, WallReq* req, long long* cnt, GenDesc* descs,
                                  unsigned long long* dc, SrcSpan* span, long long cap, int* err) {
    if (threadIdx.x >= 32) return;
    for (int k = threadIdx.x; k < nborders; k += 32) {
        const int E = Eb[k];
        Eb[k] = 0;
        const AdiBorder A = ab[k];
        long long c = 0;
        GenDesc d{};
        d.cdf = k;
        d.box = A.box >= 0 ? A.box : 0;
        if (A.spline >= 0 && E != 0) {
            const double Jb = Eeff * E / dtstep / (A.len * thickness);
            const double Tb = spline_eval(S, A.spline, Jb);
            req[k] = WallReq{A.nx, A.ny, Tb, A.Teq};
            d.x0 = A.x0;
            d.y0 = A.y0;
            d.dx = A.dx;
            d.dy = A.dy;
            d.sign = (Tb - A.Teq) >= 0 ? 1 : -1;
            c = (long long)(fabs((double)E) + 1.0e-6);
        }
        cnt[k] = c;
        d.first = 0;
        descs[k] = d;
    }
    __syncwarp();
    const unsigned long long total = warp_scan_first(cnt, nborders, descs);
    if (threadIdx.x == 0) claim_span(total, dc, span, cap, err);
}

// New particles of one planned source at A[span.base + k), k < span.total,
// each advected for a random part of the step as it is made (the sources
// of steps 2-4 of the reference's loop); an absorbed one keeps mode -1.
__global__ void be_generate_dev(PArr P, const SrcSpan* span, const GenDesc* gens, int ngen, const float* aprob,
                                const int* aalt, const signed char* asign, const double* cdfs,
                                const double* cdftot, int nmodes, unsigned long long key, const GBox* boxes,
                                const V2* hull, AdvectArgs aa) {
    const SrcSpan sp = *span;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < (long long)sp.total;
         k += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = ngen;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (gens[mid].first <= k) lo = mid; else hi = mid;
        }
        const GenDesc gd = gens[lo];
        Philox g;
        g.init(key, (uint64_t)k);
        double x, y;
        bool placed = true;
        if (gd.rect == 2) {
            const GBox& Bx = boxes[gd.box];
            placed = false;
            for (int tries = 0; tries < 100000 && !placed; ++tries) {
                x = gd.x0 + g.uniform() * gd.dx;
                y = gd.y0 + g.uniform() * gd.dy;
                placed = inside_hull(hull + Bx.hull_off, Bx.nhull, v2(x, y));
            }
        } else if (gd.rect) {
            x = gd.x0 + g.uniform() * gd.dx;
            y = gd.y0 + g.uniform() * gd.dy;
        } else {
            const double u = g.uniform();
            x = gd.x0 + u * gd.dx;
            y = gd.y0 + u * gd.dy;
        }
        int mode;
        if (gd.cdf >= 0) {
            const double* row = cdfs + (long long)gd.cdf * nmodes;
            mode = cdftot[gd.cdf] > 0. ? lower_bound_d(row, nmodes, g.uniform()) : -1;
            if (mode >= nmodes) mode = nmodes - 1;
            if (!placed) mode = -1;
        } else {
            const float* pr = aprob + gd.alias_off;
            const int* al = aalt + gd.alias_off;
            const int j = int(mulhi32(g.next32(), uint32_t(nmodes)));
            const float acc = float(g.next32() >> 8) * 0x1p-24f;
            mode = acc < __ldg(pr + j) ? j : __ldg(al + j);
        }
        int box = gd.box;
        const int sign = (gd.msign && mode >= 0) ? int(__ldg(asign + gd.alias_off + mode)) : gd.sign;
        const long long i = (long long)sp.base + k;
        if (mode >= 0) {  // a random part of the step
            Philox h;
            h.init(aa.key, (uint64_t)i);
            const double dt = aa.dt * h.uniform();
            bool alive;
            if (aa.general) {
                BePol pol;
                pol.g.init(aa.gkey, (uint64_t)i);
                int e = 0;
                alive = advect_general(aa.T, pol, aa.Eb, x, y, box, mode, sign, dt, e);
                if (e && aa.err) atomicCAS(aa.err, 0, e);
            } else {
                alive = advect_one(aa.G, aa.boxcell, aa.mv, aa.boxwall, aa.Eb, x, y, box, mode, sign, dt);
            }
            if (!alive) mode = -1;
        }
        P.x[i] = x;
        P.y[i] = y;
        P.box[i] = box;
        P.mode[i] = mode;
        P.sign[i] = sign;
    }
}

// The wall-CDF passes over every border, for the borders the step planned
// (cnt > 0); rows of the others are left as they are.
__global__ void __launch_bounds__(256) be_wall_cdf1_dev(const float* om, const float* vx, const float* vy, int n,
                                                        const WallReq* req, const long long* cnt, double* cdf,
                                                        double* chunk_tot) {
    const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
    if (cnt[blockIdx.x / nch] == 0) return;
    wall_cdf1_body(om, vx, vy, n, req, cdf, chunk_tot);
}
__global__ void __launch_bounds__(256) be_wall_cdf2_dev(int n, const long long* cnt, const double* chunk_tot,
                                                        double* cdf, double* tot) {
    const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
    if (cnt[blockIdx.x / nch] == 0) return;
    wall_cdf2_body(n, chunk_tot, cdf, tot);
}

// Cancellation on the device over [0, *n_in) with the random affine
// visiting order drawn from `key` (a coprime to n).
__device__ __forceinline__ unsigned long long gcd_u64(unsigned long long a, unsigned long long b) {
    while (b) {
        const unsigned long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}
__global__ void be_cancel_dev(PArr P, const unsigned long long* n_in, long long cap, const int* H, int* cnt,
                              int nmodes,
                              const int* reservoir, unsigned long long key) {
    const long long n = min((long long)*n_in, cap);
    if (n <= 0) return;
    // the permutation's a, b and the XOR key, drawn by one thread per block
    __shared__ unsigned long long s_ab[2];
    __shared__ unsigned s_mkey;
    if (threadIdx.x == 0) {
        const unsigned long long nch = (unsigned long long)((n + 31) >> 5);
        Philox q;
        q.init(key, 0);
        unsigned long long pa = ((unsigned long long)q.next32() << 32 | q.next32()) % nch;
        const unsigned long long pb = ((unsigned long long)q.next32() << 32 | q.next32()) % nch;
        if (pa == 0) pa = 1;
        for (int t = 0; t < 64 && gcd_u64(nch, pa) != 1ull; ++t) pa = pa + 1 < nch ? pa + 1 : 1;
        if (gcd_u64(nch, pa) != 1ull) pa = 1;  // 1 is coprime to every nch
        s_ab[0] = pa;
        s_ab[1] = pb;
        s_mkey = q.next32();
    }
    __syncthreads();
    cancel_body(P, n, H, cnt, nmodes, reservoir, s_ab[0], s_ab[1], s_mkey);
}

// Compaction of [0, *n_in) with the survivors counted into *count.
__global__ void be_compact_dev(PArr in, const unsigned long long* n_in, long long cap, PArr out,
                               unsigned long long* count) {
    compact_body(in, min((long long)*n_in, cap), out, count);
}

// dc[to] = dc[from]; record[step] = dc[DC_NP] after it.
__global__ void be_counters(unsigned long long* dc, int to, int from, long long* record, int step) {
    if (to >= 0) dc[to] = dc[from];
    if (record) {  // the end of a step: its particles alive, and the outputs of its be_advance launches
        record[step] = (long long)dc[DC_NP];
        dc[DC_OUTT] += dc[DC_NOUT];
    }
}

PArr arr(DBuf& x, DBuf& y, DBuf& m, DBuf& b, DBuf& s, long long off = 0) {
    return PArr{x.as<double>() + off, y.as<double>() + off, m.as<int>() + off, b.as<int>() + off,
                s.as<int>() + off};
}

void alloc_particles(BertaState& B, long long cap) {
    if (B.cap >= cap) return;
    for (DBuf* d : {&B.a_x, &B.a_y, &B.b_x, &B.b_y})
        d->alloc(size_t(cap) * sizeof(double));
    for (DBuf* d : {&B.a_mode, &B.a_box, &B.a_sign, &B.b_mode, &B.b_box, &B.b_sign})
        d->alloc(size_t(cap) * sizeof(int));
    B.cap = cap;
}

unsigned long long mix_key(unsigned long long seed, long long step, int phase) {
    unsigned long long k = seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(step + 1));
    k ^= (unsigned long long)phase << 56;
    return k;
}

int launch_blocks(long long n, int nsm) {
    long long b = (n + 255) / 256;
    const long long cap = (long long)nsm * 8;
    if (b > cap) b = cap;
    return int(b < 1 ? 1 : b);
}

}  // namespace

// Natural cubic spline (CubicSpline1D, src/interpolation.cpp:20-103).
void Spline1D::build(const std::vector<double>& X, const std::vector<double>& Y) {
    const int n = int(Y.size()) - 1;
    const std::size_t N = static_cast<std::size_t>(n);
    std::vector<double> A(Y), Bv(N), D(N), h(N), alpha(N), C(N + 1), l(N + 1), mu(N + 1), z(N + 1);
    for (std::size_t i = 0; i < N; i++) h[i] = X[i + 1] - X[i];
    for (std::size_t i = 1; i < N; i++)
        alpha[i] = 3. / h[i] * (A[i + 1] - A[i]) - 3. / h[i - 1] * (A[i] - A[i - 1]);
    l[0] = 1;
    mu[0] = 0;
    z[0] = 0;
    for (std::size_t i = 1; i < N; i++) {
        l[i] = 2 * (X[i + 1] - X[i - 1]) - h[i - 1] * mu[i - 1];
        mu[i] = h[i] / l[i];
        z[i] = (alpha[i] - h[i - 1] * z[i - 1]) / l[i];
    }
    l[N] = 1;
    z[N] = 0;
    C[N] = 0;
    for (int jj = n - 1; jj >= 0; jj--) {
        const std::size_t k = std::size_t(jj);
        C[k] = z[k] - mu[k] * C[k + 1];
        Bv[k] = (A[k + 1] - A[k]) / h[k] - h[k] * (C[k + 1] + 2 * C[k]) / 3;
        D[k] = (C[k + 1] - C[k]) / (3 * h[k]);
    }
    a.assign(A.begin(), A.begin() + n);
    b = Bv;
    c.assign(C.begin(), C.begin() + n);
    d = D;
    x0.assign(X.begin(), X.begin() + n);
    xs.assign(X.begin() + 1, X.end());
}

double Spline1D::interp(double x) const {
    std::size_t idx = std::size_t(std::lower_bound(xs.begin(), xs.end(), x) - xs.begin());
    if (idx >= a.size()) idx--;
    const double dx = x - x0[idx];
    return a[idx] + dx * (b[idx] + dx * (c[idx] + d[idx] * dx));
}

}  // namespace bte

using bte::Error;

extern "C" bte_status bte_load_propagator(bte_ctx* c, const bte_propagator* P) {
    if (!c) return BTE_ERR_INPUT;
    try {
        if (!P || !P->P || P->nmodes < 1) throw Error(BTE_ERR_INPUT, "empty propagator");
        if (!c->have_modes) throw Error(BTE_ERR_STATE, "load the mode table before the propagator");
        if (std::size_t(P->nmodes) + 3 != c->modes.n())
            throw Error(BTE_ERR_INPUT, "propagator size must be the number of modes minus 3");
        if (!std::isfinite(P->T) || !(P->T > 0.)) throw Error(BTE_ERR_INPUT, "propagator temperature must be positive");
        if (!c->berta) c->berta = new bte::BertaState();
        bte::BertaState& B = *c->berta;
        const int nm = P->nmodes;
        if (B.have_prop && nm != B.nm) B.props.clear();  // another mode table
        const std::size_t nn = std::size_t(nm) * std::size_t(nm);
        for (std::size_t i = 0; i < nn; ++i)
            if (!std::isfinite(P->P[i])) throw Error(BTE_ERR_VALUE, "non-finite propagator entry");
        B.props[P->T].assign(P->P, P->P + nn);
        B.props_version++;
        B.nm = nm;
        B.T = P->T;
        B.have_prop = true;
        return BTE_OK;
    } catch (const Error& e) {
        c->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_CUDA;
    }
}

namespace {

// signed_cumm of propagator_H (src/collision_operator.cpp:857-870) for every
// column of the column-major nm x nm P: running sums of |P| over the column
// sum, each with the sign of its entry.
std::vector<double> signed_cumm(const std::vector<double>& P, int nm) {
    std::vector<double> c(P.size());
    for (int j = 0; j < nm; ++j) {
        const double* col = P.data() + std::size_t(j) * nm;
        double abssum = 0.;
        for (int i = 0; i < nm; ++i) abssum += std::fabs(col[i]);
        double acc = 0.;
        for (int i = 0; i < nm; ++i) {
            acc += std::fabs(col[i]);
            c[std::size_t(j) * nm + i] = col[i] < 0. ? -acc / abssum : acc / abssum;
        }
    }
    return c;
}

// The alias table of a propagator over |P| per column, with the signs of
// the slot and of its alias in the alias word.
std::vector<bte::PAlias> propagator_alias(const std::vector<double>& P, int nm) {
    using namespace bte;
    const std::size_t nn = std::size_t(nm) * std::size_t(nm);
    std::vector<PAlias> tab(nn);
    std::vector<double> w(static_cast<std::size_t>(nm));
    std::vector<Alias> al(static_cast<std::size_t>(nm));
    for (int j = 0; j < nm; ++j) {
        const double* col = P.data() + std::size_t(j) * nm;
        for (int i = 0; i < nm; ++i) w[std::size_t(i)] = std::fabs(col[i]);
        alias_table(w.data(), nm, al.data());
        for (int i = 0; i < nm; ++i) {
            PAlias e;
            e.prob = al[std::size_t(i)].prob;
            const int alt = al[std::size_t(i)].alt;
            e.alt = unsigned(alt) | (col[alt] < 0. ? (1u << 30) : 0u) | (col[i] < 0. ? (1u << 31) : 0u);
            tab[std::size_t(j) * nm + std::size_t(i)] = e;
        }
    }
    return tab;
}

// The scattering table of every box at its Teq (Scattering,
// src/beyondRTA_MC2d.cpp:1130-1165): the tabulated propagator when Teq is in
// the table, sampled through per-column alias tables; otherwise lirp
// (src/collision_operator.cpp:918-929) between the first tabulated
// temperature above Teq and the next one -- both above Teq, as the
// reference picks them -- sampled through the signed CDFs interpolated on
// the fly.  Uploads the per-box BoxProp records; returns the alias table
// every scattering box uses when they all use the same one, else null.
const bte::PAlias* select_box_propagators(bte_ctx* c, bte::BertaState& B, const bte::HostGeometry& g) {
    using namespace bte;
    if (B.dev_version != B.props_version) {
        B.dev_alias.clear();
        B.dev_cdf.clear();
        B.dev_version = B.props_version;
    }
    const int nm = B.nm;
    auto alias_of = [&](double T) -> const PAlias* {
        DBuf& d = B.dev_alias[T];
        if (!d.p) d.upload(propagator_alias(B.props.at(T), nm), c->stream);
        return d.as<PAlias>();
    };
    auto cdf_of = [&](double T) -> const double* {
        DBuf& d = B.dev_cdf[T];
        if (!d.p) d.upload(signed_cumm(B.props.at(T), nm), c->stream);
        return d.as<double>();
    };
    const std::size_t nbx = g.boxes.size();
    std::vector<BoxProp> bp(nbx, BoxProp{nullptr, nullptr, nullptr, 0., 0., 0.});
    const PAlias* uniform = nullptr;
    bool same = true, any = false;
    const double Tlow = B.props.begin()->first;
    for (std::size_t b = 0; b < nbx; ++b) {
        if (g.reservoir[b] || g.tto[b] >= 0) continue;
        const double Teq = g.Teq[b];
        BoxProp& r = bp[b];
        r.T = Teq;
        if (B.props.count(Teq)) {
            r.alias = alias_of(Teq);
        } else {
            const auto m1 = B.props.lower_bound(Teq);
            if (m1 == B.props.end() || std::next(m1) == B.props.end() || Teq < Tlow)
                throw Error(BTE_ERR_INPUT,
                            "Extrapolation is not allowed: limit Tref between the min and max temperatures "
                            "used in the propagator calculation");
            const auto m2 = std::next(m1);
            r.T1 = m1->first;
            r.T2 = m2->first;
            r.c1 = cdf_of(r.T1);
            r.c2 = cdf_of(r.T2);
        }
        if (!any) uniform = r.alias;
        else if (r.alias != uniform) same = false;
        any = true;
    }
    B.d_boxprop.upload(bp, c->stream);
    sync(c);
    return same ? uniform : nullptr;
}

std::size_t n_to_generate(double gen, bte::Pcg64& rng) {
    std::size_t np = std::size_t(gen);
    if (bte::canonical_from(rng.next()) <= gen - std::floor(gen)) np++;
    return np;
}

// Isothermal_wall_distribution pmf for normal n (src/sampling.cpp:189-269);
// returns cumulsum = 1e12 hbar sum(pmf).
double wall_pmf(const bte::HostModes& m, bte::V2 n, double Tw, double Te, std::vector<double>& pmf) {
    pmf.assign(m.n(), 0.);
    for (std::size_t k = 0; k < m.n(); ++k) {
        const double vn = n.x * m.vx[k] + n.y * m.vy[k] + 0. * m.vz[k];
        if (vn <= 0. || bte::almost_equal(0., m.omega[k]))
            pmf[k] = 0.;
        else
            pmf[k] = vn * m.omega[k] *
                     std::fabs(bte::bose_einstein(m.omega[k], Tw) - bte::bose_einstein(m.omega[k], Te));
    }
    double s = 0.;
    for (double x : pmf) s += x;
    return 1.0e+12 * 1.054571726e-34 * s;
}

[[noreturn]] void throw_step_error(int e) {
    throw Error(bte_status(e), e == BTE_ERR_LIMIT      ? "particle capacity or step cap exceeded"
                               : e == BTE_ERR_GEOMETRY ? "geometry error in the advection"
                                                       : "particle without a propagator column");
}

}  // namespace

extern "C" bte_status bte_berta_run(bte_ctx* c, const bte_berta_params* p, bte_berta_result* out) {
    using namespace bte;
    if (!c || !p || !out) return BTE_ERR_INPUT;
    const auto t_start = std::chrono::steady_clock::now();
    try {
        if (!(p->dt > 0.) || !(p->maxtime >= 0.) || !(p->Eeff > 0.) || !(p->T0 > 0.))
            throw Error(BTE_ERR_INPUT, "dt, Eeff and T0 must be positive and maxtime >= 0");
        if (p->mode != BTE_MODE_PRODUCTION)
            throw Error(BTE_ERR_INPUT, "beyond-RTA runs support the production mode only");
        if (!c->have_modes || !c->have_geom) throw Error(BTE_ERR_STATE, "load modes and geometry first");
        if (!p->rta && (!c->berta || !c->berta->have_prop))
            throw Error(BTE_ERR_STATE, "load a propagator (or set rta) before a beyond-RTA run");
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        ensure_static(c);
        const HostModes& m = c->modes;
        const HostGeometry& g = c->geom;
        if (c->nmat > 0) throw Error(BTE_ERR_INPUT, "materials are for transient batched runs");
        // RTA scattering uses the mode table's rates, given at T0 only: every
        // box that scatters needs Teq = T0.  With the propagator each box
        // scatters at its own Teq.
        if (p->rta)
            for (std::size_t b = 0; b < g.boxes.size(); ++b)
                if (!g.reservoir[b] && g.tto[b] < 0 && g.Teq[b] != p->T0)
                    throw Error(BTE_ERR_INPUT, "RTA scattering needs Teq = T0 in every box (rates at T0 only)");
        if (p->gradient_mode != 0 && p->gradient_mode != 1) throw Error(BTE_ERR_INPUT, "bad gradient_mode");
        if (p->gradient_mode == 1 && !(std::isfinite(p->gradient[0]) && std::isfinite(p->gradient[1])))
            throw Error(BTE_ERR_INPUT, "gradient must be finite");
        const PAlias* pal = nullptr;
        if (p->rta) ensure_resample(c, p->T0);
        else pal = select_box_propagators(c, *c->berta, g);
        if (!c->berta) c->berta = new BertaState();
        BertaState& B = *c->berta;
        const int n = int(m.n());
        const int nbx = int(g.boxes.size());
        const int nborders = int(g.borders.size());
        const double vuc = m.V * g.thickness / m.c;
        cudaStream_t s = c->stream;
        // walls of each box: global border index of its +x, -x, +y, -y border
        std::vector<int4> boxwall(std::size_t(nbx), make_int4(-1, -1, -1, -1));
        for (int b = 0; b < nbx; ++b) {
            const GBox& bx = g.boxes[std::size_t(b)];
            for (int k = 0; k < bx.nborders; ++k) {
                const V2 np = g.borders[std::size_t(bx.border_off + k)].np;
                const int gb = bx.border_off + k;
                if (np.x == 1. && np.y == 0.) boxwall[std::size_t(b)].x = gb;
                if (np.x == -1. && np.y == 0.) boxwall[std::size_t(b)].y = gb;
                if (np.x == 0. && np.y == 1.) boxwall[std::size_t(b)].z = gb;
                if (np.x == 0. && np.y == -1.) boxwall[std::size_t(b)].w = gb;
            }
        }
        std::vector<int> border_box(std::size_t(nborders), -1);
        for (int b = 0; b < nbx; ++b)
            for (int k = 0; k < g.boxes[std::size_t(b)].nborders; ++k)
                border_box[std::size_t(g.boxes[std::size_t(b)].border_off + k)] = b;
        B.d_boxwall.upload(boxwall, s);
        B.d_Eb.alloc(std::size_t(nborders) * sizeof(int));
        // per-step buffers at their largest size (one request per border),
        // so that no step reallocates
        B.d_req.alloc(std::size_t(nborders) * sizeof(WallReq));
        B.d_cdf.alloc(std::size_t(nborders) * std::size_t(m.n()) * sizeof(double));
        B.d_cdftot.alloc(std::size_t(nborders) * sizeof(double));
        B.d_ctot.alloc(std::size_t(nborders) * ((m.n() + WCDF_CHUNK - 1) / WCDF_CHUNK) * sizeof(double));
        ck(cudaMemsetAsync(B.d_Eb.p, 0, std::size_t(nborders) * sizeof(int), s), "memset");
        if (int(B.spl.size()) != nborders || B.spl_version != c->tables_version) {
            B.spl.assign(std::size_t(nborders), Spline1D());
            B.spl_ok.assign(std::size_t(nborders), 0);
            B.spl_version = c->tables_version;
        }
        B.d_rvx.upload(m.vx, s);
        B.d_rvy.upload(m.vy, s);
        B.d_H.alloc(std::size_t(nbx) * n * sizeof(int));
        B.d_cnt.alloc(std::size_t(nbx) * n * sizeof(int));
        B.d_props.alloc(std::size_t(nbx) * 3 * sizeof(double));
        c->d_err.alloc(4 * sizeof(int));
        ck(cudaMemsetAsync(c->d_err.p, 0, 4 * sizeof(int), s), "memset");
        std::vector<int> hres(g.reservoir.begin(), g.reservoir.end());
        DBuf d_res;
        d_res.upload(hres, s);
        const long long cap = p->capacity > 0 ? p->capacity : (1ll << 24);
        alloc_particles(B, cap);
        // sources: isothermal walls (static tables) and the initial deviation
        Generators iso;
        try {
            iso = build_wall_generators(m, g);
        } catch (const Error&) {
            iso = Generators();
        }
        Generators ini;
        bool have_ini = false;
        try {
            ini = build_initial_generators(m, g);
            have_ini = true;
        } catch (const Error&) {
            have_ini = false;
        }
        std::vector<std::pair<int, int>> cellof(std::size_t(nbx), {-1, -1});
        for (int i = 0; i < g.gnx; ++i)
            for (int j = 0; j < g.gny; ++j) {
                const int v = g.gcell[std::size_t(i) * g.gny + j];
                const int b = v >= 0 ? v : (v <= -2 ? -2 - v : -1);
                if (b >= 0) cellof[std::size_t(b)] = {i, j};
            }
        Pcg64 rng;
        rng.seed(p->seed, 0);
        const GridArgs GA = [&] {
            GridArgs A{};
            A.G.nx = g.gnx;
            A.G.ny = g.gny;
            A.G.gx = c->d_gx.as<double>();
            A.G.gy = c->d_gy.as<double>();
            A.G.cell = c->d_gcell.as<int>();
            A.boxcell = c->d_boxcell.as<int2>();
            A.mv = c->d_mv.as<ModeVel>();
            return A;
        }();
        int* err = c->d_err.as<int>();
        // convex-box tables for geometries that are not a grid (or have
        // periodic boxes)
        const int general = g.rect_grid ? 0 : 1;
        DevTables TT{};
        fill_static_tables(c, TT);
        std::vector<float> aprob;
        std::vector<int> aalt;
        std::vector<GenDesc> descs;
        B.d_gens.alloc(std::size_t(std::max({nborders, nbx, int(iso.walls.size())}) + 1) * sizeof(GenDesc));
        // a source spread over box b: its grid cell, or its bounding box with
        // rejection (geometry_2d::get_random_point)
        auto box_desc = [&](int b) {
            GenDesc d{};
            if (g.rect_grid) {
                const auto ij = cellof[std::size_t(b)];
                d.x0 = g.gx[std::size_t(ij.first)];
                d.dx = g.gx[std::size_t(ij.first) + 1] - d.x0;
                d.y0 = g.gy[std::size_t(ij.second)];
                d.dy = g.gy[std::size_t(ij.second) + 1] - d.y0;
                d.rect = 1;
            } else {
                const GBox& bx = g.boxes[std::size_t(b)];
                double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
                for (int h = 0; h < bx.nhull; ++h) {
                    const V2 q = g.hull[std::size_t(bx.hull_off + h)];
                    x0 = std::min(x0, q.x);
                    x1 = std::max(x1, q.x);
                    y0 = std::min(y0, q.y);
                    y1 = std::max(y1, q.y);
                }
                d.x0 = x0;
                d.dx = x1 - x0;
                d.y0 = y0;
                d.dy = y1 - y0;
                d.rect = 2;
            }
            d.box = b;
            d.cdf = -1;
            return d;
        };
        // the gradient source term (source_term_gradient,
        // src/beyondRTA_MC2d.cpp:597-676): a homogeneous <gradient> on every
        // box that is neither a reservoir nor periodic, or the least-squares
        // gradients of the boxes' Teq (calculate_gradientT, the reference's
        // default, src/beyondRTA_MC2d.cpp:1441-1458); Nabla_T rows at each
        // box's Teq for the boxes with a gradient, built once as the
        // reference's static generators are
        GradGenerators grad = p->gradient_mode == 1
                                  ? build_gradient_generators(m, g, p->gradient[0], p->gradient[1])
                                  : build_gradient_generators_boxes(m, g, calculate_gradientT(g));
        if (!grad.box.empty()) {
            std::vector<float> gp(grad.alias.size());
            std::vector<int> ga(grad.alias.size());
            for (std::size_t i = 0; i < grad.alias.size(); ++i) {
                gp[i] = grad.alias[i].prob;
                ga[i] = grad.alias[i].alt;
            }
            B.d_gprob.upload(gp, s);
            B.d_galt.upload(ga, s);
            B.d_gsign.upload(grad.sign, s);
        }
        // generate the sources in `descs` (alias rows in aprob/aalt) at A[base..)
        // the isothermal walls' alias rows do not change during a run
        {
            std::vector<float> ip(iso.alias.size());
            std::vector<int> ia(iso.alias.size());
            for (std::size_t i = 0; i < iso.alias.size(); ++i) {
                ip[i] = iso.alias[i].prob;
                ia[i] = iso.alias[i].alt;
            }
            B.d_isoprob.upload(ip, s);
            B.d_isoalt.upload(ia, s);
            // FP32 copies for the adiabatic walls' pmf (omega = 0 where
            // almost_equal(0, omega): those modes take no part)
            std::vector<float> omf(m.omega.size()), vxf(m.omega.size()), vyf(m.omega.size());
            for (std::size_t k = 0; k < omf.size(); ++k) {
                omf[k] = almost_equal(0., m.omega[k]) ? 0.f : float(m.omega[k]);
                vxf[k] = float(m.vx[k]);
                vyf[k] = float(m.vy[k]);
            }
            B.d_om.upload(omf, s);
            B.d_vx.upload(vxf, s);
            B.d_vy.upload(vyf, s);
        }
        // generate the sources in `descs` at A[base..): alias rows from
        // aprob/aalt (uploaded here) or from a table already on the device
        // (rprob/ralt, with per-mode signs rsign), CDF rows from B.d_cdf
        // the initial deviation's particles (descs, alias rows aprob/aalt) at A[base..)
        auto generate = [&](long long base, long long total, long long step, int phase) {
            if (total <= 0) return;
            if (base + total > cap) throw Error(BTE_ERR_LIMIT, "particle capacity exceeded: raise capacity");
            upload_pinned(B.d_gens, B.h_gens[0], descs, s);
            const float* dprob = nullptr;
            const int* dalt = nullptr;
            if (!aprob.empty()) {
                B.d_alias.alloc(aprob.size() * sizeof(float) + aalt.size() * sizeof(int));
                ck(cudaMemcpyAsync(B.d_alias.p, aprob.data(), aprob.size() * sizeof(float), cudaMemcpyHostToDevice, s), "h2d");
                int* a2 = reinterpret_cast<int*>(B.d_alias.as<char>() + aprob.size() * sizeof(float));
                ck(cudaMemcpyAsync(a2, aalt.data(), aalt.size() * sizeof(int), cudaMemcpyHostToDevice, s), "h2d");
                dprob = B.d_alias.as<float>();
                dalt = a2;
            }
            PArr A = arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign);
            be_generate<<<launch_blocks(total, c->nsm), 256, 0, s>>>(
                A, base, total, B.d_gens.as<GenDesc>(), int(descs.size()), dprob, dalt, nullptr,
                B.d_cdf.as<double>(), B.d_cdftot.as<double>(), n, mix_key(p->seed, step, phase),
                c->d_boxes.as<GBox>(), c->d_hull.as<V2>());
        };
        std::vector<double> hprops(std::size_t(nbx) * 3);
        std::vector<double> vol(static_cast<std::size_t>(nbx));
        for (int b = 0; b < nbx; ++b) vol[std::size_t(b)] = g.boxes[std::size_t(b)].area * g.thickness;
        auto props = [&](long long nn, int sidx) {
            ck(cudaMemsetAsync(B.d_H.p, 0, std::size_t(nbx) * n * sizeof(int), s), "memset");
            if (nn > 0)
                be_hist<<<launch_blocks(nn, c->nsm), 256, 0, s>>>(arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign),
                                                                  nn, B.d_H.as<int>(), n);
            be_props<<<nbx, 256, 0, s>>>(B.d_H.as<int>(), n, B.d_rvx.as<double>(), B.d_rvy.as<double>(),
                                          B.d_props.as<double>());
            ck(cudaMemcpyAsync(hprops.data(), B.d_props.p, hprops.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "d2h");
            sync(c);
            for (int b = 0; b < nbx; ++b) {
                const double f1 = p->Eeff / vol[std::size_t(b)] * 1.0e+27;
                const double f2 = p->Eeff / vol[std::size_t(b)] * 1.0e+30;
                if (out->ed) out->ed[std::size_t(sidx) * nbx + b] = f1 * hprops[3 * std::size_t(b)];
                if (out->flux) {
                    out->flux[(std::size_t(sidx) * nbx + b) * 2] = f2 * hprops[3 * std::size_t(b) + 1];
                    out->flux[(std::size_t(sidx) * nbx + b) * 2 + 1] = f2 * hprops[3 * std::size_t(b) + 2];
                }
            }
            if (out->nparticles) out->nparticles[sidx] = nn;
        };
        ck(cudaEventRecord(c->ev0, s), "event");
        // initial deviation (init_particles, src/beyondRTA_MC2d.cpp:211-269)
        long long np = 0;
        descs.clear();
        aprob.clear();
        aalt.clear();
        if (have_ini) {
            long long first = 0;
            for (std::size_t k = 0; k < ini.init_box.size(); ++k) {
                const long long cnt = (long long)n_to_generate(ini.init_energy[k] / p->Eeff, rng);
                if (cnt == 0) continue;
                const int b = ini.init_box[k];
                GenDesc d = box_desc(b);
                d.sign = ini.init_sign[k];
                d.cdf = -1;
                const long long off = (long long)aprob.size();
                for (std::size_t q = 0; q < std::size_t(n); ++q) {
                    aprob.push_back(ini.alias[k * std::size_t(n) + q].prob);
                    aalt.push_back(ini.alias[k * std::size_t(n) + q].alt);
                }
                d.alias_off = off;
                d.first = first;
                descs.push_back(d);
                first += cnt;
            }
            generate(0, first, -1, 0);
            np = first;
        }
        props(np, 0);
        long long psteps = 0, branchings = 0, adv_in = 0, adv_out = 0;
        // ---- the step loop, resident on the device: particle numbers stay in
        // device counters, the sources are planned on the device, and the
        // step's properties are recorded there; the host synchronises only
        // when a per-step hook asks for each step's histogram
        int nsteps = 0;
        for (double t = 0.; t <= p->maxtime; t += p->dt) ++nsteps;
        B.d_dc.alloc(DC_COUNT * sizeof(unsigned long long));
        auto* dc = B.d_dc.as<unsigned long long>();
        B.d_span.alloc(3 * sizeof(SrcSpan));
        SrcSpan* span = B.d_span.as<SrcSpan>();
        {
            std::vector<unsigned long long> h0(DC_COUNT, 0ull);
            h0[DC_NP] = (unsigned long long)np;
            B.d_dc.upload(h0, s);
        }
        B.d_phist.alloc(std::size_t(nsteps + 1) * std::size_t(nbx) * 3 * sizeof(double));
        B.d_nhist.alloc(std::size_t(nsteps + 1) * sizeof(long long));
        // sources with fixed descriptors: gradient boxes and isothermal walls,
        // with the expected particle numbers of a step
        std::vector<GenDesc> gdesc, idesc;
        std::vector<double> ggenf, igenf;
        for (std::size_t k = 0; k < grad.box.size(); ++k) {
            GenDesc d = box_desc(grad.box[k]);
            d.alias_off = (long long)k * n;
            d.msign = 1;
            gdesc.push_back(d);
            ggenf.push_back(p->dt * grad.energy[k] / p->Eeff);
        }
        for (std::size_t k = 0; k < iso.walls.size(); ++k) {
            const WallGenerator& W = iso.walls[k];
            const double Lb = norm(sub(W.sb, W.sa));
            const double spf = Lb * g.thickness / (m.V * g.thickness / m.c);
            const double cumulsum = std::fabs(W.flux) * double(m.nq) * vuc;
            GenDesc d{};
            d.x0 = W.p1.x;
            d.y0 = W.p1.y;
            d.dx = W.nd.x;
            d.dy = W.nd.y;
            d.box = W.box;
            d.sign = W.sign;
            d.cdf = -1;
            d.alias_off = (long long)k * n;
            idesc.push_back(d);
            igenf.push_back(p->dt * spf * cumulsum / (p->Eeff * double(m.nq)));
        }
        const int ngd = int(gdesc.size()), nid = int(idesc.size());
        if (ngd) {
            B.d_gdesc.upload(gdesc, s);
            B.d_ggenf.upload(ggenf, s);
            B.d_gcnt.alloc(std::size_t(ngd) * sizeof(long long));
        }
        if (nid) {
            B.d_idesc.upload(idesc, s);
            B.d_igenf.upload(igenf, s);
            B.d_icnt.alloc(std::size_t(nid) * sizeof(long long));
        }
        // adiabatic re-emission per void border: segment, inward normal, Teq
        // and the J(T) -> T spline of its wall (one per normal and Teq)
        std::vector<AdiBorder> adi(static_cast<std::size_t>(nborders));
        std::vector<double> sa, sb, sc, sd, sx0, sxs;
        std::map<std::tuple<double, double, double>, int> spline_of;
        int spl_nk = 0;
        std::vector<double> pmf;
        for (int gb = 0; gb < nborders; ++gb) {
            AdiBorder& A = adi[std::size_t(gb)];
            const int b = border_box[std::size_t(gb)];
            const GBorder& br = g.borders[std::size_t(gb)];
            A.x0 = br.p1.x;
            A.y0 = br.p1.y;
            A.dx = br.nd.x;
            A.dy = br.nd.y;
            A.nx = -br.np.x;
            A.ny = -br.np.y;
            A.len = norm(sub(br.p2, br.p1));
            A.box = b;
            A.spline = -1;
            if (b < 0 || g.reservoir[std::size_t(b)] || g.tto[std::size_t(b)] >= 0) continue;
            const double Teq = g.Teq[std::size_t(b)];
            A.Teq = Teq;
            const auto key = std::make_tuple(A.nx, A.ny, Teq);
            auto it = spline_of.find(key);
            if (it == spline_of.end()) {
                std::vector<double> J(100), Tv(100);
                for (int t = 0; t < 100; ++t) {
                    const double T = 10.0 + 10.0 * t;
                    Tv[std::size_t(t)] = T;
                    const double cs = wall_pmf(m, v2(A.nx, A.ny), T, Teq, pmf);
                    J[std::size_t(t)] = ((T - Teq) >= 0 ? 1 : -1) * (cs / (double(m.nq) * vuc));
                }
                Spline1D sp;
                sp.build(J, Tv);
                spl_nk = int(sp.a.size());
                sa.insert(sa.end(), sp.a.begin(), sp.a.end());
                sb.insert(sb.end(), sp.b.begin(), sp.b.end());
                sc.insert(sc.end(), sp.c.begin(), sp.c.end());
                sd.insert(sd.end(), sp.d.begin(), sp.d.end());
                sx0.insert(sx0.end(), sp.x0.begin(), sp.x0.end());
                sxs.insert(sxs.end(), sp.xs.begin(), sp.xs.end());
                it = spline_of.emplace(key, int(spline_of.size())).first;
            }
            A.spline = it->second;
        }
        B.d_adi.upload(adi, s);
        B.d_adesc.alloc(std::size_t(nborders) * sizeof(GenDesc));
        B.d_acnt.alloc(std::size_t(nborders) * sizeof(long long));
        SplineDev SP{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, spl_nk};
        if (!sa.empty()) {
            B.d_sa.upload(sa, s);
            B.d_sb.upload(sb, s);
            B.d_sc.upload(sc, s);
            B.d_sd.upload(sd, s);
            B.d_sx0.upload(sx0, s);
            B.d_sxs.upload(sxs, s);
            SP = SplineDev{B.d_sa.as<double>(), B.d_sb.as<double>(), B.d_sc.as<double>(), B.d_sd.as<double>(),
                           B.d_sx0.as<double>(), B.d_sxs.as<double>(), spl_nk};
        }
        const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
        const unsigned pblocks = unsigned(c->nsm) * 8u;  // persistent grids of the step kernels
        const BoxProp* bprop = p->rta ? nullptr : B.d_boxprop.as<BoxProp>();
        int istep = 0;
        double time = 0.;
        // phase timing (the reference's timer buckets): events at the phase
        // borders of every step, read at the end
        enum { PH_ADV, PH_CANCEL, PH_GEN, PH_HIST, PH_PROPS, PH_READ, PH_SAVE, PH_SCAT };
        double phase[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        std::vector<cudaEvent_t> pev(std::size_t(nsteps) * 7, nullptr);
        struct EvGuard {
            std::vector<cudaEvent_t>* e;
            ~EvGuard() {
                for (auto ev : *e)
                    if (ev) cudaEventDestroy(ev);
            }
        } pe_guard{&pev};
        for (auto& e : pev) ck(cudaEventCreate(&e), "cudaEventCreate");
        phase[PH_READ] = 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        std::vector<int> hH;
        const int cancel_every = p->cancel_every > 0 ? p->cancel_every : 4;
        const std::size_t hbytes = std::size_t(nbx) * n * sizeof(int);
        auto swap_ab = [&] {
            std::swap(B.a_x.p, B.b_x.p);
            std::swap(B.a_y.p, B.b_y.p);
            std::swap(B.a_mode.p, B.b_mode.p);
            std::swap(B.a_box.p, B.b_box.p);
            std::swap(B.a_sign.p, B.b_sign.p);
        };
        while (time <= p->maxtime && istep < nsteps) {
            cudaEvent_t* ev = pev.data() + std::size_t(istep) * 7;
            ck(cudaEventRecord(ev[0], s), "event");
            // 1 + 6 + 7 for the particles of the last step: advection,
            // scattering and histogram in one pass, into B
            ck(cudaMemsetAsync(B.d_H.p, 0, hbytes, s), "memset");
            ck(cudaMemsetAsync(dc + DC_NOUT, 0, 2 * sizeof(unsigned long long), s), "memset");
            const AdvectArgs a_step{GA.G, GA.boxcell, GA.mv, B.d_boxwall.as<int4>(), B.d_Eb.as<int>(), p->dt, 0ull, 0,
                                    general, mix_key(p->seed, istep, 31), err, TT};
            be_advance<<<pblocks, 256, 0, s>>>(arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign), dc + DC_NP,
                                               arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), dc, cap, 1, a_step,
                                               p->rta, pal, bprop, B.nm, c->d_w.as<double>(),
                                               c->d_rprob.as<float>(), c->d_ralt.as<int>(), n,
                                               mix_key(p->seed, istep, 64), B.d_H.as<int>(), err);
            ck(cudaEventRecord(ev[1], s), "event");
            // 2-4 the step's sources, made at A[0..) (A is free now) and each
            // advected for a random part of the step as it is made
            ck(cudaMemsetAsync(dc + DC_NGEN, 0, sizeof(unsigned long long), s), "memset");
            const PArr A = arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign);
            auto gen_args = [&](int ph) {
                return AdvectArgs{GA.G, GA.boxcell, GA.mv, B.d_boxwall.as<int4>(), B.d_Eb.as<int>(), p->dt,
                                  mix_key(p->seed, istep, ph + 1), 1, general, mix_key(p->seed, istep, ph + 17), err,
                                  TT};
            };
            if (ngd) {
                be_plan_sources<<<1, 32, 0, s>>>(B.d_gdesc.as<GenDesc>(), B.d_ggenf.as<double>(), B.d_gcnt.as<long long>(),
                                                 ngd, mix_key(p->seed, istep, 40), dc, span + 0, cap, err);
                be_generate_dev<<<pblocks, 256, 0, s>>>(A, span + 0, B.d_gdesc.as<GenDesc>(), ngd, B.d_gprob.as<float>(),
                                                        B.d_galt.as<int>(), B.d_gsign.as<signed char>(),
                                                        B.d_cdf.as<double>(), B.d_cdftot.as<double>(), n,
                                                        mix_key(p->seed, istep, 8), c->d_boxes.as<GBox>(),
                                                        c->d_hull.as<V2>(), gen_args(8));
            }
            if (nid) {
                be_plan_sources<<<1, 32, 0, s>>>(B.d_idesc.as<GenDesc>(), B.d_igenf.as<double>(), B.d_icnt.as<long long>(),
                                                 nid, mix_key(p->seed, istep, 41), dc, span + 1, cap, err);
                be_generate_dev<<<pblocks, 256, 0, s>>>(A, span + 1, B.d_idesc.as<GenDesc>(), nid, B.d_isoprob.as<float>(),
                                                        B.d_isoalt.as<int>(), nullptr, B.d_cdf.as<double>(),
                                                        B.d_cdftot.as<double>(), n, mix_key(p->seed, istep, 2),
                                                        c->d_boxes.as<GBox>(), c->d_hull.as<V2>(), gen_args(2));
            }
            if (nborders > 0) {
                be_plan_adiabatic<<<1, 32, 0, s>>>(B.d_Eb.as<int>(), B.d_adi.as<AdiBorder>(), nborders, SP, p->Eeff,
                                                   p->dt, g.thickness, B.d_req.as<WallReq>(), B.d_acnt.as<long long>(),
                                                   B.d_adesc.as<GenDesc>(), dc, span + 2, cap, err);
                be_wall_cdf1_dev<<<unsigned(nborders) * unsigned(nch), 256, 0, s>>>(
                    B.d_om.as<float>(), B.d_vx.as<float>(), B.d_vy.as<float>(), n, B.d_req.as<WallReq>(),
                    B.d_acnt.as<long long>(), B.d_cdf.as<double>(), B.d_ctot.as<double>());
                be_wall_cdf2_dev<<<unsigned(nborders) * unsigned(nch), 256, 0, s>>>(
                    n, B.d_acnt.as<long long>(), B.d_ctot.as<double>(), B.d_cdf.as<double>(), B.d_cdftot.as<double>());
                be_generate_dev<<<pblocks, 256, 0, s>>>(A, span + 2, B.d_adesc.as<GenDesc>(), nborders, nullptr, nullptr,
                                                        nullptr, B.d_cdf.as<double>(), B.d_cdftot.as<double>(), n,
                                                        mix_key(p->seed, istep, 4), c->d_boxes.as<GBox>(),
                                                        c->d_hull.as<V2>(), gen_args(4));
            }
            ck(cudaEventRecord(ev[2], s), "event");
            // 5-7 for the new particles: the absorbed ones dropped, the others
            // scattered and counted in the histogram, appended to B
            ck(cudaMemsetAsync(dc + DC_WORK, 0, sizeof(unsigned long long), s), "memset");
            be_advance<<<pblocks, 256, 0, s>>>(A, dc + DC_NGEN, arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), dc,
                                               cap, 0, a_step, p->rta, pal, bprop, B.nm, c->d_w.as<double>(),
                                               c->d_rprob.as<float>(), c->d_ralt.as<int>(), n,
                                               mix_key(p->seed, istep, 65), B.d_H.as<int>(), err);
            ck(cudaEventRecord(ev[3], s), "event");
            ck(cudaEventRecord(ev[4], s), "event");  // the histogram is made in the passes above
            // 8. cancellation every cancel_every steps: B -> A; otherwise B is the population
            if (istep % cancel_every == 0) {
                ck(cudaMemsetAsync(B.d_cnt.p, 0, hbytes, s), "memset");
                be_cancel_dev<<<pblocks, 256, 0, s>>>(arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), dc + DC_NOUT, cap,
                                                      B.d_H.as<int>(), B.d_cnt.as<int>(), n, d_res.as<int>(),
                                                      mix_key(p->seed, istep, 77));
                ck(cudaMemsetAsync(dc + DC_NP, 0, sizeof(unsigned long long), s), "memset");
                be_compact_dev<<<pblocks, 256, 0, s>>>(arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), dc + DC_NOUT, cap,
                                                       arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign), dc + DC_NP);
            } else {
                be_counters<<<1, 1, 0, s>>>(dc, DC_NP, DC_NOUT, nullptr, 0);
                swap_ab();
            }
            ck(cudaEventRecord(ev[5], s), "event");
            // 9. properties of the step (calculate_prop), recorded on the device
            be_props<<<nbx, 256, 0, s>>>(B.d_H.as<int>(), n, B.d_rvx.as<double>(), B.d_rvy.as<double>(),
                                          B.d_phist.as<double>() + std::size_t(istep + 1) * nbx * 3);
            be_counters<<<1, 1, 0, s>>>(dc, -1, 0, B.d_nhist.as<long long>(), istep + 1);
            ck(cudaGetLastError(), "step launch");
            ck(cudaEventRecord(ev[6], s), "event");
            if (p->on_step) {
                hH.resize(std::size_t(nbx) * n);
                int herr[4];
                long long hnp = 0;
                ck(cudaMemcpyAsync(hH.data(), B.d_H.p, hbytes, cudaMemcpyDeviceToHost, s), "d2h");
                ck(cudaMemcpyAsync(hprops.data(), B.d_phist.as<double>() + std::size_t(istep + 1) * nbx * 3,
                                   hprops.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "d2h");
                ck(cudaMemcpyAsync(&hnp, B.d_nhist.as<long long>() + istep + 1, sizeof hnp, cudaMemcpyDeviceToHost, s),
                   "d2h");
                ck(cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s), "d2h");
                sync(c);
                if (herr[0] != 0) throw_step_error(herr[0]);
                std::vector<double> ed(static_cast<std::size_t>(nbx)), fl(std::size_t(nbx) * 2);
                for (int b = 0; b < nbx; ++b) {
                    ed[std::size_t(b)] = p->Eeff / vol[std::size_t(b)] * 1.0e+27 * hprops[3 * std::size_t(b)];
                    fl[2 * std::size_t(b)] = p->Eeff / vol[std::size_t(b)] * 1.0e+30 * hprops[3 * std::size_t(b) + 1];
                    fl[2 * std::size_t(b) + 1] = p->Eeff / vol[std::size_t(b)] * 1.0e+30 * hprops[3 * std::size_t(b) + 2];
                }
                const auto t_save = std::chrono::steady_clock::now();
                p->on_step(p->user, istep + 1, time + p->dt, hnp, hH.data(), nbx, n, ed.data(), fl.data());
                phase[PH_SAVE] += 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t_save).count();
            }
            istep++;
            time += p->dt;
        }
        // the records of every step
        {
            int herr[4];
            std::vector<double> ph(std::size_t(nsteps + 1) * nbx * 3);
            std::vector<long long> nh(std::size_t(nsteps + 1));
            std::vector<unsigned long long> hdc(DC_COUNT);
            ck(cudaMemcpyAsync(ph.data(), B.d_phist.p, ph.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(nh.data(), B.d_nhist.p, nh.size() * sizeof(long long), cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(hdc.data(), dc, DC_COUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s), "d2h");
            sync(c);
            if (herr[0] != 0) throw_step_error(herr[0]);
            for (int st = 1; st <= istep; ++st) {
                for (int b = 0; b < nbx; ++b) {
                    const double f1 = p->Eeff / vol[std::size_t(b)] * 1.0e+27;
                    const double f2 = p->Eeff / vol[std::size_t(b)] * 1.0e+30;
                    const std::size_t q = (std::size_t(st) * nbx + std::size_t(b)) * 3;
                    if (out->ed) out->ed[std::size_t(st) * nbx + b] = f1 * ph[q];
                    if (out->flux) {
                        out->flux[(std::size_t(st) * nbx + b) * 2] = f2 * ph[q + 1];
                        out->flux[(std::size_t(st) * nbx + b) * 2 + 1] = f2 * ph[q + 2];
                    }
                }
                if (out->nparticles) out->nparticles[st] = nh[std::size_t(st)];
            }
            psteps = (long long)hdc[DC_PSTEPS];
            branchings = (long long)hdc[DC_FLIPS];
            adv_in = (long long)hdc[DC_IN];
            adv_out = (long long)hdc[DC_OUTT];
            const int bucket[6] = {PH_ADV, PH_GEN, PH_SCAT, PH_HIST, PH_CANCEL, PH_PROPS};
            for (int st = 0; st < istep; ++st)
                for (int k = 0; k < 6; ++k) {
                    float pms = 0.f;
                    if (cudaEventElapsedTime(&pms, pev[std::size_t(st) * 7 + k], pev[std::size_t(st) * 7 + k + 1]) ==
                        cudaSuccess)
                        phase[bucket[k]] += pms;
                }
        }
        ck(cudaEventRecord(c->ev1, s), "event");
        sync(c);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        if (out->histogram)
            ck(cudaMemcpy(out->histogram, B.d_H.p, std::size_t(nbx) * n * sizeof(int), cudaMemcpyDeviceToHost), "d2h");
        out->nboxes = nbx;
        out->nsteps = istep;
        out->particle_steps = psteps;
        out->branchings = branchings;
        out->advance_in = adv_in;
        out->advance_out = adv_out;
        out->kernel_ms = ms;
        for (int k = 0; k < 8; ++k) out->phase_ms[k] = phase[k];
        return BTE_OK;
    } catch (const Error& e) {
        c->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_CUDA;
    }
}
