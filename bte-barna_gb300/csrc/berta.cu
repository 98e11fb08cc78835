// berta.cu - beyond-RTA deviational MC (beRTAMC2D) on the device.
//
// The step loop of src/beyondRTA_MC2d.cpp:2138-2425, production mode:
//   1 advection by dt; void walls absorb and count Eborder, reservoirs absorb
//     (evolparticle :708-970)                                      be_advect
//   2 gradient source term: Nabla_T particles at random points of every box
//     with a gradient, random sub-step (source_term_gradient :597-676,
//     Nabla_T_distribution src/sampling.cpp:118-187)            be_generate
//   3 isothermal-wall injection, random sub-step            be_generate
//     (Isothermal_walls :446-585, Ntogenerate src/sampling.cpp:243-260)
//   4 adiabatic diffuse re-emission of |Eborder| at the wall temperature from
//     the J(T) cubic spline (adiabatic_diffuse_walls :281-435)    be_generate
//   5 deletion                                                  be_compact
//   6 propagator scattering with sign branching (Scattering :1073-1210,
//     propagator_H::get src/collision_operator.cpp:892-903), each parent's
//     branching attempts made in place by its thread, or the RTA
//     alternative (ScatteringRTA :983-1062)          be_scatter / be_scatter_rta
//   7 histogram H[box][mode] += sign                            be_hist
//   8 cancellation every 4th step: keep |H| particles of the majority sign
//     per (box, mode) (:2295-2370), by per-key ranks, no sort   be_cancel
//   9 calculate_prop: ed and flux per box from H (:1538-1602)   be_props
// Particles live in HBM as structure-of-arrays (x, y FP64; mode, box, sign
// int32).  Draws: Philox4x32-10 keyed by (seed, step, phase), counter =
// particle index.  Geometry: boxes that tile an axis-aligned grid.
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

// Page-locked staging for the per-step uploads: a copy from pageable memory
// may wait for the stream's earlier work, a copy from here does not.  Each
// upload site has its own buffer, written again only after a later sync.
struct Pinned {
    void* p = nullptr;
    size_t bytes = 0;
    Pinned() = default;
    Pinned(const Pinned&) = delete;
    Pinned& operator=(const Pinned&) = delete;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
    void reserve(size_t n) {
        if (bytes >= n) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        ck(cudaMallocHost(&p, n), "cudaMallocHost");
        bytes = n;
    }
};

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
    // what the device holds: the alias table of the propagator at sel_T, or
    // (sel_lirp) the interpolated signed CDF at sel_T
    double sel_T = 0;
    bool sel_lirp = false;
    long long sel_version = -1;
    DBuf d_palias, d_pcdf;
    long long cap = 0;
    DBuf a_x, a_y, a_mode, a_box, a_sign;   // particles
    DBuf b_x, b_y, b_mode, b_box, b_sign;   // compaction / scattering output
    DBuf d_H, d_cnt, d_Eb, d_props, d_counts, d_boxwall, d_gens, d_alias, d_rvx, d_rvy;
    DBuf d_om, d_vx, d_vy, d_req, d_cdf, d_cdftot, d_isoprob, d_isoalt;
    DBuf d_gprob, d_galt, d_gsign;          // gradient source rows
    DBuf d_ne, d_ctot;                      // n(omega, T0) per mode; wall-CDF chunk sums
    Pinned h_gens[4], h_req;                // staging: descriptors per phase, wall requests

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

__global__ void be_advect(PArr P, long long begin, long long end, AdvectArgs a) {
    for (long long i = begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < end;
         i += (long long)gridDim.x * blockDim.x) {
        int mode = P.mode[i];
        if (mode < 0) continue;
        double dt = a.dt;
        if (a.random_substep) {
            Philox g;
            g.init(a.key, (uint64_t)i);
            dt = a.dt * g.uniform();
        }
        double x = P.x[i], y = P.y[i];
        int box = P.box[i];
        if (a.general) {
            BePol pol;
            pol.g.init(a.gkey, (uint64_t)i);
            int err = 0;
            if (!advect_general(a.T, pol, a.Eb, x, y, box, mode, P.sign[i], dt, err)) mode = -1;
            if (err && a.err) atomicCAS(a.err, 0, err);
        } else if (!advect_one(a.G, a.boxcell, a.mv, a.boxwall, a.Eb, x, y, box, mode, P.sign[i], dt)) {
            mode = -1;
        }
        P.x[i] = x;
        P.y[i] = y;
        P.box[i] = box;
        P.mode[i] = mode;
    }
}

// Isothermal_wall_distribution (src/sampling.cpp:189-269) of each request:
// pmf_k = v_n omega_k |n(omega_k, Tw) - n(omega_k, Te)| for v_n > 0, turned
// into a CDF row; tot[r] keeps the sum.  Each request's row is split into
// chunks of WCDF_CHUNK modes, one block each, so that every SM's FP64 units
// take part.  ne[k] = n(omega_k, Te_ref) is precomputed: a request at that
// Te needs one exponential per mode instead of two.
constexpr int WCDF_CHUNK = 1024;

// pass 1: the chunk's running sums in place and its total
__global__ void __launch_bounds__(256) be_wall_cdf1(const double* om, const double* vx, const double* vy,
                                                    const double* ne, double Te_ref, int n,
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
    const bool pre_e = R.Te == Te_ref;
    double acc = 0.;
    for (int k = k0; k < k1; ++k) {
        const double w = om[k];
        const double vn = R.nx * vx[k] + R.ny * vy[k];
        double p = 0.;
        if (vn > 0. && !almost_equal(0., w)) {
            const double nw = 1. / (exp(pre * w / R.Tw) - 1.);
            const double nE = pre_e ? ne[k] : 1. / (exp(pre * w / R.Te) - 1.);
            p = vn * w * fabs(nw - nE);
        }
        acc += p;
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
__global__ void __launch_bounds__(256) be_wall_cdf2(int n, const double* chunk_tot, double* cdf, double* tot) {
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
__global__ void be_compact(PArr in, long long n, PArr out, unsigned long long* count) {
    const int lane = threadIdx.x & 31;
    for (long long base = blockIdx.x * (long long)blockDim.x; base < n;
         base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + threadIdx.x;
        const bool live = i < n && in.mode[i] >= 0;
        const unsigned m = __ballot_sync(0xffffffffu, live);
        unsigned long long w = 0;
        if (lane == 0 && m) w = atomicAdd(count, (unsigned long long)__popc(m));
        w = __shfl_sync(0xffffffffu, w, 0);
        if (live) {
            const long long o = (long long)w + __popc(m & ((1u << lane) - 1u));
            out.x[o] = in.x[i];
            out.y[o] = in.y[i];
            out.mode[o] = in.mode[i];
            out.box[o] = in.box[i];
            out.sign[o] = in.sign[i];
        }
    }
}

// Propagator scattering with sign branching (Scattering, src/beyondRTA_MC2d.cpp:
// 1073-1210).  Every scattering attempt of a parent draws its next mode from
// the parent's column and emits one outgoing particle; when the drawn sign
// differs from the parent's, the reference puts two copies of the parent
// back into the queue, and each copy makes an attempt of its own.  The copies
// are identical to the parent, so here a thread keeps only the number of
// attempts its parent still owes and makes them in place, with fresh draws,
// until none is left: one launch per step instead of one per round.  The
// outgoing particles are appended warp by warp.  BRANCH_CAP bounds the
// attempts of one parent (a supercritical propagator never stops).
constexpr unsigned BRANCH_CAP = 1u << 20;

// Persistent warps: a lane whose parent owes no attempt takes the next
// parent from a global counter (one atomic per warp), so the warp keeps its
// lanes busy while chains of different lengths run out.
// propagator_H::lower_bound (include/collision_operator.hpp:263-269): the
// first entry whose |value| is not below u, by std::lower_bound's own
// probing, so that an interpolated column whose |values| are not monotone
// gives the same index as in the reference; clamped to the last entry.
__device__ __forceinline__ int lower_bound_abs(const double* a, int n, double u) {
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int step = cnt >> 1;
        const int it = lo + step;
        if (fabs(__ldg(a + it)) < fabs(u)) {
            lo = it + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    return lo < n ? lo : n - 1;
}

// pcdf set: draw from the signed CDF columns instead of the alias table (an
// interpolated propagator, which has no alias form in general).
__global__ void be_scatter(PArr in, long long n, PArr out, unsigned long long* ocount, long long ocap,
                           unsigned long long* nflips, unsigned long long* work, const PAlias* pal,
                           const double* pcdf, int nm, unsigned long long key, int* err) {
    const int lane = threadIdx.x & 31;
    unsigned long long flips = 0;
    int mode = 0, sign = 1, box = 0, col = 0;
    double x = 0., y = 0.;
    unsigned todo = 0, made = 0;
    bool done = false, valid = false;
    Philox g;
    g.init(key, 0);
    for (;;) {
        // refill the lanes whose parent is finished
        const unsigned idle = __ballot_sync(0xffffffffu, todo == 0 && !done);
        if (idle) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (todo == 0 && !done) {
                const long long i = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    mode = in.mode[i];
                    sign = in.sign[i];
                    box = in.box[i];
                    x = in.x[i];
                    y = in.y[i];
                    col = mode - 3;
                    valid = col >= 0 && col < nm;
                    if (!valid) atomicCAS(err, 0, E_VALUE);
                    g.init(key, (uint64_t)i);
                    todo = 1;
                    made = 0;
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        const bool act = todo > 0;
        int nmode = mode, nsign = sign;
        if (act && valid && pcdf) {
            const double* c = pcdf + (long long)col * nm;
            const int im = lower_bound_abs(c, nm, g.uniform());
            nmode = im + 3;
            nsign = __ldg(c + im) > 0. ? sign : -sign;
        } else if (act && valid) {
            const int j = int(mulhi32(g.next32(), uint32_t(nm)));
            const float acc = float(g.next32() >> 8) * 0x1p-24f;
            const PAlias e = pal[(long long)col * nm + j];
            const bool keep = acc < e.prob;
            const int slot = keep ? j : int(e.alt & 0x3fffffffu);
            const bool neg = keep ? (e.alt >> 31) != 0u : ((e.alt >> 30) & 1u) != 0u;
            nmode = slot + 3;
            nsign = neg ? -sign : sign;
        }
        // append the outgoing particle of this attempt
        const unsigned m1 = __ballot_sync(0xffffffffu, act);
        unsigned long long w = 0;
        if (lane == 0 && m1) w = atomicAdd(ocount, (unsigned long long)__popc(m1));
        w = __shfl_sync(0xffffffffu, w, 0);
        if (act) {
            const long long o = (long long)w + __popc(m1 & ((1u << lane) - 1u));
            if (o < ocap) {
                out.x[o] = x;
                out.y[o] = y;
                out.box[o] = box;
                out.mode[o] = nmode;
                out.sign[o] = nsign;
            } else {
                atomicCAS(err, 0, E_LIMIT);
            }
            --todo;
            if (nsign != sign) {  // two more attempts of the parent
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
    if (lane == 0 && flips) atomicAdd(nflips, flips);
}

// RTA scattering: with probability 1 - exp(-w dt) a particle is resampled
// from the C w distribution.
__global__ void be_scatter_rta(PArr P, long long n, const double* w, double dt, const float* rprob,
                               const int* ralt, int nmodes, unsigned long long key) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int mode = P.mode[i];
        Philox g;
        g.init(key, (uint64_t)i);
        const double u = g.uniform();
        if (u < 1. - exp(-__ldg(w + mode) * dt)) {
            const int j = int(mulhi32(g.next32(), uint32_t(nmodes)));
            const float acc = float(g.next32() >> 8) * 0x1p-24f;
            P.mode[i] = acc < __ldg(rprob + j) ? j : __ldg(ralt + j);
        }
    }
}

__global__ void be_hist(PArr P, long long n, int* H, int nmodes) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        atomicAdd(H + (long long)P.box[i] * nmodes + P.mode[i], P.sign[i]);
}

// Cancellation: a particle survives when its sign is the sign of H at its
// (box, mode) and its rank among those particles is below |H|.  Threads
// visit the particles in the order of a random affine permutation
// t -> (a t + b) mod n (a coprime to n), so the ranks, and with them the
// survivors, do not follow the order of the particle list.
__global__ void be_cancel(PArr P, long long n, const int* H, int* cnt, int nmodes, const int* reservoir,
                          unsigned long long pa, unsigned long long pb) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = (long long)((unsigned __int128)(pa % (unsigned long long)n) * (unsigned long long)t %
                                        (unsigned long long)n + pb % (unsigned long long)n) % n;
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

// The device tables of the propagator at Teq = T0 (Scattering,
// src/beyondRTA_MC2d.cpp:1130-1165): the tabulated one when T0 is in the
// table, sampled through per-column alias tables; otherwise lirp
// (src/collision_operator.cpp:918-929) between the first tabulated
// temperature above T0 and the next one -- both above T0, as the reference
// picks them -- sampled through the interpolated signed CDF.
void select_propagator(bte_ctx* c, bte::BertaState& B, double T0) {
    using namespace bte;
    if (B.sel_version == B.props_version && B.sel_T == T0) return;
    const int nm = B.nm;
    const std::size_t nn = std::size_t(nm) * std::size_t(nm);
    auto it = B.props.find(T0);
    if (it != B.props.end()) {
        const std::vector<double>& P = it->second;
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
        B.d_palias.upload(tab, c->stream);
        B.sel_lirp = false;
    } else {
        auto m1 = B.props.lower_bound(T0);
        const double Tlow = B.props.begin()->first;
        if (m1 == B.props.end() || std::next(m1) == B.props.end() || T0 < Tlow)
            throw Error(BTE_ERR_INPUT,
                        "Extrapolation is not allowed: limit Tref between the min and max temperatures "
                        "used in the propagator calculation");
        const auto m2 = std::next(m1);
        const double T1 = m1->first, T2 = m2->first;
        const std::vector<double> c1 = signed_cumm(m1->second, nm), c2 = signed_cumm(m2->second, nm);
        std::vector<double> pint(nn);
        for (std::size_t i = 0; i < nn; ++i) pint[i] = c1[i] + (T0 - T1) * (c2[i] - c1[i]) / (T2 - T1);
        B.d_pcdf.upload(pint, c->stream);
        B.sel_lirp = true;
    }
    sync(c);
    B.sel_T = T0;
    B.sel_version = B.props_version;
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
        // one temperature for the scattering tables: every box that is
        // neither a reservoir nor periodic at T0, so the gradients of the
        // boxes' Teq (calculate_gradientT, src/geometry_2d.cpp:524-575) are
        // zero and only a homogeneous <gradient> adds a source term
        for (std::size_t b = 0; b < g.boxes.size(); ++b)
            if (!g.reservoir[b] && g.tto[b] < 0 && g.Teq[b] != p->T0)
                throw Error(BTE_ERR_INPUT, "every box needs Teq = T0 (one scattering temperature per run)");
        if (p->gradient_mode != 0 && p->gradient_mode != 1) throw Error(BTE_ERR_INPUT, "bad gradient_mode");
        if (p->gradient_mode == 1 && !(std::isfinite(p->gradient[0]) && std::isfinite(p->gradient[1])))
            throw Error(BTE_ERR_INPUT, "gradient must be finite");
        if (p->rta) ensure_resample(c, p->T0);
        else select_propagator(c, *c->berta, p->T0);
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
        B.d_counts.alloc(4 * sizeof(unsigned long long));
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
        auto* counts = B.d_counts.as<unsigned long long>();
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
        std::vector<WallReq> reqs;
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
        // the gradient source term: a homogeneous <gradient> on every box
        // that is neither a reservoir nor periodic (the gradients of the
        // boxes' Teq are zero here); Nabla_T rows at each box's Teq, built
        // once as the reference's static generators are
        GradGenerators grad;
        if (p->gradient_mode == 1 && !almost_equal(std::hypot(p->gradient[0], p->gradient[1]), 0.)) {
            grad = build_gradient_generators(m, g, p->gradient[0], p->gradient[1]);
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
            B.d_om.upload(m.omega, s);
            B.d_vx.upload(m.vx, s);
            B.d_vy.upload(m.vy, s);
            // n(omega, T0) of every mode for the adiabatic re-emission rows
            std::vector<double> ne(m.omega.size(), 0.);
            const double pre = 1e12 * 1.054571726e-34 / 1.3806488e-23;
            for (std::size_t k = 0; k < ne.size(); ++k)
                if (m.omega[k] > 0.) ne[k] = 1. / (std::exp(pre * m.omega[k] / p->T0) - 1.);
            B.d_ne.upload(ne, s);
        }
        // generate the sources in `descs` at A[base..): alias rows from
        // aprob/aalt (uploaded here) or from a table already on the device
        // (rprob/ralt, with per-mode signs rsign), CDF rows from B.d_cdf
        auto generate = [&](long long base, long long total, long long step, int phase, bool advect,
                            const float* rprob = nullptr, const int* ralt = nullptr,
                            const signed char* rsign = nullptr) {
            if (total <= 0) return;
            if (base + total > cap) throw Error(BTE_ERR_LIMIT, "particle capacity exceeded: raise capacity");
            // one staging buffer per phase (initial, gradient, isothermal, adiabatic)
            const int slot = phase == 0 ? 0 : phase == 8 ? 1 : phase == 2 ? 2 : 3;
            upload_pinned(B.d_gens, B.h_gens[slot], descs, s);
            const float* dprob = rprob;
            const int* dalt = ralt;
            if (!rprob && !aprob.empty()) {
                B.d_alias.alloc(aprob.size() * sizeof(float) + aalt.size() * sizeof(int));
                ck(cudaMemcpyAsync(B.d_alias.p, aprob.data(), aprob.size() * sizeof(float), cudaMemcpyHostToDevice, s), "h2d");
                int* a2 = reinterpret_cast<int*>(B.d_alias.as<char>() + aprob.size() * sizeof(float));
                ck(cudaMemcpyAsync(a2, aalt.data(), aalt.size() * sizeof(int), cudaMemcpyHostToDevice, s), "h2d");
                dprob = B.d_alias.as<float>();
                dalt = a2;
            }
            PArr A = arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign);
            be_generate<<<launch_blocks(total, c->nsm), 256, 0, s>>>(
                A, base, total, B.d_gens.as<GenDesc>(), int(descs.size()), dprob, dalt, rsign,
                B.d_cdf.as<double>(), B.d_cdftot.as<double>(), n, mix_key(p->seed, step, phase),
                c->d_boxes.as<GBox>(), c->d_hull.as<V2>());
            if (advect) {
                AdvectArgs aa{GA.G, GA.boxcell, GA.mv, B.d_boxwall.as<int4>(), B.d_Eb.as<int>(), p->dt,
                              mix_key(p->seed, step, phase + 1), 1,
                              general, mix_key(p->seed, step, phase + 17), err, TT};
                be_advect<<<launch_blocks(total, c->nsm), 256, 0, s>>>(A, base, base + total, aa);
            }
        };
        auto read_count = [&](int k) {
            unsigned long long v = 0;
            ck(cudaMemcpyAsync(&v, counts + k, sizeof v, cudaMemcpyDeviceToHost, s), "d2h");
            sync(c);
            return (long long)v;
        };
        auto compact = [&](long long nn) {
            ck(cudaMemsetAsync(counts, 0, sizeof(unsigned long long), s), "memset");
            if (nn > 0)
                be_compact<<<launch_blocks(nn, c->nsm), 256, 0, s>>>(
                    arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign), nn,
                    arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), counts);
            const long long m2 = read_count(0);
            std::swap(B.a_x.p, B.b_x.p);
            std::swap(B.a_y.p, B.b_y.p);
            std::swap(B.a_mode.p, B.b_mode.p);
            std::swap(B.a_box.p, B.b_box.p);
            std::swap(B.a_sign.p, B.b_sign.p);
            return m2;
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
            generate(0, first, -1, 0, false);
            np = first;
        }
        props(np, 0);
        const PArr A0 = arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign);
        (void)A0;
        long long psteps = 0, branchings = 0;
        int istep = 0;
        double time = 0.;
        // phase timing (the reference's timer buckets): events at the phase
        // borders of every step, read after the step's last sync
        enum { PH_ADV, PH_CANCEL, PH_GEN, PH_HIST, PH_PROPS, PH_READ, PH_SAVE, PH_SCAT };
        double phase[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        cudaEvent_t pe[7];
        for (auto& e : pe) ck(cudaEventCreate(&e), "cudaEventCreate");
        struct EvGuard {
            cudaEvent_t* e;
            ~EvGuard() {
                for (int i = 0; i < 7; ++i) cudaEventDestroy(e[i]);
            }
        } pe_guard{pe};
        phase[PH_READ] = 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        std::vector<int> hE(static_cast<std::size_t>(nborders));
        std::vector<int> hH;
        std::vector<double> pmf;
        const int cancel_every = p->cancel_every > 0 ? p->cancel_every : 4;
        while (time <= p->maxtime) {
            ck(cudaEventRecord(pe[0], s), "event");
            // 1. advection
            if (np > 0) {
                AdvectArgs aa{GA.G, GA.boxcell, GA.mv, B.d_boxwall.as<int4>(), B.d_Eb.as<int>(), p->dt, 0ull, 0,
                              general, mix_key(p->seed, istep, 31), err, TT};
                be_advect<<<launch_blocks(np, c->nsm), 256, 0, s>>>(arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign),
                                                                    0, np, aa);
            }
            psteps += np;
            ck(cudaEventRecord(pe[1], s), "event");
            // 2. gradient source term: Ntogenerate(dt, vol, Eeff) per box
            if (!grad.box.empty()) {
                descs.clear();
                long long nnew = 0;
                for (std::size_t k = 0; k < grad.box.size(); ++k) {
                    const long long cnt = (long long)n_to_generate(p->dt * grad.energy[k] / p->Eeff, rng);
                    if (cnt == 0) continue;
                    GenDesc d = box_desc(grad.box[k]);
                    d.alias_off = (long long)k * n;
                    d.msign = 1;
                    d.first = nnew;
                    descs.push_back(d);
                    nnew += cnt;
                }
                generate(np, nnew, istep, 8, true, B.d_gprob.as<float>(), B.d_galt.as<int>(),
                         B.d_gsign.as<signed char>());
                np += nnew;
            }
            // 3. isothermal walls
            descs.clear();
            aprob.clear();
            aalt.clear();
            long long nnew = 0;
            for (std::size_t k = 0; k < iso.walls.size(); ++k) {
                const WallGenerator& W = iso.walls[k];
                const double Lb = norm(sub(W.sb, W.sa));
                const double spf = Lb * g.thickness / (m.V * g.thickness / m.c);
                const double cumulsum = std::fabs(W.flux) * double(m.nq) * vuc;
                const long long cnt = (long long)n_to_generate(p->dt * spf * cumulsum / (p->Eeff * double(m.nq)), rng);
                if (cnt == 0) continue;
                GenDesc d{};
                d.x0 = W.p1.x;
                d.y0 = W.p1.y;
                d.dx = W.nd.x;
                d.dy = W.nd.y;
                d.box = W.box;
                d.sign = W.sign;
                d.rect = 0;
                d.cdf = -1;
                d.alias_off = (long long)k * n;
                d.first = nnew;
                descs.push_back(d);
                nnew += cnt;
            }
            generate(np, nnew, istep, 2, true, B.d_isoprob.as<float>(), B.d_isoalt.as<int>());
            np += nnew;
            // 4. adiabatic diffuse walls: |Eborder| at the spline temperature
            ck(cudaMemcpyAsync(hE.data(), B.d_Eb.p, hE.size() * sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
            sync(c);
            ck(cudaMemsetAsync(B.d_Eb.p, 0, hE.size() * sizeof(int), s), "memset");
            descs.clear();
            aprob.clear();
            aalt.clear();
            reqs.clear();
            nnew = 0;
            for (int gb = 0; gb < nborders; ++gb) {
                const int E = hE[std::size_t(gb)];
                if (E == 0) continue;
                const int b = border_box[std::size_t(gb)];
                if (b < 0 || g.reservoir[std::size_t(b)] || g.tto[std::size_t(b)] >= 0) continue;
                const GBorder& br = g.borders[std::size_t(gb)];
                const V2 nwall = v2(-br.np.x, -br.np.y);
                const double Teq = g.Teq[std::size_t(b)];
                if (!B.spl_ok[std::size_t(gb)]) {
                    std::vector<double> J(100), Tv(100);
                    for (int t = 0; t < 100; ++t) {
                        const double T = 10.0 + 10.0 * t;
                        Tv[std::size_t(t)] = T;
                        const double cs = wall_pmf(m, nwall, T, Teq, pmf);
                        J[std::size_t(t)] = ((T - Teq) >= 0 ? 1 : -1) * (cs / (double(m.nq) * vuc));
                    }
                    B.spl[std::size_t(gb)].build(J, Tv);
                    B.spl_ok[std::size_t(gb)] = 1;
                }
                const double len = norm(sub(br.p2, br.p1));
                const double Jb = p->Eeff * E / p->dt / (len * g.thickness);
                const double Tb = B.spl[std::size_t(gb)].interp(Jb);
                GenDesc d{};
                d.x0 = br.p1.x;
                d.y0 = br.p1.y;
                d.dx = br.nd.x;
                d.dy = br.nd.y;
                d.box = b;
                d.sign = (Tb - Teq) >= 0 ? 1 : -1;
                d.rect = 0;
                d.cdf = int(reqs.size());
                d.alias_off = 0;
                d.first = nnew;
                descs.push_back(d);
                reqs.push_back(WallReq{nwall.x, nwall.y, Tb, Teq});
                nnew += (long long)(std::abs(E) + 1.0e-6);
            }
            if (!reqs.empty()) {
                // the re-emission distributions at the border temperatures,
                // built on the device (one block per border)
                upload_pinned(B.d_req, B.h_req, reqs, s);
                const int nch = (n + WCDF_CHUNK - 1) / WCDF_CHUNK;
                be_wall_cdf1<<<unsigned(reqs.size()) * unsigned(nch), 256, 0, s>>>(
                    B.d_om.as<double>(), B.d_vx.as<double>(), B.d_vy.as<double>(), B.d_ne.as<double>(), p->T0, n,
                    B.d_req.as<WallReq>(), B.d_cdf.as<double>(), B.d_ctot.as<double>());
                be_wall_cdf2<<<unsigned(reqs.size()) * unsigned(nch), 256, 0, s>>>(
                    n, B.d_ctot.as<double>(), B.d_cdf.as<double>(), B.d_cdftot.as<double>());
            }
            generate(np, nnew, istep, 4, true);
            np += nnew;
            ck(cudaEventRecord(pe[2], s), "event");
            // 5. delete absorbed particles
            np = compact(np);
            // 6. scattering
            if (p->rta) {
                if (np > 0)
                    be_scatter_rta<<<launch_blocks(np, c->nsm), 256, 0, s>>>(
                        arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign), np, c->d_w.as<double>(), p->dt,
                        c->d_rprob.as<float>(), c->d_ralt.as<int>(), n, mix_key(p->seed, istep, 6));
            } else if (np > 0) {
                // counts: [0] outgoing particles, [1] sign flips, [2] parents taken
                ck(cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), s), "memset");
                long long sblocks = (np + 255) / 256;
                if (sblocks > 8ll * c->nsm) sblocks = 8ll * c->nsm;
                be_scatter<<<unsigned(sblocks), 256, 0, s>>>(
                    arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign), np,
                    arr(B.b_x, B.b_y, B.b_mode, B.b_box, B.b_sign), counts, cap, counts + 1, counts + 2,
                    B.d_palias.as<PAlias>(), B.sel_lirp ? B.d_pcdf.as<double>() : nullptr, B.nm,
                    mix_key(p->seed, istep, 64), err);
                unsigned long long hcnt[2] = {0, 0};
                ck(cudaMemcpyAsync(hcnt, counts, sizeof hcnt, cudaMemcpyDeviceToHost, s), "d2h");
                sync(c);
                branchings += (long long)hcnt[1];
                np = (long long)hcnt[0];
                if (np > cap) throw Error(BTE_ERR_LIMIT, "particle capacity exceeded in scattering");
                std::swap(B.a_x.p, B.b_x.p);
                std::swap(B.a_y.p, B.b_y.p);
                std::swap(B.a_mode.p, B.b_mode.p);
                std::swap(B.a_box.p, B.b_box.p);
                std::swap(B.a_sign.p, B.b_sign.p);
            }
            ck(cudaEventRecord(pe[3], s), "event");
            // 7.-9. histogram, cancellation, properties
            ck(cudaMemsetAsync(B.d_H.p, 0, std::size_t(nbx) * n * sizeof(int), s), "memset");
            if (np > 0)
                be_hist<<<launch_blocks(np, c->nsm), 256, 0, s>>>(arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign),
                                                                  np, B.d_H.as<int>(), n);
            ck(cudaEventRecord(pe[4], s), "event");
            if (istep % cancel_every == 0 && np > 0) {
                ck(cudaMemsetAsync(B.d_cnt.p, 0, std::size_t(nbx) * n * sizeof(int), s), "memset");
                // random affine permutation of the visiting order (a coprime to np)
                unsigned long long pa = rng.next() | 1ull, pb = rng.next();
                while (std::gcd((unsigned long long)np, pa % (unsigned long long)np) != 1ull) pa += 2;
                be_cancel<<<launch_blocks(np, c->nsm), 256, 0, s>>>(arr(B.a_x, B.a_y, B.a_mode, B.a_box, B.a_sign),
                                                                    np, B.d_H.as<int>(), B.d_cnt.as<int>(), n,
                                                                    d_res.as<int>(), pa, pb);
                np = compact(np);
            }
            ck(cudaEventRecord(pe[5], s), "event");
            be_props<<<nbx, 256, 0, s>>>(B.d_H.as<int>(), n, B.d_rvx.as<double>(), B.d_rvy.as<double>(),
                                          B.d_props.as<double>());
            int herr[4];
            ck(cudaMemcpyAsync(hprops.data(), B.d_props.p, hprops.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaEventRecord(pe[6], s), "event");
            sync(c);
            {
                const int bucket[6] = {PH_ADV, PH_GEN, PH_SCAT, PH_HIST, PH_CANCEL, PH_PROPS};
                for (int k = 0; k < 6; ++k) {
                    float ms = 0.f;
                    if (cudaEventElapsedTime(&ms, pe[k], pe[k + 1]) == cudaSuccess) phase[bucket[k]] += ms;
                }
            }
            for (int b = 0; b < nbx; ++b) {
                const double f1 = p->Eeff / vol[std::size_t(b)] * 1.0e+27;
                const double f2 = p->Eeff / vol[std::size_t(b)] * 1.0e+30;
                const std::size_t sidx = std::size_t(istep) + 1;
                if (out->ed) out->ed[sidx * nbx + b] = f1 * hprops[3 * std::size_t(b)];
                if (out->flux) {
                    out->flux[(sidx * nbx + b) * 2] = f2 * hprops[3 * std::size_t(b) + 1];
                    out->flux[(sidx * nbx + b) * 2 + 1] = f2 * hprops[3 * std::size_t(b) + 2];
                }
            }
            if (out->nparticles) out->nparticles[istep + 1] = np;
            if (p->on_step) {
                hH.resize(std::size_t(nbx) * n);
                ck(cudaMemcpyAsync(hH.data(), B.d_H.p, hH.size() * sizeof(int), cudaMemcpyDeviceToHost, s), "d2h");
                sync(c);
                std::vector<double> ed(static_cast<std::size_t>(nbx)), fl(std::size_t(nbx) * 2);
                for (int b = 0; b < nbx; ++b) {
                    ed[std::size_t(b)] = p->Eeff / vol[std::size_t(b)] * 1.0e+27 * hprops[3 * std::size_t(b)];
                    fl[2 * std::size_t(b)] = p->Eeff / vol[std::size_t(b)] * 1.0e+30 * hprops[3 * std::size_t(b) + 1];
                    fl[2 * std::size_t(b) + 1] = p->Eeff / vol[std::size_t(b)] * 1.0e+30 * hprops[3 * std::size_t(b) + 2];
                }
                const auto t_save = std::chrono::steady_clock::now();
                p->on_step(p->user, istep + 1, time + p->dt, np, hH.data(), nbx, n, ed.data(), fl.data());
                phase[PH_SAVE] += 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t_save).count();
            }
            if (herr[0] != 0)
                throw Error(bte_status(herr[0]), herr[0] == BTE_ERR_LIMIT      ? "particle capacity or step cap exceeded"
                                                 : herr[0] == BTE_ERR_GEOMETRY ? "geometry error in the advection"
                                                                               : "particle without a propagator column");
            istep++;
            time += p->dt;
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
