// rta_prod.cu - production mode of the RTA particle loop.
//
// Draws come from counter-based Philox4x32-10 streams keyed by (seed,
// particle); mode distributions and Lambert rows are sampled through alias
// tables; positions, times and tallies stay FP64, with tallies reduced by FP64
// atomics.  Two kernels:
//   rta_prod_general  any convex-box geometry, the flight logic of
//                     rta_flight.cuh (one particle per thread);
//   rta_prod_grid     boxes that tile an axis-aligned grid: a persistent
//                     kernel whose warps refill idle lanes with new particles
//                     and that walks cells by exit times, with a per-lane
//                     pending tally flushed when the (box, bin) key changes.
#include "kernels.h"

namespace bte {

__device__ __forceinline__ void record_error(int* err, int e, long long pid) {
    if (atomicCAS(err, 0, e) == 0) {
        err[1] = int(pid & 0x7fffffff);
        err[2] = int(pid >> 31);
    }
}

__device__ __forceinline__ void flush_counters_p(const Counters& c, unsigned long long* out) {
    unsigned long long v[8] = {c.events, c.wall_hits, c.crossings, c.absorbed,
                               c.specular, c.nudges, c.quirks, c.tallies};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        unsigned long long x = v[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + i, x);
    }
}

// Alias draw over n slots: slot from the high bits of one word, acceptance
// from 24 bits of another.
__device__ __forceinline__ int alias_draw(Philox& g, const float* prob, const int* alt, int n) {
    const int j = int(mulhi32(g.next32(), uint32_t(n)));
    const float a = float(g.next32() >> 8) * 0x1p-24f;
    return a < __ldg(prob + j) ? j : __ldg(alt + j);
}

struct ProdPolicy {
    Philox g;
    double* out;
    unsigned long long ntally;

    __device__ double u() { return g.uniform(); }
    __device__ int choose(int n) { return uniform_below(g, uint32_t(n)); }
    __device__ double flight(const DevTables& T, int k) {
        return double(-logf(g.uniformf())) * __ldg(T.tau + k);
    }
    __device__ int resample(const DevTables& T) {
        return alias_draw(g, T.resample_prob, T.resample_alt, T.n);
    }
    __device__ int gen_mode(const DevTables& T, int gi) {
        const long long o = (long long)gi * T.n;
        const int j = alias_draw(g, T.gen_prob + o, T.gen_alt + o, T.n);
        return j;
    }
    __device__ int bounce(const DevTables& T, int cls, int mode) {
        const long long a = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + mode);
        const long long b = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + mode + 1);
        const int len = int(b - a);
        if (len <= 0) return -1;
        const int j = int(mulhi32(g.next32(), uint32_t(len)));
        const int4 e = __ldg(T.lalias + a + j);
        const float acc = float(g.next32() >> 8) * 0x1p-24f;
        return acc < __int_as_float(e.x) ? e.y : e.z;
    }
    __device__ int tally(const DevTables& T, int box, double t0, double t1, int sign, V2 v) {
        int sb = int(t0 * T.inv_dt), eb = int(t1 * T.inv_dt);
        const int last = T.nbins - 1;
        sb = sb < 0 ? 0 : (sb > last ? last : sb);
        eb = eb < 0 ? 0 : (eb > last ? last : eb);
        const double* g = T.timegrid;
        for (int i = sb; i <= eb; ++i) {
            const double lo = fmax(g[i] - t0, 0.);
            const double hi = fmin(g[i + 1] - t0, t1 - t0);
            const double contr = double(sign) * fmax(hi - lo, 0.);
            if (contr != 0.) {
                double* base = out + 3ll * ((long long)box * T.nbins + i);
                atomicAdd(base + 0, contr);
                atomicAdd(base + 1, v.x * contr);
                atomicAdd(base + 2, v.y * contr);
                ntally++;
            }
        }
        return 0;
    }
};

__global__ void __launch_bounds__(128) rta_prod_general(DevTables T, double* tally,
                                                        unsigned long long* counters, int* err) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n = T.pend - T.pbegin;
    const long long trips = (n + stride - 1) / stride;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long it = 0; it < trips; ++it) {
        const long long pid = T.pbegin + it * stride + tid;
        if (pid >= T.pend) continue;
        ProdPolicy pol;
        pol.g.init(T.seed, (uint64_t)pid);
        pol.out = tally;
        pol.ntally = 0;
        const int e = run_particle(T, pol, pid, c);
        c.tallies += pol.ntally;
        if (e) record_error(err, e, pid);
    }
    flush_counters_p(c, counters);
}

void launch_prod_general(const DevTables& T, double* tally, unsigned long long* counters,
                         int* err, int nsm, cudaStream_t s) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return;
    long long blocks = (n + 127) / 128;
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    rta_prod_general<<<unsigned(blocks), 128, 0, s>>>(T, tally, counters, err);
}

// ------------------------------------------------------------------ grid path

struct GridParticle {
    double x, y, t;
    int i, j;      // cell
    int mode;
    int sign;
    int box;
};

// Pending tally of one lane: unsigned contributions to one (box, bin) key
// summed in registers; the particle sign is applied to the sign bit when
// the key changes and the sums go out as three FP64 atomics.
struct Pending {
    int key;
    unsigned adds;
    double c0, c1, c2;
    __device__ __forceinline__ void flush(double* tally, unsigned long long signbit) {
        if (key >= 0) {
            double* b = tally + 3ll * key;
            atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(c0) ^ signbit));
            atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(c1) ^ signbit));
            atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(c2) ^ signbit));
        }
        key = -1;
        c0 = c1 = c2 = 0.;
    }
    __device__ __forceinline__ void add(double* tally, unsigned long long signbit, int k, double d,
                                        double vx, double vy) {
        if (k != key) {
            flush(tally, signbit);
            key = k;
        }
        c0 += d;
        c1 = fma(vx, d, c1);
        c2 = fma(vy, d, c2);
        adds++;
    }
};

__device__ __forceinline__ int grid_cell(const DevGrid& G, int i, int j) {
    if (i < 0 || j < 0 || i >= G.nx || j >= G.ny) return -1;
    return __ldg(G.cell + i * G.ny + j);
}

// Generate particle `pid` on the grid.  Returns 0 or an error code.
__device__ int grid_generate(const DevTables& T, const DevGrid& G, const int2* boxcell, Philox& g,
                             long long pid, GridParticle& p) {
    int box;
    if (T.source == 0) {
        (void)g.uniform();  // generator-type draw of Init_generator
        const double where = g.uniform();
        int gi = lower_bound_d(T.wall_cum, T.ngen, where);
        if (gi >= T.ngen) gi = T.ngen - 1;
        const WallGenDev W = T.walls[gi];
        const double u = g.uniform();
        p.x = W.p1.x + u * W.nd.x;
        p.y = W.p1.y + u * W.nd.y;
        box = W.box;
        p.sign = W.sign;
        const long long o = (long long)gi * T.n;
        p.mode = alias_draw(g, T.gen_prob + o, T.gen_alt + o, T.n);
    } else {
        int lo = 0, hi = T.ngen;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(T.init_first + mid) <= pid) lo = mid; else hi = mid;
        }
        box = __ldg(T.init_box + lo);
        const int2 ij = __ldg(boxcell + box);
        const double x0 = __ldg(G.gx + ij.x), x1 = __ldg(G.gx + ij.x + 1);
        const double y0 = __ldg(G.gy + ij.y), y1 = __ldg(G.gy + ij.y + 1);
        p.x = x0 + g.uniform() * (x1 - x0);
        p.y = y0 + g.uniform() * (y1 - y0);
        p.sign = __ldg(T.init_sign + lo);
        const long long o = (long long)lo * T.n;
        p.mode = alias_draw(g, T.gen_prob + o, T.gen_alt + o, T.n);
    }
    const int2 ij = __ldg(boxcell + box);
    p.i = ij.x;
    p.j = ij.y;
    p.box = box;
    p.t = 0.;
    return 0;
}

// One lane carries one particle; each pass of the loop advances every active
// lane by exactly one segment -- to the end of its free flight or to the
// next cell border -- so the FP64 work of a warp stays converged however
// many cells a flight crosses.  Idle lanes take new particles from a global
// counter, one atomic per warp.
template <bool SMEM_TALLY>
__global__ void __launch_bounds__(256) rta_prod_grid(DevTables T, GridArgs A, double* gtally,
                                                     unsigned long long* counters, int* err,
                                                     unsigned long long* work) {
    extern __shared__ double stally[];
    const int nk3 = 3 * T.nboxes * T.nbins;
    double* tally = gtally;
    if (SMEM_TALLY) {
        for (int k = threadIdx.x; k < nk3; k += blockDim.x) stally[k] = 0.;
        __syncthreads();
        tally = stally;
    }
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const long long total = T.pend - T.pbegin;
    const int last_bin = T.nbins - 1;
    Pending pd;
    pd.key = -1;
    pd.adds = 0;
    pd.c0 = pd.c1 = pd.c2 = 0.;
    GridParticle p;
    p.i = p.j = p.mode = p.box = 0;
    p.sign = 1;
    p.x = p.y = p.t = 0.;
    Philox g;
    g.init(0, 0);
    ModeVel mv = {0., 0., 0., 0.};
    double dt = 0., tnb = 0.;
    long long pid = -1, nev = 0;
    int bin = 0;
    unsigned long long signbit = 0;
    bool active = false, done = false, need_flight = false;
    for (;;) {
        // refill idle lanes of the warp with new particles
        const unsigned idle = __ballot_sync(0xffffffffu, !active && !done);
        if (idle) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && !done) {
                const long long mine = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (mine < total) {
                    pid = T.pbegin + mine;
                    g.init(T.seed, (uint64_t)pid);
                    const int e = grid_generate(T, A.G, A.boxcell, g, pid, p);
                    if (e) {
                        record_error(err, e, pid);
                        done = true;
                    } else {
                        active = true;
                        need_flight = true;
                        nev = 0;
                        bin = 0;
                        tnb = __ldg(T.timegrid + 1);
                        signbit = p.sign < 0 ? 0x8000000000000000ull : 0ull;
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        if (need_flight) {
            // a new free flight: u in (0, 1) -> dt = -tau ln u (FP32 log)
            const int k = p.mode;
            mv = A.mv[k];
            dt = double(-logf(g.uniformf())) * __ldg(T.tau + k);
            c.events++;
            if (!(dt > 0.) || ++nev > EVENT_CAP) {  // zero rate or runaway particle
                record_error(err, dt > 0. ? E_LIMIT : E_VALUE, pid);
                active = false;
                done = true;
                pd.flush(tally, signbit);
                continue;
            }
            if (p.t + dt > T.maxtime) dt = T.maxtime - p.t;
            need_flight = false;
        }
        // exit times of the current cell.  A zero velocity component takes
        // the upper cell line, so (line - position) >= 0 times its +inf
        // inverse gives +inf (or NaN on the line), and fmin ignores a NaN.
        const double xw = __ldg(A.G.gx + p.i + (mv.vx >= 0. ? 1 : 0));
        const double yw = __ldg(A.G.gy + p.j + (mv.vy >= 0. ? 1 : 0));
        const double tx = (xw - p.x) * mv.ivx;
        const double ty = (yw - p.y) * mv.ivy;
        const double te = fmin(tx, ty);
        const bool ends = !(dt > te);              // stays in the cell (also for te = NaN)
        const double seg = ends ? dt : fmax(te, 0.);
        // tally [t, t + seg] in (box, bin), splitting at bin borders
        const double t1 = p.t + seg;
        double t0 = p.t;
        while (t1 > tnb && bin < last_bin) {
            pd.add(tally, signbit, p.box * T.nbins + bin, tnb - t0, mv.vx, mv.vy);
            t0 = tnb;
            ++bin;
            tnb = __ldg(T.timegrid + bin + 1);
        }
        pd.add(tally, signbit, p.box * T.nbins + bin, t1 - t0, mv.vx, mv.vy);
        p.t = t1;
        dt -= seg;
        if (ends) {
            p.x = fma(seg, mv.vx, p.x);
            p.y = fma(seg, mv.vy, p.y);
            if (!T.ballistic) p.mode = alias_draw(g, T.resample_prob, T.resample_alt, T.n);
            need_flight = true;
        } else {
            // reaches a cell border: snap the crossed coordinate to the grid line
            int ni = p.i, nj = p.j, wall;
            if (tx <= ty) {
                p.x = xw;
                p.y = fma(seg, mv.vy, p.y);
                if (mv.vx > 0.) { ni = p.i + 1; wall = 0; } else { ni = p.i - 1; wall = 1; }
            } else {
                p.y = yw;
                p.x = fma(seg, mv.vx, p.x);
                if (mv.vy > 0.) { nj = p.j + 1; wall = 2; } else { nj = p.j - 1; wall = 3; }
            }
            const int nb = grid_cell(A.G, ni, nj);
            if (nb >= 0) {
                p.i = ni;
                p.j = nj;
                p.box = nb;
                c.crossings++;
            } else if (nb <= -2) {
                c.absorbed++;
                active = false;
                pd.flush(tally, signbit);
                continue;
            } else {
                // void: reflect at the wall; a new flight follows
                const int cls = A.cls[wall];
                if (cls < 0) {
                    record_error(err, E_GEOM, pid);
                    active = false;
                    done = true;
                    pd.flush(tally, signbit);
                    continue;
                }
                const int k = p.mode;
                int nm = -1;
                if (T.specularity > 0. && g.uniform() < T.specularity && T.mirror) {
                    nm = __ldg(T.mirror + (long long)cls * T.n + k);
                    if (nm >= 0) c.specular++;
                }
                if (nm < 0) {
                    const long long a = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k);
                    const long long b = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k + 1);
                    const int len = int(b - a);
                    if (len <= 0) {
                        record_error(err, E_GEOM, pid);
                        active = false;
                        done = true;
                        pd.flush(tally, signbit);
                        continue;
                    }
                    const int jj = int(mulhi32(g.next32(), uint32_t(len)));
                    const int4 e = __ldg(T.lalias + a + jj);
                    const float acc = float(g.next32() >> 8) * 0x1p-24f;
                    nm = acc < __int_as_float(e.x) ? e.y : e.z;
                }
                p.mode = nm;
                c.wall_hits++;
                need_flight = true;
            }
        }
        if (p.t >= T.maxtime) {
            active = false;
            pd.flush(tally, signbit);
        }
    }
    pd.flush(tally, signbit);
    c.tallies = pd.adds;
    flush_counters_p(c, counters);
    if (SMEM_TALLY) {
        __syncthreads();
        for (int k = threadIdx.x; k < nk3; k += blockDim.x) {
            const double x = stally[k];
            if (x != 0.) atomicAdd(gtally + k, x);
        }
    }
}

bool launch_prod_grid(const DevTables& T, const GridArgs& A, double* tally,
                           unsigned long long* counters, int* err, unsigned long long* work,
                           const ProdTuning& tune, int nsm, cudaStream_t s) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return true;
    const int threads = tune.block_threads > 0 ? tune.block_threads : 256;
    if (threads > 256 || threads % 32) return false;
    const size_t smem = size_t(3) * T.nboxes * T.nbins * sizeof(double);
    bool use_smem = tune.smem_tally != 0 && smem <= 200 * 1024;
    int bps = tune.blocks_per_sm > 0 ? tune.blocks_per_sm : (use_smem ? 1 : 8);
    if (use_smem) {
        if (cudaFuncSetAttribute(rta_prod_grid<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(smem)) != cudaSuccess)
            return false;
        int maxb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, rta_prod_grid<true>, threads, smem);
        if (maxb < 1) return false;
        if (bps > maxb) bps = maxb;
    }
    long long blocks = (long long)nsm * bps;
    const long long need = (n + threads - 1) / threads;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    if (use_smem)
        rta_prod_grid<true><<<unsigned(blocks), threads, smem, s>>>(T, A, tally, counters, err, work);
    else
        rta_prod_grid<false><<<unsigned(blocks), threads, 0, s>>>(T, A, tally, counters, err, work);
    return true;
}

}  // namespace bte
