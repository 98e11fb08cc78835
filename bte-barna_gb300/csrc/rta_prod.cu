// rta_prod.cu - production mode of the RTA particle loop.
//
// Draws come from counter-based Philox4x32-10 streams keyed by (seed,
// particle); mode distributions and Lambert rows are sampled through alias
// tables; positions, times and tallies stay FP64, with tallies reduced by FP64
// atomics.  Three kernels:
//   rta_prod_general  any convex-box geometry, the flight logic of
//                     rta_flight.cuh (one evolparticle step per pass);
//   rta_prod_grid     boxes that tile an axis-aligned grid: a persistent
//                     kernel whose warps refill idle lanes with new particles
//                     and that walks cells by exit times, with a per-lane
//                     pending tally flushed when the (box, bin) key changes;
//   rta_prod_poly     the grid kernel's loop over any convex boxes, exit
//                     times taken against each box's border lines.
#include "kernels.h"
#include "rta_steady.cuh"

namespace bte {

__device__ __forceinline__ void record_error(int* err, int e, long long pid) {
    if (atomicCAS(err, 0, e) == 0) {
        err[1] = int(pid & 0x7fffffff);
        err[2] = int(pid >> 31);
    }
}

// Warp-reduced counters: the first NC of (events, wall hits, crossings,
// absorbed, specular, nudges, quirks, tally updates, translations,
// steady-state scatters, steady-state drops, interface hits, interface
// transmissions).
template <int NC = 11>
__device__ __forceinline__ void flush_counters_p(const Counters& c, unsigned long long* out) {
    unsigned long long v[13] = {c.events, c.wall_hits, c.crossings, c.absorbed,
                                c.specular, c.nudges, c.quirks, c.tallies, c.translations,
                                c.scattered, c.lost, c.ifc_hits, c.ifc_trans};
#pragma unroll
    for (int i = 0; i < NC; ++i) {
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
        return double(-logf(g.uniformf())) * __ldg(T.tau + k);  // k: material offset + mode
    }
    __device__ int resample(const DevTables& T, int mo) {
        return alias_draw(g, T.resample_prob + mo, T.resample_alt + mo, T.n);
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
    __device__ int dist(const double*, const float* prob, const int* alt, int n) {
        return alias_draw(g, prob, alt, n);
    }
    // process_segment (periodic), src/RTA_MC2D.cpp:784-834
    __device__ int tally_dt(const DevTables& T, int box, double d, int sign, V2 v, int mode) {
        const double contr = double(sign) * d;
        double* base = out + 3ll * box;
        atomicAdd(base + 0, contr);
        atomicAdd(base + 1, v.x * contr);
        atomicAdd(base + 2, v.y * contr);
        const int loc = T.spec_loc ? __ldg(T.spec_loc + box) : -1;
        if (loc >= 0) {
            const long long o = (long long)loc * T.n + mode;
            atomicAdd(T.spec + o, contr);
            atomicAdd(T.spec_cnt + o, (unsigned long long)(long long)sign);
        }
        ntally++;
        return 0;
    }
    __device__ int tally(const DevTables& T, int box, double t0, double t1, int sign, V2 v, int mode) {
        const int loc = T.spec_loc ? __ldg(T.spec_loc + box) : -1;
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
                if (loc >= 0) atomicAdd(T.spec + (long long)(loc * T.nbins + i) * T.n + mode, contr);
                ntally++;
            }
        }
        return 0;
    }
};

// Any convex-box geometry, the flight logic of rta_flight.cuh (run_particle
// unrolled into one evolparticle step per loop pass).  Warps are persistent
// and a lane whose particle has finished takes the next one from a global
// counter (one atomic per warp), so lanes stay busy while particles of very
// different lifetimes run out; each particle keeps its own Philox stream,
// so its trajectory is the one run_particle would draw.
__global__ void __launch_bounds__(128) rta_prod_general(DevTables T, double* tally,
                                                        unsigned long long* counters, int* err,
                                                        unsigned long long* work) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const long long total = T.pend - T.pbegin;
    ProdPolicy pol;
    pol.g.init(0, 0);
    pol.out = tally;
    pol.ntally = 0;
    Particle p;
    p.pos = v2(0., 0.);
    p.mode = 0;
    p.sign = 1;
    p.t = 0.;
    p.box = 0;
    p.mo = 0;
    V2 v = v2(0., 0.);
    double dt = 0., time = 0.;
    int nudges = 0, guard = 0, fate = FATE_LOST;
    long long nev = 0, pid = -1;
    bool active = false, done = false, need_flight = false;
    for (;;) {
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
                    pol.g.init(T.seed, (uint64_t)pid);
                    const int e = generate(T, pol, pid, p);
                    if (e) {
                        record_error(err, e, pid);
                    } else {
                        active = true;
                        need_flight = true;
                        time = 0.;
                        nudges = 0;
                        nev = 0;
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        if (need_flight) {  // the body of run_particle's outer loop
            if (!(time < T.maxtime)) {
                active = false;
                continue;
            }
            const int k = p.mode;
            if (++nev > T.flight_cap || T.w[p.mo + k] == 0.) {
                record_error(err, nev > T.flight_cap ? E_LIMIT : E_VALUE, pid);
                active = false;
                continue;
            }
            v = v2(T.vxc[k], T.vyc[k]);
            dt = pol.flight(T, p.mo + k);
            c.events++;
            if (time + dt > T.maxtime) dt = T.maxtime - time + 1.0e-8;
            guard = 0;
            fate = FATE_LOST;
            need_flight = false;
        }
        if (!almost_equal(dt, 0.)) {
            int e = ++guard > FLIGHT_CAP ? E_LIMIT : 0;
            if (!e) e = evolparticle(T, pol, p, v, dt, c, nudges, fate);
            if (e) {
                record_error(err, e, pid);
                active = false;
                continue;
            }
        }
        if (almost_equal(dt, 0.)) {  // the flight is over
            if (p.mode == 0) {       // absorbed
                active = false;
                continue;
            }
            time = p.t;
            need_flight = true;
        }
    }
    c.tallies += pol.ntally;
    flush_counters_p<13>(c, counters);
}

// Generation 0: 1 per slot whose first draw picks a gradient generator.
__global__ void steady_select_prod(SteadyArgs A, unsigned long long seed, unsigned* flags) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < A.n; s += stride) {
        Philox g;
        g.init(seed, steady_stream(0, s));
        flags[s] = steady_gen_type(A, g.uniform()) == 1 ? 1u : 0u;
    }
}

// One generation: each slot's one flight, one evolparticle step per loop
// pass, with persistent warps whose finished lanes take the next slot.
__global__ void __launch_bounds__(128) rta_steady_prod(DevTables T, SteadyArgs A, double* tally,
                                                       unsigned long long* counters, int* err) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    ProdPolicy pol;
    pol.g.init(0, 0);
    pol.out = tally;
    pol.ntally = 0;
    Particle p;
    p.pos = v2(0., 0.);
    p.mode = 0;
    p.sign = 1;
    p.t = 0.;
    p.box = 0;
    p.mo = 0;
    V2 v = v2(0., 0.);
    double dt = 0.;
    int nudges = 0, guard = 0, fate = FATE_LOST;
    long long slot = -1;
    bool active = false, done = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active && !done);
        if (idle) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader) base = atomicAdd(A.work, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && !done) {
                slot = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (slot < A.n) {
                    pol.g.init(T.seed, steady_stream(A.gen, slot));
                    const int e = steady_begin(T, A, pol, slot, c, p, v, dt);
                    if (e) {
                        record_error(err, e, slot);
                        A.flag[slot] = 0;
                    } else {
                        active = true;
                        fate = FATE_LOST;
                        guard = 0;
                        nudges = 0;
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        if (!almost_equal(dt, 0.)) {
            int e = ++guard > FLIGHT_CAP ? E_LIMIT : 0;
            if (!e) e = evolparticle<ProdPolicy, true>(T, pol, p, v, dt, c, nudges, fate);
            if (e) {
                record_error(err, e, slot);
                A.flag[slot] = 0;
                active = false;
                continue;
            }
        }
        if (almost_equal(dt, 0.)) {  // the flight is over
            if (fate == FATE_LOST) c.lost++;
            steady_emit(A, slot, fate, p);
            active = false;
        }
    }
    c.tallies += pol.ntally;
    flush_counters_p<13>(c, counters);
}

void launch_steady_prod(const DevTables& T, const SteadyArgs& A, double* tally,
                        unsigned long long* counters, int* err, unsigned* select_flags, int nsm,
                        cudaStream_t s) {
    if (A.n <= 0) return;
    long long blocks = (A.n + 127) / 128;
    if (select_flags) {
        const long long cap = (long long)nsm * 16;
        if (blocks > cap) blocks = cap;
        steady_select_prod<<<unsigned(blocks), 128, 0, s>>>(A, T.seed, select_flags);
        return;
    }
    const long long cap = (long long)nsm * 4;  // resident blocks of the persistent kernel (128 registers)
    if (blocks > cap) blocks = cap;
    cudaMemsetAsync(A.work, 0, sizeof(unsigned long long), s);
    rta_steady_prod<<<unsigned(blocks), 128, 0, s>>>(T, A, tally, counters, err);
}

void launch_prod_general(const DevTables& T, double* tally, unsigned long long* counters,
                         int* err, unsigned long long* work, int nsm, cudaStream_t s) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return;
    long long blocks = (n + 127) / 128;
    const long long cap = (long long)nsm * 3;  // resident blocks (145 registers x 128 threads)
    if (blocks > cap) blocks = cap;
    rta_prod_general<<<unsigned(blocks), 128, 0, s>>>(T, tally, counters, err, work);
}

// ------------------------------------------------------------------ grid path

struct GridParticle {
    double x, y, t;
    int i, j;      // cell
    int mode;
    int sign;
    int box;
    int mo;        // material offset (material * n)
};

// Order of non-negative doubles (and +inf, and NaN above +inf) through their
// bit patterns as signed 64-bit integers, on the integer pipe: a negative
// operand keeps the sign bit and stays below every non-negative one.
__device__ __forceinline__ long long ob(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double obd(long long b) { return __longlong_as_double(b); }

// float -> double for a positive normal float, by moving its exponent and
// mantissa fields (integer pipe).
__device__ __forceinline__ double widen_pos(float f) {
    const unsigned fb = __float_as_uint(f);
    const unsigned long long e = ((fb >> 23) & 0xffu) + (1023u - 127u);
    return __longlong_as_double((long long)((e << 52) | ((unsigned long long)(fb & 0x7fffffu) << 29)));
}

// Pending tally of one lane.  Inside one (box, time bin) key the particle
// moves continuously, so the key's contributions telescope: time spent =
// r0 - r, r the time left to the bin's end, and the velocity-weighted sums
// are the displacement x - x0, y - y0 (sum of v * dt over the segments).
// Nothing is accumulated per segment; when the key changes the three
// differences go out as FP64 atomics, with the particle sign applied to the
// sign bit.
struct Pending {
    int key;
    unsigned flushes;
    double r0, x0, y0;
    __device__ __forceinline__ void start(int k, double r, double x, double y) {
        key = k;
        r0 = r;
        x0 = x;
        y0 = y;
    }
    __device__ __forceinline__ void flush(double* tally, unsigned long long signbit, double r, double x,
                                          double y) {
        if (key >= 0) {
            double* b = tally + 3ll * key;
            atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(r0 - r) ^ signbit));
            atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(x - x0) ^ signbit));
            atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(y - y0) ^ signbit));
            flushes++;
        }
        key = -1;
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
    p.mo = mat_off(T, box);
    p.t = 0.;
    return 0;
}

// The draws of one loop pass: Philox4x32-10 block (pass, 2^30, particle)
// under the run's seed, a counter range the particle's generation draws
// (counter words from 0) never reach.  Every active lane computes one block
// per pass at the same point of the loop, so the generator runs with the
// whole warp instead of once per call site that finds its queue empty.
// x: the free flight, y and z: the alias draw (slot, acceptance), w: the
// specular test.
__device__ __forceinline__ uint4 pass_block(uint32_t pass, uint64_t pid, uint64_t seed) {
    Philox q;
    q.init(seed, pid);
    q.c0 = pass;
    q.c1 = 0x40000000u;
    q.block();
    return make_uint4(q.b0, q.b1, q.b2, q.b3);
}

// One lane carries one particle; each pass of the loop advances every active
// lane by exactly one segment, which ends at the first of: the end of the
// free flight, the next cell line, the next time-bin border (the last one is
// maxtime).  Every pass therefore runs one fixed FP64 sequence on all lanes
// -- the two exit times, the bin border, the advance and the three
// differences of the pending tally -- and a lane flushes at most once per
// pass, at the segment end; the FP64 pipe, the limit of this kernel on
// GB300, never sees the same operation issued twice for different lanes.
// Idle lanes take new particles from a global counter, one atomic per warp.
// Comparisons, min/max and the float -> double widening run on the integer
// pipe.  The random words of a pass come from one Philox block per lane
// (pass_block); a flight that ends at a void wall or by scattering draws
// its next mode in one block for both cases (Lambert row or post-scattering
// alias table) and draws the next flight length there.
//
// ADJ selects the two passes of the adjoint (ADJ = 0 is the plain kernel):
// 1 forward: also accumulates each particle's contribution to a linear
//   functional Phi = sum W[box][bin][q] tally[box][bin][q] and stores it;
// 2 adjoint: replays every particle from its Philox counter (the same draws
//   as pass 1) and adds likelihood-ratio terms, each weighted by the
//   particle's future contribution R = Phi_total - Phi so far:
//   free flight of mode k, dt = tau_k e:  d log f / d tau_k = (e - 1) / tau_k
//   post-scattering draw of mode k (p_k ~ C_k / tau_k): -1 / tau_k on tau_k,
//     plus p_i / tau_i on every tau_i (summed once on the host from sum R)
//   specularity draw at a void wall:       1 / p (specular) or -1 / (1 - p)
// CHECK: the checked variant (BTE_FLAG_CHECKS): every table, tally and grid
// index is tested before use; a violation stops the particle with E_CHECK.
// The checks draw nothing, so the trajectories are the plain variant's.
template <bool SMEM_TALLY, int MINB, int ADJ, bool CHECK = false>
__global__ void __launch_bounds__(256, MINB) rta_prod_grid(DevTables T, GridArgs A, double* gtally,
                                                     unsigned long long* counters, int* err,
                                                     unsigned long long* work, AdjArgs adj) {
    extern __shared__ double stally[];
    const int nk3 = 3 * T.nboxes * T.nbins;
    double* tally = gtally;
    if (SMEM_TALLY) {
        for (int k = threadIdx.x; k < nk3; k += blockDim.x) stally[k] = 0.;
        __syncthreads();
        tally = stally;
    }
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const long long total = T.pend - T.pbegin;
    const int last_bin = T.nbins - 1;
    // specular draw on the integer pipe: u32 < p 2^32 (p >= 1: always);
    // 0 when the walls are diffuse
    const unsigned long long spec_thr =
        T.specularity >= 1.0 ? (1ull << 32)
                             : (T.specularity > 0. ? (unsigned long long)(T.specularity * 4294967296.0) : 0ull);
    Pending pd;
    pd.key = -1;
    pd.flushes = 0;
    pd.r0 = pd.x0 = pd.y0 = 0.;
    GridParticle p;
    p.i = p.j = p.mode = p.box = p.mo = 0;
    p.sign = 1;
    p.x = p.y = p.t = 0.;
    Philox g;
    g.init(0, 0);
    ModeVel mv = {0., 0., 0., 0.};
    // dt: time left in the free flight; rb: time left to the end of the
    // current time bin (bin widths follow the ntime grid points)
    const double* binw = T.timegrid + T.ntime;
    double dt = 0., rb = 0.;
    long long pid = -1, nev = 0;
    double* tgrp = tally;  // the tally of the particle's replica group
    uint32_t npass = 0;
    int bin = 0;
    unsigned long long signbit = 0;
    bool active = false, done = false;
    // adjoint state: Phi so far, the particle's total, pending score terms
    double phi_run = 0., phi_tot = 0., spec_score = 0.;
    double sum_r = 0., g_p = 0., phi_all = 0.;
    long long slot = 0;
    int pend_kind = 0;
    // A new free flight of the current mode from one random word:
    // dt = -tau ln u (FP32 log), u = (k + 1/2) 2^-23 from 23 bits, never 0
    // or 1; its velocities stay in registers for the segments that follow.
    // Returns false when the particle stops with an error.
    // a failed index check stops the particle (checked variant only)
    auto check_fail = [&]() {
        record_error(err, E_CHECK, pid);
        active = false;
        done = true;
    };
    auto new_flight = [&](uint32_t word) -> bool {
        const int k = p.mode;
        if (CHECK && (k < 0 || k >= T.n || p.mo < 0)) {
            check_fail();
            return false;
        }
        mv = A.mv[k];
        const float ef = -logf((float(word >> 9) + 0.5f) * 0x1p-23f);
        const double tau_k = __ldg(T.tau + p.mo + k);
        dt = widen_pos(ef) * tau_k;
        c.events++;
        if (ADJ == 2) {
            // future contribution from here: Phi_total - (flushed + pending part)
            const double* Wk = adj.W + 3ll * pd.key;
            const double part = __ldg(Wk) * (pd.r0 - rb) + __ldg(Wk + 1) * (p.x - pd.x0) +
                                __ldg(Wk + 2) * (p.y - pd.y0);
            const double R = phi_tot - (phi_run + (p.sign < 0 ? -part : part));
            double gk = (widen_pos(ef) - 1.0) / tau_k * R;
            if (pend_kind & 1) {  // this mode came from a post-scattering draw
                gk -= R / tau_k;
                sum_r += R;
            }
            if (pend_kind & 2) g_p += spec_score * R;
            pend_kind = 0;
            atomicAdd(adj.g_tau + k, gk);
        }
        if (ob(dt) <= 0 || ++nev > T.flight_cap) {  // zero rate or runaway particle
            record_error(err, ob(dt) > 0 ? E_LIMIT : E_VALUE, pid);
            active = false;
            done = true;
            pd.flush(tgrp, signbit, rb, p.x, p.y);
            return false;
        }
        return true;
    };
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
                    tgrp = T.ngroups > 1 ? tally + (long long)(pid % T.ngroups) * T.group_stride : tally;
                    g.init(T.seed, (uint64_t)pid);
                    int e = grid_generate(T, A.G, A.boxcell, g, pid, p);
                    if (CHECK && !e &&
                        (p.box < 0 || p.box >= T.nboxes || p.i < 0 || p.i >= A.G.nx || p.j < 0 || p.j >= A.G.ny))
                        e = E_CHECK;
                    if (e) {
                        record_error(err, e, pid);
                        done = true;
                    } else {
                        active = true;
                        nev = 0;
                        npass = 0;
                        if (ADJ) {
                            slot = mine;
                            phi_run = 0.;
                            pend_kind = 0;
                            if (ADJ == 2) phi_tot = adj.phi_total[mine];
                        }
                        bin = 0;
                        rb = __ldg(binw);
                        signbit = p.sign < 0 ? 0x8000000000000000ull : 0ull;
                        pd.start(p.box * T.nbins, rb, p.x, p.y);
                        new_flight(g.next32());  // the first flight, from the generation stream
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        // this pass's random words (used at its end); computed ahead of the
        // segment, with which it shares no data
        const uint4 rr = pass_block(npass++, (uint64_t)pid, T.seed);
        // segment end.  A zero velocity component takes the upper cell line,
        // so (line - position) >= 0 times its +inf inverse gives +inf (or NaN
        // on the line, ordered above +inf); a negative value (a position that
        // rounded past its line) orders below 0 and ends the segment at once.
        if (CHECK && (p.i < 0 || p.i >= A.G.nx || p.j < 0 || p.j >= A.G.ny || p.box < 0 || p.box >= T.nboxes ||
                      bin < 0 || bin > last_bin)) {
            check_fail();
            continue;
        }
        const int upx = ob(mv.vx) >= 0 ? 1 : 0;
        const int upy = ob(mv.vy) >= 0 ? 1 : 0;
        const double xw = __ldg(A.G.gx + p.i + upx);
        const double yw = __ldg(A.G.gy + p.j + upy);
        const double tx = (xw - p.x) * mv.ivx;
        const double ty = (yw - p.y) * mv.ivy;
        const double tb = rb;
        const bool xfirst = ob(tx) <= ob(ty);
        long long te_b = xfirst ? ob(tx) : ob(ty);
        long long tb_b = ob(tb);
        te_b = te_b > 0 ? te_b : 0;
        tb_b = tb_b > 0 ? tb_b : 0;
        const long long dt_b = ob(dt);
        const long long lim_b = te_b < tb_b ? te_b : tb_b;
        const bool flight_end = !(dt_b > lim_b);             // the flight ends first (or ties)
        const long long seg_b = flight_end ? dt_b : lim_b;
        const bool wall = !flight_end && te_b <= tb_b;         // reaches a cell line
        const bool bin_end = tb_b <= seg_b;                    // reaches the bin border
        const double seg = obd(seg_b);
        double r1 = rb - seg;
        double nx = fma(seg, mv.vx, p.x);
        double ny = fma(seg, mv.vy, p.y);
        dt -= seg;
        if (bin_end) r1 = 0.;
        int ni = p.i, nj = p.j, wside = 0;
        if (wall) {  // the crossed coordinate is the grid line
            if (xfirst) {
                nx = xw;
                ni = p.i + (upx ? 1 : -1);
                wside = upx ? 0 : 1;
            } else {
                ny = yw;
                nj = p.j + (upy ? 1 : -1);
                wside = upy ? 2 : 3;
            }
        }
        // spectral decomposition: the segment's time per mode at selected boxes
        if (ADJ == 0 && T.spec_loc) {
            const int loc = __ldg(T.spec_loc + p.box);
            if (loc >= 0) {
                const double ds = rb - r1;
                atomicAdd(T.spec + (long long)(loc * T.nbins + bin) * T.n + p.mode, p.sign < 0 ? -ds : ds);
            }
        }
        // differences of the pending tally at the segment end (telescoping)
        const double d0 = pd.r0 - r1, d1 = nx - pd.x0, d2 = ny - pd.y0;
        rb = r1;
        p.x = nx;
        p.y = ny;
        int nb = p.box;
        if (wall) nb = grid_cell(A.G, ni, nj);
        const bool move = wall && nb >= 0;        // into the next cell
        const bool absorbed = wall && nb <= -2;   // into a reservoir
        const bool reflect = wall && nb == -1;    // void: reflection, a new flight follows
        const bool last = bin_end && bin == last_bin;
        if (ADJ && (move || absorbed || bin_end)) {
            const double* Wk = adj.W + 3ll * pd.key;
            const double cphi = __ldg(Wk) * d0 + __ldg(Wk + 1) * d1 + __ldg(Wk + 2) * d2;
            phi_run += p.sign < 0 ? -cphi : cphi;
        }
        if (CHECK && (move || absorbed || bin_end) && (pd.key < 0 || pd.key >= T.nboxes * T.nbins)) {
            check_fail();
            continue;
        }
        if (CHECK && move && nb >= T.nboxes) {
            check_fail();
            continue;
        }
        if (move || absorbed || bin_end) {
            double* b = tgrp + 3ll * pd.key;
            atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(d0) ^ signbit));
            atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(d1) ^ signbit));
            atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(d2) ^ signbit));
            pd.flushes++;
            pd.key = -1;
        }
        if (absorbed || last) {
            if (absorbed) c.absorbed++;
            active = false;
            if (ADJ == 1) {
                adj.phi_total[slot] = phi_run;
                phi_all += phi_run;
            }
            continue;
        }
        if (bin_end) {
            ++bin;
            rb = __ldg(binw + bin);
        }
        if (move) {
            p.i = ni;
            p.j = nj;
            p.box = nb;
            c.crossings++;
        }
        if (move || bin_end) pd.start(p.box * T.nbins + bin, rb, nx, ny);
        if (reflect || flight_end) {
            // the next mode: a Lambert row at a void wall (or the mirror
            // mode on a specular draw), the post-scattering table after a
            // scattering (none for ballistic runs)
            const int k = p.mode;
            int nm = k;
            if (reflect || !T.ballistic) {
                float pr = 0.f;
                int keep = k, alt = k;
                if (reflect) {
                    // (selects, not an indexed parameter array, which would live in local memory)
                    const int cls =
                        wside == 0 ? A.cls[0] : wside == 1 ? A.cls[1] : wside == 2 ? A.cls[2] : A.cls[3];
                    if (cls < 0) {
                        record_error(err, E_GEOM, pid);
                        active = false;
                        done = true;
                        pd.flush(tgrp, signbit, rb, p.x, p.y);
                        continue;
                    }
                    if (CHECK && cls >= T.nclass) {
                        check_fail();
                        continue;
                    }
                    int mirror_mode = -1;
                    if (spec_thr) {
                        const bool spec = (unsigned long long)rr.w < spec_thr;
                        if (ADJ == 2) {
                            spec_score = spec ? 1.0 / T.specularity : -1.0 / (1.0 - T.specularity);
                            pend_kind |= 2;
                        }
                        if (spec && T.mirror) mirror_mode = __ldg(T.mirror + (long long)cls * T.n + k);
                    }
                    if (mirror_mode >= 0) {
                        c.specular++;
                        pr = 2.f;  // keep = the mirror mode whatever the acceptance word
                        keep = mirror_mode;
                    } else {
                        const long long a = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k);
                        const long long bb = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k + 1);
                        const int len = int(bb - a);
                        if (len <= 0) {
                            record_error(err, E_GEOM, pid);
                            active = false;
                            done = true;
                            pd.flush(tgrp, signbit, rb, p.x, p.y);
                            continue;
                        }
                        const int4 e = __ldg(T.lalias + a + int(mulhi32(rr.y, uint32_t(len))));
                        pr = __int_as_float(e.x);
                        keep = e.y;
                        alt = e.z;
                    }
                    c.wall_hits++;
                } else {
                    const int j = int(mulhi32(rr.y, uint32_t(T.n)));
                    pr = __ldg(T.resample_prob + p.mo + j);
                    keep = j;
                    alt = __ldg(T.resample_alt + p.mo + j);
                    if (ADJ == 2) pend_kind |= 1;
                }
                const float acc = float(rr.z >> 8) * 0x1p-24f;
                nm = acc < pr ? keep : alt;
            }
            p.mode = nm;
            if (!new_flight(rr.x)) continue;
        }
    }
    if (ADJ) {
        for (int o = 16; o > 0; o >>= 1) {
            sum_r += __shfl_down_sync(0xffffffffu, sum_r, o);
            g_p += __shfl_down_sync(0xffffffffu, g_p, o);
            phi_all += __shfl_down_sync(0xffffffffu, phi_all, o);
        }
        if (lane == 0) {
            atomicAdd(adj.g_scalar + 0, g_p);
            atomicAdd(adj.g_scalar + 1, sum_r);
            atomicAdd(adj.g_scalar + 2, phi_all);
        }
    }
    c.tallies = pd.flushes;
    flush_counters_p<8>(c, counters);  // no periodic boxes on the grid path
    if (SMEM_TALLY) {
        __syncthreads();
        for (int k = threadIdx.x; k < nk3; k += blockDim.x) {
            const double x = stally[k];
            if (x != 0.) atomicAdd(gtally + k, x);
        }
    }
}

// ------------------------------------------------ grid path, PPT per thread

// One particle slot of the interleaved grid kernel.
struct GridSlot {
    GridParticle p;
    Pending pd;
    Philox g;
    ModeVel mv;
    double* tb;  // the tally of the particle's replica group
    double dt, rb;
    long long pid, nev;
    uint32_t npass;
    int bin;
    unsigned long long signbit;
    bool active, done;
};

// The segment one slot takes in one pass.
struct GridSeg {
    uint4 rr;
    double r1, nx, ny, dt, d0, d1, d2;
    int ni, nj, wside;
    bool xfirst, flight_end, wall, bin_end;
};

// The plain production grid kernel (global tally, no spectral locations)
// with PPT particles per thread.  It follows rta_prod_grid's loop (same
// draws, same segments, same tallies) but splits every pass in two phases:
// first the segment of each slot, a straight-line FP64 sequence computed for
// every slot (a slot without a particle computes on its last state, whose
// indices stay in range, and drops the result), so that the FP64 chains of
// the PPT particles interleave and hide each other's latency; then, slot
// by slot, the branchy end of the segment (tally flush, crossing, wall or
// scattering redraw).  Each slot refills from the global particle counter
// on its own ballot.
template <int PPT, int MINB>
__global__ void __launch_bounds__(256, MINB) rta_prod_grid_ilp(DevTables T, GridArgs A, double* tally,
                                                         unsigned long long* counters, int* err,
                                                         unsigned long long* work) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const long long total = T.pend - T.pbegin;
    const int last_bin = T.nbins - 1;
    const unsigned long long spec_thr =
        T.specularity >= 1.0 ? (1ull << 32)
                             : (T.specularity > 0. ? (unsigned long long)(T.specularity * 4294967296.0) : 0ull);
    const double* binw = T.timegrid + T.ntime;
    GridSlot S[PPT];
#pragma unroll
    for (int s = 0; s < PPT; ++s) {
        GridSlot& L = S[s];
        L.pd.key = -1;
        L.pd.flushes = 0;
        L.pd.r0 = L.pd.x0 = L.pd.y0 = 0.;
        L.p.i = L.p.j = L.p.mode = L.p.box = L.p.mo = 0;
        L.p.sign = 1;
        L.p.x = L.p.y = L.p.t = 0.;
        L.g.init(0, 0);
        L.mv = ModeVel{0., 0., 0., 0.};
        L.dt = L.rb = 0.;
        L.pid = -1;
        L.tb = tally;
        L.nev = 0;
        L.npass = 0;
        L.bin = 0;
        L.signbit = 0;
        L.active = L.done = false;
    }
    // a new free flight of the slot's current mode from one random word (as
    // rta_prod_grid's new_flight); false when the particle stops with an error
    auto new_flight = [&](GridSlot& L, uint32_t word) -> bool {
        const int k = L.p.mode;
        L.mv = A.mv[k];
        const float ef = -logf((float(word >> 9) + 0.5f) * 0x1p-23f);
        L.dt = widen_pos(ef) * __ldg(T.tau + L.p.mo + k);
        c.events++;
        if (ob(L.dt) <= 0 || ++L.nev > T.flight_cap) {
            record_error(err, ob(L.dt) > 0 ? E_LIMIT : E_VALUE, L.pid);
            L.active = false;
            L.done = true;
            L.pd.flush(L.tb, L.signbit, L.rb, L.p.x, L.p.y);
            return false;
        }
        return true;
    };
    // the branchy end of one slot's segment
    auto finish = [&](GridSlot& L, const GridSeg& G) {
        L.dt = G.dt;
        L.rb = G.r1;
        L.p.x = G.nx;
        L.p.y = G.ny;
        int nb = L.p.box;
        if (G.wall) nb = grid_cell(A.G, G.ni, G.nj);
        const bool move = G.wall && nb >= 0;
        const bool absorbed = G.wall && nb <= -2;
        const bool reflect = G.wall && nb == -1;
        const bool last = G.bin_end && L.bin == last_bin;
        if (move || absorbed || G.bin_end) {
            double* b = L.tb + 3ll * L.pd.key;
            atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(G.d0) ^ L.signbit));
            atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(G.d1) ^ L.signbit));
            atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(G.d2) ^ L.signbit));
            L.pd.flushes++;
            L.pd.key = -1;
        }
        if (absorbed || last) {
            if (absorbed) c.absorbed++;
            L.active = false;
            return;
        }
        if (G.bin_end) {
            ++L.bin;
            L.rb = __ldg(binw + L.bin);
        }
        if (move) {
            L.p.i = G.ni;
            L.p.j = G.nj;
            L.p.box = nb;
            c.crossings++;
        }
        if (move || G.bin_end) L.pd.start(L.p.box * T.nbins + L.bin, L.rb, G.nx, G.ny);
        if (reflect || G.flight_end) {
            const int k = L.p.mode;
            int nm = k;
            if (reflect || !T.ballistic) {
                float pr = 0.f;
                int keep = k, alt = k;
                if (reflect) {
                    const int cls = G.wside == 0   ? A.cls[0]
                                    : G.wside == 1 ? A.cls[1]
                                    : G.wside == 2 ? A.cls[2]
                                                   : A.cls[3];
                    if (cls < 0) {
                        record_error(err, E_GEOM, L.pid);
                        L.active = false;
                        L.done = true;
                        L.pd.flush(L.tb, L.signbit, L.rb, L.p.x, L.p.y);
                        return;
                    }
                    int mirror_mode = -1;
                    if (spec_thr && (unsigned long long)G.rr.w < spec_thr && T.mirror)
                        mirror_mode = __ldg(T.mirror + (long long)cls * T.n + k);
                    if (mirror_mode >= 0) {
                        c.specular++;
                        pr = 2.f;
                        keep = mirror_mode;
                    } else {
                        const long long a = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k);
                        const long long bb = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k + 1);
                        const int len = int(bb - a);
                        if (len <= 0) {
                            record_error(err, E_GEOM, L.pid);
                            L.active = false;
                            L.done = true;
                            L.pd.flush(L.tb, L.signbit, L.rb, L.p.x, L.p.y);
                            return;
                        }
                        const int4 e = __ldg(T.lalias + a + int(mulhi32(G.rr.y, uint32_t(len))));
                        pr = __int_as_float(e.x);
                        keep = e.y;
                        alt = e.z;
                    }
                    c.wall_hits++;
                } else {
                    const int j = int(mulhi32(G.rr.y, uint32_t(T.n)));
                    pr = __ldg(T.resample_prob + L.p.mo + j);
                    keep = j;
                    alt = __ldg(T.resample_alt + L.p.mo + j);
                }
                const float acc = float(G.rr.z >> 8) * 0x1p-24f;
                nm = acc < pr ? keep : alt;
            }
            L.p.mode = nm;
            new_flight(L, G.rr.x);
        }
    };
    for (;;) {
#pragma unroll
        for (int s = 0; s < PPT; ++s) {
            GridSlot& L = S[s];
            const unsigned idle = __ballot_sync(0xffffffffu, !L.active && !L.done);
            if (idle) {
                unsigned long long base = 0;
                const int leader = __ffs(idle) - 1;
                if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!L.active && !L.done) {
                    const long long mine = (long long)base + __popc(idle & ((1u << lane) - 1u));
                    if (mine < total) {
                        L.pid = T.pbegin + mine;
                        L.tb = T.ngroups > 1 ? tally + (long long)(L.pid % T.ngroups) * T.group_stride : tally;
                        L.g.init(T.seed, (uint64_t)L.pid);
                        const int e = grid_generate(T, A.G, A.boxcell, L.g, L.pid, L.p);
                        if (e) {
                            record_error(err, e, L.pid);
                            L.done = true;
                        } else {
                            L.active = true;
                            L.nev = 0;
                            L.npass = 0;
                            L.bin = 0;
                            L.rb = __ldg(binw);
                            L.signbit = L.p.sign < 0 ? 0x8000000000000000ull : 0ull;
                            L.pd.start(L.p.box * T.nbins, L.rb, L.p.x, L.p.y);
                            new_flight(L, L.g.next32());
                        }
                    } else {
                        L.done = true;
                    }
                }
            }
        }
        bool finished = true;
#pragma unroll
        for (int s = 0; s < PPT; ++s) finished = finished && S[s].done;
        if (__all_sync(0xffffffffu, finished)) break;
        // phase 1: every slot's segment, straight-line
        GridSeg G[PPT];
#pragma unroll
        for (int s = 0; s < PPT; ++s) {
            GridSlot& L = S[s];
            GridSeg& q = G[s];
            q.rr = pass_block(L.npass, (uint64_t)L.pid, T.seed);
            L.npass += L.active ? 1u : 0u;
            const int upx = ob(L.mv.vx) >= 0 ? 1 : 0;
            const int upy = ob(L.mv.vy) >= 0 ? 1 : 0;
            const double xw = __ldg(A.G.gx + L.p.i + upx);
            const double yw = __ldg(A.G.gy + L.p.j + upy);
            const double tx = (xw - L.p.x) * L.mv.ivx;
            const double ty = (yw - L.p.y) * L.mv.ivy;
            q.xfirst = ob(tx) <= ob(ty);
            long long te_b = q.xfirst ? ob(tx) : ob(ty);
            long long tb_b = ob(L.rb);
            te_b = te_b > 0 ? te_b : 0;
            tb_b = tb_b > 0 ? tb_b : 0;
            const long long dt_b = ob(L.dt);
            const long long lim_b = te_b < tb_b ? te_b : tb_b;
            q.flight_end = !(dt_b > lim_b);
            const long long seg_b = q.flight_end ? dt_b : lim_b;
            q.wall = !q.flight_end && te_b <= tb_b;
            q.bin_end = tb_b <= seg_b;
            const double seg = obd(seg_b);
            q.r1 = q.bin_end ? 0. : L.rb - seg;
            q.nx = fma(seg, L.mv.vx, L.p.x);
            q.ny = fma(seg, L.mv.vy, L.p.y);
            q.dt = L.dt - seg;
            q.ni = L.p.i;
            q.nj = L.p.j;
            q.wside = 0;
            if (q.wall) {
                if (q.xfirst) {
                    q.nx = xw;
                    q.ni = L.p.i + (upx ? 1 : -1);
                    q.wside = upx ? 0 : 1;
                } else {
                    q.ny = yw;
                    q.nj = L.p.j + (upy ? 1 : -1);
                    q.wside = upy ? 2 : 3;
                }
            }
            q.d0 = L.pd.r0 - q.r1;
            q.d1 = q.nx - L.pd.x0;
            q.d2 = q.ny - L.pd.y0;
        }
        // phase 2: the ends of the segments, slot by slot
#pragma unroll
        for (int s = 0; s < PPT; ++s)
            if (S[s].active) finish(S[s], G[s]);
    }
    unsigned flushes = 0;
#pragma unroll
    for (int s = 0; s < PPT; ++s) flushes += S[s].pd.flushes;
    c.tallies = flushes;
    flush_counters_p<8>(c, counters);
}

// ------------------------------------------------------------ polygon path

// Production loop of geometries that are not a grid: the grid kernel's
// organisation (persistent warps refilling idle lanes, one segment per lane
// per pass, time left in the bin, telescoping pending tally, one Philox block
// per pass, one mode-redraw block) with the convex box's border lines in
// place of cell lines.  A segment ends at the flight end, the bin border or
// the first border line the flight leaves through (n.v > 0, exit time
// (c - n.x) / n.v, compared without divisions); across that border the
// piece holding the exit point names the neighbour: a box (the flight goes
// on there), a reservoir (absorbed), a periodic box (translated as
// geometry_2d::translate does, the flight goes on) or none (a void wall:
// Lambert or specular redraw).  The reference's handling of corners and ties
// between borders, which has measure zero, is not repeated here.  A flight
// that runs more than POLY_SEG_CAP segments stops the run with E_LIMIT.
constexpr uint32_t POLY_SEG_CAP = 1u << 20;
__global__ void __launch_bounds__(256) rta_prod_poly(DevTables T, PolyArgs A, double* tally,
                                                      unsigned long long* counters, int* err,
                                                      unsigned long long* work) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    const long long total = T.pend - T.pbegin;
    const int last_bin = T.nbins - 1;
    const unsigned long long spec_thr =
        T.specularity >= 1.0 ? (1ull << 32)
                             : (T.specularity > 0. ? (unsigned long long)(T.specularity * 4294967296.0) : 0ull);
    Pending pd;
    pd.key = -1;
    pd.flushes = 0;
    pd.r0 = pd.x0 = pd.y0 = 0.;
    ProdPolicy pol;  // generation and translation draws
    pol.g.init(0, 0);
    pol.out = tally;
    pol.ntally = 0;
    Particle p;
    p.pos = v2(0., 0.);
    p.mode = p.box = p.mo = 0;
    p.sign = 1;
    p.t = 0.;
    ModeVel mv = {0., 0., 0., 0.};
    const double* binw = T.timegrid + T.ntime;
    double dt = 0., rb = 0.;
    long long pid = -1, nev = 0;
    uint32_t npass = 0, nseg = 0;
    int bin = 0;
    unsigned long long signbit = 0;
    bool active = false, done = false;
    auto new_flight = [&](uint32_t word) -> bool {
        const int k = p.mode;
        mv = A.mv[k];
        const float ef = -logf((float(word >> 9) + 0.5f) * 0x1p-23f);
        dt = widen_pos(ef) * __ldg(T.tau + p.mo + k);
        c.events++;
        nseg = 0;
        if (ob(dt) <= 0 || ++nev > T.flight_cap) {  // zero rate or runaway particle
            record_error(err, ob(dt) > 0 ? E_LIMIT : E_VALUE, pid);
            active = false;
            done = true;
            pd.flush(tally, signbit, rb, p.pos.x, p.pos.y);
            return false;
        }
        return true;
    };
    for (;;) {
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
                    pol.g.init(T.seed, (uint64_t)pid);
                    const int e = generate(T, pol, pid, p);
                    if (e) {
                        record_error(err, e, pid);
                        done = true;
                    } else {
                        active = true;
                        nev = 0;
                        npass = 0;
                        bin = 0;
                        rb = __ldg(binw);
                        signbit = p.sign < 0 ? 0x8000000000000000ull : 0ull;
                        pd.start(p.box * T.nbins, rb, p.pos.x, p.pos.y);
                        new_flight(pol.g.next32());  // the first flight, from the generation stream
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        const uint4 rr = pass_block(npass++, (uint64_t)pid, T.seed);
        if (++nseg > POLY_SEG_CAP) {  // a flight that keeps meeting borders without advancing
            record_error(err, E_LIMIT, pid);
            active = false;
            done = true;
            continue;
        }
        // the first border line the flight leaves through: smallest
        // num / den over the borders with den = n.v > 0, num = c - n.x >= 0
        const GBox& B = T.boxes[p.box];
        int best = -1;
        double te = HUGE_VAL;
        // an axis-aligned rectangle: the cell-line test of the grid kernel,
        // the line ahead in x and in y (a zero velocity component has
        // 1/v = +inf and never exits), the nearer one first on ties
        PolyRect R;
        R.kx1 = -1;
        if (A.rect) R = A.rect[p.box];
        const bool rectb = R.kx1 >= 0;
        bool xfirst = false;
        double xw = 0., yw = 0.;
        int side_nb = -2, side_fl = 0, side_cls = 0;  // what lies across the exit side
        if (rectb) {
            const bool upx = ob(mv.ivx) >= 0, upy = ob(mv.ivy) >= 0;
            xw = upx ? R.x1 : R.x0;
            yw = upy ? R.y1 : R.y0;
            long long bx = ob((xw - p.pos.x) * mv.ivx), by = ob((yw - p.pos.y) * mv.ivy);
            bx = bx > 0 ? bx : 0;
            by = by > 0 ? by : 0;
            // a strip spanning the period never exits through those sides:
            // its flight wraps (below) instead of translating side by side
            if (R.perx) bx = ob(HUGE_VAL);
            if (R.pery) by = ob(HUGE_VAL);
            xfirst = bx <= by;
            best = xfirst ? (upx ? R.kx1 : R.kx0) : (upy ? R.ky1 : R.ky0);
            side_nb = xfirst ? (upx ? R.nx1 : R.nx0) : (upy ? R.ny1 : R.ny0);
            side_fl = xfirst ? (upx ? R.fx1 : R.fx0) : (upy ? R.fy1 : R.fy0);
            side_cls = xfirst ? (upx ? R.cx1 : R.cx0) : (upy ? R.cy1 : R.cy0);
            te = obd(xfirst ? bx : by);
        } else if (A.inv_den) {
            // 1 / den from the table of the border's normal class: one
            // multiplication per border, compared as integers (both >= 0)
            const double* inv = A.inv_den + p.mode;
            for (int k = 0; k < B.nborders; ++k) {
                const PolyBorder& L = A.pb[B.border_off + k];
                const double iv = __ldg(inv + (long long)L.cls * T.n);
                double num = L.c - (L.nx * p.pos.x + L.ny * p.pos.y);
                num = num > 0. ? num : 0.;
                const double tk = num * iv;
                if (iv > 0. && ob(tk) < ob(te)) {
                    best = k;
                    te = tk;
                }
            }
        } else {
            double bnum = 0., bden = 1.;
            for (int k = 0; k < B.nborders; ++k) {
                const PolyBorder& L = A.pb[B.border_off + k];
                const double den = L.nx * mv.vx + L.ny * mv.vy;
                if (!(den > 0.)) continue;
                double num = L.c - (L.nx * p.pos.x + L.ny * p.pos.y);
                num = num > 0. ? num : 0.;
                if (best < 0 || num * bden < bnum * den) {
                    best = k;
                    bnum = num;
                    bden = den;
                }
            }
            te = best >= 0 ? bnum / bden : HUGE_VAL;
        }
        // time bins that end before the flight end and the exit border are
        // closed here, without a pass each: advance to the bin end, flush
        // the pending tally, open the next bin (two FMAs per bin instead of
        // a new exit-time search).  The last bin is left to the pass below.
        {
            long long lim0 = ob(te) < ob(dt) ? ob(te) : ob(dt);
            while (ob(rb) < lim0 && bin < last_bin) {
                const double adv = ob(rb) > 0 ? rb : 0.;
                const double xb = fma(adv, mv.vx, p.pos.x);
                const double yb = fma(adv, mv.vy, p.pos.y);
                if (T.spec_loc) {
                    const int loc = __ldg(T.spec_loc + p.box);
                    if (loc >= 0)
                        atomicAdd(T.spec + (long long)(loc * T.nbins + bin) * T.n + p.mode, p.sign < 0 ? -adv : adv);
                }
                double* b = tally + 3ll * pd.key;
                atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(pd.r0) ^ signbit));
                atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(xb - pd.x0) ^ signbit));
                atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(yb - pd.y0) ^ signbit));
                pd.flushes++;
                dt -= adv;
                te -= adv;
                p.pos = v2(xb, yb);
                ++bin;
                rb = __ldg(binw + bin);
                pd.start(p.box * T.nbins + bin, rb, xb, yb);
                lim0 = ob(te) < ob(dt) ? ob(te) : ob(dt);
            }
        }
        long long te_b = ob(te);
        long long tb_b = ob(rb);
        tb_b = tb_b > 0 ? tb_b : 0;
        const long long dt_b = ob(dt);
        const long long lim_b = te_b < tb_b ? te_b : tb_b;
        const bool flight_end = !(dt_b > lim_b);
        const long long seg_b = flight_end ? dt_b : lim_b;
        const bool wall = !flight_end && te_b <= tb_b;
        const bool bin_end = tb_b <= seg_b;
        const double seg = obd(seg_b);
        double r1 = rb - seg;
        double nx = fma(seg, mv.vx, p.pos.x);
        double ny = fma(seg, mv.vy, p.pos.y);
        dt -= seg;
        if (bin_end) r1 = 0.;
        if (rectb && (R.perx | R.pery)) {
            // the translations the flight made in a strip spanning the
            // period: back into the box by whole periods, the pending
            // tally's start shifted alike (its displacement is the flight's)
            if (R.perx && (nx >= R.x1 || nx < R.x0)) {
                const double W = R.x1 - R.x0, k = floor((nx - R.x0) / W);
                nx -= k * W;
                pd.x0 -= k * W;
                c.translations += (unsigned)fabs(k);
            }
            if (R.pery && (ny >= R.y1 || ny < R.y0)) {
                const double H = R.y1 - R.y0, k = floor((ny - R.y0) / H);
                ny -= k * H;
                pd.y0 -= k * H;
                c.translations += (unsigned)fabs(k);
            }
        }
        // what lies across the exit border
        int target = -1, cls = 0, dmm_t = -1, tflags = 0;
        if (wall && rectb && side_nb != -2) {
            // a side that is void or one neighbour: no piece lookup
            if (xfirst) nx = xw;
            else ny = yw;
            target = side_nb;
            tflags = side_fl;
            cls = side_cls;
        } else if (wall) {
            const PolyBorder& L = A.pb[B.border_off + best];
            cls = L.cls;
            // onto the border line
            double sx;
            if (rectb) {
                if (xfirst) {
                    nx = xw;
                    sx = (ny - L.py) * L.uy;
                } else {
                    ny = yw;
                    sx = (nx - L.px) * L.ux;
                }
            } else {
                const double off = L.nx * nx + L.ny * ny - L.c;
                nx -= off * L.nx;
                ny -= off * L.ny;
                sx = (nx - L.px) * L.ux + (ny - L.py) * L.uy;
            }
            for (int j = 0; j < L.npieces; ++j) {
                const PolyPiece pc = A.pieces[L.piece_off + j];
                if (sx >= pc.s0 && sx <= pc.s1) {
                    target = pc.box;
                    dmm_t = pc.pad;
                    break;
                }
            }
            if (target >= 0) tflags = (T.boxes[target].reservoir ? 1 : 0) | (T.boxes[target].tto >= 0 ? 2 : 0);
        }
        // a contact between crystals (change_material_diffuse,
        // src/RTA_MC2D.cpp:871-964): the interface's table re-emits the
        // particle on either side (Diffuse_mismatch_distribution::reemit,
        // src/sampling.cpp:831-902: p uniform between the first and the last
        // cumulative value of the incident mode's entries, the first entry
        // not below p); the flight ends there.  Without entries the particle
        // crosses in its mode, as the reference's 'X'.
        const bool iface = wall && target >= 0 && dmm_t >= 0 && A.dmm_row;
        bool dmm_back = false;
        int dmm_mode = -1;
        if (iface) {
            const long long* row = A.dmm_row + (long long)dmm_t * (T.n + 1);
            const long long e0 = __ldg(row + p.mode), e1 = __ldg(row + p.mode + 1);
            if (e1 > e0) {
                const double lo = A.dmm_ent[e0].cum, hi = A.dmm_ent[e1 - 1].cum;
                const double u = double((((unsigned long long)rr.y << 32) | rr.z) >> 11) * 0x1p-53;
                const double pp = u * (hi - lo) + lo;
                long long a = e0, b = e1 - 1;
                while (a < b) {
                    const long long mid = (a + b) >> 1;
                    if (A.dmm_ent[mid].cum >= pp) b = mid;
                    else a = mid + 1;
                }
                const DmmEnt en = A.dmm_ent[a];
                dmm_mode = en.out;
                dmm_back = en.side == 0;
            } else {  // no entries: across with the index kept within the crystal
                c.quirks++;
                dmm_mode = dmm_same_index(T, p.mode, T.box_mat[p.box], T.box_mat[target]);
                if (dmm_mode < 0) {
                    record_error(err, E_VALUE, pid);
                    active = false;
                    done = true;
                    continue;
                }
            }
            c.ifc_hits++;
            if (!dmm_back) c.ifc_trans++;
        }
        if (T.spec_loc) {
            const int loc = __ldg(T.spec_loc + p.box);
            if (loc >= 0) {
                const double ds = rb - r1;
                atomicAdd(T.spec + (long long)(loc * T.nbins + bin) * T.n + p.mode, p.sign < 0 ? -ds : ds);
            }
        }
        const double d0 = pd.r0 - r1, d1 = nx - pd.x0, d2 = ny - pd.y0;
        rb = r1;
        p.pos = v2(nx, ny);
        const bool cross = wall && target >= 0 && !dmm_back;
        const bool absorbed = cross && (tflags & 1);
        const bool periodic = cross && !absorbed && (tflags & 2);
        const bool move = cross && !absorbed;
        const bool reflect = wall && target < 0;
        const bool last = bin_end && bin == last_bin;
        if (move || absorbed || bin_end) {
            double* b = tally + 3ll * pd.key;
            atomicAdd(b + 0, __longlong_as_double(__double_as_longlong(d0) ^ signbit));
            atomicAdd(b + 1, __longlong_as_double(__double_as_longlong(d1) ^ signbit));
            atomicAdd(b + 2, __longlong_as_double(__double_as_longlong(d2) ^ signbit));
            pd.flushes++;
            pd.key = -1;
        }
        if (absorbed || last) {
            if (absorbed) c.absorbed++;
            active = false;
            continue;
        }
        if (bin_end) {
            ++bin;
            rb = __ldg(binw + bin);
        }
        if (move) {
            int nb = target;
            if (periodic) {  // translated into the target of the periodic box
                V2 rf;
                const int e = translate<ProdPolicy, true>(T, pol, target, p.pos, v2(mv.vx, mv.vy), nb, rf);
                if (e) {
                    record_error(err, e, pid);
                    active = false;
                    done = true;
                    continue;
                }
                p.pos = rf;
                c.translations++;
            }
            p.box = nb;
            p.mo = mat_off(T, nb);
            c.crossings++;
        }
        if (move || bin_end) pd.start(p.box * T.nbins + bin, rb, p.pos.x, p.pos.y);
        if (iface) {  // a new flight in the re-emitted mode
            if (dmm_mode >= 0) p.mode = dmm_mode;
            if (!new_flight(rr.x)) continue;
        } else if (reflect || flight_end) {
            const int k = p.mode;
            int nm = k;
            if (reflect || !T.ballistic) {
                float pr = 0.f;
                int keep = k, alt = k;
                if (reflect) {
                    int mirror_mode = -1;
                    if (spec_thr && (unsigned long long)rr.w < spec_thr && T.mirror)
                        mirror_mode = __ldg(T.mirror + (long long)cls * T.n + k);
                    if (mirror_mode >= 0) {
                        c.specular++;
                        pr = 2.f;
                        keep = mirror_mode;
                    } else {
                        const long long a = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k);
                        const long long bb = __ldg(T.row_ptr + (long long)cls * (T.n + 1) + k + 1);
                        const int len = int(bb - a);
                        if (len <= 0) {
                            record_error(err, E_GEOM, pid);
                            active = false;
                            done = true;
                            continue;
                        }
                        const int4 e = __ldg(T.lalias + a + int(mulhi32(rr.y, uint32_t(len))));
                        pr = __int_as_float(e.x);
                        keep = e.y;
                        alt = e.z;
                    }
                    c.wall_hits++;
                } else {
                    const int j = int(mulhi32(rr.y, uint32_t(T.n)));
                    pr = __ldg(T.resample_prob + p.mo + j);
                    keep = j;
                    alt = __ldg(T.resample_alt + p.mo + j);
                }
                const float acc = float(rr.z >> 8) * 0x1p-24f;
                nm = acc < pr ? keep : alt;
            }
            p.mode = nm;
            if (!new_flight(rr.x)) continue;
        }
    }
    c.tallies = pd.flushes;
    flush_counters_p<13>(c, counters);
}

bool launch_prod_poly(const DevTables& T, const PolyArgs& A, double* tally, unsigned long long* counters,
                      int* err, unsigned long long* work, int nsm, cudaStream_t s) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return true;
    int maxb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, rta_prod_poly, 256, 0);
    if (maxb < 1) return false;
    long long blocks = (long long)nsm * maxb;
    const long long need = (n + 255) / 256;
    if (blocks > need) blocks = need;
    rta_prod_poly<<<unsigned(blocks), 256, 0, s>>>(T, A, tally, counters, err, work);
    return true;
}

// One steady-state generation on convex boxes, the polygon kernel's segment
// walk: each slot's one flight runs box to box by exit times against the
// border lines (one box visit per pass, tallied at its end as the reference's
// periodic process_segment does) until it scatters inside a box (phi +=
// sign), reaches a void wall (redrawn and carried over), enters a reservoir
// (absorbed) or a periodic box (translated, the flight goes on).  With
// crystals (PA.dmm_row), a contact between crystals re-emits the particle
// and carries it over as a void wall does.
__global__ void __launch_bounds__(128) rta_steady_poly(DevTables T, SteadyArgs A, PolyArgs PA, double* tally,
                                                       unsigned long long* counters, int* err) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int lane = threadIdx.x & 31;
    ProdPolicy pol;
    pol.g.init(0, 0);
    pol.out = tally;
    pol.ntally = 0;
    Particle p;
    p.pos = v2(0., 0.);
    p.mode = p.box = p.mo = 0;
    p.sign = 1;
    p.t = 0.;
    V2 v = v2(0., 0.);
    double dt = 0.;
    long long slot = -1;
    uint32_t nseg = 0;
    bool active = false, done = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active && !done);
        if (idle) {
            unsigned long long base = 0;
            const int leader = __ffs(idle) - 1;
            if (lane == leader) base = atomicAdd(A.work, (unsigned long long)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && !done) {
                slot = (long long)base + __popc(idle & ((1u << lane) - 1u));
                if (slot < A.n) {
                    pol.g.init(T.seed, steady_stream(A.gen, slot));
                    const int e = steady_begin(T, A, pol, slot, c, p, v, dt);
                    if (e) {
                        record_error(err, e, slot);
                        A.flag[slot] = 0;
                    } else {
                        active = true;
                        nseg = 0;
                        if (PA.dmm_row) {
                            // carried over across an interface into a
                            // reservoir (absorbed) or a periodic box
                            // (translated), as the next evolparticle call
                            // does (src/RTA_MC2D.cpp:1449-1467)
                            const GBox& B0 = T.boxes[p.box];
                            if (B0.reservoir) {
                                c.absorbed++;
                                steady_emit(A, slot, FATE_ABSORBED, p);
                                active = false;
                            } else if (B0.tto >= 0) {
                                V2 rf;
                                int nb = p.box;
                                const int e2 = translate<ProdPolicy, true>(T, pol, p.box, p.pos, v, nb, rf);
                                if (e2) {
                                    record_error(err, e2, slot);
                                    A.flag[slot] = 0;
                                    active = false;
                                } else {
                                    p.pos = rf;
                                    p.box = nb;
                                    p.mo = mat_off(T, nb);
                                    c.translations++;
                                }
                            }
                        }
                    }
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (!active) continue;
        if (++nseg > POLY_SEG_CAP) {
            record_error(err, E_LIMIT, slot);
            A.flag[slot] = 0;
            active = false;
            continue;
        }
        const GBox& B = T.boxes[p.box];
        int best = -1;
        double bnum = 0., bden = 1.;
        for (int k = 0; k < B.nborders; ++k) {
            const PolyBorder& L = PA.pb[B.border_off + k];
            const double den = L.nx * v.x + L.ny * v.y;
            if (!(den > 0.)) continue;
            double num = L.c - (L.nx * p.pos.x + L.ny * p.pos.y);
            num = num > 0. ? num : 0.;
            if (best < 0 || num * bden < bnum * den) {
                best = k;
                bnum = num;
                bden = den;
            }
        }
        const double te = best >= 0 ? bnum / bden : HUGE_VAL;
        const bool wall = dt > te;
        const double seg = wall ? te : dt;
        double nx = fma(seg, v.x, p.pos.x);
        double ny = fma(seg, v.y, p.pos.y);
        dt -= seg;
        int target = -1, cls = 0, dmm_t = -1;
        if (wall) {
            const PolyBorder& L = PA.pb[B.border_off + best];
            cls = L.cls;
            const double off = L.nx * nx + L.ny * ny - L.c;
            nx -= off * L.nx;
            ny -= off * L.ny;
            const double sx = (nx - L.px) * L.ux + (ny - L.py) * L.uy;
            for (int j = 0; j < L.npieces; ++j) {
                const PolyPiece pc = PA.pieces[L.piece_off + j];
                if (sx >= pc.s0 && sx <= pc.s1) {
                    target = pc.box;
                    dmm_t = pc.pad;
                    break;
                }
            }
        }
        pol.tally_dt(T, p.box, seg, p.sign, v, p.mode);
        p.pos = v2(nx, ny);
        int fate = -1;
        if (!wall) {  // scattering inside the box
            fate = FATE_SCATTER;
            c.scattered++;
        } else if (target < 0) {  // void wall: the new mode, carried to the next generation
            int nm = -1;
            if (T.specularity > 0. && pol.u() < T.specularity) {
                const int mm = T.mirror ? T.mirror[cls * T.n + p.mode] : -1;
                if (mm >= 0) {
                    nm = mm;
                    c.specular++;
                }
            }
            if (nm < 0) nm = pol.bounce(T, cls, p.mode);
            if (nm < 0) {
                record_error(err, E_GEOM, slot);
                A.flag[slot] = 0;
                active = false;
                continue;
            }
            p.mode = nm;
            c.wall_hits++;
            fate = FATE_BOUNCE;
        } else if (dmm_t >= 0 && PA.dmm_row) {
            // a contact between crystals (change_material_diffuse in the
            // periodic evolparticle, src/RTA_MC2D.cpp:1672-1689, 1751-1779):
            // the interface's table re-emits the particle on either side
            // (Diffuse_mismatch_distribution::reemit, src/sampling.cpp:
            // 831-902) and it joins the next generation; an incident mode
            // without entries crosses in its mode, as the reference's 'X'
            const long long* row = PA.dmm_row + (long long)dmm_t * (T.n + 1);
            const long long e0 = __ldg(row + p.mode), e1 = __ldg(row + p.mode + 1);
            bool across = true;
            if (e1 > e0) {
                const double lo = PA.dmm_ent[e0].cum, hi = PA.dmm_ent[e1 - 1].cum;
                const double pp = pol.u() * (hi - lo) + lo;
                long long a = e0, b = e1 - 1;
                while (a < b) {
                    const long long mid = (a + b) >> 1;
                    if (PA.dmm_ent[mid].cum >= pp) b = mid;
                    else a = mid + 1;
                }
                const DmmEnt en = PA.dmm_ent[a];
                p.mode = en.out;
                across = en.side != 0;
            } else {  // no entries: across with the index kept within the crystal
                c.quirks++;
                const int k = dmm_same_index(T, p.mode, T.box_mat[p.box], T.box_mat[target]);
                if (k < 0) {
                    record_error(err, E_VALUE, slot);
                    A.flag[slot] = 0;
                    active = false;
                    continue;
                }
                p.mode = k;
            }
            c.ifc_hits++;
            if (across) {
                c.ifc_trans++;
                p.box = target;
                p.mo = mat_off(T, target);
            }
            fate = FATE_BOUNCE;
        } else if (T.boxes[target].reservoir) {
            c.absorbed++;
            fate = FATE_ABSORBED;
        } else {
            int nb = target;
            if (T.boxes[target].tto >= 0) {
                V2 rf;
                const int e = translate<ProdPolicy, true>(T, pol, target, p.pos, v, nb, rf);
                if (e) {
                    record_error(err, e, slot);
                    A.flag[slot] = 0;
                    active = false;
                    continue;
                }
                p.pos = rf;
                c.translations++;
            }
            p.box = nb;
            p.mo = mat_off(T, nb);
            c.crossings++;
        }
        if (fate >= 0) {
            steady_emit(A, slot, fate, p);
            active = false;
        }
    }
    c.tallies += pol.ntally;
    flush_counters_p<13>(c, counters);
}

bool launch_steady_poly(const DevTables& T, const SteadyArgs& A, const PolyArgs& PA, double* tally,
                        unsigned long long* counters, int* err, int nsm, cudaStream_t s) {
    if (A.n <= 0) return true;
    int maxb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, rta_steady_poly, 128, 0);
    if (maxb < 1) return false;
    long long blocks = (long long)nsm * maxb;
    const long long need = (A.n + 127) / 128;
    if (blocks > need) blocks = need;
    cudaMemsetAsync(A.work, 0, sizeof(unsigned long long), s);
    rta_steady_poly<<<unsigned(blocks), 128, 0, s>>>(T, A, PA, tally, counters, err);
    return true;
}

bool launch_prod_grid(const DevTables& T, const GridArgs& A, double* tally,
                      unsigned long long* counters, int* err, unsigned long long* work,
                      const ProdTuning& tune, int nsm, cudaStream_t s, int adj_pass,
                      const AdjArgs* adj) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return true;
    const int threads = tune.block_threads > 0 ? tune.block_threads : 256;
    if (threads > 256 || threads % 32) return false;
    const size_t smem = size_t(3) * T.nboxes * T.nbins * sizeof(double);
    // the adjoint passes run with the tally in global memory
    const bool use_smem = tune.smem_tally != 0 && smem <= 200 * 1024 && adj_pass == 0 && T.ngroups <= 1;
    // residency variants: 4 blocks of 256 threads per SM (64 registers, a
    // few spills), 3 (80 registers) or 2 (no register cap); the
    // shared-memory tally allows one block per SM
    int bps = tune.blocks_per_sm > 0 ? tune.blocks_per_sm : (use_smem ? 1 : 3);
    const AdjArgs none{};
    const AdjArgs& aa = adj ? *adj : none;
    if (T.checks && adj_pass == 0) {  // the checked variant, at its own residency
        int maxb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, rta_prod_grid<false, 2, 0, true>, 256, 0);
        if (maxb < 1) return false;
        long long blocks = (long long)nsm * (maxb < 2 ? maxb : 2);
        const long long need = (n + 255) / 256;
        if (blocks > need) blocks = need;
        rta_prod_grid<false, 2, 0, true><<<unsigned(blocks), 256, 0, s>>>(T, A, tally, counters, err, work, aa);
        return true;
    }
    if (tune.particles_per_thread == 2 && adj_pass == 0 && !use_smem && !T.spec_loc) {
        // two particles per thread: the register cap follows the resident
        // threads (152 registers up to 384 threads per SM, 128 above)
        const bool capped = threads * bps > 384;
        const void* f2 = capped ? reinterpret_cast<const void*>(rta_prod_grid_ilp<2, 2>)
                                : reinterpret_cast<const void*>(rta_prod_grid_ilp<2, 1>);
        int maxb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, f2, threads, 0);
        if (maxb < 1) return false;
        const int b2 = bps > maxb ? maxb : bps;
        long long blocks = (long long)nsm * b2;
        const long long need = (n + 2ll * threads - 1) / (2ll * threads);
        if (blocks > need) blocks = need;
        if (blocks < 1) blocks = 1;
        if (capped)
            rta_prod_grid_ilp<2, 2><<<unsigned(blocks), threads, 0, s>>>(T, A, tally, counters, err, work);
        else
            rta_prod_grid_ilp<2, 1><<<unsigned(blocks), threads, 0, s>>>(T, A, tally, counters, err, work);
        return true;
    }
    const void* fn;
    if (use_smem) {
        fn = reinterpret_cast<const void*>(rta_prod_grid<true, 1, 0>);
        if (cudaFuncSetAttribute(rta_prod_grid<true, 1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(smem)) != cudaSuccess)
            return false;
    } else if (adj_pass == 1) {
        fn = reinterpret_cast<const void*>(rta_prod_grid<false, 2, 1>);
    } else if (adj_pass == 2) {
        fn = reinterpret_cast<const void*>(rta_prod_grid<false, 2, 2>);
    } else if (threads * bps > 768) {  // the register cap follows the resident threads
        fn = reinterpret_cast<const void*>(rta_prod_grid<false, 4, 0>);
    } else if (threads * bps > 512) {
        fn = reinterpret_cast<const void*>(rta_prod_grid<false, 3, 0>);
    } else {
        fn = reinterpret_cast<const void*>(rta_prod_grid<false, 2, 0>);
    }
    int maxb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, fn, threads, use_smem ? smem : 0);
    if (maxb < 1) return false;
    if (bps > maxb) bps = maxb;
    long long blocks = (long long)nsm * bps;
    const long long need = (n + threads - 1) / threads;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    const unsigned nb = unsigned(blocks);
    if (use_smem)
        rta_prod_grid<true, 1, 0><<<nb, threads, smem, s>>>(T, A, tally, counters, err, work, aa);
    else if (adj_pass == 1)
        rta_prod_grid<false, 2, 1><<<nb, threads, 0, s>>>(T, A, tally, counters, err, work, aa);
    else if (adj_pass == 2)
        rta_prod_grid<false, 2, 2><<<nb, threads, 0, s>>>(T, A, tally, counters, err, work, aa);
    else if (fn == reinterpret_cast<const void*>(rta_prod_grid<false, 4, 0>))
        rta_prod_grid<false, 4, 0><<<nb, threads, 0, s>>>(T, A, tally, counters, err, work, aa);
    else if (fn == reinterpret_cast<const void*>(rta_prod_grid<false, 3, 0>))
        rta_prod_grid<false, 3, 0><<<nb, threads, 0, s>>>(T, A, tally, counters, err, work, aa);
    else
        rta_prod_grid<false, 2, 0><<<nb, threads, 0, s>>>(T, A, tally, counters, err, work, aa);
    return true;
}

}  // namespace bte
