// rta_replay.cu - deterministic replay mode of the RTA particle loop.
//
// Compiled with -fmad=false: every floating-point operation is a separate
// IEEE-754 operation, as in the CPU restatement (g++ -ffp-contract=off), so
// positions, times and tally contributions agree bit for bit.  Draws come
// from one pcg64 stream per particle; distributions are inverted with
// lower_bound as Grid_distribution::sample does (include/sampling.hpp:92-114);
// tallies are exact 128-bit fixed-point sums, independent of thread order.
#include "rta_flight.cuh"
#include "rta_steady.cuh"
#include "kernels.h"

namespace bte {

__device__ __forceinline__ double mx(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }  // std::min

// Order-independent 128-bit accumulation: p[0] = high word, p[1] = low word.
__device__ __forceinline__ void add128(unsigned long long* p, long long q) {
    const unsigned long long lo_add = (unsigned long long)q;
    const unsigned long long hi_add = q < 0 ? ~0ull : 0ull;
    const unsigned long long old = atomicAdd(p + 1, lo_add);
    const unsigned long long carry = (old + lo_add < old) ? 1ull : 0ull;
    const unsigned long long h = hi_add + carry;
    if (h) atomicAdd(p, h);
}

struct ReplayPolicy {
    Pcg64 g;
    unsigned long long* ex;
    unsigned long long ntally;

    __device__ double u() { return canonical_from(g.next()); }
    __device__ int choose(int n) { return uniform_below(g, uint32_t(n)); }
    __device__ double flight(const DevTables& T, int k) {
        const double uu = u();
        return -bte_log(uu) / T.w[k];  // k: material offset + mode
    }
    __device__ int resample(const DevTables& T, int mo) {
        return lower_bound_d(T.resample_cdf + mo, T.n, u());
    }
    __device__ int gen_mode(const DevTables& T, int gi) {
        return lower_bound_d(T.gen_cdf + (long long)gi * T.n, T.n, u());
    }
    __device__ int bounce(const DevTables& T, int cls, int mode) {
        const long long a = T.row_ptr[(long long)cls * (T.n + 1) + mode];
        const long long b = T.row_ptr[(long long)cls * (T.n + 1) + mode + 1];
        const int len = int(b - a);
        if (len <= 0) return -1;
        const double s = u();
        int j = lower_bound_d(T.lcdf + a, len, s);
        if (j == len) j = len - 1;
        return T.lcol[a + j];
    }
    // Grid_distribution::sample over a CDF (the alias arguments are unused)
    __device__ int dist(const double* cdf, const float*, const int*, int n) {
        return lower_bound_d(cdf, n, u());
    }
    // process_segment (periodic), src/RTA_MC2D.cpp:784-834: one value per box;
    // at a spectral location also the mode's time and its signed segment
    // count (fd_qmesh adds contr / omega per segment there, not per time)
    __device__ int tally_dt(const DevTables& T, int box, double d, int sign, V2 v, int mode) {
        const double contr = double(sign);
        long long q0, q1, q2;
        if (!quantise(contr * d, q0) || !quantise(v.x * contr * d, q1) || !quantise(v.y * contr * d, q2))
            return E_LIMIT;
        unsigned long long* base = ex + 6ll * box;
        add128(base + 0, q0);
        add128(base + 2, q1);
        add128(base + 4, q2);
        const int loc = T.spec_loc ? T.spec_loc[box] : -1;
        if (loc >= 0) {
            const long long o = (long long)loc * T.n + mode;
            add128(T.spec_ex + 2 * o, q0);
            atomicAdd(T.spec_cnt + o, (unsigned long long)(long long)sign);
        }
        ntally++;
        return 0;
    }
    // process_segment (transient), src/RTA_MC2D.cpp:699-769
    __device__ int tally(const DevTables& T, int box, double t0, double t1, int sign, V2 v, int mode) {
        const int loc = T.spec_loc ? T.spec_loc[box] : -1;
        const double* g = T.timegrid;
        int sb = lower_bound_d(g, T.ntime, t0) - 1;
        int eb = lower_bound_d(g, T.ntime, t1) - 1;
        sb = sb < 0 ? 0 : (sb > T.ntime - 2 ? T.ntime - 2 : sb);
        eb = eb < 0 ? 0 : (eb > T.ntime - 2 ? T.ntime - 2 : eb);
        const double delta_t = t1 - t0;
        for (int i = sb; i <= eb; ++i) {
            const double lo = mx(g[i] - t0, 0.);
            const double hi = mn(g[i + 1] - t0, delta_t);
            const double contr = double(sign) * mx(hi - lo, 0.);
            long long q0, q1, q2;
            if (!quantise(contr, q0) || !quantise(v.x * contr, q1) || !quantise(v.y * contr, q2))
                return E_LIMIT;
            unsigned long long* base = ex + 6ll * ((long long)box * T.nbins + i);
            add128(base + 0, q0);
            add128(base + 2, q1);
            add128(base + 4, q2);
            if (loc >= 0) add128(T.spec_ex + 2ll * ((long long)(loc * T.nbins + i) * T.n + mode), q0);
            ntally++;
        }
        return 0;
    }
};

__device__ __forceinline__ void flush_counters(const Counters& c, unsigned long long* out) {
    unsigned long long v[13] = {c.events, c.wall_hits, c.crossings, c.absorbed,
                                c.specular, c.nudges, c.quirks, c.tallies, c.translations,
                                c.scattered, c.lost, c.ifc_hits, c.ifc_trans};
#pragma unroll
    for (int i = 0; i < 13; ++i) {
        unsigned long long x = v[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + i, x);
    }
}

__global__ void __launch_bounds__(128) rta_replay_kernel(DevTables T, unsigned long long* ex,
                                                         unsigned long long* counters, int* err) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    // every lane runs the same trip count so the closing shuffles see a full warp
    const long long n = T.pend - T.pbegin;
    const long long trips = (n + stride - 1) / stride;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long it = 0; it < trips; ++it) {
        const long long pid = T.pbegin + it * stride + tid;
        if (pid >= T.pend) continue;
        ReplayPolicy pol;
        pol.g.seed(T.seed, (uint64_t)pid);
        pol.ex = ex;
        pol.ntally = 0;
        const int e = run_particle(T, pol, pid, c);
        c.tallies += pol.ntally;
        if (e) {
            if (atomicCAS(err, 0, e) == 0) {
                err[1] = int(pid & 0x7fffffff);
                err[2] = int(pid >> 31);
            }
        }
    }
    flush_counters(c, counters);
}

__device__ __forceinline__ void record_error_r(int* err, int e, long long pid) {
    if (atomicCAS(err, 0, e) == 0) {
        err[1] = int(pid & 0x7fffffff);
        err[2] = int(pid >> 31);
    }
}

// Generation 0: 1 per slot whose first draw picks a gradient generator.
__global__ void steady_select_replay(SteadyArgs A, unsigned long long seed, unsigned* flags) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < A.n; s += stride) {
        Pcg64 g;
        g.seed(seed, steady_stream(0, s));
        flags[s] = steady_gen_type(A, canonical_from(g.next())) == 1 ? 1u : 0u;
    }
}

__global__ void __launch_bounds__(128) rta_steady_replay(DevTables T, SteadyArgs A, unsigned long long* ex,
                                                         unsigned long long* counters, int* err) {
    Counters c = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long trips = (A.n + stride - 1) / stride;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long it = 0; it < trips; ++it) {
        const long long slot = it * stride + tid;
        if (slot >= A.n) continue;
        ReplayPolicy pol;
        pol.g.seed(T.seed, steady_stream(A.gen, slot));
        pol.ex = ex;
        pol.ntally = 0;
        Particle p;
        int fate = FATE_LOST;
        const int e = steady_slot(T, A, pol, slot, c, fate, p);
        c.tallies += pol.ntally;
        if (e) {
            record_error_r(err, e, slot);
            A.flag[slot] = 0;
        } else {
            steady_emit(A, slot, fate, p);
        }
    }
    flush_counters(c, counters);
}

void launch_steady_replay(const DevTables& T, const SteadyArgs& A, unsigned long long* ex,
                          unsigned long long* counters, int* err, unsigned* select_flags, int nsm,
                          cudaStream_t s) {
    if (A.n <= 0) return;
    long long blocks = (A.n + 127) / 128;
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    if (select_flags) steady_select_replay<<<unsigned(blocks), 128, 0, s>>>(A, T.seed, select_flags);
    else rta_steady_replay<<<unsigned(blocks), 128, 0, s>>>(T, A, ex, counters, err);
}

void launch_replay(const DevTables& T, unsigned long long* ex, unsigned long long* counters,
                   int* err, int nsm, cudaStream_t s) {
    const long long n = T.pend - T.pbegin;
    if (n <= 0) return;
    long long blocks = (n + 127) / 128;
    const long long cap = (long long)nsm * 16;
    if (blocks > cap) blocks = cap;
    rta_replay_kernel<<<unsigned(blocks), 128, 0, s>>>(T, ex, counters, err);
}

}  // namespace bte
