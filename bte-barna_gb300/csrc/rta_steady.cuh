// rta_steady.cuh - one generation of the periodic / gradient steady state of
// RTAMC2D (src/RTA_MC2D.cpp:2544-2842) on the device.
//
// A generation is a list of slots.  Each slot carries one particle through
// exactly one free flight (the body of the parallel_for, :2575-2627):
//   generation 0   Init_generator with a gradient (:443-529): a wall particle
//                  or a Nabla_T particle of a box, whose sign alternates -,+,-
//                  over the gradient-generated particles in slot order;
//   later          first the particles reflected at a void wall in the
//                  previous generation (in slot order), then |phi(box)| new
//                  particles per box with the sign of phi (:2640-2658).
// A flight ends by scattering inside a box (phi += sign), by reflection
// (carried over), by absorption in a reservoir, or is dropped when the time
// left at a crossing rounds to zero.  Slot s of generation g draws from its
// own stream, keyed by (g << 40) | s.
#pragma once

#include "rta_flight.cuh"

namespace bte {

struct SteadyP {
    double x, y;
    int mode, box, sign, pad;
};

struct SteadyArgs {
    int gen;
    long long n;               // slots of this generation
    const SteadyP* in;         // reflected particles carried into this generation
    long long nin;
    // generation 0: generator type (ExGen of Init_generator) and gradient sources
    double exg0, exg1;         // cumulative weights: walls, walls + gradient
    int nwall, ngrad;
    const int* grad_box;       // [ngrad]
    const double* grad_cum;    // [ngrad] cumulative box weights
    const double* grad_cdf;    // [ngrad][n] Nabla_T CDFs (replay)
    const float* grad_prob;    // [ngrad][n] alias (production)
    const int* grad_alt;
    const signed char* grad_sign;  // [ngrad][n] sign of -gradT . v
    const unsigned* grad_rank; // [slots] gradient-generated slots before this one
    // births from phi of the previous generation
    int nbirth;
    const long long* birth_first;  // [nbirth + 1] first birth slot per box (relative)
    const int* birth_box;
    const int* birth_sign;
    // outputs
    SteadyP* out;              // [slots] the reflected particle of each slot
    unsigned* flag;            // [slots] 1 when the slot's particle was reflected
    unsigned long long* phi;   // [nboxes] signed counts, two's complement
    unsigned long long* work;  // slots taken (production kernel), zeroed per launch
};

__device__ __forceinline__ uint64_t steady_stream(int gen, long long slot) {
    return ((uint64_t)(unsigned)gen << 40) | (uint64_t)slot;
}

// Generator type of generation-0 slot: 0 walls, 1 gradient
// (lower_bound over ExGen, :449-451; a draw past the end keeps the last
// generator that exists).
__device__ __forceinline__ int steady_gen_type(const SteadyArgs& A, double u) {
    int id = u <= A.exg0 ? 0 : 1;
    if (id == 0 && A.nwall == 0) id = 1;
    if (id == 1 && A.ngrad == 0) id = 0;
    return id;
}

template <class P>
__device__ int steady_generate0(const DevTables& T, const SteadyArgs& A, P& pol, long long slot,
                                Particle& p) {
    const double selectGenR = pol.u();
    if (steady_gen_type(A, selectGenR) == 0) return generate_wall(T, pol, p);
    // case 1, :499-521
    const double whereGenR = pol.u();
    int gi = lower_bound_d(A.grad_cum, A.ngrad, whereGenR);
    if (gi >= A.ngrad) gi = A.ngrad - 1;
    const int b = A.grad_box[gi];
    V2 r;
    int e = random_point(T, pol, b, r);
    if (e) return e;
    const int want = (A.grad_rank[slot] & 1u) ? 1 : -1;  // gsign starts negative
    const long long o = (long long)gi * T.n;
    int k = 0, tries = 0;
    for (;;) {
        if (++tries > 1000000) return E_LIMIT;
        k = pol.dist(A.grad_cdf + o, A.grad_prob + o, A.grad_alt + o, T.n);
        if (A.grad_sign[o + k] == want) break;
    }
    p.pos = r;
    p.mode = k;
    p.sign = want;
    p.t = 0.;
    p.box = b;
    p.mo = mat_off(T, b);
    return 0;
}

// One new particle from phi: random point of the box, mode from the
// post-scattering distribution at T0 (material_sampler.sample()).
template <class P>
__device__ int steady_birth(const DevTables& T, const SteadyArgs& A, P& pol, long long k,
                            Particle& p) {
    int lo = 0, hi = A.nbirth;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (A.birth_first[mid] <= k) lo = mid; else hi = mid;
    }
    const int b = A.birth_box[lo];
    V2 r;
    const int e = random_point(T, pol, b, r);
    if (e) return e;
    p.mo = mat_off(T, b);
    p.pos = r;
    p.mode = pol.resample(T, p.mo);
    p.sign = A.birth_sign[lo];
    p.t = 0.;
    p.box = b;
    return 0;
}

// The slot's particle and the draw of its one flight (v, dt).  Returns 0 or
// an error code.
template <class P>
__device__ int steady_begin(const DevTables& T, const SteadyArgs& A, P& pol, long long slot,
                            Counters& c, Particle& p, V2& v, double& dt) {
    int e;
    if (A.gen == 0) {
        e = steady_generate0(T, A, pol, slot, p);
    } else if (slot < A.nin) {
        const SteadyP q = A.in[slot];
        p.pos = v2(q.x, q.y);
        p.mode = q.mode;
        p.box = q.box;
        p.sign = q.sign;
        p.t = 0.;
        p.mo = mat_off(T, q.box);
        e = 0;
    } else {
        e = steady_birth(T, A, pol, slot - A.nin, p);
    }
    if (e) return e;
    const int k = p.mode;
    v = v2(T.vxc[k], T.vyc[k]);
    if (T.w[p.mo + k] == 0.) return E_VALUE;
    dt = pol.flight(T, p.mo + k);
    c.events++;
    return 0;
}

// The slot's particle and its one flight.  Returns 0 or an error code.
template <class P>
__device__ int steady_slot(const DevTables& T, const SteadyArgs& A, P& pol, long long slot,
                           Counters& c, int& fate, Particle& p) {
    V2 v;
    double dt = 0.;
    int e = steady_begin(T, A, pol, slot, c, p, v, dt);
    if (e) return e;
    fate = FATE_LOST;
    int guard = 0, nudges = 0;
    while (!almost_equal(dt, 0.)) {
        if (++guard > FLIGHT_CAP) return E_LIMIT;
        e = evolparticle<P, true>(T, pol, p, v, dt, c, nudges, fate);
        if (e) return e;
    }
    if (fate == FATE_LOST) c.lost++;
    return 0;
}

// Writes the slot's outcome: the reflected particle, its flag, phi.
__device__ __forceinline__ void steady_emit(const SteadyArgs& A, long long slot, int fate,
                                            const Particle& p) {
    const bool bounced = fate == FATE_BOUNCE;
    A.flag[slot] = bounced ? 1 : 0;
    if (bounced) {
        SteadyP q;
        q.x = p.pos.x;
        q.y = p.pos.y;
        q.mode = p.mode;
        q.box = p.box;
        q.sign = p.sign;
        q.pad = 0;
        A.out[slot] = q;
    } else if (fate == FATE_SCATTER) {
        atomicAdd(A.phi + p.box, (unsigned long long)(long long)p.sign);
    }
}

}  // namespace bte
