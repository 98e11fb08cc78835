/*
 * btegpu.h - C ABI of the GB300 deviational Monte Carlo engine for the
 * RTAMC2D / beRTAMC2D particle loop of BTE-Barna.
 *
 * The reference has no library or plugin interface: its boundary is the
 * executable plus files (src/RTA_MC2D.cpp:2085-2101 argv, :1806-2055 XML,
 * src/bulk_hdf5.cpp:443 mode table, :2437-2471 CSV outputs).  Each entry point
 * below replaces one step of that pipeline; the citation on each names the
 * reference code whose role it takes.
 *
 * Conventions
 *  - Plain C types only; caller-owned host buffers are copied in, results go
 *    to caller-allocated host buffers, device memory is owned by the context.
 *  - No exception crosses the ABI: every call returns a bte_status, and
 *    bte_last_error() gives the message of the last failing call.
 *  - One context per host thread; calls on one context are serialised; the
 *    context owns one CUDA stream and results are valid when a call returns.
 *  - Mode index = iq * nb + ib (src/RTA_MC2D.cpp:1250-1254).
 *  - Units follow the reference: omega rad/ps, velocities nm/ps, lengths nm,
 *    times ps, energies J (include/constants.hpp:27-56).
 */
#ifndef BTEGPU_H
#define BTEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BTEGPU_VERSION 1

/* Status codes.  The first three mirror the reference's exception types
 * (include/exceptions.hpp:25-55). */
typedef enum bte_status {
    BTE_OK = 0,
    BTE_ERR_INPUT = 1,    /* alma::input_error: malformed or unsupported input */
    BTE_ERR_VALUE = 2,    /* alma::value_error: e.g. a zero scattering rate   */
    BTE_ERR_GEOMETRY = 3, /* alma::geometry_error: inconsistent geometry      */
    BTE_ERR_LIMIT = 4,    /* a device loop reached its iteration cap          */
    BTE_ERR_CUDA = 5,     /* CUDA runtime failure                             */
    BTE_ERR_STATE = 6,    /* wrong call order (e.g. run before load)          */
    BTE_ERR_CHECK = 7     /* an index check of BTE_FLAG_CHECKS failed          */
} bte_status;

/* Run modes. */
enum {
    /* Deterministic replay: one pcg64 stream per particle (seed, stream =
     * particle index), CDF inversion by lower_bound, FP64 everywhere, exact
     * fixed-point tallies.  Bit-identical to the CPU restatement in oracle/. */
    BTE_MODE_REPLAY = 0,
    /* Production: counter-based Philox4x32-10 streams keyed by (seed,
     * particle), alias tables, FP64 position/time/tallies with FP64 atomics. */
    BTE_MODE_PRODUCTION = 1
};

/* Particle sources of an RTA run. */
enum {
    /* Isothermal reservoir walls inject at t=0; the tally is integrated in
     * time into a step response (src/RTA_MC2D.cpp:272-449, :2380-2384). */
    BTE_SOURCE_WALLS = 0,
    /* Initial deviation Tinit - Teq per box (outTref_distribution,
     * src/sampling.cpp:271-330); tallies are bin averages, not integrated. */
    BTE_SOURCE_INITIAL = 1
};

typedef struct bte_ctx bte_ctx;

typedef struct bte_device_opts {
    int32_t device;  /* CUDA device ordinal */
    int32_t verbose; /* 0 = silent, 1 = banners like the reference's stdout */
} bte_device_opts;

/* Phonon mode table of one material (replaces alma::Gamma_grid +
 * Crystal_structure as loaded by load_bulk_hdf5, src/bulk_hdf5.cpp:443-686,
 * and the RTA rates of calc_w0_threeph + calc_w0_twoph,
 * src/RTA_MC2D.cpp:1899-1907).  iq = 0 must be the Gamma point. */
typedef struct bte_mode_table {
    int32_t nq;            /* number of q points                                */
    int32_t nb;            /* branches per q point                              */
    int32_t grid[3];       /* q-grid divisions; q index iq = i*grid[1] + j     */
    const double* omega;   /* [nq*nb] angular frequency, rad/ps                */
    const double* vg;      /* [nq*nb*3] group velocity (vx,vy,vz), nm/ps       */
    const double* w;       /* [nq*nb] RTA scattering rate 1/tau, 1/ps          */
    const double* dq;      /* [9] column-major q-grid steps, nm^-1
                              (Gamma_grid::dq, include/qpoint_grid.hpp:45)      */
    double V;              /* unit-cell volume, nm^3 (Crystal_structure::V)     */
    double c_lat;          /* out-of-plane lattice vector lattvec(2,2), nm      */
} bte_mode_table;

/* Convex boxes of a geometry XML (replaces read_geometry_XML,
 * src/geometry_2d.cpp:408-522, and the geometry_2d constructor :127-153). */
typedef struct bte_geometry {
    int32_t nboxes;
    const int32_t* npoints;   /* [nboxes] vertices per box                     */
    const double* vertices;   /* (x,y) pairs of all boxes, concatenated, nm     */
    const double* Teq;        /* [nboxes] initCnd Teq, K                        */
    const double* Tinit;      /* [nboxes] initCnd Tinit (= Teq when absent), K  */
    const int32_t* reservoir; /* [nboxes] 1 for <Reservoir/>                    */
    double thickness;         /* material thickness, nm (<material thickness>)  */
    /* Periodic boxes, <Translate_to id="j"> tx ty </Translate_to>
     * (src/geometry_2d.cpp:467-475, geometry_2d::translate
     * include/geometry_2d.hpp:366-493).  Both NULL: no periodic box. */
    const int32_t* translate_to; /* [nboxes] target box j, -1 = not periodic   */
    const double* translation;   /* [nboxes][2] translation vector, nm         */
    /* Material of each box for batched sweeps (NULL: every box is material
     * 0); materials come from bte_load_materials. */
    const int32_t* material;     /* [nboxes] */
} bte_geometry;

/* Parameters of one RTA run (the <RTA_MC2d> XML of src/RTA_MC2D.cpp:1818-1947
 * plus the knobs of this engine). */
typedef struct bte_rta_params {
    double T0;               /* reference temperature, K                        */
    double dt;               /* width of a time bin, ps                         */
    double maxtime;          /* simulated time, ps                              */
    int64_t nparticles;      /* N: sets Eeff = |E|/N                            */
    uint64_t seed;           /* master seed of all particle streams             */
    int32_t mode;            /* BTE_MODE_*                                      */
    int32_t source;          /* BTE_SOURCE_*                                    */
    int32_t ballistic;       /* 1: no intrinsic scattering (<ballistic/>)       */
    int32_t flags;           /* BTE_FLAG_* (0: none)                            */
    double specularity;      /* p of void walls; 0 = the reference's diffuse    */
    int64_t particle_begin;  /* simulate particles [begin, end) of the N;      */
    int64_t particle_end;    /*   end <= 0 means N                              */
    int64_t flight_cap;      /* free flights per particle before BTE_ERR_LIMIT
                                (0: 2^26); a small cap injects the limit path   */
} bte_rta_params;

/* Run flags.  BTE_FLAG_CHECKS runs the production grid kernel in its checked
 * variant: every table, tally and grid index is tested before use and a
 * violation stops the particle with BTE_ERR_CHECK instead of an out-of-range
 * access (the same draws as the plain variant, so the same trajectories). */
#define BTE_FLAG_CHECKS 1
/* BTE_FLAG_GENERAL runs production boxes that do not tile a grid through the
 * evolparticle-faithful kernel (the reference's corner and nudge handling,
 * one evolparticle step per pass) instead of the convex-polygon kernel
 * (exit times against the box's border lines, one segment per pass). */
#define BTE_FLAG_GENERAL 2

/* Results of one RTA run.  Every array pointer may be NULL (not written).
 * Arrays are row-major [nboxes][nbins]. */
typedef struct bte_rta_result {
    int32_t nboxes;          /* out */
    int32_t nbins;           /* out: ntime - 1                                   */
    double* gz;              /* raw sign-weighted particle time per box and bin  */
    double* gz_jx;           /* raw vx-weighted tally                            */
    double* gz_jy;           /* raw vy-weighted tally                            */
    double* temperature;     /* K, as written to temperature_*.csv               */
    double* jx;              /* J m^-2 s^-1, as written to jx_*.csv              */
    double* jy;              /* J m^-2 s^-1, as written to jy_*.csv              */
    int64_t* exact;          /* replay mode: [nboxes][nbins][3][2] 128-bit
                                fixed-point sums (hi, lo) scaled by 2^44       */
    double Eeff;             /* energy per particle, J/ps (src/RTA_MC2D.cpp:2177) */
    double energy_rate;      /* |E| injected per ps or initial energy, J         */
    int64_t events;          /* free-flight draws (random_dt calls)              */
    int64_t wall_hits;       /* void-wall reflections                            */
    int64_t crossings;       /* box-to-box transfers                             */
    int64_t absorbed;        /* particles that reached a reservoir               */
    int64_t specular_hits;   /* specular reflections (p > 0)                     */
    int64_t tally_updates;   /* (box, time-bin) contributions made               */
    double kernel_ms;        /* device time of the particle loop                 */
    int64_t translations;    /* jumps through periodic boxes                     */
    int64_t interface_hits;  /* arrivals at contacts between crystals (diffuse
                                mismatch re-emissions)                        */
    int64_t interface_transmissions; /* of those, re-emitted into the other crystal */
} bte_rta_result;

/* Propagator exp(B dt) of one material at one temperature over the modes
 * 3..n-1 (the three Gamma acoustic modes have no column), as stored in
 * *.P.eigen.bin by save_P (src/collision_operator.cpp:931-970). */
typedef struct bte_propagator {
    int32_t nmodes;      /* n - 3 */
    double T;            /* temperature the propagator was built at, K */
    const double* P;     /* [nmodes * nmodes] column-major: column j = mode j + 3 */
} bte_propagator;

/* Called after every step of a beyond-RTA run with that step's signed
 * histogram H [nboxes][nmodes] (host memory, valid during the call) and
 * its properties ed [nboxes], flux [nboxes][2]; the hook of the reference's
 * stdout table and msgpack frames (src/beyondRTA_MC2d.cpp:2374-2423). */
typedef void (*bte_berta_step_fn)(void* user, int32_t step, double time, int64_t nparticles,
                                  const int32_t* H, int32_t nboxes, int32_t nmodes,
                                  const double* ed, const double* flux);

/* Parameters of one beRTAMC2D run (<beRTAMC2D> XML,
 * src/beyondRTA_MC2d.cpp:1299-1462). */
typedef struct bte_berta_params {
    double dt;               /* time step, ps                                    */
    double maxtime;          /* the loop runs while time <= maxtime              */
    double Eeff;             /* energy per particle, J (<Eeff Ed=...>)          */
    double T0;               /* temperature of the mode table's rates, K: with
                                rta = 1 every box that scatters needs Teq = T0;
                                with the propagator each box scatters at its own
                                Teq (the tabulated propagator, or lirp between
                                the two tabulated temperatures above it)      */
    uint64_t seed;
    int32_t mode;            /* BTE_MODE_PRODUCTION                              */
    int32_t rta;             /* 1: RTA scattering (<RTA/>), 0: propagator        */
    int32_t cancel_every;    /* cancellation period in steps (reference: 4)     */
    int32_t gradient_mode;   /* source term of step 2 (source_term_gradient,
                                src/beyondRTA_MC2d.cpp:597-676):
                                0: gradients from the boxes' Teq
                                   (calculate_gradientT, the reference's
                                   default: the minimum-norm least-squares
                                   gradient over each box's neighbours; zero
                                   where they share its Teq)
                                1: the homogeneous <gradient x y> below on
                                   every box that is neither a reservoir nor
                                   periodic                                 */
    int64_t capacity;        /* particle capacity on the device (0 = auto)       */
    bte_berta_step_fn on_step; /* optional per-step hook (NULL: none)          */
    void* user;              /* passed to on_step                                */
    double gradient[2];      /* K/nm, gradient_mode 1                            */
} bte_berta_params;

/* Results of one beRTAMC2D run; per step s = 0..nsteps (s = 0 is the
 * initial state), the stdout table of src/beyondRTA_MC2d.cpp:2418-2423. */
typedef struct bte_berta_result {
    int32_t nboxes;          /* out */
    int32_t nsteps;          /* out: loop iterations                             */
    double* ed;              /* [nsteps+1][nboxes] deviational energy density, J m^-3 */
    double* flux;            /* [nsteps+1][nboxes][2] heat flux, J m^-2 s^-1   */
    int64_t* nparticles;     /* [nsteps+1] particles alive                       */
    int32_t* histogram;      /* [nboxes][nmodes] final signed histogram (may be NULL) */
    int64_t particle_steps;  /* particles advected, summed over steps           */
    int64_t branchings;      /* sign flips that re-entered the scattering queue  */
    double kernel_ms;        /* device time of the step loop                     */
    double phase_ms[8];      /* out: the reference's timer buckets (src/beyondRTA_MC2d.cpp:
                                1838-1897), sorted by name: advection, cancelling,
                                generators, histogram, properties, read_data, saving,
                                scattering; device time per step phase, host time
                                for read_data (set-up) and saving (on_step)     */
    int64_t advance_in;      /* out: particles read by the fused step kernel, summed
                                over its launches (existing and new particles)  */
    int64_t advance_out;     /* out: particles it wrote (outgoing after scattering) */
} bte_berta_result;

/* Parameters of a steady-state run of a periodic structure under an applied
 * temperature gradient (the gradient branch of RTAMC2D,
 * src/RTA_MC2D.cpp:2544-2842; <gradient x= y=/> and <convergence energy=
 * flux=/> of the <RTA_MC2d> XML, :1828-1840). */
typedef struct bte_steady_params {
    double T0;               /* reference temperature, K                       */
    double gradient[2];      /* applied gradient, K/nm (must not be zero)      */
    double eps_energy;       /* relative change of gz that ends the loop; <= 0: never */
    double eps_flux;         /* relative change of the flux tallies; <= 0: never */
    int64_t nparticles;      /* N: Eeff = |E|/N                                */
    uint64_t seed;           /* master seed of all slot streams                 */
    int32_t mode;            /* BTE_MODE_*                                      */
    int32_t max_generations; /* safety cap of the generation loop (0: 100000)  */
    double specularity;      /* p of void walls; 0 = the reference's diffuse    */
    int32_t flags;           /* BTE_FLAG_GENERAL: the evolparticle-faithful
                                kernel instead of the convex-polygon one       */
    int32_t reserved0;
} bte_steady_params;

/* Results of a steady-state run: one value per box (the rows of
 * steady_<T0>K_run_<i>.csv) and the per-generation convergence table. */
typedef struct bte_steady_result {
    int32_t nboxes;          /* out */
    int32_t generations;     /* out: iterations of the generation loop          */
    int32_t converged;       /* out: 1 when the eps criteria ended the loop     */
    int32_t log_cap;         /* in: rows available in `log`                     */
    double* gz;              /* [nboxes] raw sign-weighted particle time        */
    double* gz_jx;           /* [nboxes] raw vx-weighted tally                  */
    double* gz_jy;           /* [nboxes] raw vy-weighted tally                  */
    double* temperature;     /* [nboxes] K                                      */
    double* jx;              /* [nboxes] J m^-2 s^-1                            */
    double* jy;              /* [nboxes] J m^-2 s^-1                            */
    int64_t* exact;          /* replay: [nboxes][3][2] 128-bit sums (hi, lo), 2^44 */
    double* log;             /* [log_cap][4]: particles, rgz, rjx, rjy per generation */
    double Eeff;             /* energy per particle, J/ps                       */
    double energy_rate;      /* |E| of all generators, J/ps                     */
    int64_t events;          /* free flights                                    */
    int64_t wall_hits;       /* void-wall reflections (carried over)            */
    int64_t crossings;
    int64_t absorbed;
    int64_t translations;
    int64_t scattered;       /* flights ending inside a box (phi)               */
    int64_t births;          /* particles created from phi                      */
    int64_t lost;            /* flights dropped at a crossing with no time left */
    double kernel_ms;        /* device time of the generation kernels           */
    int64_t interface_hits;  /* contacts met between crystals (re-emitted and
                                carried over, as void-wall reflections)        */
    int64_t interface_transmissions; /* of which re-emitted across          */
} bte_steady_result;

/* Tuning knobs of the production kernels (project-written autotuner picks
 * them; 0 selects the built-in default). */
typedef struct bte_tuning {
    int32_t block_threads;   /* threads per block                              */
    int32_t blocks_per_sm;   /* resident blocks per SM of the persistent grid  */
    int32_t smem_tally;      /* 1: privatise tallies in shared memory           */
    int32_t particles_per_thread; /* particles each thread carries at once in
                                the grid kernel: 1, or 2 for the interleaved
                                variant (plain production runs with a global
                                tally and no spectral locations; others use 1) */
} bte_tuning;

/* ------------------------------------------------------------------------ */

/* Create a context on a device (replaces the start of main,
 * src/RTA_MC2D.cpp:2061-2118). */
bte_status bte_create(bte_ctx** ctx, const bte_device_opts* opts);

/* Release all device memory and the stream of a context. */
bte_status bte_destroy(bte_ctx* ctx);

/* Copy the last error message of ctx (or of bte_create when ctx is NULL). */
bte_status bte_last_error(const bte_ctx* ctx, char* buf, size_t size);

/* Load the mode table of the (single) material and build the device tables:
 * resampling CDF/alias (BE_derivative_distribution, src/sampling.cpp:47-68)
 * and the energy-conserving Lambert wall table
 * (generators::diffusive_bouncing, src/RTA_MC2D.cpp:556-626). */
bte_status bte_load_modes(bte_ctx* ctx, const bte_mode_table* modes);

/* Load the boxes and build borders and contacts (geometry_2d::get_sides and
 * calculate_contacts, src/geometry_2d.cpp:51-124, :295-381). */
bte_status bte_load_geometry(bte_ctx* ctx, const bte_geometry* geom);

/* Materials of batched sweeps: nmat relaxation-rate sets over the loaded
 * mode table (the same crystal at several temperatures).  Material m has
 * rates w[m][mode] and reference temperature T0[m], which set its
 * lifetimes, its post-scattering distribution and its temperature
 * conversion; a box of geometry.material = m uses material m, and a run
 * checks each box's Teq against its material's T0 (bte_rta_params.T0 is
 * then unused).  The reference keeps rates, sampler and C_v per material
 * too (inpars.material_w0 / material_sampler / material_cv,
 * src/RTA_MC2D.cpp:1893-1923); here the materials share the mode table and
 * the Lambert wall table.  Boxes of different materials must not touch: a
 * particle keeps its material.  nmat = 0 returns to the single table.
 *
 * share (optional, [nmat], summing to 1) gives each material its own
 * particle budget in a walls-source run: a wall of material m is drawn with
 * probability share[m] E_w / E_m instead of E_w / E (the reference's
 * energy-weighted choice, src/RTA_MC2D.cpp:390-418), and the particles of
 * material m carry Eeff_m = E_m / (share[m] N) (:2177) in the conversion of
 * its boxes.  NULL keeps the energy-weighted choice and one Eeff. */
bte_status bte_load_materials(bte_ctx* ctx, int32_t nmat, const double* w, const double* T0,
                              const double* share);

/* Several crystals, each with its own mode table (and rates), in one
 * geometry: box b is in crystal bte_geometry.material[b].  Particles that
 * reach a contact between crystals are re-emitted by the diffuse mismatch
 * model (Diffuse_mismatch_distribution, src/sampling.cpp:437-902, as
 * change_material_diffuse uses it, src/RTA_MC2D.cpp:871-964): one table per
 * (crystal, other crystal, contact normal), built at the Teq of the first
 * box that meets it.  Replaces bte_load_modes and any rate sets of
 * bte_load_materials; reservoirs inject into their own crystal only
 * (BTE_ERR_INPUT "Injection from material A to B is not allowed").
 * thickness: each crystal's <material thickness> (nm), the thickness of
 * its boxes (the reference's thicknesses[box]); NULL: the geometry's
 * thickness for every crystal.  Transient and steady runs, replay and
 * production; the layer coupling of LDMM is not available (it needs the
 * modes' eigenvectors and a layer description the mode tables do not
 * carry). */
bte_status bte_load_mode_tables(bte_ctx* ctx, int32_t ntables, const bte_mode_table* tables,
                                const double* thickness);

/* The diffuse mismatch table of the interface from table A to table B
 * (normal (nx, ny) pointing from A to B, the thicknesses of A's and B's
 * boxes, Tref), built on
 * the host (no device needed): for incident mode i of A (v.n > 0), entries
 * [first[i], first[i+1]) of (side out: 0 = A, 1 = B; mode out in that
 * side's table; cumulative probability over A's incident modes).  first
 * has nq*nb of A + 1 values; with side, mode or cum NULL only first and
 * *nentries are filled.  The reference records the closest-frequency
 * reflection of an incident mode without a transition with side B; kept. */
bte_status bte_interface_table(const bte_mode_table* A, const bte_mode_table* B, double nx, double ny,
                               double thickness_a, double thickness_b, double Tref, int64_t* first,
                               int64_t* nentries, int32_t* side, int32_t* mode, double* cum);

/* Run the RTA particle loop for one run and fill `out` (replaces one
 * iteration of the run loop of src/RTA_MC2D.cpp:2188-2543: generation,
 * the parallel_for over evolparticle, and the post-processing). */
bte_status bte_rta_run(bte_ctx* ctx, const bte_rta_params* params,
                       bte_rta_result* out);

/* Set the production-kernel tuning; NULL restores the defaults. */
bte_status bte_set_tuning(bte_ctx* ctx, const bte_tuning* tuning);

/* Number of modes and boxes loaded; sizes of the result arrays. */
bte_status bte_query_sizes(const bte_ctx* ctx, const bte_rta_params* params,
                           int32_t* nboxes, int32_t* nbins, int64_t* nmodes);

/* Library version (BTEGPU_VERSION). */
int32_t bte_version(void);

/* Load the propagator of the (single) material at temperature P->T for
 * beyond-RTA runs (replaces load_P and the propagator_H columns of
 * process_input, src/collision_operator.cpp:972-1013,
 * src/beyondRTA_MC2d.cpp:1363-1377).  Calls with different T tabulate the
 * propagator in temperature (a call at a T already loaded replaces it).  A
 * run at T0 uses the propagator at T0 when it is tabulated; otherwise it
 * interpolates as the reference does (Scattering :1130-1165, lirp
 * src/collision_operator.cpp:918-929): linearly in the signed CDFs between
 * the first tabulated temperature above T0 and the next one, and fails with
 * BTE_ERR_INPUT when those two do not exist or T0 is below the lowest.
 * bte_load_modes forgets every loaded propagator. */
bte_status bte_load_propagator(bte_ctx* ctx, const bte_propagator* P);

/* Run the beRTAMC2D step loop (replaces the loop of
 * src/beyondRTA_MC2d.cpp:2138-2425 and its stdout table).  Production mode;
 * the boxes must tile an axis-aligned grid and share Teq = T0. */
bte_status bte_berta_run(bte_ctx* ctx, const bte_berta_params* params,
                         bte_berta_result* out);

/* Run the steady state of a periodic structure under a temperature
 * gradient: generations of one free flight per particle, phi re-emission
 * and the convergence test (replaces the gradient branch of the run loop,
 * src/RTA_MC2D.cpp:2544-2842, with generation by Init_generator,
 * :272-533, and the periodic evolparticle / process_segment, :784-834,
 * :1406-1799). */
bte_status bte_steady_run(bte_ctx* ctx, const bte_steady_params* params,
                          bte_steady_result* out);

/* Gradient of a linear functional of the tallies of a production run,
 *   Phi = sum_{box, bin} W[box][bin][0] gz + W[..][1] gz_jx + W[..][2] gz_jy
 * (raw tallies as in bte_rta_result; kappa_eff and any time- or
 * box-averaged flux or temperature are such functionals), with respect to
 * every mode's lifetime tau and the wall specularity p.  Likelihood-ratio
 * weights of the free-flight, post-scattering and specularity draws; the
 * adjoint pass recomputes each trajectory from its Philox counter after a
 * forward pass has stored each particle's contribution.  Boxes that tile
 * an axis-aligned grid, one material.  No reference counterpart: the
 * reference has no derivatives (its finite differences are the check). */
typedef struct bte_adjoint_result {
    double phi;              /* the functional from the same particles        */
    double* dphi_dtau;       /* [nmodes] dPhi/dtau_k, per ps                   */
    double dphi_dp;          /* dPhi/dp (meaningful for 0 < p < 1)            */
    int64_t events;          /* flight events of one pass                      */
    double kernel_ms;        /* device time of both passes                     */
} bte_adjoint_result;

bte_status bte_rta_adjoint(bte_ctx* ctx, const bte_rta_params* params, const double* weights,
                           bte_adjoint_result* out);

/* Spectral decomposition at selected boxes (<spectral><resolution
 * ticks=/><location bin=/>..., src/RTA_MC2D.cpp:150-175, :699-766,
 * :1979-2052): the following bte_rta_run and bte_steady_run calls also
 * tally, per location, time bin and mode, the time spent there (a steady
 * run has one bin and also counts the signed segments per mode,
 * process_segment :784-834); bte_get_spectral turns the last run's tally
 * into the reference's four outputs (transient :2350-2420, :2473-2541;
 * steady :2729-2830).  nloc = 0 switches it off. */
bte_status bte_set_spectral(bte_ctx* ctx, int32_t nloc, const int32_t* boxes, int32_t nomega);

/* Spectral outputs of the last run, each [nloc][nbins][...], cumulated in
 * time after a transient run as the reference writes them (a steady run has
 * nbins = 1 and no cumulation):
 *   dT_omega  Gamma-pdf weighted temperature per omega tick (deltaT_omega_*.csv)
 *   jx_omega, jy_omega  the flux per omega tick (jx_omega_*, jy_omega_*.csv)
 *   fd_q      the distribution per q point (fd_q_*.csv); after a steady run
 *             the reference adds sign / omega per segment, not per time
 * with omega[nloc][nomega] the tick centres and q1bz[nq][2] the q points.
 * Any pointer may be NULL. */
typedef struct bte_spectral_result {
    int32_t nloc, nbins, nomega, nq;   /* out */
    double* omega;
    double* dT_omega;
    double* jx_omega;
    double* jy_omega;
    double* fd_q;
    double* q1bz;
    double* raw;     /* [nloc][nbins][nmodes] sign-weighted time per mode (unscaled) */
    int32_t steady;  /* out: 1 when the last run was a steady-state run      */
    int32_t reserved0;
    double* counts;  /* [nloc][nmodes] signed segments per mode (steady runs) */
} bte_spectral_result;

bte_status bte_get_spectral(bte_ctx* ctx, bte_spectral_result* out);

/* Replica groups of the following production runs on boxes that tile a
 * grid: particle p tallies into group p mod ngroups, so one run gives
 * ngroups independent estimates of every output (batch means inside one
 * launch); the run's own outputs are the sums over the groups.  The
 * reference estimates errors from independent runs (nruns,
 * src/RTA_MC2D.cpp:2099-2101, :2188); a group is one such run made with
 * 1/ngroups of the particles.  ngroups = 0 or 1 switches it off; a replay
 * run or a geometry off a grid fails with BTE_ERR_INPUT while it is on. */
bte_status bte_set_groups(bte_ctx* ctx, int32_t ngroups);

/* Outputs of group `group` of the last run with replica groups, scaled to
 * estimate the whole run (the group's tallies x ngroups, then the run's
 * post-processing): gz, gz_jx, gz_jy, temperature, jx, jy as in
 * bte_rta_result (exact, counters and kernel_ms are not kept per group and
 * come back as 0).  Valid until the next run, load or bte_set_groups. */
bte_status bte_get_group_result(bte_ctx* ctx, int32_t group, bte_rta_result* out);

/* Largest number of time bins bte_rta_run_noalloc accepts. */
#define BTE_NOALLOC_MAX_BINS 4096

/* The production RTA particle loop with no device allocation during the
 * call.  No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc at run time -- a framework that owns all device memory through
 * its own pool and forbids other allocations, or a loop that must not reach
 * the driver's allocator, whose calls can synchronise the device and take
 * unbounded time.  The caller passes the run parameters and a device buffer
 * d_tally of nboxes * nbins * 3 doubles, written as [box][bin][gz, gz_jx,
 * gz_jy] (the raw tallies of bte_rta_run); counters, Eeff and kernel_ms come
 * back in `out` (its array pointers are ignored).  The call synchronises the
 * context's stream before it returns.  The kernel's scratch is one fixed
 * device array of the library (at most BTE_NOALLOC_MAX_BINS time bins),
 * shared by every call and held by every GPU that loads the library until
 * the process exits: calls that overlap on the GPU race and must be
 * serialised.  The context must already hold the tables for these
 * parameters (one bte_rta_run with the same T0 and source, and for the
 * initial source the same N and seed); the boxes must tile an axis-aligned
 * grid and mode must be BTE_MODE_PRODUCTION.  The first call on a device
 * does the set-up: it looks up the scratch address once (kept until the
 * process exits, so not after a cudaDeviceReset).  Since every call
 * synchronises its stream, no call can be recorded in a stream capture. */
bte_status bte_rta_run_noalloc(bte_ctx* ctx, const bte_rta_params* params,
                               double* d_tally, bte_rta_result* out);

#ifdef __cplusplus
}
#endif

#endif /* BTEGPU_H */
