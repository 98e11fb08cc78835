// kernels.h - launch wrappers of the particle-loop kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include "rta_flight.cuh"

namespace bte {

// Grid description of the axis-aligned fast path (production mode).
struct DevGrid {
    int nx, ny;
    const double* gx;   // nx + 1 grid lines
    const double* gy;   // ny + 1 grid lines
    const int* cell;    // [nx*ny] box id, -1 void, -2 - b reservoir box b
};

struct ProdTuning {
    int block_threads;
    int blocks_per_sm;
    int smem_tally;
    int particles_per_thread;  // 1 or 2 (the interleaved grid kernel)
};

void launch_replay(const DevTables& T, unsigned long long* ex, unsigned long long* counters,
                   int* err, int nsm, cudaStream_t s);

// General convex-box production kernel (any geometry); `work` is a zeroed
// particle counter.
void launch_prod_general(const DevTables& T, double* tally, unsigned long long* counters,
                         int* err, unsigned long long* work, int nsm, cudaStream_t s);

// One generation of the periodic / gradient steady state (rta_steady.cuh).
// With `select_flags` set, only the generation-0 pre-pass runs: it writes 1
// per slot whose first draw picks a gradient generator.
struct SteadyArgs;
void launch_steady_replay(const DevTables& T, const SteadyArgs& A, unsigned long long* ex,
                          unsigned long long* counters, int* err, unsigned* select_flags, int nsm,
                          cudaStream_t s);
void launch_steady_prod(const DevTables& T, const SteadyArgs& A, double* tally,
                        unsigned long long* counters, int* err, unsigned* select_flags, int nsm,
                        cudaStream_t s);

// Per-mode velocity record of the grid path.
struct __align__(32) ModeVel {
    double vx, vy;    // get_v velocities, nm/ps
    double ivx, ivy;  // their inverses (+inf where the component is 0)
};

// Grid-path kernel parameters beyond the tables.
struct GridArgs {
    DevGrid G;
    const int2* boxcell;     // box -> (i, j)
    const ModeVel* mv;       // per mode velocities and inverses
    int cls[4];              // normal classes of the +x, -x, +y, -y walls (-1: none)
};

// Convex-polygon production path: every border as the line n.x = c (n its
// outward unit normal) with its start p, unit direction u, its wall class,
// and the pieces of it that touch a neighbour box, as intervals of the
// arc length s = (x - p).u.
struct PolyBorder {
    double nx, ny, c;
    double px, py, ux, uy;
    int piece_off, npieces, cls, pad;
};
struct PolyPiece {
    double s0, s1;  // the interval of s, widened by 1e-9 at both ends
    int box, pad;   // pad: the mismatch table of the contact (-1: same crystal)
};
// An axis-aligned rectangular box of the polygon path: its lines and the
// box's own indices of its +x, -x, +y, -y borders (kx1 = -1: not such a
// box, the general border search applies); across each side the
// neighbour box when one piece covers the whole side (-1: a void side,
// -2: look the side's pieces up), that box's flags (1: reservoir, 2:
// periodic) and the side's wall class.
struct PolyRect {
    double x0, x1, y0, y1;
    int kx1, kx0, ky1, ky0;
    int nx1, nx0, ny1, ny0;
    int fx1, fx0, fy1, fy0;
    int cx1, cx0, cy1, cy0;
    // 1: the box's +x and -x sides lead through periodic boxes that
    // translate by its width back into the box itself (a strip spanning
    // the period in x); likewise in y
    int perx, pery;
};
struct PolyArgs {
    const PolyBorder* pb;     // [global border index]
    const PolyPiece* pieces;
    const ModeVel* mv;
    // 1 / (n.v) per border normal class and mode ([nclass][n], -1 where the
    // flight does not leave through such a border); null: divide per pass
    const double* inv_den;
    const PolyRect* rect;     // [box] or null
    // diffuse mismatch interfaces between crystals: a piece whose pad is
    // t >= 0 leads through table t; its rows for global mode K are
    // dmm_row[t * (n + 1) + K .. + 1] into dmm_ent
    const long long* dmm_row;
    const DmmEnt* dmm_ent;
};

// Adjoint passes of the grid kernel: the functional's weights per tally
// value, each particle's total contribution (slot = particle - first),
// per-mode gradient accumulators and {d/dp, sum of R over post-scattering
// draws, sum of Phi}.
struct AdjArgs {
    const double* W;      // [nboxes * nbins][3]
    double* phi_total;    // [particles]
    double* g_tau;        // [nmodes]
    double* g_scalar;     // [3]
};

// Axis-aligned grid production kernel (persistent, warp-refilled work).
// adj_pass 1 / 2 runs the forward / adjoint pass of the adjoint with `adj`.
// Returns false when the tuning cannot be honoured (e.g. smem too small).
// Production kernel of geometries that are not a grid: exit times from the
// convex box's border lines, neighbours from the border pieces.
bool launch_prod_poly(const DevTables& T, const PolyArgs& A, double* tally, unsigned long long* counters,
                      int* err, unsigned long long* work, int nsm, cudaStream_t s);
bool launch_steady_poly(const DevTables& T, const SteadyArgs& A, const PolyArgs& PA, double* tally,
                        unsigned long long* counters, int* err, int nsm, cudaStream_t s);

bool launch_prod_grid(const DevTables& T, const GridArgs& A, double* tally,
                      unsigned long long* counters, int* err, unsigned long long* work,
                      const ProdTuning& tune, int nsm, cudaStream_t s, int adj_pass = 0,
                      const AdjArgs* adj = nullptr);

// Kernel arguments of a context already prepared for one set of run
// parameters (see prepared_grid_run in capi.cu).
struct PreparedRun {
    DevTables T;
    GridArgs A;
    double Eeff, energy, maxtime, step;
    int nboxes, nbins, ntime;
    cudaStream_t stream;
    cudaEvent_t ev0, ev1;
    int device, nsm;
    ProdTuning tune;
};

}  // namespace bte
