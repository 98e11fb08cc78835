// tables.hpp - host construction of the device-side tables of the particle
// loop: geometry records, sampling distributions (CDF for replay, alias for
// production), the energy-conserving Lambert wall table and the particle
// generators.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/btegpu.h"
#include "bte_device.cuh"

namespace bte {

// Status-carrying exception used inside the library only; the C ABI turns
// it into a bte_status and a message.
struct Error : std::runtime_error {
    bte_status code;
    Error(bte_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

struct HostModes {
    int nq = 0, nb = 0, grid[3] = {0, 0, 0};
    std::vector<double> omega, vx, vy, vz, w;
    std::vector<double> vxc, vyc;  // get_v: components almost equal to 0 set to 0
    double dq[9] = {0};
    double V = 0, c = 0;
    std::size_t n() const { return std::size_t(nq) * std::size_t(nb); }
};

struct HostGeometry {
    std::vector<GBox> boxes;
    std::vector<V2> hull;
    std::vector<GBorder> borders;
    std::vector<GContact> contacts;
    std::vector<GBorder> contact_borders;  // host copy of each contact border
    std::vector<V2> normals;  // distinct border normals; GBorder::ncls indexes it
    std::vector<double> Teq, Tinit;
    std::vector<int> reservoir;
    std::vector<int> tto;              // periodic: target box, -1 otherwise
    std::vector<V2> translation;       // periodic: translation vector
    std::vector<V2> contact_seg;       // [contact][2]: lengthened contact segment
    std::vector<int> mat;              // material of each box (batched runs)
    bool periodic = false;             // any periodic box
    double thickness = 0;
    // axis-aligned grid description (production fast path); valid when
    // rect_grid is true: cell (i, j) -> box id or -1 (void / pore),
    // -2 - r for reservoir r.
    bool rect_grid = false;
    int gnx = 0, gny = 0;
    std::vector<double> gx, gy;    // grid lines, gnx+1 and gny+1 values
    std::vector<int> gcell;        // [gnx * gny], i-major
};

// Translations that need no search (geometry_2d::translate,
// include/geometry_2d.hpp:366-493): for each periodic box P with target TB
// and translation t, the unit normal u of t and the intervals of r0.u
// (r0 the entry point into P) in which the segment r0 -> r0 + 1.0005 t
// can meet exactly one candidate contact of TB (neither TB itself, a
// periodic box nor a reservoir), kept `margin` nm away from the ends of
// every candidate's interval.  rng[box] = (first interval, count).
struct IntPair {  // the layout of int2
    int x, y;
};
struct TranslationFast {
    std::vector<TransFast> iv;
    std::vector<IntPair> rng;
    std::vector<V2> u;
};
TranslationFast build_translation_fast(const HostGeometry& g, double margin = 1.0e-2);

// Alias entry of a Lambert row: pick slot j, keep its mode with probability
// prob, else take alt (Walker / Vose).
struct AliasRow {
    float prob;
    int keep;
    int alt;
    int pad;
};
// Alias entry of a mode distribution: keep = the slot itself.
struct Alias {
    float prob;
    int alt;
};

struct LambertTable {
    int nclass = 0;
    std::vector<long long> row_ptr;  // [nclass][n + 1]
    std::vector<int> col;            // outgoing mode of each entry
    std::vector<double> cdf;         // replay: cumulative values (std::map semantics)
    std::vector<AliasRow> alias;     // production
};

struct WallGenerator {
    int res, box, sign;
    V2 p1, nd, sa, sb;  // contact border seen from the reservoir
    double flux;        // J nm^-2 ps^-1
    double energy;      // J / ps (|flux| * length * thickness)
};

struct Generators {
    // BTE_SOURCE_WALLS
    std::vector<WallGenerator> walls;
    std::vector<double> wall_cum;  // cumulative weights of the walls
    // BTE_SOURCE_INITIAL
    std::vector<int> init_box;            // boxes with Tinit != Teq
    std::vector<int> init_sign;
    std::vector<long long> init_first;    // first particle of each box (prefix)
    std::vector<double> init_energy;      // J per box
    // distributions: one row of n modes per generator (walls or init boxes)
    std::vector<double> cdf;              // [ngen][n]
    std::vector<Alias> alias;             // [ngen][n]
    double total_energy = 0;              // J/ps (walls) or J (initial)
};

HostModes build_modes(const bte_mode_table* mt);
HostGeometry build_geometry(const bte_geometry* g);

// Broadening width of every mode (base_sigma with the outliers clipped).
std::vector<double> mode_sigmas(const HostModes& m);

// Resampling distribution after an RTA scattering: pmf ~ C(omega, T) w.
void build_resample(const HostModes& m, double T0, std::vector<double>& cdf,
                    std::vector<Alias>& alias);

// Lambert table rows per (wall-normal class, incoming mode).
LambertTable build_lambert(const HostModes& m, const HostGeometry& g, int nthreads);

// A crystal's generators inside the concatenated mode space of several
// crystals: only the reservoirs (walls) or boxes (initial deviation) of
// material `mat`, their rows `n` long with the crystal's modes from `off`
// and zeros elsewhere.
struct GenEmbed {
    int mat;
    std::size_t off, n;
    double thickness = 0.;  // of the crystal's boxes (0: the geometry's)
};
Generators build_wall_generators(const HostModes& m, const HostGeometry& g, bool required = true,
                                 const GenEmbed* e = nullptr);

// Temperature-gradient sources of the steady state: one Nabla_T_distribution
// per box that is neither a reservoir nor periodic (src/sampling.cpp:118-187,
// Init_generator src/RTA_MC2D.cpp:354-437), in ascending box order.
struct GradGenerators {
    std::vector<int> box;
    std::vector<double> cum;            // cumulative box weights
    std::vector<double> cdf;            // [nbox][n]
    std::vector<Alias> alias;           // [nbox][n]
    std::vector<signed char> sign;      // [nbox][n] sign of -gradT . v
    std::vector<double> energy;         // get_energy(Vbox / Vucell) per box
    double total_energy = 0;
};
GradGenerators build_gradient_generators(const HostModes& m, const HostGeometry& g, double gx,
                                         double gy);
// Nabla_T sources with a gradient per box (grad[box], K/nm); boxes without
// a gradient get no source.  With an embedding: only the boxes of crystal
// e->mat, rows over the concatenated modes (the crystal's at e->off).
GradGenerators build_gradient_generators_boxes(const HostModes& m, const HostGeometry& g,
                                               const std::vector<V2>& grad, const GenEmbed* e = nullptr);
// Several crystals' gradient sources as one set in ascending box order,
// the box weights renormalised over all of them.
GradGenerators merge_gradient_generators(const std::vector<GradGenerators>& G);
// calculate_gradientT (src/geometry_2d.cpp:524-575): per box that is neither
// a reservoir nor periodic, the least-squares gradient of Teq from the
// centres of its neighbours of that kind, the minimum-norm one when they are
// collinear (the reference solves with Eigen's complete orthogonal
// decomposition); zero for every other box, K/nm.
std::vector<V2> calculate_gradientT(const HostGeometry& g);
// The minimum-norm least-squares solution g of rows (hx_i, hy_i) . g = d_i
// (zero without rows).
V2 min_norm_lstsq2(const std::vector<double>& hx, const std::vector<double>& hy, const std::vector<double>& d);
// Distributions of the initial deviation per box (no particle counts).
Generators build_initial_generators(const HostModes& m, const HostGeometry& g, const GenEmbed* e = nullptr);
// Particle counts per box for N particles (Ntogenerate stochastic rounding):
// fills init_first and returns Eeff.
double initial_counts(Generators& G, int64_t nparticles, uint64_t seed);

// Walker/Vose alias table of unnormalised non-negative weights.
void alias_table(const double* w, int n, Alias* out);

// Mode-mirror maps for specular reflection on the q grid: for each wall
// normal class, the mode with v_n reversed (or -1 when the class is not
// axis-aligned or the grid has no mirror image).
std::vector<int> build_mirror(const HostModes& m, const HostGeometry& g);

// Natural cubic spline through (X, Y), X ascending (CubicSpline1D,
// src/interpolation.cpp:20-103).
struct Spline1D {
    std::vector<double> a, b, c, d, x0, xs;
    void build(const std::vector<double>& X, const std::vector<double>& Y);
    double interp(double x) const;
};

double calc_cv(const HostModes& m, double T);
double bose_einstein(double omega, double T);
double bose_einstein_kernel(double omega, double T);

// ---- several crystals (one mode table per material, joined by diffuse
// mismatch interfaces).  Their modes are concatenated: global mode
// off[k] + j is mode j of crystal k.
HostModes concat_modes(const std::vector<HostModes>& crys, std::vector<std::size_t>& off);
// The crystals' Lambert tables (each built on its own modes) as one table
// over the global modes; rows keep their crystal's modes.
LambertTable merge_lambert(const std::vector<LambertTable>& L, const std::vector<HostModes>& crys,
                           const std::vector<std::size_t>& off);
std::vector<int> merge_mirror(const std::vector<std::vector<int>>& mir, const std::vector<HostModes>& crys,
                              const std::vector<std::size_t>& off, int nclass);
// Generators of each crystal (embedded rows) as one set: walls in crystal
// order, the wall weights over all of them.
Generators merge_generators(std::vector<Generators>& G, bool walls, bool required);

// The diffuse mismatch table of the interface from crystal A (modes at
// offset offA) to crystal B (offB), normal n from A to B, cells' volumes VA,
// VB (scaled to the thickness), broadening factor 0.1, at Tref
// (Diffuse_mismatch_distribution, src/sampling.cpp:437-830, side A lists):
// for global incident mode K, entries [row[K], row[K + 1]) of (global mode
// out, side out: 0 = A, 1 = B, cumulative).
struct DmmTable {
    std::vector<long long> row;  // n_total + 1
    std::vector<int> out, side;
    std::vector<double> cum;
};
DmmTable build_dmm_table(const HostModes& A, std::size_t offA, const HostModes& B, std::size_t offB,
                         std::size_t n_total, V2 n, double VA, double VB, double Tref, int nthreads);

}  // namespace bte
