// ref_pins.cpp - golden vectors computed by the reference's own code.
//
// Test infrastructure.  oracle/build_ref.py copies the cited reference
// functions, by line range, into oracle/_ref/snip/*.inc (never into the
// repository), compiles this harness against them and against the
// reference's vendored Eigen and pcg-cpp headers, runs it on the inputs it
// writes to oracle/_ref/, and stores the output as tests/golden/ref_pins.json.
// tests/test_ref_pins.py then feeds the same inputs to the CPU restatement
// (oracle/rta_oracle.cpp) and requires the same results.
//
// The reference's full headers need Boost, TBB and MPI, which are absent, so
// this file provides small stand-ins for the few names the extracted code
// uses: boost::math::normal and its pdf (closed form), the Gamma pdf of the
// spectral weights (not exercised), serialization::access (a declaration),
// an MPI communicator of one rank, and a serial tbb::parallel_for.  The
// stand-in Gamma_grid holds a mode table with trivial q-point symmetry
// (every q point is its own class), as the restatement does.  What the
// stand-ins compute is not pinned by this file; everything else is the
// reference's code.
//
// Functions pinned (reference file:line of the extracted definitions):
//   include/utilities.hpp:214 almost_equal, :343 my_jobs,
//     :385 bose_einstein, :401 bose_einstein_kernel
//   include/deviational_particle.hpp:27-38 particle_sign, get_particle_sign
//   src/isotopic_scattering.cpp:31 calc_percentiles_log
//   include/qpoint_grid.hpp:179 Gamma_grid::base_sigma
//   include/sampling.hpp:36-315 random_dt and the distribution classes
//   src/sampling.cpp:26-364 fill_cumulative, BE_derivative, Nabla_T, ref,
//     Isothermal_wall, outTref and planar_source distributions
//   src/RTA_MC2D.cpp:140 get_bin_index, :150 spectral_decomposition,
//     :547 diffusive_bouncing (table and bounce), :699 process_segment
//     (transient), :784 process_segment (periodic), :843 get_v
//   include/collision_operator.hpp:216 error_bound, :241 propagator_H
//   src/collision_operator.cpp:815 Arnoldi_algorithm, :854-929
//     propagator_H methods and lirp, :931-1064 save_P, load_P, build_P
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <vector>

#include <Eigen/Dense>
#include <unsupported/Eigen/MatrixFunctions>
#include <pcg_random.hpp>

#include <constants.hpp>   // reference include/constants.hpp (standard headers only)
#include <exceptions.hpp>  // reference include/exceptions.hpp (standard headers only)

// ------------------------------------------------------------ stand-ins
namespace boost {
namespace math {
struct normal {
    double mean, sd;
    normal(double m, double s) : mean(m), sd(s) {}
};
// Closed form of the normal density (the restatement uses the same).
inline double pdf(const normal& d, double x) {
    double e = x - d.mean;
    e *= -e;
    e /= 2 * d.sd * d.sd;
    double r = std::exp(e);
    r /= d.sd * std::sqrt(2. * alma::constants::pi);
    return r;
}
// Derivative of the regularised lower incomplete gamma function: the Gamma
// density x^(a-1) e^-x / Gamma(a), in log space.
inline double gamma_p_derivative(double a, double x) {
    return std::exp((a - 1.) * std::log(x) - x - std::lgamma(a));
}
}  // namespace math
namespace serialization {
class access;
}
namespace mpi {
struct communicator {
    int rank() const { return 0; }
    int size() const { return 1; }
    void barrier() const {}
    void abort(int code) const { std::exit(code); }
};
template <class A, class B, class R>
void scatter(const communicator&, A&, B&, R) {}
}  // namespace mpi
}  // namespace boost

namespace tbb {
template <class T>
struct blocked_range {
    T b, e;
    blocked_range(T b_, T e_) : b(b_), e(e_) {}
    T begin() const { return b; }
    T end() const { return e; }
};
template <class R, class F>
void parallel_for(const R& r, const F& f) { f(r); }
}  // namespace tbb

namespace alma {
#include "utilities_almost_equal.inc"
#include "utilities_my_jobs.inc"
#include "utilities_bose_einstein.inc"
#include "utilities_bose_einstein_kernel.inc"
#include "particle_sign.inc"
#include "calc_percentiles_log.inc"

// One q point of the stand-in grid: omega (nb) and group velocities (3 x nb)
// (wfs: eigenvectors, read only by the layer-coupling branch of the
// mismatch model, which the pins do not take).
struct Spectrum_at_point {
    Eigen::ArrayXd omega;
    Eigen::ArrayXXd vg;
    Eigen::MatrixXcd wfs;
};

// Stand-in for alma::Gamma_grid with trivial symmetry.
class Gamma_grid {
public:
    std::size_t nqpoints = 0;
    Eigen::Matrix3d dq;
    std::vector<Spectrum_at_point> spectra;
    const Spectrum_at_point& get_spectrum_at_q(std::size_t iq) const { return spectra.at(iq); }
    std::size_t get_nequivalences() const { return nqpoints; }
    std::size_t get_representative(std::size_t ic) const { return ic; }
    std::vector<std::array<std::size_t, 2>> equivalent_qpairs(const std::array<std::size_t, 2>& q) const {
        return {q};
    }
#include "qpoint_grid_base_sigma.inc"
};

#include "sampling_hpp.inc"
#include "sampling_cpp.inc"

// Stand-ins of Crystal_structure (the cell volume and lattice vectors) and of
// D_particle (its mode indices) for the diffuse mismatch model.
struct Crystal_structure {
    double V = 0;
    Eigen::Matrix3d lattvec = Eigen::Matrix3d::Identity();
};
struct D_particle {
    std::size_t q = 0, alpha = 0;
};
#include "dos_gaussian.inc"
// the lookup tables of the mismatch model are private: the pins read them
#define private public
#include "sampling_hpp_dmm.inc"
#undef private
#include "sampling_cpp_dmm.inc"

#include "collision_error_bound.inc"
void Arnoldi_algorithm(const Eigen::MatrixXd& A, const Eigen::VectorXd& b, int n, Eigen::MatrixXd& B,
                       Eigen::MatrixXd& H, double t = 1.0);
#include "collision_propagator_H_class.inc"
alma::propagator_H lirp(alma::propagator_H& H1, alma::propagator_H& H2, double T1, double T2, double Tx);
void build_P(Eigen::MatrixXd& A, Eigen::MatrixXd& P, double t, boost::mpi::communicator& world,
             double eps = 1.0e-8);
#include "collision_arnoldi.inc"
#include "collision_propagator_H_methods.inc"
#include "collision_save_load_build_P.inc"

// Stand-in of geometry_2d for calculate_gradientT: the flags, Teq, centre,
// id and contact map (keyed by neighbour id) it reads.
struct geom2d_border {};
class geometry_2d {
public:
    double Teq = -1.;
    bool reservoir = false, periodic = false;
    Eigen::Vector2d center = Eigen::Vector2d::Zero();
    std::size_t id = 0;
    std::map<std::size_t, std::vector<geom2d_border>> contacts;
    Eigen::Vector2d get_center() const { return center; }
    std::size_t get_id() { return id; }
    std::map<std::size_t, std::vector<geom2d_border>>& get_contacts() { return contacts; }
};
#include "geometry_calculate_gradientT.inc"
}  // namespace alma

#include "rta_gamma_pdf.inc"
#include "rta_get_bin_index.inc"
#include "rta_spectral_decomposition.inc"
using gridData = std::unordered_map<std::string, std::unique_ptr<alma::Gamma_grid>>;
namespace generators {
#include "rta_diffusive_bouncing.inc"
}
#include "rta_process_segment_transient.inc"
#include "rta_process_segment_periodic.inc"
#include "rta_get_v.inc"

// ------------------------------------------------------------ harness
namespace {

// Read access to the protected state of the distributions.
template <class D>
struct Probe : D {
    using D::D;
    const std::vector<double>& cum() const { return this->cumulative; }
    const std::vector<alma::particle_sign>& sg() const { return this->signs; }
    double csum() const { return this->cumulsum; }
};

std::string num(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "Infinity" : "-Infinity";
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", x);
    return b;
}

struct Json {
    std::ostringstream o;
    bool first = true;
    void key(const char* k) {
        o << (first ? "\n" : ",\n") << " \"" << k << "\": ";
        first = false;
    }
};

std::string arr(const std::vector<double>& v) {
    std::string s = "[";
    for (std::size_t i = 0; i < v.size(); ++i) s += (i ? ", " : "") + num(v[i]);
    return s + "]";
}
std::string arri(const std::vector<long long>& v) {
    std::string s = "[";
    for (std::size_t i = 0; i < v.size(); ++i) s += (i ? ", " : "") + std::to_string(v[i]);
    return s + "]";
}
template <class E>
std::vector<double> vec(const E& e) {
    std::vector<double> v(std::size_t(e.size()));
    for (Eigen::Index i = 0; i < e.size(); ++i) v[std::size_t(i)] = e(i);
    return v;
}
std::vector<long long> signs_of(const std::vector<alma::particle_sign>& s) {
    std::vector<long long> v;
    for (auto x : s) v.push_back(static_cast<long long>(x));
    return v;
}

struct Table {
    std::size_t nq = 0, nb = 0;
    std::vector<double> omega, vg, w, dq;
    double V = 0, c = 0;
};

Table read_table(const char* path) {
    std::ifstream in(path);
    Table t;
    in >> t.nq >> t.nb;
    const std::size_t n = t.nq * t.nb;
    t.omega.resize(n);
    t.vg.resize(3 * n);
    t.w.resize(n);
    for (std::size_t k = 0; k < n; ++k) in >> t.omega[k] >> t.vg[3 * k] >> t.vg[3 * k + 1] >> t.vg[3 * k + 2] >> t.w[k];
    t.dq.resize(9);
    for (auto& x : t.dq) in >> x;
    in >> t.V >> t.c;
    if (!in) {
        std::fprintf(stderr, "bad table file %s\n", path);
        std::exit(2);
    }
    return t;
}

std::unique_ptr<alma::Gamma_grid> make_grid(const Table& t) {
    auto g = std::make_unique<alma::Gamma_grid>();
    g->nqpoints = t.nq;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) g->dq(r, c) = t.dq[std::size_t(3 * c + r)];  // column-major
    g->spectra.resize(t.nq);
    for (std::size_t iq = 0; iq < t.nq; ++iq) {
        auto& s = g->spectra[iq];
        s.omega.resize(Eigen::Index(t.nb));
        s.vg.resize(3, Eigen::Index(t.nb));
        for (std::size_t ib = 0; ib < t.nb; ++ib) {
            const std::size_t k = iq * t.nb + ib;
            s.omega(Eigen::Index(ib)) = t.omega[k];
            for (int a = 0; a < 3; ++a) s.vg(a, Eigen::Index(ib)) = t.vg[3 * k + std::size_t(a)];
        }
    }
    return g;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_pins <mode table file> <scratch dir>  (writes <scratch dir>/ref_pins.json)\n");
        return 2;
    }
    const Table tab = read_table(argv[1]);
    const std::string scratch = argv[2];
    auto gridp = make_grid(tab);
    const alma::Gamma_grid& grid = *gridp;
    const std::size_t n = tab.nq * tab.nb;
    Json J;

    // --- utilities
    {
        const double pairs[][2] = {{1.0, 1.0},    {1.0, 1.0 + 1e-6}, {1.0, 1.0 + 2e-5}, {0.0, 5e-9},
                                   {0.0, 2e-8},   {1e-9, 0.0},       {-3.0, -3.00002},  {100.0, 100.001},
                                   {100.0, 100.0011}, {0.0, 0.0}};
        std::string s = "[";
        for (std::size_t i = 0; i < std::size(pairs); ++i) {
            const bool r = alma::almost_equal(pairs[i][0], pairs[i][1]);
            s += (i ? ", [" : "[") + num(pairs[i][0]) + ", " + num(pairs[i][1]) + ", " + (r ? "1" : "0") + "]";
        }
        J.key("almost_equal");
        J.o << s << "]";
        std::vector<double> om, Ts, be, ke;
        const double oms[] = {0.0, 1e-320, 1e-300, 1e-10, 1e-3, 0.5, 3.0, 10.0, 60.0, 150.0, 188.0, 1e4, 3e5};
        const double tts[] = {1.0, 100.0, 300.0, 1000.0};
        for (double T : tts)
            for (double o : oms) {
                om.push_back(o);
                Ts.push_back(T);
                be.push_back(alma::bose_einstein(o, T));
                ke.push_back(alma::bose_einstein_kernel(o, T));
            }
        J.key("bose");
        J.o << "{\"omega\": " << arr(om) << ", \"T\": " << arr(Ts) << ", \"be\": " << arr(be)
            << ", \"kernel\": " << arr(ke) << "}";
        std::vector<long long> jobs;
        for (std::size_t nj : {0, 1, 7, 100})
            for (std::size_t np : {1, 3, 16})
                for (std::size_t id = 0; id < np; ++id) {
                    auto r = alma::my_jobs(nj, np, id);
                    jobs.push_back((long long)nj);
                    jobs.push_back((long long)np);
                    jobs.push_back((long long)id);
                    jobs.push_back((long long)r[0]);
                    jobs.push_back((long long)r[1]);
                }
        J.key("my_jobs");
        J.o << arri(jobs);
    }

    // --- time grid, bins and the segment split
    {
        const double dt = 10., maxtime_in = 100.;
        std::size_t ntime = std::size_t(std::floor(maxtime_in / dt + 1.0e-6)) + 1;
        const double maxtime = double(ntime - 1) * dt;
        Eigen::VectorXd timegrid = Eigen::VectorXd::LinSpaced(Eigen::Index(ntime), 0.0, maxtime);
        const double ts[] = {-5.0, 0.0, 1e-300, 5.0, 10.0, 10.000000000000002, 9.999999999999998, 55.5,
                             90.0, 99.99, 100.0, 100.00000001, 150.0};
        std::vector<double> tv;
        std::vector<long long> idx;
        for (double t : ts) {
            tv.push_back(t);
            idx.push_back((long long)get_bin_index(timegrid, t));
        }
        J.key("bin_index");
        J.o << "{\"grid\": " << arr(vec(timegrid)) << ", \"t\": " << arr(tv) << ", \"index\": " << arri(idx) << "}";

        const double segs[][4] = {{0.0, 3.5, 1, 0},     {2.0, 27.0, -1, 1},    {10.0, 20.0, 1, 0},
                                  {9.5, 10.0, 1, 1},    {-4.0, 12.0, 1, 0},    {95.0, 100.00000001, -1, 1},
                                  {33.3, 33.3, 1, 0},   {0.0, 100.0, 1, 1},    {47.123456789, 61.987654321, -1, 0},
                                  {99.0, 130.0, 1, 1}};
        const double vels[][2] = {{1.25, -0.5}, {-3.0, 0.0}, {0.0, 2.0}, {0.7, 0.3}, {-1.1, -2.2},
                                  {5.0, 5.0},  {0.0, 0.0}, {2.5, -1.5}, {-0.25, 4.0}, {1.0, 1.0}};
        std::string s = "[";
        spectral_decomposition sd;
        for (std::size_t c = 0; c < std::size(segs); ++c) {
            Eigen::ArrayXXd gz = Eigen::ArrayXXd::Zero(2, Eigen::Index(ntime - 1));
            Eigen::ArrayXXd gx = gz, gy = gz;
            alma::particle_sign sign = segs[c][2] > 0 ? alma::particle_sign::plus : alma::particle_sign::minus;
            Eigen::Vector2d vg(vels[c][0], vels[c][1]);
            const std::size_t ibox = std::size_t(segs[c][3]);
            process_segment(ibox, segs[c][0], segs[c][1], sign, timegrid, vg, gz, gx, gy, 1.0, 0, 0, sd);
            s += std::string(c ? ", " : "") + "{\"box\": " + std::to_string(ibox) + ", \"t0\": " + num(segs[c][0]) +
                 ", \"t1\": " + num(segs[c][1]) + ", \"sign\": " + num(segs[c][2]) + ", \"v\": [" +
                 num(vels[c][0]) + ", " + num(vels[c][1]) + "], \"gz\": " + arr(vec(gz.row(Eigen::Index(ibox)))) +
                 ", \"jx\": " + arr(vec(gx.row(Eigen::Index(ibox)))) + ", \"jy\": " +
                 arr(vec(gy.row(Eigen::Index(ibox)))) + "}";
        }
        J.key("segment");
        J.o << s << "]";

        std::string p = "[";
        for (std::size_t c = 0; c < std::size(vels); ++c) {
            Eigen::ArrayXd gz = Eigen::ArrayXd::Zero(3), gx = gz, gy = gz, phi = gz;
            alma::particle_sign sign = (c % 3 == 1) ? alma::particle_sign::minus : alma::particle_sign::plus;
            Eigen::Vector2d vg(vels[c][0], vels[c][1]);
            const double d = 0.37 + 1.91 * double(c);
            process_segment(c % 3, sign, d, vg, gz, gx, gy, phi, 1.0, 0, 0, sd, c % 2 == 0);
            p += std::string(c ? ", " : "") + "{\"box\": " + std::to_string(c % 3) + ", \"sign\": " +
                 std::to_string(static_cast<int>(sign)) + ", \"dt\": " + num(d) + ", \"v\": [" + num(vels[c][0]) +
                 ", " + num(vels[c][1]) + "], \"evalphi\": " + std::to_string(c % 2 == 0 ? 1 : 0) +
                 ", \"gz\": " + arr(vec(gz)) + ", \"jx\": " + arr(vec(gx)) + ", \"jy\": " + arr(vec(gy)) +
                 ", \"phi\": " + arr(vec(phi)) + "}";
        }
        J.key("segment_periodic");
        J.o << p << "]";
    }

    // --- velocities
    {
        std::vector<double> vx, vy;
        for (std::size_t iq = 0; iq < tab.nq; ++iq)
            for (std::size_t ib = 0; ib < tab.nb; ++ib) {
                Eigen::Vector2d v = get_v(grid, ib, iq);
                vx.push_back(v(0));
                vy.push_back(v(1));
            }
        J.key("get_v");
        J.o << "{\"vx\": " << arr(vx) << ", \"vy\": " << arr(vy) << "}";
    }

    // --- distributions
    {
        Eigen::ArrayXXd w(Eigen::Index(tab.nb), Eigen::Index(tab.nq));
        for (std::size_t iq = 0; iq < tab.nq; ++iq)
            for (std::size_t ib = 0; ib < tab.nb; ++ib) w(Eigen::Index(ib), Eigen::Index(iq)) = tab.w[iq * tab.nb + ib];
        pcg64 r0(20261203ULL, 41ULL);
        Probe<alma::BE_derivative_distribution> be(grid, w, 300.0, r0);
        std::vector<long long> smp;
        for (int i = 0; i < 64; ++i) {
            auto a = be.sample();
            smp.push_back((long long)(a[1] * tab.nb + a[0]));
        }
        J.key("be_derivative");
        J.o << "{\"T\": 300.0, \"seed\": 20261203, \"stream\": 41, \"cumulative\": " << arr(be.cum())
            << ", \"samples\": " << arri(smp) << "}";

        const double normals[][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0.6, 0.8, 0}};
        const double temps[][2] = {{301.0, 300.0}, {299.0, 300.0}, {301.0, 300.0}, {299.0, 300.0}, {310.0, 300.0}};
        const double vuc = tab.V * 100.0 / tab.c;
        std::string s = "[";
        for (std::size_t c = 0; c < std::size(normals); ++c) {
            pcg64 r(7ULL, 100ULL + c);
            Eigen::Vector3d nrm(normals[c][0], normals[c][1], normals[c][2]);
            Probe<alma::Isothermal_wall_distribution> d(grid, temps[c][0], temps[c][1], nrm, r);
            std::vector<long long> ng;
            for (int i = 0; i < 16; ++i) ng.push_back((long long)d.Ntogenerate(1.0 + 0.25 * i, 37.5, 2.5e-22));
            s += std::string(c ? ", " : "") + "{\"normal\": [" + num(normals[c][0]) + ", " + num(normals[c][1]) +
                 ", " + num(normals[c][2]) + "], \"Tw\": " + num(temps[c][0]) + ", \"Teq\": " +
                 num(temps[c][1]) + ", \"stream\": " + std::to_string(100 + c) + ", \"cumulative\": " +
                 arr(d.cum()) + ", \"cumulsum\": " + num(d.csum()) + ", \"sign\": " +
                 std::to_string(static_cast<int>(d.sg()[0])) + ", \"vuc\": " + num(vuc) + ", \"flux\": " +
                 num(d.get_flux(vuc)) + ", \"ntogen\": " + arri(ng) + "}";
        }
        J.key("isothermal_wall");
        J.o << s << "]";

        pcg64 r2(7ULL, 200ULL);
        Probe<alma::outTref_distribution> ot(grid, 301.3, 300.0, r2);
        std::vector<long long> ng;
        for (int i = 0; i < 16; ++i) ng.push_back((long long)ot.Ntogenerate(400.0 + 37.0 * i, 3e-21));
        J.key("out_tref");
        J.o << "{\"Tinit\": 301.3, \"Tref\": 300.0, \"seed\": 7, \"stream\": 200, \"cumulative\": "
            << arr(ot.cum()) << ", \"cumulsum\": " << num(ot.csum()) << ", \"energy\": " << num(ot.get_energy(400.0))
            << ", \"sign\": " << static_cast<int>(ot.sg()[0]) << ", \"ntogen\": " << arri(ng) << "}";

        pcg64 r3(7ULL, 300ULL);
        Eigen::Vector3d grad(0.01, -0.003, 0.0);
        Probe<alma::Nabla_T_distribution> nt(grid, grad, 300.0, r3);
        std::vector<long long> ng2;
        for (int i = 0; i < 16; ++i) ng2.push_back((long long)nt.Ntogenerate(1.0, 400.0 + 37.0 * i, 3e-22));
        J.key("nabla_t");
        J.o << "{\"gradient\": [0.01, -0.003, 0.0], \"T\": 300.0, \"seed\": 7, \"stream\": 300, \"cumulative\": "
            << arr(nt.cum()) << ", \"signs\": " << arri(signs_of(nt.sg())) << ", \"cumulsum\": " << num(nt.csum())
            << ", \"energy\": " << num(nt.get_energy(400.0)) << ", \"ntogen\": " << arri(ng2) << "}";

        pcg64 r4(20261203ULL, 9ULL);
        std::vector<double> dts;
        const double ws[] = {0.5, 2.0, 0.013, 7.5};
        for (int i = 0; i < 32; ++i) dts.push_back(alma::random_dt(ws[i % 4], r4));
        J.key("random_dt");
        J.o << "{\"seed\": 20261203, \"stream\": 9, \"w\": [0.5, 2.0, 0.013, 7.5], \"dt\": " << arr(dts) << "}";
    }

    // --- Lambert table and bounces
    {
        gridData gd;
        gd["m"] = make_grid(tab);
        generators::diffusive_bouncing db(gd);
        const auto& lam = db.lambert["m"];
        std::vector<long long> nnz;
        std::vector<double> sums;
        for (std::size_t k = 0; k < n; ++k) {
            std::map<std::size_t, double> row(lam[k].begin(), lam[k].end());
            double s = 0.;
            for (auto& [f, v] : row) s += v;
            nnz.push_back((long long)row.size());
            sums.push_back(s);
        }
        std::string rows = "[";
        const std::size_t picks[] = {3, 4, n / 3 + 1, n / 2 + 5, n - 1};
        for (std::size_t c = 0; c < std::size(picks); ++c) {
            std::map<std::size_t, double> row(lam[picks[c]].begin(), lam[picks[c]].end());
            std::vector<long long> idx;
            std::vector<double> val;
            for (auto& [f, v] : row) {
                idx.push_back((long long)f);
                val.push_back(v);
            }
            rows += std::string(c ? ", " : "") + "{\"mode\": " + std::to_string(picks[c]) + ", \"index\": " +
                    arri(idx) + ", \"value\": " + arr(val) + "}";
        }
        J.key("lambert");
        J.o << "{\"nnz\": " << arri(nnz) << ", \"sum\": " << arr(sums) << ", \"rows\": " << rows << "]}";

        const double nps[][3] = {{0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
        std::string b = "[";
        int cnt = 0;
        // incoming modes that move (a mode without velocity never reaches a
        // wall; for it the reference's bounce would read end() of an empty map)
        std::vector<std::size_t> movers;
        for (std::size_t want : {std::size_t(7), n / 4 + 2, n / 2 + 1, n - 2}) {
            std::size_t k = want;
            while (k < n && (lam[k].empty() || (grid.get_spectrum_at_q(k / tab.nb).vg.col(k % tab.nb).abs().maxCoeff() == 0.)))
                k = (k + 1) % n;
            movers.push_back(k);
        }
        for (std::size_t c = 0; c < std::size(nps); ++c)
            for (std::size_t imode : movers) {
                pcg64 r(31ULL, 1000ULL + 10 * c + imode);
                std::vector<long long> out;
                for (int i = 0; i < 24; ++i) {
                    auto pr = db.bounce(Eigen::Vector3d(nps[c][0], nps[c][1], nps[c][2]), "m", imode, gd, r);
                    out.push_back((long long)(pr.second * tab.nb + pr.first));
                }
                b += std::string(cnt++ ? ", " : "") + "{\"npout\": [" + num(nps[c][0]) + ", " + num(nps[c][1]) +
                     "], \"mode\": " + std::to_string(imode) + ", \"seed\": 31, \"stream\": " +
                     std::to_string(1000 + 10 * c + imode) + ", \"out\": " + arri(out) + "}";
            }
        J.key("bounce");
        J.o << b << "]";
    }

    // --- propagators
    {
        const int m = 7;
        Eigen::MatrixXd P(m, m), Q(m, m);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) {
                P(i, j) = std::sin(1.3 * i + 0.7 * j + 0.1) * ((i * 3 + j) % 4 == 0 ? -0.5 : 1.0);
                Q(i, j) = std::cos(0.9 * i - 0.4 * j + 0.2) * ((i + 2 * j) % 5 == 0 ? -1.0 : 0.8);
            }
        P(2, 3) = 0.0;
        std::string s = "[";
        for (int j = 0; j < m; ++j) {
            Eigen::VectorXd col = P.col(j);
            alma::propagator_H h(col);
            std::vector<double> Rs = {0.0, 1.0, 0.5, 1e-300};
            auto sc = h.get_signed_cumm();
            for (Eigen::Index i = 0; i < sc.size(); ++i) {
                Rs.push_back(std::fabs(sc(i)));
                Rs.push_back(std::nextafter(std::fabs(sc(i)), 0.0));
                if (std::fabs(sc(i)) < 1.0) Rs.push_back(std::nextafter(std::fabs(sc(i)), 2.0));
            }
            // the reference draws R in [0, 1); its last |cumm| can sit an ulp
            // below 1 (a running sum over Eigen's vectorised total), so probes
            // stay at or below it
            const double top = std::fabs(sc(sc.size() - 1));
            Rs.erase(std::remove_if(Rs.begin(), Rs.end(), [top](double r) { return r > top; }), Rs.end());
            std::vector<long long> gs;
            for (double R : Rs) {
                auto g = h.get(R);
                gs.push_back(g.first);
                gs.push_back((long long)g.second);
            }
            s += std::string(j ? ", " : "") + "{\"col\": " + std::to_string(j) + ", \"signed_cumm\": " + arr(vec(sc)) +
                 ", \"abssum\": " + num(h.get_pcol_abssum()) + ", \"R\": " + arr(Rs) + ", \"get\": " + arri(gs) + "}";
        }
        std::string L = "[";
        int c = 0;
        for (double Tx : {300.0, 150.0, 400.0}) {
            Eigen::VectorXd a = P.col(1), bq = Q.col(1);
            alma::propagator_H h1(a), h2(bq);
            alma::propagator_H hx = alma::lirp(h1, h2, 200.0, 400.0, Tx);
            L += std::string(c++ ? ", " : "") + "{\"T1\": 200.0, \"T2\": 400.0, \"Tx\": " + num(Tx) +
                 ", \"signed_cumm\": " + arr(vec(hx.get_signed_cumm())) + ", \"abssum\": " +
                 num(hx.get_pcol_abssum()) + "}";
        }
        J.key("propagator");
        J.o << "{\"n\": " << m << ", \"P\": " << arr(std::vector<double>(P.data(), P.data() + P.size()))
            << ", \"Q\": " << arr(std::vector<double>(Q.data(), Q.data() + Q.size())) << ", \"columns\": " << s
            << "], \"lirp\": " << L << "]}";

        // save_P / load_P file layout and round trip
        boost::mpi::communicator world;
        Eigen::MatrixXd S3(3, 3);
        S3 << 0.9, -0.05, 0.01, 0.07, 0.8, -0.02, 0.03, 0.25, 1.01;
        const std::string fn = scratch + "/pin.P.eigen.bin";
        alma::save_P(fn, S3, world);
        std::ifstream f(fn, std::ios::binary);
        std::vector<unsigned char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        std::string hex;
        for (unsigned char ch : bytes) {
            char h[3];
            std::snprintf(h, sizeof h, "%02x", ch);
            hex += h;
        }
        Eigen::MatrixXd back;
        alma::load_P(fn, back, world);
        J.key("save_P");
        J.o << "{\"matrix\": " << arr(std::vector<double>(S3.data(), S3.data() + S3.size())) << ", \"hex\": \"" << hex
            << "\", \"loaded\": " << arr(std::vector<double>(back.data(), back.data() + back.size())) << "}";

        // build_P on a small energy-form operator: off-diagonal couplings
        // s_ij >= 0, diagonal -sum (columns sum to zero), symmetric
        const int nb = 10;
        Eigen::MatrixXd B = Eigen::MatrixXd::Zero(nb, nb);
        for (int i = 0; i < nb; ++i)
            for (int j = i + 1; j < nb; ++j) {
                const double sij = 0.05 + 0.4 * std::fabs(std::sin(2.1 * i + 3.7 * j));
                B(i, j) = B(j, i) = sij;
            }
        for (int j = 0; j < nb; ++j) B(j, j) = -(B.col(j).sum() - B(j, j));
        Eigen::MatrixXd Pb;
        const double t = 1.0;
        alma::build_P(B, Pb, t, world);
        int ks = 2;
        while (!(alma::error_bound(B, ks, t) / double(B.size()) < 1.0e-8)) ++ks;
        J.key("build_P");
        J.o << "{\"n\": " << nb << ", \"t\": " << num(t) << ", \"B\": "
            << arr(std::vector<double>(B.data(), B.data() + B.size())) << ", \"P\": "
            << arr(std::vector<double>(Pb.data(), Pb.data() + Pb.size())) << ", \"krylov\": " << ks << "}";
    }

    // the input table, so that the tests need nothing else
    J.key("modes");
    J.o << "{\"nq\": " << tab.nq << ", \"nb\": " << tab.nb << ", \"omega\": " << arr(tab.omega)
        << ", \"vg\": " << arr(tab.vg) << ", \"w\": " << arr(tab.w) << ", \"dq\": " << arr(tab.dq)
        << ", \"V\": " << num(tab.V) << ", \"c_lat\": " << num(tab.c) << "}";
    std::ofstream out(scratch + "/ref_pins.json");
    out << "{" << J.o.str() << "\n}\n";
    if (argc > 5) {  // calculate_gradientT on the boxes of argv[5]
        std::ifstream in(argv[5]);
        std::size_t nb = 0;
        in >> nb;
        std::vector<alma::geometry_2d> sys(nb);
        for (std::size_t i = 0; i < nb; ++i) {
            int res = 0, per = 0;
            std::size_t nc = 0;
            in >> sys[i].id >> res >> per >> sys[i].Teq >> sys[i].center(0) >> sys[i].center(1) >> nc;
            sys[i].reservoir = res != 0;
            sys[i].periodic = per != 0;
            for (std::size_t k = 0; k < nc; ++k) {
                std::size_t c = 0;
                in >> c;
                sys[i].contacts[c] = {alma::geom2d_border{}};
            }
        }
        if (!in) {
            std::fprintf(stderr, "bad gradient geometry file %s\n", argv[5]);
            return 2;
        }
        const Eigen::MatrixXd G = alma::calculate_gradientT(sys);
        std::ofstream og(scratch + "/ref_pins_grad.json");
        og << "{\"gradients\": [";
        for (std::size_t i = 0; i < nb; ++i)
            og << (i ? ", [" : "[") << num(G(0, Eigen::Index(i))) << ", " << num(G(1, Eigen::Index(i))) << "]";
        og << "]}\n";
        if (!og) return 1;
    }
    if (argc > 3) {  // the diffuse mismatch model between the tables of argv[3] and argv[4]
        const Table ta = read_table(argv[3]), tb = read_table(argv[4]);
        auto ga = make_grid(ta), gb = make_grid(tb);
        alma::Crystal_structure ca, cb;
        ca.V = ta.V;
        ca.lattvec(2, 2) = ta.c;
        cb.V = tb.V;
        cb.lattvec(2, 2) = tb.c;
        Json D;
        const double normals[][2] = {{1.0, 0.0}, {0.6, -0.8}};
        const double thick = 0.335, Tref = 300.0;
        D.key("cases");
        D.o << "[";
        for (int c = 0; c < 2; ++c) {
            Eigen::Vector3d nw(normals[c][0], normals[c][1], 0.);
            pcg64 rng(20261204ull, 900ull + unsigned(c));
            alma::Diffuse_mismatch_distribution dm(*ga, ca, *gb, cb, nw, 0.1, rng, Tref, thick, thick);
            std::string L;
            for (int side = 0; side < 2; ++side) {
                const auto& look = side == 0 ? dm.lookup_incidentA : dm.lookup_incidentB;
                std::string s = "[";
                for (std::size_t i = 0; i < look.size(); ++i) {
                    s += (i ? ", [" : "[");
                    for (std::size_t j = 0; j < look[i].size(); ++j)
                        s += std::string(j ? ", " : "") + "[" + std::to_string(std::get<0>(look[i][j]) == 'A' ? 0 : 1) +
                             ", " + std::to_string(std::get<1>(look[i][j])) + ", " + num(std::get<2>(look[i][j])) + "]";
                    s += "]";
                }
                L += std::string(side ? ", \"B\": " : "\"A\": ") + s + "]";
            }
            // draws of reemit from the object's own pcg64 (a copy of rng
            // taken at construction): incident modes of A, 8 draws each
            std::string R = "[";
            int cnt = 0;
            for (std::size_t i = 0; i < dm.lookup_incidentA.size() && cnt < 12; ++i) {
                if (dm.lookup_incidentA[i].size() < 3) continue;
                for (int d = 0; d < 8; ++d) {
                    alma::D_particle p;
                    p.q = i / ta.nb;
                    p.alpha = i % ta.nb;
                    const char side = dm.reemit('A', p);
                    R += std::string(cnt || d ? ", " : "") + "[" + std::to_string(i) + ", " +
                         std::to_string(side == 'A' ? 0 : 1) + ", " + std::to_string(p.q) + ", " +
                         std::to_string(p.alpha) + "]";
                }
                ++cnt;
            }
            R += "]";
            D.o << (c ? ", " : "") << "{\"normal\": [" << num(normals[c][0]) << ", " << num(normals[c][1])
                << "], \"seed\": 20261204, \"stream\": " << (900 + c) << ", " << L << ", \"reemit\": " << R << "}";
        }
        D.o << "]";
        D.key("thickness");
        D.o << num(thick);
        D.key("Tref");
        D.o << num(Tref);
        D.key("scalebroad");
        D.o << num(0.1);
        for (int t = 0; t < 2; ++t) {
            const Table& tt = t == 0 ? ta : tb;
            D.key(t == 0 ? "modes_A" : "modes_B");
            D.o << "{\"nq\": " << tt.nq << ", \"nb\": " << tt.nb << ", \"omega\": " << arr(tt.omega)
                << ", \"vg\": " << arr(tt.vg) << ", \"w\": " << arr(tt.w) << ", \"dq\": " << arr(tt.dq)
                << ", \"V\": " << num(tt.V) << ", \"c_lat\": " << num(tt.c) << "}";
        }
        std::ofstream od(scratch + "/ref_pins_dmm.json");
        od << "{" << D.o.str() << "\n}\n";
        if (!od) return 1;
    }
    return out ? 0 : 1;
}
