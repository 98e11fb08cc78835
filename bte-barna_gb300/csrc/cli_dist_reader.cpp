// cli_dist_reader.cpp - dist_reader_gpu, the drop-in for ALMA's dist_reader.
//
//   dist_reader_gpu <input.xml> <histogram.msgpack.bin>   (src/dist_reader.cpp:515-600)
//
// Reads the properties.msgpack.bin frames that bertamc2d_gpu (and the
// reference's beRTAMC2D) write, and for each frame whose time is one of the
// <spectral><time t=/> entries writes the phonon distribution of the
// <spectral><location bin=/> boxes (print_distribution, :270-508):
//   deltaT_omega_<box>.csv  Gamma-pdf weighted temperature per omega tick
//   jx_omega_<box>.csv, jy_omega_<box>.csv  the same weighted by v (m/s)
//   fd_<box>.csv            the distribution per q point
// Input (process_input, :75-158): the <beRTAMC2D> XML with <geometry file>,
// one <material database thickness> (the engine's BTEMODE1 mode table) and
// <spectral><resolution ticks/><location bin/><time t/></spectral>.
// Host code only: no GPU is needed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cli_io.hpp"

namespace {

using namespace bte_cli;

constexpr double kB = 1.3806488e-23;     // include/constants.hpp
constexpr double hbar = 1.054571726e-34;

bool almost_equal(double a, double b, double abstol = 1e-8, double reltol = 1e-5) {
    return std::fabs(a - b) < std::fabs(abstol) + std::fabs(reltol * b);
}

// (x / sinh x)^2, x = hbar omega / 2 kB T (include/utilities.hpp:403-417)
double be_kernel(double omega, double T) {
    const double x = 0.5 * 1e12 * hbar / kB * omega / T;
    if (x < 1e-320) return 1.;
    if (x > 300.) return 0.;
    const double s = x / std::sinh(x);
    return s * s;
}

// Gamma pdf of shape k and scale theta at x, in log space
// (boost gamma_p_derivative(k, x / theta) / theta)
double gamma_pdf(double k, double theta, double x) {
    if (!(x > 0.)) return 0.;
    const double z = x / theta;
    const double lp = (k - 1.0) * std::log(z) - z - std::lgamma(k) - std::log(theta);
    return lp > -745. ? std::exp(lp) : 0.;
}

// --------------------------------------------------------------- msgpack
// The subset the frames use: arrays, float64/float32, integers.
struct MsgReader {
    const unsigned char* p;
    const unsigned char* end;
    unsigned char byte() {
        if (p >= end) throw std::runtime_error("truncated msgpack frame");
        return *p++;
    }
    uint64_t be(int n) {
        uint64_t v = 0;
        for (int i = 0; i < n; ++i) v = (v << 8) | byte();
        return v;
    }
    std::size_t array() {
        const unsigned char c = byte();
        if ((c & 0xf0) == 0x90) return c & 0x0f;
        if (c == 0xdc) return std::size_t(be(2));
        if (c == 0xdd) return std::size_t(be(4));
        throw std::runtime_error("msgpack: expected an array");
    }
    double number() {
        const unsigned char c = byte();
        if (c <= 0x7f) return double(c);
        if (c >= 0xe0) return double(int(c) - 256);
        switch (c) {
            case 0xca: {
                const uint32_t b = uint32_t(be(4));
                float f;
                std::memcpy(&f, &b, 4);
                return double(f);
            }
            case 0xcb: {
                const uint64_t b = be(8);
                double d;
                std::memcpy(&d, &b, 8);
                return d;
            }
            case 0xcc: return double(be(1));
            case 0xcd: return double(be(2));
            case 0xce: return double(be(4));
            case 0xcf: return double(be(8));
            case 0xd0: return double(int8_t(be(1)));
            case 0xd1: return double(int16_t(be(2)));
            case 0xd2: return double(int32_t(be(4)));
            case 0xd3: return double(int64_t(be(8)));
            default: throw std::runtime_error("msgpack: unsupported type");
        }
    }
};

struct Input {
    std::vector<double> area;      // hull area per box
    std::vector<int> reservoir;
    double thickness = 0.;
    ModesFile modes;
    int nbins = 0;                  // omega ticks
    std::vector<int> boxes;         // locations
    std::vector<double> dumptimes;  // sorted
};

// convex hull area of a point set (Andrew's monotone chain), as the
// reference's boxes take the hull of their vertices (src/geometry_2d.cpp:127-153)
double hull_area(std::vector<std::pair<double, double>> p) {
    std::sort(p.begin(), p.end());
    p.erase(std::unique(p.begin(), p.end()), p.end());
    if (p.size() < 3) return 0.;
    auto cross = [](const std::pair<double, double>& o, const std::pair<double, double>& a,
                    const std::pair<double, double>& b) {
        return (a.first - o.first) * (b.second - o.second) - (a.second - o.second) * (b.first - o.first);
    };
    std::vector<std::pair<double, double>> h(2 * p.size());
    std::size_t k = 0;
    for (std::size_t i = 0; i < p.size(); ++i) {
        while (k >= 2 && cross(h[k - 2], h[k - 1], p[i]) <= 0) --k;
        h[k++] = p[i];
    }
    for (std::size_t i = p.size() - 1, t = k + 1; i > 0; --i) {
        while (k >= t && cross(h[k - 2], h[k - 1], p[i - 1]) <= 0) --k;
        h[k++] = p[i - 1];
    }
    h.resize(k - 1);
    double a2 = 0.;
    for (std::size_t i = 0; i < h.size(); ++i) {
        const auto& u = h[i];
        const auto& v = h[(i + 1) % h.size()];
        a2 += u.first * v.second - v.first * u.second;
    }
    return std::fabs(0.5 * a2);
}

Input read_input(const std::string& path) {
    auto root = read_xml(path);
    if (root->name != "beRTAMC2D") throw std::runtime_error("root element must be <beRTAMC2D>");
    const std::string base = dir_of(path);
    Input in;
    std::string gfile, dbfile;
    int nmat = 0;
    for (auto& k : root->kids) {
        if (k->name == "geometry") gfile = k->get("file");
        if (k->name == "material") {
            dbfile = k->get("database");
            in.thickness = std::stod(k->get("thickness"));
            ++nmat;
        }
        if (k->name == "spectral") {
            for (auto& q : k->kids) {
                if (q->name == "resolution") in.nbins = std::stoi(q->get("ticks"));
                if (q->name == "location") in.boxes.push_back(std::stoi(q->get("bin")));
                if (q->name == "time") in.dumptimes.push_back(std::stod(q->get("t")));
            }
        }
    }
    if (nmat != 1) throw std::runtime_error("This is currently not supported");  // one material (:148-151)
    if (gfile.empty()) throw std::runtime_error("no <geometry file>");
    if (in.nbins < 2) throw std::runtime_error("<spectral> needs <resolution ticks> of at least 2");
    if (in.dumptimes.empty()) throw std::runtime_error("<spectral> has no <time t>");
    std::sort(in.dumptimes.begin(), in.dumptimes.end());
    auto groot = read_xml(resolve(base, gfile));
    for (auto& b : groot->kids) {
        if (b->name != "Box") continue;
        const Node* v = b->child("Vertices");
        if (!v) throw std::runtime_error("<Box> without <Vertices>");
        const int rows = std::stoi(v->get("dim")), cols = std::stoi(v->get("npoints"));
        if (rows != 2) throw std::runtime_error("Error in provided vertices, bad dimension");
        std::stringstream ds(v->text);
        std::vector<double> xy(static_cast<std::size_t>(2 * cols));
        for (auto& x : xy) ds >> x;
        // <Vertices dim="2" npoints="n">: one (x, y) pair per point
        std::vector<std::pair<double, double>> pts(static_cast<std::size_t>(cols));
        for (int i = 0; i < cols; ++i) pts[std::size_t(i)] = {xy[std::size_t(2 * i)], xy[std::size_t(2 * i + 1)]};
        in.area.push_back(hull_area(pts));
        in.reservoir.push_back(b->child("Reservoir") ? 1 : 0);
    }
    for (int b : in.boxes)
        if (b < 0 || b >= int(in.area.size())) throw std::runtime_error("<location bin> beyond the boxes");
    in.modes = read_modes(resolve(base, dbfile));
    return in;
}

struct Writer {
    const Input& in;
    const std::size_t nb, nq, n;
    std::vector<double> sigma, mesh, qx, qy;
    double Cvtot = 0.;
    bool tables = false;
    std::vector<std::ofstream> od, ox, oy, of;
    std::vector<bool> first;

    explicit Writer(const Input& i)
        : in(i), nb(std::size_t(i.modes.head[1])), nq(std::size_t(i.modes.head[0])), n(nb * nq) {
        const std::size_t nbx = in.area.size();
        od.resize(nbx);
        ox.resize(nbx);
        oy.resize(nbx);
        of.resize(nbx);
        first.assign(nbx, true);
        for (int b : in.boxes) {
            const std::string id = std::to_string(b);
            od[std::size_t(b)].open("deltaT_omega_" + id + ".csv");
            ox[std::size_t(b)].open("jx_omega_" + id + ".csv");
            oy[std::size_t(b)].open("jy_omega_" + id + ".csv");
            of[std::size_t(b)].open("fd_" + id + ".csv");
        }
    }

    // broadening (base_sigma, 0 for omega = 0, log-percentile clip), the
    // omega mesh, the q points and the heat capacity at the first listed
    // box's temperature (:283-365)
    void build_tables(const std::vector<double>& temps) {
        const ModesFile& m = in.modes;
        sigma.assign(n, 0.);
        double maxf = 0.;
        for (std::size_t k = 0; k < n; ++k) {
            maxf = std::max(maxf, m.omega[k]);
            if (almost_equal(m.omega[k], 0.)) continue;
            double r[3];
            for (int j = 0; j < 3; ++j)
                r[j] = m.vg[3 * k] * m.dq[3 * j] + m.vg[3 * k + 1] * m.dq[1 + 3 * j] + m.vg[3 * k + 2] * m.dq[2 + 3 * j];
            sigma[k] = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / std::sqrt(12.);
        }
        std::vector<double> ls(n);
        for (std::size_t k = 0; k < n; ++k)
            ls[k] = sigma[k] == 0. ? std::numeric_limits<double>::lowest() : std::log(sigma[k]);
        std::sort(ls.begin(), ls.end());
        const double p25 = ls[25 * n / 100], p75 = ls[75 * n / 100];
        const double lbound = std::exp(p25 - 1.5 * (p75 - p25));
        for (auto& s : sigma)
            if (s < lbound) s = lbound;
        // LinSpaced(nbins, 0, maxf) shifted by half its first step
        mesh.resize(std::size_t(in.nbins));
        for (int i = 0; i < in.nbins; ++i) mesh[std::size_t(i)] = maxf * double(i) / double(in.nbins - 1);
        const double half = mesh[1] / 2.0;
        for (auto& x : mesh) x += half;
        // q points wrapped to [-1/2, 1/2) on the Gamma-centred n1 x n2 grid
        const int n1 = m.head[2] > 0 ? m.head[2] : 1, n2 = m.head[3] > 0 ? m.head[3] : 1;
        qx.assign(nq, 0.);
        qy.assign(nq, 0.);
        for (std::size_t iq = 0; iq < nq; ++iq) {
            const int i = int(iq) / n2, j = int(iq) % n2;
            const int ii = (i + n1 / 2) % n1 - n1 / 2, jj = (j + n2 / 2) % n2 - n2 / 2;
            qx[iq] = ii * m.dq[0] + jj * m.dq[3];
            qy[iq] = ii * m.dq[1] + jj * m.dq[4];
        }
        const double T = temps[std::size_t(in.boxes.front())];
        const double prefactor = kB / (m.V * in.thickness / m.c) / double(nq);
        Cvtot = 0.;
        for (std::size_t k = 0; k < n; ++k)
            if (!almost_equal(0., m.omega[k])) Cvtot += be_kernel(m.omega[k], T);
        Cvtot *= prefactor;
        tables = true;
    }

    void dump(double time, double Eeff, const std::vector<double>& temps,
              const std::vector<std::vector<std::pair<std::size_t, double>>>& H) {
        if (!tables) build_tables(temps);
        const ModesFile& m = in.modes;
        const std::size_t nw = mesh.size();
        for (int box : in.boxes) {
            const std::size_t b = std::size_t(box);
            if (in.reservoir[b]) continue;
            std::vector<double> d(nw, 0.), dvx(nw, 0.), dvy(nw, 0.), dfd(nq, 0.);
            const double vol = in.area[b] * in.thickness;
            double Ebox = 0.;
            for (auto& [k, value] : H[b]) {
                if (value == 0.) continue;
                const std::size_t iq = k / nb;
                const double omega = m.omega[k];
                dfd[iq] += value / omega;
                const double s = sigma[k];
                Ebox += value;
                if (almost_equal(omega, 0) || almost_equal(s, 0)) continue;
                const double kk = omega * omega / s, th = s / omega;
                for (std::size_t i = 0; i < nw; ++i) {
                    const double v = value * gamma_pdf(kk, th, mesh[i]);
                    d[i] += v;
                    dvx[i] += v * 1.0e+3 * m.vg[3 * k];
                    dvy[i] += v * 1.0e+3 * m.vg[3 * k + 1];
                }
            }
            const double vuc = m.V * in.thickness / m.c;
            for (auto& x : dfd) x *= Eeff * vuc * double(nq) / (1.0e+12 * vol * hbar);
            for (auto& x : dvx) x *= Eeff * 1.0e+27 / vol;
            for (auto& x : dvy) x *= Eeff * 1.0e+27 / vol;
            for (auto& x : d) x *= Eeff / (vol * Cvtot);
            Ebox *= Eeff / vol;
            std::cout << "Energy density of box " << box << " is " << Ebox << std::endl;
            std::cout << "Specific heat " << Cvtot * 1.0e+27 << " J/(m**3 * K)" << std::endl;
            if (first[b]) {
                for (auto* o : {&od[b], &ox[b], &oy[b]}) {
                    *o << -1 << ',';
                    for (std::size_t i = 0; i < nw; ++i) *o << mesh[i] << (i + 1 < nw ? "," : "");
                    *o << std::endl;
                }
                for (const auto* q : {&qx, &qy}) {
                    of[b] << "# ";
                    for (std::size_t i = 0; i < nq; ++i) of[b] << (*q)[i] << (i + 1 < nq ? "," : "");
                    of[b] << std::endl;
                }
                first[b] = false;
            }
            const std::vector<double>* rows[3] = {&d, &dvx, &dvy};
            std::ofstream* outs[3] = {&od[b], &ox[b], &oy[b]};
            for (int r = 0; r < 3; ++r) {
                *outs[r] << time << ',';
                for (std::size_t i = 0; i < nw; ++i) *outs[r] << (*rows[r])[i] << (i + 1 < nw ? "," : "");
                *outs[r] << std::endl;
            }
            of[b] << time << ',';
            for (std::size_t i = 0; i < nq; ++i) of[b] << dfd[i] << (i + 1 < nq ? "," : "");
            of[b] << std::endl;
        }
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::cout << "USAGE: dist_reader <input.xml> <histogram.msgpack.bin> " << std::endl;
        return 1;
    }
    std::cout << "***********************************\n"
              << "This is dist_reader_gpu (host tool of the GB300 engine)\n"
              << "***********************************" << std::endl;
    try {
        std::cout << "Reading " << argv[1] << std::endl;
        const Input in = read_input(argv[1]);
        std::ifstream f(argv[2], std::ios::binary);
        if (!f) {
            std::cout << "ERROR:\nmsgpack file \"" << argv[2] << "\" does not exist." << std::endl;
            return 1;
        }
        std::cout << "Init data storing" << std::endl;
        Writer w(in);
        const std::size_t nbx = in.area.size();
        std::vector<bool> listed(nbx, false);
        for (int b : in.boxes) listed[std::size_t(b)] = true;
        for (std::size_t istep = 0;; ++istep) {
            std::string size;
            if (!std::getline(f, size, '#')) throw std::runtime_error("frames end without the closing 0#");
            const std::size_t len = std::size_t(std::stoull(size));
            if (len == 0) break;
            std::vector<unsigned char> buf(len);
            f.read(reinterpret_cast<char*>(buf.data()), std::streamsize(len));
            if (!f) throw std::runtime_error("truncated frame");
            std::cout << "*Read line " << istep << std::endl;
            // [time, Eeff, [T per box], per box: nelements, [mode, count, ...]]
            MsgReader r{buf.data(), buf.data() + len};
            const std::size_t top = r.array();
            if (top < 3 + 2 * nbx) throw std::runtime_error("frame has fewer boxes than the geometry");
            const double time = r.number(), Eeff = r.number();
            std::cout << "time " << time << std::endl;
            std::cout << "Eeff " << Eeff << std::endl;
            const std::size_t nt = r.array();
            if (nt < nbx) throw std::runtime_error("frame has fewer temperatures than boxes");
            std::vector<double> temps(nt);
            for (auto& t : temps) t = r.number();
            std::vector<std::vector<std::pair<std::size_t, double>>> H(nbx);
            for (std::size_t b = 0; b < nbx; ++b) {
                const std::size_t nel = std::size_t(r.number());
                const std::size_t na = r.array();
                if (listed[b]) std::cout << "nelements " << nel << std::endl;
                for (std::size_t j = 0; j < na; ++j) {
                    const double v = r.number();
                    if (listed[b] && j % 2 == 1 && j / 2 < nel / 2) H[b].back().second = v;
                    if (listed[b] && j % 2 == 0 && j / 2 < nel / 2) {
                        const std::size_t k = std::size_t(v);
                        if (k >= w.n) throw std::runtime_error("mode index beyond the mode table");
                        H[b].push_back({k, 0.});
                    }
                }
            }
            bool dump = false;
            for (double t : in.dumptimes) dump = dump || almost_equal(time, t);
            if (!dump) continue;
            w.dump(time, Eeff, temps, H);
            if (almost_equal(time, in.dumptimes.back())) break;  // the last dump time is done
        }
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 2;
    }
    return 0;
}
