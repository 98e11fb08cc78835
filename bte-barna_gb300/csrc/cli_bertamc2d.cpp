// cli_bertamc2d.cpp - bertamc2d_gpu, the drop-in for the beRTAMC2D executable.
//
//   bertamc2d_gpu <inputfile.xml> nthreads          (src/beyondRTA_MC2d.cpp:1928-1942)
//
// Reads the <beRTAMC2D> XML (src/beyondRTA_MC2d.cpp:1299-1462): geometry,
// time, material with <propagator T file> entries (*.P.eigen.bin, save_P
// format), <Eeff particles=|Ed=|Tmax Tmin>, <RTA/>; runs the step loop on the
// GPU through the C ABI; prints the per-step table "step time N (ed jx jy)
// per box" (:2418-2423) and writes properties.msgpack.bin frames
// (:1604-1769).  nthreads is accepted and ignored.  The material database is
// the engine's BTEMODE1 mode table.  Extensions: <engine seed="N"
// capacity="M"/>.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/btegpu.h"
#include "cli_io.hpp"
#include "frames.hpp"

namespace {

using namespace bte_cli;

void write_csv(const std::string& fn, const std::vector<double>& data, int nboxes, int nbins, double dt) {
    std::ofstream o(fn);
    if (!o) throw std::runtime_error("cannot write " + fn);
    for (int i = 0; i < nbins; ++i) {
        o << (i + 0.5) * dt;
        for (int b = 0; b < nboxes; ++b) o << ',' << data[std::size_t(b) * nbins + i];
        o << '\n';
    }
}

void check(bte_ctx* ctx, bte_status s, const char* what) {
    if (s != BTE_OK) {
        char buf[512];
        bte_last_error(ctx, buf, sizeof buf);
        throw std::runtime_error(std::string(what) + ": " + buf);
    }
}

}  // namespace

namespace {

std::vector<double> read_P(const std::string& path, int64_t& n) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open propagator " + path);
    f.read(reinterpret_cast<char*>(&n), sizeof n);
    if (!f || n < 1 || n > 200000) throw std::runtime_error("bad propagator header in " + path);
    std::vector<double> P(std::size_t(n) * std::size_t(n));
    f.read(reinterpret_cast<char*>(P.data()), std::streamsize(P.size() * sizeof(double)));
    if (!f) throw std::runtime_error("truncated propagator " + path);
    return P;
}

double bose(double omega, double T) {
    constexpr double prefactor = 1e12 * 1.054571726e-34 / 1.3806488e-23;
    return 1. / (std::exp(prefactor * omega / T) - 1.);
}

// calc_Eeff, src/beyondRTA_MC2d.cpp:100-128
double calc_Eeff(const ModesFile& m, double Thot, double Tcold, double Tref, double volume, double nparticles) {
    long double dE_hot = 0., dE_cold = 0.;
    const std::size_t n = m.omega.size();
    for (std::size_t k = 0; k < n; ++k) {
        const double om = m.omega[k];
        if (std::fabs(0. - om) < 1e-8 + std::fabs(1e-5 * om)) continue;
        dE_hot += 1e12 * 1.054571726e-34 * om * std::fabs(bose(om, Thot) - bose(om, Tref));
        dE_cold += 1e12 * 1.054571726e-34 * om * std::fabs(bose(om, Tcold) - bose(om, Tref));
    }
    return double(volume * (dE_cold + dE_hot) / m.head[0] / nparticles);
}

struct StepOut {
    std::ofstream frames;
    double Eeff;
    std::vector<double> temperatures;
};

void on_step(void* user, int32_t step, double time, int64_t np, const int32_t* H, int32_t nboxes,
             int32_t nmodes, const double* ed, const double* flux) {
    auto* so = static_cast<StepOut*>(user);
    std::cout << step << '\t' << time << '\t' << np << '\t';
    for (int b = 0; b < nboxes; ++b) std::cout << ed[b] << '\t' << flux[2 * b] << '\t' << flux[2 * b + 1] << '\t';
    std::cout << '\n';
    so->frames << bte::berta_frame(time, so->Eeff, so->temperatures, H, std::size_t(nboxes), std::size_t(nmodes));
}

}  // namespace

int main(int argc, char** argv) {
    std::cout << "********************************************\n"
              << "This is bertamc2d_gpu (GB300 engine, C ABI v" << bte_version() << ")\n"
              << "********************************************" << std::endl;
    if (argc != 3) {
        std::cerr << "Usage: " << argv[0] << " <inputfile.xml> nthreads" << std::endl;
        return 1;
    }
    try {
        const std::string input = argv[1];
        auto root = read_xml(input);
        if (root->name != "beRTAMC2D") throw std::runtime_error("root element must be <beRTAMC2D>");
        const std::string base = dir_of(input);
        std::string gfile, dbfile;
        std::vector<std::pair<double, std::string>> pfiles;  // <propagator T file>, one per temperature
        double dt = 0, maxtime = 0, thickness = 0, Ed = -1, Tmax = 0, Tmin = 0, particles = 0;
        bool rta = false, have_grad = false;
        double grad[2] = {0., 0.};
        unsigned long long seed = 20261203ULL;
        long long capacity = 0;
        for (auto& k : root->kids) {
            if (k->name == "geometry") gfile = k->get("file");
            if (k->name == "time") {
                dt = std::stod(k->get("dt"));
                maxtime = std::stod(k->get("maxtime"));
            }
            if (k->name == "material") {
                dbfile = k->get("database");
                thickness = std::stod(k->get("thickness"));
                for (auto& q : k->kids)
                    if (q->name == "propagator") {
                        pfiles.emplace_back(std::stod(q->get("T")), q->get("file"));
                    }
            }
            if (k->name == "Eeff") {
                if (k->has("particles")) particles = std::stod(k->get("particles"));
                if (k->has("Ed")) Ed = std::stod(k->get("Ed"));
                if (k->has("Tmax")) {
                    Tmax = std::stod(k->get("Tmax"));
                    Tmin = std::stod(k->get("Tmin"));
                }
            }
            if (k->name == "RTA") rta = true;
            // <gradient x y/>: homogeneous gradient in K/nm (:1328-1333)
            if (k->name == "gradient") {
                have_grad = true;
                grad[0] = std::stod(k->get("x"));
                grad[1] = std::stod(k->get("y"));
            }
            if (k->name == "transmission") throw std::runtime_error("This is currently not supported");
            if (k->name == "init_distribution") throw std::runtime_error("<init_distribution> is not supported");
            if (k->name == "engine") {
                if (k->has("seed")) seed = std::stoull(k->get("seed"));
                if (k->has("capacity")) capacity = std::stoll(k->get("capacity"));
            }
        }
        auto groot = read_xml(resolve(base, gfile));
        std::vector<int32_t> npts, res, tto;
        std::vector<double> verts, teq, tinit, transl;
        bool any_periodic = false;
        for (auto& b : groot->kids) {
            if (b->name != "Box") continue;
            const Node* v = b->child("Vertices");
            if (!v) throw std::runtime_error("<Box> without <Vertices>");
            const int rows = std::stoi(v->get("dim")), cols = std::stoi(v->get("npoints"));
            if (rows != 2) throw std::runtime_error("Error in provided vertices, bad dimension");
            std::stringstream ds(v->text);
            for (int i = 0; i < rows * cols; ++i) {
                double x;
                ds >> x;
                verts.push_back(x);
            }
            npts.push_back(cols);
            const Node* ic = b->child("initCnd");
            const double te = ic ? std::stod(ic->get("Teq")) : -1.;
            teq.push_back(te);
            tinit.push_back(ic && ic->has("Tinit") ? std::stod(ic->get("Tinit")) : te);
            res.push_back(b->child("Reservoir") ? 1 : 0);
            // <Translate_to id="j"> tx ty [tz] </Translate_to>, src/geometry_2d.cpp:467-475
            const Node* tr = b->child("Translate_to");
            tto.push_back(tr ? std::stoi(tr->get("id")) : -1);
            double tx = 0., ty = 0.;
            if (tr) {
                std::stringstream ts(tr->text);
                ts >> tx >> ty;
                any_periodic = true;
            }
            transl.push_back(tx);
            transl.push_back(ty);
        }
        ModesFile mf = read_modes(resolve(base, dbfile));
        // Eeff: <Eeff Ed> or the minimum of calc_Eeff over the boxes (:1995-2070)
        double T0 = -1.;
        for (std::size_t b = 0; b < teq.size(); ++b)
            if (!res[b] && tto[b] < 0) T0 = teq[b];
        double Eeff = Ed;
        if (Eeff < 0.) {
            if (!(particles > 0.)) throw std::runtime_error("<Eeff> needs particles= or Ed=");
            // periodic boxes take no part (src/beyondRTA_MC2d.cpp:2020-2066)
            double maxT = 0., minT = 1.416784e+32, meanT = 0.;
            std::size_t nT = 0;
            for (std::size_t b = 0; b < teq.size(); ++b) {
                if (tto[b] >= 0) continue;
                meanT += teq[b];
                maxT = std::max(maxT, teq[b]);
                minT = std::min(minT, teq[b]);
                ++nT;
            }
            if (Tmax != 0) {
                maxT = Tmax;
                minT = Tmin;
            }
            meanT /= double(nT);
            Eeff = 1e300;
            std::size_t off = 0;
            for (std::size_t b = 0; b < teq.size(); ++b) {
                double a2 = 0.;
                const int np = npts[b];
                for (int i = 0; i < np; ++i) {
                    const double x1 = verts[2 * (off + i)], y1 = verts[2 * (off + i) + 1];
                    const double x2 = verts[2 * (off + (i + 1) % np)], y2 = verts[2 * (off + (i + 1) % np) + 1];
                    a2 += x1 * y2 - x2 * y1;
                }
                off += std::size_t(np);
                if (res[b] || tto[b] >= 0) continue;
                const double area = std::fabs(0.5 * a2);
                const double vuc = thickness * mf.V / mf.c;
                Eeff = std::min(Eeff, calc_Eeff(mf, maxT, minT, meanT, area * thickness / vuc, particles));
            }
        }
        bte_ctx* ctx = nullptr;
        bte_device_opts opts{0, 1};
        if (bte_create(&ctx, &opts) != BTE_OK) throw std::runtime_error("bte_create failed");
        std::unique_ptr<bte_ctx, bte_status (*)(bte_ctx*)> guard(ctx, bte_destroy);
        bte_mode_table mt{};
        mt.nq = mf.head[0];
        mt.nb = mf.head[1];
        for (int i = 0; i < 3; ++i) mt.grid[i] = mf.head[2 + i];
        mt.omega = mf.omega.data();
        mt.vg = mf.vg.data();
        mt.w = mf.w.data();
        mt.dq = mf.dq;
        mt.V = mf.V;
        mt.c_lat = mf.c;
        check(ctx, bte_load_modes(ctx, &mt), "load modes");
        bte_geometry gm{};
        gm.nboxes = int32_t(npts.size());
        gm.npoints = npts.data();
        gm.vertices = verts.data();
        gm.Teq = teq.data();
        gm.Tinit = tinit.data();
        gm.reservoir = res.data();
        gm.thickness = thickness;
        if (any_periodic) {
            gm.translate_to = tto.data();
            gm.translation = transl.data();
        }
        check(ctx, bte_load_geometry(ctx, &gm), "load geometry");
        if (!rta) {
            if (pfiles.empty()) throw std::runtime_error("no <propagator> given and no <RTA/>");
            // every tabulated temperature; a run at a Teq in between
            // interpolates (lirp, src/collision_operator.cpp:918-929)
            for (auto& [Tp, file] : pfiles) {
                int64_t nP = 0;
                const std::vector<double> P = read_P(resolve(base, file), nP);
                bte_propagator pr{int32_t(nP), Tp, P.data()};
                check(ctx, bte_load_propagator(ctx, &pr), "load propagator");
            }
        }
        std::cout << "#Eeff is: " << Eeff << " J" << std::endl;
        StepOut so;
        so.frames.open("properties.msgpack.bin", std::ios::binary);
        so.Eeff = Eeff;
        so.temperatures = teq;
        bte_berta_params bp{};
        bp.dt = dt;
        bp.maxtime = maxtime;
        bp.Eeff = Eeff;
        bp.T0 = T0;
        bp.seed = seed;
        bp.mode = BTE_MODE_PRODUCTION;
        bp.rta = rta ? 1 : 0;
        bp.cancel_every = 4;
        if (have_grad) {
            bp.gradient_mode = 1;
            bp.gradient[0] = grad[0];
            bp.gradient[1] = grad[1];
        }
        bp.capacity = capacity;
        bp.on_step = on_step;
        bp.user = &so;
        bte_berta_result out{};
        auto t0 = std::chrono::high_resolution_clock::now();
        check(ctx, bte_berta_run(ctx, &bp, &out), "run");
        auto t1 = std::chrono::high_resolution_clock::now();
        so.frames << "0#";
        std::cout << "#steps " << out.nsteps << ", particle-steps " << out.particle_steps << " in "
                  << std::chrono::duration<double>(t1 - t0).count() << " s (device " << out.kernel_ms << " ms)"
                  << std::endl;
        // the reference's time report (timer::print_report, src/beyondRTA_MC2d.cpp:1883-1896)
        static const char* names[8] = {"advection", "cancelling", "generators", "histogram",
                                       "properties", "read_data", "saving", "scattering"};
        std::cout << "###################\n#TIME report:" << std::endl;
        for (int k = 0; k < 8; ++k) std::cout << " *" << names[k] << " : " << out.phase_ms[k] * 1e-3 << " s " << std::endl;
        std::cout << "###################\n";
        std::cout << "TOTAL TIME : " << std::chrono::duration<double>(t1 - t0).count() << " s " << std::endl;
        std::cout << "###################\n";
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 2;
    }
    return 0;
}
