// cli_rtamc2d.cpp - rtamc2d_gpu, the drop-in for the RTAMC2D executable.
//
//   rtamc2d_gpu <inputfile.xml> nthreads [nruns]        (src/RTA_MC2D.cpp:2085-2101)
//
// Reads the <RTA_MC2d> XML (src/RTA_MC2D.cpp:1806-2055) and the geometry XML
// (src/geometry_2d.cpp:408-522), runs the particle loop on the GPU through
// the C ABI and writes temperature_/jx_/jy_{T0}K_run_{i}.csv with rows
// [t_mid, box0, box1, ...] (src/RTA_MC2D.cpp:2437-2471).  `nthreads` is
// accepted and ignored.  The material database is the engine's binary mode
// table (magic BTEMODE1); almaBTE HDF5 files need libhdf5, which this build
// does not link.  Several <material>s (boxes name theirs in <MaterialID>)
// run as crystals joined by diffuse mismatch interfaces, all of one
// thickness.  Extensions live in an <engine .../> element:
//   mode="replay|production" seed="N" specularity="p" source="walls|initial"
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

void check(bte_ctx* ctx, bte_status s, const char* what);

// The spectral CSVs of one run (src/RTA_MC2D.cpp:2473-2541): per location,
// deltaT_omega_, jx_omega_, jy_omega_ with a first row [-1, omega ticks] and
// rows [(i + 0.5) dt, values of bin i-1] for i = 1..nbins (the reference's
// time column), and fd_q_ with two header lines of q coordinates; the
// reference's writer leaves the first data row on the third "# " line.
void write_spectral(bte_ctx* ctx, const std::vector<int32_t>& boxes, int nw, int nbins, double dt,
                    const std::string& T0s, long irun) {
    bte_spectral_result r{};
    check(ctx, bte_get_spectral(ctx, &r), "spectral outputs");
    const std::size_t nloc = boxes.size(), nq = std::size_t(r.nq);
    std::vector<double> om(nloc * nw), dT(nloc * nbins * nw), jx(dT.size()), jy(dT.size()),
        fq(nloc * nbins * nq), q(2 * nq);
    r.omega = om.data();
    r.dT_omega = dT.data();
    r.jx_omega = jx.data();
    r.jy_omega = jy.data();
    r.fd_q = fq.data();
    r.q1bz = q.data();
    check(ctx, bte_get_spectral(ctx, &r), "spectral outputs");
    for (std::size_t l = 0; l < nloc; ++l) {
        const std::string tail = std::to_string(boxes[l]) + "_" + T0s + "K_run_" + std::to_string(irun) + ".csv";
        const std::pair<const char*, const std::vector<double>*> sets[3] = {
            {"deltaT_omega_", &dT}, {"jx_omega_", &jx}, {"jy_omega_", &jy}};
        for (auto& [name, data] : sets) {
            std::ofstream o(std::string(name) + tail);
            if (!o) throw std::runtime_error(std::string("cannot write ") + name + tail);
            o << -1.0;
            for (int i = 0; i < nw; ++i) o << ',' << om[l * nw + std::size_t(i)];
            o << '\n';
            for (int i = 1; i <= nbins; ++i) {
                o << (i + 0.5) * dt;
                for (int k = 0; k < nw; ++k) o << ',' << (*data)[(l * nbins + std::size_t(i - 1)) * nw + std::size_t(k)];
                o << '\n';
            }
        }
        std::ofstream o("fd_q_" + tail);
        if (!o) throw std::runtime_error("cannot write fd_q_" + tail);
        for (int a = 0; a < 2; ++a) {
            o << "# ";
            for (std::size_t iq = 0; iq < nq; ++iq) o << (iq ? "," : "") << std::to_string(q[2 * iq + std::size_t(a)]);
            o << '\n';
        }
        o << "# ";
        for (int i = 0; i < nbins; ++i) {
            for (std::size_t iq = 0; iq < nq; ++iq)
                o << (iq ? "," : "") << fq[(l * nbins + std::size_t(i)) * nq + iq];
            o << '\n';
        }
    }
}

// The spectral CSVs of one steady run (src/RTA_MC2D.cpp:2775-2830): per
// location steady_deltaT_omega_, steady_jx_omega_, steady_jy_omega_ with
// the omega ticks on the first row and the values on the second, and
// steady_fd_q_ with the two q-coordinate header lines, the one data row
// left on the third "# " line as in the transient writer.
void write_spectral_steady(bte_ctx* ctx, const std::vector<int32_t>& boxes, int nw, const std::string& T0s,
                           long irun) {
    bte_spectral_result r{};
    check(ctx, bte_get_spectral(ctx, &r), "spectral outputs");
    const std::size_t nloc = boxes.size(), nq = std::size_t(r.nq);
    std::vector<double> om(nloc * nw), dT(nloc * nw), jx(dT.size()), jy(dT.size()), fq(nloc * nq), q(2 * nq);
    r.omega = om.data();
    r.dT_omega = dT.data();
    r.jx_omega = jx.data();
    r.jy_omega = jy.data();
    r.fd_q = fq.data();
    r.q1bz = q.data();
    check(ctx, bte_get_spectral(ctx, &r), "spectral outputs");
    std::cout << "# Writing spectral decompositions" << std::endl;
    for (std::size_t l = 0; l < nloc; ++l) {
        const std::string tail = std::to_string(boxes[l]) + "_" + T0s + "K_run_" + std::to_string(irun) + ".csv";
        auto two_rows = [&](const std::string& name, const std::vector<double>& data) {
            std::ofstream o(name + tail);
            if (!o) throw std::runtime_error("cannot write " + name + tail);
            for (int i = 0; i < nw; ++i) o << (i ? "," : "") << om[l * nw + std::size_t(i)];
            o << '\n';
            for (int i = 0; i < nw; ++i) o << (i ? "," : "") << data[l * nw + std::size_t(i)];
            o << '\n';
        };
        two_rows("steady_deltaT_omega_", dT);
        {
            std::ofstream o("steady_fd_q_" + tail);
            if (!o) throw std::runtime_error("cannot write steady_fd_q_" + tail);
            for (int a = 0; a < 2; ++a) {
                o << "# ";
                for (std::size_t iq = 0; iq < nq; ++iq)
                    o << (iq ? "," : "") << std::to_string(q[2 * iq + std::size_t(a)]);
                o << '\n';
            }
            o << "# ";
            for (std::size_t iq = 0; iq < nq; ++iq) o << (iq ? "," : "") << fq[l * nq + iq];
            o << '\n';
        }
        two_rows("steady_jx_omega_", jx);
        two_rows("steady_jy_omega_", jy);
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

int main(int argc, char** argv) {
    auto tA = std::chrono::high_resolution_clock::now();
    std::cout << "********************************************\n"
              << "This is rtamc2d_gpu (GB300 engine, C ABI v" << bte_version() << ")\n"
              << "********************************************" << std::endl;
    if (argc != 3 && argc != 4) {
        std::cerr << "Usage: " << argv[0] << " <inputfile.xml> nthreads nruns" << std::endl;
        return 1;
    }
    const long nruns = argc == 4 ? std::atol(argv[3]) : 1;
    try {
        const std::string input = argv[1];
        auto root = read_xml(input);
        if (root->name != "RTA_MC2d") throw std::runtime_error("root element must be <RTA_MC2d>");
        const std::string base = dir_of(input);
        std::string gfile, dbfile;
        double dt = 0, maxtime = 0, thickness = 0, T0 = -1, p = 0;
        // every <material name database thickness T0> (src/RTA_MC2D.cpp:1886-1923)
        std::vector<std::string> mnames, mfiles;
        std::vector<double> mthick;
        long long N = 0;
        double grad[2] = {0., 0.}, eps_energy = -42.0, eps_flux = -42.0;
        std::vector<int32_t> spec_boxes;
        int spec_ticks = 0;
        unsigned long long seed = 20261203ULL;
        int mode = BTE_MODE_PRODUCTION, source = BTE_SOURCE_WALLS, ballistic = 0;
        for (auto& k : root->kids) {
            if (k->name == "geometry") gfile = k->get("file");
            if (k->name == "time") {
                dt = std::stod(k->get("dt"));
                maxtime = std::stod(k->get("maxtime"));
            }
            if (k->name == "material") {
                dbfile = k->get("database");
                thickness = std::stod(k->get("thickness"));
                T0 = std::stod(k->get("T0"));
                mnames.push_back(k->has("name") ? k->get("name") : "");
                mfiles.push_back(dbfile);
                mthick.push_back(thickness);
            }
            if (k->name == "particles") N = std::stoll(k->get("N"));
            if (k->name == "ballistic") ballistic = 1;
            // <gradient x= y=/> and <convergence energy= flux=/>, src/RTA_MC2D.cpp:1828-1840
            if (k->name == "gradient") {
                grad[0] = std::stod(k->get("x"));
                grad[1] = std::stod(k->get("y"));
            }
            // <spectral><resolution ticks=/><location bin=/>...</spectral>
            if (k->name == "spectral") {
                for (auto& sk : k->kids) {
                    if (sk->name == "resolution") spec_ticks = std::stoi(sk->get("ticks"));
                    if (sk->name == "location") spec_boxes.push_back(std::stoi(sk->get("bin")));
                }
            }
            if (k->name == "convergence") {
                eps_energy = std::stod(k->get("energy"));
                eps_flux = std::stod(k->get("flux"));
            }
            if (k->name == "layer" || k->name == "layers_connection")
                throw std::runtime_error("multi-material layers are not supported");
            if (k->name == "engine") {
                if (k->has("mode")) mode = k->get("mode") == "replay" ? BTE_MODE_REPLAY : BTE_MODE_PRODUCTION;
                if (k->has("seed")) seed = std::stoull(k->get("seed"));
                if (k->has("specularity")) p = std::stod(k->get("specularity"));
                if (k->has("source")) source = k->get("source") == "initial" ? BTE_SOURCE_INITIAL : BTE_SOURCE_WALLS;
            }
        }
        // geometry
        auto groot = read_xml(resolve(base, gfile));
        std::vector<int32_t> npts, res, tto, bmat;
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
            double te = ic ? std::stod(ic->get("Teq")) : -1.;
            teq.push_back(te);
            tinit.push_back(ic && ic->has("Tinit") ? std::stod(ic->get("Tinit")) : te);
            res.push_back(b->child("Reservoir") ? 1 : 0);
            // <MaterialID name=...>: the box's crystal among the <material>s
            const Node* mid = b->child("MaterialID");
            int mk = 0;
            if (mid && mnames.size() > 1) {
                mk = -1;
                for (std::size_t i = 0; i < mnames.size(); ++i)
                    if (mnames[i] == mid->get("name")) mk = int(i);
                if (mk < 0) throw std::runtime_error("box material " + mid->get("name") + " is not a <material>");
            }
            bmat.push_back(mk);
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
        bte_ctx* ctx = nullptr;
        bte_device_opts opts{0, 1};
        if (bte_create(&ctx, &opts) != BTE_OK) {
            char buf[256];
            bte_last_error(nullptr, buf, sizeof buf);
            throw std::runtime_error(std::string("bte_create: ") + buf);
        }
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
        // several crystals: one mode table per <material>, diffuse mismatch
        // at their contacts
        std::vector<ModesFile> mfs;
        std::vector<bte_mode_table> mts;
        if (mnames.size() > 1) {
            for (auto& f : mfiles) mfs.push_back(read_modes(resolve(base, f)));
            for (auto& x : mfs) {
                bte_mode_table t{};
                t.nq = x.head[0];
                t.nb = x.head[1];
                for (int i = 0; i < 3; ++i) t.grid[i] = x.head[2 + i];
                t.omega = x.omega.data();
                t.vg = x.vg.data();
                t.w = x.w.data();
                t.dq = x.dq;
                t.V = x.V;
                t.c_lat = x.c;
                mts.push_back(t);
            }
            // each crystal's boxes take its <material thickness> (thicknesses[box])
            check(ctx, bte_load_mode_tables(ctx, int32_t(mts.size()), mts.data(), mthick.data()), "load mode tables");
        } else {
            check(ctx, bte_load_modes(ctx, &mt), "load modes");
        }
        bte_geometry gm{};
        gm.nboxes = int32_t(npts.size());
        gm.npoints = npts.data();
        gm.vertices = verts.data();
        gm.Teq = teq.data();
        gm.Tinit = tinit.data();
        gm.reservoir = res.data();
        gm.thickness = thickness;
        if (mnames.size() > 1) gm.material = bmat.data();
        if (any_periodic) {
            gm.translate_to = tto.data();
            gm.translation = transl.data();
        }
        check(ctx, bte_load_geometry(ctx, &gm), "load geometry");
        if (!spec_boxes.empty()) {
            if (spec_ticks < 1) throw std::runtime_error("<spectral> needs <resolution ticks>");
            check(ctx, bte_set_spectral(ctx, int32_t(spec_boxes.size()), spec_boxes.data(), spec_ticks),
                  "spectral locations");
        }
        auto tB = std::chrono::high_resolution_clock::now();
        std::cout << "#Init variables -> Done (" << std::chrono::duration<double>(tB - tA).count() << " s )\n";
        const double gnorm = std::sqrt(grad[0] * grad[0] + grad[1] * grad[1]);
        if (!(std::fabs(gnorm) < 1e-8)) {
            // periodic structure under a gradient: steady state only, :2544-2842
            std::cout << "PERIODIC CASE: [only steady state is simulated]\n";
            if (eps_energy > 0.) std::cout << "#energy convergence " << eps_energy << std::endl;
            if (eps_flux > 0.) std::cout << "#flux convergence " << eps_flux << std::endl;
            const int nbx = int(npts.size());
            for (long irun = 0; irun < nruns; ++irun) {
                bte_steady_params sp{};
                sp.T0 = T0;
                sp.gradient[0] = grad[0];
                sp.gradient[1] = grad[1];
                sp.eps_energy = eps_energy;
                sp.eps_flux = eps_flux;
                sp.nparticles = N;
                sp.seed = seed + (unsigned long long)irun;
                sp.mode = mode;
                std::vector<double> T(static_cast<std::size_t>(nbx)), jx(T.size()), jy(T.size());
                std::vector<double> log(static_cast<std::size_t>(4) * 100000);
                bte_steady_result out{};
                out.temperature = T.data();
                out.jx = jx.data();
                out.jy = jy.data();
                out.log = log.data();
                out.log_cap = 100000;
                std::cout << "#Run: " << irun << std::endl;
                auto t0 = std::chrono::high_resolution_clock::now();
                check(ctx, bte_steady_run(ctx, &sp, &out), "steady run");
                auto t1 = std::chrono::high_resolution_clock::now();
                for (int gi = 0; gi < out.generations && gi < out.log_cap; ++gi) {
                    const double* r = &log[std::size_t(gi) * 4];
                    std::cout << gi + 1 << '\t' << (long long)r[0] << '\t' << r[1];
                    if (std::fabs(grad[0]) < 1e-8 || std::fabs(grad[1]) < 1e-8)
                        std::cout << '\t' << (std::fabs(grad[0]) < 1e-8 ? r[3] : r[2]) << '\n';
                    else
                        std::cout << '\t' << r[2] << '\t' << r[3] << '\n';
                }
                std::cout << "#|E| =" << out.energy_rate << " J/ps\n#Eeff = " << out.Eeff << "\n"
                          << "#MC loop -> Done ( " << std::chrono::duration<double>(t1 - t0).count()
                          << " s ), " << out.generations << " generations, " << out.events
                          << " flight events" << std::endl;
                std::cout << "# Writing steady state" << std::endl;
                const std::string fn = "steady_" + fmt_g(T0) + "K_run_" + std::to_string(irun) + ".csv";
                std::ofstream o(fn);
                if (!o) throw std::runtime_error("cannot write " + fn);
                const std::vector<double>* rows[3] = {&T, &jx, &jy};
                for (auto* row : rows) {
                    for (int b = 0; b < nbx; ++b) o << (b ? "," : "") << (*row)[std::size_t(b)];
                    o << '\n';
                }
                if (!spec_boxes.empty()) write_spectral_steady(ctx, spec_boxes, spec_ticks, fmt_g(T0), irun);
            }
            return 0;
        }
        for (long irun = 0; irun < nruns; ++irun) {
            bte_rta_params rp{};
            rp.T0 = T0;
            rp.dt = dt;
            rp.maxtime = maxtime;
            rp.nparticles = N;
            rp.seed = seed + (unsigned long long)irun;
            rp.mode = mode;
            rp.source = source;
            rp.ballistic = ballistic;
            rp.specularity = p;
            int32_t nbx = 0, nbn = 0;
            int64_t nm = 0;
            bte_query_sizes(ctx, &rp, &nbx, &nbn, &nm);
            std::vector<double> T(std::size_t(nbx) * nbn), jx(T.size()), jy(T.size());
            bte_rta_result out{};
            out.temperature = T.data();
            out.jx = jx.data();
            out.jy = jy.data();
            std::cout << "#Run: " << irun << std::endl;
            auto t0 = std::chrono::high_resolution_clock::now();
            check(ctx, bte_rta_run(ctx, &rp, &out), "run");
            auto t1 = std::chrono::high_resolution_clock::now();
            std::cout << "#|E| =" << out.energy_rate << " J/ps\n#Eeff = " << out.Eeff << "\n"
                      << "#MC loop -> Done ( " << std::chrono::duration<double>(t1 - t0).count()
                      << " s ), kernel " << out.kernel_ms << " ms, " << out.events << " flight events ("
                      << double(out.events) / (out.kernel_ms * 1e-3) << " /s)" << std::endl;
            const std::string tag = fmt_g(T0) + "K_run_" + std::to_string(irun) + ".csv";
            write_csv("temperature_" + tag, T, nbx, nbn, dt);
            write_csv("jx_" + tag, jx, nbx, nbn, dt);
            write_csv("jy_" + tag, jy, nbx, nbn, dt);
            if (!spec_boxes.empty()) write_spectral(ctx, spec_boxes, spec_ticks, nbn, dt, fmt_g(T0), irun);
        }
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 2;
    }
    return 0;
}
