// steady.cu - the periodic / gradient steady state of RTAMC2D
// (src/RTA_MC2D.cpp:2544-2842): the host loop over generations.
//
// Per generation: one kernel flies every slot once (rta_steady.cuh), a
// three-pass exclusive scan of the reflection flags compacts the reflected
// particles, in slot order, into the next generation's input, and the host
// reads phi and the cumulative tallies (3 values per box) to build the next
// births and test convergence.  Generation 0 first scans the slots that
// pick a gradient generator, which fixes the alternating sign of the
// gradient particles in slot order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ctx.hpp"
#include "rta_steady.cuh"

namespace bte {

struct SteadyState {
    DBuf walls, wcum, gcdf, gprob, galt;          // wall generators
    DBuf sbox, scum, scdf, sprob, salt, ssign;    // gradient generators
    DBuf pin, ptmp, flag, pos, sums, rank, phi;   // particles and scan scratch
    DBuf bfirst, bbox, bsign;                     // births
    DBuf tally, counters, err, work;
};

namespace {

constexpr int SCAN_B = 1024;

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned& total) {
    __shared__ unsigned ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned t = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    const unsigned pre = (warp > 0 ? ws[warp - 1] : 0u) + x - v;
    total = ws[31];
    __syncthreads();
    return pre;
}

__global__ void __launch_bounds__(SCAN_B) scan_blocks(const unsigned* in, unsigned* out, unsigned* sums,
                                                      long long n) {
    const long long i = (long long)blockIdx.x * SCAN_B + threadIdx.x;
    const unsigned v = i < n ? in[i] : 0u;
    unsigned total;
    const unsigned pre = block_exclusive_scan(v, total);
    if (i < n) out[i] = pre;
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_B) scan_sums(unsigned* sums, long long nb, unsigned* grand) {
    unsigned carry = 0;
    for (long long base = 0; base < nb; base += SCAN_B) {
        const long long i = base + threadIdx.x;
        const unsigned v = i < nb ? sums[i] : 0u;
        unsigned total;
        const unsigned pre = block_exclusive_scan(v, total);
        if (i < nb) sums[i] = carry + pre;
        carry += total;
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void scan_add(unsigned* out, const unsigned* sums, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / SCAN_B];
}

__global__ void compact(const SteadyP* src, const unsigned* flag, const unsigned* pos, SteadyP* dst,
                        long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) dst[pos[i]] = src[i];
}

// Exclusive scan of n flags into pos; returns the total (synchronises).
unsigned long long scan_flags(SteadyState& S, const unsigned* flag, unsigned* pos, long long n,
                              cudaStream_t s) {
    const long long nb = (n + SCAN_B - 1) / SCAN_B;
    unsigned* sums = S.sums.as<unsigned>();
    scan_blocks<<<unsigned(nb), SCAN_B, 0, s>>>(flag, pos, sums, n);
    scan_sums<<<1, SCAN_B, 0, s>>>(sums, nb, sums + nb);
    scan_add<<<unsigned((n + 255) / 256), 256, 0, s>>>(pos, sums, n);
    ck(cudaGetLastError(), "scan launch");
    unsigned tot = 0;
    ck(cudaMemcpyAsync(&tot, sums + nb, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "d2h");
    ck(cudaStreamSynchronize(s), "scan");
    return tot;
}

double norm_of(const std::vector<double>& a) {
    double s = 0.;
    for (double x : a) s += x * x;
    return std::sqrt(s);
}

double rel_change(const std::vector<double>& old, const std::vector<double>& cur) {
    std::vector<double> d(cur.size());
    for (std::size_t i = 0; i < cur.size(); ++i) d[i] = old[i] - cur[i];
    return norm_of(d) / norm_of(cur);
}

}  // namespace

void destroy_steady(bte_ctx* c) {
    delete c->steady;
    c->steady = nullptr;
}

}  // namespace bte

using bte::Error;

bte_status bte_steady_run(bte_ctx* c, const bte_steady_params* p, bte_steady_result* out) {
    if (!c || !p || !out) return BTE_ERR_INPUT;
    try {
        using namespace bte;
        if (!c->have_modes || !c->have_geom)
            throw Error(BTE_ERR_STATE, "load the mode table and the geometry before running");
        const bool crystals = c->ncrys > 0;
        if (c->nmat > 0 && !crystals) throw Error(BTE_ERR_INPUT, "materials are for transient batched runs");
        if (!(p->T0 > 0.) || !std::isfinite(p->T0)) throw Error(BTE_ERR_INPUT, "T0 must be > 0");
        if (p->nparticles < 1 || p->nparticles > 0x7fffffffll)
            throw Error(BTE_ERR_INPUT, "nparticles must be in [1, 2^31)");
        if (p->mode != BTE_MODE_REPLAY && p->mode != BTE_MODE_PRODUCTION)
            throw Error(BTE_ERR_INPUT, "unknown mode");
        const double gx = p->gradient[0], gy = p->gradient[1];
        if (!std::isfinite(gx) || !std::isfinite(gy) || almost_equal(std::sqrt(gx * gx + gy * gy), 0.))
            throw Error(BTE_ERR_INPUT, "the steady state needs a non-zero temperature gradient");
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        const HostModes& m = c->modes;
        const HostGeometry& g = c->geom;
        for (std::size_t b = 0; b < g.boxes.size(); ++b)
            if (!g.reservoir[b] && !almost_equal(g.Teq[b], p->T0) && g.Teq[b] != p->T0)
                throw Error(BTE_ERR_INPUT, "Tref in xml is different from provided T0");
        if (!(p->specularity >= 0. && p->specularity <= 1.))
            throw Error(BTE_ERR_INPUT, "specularity must be in [0, 1]");
        if (crystals) {
            // crystals joined by mismatch interfaces, every crystal at T0
            if (c->mat_T0.empty() || c->mat_T0[0] != p->T0) {
                c->mat_T0.assign(std::size_t(c->ncrys), p->T0);
                c->resample_T0 = -1;
            }
        }
        ensure_static(c);
        if (p->specularity > 0. && !c->have_mirror)
            throw Error(BTE_ERR_INPUT, "specular walls need an axis-aligned q grid with mirror images");
        ensure_resample(c, p->T0);
        if (!c->steady) c->steady = new SteadyState();
        SteadyState& S = *c->steady;
        const int n = int(m.n());
        const int nbx = int(g.boxes.size());
        const long long N = p->nparticles;
        const bool replay = p->mode == BTE_MODE_REPLAY;
        cudaStream_t st = c->stream;

        // generators (Init_generator with a gradient, src/RTA_MC2D.cpp:289-447)
        Generators W;
        GradGenerators G;
        if (crystals) {
            // each crystal's sources over its own boxes, rows over the
            // concatenated modes (Init_generator takes each box's material)
            std::vector<Generators> Ws;
            std::vector<GradGenerators> Gs;
            const std::vector<V2> grad(g.boxes.size(), v2(gx, gy));
            for (int k = 0; k < c->ncrys; ++k) {
                const GenEmbed e{k, c->crys_off[std::size_t(k)], m.n(), crystal_thickness(c, k)};
                Ws.push_back(build_wall_generators(c->crys[std::size_t(k)], g, false, &e));
                Gs.push_back(build_gradient_generators_boxes(c->crys[std::size_t(k)], g, grad, &e));
            }
            W = merge_generators(Ws, true, false);
            G = merge_gradient_generators(Gs);
        } else {
            W = build_wall_generators(m, g, false);
            G = build_gradient_generators(m, g, gx, gy);
        }
        double E0 = 0.;
        for (auto& w : W.walls) E0 += w.energy;
        const double E1 = G.total_energy;
        const double total = E0 + E1;
        if (!(total > 0.)) throw Error(BTE_ERR_INPUT, "the generators inject no energy");
        const double exg0 = E0 / total;
        const double exg1 = E1 / total + exg0;
        const double Eeff = total / double(N);
        {
            std::vector<WallGenDev> wd;
            for (auto& w : W.walls) {
                WallGenDev d{};
                d.p1 = w.p1;
                d.nd = w.nd;
                d.sa = w.sa;
                d.sb = w.sb;
                d.box = w.box;
                d.sign = w.sign;
                wd.push_back(d);
            }
            S.walls.upload(wd, st);
            S.wcum.upload(W.wall_cum, st);
            S.gcdf.upload(W.cdf, st);
            std::vector<float> pr(W.alias.size());
            std::vector<int> al(W.alias.size());
            for (std::size_t i = 0; i < W.alias.size(); ++i) {
                pr[i] = W.alias[i].prob;
                al[i] = W.alias[i].alt;
            }
            S.gprob.upload(pr, st);
            S.galt.upload(al, st);
            S.sbox.upload(G.box, st);
            S.scum.upload(G.cum, st);
            S.scdf.upload(G.cdf, st);
            std::vector<float> gp(G.alias.size());
            std::vector<int> ga(G.alias.size());
            for (std::size_t i = 0; i < G.alias.size(); ++i) {
                gp[i] = G.alias[i].prob;
                ga[i] = G.alias[i].alt;
            }
            S.sprob.upload(gp, st);
            S.salt.upload(ga, st);
            S.ssign.upload(G.sign, st);
        }
        // buffers
        S.pin.alloc(size_t(N) * sizeof(SteadyP));
        S.ptmp.alloc(size_t(N) * sizeof(SteadyP));
        S.flag.alloc(size_t(N) * sizeof(unsigned));
        S.pos.alloc(size_t(N) * sizeof(unsigned));
        S.rank.alloc(size_t(N) * sizeof(unsigned));
        S.sums.alloc(size_t((N + SCAN_B - 1) / SCAN_B + 1) * sizeof(unsigned));
        S.phi.alloc(size_t(nbx) * sizeof(unsigned long long));
        const size_t tally_bytes = replay ? size_t(nbx) * 6 * sizeof(unsigned long long)
                                          : size_t(nbx) * 3 * sizeof(double);
        S.tally.alloc(tally_bytes);
        S.counters.alloc(16 * sizeof(unsigned long long));
        S.err.alloc(4 * sizeof(int));
        ck(cudaMemsetAsync(S.tally.p, 0, tally_bytes, st), "memset");
        ck(cudaMemsetAsync(S.counters.p, 0, 16 * sizeof(unsigned long long), st), "memset");
        ck(cudaMemsetAsync(S.err.p, 0, 4 * sizeof(int), st), "memset");

        DevTables T{};
        fill_static_tables(c, T);
        T.source = 0;
        T.ngen = int(W.walls.size());
        T.walls = S.walls.as<WallGenDev>();
        T.wall_cum = S.wcum.as<double>();
        T.gen_cdf = S.gcdf.as<double>();
        T.gen_prob = S.gprob.as<float>();
        T.gen_alt = S.galt.as<int>();
        T.seed = p->seed;
        T.flight_cap = EVENT_CAP;
        T.nbins = 1;
        T.specularity = p->specularity;
        // spectral decomposition at the selected boxes: per-mode time and
        // signed segment counts, summed over every generation
        const size_t nloc = c->spec_boxes.size();
        const size_t spec_vals = nloc * size_t(n);
        c->spec_valid = false;
        if (nloc > 0) {
            std::vector<int> loc(size_t(nbx), -1);
            for (size_t i = 0; i < nloc; ++i) loc[size_t(c->spec_boxes[i])] = int(i);
            c->d_specloc.upload(loc, st);
            const size_t bytes = spec_vals * (replay ? 2 * sizeof(unsigned long long) : sizeof(double));
            c->d_spec.alloc(bytes);
            c->d_speccnt.alloc(spec_vals * sizeof(unsigned long long));
            ck(cudaMemsetAsync(c->d_spec.p, 0, bytes, st), "memset");
            ck(cudaMemsetAsync(c->d_speccnt.p, 0, spec_vals * sizeof(unsigned long long), st), "memset");
            T.spec_loc = c->d_specloc.as<int>();
            T.spec = c->d_spec.as<double>();
            T.spec_ex = c->d_spec.as<unsigned long long>();
            T.spec_cnt = c->d_speccnt.as<unsigned long long>();
        }

        SteadyArgs A{};
        A.exg0 = exg0;
        A.exg1 = exg1;
        A.nwall = int(W.walls.size());
        A.ngrad = int(G.box.size());
        A.grad_box = S.sbox.as<int>();
        A.grad_cum = S.scum.as<double>();
        A.grad_cdf = S.scdf.as<double>();
        A.grad_prob = S.sprob.as<float>();
        A.grad_alt = S.salt.as<int>();
        A.grad_sign = S.ssign.as<signed char>();
        A.grad_rank = S.rank.as<unsigned>();
        A.in = S.pin.as<SteadyP>();
        A.out = S.ptmp.as<SteadyP>();
        A.flag = S.flag.as<unsigned>();
        A.phi = S.phi.as<unsigned long long>();
        S.work.alloc(sizeof(unsigned long long));
        A.work = S.work.as<unsigned long long>();

        const PolyArgs PA{c->d_pborders.as<PolyBorder>(), c->d_ppieces.as<PolyPiece>(), c->d_mv.as<ModeVel>(),
                          nullptr, nullptr,
                          crystals ? c->d_dmm_row.as<long long>() : nullptr,
                          crystals ? c->d_dmm_ent.as<DmmEnt>() : nullptr};
        const int max_gen = p->max_generations > 0 ? p->max_generations : 100000;
        std::vector<double> oldv(size_t(3) * nbx, 0.), cur(size_t(3) * nbx, 0.);
        std::vector<unsigned long long> hex, hphi(static_cast<size_t>(nbx));
        std::vector<double> htal;
        std::vector<long long> bfirst;
        std::vector<int> bbox, bsign;
        long long nin = 0, nbirth = 0, births_total = 0;
        int gen = 0, converged = 0;
        float kms = 0.f;
        for (;;) {
            A.gen = gen;
            A.n = gen == 0 ? N : nin + nbirth;
            A.nin = gen == 0 ? 0 : nin;
            if (gen == 0) {
                if (replay)
                    launch_steady_replay(T, A, nullptr, nullptr, nullptr, A.flag, c->nsm, st);
                else
                    launch_steady_prod(T, A, nullptr, nullptr, nullptr, A.flag, c->nsm, st);
                ck(cudaGetLastError(), "select launch");
                scan_flags(S, A.flag, S.rank.as<unsigned>(), A.n, st);
            }
            ck(cudaMemsetAsync(S.phi.p, 0, size_t(nbx) * sizeof(unsigned long long), st), "memset");
            ck(cudaEventRecord(c->ev0, st), "cudaEventRecord");
            if (replay)
                launch_steady_replay(T, A, S.tally.as<unsigned long long>(), S.counters.as<unsigned long long>(),
                                     S.err.as<int>(), nullptr, c->nsm, st);
            else if (p->flags & BTE_FLAG_GENERAL)
                launch_steady_prod(T, A, S.tally.as<double>(), S.counters.as<unsigned long long>(),
                                   S.err.as<int>(), nullptr, c->nsm, st);
            else if (!launch_steady_poly(T, A, PA, S.tally.as<double>(), S.counters.as<unsigned long long>(),
                                         S.err.as<int>(), c->nsm, st))
                throw Error(BTE_ERR_CUDA, "steady polygon kernel does not fit on the device");
            ck(cudaGetLastError(), "steady launch");
            ck(cudaEventRecord(c->ev1, st), "cudaEventRecord");
            int herr[4];
            ck(cudaMemcpyAsync(herr, S.err.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, st), "d2h");
            ck(cudaStreamSynchronize(st), "steady generation");
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
            kms += ms;
            if (herr[0] != 0) {
                const long long slot = (long long)herr[1] | ((long long)herr[2] << 31);
                char msg[160];
                std::snprintf(msg, sizeof msg, "generation %d, slot %lld: %s", gen, slot,
                              herr[0] == BTE_ERR_VALUE ? "invalid scattering rate"
                              : herr[0] == BTE_ERR_LIMIT ? "iteration cap reached"
                                                          : "geometry error");
                throw Error(bte_status(herr[0]), msg);
            }
            // reflected particles, in slot order, become the next input
            const unsigned long long nref = scan_flags(S, A.flag, S.pos.as<unsigned>(), A.n, st);
            compact<<<unsigned((A.n + 255) / 256), 256, 0, st>>>(A.out, A.flag, S.pos.as<unsigned>(),
                                                                 S.pin.as<SteadyP>(), A.n);
            ck(cudaGetLastError(), "compact launch");
            // phi and the cumulative tallies
            ck(cudaMemcpyAsync(hphi.data(), S.phi.p, size_t(nbx) * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st), "d2h");
            if (replay) {
                hex.resize(size_t(nbx) * 6);
                ck(cudaMemcpyAsync(hex.data(), S.tally.p, tally_bytes, cudaMemcpyDeviceToHost, st), "d2h");
            } else {
                htal.resize(size_t(nbx) * 3);
                ck(cudaMemcpyAsync(htal.data(), S.tally.p, tally_bytes, cudaMemcpyDeviceToHost, st), "d2h");
            }
            ck(cudaStreamSynchronize(st), "steady readback");
            for (int b = 0; b < nbx; ++b)
                for (int q = 0; q < 3; ++q) {
                    double v;
                    if (replay) {
                        const unsigned long long hi = hex[6 * b + 2 * q], lo = hex[6 * b + 2 * q + 1];
                        v = double((__int128)(((unsigned __int128)hi << 64) | lo)) / FIX_SCALE;
                    } else {
                        v = htal[3 * b + q];
                    }
                    cur[size_t(q) * nbx + b] = v;
                }
            // births from phi, src/RTA_MC2D.cpp:2640-2658 (ascending box order)
            bfirst.clear();
            bbox.clear();
            bsign.clear();
            nbirth = 0;
            for (int b = 0; b < nbx; ++b) {
                const long long v = (long long)hphi[size_t(b)];
                if (v == 0) continue;
                bfirst.push_back(nbirth);
                bbox.push_back(b);
                bsign.push_back(v >= 0 ? 1 : -1);
                nbirth += v >= 0 ? v : -v;
            }
            bfirst.push_back(nbirth);
            births_total += nbirth;
            nin = (long long)nref;
            if (nin + nbirth > N) throw Error(BTE_ERR_LIMIT, "generation larger than the particle buffers");
            S.bfirst.upload(bfirst, st);
            S.bbox.upload(bbox, st);
            S.bsign.upload(bsign, st);
            A.nbirth = int(bbox.size());
            A.birth_first = S.bfirst.as<long long>();
            A.birth_box = S.bbox.as<int>();
            A.birth_sign = S.bsign.as<int>();
            // convergence, src/RTA_MC2D.cpp:2661-2694
            auto slice = [&](const std::vector<double>& v, int q) {
                return std::vector<double>(v.begin() + size_t(q) * nbx, v.begin() + size_t(q + 1) * nbx);
            };
            const double rgz = rel_change(slice(oldv, 0), slice(cur, 0));
            const double rjx = rel_change(slice(oldv, 1), slice(cur, 1));
            const double rjy = rel_change(slice(oldv, 2), slice(cur, 2));
            if (almost_equal(gx, 0.))
                converged = rgz < p->eps_energy && rjy < p->eps_flux;
            else if (almost_equal(gy, 0.))
                converged = rgz < p->eps_energy && rjx < p->eps_flux;
            else
                converged = rgz < p->eps_energy && rjx < p->eps_flux && rjy < p->eps_flux;
            if (out->log && gen < out->log_cap) {
                double* row = out->log + size_t(gen) * 4;
                row[0] = double(nin + nbirth);
                row[1] = rgz;
                row[2] = rjx;
                row[3] = rjy;
            }
            oldv = cur;
            gen++;
            if (nin + nbirth == 0 || converged || gen >= max_gen) break;
        }
        std::vector<unsigned long long> hc(16);
        ck(cudaMemcpyAsync(hc.data(), S.counters.p, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           st), "d2h");
        std::vector<unsigned long long> hspec, hcnt;
        if (nloc > 0) {
            hspec.resize(replay ? 2 * spec_vals : spec_vals);
            hcnt.resize(spec_vals);
            ck(cudaMemcpyAsync(hspec.data(), c->d_spec.p, hspec.size() * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st), "d2h");
            ck(cudaMemcpyAsync(hcnt.data(), c->d_speccnt.p, spec_vals * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st), "d2h");
        }
        ck(cudaStreamSynchronize(st), "counters");
        if (nloc > 0) {
            c->spec_raw.resize(spec_vals);
            c->spec_cnt.resize(spec_vals);
            for (size_t i = 0; i < spec_vals; ++i) {
                if (replay) {
                    const __int128 v = (__int128)(((unsigned __int128)hspec[2 * i] << 64) | hspec[2 * i + 1]);
                    c->spec_raw[i] = double(v) / FIX_SCALE;
                } else {
                    std::memcpy(&c->spec_raw[i], &hspec[i], sizeof(double));
                }
                c->spec_cnt[i] = (long long)hcnt[i];
            }
            c->spec_nbins = 1;
            c->spec_T0 = p->T0;
            c->spec_Eeff = Eeff;
            c->spec_steady = true;
            c->spec_valid = true;
        }
        out->nboxes = nbx;
        out->generations = gen;
        out->converged = converged;
        out->Eeff = Eeff;
        out->energy_rate = total;
        out->events = (int64_t)hc[0];
        out->wall_hits = (int64_t)hc[1];
        out->crossings = (int64_t)hc[2];
        out->absorbed = (int64_t)hc[3];
        out->translations = (int64_t)hc[8];
        out->scattered = (int64_t)hc[9];
        out->lost = (int64_t)hc[10];
        out->births = births_total;
        out->kernel_ms = kms;
        out->interface_hits = (int64_t)hc[11];
        out->interface_transmissions = (int64_t)hc[12];
        if (out->exact && replay) std::memcpy(out->exact, hex.data(), size_t(nbx) * 6 * sizeof(long long));
        // post-processing, src/RTA_MC2D.cpp:2698-2731: C_v and vcorr of each
        // box's crystal
        std::vector<double> cvs, vcorrs;
        if (crystals) {
            for (int k = 0; k < c->ncrys; ++k) {
                cvs.push_back(calc_cv(c->crys[std::size_t(k)], p->T0));
                vcorrs.push_back(crystal_thickness(c, k) / c->crys[std::size_t(k)].c);
            }
        } else {
            cvs.push_back(calc_cv(m, p->T0));
            vcorrs.push_back(g.thickness / m.c);
        }
        for (int b = 0; b < nbx; ++b) {
            const std::size_t mk = crystals ? std::size_t(g.mat[std::size_t(b)]) : 0;
            const double cv = cvs[mk], vcorr = vcorrs[mk];
            const double vbox = g.boxes[size_t(b)].area * box_thickness(c, b);
            const double z = cur[size_t(b)], zx = cur[size_t(nbx) + b], zy = cur[size_t(2) * nbx + b];
            if (out->gz) out->gz[b] = z;
            if (out->gz_jx) out->gz_jx[b] = zx;
            if (out->gz_jy) out->gz_jy[b] = zy;
            const double ed = z / vbox * Eeff;
            if (out->temperature) out->temperature[b] = ed / (cv / vcorr) + p->T0;
            if (out->jx) out->jx[b] = zx / vbox * (Eeff * 1e12 * 1e9 * 1e9);
            if (out->jy) out->jy[b] = zy / vbox * (Eeff * 1e12 * 1e9 * 1e9);
        }
        return BTE_OK;
    } catch (const Error& e) {
        c->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_CUDA;
    }
}
