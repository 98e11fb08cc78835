// adjoint.cu - gradients of a linear functional of the RTA tallies with
// respect to the mode lifetimes and the wall specularity (bte_rta_adjoint).
//
// Two launches of the grid kernel over the same particles (the same Philox
// counters): pass 1 stores each particle's contribution Phi_p; pass 2
// replays every trajectory and weights the score of each random draw by the
// particle's contribution after it (rta_prod.cu, ADJ = 2).  The
// post-scattering score has a part on every tau_i, p_i / tau_i times the sum
// of those weights, added here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.hpp"

using bte::Error;

bte_status bte_rta_adjoint(bte_ctx* c, const bte_rta_params* p, const double* weights,
                           bte_adjoint_result* out) {
    if (!c || !p || !weights || !out || !out->dphi_dtau) return BTE_ERR_INPUT;
    try {
        using namespace bte;
        if (p->mode != BTE_MODE_PRODUCTION) throw Error(BTE_ERR_INPUT, "the adjoint runs in production mode");
        if (c->nmat > 0) throw Error(BTE_ERR_INPUT, "the adjoint runs with one material");
        prepare_run(c, p);
        if (!c->geom.rect_grid)
            throw Error(BTE_ERR_INPUT, "the adjoint needs boxes that tile an axis-aligned grid");
        PreparedRun r;
        std::string why;
        const bte_status st = prepared_grid_run(c, p, &r, &why);
        if (st != BTE_OK) throw Error(st, why);
        // time grid, src/RTA_MC2D.cpp:2118-2124
        c->d_time.upload(time_grid_with_widths(r.ntime, r.maxtime, r.step), c->stream);
        r.T.timegrid = c->d_time.as<double>();
        const std::size_t nk = std::size_t(r.nboxes) * std::size_t(r.nbins);
        const std::size_t n = c->modes.n();
        const long long np = r.T.pend - r.T.pbegin;
        DBuf dW, dphi, dg, ds, dtal, dcnt, derr, dwork;
        std::vector<double> W(weights, weights + nk * 3);
        dW.upload(W, c->stream);
        dphi.alloc(size_t(np > 0 ? np : 1) * sizeof(double));
        dg.alloc(n * sizeof(double));
        ds.alloc(4 * sizeof(double));
        dtal.alloc(nk * 3 * sizeof(double));
        dcnt.alloc(16 * sizeof(unsigned long long));
        derr.alloc(4 * sizeof(int));
        dwork.alloc(sizeof(unsigned long long));
        cudaStream_t s = c->stream;
        ck(cudaMemsetAsync(dg.p, 0, n * sizeof(double), s), "memset");
        ck(cudaMemsetAsync(ds.p, 0, 4 * sizeof(double), s), "memset");
        ck(cudaMemsetAsync(derr.p, 0, 4 * sizeof(int), s), "memset");
        AdjArgs a{dW.as<double>(), dphi.as<double>(), dg.as<double>(), ds.as<double>()};
        float ms_total = 0.f;
        unsigned long long ev = 0;
        for (int pass = 1; pass <= 2; ++pass) {
            ck(cudaMemsetAsync(dtal.p, 0, nk * 3 * sizeof(double), s), "memset");
            ck(cudaMemsetAsync(dcnt.p, 0, 16 * sizeof(unsigned long long), s), "memset");
            ck(cudaMemsetAsync(dwork.p, 0, sizeof(unsigned long long), s), "memset");
            ck(cudaEventRecord(c->ev0, s), "cudaEventRecord");
            if (!launch_prod_grid(r.T, r.A, dtal.as<double>(), dcnt.as<unsigned long long>(), derr.as<int>(),
                                  dwork.as<unsigned long long>(), r.tune, r.nsm, s, pass, &a))
                throw Error(BTE_ERR_INPUT, "tuning not supported by the grid kernel");
            ck(cudaGetLastError(), "adjoint launch");
            ck(cudaEventRecord(c->ev1, s), "cudaEventRecord");
            ck(cudaStreamSynchronize(s), "adjoint pass");
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
            ms_total += ms;
            if (pass == 1) {
                ck(cudaMemcpy(&ev, dcnt.p, sizeof ev, cudaMemcpyDeviceToHost), "d2h");
            }
        }
        int herr[4];
        std::vector<double> g(n);
        double sc[4];
        ck(cudaMemcpy(herr, derr.p, sizeof herr, cudaMemcpyDeviceToHost), "d2h");
        ck(cudaMemcpy(g.data(), dg.p, n * sizeof(double), cudaMemcpyDeviceToHost), "d2h");
        ck(cudaMemcpy(sc, ds.p, sizeof sc, cudaMemcpyDeviceToHost), "d2h");
        if (herr[0] != 0) throw Error(bte_status(herr[0]), "device error in the adjoint passes");
        // post-scattering score on every tau_i: p_i / tau_i * sum R, with
        // p_i ~ C(omega_i, T0) w_i (BE_derivative_distribution)
        const HostModes& m = c->modes;
        std::vector<double> pm(n, 0.);
        double Z = 0.;
        for (std::size_t k = 0; k < n; ++k) {
            if (m.omega[k] > 0.) pm[k] = bose_einstein_kernel(m.omega[k], p->T0) * m.w[k];
            Z += pm[k];
        }
        const double sumR = p->ballistic ? 0. : sc[1];
        for (std::size_t k = 0; k < n; ++k) {
            const double tau = m.w[k] > 0. ? 1.0 / m.w[k] : 0.;
            out->dphi_dtau[k] = g[k] + (tau > 0. && Z > 0. ? (pm[k] / Z) / tau * sumR : 0.);
        }
        out->phi = sc[2];
        out->dphi_dp = sc[0];
        out->events = (int64_t)ev;
        out->kernel_ms = ms_total;
        return BTE_OK;
    } catch (const Error& e) {
        c->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_CUDA;
    }
}
