// capi.cu - the C ABI of include/btegpu.h: context, device tables, run
// orchestration and the post-processing of src/RTA_MC2D.cpp:2326-2435.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "../../include/btegpu.h"
#include "btegpu_debug.h"
#include "kernels.h"
#include "tables.hpp"
#include "ctx.hpp"
#include "frames.hpp"

using bte::Error;

namespace {

thread_local std::string g_create_error;

}  // namespace

using bte::ck;
using bte::DBuf;
using bte::hw_threads;

namespace bte {

void sync(bte_ctx* c) { ck(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"); }

void ensure_static(bte_ctx* c) {
    const bte::HostModes& m = c->modes;
    const bte::HostGeometry& g = c->geom;
    const std::size_t n = m.n();
    if (!c->modes_dev) {
        // rates of every material, [nmat][n] (one set without materials)
        const std::vector<double>& wall = c->nmat > 0 ? c->mat_w : m.w;
        std::vector<double> tau(wall.size());
        for (std::size_t k = 0; k < wall.size(); ++k) tau[k] = wall[k] > 0. ? 1.0 / wall[k] : 0.;
        std::vector<bte::ModeVel> mv(n);
        for (std::size_t k = 0; k < n; ++k) {
            mv[k].vx = m.vxc[k];
            mv[k].vy = m.vyc[k];
            mv[k].ivx = m.vxc[k] != 0. ? 1.0 / m.vxc[k] : HUGE_VAL;
            mv[k].ivy = m.vyc[k] != 0. ? 1.0 / m.vyc[k] : HUGE_VAL;
        }
        c->d_vxc.upload(m.vxc, c->stream);
        c->d_vyc.upload(m.vyc, c->stream);
        c->d_w.upload(wall, c->stream);
        c->d_tau.upload(tau, c->stream);
        c->d_mv.upload(mv, c->stream);
        sync(c);
        c->modes_dev = true;
    }
    if (!c->geom_dev) {
        c->d_boxes.upload(g.boxes, c->stream);
        c->d_hull.upload(g.hull, c->stream);
        c->d_borders.upload(g.borders, c->stream);
        c->d_contacts.upload(g.contacts, c->stream);
        c->d_cseg.upload(g.contact_seg, c->stream);
        c->d_transl.upload(g.translation, c->stream);
        c->d_boxmat.upload(g.mat, c->stream);
        {
            const bte::TranslationFast tf = bte::build_translation_fast(g);
            c->have_tfast = !tf.iv.empty();
            if (c->have_tfast) {
                c->d_tfast.upload(tf.iv, c->stream);
                c->d_tfast_rng.upload(tf.rng, c->stream);
                c->d_tfast_u.upload(tf.u, c->stream);
            }
        }
        if (g.rect_grid) {
            c->d_gx.upload(g.gx, c->stream);
            c->d_gy.upload(g.gy, c->stream);
            c->d_gcell.upload(g.gcell, c->stream);
            std::vector<int2> bc(g.boxes.size(), make_int2(-1, -1));
            for (int i = 0; i < g.gnx; ++i)
                for (int j = 0; j < g.gny; ++j) {
                    int v = g.gcell[std::size_t(i) * g.gny + j];
                    int b = v >= 0 ? v : (v <= -2 ? -2 - v : -1);
                    if (b >= 0) bc[std::size_t(b)] = make_int2(i, j);
                }
            c->d_boxcell.upload(bc, c->stream);
        }
        {
            // border lines and neighbour pieces of the convex-polygon path
            // (transient boxes off a grid, every steady-state geometry):
            // a segment contact of box a lies on the border of a whose
            // outward normal is the contact's normal; its ends give the
            // interval of arc length that leads into the neighbour
            std::vector<bte::PolyBorder> pb(g.borders.size());
            std::vector<bte::PolyPiece> pieces;
            for (std::size_t a = 0; a < g.boxes.size(); ++a) {
                const bte::GBox& bx = g.boxes[a];
                for (int k = 0; k < bx.nborders; ++k) {
                    const std::size_t gb = std::size_t(bx.border_off + k);
                    const bte::GBorder& br = g.borders[gb];
                    bte::PolyBorder& P = pb[gb];
                    const double len = std::hypot(br.p2.x - br.p1.x, br.p2.y - br.p1.y);
                    P.nx = br.np.x;
                    P.ny = br.np.y;
                    P.c = br.np.x * br.p1.x + br.np.y * br.p1.y;
                    P.px = br.p1.x;
                    P.py = br.p1.y;
                    P.ux = len > 0. ? (br.p2.x - br.p1.x) / len : 0.;
                    P.uy = len > 0. ? (br.p2.y - br.p1.y) / len : 0.;
                    P.cls = br.ncls;
                    P.piece_off = int(pieces.size());
                    for (int i = 0; i < bx.ncontacts; ++i) {
                        const std::size_t ci = std::size_t(bx.contact_off + i);
                        const bte::GBorder& cb = g.contact_borders[ci];
                        if (cb.p1.x == cb.p2.x && cb.p1.y == cb.p2.y) continue;  // point contact
                        const bte::GContact& gc = g.contacts[ci];
                        if (std::fabs(gc.np.x - br.np.x) > 1e-9 || std::fabs(gc.np.y - br.np.y) > 1e-9) continue;
                        const double d1 = br.np.x * cb.p1.x + br.np.y * cb.p1.y - P.c;
                        const double d2 = br.np.x * cb.p2.x + br.np.y * cb.p2.y - P.c;
                        if (std::fabs(d1) > 1e-6 || std::fabs(d2) > 1e-6) continue;  // on another line
                        double s0 = (cb.p1.x - P.px) * P.ux + (cb.p1.y - P.py) * P.uy;
                        double s1 = (cb.p2.x - P.px) * P.ux + (cb.p2.y - P.py) * P.uy;
                        if (s0 > s1) std::swap(s0, s1);
                        pieces.push_back(bte::PolyPiece{s0 - 1.0e-9, s1 + 1.0e-9, gc.id, -1});
                    }
                    P.npieces = int(pieces.size()) - P.piece_off;
                }
            }
            if (pieces.empty()) pieces.push_back(bte::PolyPiece{0., 0., -1, -1});
            c->d_pborders.upload(pb, c->stream);
            c->d_ppieces.upload(pieces, c->stream);
            c->pieces_host = pieces;
            c->pborders_host = pb;
            c->dmm_dev = false;
            // axis-aligned rectangles: four borders with normals +x, -x, +y, -y
            std::vector<bte::PolyRect> rect(g.boxes.size());
            for (std::size_t a = 0; a < g.boxes.size(); ++a) {
                const bte::GBox& bx = g.boxes[a];
                bte::PolyRect R{0., 0., 0., 0., -1, -1, -1, -1, -2, -2, -2, -2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                int k4[4] = {-1, -1, -1, -1};
                double c4[4] = {0., 0., 0., 0.};
                bool ok = bx.nborders == 4;
                for (int k = 0; ok && k < 4; ++k) {
                    const bte::PolyBorder& P = pb[std::size_t(bx.border_off + k)];
                    const int side = P.nx == 1. && P.ny == 0. ? 0 : P.nx == -1. && P.ny == 0. ? 1
                                   : P.nx == 0. && P.ny == 1. ? 2 : P.nx == 0. && P.ny == -1. ? 3 : -1;
                    if (side < 0 || k4[side] >= 0) ok = false;
                    else {
                        k4[side] = k;
                        c4[side] = P.c;
                    }
                }
                if (ok) {
                    R.x0 = -c4[1];
                    R.x1 = c4[0];
                    R.y0 = -c4[3];
                    R.y1 = c4[2];
                    R.kx1 = k4[0];
                    R.kx0 = k4[1];
                    R.ky1 = k4[2];
                    R.ky0 = k4[3];
                    if (!(R.x0 < R.x1 && R.y0 < R.y1)) R.kx1 = -1;
                    // what lies across each whole side
                    int nbs[4], fls[4], cls[4];
                    for (int sd = 0; sd < 4; ++sd) {
                        const bte::PolyBorder& P = pb[std::size_t(bx.border_off + k4[sd])];
                        const double len = sd < 2 ? R.y1 - R.y0 : R.x1 - R.x0;
                        cls[sd] = P.cls;
                        fls[sd] = 0;
                        if (P.npieces == 0) {
                            nbs[sd] = -1;
                        } else if (P.npieces == 1 && pieces[std::size_t(P.piece_off)].s0 <= 0. &&
                                   pieces[std::size_t(P.piece_off)].s1 >= len) {
                            const int nb = pieces[std::size_t(P.piece_off)].box;
                            nbs[sd] = nb;
                            fls[sd] = (g.reservoir[std::size_t(nb)] ? 1 : 0) | (g.tto[std::size_t(nb)] >= 0 ? 2 : 0);
                            // a contact between crystals takes the piece lookup (its table)
                            if (g.mat[std::size_t(nb)] != g.mat[a]) nbs[sd] = -2;
                        } else {
                            nbs[sd] = -2;
                        }
                    }
                    R.nx1 = nbs[0];
                    R.nx0 = nbs[1];
                    R.ny1 = nbs[2];
                    R.ny0 = nbs[3];
                    R.fx1 = fls[0];
                    R.fx0 = fls[1];
                    R.fy1 = fls[2];
                    R.fy0 = fls[3];
                    R.cx1 = cls[0];
                    R.cx0 = cls[1];
                    R.cy1 = cls[2];
                    R.cy0 = cls[3];
                    // a strip spanning the period: the periodic box across
                    // one side translates by the box's extent onto the
                    // periodic box across the other side, whose whole side
                    // this box is (geometry_2d::translate lands there)
                    auto self_periodic = [&](int hi, int lo, double ext, bool along_x) {
                        if (hi < 0 || lo < 0 || !(fls[along_x ? 0 : 2] & 2) || !(fls[along_x ? 1 : 3] & 2)) return 0;
                        const bte::V2 th = g.translation[std::size_t(hi)], tl = g.translation[std::size_t(lo)];
                        const bool ok = g.tto[std::size_t(hi)] == lo && g.tto[std::size_t(lo)] == hi &&
                                        (along_x ? (th.x == -ext && th.y == 0. && tl.x == ext && tl.y == 0.)
                                                 : (th.y == -ext && th.x == 0. && tl.y == ext && tl.x == 0.));
                        return ok ? 1 : 0;
                    };
                    if (R.kx1 >= 0) {
                        R.perx = self_periodic(R.nx1, R.nx0, R.x1 - R.x0, true);
                        R.pery = self_periodic(R.ny1, R.ny0, R.y1 - R.y0, false);
                    }
                }
                rect[a] = R;
            }
            c->d_prect.upload(rect, c->stream);
        }
        sync(c);
        c->geom_dev = true;
    }
    if (!c->lambert_dev) {
        bte::LambertTable L;
        std::vector<int> mir;
        if (c->ncrys > 0) {  // each crystal's rows over its own modes, then offset
            std::vector<bte::LambertTable> Ls;
            std::vector<std::vector<int>> ms;
            for (const bte::HostModes& cm : c->crys) {
                Ls.push_back(bte::build_lambert(cm, g, hw_threads()));
                ms.push_back(bte::build_mirror(cm, g));
            }
            L = bte::merge_lambert(Ls, c->crys, c->crys_off);
            mir = bte::merge_mirror(ms, c->crys, c->crys_off, L.nclass);
        } else {
            L = bte::build_lambert(m, g, hw_threads());
            mir = bte::build_mirror(m, g);
        }
        c->nclass = L.nclass;
        c->d_row_ptr.upload(L.row_ptr, c->stream);
        c->d_lcol.upload(L.col, c->stream);
        c->d_lcdf.upload(L.cdf, c->stream);
        c->d_lalias.upload(L.alias, c->stream);
        c->have_mirror = std::any_of(mir.begin(), mir.end(), [](int x) { return x >= 0; });
        c->d_mirror.upload(mir, c->stream);
        // exit times of the convex-polygon path without a division: 1 / (n.v)
        // per border normal and mode, -1 where such a border is not left
        // (n.v <= 0); only for tables of at most 256 MB
        const std::size_t n = m.n(), ncl = g.normals.size();
        c->d_invden.release();
        if (ncl > 0 && ncl * n * sizeof(double) <= (std::size_t(256) << 20)) {
            std::vector<double> inv(ncl * n);
            for (std::size_t k = 0; k < ncl; ++k)
                for (std::size_t j = 0; j < n; ++j) {
                    const double den = g.normals[k].x * m.vxc[j] + g.normals[k].y * m.vyc[j];
                    inv[k * n + j] = den > 0. ? 1.0 / den : -1.0;
                }
            c->d_invden.upload(inv, c->stream);
        }
        sync(c);
        c->lambert_dev = true;
        if (c->verbose)
            std::printf("#Diffusive table: %d wall normals, %zu entries\n", L.nclass, L.col.size());
    }
    if (c->ncrys > 0 && !c->dmm_dev) {
        // one mismatch table per (crystal A, crystal B, contact normal) over
        // the contacts from a box that is neither a reservoir nor periodic to
        // a box of another crystal, at the Teq of the first such box
        std::map<std::tuple<int, int, double, double>, int> tab_of;
        std::vector<long long> rows;
        std::vector<bte::DmmEnt> ents;
        const std::size_t ntot = m.n();
        for (std::size_t a = 0; a < g.boxes.size(); ++a) {
            if (g.reservoir[a] || g.tto[a] >= 0) continue;
            const bte::GBox& B = g.boxes[a];
            for (int i = 0; i < B.ncontacts; ++i) {
                const std::size_t ci = std::size_t(B.contact_off + i);
                const int b = g.contacts[ci].id;
                const int ma = g.mat[a], mb = g.mat[std::size_t(b)];
                if (ma == mb) continue;
                const bte::V2 nw = g.contact_borders[ci].np;
                const auto key = std::make_tuple(ma, mb, nw.x, nw.y);
                if (tab_of.count(key)) continue;
                const bte::HostModes& A = c->crys[std::size_t(ma)];
                const bte::HostModes& Bm = c->crys[std::size_t(mb)];
                const bte::DmmTable D = bte::build_dmm_table(
                    A, c->crys_off[std::size_t(ma)], Bm, c->crys_off[std::size_t(mb)], ntot, nw,
                    A.V * bte::crystal_thickness(c, ma) / A.c, Bm.V * bte::crystal_thickness(c, mb) / Bm.c,
                    g.Teq[a], hw_threads());
                tab_of[key] = int(tab_of.size());
                const long long base = (long long)ents.size();
                for (std::size_t K = 0; K <= ntot; ++K) rows.push_back(base + D.row[K]);
                for (std::size_t e = 0; e < D.out.size(); ++e) ents.push_back(bte::DmmEnt{D.cum[e], D.out[e], D.side[e]});
            }
        }
        // each piece that leads into another crystal names its table
        std::vector<bte::PolyPiece>& pcs = c->pieces_host;
        for (std::size_t a = 0; a < g.boxes.size(); ++a) {
            if (g.reservoir[a] || g.tto[a] >= 0) continue;
            const bte::GBox& B = g.boxes[a];
            for (int i = 0; i < B.ncontacts; ++i) {
                const std::size_t ci = std::size_t(B.contact_off + i);
                const int b = g.contacts[ci].id;
                if (g.mat[a] == g.mat[std::size_t(b)]) continue;
                const bte::V2 nw = g.contact_borders[ci].np;
                const int t = tab_of.at(std::make_tuple(g.mat[a], g.mat[std::size_t(b)], nw.x, nw.y));
                for (int k = 0; k < B.nborders; ++k) {
                    const bte::PolyBorder& P = c->pborders_host[std::size_t(B.border_off + k)];
                    for (int j = 0; j < P.npieces; ++j) {
                        bte::PolyPiece& pc = pcs[std::size_t(P.piece_off + j)];
                        if (pc.box == b) pc.pad = t;
                    }
                }
            }
        }
        // the same tables per contact, for the evolparticle-faithful kernels
        std::vector<int> cdmm(g.contacts.size(), -1);
        for (std::size_t a = 0; a < g.boxes.size(); ++a) {
            if (g.reservoir[a] || g.tto[a] >= 0) continue;
            const bte::GBox& B = g.boxes[a];
            for (int i = 0; i < B.ncontacts; ++i) {
                const std::size_t ci = std::size_t(B.contact_off + i);
                const int b = g.contacts[ci].id;
                if (g.mat[a] == g.mat[std::size_t(b)]) continue;
                const bte::V2 nw = g.contact_borders[ci].np;
                cdmm[ci] = tab_of.at(std::make_tuple(g.mat[a], g.mat[std::size_t(b)], nw.x, nw.y));
            }
        }
        std::vector<int> coff;
        for (int k = 0; k <= c->ncrys; ++k)
            coff.push_back(k < c->ncrys ? int(c->crys_off[std::size_t(k)]) : int(m.n()));
        if (cdmm.empty()) cdmm.push_back(-1);
        if (rows.empty()) rows.push_back(0);
        if (ents.empty()) ents.push_back(bte::DmmEnt{0., 0, 0});
        c->d_dmm_row.upload(rows, c->stream);
        c->d_dmm_ent.upload(ents, c->stream);
        c->d_cdmm.upload(cdmm, c->stream);
        c->d_crysoff.upload(coff, c->stream);
        c->d_ppieces.upload(pcs, c->stream);
        c->ndmm = int(tab_of.size());
        sync(c);
        c->dmm_dev = true;
    }
}

void ensure_resample(bte_ctx* c, double T0) {
    if (c->nmat > 0) T0 = -2.0;  // one table per material, at the material's T0
    if (c->resample_T0 == T0) return;
    std::vector<double> cdf;
    std::vector<bte::Alias> al;
    if (c->nmat > 0) {
        bte::HostModes mm = c->modes;
        const std::size_t n = mm.n();
        for (int k = 0; k < c->nmat; ++k) {
            std::vector<double> ck;
            std::vector<bte::Alias> ak;
            mm.w.assign(c->mat_w.begin() + std::ptrdiff_t(k * n), c->mat_w.begin() + std::ptrdiff_t((k + 1) * n));
            bte::build_resample(mm, c->mat_T0[std::size_t(k)], ck, ak);
            cdf.insert(cdf.end(), ck.begin(), ck.end());
            al.insert(al.end(), ak.begin(), ak.end());
        }
    } else {
        bte::build_resample(c->modes, T0, cdf, al);
    }
    std::vector<float> prob(al.size());
    std::vector<int> alt(al.size());
    for (std::size_t i = 0; i < al.size(); ++i) {
        prob[i] = al[i].prob;
        alt[i] = al[i].alt;
    }
    c->d_rcdf.upload(cdf, c->stream);
    c->d_rprob.upload(prob, c->stream);
    c->d_ralt.upload(alt, c->stream);
    sync(c);
    c->resample_T0 = T0;
}

}  // namespace bte

namespace {
using bte::ensure_resample;
using bte::ensure_static;
using bte::sync;

// Per-material budgets of a walls-source run: wall w of material m is drawn
// with probability share[m] E_w / E_m (energy-weighted when no shares).
void apply_shares(bte_ctx* c, bool upload) {
    c->shares_dirty = false;
    if (c->mat_share.empty()) return;
    const std::size_t nm = c->mat_share.size();
    c->mat_energy.assign(nm, 0.);
    for (auto& W : c->gens.walls) {
        const std::size_t k = std::size_t(c->geom.mat[std::size_t(W.box)]);
        if (k >= nm) throw Error(BTE_ERR_INPUT, "box material without loaded rates (bte_load_materials)");
        c->mat_energy[k] += W.energy;
    }
    for (std::size_t k = 0; k < nm; ++k)
        if (c->mat_share[k] > 0. && !(c->mat_energy[k] > 0.))
            throw Error(BTE_ERR_INPUT, "a material with a particle share has no isothermal wall");
    double cum = 0.;
    for (std::size_t i = 0; i < c->gens.walls.size(); ++i) {
        const auto& W = c->gens.walls[i];
        const std::size_t k = std::size_t(c->geom.mat[std::size_t(W.box)]);
        cum += c->mat_share[k] * W.energy / c->mat_energy[k];
        c->gens.wall_cum[i] = cum;
    }
    if (upload) {
        c->d_wcum.upload(c->gens.wall_cum, c->stream);
        sync(c);
    }
}

void ensure_generators(bte_ctx* c, const bte_rta_params* p) {
    if (c->gen_key_source == p->source) {
        if (p->source == BTE_SOURCE_WALLS && c->shares_dirty) apply_shares(c, true);
        if (p->source == BTE_SOURCE_INITIAL &&
            (c->gen_key_n != p->nparticles || c->gen_key_seed != p->seed)) {
            c->gen_Eeff = bte::initial_counts(c->gens, p->nparticles, p->seed);
            c->d_ifirst.upload(c->gens.init_first, c->stream);
            sync(c);
            c->gen_key_n = p->nparticles;
            c->gen_key_seed = p->seed;
        }
        return;
    }
    if (c->ncrys > 0) {
        // each crystal's generators, rows over the concatenated modes
        std::vector<bte::Generators> G;
        for (int k = 0; k < c->ncrys; ++k) {
            const bte::GenEmbed e{k, c->crys_off[std::size_t(k)], c->modes.n(), bte::crystal_thickness(c, k)};
            G.push_back(p->source == BTE_SOURCE_WALLS
                            ? bte::build_wall_generators(c->crys[std::size_t(k)], c->geom, false, &e)
                            : bte::build_initial_generators(c->crys[std::size_t(k)], c->geom, &e));
        }
        c->gens = bte::merge_generators(G, p->source == BTE_SOURCE_WALLS, true);
        if (p->source == BTE_SOURCE_INITIAL) c->gen_Eeff = bte::initial_counts(c->gens, p->nparticles, p->seed);
    } else if (p->source == BTE_SOURCE_WALLS) {
        c->gens = bte::build_wall_generators(c->modes, c->geom);
        apply_shares(c, false);
    } else {
        if (!c->mat_share.empty()) throw Error(BTE_ERR_INPUT, "particle shares need the walls source");
        c->gens = bte::build_initial_generators(c->modes, c->geom);
        c->gen_Eeff = bte::initial_counts(c->gens, p->nparticles, p->seed);
    }
    std::vector<float> prob(c->gens.alias.size());
    std::vector<int> alt(c->gens.alias.size());
    for (std::size_t i = 0; i < prob.size(); ++i) {
        prob[i] = c->gens.alias[i].prob;
        alt[i] = c->gens.alias[i].alt;
    }
    c->d_gcdf.upload(c->gens.cdf, c->stream);
    c->d_gprob.upload(prob, c->stream);
    c->d_galt.upload(alt, c->stream);
    std::vector<bte::WallGenDev> wd;
    for (auto& W : c->gens.walls) {
        bte::WallGenDev d;
        d.p1 = W.p1;
        d.nd = W.nd;
        d.sa = W.sa;
        d.sb = W.sb;
        d.box = W.box;
        d.sign = W.sign;
        wd.push_back(d);
    }
    c->d_walls.upload(wd, c->stream);
    c->d_wcum.upload(c->gens.wall_cum, c->stream);
    c->d_ifirst.upload(c->gens.init_first, c->stream);
    c->d_ibox.upload(c->gens.init_box, c->stream);
    c->d_isign.upload(c->gens.init_sign, c->stream);
    sync(c);
    c->gen_key_source = p->source;
    c->gen_key_n = p->nparticles;
    c->gen_key_seed = p->seed;
}

bte_status fail(bte_ctx* c, const Error& e) {
    c->err = e.what();
    return e.code;
}

void validate(const bte_rta_params* p) {
    if (!p) throw Error(BTE_ERR_INPUT, "null parameters");
    if (!(p->dt > 0.) || !(p->maxtime > 0.) || !std::isfinite(p->dt) || !std::isfinite(p->maxtime))
        throw Error(BTE_ERR_INPUT, "time dt and maxtime must be positive");
    if (p->maxtime / p->dt > 1.0e7) throw Error(BTE_ERR_INPUT, "too many time bins");
    if (p->nparticles < 1) throw Error(BTE_ERR_INPUT, "particles N must be >= 1");
    if (p->mode != BTE_MODE_REPLAY && p->mode != BTE_MODE_PRODUCTION)
        throw Error(BTE_ERR_INPUT, "unknown mode");
    if (p->source != BTE_SOURCE_WALLS && p->source != BTE_SOURCE_INITIAL)
        throw Error(BTE_ERR_INPUT, "unknown particle source");
    if (!(p->specularity >= 0. && p->specularity <= 1.))
        throw Error(BTE_ERR_INPUT, "specularity must lie in [0, 1]");
    if (!(p->T0 > 0.)) throw Error(BTE_ERR_INPUT, "T0 must be positive");
}

}  // namespace

namespace bte {
// Validation and tables of one RTA run (shared by bte_rta_run and
// bte_rta_adjoint).
void prepare_run(bte_ctx* c, const bte_rta_params* p) {
    validate(p);
    if (!c->have_modes || !c->have_geom)
        throw Error(BTE_ERR_STATE, "load the mode table and the geometry before running");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    if (c->ncrys > 0) {
        // crystals joined by mismatch interfaces: every crystal at the run's T0
        if (c->mat_T0.empty() || c->mat_T0[0] != p->T0) {
            c->mat_T0.assign(std::size_t(c->ncrys), p->T0);
            c->resample_T0 = -1;
        }
    }
    for (std::size_t b = 0; b < c->geom.boxes.size(); ++b) {
        if (c->geom.mat[b] >= std::max(c->nmat, 1))
            throw Error(BTE_ERR_INPUT, "box material without loaded rates (bte_load_materials)");
        const double T0b = bte::box_T0(c, int(b), p->T0);
        if (c->nmat > 0 && c->ncrys == 0) {  // a particle keeps its material: materials must not touch
            const bte::GBox& B = c->geom.boxes[b];
            for (int i = 0; i < B.ncontacts; ++i) {
                const int o = c->geom.contacts[std::size_t(B.contact_off + i)].id;
                if (c->geom.mat[std::size_t(o)] != c->geom.mat[b])
                    throw Error(BTE_ERR_INPUT, "boxes of different materials touch");
            }
            if (c->geom.tto[b] >= 0 && c->geom.mat[std::size_t(c->geom.tto[b])] != c->geom.mat[b])
                throw Error(BTE_ERR_INPUT, "a periodic box maps to another material");
        }
        if (!c->geom.reservoir[b] && !bte::almost_equal(c->geom.Teq[b], T0b) && c->geom.Teq[b] != T0b)
            throw Error(BTE_ERR_INPUT, "Tref in xml is different from provided T0");
    }
    ensure_static(c);
    if (p->specularity > 0. && !c->have_mirror)
        throw Error(BTE_ERR_INPUT, "specular walls need an axis-aligned q grid with mirror images");
    ensure_resample(c, p->T0);
    ensure_generators(c, p);
}
}  // namespace bte

namespace bte {
// The post-processing of one run's raw tallies into its outputs
// (src/RTA_MC2D.cpp:2336-2435): / V_box, x Eeff (per material with shares),
// the flux factor, the time integration of a walls source (or bin averages
// of an initial deviation) and T = gz / (C_v / vcorr) + T0.
void rta_post(bte_ctx* c, const bte_rta_params* p, int nbx, int nbins, double Eeff, double step,
              std::vector<double>& gz, std::vector<double>& jx, std::vector<double>& jy, bte_rta_result* out) {
    const bte::HostModes& m = c->modes;
    const bte::HostGeometry& g = c->geom;
    const std::size_t nk = std::size_t(nbx) * std::size_t(nbins);
    // only the tallies an output needs: gz for the temperature, jx, jy
    const bool need_gz = out->temperature != nullptr, need_jx = out->jx != nullptr, need_jy = out->jy != nullptr;
    auto each = [&](auto&& f) {
        if (need_gz) f(gz);
        if (need_jx) f(jx);
        if (need_jy) f(jy);
    };
    // post-processing, src/RTA_MC2D.cpp:2336-2435
    each([&](std::vector<double>& v) {
        for (int ir = 0; ir < nbx; ++ir) {
            const double vbox = g.boxes[std::size_t(ir)].area * bte::box_thickness(c, ir);
            for (int i = 0; i < nbins; ++i) v[std::size_t(ir) * nbins + i] /= vbox;
        }
    });
    if (!c->mat_share.empty() && p->source == BTE_SOURCE_WALLS) {
        // Eeff_m = E_m / (share_m N) per material
        for (int ir = 0; ir < nbx; ++ir) {
            const std::size_t k = std::size_t(g.mat[std::size_t(ir)]);
            const double Em = c->mat_share[k] > 0. ? c->mat_energy[k] / (c->mat_share[k] * double(p->nparticles)) : 0.;
            for (int i = 0; i < nbins; ++i) {
                const std::size_t q = std::size_t(ir) * nbins + i;
                if (need_gz) gz[q] *= Em;
                if (need_jx) jx[q] *= Em * 1e12 * 1e9 * 1e9;
                if (need_jy) jy[q] *= Em * 1e12 * 1e9 * 1e9;
            }
        }
    } else {
        if (need_gz)
            for (auto& x : gz) x *= Eeff;
        if (need_jx)
            for (auto& x : jx) x *= Eeff * 1e12 * 1e9 * 1e9;
        if (need_jy)
            for (auto& x : jy) x *= Eeff * 1e12 * 1e9 * 1e9;
    }
    if (p->source == BTE_SOURCE_WALLS) {
        // step response: integrate in time
        each([&](std::vector<double>& v) {
            for (int ir = 0; ir < nbx; ++ir)
                for (int i = 1; i < nbins; ++i) {
                    const std::size_t k = std::size_t(ir) * nbins + i;
                    v[k] += v[k - 1];
                }
        });
    } else {
        // relaxation of an initial deviation: bin averages
        each([&](std::vector<double>& v) {
            for (std::size_t k = 0; k < nk; ++k) v[k] /= step;
        });
    }
    if (out->temperature) {
        // C_v per material (per crystal: over its own modes, q points and
        // cell), cached while the tables and temperatures stay
        std::vector<double> T0s(std::size_t(std::max(c->nmat, 1)));
        for (std::size_t k = 0; k < T0s.size(); ++k) T0s[k] = c->nmat > 0 ? c->mat_T0[k] : p->T0;
        if (c->cv_version != c->tables_version || c->cv_T0s != T0s) {
            c->cv_cache.resize(T0s.size());
            for (std::size_t k = 0; k < T0s.size(); ++k)
                c->cv_cache[k] = bte::calc_cv(c->ncrys > 0 ? c->crys[k] : m, T0s[k]);
            c->cv_T0s = T0s;
            c->cv_version = c->tables_version;
        }
        const std::vector<double>& cvm = c->cv_cache;
        for (int ir = 0; ir < nbx; ++ir) {
            const std::size_t mk = std::size_t(c->nmat > 0 ? g.mat[std::size_t(ir)] : 0);
            const double cv = cvm[mk];
            const double vcorr = bte::box_thickness(c, ir) / (c->ncrys > 0 ? c->crys[mk].c : m.c);
            const double T0b = bte::box_T0(c, ir, p->T0);
            for (int i = 0; i < nbins; ++i) {
                const std::size_t k = std::size_t(ir) * nbins + i;
                out->temperature[k] = gz[k] / (cv / vcorr) + T0b;
            }
        }
    }
    if (out->jx) std::copy(jx.begin(), jx.end(), out->jx);
    if (out->jy) std::copy(jy.begin(), jy.end(), out->jy);
}
}  // namespace bte

extern "C" {

int32_t bte_version(void) { return BTEGPU_VERSION; }

bte_status bte_create(bte_ctx** out, const bte_device_opts* opts) {
    if (!out) return BTE_ERR_INPUT;
    *out = nullptr;
    try {
        std::unique_ptr<bte_ctx> c(new bte_ctx());
        c->device = opts ? opts->device : 0;
        c->verbose = opts ? opts->verbose : 0;
        int ndev = 0;
        ck(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
        if (c->device < 0 || c->device >= ndev) throw Error(BTE_ERR_INPUT, "no such CUDA device");
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        ck(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device), "attribute");
        ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaEventCreate(&c->ev0), "cudaEventCreate");
        ck(cudaEventCreate(&c->ev1), "cudaEventCreate");
        *out = c.release();
        return BTE_OK;
    } catch (const Error& e) {
        g_create_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return BTE_ERR_CUDA;
    }
}

bte_status bte_destroy(bte_ctx* c) {
    if (!c) return BTE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    cudaStream_t s = c->stream;
    bte::destroy_berta(c);
    bte::destroy_steady(c);
    delete c;
    if (s) cudaStreamDestroy(s);
    return BTE_OK;
}

bte_status bte_last_error(const bte_ctx* c, char* buf, size_t size) {
    if (!buf || size == 0) return BTE_ERR_INPUT;
    const std::string& m = c ? c->err : g_create_error;
    std::snprintf(buf, size, "%s", m.c_str());
    return BTE_OK;
}

bte_status bte_set_tuning(bte_ctx* c, const bte_tuning* t) {
    if (!c) return BTE_ERR_INPUT;
    if (!t) {
        c->tune = bte::ProdTuning{0, 0, 0, 0};
        return BTE_OK;
    }
    if (t->block_threads < 0 || t->block_threads > 256 || (t->block_threads % 32) != 0) {
        c->err = "block_threads must be a multiple of 32 in [32, 256] (0 = default)";
        return BTE_ERR_INPUT;
    }
    c->tune.block_threads = t->block_threads;
    c->tune.blocks_per_sm = t->blocks_per_sm;
    c->tune.smem_tally = t->smem_tally;
    if (t->particles_per_thread < 0 || t->particles_per_thread > 2) {
        c->err = "particles_per_thread must be 1 or 2 (0 = default)";
        return BTE_ERR_INPUT;
    }
    c->tune.particles_per_thread = t->particles_per_thread;
    return BTE_OK;
}

bte_status bte_load_modes(bte_ctx* c, const bte_mode_table* mt) {
    if (!c) return BTE_ERR_INPUT;
    c->group_valid = false;
    try {
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        c->modes = bte::build_modes(mt);
        c->have_modes = true;
        c->tables_version++;
        bte::reset_propagators(c);
        c->ncrys = 0;
        c->crys.clear();
        c->crys_off.clear();
        c->crys_thick.clear();
        c->dmm_dev = false;
        c->nmat = 0;  // materials are rate sets over one table
        c->mat_w.clear();
        c->mat_T0.clear();
        c->modes_dev = false;
        c->lambert_dev = false;
        c->resample_T0 = -1;
        c->gen_key_source = -1;
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_load_geometry(bte_ctx* c, const bte_geometry* g) {
    if (!c) return BTE_ERR_INPUT;
    c->group_valid = false;
    try {
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        bte::HostGeometry ng = bte::build_geometry(g);
        // the Lambert wall table depends on the geometry only through its
        // distinct wall normals: keep it when they are the same
        const bool same_normals = c->have_geom && ng.normals.size() == c->geom.normals.size() &&
                                  std::equal(ng.normals.begin(), ng.normals.end(), c->geom.normals.begin(),
                                             [](const bte::V2& a, const bte::V2& b) {
                                                 return a.x == b.x && a.y == b.y;
                                             });
        c->geom = std::move(ng);
        c->have_geom = true;
        c->tables_version++;
        c->geom_dev = false;
        c->dmm_dev = false;
        if (!same_normals) c->lambert_dev = false;
        c->gen_key_source = -1;
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_load_mode_tables(bte_ctx* c, int32_t ntables, const bte_mode_table* tables,
                                const double* thickness) {
    if (!c) return BTE_ERR_INPUT;
    c->group_valid = false;
    try {
        if (ntables < 1 || !tables) throw Error(BTE_ERR_INPUT, "no mode tables");
        std::vector<double> th;
        if (thickness)
            for (int k = 0; k < ntables; ++k) {
                if (!(thickness[k] > 0.) || !std::isfinite(thickness[k]))
                    throw Error(BTE_ERR_INPUT, "crystal thickness must be > 0");
                th.push_back(thickness[k]);
            }
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        std::vector<bte::HostModes> crys;
        for (int k = 0; k < ntables; ++k) crys.push_back(bte::build_modes(&tables[k]));
        std::vector<std::size_t> off;
        bte::HostModes all = bte::concat_modes(crys, off);
        if (all.n() > (std::size_t(1) << 30)) throw Error(BTE_ERR_INPUT, "too many modes");
        // the materials machinery with one rate set per crystal, each masked
        // to its crystal's modes (zero rate, so zero weight, elsewhere)
        const std::size_t n = all.n();
        std::vector<double> mw(std::size_t(ntables) * n, 0.);
        for (int k = 0; k < ntables; ++k)
            for (std::size_t j = 0; j < crys[std::size_t(k)].n(); ++j)
                mw[std::size_t(k) * n + off[std::size_t(k)] + j] = crys[std::size_t(k)].w[j];
        c->modes = std::move(all);
        c->crys = std::move(crys);
        c->crys_off = std::move(off);
        c->crys_thick = std::move(th);
        c->ncrys = ntables;
        c->have_modes = true;
        c->tables_version++;
        bte::reset_propagators(c);
        c->nmat = ntables;
        c->mat_w = std::move(mw);
        c->mat_T0.clear();  // set to each run's T0
        c->mat_share.clear();
        c->modes_dev = false;
        c->lambert_dev = false;
        c->dmm_dev = false;
        c->resample_T0 = -1;
        c->gen_key_source = -1;
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_interface_table(const bte_mode_table* A, const bte_mode_table* B, double nx, double ny,
                               double thickness_a, double thickness_b, double Tref, int64_t* first,
                               int64_t* nentries, int32_t* side, int32_t* mode, double* cum) {
    try {
        if (!A || !B || !first || !nentries || !(thickness_a > 0.) || !(thickness_b > 0.) || !(Tref > 0.))
            return BTE_ERR_INPUT;
        const bte::HostModes a = bte::build_modes(A), b = bte::build_modes(B);
        const std::size_t na = a.n();
        const bte::DmmTable D = bte::build_dmm_table(a, 0, b, na, na + b.n(), bte::v2(nx, ny),
                                                     a.V * thickness_a / a.c, b.V * thickness_b / b.c, Tref,
                                                     hw_threads());
        for (std::size_t i = 0; i <= na; ++i) first[i] = D.row[i];
        *nentries = (int64_t)D.out.size();
        if (side && mode && cum)
            for (std::size_t e = 0; e < D.out.size(); ++e) {
                side[e] = D.side[e];
                mode[e] = D.side[e] == 0 ? D.out[e] : int32_t(std::size_t(D.out[e]) - na);
                cum[e] = D.cum[e];
            }
        return BTE_OK;
    } catch (const Error& e) {
        g_create_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return BTE_ERR_INPUT;
    }
}

bte_status bte_load_materials(bte_ctx* c, int32_t nmat, const double* w, const double* T0,
                              const double* share) {
    if (!c) return BTE_ERR_INPUT;
    c->group_valid = false;
    try {
        if (c->ncrys > 0) throw Error(BTE_ERR_STATE, "rate sets are for one mode table; crystals carry their own rates");
        if (nmat < 0 || (nmat > 0 && (!w || !T0))) throw Error(BTE_ERR_INPUT, "bad material arrays");
        if (share && nmat > 0) {
            double sum = 0.;
            for (int k = 0; k < nmat; ++k) {
                if (!(share[k] >= 0.) || !std::isfinite(share[k])) throw Error(BTE_ERR_INPUT, "bad share");
                sum += share[k];
            }
            if (std::fabs(sum - 1.0) > 1e-9) throw Error(BTE_ERR_INPUT, "material shares must sum to 1");
        }
        if (nmat > 0 && !c->have_modes) throw Error(BTE_ERR_STATE, "load the mode table first");
        const std::size_t n = c->modes.n();
        for (int k = 0; k < nmat; ++k) {
            if (!(T0[k] > 0.) || !std::isfinite(T0[k])) throw Error(BTE_ERR_INPUT, "material T0 must be > 0");
            for (std::size_t i = 0; i < n; ++i)
                if (!std::isfinite(w[size_t(k) * n + i]) || w[size_t(k) * n + i] < 0.)
                    throw Error(BTE_ERR_VALUE, "non-finite or negative material rate");
        }
        const bool same_rates = nmat > 0 && nmat == c->nmat &&
                                std::equal(w, w + size_t(nmat) * n, c->mat_w.begin()) &&
                                std::equal(T0, T0 + nmat, c->mat_T0.begin());
        if (same_rates && share && !c->mat_share.empty()) {
            // only the particle budgets change: reweight the walls
            c->mat_share.assign(share, share + nmat);
            c->shares_dirty = true;
            return BTE_OK;
        }
        c->nmat = nmat;
        c->mat_w.assign(w ? w : nullptr, w ? w + size_t(nmat) * n : nullptr);
        c->mat_T0.assign(T0 ? T0 : nullptr, T0 ? T0 + nmat : nullptr);
        c->mat_share.assign(share && nmat > 0 ? share : nullptr, share && nmat > 0 ? share + nmat : nullptr);
        c->gen_key_source = -1;  // wall weights depend on the shares
        c->modes_dev = false;    // rates and lifetimes
        c->geom_dev = false;     // box materials
        c->resample_T0 = -1;     // post-scattering tables
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_set_spectral(bte_ctx* c, int32_t nloc, const int32_t* boxes, int32_t nomega) {
    if (!c) return BTE_ERR_INPUT;
    try {
        if (nloc < 0 || (nloc > 0 && (!boxes || nomega < 1)))
            throw Error(BTE_ERR_INPUT, "spectral locations need boxes and ticks >= 1");
        if (nloc > 0 && !c->have_geom) throw Error(BTE_ERR_STATE, "load the geometry first");
        for (int i = 0; i < nloc; ++i) {
            if (boxes[i] < 0 || boxes[i] >= int(c->geom.boxes.size()))
                throw Error(BTE_ERR_INPUT, "spectral location is not a box");
            for (int j = 0; j < i; ++j)
                if (boxes[j] == boxes[i]) throw Error(BTE_ERR_INPUT, "repeated spectral location");
        }
        c->spec_boxes.assign(boxes ? boxes : nullptr, boxes ? boxes + nloc : nullptr);
        c->spec_nomega = nloc > 0 ? nomega : 0;
        c->spec_valid = false;
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_get_spectral(bte_ctx* c, bte_spectral_result* out) {
    if (!c || !out) return BTE_ERR_INPUT;
    try {
        if (!c->spec_valid) throw Error(BTE_ERR_STATE, "no run with spectral locations yet");
        const bte::HostGeometry& g = c->geom;
        const std::size_t n = c->modes.n();  // global modes (the crystals' one after the other)
        const std::size_t nloc = c->spec_boxes.size(), nbins = std::size_t(c->spec_nbins);
        const std::size_t nw = std::size_t(c->spec_nomega);
        // each location's crystal (the reference takes the location's
        // material's grid, :1987-2048): its modes and their first global index
        auto crystal_of = [&](std::size_t l) -> int {
            return c->ncrys > 0 ? g.mat[std::size_t(c->spec_boxes[l])] : -1;
        };
        auto modes_of = [&](int k) -> const bte::HostModes& {
            return k >= 0 ? c->crys[std::size_t(k)] : c->modes;
        };
        const bte::HostModes& m0 = modes_of(nloc > 0 ? crystal_of(0) : -1);
        const std::size_t nq = std::size_t(m0.nq);
        for (std::size_t l = 1; l < nloc; ++l) {
            const bte::HostModes& ml = modes_of(crystal_of(l));
            if (ml.nq != m0.nq || ml.grid[0] != m0.grid[0] || ml.grid[1] != m0.grid[1])
                throw Error(BTE_ERR_INPUT, "spectral locations in crystals of different q grids");
        }
        out->nloc = int32_t(nloc);
        out->nbins = int32_t(nbins);
        out->nomega = int32_t(nw);
        out->nq = int32_t(nq);
        const double hbar = 1.054571726e-34;
        for (std::size_t l = 0; l < nloc; ++l) {
            const int kc = crystal_of(l);
            const bte::HostModes& m = modes_of(kc);
            const std::size_t off = kc >= 0 ? c->crys_off[std::size_t(kc)] : 0, nk = m.n();
            const std::size_t nb = std::size_t(m.nb);
            // omega ticks of the location's crystal: LinSpaced(nomega, 0,
            // max omega) + delta/2 (:2041-2045)
            double maxw = 0.;
            for (double w : m.omega) maxw = std::max(maxw, w);
            std::vector<double> grid(nw);
            for (std::size_t i = 0; i < nw; ++i)
                grid[i] = (nw > 1 ? maxw * double(i) / double(nw - 1) : 0.) + 0.5 * maxw / double(nw);
            if (out->omega) std::copy(grid.begin(), grid.end(), out->omega + l * nw);
            // Gamma pdf of every mode over the ticks, shape k = w^2 / sigma,
            // scale theta = sigma / w (gamma_pdf, :61-63), kept where it is not
            // negligible
            const std::vector<double> sig = bte::mode_sigmas(m);
            std::vector<std::vector<std::pair<int, double>>> gw(nk);
            for (std::size_t k = 0; k < nk; ++k) {
                const double w = m.omega[k];
                if (!(w > 0.)) continue;
                const double kk = w * w / sig[k], th = sig[k] / w;
                const double lg = std::lgamma(kk);
                for (std::size_t i = 0; i < nw; ++i) {
                    const double x = grid[i] / th;
                    const double lp = (kk - 1.0) * std::log(x) - x - lg - std::log(th);
                    if (lp > -700.) {
                        const double pdf = std::exp(lp);
                        if (pdf > 0.) gw[k].emplace_back(int(i), pdf);
                    }
                }
            }
            const int box = c->spec_boxes[l];
            const double tb = bte::box_thickness(c, box);
            const double vcorr = tb / m.c;
            const double vbox = g.boxes[std::size_t(box)].area * tb;
            const double T0b = bte::box_T0(c, box, c->spec_T0);
            const double cv = bte::calc_cv(m, T0b);
            const double Eeff = c->spec_Eeff;
            std::vector<double> dT(nbins * nw, 0.), jx(nbins * nw, 0.), jy(nbins * nw, 0.), fq(nbins * nq, 0.);
            const bool steady = c->spec_steady;
            for (std::size_t b = 0; b < nbins; ++b) {
                const double* Tm = c->spec_raw.data() + (l * nbins + b) * n + off;
                for (std::size_t k = 0; k < nk; ++k) {
                    const double t = Tm[k];
                    // fd_qmesh: time / omega (transient, :757), sign / omega
                    // per segment (steady, :829)
                    const double f = steady ? double(c->spec_cnt[l * n + off + k]) : t;
                    if (f != 0. && m.omega[k] > 0.) fq[b * nq + k / nb] += f / m.omega[k];
                    if (t == 0.) continue;
                    for (auto& [i, wgt] : gw[k]) {
                        dT[b * nw + std::size_t(i)] += t * wgt;
                        jx[b * nw + std::size_t(i)] += m.vxc[k] * t * wgt;
                        jy[b * nw + std::size_t(i)] += m.vyc[k] * t * wgt;
                    }
                }
            }
            // scaling (:2350-2376) and integration in time (:2386-2413)
            const double sdT = Eeff / vbox, sj = Eeff * 1e12 * 1e9 * 1e9 / vbox;
            const double sq = Eeff * vcorr * double(nq) / (vbox * 1.0e+12 * hbar);
            for (auto& x : dT) x *= sdT;
            for (auto& x : jx) x *= sj;
            for (auto& x : jy) x *= sj;
            for (auto& x : fq) x *= sq;
            for (std::size_t b = 1; b < nbins && !steady; ++b) {
                for (std::size_t i = 0; i < nw; ++i) {
                    dT[b * nw + i] += dT[(b - 1) * nw + i];
                    jx[b * nw + i] += jx[(b - 1) * nw + i];
                    jy[b * nw + i] += jy[(b - 1) * nw + i];
                }
                for (std::size_t q = 0; q < nq; ++q) fq[b * nq + q] += fq[(b - 1) * nq + q];
            }
            for (auto& x : dT) x = x / (cv / vcorr);
            if (out->dT_omega) std::copy(dT.begin(), dT.end(), out->dT_omega + l * nbins * nw);
            if (out->jx_omega) std::copy(jx.begin(), jx.end(), out->jx_omega + l * nbins * nw);
            if (out->jy_omega) std::copy(jy.begin(), jy.end(), out->jy_omega + l * nbins * nw);
            if (out->fd_q) std::copy(fq.begin(), fq.end(), out->fd_q + l * nbins * nq);
        }
        if (out->raw) std::copy(c->spec_raw.begin(), c->spec_raw.end(), out->raw);
        out->steady = c->spec_steady ? 1 : 0;
        if (out->counts && c->spec_steady)
            for (std::size_t i = 0; i < c->spec_cnt.size(); ++i) out->counts[i] = double(c->spec_cnt[i]);
        if (out->q1bz) {
            // q points in Cartesian coordinates, reduced coordinates wrapped
            // to [-1/2, 1/2) (a Gamma-centred n1 x n2 grid, iq = i n2 + j)
            const bte::HostModes& m = m0;
            const int n1 = m.grid[0] > 0 ? m.grid[0] : 1, n2 = m.grid[1] > 0 ? m.grid[1] : 1;
            for (std::size_t iq = 0; iq < nq; ++iq) {
                const int i = int(iq) / n2, j = int(iq) % n2;
                const int ii = (i + n1 / 2) % n1 - n1 / 2, jj = (j + n2 / 2) % n2 - n2 / 2;
                out->q1bz[2 * iq + 0] = ii * m.dq[0] + jj * m.dq[3];
                out->q1bz[2 * iq + 1] = ii * m.dq[1] + jj * m.dq[4];
            }
        }
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    }
}

bte_status bte_set_groups(bte_ctx* c, int32_t ngroups) {
    if (!c) return BTE_ERR_INPUT;
    if (ngroups < 0 || ngroups > 4096) {
        c->err = "ngroups must be in [0, 4096]";
        return BTE_ERR_INPUT;
    }
    c->ngroups = ngroups;
    c->group_valid = false;
    return BTE_OK;
}

bte_status bte_get_group_result(bte_ctx* c, int32_t group, bte_rta_result* out) {
    if (!c || !out) return BTE_ERR_INPUT;
    if (!c->group_valid) {
        c->err = "no run with replica groups since the last bte_set_groups";
        return BTE_ERR_STATE;
    }
    if (group < 0 || group >= c->group_n) {
        c->err = "group index out of range";
        return BTE_ERR_INPUT;
    }
    try {
        const std::size_t nk = std::size_t(c->group_nbx) * std::size_t(c->group_nbins);
        const double* raw = c->group_raw.data() + std::size_t(group) * nk * 3;
        const double G = double(c->group_n);
        // the group holds 1/G of the run's particles: x G estimates the whole run
        const bool want[3] = {out->gz || out->temperature, out->gz_jx || out->jx, out->gz_jy || out->jy};
        std::vector<double> v[3];
        for (int q = 0; q < 3; ++q) {
            if (!want[q]) continue;
            v[q].resize(nk);
            for (std::size_t k = 0; k < nk; ++k) v[q][k] = raw[3 * k + std::size_t(q)] * G;
        }
        std::vector<double>& gz = v[0];
        std::vector<double>& jx = v[1];
        std::vector<double>& jy = v[2];
        out->nboxes = c->group_nbx;
        out->nbins = c->group_nbins;
        out->Eeff = c->group_Eeff;
        out->energy_rate = c->gens.total_energy;
        out->events = out->wall_hits = out->crossings = out->absorbed = 0;
        out->specular_hits = out->tally_updates = out->translations = 0;
        out->kernel_ms = 0.;
        if (out->gz) std::copy(gz.begin(), gz.end(), out->gz);
        if (out->gz_jx) std::copy(jx.begin(), jx.end(), out->gz_jx);
        if (out->gz_jy) std::copy(jy.begin(), jy.end(), out->gz_jy);
        bte::rta_post(c, &c->group_params, c->group_nbx, c->group_nbins, c->group_Eeff, c->group_step, gz, jx, jy,
                      out);
        return BTE_OK;
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_INPUT;
    }
}

bte_status bte_query_sizes(const bte_ctx* c, const bte_rta_params* p, int32_t* nboxes,
                           int32_t* nbins, int64_t* nmodes) {
    if (!c || !p) return BTE_ERR_INPUT;
    if (nboxes) *nboxes = int32_t(c->geom.boxes.size());
    if (nbins) *nbins = p->dt > 0 ? int32_t(std::floor(p->maxtime / p->dt + 1.0e-6)) : 0;
    if (nmodes) *nmodes = int64_t(c->modes.n());
    return BTE_OK;
}

bte_status bte_rta_run(bte_ctx* c, const bte_rta_params* p, bte_rta_result* out) {
    if (!c || !out) return BTE_ERR_INPUT;
    try {
        bte::prepare_run(c, p);
        const bte::HostModes& m = c->modes;
        const bte::HostGeometry& g = c->geom;
        // time grid, src/RTA_MC2D.cpp:2118-2124
        const std::size_t ntime = std::size_t(std::floor(p->maxtime / p->dt + 1.0e-6)) + 1;
        if (ntime < 2) throw Error(BTE_ERR_INPUT, "maxtime shorter than one time bin");
        const double maxtime = double(ntime - 1) * p->dt;
        const double step = (maxtime - 0.0) / double(ntime - 1);
        {
            const std::vector<double> tg = bte::time_grid_with_widths(int(ntime), maxtime, step);
            c->h_time.assign(tg.begin(), tg.begin() + std::ptrdiff_t(ntime));
            c->d_time.upload(tg, c->stream);
        }
        const int nbins = int(ntime - 1);
        const int nbx = int(g.boxes.size());
        const std::size_t nk = std::size_t(nbx) * std::size_t(nbins);
        const bool replay = p->mode == BTE_MODE_REPLAY;
        c->group_valid = false;
        if (c->ngroups > 1 && (replay || !g.rect_grid))
            throw Error(BTE_ERR_INPUT, "replica groups need production mode on boxes that tile a grid");
        const int ngroups = c->ngroups > 1 ? c->ngroups : 1;
        const std::size_t tally_bytes =
            replay ? nk * 6 * sizeof(unsigned long long) : nk * 3 * sizeof(double) * std::size_t(ngroups);
        c->d_tally.alloc(tally_bytes);
        c->d_counters.alloc(16 * sizeof(unsigned long long));
        c->d_err.alloc(4 * sizeof(int));
        c->d_work.alloc(sizeof(unsigned long long));
        ck(cudaMemsetAsync(c->d_tally.p, 0, tally_bytes, c->stream), "memset");
        ck(cudaMemsetAsync(c->d_counters.p, 0, 16 * sizeof(unsigned long long), c->stream), "memset");
        ck(cudaMemsetAsync(c->d_err.p, 0, 4 * sizeof(int), c->stream), "memset");
        ck(cudaMemsetAsync(c->d_work.p, 0, sizeof(unsigned long long), c->stream), "memset");

        // Eeff (src/RTA_MC2D.cpp:2177) and the particle range
        double Eeff;
        long long total;
        if (p->source == BTE_SOURCE_WALLS) {
            Eeff = c->gens.total_energy / double(p->nparticles);
            total = p->nparticles;
        } else {
            Eeff = c->gen_Eeff;
            total = c->gens.init_first.back();
        }
        long long pbeg = std::max<long long>(0, p->particle_begin);
        long long pend = p->particle_end > 0 ? std::min<long long>(p->particle_end, total) : total;
        if (pend < pbeg) pend = pbeg;

        bte::DevTables T{};
        T.n = int(m.n());
        T.nb = m.nb;
        T.vxc = c->d_vxc.as<double>();
        T.vyc = c->d_vyc.as<double>();
        T.w = c->d_w.as<double>();
        T.tau = c->d_tau.as<double>();
        T.resample_cdf = c->d_rcdf.as<double>();
        T.resample_prob = c->d_rprob.as<float>();
        T.resample_alt = c->d_ralt.as<int>();
        T.nboxes = nbx;
        T.boxes = c->d_boxes.as<bte::GBox>();
        T.hull = c->d_hull.as<bte::V2>();
        T.borders = c->d_borders.as<bte::GBorder>();
        T.contacts = c->d_contacts.as<bte::GContact>();
        T.cseg = c->d_cseg.as<bte::V2>();
        T.translation = c->d_transl.as<bte::V2>();
        T.tfast = c->have_tfast ? c->d_tfast.as<bte::TransFast>() : nullptr;
        T.tfast_rng = c->d_tfast_rng.as<int2>();
        T.tfast_u = c->d_tfast_u.as<bte::V2>();
        T.nclass = c->nclass;
        T.row_ptr = c->d_row_ptr.as<long long>();
        T.lcol = c->d_lcol.as<int>();
        T.lcdf = c->d_lcdf.as<double>();
        T.lalias = c->d_lalias.as<int4>();
        T.mirror = c->have_mirror ? c->d_mirror.as<int>() : nullptr;
        T.box_mat = c->nmat > 0 ? c->d_boxmat.as<int>() : nullptr;
        bte::set_crystal_tables(c, T);
        T.ntime = int(ntime);
        T.timegrid = c->d_time.as<double>();
        T.maxtime = maxtime;
        T.inv_dt = 1.0 / step;
        T.source = p->source;
        T.ngen = p->source == BTE_SOURCE_WALLS ? int(c->gens.walls.size()) : int(c->gens.init_box.size());
        T.gen_cdf = c->d_gcdf.as<double>();
        T.gen_prob = c->d_gprob.as<float>();
        T.gen_alt = c->d_galt.as<int>();
        T.walls = c->d_walls.as<bte::WallGenDev>();
        T.wall_cum = c->d_wcum.as<double>();
        T.init_first = c->d_ifirst.as<long long>();
        T.init_box = c->d_ibox.as<int>();
        T.init_sign = c->d_isign.as<int>();
        T.seed = p->seed;
        T.flight_cap = p->flight_cap > 0 ? p->flight_cap : bte::EVENT_CAP;
        T.checks = (p->flags & BTE_FLAG_CHECKS) ? 1 : 0;
        T.ballistic = p->ballistic;
        T.specularity = p->specularity;
        T.pbegin = pbeg;
        T.pend = pend;
        T.nbins = nbins;
        T.ngroups = ngroups;
        T.group_stride = (long long)(nk * 3);
        // spectral decomposition: per-mode time at the selected boxes
        const std::size_t nloc = c->spec_boxes.size();
        const std::size_t spec_vals = nloc * std::size_t(nbins) * m.n();
        if (nloc > 0) {
            std::vector<int> loc(std::size_t(nbx), -1);
            for (std::size_t i = 0; i < nloc; ++i) loc[std::size_t(c->spec_boxes[i])] = int(i);
            c->d_specloc.upload(loc, c->stream);
            const std::size_t bytes = spec_vals * (replay ? 2 * sizeof(unsigned long long) : sizeof(double));
            c->d_spec.alloc(bytes);
            ck(cudaMemsetAsync(c->d_spec.p, 0, bytes, c->stream), "memset");
            T.spec_loc = c->d_specloc.as<int>();
            T.spec = c->d_spec.as<double>();
            T.spec_ex = c->d_spec.as<unsigned long long>();
        }
        c->spec_valid = false;

        auto* counters = c->d_counters.as<unsigned long long>();
        auto* err = c->d_err.as<int>();
        ck(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
        if (replay) {
            bte::launch_replay(T, c->d_tally.as<unsigned long long>(), counters, err, c->nsm, c->stream);
        } else if (g.rect_grid && c->ncrys == 0) {
            bte::GridArgs A{};
            A.G.nx = g.gnx;
            A.G.ny = g.gny;
            A.G.gx = c->d_gx.as<double>();
            A.G.gy = c->d_gy.as<double>();
            A.G.cell = c->d_gcell.as<int>();
            A.boxcell = c->d_boxcell.as<int2>();
            A.mv = c->d_mv.as<bte::ModeVel>();
            const bte::V2 want[4] = {bte::v2(1, 0), bte::v2(-1, 0), bte::v2(0, 1), bte::v2(0, -1)};
            for (int w = 0; w < 4; ++w) {
                A.cls[w] = -1;
                for (std::size_t k = 0; k < g.normals.size(); ++k)
                    if (g.normals[k].x == want[w].x && g.normals[k].y == want[w].y) A.cls[w] = int(k);
            }
            if (!bte::launch_prod_grid(T, A, c->d_tally.as<double>(), counters, err,
                                       c->d_work.as<unsigned long long>(), c->tune, c->nsm, c->stream))
                throw Error(BTE_ERR_INPUT, "tuning not supported by the grid kernel");
        } else if (p->flags & BTE_FLAG_GENERAL) {
            bte::launch_prod_general(T, c->d_tally.as<double>(), counters, err,
                                     c->d_work.as<unsigned long long>(), c->nsm, c->stream);
        } else {
            const bte::PolyArgs A{c->d_pborders.as<bte::PolyBorder>(), c->d_ppieces.as<bte::PolyPiece>(),
                                  c->d_mv.as<bte::ModeVel>(), c->d_invden.as<double>(),
                                  c->d_prect.as<bte::PolyRect>(),
                                  c->ncrys > 0 ? c->d_dmm_row.as<long long>() : nullptr,
                                  c->ncrys > 0 ? c->d_dmm_ent.as<bte::DmmEnt>() : nullptr};
            if (!bte::launch_prod_poly(T, A, c->d_tally.as<double>(), counters, err,
                                       c->d_work.as<unsigned long long>(), c->nsm, c->stream))
                throw Error(BTE_ERR_CUDA, "polygon kernel does not fit on the device");
        }
        ck(cudaGetLastError(), "kernel launch");
        ck(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
        std::vector<unsigned long long> hc(16);
        int herr[4];
        std::vector<unsigned long long> hex;
        const double* htal = nullptr;  // the production tally, in the page-locked readback buffer
        if (replay) {
            hex.resize(nk * 6);
            ck(cudaMemcpyAsync(hex.data(), c->d_tally.p, tally_bytes, cudaMemcpyDeviceToHost, c->stream), "d2h");
        } else {
            c->h_tally.reserve(tally_bytes);
            htal = static_cast<const double*>(c->h_tally.p);
            ck(cudaMemcpyAsync(c->h_tally.p, c->d_tally.p, tally_bytes, cudaMemcpyDeviceToHost, c->stream), "d2h");
        }
        ck(cudaMemcpyAsync(hc.data(), counters, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream), "d2h");
        ck(cudaMemcpyAsync(herr, err, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream), "d2h");
        std::vector<unsigned long long> hspec;
        if (nloc > 0) {
            hspec.resize(replay ? 2 * spec_vals : spec_vals);
            ck(cudaMemcpyAsync(hspec.data(), c->d_spec.p, hspec.size() * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, c->stream), "d2h");
        }
        sync(c);
        if (nloc > 0) {
            c->spec_raw.resize(spec_vals);
            for (std::size_t i = 0; i < spec_vals; ++i) {
                if (replay) {
                    const __int128 v = (__int128)(((unsigned __int128)hspec[2 * i] << 64) | hspec[2 * i + 1]);
                    c->spec_raw[i] = double(v) / bte::FIX_SCALE;
                } else {
                    std::memcpy(&c->spec_raw[i], &hspec[i], sizeof(double));
                }
            }
            c->spec_nbins = nbins;
            c->spec_T0 = p->T0;
            c->spec_steady = false;
            c->spec_cnt.clear();
            c->spec_valid = true;
        }
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
        out->kernel_ms = ms;
        if (herr[0] != 0) {
            const long long pid = (long long)herr[1] | ((long long)herr[2] << 31);
            char msg[160];
            std::snprintf(msg, sizeof msg, "particle %lld: %s", pid,
                          herr[0] == BTE_ERR_VALUE ? "invalid scattering rate"
                          : herr[0] == BTE_ERR_LIMIT ? "iteration cap reached"
                          : herr[0] == BTE_ERR_CHECK ? "index check failed"
                                                      : "geometry error");
            throw Error(bte_status(herr[0]), msg);
        }
        std::vector<double> sum;
        if (ngroups > 1) {
            // keep the groups; the run's outputs are their sum, in group order
            c->group_raw.assign(htal, htal + nk * 3 * std::size_t(ngroups));
            sum.assign(nk * 3, 0.);
            for (int gi = 0; gi < ngroups; ++gi)
                for (std::size_t k = 0; k < nk * 3; ++k) sum[k] += htal[std::size_t(gi) * nk * 3 + k];
            htal = sum.data();
            c->group_n = ngroups;
            c->group_nbx = nbx;
            c->group_nbins = nbins;
            c->group_Eeff = Eeff;
            c->group_step = step;
            c->group_params = *p;
            c->group_valid = true;
        }
        // raw tallies
        std::vector<double>& gz = c->post_gz;
        std::vector<double>& jx = c->post_jx;
        std::vector<double>& jy = c->post_jy;
        gz.resize(nk);
        jx.resize(nk);
        jy.resize(nk);
        if (replay) {
            for (std::size_t k = 0; k < nk; ++k) {
                double* dst[3] = {&gz[k], &jx[k], &jy[k]};
                for (int q = 0; q < 3; ++q) {
                    const unsigned long long hi = hex[6 * k + 2 * q], lo = hex[6 * k + 2 * q + 1];
                    const __int128 v = (__int128)(((unsigned __int128)hi << 64) | lo);
                    *dst[q] = double(v) / bte::FIX_SCALE;
                }
            }
            if (out->exact) std::memcpy(out->exact, hex.data(), nk * 6 * sizeof(long long));
        } else {
            for (std::size_t k = 0; k < nk; ++k) {
                gz[k] = htal[3 * k];
                jx[k] = htal[3 * k + 1];
                jy[k] = htal[3 * k + 2];
            }
        }
        out->nboxes = nbx;
        out->nbins = nbins;
        out->Eeff = Eeff;
        c->spec_Eeff = Eeff;
        out->energy_rate = c->gens.total_energy;
        out->events = (int64_t)hc[0];
        out->wall_hits = (int64_t)hc[1];
        out->crossings = (int64_t)hc[2];
        out->absorbed = (int64_t)hc[3];
        out->specular_hits = (int64_t)hc[4];
        out->tally_updates = (int64_t)hc[7];
        out->translations = (int64_t)hc[8];
        out->interface_hits = (int64_t)hc[11];
        out->interface_transmissions = (int64_t)hc[12];
        if (out->gz) std::copy(gz.begin(), gz.end(), out->gz);
        if (out->gz_jx) std::copy(jx.begin(), jx.end(), out->gz_jx);
        if (out->gz_jy) std::copy(jy.begin(), jy.end(), out->gz_jy);
        bte::rta_post(c, p, nbx, nbins, Eeff, step, gz, jx, jy, out);
        return BTE_OK;
    } catch (const Error& e) {
        return fail(c, e);
    } catch (const std::exception& e) {
        c->err = e.what();
        return BTE_ERR_CUDA;
    }
}

// ------------------------------------------------------------------ debug
// Host-only views of the tables for the CPU tests (no GPU needed).

long long btegpu_debug_geometry(const bte_geometry* gm, double* out, long long cap) {
    try {
        bte::HostGeometry g = bte::build_geometry(gm);
        long long k = 0;
        auto put = [&](double x) {
            if (k < cap) out[k] = x;
            k++;
        };
        for (std::size_t b = 0; b < g.boxes.size(); ++b) {
            const bte::GBox& B = g.boxes[b];
            put(double(B.nborders));
            for (int i = 0; i < B.nborders; ++i) {
                const bte::GBorder& br = g.borders[std::size_t(B.border_off + i)];
                put(br.p1.x); put(br.p1.y); put(br.p2.x); put(br.p2.y);
                put(br.np.x); put(br.np.y);
            }
            put(double(B.ncontacts));
            for (int i = 0; i < B.ncontacts; ++i) {
                const bte::GContact& ct = g.contacts[std::size_t(B.contact_off + i)];
                put(double(ct.id)); put(ct.np.x); put(ct.np.y);
            }
            put(B.center.x); put(B.center.y); put(B.area);
        }
        return k;
    } catch (const std::exception&) {
        return -1;
    }
}

int btegpu_debug_grid(const bte_geometry* gm, int* nx, int* ny) {
    try {
        bte::HostGeometry g = bte::build_geometry(gm);
        *nx = g.gnx;
        *ny = g.gny;
        return g.rect_grid ? 1 : 0;
    } catch (const std::exception&) {
        return -1;
    }
}

long long btegpu_debug_lambert(const bte_mode_table* mt, const bte_geometry* gm, long long* nnz_per_class,
                               int maxclass) {
    try {
        bte::HostModes m = bte::build_modes(mt);
        bte::HostGeometry g = bte::build_geometry(gm);
        bte::LambertTable L = bte::build_lambert(m, g, hw_threads());
        const std::size_t n = m.n();
        for (int c = 0; c < L.nclass && c < maxclass; ++c)
            nnz_per_class[c] = L.row_ptr[std::size_t(c) * (n + 1) + n] - L.row_ptr[std::size_t(c) * (n + 1)];
        return (long long)L.col.size();
    } catch (const std::exception&) {
        return -1;
    }
}

long long btegpu_debug_frame(double time, double Eeff, const double* temps, const int* H, int nboxes,
                             int nmodes, char* out, long long cap) {
    std::vector<double> t(temps, temps + nboxes);
    const std::string f = bte::berta_frame(time, Eeff, t, H, std::size_t(nboxes), std::size_t(nmodes));
    if ((long long)f.size() <= cap) std::memcpy(out, f.data(), f.size());
    return (long long)f.size();
}

int btegpu_debug_log(const double* x, double* y, long long n) {
    for (long long i = 0; i < n; ++i) y[i] = bte::bte_log(x[i]);
    return 0;
}

}  // extern "C"

// ------------------------------------------------------------------ prepared runs
// Read-only view of a context whose tables an earlier bte_rta_run built for
// the same parameters: fills the kernel arguments without allocating or
// uploading anything.  Used by the allocation-free entry point (noalloc.cu).
namespace bte {

bte_status prepared_grid_run(bte_ctx* c, const bte_rta_params* p, PreparedRun* r, std::string* why) {
    if (!c || !p || !r) {
        *why = "null argument";
        return BTE_ERR_INPUT;
    }
    if (p->mode != BTE_MODE_PRODUCTION) {
        *why = "the allocation-free run is the production grid kernel: mode must be BTE_MODE_PRODUCTION";
        return BTE_ERR_INPUT;
    }
    if (!(p->dt > 0.) || !(p->maxtime > 0.) || p->nparticles < 1 ||
        !(p->specularity >= 0. && p->specularity <= 1.) || !(p->T0 > 0.)) {
        *why = "invalid run parameters";
        return BTE_ERR_INPUT;
    }
    if (!c->have_modes || !c->have_geom || !c->modes_dev || !c->geom_dev || !c->lambert_dev) {
        *why = "context not prepared: load the tables and run bte_rta_run once with these parameters";
        return BTE_ERR_STATE;
    }
    const HostGeometry& g = c->geom;
    const HostModes& m = c->modes;
    if (!g.rect_grid) {
        *why = "the allocation-free run needs boxes that tile an axis-aligned grid";
        return BTE_ERR_INPUT;
    }
    if (c->resample_T0 != (c->nmat > 0 ? -2.0 : p->T0) || c->gen_key_source != p->source ||
        (p->source == BTE_SOURCE_INITIAL &&
         (c->gen_key_n != p->nparticles || c->gen_key_seed != p->seed))) {
        *why = "context prepared for other parameters: run bte_rta_run once with this T0, source "
               "(and, for the initial source, N and seed) first";
        return BTE_ERR_STATE;
    }
    if (p->specularity > 0. && !c->have_mirror) {
        *why = "specular walls need an axis-aligned q grid with mirror images";
        return BTE_ERR_INPUT;
    }
    const std::size_t ntime = std::size_t(std::floor(p->maxtime / p->dt + 1.0e-6)) + 1;
    if (ntime < 2) {
        *why = "maxtime shorter than one time bin";
        return BTE_ERR_INPUT;
    }
    r->ntime = int(ntime);
    r->nbins = int(ntime - 1);
    r->maxtime = double(ntime - 1) * p->dt;
    r->step = (r->maxtime - 0.0) / double(ntime - 1);
    r->nboxes = int(g.boxes.size());
    long long total;
    if (p->source == BTE_SOURCE_WALLS) {
        r->Eeff = c->gens.total_energy / double(p->nparticles);
        total = p->nparticles;
    } else {
        r->Eeff = c->gen_Eeff;
        total = c->gens.init_first.back();
    }
    r->energy = c->gens.total_energy;
    long long pbeg = std::max<long long>(0, p->particle_begin);
    long long pend = p->particle_end > 0 ? std::min<long long>(p->particle_end, total) : total;
    if (pend < pbeg) pend = pbeg;
    DevTables& T = r->T;
    T = DevTables{};
    T.n = int(m.n());
    T.nb = m.nb;
    T.vxc = c->d_vxc.as<double>();
    T.vyc = c->d_vyc.as<double>();
    T.w = c->d_w.as<double>();
    T.tau = c->d_tau.as<double>();
    T.resample_cdf = c->d_rcdf.as<double>();
    T.resample_prob = c->d_rprob.as<float>();
    T.resample_alt = c->d_ralt.as<int>();
    T.nboxes = r->nboxes;
    T.boxes = c->d_boxes.as<GBox>();
    T.hull = c->d_hull.as<V2>();
    T.borders = c->d_borders.as<GBorder>();
    T.contacts = c->d_contacts.as<GContact>();
    T.cseg = c->d_cseg.as<V2>();
    T.translation = c->d_transl.as<V2>();
    T.tfast = c->have_tfast ? c->d_tfast.as<TransFast>() : nullptr;
    T.tfast_rng = c->d_tfast_rng.as<int2>();
    T.tfast_u = c->d_tfast_u.as<V2>();
    T.nclass = c->nclass;
    T.row_ptr = c->d_row_ptr.as<long long>();
    T.lcol = c->d_lcol.as<int>();
    T.lcdf = c->d_lcdf.as<double>();
    T.lalias = c->d_lalias.as<int4>();
    T.mirror = c->have_mirror ? c->d_mirror.as<int>() : nullptr;
    T.box_mat = c->nmat > 0 ? c->d_boxmat.as<int>() : nullptr;
    set_crystal_tables(c, T);
    T.ntime = r->ntime;
    T.timegrid = nullptr;  // set by the caller
    T.maxtime = r->maxtime;
    T.inv_dt = 1.0 / r->step;
    T.source = p->source;
    T.ngen = p->source == BTE_SOURCE_WALLS ? int(c->gens.walls.size()) : int(c->gens.init_box.size());
    T.gen_cdf = c->d_gcdf.as<double>();
    T.gen_prob = c->d_gprob.as<float>();
    T.gen_alt = c->d_galt.as<int>();
    T.walls = c->d_walls.as<WallGenDev>();
    T.wall_cum = c->d_wcum.as<double>();
    T.init_first = c->d_ifirst.as<long long>();
    T.init_box = c->d_ibox.as<int>();
    T.init_sign = c->d_isign.as<int>();
    T.seed = p->seed;
    T.flight_cap = p->flight_cap > 0 ? p->flight_cap : EVENT_CAP;
    T.checks = (p->flags & BTE_FLAG_CHECKS) ? 1 : 0;
    T.ballistic = p->ballistic;
    T.specularity = p->specularity;
    T.pbegin = pbeg;
    T.pend = pend;
    T.nbins = r->nbins;
    GridArgs& A = r->A;
    A = GridArgs{};
    A.G.nx = g.gnx;
    A.G.ny = g.gny;
    A.G.gx = c->d_gx.as<double>();
    A.G.gy = c->d_gy.as<double>();
    A.G.cell = c->d_gcell.as<int>();
    A.boxcell = c->d_boxcell.as<int2>();
    A.mv = c->d_mv.as<ModeVel>();
    const V2 want[4] = {v2(1, 0), v2(-1, 0), v2(0, 1), v2(0, -1)};
    for (int w = 0; w < 4; ++w) {
        A.cls[w] = -1;
        for (std::size_t k = 0; k < g.normals.size(); ++k)
            if (g.normals[k].x == want[w].x && g.normals[k].y == want[w].y) A.cls[w] = int(k);
    }
    r->stream = c->stream;
    r->ev0 = c->ev0;
    r->ev1 = c->ev1;
    r->device = c->device;
    r->nsm = c->nsm;
    r->tune = c->tune;
    return BTE_OK;
}

std::vector<double> time_grid_with_widths(int ntime, double maxtime, double step) {
    std::vector<double> g(std::size_t(2 * ntime - 1));
    for (int i = 0; i < ntime; ++i) g[std::size_t(i)] = (i == ntime - 1) ? maxtime : 0.0 + double(i) * step;
    for (int i = 0; i + 1 < ntime; ++i) g[std::size_t(ntime + i)] = g[std::size_t(i + 1)] - g[std::size_t(i)];
    return g;
}

void fill_static_tables(bte_ctx* c, DevTables& T) {
    T.n = int(c->modes.n());
    T.nb = c->modes.nb;
    T.vxc = c->d_vxc.as<double>();
    T.vyc = c->d_vyc.as<double>();
    T.w = c->d_w.as<double>();
    T.tau = c->d_tau.as<double>();
    T.resample_cdf = c->d_rcdf.as<double>();
    T.resample_prob = c->d_rprob.as<float>();
    T.resample_alt = c->d_ralt.as<int>();
    T.nboxes = int(c->geom.boxes.size());
    T.boxes = c->d_boxes.as<GBox>();
    T.hull = c->d_hull.as<V2>();
    T.borders = c->d_borders.as<GBorder>();
    T.contacts = c->d_contacts.as<GContact>();
    T.cseg = c->d_cseg.as<V2>();
    T.translation = c->d_transl.as<V2>();
    T.tfast = c->have_tfast ? c->d_tfast.as<TransFast>() : nullptr;
    T.tfast_rng = c->d_tfast_rng.as<int2>();
    T.tfast_u = c->d_tfast_u.as<V2>();
    T.nclass = c->nclass;
    T.row_ptr = c->d_row_ptr.as<long long>();
    T.lcol = c->d_lcol.as<int>();
    T.lcdf = c->d_lcdf.as<double>();
    T.lalias = c->d_lalias.as<int4>();
    T.mirror = c->have_mirror ? c->d_mirror.as<int>() : nullptr;
    T.box_mat = c->nmat > 0 ? c->d_boxmat.as<int>() : nullptr;
    set_crystal_tables(c, T);
}

// The interface tables of crystals joined by mismatch interfaces (null
// with one crystal).
void set_crystal_tables(const bte_ctx* c, DevTables& T) {
    const bool crys = c->ncrys > 0 && c->dmm_dev;
    T.contact_dmm = crys ? c->d_cdmm.as<int>() : nullptr;
    T.dmm_row = crys ? c->d_dmm_row.as<long long>() : nullptr;
    T.dmm_ent = crys ? c->d_dmm_ent.as<DmmEnt>() : nullptr;
    T.crys_off = crys ? c->d_crysoff.as<int>() : nullptr;
}

double crystal_thickness(const bte_ctx* c, int k) {
    return c->crys_thick.empty() ? c->geom.thickness : c->crys_thick[std::size_t(k)];
}

double box_thickness(const bte_ctx* c, int b) {
    return c->ncrys > 0 ? crystal_thickness(c, c->geom.mat[std::size_t(b)]) : c->geom.thickness;
}

double box_T0(const bte_ctx* c, int b, double T0) {
    return c->nmat > 0 ? c->mat_T0[std::size_t(c->geom.mat[std::size_t(b)])] : T0;
}

void set_ctx_error(bte_ctx* c, const std::string& m) {
    if (c) c->err = m;
}

}  // namespace bte
