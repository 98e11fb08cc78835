// ctx.hpp - the engine context shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <thread>
#include <vector>

#include "../../include/btegpu.h"
#include "kernels.h"
#include "tables.hpp"

namespace bte {

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw Error(BTE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Owned device allocation.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t n) {
        if (n == 0) n = 16;
        if (p && bytes >= n) return;
        release();
        ck(cudaMalloc(&p, n), "cudaMalloc");
        bytes = n;
    }
    template <class T>
    void upload(const std::vector<T>& v, cudaStream_t s) {
        alloc(v.size() * sizeof(T));
        if (!v.empty()) ck(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

// Page-locked host memory, grown as needed and kept: device copies from or
// into it run at full bus speed and need no staging.
struct Pinned {
    void* p = nullptr;
    size_t bytes = 0;
    Pinned() = default;
    Pinned(const Pinned&) = delete;
    Pinned& operator=(const Pinned&) = delete;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
    void reserve(size_t n) {
        if (bytes >= n) return;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        ck(cudaMallocHost(&p, n), "cudaMallocHost");
        bytes = n;
    }
};


inline int hw_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n ? int(n < 64u ? n : 64u) : 4;
}

struct BertaState;   // berta.cu
struct SteadyState;  // steady.cu

}  // namespace bte

struct bte_ctx {
    int device = 0;
    int nsm = 0;
    int verbose = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    bte::ProdTuning tune{0, 0, 0, 0};

    bool have_modes = false, have_geom = false;
    long long tables_version = 0;  // bumped by every load of modes or geometry
    bte::HostModes modes;
    bte::HostGeometry geom;

    // static tables
    bool modes_dev = false, geom_dev = false, lambert_dev = false;
    bte::DBuf d_vxc, d_vyc, d_w, d_tau, d_mv;
    bte::DBuf d_boxes, d_hull, d_borders, d_contacts, d_cseg, d_transl;
    bte::DBuf d_tfast, d_tfast_rng, d_tfast_u;  // translations without a search
    bool have_tfast = false;
    bte::DBuf d_invden;                           // 1 / (n.v) per normal class and mode
    bte::DBuf d_prect;                            // PolyRect per box
    // several crystals (bte_load_mode_tables): their own mode tables, the
    // concatenation in `modes` (global mode off[k] + j), the rate sets of the
    // materials machinery masked to each crystal, mismatch tables per interface
    int ncrys = 0;
    std::vector<double> crys_thick;  // per crystal (empty: the geometry's thickness)
    std::vector<bte::HostModes> crys;
    std::vector<std::size_t> crys_off;
    std::vector<bte::PolyPiece> pieces_host;      // the polygon path's pieces (pads: mismatch tables)
    std::vector<bte::PolyBorder> pborders_host;
    bool dmm_dev = false;
    int ndmm = 0;
    bte::DBuf d_dmm_row, d_dmm_ent;
    bte::DBuf d_cdmm, d_crysoff;  // per contact its interface table (-1: none); crystals' first modes
    bte::DBuf d_gx, d_gy, d_gcell, d_boxcell;
    bte::DBuf d_pborders, d_ppieces;  // convex-polygon path (geometries that are not a grid)
    bte::DBuf d_row_ptr, d_lcol, d_lcdf, d_lalias, d_mirror;
    int nclass = 0;
    bool have_mirror = false;
    // materials of batched runs (0: the mode table's own rates at the run's T0)
    int nmat = 0;
    std::vector<double> mat_w, mat_T0, mat_share;
    std::vector<double> mat_energy;   // walls-source energy rate per material (with shares)
    // C_v per material (or at the run's T0 without materials), kept for the
    // temperature conversion of successive runs: valid for these tables,
    // these material temperatures and that T0
    std::vector<double> cv_cache;
    std::vector<double> cv_T0s;
    long long cv_version = -1;
    bool shares_dirty = false;        // shares changed since the wall weights were set
    bte::DBuf d_boxmat;
    // per-T0 (or per-material) resampling
    double resample_T0 = -1;
    bte::DBuf d_rcdf, d_rprob, d_ralt;
    // generators
    int gen_key_source = -1;
    long long gen_key_n = -1;
    unsigned long long gen_key_seed = 0;
    bte::Generators gens;
    double gen_Eeff = 0;
    bte::DBuf d_gcdf, d_gprob, d_galt, d_walls, d_wcum, d_ifirst, d_ibox, d_isign;
    // spectral decomposition: selected boxes, ticks, the last run's tally
    std::vector<int> spec_boxes;
    int spec_nomega = 0;
    bte::DBuf d_specloc, d_spec;
    std::vector<double> spec_raw;      // [nloc][nbins][n] of the last run
    bte::DBuf d_speccnt;
    std::vector<long long> spec_cnt;   // steady runs: signed segments [nloc][n]
    bool spec_steady = false;
    int spec_nbins = 0;
    double spec_Eeff = 0., spec_T0 = 0.;
    bool spec_valid = false;
    // replica groups (bte_set_groups): the last grid-kernel run's raw
    // tallies per group, [group][box][bin][3], with what their outputs need
    int ngroups = 0;
    bool group_valid = false;
    int group_n = 0, group_nbx = 0, group_nbins = 0;
    double group_Eeff = 0., group_step = 0.;
    bte_rta_params group_params{};
    std::vector<double> group_raw;
    // the production tally's readback (page-locked) and the raw tallies
    // handed to the post-processing, kept across runs
    bte::Pinned h_tally;
    std::vector<double> post_gz, post_jx, post_jy;
    // run buffers
    bte::DBuf d_time, d_tally, d_counters, d_err, d_work;
    std::vector<double> h_time;
    // beyond-RTA (berta.cu)
    bte::BertaState* berta = nullptr;
    // periodic / gradient steady state (steady.cu)
    bte::SteadyState* steady = nullptr;
};

namespace bte {
// Device tables shared by every run type (capi.cu).
void ensure_static(bte_ctx* c);
void ensure_resample(bte_ctx* c, double T0);
void sync(bte_ctx* c);
void destroy_berta(bte_ctx* c);
// Forget the loaded propagators (they refer to the previous mode table).
void reset_propagators(bte_ctx* c);
void destroy_steady(bte_ctx* c);
// T0 of box b's material (the run's T0 without materials).
double box_T0(const bte_ctx* c, int b, double T0);
// Validation and tables of one RTA run (capi.cu).
void prepare_run(bte_ctx* c, const bte_rta_params* p);
// Kernel arguments of a prepared grid-path run (capi.cu); BTE_OK or a code
// with the reason in *why.
bte_status prepared_grid_run(bte_ctx* c, const bte_rta_params* p, PreparedRun* r, std::string* why);
// Mode, geometry and Lambert tables of a context into the kernel tables.
void fill_static_tables(bte_ctx* c, DevTables& T);
// The interface tables of several crystals into the kernel tables.
void set_crystal_tables(const bte_ctx* c, DevTables& T);
// Thickness of crystal k's boxes (the geometry's without crystal values)
// and of box b.
double crystal_thickness(const bte_ctx* c, int k);
double box_thickness(const bte_ctx* c, int b);
// The ntime points of the time grid (src/RTA_MC2D.cpp:2118-2124: i * step,
// the last exactly maxtime) followed by the ntime - 1 bin widths, the
// layout DevTables::timegrid points to.
std::vector<double> time_grid_with_widths(int ntime, double maxtime, double step);
}  // namespace bte
