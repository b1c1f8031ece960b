// engine.cu - pool management and kernel launches of the packed multi-system LJ MD engine; the
// kernels are in dev_common.cuh (shared device helpers), dev_step.cuh (drift, list rebuild,
// force kernels), dev_cluster.cuh (cluster-list variants) and dev_step_end.cuh (kick, fused step,
// step end, bookkeeping), included below in that order.
//
// Per velocity-Verlet step every active slot goes through (one launch each, over the pool):
//   k_integrate1   a_t = F/m; x += v dt + (a_t/2) dt^2; periodic wrap; skin-displacement test;
//                  cell-relative FP32 coordinates for the mixed path
//   k_bin .. k_build  neighbour-list rebuild, each kernel a no-op for slots whose rebuild flag
//                  is clear: counting sort of atoms into cells (bin -> scan -> scatter), a
//                  per-cell id sort + gather that physically reorders the atoms by cell, then
//                  the list build at rcut + skin; k_rebuild_done clears the flags. In step graphs
//                  these sit in a conditional node that runs only when some slot rebuilds.
//   k_force_*      LJ forces and energy (FP64 half list with atomics, FP64 full list, or mixed
//                  FP32 full list)
//   k_integrate2   v += (a_t + a_tdt)/2 dt; chunk partial sums of KE (and virial on demand)
//   k_step_end     per-slot deterministic reductions, history, counters
// The mixed path's default shape replaces force + kick + the next drift by one kernel
// (k_step_mixed). Everything a step needs lives in device memory, so chunks of steps are captured
// as one CUDA graph and replayed without host round trips.
//
// Reference arithmetic (FP64 path): src/potentials/potential.rs:15-33 (NVE step),
// src/simulation_box.rs:17-42 (min-image, wrap), src/potentials/lennard_jones.rs:33-55 (pair),
// src/atoms/properties.rs:17-51 (a = F/m, KE, virial). Rounding is pinned with __d*_rn
// intrinsics so no multiply-add is fused where the reference has two roundings.
#include "engine.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace cg = cooperative_groups;

namespace pis {

static std::atomic<int64_t> g_launches{0};
int64_t Engine::launches() { return g_launches.load(); }

}  // namespace pis

#include "dev_common.cuh"
#include "dev_step.cuh"
#include "dev_cluster.cuh"
#include "dev_step_end.cuh"

namespace pis {

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
#define LAUNCH(kern, grid, block, ...)                                \
    do {                                                               \
        kern<<<(grid), (block), 0, ls_>>>(__VA_ARGS__);               \
        g_launches.fetch_add(1);                                       \
    } while (0)

Engine::Engine() {}

Engine::~Engine() {
    for (auto& kv : graphs_) {
        cudaGraphExecDestroy(kv.second.exec);
        for (auto e : kv.second.ev) cudaEventDestroy(e);
    }
    if (d_ && d_->keep) cudaFree(d_->keep);
    if (nbr_own_) cudaFree(nbr_own_);
    if (save_) cudaFree(save_);
    if (mem_) cudaFree(mem_);
    if (stream_) cudaStreamDestroy(stream_);
    if (side_) cudaStreamDestroy(side_);
    delete d_;
}

pis_status Engine::check(cudaError_t e, const char* what, std::string& err) {
    if (e == cudaSuccess) return PIS_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return PIS_ERR_NO_MEMORY;
    return PIS_ERR_CUDA;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }


static cudaError_t allow_all_mixed_tma_smem();

pis_status Engine::init(const PoolOptions& opt, std::string& err) {
    opt_ = opt;
    if (opt.max_atoms <= 0 || opt.max_slots <= 0) {
        err = "pool needs atoms and slots";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.blk != 256) {
        err = "chunk size must be 256";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.lpa != 1 && opt.lpa != 4 && opt.lpa != 8 && opt.lpa != 16 && opt.lpa != 32 &&
        !(opt.lpa == 2 && opt.cluster == 2)) {
        err = "lanes per atom must be 1, 4, 8, 16 or 32 (2 only with clusters of 2)";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    half_ = opt.list_kind == PIS_LIST_HALF ||
            (opt.list_kind == PIS_LIST_DEFAULT && opt.precision == PIS_PRECISION_FP64 && !opt.ref_order);
    if (opt.ref_order && (opt.precision != PIS_PRECISION_FP64 || half_ || opt.lpa != 1 || opt.fp64_fast)) {
        err = "reference-order forces need the FP64 path with a full list, one thread per atom, exact arithmetic";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.precision == PIS_PRECISION_MIXED && half_ &&
        (opt.lpa != 1 || opt.list_tma || opt.cell_tiles || opt.cluster || opt.build_cluster > 1)) {
        err = "the mixed-precision half list is a variant of the thread-per-atom force kernel";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.list_tma && (opt.precision != PIS_PRECISION_MIXED || opt.lpa != 1)) {
        err = "the bulk-copy list stream is a variant of the mixed, thread-per-atom force kernel";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.list_tma) {
        pis_status st0 = check(allow_all_mixed_tma_smem(), "shared-memory attribute", err);
        if (st0) return st0;
    }
    if (opt.cell_tiles && (opt.precision != PIS_PRECISION_MIXED || opt.lpa != 1 || opt.list_tma || opt.cluster)) {
        err = "neighbour-cell tiles are a variant of the mixed, thread-per-atom force kernel";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.cell_tiles) {
        cudaError_t e = allow_tile_smem<0, true>();
        if (e == cudaSuccess) e = allow_tile_smem<0, false>();
        if (e == cudaSuccess) e = allow_tile_smem<1, true>();
        if (e == cudaSuccess) e = allow_tile_smem<1, false>();
        pis_status st0 = check(e, "shared-memory attribute", err);
        if (st0) return st0;
    }
    if (opt.cluster != 0 && opt.cluster != 2 && opt.cluster != 4) {
        err = "atoms per cluster must be 2 or 4";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.cluster && (opt.precision != PIS_PRECISION_MIXED || (opt.lpa != 1 && opt.lpa != opt.cluster) ||
                        opt.list_tma)) {
        err = "the cluster list is a variant of the mixed path with one thread per cluster or one lane per member";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.build_cluster != 0 && opt.build_cluster != 1 && opt.build_cluster != 2 && opt.build_cluster != 4) {
        err = "atoms per build cluster must be 1, 2 or 4";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    // cluster table: built for the cluster-list force path, and for the per-atom list build when
    // it scans candidates per cluster (thread-per-atom layout only)
    clm_ = opt.cluster ? opt.cluster : ((opt.lpa == 1 && opt.build_cluster > 1) ? opt.build_cluster : 0);
    if (opt.max_atoms >= (int64_t)JMASK) {
        err = "a pool holds at most 2^26 - 1 atoms (neighbour entries carry a 26-bit index)";
        return PIS_ERR_UNSUPPORTED;
    }
    cap_ = opt.list_cap > 0 ? opt.list_cap : 192;
    cap_ = (cap_ + 31) / 32 * 32;  // whole row groups for every lanes-per-atom choice
    if (opt.ref_order && cap_ > 512) {
        err = "reference-order forces keep a 9-bit list slot per entry: list capacity must be at most 512";
        return PIS_ERR_UNSUPPORTED;
    }
    npad_ = (int64_t)align_up((size_t)opt.max_atoms, 32);
    if ((double)npad_ * (double)cap_ >= 4294967296.0) {
        err = "neighbour list of the pool exceeds 2^32 entries (atoms x capacity)";
        return PIS_ERR_NO_MEMORY;
    }
    max_chunks_ = (opt.max_atoms + opt.blk - 1) / opt.blk + opt.max_slots;
    int64_t max_cells = opt.max_cells > 0 ? opt.max_cells : opt.max_atoms + opt.max_slots;
    opt_.max_cells = max_cells;
    if (clm_) {
        // per slot: ceil(n / M) clusters plus at most one partial cluster per cell
        const int M = clm_;
        max_clusters_ = (opt.max_atoms + M - 1) / M + max_cells + opt.max_slots;
        clpad_ = (int64_t)align_up((size_t)max_clusters_, 32);
        // union of M members' lists: ~1.4x (M = 2) / ~1.9x (M = 4) one atom's list
        ccap_ = (int64_t)std::ceil((double)cap_ * (M == 2 ? 1.5 : 2.0));
        ccap_ = (ccap_ + 31) / 32 * 32;
        max_cchunks_ = (max_clusters_ + CL_THREADS - 1) / CL_THREADS + opt.max_slots;
        if ((double)clpad_ * (double)ccap_ >= 4294967296.0) {
            err = "cluster list of the pool exceeds 2^32 entries (clusters x capacity)";
            return PIS_ERR_NO_MEMORY;
        }
    }
    pis_status st = check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream", err);
    if (st) return st;
    st = check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "stream", err);
    if (st) return st;
    ls_ = stream_;
    // PIS_GPU_PLAIN_GRAPHS=1 in the environment selects plain step graphs for every pool of the
    // process (for profilers that cannot look inside graphs holding conditional nodes)
    const char* plain_env = std::getenv("PIS_GPU_PLAIN_GRAPHS");
    cond_rebuild_ = !opt.plain_graphs && !(plain_env && plain_env[0] && std::strcmp(plain_env, "0") != 0);

    const size_t NA = (size_t)opt.max_atoms, NC = (size_t)max_cells, NCH = (size_t)max_chunks_,
                 NS = (size_t)opt.max_slots, NCL = (size_t)max_clusters_, NCC = (size_t)max_cchunks_;
    // the per-atom list is not used (and kept minimal) when the cluster list is
    const size_t nbr_bytes = opt.cluster ? 256 : 4 * (size_t)npad_ * cap_;
    // the fused step kernel serves the mixed path's default shape (thread per atom, per-atom full
    // list, gathers from global memory, 4- or 8-entry batches)
    const bool default_shape = opt.precision == PIS_PRECISION_MIXED && opt.lpa == 1 && !opt.list_tma &&
                               !opt.cell_tiles && !opt.cluster && !clm_ && !half_ && opt.blk == 256;
    fused_ = default_shape && !opt.unfused && (opt.mix_batch == 4 || opt.mix_batch == 8);
    // grouped list layout wherever the thread-per-atom mixed force kernel reads the list
    list_groups_ = default_shape && opt.mix_batch % 4 == 0;
    struct Item {
        void** p;
        size_t bytes;
    };
    d_ = new DevPtrs();
    std::memset(d_, 0, sizeof(DevPtrs));
    std::vector<Item> items = {
        {(void**)&d_->pos[0], 32 * NA}, {(void**)&d_->pos[1], 32 * NA}, {(void**)&d_->vel[0], 32 * NA},
        {(void**)&d_->vel[1], 32 * NA}, {(void**)&d_->acc[0], 32 * NA}, {(void**)&d_->acc[1], 32 * NA},
        {(void**)&d_->id[0], 4 * NA},   {(void**)&d_->id[1], 4 * NA},   {(void**)&d_->frc, 32 * NA},
        {(void**)&d_->posb, 32 * NA},   {(void**)&d_->prel, 16 * NA}, {(void**)&d_->prelb, 16 * NA},   {(void**)&d_->cellof, 4 * NA},
        {(void**)&d_->lcell, 4 * NA},   {(void**)&d_->slotin, 4 * NA},  {(void**)&d_->perm, 4 * NA},
        {(void**)&d_->nn, 4 * NA},      {(void**)&d_->nbr, nbr_bytes},
        {(void**)&d_->cell_count, 4 * NC}, {(void**)&d_->cell_start, 4 * NC},
        {(void**)&d_->cell_sys, 4 * NC}, {(void**)&d_->blk_sys, 4 * NCH},
        {(void**)&d_->blk_first, 4 * NCH}, {(void**)&d_->sp, sizeof(SysParams) * NS},
        {(void**)&d_->st, sizeof(SysState) * NS}, {(void**)&d_->tab, sizeof(LJDev) * (size_t)opt.max_types_total},
        {(void**)&d_->pe_part, 8 * std::max(NCH * 32, NCC * 4)}, {(void**)&d_->ke_part, 8 * NCH},
        {(void**)&d_->vir_part, 72 * NCH}, {(void**)&d_->pe_hist, 8 * NS * (size_t)opt.hist},
        {(void**)&d_->ke_hist, 8 * NS * (size_t)opt.hist}, {(void**)&d_->tr_hist, 8 * NS * (size_t)opt.hist},
        {(void**)&d_->tr_part, 8 * NCH}, {(void**)&d_->kt_part, 72 * NCH},
        {(void**)&d_->ctl, 256},
        {(void**)&d_->seg_tot, sizeof(int2) * NS * (size_t)(NC / SCAN_SEG + 2)},
    };
    if (fused_) {
        items.push_back({&prel_buf_[1], 16 * NA});
        items.push_back({(void**)&d_->ring, 8 * 3 * (size_t)RING_STEPS * NCH});
    }
    // replica pools: the rebuild kernels stride over a list of the rebuilding slots' chunks and
    // cells (1.028 vs 1.078 ms per step of the 512-replica mix)
    listed_ = opt.max_slots > 1 && opt.lpa == 1 && !opt.cluster && !clm_;
    if (listed_) {
        items.push_back({(void**)&d_->rb_list, 4 * (NCH + NC)});
        int dev = 0, sms = 0;
        st = check(cudaGetDevice(&dev), "device query", err);
        if (st) return st;
        st = check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device query", err);
        if (st) return st;
        listed_grid_ = 8 * sms;  // twice the resident blocks of the 64-register build and gather kernels
    }
    const bool exact = opt.precision == PIS_PRECISION_FP64;
    if (exact) {
        items.push_back({(void**)&d_->xpe_part, 8 * XS_WORDS * NCH * 32});
        items.push_back({(void**)&d_->xke_part, 8 * XS_WORDS * NCH});
        items.push_back({(void**)&d_->xvir_part, 8 * XS_WORDS * 9 * NCH});
        items.push_back({(void**)&d_->xtr_part, 8 * XS_WORDS * NCH});
        items.push_back({(void**)&d_->xkt_part, 8 * XS_WORDS * 9 * NCH});
    }
    if (clm_) {
        items.push_back({(void**)&d_->cl_atom, 4 * NCL});
        items.push_back({(void**)&d_->cl_start, 4 * NC});
        items.push_back({(void**)&d_->cblk_sys, 4 * NCC});
        items.push_back({(void**)&d_->cblk_first, 4 * NCC});
    }
    if (clm_) {
        items.push_back({(void**)&d_->cl_nn, 4 * NCL});
        items.push_back({(void**)&d_->cl_nbr, 4 * (size_t)clpad_ * (size_t)ccap_});
    }
    size_t total = 0;
    for (auto& it : items) total += align_up(it.bytes, 256);
    st = check(cudaMalloc(&mem_, total), "device allocation", err);
    if (st) return st;
    mem_bytes_ = total;
    char* base = (char*)mem_;
    for (auto& it : items) {
        *it.p = base;
        base += align_up(it.bytes, 256);
    }
    d_->keep = nullptr;
    d_->exact_sums = exact ? 1 : 0;
    d_->wait_limit = opt.wait_limit < 0 ? MBAR_WAIT_LIMIT : (uint32_t)std::min<int64_t>(opt.wait_limit, MBAR_WAIT_LIMIT);
    d_->npad = npad_;
    d_->cap = (int32_t)cap_;
    d_->hist = opt.hist;
    d_->max_slots = opt.max_slots;
    d_->max_segs = (int32_t)(NC / SCAN_SEG + 2);
    d_->ring_stride = (int64_t)NCH;
    d_->rb_cells_off = (int64_t)NCH;
    d_->zero_forces = half_ ? 1 : 0;
    d_->full_list = half_ ? 0 : 1;
    d_->pe_stride = opt_.lpa;
    d_->lq = opt_.lpa > 1 ? opt_.lpa : (list_groups_ ? FUSED_LQ : 1);
    d_->clpad = clpad_;
    d_->ccap = (int32_t)ccap_;
    d_->clm = clm_;
    d_->cl_force = opt.cluster ? 1 : 0;
    d_->cl_lanes = (opt.cluster && opt.lpa == opt.cluster) ? opt.cluster : 1;
    prel_buf_[0] = d_->prel;
    d_->prel_out = nullptr;
    st = check(cudaMemsetAsync(mem_, 0, total, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->cell_sys, 0xff, 4 * NC, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->blk_sys, 0xff, 4 * NCH, stream_), "memset", err);
    if (st) return st;
    if (clm_) {
        st = check(cudaMemsetAsync(d_->cblk_sys, 0xff, 4 * NCC, stream_), "memset", err);
        if (st) return st;
    }
    hp_.assign(NS, SysParams{});
    slot_rlist_.assign(NS, 0.0);
    slot_rcmax_.assign(NS, 0.0);
    slot_tab_host_.assign(NS, std::vector<LJDev>());
    free_atoms_.clear();
    free_cells_.clear();
    free_atoms_[0] = NA;
    free_cells_[0] = NC;
    free_clusters_.clear();
    if (clm_) free_clusters_[0] = (int64_t)NCL;
    free_tab_.assign(opt.max_types_total, 1);
    slot_tab_size_.assign(NS, 0);
    dirty_map_ = true;
    return sync(err);
}

static bool take_range(std::map<int64_t, int64_t>& fr, int64_t len, int64_t& at) {
    for (auto it = fr.begin(); it != fr.end(); ++it) {
        if (it->second >= len) {
            at = it->first;
            int64_t rest = it->second - len;
            fr.erase(it);
            if (rest > 0) fr[at + len] = rest;
            return true;
        }
    }
    return false;
}

static void give_range(std::map<int64_t, int64_t>& fr, int64_t at, int64_t len) {
    auto it = fr.emplace(at, len).first;
    auto nx = std::next(it);
    if (nx != fr.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        fr.erase(nx);
    }
    if (it != fr.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            fr.erase(it);
        }
    }
}

// Cell grid at rcut + skin: n_d = floor(L_d / rlist) (Atoms::divide_into_cells,
// src/atoms/neighbour_list.rs:45-57, evaluated at the list radius).
static bool diagonal_box(const double* h) {
    return h[1] == 0.0 && h[2] == 0.0 && h[3] == 0.0 && h[5] == 0.0 && h[6] == 0.0 && h[7] == 0.0;
}
// nalgebra's 3x3 inverse, as the reference inverts its box (src/simulation_box.rs:13,
// src/atoms/transformations.rs:12): the adjugate over the determinant by first-row cofactors.
// m and out are row-major. Returns false for a singular matrix.
static bool inverse3_ref(const double* m, double* out) {
    const double c00 = m[4] * m[8] - m[7] * m[5];
    const double c10 = m[3] * m[8] - m[6] * m[5];
    const double c20 = m[3] * m[7] - m[6] * m[4];
    const double det = m[0] * c00 - m[1] * c10 + m[2] * c20;
    if (det == 0.0) return false;
    out[0] = c00 / det;
    out[1] = (m[2] * m[7] - m[8] * m[1]) / det;
    out[2] = (m[1] * m[5] - m[4] * m[2]) / det;
    out[3] = -c10 / det;
    out[4] = (m[0] * m[8] - m[6] * m[2]) / det;
    out[5] = (m[2] * m[3] - m[5] * m[0]) / det;
    out[6] = c20 / det;
    out[7] = (m[1] * m[6] - m[7] * m[0]) / det;
    out[8] = (m[0] * m[4] - m[3] * m[1]) / det;
    return true;
}
// Widths of the box across each pair of faces: the edges of a diagonal box; for a general box
// |det h| / |a_e x a_f| with a_d the columns (box vectors). A cell grid of n_d cells along a_d with
// width_d / n_d >= the list radius keeps every pair within that radius in neighbouring cells.
static void box_widths(const double* h, double w[3]) {
    if (diagonal_box(h)) {
        for (int a = 0; a < 3; ++a) w[a] = h[4 * a];
        return;
    }
    double col[3][3];
    for (int d = 0; d < 3; ++d)
        for (int r = 0; r < 3; ++r) col[d][r] = h[3 * r + d];
    const double vol = std::fabs(col[0][0] * (col[1][1] * col[2][2] - col[1][2] * col[2][1]) -
                                 col[1][0] * (col[0][1] * col[2][2] - col[0][2] * col[2][1]) +
                                 col[2][0] * (col[0][1] * col[1][2] - col[0][2] * col[1][1]));
    for (int d = 0; d < 3; ++d) {
        const double* e = col[(d + 1) % 3];
        const double* f = col[(d + 2) % 3];
        const double cx = e[1] * f[2] - e[2] * f[1], cy = e[2] * f[0] - e[0] * f[2], cz = e[0] * f[1] - e[1] * f[0];
        w[d] = vol / std::sqrt(cx * cx + cy * cy + cz * cz);
    }
}

static void cell_grid(const SlotDesc& d, double rlist, int nc[3]) {
    double w[3];
    box_widths(d.h, w);
    for (int a = 0; a < 3; ++a) {
        double q = std::floor(w[a] / rlist);
        nc[a] = q < 1.0 ? 1 : (q > 2000.0 ? 2000 : (int)q);
    }
}

// Box fields of a slot from a row-major h and its inverse (p.nc set): diagonals (h, hinv) for the
// orthorhombic kernels, the full matrices and cell edge vectors for a triclinic box, cell widths.
// rl: the padded list radius (the FP32 list test's radius, in length units)
static void set_box(SysParams& p, const double* h, const double* hi, double rl) {
    double w[3];
    box_widths(h, w);
    p.tric = diagonal_box(h) ? 0 : 1;
    for (int k = 0; k < 9; ++k) {
        p.H[k] = h[k];
        p.HI[k] = hi[k];
    }
    for (int a = 0; a < 3; ++a) {
        p.h[a] = h[4 * a];
        p.hinv[a] = hi[4 * a];
        p.cs[a] = w[a] / p.nc[a];
    }
    p.sc = p.tric ? 1.0 : p.cs[0];
    p.isc = p.tric ? 1.0 : 1.0 / p.cs[0];
    p.fisc_hi = (float)p.isc;
    p.fisc_lo = (float)(p.isc - (double)p.fisc_hi);
    for (int a = 0; a < 3; ++a) {
        p.fcs[a] = (float)(p.cs[a] * p.isc);
        p.fsub[a] = (float)(4.0 * p.sc / p.cs[a]);
    }
    p.frlist2 = (float)(rl * rl * (p.isc * p.isc));
    for (int d = 0; d < 3; ++d)
        for (int r = 0; r < 3; ++r) p.fcv[3 * d + r] = (float)(h[3 * r + d] / p.nc[d]);
}

// FP32 constants of a pair-table entry for FP32 coordinates in units of sc (r' = r / sc):
// sigma^2 / r^2 and the cutoff test keep their values with sigma' = sigma / sc, rc' = rc / sc, and
// the force 24 eps s6 (2 s6 - 1) r / r^2 is c' r' with eps24' = 24 eps / sc.
static void set_fp32_constants(LJDev& t, double sc) {
    const double is2 = 1.0 / (sc * sc);
    t.feps4 = (float)t.eps4;
    t.feps24 = (float)(t.eps24 / sc);
    t.fsigma2 = (float)(t.sigma2 * is2);
    t.frc2 = (float)(t.rcut * t.rcut * is2);
    t.fucut = (float)t.ucut;
}

// The 27-cell walk (k_build1) serves axes of two cells too: there the -1 and +1 neighbours are
// the same cell seen through two images, and the box edge (2 cells of at least the list radius)
// exceeds twice the padded list radius, so at most one image of a pair passes the distance test
// and no pair is listed twice. Only an edge within 1e-5 of that bound is left to the generic walk,
// which keeps the nearer image per pair. rl: the padded list radius (its FP32 square decides).
static int walk27_valid(const SysParams& p, double rl) {
    const double rlf = std::sqrt((double)(float)(rl * rl));
    for (int a = 0; a < 3; ++a)
        if (p.nc[a] < 2 || (p.nc[a] == 2 && !(p.h[a] > 2.0 * rlf * (1.0 + 1e-5)))) return 0;
    return 1;
}

// The reference's own cell grid at the largest cutoff (Atoms::divide_into_cells,
// src/atoms/neighbour_list.rs:45-57: floor(|h column| / rcut), at least 1), for the reference-order
// forces. h is row-major.
static void reference_cells(const double* h, double rc_max, int32_t rnc[3]) {
    for (int a = 0; a < 3; ++a) {
        const double col[3] = {h[a], h[3 + a], h[6 + a]};
        const double len = std::sqrt(col[0] * col[0] + col[1] * col[1] + col[2] * col[2]);
        const double q = std::floor(len / rc_max);
        rnc[a] = q < 1.0 ? 1 : (q > 1e9 ? 1000000000 : (int)q);
    }
}
// The reference-order keys need at least 3 cells per axis and fewer than 2^25 cells.
static bool reference_cells_ok(const int32_t rnc[3]) {
    const double cells = (double)rnc[0] * rnc[1] * rnc[2];
    return rnc[0] >= 3 && rnc[1] >= 3 && rnc[2] >= 3 && cells < 33554432.0;
}

static double slot_rlist(const SlotDesc& d) {
    double rc = 0.0;
    for (auto& e : d.table)
        if (e.present && e.rcut > rc) rc = e.rcut;
    return rc + d.skin;
}

int64_t Engine::cells_for(const SlotDesc& d) {
    int nc[3];
    cell_grid(d, slot_rlist(d), nc);
    return (int64_t)nc[0] * nc[1] * nc[2];
}

bool Engine::fits(const SlotDesc& d) const {
    int nc[3];
    cell_grid(d, slot_rlist(d), nc);
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2] + 1;
    bool a = false, c = false;
    for (auto& kv : free_atoms_) a |= kv.second >= d.n;
    for (auto& kv : free_cells_) c |= kv.second >= ncell;
    int free_tab = 0, run = 0;
    for (int v : free_tab_) {
        run = v ? run + 1 : 0;
        free_tab = std::max(free_tab, run);
    }
    int slots = 0;
    for (auto& p : hp_) slots += !p.active;
    bool cl = true;
    if (clm_) {
        const int64_t need = (d.n + clm_ - 1) / clm_ + ncell;
        cl = false;
        for (auto& kv : free_clusters_) cl |= kv.second >= need;
    }
    return a && c && cl && slots > 0 && free_tab >= d.n_types * d.n_types;
}

int Engine::add_slot(const SlotDesc& d, const int32_t* type_ids, const double* pos, const double* vel,
                     const double* force, std::string& err, bool defer_map) {
    if (d.n <= 0) {
        err = "no atoms defined";
        return -PIS_ERR_NO_ATOMS;
    }
    if (!diagonal_box(d.h) && !triclinic_capable()) {
        err = "general (triclinic) boxes run on the FP64 path with exact arithmetic, one thread per atom";
        return -PIS_ERR_UNSUPPORTED;
    }
    double hinv_full[9];
    if (!inverse3_ref(d.h, hinv_full)) {
        err = "box matrix is singular";
        return -PIS_ERR_INVALID_ARGUMENT;
    }
    for (int a = 0; a < 3; ++a)
        if (!d.pbc[a]) {
            err = "only fully periodic boxes are supported";
            return -PIS_ERR_UNSUPPORTED;
        }
    const int nt = d.n_types;
    if (nt < 1 || (int)d.table.size() != nt * nt || (int)d.masses.size() < nt) {
        err = "pair table / masses do not match the number of types";
        return -PIS_ERR_INVALID_ARGUMENT;
    }
    double rlist = slot_rlist(d);
    if (rlist <= d.skin) {
        err = "no pair potential defined";
        return -PIS_ERR_MISSING_POTENTIAL;
    }
    {
        double w[3];
        box_widths(d.h, w);
        for (int a = 0; a < 3; ++a) {
            const double L = w[a];
            if (!(L > 2.0 * rlist)) {
                err = "box width " + std::to_string(L) + " is not longer than 2 (rcut + skin) = " +
                      std::to_string(2.0 * rlist);
                return -PIS_ERR_BOX_TOO_SMALL;
            }
            if (!diagonal_box(d.h) && !(L >= 3.0 * rlist)) {
                err = "a triclinic box needs at least 3 cells of the list radius across each pair of faces";
                return -PIS_ERR_BOX_TOO_SMALL;
            }
        }
    }
    for (int64_t k = 0; k < d.n; ++k)
        if (type_ids[k] < 1 || type_ids[k] > nt) {
            err = "atom type " + std::to_string(type_ids[k]) + " out of range";
            return -PIS_ERR_INVALID_ATOM_TYPE;
        }
    int slot = -1;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (!hp_[s].active) {
            slot = s;
            break;
        }
    if (slot < 0) {
        err = "no free slot";
        return -PIS_ERR_NO_MEMORY;
    }
    int nc[3];
    cell_grid(d, rlist, nc);
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t a0 = 0, c0 = 0;
    if (!take_range(free_atoms_, d.n, a0)) {
        err = "not enough free atom capacity in the pool";
        return -PIS_ERR_NO_MEMORY;
    }
    if (!take_range(free_cells_, ncell + 1, c0)) {
        give_range(free_atoms_, a0, d.n);
        err = "not enough free cell capacity in the pool";
        return -PIS_ERR_NO_MEMORY;
    }
    int64_t cl0 = 0, clcap = 0;
    if (clm_) {
        clcap = (d.n + clm_ - 1) / clm_ + ncell;
        if (!take_range(free_clusters_, clcap, cl0)) {
            give_range(free_atoms_, a0, d.n);
            give_range(free_cells_, c0, ncell + 1);
            err = "not enough free cluster capacity in the pool";
            return -PIS_ERR_NO_MEMORY;
        }
    }
    int tab0 = -1;
    {
        int need = nt * nt, run = 0;
        for (int k = 0; k < (int)free_tab_.size(); ++k) {
            run = free_tab_[k] ? run + 1 : 0;
            if (run == need) {
                tab0 = k - need + 1;
                break;
            }
        }
        if (tab0 < 0) {
            give_range(free_atoms_, a0, d.n);
            give_range(free_cells_, c0, ncell + 1);
            if (clm_) give_range(free_clusters_, cl0, clcap);
            err = "pair table capacity exhausted";
            return -PIS_ERR_NO_MEMORY;
        }
        for (int k = 0; k < need; ++k) free_tab_[tab0 + k] = 0;
    }
    slot_tab_size_[slot] = nt * nt;

    // pair table
    std::vector<LJDev> tab((size_t)nt * nt);
    for (int k = 0; k < nt * nt; ++k) {
        const LJHost& e = d.table[k];
        LJDev& t = tab[k];
        std::memset(&t, 0, sizeof(t));
        t.present = e.present;
        if (!e.present) continue;
        // exactly the reference's per-pair constants: 4.0*eps, 24.0*eps, sigma.powi(2),
        // u_cut from (sigma/rcut).powi(2) (src/potentials/lennard_jones.rs:33-55)
        t.eps4 = 4.0 * e.epsilon;
        t.eps24 = 24.0 * e.epsilon;
        t.sigma2 = e.sigma * e.sigma;
        t.rcut = e.rcut;
        double rc2 = e.rcut * e.rcut;
        t.rc2_lo = rc2 * (1.0 - 1e-12);
        t.rc2_hi = rc2 * (1.0 + 1e-12);
        double ucut = 0.0;
        if (e.shift) {
            double q = e.sigma / e.rcut;
            double ci2 = q * q;
            double ca = ci2 * (ci2 * ci2);
            double cr = ca * ca;
            ucut = 4.0 * e.epsilon * (cr - ca);
        }
        t.ucut = ucut;
    }

    SysParams p;
    std::memset(&p, 0, sizeof(p));
    p.a0 = a0;
    p.c0 = c0;
    p.n = (int32_t)d.n;
    p.active = 1;
    p.nt = nt;
    p.tab0 = tab0;
    for (int a = 0; a < 3; ++a) {
        p.nc[a] = nc[a];
        p.pbc[a] = 1;
    }
    // h^-1 by adjugate / determinant, the reference's 3x3 inverse (src/simulation_box.rs:13)
    const double rl = rlist * (1.0 + 1e-5);
    set_box(p, d.h, hinv_full, rl);
    p.half_skin2 = 0.25 * d.skin * d.skin;
    p.dt = d.dt;
    p.dt2 = d.dt * d.dt;
    p.hdt = 0.5 * p.dt;
    p.hdt2 = 0.5 * p.dt2;
    p.walk27 = walk27_valid(p, rl);
    // the pair table, FP32 constants in the slot's coordinate unit
    for (auto& t : tab)
        if (t.present) set_fp32_constants(t, p.sc);
    slot_tab_host_[slot] = tab;
    // deferred placement: nothing waits for these copies, so their sources are held
    auto src = [&](const void* q, size_t bytes) { return defer_map ? hold(q, bytes) : q; };
    pis_status st = check(cudaMemcpyAsync(d_->tab + tab0, src(tab.data(), sizeof(LJDev) * tab.size()),
                                          sizeof(LJDev) * tab.size(), cudaMemcpyHostToDevice, stream_),
                          "table upload", err);
    if (st) return -st;
    // the reference's own cell grid at the largest cutoff (Atoms::divide_into_cells,
    // src/atoms/neighbour_list.rs:45-57: floor(|h column| / rcut), at least 1)
    double rc_max = 0.0;  // PairPotentialManager::max_rcut (src/potentials/potential.rs:170-179)
    for (auto& e : d.table)
        if (e.present && rc_max < e.rcut) rc_max = e.rcut;
    reference_cells(d.h, rc_max, p.rnc);
    if (opt_.ref_order) {
        if (!reference_cells_ok(p.rnc)) {
            give_range(free_atoms_, a0, d.n);
            give_range(free_cells_, c0, ncell + 1);
            for (int k = 0; k < nt * nt; ++k) free_tab_[tab0 + k] = 1;
            err = "reference-order forces need 3 to 2^25 reference cells (at the largest cutoff), at least 3 per axis";
            return -PIS_ERR_UNSUPPORTED;
        }
    }
    // chunks
    p.nch = (int32_t)((d.n + opt_.blk - 1) / opt_.blk);
    p.ch0 = 0;  // assigned by the block map
    p.cl0 = (int32_t)cl0;
    p.clcap = (int32_t)clcap;
    p.ncch = (int32_t)((clcap + CL_THREADS - 1) / CL_THREADS);
    p.cch0 = 0;  // assigned by the block map
    hp_[slot] = p;
    slot_rlist_[slot] = rlist;
    slot_rcmax_[slot] = rc_max;

    // atom state: the caller's x,y,z-per-atom arrays and types go to the device as they are, and
    // k_load_slot builds the device layout
    if (nt > 16) {
        err = "at most 16 atom types per system";
        return -PIS_ERR_UNSUPPORTED;
    }
    MassArg ma;
    std::memset(&ma, 0, sizeof(ma));
    for (int t = 0; t < nt; ++t) ma.m[t] = d.masses[t];
    SysState ss;
    std::memset(&ss, 0, sizeof(ss));
    ss.cur = 0;
    ss.rebuild = 1;
    ss.steps_left = d.steps > 0 ? d.steps : 0;
    std::vector<int32_t> csys(ncell + 1, slot);
#define CP(dst, from, bytes)                                                                            \
    do {                                                                                                \
        st = check(cudaMemcpyAsync((dst), src((from), (bytes)), (bytes), cudaMemcpyHostToDevice, stream_), \
                   "upload", err);                                                                      \
        if (st) return -st;                                                                             \
    } while (0)
    CP(d_->pos[1] + a0, pos, 24 * d.n);
    if (vel) CP(d_->vel[1] + a0, vel, 24 * d.n);
    if (force) CP(d_->acc[1] + a0, force, 24 * d.n);
    CP(d_->id[1] + a0, type_ids, 4 * d.n);
    LAUNCH(k_load_slot, (unsigned)((d.n + 255) / 256), 256, *d_, a0, (int)d.n, ma, vel ? 1 : 0, force ? 1 : 0);
    st = check(cudaGetLastError(), "upload", err);
    if (st) return -st;
    st = check(cudaMemsetAsync(d_->cellof + a0, 0, 4 * d.n, stream_), "upload", err);
    if (st) return -st;
    st = check(cudaMemsetAsync(d_->nn + a0, 0, 4 * d.n, stream_), "upload", err);
    if (st) return -st;
    st = check(cudaMemsetAsync(d_->cell_count + c0, 0, 4 * (ncell + 1), stream_), "upload", err);
    if (st) return -st;
    CP(d_->cell_sys + c0, csys.data(), 4 * (ncell + 1));
    CP(d_->st + slot, &ss, sizeof(ss));
#undef CP
    dirty_map_ = true;
    if (defer_map) return slot;
    st = rebuild_block_map(err);
    if (st) return -st;
    st = sync(err);
    if (st) return -st;
    return slot;
}

void Engine::remove_slot(int slot, bool defer_map) {
    if (slot < 0 || slot >= opt_.max_slots || !hp_[slot].active) return;
    if ((int)slot_thermo_.size() > slot && slot_thermo_[slot]) {
        slot_thermo_[slot] = 0;
        thermo_slots_ -= 1;
    }
    SysParams& p = hp_[slot];
    int64_t ncell = (int64_t)p.nc[0] * p.nc[1] * p.nc[2];
    give_range(free_atoms_, p.a0, p.n);
    give_range(free_cells_, p.c0, ncell + 1);
    if (clm_) give_range(free_clusters_, p.cl0, p.clcap);
    for (int k = 0; k < slot_tab_size_[slot]; ++k) free_tab_[p.tab0 + k] = 1;
    std::vector<int32_t> csys(ncell + 1, -1);
    cudaMemcpyAsync(d_->cell_sys + p.c0, defer_map ? hold(csys.data(), 4 * (ncell + 1)) : csys.data(),
                    4 * (ncell + 1), cudaMemcpyHostToDevice, stream_);
    p.active = 0;
    dirty_map_ = true;
    if (defer_map) return;
    std::string err;
    rebuild_block_map(err);
    cudaStreamSynchronize(stream_);
}

int Engine::n_active() const {
    int k = 0;
    for (auto& p : hp_) k += p.active;
    return k;
}

// Chunk table: every active slot gets ceil(n / blk) consecutive chunks; the grid is always
// max_chunks blocks so captured graphs stay valid when slots come and go.
pis_status Engine::rebuild_block_map(std::string& err) {
    if (!dirty_map_) return PIS_OK;
    std::vector<int32_t> bs(max_chunks_, -1), bf(max_chunks_, 0);
    // Slots with the most atoms per cell first: their list-build blocks walk the most candidates
    // per atom (small boxes have cells well above the list radius) and, scheduled last, were the
    // tail of every rebuild in a mixed pool. A slot's chunks stay consecutive, so its sums and
    // results do not depend on the order.
    std::vector<int> order;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (hp_[s].active) order.push_back(s);
    auto per_cell = [&](int s) {
        const SysParams& p = hp_[s];
        return (double)p.n / ((double)p.nc[0] * p.nc[1] * p.nc[2]);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return per_cell(a) > per_cell(b); });
    int64_t c = 0;
    for (int s : order) {
        SysParams& p = hp_[s];
        p.ch0 = (int32_t)c;
        for (int k = 0; k < p.nch; ++k, ++c) {
            bs[c] = s;
            bf[c] = (int32_t)(p.a0 + (int64_t)k * opt_.blk);
        }
    }
    pis_status st = check(cudaMemcpyAsync(d_->blk_sys, hold(bs.data(), 4 * max_chunks_), 4 * max_chunks_, cudaMemcpyHostToDevice, stream_),
                          "block map", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(d_->blk_first, hold(bf.data(), 4 * max_chunks_), 4 * max_chunks_, cudaMemcpyHostToDevice, stream_),
               "block map", err);
    if (st) return st;
    // cluster kernels: every active slot gets ceil(cluster capacity / CL_THREADS) chunks
    std::vector<int32_t> cbs, cbf;
    if (clm_) {
        cbs.assign(max_cchunks_, -1);
        cbf.assign(max_cchunks_, 0);
        int64_t q = 0;
        for (int s = 0; s < opt_.max_slots; ++s) {
            SysParams& p = hp_[s];
            if (!p.active) continue;
            p.cch0 = (int32_t)q;
            for (int k = 0; k < p.ncch; ++k, ++q) {
                cbs[q] = s;
                cbf[q] = p.cl0 + k * CL_THREADS;
            }
        }
        st = check(cudaMemcpyAsync(d_->cblk_sys, hold(cbs.data(), 4 * max_cchunks_), 4 * max_cchunks_, cudaMemcpyHostToDevice, stream_),
                   "block map", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(d_->cblk_first, hold(cbf.data(), 4 * max_cchunks_), 4 * max_cchunks_, cudaMemcpyHostToDevice, stream_),
                   "block map", err);
        if (st) return st;
    }
    st = check(cudaMemcpyAsync(d_->sp, hold(hp_.data(), sizeof(SysParams) * hp_.size()), sizeof(SysParams) * hp_.size(), cudaMemcpyHostToDevice, stream_),
               "params", err);
    if (st) return st;
    // No synchronisation here (the sources are held), so a host loop can change the map while
    // earlier graphs still run: the copies are ordered after them on the stream.
    dirty_map_ = false;
    // kernel choices that follow the active slots (the force kernel for single-type pools, the
    // triclinic rebuild kernels, the generic walk, the cell-scan grid); step graphs are kept per
    // combination (Engine::run)
    bool one = true, tric = false, gen = false;
    int segs = 1;  // cell-scan segments of the largest slot (the scan kernels' grid)
    for (int s = 0; s < opt_.max_slots; ++s) {
        if (hp_[s].active && hp_[s].nt != 1) one = false;
        if (hp_[s].active && hp_[s].tric) tric = true;
        if (hp_[s].active && !hp_[s].walk27) gen = true;
        if (hp_[s].active) {
            const int64_t nc = (int64_t)hp_[s].nc[0] * hp_[s].nc[1] * hp_[s].nc[2];
            segs = std::max(segs, (int)((nc + SCAN_SEG - 1) / SCAN_SEG));
        }
    }
    single_type_ = one;
    any_tric_ = tric;
    scan_segs_ = segs;
    any_generic_ = gen;
    return st;
}

pis_status Engine::sync(std::string& err) {
    pis_status st = check(cudaStreamSynchronize(stream_), "stream sync", err);
    if (!st) {
        account_body_launches();
        held_.clear();
    }
    return st;
}

const void* Engine::hold(const void* src, size_t bytes) {
    if (!src || bytes == 0) return src;
    held_.push_back(Held{held_seq_, std::vector<unsigned char>((const unsigned char*)src,
                                                                (const unsigned char*)src + bytes)});
    return held_.back().buf.data();
}

pis_status Engine::wait_event(cudaEvent_t e, std::string& err) {
    return check(cudaEventSynchronize(e), "event wait", err);
}

void Engine::retire_staging(uint64_t mark) {
    while (!held_.empty() && held_.front().seq < mark) held_.pop_front();
}

pis_status Engine::set_dt(int slot, double dt, std::string& err) {
    SysParams& p = hp_[slot];
    if (p.dt == dt) return PIS_OK;
    p.dt = dt;
    p.dt2 = dt * dt;
    p.hdt = 0.5 * p.dt;
    p.hdt2 = 0.5 * p.dt2;
    pis_status st = check(cudaMemcpyAsync(d_->sp + slot, &p, sizeof(SysParams), cudaMemcpyHostToDevice, stream_),
                          "params", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::set_steps(int slot, int64_t steps, std::string& err) {
    pis_status st = check(cudaMemcpyAsync(&d_->st[slot].steps_left, &steps, 8, cudaMemcpyHostToDevice, stream_),
                          "steps", err);
    if (st) return st;
    return sync(err);
}

void Engine::enqueue_rebuild(bool respect, int q) {
    const DP& P = *d_;
    int r = respect ? 1 + q : 0;
    const int64_t start = g_launches.load();
    const unsigned ga = (unsigned)max_chunks_;
    const unsigned gl = (unsigned)listed_grid_;
    if (listed_) {
        LAUNCH(k_rebuild_list, (unsigned)opt_.max_slots, 256, P, r);
        LAUNCH(k_bin_list, gl, opt_.blk, P, r);
    } else {
        LAUNCH(k_bin, ga, opt_.blk, P, r);
    }
    if (scan_segs_ <= 1) {
        LAUNCH(k_scan, (unsigned)opt_.max_slots, SCAN_THREADS, P, r);
    } else {  // a slot of more than SCAN_SEG cells: segmented scan, one block per segment
        const dim3 g((unsigned)opt_.max_slots, (unsigned)scan_segs_);
        LAUNCH(k_scan_seg, g, SCAN_THREADS, P, r);
        LAUNCH(k_scan_fix, g, 256, P, r);
    }
    unsigned gcells = (unsigned)((opt_.max_cells * 32 + 255) / 256);
    if (listed_) {
        LAUNCH(k_scatter_list, gl, opt_.blk, P, r);
        if (any_tric_)
            LAUNCH(k_gather_list<true>, gl, 256, P, r);
        else
            LAUNCH(k_gather_list<false>, gl, 256, P, r);
    } else {
        LAUNCH(k_scatter, ga, opt_.blk, P, r);
        if (any_tric_)
            LAUNCH(k_gather<true>, gcells, 256, P, (int64_t)opt_.max_cells, r);
        else
            LAUNCH(k_gather<false>, gcells, 256, P, (int64_t)opt_.max_cells, r);
    }
    launch_build(r);
    // inside a conditional body the last kernel adds the body's kernel count on the device
    const int body = ls_ == side_ ? (int)(g_launches.load() - start + 1) : 0;
    LAUNCH(k_rebuild_done, (unsigned)((opt_.max_slots + 127) / 128), 128, P, r, body);
}

// Lanes-per-atom kernels are templates; these dispatch on the pool's runtime choice. Their grid
// has lpa blocks per chunk.
// List build over `chunks` (L blocks per chunk for lanes-per-atom layouts).
template <bool HALF>
static void launch_build1(const DP& P, bool tric, unsigned g, cudaStream_t st, int r, int only_two_cell) {
    if (tric)
        k_build1<HALF, true><<<g, 256, 0, st>>>(P, r, only_two_cell);
    else
        k_build1<HALF, false><<<g, 256, 0, st>>>(P, r, only_two_cell);
}

// generic: some slot needs the generic walk (its kernel is launched only then). listed > 0: the
// grid of the listed rebuild of a replica pool.
template <int L>
static void launch_build_t(const DP& P, bool half, bool tric, unsigned chunks, cudaStream_t st, int r, bool generic,
                           unsigned listed) {
    const unsigned g = chunks * L;
    if (L == 1 && listed) {
        if (half)
            tric ? k_build1_list<true, true><<<listed, 256, 0, st>>>(P, r) : k_build1_list<true, false><<<listed, 256, 0, st>>>(P, r);
        else
            tric ? k_build1_list<false, true><<<listed, 256, 0, st>>>(P, r) : k_build1_list<false, false><<<listed, 256, 0, st>>>(P, r);
        if (generic) {
            if (half)
                k_build1_generic_list<true><<<listed, 256, 0, st>>>(P, r);
            else
                k_build1_generic_list<false><<<listed, 256, 0, st>>>(P, r);
        }
        g_launches.fetch_add(generic ? 2 : 1);
        return;
    }
    if (L == 1) {
        // lean kernel for the 27-cell walk, generic kernel for the other slots
        if (half) {
            launch_build1<true>(P, tric, g, st, r, 0);
            if (generic) k_build1_generic<true><<<g, 256, 0, st>>>(P, r);
        } else {
            launch_build1<false>(P, tric, g, st, r, 0);
            if (generic) k_build1_generic<false><<<g, 256, 0, st>>>(P, r);
        }
        g_launches.fetch_add(generic ? 2 : 1);
        return;
    }
    if (half)
        k_build<true, L><<<g, 256, 0, st>>>(P, r);
    else
        k_build<false, L><<<g, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

template <int L, int B>
static void launch_mixed_tb(const DP& P, bool kahan, bool one, unsigned chunks, cudaStream_t st, int r) {
    if (L == 1 && P.lq == FUSED_LQ) {  // the fused step's pools: FUSED_LQ-entry list groups
        if (kahan && one)
            k_force_mixed<1, 1, true, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else if (kahan)
            k_force_mixed<1, 1, false, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else if (one)
            k_force_mixed<0, 1, true, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else
            k_force_mixed<0, 1, false, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        g_launches.fetch_add(1);
        return;
    }
    if (kahan && one)
        k_force_mixed<1, L, true, B><<<chunks * L, 256, 0, st>>>(P, r);
    else if (kahan)
        k_force_mixed<1, L, false, B><<<chunks * L, 256, 0, st>>>(P, r);
    else if (one)
        k_force_mixed<0, L, true, B><<<chunks * L, 256, 0, st>>>(P, r);
    else
        k_force_mixed<0, L, false, B><<<chunks * L, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

// Entries per batch (list words loaded before their gathers): a tuning knob for thread-per-atom;
// groups of lanes always use 4.
template <int L>
static void launch_mixed_t(const DP& P, bool kahan, bool one, int batch, unsigned chunks, cudaStream_t st, int r) {
    if (L == 1 && batch == 4)
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
    else if (L == 1 && batch == 16)
        launch_mixed_tb<L, 16>(P, kahan, one, chunks, st, r);
    else if (L == 1 && batch == 8)
        launch_mixed_tb<L, 8>(P, kahan, one, chunks, st, r);
    else if (L == 1)
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
    else
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
}

template <int L>
static void launch_fp64_t(const DP& P, bool half, bool fast, unsigned chunks, cudaStream_t st, int r) {
    if (half && !fast)
        k_force_fp64<false, false, L><<<chunks * L, 256, 0, st>>>(P, r);
    else if (half)
        k_force_fp64<false, true, L><<<chunks * L, 256, 0, st>>>(P, r);
    else if (!fast)
        k_force_fp64<true, false, L><<<chunks * L, 256, 0, st>>>(P, r);
    else
        k_force_fp64<true, true, L><<<chunks * L, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

#define PIS_LPA_DISPATCH(lpa, CALL) \
    switch (lpa) {                  \
        case 4: CALL(4); break;     \
        case 8: CALL(8); break;     \
        case 16: CALL(16); break;   \
        case 32: CALL(32); break;   \
        default: CALL(1); break;    \
    }

template <int ACC, bool ONE, int M>
static void launch_cluster_t(const DP& P, int batch, bool lanes, unsigned chunks, cudaStream_t st, int r) {
    if (lanes) {
        if (batch >= 8)
            k_force_cl_lane<ACC, ONE, M, 8><<<chunks * M, CL_THREADS, 0, st>>>(P, r);
        else
            k_force_cl_lane<ACC, ONE, M, 4><<<chunks * M, CL_THREADS, 0, st>>>(P, r);
        return;
    }
    if (batch >= 8)
        k_force_cl<ACC, ONE, M, 8><<<chunks, CL_THREADS, 0, st>>>(P, r);
    else
        k_force_cl<ACC, ONE, M, 4><<<chunks, CL_THREADS, 0, st>>>(P, r);
}

template <int M>
static void launch_cluster_m(const DP& P, bool kahan, bool one, int batch, bool lanes, unsigned chunks, cudaStream_t st,
                             int r) {
    if (kahan)
        one ? launch_cluster_t<1, true, M>(P, batch, lanes, chunks, st, r)
            : launch_cluster_t<1, false, M>(P, batch, lanes, chunks, st, r);
    else
        one ? launch_cluster_t<0, true, M>(P, batch, lanes, chunks, st, r)
            : launch_cluster_t<0, false, M>(P, batch, lanes, chunks, st, r);
}

// Cluster-list forces: entries per batch = the batch knob (4 or 8); lanes per atom = M selects the
// lane-per-member kernel.
void Engine::launch_force_cluster(int r) {
    const unsigned ch = (unsigned)max_cchunks_;
    const bool lanes = opt_.lpa == opt_.cluster;
    if (opt_.cluster == 2)
        launch_cluster_m<2>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, lanes, ch, stream_, r);
    else
        launch_cluster_m<4>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, lanes, ch, stream_, r);
    g_launches.fetch_add(1);
}

void Engine::launch_build(int r) {
    const unsigned ch = (unsigned)max_chunks_;
    const unsigned gc = (unsigned)max_cchunks_, ga = (unsigned)max_chunks_;
    if (opt_.cluster) {
        if (opt_.cluster == 2)
            k_build_cl<2><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 0);
        else
            k_build_cl<4><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 0);
        g_launches.fetch_add(1);
        return;
    }
    if (clm_ && opt_.lpa == 1) {
        // two-stage per-atom build: cluster union lists, filtered per member; slots with a
        // two-cell axis use the 27-cell walk (or, at the two-cell edge bound, the generic kernel)
        if (clm_ == 2) {
            k_build_cl<2><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 1);
            if (half_)
                k_filter_cl<true, 2><<<gc * 2, CL_THREADS, 0, ls_>>>(*d_, r);
            else
                k_filter_cl<false, 2><<<gc * 2, CL_THREADS, 0, ls_>>>(*d_, r);
        } else {
            k_build_cl<4><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 1);
            if (half_)
                k_filter_cl<true, 4><<<gc * 4, CL_THREADS, 0, ls_>>>(*d_, r);
            else
                k_filter_cl<false, 4><<<gc * 4, CL_THREADS, 0, ls_>>>(*d_, r);
        }
        if (half_) {
            launch_build1<true>(*d_, any_tric_, ga, ls_, r, 1);
            k_build1_generic<true><<<ga, 256, 0, ls_>>>(*d_, r);
        } else {
            launch_build1<false>(*d_, any_tric_, ga, ls_, r, 1);
            k_build1_generic<false><<<ga, 256, 0, ls_>>>(*d_, r);
        }
        g_launches.fetch_add(4);
        return;
    }
#define PIS_CALL(L) launch_build_t<L>(*d_, half_, any_tric_, ch, ls_, r, any_generic_, listed_ ? (unsigned)listed_grid_ : 0u)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

template <int ACC, bool ONE, int KB>
static void launch_mixed_tma_t(const DP& P, unsigned chunks, cudaStream_t st, int r) {
    k_force_mixed_tma<ACC, ONE, KB><<<chunks, 256, mix_tma_smem_bytes<KB>(), st>>>(P, r);
}

// Bulk-copy-fed variant: rows per stage = the batch knob (8 or 16).
static void launch_mixed_tma(const DP& P, bool kahan, bool one, int batch, unsigned chunks, cudaStream_t st, int r) {
    const bool b16 = batch == 16;
    if (kahan) {
        if (one)
            b16 ? launch_mixed_tma_t<1, true, 16>(P, chunks, st, r) : launch_mixed_tma_t<1, true, 8>(P, chunks, st, r);
        else
            b16 ? launch_mixed_tma_t<1, false, 16>(P, chunks, st, r) : launch_mixed_tma_t<1, false, 8>(P, chunks, st, r);
    } else {
        if (one)
            b16 ? launch_mixed_tma_t<0, true, 16>(P, chunks, st, r) : launch_mixed_tma_t<0, true, 8>(P, chunks, st, r);
        else
            b16 ? launch_mixed_tma_t<0, false, 16>(P, chunks, st, r) : launch_mixed_tma_t<0, false, 8>(P, chunks, st, r);
    }
    g_launches.fetch_add(1);
}

// Dynamic shared memory of the bulk-copy-fed kernels (the 16-row ring exceeds the 48 KB default).
template <int ACC, bool ONE, int KB>
static cudaError_t allow_mixed_tma_smem() {
    return cudaFuncSetAttribute(k_force_mixed_tma<ACC, ONE, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mix_tma_smem_bytes<KB>());
}

static cudaError_t allow_all_mixed_tma_smem() {
    cudaError_t e = cudaSuccess, q;
    if ((q = allow_mixed_tma_smem<0, true, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, true, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, false, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, false, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, true, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, true, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, false, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, false, 16>()) != cudaSuccess) e = q;
    return e;
}

void Engine::launch_force_mixed(int r) {
    const unsigned ch = (unsigned)max_chunks_;
    if (opt_.cluster) {
        launch_force_cluster(r);
        return;
    }
    if (opt_.cell_tiles) {
        const size_t smem = TILE_ATOMS * sizeof(float4);
        if (opt_.mixed_kahan)
            single_type_ ? k_force_mixed_tile<1, true><<<ch, 256, smem, stream_>>>(*d_, r)
                         : k_force_mixed_tile<1, false><<<ch, 256, smem, stream_>>>(*d_, r);
        else
            single_type_ ? k_force_mixed_tile<0, true><<<ch, 256, smem, stream_>>>(*d_, r)
                         : k_force_mixed_tile<0, false><<<ch, 256, smem, stream_>>>(*d_, r);
        g_launches.fetch_add(1);
        return;
    }
    if (opt_.list_tma && opt_.lpa == 1) {
        launch_mixed_tma(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, ch, stream_, r);
        return;
    }
    if (half_) {  // Newton-3 half list: F_j by FP64 atomics
        if (opt_.mixed_kahan)
            single_type_ ? k_force_mixed_half<1, true, 4><<<ch, 256, 0, stream_>>>(*d_, r)
                         : k_force_mixed_half<1, false, 4><<<ch, 256, 0, stream_>>>(*d_, r);
        else
            single_type_ ? k_force_mixed_half<0, true, 4><<<ch, 256, 0, stream_>>>(*d_, r)
                         : k_force_mixed_half<0, false, 4><<<ch, 256, 0, stream_>>>(*d_, r);
        g_launches.fetch_add(1);
        return;
    }
#define PIS_CALL(L) launch_mixed_t<L>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, ch, stream_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

void Engine::launch_force_fp64(int r) {
    const unsigned ch = (unsigned)max_chunks_;
    if (opt_.ref_order) {
        LAUNCH(k_force_fp64_ref, ch, 256, *d_, r);
        return;
    }
#define PIS_CALL(L) launch_fp64_t<L>(*d_, half_, opt_.fp64_fast, ch, stream_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

// Step q of a g-step graph. Unfused: drift, rebuild, forces, kick, step end. Fused (mixed path,
// default kernel shape): the graph's first step drifts alone, every step then runs rebuild, the
// fused forces + kick + next drift (no drift in the graph's last step), step end; step q reads
// cell-relative coordinates from buffer q & 1 (its list rebuild writes them there) and the drift
// writes the other.
void Engine::enqueue_step(bool respect, cudaEvent_t* ev, int64_t q, int64_t g) {
    const DP& P = *d_;
    int r = respect ? 1 : 0;
    const bool mixed = opt_.precision == PIS_PRECISION_MIXED;
    const bool fused = mixed && fused_;
    if (ev) cudaEventRecordWithFlags(ev[0], stream_, cudaEventRecordExternal);
    if (!fused || q == 0) {
        if (mixed)
            LAUNCH(k_integrate1<true>, (unsigned)max_chunks_, opt_.blk, P);
        else
            LAUNCH(k_integrate1<false>, (unsigned)max_chunks_, opt_.blk, P);
    }
    if (ev) cudaEventRecordWithFlags(ev[1], stream_, cudaEventRecordExternal);
    if (fused) {
        d_->prel = (float4*)prel_buf_[q & 1];
        d_->prel_out = (float4*)prel_buf_[(q + 1) & 1];
    }
    // fused steps keep the step counters fixed through the graph: the rebuild kernels of step q
    // see the slots with more than q steps left
    const int qs = fused ? (int)q : 0;
    if (cond_step_)
        cond_error_ = cond_error_ ? cond_error_ : enqueue_rebuild_conditional(respect, qs);
    else
        enqueue_rebuild(respect, qs);
    if (ev) cudaEventRecordWithFlags(ev[2], stream_, cudaEventRecordExternal);
    if (fused)
        launch_step_mixed(q + 1 < g, (int)q);
    else if (mixed)
        launch_force_mixed(r);
    else
        launch_force_fp64(r);
    if (ev) cudaEventRecordWithFlags(ev[3], stream_, cudaEventRecordExternal);
    if (!fused) {
        if (mixed)
            LAUNCH((k_integrate2<true, false>), (unsigned)max_chunks_, opt_.blk, P, r);
        else
            LAUNCH((k_integrate2<true, true>), (unsigned)max_chunks_, opt_.blk, P, r);
    }
    if (ev) cudaEventRecordWithFlags(ev[4], stream_, cudaEventRecordExternal);
    if (!fused) launch_step_end(0);  // fused steps: k_ring_sums / k_ring_commit after the graph's last step
    if (ev) cudaEventRecordWithFlags(ev[5], stream_, cudaEventRecordExternal);
    if (fused) {
        d_->prel = (float4*)prel_buf_[0];
        d_->prel_out = nullptr;
    }
}

template <int ACC, bool ONE, int B, bool TRACE>
static void launch_step_mixed_tt(const DP& P, bool drift, int q, unsigned chunks, cudaStream_t st) {
    if (drift)
        k_step_mixed<ACC, ONE, B, true, TRACE><<<chunks, 256, 0, st>>>(P, q);
    else
        k_step_mixed<ACC, ONE, B, false, TRACE><<<chunks, 256, 0, st>>>(P, q);
}
template <int ACC, bool ONE, int B>
static void launch_step_mixed_t(const DP& P, bool drift, bool trace, int q, unsigned chunks, cudaStream_t st) {
    if (trace)
        launch_step_mixed_tt<ACC, ONE, B, true>(P, drift, q, chunks, st);
    else
        launch_step_mixed_tt<ACC, ONE, B, false>(P, drift, q, chunks, st);
}

void Engine::launch_step_end(int mode) {
    if (d_->exact_sums)
        LAUNCH(k_step_end<true>, (unsigned)opt_.max_slots, END_THREADS, *d_, mode);
    else
        LAUNCH(k_step_end<false>, (unsigned)opt_.max_slots, END_THREADS, *d_, mode);
}

void Engine::launch_step_mixed(bool drift, int q) {
    const unsigned ch = (unsigned)max_chunks_;
    const bool b8 = opt_.mix_batch == 8;
    const bool tr = thermo_slots_ > 0;
    if (opt_.mixed_kahan) {
        if (single_type_)
            b8 ? launch_step_mixed_t<1, true, 8>(*d_, drift, tr, q, ch, stream_)
               : launch_step_mixed_t<1, true, 4>(*d_, drift, tr, q, ch, stream_);
        else
            b8 ? launch_step_mixed_t<1, false, 8>(*d_, drift, tr, q, ch, stream_)
               : launch_step_mixed_t<1, false, 4>(*d_, drift, tr, q, ch, stream_);
    } else {
        if (single_type_)
            b8 ? launch_step_mixed_t<0, true, 8>(*d_, drift, tr, q, ch, stream_)
               : launch_step_mixed_t<0, true, 4>(*d_, drift, tr, q, ch, stream_);
        else
            b8 ? launch_step_mixed_t<0, false, 8>(*d_, drift, tr, q, ch, stream_)
               : launch_step_mixed_t<0, false, 4>(*d_, drift, tr, q, ch, stream_);
    }
    g_launches.fetch_add(1);
}

void Engine::enqueue_potential(int only) {
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    LAUNCH(k_mark_eval, sg, 128, P, only, 1, 0);
    LAUNCH(k_zero_forces, (unsigned)max_chunks_, opt_.blk, P);
    enqueue_rebuild(false);
    if (opt_.precision == PIS_PRECISION_MIXED)
        launch_force_mixed(0);
    else
        launch_force_fp64(0);
    launch_step_end(1);
}

// Inside a stream capture of stream_: a 1-thread kernel sets the condition from the rebuild word,
// then a conditional IF node whose body (the rebuild kernels, captured on side_) runs only when
// some slot rebuilds. On the ~8 steps in 9 without a rebuild the step then launches no rebuild
// kernel at all.
pis_status Engine::enqueue_rebuild_conditional(bool respect, int q) {
    cudaStreamCaptureStatus cs;
    unsigned long long id = 0;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(stream_, &cs, &id, &g, &deps, &edges, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return PIS_ERR_CUDA;
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return PIS_ERR_CUDA;
    k_set_rebuild_cond<<<1, 1, 0, stream_>>>(*d_, h);
    g_launches.fetch_add(1);
    if (cudaStreamGetCaptureInfo(stream_, &cs, &id, &g, &deps, &edges, &nd) != cudaSuccess) return PIS_ERR_CUDA;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, edges, nd, &cp) != cudaSuccess) return PIS_ERR_CUDA;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (cudaStreamUpdateCaptureDependencies(stream_, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
        return PIS_ERR_CUDA;
    if (cudaStreamBeginCaptureToGraph(side_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return PIS_ERR_CUDA;
    const int64_t before = g_launches.load();
    ls_ = side_;
    enqueue_rebuild(respect, q);
    ls_ = stream_;
    const int64_t n_body = g_launches.load() - before;
    g_launches.fetch_sub(n_body);  // counted when a body actually runs (account_body_launches)
    body_counting_ = true;
    cudaGraph_t out = nullptr;
    if (cudaStreamEndCapture(side_, &out) != cudaSuccess) return PIS_ERR_CUDA;
    return PIS_OK;
}

void Engine::account_body_launches() {
    if (!body_counting_ || !d_) return;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, d_->ctl + 2, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return;
    if (n > body_seen_) {
        g_launches.fetch_add((int64_t)(n - body_seen_));
        body_seen_ = n;
    }
}

pis_status Engine::compute_potential(std::string& err) { return compute_potential_slot(-1, err); }

pis_status Engine::compute_potential_slot(int only, std::string& err) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    enqueue_potential(only);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return reduce_state_slot(true, only, err);
}

// Force evaluation and reductions for a set of slots (each marked, then one kernel sequence for
// all): the serving loop evaluates the jobs it admits between two graphs together. Every slot's
// results are those of compute_potential_slot on it alone.
pis_status Engine::compute_potential_slots(const std::vector<int>& slots, std::string& err, bool wait) {
    if (slots.empty()) return PIS_OK;
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    for (int s : slots) LAUNCH(k_mark_eval, sg, 128, P, s, 1, 0);
    LAUNCH(k_zero_forces, (unsigned)max_chunks_, opt_.blk, P);
    enqueue_rebuild(false);
    if (opt_.precision == PIS_PRECISION_MIXED)
        launch_force_mixed(0);
    else
        launch_force_fp64(0);
    launch_step_end(1);
    for (int s : slots) LAUNCH(k_mark_eval, sg, 128, P, s, 0, 1);
    if (opt_.precision == PIS_PRECISION_MIXED)
        LAUNCH((k_integrate2<false, false>), (unsigned)max_chunks_, opt_.blk, P, 0);
    else
        LAUNCH((k_integrate2<false, true>), (unsigned)max_chunks_, opt_.blk, P, 0);
    launch_step_end(2);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return wait ? sync(err) : PIS_OK;
}

pis_status Engine::reduce_state(bool virial, std::string& err) { return reduce_state_slot(virial, -1, err); }

pis_status Engine::reduce_state_slot(bool virial, int only, std::string& err, bool ktensor) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    LAUNCH(k_mark_eval, sg, 128, P, only, 0, (virial ? 1 : 0) | (ktensor ? 2 : 0));
    if (opt_.precision == PIS_PRECISION_MIXED)
        LAUNCH((k_integrate2<false, false>), (unsigned)max_chunks_, opt_.blk, P, 0);
    else
        LAUNCH((k_integrate2<false, true>), (unsigned)max_chunks_, opt_.blk, P, 0);
    launch_step_end(2);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return sync(err);
}

void Engine::reset_stage_times() {
    for (double& v : stage_ms_) v = 0.0;
    stage_steps_ = 0;
}

pis_status Engine::run(int64_t k, std::string& err) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    // fused steps: a graph holds at most RING_STEPS steps (the rows of the partial ring), and no
    // more than the energy history holds (its entries are written by parallel blocks at the end)
    int64_t G = graph_steps_;
    if (fused_) G = std::min<int64_t>(G, std::min<int64_t>(RING_STEPS, opt_.hist));
    while (k > 0) {
        int64_t g = k >= G ? G : k;
        // graphs differ by length, instrumentation, whether the fused step records thermo, and
        // the kernel choices the pool's slots imply (one type, a triclinic slot, a slot on the
        // generic walk, the cell-scan segments): a pool whose slots come and go keeps one graph
        // per combination instead of recapturing at every change
        int64_t key = 4 * g + (instrument_ ? 1 : 0) + (thermo_slots_ > 0 ? 2 : 0);
        key = key * 8 + (single_type_ ? 4 : 0) + (any_tric_ ? 2 : 0) + (any_generic_ ? 1 : 0);
        key = key * 4096 + std::min(scan_segs_, 4095);
        auto it = graphs_.find(key);
        if (it == graphs_.end()) {
            GraphRec rec;
            if (instrument_) {
                rec.ev.resize((size_t)(6 * g + 1));  // + the end of the graph's ring kernels
                for (auto& e : rec.ev) {
                    st = check(cudaEventCreate(&e), "event", err);
                    if (st) return st;
                }
            }
            cudaGraph_t graph = nullptr;
            for (int attempt = 0; attempt < 2; ++attempt) {
                st = check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture", err);
                if (st) return st;
                int64_t before = g_launches.load();
                cond_step_ = cond_rebuild_;
                cond_error_ = PIS_OK;
                for (int64_t q = 0; q < g; ++q)
                    enqueue_step(true, instrument_ ? rec.ev.data() + 6 * q : nullptr, q, g);
                cond_step_ = false;
                if (fused_ && opt_.precision == PIS_PRECISION_MIXED) {
                    // the step ends of the graph's fused steps: energies per step, then counters
                    LAUNCH(k_ring_sums, dim3((unsigned)opt_.max_slots, (unsigned)g), END_THREADS, *d_);
                    LAUNCH(k_ring_commit, (unsigned)((opt_.max_slots + 127) / 128), 128, *d_, (int)g);
                }
                if (instrument_) cudaEventRecordWithFlags(rec.ev[6 * g], stream_, cudaEventRecordExternal);
                int64_t captured = g_launches.load() - before;
                g_launches.fetch_sub(captured);
                rec.kernels = captured;
                kernels_per_step_ = captured / g;
                cudaError_t ce = cudaStreamEndCapture(stream_, &graph);
                if (ce == cudaSuccess && cond_error_ == PIS_OK) {
                    ce = cudaGraphInstantiate(&rec.exec, graph, 0);
                    cudaGraphDestroy(graph);
                    if (ce == cudaSuccess) break;
                } else if (graph) {
                    cudaGraphDestroy(graph);
                }
                graph = nullptr;
                cudaGetLastError();
                if (!cond_rebuild_) return check(ce == cudaSuccess ? cudaErrorUnknown : ce, "capture", err);
                // conditional nodes unavailable: capture the plain step sequence instead
                cond_rebuild_ = false;
                body_counting_ = false;
            }
            it = graphs_.emplace(key, rec).first;
        }
        st = check(cudaGraphLaunch(it->second.exec, stream_), "graph launch", err);
        if (st) return st;
        g_launches.fetch_add(it->second.kernels);
        if (instrument_) {
            st = sync(err);
            if (st) return st;
            for (int64_t q = 0; q < g; ++q)
                for (int t = 0; t < 5; ++t) {
                    float ms = 0.f;
                    st = check(cudaEventElapsedTime(&ms, it->second.ev[6 * q + t], it->second.ev[6 * q + t + 1]),
                               "event timing", err);
                    if (st) return st;
                    stage_ms_[t] += ms;
                }
            // the ring kernels (fused steps) belong to the step-end stage
            float ms = 0.f;
            st = check(cudaEventElapsedTime(&ms, it->second.ev[6 * g - 1], it->second.ev[6 * g]), "event timing", err);
            if (st) return st;
            stage_ms_[4] += ms;
            stage_steps_ += g;
        }
        k -= g;
    }
    return check(cudaGetLastError(), "run", err);
}

pis_status Engine::download(int slot, double* pos, double* vel, double* force, std::string& err) {
    const SysParams& p = hp_[slot];
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (!pos && !vel && !force) return PIS_OK;
    const int cur = ss.cur;
    LAUNCH(k_store_slot, (unsigned)((p.n + 255) / 256), 256, *d_, p.a0, p.n, cur, pos ? 1 : 0, vel ? 1 : 0,
           force ? 1 : 0);
    st = check(cudaGetLastError(), "download", err);
    if (st) return st;
    const size_t bytes = 24 * (size_t)p.n;
    if (pos) {
        st = check(cudaMemcpyAsync(pos, d_->pos[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (vel) {
        st = check(cudaMemcpyAsync(vel, d_->vel[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (force) {
        st = check(cudaMemcpyAsync(force, d_->acc[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    return sync(err);
}

pis_status Engine::read_state(int slot, SysState& ss, std::string& err) {
    pis_status st = check(cudaMemcpyAsync(&ss, d_->st + slot, sizeof(SysState), cudaMemcpyDeviceToHost, stream_), "state", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::snapshot_states(SysState* host, cudaEvent_t done, std::string& err) {
    pis_status st = check(cudaMemcpyAsync(host, d_->st, sizeof(SysState) * opt_.max_slots, cudaMemcpyDeviceToHost,
                                          stream_), "state", err);
    if (st) return st;
    return check(cudaEventRecord(done, stream_), "state", err);
}

pis_status Engine::read_states(std::vector<SysState>& out, std::string& err) {
    out.resize(opt_.max_slots);
    pis_status st = check(cudaMemcpyAsync(out.data(), d_->st, sizeof(SysState) * opt_.max_slots,
                                          cudaMemcpyDeviceToHost, stream_), "state", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::set_thermo(int slot, bool on, std::string& err) {
    if (slot_thermo_.size() != hp_.size()) slot_thermo_.assign(hp_.size(), 0);
    if (slot_thermo_[slot] != (on ? 1 : 0)) {
        thermo_slots_ += on ? 1 : -1;
        slot_thermo_[slot] = on ? 1 : 0;
    }
    const int32_t v = on ? 1 : 0;
    pis_status st = check(cudaMemcpyAsync(&d_->st[slot].thermo, &v, 4, cudaMemcpyHostToDevice, stream_), "thermo", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::read_history(int slot, int64_t n, double* pe, double* ke, double* trace, std::string& err) {
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (n > opt_.hist || n > ss.steps_done) {
        err = "history holds fewer steps than requested";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    double* outs[3] = {pe, ke, trace};
    double* rings[3] = {d_->pe_hist, d_->ke_hist, d_->tr_hist};
    std::vector<double> ring(opt_.hist);
    for (int r = 0; r < 3; ++r) {
        if (!outs[r]) continue;
        st = check(cudaMemcpyAsync(ring.data(), rings[r] + (int64_t)slot * opt_.hist, 8 * opt_.hist,
                                   cudaMemcpyDeviceToHost, stream_), "history", err);
        if (st) return st;
        st = sync(err);
        if (st) return st;
        for (int64_t q = 0; q < n; ++q) outs[r][q] = ring[(ss.steps_done - n + q) % opt_.hist];
    }
    return PIS_OK;
}

pis_status Engine::read_pe_history(int slot, int64_t n, double* out, std::string& err) {
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (n > opt_.hist || n > ss.steps_done) {
        err = "energy history holds fewer steps than requested";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    std::vector<double> ring(opt_.hist);
    st = check(cudaMemcpyAsync(ring.data(), d_->pe_hist + (int64_t)slot * opt_.hist, 8 * opt_.hist,
                               cudaMemcpyDeviceToHost, stream_), "history", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    for (int64_t q = 0; q < n; ++q) out[q] = ring[(ss.steps_done - n + q) % opt_.hist];
    return PIS_OK;
}

pis_status Engine::list_entries(int slot, int64_t& total, std::string& err) {
    const SysParams& p = hp_[slot];
    if (opt_.cluster) {
        SysState ss;
        pis_status st = read_state(slot, ss, err);
        if (st) return st;
        std::vector<int32_t> nn(ss.ncl);
        st = check(cudaMemcpyAsync(nn.data(), d_->cl_nn + p.cl0, 4 * (size_t)ss.ncl, cudaMemcpyDeviceToHost, stream_),
                   "nn", err);
        if (st) return st;
        st = sync(err);
        if (st) return st;
        total = 0;
        for (int32_t v : nn) total += v;
        return PIS_OK;
    }
    std::vector<int32_t> nn(p.n);
    pis_status st = check(cudaMemcpyAsync(nn.data(), d_->nn + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    total = 0;
    for (int32_t v : nn) total += v;
    return PIS_OK;
}

pis_status Engine::neighbour_sets(int slot, std::vector<int64_t>& offsets, std::vector<int32_t>& idx,
                                  std::string& err) {
    const SysParams& p = hp_[slot];
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (opt_.cluster) return neighbour_sets_cluster(slot, ss, offsets, idx, err);
    if (!d_->keep) {
        st = check(cudaMalloc(&d_->keep, (size_t)npad_ * cap_), "keep mask", err);
        if (st) return st;
    }
    LAUNCH(k_keep, (unsigned)max_chunks_, opt_.blk, *d_, slot);
    st = check(cudaGetLastError(), "keep", err);
    if (st) return st;
    std::vector<int32_t> nn(p.n), id(p.n);
    st = check(cudaMemcpyAsync(nn.data(), d_->nn + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(id.data(), d_->id[ss.cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "id", err);
    if (st) return st;
    int32_t maxnn = 0;
    st = sync(err);
    if (st) return st;
    for (int32_t v : nn) maxnn = std::max(maxnn, v);
    const int L = d_->lq;
    const int groups = (maxnn + L - 1) / L;
    const size_t gsz = (size_t)p.n * L;  // words of one row group for this slot's atoms
    std::vector<uint32_t> ent((size_t)groups * gsz);
    std::vector<uint8_t> kp((size_t)groups * gsz);
    for (int r = 0; r < groups; ++r) {
        const int64_t off = (int64_t)r * npad_ * L + p.a0 * L;
        st = check(cudaMemcpyAsync(ent.data() + r * gsz, d_->nbr + off, 4 * gsz, cudaMemcpyDeviceToHost, stream_), "nbr", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(kp.data() + r * gsz, d_->keep + off, gsz, cudaMemcpyDeviceToHost, stream_), "keep", err);
        if (st) return st;
    }
    st = sync(err);
    if (st) return st;
    std::vector<std::vector<int32_t>> sets(p.n);
    for (int i = 0; i < p.n; ++i)
        for (int k = 0; k < nn[i]; ++k) {
            const size_t q = (size_t)(k / L) * gsz + (size_t)i * L + k % L;
            if (!kp[q]) continue;
            int j = (int)(ent[q] & JMASK) - (int)p.a0;
            sets[id[i]].push_back(id[j]);
            if (half_) sets[id[j]].push_back(id[i]);
        }
    offsets.assign(p.n + 1, 0);
    idx.clear();
    for (int i = 0; i < p.n; ++i) {
        std::sort(sets[i].begin(), sets[i].end());
        idx.insert(idx.end(), sets[i].begin(), sets[i].end());
        offsets[i + 1] = (int64_t)idx.size();
    }
    return PIS_OK;
}

// Per-atom sets from the cluster lists: every (member, entry) pair that passes the exact cutoff
// test, in original indices, sorted; an atom listed under two images (two-cell axes) counts once.
pis_status Engine::neighbour_sets_cluster(int slot, const SysState& ss, std::vector<int64_t>& offsets,
                                          std::vector<int32_t>& idx, std::string& err) {
    const SysParams& p = hp_[slot];
    pis_status st;
    if (!d_->keep) {
        st = check(cudaMalloc(&d_->keep, (size_t)clpad_ * ccap_), "keep mask", err);
        if (st) return st;
    }
    LAUNCH(k_keep_cl, (unsigned)max_cchunks_, CL_THREADS, *d_, slot);
    st = check(cudaGetLastError(), "keep", err);
    if (st) return st;
    const size_t ncl = (size_t)ss.ncl;
    std::vector<int32_t> atom(ncl), nn(ncl), id(p.n);
    st = check(cudaMemcpyAsync(atom.data(), d_->cl_atom + p.cl0, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "clusters", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(nn.data(), d_->cl_nn + p.cl0, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(id.data(), d_->id[ss.cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "id", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    int32_t maxnn = 0;
    for (int32_t v : nn) maxnn = std::max(maxnn, v);
    std::vector<uint32_t> ent((size_t)maxnn * ncl);
    std::vector<uint8_t> kp((size_t)maxnn * ncl);
    for (int r = 0; r < maxnn; ++r) {
        const int64_t off = (int64_t)r * clpad_ + p.cl0;
        st = check(cudaMemcpyAsync(ent.data() + r * ncl, d_->cl_nbr + off, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "nbr", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(kp.data() + r * ncl, d_->keep + off, ncl, cudaMemcpyDeviceToHost, stream_), "keep", err);
        if (st) return st;
    }
    st = sync(err);
    if (st) return st;
    std::vector<std::vector<int32_t>> sets(p.n);
    for (size_t c = 0; c < ncl; ++c) {
        const uint32_t pk = (uint32_t)atom[c];
        const int first = (int)(pk & JMASK) - (int)p.a0, n = (int)(pk >> JBITS) + 1;
        for (int k = 0; k < nn[c]; ++k) {
            const uint8_t mask = kp[(size_t)k * ncl + c];
            if (!mask) continue;
            const int j = (int)(ent[(size_t)k * ncl + c] & JMASK) - (int)p.a0;
            for (int m = 0; m < n; ++m)
                if (mask & (1u << m)) sets[id[first + m]].push_back(id[j]);
        }
    }
    offsets.assign(p.n + 1, 0);
    idx.clear();
    for (int i = 0; i < p.n; ++i) {
        std::sort(sets[i].begin(), sets[i].end());
        sets[i].erase(std::unique(sets[i].begin(), sets[i].end()), sets[i].end());
        idx.insert(idx.end(), sets[i].begin(), sets[i].end());
        offsets[i + 1] = (int64_t)idx.size();
    }
    return PIS_OK;
}

// Checkpoint of one slot: its current positions, velocities, accelerations, forces and original
// indices (device order) and its SysState. Restoring writes them back into the buffer set they came
// from and asks for a list rebuild, so the next step starts exactly from the saved state.
pis_status Engine::save_state(int slot, std::string& err) {
    const SysParams& p = hp_[slot];
    const size_t NA = (size_t)opt_.max_atoms;
    if (!save_) {
        pis_status st = check(cudaMalloc(&save_, (4 * 32 + 4) * NA), "checkpoint allocation", err);
        if (st) return st;
    }
    pis_status st = read_state(slot, save_state_, err);
    if (st) return st;
    const int cur = save_state_.cur;
    char* b = (char*)save_;
    const size_t n32 = 32 * (size_t)p.n, a32 = 32 * (size_t)p.a0;
    const void* src[4] = {d_->pos[cur], d_->vel[cur], d_->acc[cur], d_->frc};
    for (int k = 0; k < 4; ++k) {
        st = check(cudaMemcpyAsync(b + 32 * NA * k, (const char*)src[k] + a32, n32, cudaMemcpyDeviceToDevice, stream_),
                   "checkpoint", err);
        if (st) return st;
    }
    st = check(cudaMemcpyAsync(b + 128 * NA, d_->id[cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToDevice, stream_),
               "checkpoint", err);
    if (st) return st;
    save_slot_ = slot;
    return PIS_OK;
}

pis_status Engine::restore_state(int slot, std::string& err) {
    if (save_slot_ != slot || !save_) {
        err = "no checkpoint of this slot";
        return PIS_ERR_STATE;
    }
    const SysParams& p = hp_[slot];
    const size_t NA = (size_t)opt_.max_atoms;
    SysState ss = save_state_;
    const int cur = ss.cur;
    const char* b = (const char*)save_;
    const size_t n32 = 32 * (size_t)p.n, a32 = 32 * (size_t)p.a0;
    void* dst[4] = {d_->pos[cur], d_->vel[cur], d_->acc[cur], d_->frc};
    pis_status st = PIS_OK;
    for (int k = 0; k < 4; ++k) {
        st = check(cudaMemcpyAsync((char*)dst[k] + a32, b + 32 * NA * k, n32, cudaMemcpyDeviceToDevice, stream_),
                   "restore", err);
        if (st) return st;
    }
    st = check(cudaMemcpyAsync(d_->id[cur] + p.a0, b + 128 * NA, 4 * (size_t)p.n, cudaMemcpyDeviceToDevice, stream_),
               "restore", err);
    if (st) return st;
    ss.rebuild = 1;
    ss.flags = 0;
    ss.need_nn = 0;
    st = check(cudaMemcpyAsync(d_->st + slot, &ss, sizeof(ss), cudaMemcpyHostToDevice, stream_), "restore", err);
    if (st) return st;
    return sync(err);
}

// A larger per-atom list: entry k of atom i sits at (k / lq) * npad * lq + i * lq + k % lq whatever
// the capacity, so the grown array only adds rows of groups; graphs captured with the old pointer
// and capacity are dropped.
pis_status Engine::grow_list(int64_t new_cap, std::string& err) {
    if (opt_.cluster) {
        err = "the cluster-list variant does not grow its list";
        return PIS_ERR_UNSUPPORTED;
    }
    new_cap = (new_cap + 31) / 32 * 32;
    if (new_cap <= cap_) return PIS_OK;
    if ((double)npad_ * (double)new_cap >= 4294967296.0) {
        err = "neighbour list of the pool would exceed 2^32 entries (atoms x capacity)";
        return PIS_ERR_NO_MEMORY;
    }
    void* p = nullptr;
    pis_status st = check(cudaMalloc(&p, 4 * (size_t)npad_ * (size_t)new_cap), "list allocation", err);
    if (st) return st;
    st = sync(err);
    if (st) {
        cudaFree(p);
        return st;
    }
    if (nbr_own_) cudaFree(nbr_own_);
    nbr_own_ = p;
    d_->nbr = (uint32_t*)p;
    if (d_->keep) {  // the export mask is sized by the capacity: reallocated on next use
        cudaFree(d_->keep);
        d_->keep = nullptr;
    }
    d_->cap = (int32_t)new_cap;
    cap_ = new_cap;
    for (auto& kv : graphs_) {
        cudaGraphExecDestroy(kv.second.exec);
        for (auto e : kv.second.ev) cudaEventDestroy(e);
    }
    graphs_.clear();
    // every slot's list is rebuilt at its next step or evaluation
    std::vector<SysState> all;
    st = read_states(all, err);
    if (st) return st;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (hp_[s].active) all[s].rebuild = 1;
    st = check(cudaMemcpyAsync(d_->st, all.data(), sizeof(SysState) * all.size(), cudaMemcpyHostToDevice, stream_),
               "list growth", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::scale_velocities(int slot, const double* m, std::string& err) {
    Mat3Arg M;
    for (int k = 0; k < 9; ++k) M.m[k] = m[k];
    LAUNCH(k_scale_vel, (unsigned)max_chunks_, opt_.blk, *d_, slot, M);
    pis_status st = check(cudaGetLastError(), "scale velocities", err);
    if (st) return st;
    return sync(err);
}

// Atoms::scale_box (src/atoms/transformations.rs:5-16): h <- M h, h^-1 <- inverse(h), positions
// carried in fractional coordinates. The cell grid keeps its counts (the pool's cell ranges are
// fixed); the box may not shrink below one list radius per cell. Everything is checked before any
// state changes.
pis_status Engine::scale_box(int slot, const double* m, std::string& err) {
    SysParams p = hp_[slot];
    double nh[9], nhi[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            nh[3 * r + c] = m[3 * r] * p.H[c] + m[3 * r + 1] * p.H[3 + c] + m[3 * r + 2] * p.H[6 + c];
    if (!inverse3_ref(nh, nhi)) {
        err = "scaled box matrix is singular";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (!diagonal_box(nh) && !triclinic_capable()) {
        err = "box scaling that tilts the box needs the FP64 path with exact arithmetic, one thread per atom";
        return PIS_ERR_UNSUPPORTED;
    }
    const double rl = slot_rlist_[slot];
    double w[3];
    box_widths(nh, w);
    for (int a = 0; a < 3; ++a) {
        if (!(w[a] > 2.0 * rl)) {
            err = "scaled box is shorter than 2 (rcut + skin)";
            return PIS_ERR_BOX_TOO_SMALL;
        }
        if (w[a] / p.nc[a] < rl) {
            err = "box shrank below the cell size; re-create the state to re-grid";
            return PIS_ERR_UNSUPPORTED;
        }
    }
    if (!diagonal_box(nh) && (p.nc[0] < 3 || p.nc[1] < 3 || p.nc[2] < 3)) {
        err = "a triclinic box needs at least 3 cells of the list radius across each pair of faces";
        return PIS_ERR_BOX_TOO_SMALL;
    }
    Mat3Arg hi_old, h_new;
    for (int k = 0; k < 9; ++k) {
        hi_old.m[k] = p.HI[k];
        h_new.m[k] = nh[k];
    }
    const int full = (p.tric || !diagonal_box(nh)) ? 1 : 0;
    set_box(p, nh, nhi, rl * (1.0 + 1e-5));
    reference_cells(nh, slot_rcmax_[slot], p.rnc);
    if (opt_.ref_order && !reference_cells_ok(p.rnc)) {
        err = "reference-order forces need at least 3 cells of the largest cutoff per axis";
        return PIS_ERR_UNSUPPORTED;
    }
    // the 27-cell walk's two-cell condition for the new edges
    p.walk27 = walk27_valid(p, rl * (1.0 + 1e-5));
    // the FP32 pair constants follow the coordinate unit (the x cell edge)
    std::vector<LJDev>& tab = slot_tab_host_[slot];
    for (auto& t : tab)
        if (t.present) set_fp32_constants(t, p.sc);
    pis_status st = check(cudaMemcpyAsync(d_->tab + p.tab0, tab.data(), sizeof(LJDev) * tab.size(),
                                          cudaMemcpyHostToDevice, stream_), "table upload", err);
    if (st) return st;
    LAUNCH(k_scale_pos, (unsigned)max_chunks_, opt_.blk, *d_, slot, hi_old, h_new, full);
    if (p.tric && !any_tric_) dirty_map_ = true;  // the next launch selects the triclinic kernels
    if (!p.walk27 && !any_generic_) dirty_map_ = true;  // ... or launches the generic list walk
    hp_[slot] = p;
    st = check(cudaMemcpyAsync(d_->sp + slot, &hp_[slot], sizeof(SysParams), cudaMemcpyHostToDevice, stream_),
               "params", err);
    if (st) return st;
    int32_t one = 1;
    st = check(cudaMemcpyAsync(&d_->st[slot].rebuild, &one, 4, cudaMemcpyHostToDevice, stream_), "params", err);
    if (st) return st;
    return sync(err);
}

}  // namespace pis
