// pis_gpu.cu - single-system C ABI (include/pis_gpu.h) over the packed engine.
//
// A pis_gpu_ctx is the GPU counterpart of one PotentialManager bound to one Atoms state: the
// pair table is fixed at creation, set_state places the atoms in a one-slot engine pool, and
// compute_potential / verlet_step_nve run on the device with the state kept resident.
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"
#include "pis_gpu.h"

struct pis_gpu_ctx {
    std::vector<pis::LJHost> table;
    int n_types = 0;
    double skin = 0.3;
    int precision = PIS_PRECISION_FP64;
    int list_kind = PIS_LIST_DEFAULT;
    bool fp64_fast = false;
    bool mixed_kahan = false;
    int lpa = 1;
    int mix_batch = 4;
    bool list_tma = false;
    int cluster = 0;
    int build_cluster = 0;
    bool cell_tiles = false;
    bool plain_graphs = false;
    bool unfused = false;
    bool ref_order = false;
    int list_cap_req = 0;   // per-atom list capacity asked for (0 = from the density)
    bool auto_grow = true;  // grow the list and run again when it overflows
    int64_t wait_limit = -1;  // polls of a bulk-copy pipeline wait (< 0: the default)
    std::unique_ptr<pis::Engine> eng;
    pis::PoolOptions pool;  // options the current engine was created with
    int slot = -1;
    int64_t n = 0;
    double dt = 0.0;
    std::string err;
};

namespace {

pis_status fail(pis_gpu_ctx* ctx, pis_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}

bool have_state(pis_gpu_ctx* ctx) { return ctx && ctx->eng && ctx->slot >= 0; }

// Per-atom list capacity from the mean density: 1.6x the expected full-list count + 32.
int list_capacity(int64_t n, const double* h_rowmajor, double rlist) {
    double vol = std::fabs(h_rowmajor[0] * h_rowmajor[4] * h_rowmajor[8]);
    double rho = vol > 0 ? (double)n / vol : 0.0;
    double full = rho * 4.0 / 3.0 * M_PI * rlist * rlist * rlist;
    double cap = 1.6 * full + 32.0;
    if (cap > 4096) cap = 4096;
    return ((int)std::ceil(cap) + 7) / 8 * 8;
}

// Two states with equal pool options (atom count, cell grid, list capacity, variants) share one
// engine: its memory and captured step graphs are reused.
bool same_pool(const pis::PoolOptions& a, const pis::PoolOptions& b) {
    return a.precision == b.precision && a.list_kind == b.list_kind && a.blk == b.blk && a.list_cap == b.list_cap &&
           a.max_atoms == b.max_atoms && a.max_slots == b.max_slots && a.max_cells == b.max_cells &&
           a.max_types_total == b.max_types_total && a.hist == b.hist && a.fp64_fast == b.fp64_fast &&
           a.mixed_kahan == b.mixed_kahan && a.lpa == b.lpa && a.mix_batch == b.mix_batch &&
           a.list_tma == b.list_tma && a.cluster == b.cluster && a.build_cluster == b.build_cluster &&
           a.cell_tiles == b.cell_tiles && a.plain_graphs == b.plain_graphs &&
           a.unfused == b.unfused && a.ref_order == b.ref_order && a.wait_limit == b.wait_limit;
}

pis_status flags_to_status(pis_gpu_ctx* ctx, const pis::SysState& ss) {
    if (ss.flags & pis::FLAG_NAN) return fail(ctx, PIS_ERR_NAN_DETECTED, "NaN detected in positions or energies");
    if (ss.flags & pis::FLAG_LIST_OVERFLOW)
        return fail(ctx, PIS_ERR_LIST_OVERFLOW, "neighbour list capacity exceeded; results are invalid");
    if (ss.flags & pis::FLAG_TIMEOUT)
        return fail(ctx, PIS_ERR_TIMEOUT, "a device-side wait expired; results are invalid");
    return PIS_OK;
}

// After a list overflow: a capacity that holds the longest list the build asked for, with room.
int64_t grown_capacity(const pis::Engine& e, const pis::SysState& ss) {
    const int64_t cap = e.list_cap();
    const int64_t need = (int64_t)ss.need_nn + ss.need_nn / 8 + 8;
    return std::max(cap + cap / 4, need);
}

bool overflowed(const pis::SysState& ss) { return (ss.flags & pis::FLAG_LIST_OVERFLOW) != 0; }

constexpr int MAX_GROWTH = 6;  // list growths per call before the overflow is returned

pis_status compute_with_growth(pis_gpu_ctx* ctx, pis::SysState& ss, std::string& err) {
    pis::Engine& e = *ctx->eng;
    const bool grow = ctx->auto_grow && e.per_atom_list();
    for (int attempt = 0;; ++attempt) {
        pis_status st = PIS_OK;
        if (grow) {
            st = e.save_state(ctx->slot, err);
            if (st) return st;
        }
        st = e.compute_potential(err);
        if (st) return st;
        st = e.read_state(ctx->slot, ss, err);
        if (st) return st;
        if (!grow || !overflowed(ss) || attempt >= MAX_GROWTH) return PIS_OK;
        st = e.grow_list(grown_capacity(e, ss), err);
        if (st) return st;
        st = e.restore_state(ctx->slot, err);
        if (st) return st;
    }
}

}  // namespace

extern "C" {

pis_status pis_gpu_create(const pis_lj_pair* table, int32_t n_pairs, int32_t n_types, double skin,
                          int32_t precision, pis_gpu_ctx** out) {
    if (!out) return PIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n_types < 1 || n_types > 8) return PIS_ERR_INVALID_ARGUMENT;
    if (n_pairs < 1 || !table) return PIS_ERR_MISSING_POTENTIAL;
    if (!(skin >= 0.0)) return PIS_ERR_INVALID_ARGUMENT;
    if (precision != PIS_PRECISION_FP64 && precision != PIS_PRECISION_MIXED) return PIS_ERR_INVALID_ARGUMENT;
    auto* ctx = new pis_gpu_ctx();
    ctx->n_types = n_types;
    ctx->skin = skin;
    ctx->precision = precision;
    ctx->table.assign((size_t)n_types * n_types, pis::LJHost{});
    for (int k = 0; k < n_pairs; ++k) {
        const pis_lj_pair& p = table[k];
        if (p.ti < 1 || p.tj < 1 || p.ti > n_types || p.tj > n_types || !(p.rcut > 0.0) || !(p.sigma > 0.0)) {
            delete ctx;
            return PIS_ERR_INVALID_ARGUMENT;
        }
        pis::LJHost e;
        e.epsilon = p.epsilon;
        e.sigma = p.sigma;
        e.rcut = p.rcut;
        e.present = 1;
        e.shift = p.shift;
        // the reference looks pairs up by (min, max) type (src/potentials/potential.rs:181-192)
        ctx->table[(size_t)(p.ti - 1) * n_types + (p.tj - 1)] = e;
        ctx->table[(size_t)(p.tj - 1) * n_types + (p.ti - 1)] = e;
    }
    *out = ctx;
    return PIS_OK;
}

pis_status pis_gpu_set_options(pis_gpu_ctx* ctx, int32_t list_kind, int32_t flags) {
    if (!ctx) return PIS_ERR_INVALID_ARGUMENT;
    if (list_kind < PIS_LIST_DEFAULT || list_kind > PIS_LIST_FULL)
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "unknown list kind");
    if (flags & ~(PIS_OPT_FP64_FAST | PIS_OPT_MIXED_KAHAN | PIS_OPT_LIST_TMA | PIS_OPT_TILE | PIS_OPT_PLAIN_GRAPHS | PIS_OPT_UNFUSED | PIS_OPT_REF_ORDER |
                  PIS_OPT_LANES(0xff) | PIS_OPT_BATCH(0xff) | PIS_OPT_CLUSTER(0xf) | PIS_OPT_SCAN(0x7)))
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "unknown option flag");
    const int batch = (flags >> 16) & 0xff;
    if (batch != 0 && batch != 4 && batch != 8 && batch != 16)
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "batch must be 4, 8 or 16");
    ctx->mix_batch = batch ? batch : 4;
    const int lanes = (flags >> 8) & 0xff;
    const int cl_req = (flags >> 24) & 0xf;
    if (lanes != 0 && lanes != 1 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32 &&
        !(lanes == 2 && cl_req == 2))
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "lanes per atom must be 1, 4, 8, 16 or 32 (2 only with clusters of 2)");
    ctx->lpa = lanes ? lanes : 1;
    ctx->fp64_fast = (flags & PIS_OPT_FP64_FAST) != 0;
    ctx->mixed_kahan = (flags & PIS_OPT_MIXED_KAHAN) != 0;
    ctx->list_tma = (flags & PIS_OPT_LIST_TMA) != 0;
    const int cl = (flags >> 24) & 0xf;
    if (cl > 1 && cl != 2 && cl != 4) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "atoms per cluster must be 1, 2 or 4");
    ctx->cluster = cl > 1 ? cl : 0;
    const int scan = (flags >> 28) & 0x7;
    if (scan != 0 && scan != 1 && scan != 2 && scan != 4)
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "atoms per build cluster must be 1, 2 or 4");
    ctx->build_cluster = scan;
    ctx->cell_tiles = (flags & PIS_OPT_TILE) != 0;
    ctx->plain_graphs = (flags & PIS_OPT_PLAIN_GRAPHS) != 0;
    ctx->unfused = (flags & PIS_OPT_UNFUSED) != 0;
    ctx->ref_order = (flags & PIS_OPT_REF_ORDER) != 0;
    if (ctx->ref_order && (ctx->precision != PIS_PRECISION_FP64 || list_kind == PIS_LIST_HALF || ctx->lpa != 1 ||
                           ctx->fp64_fast))
        return fail(ctx, PIS_ERR_UNSUPPORTED,
                    "reference-order forces need FP64 precision, a full list, one thread per atom, exact arithmetic");
    if (ctx->cell_tiles && (ctx->precision != PIS_PRECISION_MIXED || ctx->lpa != 1 || ctx->list_tma || ctx->cluster))
        return fail(ctx, PIS_ERR_UNSUPPORTED, "neighbour-cell tiles need the mixed path, thread per atom, per-atom lists");
    if (ctx->cluster && (ctx->precision != PIS_PRECISION_MIXED || (ctx->lpa != 1 && ctx->lpa != ctx->cluster) ||
                         ctx->list_tma))
        return fail(ctx, PIS_ERR_UNSUPPORTED,
                    "the cluster list needs the mixed path, one thread per cluster or one lane per member");
    if (ctx->list_tma && (ctx->precision != PIS_PRECISION_MIXED || ctx->lpa != 1))
        return fail(ctx, PIS_ERR_UNSUPPORTED, "the bulk-copy list stream needs the mixed path, thread per atom");
    if (ctx->precision == PIS_PRECISION_MIXED && list_kind == PIS_LIST_HALF &&
        (ctx->lpa != 1 || ctx->list_tma || ctx->cell_tiles || ctx->cluster || ctx->build_cluster > 1))
        return fail(ctx, PIS_ERR_UNSUPPORTED,
                    "the mixed-precision half list is a variant of the thread-per-atom force kernel");
    ctx->list_kind = list_kind;
    return PIS_OK;
}

pis_status pis_gpu_set_state(pis_gpu_ctx* ctx, int64_t n, const int32_t* type_ids, const double* masses_per_type,
                             const double* pos, const double* vel, const double* force, const double* h_colmajor,
                             const uint8_t* pbc) {
    if (!ctx) return PIS_ERR_INVALID_ARGUMENT;
    if (n <= 0) return fail(ctx, PIS_ERR_NO_ATOMS, "no atoms defined");
    if (!type_ids || !masses_per_type || !pos || !h_colmajor)
        return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null state array");
    pis::SlotDesc d;
    d.n = n;
    d.n_types = ctx->n_types;
    d.table = ctx->table;
    d.masses.assign(masses_per_type, masses_per_type + ctx->n_types);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) d.h[3 * r + c] = h_colmajor[3 * c + r];
    for (int a = 0; a < 3; ++a) d.pbc[a] = pbc ? (pbc[a] ? 1 : 0) : 1;
    d.skin = ctx->skin;
    d.dt = ctx->dt > 0 ? ctx->dt : 0.005;
    double rc = 0.0;
    for (auto& e : d.table)
        if (e.present && e.rcut > rc) rc = e.rcut;
    double rlist = rc + ctx->skin;

    pis::PoolOptions opt;
    opt.precision = ctx->precision;
    opt.list_kind = ctx->list_kind;
    opt.fp64_fast = ctx->fp64_fast;
    opt.mixed_kahan = ctx->mixed_kahan;
    opt.lpa = ctx->lpa;
    opt.mix_batch = ctx->mix_batch;
    opt.list_tma = ctx->list_tma;
    opt.cluster = ctx->cluster;
    opt.build_cluster = ctx->build_cluster;
    opt.cell_tiles = ctx->cell_tiles;
    opt.plain_graphs = ctx->plain_graphs;
    opt.unfused = ctx->unfused;
    opt.ref_order = ctx->ref_order;
    opt.wait_limit = ctx->wait_limit;
    opt.max_atoms = n;
    opt.max_slots = 1;
    opt.max_cells = pis::Engine::cells_for(d) + 1;
    opt.max_types_total = ctx->n_types * ctx->n_types;
    opt.list_cap = ctx->list_cap_req > 0 ? ctx->list_cap_req : list_capacity(n, d.h, rlist);
    std::string err;
    if (ctx->eng && ctx->slot >= 0 && same_pool(ctx->pool, opt)) {
        // same pool shape: replace the system in place
        ctx->eng->remove_slot(ctx->slot);
        ctx->slot = -1;
        ctx->n = 0;
        int slot = ctx->eng->add_slot(d, type_ids, pos, vel, force, err);
        if (slot < 0) return fail(ctx, (pis_status)(-slot), err);
        ctx->slot = slot;
        ctx->n = n;
        return PIS_OK;
    }
    ctx->eng.reset();
    ctx->slot = -1;
    ctx->n = 0;
    auto eng = std::make_unique<pis::Engine>();
    pis_status st = eng->init(opt, err);
    if (st) return fail(ctx, st, err);
    int slot = eng->add_slot(d, type_ids, pos, vel, force, err);
    if (slot < 0) return fail(ctx, (pis_status)(-slot), err);
    ctx->eng = std::move(eng);
    ctx->pool = opt;
    ctx->slot = slot;
    ctx->n = n;
    return PIS_OK;
}

pis_status pis_gpu_set_wait_limit(pis_gpu_ctx* ctx, int64_t polls) {
    if (!ctx) return PIS_ERR_INVALID_ARGUMENT;
    ctx->wait_limit = polls;
    return PIS_OK;
}

pis_status pis_gpu_set_list_capacity(pis_gpu_ctx* ctx, int32_t per_atom, int32_t auto_grow) {
    if (!ctx) return PIS_ERR_INVALID_ARGUMENT;
    if (per_atom < 0 || per_atom > 65536) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "list capacity out of range");
    ctx->list_cap_req = per_atom;
    ctx->auto_grow = auto_grow != 0;
    return PIS_OK;
}

pis_status pis_gpu_compute_potential(pis_gpu_ctx* ctx, double* pe_out, double* forces) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    std::string err;
    pis::SysState ss;
    pis_status st = compute_with_growth(ctx, ss, err);
    if (st) return fail(ctx, st, err);
    if (pe_out) *pe_out = ss.pe;
    if (forces) {
        st = ctx->eng->download(ctx->slot, nullptr, nullptr, forces, err);
        if (st) return fail(ctx, st, err);
    }
    return flags_to_status(ctx, ss);
}

pis_status pis_gpu_verlet_step_nve(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* pe_out) {
    return pis_gpu_verlet_step_nve_thermo(ctx, dt, n_steps, pe_out, nullptr, nullptr);
}

pis_status pis_gpu_verlet_step_nve_thermo(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* pe_out, double* ke_out,
                                          double* virial_trace_out) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (n_steps < 0 || !(dt == dt)) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "bad step count or dt");
    std::string err;
    pis_status st = ctx->eng->set_dt(ctx->slot, dt, err);
    if (st) return fail(ctx, st, err);
    ctx->dt = dt;
    const int64_t chunk = 1000;  // within the 1024-step history rings
    int64_t done = 0;
    pis::Engine& e = *ctx->eng;
    const bool grow = ctx->auto_grow && e.per_atom_list();
    const bool thermo = virial_trace_out != nullptr;
    if (thermo) {
        st = e.set_thermo(ctx->slot, true, err);
        if (st) return fail(ctx, st, err);
    }
    auto finish = [&](pis_status r) {
        if (thermo) {
            std::string e2;
            e.set_thermo(ctx->slot, false, e2);
        }
        return r;
    };
    while (done < n_steps) {
        int64_t k = std::min(chunk, n_steps - done);
        pis::SysState ss;
        // a chunk whose list overflowed is run again from its checkpoint with a larger list
        for (int attempt = 0;; ++attempt) {
            if (grow) {
                st = e.save_state(ctx->slot, err);
                if (st) return finish(fail(ctx, st, err));
            }
            st = e.set_steps(ctx->slot, k, err);
            if (st) return finish(fail(ctx, st, err));
            st = e.run(k, err);
            if (st) return finish(fail(ctx, st, err));
            st = e.read_state(ctx->slot, ss, err);
            if (st) return finish(fail(ctx, st, err));
            if (!grow || !overflowed(ss) || attempt >= MAX_GROWTH) break;
            st = e.grow_list(grown_capacity(e, ss), err);
            if (st) return finish(fail(ctx, st, err));
            st = e.restore_state(ctx->slot, err);
            if (st) return finish(fail(ctx, st, err));
        }
        if (pe_out || ke_out || virial_trace_out) {
            st = e.read_history(ctx->slot, k, pe_out ? pe_out + done : nullptr, ke_out ? ke_out + done : nullptr,
                                virial_trace_out ? virial_trace_out + done : nullptr, err);
            if (st) return finish(fail(ctx, st, err));
        }
        st = flags_to_status(ctx, ss);
        if (st) return finish(st);
        done += k;
    }
    return finish(PIS_OK);
}

pis_status pis_gpu_run_timed(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* device_ms, double* stage_ms) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (n_steps < 1 || !(dt == dt)) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "bad step count or dt");
    std::string err;
    pis::Engine& e = *ctx->eng;
    pis_status st = e.set_dt(ctx->slot, dt, err);
    if (st) return fail(ctx, st, err);
    ctx->dt = dt;
    st = e.set_steps(ctx->slot, n_steps, err);
    if (st) return fail(ctx, st, err);
    e.set_instrument(stage_ms != nullptr);
    e.reset_stage_times();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, e.stream());
    st = e.run(n_steps, err);
    cudaEventRecord(b, e.stream());
    cudaError_t ce = cudaEventSynchronize(b);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    e.set_instrument(false);
    if (st) return fail(ctx, st, err);
    if (ce != cudaSuccess) return fail(ctx, PIS_ERR_CUDA, cudaGetErrorString(ce));
    if (device_ms) *device_ms = ms;
    if (stage_ms)
        for (int t = 0; t < 5; ++t) stage_ms[t] = e.stage_ms()[t];
    pis::SysState ss;
    st = e.read_state(ctx->slot, ss, err);
    if (st) return fail(ctx, st, err);
    return flags_to_status(ctx, ss);
}

pis_status pis_gpu_get_state(pis_gpu_ctx* ctx, double* pos, double* vel, double* force) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    std::string err;
    pis_status st = ctx->eng->download(ctx->slot, pos, vel, force, err);
    return st ? fail(ctx, st, err) : PIS_OK;
}

pis_status pis_gpu_reductions(pis_gpu_ctx* ctx, double* ke, double* virial) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    std::string err;
    pis_status st = ctx->eng->reduce_state(virial != nullptr, err);
    if (st) return fail(ctx, st, err);
    pis::SysState ss;
    st = ctx->eng->read_state(ctx->slot, ss, err);
    if (st) return fail(ctx, st, err);
    if (ke) *ke = ss.ke;
    if (virial)
        for (int q = 0; q < 9; ++q) virial[q] = ss.virial[q];
    return PIS_OK;
}

pis_status pis_gpu_neighbour_list(pis_gpu_ctx* ctx, int64_t* offsets, int32_t* idx, int64_t cap, int64_t* total) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!offsets) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "offsets is null");
    std::string err;
    pis::SysState ss;
    pis_status st = ctx->eng->read_state(ctx->slot, ss, err);
    if (st) return fail(ctx, st, err);
    if (ss.rebuild) {
        // no list for the current positions yet: evaluate once (builds it)
        st = ctx->eng->compute_potential(err);
        if (st) return fail(ctx, st, err);
    }
    std::vector<int64_t> off;
    std::vector<int32_t> id;
    st = ctx->eng->neighbour_sets(ctx->slot, off, id, err);
    if (st) return fail(ctx, st, err);
    std::memcpy(offsets, off.data(), sizeof(int64_t) * off.size());
    if (idx) std::memcpy(idx, id.data(), sizeof(int32_t) * (size_t)std::min<int64_t>(cap, (int64_t)id.size()));
    if (total) *total = (int64_t)id.size();
    return PIS_OK;
}

pis_status pis_gpu_scale_velocities(pis_gpu_ctx* ctx, const double* m) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!m) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null matrix");
    std::string err;
    pis_status st = ctx->eng->scale_velocities(ctx->slot, m, err);
    return st ? fail(ctx, st, err) : PIS_OK;
}

pis_status pis_gpu_scale_box(pis_gpu_ctx* ctx, const double* m) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!m) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null matrix");
    std::string err;
    pis_status st = ctx->eng->scale_box(ctx->slot, m, err);
    return st ? fail(ctx, st, err) : PIS_OK;
}

pis_status pis_gpu_pressure_tensor(pis_gpu_ctx* ctx, double* p) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!p) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null output");
    std::string err;
    pis_status st = ctx->eng->reduce_state_slot(true, ctx->slot, err, true);
    if (st) return fail(ctx, st, err);
    pis::SysState ss;
    st = ctx->eng->read_state(ctx->slot, ss, err);
    if (st) return fail(ctx, st, err);
    // SimulationBox::volume (src/simulation_box.rs:67-69): |det h| by first-row cofactors
    const double* m = ctx->eng->params(ctx->slot).H;
    const double det = m[0] * (m[4] * m[8] - m[7] * m[5]) - m[1] * (m[3] * m[8] - m[6] * m[5]) +
                       m[2] * (m[3] * m[7] - m[6] * m[4]);
    const double vol = std::fabs(det);
    for (int q = 0; q < 9; ++q) p[q] = (ss.ktensor[q] + ss.virial[q]) / vol;
    return PIS_OK;
}

pis_status pis_gpu_get_box(pis_gpu_ctx* ctx, double* h_colmajor) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!h_colmajor) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null output");
    const double* m = ctx->eng->params(ctx->slot).H;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) h_colmajor[3 * c + r] = m[3 * r + c];
    return PIS_OK;
}

pis_status pis_gpu_get_stats(pis_gpu_ctx* ctx, pis_gpu_stats* out) {
    if (!have_state(ctx)) return fail(ctx, PIS_ERR_STATE, "no atoms uploaded");
    if (!out) return fail(ctx, PIS_ERR_INVALID_ARGUMENT, "null output");
    std::string err;
    pis::SysState ss;
    pis_status st = ctx->eng->read_state(ctx->slot, ss, err);
    if (st) return fail(ctx, st, err);
    int64_t entries = 0;
    st = ctx->eng->list_entries(ctx->slot, entries, err);
    if (st) return fail(ctx, st, err);
    std::memset(out, 0, sizeof(*out));
    out->n_atoms = ctx->n;
    out->steps = ss.steps_done;
    out->rebuilds = ss.rebuilds;
    out->list_entries = entries;
    out->list_capacity = (int32_t)ctx->eng->list_cap();
    const pis::SysParams& p = ctx->eng->params(ctx->slot);
    for (int a = 0; a < 3; ++a) out->cells[a] = p.nc[a];
    out->pe = ss.pe;
    out->ke = ss.ke;
    for (int q = 0; q < 9; ++q) out->virial[q] = ss.virial[q];
    out->fused_step = ctx->eng->fused_step() ? 1 : 0;
    return PIS_OK;
}

const char* pis_gpu_last_error(const pis_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void pis_gpu_destroy(pis_gpu_ctx* ctx) { delete ctx; }

int64_t pis_gpu_kernel_launches(void) { return pis::Engine::launches(); }

const char* pis_gpu_version(void) { return "pis_gb300 0.1 (sm_103a)"; }

}  // extern "C"
