// pis_batch.cu - batched replicas and the served-job loop (include/pis_gpu.h, pis_batch_*,
// pis_serve_run) over the packed engine.
//
// A batch is one engine pool sized once (atoms, slots, cells = its device-memory budget). Jobs
// are admitted into free ranges of the pool, advanced together by the step graphs, and released
// when their step count is done; admission, release and the request queue of the served loop run
// on the host between graph launches.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"
#include "pis_gpu.h"

struct pis_batch {
    pis::Engine eng;
    pis::PoolOptions opt;
    std::string err;
    std::vector<int64_t> atoms;  // per slot, 0 when free
    pis_serve_stats serve{};     // the last pis_serve_run's accounting
};

namespace {

pis_status bfail(pis_batch* b, pis_status st, const std::string& msg) {
    if (b) b->err = msg;
    return st;
}

// SplitMix64: the seeded stream behind the synthetic jobs' velocities.
struct SplitMix64 {
    uint64_t x;
    uint64_t next() {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }  // (0, 1)
};

double lj_lattice_constant(double rho) { return std::cbrt(4.0 / rho); }

// FCC lattice in the reference generator's order and Maxwell-Boltzmann velocities (Box-Muller
// pairs from SplitMix64), centre-of-mass drift removed, rescaled to T* (unit masses, k_B = 1).
void make_lj_state(const pis_lj_job& j, std::vector<double>& pos, std::vector<double>& vel, double& L) {
    const int k = j.k;
    const double a = lj_lattice_constant(j.rho);
    L = a * k;
    const int64_t n = 4ll * k * k * k;
    pos.resize(3 * n);
    vel.resize(3 * n);
    static const double B[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}};
    int64_t q = 0;
    for (int ix = 0; ix < k; ++ix)
        for (int iy = 0; iy < k; ++iy)
            for (int iz = 0; iz < k; ++iz)
                for (int b = 0; b < 4; ++b) {
                    pos[3 * q] = a * (ix + B[b][0]);
                    pos[3 * q + 1] = a * (iy + B[b][1]);
                    pos[3 * q + 2] = a * (iz + B[b][2]);
                    ++q;
                }
    SplitMix64 rng{j.seed * 0x2545f4914f6cdd1dull + 0x1234567ull};
    for (int64_t c = 0; c < 3 * n; c += 2) {
        const double u1 = rng.uniform(), u2 = rng.uniform();
        const double r = std::sqrt(-2.0 * std::log(u1));
        vel[c] = r * std::cos(2.0 * M_PI * u2);
        if (c + 1 < 3 * n) vel[c + 1] = r * std::sin(2.0 * M_PI * u2);
    }
    double p[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) p[d] += vel[3 * i + d];
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) vel[3 * i + d] -= p[d] / (double)n;
    double ke = 0.0;
    for (int64_t c = 0; c < 3 * n; ++c) ke += 0.5 * vel[c] * vel[c];
    const double t_now = 2.0 * ke / (3.0 * (double)n);
    const double lam = t_now > 0 ? std::sqrt(j.t_star / t_now) : 0.0;
    for (auto& v : vel) v *= lam;
}

pis::SlotDesc lj_desc(const pis_lj_job& j, double L) {
    pis::SlotDesc d;
    d.n = 4ll * j.k * j.k * j.k;
    d.n_types = 1;
    pis::LJHost e;
    e.epsilon = 1.0;
    e.sigma = 1.0;
    e.rcut = j.rcut;
    e.present = 1;
    e.shift = 1;
    d.table = {e};
    d.masses = {1.0};
    for (int a = 0; a < 9; ++a) d.h[a] = 0.0;
    d.h[0] = d.h[4] = d.h[8] = L;
    d.skin = j.skin;
    d.dt = j.dt;
    return d;
}

// Place a job in the pool and set its step count; `evaluate`: also its first force evaluation
// (otherwise the caller evaluates the new slots together, Engine::compute_potential_slots).
pis_status place_desc(pis_batch* b, const pis::SlotDesc& d0, const int32_t* types, const double* pos,
                      const double* vel, int64_t steps, bool evaluate, int32_t* slot_out) {
    if (steps < 0) return bfail(b, PIS_ERR_INVALID_ARGUMENT, "negative step count");
    std::string err;
    pis::SlotDesc d = d0;
    d.steps = steps;
    // without the evaluation (the serving loop): placed with the chunk map left for the next
    // evaluation, which covers every job admitted between two graphs
    int slot = b->eng.add_slot(d, types, pos, vel, nullptr, err, !evaluate);
    if (slot < 0) return bfail(b, (pis_status)(-slot), err);
    pis_status st = evaluate ? b->eng.compute_potential_slot(slot, err) : PIS_OK;
    if (st) {
        b->eng.remove_slot(slot);
        return bfail(b, st, err);
    }
    if ((int)b->atoms.size() <= slot) b->atoms.resize(slot + 1, 0);
    b->atoms[slot] = d.n;
    if (slot_out) *slot_out = slot;
    return PIS_OK;
}

pis_status admit_desc(pis_batch* b, const pis::SlotDesc& d, const int32_t* types, const double* pos,
                      const double* vel, int64_t steps, int32_t* slot_out) {
    return place_desc(b, d, types, pos, vel, steps, true, slot_out);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

pis_status pis_batch_create(int64_t max_atoms, int32_t max_slots, int64_t max_cells, int32_t precision,
                            int32_t flags, pis_batch** out) {
    if (!out) return PIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (max_atoms < 1 || max_slots < 1) return PIS_ERR_INVALID_ARGUMENT;
    auto b = std::make_unique<pis_batch>();
    b->opt.precision = precision;
    b->opt.max_atoms = max_atoms;
    b->opt.max_slots = max_slots;
    b->opt.max_cells = max_cells > 0 ? max_cells : max_atoms / 8 + 2 * (int64_t)max_slots + 64;
    b->opt.max_types_total = std::max(64, 4 * max_slots);
    b->opt.fp64_fast = (flags & PIS_OPT_FP64_FAST) != 0;
    b->opt.mixed_kahan = (flags & PIS_OPT_MIXED_KAHAN) != 0;
    const int lanes = (flags >> 8) & 0xff;
    b->opt.lpa = lanes ? lanes : 1;
    const int batch = (flags >> 16) & 0xff;
    b->opt.mix_batch = batch ? batch : 4;
    b->opt.list_tma = (flags & PIS_OPT_LIST_TMA) != 0;
    const int cl = (flags >> 24) & 0xf;
    b->opt.cluster = cl > 1 ? cl : 0;
    b->opt.build_cluster = (flags >> 28) & 0x7;
    b->opt.cell_tiles = (flags & PIS_OPT_TILE) != 0;
    b->opt.plain_graphs = (flags & PIS_OPT_PLAIN_GRAPHS) != 0;
    b->opt.unfused = (flags & PIS_OPT_UNFUSED) != 0;
    b->opt.list_cap = 224;  // density up to 0.95 at rc + skin = 2.8 (expected ~88 full-list entries)
    b->opt.hist = 1024;
    std::string err;
    pis_status st = b->eng.init(b->opt, err);
    if (st) return st;
    b->atoms.assign(max_slots, 0);
    *out = b.release();
    return PIS_OK;
}

pis_status pis_batch_admit(pis_batch* b, const pis_job* job, int32_t* slot) {
    if (!b || !job) return PIS_ERR_INVALID_ARGUMENT;
    if (job->n < 1) return bfail(b, PIS_ERR_NO_ATOMS, "no atoms defined");
    if (!job->type_ids || !job->masses_per_type || !job->pos || !job->h_colmajor || !job->table)
        return bfail(b, PIS_ERR_INVALID_ARGUMENT, "null job array");
    const int nt = job->n_types;
    if (nt < 1 || nt > 8) return bfail(b, PIS_ERR_INVALID_ARGUMENT, "1 to 8 atom types");
    pis::SlotDesc d;
    d.n = job->n;
    d.n_types = nt;
    d.table.assign((size_t)nt * nt, pis::LJHost{});
    for (int k = 0; k < job->n_pairs; ++k) {
        const pis_lj_pair& p = job->table[k];
        if (p.ti < 1 || p.tj < 1 || p.ti > nt || p.tj > nt || !(p.rcut > 0))
            return bfail(b, PIS_ERR_INVALID_ARGUMENT, "bad pair table row");
        pis::LJHost e;
        e.epsilon = p.epsilon;
        e.sigma = p.sigma;
        e.rcut = p.rcut;
        e.present = 1;
        e.shift = p.shift;
        d.table[(size_t)(p.ti - 1) * nt + (p.tj - 1)] = e;
        d.table[(size_t)(p.tj - 1) * nt + (p.ti - 1)] = e;
    }
    d.masses.assign(job->masses_per_type, job->masses_per_type + nt);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) d.h[3 * r + c] = job->h_colmajor[3 * c + r];
    d.skin = job->skin;
    d.dt = job->dt;
    return admit_desc(b, d, job->type_ids, job->pos, job->vel, job->steps, slot);
}

int32_t pis_batch_fits_lj(const pis_batch* b, const pis_lj_job* job) {
    if (!b || !job || job->k < 1) return 0;
    const double L = lj_lattice_constant(job->rho) * job->k;
    return b->eng.fits(lj_desc(*job, L)) ? 1 : 0;
}

pis_status pis_batch_admit_lj(pis_batch* b, const pis_lj_job* job, int32_t* slot) {
    if (!b || !job) return PIS_ERR_INVALID_ARGUMENT;
    if (job->k < 1 || !(job->rho > 0) || !(job->t_star >= 0) || !(job->rcut > 0))
        return bfail(b, PIS_ERR_INVALID_ARGUMENT, "bad LJ job parameters");
    std::vector<double> pos, vel;
    double L = 0;
    make_lj_state(*job, pos, vel, L);
    pis::SlotDesc d = lj_desc(*job, L);
    std::vector<int32_t> types((size_t)d.n, 1);
    return admit_desc(b, d, types.data(), pos.data(), vel.data(), job->steps, slot);
}

pis_status pis_batch_advance(pis_batch* b, int64_t k) {
    if (!b) return PIS_ERR_INVALID_ARGUMENT;
    std::string err;
    pis_status st = b->eng.run(k, err);
    if (!st) st = b->eng.sync(err);
    return st ? bfail(b, st, err) : PIS_OK;
}

pis_status pis_batch_run_timed(pis_batch* b, int64_t k, double* device_ms) {
    if (!b) return PIS_ERR_INVALID_ARGUMENT;
    std::string err;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, b->eng.stream());
    pis_status st = b->eng.run(k, err);
    cudaEventRecord(e1, b->eng.stream());
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return bfail(b, st, err);
    if (ce != cudaSuccess) return bfail(b, PIS_ERR_CUDA, cudaGetErrorString(ce));
    if (device_ms) *device_ms = ms;
    return PIS_OK;
}

pis_status pis_batch_poll(pis_batch* b, int32_t* done, int32_t cap, int32_t* n_done) {
    if (!b) return PIS_ERR_INVALID_ARGUMENT;
    std::vector<pis::SysState> ss;
    std::string err;
    pis_status st = b->eng.read_states(ss, err);
    if (st) return bfail(b, st, err);
    int32_t k = 0;
    for (int s = 0; s < (int)ss.size(); ++s)
        if (b->atoms[s] > 0 && ss[s].steps_left <= 0) {
            if (done && k < cap) done[k] = s;
            ++k;
        }
    if (n_done) *n_done = k;
    return PIS_OK;
}

pis_status pis_batch_result(pis_batch* b, int32_t slot, double* pos, double* vel, double* force, double* pe,
                            double* ke, int64_t* steps_done) {
    if (!b || slot < 0 || slot >= (int)b->atoms.size() || b->atoms[slot] == 0)
        return bfail(b, PIS_ERR_INVALID_ARGUMENT, "no such slot");
    std::string err;
    pis_status st = b->eng.reduce_state_slot(false, slot, err);
    if (st) return bfail(b, st, err);
    pis::SysState ss;
    st = b->eng.read_state(slot, ss, err);
    if (st) return bfail(b, st, err);
    if (pos || vel || force) {
        st = b->eng.download(slot, pos, vel, force, err);
        if (st) return bfail(b, st, err);
    }
    if (pe) *pe = ss.pe;
    if (ke) *ke = ss.ke;
    if (steps_done) *steps_done = ss.steps_done;
    if (ss.flags & pis::FLAG_NAN) return bfail(b, PIS_ERR_NAN_DETECTED, "NaN detected in this slot");
    if (ss.flags & pis::FLAG_LIST_OVERFLOW) return bfail(b, PIS_ERR_LIST_OVERFLOW, "neighbour list overflow");
    if (ss.flags & pis::FLAG_TIMEOUT) return bfail(b, PIS_ERR_TIMEOUT, "a device-side wait expired in this slot");
    return PIS_OK;
}

pis_status pis_batch_pe_history(pis_batch* b, int32_t slot, int64_t n, double* pe) {
    if (!b || slot < 0 || slot >= (int)b->atoms.size() || b->atoms[slot] == 0 || !pe)
        return bfail(b, PIS_ERR_INVALID_ARGUMENT, "no such slot");
    std::string err;
    pis_status st = b->eng.read_pe_history(slot, n, pe, err);
    return st ? bfail(b, st, err) : PIS_OK;
}

pis_status pis_batch_release(pis_batch* b, int32_t slot) {
    if (!b || slot < 0 || slot >= (int)b->atoms.size() || b->atoms[slot] == 0)
        return bfail(b, PIS_ERR_INVALID_ARGUMENT, "no such slot");
    b->eng.remove_slot(slot);
    b->atoms[slot] = 0;
    return PIS_OK;
}

pis_status pis_serve_last_stats(const pis_batch* b, pis_serve_stats* out) {
    if (!b || !out) return PIS_ERR_INVALID_ARGUMENT;
    *out = b->serve;
    return PIS_OK;
}

int64_t pis_batch_atoms(const pis_batch* b) {
    if (!b) return 0;
    int64_t t = 0;
    for (int64_t a : b->atoms) t += a;
    return t;
}

const char* pis_batch_last_error(const pis_batch* b) { return b ? b->err.c_str() : "null batch"; }

void pis_batch_destroy(pis_batch* b) { delete b; }

pis_status pis_serve_run(pis_batch* b, const pis_request* reqs, int32_t n, int64_t graph_steps,
                         pis_request_result* out, double* wall_s) {
    if (!b || (n > 0 && (!reqs || !out))) return PIS_ERR_INVALID_ARGUMENT;
    if (graph_steps < 1) graph_steps = 50;
    std::vector<int32_t> order(n);
    for (int32_t q = 0; q < n; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return reqs[x].arrival_s < reqs[y].arrival_s; });
    for (int32_t q = 0; q < n; ++q) {
        std::memset(&out[q], 0, sizeof(out[q]));
        out[q].status = -1;
    }
    std::vector<int32_t> slot_req(b->opt.max_slots, -1);
    std::deque<int32_t> queue;
    size_t next = 0;
    int32_t finished = 0;
    int active = 0;
    const auto t0 = std::chrono::steady_clock::now();
    std::string err;
    // Initial states of queued jobs, generated on the host while the GPU runs the previous graph
    // (the generation is deterministic per job, so results do not depend on when it happens).
    struct Prepared {
        std::vector<double> pos, vel;
        double L = 0;
    };
    std::unordered_map<int32_t, Prepared> ready;
    auto prepare = [&](int32_t q) {
        if (ready.count(q)) return;
        Prepared p;
        make_lj_state(reqs[q].job, p.pos, p.vel, p.L);
        ready.emplace(q, std::move(p));
    };
    auto admit_ready = [&](int32_t q, int32_t* slot) {
        prepare(q);
        Prepared& p = ready[q];
        const pis_lj_job& job = reqs[q].job;
        if (job.k < 1 || !(job.rho > 0) || !(job.t_star >= 0) || !(job.rcut > 0))
            return bfail(b, PIS_ERR_INVALID_ARGUMENT, "bad LJ job parameters");
        pis::SlotDesc d = lj_desc(job, p.L);
        std::vector<int32_t> types((size_t)d.n, 1);
        // placed now, evaluated with the other jobs admitted before the next graph
        pis_status st = place_desc(b, d, types.data(), p.pos.data(), p.vel.data(), job.steps, false, slot);
        ready.erase(q);
        return st;
    };
    auto arrivals = [&]() {
        const double now = seconds_since(t0);
        while (next < order.size() && reqs[order[next]].arrival_s <= now) queue.push_back(order[next++]);
    };
    // Pipelined cycle: graph k+1 is queued before the state snapshot taken after graph k is read,
    // so releases, admissions (host-side state generation, uploads, the map rebuild) and the
    // evaluation of admitted jobs are prepared on the host while graph k+1 runs, and the work they
    // queue follows it on the stream. A job is seen finished in the snapshot of the graph it
    // finished in; slots placed after a graph was queued are not read from its snapshot.
    const int S = b->opt.max_slots;
    // snapshot buffers alternate between the graph in flight and the one being read; the events
    // that close each graph form a ring of 4 (a graph's interval starts at its predecessor's)
    constexpr int RING = 4;
    pis::SysState* snap[2] = {nullptr, nullptr};
    cudaEvent_t ev[RING] = {nullptr, nullptr, nullptr, nullptr};
    struct Cleanup {
        pis::SysState** snap;
        cudaEvent_t* ev;
        ~Cleanup() {
            for (int k = 0; k < 2; ++k)
                if (snap[k]) cudaFreeHost(snap[k]);
            for (int k = 0; k < RING; ++k)
                if (ev[k]) cudaEventDestroy(ev[k]);
        }
    } cleanup{snap, ev};
    for (int k = 0; k < 2; ++k)
        if (cudaMallocHost((void**)&snap[k], sizeof(pis::SysState) * S) != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, PIS_ERR_NO_MEMORY, "pinned state snapshot");
        }
    for (int k = 0; k < RING; ++k)
        if (cudaEventCreate(&ev[k]) != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, PIS_ERR_CUDA, "event");
        }
    // graph g (from 1) ends at ev[g % RING]; ev[0] is recorded now as the start of graph 1
    if (cudaEventRecord(ev[0], b->eng.stream()) != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, PIS_ERR_CUDA, "event");
    }
    std::vector<int64_t> placed_at(S, 0);  // first graph that steps each slot's current job
    std::vector<int64_t> seen_steps(S, 0);  // steps_done of each slot's job at the last snapshot read
    std::vector<char> saturated(1, 0);      // per graph: queued while a request waited for space
    pis_serve_stats stats{};
    int64_t graphs = 0;                    // graphs queued so far
    int inflight = -1;                     // snapshot buffer of the last graph queued and not read
    uint64_t mark[2] = {0, 0};
    int64_t snap_graph[2] = {0, 0};
    auto read_snapshot = [&](int k) -> pis_status {
        const int64_t g = snap_graph[k];
        pis_status rs = b->eng.wait_event(ev[g % RING], err);
        if (rs) return rs;
        b->eng.retire_staging(mark[k]);
        const double t_done = seconds_since(t0);
        const pis::SysState* ss = snap[k];
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev[(g - 1) % RING], ev[g % RING]) != cudaSuccess) {
            cudaGetLastError();
            ms = 0.f;
        }
        double done = 0.0;  // atom-steps of graph g
        for (int s = 0; s < S; ++s) {
            if (slot_req[s] < 0 || placed_at[s] > g) continue;
            done += (double)b->atoms[s] * (double)(ss[s].steps_done - seen_steps[s]);
            seen_steps[s] = ss[s].steps_done;
        }
        stats.atom_steps += done;
        stats.device_s += 1e-3 * ms;
        if (saturated[g]) {
            stats.saturated_graphs += 1;
            stats.saturated_atom_steps += done;
            stats.saturated_device_s += 1e-3 * ms;
        }
        // finished jobs: energies and counters as their last step left them (the step end writes
        // PE and KE every step); released with the chunk map rebuilt once, before the next graph
        for (int s = 0; s < S; ++s) {
            const int32_t q = slot_req[s];
            if (q < 0 || placed_at[s] > g || ss[s].steps_left > 0) continue;
            out[q].finished_s = t_done;
            out[q].pe = ss[s].pe;
            out[q].ke = ss[s].ke;
            out[q].steps = ss[s].steps_done;
            out[q].status = (ss[s].flags & pis::FLAG_NAN)             ? PIS_ERR_NAN_DETECTED
                            : (ss[s].flags & pis::FLAG_LIST_OVERFLOW) ? PIS_ERR_LIST_OVERFLOW
                            : (ss[s].flags & pis::FLAG_TIMEOUT)       ? PIS_ERR_TIMEOUT
                                                                      : PIS_OK;
            b->eng.remove_slot(s, true);
            b->atoms[s] = 0;
            slot_req[s] = -1;
            --active;
            ++finished;
        }
        return PIS_OK;
    };
    while (finished < n) {
        arrivals();
        // admit in arrival order while the head of the queue fits
        std::vector<int> fresh;
        while (!queue.empty()) {
            const int32_t q = queue.front();
            if (!pis_batch_fits_lj(b, &reqs[q].job)) {
                if (active > 0) break;  // wait for a release
                out[q].status = PIS_ERR_NO_MEMORY;  // never fits, even in an empty pool
                queue.pop_front();
                ++finished;
                continue;
            }
            int32_t slot = -1;
            pis_status st = admit_ready(q, &slot);
            queue.pop_front();
            out[q].admitted_s = seconds_since(t0);
            out[q].atoms = 4ll * reqs[q].job.k * reqs[q].job.k * reqs[q].job.k;
            if (st) {
                out[q].status = st;
                out[q].finished_s = out[q].admitted_s;
                ++finished;
                continue;
            }
            slot_req[slot] = q;
            placed_at[slot] = graphs + 1;
            seen_steps[slot] = 0;
            fresh.push_back(slot);
            ++active;
        }
        const bool waiting = !queue.empty();  // the head did not fit: the pool is the limit
        if (!fresh.empty()) {
            // no synchronisation: the graph follows on the same stream
            pis_status st = b->eng.compute_potential_slots(fresh, err, false);
            if (st) return bfail(b, st, err);
        }
        int queued = -1;
        if (active > 0) {
            pis_status st = b->eng.run(graph_steps, err);
            if (st) return bfail(b, st, err);
            queued = inflight == 0 ? 1 : 0;
            ++graphs;
            saturated.push_back(waiting ? 1 : 0);
            snap_graph[queued] = graphs;
            mark[queued] = b->eng.staging_mark();
            st = b->eng.snapshot_states(snap[queued], ev[graphs % RING], err);
            if (st) return bfail(b, st, err);
        }
        if (inflight >= 0) {
            pis_status st = read_snapshot(inflight);
            if (st) return bfail(b, st, err);
            inflight = -1;
        }
        if (queued >= 0) {
            inflight = queued;
            // while the graph runs: the initial states of the next queued jobs
            arrivals();
            int k = 0;
            for (int32_t q : queue) {
                if (k++ >= 8) break;
                prepare(q);
            }
            continue;
        }
        // nothing running and nothing admitted: wait for the next arrival
        if (next < order.size()) {
            const double wait = reqs[order[next]].arrival_s - seconds_since(t0);
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
        }
    }
    if (inflight >= 0) {  // a last graph queued after every job had finished (it steps nothing)
        pis_status st = read_snapshot(inflight);
        if (st) return bfail(b, st, err);
    }
    std::string serr;
    pis_status st = b->eng.sync(serr);
    if (st) return bfail(b, st, serr);
    stats.graphs = graphs;
    b->serve = stats;
    if (wall_s) *wall_s = seconds_since(t0);
    return PIS_OK;
}

}  // extern "C"
