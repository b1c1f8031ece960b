// engine.h - host interface of the packed multi-system MD engine (GB300, sm_103a).
//
// One Engine owns a pool of device memory that holds any number of independent periodic
// Lennard-Jones systems ("slots") packed back to back: atoms of slot s occupy a contiguous
// atom range, its cells a contiguous cell range. Every kernel runs over the whole pool in one
// launch; blocks map to (slot, chunk of atoms) through a device-side table, so the same
// captured CUDA graph serves one 2M-atom system, 512 replicas, or a changing set of served
// jobs. Per-slot device state (rebuild flag, steps left, energies) lives in device memory so a
// multi-step graph needs no host round trip.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include <map>
#include <deque>

#include "pis_gpu.h"

namespace pis {

// One entry of a dense per-slot type-pair table (both (ti,tj) and (tj,ti) filled).
struct LJHost {
    double epsilon = 0, sigma = 0, rcut = 0;
    int present = 0;
    int shift = 1;
};

struct SlotDesc {
    int64_t n = 0;
    int n_types = 1;
    std::vector<LJHost> table;      // n_types * n_types
    std::vector<double> masses;     // per type
    double h[9] = {0};              // row-major box matrix (diagonal, or general on the FP64 path)
    int pbc[3] = {1, 1, 1};
    double skin = 0.3;
    double dt = 0.005;
    int64_t steps = 0;              // steps the slot takes in the following runs
};

// Device-side per-slot parameters (read-only inside kernels).
struct SysParams {
    int64_t a0;        // first atom of the slot
    int64_t c0;        // first entry of the slot's cell arrays (ncells + 1 entries)
    int32_t n;         // atoms
    int32_t active;
    int32_t nt;        // types
    int32_t tab0;      // first entry in the global pair table
    int32_t nc[3];     // cells per axis
    int32_t pbc[3];
    int32_t ch0, nch;  // chunk range of the slot
    int32_t cl0, clcap;  // cluster-list path: first cluster entry of the slot and its capacity
    int32_t cch0, ncch;  // cluster-list path: chunk range of the slot's cluster kernels
    double h[3];       // diagonal of h
    double hinv[3];    // diagonal of h^-1 (adjugate / determinant, as the reference)
    double cs[3];      // cell edge
    double half_skin2; // (skin / 2)^2
    double dt, dt2;    // dt, dt*dt
    double hdt, hdt2;  // dt/2, dt*dt/2 (mixed-path integrators)
    // FP32 cell-relative coordinates (prel) are in units of sc, the x cell edge (1 for a triclinic
    // box: Cartesian), so in a box with cubic cells an image shift is exactly +-1; the FP32 pair
    // constants of the slot's table are scaled to match
    double sc, isc;    // the unit and its inverse
    float fisc_hi, fisc_lo;  // isc as the sum of two floats (FP32 scaling of small displacements)
    float fcs[3];      // cell edges in units of sc
    float frlist2;     // FP32 list radius squared in units of sc, padded so the FP32 test is a superset
    float fsub[3];     // 4 sc / cell edge: sub-cell index scale of the in-cell atom order
    int32_t walk27;    // the 27-cell walk of the thread-per-atom build is valid (see add_slot)
    int32_t rnc[3];    // the reference's own cell grid at the largest cutoff (reference-order forces)
    int32_t tric;      // the box has off-diagonal elements (FP64 path only): H / HI below are used
    double H[9];       // row-major box matrix (columns = box vectors) and its inverse (adjugate /
    double HI[9];      // determinant, as the reference's 3x3 inverse); diagonal boxes use h / hinv
    float fcv[9];      // triclinic cell edge vectors: column d of H / nc[d] in fcv[3d..3d+2]
};

// Device-side pair parameters: FP64 quantities computed exactly as the reference does per pair,
// plus FP32 copies for the mixed path.
struct LJDev {
    double eps4, eps24, sigma2, rcut, rc2_lo, rc2_hi, ucut;
    float feps4, feps24, fsigma2, frc2, fucut;
    int32_t present;
};

// Mutable per-slot device state.
struct SysState {
    int32_t cur;          // which of the two atom buffer sets is current
    int32_t rebuild;      // neighbour list must be rebuilt in this step
    int32_t flags;        // FLAG_* bits
    int32_t want_virial;  // compute sum_i r_i F_i^T in the next reductions
    int32_t eval;         // slot takes part in the next host-requested evaluation / reduction
    int32_t ncl;          // clusters of the current build (cluster-list path)
    int32_t need_nn;      // longest per-atom list a build asked for (more than the capacity on overflow)
    int32_t thermo;       // steps also record KE and the virial trace sum_i r_i . F_i in history rings
    int64_t steps_left;   // steps still to take; a slot at 0 is frozen during run()
    int64_t steps_done;
    int64_t rebuilds;
    double pe, ke;
    double virial[9];
    double ktensor[9];    // sum_i v_i v_i^T (Atoms::kinetic_tensor, no masses), on request
};

enum : int32_t { FLAG_NAN = 1, FLAG_LIST_OVERFLOW = 2, FLAG_CELL_OVERFLOW = 4, FLAG_TIMEOUT = 8 };

struct PoolOptions {
    int precision = PIS_PRECISION_FP64;
    int list_kind = PIS_LIST_DEFAULT;
    int blk = 256;             // atoms per chunk = threads per block of every atom kernel
    int list_cap = 0;          // per-atom neighbour capacity (0 = from density)
    int64_t max_atoms = 0;
    int max_slots = 1;
    int64_t max_cells = 0;     // total cell entries (including one sentinel per slot)
    int max_types_total = 64;  // pair-table entries
    int hist = 1024;           // per-slot energy history ring
    bool fp64_fast = false;    // FP64 force kernel with FMAs and Newton reciprocal (variant)
    bool mixed_kahan = false;  // mixed force kernel with compensated FP32 sums (variant)
    int lpa = 1;               // lanes per atom in the list build and force kernels (1,4,8,16,32)
    int mix_batch = 4;         // list entries per gather batch in the mixed force kernel (4, 8, 16)
    bool list_tma = false;     // mixed, thread per atom: list rows streamed to shared memory by bulk copies
    bool cell_tiles = false;   // mixed, thread per atom: neighbour-cell tiles staged in shared memory
    bool plain_graphs = false; // step graphs without the conditional rebuild node (profilers cannot
                               // look inside graphs holding conditional nodes)
    int cluster = 0;           // mixed: atoms per cluster of the cluster-list kernels (2 or 4); 0 = per-atom list
    int build_cluster = 0;     // per-atom list, thread per atom: build scans candidates per cluster of this
                               // many atoms (2 or 4; 0 or 1 = per atom)
    bool unfused = false;      // mixed, default kernel shape: separate force, kick and drift kernels
                               // (otherwise one fused step kernel does all three)
    bool ref_order = false;    // FP64, full list: forces summed in the reference's own order
    int64_t wait_limit = -1;   // polls of a bulk-copy pipeline wait (< 0: the default, 2^22)
};

class Engine {
  public:
    Engine();
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    pis_status init(const PoolOptions& opt, std::string& err);
    // Place a system in the pool. Returns the slot id (>= 0) or a negative pis_status.
    // defer_map: leave the chunk map and the stream unsynchronised (the next evaluation or run
    // rebuilds the map once for every slot placed or removed since), so a host loop can place and
    // remove many slots between two graphs with one synchronisation.
    int add_slot(const SlotDesc& d, const int32_t* type_ids, const double* pos, const double* vel,
                 const double* force, std::string& err, bool defer_map = false);
    void remove_slot(int slot, bool defer_map = false);
    // Ask whether a system of this shape fits in the free space right now.
    bool fits(const SlotDesc& d) const;
    // Cells of a system's list grid (at rcut + skin across each pair of box faces).
    static int64_t cells_for(const SlotDesc& d);
    int64_t list_cap() const { return opt_.cluster ? ccap_ : cap_; }
    int cluster_size() const { return opt_.cluster; }
    int precision() const { return opt_.precision; }
    bool half_list() const { return half_; }

    pis_status set_dt(int slot, double dt, std::string& err);
    pis_status set_steps(int slot, int64_t steps, std::string& err);
    // Zero forces, rebuild lists, evaluate forces + PE (+ KE and virial) for every active slot.
    pis_status compute_potential(std::string& err);
    // The same for one slot only (the others keep their state untouched).
    pis_status compute_potential_slot(int slot, std::string& err);
    // The same for several slots at once (one kernel sequence; each slot's results as alone).
    // wait = false leaves the stream running (the caller's next launch or synchronisation follows)
    // every slot's SysState copied to `host` (pinned, max_slots entries) after the work queued so
    // far, then `done` recorded; nothing waits
    pis_status snapshot_states(SysState* host, cudaEvent_t done, std::string& err);
    // Host sources of uploads that no synchronisation follows (the map rebuild, deferred slot
    // placement and removal) are copied here and kept until the stream has passed them: until the
    // next sync(), or retire_staging(mark) once an event recorded after staging_mark() returned
    // `mark` has completed.
    uint64_t staging_mark() { return ++held_seq_; }
    pis_status wait_event(cudaEvent_t e, std::string& err);
    void retire_staging(uint64_t mark);
    pis_status compute_potential_slots(const std::vector<int>& slots, std::string& err, bool wait = true);
    // Run k velocity-Verlet steps on every active slot with steps_left > 0 (graph chunks).
    pis_status run(int64_t k, std::string& err);
    // KE and virial of every active slot at the current state.
    pis_status reduce_state(bool virial, std::string& err);
    pis_status reduce_state_slot(bool virial, int slot, std::string& err, bool ktensor = false);
    pis_status sync(std::string& err);

    pis_status download(int slot, double* pos, double* vel, double* force, std::string& err);
    pis_status read_state(int slot, SysState& st, std::string& err);
    pis_status read_states(std::vector<SysState>& st, std::string& err);
    // Last n energies of the slot's history ring (oldest first).
    pis_status read_pe_history(int slot, int64_t n, double* out, std::string& err);
    // Last n steps' potential energy, kinetic energy and virial trace (the latter two recorded while
    // the slot's thermo flag is set); any output may be null.
    pis_status read_history(int slot, int64_t n, double* pe, double* ke, double* trace, std::string& err);
    pis_status set_thermo(int slot, bool on, std::string& err);
    pis_status neighbour_sets(int slot, std::vector<int64_t>& offsets, std::vector<int32_t>& idx,
                              std::string& err);
    pis_status list_entries(int slot, int64_t& total, std::string& err);
    // List-overflow recovery: keep a device copy of one slot's state, put it back (the list is
    // rebuilt at the next step), and enlarge the per-atom list capacity (the list layout does not
    // depend on the capacity, so only its allocation grows; captured graphs are dropped).
    pis_status save_state(int slot, std::string& err);
    pis_status restore_state(int slot, std::string& err);
    pis_status grow_list(int64_t new_cap, std::string& err);
    bool per_atom_list() const { return !opt_.cluster; }
    // General (triclinic) boxes are supported by the FP64 path with exact arithmetic, one thread
    // per atom and per-atom lists.
    bool triclinic_capable() const {
        return opt_.precision == PIS_PRECISION_FP64 && !opt_.fp64_fast && opt_.lpa == 1 && !opt_.cluster && !clm_;
    }
    pis_status scale_velocities(int slot, const double* m, std::string& err);
    pis_status scale_box(int slot, const double* m, std::string& err);
    const SysParams& params(int slot) const { return hp_[slot]; }
    int n_active() const;
    cudaStream_t stream() const { return stream_; }
    // Kernel launches issued (graph launches count every captured kernel).
    static int64_t launches();
    // Kernels launched per captured step (for launch accounting).
    int64_t graph_kernels_per_step() const { return kernels_per_step_; }
    bool fused_step() const { return fused_; }
    // Stage timing with CUDA events captured into the step graphs (integrate1, list rebuild,
    // force, integrate2, reductions); costs one host sync per graph launch while enabled.
    void set_instrument(bool on) { instrument_ = on; }
    void reset_stage_times();
    const double* stage_ms() const { return stage_ms_; }
    int64_t stage_steps() const { return stage_steps_; }
    void set_graph_steps(int64_t g) { graph_steps_ = g > 0 ? g : 1; }

    struct DevPtrs;  // device pointer bundle passed by value to every kernel

  private:
    pis_status rebuild_block_map(std::string& err);
    // Step q of a g-step graph.
    void enqueue_step(bool respect_steps, cudaEvent_t* ev, int64_t q, int64_t g);
    void enqueue_rebuild(bool respect_steps, int q = 0);
    // The rebuild kernels of a captured step inside a conditional graph node that runs only when
    // some slot rebuilds in that step (the condition is set on the device).
    pis_status enqueue_rebuild_conditional(bool respect_steps, int q = 0);
    // Conditional rebuild bodies executed since the last call, counted on the device.
    void account_body_launches();
    void enqueue_potential(int only);
    void launch_force_fp64(int respect_steps);
    void launch_force_mixed(int respect_steps);
    void launch_step_mixed(bool drift, int q);
    void launch_step_end(int mode);
    void launch_build(int respect_steps);
    void launch_force_cluster(int respect_steps);
    pis_status check(cudaError_t e, const char* what, std::string& err);
    pis_status neighbour_sets_cluster(int slot, const SysState& ss, std::vector<int64_t>& offsets,
                                      std::vector<int32_t>& idx, std::string& err);

    PoolOptions opt_;
    bool half_ = true;
    int64_t cap_ = 0;
    int64_t npad_ = 0;
    int64_t max_chunks_ = 0;
    int64_t max_clusters_ = 0, clpad_ = 0, ccap_ = 0, max_cchunks_ = 0;
    int clm_ = 0;  // atoms per cluster of the cluster table (0: no table)
    cudaStream_t ls_ = nullptr;    // stream the rebuild kernels are launched on (stream_, or side_ while a
                                   // conditional body is captured)
    cudaStream_t side_ = nullptr;  // capture stream of conditional bodies
    bool cond_rebuild_ = true;     // step graphs skip the rebuild kernels through a conditional node
    bool body_counting_ = false;   // conditional rebuild bodies count their kernels on the device
    uint64_t body_seen_ = 0;       // body kernels already counted into the launch counter
    bool cond_step_ = false;       // a capture with conditional rebuild nodes is in progress
    pis_status cond_error_ = PIS_OK;
    cudaStream_t stream_ = nullptr;
    std::vector<SysParams> hp_;
    std::vector<int> slot_tab_size_;
    std::vector<double> slot_rlist_;
    std::vector<double> slot_rcmax_;  // largest cutoff of each slot's pair table
    std::vector<std::vector<LJDev>> slot_tab_host_;  // each slot's pair table as uploaded
    // free-space bookkeeping (first fit over atom and cell index ranges)
    std::map<int64_t, int64_t> free_atoms_, free_cells_, free_clusters_;
    std::vector<int> free_tab_;
    // device allocations
    void* mem_ = nullptr;
    size_t mem_bytes_ = 0;
    DevPtrs* d_ = nullptr;
    struct GraphRec {
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaEvent_t> ev;  // 6 per step when instrumented
        int64_t kernels = 0;          // kernels launched by one replay (conditional bodies aside)
    };
    std::map<int64_t, GraphRec> graphs_;
    bool instrument_ = false;
    int64_t graph_steps_ = 50;
    double stage_ms_[5] = {0, 0, 0, 0, 0};
    int64_t stage_steps_ = 0;
    int64_t kernels_per_step_ = 0;
    bool dirty_map_ = true;
    struct Held {
        uint64_t seq;
        std::vector<unsigned char> buf;
    };
    std::deque<Held> held_;  // upload sources kept until the stream has passed them
    uint64_t held_seq_ = 0;
    const void* hold(const void* src, size_t bytes);
    bool single_type_ = true;  // every active slot has one atom type (selects the force kernel)
    bool any_tric_ = false;    // some active slot has a triclinic box (selects the rebuild kernels)
    int scan_segs_ = 1;        // cell-scan segments of the largest slot (1: one scan block per slot)
    bool any_generic_ = false; // some active slot needs the generic list walk (not the 27-cell walk)
    // replica pools with the thread-per-atom list: the rebuild kernels run a grid of listed_grid_
    // blocks over a list of the rebuilding slots' chunks and cells
    bool listed_ = false;
    int listed_grid_ = 0;
    bool fused_ = false;       // mixed steps run the fused force + kick + drift kernel
    bool list_groups_ = false; // the per-atom list is stored in groups of consecutive entries
    void* prel_buf_[2] = {nullptr, nullptr};  // the two cell-relative coordinate buffers (fused steps)
    int thermo_slots_ = 0;             // slots whose steps record thermo (selects the fused kernel)
    std::vector<int> slot_thermo_;
    void* nbr_own_ = nullptr;   // a grown neighbour list (allocated apart from the pool)
    void* save_ = nullptr;      // checkpoint of one slot's per-atom arrays (allocated on first use)
    int save_slot_ = -1;
    SysState save_state_{};
};

}  // namespace pis
