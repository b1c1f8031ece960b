/*
 * pis_gpu.h - C ABI of the GB300 (sm_103a) Lennard-Jones MD-step library.
 *
 * This is the drop-in boundary for the MD hot path of PIS (vivekadishankara/pis): the
 * Lennard-Jones pair force / energy / virial evaluation over a Verlet neighbour list, the
 * cell-binned list build with its skin-displacement rebuild check, and velocity-Verlet NVE
 * integration with periodic wrapping. Each entry point names the reference interface it
 * replaces (file:line in the reference crate).
 *
 * Conventions (chosen so a Rust caller can pass nalgebra storage unchanged):
 *   - positions / velocities / forces are 3 x N column-major (x,y,z per atom), the
 *     Matrix3xX<f64> layout of src/atoms/new.rs:9-17 (`positions.as_slice()`);
 *   - the box matrix h is 3x3 column-major (Matrix3<f64> storage, src/simulation_box.rs:5-9);
 *   - type ids are 1-based (src/atoms/properties.rs:9-13), masses are per type;
 *   - every call returns a pis_status; on failure pis_gpu_last_error() holds the message.
 * One context owns one CUDA stream and its device state; a context is not thread-safe, but
 * separate contexts are independent. Nothing here falls back to the CPU: a call that needs
 * the GPU and cannot get one fails with PIS_ERR_CUDA.
 */
#ifndef PIS_GPU_H
#define PIS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The first block mirrors PisError (src/errors.rs:5-98); the second block is
 * GPU-specific. */
typedef enum {
    PIS_OK = 0,
    PIS_ERR_INVALID_ARGUMENT = 1,  /* PisError::InvalidArgument / MissingArgument / NegativeValue */
    PIS_ERR_NO_ATOMS = 2,          /* PisError::NoAtomsDefined */
    PIS_ERR_INVALID_ATOM_TYPE = 3, /* PisError::InvalidAtomType */
    PIS_ERR_MISSING_POTENTIAL = 4, /* PisError::PotentialNotInitialized / MissingPotential */
    PIS_ERR_IO = 5,                /* PisError::InputFileError / DataFileError / Dump*Error */
    PIS_ERR_PARSE = 6,             /* PisError::FloatParseError / IntParseError / UnknownCommand */
    PIS_ERR_ATOM_COUNT = 7,        /* PisError::AtomCountMismatch */
    PIS_ERR_UNKNOWN_PAIR_STYLE = 8,/* PisError::UnknownPairStyle */
    PIS_ERR_NAN_DETECTED = 20,     /* PisError::NaNEnergy (never raised by the reference) */
    PIS_ERR_BOX_TOO_SMALL = 21,    /* box shorter than 2 (rcut + skin) along an axis */
    PIS_ERR_NO_MEMORY = 22,        /* device allocation failed / job does not fit */
    PIS_ERR_LIST_OVERFLOW = 23,    /* a neighbour or cell list outgrew its capacity */
    PIS_ERR_CUDA = 24,             /* any CUDA runtime error */
    PIS_ERR_STATE = 25,            /* call out of order (e.g. no atoms uploaded yet) */
    PIS_ERR_UNSUPPORTED = 26,      /* e.g. a triclinic box in mixed precision */
    PIS_ERR_TIMEOUT = 27           /* a bounded device-side wait expired (the kernel stopped early) */
} pis_status;

/* One pair_coeff / PairCoeffs row: LennardJones::new(epsilon, sigma, rcut, shift)
 * (src/potentials/lennard_jones.rs:14-31), keyed (ti, tj) like the Table of
 * src/potentials/potential.rs:143-144 (order-insensitive lookup, :181-192). */
typedef struct {
    int32_t ti, tj;
    double epsilon, sigma, rcut;
    int32_t shift;
} pis_lj_pair;

typedef enum {
    PIS_PRECISION_FP64 = 0,  /* reference arithmetic in FP64, operation for operation */
    PIS_PRECISION_MIXED = 1  /* FP32 pair math on cell-relative coordinates, FP64 elsewhere */
} pis_precision;

typedef enum {
    PIS_LIST_DEFAULT = 0,    /* half list for FP64, full list for MIXED */
    PIS_LIST_HALF = 1,       /* Newton-3 half list, forces on j scattered with FP64 atomics (MIXED: thread
                              * per atom, separate force and integration kernels; a measured variant) */
    PIS_LIST_FULL = 2        /* full list, each pair evaluated from both ends, no atomics */
} pis_list_kind;

typedef struct pis_gpu_ctx pis_gpu_ctx;

/* Counters and the last reductions of a context. */
typedef struct {
    int64_t n_atoms;
    int64_t steps;            /* velocity-Verlet steps taken since set_state */
    int64_t rebuilds;         /* neighbour-list builds since set_state */
    int64_t list_entries;     /* entries in the current neighbour list */
    int32_t list_capacity;    /* per-atom capacity of the list */
    int32_t cells[3];         /* cell grid used by the list build */
    double pe, ke;            /* energies after the last force evaluation / step */
    double virial[9];         /* sum_i r_i F_i^T (row-major), as src/atoms/properties.rs:49-51 */
    int32_t fused_step;       /* 1 when steps run the fused force + kick + drift kernel */
    int32_t reserved_;
} pis_gpu_stats;

/* Create a context for a pair table (the PotentialManager built in System::contextualize,
 * src/system.rs:130-165, or run_read_data, src/readers/input_file/commands.rs:171,367-369).
 * skin is the Verlet skin added to the largest cutoff; precision is a pis_precision. */
pis_status pis_gpu_create(const pis_lj_pair* table, int32_t n_pairs, int32_t n_types, double skin,
                          int32_t precision, pis_gpu_ctx** out);

/* Variant flags for pis_gpu_set_options. */
#define PIS_OPT_FP64_FAST 1  /* FP64 forces with fused multiply-adds and a Newton reciprocal; the
                              * cutoff is still decided with the reference's exact arithmetic */
#define PIS_OPT_MIXED_KAHAN 2 /* mixed path: compensated FP32 sums instead of FP64 batch sums */
#define PIS_OPT_LANES(n) ((n) << 8) /* lanes per atom in the list build and force kernels:
                                     * 1 (thread per atom, default), 4, 8, 16 or 32 (warp per atom);
                                     * with PIS_OPT_CLUSTER(m), 1 = a thread per cluster and m = a
                                     * lane per cluster member */
#define PIS_OPT_BATCH(n) ((n) << 16) /* mixed path, thread per atom: list entries loaded per gather
                                      * batch, 4 (default), 8 or 16 */
#define PIS_OPT_LIST_TMA 4 /* mixed path, thread per atom: the neighbour list is streamed into shared
                            * memory by bulk (TMA) copies several batches ahead of the pair loop;
                            * PIS_OPT_BATCH(8 or 16) sets the rows per copy stage (4 counts as 8) */
#define PIS_OPT_TILE 8 /* mixed path, thread per atom: the neighbour cells of each 256-atom chunk are
                        * staged in shared memory by bulk (TMA) copies and the pair loop gathers
                        * neighbour positions from there */
#define PIS_OPT_PLAIN_GRAPHS 16 /* step graphs launch the list-rebuild kernels on every step (they exit at
                                 * once when nothing rebuilds) instead of behind a conditional graph node:
                                 * for profilers that cannot look inside graphs holding conditional nodes;
                                 * PIS_GPU_PLAIN_GRAPHS=1 in the environment does the same for every
                                 * context and batch of the process */
#define PIS_OPT_UNFUSED 32 /* mixed precision, default kernel shape: separate force, kick and drift kernels
                            * in each step instead of the fused step kernel (same results bit for bit) */
#define PIS_OPT_REF_ORDER 64 /* FP64 precision, full list: every atom's force terms are summed in the order of the
                             * reference's cell walk (LJVOffsetManager::compute_potential,
                             * src/potentials/lennard_jones.rs:186-244, cells at the largest cutoff,
                             * src/atoms/neighbour_list.rs:9-165), so forces and trajectories equal the
                             * reference's bit for bit; needs at least 3 cells of the largest cutoff per axis */
#define PIS_OPT_CLUSTER(m) ((m) << 24) /* mixed path, neighbour-list shape: 1 = one list per atom,
                                        * 2 or 4 = one list per cluster of m spatially adjacent atoms
                                        * of a cell (each neighbour read serves m pairs);
                                        * PIS_OPT_BATCH(4 or 8) sets the entries per gather batch */
#define PIS_OPT_SCAN(m) ((m) << 28) /* per-atom lists, one thread per atom: the list build scans the
                                     * candidates of m spatially adjacent atoms of a cell per thread
                                     * (2 or 4) or of one atom (1); the lists are the same either way */

/* Select a measured variant: list kind (pis_list_kind) and PIS_OPT_* flags. Takes effect at the
 * next set_state. */
pis_status pis_gpu_set_options(pis_gpu_ctx* ctx, int32_t list_kind, int32_t flags);

/* Neighbour-list capacity (no counterpart in the reference, which rebuilds its cells at every
 * evaluation and keeps no list): per_atom entries per atom (0, the default, sizes it from the mean
 * density: 1.6 x the expected count + 32). With auto_grow = 1 (the default) an evaluation or a run
 * of steps whose list outgrows the capacity is repeated from its own start with a larger list (the
 * state before it is kept on the device), so the results are those of a run that never overflowed;
 * with auto_grow = 0 it returns PIS_ERR_LIST_OVERFLOW and its results are invalid. per_atom takes
 * effect at the next set_state, auto_grow at once. */
pis_status pis_gpu_set_list_capacity(pis_gpu_ctx* ctx, int32_t per_atom, int32_t auto_grow);

/* Poll budget of the bounded waits in the bulk-copy (TMA) force variants (PIS_OPT_LIST_TMA,
 * PIS_OPT_TILE; no counterpart in the reference): polls < 0 restores the default (2^22 polls).
 * A wait that runs out stops the block's pipeline, waits (with the full budget) for the block's own
 * copies in flight and returns PIS_ERR_TIMEOUT from the call; a budget of 0 makes every such wait
 * run out at once, so tests can exercise that path on a correct kernel. Takes effect at the next
 * set_state. */
pis_status pis_gpu_set_wait_limit(pis_gpu_ctx* ctx, int64_t polls);

/* Upload the Atoms state (src/atoms/new.rs:9-17). force may be NULL (zero forces, as the
 * data-file reader leaves them, src/readers/input_file/commands.rs:367). The only
 * AoS <-> device-layout transpose happens here and in pis_gpu_get_state. */
pis_status pis_gpu_set_state(pis_gpu_ctx* ctx, int64_t n, const int32_t* type_ids,
                             const double* masses_per_type, const double* pos, const double* vel,
                             const double* force, const double* h_colmajor, const uint8_t* pbc);

/* PotentialManager::compute_potential after zeroing the forces (src/potentials/potential.rs:13,24-26;
 * LJVOffsetManager, src/potentials/lennard_jones.rs:186-244). Writes the potential energy and,
 * if forces is non-NULL, the forces (3 x N). */
pis_status pis_gpu_compute_potential(pis_gpu_ctx* ctx, double* pe_out, double* forces);

/* n_steps calls of PotentialManager::verlet_step_nve (src/potentials/potential.rs:15-33).
 * pe_out, if non-NULL, receives the potential energy each step returns (n_steps values).
 * The state stays on the device; chunks of steps run as captured CUDA graphs. */
pis_status pis_gpu_verlet_step_nve(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* pe_out);

/* pis_gpu_verlet_step_nve with the thermo of every step kept on the device and read back once per
 * run (Simulation::output prints PE, KE, H, T and P after each step, src/simulation.rs:66-88):
 * ke_out receives Atoms::kinetic_energy (src/atoms/properties.rs:17-24) after each step and
 * virial_trace_out the trace of Atoms::virial_tensor (:49-51), sum_i r_i . F_i, which with KE gives
 * the pressure (:61-65). Any output may be NULL; the trace costs one more block sum per step and is
 * only formed when virial_trace_out is given. */
pis_status pis_gpu_verlet_step_nve_thermo(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* pe_out,
                                          double* ke_out, double* virial_trace_out);

/* Download positions / velocities / forces (3 x N each, any may be NULL). */
pis_status pis_gpu_get_state(pis_gpu_ctx* ctx, double* pos, double* vel, double* force);

/* Atoms::kinetic_energy and Atoms::virial_tensor (src/atoms/properties.rs:17-24, 49-51) of the
 * current device state; virial is row-major W[a][b] = sum_i r_i[a] F_i[b]. Either may be NULL.
 * In FP64 precision every energy and virial this library returns is an exact sum, independent of
 * summation order: each term t quantised to sign(t) floor(|t| 2^104), the integers added exactly,
 * the total rounded to the nearest double (NaN if a term is not finite or reaches 2^56). For terms
 * of magnitude 2^-52 or more this is the exactly rounded sum of the reference's own terms. */
pis_status pis_gpu_reductions(pis_gpu_ctx* ctx, double* ke, double* virial);

/* Per-atom neighbour sets within each pair's cutoff at the current positions, in original atom
 * indices, ascending per atom - the sets of LJVPBuildListManager::build_neighbour_list
 * (src/potentials/lennard_jones.rs:345-415). offsets has n+1 entries; idx receives up to cap
 * entries; total receives the full count. */
pis_status pis_gpu_neighbour_list(pis_gpu_ctx* ctx, int64_t* offsets, int32_t* idx, int64_t cap,
                                  int64_t* total);

/* Ensemble hooks (src/potentials/potential.rs:45-50, 119-134): v <- M v for every atom, and
 * Atoms::scale_box (src/atoms/transformations.rs:5-16): r <- (M h) h^-1 r with h <- M h. Both
 * take row-major 3x3 M. scale_box forces a neighbour-list rebuild at the next evaluation. A matrix
 * M with off-diagonal elements makes the box triclinic, which the FP64 path with exact arithmetic
 * and one thread per atom supports (the MTK barostat's box update, src/ensemble/npt.rs:49-56); the
 * cell grid keeps its counts, so the box may not shrink below one list radius per cell. */
pis_status pis_gpu_scale_velocities(pis_gpu_ctx* ctx, const double* m_rowmajor);
pis_status pis_gpu_scale_box(pis_gpu_ctx* ctx, const double* m_rowmajor);

/* Atoms::pressure_tensor (src/atoms/properties.rs:53-59): (sum_i v_i v_i^T + sum_i r_i F_i^T) /
 * volume, row-major, the kinetic tensor without masses as in the reference; and the current box
 * (3x3 column-major, nalgebra storage). */
pis_status pis_gpu_pressure_tensor(pis_gpu_ctx* ctx, double* p_rowmajor);
pis_status pis_gpu_get_box(pis_gpu_ctx* ctx, double* h_colmajor);

pis_status pis_gpu_get_stats(pis_gpu_ctx* ctx, pis_gpu_stats* out);
const char* pis_gpu_last_error(const pis_gpu_ctx* ctx);
void pis_gpu_destroy(pis_gpu_ctx* ctx);

/* Measurement hook (no counterpart in the reference): run n_steps NVE steps like
 * pis_gpu_verlet_step_nve, timing them with CUDA events on the context's stream; device_ms gets
 * the elapsed device time. If stage_ms is non-NULL, events captured into the step graphs also
 * time the five stages of a step (integrate-1, list rebuild, forces, integrate-2, reductions),
 * summed over the steps, at the cost of one host sync per 50-step graph. */
pis_status pis_gpu_run_timed(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* device_ms, double* stage_ms);

/* Measurement hook (no counterpart in the reference): the arithmetic peak of the current GPU's
 * FP32 and FP64 pipes in TFLOP/s (one fused multiply-add = 2 flops), measured with independent
 * multiply-add chains on every SM; the denominators of the force kernels' pipe fractions. */
pis_status pis_gpu_probe_peaks(double* fp32_tflops, double* fp64_tflops);

/* Force evaluation that allocates no device memory (no counterpart in the reference). For callers
 * that cannot allocate device memory while running - a host whose framework owns the whole device
 * memory pool, or a real-time loop where cudaMalloc's latency and implicit synchronisation are not
 * allowed. Same result as pis_gpu_compute_potential (FP64, reference arithmetic, the energy as the
 * same exact sum) on buffers the caller owns: d_type_ids (n, 1-based), d_pos (3 x n) are device
 * inputs; d_forces (3 x n) and d_pe (1 value) are device outputs; table and h_colmajor are host
 * arrays; stream is a cudaStream_t (NULL = default stream) and the call returns once the work is
 * enqueued on it. Type ids must lie in [1, n_types]: the device cannot report a bad one through the
 * return value, so an atom with an id outside that range gets zero force, its pairs are skipped and
 * *d_pe is NaN.
 * Limits of the fixed scratch: n <= 262144 atoms, at most 65536 cells at the largest cutoff, at
 * least 3 cells per axis, at most 4 atom types; larger inputs return PIS_ERR_INVALID_ARGUMENT
 * (PIS_ERR_BOX_TOO_SMALL below 3 cells). The scratch is one device array shared by every call on
 * a device: calls that overlap on the GPU race and must be serialised by the caller. The first
 * call on a device looks up the scratch address in the device's primary context and keeps it for
 * the life of that context (calls after cudaDeviceReset are not supported); make the first call
 * before any stream capture. A launch error already pending from the caller's earlier work is
 * neither reported nor cleared. */
pis_status pis_gpu_compute_potential_noalloc(const pis_lj_pair* table, int32_t n_pairs, int32_t n_types, int64_t n,
                                             const int32_t* d_type_ids, const double* d_pos,
                                             const double* h_colmajor, double* d_forces, double* d_pe,
                                             void* stream);

/* ---- Batched replicas and served jobs -------------------------------------------------------
 * A batch is one device pool holding many independent periodic systems ("slots"). Every step of
 * pis_batch_advance advances all slots that still have steps left, in one launch per kernel over
 * the whole pool, captured as CUDA graphs of up to 50 steps; a slot whose step count runs out
 * mid-graph stops exactly there. Slots are admitted and released between advances (continuous
 * batching). Each slot's arithmetic is independent of the others': a job gives the same result
 * alone and in any mix. No counterpart in the reference, which runs one system per process
 * (src/simulation.rs:8-39); each slot follows the same NVE step as pis_gpu_verlet_step_nve. */
typedef struct pis_batch pis_batch;

/* A job given by its state (the arrays of pis_gpu_set_state) and its run length. */
typedef struct {
    int64_t n;
    int32_t n_types;
    const int32_t* type_ids;
    const double* masses_per_type;
    const double* pos;
    const double* vel;         /* may be NULL */
    const double* h_colmajor;
    const pis_lj_pair* table;
    int32_t n_pairs;
    double skin;
    double dt;
    int64_t steps;
} pis_job;

/* A job given by the synthetic LJ-liquid recipe (reduced units, eps = sigma = mass = 1): 4 k^3
 * atoms on an FCC lattice at number density rho in the atom order of the reference's lattice
 * generator (src/bin/sapphire/main.rs:61-76), Maxwell-Boltzmann velocities at T* from `seed`
 * (drift removed and rescaled as src/atoms/velocities.rs:35-59), shifted LJ cut at rcut. */
typedef struct {
    int32_t k;
    double rho, t_star, rcut, skin, dt;
    int64_t steps;
    uint64_t seed;
} pis_lj_job;

pis_status pis_batch_create(int64_t max_atoms, int32_t max_slots, int64_t max_cells, int32_t precision,
                            int32_t flags, pis_batch** out);
/* Admit a job: place it in free pool space, evaluate its initial forces, set its step count.
 * PIS_ERR_NO_MEMORY when it does not fit right now (retry after a release). */
pis_status pis_batch_admit(pis_batch* b, const pis_job* job, int32_t* slot);
pis_status pis_batch_admit_lj(pis_batch* b, const pis_lj_job* job, int32_t* slot);
/* 1 if the job fits in the free pool space now, else 0 (admission by device-memory footprint). */
int32_t pis_batch_fits_lj(const pis_batch* b, const pis_lj_job* job);
/* Advance every slot with steps left by up to k steps. */
pis_status pis_batch_advance(pis_batch* b, int64_t k);
/* Same, timed with CUDA events on the batch's stream (device milliseconds). */
pis_status pis_batch_run_timed(pis_batch* b, int64_t k, double* device_ms);
/* Slots whose steps are done and not yet released (up to cap of them). */
pis_status pis_batch_poll(pis_batch* b, int32_t* done, int32_t cap, int32_t* n_done);
/* State of a slot (3 x n arrays, any may be NULL) and its last energies and step count. */
pis_status pis_batch_result(pis_batch* b, int32_t slot, double* pos, double* vel, double* force, double* pe,
                            double* ke, int64_t* steps_done);
/* Per-step potential energies of a slot's last n steps (n <= 1024). */
pis_status pis_batch_pe_history(pis_batch* b, int32_t slot, int64_t n, double* pe);
pis_status pis_batch_release(pis_batch* b, int32_t slot);
int64_t pis_batch_atoms(const pis_batch* b);
const char* pis_batch_last_error(const pis_batch* b);
void pis_batch_destroy(pis_batch* b);

/* One request of a served stream: an LJ job arriving `arrival_s` seconds after the start. */
typedef struct {
    double arrival_s;
    pis_lj_job job;
} pis_request;

typedef struct {
    double admitted_s;  /* wall seconds after the start */
    double finished_s;
    int64_t atoms;
    int64_t steps;
    double pe, ke;      /* energies after the last step */
    int32_t status;     /* pis_status of the job */
} pis_request_result;

/* Serve a request stream in wall-clock time: requests are queued at their arrival times,
 * admitted as soon as pool space allows (continuous batching: they join slots already running),
 * advanced in graphs of graph_steps steps, and released when done. Returns per-request times and
 * the total wall seconds. */
pis_status pis_serve_run(pis_batch* b, const pis_request* reqs, int32_t n, int64_t graph_steps,
                         pis_request_result* out, double* wall_s);

/* Accounting of the last pis_serve_run on a batch, per graph: atom-steps done (sum over slots of
 * atoms x steps taken in the graph) and device seconds from the end of the previous graph to the
 * end of this one (CUDA events; admissions, evaluations and any wait for the host included).
 * "Saturated" graphs are those queued while a request was waiting for pool space: their rate is
 * the served throughput at saturation, free of the stream's ramp-up and drain. */
typedef struct {
    int64_t graphs, saturated_graphs;
    double atom_steps, device_s;
    double saturated_atom_steps, saturated_device_s;
} pis_serve_stats;
pis_status pis_serve_last_stats(const pis_batch* b, pis_serve_stats* out);

/* Number of kernel launches this library issued on the calling thread's contexts since load
 * (every kernel of this library, graph launches counted per contained kernel). */
int64_t pis_gpu_kernel_launches(void);

/* Library / device identification, for logs. */
const char* pis_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PIS_GPU_H */
