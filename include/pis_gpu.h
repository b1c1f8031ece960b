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
    PIS_ERR_UNSUPPORTED = 26       /* e.g. non-orthorhombic box */
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
    PIS_LIST_HALF = 1,       /* Newton-3 half list, forces on j scattered with FP64 atomics */
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

/* Select a measured variant: list kind (pis_list_kind) and PIS_OPT_* flags. Takes effect at the
 * next set_state. */
pis_status pis_gpu_set_options(pis_gpu_ctx* ctx, int32_t list_kind, int32_t flags);

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

/* Download positions / velocities / forces (3 x N each, any may be NULL). */
pis_status pis_gpu_get_state(pis_gpu_ctx* ctx, double* pos, double* vel, double* force);

/* Atoms::kinetic_energy and Atoms::virial_tensor (src/atoms/properties.rs:17-24, 49-51) of the
 * current device state; virial is row-major W[a][b] = sum_i r_i[a] F_i[b]. Either may be NULL. */
pis_status pis_gpu_reductions(pis_gpu_ctx* ctx, double* ke, double* virial);

/* Per-atom neighbour sets within each pair's cutoff at the current positions, in original atom
 * indices, ascending per atom - the sets of LJVPBuildListManager::build_neighbour_list
 * (src/potentials/lennard_jones.rs:345-415). offsets has n+1 entries; idx receives up to cap
 * entries; total receives the full count. */
pis_status pis_gpu_neighbour_list(pis_gpu_ctx* ctx, int64_t* offsets, int32_t* idx, int64_t cap,
                                  int64_t* total);

/* Ensemble hooks (src/potentials/potential.rs:45-50, 119-134): v <- M v for every atom, and
 * Atoms::scale_box (src/atoms/transformations.rs:5-16): r <- (M h) h^-1 r with h <- M h. Both
 * take row-major 3x3 M. scale_box forces a neighbour-list rebuild at the next evaluation. */
pis_status pis_gpu_scale_velocities(pis_gpu_ctx* ctx, const double* m_rowmajor);
pis_status pis_gpu_scale_box(pis_gpu_ctx* ctx, const double* m_rowmajor);

pis_status pis_gpu_get_stats(pis_gpu_ctx* ctx, pis_gpu_stats* out);
const char* pis_gpu_last_error(const pis_gpu_ctx* ctx);
void pis_gpu_destroy(pis_gpu_ctx* ctx);

/* Measurement hook (no counterpart in the reference): run n_steps NVE steps like
 * pis_gpu_verlet_step_nve, timing them with CUDA events on the context's stream; device_ms gets
 * the elapsed device time. If stage_ms is non-NULL, events captured into the step graphs also
 * time the five stages of a step (integrate-1, list rebuild, forces, integrate-2, reductions),
 * summed over the steps, at the cost of one host sync per 50-step graph. */
pis_status pis_gpu_run_timed(pis_gpu_ctx* ctx, double dt, int64_t n_steps, double* device_ms, double* stage_ms);

/* Force evaluation that allocates no device memory (no counterpart in the reference). For callers
 * that cannot allocate device memory while running - a host whose framework owns the whole device
 * memory pool, or a real-time loop where cudaMalloc's latency and implicit synchronisation are not
 * allowed. Same result as pis_gpu_compute_potential (FP64, reference arithmetic) on buffers the
 * caller owns: d_type_ids (n, 1-based), d_pos (3 x n) are device inputs; d_forces (3 x n) and d_pe
 * (1 value) are device outputs; table and h_colmajor are host arrays; stream is a cudaStream_t
 * (NULL = default stream) and the call returns once the work is enqueued on it.
 * Limits of the fixed scratch: n <= 262144 atoms, at most 65536 cells at the largest cutoff, at
 * least 3 cells per axis, at most 4 atom types; larger inputs return PIS_ERR_INVALID_ARGUMENT
 * (PIS_ERR_BOX_TOO_SMALL below 3 cells). The scratch is one device array shared by every call on
 * a device: calls that overlap on the GPU race and must be serialised by the caller. The first
 * call on a device looks up the scratch address; make it before any stream capture. */
pis_status pis_gpu_compute_potential_noalloc(const pis_lj_pair* table, int32_t n_pairs, int32_t n_types, int64_t n,
                                             const int32_t* d_type_ids, const double* d_pos,
                                             const double* h_colmajor, double* d_forces, double* d_pe,
                                             void* stream);

/* Number of kernel launches this library issued on the calling thread's contexts since load
 * (every kernel of this library, graph launches counted per contained kernel). */
int64_t pis_gpu_kernel_launches(void);

/* Library / device identification, for logs. */
const char* pis_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PIS_GPU_H */
