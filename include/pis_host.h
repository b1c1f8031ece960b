/*
 * pis_host.h - C ABI of the host side around the GPU MD step: the reference's input-file and
 * data-file readers, its System driver (read -> contextualize -> run with thermo output and
 * trajectory dumps) and its .lammpstrj writer, restated in C++ on top of pis_gpu.h.
 * Functions that only read or write files need no GPU.
 */
#ifndef PIS_HOST_H
#define PIS_HOST_H

#include <stdint.h>

#include "pis_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A parsed LAMMPS-style data file: run_read_data, src/readers/input_file/commands.rs:147-384
 * (sections Masses / PairCoeffs / Atoms / Velocities, 1-based ids, default rcut 2.5 sigma, the
 * single-type PairCoeffs form taking precedence whenever the second token parses as a float). */
typedef struct pis_data pis_data;

pis_status pis_data_read(const char* path, pis_data** out, char* err, int32_t errlen);
int64_t pis_data_n_atoms(const pis_data* d);
int32_t pis_data_n_types(const pis_data* d);
int32_t pis_data_n_pairs(const pis_data* d);
/* bounds = xlo xhi ylo yhi zlo zhi; has_velocities = a Velocities section was present (which
 * turns off Maxwell-Boltzmann initialisation, commands.rs:194-197). Any pointer may be NULL. */
pis_status pis_data_get(const pis_data* d, int32_t* type_ids, double* masses, double* pos, double* vel,
                        double* bounds, int32_t* has_velocities);
pis_status pis_data_pairs(const pis_data* d, pis_lj_pair* out);
void pis_data_free(pis_data* d);

/* Write a data file with Masses, PairCoeffs, Atoms and Velocities sections: the restart format
 * (the reference reads exactly these sections back). Floats are written in shortest round-trip
 * form, so a read of the written file restores the state bit for bit. */
pis_status pis_data_write(const char* path, int64_t n, int32_t n_types, const int32_t* type_ids, const double* masses,
                          const double* pos, const double* vel, const double* bounds, const pis_lj_pair* pairs,
                          int32_t n_pairs);

/* Maxwell-Boltzmann velocities (3 x n) for per-atom masses at temperature T (reference units:
 * sigma_v = sqrt(KB T / m), KB = 0.0083144621) from `seed`, then drift removal and rescaling to T
 * (Atoms::start_velocities, src/atoms/velocities.rs:10-59). The random stream is this library's
 * (SplitMix64 + Box-Muller), not the reference's rand crate stream. */
pis_status pis_maxwell_boltzmann(int64_t n, const double* masses_per_atom, double temperature, uint64_t seed,
                                 double* vel);

/* Format a double like Rust's `{}` (shortest round-trip decimal, no exponent) into buf (at most
 * buflen - 1 characters and a terminator); returns the full length (up to 342), so a call with
 * buf = NULL sizes the buffer. */
int32_t pis_format_f64(double v, char* buf, int32_t buflen);

/* System::new(infile).read().contextualize() (src/system.rs:41-175), with the GPU manager in place
 * of LJVOffsetManager: precision is a pis_precision, skin the Verlet skin. */
typedef struct pis_system pis_system;

pis_status pis_system_open(const char* infile, int32_t precision, double skin, pis_system** out);
/* Simulation::run (src/simulation.rs:8-88): dump at step 0, initial force evaluation and "0 PE",
 * then `run` steps of the selected ensemble, a thermo line "i PE KE H T P" per step (thermo_path,
 * or stdout when NULL) and a dump every dump_step steps. */
pis_status pis_system_run(pis_system* s, const char* thermo_path);
/* Accessors for tests and tools. */
int64_t pis_system_steps(const pis_system* s);
double pis_system_timestep(const pis_system* s);
int32_t pis_system_ensemble(const pis_system* s); /* 0 NVE, 1 NVT, 2 NPT (simulation.rs:118-132) */
/* Positions, velocities and forces (x,y,z per atom; any pointer may be NULL). Before the run
 * has put the state on the GPU: the state contextualize built (positions as read, velocities as
 * read or drawn by `velocity create`, zero forces). */
pis_status pis_system_state(pis_system* s, double* pos, double* vel, double* force);
/* The pair table contextualize built (the data file's PairCoeffs, replaced by `pair_style lj/cut`
 * and its `pair_coeff` rows when those are given, src/system.rs:120-168): writes up to `cap`
 * entries to `out` (may be NULL) and returns how many there are. */
int32_t pis_system_pairs(const pis_system* s, pis_lj_pair* out, int32_t cap);
/* The `dump` command's step and file name (run_dump, src/readers/input_file/commands.rs:485-496;
 * defaults 1 and "dump.lammpstrj"); `file` receives at most cap - 1 characters. */
pis_status pis_system_dump(const pis_system* s, int64_t* dump_step, char* file, int32_t cap);
const char* pis_system_last_error(const pis_system* s);
void pis_system_close(pis_system* s);

#ifdef __cplusplus
}
#endif
#endif /* PIS_HOST_H */
