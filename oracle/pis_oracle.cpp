// CPU oracle for the PIS Lennard-Jones MD step: TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++ with FP64 scalar arithmetic, the algorithms of
// the reference crate (vivekadishankara/pis, a Rust program) on the MD hot path.
// It exists so that tests, the smoke check and the CPU-baseline leg of the benchmark
// can compare the CUDA library against the reference's own arithmetic. The product
// library never links, loads or calls it.
//
// Parity status: the reference cannot be compiled here (Rust toolchain absent) and
// its own tests pin no forces, energies or trajectories, so this restatement is
// "parity unpinned" with respect to reference outputs. It is anchored instead on
// known-answer tests derived from the reference's example inputs (FCC shell counts,
// closed-form lattice energies, Newton's third law, agreement between the five
// reference force managers) - see tests/test_oracle_known_answers.py - and its answers on
// seeded states and on those inputs are committed under tests/golden.
//
// Operation order follows the Rust source literally and this file must be compiled
// with -ffp-contract=off: Rust never fuses a*b+c into an FMA, and GCC on aarch64
// would otherwise do so at -O2.
//
// Third-party arithmetic at the boundary: nalgebra 0.34.1 supplies the 3x3 inverse
// (adjugate over determinant, determinant by first-row cofactor expansion), the 3x3
// determinant, matrix-vector products and Vector3::norm (sqrt of x*x+y*y+z*z). Those
// published algorithms are restated below; for the orthorhombic boxes the data-file
// reader produces (src/readers/input_file/commands.rs:352,362 pass xy=xz=yz=0) every
// summation order gives the same bits.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <unordered_set>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Mirror of the reference's Atoms + SimulationBox + pair table (src/atoms/new.rs:9-17,
// src/simulation_box.rs:5-9, src/potentials/potential.rs:143-144). Matrices are row-major
// h[3*r + c]. Positions/velocities/forces are 3 x N column-major (x,y,z per atom), the
// nalgebra Matrix3xX layout. Type ids are 1-based. The pair table is dense
// n_types x n_types, addressed with key (min(ti,tj), max(ti,tj)) as get_potential_ij does.
typedef struct {
    int64_t n;
    int32_t n_types;
    int32_t pbc[3];
    const int32_t* type_ids;
    const double* masses;
    double* pos;
    double* vel;
    double* force;
    double h[9];
    double hinv[9];
    const double* eps;
    const double* sigma;
    const double* rcut;
    const int32_t* present;
    int32_t shift;
} or_system;

// 3x3 inverse as adjugate / determinant (nalgebra try_inverse for 3x3; used by
// src/simulation_box.rs:13 and src/atoms/transformations.rs:12).
void or_inverse3(const double* m, double* out) {
    #define M(r, c) m[3 * (r) + (c)]
    double minor_m12_m23 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    double minor_m11_m23 = M(1, 0) * M(2, 2) - M(2, 0) * M(1, 2);
    double minor_m11_m22 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    double det = M(0, 0) * minor_m12_m23 - M(0, 1) * minor_m11_m23 + M(0, 2) * minor_m11_m22;
    out[0] = minor_m12_m23 / det;
    out[1] = (M(0, 2) * M(2, 1) - M(2, 2) * M(0, 1)) / det;
    out[2] = (M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2)) / det;
    out[3] = -minor_m11_m23 / det;
    out[4] = (M(0, 0) * M(2, 2) - M(2, 0) * M(0, 2)) / det;
    out[5] = (M(0, 2) * M(1, 0) - M(1, 2) * M(0, 0)) / det;
    out[6] = minor_m11_m22 / det;
    out[7] = (M(0, 1) * M(2, 0) - M(2, 1) * M(0, 0)) / det;
    out[8] = (M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1)) / det;
    #undef M
}

// Determinant by first-row cofactor expansion (SimulationBox::volume,
// src/simulation_box.rs:67-69, takes its absolute value).
double or_determinant3(const double* m) {
    #define M(r, c) m[3 * (r) + (c)]
    double minor_m12_m23 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    double minor_m11_m23 = M(1, 0) * M(2, 2) - M(2, 0) * M(1, 2);
    double minor_m11_m22 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    return M(0, 0) * minor_m12_m23 - M(0, 1) * minor_m11_m23 + M(0, 2) * minor_m11_m22;
    #undef M
}

static inline void matvec(const double* m, const double* v, double* out) {
    for (int r = 0; r < 3; ++r) out[r] = m[3 * r] * v[0] + m[3 * r + 1] * v[1] + m[3 * r + 2] * v[2];
}

// Minimum image of a displacement: s = h^-1 r; s -= round(s) where periodic; r = h s.
// src/simulation_box.rs:17-27. round() is half away from zero, as Rust's f64::round.
void or_min_image(const or_system* sys, double* r) {
    double s[3];
    matvec(sys->hinv, r, s);
    for (int d = 0; d < 3; ++d)
        if (sys->pbc[d]) s[d] -= std::round(s[d]);
    matvec(sys->h, s, r);
}

// Wrap a position into the box: s -= floor(s). src/simulation_box.rs:29-42.
void or_wrap(const or_system* sys, double* r) {
    double s[3];
    matvec(sys->hinv, r, s);
    for (int d = 0; d < 3; ++d)
        if (sys->pbc[d]) s[d] -= std::floor(s[d]);
    matvec(sys->h, s, r);
}

static inline double norm_squared(const double* r) { return r[0] * r[0] + r[1] * r[1] + r[2] * r[2]; }

// LennardJones::compute_potential, src/potentials/lennard_jones.rs:33-55.
// rij = r_j - r_i; returns u and the vector f that the managers subtract from F_i and
// add to F_j. powi(n) is repeated multiplication (x*x, x*(x*x)).
void or_lj_pair(double epsilon, double sigma, double rcut, int32_t shift, const double* rij,
                double* u_out, double* f_out) {
    double rij2 = norm_squared(rij);
    double inv_rij2 = 1.0 / rij2;
    double s2 = sigma * sigma * inv_rij2;
    double vdw = s2 * (s2 * s2);
    double rep = vdw * vdw;
    double u = 4.0 * epsilon * (rep - vdw);
    double c = 24.0 * epsilon * (2.0 * rep - vdw) * inv_rij2;
    f_out[0] = c * rij[0];
    f_out[1] = c * rij[1];
    f_out[2] = c * rij[2];
    if (shift) {
        double ci2 = (sigma / rcut) * (sigma / rcut);
        double ca = ci2 * (ci2 * ci2);
        double cr = ca * ca;
        double u_cut = 4.0 * epsilon * (cr - ca);
        u -= u_cut;
    }
    *u_out = u;
}

// get_potential_ij, src/potentials/potential.rs:181-192. Returns the dense-table slot or -1.
static inline int pair_slot(const or_system* sys, int64_t i, int64_t j) {
    int ti = sys->type_ids[i], tj = sys->type_ids[j];
    int a = ti < tj ? ti : tj, b = ti < tj ? tj : ti;
    if (a < 1 || b > sys->n_types) return -1;
    int k = (a - 1) * sys->n_types + (b - 1);
    return sys->present[k] ? k : -1;
}

// PairPotentialManager::max_rcut, src/potentials/potential.rs:170-179.
double or_max_rcut(const or_system* sys) {
    double m = 0.0;
    int nt = sys->n_types;
    for (int k = 0; k < nt * nt; ++k)
        if (sys->present[k] && m < sys->rcut[k]) m = sys->rcut[k];
    return m;
}

// Atoms::divide_into_cells, src/atoms/neighbour_list.rs:45-57.
void or_divide_into_cells(const or_system* sys, double rcut, int64_t* ncell) {
    for (int d = 0; d < 3; ++d) {
        double col[3] = {sys->h[d], sys->h[3 + d], sys->h[6 + d]};
        double len = std::sqrt(norm_squared(col));
        double q = std::floor(len / rcut);
        int64_t n = (q >= 1.0 && q < 9.0e18) ? (int64_t)q : 0;
        ncell[d] = n == 0 ? 1 : n;
    }
}

// Rust `f64 as usize` saturates: negatives and NaN become 0.
static inline uint64_t as_usize(double v) {
    if (!(v > 0.0)) return 0;
    if (v >= 1.8446744073709552e19) return UINT64_MAX;
    return (uint64_t)v;
}

static inline int64_t cell_index(int64_t cx, int64_t cy, int64_t cz, int64_t nx, int64_t ny) {
    return (cz * ny + cy) * nx + cx;
}

// Atoms::rcut_cells, src/atoms/neighbour_list.rs:9-42. Atoms are pushed in index order.
static std::vector<std::vector<int64_t>> rcut_cells(const or_system* sys, int64_t nx, int64_t ny, int64_t nz) {
    std::vector<std::vector<int64_t>> cells((size_t)(nx * ny * nz));
    for (int64_t i = 0; i < sys->n; ++i) {
        double s[3];
        matvec(sys->hinv, sys->pos + 3 * i, s);
        uint64_t c[3] = {as_usize(std::floor(s[0] * (double)nx)), as_usize(std::floor(s[1] * (double)ny)),
                         as_usize(std::floor(s[2] * (double)nz))};
        uint64_t n3[3] = {(uint64_t)nx, (uint64_t)ny, (uint64_t)nz};
        for (int d = 0; d < 3; ++d)
            if (sys->pbc[d]) c[d] = c[d] % n3[d];
        // A non-periodic coordinate outside the box would index out of range and panic in
        // the reference; clamp so the oracle stays defined (never reached by the tests).
        for (int d = 0; d < 3; ++d)
            if (c[d] >= n3[d]) c[d] = n3[d] - 1;
        cells[(size_t)cell_index((int64_t)c[0], (int64_t)c[1], (int64_t)c[2], nx, ny)].push_back(i);
    }
    return cells;
}

// Copy of the 14-entry forward half stencil of src/atoms/neighbour_list.rs:94-165
// (self cell first, then 13 forward cells) - the order fixes the summation order.
static const int FWD[14][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 1, 0}, {0, 1, 0},  {1, 1, 0},
                               {-1, -1, 1}, {0, -1, 1}, {1, -1, 1}, {-1, 0, 1}, {0, 0, 1},
                               {1, 0, 1},  {-1, 1, 1},  {0, 1, 1},  {1, 1, 1}};

static inline int64_t rem_euclid(int64_t a, int64_t n) {
    int64_t r = a % n;
    return r < 0 ? r + n : r;
}

// Shared pair evaluation of every manager: min-image, table lookup, `> rcut` skip (so
// r == rcut is kept), pair energy/force. Returns 0 when the pair is skipped.
static inline int eval_pair(const or_system* sys, int64_t i, int64_t j, double* u, double* f) {
    double rij[3] = {sys->pos[3 * j] - sys->pos[3 * i], sys->pos[3 * j + 1] - sys->pos[3 * i + 1],
                     sys->pos[3 * j + 2] - sys->pos[3 * i + 2]};
    or_min_image(sys, rij);
    int k = pair_slot(sys, i, j);
    if (k < 0) return 0;  // reference prints "potential was missing" and continues
    if (std::sqrt(norm_squared(rij)) > sys->rcut[k]) return 0;
    or_lj_pair(sys->eps[k], sys->sigma[k], sys->rcut[k], sys->shift, rij, u, f);
    return 1;
}

// LJManager::compute_potential, src/potentials/lennard_jones.rs:62-99 (all pairs i<j).
double or_compute_allpairs(or_system* sys) {
    double pe = 0.0;
    for (int64_t i = 0; i < sys->n; ++i)
        for (int64_t j = i + 1; j < sys->n; ++j) {
            double u, f[3];
            if (!eval_pair(sys, i, j, &u, f)) continue;
            pe += u;
            for (int d = 0; d < 3; ++d) {
                sys->force[3 * i + d] -= f[d];
                sys->force[3 * j + d] += f[d];
            }
        }
    return pe;
}

// LJVerletManager::compute_potential, src/potentials/lennard_jones.rs:103-178: 27 cells,
// deduplicated per home cell, pairs with i > j only.
double or_compute_verlet27(or_system* sys) {
    int64_t nc[3];
    or_divide_into_cells(sys, or_max_rcut(sys), nc);
    int64_t nx = nc[0], ny = nc[1], nz = nc[2];
    auto cells = rcut_cells(sys, nx, ny, nz);
    double pe = 0.0;
    std::vector<int64_t> seen;
    for (int64_t cx = 0; cx < nx; ++cx)
        for (int64_t cy = 0; cy < ny; ++cy)
            for (int64_t cz = 0; cz < nz; ++cz) {
                int64_t cur = cell_index(cx, cy, cz, nx, ny);
                seen.clear();
                for (int dx = -1; dx <= 1; ++dx)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dz = -1; dz <= 1; ++dz) {
                            int64_t nb = cell_index(rem_euclid(cx + dx, nx), rem_euclid(cy + dy, ny),
                                                    rem_euclid(cz + dz, nz), nx, ny);
                            if (std::find(seen.begin(), seen.end(), nb) != seen.end()) continue;
                            seen.push_back(nb);
                            for (int64_t i : cells[cur])
                                for (int64_t j : cells[nb]) {
                                    if (i <= j) continue;
                                    double u, f[3];
                                    if (!eval_pair(sys, i, j, &u, f)) continue;
                                    pe += u;
                                    for (int d = 0; d < 3; ++d) {
                                        sys->force[3 * i + d] -= f[d];
                                        sys->force[3 * j + d] += f[d];
                                    }
                                }
                        }
            }
    return pe;
}

// ---- Exact sums (not part of the reference) -----------------------------------------------------
// The reference adds energies in its cell-walk order and the virial through a blocked matrix
// product; a parallel GPU sums in another order, so two correct programs differ in the last bits
// of every reduction. To compare them without depending on the order, both sides can also form
// one defined sum: each term t is quantised to q(t) = sign(t) * floor(|t| * 2^104) (an integer),
// the integers are added exactly, and the result is the double nearest to (sum q) * 2^-104, ties
// to even. A term of magnitude 2^56 or more, an infinity or a NaN makes the sum NaN. Terms of
// magnitude 2^-52 or more are represented exactly, so for them this is the exactly rounded sum.
// This implementation (four 64-bit two's-complement limbs, full carry on every add) is written
// independently of the GPU library's (lazily carried 32-bit limbs), so each checks the other.
typedef struct {
    uint64_t w[4];
    int64_t bad;
} or_xsum;

static const int XSUM_FRAC = 104;

void or_xsum_clear(or_xsum* x) {
    std::memset(x, 0, sizeof(*x));
}

void or_xsum_add(or_xsum* x, double t) {
    if (!std::isfinite(t) || std::fabs(t) >= 0x1p56) {
        x->bad++;
        return;
    }
    if (t == 0.0) return;
    int e = 0;
    const double m = std::frexp(std::fabs(t), &e);  // |t| = m 2^e, m in [0.5, 1)
    const uint64_t mant = (uint64_t)std::ldexp(m, 53);  // exact, in [2^52, 2^53)
    const int sh = e - 53 + XSUM_FRAC;                // q = floor(mant * 2^sh)
    uint64_t q[4] = {0, 0, 0, 0};
    if (sh >= 0) {
        const int w = sh / 64, b = sh % 64;
        q[w] |= mant << b;
        if (b && w + 1 < 4) q[w + 1] |= mant >> (64 - b);
    } else if (sh > -64) {
        q[0] = mant >> (-sh);
    }
    if (t < 0.0) {  // two's complement negation of the 256-bit q
        unsigned carry = 1;
        for (int k = 0; k < 4; ++k) {
            const uint64_t v = ~q[k];
            q[k] = v + carry;
            carry = (carry && q[k] == 0) ? 1u : 0u;
        }
    }
    unsigned __int128 c = 0;
    for (int k = 0; k < 4; ++k) {
        c += (unsigned __int128)x->w[k] + q[k];
        x->w[k] = (uint64_t)c;
        c >>= 64;
    }
}

double or_xsum_value(const or_xsum* x) {
    if (x->bad) return std::nan("");
    uint64_t w[4] = {x->w[0], x->w[1], x->w[2], x->w[3]};
    const bool neg = (w[3] >> 63) != 0;
    if (neg) {
        unsigned carry = 1;
        for (int k = 0; k < 4; ++k) {
            const uint64_t v = ~w[k];
            w[k] = v + carry;
            carry = (carry && w[k] == 0) ? 1u : 0u;
        }
    }
    int p = -1;  // highest set bit
    for (int k = 3; k >= 0 && p < 0; --k)
        if (w[k]) p = 64 * k + 63 - __builtin_clzll(w[k]);
    if (p < 0) return 0.0;
    auto bit = [&](int i) -> uint64_t { return (w[i / 64] >> (i % 64)) & 1u; };
    uint64_t mant = 0;
    int lo = p - 52;  // lowest bit kept
    if (lo <= 0) {
        mant = w[0];  // p <= 52: the whole value fits in the mantissa
        lo = 0;
    } else {
        for (int i = p; i >= lo; --i) mant = (mant << 1) | bit(i);
        const uint64_t half = bit(lo - 1);
        bool sticky = false;
        for (int i = lo - 2; i >= 0 && !sticky; --i) sticky = bit(i) != 0;
        if (half && (sticky || (mant & 1u))) {
            mant += 1;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                lo += 1;
            }
        }
    }
    const double v = std::ldexp((double)mant, lo - XSUM_FRAC);
    return neg ? -v : v;
}

// Exact sum of an array (for tests of the definition itself).
double or_xsum_array(const double* v, int64_t n) {
    or_xsum x;
    or_xsum_clear(&x);
    for (int64_t i = 0; i < n; ++i) or_xsum_add(&x, v[i]);
    return or_xsum_value(&x);
}

// Sink for the exact energy sum of the offset manager's walk (set by the exact run loops).
static or_xsum* g_pe_sink = nullptr;

// LJVOffsetManager::compute_potential, src/potentials/lennard_jones.rs:186-244: the
// production path. Cells at max_rcut, 14-offset half stencil, same-cell pairs need i > j.
// Forces are accumulated (the caller zeroes them, src/potentials/potential.rs:24).
double or_compute_offset(or_system* sys) {
    int64_t nc[3];
    or_divide_into_cells(sys, or_max_rcut(sys), nc);
    int64_t nx = nc[0], ny = nc[1], nz = nc[2];
    auto cells = rcut_cells(sys, nx, ny, nz);
    double pe = 0.0;
    for (int64_t cx = 0; cx < nx; ++cx)
        for (int64_t cy = 0; cy < ny; ++cy)
            for (int64_t cz = 0; cz < nz; ++cz) {
                int64_t cur = cell_index(cx, cy, cz, nx, ny);
                for (int o = 0; o < 14; ++o) {
                    int64_t nb = cell_index(rem_euclid(cx + FWD[o][0], nx), rem_euclid(cy + FWD[o][1], ny),
                                            rem_euclid(cz + FWD[o][2], nz), nx, ny);
                    for (int64_t i : cells[cur])
                        for (int64_t j : cells[nb]) {
                            if (cur == nb && i <= j) continue;
                            double u, f[3];
                            if (!eval_pair(sys, i, j, &u, f)) continue;
                            pe += u;
                            if (g_pe_sink) or_xsum_add(g_pe_sink, u);
                            for (int d = 0; d < 3; ++d) {
                                sys->force[3 * i + d] -= f[d];
                                sys->force[3 * j + d] += f[d];
                            }
                        }
                }
            }
    return pe;
}

// LJVParallelManager::compute_potential, src/potentials/lennard_jones.rs:253-336, with
// OpenMP threads in place of rayon: cells in cx-major order (cell_indices_for_parallel,
// src/atoms/neighbour_list.rs:67-82), per-thread force buffers and energies, then a serial
// reduction into the forces. Unlike the Rust original, whose closures hold a global write
// lock, the threads here really run concurrently. Stencil cells are de-duplicated per home
// cell as in the original.
double or_compute_parallel(or_system* sys, int32_t nthreads) {
    int64_t nc[3];
    or_divide_into_cells(sys, or_max_rcut(sys), nc);
    int64_t nx = nc[0], ny = nc[1], nz = nc[2];
    auto cells = rcut_cells(sys, nx, ny, nz);
    int nt = nthreads > 0 ? nthreads : 1;
#ifndef _OPENMP
    nt = 1;
#endif
    int64_t ncells = nx * ny * nz;
    std::vector<std::vector<double>> tf((size_t)nt);
    std::vector<double> tpe((size_t)nt, 0.0);
#ifdef _OPENMP
    #pragma omp parallel num_threads(nt)
#endif
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        std::vector<double>& f_t = tf[(size_t)tid];
        f_t.assign((size_t)(3 * sys->n), 0.0);
        double pe_t = 0.0;
        int64_t seen[14];
#ifdef _OPENMP
        #pragma omp for schedule(static)
#endif
        for (int64_t c = 0; c < ncells; ++c) {
            int64_t cz = c % nz, cy = (c / nz) % ny, cx = c / (nz * ny);
            int64_t cur = cell_index(cx, cy, cz, nx, ny);
            int nseen = 0;
            for (int o = 0; o < 14; ++o) {
                int64_t nb = cell_index(rem_euclid(cx + FWD[o][0], nx), rem_euclid(cy + FWD[o][1], ny),
                                        rem_euclid(cz + FWD[o][2], nz), nx, ny);
                bool dup = false;
                for (int q = 0; q < nseen; ++q) dup |= seen[q] == nb;
                if (dup) continue;
                seen[nseen++] = nb;
                for (int64_t i : cells[cur])
                    for (int64_t j : cells[nb]) {
                        if (cur == nb && i <= j) continue;
                        double u, f[3];
                        if (!eval_pair(sys, i, j, &u, f)) continue;
                        pe_t += u;
                        for (int d = 0; d < 3; ++d) {
                            f_t[3 * i + d] -= f[d];
                            f_t[3 * j + d] += f[d];
                        }
                    }
            }
        }
        tpe[(size_t)tid] = pe_t;
    }
    for (int t = 0; t < nt; ++t)
        for (int64_t k = 0; k < 3 * sys->n; ++k) sys->force[k] += tf[(size_t)t][k];
    double pe = 0.0;
    for (int t = 0; t < nt; ++t) pe += tpe[(size_t)t];
    return pe;
}

// LJVPBuildListManager::build_neighbour_list, src/potentials/lennard_jones.rs:345-415:
// full list (every j != i with |minimg(r_j - r_i)| <= rcut) over the 27 cells. The
// de-duplication set is cleared inside the dx loop (:410), exactly as the original.
// Writes CSR offsets[n+1] and idx[]; returns the total count (idx filled only up to cap).
int64_t or_build_full_list(const or_system* sys, int64_t* offsets, int32_t* idx, int64_t cap) {
    int64_t nc[3];
    or_divide_into_cells(sys, or_max_rcut(sys), nc);
    int64_t nx = nc[0], ny = nc[1], nz = nc[2];
    auto cells = rcut_cells(sys, nx, ny, nz);
    std::vector<std::vector<int32_t>> lists((size_t)sys->n);
    std::vector<int64_t> seen;
    for (int64_t cx = 0; cx < nx; ++cx)
        for (int64_t cy = 0; cy < ny; ++cy)
            for (int64_t cz = 0; cz < nz; ++cz) {
                int64_t cur = cell_index(cx, cy, cz, nx, ny);
                seen.clear();
                for (int dx = -1; dx <= 1; ++dx) {
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dz = -1; dz <= 1; ++dz) {
                            int64_t nb = cell_index(rem_euclid(cx + dx, nx), rem_euclid(cy + dy, ny),
                                                    rem_euclid(cz + dz, nz), nx, ny);
                            if (std::find(seen.begin(), seen.end(), nb) != seen.end()) continue;
                            seen.push_back(nb);
                            for (int64_t i : cells[cur])
                                for (int64_t j : cells[nb]) {
                                    if (cur == nb && i == j) continue;
                                    double rij[3] = {sys->pos[3 * j] - sys->pos[3 * i],
                                                     sys->pos[3 * j + 1] - sys->pos[3 * i + 1],
                                                     sys->pos[3 * j + 2] - sys->pos[3 * i + 2]};
                                    or_min_image(sys, rij);
                                    int k = pair_slot(sys, i, j);
                                    if (k < 0) continue;
                                    if (std::sqrt(norm_squared(rij)) > sys->rcut[k]) continue;
                                    lists[(size_t)i].push_back((int32_t)j);
                                }
                        }
                    seen.clear();
                }
            }
    int64_t total = 0;
    offsets[0] = 0;
    for (int64_t i = 0; i < sys->n; ++i) {
        for (int32_t j : lists[(size_t)i]) {
            if (total < cap) idx[total] = j;
            ++total;
        }
        offsets[i + 1] = total;
    }
    return total;
}

// LJVPBuildListManager::compute_potential, src/potentials/lennard_jones.rs:419-455:
// per-atom loop over the full list, F_i -= f only, forces OVERWRITTEN, PE = sum_i PE_i / 2.
double or_compute_full_list(or_system* sys) {
    std::vector<int64_t> off((size_t)sys->n + 1);
    int64_t total = or_build_full_list(sys, off.data(), nullptr, 0);
    std::vector<int32_t> idx((size_t)total);
    or_build_full_list(sys, off.data(), idx.data(), total);
    std::vector<double> tpe((size_t)sys->n, 0.0);
    for (int64_t i = 0; i < sys->n; ++i) {
        double fi[3] = {0.0, 0.0, 0.0};
        for (int64_t q = off[(size_t)i]; q < off[(size_t)i + 1]; ++q) {
            int64_t j = idx[(size_t)q];
            double rij[3] = {sys->pos[3 * j] - sys->pos[3 * i], sys->pos[3 * j + 1] - sys->pos[3 * i + 1],
                             sys->pos[3 * j + 2] - sys->pos[3 * i + 2]};
            or_min_image(sys, rij);
            int k = pair_slot(sys, i, j);
            if (k < 0) continue;
            double u, f[3];
            or_lj_pair(sys->eps[k], sys->sigma[k], sys->rcut[k], sys->shift, rij, &u, f);
            tpe[(size_t)i] += u;
            for (int d = 0; d < 3; ++d) fi[d] += -f[d];
        }
        for (int d = 0; d < 3; ++d) sys->force[3 * i + d] = fi[d];
    }
    double pe = 0.0;
    for (int64_t i = 0; i < sys->n; ++i) pe += tpe[(size_t)i];
    return pe / 2.0;
}

// Manager selector for the step functions.
enum { OR_OFFSET = 0, OR_ALLPAIRS = 1, OR_VERLET27 = 2, OR_PARALLEL = 3, OR_FULLLIST = 4 };

static double compute(or_system* sys, int32_t manager, int32_t nthreads) {
    switch (manager) {
        case OR_ALLPAIRS: return or_compute_allpairs(sys);
        case OR_VERLET27: return or_compute_verlet27(sys);
        case OR_PARALLEL: return or_compute_parallel(sys, nthreads);
        case OR_FULLLIST: return or_compute_full_list(sys);
        default: return or_compute_offset(sys);
    }
}

// PotentialManager::compute_potential as the caller sees it after zeroing the forces.
double or_compute_potential(or_system* sys, int32_t manager, int32_t nthreads) {
    std::memset(sys->force, 0, sizeof(double) * 3 * (size_t)sys->n);
    return compute(sys, manager, nthreads);
}

static inline double mass_i(const or_system* sys, int64_t i) { return sys->masses[sys->type_ids[i] - 1]; }

// PotentialManager::verlet_step_nve, src/potentials/potential.rs:15-33, with
// Atoms::current_acceleration (src/atoms/properties.rs:32-39) inlined:
//   a_t = F/m;  x += v*dt + (a_t*0.5)*dt^2;  wrap;  F = 0;  PE = compute;  a_tdt = F/m;
//   v += ((a_t + a_tdt)*0.5)*dt.
double or_verlet_step_nve(or_system* sys, double dt, int32_t manager, int32_t nthreads) {
    int64_t n = sys->n;
    std::vector<double> a_t((size_t)(3 * n));
    for (int64_t i = 0; i < n; ++i) {
        double m = mass_i(sys, i);
        for (int d = 0; d < 3; ++d) a_t[3 * i + d] = 0.0 + sys->force[3 * i + d] / m;
    }
    double dt2 = dt * dt;
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double inc = sys->vel[3 * i + d] * dt + a_t[3 * i + d] * 0.5 * dt2;
            sys->pos[3 * i + d] = sys->pos[3 * i + d] + inc;
        }
    for (int64_t i = 0; i < n; ++i) or_wrap(sys, sys->pos + 3 * i);
    std::memset(sys->force, 0, sizeof(double) * 3 * (size_t)n);
    double pe = compute(sys, manager, nthreads);
    for (int64_t i = 0; i < n; ++i) {
        double m = mass_i(sys, i);
        for (int d = 0; d < 3; ++d) {
            double a_tdt = 0.0 + sys->force[3 * i + d] / m;
            sys->vel[3 * i + d] = sys->vel[3 * i + d] + (a_t[3 * i + d] + a_tdt) * 0.5 * dt;
        }
    }
    return pe;
}

// Atoms::kinetic_energy, src/atoms/properties.rs:17-24.
double or_kinetic_energy(const or_system* sys) {
    double ek = 0.0;
    for (int64_t i = 0; i < sys->n; ++i) ek += 0.5 * mass_i(sys, i) * norm_squared(sys->vel + 3 * i);
    return ek;
}

// Atoms::virial_tensor, src/atoms/properties.rs:49-51: W = positions * forces^T, i.e.
// W[a][b] = sum_i r_i[a] F_i[b] (row-major out). The reference's dynamic-size product goes
// through a blocked GEMM whose summation order is not restated; compare with a tolerance.
void or_virial_tensor(const or_system* sys, double* w) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0.0;
            for (int64_t i = 0; i < sys->n; ++i) s += sys->pos[3 * i + a] * sys->force[3 * i + b];
            w[3 * a + b] = s;
        }
}

// Atoms::pressure, src/atoms/properties.rs:61-65: (2 KE + tr W) / (3 V).
double or_pressure(const or_system* sys, double ke) {
    double w[9];
    or_virial_tensor(sys, w);
    double tr = w[0] + w[4] + w[8];
    double vol = std::fabs(or_determinant3(sys->h));
    return (2.0 * ke + tr) / (3.0 * vol);
}

// Atoms::temerature, src/atoms/properties.rs:28-30, with KB from src/constants.rs:3.
double or_temperature(const or_system* sys, double ke) {
    return (2.0 * ke) / ((double)(3 * sys->n) * 0.0083144621);
}

// Simulation::run for the NVE ensemble (src/simulation.rs:8-39, :41-64): one initial
// compute_potential on zeroed forces, then `steps` velocity-Verlet steps. pe_out[0] is the
// initial energy and pe_out[k] the energy returned by step k; ke_out[k] the kinetic energy
// after step k (ke_out[0] before the first step). Either output may be null.
void or_run_nve(or_system* sys, double dt, int64_t steps, int32_t manager, int32_t nthreads,
                double* pe_out, double* ke_out) {
    double pe0 = or_compute_potential(sys, manager, nthreads);
    if (pe_out) pe_out[0] = pe0;
    if (ke_out) ke_out[0] = or_kinetic_energy(sys);
    for (int64_t s = 1; s <= steps; ++s) {
        double pe = or_verlet_step_nve(sys, dt, manager, nthreads);
        if (pe_out) pe_out[s] = pe;
        if (ke_out) ke_out[s] = or_kinetic_energy(sys);
    }
}

// Exact-sum forms of the reductions (see or_xsum_add). Kinetic energy: the terms m_i |v_i|^2 are
// summed and the total halved (halving is exact), so the sum does not depend on whether 1/2 is
// applied per term; virial: W[a][b] = xsum_i r_i[a] F_i[b].
double or_exact_kinetic_energy(const or_system* sys) {
    or_xsum x;
    or_xsum_clear(&x);
    for (int64_t i = 0; i < sys->n; ++i) or_xsum_add(&x, mass_i(sys, i) * norm_squared(sys->vel + 3 * i));
    return 0.5 * or_xsum_value(&x);
}

void or_exact_virial_tensor(const or_system* sys, double* w) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            or_xsum x;
            or_xsum_clear(&x);
            for (int64_t i = 0; i < sys->n; ++i) or_xsum_add(&x, sys->pos[3 * i + a] * sys->force[3 * i + b]);
            w[3 * a + b] = or_xsum_value(&x);
        }
}

// compute_potential with the offset manager (forces exactly as the reference's walk leaves them)
// and the exact sum of the same pair energies; returns the walk-order sum, *pe_exact the exact one.
double or_compute_offset_exact(or_system* sys, double* pe_exact) {
    std::memset(sys->force, 0, sizeof(double) * 3 * (size_t)sys->n);
    or_xsum x;
    or_xsum_clear(&x);
    g_pe_sink = &x;
    const double pe = or_compute_offset(sys);
    g_pe_sink = nullptr;
    if (pe_exact) *pe_exact = or_xsum_value(&x);
    return pe;
}

// or_run_nve with the offset manager, reporting exact sums: pe_out[k] the exact energy of step k
// (entry 0 before the first step), ke_out[k] the exact kinetic energy after it, pe_walk_out[k]
// the reference's own walk-order energy. The trajectory is the reference's (sums do not feed
// back into an NVE step). Outputs may be null.
void or_run_nve_exact(or_system* sys, double dt, int64_t steps, double* pe_out, double* ke_out, double* pe_walk_out) {
    double pex = 0.0;
    const double pe0 = or_compute_offset_exact(sys, &pex);
    if (pe_out) pe_out[0] = pex;
    if (pe_walk_out) pe_walk_out[0] = pe0;
    if (ke_out) ke_out[0] = or_exact_kinetic_energy(sys);
    or_xsum x;
    for (int64_t s = 1; s <= steps; ++s) {
        or_xsum_clear(&x);
        g_pe_sink = &x;
        const double pe = or_verlet_step_nve(sys, dt, OR_OFFSET, 1);
        g_pe_sink = nullptr;
        if (pe_out) pe_out[s] = or_xsum_value(&x);
        if (pe_walk_out) pe_walk_out[s] = pe;
        if (ke_out) ke_out[s] = or_exact_kinetic_energy(sys);
    }
}

// Nose-Hoover chain thermostat, src/ensemble/nvt.rs, with the chain length 3 that
// NHThermostatChain::new_from_args (:99-112) builds and its literal arithmetic: q_i =
// KB T tau^2 / 10^i (:37-42), forces (:59-70), the half-step that assigns xi rather than
// integrating it (:72-80, eta is never advanced), thermostat kinetic and potential energy
// (:82-97) and the linear target-temperature ramp (:114-124).
static const double KB = 0.0083144621;  // src/constants.rs:3

struct or_nhc {
    int32_t m;
    double t_start, t_end, t_target;
    double xi[3], eta[3], g[3], q[3];
};

void or_nhc_init(or_nhc* c, double t_start, double t_end, double tau) {
    c->m = 3;
    c->t_start = t_start;
    c->t_end = t_end;
    c->t_target = t_start;
    const double q_value = KB * c->t_target * (tau * tau);
    double p = 1.0;  // 10^i by repeated multiplication (powi)
    for (int i = 0; i < 3; ++i) {
        c->xi[i] = 0.0;
        c->eta[i] = 0.0;
        c->g[i] = 0.0;
        c->q[i] = q_value / p;
        p = p * 10.0;
    }
}

void or_nhc_compute_forces(or_nhc* c, double kinetic_energy, int64_t n_atoms) {
    c->g[0] = 2.0 * kinetic_energy - ((double)(n_atoms * 3)) * KB * c->t_target;
    for (int j = 1; j < c->m; ++j) c->g[j] = c->q[j - 1] * (c->xi[j - 1] * c->xi[j - 1]) - KB * c->t_target;
}

void or_nhc_propagate_half_step(or_nhc* c, double dt) {
    const int j = c->m - 1;
    c->xi[j] = 0.5 * dt * c->g[j] / c->q[j];
    for (int l = j - 1; l >= 0; --l) c->xi[l] = (0.5 * dt * c->g[l] / c->q[l]) * std::exp(-0.25 * dt * c->xi[l + 1]);
}

double or_nhc_kinetic_energy(const or_nhc* c) {
    double e = 0.0;
    for (int i = 0; i < c->m; ++i) e += 0.5 * c->q[i] * (c->xi[i] * c->xi[i]);
    return e;
}

double or_nhc_potential_energy(const or_nhc* c, int64_t n_atoms) {
    double e = (double)(n_atoms * 3) * KB * c->t_target * c->eta[0];
    for (int i = 1; i < c->m; ++i) e += KB * c->t_target * c->eta[i];
    return e;
}

void or_nhc_target(or_nhc* c, int64_t step, int64_t steps) {
    c->t_target = c->t_start + ((c->t_end - c->t_start) / (double)steps) * (double)step;
}

// PotentialManager::verlet_step_nvt_nhc, src/potentials/potential.rs:35-58: thermostat half
// step, velocities scaled by exp(-dt xi_0 / 2), the NVE step, the same scale again, then the
// thermostat half step on the new kinetic energy.
double or_verlet_step_nvt_nhc(or_system* sys, double dt, or_nhc* c, int32_t manager, int32_t nthreads) {
    double kinetic_energy = or_kinetic_energy(sys);
    or_nhc_compute_forces(c, kinetic_energy, sys->n);
    or_nhc_propagate_half_step(c, dt);
    const double scale = std::exp(-0.5 * dt * c->xi[0]);
    for (int64_t k = 0; k < 3 * sys->n; ++k) sys->vel[k] = sys->vel[k] * scale;
    const double pe = or_verlet_step_nve(sys, dt, manager, nthreads);
    for (int64_t k = 0; k < 3 * sys->n; ++k) sys->vel[k] = sys->vel[k] * scale;
    kinetic_energy = or_kinetic_energy(sys);
    or_nhc_compute_forces(c, kinetic_energy, sys->n);
    or_nhc_propagate_half_step(c, dt);
    return pe;
}

// Simulation::run for the NVT ensemble (src/simulation.rs:8-39, :41-64, :66-88, :90-115): the
// initial compute_potential, then per step verlet_step_nvt_nhc followed by the target ramp
// (calculate_target_temperature(i, steps)), and the printed energies. pe_out[0] / ke_out[0] are
// the initial energies and ham_out[0] their sum; entry k >= 1 holds step k's potential energy,
// kinetic energy and Hamiltonian PE + KE + thermostat KE + thermostat PE. Outputs may be null;
// `c` (may be null) receives the final thermostat state.
void or_run_nvt(or_system* sys, double dt, int64_t steps, double t_start, double t_end, double tau,
                int32_t manager, int32_t nthreads, double* pe_out, double* ke_out, double* ham_out, or_nhc* c) {
    or_nhc local;
    or_nhc* nhc = c ? c : &local;
    or_nhc_init(nhc, t_start, t_end, tau);
    const double pe0 = or_compute_potential(sys, manager, nthreads);
    const double ke0 = or_kinetic_energy(sys);
    if (pe_out) pe_out[0] = pe0;
    if (ke_out) ke_out[0] = ke0;
    if (ham_out) ham_out[0] = pe0 + ke0;
    for (int64_t i = 0; i < steps; ++i) {
        const double pe = or_verlet_step_nvt_nhc(sys, dt, nhc, manager, nthreads);
        or_nhc_target(nhc, i, steps);
        const double ke = or_kinetic_energy(sys);
        if (pe_out) pe_out[i + 1] = pe;
        if (ke_out) ke_out[i + 1] = ke;
        if (ham_out) ham_out[i + 1] = pe + ke + or_nhc_kinetic_energy(nhc) + or_nhc_potential_energy(nhc, sys->n);
    }
}

// ---- NPT: the Martyna-Tobias-Klein barostat of src/ensemble/npt.rs ----------------------------
// 3x3 matrices are row-major arrays of the mathematical matrix (h: box vectors as columns).

static void m3_mul(const double* a, const double* b, double* c) {
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) t[3 * r + q] = a[3 * r] * b[q] + a[3 * r + 1] * b[3 + q] + a[3 * r + 2] * b[6 + q];
    std::memcpy(c, t, sizeof(t));
}

static void m3_symmetrize(const double* a, double* out) {  // src/math.rs symmetrize: (A + A^T) * 0.5
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) t[3 * r + q] = (a[3 * r + q] + a[3 * q + r]) * 0.5;
    std::memcpy(out, t, sizeof(t));
}

// Solve P X = Q for 3x3 X (Gaussian elimination with partial pivoting, column by column).
static void m3_solve(const double* p_in, const double* q_in, double* x) {
    double a[9], b[9];
    std::memcpy(a, p_in, sizeof(a));
    std::memcpy(b, q_in, sizeof(b));
    for (int k = 0; k < 3; ++k) {
        int piv = k;
        for (int r = k + 1; r < 3; ++r)
            if (std::fabs(a[3 * r + k]) > std::fabs(a[3 * piv + k])) piv = r;
        if (piv != k)
            for (int q = 0; q < 3; ++q) {
                std::swap(a[3 * k + q], a[3 * piv + q]);
                std::swap(b[3 * k + q], b[3 * piv + q]);
            }
        for (int r = k + 1; r < 3; ++r) {
            const double f = a[3 * r + k] / a[3 * k + k];
            for (int q = 0; q < 3; ++q) {
                a[3 * r + q] -= f * a[3 * k + q];
                b[3 * r + q] -= f * b[3 * k + q];
            }
        }
    }
    for (int q = 0; q < 3; ++q)
        for (int r = 2; r >= 0; --r) {
            double v = b[3 * r + q];
            for (int c = r + 1; c < 3; ++c) v -= a[3 * r + c] * x[3 * c + q];
            x[3 * r + q] = v / a[3 * r + r];
        }
}

// Matrix exponential (Matrix3::exp, npt.rs:55): the published scaling-and-squaring method with
// diagonal Pade approximants of degree 3, 5, 7, 9 or 13 chosen by the 1-norm (N. J. Higham,
// "The scaling and squaring method for the matrix exponential revisited", SIAM J. Matrix Anal.
// Appl. 26 (2005), Algorithm 2.3). nalgebra's own selection logic is not restated, so results
// agree with the reference to rounding, not bit for bit.
void or_expm3(const double* a_in, double* out) {
    static const double theta[4] = {1.495585217958292e-2, 2.539398330063230e-1, 9.504178996162932e-1,
                                    2.097847961257068e0};
    static const double theta13 = 5.371920351148152e0;
    static const double b3[4] = {120.0, 60.0, 12.0, 1.0};
    static const double b5[6] = {30240.0, 15120.0, 3360.0, 420.0, 30.0, 1.0};
    static const double b7[8] = {17297280.0, 8648640.0, 1995840.0, 277200.0, 25200.0, 1512.0, 56.0, 1.0};
    static const double b9[10] = {17643225600.0, 8821612800.0, 2075673600.0, 302702400.0, 30270240.0,
                                  2162160.0, 110880.0, 3960.0, 90.0, 1.0};
    static const double b13[14] = {64764752532480000.0, 32382376266240000.0, 7771770303897600.0,
                                   1187353796428800.0, 129060195264000.0, 10559470521600.0, 670442572800.0,
                                   33522128640.0, 1323241920.0, 40840800.0, 960960.0, 16380.0, 182.0, 1.0};
    static const double* bs[4] = {b3, b5, b7, b9};
    static const int ms[4] = {3, 5, 7, 9};
    double a[9];
    std::memcpy(a, a_in, sizeof(a));
    double norm1 = 0.0;
    for (int q = 0; q < 3; ++q) norm1 = std::max(norm1, std::fabs(a[q]) + std::fabs(a[3 + q]) + std::fabs(a[6 + q]));
    const double eye[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    double u[9], v[9];
    int squarings = 0;
    int pick = -1;
    for (int k = 0; k < 4; ++k)
        if (norm1 <= theta[k]) {
            pick = k;
            break;
        }
    if (pick >= 0) {
        // powers A^0, A^2, ..., A^(m-1): U = A sum_j b_{2j+1} A^{2j}, V = sum_j b_{2j} A^{2j}
        const int m = ms[pick];
        const double* b = bs[pick];
        double a2[9], pw[9], us[9] = {0}, vs[9] = {0};
        m3_mul(a, a, a2);
        std::memcpy(pw, eye, sizeof(pw));
        for (int j = 0; 2 * j <= m - 1; ++j) {
            for (int e = 0; e < 9; ++e) {
                us[e] += b[2 * j + 1] * pw[e];
                vs[e] += b[2 * j] * pw[e];
            }
            m3_mul(pw, a2, pw);
        }
        m3_mul(a, us, u);
        std::memcpy(v, vs, sizeof(v));
    } else {
        squarings = std::max(0, (int)std::ceil(std::log2(norm1 / theta13)));
        const double sc = std::ldexp(1.0, -squarings);
        for (double& x : a) x *= sc;
        const double* b = b13;
        double a2[9], a4[9], a6[9], t1[9], t2[9];
        m3_mul(a, a, a2);
        m3_mul(a2, a2, a4);
        m3_mul(a4, a2, a6);
        for (int e = 0; e < 9; ++e) t1[e] = b[13] * a6[e] + b[11] * a4[e] + b[9] * a2[e];
        m3_mul(a6, t1, t1);
        for (int e = 0; e < 9; ++e) t1[e] += b[7] * a6[e] + b[5] * a4[e] + b[3] * a2[e] + b[1] * eye[e];
        m3_mul(a, t1, u);
        for (int e = 0; e < 9; ++e) t2[e] = b[12] * a6[e] + b[10] * a4[e] + b[8] * a2[e];
        m3_mul(a6, t2, t2);
        for (int e = 0; e < 9; ++e) v[e] = t2[e] + b[6] * a6[e] + b[4] * a4[e] + b[2] * a2[e] + b[0] * eye[e];
    }
    double p[9], q[9];
    for (int e = 0; e < 9; ++e) {
        p[e] = v[e] - u[e];
        q[e] = v[e] + u[e];
    }
    m3_solve(p, q, out);
    for (int k = 0; k < squarings; ++k) m3_mul(out, out, out);
}

struct or_mtk {
    double p_target[9];
    double momentum[9];
    double w;
};

// MTKBarostat::new / new_from_args (npt.rs:23-40, :68-88): target pressure p_start * I, zero
// momentum, mass W = 3N KB T tau^2 with T the thermostat's start temperature (300 without one).
void or_mtk_init(or_mtk* b, double p_start, double tau, int64_t n_atoms, double t_target) {
    for (int e = 0; e < 9; ++e) {
        b->p_target[e] = (e % 4 == 0) ? p_start : 0.0;
        b->momentum[e] = 0.0;
    }
    b->w = ((double)(3 * n_atoms)) * KB * t_target * (tau * tau);
}

// Atoms::pressure_tensor (src/atoms/properties.rs:45-59): (V V^T + R F^T) / volume. The kinetic
// tensor carries no masses, as in the reference.
void or_pressure_tensor(const or_system* sys, double* p) {
    double k[9] = {0}, w[9];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            double sum = 0.0;
            for (int64_t i = 0; i < sys->n; ++i) sum += sys->vel[3 * i + a] * sys->vel[3 * i + c];
            k[3 * a + c] = sum;
        }
    or_virial_tensor(sys, w);
    const double vol = std::fabs(or_determinant3(sys->h));
    for (int e = 0; e < 9; ++e) p[e] = (k[e] + w[e]) / vol;
}

// delta_momentum (npt.rs:42-47): symmetrize((P - P_target) * (V * 0.5 * dt)).
void or_mtk_delta_momentum(const or_mtk* b, const or_system* sys, double dt, double* out) {
    double p[9];
    or_pressure_tensor(sys, p);
    const double f = std::fabs(or_determinant3(sys->h)) * 0.5 * dt;
    for (int e = 0; e < 9; ++e) p[e] = (p[e] - b->p_target[e]) * f;
    m3_symmetrize(p, out);
}

// scale (npt.rs:49-56): exp(symmetrize(momentum / W) * factor * dt), factor -0.5 for the
// velocities and 1 for the box.
void or_mtk_scale(const or_mtk* b, double dt, int32_t velocity_scaling, double* out) {
    double e[9];
    for (int k = 0; k < 9; ++k) e[k] = b->momentum[k] / b->w;
    m3_symmetrize(e, e);
    const double factor = velocity_scaling ? -0.5 : 1.0;
    for (int k = 0; k < 9; ++k) e[k] = e[k] * factor * dt;
    or_expm3(e, out);
}

// kinetic_energy (npt.rs:58-60): tr(M M^T) / (2 W); potential_energy (:62-64): tr(P_target^T h).
double or_mtk_kinetic_energy(const or_mtk* b) {
    double t = 0.0;
    for (int k = 0; k < 9; ++k) t += b->momentum[k] * b->momentum[k];
    return t / (2.0 * b->w);
}

double or_mtk_potential_energy(const or_mtk* b, const double* h) {
    double t = 0.0;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t += b->p_target[3 * c + r] * h[3 * c + r];
    return t;
}

// Atoms::scale_box (src/atoms/transformations.rs:6-15): fractional coordinates s = h^-1 r, then
// h = scale h, h^-1 = inverse(h), r = h s.
void or_scale_box(or_system* sys, const double* scale) {
    std::vector<double> frac((size_t)(3 * sys->n));
    for (int64_t i = 0; i < sys->n; ++i) matvec(sys->hinv, sys->pos + 3 * i, frac.data() + 3 * i);
    m3_mul(scale, sys->h, sys->h);
    or_inverse3(sys->h, sys->hinv);
    for (int64_t i = 0; i < sys->n; ++i) matvec(sys->h, frac.data() + 3 * i, sys->pos + 3 * i);
}

static void scale_velocities(or_system* sys, const double* m) {
    for (int64_t i = 0; i < sys->n; ++i) {
        double v[3];
        matvec(m, sys->vel + 3 * i, v);
        std::memcpy(sys->vel + 3 * i, v, sizeof(v));
    }
}

// PotentialManager::verlet_step_npt_mtk (src/potentials/potential.rs:115-135).
double or_verlet_step_npt_mtk(or_system* sys, double dt, or_mtk* b, or_nhc* c, int32_t manager, int32_t nthreads) {
    double d[9], scale[9], scale_h[9];
    or_mtk_delta_momentum(b, sys, dt, d);
    for (int k = 0; k < 9; ++k) b->momentum[k] += d[k];
    or_mtk_scale(b, dt, 1, scale);
    scale_velocities(sys, scale);
    or_mtk_scale(b, dt, 0, scale_h);
    or_scale_box(sys, scale_h);
    const double pe = or_verlet_step_nvt_nhc(sys, dt, c, manager, nthreads);
    scale_velocities(sys, scale);
    or_mtk_delta_momentum(b, sys, dt, d);
    for (int k = 0; k < 9; ++k) b->momentum[k] += d[k];
    return pe;
}

// Simulation::run for the NPT ensemble (src/simulation.rs:8-115): per step verlet_step_npt_mtk,
// the thermostat's target ramp, and the Hamiltonian PE + KE + thermostat KE + PE + barostat KE +
// PE. Entry 0 holds the initial energies. box_out (may be null) receives h after each step
// (9 values per entry, entry 0 the initial box).
void or_run_npt(or_system* sys, double dt, int64_t steps, double t_start, double t_end, double tau_t, double p_start,
                double tau_p, int32_t manager, int32_t nthreads, double* pe_out, double* ke_out, double* ham_out,
                double* box_out) {
    or_nhc nhc;
    or_nhc_init(&nhc, t_start, t_end, tau_t);
    or_mtk b;
    or_mtk_init(&b, p_start, tau_p, sys->n, t_start);
    const double pe0 = or_compute_potential(sys, manager, nthreads);
    const double ke0 = or_kinetic_energy(sys);
    if (pe_out) pe_out[0] = pe0;
    if (ke_out) ke_out[0] = ke0;
    if (ham_out) ham_out[0] = pe0 + ke0;
    if (box_out) std::memcpy(box_out, sys->h, sizeof(double) * 9);
    for (int64_t i = 0; i < steps; ++i) {
        const double pe = or_verlet_step_npt_mtk(sys, dt, &b, &nhc, manager, nthreads);
        or_nhc_target(&nhc, i, steps);
        const double ke = or_kinetic_energy(sys);
        if (pe_out) pe_out[i + 1] = pe;
        if (ke_out) ke_out[i + 1] = ke;
        if (ham_out)
            ham_out[i + 1] = pe + ke + or_nhc_kinetic_energy(&nhc) + or_nhc_potential_energy(&nhc, sys->n) +
                             or_mtk_kinetic_energy(&b) + or_mtk_potential_energy(&b, sys->h);
        if (box_out) std::memcpy(box_out + 9 * (i + 1), sys->h, sizeof(double) * 9);
    }
}

// FCC supercell in the order of src/bin/sapphire/main.rs:61-76 (ix, iy, iz, then basis
// (0,0,0), (0,1/2,1/2), (1/2,0,1/2), (1/2,1/2,0)); positions = h * (cell + basis), h = a I.
void or_fcc_lattice(double a, int64_t nx, int64_t ny, int64_t nz, double* pos) {
    static const double B[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}};
    double h[9] = {a, 0, 0, 0, a, 0, 0, 0, a};
    int64_t k = 0;
    for (int64_t ix = 0; ix < nx; ++ix)
        for (int64_t iy = 0; iy < ny; ++iy)
            for (int64_t iz = 0; iz < nz; ++iz)
                for (int b = 0; b < 4; ++b) {
                    double frac[3] = {(double)ix + B[b][0], (double)iy + B[b][1], (double)iz + B[b][2]};
                    matvec(h, frac, pos + 3 * k);
                    ++k;
                }
}

// Atoms::remove_drift and rescale_to_temperature, src/atoms/velocities.rs:35-59, applied to
// the given raw velocities in place.
void or_remove_drift_and_rescale(or_system* sys, double temperature) {
    double total_mass = 0.0, p[3] = {0.0, 0.0, 0.0};
    for (int64_t i = 0; i < sys->n; ++i) {
        double m = mass_i(sys, i);
        total_mass += m;
        for (int d = 0; d < 3; ++d) p[d] += sys->vel[3 * i + d] * m;
    }
    double vcm[3] = {p[0] / total_mass, p[1] / total_mass, p[2] / total_mass};
    for (int64_t i = 0; i < sys->n; ++i)
        for (int d = 0; d < 3; ++d) sys->vel[3 * i + d] -= vcm[d] * 1.0;
    double ke = or_kinetic_energy(sys);
    double t = or_temperature(sys, ke);
    double lambda = std::sqrt(temperature / t);
    for (int64_t k = 0; k < 3 * sys->n; ++k) sys->vel[k] *= lambda;
}

// The raw Gaussian draw of this project's velocity generator (SplitMix64 stream, Box-Muller pairs,
// sigma = sqrt(KB T / m); not the reference's rand SmallRng stream, which is not reproduced), so the
// CPU baseline can rebuild the benchmark's start state without loading the GPU library. Followed by
// or_remove_drift_and_rescale it gives the library's pis_maxwell_boltzmann bit for bit on one
// machine (same libm).
static uint64_t splitmix64_next(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

void or_gaussian_velocities(int64_t n, const double* m_per_atom, double temperature, uint64_t seed, double* v) {
    uint64_t state = seed * 0x2545f4914f6cdd1dull + 0x51ed27fa2cbb8d3ull;
    auto uniform = [&]() { return ((splitmix64_next(state) >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    double spare = 0.0;
    bool have = false;
    for (int64_t i = 0; i < n; ++i) {
        const double sigma = std::sqrt(KB * temperature / m_per_atom[i]);
        for (int d = 0; d < 3; ++d) {
            double z;
            if (have) {
                z = spare;
                have = false;
            } else {
                const double u1 = uniform(), u2 = uniform();
                const double r = std::sqrt(-2.0 * std::log(u1));
                z = r * std::cos(2.0 * M_PI * u2);
                spare = r * std::sin(2.0 * M_PI * u2);
                have = true;
            }
            v[3 * i + d] = sigma * z;
        }
    }
}

int32_t or_num_threads_available(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

}  // extern "C"
