// host_system.cpp - the reference's System / Simulation driver restated on the GPU manager
// (include/pis_host.h): System::read (src/system.rs:49-94) parses the command file,
// System::contextualize (:100-175) builds the velocities and the LJ table, Simulation::run
// (src/simulation.rs:8-88) steps the ensemble, prints thermo lines and writes .lammpstrj dumps
// (src/writers/dump_traj.rs:18-74). NVE and the Nose-Hoover-chain NVT (src/ensemble/nvt.rs) run;
// NPT runs on the FP64 path, whose engine supports the triclinic boxes the barostat produces.
#include <charconv>
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "host_io.h"
#include "pis_host.h"

namespace {

using pis::format_f64;
using pis::parse_f64;
using pis::parse_i32;

constexpr double KB = 0.0083144621;  // src/constants.rs:3

struct StartVelocity {
    bool present = false;
    bool start = true;
    bool has_t = false, has_seed = false;
    double t = 0.0;
    int64_t seed = 0;
};

struct NhcArgs {
    bool present = false;
    double t_start = 0, t_end = 0, tau = 0;
};

struct MtkArgs {
    bool present = false;
    double p_start = 0, tau = 0;
};

// Nose-Hoover chain of length 3 (src/ensemble/nvt.rs:4-124), literally.
struct Nhc {
    int m = 3;
    double t_start = 0, t_end = 0, t_target = 0;
    double xi[3] = {0, 0, 0}, eta[3] = {0, 0, 0}, g[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    void init(double t0, double t1, double tau) {
        t_start = t0;
        t_end = t1;
        t_target = t0;
        double qv = KB * t_target * (tau * tau);
        double p = 1.0;
        for (int i = 0; i < m; ++i) {
            q[i] = qv / p;
            p *= 10.0;
        }
    }
    void compute_forces(double ke, int64_t n) {
        g[0] = 2.0 * ke - ((double)(n * 3)) * KB * t_target;
        for (int j = 1; j < m; ++j) g[j] = q[j - 1] * (xi[j - 1] * xi[j - 1]) - KB * t_target;
    }
    void propagate_half_step(double dt) {
        int j = m - 1;
        xi[j] = 0.5 * dt * g[j] / q[j];
        for (int l = j - 1; l >= 0; --l) xi[l] = (0.5 * dt * g[l] / q[l]) * std::exp(-0.25 * dt * xi[l + 1]);
    }
    double kinetic_energy() const {
        double e = 0.0;
        for (int i = 0; i < m; ++i) e += 0.5 * q[i] * (xi[i] * xi[i]);
        return e;
    }
    double potential_energy(int64_t n) const {
        double e = (double)(n * 3) * KB * t_target * eta[0];
        for (int i = 1; i < m; ++i) e += KB * t_target * eta[i];
        return e;
    }
    void target(int64_t step, int64_t steps) {
        t_target = t_start + ((t_end - t_start) / (double)steps) * (double)step;
    }
};

// ---- 3x3 matrices (row-major) for the MTK barostat ------------------------------------------------
void m3_mul(const double* a, const double* b, double* c) {
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) c[3 * r + k] = a[3 * r] * b[k] + a[3 * r + 1] * b[3 + k] + a[3 * r + 2] * b[6 + k];
}
// math::symmetrize: (A + A^T) * 0.5
void m3_sym(const double* a, double* out) {
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t[3 * r + c] = (a[3 * r + c] + a[3 * c + r]) * 0.5;
    std::memcpy(out, t, sizeof(t));
}
// Matrix exponential by scaling and squaring of a Taylor series: A / 2^s with a 1-norm at most 1/4,
// terms until they fall below 1e-18 (at most 30), then s squarings. The barostat's arguments are
// symmetric and small (|A| ~ dt / tau_p), where this is exact to rounding.
void m3_exp(const double* a, double* out) {
    double norm = 0.0;
    for (int c = 0; c < 3; ++c) norm = std::max(norm, std::fabs(a[c]) + std::fabs(a[3 + c]) + std::fabs(a[6 + c]));
    int sq = 0;
    while (norm > 0.25 && sq < 60) {
        norm *= 0.5;
        ++sq;
    }
    const double scale = std::ldexp(1.0, -sq);
    double b[9], term[9], sum[9], tmp[9];
    for (int k = 0; k < 9; ++k) {
        b[k] = a[k] * scale;
        term[k] = (k % 4 == 0) ? 1.0 : 0.0;
        sum[k] = term[k];
    }
    for (int n = 1; n <= 30; ++n) {
        m3_mul(term, b, tmp);
        double tn = 0.0;
        for (int k = 0; k < 9; ++k) {
            term[k] = tmp[k] / n;
            sum[k] += term[k];
            tn = std::max(tn, std::fabs(term[k]));
        }
        if (tn < 1e-18) break;
    }
    for (int q = 0; q < sq; ++q) {
        m3_mul(sum, sum, tmp);
        std::memcpy(sum, tmp, sizeof(tmp));
    }
    std::memcpy(out, sum, sizeof(sum));
}

// MTKBarostat (src/ensemble/npt.rs:11-91): target pressure p_start I, momentum, mass
// W = 3 N KB T tau^2 with T the thermostat's start temperature.
struct Mtk {
    double pt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double mom[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double w = 0.0;
    void init(double p_start, double tau, int64_t n, double t_target) {
        for (int k = 0; k < 9; ++k) pt[k] = (k % 4 == 0) ? p_start : 0.0;
        w = ((double)(3 * n)) * KB * t_target * (tau * tau);
    }
    // delta_momentum (:42-47): symmetrize((P - P_target) * (V * 0.5 * dt))
    void add_delta(const double* p, double vol, double dt) {
        double d[9];
        const double f = vol * 0.5 * dt;
        for (int k = 0; k < 9; ++k) d[k] = (p[k] - pt[k]) * f;
        m3_sym(d, d);
        for (int k = 0; k < 9; ++k) mom[k] += d[k];
    }
    // scale (:49-56): exp(symmetrize(momentum / W) * factor * dt), factor -0.5 for velocities, 1 for the box
    void scale(double dt, bool velocity, double* out) const {
        double e[9];
        for (int k = 0; k < 9; ++k) e[k] = mom[k] / w;
        m3_sym(e, e);
        const double factor = velocity ? -0.5 : 1.0;
        for (int k = 0; k < 9; ++k) e[k] = e[k] * factor * dt;
        m3_exp(e, out);
    }
    // kinetic_energy (:58-60): tr(M M^T) / (2 W); potential_energy (:62-64): tr(P_target^T h)
    double kinetic_energy() const {
        double d[3];
        for (int r = 0; r < 3; ++r)
            d[r] = mom[3 * r] * mom[3 * r] + mom[3 * r + 1] * mom[3 * r + 1] + mom[3 * r + 2] * mom[3 * r + 2];
        return (d[0] + d[1] + d[2]) / (2.0 * w);
    }
    double potential_energy(const double* h) const {
        double d[3];
        for (int r = 0; r < 3; ++r) d[r] = pt[r] * h[r] + pt[3 + r] * h[3 + r] + pt[6 + r] * h[6 + r];
        return d[0] + d[1] + d[2];
    }
};

// |det h| by first-row cofactors (SimulationBox::volume, src/simulation_box.rs:67-69), row-major h
double volume3(const double* m) {
    return std::fabs(m[0] * (m[4] * m[8] - m[7] * m[5]) - m[1] * (m[3] * m[8] - m[6] * m[5]) +
                     m[2] * (m[3] * m[7] - m[6] * m[4]));
}

}  // namespace

struct pis_system {
    std::string err;
    // SimulationContext (src/readers/simulation_context.rs:105-131) and its defaults
    double timestep = 0.01;
    int64_t steps = 100;
    bool have_atoms = false;
    pis::DataFile data;
    StartVelocity sv;
    bool have_style = false;
    std::vector<std::string> style_args;
    int style_line = 0;
    std::vector<std::vector<std::string>> coeff_args;
    std::vector<int> coeff_lines;
    NhcArgs nhc;
    MtkArgs mtk;
    int64_t dump_step = 1;
    std::string dump_file = "dump.lammpstrj";
    // contextualized state
    std::vector<pis_lj_pair> table;
    int32_t n_types = 0;
    int precision = PIS_PRECISION_FP64;
    double skin = 0.3;
    pis_gpu_ctx* ctx = nullptr;
    ~pis_system() {
        if (ctx) pis_gpu_destroy(ctx);
    }
};

namespace {

pis_status sfail(pis_system* s, pis_status st, const std::string& m) {
    s->err = m;
    return st;
}

// PisError::MissingArgument / NegativeValue / InvalidArgument (src/errors.rs:26-48)
pis_status missing_argument(pis_system* s, int line) {
    return sfail(s, PIS_ERR_INVALID_ARGUMENT, "Missing argument on line " + std::to_string(line));
}
pis_status negative_value(pis_system* s, int32_t v, int line) {
    return sfail(s, PIS_ERR_INVALID_ARGUMENT,
                 "Negative value " + std::to_string(v) + " not allowed on line: " + std::to_string(line));
}
pis_status invalid_argument(pis_system* s, const std::string& t, int line) {
    return sfail(s, PIS_ERR_INVALID_ARGUMENT, "Invalid argument: " + t + " at line: " + std::to_string(line));
}

// One command line (src/readers/input_file/commands.rs:25-63, 66-144, 387-496).
pis_status run_command(pis_system* s, const std::string& cmd, const std::vector<std::string>& a, int line) {
    auto missing = [&]() { return missing_argument(s, line); };
    auto bad_f = [&](const std::string& t) { return sfail(s, PIS_ERR_PARSE, pis::float_parse_message(t)); };
    auto bad_i = [&](const std::string& t) { return sfail(s, PIS_ERR_PARSE, pis::int_parse_message(t)); };
    auto negative = [&](int32_t v) { return negative_value(s, v, line); };
    auto invalid = [&](const std::string& t) { return invalid_argument(s, t, line); };
    if (cmd == "timestep") {
        if (a.empty()) return missing();
        if (!parse_f64(a[0], s->timestep)) return bad_f(a[0]);
    } else if (cmd == "run") {
        int32_t v;
        if (a.empty()) return missing();
        if (!parse_i32(a[0], v)) return bad_i(a[0]);
        if (v < 0) return negative(v);
        s->steps = v;
    } else if (cmd == "velocity") {
        if (a.size() < 2) return missing();
        if (a[1] != "create") return invalid(a[1]);
        StartVelocity v;
        v.present = true;
        size_t k = 2;
        if (k >= a.size()) return missing();
        if (!parse_f64(a[k], v.t)) return bad_f(a[k]);
        v.has_t = true;
        ++k;
        int32_t seed;
        v.has_seed = true;
        v.seed = 0;
        if (k < a.size() && parse_i32(a[k], seed)) {
            if (seed < 0) return negative(seed);
            v.seed = seed;
            ++k;
        }
        while (k < a.size()) {
            const std::string& kw = a[k++];
            if (kw != "dist") return invalid(kw);
            if (k >= a.size()) return missing();
            const std::string& d = a[k++];
            if (d != "uniform" && d != "gaussian") return invalid(d);
        }
        s->sv = v;  // replaces whatever read_data set (commands.rs:139)
    } else if (cmd == "read_data") {
        if (a.empty()) return missing();
        std::string e;
        pis_status st = pis::read_data_file(a[0], s->data, e);
        if (st) return sfail(s, st, e);
        s->have_atoms = true;
        if (s->sv.present) {
            s->sv.start = !s->data.has_velocities;
        } else {
            s->sv = StartVelocity();
            s->sv.present = true;
            s->sv.start = !s->data.has_velocities;
        }
    } else if (cmd == "fix") {
        if (a.size() < 3) return missing();
        const std::string& style = a[2];
        size_t k = 3;
        while (k < a.size()) {
            const std::string& kw = a[k++];
            double x[3];
            if (kw != "temp" && kw != "iso") return invalid(kw);
            for (int q = 0; q < 3; ++q) {
                if (k >= a.size()) return missing();
                if (!parse_f64(a[k], x[q])) return bad_f(a[k]);
                ++k;
            }
            if (kw == "temp" && (style == "npt" || style == "nvt")) {
                s->nhc.present = true;
                s->nhc.t_start = x[0];
                s->nhc.t_end = x[1];
                s->nhc.tau = x[2];
            }
            if (kw == "iso" && style == "npt") {
                s->mtk.present = true;
                s->mtk.p_start = x[0];
                s->mtk.tau = x[2];
            }
        }
    } else if (cmd == "pair_style") {
        s->have_style = true;
        s->style_args = a;
        s->style_line = line;
        s->coeff_args.clear();
        s->coeff_lines.clear();
    } else if (cmd == "pair_coeff") {
        if (!s->have_style)
            return sfail(s, PIS_ERR_MISSING_POTENTIAL,
                         "Potential manager not initialized - missing pair_style or pair_coeff commands");
        s->coeff_args.push_back(a);
        s->coeff_lines.push_back(line);
    } else if (cmd == "dump") {
        if (a.size() < 4) return missing();
        int32_t v;
        if (!parse_i32(a[3], v)) return bad_i(a[3]);
        if (v < 0) return negative(v);
        if (a.size() < 5) return missing();
        s->dump_step = v;
        s->dump_file = a[4];
    } else {
        return sfail(s, PIS_ERR_PARSE, "Invalid command " + cmd + " found line: " + std::to_string(line));
    }
    return PIS_OK;
}

// System::contextualize (src/system.rs:100-175).
pis_status contextualize(pis_system* s) {
    if (s->have_atoms) {
        if (s->data.n == 0) return sfail(s, PIS_ERR_NO_ATOMS, "No atoms defined in input file");
        if (s->sv.present && s->sv.start) {
            const double t = s->sv.has_t ? s->sv.t : 300.0;
            const uint64_t seed = s->sv.has_seed ? (uint64_t)s->sv.seed : 0;
            std::vector<double> m(s->data.n);
            for (int64_t i = 0; i < s->data.n; ++i) {
                int32_t ty = s->data.type_ids[i];
                if (ty < 1 || ty > (int32_t)s->data.masses.size())
                    return sfail(s, PIS_ERR_INVALID_ATOM_TYPE, "Atom type " + std::to_string(ty) + " out of range");
                m[i] = s->data.masses[ty - 1];
            }
            pis::maxwell_boltzmann(s->data.n, m.data(), t, seed, s->data.vel.data());
        }
    }
    s->table = s->data.pairs;  // the data file's PairCoeffs manager (commands.rs:367-369)
    if (s->have_style) {
        // the arguments are parsed in order, each failure reported at its own line
        // (src/system.rs:120-168)
        if (s->style_args.empty()) return missing_argument(s, s->style_line);
        if (s->style_args[0] != "lj/cut")
            return sfail(s, PIS_ERR_UNKNOWN_PAIR_STYLE, "Unknown pair style: '" + s->style_args[0] + "'");
        double rc_global;
        if (s->style_args.size() < 2) return missing_argument(s, s->style_line);
        if (!parse_f64(s->style_args[1], rc_global))
            return sfail(s, PIS_ERR_PARSE, pis::float_parse_message(s->style_args[1]));
        s->table.clear();
        for (size_t r = 0; r < s->coeff_args.size(); ++r) {
            const std::vector<std::string>& c = s->coeff_args[r];
            const int line = s->coeff_lines[r];
            int32_t ij[2];
            double x[2];
            for (int q = 0; q < 2; ++q) {
                if ((size_t)q >= c.size()) return missing_argument(s, line);
                if (!parse_i32(c[q], ij[q])) return sfail(s, PIS_ERR_PARSE, pis::int_parse_message(c[q]));
                if (ij[q] < 0) return negative_value(s, ij[q], line);
            }
            for (int q = 0; q < 2; ++q) {
                if ((size_t)(q + 2) >= c.size()) return missing_argument(s, line);
                if (!parse_f64(c[q + 2], x[q])) return sfail(s, PIS_ERR_PARSE, pis::float_parse_message(c[q + 2]));
            }
            const int32_t i = ij[0], j = ij[1];
            double rc;
            if (c.size() < 5 || !parse_f64(c[4], rc)) rc = rc_global;
            // the reference keys the table by (i, j) as written and looks pairs up by (min, max):
            // a row written with i > j is never found, so it is not entered here either
            if (i > j) continue;
            pis_lj_pair p{i, j, x[0], x[1], rc, 1};
            bool replaced = false;
            for (auto& q : s->table)
                if (q.ti == i && q.tj == j) {
                    q = p;
                    replaced = true;
                }
            if (!replaced) s->table.push_back(p);
        }
    }
    // two-type PairCoeffs rows written "i j ..." with i > j are unreachable likewise
    std::vector<pis_lj_pair> t2;
    for (const auto& p : s->table)
        if (p.ti <= p.tj) t2.push_back(p);
    s->table = t2;
    s->n_types = (int32_t)s->data.masses.size();
    return PIS_OK;
}

// Atom lines [i0, i1) of a dump ("id type x y z"), appended to out.
void format_dump_lines(std::vector<char>& out, int64_t i0, int64_t i1, const int32_t* types, const double* pos) {
    out.resize((size_t)(i1 - i0) * 80 + 2048);
    size_t len = 0;
    for (int64_t i = i0; i < i1; ++i) {
        if (len + 1300 > out.size()) out.resize(out.size() * 2);  // room for a line of three maximal numbers
        char* p = out.data() + len;
        p = std::to_chars(p, p + 24, (long long)(i + 1)).ptr;
        *p++ = ' ';
        p = std::to_chars(p, p + 16, types[i]).ptr;
        for (int a = 0; a < 3; ++a) {
            *p++ = ' ';
            p += pis::format_f64_buf(pos[3 * i + a], p);
        }
        *p++ = '\n';
        len = (size_t)(p - out.data());
    }
    out.resize(len);
}

// DumpTraj::write_step (src/writers/dump_traj.rs:68-74). Large frames are formatted by up to 8
// threads, each over a contiguous range of atoms, and written in order.
void write_dump(std::ofstream& o, int64_t step, int64_t n, const int32_t* types, const double* pos, const double h[3]) {
    o << "ITEM: TIMESTEP\n" << step << "\nITEM: NUMBER OF ATOMS\n" << n << "\nITEM: BOX BOUNDS pp pp pp\n";
    for (int a = 0; a < 3; ++a) o << "0 " << format_f64(h[a]) << "\n";
    o << "ITEM: ATOMS id type x y z\n";
    const unsigned hw = std::thread::hardware_concurrency();
    const int T = n < 65536 ? 1 : (int)std::min<unsigned>(8, hw > 1 ? hw : 1);
    std::vector<std::vector<char>> parts((size_t)T);
    std::vector<std::thread> workers;
    for (int t = 1; t < T; ++t)
        workers.emplace_back([&, t] { format_dump_lines(parts[t], n * t / T, n * (t + 1) / T, types, pos); });
    format_dump_lines(parts[0], 0, n / T, types, pos);
    for (auto& w : workers) w.join();
    for (auto& q : parts) o.write(q.data(), (std::streamsize)q.size());
}

}  // namespace

extern "C" {

pis_status pis_system_open(const char* infile, int32_t precision, double skin, pis_system** out) {
    if (!infile || !out) return PIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto s = std::make_unique<pis_system>();
    s->precision = precision;
    s->skin = skin;
    errno = 0;
    std::ifstream in(infile);
    if (!in) {
        s->err = pis::open_error_message(infile, errno ? errno : ENOENT);
        *out = s.release();
        return PIS_ERR_IO;
    }
    std::string raw;
    int line = 0;
    while (std::getline(in, raw)) {
        ++line;
        std::string l = pis::trim(raw);
        if (l.empty() || l[0] == '#') continue;
        size_t h = l.find('#');
        if (h != std::string::npos) l = pis::trim(l.substr(0, h));
        std::vector<std::string> sp = pis::split_ws(l);
        if (sp.size() < 2) continue;
        std::vector<std::string> args(sp.begin() + 1, sp.end());
        pis_status st = run_command(s.get(), sp[0], args, line);
        if (st) {
            *out = s.release();
            return st;
        }
    }
    pis_status st = contextualize(s.get());
    *out = s.release();
    return st;
}

int64_t pis_system_steps(const pis_system* s) { return s ? s->steps : 0; }
double pis_system_timestep(const pis_system* s) { return s ? s->timestep : 0.0; }
int32_t pis_system_ensemble(const pis_system* s) {
    if (!s) return -1;
    if (s->nhc.present && s->mtk.present) return 2;
    return s->nhc.present ? 1 : 0;
}
const char* pis_system_last_error(const pis_system* s) { return s ? s->err.c_str() : "null system"; }
void pis_system_close(pis_system* s) { delete s; }

pis_status pis_system_state(pis_system* s, double* pos, double* vel, double* force) {
    if (!s) return PIS_ERR_INVALID_ARGUMENT;
    if (s->ctx) return pis_gpu_get_state(s->ctx, pos, vel, force);
    if (!s->have_atoms) return sfail(s, PIS_ERR_NO_ATOMS, "No atoms defined in input file");
    const size_t m = 3 * (size_t)s->data.n;
    if (pos) std::memcpy(pos, s->data.pos.data(), sizeof(double) * m);
    if (vel) std::memcpy(vel, s->data.vel.data(), sizeof(double) * m);
    if (force) std::memset(force, 0, sizeof(double) * m);
    return PIS_OK;
}

int32_t pis_system_pairs(const pis_system* s, pis_lj_pair* out, int32_t cap) {
    if (!s) return 0;
    const int32_t n = (int32_t)s->table.size();
    for (int32_t k = 0; out && k < n && k < cap; ++k) out[k] = s->table[k];
    return n;
}

pis_status pis_system_dump(const pis_system* s, int64_t* dump_step, char* file, int32_t cap) {
    if (!s) return PIS_ERR_INVALID_ARGUMENT;
    if (dump_step) *dump_step = s->dump_step;
    if (file && cap > 0) {
        const size_t k = std::min(s->dump_file.size(), (size_t)cap - 1);
        std::memcpy(file, s->dump_file.data(), k);
        file[k] = '\0';
    }
    return PIS_OK;
}

pis_status pis_system_run(pis_system* s, const char* thermo_path) {
    if (!s) return PIS_ERR_INVALID_ARGUMENT;
    // System::run takes the manager before Simulation::run asks for the atoms (src/system.rs:177-181)
    if (s->table.empty())
        return sfail(s, PIS_ERR_MISSING_POTENTIAL, "Potential manager not initialized - missing pair_style or pair_coeff commands");
    if (!s->have_atoms) return sfail(s, PIS_ERR_NO_ATOMS, "No atoms defined in input file");
    const int ens = pis_system_ensemble(s);
    if (ens == 2 && s->precision != PIS_PRECISION_FP64)
        return sfail(s, PIS_ERR_UNSUPPORTED, "NPT tilts the box: it runs on the FP64 path");
    FILE* th = thermo_path ? std::fopen(thermo_path, "w") : stdout;
    if (!th) return sfail(s, PIS_ERR_IO, "cannot open thermo output");
    std::unique_ptr<FILE, int (*)(FILE*)> th_guard(thermo_path ? th : nullptr, [](FILE* f) { return f ? std::fclose(f) : 0; });
    std::ofstream dump(s->dump_file);
    if (!dump) return sfail(s, PIS_ERR_IO, "Failed to create trajectory file '" + s->dump_file + "'");
    const pis::DataFile& d = s->data;
    const int64_t n = d.n;
    if (s->ctx) {  // a second run starts again from the input's state
        pis_gpu_destroy(s->ctx);
        s->ctx = nullptr;
    }
    pis_status st = pis_gpu_create(s->table.data(), (int32_t)s->table.size(), s->n_types, s->skin, s->precision, &s->ctx);
    if (st) return sfail(s, st, "pis_gpu_create failed");
    const double h[3] = {d.bounds[1] - d.bounds[0], d.bounds[3] - d.bounds[2], d.bounds[5] - d.bounds[4]};
    const double hc[9] = {h[0], 0, 0, 0, h[1], 0, 0, 0, h[2]};
    const uint8_t pbc[3] = {1, 1, 1};
    st = pis_gpu_set_state(s->ctx, n, d.type_ids.data(), d.masses.data(), d.pos.data(), d.vel.data(), nullptr, hc, pbc);
    if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
    const double vol = std::fabs(h[0] * (h[1] * h[2]));
    std::vector<double> pos(3 * n);
    // the step-0 dump (the input's positions) is written while the first steps run
    std::thread writer0([&dump, n, &d, h] { write_dump(dump, 0, n, d.type_ids.data(), d.pos.data(), h); });
    struct Join {
        std::thread& t;
        ~Join() {
            if (t.joinable()) t.join();
        }
    } join0{writer0};
    double pe = 0.0;
    st = pis_gpu_compute_potential(s->ctx, &pe, nullptr);
    if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
    std::fprintf(th, "%d %s\n", 0, format_f64(pe).c_str());
    Nhc nhc;
    if (ens >= 1) nhc.init(s->nhc.t_start, s->nhc.t_end, s->nhc.tau);
    Mtk mtk;
    if (ens == 2) mtk.init(s->mtk.p_start, s->mtk.tau, n, s->nhc.t_start);
    // the current box, row-major (NPT changes it every step)
    auto current_box = [&](double* hr) {
        double hcm[9];
        pis_status q = pis_gpu_get_box(s->ctx, hcm);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) hr[3 * r + c] = hcm[3 * c + r];
        return q;
    };
    // MTKBarostat::delta_momentum on the device's pressure tensor (src/ensemble/npt.rs:42-47)
    auto barostat_kick = [&](double dtk) {
        double pt[9], hr[9];
        pis_status q = pis_gpu_pressure_tensor(s->ctx, pt);
        if (!q) q = current_box(hr);
        if (!q) mtk.add_delta(pt, volume3(hr), dtk);
        return q;
    };
    const double dt = s->timestep;
    if (ens == 0) {
        // NVE: runs of up to 1000 steps (or up to the next dump) with every step's PE, KE and virial
        // trace kept on the device and read back once per run; each dump's positions are
        // downloaded at its step and written by a worker thread while the GPU runs on.
        const int64_t run_max = 1000;
        std::vector<double> pe_k(run_max), ke_k(run_max), tr_k(run_max);
        std::vector<double> dump_pos[2] = {std::vector<double>(3 * n), std::vector<double>(3 * n)};
        std::thread writer;
        int buf = 0;
        for (int64_t i = 0; i < s->steps;) {
            int64_t k = std::min(run_max, s->steps - i);
            if (s->dump_step > 0) k = std::min(k, s->dump_step - (i % s->dump_step));
            st = pis_gpu_verlet_step_nve_thermo(s->ctx, dt, k, pe_k.data(), ke_k.data(), tr_k.data());
            if (st) {
                if (writer.joinable()) writer.join();
                return sfail(s, st, pis_gpu_last_error(s->ctx));
            }
            if (s->dump_step > 0 && ((i + k) % s->dump_step) == 0) {
                if (writer0.joinable()) writer0.join();  // dumps are written in step order
                if (writer.joinable()) writer.join();  // the buffer written two dumps ago is free again
                st = pis_gpu_get_state(s->ctx, dump_pos[buf].data(), nullptr, nullptr);
                if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
                const double* pp = dump_pos[buf].data();
                const int64_t step = i + k;
                writer = std::thread([&dump, step, n, &d, pp, h] { write_dump(dump, step, n, d.type_ids.data(), pp, h); });
                buf ^= 1;
            }
            for (int64_t q = 0; q < k; ++q) {
                const double ke = ke_k[q];
                const double temp = (2.0 * ke) / ((double)(3 * n) * KB);
                const double press = (2.0 * ke + tr_k[q]) / (3.0 * vol);
                std::fprintf(th, "%lld %.3f %.3f %.3f %.3f %.3f\n", (long long)(i + q + 1), pe_k[q], ke, pe_k[q] + ke, temp,
                             press);
            }
            i += k;
        }
        if (writer0.joinable()) writer0.join();
        if (writer.joinable()) writer.join();
        std::fflush(th);
        return dump.good() ? PIS_OK : sfail(s, PIS_ERR_IO, "Failed to write trajectory file");
    }
    if (writer0.joinable()) writer0.join();  // the thermostatted loop writes its dumps in line
    for (int64_t i = 0; i < s->steps; ++i) {
        double ke = 0.0, w[9];
        double sv[9];
        if (ens == 2) {
            // verlet_step_npt_mtk (src/potentials/potential.rs:112-135): barostat half kick, velocity
            // and box scaling, the thermostatted step, velocity scaling, barostat half kick
            st = barostat_kick(dt);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
            double sh[9];
            mtk.scale(dt, true, sv);
            mtk.scale(dt, false, sh);
            st = pis_gpu_scale_velocities(s->ctx, sv);
            if (!st) st = pis_gpu_scale_box(s->ctx, sh);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
        }
        if (ens >= 1) {
            // verlet_step_nvt_nhc (src/potentials/potential.rs:35-58)
            st = pis_gpu_reductions(s->ctx, &ke, nullptr);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
            nhc.compute_forces(ke, n);
            nhc.propagate_half_step(dt);
            const double scale = std::exp(-0.5 * dt * nhc.xi[0]);
            const double m[9] = {scale, 0, 0, 0, scale, 0, 0, 0, scale};
            st = pis_gpu_scale_velocities(s->ctx, m);
            if (!st) st = pis_gpu_verlet_step_nve(s->ctx, dt, 1, &pe);
            if (!st) st = pis_gpu_scale_velocities(s->ctx, m);
            if (!st) st = pis_gpu_reductions(s->ctx, &ke, nullptr);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
            nhc.compute_forces(ke, n);
            nhc.propagate_half_step(dt);
            if (ens == 2) {
                st = pis_gpu_scale_velocities(s->ctx, sv);
                if (!st) st = barostat_kick(dt);
                if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
            }
            nhc.target(i, s->steps);
        } else {
            st = pis_gpu_verlet_step_nve(s->ctx, dt, 1, &pe);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
        }
        double hr[9];
        st = current_box(hr);
        if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
        const double hdiag[3] = {hr[0], hr[4], hr[8]};
        // Simulation::output (src/simulation.rs:66-88)
        if (s->dump_step > 0 && ((i + 1) % s->dump_step) == 0) {
            st = pis_gpu_get_state(s->ctx, pos.data(), nullptr, nullptr);
            if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
            write_dump(dump, i + 1, n, d.type_ids.data(), pos.data(), hdiag);
        }
        st = pis_gpu_reductions(s->ctx, &ke, w);
        if (st) return sfail(s, st, pis_gpu_last_error(s->ctx));
        // Simulation::compute_hamiltonian (src/simulation.rs:90-115)
        double ham = pe + ke;
        if (ens >= 1) ham = ham + nhc.kinetic_energy() + nhc.potential_energy(n);
        if (ens == 2) ham = ham + mtk.kinetic_energy() + mtk.potential_energy(hr);
        const double temp = (2.0 * ke) / ((double)(3 * n) * KB);
        const double press = (2.0 * ke + (w[0] + w[4] + w[8])) / (3.0 * (ens == 2 ? volume3(hr) : vol));
        std::fprintf(th, "%lld %.3f %.3f %.3f %.3f %.3f\n", (long long)(i + 1), pe, ke, ham, temp, press);
    }
    std::fflush(th);
    return dump.good() ? PIS_OK : sfail(s, PIS_ERR_IO, "Failed to write trajectory file");
}

}  // extern "C"
