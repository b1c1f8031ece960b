// host_io.cpp - data-file reader and writer, number parsing and formatting with the reference's
// rules, and the Maxwell-Boltzmann velocity generator (include/pis_host.h).
#include <cctype>
#include <charconv>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "host_io.h"
#include "pis_host.h"

namespace pis {

// Rust `str::parse::<i32>`: optional sign, decimal digits, in range.
bool parse_i32(const std::string& t, int32_t& out) {
    if (t.empty()) return false;
    size_t k = (t[0] == '+' || t[0] == '-') ? 1 : 0;
    if (k == t.size()) return false;
    for (size_t q = k; q < t.size(); ++q)
        if (!std::isdigit((unsigned char)t[q])) return false;
    errno = 0;
    long long v = std::strtoll(t.c_str(), nullptr, 10);
    if (errno || v < INT32_MIN || v > INT32_MAX) return false;
    out = (int32_t)v;
    return true;
}

// Rust `str::parse::<f64>`: decimal literal with optional sign, fraction and exponent, or the
// inf / infinity / nan spellings (any case); no hexadecimal.
bool parse_f64(const std::string& t, double& out) {
    if (t.empty()) return false;
    size_t k = (t[0] == '+' || t[0] == '-') ? 1 : 0;
    std::string rest = t.substr(k);
    std::string low;
    for (char c : rest) low += (char)std::tolower((unsigned char)c);
    if (low == "inf" || low == "infinity" || low == "nan") {
        out = low == "nan" ? NAN : (t[0] == '-' ? -INFINITY : INFINITY);
        return true;
    }
    size_t q = k, digits = 0;
    while (q < t.size() && std::isdigit((unsigned char)t[q])) ++q, ++digits;
    if (q < t.size() && t[q] == '.') {
        ++q;
        while (q < t.size() && std::isdigit((unsigned char)t[q])) ++q, ++digits;
    }
    if (digits == 0) return false;
    if (q < t.size() && (t[q] == 'e' || t[q] == 'E')) {
        ++q;
        if (q < t.size() && (t[q] == '+' || t[q] == '-')) ++q;
        size_t e0 = q;
        while (q < t.size() && std::isdigit((unsigned char)t[q])) ++q;
        if (q == e0) return false;
    }
    if (q != t.size()) return false;
    out = std::strtod(t.c_str(), nullptr);
    return true;
}

std::vector<std::string> split_ws(const std::string& line) {
    std::vector<std::string> out;
    std::istringstream is(line);
    std::string w;
    while (is >> w) out.push_back(w);
    return out;
}

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// Rust `{}` for f64: the shortest decimal that reads back to the same value, written without an
// exponent ("1", "0.1", "-0", "123456789000000000000", "0.000001").
// Rust's `{}` for f64: the shortest digit string that parses back to the same value (among those,
// the one nearest the value), written in positional notation without an exponent. The digits come
// from std::to_chars in scientific form without a precision (a shortest round-trip conversion);
// they are then placed around the decimal point. out holds at least 400 characters (the longest
// case is a subnormal: "0.", 323 zeros and 17 digits); returns the length written.
int format_f64_buf(double v, char* out) {
    if (std::isnan(v)) return (int)(std::memcpy(out, "NaN", 3), 3);
    if (std::isinf(v)) {
        if (v > 0) return (int)(std::memcpy(out, "inf", 3), 3);
        return (int)(std::memcpy(out, "-inf", 4), 4);
    }
    if (v == 0.0) {
        if (std::signbit(v)) return (int)(std::memcpy(out, "-0", 2), 2);
        out[0] = '0';
        return 1;
    }
    char sci[40];
    const auto r = std::to_chars(sci, sci + sizeof sci, v, std::chars_format::scientific);
    const char* p = sci;
    int len = 0;
    if (*p == '-') {
        out[len++] = '-';
        ++p;
    }
    // p = d[.ddd]e[+-]xx
    char digits[24];
    int nd = 0;
    const char* q = p;
    for (; q < r.ptr && *q != 'e'; ++q)
        if (*q != '.') digits[nd++] = *q;
    // exponent: sign and digits up to r.ptr (to_chars writes no terminator)
    int exp10 = 0;
    const bool eneg = q + 1 < r.ptr && q[1] == '-';
    for (const char* e = q + 2; e < r.ptr; ++e) exp10 = 10 * exp10 + (*e - '0');
    if (eneg) exp10 = -exp10;
    while (nd > 1 && digits[nd - 1] == '0') --nd;
    const int point = exp10 + 1;  // digits before the decimal point
    if (point <= 0) {
        out[len++] = '0';
        out[len++] = '.';
        for (int z = 0; z < -point; ++z) out[len++] = '0';
        for (int z = 0; z < nd; ++z) out[len++] = digits[z];
    } else if (point >= nd) {
        for (int z = 0; z < nd; ++z) out[len++] = digits[z];
        for (int z = nd; z < point; ++z) out[len++] = '0';
    } else {
        for (int z = 0; z < point; ++z) out[len++] = digits[z];
        out[len++] = '.';
        for (int z = point; z < nd; ++z) out[len++] = digits[z];
    }
    return len;
}

std::string format_f64(double v) {
    char buf[400];
    return std::string(buf, (size_t)format_f64_buf(v, buf));
}

std::string int_parse_message(const std::string& t) {
    // core::num::IntErrorKind for i32::from_str: an optional sign, then at least one digit; a
    // token of digits that parse_i32 rejected overflowed
    const char* why;
    if (t.empty()) {
        why = "cannot parse integer from empty string";
    } else {
        const size_t k = (t[0] == '+' || t[0] == '-') ? 1 : 0;
        bool digits = k < t.size();
        for (size_t q = k; q < t.size(); ++q)
            if (t[q] < '0' || t[q] > '9') digits = false;
        why = !digits ? "invalid digit found in string"
              : t[0] == '-' ? "number too small to fit in target type"
                            : "number too large to fit in target type";
    }
    return "Error parsing integer number from string " + t + ": " + why;
}

std::string float_parse_message(const std::string& t) {
    return "Error parsing floating number from string " + t + ": " +
           (t.empty() ? "cannot parse float from empty string" : "invalid float literal");
}

std::string open_error_message(const std::string& path, int os_errno) {
    // the reference's format string closes with a stray ')' (src/errors.rs:7)
    return "Failed to open input file '" + path + "': " + std::strerror(os_errno) + " (os error " +
           std::to_string(os_errno) + "))";
}

// run_read_data (src/readers/input_file/commands.rs:147-384).
pis_status read_data_file(const std::string& path, DataFile& d, std::string& err) {
    errno = 0;
    std::ifstream in(path);
    if (!in) {
        err = open_error_message(path, errno ? errno : ENOENT);
        return PIS_ERR_IO;
    }
    d = DataFile();
    std::string section, raw;
    int64_t n_atoms = 0;
    int line_num = -1;
    auto req = [&](const std::vector<std::string>& sp, size_t k, std::string& tok) -> pis_status {
        if (k >= sp.size()) {
            err = "Missing argument on line " + std::to_string(line_num);
            return PIS_ERR_INVALID_ARGUMENT;
        }
        tok = sp[k];
        return PIS_OK;
    };
    auto pint = [&](const std::vector<std::string>& sp, size_t k, int32_t& v) -> pis_status {
        std::string tok;
        pis_status st = req(sp, k, tok);
        if (st) return st;
        if (!parse_i32(tok, v)) {
            err = int_parse_message(tok);
            return PIS_ERR_PARSE;
        }
        return PIS_OK;
    };
    auto puint = [&](const std::vector<std::string>& sp, size_t k, int64_t& v) -> pis_status {
        int32_t x = 0;
        pis_status st = pint(sp, k, x);
        if (st) return st;
        if (x < 0) {
            err = "Negative value " + std::to_string(x) + " not allowed on line: " + std::to_string(line_num);
            return PIS_ERR_INVALID_ARGUMENT;
        }
        v = x;
        return PIS_OK;
    };
    auto pflt = [&](const std::vector<std::string>& sp, size_t k, double& v) -> pis_status {
        std::string tok;
        pis_status st = req(sp, k, tok);
        if (st) return st;
        if (!parse_f64(tok, v)) {
            err = float_parse_message(tok);
            return PIS_ERR_PARSE;
        }
        return PIS_OK;
    };
#define TRY(x)                         \
    do {                               \
        pis_status _s = (x);           \
        if (_s) return _s;             \
    } while (0)
    while (std::getline(in, raw)) {
        ++line_num;
        std::string line = trim(raw);
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> sp = split_ws(line);
        const std::string& first = sp[0];
        if (first == "Masses" || first == "Atoms" || first == "PairCoeffs") {
            section = first;
            continue;
        }
        if (first == "Velocities") {
            d.has_velocities = true;
            section = first;
            continue;
        }
        if (sp.size() > 1) {
            if (sp[1] == "atoms") {
                TRY(puint(sp, 0, n_atoms));
                d.n = n_atoms;
                d.type_ids.assign(n_atoms, 0);
                d.pos.assign(3 * n_atoms, 0.0);
                d.vel.assign(3 * n_atoms, 0.0);
                continue;
            }
            if (sp[1] == "atom") {
                int64_t nt = 0;
                TRY(puint(sp, 0, nt));
                d.masses.resize(nt, 0.0);
                continue;
            }
        }
        if (sp.size() > 2) {
            if (sp[2] == "xlo" || sp[2] == "ylo" || sp[2] == "zlo") {
                const int a = sp[2] == "xlo" ? 0 : (sp[2] == "ylo" ? 1 : 2);
                TRY(pflt(sp, 0, d.bounds[2 * a]));
                TRY(pflt(sp, 1, d.bounds[2 * a + 1]));
                continue;
            }
        }
        if (section == "Masses") {
            int64_t t = 0;
            double m = 0;
            TRY(puint(sp, 0, t));
            TRY(pflt(sp, 1, m));
            if (t < 1 || t > (int64_t)d.masses.size()) {
                err = "Atom type " + std::to_string(t) + " out of range";
                return PIS_ERR_INVALID_ATOM_TYPE;
            }
            d.masses[t - 1] = m;
        } else if (section == "PairCoeffs") {
            int64_t i = 0;
            TRY(puint(sp, 0, i));
            double eps = 0, sigma = 0, rc = 0;
            if (sp.size() > 1 && parse_f64(sp[1], eps)) {
                TRY(pflt(sp, 2, sigma));
                if (sp.size() <= 3 || !parse_f64(sp[3], rc)) rc = 2.5 * sigma;
                d.set_pair((int)i, (int)i, eps, sigma, rc);
            } else {
                int64_t j = 0;
                TRY(puint(sp, 1, j));
                TRY(pflt(sp, 2, eps));
                TRY(pflt(sp, 3, sigma));
                if (sp.size() <= 4 || !parse_f64(sp[4], rc)) rc = 2.5 * sigma;
                d.set_pair((int)i, (int)j, eps, sigma, rc);
            }
        } else if (section == "Atoms" || section == "Velocities") {
            int64_t id = 0;
            TRY(puint(sp, 0, id));
            if (id == 0 || id > n_atoms) {
                err = "Atom count mismatch: expected " + std::to_string(n_atoms) + ", found " + std::to_string(id);
                return PIS_ERR_ATOM_COUNT;
            }
            --id;
            if (section == "Atoms") {
                int64_t t = 0;
                TRY(puint(sp, 1, t));
                d.type_ids[id] = (int32_t)t;
                for (int a = 0; a < 3; ++a) TRY(pflt(sp, 2 + a, d.pos[3 * id + a]));
            } else {
                for (int a = 0; a < 3; ++a) TRY(pflt(sp, 1 + a, d.vel[3 * id + a]));
            }
        }
    }
#undef TRY
    return PIS_OK;
}

void DataFile::set_pair(int i, int j, double eps, double sigma, double rc) {
    for (auto& p : pairs)
        if (p.ti == i && p.tj == j) {
            p.epsilon = eps;
            p.sigma = sigma;
            p.rcut = rc;
            return;
        }
    pis_lj_pair p;
    p.ti = i;
    p.tj = j;
    p.epsilon = eps;
    p.sigma = sigma;
    p.rcut = rc;
    p.shift = 1;
    pairs.push_back(p);
}

uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Atoms::start_velocities (src/atoms/velocities.rs:10-59) with this library's random stream.
void maxwell_boltzmann(int64_t n, const double* m, double temperature, uint64_t seed, double* v) {
    const double KB = 0.0083144621;
    uint64_t state = seed * 0x2545f4914f6cdd1dull + 0x51ed27fa2cbb8d3ull;
    auto uniform = [&]() { return ((splitmix64(state) >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    double spare = 0.0;
    bool have = false;
    for (int64_t i = 0; i < n; ++i) {
        const double sigma = std::sqrt(KB * temperature / m[i]);
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
    // remove_drift: v -= (sum m v) / (sum m)
    double total_mass = 0.0, p[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        total_mass += m[i];
        for (int d = 0; d < 3; ++d) p[d] += v[3 * i + d] * m[i];
    }
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) v[3 * i + d] -= p[d] / total_mass;
    // rescale_to_temperature: lambda = sqrt(T / T_now), T_now = 2 KE / (3 N KB)
    double ke = 0.0;
    for (int64_t i = 0; i < n; ++i)
        ke += 0.5 * m[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    const double t_now = (2.0 * ke) / ((double)(3 * n) * KB);
    const double lambda = std::sqrt(temperature / t_now);
    for (int64_t c = 0; c < 3 * n; ++c) v[c] *= lambda;
}

}  // namespace pis

struct pis_data {
    pis::DataFile d;
};

extern "C" {

pis_status pis_data_read(const char* path, pis_data** out, char* err, int32_t errlen) {
    if (!path || !out) return PIS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto* h = new pis_data();
    std::string e;
    pis_status st = pis::read_data_file(path, h->d, e);
    if (st) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.c_str());
        delete h;
        return st;
    }
    *out = h;
    return PIS_OK;
}

int64_t pis_data_n_atoms(const pis_data* d) { return d ? d->d.n : 0; }
int32_t pis_data_n_types(const pis_data* d) { return d ? (int32_t)d->d.masses.size() : 0; }
int32_t pis_data_n_pairs(const pis_data* d) { return d ? (int32_t)d->d.pairs.size() : 0; }

pis_status pis_data_get(const pis_data* h, int32_t* type_ids, double* masses, double* pos, double* vel, double* bounds,
                        int32_t* has_velocities) {
    if (!h) return PIS_ERR_INVALID_ARGUMENT;
    const pis::DataFile& d = h->d;
    if (type_ids) std::memcpy(type_ids, d.type_ids.data(), 4 * d.type_ids.size());
    if (masses) std::memcpy(masses, d.masses.data(), 8 * d.masses.size());
    if (pos) std::memcpy(pos, d.pos.data(), 8 * d.pos.size());
    if (vel) std::memcpy(vel, d.vel.data(), 8 * d.vel.size());
    if (bounds) std::memcpy(bounds, d.bounds, sizeof(d.bounds));
    if (has_velocities) *has_velocities = d.has_velocities ? 1 : 0;
    return PIS_OK;
}

pis_status pis_data_pairs(const pis_data* h, pis_lj_pair* out) {
    if (!h || !out) return PIS_ERR_INVALID_ARGUMENT;
    std::memcpy(out, h->d.pairs.data(), sizeof(pis_lj_pair) * h->d.pairs.size());
    return PIS_OK;
}

void pis_data_free(pis_data* d) { delete d; }

pis_status pis_data_write(const char* path, int64_t n, int32_t n_types, const int32_t* type_ids, const double* masses,
                          const double* pos, const double* vel, const double* bounds, const pis_lj_pair* pairs,
                          int32_t n_pairs) {
    if (!path || n < 0 || !type_ids || !masses || !pos || !bounds) return PIS_ERR_INVALID_ARGUMENT;
    std::ofstream o(path);
    if (!o) return PIS_ERR_IO;
    using pis::format_f64;
    o << "# written by pis_gb300 (restart: Atoms + Velocities)\n\n";
    o << n << " atoms\n" << n_types << " atom types\n\n";
    const char* ax[3] = {"x", "y", "z"};
    for (int a = 0; a < 3; ++a)
        o << format_f64(bounds[2 * a]) << " " << format_f64(bounds[2 * a + 1]) << " " << ax[a] << "lo " << ax[a]
          << "hi\n";
    o << "\nMasses\n\n";
    for (int t = 0; t < n_types; ++t) o << (t + 1) << " " << format_f64(masses[t]) << "\n";
    if (pairs && n_pairs > 0) {
        // only the single-type rows read back unchanged (the reader's PairCoeffs rule)
        o << "\nPairCoeffs\n\n";
        for (int k = 0; k < n_pairs; ++k) {
            if (pairs[k].ti != pairs[k].tj) continue;
            o << pairs[k].ti << " " << format_f64(pairs[k].epsilon) << " " << format_f64(pairs[k].sigma) << " "
              << format_f64(pairs[k].rcut) << "\n";
        }
    }
    o << "\nAtoms\n\n";
    for (int64_t i = 0; i < n; ++i)
        o << (i + 1) << " " << type_ids[i] << " " << format_f64(pos[3 * i]) << " " << format_f64(pos[3 * i + 1]) << " "
          << format_f64(pos[3 * i + 2]) << "\n";
    if (vel) {
        o << "\nVelocities\n\n";
        for (int64_t i = 0; i < n; ++i)
            o << (i + 1) << " " << format_f64(vel[3 * i]) << " " << format_f64(vel[3 * i + 1]) << " "
              << format_f64(vel[3 * i + 2]) << "\n";
    }
    return o.good() ? PIS_OK : PIS_ERR_IO;
}

pis_status pis_maxwell_boltzmann(int64_t n, const double* masses_per_atom, double temperature, uint64_t seed,
                                 double* vel) {
    if (n < 1 || !masses_per_atom || !vel || !(temperature >= 0)) return PIS_ERR_INVALID_ARGUMENT;
    pis::maxwell_boltzmann(n, masses_per_atom, temperature, seed, vel);
    return PIS_OK;
}

int32_t pis_format_f64(double v, char* buf, int32_t buflen) {
    std::string s = pis::format_f64(v);
    if (buf && buflen > 0) std::snprintf(buf, (size_t)buflen, "%s", s.c_str());
    return (int32_t)s.size();
}

}  // extern "C"
