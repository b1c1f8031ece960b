// host_io.h - shared host helpers (number parsing / formatting with the reference's rules, the
// data-file reader, the velocity generator) for the C++ host side.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "pis_gpu.h"

namespace pis {

struct DataFile {
    int64_t n = 0;
    std::vector<double> masses;
    std::vector<int32_t> type_ids;
    std::vector<double> pos, vel;
    double bounds[6] = {0.0, 1.0, 0.0, 1.0, 0.0, 1.0};  // reader defaults (commands.rs:160-162)
    bool has_velocities = false;
    std::vector<pis_lj_pair> pairs;  // insertion order, later rows replace earlier ones
    void set_pair(int i, int j, double eps, double sigma, double rc);
};

bool parse_i32(const std::string& t, int32_t& out);
bool parse_f64(const std::string& t, double& out);
// Messages of PisError::IntParseError / FloatParseError (src/errors.rs:29-41) for a token that
// parse_i32 / parse_f64 rejected, with the text Rust's ParseIntError / ParseFloatError displays.
std::string int_parse_message(const std::string& t);
std::string float_parse_message(const std::string& t);
// PisError::InputFileError (src/errors.rs:7): the path and the OS error as Rust's io::Error shows it.
std::string open_error_message(const std::string& path, int os_errno);
std::vector<std::string> split_ws(const std::string& line);
std::string trim(const std::string& s);
std::string format_f64(double v);
int format_f64_buf(double v, char* out);  // out: >= 400 chars; returns the length
pis_status read_data_file(const std::string& path, DataFile& d, std::string& err);
void maxwell_boltzmann(int64_t n, const double* m, double temperature, uint64_t seed, double* v);

}  // namespace pis
