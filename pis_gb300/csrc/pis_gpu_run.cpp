// pis_gpu_run - command-line driver: `pis_gpu_run -i input.pis [--precision fp64|mixed] [--skin S]
// [--thermo FILE]`, the counterpart of the reference's `pis -i <infile>` (src/main.rs:50-62,
// src/args_parser.rs:5-10) with the GPU manager in place of the CPU one.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "pis_host.h"

int main(int argc, char** argv) {
    const char* infile = nullptr;
    const char* thermo = nullptr;
    int precision = PIS_PRECISION_FP64;
    double skin = 0.3;
    for (int k = 1; k < argc; ++k) {
        std::string a = argv[k];
        if ((a == "-i" || a == "--infile") && k + 1 < argc) {
            infile = argv[++k];
        } else if (a == "--precision" && k + 1 < argc) {
            std::string p = argv[++k];
            precision = p == "mixed" ? PIS_PRECISION_MIXED : PIS_PRECISION_FP64;
        } else if (a == "--skin" && k + 1 < argc) {
            skin = std::atof(argv[++k]);
        } else if (a == "--thermo" && k + 1 < argc) {
            thermo = argv[++k];
        } else {
            std::fprintf(stderr, "usage: %s -i <infile> [--precision fp64|mixed] [--skin S] [--thermo FILE]\n", argv[0]);
            return 2;
        }
    }
    if (!infile) {
        std::fprintf(stderr, "usage: %s -i <infile> [--precision fp64|mixed] [--skin S] [--thermo FILE]\n", argv[0]);
        return 2;
    }
    pis_system* s = nullptr;
    pis_status st = pis_system_open(infile, precision, skin, &s);
    if (st == PIS_OK) st = pis_system_run(s, thermo);
    if (st != PIS_OK) std::fprintf(stderr, "Error: %s\n", s ? pis_system_last_error(s) : "cannot open input file");
    pis_system_close(s);
    return st == PIS_OK ? 0 : 1;
}
