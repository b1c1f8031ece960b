// noalloc.cu - force evaluation that allocates no device memory.
//
// Some callers cannot allocate device memory once they are running: a host whose framework has
// reserved the whole device for its own memory pool, or a real-time control loop in which the
// latency and implicit synchronisation of cudaMalloc / cudaFree are not allowed. For them,
// pis_gpu_compute_potential_noalloc evaluates LJ forces and energy on buffers the caller already
// owns. The scratch it needs (cell counts and starts, the atoms sorted by cell, per-block energy
// partial sums) lives in one file-scope __device__ array of fixed size, which every GPU that loads
// this library holds until the process exits.
//
// The kernels are a variant of the engine's cell binning and FP64 force evaluation: cells are
// built at the largest cutoff every call (as LJVOffsetManager does, src/potentials/
// lennard_jones.rs:186-244), every atom walks its 27 neighbour cells and sums F_i -= f over all
// j != i with the reference's FP64 pair arithmetic (src/potentials/lennard_jones.rs:33-55,
// src/simulation_box.rs:17-27), and PE is half the exact sum of the pair energies (the FP64 path's
// order-independent sum, so it equals pis_gpu_compute_potential's energy bit for bit).
// Type ids outside [1, n_types] cannot be reported by the call, which returns once the work is
// enqueued: the kernels skip every pair of such an atom (its force is zero) and write NaN as the
// energy, so the caller sees the fault in its output.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "pis_gpu.h"
#include "xsum.cuh"

using pis::XAcc;
using pis::XS_WORDS;

namespace {

constexpr int NA_MAX_ATOMS = 262144;
constexpr int NA_MAX_CELLS = 65536;
constexpr int NA_MAX_TYPES = 4;
constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = NA_MAX_ATOMS / NA_THREADS;
constexpr int NA_MAX_DEVICES = 64;

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t NA_OFF_COUNT = 0;
constexpr size_t NA_OFF_START = NA_OFF_COUNT + 4 * (size_t)NA_MAX_CELLS;
constexpr size_t NA_OFF_SLOT = NA_OFF_START + 4 * ((size_t)NA_MAX_CELLS + 64);
constexpr size_t NA_OFF_CELL = NA_OFF_SLOT + 4 * (size_t)NA_MAX_ATOMS;
constexpr size_t NA_OFF_SORTED = NA_OFF_CELL + 4 * (size_t)NA_MAX_ATOMS;
constexpr size_t NA_OFF_PE = NA_OFF_SORTED + 4 * (size_t)NA_MAX_ATOMS;
constexpr size_t NA_OFF_STATUS = NA_OFF_PE + 8 * XS_WORDS * (size_t)NA_MAX_BLOCKS;
constexpr size_t NA_SCRATCH_BYTES = NA_OFF_STATUS + 256;  // about 3.5 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

struct NaPair {
    double eps4, eps24, sigma2, rcut, ucut;
    int32_t present;
};

struct NaParams {
    int32_t n, nt;
    int32_t nc[3];
    double h[3], hinv[3];
    NaPair pair[NA_MAX_TYPES * NA_MAX_TYPES];
};

struct NaScratch {
    int32_t* count;
    int32_t* start;
    int32_t* slot;
    int32_t* cell;
    int32_t* sorted;
    long long* pe;    // per-block exact-sum partials of the pair energies (XS_WORDS words each)
    int32_t* status;  // nonzero when a type id was out of range in this call
};

__device__ __forceinline__ NaScratch na_carve(unsigned char* base) {
    NaScratch s;
    s.count = (int32_t*)(base + NA_OFF_COUNT);
    s.start = (int32_t*)(base + NA_OFF_START);
    s.slot = (int32_t*)(base + NA_OFF_SLOT);
    s.cell = (int32_t*)(base + NA_OFF_CELL);
    s.sorted = (int32_t*)(base + NA_OFF_SORTED);
    s.pe = (long long*)(base + NA_OFF_PE);
    s.status = (int32_t*)(base + NA_OFF_STATUS);
    return s;
}

__device__ __forceinline__ double na_min_image(double r, double h, double hinv) {
    double s = __dmul_rn(hinv, r);
    s = __dsub_rn(s, rint(s));
    return __dmul_rn(h, s);
}

__global__ void na_clear(unsigned char* base, int ncells) {
    NaScratch s = na_carve(base);
    if (blockIdx.x == 0 && threadIdx.x == 0) *s.status = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) s.count[c] = 0;
}

__global__ void na_bin(unsigned char* base, const NaParams P, const double* __restrict__ pos) {
    NaScratch s = na_carve(base);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        long long k = __double2ll_rd(__dmul_rn(__dmul_rn(P.hinv[d], pos[3 * i + d]), (double)P.nc[d]));
        k %= P.nc[d];
        if (k < 0) k += P.nc[d];
        c[d] = (int)k;
    }
    int lc = (c[2] * P.nc[1] + c[1]) * P.nc[0] + c[0];
    s.cell[i] = lc;
    s.slot[i] = atomicAdd(&s.count[lc], 1);
}

// One block: exclusive scan of the cell counts (then zero them for the next call).
__global__ void __launch_bounds__(1024) na_scan(unsigned char* base, int ncells) {
    NaScratch s = na_carve(base);
    __shared__ int wsum[32];
    __shared__ int tot_sh;
    int carry = 0;
    const int t = threadIdx.x, l = t & 31, w = t >> 5;
    for (int b = 0; b < ncells; b += 1024) {
        int c = b + t;
        int v = c < ncells ? s.count[c] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (l >= o) x += y;
        }
        if (l == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            int q = wsum[l], qi = q;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, qi, o);
                if (l >= o) qi += y;
            }
            wsum[l] = qi - q;
            if (l == 31) tot_sh = qi;
        }
        __syncthreads();
        if (c < ncells) {
            s.start[c] = carry + wsum[w] + x - v;
            s.count[c] = 0;
        }
        carry += tot_sh;
        __syncthreads();
    }
    if (t == 0) s.start[ncells] = carry;
}

__global__ void na_scatter(unsigned char* base, int n) {
    NaScratch s = na_carve(base);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    s.sorted[s.start[s.cell[i]] + s.slot[i]] = i;
}

__device__ __forceinline__ int na_wrap(int c, int n) {
    c += (c < 0) ? n : 0;
    return c - ((c >= n) ? n : 0);
}

__global__ void __launch_bounds__(NA_THREADS) na_force(unsigned char* base, const NaParams P,
                                                       const double* __restrict__ pos,
                                                       const int32_t* __restrict__ types, double* forces) {
    NaScratch s = na_carve(base);
    __shared__ long long shx[XS_WORDS * (NA_THREADS / 32)];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    XAcc e;
    pis::xacc_zero(e);
    if (i < P.n) {
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
        const int ti = types[i] - 1;
        const int lc = s.cell[i];
        const int cx = lc % P.nc[0], cy = (lc / P.nc[0]) % P.nc[1], cz = lc / (P.nc[0] * P.nc[1]);
        double fx = 0.0, fy = 0.0, fz = 0.0;
        bool bad = ti < 0 || ti >= P.nt;
        if (!bad)
            for (int oz = -1; oz <= 1; ++oz)
                for (int oy = -1; oy <= 1; ++oy)
                    for (int ox = -1; ox <= 1; ++ox) {
                        const int nb = (na_wrap(cz + oz, P.nc[2]) * P.nc[1] + na_wrap(cy + oy, P.nc[1])) * P.nc[0] +
                                       na_wrap(cx + ox, P.nc[0]);
                        for (int q = s.start[nb]; q < s.start[nb + 1]; ++q) {
                            const int j = s.sorted[q];
                            if (j == i) continue;
                            const int tj = types[j] - 1;
                            if (tj < 0 || tj >= P.nt) {  // flagged below; the pair is skipped
                                bad = true;
                                continue;
                            }
                            const NaPair& L = P.pair[ti * P.nt + tj];
                            if (!L.present) continue;
                            double rx = na_min_image(__dsub_rn(pos[3 * j], xi), P.h[0], P.hinv[0]);
                            double ry = na_min_image(__dsub_rn(pos[3 * j + 1], yi), P.h[1], P.hinv[1]);
                            double rz = na_min_image(__dsub_rn(pos[3 * j + 2], zi), P.h[2], P.hinv[2]);
                            double r2 =
                                __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
                            if (sqrt(r2) > L.rcut) continue;
                            double inv = __ddiv_rn(1.0, r2);
                            double s2 = __dmul_rn(L.sigma2, inv);
                            double vdw = __dmul_rn(s2, __dmul_rn(s2, s2));
                            double rep = __dmul_rn(vdw, vdw);
                            double u = __dsub_rn(__dmul_rn(L.eps4, __dsub_rn(rep, vdw)), L.ucut);
                            double c = __dmul_rn(__dmul_rn(L.eps24, __dsub_rn(__dmul_rn(2.0, rep), vdw)), inv);
                            fx = __dsub_rn(fx, __dmul_rn(c, rx));
                            fy = __dsub_rn(fy, __dmul_rn(c, ry));
                            fz = __dsub_rn(fz, __dmul_rn(c, rz));
                            pis::xacc_add(e, u);
                        }
                    }
        if (bad) atomicOr(s.status, 1);
        forces[3 * i] = fx;
        forces[3 * i + 1] = fy;
        forces[3 * i + 2] = fz;
    }
    pis::xacc_block_store<NA_THREADS>(e, s.pe + (int64_t)blockIdx.x * XS_WORDS, shx);
}

// Energy: half the exact sum of the blocks' partials (every pair appears twice); NaN when a type id
// was out of range.
__global__ void __launch_bounds__(256) na_finish(unsigned char* base, int nblocks, double* pe_out) {
    NaScratch s = na_carve(base);
    __shared__ long long shx[XS_WORDS * 8];
    __shared__ long long tot[XS_WORDS];
    XAcc a;
    pis::xacc_zero(a);
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        const long long* q = s.pe + (int64_t)b * XS_WORDS;
        for (int z = 0; z < pis::XS_LIMBS; ++z) a.l[z] += q[z];
        a.bad += q[pis::XS_LIMBS];
    }
    pis::xacc_block_store<256>(a, tot, shx);
    __syncthreads();
    if (threadIdx.x == 0) *pe_out = *s.status ? __longlong_as_double(0x7ff8000000000000ll) : 0.5 * pis::xacc_value(tot);
}

// Per-device address of the scratch array, looked up once per device with that device current.
// The address belongs to the device's primary context: it stays valid for the life of that context
// (cudaDeviceReset ends it; calls after a reset are not supported).
std::mutex g_na_mutex;
void* g_na_addr[NA_MAX_DEVICES] = {nullptr};

cudaError_t na_scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_addr[dev] = p;
    }
    *out = g_na_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" pis_status pis_gpu_compute_potential_noalloc(const pis_lj_pair* table, int32_t n_pairs, int32_t n_types,
                                                        int64_t n, const int32_t* d_type_ids, const double* d_pos,
                                                        const double* h_colmajor, double* d_forces, double* d_pe,
                                                        void* stream) {
    if (!table || n_pairs < 1) return PIS_ERR_MISSING_POTENTIAL;
    if (n_types < 1 || n_types > NA_MAX_TYPES) return PIS_ERR_INVALID_ARGUMENT;
    if (n < 1) return PIS_ERR_NO_ATOMS;
    if (n > NA_MAX_ATOMS) return PIS_ERR_INVALID_ARGUMENT;  // beyond the fixed scratch size
    if (!d_type_ids || !d_pos || !h_colmajor || !d_forces || !d_pe) return PIS_ERR_INVALID_ARGUMENT;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            if (r != c && h_colmajor[3 * c + r] != 0.0) return PIS_ERR_UNSUPPORTED;
    NaParams P;
    P.n = (int32_t)n;
    P.nt = n_types;
    for (int k = 0; k < NA_MAX_TYPES * NA_MAX_TYPES; ++k) P.pair[k] = NaPair{0, 0, 0, 0, 0, 0};
    double rc_max = 0.0;
    for (int k = 0; k < n_pairs; ++k) {
        const pis_lj_pair& p = table[k];
        if (p.ti < 1 || p.tj < 1 || p.ti > n_types || p.tj > n_types || !(p.rcut > 0.0)) return PIS_ERR_INVALID_ARGUMENT;
        NaPair q;
        q.eps4 = 4.0 * p.epsilon;
        q.eps24 = 24.0 * p.epsilon;
        q.sigma2 = p.sigma * p.sigma;
        q.rcut = p.rcut;
        q.ucut = 0.0;
        if (p.shift) {
            double t = p.sigma / p.rcut;
            double ci2 = t * t;
            double ca = ci2 * (ci2 * ci2);
            double cr = ca * ca;
            q.ucut = 4.0 * p.epsilon * (cr - ca);
        }
        q.present = 1;
        P.pair[(p.ti - 1) * n_types + (p.tj - 1)] = q;
        P.pair[(p.tj - 1) * n_types + (p.ti - 1)] = q;
        if (p.rcut > rc_max) rc_max = p.rcut;
    }
    const double hx = h_colmajor[0], hy = h_colmajor[4], hz = h_colmajor[8];
    const double m11 = hy * hz, det = hx * m11;
    P.h[0] = hx;
    P.h[1] = hy;
    P.h[2] = hz;
    P.hinv[0] = m11 / det;
    P.hinv[1] = (hx * hz) / det;
    P.hinv[2] = (hx * hy) / det;
    int64_t ncells = 1;
    const double L[3] = {hx, hy, hz};
    for (int d = 0; d < 3; ++d) {
        double q = std::floor(L[d] / rc_max);
        if (!(q >= 3.0) || !(L[d] > 2.0 * rc_max)) return PIS_ERR_BOX_TOO_SMALL;  // 27 distinct cells needed
        if (q > 4096.0) q = 4096.0;
        P.nc[d] = (int32_t)q;
        ncells *= (int64_t)q;
    }
    if (ncells > NA_MAX_CELLS) return PIS_ERR_INVALID_ARGUMENT;  // beyond the fixed scratch size
    void* base = nullptr;
    if (na_scratch_address(&base) != cudaSuccess) return PIS_ERR_CUDA;
    unsigned char* b = (unsigned char*)base;
    cudaStream_t st = (cudaStream_t)stream;
    const int nblk = (int)((n + NA_THREADS - 1) / NA_THREADS);
    // an error the caller's earlier work left pending is not this call's: it is neither reported
    // nor cleared here
    const cudaError_t pending = cudaPeekAtLastError();
    na_clear<<<64, 256, 0, st>>>(b, (int)ncells);
    na_bin<<<nblk, NA_THREADS, 0, st>>>(b, P, d_pos);
    na_scan<<<1, 1024, 0, st>>>(b, (int)ncells);
    na_scatter<<<nblk, NA_THREADS, 0, st>>>(b, (int)n);
    na_force<<<nblk, NA_THREADS, 0, st>>>(b, P, d_pos, d_type_ids, d_forces);
    na_finish<<<1, 256, 0, st>>>(b, nblk, d_pe);
    const cudaError_t now = cudaPeekAtLastError();
    if (now != cudaSuccess && now != pending) {
        if (pending == cudaSuccess) cudaGetLastError();  // this call's own launch error
        return PIS_ERR_CUDA;
    }
    return PIS_OK;
}
