// engine.cu - kernels and pool management of the packed multi-system LJ MD engine.
//
// Per velocity-Verlet step every active slot goes through (one launch each, over the pool):
//   k_integrate1   a_t = F/m; x += v dt + (a_t/2) dt^2; periodic wrap; skin-displacement test;
//                  cell-relative FP32 coordinates for the mixed path
//   k_bin .. k_build  neighbour-list rebuild, each kernel a no-op for slots whose rebuild flag
//                  is clear: counting sort of atoms into cells (bin -> scan -> scatter), a
//                  per-cell id sort + gather that physically reorders the atoms by cell, then
//                  the list build at rcut + skin
//   k_force_*      LJ forces and energy (FP64 half list with atomics, FP64 full list, or mixed
//                  FP32 full list)
//   k_integrate2   v += (a_t + a_tdt)/2 dt; chunk partial sums of KE (and virial on demand)
//   k_step_end     per-slot deterministic reductions, history, counters
// Everything a step needs lives in device memory, so chunks of steps are captured as one
// CUDA graph and replayed without host round trips.
//
// Reference arithmetic (FP64 path): src/potentials/potential.rs:15-33 (NVE step),
// src/simulation_box.rs:17-42 (min-image, wrap), src/potentials/lennard_jones.rs:33-55 (pair),
// src/atoms/properties.rs:17-51 (a = F/m, KE, virial). Rounding is pinned with __d*_rn
// intrinsics so no multiply-add is fused where the reference has two roundings.
#include "engine.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

namespace cg = cooperative_groups;

namespace pis {

static std::atomic<int64_t> g_launches{0};
int64_t Engine::launches() { return g_launches.load(); }

constexpr int JBITS = 26;                  // atom-index bits of a neighbour entry
constexpr uint32_t JMASK = (1u << JBITS) - 1u;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int END_THREADS = 256;

struct Engine::DevPtrs {
    double4_32a* pos[2];
    double4_32a* vel[2];
    double4_32a* acc[2];
    int32_t* id[2];
    double4_32a* frc;
    double4_32a* posb;
    float4* prel;
    float4* prelb;
    int32_t* cellof;
    int32_t* lcell;
    int32_t* slotin;
    int32_t* perm;
    int32_t* nn;
    uint32_t* nbr;
    uint8_t* keep;
    int32_t* cell_count;
    int32_t* cell_start;
    int32_t* cell_sys;
    int32_t* blk_sys;
    int32_t* blk_first;
    SysParams* sp;
    SysState* st;
    LJDev* tab;
    double* pe_part;
    double* ke_part;
    double* vir_part;
    double* pe_hist;
    int64_t npad;
    int32_t cap;
    int32_t hist;
    int32_t max_slots;
    int32_t zero_forces;  // half list: integrate1 clears F for the atomic scatter
    int32_t full_list;
    int32_t pe_stride;    // force-kernel blocks per chunk (lanes per atom)
};
using DP = Engine::DevPtrs;

// ---------------------------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int type_of(double w) { return __double2hiint(w); }
__device__ __forceinline__ double pack_type(int t) { return __hiloint2double(t, 0); }

// One axis of SimulationBox::apply_boundary_conditions_dis for a diagonal box:
// s = hinv*r; s -= round(s); r = h*s. rint replaces round: they differ only at |s - k| = 1/2,
// i.e. |r| = L/2, which is beyond every cutoff because L > 2 (rcut + skin) is enforced.
__device__ __forceinline__ double min_image_axis(double r, double h, double hinv) {
    double s = __dmul_rn(hinv, r);
    s = __dsub_rn(s, rint(s));
    return __dmul_rn(h, s);
}
// Mixed path wrap: only a coordinate that left [0, L) moves. Tested on the bit pattern (a
// negative double has the sign bit set; non-negative doubles order like their bits), so the test
// costs no FP64 instruction.
__device__ __forceinline__ double wrap_if_out(double x, double L) {
    const long long b = __double_as_longlong(x);
    if (b < 0) return x + L;
    if (b >= __double_as_longlong(L)) return x - L;
    return x;
}
// One axis of SimulationBox::apply_boundary_conditions_pos: s = hinv*r; s -= floor(s); r = h*s.
__device__ __forceinline__ double wrap_axis(double r, double h, double hinv) {
    double s = __dmul_rn(hinv, r);
    s = __dsub_rn(s, floor(s));
    return __dmul_rn(h, s);
}
__device__ __forceinline__ double norm2_ref(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// LennardJones::compute_potential (src/potentials/lennard_jones.rs:33-55) behind the
// `|rij| > rcut => skip` test of the managers (:224-226). Returns false when skipped. The
// cutoff is decided with the reference's own sqrt comparison inside a 1e-12 band around rcut^2.
struct LJ64 {
    double eps4, eps24, sigma2, rcut, rc2_lo, rc2_hi, ucut;
};
__device__ __forceinline__ LJ64 lj64_load(const LJDev& L) {
    return LJ64{L.eps4, L.eps24, L.sigma2, L.rcut, L.rc2_lo, L.rc2_hi, L.ucut};
}
__device__ __forceinline__ bool lj_fp64(const LJ64& P, double r2, double& u, double& c) {
    if (r2 > P.rc2_hi) return false;
    if (r2 >= P.rc2_lo && sqrt(r2) > P.rcut) return false;
    double inv = __ddiv_rn(1.0, r2);
    double s2 = __dmul_rn(P.sigma2, inv);
    double vdw = __dmul_rn(s2, __dmul_rn(s2, s2));
    double rep = __dmul_rn(vdw, vdw);
    u = __dsub_rn(__dmul_rn(P.eps4, __dsub_rn(rep, vdw)), P.ucut);
    c = __dmul_rn(__dmul_rn(P.eps24, __dsub_rn(__dmul_rn(2.0, rep), vdw)), inv);
    return true;
}

// Single hardware reciprocal approximation (rcp.approx.ftz.f32); ~1 ulp, flushes denormals.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum (fixed tree). All threads must call it; result valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (l < NT / 32) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Which atom this thread owns. Returns false for padding threads; s < 0 for unused chunks.
__device__ __forceinline__ bool atom_of(const DP& P, int& s, int& i) {
    s = P.blk_sys[blockIdx.x];
    if (s < 0) return false;
    i = P.blk_first[blockIdx.x] + (int)threadIdx.x;
    const SysParams& sp = P.sp[s];
    return i < (int)(sp.a0 + sp.n);
}

// Lanes-per-atom kernels: LPA consecutive lanes (a cooperative-groups tile) share one atom and
// the grid has LPA blocks per chunk. Returns false for padding groups; s < 0 for unused chunks.
template <int LPA>
__device__ __forceinline__ bool group_atom_of(const DP& P, int& s, int& i) {
    const int chunk = blockIdx.x / LPA, sub = blockIdx.x % LPA;
    s = P.blk_sys[chunk];
    if (s < 0) return false;
    i = P.blk_first[chunk] + sub * (256 / LPA) + (int)(threadIdx.x / LPA);
    const SysParams& sp = P.sp[s];
    return i < (int)(sp.a0 + sp.n);
}

// Neighbour-list layout: entry k of atom i lives at (k / LPA) * (npad * LPA) + i * LPA + k % LPA.
// The LPA lanes of one atom read or write one contiguous run of LPA words, and consecutive atoms'
// runs are adjacent, so a warp touches whole 128-byte lines. LPA = 1 is plain column-major.
template <int LPA>
__device__ __forceinline__ int64_t nbr_index(int i, int k, int64_t npad) {
    return (int64_t)(k / LPA) * (npad * LPA) + (int64_t)i * LPA + (k % LPA);
}

// Step mode (nonzero): slots with steps left take part. Evaluation mode (0): only slots the host
// marked for a force evaluation or reduction.
__device__ __forceinline__ bool slot_runs(const DP& P, int s, int step_mode) {
    return step_mode ? P.st[s].steps_left > 0 : P.st[s].eval != 0;
}

__device__ __forceinline__ float4 cell_relative(const SysParams& sp, double4_32a p, int lc, int type) {
    int cx = lc % sp.nc[0];
    int cy = (lc / sp.nc[0]) % sp.nc[1];
    int cz = lc / (sp.nc[0] * sp.nc[1]);
    double dx = p.x - (cx + 0.5) * sp.cs[0];
    double dy = p.y - (cy + 0.5) * sp.cs[1];
    double dz = p.z - (cz + 0.5) * sp.cs[2];
    dx -= sp.h[0] * rint(dx * sp.hinv[0]);
    dy -= sp.h[1] * rint(dy * sp.hinv[1]);
    dz -= sp.h[2] * rint(dz * sp.hinv[2]);
    return make_float4((float)dx, (float)dy, (float)dz, __int_as_float(type));
}

// ---------------------------------------------------------------------------------------------
// step kernels
// ---------------------------------------------------------------------------------------------
// First half of PotentialManager::verlet_step_nve (src/potentials/potential.rs:16-24).
// a_t = F/m is not recomputed: acc holds it from the last force evaluation (same bits, one
// FP64 division fewer per component - the FP64 pipe is the scarce unit on GB300).
// EXACT (FP64 path): the reference's rounding sequence and wrap of every atom every step.
// Mixed path: FP64 with fused multiply-adds, and only atoms that left the box are wrapped.
template <bool MIXED>
__global__ void k_integrate1(const DP P) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!slot_runs(P, s, true)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    const int cur = st.cur;
    const double4_32a p = P.pos[cur][i];
    const double4_32a v = P.vel[cur][i];
    const double4_32a a = P.acc[cur][i];
    double x, y, z;
    if (!MIXED) {
        // positions += v*dt + (a*0.5)*dt^2, then s = h^-1 x; s -= floor(s); x = h s
        x = __dadd_rn(p.x, __dadd_rn(__dmul_rn(v.x, sp.dt), __dmul_rn(__dmul_rn(a.x, 0.5), sp.dt2)));
        y = __dadd_rn(p.y, __dadd_rn(__dmul_rn(v.y, sp.dt), __dmul_rn(__dmul_rn(a.y, 0.5), sp.dt2)));
        z = __dadd_rn(p.z, __dadd_rn(__dmul_rn(v.z, sp.dt), __dmul_rn(__dmul_rn(a.z, 0.5), sp.dt2)));
        x = wrap_axis(x, sp.h[0], sp.hinv[0]);
        y = wrap_axis(y, sp.h[1], sp.hinv[1]);
        z = wrap_axis(z, sp.h[2], sp.hinv[2]);
    } else {
        const double hdt2 = 0.5 * sp.dt2;
        x = p.x + fma(v.x, sp.dt, a.x * hdt2);
        y = p.y + fma(v.y, sp.dt, a.y * hdt2);
        z = p.z + fma(v.z, sp.dt, a.z * hdt2);
        x = wrap_if_out(x, sp.h[0]);
        y = wrap_if_out(y, sp.h[1]);
        z = wrap_if_out(z, sp.h[2]);
    }
    P.pos[cur][i] = make_double4_32a(x, y, z, p.w);
    if (P.zero_forces) P.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    // skin test: rebuild when any atom moved more than skin/2 since the last build. The
    // minimum image is only taken when the plain difference fails the test (moved far, or
    // crossed the periodic boundary).
    const double4_32a b = P.posb[i];
    double dx = x - b.x, dy = y - b.y, dz = z - b.z;
    double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
    // d2 >= 0, so comparing bit patterns as integers orders it like the doubles (a NaN with
    // either sign fails the test too: its magnitude bits exceed every finite value's)
    if ((__double_as_longlong(d2) & 0x7fffffffffffffffll) > __double_as_longlong(sp.half_skin2)) {
        dx = min_image_axis(dx, sp.h[0], sp.hinv[0]);
        dy = min_image_axis(dy, sp.h[1], sp.hinv[1]);
        dz = min_image_axis(dz, sp.h[2], sp.hinv[2]);
        d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        if (!(d2 <= sp.half_skin2)) st.rebuild = 1;  // NaN also requests a rebuild
        if (x != x || y != y || z != z) atomicOr(&st.flags, FLAG_NAN);
    }
    if (MIXED) {
        // cell-relative FP32 coordinates = build-time ones + displacement since the build
        const float4 q = P.prelb[i];
        P.prel[i] = make_float4(q.x + (float)dx, q.y + (float)dy, q.z + (float)dz, q.w);
    }
}

// Counting sort, pass 1: cell of every atom (reference binning of src/atoms/neighbour_list.rs:
// 9-42 at rcut + skin, with a Euclidean modulo so atoms outside the box fold back in) and its
// slot inside the cell.
__global__ void k_bin(const DP P, int respect_steps) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!slot_runs(P, s, respect_steps)) return;
    const SysParams& sp = P.sp[s];
    const SysState& st = P.st[s];
    if (!st.rebuild) return;
    double4_32a p = P.pos[st.cur][i];
    int c[3];
    double q[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        // floor and conversion in one saturating instruction
        long long k = __double2ll_rd(__dmul_rn(__dmul_rn(sp.hinv[d], q[d]), (double)sp.nc[d]));
        k %= sp.nc[d];
        if (k < 0) k += sp.nc[d];
        c[d] = (int)k;
    }
    int lc = (c[2] * sp.nc[1] + c[1]) * sp.nc[0] + c[0];
    P.lcell[i] = lc;
    P.slotin[i] = atomicAdd(&P.cell_count[sp.c0 + lc], 1);
}

// Counting sort, pass 2: exclusive scan of the cell counts of one slot (one block per slot),
// writing absolute atom indices; also flips the slot's buffer set. Counts are staged through
// shared memory so global loads and stores stay coalesced while each thread scans SCAN_ITEMS
// consecutive cells.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan(const DP P, int step_mode) {
    int s = blockIdx.x;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    if (!slot_runs(P, s, step_mode)) return;
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    __shared__ int buf[SCAN_THREADS * SCAN_ITEMS];
    __shared__ int warp_tot[SCAN_THREADS / 32];
    __shared__ int carry_sh;
    const int ncell = sp.nc[0] * sp.nc[1] * sp.nc[2];
    int32_t* __restrict__ cnt_g = P.cell_count + sp.c0;
    int32_t* __restrict__ start_g = P.cell_start + sp.c0;
    int carry = (int)sp.a0;
    const int t = threadIdx.x, l = t & 31, w = t >> 5;
    for (int base = 0; base < ncell; base += SCAN_THREADS * SCAN_ITEMS) {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const int c = base + k * SCAN_THREADS + t;
            int v = 0;
            if (c < ncell) {
                v = cnt_g[c];
                cnt_g[c] = 0;
            }
            buf[k * SCAN_THREADS + t] = v;
        }
        __syncthreads();
        int v[SCAN_ITEMS], sum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = buf[t * SCAN_ITEMS + k];
            sum += v[k];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (l >= o) incl += y;
        }
        if (l == 31) warp_tot[w] = incl;
        __syncthreads();
        if (w == 0) {
            int x = warp_tot[l];
            int xi = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, xi, o);
                if (l >= o) xi += y;
            }
            warp_tot[l] = xi - x;  // exclusive warp offsets
            if (l == 31) carry_sh = xi;
        }
        __syncthreads();
        int run = carry + warp_tot[w] + incl - sum;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            buf[t * SCAN_ITEMS + k] = run;
            run += v[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const int c = base + k * SCAN_THREADS + t;
            if (c < ncell) start_g[c] = buf[k * SCAN_THREADS + t];
        }
        carry += carry_sh;
        __syncthreads();
    }
    if (t == 0) {
        start_g[ncell] = carry;
        st.cur ^= 1;
    }
}

// Counting sort, pass 3: destination of every atom.
__global__ void k_scatter(const DP P, int respect_steps) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!slot_runs(P, s, respect_steps)) return;
    if (!P.st[s].rebuild) return;
    const SysParams& sp = P.sp[s];
    int dst = P.cell_start[sp.c0 + P.lcell[i]] + P.slotin[i];
    P.perm[dst] = i;
}

// One warp per cell: order the cell's atoms by original id (so the layout depends only on the
// physical state, not on atomics), then move every per-atom array into the new buffer set and
// record the build snapshot and cell-relative coordinates.
__global__ void k_gather(const DP P, int64_t max_cells, int respect_steps) {
    int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (g >= max_cells) return;
    int s = P.cell_sys[g];
    if (s < 0) return;
    if (!slot_runs(P, s, respect_steps)) return;
    const SysParams& sp = P.sp[s];
    const SysState& st = P.st[s];
    if (!st.rebuild) return;
    int lc = (int)(g - sp.c0);
    if (lc >= sp.nc[0] * sp.nc[1] * sp.nc[2]) return;  // sentinel entry
    const int dst_set = st.cur, src_set = st.cur ^ 1;
    const int beg = P.cell_start[g], end = P.cell_start[g + 1];
    const int cnt = end - beg;
    // rank of every member by original id: ids held in lane registers for cells of up to 64
    // atoms (one or two per lane), compared through warp shuffles; larger cells re-read ids
    int rk[2] = {0, 0}, srcs[2] = {-1, -1}, ids[2] = {0x7fffffff, 0x7fffffff};
    if (cnt <= 64) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = lane + 32 * h;
            if (k < cnt) {
                srcs[h] = P.perm[beg + k];
                ids[h] = P.id[src_set][srcs[h]];
            }
        }
        const int n0 = cnt < 32 ? cnt : 32;
        for (int q = 0; q < n0; ++q) {
            const int v = __shfl_sync(0xffffffffu, ids[0], q);
            rk[0] += v < ids[0];
            rk[1] += v < ids[1];
        }
        for (int q = 32; q < cnt; ++q) {
            const int v = __shfl_sync(0xffffffffu, ids[1], q - 32);
            rk[0] += v < ids[0];
            rk[1] += v < ids[1];
        }
    }
    for (int k = lane; k < cnt; k += 32) {
        int src, myid, rank = 0;
        if (cnt <= 64) {
            const bool hi = k >= 32;
            src = hi ? srcs[1] : srcs[0];
            myid = hi ? ids[1] : ids[0];
            rank = hi ? rk[1] : rk[0];
        } else {
            src = P.perm[beg + k];
            myid = P.id[src_set][src];
            for (int q = 0; q < cnt; ++q) rank += P.id[src_set][P.perm[beg + q]] < myid;
        }
        int dst = beg + rank;
        double4_32a p = P.pos[src_set][src];
        P.pos[dst_set][dst] = p;
        P.vel[dst_set][dst] = P.vel[src_set][src];
        P.acc[dst_set][dst] = P.acc[src_set][src];
        P.id[dst_set][dst] = myid;
        P.posb[dst] = p;
        P.cellof[dst] = lc;
        const float4 q = cell_relative(sp, p, lc, type_of(p.w));
        P.prel[dst] = q;
        P.prelb[dst] = q;
    }
}

// Neighbour-list build at rcut + skin. LPA lanes share one home atom (atoms in cell order, so
// neighbouring groups walk the same cells) and split each neighbour cell's atoms among
// themselves; the accepted pairs are compacted with a ballot over the group and a prefix
// popcount, so each group writes its new entries as one contiguous run of the list layout. The
// distance test runs in FP32 on cell-relative coordinates with a radius padded by 1e-5, so the
// list is a superset of the exact FP64 list; the force kernels apply the exact cutoff.
// Entry = j | image code << 26, the code giving the cell offset (0, +1, -1 per axis, 2 bits each)
// that makes prel_j - prel_i + offset * cell the minimum-image displacement at build time. Axes
// with only two cells reach the same neighbour cell through +1 and -1; the generic path keeps, per
// pair, whichever image is nearer.
__device__ __forceinline__ int wrapc(int c, int n) {
    c += (c < 0) ? n : 0;
    return c - ((c >= n) ? n : 0);
}

template <bool HALF, int LPA>
__device__ __forceinline__ void k_build_body(const DP& P, int step_mode) {
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of<LPA>(P, s, i);
    if (s < 0 || !live) return;  // uniform over the group (one atom per group)
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    const int gl = (int)tile.thread_rank();
    const uint32_t below = (1u << gl) - 1u;
    const int nx = sp.nc[0], ny = sp.nc[1], nz = sp.nc[2];
    const int lc = P.cellof[i];
    const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
    const float4 pi = P.prel[i];
    const float csx = sp.fcs[0], csy = sp.fcs[1], csz = sp.fcs[2];
    const float rl2 = sp.frlist2;
    const int64_t npad = P.npad;
    const int cap = P.cap;
    const int32_t* __restrict__ cstart = P.cell_start + sp.c0;
    const float4* __restrict__ prel = P.prel;
    int cnt = 0;
    const bool generic = nx < 3 || ny < 3 || nz < 3;
    const int zlo = nz >= 3 ? -1 : 0, ylo = ny >= 3 ? -1 : 0, xlo = nx >= 3 ? -1 : 0;
    // squared distance from the atom to the face of a neighbouring cell along one axis (the
    // atom sits at pi relative to its own cell centre); the padding keeps the test conservative
    const float gxm = fmaxf(pi.x + 0.5f * csx, 0.f), gxp = fmaxf(0.5f * csx - pi.x, 0.f);
    const float gym = fmaxf(pi.y + 0.5f * csy, 0.f), gyp = fmaxf(0.5f * csy - pi.y, 0.f);
    const float gzm = fmaxf(pi.z + 0.5f * csz, 0.f), gzp = fmaxf(0.5f * csz - pi.z, 0.f);
    auto append = [&](bool take, int j, uint32_t code) {
        if (LPA == 1) {
            if (take) {
                if (cnt < cap) P.nbr[nbr_index<1>(i, cnt, npad)] = (uint32_t)j | (code << JBITS);
                ++cnt;
            }
        } else {
            const uint32_t m = tile.ballot(take);
            if (take) {
                const int pos = cnt + __popc(m & below);
                if (pos < cap) P.nbr[nbr_index<LPA>(i, pos, npad)] = (uint32_t)j | (code << JBITS);
            }
            cnt += __popc(m);
        }
    };
    for (int oz = zlo; oz <= 1; ++oz) {
        const int z2 = wrapc(cz + oz, nz);
        for (int oy = ylo; oy <= 1; ++oy) {
            const int y2 = wrapc(cy + oy, ny);
            for (int ox = xlo; ox <= 1; ++ox) {
                const int x2 = wrapc(cx + ox, nx);
                const int nb = (z2 * ny + y2) * nx + x2;
                const int b0 = cstart[nb], b1 = cstart[nb + 1];
                const uint32_t cell_code = ((uint32_t)(ox < 0 ? 2 : ox)) | ((uint32_t)(oy < 0 ? 2 : oy) << 2) |
                                           ((uint32_t)(oz < 0 ? 2 : oz) << 4);
                if (!generic) {
                    // skip the whole cell when its nearest point is beyond the list radius
                    const float ex = ox < 0 ? gxm : (ox > 0 ? gxp : 0.f);
                    const float ey = oy < 0 ? gym : (oy > 0 ? gyp : 0.f);
                    const float ez = oz < 0 ? gzm : (oz > 0 ? gzp : 0.f);
                    if (LPA == 1 && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > rl2) continue;
                    const float sx = ox * csx - pi.x, sy = oy * csy - pi.y, sz = oz * csz - pi.z;
                    for (int j0 = b0; j0 < b1; j0 += LPA) {
                        const int j = j0 + gl;
                        bool take = false;
                        if (j < b1 && (HALF ? (j > i) : (j != i))) {
                            const float4 pj = prel[j];
                            const float dx = pj.x + sx, dy = pj.y + sy, dz = pj.z + sz;
                            take = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rl2;
                        }
                        append(take, j, cell_code);
                    }
                } else {
                    for (int j0 = b0; j0 < b1; j0 += LPA) {
                        const int j = j0 + gl;
                        bool take = false;
                        uint32_t code = 0;
                        if (j < b1 && (HALF ? (j > i) : (j != i))) {
                            const float4 pj = prel[j];
                            float d[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
                            const int o[3] = {ox, oy, oz}, n[3] = {nx, ny, nz};
                            const float c3[3] = {csx, csy, csz};
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
                                if (o[a] == 0) continue;
                                const float up = d[a] + c3[a], dn = d[a] - c3[a];
                                const bool usep = (n[a] == 2) ? (fabsf(up) <= fabsf(dn)) : (o[a] > 0);
                                d[a] = usep ? up : dn;
                                code |= (usep ? 1u : 2u) << (2 * a);
                            }
                            take = fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2])) <= rl2;
                        }
                        append(take, j, code);
                    }
                }
            }
        }
    }
    if (gl == 0) {
        if (cnt > cap) atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
        P.nn[i] = cnt > cap ? cap : cnt;
    }
}

template <bool HALF, int LPA>
__global__ void __launch_bounds__(256) k_build(const DP P, int step_mode) {
    k_build_body<HALF, LPA>(P, step_mode);
}

// Thread-per-atom list build (the default shape). Same contents and order as k_build<HALF, 1>;
// the inner loop is kept minimal: the home cell (the only one holding i) is walked separately,
// the capacity test is hoisted to once per neighbour cell when the cell cannot overflow the row,
// and cells whose nearest face is beyond the list radius for this atom are skipped.
template <bool HALF>
__device__ __forceinline__ void scan_cell(const float4* __restrict__ pp, int j, int jend, float sx, float sy,
                                          float sz, float rl2, uint32_t codebits, int i, bool home,
                                          uint32_t*& out, int& cnt, int64_t npad, int cap) {
    const bool roomy = cnt + (jend - j) <= cap;
    for (; j < jend; ++j, ++pp) {
        const float4 pj = *pp;
        const float dx = pj.x + sx, dy = pj.y + sy, dz = pj.z + sz;
        bool take = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rl2;
        if (HALF)
            take = take && j > i;
        else if (home)
            take = take && j != i;
        if (take) {
            if (roomy || cnt < cap) *out = (uint32_t)j | codebits;
            out += npad;
            ++cnt;
        }
    }
}

template <bool HALF>
__global__ void __launch_bounds__(256) k_build1(const DP P, int step_mode) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    const int nx = sp.nc[0], ny = sp.nc[1], nz = sp.nc[2];
    if (nx < 3 || ny < 3 || nz < 3) return;  // two-cell axes: the generic kernel handles the slot
    const int lc = P.cellof[i];
    const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
    const float4 pi = P.prel[i];
    const float csx = sp.fcs[0], csy = sp.fcs[1], csz = sp.fcs[2];
    const float rl2 = sp.frlist2;
    const int64_t npad = P.npad;
    const int cap = P.cap;
    const int32_t* __restrict__ cstart = P.cell_start + sp.c0;
    const float4* __restrict__ prel = P.prel;
    uint32_t* out = P.nbr + i;
    int cnt = 0;
    const float gxm = fmaxf(pi.x + 0.5f * csx, 0.f), gxp = fmaxf(0.5f * csx - pi.x, 0.f);
    const float gym = fmaxf(pi.y + 0.5f * csy, 0.f), gyp = fmaxf(0.5f * csy - pi.y, 0.f);
    const float gzm = fmaxf(pi.z + 0.5f * csz, 0.f), gzp = fmaxf(0.5f * csz - pi.z, 0.f);
    for (int oz = -1; oz <= 1; ++oz) {
        const int z2 = wrapc(cz + oz, nz);
        const float ez = oz < 0 ? gzm : (oz > 0 ? gzp : 0.f);
        for (int oy = -1; oy <= 1; ++oy) {
            const int y2 = wrapc(cy + oy, ny);
            const float ey = oy < 0 ? gym : (oy > 0 ? gyp : 0.f);
            const float eyz = fmaf(ey, ey, ez * ez);
            for (int ox = -1; ox <= 1; ++ox) {
                const float ex = ox < 0 ? gxm : (ox > 0 ? gxp : 0.f);
                if (fmaf(ex, ex, eyz) > rl2) continue;
                const int x2 = wrapc(cx + ox, nx);
                const int nb = (z2 * ny + y2) * nx + x2;
                const int b0 = cstart[nb], b1 = cstart[nb + 1];
                const uint32_t codebits = (((uint32_t)(ox < 0 ? 2 : ox)) | ((uint32_t)(oy < 0 ? 2 : oy) << 2) |
                                           ((uint32_t)(oz < 0 ? 2 : oz) << 4))
                                          << JBITS;
                const bool home = ox == 0 && oy == 0 && oz == 0;
                scan_cell<HALF>(prel + b0, b0, b1, ox * csx - pi.x, oy * csy - pi.y, oz * csz - pi.z, rl2, codebits,
                                i, home, out, cnt, npad, cap);
            }
        }
    }
    if (cnt > cap) atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
    P.nn[i] = cnt > cap ? cap : cnt;
}

// Slots with a two-cell axis: the group kernel's generic path, one lane per atom.
template <bool HALF>
__global__ void __launch_bounds__(256) k_build1_generic(const DP P, int step_mode) {
    int s = P.blk_sys[blockIdx.x];
    if (s < 0) return;
    const SysParams& sp = P.sp[s];
    if (sp.nc[0] >= 3 && sp.nc[1] >= 3 && sp.nc[2] >= 3) return;
    k_build_body<HALF, 1>(P, step_mode);
}

// FP64 forces: the pair evaluation of LJVOffsetManager (src/potentials/lennard_jones.rs:214-235),
// F_i -= f, F_j += f, PE += u. LPA lanes share one atom, stride through its list, and reduce
// their partial forces with tile shuffles.
//   FULL = false: Newton-3 half list, j's share scattered with FP64 atomics (forces zeroed by
//     integrate-1).
//   FULL = true: full list, F_i only, no atomics; PE halved at the reduction.
//   FAST = false: the reference's rounding sequence operation for operation (min-image through
//     h^-1 and h, x*x+y*y+z*z, true division).
//   FAST = true: fused multiply-adds, min-image as r - L*rint(r/L), and 1/r^2 by Newton-Raphson
//     (y <- y + y(1 - r^2 y), twice) from the hardware approximation rcp.approx.f64. Pairs within
//     a 1e-12 band of rcut are re-tested with the exact reference arithmetic, so the set of
//     interacting pairs is identical to the reference's.
__device__ __forceinline__ double rcp_newton(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

template <bool FULL, bool FAST, int LPA>
__global__ void __launch_bounds__(256) k_force_fp64(const DP P, int respect_steps) {
    __shared__ double sh[32];
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of<LPA>(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, respect_steps)) return;  // uniform per block (one slot per chunk)
    const int gl = (int)tile.thread_rank();
    double e = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
    if (live) {
        const SysParams& sp = P.sp[s];
        const int cur = P.st[s].cur;
        const double4_32a* __restrict__ pos = P.pos[cur];
        const double4_32a pi = pos[i];
        const int ti = type_of(pi.w);
        const LJDev* tab = P.tab + sp.tab0 + ti * sp.nt;
        const bool one_type = sp.nt == 1;
        const LJ64 P0 = lj64_load(tab[0]);
        const double hx = sp.h[0], hy = sp.h[1], hz = sp.h[2];
        const double ix = sp.hinv[0], iy = sp.hinv[1], iz = sp.hinv[2];
        const int nn = P.nn[i];
        const int64_t npad = P.npad;
        for (int k = gl; k < nn; k += LPA) {
            const int j = (int)(P.nbr[nbr_index<LPA>(i, k, npad)] & JMASK);
            const double4_32a pj = pos[j];
            LJ64 L = P0;
            if (!one_type) {
                const LJDev& T = tab[type_of(pj.w)];
                if (!T.present) continue;
                L = lj64_load(T);
            }
            double rx, ry, rz, u, c;
            if (!FAST) {
                rx = min_image_axis(__dsub_rn(pj.x, pi.x), hx, ix);
                ry = min_image_axis(__dsub_rn(pj.y, pi.y), hy, iy);
                rz = min_image_axis(__dsub_rn(pj.z, pi.z), hz, iz);
                if (!lj_fp64(L, norm2_ref(rx, ry, rz), u, c)) continue;
            } else {
                rx = pj.x - pi.x;
                ry = pj.y - pi.y;
                rz = pj.z - pi.z;
                rx = fma(-hx, rint(rx * ix), rx);
                ry = fma(-hy, rint(ry * iy), ry);
                rz = fma(-hz, rint(rz * iz), rz);
                const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
                if (r2 > L.rc2_hi) continue;
                if (r2 >= L.rc2_lo) {
                    double qx = min_image_axis(__dsub_rn(pj.x, pi.x), hx, ix);
                    double qy = min_image_axis(__dsub_rn(pj.y, pi.y), hy, iy);
                    double qz = min_image_axis(__dsub_rn(pj.z, pi.z), hz, iz);
                    if (sqrt(norm2_ref(qx, qy, qz)) > L.rcut) continue;
                }
                const double inv = rcp_newton(r2);
                const double s2 = L.sigma2 * inv;
                const double vdw = s2 * s2 * s2;
                const double rep = vdw * vdw;
                u = fma(L.eps4, rep - vdw, -L.ucut);
                c = L.eps24 * fma(2.0, rep, -vdw) * inv;
            }
            double gx, gy, gz;
            if (!FAST) {
                gx = __dmul_rn(c, rx);
                gy = __dmul_rn(c, ry);
                gz = __dmul_rn(c, rz);
                fx = __dsub_rn(fx, gx);
                fy = __dsub_rn(fy, gy);
                fz = __dsub_rn(fz, gz);
                e = __dadd_rn(e, u);
            } else {
                gx = c * rx;
                gy = c * ry;
                gz = c * rz;
                fx -= gx;
                fy -= gy;
                fz -= gz;
                e += u;
            }
            if (!FULL) {
                atomicAdd(&P.frc[j].x, gx);
                atomicAdd(&P.frc[j].y, gy);
                atomicAdd(&P.frc[j].z, gz);
            }
        }
    }
#pragma unroll
    for (int o = LPA / 2; o > 0; o >>= 1) {
        fx += tile.shfl_down(fx, o);
        fy += tile.shfl_down(fy, o);
        fz += tile.shfl_down(fz, o);
    }
    if (live && gl == 0) {
        if (FULL) {
            P.frc[i] = make_double4_32a(fx, fy, fz, 0.0);
        } else {
            atomicAdd(&P.frc[i].x, fx);
            atomicAdd(&P.frc[i].y, fy);
            atomicAdd(&P.frc[i].z, fz);
        }
    }
    double tot = block_sum<256>(e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

// Mixed precision forces, full list: FP32 pair arithmetic on cell-relative coordinates
// (displacement = prel_j - prel_i + image shift). LPA lanes share one atom and stride through its
// list; each lane consumes its entries in batches (list words first, then the position gathers,
// so several independent loads are in flight). Image shifts come from a 64-entry table in shared
// memory indexed by the entry's code. Pair terms are summed in FP32 over a batch and the batch
// sums are added in FP64 (ACC = 0), or kept as compensated FP32 sums (ACC = 1, a measured variant)
// and converted once at the end; the group's lanes are then reduced in FP64 with tile shuffles.
// PE = sum_i sum_j u_ij, halved at the reduction.
template <int ACC, int LPA, bool ONE, int MIX_BATCH>
__global__ void __launch_bounds__(256) k_force_mixed(const DP P, int step_mode) {
    __shared__ double sh[32];
    __shared__ float4 shift[64];
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of<LPA>(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    if (threadIdx.x < 64) {
        // code -> image shift; a 3 in any field marks a padding entry and sends it out of range
        const int c = threadIdx.x;
        const int bx = c & 3, by = (c >> 2) & 3, bz = (c >> 4) & 3;
        const float fx = bx == 1 ? 1.f : (bx == 2 ? -1.f : 0.f);
        const float fy = by == 1 ? 1.f : (by == 2 ? -1.f : 0.f);
        const float fz = bz == 1 ? 1.f : (bz == 2 ? -1.f : 0.f);
        const bool pad = bx == 3 || by == 3 || bz == 3;
        shift[c] = pad ? make_float4(1e18f, 1e18f, 1e18f, 0.f)
                       : make_float4(fx * sp.fcs[0], fy * sp.fcs[1], fz * sp.fcs[2], 0.f);
    }
    __syncthreads();
    const int gl = (int)tile.thread_rank();
    constexpr int FLUSH = 32;  // entries per lane between FP64 (or compensated) folds
    double e = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
    if (live) {
        const float4* __restrict__ prel = P.prel;
        const float4 pi = prel[i];
        const int ti = __float_as_int(pi.w);
        const LJDev* tab = P.tab + sp.tab0 + ti * sp.nt;
        const float frc2_0 = tab[0].frc2, fs2_0 = tab[0].fsigma2, fe24_0 = tab[0].feps24, fe4_0 = tab[0].feps4,
                    fuc_0 = tab[0].fucut;
        float cx = 0.f, cy = 0.f, cz = 0.f, ce = 0.f;  // Kahan compensation (ACC = 1)
        float sx = 0.f, sy = 0.f, sz = 0.f, se = 0.f;  // Kahan sums (ACC = 1)
        const int nn = P.nn[i];
        const int64_t row = P.npad * LPA;
        const uint32_t* __restrict__ nbp = P.nbr + (int64_t)i * LPA + gl;
        const uint32_t pad = (uint32_t)i | (63u << JBITS);
        float px = 0.f, py = 0.f, pz = 0.f, pe = 0.f;
        int since = 0;
        auto fold = [&]() {
            if (ACC == 0) {
                fx += (double)px;
                fy += (double)py;
                fz += (double)pz;
                e += (double)pe;
            } else {
                float y = px - cx, t = sx + y;
                cx = (t - sx) - y;
                sx = t;
                y = py - cy, t = sy + y;
                cy = (t - sy) - y;
                sy = t;
                y = pz - cz, t = sz + y;
                cz = (t - sz) - y;
                sz = t;
                y = pe - ce, t = se + y;
                ce = (t - se) - y;
                se = t;
            }
            px = py = pz = pe = 0.f;
        };
        // list words are addressed with 32-bit offsets from the lane's first word (the pool's list
        // is below 2^32 words, checked at init); full batches load unconditionally, the last
        // partial batch pads with an out-of-range entry
        const uint32_t row32 = (uint32_t)row;
        uint32_t qoff = 0;
        for (int k0 = 0; k0 < nn; k0 += LPA * MIX_BATCH) {
            uint32_t ent[MIX_BATCH];
            if (k0 + LPA * MIX_BATCH <= nn) {
#pragma unroll
                for (int b = 0; b < MIX_BATCH; ++b) ent[b] = __ldg(nbp + qoff + (uint32_t)b * row32);
            } else {
#pragma unroll
                for (int b = 0; b < MIX_BATCH; ++b)
                    ent[b] = (k0 + b * LPA + gl < nn) ? __ldg(nbp + qoff + (uint32_t)b * row32) : pad;
            }
            qoff += (uint32_t)MIX_BATCH * row32;
            float4 pj[MIX_BATCH];
#pragma unroll
            for (int b = 0; b < MIX_BATCH; ++b) pj[b] = __ldg(prel + (ent[b] & JMASK));
#pragma unroll
            for (int b = 0; b < MIX_BATCH; ++b) {
                const float4 sv = shift[ent[b] >> JBITS];
                const float dx = (pj[b].x - pi.x) + sv.x;
                const float dy = (pj[b].y - pi.y) + sv.y;
                const float dz = (pj[b].z - pi.z) + sv.z;
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                float frc2 = frc2_0, fs2 = fs2_0, fe24 = fe24_0, fe4 = fe4_0, fuc = fuc_0;
                if (!ONE) {
                    const LJDev& L = tab[__float_as_int(pj[b].w)];
                    frc2 = L.present ? L.frc2 : -1.f;
                    fs2 = L.fsigma2;
                    fe24 = L.feps24;
                    fe4 = L.feps4;
                    fuc = L.fucut;
                }
                // evaluated for every entry and masked, so the warp never splits on the cutoff
                // (padding entries have r2 ~ 1e36: 1/r2 -> 0, masked anyway)
                const bool in = r2 <= frc2;
                const float inv = rcp_approx(r2);
                const float s2 = fs2 * inv;
                const float s6 = s2 * s2 * s2;
                // 24 eps s6 (2 s6 - 1) / r^2 and 4 eps (s6^2 - s6) - u(rc)
                const float c = in ? (s6 * fmaf(2.0f, s6, -1.0f)) * (fe24 * inv) : 0.f;
                const float u = in ? fmaf(fe4, fmaf(s6, s6, -s6), -fuc) : 0.f;
                px = fmaf(-c, dx, px);
                py = fmaf(-c, dy, py);
                pz = fmaf(-c, dz, pz);
                pe += u;
            }
            since += MIX_BATCH;
            if (since >= FLUSH) {
                fold();
                since = 0;
            }
        }
        fold();
        if (ACC == 1) {
            fx = (double)sx - (double)cx;
            fy = (double)sy - (double)cy;
            fz = (double)sz - (double)cz;
            e = (double)se - (double)ce;
        }
    }
#pragma unroll
    for (int o = LPA / 2; o > 0; o >>= 1) {
        fx += tile.shfl_down(fx, o);
        fy += tile.shfl_down(fy, o);
        fz += tile.shfl_down(fz, o);
    }
    if (live && gl == 0) P.frc[i] = make_double4_32a(fx, fy, fz, 0.0);
    double tot = block_sum<256>(e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

// Second half of verlet_step_nve (src/potentials/potential.rs:28-30):
// a_tdt = F/m; v += ((a_t + a_tdt) * 0.5) * dt; acc <- a_tdt (the next step's a_t); then chunk
// partials of KE = sum 0.5 m |v|^2 (src/atoms/properties.rs:17-24) and, on request,
// W = sum r_i F_i^T (:49-51). UPDATE = false only refreshes acc = F/m and reduces (after a
// force evaluation). EXACT keeps the reference's division and rounding order; the mixed path
// multiplies by the stored 1/m (acc.w) and fuses.
template <bool UPDATE, bool EXACT>
__global__ void k_integrate2(const DP P, int respect_steps) {
    __shared__ double sh[32];
    int s, i;
    bool live = atom_of(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, respect_steps)) return;
    const SysParams& sp = P.sp[s];
    const SysState& st = P.st[s];
    const int cur = st.cur;
    double ke = 0.0;
    double4_32a p = make_double4_32a(0, 0, 0, 0), f = p;
    if (live) {
        double4_32a v = P.vel[cur][i];
        const double4_32a a = P.acc[cur][i];
        f = P.frc[i];
        const double m = v.w;
        double bx, by, bz;
        if (EXACT) {
            bx = __dadd_rn(0.0, __ddiv_rn(f.x, m));
            by = __dadd_rn(0.0, __ddiv_rn(f.y, m));
            bz = __dadd_rn(0.0, __ddiv_rn(f.z, m));
        } else {
            bx = f.x * a.w;
            by = f.y * a.w;
            bz = f.z * a.w;
        }
        if (UPDATE) {
            if (EXACT) {
                v.x = __dadd_rn(v.x, __dmul_rn(__dmul_rn(__dadd_rn(a.x, bx), 0.5), sp.dt));
                v.y = __dadd_rn(v.y, __dmul_rn(__dmul_rn(__dadd_rn(a.y, by), 0.5), sp.dt));
                v.z = __dadd_rn(v.z, __dmul_rn(__dmul_rn(__dadd_rn(a.z, bz), 0.5), sp.dt));
            } else {
                const double hdt = 0.5 * sp.dt;
                v.x = fma(a.x + bx, hdt, v.x);
                v.y = fma(a.y + by, hdt, v.y);
                v.z = fma(a.z + bz, hdt, v.z);
            }
            P.vel[cur][i] = v;
        }
        P.acc[cur][i] = make_double4_32a(bx, by, bz, a.w);
        ke = __dmul_rn(__dmul_rn(0.5, m), norm2_ref(v.x, v.y, v.z));
        if (st.want_virial) p = P.pos[cur][i];
    }
    double tot = block_sum<256>(ke, sh);
    if (threadIdx.x == 0) P.ke_part[blockIdx.x] = tot;
    if (st.want_virial) {
        double r[3] = {p.x, p.y, p.z}, g[3] = {f.x, f.y, f.z};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                double t = block_sum<256>(live ? r[a] * g[b] : 0.0, sh);
                if (threadIdx.x == 0) P.vir_part[(int64_t)blockIdx.x * 9 + a * 3 + b] = t;
            }
    }
}

// Per-slot end of a step (or of a force evaluation): deterministic sums of the chunk partials,
// energy history, NaN check (PisError::NaNEnergy, src/errors.rs:87-88), counters.
// mode 0: step; mode 1: force evaluation only (PE); mode 2: KE/virial only.
__global__ void __launch_bounds__(END_THREADS) k_step_end(const DP P, int mode) {
    __shared__ double sh[32];
    int s = blockIdx.x;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    SysState& st = P.st[s];
    if (mode == 0 && st.steps_left <= 0) return;
    if (mode != 0 && !st.eval) return;
    double pe = 0.0, ke = 0.0;
    const int F = P.pe_stride;
    if (mode != 2)
        for (int c = threadIdx.x; c < sp.nch * F; c += END_THREADS) pe += P.pe_part[(int64_t)sp.ch0 * F + c];
    if (mode != 1)
        for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) ke += P.ke_part[sp.ch0 + c];
    pe = block_sum<END_THREADS>(pe, sh);
    ke = block_sum<END_THREADS>(ke, sh);
    double w[9];
    const bool vir = st.want_virial && mode != 1;
    if (vir) {
        for (int q = 0; q < 9; ++q) {
            double a = 0.0;
            for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) a += P.vir_part[(int64_t)(sp.ch0 + c) * 9 + q];
            w[q] = block_sum<END_THREADS>(a, sh);
        }
    }
    if (threadIdx.x == 0) {
        if (mode != 2) {
            if (P.full_list) pe *= 0.5;
            st.pe = pe;
        }
        if (mode != 1) st.ke = ke;
        if (vir)
            for (int q = 0; q < 9; ++q) st.virial[q] = w[q];
        if ((mode != 2 && pe != pe) || (mode != 1 && ke != ke)) st.flags |= FLAG_NAN;
        if (mode != 2 && st.rebuild) {
            st.rebuilds += 1;
            st.rebuild = 0;
        }
        if (mode == 2) {
            st.eval = 0;
            st.want_virial = 0;
        }
        if (mode == 0) {
            P.pe_hist[(int64_t)s * P.hist + (st.steps_done % P.hist)] = pe;
            st.steps_done += 1;
            st.steps_left -= 1;
        }
    }
}

// Mark slots for an evaluation (all active slots, or only `only` when >= 0); with `rebuild` the
// neighbour list is rebuilt first (new positions).
__global__ void k_mark_eval(const DP P, int only, int rebuild, int virial) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.max_slots || !P.sp[s].active) return;
    if (only >= 0 && s != only) return;
    P.st[s].eval = 1;
    P.st[s].want_virial = virial;
    if (rebuild) P.st[s].rebuild = 1;
}

__global__ void k_zero_forces(const DP P) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!P.st[s].eval) return;
    P.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
}

// Exact cutoff test of every list entry of one slot with the reference arithmetic (min-image,
// Vector3::norm, `> rcut`), for neighbour-set export.
__global__ void k_keep(const DP P, int slot) {
    int s, i;
    if (!atom_of(P, s, i) || s != slot) return;
    const SysParams& sp = P.sp[s];
    const int cur = P.st[s].cur;
    const double4_32a pi = P.pos[cur][i];
    const LJDev* tab = P.tab + sp.tab0 + type_of(pi.w) * sp.nt;
    const int L = P.pe_stride;
    for (int k = 0; k < P.nn[i]; ++k) {
        const int64_t q = (int64_t)(k / L) * (P.npad * L) + (int64_t)i * L + k % L;
        int j = (int)(P.nbr[q] & JMASK);
        double4_32a pj = P.pos[cur][j];
        double rx = min_image_axis(__dsub_rn(pj.x, pi.x), sp.h[0], sp.hinv[0]);
        double ry = min_image_axis(__dsub_rn(pj.y, pi.y), sp.h[1], sp.hinv[1]);
        double rz = min_image_axis(__dsub_rn(pj.z, pi.z), sp.h[2], sp.hinv[2]);
        const LJDev& L = tab[type_of(pj.w)];
        P.keep[q] = (uint8_t)(L.present && !(sqrt(norm2_ref(rx, ry, rz)) > L.rcut));
    }
}

// v <- M v (row-major M) for one slot (ensemble velocity scaling).
__global__ void k_scale_vel(const DP P, int slot, double m0, double m1, double m2, double m3, double m4,
                            double m5, double m6, double m7, double m8) {
    int s, i;
    if (!atom_of(P, s, i) || s != slot) return;
    const int cur = P.st[s].cur;
    double4_32a v = P.vel[cur][i];
    double x = m0 * v.x + m1 * v.y + m2 * v.z;
    double y = m3 * v.x + m4 * v.y + m5 * v.z;
    double z = m6 * v.x + m7 * v.y + m8 * v.z;
    P.vel[cur][i] = make_double4_32a(x, y, z, v.w);
}

// Atoms::scale_box (src/atoms/transformations.rs:5-16) for a diagonal box and diagonal M:
// s = h^-1 r (old box), r = h' s (new box).
__global__ void k_scale_pos(const DP P, int slot, double oh0, double oh1, double oh2, double nh0, double nh1,
                            double nh2) {
    int s, i;
    if (!atom_of(P, s, i) || s != slot) return;
    const int cur = P.st[s].cur;
    double4_32a p = P.pos[cur][i];
    p.x = nh0 * (oh0 * p.x);
    p.y = nh1 * (oh1 * p.y);
    p.z = nh2 * (oh2 * p.z);
    P.pos[cur][i] = p;
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
#define LAUNCH(kern, grid, block, ...)                                \
    do {                                                               \
        kern<<<(grid), (block), 0, stream_>>>(__VA_ARGS__);           \
        g_launches.fetch_add(1);                                       \
    } while (0)

Engine::Engine() {}

Engine::~Engine() {
    for (auto& kv : graphs_) {
        cudaGraphExecDestroy(kv.second.exec);
        for (auto e : kv.second.ev) cudaEventDestroy(e);
    }
    if (d_ && d_->keep) cudaFree(d_->keep);
    if (mem_) cudaFree(mem_);
    if (stream_) cudaStreamDestroy(stream_);
    delete d_;
}

pis_status Engine::check(cudaError_t e, const char* what, std::string& err) {
    if (e == cudaSuccess) return PIS_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return PIS_ERR_NO_MEMORY;
    return PIS_ERR_CUDA;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

pis_status Engine::init(const PoolOptions& opt, std::string& err) {
    opt_ = opt;
    if (opt.max_atoms <= 0 || opt.max_slots <= 0) {
        err = "pool needs atoms and slots";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.blk != 256) {
        err = "chunk size must be 256";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.lpa != 1 && opt.lpa != 4 && opt.lpa != 8 && opt.lpa != 16 && opt.lpa != 32) {
        err = "lanes per atom must be 1, 4, 8, 16 or 32";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    half_ = opt.list_kind == PIS_LIST_HALF ||
            (opt.list_kind == PIS_LIST_DEFAULT && opt.precision == PIS_PRECISION_FP64);
    if (opt.precision == PIS_PRECISION_MIXED && half_) {
        err = "the mixed-precision path uses a full list";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.max_atoms >= (int64_t)JMASK) {
        err = "a pool holds at most 2^26 - 1 atoms (neighbour entries carry a 26-bit index)";
        return PIS_ERR_UNSUPPORTED;
    }
    cap_ = opt.list_cap > 0 ? opt.list_cap : 192;
    cap_ = (cap_ + 31) / 32 * 32;  // whole row groups for every lanes-per-atom choice
    npad_ = (int64_t)align_up((size_t)opt.max_atoms, 32);
    if ((double)npad_ * (double)cap_ >= 4294967296.0) {
        err = "neighbour list of the pool exceeds 2^32 entries (atoms x capacity)";
        return PIS_ERR_NO_MEMORY;
    }
    max_chunks_ = (opt.max_atoms + opt.blk - 1) / opt.blk + opt.max_slots;
    int64_t max_cells = opt.max_cells > 0 ? opt.max_cells : opt.max_atoms + opt.max_slots;
    opt_.max_cells = max_cells;
    pis_status st = check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream", err);
    if (st) return st;

    const size_t NA = (size_t)opt.max_atoms, NC = (size_t)max_cells, NCH = (size_t)max_chunks_,
                 NS = (size_t)opt.max_slots;
    struct Item {
        void** p;
        size_t bytes;
    };
    d_ = new DevPtrs();
    std::memset(d_, 0, sizeof(DevPtrs));
    std::vector<Item> items = {
        {(void**)&d_->pos[0], 32 * NA}, {(void**)&d_->pos[1], 32 * NA}, {(void**)&d_->vel[0], 32 * NA},
        {(void**)&d_->vel[1], 32 * NA}, {(void**)&d_->acc[0], 32 * NA}, {(void**)&d_->acc[1], 32 * NA},
        {(void**)&d_->id[0], 4 * NA},   {(void**)&d_->id[1], 4 * NA},   {(void**)&d_->frc, 32 * NA},
        {(void**)&d_->posb, 32 * NA},   {(void**)&d_->prel, 16 * NA}, {(void**)&d_->prelb, 16 * NA},   {(void**)&d_->cellof, 4 * NA},
        {(void**)&d_->lcell, 4 * NA},   {(void**)&d_->slotin, 4 * NA},  {(void**)&d_->perm, 4 * NA},
        {(void**)&d_->nn, 4 * NA},      {(void**)&d_->nbr, 4 * (size_t)npad_ * cap_},
        {(void**)&d_->cell_count, 4 * NC}, {(void**)&d_->cell_start, 4 * NC},
        {(void**)&d_->cell_sys, 4 * NC}, {(void**)&d_->blk_sys, 4 * NCH},
        {(void**)&d_->blk_first, 4 * NCH}, {(void**)&d_->sp, sizeof(SysParams) * NS},
        {(void**)&d_->st, sizeof(SysState) * NS}, {(void**)&d_->tab, sizeof(LJDev) * (size_t)opt.max_types_total},
        {(void**)&d_->pe_part, 8 * NCH * 32}, {(void**)&d_->ke_part, 8 * NCH}, {(void**)&d_->vir_part, 72 * NCH},
        {(void**)&d_->pe_hist, 8 * NS * (size_t)opt.hist},
    };
    size_t total = 0;
    for (auto& it : items) total += align_up(it.bytes, 256);
    st = check(cudaMalloc(&mem_, total), "device allocation", err);
    if (st) return st;
    mem_bytes_ = total;
    char* base = (char*)mem_;
    for (auto& it : items) {
        *it.p = base;
        base += align_up(it.bytes, 256);
    }
    d_->keep = nullptr;
    d_->npad = npad_;
    d_->cap = (int32_t)cap_;
    d_->hist = opt.hist;
    d_->max_slots = opt.max_slots;
    d_->zero_forces = half_ ? 1 : 0;
    d_->full_list = half_ ? 0 : 1;
    d_->pe_stride = opt_.lpa;
    st = check(cudaMemsetAsync(mem_, 0, total, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->cell_sys, 0xff, 4 * NC, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->blk_sys, 0xff, 4 * NCH, stream_), "memset", err);
    if (st) return st;
    hp_.assign(NS, SysParams{});
    slot_rlist_.assign(NS, 0.0);
    free_atoms_.clear();
    free_cells_.clear();
    free_atoms_[0] = NA;
    free_cells_[0] = NC;
    free_tab_.assign(opt.max_types_total, 1);
    slot_tab_size_.assign(NS, 0);
    dirty_map_ = true;
    return sync(err);
}

static bool take_range(std::map<int64_t, int64_t>& fr, int64_t len, int64_t& at) {
    for (auto it = fr.begin(); it != fr.end(); ++it) {
        if (it->second >= len) {
            at = it->first;
            int64_t rest = it->second - len;
            fr.erase(it);
            if (rest > 0) fr[at + len] = rest;
            return true;
        }
    }
    return false;
}

static void give_range(std::map<int64_t, int64_t>& fr, int64_t at, int64_t len) {
    auto it = fr.emplace(at, len).first;
    auto nx = std::next(it);
    if (nx != fr.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        fr.erase(nx);
    }
    if (it != fr.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            fr.erase(it);
        }
    }
}

// Cell grid at rcut + skin: n_d = floor(L_d / rlist) (Atoms::divide_into_cells,
// src/atoms/neighbour_list.rs:45-57, evaluated at the list radius).
static void cell_grid(const SlotDesc& d, double rlist, int nc[3]) {
    for (int a = 0; a < 3; ++a) {
        double L = d.h[4 * a];
        double q = std::floor(L / rlist);
        nc[a] = q < 1.0 ? 1 : (q > 2000.0 ? 2000 : (int)q);
    }
}

static double slot_rlist(const SlotDesc& d) {
    double rc = 0.0;
    for (auto& e : d.table)
        if (e.present && e.rcut > rc) rc = e.rcut;
    return rc + d.skin;
}

bool Engine::fits(const SlotDesc& d) const {
    int nc[3];
    cell_grid(d, slot_rlist(d), nc);
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2] + 1;
    bool a = false, c = false;
    for (auto& kv : free_atoms_) a |= kv.second >= d.n;
    for (auto& kv : free_cells_) c |= kv.second >= ncell;
    int free_tab = 0, run = 0;
    for (int v : free_tab_) {
        run = v ? run + 1 : 0;
        free_tab = std::max(free_tab, run);
    }
    int slots = 0;
    for (auto& p : hp_) slots += !p.active;
    return a && c && slots > 0 && free_tab >= d.n_types * d.n_types;
}

int Engine::add_slot(const SlotDesc& d, const int32_t* type_ids, const double* pos, const double* vel,
                     const double* force, std::string& err) {
    if (d.n <= 0) {
        err = "no atoms defined";
        return -PIS_ERR_NO_ATOMS;
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            if (a != b && d.h[3 * a + b] != 0.0) {
                err = "only orthorhombic boxes are supported (tilt factors must be zero)";
                return -PIS_ERR_UNSUPPORTED;
            }
    for (int a = 0; a < 3; ++a)
        if (!d.pbc[a]) {
            err = "only fully periodic boxes are supported";
            return -PIS_ERR_UNSUPPORTED;
        }
    const int nt = d.n_types;
    if (nt < 1 || (int)d.table.size() != nt * nt || (int)d.masses.size() < nt) {
        err = "pair table / masses do not match the number of types";
        return -PIS_ERR_INVALID_ARGUMENT;
    }
    double rlist = slot_rlist(d);
    if (rlist <= d.skin) {
        err = "no pair potential defined";
        return -PIS_ERR_MISSING_POTENTIAL;
    }
    for (int a = 0; a < 3; ++a) {
        double L = d.h[4 * a];
        if (!(L > 2.0 * rlist)) {
            err = "box edge " + std::to_string(L) + " is not longer than 2 (rcut + skin) = " +
                  std::to_string(2.0 * rlist);
            return -PIS_ERR_BOX_TOO_SMALL;
        }
    }
    for (int64_t k = 0; k < d.n; ++k)
        if (type_ids[k] < 1 || type_ids[k] > nt) {
            err = "atom type " + std::to_string(type_ids[k]) + " out of range";
            return -PIS_ERR_INVALID_ATOM_TYPE;
        }
    int slot = -1;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (!hp_[s].active) {
            slot = s;
            break;
        }
    if (slot < 0) {
        err = "no free slot";
        return -PIS_ERR_NO_MEMORY;
    }
    int nc[3];
    cell_grid(d, rlist, nc);
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t a0 = 0, c0 = 0;
    if (!take_range(free_atoms_, d.n, a0)) {
        err = "not enough free atom capacity in the pool";
        return -PIS_ERR_NO_MEMORY;
    }
    if (!take_range(free_cells_, ncell + 1, c0)) {
        give_range(free_atoms_, a0, d.n);
        err = "not enough free cell capacity in the pool";
        return -PIS_ERR_NO_MEMORY;
    }
    int tab0 = -1;
    {
        int need = nt * nt, run = 0;
        for (int k = 0; k < (int)free_tab_.size(); ++k) {
            run = free_tab_[k] ? run + 1 : 0;
            if (run == need) {
                tab0 = k - need + 1;
                break;
            }
        }
        if (tab0 < 0) {
            give_range(free_atoms_, a0, d.n);
            give_range(free_cells_, c0, ncell + 1);
            err = "pair table capacity exhausted";
            return -PIS_ERR_NO_MEMORY;
        }
        for (int k = 0; k < need; ++k) free_tab_[tab0 + k] = 0;
    }
    slot_tab_size_[slot] = nt * nt;

    // pair table
    std::vector<LJDev> tab((size_t)nt * nt);
    for (int k = 0; k < nt * nt; ++k) {
        const LJHost& e = d.table[k];
        LJDev& t = tab[k];
        std::memset(&t, 0, sizeof(t));
        t.present = e.present;
        if (!e.present) continue;
        // exactly the reference's per-pair constants: 4.0*eps, 24.0*eps, sigma.powi(2),
        // u_cut from (sigma/rcut).powi(2) (src/potentials/lennard_jones.rs:33-55)
        t.eps4 = 4.0 * e.epsilon;
        t.eps24 = 24.0 * e.epsilon;
        t.sigma2 = e.sigma * e.sigma;
        t.rcut = e.rcut;
        double rc2 = e.rcut * e.rcut;
        t.rc2_lo = rc2 * (1.0 - 1e-12);
        t.rc2_hi = rc2 * (1.0 + 1e-12);
        double ucut = 0.0;
        if (e.shift) {
            double q = e.sigma / e.rcut;
            double ci2 = q * q;
            double ca = ci2 * (ci2 * ci2);
            double cr = ca * ca;
            ucut = 4.0 * e.epsilon * (cr - ca);
        }
        t.ucut = ucut;
        t.feps4 = (float)t.eps4;
        t.feps24 = (float)t.eps24;
        t.fsigma2 = (float)t.sigma2;
        t.frc2 = (float)rc2;
        t.fucut = (float)ucut;
    }
    pis_status st = check(cudaMemcpyAsync(d_->tab + tab0, tab.data(), sizeof(LJDev) * tab.size(),
                                          cudaMemcpyHostToDevice, stream_),
                          "table upload", err);
    if (st) return -st;

    SysParams p;
    std::memset(&p, 0, sizeof(p));
    p.a0 = a0;
    p.c0 = c0;
    p.n = (int32_t)d.n;
    p.active = 1;
    p.nt = nt;
    p.tab0 = tab0;
    for (int a = 0; a < 3; ++a) {
        p.nc[a] = nc[a];
        p.pbc[a] = 1;
        p.h[a] = d.h[4 * a];
    }
    // h^-1 by adjugate / determinant, the reference's 3x3 inverse (src/simulation_box.rs:13)
    {
        const double* m = d.h;
        double m11 = m[4] * m[8] - m[7] * m[5];
        double det = m[0] * m11 - m[1] * (m[3] * m[8] - m[6] * m[5]) + m[2] * (m[3] * m[7] - m[6] * m[4]);
        p.hinv[0] = m11 / det;
        p.hinv[1] = (m[0] * m[8] - m[6] * m[2]) / det;
        p.hinv[2] = (m[0] * m[4] - m[3] * m[1]) / det;
    }
    for (int a = 0; a < 3; ++a) {
        p.cs[a] = p.h[a] / nc[a];
        p.fcs[a] = (float)p.cs[a];
    }
    p.half_skin2 = 0.25 * d.skin * d.skin;
    p.dt = d.dt;
    p.dt2 = d.dt * d.dt;
    double rl = rlist * (1.0 + 1e-5);
    p.frlist2 = (float)(rl * rl);
    // chunks
    p.nch = (int32_t)((d.n + opt_.blk - 1) / opt_.blk);
    p.ch0 = 0;  // assigned by the block map
    hp_[slot] = p;
    slot_rlist_[slot] = rlist;

    // atom state: AoS (x,y,z per atom) -> double4_32a with the type (pos.w) and mass (vel.w)
    std::vector<double4_32a> hpos(d.n), hvel(d.n), hfrc(d.n), hacc(d.n);
    std::vector<int32_t> hid(d.n);
    for (int64_t k = 0; k < d.n; ++k) {
        int t0 = type_ids[k] - 1;
        double w;
        int32_t hi = t0, lo = 0;
        uint64_t bits = ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo;
        std::memcpy(&w, &bits, 8);
        hpos[k] = make_double4_32a(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], w);
        double m = d.masses[t0];
        hvel[k] = vel ? make_double4_32a(vel[3 * k], vel[3 * k + 1], vel[3 * k + 2], m) : make_double4_32a(0, 0, 0, m);
        hfrc[k] = force ? make_double4_32a(force[3 * k], force[3 * k + 1], force[3 * k + 2], 0.0) : make_double4_32a(0, 0, 0, 0);
        // acc = 0 + F/m (Atoms::current_acceleration) and 1/m for the mixed path
        hacc[k] = make_double4_32a(0.0 + hfrc[k].x / m, 0.0 + hfrc[k].y / m, 0.0 + hfrc[k].z / m, 1.0 / m);
        hid[k] = (int32_t)k;
    }
    SysState ss;
    std::memset(&ss, 0, sizeof(ss));
    ss.cur = 0;
    ss.rebuild = 1;
    std::vector<int32_t> csys(ncell + 1, slot);
#define CP(dst, src, bytes)                                                                             \
    do {                                                                                                \
        st = check(cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyHostToDevice, stream_), "upload", err); \
        if (st) return -st;                                                                             \
    } while (0)
    CP(d_->pos[0] + a0, hpos.data(), 32 * d.n);
    CP(d_->vel[0] + a0, hvel.data(), 32 * d.n);
    CP(d_->frc + a0, hfrc.data(), 32 * d.n);
    CP(d_->posb + a0, hpos.data(), 32 * d.n);
    CP(d_->id[0] + a0, hid.data(), 4 * d.n);
    CP(d_->acc[0] + a0, hacc.data(), 32 * d.n);
    st = check(cudaMemsetAsync(d_->cellof + a0, 0, 4 * d.n, stream_), "upload", err);
    if (st) return -st;
    st = check(cudaMemsetAsync(d_->nn + a0, 0, 4 * d.n, stream_), "upload", err);
    if (st) return -st;
    st = check(cudaMemsetAsync(d_->cell_count + c0, 0, 4 * (ncell + 1), stream_), "upload", err);
    if (st) return -st;
    CP(d_->cell_sys + c0, csys.data(), 4 * (ncell + 1));
    CP(d_->st + slot, &ss, sizeof(ss));
#undef CP
    dirty_map_ = true;
    st = rebuild_block_map(err);
    if (st) return -st;
    st = sync(err);
    if (st) return -st;
    return slot;
}

void Engine::remove_slot(int slot) {
    if (slot < 0 || slot >= opt_.max_slots || !hp_[slot].active) return;
    SysParams& p = hp_[slot];
    int64_t ncell = (int64_t)p.nc[0] * p.nc[1] * p.nc[2];
    give_range(free_atoms_, p.a0, p.n);
    give_range(free_cells_, p.c0, ncell + 1);
    for (int k = 0; k < slot_tab_size_[slot]; ++k) free_tab_[p.tab0 + k] = 1;
    std::vector<int32_t> csys(ncell + 1, -1);
    cudaMemcpyAsync(d_->cell_sys + p.c0, csys.data(), 4 * (ncell + 1), cudaMemcpyHostToDevice, stream_);
    p.active = 0;
    dirty_map_ = true;
    std::string err;
    rebuild_block_map(err);
    cudaStreamSynchronize(stream_);
}

int Engine::n_active() const {
    int k = 0;
    for (auto& p : hp_) k += p.active;
    return k;
}

// Chunk table: every active slot gets ceil(n / blk) consecutive chunks; the grid is always
// max_chunks blocks so captured graphs stay valid when slots come and go.
pis_status Engine::rebuild_block_map(std::string& err) {
    if (!dirty_map_) return PIS_OK;
    std::vector<int32_t> bs(max_chunks_, -1), bf(max_chunks_, 0);
    int64_t c = 0;
    for (int s = 0; s < opt_.max_slots; ++s) {
        SysParams& p = hp_[s];
        if (!p.active) continue;
        p.ch0 = (int32_t)c;
        for (int k = 0; k < p.nch; ++k, ++c) {
            bs[c] = s;
            bf[c] = (int32_t)(p.a0 + (int64_t)k * opt_.blk);
        }
    }
    pis_status st = check(cudaMemcpyAsync(d_->blk_sys, bs.data(), 4 * max_chunks_, cudaMemcpyHostToDevice, stream_),
                          "block map", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(d_->blk_first, bf.data(), 4 * max_chunks_, cudaMemcpyHostToDevice, stream_),
               "block map", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(d_->sp, hp_.data(), sizeof(SysParams) * hp_.size(), cudaMemcpyHostToDevice, stream_),
               "params", err);
    if (st) return st;
    // host staging vectors must outlive the async copies
    st = check(cudaStreamSynchronize(stream_), "block map", err);
    dirty_map_ = false;
    // the force kernel variant depends on whether every slot is single-type; captured graphs
    // bake that choice in, so they are dropped when it flips
    bool one = true;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (hp_[s].active && hp_[s].nt != 1) one = false;
    if (one != single_type_) {
        single_type_ = one;
        for (auto& kv : graphs_) {
            cudaGraphExecDestroy(kv.second.exec);
            for (auto e : kv.second.ev) cudaEventDestroy(e);
        }
        graphs_.clear();
    }
    return st;
}

pis_status Engine::sync(std::string& err) { return check(cudaStreamSynchronize(stream_), "stream sync", err); }

pis_status Engine::set_dt(int slot, double dt, std::string& err) {
    SysParams& p = hp_[slot];
    if (p.dt == dt) return PIS_OK;
    p.dt = dt;
    p.dt2 = dt * dt;
    pis_status st = check(cudaMemcpyAsync(d_->sp + slot, &p, sizeof(SysParams), cudaMemcpyHostToDevice, stream_),
                          "params", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::set_steps(int slot, int64_t steps, std::string& err) {
    pis_status st = check(cudaMemcpyAsync(&d_->st[slot].steps_left, &steps, 8, cudaMemcpyHostToDevice, stream_),
                          "steps", err);
    if (st) return st;
    return sync(err);
}

void Engine::enqueue_rebuild(bool respect) {
    const DP& P = *d_;
    int r = respect ? 1 : 0;
    LAUNCH(k_bin, (unsigned)max_chunks_, opt_.blk, P, r);
    LAUNCH(k_scan, (unsigned)opt_.max_slots, SCAN_THREADS, P, r);
    LAUNCH(k_scatter, (unsigned)max_chunks_, opt_.blk, P, r);
    unsigned gcells = (unsigned)((opt_.max_cells * 32 + 255) / 256);
    LAUNCH(k_gather, gcells, 256, P, (int64_t)opt_.max_cells, r);
    launch_build(r);
}

// Lanes-per-atom kernels are templates; these dispatch on the pool's runtime choice. Their grid
// has lpa blocks per chunk.
template <int L>
static void launch_build_t(const DP& P, bool half, unsigned chunks, cudaStream_t st, int r) {
    if (L == 1) {
        // lean kernel for slots with >= 3 cells per axis, generic kernel for the rest
        if (half) {
            k_build1<true><<<chunks, 256, 0, st>>>(P, r);
            k_build1_generic<true><<<chunks, 256, 0, st>>>(P, r);
        } else {
            k_build1<false><<<chunks, 256, 0, st>>>(P, r);
            k_build1_generic<false><<<chunks, 256, 0, st>>>(P, r);
        }
        g_launches.fetch_add(2);
        return;
    }
    if (half)
        k_build<true, L><<<chunks * L, 256, 0, st>>>(P, r);
    else
        k_build<false, L><<<chunks * L, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

template <int L, int B>
static void launch_mixed_tb(const DP& P, bool kahan, bool one, unsigned chunks, cudaStream_t st, int r) {
    if (kahan && one)
        k_force_mixed<1, L, true, B><<<chunks * L, 256, 0, st>>>(P, r);
    else if (kahan)
        k_force_mixed<1, L, false, B><<<chunks * L, 256, 0, st>>>(P, r);
    else if (one)
        k_force_mixed<0, L, true, B><<<chunks * L, 256, 0, st>>>(P, r);
    else
        k_force_mixed<0, L, false, B><<<chunks * L, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

// Entries per batch (list words loaded before their gathers): a tuning knob for thread-per-atom;
// groups of lanes always use 4.
template <int L>
static void launch_mixed_t(const DP& P, bool kahan, bool one, int batch, unsigned chunks, cudaStream_t st, int r) {
    if (L == 1 && batch == 4)
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
    else if (L == 1 && batch == 16)
        launch_mixed_tb<L, 16>(P, kahan, one, chunks, st, r);
    else if (L == 1 && batch == 8)
        launch_mixed_tb<L, 8>(P, kahan, one, chunks, st, r);
    else if (L == 1)
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
    else
        launch_mixed_tb<L, 4>(P, kahan, one, chunks, st, r);
}

template <int L>
static void launch_fp64_t(const DP& P, bool half, bool fast, unsigned chunks, cudaStream_t st, int r) {
    if (half && !fast)
        k_force_fp64<false, false, L><<<chunks * L, 256, 0, st>>>(P, r);
    else if (half)
        k_force_fp64<false, true, L><<<chunks * L, 256, 0, st>>>(P, r);
    else if (!fast)
        k_force_fp64<true, false, L><<<chunks * L, 256, 0, st>>>(P, r);
    else
        k_force_fp64<true, true, L><<<chunks * L, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

#define PIS_LPA_DISPATCH(lpa, CALL) \
    switch (lpa) {                  \
        case 4: CALL(4); break;     \
        case 8: CALL(8); break;     \
        case 16: CALL(16); break;   \
        case 32: CALL(32); break;   \
        default: CALL(1); break;    \
    }

void Engine::launch_build(int r) {
    const unsigned ch = (unsigned)max_chunks_;

#define PIS_CALL(L) launch_build_t<L>(*d_, half_, ch, stream_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

void Engine::launch_force_mixed(int r) {
    const unsigned ch = (unsigned)max_chunks_;
#define PIS_CALL(L) launch_mixed_t<L>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, ch, stream_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

void Engine::launch_force_fp64(int r) {
    const unsigned ch = (unsigned)max_chunks_;
#define PIS_CALL(L) launch_fp64_t<L>(*d_, half_, opt_.fp64_fast, ch, stream_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

void Engine::enqueue_step(bool respect, cudaEvent_t* ev) {
    const DP& P = *d_;
    int r = respect ? 1 : 0;
    const bool mixed = opt_.precision == PIS_PRECISION_MIXED;
    if (ev) cudaEventRecordWithFlags(ev[0], stream_, cudaEventRecordExternal);
    if (mixed)
        LAUNCH(k_integrate1<true>, (unsigned)max_chunks_, opt_.blk, P);
    else
        LAUNCH(k_integrate1<false>, (unsigned)max_chunks_, opt_.blk, P);
    if (ev) cudaEventRecordWithFlags(ev[1], stream_, cudaEventRecordExternal);
    enqueue_rebuild(respect);
    if (ev) cudaEventRecordWithFlags(ev[2], stream_, cudaEventRecordExternal);
    if (mixed)
        launch_force_mixed(r);
    else
        launch_force_fp64(r);
    if (ev) cudaEventRecordWithFlags(ev[3], stream_, cudaEventRecordExternal);
    if (mixed)
        LAUNCH((k_integrate2<true, false>), (unsigned)max_chunks_, opt_.blk, P, r);
    else
        LAUNCH((k_integrate2<true, true>), (unsigned)max_chunks_, opt_.blk, P, r);
    if (ev) cudaEventRecordWithFlags(ev[4], stream_, cudaEventRecordExternal);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 0);
    if (ev) cudaEventRecordWithFlags(ev[5], stream_, cudaEventRecordExternal);
}

void Engine::enqueue_potential(int only) {
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    LAUNCH(k_mark_eval, sg, 128, P, only, 1, 0);
    LAUNCH(k_zero_forces, (unsigned)max_chunks_, opt_.blk, P);
    enqueue_rebuild(false);
    if (opt_.precision == PIS_PRECISION_MIXED)
        launch_force_mixed(0);
    else
        launch_force_fp64(0);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 1);
}

pis_status Engine::compute_potential(std::string& err) { return compute_potential_slot(-1, err); }

pis_status Engine::compute_potential_slot(int only, std::string& err) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    enqueue_potential(only);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return reduce_state_slot(true, only, err);
}

pis_status Engine::reduce_state(bool virial, std::string& err) { return reduce_state_slot(virial, -1, err); }

pis_status Engine::reduce_state_slot(bool virial, int only, std::string& err) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    LAUNCH(k_mark_eval, sg, 128, P, only, 0, virial ? 1 : 0);
    if (opt_.precision == PIS_PRECISION_MIXED)
        LAUNCH((k_integrate2<false, false>), (unsigned)max_chunks_, opt_.blk, P, 0);
    else
        LAUNCH((k_integrate2<false, true>), (unsigned)max_chunks_, opt_.blk, P, 0);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 2);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return sync(err);
}

void Engine::reset_stage_times() {
    for (double& v : stage_ms_) v = 0.0;
    stage_steps_ = 0;
}

pis_status Engine::run(int64_t k, std::string& err) {
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    const int64_t G = graph_steps_;
    while (k > 0) {
        int64_t g = k >= G ? G : k;
        int64_t key = 2 * g + (instrument_ ? 1 : 0);
        auto it = graphs_.find(key);
        if (it == graphs_.end()) {
            GraphRec rec;
            if (instrument_) {
                rec.ev.resize((size_t)(6 * g));
                for (auto& e : rec.ev) {
                    st = check(cudaEventCreate(&e), "event", err);
                    if (st) return st;
                }
            }
            cudaGraph_t graph;
            st = check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture", err);
            if (st) return st;
            int64_t before = g_launches.load();
            for (int64_t q = 0; q < g; ++q) enqueue_step(true, instrument_ ? rec.ev.data() + 6 * q : nullptr);
            int64_t captured = g_launches.load() - before;
            g_launches.fetch_sub(captured);
            kernels_per_step_ = captured / g;
            st = check(cudaStreamEndCapture(stream_, &graph), "capture", err);
            if (st) return st;
            st = check(cudaGraphInstantiate(&rec.exec, graph, 0), "instantiate", err);
            cudaGraphDestroy(graph);
            if (st) return st;
            it = graphs_.emplace(key, rec).first;
        }
        st = check(cudaGraphLaunch(it->second.exec, stream_), "graph launch", err);
        if (st) return st;
        g_launches.fetch_add(kernels_per_step_ * g);
        if (instrument_) {
            st = sync(err);
            if (st) return st;
            for (int64_t q = 0; q < g; ++q)
                for (int t = 0; t < 5; ++t) {
                    float ms = 0.f;
                    st = check(cudaEventElapsedTime(&ms, it->second.ev[6 * q + t], it->second.ev[6 * q + t + 1]),
                               "event timing", err);
                    if (st) return st;
                    stage_ms_[t] += ms;
                }
            stage_steps_ += g;
        }
        k -= g;
    }
    return check(cudaGetLastError(), "run", err);
}

pis_status Engine::download(int slot, double* pos, double* vel, double* force, std::string& err) {
    const SysParams& p = hp_[slot];
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    const int cur = ss.cur;
    std::vector<double4_32a> hp(p.n), hv(p.n), hf(p.n);
    std::vector<int32_t> hid(p.n);
    st = check(cudaMemcpyAsync(hid.data(), d_->id[cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "download", err);
    if (st) return st;
    if (pos) {
        st = check(cudaMemcpyAsync(hp.data(), d_->pos[cur] + p.a0, 32 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (vel) {
        st = check(cudaMemcpyAsync(hv.data(), d_->vel[cur] + p.a0, 32 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (force) {
        st = check(cudaMemcpyAsync(hf.data(), d_->frc + p.a0, 32 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    st = sync(err);
    if (st) return st;
    for (int k = 0; k < p.n; ++k) {
        int o = hid[k];
        if (pos) {
            pos[3 * o] = hp[k].x;
            pos[3 * o + 1] = hp[k].y;
            pos[3 * o + 2] = hp[k].z;
        }
        if (vel) {
            vel[3 * o] = hv[k].x;
            vel[3 * o + 1] = hv[k].y;
            vel[3 * o + 2] = hv[k].z;
        }
        if (force) {
            force[3 * o] = hf[k].x;
            force[3 * o + 1] = hf[k].y;
            force[3 * o + 2] = hf[k].z;
        }
    }
    return PIS_OK;
}

pis_status Engine::read_state(int slot, SysState& ss, std::string& err) {
    pis_status st = check(cudaMemcpyAsync(&ss, d_->st + slot, sizeof(SysState), cudaMemcpyDeviceToHost, stream_), "state", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::read_states(std::vector<SysState>& out, std::string& err) {
    out.resize(opt_.max_slots);
    pis_status st = check(cudaMemcpyAsync(out.data(), d_->st, sizeof(SysState) * opt_.max_slots,
                                          cudaMemcpyDeviceToHost, stream_), "state", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::read_pe_history(int slot, int64_t n, double* out, std::string& err) {
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (n > opt_.hist || n > ss.steps_done) {
        err = "energy history holds fewer steps than requested";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    std::vector<double> ring(opt_.hist);
    st = check(cudaMemcpyAsync(ring.data(), d_->pe_hist + (int64_t)slot * opt_.hist, 8 * opt_.hist,
                               cudaMemcpyDeviceToHost, stream_), "history", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    for (int64_t q = 0; q < n; ++q) out[q] = ring[(ss.steps_done - n + q) % opt_.hist];
    return PIS_OK;
}

pis_status Engine::list_entries(int slot, int64_t& total, std::string& err) {
    const SysParams& p = hp_[slot];
    std::vector<int32_t> nn(p.n);
    pis_status st = check(cudaMemcpyAsync(nn.data(), d_->nn + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    total = 0;
    for (int32_t v : nn) total += v;
    return PIS_OK;
}

pis_status Engine::neighbour_sets(int slot, std::vector<int64_t>& offsets, std::vector<int32_t>& idx,
                                  std::string& err) {
    const SysParams& p = hp_[slot];
    SysState ss;
    pis_status st = read_state(slot, ss, err);
    if (st) return st;
    if (!d_->keep) {
        st = check(cudaMalloc(&d_->keep, (size_t)npad_ * cap_), "keep mask", err);
        if (st) return st;
    }
    LAUNCH(k_keep, (unsigned)max_chunks_, opt_.blk, *d_, slot);
    st = check(cudaGetLastError(), "keep", err);
    if (st) return st;
    std::vector<int32_t> nn(p.n), id(p.n);
    st = check(cudaMemcpyAsync(nn.data(), d_->nn + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(id.data(), d_->id[ss.cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "id", err);
    if (st) return st;
    int32_t maxnn = 0;
    st = sync(err);
    if (st) return st;
    for (int32_t v : nn) maxnn = std::max(maxnn, v);
    const int L = opt_.lpa;
    const int groups = (maxnn + L - 1) / L;
    const size_t gsz = (size_t)p.n * L;  // words of one row group for this slot's atoms
    std::vector<uint32_t> ent((size_t)groups * gsz);
    std::vector<uint8_t> kp((size_t)groups * gsz);
    for (int r = 0; r < groups; ++r) {
        const int64_t off = (int64_t)r * npad_ * L + p.a0 * L;
        st = check(cudaMemcpyAsync(ent.data() + r * gsz, d_->nbr + off, 4 * gsz, cudaMemcpyDeviceToHost, stream_), "nbr", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(kp.data() + r * gsz, d_->keep + off, gsz, cudaMemcpyDeviceToHost, stream_), "keep", err);
        if (st) return st;
    }
    st = sync(err);
    if (st) return st;
    std::vector<std::vector<int32_t>> sets(p.n);
    for (int i = 0; i < p.n; ++i)
        for (int k = 0; k < nn[i]; ++k) {
            const size_t q = (size_t)(k / L) * gsz + (size_t)i * L + k % L;
            if (!kp[q]) continue;
            int j = (int)(ent[q] & JMASK) - (int)p.a0;
            sets[id[i]].push_back(id[j]);
            if (half_) sets[id[j]].push_back(id[i]);
        }
    offsets.assign(p.n + 1, 0);
    idx.clear();
    for (int i = 0; i < p.n; ++i) {
        std::sort(sets[i].begin(), sets[i].end());
        idx.insert(idx.end(), sets[i].begin(), sets[i].end());
        offsets[i + 1] = (int64_t)idx.size();
    }
    return PIS_OK;
}

pis_status Engine::scale_velocities(int slot, const double* m, std::string& err) {
    LAUNCH(k_scale_vel, (unsigned)max_chunks_, opt_.blk, *d_, slot, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
    pis_status st = check(cudaGetLastError(), "scale velocities", err);
    if (st) return st;
    return sync(err);
}

pis_status Engine::scale_box(int slot, const double* m, std::string& err) {
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            if (a != b && m[3 * a + b] != 0.0) {
                err = "box scaling must keep the box orthorhombic (diagonal matrix)";
                return PIS_ERR_UNSUPPORTED;
            }
    SysParams& p = hp_[slot];
    double nh[3] = {m[0] * p.h[0], m[4] * p.h[1], m[8] * p.h[2]};
    double rl = slot_rlist_[slot];
    for (int a = 0; a < 3; ++a)
        if (!(nh[a] > 2.0 * rl)) {
            err = "scaled box is shorter than 2 (rcut + skin)";
            return PIS_ERR_BOX_TOO_SMALL;
        }
    LAUNCH(k_scale_pos, (unsigned)max_chunks_, opt_.blk, *d_, slot, p.hinv[0], p.hinv[1], p.hinv[2], nh[0], nh[1], nh[2]);
    // new h and h^-1; the cell grid keeps its counts, the cell edge follows the box
    for (int a = 0; a < 3; ++a) {
        p.h[a] = nh[a];
        int ncnew = (int)std::floor(nh[a] / rl);
        (void)ncnew;
        p.cs[a] = nh[a] / p.nc[a];
        p.fcs[a] = (float)p.cs[a];
    }
    p.hinv[0] = (p.h[1] * p.h[2]) / (p.h[0] * (p.h[1] * p.h[2]));
    p.hinv[1] = (p.h[0] * p.h[2]) / (p.h[0] * (p.h[1] * p.h[2]));
    p.hinv[2] = (p.h[0] * p.h[1]) / (p.h[0] * (p.h[1] * p.h[2]));
    for (int a = 0; a < 3; ++a)
        if (p.cs[a] < rl) {
            err = "box shrank below the cell size; re-create the state to re-grid";
            return PIS_ERR_UNSUPPORTED;
        }
    pis_status st = check(cudaMemcpyAsync(d_->sp + slot, &p, sizeof(SysParams), cudaMemcpyHostToDevice, stream_), "params", err);
    if (st) return st;
    int32_t one = 1;
    st = check(cudaMemcpyAsync(&d_->st[slot].rebuild, &one, 4, cudaMemcpyHostToDevice, stream_), "params", err);
    if (st) return st;
    return sync(err);
}

}  // namespace pis
