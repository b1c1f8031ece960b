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
#include <cstdlib>
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
#ifndef PIS_FUSED_LQ
#define PIS_FUSED_LQ 8
#endif
// List layout factor of the fused step's pools: an atom's entries in groups of 8 consecutive words,
// so each 32-byte sector of the list holds 8 entries of one atom. The list build then fills whole
// sectors with consecutive stores (rebuild stage 0.173 vs 0.271 ms per step at 2.048M atoms with
// the column-major layout, 0.177 with groups of 4), and the force loop reads a batch of 4 entries
// as one 16-byte word.
constexpr int FUSED_LQ = PIS_FUSED_LQ;

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
    // cluster-list path (clm = atoms per cluster, 0 when the per-atom list is used)
    int32_t* cl_atom;     // per cluster: first atom | (members - 1) << JBITS
    int32_t* cl_start;    // per cell entry: first cluster of the cell (same indexing as cell_start)
    int32_t* cl_nn;       // per cluster: list length
    uint32_t* cl_nbr;     // column-major cluster list: entry k of cluster c at k * clpad + c
    int32_t* cblk_sys;    // per cluster chunk: slot (-1 unused)
    int32_t* cblk_first;  // per cluster chunk: first cluster
    int64_t clpad;
    int32_t ccap;
    int32_t clm;          // atoms per cluster of the cluster table (0: no table)
    int32_t cl_force;     // forces run over cluster lists (else per-atom lists)
    int32_t cl_lanes;     // cluster force blocks per cluster chunk (1, or M with a lane per member)
    int32_t lq;           // list layout: entry k of atom i at (k / lq) * npad * lq + i * lq + k % lq
                          // (lq = lanes per atom for lanes-per-atom pools, FUSED_LQ for the fused
                          // step's pools, whose kernels read 4 entries of a batch as one 16-byte word)
    int32_t* ctl;         // ctl[0]: some slot rebuilds its list in the current step or evaluation
    // fused step: cell-relative coordinates of the drifted atoms go to prel_out (the buffer the next
    // step reads)
    float4* prel_out;
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

// A neighbour-list word: read once per evaluation, so it is not kept in L1, which is left to the
// neighbour-position gathers (1 % faster force kernel on the 2.048M-atom liquid).
__device__ __forceinline__ uint32_t load_list_word(const uint32_t* p) {
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint4 load_list_quad(const uint32_t* p) {
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p));
    return v;
}
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Single hardware reciprocal approximation (rcp.approx.ftz.f32); ~1 ulp, flushes denormals.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- mbarrier / bulk-copy (TMA) helpers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// arrive (count 1) and announce `bytes` of bulk-copy transactions for the current phase
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of the given parity: false after `limit` unsuccessful polls (each
// poll may suspend the warp for a short hardware-defined time), so a wait can never hang.
constexpr uint32_t MBAR_WAIT_LIMIT = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < MBAR_WAIT_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Bulk copy global -> shared (no tensor map): both addresses 16-byte aligned, bytes a multiple of
// 16; completion is signalled on the mbarrier as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
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

// Which atom this thread owns in atom chunk `blk`. Returns false for padding threads; s < 0 for
// unused chunks.
__device__ __forceinline__ bool atom_of_blk(const DP& P, int blk, int& s, int& i) {
    s = P.blk_sys[blk];
    if (s < 0) return false;
    i = P.blk_first[blk] + (int)threadIdx.x;
    const SysParams& sp = P.sp[s];
    return i < (int)(sp.a0 + sp.n);
}
__device__ __forceinline__ bool atom_of(const DP& P, int& s, int& i) { return atom_of_blk(P, blockIdx.x, s, i); }

// Lanes-per-atom kernels: LPA consecutive lanes (a cooperative-groups tile) share one atom and
// there are LPA blocks per chunk. Returns false for padding groups; s < 0 for unused chunks.
template <int LPA>
__device__ __forceinline__ bool group_atom_of_blk(const DP& P, int blk, int& s, int& i) {
    const int chunk = blk / LPA, sub = blk % LPA;
    s = P.blk_sys[chunk];
    if (s < 0) return false;
    i = P.blk_first[chunk] + sub * (256 / LPA) + (int)(threadIdx.x / LPA);
    const SysParams& sp = P.sp[s];
    return i < (int)(sp.a0 + sp.n);
}
template <int LPA>
__device__ __forceinline__ bool group_atom_of(const DP& P, int& s, int& i) {
    return group_atom_of_blk<LPA>(P, blockIdx.x, s, i);
}

// The neighbour-list rebuild kernels' first test is the device-wide "some slot rebuilds this
// step" word, so on the ~9 steps in 10 without a rebuild every block exits after one cached load.
// They run one block per chunk (one warp per cell for the gather): the hardware balances the
// rebuilding chunks dynamically (a grid capped at a fixed number of blocks per SM, striding over
// chunks, left multi-wave tails and was measured slower).
__device__ __forceinline__ bool rebuild_pending(const DP& P) { return P.ctl[0] != 0; }
// The request word and the block's first table entry (its slot, or a cell's slot) are loaded
// together, so both the early exit and a rebuilding block pay one memory latency for them; then the
// slot's own flag, so that in a pool where some slot rebuilds every step (a replica mix) the blocks
// of the other slots exit after a second load.
__device__ __forceinline__ bool rebuild_block(const DP& P, const int32_t* slot_table, int64_t idx) {
    const int pending = P.ctl[0];
    const int s = slot_table[idx];
    return pending != 0 && s >= 0 && P.st[s].rebuild != 0;
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
//
// The mixed path's drift arithmetic (x + v dt + a dt^2/2 as two fused multiply-adds per axis, then
// the wrap of atoms that left the box); shared by k_integrate1 and the fused step kernel.
__device__ __forceinline__ void drift_mixed(const SysParams& sp, const double4_32a& p, const double4_32a& v,
                                            double ax, double ay, double az, double& x, double& y, double& z) {
    x = wrap_if_out(fma(ax, sp.hdt2, fma(v.x, sp.dt, p.x)), sp.h[0]);
    y = wrap_if_out(fma(ay, sp.hdt2, fma(v.y, sp.dt, p.y)), sp.h[1]);
    z = wrap_if_out(fma(az, sp.hdt2, fma(v.z, sp.dt, p.z)), sp.h[2]);
}
// Skin test: the slot rebuilds when any atom moved more than skin/2 since the last build. The
// minimum image is only taken when the plain difference fails the test (moved far, or crossed
// the periodic boundary). Returns the displacement since the build (for the cell-relative
// coordinates).
__device__ __forceinline__ void skin_test(const DP& P, const SysParams& sp, SysState& st, int i, double x,
                                          double y, double z, double& dx, double& dy, double& dz) {
    const double4_32a b = P.posb[i];
    dx = x - b.x, dy = y - b.y, dz = z - b.z;
    double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
    // d2 >= 0, so comparing bit patterns as integers orders it like the doubles (a NaN with
    // either sign fails the test too: its magnitude bits exceed every finite value's)
    if ((__double_as_longlong(d2) & 0x7fffffffffffffffll) > __double_as_longlong(sp.half_skin2)) {
        dx = min_image_axis(dx, sp.h[0], sp.hinv[0]);
        dy = min_image_axis(dy, sp.h[1], sp.hinv[1]);
        dz = min_image_axis(dz, sp.h[2], sp.hinv[2]);
        d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        if (!(d2 <= sp.half_skin2)) {  // NaN also requests a rebuild
            st.rebuild = 1;
            P.ctl[0] = 1;
        }
        if (x != x || y != y || z != z) atomicOr(&st.flags, FLAG_NAN);
    }
}
// cell-relative FP32 coordinates = build-time ones + displacement since the build
__device__ __forceinline__ float4 cell_relative_moved(const DP& P, int i, double dx, double dy, double dz) {
    const float4 q = P.prelb[i];
    return make_float4(q.x + (float)dx, q.y + (float)dy, q.z + (float)dz, q.w);
}

template <bool MIXED>
__global__ void k_integrate1(const DP P) {
    int s, i;
    if (!atom_of(P, s, i)) return;
    if (!slot_runs(P, s, true)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (threadIdx.x == 0 && st.rebuild) P.ctl[0] = 1;  // a rebuild requested before this step
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
        drift_mixed(sp, p, v, a.x, a.y, a.z, x, y, z);
    }
    P.pos[cur][i] = make_double4_32a(x, y, z, p.w);
    if (P.zero_forces) P.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    double dx, dy, dz;
    skin_test(P, sp, st, i, x, y, z, dx, dy, dz);
    if (MIXED) P.prel[i] = cell_relative_moved(P, i, dx, dy, dz);
}

// Counting sort, pass 1: cell of every atom (reference binning of src/atoms/neighbour_list.rs:
// 9-42 at rcut + skin, with a Euclidean modulo so atoms outside the box fold back in) and its
// slot inside the cell.
__device__ __forceinline__ void bin_chunk(const DP& P, int blk, int respect_steps) {
    int s, i;
    if (!atom_of_blk(P, blk, s, i)) return;
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
__global__ void k_bin(const DP P, int respect_steps) {
    if (!rebuild_block(P, P.blk_sys, blockIdx.x)) return;
    bin_chunk(P, blockIdx.x, respect_steps);
}

// One exclusive scan over a slot's cells: of the atom counts (CL = 0, the last pass, which also
// clears the counts) or of the cluster counts ceil(count / clm) (CL = 1). Writes absolute indices
// starting at `carry` and returns the total. Counts are staged through shared memory so global
// loads and stores stay coalesced while each thread scans SCAN_ITEMS consecutive cells.
template <bool CL>
__device__ __forceinline__ int scan_cells(int32_t* __restrict__ cnt_g, int32_t* __restrict__ start_g, int ncell,
                                          int carry, int clm, int* buf, int* warp_tot, int* carry_sh) {
    const int t = threadIdx.x, l = t & 31, w = t >> 5;
    const int carry0 = carry;
    for (int base = 0; base < ncell; base += SCAN_THREADS * SCAN_ITEMS) {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const int c = base + k * SCAN_THREADS + t;
            int v = 0;
            if (c < ncell) {
                v = cnt_g[c];
                if (CL)
                    v = (v + clm - 1) / clm;
                else
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
            if (l == 31) *carry_sh = xi;
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
        carry += *carry_sh;
        __syncthreads();
    }
    if (t == 0) start_g[ncell] = carry;
    return carry - carry0;
}

// Counting sort, pass 2: exclusive scans of the cell counts of one slot (one block per slot) -
// cluster starts (cluster table) and atom starts - and the flip of the slot's buffer set.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan(const DP P, int step_mode) {
    if (!rebuild_pending(P)) return;
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
    int ncl = 0;
    if (P.clm) ncl = scan_cells<true>(cnt_g, P.cl_start + sp.c0, ncell, sp.cl0, P.clm, buf, warp_tot, &carry_sh);
    scan_cells<false>(cnt_g, P.cell_start + sp.c0, ncell, (int)sp.a0, 1, buf, warp_tot, &carry_sh);
    if (threadIdx.x == 0) {
        st.ncl = ncl;
        st.cur ^= 1;
    }
}

// Counting sort, pass 3: destination of every atom.
__device__ __forceinline__ void scatter_chunk(const DP& P, int blk, int respect_steps) {
    int s, i;
    if (!atom_of_blk(P, blk, s, i)) return;
    if (!slot_runs(P, s, respect_steps)) return;
    if (!P.st[s].rebuild) return;
    const SysParams& sp = P.sp[s];
    int dst = P.cell_start[sp.c0 + P.lcell[i]] + P.slotin[i];
    P.perm[dst] = i;
}
__global__ void k_scatter(const DP P, int respect_steps) {
    if (!rebuild_block(P, P.blk_sys, blockIdx.x)) return;
    scatter_chunk(P, blockIdx.x, respect_steps);
}

// Order key of an atom inside its cell: the Morton index of its sub-cell on a 4 x 4 x 4 grid over
// the cell (6 bits, coarse bits high) above its original id (26 bits). Atoms that are consecutive
// in memory are then near each other in space, so the lanes of a warp own nearby atoms whose
// neighbour lists hold nearly the same atoms in the same order: their position gathers share cache
// sectors, and the list build's per-atom cell pruning agrees across the warp. The key depends only
// on the physical state, never on atomics.
__device__ __forceinline__ uint32_t cell_order_key(const SysParams& sp, const float4& q, uint32_t id) {
    uint32_t b[3];
    const float r[3] = {q.x, q.y, q.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int v = __float2int_rd(fmaf(r[d], sp.fsub[d], 2.0f));
        b[d] = (uint32_t)(v < 0 ? 0 : (v > 3 ? 3 : v));
    }
    const uint32_t m = (b[0] & 1u) | ((b[1] & 1u) << 1) | ((b[2] & 1u) << 2) | ((b[0] >> 1) << 3) |
                       ((b[1] >> 1) << 4) | ((b[2] >> 1) << 5);
    return (m << JBITS) | id;
}

// One warp per cell: order the cell's atoms by cell_order_key, then move every per-atom array into
// the new buffer set and record the build snapshot and cell-relative coordinates.
constexpr int GATHER_SMEM_KEYS = 256;  // per warp: order keys of cells of 65..256 atoms

__device__ __forceinline__ void gather_cell(const DP& P, int64_t g, int respect_steps, uint32_t* kb) {
    int lane = threadIdx.x & 31;
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
    // rank of every member by its order key: keys held in lane registers for cells of up to 64
    // atoms (one or two per lane), compared through warp shuffles; cells of up to 256 atoms (small
    // boxes have few, large cells) keep their keys in the warp's shared-memory buffer; larger
    // cells recompute keys
    auto key_of = [&](int src) {
        const double4_32a p = P.pos[src_set][src];
        return cell_order_key(sp, cell_relative(sp, p, lc, 0), (uint32_t)P.id[src_set][src]);
    };
    int rk[2] = {0, 0}, srcs[2] = {-1, -1};
    uint32_t keys[2] = {0xffffffffu, 0xffffffffu};
    float4 qs[2];
    if (cnt <= 64) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = lane + 32 * h;
            if (k < cnt) {
                srcs[h] = P.perm[beg + k];
                const double4_32a p = P.pos[src_set][srcs[h]];
                qs[h] = cell_relative(sp, p, lc, type_of(p.w));
                keys[h] = cell_order_key(sp, qs[h], (uint32_t)P.id[src_set][srcs[h]]);
            }
        }
        const int n0 = cnt < 32 ? cnt : 32;
        for (int q = 0; q < n0; ++q) {
            const uint32_t v = __shfl_sync(0xffffffffu, keys[0], q);
            rk[0] += v < keys[0];
            rk[1] += v < keys[1];
        }
        for (int q = 32; q < cnt; ++q) {
            const uint32_t v = __shfl_sync(0xffffffffu, keys[1], q - 32);
            rk[0] += v < keys[0];
            rk[1] += v < keys[1];
        }
    } else if (cnt <= GATHER_SMEM_KEYS) {
        for (int k = lane; k < cnt; k += 32) kb[k] = key_of(P.perm[beg + k]);
        __syncwarp();
    }
    for (int k = lane; k < cnt; k += 32) {
        int src, rank = 0;
        double4_32a p;
        float4 q;
        if (cnt <= 64) {
            const bool hi = k >= 32;
            src = hi ? srcs[1] : srcs[0];
            rank = hi ? rk[1] : rk[0];
            p = P.pos[src_set][src];
            q = hi ? qs[1] : qs[0];
        } else if (cnt <= GATHER_SMEM_KEYS) {
            src = P.perm[beg + k];
            const uint32_t mine = kb[k];
            for (int r = 0; r < cnt; ++r) rank += kb[r] < mine;
            p = P.pos[src_set][src];
            q = cell_relative(sp, p, lc, type_of(p.w));
        } else {
            src = P.perm[beg + k];
            const uint32_t mine = key_of(src);
            for (int r = 0; r < cnt; ++r) rank += key_of(P.perm[beg + r]) < mine;
            p = P.pos[src_set][src];
            q = cell_relative(sp, p, lc, type_of(p.w));
        }
        int dst = beg + rank;
        P.pos[dst_set][dst] = p;
        P.vel[dst_set][dst] = P.vel[src_set][src];
        P.acc[dst_set][dst] = P.acc[src_set][src];
        P.id[dst_set][dst] = P.id[src_set][src];
        P.posb[dst] = p;
        P.cellof[dst] = lc;
        P.prel[dst] = q;
        P.prelb[dst] = q;
    }
    // cluster table: runs of clm consecutive atoms of the cell (the last run may be shorter)
    if (P.clm) {
        const int M = P.clm;
        const int nclu = (cnt + M - 1) / M;
        const int cb = P.cl_start[g];
        for (int q = lane; q < nclu; q += 32) {
            const int m = min(M, cnt - q * M);
            P.cl_atom[cb + q] = (beg + q * M) | ((m - 1) << JBITS);
        }
    }
}
__global__ void k_gather(const DP P, int64_t max_cells, int respect_steps) {
    __shared__ uint32_t keybuf[256 / 32][GATHER_SMEM_KEYS];
    const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g < max_cells && rebuild_block(P, P.cell_sys, g)) gather_cell(P, g, respect_steps, keybuf[threadIdx.x >> 5]);
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
__device__ __forceinline__ void k_build_body(const DP& P, int blk, int step_mode) {
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of_blk<LPA>(P, blk, s, i);
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
                if (cnt < cap) {
                    const int64_t q = (int64_t)(cnt / P.lq) * (npad * P.lq) + (int64_t)i * P.lq + cnt % P.lq;
                    P.nbr[q] = (uint32_t)j | (code << JBITS);
                }
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
    if (!rebuild_block(P, P.blk_sys, blockIdx.x / LPA)) return;
    k_build_body<HALF, LPA>(P, blockIdx.x, step_mode);
}

// Thread-per-atom list build (the default shape). Same contents and order as k_build<HALF, 1>;
// cells whose nearest face is beyond the list radius for this atom are skipped.
//
template <bool HALF>
__device__ __forceinline__ void scan_cell(const float4* __restrict__ pp, int j, int jend, float sx, float sy,
                                          float sz, float rl2, uint32_t codebits, int i, bool home,
                                          uint32_t*& out, int& cnt, int64_t jump, int qmask, int cap) {
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
            ++cnt;
            // next entry: the next word of the atom's group of lq, or the next row group
            out += ((cnt & qmask) == 0) ? jump : 1;
        }
    }
}
template <bool HALF>
__device__ __forceinline__ void build1_chunk(const DP& P, int blk, int step_mode) {
    int s, i;
    if (!atom_of_blk(P, blk, s, i)) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    const int nx = sp.nc[0], ny = sp.nc[1], nz = sp.nc[2];
    if (!sp.walk27) return;  // the generic kernel handles the slot
    const int lc = P.cellof[i];
    const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
    const float4 pi = P.prel[i];
    const float csx = sp.fcs[0], csy = sp.fcs[1], csz = sp.fcs[2];
    const float rl2 = sp.frlist2;
    const int64_t npad = P.npad;
    const int cap = P.cap;
    const int32_t* __restrict__ cstart = P.cell_start + sp.c0;
    const float4* __restrict__ prel = P.prel;
    uint32_t* out = P.nbr + (int64_t)i * P.lq;
    const int qmask = P.lq - 1;
    const int64_t jump = npad * P.lq - qmask;
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
                                i, home, out, cnt, jump, qmask, cap);
            }
        }
    }
    if (cnt > cap) atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
    P.nn[i] = cnt > cap ? cap : cnt;
}
// only_two_cell: just the slots with a two-cell axis (the two-stage build covers the others).
template <bool HALF>
__global__ void __launch_bounds__(256) k_build1(const DP P, int step_mode, int only_two_cell) {
    if (!rebuild_block(P, P.blk_sys, blockIdx.x)) return;
    if (only_two_cell) {
        const SysParams& sp = P.sp[P.blk_sys[blockIdx.x]];
        if (sp.nc[0] >= 3 && sp.nc[1] >= 3 && sp.nc[2] >= 3) return;
    }
    build1_chunk<HALF>(P, blockIdx.x, step_mode);
}

// Slots the 27-cell walk does not serve (flagged !walk27: a two-cell axis within 1e-5 of twice
// the list radius): the group kernel's generic path, one lane per atom.
template <bool HALF>
__global__ void __launch_bounds__(256) k_build1_generic(const DP P, int step_mode) {
    if (!rebuild_block(P, P.blk_sys, blockIdx.x)) return;
    const int s = P.blk_sys[blockIdx.x];
    const SysParams& sp = P.sp[s];
    if (sp.walk27) return;
    k_build_body<HALF, 1>(P, blockIdx.x, step_mode);
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
// Image-shift table of the mixed kernels: code -> cell offset * cell edge; a 3 in any field marks
// a padding entry and sends it out of range.
__device__ __forceinline__ void fill_shift_table(float4* shift, const SysParams& sp) {
    if (threadIdx.x < 64) {
        const int c = threadIdx.x;
        const int bx = c & 3, by = (c >> 2) & 3, bz = (c >> 4) & 3;
        const float fx = bx == 1 ? 1.f : (bx == 2 ? -1.f : 0.f);
        const float fy = by == 1 ? 1.f : (by == 2 ? -1.f : 0.f);
        const float fz = bz == 1 ? 1.f : (bz == 2 ? -1.f : 0.f);
        const bool pad = bx == 3 || by == 3 || bz == 3;
        shift[c] = pad ? make_float4(1e18f, 1e18f, 1e18f, 0.f)
                       : make_float4(fx * sp.fcs[0], fy * sp.fcs[1], fz * sp.fcs[2], 0.f);
    }
}

// Per-axis image shifts: t[4a + c] = (0, +1, -1, pad) x cell edge along axis a for the axis's
// 2-bit code c. Three 4-word tables: the lanes of a warp read at most 4 distinct words per axis, so
// a lookup is one shared-memory wavefront, where the 64-entry float4 table's scattered 16-byte reads
// conflict on banks (~7 wavefronts per warp-wide lookup).
__device__ __forceinline__ void fill_shift_axes(float* t, const SysParams& sp) {
    if (threadIdx.x < 12) {
        const int a = threadIdx.x >> 2, c = threadIdx.x & 3;
        t[threadIdx.x] = c == 3 ? 1e18f : (c == 1 ? sp.fcs[a] : (c == 2 ? -sp.fcs[a] : 0.f));
    }
}
__device__ __forceinline__ float3 shift_of(const float4* t, uint32_t code) {
    const float4 v = t[code];
    return make_float3(v.x, v.y, v.z);
}
__device__ __forceinline__ float3 shift_of(const float* t, uint32_t code) {
    return make_float3(t[code & 3u], t[4 + ((code >> 2) & 3u)], t[8 + (code >> 4)]);
}

// Per-atom accumulator of the mixed kernels: FP32 pair terms summed over a batch, batch sums
// added in FP64 (ACC = 0) or kept as compensated FP32 sums (ACC = 1) and converted at the end.
template <int ACC>
struct MixAcc {
    double fx = 0.0, fy = 0.0, fz = 0.0, e = 0.0;
    float px = 0.f, py = 0.f, pz = 0.f, pe = 0.f;  // current batch sums
    float cx = 0.f, cy = 0.f, cz = 0.f, ce = 0.f;  // Kahan compensation (ACC = 1)
    float sx = 0.f, sy = 0.f, sz = 0.f, se = 0.f;  // Kahan sums (ACC = 1)
    __device__ __forceinline__ void fold() {
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
    }
    __device__ __forceinline__ void finish() {
        fold();
        if (ACC == 1) {
            fx = (double)sx - (double)cx;
            fy = (double)sy - (double)cy;
            fz = (double)sz - (double)cz;
            e = (double)se - (double)ce;
        }
    }
};

// Pair constants of atom i's type row (the single-type case reads entry 0 once).
struct MixLJ {
    float frc2, fs2, fe24, fe4, fuc;
};

// The FP32 LJ terms of one batch of list entries against atom i (cell-relative coordinates pi):
// gathers of every neighbour's prel first (all in flight together), then the pair math, summed
// into the accumulator's batch sums.
// SELF: the list may hold atom i itself (cluster lists), masked by r^2 > 0. pj: the entries'
// neighbour positions, already gathered.
template <bool ONE, int NB, int ACC, bool SELF = false, typename SH>
__device__ __forceinline__ void mixed_pairs_math(const uint32_t (&ent)[NB], const float4 (&pj)[NB], const float4& pi,
                                                 const SH* shift, const LJDev* tab, const MixLJ& P0,
                                                 MixAcc<ACC>& a) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const float3 sv = shift_of(shift, ent[b] >> JBITS);
        const float dx = (pj[b].x - pi.x) + sv.x;
        const float dy = (pj[b].y - pi.y) + sv.y;
        const float dz = (pj[b].z - pi.z) + sv.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float frc2 = P0.frc2, fs2 = P0.fs2, fe24 = P0.fe24, fe4 = P0.fe4, fuc = P0.fuc;
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
        const bool in = SELF ? (r2 <= frc2 && r2 > 0.f) : r2 <= frc2;
        const float inv = rcp_approx(r2);
        const float s2 = fs2 * inv;
        const float s6 = s2 * s2 * s2;
        // 24 eps s6 (2 s6 - 1) / r^2 and 4 eps (s6^2 - s6) - u(rc)
        const float c = in ? (s6 * fmaf(2.0f, s6, -1.0f)) * (fe24 * inv) : 0.f;
        const float u = in ? fmaf(fe4, fmaf(s6, s6, -s6), -fuc) : 0.f;
        a.px = fmaf(-c, dx, a.px);
        a.py = fmaf(-c, dy, a.py);
        a.pz = fmaf(-c, dz, a.pz);
        a.pe += u;
    }
}

template <bool ONE, int NB, int ACC, bool SELF = false, typename SH>
__device__ __forceinline__ void mixed_pairs(const uint32_t (&ent)[NB], const float4* __restrict__ prel,
                                            const float4& pi, const SH* shift, const LJDev* tab,
                                            const MixLJ& P0, MixAcc<ACC>& a) {
    float4 pj[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) pj[b] = __ldg(prel + (ent[b] & JMASK));
    mixed_pairs_math<ONE, NB, ACC, SELF>(ent, pj, pi, shift, tab, P0, a);
}

__device__ __forceinline__ MixLJ mix_lj_load(const LJDev& L) {
    return MixLJ{L.frc2, L.fsigma2, L.feps24, L.feps4, L.fucut};
}

constexpr int MIX_FLUSH = 32;  // entries per lane between FP64 (or compensated) folds

// The pair sum of one atom (or of lane gl of its LPA lanes) over its list: gathers in batches of
// MIX_BATCH entries, FP32 pair terms, folds every MIX_FLUSH entries. Returns the atom's
// cell-relative position. Shared by k_force_mixed and the fused step kernel.
// PF > 0 (thread per atom): the list rows of the batch PF batches ahead are prefetched into L2, so
// the list words (streamed from DRAM) arrive while the current batch's gathers are in flight.
// Q = 4 or 8 (thread per atom, pools with list layout lq = Q): an atom's entries lie in groups of Q
// consecutive words; 4 entries of a batch are one 16-byte load.
template <int ACC, int LPA, bool ONE, int MIX_BATCH, int PF = 0, int Q = 1, typename SH>
__device__ __forceinline__ float4 mixed_atom_forces(const DP& P, const SysParams& sp, int i, int gl,
                                                    const SH* shift, MixAcc<ACC>& acc) {
    if constexpr (LPA == 1 && Q >= 4) {
        static_assert(MIX_BATCH % 4 == 0 && (Q == 4 || Q == 8), "16-byte pieces of Q-entry groups");
        const float4* __restrict__ prel = P.prel;
        const float4 pi = prel[i];
        const int ti = __float_as_int(pi.w);
        const LJDev* tab = P.tab + sp.tab0 + ti * sp.nt;
        const MixLJ P0 = mix_lj_load(tab[0]);
        const int nn = P.nn[i];
        const uint32_t* __restrict__ nbp = P.nbr + (int64_t)i * Q;
        const uint32_t pad = (uint32_t)i | (63u << JBITS);
        const uint32_t grp = (uint32_t)P.npad * (uint32_t)Q;  // words between an atom's consecutive groups
        // word offset of entry k (a multiple of 4) from the atom's first word
        auto at = [&](int k) { return (uint32_t)(k / Q) * grp + (uint32_t)(k % Q); };
        int since = 0;
        for (int k0 = 0; k0 < nn; k0 += MIX_BATCH) {
            if (PF > 0) {
#pragma unroll
                for (int g = 0; g < MIX_BATCH / 4; g += Q / 4)
                    if (k0 + PF * MIX_BATCH + 4 * g < nn) prefetch_l2(nbp + at(k0 + PF * MIX_BATCH + 4 * g));
            }
            uint32_t ent[MIX_BATCH];
#pragma unroll
            for (int g = 0; g < MIX_BATCH / 4; ++g) {
                // a 16-byte piece that starts before nn lies inside the list (the capacity is a
                // multiple of Q)
                const uint4 w = (k0 + 4 * g < nn) ? load_list_quad(nbp + at(k0 + 4 * g))
                                                  : make_uint4(pad, pad, pad, pad);
                ent[4 * g] = w.x;
                ent[4 * g + 1] = w.y;
                ent[4 * g + 2] = w.z;
                ent[4 * g + 3] = w.w;
            }
            if (k0 + MIX_BATCH > nn) {
#pragma unroll
                for (int b = 0; b < MIX_BATCH; ++b)
                    if (k0 + b >= nn) ent[b] = pad;
            }
            mixed_pairs<ONE, MIX_BATCH, ACC>(ent, prel, pi, shift, tab, P0, acc);
            since += MIX_BATCH;
            if (since >= MIX_FLUSH) {
                acc.fold();
                since = 0;
            }
        }
        acc.finish();
        return pi;
    }
    const float4* __restrict__ prel = P.prel;
    const float4 pi = prel[i];
    const int ti = __float_as_int(pi.w);
    const LJDev* tab = P.tab + sp.tab0 + ti * sp.nt;
    const MixLJ P0 = mix_lj_load(tab[0]);
    const int nn = P.nn[i];
    const int64_t row = P.npad * LPA;
    const uint32_t* __restrict__ nbp = P.nbr + (int64_t)i * LPA + gl;
    const uint32_t pad = (uint32_t)i | (63u << JBITS);
    int since = 0;
    // list words are addressed with 32-bit offsets from the lane's first word (the pool's list
    // is below 2^32 words, checked at init); full batches load unconditionally, the last
    // partial batch pads with an out-of-range entry
    const uint32_t row32 = (uint32_t)row;
    uint32_t qoff = 0;
    for (int k0 = 0; k0 < nn; k0 += LPA * MIX_BATCH) {
        uint32_t ent[MIX_BATCH];
        if (PF > 0 && LPA == 1) {
#pragma unroll
            for (int b = 0; b < MIX_BATCH; ++b)
                if (k0 + PF * MIX_BATCH + b < nn) prefetch_l2(nbp + qoff + (uint32_t)(PF * MIX_BATCH + b) * row32);
        }
        if (k0 + LPA * MIX_BATCH <= nn) {
#pragma unroll
            for (int b = 0; b < MIX_BATCH; ++b) ent[b] = load_list_word(nbp + qoff + (uint32_t)b * row32);
        } else {
#pragma unroll
            for (int b = 0; b < MIX_BATCH; ++b)
                ent[b] = (k0 + b * LPA + gl < nn) ? load_list_word(nbp + qoff + (uint32_t)b * row32) : pad;
        }
        qoff += (uint32_t)MIX_BATCH * row32;
        mixed_pairs<ONE, MIX_BATCH, ACC>(ent, prel, pi, shift, tab, P0, acc);
        since += MIX_BATCH;
        if (since >= MIX_FLUSH) {
            acc.fold();
            since = 0;
        }
    }
    acc.finish();
    return pi;
}

template <int ACC, int LPA, bool ONE, int MIX_BATCH, int Q = 1>
__global__ void __launch_bounds__(256) k_force_mixed(const DP P, int step_mode) {
    __shared__ double sh[32];
    __shared__ float shift[12];
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of<LPA>(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    fill_shift_axes(shift, sp);
    __syncthreads();
    const int gl = (int)tile.thread_rank();
    MixAcc<ACC> acc;
    if (live) mixed_atom_forces<ACC, LPA, ONE, MIX_BATCH, 0, Q>(P, sp, i, gl, shift, acc);
    double fx = acc.fx, fy = acc.fy, fz = acc.fz, e = acc.e;
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

// Mixed precision forces, thread per atom, with the neighbour list streamed into shared memory by
// bulk copies (cp.async.bulk, the TMA engine's untiled mode). In the column-major list, row k of a
// 256-atom chunk is one contiguous run of 256 words, so the chunk's list is a stack of 1 KB rows.
// Thread 0 keeps MIX_TMA_STAGES batches of KB rows in flight in a shared-memory ring (one
// mbarrier per stage counts the copied bytes); the threads read their entries from shared memory
// instead of waiting on DRAM for each batch, then gather neighbour positions and do the same pair
// arithmetic as k_force_mixed. A stage is refilled once all 8 warps have released it (a second
// mbarrier per stage). Every wait is bounded: on expiry the block sets FLAG_TIMEOUT and stops.
// A row copy starts at the chunk's first atom rounded down to 4 (16-byte alignment) and covers
// the chunk's atoms rounded up to 4, which stays inside the list row (npad is a multiple of 32).
constexpr int MIX_TMA_STAGES = 4;
constexpr int MIX_TMA_ROW = 260;  // words per ring row: 256 atoms + up to 3 of alignment offset

template <int KB>
constexpr size_t mix_tma_smem_bytes() {
    return (size_t)MIX_TMA_STAGES * KB * MIX_TMA_ROW * sizeof(uint32_t);
}

template <int ACC, bool ONE, int KB>
__global__ void __launch_bounds__(256, KB <= 8 ? 4 : 2) k_force_mixed_tma(const DP P, int step_mode) {
    constexpr int S = MIX_TMA_STAGES;
    extern __shared__ __align__(128) uint32_t ring[];  // S * KB * MIX_TMA_ROW words
    __shared__ double sh[32];
    __shared__ float4 shift[64];
    __shared__ __align__(8) uint64_t full[S];
    __shared__ __align__(8) uint64_t empty[S];
    __shared__ int wmax[8];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;                             // uniform per block (one slot per chunk)
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    fill_shift_table(shift, sp);
    const int first = P.blk_first[blockIdx.x];
    const int cnt = min(256, (int)(sp.a0 + sp.n) - first);
    const int off = first & 3;
    const uint32_t row_bytes = (uint32_t)((off + cnt + 3) & ~3) * 4u;
    const int nn = live ? P.nn[i] : 0;
    const int m = __reduce_max_sync(0xffffffffu, nn);
    if (lane == 0) wmax[w] = m;
    if (t == 0) {
        for (int q = 0; q < S; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 8);
        }
        mbar_fence_init();
    }
    __syncthreads();
    int nmax = wmax[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) nmax = max(nmax, wmax[q]);
    const int R = (nmax + KB - 1) / KB;
    const uint32_t* __restrict__ src0 = P.nbr + (first - off);
    const int64_t npad = P.npad;
    auto issue = [&](int r) {
        const int q0 = r % S, k0 = r * KB;
        const int rows = min(KB, nmax - k0);
        mbar_arrive_tx(&full[q0], (uint32_t)rows * row_bytes);
        for (int q = 0; q < rows; ++q)
            bulk_g2s(ring + (q0 * KB + q) * MIX_TMA_ROW, src0 + (int64_t)(k0 + q) * npad, row_bytes, &full[q0]);
    };
    int issued = 0;
    if (t == 0)
        for (; issued < min(S, R); ++issued) issue(issued);

    MixAcc<ACC> acc;
    const float4* __restrict__ prel = P.prel;
    const float4 pi = live ? prel[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const LJDev* tab = P.tab + sp.tab0 + (live ? __float_as_int(pi.w) : 0) * sp.nt;
    const MixLJ P0 = mix_lj_load(tab[0]);
    const uint32_t pad = (uint32_t)(live ? i : first) | (63u << JBITS);
    const int col = off + t;
    // A thread whose wait expires stops waiting (and thread 0 stops issuing) but keeps running the
    // loop, so every lane still reaches each warp-level sync; its remaining entries are skipped.
    bool failed = false;
    int done = 0;  // batches this thread has seen arrive
    for (int r = 0; r < R; ++r) {
        const int q0 = r % S;
        const uint32_t par = (uint32_t)(r / S) & 1u;
        if (!failed && !mbar_wait(&full[q0], par)) failed = true;
        if (!failed) {
            done = r + 1;
            const int k0 = r * KB;
            if (k0 < nn) {
                uint32_t ent[KB];
                const uint32_t* rp = ring + q0 * KB * MIX_TMA_ROW + col;
#pragma unroll
                for (int b = 0; b < KB; ++b) ent[b] = (k0 + b < nn) ? rp[b * MIX_TMA_ROW] : pad;
                mixed_pairs<ONE, KB, ACC>(ent, prel, pi, shift, tab, P0, acc);
                if (((r + 1) * KB) % MIX_FLUSH == 0) acc.fold();
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[q0]);
        if (t == 0 && !failed && issued < R) {
            // refill this stage with batch r + S once every warp has released batch r
            if (mbar_wait(&empty[q0], par))
                issue(issued++);
            else
                failed = true;
        }
    }
    if (failed) {
        atomicOr(&st.flags, FLAG_TIMEOUT);
        // no copies are left in flight into shared memory: thread 0 waits (bounded) for every
        // batch it issued and has not seen arrive
        if (t == 0)
            for (int r = done; r < issued; ++r) mbar_wait(&full[r % S], (uint32_t)(r / S) & 1u);
    }
    acc.finish();
    if (live) P.frc[i] = make_double4_32a(acc.fx, acc.fy, acc.fz, 0.0);
    double tot = block_sum<256>(acc.e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

// Mixed precision forces with the neighbour-cell tiles staged in shared memory by bulk copies
// (cp.async.bulk, the TMA engine's untiled mode). Atoms are sorted by cell with x fastest, so when
// a 256-atom chunk lies in one cell row its neighbours lie in 9 rows (y, z = home +- 1), each a
// contiguous run of cells [xa - 1, xb + 1] - one contiguous atom range - plus, where the chunk
// touches x = 0 or x = nx - 1, the single wrapped cell at the other end of each row. Thread 0
// copies these <= 27 pieces of cell-relative positions into shared memory with one mbarrier
// counting the bytes. A list entry j | code then lives in shared memory at j + delta, delta
// depending only on the entry's piece - given by its image code and by whether the owning atom sits
// at a row end (x = 0 or nx - 1, where the -1 or +1 neighbour is the wrapped cell) - so delta is
// carried in the w field of the image-shift table (3 x 64 entries), and the gather becomes one
// shared-memory load with no extra instruction. The pair arithmetic is k_force_mixed's. Chunks
// that span two rows, or whose tiles exceed the buffer, gather from global memory as usual; the
// mbarrier wait is bounded (on expiry: FLAG_TIMEOUT, and the chunk gathers from global memory).
constexpr int TILE_ATOMS = 3328;  // 52 KB of float4 per block: four blocks per SM

template <int ACC, bool ONE>
__global__ void __launch_bounds__(256) k_force_mixed_tile(const DP P, int step_mode) {
    extern __shared__ __align__(16) float4 tile[];  // TILE_ATOMS
    __shared__ float4 shd[3 * 64];                 // (wrap state, code) -> image shift, delta bits in w
    __shared__ int psrc[27], plen[27], poff[27];   // pieces: first atom, atoms, shared-memory offset
    __shared__ int use_tile;
    __shared__ __align__(8) uint64_t bar;
    __shared__ double sh[32];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;  // uniform per block (one slot per chunk)
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    const int t = threadIdx.x;
    const int nx = sp.nc[0], ny = sp.nc[1], nz = sp.nc[2];
    const int first = P.blk_first[blockIdx.x];
    const int cnt = min(256, (int)(sp.a0 + sp.n) - first);
    if (t == 0) {
        int ok = 0;
        if (nx >= 3 && ny >= 3 && nz >= 3) {
            const int la = P.cellof[first], lb = P.cellof[first + cnt - 1];
            const int xa = la % nx, ya = (la / nx) % ny, za = la / (nx * ny);
            const int xb = lb % nx, yb = (lb / nx) % ny, zb = lb / (nx * ny);
            if (ya == yb && za == zb && !(xa == 0 && xb == nx - 1)) {
                const int32_t* cs = P.cell_start + sp.c0;
                const int xl = max(xa - 1, 0), xh = min(xb + 1, nx - 1);
                int off = 0;
                for (int oz = -1; oz <= 1; ++oz)
                    for (int oy = -1; oy <= 1; ++oy) {
                        const int row = (oz + 1) * 3 + (oy + 1);
                        const int rb = (wrapc(za + oz, nz) * ny + wrapc(ya + oy, ny)) * nx;
                        psrc[row] = cs[rb + xl];
                        plen[row] = cs[rb + xh + 1] - cs[rb + xl];
                        poff[row] = off;
                        off += plen[row];
                        psrc[9 + row] = cs[rb + nx - 1];  // wrapped -1 neighbour of x = 0
                        plen[9 + row] = xa == 0 ? cs[rb + nx] - cs[rb + nx - 1] : 0;
                        poff[9 + row] = off;
                        off += plen[9 + row];
                        psrc[18 + row] = cs[rb];  // wrapped +1 neighbour of x = nx - 1
                        plen[18 + row] = xb == nx - 1 ? cs[rb + 1] - cs[rb] : 0;
                        poff[18 + row] = off;
                        off += plen[18 + row];
                    }
                ok = off <= TILE_ATOMS;
            }
        }
        use_tile = ok;
        if (ok) {
            mbar_init(&bar, 1);
            mbar_fence_init();
        }
    }
    __syncthreads();
    const bool tiled = use_tile != 0;
    if (tiled && t == 0) {
        uint32_t bytes = 0;
        for (int p = 0; p < 27; ++p) bytes += (uint32_t)plen[p] * 16u;
        mbar_arrive_tx(&bar, bytes);
        for (int p = 0; p < 27; ++p)
            if (plen[p] > 0) bulk_g2s(tile + poff[p], P.prel + psrc[p], (uint32_t)plen[p] * 16u, &bar);
    }
    if (t < 3 * 64) {
        const int c = t & 63, w = t >> 6;
        const int bx = c & 3, by = (c >> 2) & 3, bz = (c >> 4) & 3;
        const bool pad = bx == 3 || by == 3 || bz == 3;
        const int ox = bx == 1 ? 1 : (bx == 2 ? -1 : 0);
        const int oy = by == 1 ? 1 : (by == 2 ? -1 : 0);
        const int oz = bz == 1 ? 1 : (bz == 2 ? -1 : 0);
        int delta = 0;
        if (tiled) {
            // padding entries point at the owning atom, which is in the home row's main piece
            const int row = pad ? 4 : (oz + 1) * 3 + (oy + 1);
            int p = row;
            if (!pad && w == 1 && ox == -1) p = 9 + row;
            if (!pad && w == 2 && ox == 1) p = 18 + row;
            delta = poff[p] - psrc[p];
        }
        shd[t] = pad ? make_float4(1e18f, 1e18f, 1e18f, __int_as_float(delta))
                     : make_float4(ox * sp.fcs[0], oy * sp.fcs[1], oz * sp.fcs[2], __int_as_float(delta));
    }
    __syncthreads();
    bool got = tiled && mbar_wait(&bar, 0u);
    if (tiled && !got) atomicOr(&st.flags, FLAG_TIMEOUT);
    // every thread uses the tile only if the whole block saw it arrive
    got = __syncthreads_and(got ? 1 : 0) != 0;
    MixAcc<ACC> acc;
    if (live) {
        const float4* __restrict__ prel = P.prel;
        const float4 pi = prel[i];
        const int ti = __float_as_int(pi.w);
        const LJDev* tab = P.tab + sp.tab0 + ti * sp.nt;
        const MixLJ P0 = mix_lj_load(tab[0]);
        const int cx = P.cellof[i] % nx;
        const float4* shift = shd + (got ? 64 * (cx == 0 ? 1 : (cx == nx - 1 ? 2 : 0)) : 0);
        const int nn = P.nn[i];
        const uint32_t row32 = (uint32_t)P.npad;
        const uint32_t* __restrict__ nbp = P.nbr + i;
        const uint32_t pad = (uint32_t)i | (63u << JBITS);
        constexpr int NB = 4;
        int since = 0;
        uint32_t qoff = 0;
        for (int k0 = 0; k0 < nn; k0 += NB) {
            uint32_t ent[NB];
            if (k0 + NB <= nn) {
#pragma unroll
                for (int b = 0; b < NB; ++b) ent[b] = load_list_word(nbp + qoff + (uint32_t)b * row32);
            } else {
#pragma unroll
                for (int b = 0; b < NB; ++b)
                    ent[b] = (k0 + b < nn) ? load_list_word(nbp + qoff + (uint32_t)b * row32) : pad;
            }
            qoff += (uint32_t)NB * row32;
            float4 pj[NB];
            if (got) {
#pragma unroll
                for (int b = 0; b < NB; ++b)
                    pj[b] = tile[(int)(ent[b] & JMASK) + __float_as_int(shift[ent[b] >> JBITS].w)];
            } else {
#pragma unroll
                for (int b = 0; b < NB; ++b) pj[b] = __ldg(prel + (ent[b] & JMASK));
            }
            mixed_pairs_math<ONE, NB, ACC>(ent, pj, pi, shift, tab, P0, acc);
            since += NB;
            if (since >= MIX_FLUSH) {
                acc.fold();
                since = 0;
            }
        }
        acc.finish();
        P.frc[i] = make_double4_32a(acc.fx, acc.fy, acc.fz, 0.0);
    }
    // no copy may still be writing into shared memory when the block exits
    if (tiled && !got && t == 0) mbar_wait(&bar, 0u);
    double tot = block_sum<256>(acc.e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

template <int ACC, bool ONE>
static cudaError_t allow_tile_smem() {
    return cudaFuncSetAttribute(k_force_mixed_tile<ACC, ONE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(TILE_ATOMS * sizeof(float4)));
}

// ---------------------------------------------------------------------------------------------
// Cluster-list path (mixed precision). A cluster is a run of up to M consecutive atoms of one
// cell; atoms are ordered inside each cell along a Morton curve, so a cluster's members are close
// in space. One thread owns a cluster: its members' coordinates live in registers, and its list
// holds every atom within the list radius of ANY member. Each list word and each neighbour
// gather then serves M pair evaluations instead of one, which cuts the scattered cache traffic
// that bounds the per-atom kernel; the price is the pairs of the union that a given member does
// not need (masked by the cutoff test).
// ---------------------------------------------------------------------------------------------
constexpr int CL_THREADS = 128;

// Build: thread per cluster. Every one of the 27 neighbour cell images whose box lies within the
// list radius of the members' bounding box is scanned, and an atom is appended when it is within
// the list radius of any member (FP32 on cell-relative coordinates, radius padded so the list is
// a superset). Lanes of one home cell walk the same cells in the same order, so their candidate
// loads coincide. On an axis with two cells the -1 and +1 images are the same cell at two shifts:
// both are scanned and an atom may be listed once per image; for any one member at most one image
// lies within the radius (the box is longer than twice the radius), so no pair counts twice.
template <int M>
__device__ __forceinline__ void build_cl_chunk(const DP& P, int blk, int step_mode, bool only_big) {
    const int s = P.cblk_sys[blk];
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    if (only_big && (sp.nc[0] < 3 || sp.nc[1] < 3 || sp.nc[2] < 3)) return;
    const int c = P.cblk_first[blk] + (int)threadIdx.x;
    if (c >= sp.cl0 + st.ncl) return;
    const uint32_t pk = (uint32_t)P.cl_atom[c];
    const int first = (int)(pk & JMASK), n = (int)(pk >> JBITS) + 1;
    const int nx = sp.nc[0], ny = sp.nc[1], nz = sp.nc[2];
    const int lc = P.cellof[first];
    const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
    const float4* __restrict__ prel = P.prel;
    float mx[M], my[M], mz[M];
    float lox = 1e30f, loy = 1e30f, loz = 1e30f, hix = -1e30f, hiy = -1e30f, hiz = -1e30f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        if (m < n) {
            const float4 q = prel[first + m];
            mx[m] = q.x;
            my[m] = q.y;
            mz[m] = q.z;
            lox = fminf(lox, q.x);
            loy = fminf(loy, q.y);
            loz = fminf(loz, q.z);
            hix = fmaxf(hix, q.x);
            hiy = fmaxf(hiy, q.y);
            hiz = fmaxf(hiz, q.z);
        } else {
            mx[m] = my[m] = mz[m] = 1e18f;  // padding member: never within the radius
        }
    }
    const float csx = sp.fcs[0], csy = sp.fcs[1], csz = sp.fcs[2];
    const float rl2 = sp.frlist2;
    const int64_t clpad = P.clpad;
    const int cap = P.ccap;
    const int32_t* __restrict__ cstart = P.cell_start + sp.c0;
    uint32_t* out = P.cl_nbr + c;
    int cnt = 0;
    for (int oz = -1; oz <= 1; ++oz) {
        const int z2 = wrapc(cz + oz, nz);
        // gap between the members' extent and the neighbour image's extent (home-cell frame)
        const float gz = fmaxf(fmaxf((oz - 0.5f) * csz - hiz, loz - (oz + 0.5f) * csz), 0.f);
        for (int oy = -1; oy <= 1; ++oy) {
            const int y2 = wrapc(cy + oy, ny);
            const float gy = fmaxf(fmaxf((oy - 0.5f) * csy - hiy, loy - (oy + 0.5f) * csy), 0.f);
            const float gyz = fmaf(gy, gy, gz * gz);
            if (gyz > rl2) continue;
            for (int ox = -1; ox <= 1; ++ox) {
                const float gx = fmaxf(fmaxf((ox - 0.5f) * csx - hix, lox - (ox + 0.5f) * csx), 0.f);
                if (fmaf(gx, gx, gyz) > rl2) continue;
                const int x2 = wrapc(cx + ox, nx);
                const int nb = (z2 * ny + y2) * nx + x2;
                const int b0 = cstart[nb], b1 = cstart[nb + 1];
                const uint32_t codebits = (((uint32_t)(ox < 0 ? 2 : ox)) | ((uint32_t)(oy < 0 ? 2 : oy) << 2) |
                                           ((uint32_t)(oz < 0 ? 2 : oz) << 4))
                                          << JBITS;
                // the members in the frame of this neighbour image
                float qx[M], qy[M], qz[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    qx[m] = mx[m] - ox * csx;
                    qy[m] = my[m] - oy * csy;
                    qz[m] = mz[m] - oz * csz;
                }
                const bool roomy = cnt + (b1 - b0) <= cap;
                for (int j = b0; j < b1; ++j) {
                    const float4 pj = prel[j];
                    bool take = false;
#pragma unroll
                    for (int m = 0; m < M; ++m) {
                        const float dx = pj.x - qx[m], dy = pj.y - qy[m], dz = pj.z - qz[m];
                        take |= fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rl2;
                    }
                    if (take) {
                        if (roomy || cnt < cap) *out = (uint32_t)j | codebits;
                        out += clpad;
                        ++cnt;
                    }
                }
            }
        }
    }
    if (cnt > cap) atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
    P.cl_nn[c] = cnt > cap ? cap : cnt;
}
// only_big: skip slots with a two-cell axis (the two-stage per-atom build leaves them to
// k_build1_generic)
template <int M>
__global__ void __launch_bounds__(CL_THREADS) k_build_cl(const DP P, int step_mode, int only_big) {
    if (!rebuild_block(P, P.cblk_sys, blockIdx.x)) return;
    build_cl_chunk<M>(P, blockIdx.x, step_mode, only_big != 0);
}

// Per-atom lists from cluster union lists (two-stage build, PIS_OPT_SCAN): after k_build_cl has
// listed, per cluster, every atom within the list radius of any member, one lane per member
// filters its cluster's union list into the member's own list. The filter applies k_build1's
// tests with k_build1's arithmetic - the per-atom face-distance skip of the entry's neighbour cell,
// the FP32 distance test on the same expressions, self / half exclusion - and the union list
// holds its candidates in k_build1's cell and atom order, so every member gets exactly the list
// k_build1 gives it. Cheaper than k_build1 because the candidate scan runs once per cluster, and
// the M lanes of a cluster share each union entry and each neighbour load. Slots with a two-cell
// axis are left to k_build1_generic.
template <bool HALF, int M>
__global__ void __launch_bounds__(CL_THREADS) k_filter_cl(const DP P, int step_mode) {
    const int chunk = blockIdx.x / M, sub = blockIdx.x % M;
    if (!rebuild_block(P, P.cblk_sys, chunk)) return;
    const int s = P.cblk_sys[chunk];
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    if (sp.nc[0] < 3 || sp.nc[1] < 3 || sp.nc[2] < 3) return;
    const int c = P.cblk_first[chunk] + sub * (CL_THREADS / M) + (int)threadIdx.x / M;
    if (c >= sp.cl0 + st.ncl) return;
    const uint32_t pk = (uint32_t)P.cl_atom[c];
    const int first = (int)(pk & JMASK), n = (int)(pk >> JBITS) + 1;
    const int m = (int)threadIdx.x % M;
    if (m >= n) return;
    const int i = first + m;
    const float4* __restrict__ prel = P.prel;
    const float4 pi = prel[i];
    const float csx = sp.fcs[0], csy = sp.fcs[1], csz = sp.fcs[2];
    const float rl2 = sp.frlist2;
    const float gxm = fmaxf(pi.x + 0.5f * csx, 0.f), gxp = fmaxf(0.5f * csx - pi.x, 0.f);
    const float gym = fmaxf(pi.y + 0.5f * csy, 0.f), gyp = fmaxf(0.5f * csy - pi.y, 0.f);
    const float gzm = fmaxf(pi.z + 0.5f * csz, 0.f), gzp = fmaxf(0.5f * csz - pi.z, 0.f);
    const int64_t npad = P.npad;
    const int cap = P.cap;
    const int nu = P.cl_nn[c];
    const uint32_t* __restrict__ un = P.cl_nbr + c;
    const uint32_t row = (uint32_t)P.clpad;
    uint32_t* out = P.nbr + i;
    int cnt = 0;
    for (int k = 0; k < nu; ++k) {
        const uint32_t e = load_list_word(un + (uint32_t)k * row);
        const int j = (int)(e & JMASK);
        const uint32_t code = e >> JBITS;
        const int ox = (code & 3u) == 2u ? -1 : (int)(code & 3u);
        const int oy = ((code >> 2) & 3u) == 2u ? -1 : (int)((code >> 2) & 3u);
        const int oz = ((code >> 4) & 3u) == 2u ? -1 : (int)((code >> 4) & 3u);
        const float ex = ox < 0 ? gxm : (ox > 0 ? gxp : 0.f);
        const float ey = oy < 0 ? gym : (oy > 0 ? gyp : 0.f);
        const float ez = oz < 0 ? gzm : (oz > 0 ? gzp : 0.f);
        const float eyz = fmaf(ey, ey, ez * ez);
        if (fmaf(ex, ex, eyz) > rl2) continue;  // k_build1 never scans this cell for atom i
        const float4 pj = prel[j];
        const float dx = pj.x + (ox * csx - pi.x), dy = pj.y + (oy * csy - pi.y), dz = pj.z + (oz * csz - pi.z);
        bool take = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rl2;
        if (HALF)
            take = take && j > i;
        else if (ox == 0 && oy == 0 && oz == 0)
            take = take && j != i;
        if (take) {
            if (cnt < cap) *out = e;
            out += npad;
            ++cnt;
        }
    }
    if (cnt > cap) atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
    P.nn[i] = cnt > cap ? cap : cnt;
}

// Forces: thread per cluster. For each batch of NB list entries the words are loaded, then the
// NB neighbour gathers, then every (member, entry) pair is evaluated with the same FP32
// arithmetic as the per-atom kernel, masked by the pair's cutoff and by r^2 > 0 (a member meets
// itself in the list at distance exactly zero). Per member the FP32 batch sums are folded into
// FP64 every MIX_FLUSH entries (ACC = 0) or kept as compensated FP32 sums (ACC = 1).
template <int ACC, bool ONE, int M, int NB>
__global__ void __launch_bounds__(CL_THREADS) k_force_cl(const DP P, int step_mode) {
    __shared__ double sh[32];
    __shared__ float4 shift[64];
    const int s = P.cblk_sys[blockIdx.x];
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    fill_shift_table(shift, sp);
    __syncthreads();
    const int c = P.cblk_first[blockIdx.x] + (int)threadIdx.x;
    const bool live = c < sp.cl0 + P.st[s].ncl;
    double etot = 0.0;
    if (live) {
        const uint32_t pk = (uint32_t)P.cl_atom[c];
        const int first = (int)(pk & JMASK), n = (int)(pk >> JBITS) + 1;
        const float4* __restrict__ prel = P.prel;
        const LJDev* tab0 = P.tab + sp.tab0;
        float mx[M], my[M], mz[M];
        const LJDev* tabm[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            if (m < n) {
                const float4 q = prel[first + m];
                mx[m] = q.x;
                my[m] = q.y;
                mz[m] = q.z;
                tabm[m] = tab0 + __float_as_int(q.w) * sp.nt;
            } else {
                mx[m] = my[m] = mz[m] = 1e18f;
                tabm[m] = tab0;
            }
        }
        const MixLJ P0 = mix_lj_load(tab0[0]);
        MixAcc<ACC> acc[M];
        const int nn = P.cl_nn[c];
        const uint32_t* __restrict__ nbp = P.cl_nbr + c;
        const uint32_t row = (uint32_t)P.clpad;
        const uint32_t pad = (uint32_t)first | (63u << JBITS);
        int since = 0;
        // list words of batch k0 + NB are loaded before batch k0 is evaluated, so the DRAM latency
        // of the list stream overlaps the pair arithmetic
        auto load_batch = [&](int k0, uint32_t (&e)[NB]) {
            const uint32_t q = (uint32_t)k0 * row;
            if (k0 + NB <= nn) {
#pragma unroll
                for (int b = 0; b < NB; ++b) e[b] = __ldg(nbp + q + (uint32_t)b * row);
            } else {
#pragma unroll
                for (int b = 0; b < NB; ++b) e[b] = (k0 + b < nn) ? __ldg(nbp + q + (uint32_t)b * row) : pad;
            }
        };
        uint32_t next[NB];
        load_batch(0, next);
        for (int k0 = 0; k0 < nn; k0 += NB) {
            uint32_t ent[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) ent[b] = next[b];
            if (k0 + NB < nn) load_batch(k0 + NB, next);
            float4 pj[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) pj[b] = __ldg(prel + (ent[b] & JMASK));
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                const float4 sv = shift[ent[b] >> JBITS];
                const float jx = pj[b].x + sv.x, jy = pj[b].y + sv.y, jz = pj[b].z + sv.z;
                const int tj = __float_as_int(pj[b].w);
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float dx = jx - mx[m], dy = jy - my[m], dz = jz - mz[m];
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    float frc2 = P0.frc2, fs2 = P0.fs2, fe24 = P0.fe24, fe4 = P0.fe4, fuc = P0.fuc;
                    if (!ONE) {
                        const LJDev& L = tabm[m][tj];
                        frc2 = L.present ? L.frc2 : -1.f;
                        fs2 = L.fsigma2;
                        fe24 = L.feps24;
                        fe4 = L.feps4;
                        fuc = L.fucut;
                    }
                    const bool in = r2 <= frc2 && r2 > 0.f;
                    const float inv = rcp_approx(r2);
                    const float s2 = fs2 * inv;
                    const float s6 = s2 * s2 * s2;
                    const float cf = in ? (s6 * fmaf(2.0f, s6, -1.0f)) * (fe24 * inv) : 0.f;
                    const float u = in ? fmaf(fe4, fmaf(s6, s6, -s6), -fuc) : 0.f;
                    acc[m].px = fmaf(-cf, dx, acc[m].px);
                    acc[m].py = fmaf(-cf, dy, acc[m].py);
                    acc[m].pz = fmaf(-cf, dz, acc[m].pz);
                    acc[m].pe += u;
                }
            }
            since += NB;
            if (since >= MIX_FLUSH) {
#pragma unroll
                for (int m = 0; m < M; ++m) acc[m].fold();
                since = 0;
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            acc[m].finish();
            if (m < n) {
                P.frc[first + m] = make_double4_32a(acc[m].fx, acc[m].fy, acc[m].fz, 0.0);
                etot += acc[m].e;
            }
        }
    }
    double tot = block_sum<CL_THREADS>(etot, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

// Forces over cluster lists, one lane per member: the M lanes of a cluster load the same list word
// and the same neighbour position (a broadcast), and each evaluates its own member with the
// per-atom kernel's arithmetic. A warp's gather then touches 32 / M addresses instead of 32, with
// the registers and per-lane work of the per-atom kernel; a member meets itself in the list
// (masked by r^2 > 0) and a padding lane of a short cluster idles. M blocks per cluster chunk.
template <int ACC, bool ONE, int M, int NB>
__global__ void __launch_bounds__(CL_THREADS) k_force_cl_lane(const DP P, int step_mode) {
    __shared__ double sh[32];
    __shared__ float4 shift[64];
    const int chunk = blockIdx.x / M, sub = blockIdx.x % M;
    const int s = P.cblk_sys[chunk];
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    fill_shift_table(shift, sp);
    __syncthreads();
    const int c = P.cblk_first[chunk] + sub * (CL_THREADS / M) + (int)threadIdx.x / M;
    const int m = (int)threadIdx.x % M;
    MixAcc<ACC> acc;
    if (c < sp.cl0 + P.st[s].ncl) {
        const uint32_t pk = (uint32_t)P.cl_atom[c];
        const int first = (int)(pk & JMASK), n = (int)(pk >> JBITS) + 1;
        const bool live = m < n;
        const float4* __restrict__ prel = P.prel;
        const float4 pi = live ? prel[first + m] : make_float4(1e18f, 1e18f, 1e18f, 0.f);
        const LJDev* tab = P.tab + sp.tab0 + (live ? __float_as_int(pi.w) : 0) * sp.nt;
        const MixLJ P0 = mix_lj_load(tab[0]);
        const int nn = P.cl_nn[c];
        const uint32_t* __restrict__ nbp = P.cl_nbr + c;
        const uint32_t row = (uint32_t)P.clpad;
        const uint32_t pad = (uint32_t)first | (63u << JBITS);
        int since = 0;
        for (int k0 = 0; k0 < nn; k0 += NB) {
            uint32_t ent[NB];
            const uint32_t q = (uint32_t)k0 * row;
            if (k0 + NB <= nn) {
#pragma unroll
                for (int b = 0; b < NB; ++b) ent[b] = load_list_word(nbp + q + (uint32_t)b * row);
            } else {
#pragma unroll
                for (int b = 0; b < NB; ++b) ent[b] = (k0 + b < nn) ? load_list_word(nbp + q + (uint32_t)b * row) : pad;
            }
            mixed_pairs<ONE, NB, ACC, true>(ent, prel, pi, shift, tab, P0, acc);
            since += NB;
            if (since >= MIX_FLUSH) {
                acc.fold();
                since = 0;
            }
        }
        acc.finish();
        if (live) P.frc[first + m] = make_double4_32a(acc.fx, acc.fy, acc.fz, 0.0);
    }
    double tot = block_sum<CL_THREADS>(acc.e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = tot;
}

// Exact cutoff test of every (member, entry) pair of one slot's cluster lists with the reference
// arithmetic (min-image, Vector3::norm, `> rcut`), for neighbour-set export: bit m of keep marks
// member m.
__global__ void __launch_bounds__(CL_THREADS) k_keep_cl(const DP P, int slot) {
    const int s = P.cblk_sys[blockIdx.x];
    if (s != slot) return;
    const SysParams& sp = P.sp[s];
    const int c = P.cblk_first[blockIdx.x] + (int)threadIdx.x;
    if (c >= sp.cl0 + P.st[s].ncl) return;
    const uint32_t pk = (uint32_t)P.cl_atom[c];
    const int first = (int)(pk & JMASK), n = (int)(pk >> JBITS) + 1;
    const int cur = P.st[s].cur;
    const double4_32a* pos = P.pos[cur];
    for (int k = 0; k < P.cl_nn[c]; ++k) {
        const int64_t q = (int64_t)k * P.clpad + c;
        const int j = (int)(P.cl_nbr[q] & JMASK);
        const double4_32a pj = pos[j];
        uint8_t mask = 0;
        for (int m = 0; m < n; ++m) {
            const int i = first + m;
            if (i == j) continue;
            const double4_32a pi = pos[i];
            const double rx = min_image_axis(__dsub_rn(pj.x, pi.x), sp.h[0], sp.hinv[0]);
            const double ry = min_image_axis(__dsub_rn(pj.y, pi.y), sp.h[1], sp.hinv[1]);
            const double rz = min_image_axis(__dsub_rn(pj.z, pi.z), sp.h[2], sp.hinv[2]);
            const LJDev& L = P.tab[sp.tab0 + type_of(pi.w) * sp.nt + type_of(pj.w)];
            if (L.present && !(sqrt(norm2_ref(rx, ry, rz)) > L.rcut)) mask |= (uint8_t)(1u << m);
        }
        P.keep[q] = mask;
    }
}

// Second half of verlet_step_nve (src/potentials/potential.rs:28-30):
// a_tdt = F/m; v += ((a_t + a_tdt) * 0.5) * dt; acc <- a_tdt (the next step's a_t); then chunk
// partials of KE = sum 0.5 m |v|^2 (src/atoms/properties.rs:17-24) and, on request,
// W = sum r_i F_i^T (:49-51). UPDATE = false only refreshes acc = F/m and reduces (after a
// force evaluation). EXACT keeps the reference's division and rounding order; the mixed path
// multiplies by the stored 1/m (acc.w) and fuses.
//
// The mixed path's arithmetic (a_tdt = F * (1/m) with 1/m stored in acc.w; v += (a_t + a_tdt) dt/2
// as one fused multiply-add per axis; m |v|^2 with m in vel.w) is shared by k_integrate2 and the
// fused step kernel, with explicit roundings so that both compile to the same operations.
__device__ __forceinline__ void accel_mixed(const double4_32a& f, double inv_m, double& bx, double& by,
                                            double& bz) {
    bx = __dmul_rn(f.x, inv_m);
    by = __dmul_rn(f.y, inv_m);
    bz = __dmul_rn(f.z, inv_m);
}
__device__ __forceinline__ void kick_mixed(const SysParams& sp, double4_32a& v, const double4_32a& a, double bx,
                                           double by, double bz) {
    v.x = fma(__dadd_rn(a.x, bx), sp.hdt, v.x);
    v.y = fma(__dadd_rn(a.y, by), sp.hdt, v.y);
    v.z = fma(__dadd_rn(a.z, bz), sp.hdt, v.z);
}
__device__ __forceinline__ double twice_ke_mixed(const double4_32a& v) {
    return __dmul_rn(v.w, fma(v.x, v.x, fma(v.y, v.y, __dmul_rn(v.z, v.z))));
}

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
            accel_mixed(f, a.w, bx, by, bz);
        }
        if (UPDATE) {
            if (EXACT) {
                v.x = __dadd_rn(v.x, __dmul_rn(__dmul_rn(__dadd_rn(a.x, bx), 0.5), sp.dt));
                v.y = __dadd_rn(v.y, __dmul_rn(__dmul_rn(__dadd_rn(a.y, by), 0.5), sp.dt));
                v.z = __dadd_rn(v.z, __dmul_rn(__dmul_rn(__dadd_rn(a.z, bz), 0.5), sp.dt));
            } else {
                kick_mixed(sp, v, a, bx, by, bz);
            }
            P.vel[cur][i] = v;
        }
        P.acc[cur][i] = make_double4_32a(bx, by, bz, a.w);
        // m |v|^2 here and the factor 1/2 on the block sum: halving is exact, so this equals the
        // sum of (0.5 m) |v|^2 (properties.rs:17-24) bit for bit
        ke = EXACT ? __dmul_rn(m, norm2_ref(v.x, v.y, v.z)) : twice_ke_mixed(v);
        if (st.want_virial) p = P.pos[cur][i];
    }
    double tot = block_sum<256>(ke, sh);
    if (threadIdx.x == 0) P.ke_part[blockIdx.x] = 0.5 * tot;
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

// One velocity-Verlet step of the mixed path in a single pass over the atoms (thread per atom):
// the forces of step t (k_force_mixed's arithmetic), the kick that ends step t (k_integrate2's),
// and, when DRIFT and the slot runs another step, the drift and skin test that start step t + 1
// (k_integrate1's). The drift and the kick are FP64 work that now overlaps the gather-bound pair
// loop of other warps (the FP64 pipe is otherwise nearly idle in the force kernel), and the
// separate passes over velocities, accelerations and positions disappear.
// Other threads are still gathering neighbour positions from P.prel when an atom drifts, so the
// new cell-relative coordinates go to the other buffer (P.prel_out); the step graph alternates
// the two buffers. A slot runs step t + 1 exactly when it drifted here, and the coordinates are a
// function of the FP64 state (the list build writes them, every drift rewrites them from the build
// snapshot), so nothing else ever reads a stale buffer. Results equal those of the three separate
// kernels bit for bit (same arithmetic, same block partial sums).
// Compiled for five resident blocks per SM with 4-entry batches (at most 51 registers; a few bytes
// of the FP64 epilogue spill) and four with 8-entry batches: the pair loop is latency-bound and
// needs the warps (measured on the 2.048M liquid: 4-entry batches 0.48 ms at five blocks, 0.56 ms at
// four, 0.64 ms unconstrained at 64-72 registers; 8-entry batches 0.55 ms at four, 0.60 at five).
template <int MIX_BATCH>
__host__ __device__ constexpr int step_min_blocks() {
    return MIX_BATCH == 4 ? 5 : 4;
}
// List rows prefetched into L2 this many gather batches ahead (measured on the 2.048M liquid:
// 4-entry batches 0.448 / 0.451 / 0.461 ms at 1 / 2 / 4 batches ahead, 0.481 without; 8-entry
// batches 0.495 / 0.499 / 0.481 ms, 0.547 without). The unfused force kernel gains nothing from it.
template <int MIX_BATCH>
__host__ __device__ constexpr int step_list_prefetch() {
    return MIX_BATCH == 4 ? 1 : 4;
}
template <int ACC, bool ONE, int MIX_BATCH, bool DRIFT>
__global__ void __launch_bounds__(256, step_min_blocks<MIX_BATCH>()) k_step_mixed(const DP P) {
    __shared__ double sh[32];
    __shared__ float shift[12];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, 1)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    fill_shift_axes(shift, sp);
    __syncthreads();
    MixAcc<ACC> acc;
    if (live)
        mixed_atom_forces<ACC, 1, ONE, MIX_BATCH, step_list_prefetch<MIX_BATCH>(), FUSED_LQ>(P, sp, i, 0, shift, acc);
    const bool drift = DRIFT && st.steps_left > 1;
    const bool want_virial = st.want_virial != 0;
    double ke = 0.0;
    double4_32a p = make_double4_32a(0.0, 0.0, 0.0, 0.0), f = p;
    if (live) {
        f = make_double4_32a(acc.fx, acc.fy, acc.fz, 0.0);
        P.frc[i] = f;
        const int cur = st.cur;
        double4_32a v = P.vel[cur][i];
        const double4_32a a = P.acc[cur][i];
        double bx, by, bz;
        accel_mixed(f, a.w, bx, by, bz);
        kick_mixed(sp, v, a, bx, by, bz);
        P.vel[cur][i] = v;
        P.acc[cur][i] = make_double4_32a(bx, by, bz, a.w);
        ke = twice_ke_mixed(v);
        if (want_virial || drift) p = P.pos[cur][i];
        if (drift) {
            double x, y, z;
            drift_mixed(sp, p, v, bx, by, bz, x, y, z);
            P.pos[cur][i] = make_double4_32a(x, y, z, p.w);
            double dx, dy, dz;
            skin_test(P, sp, st, i, x, y, z, dx, dy, dz);
            P.prel_out[i] = cell_relative_moved(P, i, dx, dy, dz);
        }
    }
    const double pe_tot = block_sum<256>(acc.e, sh);
    if (threadIdx.x == 0) P.pe_part[blockIdx.x] = pe_tot;
    const double ke_tot = block_sum<256>(ke, sh);
    if (threadIdx.x == 0) P.ke_part[blockIdx.x] = 0.5 * ke_tot;
    if (want_virial) {
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
    if (mode != 2) {
        if (P.cl_force) {  // cluster kernels: cl_lanes partials per cluster chunk
            const int L = P.cl_lanes;
            for (int c = threadIdx.x; c < sp.ncch * L; c += END_THREADS) pe += P.pe_part[(int64_t)sp.cch0 * L + c];
        }
        else
            for (int c = threadIdx.x; c < sp.nch * F; c += END_THREADS) pe += P.pe_part[(int64_t)sp.ch0 * F + c];
    }
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

// End of a rebuild phase (its last kernel, so every rebuild kernel has read the request flags):
// count and clear the rebuilt slots' flags and lower the device-wide request word. A drift that
// runs later in the same step (the fused step kernel) may raise them again for the next step.
__global__ void k_rebuild_done(const DP P, int step_mode) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) P.ctl[0] = 0;
    if (s >= P.max_slots || !P.sp[s].active) return;
    if (!slot_runs(P, s, step_mode)) return;
    SysState& st = P.st[s];
    if (st.rebuild) {
        st.rebuilds += 1;
        st.rebuild = 0;
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
    if (rebuild) {
        P.st[s].rebuild = 1;
        P.ctl[0] = 1;
    }
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
    const int L = P.lq;
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

// Condition of a step's rebuild node: some slot rebuilds in this step (the device-wide word).
// Also counts executed rebuild bodies (ctl[2..3], 64 bits) for the launch counter.
__global__ void k_set_rebuild_cond(const DP P, cudaGraphConditionalHandle h) {
    const bool go = P.ctl[0] != 0;
    cudaGraphSetConditional(h, go ? 1u : 0u);
    if (go) ++*reinterpret_cast<unsigned long long*>(P.ctl + 2);
}

// Upload of one slot's state. The caller's arrays (x,y,z per atom, 1-based types) are copied as
// they are into the slot's range of the idle buffer set (pos[1], vel[1], acc[1], id[1]: nothing
// lives there before the first rebuild) and converted here: type bits in pos.w, the type's mass in
// vel.w, a = 0 + F/m and 1/m in acc (the host arithmetic of Atoms::current_acceleration,
// src/atoms/properties.rs:32-39, with IEEE division), the build snapshot, original indices.
struct MassArg {
    double m[16];
};
__global__ void k_load_slot(const DP P, int64_t a0, int n, const MassArg masses, int has_vel, int has_force) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double* xs = reinterpret_cast<const double*>(P.pos[1] + a0);
    const double* vs = reinterpret_cast<const double*>(P.vel[1] + a0);
    const double* fs = reinterpret_cast<const double*>(P.acc[1] + a0);
    const int t0 = P.id[1][a0 + k] - 1;
    const double m = masses.m[t0];
    const double4_32a p = make_double4_32a(xs[3 * k], xs[3 * k + 1], xs[3 * k + 2], pack_type(t0));
    const double vx = has_vel ? vs[3 * k] : 0.0, vy = has_vel ? vs[3 * k + 1] : 0.0, vz = has_vel ? vs[3 * k + 2] : 0.0;
    const double fx = has_force ? fs[3 * k] : 0.0, fy = has_force ? fs[3 * k + 1] : 0.0,
                 fz = has_force ? fs[3 * k + 2] : 0.0;
    P.pos[0][a0 + k] = p;
    P.posb[a0 + k] = p;
    P.vel[0][a0 + k] = make_double4_32a(vx, vy, vz, m);
    P.frc[a0 + k] = make_double4_32a(fx, fy, fz, 0.0);
    P.acc[0][a0 + k] = make_double4_32a(__dadd_rn(0.0, __ddiv_rn(fx, m)), __dadd_rn(0.0, __ddiv_rn(fy, m)),
                                        __dadd_rn(0.0, __ddiv_rn(fz, m)), __ddiv_rn(1.0, m));
    P.id[0][a0 + k] = k;
}

// Download of one slot's state in the caller's atom order: the current arrays are un-permuted
// (device order -> original index) into x,y,z-per-atom staging in the idle buffer set, which the
// host then copies out in one transfer per array.
__global__ void k_store_slot(const DP P, int64_t a0, int n, int cur, int want_pos, int want_vel, int want_force) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int o = P.id[cur][a0 + k];
    if (want_pos) {
        const double4_32a v = P.pos[cur][a0 + k];
        double* out = reinterpret_cast<double*>(P.pos[cur ^ 1] + a0) + 3 * (int64_t)o;
        out[0] = v.x;
        out[1] = v.y;
        out[2] = v.z;
    }
    if (want_vel) {
        const double4_32a v = P.vel[cur][a0 + k];
        double* out = reinterpret_cast<double*>(P.vel[cur ^ 1] + a0) + 3 * (int64_t)o;
        out[0] = v.x;
        out[1] = v.y;
        out[2] = v.z;
    }
    if (want_force) {
        const double4_32a v = P.frc[a0 + k];
        double* out = reinterpret_cast<double*>(P.acc[cur ^ 1] + a0) + 3 * (int64_t)o;
        out[0] = v.x;
        out[1] = v.y;
        out[2] = v.z;
    }
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
#define LAUNCH(kern, grid, block, ...)                                \
    do {                                                               \
        kern<<<(grid), (block), 0, ls_>>>(__VA_ARGS__);               \
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
    if (side_) cudaStreamDestroy(side_);
    delete d_;
}

pis_status Engine::check(cudaError_t e, const char* what, std::string& err) {
    if (e == cudaSuccess) return PIS_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return PIS_ERR_NO_MEMORY;
    return PIS_ERR_CUDA;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }


static cudaError_t allow_all_mixed_tma_smem();

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
    if (opt.lpa != 1 && opt.lpa != 4 && opt.lpa != 8 && opt.lpa != 16 && opt.lpa != 32 &&
        !(opt.lpa == 2 && opt.cluster == 2)) {
        err = "lanes per atom must be 1, 4, 8, 16 or 32 (2 only with clusters of 2)";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    half_ = opt.list_kind == PIS_LIST_HALF ||
            (opt.list_kind == PIS_LIST_DEFAULT && opt.precision == PIS_PRECISION_FP64);
    if (opt.precision == PIS_PRECISION_MIXED && half_) {
        err = "the mixed-precision path uses a full list";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.list_tma && (opt.precision != PIS_PRECISION_MIXED || opt.lpa != 1)) {
        err = "the bulk-copy list stream is a variant of the mixed, thread-per-atom force kernel";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.list_tma) {
        pis_status st0 = check(allow_all_mixed_tma_smem(), "shared-memory attribute", err);
        if (st0) return st0;
    }
    if (opt.cell_tiles && (opt.precision != PIS_PRECISION_MIXED || opt.lpa != 1 || opt.list_tma || opt.cluster)) {
        err = "neighbour-cell tiles are a variant of the mixed, thread-per-atom force kernel";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.cell_tiles) {
        cudaError_t e = allow_tile_smem<0, true>();
        if (e == cudaSuccess) e = allow_tile_smem<0, false>();
        if (e == cudaSuccess) e = allow_tile_smem<1, true>();
        if (e == cudaSuccess) e = allow_tile_smem<1, false>();
        pis_status st0 = check(e, "shared-memory attribute", err);
        if (st0) return st0;
    }
    if (opt.cluster != 0 && opt.cluster != 2 && opt.cluster != 4) {
        err = "atoms per cluster must be 2 or 4";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    if (opt.cluster && (opt.precision != PIS_PRECISION_MIXED || (opt.lpa != 1 && opt.lpa != opt.cluster) ||
                        opt.list_tma)) {
        err = "the cluster list is a variant of the mixed path with one thread per cluster or one lane per member";
        return PIS_ERR_UNSUPPORTED;
    }
    if (opt.build_cluster != 0 && opt.build_cluster != 1 && opt.build_cluster != 2 && opt.build_cluster != 4) {
        err = "atoms per build cluster must be 1, 2 or 4";
        return PIS_ERR_INVALID_ARGUMENT;
    }
    // cluster table: built for the cluster-list force path, and for the per-atom list build when
    // it scans candidates per cluster (thread-per-atom layout only)
    clm_ = opt.cluster ? opt.cluster : ((opt.lpa == 1 && opt.build_cluster > 1) ? opt.build_cluster : 0);
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
    if (clm_) {
        // per slot: ceil(n / M) clusters plus at most one partial cluster per cell
        const int M = clm_;
        max_clusters_ = (opt.max_atoms + M - 1) / M + max_cells + opt.max_slots;
        clpad_ = (int64_t)align_up((size_t)max_clusters_, 32);
        // union of M members' lists: ~1.4x (M = 2) / ~1.9x (M = 4) one atom's list
        ccap_ = (int64_t)std::ceil((double)cap_ * (M == 2 ? 1.5 : 2.0));
        ccap_ = (ccap_ + 31) / 32 * 32;
        max_cchunks_ = (max_clusters_ + CL_THREADS - 1) / CL_THREADS + opt.max_slots;
        if ((double)clpad_ * (double)ccap_ >= 4294967296.0) {
            err = "cluster list of the pool exceeds 2^32 entries (clusters x capacity)";
            return PIS_ERR_NO_MEMORY;
        }
    }
    pis_status st = check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream", err);
    if (st) return st;
    st = check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "stream", err);
    if (st) return st;
    ls_ = stream_;
    // PIS_GPU_PLAIN_GRAPHS=1 in the environment selects plain step graphs for every pool of the
    // process (for profilers that cannot look inside graphs holding conditional nodes)
    const char* plain_env = std::getenv("PIS_GPU_PLAIN_GRAPHS");
    cond_rebuild_ = !opt.plain_graphs && !(plain_env && plain_env[0] && std::strcmp(plain_env, "0") != 0);

    const size_t NA = (size_t)opt.max_atoms, NC = (size_t)max_cells, NCH = (size_t)max_chunks_,
                 NS = (size_t)opt.max_slots, NCL = (size_t)max_clusters_, NCC = (size_t)max_cchunks_;
    // the per-atom list is not used (and kept minimal) when the cluster list is
    const size_t nbr_bytes = opt.cluster ? 256 : 4 * (size_t)npad_ * cap_;
    // the fused step kernel serves the mixed path's default shape (thread per atom, per-atom full
    // list, gathers from global memory, 4- or 8-entry batches)
    const bool default_shape = opt.precision == PIS_PRECISION_MIXED && opt.lpa == 1 && !opt.list_tma &&
                               !opt.cell_tiles && !opt.cluster && !clm_ && !half_ && opt.blk == 256;
    fused_ = default_shape && !opt.unfused && (opt.mix_batch == 4 || opt.mix_batch == 8);
    // grouped list layout wherever the thread-per-atom mixed force kernel reads the list
    list_groups_ = default_shape && opt.mix_batch % 4 == 0;
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
        {(void**)&d_->nn, 4 * NA},      {(void**)&d_->nbr, nbr_bytes},
        {(void**)&d_->cell_count, 4 * NC}, {(void**)&d_->cell_start, 4 * NC},
        {(void**)&d_->cell_sys, 4 * NC}, {(void**)&d_->blk_sys, 4 * NCH},
        {(void**)&d_->blk_first, 4 * NCH}, {(void**)&d_->sp, sizeof(SysParams) * NS},
        {(void**)&d_->st, sizeof(SysState) * NS}, {(void**)&d_->tab, sizeof(LJDev) * (size_t)opt.max_types_total},
        {(void**)&d_->pe_part, 8 * std::max(NCH * 32, NCC * 4)}, {(void**)&d_->ke_part, 8 * NCH},
        {(void**)&d_->vir_part, 72 * NCH}, {(void**)&d_->pe_hist, 8 * NS * (size_t)opt.hist},
        {(void**)&d_->ctl, 256},
    };
    if (fused_) items.push_back({&prel_buf_[1], 16 * NA});
    if (clm_) {
        items.push_back({(void**)&d_->cl_atom, 4 * NCL});
        items.push_back({(void**)&d_->cl_start, 4 * NC});
        items.push_back({(void**)&d_->cblk_sys, 4 * NCC});
        items.push_back({(void**)&d_->cblk_first, 4 * NCC});
    }
    if (clm_) {
        items.push_back({(void**)&d_->cl_nn, 4 * NCL});
        items.push_back({(void**)&d_->cl_nbr, 4 * (size_t)clpad_ * (size_t)ccap_});
    }
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
    d_->lq = opt_.lpa > 1 ? opt_.lpa : (list_groups_ ? FUSED_LQ : 1);
    d_->clpad = clpad_;
    d_->ccap = (int32_t)ccap_;
    d_->clm = clm_;
    d_->cl_force = opt.cluster ? 1 : 0;
    d_->cl_lanes = (opt.cluster && opt.lpa == opt.cluster) ? opt.cluster : 1;
    prel_buf_[0] = d_->prel;
    d_->prel_out = nullptr;
    st = check(cudaMemsetAsync(mem_, 0, total, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->cell_sys, 0xff, 4 * NC, stream_), "memset", err);
    if (st) return st;
    st = check(cudaMemsetAsync(d_->blk_sys, 0xff, 4 * NCH, stream_), "memset", err);
    if (st) return st;
    if (clm_) {
        st = check(cudaMemsetAsync(d_->cblk_sys, 0xff, 4 * NCC, stream_), "memset", err);
        if (st) return st;
    }
    hp_.assign(NS, SysParams{});
    slot_rlist_.assign(NS, 0.0);
    free_atoms_.clear();
    free_cells_.clear();
    free_atoms_[0] = NA;
    free_cells_[0] = NC;
    free_clusters_.clear();
    if (clm_) free_clusters_[0] = (int64_t)NCL;
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
    bool cl = true;
    if (clm_) {
        const int64_t need = (d.n + clm_ - 1) / clm_ + ncell;
        cl = false;
        for (auto& kv : free_clusters_) cl |= kv.second >= need;
    }
    return a && c && cl && slots > 0 && free_tab >= d.n_types * d.n_types;
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
    int64_t cl0 = 0, clcap = 0;
    if (clm_) {
        clcap = (d.n + clm_ - 1) / clm_ + ncell;
        if (!take_range(free_clusters_, clcap, cl0)) {
            give_range(free_atoms_, a0, d.n);
            give_range(free_cells_, c0, ncell + 1);
            err = "not enough free cluster capacity in the pool";
            return -PIS_ERR_NO_MEMORY;
        }
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
            if (clm_) give_range(free_clusters_, cl0, clcap);
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
        p.fsub[a] = (float)(4.0 / p.cs[a]);
    }
    p.half_skin2 = 0.25 * d.skin * d.skin;
    p.dt = d.dt;
    p.dt2 = d.dt * d.dt;
    p.hdt = 0.5 * p.dt;
    p.hdt2 = 0.5 * p.dt2;
    double rl = rlist * (1.0 + 1e-5);
    p.frlist2 = (float)(rl * rl);
    // The 27-cell walk (k_build1) serves axes of two cells too: there the -1 and +1 neighbours are
    // the same cell seen through two images, and the box edge (2 cells of at least the list radius)
    // exceeds twice the padded list radius, so at most one image of a pair passes the distance
    // test and no pair is listed twice. Only an edge within 1e-5 of that bound is left to the
    // generic walk, which keeps the nearer image per pair.
    p.walk27 = 1;
    for (int a = 0; a < 3; ++a)
        if (nc[a] < 2 || (nc[a] == 2 && !(p.h[a] > 2.0 * std::sqrt((double)p.frlist2) * (1.0 + 1e-5)))) p.walk27 = 0;
    // chunks
    p.nch = (int32_t)((d.n + opt_.blk - 1) / opt_.blk);
    p.ch0 = 0;  // assigned by the block map
    p.cl0 = (int32_t)cl0;
    p.clcap = (int32_t)clcap;
    p.ncch = (int32_t)((clcap + CL_THREADS - 1) / CL_THREADS);
    p.cch0 = 0;  // assigned by the block map
    hp_[slot] = p;
    slot_rlist_[slot] = rlist;

    // atom state: the caller's x,y,z-per-atom arrays and types go to the device as they are, and
    // k_load_slot builds the device layout
    if (nt > 16) {
        err = "at most 16 atom types per system";
        return -PIS_ERR_UNSUPPORTED;
    }
    MassArg ma;
    std::memset(&ma, 0, sizeof(ma));
    for (int t = 0; t < nt; ++t) ma.m[t] = d.masses[t];
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
    CP(d_->pos[1] + a0, pos, 24 * d.n);
    if (vel) CP(d_->vel[1] + a0, vel, 24 * d.n);
    if (force) CP(d_->acc[1] + a0, force, 24 * d.n);
    CP(d_->id[1] + a0, type_ids, 4 * d.n);
    LAUNCH(k_load_slot, (unsigned)((d.n + 255) / 256), 256, *d_, a0, (int)d.n, ma, vel ? 1 : 0, force ? 1 : 0);
    st = check(cudaGetLastError(), "upload", err);
    if (st) return -st;
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
    if (clm_) give_range(free_clusters_, p.cl0, p.clcap);
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
    // Slots with the most atoms per cell first: their list-build blocks walk the most candidates
    // per atom (small boxes have cells well above the list radius) and, scheduled last, were the
    // tail of every rebuild in a mixed pool. A slot's chunks stay consecutive, so its sums and
    // results do not depend on the order.
    std::vector<int> order;
    for (int s = 0; s < opt_.max_slots; ++s)
        if (hp_[s].active) order.push_back(s);
    auto per_cell = [&](int s) {
        const SysParams& p = hp_[s];
        return (double)p.n / ((double)p.nc[0] * p.nc[1] * p.nc[2]);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return per_cell(a) > per_cell(b); });
    int64_t c = 0;
    for (int s : order) {
        SysParams& p = hp_[s];
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
    // cluster kernels: every active slot gets ceil(cluster capacity / CL_THREADS) chunks
    std::vector<int32_t> cbs, cbf;
    if (clm_) {
        cbs.assign(max_cchunks_, -1);
        cbf.assign(max_cchunks_, 0);
        int64_t q = 0;
        for (int s = 0; s < opt_.max_slots; ++s) {
            SysParams& p = hp_[s];
            if (!p.active) continue;
            p.cch0 = (int32_t)q;
            for (int k = 0; k < p.ncch; ++k, ++q) {
                cbs[q] = s;
                cbf[q] = p.cl0 + k * CL_THREADS;
            }
        }
        st = check(cudaMemcpyAsync(d_->cblk_sys, cbs.data(), 4 * max_cchunks_, cudaMemcpyHostToDevice, stream_),
                   "block map", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(d_->cblk_first, cbf.data(), 4 * max_cchunks_, cudaMemcpyHostToDevice, stream_),
                   "block map", err);
        if (st) return st;
    }
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

pis_status Engine::sync(std::string& err) {
    pis_status st = check(cudaStreamSynchronize(stream_), "stream sync", err);
    if (!st) account_body_launches();
    return st;
}

pis_status Engine::set_dt(int slot, double dt, std::string& err) {
    SysParams& p = hp_[slot];
    if (p.dt == dt) return PIS_OK;
    p.dt = dt;
    p.dt2 = dt * dt;
    p.hdt = 0.5 * p.dt;
    p.hdt2 = 0.5 * p.dt2;
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
    const unsigned ga = (unsigned)max_chunks_;
    LAUNCH(k_bin, ga, opt_.blk, P, r);
    LAUNCH(k_scan, (unsigned)opt_.max_slots, SCAN_THREADS, P, r);
    LAUNCH(k_scatter, ga, opt_.blk, P, r);
    unsigned gcells = (unsigned)((opt_.max_cells * 32 + 255) / 256);
    LAUNCH(k_gather, gcells, 256, P, (int64_t)opt_.max_cells, r);
    launch_build(r);
    LAUNCH(k_rebuild_done, (unsigned)((opt_.max_slots + 127) / 128), 128, P, r);
}

// Lanes-per-atom kernels are templates; these dispatch on the pool's runtime choice. Their grid
// has lpa blocks per chunk.
// List build over `chunks` (L blocks per chunk for lanes-per-atom layouts).
template <int L>
static void launch_build_t(const DP& P, bool half, unsigned chunks, cudaStream_t st, int r) {
    const unsigned g = chunks * L;
    if (L == 1) {
        // lean kernel for slots with >= 3 cells per axis, generic kernel for the rest
        if (half) {
            k_build1<true><<<g, 256, 0, st>>>(P, r, 0);
            k_build1_generic<true><<<g, 256, 0, st>>>(P, r);
        } else {
            k_build1<false><<<g, 256, 0, st>>>(P, r, 0);
            k_build1_generic<false><<<g, 256, 0, st>>>(P, r);
        }
        g_launches.fetch_add(2);
        return;
    }
    if (half)
        k_build<true, L><<<g, 256, 0, st>>>(P, r);
    else
        k_build<false, L><<<g, 256, 0, st>>>(P, r);
    g_launches.fetch_add(1);
}

template <int L, int B>
static void launch_mixed_tb(const DP& P, bool kahan, bool one, unsigned chunks, cudaStream_t st, int r) {
    if (L == 1 && P.lq == FUSED_LQ) {  // the fused step's pools: FUSED_LQ-entry list groups
        if (kahan && one)
            k_force_mixed<1, 1, true, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else if (kahan)
            k_force_mixed<1, 1, false, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else if (one)
            k_force_mixed<0, 1, true, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        else
            k_force_mixed<0, 1, false, B, FUSED_LQ><<<chunks, 256, 0, st>>>(P, r);
        g_launches.fetch_add(1);
        return;
    }
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

template <int ACC, bool ONE, int M>
static void launch_cluster_t(const DP& P, int batch, bool lanes, unsigned chunks, cudaStream_t st, int r) {
    if (lanes) {
        if (batch >= 8)
            k_force_cl_lane<ACC, ONE, M, 8><<<chunks * M, CL_THREADS, 0, st>>>(P, r);
        else
            k_force_cl_lane<ACC, ONE, M, 4><<<chunks * M, CL_THREADS, 0, st>>>(P, r);
        return;
    }
    if (batch >= 8)
        k_force_cl<ACC, ONE, M, 8><<<chunks, CL_THREADS, 0, st>>>(P, r);
    else
        k_force_cl<ACC, ONE, M, 4><<<chunks, CL_THREADS, 0, st>>>(P, r);
}

template <int M>
static void launch_cluster_m(const DP& P, bool kahan, bool one, int batch, bool lanes, unsigned chunks, cudaStream_t st,
                             int r) {
    if (kahan)
        one ? launch_cluster_t<1, true, M>(P, batch, lanes, chunks, st, r)
            : launch_cluster_t<1, false, M>(P, batch, lanes, chunks, st, r);
    else
        one ? launch_cluster_t<0, true, M>(P, batch, lanes, chunks, st, r)
            : launch_cluster_t<0, false, M>(P, batch, lanes, chunks, st, r);
}

// Cluster-list forces: entries per batch = the batch knob (4 or 8); lanes per atom = M selects the
// lane-per-member kernel.
void Engine::launch_force_cluster(int r) {
    const unsigned ch = (unsigned)max_cchunks_;
    const bool lanes = opt_.lpa == opt_.cluster;
    if (opt_.cluster == 2)
        launch_cluster_m<2>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, lanes, ch, stream_, r);
    else
        launch_cluster_m<4>(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, lanes, ch, stream_, r);
    g_launches.fetch_add(1);
}

void Engine::launch_build(int r) {
    const unsigned ch = (unsigned)max_chunks_;
    const unsigned gc = (unsigned)max_cchunks_, ga = (unsigned)max_chunks_;
    if (opt_.cluster) {
        if (opt_.cluster == 2)
            k_build_cl<2><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 0);
        else
            k_build_cl<4><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 0);
        g_launches.fetch_add(1);
        return;
    }
    if (clm_ && opt_.lpa == 1) {
        // two-stage per-atom build: cluster union lists, filtered per member; slots with a
        // two-cell axis use the 27-cell walk (or, at the two-cell edge bound, the generic kernel)
        if (clm_ == 2) {
            k_build_cl<2><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 1);
            if (half_)
                k_filter_cl<true, 2><<<gc * 2, CL_THREADS, 0, ls_>>>(*d_, r);
            else
                k_filter_cl<false, 2><<<gc * 2, CL_THREADS, 0, ls_>>>(*d_, r);
        } else {
            k_build_cl<4><<<gc, CL_THREADS, 0, ls_>>>(*d_, r, 1);
            if (half_)
                k_filter_cl<true, 4><<<gc * 4, CL_THREADS, 0, ls_>>>(*d_, r);
            else
                k_filter_cl<false, 4><<<gc * 4, CL_THREADS, 0, ls_>>>(*d_, r);
        }
        if (half_) {
            k_build1<true><<<ga, 256, 0, ls_>>>(*d_, r, 1);
            k_build1_generic<true><<<ga, 256, 0, ls_>>>(*d_, r);
        } else {
            k_build1<false><<<ga, 256, 0, ls_>>>(*d_, r, 1);
            k_build1_generic<false><<<ga, 256, 0, ls_>>>(*d_, r);
        }
        g_launches.fetch_add(4);
        return;
    }
#define PIS_CALL(L) launch_build_t<L>(*d_, half_, ch, ls_, r)
    PIS_LPA_DISPATCH(opt_.lpa, PIS_CALL)
#undef PIS_CALL
}

template <int ACC, bool ONE, int KB>
static void launch_mixed_tma_t(const DP& P, unsigned chunks, cudaStream_t st, int r) {
    k_force_mixed_tma<ACC, ONE, KB><<<chunks, 256, mix_tma_smem_bytes<KB>(), st>>>(P, r);
}

// Bulk-copy-fed variant: rows per stage = the batch knob (8 or 16).
static void launch_mixed_tma(const DP& P, bool kahan, bool one, int batch, unsigned chunks, cudaStream_t st, int r) {
    const bool b16 = batch == 16;
    if (kahan) {
        if (one)
            b16 ? launch_mixed_tma_t<1, true, 16>(P, chunks, st, r) : launch_mixed_tma_t<1, true, 8>(P, chunks, st, r);
        else
            b16 ? launch_mixed_tma_t<1, false, 16>(P, chunks, st, r) : launch_mixed_tma_t<1, false, 8>(P, chunks, st, r);
    } else {
        if (one)
            b16 ? launch_mixed_tma_t<0, true, 16>(P, chunks, st, r) : launch_mixed_tma_t<0, true, 8>(P, chunks, st, r);
        else
            b16 ? launch_mixed_tma_t<0, false, 16>(P, chunks, st, r) : launch_mixed_tma_t<0, false, 8>(P, chunks, st, r);
    }
    g_launches.fetch_add(1);
}

// Dynamic shared memory of the bulk-copy-fed kernels (the 16-row ring exceeds the 48 KB default).
template <int ACC, bool ONE, int KB>
static cudaError_t allow_mixed_tma_smem() {
    return cudaFuncSetAttribute(k_force_mixed_tma<ACC, ONE, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mix_tma_smem_bytes<KB>());
}

static cudaError_t allow_all_mixed_tma_smem() {
    cudaError_t e = cudaSuccess, q;
    if ((q = allow_mixed_tma_smem<0, true, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, true, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, false, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<0, false, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, true, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, true, 16>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, false, 8>()) != cudaSuccess) e = q;
    if ((q = allow_mixed_tma_smem<1, false, 16>()) != cudaSuccess) e = q;
    return e;
}

void Engine::launch_force_mixed(int r) {
    const unsigned ch = (unsigned)max_chunks_;
    if (opt_.cluster) {
        launch_force_cluster(r);
        return;
    }
    if (opt_.cell_tiles) {
        const size_t smem = TILE_ATOMS * sizeof(float4);
        if (opt_.mixed_kahan)
            single_type_ ? k_force_mixed_tile<1, true><<<ch, 256, smem, stream_>>>(*d_, r)
                         : k_force_mixed_tile<1, false><<<ch, 256, smem, stream_>>>(*d_, r);
        else
            single_type_ ? k_force_mixed_tile<0, true><<<ch, 256, smem, stream_>>>(*d_, r)
                         : k_force_mixed_tile<0, false><<<ch, 256, smem, stream_>>>(*d_, r);
        g_launches.fetch_add(1);
        return;
    }
    if (opt_.list_tma && opt_.lpa == 1) {
        launch_mixed_tma(*d_, opt_.mixed_kahan, single_type_, opt_.mix_batch, ch, stream_, r);
        return;
    }
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

// Step q of a g-step graph. Unfused: drift, rebuild, forces, kick, step end. Fused (mixed path,
// default kernel shape): the graph's first step drifts alone, every step then runs rebuild, the
// fused forces + kick + next drift (no drift in the graph's last step), step end; step q reads
// cell-relative coordinates from buffer q & 1 (its list rebuild writes them there) and the drift
// writes the other.
void Engine::enqueue_step(bool respect, cudaEvent_t* ev, int64_t q, int64_t g) {
    const DP& P = *d_;
    int r = respect ? 1 : 0;
    const bool mixed = opt_.precision == PIS_PRECISION_MIXED;
    const bool fused = mixed && fused_;
    if (ev) cudaEventRecordWithFlags(ev[0], stream_, cudaEventRecordExternal);
    if (!fused || q == 0) {
        if (mixed)
            LAUNCH(k_integrate1<true>, (unsigned)max_chunks_, opt_.blk, P);
        else
            LAUNCH(k_integrate1<false>, (unsigned)max_chunks_, opt_.blk, P);
    }
    if (ev) cudaEventRecordWithFlags(ev[1], stream_, cudaEventRecordExternal);
    if (fused) {
        d_->prel = (float4*)prel_buf_[q & 1];
        d_->prel_out = (float4*)prel_buf_[(q + 1) & 1];
    }
    if (cond_step_)
        cond_error_ = cond_error_ ? cond_error_ : enqueue_rebuild_conditional(respect);
    else
        enqueue_rebuild(respect);
    if (ev) cudaEventRecordWithFlags(ev[2], stream_, cudaEventRecordExternal);
    if (fused)
        launch_step_mixed(q + 1 < g);
    else if (mixed)
        launch_force_mixed(r);
    else
        launch_force_fp64(r);
    if (ev) cudaEventRecordWithFlags(ev[3], stream_, cudaEventRecordExternal);
    if (!fused) {
        if (mixed)
            LAUNCH((k_integrate2<true, false>), (unsigned)max_chunks_, opt_.blk, P, r);
        else
            LAUNCH((k_integrate2<true, true>), (unsigned)max_chunks_, opt_.blk, P, r);
    }
    if (ev) cudaEventRecordWithFlags(ev[4], stream_, cudaEventRecordExternal);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 0);
    if (ev) cudaEventRecordWithFlags(ev[5], stream_, cudaEventRecordExternal);
    if (fused) {
        d_->prel = (float4*)prel_buf_[0];
        d_->prel_out = nullptr;
    }
}

template <int ACC, bool ONE, int B>
static void launch_step_mixed_t(const DP& P, bool drift, unsigned chunks, cudaStream_t st) {
    if (drift)
        k_step_mixed<ACC, ONE, B, true><<<chunks, 256, 0, st>>>(P);
    else
        k_step_mixed<ACC, ONE, B, false><<<chunks, 256, 0, st>>>(P);
}

void Engine::launch_step_mixed(bool drift) {
    const unsigned ch = (unsigned)max_chunks_;
    const bool b8 = opt_.mix_batch == 8;
    if (opt_.mixed_kahan) {
        if (single_type_)
            b8 ? launch_step_mixed_t<1, true, 8>(*d_, drift, ch, stream_)
               : launch_step_mixed_t<1, true, 4>(*d_, drift, ch, stream_);
        else
            b8 ? launch_step_mixed_t<1, false, 8>(*d_, drift, ch, stream_)
               : launch_step_mixed_t<1, false, 4>(*d_, drift, ch, stream_);
    } else {
        if (single_type_)
            b8 ? launch_step_mixed_t<0, true, 8>(*d_, drift, ch, stream_)
               : launch_step_mixed_t<0, true, 4>(*d_, drift, ch, stream_);
        else
            b8 ? launch_step_mixed_t<0, false, 8>(*d_, drift, ch, stream_)
               : launch_step_mixed_t<0, false, 4>(*d_, drift, ch, stream_);
    }
    g_launches.fetch_add(1);
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

// Inside a stream capture of stream_: a 1-thread kernel sets the condition from the rebuild word,
// then a conditional IF node whose body (the rebuild kernels, captured on side_) runs only when
// some slot rebuilds. On the ~8 steps in 9 without a rebuild the step then launches no rebuild
// kernel at all.
pis_status Engine::enqueue_rebuild_conditional(bool respect) {
    cudaStreamCaptureStatus cs;
    unsigned long long id = 0;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(stream_, &cs, &id, &g, &deps, &edges, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return PIS_ERR_CUDA;
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return PIS_ERR_CUDA;
    k_set_rebuild_cond<<<1, 1, 0, stream_>>>(*d_, h);
    g_launches.fetch_add(1);
    if (cudaStreamGetCaptureInfo(stream_, &cs, &id, &g, &deps, &edges, &nd) != cudaSuccess) return PIS_ERR_CUDA;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, g, deps, edges, nd, &cp) != cudaSuccess) return PIS_ERR_CUDA;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (cudaStreamUpdateCaptureDependencies(stream_, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
        return PIS_ERR_CUDA;
    if (cudaStreamBeginCaptureToGraph(side_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return PIS_ERR_CUDA;
    const int64_t before = g_launches.load();
    ls_ = side_;
    enqueue_rebuild(respect);
    ls_ = stream_;
    const int64_t n_body = g_launches.load() - before;
    g_launches.fetch_sub(n_body);  // counted when a body actually runs (account_body_launches)
    body_kernels_ = n_body;
    cudaGraph_t out = nullptr;
    if (cudaStreamEndCapture(side_, &out) != cudaSuccess) return PIS_ERR_CUDA;
    return PIS_OK;
}

void Engine::account_body_launches() {
    if (!body_kernels_ || !d_) return;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, d_->ctl + 2, sizeof(n), cudaMemcpyDeviceToHost) != cudaSuccess) return;
    if (n > body_seen_) {
        g_launches.fetch_add((int64_t)(n - body_seen_) * body_kernels_);
        body_seen_ = n;
    }
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

// Force evaluation and reductions for a set of slots (each marked, then one kernel sequence for
// all): the serving loop evaluates the jobs it admits between two graphs together. Every slot's
// results are those of compute_potential_slot on it alone.
pis_status Engine::compute_potential_slots(const std::vector<int>& slots, std::string& err) {
    if (slots.empty()) return PIS_OK;
    pis_status st = rebuild_block_map(err);
    if (st) return st;
    const DP& P = *d_;
    const unsigned sg = (unsigned)((opt_.max_slots + 127) / 128);
    for (int s : slots) LAUNCH(k_mark_eval, sg, 128, P, s, 1, 0);
    LAUNCH(k_zero_forces, (unsigned)max_chunks_, opt_.blk, P);
    enqueue_rebuild(false);
    if (opt_.precision == PIS_PRECISION_MIXED)
        launch_force_mixed(0);
    else
        launch_force_fp64(0);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 1);
    for (int s : slots) LAUNCH(k_mark_eval, sg, 128, P, s, 0, 1);
    if (opt_.precision == PIS_PRECISION_MIXED)
        LAUNCH((k_integrate2<false, false>), (unsigned)max_chunks_, opt_.blk, P, 0);
    else
        LAUNCH((k_integrate2<false, true>), (unsigned)max_chunks_, opt_.blk, P, 0);
    LAUNCH(k_step_end, (unsigned)opt_.max_slots, END_THREADS, P, 2);
    st = check(cudaGetLastError(), "launch", err);
    if (st) return st;
    return sync(err);
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
            cudaGraph_t graph = nullptr;
            for (int attempt = 0; attempt < 2; ++attempt) {
                st = check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture", err);
                if (st) return st;
                int64_t before = g_launches.load();
                cond_step_ = cond_rebuild_;
                cond_error_ = PIS_OK;
                for (int64_t q = 0; q < g; ++q)
                    enqueue_step(true, instrument_ ? rec.ev.data() + 6 * q : nullptr, q, g);
                cond_step_ = false;
                int64_t captured = g_launches.load() - before;
                g_launches.fetch_sub(captured);
                rec.kernels = captured;
                kernels_per_step_ = captured / g;
                cudaError_t ce = cudaStreamEndCapture(stream_, &graph);
                if (ce == cudaSuccess && cond_error_ == PIS_OK) {
                    ce = cudaGraphInstantiate(&rec.exec, graph, 0);
                    cudaGraphDestroy(graph);
                    if (ce == cudaSuccess) break;
                } else if (graph) {
                    cudaGraphDestroy(graph);
                }
                graph = nullptr;
                cudaGetLastError();
                if (!cond_rebuild_) return check(ce == cudaSuccess ? cudaErrorUnknown : ce, "capture", err);
                // conditional nodes unavailable: capture the plain step sequence instead
                cond_rebuild_ = false;
                body_kernels_ = 0;
            }
            it = graphs_.emplace(key, rec).first;
        }
        st = check(cudaGraphLaunch(it->second.exec, stream_), "graph launch", err);
        if (st) return st;
        g_launches.fetch_add(it->second.kernels);
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
    if (!pos && !vel && !force) return PIS_OK;
    const int cur = ss.cur;
    LAUNCH(k_store_slot, (unsigned)((p.n + 255) / 256), 256, *d_, p.a0, p.n, cur, pos ? 1 : 0, vel ? 1 : 0,
           force ? 1 : 0);
    st = check(cudaGetLastError(), "download", err);
    if (st) return st;
    const size_t bytes = 24 * (size_t)p.n;
    if (pos) {
        st = check(cudaMemcpyAsync(pos, d_->pos[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (vel) {
        st = check(cudaMemcpyAsync(vel, d_->vel[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    if (force) {
        st = check(cudaMemcpyAsync(force, d_->acc[cur ^ 1] + p.a0, bytes, cudaMemcpyDeviceToHost, stream_), "download", err);
        if (st) return st;
    }
    return sync(err);
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
    if (opt_.cluster) {
        SysState ss;
        pis_status st = read_state(slot, ss, err);
        if (st) return st;
        std::vector<int32_t> nn(ss.ncl);
        st = check(cudaMemcpyAsync(nn.data(), d_->cl_nn + p.cl0, 4 * (size_t)ss.ncl, cudaMemcpyDeviceToHost, stream_),
                   "nn", err);
        if (st) return st;
        st = sync(err);
        if (st) return st;
        total = 0;
        for (int32_t v : nn) total += v;
        return PIS_OK;
    }
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
    if (opt_.cluster) return neighbour_sets_cluster(slot, ss, offsets, idx, err);
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
    const int L = d_->lq;
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

// Per-atom sets from the cluster lists: every (member, entry) pair that passes the exact cutoff
// test, in original indices, sorted; an atom listed under two images (two-cell axes) counts once.
pis_status Engine::neighbour_sets_cluster(int slot, const SysState& ss, std::vector<int64_t>& offsets,
                                          std::vector<int32_t>& idx, std::string& err) {
    const SysParams& p = hp_[slot];
    pis_status st;
    if (!d_->keep) {
        st = check(cudaMalloc(&d_->keep, (size_t)clpad_ * ccap_), "keep mask", err);
        if (st) return st;
    }
    LAUNCH(k_keep_cl, (unsigned)max_cchunks_, CL_THREADS, *d_, slot);
    st = check(cudaGetLastError(), "keep", err);
    if (st) return st;
    const size_t ncl = (size_t)ss.ncl;
    std::vector<int32_t> atom(ncl), nn(ncl), id(p.n);
    st = check(cudaMemcpyAsync(atom.data(), d_->cl_atom + p.cl0, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "clusters", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(nn.data(), d_->cl_nn + p.cl0, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "nn", err);
    if (st) return st;
    st = check(cudaMemcpyAsync(id.data(), d_->id[ss.cur] + p.a0, 4 * (size_t)p.n, cudaMemcpyDeviceToHost, stream_), "id", err);
    if (st) return st;
    st = sync(err);
    if (st) return st;
    int32_t maxnn = 0;
    for (int32_t v : nn) maxnn = std::max(maxnn, v);
    std::vector<uint32_t> ent((size_t)maxnn * ncl);
    std::vector<uint8_t> kp((size_t)maxnn * ncl);
    for (int r = 0; r < maxnn; ++r) {
        const int64_t off = (int64_t)r * clpad_ + p.cl0;
        st = check(cudaMemcpyAsync(ent.data() + r * ncl, d_->cl_nbr + off, 4 * ncl, cudaMemcpyDeviceToHost, stream_), "nbr", err);
        if (st) return st;
        st = check(cudaMemcpyAsync(kp.data() + r * ncl, d_->keep + off, ncl, cudaMemcpyDeviceToHost, stream_), "keep", err);
        if (st) return st;
    }
    st = sync(err);
    if (st) return st;
    std::vector<std::vector<int32_t>> sets(p.n);
    for (size_t c = 0; c < ncl; ++c) {
        const uint32_t pk = (uint32_t)atom[c];
        const int first = (int)(pk & JMASK) - (int)p.a0, n = (int)(pk >> JBITS) + 1;
        for (int k = 0; k < nn[c]; ++k) {
            const uint8_t mask = kp[(size_t)k * ncl + c];
            if (!mask) continue;
            const int j = (int)(ent[(size_t)k * ncl + c] & JMASK) - (int)p.a0;
            for (int m = 0; m < n; ++m)
                if (mask & (1u << m)) sets[id[first + m]].push_back(id[j]);
        }
    }
    offsets.assign(p.n + 1, 0);
    idx.clear();
    for (int i = 0; i < p.n; ++i) {
        std::sort(sets[i].begin(), sets[i].end());
        sets[i].erase(std::unique(sets[i].begin(), sets[i].end()), sets[i].end());
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
        p.fsub[a] = (float)(4.0 / p.cs[a]);
    }
    p.hinv[0] = (p.h[1] * p.h[2]) / (p.h[0] * (p.h[1] * p.h[2]));
    p.hinv[1] = (p.h[0] * p.h[2]) / (p.h[0] * (p.h[1] * p.h[2]));
    p.hinv[2] = (p.h[0] * p.h[1]) / (p.h[0] * (p.h[1] * p.h[2]));
    for (int a = 0; a < 3; ++a)
        if (p.cs[a] < rl) {
            err = "box shrank below the cell size; re-create the state to re-grid";
            return PIS_ERR_UNSUPPORTED;
        }
    // the 27-cell walk's two-cell condition (add_slot) for the new edges
    p.walk27 = 1;
    for (int a = 0; a < 3; ++a)
        if (p.nc[a] < 2 || (p.nc[a] == 2 && !(p.h[a] > 2.0 * std::sqrt((double)p.frlist2) * (1.0 + 1e-5)))) p.walk27 = 0;
    pis_status st = check(cudaMemcpyAsync(d_->sp + slot, &p, sizeof(SysParams), cudaMemcpyHostToDevice, stream_), "params", err);
    if (st) return st;
    int32_t one = 1;
    st = check(cudaMemcpyAsync(&d_->st[slot].rebuild, &one, 4, cudaMemcpyHostToDevice, stream_), "params", err);
    if (st) return st;
    return sync(err);
}

}  // namespace pis
