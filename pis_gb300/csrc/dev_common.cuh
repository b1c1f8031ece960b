// dev_common.cuh - Device side of the engine, part 1: constants, the device pointer bundle, and the helpers the
// kernels share (type packing, min-image and wrap arithmetic, block sums, list-word loads, the
// approximate reciprocal, mbarrier and bulk-copy primitives, block-to-atom maps).
// Included by engine.cu, in this order: dev_common.cuh, dev_step.cuh, dev_cluster.cuh,
// dev_step_end.cuh.
#pragma once

#include "xsum.cuh"

namespace pis {

constexpr int JBITS = 26;                  // atom-index bits of a neighbour entry
constexpr uint32_t JMASK = (1u << JBITS) - 1u;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_SEG = SCAN_THREADS * SCAN_ITEMS;  // cells per block of the segmented scan
constexpr int RING_STEPS = 64;  // longest graph of fused steps (rows of the partial ring)
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
    double* ke_hist;      // per-slot rings beside pe_hist: kinetic energy of every step
    double* tr_hist;      // and the virial trace of every step run with the slot's thermo flag set
    double* tr_part;      // chunk partials of the virial trace
    long long* xtr_part;  // FP64 pools: the same as exact-sum partials
    double* kt_part;      // chunk partials of the kinetic tensor sum_i v_i v_i^T (9 per chunk)
    long long* xkt_part;  // FP64 pools: the same as exact-sum partials
    uint32_t wait_limit;  // polls of a bulk-copy pipeline wait before it expires
    int64_t npad;
    int32_t cap;
    int32_t hist;
    int32_t max_slots;
    int32_t zero_forces;  // half list: integrate1 clears F for the atomic scatter
    int2* seg_tot;        // segmented cell scan: per slot and segment, (atoms, clusters) in the segment
    double* ring;         // fused steps: per step of a graph, PE, KE and trace block partials
    int64_t ring_stride;  // partials per quantity and step (the chunk count)
    int32_t max_segs;     // segments per slot in seg_tot
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
    int32_t* ctl;         // ctl[0]: some slot rebuilds its list in the current step or evaluation;
                          // ctl[8], ctl[9]: listed chunks and cells of the rebuilding slots
    int32_t* rb_list;     // listed rebuild: chunk ids, then (from rb_cells_off) cell entries
    int64_t rb_cells_off;
    // fused step: cell-relative coordinates of the drifted atoms go to prel_out (the buffer the next
    // step reads)
    float4* prel_out;
    // FP64 pools: energy, kinetic energy and virial as exact sums (XS_WORDS words per block partial;
    // the virial's nine components one after another)
    int32_t exact_sums;
    long long* xpe_part;
    long long* xke_part;
    long long* xvir_part;
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

// General (triclinic) boxes, FP64 path: the reference's own 3x3 arithmetic. A matrix-vector
// product sums each row left to right without fused multiply-adds (nalgebra, as the reference's
// SimulationBox uses it); m is row-major.
__device__ __forceinline__ void matvec_ref(const double* m, double x, double y, double z, double& a, double& b,
                                           double& c) {
    a = __dadd_rn(__dadd_rn(__dmul_rn(m[0], x), __dmul_rn(m[1], y)), __dmul_rn(m[2], z));
    b = __dadd_rn(__dadd_rn(__dmul_rn(m[3], x), __dmul_rn(m[4], y)), __dmul_rn(m[5], z));
    c = __dadd_rn(__dadd_rn(__dmul_rn(m[6], x), __dmul_rn(m[7], y)), __dmul_rn(m[8], z));
}
// SimulationBox::apply_boundary_conditions_dis (src/simulation_box.rs:17-27): s = h^-1 r,
// s -= round(s), r = h s (rint for round: they differ only at |s| = 1/2, beyond every cutoff).
__device__ __forceinline__ void min_image_full(const double* H, const double* HI, double& x, double& y, double& z) {
    double s0, s1, s2;
    matvec_ref(HI, x, y, z, s0, s1, s2);
    s0 = __dsub_rn(s0, rint(s0));
    s1 = __dsub_rn(s1, rint(s1));
    s2 = __dsub_rn(s2, rint(s2));
    matvec_ref(H, s0, s1, s2, x, y, z);
}
// SimulationBox::apply_boundary_conditions_pos (src/simulation_box.rs:29-42): s -= floor(s).
__device__ __forceinline__ void wrap_full(const double* H, const double* HI, double& x, double& y, double& z) {
    double s0, s1, s2;
    matvec_ref(HI, x, y, z, s0, s1, s2);
    s0 = __dsub_rn(s0, floor(s0));
    s1 = __dsub_rn(s1, floor(s1));
    s2 = __dsub_rn(s2, floor(s2));
    matvec_ref(H, s0, s1, s2, x, y, z);
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
// The same with a caller-given poll budget: the pipelines' waits take the pool's budget
// (DevPtrs::wait_limit, MBAR_WAIT_LIMIT unless a test lowers it to make the expiry path run on a
// correct kernel); the final wait for a block's own copies in flight always takes the full one.
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
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

// Step mode (1 + q for step q of a graph whose step counters are updated at the graph's end, 1
// where they are updated after every step): slots with more than q steps left take part.
// Evaluation mode (0): only slots the host marked for a force evaluation or reduction.
__device__ __forceinline__ bool slot_runs(const DP& P, int s, int step_mode) {
    return step_mode ? P.st[s].steps_left > step_mode - 1 : P.st[s].eval != 0;
}

// TRIC = false: the instantiation for pools without triclinic slots (the general branch costs the
// cell sort registers).
template <bool TRIC = true>
__device__ __forceinline__ float4 cell_relative(const SysParams& sp, double4_32a p, int lc, int type) {
    int cx = lc % sp.nc[0];
    int cy = (lc / sp.nc[0]) % sp.nc[1];
    int cz = lc / (sp.nc[0] * sp.nc[1]);
    if (TRIC && sp.tric) {  // position relative to the cell centre H ((c + 1/2) / n), minimum image
        double x, y, z;
        matvec_ref(sp.H, (cx + 0.5) / sp.nc[0], (cy + 0.5) / sp.nc[1], (cz + 0.5) / sp.nc[2], x, y, z);
        x = p.x - x;
        y = p.y - y;
        z = p.z - z;
        min_image_full(sp.H, sp.HI, x, y, z);
        return make_float4((float)x, (float)y, (float)z, __int_as_float(type));
    }
    // the offset from the cell centre in FP64 (one fused multiply-add and one subtraction per axis),
    // then in FP32: rounded and scaled to units of the x cell edge (SysParams::sc) by 1/sc as the
    // sum of two floats. The minimum image applies only to a position on the upper box face binned
    // into cell 0 (an atom binned from its own position lies within half a cell of the centre).
    double d[3] = {p.x - fma((double)cx, sp.cs[0], 0.5 * sp.cs[0]), p.y - fma((double)cy, sp.cs[1], 0.5 * sp.cs[1]),
                   p.z - fma((double)cz, sp.cs[2], 0.5 * sp.cs[2])};
    float q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = (float)d[a];
        q[a] = fmaf(f, sp.fisc_lo, f * sp.fisc_hi);
        if (fabsf(q[a]) > 0.75f * sp.fcs[a]) {
            f = (float)(d[a] - sp.h[a] * rint(d[a] * sp.hinv[a]));
            q[a] = fmaf(f, sp.fisc_lo, f * sp.fisc_hi);
        }
    }
    return make_float4(q[0], q[1], q[2], __int_as_float(type));
}

}  // namespace pis
