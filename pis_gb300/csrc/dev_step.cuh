// dev_step.cuh - Device side of the engine, part 2: the per-atom step kernels - drift (k_integrate1), the
// neighbour-list rebuild (bin, scan, scatter, gather, build) and the force kernels (FP64, mixed,
// and their variants: lanes per atom, bulk-copied list stream, cell tiles).
// Included by engine.cu, in this order: dev_common.cuh, dev_step.cuh, dev_cluster.cuh,
// dev_step_end.cuh.
#pragma once

namespace pis {

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
        if (sp.tric) {
            min_image_full(sp.H, sp.HI, dx, dy, dz);
        } else {
            dx = min_image_axis(dx, sp.h[0], sp.hinv[0]);
            dy = min_image_axis(dy, sp.h[1], sp.hinv[1]);
            dz = min_image_axis(dz, sp.h[2], sp.hinv[2]);
        }
        d2 = fma(dx, dx, fma(dy, dy, dz * dz));
        if (!(d2 <= sp.half_skin2)) {  // NaN also requests a rebuild
            st.rebuild = 1;
            P.ctl[0] = 1;
        }
        if (x != x || y != y || z != z) atomicOr(&st.flags, FLAG_NAN);
    }
}
// cell-relative FP32 coordinates = build-time ones + displacement since the build, in units of
// the slot's x cell edge (SysParams::sc); the displacement (below the skin) is scaled in FP32 by
// 1/sc as the sum of two floats, so the scale carries no FP32 rounding of its own
__device__ __forceinline__ float scaled_step(float d, const SysParams& sp) {
    return fmaf(d, sp.fisc_lo, d * sp.fisc_hi);
}
__device__ __forceinline__ float4 cell_relative_moved(const DP& P, const SysParams& sp, int i, double dx, double dy,
                                                      double dz) {
    const float4 q = P.prelb[i];
    return make_float4(q.x + scaled_step((float)dx, sp), q.y + scaled_step((float)dy, sp),
                       q.z + scaled_step((float)dz, sp), q.w);
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
        if (sp.tric) {
            wrap_full(sp.H, sp.HI, x, y, z);
        } else {
            x = wrap_axis(x, sp.h[0], sp.hinv[0]);
            y = wrap_axis(y, sp.h[1], sp.hinv[1]);
            z = wrap_axis(z, sp.h[2], sp.hinv[2]);
        }
    } else {
        drift_mixed(sp, p, v, a.x, a.y, a.z, x, y, z);
    }
    P.pos[cur][i] = make_double4_32a(x, y, z, p.w);
    if (P.zero_forces) P.frc[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    double dx, dy, dz;
    skin_test(P, sp, st, i, x, y, z, dx, dy, dz);
    if (MIXED) P.prel[i] = cell_relative_moved(P, sp, i, dx, dy, dz);
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
    if (sp.tric) {  // fractional coordinates s = H^-1 r; the cell grid divides them
        matvec_ref(sp.HI, p.x, p.y, p.z, q[0], q[1], q[2]);
    } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) q[d] = __dmul_rn(sp.hinv[d], q[d]);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        // floor and conversion in one saturating instruction
        long long k = __double2ll_rd(__dmul_rn(q[d], (double)sp.nc[d]));
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
// Replica pools: the first kernel of a rebuild lists the chunks and cells of the rebuilding slots
// (block per slot), and the rebuild kernels run a grid sized to the GPU that strides over the
// list, instead of a block per chunk (per cell for the sort) of the whole pool: in a replica mix a
// few slots rebuild per step, and the blocks of the others only exit. A slot's place in the list
// is the count of rebuilding slots' chunks (cells) placed before it in the pool's chunk order, so
// the list keeps that order (slots with the most atoms per cell first); every chunk and cell is
// processed on its own, so results do not depend on the grid. k_rebuild_done clears the counts.
__global__ void __launch_bounds__(256) k_rebuild_list(const DP P, int step_mode) {
    __shared__ int part[2][8];
    const int s = blockIdx.x;
    if (!rebuild_pending(P)) return;
    const SysParams& sp = P.sp[s];
    if (!sp.active || !slot_runs(P, s, step_mode) || !P.st[s].rebuild) return;  // uniform per block
    int bc = 0, bg = 0;
    for (int t = threadIdx.x; t < P.max_slots; t += blockDim.x) {
        const SysParams& o = P.sp[t];
        if (o.active && o.ch0 < sp.ch0 && slot_runs(P, t, step_mode) && P.st[t].rebuild) {
            bc += o.nch;
            bg += o.nc[0] * o.nc[1] * o.nc[2];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bc += __shfl_xor_sync(0xffffffffu, bc, o);
        bg += __shfl_xor_sync(0xffffffffu, bg, o);
    }
    if ((threadIdx.x & 31) == 0) {
        part[0][threadIdx.x >> 5] = bc;
        part[1][threadIdx.x >> 5] = bg;
    }
    __syncthreads();
    bc = 0;
    bg = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        bc += part[0][w];
        bg += part[1][w];
    }
    const int ncell = sp.nc[0] * sp.nc[1] * sp.nc[2];
    if (threadIdx.x == 0) {
        atomicAdd(&P.ctl[8], sp.nch);
        atomicAdd(&P.ctl[9], ncell);
    }
    for (int k = threadIdx.x; k < sp.nch; k += blockDim.x) P.rb_list[bc + k] = sp.ch0 + k;
    int32_t* __restrict__ cells = P.rb_list + P.rb_cells_off;
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) cells[bg + k] = (int32_t)(sp.c0 + k);
}
__global__ void k_bin_list(const DP P, int respect_steps) {
    const int n = P.ctl[8];
    for (int q = blockIdx.x; q < n; q += gridDim.x) bin_chunk(P, P.rb_list[q], respect_steps);
}

// One exclusive scan over a slot's cells: of the atom counts (CL = 0, the last pass, which also
// clears the counts) or of the cluster counts ceil(count / clm) (CL = 1). Writes absolute indices
// starting at `carry` and returns the total. Counts are staged through shared memory so global
// loads and stores stay coalesced while each thread scans SCAN_ITEMS consecutive cells.
template <bool CL>
__device__ __forceinline__ int scan_cells(int32_t* __restrict__ cnt_g, int32_t* __restrict__ start_g, int ncell,
                                          int carry, int clm, int* buf, int* warp_tot, int* carry_sh,
                                          bool write_total = true) {
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
    if (t == 0 && write_total) start_g[ncell] = carry;
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

// Counting sort, pass 2 for pools with a slot of more than SCAN_SEG cells, in two kernels: each
// block scans one segment of SCAN_SEG cells of a slot from 0 and records the segment's totals;
// k_scan_fix then adds the slot's base and the preceding segments' totals, writes the closing
// entries and flips the slot's buffer set. The starts equal k_scan's (integer sums).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_seg(const DP P, int step_mode) {
    if (!rebuild_pending(P)) return;
    const int s = blockIdx.x, seg = blockIdx.y;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    if (!slot_runs(P, s, step_mode)) return;
    if (!P.st[s].rebuild) return;
    const int ncell = sp.nc[0] * sp.nc[1] * sp.nc[2];
    const int c0 = seg * SCAN_SEG;
    if (c0 >= ncell) return;
    const int m = min(SCAN_SEG, ncell - c0);
    __shared__ int buf[SCAN_THREADS * SCAN_ITEMS];
    __shared__ int warp_tot[SCAN_THREADS / 32];
    __shared__ int carry_sh;
    int32_t* __restrict__ cnt_g = P.cell_count + sp.c0 + c0;
    int ncl = 0;
    if (P.clm) ncl = scan_cells<true>(cnt_g, P.cl_start + sp.c0 + c0, m, 0, P.clm, buf, warp_tot, &carry_sh, false);
    const int na = scan_cells<false>(cnt_g, P.cell_start + sp.c0 + c0, m, 0, 1, buf, warp_tot, &carry_sh, false);
    if (threadIdx.x == 0) P.seg_tot[(int64_t)s * P.max_segs + seg] = make_int2(na, ncl);
}
__global__ void __launch_bounds__(256) k_scan_fix(const DP P, int step_mode) {
    if (!rebuild_pending(P)) return;
    const int s = blockIdx.x, seg = blockIdx.y;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    if (!slot_runs(P, s, step_mode)) return;
    SysState& st = P.st[s];
    if (!st.rebuild) return;
    const int ncell = sp.nc[0] * sp.nc[1] * sp.nc[2];
    const int nseg = (ncell + SCAN_SEG - 1) / SCAN_SEG;
    if (seg >= nseg) return;
    __shared__ int2 carry_sh;
    const int2* __restrict__ tot = P.seg_tot + (int64_t)s * P.max_segs;
    if (threadIdx.x < 32) {
        int a = 0, c = 0;
        for (int k = threadIdx.x; k < seg; k += 32) {
            const int2 t = tot[k];
            a += t.x;
            c += t.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
        }
        if (threadIdx.x == 0) carry_sh = make_int2(a, c);
    }
    __syncthreads();
    const int ca = (int)sp.a0 + carry_sh.x, cc = sp.cl0 + carry_sh.y;
    const int c0 = seg * SCAN_SEG, m = min(SCAN_SEG, ncell - c0);
    int32_t* __restrict__ sa = P.cell_start + sp.c0 + c0;
    for (int k = threadIdx.x; k < m; k += blockDim.x) sa[k] += ca;
    int32_t* __restrict__ sc = P.clm ? P.cl_start + sp.c0 + c0 : nullptr;
    if (P.clm)
        for (int k = threadIdx.x; k < m; k += blockDim.x) sc[k] += cc;
    if (seg == nseg - 1 && threadIdx.x == 0) {
        const int2 t = tot[seg];
        sa[m] = ca + t.x;
        if (P.clm) sc[m] = cc + t.y;
        st.ncl = carry_sh.y + t.y;
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
__global__ void k_scatter_list(const DP P, int respect_steps) {
    const int n = P.ctl[8];
    for (int q = blockIdx.x; q < n; q += gridDim.x) scatter_chunk(P, P.rb_list[q], respect_steps);
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

template <bool TRIC>
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
        return cell_order_key(sp, cell_relative<TRIC>(sp, p, lc, 0), (uint32_t)P.id[src_set][src]);
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
                qs[h] = cell_relative<TRIC>(sp, p, lc, type_of(p.w));
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
            q = cell_relative<TRIC>(sp, p, lc, type_of(p.w));
        } else {
            src = P.perm[beg + k];
            const uint32_t mine = key_of(src);
            for (int r = 0; r < cnt; ++r) rank += key_of(P.perm[beg + r]) < mine;
            p = P.pos[src_set][src];
            q = cell_relative<TRIC>(sp, p, lc, type_of(p.w));
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
template <bool TRIC>
__global__ void k_gather(const DP P, int64_t max_cells, int respect_steps) {
    __shared__ uint32_t keybuf[256 / 32][GATHER_SMEM_KEYS];
    const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g < max_cells && rebuild_block(P, P.cell_sys, g)) gather_cell<TRIC>(P, g, respect_steps, keybuf[threadIdx.x >> 5]);
}
template <bool TRIC>
__global__ void k_gather_list(const DP P, int respect_steps) {
    __shared__ uint32_t keybuf[256 / 32][GATHER_SMEM_KEYS];
    const int n = P.ctl[9];
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int32_t* __restrict__ cells = P.rb_list + P.rb_cells_off;
    for (int q = w; q < n; q += nw) gather_cell<TRIC>(P, cells[q], respect_steps, keybuf[threadIdx.x >> 5]);
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
        if (cnt > cap) {
            atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
            atomicMax(&st.need_nn, cnt);
        }
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
// Candidates of one neighbour cell [j, jend), tested against the padded list radius and written
// in candidate order. Two phases per run of up to 32 candidates: a branch-free pass that records one
// bit per candidate in a mask, then the accepted ones written in order, so the lanes of a warp
// diverge only in how many candidates and entries they have (a loop that branched on every
// candidate to store it made rebuilds 2 % slower).
// SHIFT: the mask is shifted one bit per candidate (candidate k ends at bit m - 1 - k) and the
// tests against atom i itself (half list: above i; full list: not i) are one mask operation per
// run: the single-system build (every chunk rebuilds at once) runs 6 % faster so. Otherwise bit k
// is set with the self tests per candidate: the listed build of replica pools, where few chunks
// rebuild at once, ran 6 % slower with the other form.
template <bool HALF, bool SHIFT>
__device__ __forceinline__ void scan_cell_mask(const float4* __restrict__ prel, int j, int jend, float sx, float sy,
                                               float sz, float rl2, uint32_t codebits, int i, bool home,
                                               uint32_t*& out, int& cnt, int64_t jump, int qmask, int cap) {
    for (int j0 = j; j0 < jend; j0 += 32) {
        const int m = min(32, jend - j0);
        const float4* __restrict__ pp = prel + j0;
        uint32_t mask = 0;  // SHIFT: candidate k at bit m - 1 - k; otherwise at bit k
#pragma unroll 4
        for (int k = 0; k < m; ++k) {
            const float4 pj = pp[k];
            const float dx = pj.x + sx, dy = pj.y + sy, dz = pj.z + sz;
            bool take = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rl2;
            if (SHIFT) {
                mask = (mask << 1) | (uint32_t)take;
            } else {
                if (HALF)
                    take = take && j0 + k > i;
                else if (home)
                    take = take && j0 + k != i;
                mask |= (uint32_t)take << k;
            }
        }
        if (SHIFT) {  // the run's candidates j0 + k against atom i: above i (half list) or not i
            const int t = i - j0;
            if (HALF)
                mask = t >= m - 1 ? 0u : (t >= 0 ? mask & ((1u << (m - 1 - t)) - 1u) : mask);
            else if (home && t >= 0 && t < m)
                mask &= ~(1u << (m - 1 - t));
        }
        while (mask) {
            int k;
            if (SHIFT) {
                const int b = 31 - __clz(mask);
                k = m - 1 - b;
                mask ^= 1u << b;
            } else {
                k = __ffs(mask) - 1;
                mask &= mask - 1;
            }
            if (cnt < cap) *out = (uint32_t)(j0 + k) | codebits;
            ++cnt;
            out += ((cnt & qmask) == 0) ? jump : 1;
        }
    }
}
template <bool HALF, bool TRIC, bool SHIFT = true>
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
    // squared distance to the faces of neighbouring cells (orthorhombic cells: skip the cells out of
    // range for this atom; the parallelepiped cells of a triclinic box are all scanned)
    const bool tric = TRIC && sp.tric;
    const bool prune = !tric;
    const float gxm = prune ? fmaxf(pi.x + 0.5f * csx, 0.f) : 0.f, gxp = prune ? fmaxf(0.5f * csx - pi.x, 0.f) : 0.f;
    const float gym = prune ? fmaxf(pi.y + 0.5f * csy, 0.f) : 0.f, gyp = prune ? fmaxf(0.5f * csy - pi.y, 0.f) : 0.f;
    const float gzm = prune ? fmaxf(pi.z + 0.5f * csz, 0.f) : 0.f, gzp = prune ? fmaxf(0.5f * csz - pi.z, 0.f) : 0.f;
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
                float shx = ox * csx, shy = oy * csy, shz = oz * csz;
                if (tric) {  // image shift ox C0 + oy C1 + oz C2 of the cell edge vectors
                    shx = (float)ox * sp.fcv[0] + (float)oy * sp.fcv[3] + (float)oz * sp.fcv[6];
                    shy = (float)ox * sp.fcv[1] + (float)oy * sp.fcv[4] + (float)oz * sp.fcv[7];
                    shz = (float)ox * sp.fcv[2] + (float)oy * sp.fcv[5] + (float)oz * sp.fcv[8];
                }
                scan_cell_mask<HALF, SHIFT>(prel, b0, b1, shx - pi.x, shy - pi.y, shz - pi.z, rl2, codebits, i, home, out,
                                cnt, jump, qmask, cap);
            }
        }
    }
    if (cnt > cap) {
        atomicOr(&st.flags, FLAG_LIST_OVERFLOW);
        atomicMax(&st.need_nn, cnt);
    }
    P.nn[i] = cnt > cap ? cap : cnt;
}
// only_two_cell: just the slots with a two-cell axis (the two-stage build covers the others).
template <bool HALF, bool TRIC>
__global__ void __launch_bounds__(256) k_build1(const DP P, int step_mode, int only_two_cell) {
    if (!rebuild_block(P, P.blk_sys, blockIdx.x)) return;
    if (only_two_cell) {
        const SysParams& sp = P.sp[P.blk_sys[blockIdx.x]];
        if (sp.nc[0] >= 3 && sp.nc[1] >= 3 && sp.nc[2] >= 3) return;
    }
    build1_chunk<HALF, TRIC>(P, blockIdx.x, step_mode);
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
// The two list builds over the listed chunks of a replica pool's rebuilding slots.
template <bool HALF, bool TRIC>
__global__ void __launch_bounds__(256) k_build1_list(const DP P, int step_mode) {
    const int n = P.ctl[8];
    for (int q = blockIdx.x; q < n; q += gridDim.x) build1_chunk<HALF, TRIC, false>(P, P.rb_list[q], step_mode);
}
template <bool HALF>
__global__ void __launch_bounds__(256) k_build1_generic_list(const DP P, int step_mode) {
    const int n = P.ctl[8];
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
        const int blk = P.rb_list[q];
        if (!P.sp[P.blk_sys[blk]].walk27) k_build_body<HALF, 1>(P, blk, step_mode);
    }
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
    __shared__ long long shx[XS_WORDS * 8];
    auto tile = cg::tiled_partition<LPA>(cg::this_thread_block());
    int s, i;
    const bool live = group_atom_of<LPA>(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, respect_steps)) return;  // uniform per block (one slot per chunk)
    const int gl = (int)tile.thread_rank();
    double fx = 0.0, fy = 0.0, fz = 0.0;
    XAcc e;  // pair energies as an exact sum (order-independent)
    xacc_zero(e);
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
        const bool tric = sp.tric != 0;
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
                rx = __dsub_rn(pj.x, pi.x);
                ry = __dsub_rn(pj.y, pi.y);
                rz = __dsub_rn(pj.z, pi.z);
                if (tric) {
                    min_image_full(sp.H, sp.HI, rx, ry, rz);
                } else {
                    rx = min_image_axis(rx, hx, ix);
                    ry = min_image_axis(ry, hy, iy);
                    rz = min_image_axis(rz, hz, iz);
                }
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
            } else {
                gx = c * rx;
                gy = c * ry;
                gz = c * rz;
                fx -= gx;
                fy -= gy;
                fz -= gz;
            }
            xacc_add(e, u);
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
    xacc_block_store<256>(e, P.xpe_part + (int64_t)blockIdx.x * XS_WORDS, shx);
}

// FP64 forces in the reference's own order (PIS_OPT_REF_ORDER): forces bit-identical to
// LJVOffsetManager::compute_potential (src/potentials/lennard_jones.rs:186-244).
// The reference walks its cells at max_rcut (cx outermost, cz innermost; src/atoms/neighbour_list.rs:
// 9-63), the 14 forward offsets of each cell in their fixed order (:94-165), then i over the home
// cell's atoms and j over the neighbour cell's atoms, both in ascending atom index; it subtracts
// f = c r_ij from F_i and adds it to F_j. Seen from one atom a, every pair term is subtracted as
// F_a -= c r_ab (r_ab = minimum image of r_b - r_a): when a is the walk's j, f is computed from
// r_ba = -r_ab exactly, so F_a + f = F_a - c r_ab bit for bit. The sequence of terms reaching F_a is
// ordered by the walk's key (visit rank of the i atom's cell, offset index, then the partner's
// index), which depends only on the pair and the current cells. So each thread collects the keys
// of its in-range list entries, sorts them, and subtracts the terms in that order from zero: the
// same roundings in the same order as the reference, hence the same forces, trajectory and
// energies for every step. Needs >= 3 reference cells per axis (below that the reference visits a
// neighbour cell twice) and a full list.
// Key (64 bits): cell visit rank (25) | offset index (4) | partner's original index (26) | list slot (9).
__device__ __forceinline__ int ref_fwd_index(int dx, int dy, int dz) {
    // index of (dx, dy, dz) in FORWARD_NEIGHBOUR_OFFSETS, -1 when it is a backward offset
    if (dz == 1) return 5 + (dy + 1) * 3 + (dx + 1);
    if (dz == 0 && dy == 1) return 2 + (dx + 1);
    if (dz == 0 && dy == 0) return dx == 0 ? 0 : (dx == 1 ? 1 : -1);
    return -1;
}
// Reference cell of a wrapped position: floor(s_d n_d) with s = h^-1 r, saturated at 0 as Rust's
// `f64 as usize`, then modulo n_d (src/atoms/neighbour_list.rs:17-33).
__device__ __forceinline__ int ref_cell_axis(double s, int n) {  // s: fractional coordinate
    long long c = __double2ll_rd(__dmul_rn(s, (double)n));
    if (c < 0) c = 0;
    return (int)(c % n);
}
__device__ __forceinline__ void ref_cell(const SysParams& sp, const double4_32a& p, int& a, int& b, int& c) {
    double s0, s1, s2;
    if (sp.tric) {
        matvec_ref(sp.HI, p.x, p.y, p.z, s0, s1, s2);
    } else {
        s0 = __dmul_rn(sp.hinv[0], p.x);
        s1 = __dmul_rn(sp.hinv[1], p.y);
        s2 = __dmul_rn(sp.hinv[2], p.z);
    }
    a = ref_cell_axis(s0, sp.rnc[0]);
    b = ref_cell_axis(s1, sp.rnc[1]);
    c = ref_cell_axis(s2, sp.rnc[2]);
}
__device__ __forceinline__ void ref_min_image(const SysParams& sp, double& x, double& y, double& z) {
    if (sp.tric) {
        min_image_full(sp.H, sp.HI, x, y, z);
    } else {
        x = min_image_axis(x, sp.h[0], sp.hinv[0]);
        y = min_image_axis(y, sp.h[1], sp.hinv[1]);
        z = min_image_axis(z, sp.h[2], sp.hinv[2]);
    }
}
__device__ __forceinline__ int ref_wrap_delta(int d, int n) {
    if (d > 1) d -= n;
    if (d < -1) d += n;
    return d;
}
constexpr int REF_MAX_ENTRIES = 256;  // in-range pairs per atom (local memory: 2 KB per thread)

__global__ void __launch_bounds__(256) k_force_fp64_ref(const DP P, int respect_steps) {
    __shared__ long long shx[XS_WORDS * 8];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, respect_steps)) return;
    XAcc e;
    xacc_zero(e);
    if (live) {
        uint64_t keys[REF_MAX_ENTRIES];
        const SysParams& sp = P.sp[s];
        const int cur = P.st[s].cur;
        const double4_32a* __restrict__ pos = P.pos[cur];
        const int32_t* __restrict__ oid = P.id[cur];
        const double4_32a pi = pos[i];
        const LJDev* tab = P.tab + sp.tab0 + type_of(pi.w) * sp.nt;
        const int nx = sp.rnc[0], ny = sp.rnc[1], nz = sp.rnc[2];
        int ax, ay, az;
        ref_cell(sp, pi, ax, ay, az);
        const uint64_t rank_a = (uint64_t)((ax * ny + ay) * nz + az);
        const int nn = P.nn[i];
        const int64_t npad = P.npad;
        int m = 0;
        for (int k = 0; k < nn; ++k) {
            const int j = (int)(P.nbr[(int64_t)k * npad + i] & JMASK);
            const double4_32a pj = pos[j];
            const LJDev& T = tab[type_of(pj.w)];
            if (!T.present) continue;
            double rx = __dsub_rn(pj.x, pi.x), ry = __dsub_rn(pj.y, pi.y), rz = __dsub_rn(pj.z, pi.z);
            ref_min_image(sp, rx, ry, rz);
            const double r2 = norm2_ref(rx, ry, rz);
            if (r2 > T.rc2_hi || (r2 >= T.rc2_lo && sqrt(r2) > T.rcut)) continue;
            int bx, by, bz;
            ref_cell(sp, pj, bx, by, bz);
            const int dx = ref_wrap_delta(bx - ax, nx), dy = ref_wrap_delta(by - ay, ny), dz = ref_wrap_delta(bz - az, nz);
            int o = ref_fwd_index(dx, dy, dz);
            uint64_t rank = rank_a;
            if (o < 0) {  // the partner's cell is the walk's home cell
                o = ref_fwd_index(-dx, -dy, -dz);
                rank = (uint64_t)((bx * ny + by) * nz + bz);
            }
            const uint64_t key = (rank << 39) | ((uint64_t)(o & 15) << 35) | ((uint64_t)oid[j] << 9) | (uint64_t)k;
            if (m < REF_MAX_ENTRIES) keys[m] = key;
            ++m;
        }
        if (m > REF_MAX_ENTRIES) {
            atomicOr(&P.st[s].flags, FLAG_LIST_OVERFLOW);
            m = REF_MAX_ENTRIES;
        }
        for (int a = 1; a < m; ++a) {  // insertion sort (a few dozen keys)
            const uint64_t v = keys[a];
            int b = a - 1;
            while (b >= 0 && keys[b] > v) {
                keys[b + 1] = keys[b];
                --b;
            }
            keys[b + 1] = v;
        }
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int a = 0; a < m; ++a) {
            const int k = (int)(keys[a] & 511u);
            const int j = (int)(P.nbr[(int64_t)k * npad + i] & JMASK);
            const double4_32a pj = pos[j];
            const LJ64 L = lj64_load(tab[type_of(pj.w)]);
            double rx = __dsub_rn(pj.x, pi.x), ry = __dsub_rn(pj.y, pi.y), rz = __dsub_rn(pj.z, pi.z);
            ref_min_image(sp, rx, ry, rz);
            double u, c;
            lj_fp64(L, norm2_ref(rx, ry, rz), u, c);
            fx = __dsub_rn(fx, __dmul_rn(c, rx));
            fy = __dsub_rn(fy, __dmul_rn(c, ry));
            fz = __dsub_rn(fz, __dmul_rn(c, rz));
            xacc_add(e, u);
        }
        P.frc[i] = make_double4_32a(fx, fy, fz, 0.0);
    }
    xacc_block_store<256>(e, P.xpe_part + (int64_t)blockIdx.x * XS_WORDS, shx);
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

// Mixed precision forces on a Newton-3 half list (PIS_LIST_HALF with the mixed path; the
// reference's own managers walk half shells, src/potentials/lennard_jones.rs:186-244): thread per
// atom, column-major list, the same FP32 pair arithmetic as k_force_mixed. Atom i keeps its share in
// the usual batch sums; each pair's force on j, -F_ij, is added to F_j with FP64 atomics, and so is
// i's own total at the end (other threads add to it as their j), so forces must be zeroed before
// (integrate-1 and every evaluation do). The order of the atomic additions varies from launch to
// launch, so results are reproducible to FP64 rounding of the sums, not bit for bit.
template <int ACC, bool ONE, int NB>
__global__ void __launch_bounds__(256) k_force_mixed_half(const DP P, int step_mode) {
    __shared__ double sh[32];
    __shared__ float shift[12];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, step_mode)) return;
    const SysParams& sp = P.sp[s];
    fill_shift_axes(shift, sp);
    __syncthreads();
    MixAcc<ACC> acc;
    if (live) {
        const float4* __restrict__ prel = P.prel;
        const float4 pi = prel[i];
        const LJDev* tab = P.tab + sp.tab0 + __float_as_int(pi.w) * sp.nt;
        const MixLJ P0 = mix_lj_load(tab[0]);
        const int nn = P.nn[i];
        const uint32_t* __restrict__ nbp = P.nbr + i;
        const uint32_t row32 = (uint32_t)P.npad;
        uint32_t qoff = 0;
        int since = 0;
        for (int k0 = 0; k0 < nn; k0 += NB) {
            uint32_t ent[NB];
            float4 pj[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                ent[b] = (k0 + b < nn) ? load_list_word(nbp + qoff + (uint32_t)b * row32) : 0xffffffffu;
                pj[b] = ent[b] != 0xffffffffu ? __ldg(prel + (ent[b] & JMASK)) : pi;
            }
            qoff += (uint32_t)NB * row32;
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                if (ent[b] == 0xffffffffu) continue;
                const float3 sv = shift_of(shift, ent[b] >> JBITS);
                const float dx = (pj[b].x - pi.x) + sv.x;
                const float dy = (pj[b].y - pi.y) + sv.y;
                const float dz = (pj[b].z - pi.z) + sv.z;
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                MixLJ L = P0;
                if (!ONE) {
                    const LJDev& T = tab[__float_as_int(pj[b].w)];
                    L = T.present ? mix_lj_load(T) : MixLJ{-1.f, 0.f, 0.f, 0.f, 0.f};
                }
                if (!(r2 <= L.frc2)) continue;
                const float inv = rcp_approx(r2);
                const float s2 = L.fs2 * inv;
                const float s6 = s2 * s2 * s2;
                const float c = (s6 * fmaf(2.0f, s6, -1.0f)) * (L.fe24 * inv);
                const float u = fmaf(L.fe4, fmaf(s6, s6, -s6), -L.fuc);
                acc.px = fmaf(-c, dx, acc.px);
                acc.py = fmaf(-c, dy, acc.py);
                acc.pz = fmaf(-c, dz, acc.pz);
                acc.pe += u;
                double4_32a* fj = P.frc + (ent[b] & JMASK);
                atomicAdd(&fj->x, (double)(c * dx));
                atomicAdd(&fj->y, (double)(c * dy));
                atomicAdd(&fj->z, (double)(c * dz));
            }
            since += NB;
            if (since >= MIX_FLUSH) {
                acc.fold();
                since = 0;
            }
        }
        acc.finish();
        atomicAdd(&P.frc[i].x, acc.fx);
        atomicAdd(&P.frc[i].y, acc.fy);
        atomicAdd(&P.frc[i].z, acc.fz);
    }
    double tot = block_sum<256>(live ? acc.e : 0.0, sh);
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
        if (!failed && !mbar_wait_n(&full[q0], par, P.wait_limit)) failed = true;
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
            if (mbar_wait_n(&empty[q0], par, P.wait_limit))
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
    bool got = tiled && mbar_wait_n(&bar, 0u, P.wait_limit);
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

}  // namespace pis
