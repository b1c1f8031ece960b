// dev_cluster.cuh - Device side of the engine, part 3: the cluster-list variants (union lists per cluster of up to
// four atoms, their build, filter and force kernels, and the exact-set mask for their export).
// Included by engine.cu, in this order: dev_common.cuh, dev_step.cuh, dev_cluster.cuh,
// dev_step_end.cuh.
#pragma once

namespace pis {

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

}  // namespace pis
