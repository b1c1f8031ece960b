// dev_step_end.cuh - Device side of the engine, part 4: the kick (k_integrate2), the fused step kernel
// (k_step_mixed), the step end and the small bookkeeping kernels (evaluation marks, rebuild done,
// uploads and downloads of a slot, box and velocity scaling).
// Included by engine.cu, in this order: dev_common.cuh, dev_step.cuh, dev_cluster.cuh,
// dev_step_end.cuh.
#pragma once

namespace pis {

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

// r_i . F_i, the atom's share of the virial trace (the pressure of Atoms::pressure,
// src/atoms/properties.rs:61-65, needs only tr W)
__device__ __forceinline__ double virial_trace(const double4_32a& p, const double4_32a& f) {
    return __dadd_rn(__dadd_rn(__dmul_rn(p.x, f.x), __dmul_rn(p.y, f.y)), __dmul_rn(p.z, f.z));
}

template <bool UPDATE, bool EXACT>
__global__ void k_integrate2(const DP P, int respect_steps) {
    __shared__ double sh[32];
    __shared__ long long shx[XS_WORDS * 8];
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
        if (st.want_virial || st.thermo) p = P.pos[cur][i];
    }
    const bool trace = UPDATE && st.thermo;
    if (EXACT) {
        // FP64 path: exact sums of m |v|^2 (halved at the step end) and of r_i[a] F_i[b]
        XAcc x;
        xacc_zero(x);
        if (live) xacc_add(x, ke);
        xacc_block_store<256>(x, P.xke_part + (int64_t)blockIdx.x * XS_WORDS, shx);
        if (trace) {
            xacc_zero(x);
            if (live) xacc_add(x, virial_trace(p, f));
            xacc_block_store<256>(x, P.xtr_part + (int64_t)blockIdx.x * XS_WORDS, shx);
        }
        if (st.want_virial & 1) {
            const double r[3] = {p.x, p.y, p.z}, g[3] = {f.x, f.y, f.z};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    xacc_zero(x);
                    if (live) xacc_add(x, __dmul_rn(r[a], g[b]));
                    xacc_block_store<256>(x, P.xvir_part + ((int64_t)blockIdx.x * 9 + a * 3 + b) * XS_WORDS, shx);
                }
        }
        if (!UPDATE && (st.want_virial & 2)) {  // kinetic tensor sum_i v_i v_i^T
            const double4_32a v = live ? P.vel[cur][i] : make_double4_32a(0.0, 0.0, 0.0, 0.0);
            const double u[3] = {v.x, v.y, v.z};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    xacc_zero(x);
                    if (live) xacc_add(x, __dmul_rn(u[a], u[b]));
                    xacc_block_store<256>(x, P.xkt_part + ((int64_t)blockIdx.x * 9 + a * 3 + b) * XS_WORDS, shx);
                }
        }
        return;
    }
    double tot = block_sum<256>(ke, sh);
    if (threadIdx.x == 0) P.ke_part[blockIdx.x] = 0.5 * tot;
    if (trace) {
        const double t = block_sum<256>(live ? virial_trace(p, f) : 0.0, sh);
        if (threadIdx.x == 0) P.tr_part[blockIdx.x] = t;
    }
    if (st.want_virial & 1) {
        double r[3] = {p.x, p.y, p.z}, g[3] = {f.x, f.y, f.z};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                double t = block_sum<256>(live ? r[a] * g[b] : 0.0, sh);
                if (threadIdx.x == 0) P.vir_part[(int64_t)blockIdx.x * 9 + a * 3 + b] = t;
            }
    }
    if (!UPDATE && (st.want_virial & 2)) {  // kinetic tensor sum_i v_i v_i^T
        const double4_32a v = live ? P.vel[cur][i] : make_double4_32a(0.0, 0.0, 0.0, 0.0);
        const double u[3] = {v.x, v.y, v.z};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const double t = block_sum<256>(__dmul_rn(u[a], u[b]), sh);
                if (threadIdx.x == 0) P.kt_part[(int64_t)blockIdx.x * 9 + a * 3 + b] = t;
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
// TRACE: the instantiation launched while some slot records its thermo (the virial trace of every
// step); the default one carries no trace code (with it the pair loop was measured 6 % slower).
// q: the step's index in its graph. The step counters are updated once per graph (k_ring_commit),
// so a slot takes part while it has more than q steps left, and the step's PE, KE and trace block
// partials go to row q of the partial ring, summed per step after the graph's last step
// (k_ring_sums) in the order k_step_end sums them.
template <int ACC, bool ONE, int MIX_BATCH, bool DRIFT, bool TRACE>
__global__ void __launch_bounds__(256, step_min_blocks<MIX_BATCH>()) k_step_mixed(const DP P, int q) {
    __shared__ double sh[32];
    __shared__ float shift[12];
    int s, i;
    const bool live = atom_of(P, s, i);
    if (s < 0) return;
    if (!slot_runs(P, s, 1 + q)) return;
    const SysParams& sp = P.sp[s];
    SysState& st = P.st[s];
    fill_shift_axes(shift, sp);
    __syncthreads();
    MixAcc<ACC> acc;
    if (live)
        mixed_atom_forces<ACC, 1, ONE, MIX_BATCH, step_list_prefetch<MIX_BATCH>(), FUSED_LQ>(P, sp, i, 0, shift, acc);
    const bool drift = DRIFT && st.steps_left > q + 1;
    const bool want_virial = (st.want_virial & 1) != 0;
    const bool want_trace = TRACE && st.thermo != 0;
    double ke = 0.0;
    double4_32a p = make_double4_32a(0.0, 0.0, 0.0, 0.0), f = p;
    if (live) {
        f = make_double4_32a(acc.fx, acc.fy, acc.fz, 0.0);
        // The forces themselves are only read by the host (downloads happen between graphs) and by
        // the unfused kick, never inside a fused run: a = F/m carries them to the next step. So they
        // are stored only in a step that does not drift - the last step of every graph and of every
        // slot's run - which saves a 32-byte store per atom on the other steps.
        if (!drift) P.frc[i] = f;
        const int cur = st.cur;
        double4_32a v = P.vel[cur][i];
        const double4_32a a = P.acc[cur][i];
        double bx, by, bz;
        accel_mixed(f, a.w, bx, by, bz);
        kick_mixed(sp, v, a, bx, by, bz);
        P.vel[cur][i] = v;
        P.acc[cur][i] = make_double4_32a(bx, by, bz, a.w);
        ke = twice_ke_mixed(v);
        if (want_virial || want_trace || drift) p = P.pos[cur][i];
        if (drift) {
            double x, y, z;
            drift_mixed(sp, p, v, bx, by, bz, x, y, z);
            P.pos[cur][i] = make_double4_32a(x, y, z, p.w);
            double dx, dy, dz;
            skin_test(P, sp, st, i, x, y, z, dx, dy, dz);
            P.prel_out[i] = cell_relative_moved(P, sp, i, dx, dy, dz);
        }
    }
    double* __restrict__ ring = P.ring + (int64_t)q * 3 * P.ring_stride;
    const double pe_tot = block_sum<256>(acc.e, sh);
    if (threadIdx.x == 0) ring[blockIdx.x] = pe_tot;
    const double ke_tot = block_sum<256>(ke, sh);
    if (threadIdx.x == 0) ring[P.ring_stride + blockIdx.x] = 0.5 * ke_tot;
    if (TRACE && want_trace) {
        const double t = block_sum<256>(live ? virial_trace(p, f) : 0.0, sh);
        if (threadIdx.x == 0) ring[2 * P.ring_stride + blockIdx.x] = t;
    }
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
// Exact-sum partials of a slot: words of partials first .. first + count - 1 (XS_WORDS each, `stride`
// apart) added and converted. All threads must call it; the value is valid in thread 0.
__device__ __forceinline__ double xacc_slot_value(const long long* part, int64_t first, int64_t count, int stride,
                                                  long long* shx) {
    XAcc a;
    xacc_zero(a);
    for (int64_t c = threadIdx.x; c < count; c += END_THREADS) {
        const long long* q = part + (first + c) * stride;
#pragma unroll
        for (int z = 0; z < XS_LIMBS; ++z) a.l[z] += q[z];
        a.bad += q[XS_LIMBS];
    }
    __shared__ long long tot[XS_WORDS];
    xacc_block_store<END_THREADS>(a, tot, shx);
    __syncthreads();
    double v = 0.0;
    if (threadIdx.x == 0) v = xacc_value(tot);
    __syncthreads();
    return v;
}

// EXACT: an FP64 pool (exact-sum partials); the mixed path's pools sum doubles.
template <bool EXACT>
__global__ void __launch_bounds__(END_THREADS) k_step_end(const DP P, int mode) {
    __shared__ double sh[32];
    __shared__ long long shx[EXACT ? XS_WORDS * (END_THREADS / 32) : 1];
    int s = blockIdx.x;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    SysState& st = P.st[s];
    if (mode == 0 && st.steps_left <= 0) return;
    if (mode != 0 && !st.eval) return;
    double pe = 0.0, ke = 0.0;
    const int F = P.pe_stride;
    if (EXACT) {
        // FP64 pools: exact sums (PE over the force kernel's blocks, m |v|^2 and r_i F_i per chunk)
        double w[9];
        const bool vir = (st.want_virial & 1) && mode != 1;
        if (mode != 2) pe = xacc_slot_value(P.xpe_part, (int64_t)sp.ch0 * F, (int64_t)sp.nch * F, XS_WORDS, shx);
        if (mode != 1) ke = 0.5 * xacc_slot_value(P.xke_part, sp.ch0, sp.nch, XS_WORDS, shx);
        if (vir)
            for (int q = 0; q < 9; ++q)
                w[q] = xacc_slot_value(P.xvir_part + (int64_t)q * XS_WORDS, sp.ch0, sp.nch, 9 * XS_WORDS, shx);
        double tr = 0.0, kt[9];
        if (mode == 0 && st.thermo) tr = xacc_slot_value(P.xtr_part, sp.ch0, sp.nch, XS_WORDS, shx);
        const bool ktn = mode == 2 && (st.want_virial & 2);
        if (ktn)
            for (int q = 0; q < 9; ++q)
                kt[q] = xacc_slot_value(P.xkt_part + (int64_t)q * XS_WORDS, sp.ch0, sp.nch, 9 * XS_WORDS, shx);
        if (threadIdx.x == 0) {
            if (mode != 2) {
                if (P.full_list) pe *= 0.5;
                st.pe = pe;
            }
            if (mode != 1) st.ke = ke;
            if (vir)
                for (int q = 0; q < 9; ++q) st.virial[q] = w[q];
            if (ktn)
                for (int q = 0; q < 9; ++q) st.ktensor[q] = kt[q];
            if ((mode != 2 && pe != pe) || (mode != 1 && ke != ke)) st.flags |= FLAG_NAN;
            if (mode == 2) {
                st.eval = 0;
                st.want_virial = 0;
            }
            if (mode == 0) {
                const int64_t h = (int64_t)s * P.hist + (st.steps_done % P.hist);
                P.pe_hist[h] = pe;
                P.ke_hist[h] = ke;
                if (st.thermo) P.tr_hist[h] = tr;
                st.steps_done += 1;
                st.steps_left -= 1;
            }
        }
        return;
    }
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
    const bool vir = (st.want_virial & 1) && mode != 1;
    if (vir) {
        for (int q = 0; q < 9; ++q) {
            double a = 0.0;
            for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) a += P.vir_part[(int64_t)(sp.ch0 + c) * 9 + q];
            w[q] = block_sum<END_THREADS>(a, sh);
        }
    }
    double tr = 0.0;
    if (mode == 0 && st.thermo) {
        for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) tr += P.tr_part[sp.ch0 + c];
        tr = block_sum<END_THREADS>(tr, sh);
    }
    double kt[9];
    const bool ktn = mode == 2 && (st.want_virial & 2);
    if (ktn) {
        for (int q = 0; q < 9; ++q) {
            double a = 0.0;
            for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) a += P.kt_part[(int64_t)(sp.ch0 + c) * 9 + q];
            kt[q] = block_sum<END_THREADS>(a, sh);
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
        if (ktn)
            for (int q = 0; q < 9; ++q) st.ktensor[q] = kt[q];
        if ((mode != 2 && pe != pe) || (mode != 1 && ke != ke)) st.flags |= FLAG_NAN;
        if (mode == 2) {
            st.eval = 0;
            st.want_virial = 0;
        }
        if (mode == 0) {
            const int64_t h = (int64_t)s * P.hist + (st.steps_done % P.hist);
            P.pe_hist[h] = pe;
            P.ke_hist[h] = ke;
            if (st.thermo) P.tr_hist[h] = tr;
            st.steps_done += 1;
            st.steps_left -= 1;
        }
    }
}

// End of a graph of fused steps, pass 1: block (slot, q) sums step q's partials from the ring (the
// thread-strided sums and block tree of k_step_end, so every value equals the per-step reduction's)
// into the slot's energy history, and flags a NaN. The counters are still the graph's start values.
__global__ void __launch_bounds__(END_THREADS) k_ring_sums(const DP P) {
    __shared__ double sh[32];
    const int s = blockIdx.x, q = blockIdx.y;
    const SysParams& sp = P.sp[s];
    if (!sp.active) return;
    SysState& st = P.st[s];
    if (st.steps_left <= q) return;
    const double* __restrict__ r = P.ring + (int64_t)q * 3 * P.ring_stride;
    double pe = 0.0, ke = 0.0, tr = 0.0;
    for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) pe += r[sp.ch0 + c];
    for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) ke += r[P.ring_stride + sp.ch0 + c];
    pe = block_sum<END_THREADS>(pe, sh);
    ke = block_sum<END_THREADS>(ke, sh);
    if (st.thermo) {
        for (int c = threadIdx.x; c < sp.nch; c += END_THREADS) tr += r[2 * P.ring_stride + sp.ch0 + c];
        tr = block_sum<END_THREADS>(tr, sh);
    }
    if (threadIdx.x == 0) {
        if (P.full_list) pe *= 0.5;
        const int64_t h = (int64_t)s * P.hist + (st.steps_done + q) % P.hist;
        P.pe_hist[h] = pe;
        P.ke_hist[h] = ke;
        if (st.thermo) P.tr_hist[h] = tr;
        if (pe != pe || ke != ke) atomicOr(&st.flags, FLAG_NAN);
    }
}
// Pass 2, thread per slot: the last step's energies into the state, and the counters advanced by
// the steps the slot took in the graph (g steps, or fewer if its run ended inside the graph).
__global__ void k_ring_commit(const DP P, int g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.max_slots || !P.sp[s].active) return;
    SysState& st = P.st[s];
    const int64_t left = st.steps_left;
    if (left <= 0) return;
    const int64_t n = left < g ? left : g;
    const int64_t h = (int64_t)s * P.hist + (st.steps_done + n - 1) % P.hist;
    st.pe = P.pe_hist[h];
    st.ke = P.ke_hist[h];
    st.steps_done += n;
    st.steps_left -= n;
}

// End of a rebuild phase (its last kernel, so every rebuild kernel has read the request flags):
// count and clear the rebuilt slots' flags and lower the device-wide request word. A drift that
// runs later in the same step (the fused step kernel) may raise them again for the next step.
// body_kernels > 0 (the last kernel of a conditional rebuild body): the body's kernel count is
// added to ctl[2..3] (64 bits), which the host folds into its launch counter.
__global__ void k_rebuild_done(const DP P, int step_mode, int body_kernels) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {
        if (body_kernels > 0) *reinterpret_cast<unsigned long long*>(P.ctl + 2) += (unsigned long long)body_kernels;
        P.ctl[0] = 0;
        P.ctl[8] = 0;  // the listed rebuild's counts
        P.ctl[9] = 0;
    }
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
        double rx = __dsub_rn(pj.x, pi.x), ry = __dsub_rn(pj.y, pi.y), rz = __dsub_rn(pj.z, pi.z);
        if (sp.tric) {
            min_image_full(sp.H, sp.HI, rx, ry, rz);
        } else {
            rx = min_image_axis(rx, sp.h[0], sp.hinv[0]);
            ry = min_image_axis(ry, sp.h[1], sp.hinv[1]);
            rz = min_image_axis(rz, sp.h[2], sp.hinv[2]);
        }
        const LJDev& L = tab[type_of(pj.w)];
        P.keep[q] = (uint8_t)(L.present && !(sqrt(norm2_ref(rx, ry, rz)) > L.rcut));
    }
}

struct Mat3Arg {
    double m[9];  // row-major
};

// v <- M v (row-major M) for one slot (ensemble velocity scaling, `&scale * &atoms.velocities`,
// src/potentials/potential.rs:45-50,119-134), each row summed left to right without fused
// multiply-adds.
__global__ void k_scale_vel(const DP P, int slot, const Mat3Arg M) {
    int s, i;
    if (!atom_of(P, s, i) || s != slot) return;
    const int cur = P.st[s].cur;
    double4_32a v = P.vel[cur][i];
    double x, y, z;
    matvec_ref(M.m, v.x, v.y, v.z, x, y, z);
    P.vel[cur][i] = make_double4_32a(x, y, z, v.w);
}

// Atoms::scale_box (src/atoms/transformations.rs:5-16): s = h^-1 r with the old inverse, r = h' s
// with the new box. Diagonal boxes use their diagonals (the same products as the full form).
__global__ void k_scale_pos(const DP P, int slot, const Mat3Arg HI_old, const Mat3Arg H_new, int tric) {
    int s, i;
    if (!atom_of(P, s, i) || s != slot) return;
    const int cur = P.st[s].cur;
    double4_32a p = P.pos[cur][i];
    if (tric) {
        double s0, s1, s2;
        matvec_ref(HI_old.m, p.x, p.y, p.z, s0, s1, s2);
        matvec_ref(H_new.m, s0, s1, s2, p.x, p.y, p.z);
    } else {
        p.x = __dmul_rn(H_new.m[0], __dmul_rn(HI_old.m[0], p.x));
        p.y = __dmul_rn(H_new.m[4], __dmul_rn(HI_old.m[4], p.y));
        p.z = __dmul_rn(H_new.m[8], __dmul_rn(HI_old.m[8], p.z));
    }
    P.pos[cur][i] = p;
}

// Condition of a step's rebuild node: some slot rebuilds in this step (the device-wide word).
__global__ void k_set_rebuild_cond(const DP P, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, P.ctl[0] != 0 ? 1u : 0u);
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

}  // namespace pis
