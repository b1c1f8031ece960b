// xsum.cuh - exact, order-independent sums of doubles on the device (the FP64 path's energy,
// kinetic-energy and virial reductions, and the no-allocation entry point's energy).
#pragma once

#include <cstdint>

namespace pis {

__device__ __forceinline__ long long xs_warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- Exact sums -----------------------------------------------------------------------------------
// The FP64 path reduces energy, kinetic energy and virial with one defined sum that does not depend
// on the order of the terms: every term t is quantised to q(t) = sign(t) floor(|t| 2^104), the
// integers are added exactly, and the result is the double nearest (sum q) 2^-104, ties to even. A
// term of magnitude >= 2^56 or a non-finite term makes the sum NaN. Terms of magnitude >= 2^-52 are
// represented exactly, so for them this is the exactly rounded sum. Integer addition is
// associative, so threads, blocks, chunks and slots combine in any order: a slot's energy is the
// same whatever the grid, the list order or the other slots in the pool, and it equals a serial
// evaluation of the same definition (the test oracle's, written independently).
// A thread accumulates into six signed 64-bit limbs of 32 payload bits (limb k weighs
// 2^(32k - 104)) plus a count of invalid terms; carries are propagated when a block writes its
// partial, so limbs 0-4 of a partial lie in [0, 2^32) and any number of partials can be added.
constexpr int XS_FRAC = 104;
constexpr int XS_LIMBS = 6;
constexpr int XS_WORDS = 7;
struct XAcc {
    long long l[XS_LIMBS];
    long long bad;
};
__device__ __forceinline__ void xacc_zero(XAcc& a) {
#pragma unroll
    for (int z = 0; z < XS_LIMBS; ++z) a.l[z] = 0;
    a.bad = 0;
}
__device__ __forceinline__ void xacc_add(XAcc& a, double t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    const int e = (int)((b >> 52) & 0x7ff);
    unsigned long long m = b & 0xfffffffffffffull;
    if (e >= 1023 + 56) {  // |t| >= 2^56, infinity or NaN
        a.bad += 1;
        return;
    }
    // |t| = m 2^(q - 104) with the implicit bit (subnormals have exponent 1 - 1075)
    int q;
    if (e == 0) {
        q = 1 - 1075 + XS_FRAC;
    } else {
        m |= 1ull << 52;
        q = e - 1075 + XS_FRAC;
    }
    if (q < 0) {  // bits below 2^-104 are dropped: floor of the magnitude
        m = q > -64 ? (m >> (-q)) : 0ull;
        q = 0;
    }
    const int k = q >> 5, sh = q & 31;  // q <= 107, so k + 2 <= 5
    const unsigned long long lo = m << sh;
    const unsigned long long hi = sh ? (m >> (64 - sh)) : 0ull;
    const long long c0 = (long long)(lo & 0xffffffffull), c1 = (long long)(lo >> 32), c2 = (long long)hi;
    const bool neg = (b >> 63) != 0;
#pragma unroll
    for (int z = 0; z < XS_LIMBS; ++z) {
        const long long v = z == k ? c0 : (z == k + 1 ? c1 : (z == k + 2 ? c2 : 0ll));
        a.l[z] += neg ? -v : v;
    }
}
// Carry propagation: limbs 0-4 into [0, 2^32), the rest into the signed top limb.
__device__ __forceinline__ void xacc_normalise(long long* l) {
#pragma unroll
    for (int z = 0; z < XS_LIMBS - 1; ++z) {
        const long long c = l[z] >> 32;  // arithmetic shift: floor division by 2^32
        l[z] -= c * 4294967296ll;
        l[z + 1] += c;
    }
}
// Sum of every thread's accumulator over the block; thread 0 writes the normalised partial
// (XS_WORDS words) to out. sh holds at least XS_WORDS * NT / 32 words; all threads must call it.
template <int NT>
__device__ __forceinline__ void xacc_block_store(const XAcc& a, long long* out, long long* sh) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    long long v[XS_WORDS];
#pragma unroll
    for (int z = 0; z < XS_LIMBS; ++z) v[z] = a.l[z];
    v[XS_LIMBS] = a.bad;
#pragma unroll
    for (int z = 0; z < XS_WORDS; ++z) v[z] = xs_warp_sum(v[z]);
    __syncthreads();
    if (l == 0)
#pragma unroll
        for (int z = 0; z < XS_WORDS; ++z) sh[w * XS_WORDS + z] = v[z];
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t[XS_WORDS];
        for (int z = 0; z < XS_WORDS; ++z) t[z] = 0;
        for (int q = 0; q < NT / 32; ++q)
            for (int z = 0; z < XS_WORDS; ++z) t[z] += sh[q * XS_WORDS + z];
        xacc_normalise(t);
        for (int z = 0; z < XS_WORDS; ++z) out[z] = t[z];
    }
}
// The double nearest to a sum of normalised partials (limbs, then the invalid-term count), ties to
// even; NaN when an invalid term was seen.
__device__ __forceinline__ double xacc_value(const long long* in) {
    if (in[XS_LIMBS] != 0) return __longlong_as_double(0x7ff8000000000000ll);
    long long l[XS_LIMBS];
    for (int z = 0; z < XS_LIMBS; ++z) l[z] = in[z];
    xacc_normalise(l);
    // 256-bit two's complement: l[5] is the signed top limb (|l[5]| < 2^62)
    unsigned long long w[4];
    w[0] = (unsigned long long)l[0] | ((unsigned long long)l[1] << 32);
    w[1] = (unsigned long long)l[2] | ((unsigned long long)l[3] << 32);
    w[2] = (unsigned long long)l[4] | ((unsigned long long)l[5] << 32);
    w[3] = (unsigned long long)(l[5] >> 32);
    const bool neg = (long long)w[3] < 0;
    if (neg) {
        unsigned long long c = 1;
        for (int z = 0; z < 4; ++z) {
            w[z] = ~w[z] + c;
            c = (c && w[z] == 0) ? 1ull : 0ull;
        }
    }
    int p = -1;
    for (int z = 3; z >= 0 && p < 0; --z)
        if (w[z]) p = 64 * z + 63 - __clzll((long long)w[z]);
    if (p < 0) return 0.0;
    unsigned long long mant;
    int lo = p - 52;
    if (lo <= 0) {
        mant = w[0];
        lo = 0;
    } else {
        const int z = lo >> 6, b = lo & 63;
        unsigned long long v = w[z] >> b;
        if (b && z + 1 < 4) v |= w[z + 1] << (64 - b);
        mant = v & ((1ull << 53) - 1);
        const int hb = lo - 1;
        const unsigned long long half = (w[hb >> 6] >> (hb & 63)) & 1ull;
        bool sticky = (w[hb >> 6] & ((1ull << (hb & 63)) - 1ull)) != 0;
        for (int q = 0; q < (hb >> 6); ++q) sticky = sticky || w[q] != 0;
        if (half && (sticky || (mant & 1ull))) {
            mant += 1;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                lo += 1;
            }
        }
    }
    const double v = scalbn((double)mant, lo - XS_FRAC);
    return neg ? -v : v;
}

}  // namespace pis
