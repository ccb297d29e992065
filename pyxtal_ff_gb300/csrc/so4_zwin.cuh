// so4_zwin.cuh -- Z contractions by sliding windows, atoms across lanes.
//
// Same CTA layout as so4_zlanes.cuh (32 atoms per CTA, lane = atom, U tiles in
// shared memory as Uf[entry][lane]), but a work unit computes K <= ZW_KMAX
// neighbouring entries (ma0 .. ma0 + K - 1) of one row of a Z block together.
// For block (a, b, lam), d = (a + b - lam) / 2, and one row pair (mb1, mb2):
//   Z[ma0 + k] += Cb sum_j Ca[j][k] U_a[ma0 + k + d - lo - j, mb1] U_b[lo + j, mb2].
// Step j reads one U_b value and one new U_a value; the K U_a values in use sit
// in a register ring (entry k at step j is the one entry k - 1 had at step j - 1),
// so each shared-memory load feeds up to K products instead of one.
#pragma once

#include "so4_zlanes.cuh"

constexpr int ZW_THREADS = 256;  // 8 warps share one CTA's 32 atoms
constexpr int ZW_TPA = ZW_THREADS / 32;  // threads per atom in the U-tile load

// U tiles with ZW_PAD zero rows before and after: Ub[(ZW_PAD + f) * ZL_PITCH + lane].
// The half rows of the CTA's 32 consecutive atoms are one contiguous run of 32 nh values.
// ZW_TPA threads share an atom (thread t: atom t / ZW_TPA, half entries t % ZW_TPA +
// ZW_TPA i), each reading ZW_LD entries per round with independent loads, then writing
// each to its full-layout position and, below the middle row, to its mirror (hfull);
// atoms past natoms are zero.
constexpr int ZW_LD = 10;
constexpr int ZW_CAR = 8;  // Ca-table float4 per thread read ahead in the prologue
constexpr int ZW_BR = 8;   // beta values per thread read ahead
__device__ __forceinline__ void zw_load_utot(const float2 *__restrict__ utot, const int2 *__restrict__ hfull, int a0,
                                             int natoms, int nh, int nu, float2 *Ub) {
    for (int idx = threadIdx.x; idx < 2 * ZW_PAD * ZL_PITCH; idx += ZW_THREADS) {
        const int r = idx / ZL_PITCH, c = idx - r * ZL_PITCH;
        const int row = (r < ZW_PAD) ? r : nu + r;  // rows 0.. ZW_PAD-1 and ZW_PAD+nu .. nu+2 ZW_PAD-1
        Ub[row * ZL_PITCH + c] = make_float2(0.f, 0.f);
    }
    float2 *Uf = Ub + ZW_PAD * ZL_PITCH;
    const int l = threadIdx.x / ZW_TPA;
    const bool live = a0 + l < natoms;
    const float2 *src = utot + (size_t)(a0 + l) * nh;
    for (int h0 = threadIdx.x % ZW_TPA; h0 < nh; h0 += ZW_TPA * ZW_LD) {
        float2 v[ZW_LD];
#pragma unroll
        for (int r = 0; r < ZW_LD; ++r) {
            const int h = h0 + r * ZW_TPA;
            v[r] = (live && h < nh) ? __ldg(src + h) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < ZW_LD; ++r) {
            const int h = h0 + r * ZW_TPA;
            if (h < nh) {
                const int2 m = __ldg(hfull + h);
                Uf[m.x * ZL_PITCH + l] = v[r];
                if (m.y >= 0) {
                    float2 w = v[r];
                    if (m.y & (1 << 15)) w.y = -w.y;
                    if (m.y & (1 << 14)) {
                        w.x = -w.x;
                        w.y = -w.y;
                    }
                    Uf[(m.y & 0x3fff) * ZL_PITCH + l] = w;
                }
            }
        }
    }
}

// Per-atom sums of scratch slots: the sum of slots [pos[k], pos[k + 1]) of the slot-major
// scratch sc[q * natoms + a0 + l], for every k < ncomp and every l < NA with a0 + l <
// natoms, handed to f(k, l, sum, pre(k, l)).  The CTA (NT threads, NA atoms) copies its
// nslot x NA values into shared memory (stage: nslot x (NA + 1) floats) with independent
// loads, issued together with pre() of the thread's first NPRE (k, l) pairs, then sums from
// there in slot order.
constexpr int ZW_SLD = 24;
template <int NPRE, int NA = 32, int NT = ZW_THREADS, typename P, typename F>
__device__ __forceinline__ void zw_slot_sums(const float *sc, const int *__restrict__ pos, int ncomp, int nslot,
                                             int natoms, int a0, float *stage, P pre, F f) {
    constexpr int SP = NA + 1;
    const int nl = min(NA, natoms - a0);
    float pv[NPRE];
#pragma unroll
    for (int r = 0; r < NPRE; ++r) {
        const int idx = threadIdx.x + r * NT, k = idx / NA, l = idx % NA;
        pv[r] = (idx < NA * ncomp && l < nl) ? pre(k, l) : 0.f;
    }
    for (int i0 = threadIdx.x; i0 < NA * nslot; i0 += ZW_SLD * NT) {
        float v[ZW_SLD];
#pragma unroll
        for (int r = 0; r < ZW_SLD; ++r) {
            const int i = i0 + r * NT, q = i / NA, l = i % NA;
            v[r] = (i < NA * nslot && l < nl) ? sc[(size_t)q * natoms + a0 + l] : 0.f;
        }
#pragma unroll
        for (int r = 0; r < ZW_SLD; ++r) {
            const int i = i0 + r * NT;
            if (i < NA * nslot) stage[(i / NA) * SP + (i % NA)] = v[r];
        }
    }
    __syncthreads();
    auto sum = [&](int k, int l) {
        float acc = 0.f;
        const int q1 = __ldg(pos + k + 1);
        for (int q = __ldg(pos + k); q < q1; ++q) acc += stage[q * SP + l];
        return acc;
    };
#pragma unroll
    for (int r = 0; r < NPRE; ++r) {
        const int idx = threadIdx.x + r * NT, k = idx / NA, l = idx % NA;
        if (idx < NA * ncomp && l < nl) f(k, l, sum(k, l), pv[r]);
    }
    for (int idx = threadIdx.x + NPRE * NT; idx < NA * ncomp; idx += NT) {
        const int k = idx / NA, l = idx % NA;
        if (l < nl) f(k, l, sum(k, l), pre(k, l));
    }
}

// zw_slot_sums without its single staging pass: components are taken in chunks whose slots
// (at most `cap` of them, the slot rows that fit in `stage`) are staged together, summed,
// and the stage reused for the next chunk.  Every component owns at most cap slots (the
// host checks it).  f(k, l, sum) for every k < ncomp and l < NA with a0 + l < natoms.
template <int NA = 32, int NT = ZW_THREADS, typename F>
__device__ __forceinline__ void zw_slot_sums_chunked(const float *sc, const int *__restrict__ pos, int ncomp,
                                                     int natoms, int a0, float *stage, int cap, F f) {
    constexpr int SP = NA + 1;
    const int nl = min(NA, natoms - a0);
    int k0 = 0;
    while (k0 < ncomp) {
        // the chunk [k0, k1): as many whole components as fit (the same k1 in every thread)
        const int q0 = __ldg(pos + k0);
        int k1 = k0 + 1;
        while (k1 < ncomp && __ldg(pos + k1 + 1) - q0 <= cap) ++k1;
        const int nq = __ldg(pos + k1) - q0;
        for (int i0 = threadIdx.x; i0 < NA * nq; i0 += ZW_SLD * NT) {
            float v[ZW_SLD];
#pragma unroll
            for (int r = 0; r < ZW_SLD; ++r) {
                const int i = i0 + r * NT, q = i / NA, l = i % NA;
                v[r] = (i < NA * nq && l < nl) ? sc[(size_t)(q0 + q) * natoms + a0 + l] : 0.f;
            }
#pragma unroll
            for (int r = 0; r < ZW_SLD; ++r) {
                const int i = i0 + r * NT;
                if (i < NA * nq) stage[(i / NA) * SP + (i % NA)] = v[r];
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < NA * (k1 - k0); idx += NT) {
            const int k = k0 + idx / NA, l = idx % NA;
            if (l < nl) {
                float acc = 0.f;
                const int qa = __ldg(pos + k) - q0, qb = __ldg(pos + k + 1) - q0;
                for (int q = qa; q < qb; ++q) acc += stage[q * SP + l];
                f(k, l, acc);
            }
        }
        __syncthreads();  // before the next chunk overwrites the stage
        k0 = k1;
    }
}

// One sub-segment {f1 | f2 << 16, Ca offset, steps S, bits of Cb}: adds
// Cb sum_j Ca[j][k] U_a[f2 - j + k] U_b[f1 + j] to z[k] = (re, im), k < K, for this
// lane's atom (offsets in Ub rows, pre-scaled by the pitch; Ul = Ub + lane).  Ca rows
// hold KP = K rounded up to 4 floats.  Packed FP32 pairs (sm_100+): the ring keeps each
// U_a value w as (w.x, w.x) and (-w.y, w.y), so with a = Cb U_b and as = (a.y, a.x) the
// complex product is (w.x, w.x) * a + (-w.y, w.y) * as, and one more packed FMA adds
// Ca[j][k] times it: three packed instructions per (step, entry).
template <int K>
__device__ __forceinline__ void zw_rows(const float2 *Ul, const int4 hd, const float *__restrict__ ca,
                                        float2 (&z)[K]) {
    constexpr int KQ = (K + 3) / 4;  // float4 loads per Ca row
    const int f1 = hd.x & 0xffff, f2 = (int)((unsigned)hd.x >> 16);
    const int S = hd.z;
    const float cb = __int_as_float(hd.w);
    const float2 cb2 = make_float2(cb, cb);
    const float4 *cw = reinterpret_cast<const float4 *>(ca + hd.y);
    float2 WX[K], WY[K];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const float2 w = Ul[f2 + k * ZL_PITCH];
        WX[k] = make_float2(w.x, w.x);
        WY[k] = make_float2(-w.y, w.y);
    }
    WX[0] = WY[0] = make_float2(0.f, 0.f);
    for (int j0 = 0; j0 < S; j0 += K) {
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int j = j0 + t;
            if (j < S) {
                // ring slot of entry k at step j is (k - j) mod K; entry 0 is new
                const float2 w = Ul[f2 - j * ZL_PITCH];
                WX[(K - t) % K] = make_float2(w.x, w.x);
                WY[(K - t) % K] = make_float2(-w.y, w.y);
                const float2 a = __fmul2_rn(Ul[f1 + j * ZL_PITCH], cb2);
                const float2 as = make_float2(a.y, a.x);
                float cc[4 * KQ];
#pragma unroll
                for (int q = 0; q < KQ; ++q) {
                    const float4 c4 = cw[j * KQ + q];  // shared memory or the read-only global table
                    cc[4 * q] = c4.x;
                    cc[4 * q + 1] = c4.y;
                    cc[4 * q + 2] = c4.z;
                    cc[4 * q + 3] = c4.w;
                }
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const int r = (k - t + K) % K;
                    const float2 p = __ffma2_rn(WY[r], as, __fmul2_rn(WX[r], a));
                    z[k] = __ffma2_rn(make_float2(cc[k], cc[k]), p, z[k]);
                }
            }
        }
    }
}

// Two sub-segments of one segment together.  The rows of a segment share the Ca table
// and the step count S (only f1, f2 and Cb differ), so per (step, entry) the two rows'
// complex products are summed first and Ca[j][k] is applied once: five packed
// instructions for two products instead of six, and the Ca loads serve both rows.
template <int K>
__device__ __forceinline__ void zw_rows2(const float2 *Ul, const int4 h1, const int4 h2,
                                         const float *__restrict__ ca, float2 (&z)[K]) {
    constexpr int KQ = (K + 3) / 4;
    const int f1 = h1.x & 0xffff, f2 = (int)((unsigned)h1.x >> 16);
    const int g1 = h2.x & 0xffff, g2 = (int)((unsigned)h2.x >> 16);
    const int S = h1.z;
    const float cb = __int_as_float(h1.w), db = __int_as_float(h2.w);
    const float2 cb2 = make_float2(cb, cb), db2 = make_float2(db, db);
    const float4 *cw = reinterpret_cast<const float4 *>(ca + h1.y);
    float2 WX[K], WY[K], VX[K], VY[K];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const float2 w = Ul[f2 + k * ZL_PITCH];
        WX[k] = make_float2(w.x, w.x);
        WY[k] = make_float2(-w.y, w.y);
        const float2 v = Ul[g2 + k * ZL_PITCH];
        VX[k] = make_float2(v.x, v.x);
        VY[k] = make_float2(-v.y, v.y);
    }
    WX[0] = WY[0] = VX[0] = VY[0] = make_float2(0.f, 0.f);
    for (int j0 = 0; j0 < S; j0 += K) {
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int j = j0 + t;
            if (j < S) {
                const float2 w = Ul[f2 - j * ZL_PITCH];
                WX[(K - t) % K] = make_float2(w.x, w.x);
                WY[(K - t) % K] = make_float2(-w.y, w.y);
                const float2 v = Ul[g2 - j * ZL_PITCH];
                VX[(K - t) % K] = make_float2(v.x, v.x);
                VY[(K - t) % K] = make_float2(-v.y, v.y);
                const float2 a = __fmul2_rn(Ul[f1 + j * ZL_PITCH], cb2);
                const float2 as = make_float2(a.y, a.x);
                const float2 b = __fmul2_rn(Ul[g1 + j * ZL_PITCH], db2);
                const float2 bs = make_float2(b.y, b.x);
                float cc[4 * KQ];
#pragma unroll
                for (int q = 0; q < KQ; ++q) {
                    const float4 c4 = cw[j * KQ + q];
                    cc[4 * q] = c4.x;
                    cc[4 * q + 1] = c4.y;
                    cc[4 * q + 2] = c4.z;
                    cc[4 * q + 3] = c4.w;
                }
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const int r = (k - t + K) % K;
                    float2 p = __fmul2_rn(WX[r], a);
                    p = __ffma2_rn(WY[r], as, p);
                    p = __ffma2_rn(VX[r], b, p);
                    p = __ffma2_rn(VY[r], bs, p);
                    z[k] = __ffma2_rn(make_float2(cc[k], cc[k]), p, z[k]);
                }
            }
        }
    }
}
