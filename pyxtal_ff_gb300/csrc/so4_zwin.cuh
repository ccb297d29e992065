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

// U tiles with ZW_PAD zero rows before and after: Ub[(ZW_PAD + f) * ZL_PITCH + lane]
__device__ __forceinline__ void zw_load_utot(const float2 *__restrict__ utot, const int *__restrict__ fmap, int a0,
                                             int natoms, int nh, int nu, float2 *Ub) {
    for (int idx = threadIdx.x; idx < 2 * ZW_PAD * ZL_PITCH; idx += blockDim.x) {
        const int r = idx / ZL_PITCH, c = idx - r * ZL_PITCH;
        const int row = (r < ZW_PAD) ? r : nu + r;  // rows 0.. ZW_PAD-1 and ZW_PAD+nu .. nu+2 ZW_PAD-1
        Ub[row * ZL_PITCH + c] = make_float2(0.f, 0.f);
    }
    zl_load_utot(utot, fmap, a0, natoms, nh, nu, Ub + ZW_PAD * ZL_PITCH);
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
