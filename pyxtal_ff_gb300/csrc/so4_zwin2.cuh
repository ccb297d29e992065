// so4_zwin2.cuh -- the window Z pass with two atoms per lane.
//
// A CTA owns 64 consecutive centre atoms; lane l holds atoms l and 32 + l of them.  Their
// U tiles sit in shared memory as one float4 per (entry, lane):
//   Uq[(ZW_PAD + f) * ZL_PITCH + l] = (re U_f(atom l), re U_f(atom 32 + l),
//                                      im U_f(atom l), im U_f(atom 32 + l)),
// so one 16-byte shared load gives a lane the real parts of its two atoms as one packed
// FP32 pair and the imaginary parts as another.  The complex products of the window step
// (so4_zwin.cuh) then take two atoms per packed instruction with both operands as loaded:
// the one-atom layout spends register moves on (w.x, w.x), (-w.y, w.y), (a.y, a.x) per
// value.  The step's headers, Ca loads, address arithmetic and branches serve two atoms.
// Per atom every product and sum is the one of the one-atom kernel, in the same order, so
// both layouts give the same bits.
#pragma once

#include "so4_zwin.cuh"

constexpr int ZW2_ATOMS = 64;
constexpr int ZW2_SP = ZW2_ATOMS + 1;  // stage pitch (floats) of the slot sums

// The two-atom U tiles from U_tot ([natoms][nh] half layout), zero pad rows before and
// after, atoms past natoms zero.  NT / 64 threads share an atom (thread t: atom t / TPA,
// half entries t % TPA + TPA i), each with ZW_LD independent loads per round, then one
// scalar store per real and imaginary part at the entry's full position and its mirror.
template <int NT>
__device__ __forceinline__ void zw2_load_utot(const float2 *__restrict__ utot, const int2 *__restrict__ hfull, int a0,
                                              int natoms, int nh, int nu, float4 *Uq) {
    for (int idx = threadIdx.x; idx < 2 * ZW_PAD * ZL_PITCH; idx += NT) {
        const int r = idx / ZL_PITCH, c = idx - r * ZL_PITCH;
        const int row = (r < ZW_PAD) ? r : nu + r;
        Uq[row * ZL_PITCH + c] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    constexpr int TPA = NT / ZW2_ATOMS;
    float *Uf = reinterpret_cast<float *>(Uq + ZW_PAD * ZL_PITCH);
    const int i = threadIdx.x / TPA;
    const int col = 4 * (i & 31) + (i >> 5);  // float index of the real part within a row
    const bool live = a0 + i < natoms;
    const float2 *src = utot + (size_t)(a0 + i) * nh;
    for (int h0 = threadIdx.x % TPA; h0 < nh; h0 += TPA * ZW_LD) {
        float2 v[ZW_LD];
#pragma unroll
        for (int r = 0; r < ZW_LD; ++r) {
            const int h = h0 + r * TPA;
            v[r] = (live && h < nh) ? __ldg(src + h) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int r = 0; r < ZW_LD; ++r) {
            const int h = h0 + r * TPA;
            if (h < nh) {
                const int2 m = __ldg(hfull + h);
                float *d = Uf + (size_t)m.x * 4 * ZL_PITCH + col;
                d[0] = v[r].x;
                d[2] = v[r].y;
                if (m.y >= 0) {
                    float2 w = v[r];
                    if (m.y & (1 << 15)) w.y = -w.y;
                    if (m.y & (1 << 14)) {
                        w.x = -w.x;
                        w.y = -w.y;
                    }
                    float *e = Uf + (size_t)(m.y & 0x3fff) * 4 * ZL_PITCH + col;
                    e[0] = w.x;
                    e[2] = w.y;
                }
            }
        }
    }
}

// zw_rows for two atoms: adds Cb sum_j Ca[j][k] U_a[f2 - j + k] U_b[f1 + j] to
// (zr[k], zi[k]) = (re, im) of entry k, each a pair over the lane's two atoms.  Per atom,
// with a = Cb U_b: re = fma(-w.y, a.y, w.x a.x), im = fma(w.y, a.x, w.x a.y), then
// z += Ca p, as in zw_rows (the negation is folded into -Cb, which rounds the same).
template <int K>
__device__ __forceinline__ void zw2_rows(const float4 *Ul, const int4 hd, const float *__restrict__ ca,
                                         float2 (&zr)[K], float2 (&zi)[K]) {
    constexpr int KQ = (K + 3) / 4;
    const int f1 = hd.x & 0xffff, f2 = (int)((unsigned)hd.x >> 16);
    const int S = hd.z;
    const float cb = __int_as_float(hd.w);
    const float2 cb2 = make_float2(cb, cb), ncb2 = make_float2(-cb, -cb);
    const float4 *cw = reinterpret_cast<const float4 *>(ca + hd.y);
    float2 WR[K], WI[K];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const float4 w = Ul[f2 + k * ZL_PITCH];
        WR[k] = make_float2(w.x, w.y);
        WI[k] = make_float2(w.z, w.w);
    }
    WR[0] = WI[0] = make_float2(0.f, 0.f);
    for (int j0 = 0; j0 < S; j0 += K) {
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int j = j0 + t;
            if (j < S) {
                const float4 w = Ul[f2 - j * ZL_PITCH];
                WR[(K - t) % K] = make_float2(w.x, w.y);
                WI[(K - t) % K] = make_float2(w.z, w.w);
                const float4 u = Ul[f1 + j * ZL_PITCH];
                const float2 ar = __fmul2_rn(make_float2(u.x, u.y), cb2);
                const float2 ai = __fmul2_rn(make_float2(u.z, u.w), cb2);
                const float2 nai = __fmul2_rn(make_float2(u.z, u.w), ncb2);
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
                    const float2 pr = __ffma2_rn(WI[r], nai, __fmul2_rn(WR[r], ar));
                    const float2 pi = __ffma2_rn(WI[r], ar, __fmul2_rn(WR[r], ai));
                    const float2 c2 = make_float2(cc[k], cc[k]);
                    zr[k] = __ffma2_rn(c2, pr, zr[k]);
                    zi[k] = __ffma2_rn(c2, pi, zi[k]);
                }
            }
        }
    }
}

// zw_rows2 for two atoms: the two rows of a segment together, their products summed in
// the order of zw_rows2 (row 1's two terms, then row 2's) before Ca is applied once.
template <int K>
__device__ __forceinline__ void zw2_rows2(const float4 *Ul, const int4 h1, const int4 h2,
                                          const float *__restrict__ ca, float2 (&zr)[K], float2 (&zi)[K]) {
    constexpr int KQ = (K + 3) / 4;
    const int f1 = h1.x & 0xffff, f2 = (int)((unsigned)h1.x >> 16);
    const int g1 = h2.x & 0xffff, g2 = (int)((unsigned)h2.x >> 16);
    const int S = h1.z;
    const float cb = __int_as_float(h1.w), db = __int_as_float(h2.w);
    const float2 cb2 = make_float2(cb, cb), ncb2 = make_float2(-cb, -cb);
    const float2 db2 = make_float2(db, db), ndb2 = make_float2(-db, -db);
    const float4 *cw = reinterpret_cast<const float4 *>(ca + h1.y);
    float2 WR[K], WI[K], VR[K], VI[K];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const float4 w = Ul[f2 + k * ZL_PITCH];
        WR[k] = make_float2(w.x, w.y);
        WI[k] = make_float2(w.z, w.w);
        const float4 v = Ul[g2 + k * ZL_PITCH];
        VR[k] = make_float2(v.x, v.y);
        VI[k] = make_float2(v.z, v.w);
    }
    WR[0] = WI[0] = VR[0] = VI[0] = make_float2(0.f, 0.f);
    for (int j0 = 0; j0 < S; j0 += K) {
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int j = j0 + t;
            if (j < S) {
                const float4 w = Ul[f2 - j * ZL_PITCH];
                WR[(K - t) % K] = make_float2(w.x, w.y);
                WI[(K - t) % K] = make_float2(w.z, w.w);
                const float4 v = Ul[g2 - j * ZL_PITCH];
                VR[(K - t) % K] = make_float2(v.x, v.y);
                VI[(K - t) % K] = make_float2(v.z, v.w);
                const float4 u = Ul[f1 + j * ZL_PITCH];
                const float2 ar = __fmul2_rn(make_float2(u.x, u.y), cb2);
                const float2 ai = __fmul2_rn(make_float2(u.z, u.w), cb2);
                const float2 nai = __fmul2_rn(make_float2(u.z, u.w), ncb2);
                const float4 x = Ul[g1 + j * ZL_PITCH];
                const float2 br = __fmul2_rn(make_float2(x.x, x.y), db2);
                const float2 bi = __fmul2_rn(make_float2(x.z, x.w), db2);
                const float2 nbi = __fmul2_rn(make_float2(x.z, x.w), ndb2);
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
                    float2 pr = __fmul2_rn(WR[r], ar);
                    pr = __ffma2_rn(WI[r], nai, pr);
                    pr = __ffma2_rn(VR[r], br, pr);
                    pr = __ffma2_rn(VI[r], nbi, pr);
                    float2 pi = __fmul2_rn(WR[r], ai);
                    pi = __ffma2_rn(WI[r], ar, pi);
                    pi = __ffma2_rn(VR[r], bi, pi);
                    pi = __ffma2_rn(VI[r], br, pi);
                    const float2 c2 = make_float2(cc[k], cc[k]);
                    zr[k] = __ffma2_rn(c2, pr, zr[k]);
                    zi[k] = __ffma2_rn(c2, pi, zi[k]);
                }
            }
        }
    }
}
