// so4_rowchain.cuh -- register-resident U / dU recursion, one row chain per lane.
//
// Row mb of level l depends only on row mb of level l-1 (the recursion of
// compute_uarray_recursive, pyxtal_ff/descriptors/SO4.py:888-906), except that
// the middle row of an even level l = 2mb starts from row mb-1 of level l-1,
// mirrored by the inversion symmetry (:908-925).  So each lane owns one chain
// mb = 0..TWOL/2 of one image and keeps its row (U and the three dU/dr
// components) in registers from level 2mb up to TWOL, updated in place; the
// only exchange is one shuffle of the previous chain's row at the chain start.
// TWOL is a template parameter so every row index is a compile-time constant.
#pragma once

#include "so4_common.cuh"

// sqrt(k) for k = 0..16, the numerators of rootpq[p][q] = sqrt(p / q)
__constant__ float c_sqrtk[17] = {0.0f,
                                  1.0f,
                                  1.41421356237309515f,
                                  1.73205080756887719f,
                                  2.0f,
                                  2.23606797749978981f,
                                  2.44948974278317788f,
                                  2.64575131106459072f,
                                  2.82842712474619029f,
                                  3.0f,
                                  3.16227766016837952f,
                                  3.31662479035539981f,
                                  3.46410161513775439f,
                                  3.60555127546398912f,
                                  3.74165738677394133f,
                                  3.87298334620741702f,
                                  4.0f};

template <int TWOL>
struct RowChain {
    static constexpr int NCH = TWOL / 2 + 1;   // chains per image
    static constexpr int IPW = 32 / NCH;       // images per warp
    static constexpr int W = TWOL + 1;         // longest row
};

// Advance one image's chain `mb` from level L-1 to level L (in place).
// u, d0, d1, d2: the row (re, im) of U and of dU/dx, dU/dy, dU/dz.
template <int TWOL, int L, bool DERIV>
__device__ __forceinline__ void rc_level(int mb, const CK<float> &ck, float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                         float (&dr)[3][TWOL + 1], float (&di)[3][TWOL + 1]) {
    // 1 / sqrt(l - mb); lanes whose chain has not started (mb > L/2) compute values nobody reads
    const float inv_q = rsqrtf((float)max(L - mb, 1));
    // descending in place: new[ma] uses old[ma] (a-term) and old[ma-1] (b-term)
#pragma unroll
    for (int ma = L; ma >= 0; --ma) {
        float vr = 0.f, vi = 0.f;
        float er[3] = {0.f, 0.f, 0.f}, ei[3] = {0.f, 0.f, 0.f};
        if (ma > 0) {
            const float rp = -c_sqrtk[ma] * inv_q;
            const float pr = ur[ma - 1], pi = ui[ma - 1];
            // conj(b) * P
            const float br = ck.cb.re * pr - ck.cb.im * pi;
            const float bi = ck.cb.re * pi + ck.cb.im * pr;
            vr = rp * br;
            vi = rp * bi;
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float qr = dr[c][ma - 1], qi = di[c][ma - 1];
                    const float tr = ck.cdb[c].re * pr - ck.cdb[c].im * pi + ck.cb.re * qr - ck.cb.im * qi;
                    const float ti = ck.cdb[c].re * pi + ck.cdb[c].im * pr + ck.cb.re * qi + ck.cb.im * qr;
                    er[c] = rp * tr;
                    ei[c] = rp * ti;
                }
            }
        }
        if (ma < L) {
            const float rp = c_sqrtk[L - ma] * inv_q;
            const float pr = ur[ma], pi = ui[ma];
            const float ar = ck.ca.re * pr - ck.ca.im * pi;
            const float ai = ck.ca.re * pi + ck.ca.im * pr;
            vr += rp * ar;
            vi += rp * ai;
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float qr = dr[c][ma], qi = di[c][ma];
                    const float tr = ck.cda[c].re * pr - ck.cda[c].im * pi + ck.ca.re * qr - ck.ca.im * qi;
                    const float ti = ck.cda[c].re * pi + ck.cda[c].im * pr + ck.ca.re * qi + ck.ca.im * qr;
                    er[c] += rp * tr;
                    ei[c] += rp * ti;
                }
            }
        }
        ur[ma] = vr;
        ui[ma] = vi;
        if (DERIV) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                dr[c][ma] = er[c];
                di[c][ma] = ei[c];
            }
        }
    }
    if ((L & 1) == 0 && 2 * mb == L) {
        // middle row: centre -> conj, upper half -> (-1)^(L/2+ma) conj(lower mirror)
        constexpr int H = L / 2;
        ui[H] = -ui[H];
        if (DERIV) {
#pragma unroll
            for (int c = 0; c < 3; ++c) di[c][H] = -di[c][H];
        }
#pragma unroll
        for (int ma = H + 1; ma <= L; ++ma) {
            const float s = ((H + ma) & 1) ? -1.f : 1.f;
            ur[ma] = s * ur[L - ma];
            ui[ma] = -s * ui[L - ma];
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    dr[c][ma] = s * dr[c][L - ma];
                    di[c][ma] = -s * di[c][L - ma];
                }
            }
        }
    }
}

// At an even level L the chain mb = L/2 starts: its previous row is row L/2 of
// level L-1, i.e. the mirror of row L/2-1 of level L-1 held by lane-1:
//   P[c] = (-1)^(L/2 + c) conj(row_{L/2-1}[L-1-c]),  c = 0..L-1.
// Every lane shuffles (the warp stays converged); only mb == L/2 keeps the
// values.  The source lane is never the taking lane, so writing slot c while
// later shuffles read slots L-1-c of lane-1 is safe.
template <int TWOL, int L, bool DERIV>
__device__ __forceinline__ void rc_start(int mb, float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                         float (&dr)[3][TWOL + 1], float (&di)[3][TWOL + 1]) {
    constexpr int H = L / 2;
    const bool take = (mb == H);
#pragma unroll
    for (int c = 0; c < L; ++c) {
        const float s = ((H + c) & 1) ? -1.f : 1.f;
        const float vr = __shfl_up_sync(0xffffffffu, ur[L - 1 - c], 1);
        const float vi = __shfl_up_sync(0xffffffffu, ui[L - 1 - c], 1);
        if (take) {
            ur[c] = s * vr;
            ui[c] = -s * vi;
        }
        if (DERIV) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float wr = __shfl_up_sync(0xffffffffu, dr[k][L - 1 - c], 1);
                const float wi = __shfl_up_sync(0xffffffffu, di[k][L - 1 - c], 1);
                if (take) {
                    dr[k][c] = s * wr;
                    di[k][c] = -s * wi;
                }
            }
        }
    }
}

// offset of level L in the half layout: sum_{l<L} (l/2+1)(l+1)
__host__ __device__ constexpr int half_block(int L) { return L == 0 ? 0 : half_block(L - 1) + ((L - 1) / 2 + 1) * L; }

// Levels L..TWOL of the recursion with, after each level, the contraction of
// the lane's row with the adjoint array Y (half layout of one centre):
//   su += Re conj(U) Y,  sc += Re conj(dU_c) Y.
template <int TWOL, int L>
struct RcDeidrj {
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, const float2 *__restrict__ Y,
                                               float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                               float (&dr)[3][TWOL + 1], float (&di)[3][TWOL + 1], float &su,
                                               float (&sc)[3]) {
        if ((L & 1) == 0) rc_start<TWOL, L, true>(mb, ur, ui, dr, di);
        rc_level<TWOL, L, true>(mb, ck, ur, ui, dr, di);
        if (2 * mb <= L) {
            const float2 *Yl = Y + half_block(L) + mb * (L + 1);
#pragma unroll
            for (int ma = 0; ma <= L; ++ma) {
                const float2 y = __ldg(Yl + ma);
                su += ur[ma] * y.x + ui[ma] * y.y;
#pragma unroll
                for (int c = 0; c < 3; ++c) sc[c] += dr[c][ma] * y.x + di[c][ma] * y.y;
            }
        }
        RcDeidrj<TWOL, L + 1>::run(mb, ck, Y, ur, ui, dr, di, su, sc);
    }
};
template <int TWOL>
struct RcDeidrj<TWOL, TWOL + 1> {
    __device__ __forceinline__ static void run(int, const CK<float> &, const float2 *, float (&)[TWOL + 1],
                                               float (&)[TWOL + 1], float (&)[3][TWOL + 1],
                                               float (&)[3][TWOL + 1], float &, float (&)[3]) {}
};

// centre atom of image m: the largest i with img_ptr[i] <= m
__device__ __forceinline__ int centre_of(const int32_t *img_ptr, int natoms, int m) {
    int lo = 0, hi = natoms - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(img_ptr + mid) <= m) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// offset of level L in a lane's accumulator: sum_{l<L} (l+1)
__host__ __device__ constexpr int acc_block(int L) { return L * (L + 1) / 2; }

// Levels L..TWOL of the U recursion (no derivatives); after each level the
// lane adds w sfac U of its row into its accumulator for that level.
template <int TWOL, int L>
struct RcUtot {
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, float wsf, float (&ur)[TWOL + 1],
                                               float (&ui)[TWOL + 1], float (&dr)[3][TWOL + 1],
                                               float (&di)[3][TWOL + 1], float (&accr)[acc_block(TWOL + 1)],
                                               float (&acci)[acc_block(TWOL + 1)]) {
        if ((L & 1) == 0) rc_start<TWOL, L, false>(mb, ur, ui, dr, di);
        rc_level<TWOL, L, false>(mb, ck, ur, ui, dr, di);
        if (2 * mb <= L) {
#pragma unroll
            for (int ma = 0; ma <= L; ++ma) {
                accr[acc_block(L) + ma] += wsf * ur[ma];
                acci[acc_block(L) + ma] += wsf * ui[ma];
            }
        }
        RcUtot<TWOL, L + 1>::run(mb, ck, wsf, ur, ui, dr, di, accr, acci);
    }
};
template <int TWOL>
struct RcUtot<TWOL, TWOL + 1> {
    __device__ __forceinline__ static void run(int, const CK<float> &, float, float (&)[TWOL + 1], float (&)[TWOL + 1],
                                               float (&)[3][TWOL + 1], float (&)[3][TWOL + 1],
                                               float (&)[acc_block(TWOL + 1)], float (&)[acc_block(TWOL + 1)]) {}
};

// Levels L..TWOL with derivatives; after each level the lane adds the
// directional derivative of its row along the image displacement dr_m,
//   w (sfac sum_c dU_c dr_c + dsfac (r^ . dr) U),
// into its accumulator (the tangent of U_tot used by the JVP).
template <int TWOL, int L>
struct RcJvp {
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, float a_du, float a_dx, float a_dy,
                                               float a_dz, float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                               float (&dr)[3][TWOL + 1], float (&di)[3][TWOL + 1],
                                               float (&accr)[acc_block(TWOL + 1)], float (&acci)[acc_block(TWOL + 1)]) {
        if ((L & 1) == 0) rc_start<TWOL, L, true>(mb, ur, ui, dr, di);
        rc_level<TWOL, L, true>(mb, ck, ur, ui, dr, di);
        if (2 * mb <= L) {
#pragma unroll
            for (int ma = 0; ma <= L; ++ma) {
                accr[acc_block(L) + ma] += a_du * ur[ma] + a_dx * dr[0][ma] + a_dy * dr[1][ma] + a_dz * dr[2][ma];
                acci[acc_block(L) + ma] += a_du * ui[ma] + a_dx * di[0][ma] + a_dy * di[1][ma] + a_dz * di[2][ma];
            }
        }
        RcJvp<TWOL, L + 1>::run(mb, ck, a_du, a_dx, a_dy, a_dz, ur, ui, dr, di, accr, acci);
    }
};
template <int TWOL>
struct RcJvp<TWOL, TWOL + 1> {
    __device__ __forceinline__ static void run(int, const CK<float> &, float, float, float, float, float (&)[TWOL + 1],
                                               float (&)[TWOL + 1], float (&)[3][TWOL + 1], float (&)[3][TWOL + 1],
                                               float (&)[acc_block(TWOL + 1)], float (&)[acc_block(TWOL + 1)]) {}
};
