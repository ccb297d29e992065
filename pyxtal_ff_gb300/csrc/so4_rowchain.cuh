// so4_rowchain.cuh -- register-resident U / dU recursion, one row chain per lane.
//
// Row mb of level l depends only on row mb of level l-1 (the recursion of
// compute_uarray_recursive, pyxtal_ff/descriptors/SO4.py:888-906), except that
// the middle row of an even level l = 2mb starts from row mb-1 of level l-1,
// mirrored by the inversion symmetry (:908-925).  So each lane owns one chain
// mb = 0..TWOL/2 of one image and keeps its row (U, and for the JVP the three
// dU/dr components) in registers from level 2mb up to TWOL, updated in place;
// the only exchange is one shuffle of the previous chain's row at the chain start.
// TWOL is a template parameter so every row index is a compile-time constant.
//
// Rows are carried scaled: V_l[ma] = U_l[ma][mb] sqrt(C(l, ma) / C(l, mb)) (C the
// binomial coefficient).  The reference's step
//   U_l[ma] = sqrt(l-ma)/sqrt(l-mb) conj(a) U_{l-1}[ma] - sqrt(ma)/sqrt(l-mb) conj(b) U_{l-1}[ma-1]
// then reads V_l[ma] = conj(a) V_{l-1}[ma] - conj(b) V_{l-1}[ma-1] (the square roots
// cancel against the scale), while the chain-start mirror and the middle-row
// symmetry hold unchanged because C(l, ma) = C(l, l - ma).  Consumers undo the scale
// per half entry: the U_tot epilogue through its table, the reverse sweep by reading
// a Y that the window kernel scaled by the same factor.
#pragma once

#include "so4_common.cuh"

template <int TWOL>
struct RowChain {
    static constexpr int NCH = TWOL / 2 + 1;   // chains per image
    static constexpr int IPW = 32 / NCH;       // images per warp
    static constexpr int W = TWOL + 1;         // longest row
};

// Advance one image's chain `mb` from level L-1 to level L (in place), scaled rows:
// V_L[ma] = conj(a) V_{L-1}[ma] - conj(b) V_{L-1}[ma-1].
// u, d0, d1, d2: the row (re, im) of V and of dV/dx, dV/dy, dV/dz.  Lanes whose chain
// has not started (mb > L/2) compute values nobody reads.
template <int TWOL, int L, bool DERIV, int NDER = 3>
__device__ __forceinline__ void rc_level(int mb, const CK<float> &ck, float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                         float (&dr)[NDER][TWOL + 1], float (&di)[NDER][TWOL + 1]) {
    // descending in place: new[ma] uses old[ma] (a-term) and old[ma-1] (b-term)
#pragma unroll
    for (int ma = L; ma >= 0; --ma) {
        float vr = 0.f, vi = 0.f;
        float er[NDER], ei[NDER];
#pragma unroll
        for (int c = 0; c < NDER; ++c) er[c] = ei[c] = 0.f;
        if (ma > 0) {
            // - conj(b) * P[ma-1]
            const float pr = ur[ma - 1], pi = ui[ma - 1];
            vr = fmaf(ck.cb.im, pi, -ck.cb.re * pr);
            vi = fmaf(-ck.cb.im, pr, -ck.cb.re * pi);
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < NDER; ++c) {
                    const float qr = dr[c][ma - 1], qi = di[c][ma - 1];
                    er[c] = -(ck.cdb[c].re * pr - ck.cdb[c].im * pi + ck.cb.re * qr - ck.cb.im * qi);
                    ei[c] = -(ck.cdb[c].re * pi + ck.cdb[c].im * pr + ck.cb.re * qi + ck.cb.im * qr);
                }
            }
        }
        if (ma < L) {
            // + conj(a) * P[ma]
            const float pr = ur[ma], pi = ui[ma];
            vr = fmaf(ck.ca.re, pr, fmaf(-ck.ca.im, pi, vr));
            vi = fmaf(ck.ca.re, pi, fmaf(ck.ca.im, pr, vi));
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < NDER; ++c) {
                    const float qr = dr[c][ma], qi = di[c][ma];
                    er[c] += ck.cda[c].re * pr - ck.cda[c].im * pi + ck.ca.re * qr - ck.ca.im * qi;
                    ei[c] += ck.cda[c].re * pi + ck.cda[c].im * pr + ck.ca.re * qi + ck.ca.im * qr;
                }
            }
        }
        ur[ma] = vr;
        ui[ma] = vi;
        if (DERIV) {
#pragma unroll
            for (int c = 0; c < NDER; ++c) {
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
            for (int c = 0; c < NDER; ++c) di[c][H] = -di[c][H];
        }
#pragma unroll
        for (int ma = H + 1; ma <= L; ++ma) {
            const float s = ((H + ma) & 1) ? -1.f : 1.f;
            ur[ma] = s * ur[L - ma];
            ui[ma] = -s * ui[L - ma];
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < NDER; ++c) {
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
template <int TWOL, int L, bool DERIV, int NDER = 3>
__device__ __forceinline__ void rc_start(int mb, float (&ur)[TWOL + 1], float (&ui)[TWOL + 1],
                                         float (&dr)[NDER][TWOL + 1], float (&di)[NDER][TWOL + 1]) {
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
            for (int k = 0; k < NDER; ++k) {
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

// centre atom of image m: the largest i with img_ptr[i] <= m (img_ptr[0] = mbase <= m <
// img_ptr[natoms], mtot images).  The search starts from the guess
// (m - mbase) * natoms / mtot (images per centre are close to
// uniform in practice) and gallops outwards before bisecting, so the chain of
// dependent loads is a few steps instead of log2(natoms).
__device__ __forceinline__ int centre_of(const int32_t *img_ptr, int natoms, int m, int mbase, int64_t mtot) {
    int g = (int)(((int64_t)(m - mbase) * natoms) / (mtot > 0 ? mtot : 1));
    g = min(max(g, 0), natoms - 1);
    int lo, hi;  // img_ptr[lo] <= m < img_ptr[hi] (img_ptr[natoms] > m)
    if (__ldg(img_ptr + g) <= m) {
        lo = g;
        hi = g + 1;
        int step = 1;
        while (hi < natoms && __ldg(img_ptr + hi) <= m) {
            lo = hi;
            step <<= 1;
            hi = min(lo + step, natoms);
        }
    } else {
        hi = g;
        lo = g - 1;  // g > 0 here, since img_ptr[0] = 0 <= m
        int step = 1;
        while (lo > 0 && __ldg(img_ptr + lo) > m) {
            hi = lo;
            step <<= 1;
            lo = max(hi - step, 0);
        }
    }
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(img_ptr + mid) <= m)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// offset of level L in a lane's accumulator: sum_{l<L} (l+1)
__host__ __device__ constexpr int acc_block(int L) { return L * (L + 1) / 2; }

// ---------------------------------------------------------------------------
// U_tot (no derivatives), rows as (re, im) pairs so that the weighted accumulation is one
// packed FMA per entry; the recursion and the chain start are rc_level / rc_start's own
// operations on the pair's halves.
//
// Lanes per image: one per row chain, except at TWOL 8, where the last lane of an image
// runs chains 3 and 4 (UtotLanes::LPI = 4, eight images per pass instead of six): chain 4
// exists at level 8 only and starts from chain 3's row of level 7, which that lane holds.
// Its accumulators take chain 4's level-8 row in slots 0..8, which chain 3 (levels 6..8,
// slots acc_block(6)..) leaves free.
template <int TWOL>
struct UtotLanes {
    static constexpr int NCH = TWOL / 2 + 1;
    static constexpr bool PAIR = (TWOL == 8);  // the last lane also runs the last chain
    static constexpr int LPI = PAIR ? NCH - 1 : NCH;  // lanes per image
    static constexpr int IPW = 32 / LPI;              // images per pass
    // lane (within the image) and accumulator slot of the entry (chain mb, level L, ma)
    __host__ __device__ static constexpr int lane_of(int mb) { return (PAIR && mb == NCH - 1) ? LPI - 1 : mb; }
    __host__ __device__ static constexpr int slot_of(int mb, int slot) {
        return (PAIR && mb == NCH - 1) ? slot - acc_block(TWOL) : slot;
    }
};

template <int TWOL, int L>
__device__ __forceinline__ void rc2_level(int mb, const CK<float> &ck, float2 (&u)[TWOL + 1]) {
#pragma unroll
    for (int ma = L; ma >= 0; --ma) {
        float vr = 0.f, vi = 0.f;
        if (ma > 0) {
            const float pr = u[ma - 1].x, pi = u[ma - 1].y;
            vr = fmaf(ck.cb.im, pi, -ck.cb.re * pr);
            vi = fmaf(-ck.cb.im, pr, -ck.cb.re * pi);
        }
        if (ma < L) {
            const float pr = u[ma].x, pi = u[ma].y;
            vr = fmaf(ck.ca.re, pr, fmaf(-ck.ca.im, pi, vr));
            vi = fmaf(ck.ca.re, pi, fmaf(ck.ca.im, pr, vi));
        }
        u[ma] = make_float2(vr, vi);
    }
    if ((L & 1) == 0 && 2 * mb == L) {
        constexpr int H = L / 2;
        u[H].y = -u[H].y;
#pragma unroll
        for (int ma = H + 1; ma <= L; ++ma) {
            const float s = ((H + ma) & 1) ? -1.f : 1.f;
            u[ma] = make_float2(s * u[L - ma].x, -s * u[L - ma].y);
        }
    }
}

// the start of chain H = L/2 from row H-1 of level L-1, mirrored: from lane - 1 (shuffle)
template <int TWOL, int L>
__device__ __forceinline__ void rc2_start(int mb, float2 (&u)[TWOL + 1]) {
    constexpr int H = L / 2;
    const bool take = (mb == H);
#pragma unroll
    for (int c = 0; c < L; ++c) {
        const float s = ((H + c) & 1) ? -1.f : 1.f;
        const float vr = __shfl_up_sync(0xffffffffu, u[L - 1 - c].x, 1);
        const float vi = __shfl_up_sync(0xffffffffu, u[L - 1 - c].y, 1);
        if (take) u[c] = make_float2(s * vr, -s * vi);
    }
}

// The last chain (H = TWOL/2) at level TWOL, from the previous chain's row of level
// TWOL-1 held in u (and its derivative along one direction in du), entry by entry and
// without a row of its own: P[c] = (-1)^(H+c) conj(u[TWOL-1-c]) is the start row, the
// entries ma <= H are rc_level's recursion, the centre is conjugated and the upper half
// is the middle-row mirror.  Adds wu V[ma] (+ wd dV[ma]) to acc[ma], ma = 0..TWOL.
template <int TWOL, bool DERIV>
__device__ __forceinline__ void rc2_last_chain(const CK<float> &ck, const float2 (&u)[TWOL + 1],
                                               const float2 (&du)[TWOL + 1], float wu, float wd,
                                               float2 (&acc)[acc_block(TWOL + 1)]) {
    constexpr int L = TWOL, H = L / 2;
    const float2 w2 = make_float2(wu, wu), d2 = make_float2(wd, wd);
    auto sgn = [](int c) { return ((H + c) & 1) ? -1.f : 1.f; };
#pragma unroll
    for (int ma = 0; ma <= H; ++ma) {
        float vr = 0.f, vi = 0.f, er = 0.f, ei = 0.f;
        if (ma > 0) {
            const float s = sgn(ma - 1);
            const float pr = s * u[L - ma].x, pi = -s * u[L - ma].y;
            vr = fmaf(ck.cb.im, pi, -ck.cb.re * pr);
            vi = fmaf(-ck.cb.im, pr, -ck.cb.re * pi);
            if (DERIV) {
                const float qr = s * du[L - ma].x, qi = -s * du[L - ma].y;
                er = -(ck.cdb[0].re * pr - ck.cdb[0].im * pi + ck.cb.re * qr - ck.cb.im * qi);
                ei = -(ck.cdb[0].re * pi + ck.cdb[0].im * pr + ck.cb.re * qi + ck.cb.im * qr);
            }
        }
        {
            const float s = sgn(ma);
            const float pr = s * u[L - 1 - ma].x, pi = -s * u[L - 1 - ma].y;
            vr = fmaf(ck.ca.re, pr, fmaf(-ck.ca.im, pi, vr));
            vi = fmaf(ck.ca.re, pi, fmaf(ck.ca.im, pr, vi));
            if (DERIV) {
                const float qr = s * du[L - 1 - ma].x, qi = -s * du[L - 1 - ma].y;
                er += ck.cda[0].re * pr - ck.cda[0].im * pi + ck.ca.re * qr - ck.ca.im * qi;
                ei += ck.cda[0].re * pi + ck.cda[0].im * pr + ck.ca.re * qi + ck.ca.im * qr;
            }
        }
        if (ma == H) {
            vi = -vi;
            ei = -ei;
        }
        float2 a = __ffma2_rn(w2, make_float2(vr, vi), acc[ma]);
        if (DERIV) a = __ffma2_rn(d2, make_float2(er, ei), a);
        acc[ma] = a;
        if (ma < H) {
            // the mirror entry L - ma: (-1)^(H + L - ma) conj(V[ma])
            const float m = sgn(L - ma);
            float2 b = __ffma2_rn(w2, make_float2(m * vr, -m * vi), acc[L - ma]);
            if (DERIV) b = __ffma2_rn(d2, make_float2(m * er, -m * ei), b);
            acc[L - ma] = b;
        }
    }
}

// Levels L..TWOL of one image's chain mb (lane chain; with UtotLanes::PAIR the lane of
// chain NCH-2 also runs chain NCH-1 at level TWOL), accumulating wsf times each row.
template <int TWOL, int L>
struct RcUtot2 {
    using UL = UtotLanes<TWOL>;
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, float wsf, float2 (&u)[TWOL + 1],
                                               float2 (&acc)[acc_block(TWOL + 1)]) {
        const float2 w2 = make_float2(wsf, wsf);
        if constexpr (UL::PAIR && L == TWOL) {
            if (mb == L / 2 - 1) rc2_last_chain<TWOL, false>(ck, u, u, wsf, 0.f, acc);
        } else if constexpr ((L & 1) == 0) {
            rc2_start<TWOL, L>(mb, u);
        }
        rc2_level<TWOL, L>(mb, ck, u);
        if (2 * mb <= L) {
#pragma unroll
            for (int ma = 0; ma <= L; ++ma) acc[acc_block(L) + ma] = __ffma2_rn(w2, u[ma], acc[acc_block(L) + ma]);
        }
        RcUtot2<TWOL, L + 1>::run(mb, ck, wsf, u, acc);
    }
};
template <int TWOL>
struct RcUtot2<TWOL, TWOL + 1> {
    __device__ __forceinline__ static void run(int, const CK<float> &, float, float2 (&)[TWOL + 1],
                                               float2 (&)[acc_block(TWOL + 1)]) {}
};

// rc2_level with the derivative along one direction (ck.cda[0], ck.cdb[0]): du is the
// row of dV, updated with rc_level's expressions
template <int TWOL, int L>
__device__ __forceinline__ void rc2_level_d(int mb, const CK<float> &ck, float2 (&u)[TWOL + 1],
                                            float2 (&du)[TWOL + 1]) {
#pragma unroll
    for (int ma = L; ma >= 0; --ma) {
        float vr = 0.f, vi = 0.f, er = 0.f, ei = 0.f;
        if (ma > 0) {
            const float pr = u[ma - 1].x, pi = u[ma - 1].y, qr = du[ma - 1].x, qi = du[ma - 1].y;
            vr = fmaf(ck.cb.im, pi, -ck.cb.re * pr);
            vi = fmaf(-ck.cb.im, pr, -ck.cb.re * pi);
            er = -(ck.cdb[0].re * pr - ck.cdb[0].im * pi + ck.cb.re * qr - ck.cb.im * qi);
            ei = -(ck.cdb[0].re * pi + ck.cdb[0].im * pr + ck.cb.re * qi + ck.cb.im * qr);
        }
        if (ma < L) {
            const float pr = u[ma].x, pi = u[ma].y, qr = du[ma].x, qi = du[ma].y;
            vr = fmaf(ck.ca.re, pr, fmaf(-ck.ca.im, pi, vr));
            vi = fmaf(ck.ca.re, pi, fmaf(ck.ca.im, pr, vi));
            er += ck.cda[0].re * pr - ck.cda[0].im * pi + ck.ca.re * qr - ck.ca.im * qi;
            ei += ck.cda[0].re * pi + ck.cda[0].im * pr + ck.ca.re * qi + ck.ca.im * qr;
        }
        u[ma] = make_float2(vr, vi);
        du[ma] = make_float2(er, ei);
    }
    if ((L & 1) == 0 && 2 * mb == L) {
        constexpr int H = L / 2;
        u[H].y = -u[H].y;
        du[H].y = -du[H].y;
#pragma unroll
        for (int ma = H + 1; ma <= L; ++ma) {
            const float s = ((H + ma) & 1) ? -1.f : 1.f;
            u[ma] = make_float2(s * u[L - ma].x, -s * u[L - ma].y);
            du[ma] = make_float2(s * du[L - ma].x, -s * du[L - ma].y);
        }
    }
}

// the JVP's tangent of U_tot: levels L..TWOL of chain mb with the derivative along the
// image's tangent, adding a_du V + a_d dV of each row (lanes as in RcUtot2)
template <int TWOL, int L>
struct RcJvp2 {
    using UL = UtotLanes<TWOL>;
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, float a_du, float a_d, float2 (&u)[TWOL + 1],
                                               float2 (&du)[TWOL + 1], float2 (&acc)[acc_block(TWOL + 1)]) {
        if constexpr (UL::PAIR && L == TWOL) {
            if (mb == L / 2 - 1) rc2_last_chain<TWOL, true>(ck, u, du, a_du, a_d, acc);
        } else if constexpr ((L & 1) == 0) {
            rc2_start<TWOL, L>(mb, u);
            rc2_start<TWOL, L>(mb, du);
        }
        rc2_level_d<TWOL, L>(mb, ck, u, du);
        if (2 * mb <= L) {
            const float2 w2 = make_float2(a_du, a_du), d2 = make_float2(a_d, a_d);
#pragma unroll
            for (int ma = 0; ma <= L; ++ma)
                acc[acc_block(L) + ma] = __ffma2_rn(d2, du[ma], __ffma2_rn(w2, u[ma], acc[acc_block(L) + ma]));
        }
        RcJvp2<TWOL, L + 1>::run(mb, ck, a_du, a_d, u, du, acc);
    }
};
template <int TWOL>
struct RcJvp2<TWOL, TWOL + 1> {
    __device__ __forceinline__ static void run(int, const CK<float> &, float, float, float2 (&)[TWOL + 1],
                                               float2 (&)[TWOL + 1], float2 (&)[acc_block(TWOL + 1)]) {}
};

// ---------------------------------------------------------------------------
// Reverse mode.  The contraction the adjoint needs per image,
//   f = sum_half Re(conj(U) Y)  and  df/dr_c = sum_half Re(conj(dU/dr_c) Y),
// depends on r only through a and b, so one backward sweep of Y through the
// recursion gives the gradients G_ca, G_cb of f with respect to conj(a) and
// conj(b) (real-gradient convention G_z = df/dRe z + i df/dIm z), and then
//   df/dr_c = Re(conj(G_ca) d conj(a)/dr_c) + Re(conj(G_cb) d conj(b)/dr_c)
// -- about half the arithmetic of carrying dU/dx, dU/dy, dU/dz forward.
// The forward sweep stores every row a lane computes (levels 2mb .. TWOL, and at
// a chain start the mirrored row it started from, as level 2mb - 1) in shared
// memory at st[(acc_block(L) + ma) * NT] (NT = threads per CTA, st = base + tid).
template <int TWOL, int L, int NT>
struct RvFwd {
    __device__ __forceinline__ static void run(int mb, const CK<float> &ck, float (&ur)[TWOL + 1],
                                               float (&ui)[TWOL + 1], float2 *st) {
        float dr[3][TWOL + 1], di[3][TWOL + 1];  // unused (no derivatives)
        if ((L & 1) == 0) {
            rc_start<TWOL, L, false>(mb, ur, ui, dr, di);
            if (mb == L / 2) {
#pragma unroll
                for (int c = 0; c < L; ++c) st[(acc_block(L - 1) + c) * NT] = make_float2(ur[c], ui[c]);
            }
        }
        rc_level<TWOL, L, false>(mb, ck, ur, ui, dr, di);
#pragma unroll
        for (int ma = 0; ma <= L; ++ma) st[(acc_block(L) + ma) * NT] = make_float2(ur[ma], ui[ma]);
        RvFwd<TWOL, L + 1, NT>::run(mb, ck, ur, ui, st);
    }
};
template <int TWOL, int NT>
struct RvFwd<TWOL, TWOL + 1, NT> {
    __device__ __forceinline__ static void run(int, const CK<float> &, float (&)[TWOL + 1], float (&)[TWOL + 1],
                                               float2 *) {}
};

// Backward sweep, level L down to 1, in packed FP32 pairs.  g: on entry the adjoint of
// this lane's row of level L arriving from level L + 1; on exit that of its row of level
// L - 1.  Adds Y's row, forms f, back-propagates through the middle-row construction and
// the recursion.  Sums are kept as elementwise pairs and folded by the caller:
//   f = su.x + su.y,  G_ca = (sa1.x + sa1.y, sa2.x - sa2.y),
//   G_cb = -(sb1.x + sb1.y, sb2.x - sb2.y).
// With a = conj(conj a) = (ar, ai), b = (br, bi): AX = (ar, ar), AYn = (-ai, ai),
// BXn = (-br, -br), BY = (bi, -bi), so that a g = AX g + AYn swap(g) and
// -b h = BXn h + BY swap(h) (elementwise products, swap(v) = (v.y, v.x)).
struct RvPairs {
    float2 ax, ayn, bxn, by;
};
__device__ __forceinline__ RvPairs rv_pairs(const CK<float> &ck) {
    const float ar = ck.ca.re, ai = -ck.ca.im, br = ck.cb.re, bi = -ck.cb.im;
    RvPairs q;
    q.ax = make_float2(ar, ar);
    q.ayn = make_float2(-ai, ai);
    q.bxn = make_float2(-br, -br);
    q.by = make_float2(bi, -bi);
    return q;
}
template <int TWOL, int L, int NT>
struct RvBack {
    __device__ __forceinline__ static void run(int mb, const RvPairs &q, const float2 *__restrict__ Y,
                                               const float2 *st, float2 (&g)[TWOL + 1], float2 &su, float2 &sa1,
                                               float2 &sa2, float2 &sb1, float2 &sb2) {
        constexpr int H = L / 2;
        if (2 * mb <= L) {
            const float2 *Yr = Y + half_block(L) + mb * (L + 1);
#pragma unroll
            for (int ma = 0; ma <= L; ++ma) {
                // the middle row of an even level carries no Y past its centre (not stored)
                const bool none = (L & 1) == 0 && ma > H && mb == H;
                const float2 y = none ? make_float2(0.f, 0.f) : __ldg(Yr + ma);
                su = __ffma2_rn(st[(acc_block(L) + ma) * NT], y, su);
                g[ma] = __fadd2_rn(g[ma], y);
            }
            if ((L & 1) == 0 && mb == H) {
                // row = (V[0..H-1], conj V[H], (-1)^(H+ma) conj V[L-ma] for ma > H): adjoint onto V
#pragma unroll
                for (int ma = 0; ma < H; ++ma) {
                    const float s = ((H + ma) & 1) ? -1.f : 1.f;
                    g[ma].x += s * g[L - ma].x;
                    g[ma].y -= s * g[L - ma].y;
                }
                g[H].y = -g[H].y;
#pragma unroll
                for (int ma = H + 1; ma <= L; ++ma) g[ma] = make_float2(0.f, 0.f);
            }
            // scaled rows: V[ma] = conj(a) P[ma] - conj(b) P[ma-1]; in place, ascending: the
            // new G[ma] = a G[ma] - b G[ma+1] reads G[ma + 1] before it is replaced
#pragma unroll
            for (int ma = 0; ma < L; ++ma) {
                const float2 gv = g[ma], hv = g[ma + 1];
                const float2 gs = make_float2(gv.y, gv.x), hs = make_float2(hv.y, hv.x);
                const float2 p = st[(acc_block(L - 1) + ma) * NT];
                // G_ca += conj(P) G[ma];  G_cb -= conj(P) G[ma+1]  (as elementwise pairs)
                sa1 = __ffma2_rn(p, gv, sa1);
                sa2 = __ffma2_rn(p, gs, sa2);
                sb1 = __ffma2_rn(p, hv, sb1);
                sb2 = __ffma2_rn(p, hs, sb2);
                g[ma] = __ffma2_rn(q.ax, gv, __ffma2_rn(q.ayn, gs, __ffma2_rn(q.bxn, hv, __fmul2_rn(q.by, hs))));
            }
            g[L] = make_float2(0.f, 0.f);
        }
        if ((L & 1) == 0) {
            // the chain mb = H started at this level from P[c] = (-1)^(H+c) conj(Q[L-1-c]),
            // Q the row H-1 of level L-1 on lane - 1: hand it the adjoint of Q
#pragma unroll
            for (int k = 0; k < L; ++k) {
                const float vr = __shfl_down_sync(0xffffffffu, g[L - 1 - k].x, 1);
                const float vi = __shfl_down_sync(0xffffffffu, g[L - 1 - k].y, 1);
                if (mb == H - 1) {
                    const float s = ((H + L - 1 - k) & 1) ? -1.f : 1.f;
                    g[k].x += s * vr;
                    g[k].y -= s * vi;
                }
            }
        }
        RvBack<TWOL, L - 1, NT>::run(mb, q, Y, st, g, su, sa1, sa2, sb1, sb2);
    }
};
template <int TWOL, int NT>
struct RvBack<TWOL, 0, NT> {
    __device__ __forceinline__ static void run(int mb, const RvPairs &, const float2 *__restrict__ Y, const float2 *,
                                               float2 (&)[TWOL + 1], float2 &su, float2 &, float2 &, float2 &,
                                               float2 &) {
        if (mb == 0) su.x += __ldg(Y).x;  // level 0: U = 1
    }
};
