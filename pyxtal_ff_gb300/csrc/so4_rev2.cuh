// so4_rev2.cuh -- the per-image reverse sweep with two lanes per image.
//
// The row-chain kernels give each chain mb = 0..TWOL/2 of an image its own lane and step
// all lanes through every level together, so a chain that starts late (chain mb starts at
// level 2 mb) idles until then: at TWOL 8 the five lanes of an image spend 5 x 44 entry
// steps on its 154 entries.  Here an image has two lanes, A (even) and B (odd), and chain c
// goes to A when c mod 4 is 0 or 3 and to B when it is 1 or 2, in slot 2 floor(c / 4) + (0
// for c mod 4 in {0, 1}, 1 otherwise):
//   TWOL 8:  A = chains 0, 3, 4 (slots 0, 1, 2)   B = chains 1, 2 (slots 0, 1)
//   TWOL 6:  A = chains 0, 3                      B = chains 1, 2
// At each level a lane updates every slot whose chain has started, so the pair's lanes hold
// rows 1, 1, 1, 2, 2, 2, 2, 3 (TWOL 8, levels 1..8): 88 entry steps per 16 images instead of
// 44 per 6, a quarter fewer.  A chain starts from the previous chain's row of the level
// below, mirrored (SO4.py:908-925): from the other lane of the pair (one shuffle) when the
// roles differ (chains 1 and 3), from a slot of the same lane otherwise (chains 2 and 4).
// The recursion itself is the scaled one of so4_rowchain.cuh (rc_level), and the backward
// sweep the same adjoint steps as RvBack, slot by slot.
//
// Each lane keeps the rows it computes in shared memory, slot s from level base(s) up to
// TWOL - 1: slot s's region starts at SOFF(s) and row (L, ma) sits at SOFF(s) + acc_block(L)
// - acc_block(base(s)) + ma; at a chain start the mirrored starting row is stored as level
// L - 1 of the new chain's slot.  The rows of level TWOL are not stored: they are still in
// the forward sweep's registers when the backward sweep starts there (74 entries per lane at
// TWOL 8, 36 at TWOL 6).
#pragma once

#include "so4_rowchain.cuh"

namespace rev2 {

__host__ __device__ constexpr int role_of(int c) { return (c % 4 == 0 || c % 4 == 3) ? 0 : 1; }
__host__ __device__ constexpr int slot_of(int c) { return 2 * (c / 4) + ((c % 4 == 0 || c % 4 == 1) ? 0 : 1); }
// the level from which a chain's row is stored (its mirrored starting row is level 2c - 1)
__host__ __device__ constexpr int store_from(int c) { return c == 0 ? 0 : 2 * c - 1; }
// the first level at which a chain is updated
__host__ __device__ constexpr int first_level(int c) { return c == 0 ? 1 : 2 * c; }

template <int TWOL>
struct Layout {
    static constexpr int NCH = TWOL / 2 + 1;
    static constexpr int W = TWOL + 1;
    __host__ __device__ static constexpr int ns() {
        int n = 0;
        for (int c = 0; c < NCH; ++c)
            if (slot_of(c) + 1 > n) n = slot_of(c) + 1;
        return n;
    }
    static constexpr int NS = ns();  // slots per lane
    // lowest stored level of slot s over both roles
    __host__ __device__ static constexpr int base(int s) {
        int b = 1 << 20;
        for (int c = 0; c < NCH; ++c)
            if (slot_of(c) == s && store_from(c) < b) b = store_from(c);
        return b;
    }
    // lowest level at which slot s is updated in either role
    __host__ __device__ static constexpr int act(int s) {
        int a = 1 << 20;
        for (int c = 0; c < NCH; ++c)
            if (slot_of(c) == s && first_level(c) < a) a = first_level(c);
        return a;
    }
    __host__ __device__ static constexpr int soff(int s) {
        int o = 0;
        for (int q = 0; q < s; ++q) o += acc_block(TWOL) - acc_block(base(q));
        return o;
    }
    static constexpr int SLOTW = soff(NS);  // stored entries per lane
    __host__ __device__ static constexpr int idx(int s, int L) { return soff(s) + acc_block(L) - acc_block(base(s)); }
};

// Forward sweep, levels L..TWOL.  ch[s]: this lane's chain in slot s (-1: none); role: 0 A, 1 B.
// Rows are (re, im) pairs (rc2_level: rc_level's arithmetic), stored to shared memory as they are.
template <int TWOL, int L, int NT>
struct Fwd {
    using Y = Layout<TWOL>;
    __device__ __forceinline__ static void run(int role, const int (&ch)[Y::NS], const CK<float> &ck,
                                               float2 (&u)[Y::NS][TWOL + 1], float2 *st) {
        if constexpr ((L & 1) == 0) {
            // chain c = L/2 starts from chain c - 1's row of level L - 1:
            //   P[k] = (-1)^(c + k) conj(Q[L - 1 - k]),  k = 0 .. L - 1
            constexpr int c = L / 2, sd = slot_of(c), ss = slot_of(c - 1);
            constexpr bool cross = role_of(c) != role_of(c - 1);
            const bool take = role == role_of(c);
#pragma unroll
            for (int k = 0; k < L; ++k) {
                float qr = u[ss][L - 1 - k].x, qi = u[ss][L - 1 - k].y;
                if (cross) {
                    qr = __shfl_xor_sync(0xffffffffu, qr, 1);
                    qi = __shfl_xor_sync(0xffffffffu, qi, 1);
                }
                const float s = ((c + k) & 1) ? -1.f : 1.f;
                if (take) u[sd][k] = make_float2(s * qr, -s * qi);
            }
            if (take) {
#pragma unroll
                for (int k = 0; k < L; ++k) st[(Y::idx(sd, L - 1) + k) * NT] = u[sd][k];
            }
        }
#pragma unroll
        for (int s = 0; s < Y::NS; ++s) {
            if (Y::act(s) <= L) {
                rc2_level<TWOL, L>(ch[s], ck, u[s]);
                if (L < TWOL && ch[s] >= 0 && 2 * ch[s] <= L) {
#pragma unroll
                    for (int ma = 0; ma <= L; ++ma) st[(Y::idx(s, L) + ma) * NT] = u[s][ma];
                }
            }
        }
        Fwd<TWOL, L + 1, NT>::run(role, ch, ck, u, st);
    }
};
template <int TWOL, int NT>
struct Fwd<TWOL, TWOL + 1, NT> {
    using Y = Layout<TWOL>;
    __device__ __forceinline__ static void run(int, const int (&)[Y::NS], const CK<float> &,
                                               float2 (&)[Y::NS][TWOL + 1], float2 *) {}
};

// Backward sweep, level L down to 1, per slot as RvBack does per lane; at a chain start
// the adjoint of the starting row goes to the slot (this lane or the other) it came from.
template <int TWOL, int L, int NT>
struct Back {
    using Y = Layout<TWOL>;
    __device__ __forceinline__ static void run(int role, const int (&ch)[Y::NS], const RvPairs &q,
                                               const float2 *__restrict__ Yc, const float2 *st,
                                               const float2 (&u)[Y::NS][TWOL + 1], float2 (&g)[Y::NS][TWOL + 1],
                                               float2 &su, float2 &sa1, float2 &sa2, float2 &sb1, float2 &sb2) {
        constexpr int H = L / 2;
#pragma unroll
        for (int s = 0; s < Y::NS; ++s) {
            if (Y::act(s) <= L) {
                const int mb = ch[s];
                if (mb >= 0 && 2 * mb <= L) {
                    const float2 *Yr = Yc + half_block(L) + mb * (L + 1);
#pragma unroll
                    for (int ma = 0; ma <= L; ++ma) {
                        // the middle row of an even level carries no Y past its centre (not stored)
                        const bool none = (L & 1) == 0 && ma > H && mb == H;
                        const float2 y = none ? make_float2(0.f, 0.f) : __ldg(Yr + ma);
                        // level TWOL from the forward sweep's registers, lower levels from shared memory
                        const float2 row = (L == TWOL) ? u[s][ma] : st[(Y::idx(s, L) + ma) * NT];
                        su = __ffma2_rn(row, y, su);
                        g[s][ma] = __fadd2_rn(g[s][ma], y);
                    }
                    if ((L & 1) == 0 && mb == H) {
#pragma unroll
                        for (int ma = 0; ma < H; ++ma) {
                            const float sg = ((H + ma) & 1) ? -1.f : 1.f;
                            g[s][ma].x += sg * g[s][L - ma].x;
                            g[s][ma].y -= sg * g[s][L - ma].y;
                        }
                        g[s][H].y = -g[s][H].y;
#pragma unroll
                        for (int ma = H + 1; ma <= L; ++ma) g[s][ma] = make_float2(0.f, 0.f);
                    }
#pragma unroll
                    for (int ma = 0; ma < L; ++ma) {
                        const float2 gv = g[s][ma], hv = g[s][ma + 1];
                        const float2 gs = make_float2(gv.y, gv.x), hs = make_float2(hv.y, hv.x);
                        const float2 p = st[(Y::idx(s, L - 1) + ma) * NT];
                        sa1 = __ffma2_rn(p, gv, sa1);
                        sa2 = __ffma2_rn(p, gs, sa2);
                        sb1 = __ffma2_rn(p, hv, sb1);
                        sb2 = __ffma2_rn(p, hs, sb2);
                        g[s][ma] = __ffma2_rn(q.ax, gv, __ffma2_rn(q.ayn, gs, __ffma2_rn(q.bxn, hv, __fmul2_rn(q.by, hs))));
                    }
                    g[s][L] = make_float2(0.f, 0.f);
                }
            }
        }
        if constexpr ((L & 1) == 0) {
            // chain c = H started here from Q = chain c - 1's row of level L - 1:
            // Q[k] receives (-1)^(c + L - 1 - k) conj of the adjoint of P[L - 1 - k]
            constexpr int c = H, sd = slot_of(c), ss = slot_of(c - 1);
            constexpr bool cross = role_of(c) != role_of(c - 1);
            const bool take = role == role_of(c - 1);
#pragma unroll
            for (int k = 0; k < L; ++k) {
                float vr = g[sd][L - 1 - k].x, vi = g[sd][L - 1 - k].y;
                if (cross) {
                    vr = __shfl_xor_sync(0xffffffffu, vr, 1);
                    vi = __shfl_xor_sync(0xffffffffu, vi, 1);
                }
                if (take) {
                    const float sg = ((c + L - 1 - k) & 1) ? -1.f : 1.f;
                    g[ss][k].x += sg * vr;
                    g[ss][k].y -= sg * vi;
                }
            }
        }
        Back<TWOL, L - 1, NT>::run(role, ch, q, Yc, st, u, g, su, sa1, sa2, sb1, sb2);
    }
};
template <int TWOL, int NT>
struct Back<TWOL, 0, NT> {
    using Y = Layout<TWOL>;
    __device__ __forceinline__ static void run(int role, const int (&)[Y::NS], const RvPairs &,
                                               const float2 *__restrict__ Yc, const float2 *,
                                               const float2 (&)[Y::NS][TWOL + 1], float2 (&)[Y::NS][TWOL + 1],
                                               float2 &su, float2 &, float2 &, float2 &, float2 &) {
        if (role == 0) su.x += __ldg(Yc).x;  // level 0: U = 1 (chain 0, lane A)
    }
};

}  // namespace rev2
