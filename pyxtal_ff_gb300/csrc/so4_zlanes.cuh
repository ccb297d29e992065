// so4_zlanes.cuh -- Z contractions with atoms across lanes.
//
// A CTA owns 32 consecutive centre atoms, one per lane.  Their U_tot (full
// layout, rebuilt from the half layout by the inversion symmetry) sits in shared
// memory as Uf[entry][lane] (row pitch 33 to spread the bank accesses of the
// transposing load).  Every warp evaluates the same Z entry for its 32 atoms:
// control flow is uniform, the term list (c = cg_a cg_b, i1, i2) is read once per
// warp as a broadcast, and each lane reads its own atom's U without bank
// conflicts.  Warps take work units from a shared counter, most expensive first.
#pragma once

#include "so4_common.cuh"

constexpr int ZL_PITCH = 33;

// Uf[f][lane] for the 32 atoms a0.. (zeros past natoms)
__device__ __forceinline__ void zl_load_utot(const float2 *__restrict__ utot, const int *__restrict__ fmap, int a0,
                                             int natoms, int nh, int nu, float2 *Uf) {
    // unrolled: each iteration is a dependent pair of loads (map, then U), so several
    // iterations are kept in flight
#pragma unroll 4
    for (int idx = threadIdx.x; idx < 32 * nu; idx += blockDim.x) {
        const int lane = idx / nu, f = idx - lane * nu;
        const int a = a0 + lane;
        float2 v = make_float2(0.f, 0.f);
        if (a < natoms) {
            const int m = __ldg(fmap + f);
            v = __ldg(utot + (size_t)a * nh + (m & 0x3fff));
            if (m & (1 << 15)) v.y = -v.y;
            if (m & (1 << 14)) {
                v.x = -v.x;
                v.y = -v.y;
            }
        }
        Uf[f * ZL_PITCH + lane] = v;
    }
}

// sum over the terms [t0, t1) of c * U[i1] * U[i2] for this lane's atom.  Ul = Uf + lane;
// term offsets are pre-scaled by the pitch; lists have even length and start even, so
// two terms arrive in one 16-byte load.  The term words come from L2 and are the
// critical latency: each iteration consumes two words while the next two are in flight.
__device__ __forceinline__ void zl_pair(const int4 w, const float2 *Ul, float &r0, float &i0, float &r1, float &i1) {
    const float ca = __int_as_float(w.x), cb = __int_as_float(w.z);
    const float2 ua = Ul[w.y & 0xffff], va = Ul[(unsigned)w.y >> 16];
    const float2 ub = Ul[w.w & 0xffff], vb = Ul[(unsigned)w.w >> 16];
    r0 += ca * (ua.x * va.x - ua.y * va.y);
    i0 += ca * (ua.x * va.y + ua.y * va.x);
    r1 += cb * (ub.x * vb.x - ub.y * vb.y);
    i1 += cb * (ub.x * vb.y + ub.y * vb.x);
}

__device__ __forceinline__ float2 zl_entry(const ZTerm *__restrict__ terms, int t0, int t1, const float2 *Ul) {
    float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f, r2 = 0.f, i2 = 0.f, r3 = 0.f, i3 = 0.f;
    const int4 *tp = reinterpret_cast<const int4 *>(terms + t0);
    const int n2 = (t1 - t0) >> 1;
    const int4 zero = make_int4(0, 0, 0, 0);
    int4 wa = (n2 > 0) ? __ldg(tp) : zero;
    int4 wb = (n2 > 1) ? __ldg(tp + 1) : zero;
    int q = 0;
    for (; q + 1 < n2; q += 2) {
        const int4 ca = wa, cb = wb;
        wa = (q + 2 < n2) ? __ldg(tp + q + 2) : zero;
        wb = (q + 3 < n2) ? __ldg(tp + q + 3) : zero;
        zl_pair(ca, Ul, r0, i0, r1, i1);
        zl_pair(cb, Ul, r2, i2, r3, i3);
    }
    if (q < n2) zl_pair(wa, Ul, r0, i0, r1, i1);
    return make_float2((r0 + r1) + (r2 + r3), (i0 + i1) + (i2 + i3));
}

// next work unit for the calling warp (lane 0 draws from the CTA counter)
__device__ __forceinline__ int zl_next(int *counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, u, 0);
}
