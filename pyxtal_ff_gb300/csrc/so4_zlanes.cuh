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

// sum over the terms [t0, t1) of c * U[i1] * U[i2] for this lane's atom
__device__ __forceinline__ float2 zl_entry(const ZTerm *__restrict__ terms, int t0, int t1, const float2 *Uf, int lane) {
    float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f;
    int t = t0;
    for (; t + 1 < t1; t += 2) {
        const ZTerm a = terms[t], b = terms[t + 1];
        const float2 ua = Uf[a.i1 * ZL_PITCH + lane], va = Uf[a.i2 * ZL_PITCH + lane];
        const float2 ub = Uf[b.i1 * ZL_PITCH + lane], vb = Uf[b.i2 * ZL_PITCH + lane];
        const float par = ua.x * va.x - ua.y * va.y, pai = ua.x * va.y + ua.y * va.x;
        const float pbr = ub.x * vb.x - ub.y * vb.y, pbi = ub.x * vb.y + ub.y * vb.x;
        r0 += a.c * par;
        i0 += a.c * pai;
        r1 += b.c * pbr;
        i1 += b.c * pbi;
    }
    if (t < t1) {
        const ZTerm a = terms[t];
        const float2 ua = Uf[a.i1 * ZL_PITCH + lane], va = Uf[a.i2 * ZL_PITCH + lane];
        r0 += a.c * (ua.x * va.x - ua.y * va.y);
        i0 += a.c * (ua.x * va.y + ua.y * va.x);
    }
    return make_float2(r0 + r1, i0 + i1);
}

// next work unit for the calling warp (lane 0 draws from the CTA counter)
__device__ __forceinline__ int zl_next(int *counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, u, 0);
}
