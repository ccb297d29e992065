// so4_zlanes.cuh -- the atoms-across-lanes layout of the window kernels.
//
// A CTA owns 32 consecutive centre atoms, one per lane.  Their U_tot (full
// layout, rebuilt from the half layout by the inversion symmetry) sits in shared
// memory as Uf[entry][lane] (row pitch 33 to spread the bank accesses of the
// transposing load), so each lane reads its own atom's U without bank conflicts
// while the warp's control flow is uniform.  Warps take work units from a shared
// counter.
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

// next work unit for the calling warp (lane 0 draws from the CTA counter)
__device__ __forceinline__ int zl_next(int *counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, u, 0);
}
