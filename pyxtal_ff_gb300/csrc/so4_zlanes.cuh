// so4_zlanes.cuh -- the atoms-across-lanes layout of the window kernels.
//
// A CTA owns 32 consecutive centre atoms, one per lane.  Their U_tot (full
// layout, rebuilt from the half layout by the inversion symmetry) sits in shared
// memory as Uf[entry][lane] (row pitch 33 to spread the bank accesses of the
// transposing store), so each lane reads its own atom's U without bank conflicts
// while the warp's control flow is uniform.  Warps take work units from a shared
// counter.
#pragma once

#include "so4_common.cuh"

constexpr int ZL_PITCH = 33;

// next work unit for the calling warp (lane 0 draws from the CTA counter)
__device__ __forceinline__ int zl_next(int *counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, u, 0);
}
