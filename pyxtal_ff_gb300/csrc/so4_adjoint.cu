// so4_adjoint.cu -- FP32 forward (U_tot, B) and the adjoint: forces and virial
// from beta = dE/dB without materialising dB/dr.
//
// The reference forms dB_k/dr per neighbour image (compute_dbidrj,
// pyxtal_ff/descriptors/SO4.py:1113-1227) as
//   dB_k = 2 S(l; Z(l1,l2,l)) + 2 (l+1)/(l1+1) S(l1; Z(l,l2,l1)) + 2 (l+1)/(l2+1) S(l2; Z(l,l1,l2)),
//   S(lam; Zb) = Re sum'_{half layer of lam} conj(dU_tot_lam) Zb,
// and its consumers contract it with beta = dE/dB (neuralnetwork.py:492, 497).
// Collecting, per level lam, every Z block times the beta of the components
// that read it gives one adjoint array per centre,
//   Y_lam = u_norm_lam w_mid * sum_{blocks (a,b,lam)} (sum_roles f beta_k) Z(a,b,lam),
// (w_mid = 1, 1/2 at the middle-row centre, 0 on the upper middle row) and then
//   dE_i/dr_image = w_j Re sum_half conj(sfac dU + dsfac r^ U) Y_i.
// Forces: F_i = sum_{images m of i} (g_m - g_rev(m)); virial: sum_m r_m (x) g_m.
#include <algorithm>

#include "so4_atom.cuh"

namespace {

constexpr int NWF = 4;  // warps per CTA, forward
constexpr int NWY = 4;  // warps per CTA, Y build
constexpr int NWD = 8;  // warps per CTA, per-image contraction

struct AdjWork {
    int *status;
    float2 *Y;       // natoms * n_half
    float *g;        // nimg * 3
    double *vatom;   // natoms * 9
};

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t carve_adj(AdjWork &w, void *base, int natoms, int nh, int64_t nimg) {
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void *q = p ? (void *)(p + off) : nullptr;
        off += a256(bytes);
        return q;
    };
    w.status = (int *)take(SO4_WS_HEADER);
    w.Y = (float2 *)take(sizeof(float2) * (size_t)natoms * nh + 8);
    w.g = (float *)take(sizeof(float) * 3 * (size_t)(nimg + 1));
    w.vatom = (double *)take(sizeof(double) * 9 * (size_t)(natoms + 1));
    return off;
}

struct FwdArgs {
    so4_params prm;
    int natoms, nh, nu, nz, nB;
    const double *w_nb, *w_site, *img_r;
    const int32_t *img_ptr, *img_j;
    const float *cg, *rootpq;
    const ZEnt *zent;
    const BEnt *bent;
    SmallTables st;
    float *utot, *x;
};

__global__ void __launch_bounds__(NWF * 32) k_forward32(FwdArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
    const int tid = threadIdx.x;
    const int a = blockIdx.x;
    if (tid == 0) st = A.st;
    const int ldim = A.st.twol + 1;
    const int nh = A.nh, nu = A.nu, nz = A.nz;
    float *rootpq = (float *)smem_raw;
    cx<float> *Uh = (cx<float> *)(rootpq + ((ldim * ldim + 1) & ~1));
    cx<float> *Uf = Uh + nh;
    cx<float> *Z = Uf + nu;
    cx<float> *W = Z + nz;  // per warp: H[nh], P[nh]
    for (int q = tid; q < ldim * ldim; q += NWF * 32) rootpq[q] = A.rootpq[q];
    __syncthreads();
    const float rc = (float)A.prm.rcut;
    const float psi_fac = (float)(A.prm.rfac0 * SO4_PI / A.prm.rcut);
    block_utot<float, NWF>(st, rootpq, a, A.img_r, A.img_j, A.img_ptr[a], A.img_ptr[a + 1], A.w_nb, A.w_site[a], rc,
                           psi_fac, A.prm.cutoff_id, nh, W, W + nh, 2 * nh, Uh);
    float2 *ug = (float2 *)A.utot + (size_t)a * nh;
    for (int e = tid; e < nh; e += NWF * 32) ug[e] = make_float2(Uh[e].re, Uh[e].im);
    block_expand<float, NWF>(st, Uh, nu, Uf);
    block_z<float, NWF>(A.zent, nz, A.cg, Uf, Z);
    block_b<float, NWF, float>(A.bent, A.nB, Uh, Z, A.x + (size_t)a * A.nB);
}

struct YArgs {
    int natoms, nh, nu, nz, nB, nblk;
    const float *utot, *beta, *cg;
    const ZEnt *zent;
    const ZBlk *blk;
    const int *yptr, *ylist;
    SmallTables st;
    float2 *Y;
};

__global__ void __launch_bounds__(NWY * 32) k_yi(YArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
    const int tid = threadIdx.x;
    const int a = blockIdx.x;
    if (tid == 0) st = A.st;
    const int nh = A.nh, nu = A.nu, nz = A.nz;
    cx<float> *Uh = (cx<float> *)smem_raw;
    cx<float> *Uf = Uh + nh;
    cx<float> *Z = Uf + nu;
    float *coef = (float *)(Z + nz);
    const float2 *ug = (const float2 *)A.utot + (size_t)a * nh;
    for (int e = tid; e < nh; e += NWY * 32) Uh[e] = mk<float>(ug[e].x, ug[e].y);
    const float *bt = A.beta + (size_t)a * A.nB;
    for (int b = tid; b < A.nblk; b += NWY * 32) {
        const ZBlk bk = A.blk[b];
        float c = 0.f;
        for (int r = 0; r < bk.nrole; ++r) c += (float)bk.role_f[r] * bt[bk.role_k[r]];
        coef[b] = c;
    }
    __syncthreads();
    block_expand<float, NWY>(st, Uh, nu, Uf);
    block_z<float, NWY>(A.zent, nz, A.cg, Uf, Z);
    const int ldim = st.twol + 1;
    float2 *Yg = A.Y + (size_t)a * nh;
    for (int e = tid; e < nh; e += NWY * 32) {
        const int lam = level_of(st.h_block, ldim, e);
        const int off = e - st.h_block[lam];
        const int mb = off / (lam + 1), ma = off - mb * (lam + 1);
        float wmid = 1.f;
        if (2 * mb == lam) wmid = (2 * ma < lam) ? 1.f : ((2 * ma == lam) ? 0.5f : 0.f);
        float yr = 0.f, yi = 0.f;
        if (wmid != 0.f) {
            for (int q = A.yptr[lam]; q < A.yptr[lam + 1]; ++q) {
                const int b = A.ylist[q];
                const float c = coef[b];
                const cx<float> zv = Z[A.blk[b].z0 + off];
                yr += c * zv.re;
                yi += c * zv.im;
            }
        }
        const float s = (float)st.unorm[lam] * wmid;
        Yg[e] = make_float2(s * yr, s * yi);
    }
}

struct DArgs {
    so4_params prm;
    int natoms, nh;
    const double *w_nb, *img_r;
    const int32_t *img_ptr, *img_j;
    const float *rootpq;
    SmallTables st;
    const float2 *Y;
    float *g;
    double *vatom;
};

// One CTA per centre, warps over its images: U and dU by the recursion, then
// dE/dr_image = w_j (sfac Re sum conj(dU) Y + dsfac r^ Re sum conj(U) Y).
__global__ void __launch_bounds__(NWD * 32) k_deidrj(DArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
    __shared__ double vred[NWD][9];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int a = blockIdx.x;
    if (tid == 0) st = A.st;
    const int ldim = A.st.twol + 1;
    const int nh = A.nh;
    float *rootpq = (float *)smem_raw;
    cx<float> *Ys = (cx<float> *)(rootpq + ((ldim * ldim + 1) & ~1));
    cx<float> *Hw = Ys + nh + wid * 4 * nh;
    cx<float> *dHw = Hw + nh;
    for (int q = tid; q < ldim * ldim; q += NWD * 32) rootpq[q] = A.rootpq[q];
    const float2 *Yg = A.Y + (size_t)a * nh;
    for (int e = tid; e < nh; e += NWD * 32) Ys[e] = mk<float>(Yg[e].x, Yg[e].y);
    __syncthreads();
    const float rc = (float)A.prm.rcut;
    const float psi_fac = (float)(A.prm.rfac0 * SO4_PI / A.prm.rcut);
    double vw[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) vw[q] = 0.0;
    const int m0 = A.img_ptr[a], m1 = A.img_ptr[a + 1];
    for (int m = m0 + wid; m < m1; m += NWD) {
        const double xd = A.img_r[3 * m], yd = A.img_r[3 * m + 1], zd = A.img_r[3 * m + 2];
        const float x = (float)xd, y = (float)yd, z = (float)zd;
        const float r = sqrtf(x * x + y * y + z * z);
        if (r < 1e-8f) {
            if (lane == 0) A.g[3 * m] = A.g[3 * m + 1] = A.g[3 * m + 2] = 0.f;
            continue;
        }
        CK<float> ck;
        make_ck<float, true>(x, y, z, r, psi_fac * r, ck);
        warp_uarray<float, true>(st, rootpq, ck, Hw, dHw, nh, lane);
        float su = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f;
        for (int e = lane; e < nh; e += 32) {
            const cx<float> yv = Ys[e];
            su += redot(Hw[e], yv);
            s0 += redot(dHw[e], yv);
            s1 += redot(dHw[nh + e], yv);
            s2 += redot(dHw[2 * nh + e], yv);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            su += __shfl_xor_sync(0xffffffffu, su, d);
            s0 += __shfl_xor_sync(0xffffffffu, s0, d);
            s1 += __shfl_xor_sync(0xffffffffu, s1, d);
            s2 += __shfl_xor_sync(0xffffffffu, s2, d);
        }
        float sf, dsf;
        cutoff_fn<float>(A.prm.cutoff_id, r, rc, sf, dsf);
        const float wj = (float)A.w_nb[A.img_j[m]];
        const float gx = wj * (sf * s0 + dsf * (x / r) * su);
        const float gy = wj * (sf * s1 + dsf * (y / r) * su);
        const float gz = wj * (sf * s2 + dsf * (z / r) * su);
        if (lane == 0) {
            A.g[3 * m] = gx;
            A.g[3 * m + 1] = gy;
            A.g[3 * m + 2] = gz;
        }
        const double rv[3] = {xd, yd, zd}, gv[3] = {gx, gy, gz};
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) vw[3 * p + q] += rv[p] * gv[q];
        __syncwarp();
    }
    if (lane == 0)
        for (int q = 0; q < 9; ++q) vred[wid][q] = vw[q];
    __syncthreads();
    if (tid < 9) {
        double s = 0.0;
        for (int w = 0; w < NWD; ++w) s += vred[w][tid];
        A.vatom[9 * (size_t)a + tid] = s;
    }
}

// F_i = sum over images m of i of (g_m - g_rev(m))  (FP64 accumulation)
__global__ void k_gather(int natoms, const int32_t *img_ptr, const int32_t *img_rev, const float *g, double *forces) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int m = img_ptr[a]; m < img_ptr[a + 1]; ++m) {
        const int r = img_rev[m];
        f0 += (double)g[3 * m] - (double)g[3 * r];
        f1 += (double)g[3 * m + 1] - (double)g[3 * r + 1];
        f2 += (double)g[3 * m + 2] - (double)g[3 * r + 2];
    }
    forces[3 * a] = f0;
    forces[3 * a + 1] = f1;
    forces[3 * a + 2] = f2;
}

// per-structure virial: fixed-order block reduction of the per-atom virials
__global__ void k_virial(const int *atom_ptr, const double *vatom, double *virial) {
    __shared__ double red[256];
    const int s = blockIdx.x, t = threadIdx.x;
    const int a0 = atom_ptr[s], a1 = atom_ptr[s + 1];
    for (int q = 0; q < 9; ++q) {
        double acc = 0.0;
        for (int a = a0 + t; a < a1; a += blockDim.x) acc += vatom[9 * (size_t)a + q];
        red[t] = acc;
        __syncthreads();
        for (int d = blockDim.x / 2; d > 0; d >>= 1) {
            if (t < d) red[t] += red[t + d];
            __syncthreads();
        }
        if (t == 0) virial[9 * s + q] = red[0];
        __syncthreads();
    }
}

template <typename K>
int set_smem(K kern, size_t smem) {
    if (smem > 227 * 1024) return SO4_ERR_UNSUPPORTED;
    if (smem > 48 * 1024)
        SO4_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return SO4_OK;
}

size_t rootpq_floats(int ldim) { return (size_t)((ldim * ldim + 1) & ~1); }

}  // namespace

extern "C" int so4_forward32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                             const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
                             const double *d_img_r, float *d_utot, float *d_x, void *stream) {
    if (!t || !p || natoms < 0 || !d_utot || !d_x) return SO4_ERR_ARG;
    if (p->twol != t->twol || !(p->rcut > 0.0) || !(p->rfac0 > 0.0)) return SO4_ERR_ARG;
    if (p->cutoff_id < 1 || p->cutoff_id > 7) return SO4_ERR_UNSUPPORTED;
    if (natoms == 0) return SO4_OK;
    FwdArgs A;
    A.prm = *p;
    A.natoms = natoms;
    A.nh = t->n_half;
    A.nu = t->n_u;
    A.nz = t->n_z;
    A.nB = t->n_b;
    A.w_nb = d_w_nb;
    A.w_site = d_w_site;
    A.img_r = d_img_r;
    A.img_ptr = d_img_ptr;
    A.img_j = d_img_j;
    A.cg = t->d_cg32;
    A.rootpq = t->d_rootpq32;
    A.zent = t->d_z;
    A.bent = t->d_b;
    fill_small_tables(t, A.st);
    A.utot = d_utot;
    A.x = d_x;
    const size_t smem = sizeof(float) * rootpq_floats(t->ldim) +
                        sizeof(cx<float>) * ((size_t)t->n_half + t->n_u + t->n_z + (size_t)NWF * 2 * t->n_half);
    int rc = set_smem(k_forward32, smem);
    if (rc) return rc;
    k_forward32<<<natoms, NWF * 32, smem, (cudaStream_t)stream>>>(A);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" size_t so4_adjoint_workspace_size(const so4_tables *t, int natoms, int64_t nimg) {
    if (!t) return 0;
    AdjWork w;
    return carve_adj(w, nullptr, natoms, t->n_half, nimg);
}

extern "C" int so4_adjoint_y32(const so4_tables *t, int natoms, const float *d_utot, const float *d_beta, float *d_y,
                               void *stream) {
    if (!t || natoms < 0 || !d_utot || !d_beta || !d_y) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    YArgs Y;
    Y.natoms = natoms;
    Y.nh = t->n_half;
    Y.nu = t->n_u;
    Y.nz = t->n_z;
    Y.nB = t->n_b;
    Y.nblk = t->n_blk;
    Y.utot = d_utot;
    Y.beta = d_beta;
    Y.cg = t->d_cg32;
    Y.zent = t->d_z;
    Y.blk = t->d_blk;
    Y.yptr = t->d_yblk_ptr;
    Y.ylist = t->d_yblk;
    fill_small_tables(t, Y.st);
    Y.Y = (float2 *)d_y;
    const size_t smy = sizeof(cx<float>) * ((size_t)t->n_half + t->n_u + t->n_z) + sizeof(float) * ((t->n_blk + 3) & ~3);
    int rc = set_smem(k_yi, smy);
    if (rc) return rc;
    k_yi<<<natoms, NWY * 32, smy, (cudaStream_t)stream>>>(Y);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_adjoint_deidrj32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                                    const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                                    const float *d_y, float *d_g, double *d_vatom, void *stream) {
    if (!t || !p || natoms < 0 || !d_y || !d_g || !d_vatom) return SO4_ERR_ARG;
    if (p->twol != t->twol || !(p->rcut > 0.0) || !(p->rfac0 > 0.0)) return SO4_ERR_ARG;
    if (p->cutoff_id < 1 || p->cutoff_id > 7) return SO4_ERR_UNSUPPORTED;
    if (natoms == 0) return SO4_OK;
    DArgs D;
    D.prm = *p;
    D.natoms = natoms;
    D.nh = t->n_half;
    D.w_nb = d_w_nb;
    D.img_r = d_img_r;
    D.img_ptr = d_img_ptr;
    D.img_j = d_img_j;
    D.rootpq = t->d_rootpq32;
    fill_small_tables(t, D.st);
    D.Y = (const float2 *)d_y;
    D.g = d_g;
    D.vatom = d_vatom;
    const size_t smd =
        sizeof(float) * rootpq_floats(t->ldim) + sizeof(cx<float>) * ((size_t)t->n_half + (size_t)NWD * 4 * t->n_half);
    int rc = set_smem(k_deidrj, smd);
    if (rc) return rc;
    k_deidrj<<<natoms, NWD * 32, smd, (cudaStream_t)stream>>>(D);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_adjoint_gather(int natoms, int nstruct, const int *d_atom_ptr, const int32_t *d_img_ptr,
                                  const int32_t *d_img_rev, const float *d_g, const double *d_vatom, double *d_forces,
                                  double *d_virial, void *stream) {
    if (natoms < 0 || nstruct < 0) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (natoms > 0) {
        k_gather<<<(natoms + 127) / 128, 128, 0, st>>>(natoms, d_img_ptr, d_img_rev, d_g, d_forces);
        so4_count_launch();
    }
    if (nstruct > 0) {
        k_virial<<<nstruct, 256, 0, st>>>(d_atom_ptr, d_vatom, d_virial);
        so4_count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_adjoint32(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                             const int *d_atom_ptr, int natoms, const double *d_w_nb, const int32_t *d_img_ptr,
                             const int32_t *d_img_j, const double *d_img_r, const int32_t *d_img_rev, int64_t nimg,
                             const float *d_utot, const float *d_beta, double *d_forces, double *d_virial,
                             void *d_work, size_t work_bytes, void *stream) {
    (void)d_atom_struct;
    if (!t || !p || natoms < 0 || nstruct < 0 || nimg < 0 || !d_work) return SO4_ERR_ARG;
    AdjWork w;
    if (carve_adj(w, nullptr, natoms, t->n_half, nimg) > work_bytes) return SO4_ERR_WORKSPACE;
    carve_adj(w, d_work, natoms, t->n_half, nimg);
    int rc = so4_adjoint_y32(t, natoms, d_utot, d_beta, (float *)w.Y, stream);
    if (rc) return rc;
    rc = so4_adjoint_deidrj32(t, p, natoms, d_w_nb, d_img_ptr, d_img_j, d_img_r, (const float *)w.Y, w.g, w.vatom,
                              stream);
    if (rc) return rc;
    return so4_adjoint_gather(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev, w.g, w.vatom, d_forces, d_virial,
                              stream);
}

// ---------------------------------------------------------------------------
// so4_adjoint32_noalloc: the adjoint with its scratch in a fixed device array.
//
// Some callers cannot allocate device memory at the moment they need forces:
// an MD engine's force plugin that is handed only its input and output
// buffers, code running while another allocator owns the whole of HBM (a
// pre-reserved pool), or a path that must not call cudaMalloc because that
// call can synchronise the device or fail under memory pressure mid-run.  For
// them this entry point takes the adjoint's scratch (Y, the per-image dE/dr
// and the per-atom virials) from g_noalloc_scratch below instead of a
// caller-provided workspace.  It calls no cudaMalloc, no cudaFree and no
// allocating library routine.
//
// Limit: the scratch one call needs is so4_adjoint_workspace_size(t, natoms,
// nimg) bytes; problems needing more than SO4_NOALLOC_SCRATCH_BYTES (64 MiB,
// e.g. 32,000 atoms with ~900k images at lmax 4) are rejected with
// SO4_ERR_TOO_LARGE.  The array lives on every GPU that loads this library,
// until the process exits.
//
// Every call on a device uses the same array and leaves its contents behind.
// Nothing in it needs to start at zero: each byte a kernel reads was written
// earlier in the same call.  Calls that overlap on the GPU (different streams,
// or host threads sharing a device) race on the array; serialise them.
//
// The device address of the array is looked up with cudaGetSymbolAddress the
// first time the entry point runs on each device (with that device current);
// that first call should come before any stream capture.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SO4_NOALLOC_SCRATCH_BYTES];

#include <mutex>

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kNoallocMaxDevices] = {nullptr};
}  // namespace

extern "C" int so4_adjoint32_noalloc(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                                     const int *d_atom_ptr, int natoms, const double *d_w_nb,
                                     const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                                     const int32_t *d_img_rev, int64_t nimg, const float *d_utot,
                                     const float *d_beta, double *d_forces, double *d_virial, void *stream) {
    (void)d_atom_struct;
    if (!t || !p || natoms < 0 || nstruct < 0 || nimg < 0) return SO4_ERR_ARG;
    AdjWork w;
    if (carve_adj(w, nullptr, natoms, t->n_half, nimg) > (size_t)SO4_NOALLOC_SCRATCH_BYTES) return SO4_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SO4_ERR_CUDA;
    if (dev < 0 || dev >= kNoallocMaxDevices) return SO4_ERR_UNSUPPORTED;
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *q = nullptr;
            if (cudaGetSymbolAddress(&q, g_noalloc_scratch) != cudaSuccess || !q) return SO4_ERR_CUDA;
            g_noalloc_ptr[dev] = q;
        }
        scratch = g_noalloc_ptr[dev];
    }
    carve_adj(w, scratch, natoms, t->n_half, nimg);
    int rc = so4_adjoint_y32(t, natoms, d_utot, d_beta, (float *)w.Y, stream);
    if (rc) return rc;
    rc = so4_adjoint_deidrj32(t, p, natoms, d_w_nb, d_img_ptr, d_img_j, d_img_r, (const float *)w.Y, w.g, w.vatom,
                              stream);
    if (rc) return rc;
    return so4_adjoint_gather(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev, w.g, w.vatom, d_forces, d_virial,
                              stream);
}
