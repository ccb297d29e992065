// so4_plain.cu -- the "plain" path: B, dB/dr per (i, j) pair and the per-pair
// virial rdxdr, as pyxtal_ff/descriptors/SO4.py:1409-1548 (derivative + stress
// branch of get_bispectrum_components) returns them through calculate()
// (SO4.py:190-199).  One CTA per centre atom:
//   1. U_tot = sum_images w_j sfac U(r) + self term, times u_norm  (:1480-1505)
//      warps split the images, each warp keeps a private partial sum, the
//      partials are added in warp order (deterministic);
//   2. all Z entries (compute_zi, :1020-1068) into shared memory;
//   3. B (compute_bi, :1071-1111);
//   4. warps split the pairs; per image: U and dU (the recursions :840-987) in the
//      scaled row form of warp_vrows, contracted with Z pre-scaled by the row scale.
//      The sections S(Z block) = Re sum' conj(dU_lam) Z of every distinct block the
//      components read are formed once per image (lanes take the blocks, balanced by
//      entry count: several components share a block), then each lane owns
//      bispectrum components k and forms
//      dB_k/dr = 2 S_l + 2 (l+1)/(l1+1) S_l1 + 2 (l+1)/(l2+1) S_l2  (:1113-1227)
//      with S_lam = w u_norm Re sum' conj(sfac dU + dsfac r^ U) Z (dudr, :1001-1018);
//      per pair it keeps D = sum t and E = sum r (x) t over the pair's images;
//   5. rows: dxdr[p] = D (j != i), dxdr[(i,i)] = -sum_{j != i} D,
//      rdxdr[p] = (R_i (x) dxdr[p] + E_p) / vol for every pair -- algebraically
//      the reference's -bstress/vol with bstress[(i,i)] += R_i (x) t and
//      bstress[p] -= R_j (x) t (:1458-1468).
#include <cstdio>

#include <algorithm>

#include "so4_atom.cuh"

namespace {

template <typename T>
struct PlainArgs {
    so4_params prm;
    int natoms, n_u, n_half, n_z, n_b;
    const so4_geom *geom;
    const int *astruct;
    const double *pos, *w_nb, *w_site, *img_r;
    const int32_t *img_ptr, *img_j, *pair_ptr, *pair_img, *nsite;
    const T *cg, *rootpq;
    const T *fscale;  // n_half: the row scale F of each half entry (U = F V)
    const int4 *psec;  // distinct Z blocks of the dB/dr sections, lane by lane (so4_tables.cu)
    const int *psec_ptr, *ksec;
    int n_psec;
    const ZEnt *zent;
    const BEnt *bent;
    SmallTables st;
    int want_deriv, want_stress;
    T *x, *dxdr, *rdxdr;
    cx<T> *zg;  // global Z slots (k_plain<..., true>), one per CTA
};

// One centre atom: steps 1-5 above.  Z is in shared memory, or (when it does not fit
// beside the rest) in this CTA's slot of a global scratch; HB holds the per-warp H / dH
// buffers (and, during step 1, the per-warp U_tot partials).
template <typename T, int NW, int KS>
__device__ __forceinline__ void plain_centre(const PlainArgs<T> &A, int a, const SmallTables &st, const T *rootpq,
                                             cx<T> *Uh, cx<T> *Uf, cx<T> *Z, cx<T> *HB, T *Dsum, T *Eself,
                                             T *Sw) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nh = A.n_half, nu = A.n_u, nz = A.n_z, nB = A.n_b;
    cx<T> *Hw = HB + wid * 4 * nh;  // per warp: H[nh], dH[3 nh]
    cx<T> *dHw = Hw + nh;
    const so4_geom &g = A.geom[A.astruct[a]];
    const T rc = (T)A.prm.rcut;
    const T psi_fac = (T)(A.prm.rfac0 * SO4_PI / A.prm.rcut);
    const int cid = A.prm.cutoff_id;
    const int m0 = A.img_ptr[a], m1 = A.img_ptr[a + 1];

    // ---- 1. U_tot (per-warp partials live in the dH buffers, unused until step 4)
    block_utot<T, NW>(st, rootpq, a, A.img_r, A.img_j, m0, m1, A.w_nb, A.w_site[a], rc, psi_fac, cid, nh, HB,
                      HB + nh, 4 * nh, Uh);
    block_expand<T, NW>(st, Uh, nu, Uf);
    // ---- 2. Z
    block_z<T, NW>(A.zent, nz, A.cg, Uf, Z);
    // ---- 3. B
    block_b<T, NW, T>(A.bent, nB, Uh, Z, A.x + (size_t)a * nB);
    if (!A.want_deriv) return;
    // the derivative pass carries the rows in the scaled form V (warp_vrows): Z times the
    // row scale F of its half entry, so that Re conj(dU) Z = Re conj(dV) (F Z)
    __syncthreads();
    for (int q = tid; q < nz; q += NW * 32) Z[q] = cscale(Z[q], A.fscale[A.zent[q].jh]);
    __syncthreads();

    // ---- 4. dB/dr per image, accumulated per pair
    const double Ri[3] = {A.pos[3 * a], A.pos[3 * a + 1], A.pos[3 * a + 2]};
    const int p0 = A.pair_ptr[a], p1 = A.pair_ptr[a + 1];
    const int ns = A.nsite[a];
    const T inv_vol = (T)(1.0 / g.vol);
    T dsum[KS][3];
#pragma unroll
    for (int s = 0; s < KS; ++s) dsum[s][0] = dsum[s][1] = dsum[s][2] = T(0);
    for (int p = p0 + wid; p < p1; p += NW) {
        T D[KS][3], E[KS][9];
#pragma unroll
        for (int s = 0; s < KS; ++s) {
#pragma unroll
            for (int c = 0; c < 3; ++c) D[s][c] = T(0);
#pragma unroll
            for (int c = 0; c < 9; ++c) E[s][c] = T(0);
        }
        const int q0 = A.pair_img[p], q1 = A.pair_img[p + 1];
        for (int m = q0; m < q1; ++m) {
            const T x = (T)A.img_r[3 * m], y = (T)A.img_r[3 * m + 1], z = (T)A.img_r[3 * m + 2];
            const T r = sqrt(x * x + y * y + z * z);
            if (r < T(1e-8)) continue;
            CK<T> ck;
            make_ck<T, true>(x, y, z, r, psi_fac * r, ck);
            warp_vrows<T, true>(st, ck, Hw, dHw, nh, lane);
            // every distinct Z block of the sections once: lane `lane` contracts its share of
            // the list, four sums per block (U and the three dU components) into Sw
            const int u1 = __ldg(A.psec_ptr + lane + 1);
            for (int u = __ldg(A.psec_ptr + lane); u < u1; ++u) {
                const int4 ps = __ldg(A.psec + u);  // first Z entry, half offset, entries, level
                const int zo = ps.x, h = ps.y, cnt = ps.z, lam = ps.w;
                T su = T(0), s0 = T(0), s1 = T(0), s2 = T(0);
                // entries of weight 1 as two FMAs per accumulator; an even level's section
                // ends at the middle-row centre, weight 1/2, added after the loop
                const int cfull = (lam & 1) ? cnt : cnt - 1;
                for (int e = 0; e < cfull; ++e) {
                    const cx<T> zv = Z[zo + e];
                    const cx<T> hv = Hw[h + e], d0 = dHw[h + e], d1 = dHw[nh + h + e], d2 = dHw[2 * nh + h + e];
                    su = fma(hv.re, zv.re, fma(hv.im, zv.im, su));
                    s0 = fma(d0.re, zv.re, fma(d0.im, zv.im, s0));
                    s1 = fma(d1.re, zv.re, fma(d1.im, zv.im, s1));
                    s2 = fma(d2.re, zv.re, fma(d2.im, zv.im, s2));
                }
                if (cfull < cnt) {
                    const int e = cfull;
                    const cx<T> zv = Z[zo + e];
                    const T zr = T(0.5) * zv.re, zi = T(0.5) * zv.im;
                    const cx<T> hv = Hw[h + e], d0 = dHw[h + e], d1 = dHw[nh + h + e], d2 = dHw[2 * nh + h + e];
                    su = fma(hv.re, zr, fma(hv.im, zi, su));
                    s0 = fma(d0.re, zr, fma(d0.im, zi, s0));
                    s1 = fma(d1.re, zr, fma(d1.im, zi, s1));
                    s2 = fma(d2.re, zr, fma(d2.im, zi, s2));
                }
                Sw[4 * u] = su;
                Sw[4 * u + 1] = s0;
                Sw[4 * u + 2] = s1;
                Sw[4 * u + 3] = s2;
            }
            __syncwarp();
            T sf, dsf;
            cutoff_fn<T>(cid, r, rc, sf, dsf);
            const T wj = (T)A.w_nb[A.img_j[m]];
            const T gr[3] = {x / r, y / r, z / r};
#pragma unroll
            for (int s = 0; s < KS; ++s) {
                const int k = lane + 32 * s;
                if (k >= nB) break;
                const BEnt be = A.bent[k];
                T t[3] = {T(0), T(0), T(0)};
#pragma unroll
                for (int sec = 0; sec < 3; ++sec) {
                    const T *S = Sw + 4 * __ldg(A.ksec + 3 * k + sec);
                    const T f = wj * (T)st.unorm[be.lam[sec]] * (T)be.fac[sec];
                    t[0] += f * (sf * S[1] + dsf * gr[0] * S[0]);
                    t[1] += f * (sf * S[2] + dsf * gr[1] * S[0]);
                    t[2] += f * (sf * S[3] + dsf * gr[2] * S[0]);
                }
                const T rv[3] = {x, y, z};
#pragma unroll
                for (int c = 0; c < 3; ++c) D[s][c] += t[c];
#pragma unroll
                for (int aa = 0; aa < 3; ++aa)
#pragma unroll
                    for (int c = 0; c < 3; ++c) E[s][3 * aa + c] += rv[aa] * t[c];
            }
            __syncwarp();
        }
        const bool self = (p == ns);
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            const int k = lane + 32 * s;
            if (k >= nB) break;
            if (self) {
                for (int c = 0; c < 9; ++c) Eself[9 * k + c] = E[s][c];
            } else {
                for (int c = 0; c < 3; ++c) dsum[s][c] += D[s][c];
                T *dx = A.dxdr + ((size_t)p * nB + k) * 3;
                dx[0] = D[s][0];
                dx[1] = D[s][1];
                dx[2] = D[s][2];
                if (A.want_stress) {
                    T *rd = A.rdxdr + ((size_t)p * nB + k) * 9;
#pragma unroll
                    for (int aa = 0; aa < 3; ++aa)
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            rd[3 * aa + c] = ((T)Ri[aa] * D[s][c] + E[s][3 * aa + c]) * inv_vol;
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < KS; ++s) {
        const int k = lane + 32 * s;
        if (k < nB)
            for (int c = 0; c < 3; ++c) Dsum[(wid * nB + k) * 3 + c] = dsum[s][c];
    }
    __syncthreads();
    // ---- 5. the (i, i) row
    for (int k = tid; k < nB; k += NW * 32) {
        T d[3];
        for (int c = 0; c < 3; ++c) {
            T s = T(0);
            for (int w = 0; w < NW; ++w) s += Dsum[(w * nB + k) * 3 + c];
            d[c] = -s;
        }
        T *dx = A.dxdr + ((size_t)ns * nB + k) * 3;
        dx[0] = d[0];
        dx[1] = d[1];
        dx[2] = d[2];
        if (A.want_stress) {
            T *rd = A.rdxdr + ((size_t)ns * nB + k) * 9;
            for (int aa = 0; aa < 3; ++aa)
                for (int c = 0; c < 3; ++c) rd[3 * aa + c] = ((T)Ri[aa] * d[c] + Eself[9 * k + 3 * aa + c]) * inv_vol;
        }
    }
}

// ZG false: one CTA per centre, Z in shared memory.  ZG true: gridDim.x CTAs take the centres
// in turn, each with its own Z slot of nz entries in A.zg (the FP64 path above twol 10, where
// Z alone is 95-207 KB): resident CTAs keep their slots in L2.
template <typename T, int NW, int KS, bool ZG>
__global__ void __launch_bounds__(NW * 32) k_plain(PlainArgs<T> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
    const int tid = threadIdx.x, wid = tid >> 5;
    if (tid == 0) st = A.st;
    const int ldim = A.st.twol + 1;
    const int nh = A.n_half, nu = A.n_u, nz = A.n_z, nB = A.n_b;
    // carve shared memory
    T *rootpq = (T *)smem_raw;
    cx<T> *Uh = (cx<T> *)(rootpq + ((ldim * ldim + 1) & ~1));
    cx<T> *Uf = Uh + nh;
    cx<T> *Zs = Uf + nu;
    cx<T> *HB = Zs + (ZG ? 0 : nz);
    T *Dsum = (T *)(HB + NW * 4 * nh);  // [NW][nB][3]
    T *Eself = Dsum + NW * nB * 3;      // [nB][9]
    T *Sw = Eself + nB * 9 + wid * 4 * A.n_psec;  // per warp: [n_psec][4] section sums of one image
    for (int q = tid; q < ldim * ldim; q += NW * 32) rootpq[q] = A.rootpq[q];
    __syncthreads();
    cx<T> *Z = ZG ? A.zg + (size_t)blockIdx.x * nz : Zs;
    for (int a = blockIdx.x; a < A.natoms; a += gridDim.x) {
        plain_centre<T, NW, KS>(A, a, st, rootpq, Uh, Uf, Z, HB, Dsum, Eself, Sw);
        __syncthreads();  // before the next centre reuses the buffers
    }
}

template <typename T>
size_t plain_smem_bytes(const so4_tables *t, int NW, bool zg = false) {
    const int ld = t->ldim;
    size_t b = sizeof(T) * ((ld * ld + 1) & ~1);
    b += sizeof(cx<T>) * ((size_t)t->n_half + t->n_u + (zg ? 0 : t->n_z) + (size_t)NW * 4 * t->n_half);
    b += sizeof(T) * ((size_t)NW * t->n_b * 3 + (size_t)t->n_b * 9 + (size_t)NW * 4 * t->n_psec);
    return b;
}

template <typename T, int NW, int KS, bool ZG = false>
int launch_plain(const PlainArgs<T> &A, size_t smem, int grid, cudaStream_t st) {
    auto kern = k_plain<T, NW, KS, ZG>;
    const int rc = so4_set_smem((const void *)kern, smem);
    if (rc) return rc;
    kern<<<grid, NW * 32, smem, st>>>(A);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

constexpr int PLAIN_NW = 4;

// Global Z slots of the FP64 path where Z does not fit in shared memory beside the rest
// (twol 12): one per CTA of a grid of min(natoms, 2 x SMs) CTAs.  0 where Z fits.
int plain_zslots(const so4_tables *t, int natoms) {
    if (plain_smem_bytes<double>(t, PLAIN_NW) <= 227 * 1024) return 0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 160;
    return std::max(1, std::min(natoms, 2 * sms));
}

template <typename T>
int run_plain(const so4_tables *t, const so4_params *p, const so4_geom *geom, const int *astruct, int natoms,
              const double *pos, const double *w_nb, const double *w_site, const int32_t *img_ptr,
              const int32_t *img_j, const double *img_r, const int32_t *pair_ptr, const int32_t *pair_img,
              const int32_t *nsite, int want_deriv, int want_stress, void *x, void *dxdr, void *rdxdr,
              void *work, size_t work_bytes, cudaStream_t st) {
    constexpr int NW = PLAIN_NW;
    PlainArgs<T> A;
    A.prm = *p;
    A.natoms = natoms;
    A.n_u = t->n_u;
    A.n_half = t->n_half;
    A.n_z = t->n_z;
    A.n_b = t->n_b;
    A.geom = geom;
    A.astruct = astruct;
    A.pos = pos;
    A.w_nb = w_nb;
    A.w_site = w_site;
    A.img_r = img_r;
    A.img_ptr = img_ptr;
    A.img_j = img_j;
    A.pair_ptr = pair_ptr;
    A.pair_img = pair_img;
    A.nsite = nsite;
    A.cg = (const T *)(sizeof(T) == 8 ? (const void *)t->d_cg64 : (const void *)t->d_cg32);
    A.rootpq = (const T *)(sizeof(T) == 8 ? (const void *)t->d_rootpq64 : (const void *)t->d_rootpq32);
    A.fscale = (const T *)(sizeof(T) == 8 ? (const void *)t->d_yscale64 : (const void *)t->d_yscale);
    A.psec = t->d_psec;
    A.psec_ptr = t->d_psec_ptr;
    A.ksec = t->d_ksec;
    A.n_psec = t->n_psec;
    A.zent = t->d_z;
    A.bent = t->d_b;
    fill_small_tables(t, A.st);
    A.want_deriv = want_deriv;
    A.want_stress = want_stress;
    A.x = (T *)x;
    A.dxdr = (T *)dxdr;
    A.rdxdr = (T *)rdxdr;
    A.zg = nullptr;
    const size_t smem = plain_smem_bytes<T>(t, NW);
    const int ks = (t->n_b + 31) / 32;
    if (smem > 227 * 1024) {
        // Z in global slots: built for the FP64 path at twol 12 (nB 140); FP32 fits in shared memory
        const size_t smg = plain_smem_bytes<T>(t, NW, true);
        if (sizeof(T) != 8 || smg > 227 * 1024 || ks != 5) return SO4_ERR_UNSUPPORTED;
        if (natoms == 0) return SO4_OK;
        const int slots = plain_zslots(t, natoms);
        if (!work || work_bytes < SO4_WS_HEADER + sizeof(cx<T>) * (size_t)slots * t->n_z) return SO4_ERR_WORKSPACE;
        A.zg = (cx<T> *)((char *)work + SO4_WS_HEADER);
        if constexpr (sizeof(T) == 8) return launch_plain<T, NW, 5, true>(A, smg, slots, st);
        return SO4_ERR_UNSUPPORTED;
    }
    if (natoms == 0) return SO4_OK;
    if (ks <= 1) return launch_plain<T, NW, 1>(A, smem, natoms, st);
    if (ks <= 2) return launch_plain<T, NW, 2>(A, smem, natoms, st);
    if (ks <= 3) return launch_plain<T, NW, 3>(A, smem, natoms, st);
    if (ks <= 5) return launch_plain<T, NW, 5>(A, smem, natoms, st);
    return SO4_ERR_UNSUPPORTED;
}

}  // namespace

extern "C" size_t so4_plain_workspace_size(const so4_tables *t, int natoms) {
    if (!t || natoms < 0) return SO4_WS_HEADER;
    // the FP64 path's global Z slots where Z does not fit in shared memory (twol 12)
    return SO4_WS_HEADER + sizeof(cx<double>) * (size_t)plain_zslots(t, natoms) * t->n_z;
}

extern "C" int so4_plain(const so4_tables *t, const so4_params *p, int precision, const so4_geom *d_geom,
                         const int *d_astruct, int natoms, const double *d_pos, const double *d_w_nb,
                         const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
                         const double *d_img_r, const int32_t *d_pair_ptr, const int32_t *d_pair_img,
                         const int32_t *d_nsite, int want_deriv, int want_stress, void *d_x, void *d_dxdr,
                         void *d_rdxdr, void *d_work, size_t work_bytes, void *stream) {
    if (!t || !p || natoms < 0 || !d_x) return SO4_ERR_ARG;
    if (p->twol != t->twol) return SO4_ERR_ARG;
    if (p->cutoff_id < 1 || p->cutoff_id > 7) return SO4_ERR_UNSUPPORTED;
    if (!(p->rcut > 0.0) || !(p->rfac0 > 0.0)) return SO4_ERR_ARG;
    if (want_deriv && !d_dxdr) return SO4_ERR_ARG;
    if (want_deriv && want_stress && !d_rdxdr) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == 0)
        return run_plain<double>(t, p, d_geom, d_astruct, natoms, d_pos, d_w_nb, d_w_site, d_img_ptr, d_img_j, d_img_r,
                                 d_pair_ptr, d_pair_img, d_nsite, want_deriv, want_deriv && want_stress, d_x, d_dxdr,
                                 d_rdxdr, d_work, work_bytes, st);
    if (precision == 1)
        return run_plain<float>(t, p, d_geom, d_astruct, natoms, d_pos, d_w_nb, d_w_site, d_img_ptr, d_img_j, d_img_r,
                                d_pair_ptr, d_pair_img, d_nsite, want_deriv, want_deriv && want_stress, d_x, d_dxdr,
                                d_rdxdr, d_work, work_bytes, st);
    return SO4_ERR_ARG;
}

// ---------------------------------------------------------------------------
// Per-atom stress rows.  The reference's caller turns the per-pair rdxdr of
// calculate() into one row per centre (pyxtal_ff/utilities/__init__.py:226-233):
//   out[m, k, :] = sum over the pairs (m, j) of rdxdr[p, k, a, b], (a, b) in the Voigt
//   order (0,0) (1,1) (2,2) (0,1) (0,2) (1,2),
// with a Python loop over atoms.  Pairs are grouped by centre here (pair_ptr), so
// one thread per (m, k, component) sums its centre's pairs in pair order.
namespace {
template <typename T>
__global__ void k_rdxdr_atom(const T *__restrict__ rdxdr, const int32_t *__restrict__ pair_ptr, int natoms, int nB,
                             T *__restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)natoms * nB * 6;
    if (idx >= total) return;
    const int v = (int)(idx % 6);
    const int64_t mk = idx / 6;
    const int k = (int)(mk % nB);
    const int m = (int)(mk / nB);
    const int comp = (v < 3) ? 4 * v : ((v == 3) ? 1 : ((v == 4) ? 2 : 5));  // row-major a * 3 + b
    T s = T(0);
    const int p1 = __ldg(pair_ptr + m + 1);
    for (int p = __ldg(pair_ptr + m); p < p1; ++p) s += __ldg(rdxdr + ((size_t)p * nB + k) * 9 + comp);
    out[idx] = s;
}
}  // namespace

extern "C" int so4_rdxdr_atom(int precision, const void *d_rdxdr, const int32_t *d_pair_ptr, int natoms, int nB,
                              void *d_out, void *stream) {
    if (natoms < 0 || nB <= 0 || (natoms > 0 && (!d_rdxdr || !d_pair_ptr || !d_out))) return SO4_ERR_ARG;
    if (precision != 0 && precision != 1) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    const int64_t total = (int64_t)natoms * nB * 6;
    const unsigned grid = (unsigned)((total + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == 0)
        k_rdxdr_atom<double><<<grid, 256, 0, st>>>((const double *)d_rdxdr, d_pair_ptr, natoms, nB, (double *)d_out);
    else
        k_rdxdr_atom<float><<<grid, 256, 0, st>>>((const float *)d_rdxdr, d_pair_ptr, natoms, nB, (float *)d_out);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}
