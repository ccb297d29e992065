// so4_atom.cuh -- per-centre-atom phases shared by the plain and adjoint kernels.
// Each function is called by all threads of a CTA of NW warps and ends with
// __syncthreads().
#pragma once

#include "so4_common.cuh"

__device__ __forceinline__ int level_of(const int *blk, int ldim, int idx) {
    int l = 0;
    while (l + 1 < ldim && blk[l + 1] <= idx) ++l;
    return l;
}

// U_tot of centre `a` in the half layout (SO4.py:1480-1505 with
// addself_uarraytot :560-597): sum over images of (w_j U) sfac, plus the self
// term f_c(0) w_site on the diagonal, times u_norm.  Warps split the images;
// warp w accumulates into P + w*pstride, the partials are added in warp order.
template <typename T, int NW>
__device__ void block_utot(const SmallTables &st, const T *rootpq, int a, const double *img_r,
                           const int32_t *img_j, int m0, int m1, const double *w_nb, double w_site,
                           T rc, T psi_fac, int cid, int nh, cx<T> *H, cx<T> *P, int pstride, cx<T> *Uh) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int ldim = st.twol + 1;
    cx<T> *Hw = H + wid * pstride;
    cx<T> *Pw = P + wid * pstride;
    for (int e = lane; e < nh; e += 32) Pw[e] = mk<T>(T(0), T(0));
    __syncwarp();
    for (int m = m0 + wid; m < m1; m += NW) {
        const T x = (T)img_r[3 * m], y = (T)img_r[3 * m + 1], z = (T)img_r[3 * m + 2];
        const T r = sqrt(x * x + y * y + z * z);
        if (r < T(1e-8)) continue;
        CK<T> ck;
        make_ck<T, false>(x, y, z, r, psi_fac * r, ck);
        warp_uarray<T, false>(st, rootpq, ck, Hw, nullptr, nh, lane);
        T sf, dsf;
        cutoff_fn<T>(cid, r, rc, sf, dsf);
        const T wj = (T)w_nb[img_j[m]];
        for (int e = lane; e < nh; e += 32) Pw[e] = cadd(Pw[e], cscale(cscale(Hw[e], wj), sf));
        __syncwarp();
    }
    __syncthreads();
    T f0, df0;
    cutoff_fn<T>(cid, T(0), rc, f0, df0);
    const T ws = (T)w_site;
    for (int e = tid; e < nh; e += NW * 32) {
        cx<T> s = mk<T>(T(0), T(0));
        for (int w = 0; w < NW; ++w) s = cadd(s, P[w * pstride + e]);
        const int l = level_of(st.h_block, ldim, e);
        const int off = e - st.h_block[l];
        const int mb = off / (l + 1), ma = off - mb * (l + 1);
        if (ma == mb) s = cadd(s, mk<T>(f0 * ws, T(0)));
        Uh[e] = cscale(s, (T)st.unorm[l]);
    }
    __syncthreads();
}

// Full (l+1)^2 layers from the half layout by the inversion symmetry (SO4.py:908-925).
template <typename T, int NW>
__device__ void block_expand(const SmallTables &st, const cx<T> *Uh, int nu, cx<T> *Uf) {
    const int ldim = st.twol + 1;
    for (int f = threadIdx.x; f < nu; f += NW * 32) {
        const int l = level_of(st.u_block, ldim, f);
        const int off = f - st.u_block[l];
        const int mb = off / (l + 1), ma = off - mb * (l + 1);
        cx<T> v;
        if (2 * mb <= l) {
            v = Uh[st.h_block[l] + mb * (l + 1) + ma];
        } else {
            v = cconj(Uh[st.h_block[l] + (l - mb) * (l + 1) + (l - ma)]);
            if ((mb + ma) & 1) {
                v.re = -v.re;
                v.im = -v.im;
            }
        }
        Uf[f] = v;
    }
    __syncthreads();
}

// One Z entry (compute_zi, SO4.py:1020-1068).
template <typename T>
__device__ __forceinline__ cx<T> z_entry(const ZEnt &ze, const T *cg, const cx<T> *Uf) {
    cx<T> zz = mk<T>(T(0), T(0));
    int u1 = ze.u1 + ze.ma1min, u2 = ze.u2 + ze.ma2max, icgb = ze.cgb;
    for (int ib = 0; ib < ze.nb; ++ib) {
        cx<T> s = mk<T>(T(0), T(0));
        int icga = ze.cga;
        for (int ia = 0; ia < ze.na; ++ia) {
            cfma(s, cscale(Uf[u1 + ia], cg[icga]), Uf[u2 - ia]);
            icga += ze.l2;
        }
        zz = cadd(zz, cscale(s, cg[icgb]));
        u1 += ze.l1 + 1;
        u2 -= ze.l2 + 1;
        icgb += ze.l2;
    }
    return zz;
}

template <typename T, int NW>
__device__ void block_z(const ZEnt *zent, int nz, const T *cg, const cx<T> *Uf, cx<T> *Z) {
    for (int q = threadIdx.x; q < nz; q += NW * 32) Z[q] = z_entry<T>(zent[q], cg, Uf);
    __syncthreads();
}

// The Z entries of a list (e.g. only the blocks B reads), each to its own slot.
template <typename T, int NW>
__device__ void block_z_list(const ZEnt *list, int n, const T *cg, const cx<T> *Uf, cx<T> *Z) {
    for (int q = threadIdx.x; q < n; q += NW * 32) {
        const ZEnt ze = list[q];
        Z[ze.jz] = z_entry<T>(ze, cg, Uf);
    }
    __syncthreads();
}

// B_k = 2 Re sum' conj(U_l) Z(l1,l2,l) (compute_bi, SO4.py:1071-1111).
template <typename T, int NW, typename TO>
__device__ void block_b(const BEnt *bent, int nB, const cx<T> *Uh, const cx<T> *Z, TO *x) {
    for (int k = threadIdx.x; k < nB; k += NW * 32) {
        const BEnt be = bent[k];
        const int lam = be.lam[0], cnt = be.cnt[0];
        T s = T(0);
        for (int e = 0; e < cnt; ++e) {
            T v = redot(Uh[be.h[0] + e], Z[be.z[0] + e]);
            if ((lam % 2 == 0) && e == cnt - 1) v *= T(0.5);
            s += v;
        }
        x[k] = (TO)(T(2) * s);
    }
}

inline void fill_small_tables(const so4_tables *t, SmallTables &st) {
    st.twol = t->twol;
    for (int l = 0; l <= SO4_LDIM_MAX; ++l) {
        st.h_block[l] = (l <= t->ldim) ? t->h_block[l] : t->n_half;
        st.u_block[l] = (l < t->ldim) ? t->idxu_block[l] : t->n_u;
    }
    for (int l = 0; l < SO4_LDIM_MAX; ++l) st.unorm[l] = (l < t->ldim) ? t->unorm_l[l] : 1.0;
}
