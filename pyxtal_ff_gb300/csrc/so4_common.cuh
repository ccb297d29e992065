// so4_common.cuh -- shared device code of the SO(4)/SNAP bispectrum kernels.
//
// Layouts (see include/so4_gb300.h):
//   full layout  U_l[mb][ma], l = 0..twol, offset u_block[l] + mb*(l+1) + ma
//                (the reference's ulist / ulisttot, SO4.py:1288-1297)
//   half layout  rows mb = 0..floor(l/2) only, offset h_block[l] + mb*(l+1) + ma.
//                Rows above follow from U_l[l-mb][l-ma] = (-1)^(mb+ma) conj(U_l[mb][ma]),
//                the inversion-symmetry copy of SO4.py:908-925.
#pragma once

#include <utility>

#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

#include "../../include/so4_gb300.h"

#define SO4_PI 3.141592653589793
#define SO4_LDIM_MAX (SO4_TWOL_MAX + 1)

// ------------------------------------------------------------------ complex
template <typename T>
struct cx {
    T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T r, T i) {
    cx<T> z;
    z.re = r;
    z.im = i;
    return z;
}
template <typename T>
__device__ __forceinline__ cx<T> cconj(cx<T> a) { return mk<T>(a.re, -a.im); }
template <typename T>
__device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return mk<T>(a.re + b.re, a.im + b.im); }
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return mk<T>(a.re * s, a.im * s); }
// acc += a * b
template <typename T>
__device__ __forceinline__ void cfma(cx<T> &acc, cx<T> a, cx<T> b) {
    acc.re += a.re * b.re - a.im * b.im;
    acc.im += a.re * b.im + a.im * b.re;
}
// Re(conj(a) * b)
template <typename T>
__device__ __forceinline__ T redot(cx<T> a, cx<T> b) { return a.re * b.re + a.im * b.im; }

// ------------------------------------------------------------------ tables
// One Z entry (SO4.py:1344-1395 idxz row) with its CG offset and the full-layout
// offsets of the first U_l1 / U_l2 elements it reads.
struct ZEnt {
    int na, nb;          // inner / outer trip counts
    int ma1min, ma2max;  // first column of U_l1, U_l2
    int cga, cgb;        // CG offsets of the first inner / outer coefficient
    int u1, u2;          // full offsets of U_l1[mb1min][0], U_l2[mb2max][0]
    int l1, l2;          // row strides - 1
    int jh;              // half offset of (l, mb, ma)
    int blk;             // Z block index
    int jz;              // index of this entry in the full Z list
};

// One bispectrum component k = (l1, l2, l), l >= l1 >= l2 (SO4.py:1314-1327),
// with the three Z blocks its derivative reads (SO4.py:1113-1227).
struct BEnt {
    int l1, l2, l;
    int z[3];     // idxz_block[l1][l2][l], [l][l2][l1], [l][l1][l2]
    int h[3];     // half offsets of levels l, l1, l2
    int cnt[3];   // entries of each section (2mb < lam rows + first half of middle row)
    int lam[3];   // l, l1, l2
    double fac[3];  // 2, 2 (l+1)/(l1+1), 2 (l+1)/(l2+1)
};

// One Z block (l1, l2, l), l1 >= l2; the bispectrum components that read it and
// with which factor (used to build the adjoint array Y).
struct ZBlk {
    int l1, l2, l;
    int z0, n;       // first entry, entry count ((l/2+1) (l+1))
    int nrole;
    int role_k[3];
    double role_f[3];
    float role_f32[3];  // role_f in FP32 for the FP32 kernels (no FP64 conversion on the device)
};

struct so4_tables {
    int twol, ldim, normalize_u;
    so4_tuning tune;  // launch shapes, defaults filled in (so4_tables_create_tuned)
    int n_u, n_half, n_z, n_b, n_cg, n_blk;
    // host copies (reference-visible)
    std::vector<double> cglist;
    std::vector<int> idxb, idxz, idxu_block, idxz_block, idxcg_block;
    std::vector<int> h_block;  // ldim + 1
    std::vector<double> unorm_l;  // per level
    // device copies
    double *d_cg64 = nullptr;
    float *d_cg32 = nullptr;
    double *d_rootpq64 = nullptr;  // ldim x ldim
    float *d_rootpq32 = nullptr;
    ZEnt *d_z = nullptr;
    BEnt *d_b = nullptr;
    ZBlk *d_blk = nullptr;
    // per Z block, packed for the window kernels' coefficient loop: the components of its
    // roles {k0, k1, k2, nrole} (missing roles repeat k0) and their FP32 factors (0 when missing)
    int4 *d_blk_rk = nullptr;
    float4 *d_blk_rf = nullptr;
    int *d_yblk_ptr = nullptr;  // ldim + 1 : blocks grouped by their third index
    int *d_yblk = nullptr;      // n_blk
    // n_half: half entry -> {full position, mirror position | conj << 15 | negate << 14 or -1}
    int2 *d_hfull = nullptr;
    // n_half: per half entry (level L, row, ma) {L(L+1)/2 + ma | row << 8 | (ma == row) << 15,
    // bits of u_norm[L] F, bits of u_norm[L], 0}: where the row-chain kernels keep it and how
    // it is finished (F the row scale of the scaled recursion, so4_tables.cu)
    int4 *d_hmap = nullptr;
    float *d_yscale = nullptr;  // n_half: the row-scale F of each half entry (so4_tables.cu)
    double *d_yscale64 = nullptr;  // the same in FP64 (the plain path's scaled derivative pass)
    // The plain path's dB/dr sections: every distinct Z block they read, contracted once per
    // image by one lane of a warp, {first Z entry, half offset, entry count, level}, listed
    // lane by lane (lane l owns [psec_ptr[l], psec_ptr[l + 1])) with the lanes' entry counts
    // balanced; ksec[3 k + s]: the list position of component k's section s.
    int4 *d_psec = nullptr;
    int *d_psec_ptr = nullptr;  // 33
    int *d_ksec = nullptr;      // 3 nB
    int n_psec = 0;
    // B partial slots of the window kernels: one per (window unit, B block), component k
    // owning slots [bpos[k], bpos[k + 1]) in row order
    int *d_bpos = nullptr;  // nB + 1
    int n_bsec = 0;
    // window work lists (so4_zwin.cuh), most expensive unit first:
    //   unit {lam | mb << 8 | ma0 << 16 | K << 24, seg0, seg1, bits of u_norm[lam]}
    //   segment {sub0, sub1, block, B partial slot or -1}
    //   sub-segment {f1 | f2 << 16 (shared-memory offsets), Ca offset, steps, bits of Cb}
    // wunit_y/wseg_y cover every half entry and every block (Y, and B in the fused
    // path); wunit_b/wseg_b only the B-section entries and the B blocks.
    int4 *d_wunit_y = nullptr, *d_wseg_y = nullptr, *d_wunit_b = nullptr, *d_wseg_b = nullptr;
    int4 *d_wsub = nullptr;
    float *d_wca = nullptr;
    int n_wunit_y = 0, n_wunit_b = 0, n_wca = 0;
    // window JVP lists (units of the B sections, blocks with a role; segment .w = the unit's
    // section index), the slot range of each component, and per (block, role) slot base / factor
    int4 *d_wunit_j = nullptr, *d_wseg_j = nullptr;
    int *d_jpos = nullptr, *d_jbase = nullptr;
    float *d_jfac = nullptr;
    int n_wunit_j = 0, n_jslot = 0;
    int n_jmax = 0;  // the most slots one component owns
    int n_wsub = 0;  // window sub-segments
};

// Window Z contractions: most entries per unit, and the zero rows kept before
// and after the U tiles in shared memory (a window may reach ZW_KMAX - 1 entries
// past either end of the full layout, always with a zero coefficient).
constexpr int ZW_KMAX = 5;
constexpr int ZW_KPAIR = 5;  // window units of K <= ZW_KPAIR walk their rows in pairs (here every unit)
constexpr int ZW_PAD = ZW_KMAX - 1;

// Table data every kernel stages into shared memory at start.
struct SmallTables {
    int twol;
    int h_block[SO4_LDIM_MAX + 1];
    int u_block[SO4_LDIM_MAX + 1];
    double unorm[SO4_LDIM_MAX];
};

// ------------------------------------------------------------------ cutoff
// Cutoff functions and derivatives of SO4.py:306-408 (compute_sfac/dsfac :482-558).
template <typename T>
__device__ __forceinline__ void cutoff_fn(int id, T r, T rc, T &f, T &df) {
    if (r > rc) {
        f = T(0);
        df = T(0);
        return;
    }
    const T x = r / rc;
    switch (id) {
        case 1: {
            T s, c;
            if (sizeof(T) == 8) {
                double sd, cd;
                sincospi((double)(r / rc), &sd, &cd);
                s = (T)sd;
                c = (T)cd;
            } else {
                float sf, cf;
                sincospif((float)(r / rc), &sf, &cf);
                s = (T)sf;
                c = (T)cf;
            }
            f = T(0.5) * (c + T(1));
            df = T(-0.5) * T(SO4_PI) / rc * s;
            break;
        }
        case 2: {
            T t = tanh(T(1) - x);
            T t2 = t * t;
            f = t2 * t;
            df = -(T(3) / rc) * t2 * (T(1) - t2);
            break;
        }
        case 3:
            f = x * x * (T(2) * x - T(3)) + T(1);
            df = (T(6) / (rc * rc)) * r * (x - T(1));
            break;
        case 4:
            f = x * x * x * (x * (T(15) - T(6) * x) - T(10)) + T(1);
            df = (T(-30) / rc) * (x * x * (x - T(1)) * (x - T(1)));
            break;
        case 5: {
            T y = x - T(1);
            f = x * x * x * x * (x * (x * (T(20) * x - T(70)) + T(84)) - T(35)) + T(1);
            df = (T(140) / rc) * (x * x * x * (y * y * y));
            break;
        }
        case 6: {
            T y = x - T(1);
            f = x * x * x * x * x * (x * (x * (x * (T(315) - T(70) * x) - T(540)) + T(420)) - T(126)) + T(1);
            df = (T(-630) / rc) * (x * x * x * x * (y * y * y * y));
            break;
        }
        case 7: {
            // the reference's Exponent / ExponentPrime as written (SO4.py:391-408)
            T d = T(1) - x * x;
            if (d == T(0)) {
                f = T(0);
                df = T(0);
            } else {
                T e = exp(T(1) - T(1) / d);
                T q = T(1) + x * x;
                f = e;
                df = T(2) * x * e / (q * q);
            }
            break;
        }
        default:
            f = T(0);
            df = T(0);
    }
}

// ------------------------------------------------------------------ U recursion
// Cayley-Klein parameters and their gradients (SO4.py:879-884, 935-948).
template <typename T>
struct CK {
    cx<T> ca, cb;          // conj(a), conj(b)
    cx<T> cda[3], cdb[3];  // conj(da/dr_c), conj(db/dr_c)
};

template <typename T, bool DERIV>
__device__ __forceinline__ void make_ck(T x, T y, T z, T r, T psi, CK<T> &ck) {
    T sn, cs;
    if (sizeof(T) == 8) {
        double s_, c_;
        sincos((double)psi, &s_, &c_);
        sn = (T)s_;
        cs = (T)c_;
    } else {
        float s_, c_;
        sincosf((float)psi, &s_, &c_);
        sn = (T)s_;
        cs = (T)c_;
    }
    const T sr = sn / r;
    // a = cos(psi) - i sin(psi) z / r ; b = sin(psi) / r (y - i x)
    ck.ca = mk<T>(cs, sr * z);
    ck.cb = mk<T>(sr * y, sr * x);
    if (DERIV) {
        const T g[3] = {x / r, y / r, z / r};
        const T r2 = r * r;
        const T fa = -sn * psi / r;                     // d Re(a)
        const T fai = -z * cs / r2 * psi + z * sn / r2;  // d Im(a) (radial part)
        const T fb = cs / r2 * psi - sn / r2;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cx<T> da = mk<T>(fa * g[c], fai * g[c]);
            cx<T> db = mk<T>(fb * y * g[c], -(fb * x) * g[c]);
            if (c == 2) da.im -= sr;
            if (c == 1) db.re += sr;
            if (c == 0) db.im -= sr;
            ck.cda[c] = cconj(da);
            ck.cdb[c] = cconj(db);
        }
    }
}

// Value of row mb of level l-1 at column c, read from the half layout of level
// l-1 (mirror of row l/2-1 when mb = l/2 > floor((l-1)/2)).
template <typename T>
__device__ __forceinline__ cx<T> prev_row(const cx<T> *Hp, int l, int mb, int c) {
    const int L = l - 1;
    if (2 * mb <= L) return Hp[mb * l + c];
    cx<T> v = Hp[(L - mb) * l + (L - c)];
    v = cconj(v);
    if ((mb + c + L + L) & 1) {  // (-1)^((L-mb)+(L-c))
        v.re = -v.re;
        v.im = -v.im;
    }
    return v;
}

// Warp-cooperative Wigner-U (and dU/dr) of one image on the half layout
// (compute_uarray_recursive / compute_duarray_recursive, SO4.py:840-987):
//   U_l[mb][ma] = rootpq[l-ma][l-mb] conj(a) U_{l-1}[mb][ma]
//               - rootpq[ma][l-mb]  conj(b) U_{l-1}[mb][ma-1]
// then, for even l, the middle row's centre is conjugated and its upper half
// set from the lower half, as the reference's symmetry copy does.
// H[n_half] and dH[3][n_half] are per-warp shared buffers; lanes split the
// entries of each level.  rootpq is (twol+1)^2 in shared memory.
template <typename T, bool DERIV>
__device__ void warp_uarray(const SmallTables &st, const T *rootpq, const CK<T> &ck, cx<T> *H, cx<T> *dH,
                            int n_half, int lane) {
    const int ldim = st.twol + 1;
    if (lane == 0) {
        H[0] = mk<T>(T(1), T(0));
        if (DERIV) {
            dH[0] = mk<T>(T(0), T(0));
            dH[n_half] = mk<T>(T(0), T(0));
            dH[2 * n_half] = mk<T>(T(0), T(0));
        }
    }
    __syncwarp();
    for (int l = 1; l < ldim; ++l) {
        const int ncol = l + 1;
        const int n = (l / 2 + 1) * ncol;
        cx<T> *Hl = H + st.h_block[l];
        const cx<T> *Hp = H + st.h_block[l - 1];
        for (int e = lane; e < n; e += 32) {
            const int mb = e / ncol;
            const int ma = e - mb * ncol;
            cx<T> v = mk<T>(T(0), T(0));
            cx<T> dv[3];
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) dv[c] = mk<T>(T(0), T(0));
            }
            if (ma > 0) {
                const T rp = -rootpq[ma * ldim + (l - mb)];
                const cx<T> P = prev_row(Hp, l, mb, ma - 1);
                v = cscale(cmul(ck.cb, P), rp);
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const cx<T> dP = prev_row(dH + c * n_half + st.h_block[l - 1], l, mb, ma - 1);
                        dv[c] = cscale(cadd(cmul(ck.cdb[c], P), cmul(ck.cb, dP)), rp);
                    }
                }
            }
            if (ma < l) {
                const T rp = rootpq[(l - ma) * ldim + (l - mb)];
                const cx<T> P = prev_row(Hp, l, mb, ma);
                v = cadd(v, cscale(cmul(ck.ca, P), rp));
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const cx<T> dP = prev_row(dH + c * n_half + st.h_block[l - 1], l, mb, ma);
                        dv[c] = cadd(dv[c], cscale(cadd(cmul(ck.cda[c], P), cmul(ck.ca, dP)), rp));
                    }
                }
            }
            Hl[e] = v;
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) dH[c * n_half + st.h_block[l] + e] = dv[c];
            }
        }
        __syncwarp();
        if ((l & 1) == 0) {
            // middle row mb = l/2: centre -> conj, upper half -> mirror of lower half
            const int mid = (l / 2) * ncol;
            const int h = l / 2;
            for (int ma = h + lane; ma <= l; ma += 32) {
                const int src = (ma == h) ? ma : (l - ma);
                const bool neg = ((h + ma) & 1) != 0;
                cx<T> v = cconj(Hl[mid + src]);
                if (neg && ma != h) {
                    v.re = -v.re;
                    v.im = -v.im;
                }
                Hl[mid + ma] = v;
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        cx<T> *dHl = dH + c * n_half + st.h_block[l];
                        cx<T> dv = cconj(dHl[mid + src]);
                        if (neg && ma != h) {
                            dv.re = -dv.re;
                            dv.im = -dv.im;
                        }
                        dHl[mid + ma] = dv;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// acc += a b and acc -= a b on complex values, as four FMAs each.
template <typename T>
__device__ __forceinline__ void cmac(cx<T> &acc, const cx<T> &a, const cx<T> &b) {
    acc.re = fma(a.re, b.re, fma(-a.im, b.im, acc.re));
    acc.im = fma(a.re, b.im, fma(a.im, b.re, acc.im));
}
template <typename T>
__device__ __forceinline__ void cmsub(cx<T> &acc, const cx<T> &a, const cx<T> &b) {
    acc.re = fma(-a.re, b.re, fma(a.im, b.im, acc.re));
    acc.im = fma(-a.re, b.im, fma(-a.im, b.re, acc.im));
}

// warp_uarray in the scaled form V_l[mb][ma] = U_l[mb][ma] / F, F = sqrt(C(l, mb) / C(l, ma))
// (C binomial; the row-scale table of so4_tables.cu).  The recursion's coefficients
// rootpq[l-ma][l-mb] and rootpq[ma][l-mb] cancel against the scale:
//   V_l[mb][ma] = conj(a) V_{l-1}[mb][ma] - conj(b) V_{l-1}[mb][ma-1],
// and the chain-start mirror and the middle-row symmetry keep their form, because
// C(l, ma) = C(l, l - ma).  So U = F V, and a contraction Re sum conj(dU) Z equals
// Re sum conj(dV) (F Z): callers pre-scale Z by F instead of unscaling every row.
// 56 FMAs per entry with DERIV against about 92 operations in warp_uarray.
template <typename T, bool DERIV>
__device__ void warp_vrows(const SmallTables &st, const CK<T> &ck, cx<T> *H, cx<T> *dH, int n_half, int lane) {
    const int ldim = st.twol + 1;
    if (lane == 0) {
        H[0] = mk<T>(T(1), T(0));
        if (DERIV) {
            dH[0] = mk<T>(T(0), T(0));
            dH[n_half] = mk<T>(T(0), T(0));
            dH[2 * n_half] = mk<T>(T(0), T(0));
        }
    }
    __syncwarp();
    for (int l = 1; l < ldim; ++l) {
        const int ncol = l + 1;
        const int n = (l / 2 + 1) * ncol;
        cx<T> *Hl = H + st.h_block[l];
        const cx<T> *Hp = H + st.h_block[l - 1];
        for (int e = lane; e < n; e += 32) {
            const int mb = e / ncol;
            const int ma = e - mb * ncol;
            cx<T> v = mk<T>(T(0), T(0));
            cx<T> dv[3];
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) dv[c] = mk<T>(T(0), T(0));
            }
            if (ma > 0) {
                const cx<T> P = prev_row(Hp, l, mb, ma - 1);
                cmsub(v, ck.cb, P);
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const cx<T> dP = prev_row(dH + c * n_half + st.h_block[l - 1], l, mb, ma - 1);
                        cmsub(dv[c], ck.cdb[c], P);
                        cmsub(dv[c], ck.cb, dP);
                    }
                }
            }
            if (ma < l) {
                const cx<T> P = prev_row(Hp, l, mb, ma);
                cmac(v, ck.ca, P);
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const cx<T> dP = prev_row(dH + c * n_half + st.h_block[l - 1], l, mb, ma);
                        cmac(dv[c], ck.cda[c], P);
                        cmac(dv[c], ck.ca, dP);
                    }
                }
            }
            Hl[e] = v;
            if (DERIV) {
#pragma unroll
                for (int c = 0; c < 3; ++c) dH[c * n_half + st.h_block[l] + e] = dv[c];
            }
        }
        __syncwarp();
        if ((l & 1) == 0) {
            // middle row mb = l/2: centre -> conj, upper half -> mirror of lower half
            const int mid = (l / 2) * ncol;
            const int h = l / 2;
            for (int ma = h + lane; ma <= l; ma += 32) {
                const int src = (ma == h) ? ma : (l - ma);
                const bool neg = ((h + ma) & 1) != 0;
                cx<T> v = cconj(Hl[mid + src]);
                if (neg && ma != h) {
                    v.re = -v.re;
                    v.im = -v.im;
                }
                Hl[mid + ma] = v;
                if (DERIV) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        cx<T> *dHl = dH + c * n_half + st.h_block[l];
                        cx<T> dv = cconj(dHl[mid + src]);
                        if (neg && ma != h) {
                            dv.re = -dv.re;
                            dv.im = -dv.im;
                        }
                        dHl[mid + ma] = dv;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Number of half-layout entries one dB/dr section of level lam sums over
// (rows 2mb < lam, plus the first lam/2+1 entries of the middle row for even lam).
__host__ __device__ __forceinline__ int section_count(int lam) {
    const int full = (lam + 1) / 2;  // rows with 2mb < lam
    return full * (lam + 1) + ((lam % 2 == 0) ? lam / 2 + 1 : 0);
}

#define SO4_CUDA_TRY(expr)                       \
    do {                                         \
        cudaError_t e_ = (expr);                 \
        if (e_ != cudaSuccess) return SO4_ERR_CUDA; \
    } while (0)

// status word at the start of every workspace
#define SO4_WS_HEADER 256

// Dynamic shared memory of the window kernels in each of their four modes (so4_adjoint.cu).
void so4_zw_smem_modes(const so4_tables *t, size_t out[4]);

// number of kernels this library has launched (so4_launch_count)
void so4_count_launch(int n = 1);

// Programmatic dependent launch (PDL).  While so4_set_pdl(1) is in effect on the calling
// host thread, so4_launch_pdl gives its launch the programmatic-stream-serialization
// attribute: the kernel may be scheduled as soon as every CTA of the kernel before it in
// the stream has called pdl_trigger() (or exited), and runs its code up to pdl_wait()
// while that kernel finishes.  A kernel launched this way calls pdl_wait() before it
// reads anything an earlier kernel of the stream writes and before its first global
// store; what it does before (index set-up, loads of constant tables) overlaps the
// previous kernel's tail.  Launched without the attribute, pdl_wait() returns at once.
int so4_pdl_on();
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <typename... KArgs, typename... Args>
int so4_launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = so4_pdl_on() ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
    so4_count_launch();
    return e == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}
// Raise a kernel's dynamic shared-memory limit to at least smem bytes on the current
// device.  The attribute is set only when the limit grows, so launches after the
// first make no runtime call besides the launch (safe inside stream capture).
int so4_set_smem(const void *kern, size_t smem);
// The JVP's Z contraction by the window kernel (so4_adjoint.cu): dB [natoms][nB] from
// U_tot and its tangent dU (both [natoms][nh] float2), with n_jslot x natoms floats of
// slot scratch.
int so4_zw_jvp32(const so4_tables *t, int natoms, const float *d_utot, const float *d_du, float *d_slots, float *d_dB,
                 cudaStream_t stream);
