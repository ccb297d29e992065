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
#include "so4_rev2.cuh"
#include "so4_rowchain.cuh"
#include "so4_zwin.cuh"
#include "so4_zwin2.cuh"

namespace {

constexpr int NWF = 4;  // warps per CTA, forward
constexpr int NWD = 8;  // warps per CTA, per-image contraction

struct AdjWork {
    int *status;
    float2 *Y;       // natoms * n_half
    float *g;        // nimg * 3
    double *part;    // gather_part_doubles(natoms): per-chunk virial + energy partials
};

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int GCH = 32;    // atoms per gather chunk (one CTA)
constexpr int GPART = 10;  // doubles per chunk partial: virial (9) + energy

size_t gather_part_doubles(int natoms) { return (size_t)GPART * ((size_t)(natoms + GCH - 1) / GCH + 1); }

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
    w.part = (double *)take(sizeof(double) * gather_part_doubles(natoms));
    return off;
}

template <typename K>
int set_smem(K kern, size_t smem) {
    return so4_set_smem((const void *)kern, smem);
}

struct FwdArgs {
    so4_params prm;
    float psi_fac, rc32;  // rfac0 pi / rcut and rcut in FP32, set on the host
    int natoms, nh, nu, nz, nB;
    const double *w_nb, *w_site, *img_r;
    const int32_t *img_ptr, *img_j;
    const float *cg, *rootpq;
    const BEnt *bent;
    SmallTables st;
    const int4 *hmap;  // per half entry: accumulator slot, row, diagonal flag, u_norm F, u_norm
    float *utot, *x;
};

// U_tot of one centre per CTA (half layout, to global).
__global__ void __launch_bounds__(NWF * 32) k_utot32(FwdArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
    const int tid = threadIdx.x;
    const int a = blockIdx.x;
    if (tid == 0) st = A.st;
    const int ldim = A.st.twol + 1;
    const int nh = A.nh;
    float *rootpq = (float *)smem_raw;
    cx<float> *Uh = (cx<float> *)(rootpq + ((ldim * ldim + 1) & ~1));
    cx<float> *W = Uh + nh;  // per warp: H[nh], P[nh]
    for (int q = tid; q < ldim * ldim; q += NWF * 32) rootpq[q] = A.rootpq[q];
    __syncthreads();
    const float rc = (float)A.prm.rcut;
    const float psi_fac = (float)(A.prm.rfac0 * SO4_PI / A.prm.rcut);
    block_utot<float, NWF>(st, rootpq, a, A.img_r, A.img_j, A.img_ptr[a], A.img_ptr[a + 1], A.w_nb, A.w_site[a], rc,
                           psi_fac, A.prm.cutoff_id, nh, W, W + nh, 2 * nh, Uh);
    float2 *ug = (float2 *)A.utot + (size_t)a * nh;
    for (int e = tid; e < nh; e += NWF * 32) ug[e] = make_float2(Uh[e].re, Uh[e].im);
}

// U_tot with the row-chain recursion: one warp per centre, UtotLanes<TWOL>::IPW
// images per round (lanes per image: one per row chain; at twol 8 the last lane runs the
// last two chains).  Each lane accumulates w_j sfac U over its images for its chain's rows;
// the image groups are then added through shared memory in group order, the self term
// f_c(0) w_site is put on the diagonal and u_norm applied (SO4.py:1480-1505, 560-597).
template <int TWOL, int NW>
__global__ void __launch_bounds__(NW * 32, (TWOL <= 8) ? 16 / NW : 1) k_utot_rc(FwdArgs A) {
    using UL = UtotLanes<TWOL>;
    constexpr int W = TWOL + 1, NACC = acc_block(TWOL + 1);
    extern __shared__ __align__(16) float ut_smem[];  // [NW][32][2 * NACC]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int a = blockIdx.x * NW + wid;
    const int grp = lane / UL::LPI, mb = lane - grp * UL::LPI;
    float2 acc[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) acc[q] = make_float2(0.f, 0.f);
    pdl_wait();  // the neighbour list comes from the kernel before
    if (a < A.natoms) {
        const int m0 = A.img_ptr[a], m1 = A.img_ptr[a + 1];
        // Cayley-Klein parameters and weights of up to 32 images at once, one per lane;
        // each recursion iteration then takes its IPW images' values by shuffles (one
        // setup pass per 32 images instead of one per IPW)
        for (int base = m0; base < m1; base += 32) {
            float x = 1.f, y = 0.f, z = 0.f, wsf0 = 0.f;
            const int m = base + lane;
            if (m < m1) {
                x = (float)A.img_r[3 * m];
                y = (float)A.img_r[3 * m + 1];
                z = (float)A.img_r[3 * m + 2];
                const float rr = sqrtf(x * x + y * y + z * z);
                if (rr >= 1e-8f) {
                    float sf, dsf;
                    cutoff_fn<float>(A.prm.cutoff_id, rr, A.rc32, sf, dsf);
                    wsf0 = (float)A.w_nb[A.img_j[m]] * sf;
                } else {
                    x = 1.f;
                    y = z = 0.f;
                }
            }
            CK<float> ck0;
            {
                const float r = sqrtf(x * x + y * y + z * z);
                make_ck<float, false>(x, y, z, r, A.psi_fac * r, ck0);
            }
            const int nimg = min(32, m1 - base);
            for (int sub = 0; sub < nimg; sub += UL::IPW) {
                // lane (grp, mb) takes image sub + grp; lanes past the images take a zero weight
                const int src = sub + grp;
                const bool ok = grp < UL::IPW && src < nimg;
                const int sl = ok ? src : 0;
                CK<float> ck;
                ck.ca.re = __shfl_sync(0xffffffffu, ck0.ca.re, sl);
                ck.ca.im = __shfl_sync(0xffffffffu, ck0.ca.im, sl);
                ck.cb.re = __shfl_sync(0xffffffffu, ck0.cb.re, sl);
                ck.cb.im = __shfl_sync(0xffffffffu, ck0.cb.im, sl);
                float wsf = __shfl_sync(0xffffffffu, wsf0, sl);
                if (!ok) wsf = 0.f;
                float2 u[W];
#pragma unroll
                for (int q = 0; q < W; ++q) u[q] = make_float2(0.f, 0.f);
                u[0].x = 1.f;
                if (mb == 0) acc[0].x += wsf;
                RcUtot2<TWOL, 1>::run(mb, ck, wsf, u, acc);
            }
        }
    }
    pdl_trigger();  // the next kernel may start its set-up during this epilogue
    float2 *sw = reinterpret_cast<float2 *>(ut_smem) + (size_t)wid * 32 * NACC;
#pragma unroll
    for (int q = 0; q < NACC; ++q) sw[lane * NACC + q] = acc[q];
    __syncwarp();
    if (a >= A.natoms) return;
    float f0, df0;
    cutoff_fn<float>(A.prm.cutoff_id, 0.f, A.rc32, f0, df0);
    const float selfw = f0 * (float)A.w_site[a];
    float2 *ug = (float2 *)A.utot + (size_t)a * A.nh;
    for (int e = lane; e < A.nh; e += 32) {
        const int4 h = __ldg(A.hmap + e);
        const int slot = h.x & 0xff, row = (h.x >> 8) & 0x7f;
        const int ln = UL::lane_of(row), sq = UL::slot_of(row, slot);
        float sr = 0.f, si = 0.f;
#pragma unroll
        for (int g = 0; g < UL::IPW; ++g) {
            const float2 v = sw[(g * UL::LPI + ln) * NACC + sq];
            sr += v.x;
            si += v.y;
        }
        // sums of scaled rows: times u_norm F; the self term (diagonal) times u_norm
        const float unf = __int_as_float(h.y), un = __int_as_float(h.z);
        sr *= unf;
        if (h.x & (1 << 15)) sr = fmaf(selfw, un, sr);
        ug[e] = make_float2(sr, si * unf);
    }
}

template <int TWOL, int NW>
int launch_utot_rc_nw(const FwdArgs &A, cudaStream_t st) {
    const size_t smem = sizeof(float) * NW * 32 * 2 * acc_block(TWOL + 1);
    int rc = set_smem(k_utot_rc<TWOL, NW>, smem);
    if (rc) return rc;
    return so4_launch_pdl(k_utot_rc<TWOL, NW>, dim3((A.natoms + NW - 1) / NW), dim3(NW * 32), smem, st, A);
}

// nw: warps (centres) per CTA, from the tables' tuning; 2 and 8 are built for twol 6 and 8
template <int TWOL>
int launch_utot_rc(const FwdArgs &A, int nw, cudaStream_t st) {
    if constexpr (TWOL == 6 || TWOL == 8) {
        if (nw == 2) return launch_utot_rc_nw<TWOL, 2>(A, st);
        if (nw == 8) return launch_utot_rc_nw<TWOL, 8>(A, st);
    }
    return launch_utot_rc_nw<TWOL, 4>(A, st);
}

struct ZLArgs {
    int natoms, nh, nu, nB, nblk, nunit;
    const float2 *utot;
    const int2 *hfull;
    const int4 *unit, *seg;
    const BEnt *bent;
    const ZBlk *blk;
    const int4 *blk_rk;    // per block: role components (so4_tables: d_blk_rk)
    const float4 *blk_rf;  // per block: role factors
    const int *yptr, *ylist;
    const float *beta;
    const int *bpos;  // nB + 1: first B partial slot of each component
    int nbsec;  // slots of the B partial (MODE 0, 2) or JVP (MODE 3) scratch
    SmallTables st;
    float *x;    // B out  (k_zb32, k_zby32)
    float2 *Y;   // Y out  (k_zy32, k_zby32)
    float *bc;   // B partial sums, slot-major [nbsec][natoms]
    float *eatom;  // fused path: sum_k beta_k B_k per atom (may be null)
    const int4 *wsub;  // window sub-segments
    const float *wca;  // window Ca rows
    int nwca;          // their floats (a multiple of 4)
    // JVP (MODE 3): tangent dU [natoms][nh], per (block, role) slot base / factor, slot range
    // of each component; the slots go to bc and dB to x
    const float2 *dU;
    const int *jbase, *jpos;
    const float *jfac;
    const float *yscale;  // n_half: Y is stored times the row scale F of its entry
    int stage_cap;        // MODE 3: slot rows the epilogue stages at a time (those fitting over the U tiles)
};


// One window unit of K entries: Z of every block feeding its level; Y (MODE 1, 2),
// the B-section scratch (MODE 0, 2) or the JVP section scratch (MODE 3).
template <int MODE, int K>
__device__ __forceinline__ void zw_unit(const ZLArgs &A, const int4 un, const float2 *Ul, const float *coef,
                                        const float *__restrict__ ca, int a,
                                        int lane) {
    const int lam = un.x & 0xff, mb = (un.x >> 8) & 0xff, ma0 = (un.x >> 16) & 0xff;
    const int off0 = mb * (lam + 1) + ma0;
    const int cnt = section_count(lam);
    float2 y[K];
#pragma unroll
    for (int k = 0; k < K; ++k) y[k] = make_float2(0.f, 0.f);
    // MODE 3: w_e dU[e] of the unit's entries in the section (0 past its end), reused by every block
    float dur[K], dui[K];
    if (MODE == 3) {
        const float2 *dp = A.dU + (size_t)min(a, A.natoms - 1) * A.nh + A.st.h_block[lam] + off0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int off = off0 + k;
            float2 d = make_float2(0.f, 0.f);
            if (off < cnt) d = __ldg(dp + k);
            const float w = ((lam & 1) == 0 && off == cnt - 1) ? 0.5f : 1.f;
            dur[k] = w * d.x;
            dui[k] = w * d.y;
        }
    }
    // headers are prefetched one ahead: the next segment's and the next sub-segment's
    // loads are in flight while the current one computes
    int4 sgn = (un.y < un.z) ? __ldg(A.seg + un.y) : make_int4(0, 0, 0, -1);
    for (int q = un.y; q < un.z; ++q) {
        const int4 sg = sgn;
        if (q + 1 < un.z) sgn = __ldg(A.seg + q + 1);
        float2 z[K];
#pragma unroll
        for (int k = 0; k < K; ++k) z[k] = make_float2(0.f, 0.f);
        // rows two at a time (they share the Ca table and S), the odd one alone; the two
        // register rings fit without spills up to K = ZW_KPAIR
        int r = sg.x;
        int4 h1 = (r < sg.y) ? __ldg(A.wsub + r) : make_int4(0, 0, 0, 0);
        if (K <= ZW_KPAIR) {
            int4 h2 = (r + 1 < sg.y) ? __ldg(A.wsub + r + 1) : make_int4(0, 0, 0, 0);
            for (; r + 1 < sg.y; r += 2) {
                const int4 c1 = h1, c2 = h2;
                if (r + 2 < sg.y) h1 = __ldg(A.wsub + r + 2);
                if (r + 3 < sg.y) h2 = __ldg(A.wsub + r + 3);
                zw_rows2<K>(Ul, c1, c2, ca, z);
            }
            if (r < sg.y) zw_rows<K>(Ul, h1, ca, z);
        } else {
            for (; r < sg.y; ++r) {
                const int4 hd = h1;
                if (r + 1 < sg.y) h1 = __ldg(A.wsub + r + 1);
                zw_rows<K>(Ul, hd, ca, z);
            }
        }
        if (MODE == 3) {
            // sum_e w_e Re(conj(dU[e]) Z[e]) over the unit's section entries, once per role of
            // the block: slot (jbase + unit index) of the role's component, scaled by fac_s
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) v = fmaf(dur[k], z[k].x, fmaf(dui[k], z[k].y, v));
            if (a < A.natoms) {
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const int jb = __ldg(A.jbase + 3 * sg.z + r);
                    if (jb < 0) break;
                    A.bc[(size_t)(jb + sg.w) * A.natoms + a] = __ldg(A.jfac + 3 * sg.z + r) * v;
                }
            }
        }
        if (MODE == 1 || MODE == 2) {
            const float c = coef[sg.z * ZL_PITCH + lane];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                y[k] = __ffma2_rn(make_float2(c, c), z[k], y[k]);
            }
        }
        if ((MODE == 0 || MODE == 2) && sg.w >= 0) {
            // this unit's part of the B component of the block: sum over its entries in the
            // B section of w_e Re(conj(U_lam[e]) Z[e]), w_e = 1/2 at the middle-row centre
            const float2 *ul = Ul + (ZW_PAD + A.st.u_block[lam] + off0) * ZL_PITCH;
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int off = off0 + k;
                if (off < cnt) {
                    const float2 uv = ul[k * ZL_PITCH];
                    const float d = __fmaf_rn(uv.y, z[k].y, __fmul_rn(uv.x, z[k].x));
                    v += ((lam & 1) == 0 && off == cnt - 1) ? 0.5f * d : d;
                }
            }
            // scratch is slot-major, so the 32 lanes (atoms) store one contiguous line
            if (a < A.natoms) A.bc[(size_t)sg.w * A.natoms + a] = v;
        }
    }
    if ((MODE == 1 || MODE == 2) && a < A.natoms) {
        const float un_l = __int_as_float(un.w);
        float2 *Yo = A.Y + (size_t)a * A.nh + A.st.h_block[lam] + off0;
        const float *ys = A.yscale + A.st.h_block[lam] + off0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int ma = ma0 + k;
            const float wmid = (2 * mb < lam) ? 1.f : ((2 * ma < lam) ? 1.f : ((2 * ma == lam) ? 0.5f : 0.f));
            // times the row scale F: the reverse sweep contracts the scaled rows with it
            const float s = un_l * wmid * __ldg(ys + k);
            Yo[k] = make_float2(s * y[k].x, s * y[k].y);
        }
        // no unit computes the upper half of an even level's middle row (its Y is zero): the
        // unit ending at the row's centre writes those zeros, so every Y entry is defined
        if (2 * mb == lam && ma0 + K - 1 == lam / 2) {
            for (int ma = lam / 2 + 1; ma <= lam; ++ma) Yo[ma - ma0] = make_float2(0.f, 0.f);
        }
    }
}


// zw_unit for the unit's K (1 <= k <= ZW_KMAX, from the work list)
template <int MODE, int K = ZW_KMAX>
__device__ __forceinline__ void zw_unit_k(int k, const ZLArgs &A, const int4 un, const float2 *Ul, const float *coef,
                                          const float *__restrict__ ca, int a, int lane) {
    if constexpr (K > 1) {
        if (k != K) {
            zw_unit_k<MODE, K - 1>(k, A, un, Ul, coef, ca, a, lane);
            return;
        }
    }
    zw_unit<MODE, K>(A, un, Ul, coef, ca, a, lane);
}

// Window form of k_zb32 / k_zy32 / k_zby32 (so4_zwin.cuh), 32 atoms per CTA.
// MODE 0: B only (units of the B sections, B blocks only); 1: Y only; 2: Y and,
// per (unit, B block), the unit's part of the section sum sum_e w_e Re(conj(U_lam[e]) Z[e])
// into the slot-major scratch d_bc, then B_k = 2 x the sum of component k's slots in
// a fixed order (compute_bi, SO4.py:1071-1111) and, with d_eatom, beta . B per atom.
// MODE 3: the JVP dB_k = sum_s fac_s sum_e w_e Re(conj(dU[e]) Z_s[e]) (compute_dbidrj,
// SO4.py:1113-1227, along one tangent dU): per (unit, block, role) slots, summed per k.
template <int MODE, bool CA_SMEM>
__global__ void __launch_bounds__(ZW_THREADS, 2) k_zw32(ZLArgs A) {
    extern __shared__ __align__(16) float2 zw_smem[];
    __shared__ int s_unit;
    const int lane = threadIdx.x & 31;
    const int a0 = blockIdx.x * 32, a = a0 + lane;
    float2 *Ub = zw_smem;
    float *coef = (float *)(Ub + (size_t)(A.nu + 2 * ZW_PAD) * ZL_PITCH);  // [nblk][33], MODE 1 and 2
    if (threadIdx.x == 0) s_unit = 0;
    // the window coefficients (read at every step) in shared memory when they fit
    // (16-byte aligned for the float4 reads; the launch adds 16 bytes of slack).  Offset
    // arithmetic on the shared array, not integer casts, so that the compiler keeps the
    // shared address space and issues shared loads for the table
    float *ca_s = reinterpret_cast<float *>(zw_smem) +
                  ((2 * (size_t)(A.nu + 2 * ZW_PAD) * ZL_PITCH + (size_t)A.nblk * ZL_PITCH + 3) & ~(size_t)3);
    // Every independent global load of the prologue is in flight before any is waited on:
    // the first ZW_CAR float4 per thread of the Ca table, the first ZW_BR values per thread
    // of the 32 atoms' beta rows (one contiguous run; MODE 1 and 2 stage them in the Ca area
    // when it can hold them), then the U tiles.  What exceeds the register batches (larger
    // lmax) is copied by plain loops afterwards.
    const bool staged = (MODE == 1 || MODE == 2) && CA_SMEM && 32 * A.nB <= A.nwca;
    const int nca4 = CA_SMEM ? A.nwca / 4 : 0;
    const float4 *csrc = reinterpret_cast<const float4 *>(A.wca);
    float4 cr[ZW_CAR];
#pragma unroll
    for (int r = 0; r < ZW_CAR; ++r) {
        const int i = threadIdx.x + r * ZW_THREADS;
        cr[r] = (i < nca4) ? __ldg(csrc + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const int nbt = staged ? min(32, A.natoms - a0) * A.nB : 0;
    const float *bsrc = A.beta + (size_t)a0 * A.nB;
    float br[ZW_BR];
#pragma unroll
    for (int r = 0; r < ZW_BR; ++r) {
        const int i = threadIdx.x + r * ZW_THREADS;
        br[r] = (i < nbt) ? __ldg(bsrc + i) : 0.f;
    }
    pdl_wait();  // U_tot (and, in the JVP, dU) come from the kernel before
    zw_load_utot(A.utot, A.hfull, a0, A.natoms, A.nh, A.nu, Ub);
    if (MODE == 1 || MODE == 2) {
        // coef[b][lane] = sum over the block's roles of role_f beta[atom][role_k], from the
        // staged rows, else from global memory
        if (staged) {
#pragma unroll
            for (int r = 0; r < ZW_BR; ++r) {
                const int i = threadIdx.x + r * ZW_THREADS;
                if (i < 32 * A.nB) ca_s[i] = br[r];
            }
            for (int i = threadIdx.x + ZW_BR * ZW_THREADS; i < 32 * A.nB; i += ZW_THREADS)
                ca_s[i] = (i < nbt) ? __ldg(bsrc + i) : 0.f;
            __syncthreads();
        }
        // one block per warp and step (its table entry is the same for all lanes), lane = atom;
        // the packed role table (missing roles: factor 0 on a present component) takes two
        // independent loads per block instead of a chain of dependent reads of the block record
#pragma unroll 4
        for (int b = threadIdx.x >> 5; b < A.nblk; b += ZW_THREADS / 32) {
            const int4 rk = __ldg(A.blk_rk + b);
            const float4 rf = __ldg(A.blk_rf + b);
            float c = 0.f;
            if (a < A.natoms) {
                if (staged) {
                    const float *bl = ca_s + lane * A.nB;
                    c = fmaf(rf.x, bl[rk.x], c);
                    c = fmaf(rf.y, bl[rk.y], c);
                    c = fmaf(rf.z, bl[rk.z], c);
                } else {
                    const float *bl = A.beta + (size_t)a * A.nB;
                    c = fmaf(rf.x, __ldg(bl + rk.x), c);
                    c = fmaf(rf.y, __ldg(bl + rk.y), c);
                    c = fmaf(rf.z, __ldg(bl + rk.z), c);
                }
            }
            coef[b * ZL_PITCH + lane] = c;
        }
        if (staged) __syncthreads();  // before the Ca copy overwrites the staged beta
    }
    if (CA_SMEM) {
        float4 *dst = reinterpret_cast<float4 *>(ca_s);
#pragma unroll
        for (int r = 0; r < ZW_CAR; ++r) {
            const int i = threadIdx.x + r * ZW_THREADS;
            if (i < nca4) dst[i] = cr[r];
        }
        for (int i = threadIdx.x + ZW_CAR * ZW_THREADS; i < nca4; i += ZW_THREADS) dst[i] = __ldg(csrc + i);
    }
    const float *ca = CA_SMEM ? ca_s : A.wca;
    __syncthreads();
    const float2 *Ul = Ub + lane;
    for (int u = zl_next(&s_unit); u < A.nunit; u = zl_next(&s_unit)) {
        const int4 un = __ldg(A.unit + u);
        zw_unit_k<MODE>(un.x >> 24, A, un, Ul, coef, ca, a, lane);
    }
    pdl_trigger();  // the next kernel may start its set-up during the slot sums
    if (MODE == 1) return;
    __syncthreads();
    // the sums of the slots, staged in shared memory over the U tiles (no longer read) when
    // they fit there (the host sizes the launch so), in the fixed slot order
    float *stage = (float *)zw_smem;
    if (MODE == 3) {
        // dB_k: the sum of component k's slots (sections 0, 1, 2, each in unit order), staged a
        // chunk of components at a time over the U tiles, so the JVP mode needs no more shared
        // memory than the others
        zw_slot_sums_chunked(A.bc, A.jpos, A.nB, A.natoms, a0, stage, A.stage_cap,
                             [&](int k, int l, float acc) { A.x[(size_t)(a0 + l) * A.nB + k] = acc; });
        return;
    }
    // B_k = 2 x the sum of its slots; in the fused pass also beta_k B_k per atom (beta read
    // ahead with the slots), kept in shared memory after the staged slots for the energy
    float *eb = stage + (size_t)A.nbsec * ZL_PITCH;  // [nB][33]
    zw_slot_sums<ZW_BR>(
        A.bc, A.bpos, A.nB, A.nbsec, A.natoms, a0, stage,
        [&](int k, int l) { return (MODE == 2) ? __ldg(A.beta + (size_t)(a0 + l) * A.nB + k) : 0.f; },
        [&](int k, int l, float acc, float bk) {
            acc *= 2.f;
            A.x[(size_t)(a0 + l) * A.nB + k] = acc;
            if (MODE == 2) eb[k * ZL_PITCH + l] = acc * bk;
        });
    if (MODE != 2 || A.eatom == nullptr) return;
    __syncthreads();
    if (threadIdx.x < 32 && a < A.natoms) {
        float e = 0.f;
        for (int k = 0; k < A.nB; ++k) e += eb[k * ZL_PITCH + threadIdx.x];
        A.eatom[a] = e;
    }
}


// zw_unit with two atoms per lane (so4_zwin2.cuh): the lane's atoms are a = a0 + lane
// and a + 32; every per-atom quantity is a pair (atom a, atom a + 32).
template <int MODE, int K>
__device__ __forceinline__ void zw2_unit(const ZLArgs &A, const int4 un, const float4 *Ul, const float2 *coef,
                                         const float *__restrict__ ca, int a, int lane) {
    const int lam = un.x & 0xff, mb = (un.x >> 8) & 0xff, ma0 = (un.x >> 16) & 0xff;
    const int off0 = mb * (lam + 1) + ma0;
    const int cnt = section_count(lam);
    const int b = a + 32;
    float2 yr[K], yi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) yr[k] = yi[k] = make_float2(0.f, 0.f);
    // MODE 3: w_e dU[e] of the unit's entries for both atoms (0 past the section's end)
    float2 dr[K], di[K];
    if (MODE == 3) {
        const size_t hb = A.st.h_block[lam] + off0;
        const float2 *dp = A.dU + (size_t)min(a, A.natoms - 1) * A.nh + hb;
        const float2 *dq = A.dU + (size_t)min(b, A.natoms - 1) * A.nh + hb;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int off = off0 + k;
            float2 d = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
            if (off < cnt) {
                d = __ldg(dp + k);
                e = __ldg(dq + k);
            }
            const float w = ((lam & 1) == 0 && off == cnt - 1) ? 0.5f : 1.f;
            dr[k] = make_float2(w * d.x, w * e.x);
            di[k] = make_float2(w * d.y, w * e.y);
        }
    }
    int4 sgn = (un.y < un.z) ? __ldg(A.seg + un.y) : make_int4(0, 0, 0, -1);
    for (int q = un.y; q < un.z; ++q) {
        const int4 sg = sgn;
        if (q + 1 < un.z) sgn = __ldg(A.seg + q + 1);
        float2 zr[K], zi[K];
#pragma unroll
        for (int k = 0; k < K; ++k) zr[k] = zi[k] = make_float2(0.f, 0.f);
        int r = sg.x;
        int4 h1 = (r < sg.y) ? __ldg(A.wsub + r) : make_int4(0, 0, 0, 0);
        if (K <= ZW_KPAIR) {
            int4 h2 = (r + 1 < sg.y) ? __ldg(A.wsub + r + 1) : make_int4(0, 0, 0, 0);
            for (; r + 1 < sg.y; r += 2) {
                const int4 c1 = h1, c2 = h2;
                if (r + 2 < sg.y) h1 = __ldg(A.wsub + r + 2);
                if (r + 3 < sg.y) h2 = __ldg(A.wsub + r + 3);
                zw2_rows2<K>(Ul, c1, c2, ca, zr, zi);
            }
            if (r < sg.y) zw2_rows<K>(Ul, h1, ca, zr, zi);
        } else {
            for (; r < sg.y; ++r) {
                const int4 hd = h1;
                if (r + 1 < sg.y) h1 = __ldg(A.wsub + r + 1);
                zw2_rows<K>(Ul, hd, ca, zr, zi);
            }
        }
        if (MODE == 3) {
            float2 v = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < K; ++k) v = __ffma2_rn(dr[k], zr[k], __ffma2_rn(di[k], zi[k], v));
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const int jb = __ldg(A.jbase + 3 * sg.z + t);
                if (jb < 0) break;
                const float f = __ldg(A.jfac + 3 * sg.z + t);
                float *row = A.bc + (size_t)(jb + sg.w) * A.natoms;
                if (a < A.natoms) row[a] = f * v.x;
                if (b < A.natoms) row[b] = f * v.y;
            }
        }
        if (MODE == 1 || MODE == 2) {
            const float2 c = coef[sg.z * ZL_PITCH + lane];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                yr[k] = __ffma2_rn(c, zr[k], yr[k]);
                yi[k] = __ffma2_rn(c, zi[k], yi[k]);
            }
        }
        if ((MODE == 0 || MODE == 2) && sg.w >= 0) {
            const float4 *ul = Ul + (ZW_PAD + A.st.u_block[lam] + off0) * ZL_PITCH;
            float v = 0.f, w = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int off = off0 + k;
                if (off < cnt) {
                    const float4 uv = ul[k * ZL_PITCH];
                    const float d = __fmaf_rn(uv.z, zi[k].x, __fmul_rn(uv.x, zr[k].x));
                    const float e = __fmaf_rn(uv.w, zi[k].y, __fmul_rn(uv.y, zr[k].y));
                    const bool half = (lam & 1) == 0 && off == cnt - 1;
                    v += half ? 0.5f * d : d;
                    w += half ? 0.5f * e : e;
                }
            }
            float *row = A.bc + (size_t)sg.w * A.natoms;
            if (a < A.natoms) row[a] = v;
            if (b < A.natoms) row[b] = w;
        }
    }
    if (MODE == 1 || MODE == 2) {
        const float un_l = __int_as_float(un.w);
        const size_t hb = A.st.h_block[lam] + off0;
        const float *ys = A.yscale + hb;
        float2 *Ya = A.Y + (size_t)a * A.nh + hb;
        float2 *Yb = A.Y + (size_t)b * A.nh + hb;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int ma = ma0 + k;
            const float wmid = (2 * mb < lam) ? 1.f : ((2 * ma < lam) ? 1.f : ((2 * ma == lam) ? 0.5f : 0.f));
            const float s = un_l * wmid * __ldg(ys + k);
            if (a < A.natoms) Ya[k] = make_float2(s * yr[k].x, s * yi[k].x);
            if (b < A.natoms) Yb[k] = make_float2(s * yr[k].y, s * yi[k].y);
        }
        if (2 * mb == lam && ma0 + K - 1 == lam / 2) {  // the zero upper half of the middle row
            for (int ma = lam / 2 + 1; ma <= lam; ++ma) {
                if (a < A.natoms) Ya[ma - ma0] = make_float2(0.f, 0.f);
                if (b < A.natoms) Yb[ma - ma0] = make_float2(0.f, 0.f);
            }
        }
    }
}

template <int MODE, int K = ZW_KMAX>
__device__ __forceinline__ void zw2_unit_k(int k, const ZLArgs &A, const int4 un, const float4 *Ul,
                                           const float2 *coef, const float *__restrict__ ca, int a, int lane) {
    if constexpr (K > 1) {
        if (k != K) {
            zw2_unit_k<MODE, K - 1>(k, A, un, Ul, coef, ca, a, lane);
            return;
        }
    }
    zw2_unit<MODE, K>(A, un, Ul, coef, ca, a, lane);
}

// k_zw32 with two atoms per lane: 64 atoms per CTA of NT threads, one CTA per SM (the
// two-atom U tiles of twol 8 take 155 KB).  The same work lists, modes and outputs.
template <int MODE, bool CA_SMEM, int NT>
__global__ void __launch_bounds__(NT, 1) k_zw64(ZLArgs A) {
    extern __shared__ __align__(16) float4 zw2_smem[];
    __shared__ int s_unit;
    const int lane = threadIdx.x & 31;
    const int a0 = blockIdx.x * ZW2_ATOMS, a = a0 + lane;
    float4 *Uq = zw2_smem;
    const size_t ntile = (size_t)(A.nu + 2 * ZW_PAD) * ZL_PITCH;  // float4
    float2 *coef = reinterpret_cast<float2 *>(zw2_smem + ntile);  // [nblk][33] pairs, MODE 1 and 2
    if (threadIdx.x == 0) s_unit = 0;
    float *ca_s = reinterpret_cast<float *>(zw2_smem) + ((4 * ntile + 2 * (size_t)A.nblk * ZL_PITCH + 3) & ~(size_t)3);
    const bool staged = (MODE == 1 || MODE == 2) && CA_SMEM && ZW2_ATOMS * A.nB <= A.nwca;
    const int nca4 = CA_SMEM ? A.nwca / 4 : 0;
    const float4 *csrc = reinterpret_cast<const float4 *>(A.wca);
    float4 cr[ZW_CAR];
#pragma unroll
    for (int r = 0; r < ZW_CAR; ++r) {
        const int i = threadIdx.x + r * NT;
        cr[r] = (i < nca4) ? __ldg(csrc + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const int nbt = staged ? min(ZW2_ATOMS, A.natoms - a0) * A.nB : 0;
    const float *bsrc = A.beta + (size_t)a0 * A.nB;
    float br[ZW_BR];
#pragma unroll
    for (int r = 0; r < ZW_BR; ++r) {
        const int i = threadIdx.x + r * NT;
        br[r] = (i < nbt) ? __ldg(bsrc + i) : 0.f;
    }
    pdl_wait();
    zw2_load_utot<NT>(A.utot, A.hfull, a0, A.natoms, A.nh, A.nu, Uq);
    if (MODE == 1 || MODE == 2) {
        if (staged) {
#pragma unroll
            for (int r = 0; r < ZW_BR; ++r) {
                const int i = threadIdx.x + r * NT;
                if (i < ZW2_ATOMS * A.nB) ca_s[i] = br[r];
            }
            for (int i = threadIdx.x + ZW_BR * NT; i < ZW2_ATOMS * A.nB; i += NT)
                ca_s[i] = (i < nbt) ? __ldg(bsrc + i) : 0.f;
            __syncthreads();
        }
        // coef[b][lane] = (c of atom a, c of atom a + 32), c = sum over the block's roles
        // of role_f beta[atom][role_k], in the order of k_zw32
#pragma unroll 4
        for (int bk = threadIdx.x >> 5; bk < A.nblk; bk += NT / 32) {
            const int4 rk = __ldg(A.blk_rk + bk);
            const float4 rf = __ldg(A.blk_rf + bk);
            float c[2] = {0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int at = a + 32 * h;
                if (at < A.natoms) {
                    if (staged) {
                        const float *bl = ca_s + (lane + 32 * h) * A.nB;
                        c[h] = fmaf(rf.x, bl[rk.x], c[h]);
                        c[h] = fmaf(rf.y, bl[rk.y], c[h]);
                        c[h] = fmaf(rf.z, bl[rk.z], c[h]);
                    } else {
                        const float *bl = A.beta + (size_t)at * A.nB;
                        c[h] = fmaf(rf.x, __ldg(bl + rk.x), c[h]);
                        c[h] = fmaf(rf.y, __ldg(bl + rk.y), c[h]);
                        c[h] = fmaf(rf.z, __ldg(bl + rk.z), c[h]);
                    }
                }
            }
            coef[bk * ZL_PITCH + lane] = make_float2(c[0], c[1]);
        }
        if (staged) __syncthreads();
    }
    if (CA_SMEM) {
        float4 *dst = reinterpret_cast<float4 *>(ca_s);
#pragma unroll
        for (int r = 0; r < ZW_CAR; ++r) {
            const int i = threadIdx.x + r * NT;
            if (i < nca4) dst[i] = cr[r];
        }
        for (int i = threadIdx.x + ZW_CAR * NT; i < nca4; i += NT) dst[i] = __ldg(csrc + i);
    }
    const float *ca = CA_SMEM ? ca_s : A.wca;
    __syncthreads();
    const float4 *Ul = Uq + lane;
    for (int u = zl_next(&s_unit); u < A.nunit; u = zl_next(&s_unit)) {
        const int4 un = __ldg(A.unit + u);
        zw2_unit_k<MODE>(un.x >> 24, A, un, Ul, coef, ca, a, lane);
    }
    pdl_trigger();
    if (MODE == 1) return;
    __syncthreads();
    float *stage = reinterpret_cast<float *>(zw2_smem);
    if (MODE == 3) {
        zw_slot_sums_chunked<ZW2_ATOMS, NT>(
            A.bc, A.jpos, A.nB, A.natoms, a0, stage, A.stage_cap,
            [&](int k, int l, float acc) { A.x[(size_t)(a0 + l) * A.nB + k] = acc; });
        return;
    }
    float *eb = stage + (size_t)A.nbsec * ZW2_SP;  // [nB][65]
    zw_slot_sums<ZW_BR, ZW2_ATOMS, NT>(
        A.bc, A.bpos, A.nB, A.nbsec, A.natoms, a0, stage,
        [&](int k, int l) { return (MODE == 2) ? __ldg(A.beta + (size_t)(a0 + l) * A.nB + k) : 0.f; },
        [&](int k, int l, float acc, float bk) {
            acc *= 2.f;
            A.x[(size_t)(a0 + l) * A.nB + k] = acc;
            if (MODE == 2) eb[k * ZW2_SP + l] = acc * bk;
        });
    if (MODE != 2 || A.eatom == nullptr) return;
    __syncthreads();
    if (threadIdx.x < ZW2_ATOMS && a0 + (int)threadIdx.x < A.natoms) {
        float e = 0.f;
        for (int k = 0; k < A.nB; ++k) e += eb[k * ZW2_SP + threadIdx.x];
        A.eatom[a0 + threadIdx.x] = e;
    }
}

struct DArgs {
    so4_params prm;
    float psi_fac, rc32;  // rfac0 pi / rcut and rcut in FP32, set on the host
    int natoms, nh;
    const double *w_nb, *img_r;
    const int32_t *img_ptr, *img_j;
    const float *rootpq;
    SmallTables st;
    const float2 *Y;
    const float *yscale;  // n_half: the row scale F by which the window kernels stored Y
    float *g;
};

// One CTA per centre, warps over its images: U and dU by the recursion, then
// dE/dr_image = w_j (sfac Re sum conj(dU) Y + dsfac r^ Re sum conj(U) Y).  The recursion
// gives U itself, not the scaled rows the row-chain kernels contract, so Y is taken back
// from its stored form (times the row scale F) to Y / F.
__global__ void __launch_bounds__(NWD * 32) k_deidrj(DArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ SmallTables st;
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
    for (int e = tid; e < nh; e += NWD * 32) {
        const float f = __ldg(A.yscale + e);
        Ys[e] = mk<float>(Yg[e].x / f, Yg[e].y / f);
    }
    __syncthreads();
    const float rc = (float)A.prm.rcut;
    const float psi_fac = (float)(A.prm.rfac0 * SO4_PI / A.prm.rcut);
    const int m0 = A.img_ptr[a], m1 = A.img_ptr[a + 1];
    for (int m = m0 + wid; m < m1; m += NWD) {
        const float x = (float)A.img_r[3 * m], y = (float)A.img_r[3 * m + 1], z = (float)A.img_r[3 * m + 2];
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
        __syncwarp();
    }
}

// Per-image dE/dr in reverse mode (RvFwd / RvBack, so4_rowchain.cuh).  Images are
// flattened over all centres (load balance independent of the per-atom count):
// warp w takes images [w*IPW, (w+1)*IPW), lane = image_in_warp * NCH + chain mb.
// U rows are kept in shared memory by the forward sweep; one backward sweep of Y
// gives the gradients with respect to conj(a), conj(b).
template <int TWOL, int NT>
__global__ void __launch_bounds__(NT, (TWOL <= 8) ? 512 / NT : 1) k_deidrj_rev(DArgs A, int64_t nimg) {
    using RC = RowChain<TWOL>;
    constexpr int W = TWOL + 1;
    constexpr int NIT = 32 / RC::IPW, PASS = NIT * RC::IPW;  // images per warp: one per lane
    extern __shared__ __align__(16) float2 rv_smem[];  // [acc_block(TWOL + 1)][NT]
    float2 *st = rv_smem + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    pdl_wait();  // Y comes from the kernel before
    const int grp = lane / RC::NCH, mb = lane - grp * RC::NCH;
    // the images are [img_ptr[0], img_ptr[natoms]) (img_ptr may point into a longer list
    // for a range of centres); nimg bounds their count (a capacity will do).  Warps past
    // the end leave at once (uniform over the warp; there is no block barrier)
    const int64_t mbase = __ldg(A.img_ptr);
    const int64_t mtot = min(nimg, (int64_t)__ldg(A.img_ptr + A.natoms) - mbase);
    const int64_t p0 = wg * PASS;  // this warp's first image, relative to mbase
    if (p0 >= mtot) return;
    // one pass over the warp's images, one per lane: vector, weight, centre, the Cayley-Klein
    // parameters with their derivatives and the cutoff; the recursion iterations below take
    // their images' parameters by shuffles and hand the sums back to the owning lane
    const int64_t mo = mbase + p0 + lane;
    const bool own = lane < PASS && (p0 + lane < mtot);
    float x = 1.f, y = 0.f, z = 0.f, wj = 0.f;
    int centre = 0;
    if (own) {
        x = (float)A.img_r[3 * mo];
        y = (float)A.img_r[3 * mo + 1];
        z = (float)A.img_r[3 * mo + 2];
        wj = (float)A.w_nb[A.img_j[mo]];
        centre = centre_of(A.img_ptr, A.natoms, (int)mo, (int)mbase, mtot);
    }
    float r = sqrtf(x * x + y * y + z * z);
    const bool skip = !(r >= 1e-8f);  // SO4.py:1441 skips r < 1e-8
    if (skip) {
        x = 1.f;
        y = z = 0.f;
        r = 1.f;
    }
    CK<float> ck0;
    make_ck<float, true>(x, y, z, r, A.psi_fac * r, ck0);
    const int nit = (int)min((int64_t)NIT, (mtot - p0 + RC::IPW - 1) / RC::IPW);
    for (int it = 0; it < nit; ++it) {
        const int src = it * RC::IPW + grp;  // owning lane of this lane's image
        const bool valid = grp < RC::IPW && p0 + src < mtot;
        const int sl = valid ? src : 0;
        CK<float> ck;
        ck.ca.re = __shfl_sync(0xffffffffu, ck0.ca.re, sl);
        ck.ca.im = __shfl_sync(0xffffffffu, ck0.ca.im, sl);
        ck.cb.re = __shfl_sync(0xffffffffu, ck0.cb.re, sl);
        ck.cb.im = __shfl_sync(0xffffffffu, ck0.cb.im, sl);
        const int c_it = __shfl_sync(0xffffffffu, centre, sl);
        if (valid) {
            // the backward sweep reads this centre's Y level by level, one 128-byte line per
            // level: ask for all of its lines now, so the forward sweep hides their latency
            const char *yb = reinterpret_cast<const char *>(A.Y + (size_t)c_it * A.nh);
            const int nlines = (A.nh * (int)sizeof(float2) + 127) / 128;
            for (int l = mb; l < nlines; l += RC::NCH) asm volatile("prefetch.global.L1 [%0];" ::"l"(yb + 128 * l));
        }
        float ur[W], ui[W];
#pragma unroll
        for (int q = 0; q < W; ++q) ur[q] = ui[q] = 0.f;
        ur[0] = 1.f;
        st[0] = make_float2(1.f, 0.f);  // level 0
        RvFwd<TWOL, 1, NT>::run(mb, ck, ur, ui, st);
        // backward sweep (packed pairs), the adjoint carry in g
        float2 g[W];
#pragma unroll
        for (int q = 0; q < W; ++q) g[q] = make_float2(0.f, 0.f);
        const float2 *Y = A.Y + (size_t)c_it * A.nh;
        const float2 z2 = make_float2(0.f, 0.f);
        float2 su2 = z2, sa1 = z2, sa2 = z2, sb1 = z2, sb2 = z2;
        RvBack<TWOL, TWOL, NT>::run(mb, rv_pairs(ck), Y, st, g, su2, sa1, sa2, sb1, sb2);
        const float su = su2.x + su2.y, gar = sa1.x + sa1.y, gai = sa2.x - sa2.y;
        const float gbr = -(sb1.x + sb1.y), gbi = -(sb2.x - sb2.y);
        // sum the chains of each image into its mb == 0 lane
        float tu = su, t0 = gar, t1 = gai, t2 = gbr, t3 = gbi;
#pragma unroll
        for (int k = 1; k < RC::NCH; ++k) {
            tu += __shfl_down_sync(0xffffffffu, su, k);
            t0 += __shfl_down_sync(0xffffffffu, gar, k);
            t1 += __shfl_down_sync(0xffffffffu, gai, k);
            t2 += __shfl_down_sync(0xffffffffu, gbr, k);
            t3 += __shfl_down_sync(0xffffffffu, gbi, k);
        }
        // the owning lanes of this iteration's images take the sums of their mb == 0 lane
        const int ol = lane - it * RC::IPW;
        const bool mine = own && ol >= 0 && ol < RC::IPW;
        const int from = mine ? ol * RC::NCH : 0;
        tu = __shfl_sync(0xffffffffu, tu, from);
        t0 = __shfl_sync(0xffffffffu, t0, from);
        t1 = __shfl_sync(0xffffffffu, t1, from);
        t2 = __shfl_sync(0xffffffffu, t2, from);
        t3 = __shfl_sync(0xffffffffu, t3, from);
        if (mine) {
            float sf, dsf;
            cutoff_fn<float>(A.prm.cutoff_id, r, A.rc32, sf, dsf);
            const float xr[3] = {x / r, y / r, z / r};
            float gv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                // d f / d r_c = Re(conj(G_ca) d conj(a)/dr_c) + Re(conj(G_cb) d conj(b)/dr_c)
                const float sc = t0 * ck0.cda[c].re + t1 * ck0.cda[c].im + t2 * ck0.cdb[c].re + t3 * ck0.cdb[c].im;
                gv[c] = skip ? 0.f : wj * (sf * sc + dsf * xr[c] * tu);
            }
            A.g[3 * mo] = gv[0];
            A.g[3 * mo + 1] = gv[1];
            A.g[3 * mo + 2] = gv[2];
        }
    }
}

// k_deidrj_rev with two lanes per image (so4_rev2.cuh): a warp takes 32 images, one per lane
// for the set-up as above, then two iterations of 16 images, lane = 2 image + role.
template <int TWOL, int NT>
__global__ void __launch_bounds__(NT, (TWOL == 8) ? 3 : 2) k_deidrj_rev2(DArgs A, int64_t nimg) {
    using Y = rev2::Layout<TWOL>;
    constexpr int W = TWOL + 1, NS = Y::NS;
    constexpr int IPI = 16, PASS = 32;  // images per iteration (two lanes each) and per warp
    extern __shared__ __align__(16) float2 rv_smem[];  // [Y::SLOTW][NT]
    float2 *st = rv_smem + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    pdl_wait();  // Y comes from the kernel before
    const int role = lane & 1, pimg = lane >> 1;
    int ch[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) ch[q] = -1;
#pragma unroll
    for (int c = 0; c < Y::NCH; ++c)
        if (rev2::role_of(c) == role) ch[rev2::slot_of(c)] = c;
    const int64_t mbase = __ldg(A.img_ptr);
    const int64_t mtot = min(nimg, (int64_t)__ldg(A.img_ptr + A.natoms) - mbase);
    const int64_t p0 = wg * PASS;  // this warp's first image, relative to mbase
    if (p0 >= mtot) return;
    const int64_t mo = mbase + p0 + lane;
    const bool own = p0 + lane < mtot;
    float x = 1.f, y = 0.f, z = 0.f, wj = 0.f;
    int centre = 0;
    if (own) {
        x = (float)A.img_r[3 * mo];
        y = (float)A.img_r[3 * mo + 1];
        z = (float)A.img_r[3 * mo + 2];
        wj = (float)A.w_nb[A.img_j[mo]];
        centre = centre_of(A.img_ptr, A.natoms, (int)mo, (int)mbase, mtot);
    }
    float r = sqrtf(x * x + y * y + z * z);
    const bool skip = !(r >= 1e-8f);  // SO4.py:1441 skips r < 1e-8
    if (skip) {
        x = 1.f;
        y = z = 0.f;
        r = 1.f;
    }
    CK<float> ck0;
    make_ck<float, true>(x, y, z, r, A.psi_fac * r, ck0);
    const int nit = (int)min((int64_t)(PASS / IPI), (mtot - p0 + IPI - 1) / IPI);
    for (int it = 0; it < nit; ++it) {
        const int src = it * IPI + pimg;  // owning lane of this lane's image
        const bool valid = p0 + src < mtot;
        const int sl = valid ? src : 0;
        CK<float> ck;
        ck.ca.re = __shfl_sync(0xffffffffu, ck0.ca.re, sl);
        ck.ca.im = __shfl_sync(0xffffffffu, ck0.ca.im, sl);
        ck.cb.re = __shfl_sync(0xffffffffu, ck0.cb.re, sl);
        ck.cb.im = __shfl_sync(0xffffffffu, ck0.cb.im, sl);
        const int c_it = __shfl_sync(0xffffffffu, centre, sl);
        if (valid) {
            // the backward sweep reads this centre's Y level by level: ask for its lines now
            const char *yb = reinterpret_cast<const char *>(A.Y + (size_t)c_it * A.nh);
            const int nlines = (A.nh * (int)sizeof(float2) + 127) / 128;
            for (int l = role; l < nlines; l += 2) asm volatile("prefetch.global.L1 [%0];" ::"l"(yb + 128 * l));
        }
        float2 u[NS][W];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int e = 0; e < W; ++e) u[q][e] = make_float2(0.f, 0.f);
        if (role == 0) {
            u[0][0].x = 1.f;  // level 0 of chain 0
            st[Y::idx(0, 0) * NT] = make_float2(1.f, 0.f);
        }
        rev2::Fwd<TWOL, 1, NT>::run(role, ch, ck, u, st);
        float2 g[NS][W];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int e = 0; e < W; ++e) g[q][e] = make_float2(0.f, 0.f);
        const float2 *Yc = A.Y + (size_t)c_it * A.nh;
        const float2 z2 = make_float2(0.f, 0.f);
        float2 su2 = z2, sa1 = z2, sa2 = z2, sb1 = z2, sb2 = z2;
        rev2::Back<TWOL, TWOL, NT>::run(role, ch, rv_pairs(ck), Yc, st, u, g, su2, sa1, sa2, sb1, sb2);
        float tu = su2.x + su2.y, t0 = sa1.x + sa1.y, t1 = sa2.x - sa2.y;
        float t2 = -(sb1.x + sb1.y), t3 = -(sb2.x - sb2.y);
        // the pair's two lanes: both hold the image's sums
        tu += __shfl_xor_sync(0xffffffffu, tu, 1);
        t0 += __shfl_xor_sync(0xffffffffu, t0, 1);
        t1 += __shfl_xor_sync(0xffffffffu, t1, 1);
        t2 += __shfl_xor_sync(0xffffffffu, t2, 1);
        t3 += __shfl_xor_sync(0xffffffffu, t3, 1);
        // the owning lanes of this iteration's images take the sums of their pair
        const int ol = lane - it * IPI;
        const bool mine = own && ol >= 0 && ol < IPI;
        const int from = mine ? 2 * ol : 0;
        tu = __shfl_sync(0xffffffffu, tu, from);
        t0 = __shfl_sync(0xffffffffu, t0, from);
        t1 = __shfl_sync(0xffffffffu, t1, from);
        t2 = __shfl_sync(0xffffffffu, t2, from);
        t3 = __shfl_sync(0xffffffffu, t3, from);
        if (mine) {
            float sf, dsf;
            cutoff_fn<float>(A.prm.cutoff_id, r, A.rc32, sf, dsf);
            const float xr[3] = {x / r, y / r, z / r};
            float gv[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float sc = t0 * ck0.cda[c].re + t1 * ck0.cda[c].im + t2 * ck0.cdb[c].re + t3 * ck0.cdb[c].im;
                gv[c] = skip ? 0.f : wj * (sf * sc + dsf * xr[c] * tu);
            }
            A.g[3 * mo] = gv[0];
            A.g[3 * mo + 1] = gv[1];
            A.g[3 * mo + 2] = gv[2];
        }
    }
}

template <int TWOL, int NT>
int launch_deidrj_rev2(const DArgs &D, int64_t nimg, cudaStream_t st) {
    if (nimg <= 0) return SO4_OK;
    const size_t smem = sizeof(float2) * (size_t)rev2::Layout<TWOL>::SLOTW * NT;
    const int rc = so4_set_smem((const void *)k_deidrj_rev2<TWOL, NT>, smem);
    if (rc) return rc;
    const int64_t warps = (nimg + 31) / 32;
    const int64_t blocks = (warps + NT / 32 - 1) / (NT / 32);
    return so4_launch_pdl(k_deidrj_rev2<TWOL, NT>, dim3((unsigned)blocks), dim3(NT), smem, st, D, nimg);
}

template <int TWOL, int NT>
int launch_deidrj_rev_nt(const DArgs &D, int64_t nimg, cudaStream_t st) {
    using RC = RowChain<TWOL>;
    if (nimg <= 0) return SO4_OK;
    const size_t smem = sizeof(float2) * (size_t)acc_block(TWOL + 1) * NT;
    const int rc = so4_set_smem((const void *)k_deidrj_rev<TWOL, NT>, smem);
    if (rc) return rc;
    constexpr int PASS = (32 / RC::IPW) * RC::IPW;  // images per warp (k_deidrj_rev)
    const int64_t warps = (nimg + PASS - 1) / PASS;
    const int64_t blocks = (warps + NT / 32 - 1) / (NT / 32);
    return so4_launch_pdl(k_deidrj_rev<TWOL, NT>, dim3((unsigned)blocks), dim3(NT), smem, st, D, nimg);
}

// nt: threads per CTA, from the tables' tuning (256 up to twol 8, 128 above; both for twol 6, 8);
// pair: two lanes per image (k_deidrj_rev2, twol 6 and 8: 256 threads at twol 6 with two
// CTAs per SM, 128 at 8 with three) instead of one lane per row chain
template <int TWOL>
int launch_deidrj_rev(const DArgs &D, int64_t nimg, int nt, int pair, cudaStream_t st) {
    if constexpr (TWOL == 6 || TWOL == 8) {
        if (pair) return launch_deidrj_rev2<TWOL, (TWOL == 6) ? 256 : 128>(D, nimg, st);
        if (nt == 128) return launch_deidrj_rev_nt<TWOL, 128>(D, nimg, st);
        return launch_deidrj_rev_nt<TWOL, 256>(D, nimg, st);
    }
    return launch_deidrj_rev_nt<TWOL, (TWOL <= 8) ? 256 : 128>(D, nimg, st);
}


// ---------------------------------------------------------------------------
// Gather: forces, per-structure virial and energy in a fixed order.
//
// Atoms are cut into chunks of GCH consecutive atoms, one CTA per chunk and
// GSUB lanes per atom (lanes over the atom's images).  A chunk belongs to the
// structure of its first atom; the CTA writes forces for all its atoms and the
// chunk's partial sums (9 virial components + energy, FP64) over the atoms of
// that structure only.  The structure pass then adds, for structure s, the
// atoms before its first whole chunk (recomputed from their images) and the
// partials of the chunks that begin inside s.  Every sum has a fixed order, so
// results do not depend on scheduling.
//
// FP64 runs at a small fraction of the FP32 rate on this GPU, so per-atom sums
// are FP32: the force sum sum_m g_m - g_rev(m) is compensated (TwoSum, Knuth),
// which keeps it at FP64 quality despite the cancellation between g_m and
// g_rev(m); the per-atom virial r (x) g is plain FP32 (its error, ~1e-7 of one
// atom's virial, is far below the FP32 error already in g), and everything
// summed across atoms is FP64.
constexpr int GSUB = 8;  // lanes per atom

__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float b) {
    const float s = hi + b;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (b - bb);
    hi = s;
}

// s with atom_ptr[s] <= a < atom_ptr[s + 1] (atom_ptr[0] = 0 <= a < atom_ptr[nstruct])
__device__ __forceinline__ int struct_of(const int *__restrict__ atom_ptr, int nstruct, int a) {
    int lo = 0, hi = nstruct;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(atom_ptr + mid) <= a)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// The GSUB-lane group of the calling lane sums over the images m of atom a
// (a < 0: nothing) g_m - g_rev(m) (FORCES; fh + fl) and r_m (x) g_m (v).  Every
// lane of the warp must call it (the group reduction shuffles).
template <bool FORCES>
__device__ __forceinline__ void group_atom_fv(int a, const int32_t *__restrict__ img_ptr,
                                              const int32_t *__restrict__ img_rev, const double *__restrict__ img_r,
                                              const float *__restrict__ g, float (&fh)[3], float (&fl)[3],
                                              float (&v)[9]) {
#pragma unroll
    for (int q = 0; q < 3; ++q) fh[q] = fl[q] = 0.f;
#pragma unroll
    for (int q = 0; q < 9; ++q) v[q] = 0.f;
    if (a >= 0) {
        const int m1 = __ldg(img_ptr + a + 1);
        for (int m = __ldg(img_ptr + a) + (int)(threadIdx.x & (GSUB - 1)); m < m1; m += GSUB) {
            const float gm[3] = {__ldg(g + 3 * (size_t)m), __ldg(g + 3 * (size_t)m + 1), __ldg(g + 3 * (size_t)m + 2)};
            const float rm[3] = {(float)__ldg(img_r + 3 * (size_t)m), (float)__ldg(img_r + 3 * (size_t)m + 1),
                                 (float)__ldg(img_r + 3 * (size_t)m + 2)};
            if (FORCES) {
                const size_t rv = (size_t)__ldg(img_rev + m);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    two_sum_add(fh[q], fl[q], gm[q]);
                    two_sum_add(fh[q], fl[q], -__ldg(g + 3 * rv + q));
                }
            }
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q) v[3 * p + q] = fmaf(rm[p], gm[q], v[3 * p + q]);
        }
    }
#pragma unroll
    for (int d = GSUB / 2; d > 0; d >>= 1) {
        if (FORCES) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float oh = __shfl_xor_sync(0xffffffffu, fh[q], d);
                const float ol = __shfl_xor_sync(0xffffffffu, fl[q], d);
                two_sum_add(fh[q], fl[q], oh);
                fl[q] += ol;
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], d);
    }
}

__global__ void __launch_bounds__(GCH * GSUB) k_gather_fv(int natoms, int nstruct, const int *__restrict__ atom_ptr,
                                                         const int32_t *__restrict__ img_ptr,
                                                         const int32_t *__restrict__ img_rev,
                                                         const double *__restrict__ img_r,
                                                         const float *__restrict__ g, const float *__restrict__ eatom,
                                                         double *__restrict__ part, double *__restrict__ forces) {
    __shared__ float vs[GCH][GPART];
    __shared__ int s_end;
    const int c = blockIdx.x;
    const int slot = threadIdx.x / GSUB;  // atom of the chunk
    const int a = c * GCH + slot;
    if (threadIdx.x == 0) s_end = __ldg(atom_ptr + struct_of(atom_ptr, nstruct, c * GCH) + 1);
    float fh[3], fl[3], v[9];
    group_atom_fv<true>(a < natoms ? a : -1, img_ptr, img_rev, img_r, g, fh, fl, v);
    if ((threadIdx.x & (GSUB - 1)) == 0) {
        if (a < natoms) {
#pragma unroll
            for (int q = 0; q < 3; ++q) forces[3 * (size_t)a + q] = (double)fh[q] + (double)fl[q];
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) vs[slot][q] = v[q];
        vs[slot][9] = (eatom && a < natoms) ? __ldg(eatom + a) : 0.f;
    }
    __syncthreads();
    if (threadIdx.x < GPART) {
        const int lim = min(natoms, s_end) - c * GCH;  // atoms of the chunk in its first structure
        double p = 0.0;
        for (int k = 0; k < GCH && k < lim; ++k) p += (double)vs[k][threadIdx.x];
        part[(size_t)GPART * c + threadIdx.x] = p;
    }
}

// One CTA per structure: virial[s] (9) and energy[s] from the head atoms and the chunk partials.
constexpr int GSS = GCH * GSUB;  // threads of the structure pass: one group per possible head atom
__global__ void __launch_bounds__(GSS) k_struct_sum(const int *__restrict__ atom_ptr,
                                                   const int32_t *__restrict__ img_ptr,
                                                   const int32_t *__restrict__ img_rev,
                                                   const double *__restrict__ img_r, const float *__restrict__ g,
                                                   const float *__restrict__ eatom, const double *__restrict__ part,
                                                   double *__restrict__ virial, double *__restrict__ energy) {
    constexpr int NSLOT = GSS / GPART;
    __shared__ float hv[GCH][GPART];
    __shared__ double red[NSLOT][GPART];
    const int s = blockIdx.x, t = threadIdx.x;
    const int a0 = __ldg(atom_ptr + s), a1 = __ldg(atom_ptr + s + 1);
    const int c0 = (a0 + GCH - 1) / GCH;                       // first chunk starting inside s
    const int h1 = min(a1, c0 * GCH);                          // head atoms [a0, h1), fewer than GCH
    const int c1 = (a1 > c0 * GCH) ? (a1 - 1) / GCH : c0 - 1;  // last chunk starting inside s
    {
        const int k = t / GSUB, a = a0 + k;
        float fh[3], fl[3], v[9];
        group_atom_fv<false>(a < h1 ? a : -1, img_ptr, img_rev, img_r, g, fh, fl, v);
        if ((t & (GSUB - 1)) == 0) {
#pragma unroll
            for (int q = 0; q < 9; ++q) hv[k][q] = v[q];
            hv[k][9] = (eatom && a < h1) ? __ldg(eatom + a) : 0.f;
        }
    }
    // chunk partials: thread t < NSLOT * GPART adds component q of chunks c0 + slot, c0 + slot + NSLOT, ...
    const int q = t % GPART, slot = t / GPART;
    if (slot < NSLOT) {
        double acc = 0.0;
        for (int c = c0 + slot; c <= c1; c += NSLOT) acc += __ldg(part + (size_t)GPART * c + q);
        red[slot][q] = acc;
    }
    __syncthreads();
    if (t < GPART) {
        double tot = 0.0;
        for (int k = 0; k < GCH; ++k) tot += (double)hv[k][t];
        for (int k = 0; k < NSLOT; ++k) tot += red[k][t];
        if (t < 9)
            virial[9 * (size_t)s + t] = tot;
        else if (energy)
            energy[s] = tot;
    }
}

size_t rootpq_floats(int ldim) { return (size_t)((ldim * ldim + 1) & ~1); }

}  // namespace

static ZLArgs zl_args(const so4_tables *t, int natoms) {
    ZLArgs Z{};
    Z.natoms = natoms;
    Z.nh = t->n_half;
    Z.nu = t->n_u;
    Z.nB = t->n_b;
    Z.nblk = t->n_blk;
    Z.hfull = t->d_hfull;
    Z.bent = t->d_b;
    Z.blk = t->d_blk;
    Z.blk_rk = t->d_blk_rk;
    Z.blk_rf = t->d_blk_rf;
    Z.yptr = t->d_yblk_ptr;
    Z.ylist = t->d_yblk;
    Z.wsub = t->d_wsub;
    Z.wca = t->d_wca;
    Z.nwca = t->n_wca;
    Z.yscale = t->d_yscale;
    fill_small_tables(t, Z.st);
    return Z;
}

// shared memory of k_zw32 (without the Ca table): padded U tiles and the per-block
// coefficients; the epilogue stages nslot slot rows (and, in the fused pass, beta B) over
// the U tiles.  k_zw64: the two-atom tiles (a float4 per entry and lane), coefficient
// pairs, stage rows of 65 floats.
static size_t zw_smem_bytes(const so4_tables *t, int nslot, bool with_eb) {
    const size_t rows = (size_t)(t->n_u + 2 * ZW_PAD) * ZL_PITCH, nst = nslot + (with_eb ? t->n_b : 0);
    if (t->tune.zw_atoms == ZW2_ATOMS)
        return std::max(sizeof(float4) * rows, sizeof(float) * nst * ZW2_SP) + sizeof(float2) * (size_t)t->n_blk * ZL_PITCH;
    return std::max(sizeof(float2) * rows, sizeof(float) * nst * ZL_PITCH) + sizeof(float) * (size_t)t->n_blk * ZL_PITCH;
}

// Slot rows the JVP epilogue stages at a time: those that fit over the padded U tiles.
static int zw_stage_cap(const so4_tables *t) {
    const size_t rows = (size_t)(t->n_u + 2 * ZW_PAD) * ZL_PITCH;
    return (t->tune.zw_atoms == ZW2_ATOMS) ? (int)(4 * rows / ZW2_SP) : (int)(2 * rows / ZL_PITCH);
}

// Dynamic shared memory the window kernels need in each mode (without the Ca table, which
// they drop when it does not fit): B only, Y only, B + Y, JVP.  The check of a tuned
// table's work lists.
void so4_zw_smem_modes(const so4_tables *t, size_t out[4]) {
    out[0] = zw_smem_bytes(t, t->n_bsec, false);
    out[1] = zw_smem_bytes(t, 0, false);
    out[2] = zw_smem_bytes(t, t->n_bsec, true);
    out[3] = zw_smem_bytes(t, 0, false);  // the JVP stages its slots in chunks over the U tiles
}

// k_zw64 with NT threads, the Ca table in shared memory when the one CTA per SM still
// fits with it
template <int MODE, int NT>
static int launch_zw64(const so4_tables *t, const ZLArgs &Z, int natoms, size_t smz, cudaStream_t st) {
    const size_t with_ca = smz + 16 + sizeof(float) * (size_t)t->n_wca;
    const int groups = (natoms + ZW2_ATOMS - 1) / ZW2_ATOMS;
    int rc;
    if (with_ca <= 227 * 1024) {
        rc = set_smem(k_zw64<MODE, true, NT>, with_ca);
        if (rc) return rc;
        return so4_launch_pdl(k_zw64<MODE, true, NT>, dim3(groups), dim3(NT), with_ca, st, Z);
    }
    rc = set_smem(k_zw64<MODE, false, NT>, smz);
    if (rc) return rc;
    return so4_launch_pdl(k_zw64<MODE, false, NT>, dim3(groups), dim3(NT), smz, st, Z);
}

// Launch the window kernel of the tables' layout: k_zw64 (two atoms per lane) or k_zw32
// with the Ca table in shared memory when two CTAs per SM still fit.  nslot: the slot
// rows its epilogue stages; with_eb: and beta B.
template <int MODE>
static int launch_zw(const so4_tables *t, const ZLArgs &Z, int natoms, int nslot, bool with_eb, cudaStream_t st) {
    const size_t smz = zw_smem_bytes(t, nslot, with_eb);
    if (t->tune.zw_atoms == ZW2_ATOMS) {
        if (t->tune.zw_threads == 512) return launch_zw64<MODE, 512>(t, Z, natoms, smz, st);
        return launch_zw64<MODE, 256>(t, Z, natoms, smz, st);
    }
    const size_t with_ca = smz + 16 + sizeof(float) * (size_t)t->n_wca;
    const int groups = (natoms + 31) / 32;
    int rc;
    if (2 * (with_ca + 1024) <= 228 * 1024) {
        rc = set_smem(k_zw32<MODE, true>, with_ca);
        if (rc) return rc;
        return so4_launch_pdl(k_zw32<MODE, true>, dim3(groups), dim3(ZW_THREADS), with_ca, st, Z);
    }
    rc = set_smem(k_zw32<MODE, false>, smz);
    if (rc) return rc;
    return so4_launch_pdl(k_zw32<MODE, false>, dim3(groups), dim3(ZW_THREADS), smz, st, Z);
}

extern "C" size_t so4_forward32_workspace_size(const so4_tables *t, int natoms) {
    if (!t || natoms < 0) return 0;
    return ((sizeof(float) * (size_t)(natoms + 1) * t->n_bsec) + 255) & ~(size_t)255;
}

extern "C" int so4_forward32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                             const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
                             const double *d_img_r, float *d_utot, float *d_x, void *d_work, size_t work_bytes,
                             void *stream) {
    if (!t || !p || natoms < 0 || !d_utot || !d_x) return SO4_ERR_ARG;
    if (p->twol != t->twol || !(p->rcut > 0.0) || !(p->rfac0 > 0.0)) return SO4_ERR_ARG;
    if (p->cutoff_id < 1 || p->cutoff_id > 7) return SO4_ERR_UNSUPPORTED;
    if (natoms == 0) return SO4_OK;
    if (!d_work || work_bytes < so4_forward32_workspace_size(t, natoms)) return SO4_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
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
    A.bent = t->d_b;
    fill_small_tables(t, A.st);
    A.hmap = t->d_hmap;
    A.utot = d_utot;
    A.x = d_x;
    A.psi_fac = (float)(p->rfac0 * SO4_PI / p->rcut);
    A.rc32 = (float)p->rcut;
    int rc = SO4_OK;
    switch (t->twol) {
        case 2: rc = launch_utot_rc<2>(A, t->tune.utot_warps, st); break;
        case 3: rc = launch_utot_rc<3>(A, t->tune.utot_warps, st); break;
        case 4: rc = launch_utot_rc<4>(A, t->tune.utot_warps, st); break;
        case 5: rc = launch_utot_rc<5>(A, t->tune.utot_warps, st); break;
        case 6: rc = launch_utot_rc<6>(A, t->tune.utot_warps, st); break;
        case 7: rc = launch_utot_rc<7>(A, t->tune.utot_warps, st); break;
        case 8: rc = launch_utot_rc<8>(A, t->tune.utot_warps, st); break;
        case 9: rc = launch_utot_rc<9>(A, t->tune.utot_warps, st); break;
        case 10: rc = launch_utot_rc<10>(A, t->tune.utot_warps, st); break;
        case 11: rc = launch_utot_rc<11>(A, t->tune.utot_warps, st); break;
        case 12: rc = launch_utot_rc<12>(A, t->tune.utot_warps, st); break;
        default: {
            const size_t smu =
                sizeof(float) * rootpq_floats(t->ldim) + sizeof(cx<float>) * ((size_t)t->n_half * (1 + 2 * NWF));
            rc = set_smem(k_utot32, smu);
            if (rc) return rc;
            k_utot32<<<natoms, NWF * 32, smu, st>>>(A);
            so4_count_launch();
        }
    }
    if (rc) return rc;
    // B by the window kernel (B blocks only), partial sums per (unit, B block) in d_work
    ZLArgs Z = zl_args(t, natoms);
    Z.utot = (const float2 *)d_utot;
    Z.unit = t->d_wunit_b;
    Z.seg = t->d_wseg_b;
    Z.nunit = t->n_wunit_b;
    Z.x = d_x;
    Z.bpos = t->d_bpos;
    Z.nbsec = t->n_bsec;
    Z.bc = (float *)d_work;
    return launch_zw<0>(t, Z, natoms, t->n_bsec, false, st);
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
    ZLArgs Z = zl_args(t, natoms);
    Z.utot = (const float2 *)d_utot;
    Z.unit = t->d_wunit_y;
    Z.seg = t->d_wseg_y;
    Z.nunit = t->n_wunit_y;
    Z.beta = d_beta;
    Z.Y = (float2 *)d_y;
    return launch_zw<1>(t, Z, natoms, 0, false, (cudaStream_t)stream);
}

int so4_zw_jvp32(const so4_tables *t, int natoms, const float *d_utot, const float *d_du, float *d_slots, float *d_dB,
                 cudaStream_t stream) {
    ZLArgs Z = zl_args(t, natoms);
    Z.utot = (const float2 *)d_utot;
    Z.unit = t->d_wunit_j;
    Z.seg = t->d_wseg_j;
    Z.nunit = t->n_wunit_j;
    Z.dU = (const float2 *)d_du;
    Z.jbase = t->d_jbase;
    Z.jpos = t->d_jpos;
    Z.jfac = t->d_jfac;
    Z.bc = d_slots;
    Z.nbsec = t->n_jslot;  // the epilogue's slot count
    Z.stage_cap = zw_stage_cap(t);
    if (t->n_jmax > Z.stage_cap) return SO4_ERR_UNSUPPORTED;  // a component's slots must fit one chunk
    Z.x = d_dB;
    return launch_zw<3>(t, Z, natoms, 0, false, stream);
}

extern "C" int so4_adjoint_deidrj32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                                    const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                                    int64_t nimg, const float *d_y, float *d_g, void *stream) {
    if (!t || !p || natoms < 0 || nimg < 0 || !d_y || !d_g) return SO4_ERR_ARG;
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
    D.psi_fac = (float)(p->rfac0 * SO4_PI / p->rcut);
    D.rc32 = (float)p->rcut;
    D.Y = (const float2 *)d_y;
    D.yscale = t->d_yscale;
    D.g = d_g;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = SO4_OK;
    switch (t->twol) {
        case 2: rc = launch_deidrj_rev<2>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 3: rc = launch_deidrj_rev<3>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 4: rc = launch_deidrj_rev<4>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 5: rc = launch_deidrj_rev<5>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 6: rc = launch_deidrj_rev<6>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 7: rc = launch_deidrj_rev<7>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 8: rc = launch_deidrj_rev<8>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 9: rc = launch_deidrj_rev<9>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 10: rc = launch_deidrj_rev<10>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 11: rc = launch_deidrj_rev<11>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        case 12: rc = launch_deidrj_rev<12>(D, nimg, t->tune.rev_threads, t->tune.rev_pair == 1, st); break;
        default: {
            const size_t smd = sizeof(float) * rootpq_floats(t->ldim) +
                               sizeof(cx<float>) * ((size_t)t->n_half + (size_t)NWD * 4 * t->n_half);
            rc = set_smem(k_deidrj, smd);
            if (rc) return rc;
            k_deidrj<<<natoms, NWD * 32, smd, st>>>(D);
            so4_count_launch();
            return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
        }
    }
    if (rc) return rc;
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" size_t so4_gather_workspace_size(int natoms) {
    return natoms < 0 ? 0 : sizeof(double) * gather_part_doubles(natoms);
}

extern "C" int so4_adjoint_gather(int natoms, int nstruct, const int *d_atom_ptr, const int32_t *d_img_ptr,
                                  const int32_t *d_img_rev, const double *d_img_r, const float *d_g,
                                  const float *d_eatom, double *d_part, double *d_forces, double *d_virial,
                                  double *d_energy, void *stream) {
    if (natoms < 0 || nstruct < 0) return SO4_ERR_ARG;
    if (natoms > 0 && (!d_atom_ptr || !d_img_ptr || !d_img_rev || !d_img_r || !d_g || !d_part || !d_forces))
        return SO4_ERR_ARG;
    if (nstruct > 0 && !d_virial) return SO4_ERR_ARG;
    if (natoms > 0 && nstruct == 0) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (natoms > 0) {
        k_gather_fv<<<(natoms + GCH - 1) / GCH, GCH * GSUB, 0, st>>>(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev,
                                                                   d_img_r, d_g, d_eatom, d_part, d_forces);
        so4_count_launch();
    }
    if (nstruct > 0) {
        k_struct_sum<<<nstruct, GSS, 0, st>>>(d_atom_ptr, d_img_ptr, d_img_rev, d_img_r, d_g, d_eatom, d_part,
                                              d_virial, d_energy);
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
    rc = so4_adjoint_deidrj32(t, p, natoms, d_w_nb, d_img_ptr, d_img_j, d_img_r, nimg, (const float *)w.Y, w.g,
                              stream);
    if (rc) return rc;
    return so4_adjoint_gather(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev, d_img_r, w.g, nullptr, w.part,
                              d_forces, d_virial, nullptr, stream);
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
// that first call should come before any stream capture.  The address is kept
// for the life of the process: after cudaDeviceReset (or any teardown of the
// device's primary context) the module is loaded again at another address, so
// the entry point must not be used across a device reset.
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
    rc = so4_adjoint_deidrj32(t, p, natoms, d_w_nb, d_img_ptr, d_img_j, d_img_r, nimg, (const float *)w.Y, w.g,
                              stream);
    if (rc) return rc;
    return so4_adjoint_gather(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev, d_img_r, w.g, nullptr, w.part,
                              d_forces, d_virial, nullptr, stream);
}

// ---------------------------------------------------------------------------
// Energy linear in B: forward and adjoint with Z computed once.
// linear-path scratch after the adjoint's: U_tot, the B-section rows, the per-atom energy
static size_t carve_linear(const so4_tables *t, void *base, int natoms, int64_t nimg, AdjWork &w, float **utot,
                           float **bc, float **eatom) {
    size_t off = carve_adj(w, base, natoms, t->n_half, nimg);
    char *p = (char *)base;
    *utot = p ? (float *)(p + off) : nullptr;
    off += a256(sizeof(float2) * (size_t)natoms * t->n_half + 8);
    *bc = p ? (float *)(p + off) : nullptr;
    off += a256(sizeof(float) * (size_t)(natoms + 1) * t->n_bsec);
    *eatom = p ? (float *)(p + off) : nullptr;
    off += a256(sizeof(float) * (size_t)(natoms + 1));
    return off;
}

extern "C" size_t so4_linear_workspace_size(const so4_tables *t, int natoms, int64_t nimg) {
    if (!t) return 0;
    AdjWork w;
    float *u, *b, *e;
    return carve_linear(t, nullptr, natoms, nimg, w, &u, &b, &e);
}

extern "C" int so4_utot32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                          const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
                          const double *d_img_r, float *d_utot, void *stream) {
    if (!t || !p || natoms < 0 || !d_utot) return SO4_ERR_ARG;
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
    A.bent = t->d_b;
    fill_small_tables(t, A.st);
    A.hmap = t->d_hmap;
    A.utot = d_utot;
    A.x = nullptr;
    A.psi_fac = (float)(p->rfac0 * SO4_PI / p->rcut);
    A.rc32 = (float)p->rcut;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = SO4_OK;
    switch (t->twol) {
        case 2: rc = launch_utot_rc<2>(A, t->tune.utot_warps, st); break;
        case 3: rc = launch_utot_rc<3>(A, t->tune.utot_warps, st); break;
        case 4: rc = launch_utot_rc<4>(A, t->tune.utot_warps, st); break;
        case 5: rc = launch_utot_rc<5>(A, t->tune.utot_warps, st); break;
        case 6: rc = launch_utot_rc<6>(A, t->tune.utot_warps, st); break;
        case 7: rc = launch_utot_rc<7>(A, t->tune.utot_warps, st); break;
        case 8: rc = launch_utot_rc<8>(A, t->tune.utot_warps, st); break;
        case 9: rc = launch_utot_rc<9>(A, t->tune.utot_warps, st); break;
        case 10: rc = launch_utot_rc<10>(A, t->tune.utot_warps, st); break;
        case 11: rc = launch_utot_rc<11>(A, t->tune.utot_warps, st); break;
        case 12: rc = launch_utot_rc<12>(A, t->tune.utot_warps, st); break;
        default: {
            const size_t smu =
                sizeof(float) * rootpq_floats(t->ldim) + sizeof(cx<float>) * ((size_t)t->n_half * (1 + 2 * NWF));
            rc = set_smem(k_utot32, smu);
            if (rc) return rc;
            k_utot32<<<natoms, NWF * 32, smu, st>>>(A);
            so4_count_launch();
        }
    }
    if (rc) return rc;
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_linear_by32(const so4_tables *t, int natoms, const float *d_utot, const float *d_beta, float *d_x,
                               float *d_y, float *d_bc, float *d_eatom, void *stream) {
    if (!t || natoms < 0 || !d_utot || !d_beta || !d_x || !d_y || !d_bc) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    ZLArgs Z = zl_args(t, natoms);
    Z.utot = (const float2 *)d_utot;
    Z.unit = t->d_wunit_y;
    Z.seg = t->d_wseg_y;
    Z.nunit = t->n_wunit_y;
    Z.beta = d_beta;
    Z.Y = (float2 *)d_y;
    Z.x = d_x;
    Z.bpos = t->d_bpos;
    Z.nbsec = t->n_bsec;
    Z.bc = d_bc;
    Z.eatom = d_eatom;
    return launch_zw<2>(t, Z, natoms, t->n_bsec, true, (cudaStream_t)stream);
}

extern "C" int so4_adjoint_linear32(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                                    const int *d_atom_ptr, int natoms, const double *d_w_nb, const double *d_w_site,
                                    const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                                    const int32_t *d_img_rev, int64_t nimg, const float *d_beta, float *d_x,
                                    double *d_forces, double *d_virial, double *d_energy, void *d_work,
                                    size_t work_bytes, void *stream) {
    (void)d_atom_struct;
    if (!t || !p || natoms < 0 || nstruct < 0 || nimg < 0 || !d_work || !d_x) return SO4_ERR_ARG;
    if (so4_linear_workspace_size(t, natoms, nimg) > work_bytes) return SO4_ERR_WORKSPACE;
    AdjWork w;
    float *utot, *bc, *eatom;
    carve_linear(t, d_work, natoms, nimg, w, &utot, &bc, &eatom);
    int rc = so4_utot32(t, p, natoms, d_w_nb, d_w_site, d_img_ptr, d_img_j, d_img_r, utot, stream);
    if (rc) return rc;
    rc = so4_linear_by32(t, natoms, utot, d_beta, d_x, (float *)w.Y, bc, d_energy ? eatom : nullptr, stream);
    if (rc) return rc;
    rc = so4_adjoint_deidrj32(t, p, natoms, d_w_nb, d_img_ptr, d_img_j, d_img_r, nimg, (const float *)w.Y, w.g,
                              stream);
    if (rc) return rc;
    return so4_adjoint_gather(natoms, nstruct, d_atom_ptr, d_img_ptr, d_img_rev, d_img_r, w.g,
                              d_energy ? eatom : nullptr, w.part, d_forces, d_virial, d_energy, stream);
}
