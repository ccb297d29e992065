// so4_jvp.cu -- the adjoint's backward: the Jacobian-vector product of B.
//
// For a displacement field given per image as dr_m = (v_j - v_i) + G_s^T r_m
// (v: per-atom vectors, G: a per-structure 3x3 matrix), returns
//   dB_i = sum_{images m of i} (dB_i/dr_m) . dr_m
// with dB/dr in the reference's form (compute_dbidrj, pyxtal_ff/descriptors/SO4.py:1113-1227):
//   dB_k = Re [2 S(l; dU, Z(l1,l2,l)) + 2 (l+1)/(l1+1) S(l1; dU, Z(l,l2,l1)) + 2 (l+1)/(l2+1) S(l2; dU, Z(l,l1,l2))]
// where dU is the tangent of U_tot, sum_m u_norm w_j (sfac dU_m . dr_m + dsfac (r^ . dr_m) U_m)
// (dudr, :1001-1018).  With v = -dL/dF and G = dL/dW this is dL/dbeta of the
// adjoint's forces F and virial W, which is how forces enter a training loss.
#include <algorithm>

#include "so4_atom.cuh"
#include "so4_rowchain.cuh"

namespace {

template <typename K>
int set_smem_j(K kern, size_t smem) {
    return so4_set_smem((const void *)kern, smem);
}

struct JArgs {
    int cutoff_id, natoms, nh, nu, nB;
    float psi_fac, rc32;
    const int *astruct;
    const double *w_nb, *img_r, *v, *G;
    const int32_t *img_ptr, *img_j;
    SmallTables st;
    const int4 *hmap;  // per half entry: accumulator slot, row, diagonal flag, u_norm F, u_norm
    float2 *dU;
    float *dB;
};

// tangent of U_tot, one warp per centre (same lanes as k_utot_rc: UtotLanes)
template <int TWOL, int NW>
__global__ void __launch_bounds__(NW * 32, (TWOL <= 4) ? 4 : ((TWOL <= 8) ? 3 : 1)) k_jvp_du_rc(JArgs A) {
    using UL = UtotLanes<TWOL>;
    constexpr int W = TWOL + 1, NACC = acc_block(TWOL + 1);
    extern __shared__ __align__(16) float jv_smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int a = blockIdx.x * NW + wid;
    const int grp = lane / UL::LPI, mb = lane - grp * UL::LPI;
    float2 acc[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) acc[q] = make_float2(0.f, 0.f);
    if (a < A.natoms) {
        const int m0 = A.img_ptr[a], m1 = A.img_ptr[a + 1];
        float vi[3] = {0.f, 0.f, 0.f}, G[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) G[q] = 0.f;
        if (A.v)
            for (int c = 0; c < 3; ++c) vi[c] = (float)A.v[3 * a + c];
        if (A.G) {
            const int s = A.astruct[a];
            for (int q = 0; q < 9; ++q) G[q] = (float)A.G[9 * s + q];
        }
        // per-image setup (vector, weight, tangent, Cayley-Klein parameters and their
        // derivative along the tangent) for up to 32 images at once, one per lane; each
        // recursion iteration takes its IPW images' values by shuffles
        for (int base = m0; base < m1; base += 32) {
            const int m = base + lane;
            float x = 1.f, y = 0.f, z = 0.f, a_du0 = 0.f, a_d0 = 0.f;
            float d[3] = {0.f, 0.f, 0.f};
            if (m < m1) {
                x = (float)A.img_r[3 * m];
                y = (float)A.img_r[3 * m + 1];
                z = (float)A.img_r[3 * m + 2];
                const float rr = sqrtf(x * x + y * y + z * z);
                if (rr >= 1e-8f) {
                    const int j = A.img_j[m];
                    if (A.v)
                        for (int c = 0; c < 3; ++c) d[c] = (float)A.v[3 * j + c] - vi[c];
                    // dr_b += sum_a G_ab r_a
                    d[0] += G[0] * x + G[3] * y + G[6] * z;
                    d[1] += G[1] * x + G[4] * y + G[7] * z;
                    d[2] += G[2] * x + G[5] * y + G[8] * z;
                    float sf, dsf;
                    cutoff_fn<float>(A.cutoff_id, rr, A.rc32, sf, dsf);
                    const float w = (float)A.w_nb[j];
                    a_du0 = w * dsf * (x * d[0] + y * d[1] + z * d[2]) / rr;
                    a_d0 = w * sf;
                } else {
                    x = 1.f;
                    y = z = 0.f;
                }
            }
            CK<float> ck0;
            {
                const float r = sqrtf(x * x + y * y + z * z);
                make_ck<float, true>(x, y, z, r, A.psi_fac * r, ck0);
            }
            // the derivative of conj(a), conj(b) along dr_m
            cx<float> da0 = mk<float>(0.f, 0.f), db0 = mk<float>(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                da0.re += d[c] * ck0.cda[c].re;
                da0.im += d[c] * ck0.cda[c].im;
                db0.re += d[c] * ck0.cdb[c].re;
                db0.im += d[c] * ck0.cdb[c].im;
            }
            const int nimg = min(32, m1 - base);
            for (int sub = 0; sub < nimg; sub += UL::IPW) {
                const int src = sub + grp;
                const bool ok = grp < UL::IPW && src < nimg;
                const int sl = ok ? src : 0;
                CK<float> ck;  // slot 0 of the derivatives holds the one direction
                ck.ca.re = __shfl_sync(0xffffffffu, ck0.ca.re, sl);
                ck.ca.im = __shfl_sync(0xffffffffu, ck0.ca.im, sl);
                ck.cb.re = __shfl_sync(0xffffffffu, ck0.cb.re, sl);
                ck.cb.im = __shfl_sync(0xffffffffu, ck0.cb.im, sl);
                ck.cda[0].re = __shfl_sync(0xffffffffu, da0.re, sl);
                ck.cda[0].im = __shfl_sync(0xffffffffu, da0.im, sl);
                ck.cdb[0].re = __shfl_sync(0xffffffffu, db0.re, sl);
                ck.cdb[0].im = __shfl_sync(0xffffffffu, db0.im, sl);
                float a_du = __shfl_sync(0xffffffffu, a_du0, sl);
                float a_d = __shfl_sync(0xffffffffu, a_d0, sl);
                if (!ok) a_du = a_d = 0.f;
                float2 u[W], du[W];
#pragma unroll
                for (int q = 0; q < W; ++q) u[q] = du[q] = make_float2(0.f, 0.f);
                u[0].x = 1.f;
                if (mb == 0) acc[0].x += a_du;  // level 0: U = 1, dU = 0
                RcJvp2<TWOL, 1>::run(mb, ck, a_du, a_d, u, du, acc);
            }
        }
    }
    float2 *sw = reinterpret_cast<float2 *>(jv_smem) + (size_t)wid * 32 * NACC;
#pragma unroll
    for (int q = 0; q < NACC; ++q) sw[lane * NACC + q] = acc[q];
    __syncwarp();
    if (a >= A.natoms) return;
    float2 *out = A.dU + (size_t)a * A.nh;
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
        const float unf = __int_as_float(h.y);  // u_norm times the row scale
        out[e] = make_float2(sr * unf, si * unf);
    }
}

template <int TWOL>
int launch_jvp_du(const JArgs &A, cudaStream_t st) {
    constexpr int NW = 4;
    const size_t smem = sizeof(float) * NW * 32 * 2 * acc_block(TWOL + 1);
    int rc = set_smem_j(k_jvp_du_rc<TWOL, NW>, smem);
    if (rc) return rc;
    k_jvp_du_rc<TWOL, NW><<<(A.natoms + NW - 1) / NW, NW * 32, smem, st>>>(A);
    so4_count_launch();
    return SO4_OK;
}

size_t a256j(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" size_t so4_jvp_workspace_size(const so4_tables *t, int natoms) {
    if (!t) return 0;
    return a256j(SO4_WS_HEADER) + a256j(sizeof(float2) * (size_t)t->n_half * (natoms + 1)) +
           a256j(sizeof(float) * (size_t)t->n_jslot * (natoms + 1));
}

extern "C" int so4_jvp32(const so4_tables *t, const so4_params *p, const int *d_atom_struct, int natoms,
                         const double *d_w_nb, const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                         const float *d_utot, const double *d_v, const double *d_G, float *d_dB, void *d_work,
                         size_t work_bytes, void *stream) {
    if (!t || !p || natoms < 0 || !d_utot || !d_dB || !d_work) return SO4_ERR_ARG;
    if (p->twol != t->twol || !(p->rcut > 0.0) || !(p->rfac0 > 0.0)) return SO4_ERR_ARG;
    if (p->cutoff_id < 1 || p->cutoff_id > 7) return SO4_ERR_UNSUPPORTED;
    if (d_G && !d_atom_struct) return SO4_ERR_ARG;
    if (so4_jvp_workspace_size(t, natoms) > work_bytes) return SO4_ERR_WORKSPACE;
    if (natoms == 0) return SO4_OK;
    cudaStream_t st = (cudaStream_t)stream;
    JArgs A;
    A.cutoff_id = p->cutoff_id;
    A.natoms = natoms;
    A.nh = t->n_half;
    A.nu = t->n_u;
    A.nB = t->n_b;
    A.psi_fac = (float)(p->rfac0 * SO4_PI / p->rcut);
    A.rc32 = (float)p->rcut;
    A.astruct = d_atom_struct;
    A.w_nb = d_w_nb;
    A.img_r = d_img_r;
    A.v = d_v;
    A.G = d_G;
    A.img_ptr = d_img_ptr;
    A.img_j = d_img_j;
    fill_small_tables(t, A.st);
    A.hmap = t->d_hmap;
    A.dU = (float2 *)((char *)d_work + a256j(SO4_WS_HEADER));
    A.dB = d_dB;
    int rc;
    switch (t->twol) {
        case 2: rc = launch_jvp_du<2>(A, st); break;
        case 3: rc = launch_jvp_du<3>(A, st); break;
        case 4: rc = launch_jvp_du<4>(A, st); break;
        case 5: rc = launch_jvp_du<5>(A, st); break;
        case 6: rc = launch_jvp_du<6>(A, st); break;
        case 7: rc = launch_jvp_du<7>(A, st); break;
        case 8: rc = launch_jvp_du<8>(A, st); break;
        case 9: rc = launch_jvp_du<9>(A, st); break;
        case 10: rc = launch_jvp_du<10>(A, st); break;
        case 11: rc = launch_jvp_du<11>(A, st); break;
        case 12: rc = launch_jvp_du<12>(A, st); break;
        default: return SO4_ERR_UNSUPPORTED;
    }
    if (rc) return rc;
    float *slots = (float *)((char *)d_work + a256j(SO4_WS_HEADER) + a256j(sizeof(float2) * (size_t)t->n_half * (natoms + 1)));
    return so4_zw_jvp32(t, natoms, d_utot, (const float *)A.dU, slots, d_dB, st);
}
