// so4_tables.cu -- FP64 Clebsch-Gordan list, rootpq and index tables (host),
// copied once to the device.  The loops follow the reference:
//   factorial table / deltacg     pyxtal_ff/descriptors/angular_momentum.py:9-190
//   init_clebsch_gordan           pyxtal_ff/descriptors/SO4.py:410-480
//   init_rootpqarray              SO4.py:831-838
//   idxcg/idxu/idxb/idxz tables   SO4.py:1265-1396
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <algorithm>
#include <map>
#include <queue>
#include <tuple>
#include <utility>

#include "so4_common.cuh"

namespace {

// n! as the reference tabulates it: exact up to 20!, rounded to 15 significant
// decimal digits above (angular_momentum.py:14-182).
double factorial_ref(int n) {
    static double tab[40];
    static bool ready = false;
    if (!ready) {
        unsigned __int128 f = 1;
        for (int k = 0; k < 40; ++k) {
            if (k > 0) f *= (unsigned __int128)k;
            if (k <= 20) {
                tab[k] = (double)(uint64_t)f;
            } else if (k <= 34) {
                std::string s;
                unsigned __int128 t = f;
                while (t > 0) {
                    s.insert(s.begin(), (char)('0' + (int)(t % 10)));
                    t /= 10;
                }
                std::string m = s.substr(0, 15);
                bool carry = s[15] >= '5';
                for (int q = 14; q >= 0 && carry; --q) {
                    if (m[q] == '9') {
                        m[q] = '0';
                    } else {
                        m[q]++;
                        carry = false;
                    }
                }
                int e10 = (int)s.size() - 1;
                if (carry) {
                    m = "1" + m.substr(0, 14);
                    e10++;
                }
                std::string sci = m.substr(0, 1) + "." + m.substr(1) + "e" + std::to_string(e10);
                tab[k] = std::strtod(sci.c_str(), nullptr);
            } else {
                tab[k] = NAN;
            }
        }
        ready = true;
    }
    return (n >= 0 && n < 40) ? tab[n] : NAN;
}

double deltacg(int l1, int l2, int l) {
    double s = factorial_ref((l1 + l2 + l) / 2 + 1);
    return std::sqrt(factorial_ref((l1 + l2 - l) / 2) * factorial_ref((l1 - l2 + l) / 2) *
                     factorial_ref((-l1 + l2 + l) / 2) / s);
}

int b3(int ld, int a, int b, int c) { return (a * ld + b) * ld + c; }

template <typename T>
int upload(T **dst, const std::vector<T> &src) {
    size_t bytes = sizeof(T) * (src.empty() ? 1 : src.size());
    if (cudaMalloc((void **)dst, bytes) != cudaSuccess) return SO4_ERR_CUDA;
    if (!src.empty() && cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return SO4_ERR_CUDA;
    return SO4_OK;
}

void free_device(so4_tables *t) {
    cudaFree(t->d_cg64);
    cudaFree(t->d_cg32);
    cudaFree(t->d_rootpq64);
    cudaFree(t->d_rootpq32);
    cudaFree(t->d_z);
    cudaFree(t->d_b);
    cudaFree(t->d_blk);
    cudaFree(t->d_blk_rk);
    cudaFree(t->d_blk_rf);
    cudaFree(t->d_yblk_ptr);
    cudaFree(t->d_yblk);
    cudaFree(t->d_hfull);
    cudaFree(t->d_hmap);
    cudaFree(t->d_yscale);
    cudaFree(t->d_yscale64);
    cudaFree(t->d_psec);
    cudaFree(t->d_psec_ptr);
    cudaFree(t->d_ksec);
    cudaFree(t->d_bpos);
    cudaFree(t->d_wunit_y);
    cudaFree(t->d_wseg_y);
    cudaFree(t->d_wunit_b);
    cudaFree(t->d_wseg_b);
    cudaFree(t->d_wsub);
    cudaFree(t->d_wunit_j);
    cudaFree(t->d_wseg_j);
    cudaFree(t->d_jpos);
    cudaFree(t->d_jbase);
    cudaFree(t->d_jfac);
    cudaFree(t->d_wca);
}

}  // namespace

// Default layout of the per-image pass at twol 6 and 8 (1: two lanes per image).
#define REV_PAIR_DEFAULT 1
// Default atoms per CTA of the window Z pass up to twol 8 (32 or 64), and threads per
// CTA of the 64-atom pass (256 or 512).
#define ZW_ATOMS_DEFAULT 64
#define ZW_THREADS_DEFAULT 512

// The defaults of so4_tuning for one twol, and whether a requested tuning is built.
static so4_tuning tuning_defaults(int twol) {
    so4_tuning d;
    d.wkmax = ZW_KMAX;
    d.rev_threads = (twol <= 8) ? 256 : 128;
    d.utot_warps = 4;
    d.rev_pair = (twol == 6 || twol == 8) ? REV_PAIR_DEFAULT : 2;
    d.zw_atoms = (twol <= 8) ? ZW_ATOMS_DEFAULT : 32;
    d.zw_threads = ZW_THREADS_DEFAULT;
    return d;
}

static int tuning_resolve(int twol, const so4_tuning *req, so4_tuning &out) {
    out = tuning_defaults(twol);
    if (!req) return SO4_OK;
    if (req->wkmax < 0 || req->wkmax > ZW_KMAX || req->rev_threads < 0 || req->utot_warps < 0) return SO4_ERR_ARG;
    if (req->rev_pair < 0 || req->rev_pair > 2 || req->zw_atoms < 0 || req->zw_threads < 0) return SO4_ERR_ARG;
    if (req->rev_threads && req->rev_threads != 128 && req->rev_threads != 256) return SO4_ERR_ARG;
    if (req->utot_warps && req->utot_warps != 2 && req->utot_warps != 4 && req->utot_warps != 8) return SO4_ERR_ARG;
    if (req->wkmax) out.wkmax = req->wkmax;
    const bool shapes = (twol == 6 || twol == 8);  // the twol with every launch shape instantiated
    if (req->rev_threads && req->rev_threads != out.rev_threads) {
        if (!shapes) return SO4_ERR_UNSUPPORTED;
        out.rev_threads = req->rev_threads;
    }
    if (req->utot_warps && req->utot_warps != out.utot_warps) {
        if (!shapes) return SO4_ERR_UNSUPPORTED;
        out.utot_warps = req->utot_warps;
    }
    if (req->rev_pair && req->rev_pair != out.rev_pair) {
        if (!shapes) return SO4_ERR_UNSUPPORTED;
        out.rev_pair = req->rev_pair;
    }
    if (req->zw_atoms && req->zw_atoms != 32 && req->zw_atoms != 64) return SO4_ERR_ARG;
    if (req->zw_threads && req->zw_threads != 256 && req->zw_threads != 512) return SO4_ERR_ARG;
    if (req->zw_atoms) {
        if (req->zw_atoms == 64 && twol > 8) return SO4_ERR_UNSUPPORTED;  // the tiles exceed shared memory
        out.zw_atoms = req->zw_atoms;
    }
    if (req->zw_threads) out.zw_threads = req->zw_threads;
    return SO4_OK;
}

extern "C" int so4_tables_create(int twol, int normalize_u, so4_tables **out) {
    return so4_tables_create_tuned(twol, normalize_u, nullptr, out);
}

extern "C" int so4_tables_get_tuning(const so4_tables *t, so4_tuning *out) {
    if (!t || !out) return SO4_ERR_ARG;
    *out = t->tune;
    return SO4_OK;
}

extern "C" int so4_tables_create_tuned(int twol, int normalize_u, const so4_tuning *tune, so4_tables **out) {
    if (!out) return SO4_ERR_ARG;
    *out = nullptr;
    if (twol < 0) return SO4_ERR_ARG;
    if (twol > SO4_TWOL_MAX) return SO4_ERR_UNSUPPORTED;
    so4_tuning tn;
    const int trc = tuning_resolve(twol, tune, tn);
    if (trc) return trc;
    so4_tables *t = new so4_tables();
    const int ld = twol + 1;
    t->twol = twol;
    t->ldim = ld;
    t->normalize_u = normalize_u ? 1 : 0;
    t->tune = tn;

    // idxcg_block and CG list (SO4.py:1269-1285, 410-480)
    t->idxcg_block.assign(ld * ld * ld, 0);
    int n = 0;
    for (int l1 = 0; l1 < ld; ++l1)
        for (int l2 = 0; l2 <= l1; ++l2)
            for (int l = l1 - l2; l <= std::min(twol, l1 + l2); l += 2) {
                t->idxcg_block[b3(ld, l1, l2, l)] = n;
                n += (l1 + 1) * (l2 + 1);
            }
    t->n_cg = n;
    t->cglist.assign(n, 0.0);
    n = 0;
    for (int l1 = 0; l1 < ld; ++l1)
        for (int l2 = 0; l2 <= l1; ++l2)
            for (int l = l1 - l2; l <= std::min(twol, l1 + l2); l += 2)
                for (int m1 = 0; m1 <= l1; ++m1) {
                    const int aa2 = 2 * m1 - l1;
                    for (int m2 = 0; m2 <= l2; ++m2) {
                        const int bb2 = 2 * m2 - l2;
                        const int m = (aa2 + bb2 + l) / 2;
                        if (m < 0 || m > l) {
                            t->cglist[n++] = 0.0;
                            continue;
                        }
                        double sum = 0.0;
                        const int zlo = std::max(0, std::max(-(l - l2 + aa2) / 2, -(l - l1 - bb2) / 2));
                        const int zhi = std::min((l1 + l2 - l) / 2, std::min((l1 - aa2) / 2, (l2 + bb2) / 2));
                        for (int z = zlo; z <= zhi; ++z) {
                            const double ifac = (z % 2 == 0) ? 1.0 : -1.0;
                            sum += ifac / (factorial_ref(z) * factorial_ref((l1 + l2 - l) / 2 - z) *
                                           factorial_ref((l1 - aa2) / 2 - z) * factorial_ref((l2 + bb2) / 2 - z) *
                                           factorial_ref((l - l2 + aa2) / 2 + z) *
                                           factorial_ref((l - l1 - bb2) / 2 + z));
                        }
                        const int cc2 = 2 * m - l;
                        const double dcg = deltacg(l1, l2, l);
                        const double sfaccg =
                            std::sqrt(factorial_ref((l1 + aa2) / 2) * factorial_ref((l1 - aa2) / 2) *
                                      factorial_ref((l2 + bb2) / 2) * factorial_ref((l2 - bb2) / 2) *
                                      factorial_ref((l + cc2) / 2) * factorial_ref((l - cc2) / 2) * (double)(l + 1));
                        t->cglist[n++] = sum * dcg * sfaccg;
                    }
                }

    // U offsets: full and half layouts, u_norm per level (SO4.py:1288-1311)
    t->idxu_block.assign(ld, 0);
    t->h_block.assign(ld + 1, 0);
    t->unorm_l.assign(ld, 1.0);
    int nu = 0, nh = 0;
    for (int l = 0; l < ld; ++l) {
        t->idxu_block[l] = nu;
        t->h_block[l] = nh;
        nu += (l + 1) * (l + 1);
        nh += (l / 2 + 1) * (l + 1);
        if (normalize_u) t->unorm_l[l] = 4 * SO4_PI / std::sqrt((double)(l + 1));
    }
    t->h_block[ld] = nh;
    t->n_u = nu;
    t->n_half = nh;

    // idxb (SO4.py:1314-1327)
    for (int l1 = 0; l1 < ld; ++l1)
        for (int l2 = 0; l2 <= l1; ++l2)
            for (int l = l1 - l2; l <= std::min(twol, l1 + l2); l += 2)
                if (l >= l1) {
                    t->idxb.push_back(l1);
                    t->idxb.push_back(l2);
                    t->idxb.push_back(l);
                }
    t->n_b = (int)t->idxb.size() / 3;

    // idxz and idxz_block (SO4.py:1329-1395), plus the device entry list
    t->idxz_block.assign(ld * ld * ld, 0);
    std::vector<ZEnt> zent;
    std::vector<ZBlk> blks;
    n = 0;
    for (int l1 = 0; l1 < ld; ++l1)
        for (int l2 = 0; l2 <= l1; ++l2)
            for (int l = l1 - l2; l <= std::min(twol, l1 + l2); l += 2) {
                t->idxz_block[b3(ld, l1, l2, l)] = n;
                ZBlk bk;
                std::memset(&bk, 0, sizeof bk);
                bk.l1 = l1;
                bk.l2 = l2;
                bk.l = l;
                bk.z0 = n;
                for (int mb = 0; 2 * mb <= l; ++mb)
                    for (int ma = 0; ma <= l; ++ma) {
                        int q[10];
                        q[0] = l1;
                        q[1] = l2;
                        q[2] = l;
                        q[3] = std::max(0, (2 * ma - l - l2 + l1) / 2);
                        q[4] = (2 * ma - l - (2 * q[3] - l1) + l2) / 2;
                        q[5] = std::min(l1, (2 * ma - l + l2 + l1) / 2) - q[3] + 1;
                        q[6] = std::max(0, (2 * mb - l - l2 + l1) / 2);
                        q[7] = (2 * mb - l - (2 * q[6] - l1) + l2) / 2;
                        q[8] = std::min(l1, (2 * mb - l + l2 + l1) / 2) - q[6] + 1;
                        q[9] = t->idxu_block[l] + (l + 1) * mb + ma;
                        for (int c = 0; c < 10; ++c) t->idxz.push_back(q[c]);
                        ZEnt z;
                        const int cgbase = t->idxcg_block[b3(ld, l1, l2, l)];
                        z.na = q[5];
                        z.nb = q[8];
                        z.ma1min = q[3];
                        z.ma2max = q[4];
                        z.cga = cgbase + q[3] * (l2 + 1) + q[4];
                        z.cgb = cgbase + q[6] * (l2 + 1) + q[7];
                        z.u1 = t->idxu_block[l1] + (l1 + 1) * q[6];
                        z.u2 = t->idxu_block[l2] + (l2 + 1) * q[7];
                        z.l1 = l1;
                        z.l2 = l2;
                        z.jh = t->h_block[l] + (l + 1) * mb + ma;
                        z.blk = (int)blks.size();
                        z.jz = n;
                        zent.push_back(z);
                        n++;
                    }
                bk.n = n - bk.z0;
                blks.push_back(bk);
            }
    t->n_z = n;
    t->n_blk = (int)blks.size();

    // bispectrum components and the roles of each Z block in dB/dr (SO4.py:1113-1227)
    std::vector<BEnt> bent(t->n_b);
    for (int k = 0; k < t->n_b; ++k) {
        const int l1 = t->idxb[3 * k], l2 = t->idxb[3 * k + 1], l = t->idxb[3 * k + 2];
        BEnt &b = bent[k];
        b.l1 = l1;
        b.l2 = l2;
        b.l = l;
        b.lam[0] = l;
        b.lam[1] = l1;
        b.lam[2] = l2;
        b.z[0] = t->idxz_block[b3(ld, l1, l2, l)];
        b.z[1] = t->idxz_block[b3(ld, l, l2, l1)];
        b.z[2] = t->idxz_block[b3(ld, l, l1, l2)];
        b.fac[0] = 2.0;
        b.fac[1] = 2.0 * ((double)(l + 1) / (l1 + 1.0));
        b.fac[2] = 2.0 * ((double)(l + 1) / (l2 + 1.0));
        for (int s = 0; s < 3; ++s) {
            b.h[s] = t->h_block[b.lam[s]];
            b.cnt[s] = section_count(b.lam[s]);
        }
        const int blk_of[3] = {b.z[0], b.z[1], b.z[2]};
        for (int s = 0; s < 3; ++s) {
            for (auto &bk : blks)
                if (bk.z0 == blk_of[s]) {
                    bk.role_k[bk.nrole] = k;
                    bk.role_f[bk.nrole] = b.fac[s];
                    bk.role_f32[bk.nrole] = (float)b.fac[s];
                    bk.nrole++;
                }
        }
    }
    // The plain path's dB/dr: the three sections of every component read Z blocks that
    // several components share (165 sections over 125 distinct blocks at lmax 4), and the
    // components' section sizes differ several-fold.  So each distinct block is contracted
    // once per image, the blocks dealt to the 32 lanes of a warp largest first, each to the
    // lane with the fewest entries so far (ties: the lower lane), and listed lane by lane.
    std::vector<int4> usec;  // {first Z entry, half offset, entry count, level}
    std::vector<int> ksec_u(3 * (size_t)t->n_b);
    for (int k = 0; k < t->n_b; ++k)
        for (int s = 0; s < 3; ++s) {
            int u = 0;
            while (u < (int)usec.size() && usec[u].x != bent[k].z[s]) ++u;
            if (u == (int)usec.size()) usec.push_back(make_int4(bent[k].z[s], bent[k].h[s], bent[k].cnt[s], bent[k].lam[s]));
            ksec_u[3 * k + s] = u;
        }
    std::vector<int> order(usec.size());
    for (size_t u = 0; u < usec.size(); ++u) order[u] = (int)u;
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return usec[p].z > usec[q].z; });
    std::vector<int> lane_of(usec.size()), load(32, 0);
    for (int u : order) {
        int best = 0;
        for (int l = 1; l < 32; ++l)
            if (load[l] < load[best]) best = l;
        lane_of[u] = best;
        load[best] += usec[u].z;
    }
    std::vector<int4> psec;
    std::vector<int> psec_ptr(33, 0), pos_of(usec.size());
    for (int l = 0; l < 32; ++l) {
        psec_ptr[l] = (int)psec.size();
        for (int u : order)
            if (lane_of[u] == l) {
                pos_of[u] = (int)psec.size();
                psec.push_back(usec[u]);
            }
    }
    psec_ptr[32] = (int)psec.size();
    std::vector<int> ksec(3 * (size_t)t->n_b);
    for (size_t i = 0; i < ksec.size(); ++i) ksec[i] = pos_of[ksec_u[i]];
    t->n_psec = (int)psec.size();

    // blocks grouped by their third index (the level of Y they feed)
    std::vector<int> yptr(ld + 1, 0), ylist;
    for (int lam = 0; lam < ld; ++lam) {
        yptr[lam] = (int)ylist.size();
        for (int bi = 0; bi < t->n_blk; ++bi)
            if (blks[bi].l == lam) ylist.push_back(bi);
    }
    yptr[ld] = (int)ylist.size();

    std::vector<double> rp64(ld * ld, 0.0);
    std::vector<float> rp32(ld * ld, 0.f);
    for (int p = 1; p < ld; ++p)
        for (int q = 1; q < ld; ++q) {
            rp64[p * ld + q] = std::sqrt((double)p / (double)q);
            rp32[p * ld + q] = (float)rp64[p * ld + q];
        }
    std::vector<float> cg32(t->cglist.begin(), t->cglist.end());
    // B component of each block (blocks with l >= l1)
    std::vector<int> blk_k(t->n_blk, -1);
    for (int k = 0; k < t->n_b; ++k)
        for (int bi = 0; bi < t->n_blk; ++bi)
            if (blks[bi].z0 == bent[k].z[0]) blk_k[bi] = k;

    // Window work lists.  For block (a, b, lam) with d = (a + b - lam) / 2, the Z entry
    // (ma, mb) is (SO4.py:1042-1063)
    //   sum_{mb1} Cb(mb, mb1) sum_{ma2} Ca(ma, ma2) U_a[ma + d - ma2, mb1] U_b[ma2, mb + d - mb1].
    // A unit holds K <= wkmax (<= ZW_KMAX) consecutive entries ma0.. of one half row (rows
    // longer than wkmax are cut into near-equal parts).  Per block and per mb1 a sub-segment
    // walks ma2 = lo .. hi (the union of the entries' ranges, at most b + 1 <= a + 1
    // values, so the smaller U is the one stepped) with the K values of U_a in a
    // register ring.  Ca[j][k] = cg(a, ma0 + k + d - lo - j, b, lo + j), 0 outside the
    // ranges, in rows of KP = K rounded up to 4 floats; the Ca table of a
    // (block, ma0, K) is shared by every row.  The middle row of an even level
    // (2 mb = lam) is cut at its centre: Y weighs its entries ma > lam / 2 by zero and B's
    // section ends at the centre, so those entries are neither computed nor stored (the
    // reverse sweep reads them as zero).
    std::vector<int4> wunit_y, wseg_y, wunit_b, wseg_b, wsub;
    std::vector<float> wca;
    std::map<std::tuple<int, int, int>, int> ca_off;  // (block, ma0, K) -> offset
    auto row_len = [](int lam, int mb) { return (2 * mb == lam) ? lam / 2 + 1 : lam + 1; };
    auto cg_of = [&](const ZBlk &bk, int m1, int m2) {
        const int cgbase = t->idxcg_block[b3(ld, bk.l1, bk.l2, bk.l)];
        return t->cglist[cgbase + m1 * (bk.l2 + 1) + m2];
    };
    std::vector<std::pair<long, int>> wcy, wcb;
    struct WUnit {
        int lam, mb, ma0, nk;
        int sy0, sy1, sb0, sb1;  // segments in wseg_y / wseg_b
        int bslot;               // index among the level's units that start in the B section, or -1
    };
    std::vector<WUnit> wun;
    std::vector<int4> segy_all, segb_all;
    std::vector<long> segy_cost;  // the work of each segment of segy_all
    // B partial slots: component k owns nbu(lam_k) consecutive slots, one per window
    // unit of level lam_k that starts inside the B section, in (mb, ma0) order
    std::vector<int> nbu(ld, 0);
    const int wk = t->tune.wkmax;  // entries per unit at most (ZW_KMAX unless tuned lower)
    for (int lam = 0; lam < ld; ++lam) {
        for (int mb = 0; 2 * mb <= lam; ++mb) {
            const int n = row_len(lam, mb), ng = (n + wk - 1) / wk;
            for (int g = 0, ma0 = 0; g < ng; ++g) {
                if (mb * (lam + 1) + ma0 < section_count(lam)) nbu[lam]++;
                ma0 += n / ng + (g < n % ng ? 1 : 0);
            }
        }
    }
    std::vector<int> bpos(t->n_b + 1, 0);
    for (int k = 0; k < t->n_b; ++k) bpos[k + 1] = bpos[k] + nbu[bent[k].lam[0]];
    t->n_bsec = bpos[t->n_b];
    for (int lam = 0; lam < ld; ++lam) {
        int bu = 0;  // index of the next B-section unit of this level
        for (int mb = 0; 2 * mb <= lam; ++mb) {
            const int n = row_len(lam, mb), ng = (n + wk - 1) / wk;
            for (int g = 0, ma0 = 0; g < ng; ++g) {
                WUnit u;
                u.lam = lam;
                u.mb = mb;
                u.ma0 = ma0;
                u.nk = n / ng + (g < n % ng ? 1 : 0);
                const int K = u.nk, KP = (K + 3) / 4 * 4;
                ma0 += K;
                const int off0 = mb * (lam + 1) + u.ma0;
                const bool in_bsec = off0 < section_count(lam);  // the unit's first entry is in the B section
                const int bslot = in_bsec ? bu++ : -1;
                u.bslot = bslot;
                long costy = 0, costb = 0;
                u.sy0 = (int)segy_all.size();
                u.sb0 = (int)segb_all.size();
                for (int qq = yptr[lam]; qq < yptr[lam + 1]; ++qq) {
                    const int bi = ylist[qq];
                    const ZBlk &bk = blks[bi];
                    const int a = bk.l1, b = bk.l2, d = (a + b - lam) / 2;
                    const int lo = std::max(0, u.ma0 + d - a), hi = std::min(b, u.ma0 + K - 1 + d);
                    const int S = hi - lo + 1;
                    if (S <= 0) continue;
                    auto key = std::make_tuple(bi, u.ma0, K);
                    if (!ca_off.count(key)) {
                        ca_off[key] = (int)wca.size();
                        for (int j = 0; j < S; ++j)
                            for (int k = 0; k < KP; ++k) {
                                const int ma = u.ma0 + k, ma2 = lo + j, ma1 = ma + d - ma2;
                                const bool ok = k < K && ma <= lam && ma1 >= 0 && ma1 <= a;
                                wca.push_back(ok ? (float)cg_of(bk, ma1, ma2) : 0.f);
                            }
                    }
                    const int s0 = (int)wsub.size();
                    for (int mb1 = std::max(0, mb + d - b); mb1 <= std::min(a, mb + d); ++mb1) {
                        const int mb2 = mb + d - mb1;
                        // a == b: the row pairs (mb1, mb2) and (mb2, mb1) hold the same products with
                        // the same coefficients (cg(j m1 j m2) = (-1)^d cg(j m2 j m1), once in Ca and
                        // once in Cb), so only mb1 <= mb2 is walked, mb1 < mb2 with 2 Cb
                        if (a == b && mb1 > mb2) continue;
                        const double sym = (a == b && mb1 < mb2) ? 2.0 : 1.0;
                        // stepped: U_b[lo + j, mb2]; ring base: U_a[ma0 + d - lo, mb1]
                        const int f1 = (ZW_PAD + t->idxu_block[b] + mb2 * (b + 1) + lo) * 33;
                        const int f2 = (ZW_PAD + t->idxu_block[a] + mb1 * (a + 1) + u.ma0 + d - lo) * 33;
                        const float cb = (float)(sym * cg_of(bk, mb1, mb2));
                        int cbits;
                        std::memcpy(&cbits, &cb, sizeof cbits);
                        wsub.push_back(make_int4(f1 | (f2 << 16), ca_off[key], S, cbits));
                    }
                    const int s1 = (int)wsub.size();
                    const long c = (long)(s1 - s0) * (S * (6 * K + 8) + 12) + 16;
                    const int k = blk_k[bi];
                    const int bcode = (k >= 0 && in_bsec) ? bpos[k] + bslot : -1;
                    segy_all.push_back(make_int4(s0, s1, bi, bcode));
                    segy_cost.push_back(c);
                    costy += c;
                    if (bcode >= 0) {
                        segb_all.push_back(make_int4(s0, s1, bi, bcode));
                        costb += c;
                    }
                }
                u.sy1 = (int)segy_all.size();
                u.sb1 = (int)segb_all.size();
                wcy.push_back({-costy, (int)wun.size()});
                if (u.sb1 > u.sb0) wcb.push_back({-costb, (int)wun.size()});
                wun.push_back(u);
            }
        }
    }
    auto by_k_cost = [&](const std::pair<long, int> &x, const std::pair<long, int> &y) {
        const int kx = wun[x.second].nk, ky = wun[y.second].nk;
        if (kx != ky) return kx > ky;
        return x.first < y.first;
    };
    // The warps of a CTA take units in list order, each the next one when it is free, and
    // the CTA ends with its last warp.  Units are grouped by K (largest first: the warps of
    // a CTA mostly run one K specialisation at a time, so fewer instruction-cache misses),
    // most expensive first within a K; then swaps of two units of the same K that make the
    // simulated finish time, by the cost model, earlier for the layout's warps per CTA.
    const int zwarps = (t->tune.zw_atoms == 64 ? t->tune.zw_threads : 256) / 32;
    auto order_units = [&](std::vector<std::pair<long, int>> &wc) {
        auto finish = [&](const std::vector<std::pair<long, int>> &v) {
            std::priority_queue<long, std::vector<long>, std::greater<long>> free_at;
            for (int w = 0; w < zwarps; ++w) free_at.push(0);
            long end = 0;
            for (auto &e : v) {
                const long t0 = free_at.top();
                free_at.pop();
                free_at.push(t0 - e.first);  // e.first = -cost
                end = std::max(end, t0 - e.first);
            }
            return end;
        };
        std::stable_sort(wc.begin(), wc.end(), by_k_cost);
        long best = finish(wc);
        for (int pass = 0; pass < 3; ++pass) {
            bool better = false;
            for (size_t i = 0; i < wc.size(); ++i)
                for (size_t j = i + 1; j < wc.size(); ++j) {
                    if (wc[i].first == wc[j].first || wun[wc[i].second].nk != wun[wc[j].second].nk) continue;
                    std::swap(wc[i], wc[j]);
                    const long f = finish(wc);
                    if (f < best) {
                        best = f;
                        better = true;
                    } else {
                        std::swap(wc[i], wc[j]);
                    }
                }
            if (!better) break;
        }
    };
    order_units(wcy);
    order_units(wcb);
    for (int pass = 0; pass < 2; ++pass) {
        auto &order = pass ? wcb : wcy;
        auto &units = pass ? wunit_b : wunit_y;
        auto &segs = pass ? wseg_b : wseg_y;
        const auto &src = pass ? segb_all : segy_all;
        for (auto &v : order) {
            const WUnit &u = wun[v.second];
            const float un = (float)t->unorm_l[u.lam];
            int ubits;
            std::memcpy(&ubits, &un, sizeof ubits);
            const int q0 = pass ? u.sb0 : u.sy0, q1 = pass ? u.sb1 : u.sy1;
            const int s0 = (int)segs.size();
            for (int q = q0; q < q1; ++q) segs.push_back(src[q]);
            units.push_back(make_int4(u.lam | (u.mb << 8) | (u.ma0 << 16) | (u.nk << 24), s0, (int)segs.size(), ubits));
        }
    }
    t->n_wunit_y = (int)wunit_y.size();
    t->n_wsub = (int)wsub.size();
    t->n_wunit_b = (int)wunit_b.size();

    // JVP lists: the section entries of every level (units starting in the B section) and
    // every block with a role; a segment's .w is the unit's section-unit index.  Component
    // k owns the slots [jpos[k], jpos[k+1]): for each section s, nbu(lam_s) of them.  The
    // r-th role of block b (component k, section s) writes slot jbase[3b + r] + index,
    // scaled by jfac[3b + r] = fac_s.
    std::vector<int> jpos(t->n_b + 1, 0), jbase(3 * t->n_blk, 0), rdone(t->n_blk, 0);
    std::vector<float> jfac(3 * t->n_blk, 0.f);
    std::vector<int> zb_of(t->n_z + 1, -1);
    for (int bi = 0; bi < t->n_blk; ++bi) zb_of[blks[bi].z0] = bi;
    for (int k = 0; k < t->n_b; ++k) {
        int base = jpos[k];
        for (int sct = 0; sct < 3; ++sct) {
            const int bi = zb_of[bent[k].z[sct]];
            const int r = rdone[bi]++;  // roles were appended to each block in this (k, s) order
            jbase[3 * bi + r] = base;
            jfac[3 * bi + r] = (float)bent[k].fac[sct];
            base += nbu[bent[k].lam[sct]];
        }
        jpos[k + 1] = base;
    }
    t->n_jslot = jpos[t->n_b];
    for (int k = 0; k < t->n_b; ++k) t->n_jmax = std::max(t->n_jmax, jpos[k + 1] - jpos[k]);
    for (int bi = 0; bi < t->n_blk; ++bi)
        for (int r = blks[bi].nrole; r < 3; ++r) jbase[3 * bi + r] = -1;  // no role r
    std::vector<std::pair<long, int>> wcj;
    for (int ui = 0; ui < (int)wun.size(); ++ui) {
        const WUnit &u = wun[ui];
        if (u.bslot < 0) continue;
        long c = 0;
        for (int q = u.sy0; q < u.sy1; ++q)
            if (blks[segy_all[q].z].nrole > 0) c += segy_cost[q];
        wcj.push_back({-c, ui});
    }
    order_units(wcj);
    std::vector<int4> wunit_j, wseg_j;
    std::vector<int> jwrites(jpos[t->n_b], 0);
    for (auto &v : wcj) {
        const WUnit &u = wun[v.second];
        const int s0 = (int)wseg_j.size();
        for (int q = u.sy0; q < u.sy1; ++q) {
            const int4 sg = segy_all[q];
            if (blks[sg.z].nrole == 0) continue;
            wseg_j.push_back(make_int4(sg.x, sg.y, sg.z, u.bslot));
            for (int r = 0; r < blks[sg.z].nrole; ++r) jwrites[jbase[3 * sg.z + r] + u.bslot]++;
        }
        if ((int)wseg_j.size() > s0) {
            const float un = (float)t->unorm_l[u.lam];
            int ubits;
            std::memcpy(&ubits, &un, sizeof ubits);
            wunit_j.push_back(make_int4(u.lam | (u.mb << 8) | (u.ma0 << 16) | (u.nk << 24), s0, (int)wseg_j.size(),
                                        ubits));
        }
    }
    t->n_wunit_j = (int)wunit_j.size();
    // every slot is written by exactly one (unit, block, role): the sums read no stale scratch
    int jrc = SO4_OK;
    for (int q = 0; q < t->n_jslot; ++q)
        if (jwrites[q] != 1) jrc = SO4_ERR_UNSUPPORTED;
    t->n_wca = (int)wca.size();

    // hfull: per half entry (l, mb <= l / 2, ma) its full-layout position and, for the rows
    // below the middle, the position of its mirror (l, l - mb, l - ma) = (-1)^(mb + ma)
    // conj U (conj << 15 | negate << 14), else -1; the window kernels scatter U_tot with it
    std::vector<int2> hfull(t->n_half);
    for (int l = 0; l < ld; ++l)
        for (int mb = 0; 2 * mb <= l; ++mb)
            for (int ma = 0; ma <= l; ++ma) {
                const int h = t->h_block[l] + mb * (l + 1) + ma;
                const int f = t->idxu_block[l] + mb * (l + 1) + ma;
                const int fm = t->idxu_block[l] + (l - mb) * (l + 1) + (l - ma);
                hfull[h] = make_int2(f, (2 * mb < l) ? (fm | (1 << 15) | (((mb + ma) & 1) << 14)) : -1);
            }

    int rc = jrc;
    // The FP32 row-chain kernels carry each row in the scaled form V with
    //   U_l[ma][mb] = sqrt(C(l, mb) / C(l, ma)) V_l[ma][mb],
    // in which the recursion's coefficients sqrt(l - ma) / sqrt(l - mb) and
    // -sqrt(ma) / sqrt(l - mb) become 1 and -1; the chain-start mirror and the middle-row
    // symmetry keep their form.  hmap: per half entry {slot | row << 8 | diagonal << 15,
    // bits of u_norm F, bits of u_norm, 0}; yscale: F, by which the window kernels scale Y so
    // that the reverse sweep contracts V with it.
    auto binom = [](int n, int k) {
        double c = 1.0;
        for (int i = 1; i <= k; ++i) c = c * (double)(n - k + i) / (double)i;
        return c;
    };
    std::vector<int4> hmap;
    std::vector<float> yscale;
    std::vector<double> yscale64;
    for (int l = 0; l < ld; ++l) {
        const float un = (float)t->unorm_l[l];
        for (int mb = 0; 2 * mb <= l; ++mb)
            for (int ma = 0; ma <= l; ++ma) {
                const double F = std::sqrt(binom(l, mb) / binom(l, ma));
                const float unf = (float)(t->unorm_l[l] * F);
                int b_unf, b_un;
                std::memcpy(&b_unf, &unf, sizeof b_unf);
                std::memcpy(&b_un, &un, sizeof b_un);
                hmap.push_back(make_int4((l * (l + 1) / 2 + ma) | (mb << 8) | ((ma == mb ? 1 : 0) << 15), b_unf, b_un, 0));
                yscale.push_back((float)F);
                yscale64.push_back(F);
            }
    }
    if (!rc) rc = upload(&t->d_hfull, hfull);
    if (!rc) rc = upload(&t->d_hmap, hmap);
    if (!rc) rc = upload(&t->d_yscale, yscale);
    if (!rc) rc = upload(&t->d_yscale64, yscale64);
    if (!rc) rc = upload(&t->d_bpos, bpos);
    if (!rc) rc = upload(&t->d_wunit_y, wunit_y);
    if (!rc) rc = upload(&t->d_wseg_y, wseg_y);
    if (!rc && !wunit_b.empty()) rc = upload(&t->d_wunit_b, wunit_b);
    if (!rc && !wseg_b.empty()) rc = upload(&t->d_wseg_b, wseg_b);
    if (!rc) rc = upload(&t->d_wsub, wsub);
    if (!rc) rc = upload(&t->d_wunit_j, wunit_j);
    if (!rc) rc = upload(&t->d_wseg_j, wseg_j);
    if (!rc) rc = upload(&t->d_jpos, jpos);
    if (!rc) rc = upload(&t->d_jbase, jbase);
    if (!rc) rc = upload(&t->d_jfac, jfac);
    if (!rc) rc = upload(&t->d_wca, wca);
    if (!rc) rc = upload(&t->d_cg64, t->cglist);
    if (!rc) rc = upload(&t->d_cg32, cg32);
    if (!rc) rc = upload(&t->d_rootpq64, rp64);
    if (!rc) rc = upload(&t->d_rootpq32, rp32);
    if (!rc) rc = upload(&t->d_z, zent);
    if (!rc) rc = upload(&t->d_b, bent);
    if (!rc) rc = upload(&t->d_psec, psec);
    if (!rc) rc = upload(&t->d_psec_ptr, psec_ptr);
    if (!rc) rc = upload(&t->d_ksec, ksec);
    if (!rc) rc = upload(&t->d_blk, blks);
    if (!rc) {
        std::vector<int4> rk(t->n_blk);
        std::vector<float4> rf(t->n_blk);
        for (int bi = 0; bi < t->n_blk; ++bi) {
            const ZBlk &bk = blks[bi];
            int k[3];
            float f[3];
            for (int r = 0; r < 3; ++r) {
                k[r] = (r < bk.nrole) ? bk.role_k[r] : (bk.nrole > 0 ? bk.role_k[0] : 0);
                f[r] = (r < bk.nrole) ? bk.role_f32[r] : 0.f;
            }
            rk[bi] = make_int4(k[0], k[1], k[2], bk.nrole);
            rf[bi] = make_float4(f[0], f[1], f[2], 0.f);
        }
        rc = upload(&t->d_blk_rk, rk);
        if (!rc) rc = upload(&t->d_blk_rf, rf);
    }
    if (!rc) rc = upload(&t->d_yblk_ptr, yptr);
    if (!rc) rc = upload(&t->d_yblk, ylist);
    // a unit cap below the default means more units and so more B / JVP slots, which the
    // window kernels stage in shared memory, and the other window layout has other tiles:
    // refuse a tuning whose window kernels would not run in every mode where the default
    // ones do
    if (!rc && (t->tune.wkmax != ZW_KMAX || t->tune.zw_atoms != tuning_defaults(twol).zw_atoms)) {
        size_t mt[4], md[4];
        so4_zw_smem_modes(t, mt);
        if (std::max(std::max(mt[0], mt[1]), std::max(mt[2], mt[3])) > 227 * 1024) {
            so4_tuning d = tuning_defaults(twol);
            so4_tables *t0 = nullptr;
            if (so4_tables_create_tuned(twol, normalize_u, &d, &t0) == SO4_OK) {
                so4_zw_smem_modes(t0, md);
                for (int q = 0; q < 4; ++q)
                    if (mt[q] > 227 * 1024 && md[q] <= 227 * 1024) rc = SO4_ERR_UNSUPPORTED;
                so4_tables_destroy(t0);
            }
        }
    }
    if (rc) {
        free_device(t);
        delete t;
        return rc;
    }
    *out = t;
    return SO4_OK;
}

extern "C" int so4_tables_destroy(so4_tables *t) {
    if (!t) return SO4_OK;
    free_device(t);
    delete t;
    return SO4_OK;
}

extern "C" int so4_tables_sizes(const so4_tables *t, int *s) {
    if (!t || !s) return SO4_ERR_ARG;
    s[0] = t->n_u;
    s[1] = t->n_half;
    s[2] = t->n_z;
    s[3] = t->n_b;
    s[4] = t->n_cg;
    s[5] = t->n_blk;
    s[6] = t->n_bsec;
    s[7] = t->n_wsub;
    return SO4_OK;
}

extern "C" int so4_tables_export(const so4_tables *t, double *cg, int *idxb, int *idxz, int *idxu_block,
                                 int *idxz_block, int *idxcg_block) {
    if (!t) return SO4_ERR_ARG;
    const size_t l3 = (size_t)t->ldim * t->ldim * t->ldim;
    if (cg) std::memcpy(cg, t->cglist.data(), sizeof(double) * t->n_cg);
    if (idxb) std::memcpy(idxb, t->idxb.data(), sizeof(int) * t->idxb.size());
    if (idxz) std::memcpy(idxz, t->idxz.data(), sizeof(int) * t->idxz.size());
    if (idxu_block) std::memcpy(idxu_block, t->idxu_block.data(), sizeof(int) * t->ldim);
    if (idxz_block) std::memcpy(idxz_block, t->idxz_block.data(), sizeof(int) * l3);
    if (idxcg_block) std::memcpy(idxcg_block, t->idxcg_block.data(), sizeof(int) * l3);
    return SO4_OK;
}

extern "C" const char *so4_version(void) { return "so4_gb300 0.1.0 (sm_103a)"; }

#include <atomic>
#include <mutex>
static std::atomic<long long> g_launches{0};

namespace {
struct SmemLimit {
    const void *kern;
    int dev;
    size_t bytes;
};
std::mutex g_smem_mu;
std::vector<SmemLimit> g_smem;
}  // namespace

int so4_set_smem(const void *kern, size_t smem) {
    if (smem > 227 * 1024) return SO4_ERR_UNSUPPORTED;
    if (smem <= 48 * 1024) return SO4_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SO4_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_smem_mu);
    for (auto &e : g_smem)
        if (e.kern == kern && e.dev == dev) {
            if (e.bytes >= smem) return SO4_OK;
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return SO4_ERR_CUDA;
            e.bytes = smem;
            return SO4_OK;
        }
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SO4_ERR_CUDA;
    g_smem.push_back({kern, dev, smem});
    return SO4_OK;
}
void so4_count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Programmatic dependent launch of the kernels that support it (so4_launch_pdl), for the
// launches this host thread makes while it is on.
static thread_local int g_pdl = 0;
int so4_pdl_on() { return g_pdl; }
extern "C" int so4_set_pdl(int on) {
    const int prev = g_pdl;
    g_pdl = on ? 1 : 0;
    return prev;
}
extern "C" long long so4_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }
