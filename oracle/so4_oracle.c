/*
 * so4_oracle.c -- FP64 CPU restatement of PyXtal_FF's SO(4)/SNAP bispectrum path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: it is compiled into
 * oracle/_build/libso4oracle.so and may be loaded only by tests/, by
 * __graft_entry__.smoke() and by bench.py (its cpu_baseline leg and its
 * reference arm), always as the checker or the timed CPU baseline.  The
 * product path (pyxtal_ff_gb300) never loads it and has no CPU fallback.
 *
 * It restates, loop for loop, the algorithm of the reference
 * (pyxtal_ff/descriptors/SO4.py and SNAP.py):
 *   - factorial table / deltacg          angular_momentum.py:9-190
 *   - init_clebsch_gordan                SO4.py:410-480
 *   - cutoff functions + derivatives     SO4.py:306-408, 482-558
 *   - addself_uarraytot                  SO4.py:560-597
 *   - init_rootpqarray                   SO4.py:831-838
 *   - compute_uarray_recursive           SO4.py:840-926
 *   - compute_duarray_recursive          SO4.py:928-987
 *   - add_uarraytot / dudr               SO4.py:989-1018
 *   - compute_zi / compute_bi            SO4.py:1020-1111
 *   - compute_dbidrj                     SO4.py:1113-1227
 *   - index tables + driver              SO4.py:1265-1548 (derivative+stress branch)
 *   - neighbour grouping (seq)           SO4.py:211-287
 * The SNAP variant differs only in the neighbour/site weights and in
 * psi = rfac0*pi*r/rc (SNAP.py:273, 299-301, 1473...).
 *
 * The ASE neighbour list the reference calls (ase.neighborlist.NeighborList,
 * ASE >= 3.22.1, not vendored) is restated as: every periodic image
 * (j, o) with |pos[j] + o.cell - pos[i]| < rc, excluding (i, o=0); the
 * images of one (i, j) group are ordered by the integer offset o
 * (lexicographic).  That intra-group order is not pinned by any
 * reference test (it only changes FP64 summation order).
 *
 * The descriptor loop runs one centre atom per OpenMP iteration; each atom
 * owns its output rows, so there are no races.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_PI 3.141592653589793

typedef struct { double re, im; } cx;

static inline cx cx_make(double re, double im) { cx z; z.re = re; z.im = im; return z; }
static inline cx cx_add(cx a, cx b) { return cx_make(a.re + b.re, a.im + b.im); }
static inline cx cx_mul(cx a, cx b) { return cx_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cx_scale(cx a, double s) { return cx_make(a.re * s, a.im * s); }
static inline cx cx_conj(cx a) { return cx_make(a.re, -a.im); }

/* ------------------------------------------------------------------ */
/* factorials as tabulated by the reference (angular_momentum.py:9-182):
 * exact for n <= 20, n! rounded to 15 significant digits above.        */
static double fact_tab[64];
static int fact_ready = 0;

static void fact_init(void) {
    if (fact_ready) return;
    unsigned __int128 f = 1;
    for (int n = 0; n < 64; ++n) {
        if (n > 0) f *= (unsigned __int128)n;
        if (n <= 20) {
            fact_tab[n] = (double)(uint64_t)f;
        } else if (n <= 34) {
            char digits[64]; int nd = 0;
            unsigned __int128 t = f;
            while (t > 0) { digits[nd++] = (char)('0' + (int)(t % 10)); t /= 10; }
            /* digits are little-endian; build "d.ddddddddddddddde+XX" from the exact integer */
            char buf[96]; int k = 0;
            for (int q = nd - 1; q >= 0; --q) buf[k++] = digits[q];
            buf[k] = 0;
            /* round the decimal string to 15 significant digits (half up, as printf) */
            char m[20]; memcpy(m, buf, 15); m[15] = 0;
            int carry = (buf[15] >= '5');
            for (int q = 14; q >= 0 && carry; --q) {
                if (m[q] == '9') { m[q] = '0'; } else { m[q]++; carry = 0; }
            }
            int exp10 = nd - 1;
            char s[64];
            if (carry) { snprintf(s, sizeof s, "1.%.14se%d", "00000000000000", exp10 + 1); }
            else { snprintf(s, sizeof s, "%c.%se%d", m[0], m + 1, exp10); }
            fact_tab[n] = strtod(s, NULL);
        } else {
            fact_tab[n] = NAN;  /* beyond any supported twol */
        }
    }
    fact_ready = 1;
}

static inline double fac(int n) { return fact_tab[n]; }

double so4o_factorial(int n) { fact_init(); return (n >= 0 && n < 64) ? fact_tab[n] : NAN; }

/* deltacg, angular_momentum.py:184-190 */
static double deltacg(int l1, int l2, int l) {
    double sfaccg = fac((l1 + l2 + l) / 2 + 1);
    return sqrt(fac((l1 + l2 - l) / 2) * fac((l1 - l2 + l) / 2) * fac((-l1 + l2 + l) / 2) / sfaccg);
}

/* ------------------------------------------------------------------ */
/* index tables, SO4.py:1265-1396                                     */
typedef struct {
    int twol, ldim;
    int idxcg_count, idxu_count, idxb_count, idxz_count;
    int *idxcg_block;   /* ldim^3 */
    int *idxu_block;    /* ldim   */
    int *idxz_block;    /* ldim^3 */
    int *idxb;          /* nB x 3 */
    int *idxz;          /* nZ x 10 */
    double *cglist;
    double *unorm;      /* idxu_count */
    double *rootpq;     /* ldim x ldim */
} tables_t;

static int b3(int ldim, int a, int b, int c) { return (a * ldim + b) * ldim + c; }

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

static void tables_free(tables_t *t) {
    free(t->idxcg_block); free(t->idxu_block); free(t->idxz_block); free(t->idxb);
    free(t->idxz); free(t->cglist); free(t->unorm); free(t->rootpq);
}

/* init_clebsch_gordan, SO4.py:410-480 (Varshalovich 8.2.1(3)) */
static void init_cg(int twol, double *cglist) {
    int ldim = twol + 1, n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2)
    for (int m1 = 0; m1 <= l1; ++m1) {
        int aa2 = 2 * m1 - l1;
        for (int m2 = 0; m2 <= l2; ++m2) {
            int bb2 = 2 * m2 - l2;
            int m2x = aa2 + bb2 + l;           /* = 2m, always even */
            int m = m2x / 2;
            if (m < 0 || m > l) { cglist[n++] = 0.0; continue; }
            double sum = 0.0;
            int zlo = imax(0, imax(-(l - l2 + aa2) / 2, -(l - l1 - bb2) / 2));
            int zhi = imin((l1 + l2 - l) / 2, imin((l1 - aa2) / 2, (l2 + bb2) / 2));
            for (int z = zlo; z <= zhi; ++z) {
                double ifac = (z % 2 == 0) ? 1.0 : -1.0;
                sum += ifac / (fac(z) * fac((l1 + l2 - l) / 2 - z) * fac((l1 - aa2) / 2 - z) *
                               fac((l2 + bb2) / 2 - z) * fac((l - l2 + aa2) / 2 + z) *
                               fac((l - l1 - bb2) / 2 + z));
            }
            int cc2 = 2 * m - l;
            double dcg = deltacg(l1, l2, l);
            double sfaccg = sqrt(fac((l1 + aa2) / 2) * fac((l1 - aa2) / 2) * fac((l2 + bb2) / 2) *
                                 fac((l2 - bb2) / 2) * fac((l + cc2) / 2) * fac((l - cc2) / 2) *
                                 (double)(l + 1));
            cglist[n++] = sum * dcg * sfaccg;
        }
    }
}

static int tables_init(tables_t *t, int twol, int norm) {
    fact_init();
    memset(t, 0, sizeof *t);
    if (twol < 0 || twol > 20) return 1;
    int ldim = twol + 1;
    t->twol = twol; t->ldim = ldim;
    t->idxcg_block = (int *)calloc((size_t)ldim * ldim * ldim, sizeof(int));
    t->idxz_block = (int *)calloc((size_t)ldim * ldim * ldim, sizeof(int));
    t->idxu_block = (int *)calloc((size_t)ldim, sizeof(int));
    int n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2) {
        t->idxcg_block[b3(ldim, l1, l2, l)] = n;
        n += (l1 + 1) * (l2 + 1);
    }
    t->idxcg_count = n;
    t->cglist = (double *)calloc((size_t)n, sizeof(double));
    init_cg(twol, t->cglist);

    n = 0;
    for (int l = 0; l < ldim; ++l) { t->idxu_block[l] = n; n += (l + 1) * (l + 1); }
    t->idxu_count = n;
    t->unorm = (double *)malloc((size_t)n * sizeof(double));
    for (int l = 0; l < ldim; ++l)
        for (int e = 0; e < (l + 1) * (l + 1); ++e)
            t->unorm[t->idxu_block[l] + e] = norm ? 4.0 * O_PI / sqrt((double)(l + 1)) : 1.0;

    n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2)
        if (l >= l1) n++;
    t->idxb_count = n;
    t->idxb = (int *)malloc((size_t)3 * (n ? n : 1) * sizeof(int));
    n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2)
        if (l >= l1) { t->idxb[3 * n] = l1; t->idxb[3 * n + 1] = l2; t->idxb[3 * n + 2] = l; n++; }

    n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2)
        for (int mb = 0; 2 * mb <= l; ++mb) n += l + 1;
    t->idxz_count = n;
    t->idxz = (int *)malloc((size_t)10 * n * sizeof(int));
    n = 0;
    for (int l1 = 0; l1 < ldim; ++l1)
    for (int l2 = 0; l2 <= l1; ++l2)
    for (int l = l1 - l2; l <= imin(twol, l1 + l2); l += 2) {
        t->idxz_block[b3(ldim, l1, l2, l)] = n;
        for (int mb = 0; 2 * mb <= l; ++mb)
        for (int ma = 0; ma <= l; ++ma) {
            int *z = t->idxz + 10 * n;
            z[0] = l1; z[1] = l2; z[2] = l;
            z[3] = imax(0, (2 * ma - l - l2 + l1) / 2);
            z[4] = (2 * ma - l - (2 * z[3] - l1) + l2) / 2;
            z[5] = imin(l1, (2 * ma - l + l2 + l1) / 2) - z[3] + 1;
            z[6] = imax(0, (2 * mb - l - l2 + l1) / 2);
            z[7] = (2 * mb - l - (2 * z[6] - l1) + l2) / 2;
            z[8] = imin(l1, (2 * mb - l + l2 + l1) / 2) - z[6] + 1;
            z[9] = t->idxu_block[l] + (l + 1) * mb + ma;
            n++;
        }
    }
    t->rootpq = (double *)calloc((size_t)ldim * ldim, sizeof(double));
    for (int p = 1; p < ldim; ++p)
        for (int q = 1; q < ldim; ++q)
            t->rootpq[p * ldim + q] = sqrt((double)p / (double)q);
    return 0;
}

/* sizes: out[0..4] = idxu, idxz, idxcg, nB, idxu_half */
int so4o_sizes(int twol, int *out) {
    tables_t t;
    if (tables_init(&t, twol, 0)) return 1;
    int half = 0;
    for (int l = 0; l <= twol; ++l) half += (l / 2 + 1) * (l + 1);
    out[0] = t.idxu_count; out[1] = t.idxz_count; out[2] = t.idxcg_count; out[3] = t.idxb_count;
    out[4] = half;
    tables_free(&t);
    return 0;
}

/* copies of the tables, so tests can compare them with the reference's */
int so4o_tables(int twol, int norm, double *cglist, int *idxb, int *idxz, int *idxu_block,
                int *idxz_block, int *idxcg_block, double *unorm) {
    tables_t t;
    if (tables_init(&t, twol, norm)) return 1;
    int l3 = t.ldim * t.ldim * t.ldim;
    if (cglist) memcpy(cglist, t.cglist, sizeof(double) * t.idxcg_count);
    if (idxb) memcpy(idxb, t.idxb, sizeof(int) * 3 * t.idxb_count);
    if (idxz) memcpy(idxz, t.idxz, sizeof(int) * 10 * t.idxz_count);
    if (idxu_block) memcpy(idxu_block, t.idxu_block, sizeof(int) * t.ldim);
    if (idxz_block) memcpy(idxz_block, t.idxz_block, sizeof(int) * l3);
    if (idxcg_block) memcpy(idxcg_block, t.idxcg_block, sizeof(int) * l3);
    if (unorm) memcpy(unorm, t.unorm, sizeof(double) * t.idxu_count);
    tables_free(&t);
    return 0;
}

/* ------------------------------------------------------------------ */
/* cutoff functions, SO4.py:306-408 and compute_sfac/dsfac 482-558     */
static double sfac_fn(double r, double rc, int id) {
    if (r > rc) return 0.0;
    double x = r / rc;
    switch (id) {
    case 1: return 0.5 * (cos(O_PI * r / rc) + 1.0);
    case 2: { double t = tanh(1.0 - r / rc); return t * t * t; }
    case 3: return x * x * (2.0 * x - 3.0) + 1.0;
    case 4: return x * x * x * (x * (15.0 - 6.0 * x) - 10.0) + 1.0;
    case 5: return x * x * x * x * (x * (x * (20.0 * x - 70.0) + 84.0) - 35.0) + 1.0;
    case 6: return x * x * x * x * x * (x * (x * (x * (315.0 - 70.0 * x) - 540.0) + 420.0) - 126.0) + 1.0;
    case 7: { double d = 1.0 - x * x; if (d == 0.0) return 0.0; return exp(1.0 - 1.0 / d); }
    default: return NAN;
    }
}

static double dsfac_fn(double r, double rc, int id) {
    if (r > rc) return 0.0;
    double x = r / rc;
    switch (id) {
    case 1: return -0.5 * O_PI / rc * sin(O_PI * r / rc);
    case 2: { double t = tanh(1.0 - r / rc); double t2 = t * t; return -(3.0 / rc) * t2 * (1.0 - t2); }
    case 3: return (6.0 / (rc * rc)) * r * (r / rc - 1.0);
    case 4: return (-30.0 / rc) * (x * x * (x - 1.0) * (x - 1.0));
    case 5: { double y = x - 1.0; return (140.0 / rc) * (x * x * x * (y * y * y)); }
    case 6: { double y = x - 1.0; return (-630.0 / rc) * (x * x * x * x * (y * y * y * y)); }
    case 7: { /* the reference's ExponentPrime, kept as written (SO4.py:401-408) */
        double d = 1.0 - x * x; if (d == 0.0) return 0.0;
        double q = 1.0 + x * x;
        return 2.0 * x * exp(1.0 - 1.0 / d) / (q * q); }
    default: return NAN;
    }
}

double so4o_sfac(double r, double rc, int id) { return sfac_fn(r, rc, id); }
double so4o_dsfac(double r, double rc, int id) { return dsfac_fn(r, rc, id); }

/* ------------------------------------------------------------------ */
/* compute_uarray_recursive, SO4.py:840-926 (full (l+1)^2 layers)      */
static void uarray(const tables_t *t, double x, double y, double z, double psi, double r, cx *u) {
    const int ldim = t->ldim;
    double cs = cos(psi), sn = sin(psi);
    cx a = cx_make(cs, -(sn / r) * z);
    cx b = cx_make((sn / r) * y, -((sn / r) * x));
    cx ca = cx_conj(a), cb = cx_conj(b);
    for (int e = 0; e < t->idxu_count; ++e) u[e] = cx_make(0.0, 0.0);
    u[0] = cx_make(1.0, 0.0);
    for (int l = 1; l < ldim; ++l) {
        int llu = t->idxu_block[l], llup = t->idxu_block[l - 1];
        for (int mb = 0; 2 * mb <= l; ++mb) {
            u[llu] = cx_make(0.0, 0.0);
            for (int ma = 0; ma < l; ++ma) {
                double rp = t->rootpq[(l - ma) * ldim + (l - mb)];
                u[llu] = cx_add(u[llu], cx_mul(cx_scale(ca, rp), u[llup]));
                rp = t->rootpq[(ma + 1) * ldim + (l - mb)];
                u[llu + 1] = cx_add(u[llu + 1], cx_mul(cx_scale(cb, -rp), u[llup]));
                llu++; llup++;
            }
            llu++;
        }
        llu = t->idxu_block[l];
        llup = llu + (l + 1) * (l + 1) - 1;
        int mbpar = 1;
        for (int mb = 0; 2 * mb <= l; ++mb) {
            int mapar = mbpar;
            for (int ma = 0; ma <= l; ++ma) {
                cx c = cx_conj(u[llu]);
                u[llup] = (mapar == 1) ? c : cx_make(-c.re, -c.im);
                mapar = -mapar; llu++; llup--;
            }
            mbpar = -mbpar;
        }
    }
}

/* compute_duarray_recursive, SO4.py:928-987; du[e*3+c] */
static void duarray(const tables_t *t, double x, double y, double z, double psi, double r,
                    const cx *u, cx *du) {
    const int ldim = t->ldim;
    double cs = cos(psi), sn = sin(psi);
    cx a = cx_make(cs, -(sn / r) * z);
    cx b = cx_make((sn / r) * y, -((sn / r) * x));
    double g[3] = {x / r, y / r, z / r};
    cx da[3], db[3];
    for (int c = 0; c < 3; ++c) {
        da[c] = cx_make(-sn * psi / r * g[c], -z * cs / r / r * psi * g[c] + z * sn / r / r * g[c]);
        double f = cs / r / r * psi - sn / r / r;
        db[c] = cx_make(f * y * g[c], -(f * x) * g[c]);
    }
    da[2].im += -sn / r;
    db[1].re += sn / r;
    db[0].im += -sn / r;
    cx ca = cx_conj(a), cb = cx_conj(b);
    cx cda[3], cdb[3];
    for (int c = 0; c < 3; ++c) { cda[c] = cx_conj(da[c]); cdb[c] = cx_conj(db[c]); }
    for (int e = 0; e < 3 * t->idxu_count; ++e) du[e] = cx_make(0.0, 0.0);
    for (int l = 1; l < ldim; ++l) {
        int llu = t->idxu_block[l], llup = t->idxu_block[l - 1];
        for (int mb = 0; 2 * mb <= l; ++mb) {
            for (int c = 0; c < 3; ++c) du[3 * llu + c] = cx_make(0.0, 0.0);
            for (int ma = 0; ma < l; ++ma) {
                double rp = t->rootpq[(l - ma) * ldim + (l - mb)];
                for (int c = 0; c < 3; ++c) {
                    cx v = cx_add(cx_mul(cda[c], u[llup]), cx_mul(ca, du[3 * llup + c]));
                    du[3 * llu + c] = cx_add(du[3 * llu + c], cx_scale(v, rp));
                }
                rp = t->rootpq[(ma + 1) * ldim + (l - mb)];
                for (int c = 0; c < 3; ++c) {
                    cx v = cx_add(cx_mul(cdb[c], u[llup]), cx_mul(cb, du[3 * llup + c]));
                    du[3 * (llu + 1) + c] = cx_scale(v, -rp);
                }
                llu++; llup++;
            }
            llu++;
        }
        llu = t->idxu_block[l];
        llup = llu + (l + 1) * (l + 1) - 1;
        int mbpar = 1;
        for (int mb = 0; 2 * mb <= l; ++mb) {
            int mapar = mbpar;
            for (int ma = 0; ma <= l; ++ma) {
                for (int c = 0; c < 3; ++c) {
                    cx v = cx_conj(du[3 * llu + c]);
                    du[3 * llup + c] = (mapar == 1) ? v : cx_make(-v.re, -v.im);
                }
                mapar = -mapar; llu++; llup--;
            }
            mbpar = -mbpar;
        }
    }
}

/* compute_zi, SO4.py:1020-1068 */
static void compute_z(const tables_t *t, const cx *ut, cx *zl) {
    const int ldim = t->ldim;
    for (int jjz = 0; jjz < t->idxz_count; ++jjz) {
        const int *q = t->idxz + 10 * jjz;
        int l1 = q[0], l2 = q[1], l = q[2], ma1min = q[3], ma2max = q[4], na = q[5];
        int mb1min = q[6], mb2max = q[7], nb = q[8];
        const double *cgb = t->cglist + t->idxcg_block[b3(ldim, l1, l2, l)];
        cx zz = cx_make(0.0, 0.0);
        int llu1 = t->idxu_block[l1] + (l1 + 1) * mb1min;
        int llu2 = t->idxu_block[l2] + (l2 + 1) * mb2max;
        int icgb = mb1min * (l2 + 1) + mb2max;
        for (int ib = 0; ib < nb; ++ib) {
            cx suma1 = cx_make(0.0, 0.0);
            int ma1 = ma1min, ma2 = ma2max;
            int icga = ma1min * (l2 + 1) + ma2max;
            for (int ia = 0; ia < na; ++ia) {
                suma1 = cx_add(suma1, cx_mul(cx_scale(ut[llu1 + ma1], cgb[icga]), ut[llu2 + ma2]));
                ma1++; ma2--; icga += l2;
            }
            zz = cx_add(zz, cx_scale(suma1, cgb[icgb]));
            llu1 += l1 + 1; llu2 -= l2 + 1; icgb += l2;
        }
        zl[jjz] = zz;
    }
}

/* compute_bi, SO4.py:1071-1111 (real part kept, as 'x' = blist.real) */
static void compute_b(const tables_t *t, const cx *ut, const cx *zl, double *bl) {
    const int ldim = t->ldim;
    for (int k = 0; k < t->idxb_count; ++k) {
        int l1 = t->idxb[3 * k], l2 = t->idxb[3 * k + 1], l = t->idxb[3 * k + 2];
        int jjz = t->idxz_block[b3(ldim, l1, l2, l)];
        int jju = t->idxu_block[l];
        cx s = cx_make(0.0, 0.0);
        for (int mb = 0; 2 * mb < l; ++mb)
            for (int ma = 0; ma <= l; ++ma) { s = cx_add(s, cx_mul(cx_conj(ut[jju]), zl[jjz])); jjz++; jju++; }
        if (l % 2 == 0) {
            int mb = l / 2;
            for (int ma = 0; ma < mb; ++ma) { s = cx_add(s, cx_mul(cx_conj(ut[jju]), zl[jjz])); jjz++; jju++; }
            s = cx_add(s, cx_scale(cx_mul(cx_conj(ut[jju]), zl[jjz]), 0.5));
        }
        bl[k] = 2.0 * s.re;
    }
}


/* one section of compute_dbidrj (SO4.py:1128-1156): the half layer of dU_lam
 * (rows 2mb < lam, plus the first half of the middle row for even lam, whose
 * centre entry carries weight 1/2) dotted with one Z block.             */
static void dbsection(const tables_t *t, int lam, int jjz, const cx *du, const cx *zl, cx s[3]) {
    int jju = t->idxu_block[lam];
    for (int c = 0; c < 3; ++c) s[c] = cx_make(0.0, 0.0);
    for (int mb = 0; 2 * mb < lam; ++mb)
        for (int ma = 0; ma <= lam; ++ma) {
            for (int c = 0; c < 3; ++c) s[c] = cx_add(s[c], cx_mul(cx_conj(du[3 * jju + c]), zl[jjz]));
            jju++; jjz++;
        }
    if (lam % 2 == 0) {
        int mb = lam / 2;
        for (int ma = 0; ma < mb; ++ma) {
            for (int c = 0; c < 3; ++c) s[c] = cx_add(s[c], cx_mul(cx_conj(du[3 * jju + c]), zl[jjz]));
            jju++; jjz++;
        }
        for (int c = 0; c < 3; ++c) s[c] = cx_add(s[c], cx_scale(cx_mul(cx_conj(du[3 * jju + c]), zl[jjz]), 0.5));
    }
}

/* compute_dbidrj, SO4.py:1113-1227; tdb[k*3+c] = Re(dB_k/dr_c) */
static void compute_db(const tables_t *t, const cx *du, const cx *zl, double *tdb) {
    const int ldim = t->ldim;
    for (int k = 0; k < t->idxb_count; ++k) {
        int l1 = t->idxb[3 * k], l2 = t->idxb[3 * k + 1], l = t->idxb[3 * k + 2];
        cx s[3], acc[3];
        dbsection(t, l, t->idxz_block[b3(ldim, l1, l2, l)], du, zl, s);
        for (int c = 0; c < 3; ++c) acc[c] = cx_scale(s[c], 2.0);
        double l1fac = (double)(l + 1) / (l1 + 1.0);
        dbsection(t, l1, t->idxz_block[b3(ldim, l, l2, l1)], du, zl, s);
        for (int c = 0; c < 3; ++c) acc[c] = cx_add(acc[c], cx_scale(cx_scale(s[c], 2.0), l1fac));
        double l2fac = (double)(l + 1) / (l2 + 1.0);
        dbsection(t, l2, t->idxz_block[b3(ldim, l, l1, l2)], du, zl, s);
        for (int c = 0; c < 3; ++c) acc[c] = cx_add(acc[c], cx_scale(cx_scale(s[c], 2.0), l2fac));
        for (int c = 0; c < 3; ++c) tdb[3 * k + c] = acc[c].re;
    }
}

/* ------------------------------------------------------------------ */
/* Neighbour list.  Bins on wrapped fractional coordinates (periodic axes),
 * then every image is re-expressed as an integer offset of the ORIGINAL
 * positions and its vector computed as (pos[j] + (o1*a1 + o2*a2 + o3*a3)) - pos[i],
 * accepted when sqrt((x*x + y*y) + z*z) < rc (as SO4.py:1440 forms r).  */
typedef struct {
    int n;
    int64_t nimg, npair;
    int64_t *img_ptr;      /* n+1 */
    int32_t *img_j;        /* nimg */
    int32_t *img_off;      /* nimg*3 */
    double *img_r;         /* nimg*3 */
    int64_t *pair_ptr;     /* n+1: pairs of centre i are [pair_ptr[i], pair_ptr[i+1]) */
    int64_t *seq;          /* npair*2 */
    int64_t *pair_img;     /* npair+1: images of pair p are [pair_img[p], pair_img[p+1]) */
    int64_t *nsite;        /* n: index of the (i,i) pair */
} so4o_nl;

typedef struct { int32_t j, o0, o1, o2; double r[3]; } cand_t;

static int cand_cmp(const void *pa, const void *pb) {
    const cand_t *a = (const cand_t *)pa, *b = (const cand_t *)pb;
    if (a->j != b->j) return a->j < b->j ? -1 : 1;
    if (a->o0 != b->o0) return a->o0 < b->o0 ? -1 : 1;
    if (a->o1 != b->o1) return a->o1 < b->o1 ? -1 : 1;
    if (a->o2 != b->o2) return a->o2 < b->o2 ? -1 : 1;
    return 0;
}

static int inv3(const double *m, double *inv) {
    double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                 m[2] * (m[3] * m[7] - m[4] * m[6]);
    if (!(fabs(det) > 0.0) || !isfinite(det)) return 1;
    inv[0] = (m[4] * m[8] - m[5] * m[7]) / det; inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
    inv[2] = (m[1] * m[5] - m[2] * m[4]) / det; inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
    inv[4] = (m[0] * m[8] - m[2] * m[6]) / det; inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
    inv[6] = (m[3] * m[7] - m[4] * m[6]) / det; inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
    inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
    return 0;
}

void so4o_nl_free(so4o_nl *nl) {
    if (!nl) return;
    free(nl->img_ptr); free(nl->img_j); free(nl->img_off); free(nl->img_r);
    free(nl->pair_ptr); free(nl->seq); free(nl->pair_img); free(nl->nsite);
    free(nl);
}

/* n_center <= n atoms are centres (a prefix, as the reference's atom_ids). */
so4o_nl *so4o_nl_build(int n, int n_center, const double *pos, const double *cell, const int *pbc, double rc) {
    if (n <= 0 || n_center < 0 || n_center > n || !(rc > 0.0)) return NULL;
    double inv[9];
    int np = (pbc[0] != 0) + (pbc[1] != 0) + (pbc[2] != 0);
    if (inv3(cell, inv)) {
        if (np) return NULL;
        /* fully open boundaries: any non-singular frame works */
        double eye[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        memcpy(inv, eye, sizeof eye);
    }
    /* plane spacing d_k = 1/|row k of inv^T| = 1/|column k of inv| */
    int nb[3], ms[3];
    for (int k = 0; k < 3; ++k) {
        double cn = sqrt(inv[0 + k] * inv[0 + k] + inv[3 + k] * inv[3 + k] + inv[6 + k] * inv[6 + k]);
        double d = 1.0 / cn;
        if (pbc[k]) {
            nb[k] = (int)floor(d / rc); if (nb[k] < 1) nb[k] = 1; if (nb[k] > 256) nb[k] = 256;
            ms[k] = (int)floor(rc * nb[k] / d) + 1;
        } else { nb[k] = 1; ms[k] = 0; }
    }
    /* wrapped fractional coordinates, wrap shifts and bins */
    double *fw = (double *)malloc(sizeof(double) * 3 * n);
    int *sh = (int *)malloc(sizeof(int) * 3 * n);
    int *bin = (int *)malloc(sizeof(int) * n);
    int nbins = nb[0] * nb[1] * nb[2];
    int *bcnt = (int *)calloc((size_t)nbins + 1, sizeof(int));
    for (int i = 0; i < n; ++i) {
        int bb[3];
        for (int k = 0; k < 3; ++k) {
            double f = pos[3 * i] * inv[0 + k] + pos[3 * i + 1] * inv[3 + k] + pos[3 * i + 2] * inv[6 + k];
            if (pbc[k]) {
                double fl = floor(f);
                sh[3 * i + k] = -(int)fl;
                f -= fl;
                int b = (int)floor(f * nb[k]); if (b >= nb[k]) b = nb[k] - 1; if (b < 0) b = 0;
                bb[k] = b;
            } else { sh[3 * i + k] = 0; bb[k] = 0; }
            fw[3 * i + k] = f;
        }
        bin[i] = (bb[0] * nb[1] + bb[1]) * nb[2] + bb[2];
        bcnt[bin[i] + 1]++;
    }
    for (int b = 0; b < nbins; ++b) bcnt[b + 1] += bcnt[b];
    int *bidx = (int *)malloc(sizeof(int) * n);
    int *bcur = (int *)malloc(sizeof(int) * nbins);
    memcpy(bcur, bcnt, sizeof(int) * nbins);
    for (int i = 0; i < n; ++i) bidx[bcur[bin[i]]++] = i;

    so4o_nl *nl = (so4o_nl *)calloc(1, sizeof(so4o_nl));
    nl->n = n_center;
    nl->img_ptr = (int64_t *)calloc((size_t)n_center + 1, sizeof(int64_t));
    size_t cap = 1024, used = 0;
    cand_t *all = (cand_t *)malloc(sizeof(cand_t) * cap);
    size_t ccap = 256;
    cand_t *cl = (cand_t *)malloc(sizeof(cand_t) * ccap);
    for (int i = 0; i < n_center; ++i) {
        size_t nc = 0;
        int bi[3] = {bin[i] / (nb[1] * nb[2]), (bin[i] / nb[2]) % nb[1], bin[i] % nb[2]};
        for (int d0 = -ms[0]; d0 <= ms[0]; ++d0)
        for (int d1 = -ms[1]; d1 <= ms[1]; ++d1)
        for (int d2 = -ms[2]; d2 <= ms[2]; ++d2) {
            int dd[3] = {d0, d1, d2}, tb[3], img[3];
            for (int k = 0; k < 3; ++k) {
                int tt = bi[k] + dd[k];
                int w = ((tt % nb[k]) + nb[k]) % nb[k];
                img[k] = (tt - w) / nb[k];
                tb[k] = w;
            }
            int b = (tb[0] * nb[1] + tb[1]) * nb[2] + tb[2];
            for (int q = bcnt[b]; q < bcnt[b + 1]; ++q) {
                int j = bidx[q];
                int o[3];
                for (int k = 0; k < 3; ++k) o[k] = img[k] + sh[3 * j + k] - sh[3 * i + k];
                if (j == i && o[0] == 0 && o[1] == 0 && o[2] == 0) continue;
                double r[3];
                for (int c = 0; c < 3; ++c) {
                    double sc = ((double)o[0] * cell[c] + (double)o[1] * cell[3 + c]) + (double)o[2] * cell[6 + c];
                    r[c] = (pos[3 * j + c] + sc) - pos[3 * i + c];
                }
                double rr = sqrt((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
                if (!(rr < rc)) continue;
                if (nc == ccap) { ccap *= 2; cl = (cand_t *)realloc(cl, sizeof(cand_t) * ccap); }
                cand_t cd; cd.j = j; cd.o0 = o[0]; cd.o1 = o[1]; cd.o2 = o[2];
                cd.r[0] = r[0]; cd.r[1] = r[1]; cd.r[2] = r[2];
                cl[nc++] = cd;
            }
        }
        qsort(cl, nc, sizeof(cand_t), cand_cmp);
        if (used + nc > cap) { while (used + nc > cap) cap *= 2; all = (cand_t *)realloc(all, sizeof(cand_t) * cap); }
        memcpy(all + used, cl, sizeof(cand_t) * nc);
        used += nc;
        nl->img_ptr[i + 1] = (int64_t)used;
    }
    free(cl);
    nl->nimg = (int64_t)used;
    size_t ni = used ? used : 1;
    nl->img_j = (int32_t *)malloc(sizeof(int32_t) * ni);
    nl->img_off = (int32_t *)malloc(sizeof(int32_t) * 3 * ni);
    nl->img_r = (double *)malloc(sizeof(double) * 3 * ni);
    for (size_t m = 0; m < used; ++m) {
        nl->img_j[m] = all[m].j;
        nl->img_off[3 * m] = all[m].o0; nl->img_off[3 * m + 1] = all[m].o1; nl->img_off[3 * m + 2] = all[m].o2;
        for (int c = 0; c < 3; ++c) nl->img_r[3 * m + c] = all[m].r[c];
    }
    free(all);
    /* pairs: sorted unique j per centre, with (i,i) forced (SO4.py:250-266) */
    int64_t npair = 0;
    for (int i = 0; i < n_center; ++i) {
        int has_self = 0; int64_t u = 0;
        for (int64_t m = nl->img_ptr[i]; m < nl->img_ptr[i + 1]; ++m) {
            if (m == nl->img_ptr[i] || nl->img_j[m] != nl->img_j[m - 1]) u++;
            if (nl->img_j[m] == i) has_self = 1;
        }
        npair += u + (has_self ? 0 : 1);
    }
    nl->npair = npair;
    nl->pair_ptr = (int64_t *)calloc((size_t)n_center + 1, sizeof(int64_t));
    nl->seq = (int64_t *)malloc(sizeof(int64_t) * 2 * (npair ? npair : 1));
    nl->pair_img = (int64_t *)malloc(sizeof(int64_t) * (npair + 1));
    nl->nsite = (int64_t *)malloc(sizeof(int64_t) * (n_center ? n_center : 1));
    int64_t p = 0;
    for (int i = 0; i < n_center; ++i) {
        int64_t m = nl->img_ptr[i], me = nl->img_ptr[i + 1];
        int self_done = 0;
        while (m < me || !self_done) {
            int j = (m < me) ? nl->img_j[m] : 0x7fffffff;
            if (!self_done && i < j) {         /* (i,i) with no images */
                nl->seq[2 * p] = i; nl->seq[2 * p + 1] = i; nl->pair_img[p] = m;
                nl->nsite[i] = p; p++; self_done = 1;
                continue;
            }
            nl->seq[2 * p] = i; nl->seq[2 * p + 1] = j; nl->pair_img[p] = m;
            if (j == i) { nl->nsite[i] = p; self_done = 1; }
            while (m < me && nl->img_j[m] == j) m++;
            p++;
        }
        nl->pair_ptr[i + 1] = p;
    }
    nl->pair_img[npair] = nl->nimg;
    free(fw); free(sh); free(bin); free(bcnt); free(bidx); free(bcur);
    return nl;
}

/* ------------------------------------------------------------------ */
/* Driver: get_bispectrum_components, derivative + stress branch
 * (SO4.py:1409-1548), restated per centre atom.
 *   w_nb[j]   neighbour weight (SO4: atomic number; SNAP: weights[symbol])
 *   w_site[i] site weight      (SO4: atomic number; SNAP: 1)
 *   psi = rfac0 * pi * r / rc  (rfac0 = 1 for SO4)
 * Outputs (any may be NULL):
 *   x[n_center*nB]; dxdr[npair*nB*3]; rdxdr[npair*nB*9] = -bstress/vol;
 *   beta[n_center*nB] with forces[n*3] (-dE/dr) and vir[9] =
 *   sum_i beta_i . sum_{pairs of i} rdxdr  (the consumers' contraction).  */
typedef struct {
    int twol, cutoff_id, normalize_u;
    double rcut, rfac0, vol;
} so4o_params;

int so4o_compute(const so4o_params *prm, const so4o_nl *nl, int n_atoms, const double *pos,
                 const double *w_nb, const double *w_site, double *x, double *dxdr, double *rdxdr,
                 const double *beta, double *forces, double *vir, int nthreads) {
    tables_t T;
    if (tables_init(&T, prm->twol, prm->normalize_u)) return 1;
    const int nB = T.idxb_count, nU = T.idxu_count, nZ = T.idxz_count;
    const int n = nl->n;
    const double rc = prm->rcut, rfac0 = prm->rfac0, vol = prm->vol;
    const int cid = prm->cutoff_id;
    if (cid < 1 || cid > 7) { tables_free(&T); return 2; }
    int nth = 1;
#ifdef _OPENMP
    nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
#endif
    /* per-thread force / virial accumulators, reduced in thread order */
    double *facc = NULL, *vacc = NULL;
    if (beta) {
        facc = (double *)calloc((size_t)nth * 3 * n_atoms, sizeof(double));
        vacc = (double *)calloc((size_t)nth * 9, sizeof(double));
    }
    int err = 0;
    if (dxdr) memset(dxdr, 0, sizeof(double) * (size_t)nl->npair * nB * 3);
    if (rdxdr) memset(rdxdr, 0, sizeof(double) * (size_t)nl->npair * nB * 9);
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        cx *ut = (cx *)malloc(sizeof(cx) * nU);
        cx *u = (cx *)malloc(sizeof(cx) * nU);
        cx *du = (cx *)malloc(sizeof(cx) * 3 * nU);
        cx *zl = (cx *)malloc(sizeof(cx) * (nZ ? nZ : 1));
        double *tdb = (double *)malloc(sizeof(double) * 3 * nB);
        double *bl = (double *)malloc(sizeof(double) * nB);
        double *myf = facc ? facc + (size_t)tid * 3 * n_atoms : NULL;
        double *myv = vacc ? vacc + (size_t)tid * 9 : NULL;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int i = 0; i < n; ++i) {
            /* first pass (SO4.py:1480-1499): U_tot = sum_images sfac * (w_j U) */
            for (int e = 0; e < nU; ++e) ut[e] = cx_make(0.0, 0.0);
            for (int64_t m = nl->img_ptr[i]; m < nl->img_ptr[i + 1]; ++m) {
                double rx = nl->img_r[3 * m], ry = nl->img_r[3 * m + 1], rz = nl->img_r[3 * m + 2];
                double r = sqrt(rx * rx + ry * ry + rz * rz);
                if (r < 1e-8) continue;
                double psi = rfac0 * O_PI * r / rc;
                uarray(&T, rx, ry, rz, psi, r, u);
                double w = w_nb[nl->img_j[m]];
                double sf = sfac_fn(r, rc, cid);
                for (int e = 0; e < nU; ++e) ut[e] = cx_add(ut[e], cx_scale(cx_scale(u[e], w), sf));
            }
            /* self term, site weight, normalisation (SO4.py:1501-1505, 560-597) */
            {
                double fcut = sfac_fn(0.0, rc, cid);
                for (int e = 0; e < nU; ++e) u[e] = cx_make(0.0, 0.0);
                for (int l = 0; l <= T.twol; ++l) {
                    int llu = T.idxu_block[l];
                    for (int ma = 0; ma <= l; ++ma) { u[llu] = cx_make(fcut, 0.0); llu += l + 2; }
                }
                for (int e = 0; e < nU; ++e) ut[e] = cx_scale(cx_add(ut[e], cx_scale(u[e], w_site[i])), T.unorm[e]);
            }
            compute_z(&T, ut, zl);
            compute_b(&T, ut, zl, bl);
            if (x) for (int k = 0; k < nB; ++k) x[(size_t)i * nB + k] = bl[k];
            if (!dxdr && !rdxdr && !beta) continue;
            /* derivative pass (SO4.py:1510-1547) */
            const double *Ri = pos + 3 * i;
            int64_t nsite = nl->nsite[i];
            for (int64_t N = nl->pair_ptr[i]; N < nl->pair_ptr[i + 1]; ++N) {
                int J = (int)nl->seq[2 * N + 1];
                for (int64_t m = nl->pair_img[N]; m < nl->pair_img[N + 1]; ++m) {
                    double rx = nl->img_r[3 * m], ry = nl->img_r[3 * m + 1], rz = nl->img_r[3 * m + 2];
                    double r = sqrt(rx * rx + ry * ry + rz * rz);
                    if (r < 1e-8) continue;
                    double psi = rfac0 * O_PI * r / rc;
                    uarray(&T, rx, ry, rz, psi, r, u);
                    duarray(&T, rx, ry, rz, psi, r, u, du);
                    /* dudr (SO4.py:1001-1018), then * Weight * u_norm (:1450-1451) */
                    double sf = sfac_fn(r, rc, cid);
                    double ds = dsfac_fn(r, rc, cid);
                    double g[3] = {rx / r, ry / r, rz / r};
                    double W = w_nb[J];
                    for (int e = 0; e < nU; ++e)
                        for (int c = 0; c < 3; ++c) {
                            cx v = cx_add(cx_scale(du[3 * e + c], sf), cx_scale(u[e], ds * g[c]));
                            du[3 * e + c] = cx_scale(cx_scale(v, W), T.unorm[e]);
                        }
                    compute_db(&T, du, zl, tdb);
                    double Rj[3] = {rx + Ri[0], ry + Ri[1], rz + Ri[2]};
                    if (dxdr && J != i) {
                        double *ds_ = dxdr + (size_t)nsite * nB * 3, *dn = dxdr + (size_t)N * nB * 3;
                        for (int q = 0; q < 3 * nB; ++q) { ds_[q] -= tdb[q]; dn[q] += tdb[q]; }
                    }
                    if (rdxdr) {
                        /* bstress[nsite] += Ri (x) t ; bstress[N] -= Rj (x) t ; rdxdr = -bstress/vol */
                        double *rs = rdxdr + (size_t)nsite * nB * 9, *rn = rdxdr + (size_t)N * nB * 9;
                        for (int k = 0; k < nB; ++k)
                            for (int a = 0; a < 3; ++a)
                                for (int b = 0; b < 3; ++b) {
                                    rs[9 * k + 3 * a + b] += Ri[a] * tdb[3 * k + b];
                                    rn[9 * k + 3 * a + b] -= Rj[a] * tdb[3 * k + b];
                                }
                    }
                    if (beta) {
                        double gsum[3] = {0, 0, 0};
                        for (int k = 0; k < nB; ++k)
                            for (int c = 0; c < 3; ++c) gsum[c] += beta[(size_t)i * nB + k] * tdb[3 * k + c];
                        if (J != i)
                            for (int c = 0; c < 3; ++c) { myf[3 * J + c] -= gsum[c]; myf[3 * i + c] += gsum[c]; }
                        double rv[3] = {rx, ry, rz};
                        for (int a = 0; a < 3; ++a)
                            for (int b = 0; b < 3; ++b) myv[3 * a + b] += rv[a] * gsum[b] / vol;
                    }
                }
            }
        }
        free(ut); free(u); free(du); free(zl); free(tdb); free(bl);
    }
    if (rdxdr) {
        /* rdxdr currently holds bstress; the reference returns -bstress/vol (SO4.py:196) */
        size_t tot = (size_t)nl->npair * nB * 9;
        for (size_t q = 0; q < tot; ++q) rdxdr[q] = -rdxdr[q] / vol;
    }
    if (beta) {
        if (forces) {
            for (int q = 0; q < 3 * n_atoms; ++q) forces[q] = 0.0;
            for (int t = 0; t < nth; ++t)
                for (int q = 0; q < 3 * n_atoms; ++q) forces[q] += facc[(size_t)t * 3 * n_atoms + q];
        }
        if (vir) {
            for (int q = 0; q < 9; ++q) vir[q] = 0.0;
            for (int t = 0; t < nth; ++t) for (int q = 0; q < 9; ++q) vir[q] += vacc[t * 9 + q];
        }
    }
    free(facc); free(vacc);
    tables_free(&T);
    return err;
}
