// so4_nlist.cu -- cell-list neighbour search and (i, j) grouping.
//
// Replaces ase.neighborlist.NeighborList(rc/2 per atom, self_interaction=False,
// bothways=True, skin=0) and the grouping loop of
// pyxtal_ff/descriptors/SO4.py:211-287:
//   - every periodic image (j, o) with |pos[j] + o.cell - pos[i]| < rcut is a
//     neighbour of centre i, except (i, o = 0);
//   - the images of centre i are sorted by (j, o0, o1, o2); the pairs are the
//     sorted unique j plus a forced (i, i) pair (SO4.py:250-266).
// Atoms are binned on wrapped fractional coordinates (a bin is at least rcut
// thick along every periodic axis); the bin-offset range covers every image
// within rcut however small the cell is.  The image vector is evaluated from
// the ORIGINAL positions and the integer offset with every FP64 operation
// separately rounded, so it is reproducible bit for bit on any host.
#include <cmath>
#include <cstring>

#include "so4_common.cuh"

namespace {

constexpr int OFF_BIAS = 512;  // image offsets are packed in 10 bits each
constexpr int OFF_MAX = 511;

struct NLWork {
    int *status;
    int *bin_cnt;    // nbins + 1
    int *bin_start;  // nbins + 1
    int *bin_cur;    // nbins
    int *bin_atoms;  // natoms
    int *atom_bin;   // natoms
    int4 *atom_shift; // natoms: the cell shifts (x, y, z, 0) that wrap each atom into its cell
    int *cnt;        // natoms (image or pair counts)
    float4 *pos32;   // natoms: FP32 copy of the positions for the prefilter
    unsigned long long *keys;  // nimg, or natoms * slot_cap in the slot mode
    int64_t cap_img;           // capacity of the image arrays (fill / sort / rev)
    int64_t cap_pair;          // capacity of the pair arrays (pairs)
    int slot_cap;              // > 0: keys of atom a in [a slot_cap, (a + 1) slot_cap)
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t carve(NLWork &w, void *base, int natoms, int nbins, int64_t nimg) {
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *q = p ? p + off : nullptr;
        off += align256(bytes);
        return (void *)q;
    };
    w.status = (int *)take(SO4_WS_HEADER);
    w.bin_cnt = (int *)take(sizeof(int) * (nbins + 1));
    w.bin_start = (int *)take(sizeof(int) * (nbins + 1));
    w.bin_cur = (int *)take(sizeof(int) * (nbins + 1));
    w.bin_atoms = (int *)take(sizeof(int) * (natoms + 1));
    w.atom_bin = (int *)take(sizeof(int) * (natoms + 1));
    w.atom_shift = (int4 *)take(sizeof(int4) * (natoms + 1));
    w.cnt = (int *)take(sizeof(int) * (natoms + 1));
    w.pos32 = (float4 *)take(sizeof(float4) * (natoms + 1));
    w.keys = (unsigned long long *)take(sizeof(unsigned long long) * (nimg + 1));
    return off;
}

__device__ __forceinline__ void flag(int *status, int code) { atomicOr(status, 1 << code); }

// fractional coordinate k of a Cartesian point: f_k = sum_c r_c inv[c][k]
__device__ __forceinline__ double frac_k(const so4_geom &g, const double *r, int k) {
    return __dadd_rn(__dadd_rn(__dmul_rn(r[0], g.inv[k]), __dmul_rn(r[1], g.inv[3 + k])), __dmul_rn(r[2], g.inv[6 + k]));
}

// image vector (pos[j] + ((o0 a1 + o1 a2) + o2 a3)) - pos[i], every op rounded
__device__ __forceinline__ void image_vec(const so4_geom &g, const double *pi, const double *pj, int o0, int o1,
                                          int o2, double *r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double sc = __dadd_rn(__dadd_rn(__dmul_rn((double)o0, g.cell[c]), __dmul_rn((double)o1, g.cell[3 + c])),
                              __dmul_rn((double)o2, g.cell[6 + c]));
        r[c] = __dsub_rn(__dadd_rn(pj[c], sc), pi[c]);
    }
}

__device__ __forceinline__ double norm_rn(const double *r) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1])), __dmul_rn(r[2], r[2])));
}

// Exact membership test |r| < rcut in FP64.  Kept out of line so the compiler
// cannot if-convert it into the FP32 loop: FP64 runs at 1/64 of the FP32 rate
// here, and the test is needed only for the rare candidates in the rounding band.
__device__ __noinline__ bool exact_inside(const so4_geom &g, const double *pi, const double *pos, int j, int o0, int o1,
                                          int o2, double rcut) {
    const double pj[3] = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
    double r[3];
    image_vec(g, pi, pj, o0, o1, o2, r);
    return norm_rn(r) < rcut;
}

__global__ void k_bin(const so4_geom *geom, const double *pos, const int *astruct, int natoms, NLWork w) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    const so4_geom &g = geom[astruct[a]];
    const double r[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    if (!isfinite(r[0]) || !isfinite(r[1]) || !isfinite(r[2])) flag(w.status, SO4_ERR_NONFINITE);
    int b[3], shift[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double f = frac_k(g, r, k);
        int sh = 0;
        int bk = 0;
        if (g.pbc[k]) {
            double fl = floor(f);
            if (!isfinite(fl)) fl = 0.0;
            sh = -(int)fl;
            f = f - fl;
            bk = (int)floor(f * g.nbin[k]);
            bk = min(max(bk, 0), g.nbin[k] - 1);
        }
        b[k] = bk;
        shift[k] = sh;
    }
    w.atom_shift[a] = make_int4(shift[0], shift[1], shift[2], 0);
    const int bin = g.bin_base + (b[0] * g.nbin[1] + b[1]) * g.nbin[2] + b[2];
    w.atom_bin[a] = bin;
    w.pos32[a] = make_float4((float)r[0], (float)r[1], (float)r[2], 0.f);
    atomicAdd(&w.bin_cnt[bin], 1);
}

__global__ void k_bin_fill(const int *astruct, int natoms, NLWork w) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    const int bin = w.atom_bin[a];
    const int slot = atomicAdd(&w.bin_cur[bin], 1);
    w.bin_atoms[w.bin_start[bin] + slot] = a;
}

// single-CTA exclusive scan: out[0..n] from in[0..n-1].  Chunks of 4096 values (four per
// thread, coalesced), warp-shuffle scans inside, a running carry across chunks; the next
// chunk's values are loaded before the current one is scanned.  With chained != 0 the scan
// continues a previous one: out[0] already holds the running total before in[0] (ranges of
// centres scanned one after another).
__global__ void __launch_bounds__(1024) k_scan(const int *in, int *out, int n, int chained = 0) {
    __shared__ int wsum[32];
    __shared__ int carry_s;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    if (t == 0) carry_s = chained ? out[0] : 0;
    int nv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) nv[q] = (4 * t + q < n) ? __ldg(in + 4 * t + q) : 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4096) {
        int v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[q] = nv[q];
            const int i = base + 4096 + 4 * t + q;
            nv[q] = (i < n) ? __ldg(in + i) : 0;
        }
        const int tot = v[0] + v[1] + v[2] + v[3];
        int inc = tot;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += y;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane];
            int winc = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, winc, d);
                if (lane >= d) winc += y;
            }
            wsum[lane] = winc - w;  // exclusive warp offsets
        }
        __syncthreads();
        int run = carry_s + wsum[wid] + inc - tot;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = base + 4 * t + q;
            if (i < n) out[i] = run;
            run += v[q];
        }
        __syncthreads();
        if (t == 1023) carry_s = run;
        __syncthreads();
    }
    if (t == 0) out[n] = carry_s;
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// pair_img[P] = M (both totals read on the device, clamped to the capacities)
__global__ void k_sentinel(const int32_t *img_ptr, const int32_t *pair_ptr, int natoms, int32_t *pair_img, NLWork w) {
    const int64_t P = pair_ptr[natoms], M = img_ptr[natoms];
    if (P <= w.cap_pair) pair_img[P] = (int32_t)(M <= w.cap_img ? M : w.cap_img);
}

__global__ void k_summary(const int32_t *img_ptr, const int32_t *pair_ptr, int natoms, const int *status, int *out) {
    out[0] = natoms > 0 ? img_ptr[natoms] : 0;
    out[1] = (natoms > 0 && pair_ptr) ? pair_ptr[natoms] : 0;
    out[2] = *status;
}

// After the summary has recorded the true totals: if a capacity was exceeded (or an
// offset did not fit), empty every image and pair range, so that kernels enqueued
// behind the list without a host check (a captured step) read nothing out of bounds.
__global__ void k_clamp(int32_t *img_ptr, int32_t *pair_ptr, int natoms, const int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > natoms || !(*status & (1 << SO4_ERR_CAPACITY))) return;
    img_ptr[i] = 0;
    if (pair_ptr) pair_ptr[i] = 0;
}

// The range form of k_clamp: after a range's sort, if any capacity was exceeded so far,
// empty the range's image ranges (img_ptr[a0 .. a1]) before work on them is enqueued.
__global__ void k_clamp_range(int32_t *img_ptr, int a0, int a1, const int *status) {
    const int i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > a1 || !(*(volatile const int *)status & (1 << SO4_ERR_CAPACITY))) return;
    img_ptr[i] = 0;
}

// One warp per centre.  MODE 0: count images into w.cnt.  MODE 1: write the
// packed (j, o) keys into w.keys[img_ptr[a] ...] (unsorted; slots are taken with
// a shared-memory counter, the order is fixed later by k_sort).
// Each candidate is classified in FP32 with a margin delta that bounds the FP32
// rounding of the image vector (about 6 ulp of the magnitudes involved, here
// taken 8x larger plus an absolute 1e-5 A): |r| > rcut + delta is surely out,
// |r| < rcut - delta surely in, and only the band in between is decided by the
// exact FP64 test, so the accepted set is exactly the FP64 one while FP64 work
// (1/64 of the FP32 rate on this GPU) is almost never issued.
template <int MODE>
__global__ void k_scan_images(const so4_geom *geom, const double *pos, const int *astruct, int natoms,
                              double rcut, const int32_t *img_ptr, NLWork w, int a0 = 0) {
    // centres a0 .. natoms - 1 (a range of the list when a0 > 0)
    __shared__ int s_cnt[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int a = a0 + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (MODE >= 1 && lane == 0) s_cnt[wib] = 0;
    __syncwarp();
    if (a >= natoms) return;
    const so4_geom &g = geom[astruct[a]];
    const double pi[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    const float4 pi32 = w.pos32[a];
    float c32[9], amax = 0.f;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        c32[q] = (float)g.cell[q];
        amax = fmaxf(amax, fabsf(c32[q]));
    }
    const float rc32 = (float)rcut;
    const float pimag = fmaxf(fabsf(pi32.x), fmaxf(fabsf(pi32.y), fabsf(pi32.z)));
    const int lb = w.atom_bin[a] - g.bin_base;
    const int bi[3] = {lb / (g.nbin[1] * g.nbin[2]), (lb / g.nbin[2]) % g.nbin[1], lb % g.nbin[2]};
    const int4 si = w.atom_shift[a];
    const int n1 = 2 * g.mshift[1] + 1, n2 = 2 * g.mshift[2] + 1;
    const int nq = (2 * g.mshift[0] + 1) * n1 * n2;
    const int64_t base = (MODE == 1) ? (int64_t)img_ptr[a] : ((MODE == 2) ? (int64_t)a * w.slot_cap : 0);
    int mine = 0;
    for (int q = lane; q < nq; q += 32) {
        const int d[3] = {q / (n1 * n2) - g.mshift[0], (q / n2) % n1 - g.mshift[1], q % n2 - g.mshift[2]};
        int tb[3], img[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // the wrapped bin and the image floor(t / nb), by whole periods: t lies within
            // mshift of [0, nb), so one step at most unless the cell is thinner than rcut
            const int nb = g.nbin[k];
            int wk = bi[k] + d[k], im = 0;
            while (wk < 0) {
                wk += nb;
                --im;
            }
            while (wk >= nb) {
                wk -= nb;
                ++im;
            }
            tb[k] = wk;
            img[k] = im;
        }
        const int bin = g.bin_base + (tb[0] * g.nbin[1] + tb[1]) * g.nbin[2] + tb[2];
        // the next candidate's index is read one ahead, so its loads do not wait on it
        const int s0 = w.bin_start[bin], s1 = w.bin_start[bin + 1];
        int jn = (s0 < s1) ? w.bin_atoms[s0] : 0;
        for (int s = s0; s < s1; ++s) {
            const int j = jn;
            if (s + 1 < s1) jn = w.bin_atoms[s + 1];
            const int4 sj = w.atom_shift[j];
            const int o[3] = {img[0] + sj.x - si.x, img[1] + sj.y - si.y, img[2] + sj.z - si.z};
            if (j == a && o[0] == 0 && o[1] == 0 && o[2] == 0) continue;
            // FP32 prefilter
            const float4 pj32 = w.pos32[j];
            const float f0 = (float)o[0], f1 = (float)o[1], f2 = (float)o[2];
            const float rx = (pj32.x + (f0 * c32[0] + f1 * c32[3] + f2 * c32[6])) - pi32.x;
            const float ry = (pj32.y + (f0 * c32[1] + f1 * c32[4] + f2 * c32[7])) - pi32.y;
            const float rz = (pj32.z + (f0 * c32[2] + f1 * c32[5] + f2 * c32[8])) - pi32.z;
            const float mag = pimag + fmaxf(fabsf(pj32.x), fmaxf(fabsf(pj32.y), fabsf(pj32.z))) +
                              (fabsf(f0) + fabsf(f1) + fabsf(f2)) * amax;
            const float delta = 2e-6f * mag + 1e-5f;
            const float d2 = rx * rx + ry * ry + rz * rz;
            const float hi = rc32 + delta, lo = rc32 - delta;
            if (d2 > hi * hi) continue;            // surely outside
            if (!(lo > 0.f && d2 < lo * lo)) {     // within the rounding band: decide in FP64
                if (!exact_inside(g, pi, pos, j, o[0], o[1], o[2], rcut)) continue;
            }
            if (MODE >= 1) {
                if (abs(o[0]) > OFF_MAX || abs(o[1]) > OFF_MAX || abs(o[2]) > OFF_MAX) {
                    flag(w.status, SO4_ERR_CAPACITY);
                    continue;
                }
                const unsigned long long key = ((unsigned long long)(unsigned)j << 30) |
                                               ((unsigned long long)(o[0] + OFF_BIAS) << 20) |
                                               ((unsigned long long)(o[1] + OFF_BIAS) << 10) |
                                               (unsigned long long)(o[2] + OFF_BIAS);
                const int slot = atomicAdd(&s_cnt[wib], 1);
                if (MODE == 1) {
                    if (base + slot < w.cap_img) w.keys[base + slot] = key;
                    else flag(w.status, SO4_ERR_CAPACITY);
                } else if (slot < w.slot_cap) {
                    w.keys[base + slot] = key;
                } else {
                    flag(w.status, SO4_ERR_SLOTS);
                    flag(w.status, SO4_ERR_CAPACITY);
                }
            }
            ++mine;
        }
    }
    if (MODE == 0 || MODE == 2) {
        int tot = mine;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, d);
        if (lane == 0) {
            w.cnt[a] = tot;
            if (tot == 0) flag(w.status, SO4_ERR_NO_NEIGHBOR);
            if (MODE == 2) atomicMax(w.status + 8, tot);
        }
    }
}

// One warp per centre: rank-sort the keys, write the sorted images and count pairs.
__global__ void k_sort(const so4_geom *geom, const double *pos, const int *astruct, int natoms,
                       const int32_t *img_ptr, int32_t *img_j, int32_t *img_off, double *img_r, NLWork w,
                       int a0 = 0) {
    // centres a0 .. natoms - 1
    const int lane = threadIdx.x & 31;
    const int a = a0 + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (a >= natoms) return;
    const so4_geom &g = geom[astruct[a]];
    const int p0 = img_ptr[a], p1 = img_ptr[a + 1];
    if (p1 > w.cap_img || (w.slot_cap > 0 && p1 - p0 > w.slot_cap)) {
        // the arrays (or this atom's key slots) are too small for this call; the host grows them
        if (lane == 0) {
            w.cnt[a] = 1;
            flag(w.status, SO4_ERR_CAPACITY);
        }
        return;
    }
    const double pi[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    // For the offset (0, 0, 0) image_vec's o . cell is, per component, a signed zero z: 0
    // times a cell entry keeps the entry's sign, and the sum is -0 only if all three terms
    // are.  p_j + z is then p_j itself, except -0 + +0 = +0, so r = p_j' - p_i with that one
    // sign fix-up on the bits rounds exactly as image_vec does, with one FP64 operation per
    // component instead of six (the FP64 pipe runs at 1/64 of FP32 on this GPU); in a cell
    // larger than twice the cutoff almost every image has the zero offset.
    bool zneg[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        zneg[c] = signbit(g.cell[c]) && signbit(g.cell[3 + c]) && signbit(g.cell[6 + c]);
    // keys of this atom: compact at [p0, p1), or in its own slots
    const unsigned long long *kk = w.keys + ((w.slot_cap > 0) ? (int64_t)a * w.slot_cap - p0 : 0);
    for (int q = p0 + lane; q < p1; q += 32) {
        const unsigned long long kq = kk[q];
        int rank = 0;
        for (int p = p0; p < p1; ++p) rank += (kk[p] < kq) ? 1 : 0;
        const int dst = p0 + rank;
        const int j = (int)(kq >> 30);
        const int o0 = (int)((kq >> 20) & 1023) - OFF_BIAS;
        const int o1 = (int)((kq >> 10) & 1023) - OFF_BIAS;
        const int o2 = (int)(kq & 1023) - OFF_BIAS;
        img_j[dst] = j;
        img_off[3 * dst] = o0;
        img_off[3 * dst + 1] = o1;
        img_off[3 * dst + 2] = o2;
        const double pj[3] = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
        double r[3];
        if ((o0 | o1 | o2) == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double p = pj[c];
                if (!zneg[c] && __double_as_longlong(p) == (long long)0x8000000000000000ULL) p = 0.0;  // -0 + +0
                r[c] = __dsub_rn(p, pi[c]);
            }
        } else {
            image_vec(g, pi, pj, o0, o1, o2, r);
        }
        img_r[3 * dst] = r[0];
        img_r[3 * dst + 1] = r[1];
        img_r[3 * dst + 2] = r[2];
    }
    __syncwarp();
    __threadfence_block();
    int uniq = 0, self = 0;
    for (int q = p0 + lane; q < p1; q += 32) {
        const int j = img_j[q];
        if (q == p0 || img_j[q - 1] != j) ++uniq;
        if (j == a) self = 1;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        uniq += __shfl_xor_sync(0xffffffffu, uniq, d);
        self |= __shfl_xor_sync(0xffffffffu, self, d);
    }
    if (lane == 0) w.cnt[a] = uniq + (self ? 0 : 1);
}

// One thread per centre: emit its pairs in (sorted j, with (i,i) forced) order.
__global__ void k_pairs(const so4_geom *geom, const int *astruct, int natoms, const int32_t *img_ptr,
                        const int32_t *img_j, const int32_t *pair_ptr, int64_t *seq, int32_t *pair_img,
                        int32_t *nsite, int32_t *img_pair, NLWork w) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms) return;
    if (img_ptr[a + 1] > w.cap_img || pair_ptr[a + 1] > w.cap_pair) {
        flag(w.status, SO4_ERR_CAPACITY);
        return;
    }
    const int base = geom[astruct[a]].atom_base;
    int p = pair_ptr[a];
    int m = img_ptr[a];
    const int me = img_ptr[a + 1];
    bool self_done = false;
    while (m < me || !self_done) {
        const int j = (m < me) ? img_j[m] : 0x7fffffff;
        if (!self_done && a < j) {
            seq[2 * p] = a - base;
            seq[2 * p + 1] = a - base;
            pair_img[p] = m;
            nsite[a] = p;
            ++p;
            self_done = true;
            continue;
        }
        seq[2 * p] = a - base;
        seq[2 * p + 1] = j - base;
        pair_img[p] = m;
        if (j == a) {
            nsite[a] = p;
            self_done = true;
        }
        while (m < me && img_j[m] == j) {
            img_pair[m] = p;
            ++m;
        }
        ++p;
    }
}

// One thread per image: index of the reverse image (i, -o) in the list of j.
__global__ void k_rev(const int *astruct, int natoms, const int32_t *img_ptr, const int32_t *img_j,
                      const int32_t *img_off, const int32_t *img_pair, int64_t nimg, const int64_t *seq,
                      const so4_geom *geom, int32_t *img_rev, NLWork w) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // after an overflow the pair arrays are incomplete: nothing here may be read
    if (*(volatile int *)w.status & (1 << SO4_ERR_CAPACITY)) return;
    const int mt = img_ptr[natoms];
    if (m >= nimg || m >= mt) return;
    const int j = img_j[m];
    int a;
    if (seq) {
        const int p = img_pair[m];
        a = (int)seq[2 * p] + geom[astruct[j]].atom_base;
    } else {
        // no pair arrays: the centre is the largest i with img_ptr[i] <= m (img_ptr[0] = 0),
        // searched from the proportional guess outwards, then by bisection
        const int g = min(max((int)((m * natoms) / (mt > 0 ? mt : 1)), 0), natoms - 1);
        int lo, hi, step = 1;  // img_ptr[lo] <= m < img_ptr[hi], img_ptr[natoms] = mt > m
        if (img_ptr[g] <= m) {
            lo = g;
            hi = g + 1;
            while (hi < natoms && img_ptr[hi] <= m) {
                lo = hi;
                step <<= 1;
                hi = min(lo + step, natoms);
            }
        } else {
            hi = g;
            lo = g - 1;  // g > 0 here
            while (lo > 0 && img_ptr[lo] > m) {
                hi = lo;
                step <<= 1;
                lo = max(hi - step, 0);
            }
        }
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (img_ptr[mid] <= m)
                lo = mid;
            else
                hi = mid;
        }
        a = lo;
    }
    const int t0 = -img_off[3 * m], t1 = -img_off[3 * m + 1], t2 = -img_off[3 * m + 2];
    int lo = img_ptr[j], hi = img_ptr[j + 1] - 1, found = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int jj = img_j[mid];
        const int c0 = img_off[3 * mid], c1 = img_off[3 * mid + 1], c2 = img_off[3 * mid + 2];
        int cmp;
        if (jj != a) cmp = jj < a ? -1 : 1;
        else if (c0 != t0) cmp = c0 < t0 ? -1 : 1;
        else if (c1 != t1) cmp = c1 < t1 ? -1 : 1;
        else if (c2 != t2) cmp = c2 < t2 ? -1 : 1;
        else cmp = 0;
        if (cmp == 0) {
            found = mid;
            break;
        }
        if (cmp < 0) lo = mid + 1;
        else hi = mid - 1;
    }
    if (found < 0) flag(w.status, SO4_ERR_REVERSE);
    img_rev[m] = found < 0 ? (int32_t)m : found;
}

}  // namespace

extern "C" int so4_geometry(const double *h_cells, const int *h_pbc, const int *h_atom_ptr, int nstruct, double rcut,
                            so4_geom *h_geom, int *h_nbins_total) {
    if (!h_cells || !h_pbc || !h_atom_ptr || !h_geom || nstruct < 0) return SO4_ERR_ARG;
    if (!(rcut > 0.0) || !std::isfinite(rcut)) return SO4_ERR_ARG;
    long long nbins = 0;
    for (int s = 0; s < nstruct; ++s) {
        so4_geom &g = h_geom[s];
        std::memset(&g, 0, sizeof g);
        const double *m = h_cells + 9 * s;
        for (int q = 0; q < 9; ++q) {
            if (!std::isfinite(m[q])) return SO4_ERR_NONFINITE;
            g.cell[q] = m[q];
        }
        int np = 0;
        for (int k = 0; k < 3; ++k) {
            g.pbc[k] = h_pbc[3 * s + k] ? 1 : 0;
            np += g.pbc[k];
        }
        const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                           m[2] * (m[3] * m[7] - m[4] * m[6]);
        g.vol = std::fabs(det);
        if (!(std::fabs(det) > 1e-300)) {
            if (np) return SO4_ERR_ARG;
            for (int q = 0; q < 9; ++q) g.inv[q] = (q % 4 == 0) ? 1.0 : 0.0;
        } else {
            g.inv[0] = (m[4] * m[8] - m[5] * m[7]) / det;
            g.inv[1] = (m[2] * m[7] - m[1] * m[8]) / det;
            g.inv[2] = (m[1] * m[5] - m[2] * m[4]) / det;
            g.inv[3] = (m[5] * m[6] - m[3] * m[8]) / det;
            g.inv[4] = (m[0] * m[8] - m[2] * m[6]) / det;
            g.inv[5] = (m[2] * m[3] - m[0] * m[5]) / det;
            g.inv[6] = (m[3] * m[7] - m[4] * m[6]) / det;
            g.inv[7] = (m[1] * m[6] - m[0] * m[7]) / det;
            g.inv[8] = (m[0] * m[4] - m[1] * m[3]) / det;
        }
        for (int k = 0; k < 3; ++k) {
            if (g.pbc[k]) {
                const double cn =
                    std::sqrt(g.inv[k] * g.inv[k] + g.inv[3 + k] * g.inv[3 + k] + g.inv[6 + k] * g.inv[6 + k]);
                const double d = 1.0 / cn;  // spacing of the lattice planes normal to axis k
                int nb = (int)std::floor(d / rcut);
                nb = std::max(1, std::min(nb, 256));
                g.nbin[k] = nb;
                g.mshift[k] = (int)std::floor(rcut * nb / d + 1e-9) + 1;
                if (g.mshift[k] > OFF_MAX / 2) return SO4_ERR_CAPACITY;
            } else {
                g.nbin[k] = 1;
                g.mshift[k] = 0;
            }
        }
        g.bin_base = (int)nbins;
        nbins += (long long)g.nbin[0] * g.nbin[1] * g.nbin[2];
        if (nbins > (1LL << 30)) return SO4_ERR_CAPACITY;
        g.atom_base = h_atom_ptr[s];
        g.natoms = h_atom_ptr[s + 1] - h_atom_ptr[s];
        if (g.natoms < 0) return SO4_ERR_ARG;
    }
    if (h_nbins_total) *h_nbins_total = (int)nbins;
    return SO4_OK;
}

extern "C" size_t so4_nl_workspace_size(int natoms, int nbins_total, int64_t nimg) {
    NLWork w;
    return carve(w, nullptr, natoms, nbins_total, nimg);
}

extern "C" int so4_nl_count(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_astruct,
                            int natoms, double rcut, int32_t *d_img_ptr, void *d_work, size_t work_bytes,
                            void *stream) {
    if (natoms < 0 || nstruct < 0 || nbins < 0 || !d_work) return SO4_ERR_ARG;
    NLWork w;
    if (carve(w, nullptr, natoms, nbins, 0) > work_bytes) return SO4_ERR_WORKSPACE;
    carve(w, d_work, natoms, nbins, 0);
    w.cap_img = 0;
    w.cap_pair = 0;
    w.slot_cap = 0;
    cudaStream_t st = (cudaStream_t)stream;
    SO4_CUDA_TRY(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    if (natoms == 0) {
        k_set_int<<<1, 1, 0, st>>>(d_img_ptr, 0);
        so4_count_launch();
        return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    }
    SO4_CUDA_TRY(cudaMemsetAsync(w.bin_cnt, 0, sizeof(int) * (nbins + 1), st));
    SO4_CUDA_TRY(cudaMemsetAsync(w.bin_cur, 0, sizeof(int) * (nbins + 1), st));
    const int tb = 256;
    k_bin<<<(natoms + tb - 1) / tb, tb, 0, st>>>(d_geom, d_pos, d_astruct, natoms, w);
    so4_count_launch();
    k_scan<<<1, 1024, 0, st>>>(w.bin_cnt, w.bin_start, nbins);
    so4_count_launch();
    k_bin_fill<<<(natoms + tb - 1) / tb, tb, 0, st>>>(d_astruct, natoms, w);
    so4_count_launch();
    const int warps = 8;
    k_scan_images<0><<<(natoms + warps - 1) / warps, 32 * warps, 0, st>>>(d_geom, d_pos, d_astruct, natoms, rcut,
                                                                          nullptr, w);
    so4_count_launch();
    k_scan<<<1, 1024, 0, st>>>(w.cnt, d_img_ptr, natoms);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_fill(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_astruct,
                           int natoms, double rcut, const int32_t *d_img_ptr, int64_t nimg, int32_t *d_img_j,
                           int32_t *d_img_off, double *d_img_r, int32_t *d_pair_ptr, void *d_work,
                           size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nimg < 0 || !d_work) return SO4_ERR_ARG;
    if (nimg > 0x7fffffff) return SO4_ERR_CAPACITY;
    NLWork w;
    if (carve(w, nullptr, natoms, nbins, nimg) > work_bytes) return SO4_ERR_WORKSPACE;
    carve(w, d_work, natoms, nbins, nimg);
    w.cap_img = nimg;
    w.cap_pair = 0;
    w.slot_cap = 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (natoms == 0) {
        k_set_int<<<1, 1, 0, st>>>(d_pair_ptr, 0);
        so4_count_launch();
        return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    }
    const int warps = 8;
    const int grid = (natoms + warps - 1) / warps;
    k_scan_images<1><<<grid, 32 * warps, 0, st>>>(d_geom, d_pos, d_astruct, natoms, rcut, d_img_ptr, w);
    so4_count_launch();
    k_sort<<<grid, 32 * warps, 0, st>>>(d_geom, d_pos, d_astruct, natoms, d_img_ptr, d_img_j, d_img_off, d_img_r, w);
    so4_count_launch();
    k_scan<<<1, 1024, 0, st>>>(w.cnt, d_pair_ptr, natoms);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

static int one_pass_work(NLWork &w, int natoms, int nbins, int slot_cap, void *d_work, size_t work_bytes) {
    const int64_t nkeys = (int64_t)natoms * slot_cap;
    if (carve(w, nullptr, natoms, nbins, nkeys) > work_bytes) return SO4_ERR_WORKSPACE;
    carve(w, d_work, natoms, nbins, nkeys);
    w.cap_img = 0;
    w.cap_pair = 0;
    w.slot_cap = slot_cap;
    return SO4_OK;
}

extern "C" int so4_nl_bins(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_astruct,
                           int natoms, int slot_cap, void *d_work, size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nbins < 0 || slot_cap <= 0 || !d_work) return SO4_ERR_ARG;
    NLWork w;
    int rc = one_pass_work(w, natoms, nbins, slot_cap, d_work, work_bytes);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    SO4_CUDA_TRY(cudaMemsetAsync(w.status, 0, 9 * sizeof(int), st));  // status, summary, largest count
    if (natoms == 0) return SO4_OK;
    SO4_CUDA_TRY(cudaMemsetAsync(w.bin_cnt, 0, sizeof(int) * (nbins + 1), st));
    SO4_CUDA_TRY(cudaMemsetAsync(w.bin_cur, 0, sizeof(int) * (nbins + 1), st));
    const int tb = 256;
    k_bin<<<(natoms + tb - 1) / tb, tb, 0, st>>>(d_geom, d_pos, d_astruct, natoms, w);
    so4_count_launch();
    k_scan<<<1, 1024, 0, st>>>(w.bin_cnt, w.bin_start, nbins);
    so4_count_launch();
    k_bin_fill<<<(natoms + tb - 1) / tb, tb, 0, st>>>(d_astruct, natoms, w);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_count_keys_range(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos,
                                       const int *d_astruct, int natoms, double rcut, int slot_cap, int a0, int a1,
                                       void *d_work, size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nbins < 0 || slot_cap <= 0 || !d_work) return SO4_ERR_ARG;
    if (a0 < 0 || a1 < a0 || a1 > natoms) return SO4_ERR_ARG;
    NLWork w;
    int rc = one_pass_work(w, natoms, nbins, slot_cap, d_work, work_bytes);
    if (rc) return rc;
    if (a1 == a0) return SO4_OK;
    const int warps = 8;
    k_scan_images<2><<<(a1 - a0 + warps - 1) / warps, 32 * warps, 0, (cudaStream_t)stream>>>(
        d_geom, d_pos, d_astruct, a1, rcut, nullptr, w, a0);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_scan_range(int natoms, int nbins, int slot_cap, int a0, int a1, int32_t *d_img_ptr,
                                 void *d_work, size_t work_bytes, void *stream) {
    if (natoms < 0 || nbins < 0 || slot_cap <= 0 || !d_work || !d_img_ptr) return SO4_ERR_ARG;
    if (a0 < 0 || a1 < a0 || a1 > natoms) return SO4_ERR_ARG;
    NLWork w;
    int rc = one_pass_work(w, natoms, nbins, slot_cap, d_work, work_bytes);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (a1 == a0) {
        if (a0 == 0) {
            k_set_int<<<1, 1, 0, st>>>(d_img_ptr, 0);
            so4_count_launch();
        }
        return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    }
    k_scan<<<1, 1024, 0, st>>>(w.cnt + a0, d_img_ptr + a0, a1 - a0, a0 > 0 ? 1 : 0);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_count_keys(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos,
                                 const int *d_astruct, int natoms, double rcut, int slot_cap, int32_t *d_img_ptr,
                                 void *d_work, size_t work_bytes, void *stream) {
    int rc = so4_nl_bins(d_geom, nstruct, nbins, d_pos, d_astruct, natoms, slot_cap, d_work, work_bytes, stream);
    if (!rc) rc = so4_nl_count_keys_range(d_geom, nstruct, nbins, d_pos, d_astruct, natoms, rcut, slot_cap, 0, natoms,
                                          d_work, work_bytes, stream);
    if (!rc && d_img_ptr) rc = so4_nl_scan_range(natoms, nbins, slot_cap, 0, natoms, d_img_ptr, d_work, work_bytes, stream);
    else if (!rc) rc = SO4_ERR_ARG;
    return rc;
}

extern "C" int so4_nl_sort_range(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos,
                                 const int *d_astruct, int natoms, int a0, int a1, int32_t *d_img_ptr, int64_t nimg,
                                 int slot_cap, int32_t *d_img_j, int32_t *d_img_off, double *d_img_r, void *d_work,
                                 size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nimg < 0 || slot_cap <= 0 || !d_work || !d_img_ptr) return SO4_ERR_ARG;
    if (a0 < 0 || a1 < a0 || a1 > natoms) return SO4_ERR_ARG;
    if (nimg > 0x7fffffff) return SO4_ERR_CAPACITY;
    NLWork w;
    int rc = one_pass_work(w, natoms, nbins, slot_cap, d_work, work_bytes);
    if (rc) return rc;
    w.cap_img = nimg;
    if (a1 == a0) return SO4_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int warps = 8;
    k_sort<<<(a1 - a0 + warps - 1) / warps, 32 * warps, 0, st>>>(d_geom, d_pos, d_astruct, a1, d_img_ptr, d_img_j,
                                                                 d_img_off, d_img_r, w, a0);
    so4_count_launch();
    k_clamp_range<<<(a1 - a0 + 1 + 255) / 256, 256, 0, st>>>(d_img_ptr, a0, a1, w.status);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_sort(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos,
                           const int *d_astruct, int natoms, const int32_t *d_img_ptr, int64_t nimg, int slot_cap,
                           int32_t *d_img_j, int32_t *d_img_off, double *d_img_r, int32_t *d_pair_ptr,
                           void *d_work, size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nimg < 0 || slot_cap <= 0 || !d_work) return SO4_ERR_ARG;
    if (nimg > 0x7fffffff) return SO4_ERR_CAPACITY;
    const int64_t nkeys = (int64_t)natoms * slot_cap;
    NLWork w;
    if (carve(w, nullptr, natoms, nbins, nkeys) > work_bytes) return SO4_ERR_WORKSPACE;
    carve(w, d_work, natoms, nbins, nkeys);
    w.cap_img = nimg;
    w.cap_pair = 0;
    w.slot_cap = slot_cap;
    cudaStream_t st = (cudaStream_t)stream;
    if (natoms == 0) {
        k_set_int<<<1, 1, 0, st>>>(d_pair_ptr, 0);
        so4_count_launch();
        return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    }
    const int warps = 8;
    const int grid = (natoms + warps - 1) / warps;
    k_sort<<<grid, 32 * warps, 0, st>>>(d_geom, d_pos, d_astruct, natoms, d_img_ptr, d_img_j, d_img_off, d_img_r, w);
    so4_count_launch();
    k_scan<<<1, 1024, 0, st>>>(w.cnt, d_pair_ptr, natoms);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_nl_pairs(const so4_geom *d_geom, int nstruct, const int *d_astruct, int natoms,
                            const int32_t *d_img_ptr, int64_t nimg, const int32_t *d_img_j, const int32_t *d_img_off,
                            const int32_t *d_pair_ptr, int64_t npair, int64_t *d_seq, int32_t *d_pair_img,
                            int32_t *d_nsite, int32_t *d_img_pair, int32_t *d_img_rev, void *d_work,
                            size_t work_bytes, void *stream) {
    if (natoms < 0 || nstruct < 0 || nimg < 0 || npair < 0 || !d_work) return SO4_ERR_ARG;
    if (work_bytes < SO4_WS_HEADER) return SO4_ERR_WORKSPACE;
    NLWork w;
    std::memset(&w, 0, sizeof w);
    w.status = (int *)d_work;
    w.cap_img = nimg;
    w.cap_pair = npair;
    cudaStream_t st = (cudaStream_t)stream;
    if (natoms == 0) {
        if (d_pair_img) {
            k_set_int<<<1, 1, 0, st>>>(d_pair_img, 0);
            so4_count_launch();
        }
        return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    }
    const bool pairs = d_seq && d_pair_img && d_nsite && d_img_pair;
    if (pairs) {
        k_sentinel<<<1, 1, 0, st>>>(d_img_ptr, d_pair_ptr, natoms, d_pair_img, w);
        so4_count_launch();
        const int tb = 128;
        k_pairs<<<(natoms + tb - 1) / tb, tb, 0, st>>>(d_geom, d_astruct, natoms, d_img_ptr, d_img_j, d_pair_ptr,
                                                       d_seq, d_pair_img, d_nsite, d_img_pair, w);
        so4_count_launch();
    }
    if (nimg > 0 && d_img_rev) {
        k_rev<<<(unsigned)((nimg + 255) / 256), 256, 0, st>>>(d_astruct, natoms, d_img_ptr, d_img_j, d_img_off,
                                                              d_img_pair, nimg, pairs ? d_seq : nullptr, d_geom,
                                                              d_img_rev, w);
        so4_count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_status_read(const void *d_work, size_t work_bytes, void *stream, int *h_status) {
    if (!d_work || !h_status || work_bytes < sizeof(int)) return SO4_ERR_ARG;
    int v = 0;
    cudaStream_t st = (cudaStream_t)stream;
    SO4_CUDA_TRY(cudaMemcpyAsync(&v, d_work, sizeof(int), cudaMemcpyDeviceToHost, st));
    SO4_CUDA_TRY(cudaStreamSynchronize(st));
    *h_status = v;
    return SO4_OK;
}

extern "C" int so4_nl_summary(const int32_t *d_img_ptr, const int32_t *d_pair_ptr, int natoms, const void *d_work,
                              size_t work_bytes, void *stream, int *h_summary) {
    if (!d_work || work_bytes < SO4_WS_HEADER || natoms < 0) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    int *dev = (int *)d_work + 4;  // header scratch after the status word
    k_summary<<<1, 1, 0, st>>>(d_img_ptr, d_pair_ptr, natoms, (const int *)d_work, dev);
    so4_count_launch();
    k_clamp<<<(natoms + 256) / 256, 256, 0, st>>>((int32_t *)d_img_ptr, (int32_t *)d_pair_ptr, natoms,
                                                  (const int *)d_work);
    so4_count_launch();
    if (!h_summary) return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
    SO4_CUDA_TRY(cudaMemcpyAsync(h_summary, dev, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    SO4_CUDA_TRY(cudaStreamSynchronize(st));
    return SO4_OK;
}
