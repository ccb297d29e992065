// so4_consumer.cu -- what the reference's NN potential does with the plain path's
// outputs (pyxtal_ff/models/neuralnetwork.py:579-678, calculate_properties):
//   forces[m] -= sum over pairs p with seq[p, 1] == m of dedx[seq[p, 0]] . dxdr[p]
//   stress    -= sum_i dedx[i] . rdxdr_atom[i]            (per structure, Voigt order)
// The reference forms the first with an (N, N, nB, 3) dense array (N <= 400) or one
// np.where over all pairs per atom (N > 400).  Here one warp per target atom m walks
// the pairs whose centre is m: the pair list is symmetric (j is within rcut of an
// image of i exactly when i is within rcut of an image of j), so the pairs that point
// at m are the reverse pairs (j, m) of m's own pairs (m, j), found by a binary search
// of m in j's sorted neighbour list.  No transpose, no atomics, a fixed summation
// order: sources in ascending j (four at a time), each lane one component over a fixed
// set of descriptor indices, then the lanes of a component in lane order.  With FP64
// arrays the FP64 pipe (one FMA per dxdr element) and HBM bound it about equally.
#include "so4_common.cuh"

namespace {

template <typename T>
struct CArgs {
    int natoms, nB;
    const int32_t *astruct, *atom_ptr, *pair_ptr;
    const int64_t *seq;  // (P, 2), structure-local (i, j), pairs grouped by centre, j ascending
    const T *dxdr;       // (P, nB, 3) or null
    const T *beta;       // (N, nB) dE/dx per atom
    const T *rdxdr;      // (N, nB, 6) per-atom Voigt rows or null
    T *forces;           // (N, 3)
    T *stress_atom;      // (N, 6)
    int *status;
};

template <typename T, int NV>
__device__ __forceinline__ void warp_sum(T (&acc)[NV]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int u = 0; u < NV; ++u) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
}

// acc[i] for a run-time i < NV without dynamic register indexing
template <typename T, int NV>
__device__ __forceinline__ T pick(const T (&acc)[NV], int i) {
    T v = acc[0];
#pragma unroll
    for (int u = 1; u < NV; ++u)
        if (u == i) v = acc[u];
    return v;
}

constexpr int CW = 8;  // warps (target atoms) per CTA
constexpr int CP = 4;  // incoming pairs read together

template <typename T>
__global__ void __launch_bounds__(CW * 32) k_contract_dxdr(CArgs<T> A) {
    const int lane = threadIdx.x & 31;
    const int m = blockIdx.x * CW + (threadIdx.x >> 5);
    if (m >= A.natoms) return;
    const int nB = A.nB, n3 = 3 * nB;
    if (A.dxdr) {
        const int base = A.atom_ptr[A.astruct[m]];
        const int64_t ml = m - base;
        const int q0 = A.pair_ptr[m], q1 = A.pair_ptr[m + 1];
        T fc = T(0);  // this lane's part of component lane % 3
        for (int qb = q0; qb < q1; qb += 32) {
            // lane t finds the reverse of pair qb + t: the pair (j, m) in centre j's list
            int p = -1, j = 0;
            const int q = qb + lane;
            if (q < q1) {
                j = base + (int)A.seq[2 * (size_t)q + 1];
                int lo = A.pair_ptr[j], hi = A.pair_ptr[j + 1] - 1;
                while (lo <= hi) {
                    const int mid = (lo + hi) >> 1;
                    const int64_t v = A.seq[2 * (size_t)mid + 1];
                    if (v < ml) {
                        lo = mid + 1;
                    } else if (v > ml) {
                        hi = mid - 1;
                    } else {
                        p = mid;
                        break;
                    }
                }
                if (p < 0) atomicOr(A.status, 1 << SO4_ERR_REVERSE);
            }
            const int nq = min(32, q1 - qb);
            // CP incoming pairs per pass, so each lane has 2 CP independent loads in flight
            for (int t0 = 0; t0 < nq; t0 += CP) {
                const T *d[CP];
                const T *b[CP];
                bool ok[CP];
#pragma unroll
                for (int u = 0; u < CP; ++u) {
                    const int pp = __shfl_sync(0xffffffffu, p, (t0 + u) & 31);
                    const int jj = __shfl_sync(0xffffffffu, j, (t0 + u) & 31);
                    ok[u] = t0 + u < nq && pp >= 0;  // warp-uniform
                    d[u] = A.dxdr + (size_t)(ok[u] ? pp : 0) * n3;
                    b[u] = A.beta + (size_t)(ok[u] ? jj : 0) * nB;
                }
                // lanes 0..29 take idx = lane + 30 s: the component c = idx % 3 = lane % 3 is
                // fixed per lane, so each element costs one FMA (k = idx / 3 = lane / 3 + 10 s)
                if (lane < 30) {
#pragma unroll 2
                    for (int idx = lane, k = lane / 3; idx < n3; idx += 30, k += 10) {
#pragma unroll
                        for (int u = 0; u < CP; ++u)
                            if (ok[u]) fc = fma(__ldg(b[u] + k), __ldg(d[u] + idx), fc);
                    }
                }
            }
        }
        // component sums in a fixed order: lanes c, c + 3, ..., c + 27 (lane % 3 == c)
        T f[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int l = 0; l < 30; ++l) {
            const T v = __shfl_sync(0xffffffffu, fc, l);
            f[l % 3] += v;
        }
        if (lane < 3) A.forces[3 * (size_t)m + lane] = -pick<T, 3>(f, lane);
    }
    if (A.rdxdr) {
        // lanes 0..29, idx = lane + 30 s: Voigt entry lane % 6 fixed per lane, k = lane / 6 + 5 s
        const T *r = A.rdxdr + (size_t)m * 6 * nB;
        const T *b = A.beta + (size_t)m * nB;
        T sv = T(0);
        if (lane < 30) {
#pragma unroll 4
            for (int idx = lane, k = lane / 6; idx < 6 * nB; idx += 30, k += 5) sv = fma(__ldg(b + k), __ldg(r + idx), sv);
        }
        T s[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int l = 0; l < 30; ++l) {
            const T v = __shfl_sync(0xffffffffu, sv, l);
            s[l % 6] += v;
        }
        if (lane < 6) A.stress_atom[6 * (size_t)m + lane] = -pick<T, 6>(s, lane);
    }
}

// per-structure sums of the per-atom stress rows, one CTA per structure: thread t adds
// atoms t, t + ST, ... in order, then the warps' shuffle trees and the warps in order
constexpr int ST = 256;
template <typename T>
__global__ void __launch_bounds__(ST) k_struct_stress(const int32_t *atom_ptr, const T *sa, T *out) {
    __shared__ T part[ST / 32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int s = blockIdx.x;
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll 4
    for (int a = atom_ptr[s] + threadIdx.x; a < atom_ptr[s + 1]; a += ST)
#pragma unroll
        for (int u = 0; u < 6; ++u) acc[u] += sa[6 * (size_t)a + u];
    warp_sum<T, 6>(acc);
    if (lane == 0)
#pragma unroll
        for (int u = 0; u < 6; ++u) part[wid][u] = acc[u];
    __syncthreads();
    if (threadIdx.x < 6) {
        T v = T(0);
        for (int w = 0; w < ST / 32; ++w) v += part[w][threadIdx.x];
        out[6 * (size_t)s + threadIdx.x] = v;
    }
}

template <typename T>
int run(int natoms, int nB, int nstruct, const int32_t *astruct, const int32_t *atom_ptr, const int32_t *pair_ptr,
        const int64_t *seq, const void *dxdr, const void *beta, const void *rdxdr, void *forces, void *stress_atom,
        void *stress, int *status, cudaStream_t st) {
    CArgs<T> A;
    A.natoms = natoms;
    A.nB = nB;
    A.astruct = astruct;
    A.atom_ptr = atom_ptr;
    A.pair_ptr = pair_ptr;
    A.seq = seq;
    A.dxdr = (const T *)dxdr;
    A.beta = (const T *)beta;
    A.rdxdr = (const T *)rdxdr;
    A.forces = (T *)forces;
    A.stress_atom = (T *)stress_atom;
    A.status = status;
    k_contract_dxdr<T><<<(natoms + CW - 1) / CW, CW * 32, 0, st>>>(A);
    so4_count_launch();
    if (rdxdr) {
        k_struct_stress<T><<<nstruct, ST, 0, st>>>(atom_ptr, (const T *)stress_atom, (T *)stress);
        so4_count_launch();
    }
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

// ---------------------------------------------------------------- linear design matrix
// Rows of the linear potential's design matrix (pyxtal_ff/models/polynomialregression.py:
// 438-682, parse_descriptors, order 1).  Columns: per element e (sorted) a block of 1 + nB,
// the bias column then the descriptors.

// Force rows, one warp per target atom m: row force_row[s] + 3 (m - atom_ptr[s]) + c holds
// in block e the columns 1 + k = -sum over the pairs p with seq[p, 1] == m whose centre has
// element e of dxdr[p, k, c].  The incoming pairs are the reverse pairs of m's own, as in
// k_contract_dxdr; each lane owns the entries idx = lane + 32 s of a per-warp shared
// accumulator [nelem][3 nB], so no two lanes touch one entry.
constexpr int DW = 4;  // warps per CTA
__global__ void __launch_bounds__(DW * 32) k_design_forces(int natoms, int nB, int nelem, const int32_t *astruct,
                                                          const int32_t *atom_ptr, const int32_t *pair_ptr,
                                                          const int64_t *seq, const int32_t *species,
                                                          const double *dxdr, const int64_t *force_row,
                                                          int64_t ncols, double *X, int *status) {
    extern __shared__ double dacc[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int m = blockIdx.x * DW + wid;
    const int n3 = 3 * nB;
    double *acc = dacc + (size_t)wid * nelem * n3;
    if (m >= natoms) return;
    for (int i = lane; i < nelem * n3; i += 32) acc[i] = 0.0;
    __syncwarp();  // entries are zeroed and accumulated by different lanes
    const int s = astruct[m], base = atom_ptr[s];
    const int64_t ml = m - base;
    const int q0 = pair_ptr[m], q1 = pair_ptr[m + 1];
    for (int qb = q0; qb < q1; qb += 32) {
        int p = -1, e = 0;
        const int q = qb + lane;
        if (q < q1) {
            const int j = base + (int)seq[2 * (size_t)q + 1];
            e = species[j];
            int lo = pair_ptr[j], hi = pair_ptr[j + 1] - 1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                const int64_t v = seq[2 * (size_t)mid + 1];
                if (v < ml) {
                    lo = mid + 1;
                } else if (v > ml) {
                    hi = mid - 1;
                } else {
                    p = mid;
                    break;
                }
            }
            if (p < 0) atomicOr(status, 1 << SO4_ERR_REVERSE);
            if (e < 0 || e >= nelem) {
                atomicOr(status, 1 << SO4_ERR_ARG);
                p = -1;
            }
        }
        const int nq = min(32, q1 - qb);
        for (int t = 0; t < nq; ++t) {
            const int pp = __shfl_sync(0xffffffffu, p, t), ee = __shfl_sync(0xffffffffu, e, t);
            if (pp < 0) continue;  // warp-uniform
            const double *d = dxdr + (size_t)pp * n3;
            double *a = acc + (size_t)ee * n3;
#pragma unroll 4
            for (int idx = lane; idx < n3; idx += 32) a[idx] -= __ldg(d + idx);
        }
    }
    __syncwarp();
    const int64_t row0 = force_row[s] + 3 * ml;
    for (int i = lane; i < nelem * n3; i += 32) {
        const int ee = i / n3, r = i - ee * n3, k = r / 3, c = r - 3 * k;
        X[(row0 + c) * ncols + (int64_t)ee * (1 + nB) + 1 + k] = acc[i];
    }
}

// Energy and stress rows of each structure, one CTA per (structure, element): the energy
// row (energy_row[s] >= 0) gets in block e the atom count and the sums of x over the
// structure's atoms of element e; the six stress rows (stress_row[s] >= 0) get
// -sum rdxdr_atom[i, k, v] in columns 1 + k.  Each thread owns columns and adds the
// atoms in order.
constexpr int DS = 128;
__global__ void __launch_bounds__(DS) k_design_struct(int nB, const int32_t *atom_ptr, const int32_t *species,
                                                      const double *x, const double *rdxdr,
                                                      const int64_t *energy_row, const int64_t *stress_row,
                                                      int64_t ncols, double *X) {
    const int s = blockIdx.x, e = blockIdx.y;
    const int a0 = atom_ptr[s], a1 = atom_ptr[s + 1];
    const int64_t col0 = (int64_t)e * (1 + nB);
    const int64_t er = energy_row[s], sr = stress_row ? stress_row[s] : -1;
    if (er >= 0)
        for (int col = threadIdx.x; col <= nB; col += DS) {
            double v = 0.0;
            for (int i = a0; i < a1; ++i)
                if (species[i] == e) v += (col == 0) ? 1.0 : x[(size_t)i * nB + col - 1];
            X[er * ncols + col0 + col] = v;
        }
    if (sr >= 0 && rdxdr)
        for (int t = threadIdx.x; t < 6 * nB; t += DS) {
            const int k = t / 6, v = t - 6 * k;
            double acc = 0.0;
            for (int i = a0; i < a1; ++i)
                if (species[i] == e) acc -= rdxdr[(size_t)i * 6 * nB + t];
            X[(sr + v) * ncols + col0 + 1 + k] = acc;
        }
}

// ---------------------------------------------------------------- quadratic features
// Order 2 (polynomialregression.py:488-559): the features of descriptors x (length d) are
// x_a (a < d), then for each d1 the square 0.5 x_d1^2 followed by the products
// x_d1 x_d2 (d2 > d1).  feat[f] = (d1, d2): (a, -1) linear, (d1, d1) square, else product.
// Their derivative along any descriptor derivative t (dxdr or rdxdr row) is t_a,
// x_d1 t_d1, or x_d2 t_d1 + x_d1 t_d2, with x the centre atom's descriptors.
__device__ __forceinline__ double qfeat_d(int2 f, const double *x, const double *t, int stride) {
    if (f.y < 0) return t[stride * f.x];
    if (f.x == f.y) return x[f.x] * t[stride * f.x];
    return fma(x[f.y], t[stride * f.x], x[f.x] * t[stride * f.y]);
}
__device__ __forceinline__ double qfeat(int2 f, const double *x) {
    if (f.y < 0) return x[f.x];
    if (f.x == f.y) return 0.5 * x[f.x] * x[f.x];
    return x[f.x] * x[f.y];
}

// Force rows for general features, one CTA per target atom m: for each pair p pointing
// at m (the reverse of m's own pairs, in ascending source order), the pair's dxdr and the
// source's descriptors are staged in shared memory and every thread adds, for the
// outputs (element, feature, component) it owns, -d feature / d r of that source.
constexpr int QT = 256, QMAXO = 16;  // threads; outputs per thread per pass
__global__ void __launch_bounds__(QT) k_design_forces_q(int nB, int nfeat, int nelem, const int2 *feat,
                                                       const int32_t *astruct, const int32_t *atom_ptr,
                                                       const int32_t *pair_ptr, const int64_t *seq,
                                                       const int32_t *species, const double *x,
                                                       const double *dxdr, const int64_t *force_row,
                                                       int64_t ncols, double *X, int *status) {
    extern __shared__ double qsm[];  // dxdr row [3 nB], source descriptors [nB]
    double *sd = qsm, *sx = qsm + 3 * nB;
    __shared__ int s_p, s_e;
    const int m = blockIdx.x, t = threadIdx.x;
    const int s = astruct[m], base = atom_ptr[s];
    const int64_t ml = m - base;
    const int q0 = pair_ptr[m], q1 = pair_ptr[m + 1];
    const int nout = nelem * nfeat * 3;
    for (int o0 = 0; o0 < nout; o0 += QT * QMAXO) {
        double acc[QMAXO];
#pragma unroll
        for (int k = 0; k < QMAXO; ++k) acc[k] = 0.0;
        for (int q = q0; q < q1; ++q) {
            if (t == 0) {
                const int j = base + (int)seq[2 * (size_t)q + 1];
                int p = -1, lo = pair_ptr[j], hi = pair_ptr[j + 1] - 1;
                while (lo <= hi) {
                    const int mid = (lo + hi) >> 1;
                    const int64_t v = seq[2 * (size_t)mid + 1];
                    if (v < ml) {
                        lo = mid + 1;
                    } else if (v > ml) {
                        hi = mid - 1;
                    } else {
                        p = mid;
                        break;
                    }
                }
                const int e = species[j];
                if (p < 0) atomicOr(status, 1 << SO4_ERR_REVERSE);
                if (e < 0 || e >= nelem) {
                    atomicOr(status, 1 << SO4_ERR_ARG);
                    p = -1;
                }
                s_p = p;
                s_e = e;
            }
            __syncthreads();
            const int pp = s_p, ee = s_e;
            if (pp >= 0) {
                const int j = base + (int)seq[2 * (size_t)q + 1];
                for (int i = t; i < 3 * nB; i += QT) sd[i] = dxdr[(size_t)pp * 3 * nB + i];
                for (int i = t; i < nB; i += QT) sx[i] = x[(size_t)j * nB + i];
            }
            __syncthreads();
            if (pp >= 0) {
#pragma unroll
                for (int k = 0; k < QMAXO; ++k) {
                    const int o = o0 + t + QT * k;
                    if (o < nout) {
                        const int c = o % 3, f = (o / 3) % nfeat, e = o / (3 * nfeat);
                        if (e == ee) acc[k] -= qfeat_d(__ldg(feat + f), sx, sd + c, 3);
                    }
                }
            }
            __syncthreads();
        }
        const int64_t row0 = force_row[s] + 3 * ml;
#pragma unroll
        for (int k = 0; k < QMAXO; ++k) {
            const int o = o0 + t + QT * k;
            if (o < nout) {
                const int c = o % 3, f = (o / 3) % nfeat, e = o / (3 * nfeat);
                X[(row0 + c) * ncols + (int64_t)e * (1 + nfeat) + 1 + f] = acc[k];
            }
        }
    }
}

// Energy and stress rows for general features, one CTA per (structure, element): the energy
// row gets the atom count and the sums of the features; the stress rows the sums of
// -d feature along the per-atom Voigt rows.
__global__ void __launch_bounds__(DS) k_design_struct_q(int nB, int nfeat, const int2 *feat,
                                                        const int32_t *atom_ptr, const int32_t *species,
                                                        const double *x, const double *rdxdr,
                                                        const int64_t *energy_row, const int64_t *stress_row,
                                                        int64_t ncols, double *X) {
    const int s = blockIdx.x, e = blockIdx.y;
    const int a0 = atom_ptr[s], a1 = atom_ptr[s + 1];
    const int64_t col0 = (int64_t)e * (1 + nfeat);
    const int64_t er = energy_row[s], sr = stress_row ? stress_row[s] : -1;
    if (er >= 0)
        for (int col = threadIdx.x; col <= nfeat; col += DS) {
            double v = 0.0;
            for (int i = a0; i < a1; ++i)
                if (species[i] == e) v += (col == 0) ? 1.0 : qfeat(__ldg(feat + col - 1), x + (size_t)i * nB);
            X[er * ncols + col0 + col] = v;
        }
    if (sr >= 0 && rdxdr)
        for (int o = threadIdx.x; o < 6 * nfeat; o += DS) {
            const int f = o / 6, v = o - 6 * f;
            double acc = 0.0;
            for (int i = a0; i < a1; ++i)
                if (species[i] == e)
                    acc -= qfeat_d(__ldg(feat + f), x + (size_t)i * nB, rdxdr + (size_t)i * 6 * nB + v, 6);
            X[(sr + v) * ncols + col0 + 1 + f] = acc;
        }
}

}  // namespace

extern "C" int so4_design_forces_q(int natoms, int nB, int nfeat, int nelem, const int2 *d_feat,
                                   const int32_t *d_atom_struct, const int32_t *d_atom_ptr, const int32_t *d_pair_ptr,
                                   const int64_t *d_seq, const int32_t *d_species, const double *d_x,
                                   const double *d_dxdr, const int64_t *d_force_row, int64_t ncols, double *d_X,
                                   int *d_status, void *stream) {
    if (natoms < 0 || nB <= 0 || nfeat <= 0 || nelem <= 0 || ncols < (int64_t)nelem * (1 + nfeat)) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    if (!d_feat || !d_atom_struct || !d_atom_ptr || !d_pair_ptr || !d_seq || !d_species || !d_x || !d_dxdr ||
        !d_force_row || !d_X || !d_status)
        return SO4_ERR_ARG;
    const size_t smem = sizeof(double) * 4 * (size_t)nB;
    if (smem > 48 * 1024) return SO4_ERR_UNSUPPORTED;
    k_design_forces_q<<<natoms, QT, smem, (cudaStream_t)stream>>>(nB, nfeat, nelem, d_feat, d_atom_struct, d_atom_ptr,
                                                                  d_pair_ptr, d_seq, d_species, d_x, d_dxdr,
                                                                  d_force_row, ncols, d_X, d_status);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_design_struct_q(int nstruct, int nB, int nfeat, int nelem, const int2 *d_feat,
                                   const int32_t *d_atom_ptr, const int32_t *d_species, const double *d_x,
                                   const double *d_rdxdr_atom, const int64_t *d_energy_row,
                                   const int64_t *d_stress_row, int64_t ncols, double *d_X, void *stream) {
    if (nstruct < 0 || nB <= 0 || nfeat <= 0 || nelem <= 0 || ncols < (int64_t)nelem * (1 + nfeat)) return SO4_ERR_ARG;
    if (nstruct == 0) return SO4_OK;
    if (!d_feat || !d_atom_ptr || !d_species || !d_x || !d_energy_row || !d_X || (d_stress_row && !d_rdxdr_atom))
        return SO4_ERR_ARG;
    k_design_struct_q<<<dim3(nstruct, nelem), DS, 0, (cudaStream_t)stream>>>(nB, nfeat, d_feat, d_atom_ptr, d_species,
                                                                             d_x, d_rdxdr_atom, d_energy_row,
                                                                             d_stress_row, ncols, d_X);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_design_forces(int natoms, int nB, int nelem, const int32_t *d_atom_struct,
                                 const int32_t *d_atom_ptr, const int32_t *d_pair_ptr, const int64_t *d_seq,
                                 const int32_t *d_species, const double *d_dxdr, const int64_t *d_force_row,
                                 int64_t ncols, double *d_X, int *d_status, void *stream) {
    if (natoms < 0 || nB <= 0 || nelem <= 0 || ncols < (int64_t)nelem * (1 + nB)) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    if (!d_atom_struct || !d_atom_ptr || !d_pair_ptr || !d_seq || !d_species || !d_dxdr || !d_force_row || !d_X ||
        !d_status)
        return SO4_ERR_ARG;
    const size_t smem = sizeof(double) * DW * (size_t)nelem * 3 * nB;
    if (smem > 227 * 1024) return SO4_ERR_UNSUPPORTED;
    int rc = so4_set_smem((const void *)k_design_forces, smem);
    if (rc) return rc;
    k_design_forces<<<(natoms + DW - 1) / DW, DW * 32, smem, (cudaStream_t)stream>>>(
        natoms, nB, nelem, d_atom_struct, d_atom_ptr, d_pair_ptr, d_seq, d_species, d_dxdr, d_force_row, ncols, d_X,
        d_status);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_design_struct(int nstruct, int nB, int nelem, const int32_t *d_atom_ptr, const int32_t *d_species,
                                 const double *d_x, const double *d_rdxdr_atom, const int64_t *d_energy_row,
                                 const int64_t *d_stress_row, int64_t ncols, double *d_X, void *stream) {
    if (nstruct < 0 || nB <= 0 || nelem <= 0 || ncols < (int64_t)nelem * (1 + nB)) return SO4_ERR_ARG;
    if (nstruct == 0) return SO4_OK;
    if (!d_atom_ptr || !d_species || !d_x || !d_energy_row || !d_X || (d_stress_row && !d_rdxdr_atom))
        return SO4_ERR_ARG;
    k_design_struct<<<dim3(nstruct, nelem), DS, 0, (cudaStream_t)stream>>>(nB, d_atom_ptr, d_species, d_x,
                                                                           d_rdxdr_atom, d_energy_row, d_stress_row,
                                                                           ncols, d_X);
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}

extern "C" int so4_contract_dxdr(int precision, int natoms, int nB, int nstruct, const int32_t *d_atom_struct,
                                 const int32_t *d_atom_ptr, const int32_t *d_pair_ptr, const int64_t *d_seq,
                                 const void *d_dxdr, const void *d_beta, const void *d_rdxdr_atom, void *d_forces,
                                 void *d_stress_atom, void *d_stress, int *d_status, void *stream) {
    if (precision != 0 && precision != 1) return SO4_ERR_ARG;
    if (natoms < 0 || nB <= 0 || nstruct < 0) return SO4_ERR_ARG;
    if (natoms == 0) return SO4_OK;
    if (!d_beta || !d_atom_ptr || !d_status || (!d_dxdr && !d_rdxdr_atom)) return SO4_ERR_ARG;
    if (d_dxdr && (!d_atom_struct || !d_pair_ptr || !d_seq || !d_forces)) return SO4_ERR_ARG;
    if (d_rdxdr_atom && (!d_stress_atom || !d_stress || nstruct < 1)) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == 0)
        return run<double>(natoms, nB, nstruct, d_atom_struct, d_atom_ptr, d_pair_ptr, d_seq, d_dxdr, d_beta,
                           d_rdxdr_atom, d_forces, d_stress_atom, d_stress, d_status, st);
    return run<float>(natoms, nB, nstruct, d_atom_struct, d_atom_ptr, d_pair_ptr, d_seq, d_dxdr, d_beta,
                      d_rdxdr_atom, d_forces, d_stress_atom, d_stress, d_status, st);
}
