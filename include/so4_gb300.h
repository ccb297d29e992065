/*
 * so4_gb300.h -- C ABI of the GB300-native SO(4)/SNAP bispectrum path.
 *
 * Replaces the numeric core of PyXtal_FF's descriptor
 *   pyxtal_ff/descriptors/SO4.py   SO4_Bispectrum.calculate          :171-209
 *                                  build_neighbor_list                :211-287
 *                                  get_bispectrum_components          :1256-1730
 *   pyxtal_ff/descriptors/SNAP.py  (same, weights / rfac0 variant)   :200-1762
 * and the contraction its consumers apply to dxdr / rdxdr
 *   pyxtal_ff/models/neuralnetwork.py:492 (forces), :497,:677-678 (stress).
 *
 * Conventions
 *  - Every entry point returns an int status (enum so4_status); nothing throws
 *    across the ABI.  Device-side failures are reported through a status word
 *    in the caller's workspace, read back by so4_status_read().
 *  - Pointers named d_* are device pointers; h_* are host pointers.  All device
 *    buffers are allocated by the caller.  No entry point allocates device
 *    memory except so4_tables_create (the constant tables it owns).
 *  - `stream` is a cudaStream_t passed as void*.  Every launch is ordered on it;
 *    no entry point synchronises the host except so4_tables_create/destroy.
 *  - Atoms of many structures are concatenated; a structure's atoms are
 *    contiguous.  Every atom is a centre (the reference's atom_ids prefix is a
 *    slice of the outputs).  seq rows hold structure-local atom indices, as
 *    the reference's seq does.
 *  - "half layout": for each 2j = l in 0..twol the rows mb = 0..floor(l/2) of
 *    the (l+1)x(l+1) Wigner-U block, all l+1 columns, stored as (re, im).
 *    idxu_half entries in total (155 at twol = 8).
 */
#ifndef SO4_GB300_H
#define SO4_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum so4_status {
    SO4_OK = 0,
    SO4_ERR_ARG = 1,          /* invalid argument (reference: ValueError)            */
    SO4_ERR_UNSUPPORTED = 2,  /* valid but not supported (reference: NotImplementedError) */
    SO4_ERR_CUDA = 3,         /* a CUDA runtime call failed                         */
    SO4_ERR_CAPACITY = 4,     /* an image offset or count exceeds the encodable range */
    SO4_ERR_NONFINITE = 5,    /* NaN/Inf in positions or cell                       */
    SO4_ERR_WORKSPACE = 6,    /* workspace smaller than the size query returned     */
    SO4_ERR_NO_NEIGHBOR = 7,  /* an atom has no neighbour image (reference raises ValueError, SO4.py:275) */
    SO4_ERR_REVERSE = 8,      /* an image has no reverse image (asymmetric list)    */
    SO4_ERR_TOO_LARGE = 9,    /* problem needs more than the fixed scratch of so4_adjoint32_noalloc */
    SO4_ERR_SLOTS = 10        /* an atom has more images than the per-atom key slots of so4_nl_count_keys */
};

/* Maximum 2*lmax the kernels are compiled for (lmax <= 6). */
#define SO4_TWOL_MAX 12

typedef struct so4_tables so4_tables;

/* Parameters of one evaluation (SO4.py:22-158, SNAP.py:22-187).
 * cutoff_id: 1 cosine, 2 tanh, 3 poly1, 4 poly2, 5 poly3, 6 poly4, 7 exp (SO4.py:134-154).
 * rfac0: 1 for SO4.py (psi = pi r / rc), the SNAP rfac0 otherwise (psi = rfac0 pi r / rc). */
typedef struct {
    int twol;
    int cutoff_id;
    double rcut;
    double rfac0;
} so4_params;

/* Per-structure geometry record, filled on the host by so4_geometry() and copied
 * to the device by the caller.  f = r . inv  gives fractional coordinates. */
typedef struct {
    double cell[9];
    double inv[9];
    double vol;
    int nbin[3];
    int mshift[3];
    int pbc[3];
    int bin_base;
    int atom_base;
    int natoms;
} so4_geom;

/* ------------------------------------------------------------------ tables */

/* FP64 Clebsch-Gordan list, rootpq and index tables for one twol, built on the
 * host exactly as the reference builds them (SO4.py:410-480, 831-838,
 * 1265-1396; angular_momentum.py:9-190) and copied to the device once.
 * normalize_u selects u_norm = 4 pi / sqrt(l+1) (SO4.py:1304-1311). */
int so4_tables_create(int twol, int normalize_u, so4_tables **out);
int so4_tables_destroy(so4_tables *t);

/* Launch shapes of the FP32 kernels, chosen per (lmax, workload, device) by the
 * autotuner (pyxtal_ff_gb300/autotune.py).  No counterpart in the reference, whose
 * serial driver loop (SO4.py:1414-1548) has nothing to tune.  Zero in a field selects
 * the default.
 *   wkmax       entries per window unit of the Z pass, 1..5 (default 5): the window
 *               work lists are built for it (a smaller unit: more units, fewer
 *               registers per ring, other rounding of the Z sums);
 *   rev_threads threads per CTA of the per-image pass, 128 or 256 (default 256 up to
 *               twol 8, 128 above; only twol 6 and 8 have both);
 *   utot_warps  warps (centres) per CTA of the U_tot pass, 2, 4 or 8 (default 4; only
 *               twol 6 and 8 have all three);
 *   rev_pair    layout of the per-image pass: 1 two lanes per image (its row chains
 *               shared out so the lanes' work per level is even), 2 one lane per row
 *               chain (built for every twol; rev_threads applies to it); 0 the default,
 *               two lanes where built (twol 6 and 8);
 *   zw_atoms    atoms per CTA of the window Z pass (so4_forward32, so4_adjoint_y32,
 *               so4_linear_by32, so4_jvp32): 32, one per lane, two CTAs per SM; or 64,
 *               two per lane (their real and imaginary parts packed in FP32 pairs), one
 *               CTA per SM, up to twol 8, where its U tiles fit in shared memory
 *               (default 64 up to twol 8, 32 above);
 *   zw_threads  threads per CTA of the 64-atom window pass, 256 or 512 (default 512:
 *               16 warps at 128 registers).
 * Every layout gives the same bits. */
typedef struct {
    int wkmax;
    int rev_threads;
    int utot_warps;
    int rev_pair;
    int zw_atoms;
    int zw_threads;
} so4_tuning;
/* so4_tables_create with a tuning (NULL: the defaults).  SO4_ERR_ARG for a value
 * outside the ranges above; SO4_ERR_UNSUPPORTED for a CTA shape not built for this
 * twol, or for a wkmax whose window kernels (more units, so more B / JVP slots staged
 * in shared memory) would not fit where the default ones do. */
int so4_tables_create_tuned(int twol, int normalize_u, const so4_tuning *tune, so4_tables **out);
/* The tuning a handle was built with, defaults filled in. */
int so4_tables_get_tuning(const so4_tables *t, so4_tuning *out);
/* sizes[0..7] = idxu, idxu_half, idxz, nB, idxcg, number of Z blocks,
 * B-section entries per atom (scratch of so4_linear_by32), window sub-segments */
int so4_tables_sizes(const so4_tables *t, int *sizes);
/* host copies of the reference-visible tables (any pointer may be NULL):
 * cglist[idxcg] f64, idxb[nB*3], idxz[idxz*10], idxu_block[twol+1],
 * idxz_block[(twol+1)^3], idxcg_block[(twol+1)^3] -- same values and order as
 * the reference's arrays. */
int so4_tables_export(const so4_tables *t, double *h_cglist, int *h_idxb, int *h_idxz,
                      int *h_idxu_block, int *h_idxz_block, int *h_idxcg_block);

/* ------------------------------------------------------------ neighbours */
/* Replaces ase.neighborlist.NeighborList(rc/2 per atom, bothways, no self) and
 * the (i, sorted unique j) grouping of SO4.py:211-287: an image (j, o) of
 * centre i is kept when |pos[j] + o.cell - pos[i]| < rcut, (i, 0) excluded;
 * images are sorted by (j, o) and every centre gets an (i, i) pair. */

/* Host: geometry records for nstruct structures.  h_cells[9*s] row-major
 * (rows a1, a2, a3), h_pbc[3*s], h_atom_ptr[nstruct+1].  Writes h_geom[nstruct]
 * and the total number of bins.  Fails with SO4_ERR_ARG on a singular cell
 * with periodic axes and SO4_ERR_NONFINITE on NaN/Inf. */
int so4_geometry(const double *h_cells, const int *h_pbc, const int *h_atom_ptr, int nstruct,
                 double rcut, so4_geom *h_geom, int *h_nbins_total);

/* Workspace bytes for so4_nl_count / so4_nl_fill / so4_nl_pairs. */
size_t so4_nl_workspace_size(int natoms, int nbins_total, int64_t nimg);

/* Pass 1: bins the atoms and counts the images of every centre.
 * d_pos[3*natoms] f64, d_atom_struct[natoms] i32.  Writes d_img_ptr[natoms+1]
 * (exclusive scan; the host reads d_img_ptr[natoms] = nimg). */
int so4_nl_count(const so4_geom *d_geom, int nstruct, int nbins_total, const double *d_pos,
                 const int *d_atom_struct, int natoms, double rcut, int32_t *d_img_ptr,
                 void *d_work, size_t work_bytes, void *stream);

/* Pass 2: writes the sorted images of every centre: d_img_j[nimg] (nimg is the
 * capacity of the image arrays; past it nothing is written and the status gets
 * SO4_ERR_CAPACITY, so a caller may pass an estimate and retry with more),
 * d_img_off[3*nimg] (integer cell offsets), d_img_r[3*nimg] (the image vectors,
 * (pos[j] + (o0 a1 + o1 a2) + o2 a3) - pos[i] in FP64 with every operation
 * separately rounded) and the pair counts as an exclusive scan d_pair_ptr[natoms+1]. */
int so4_nl_fill(const so4_geom *d_geom, int nstruct, int nbins_total, const double *d_pos,
                const int *d_atom_struct, int natoms, double rcut, const int32_t *d_img_ptr,
                int64_t nimg, int32_t *d_img_j, int32_t *d_img_off, double *d_img_r,
                int32_t *d_pair_ptr, void *d_work, size_t work_bytes, void *stream);

/* Pass 3 (npair: capacity of the pair arrays, as nimg above):
 * d_seq[2*npair] (i64, structure-local (i, j)), d_pair_img[npair+1]
 * (images of pair p are [pair_img[p], pair_img[p+1])), d_nsite[natoms] (the
 * (i, i) pair of each centre), d_img_pair[nimg] and d_img_rev[nimg] (index of
 * the image (i, -o) in the list of j).  With d_seq, d_pair_img, d_nsite and
 * d_img_pair all NULL only d_img_rev is written (what the adjoint needs). */
int so4_nl_pairs(const so4_geom *d_geom, int nstruct, const int *d_atom_struct, int natoms,
                 const int32_t *d_img_ptr, int64_t nimg, const int32_t *d_img_j,
                 const int32_t *d_img_off, const int32_t *d_pair_ptr, int64_t npair,
                 int64_t *d_seq, int32_t *d_pair_img, int32_t *d_nsite, int32_t *d_img_pair,
                 int32_t *d_img_rev, void *d_work, size_t work_bytes, void *stream);

/* One pass instead of so4_nl_count + the key pass of so4_nl_fill: counts the images of
 * every centre (d_img_ptr, as so4_nl_count) and writes their keys into slot_cap slots per
 * atom of the workspace (so4_nl_workspace_size(natoms, nbins, natoms * slot_cap) bytes at
 * least).  An atom with more than slot_cap images sets status bits SO4_ERR_SLOTS and
 * SO4_ERR_CAPACITY; the largest per-atom count is left at ((int *)d_work)[8].
 * so4_nl_sort then does the rest of so4_nl_fill from those slots (same outputs). */
int so4_nl_count_keys(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_atom_struct,
                      int natoms, double rcut, int slot_cap, int32_t *d_img_ptr, void *d_work, size_t work_bytes,
                      void *stream);
int so4_nl_sort(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_atom_struct,
                int natoms, const int32_t *d_img_ptr, int64_t nimg, int slot_cap, int32_t *d_img_j,
                int32_t *d_img_off, double *d_img_r, int32_t *d_pair_ptr, void *d_work, size_t work_bytes,
                void *stream);

/* The same one-pass list in parts, so that a graph can run the list of one range of
 * centres while another range already computes (so4_nl_count_keys = bins, then the key
 * pass and the scan of [0, natoms)):
 *   so4_nl_bins              bins every atom and clears the status;
 *   so4_nl_count_keys_range  counts and keys of the centres [a0, a1) into their slots;
 *   so4_nl_scan_range        d_img_ptr[a0 .. a1] = d_img_ptr[a0] (0 when a0 = 0) + the exclusive
 *                            scan of those counts: ranges are scanned in order, each after the
 *                            previous one's scan;
 *   so4_nl_sort_range        so4_nl_sort for the centres [a0, a1) without the pair counts, and,
 *                            if any capacity was exceeded so far, empties d_img_ptr[a0 .. a1]
 *                            so that work enqueued behind it on the range reads nothing out of
 *                            bounds.
 * The lite reverse pass (so4_nl_pairs with NULL pair arrays) and so4_nl_summary run after
 * every range is sorted. */
int so4_nl_bins(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_atom_struct,
                int natoms, int slot_cap, void *d_work, size_t work_bytes, void *stream);
int so4_nl_count_keys_range(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos,
                            const int *d_atom_struct, int natoms, double rcut, int slot_cap, int a0, int a1,
                            void *d_work, size_t work_bytes, void *stream);
int so4_nl_scan_range(int natoms, int nbins, int slot_cap, int a0, int a1, int32_t *d_img_ptr, void *d_work,
                      size_t work_bytes, void *stream);
int so4_nl_sort_range(const so4_geom *d_geom, int nstruct, int nbins, const double *d_pos, const int *d_atom_struct,
                      int natoms, int a0, int a1, int32_t *d_img_ptr, int64_t nimg, int slot_cap, int32_t *d_img_j,
                      int32_t *d_img_off, double *d_img_r, void *d_work, size_t work_bytes, void *stream);

/* {total images, total pairs, status bits} after the three passes (d_pair_ptr may
 * be NULL after pass 1 only), written to ((int *)d_work)[4..6]; with h_summary
 * non-NULL also copied there by one synchronising read.  With h_summary NULL the
 * call does not synchronise (for stream capture); the caller reads the three
 * ints later, e.g. with the step's results.  When a capacity was exceeded (status
 * bit SO4_ERR_CAPACITY) the call also empties every range of d_img_ptr and
 * d_pair_ptr, so that work enqueued behind it reads no image out of bounds. */
int so4_nl_summary(const int32_t *d_img_ptr, const int32_t *d_pair_ptr, int natoms, const void *d_work,
                   size_t work_bytes, void *stream, int *h_summary);

/* Reads the device status word of a workspace (synchronises `stream`). */
int so4_status_read(const void *d_work, size_t work_bytes, void *stream, int *h_status);

/* ------------------------------------------------------------- plain path */
/* B, dB/dr per (i, j) pair and the per-pair virial, as the reference returns
 * them (SO4.py:190-199): x = blist.real, dxdr, rdxdr = -bstress / vol.
 * precision 0 = FP64 throughout, 1 = FP32 arithmetic with FP64 tables and
 * FP32 outputs.  d_w_nb[natoms]: neighbour weight of each atom (SO4: atomic
 * number; SNAP: weights[symbol]); d_w_site[natoms]: site weight (SO4: atomic
 * number; SNAP: 1).  want_deriv / want_stress as the reference's flags; dxdr
 * and rdxdr may be NULL when not wanted.  Output element type is double
 * (precision 0) or float (precision 1).  Scratch: so4_plain_workspace_size()
 * bytes -- a status header, and at twol 12, where the FP64 path's Z does not fit in
 * shared memory, one global Z slot per CTA of the launch (min(natoms, 2 x SMs)). */
size_t so4_plain_workspace_size(const so4_tables *t, int natoms);
int so4_plain(const so4_tables *t, const so4_params *p, int precision, const so4_geom *d_geom,
              const int *d_atom_struct, int natoms, const double *d_pos, const double *d_w_nb,
              const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
              const double *d_img_r, const int32_t *d_pair_ptr, const int32_t *d_pair_img,
              const int32_t *d_nsite, int want_deriv, int want_stress, void *d_x, void *d_dxdr,
              void *d_rdxdr, void *d_work, size_t work_bytes, void *stream);

/* Per-atom stress rows from the plain path's per-pair rdxdr, as the reference's
 * caller builds them after calculate() (pyxtal_ff/utilities/__init__.py:226-233):
 * d_out[natoms*nB*6][m, k, v] = sum over the pairs p of centre m (d_pair_ptr) of
 * rdxdr[p, k, a, b], v = 0..5 the Voigt order (0,0) (1,1) (2,2) (0,1) (0,2) (1,2).
 * precision 0: double arrays, 1: float. */
int so4_rdxdr_atom(int precision, const void *d_rdxdr, const int32_t *d_pair_ptr, int natoms, int nB, void *d_out,
                   void *stream);

/* The NN potential's contraction of the plain path's outputs with dE/dx
 * (replaces the dense (N, N, nB, 3) array / per-atom np.where loop of
 * pyxtal_ff/models/neuralnetwork.py:579-678, calculate_properties):
 *   d_forces[m, c]    = -sum over pairs p with seq[p, 1] == m of beta[seq[p, 0]] . dxdr[p, :, c]
 *   d_stress_atom[m, v] = -sum_k beta[m, k] rdxdr_atom[m, k, v]
 *   d_stress[s, v]    = sum of d_stress_atom over the atoms of structure s
 * d_beta[natoms*nB] = dE/dx (normalisation already folded in), d_seq / d_pair_ptr
 * as so4_nl_pairs writes them (pairs grouped by centre, j ascending), the
 * pair list symmetric (every (i, j) has its (j, i)); a pair without its reverse
 * sets bit SO4_ERR_REVERSE in *d_status (device int, zeroed by the caller).  Pass
 * d_dxdr NULL to skip the forces, d_rdxdr_atom NULL to skip the stress.  Fixed
 * summation order (deterministic).  precision 0: double arrays, 1: float. */
int so4_contract_dxdr(int precision, int natoms, int nB, int nstruct, const int32_t *d_atom_struct,
                      const int32_t *d_atom_ptr, const int32_t *d_pair_ptr, const int64_t *d_seq,
                      const void *d_dxdr, const void *d_beta, const void *d_rdxdr_atom, void *d_forces,
                      void *d_stress_atom, void *d_stress, int *d_status, void *stream);

/* Rows of the linear (order 1) potential's design matrix d_X (row-major, ncols
 * columns, FP64), replacing the per-atom np.where loops of
 * pyxtal_ff/models/polynomialregression.py:438-682 (parse_descriptors).  Column
 * block e (element index d_species[i] in 0..nelem-1) spans [e (1 + nB), (e + 1)(1 + nB)):
 * the bias column, then the nB descriptors.
 * so4_design_forces: for every atom m of structure s, rows d_force_row[s] + 3 (m - atom_ptr[s]) + c
 *   get in block e columns 1 + k: -sum over the pairs p with seq[p, 1] == m whose centre
 *   has element e of dxdr[p, k, c] (bias columns untouched).  Pair list and status as
 *   so4_contract_dxdr; an element index outside [0, nelem) sets bit SO4_ERR_ARG.
 * so4_design_struct: for structure s with d_energy_row[s] >= 0 that row gets, per block
 *   e, the count of atoms of element e and the sums of their x; with d_stress_row[s] >= 0
 *   (d_stress_row may be NULL) rows d_stress_row[s] + v get -sum rdxdr_atom[i, k, v] in
 *   columns 1 + k. */
int so4_design_forces(int natoms, int nB, int nelem, const int32_t *d_atom_struct, const int32_t *d_atom_ptr,
                      const int32_t *d_pair_ptr, const int64_t *d_seq, const int32_t *d_species,
                      const double *d_dxdr, const int64_t *d_force_row, int64_t ncols, double *d_X,
                      int *d_status, void *stream);
int so4_design_struct(int nstruct, int nB, int nelem, const int32_t *d_atom_ptr, const int32_t *d_species,
                      const double *d_x, const double *d_rdxdr_atom, const int64_t *d_energy_row,
                      const int64_t *d_stress_row, int64_t ncols, double *d_X, void *stream);

/* The same rows for general features of the nB descriptors (order 2, quadratic SNAP:
 * polynomialregression.py:488-559): d_feat[nfeat] = (d1, d2) per feature, (a, -1) for x_a,
 * (d1, d1) for 0.5 x_d1^2, (d1, d2) for x_d1 x_d2; block e spans 1 + nfeat columns.  Force
 * rows: -sum over the pairs pointing at the atom of d feature(x of the pair's centre) / d r
 * (one CTA per atom); energy rows: the count and the sums of the features; stress rows:
 * -sum of d feature along the per-atom Voigt rows. */
int so4_design_forces_q(int natoms, int nB, int nfeat, int nelem, const int2 *d_feat, const int32_t *d_atom_struct,
                        const int32_t *d_atom_ptr, const int32_t *d_pair_ptr, const int64_t *d_seq,
                        const int32_t *d_species, const double *d_x, const double *d_dxdr, const int64_t *d_force_row,
                        int64_t ncols, double *d_X, int *d_status, void *stream);
int so4_design_struct_q(int nstruct, int nB, int nfeat, int nelem, const int2 *d_feat, const int32_t *d_atom_ptr,
                        const int32_t *d_species, const double *d_x, const double *d_rdxdr_atom,
                        const int64_t *d_energy_row, const int64_t *d_stress_row, int64_t ncols, double *d_X,
                        void *stream);

/* ------------------------------------------------------------ adjoint path */
/* Forward (FP32): U_tot per centre in the half layout (d_utot[natoms*idxu_half*2]
 * f32, kept for the adjoint) and B (d_x[natoms*nB] f32).  Scratch:
 * so4_forward32_workspace_size() bytes (per-atom partial sums of B). */
size_t so4_forward32_workspace_size(const so4_tables *t, int natoms);
int so4_forward32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                  const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
                  const double *d_img_r, float *d_utot, float *d_x, void *d_work, size_t work_bytes,
                  void *stream);

/* Adjoint (FP32 arithmetic, FP64 accumulation of forces and virial): given
 * beta = dE/dB (d_beta[natoms*nB] f32) and the forward's d_utot, writes
 *   d_forces[natoms*3] f64 = -dE/dr,
 *   d_virial[nstruct*9] f64 = sum over images of r (x) dE/dr_image (eV),
 * without materialising dB/dr.  The reference's contracted stress is
 * -virial/vol in Voigt order (xx,yy,zz,xy,xz,yz) x 160.21766 GPa.
 * Uses scratch from d_work (so4_adjoint_workspace_size). */
size_t so4_adjoint_workspace_size(const so4_tables *t, int natoms, int64_t nimg);
int so4_adjoint32(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                  const int *d_atom_ptr, int natoms, const double *d_w_nb, const int32_t *d_img_ptr,
                  const int32_t *d_img_j, const double *d_img_r, const int32_t *d_img_rev,
                  int64_t nimg, const float *d_utot, const float *d_beta, double *d_forces,
                  double *d_virial, void *d_work, size_t work_bytes, void *stream);

/* The three stages so4_adjoint32 runs, for callers that keep their own buffers:
 *   so4_adjoint_y32      Y[natoms*idxu_half*2] f32 from U_tot and beta (atoms across lanes),
 *                        each half entry (l, mb, ma) stored times sqrt(C(l, mb) / C(l, ma))
 *                        (C binomial), the row scale of the recursion so4_adjoint_deidrj32
 *                        runs; a buffer for that call, not a result to read;
 *   so4_adjoint_deidrj32 g[m*3] f32 = dE/dr of every image m of the natoms centres,
 *                        m in [d_img_ptr[0], d_img_ptr[natoms]) (U and dU by the
 *                        recursion, contracted with Y); nimg bounds the number of those
 *                        images (a capacity will do).  d_img_ptr, d_y and the per-atom
 *                        arrays may point at a range of centres of a longer list, d_g
 *                        and the per-image arrays being that list's;
 *   so4_adjoint_gather   forces[natoms*3] f64 = sum_m (g_m - g_rev(m)), the
 *                        per-structure virial[nstruct*9] f64 = sum_m r_m (x) g_m and,
 *                        when d_eatom and d_energy are both non-NULL, energy[nstruct] f64 =
 *                        the sum of the per-atom d_eatom[natoms] f32 over each structure.
 *                        All sums have a fixed order (bitwise reproducible).  d_part:
 *                        so4_gather_workspace_size(natoms) bytes of scratch. */
int so4_adjoint_y32(const so4_tables *t, int natoms, const float *d_utot, const float *d_beta, float *d_y,
                    void *stream);
int so4_adjoint_deidrj32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
                         const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                         int64_t nimg, const float *d_y, float *d_g, void *stream);
size_t so4_gather_workspace_size(int natoms);
int so4_adjoint_gather(int natoms, int nstruct, const int *d_atom_ptr, const int32_t *d_img_ptr,
                       const int32_t *d_img_rev, const double *d_img_r, const float *d_g,
                       const float *d_eatom, double *d_part, double *d_forces, double *d_virial,
                       double *d_energy, void *stream);

/* Forward and adjoint in one call for an energy linear in B (beta = dE/dB does not
 * depend on B, e.g. the reference's order-1 polynomial regression,
 * pyxtal_ff/models/polynomialregression.py:374): writes d_x (B, natoms*nB f32),
 * d_forces and d_virial as so4_forward32 + so4_adjoint32 would, with every Z entry
 * computed once for both B and Y, and, when d_energy is non-NULL, d_energy[nstruct]
 * f64 = sum over the structure's atoms of beta_i . B_i (a model's constant term is
 * the caller's to add).  Scratch: so4_linear_workspace_size() bytes. */
size_t so4_linear_workspace_size(const so4_tables *t, int natoms, int64_t nimg);
/* Its stages: U_tot alone (the first half of so4_forward32), then B and Y from U_tot
 * and beta in one pass (d_bc: sizes[6] * natoms floats of scratch, entry-major;
 * d_eatom[natoms] f32 = beta_i . B_i, may be NULL), then so4_adjoint_deidrj32 and
 * so4_adjoint_gather. */
int so4_utot32(const so4_tables *t, const so4_params *p, int natoms, const double *d_w_nb,
               const double *d_w_site, const int32_t *d_img_ptr, const int32_t *d_img_j,
               const double *d_img_r, float *d_utot, void *stream);
int so4_linear_by32(const so4_tables *t, int natoms, const float *d_utot, const float *d_beta, float *d_x,
                    float *d_y, float *d_bc, float *d_eatom, void *stream);
int so4_adjoint_linear32(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                         const int *d_atom_ptr, int natoms, const double *d_w_nb, const double *d_w_site,
                         const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
                         const int32_t *d_img_rev, int64_t nimg, const float *d_beta, float *d_x,
                         double *d_forces, double *d_virial, double *d_energy, void *d_work,
                         size_t work_bytes, void *stream);

/* The adjoint's backward: the Jacobian-vector product of B (FP32),
 *   d_dB[natoms*nB] = sum_{images m of i} dB_i/dr_m . dr_m,  dr_m = (v_j - v_i) + G_s^T r_m,
 * for per-atom vectors d_v[natoms*3] (f64, may be NULL) and per-structure
 * matrices d_G[nstruct*9] (f64, row-major G_ab, may be NULL; then d_atom_struct
 * is not read).  With v = -dL/dF and G = dL/dW it gives dL/dbeta for the forces
 * and virial of so4_adjoint32, i.e. the gradient a force/stress loss sends back
 * into an energy model.  Scratch: so4_jvp_workspace_size() bytes.  Built for twol
 * 2 to 12; SO4_ERR_UNSUPPORTED at twol 0 and 1. */
size_t so4_jvp_workspace_size(const so4_tables *t, int natoms);
int so4_jvp32(const so4_tables *t, const so4_params *p, const int *d_atom_struct, int natoms,
              const double *d_w_nb, const int32_t *d_img_ptr, const int32_t *d_img_j, const double *d_img_r,
              const float *d_utot, const double *d_v, const double *d_G, float *d_dB, void *d_work,
              size_t work_bytes, void *stream);

/* so4_adjoint32 for callers that cannot allocate device memory.  No counterpart
 * in the reference (whose CPU code has no device allocator to avoid).
 * Same arguments as so4_adjoint32 without the workspace: the scratch comes from
 * a fixed array of SO4_NOALLOC_SCRATCH_BYTES that every GPU loading the library
 * holds until exit.  Problems whose so4_adjoint_workspace_size() exceeds it
 * return SO4_ERR_TOO_LARGE.  The first call on each device looks up the
 * array's address (make it before any stream capture) and keeps it, so the
 * entry point must not be used across a cudaDeviceReset; calls that overlap on
 * the GPU race on the shared array.  Allocates nothing. */
#define SO4_NOALLOC_SCRATCH_BYTES (64u << 20)
int so4_adjoint32_noalloc(const so4_tables *t, const so4_params *p, int nstruct, const int *d_atom_struct,
                          const int *d_atom_ptr, int natoms, const double *d_w_nb, const int32_t *d_img_ptr,
                          const int32_t *d_img_j, const double *d_img_r, const int32_t *d_img_rev,
                          int64_t nimg, const float *d_utot, const float *d_beta, double *d_forces,
                          double *d_virial, void *stream);

/* FMA throughput loop (measurement aid, no counterpart in the reference): blocks CTAs
 * of 256 threads, each thread running 8 independent FMA chains for `iters` iterations;
 * kind 0 packed FP32 pairs (fma.rn.f32x2), 1 scalar FP32, 2 FP64.  Writes one float per
 * thread to d_out[blocks * 256] and the launch's flop count to *h_flop; time it on
 * `stream`. */
int so4_peak_fma(int kind, int iters, int blocks, float *d_out, double *h_flop, void *stream);

/* Number of kernels this library has launched since it was loaded. */
long long so4_launch_count(void);

/* Programmatic dependent launch for the calling host thread's launches of U_tot
 * (so4_utot32 and the forward), the window Z pass (so4_linear_by32, so4_adjoint_y32
 * and the other window modes) and the per-image pass (so4_adjoint_deidrj32): with
 * on != 0 each may be scheduled while the kernel before it in the stream finishes
 * (its set-up overlaps that kernel's tail) and waits on the device for that kernel's
 * results before reading them.  Off by default.  Only turn it on for a stream in which
 * nothing between two of these launches writes the constant inputs they read before
 * that wait (tables, beta): the captured step of a linear energy (a fixed beta) is
 * such a stream.  No counterpart in the reference (its driver loop,
 * pyxtal_ff/descriptors/SO4.py:1414-1548, is one serial CPU loop).  Returns the
 * previous setting. */
int so4_set_pdl(int on);

/* Library version string. */
const char *so4_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SO4_GB300_H */
