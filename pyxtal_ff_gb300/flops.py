"""Algorithmic floating-point work of each kernel, counted from the index tables.

Convention: complex multiply 6 flop, complex add 2, real x complex 2, and
Re(conj(a) b) 4 (two multiply-adds); a fused multiply-add counts 2.  The loops
counted are the reference's (pyxtal_ff/descriptors/SO4.py), not the kernels'
own bookkeeping:

  U     per image   the recursion over the left-half rows of every level
                    (compute_uarray_recursive :888-906): per entry, each of its
                    one or two terms is a complex multiply and a real scaling
                    (8), plus 2 per extra term;
  dU    per image   the same entries, three components, each term
                    conj(da) U + conj(a) dU scaled (16 per component), plus 6
                    per extra term (compute_duarray_recursive :950-968);
  Utot  per image   (w U) sfac accumulated: 6 per half entry (add_uarraytot);
  Z     per atom    sum_ib [na (2 + 6 + 2) + 4] per Z entry (compute_zi);
  B     per atom    4 per summed entry + 2 per component (compute_bi);
  dB    per image   per component k, three sections of 4 dot products
                    (sfac dU_c and r^ U against Z) = 16 per summed entry,
                    plus 18 for the virial outer product (compute_dbidrj :1113-1227
                    and the bstress update :1466-1468);
  Y     per atom    4 flop per (Z entry, role) plus the Z entries themselves;
  B+Y   per atom    the fused pass of a linear energy: Z once, then B and Y;
  dE    per image   U + dU + 4 dot products against Y (16 per half entry).
"""
from __future__ import annotations


def _blocks(twol):
    for l1 in range(twol + 1):
        for l2 in range(l1 + 1):
            for l in range(l1 - l2, min(twol, l1 + l2) + 1, 2):
                yield l1, l2, l


def sizes(twol):
    n_half = sum((l // 2 + 1) * (l + 1) for l in range(twol + 1))
    n_u = sum((l + 1) ** 2 for l in range(twol + 1))
    nB = sum(1 for (l1, l2, l) in _blocks(twol) if l >= l1)
    n_z = sum((l // 2 + 1) * (l + 1) for (l1, l2, l) in _blocks(twol))
    return dict(n_half=n_half, n_u=n_u, nB=nB, n_z=n_z)


def _section(lam):
    return ((lam + 1) // 2) * (lam + 1) + ((lam // 2 + 1) if lam % 2 == 0 else 0)


def per_image_u(twol):
    f = 0
    for l in range(1, twol + 1):
        for mb in range(l // 2 + 1):
            for ma in range(l + 1):
                t = (ma > 0) + (ma < l)
                f += 8 * t + 2 * (t - 1)
    return f


def per_image_du(twol):
    f = 0
    for l in range(1, twol + 1):
        for mb in range(l // 2 + 1):
            for ma in range(l + 1):
                t = (ma > 0) + (ma < l)
                f += 3 * 16 * t + 6 * (t - 1)
    return f


def _row_len(l, mb, cut_middle):
    # the window kernels stop an even level's middle row at its centre
    return l // 2 + 1 if (cut_middle and 2 * mb == l) else l + 1


def per_atom_z(twol, cut_middle=False):
    f = 0
    for (l1, l2, l) in _blocks(twol):
        for mb in range(l // 2 + 1):
            for ma in range(_row_len(l, mb, cut_middle)):
                ma1min = max(0, (2 * ma - l - l2 + l1) // 2)
                na = min(l1, (2 * ma - l + l2 + l1) // 2) - ma1min + 1
                mb1min = max(0, (2 * mb - l - l2 + l1) // 2)
                nb = min(l1, (2 * mb - l + l2 + l1) // 2) - mb1min + 1
                f += nb * (na * 10 + 4)
    return f


def per_atom_z_b_blocks(twol):
    """Z work restricted to the blocks B reads (l >= l1)."""
    f = 0
    for (l1, l2, l) in _blocks(twol):
        if l < l1:
            continue
        for mb in range(l // 2 + 1):
            for ma in range(l + 1):
                ma1min = max(0, (2 * ma - l - l2 + l1) // 2)
                na = min(l1, (2 * ma - l + l2 + l1) // 2) - ma1min + 1
                mb1min = max(0, (2 * mb - l - l2 + l1) // 2)
                nb = min(l1, (2 * mb - l + l2 + l1) // 2) - mb1min + 1
                f += nb * (na * 10 + 4)
    return f


def per_atom_b(twol):
    return sum(4 * _section(l) + 2 for (l1, l2, l) in _blocks(twol) if l >= l1)


def per_image_db(twol):
    f = 0
    for (l1, l2, l) in _blocks(twol):
        if l < l1:
            continue
        f += 16 * (_section(l) + _section(l1) + _section(l2)) + 3 * 6 + 18
    return f


def per_atom_y(twol, cut_middle=False):
    roles = 0
    for (l1, l2, l) in _blocks(twol):
        if l < l1:
            continue
        roles += 3
    nz = sum(_row_len(l, mb, cut_middle) for (l1, l2, l) in _blocks(twol) for mb in range(l // 2 + 1))
    # each Y entry gathers one complex scale-add per contributing block entry
    return 4 * nz + 2 * roles


def per_image_rev(twol):
    """The reverse-mode per-image contraction: the forward sweep of U, then per row entry
    of every level the adjoint step (the gradient pairs of conj(a), conj(b): 16 flop; the
    new adjoint a G - b H: 14) and the Y terms (f and the carry: 6), and the final
    Jacobian dot products and weights (about 60)."""
    f = per_image_u(twol)
    for l in range(1, twol + 1):
        for mb in range(l // 2 + 1):
            f += 30 * l + 6 * (l + 1)
    return f + 60


def per_image_jvp(twol):
    """The JVP's per-image pass: the U recursion, its tangent along one direction (one
    component of the dU recursion) and the tangent of U_tot accumulated (8 per half entry)."""
    return per_image_u(twol) + per_image_du(twol) // 3 + 8 * sizes(twol)["n_half"]


def kernel_flops(twol, natoms, nimg):
    """Flops of one launch of each kernel for a batch, counted from the algorithm each
    kernel runs (the window kernels' Z with middle rows cut at the centre, the reverse-mode
    per-image contraction; an upper bound where the windows also skip the mirrored row
    pairs of symmetric blocks)."""
    n = sizes(twol)
    u, du, z = per_image_u(twol), per_image_du(twol), per_atom_z(twol)
    zc = per_atom_z(twol, cut_middle=True)
    utot_img = u + 6 * n["n_half"]
    return {
        "utot32": nimg * utot_img,
        "linear_by32": natoms * (zc + per_atom_b(twol) + per_atom_y(twol, cut_middle=True)),
        "forward32": natoms * (zc + per_atom_b(twol)) + nimg * utot_img,
        "adjoint_y32": natoms * (zc + per_atom_y(twol, cut_middle=True)),
        "adjoint_deidrj32": nimg * per_image_rev(twol),
        # the JVP: the per-image tangent pass, then the window pass's Z once per atom contracted
        # with the tangent per (block, role) like Y (so4_jvp32)
        "jvp32": nimg * per_image_jvp(twol) + natoms * (zc + per_atom_y(twol, cut_middle=True)),
        "plain": natoms * (z + per_atom_b(twol)) + nimg * (utot_img + u + du + per_image_db(twol)),
    }


# Per-unit algorithmic work of the reference's algorithm as tabulated for this path
# (U, dU, dudr, dB/dr and virial per neighbour image; Z, B and the adjoint per atom),
# for lmax 3 and 4: the figures a launch's roofline is quoted against.
TABULATED_UNITS = {
    6: dict(U=1240, dU=6696, dudr=4200, dB=24816, virial=1080, Z=98076, B=3824, adj_img=12600, adj_atom=200000),
    8: dict(U=2600, dU=14040, dudr=8550, dB=72072, virial=1980, Z=455702, B=11304, adj_img=27000, adj_atom=900000),
}


def tabulated_flops(twol, natoms, nimg):
    """Algorithmic flops of one launch of each stage from the tabulated per-unit work
    (None where the table has no entry for this twol): U_tot per image; Z + Y (+ B) per
    atom; the adjoint per image; the plain path's full per-image and per-atom work."""
    t = TABULATED_UNITS.get(int(twol))
    if t is None:
        return None
    return {
        "utot32": nimg * t["U"],
        "linear_by32": natoms * (t["adj_atom"] + t["B"]),
        "adjoint_y32": natoms * t["adj_atom"],
        "adjoint_deidrj32": nimg * t["adj_img"],
        "plain": natoms * (t["Z"] + t["B"]) + nimg * (t["U"] + t["dU"] + t["dudr"] + t["dB"] + t["virial"]),
    }
