"""The work counts behind the roofline (pyxtal_ff_gb300/flops.py), on the CPU: the index
table sizes the counts iterate over equal the reference's (SO4.py:1265-1396, counted at
lmax 3 and 4: idxu, its half used by dB/dr, nB, idxz), the Z count equals the tabulated
per-atom Z work, and the counts of this code's own algorithms keep their known values."""
from pyxtal_ff_gb300 import flops as F


def test_table_sizes_match_reference():
    assert F.sizes(6) == dict(n_half=78, n_u=140, nB=30, n_z=779)
    assert F.sizes(8) == dict(n_half=155, n_u=285, nB=55, n_z=2386)
    # the reference's closed form for nB (SO4.py:299)
    for lmax in range(0, 7):
        assert F.sizes(2 * lmax)["nB"] == round((lmax + 1) * (lmax + 2) * (lmax + 1.5) // 3)


def test_z_count_matches_tabulated_units():
    for twol in (6, 8):
        assert F.per_atom_z(twol) == F.TABULATED_UNITS[twol]["Z"]


def test_executed_counts():
    # middle rows of even levels cut at their centre: 8 % less Z work at lmax 4
    assert F.per_atom_z(8, cut_middle=True) == 417224
    assert F.per_image_u(8) == 2292
    assert F.per_image_u(8) + 6 * F.sizes(8)["n_half"] == 3222
    assert F.per_image_rev(8) == 7176
    k = F.kernel_flops(8, 32000, 928000)
    t = F.tabulated_flops(8, 32000, 928000)
    assert k["utot32"] == 928000 * 3222
    assert t["linear_by32"] == 32000 * (900000 + 11304)
    # the reverse-mode pass does far less arithmetic than the tabulated dB/dr work
    assert k["adjoint_deidrj32"] < t["adjoint_deidrj32"] / 3
    assert F.tabulated_flops(10, 1, 1) is None
