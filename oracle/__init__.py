"""CPU oracle for the SO4/SNAP bispectrum path -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
reference arm) may import this package, and only as the checker or the timed
CPU baseline.  The product package pyxtal_ff_gb300 never imports it.
"""
