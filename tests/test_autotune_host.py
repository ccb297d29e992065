"""The autotuner's search and cache logic, on the CPU (no GPU, synthetic costs).

The GPU side (each candidate's check against the FP64 plain path, timing, and the
tuned kernels' parity with the oracle) is in tests/test_gpu_autotune.py."""
import dataclasses
import json

import pytest

from pyxtal_ff_gb300 import autotune as T


def _cost(best):
    """A separable synthetic cost whose minimum is `best`; evaluations are counted."""
    calls = []

    def f(c):
        calls.append(c)
        t = 1.0
        t += 0.1 * abs(c.branches - best.branches)
        t += 0.05 * abs(c.wkmax - best.wkmax)
        t += 0.07 * (c.rev_threads != best.rev_threads)
        t += 0.03 * abs(c.utot_warps - best.utot_warps) / 2
        t += 0.02 * (c.pdl != best.pdl)
        t += 0.04 * (c.rev_pair != best.rev_pair)
        return t
    return f, calls


def test_coordinate_descent_finds_the_separable_optimum_and_evaluates_each_choice_once():
    best = T.Choice(wkmax=3, rev_threads=128, utot_warps=8, branches=3, pdl=True, rev_pair=2)
    f, calls = _cost(best)
    start = T.default_choice(8)
    got, t, table = T.coordinate_descent(f, start, T.search_space(8))
    assert got == best and t == pytest.approx(1.0)
    assert len(calls) == len(set(calls)) == len(table)


def test_coordinate_descent_never_picks_a_rejected_choice():
    best = T.Choice(wkmax=3, rev_threads=128, utot_warps=8, branches=3, pdl=True)
    f, _ = _cost(best)
    bad = {dataclasses.replace(T.default_choice(8), wkmax=3), dataclasses.replace(T.default_choice(8), branches=3)}

    def g(c):
        # a candidate that fails its check anywhere in the space with wkmax 3 or 3 branches
        if c.wkmax == 3 or c.branches == 3 or c in bad:
            return None
        return f(c)
    got, t, table = T.coordinate_descent(g, T.default_choice(8), T.search_space(8))
    assert got.wkmax != 3 and got.branches != 3
    assert all(tt is None for c, tt in table if c.wkmax == 3 or c.branches == 3)
    assert t == min(tt for _, tt in table if tt is not None)


def test_coordinate_descent_raises_when_the_start_fails():
    with pytest.raises(RuntimeError):
        T.coordinate_descent(lambda c: None, T.default_choice(6), T.search_space(6))


def test_min_gain_keeps_the_default_on_a_flat_cost():
    start = T.default_choice(8)
    got, _, _ = T.coordinate_descent(lambda c: 1.0 - 0.001 * (c.branches == 4), start, T.search_space(8),
                                     min_gain=0.01)
    assert got == start


def test_search_space_by_twol_and_step_kind():
    s8, s4 = T.search_space(8), T.search_space(4)
    assert s8["rev_threads"] == (256, 128) and s8["utot_warps"] == (4, 2, 8) and s8["rev_pair"] == (0, 1, 2)
    assert s4["rev_threads"] == (0,) and s4["utot_warps"] == (4,) and s4["rev_pair"] == (0,)
    assert s8["zw_atoms"] == (32, 64) and s8["zw_threads"] == (256, 512)
    assert T.search_space(10)["zw_atoms"] == (0,)  # the 64-atom tiles exceed shared memory above twol 8
    m = T.search_space(6, linear=False)
    assert m["branches"] == (1,) and m["pdl"] == (False,)
    assert T.default_choice(8, linear=False).branches == 1


def test_cache_round_trip_and_bad_file(tmp_path):
    p = tmp_path / "sub" / "tuning.json"
    c = T.TuningCache(str(p))
    assert c.get("k") is None
    ch = T.Choice(wkmax=4, rev_threads=128, utot_warps=2, branches=3, pdl=True)
    c.put("k", ch, 1.25)
    c.put("k2", T.Choice(), 2.0)
    assert c.get("k") == (ch, 1.25)
    assert json.load(open(p))["k"]["choice"]["wkmax"] == 4
    p.write_text("{not json")
    assert T.TuningCache(str(p)).get("k") is None
    T.TuningCache(str(p)).put("k", ch, 1.0)  # a corrupt file is replaced
    assert T.TuningCache(str(p)).get("k") == (ch, 1.0)


def test_cache_path_from_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("SO4_TUNE_CACHE", str(tmp_path / "t.json"))
    assert T.cache_path() == str(tmp_path / "t.json")


def test_workload_key_classes():
    k1 = T.workload_key("GB300", 8, 32000, 928000, 1, "linear")
    k2 = T.workload_key("GB300", 8, 30000, 870000, 1, "linear")
    k3 = T.workload_key("GB300", 8, 32000, 928000, 1, "train")
    k4 = T.workload_key("GB300", 6, 32000, 928000, 1, "linear")
    assert k1 == k2 and k1 != k3 and k1 != k4


def test_choice_dict_round_trip_and_kernel_tuning():
    ch = T.Choice(wkmax=4, rev_threads=128, utot_warps=8, branches=1, pdl=True, rev_pair=1)
    assert T.Choice.from_dict(ch.as_dict()) == ch
    assert ch.kernel_tuning() == (4, 128, 8, 1, 0, 0)
    assert T.Choice(zw_atoms=64, zw_threads=512).kernel_tuning()[4:] == (64, 512)
    # a cached choice written before a knob existed reads back with that knob's default
    old = {"wkmax": 4, "rev_threads": 128, "utot_warps": 8, "branches": 1, "pdl": True}
    assert T.Choice.from_dict(old).rev_pair == 0
