"""bench.py's host-side figures, on the CPU: the ncu-derived traffic and
instruction counts it reads from the committed profile, and the issue bound."""
import bench


def test_profile_figures_are_read():
    for k in ("k_lambda", "k_correction"):
        t = bench.ncu_traffic(k)
        i = bench.ncu_warp_instructions(k)
        assert t is not None and 1e7 < t < 1e10
        assert i is not None and 1e6 < i < 1e10
    assert bench.ncu_traffic("k_other") is None
    assert bench.ncu_warp_instructions("k_other") is None


def test_issue_bound():
    r = bench.issue_bound("k_lambda", 0.09)
    assert r["unit"] == "T warp instructions/s"
    assert 1.0 < r["peak"] < 1.5
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert 0.0 < r["frac"] < 1.5
    assert bench.issue_bound("k_lambda", 0.0) is None


def test_method_label():
    assert "16 local inputs" in bench.method_of({"features": "base"})
    assert "16 local inputs" not in bench.method_of({"features": "all"})
