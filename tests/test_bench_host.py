"""bench.py's host-side figures, on the CPU: the ncu-derived traffic and
instruction counts it reads from the committed profile (only while the
profile was captured from the current kernel sources), the issue bound and
the whole-step byte model."""
import bench


def test_profile_figures_are_read(monkeypatch):
    monkeypatch.setattr(bench, "profile_current", lambda: True)
    for k in ("k_lambda", "k_correction"):
        t = bench.ncu_traffic(k)
        i = bench.ncu_warp_instructions(k)
        assert t is not None and 1e7 < t < 1e10
        assert i is not None and 1e6 < i < 1e10
        l1 = bench.ncu_l1tex(k)
        assert l1 is not None and 0.0 < l1["pct_of_peak_active"] <= 100.0
    assert bench.ncu_l1tex("k_other") is None
    assert bench.ncu_traffic("k_other") is None
    assert bench.ncu_warp_instructions("k_other") is None


def test_stale_profile_figures_are_dropped(monkeypatch):
    monkeypatch.setattr(bench, "profile_digest", lambda: "000000000000")
    assert not bench.profile_current()
    assert bench.ncu_traffic("k_lambda") is None
    assert bench.ncu_warp_instructions("k_lambda") is None
    assert bench.ncu_l1tex("k_lambda") is None
    d = bench.kernel_sources_digest()
    assert len(d) == 12 and int(d, 16) >= 0
    monkeypatch.setattr(bench, "profile_digest", lambda: d)
    assert bench.profile_current()


def test_issue_bound(monkeypatch):
    monkeypatch.setattr(bench, "profile_current", lambda: True)
    r = bench.issue_bound("k_lambda", 0.09)
    assert r["unit"] == "T warp instructions/s"
    assert 1.0 < r["peak"] < 1.5
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert 0.0 < r["frac"] < 1.5
    assert bench.issue_bound("k_lambda", 0.0) is None


def test_step_bytes():
    # B(I) = 396 + 60 I; the configured 4-iteration step is 636 B
    assert bench.step_bytes(4) == 636.0
    assert bench.step_bytes(10, warm_start=True) == 396.0 + 600.0 + 80.0
    r = bench.step_roofline(1e8, 4, 1.0)
    assert abs(r["achieved"] - 1e8 * 636.0 / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12


def test_method_label():
    assert "16 local inputs" in bench.method_of({"features": "base"})
    assert "16 local inputs" not in bench.method_of({"features": "all"})
