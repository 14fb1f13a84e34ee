"""The committed ncu summaries that bench.py reads: each names the command
that produced it and gives the DRAM bytes per launch of the frame's kernel,
for the one-kernel frame and for the two-kernel frame's primary kernel."""

from __future__ import annotations

import bench


def test_bench_reads_profiled_traffic():
    fused = bench.profiled_traffic(True)
    two = bench.profiled_traffic(False)
    assert fused is not None and two is not None
    # a few MB per 1080p launch: the BVH and the touched triangles come from L2/L1
    assert 1e6 < fused < 1e8 and 1e6 < two < 1e8


def test_profile_summaries_name_their_commands():
    root = bench.ROOT / "profiles"
    files = sorted(root.glob("*.md")) + sorted(root.glob("*.txt"))
    assert files
    for f in files:
        text = f.read_text()
        assert "ncu " in text or "ncu\n" in text, f.name
        assert "--clock-control none" in text, f.name


def test_issue_roofline_arithmetic():
    """The bench line's roofline: the committed capture's warp instructions
    over the launch's event time, against 4 warp instructions per cycle per
    SM at the sampled clock; the HBM fraction from the captured DRAM bytes."""
    prof = bench.profiled_metrics(True)
    launch_s = 0.3927e-3
    r = bench.issue_roofline(prof, launch_s, 2070.0, 152, 5_031_338_432, prof["dram_bytes_per_launch"], 6786.2,
                             "measured")
    inst = prof["warp_instructions_per_launch"]
    assert r["bound"] == "issue"
    assert abs(r["achieved"] - inst / launch_s / 1e9) < 0.1
    assert abs(r["peak"] - 4 * 152 * 2.070) < 0.1
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3
    assert 0.3 < r["frac"] <= 1.0                      # a fraction of the issue roof, not a multiple
    assert r["hbm"]["frac"] < 0.05                     # HBM is not the bound
    assert abs(r["algorithmic_gbs"] - 5_031_338_432 / launch_s / 1e9) < 0.1
    assert set(r["ncu_fracs"]) == {"issue_active_frac", "l1_throughput_frac", "l2_throughput_frac",
                                   "dram_throughput_frac"}
