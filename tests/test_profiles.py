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
