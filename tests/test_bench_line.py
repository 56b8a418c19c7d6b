"""The bench line's figures taken from the committed ncu summaries: DRAM traffic per launch and the
issue-slot fractions of the dominant tile kernels parse, and lie in their physical ranges."""
import bench


def test_profiled_traffic_of_the_headline_frames():
    for name, algorithmic in (("c5", 708_385_684), ("c2", 119_064_404)):
        traffic = bench.profiled_traffic(name)
        assert traffic is not None
        assert algorithmic < traffic < 10 * algorithmic


def test_profiled_issue_fractions():
    c5 = bench.profiled_issue("c5")
    assert set(c5) == {"raster_kernel<8,16>", "shade_kernel<8,16>", "forward_kernel<8>"}
    c2 = bench.profiled_issue("c2")
    assert set(c2) == {"raster_kernel<4,16>", "shade_kernel<4,16>"}
    for v in list(c5.values()) + list(c2.values()):
        assert 0.0 < v <= 1.0
    assert bench.profiled_issue("no such workload") is None
