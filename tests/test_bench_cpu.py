"""bench.py's choice of the roofline kernel, on kernel-time records made up
on the host: a launch that overlapped a launch on another stream does not
count towards the dominant kernel."""
import bench


def rec(name, start, ms):
    return {"name": name, "start_ms": start, "ms": ms, "rows": 1, "bytes": 1}


def test_launch_overlaps():
    run = [rec("probe_scatter", 0.0, 2.0), rec("build_scatter", 0.5, 1.0), rec("probe_lookup", 2.0, 1.0),
           rec("probe_project", 3.0, 2.5)]
    assert [bench.launch_overlaps(run, i) for i in range(4)] == [True, True, False, False]
    # back-to-back launches of one stream touch but do not overlap
    assert not bench.launch_overlaps([rec("a", 0.0, 1.0), rec("b", 1.0, 1.0)], 0)


def test_profiled_traffic_scales_with_rows():
    full = bench.profiled_traffic("probe_project", "c2")
    assert full and full > 10e9  # a full-size launch moves about 12 GB
    assert bench.profiled_traffic("probe_project", "c2", 0.125) == int(full * 0.125)
    assert bench.profiled_traffic("no_such_kernel", "c2") is None
