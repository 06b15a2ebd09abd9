"""bench.py's host-side helpers (no GPU): the DRAM traffic taken from the committed ncu
summary belongs to the configuration that summary covers only, and the traversal-mode
flags reach every view of the workload."""
import bench
import voxelrt_gb300 as v


def test_profiled_traffic_only_for_the_profiled_configuration():
    base = bench.traffic_from_profile("uneven_batch", bench.parse([]))
    assert base is not None and base > 0
    for argv in (["--aniso"], ["--glsl"], ["--worlds", "24"], ["--max-views", "8"]):
        assert bench.traffic_from_profile("uneven_batch", bench.parse(argv)) is None, argv
    assert bench.traffic_from_profile("large_world", bench.parse(["--workload", "large_world"])) is None


def test_mode_flags_reach_every_view():
    small = ["--worlds", "3", "--max-views", "2"]
    for argv, want in (([], 0), (["--glsl"], v.VIEW_GLSL), (["--aniso"], v.VIEW_GLSL | v.capi.VIEW_GLSL_ANISO)):
        args = bench.parse(small + argv)
        wl = bench.build_workload("uneven_batch", 0, args)
        assert wl.views and all((vw.flags & (v.VIEW_GLSL | v.capi.VIEW_GLSL_ANISO)) == want for vw in wl.views)
        assert bench.traversal_name(args) == {0: "cpu", v.VIEW_GLSL: "glsl"}.get(want, "glsl_aniso")
