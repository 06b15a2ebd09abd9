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


def test_reference_arm_loads_no_product_library(tmp_path):
    """The reference arm times the CPU restatement on inputs from the host-only generators:
    its process maps the oracle and libvrt_synth.so, never the product library libvrt.so."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(bench.__file__).resolve().parent
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--worlds', '2', '--max-views', '1', "
            "'--steps', '1', '--warmup', '0', '--cpu-seconds', '0.1']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'libvrt.so' in maps, 'libvrt_synth.so' in maps, 'libvrt_oracle.so' in maps)")
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
    assert '"impl": "reference"' in line
    assert "MAPS False True True" in r.stdout


def test_profiled_traffic_not_for_a_smaller_large_world():
    assert bench.traffic_from_profile("large_world", bench.parse(["--workload", "large_world", "--cameras", "8"])) is None


def test_scaled_camera_keeps_the_image_plane():
    """The oracle checks of the renderer rows run a smaller view of the same camera: the
    plane's corner d0 and its far corner d0 + W*du + H*dv stay where they were."""
    import numpy as np
    cam = v.look_at((100.5, 80.0, 30.0), (400.0, 60.0, 900.0), 90.0, 1920, 1080)
    sc = bench._scaled_camera(v, cam, 320, 180)
    assert (sc.width, sc.height) == (320, 180)
    assert list(sc.origin) == list(cam.origin) and list(sc.world_origin) == list(cam.world_origin)
    d0, du, dv = (np.array(getattr(cam, k)[:], np.float64) for k in ("d0", "du", "dv"))
    s0, su, sv = (np.array(getattr(sc, k)[:], np.float64) for k in ("d0", "du", "dv"))
    assert np.array_equal(s0, d0)
    assert np.allclose(s0 + 320 * su + 180 * sv, d0 + 1920 * du + 1080 * dv, rtol=1e-6, atol=1e-6)
