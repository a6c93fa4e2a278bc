"""The benchmark's workload definition (bench.py), checked on the CPU."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))


def test_bench_camera_stays_on_the_32_frame_path():
    """Runs longer than the configuration's 32-frame camera path play it forward, then
    back: every frame is one path step (0.01 units, 0.2 degrees) away from the last
    and inside the path's range, and after 64 frames the camera is back at its start."""
    import types

    import bench

    cam = types.SimpleNamespace(position=[0.0, 1.0, 5.0], yaw_deg=10.0)
    z0, yaw0 = cam.position[2], cam.yaw_deg
    zs, yaws = [], []
    for f in range(96):
        before = (cam.position[2], cam.yaw_deg)
        bench.move_camera(cam, f)
        assert abs(abs(cam.position[2] - before[0]) - 0.01) < 1e-9
        assert abs(abs(cam.yaw_deg - before[1]) - 0.2) < 1e-9
        zs.append(cam.position[2])
        yaws.append(cam.yaw_deg)
    assert min(zs) >= z0 - 0.01 * bench.PATH_FRAMES - 1e-9 and max(zs) <= z0 + 1e-9
    assert max(yaws) <= yaw0 + 0.2 * bench.PATH_FRAMES + 1e-9 and min(yaws) >= yaw0 - 1e-9
    assert abs(zs[63] - z0) < 1e-9 and abs(yaws[63] - yaw0) < 1e-9


def test_reference_arm_prints_the_contract_line():
    """The reference arm (the oracle's restatement of the reference's shaders on the host
    cores) on a small frame: one JSON line with the arm's own value as e2e and as its
    cpu_baseline, no host-device bytes, and at least three warm-up frames."""
    import json
    import os
    import subprocess

    import bench

    root = Path(__file__).resolve().parents[1]
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--width", "96", "--height", "64"],
                         cwd=root, capture_output=True, text=True, timeout=600,
                         env={k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")})
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "ms/frame" and line["higher_is_better"] is False and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] >= 3 and line["n_gpus"] == 1
    assert line["config"]["resolution"] == [96, 64]
    assert line["e2e"] == {"value": line["value"], "unit": "ms/frame", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] == os.cpu_count()
