"""CPU checks of bench.py's command line: `--gpus N` started without a launcher starts N ranks
itself (the launcher check runs gloo ranks, no GPU), and the reference arm builds its inputs and
times the frame without loading the product library."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _last_json(out: str) -> dict:
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert lines, out[-2000:]
    return json.loads(lines[-1])


def test_gpus_two_starts_two_ranks():
    proc = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--launch-check"],
                          capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert proc.returncode == 0, proc.stderr[-2000:]
    line = _last_json(proc.stdout)
    assert line["launch_check"] is True and line["n_gpus"] == 2
    assert sorted(r["rank"] for r in line["ranks"]) == [0, 1]
    assert len({r["pid"] for r in line["ranks"]}) == 2


SCRIPT = r"""
import json, sys, types
sys.path.insert(0, {root!r})
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
import bench
from webgs import workloads as W
W.SCENE_1M = W.SceneSpec(20_000, 1, 1, 64, 20.0)          # a small scene: the check is what gets loaded
W.CAMERA_1080P = W.CameraSpec((0.0, 1.0, -9.0), (0.0, 0.0, 0.0), 70.0, 320, 180)
bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({{"libwebgs": "libwebgs.so" in maps, "liboracle": "liboracle.so" in maps}}))
"""


def test_reference_arm_loads_only_the_oracle():
    proc = subprocess.run([sys.executable, "-c", SCRIPT.format(root=str(ROOT))], capture_output=True, text=True,
                          timeout=300, cwd=ROOT)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [json.loads(ln) for ln in proc.stdout.splitlines() if ln.startswith("{")]
    ref, maps = lines[-2], lines[-1]
    assert ref["impl"] == "reference" and ref["value"] > 0 and ref["cpu_baseline"]["kind"] == "port"
    assert maps == {"libwebgs": False, "liboracle": True}
