"""The checked build (libwebgs_checked.so, -DGS_CHECKED): the stand-in for a memory sanitizer, which
is not available on this machine. Every device buffer of a context carries a canary pad on either side
that a kernel verifies after each forward, batch and backward, and data-dependent store indices are
tested against their buffers; a violation is recorded in the frame's status word (no trap) and the
call returns GS_ERR_MEMORY.

1. The GPU parity suites run once under the checked build, in a child process with WEBGS_CHECKED=1:
   every test passes there, so no frame, batch, scan, sort or backward of those suites stored out of
   bounds or touched a pad.
2. A canary word damaged on purpose, from the host, inside the pad the checked build allocated (no
   kernel writes out of bounds), is reported by the next frame and leaves the context usable.
"""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

SUITES = ["test_gpu_parity.py", "test_gpu_batch.py", "test_gpu_backward.py", "test_gpu_primitives.py",
          "test_gpu_hostile.py", "test_gpu_camera.py", "test_gpu_seq_wrap.py", "test_gpu_dropin.py",
          "test_gpu_failure.py"]


def _env():
    env = dict(os.environ)
    env["WEBGS_CHECKED"] = "1"
    return env


# Timing comparisons are left to the product build: the checked build's bounds checks change the
# kernels' speed, and a test that the autotuner's pick is no slower than the defaults measures nothing
# about stores or pads.
TIMING_TESTS = "not autotune_pick_is_not_slower_than_the_defaults"


def test_parity_suites_pass_under_the_checked_build():
    cmd = [sys.executable, "-m", "pytest", "-m", "gpu", "-x", "-q", "-p", "no:cacheprovider", "-k", TIMING_TESTS,
           *[str(ROOT / "tests" / f) for f in SUITES]]
    proc = subprocess.run(cmd, cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=1800)
    assert proc.returncode == 0, proc.stdout[-4000:] + proc.stderr[-2000:]
    assert " passed" in proc.stdout


SCRIPT = r"""
import sys
sys.path[:0] = [{root!r}, {pkg!r}]
import numpy as np
import webgs
from webgs import workloads as W
lib = webgs.library()
assert lib.gs_checked_build() == 1, "not the checked library"
packed = W.SceneSpec(20_000, 3, 0).build()
view = W.CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 256, 192).view()
with webgs.Context() as ctx:
    sc = ctx.upload(packed, 20_000)
    clean = ctx.forward(sc, view, rgba8=True)
    assert lib.gs_debug_damage_canary(ctx.handle) == 0
    try:
        ctx.forward(sc, view, rgba8=True)
        raise SystemExit("damaged canary not reported")
    except webgs.GsError as e:
        assert e.code == webgs._abi.GS_ERR_MEMORY, e
    info = ctx.frame_info()
    assert info["status"] & webgs._abi.GS_DEV_CANARY, info
    sc.close()
with webgs.Context() as ctx:  # a new context has fresh pads: clean frames again
    sc = ctx.upload(packed, 20_000)
    again = ctx.forward(sc, view, rgba8=True)
    assert np.array_equal(again["rgba8"], clean["rgba8"])
    sc.close()
print("canary check ok")
"""


def test_damaged_canary_is_reported():
    script = SCRIPT.format(root=str(ROOT), pkg=str(ROOT / "web-gs-renderer_gb300"))
    subprocess.run([sys.executable, "-c", "import sys; sys.path.insert(0, %r); from build import build_all; "
                    "build_all(checked=True)" % str(ROOT / "web-gs-renderer_gb300")], check=True, timeout=900)
    proc = subprocess.run([sys.executable, "-c", script], cwd=ROOT, env=_env(), capture_output=True, text=True,
                          timeout=600)
    assert proc.returncode == 0 and "canary check ok" in proc.stdout, proc.stdout[-2000:] + proc.stderr[-2000:]
