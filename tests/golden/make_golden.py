"""Writes tests/golden/oracle_fixtures.json: digests of the CPU oracle's frames on small seeded cases.

These are regression pins of the restatement (the reference ships no golden vectors for this path):
the scenes come from the deterministic generator, the 176-byte view blocks are stored verbatim, and
for every case the file keeps the instance count and SHA-256 digests of the sorted keys, values, tile
ranges, fp32 RGB and rgba8 image. Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "web-gs-renderer_gb300")]

import oracle  # noqa: E402
import webgs  # noqa: E402

CASES = [
    # name, (kind, count, seed, clusters, box), eye, fov, width, height, tile, factor
    ("unit_cluster_128x96", (0, 3000, 101, 0, 0.0), (0.0, 0.3, -3.5), 60.0, 128, 96, 16, 64),
    ("mixture_inside_box_200x120", (1, 20000, 102, 16, 20.0), (0.0, 1.0, -9.0), 70.0, 200, 120, 16, 64),
    ("odd_size_33x250", (0, 2000, 103, 0, 0.0), (0.5, 0.0, -4.0), 60.0, 33, 250, 16, 64),
    ("tile8_160x90", (0, 4000, 104, 0, 0.0), (0.0, 0.0, -4.0), 60.0, 160, 90, 8, 64),
    ("tile32_256x256", (0, 4000, 105, 0, 0.0), (0.0, 0.0, -4.0), 60.0, 256, 256, 32, 64),
    ("overflow_factor1_96x96", (0, 1500, 106, 0, 0.0), (0.0, 0.0, -2.5), 60.0, 96, 96, 16, 1),
]


def digest(a) -> str:
    return hashlib.sha256(memoryview(a).cast("B")).hexdigest()


def case_frame(case):
    name, (kind, count, seed, clusters, box), eye, fov, w, h, tile, factor = case
    packed = webgs.synth_scene(kind, count, seed, clusters, box)
    view = webgs.camera_view(eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), fov, w, h, 0.2, 100.0)
    return packed, webgs.view_bytes(view)


def summarize(r) -> dict:
    return {"instance_count": int(r["instance_count"]), "sorted_count": int(r["sorted_count"]),
            "keys": digest(r["keys"]), "vals": digest(r["vals"]), "ranges": digest(r["ranges"]),
            "rgb": digest(r["rgb"]), "rgba8": digest(r["rgba8"])}


def main():
    out = []
    for case in CASES:
        name, scene, eye, fov, w, h, tile, factor = case
        packed, vb = case_frame(case)
        r = oracle.forward_f32(vb, packed, scene[1], tile=tile, factor=factor)
        out.append({"name": name, "scene": list(scene), "eye": list(eye), "fov": fov, "width": w, "height": h,
                    "tile": tile, "factor": factor, "view_hex": vb.hex(), "scene_digest": digest(packed),
                    **summarize(r)})
    path = Path(__file__).with_name("oracle_fixtures.json")
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(out)} cases to {path}")


if __name__ == "__main__":
    main()
