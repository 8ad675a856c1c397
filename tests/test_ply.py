"""PLY ingest (gs_ply_parse / webgs.load_ply) against files written here with numpy, following the
rules of the reference loader (src/loader/loader.js:56-213)."""
import numpy as np
import pytest

import webgs

REQUIRED = (["x", "y", "z", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3", "f_dc_0", "f_dc_1",
             "f_dc_2", "opacity"] + [f"f_rest_{i}" for i in range(45)])
NP_TYPES = {"char": "i1", "uchar": "u1", "int8": "i1", "uint8": "u1", "short": "<i2", "ushort": "<u2",
            "int16": "<i2", "uint16": "<u2", "int": "<i4", "uint": "<u4", "int32": "<i4", "uint32": "<u4",
            "float": "<f4", "float32": "<f4", "double": "<f8", "float64": "<f8"}


def write_ply(props, values, n, fmt="binary_little_endian", eol=b"\n", extra_elements=b"", trailer=b""):
    """props: [(type, name)]; values: {name: array of n}."""
    head = [b"ply", f"format {fmt} 1.0".encode(), b"comment written by the tests", f"element vertex {n}".encode()]
    head += [f"property {t} {name}".encode() for t, name in props]
    head.append(extra_elements.rstrip(b"\n")) if extra_elements else None
    head.append(b"end_header")
    dt = np.dtype([(name, NP_TYPES[t]) for t, name in props])
    rec = np.zeros(n, dt)
    for _, name in props:
        rec[name] = values[name]
    return eol.join(head) + eol + rec.tobytes() + trailer


def reference_packed(values, n):
    order = [["x", "y", "z"], ["scale_0", "scale_1", "scale_2"], ["rot_0", "rot_1", "rot_2", "rot_3"],
             ["f_dc_0", "f_dc_1", "f_dc_2"], ["opacity"], [f"f_rest_{i}" for i in range(45)]]
    return np.concatenate([np.stack([np.asarray(values[k], np.float64) for k in blk], 1).ravel()
                           for blk in order]).astype(np.float32)


def random_values(n, seed=0):
    rng = np.random.default_rng(seed)
    return {k: rng.normal(0, 1, n) for k in REQUIRED}


def test_float_properties_roundtrip():
    n = 257
    vals = random_values(n)
    data = write_ply([("float", k) for k in REQUIRED], vals, n)
    out = webgs.load_ply(data)
    assert out["count"] == n
    np.testing.assert_array_equal(out["packed"], reference_packed({k: v.astype(np.float32) for k, v in vals.items()}, n))


def test_mixed_types_shuffled_order_extra_properties_crlf():
    n = 40
    rng = np.random.default_rng(1)
    names = list(REQUIRED) + ["nx", "ny", "nz", "red"]
    rng.shuffle(names)
    types = list(NP_TYPES)
    props = [(types[i % len(types)], nm) for i, nm in enumerate(names)]
    vals = {}
    for t, nm in props:
        info = np.dtype(NP_TYPES[t])
        if info.kind == "f":
            vals[nm] = rng.normal(0, 3, n).astype(info)
        else:
            lo, hi = np.iinfo(info).min, np.iinfo(info).max
            vals[nm] = rng.integers(max(lo, -1000), min(hi, 1000) + 1, n).astype(info)
    data = write_ply(props, vals, n, eol=b"\r\n", extra_elements=b"element face 0\nproperty list uchar int vertex_indices\n")
    out = webgs.load_ply(data)
    ref = reference_packed({k: vals[k].astype(np.float64) for k in REQUIRED}, n)
    np.testing.assert_array_equal(out["packed"], ref)


def test_loaded_scene_renders_like_the_packed_array(tmp_path):
    n = 500
    packed = webgs.synth_scene(0, n, 9)
    blocks = np.split(packed, np.cumsum([3 * n, 3 * n, 4 * n, 3 * n, n]))
    widths = [3, 3, 4, 3, 1, 45]
    cols = np.concatenate([b.reshape(n, w) for b, w in zip(blocks, widths)], 1)
    vals = {k: cols[:, i] for i, k in enumerate(REQUIRED)}
    p = tmp_path / "scene.ply"
    p.write_bytes(write_ply([("float", k) for k in REQUIRED], vals, n))
    out = webgs.load_ply(str(p))
    np.testing.assert_array_equal(out["packed"], packed)


@pytest.mark.parametrize("mutate,msg", [
    (lambda d: d.replace(b"end_header", b"end_headr"), '"end_header" not found'),
    (lambda d: d.replace(b"format binary_little_endian 1.0\n", b""), 'missing "format" line'),
    (lambda d: d.replace(b"binary_little_endian", b"binary_big_endian"), "unsupported format"),
    (lambda d: d.replace(b"binary_little_endian", b"ascii"), "unsupported format"),
    (lambda d: d.replace(b"element vertex 8", b"element vertex 0"), "vertex count missing or zero"),
    (lambda d: d.replace(b"property float f_rest_44\n", b""), 'missing required property "f_rest_44"'),
    (lambda d: d.replace(b"property float opacity", b"property half opacity"), 'unknown property type "half"'),
    (lambda d: d.replace(b"property float opacity", b"property list uchar float opacity"), "list properties"),
    (lambda d: d[:-10], "truncated"),
])
def test_malformed_files_fail_with_the_reference_message(mutate, msg):
    n = 8
    data = write_ply([("float", k) for k in REQUIRED], random_values(n), n)
    with pytest.raises(webgs.GsError) as ei:
        webgs.load_ply(mutate(data))
    assert msg in str(ei.value) and ei.value.code == 1


def test_renderer_upload_accepts_load_ply_output():
    n = 64
    data = write_ply([("float", k) for k in REQUIRED], random_values(n, 3), n)
    out = webgs.load_ply(data)
    assert set(out) == {"count", "packed"} and out["packed"].dtype == np.float32 and out["packed"].size == 59 * n
