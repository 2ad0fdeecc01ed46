"""Scene asset decoding on the host (no GPU): the reference's own decoder
cases (tests/splats.test.ts, tests/assetFieldSemantics.test.ts) restated
against assets.py, the decoder's validation errors, and the committed subset
of the real first-smoke capture (tests/golden/first_smoke_subset, made by
make_first_smoke_subset.py)."""
import copy
import hashlib
import json
import math
import struct
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SUBSET = ROOT / "tests" / "golden" / "first_smoke_subset" / "first-smoke-subset.json"

LAYOUT = {"strideBytes": 32, "fields": [
    {"name": "position", "type": "float32", "components": 3, "byteOffset": 0},
    {"name": "color", "type": "float32", "components": 3, "byteOffset": 12},
    {"name": "opacity", "type": "float32", "components": 1, "byteOffset": 24},
    {"name": "radius", "type": "float32", "components": 1, "byteOffset": 28}]}
BOUNDS = {"min": [-1, 0, -2], "max": [3, 4, 2], "center": [1, 2, 0], "radius": 3}


@pytest.fixture(scope="module")
def A(pkg):
    return pkg.assets


def f32(values):
    return np.asarray(values, np.float64).astype(np.float32)


def valid_payload():
    return {"version": 1, "count": 2, "bounds": copy.deepcopy(BOUNDS), "layout": copy.deepcopy(LAYOUT),
            "splats": [{"position": [1, 2, 3], "color": [0.25, 0.5, 0.75], "opacity": 0.6, "radius": 0.05},
                       {"position": [-1, 0, 2], "color": [1, 0, 0.25], "opacity": 0.2, "radius": 0.1}]}


def binary_manifest():
    return {
        "schema": "scaniverse_first_smoke_splat_v1", "splat_count": 2, "endianness": "little", "stride_bytes": 32,
        "fields": [{"name": "position", "component_type": "float32", "components": 3, "byte_offset": 0},
                   {"name": "color", "component_type": "float32", "components": 3, "byte_offset": 12},
                   {"name": "opacity", "component_type": "float32", "components": 1, "byte_offset": 24},
                   {"name": "radius", "component_type": "float32", "components": 1, "byte_offset": 28}],
        "payload": {"path": "scan.f32.bin", "component_type": "float32", "byte_length": 64},
        "identity": {"scheme": "row_index_is_original_zero_based_file_order", "ids_component_type": "uint32",
                     "ids_path": "scan.ids.u32.bin"},
        "ids": {"path": "scan.ids.u32.bin", "byte_length": 8, "first_id": 0, "last_id": 1},
        "shape": {"scales_path": "scan.scales.f32.bin", "scales_component_type": "float32", "scales_byte_length": 24,
                  "rotations_path": "scan.rotations.f32.bin", "rotations_component_type": "float32",
                  "rotations_byte_length": 32, "rotation_order": "wxyz", "scale_space": "log"},
        "sh": {"degree": 1, "basis": "3dgs_real_sh", "coefficients_layout": "splat_coeff_rgb",
               "coefficients_path": "scan.sh.f32.bin", "coefficients_component_type": "float32",
               "coefficient_count": 3, "coefficients_byte_length": 72},
        "bounds": copy.deepcopy(BOUNDS),
    }


SCALES = [0, math.log(2), math.log(0.5), math.log(3), math.log(0.25), math.log(1)]
ROTATIONS = [1, 0, 0, 0, 0.5, 0.5, 0.5, 0.5]
SH = [0.25, 0.5, 0.75, 1, 1.25, 1.5, -0.25, -0.5, -0.75, 2, 2.25, 2.5, 3, 3.25, 3.5, 4, 4.25, 4.5]


def binary_sidecars():
    payload = struct.pack("<16f", 1, 2, 3, 0.25, 0.5, 0.75, 0.6, 0.05, -1, 0, 2, 1, 0, 0.25, 0.2, 0.1)
    return dict(payload=payload, ids=struct.pack("<2I", 1, 0), scales=struct.pack("<6f", *SCALES),
                rotations=struct.pack("<8f", *ROTATIONS), sh=struct.pack("<18f", *SH))


# --- the reference's cases (tests/splats.test.ts) ---------------------------

def test_decodes_rows(A):
    d = A.decode_first_smoke_payload(valid_payload())
    a = d.attributes
    assert d.count == 2 and d.source_kind == "real_scaniverse_ply"
    assert a.positions.reshape(-1).tolist() == [1, 2, 3, -1, 0, 2]
    assert a.colors.reshape(-1).tolist() == [0.25, 0.5, 0.75, 1, 0, 0.25]
    np.testing.assert_array_equal(a.opacities, f32([0.6, 0.2]))
    np.testing.assert_array_equal(d.radii, f32([0.05, 0.1]))
    assert d.original_ids.tolist() == [0, 1]
    assert d.bounds.center == (1, 2, 0)
    # rows carry no shape: log(radius) on every axis, identity rotations
    np.testing.assert_array_equal(a.scales, np.repeat(f32([math.log(np.float32(0.05)),
                                                           math.log(np.float32(0.1))])[:, None], 3, 1))
    np.testing.assert_array_equal(a.rotations, f32([[1, 0, 0, 0], [1, 0, 0, 0]]))


def test_nested_metadata_planar_arrays(A):
    row = valid_payload()
    d = A.decode_first_smoke_payload({
        "version": 1,
        "metadata": {"count": row["count"], "bounds": row["bounds"], "strideBytes": 32, "fields": LAYOUT["fields"]},
        "attributes": {"positions": [1, 2, 3, -1, 0, 2], "colors": [0.25, 0.5, 0.75, 1, 0, 0.25],
                       "opacities": [0.6, 0.2], "radii": [0.05, 0.1]},
        "originalIds": [1, 0]})
    assert d.count == 2 and d.source_kind == "real_scaniverse_ply"
    assert d.attributes.positions.reshape(-1).tolist() == [1, 2, 3, -1, 0, 2]
    assert d.original_ids.tolist() == [1, 0]


def test_binary_manifest_sidecars(A):
    s = binary_sidecars()
    d = A.decode_first_smoke_manifest(binary_manifest(), s["payload"], s["ids"], s["scales"], s["rotations"], s["sh"])
    a = d.attributes
    assert d.count == 2
    assert a.positions.reshape(-1).tolist() == [1, 2, 3, -1, 0, 2]
    assert a.colors.reshape(-1).tolist() == [0.25, 0.5, 0.75, 1, 0, 0.25]
    np.testing.assert_array_equal(a.opacities, f32([0.6, 0.2]))
    np.testing.assert_array_equal(d.radii, f32([0.05, 0.1]))
    assert d.original_ids.tolist() == [1, 0]
    np.testing.assert_array_equal(a.scales.reshape(-1), f32(SCALES))
    np.testing.assert_array_equal(a.rotations.reshape(-1), f32(ROTATIONS))
    assert a.sh_degree == 1 and a.sh.shape == (2, 9)
    np.testing.assert_array_equal(a.sh.reshape(-1), f32(SH))


def test_spz_manifest_source_kind(A):
    s = binary_sidecars()
    m = binary_manifest()
    m["source"] = {"kind": "spz", "filename": "workshop_four_cups.spz"}
    d = A.decode_first_smoke_manifest(m, s["payload"], s["ids"], s["scales"], s["rotations"], s["sh"])
    assert d.source_kind == "real_splat_spz"


def test_validates_count_bounds_and_row_fields(A):
    missing = valid_payload()
    del missing["splats"][0]["radius"]
    with pytest.raises(ValueError, match=r"splats\[0\]\.radius"):
        A.decode_first_smoke_payload(missing)
    mismatch = valid_payload()
    mismatch["count"] = 3
    with pytest.raises(ValueError, match=r"count .*2 rows"):
        A.decode_first_smoke_payload(mismatch)
    bad_bounds = valid_payload()
    bad_bounds["bounds"]["radius"] = 0
    with pytest.raises(ValueError, match=r"bounds\.radius"):
        A.decode_first_smoke_payload(bad_bounds)
    dup = valid_payload()
    dup["originalIds"] = [0, 0]
    with pytest.raises(ValueError, match="duplicates original ID"):
        A.decode_first_smoke_payload(dup)
    with pytest.raises(ValueError, match="payload sidecar byte length"):
        A.decode_first_smoke_manifest(binary_manifest(), binary_sidecars()["payload"][4:])


def test_sidecars_resolved_beside_manifest(A, tmp_path):
    s = binary_sidecars()
    m = binary_manifest()
    (tmp_path / "scan.json").write_text(json.dumps(m))
    for key, name in (("payload", "scan.f32.bin"), ("ids", "scan.ids.u32.bin"), ("scales", "scan.scales.f32.bin"),
                      ("rotations", "scan.rotations.f32.bin"), ("sh", "scan.sh.f32.bin")):
        (tmp_path / name).write_bytes(s[key])
    d = A.load_first_smoke(tmp_path / "scan.json")
    assert d.original_ids.tolist() == [1, 0]
    np.testing.assert_array_equal(d.attributes.scales.reshape(-1), f32(SCALES))
    np.testing.assert_array_equal(d.attributes.rotations.reshape(-1), f32(ROTATIONS))
    assert d.attributes.sh_degree == 1
    np.testing.assert_array_equal(d.attributes.sh.reshape(-1), np.frombuffer(s["sh"], "<f4"))
    # an inline payload through the same entry point
    (tmp_path / "inline.json").write_text(json.dumps(valid_payload()))
    assert A.load_first_smoke(tmp_path / "inline.json").count == 2


def test_framing_from_payload_bounds(A):
    d = A.decode_first_smoke_payload(valid_payload())
    f = A.framing_from_bounds(d.bounds, fov_y=math.pi / 2)
    assert f.target == (1, 2, 0)
    assert f.distance > d.bounds.radius and f.near > 0 and f.far > f.distance
    # the formula itself: radius = max(bounds.radius, half diagonal), distance = padded / sin(fov/2)
    r = max(3.0, math.hypot(4, 4, 4) / 2)
    assert f.radius == r
    assert f.distance == pytest.approx(r * 1.35 / math.sin(math.pi / 4), rel=1e-15)
    assert f.near == max(0.001, f.distance - 2 * r * 1.35) and f.far == f.distance + 2 * r * 1.35
    with pytest.raises(ValueError, match="fovY"):
        A.framing_from_bounds(d.bounds, fov_y=math.pi)
    with pytest.raises(ValueError, match="padding"):
        A.framing_from_bounds(d.bounds, padding=0.5)


# --- tests/assetFieldSemantics.test.ts: sidecars keep log scales and wxyz ----

def test_manifest_sidecars_preserve_log_scales_and_wxyz(A):
    scales = f32([[math.log(3), math.log(0.5), 0], [math.log(0.125), math.log(0.25), math.log(0.75)]])
    rot = f32([[1, 0, 0, 0], [0.25, 0.5, -0.5, 0.75]])
    m = binary_manifest()
    del m["sh"]
    rows = f32([[0, 1, 2, 0.9, 0.1, 0.6, 0.5, 3], [-1, -2, -3, 0.3, 0.55, 1, 0.98, 0.75]])
    d = A.decode_first_smoke_manifest(m, rows.tobytes(), struct.pack("<2I", 0, 1), scales.tobytes(), rot.tobytes())
    np.testing.assert_array_equal(d.attributes.scales, scales)
    np.testing.assert_array_equal(d.attributes.rotations, rot)
    np.testing.assert_array_equal(d.radii, rows[:, 7])
    assert d.attributes.sh is None and d.attributes.sh_degree == 0


# --- validation errors, in the reference's order ------------------------------

def _decode(A, mutate=None, **over):
    m = binary_manifest()
    if mutate:
        mutate(m)
    s = binary_sidecars()
    s.update(over)
    return A.decode_first_smoke_manifest(m, s["payload"], s.get("ids"), s.get("scales"), s.get("rotations"),
                                         s.get("sh"))


@pytest.mark.parametrize("mutate,message", [
    (lambda m: m.update(splat_count=0), "splat_count must be greater than zero"),
    (lambda m: m.update(splat_count=2.5), "splat_count must be a non-negative integer"),
    (lambda m: m.update(splat_count=True), "splat_count must be a non-negative integer"),
    (lambda m: m.update(endianness="big"), "manifest.endianness must be little"),
    (lambda m: m["bounds"].update(min=[0, 0]), r"bounds\.min must be a float3"),
    (lambda m: m["bounds"].update(center=[0, float("nan"), 0]), r"bounds\.center\[1\] must be a finite number"),
    (lambda m: m.update(source={"kind": ""}), "source.kind must be a non-empty string"),
    (lambda m: m.update(stride_bytes=28), "layout.strideBytes must be 32"),
    (lambda m: m.pop("fields"), "layout.fields must be an array"),
    (lambda m: (m.pop("fields"), m.pop("stride_bytes")), "layout must be an object"),
    (lambda m: m["fields"].pop(), "layout.fields must contain exactly the first-smoke row fields"),
    (lambda m: m["fields"][1].update(name="normal"), r"layout\.fields\[1\]\.name is not a first-smoke row field"),
    (lambda m: m["fields"][2].update(component_type="float16"), r"layout\.fields\[2\]\.type must be float32"),
    (lambda m: m["fields"][2].update(components=2), r"layout\.fields\[2\]\.components must be 1 or 3"),
    (lambda m: m["fields"][3].update(byte_offset=24), "layout.fields.radius must be float32x1 at byte 28"),
    (lambda m: m["fields"][3].update(name="opacity"), "layout.fields is missing radius"),
    (lambda m: m["payload"].update(byte_length=96), "payload.byte_length must be 64 for 2 rows"),
    (lambda m: m["sh"].update(degree=0), "sh.degree must be greater than zero"),
    (lambda m: m["sh"].update(basis="other"), "sh.basis must be 3dgs_real_sh"),
    (lambda m: m["sh"].update(coefficient_count=8), "sh.coefficient_count must be 3 for degree 1"),
    (lambda m: m["sh"].update(coefficients_byte_length=64), "sh.coefficients_byte_length must be 72"),
])
def test_manifest_validation(A, mutate, message):
    with pytest.raises(ValueError, match=message):
        _decode(A, mutate)


def test_row_and_sidecar_validation(A):
    rows = np.frombuffer(binary_sidecars()["payload"], "<f4").reshape(2, 8).copy()
    bad = rows.copy()
    bad[1, 6] = 1.5
    bad[1, 7] = -1  # same row: opacity is checked first
    with pytest.raises(ValueError, match=r"payload\.rows\[1\]\.opacity must be in \[0, 1\]"):
        _decode(A, payload=bad.tobytes())
    bad = rows.copy()
    bad[0, 7] = 0
    bad[1, 6] = float("nan")  # an earlier row wins
    with pytest.raises(ValueError, match=r"payload\.rows\[0\]\.radius must be greater than zero"):
        _decode(A, payload=bad.tobytes())
    bad = rows.copy()
    bad[1, 6] = float("inf")
    with pytest.raises(ValueError, match=r"payload\.rows\[1\]\.opacity must be a finite number"):
        _decode(A, payload=bad.tobytes())
    with pytest.raises(ValueError, match=r"shape\.scales\[4\] must be a finite number"):
        _decode(A, scales=struct.pack("<6f", 0, 0, 0, 0, float("nan"), 0))
    with pytest.raises(ValueError, match="shape.rotations byte length 28 does not match expected 32"):
        _decode(A, rotations=struct.pack("<7f", *ROTATIONS[:7]))
    with pytest.raises(ValueError, match="ID sidecar byte length 4 does not match expected 8"):
        _decode(A, ids=struct.pack("<I", 0))
    with pytest.raises(ValueError, match=r"originalIds\[0\] must be less than count 2"):
        _decode(A, ids=struct.pack("<2I", 2, 0))
    with pytest.raises(ValueError, match=r"originalIds\[1\] duplicates original ID 1"):
        _decode(A, ids=struct.pack("<2I", 1, 1))
    with pytest.raises(ValueError, match="SH sidecar bytes are required"):
        _decode(A, sh=None)
    # absent shape sidecars: log(radius) scales, identity rotations
    d = _decode(A, scales=None, rotations=None)
    np.testing.assert_array_equal(d.attributes.scales[:, 0], np.log(rows[:, 7].astype(np.float64)).astype(np.float32))
    np.testing.assert_array_equal(d.attributes.rotations, f32([[1, 0, 0, 0]] * 2))


def test_inline_id_validation_order(A):
    p = valid_payload()
    p["originalIds"] = [0, -1]
    with pytest.raises(ValueError, match=r"originalIds\[1\] must be a non-negative integer"):
        A.decode_first_smoke_payload(p)
    p["originalIds"] = [0, 1, 2]
    with pytest.raises(ValueError, match="originalIds must contain 2 entries"):
        A.decode_first_smoke_payload(p)
    p["originalIds"] = "01"
    with pytest.raises(ValueError, match="originalIds must be an array"):
        A.decode_first_smoke_payload(p)


# --- the committed subset of the real capture ---------------------------------

def test_subset_fixture_integrity(A):
    m = json.loads(SUBSET.read_text())
    for name, digest in m["subset"]["sha256"].items():
        assert hashlib.sha256((SUBSET.parent / name).read_bytes()).hexdigest() == digest, name
    d = A.load_first_smoke(SUBSET)
    a = d.attributes
    assert d.count == 4096 and d.source_kind == "scaniverse_ply"
    assert d.original_ids.tolist() == list(range(4096))
    src_rows = np.frombuffer((SUBSET.parent / m["subset"]["source_rows_path"]).read_bytes(), "<u4")
    assert np.all(np.diff(src_rows.astype(np.int64)) > 0) and src_rows[-1] < m["subset"]["source_splat_count"]
    # the capture's semantics: log scales, unit wxyz quaternions, unit opacities and colours
    assert np.all(a.scales < 0) and np.all(np.isfinite(a.scales))
    np.testing.assert_allclose(np.linalg.norm(a.rotations, axis=1), 1.0, atol=1e-2)
    assert a.opacities.min() >= 0 and a.opacities.max() <= 1
    assert a.colors.min() >= 0 and a.colors.max() <= 1
    assert a.roughness.shape == (4096,) and a.metalness.shape == (4096,)
    # the radius column is max(exp(scale)) of the capture's PLY decode
    np.testing.assert_allclose(d.radii, np.exp(a.scales.astype(np.float64)).max(1), rtol=1e-5)
    # bounds: the positions' box, its midpoint, half its diagonal
    lo, hi = a.positions.min(0), a.positions.max(0)
    assert d.bounds.min == tuple(lo.astype(np.float64)) and d.bounds.max == tuple(hi.astype(np.float64))
    assert d.bounds.radius == pytest.approx(np.linalg.norm(hi.astype(np.float64) - lo) / 2, rel=1e-12)


def test_subset_framing_camera(A):
    d = A.load_first_smoke(SUBSET)
    cam = A.camera_for_splat_bounds(d.bounds)
    f = A.framing_from_bounds(d.bounds, padding=1.45)
    assert cam.distance == f.distance and cam.near == f.near and cam.far == f.far
    assert (cam.azimuth, cam.elevation) == (0.0, 0.18)
    fr = cam.frame(640, 480)
    pos = d.attributes.positions.astype(np.float64)
    clip = np.c_[pos, np.ones(len(pos))] @ fr["view_proj"].astype(np.float64).reshape(4, 4)
    ndc = clip[:, :3] / clip[:, 3:4]
    # the padded bounding sphere is in view: every splat centre projects inside the frustum
    assert np.all(clip[:, 3] > 0)
    assert np.all(np.abs(ndc[:, :2]) < 1) and np.all((ndc[:, 2] > 0) & (ndc[:, 2] < 1))
