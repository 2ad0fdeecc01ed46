"""PLY scenes on the host (no GPU): the reference's PLY cases
(tests/localPly.test.ts, tests/assetFieldSemantics.test.ts) restated against
ply.py, plus the header errors, the percentile bounds and the sidecar
corrections' arithmetic."""
import json
import math
import struct

import numpy as np
import pytest

SH_C0_TEST = 0.28209479  # the constant the reference's test writes


@pytest.fixture(scope="module")
def P(pkg):
    import importlib

    return importlib.import_module(pkg.__name__ + ".ply")


def f32(values):
    with np.errstate(over="ignore"):
        return np.asarray(values, np.float64).astype(np.float32)


def ply_fixture(rows, float_type="float"):
    """binaryPlyFixture of the reference's tests: float properties in row order."""
    has_sh = any("sh_rest" in r for r in rows)
    has_n = any("normal" in r for r in rows)
    has_r = any("roughness" in r for r in rows)
    has_m = any("metallic" in r for r in rows)
    props = ["x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity", "scale_0", "scale_1", "scale_2",
             "rot_0", "rot_1", "rot_2", "rot_3"]
    props += [f"f_rest_{i}" for i in range(9)] if has_sh else []
    props += ["nx", "ny", "nz"] if has_n else []
    props += ["roughness"] if has_r else []
    props += ["metallic"] if has_m else []
    header = "\n".join(["ply", "format binary_little_endian 1.0", f"element vertex {len(rows)}",
                        *[f"property {float_type} {p}" for p in props], "end_header", ""]).encode()
    fmt = "<" + ("f" if float_type == "float" else "d") * len(props)
    body = b""
    for r in rows:
        vals = [*r["position"], *r["dc"], r["opacity"], *r["scales"], *r["rotation"]]
        vals += list(r["sh_rest"]) if has_sh else []
        vals += list(r.get("normal", [0, 0, 0])) if has_n else []
        vals += [r.get("roughness", 0.5)] if has_r else []
        vals += [r.get("metallic", 0.0)] if has_m else []
        body += struct.pack(fmt, *vals)
    return header + body


def row(position, dc=(0, 0, 0), opacity=0, scales=(0, 0, 0), rotation=(1, 0, 0, 0), **kw):
    return dict(position=position, dc=dc, opacity=opacity, scales=scales, rotation=rotation, **kw)


# --- tests/localPly.test.ts ----------------------------------------------------

def test_decodes_binary_3dgs_ply(P):
    data = ply_fixture([
        row([1, 2, 3], [0, 1, -1], 0, [0, math.log(2), math.log(0.5)], [1, 0, 0, 0],
            sh_rest=[0.25, 0.5, 0.75, 1, 1.25, 1.5, -0.25, -0.5, -0.75]),
        row([-1, 0, 2], [2, -2, 0.5], -2, [math.log(0.25), math.log(0.75), math.log(1.5)], [0.5] * 4,
            sh_rest=[2, 2.25, 2.5, 3, 3.25, 3.5, 4, 4.25, 4.5]),
    ])
    d = P.decode_local_ply("dropped.ply", data)
    a = d.attributes
    assert d.count == 2 and d.source_kind == "scaniverse_ply"
    assert a.positions.reshape(-1).tolist() == [1, 2, 3, -1, 0, 2]
    np.testing.assert_array_equal(a.colors.reshape(-1), f32([0.5, 0.5 + SH_C0_TEST, 0.5 - SH_C0_TEST, 1, 0,
                                                             0.5 + SH_C0_TEST * 0.5]))
    np.testing.assert_array_equal(a.opacities, f32([0.5, 1 / (1 + math.exp(2))]))
    np.testing.assert_array_equal(d.radii, f32([2, 1.5]))
    np.testing.assert_array_equal(a.scales.reshape(-1), f32([0, math.log(2), math.log(0.5), math.log(0.25),
                                                             math.log(0.75), math.log(1.5)]))
    np.testing.assert_array_equal(a.rotations.reshape(-1), f32([1, 0, 0, 0, 0.5, 0.5, 0.5, 0.5]))
    assert d.original_ids.tolist() == [0, 1]
    assert a.sh_degree == 1 and a.sh.shape == (2, 9)
    np.testing.assert_array_equal(a.sh.reshape(-1), f32([0.25, 1, -0.25, 0.5, 1.25, -0.5, 0.75, 1.5, -0.75,
                                                         2, 3, 4, 2.25, 3.25, 4.25, 2.5, 3.5, 4.5]))
    assert d.bounds.min == (-1, 0, 2) and d.bounds.max == (1, 2, 3) and d.bounds.center == (0, 1, 2.5)


def test_rejects_non_ply(P):
    with pytest.raises(ValueError, match="PLY header"):
        P.decode_local_ply("bad.txt", b"not ply")


def test_rejects_point_cloud_ply(P):
    data = "\n".join(["ply", "format ascii 1.0", "comment generated_by world-tracing scripts/kaminos_wt_object.py",
                      "element vertex 2", "property float x", "property float y", "property float z",
                      "property uchar red", "property uchar green", "property uchar blue", "property uchar layer",
                      "end_header", "0.01600226 -0.59024471 0.13915212 102 103 104 0",
                      "0.00055143 -0.58335477 0.12435700 75 77 79 1", ""]).encode()
    name = "ablate02-01-denser-interior_flood-alpha_wt_layers.ply"
    with pytest.raises(ValueError, match=(
            r"Unsupported PLY schema for hybrid splat renderer: parser=ply-point-cloud-v0; format=ascii 1\.0; "
            r"vertexCount=2; colorSource=rgb; properties=x,y,z,red,green,blue,layer; "
            r"file=ablate02-01-denser-interior_flood-alpha_wt_layers\.ply")):
        P.decode_local_ply(name, data)


def test_normals_roughness_metallic(P):
    d = P.decode_local_ply("baked.ply", ply_fixture([
        row([1, 2, 3], normal=[0, 1, 0], roughness=0.3, metallic=0.9),
        row([4, 5, 6], [1, 1, 1], normal=[0.577, 0.577, 0.577], roughness=0.8, metallic=0.0)]))
    a = d.attributes
    assert d.count == 2
    np.testing.assert_allclose(a.normals.reshape(-1), [0, 1, 0, 0.577, 0.577, 0.577], atol=1e-3)
    np.testing.assert_allclose(a.roughness, [0.3, 0.8], atol=1e-3)
    np.testing.assert_allclose(a.metalness, [0.9, 0.0], atol=1e-3)


def test_plain_ply_has_no_optional_fields(P):
    a = P.decode_local_ply("basic.ply", ply_fixture([row([1, 2, 3])])).attributes
    assert a.normals is None and a.roughness is None and a.metalness is None
    assert a.emissive is None and a.detail_normals is None and a.sh is None


def _sidecar(**correction):
    return {"schema": "kaminos.splat-correction.v0", "correction": correction}


def test_sidecar_centroid_offset(P):
    d = P.decode_local_ply("test.ply", ply_fixture([row([10, 20, 30]), row([12, 22, 32])]))
    r = P.apply_sidecar_corrections(d, _sidecar(centroidOffset=[10, 20, 30]))
    assert r.count == 2
    np.testing.assert_allclose(r.attributes.positions.reshape(-1), [0, 0, 0, 2, 2, 2], atol=1e-3)


def test_sidecar_axis_flips(P):
    d = P.decode_local_ply("test.ply", ply_fixture([row([1, 2, 3], normal=[0, 0.6, 0.8])]))
    r = P.apply_sidecar_corrections(d, _sidecar(axisFlips=[1, 1, -1]))
    np.testing.assert_allclose(r.attributes.positions[0], [1, 2, -3], atol=1e-3)
    assert abs(r.attributes.normals[0, 2] - (-0.8)) < 1e-3


def test_sidecar_crop_in_preview_space(P):
    d = P.decode_local_ply("test.ply", ply_fixture([row([0, 0, 0], [1, 0, 0]), row([5, 5, 5], [0, 1, 0]),
                                                    row([0.5, 0.5, 0.5], [0, 0, 1])]))
    r = P.apply_sidecar_corrections(d, _sidecar(crop={"enabled": True, "min": [-1.1] * 3, "max": [0.0] * 3}))
    assert r.count == 2


def test_sidecar_crop_then_offset(P):
    d = P.decode_local_ply("test.ply", ply_fixture([row([10, 10, 10]), row([10.5, 10.5, 10.5]), row([15, 15, 15])]))
    r = P.apply_sidecar_corrections(d, _sidecar(centroidOffset=[10, 10, 10],
                                                crop={"enabled": True, "min": [-1.1] * 3, "max": [0.0] * 3}))
    assert r.count == 2
    assert abs(r.attributes.positions[0, 0]) < 1e-3 and abs(r.attributes.positions[1, 0] - 0.5) < 1e-3


def test_sidecar_crop_that_empties_is_skipped(P):
    d = P.decode_local_ply("test.ply", ply_fixture([row([0, 0, 0]), row([1, 1, 1])]))
    r = P.apply_sidecar_corrections(d, _sidecar(crop={"enabled": True, "min": [5] * 3, "max": [10] * 3}))
    assert r.count == 2


def test_sidecar_crop_keeps_sh(P):
    d = P.decode_local_ply("test.ply", ply_fixture([
        row([0, 0, 0], sh_rest=[1, 2, 3, 4, 5, 6, 7, 8, 9]),
        row([5, 5, 5], sh_rest=[10, 20, 30, 40, 50, 60, 70, 80, 90])]))
    r = P.apply_sidecar_corrections(d, _sidecar(crop={"enabled": True, "min": [-1.1] * 3, "max": [0.0] * 3}))
    assert r.count == 1
    np.testing.assert_array_equal(r.attributes.sh.reshape(-1), f32([1, 4, 7, 2, 5, 8, 3, 6, 9]))
    assert r.original_ids.tolist() == [0]


# --- tests/assetFieldSemantics.test.ts ------------------------------------------

def test_ply_and_manifest_decode_alike(P, pkg):
    rows = [row([0, 1, 2], [2, -2, 0.5], 0, [math.log(3), math.log(0.5), 0], [1, 0, 0, 0]),
            row([-1, -2, -3], [-1, 0.25, 4], 4, [math.log(0.125), math.log(0.25), math.log(0.75)],
                [0.25, 0.5, -0.5, 0.75])]
    ply = P.decode_local_ply("field-semantics.ply", ply_fixture(rows))
    pa = ply.attributes
    payload = np.concatenate([pa.positions, pa.colors, pa.opacities[:, None], ply.radii[:, None]], 1)
    manifest = {
        "splat_count": 2, "endianness": "little", "stride_bytes": 32,
        "fields": [{"name": "position", "component_type": "float32", "components": 3, "byte_offset": 0},
                   {"name": "color", "component_type": "float32", "components": 3, "byte_offset": 12},
                   {"name": "opacity", "component_type": "float32", "components": 1, "byte_offset": 24},
                   {"name": "radius", "component_type": "float32", "components": 1, "byte_offset": 28}],
        "payload": {"path": "field.f32.bin", "byte_length": 64},
        "bounds": {"min": [-1, -2, -3], "max": [0, 1, 2], "center": [-0.5, -0.5, -0.5], "radius": 3}}
    m = pkg.assets.decode_first_smoke_manifest(manifest, payload.astype("<f4").tobytes(), struct.pack("<2I", 0, 1),
                                               pa.scales.tobytes(), pa.rotations.tobytes())
    ma = m.attributes
    for x, y in ((ma.colors, pa.colors), (ma.opacities, pa.opacities), (m.radii, ply.radii),
                 (ma.scales, pa.scales), (ma.rotations, pa.rotations)):
        np.testing.assert_array_equal(x, y)
    # the field contract: sh_dc_rgb colour, logit opacity, log scales, wxyz rotation
    np.testing.assert_array_equal(pa.colors[1], f32(np.clip(0.5 + 0.28209479177387814 * np.array([-1, 0.25, 4]), 0, 1)))
    np.testing.assert_array_equal(pa.opacities[1], f32(1 / (1 + math.exp(-4))))
    np.testing.assert_array_equal(pa.rotations[1], f32([0.25, 0.5, -0.5, 0.75]))


# --- header, types, bounds and sidecar arithmetic -------------------------------

@pytest.mark.parametrize("header,message", [
    ("plyx\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\nend_header\n",
     "does not start with a PLY header"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 0\nproperty float x\nend_header\n",
     "vertex count must be a positive integer"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1.5\nproperty float x\nend_header\n",
     "vertex count must be a positive integer"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nend_header\n", "no scalar properties"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty list uchar int x\nend_header\n",
     "list properties are not supported"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty half x\nend_header\n",
     "Unsupported PLY scalar property type: half"),
    ("ply\nformat binary_big_endian 1.0\nelement vertex 1\nproperty float x\nend_header\n",
     "Only binary_little_endian"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\nend_header\n",
     "PLY vertex property y is required"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 2\nproperty float x\nproperty float y\n"
     "property float z\nend_header\n", "ended before all 2 vertex rows"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\nproperty float y\n"
     "property float z\nproperty float f_rest_0\nproperty float f_rest_1\nend_header\n",
     "must be divisible by 3 RGB channels, got 2"),
    ("ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\nproperty float y\n"
     "property float z\n" + "".join(f"property float f_rest_{i}\n" for i in range(6)) + "end_header\n",
     "f_rest_\\* field count 6 does not describe a complete SH degree"),
])
def test_header_errors(P, header, message):
    with pytest.raises(ValueError, match=message):
        P.decode_local_ply("h.ply", header.encode() + b"\0" * 4)


def test_scalar_types_byte_colour_and_crlf(P):
    header = ("ply\r\nformat binary_little_endian\r\ncomment mixed types\r\nelement vertex 2\r\n"
              "property double x\r\nproperty int16 y\r\nproperty uint z\r\nproperty uchar red\r\n"
              "property uint8 green\r\nproperty char blue\r\nproperty ushort pad\r\nproperty float32 opacity\r\n"
              "element face 0\r\nproperty list uchar int vertex_indices\r\nend_header\r\n").encode()
    body = struct.pack("<dhIBBbHf", 0.1, -3, 7, 255, 128, -5, 9, 0) + struct.pack("<dhIBBbHf", 1e40, 2, 0, 0, 1, 100, 0, -2)
    d = P.decode_local_ply("types.ply", header + body)
    a = d.attributes
    np.testing.assert_array_equal(a.positions, f32([[0.1, -3, 7], [1e40, 2, 0]]))  # 1e40 -> inf in f32
    np.testing.assert_array_equal(a.colors, f32([[1, 128 / 255, 0], [0, 1 / 255, 100 / 255]]))
    np.testing.assert_array_equal(a.opacities, f32([0.5, 1 / (1 + math.exp(2))]))
    np.testing.assert_array_equal(d.radii, [1, 1])  # no scales: log-scale 0
    np.testing.assert_array_equal(a.rotations, f32([[1, 0, 0, 0]] * 2))
    assert d.bounds.max[0] == 1e40  # the count <= 100 extents use the raw doubles


def test_percentile_bounds_over_many_rows(P):
    rng = np.random.Generator(np.random.PCG64(5))
    pos = rng.normal(0, 1, (1000, 3)).astype(np.float32)
    pos[0] = [1e6, -1e6, 1e6]  # an outlier the P5-P95 bounds ignore
    rows = [row(list(map(float, p))) for p in pos]
    d = P.decode_local_ply("many.ply", ply_fixture(rows))
    s = np.sort(pos, axis=0)
    assert d.bounds.min == tuple(s[50].astype(np.float64)) and d.bounds.max == tuple(s[950].astype(np.float64))
    half = (s[950].astype(np.float64) - s[50]) * 0.5
    assert d.bounds.radius == pytest.approx(float(np.sqrt((half ** 2).sum())), rel=1e-15)
    # above 50,000 rows an evenly strided sample of 50,000 is sorted
    big = rng.normal(0, 1, (50_003, 3)).astype(np.float32)
    b = P.percentile_bounds(big)
    idx = np.floor(np.arange(50_000) * (50_003 / 50_000)).astype(np.int64)
    ss = np.sort(big[idx], axis=0)
    assert b.min == tuple(ss[2500].astype(np.float64)) and b.max == tuple(ss[47500].astype(np.float64))


def test_hypot_matches_v8_algorithm(P):
    # V8: scale by the largest magnitude, compensated sum of squares; exact cases and specials
    assert P.hypot_js(np.array([3.0]), np.array([4.0]))[0] == 5.0
    assert P.hypot_js(np.array([0.0]), np.array([-0.0]))[0] == 0.0
    assert math.isinf(P.hypot_js(np.array([math.inf]), np.array([math.nan]))[0])
    assert math.isnan(P.hypot_js(np.array([1.0]), np.array([math.nan]))[0])
    assert P.hypot_js(np.array([1e300]), np.array([1e300]))[0] == pytest.approx(math.sqrt(2) * 1e300, rel=1e-15)
    rng = np.random.Generator(np.random.PCG64(1))
    v = rng.normal(0, 1, (4, 1000))
    np.testing.assert_allclose(P.hypot_js(*v), np.sqrt((v ** 2).sum(0)), rtol=4e-16)


def test_orientation_and_flip_rotations(P):
    d = P.decode_local_ply("o.ply", ply_fixture([row([1, 0, 0], rotation=[1, 0, 0, 0], normal=[1, 0, 0]),
                                                 row([0, 1, 0], rotation=[0.5, 0.5, 0.5, 0.5], normal=[0, 1, 0])]))
    r = P.apply_sidecar_corrections(d, _sidecar(orientation={"rotation": [0, 0, math.pi / 2]}))
    # a quarter turn about z: x -> y, y -> -x
    np.testing.assert_allclose(r.attributes.positions, [[0, 1, 0], [-1, 0, 0]], atol=1e-6)
    np.testing.assert_allclose(r.attributes.normals, [[0, 1, 0], [-1, 0, 0]], atol=1e-6)
    q = (math.cos(math.pi / 4), 0.0, 0.0, math.sin(math.pi / 4))
    np.testing.assert_allclose(r.attributes.rotations[0], q, atol=1e-7)
    np.testing.assert_allclose(np.linalg.norm(r.attributes.rotations, axis=1), 1, atol=1e-7)
    # the identity orientation leaves every array untouched
    same = P.apply_sidecar_corrections(d, _sidecar(orientation={"rotation": [0, 0, 0]}))
    np.testing.assert_array_equal(same.attributes.rotations, d.attributes.rotations)
    # flipping x negates the y and z quaternion components, then renormalises
    f = P.apply_sidecar_corrections(d, _sidecar(axisFlips=[-1, 1, 1]))
    np.testing.assert_array_equal(f.attributes.rotations[1], f32([0.5, 0.5, -0.5, -0.5]))
    np.testing.assert_array_equal(f.attributes.positions[0], f32([-1, 0, 0]))


def test_load_local_ply_reads_sidecar(P, tmp_path):
    p = tmp_path / "scan.ply"
    p.write_bytes(ply_fixture([row([10, 20, 30]), row([12, 22, 32])]))
    assert P.load_local_ply(p).attributes.positions[0].tolist() == [10, 20, 30]
    (tmp_path / "scan.ply.kaminos-splat.json").write_text(json.dumps(_sidecar(centroidOffset=[10, 20, 30])))
    assert P.load_local_ply(p).attributes.positions[0].tolist() == [0, 0, 0]
    assert P.load_local_ply(p, use_sidecar=False).attributes.positions[0].tolist() == [10, 20, 30]
    (tmp_path / "scan.ply.kaminos-splat.json").write_text('{"schema": "x"}')  # no correction: ignored
    assert P.load_local_ply(p).attributes.positions[0].tolist() == [10, 20, 30]
