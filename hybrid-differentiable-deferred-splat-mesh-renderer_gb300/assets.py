"""Scene assets: the first-smoke splat formats and the camera that frames them.

Restates src/splats.ts of the reference:
  decode_first_smoke_manifest  decodeFirstSmokeSplatManifest (:244-344): a JSON
                               manifest, a payload of 32-byte little-endian rows
                               (position f32x3, colour f32x3, opacity f32,
                               radius f32) and optional sidecars (original ids,
                               log scales, wxyz rotations, SH coefficients,
                               roughness, metalness)
  decode_first_smoke_payload   decodeFirstSmokeSplatPayload (:211-242): the same
                               rows inline in JSON, as row objects
                               (decodeRowSplatAttributes :502-527) or planar
                               arrays (decodePlanarSplatAttributes :529-565)
  load_first_smoke             fetchFirstSmokeSplatPayload (:114-209) on files:
                               sidecar paths resolved beside the manifest
                               (sidecarIdsPath :888-902, sidecarShapePath
                               :904-913, sidecarShPath :915-921)
  framing_from_bounds          framingFromBounds (:346-374)
and src/realSmokeScene.ts configureCameraForSplatBounds (:183-194).

Validation follows the reference's helpers (requireRecord :770, requireVec3
:777, requireFiniteNumber :788, requireString :795, requirePositiveFinite
:806, requireUnitInterval :814, requirePositiveInteger :822,
requireNonNegativeInteger :830, decodeLayout :577-622, decodeFieldLayout
:642-669, decodeOriginalIds :671-701, decodeOriginalIdBytes :703-716,
decodeFloat32Bytes :718-731, decodeShSidecar :923-981, manifestSourceKind
:983-992) and raises ValueError with the same messages, for the first
offending field in the reference's order. JSON numbers are JavaScript numbers:
an integral float (32.0) is an integer, a bool is not a number.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .camera import OrbitCamera
from .splats import SplatAttributes

STRIDE_BYTES = 32
# (name, components, byte offset): REQUIRED_FIELD_LAYOUT (splats.ts:102-107)
ROW_FIELDS = (("position", 3, 0), ("color", 3, 12), ("opacity", 1, 24), ("radius", 1, 28))


@dataclass
class SplatBounds:
    min: tuple
    max: tuple
    center: tuple
    radius: float


@dataclass
class SplatScene:
    """A decoded asset: the compositor's attributes plus what the reference
    keeps beside them (per-row radii, original ids, bounds, source kind)."""

    attributes: SplatAttributes
    radii: np.ndarray
    original_ids: np.ndarray
    bounds: SplatBounds
    source_kind: str

    @property
    def count(self) -> int:
        return int(self.radii.shape[0])


def _is_number(v) -> bool:
    return isinstance(v, (int, float)) and not isinstance(v, bool)


def _first(primary, fallback):
    return fallback if primary is None else primary


def _record(value, path) -> dict:
    if not isinstance(value, dict):
        raise ValueError(f"{path} must be an object")
    return value


def _finite(value, path) -> float:
    if not _is_number(value) or not math.isfinite(value):
        raise ValueError(f"{path} must be a finite number")
    return float(value)


def _positive_finite(value, path) -> float:
    v = _finite(value, path)
    if v <= 0:
        raise ValueError(f"{path} must be greater than zero")
    return v


def _unit_interval(value, path) -> float:
    v = _finite(value, path)
    if v < 0 or v > 1:
        raise ValueError(f"{path} must be in [0, 1]")
    return v


def _non_negative_int(value, path) -> int:
    if not _is_number(value) or not math.isfinite(value) or value != int(value) or value < 0:
        raise ValueError(f"{path} must be a non-negative integer")
    return int(value)


def _positive_int(value, path) -> int:
    v = _non_negative_int(value, path)
    if v <= 0:
        raise ValueError(f"{path} must be greater than zero")
    return v


def _string(value, path) -> str:
    if not isinstance(value, str) or not value:
        raise ValueError(f"{path} must be a non-empty string")
    return value


def _vec3(value, path) -> tuple:
    if not isinstance(value, list) or len(value) != 3:
        raise ValueError(f"{path} must be a float3")
    return tuple(_finite(v, f"{path}[{i}]") for i, v in enumerate(value))


def decode_bounds(value, path: str = "bounds") -> SplatBounds:
    b = _record(value, path)
    return SplatBounds(_vec3(b.get("min"), f"{path}.min"), _vec3(b.get("max"), f"{path}.max"),
                       _vec3(b.get("center"), f"{path}.center"), _positive_finite(b.get("radius"), f"{path}.radius"))


def _layout_source(meta: dict):
    if meta.get("layout") is not None:
        return meta["layout"]
    if any(meta.get(k) is not None for k in ("strideBytes", "stride_bytes", "fields", "fieldLayout")):
        return {"strideBytes": _first(meta.get("strideBytes"), meta.get("stride_bytes")),
                "fields": _first(meta.get("fields"), meta.get("fieldLayout"))}
    return None


def decode_layout(value, path: str = "layout") -> None:
    """The row layout must be exactly position/color/opacity/radius at 0/12/24/28."""
    lay = _record(value, path)
    stride = _positive_int(lay.get("strideBytes"), f"{path}.strideBytes")
    if stride != STRIDE_BYTES:
        raise ValueError(f"{path}.strideBytes must be {STRIDE_BYTES}")
    fields = lay.get("fields")
    if not isinstance(fields, list):
        raise ValueError(f"{path}.fields must be an array")
    if len(fields) != len(ROW_FIELDS):
        raise ValueError(f"{path}.fields must contain exactly the first-smoke row fields")
    decoded = []
    for i, f in enumerate(fields):
        p = f"{path}.fields[{i}]"
        f = _record(f, p)
        name = f.get("name")
        if name not in ("position", "color", "opacity", "radius"):
            raise ValueError(f"{p}.name is not a first-smoke row field")
        if _first(f.get("type"), f.get("component_type")) != "float32":
            raise ValueError(f"{p}.type must be float32")
        comps = _positive_int(f.get("components"), f"{p}.components")
        if comps not in (1, 3):
            raise ValueError(f"{p}.components must be 1 or 3")
        off = _non_negative_int(_first(f.get("byteOffset"), f.get("byte_offset")), f"{p}.byteOffset")
        decoded.append((name, comps, off))
    for name, comps, off in ROW_FIELDS:
        got = next((d for d in decoded if d[0] == name), None)
        if got is None:
            raise ValueError(f"{path}.fields is missing {name}")
        if got[1:] != (comps, off):
            raise ValueError(f"{path}.fields.{name} must be float32x{comps} at byte {off}")


def _check_ids(ids: np.ndarray, count: int) -> np.ndarray:
    """decodeOriginalIds: every id < count and unique; the first bad index wins."""
    ids = np.asarray(ids, dtype=np.int64)
    over = np.nonzero(ids >= count)[0]
    first_over = int(over[0]) if over.size else count
    _, first_seen = np.unique(ids, return_index=True)
    repeat = np.ones(ids.shape[0], bool)
    repeat[first_seen] = False
    dups = np.nonzero(repeat)[0]
    first_dup = int(dups[0]) if dups.size else count
    if first_over < count and first_over <= first_dup:
        raise ValueError(f"originalIds[{first_over}] must be less than count {count}")
    if first_dup < count:
        raise ValueError(f"originalIds[{first_dup}] duplicates original ID {int(ids[first_dup])}")
    return ids.astype(np.uint32)


def decode_original_ids(value, count: int) -> np.ndarray:
    """An inline id array (list or integer ndarray), or None for 0..count-1."""
    if value is None:
        return np.arange(count, dtype=np.uint32)
    if not isinstance(value, (list, tuple, np.ndarray)):
        raise ValueError("originalIds must be an array or typed array")
    if len(value) != count:
        raise ValueError(f"originalIds must contain {count} entries")
    items = value.tolist() if isinstance(value, np.ndarray) else list(value)
    for i, v in enumerate(items):
        if not _is_number(v) or not math.isfinite(v) or v != int(v) or v < 0:
            _check_ids(np.array([int(x) for x in items[:i]], np.int64), count)
            raise ValueError(f"originalIds[{i}] must be a non-negative integer")
    return _check_ids(np.array([int(v) for v in items], np.int64), count)


def decode_original_id_bytes(data: bytes, count: int) -> np.ndarray:
    if len(data) != count * 4:
        raise ValueError(f"ID sidecar byte length {len(data)} does not match expected {count * 4}")
    return _check_ids(np.frombuffer(data, "<u4").astype(np.int64), count)


def decode_float32_bytes(data: bytes, n: int, path: str) -> np.ndarray:
    if len(data) != n * 4:
        raise ValueError(f"{path} byte length {len(data)} does not match expected {n * 4}")
    v = np.frombuffer(data, "<f4").astype(np.float32)
    bad = np.nonzero(~np.isfinite(v))[0]
    if bad.size:
        raise ValueError(f"{path}[{int(bad[0])}] must be a finite number")
    return v


def _decode_float32_array(value, n: int, path: str, validator=_finite) -> np.ndarray:
    if not isinstance(value, (list, tuple, np.ndarray)):
        raise ValueError(f"{path} must be an array or typed array")
    if len(value) != n:
        raise ValueError(f"{path} must contain {n} entries")
    out = np.empty(n, np.float32)
    for i, v in enumerate(value.tolist() if isinstance(value, np.ndarray) else value):
        out[i] = validator(v, f"{path}[{i}]")
    return out


def fallback_scales_from_radii(radii: np.ndarray) -> np.ndarray:
    """log(max(radius, 1e-12)) on every axis, in double, stored as f32."""
    s = np.log(np.maximum(np.asarray(radii, np.float32).astype(np.float64), 1e-12)).astype(np.float32)
    return np.repeat(s[:, None], 3, axis=1)


def identity_rotations(count: int) -> np.ndarray:
    rot = np.zeros((count, 4), np.float32)
    rot[:, 0] = 1.0
    return rot


def _source_kind(root: dict) -> str:
    source = root.get("source")
    if source is not None:
        source = _record(source, "source")
        if source.get("kind") is not None:
            kind = _string(source["kind"], "source.kind")
            return "real_splat_spz" if kind == "spz" else kind
    return "real_scaniverse_ply"


def _decode_sh(root: dict, count: int, data: bytes | None):
    if root.get("sh") is None:
        return None, 0
    sh = _record(root["sh"], "sh")
    degree = _non_negative_int(sh.get("degree"), "sh.degree")
    if degree <= 0:
        raise ValueError("sh.degree must be greater than zero when an SH sidecar is declared")
    if sh.get("basis") != "3dgs_real_sh":
        raise ValueError("sh.basis must be 3dgs_real_sh")
    if sh.get("coefficients_layout") != "splat_coeff_rgb":
        raise ValueError("sh.coefficients_layout must be splat_coeff_rgb")
    if sh.get("coefficients_component_type") != "float32":
        raise ValueError("sh.coefficients_component_type must be float32")
    k = (degree + 1) ** 2 - 1
    if _positive_int(sh.get("coefficient_count"), "sh.coefficient_count") != k:
        raise ValueError(f"sh.coefficient_count must be {k} for degree {degree}")
    expected = count * k * 3 * 4
    if _positive_int(sh.get("coefficients_byte_length"), "sh.coefficients_byte_length") != expected:
        raise ValueError(f"sh.coefficients_byte_length must be {expected} for {count} splats at degree {degree}")
    if data is None:
        raise ValueError("SH sidecar bytes are required when manifest.sh is declared")
    return decode_float32_bytes(data, count * k * 3, "sh.coefficients").reshape(count, 3 * k), degree


def _first_bad_row(opacity: np.ndarray, radius: np.ndarray, op_path: str, rad_path: str) -> None:
    """Rows are checked in order, opacity before radius within a row."""
    bad_op = ~np.isfinite(opacity) | (opacity < 0) | (opacity > 1)
    bad_rad = ~np.isfinite(radius) | (radius <= 0)
    rows = np.nonzero(bad_op | bad_rad)[0]
    if not rows.size:
        return
    r = int(rows[0])
    if bad_op[r]:
        _unit_interval(float(opacity[r]), op_path.format(r))
    _positive_finite(float(radius[r]), rad_path.format(r))


def decode_first_smoke_manifest(manifest, payload: bytes, ids: bytes | None = None, scales: bytes | None = None,
                                rotations: bytes | None = None, sh: bytes | None = None,
                                roughness: bytes | None = None, metalness: bytes | None = None) -> SplatScene:
    """The manifest dict and the sidecars' bytes (None where absent)."""
    root = _record(manifest, "manifest")
    count = _positive_int(_first(root.get("splat_count"), root.get("count")), "splat_count")
    if _first(root.get("endianness"), "little") != "little":
        raise ValueError("manifest.endianness must be little")
    bounds = decode_bounds(root.get("bounds"), "bounds")
    kind = _source_kind(root)
    decode_layout(_layout_source(root), "layout")
    info = _record(root.get("payload"), "payload")
    expected = count * STRIDE_BYTES
    declared = _positive_int(_first(info.get("byte_length"), expected), "payload.byte_length")
    if declared != expected:
        raise ValueError(f"payload.byte_length must be {expected} for {count} rows")
    if len(payload) != expected:
        raise ValueError(f"payload sidecar byte length {len(payload)} does not match expected {expected}")
    rows = np.frombuffer(payload, "<f4").reshape(count, 8).astype(np.float32)
    positions, colors = rows[:, 0:3].copy(), rows[:, 3:6].copy()
    opacity, radius = rows[:, 6].copy(), rows[:, 7].copy()
    _first_bad_row(opacity, radius, "payload.rows[{}].opacity", "payload.rows[{}].radius")
    log_scales = (fallback_scales_from_radii(radius) if scales is None
                  else decode_float32_bytes(scales, count * 3, "shape.scales").reshape(count, 3))
    rot = (identity_rotations(count) if rotations is None
           else decode_float32_bytes(rotations, count * 4, "shape.rotations").reshape(count, 4))
    coeffs, degree = _decode_sh(root, count, sh)
    rough = None if roughness is None else decode_float32_bytes(roughness, count, "materials.roughness")
    metal = None if metalness is None else decode_float32_bytes(metalness, count, "materials.metalness")
    original = decode_original_ids(None, count) if ids is None else decode_original_id_bytes(ids, count)
    attrs = SplatAttributes(positions=positions, scales=log_scales, rotations=rot, opacities=opacity, colors=colors,
                            sh=coeffs, sh_degree=degree, roughness=rough, metalness=metal)
    return SplatScene(attributes=attrs, radii=radius, original_ids=original, bounds=bounds, source_kind=kind)


def decode_first_smoke_payload(payload) -> SplatScene:
    """Inline JSON: {metadata?, splats: [rows]} or {metadata?, attributes: {planar arrays}}."""
    root = _record(payload, "payload")
    meta = root if root.get("metadata") is None else _record(root["metadata"], "metadata")
    count = _positive_int(_first(meta.get("count"), meta.get("splat_count")), "count")
    bounds = decode_bounds(meta.get("bounds"), "bounds")
    decode_layout(_layout_source(meta), "layout")
    if root.get("splats") is not None:
        splats = root["splats"]
        if not isinstance(splats, list):
            raise ValueError("splats must be an array of first-smoke splat rows")
        if len(splats) != count:
            raise ValueError(f"count {count} does not match {len(splats)} rows")
        positions = np.empty((count, 3), np.float32)
        colors = np.empty((count, 3), np.float32)
        opacity = np.empty(count, np.float32)
        radius = np.empty(count, np.float32)
        for i, row in enumerate(splats):
            row = _record(row, f"splats[{i}]")
            positions[i] = _vec3(row.get("position"), f"splats[{i}].position")
            colors[i] = _vec3(row.get("color"), f"splats[{i}].color")
            opacity[i] = _unit_interval(row.get("opacity"), f"splats[{i}].opacity")
            radius[i] = _positive_finite(row.get("radius"), f"splats[{i}].radius")
        log_scales, rot = fallback_scales_from_radii(radius), identity_rotations(count)
    else:
        a = _record(root.get("attributes"), "attributes")
        positions = _decode_float32_array(_first(a.get("positions"), a.get("position")), count * 3,
                                          "attributes.positions").reshape(count, 3)
        colors = _decode_float32_array(_first(a.get("colors"), a.get("color")), count * 3,
                                       "attributes.colors").reshape(count, 3)
        opacity = _decode_float32_array(_first(a.get("opacities"), a.get("opacity")), count,
                                        "attributes.opacities", _unit_interval)
        radius = _decode_float32_array(_first(a.get("radii"), a.get("radius")), count, "attributes.radii",
                                       _positive_finite)
        log_scales = (fallback_scales_from_radii(radius) if a.get("scales") is None
                      else _decode_float32_array(a["scales"], count * 3, "attributes.scales").reshape(count, 3))
        rot = (identity_rotations(count) if a.get("rotations") is None
               else _decode_float32_array(a["rotations"], count * 4, "attributes.rotations").reshape(count, 4))
    kind = _string(_first(meta.get("sourceKind"), "real_scaniverse_ply"), "sourceKind")
    original = decode_original_ids(root.get("originalIds"), count)
    attrs = SplatAttributes(positions=positions, scales=log_scales, rotations=rot, opacities=opacity, colors=colors)
    return SplatScene(attributes=attrs, radii=radius, original_ids=original, bounds=bounds, source_kind=kind)


def _is_sidecar_manifest(doc) -> bool:
    return (isinstance(doc, dict) and isinstance(doc.get("payload"), dict)
            and isinstance(doc["payload"].get("path"), str))


def _sidecar_ids_path(root: dict):
    if root.get("ids") is not None:
        ids = _record(root["ids"], "ids")
        if ids.get("path") is not None:
            return _string(ids["path"], "ids.path")
    if root.get("identity") is not None:
        ident = _record(root["identity"], "identity")
        if ident.get("ids_path") is not None:
            return _string(ident["ids_path"], "identity.ids_path")
    return None


def _sidecar_shape_path(root: dict, key: str):
    if root.get("shape") is None:
        return None
    shape = _record(root["shape"], "shape")
    return None if shape.get(key) is None else _string(shape[key], f"shape.{key}")


def load_first_smoke(path) -> SplatScene:
    """A manifest (sidecars read beside it) or an inline JSON payload."""
    mpath = Path(path)
    doc = json.loads(mpath.read_text())
    if not _is_sidecar_manifest(doc):
        return decode_first_smoke_payload(doc)
    base = mpath.parent

    def read(rel):
        if rel is None:
            return None
        p = Path(rel)
        return (p if p.is_absolute() else base / p).read_bytes()

    sh_path = None if doc.get("sh") is None else _string(_record(doc["sh"], "sh").get("coefficients_path"),
                                                        "sh.coefficients_path")
    materials = doc.get("materials") if isinstance(doc.get("materials"), dict) else {}
    return decode_first_smoke_manifest(
        doc, read(_string(doc["payload"]["path"], "payload.path")), ids=read(_sidecar_ids_path(doc)),
        scales=read(_sidecar_shape_path(doc, "scales_path")), rotations=read(_sidecar_shape_path(doc, "rotations_path")),
        sh=read(sh_path), roughness=read(materials.get("roughness_path")),
        metalness=read(materials.get("metalness_path")))


@dataclass
class SplatFraming:
    target: tuple
    radius: float
    distance: float
    near: float
    far: float


def framing_from_bounds(bounds: SplatBounds, fov_y: float = math.pi / 3, padding: float = 1.35,
                        min_near: float = 0.001) -> SplatFraming:
    """A camera distance at which the padded bounding sphere fills fov_y."""
    if not math.isfinite(fov_y) or fov_y <= 0 or fov_y >= math.pi:
        raise ValueError("framing.fovY must be a finite angle in (0, pi)")
    if not math.isfinite(padding) or padding < 1:
        raise ValueError("framing.padding must be a finite value >= 1")
    half_diagonal = math.hypot(*(bounds.max[i] - bounds.min[i] for i in range(3))) / 2
    radius = max(bounds.radius, half_diagonal)
    padded = radius * padding
    distance = padded / math.sin(fov_y / 2)
    return SplatFraming(target=tuple(bounds.center), radius=radius, distance=distance,
                        near=max(min_near, distance - padded * 2), far=distance + padded * 2)


def camera_for_splat_bounds(bounds: SplatBounds) -> OrbitCamera:
    """configureCameraForSplatBounds: padding 1.45, azimuth 0, elevation 0.18."""
    f = framing_from_bounds(bounds, padding=1.45)
    return OrbitCamera(azimuth=0.0, elevation=0.18, distance=f.distance, target=f.target, near=f.near, far=f.far)


# applyRealScaniverseWitnessView (src/realSmokeScene.ts:196-237): close views of
# the first-smoke capture, (distance scale, target y offset) in bounds radii
WITNESS_VIEWS = {"dessert-close": (1.25, -0.08), "dessert-porous-close": (0.72, -0.14)}


def witness_view_camera(bounds: SplatBounds, mode: str = "default") -> OrbitCamera:
    """The framing camera ("default") or one of the reference's close views."""
    if mode == "default":
        return camera_for_splat_bounds(bounds)
    if mode not in WITNESS_VIEWS:
        raise ValueError(f"Unknown real Scaniverse witness view: {mode}")
    cam = camera_for_splat_bounds(bounds)
    scale, dy = WITNESS_VIEWS[mode]
    radius = max(bounds.radius, 0.001)
    cam.target = (bounds.center[0], bounds.center[1] + radius * dy, bounds.center[2])
    cam.distance = radius * scale
    cam.azimuth, cam.elevation = 0.0, 0.18
    return cam
