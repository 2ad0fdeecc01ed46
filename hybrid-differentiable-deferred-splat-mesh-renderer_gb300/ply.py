"""Binary 3DGS / Scaniverse PLY scenes and their Kaminos correction sidecars.

Restates src/localPly.ts of the reference:
  decode_local_ply           decodeLocalPlySplatPayload (:270-434) with
                             parseBinaryLittleEndianPlyHeader (:487-546),
                             findHeaderEnd (:574-599), the scalar types
                             (:601-657), discoverPlyShLayout / writePlyShRow
                             (:442-485), the point-cloud rejection (:548-572)
  apply_sidecar_corrections  applySidecarCorrections (:50-138): crop in the
                             preview-normalised space, Euler orientation, axis
                             flips, centroid offset, bounds recomputed
  filter_splat_attributes    filterSplatAttributes (:736-830)
  percentile_bounds          percentileBounds (:696-720) / recomputeBounds
                             (:722-734) / boundsFromExtents (:667-686)
  load_local_ply             main.ts's PLY route (:767-797): the file plus an
                             optional "<file>.kaminos-splat.json" sidecar
                             (tryFetchSidecar :26-37)

Arithmetic follows JavaScript: each value is a double, every store into a
Float32Array rounds to f32. Rows are decoded column-wise with numpy in the
same operation order. Math.hypot is restated (hypot_js) as V8 evaluates it
(scale by the largest magnitude, compensated sum of squares, sqrt, rescale),
so normalised quaternions round as the reference's do; exp/log/sin/cos come
from the host libm and agree with V8 to within an ulp of the double, which the
f32 store absorbs except at rounding ties.
"""
from __future__ import annotations

import json
import math
import re
from pathlib import Path

import numpy as np

from .assets import SplatBounds, SplatScene
from .splats import SplatAttributes

SH_C0 = 0.28209479177387814
_TYPES = {"char": "i1", "uchar": "u1", "short": "<i2", "ushort": "<u2", "int": "<i4", "uint": "<u4",
          "float": "<f4", "double": "<f8"}
_ALIASES = {"int8": "char", "uint8": "uchar", "int16": "short", "uint16": "ushort", "int32": "int",
            "uint32": "uint", "float32": "float", "float64": "double"}
_SIZES = {"char": 1, "uchar": 1, "short": 2, "ushort": 2, "int": 4, "uint": 4, "float": 4, "double": 8}


def hypot_js(*cols) -> np.ndarray:
    """Math.hypot over columns, in V8's order of operations."""
    cols = [np.asarray(c, np.float64) for c in cols]
    nan = np.zeros(cols[0].shape, bool)
    for c in cols:
        nan |= np.isnan(c)
    mags = [np.where(np.isnan(c), 0.0, np.abs(c)) for c in cols]
    big = mags[0].copy()
    for m in mags[1:]:
        big = np.maximum(big, m)
    safe = np.where((big == 0) | np.isinf(big), 1.0, big)
    total = np.zeros_like(big)
    comp = np.zeros_like(big)
    with np.errstate(invalid="ignore"):
        for m in mags:
            n = m / safe
            summand = n * n - comp
            prelim = total + summand
            comp = (prelim - total) - summand
            total = prelim
        out = np.sqrt(total) * big
    out = np.where(big == 0, 0.0, out)
    out = np.where(nan, np.nan, out)
    return np.where(np.isinf(big), np.inf, out)


def _f32(x) -> np.ndarray:
    """A Float32Array store: round to nearest, out-of-range values to +-inf."""
    with np.errstate(over="ignore"):
        return np.asarray(x, np.float64).astype(np.float32)


def _find_header_end(data: bytes):
    i = data.find(b"end_header")
    if i < 0:
        raise ValueError("Dropped file does not contain a complete PLY header")
    off = i + len(b"end_header")
    text_end = off
    if off < len(data) and data[off] == 13:
        off += 1
    if off < len(data) and data[off] == 10:
        off += 1
    return text_end, off


def _js_number(text: str) -> float:
    """Number(text) for the header's count field."""
    t = text.strip()
    if t == "":
        return 0.0
    try:
        if re.fullmatch(r"[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|Infinity)", t):
            return float(t.replace("Infinity", "inf"))
        if re.fullmatch(r"0[xX][0-9a-fA-F]+", t):
            return float(int(t, 16))
    except ValueError:
        pass
    return math.nan


def parse_ply_header(file_name: str, data: bytes) -> dict:
    text_end, data_offset = _find_header_end(data)
    lines = re.split(r"\r?\n", data[:text_end].decode("ascii", errors="replace"))
    if lines[0] != "ply":
        raise ValueError("Dropped file does not start with a PLY header")
    fmt = None
    vertex_count = None
    in_vertex = False
    props = []
    stride = 0
    for line in lines[1:]:
        parts = line.strip().split()
        if not parts:
            continue
        if parts[0] == "format":
            fmt = " ".join(p for p in parts[1:3] if p)
        elif parts[0] == "element":
            in_vertex = len(parts) > 1 and parts[1] == "vertex"
            if in_vertex:
                vertex_count = _js_number(parts[2]) if len(parts) > 2 else math.nan
        elif parts[0] == "property" and in_vertex:
            if len(parts) > 1 and parts[1] == "list":
                raise ValueError("PLY vertex list properties are not supported for splat drag-drop")
            kind = parts[1] if len(parts) > 1 else ""
            kind = _ALIASES.get(kind, kind)
            if kind not in _TYPES:
                raise ValueError(f"Unsupported PLY scalar property type: {parts[1] if len(parts) > 1 else ''}")
            props.append((parts[2] if len(parts) > 2 else "undefined", kind, stride))
            stride += _SIZES[kind]
    if vertex_count is None or not math.isfinite(vertex_count) or vertex_count != int(vertex_count) \
            or vertex_count <= 0:
        raise ValueError("PLY vertex count must be a positive integer")
    if not props:
        raise ValueError("PLY vertex element has no scalar properties")
    fmt = fmt or "unknown"
    names = {p[0] for p in props}
    has = names.issuperset
    if has({"x", "y", "z"}) and has({"red", "green", "blue"}) and not (
            has({"scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"}) or "opacity" in names):
        raise ValueError(" ".join([
            "Unsupported PLY schema for hybrid splat renderer:",
            f"parser=ply-point-cloud-v0; format={fmt}; vertexCount={int(vertex_count)}; colorSource=rgb; "
            f"properties={','.join(p[0] for p in props)}; file={file_name}.",
            "This is a valid point-cloud PLY route, not a Gaussian splat PLY/SPZ payload.",
            "Kaminos cheap preview may accept it, but the hybrid renderer needs splat covariance/opacity "
            "fields before rendering it as splats."]))
    if fmt not in ("binary_little_endian 1.0", "binary_little_endian"):
        raise ValueError("Only binary_little_endian PLY drag-drop is supported")
    return {"format": fmt, "vertex_count": int(vertex_count), "properties": props, "row_stride": stride,
            "data_offset": data_offset}


def _bounds_from_extents(lo, hi) -> SplatBounds:
    lo = [float(v) for v in lo]
    hi = [float(v) for v in hi]
    center = tuple((lo[i] + hi[i]) * 0.5 for i in range(3))
    half = [np.float64((hi[i] - lo[i]) * 0.5) for i in range(3)]
    radius = float(hypot_js(*[np.array([h]) for h in half])[0])
    return SplatBounds(min=tuple(lo), max=tuple(hi), center=center, radius=radius)


def percentile_bounds(positions: np.ndarray, trim: float = 0.05) -> SplatBounds:
    """P5-P95 extents over at most 50,000 evenly strided rows."""
    pos = np.asarray(positions, np.float32).reshape(-1, 3)
    count = pos.shape[0]
    samples = min(count, 50000)
    step = count / samples
    idx = np.floor(np.arange(samples, dtype=np.float64) * step).astype(np.int64)
    cols = np.sort(pos[idx], axis=0)  # Float32Array sort: numeric, NaN last
    lo = math.floor(samples * trim)
    hi = min(math.floor(samples * (1 - trim)), samples - 1)
    return _bounds_from_extents(cols[lo].astype(np.float64), cols[hi].astype(np.float64))


def recompute_bounds(positions: np.ndarray) -> SplatBounds:
    pos = np.asarray(positions, np.float32).reshape(-1, 3)
    if pos.shape[0] > 100:
        return percentile_bounds(pos, 0.05)
    if pos.shape[0] == 0:
        return _bounds_from_extents([math.inf] * 3, [-math.inf] * 3)
    return _bounds_from_extents(pos.min(0).astype(np.float64), pos.max(0).astype(np.float64))


def _sh_layout(fields: dict):
    rest = sorted((int(n[len("f_rest_"):]), n) for n in fields if re.fullmatch(r"f_rest_\d+", n))
    if not rest:
        return None
    if len(rest) % 3:
        raise ValueError(f"PLY f_rest_* field count must be divisible by 3 RGB channels, got {len(rest)}")
    k = len(rest) // 3
    degree = math.sqrt(k + 1) - 1
    if degree != int(degree) or degree <= 0:
        raise ValueError(f"PLY f_rest_* field count {len(rest)} does not describe a complete SH degree")
    names = [n for _, n in rest]
    return int(degree), k, [names[c * k:(c + 1) * k] for c in range(3)]


def decode_local_ply(file_name: str, data: bytes) -> SplatScene:
    """A binary little-endian 3DGS PLY: raw fields decoded into activated attributes."""
    header = parse_ply_header(file_name, data)
    count = header["vertex_count"]
    stride = header["row_stride"]
    fields = {}
    for i, (name, kind, off) in enumerate(header["properties"]):
        fields[name] = (i, kind, off)  # a repeated name: the last one wins (a Map)
    for name in ("x", "y", "z"):
        if name not in fields:
            raise ValueError(f"PLY vertex property {name} is required")
    sh = _sh_layout(fields)
    if header["data_offset"] + count * stride > len(data):
        raise ValueError(f"{file_name} ended before all {count} vertex rows could be read")
    dt = np.dtype({"names": [f"p{i}" for i, _ in enumerate(header["properties"])],
                   "formats": [_TYPES[k] for _, k, _ in header["properties"]],
                   "offsets": [o for _, _, o in header["properties"]], "itemsize": stride})
    rows = np.frombuffer(data, dtype=dt, count=count, offset=header["data_offset"])

    def col(name) -> np.ndarray:
        return rows[f"p{fields[name][0]}"].astype(np.float64)

    def has(*names) -> bool:
        return all(n in fields for n in names)

    xyz = np.stack([col("x"), col("y"), col("z")], 1)
    positions = _f32(xyz)
    if has("f_dc_0", "f_dc_1", "f_dc_2"):
        colors = _f32(np.clip(np.stack([0.5 + SH_C0 * col(f"f_dc_{c}") for c in range(3)], 1), 0.0, 1.0))
    elif has("red", "green", "blue"):
        colors = _f32(np.clip(np.stack([col(c) / 255 for c in ("red", "green", "blue")], 1), 0.0, 1.0))
    else:
        colors = np.full((count, 3), 0.5, np.float32)
    opacities = _f32(1.0 / (1.0 + np.exp(-col("opacity")))) if has("opacity") else np.ones(count, np.float32)
    if has("scale_0", "scale_1", "scale_2"):
        scales = _f32(np.stack([col(f"scale_{c}") for c in range(3)], 1))
    else:
        scales = np.zeros((count, 3), np.float32)
    radii = _f32(np.exp(scales.astype(np.float64)).max(1))
    if has("rot_0", "rot_1", "rot_2", "rot_3"):
        rotations = _f32(np.stack([col(f"rot_{c}") for c in range(4)], 1))
    else:
        rotations = np.zeros((count, 4), np.float32)
        rotations[:, 0] = 1.0

    def triple(*names):
        return _f32(np.stack([col(n) for n in names], 1)) if has(*names) else None

    coeffs, degree = None, 0
    if sh is not None:
        degree, k, by_channel = sh
        coeffs = np.empty((count, k, 3), np.float32)
        for c in range(3):
            for j, name in enumerate(by_channel[c]):
                coeffs[:, j, c] = _f32(col(name))
        coeffs = coeffs.reshape(count, 3 * k)
    if count > 100:
        bounds = percentile_bounds(positions, 0.05)
    else:
        bounds = _bounds_from_extents(xyz.min(0), xyz.max(0))
    attrs = SplatAttributes(
        positions=positions, scales=scales, rotations=rotations, opacities=opacities, colors=colors, sh=coeffs,
        sh_degree=degree, normals=triple("nx", "ny", "nz"),
        detail_normals=triple("detail_normal_x", "detail_normal_y", "detail_normal_z"),
        roughness=_f32(col("roughness")) if has("roughness") else None,
        metalness=_f32(col("metallic")) if has("metallic") else None,
        emissive=triple("emissive_r", "emissive_g", "emissive_b"))
    return SplatScene(attributes=attrs, radii=radii, original_ids=np.arange(count, dtype=np.uint32), bounds=bounds,
                      source_kind="scaniverse_ply")


def filter_splat_attributes(scene: SplatScene, keep: np.ndarray) -> SplatScene:
    """The rows where keep is set, every per-splat array alike; bounds recomputed."""
    keep = np.asarray(keep, bool)
    a = scene.attributes

    def sel(x):
        return None if x is None else np.ascontiguousarray(np.asarray(x)[keep])

    attrs = SplatAttributes(
        positions=sel(a.positions), scales=sel(a.scales), rotations=sel(a.rotations), opacities=sel(a.opacities),
        colors=sel(a.colors), sh=sel(a.sh), sh_degree=a.sh_degree, normals=sel(a.normals),
        detail_normals=sel(a.detail_normals), roughness=sel(a.roughness), metalness=sel(a.metalness),
        emissive=sel(a.emissive), splat_scale=a.splat_scale)
    return SplatScene(attributes=attrs, radii=sel(scene.radii), original_ids=sel(scene.original_ids),
                      bounds=recompute_bounds(attrs.positions), source_kind=scene.source_kind)


def _normalize(q):
    """normalizeQuaternion on doubles (columns w, x, y, z)."""
    n = hypot_js(*q)
    zero = n == 0
    safe = np.where(zero, 1.0, n)
    return [np.where(zero, 1.0 if i == 0 else 0.0, q[i] / safe) for i in range(4)]


def _normalize_rows_f32(rot: np.ndarray) -> np.ndarray:
    """normalizeQuaternionInPlace on a Float32Array: hypot of the f32 values, each divided, stored f32."""
    cols = [rot[:, i].astype(np.float64) for i in range(4)]
    return _f32(np.stack(_normalize(cols), 1))


def quaternion_from_euler_xyz(rx: float, ry: float, rz: float):
    c1, c2, c3 = math.cos(rx * 0.5), math.cos(ry * 0.5), math.cos(rz * 0.5)
    s1, s2, s3 = math.sin(rx * 0.5), math.sin(ry * 0.5), math.sin(rz * 0.5)
    q = [np.array([c1 * c2 * c3 - s1 * s2 * s3]), np.array([s1 * c2 * c3 + c1 * s2 * s3]),
         np.array([c1 * s2 * c3 - s1 * c2 * s3]), np.array([c1 * c2 * s3 + s1 * s2 * c3])]
    return tuple(float(v[0]) for v in _normalize(q))


def _rotate_triples(v: np.ndarray, q) -> np.ndarray:
    w, x, y, z = q
    vx, vy, vz = (v[:, i].astype(np.float64) for i in range(3))
    tx = 2 * (y * vz - z * vy)
    ty = 2 * (z * vx - x * vz)
    tz = 2 * (x * vy - y * vx)
    return _f32(np.stack([vx + w * tx + (y * tz - z * ty), vy + w * ty + (z * tx - x * tz),
                          vz + w * tz + (x * ty - y * tx)], 1))


def _rotate_rotations(rot: np.ndarray, a) -> np.ndarray:
    b = [rot[:, i].astype(np.float64) for i in range(4)]
    m = [a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3],
         a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2],
         a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1],
         a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0]]
    return _normalize_rows_f32(_f32(np.stack(_normalize(m), 1)))


def apply_sidecar_corrections(scene: SplatScene, sidecar: dict) -> SplatScene:
    """Crop (preview-normalised space), Euler orientation, axis flips, centroid offset; in that order."""
    corr = sidecar["correction"]
    crop = corr.get("crop")
    if crop and crop.get("enabled"):
        pos = scene.attributes.positions.astype(np.float64)
        lo, hi = pos.min(0), pos.max(0)
        center = (lo + hi) * 0.5
        extent = max(float(hi[0] - lo[0]), float(hi[1] - lo[1]), float(hi[2] - lo[2]), 1e-6)
        scale = 2.0 / extent
        preview = (pos - center) * scale
        cmin = np.asarray(crop["min"], np.float64)
        cmax = np.asarray(crop["max"], np.float64)
        keep = np.all((preview >= cmin) & (preview <= cmax), axis=1)
        kept = int(keep.sum())
        if 0 < kept < scene.count:
            scene = filter_splat_attributes(scene, keep)
        # kept == 0: the crop is stale and skipped, as the reference warns and skips
    a = scene.attributes
    positions, normals, rotations = a.positions.copy(), None if a.normals is None else a.normals.copy(), \
        a.rotations.copy()
    orient = (corr.get("orientation") or {}).get("rotation")
    if orient:
        q = quaternion_from_euler_xyz(*map(float, orient))
        if not (abs(q[0] - 1) < 1e-12 and abs(q[1]) < 1e-12 and abs(q[2]) < 1e-12 and abs(q[3]) < 1e-12):
            positions = _rotate_triples(positions, q)
            if normals is not None:
                normals = _rotate_triples(normals, q)
            rotations = _rotate_rotations(rotations, q)
    flips = corr.get("axisFlips")
    if flips:
        fx, fy, fz = map(float, flips)
        if fx != 1 or fy != 1 or fz != 1:
            f = np.array([fx, fy, fz])
            positions = _f32(positions.astype(np.float64) * f)
            if normals is not None:
                normals = _f32(normals.astype(np.float64) * f)
            s = np.array([1.0, fy * fz, fx * fz, fx * fy])
            rotations = _normalize_rows_f32(_f32(rotations.astype(np.float64) * s))
    offset = corr.get("centroidOffset")
    if offset:
        positions = _f32(positions.astype(np.float64) - np.asarray(offset, np.float64))
    attrs = SplatAttributes(
        positions=positions, scales=a.scales, rotations=rotations, opacities=a.opacities, colors=a.colors, sh=a.sh,
        sh_degree=a.sh_degree, normals=normals, detail_normals=a.detail_normals, roughness=a.roughness,
        metalness=a.metalness, emissive=a.emissive, splat_scale=a.splat_scale)
    return SplatScene(attributes=attrs, radii=scene.radii, original_ids=scene.original_ids,
                      bounds=recompute_bounds(positions), source_kind=scene.source_kind)


def load_local_ply(path, use_sidecar: bool = True) -> SplatScene:
    """A PLY file, corrected by "<path>.kaminos-splat.json" when that holds a correction."""
    p = Path(path)
    scene = decode_local_ply(p.name, p.read_bytes())
    side = Path(str(p) + ".kaminos-splat.json")
    if use_sidecar and side.exists():
        try:
            doc = json.loads(side.read_text())
        except (OSError, ValueError):
            doc = None
        if isinstance(doc, dict) and doc.get("correction"):
            scene = apply_sidecar_corrections(scene, doc)
    return scene
