"""Cut a small subset of the reference's real first-smoke capture into tests/golden.

The reference ships one real scene, smoke-assets/scaniverse-first-smoke (a
94,406-splat Scaniverse capture: a manifest, 32-byte rows and sidecars for ids,
log scales, wxyz rotations, roughness and metalness). This script keeps a
seeded sample of its rows, in file order, and writes them in the same format
to tests/golden/first_smoke_subset/:
  - the rows, scales, rotations, roughness and metalness of the kept rows,
    byte for byte;
  - ids 0..n-1 (the format wants ids < splat_count; the kept rows' original
    row numbers go to a source_rows.u32.bin sidecar instead);
  - bounds recomputed over the kept positions the way the capture's own
    bounds are made (min, max, their midpoint, half the diagonal);
  - a "subset" record: the source manifest, its payload's sha256, the seed and
    the sha256 of every written sidecar.
Usage: python tests/golden/make_first_smoke_subset.py <reference_root> [count]
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "first_smoke_subset"
SEED = 20240611
NAME = "first-smoke-subset"


def main(ref_root: Path, count: int) -> None:
    src_dir = ref_root / "smoke-assets" / "scaniverse-first-smoke"
    manifest_path = src_dir / "scaniverse-first-smoke.json"
    src = json.loads(manifest_path.read_text())
    n = int(src["splat_count"])
    rows = np.random.Generator(np.random.PCG64(SEED)).choice(n, size=count, replace=False)
    rows.sort()

    payload_bytes = (src_dir / src["payload"]["path"]).read_bytes()
    payload = np.frombuffer(payload_bytes, "<f4").reshape(n, 8)
    sidecars = {
        "payload": (payload[rows].tobytes(), f"{NAME}.f32.bin"),
        "ids": (np.arange(count, dtype="<u4").tobytes(), f"{NAME}.ids.u32.bin"),
        "source_rows": (rows.astype("<u4").tobytes(), f"{NAME}.source_rows.u32.bin"),
    }
    for key, width in (("scales_path", 3), ("rotations_path", 4)):
        data = np.frombuffer((src_dir / src["shape"][key]).read_bytes(), "<f4").reshape(n, width)
        sidecars[key] = (data[rows].tobytes(), f"{NAME}.{key.split('_')[0]}.f32.bin")
    for key in ("roughness_path", "metalness_path"):
        data = np.frombuffer((src_dir / src["materials"][key]).read_bytes(), "<f4")
        sidecars[key] = (data[rows].tobytes(), f"{NAME}.{key.split('_')[0]}.f32.bin")

    pos = payload[rows, 0:3].astype(np.float64)
    lo, hi = pos.min(0), pos.max(0)
    bounds = {"min": lo.tolist(), "max": hi.tolist(), "center": ((lo + hi) / 2).tolist(),
              "radius": float(np.linalg.norm(hi - lo) / 2)}

    manifest = {
        "schema": src["schema"],
        "asset_name": NAME,
        "source": dict(src["source"]),
        "splat_count": count,
        "endianness": "little",
        "stride_bytes": 32,
        "fields": src["fields"],
        "payload": {"path": sidecars["payload"][1], "component_type": "float32", "byte_length": count * 32},
        "identity": {"scheme": "row_index_is_original_zero_based_file_order", "ids_component_type": "uint32",
                     "ids_path": sidecars["ids"][1]},
        "ids": {"path": sidecars["ids"][1], "byte_length": count * 4, "first_id": 0, "last_id": count - 1},
        "shape": {"scales_path": sidecars["scales_path"][1], "scales_component_type": "float32",
                  "scales_byte_length": count * 12, "rotations_path": sidecars["rotations_path"][1],
                  "rotations_component_type": "float32", "rotations_byte_length": count * 16,
                  "rotation_order": "wxyz", "scale_space": "log"},
        "bounds": bounds,
        "materials": {"roughness_path": sidecars["roughness_path"][1], "roughness_component_type": "float32",
                      "roughness_byte_length": count * 4, "metalness_path": sidecars["metalness_path"][1],
                      "metalness_component_type": "float32", "metalness_byte_length": count * 4},
        "subset": {
            "source_manifest": "smoke-assets/scaniverse-first-smoke/scaniverse-first-smoke.json",
            "source_splat_count": n,
            "source_payload_sha256": hashlib.sha256(payload_bytes).hexdigest(),
            "seed": SEED,
            "sampler": "numpy PCG64 choice without replacement, sorted",
            "source_rows_path": sidecars["source_rows"][1],
            "sha256": {name: hashlib.sha256(data).hexdigest() for data, name in sidecars.values()},
        },
    }
    OUT.mkdir(exist_ok=True)
    for data, name in sidecars.values():
        (OUT / name).write_bytes(data)
    (OUT / f"{NAME}.json").write_text(json.dumps(manifest, indent=2) + "\n")
    print(f"wrote {count} of {n} rows to {OUT}")


if __name__ == "__main__":
    if len(sys.argv) not in (2, 3):
        sys.exit("usage: make_first_smoke_subset.py <path of the reference checkout> [rows, default 4096]")
    main(Path(sys.argv[1]), int(sys.argv[2]) if len(sys.argv) > 2 else 4096)
