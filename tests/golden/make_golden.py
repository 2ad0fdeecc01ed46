"""Extract the reference's known-answer vectors for this path into JSON.

Reads the reference's unit tests as text (they are TypeScript / Node tests
and cannot run here) and writes reference_kats.json:
  - tests/cpuDepthSort.test.ts: back-to-front orders, view depths, the
    equal-depth tie rule and the malformed-input errors of splatSort.ts;
  - tests/renderer/computeCompositorLifecycle.test.mjs: the compositor
    constants it asserts (dispatch-safe ref cap, 8-tile footprint clamp,
    projection-cache stride).
Usage: python tests/golden/make_golden.py <reference_root>
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def floats(block: str) -> list[float]:
    body = re.sub(r"//[^\n]*", "", block)
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?", body)]


def float32_arrays(text: str) -> dict[str, list[float]]:
    out = {}
    for m in re.finditer(r"const (\w+) = new Float32Array\(\[(.*?)\]\);", text, re.S):
        out.setdefault(m.group(1), []).append(floats(m.group(2)))
    return out


def main(ref_root: Path) -> None:
    depth_src = (ref_root / "tests" / "cpuDepthSort.test.ts").read_text()
    arrays = float32_arrays(depth_src)
    cases = []
    # test 1: identity view
    t1 = depth_src.split('test("sorts packed xyz positions back-to-front by view-space z"')[1].split("\ntest(")[0]
    cases.append({
        "name": "identity_view_back_to_front",
        "positions": floats(re.search(r"positions = new Float32Array\(\[(.*?)\]\)", t1, re.S).group(1)),
        "view": arrays["identityView"][0],
        "order": [int(x) for x in floats(re.search(r"Array\.from\(order\), \[(.*?)\]", t1).group(1))],
    })
    t2 = depth_src.split('test("uses the full column-major view matrix instead of raw world z"')[1].split("\ntest(")[0]
    translated = floats(re.search(r"translatedView = new Float32Array\(\[(.*?)\]\)", t2, re.S).group(1))
    pos2 = floats(re.search(r"const positions = new Float32Array\(\[(.*?)\]\)", t2, re.S).group(1))
    depths = [float(x) for x in re.findall(r"computeViewSpaceDepth\(positions, \d, translatedView\), (-?\d+)\)", t2)]
    orders = re.findall(r"\),\s*\[(.*?)\]\s*\);", t2, re.S)
    cases.append({"name": "translated_view", "positions": pos2, "view": translated, "depths": depths,
                  "order": [int(x) for x in floats(orders[0])]})
    xview = floats(re.search(r"xDepthView = new Float32Array\(\[(.*?)\]\)", t2, re.S).group(1))
    same = floats(re.search(r"sameWorldZ = new Float32Array\(\[(.*?)\]\)", t2, re.S).group(1))
    cases.append({"name": "x_depth_view", "positions": same, "view": xview,
                  "order": [int(x) for x in floats(orders[1])]})
    t3 = depth_src.split('test("keeps equal-depth splats in original file-order id order"')[1].split("\ntest(")[0]
    cases.append({
        "name": "equal_depth_file_order",
        "positions": floats(re.search(r"positions = new Float32Array\(\[(.*?)\]\)", t3, re.S).group(1)),
        "view": arrays["identityView"][0],
        "order": [int(x) for x in floats(re.search(r"identityView\)\),\s*\[(.*?)\]", t3, re.S).group(1))],
    })
    errors = re.findall(r"assert\.throws\(\s*\(\) => sortSplatIdsBackToFront\(new Float32Array\((\[[^)]*\])\), "
                        r"(\w+|new Float32Array\(\d+\))\),\s*/(.*?)/", depth_src, re.S)
    err_cases = []
    for arg, view_arg, msg in errors:
        if view_arg == "identityView":
            view = arrays["identityView"][0]
        else:
            view = [0.0] * int(re.search(r"\((\d+)\)", view_arg).group(1))
        err_cases.append({"positions": floats(arg.strip("[]")), "view": view, "message": msg})
    life = (ref_root / "tests" / "renderer" / "computeCompositorLifecycle.test.mjs").read_text()
    m_cap = re.search(r"MAX_DISPATCH_SAFE = (\d+) \* (\d+);", life)
    m_clamp = re.search(r"clampedRadius = min\\\(radius, tileSize \\\* (\d+)\\\.0\\\)", life)
    m_stride = re.search(r"PROJ_STRIDE = (\d+)u", life)
    out = {
        "source": ["tests/cpuDepthSort.test.ts", "tests/renderer/computeCompositorLifecycle.test.mjs"],
        "cpu_depth_sort": cases,
        "cpu_depth_sort_errors": err_cases,
        "compositor_constants": {
            "max_dispatch_safe_refs": int(m_cap.group(1)) * int(m_cap.group(2)),
            "footprint_clamp_tiles": int(m_clamp.group(1)),
            "proj_stride_u32": int(m_stride.group(1)),
        },
    }
    (HERE / "reference_kats.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out["compositor_constants"]), len(cases), "sort cases", len(err_cases), "error cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    main(Path(sys.argv[1]))
