"""The real first-smoke capture (the committed 4,096-splat subset) rendered
through the C ABI with the reference's framing camera and its two close
views, checked stage by stage and bit for bit against the oracle."""
from pathlib import Path

import numpy as np
import pytest

from gpu_helpers import assert_frame_parity, render_gpu

pytestmark = pytest.mark.gpu

SUBSET = Path(__file__).resolve().parent / "golden" / "first_smoke_subset" / "first-smoke-subset.json"


@pytest.mark.parametrize("mode,W,H", [("default", 640, 480), ("default", 1280, 720),
                                      ("dessert-close", 1280, 720), ("dessert-porous-close", 960, 540)])
def test_first_smoke_subset_parity(cuda, pkg, orc, mode, W, H):
    d = pkg.assets.load_first_smoke(SUBSET)
    cam = pkg.assets.witness_view_camera(d.bounds, mode)
    g = render_gpu(pkg, d.attributes, cam, W, H)
    gpu, ref = assert_frame_parity(orc, g)
    assert ref["total_pairs"] >= d.count // 2
    # the frame is not empty: some pixels hold splats, with material from the sidecars
    alpha = gpu["color"][..., 3].astype(np.float32)
    assert (alpha > 0).mean() > 0.01
    g["res"].destroy()
