"""Differentiable frames: torch.autograd over the compositor.

The forward is the compositor frame itself (hdsr_encode_full, rgba f32
output); the backward is hdsr_encode_backward on the same handle. The scene
tensors are bound by pointer for each call, so they must be contiguous
float32 CUDA tensors in the layouts of the scene views: positions (N, 3),
log-scales (N, 3), wxyz rotations (N, 4), activated opacities (N,), SH rows
(N, 6 + 3K) = [dc | higher orders | emissive]. Opacity logits go through
torch.sigmoid before the call, so autograd supplies that factor.
sortedIndices (the back-to-front order) is an input, not differentiated.
"""
from __future__ import annotations

import numpy as np

from . import compositor as _c


class SplatFrameRenderer:
    """One handle (with the adjoint buffers) and its f32 output images."""

    def __init__(self, width: int, height: int, splat_count: int, sh_degree: int = 0, pair_capacity: int = 0,
                 device: str = "cuda"):
        import torch

        self.plan = _c.plan_tile_splat_compositor(width, height, 16, splat_count)
        self.sh_degree = sh_degree
        self.pair_capacity = pair_capacity
        self.device = device
        self.res = _c.create_tile_splat_compositor(self.plan, pair_capacity, f32_color=True, backward=True)
        self.color, self.gb = _c.create_output_textures(self.plan, f32_color=True, device=device)
        self.material = torch.zeros(splat_count, dtype=torch.int32, device=device)

    def _bind(self, positions, log_scales, rotations, opacities, sh, sorted_indices):
        bufs = {"positions": positions, "scales": log_scales, "rotations": rotations, "opacities": opacities,
                "material": self.material, "normals": None, "sh_data": sh, "sorted_indices": sorted_indices,
                "sh_degree": self.sh_degree}
        _c.create_tile_splat_bind_groups(self.res, bufs, self.color, self.gb)

    def forward_frame(self, positions, log_scales, rotations, opacities, sh, sorted_indices, uniforms):
        """Encode one frame; grows the pair capacity when the frame needs it."""
        self._bind(positions, log_scales, rotations, opacities, sh, sorted_indices)
        _c.write_frame_uniform_buffer(self.res, uniforms)
        _c.encode_full_compute_compositor_pipeline(None, self.res)
        st = self.res.query_status()
        if st["status"] != 0:
            need = int(st["total_pairs"])
            if need <= self.res.pair_capacity:
                self.res.check_frame()
            self.res.destroy()
            self.pair_capacity = int(need * 1.25) + 4096
            self.res = _c.create_tile_splat_compositor(self.plan, self.pair_capacity, f32_color=True, backward=True)
            self._bind(positions, log_scales, rotations, opacities, sh, sorted_indices)
            _c.write_frame_uniform_buffer(self.res, uniforms)
            _c.encode_full_compute_compositor_pipeline(None, self.res)
            self.res.check_frame()
        return self.color

    def render(self, positions, log_scales, rotations, opacities, sh, sorted_indices, uniforms):
        """Differentiable (H, W, 4) rgba frame."""
        return _SplatFrame.apply(positions, log_scales, rotations, opacities, sh, self, sorted_indices,
                                 np.ascontiguousarray(uniforms, np.float32))

    def destroy(self) -> None:
        self.res.destroy()


def _check(t, cols, name):
    import torch

    assert t.dtype == torch.float32 and t.is_cuda and t.is_contiguous(), f"{name}: contiguous float32 CUDA tensor"
    assert t.dim() == (1 if cols is None else 2) and (cols is None or t.shape[1] == cols), f"{name}: shape"


def _function():
    import torch

    class SplatFrame(torch.autograd.Function):
        @staticmethod
        def forward(ctx, positions, log_scales, rotations, opacities, sh, renderer, sorted_indices, uniforms):
            n = renderer.plan.splat_count
            for t, c, name in ((positions, 3, "positions"), (log_scales, 3, "log_scales"), (rotations, 4, "rotations"),
                               (opacities, None, "opacities"), (sh, 6 + 3 * ((renderer.sh_degree + 1) ** 2 - 1), "sh")):
                _check(t, c, name)
                assert t.shape[0] == n, f"{name}: {n} rows"
            ctx.renderer = renderer
            ctx.shapes = (positions, log_scales, rotations, opacities, sh)
            color = renderer.forward_frame(positions, log_scales, rotations, opacities, sh, sorted_indices, uniforms)
            return color.clone()

        @staticmethod
        def backward(ctx, d_color):
            import torch

            r = ctx.renderer
            positions, log_scales, rotations, opacities, sh = ctx.shapes
            grads = {"positions": torch.empty_like(positions), "log_scales": torch.empty_like(log_scales),
                     "rotations": torch.empty_like(rotations), "opacities": torch.empty_like(opacities),
                     "sh": torch.empty_like(sh)}
            _c.encode_backward(None, r.res, d_color.contiguous().float(), grads)
            return (grads["positions"], grads["log_scales"], grads["rotations"], grads["opacities"], grads["sh"],
                    None, None, None)

    return SplatFrame


class _Lazy:
    fn = None

    @classmethod
    def apply(cls, *args):
        if cls.fn is None:
            cls.fn = _function()
        return cls.fn.apply(*args)


_SplatFrame = _Lazy
