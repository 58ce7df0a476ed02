"""Differentiable shading of many views of one mesh, as a torch.autograd.Function.

The renderer and both shading passes are the library's (sloth_batch_render,
sloth_batch_shade, sloth_batch_shade_backward); torch only holds the device tensors,
orders the work on one CUDA stream and runs the loss and the optimiser.  The reference
renderer has no differentiable path (its shading is the normal's z of
src/rasterizer.rs:76); the image and its adjoint are documented in include/sloth_gpu.h.
"""
from __future__ import annotations

import numpy as np
import torch

import sloth_gpu as S


class ShadedViews:
    """Views of one mesh, rendered as one batch and shaded differentiably.

    mesh: host dict with x, y, z (f32 per vertex), rgb (u8 face colours), idx (optional)
    and bbox_max; views: list of dicts {w, h, image, U, R}.  All work goes to `stream`,
    which must be the current torch stream whenever this object is used.  The visibility
    of each render (8 bytes per depth cell) is kept for the backward pass when
    store_visibility is True, decoded again from the depth keys when False, and kept when
    it fits vis_budget_bytes when None."""

    VIS_BYTES_PER_CELL = 8

    def __init__(self, ctx: S.Context, mesh: dict, views: list[dict], stream: torch.cuda.Stream,
                 store_visibility: bool | None = True, vis_budget_bytes: int = 1 << 30):
        if stream.cuda_stream == 0:
            raise ValueError("ShadedViews needs a dedicated (non-default) stream")
        self.ctx, self.stream = ctx, stream
        self.device = torch.device("cuda", ctx.device)
        self.mesh = S.Mesh(ctx, mesh["x"], mesh["y"], mesh["z"], mesh["rgb"], mesh.get("idx"),
                           mesh.get("bbox_max"))
        self.nvert, self.ntri = self.mesh.nvert, self.mesh.ntri
        frames = [{"w": v["w"], "h": v["h"], "image": v["image"], "U": v["U"], "draws": [(self.mesh, v["R"])]}
                  for v in views]
        self.batch = S.Batch(ctx, frames)
        self.cells = [self.batch.depth_cells(i) for i in range(len(views))]
        self.ncells = sum(n for _, n in self.cells)
        self.face_rgb = torch.from_numpy(np.ascontiguousarray(mesh["rgb"], np.uint8).reshape(-1)).to(self.device)
        # store the visibility when it fits the budget (None), or as the caller says
        if store_visibility is None:
            store_visibility = self.ncells * self.VIS_BYTES_PER_CELL <= vis_budget_bytes
        self.store_visibility = bool(store_visibility)
        self._keep = None

    def _check_stream(self):
        if torch.cuda.current_stream(self.device).cuda_stream != self.stream.cuda_stream:
            raise RuntimeError("ShadedViews used outside its stream")

    def render(self, pos: torch.Tensor):
        """Upload (nvert, 3) positions and render every view."""
        self._check_stream()
        p = pos.detach().to(torch.float32)
        x, y, z = p[:, 0].contiguous(), p[:, 1].contiguous(), p[:, 2].contiguous()
        self._keep = (x, y, z)          # the copies read them asynchronously
        self.mesh.update_device(x.data_ptr(), y.data_ptr(), z.data_ptr(), self.face_rgb.data_ptr())
        self.batch.render()

    def shade(self, vrgb: torch.Tensor, light: torch.Tensor) -> torch.Tensor:
        """(ncells, 3) f32 image of the last render."""
        self._check_stream()
        out = torch.empty(self.ncells, 3, dtype=torch.float32, device=self.device)
        self.batch.shade(vrgb.data_ptr(), light.data_ptr(), out.data_ptr(), self.store_visibility)
        return out

    def shade_backward(self, vrgb, light, grad_rgb):
        self._check_stream()
        gpos = torch.zeros(self.nvert, 3, dtype=torch.float32, device=self.device)
        gcol = torch.zeros(self.nvert, 3, dtype=torch.float32, device=self.device)
        gl = torch.zeros(3, dtype=torch.float32, device=self.device)
        self.batch.shade_backward(vrgb.data_ptr(), light.data_ptr(), grad_rgb.data_ptr(), gpos.data_ptr(),
                                  gcol.data_ptr(), gl.data_ptr())
        return gpos, gcol, gl

    def view_image(self, rgb: torch.Tensor, i: int) -> torch.Tensor:
        a, n = self.cells[i]
        return rgb[a:a + n]

    def close(self):
        self.batch.close()
        self.mesh.close()


class _ShadeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, vrgb, light, views: ShadedViews):
        vrgb_c = vrgb.detach().contiguous().to(torch.float32)
        light_c = light.detach().contiguous().to(torch.float32)
        views.render(pos)
        rgb = views.shade(vrgb_c, light_c)
        ctx.views = views
        ctx.save_for_backward(vrgb_c, light_c)
        return rgb

    @staticmethod
    def backward(ctx, grad_rgb):
        vrgb, light = ctx.saved_tensors
        gpos, gcol, gl = ctx.views.shade_backward(vrgb, light, grad_rgb.contiguous().to(torch.float32))
        return gpos, gcol, gl, None


def shade_views(pos: torch.Tensor, vrgb: torch.Tensor, light: torch.Tensor, views: ShadedViews) -> torch.Tensor:
    """Render `views` with vertex positions `pos` (nvert, 3) and shade them with vertex
    colours `vrgb` (nvert, 3) and light direction `light` (3,); differentiable in all
    three with the render's visibility held fixed."""
    return _ShadeFn.apply(pos, vrgb, light, views)


def uniform_laplacian(idx: np.ndarray, nvert: int, device) -> "callable":
    """p -> p - mean of p over each vertex's edge neighbours (the uniform mesh Laplacian),
    for a smoothness term sum(|L p|^2) on fitted positions."""
    f = np.asarray(idx, np.int64).reshape(-1, 3)
    e = np.unique(np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), 1), axis=0)
    src = torch.from_numpy(np.concatenate([e[:, 0], e[:, 1]])).to(device)
    dst = torch.from_numpy(np.concatenate([e[:, 1], e[:, 0]])).to(device)
    deg = torch.zeros(nvert, device=device).index_add_(0, src, torch.ones(src.numel(), device=device))
    inv = (1.0 / deg.clamp(min=1.0))[:, None]

    def lap(p: torch.Tensor) -> torch.Tensor:
        return p - torch.zeros_like(p).index_add_(0, src, p[dst]) * inv

    return lap

