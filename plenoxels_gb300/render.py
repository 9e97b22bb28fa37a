"""Fused render path: one kernel per pass over a batch of rays.

``render_rays`` is the whole of scripts/train.py:130-151 (ray samples -> normalisation
-> clamp -> nearest or trilinear lookup -> in-bounds mask -> compositing) as one
``torch.autograd.Function`` whose backward is the hand-written adjoint kernel.
``FusedTrainStep`` adds the MSE loss of scripts/train.py:156 and the backward of
:181 into the same launch, writing the dense grid gradient directly (no autograd graph),
optionally generating the rays in-kernel from cameras and images.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import PgbCameras, PgbRays, check, ptr, require_cuda, stream_of
from .grid_functions import grid_origin

MODES = {"nearest": _lib.PGB_NEAREST, "trilinear": _lib.PGB_TRILINEAR}


def _mode(mode) -> int:
    if mode not in MODES:
        raise ValueError(f"mode must be 'nearest' or 'trilinear', got {mode!r}")
    return MODES[mode]


TRANSMITTANCE = {"product": 0, "logsum": 1}


def _transmittance(name: str) -> int:
    if name not in TRANSMITTANCE:
        raise ValueError(f"transmittance must be 'product' or 'logsum', got {name!r}")
    return TRANSMITTANCE[name]


def _rays_desc(origins, dirs, num_rays, num_samples, delta_step, stratified, seed, term_threshold,
               cameras=None, background=None, log_t=0, chunk_samples=0, first_ray=0,
               grad_marks=None) -> PgbRays:
    r = PgbRays()
    r.origins = ptr(origins)
    r.dirs = ptr(dirs)
    r.cameras = ctypes.pointer(cameras) if cameras is not None else None
    r.num_rays = int(num_rays)
    r.num_samples = int(num_samples)
    r.delta_step = float(delta_step)
    r.stratified = 1 if stratified else 0
    r.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    r.term_threshold = float(term_threshold)
    if background is not None:
        r.use_background = 1
        r.background[:] = [float(v) for v in background]
    r.log_transmittance = int(log_t)
    r.chunk_samples = int(chunk_samples)
    r.first_ray = int(first_ray)
    r.grad_marks = ptr(grad_marks)
    return r


def _check_rays(grid, origins, dirs):
    real = _lib.real_dtype(grid.dtype)
    for name, t in (("origins", origins), ("dirs", dirs)):
        if t.dim() != 2 or t.shape[1] != 3:
            raise ValueError(f"{name} must be [R,3], got {tuple(t.shape)}")
        if t.dtype != real:
            raise TypeError(f"{name} must be {real} for a {grid.dtype} grid, got {t.dtype}")
    if origins.shape[0] != dirs.shape[0]:
        raise ValueError("origins and dirs must have the same number of rays")


class _RenderRays(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, origins, dirs, cfg):
        lib = _lib.load()
        R = origins.shape[0]
        rgba = torch.empty(R, 4, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
        gdesc = _lib.make_grid(grid, cfg["origin"], cfg["points_distance"], cfg["mode"], cfg["clip"])
        rdesc = _rays_desc(origins, dirs, R, cfg["num_samples"], cfg["delta_step"],
                           cfg["stratified"], cfg["seed"], cfg["term_threshold"],
                           background=cfg["background"], log_t=cfg["log_t"],
                           chunk_samples=cfg["chunk_samples"])
        check(lib.pgb_render_fwd(gdesc, rdesc, ptr(rgba), stream_of(grid)), "render_rays")
        ctx.save_for_backward(grid, origins, dirs)
        ctx.cfg = cfg
        return rgba

    @staticmethod
    def backward(ctx, d_rgba):
        grid, origins, dirs = ctx.saved_tensors
        cfg = ctx.cfg
        lib = _lib.load()
        s = stream_of(grid)
        grad = torch.empty(grid.shape, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
        check(lib.pgb_fill_zero(ptr(grad), grad.numel() * grad.element_size(), s), "backward")
        d_rgba = d_rgba.to(grad.dtype).contiguous()
        gdesc = _lib.make_grid(grid, cfg["origin"], cfg["points_distance"], cfg["mode"], cfg["clip"])
        rdesc = _rays_desc(origins, dirs, origins.shape[0], cfg["num_samples"], cfg["delta_step"],
                           cfg["stratified"], cfg["seed"], cfg["term_threshold"],
                           background=cfg["background"], log_t=cfg["log_t"],
                           chunk_samples=cfg["chunk_samples"])
        check(lib.pgb_render_bwd(gdesc, rdesc, ptr(d_rgba), ptr(grad), s), "render_rays backward")
        return grad, None, None, None


def render_rays(grid, origins, dirs, delta_step, num_samples, points_distance, grid_min=None,
                mode="trilinear", clip=True, stratified=False, seed=0, term_threshold=0.0,
                background=None, transmittance="product", chunk_samples=0):
    """Premultiplied RGBA [R,4] of rays through a dense [X,Y,Z,4] grid.

    Samples sit at origins + dirs * (delta_step * k), k = 1..num_samples (minus a
    per-sample jitter in [0,1) when stratified); grid_min is the world position of cell
    (0,0,0) (default: generate_grid's layout, grid_origin()). background (3 values, e.g. white)
    composites rgb over it: rgb + (1 - alpha) * background. transmittance "logsum" evaluates
    T = exp(compensated sum of log(1 - alpha)) instead of the reference's running product
    (fp32/BF16 grids, clip=True). chunk_samples (0: automatic; 32..512) sets how many
    samples of a ray are gathered between transmittance checks; it changes speed only.
    Differentiable in grid."""
    require_cuda(grid, origins, dirs)
    _check_rays(grid, origins, dirs)
    if grid_min is None:
        grid_min = grid_origin(grid.shape, points_distance, _lib.real_dtype(grid.dtype))
    cfg = dict(origin=tuple(float(x) for x in grid_min), points_distance=float(points_distance),
               mode=_mode(mode), clip=bool(clip), num_samples=int(num_samples),
               delta_step=float(delta_step), stratified=bool(stratified), seed=int(seed),
               term_threshold=float(term_threshold),
               background=None if background is None else tuple(float(v) for v in background),
               log_t=_transmittance(transmittance), chunk_samples=int(chunk_samples))
    return _RenderRays.apply(grid.contiguous(), origins.contiguous(), dirs.contiguous(), cfg)


def render_sample_indices(grid, origins, dirs, delta_step, num_samples, points_distance,
                          grid_min=None, mode="trilinear", stratified=False, seed=0):
    """The cell indices the fused kernels read, per sample: int64 [R,S,3] (nearest) or
    [R,S,8,3] (trilinear), wrapped, and the in-bounds flags [R,S]."""
    require_cuda(grid, origins, dirs)
    _check_rays(grid, origins, dirs)
    if grid_min is None:
        grid_min = grid_origin(grid.shape, points_distance, _lib.real_dtype(grid.dtype))
    R, S = origins.shape[0], int(num_samples)
    m = _mode(mode)
    shape = (R, S, 3) if m == _lib.PGB_NEAREST else (R, S, 8, 3)
    idx = torch.empty(shape, dtype=torch.int64, device=grid.device)
    inb = torch.empty(R, S, dtype=torch.bool, device=grid.device)
    gdesc = _lib.make_grid(grid.contiguous(), grid_min, points_distance, m, True)
    rdesc = _rays_desc(origins.contiguous(), dirs.contiguous(), R, S, delta_step, stratified, seed, 0.0)
    check(_lib.load().pgb_render_sample_indices(gdesc, rdesc, ptr(idx), ptr(inb), stream_of(grid)),
          "render_sample_indices")
    return idx, inb


def _camera_desc(transforms, images, camera_angle_x, ray_seed, near) -> PgbCameras:
    require_cuda(transforms, images)
    if transforms.dtype != torch.float32 or images.dtype != torch.float32:
        raise TypeError("transforms and images must be float32")
    if not (transforms.is_contiguous() and images.is_contiguous()):
        raise ValueError("transforms and images must be contiguous")
    if images.dim() != 4 or images.shape[-1] != 4 or transforms.shape[1:] != (4, 4):
        raise ValueError("transforms must be [C,4,4] and images [C,H,W,4]")
    cams = PgbCameras()
    cams.transforms = ptr(transforms)
    cams.images = ptr(images)
    cams.num_cameras = transforms.shape[0]
    cams.height, cams.width = images.shape[1], images.shape[2]
    cams.camera_angle_x = float(camera_angle_x)
    cams.near = float(near)
    cams.seed = int(ray_seed) & 0xFFFFFFFFFFFFFFFF
    return cams


def camera_sample_indices(grid, transforms, images, camera_angle_x, num_rays, ray_seed, near,
                          delta_step, num_samples, points_distance, grid_min=None,
                          mode="trilinear", stratified=False, seed=0, return_coords=False):
    """render_sample_indices for rays generated in-kernel from cameras (the rays
    FusedTrainStep.step_cameras uses for the same arguments). return_coords=True adds the
    samples' normalised coordinates [R,S,3] as a third result."""
    require_cuda(grid)
    if grid_min is None:
        grid_min = grid_origin(grid.shape, points_distance, _lib.real_dtype(grid.dtype))
    R, S = int(num_rays), int(num_samples)
    m = _mode(mode)
    shape = (R, S, 3) if m == _lib.PGB_NEAREST else (R, S, 8, 3)
    idx = torch.empty(shape, dtype=torch.int64, device=grid.device)
    inb = torch.empty(R, S, dtype=torch.bool, device=grid.device)
    cams = _camera_desc(transforms, images, camera_angle_x, ray_seed, near)
    gdesc = _lib.make_grid(grid.contiguous(), grid_min, points_distance, m, True)
    rdesc = _rays_desc(None, None, R, S, delta_step, stratified, seed, 0.0, cameras=cams)
    check(_lib.load().pgb_render_sample_indices(gdesc, rdesc, ptr(idx), ptr(inb), stream_of(grid)),
          "camera_sample_indices")
    if not return_coords:
        return idx, inb
    coords = torch.empty(R, S, 3, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
    check(_lib.load().pgb_render_sample_coords(gdesc, rdesc, ptr(coords), stream_of(grid)),
          "camera_sample_indices")
    return idx, inb, coords


class FusedTrainStep:
    """Forward, MSE loss and backward of a batch of rays in one kernel launch.

    beta > 0 adds the reference's beta loss on the sampled opacities (scripts/train.py:
    170-177) in the same launch; ``self.losses`` holds [weighted MSE, beta term].
    transmittance="logsum" selects the compensated log-sum transmittance (see render_rays).
    chunk_samples as in render_rays (speed only).

    The gradient goes to ``self.grad`` (fp32 for fp32/bf16 grids, fp64 for fp64 grids),
    which is also attached as ``grid.grad`` when the dtypes agree, so a torch optimizer
    can step on it. Each call zeroes the gradient first (optimizer.zero_grad semantics)
    unless zero_grad=False, in which case it accumulates like autograd does. Every call
    is asynchronous; the returned loss is a device scalar.

    overlap_zero=True keeps two gradient buffers and zeroes the next step's buffer on a
    side stream while the current step's kernel runs (the 256 MiB fill of a 256^3 grid
    no longer sits on the critical path). A step's gradient then stays valid until the
    next step is launched; the buffer alternates, and ``grid.grad``/``self.grad`` follow.

    zeroing="marked" re-zeroes a gradient buffer by clearing only the 4-cell units its
    last step wrote (the kernel marks them in a bitmap of the buffer, pgb_clear_marked)
    instead of writing the whole buffer. Every step still starts from an all-zero dense
    gradient, provided the caller only reads the gradient buffers (an optimizer that
    reads grid.grad, or zeroes it) and does not add into them; an in-place all-reduce of
    the gradient over ranks adds into them.
    """

    def __init__(self, grid, points_distance, num_samples, delta_step, mode="trilinear",
                 grid_min=None, clip=True, stratified=False, seed=0, term_threshold=0.0,
                 loss_weight=1.0, overlap_zero=False, beta=0.0, beta_eps=1e-4, background=None,
                 transmittance="product", chunk_samples=0, zeroing="fill"):
        require_cuda(grid)
        if grid.dim() != 4 or grid.shape[-1] != 4 or not grid.is_contiguous():
            raise ValueError("grid must be a contiguous [X,Y,Z,4] tensor")
        self.grid = grid
        self.real = _lib.real_dtype(grid.dtype)
        self.points_distance = float(points_distance)
        self.grid_min = tuple(grid_min) if grid_min is not None else grid_origin(
            grid.shape, points_distance, self.real)
        self.num_samples = int(num_samples)
        self.delta_step = float(delta_step)
        self.mode = _mode(mode)
        self.clip = bool(clip)
        self.stratified = bool(stratified)
        self.seed = int(seed)
        self.term_threshold = float(term_threshold)
        self.loss_weight = float(loss_weight)
        self.beta = float(beta)
        self.beta_eps = float(beta_eps)
        self.background = None if background is None else tuple(float(v) for v in background)
        self.log_t = _transmittance(transmittance)
        self.chunk_samples = int(chunk_samples)
        lib = _lib.load()
        dev = grid.device
        self.workspace = torch.zeros(lib.pgb_train_workspace_bytes(), dtype=torch.uint8, device=dev)
        self._grads = [torch.zeros(grid.shape, dtype=self.real, device=dev)]
        self._side = None
        if overlap_zero:
            self._grads.append(torch.zeros(grid.shape, dtype=self.real, device=dev))
            self._side = torch.cuda.Stream(device=dev)
            self._zeroed = [None, None]  # event: buffer b is zero and free
        if zeroing not in ("fill", "marked"):
            raise ValueError(f"zeroing must be 'fill' or 'marked', got {zeroing!r}")
        cells = grid.numel() // 4
        self._marks = ([torch.zeros(lib.pgb_mark_words(cells), dtype=torch.int32, device=dev)
                        for _ in self._grads] if zeroing == "marked" else None)
        self._cur = 0
        self._buf = 0  # index of the buffer the last launch wrote
        self.grad = self._grads[0]
        # losses[0]: loss_weight * MSE; losses[1]: the beta term (scripts/train.py:170-177)
        self.losses = torch.zeros(2, dtype=self.real, device=dev)
        self.loss = self.losses[0]
        self._attach()
        self._cams = None
        self.kernel_events = None  # list of (start, end) CUDA events, when timing is wanted

    def _attach(self):
        if self.grid.dtype == self.real and self.grid.requires_grad:
            self.grid.grad = self.grad

    def _fill(self, b, stream):
        buf = self._grads[b]
        lib = _lib.load()
        if self._marks is None:
            check(lib.pgb_fill_zero(ptr(buf), buf.numel() * buf.element_size(), stream.cuda_stream),
                  "train step")
        else:
            check(lib.pgb_clear_marked(ptr(buf), 4 * buf.element_size(), buf.numel() // 4,
                                       ptr(self._marks[b]), stream.cuda_stream), "train step")

    def _gradient_for_step(self, zero_grad):
        main = torch.cuda.current_stream(self.grid.device)
        if not zero_grad:
            return self.grad
        if self._side is None:
            self._fill(0, main)
            self._buf = 0
            return self.grad
        b = self._cur
        buf = self._grads[b]
        self._buf = b
        if self._zeroed[b] is None:
            self._fill(b, main)
        else:
            main.wait_event(self._zeroed[b])
        # zero the other buffer for the next step, after everything already queued on the
        # main stream (its last reader, e.g. the optimizer step of the previous step)
        o = 1 - b
        ready = torch.cuda.Event()
        ready.record(main)
        self._side.wait_event(ready)
        self._fill(o, self._side)
        done = torch.cuda.Event()
        done.record(self._side)
        self._zeroed[o] = done
        self._cur = o
        self.grad = buf
        self._attach()
        return buf

    def _loss_target(self, loss_out):
        """Where the step writes [weighted MSE, beta term]: self.losses, or loss_out, a
        contiguous tensor of at least two elements of the step's dtype on this GPU or in
        pinned host memory. Pinned host memory is addressable by the GPU under unified
        addressing, so the kernel writes the loss there itself: the result reaches the
        host without a separate copy."""
        if loss_out is None:
            return self.losses
        if loss_out.dtype != self.real or loss_out.numel() < 2 or not loss_out.is_contiguous():
            raise ValueError(f"loss_out must be a contiguous {self.real} tensor of >= 2 elements")
        if not (loss_out.is_cuda and loss_out.device == self.grid.device) and not (
                loss_out.device.type == "cpu" and loss_out.is_pinned()):
            raise ValueError("loss_out must be on the grid's GPU or in pinned host memory")
        return loss_out

    def _launch(self, rdesc, target, rgba_out, zero_grad, loss_out=None):
        lib = _lib.load()
        losses = self._loss_target(loss_out)
        grad = self._gradient_for_step(zero_grad)
        if self._marks is not None:
            rdesc.grad_marks = ptr(self._marks[self._buf])
        stream = torch.cuda.current_stream(self.grid.device)
        gdesc = _lib.make_grid(self.grid, self.grid_min, self.points_distance, self.mode, self.clip)
        ev = None
        if self.kernel_events is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record(stream)
        if self.beta == 0.0:
            check(lib.pgb_render_train(gdesc, rdesc, ptr(target), self.loss_weight, ptr(rgba_out),
                                       ptr(grad), ptr(losses), ptr(self.workspace),
                                       stream.cuda_stream), "train step")
        else:
            terms = _lib.PgbLossTerms(self.loss_weight, self.beta, self.beta_eps)
            check(lib.pgb_render_train_terms(gdesc, rdesc, ptr(target), terms, ptr(rgba_out),
                                             ptr(grad), ptr(losses), ptr(self.workspace),
                                             stream.cuda_stream), "train step")
        if ev is not None:
            ev[1].record(stream)
            self.kernel_events.append(ev)
        return self.loss if loss_out is None else loss_out[0]

    def step_rays(self, origins, dirs, target, rgba_out=None, zero_grad=True, first_ray=0,
                  loss_out=None):
        """Explicit rays [R,3] and their target pixels [R,4]. first_ray: index of the first
        of these rays in the stratification stream, for ranks that each take a share of
        one batch (distributed.shard_rays) and must sample it as the whole batch would.
        loss_out: where the losses go instead of self.losses (see _loss_target), e.g. a
        pinned host buffer, so that reading a step's loss on the host needs no copy."""
        require_cuda(origins, dirs, target)
        _check_rays(self.grid, origins, dirs)
        if target.shape != (origins.shape[0], 4) or target.dtype != self.real:
            raise ValueError(f"target must be [R,4] {self.real}")
        rdesc = _rays_desc(origins, dirs, origins.shape[0], self.num_samples, self.delta_step,
                           self.stratified, self.seed, self.term_threshold, background=self.background,
                           log_t=self.log_t, chunk_samples=self.chunk_samples, first_ray=first_ray)
        return self._launch(rdesc, target.contiguous(), rgba_out, zero_grad, loss_out)

    def step_cameras(self, transforms, images, camera_angle_x, num_rays, ray_seed, near=0.0,
                     rgba_out=None, zero_grad=True, loss_out=None):
        """Rays generated in-kernel: num_rays spread camera-major over the cameras, pixel
        positions from the counter hash of ray_seed, origins moved `near` along each ray;
        targets are the sampled pixels of images [C,H,W,4]."""
        cams = _camera_desc(transforms, images, camera_angle_x, ray_seed, near)
        self._cams = cams  # keep alive for the call
        rdesc = _rays_desc(None, None, num_rays, self.num_samples, self.delta_step, self.stratified,
                           self.seed, self.term_threshold, cameras=cams, background=self.background,
                           log_t=self.log_t, chunk_samples=self.chunk_samples)
        return self._launch(rdesc, None, rgba_out, zero_grad, loss_out)
