"""Serving: resident scenes, continuous batching of render requests.

Not part of the reference (whose viewer renders one request at a time under
a lock, viewer/viewer.py:53). Several scenes stay on the device: their voxel
grids, signed distances and SH, and their tessellated mesh, kept with its
autograd graph as a function of the grid parameters (render-only requests
read it detached; render + gradient requests back-propagate through it
without tessellating again). Requests arrive over time, each for one scene
with its own camera and image size, either render-only or render + gradient
of an MSE loss against a target image.

``Server.run`` is the continuous-batching loop. At every turn it

* admits the requests that have arrived into a FIFO queue;
* retires finished batches (a CUDA event per batch, polled without blocking)
  and stamps their requests' completion times;
* while a stream slot is free and the estimated device bytes of the batches
  in flight leave room (``hbm_budget``; ``Scene.request_bytes`` estimates a
  request from its pixels, its scene's tile keys per pixel and, for a
  gradient request, the tessellation and gradient buffers), forms the next
  batch from the head of the queue: render-only requests of the head's scene
  (in arrival order, up to ``max_batch``) go into one ``render_cameras`` call
  for cameras of any size; render + gradient requests of the head's scene
  (up to ``max_gradient_batch``) render from the resident tessellation and
  each get the gradient of their own loss; a batch starts while another is in
  flight once
  ``overlap_backlog`` requests wait;
* launches the batch on its own CUDA stream, so batches overlap on the GPU.

``run_plain`` is the per-request form at the same arrival times: one request
at a time, rendered and completed before the next starts; a render +
gradient request tessellates the scene's parameters itself, as a training
step does.

Every request's result is the same alone and in a batch: a camera rendered
in ``render_cameras`` equals its ``render_fused`` image bit for bit, and a
gradient request's loss and gradient involve its own camera only (the
resident tessellation equals a fresh one: it is deterministic)
(tests/test_serving_gpu.py).
"""

from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch
from torch import Tensor

from . import pipeline, synthetic
from . import triangle_extraction as te
from . import triangle_rasterization as tr


@dataclass
class Scene:
    name: str
    voxels: te.Voxels
    grid_sdf: Tensor  # [G]
    grid_sh: Tensor  # [C, G, 3]
    level_sets: Tensor  # [S]
    sh_degree: int
    sharpness: Tensor  # []
    background: Tensor  # [3]
    mesh: tuple = ()  # (vertices, faces, shell face boundaries, sdf, sh) for render-only requests
    # (grid sdf leaf, grid sh leaf, vertices, triangles): the resident
    # tessellation as a function of the grid parameters, its autograd graph
    # kept for the render + gradient requests.
    grad_mesh: tuple = ()
    # Tessellated [0, 1]^3 vertices -> renderer positions (None: the 2 v - 1
    # stand-in of the synthetic scenes; a checkpoint scene uses its
    # contraction's inverse, as the reference's model does).
    vertex_map: object = None

    @staticmethod
    def build(config: str, device, seed: int = 0) -> "Scene":
        cfg = synthetic.CONFIGS[config]
        voxels = te.extract_voxels(synthetic.make_occupancy(cfg, device))
        sdf = synthetic.corner_sdf(cfg, voxels.vertices)
        if seed:
            sdf = sdf + torch.from_numpy(np.random.default_rng(seed).normal(
                0.0, cfg.noise_sigma, sdf.shape[0]).astype(np.float32)).to(device)
        scene = Scene(config, voxels, sdf.contiguous(), synthetic.corner_sh(cfg, sdf.shape[0], device),
                      synthetic.level_sets(cfg, device), cfg.sh_degree,
                      torch.tensor(cfg.sharpness, dtype=torch.float32, device=device),
                      torch.zeros(3, dtype=torch.float32, device=device))
        scene.refresh_mesh()
        return scene

    @staticmethod
    def from_checkpoint(path, layout, contraction, level_sets: Tensor, device, name: str | None = None,
                        sdf_offset=None, sharpness: float = 400.0) -> "Scene":
        """A resident scene from a reference trainer checkpoint
        (meshtryoshka_gb300.checkpoint): its tesseract voxels, signed
        distances and SH; positions through ``contraction.uncontract``."""
        from . import checkpoint

        loaded = checkpoint.load_tesseract_checkpoint(path, layout, device, sdf_offset)
        scene = Scene(name or str(path), loaded.voxels, loaded.signed_distances, loaded.spherical_harmonics,
                      level_sets.to(device=device, dtype=torch.float32).contiguous(), loaded.sh_degree,
                      torch.tensor(sharpness, dtype=torch.float32, device=device),
                      torch.zeros(3, dtype=torch.float32, device=device), vertex_map=contraction.uncontract)
        scene.refresh_mesh()
        return scene

    def tessellate(self, grid_sdf: Tensor, grid_sh: Tensor):
        v = self.voxels
        tri = te.tessellate_voxels(grid_sdf, v.vertices, grid_sh, v.neighbors, v.lower_corners, v.upper_corners,
                                   v.indices, self.level_sets)
        positions = self.vertex_map(tri.vertices) if self.vertex_map is not None else \
            pipeline.uncontract_stand_in(tri.vertices)
        return positions.detach().contiguous(), tri

    def refresh_mesh(self) -> None:
        """Re-tessellates the resident mesh (after the scene's parameters
        change). The tessellation is kept as a function of the grid
        parameters, its autograd graph retained, so that render + gradient
        requests back-propagate through it without tessellating again;
        render-only requests read its detached outputs."""
        sdf = self.grid_sdf.detach().requires_grad_(True)
        sh = self.grid_sh.detach().requires_grad_(True)
        with torch.enable_grad():
            vertices, tri = self.tessellate(sdf, sh)
        self.grad_mesh = (sdf, sh, vertices, tri)
        self.mesh = (vertices, tri.faces, tri.face_boundaries, tri.signed_distances.detach(),
                     tri.spherical_harmonics.detach())
        self.keys_per_pixel = None

    def measure_keys_per_pixel(self, shape=(512, 512)) -> float:
        """Tile keys per pixel of a render of this scene (a probe from the
        first request camera direction the scene's layout uses), for the
        server's memory estimates."""
        if getattr(self, "keys_per_pixel", None) is None:
            eye = np.array([0.0, 0.1, 0.6 if self._inside() else 2.2])
            ext = torch.from_numpy(synthetic.look_at(eye)[None]).to(self.grid_sdf.device)
            intr = torch.from_numpy(synthetic.pinhole(shape[0], shape[1], 55.0)[None]).to(self.grid_sdf.device)
            with torch.no_grad():
                tr.render_fused(ext, intr, shape, *self.mesh, self.sh_degree, self.sharpness, self.background)
            self.keys_per_pixel = max(tr.LAST_RENDER_STATS.get("num_keys", 0) / float(shape[0] * shape[1]), 1.0)
        return self.keys_per_pixel

    def _inside(self) -> bool:
        cfg = synthetic.CONFIGS.get(self.name)
        return cfg is not None and cfg.background_radius is not None

    def request_bytes(self, r: "Request") -> int:
        """Estimated device bytes a request holds while in flight: the
        compositing output and image (28 B per pixel), its tile keys (sort
        buffers and masks, 40 B per key), and for a gradient request also the
        backward's tessellation-sized buffers (gradients of the vertices,
        signed distances and SH rows, counted at the size of the tessellation
        itself, which is resident), the grid gradients, the target and the
        hit-bit store (16 B per pixel)."""
        kpp = self.measure_keys_per_pixel()
        p = r.pixels
        total = 28 * p + int(40 * kpp * p)
        if r.gradient:
            v = self.mesh[0].shape[0]
            f = self.mesh[1].shape[0]
            c = self.grid_sh.shape[0]
            g = self.grid_sdf.shape[0]
            total += v * (12 + 4 + 12 * c + 1 + 12) + f * 16 + g * (4 + 12 * c) + v * 24 + (12 + 16) * p
        return total


@dataclass
class Request:
    id: int
    scene: int
    extrinsics: Tensor  # [4, 4] (device)
    intrinsics: Tensor  # [3, 3]
    shape: tuple[int, int]  # (H, W)
    gradient: bool
    target: Tensor | None  # [3, H, W] for gradient requests
    arrival: float  # seconds after the start of the run

    @property
    def pixels(self) -> int:
        return self.shape[0] * self.shape[1]


@dataclass
class Completed:
    request: Request
    image: Tensor  # [3, H, W]
    grad_sdf: Tensor | None = None
    grad_sh: Tensor | None = None
    done: float = 0.0

    @property
    def latency(self) -> float:
        return self.done - self.request.arrival


def render_alone(scene: Scene, r: Request, tile_shape=(16, 16)) -> Completed:
    """One request on its own (the plain per-request computation)."""
    if not r.gradient:
        with torch.no_grad():
            image = tr.render_fused(r.extrinsics[None], r.intrinsics[None], r.shape, *scene.mesh, scene.sh_degree,
                                    scene.sharpness, scene.background, tile_shape=tile_shape)[0]
        return Completed(r, image)
    sdf = scene.grid_sdf.detach().requires_grad_(True)
    sh = scene.grid_sh.detach().requires_grad_(True)
    vertices, tri = scene.tessellate(sdf, sh)
    image = tr.render_fused(r.extrinsics[None], r.intrinsics[None], r.shape, vertices, tri.faces,
                            tri.face_boundaries, tri.signed_distances, tri.spherical_harmonics, scene.sh_degree,
                            scene.sharpness, scene.background, tile_shape=tile_shape)[0]
    loss = ((image - r.target) ** 2).mean()
    grad_sdf, grad_sh = torch.autograd.grad(loss, (sdf, sh))
    return Completed(r, image.detach(), grad_sdf, grad_sh)


def render_gradient_batch(scene: Scene, batch: list[Request], tile_shape=(16, 16)) -> list[Completed]:
    """Render + gradient requests of one scene over its resident
    tessellation (``Scene.grad_mesh``, built once per parameter state): per
    request its render, its MSE and the gradient of that loss alone, back
    through the retained tessellation graph (the same results as each
    request alone, which tessellates again: the tessellation is
    deterministic)."""
    sdf, sh, vertices, tri = scene.grad_mesh
    out = []
    for r in batch:
        image = tr.render_fused(r.extrinsics[None], r.intrinsics[None], r.shape, vertices, tri.faces,
                                tri.face_boundaries, tri.signed_distances, tri.spherical_harmonics, scene.sh_degree,
                                scene.sharpness, scene.background, tile_shape=tile_shape)[0]
        loss = ((image - r.target) ** 2).mean()
        grad_sdf, grad_sh = torch.autograd.grad(loss, (sdf, sh), retain_graph=True)  # keep the tessellation's graph
        out.append(Completed(r, image.detach(), grad_sdf, grad_sh))
    return out


def render_batch(scene: Scene, batch: list[Request], tile_shape=(16, 16)) -> list[Completed]:
    """Render-only requests of one scene in one pass over cameras of any size."""
    if len(batch) == 1:
        return [render_alone(scene, batch[0], tile_shape)]
    ext = torch.stack([r.extrinsics for r in batch])
    intr = torch.stack([r.intrinsics for r in batch])
    with torch.no_grad():
        images = tr.render_cameras(ext, intr, [r.shape for r in batch], *scene.mesh, scene.sh_degree,
                                   scene.sharpness, scene.background, tile_shape=tile_shape)
    return [Completed(r, img) for r, img in zip(batch, images)]


@dataclass
class _InFlight:
    results: list[Completed]
    event: torch.cuda.Event
    stream: torch.cuda.Stream
    bytes: int


@dataclass
class Server:
    scenes: list[Scene]
    streams: int = 4  # batches in flight at once
    max_batch: int = 16  # requests per render batch
    max_gradient_batch: int = 4  # render + gradient requests per batch
    hbm_budget: int = 8 << 30  # estimated device bytes of the batches in flight (Scene.request_bytes)
    overlap_backlog: int = 1  # queued requests needed to start a batch while another is in flight
    tile_shape: tuple[int, int] = (8, 8)  # the render path's fastest tile here (images do not depend on it)
    batches: int = field(default=0, init=False)
    peak_inflight_bytes: int = field(default=0, init=False)

    def __post_init__(self):
        for scene in self.scenes:  # the per-scene key density of the byte estimates, measured up front
            scene.measure_keys_per_pixel()

    def _bytes(self, r: Request) -> int:
        return self.scenes[r.scene].request_bytes(r)

    def _form_batch(self, queue: deque, budget: int, idle: bool) -> tuple[list[Request], int]:
        """The next batch from the head of the queue: requests of the head's
        scene and kind (render-only, or render + gradient), in arrival order,
        while their estimated bytes fit ``budget``. With nothing in flight
        (``idle``) the head goes alone even if it exceeds the budget."""
        head = queue[0]
        limit = self.max_gradient_batch if head.gradient else self.max_batch
        batch, used, keep = [], 0, deque()
        while queue and len(batch) < limit:
            r = queue.popleft()
            b = self._bytes(r)
            if r.scene == head.scene and r.gradient == head.gradient and (used + b <= budget or (not batch and idle)):
                batch.append(r)
                used += b
            else:
                keep.append(r)
                if len(keep) > 4 * self.max_batch or not batch:  # look ahead a bounded distance
                    break
        queue.extendleft(reversed(keep))
        if not batch:
            return [], 0
        return batch, used

    def run(self, requests: list[Request], keep_results: bool = True) -> list[Completed]:
        """Serves ``requests`` (sorted by arrival) in real time; returns them
        completed, with completion times, in completion order. With
        ``keep_results`` False a request's image and gradients are released
        once it completes (delivered to a client that needs only its timing),
        so that a long run does not hold every response on the device."""
        device = self.scenes[0].grid_sdf.device
        pool = [torch.cuda.Stream(device) for _ in range(self.streams)]
        for s in pool:
            s.wait_stream(torch.cuda.current_stream(device))
        free = list(pool)
        pending = deque(requests)
        queue: deque = deque()
        inflight: list[_InFlight] = []
        done: list[Completed] = []
        start = time.perf_counter()
        while pending or queue or inflight:
            now = time.perf_counter() - start
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            still = []
            for f in inflight:
                if f.event.query():
                    t = time.perf_counter() - start
                    for c in f.results:
                        c.done = t
                        if not keep_results:
                            c.image = c.grad_sdf = c.grad_sh = None
                    done.extend(f.results)
                    free.append(f.stream)
                else:
                    still.append(f)
            inflight = still
            launched = False
            while queue and free:
                if inflight and len(queue) < self.overlap_backlog:
                    break
                held = sum(f.bytes for f in inflight)
                batch, used = self._form_batch(queue, self.hbm_budget - held, not inflight)
                if not batch:
                    break
                stream = free.pop()
                with torch.cuda.stream(stream):
                    scene = self.scenes[batch[0].scene]
                    results = (render_batch(scene, batch, self.tile_shape) if not batch[0].gradient
                               else render_gradient_batch(scene, batch, self.tile_shape))
                    event = torch.cuda.Event()
                    event.record(stream)
                inflight.append(_InFlight(results, event, stream, used))
                self.peak_inflight_bytes = max(self.peak_inflight_bytes, held + used)
                self.batches += 1
                launched = True
            if not launched and not inflight and pending and not queue:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - start), 0.001)))
        return done


def run_plain(scenes: list[Scene], requests: list[Request], tile_shape=(16, 16),
              keep_results: bool = True) -> list[Completed]:
    """The per-request form at the same arrival times: each request rendered
    and completed before the next one starts (``keep_results`` as in
    ``Server.run``)."""
    done = []
    start = time.perf_counter()
    for r in requests:
        wait = r.arrival - (time.perf_counter() - start)
        if wait > 0:
            time.sleep(wait)
        c = render_alone(scenes[r.scene], r, tile_shape)
        torch.cuda.synchronize()
        c.done = time.perf_counter() - start
        if not keep_results:
            c.image = c.grad_sdf = c.grad_sh = None
        done.append(c)
    return done


def poisson_requests(scenes: list[Scene], rate: float, duration: float, seed: int = 4,
                     gradient_fraction: float = 0.2, first_id: int = 0) -> list[Request]:
    """Poisson arrivals at ``rate`` requests/s for ``duration`` s: uniform
    scene, camera looking at the origin from a random direction (2-2.5 units
    away; 0.5-0.7 units, near the horizontal plane, inside a scene's
    background sphere), image width U{256..1920} x height U{256..1080}, fov
    U[40, 70] degrees; a ``gradient_fraction`` of the requests also asks for
    the gradient of the MSE against a U[0, 1] target."""
    rng = np.random.default_rng(seed)
    device = scenes[0].grid_sdf.device
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        scene = int(rng.integers(len(scenes)))
        direction = rng.normal(size=3)
        if synthetic.CONFIGS[scenes[scene].name].background_radius is not None:
            # Inside the background sphere: a ring of radius 0.5-0.7 around
            # the origin, near the horizontal plane.
            direction[1] *= 0.2
            direction /= np.linalg.norm(direction)
            eye = direction * rng.uniform(0.5, 0.7)
        else:
            direction /= np.linalg.norm(direction)
            eye = direction * rng.uniform(2.0, 2.5)
        w, h = int(rng.integers(256, 1921)), int(rng.integers(256, 1081))
        fov = float(rng.uniform(40.0, 70.0))
        grad = bool(rng.random() < gradient_fraction)
        target = None
        if grad:
            target = torch.rand((3, h, w), generator=gen, device=device)
        out.append(Request(first_id + len(out), scene,
                           torch.from_numpy(synthetic.look_at(eye)).to(device),
                           torch.from_numpy(synthetic.pinhole(h, w, fov)).to(device), (h, w), grad, target, t))
    return out


def latency_summary(done: list[Completed]) -> dict:
    lat = np.array([c.latency for c in done]) * 1000.0
    if lat.size == 0:
        return {"requests": 0}
    span = max(c.done for c in done) - min(c.request.arrival for c in done)
    return {"requests": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "throughput_rps": float(lat.size / span) if span > 0 else math.inf}


def default_scenes(device) -> list[Scene]:
    """Two 256^3 scenes of the mid layout (8 spheres, different noise), one at
    128^3, and one 512^3 scene of the large layout (32 spheres inside a
    background sphere); SH degree 3 and 8 shells each."""
    return [Scene.build("serve_256", device, seed=0), Scene.build("serve_256", device, seed=7),
            Scene.build("serve_128", device), Scene.build("serve_512", device)]
