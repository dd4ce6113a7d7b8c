"""Serving: resident scenes, continuous batching of render requests.

Not part of the reference (whose viewer renders one request at a time under
a lock, viewer/viewer.py:53). Several scenes stay on the device: their voxel
grids, signed distances and SH, and the tessellated mesh used by render-only
requests. Requests arrive over time, each for one scene with its own camera
and image size, either render-only or render + gradient of an MSE loss
against a target image.

``Server.run`` is the continuous-batching loop. At every turn it

* admits the requests that have arrived into a FIFO queue;
* retires finished batches (a CUDA event per batch, polled without blocking)
  and stamps their requests' completion times;
* while a stream slot and the in-flight memory budget allow, and either
  nothing is in flight or requests have queued up (``overlap_backlog``;
  overlapping batches slow each other, which only pays when requests wait),
  forms the next batch from the head of the queue: render-only requests of
  the head's scene
  (in arrival order, up to ``max_batch`` and a pixel budget) go into one
  ``render_cameras`` call for cameras of any size; a gradient request runs
  on its own (its gradient is with respect to the scene's parameters, so it
  cannot share a loss with other requests);
* launches the batch on its own CUDA stream, so batches overlap on the GPU.

``run_plain`` is the per-request form at the same arrival times: one request
at a time, rendered and completed before the next starts.

Every request's result is the same alone and in a batch: a camera rendered
in ``render_cameras`` equals its ``render_fused`` image bit for bit, and a
gradient request is computed alone either way (tests/test_serving_gpu.py).
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

    def tessellate(self, grid_sdf: Tensor, grid_sh: Tensor):
        v = self.voxels
        tri = te.tessellate_voxels(grid_sdf, v.vertices, grid_sh, v.neighbors, v.lower_corners, v.upper_corners,
                                   v.indices, self.level_sets)
        return pipeline.uncontract_stand_in(tri.vertices).detach(), tri

    def refresh_mesh(self) -> None:
        """Re-tessellates the cached mesh (after the scene's parameters change)."""
        with torch.no_grad():
            vertices, tri = self.tessellate(self.grid_sdf, self.grid_sh)
        self.mesh = (vertices, tri.faces, tri.face_boundaries, tri.signed_distances, tri.spherical_harmonics)


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
    pixels: int


@dataclass
class Server:
    scenes: list[Scene]
    streams: int = 4  # batches in flight at once
    max_batch: int = 16  # requests per render batch
    max_pixels: int = 16 * 1920 * 1080  # in-flight pixel budget (bounds the HBM in use)
    overlap_backlog: int = 2  # queued requests needed to start a batch while another is in flight
    tile_shape: tuple[int, int] = (16, 16)
    batches: int = field(default=0, init=False)

    def _form_batch(self, queue: deque, budget: int) -> list[Request]:
        head = queue[0]
        if head.gradient:
            return [queue.popleft()] if head.pixels <= budget or budget == self.max_pixels else []
        batch, pixels, keep = [], 0, deque()
        while queue and len(batch) < self.max_batch:
            r = queue.popleft()
            if r.scene == head.scene and not r.gradient and (pixels + r.pixels <= budget or not batch):
                batch.append(r)
                pixels += r.pixels
            else:
                keep.append(r)
                if len(keep) > 4 * self.max_batch:  # look ahead a bounded distance
                    break
        queue.extendleft(reversed(keep))
        if pixels > budget and budget < self.max_pixels:  # head alone does not fit yet
            queue.extendleft(reversed(batch))
            return []
        return batch

    def run(self, requests: list[Request]) -> list[Completed]:
        """Serves ``requests`` (sorted by arrival) in real time; returns them
        completed, with completion times, in completion order."""
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
                    done.extend(f.results)
                    free.append(f.stream)
                else:
                    still.append(f)
            inflight = still
            launched = False
            while queue and free:
                if inflight and len(queue) < self.overlap_backlog:
                    break
                budget = self.max_pixels - sum(f.pixels for f in inflight)
                batch = self._form_batch(queue, budget)
                if not batch:
                    break
                stream = free.pop()
                with torch.cuda.stream(stream):
                    scene = self.scenes[batch[0].scene]
                    results = (render_batch(scene, batch, self.tile_shape) if not batch[0].gradient
                               else [render_alone(scene, batch[0], self.tile_shape)])
                    event = torch.cuda.Event()
                    event.record(stream)
                inflight.append(_InFlight(results, event, stream, sum(r.pixels for r in batch)))
                self.batches += 1
                launched = True
            if not launched and not inflight and pending and not queue:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - start), 0.001)))
        return done


def run_plain(scenes: list[Scene], requests: list[Request], tile_shape=(16, 16)) -> list[Completed]:
    """The per-request form at the same arrival times: each request rendered
    and completed before the next one starts."""
    done = []
    start = time.perf_counter()
    for r in requests:
        wait = r.arrival - (time.perf_counter() - start)
        if wait > 0:
            time.sleep(wait)
        c = render_alone(scenes[r.scene], r, tile_shape)
        torch.cuda.synchronize()
        c.done = time.perf_counter() - start
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
