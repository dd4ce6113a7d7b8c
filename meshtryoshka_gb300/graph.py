"""The fused training step captured as one CUDA graph.

The eager step reads sizes back to the host twice (the vertex / face totals
after the marching-cubes counts and the key total after the tile counts),
and each of its ~30 library kernels and ~40 tensor ops is launched from
Python. The captured step instead allocates its vertex, face and key buffers
once, at capacities (the sizes of a first eager step times a margin), keeps
the live sizes on the device, and replays tessellation, render, loss and the
whole backward as a single graph: no host synchronisation and no per-launch
host cost.

A live size above its capacity drops the excess (every kernel stays inside
its buffers: writers are capacity-guarded and faces naming a dropped vertex
cover no tile) and sets an overflow flag on the device. ``check()`` reads the
flag; on overflow it re-captures with larger capacities and the step has to
be run again.

The graph reads the workload's parameters (``grid_sdf``, ``grid_sh``) and
target in place; after each replay ``grid_sdf.grad`` / ``grid_sh.grad`` are
the step's gradients (tensors owned by the graph, overwritten by every
replay, never accumulated), so a trainer updates the parameters in place
between replays.
"""

from __future__ import annotations

import dataclasses

import torch
from torch import Tensor

from . import _native as nt
from . import pipeline
from . import triangle_rasterization as tr
from .record import recording


# The tensors a graph reads in place: the parameters, and the per-step data
# (the batch a training loop feeds every step).
PARAMETERS = ("grid_sdf", "grid_sh")
DATA = ("target", "extrinsics", "intrinsics")
INPUTS = PARAMETERS + DATA


class CapturedTrainingStep:
    """Fused forward + backward of ``pipeline.Workload`` as one CUDA graph.

    ``input_sets`` > 1 captures one graph per set of per-step data (``DATA``:
    target and cameras): set 0 is the workload's own tensors, the others are
    device copies (``self.inputs[i]``), and ``step(i)`` replays the graph that
    reads set i in place. The parameters are shared by every set (each graph
    reads the workload's parameters in place). A host pipeline can then copy
    the next step's batch into one set while the other set's graph runs, with
    no device-side copy between them. Each graph has its own memory pool, so
    the outputs of one set's replay stay valid across replays of the
    others."""

    def __init__(self, workload: pipeline.Workload, gradient_mode: str | None = None, margin: float = 1.25,
                 capacities: pipeline.Capacities | None = None, warmup: int = 2, input_sets: int = 1,
                 record: bool = False):
        self.w = workload
        # record: keep references to each graph's intermediate buffers
        # (meshtryoshka_gb300.record) in self.records[set].
        self.record = record
        self.records: list[dict] = []
        self.gradient_mode = gradient_mode
        self.margin = margin
        self.warmup = warmup
        self.inputs = [{k: getattr(workload, k) for k in INPUTS}]
        for _ in range(1, max(int(input_sets), 1)):
            data = {k: getattr(workload, k).detach().clone() for k in DATA}
            self.inputs.append({**{k: getattr(workload, k) for k in PARAMETERS}, **data})
        self._views = [dataclasses.replace(workload, **{k: v for k, v in s.items()}) for s in self.inputs]
        if capacities is None:
            capacities = pipeline.Capacities.around(self._measure(), margin)
        self.capacities = capacities
        self.recaptures = 0
        self._capture()

    def _measure(self) -> dict:
        """Live sizes of one eager forward per input set (no autograd graph is
        kept), the largest of each over the sets: the key count depends on
        each set's cameras."""
        stats = None
        with torch.no_grad():
            for view in self._views:
                _, st = pipeline.forward(view, "fused", self.gradient_mode)
                stats = st if stats is None else {k: max(stats[k], st[k]) for k in st}
        return stats

    def _step(self, slot: int = 0) -> tuple[Tensor, Tensor, Tensor, Tensor]:
        # The graph differentiates with respect to aliases of the parameters
        # (same storage, fresh autograd leaves made on the capture stream) and
        # returns the gradients instead of accumulating them: autograd state
        # left on the parameters by eager steps on another stream would
        # otherwise make the capture wait on that stream.
        loss, overflow = pipeline.forward_counted(self._views[slot], self.capacities, self.gradient_mode,
                                                  self._sdf[slot], self._sh[slot])
        grad_sdf, grad_sh = torch.autograd.grad(loss, (self._sdf[slot], self._sh[slot]))
        return loss.detach(), overflow, grad_sdf, grad_sh

    def _capture(self) -> None:
        w = self.w
        device = w.grid_sdf.device
        self.stream = torch.cuda.Stream(device)
        self.stream.wait_stream(torch.cuda.current_stream(device))
        with torch.cuda.stream(self.stream):
            self._sdf = [s["grid_sdf"].detach().requires_grad_(True) for s in self.inputs]
            self._sh = [s["grid_sh"].detach().requires_grad_(True) for s in self.inputs]
            # Warm-up on the capture stream: allocates this stream's library
            # workspace and raises kernel shared-memory limits outside capture.
            for _ in range(self.warmup):
                self._step()
            self._workspace = nt.workspace(device).buffer  # kept alive for the graphs
        torch.cuda.current_stream(device).wait_stream(self.stream)
        self.graphs, self._outputs, self.records = [], [], []
        with nt.record_launches() as rec:
            for slot in range(len(self.inputs)):
                g = torch.cuda.CUDAGraph()
                store: dict = {}
                with torch.cuda.graph(g, stream=self.stream):
                    # Loss, overflow flag and gradients written by every replay
                    # (graph-owned memory).
                    if self.record:
                        with recording(store):
                            self._outputs.append(self._step(slot))
                    else:
                        self._outputs.append(self._step(slot))
                self.graphs.append(g)
                self.records.append(store)
        self.launches_per_replay = rec.launches // len(self.inputs)
        self.graph = self.graphs[0]
        self._select(0)
        # Device tables the graph reads (ragged camera grids) stay alive with it.
        self._tables = list(tr._CAMERA_TABLES.values())

    def _select(self, slot: int) -> None:
        self.slot = slot
        self.loss, self.overflow, self.grad_sdf, self.grad_sh = self._outputs[slot]

    def __call__(self, slot: int = 0) -> Tensor:
        """Replay one step (reading input set ``slot``) on the current stream;
        returns the (device) loss. ``self.grad_sdf`` / ``self.grad_sh`` are
        that replay's gradients; for set 0 the workload parameters' ``.grad``
        point at them too."""
        self.graphs[slot].replay()
        self._select(slot)
        if slot == 0:
            self.w.grid_sdf.grad = self.grad_sdf
            self.w.grid_sh.grad = self.grad_sh
        return self.loss

    def run_uncaptured(self, slot: int = 0) -> Tensor:
        """The captured function run once outside the graph, on the capture
        stream: the same library kernels with the same capacities, each
        launched from the host (for per-kernel timing). Returns the loss."""
        with torch.cuda.stream(self.stream):
            loss = self._step(slot)[0]
        return loss

    def check(self) -> bool:
        """True when the last replay (of the last replayed input set) fit its
        capacities. Otherwise re-captures with capacities grown to the
        measured sizes (times the margin) and returns False: the step must be
        replayed again. Synchronizes."""
        if not bool(self.overflow.item()):
            return True
        grown = pipeline.Capacities.around(self._measure(), self.margin)
        c = self.capacities
        self.capacities = pipeline.Capacities(max(c.vertices, grown.vertices), max(c.faces, grown.faces),
                                              max(c.keys, grown.keys))
        self.recaptures += 1
        self._capture()
        return False
