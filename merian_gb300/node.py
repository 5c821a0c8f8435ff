"""merian graph nodes of the `pt` path, hosted on the GB300 path tracer (libgbpt.so).

`RenderPT` mirrors merian's "Render (Path-traced)" node (src/merian-graph/nodes/render_pt/
render_pt.cpp:27-35,94-124,147-186; defaults render_pt.hpp:53-73): the same type name, the same
connectors (inputs "scene" and "gbuffer", output "irradiance": RGBA32F at the GBuffer's extent,
rgb = mean radiance, a = mean squared luminance), the same JSON property keys with the same
defaults, and one render per graph iteration whose RNG lane 3 is the iteration ("seed").
Properties this build adds: "next event estimation" and "russian roulette depth" (both off by
default, which is merian's estimator).

`Accumulate` is merian's "Accumulate" for a static camera (accumulate.slang:233-257,
accumulate.cpp:170-186 for the keys), `ImageWrite` its "Image Write" for PFM files
(image_write.cpp:16-30, image_io.cpp:138-176). `Graph` loads graph JSONs of these node types in
merian's layout (examples/renderers/pt.json: "nodes" -> {"type", "properties", "outputs":
["out->node.in"]}) and runs iterations.

Errors follow the reference: an unknown property value raises ValueError (merian's node_error);
RenderPT.properties returns NEEDS_RECONNECT when the output format changes.
"""
from __future__ import annotations

import ctypes as C
import json
import math
from pathlib import Path

import numpy as np

from . import _native as N

NEEDS_RECONNECT = 1  # NodeStatusFlags (include/merian-graph/graph/node.hpp:58-65)
RESET_IN_FLIGHT_DATA = 2
REMOVE_NODE = 4


class RenderPT:
    TYPE = "Render (Path-traced)"
    INPUTS = ("scene", "gbuffer")
    OUTPUTS = ("irradiance",)
    DEFAULTS = {
        "samples per pixel": 1,
        "max path length": 5,
        "emission on primary": True,
        "shader execution reordering": False,
        "demodulate albedo": False,
        **{str(b): True for b in range(8)},
        "irradiance format": "R32G32B32A32Sfloat",
        "next event estimation": False,
        "russian roulette depth": 0,
    }
    FORMATS = ("R32G32B32A32Sfloat",)

    def __init__(self, ctx, properties: dict | None = None):
        self.ctx = ctx
        self.props = dict(self.DEFAULTS)
        self.extent = (1920, 1080)  # render_pt.hpp: the extent before a GBuffer is connected
        self.irradiance = None
        if properties:
            self.properties(properties)

    def properties(self, config: dict) -> int:
        flags = 0
        for key, value in config.items():
            if key not in self.DEFAULTS:
                raise ValueError(f"{self.TYPE}: unknown property {key!r}")
            if key == "irradiance format":
                if value not in self.FORMATS:
                    raise ValueError(f"{self.TYPE}: irradiance format {value!r} is not supported "
                                     f"(RGBA32F only)")
                if value != self.props[key]:
                    flags |= NEEDS_RECONNECT
            self.props[key] = value
        spp, L = int(self.props["samples per pixel"]), int(self.props["max path length"])
        if spp < 0 or not 1 <= L <= 64:
            raise ValueError(f"{self.TYPE}: samples per pixel must be >= 0 and max path length "
                             f"in [1, 64]")
        return flags

    def instance_mask(self) -> int:
        return sum(1 << b for b in range(8) if self.props[str(b)])

    def describe_outputs(self, gbuffer_extent: tuple[int, int]) -> dict:
        self.extent = tuple(gbuffer_extent)
        return {"irradiance": (self.props["irradiance format"], self.extent)}

    def render_params(self, iteration: int, pixels: np.ndarray | None = None):
        from . import scene as S
        W, H = self.extent
        return S.render_params(W, H, int(self.props["samples per pixel"]),
                               int(self.props["max path length"]),
                               emission_on_primary=bool(self.props["emission on primary"]),
                               instance_mask=self.instance_mask(), frame=iteration,
                               nee=bool(self.props["next event estimation"]),
                               rr_depth=int(self.props["russian roulette depth"]),
                               sort_materials=bool(self.props["shader execution reordering"]),
                               demodulate_albedo=bool(self.props["demodulate albedo"]),
                               pixels=pixels)

    def process(self, scene_id: int, camera: N.Camera, iteration: int, out=None):
        """Renders one iteration into `out` (a CUDA tensor of H*W*4 float32) or into the node's
        own irradiance tensor, enqueued on the context stream; returns the tensor."""
        import torch
        W, H = self.extent
        if out is None:
            if self.irradiance is None or self.irradiance.shape != (H, W, 4):
                self.irradiance = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
                torch.cuda.current_stream().synchronize()  # the context has its own stream
            out = self.irradiance
        p, keep = self.render_params(iteration)
        self.ctx.render_device(scene_id, camera, p, out.data_ptr())
        return out


class Accumulate:
    TYPE = "Accumulate"
    INPUTS = ("src",)
    OUTPUTS = ("out", "history")
    DEFAULTS = {"alpha": 0.0, "max history": math.inf, "inf history": False, "clear": False}

    def __init__(self, ctx, properties: dict | None = None):
        self.ctx = ctx
        self.props = dict(self.DEFAULTS)
        self.out = None
        self.history = None
        self._clear = True
        if properties:
            self.properties(properties)

    def properties(self, config: dict) -> int:
        for key, value in config.items():
            if key not in self.DEFAULTS:
                raise ValueError(f"{self.TYPE}: unknown property {key!r}")
            self.props[key] = value
        if self.props["clear"]:
            self._clear = True
            self.props["clear"] = False
        return 0

    def process(self, src, iteration: int):
        import torch
        if self.out is None or self.out.shape != src.shape:
            self.out = torch.zeros_like(src)
            self.history = torch.zeros(src.shape[:-1], dtype=torch.float32, device=src.device)
            torch.cuda.current_stream().synchronize()  # the context has its own stream
            self._clear = True
        max_hist = math.inf if self.props["inf history"] else float(self.props["max history"])
        clear = self._clear or iteration == 0
        N.check(self.ctx.lib.gbpt_accumulate(self.ctx.handle, src.data_ptr(), self.out.data_ptr(),
                                             self.history.data_ptr(), src.numel() // 4,
                                             float(self.props["alpha"]), max_hist, int(clear)))
        self._clear = False
        return self.out


class ImageWrite:
    TYPE = "Image Write"
    INPUTS = ("src",)
    OUTPUTS = ()
    DEFAULTS = {"filename": "image_{iteration:06d}.pfm", "enable": True, "every": 1}

    def __init__(self, ctx, properties: dict | None = None):
        self.ctx = ctx
        self.props = dict(self.DEFAULTS)
        self.written: list[str] = []
        if properties:
            self.properties(properties)

    def properties(self, config: dict) -> int:
        for key, value in config.items():
            if key not in self.DEFAULTS:
                raise ValueError(f"{self.TYPE}: unknown property {key!r}")
            self.props[key] = value
        if not str(self.props["filename"]).endswith(".pfm"):
            raise ValueError(f"{self.TYPE}: only PFM output is supported")
        return 0

    def process(self, src, iteration: int):
        if not self.props["enable"] or iteration % int(self.props["every"]):
            return None
        self.ctx.synchronize()
        host = np.ascontiguousarray(src.detach().cpu().numpy(), dtype=np.float32)
        H, W = host.shape[:2]
        path = str(self.props["filename"]).format(iteration=iteration)
        write_pfm(path, host, W, H)
        self.written.append(path)
        return path


def write_pfm(path: str, texels: np.ndarray, width: int, height: int) -> None:
    lib = N.load()
    t = np.ascontiguousarray(texels, dtype=np.float32)
    ch = t.size // (width * height)
    N.check(lib.gbpt_image_write_pfm(str(path).encode(), N.ptr(t), width, height, ch))


def read_pfm(path: str, channels: int = 4) -> np.ndarray:
    lib = N.load()
    w, h = C.c_uint32(), C.c_uint32()
    N.check(lib.gbpt_image_read_pfm(str(path).encode(), None, channels, C.byref(w), C.byref(h)))
    out = np.zeros((h.value, w.value, channels), np.float32)
    N.check(lib.gbpt_image_read_pfm(str(path).encode(), N.ptr(out), channels, C.byref(w),
                                    C.byref(h)))
    return out


NODE_TYPES = {cls.TYPE: cls for cls in (RenderPT, Accumulate, ImageWrite)}


class Graph:
    """A graph JSON of the node types above: nodes, their properties and "out->node.in" edges."""

    def __init__(self, ctx, config: dict | str | Path):
        if not isinstance(config, dict):
            config = json.loads(Path(config).read_text())
        self.ctx = ctx
        self.nodes: dict = {}
        self.edges: list[tuple[str, str, str, str]] = []
        for name, spec in config.get("nodes", {}).items():
            if not spec.get("enabled", True):
                continue
            t = spec.get("type")
            if t not in NODE_TYPES:
                raise ValueError(f"node {name!r}: type {t!r} is not available in this build")
            self.nodes[name] = NODE_TYPES[t](ctx, spec.get("properties"))
            for edge in spec.get("outputs", []):
                out, dst = edge.split("->")
                dst_node, dst_in = dst.split(".")
                self.edges.append((name, out, dst_node, dst_in))
        self.order = self._topological()

    def _topological(self):
        deps = {n: set() for n in self.nodes}
        for src, _, dst, _ in self.edges:
            if src in self.nodes and dst in self.nodes:
                deps[dst].add(src)
        order, done = [], set()
        while len(order) < len(self.nodes):
            ready = [n for n in self.nodes if n not in done and deps[n] <= done]
            if not ready:
                raise ValueError("graph has a cycle")
            for n in sorted(ready):
                order.append(n)
                done.add(n)
        return order

    def run(self, scene_id: int, camera: N.Camera, extent: tuple[int, int], iterations: int = 1):
        """Runs the graph `iterations` times for one scene and camera; returns the last outputs
        of every node by "node.connector"."""
        outputs: dict = {}
        for node in self.nodes.values():
            if isinstance(node, RenderPT):
                node.describe_outputs(extent)
        for it in range(iterations):
            for name in self.order:
                node = self.nodes[name]
                inputs = {dst_in: outputs.get(f"{src}.{out}")
                          for src, out, dst, dst_in in self.edges if dst == name}
                if isinstance(node, RenderPT):
                    outputs[f"{name}.irradiance"] = node.process(scene_id, camera, it)
                elif isinstance(node, Accumulate):
                    outputs[f"{name}.out"] = node.process(inputs["src"], it)
                elif isinstance(node, ImageWrite):
                    node.process(inputs["src"], it)
        self.ctx.synchronize()
        return outputs
