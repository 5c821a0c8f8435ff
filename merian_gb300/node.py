"""merian graph JSONs of the `pt` path's nodes, run by the library's C++ node graph (graph.cpp).

merian hosts its nodes as C++ classes behind a registry (src/merian-graph/graph/node_registry.cpp:
60-110) and runs a graph JSON (examples/renderers/pt.json: "nodes" -> name -> {"type", "enabled",
"properties", "outputs": ["output->node.input"]}) one iteration at a time (graph.cpp:323-360).
libgbpt does the same in C++ for the node types on this path: "Render (Path-traced)", "GBuffer
(Raytraced)", "Accumulate", "Image Write" (PFM), "Error Plot", "GLTF Scene" and "PBRT Scene",
with merian's connector names, property keys and defaults. `Graph` is the Python handle on it.

Errors follow the reference: a value a node cannot honour raises (merian's node_error);
set_property returns merian's NodeStatusFlags (NEEDS_RECONNECT when a connector layout changes).
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import _native as N

NEEDS_RECONNECT = 1  # NodeStatusFlags (include/merian-graph/graph/node.hpp:58-65)
RESET_IN_FLIGHT_DATA = 2
REMOVE_NODE = 4


class Graph:
    """A graph JSON (dict, JSON text or path) of the node types above. With ctx = None the graph
    is checked (types, properties, edges) but cannot run."""

    def __init__(self, ctx, config: dict | str | Path):
        if isinstance(config, Path) or (isinstance(config, str) and
                                        not config.lstrip().startswith("{")):
            config = Path(config).read_text()
        text = config if isinstance(config, str) else json.dumps(config)
        self.ctx = ctx
        self.lib = N.load()
        self.handle = C.c_void_p()
        N.check(self.lib.gbpt_graph_create(ctx.handle if ctx is not None else None,
                                           text.encode(), C.byref(self.handle)))

    def close(self) -> None:
        if self.handle:
            self.lib.gbpt_graph_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def order(self) -> list[str]:
        """Node names in run order (dependencies first, ties by name)."""
        n = C.c_uint32()
        N.check(self.lib.gbpt_graph_node_count(self.handle, C.byref(n)))
        names = []
        for i in range(n.value):
            name = C.c_char_p()
            N.check(self.lib.gbpt_graph_node(self.handle, i, C.byref(name), None))
            names.append(name.value.decode())
        return names

    def node_type(self, node: str) -> str:
        for i, name in enumerate(self.order):
            if name == node:
                t = C.c_char_p()
                N.check(self.lib.gbpt_graph_node(self.handle, i, None, C.byref(t)))
                return t.value.decode()
        raise KeyError(node)

    @property
    def warnings(self) -> list[str]:
        return [self.lib.gbpt_graph_warning(self.handle, i).decode()
                for i in range(self.lib.gbpt_graph_warning_count(self.handle))]

    def properties(self, node: str, key: str | None = None):
        """Every property of a node as a dict, or one value ("group/key" inside a group)."""
        n = C.c_uint64()
        k = key.encode() if key is not None else None
        N.check(self.lib.gbpt_graph_get_property(self.handle, node.encode(), k, None, 0,
                                                 C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        N.check(self.lib.gbpt_graph_get_property(self.handle, node.encode(), k, buf,
                                                 n.value + 1, None))
        return json.loads(buf.value.decode())

    def set_property(self, node: str, key: str, value) -> int:
        flags = C.c_uint32()
        N.check(self.lib.gbpt_graph_set_property(self.handle, node.encode(), key.encode(),
                                                 json.dumps(value).encode(), C.byref(flags)))
        return flags.value

    def run(self, scene_id: int, camera: N.Camera | None, extent: tuple[int, int],
            iterations: int = 1) -> None:
        """Runs `iterations` graph iterations on the context stream. Nodes whose "scene" input
        is connected to a scene node render that scene with the file's camera, the others
        `scene_id` with `camera`; `extent` (width, height) sizes a renderer that has no GBuffer
        input."""
        cam = C.byref(camera) if camera is not None else None
        N.check(self.lib.gbpt_graph_run(self.handle, scene_id, cam, int(extent[0]),
                                        int(extent[1]), iterations))

    @property
    def options(self) -> dict[str, str]:
        """The graph JSON's "cli" options: name -> JSON pointer of the property it sets."""
        out, i = {}, 0
        while True:
            name, ptr = C.c_char_p(), C.c_char_p()
            if self.lib.gbpt_graph_option(self.handle, i, C.byref(name), C.byref(ptr)) != 0:
                return out
            out[name.value.decode()] = ptr.value.decode()
            i += 1

    def set_option(self, name: str, value) -> int:
        flags = C.c_uint32()
        N.check(self.lib.gbpt_graph_set_option(self.handle, name.encode(),
                                               json.dumps(value).encode(), C.byref(flags)))
        return flags.value

    def to_json(self) -> dict:
        """The graph in merian's graph-JSON layout, every property included."""
        n = C.c_uint64()
        N.check(self.lib.gbpt_graph_to_json(self.handle, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        N.check(self.lib.gbpt_graph_to_json(self.handle, buf, n.value + 1, None))
        return json.loads(buf.value.decode())

    def save(self, directory: str | Path) -> None:
        """Checkpoint: iteration count, node properties and counters, accumulated images."""
        Path(directory).mkdir(parents=True, exist_ok=True)
        N.check(self.lib.gbpt_graph_save(self.handle, str(directory).encode()))

    def load(self, directory: str | Path) -> None:
        """Resume from a checkpoint of a graph made from the same JSON."""
        N.check(self.lib.gbpt_graph_load(self.handle, str(directory).encode()))

    def output(self, connector: str) -> np.ndarray:
        """The output "node.output" as a host array (height, width, floats per texel)."""
        w, h, f = C.c_uint32(), C.c_uint32(), C.c_uint32()
        N.check(self.lib.gbpt_graph_output(self.handle, connector.encode(), None, 0, C.byref(w),
                                           C.byref(h), C.byref(f)))
        out = np.zeros((h.value, w.value, f.value), np.float32)
        N.check(self.lib.gbpt_graph_output(self.handle, connector.encode(), N.ptr(out),
                                           out.size, None, None, None))
        return out


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
