"""Oracle-side restatement of tiny-cuda-nn's model layout rules -- TEST INFRASTRUCTURE ONLY.

From the same JSON configs the library takes, computes every nested encoding's input/output
columns and padding, the grid offset tables and the parameter layout, following
(paths relative to rptr/ext/tiny-cuda-nn/):
  src/encoding.cu:81-164                      encoding factory, per-encoding alignment
  include/tiny-cuda-nn/encodings/composite.h:136-213, 376-386   concatenation + padding
  encodings/repeated_composite.h:48-128       one nested encoding reused over repetitions
  encodings/grid.h:982-1015, 1417-1494        offset table, factory defaults
  encodings/spherical_harmonics.h:393-412, encodings/identity.h
  network_with_input_encoding.h:43-50, 113-120 (alignment 16; params network then encoding)
  src/fully_fused_mlp.cu:640-677              matrices [out][in], output padded to 16
It is written independently of the library's C++ builder so that the two can be compared.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


def _next_multiple(v: int, m: int) -> int:
    return (v + m - 1) // m * m


def _lcm(a: int, b: int) -> int:
    return a * b // math.gcd(a, b)


def grid_levels(n_levels, log2T, base_res, per_level_scale, kind):
    """Returns (offsets[n_levels+1], res[], scale[]) as grid.h computes them.

    The FP32 scale exp2f(level * log2f(s)) * base - 1 is evaluated by the C oracle with the C
    library's exp2f/log2f (numpy's float32 exp2 is not correctly rounded and differs by an ulp
    at some levels, e.g. level 4 of scale 1.5)."""
    import ctypes as C

    from . import lib

    offs = (C.c_uint32 * (n_levels + 1))()
    res = (C.c_uint32 * n_levels)()
    sc = (C.c_float * n_levels)()
    lib().orc_grid_offsets(C.c_int(n_levels), C.c_uint32(log2T), C.c_uint32(base_res), C.c_float(per_level_scale),
                           C.c_int(kind), offs, res, sc)
    return [int(v) for v in offs], [int(v) for v in res], [float(v) for v in sc]


@dataclass
class Node:
    kind: str                      # grid | sh | identity | onehot | composite | repeated
    n_dims: int
    n_out: int = 0
    n_pad: int = 0
    cfg: dict = field(default_factory=dict)
    nested: list = field(default_factory=list)
    dims_begin: list = field(default_factory=list)
    reps: int = 1

    def align(self) -> int:
        if self.kind == "grid":
            return int(self.cfg.get("n_features_per_level", 2))
        if self.kind in ("composite", "repeated"):
            a = 1
            for n in self.nested:
                a = _lcm(a, n.align())
            return a
        return 1

    def width(self) -> int:
        if self.kind == "composite":
            return sum(n.width() for n in self.nested)
        if self.kind == "repeated":
            return sum(n.width() for n in self.nested) * self.reps
        return self.n_out + self.n_pad

    def set_width(self, w: int) -> None:
        if self.kind == "composite":
            prev = self.width() - self.nested[-1].width()
            self.nested[-1].set_width(w - prev)
        elif self.kind == "repeated":
            if w != self.width():
                raise ValueError("RepeatedComposite padding unsupported")
        else:
            if w < self.n_out:
                raise ValueError("padded width below output width")
            self.n_pad = w - self.n_out

    def set_alignment(self, a: int) -> None:
        self.set_width(_next_multiple(self.width(), _lcm(a, self.align())))


def _ieq(a, b):
    return a.lower() == b.lower()


def make_node(cfg: dict, n_dims: int, alignment: int) -> Node:
    ot = cfg.get("otype", "OneBlob")
    if _ieq(ot, "Composite") or _ieq(ot, "RepeatedComposite"):
        rep = _ieq(ot, "RepeatedComposite")
        node = Node("repeated" if rep else "composite", n_dims, reps=int(cfg.get("n_repetitions", 1)) if rep else 1)
        nested = cfg["nested"]
        total = sum(int(e.get("n_dims_to_encode", 0)) for e in nested)
        unspecified = n_dims - total * (node.reps if rep else 1)
        offset = 0
        for r in range(node.reps):
            for e in nested:
                if "n_dims_to_encode" in e:
                    if "dims_to_encode_begin" in e:
                        offset = int(e["dims_to_encode_begin"])
                    nd = int(e["n_dims_to_encode"])
                else:
                    nd = unspecified
                if nd > 0:
                    if r == 0:
                        node.nested.append(make_node(e, nd, 1))
                    node.dims_begin.append(offset)
                offset += nd
        so_far = 0
        for i in range(len(node.nested) - 1):
            want = node.nested[i + 1].align()
            w = _next_multiple(so_far + node.nested[i].width(), want) - so_far
            node.nested[i].set_width(w)
            so_far += node.nested[i].width()
    elif ot.lower() in ("grid", "hashgrid", "tiledgrid", "densegrid"):
        F = int(cfg.get("n_features_per_level", 2))
        n_levels = int(cfg.get("n_levels", 16))
        node = Node("grid", n_dims, n_out=F * n_levels, cfg=dict(cfg))
    elif _ieq(ot, "SphericalHarmonics"):
        d = int(cfg.get("degree", 4))
        node = Node("sh", n_dims, n_out=d * d, cfg=dict(cfg))
    elif _ieq(ot, "Identity"):
        node = Node("identity", n_dims, n_out=n_dims, cfg=dict(cfg))
    elif _ieq(ot, "OneHot"):
        node = Node("onehot", n_dims, n_out=int(cfg.get("n_bins", 8)), cfg=dict(cfg))
    else:
        raise ValueError(f"unsupported encoding {ot}")
    if alignment > 0:
        node.set_alignment(alignment)
    return node


def model_spec(encoding: dict, network: dict, n_input: int, n_output: int) -> dict:
    """Flattened layout: slots, grids (param offsets absolute), layers, n_params."""
    root = make_node(encoding, n_input, 8)
    root.set_alignment(16)
    width = int(network.get("n_neurons", 128))
    n_hidden = int(network.get("n_hidden_layers", 5))
    acts = {"none": 0, "relu": 1, "sigmoid": 2, "exponential": 3}
    enc_width = root.width()
    layers = []
    off = 0
    for l in range(n_hidden + 1):
        nin = enc_width if l == 0 else width
        nout = 16 if l == n_hidden else width
        layers.append({"in": nin, "out": nout, "offset": off})
        off += nin * nout
    n_net = off
    slots, grids = [], []
    state = {"out": 0, "param": n_net}

    def flatten(node: Node, in_begin: int, reuse=None):
        if node.kind == "composite":
            for n, b in zip(node.nested, node.dims_begin):
                flatten(n, in_begin + b)
            return
        if node.kind == "repeated":
            k = len(node.nested)
            ids = [None] * k
            for r in range(node.reps):
                for i, n in enumerate(node.nested):
                    before = len(grids)
                    flatten(n, in_begin + node.dims_begin[r * k + i], None if r == 0 else ids[i])
                    if r == 0 and len(grids) > before:
                        ids[i] = len(grids) - 1
            return
        s = {"type": {"grid": 0, "sh": 1, "identity": 2, "onehot": 3}[node.kind], "in_begin": in_begin,
             "n_in": node.n_dims, "out_begin": state["out"], "out_width": node.width(), "n_pad": node.n_pad,
             "grid": -1, "degree": 0, "n_bins": 0, "scale": 1.0, "offset": 0.0}
        if node.kind == "grid":
            if reuse is not None:
                s["grid"] = reuse
            else:
                c = node.cfg
                ot = c.get("otype", "Grid")
                default_type = "Tiled" if _ieq(ot, "TiledGrid") else ("Dense" if _ieq(ot, "DenseGrid") else "Hash")
                kind = {"hash": 0, "dense": 1, "tiled": 2, "tile": 2}[c.get("type", default_type).lower()]
                hashk = {"coherentprime": 0, "prime": 1, "reversedprime": 2}[c.get("hash", "CoherentPrime").lower()]
                interp = {"linear": 0, "nearest": 1, "smoothstep": 2}[c.get("interpolation", "Linear").lower()]
                n_levels = int(c.get("n_levels", 16))
                offs, res, scales = grid_levels(n_levels, int(c.get("log2_hashmap_size", 19)),
                                                int(c.get("base_resolution", 16)), float(c.get("per_level_scale", 2.0)), kind)
                g = {"n_levels": n_levels, "hash": hashk, "kind": kind, "interp": interp,
                     "param_offset": state["param"], "offset": offs, "res": res, "scale": scales,
                     "n_params": offs[-1] * 2}
                state["param"] += g["n_params"]
                grids.append(g)
                s["grid"] = len(grids) - 1
        elif node.kind == "sh":
            s["degree"] = int(node.cfg.get("degree", 4))
        elif node.kind == "identity":
            s["scale"] = float(node.cfg.get("scale", 1.0))
            s["offset"] = float(node.cfg.get("offset", 0.0))
        elif node.kind == "onehot":
            s["n_bins"] = int(node.cfg.get("n_bins", 8))
        slots.append(s)
        state["out"] += s["out_width"]

    flatten(root, 0)
    return {"n_input": n_input, "n_output": n_output, "enc_width": enc_width, "width": width,
            "n_layers": n_hidden + 1, "act": acts[network.get("activation", "ReLU").lower()],
            "out_act": acts[network.get("output_activation", "None").lower()], "layers": layers,
            "slots": slots, "grids": grids, "n_params_network": n_net, "n_params": state["param"]}
