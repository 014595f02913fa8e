"""Reader for instrument definition files (IDF), the JSON format of RAMP
instruments (grammar documented in the reference's doc/user/idf.rst and
implemented by mcramp/mcramp.py:35-116, 328-384).

An IDF is a JSON object of blocks; a block is an object of components plus
the optional keys "linear" (default true) and "multi" (events of a
non-linear block, default 1).  The file is read in three steps:

1. template expansion: every ``$expr$`` is replaced by ``str(eval(expr))``
   after each instrument parameter name occurring in ``expr`` has been
   replaced by the parameter's value as text, parameter by parameter in the
   order given (a name that is a substring of another name is therefore
   substituted inside it, as the reference does);
2. comment removal: from the first ``//`` of a line to its end, after the
   expansion (an expression inside a comment is still evaluated);
3. JSON decoding, then one pass over the blocks in file order that assigns
   component indices (1 for the first component, the source included, one
   more for every following component; a component with a true "disable"
   takes none), resolves "relative" placements against the already placed
   components of the same block and builds the plugin objects.

The result is a list of ``Block`` objects; each keeps its components as an
ordered name -> dict mapping with the keys the rest of the package reads
("name", "idx", "pos", "rot", "restore_neutron", "vis", "geom_kernel",
"scat_kernel").
"""
import importlib
import json
import re
from collections import OrderedDict

import numpy as np

_TEMPLATE = re.compile(r"\$(.*?)\$")


def frame_rotate(vec, rot):
    """Rotate vec by Euler angles rot = [x, y, z] (mcramp.py:457-476): the
    rotation matrix Rz(z) Ry(y) Rx(x) written element by element and
    applied row by row with float64 dot products, so that relative
    placements come out bit for bit as the reference computes them."""
    x_a, y_a, z_a = rot[0], rot[1], rot[2]
    r00 = np.cos(y_a) * np.cos(z_a)
    r01 = -np.cos(x_a) * np.sin(z_a) + np.sin(x_a) * np.sin(y_a) * np.cos(z_a)
    r02 = np.sin(x_a) * np.sin(z_a) + np.cos(x_a) * np.sin(y_a) * np.cos(z_a)
    r10 = np.cos(y_a) * np.sin(z_a)
    r11 = np.cos(x_a) * np.cos(z_a) + np.sin(x_a) * np.sin(y_a) * np.sin(z_a)
    r12 = -np.sin(x_a) * np.cos(z_a) + np.cos(x_a) * np.sin(y_a) * np.sin(z_a)
    r20 = -np.sin(y_a)
    r21 = np.sin(x_a) * np.cos(y_a)
    r22 = np.cos(x_a) * np.cos(y_a)
    return [np.dot([r00, r01, r02], vec), np.dot([r10, r11, r12], vec),
            np.dot([r20, r21, r22], vec)]


def expand(text, params):
    """Step 1: evaluate every $expr$ of ``text`` with ``params`` (a mapping
    name -> value) substituted as text."""
    names = list(params.items())

    def one(match):
        expr = match.group(1)
        for name, value in names:
            expr = expr.replace(str(name), str(value))
        return str(eval(expr))

    return _TEMPLATE.sub(one, text)


def strip_comments(text):
    """Step 2: drop everything from the first // of each line."""
    return "\n".join(line.partition("//")[0] for line in text.split("\n"))


def resolve_plugin(name):
    """A plugin class by name: the built-in classes of this package first,
    then a module of that name on sys.path holding a class of that name
    (user plugins, as the reference looks them up)."""
    pkg = importlib.import_module(__package__)
    if hasattr(pkg, name):
        return getattr(pkg, name)
    return getattr(importlib.import_module(name), name)


def _plugin_args(spec, **extra):
    args = {k: v for k, v in spec.items() if k != "name"}
    args.update(extra)
    return args


class Block:
    """One block of an IDF: linear (every component once, in order) or
    non-linear ("multi" events of all geometries, then all scatterers)."""

    def __init__(self, linear, multi):
        self.linear = bool(linear)
        self.multi = int(multi)
        self.source = None
        self.components = OrderedDict()

    def __repr__(self):
        return "Block(linear=%s, multi=%d, components=%s)" % (
            self.linear, self.multi, list(self.components))


class Reader:
    """Step 3 for one instrument: blocks in order, running component index,
    plugin construction with the instrument's device."""

    def __init__(self, inst, device):
        self.inst = inst
        self.device = device
        self.next_idx = 1

    def read(self, doc):
        blocks = []
        for number, body in enumerate(doc.values()):
            linear = body.get("linear", True)
            multi = body["multi"] if (not linear and "multi" in body) else 1
            blocks.append(self._block(number, body, Block(linear, multi)))
        return blocks

    def _block(self, number, body, block):
        for name, spec in body.items():
            if name in ("linear", "multi") or spec.get("disable", False):
                continue
            if "source" in spec:
                mod = spec["moderator_kernel"]
                block.source = resolve_plugin(mod["name"])(
                    **_plugin_args(mod, ctx=self.device))
            else:
                block.components[name] = self._component(name, spec, number, block)
            self.next_idx += 1
        return block

    def _component(self, name, spec, number, block):
        pos = spec.get("position", [0, 0, 0])
        rot = spec.get("rotation", [0, 0, 0])
        parent = spec.get("relative")
        if parent is not None:
            # the parent's stored (float32) frame, composed in float64
            ppos, prot = block.components[parent]["pos"], block.components[parent]["rot"]
            pos = np.add(frame_rotate(pos, [prot[0], prot[1], prot[2]]),
                         [ppos[0], ppos[1], ppos[2]])
            rot = np.add(rot, [prot[0], prot[1], prot[2]])
        geom, scat = spec["geom_kernel"], spec["scat_kernel"]
        g = resolve_plugin(geom["name"])(**_plugin_args(geom, idx=self.next_idx, ctx=self.device))
        s = resolve_plugin(scat["name"])(**_plugin_args(scat, idx=self.next_idx, ctx=self.device,
                                                        inst=self.inst, block=number))
        return {"name": name,
                "idx": int(self.next_idx),
                "pos": np.array([pos[0], pos[1], pos[2]], dtype=np.float32),
                "rot": np.array([rot[0], rot[1], rot[2]], dtype=np.float32),
                "restore_neutron": np.uint32(1 if spec.get("restore_neutron", False) else 0),
                "vis": spec.get("visualise", True),
                "geom_kernel": g,
                "scat_kernel": s}


def load(fn, inst, device, params):
    """Blocks of the IDF ``fn`` with instrument parameters ``params``."""
    with open(fn, "r") as fh:
        text = strip_comments(expand(fh.read(), params))
    return Reader(inst, device).read(json.loads(text, object_pairs_hook=OrderedDict))
