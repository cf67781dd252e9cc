"""Loads the committed golden fixtures (tests/golden/, made by make_golden.py
from the reference's own code)."""
import functools
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@functools.lru_cache(None)
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


@functools.lru_cache(None)
def ltc():
    d = np.load(os.path.join(GOLDEN, "ltc_synthetic_seed0_64.npz"))
    return d["ltc0"], d["ltc1"], d["constants"]


@functools.lru_cache(None)
def scene(name):
    d = np.load(os.path.join(GOLDEN, "scene_%s.npz" % name))
    meta = manifest()["scenes"][name]
    prim = d["primitive"] if meta["has_primitive"] else None
    return dict(meta, gbuffer=d["gbuffer"], primitive=prim, lights=d["lights"], triangles=d["triangles"])


@functools.lru_cache(None)
def outputs():
    return dict(np.load(os.path.join(GOLDEN, "reference_outputs.npz")))


def config(name):
    c = manifest()["configs"][name]
    sh = c["shader"]
    return dict(scene=c["scene"], random_numbers=c["random_numbers"], candidates=int(sh.get("m", 32)),
                technique=sh.get("technique", "ltc_cp"), light_sampling=sh.get("light_sampling", "ris"),
                mis=sh.get("mis", "optimal_clamped"), sample_count=int(sh.get("sample_count", 1)),
                light_samples=int(sh.get("light_samples", 1)), fast_atan=bool(sh.get("fast_atan", 0)))


def reference_result(name):
    o = outputs()
    return o["rgb_" + name], o["reads_" + name]


def reference_chosen_index(name):
    """The reservoir's light for one RIS light sample: the last light-buffer
    read when the shader read M + 1 lights, else -1."""
    c = config(name)
    rgb, reads = reference_result(name)
    return np.where(reads[:, 0] == c["candidates"] + 1, reads[:, 1], -1)


CONFIG_NAMES = sorted(manifest()["configs"].keys())
