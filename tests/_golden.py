"""Loader for tests/golden/golden.npz (written by tests/golden/make_golden.py
from the reference's own compiled hot path)."""
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")
_cache = None


def _load():
    global _cache
    if _cache is None:
        _cache = np.load(PATH)
    return _cache


def names(prefix: str = ""):
    return [str(n) for n in _load()["_names"] if str(n).startswith(prefix)]


def case(name: str) -> dict:
    g = _load()
    out = {}
    pre = name + "/"
    for k in g.files:
        if not k.startswith(pre):
            continue
        key = k[len(pre):]
        v = g[k]
        if key.endswith("@"):
            out[key[:-1]] = g[str(v)]
        else:
            out[key] = v
    return out
