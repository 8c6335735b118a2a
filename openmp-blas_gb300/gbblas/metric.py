"""The reference's benchmark metric, in Python: per-implementation GFLOP/s
series over a size sweep, printed and saved in the reference's formats so
GPU numbers sit next to its published sweeps.

Mirrors ``amt::metric<T>`` (reference include/metric.hpp:27-512):

* ``m[name].update(gflops)`` appends one point (include/metric.hpp:38-43);
  a series' minimum starts at the peak, as in the reference (line 34);
* ``str(pattern)`` is the summary text of ``metric::str`` (lines 436-465):
  peak line, then per series min / max / speed-ups against the series whose
  name contains ``pattern`` / peak utilisation / average;
* ``csv(filename)`` writes ``metric::csv`` (lines 479-500): one header row of
  quoted series names, then one row per size;
* ``raw(filename)`` writes ``metric::raw`` (lines 467-477): "name v v v ...";
* ``head(n)`` / ``tail(n)`` as lines 414-434.

Series keep insertion order (the reference iterates an unordered_map, whose
order is unspecified).  Numbers print like C++ ostreams' default (``%g``).
The peak defaults to the reference's CPU formula 2.3 GHz x 8 cores x
(32 | 16) flop/cycle for float | double (line 30); GPU runs pass their own.
The Matplot++ plots of the reference are not reproduced (no graphics stack);
``csv`` carries the same series.
"""
from __future__ import annotations

import numpy as np


def _g(v: float) -> str:
    return f"{v:g}"


class FlopsData:
    def __init__(self, peak: float):
        self.plot: list[float] = []
        self.min = peak
        self.max = 0.0
        self.agg = 0.0

    def update(self, f: float) -> None:
        f = float(f)
        self.agg += f
        self.min = min(self.min, f)
        self.max = max(self.max, f)
        self.plot.append(f)


class Metric:
    def __init__(self, total: int, dtype=np.float32, peak: float | None = None):
        double = np.dtype(dtype) == np.float64
        self.peak = peak if peak is not None else 2.3 * 8.0 * (16.0 if double else 32.0)
        self.type_name = "[Double-Precision]" if double else "[Single-Precision]"
        self.total = int(total)
        self.data: dict[str, FlopsData] = {}

    def __getitem__(self, name: str) -> FlopsData:
        if name not in self.data:
            self.data[name] = FlopsData(self.peak)
        return self.data[name]

    def insert_or_update(self, name: str, gflops) -> FlopsData:
        d = self[name]
        if np.ndim(gflops):
            vals = [float(v) for v in gflops]
            d.plot = vals
            d.agg = float(sum(vals))
            d.min = min(vals)
            d.max = max(vals)
        else:
            d.update(gflops)
        return d

    def str(self, pattern: str | None = None) -> str:
        pref = None
        if pattern is not None:
            for k, v in self.data.items():
                if pattern in k:
                    pref = v
                    break
        out = [f"Peak Performance: {_g(self.peak)} GFlops\n"]
        for k, v in self.data.items():
            avg = v.agg / float(self.total)
            out.append(f"Name: {k}\n")
            out.append(f"\tMin GFlops: {_g(v.min)}\n")
            out.append(f"\tMax GFlops: {_g(v.max)}\n")
            if pref is not None:
                patt_avg = pref.agg / float(self.total)
                out.append(f"\tMax SpeedUp with respect to {pattern}: {_g(pref.max / v.max)}\n")
                out.append(f"\tAvg SpeedUp with respect to {pattern}: {_g(patt_avg / avg)}\n")
            out.append(f"\tMax Peak Utilization in %: {_g(v.max / self.peak * 100.0)}\n")
            out.append(f"\tAvg GFlops: {_g(avg)}\n")
            out.append(f"\tAvg Peak Utilization in %: {_g(avg / self.peak * 100.0)}\n\n")
        return "".join(out)

    __str__ = str

    def head(self, n: int = 5) -> str:
        return "".join(f"{k}: [ " + "".join(f"{_g(x)}, " for x in v.plot[:n]) + "]\n" for k, v in self.data.items())

    def tail(self, n: int = 5) -> str:
        out = []
        for k, v in self.data.items():
            last = len(v.plot) - 1 - n
            out.append(f"{k}: [ " + "".join(f"{_g(v.plot[last + i])}, " for i in range(n)) + "]\n")
        return "".join(out)

    def raw(self, filename: str = "raw_data.txt") -> None:
        with open(filename, "w") as f:
            for k, v in self.data.items():
                f.write(k + " " + "".join(f"{_g(d)} " for d in v.plot) + "\n")

    def csv(self, filename: str = "raw_data.csv") -> None:
        names = list(self.data)
        with open(filename, "w") as f:
            f.write(",".join('"' + k.replace("\\", "\\\\").replace('"', '\\"') + '"' for k in names) + "\n")
            for i in range(self.total):
                f.write(",".join(_g(self.data[k].plot[i]) for k in names) + "\n")


def reference_range(start: float, end: float, stride: float, op: str) -> list[float]:
    """amt::range(x, start, end, stride, fn) (reference include/range.hpp:27-40):
    start, fn(start, stride), ... while below end; op is "plus" or "multiplies"."""
    out = []
    v = start
    while v < end:
        out.append(v)
        v = v + stride if op == "plus" else v * stride
    return out
