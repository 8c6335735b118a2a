"""gbblas/metric.py reproduces the reference's benchmark metric formats
(include/metric.hpp): the summary of metric::str, metric::csv and
metric::raw, and amt::range's size sweeps (include/range.hpp)."""
import numpy as np

from gbblas.metric import Metric, reference_range


def make():
    m = Metric(3, np.float32)
    for v in (10.0, 20.0, 30.0):
        m["Boost.ublas.tensor"].update(v)
    for v in (40.0, 50.5, 60.0):
        m["gbblas.GB300"].update(v)
    return m


def test_summary_text_matches_metric_str():
    m = make()
    # peak = 2.3 * 8 * 32 (float), include/metric.hpp:30
    want = (
        "Peak Performance: 588.8 GFlops\n"
        "Name: Boost.ublas.tensor\n"
        "\tMin GFlops: 10\n"
        "\tMax GFlops: 30\n"
        "\tMax SpeedUp with respect to tensor: 1\n"
        "\tAvg SpeedUp with respect to tensor: 1\n"
        "\tMax Peak Utilization in %: 5.09511\n"
        "\tAvg GFlops: 20\n"
        "\tAvg Peak Utilization in %: 3.39674\n\n"
        "Name: gbblas.GB300\n"
        "\tMin GFlops: 40\n"
        "\tMax GFlops: 60\n"
        "\tMax SpeedUp with respect to tensor: 0.5\n"
        "\tAvg SpeedUp with respect to tensor: 0.398671\n"
        "\tMax Peak Utilization in %: 10.1902\n"
        "\tAvg GFlops: 50.1667\n"
        "\tAvg Peak Utilization in %: 8.52015\n\n"
    )
    assert m.str("tensor") == want


def test_double_peak_and_minimum_start_at_the_peak():
    m = Metric(1, np.float64)
    assert m.peak == 2.3 * 8 * 16
    m["x"].update(1000.0)  # above the CPU peak: the minimum keeps its start value, as in the reference
    assert m["x"].min == m.peak


def test_csv_and_raw_formats(tmp_path):
    m = make()
    m.csv(str(tmp_path / "t.csv"))
    assert (tmp_path / "t.csv").read_text() == '"Boost.ublas.tensor","gbblas.GB300"\n10,40\n20,50.5\n30,60\n'
    m.raw(str(tmp_path / "t.txt"))
    assert (tmp_path / "t.txt").read_text() == "Boost.ublas.tensor 10 20 30 \ngbblas.GB300 40 50.5 60 \n"
    assert m.head(2) == "Boost.ublas.tensor: [ 10, 20, ]\ngbblas.GB300: [ 40, 50.5, ]\n"
    assert m.tail(1) == "Boost.ublas.tensor: [ 20, ]\ngbblas.GB300: [ 50.5, ]\n"


def test_reference_size_sweeps():
    # src/mtm.cpp:371: range(x, 32, 3*1024, 32, plus)
    x = reference_range(32.0, 3 * 1024.0, 32.0, "plus")
    assert x[0] == 32 and x[-1] == 3040 and len(x) == 95
    # src/mtv.cpp:336: range(x, 2, 1<<16, 2, multiplies)
    assert reference_range(2.0, float(1 << 16), 2.0, "multiplies") == [float(2 ** k) for k in range(1, 16)]
