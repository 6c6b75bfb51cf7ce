"""ORACLE — test infrastructure only.

numpy restatement of the MAGIC weight-window update,
WeightWindows::update_weights (src/weight_windows.cpp:502-755) with
WeightWindowUpdateMethod::MAGIC, applied to a flux tally's SUM and SUM_SQ
arrays.  Only the tests use it, as the checker of
openmc_weight_windows_update_magic.
"""
from __future__ import annotations

import numpy as np


def update_weights(tally_sum, tally_sum_sq, n, volume, value="mean", threshold=1.0, ratio=5.0):
    """tally_sum, tally_sum_sq: flux score of the tally as [energy group][mesh
    bin] (the weight windows' own layout, src/weight_windows.cpp:560-640);
    n realizations; volume of one mesh element.  Returns (lower, upper) with
    the same shape.

    Steps, in the reference's order:
      mean = sum / n; rel_err = sqrt((sum_sq / n - mean^2) / (n - 1)) / mean
        where sum > 0, else the largest double (:640-659)
      bounds = mean, or 1 / rel_err for value 'rel_err' (:660-663)
      bounds /= volume (:667-673)
      per energy group: bounds *= 1 / (2 max) when max > 0 (:675-700)
      bounds = -1 where sum <= 0 or rel_err > threshold; upper = ratio x
        lower (:734-753)
    """
    if value not in ("mean", "rel_err"):
        raise ValueError(f"Invalid value '{value}' specified for weight window generation.")
    s = np.asarray(tally_sum, dtype=np.float64)
    s2 = np.asarray(tally_sum_sq, dtype=np.float64)
    mean = s / n
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(s > 0, np.sqrt((s2 / n - mean * mean) / (n - 1)) / mean, np.finfo(np.float64).max)
        b = 1.0 / rel if value == "rel_err" else mean.copy()
    b = b / volume
    for e in range(b.shape[0]):
        row = b[e]
        mx = row[row > 0].max() if (row > 0).any() else 0.0
        if mx > 0:
            b[e] = row * (1.0 / (2.0 * mx))
    lower = np.where(s <= 0, -1.0, np.where(rel > threshold, -1.0, b))
    return lower, ratio * lower
