"""Recall metrics (mirror of src/perf.jl:31-33, 71-79)."""
from __future__ import annotations

import numpy as np


def recallscore(gold, res) -> float:
    """|Set(gold) ∩ Set(res)| / length(gold)"""
    g = [int(x) for x in np.asarray(gold).ravel()]
    r = {int(x) for x in np.asarray(res).ravel()}
    return len(set(g) & r) / len(g)


def macrorecall(goldI, resI, k: int | None = None) -> float:
    """Mean per-column recallscore; columns cut to their first k entries.
    goldI / resI are (k, n) matrices like the reference's."""
    goldI = np.asarray(goldI)
    resI = np.asarray(resI)
    if k is None:
        k = goldI.shape[0]
    n = goldI.shape[1]
    s = 0.0
    for i in range(n):
        s += recallscore(goldI[:k, i], resI[:k, i])
    return s / n
