"""Event log contract (mirror of src/log.jl:6-133).

Index mutations report ``LOG(logger, event, index, ctx, sp, ep)`` with
``event`` one of ``"add!"`` (objects sp..ep were added, exactly once per
logical batch) or ``"info"`` (nothing structural changed).
"""
from __future__ import annotations

import sys
import time


class AbstractLog:
    def log(self, event, index, ctx, sp, ep):
        raise NotImplementedError


class InformativeLog(AbstractLog):
    """Throttled stderr printer (log.jl:97-133)."""

    def __init__(self, period: float = 1.0):
        self.period = period
        self.last = 0.0

    def log(self, event, index, ctx, sp, ep):
        now = time.monotonic()
        if now - self.last >= self.period:
            self.last = now
            print(f"LOG {event} {type(index).__name__} sp={sp} ep={ep} n={len(index)}", file=sys.stderr)


class RecorderLog(AbstractLog):
    """Keeps every (event, sp, ep) -- the recorder the reference's log tests use."""

    def __init__(self):
        self.events = []

    def log(self, event, index, ctx, sp, ep):
        self.events.append((event, sp, ep))


class LogList(AbstractLog):
    def __init__(self, loggers):
        self.list = list(loggers)

    def log(self, event, index, ctx, sp, ep):
        for lg in self.list:
            lg.log(event, index, ctx, sp, ep)


def LOG(logger, event, index, ctx, sp, ep):
    if logger is not None:
        logger.log(event, index, ctx, sp, ep)
