"""CPU oracle for the exhaustive k-NN path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline /
reference arm import this package.  The GPU library never calls it.
"""
from .oracle import *  # noqa: F401,F403
