"""Seeded synthetic inputs of the benchmark configurations C1-C5.

No public dataset is involved: each generator draws numpy
``Generator(PCG64(seed))`` streams with the shapes, sizes and value
distributions the configurations name, so the benchmark and the tests at
those sizes see the same data.

* C1  searchbatch, SqL2: n = 100,000 database rows and m = 1,000 queries of
      d = 128, all N(0, 1) (seeds 1, 2), k = 10.
* C2  allknn self-join, NormCosine: n = 1,000,000 rows of d = 96 from a
      1,000-cluster Gaussian mixture (centres N(0, 1), per-cluster sigma
      U[0.1, 0.5], uniform assignment; seeds 3, 4, 5), L2-normalised;
      k = 32 excluding the object itself.
* C3  Hamming: 2,000,000 sketches of 1,024 bits (16 UInt64 words, each bit
      Bernoulli(1/2); seed 6); 10,000 queries, each a random database
      sketch (seed 7) with every bit flipped with probability 0.1 (seed 8);
      k = 100.
* C4  request stream: 2,000,000 rows of d = 768 from a 4,096-cluster
      mixture (centres N(0, 1), sigma U[0.05, 0.3]; seeds 9, 10, 11) with
      row norms LogNormal(0, 0.25) (seed 12); batch sizes
      round(LogNormal(ln 64, 1)) clipped to [1, 4096] (seed 13), k uniform
      over {1, 10, 100} (seed 14); queries from the same mixture (seeds 15,
      16).
      Held-out queries (seeds 17, 18) and over-fetch calibration queries
      (seeds 19, 20) come from the same mixture.
* C5  the learned shortlist on the C4 database (SqL2, k = 10).
"""
from __future__ import annotations

import numpy as np


def make_c1(n: int = 100_000, m: int = 1_000, d: int = 128):
    """(X (n, d), Q (m, d), k) of C1."""
    X = np.random.default_rng(1).standard_normal((n, d), dtype=np.float32)
    Q = np.random.default_rng(2).standard_normal((m, d), dtype=np.float32)
    return X, Q, 10


def make_c2(n: int = 1_000_000, d: int = 96, centres: int = 1000) -> np.ndarray:
    """C2's database (n, d) Float32, rows L2-normalised."""
    C = np.random.default_rng(3).standard_normal((centres, d), dtype=np.float32)
    sig = np.random.default_rng(4).uniform(0.1, 0.5, size=centres).astype(np.float32)
    g = np.random.default_rng(5)
    lab = g.integers(0, centres, size=n)
    X = g.standard_normal((n, d), dtype=np.float32)
    X *= sig[lab, None]
    X += C[lab]
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    return X


def make_c3(n: int = 2_000_000, m: int = 10_000, words: int = 16):
    """(X (n, words) UInt64, Q (m, words) UInt64, k) of C3."""
    X = np.random.default_rng(6).integers(0, 2**64 - 1, size=(n, words), dtype=np.uint64, endpoint=True)
    src = np.random.default_rng(7).integers(0, n, size=m)
    flips = np.random.default_rng(8).random((m, words * 64)) < 0.1
    mask = np.ascontiguousarray(np.packbits(flips, axis=1)).view(np.uint64)
    return X, X[src] ^ mask, 100


def c4_draw(count: int, seed_lab: int, seed_norm: int, d: int = 768) -> np.ndarray:
    """`count` rows of C4's mixture with log-normal norms."""
    centres = np.random.default_rng(9).standard_normal((4096, d), dtype=np.float32)
    sig = np.random.default_rng(10).uniform(0.05, 0.3, size=4096).astype(np.float32)
    g = np.random.default_rng(seed_lab)
    out = np.empty((count, d), dtype=np.float32)
    for s0 in range(0, count, 250_000):
        c = min(250_000, count - s0)
        lab = g.integers(0, 4096, size=c)
        blk = g.standard_normal((c, d), dtype=np.float32)
        blk *= sig[lab, None]
        blk += centres[lab]
        blk /= np.linalg.norm(blk, axis=1, keepdims=True)
        out[s0:s0 + c] = blk
    out *= np.random.default_rng(seed_norm).lognormal(0.0, 0.25, size=(count, 1)).astype(np.float32)
    return out


def make_c4(n: int = 2_000_000, d: int = 768, batches: int = 200):
    """(X (n, d), Q (sum of sizes, d), sizes, ks) of C4's request stream."""
    X = c4_draw(n, 11, 12, d)
    sizes = np.clip(np.round(np.random.default_rng(13).lognormal(np.log(64), 1.0, size=batches)), 1, 4096)
    sizes = sizes.astype(np.int64)
    ks = np.random.default_rng(14).choice([1, 10, 100], size=batches)
    Q = c4_draw(int(sizes.sum()), 15, 16, d)
    return X, Q, sizes, ks


def c4_heldout_queries(m: int, d: int = 768) -> np.ndarray:
    """Queries from C4's mixture on seeds the request stream does not use
    (17, 18): held out from every calibration."""
    return c4_draw(m, 17, 18, d)


def c4_calibration_queries(m: int, d: int = 768) -> np.ndarray:
    """Queries from C4's mixture on their own seeds (19, 20), for tuning the
    over-fetch: neither the timed request stream nor the held-out queries."""
    return c4_draw(m, 19, 20, d)
