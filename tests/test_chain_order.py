"""CPU tests of the locality order's pivot chain (csrc/chain.h).

allknn groups the database rows by nearest pivot and lays the groups out in a
greedy chain of the pivots (ssg::greedy_chain, host code).  The bucket sort
that follows counts rows per chain place, so the chain must be a permutation
of the pivots whatever the neighbour lists hold (short lists, padding,
self-references, out-of-range entries).  The header is compiled here with g++
into a small driver and compared with a Python restatement of the rule.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "similaritysearch.jl_gb300", "csrc")
PAD = 0xFFFFFFFF

DRIVER = r"""
#include "chain.h"
#include <cstdio>
#include <vector>
int main() {
    int P, k, back;
    if (std::scanf("%d %d %d", &P, &k, &back) != 3) return 2;
    std::vector<uint32_t> near(static_cast<size_t>(P) * k);
    for (auto &v : near) {
        unsigned long long x;
        if (std::scanf("%llu", &x) != 1) return 2;
        v = static_cast<uint32_t>(x);
    }
    std::vector<uint32_t> place(static_cast<size_t>(P));
    ssg::greedy_chain(near.data(), P, k, back, place.data());
    for (int p = 0; p < P; ++p) std::printf("%u\n", place[p]);
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("chain")
    src = d / "chain_driver.cpp"
    src.write_text(DRIVER)
    exe = d / "chain_driver"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def run_chain(driver, near, back):
    P, k = near.shape
    text = f"{P} {k} {back}\n" + "\n".join(" ".join(str(int(v)) for v in row) for row in near) + "\n"
    out = subprocess.run([driver], input=text, capture_output=True, text=True, check=True).stdout
    return np.array([int(x) for x in out.split()], dtype=np.int64)


def chain_py(near, back):
    """The rule restated: start at pivot 0; the next link is the first
    unplaced pivot of the last link's list, else of the lists of up to
    `back` earlier links (latest first), else the lowest unplaced pivot."""
    P, k = near.shape
    place = np.full(P, -1, dtype=np.int64)
    chain = [0]
    place[0] = 0
    for r in range(1, P):
        nxt = None
        for b in range(0, min(back, r - 1) + 1):
            for q in near[chain[r - 1 - b]]:
                q = int(q)
                if q < P and place[q] < 0:
                    nxt = q
                    break
            if nxt is not None:
                break
        if nxt is None:
            nxt = int(np.flatnonzero(place < 0)[0])
        place[nxt] = r
        chain.append(nxt)
    return place


def knn_lists(X, k):
    d = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    return np.argsort(d, axis=1, kind="stable")[:, :k].astype(np.int64)


@pytest.mark.parametrize("P,k,back,seed", [(1, 4, 64, 0), (2, 1, 0, 1), (200, 16, 64, 2), (500, 4, 0, 3),
                                           (333, 16, 3, 4)])
def test_chain_is_the_greedy_permutation(driver, P, k, back, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((P, 8))
    near = knn_lists(X, min(k, max(P - 1, 1))) if P > 1 else np.full((1, k), PAD, dtype=np.int64)
    if near.shape[1] < k:
        near = np.concatenate([near, np.full((P, k - near.shape[1]), PAD, dtype=np.int64)], axis=1)
    place = run_chain(driver, near, back)
    assert np.array_equal(np.sort(place), np.arange(P))
    assert np.array_equal(place, chain_py(near, back))


def test_chain_survives_bad_lists(driver):
    # padding, self-references, out-of-range ids and duplicates are skipped;
    # pivots no list names are still placed (lowest unplaced first)
    rng = np.random.default_rng(9)
    P, k = 300, 6
    near = rng.integers(0, 2 * P, size=(P, k))
    near[::7] = PAD
    near[:, 0] = np.arange(P)           # each list starts with the pivot itself
    near[5] = [7, 7, 7, PAD, 10**6, 3]
    place = run_chain(driver, near, 2)
    assert np.array_equal(np.sort(place), np.arange(P))
    assert np.array_equal(place, chain_py(near, 2))


def test_chain_keeps_clusters_together(driver):
    # pivots drawn around 20 well separated centres: each centre's pivots
    # take one run of consecutive places (the reason for the chain)
    rng = np.random.default_rng(5)
    C = rng.standard_normal((20, 16)) * 10
    lab = np.repeat(np.arange(20), 8)
    X = C[lab] + rng.standard_normal((160, 16)) * 0.1
    place = run_chain(driver, knn_lists(X, 16), 64)
    order = np.argsort(place)
    runs = 1 + int(np.count_nonzero(lab[order][1:] != lab[order][:-1]))
    assert runs == 20
