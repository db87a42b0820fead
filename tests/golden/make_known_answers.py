"""Writes tests/golden/known_answers.json: the known-answer vectors that
SimilaritySearch.jl's own test-suite pins for the distances on the exhaustive
path, restated as data (the reference is Julia, which cannot run here, so the
values are read from its test files and cited per entry).

Run:  python tests/golden/make_known_answers.py
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # test/testdistances.jl:7-8,34-36 -- u=[1,2,3], v=[4,6,8]
    {"cite": "test/testdistances.jl:35", "metric": "sql2", "a": [1, 2, 3], "b": [4, 6, 8],
     "expect": 50.0, "exact": True},
    # `== sqrt(50.0f0)`: the Float32 square root of 50, compared exactly
    {"cite": "test/testdistances.jl:36", "metric": "l2", "a": [1, 2, 3], "b": [4, 6, 8],
     "expect_f32_sqrt_of": 50.0, "exact": True},
    {"cite": "test/testdistances.jl:38", "metric": "l2", "a": [1, 2, 3], "b": [1, 2, 3],
     "expect": 0.0, "exact": True},
    # 3-4-5 triangle, test/testdistances.jl:44-51
    {"cite": "test/testdistances.jl:47", "metric": "l2", "a": [3, 4], "b": [0, 0],
     "expect": 5.0, "exact": True},
    {"cite": "test/testdistances.jl:48", "metric": "sql2", "a": [3, 4], "b": [0, 0],
     "expect": 25.0, "exact": True},
    # orthogonal unit vectors, test/testdistances.jl:53-68
    {"cite": "test/testdistances.jl:58", "metric": "sql2", "a": [1, 0, 0], "b": [0, 1, 0],
     "expect": 2.0, "exact": True},
    {"cite": "test/testdistances.jl:57", "metric": "l2", "a": [1, 0, 0], "b": [0, 1, 0],
     "expect": math.sqrt(2.0), "exact": False, "atol": 1e-6},
    {"cite": "test/testdistances.jl:63", "metric": "cosine", "a": [1, 0, 0], "b": [0, 1, 0],
     "expect": 1.0, "exact": True},
    {"cite": "test/testdistances.jl:66", "metric": "normcosine", "a": [1, 0, 0], "b": [0, 1, 0],
     "expect": 1.0, "exact": True},
    {"cite": "test/testdistances.jl:68", "metric": "normcosine", "a": [1, 0, 0], "b": [1, 0, 0],
     "expect": 0.0, "exact": True},
    # binary Hamming, test/testdistances.jl:183-205
    {"cite": "test/testdistances.jl:192", "metric": "hamming", "a": [0b1010, 0b1100],
     "b": [0b1000, 0b1100], "expect": 1.0, "exact": True},
    {"cite": "test/testdistances.jl:191", "metric": "hamming", "a": [0b1010, 0b1100],
     "b": [0b1010, 0b1100], "expect": 0.0, "exact": True},
    {"cite": "test/testdistances.jl:202", "metric": "hamming", "a": [0b11110000],
     "b": [0b00001111], "expect": 8.0, "exact": True},
    {"cite": "test/testdistances.jl:203", "metric": "hamming", "a": [0b11110000],
     "b": [0b11110000], "expect": 0.0, "exact": True},
]

# test/testresults.jl:57-85 ("XKnn"): KnnSorted after every push equals the
# first k of the pushed items stably sorted by distance, for these k.
KNNSORTED_KS = [7, 8, 12, 15, 67]
KNNSORTED_PUSHES = 1000

# test/testparallelexhaustive.jl:9-77: ParallelExhaustiveSearch == ExhaustiveSearch
# for these k on n=300, dim=6 (k is clamped to n as the test does with min(k, n)).
PARALLEL_CASE = {"n": 300, "dim": 6, "m": 40, "ks": [1, 4, 300, 305], "batch_k": 5, "allknn_k": 4}

# test/testexactseq.jl:15-31,73-78: self-queries find themselves (nearest < 1e-3).
SELFQUERY_CASES = [
    {"metric": "sql2", "dim": 4, "n": 200, "m": 20, "k": 4},
    {"metric": "normcosine", "dim": 4, "n": 200, "m": 30, "k": 4},
    {"metric": "hamming", "dim": 8, "n": 200, "m": 20, "k": 4},
]


def main():
    out = {
        "source": "SimilaritySearch.jl 1.2.0 test-suite, restated as data",
        "distances": CASES,
        "knnsorted": {"cite": "test/testresults.jl:57-85", "ks": KNNSORTED_KS,
                      "pushes": KNNSORTED_PUSHES},
        "parallel": dict(PARALLEL_CASE, cite="test/testparallelexhaustive.jl:9-77"),
        "selfquery": {"cite": "test/testexactseq.jl:15-31,64-78", "cases": SELFQUERY_CASES,
                      "valid_lower": 1e-3},
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
