"""Regenerates the golden fixtures of the test suite.

1. Copies the reference's own FASTQ/FASTA fixtures (ParBLiSS/bruno test/data, Apache-2.0)
   into tests/golden/data, so tests never read the reference tree at run time.
2. Runs the CPU oracle on every fixture with every option set of the reference's
   integration scripts (unthresholded, -T -L 1/2/3, -R on/off, the 3-value form) and
   records a digest of each output in expected.json; with ":clean", the same for the graph
   after the _freq_clean driver's dead-end and bubble cleaning.

Usage: python tests/golden/make_golden.py <path of the ParBLiSS/bruno source tree>
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

FIXTURES = [
    "test.unitiqs.fastq", "test.unitiqs.fasta", "test.star.unitiqs.fastq", "test.star.unitiqs.fasta",
    "test.star2.unitiqs.fastq", "test.star2.unitiqs.fasta", "test.short.unitiqs.fastq", "test.short.unitiqs.fasta",
    "test.debruijn.small.fastq", "test.medium.fastq", "debruijn.palindrome.fastq", "debruijn.palindrome2.fastq",
    "debruijn.palindrome_chr14.fastq", "debruijn.shifted_cycle_chr14.fastq", "debruijn.bubble.fastq",
    "debruijn.bubble2.fastq", "natural.fastq", "natural.withN.fastq", "debruijn.clean1.fastq",
    "debruijn.clean2.fastq",
]
FASTQ = [f for f in FIXTURES if f.endswith(".fastq")]
# (name, thresholding, lower thresholds, upper thresholds, min_update)
OPTIONS = [
    ("u", False, (), (), True),
    ("tl1", True, (1,), (), True),
    ("tl2", True, (2,), (), True),
    ("tl2_norank", True, (2,), (), False),
    ("tl3", True, (3,), (), True),
    ("tl3v", True, (1, 2, 1), (), True),
]


def digest(result: dict) -> dict:
    def h(*arrays) -> str:
        m = hashlib.sha256()
        for a in arrays:
            m.update(a.tobytes() if hasattr(a, "tobytes") else bytes(a))
        return m.hexdigest()[:16]
    out = {n: result[n] for n in ("n_nodes", "n_branch", "n_chain_nodes", "iterations", "n_cycle_nodes",
                                   "n_isolated", "n_ranked", "n_chains", "collisions")}
    out["nodes"] = h(*result["nodes"])
    out["ranked"] = h(*result["ranked"])
    out["chains"] = h(*result["chains"])
    return out


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the ParBLiSS/bruno source tree>")
    ref = sys.argv[1]
    data = os.path.join(HERE, "data")
    os.makedirs(data, exist_ok=True)
    for f in FIXTURES:
        shutil.copy(os.path.join(ref, "test", "data", f), os.path.join(data, f))
    import bruno_gb300 as bg
    from oracle import oracle
    oracle.build()
    expected = {}
    for f in FASTQ:
        fq = open(os.path.join(data, f), "rb").read()
        for name, thr_on, lo, hi, mu in OPTIONS:
            r = oracle.run(fq, k=31, thresholding=thr_on, thresh=bg.thresholds(lo, hi), min_update=mu, clean=True)
            expected[f"{f}:{name}"] = digest(r) if r["status"] == 0 else {"status": r["status"]}
            if r["status"] == 0:
                expected[f"{f}:{name}:clean"] = dict(digest(r["clean"]), **r["clean_stats"])
    with open(os.path.join(HERE, "expected.json"), "w") as fh:
        json.dump(expected, fh, indent=1, sort_keys=True)
    print(f"{len(expected)} golden entries")


if __name__ == "__main__":
    main()
