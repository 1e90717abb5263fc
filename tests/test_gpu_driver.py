"""The reference driver's integration tests, restated: run the GB300 driver and the oracle
driver with the same flags on the same FASTQ and diff every output file (the reference's
test_compact_debruijn_graph_*.sh compare outputs of variants and rank counts the same way)."""
import os
import subprocess

import pytest

from bruno_gb300 import build
from oracle import oracle
from conftest import DATA

pytestmark = pytest.mark.gpu

CASES = [
    ("test.unitiqs.fastq", []),
    ("test.star.unitiqs.fastq", ["-T", "-L", "2", "-R"]),
    ("debruijn.palindrome_chr14.fastq", ["-T", "-L", "2", "-R"]),
    ("debruijn.shifted_cycle_chr14.fastq", ["-T", "-L", "2"]),
    ("debruijn.bubble.fastq", ["-T", "-L", "1", "-L", "2", "-L", "1", "-R"]),
    ("natural.withN.fastq", []),
    ("debruijn.palindrome_chr14.fastq", ["-T", "-L", "2", "-L", "2", "-L", "2", "-R"]),
    ("debruijn.bubble.fastq", ["-T", "-E", "-L", "2", "-R"]),
    ("test.medium.fastq", ["-T", "-E", "-L", "3"]),
]
OUTPUTS = [".chain.fasta", ".chain.components", ".chain.edges", ".chain.summary", ".branch.fasta", ".branch.edges",
           ".graph.all"]


@pytest.mark.parametrize("fname,flags", CASES)
def test_driver_outputs_identical(tmp_path, fname, flags):
    drv = build.build_driver()
    oracle.build()
    fq = os.path.join(DATA, fname)
    run = subprocess.run([drv, *flags, "-O", str(tmp_path / "gpu"), fq], check=True, capture_output=True)
    subprocess.run([oracle.CLI, *flags, "-O", str(tmp_path / "ref"), fq], check=True, capture_output=True)
    for ext in OUTPUTS:
        if ext == ".chain.summary" and not os.path.exists(tmp_path / ("gpu" + ext)):
            # declined only for chain pointers that are not mutually consistent (separate k / k+2 bounds)
            assert b"mutually consistent" in run.stderr and flags.count("-L") == 3
            continue
        a = open(tmp_path / ("gpu" + ext), "rb").read()
        b = open(tmp_path / ("ref" + ext), "rb").read()
        assert a == b, f"{fname} {' '.join(flags)}: {ext} differs"
