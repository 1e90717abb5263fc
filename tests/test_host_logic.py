"""Host-side logic: threshold parsing, configuration, k-mer decoding, the generator."""
import numpy as np
import pytest

import bruno_gb300 as bg
from bruno_gb300 import synth


def test_thresholds_single_value_is_k1_lower_bound():
    # compact_dbg_freq_construct_clean.cpp:940-945
    assert bg.thresholds([3]) == [0, 65536, 3, 65536, 0, 65536]


def test_thresholds_three_values():
    assert bg.thresholds([1, 2, 3], [100, 200, 300]) == [1, 100, 2, 200, 3, 300]


def test_thresholds_capped_at_count_max_plus_one():
    assert bg.thresholds([70000]) == [0, 65536, 65536, 65536, 0, 65536]


def test_thresholds_reject_two_values():
    with pytest.raises(ValueError):
        bg.thresholds([1, 2])


def test_config_roundtrip():
    c = bg.GraphConfig(k=63, thresh=bg.thresholds([3]), min_update=False, table_slots=123).to_c()
    assert (c.k, c.min_update, c.table_slots, list(c.thresh)) == (63, 0, 123, bg.thresholds([3]))


def test_decode_kmers():
    assert bg.decode_kmers(np.array([[0b00011011]], np.uint64), 4) == ["ACGT"]
    v = (1 << 124) | 3
    assert bg.decode_kmers(np.array([[v & (2**64 - 1), v >> 64]], np.uint64), 63) == ["C" + "A" * 61 + "T"]


def test_generator_deterministic_and_thread_independent():
    w = synth.Workload("t", 50_000, 100, 2_000, 0.01, 31, (2,), 0.05, (100, 500), (2, 4), (0.01, 0.02), seed=7)
    a = synth.make_fastq(w, threads=1)
    b = synth.make_fastq(w, threads=4)
    assert np.array_equal(a, b)
    assert a.nbytes == synth.fastq_size(w)
    lines = a.tobytes().split(b"\n")
    assert lines[0] == b"@r0" and lines[2] == b"+" and len(lines[1]) == 100 and set(lines[3]) == {ord("I")}


def test_workloads_match_configs():
    s, m = synth.WORKLOADS["plain-small"], synth.WORKLOADS["plain-scale"]
    assert (s.genome_len, s.n_reads, s.read_len, s.sub_rate, s.k) == (1_000_000, 100_000, 100, 0.01, 31)
    assert (m.genome_len, m.read_len, m.k, round(m.coverage)) == (50_000_000, 150, 31, 30)


def test_partition_mix_is_a_bijection():
    """the 62-bit mix that lets an 8-byte record carry a k-mer (kmer.cuh bj_fwd/bj_inv),
    restated here with the constants read from the source"""
    import os
    import random
    import re
    src = open(os.path.join(os.path.dirname(bg.__file__), "csrc", "kmer.cuh")).read()
    c1 = int(re.search(r"BJ_C1 = (0x[0-9A-Fa-f]+)ull", src).group(1), 16)
    c2 = int(re.search(r"BJ_C2 = (0x[0-9A-Fa-f]+)ull", src).group(1), 16)
    m = (1 << 62) - 1
    c1, c2 = c1 & m, c2 & m
    assert c1 & 1 and c2 & 1

    def inv(c):
        x = c
        for _ in range(6):
            x = (x * (2 - c * x)) % (1 << 64)
        return x

    def fwd(x):
        x ^= x >> 31; x = (x * c1) & m; x ^= x >> 29; x = (x * c2) & m; x ^= x >> 32
        return x

    def xs_inv(y, s):
        x, t = y, s
        while t < 62:
            x, t = y ^ (x >> s), t + s
        return x

    def back(h):
        x = xs_inv(h, 32); x = (x * inv(c2)) & m; x = xs_inv(x, 29); x = (x * inv(c1)) & m
        return xs_inv(x, 31)

    rnd = random.Random(5)
    for _ in range(20000):
        v = rnd.getrandbits(62)
        h = fwd(v)
        assert h <= m and back(h) == v


# ----------------------------------------------------- host FASTQ piece boundaries
PIECE_HARNESS = r'''
#include "piece_cuts.h"
#include <cstdio>
#include <string>
int main(int argc, char **argv) {
  FILE *f = fopen(argv[1], "rb");
  std::string b;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) b.append(buf, n);
  fclose(f);
  for (uint64_t c : piece_cuts(b.data(), b.size(), strtoull(argv[2], 0, 10))) printf("%llu\n", (unsigned long long)c);
}
'''


@pytest.fixture(scope="module")
def piece_cuts_cli(tmp_path_factory):
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("pc")
    src, exe = d / "pc.cpp", d / "pc"
    src.write_text(PIECE_HARNESS)
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(bg.__file__), "csrc"), str(src),
                    "-o", str(exe)], check=True)

    def run(data: bytes, piece: int):
        f = d / "in.fq"
        f.write_bytes(data)
        return [int(x) for x in subprocess.check_output([str(exe), str(f), str(piece)]).split()]
    return run


def _record_starts(fq: bytes):
    starts, pos = set(), 0
    for i, line in enumerate(fq.split(b"\n")):
        if i % 4 == 0:
            starts.add(pos)
        pos += len(line) + 1
    return starts


@pytest.mark.parametrize("piece", [1024, 4096, 1 << 16])
def test_piece_cuts_fall_on_record_starts(piece_cuts_cli, piece):
    """bruno_load_fastq cuts host FASTQ only at record starts, even where every quality line
    begins with '@', and about every `piece` bytes"""
    w = synth.Workload("pc", 50_000, 100, 2_000, 0.01, 31, (2,), 0.0, (1000, 2000), (2, 2), (0.01, 0.01), 5)
    lines = bytes(synth.make_fastq(w)).split(b"\n")
    for i in range(3, len(lines), 4):
        if lines[i]:
            lines[i] = b"@" + lines[i][1:]
    fq = b"\n".join(lines)
    cuts = piece_cuts_cli(fq, piece)
    assert cuts[0] == 0 and cuts == sorted(set(cuts))
    assert set(cuts) <= _record_starts(fq)
    assert len(cuts) >= len(fq) // piece - 2
    assert all(b - a < 2 * piece + 1024 for a, b in zip(cuts, cuts[1:] + [len(fq)]))


def test_piece_cuts_small_or_unsplittable_inputs(piece_cuts_cli):
    rec = b"@r\nACGT\n+\nIIII\n"
    assert piece_cuts_cli(rec * 10, 1 << 20) == [0]          # under two pieces: one copy
    assert piece_cuts_cli(rec * 10, 0) == [0]
    one = b"@r\n" + b"A" * 5000 + b"\n+\n" + b"I" * 5000 + b"\n"
    assert piece_cuts_cli(one, 1024) == [0]                  # one record: nowhere to cut


# ----------------------------------------------------------------- pool admission rules
RULES_HARNESS = r'''
#include "pool_admission.h"
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
/* each line: op budget w est solo running n held... busy...  ->  prints 0 or 1 (E n -> the estimate) */
int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    std::string op;
    in >> op;
    if (op == "E") { unsigned long long n; in >> n; printf("%llu\n", (unsigned long long)bruno_pool_rules::estimate(n)); continue; }
    unsigned long long budget, est; int w, solo, running, n;
    in >> budget >> w >> est >> solo >> running >> n;
    std::vector<uint64_t> held(n);
    std::vector<bool> busy(n);
    for (auto &h : held) { unsigned long long x; in >> x; h = x; }
    for (int i = 0; i < n; ++i) { int b; in >> b; busy[i] = b != 0; }
    const bool r = op == "A" ? bruno_pool_rules::admits(held, busy, budget, w, est, solo != 0, running != 0)
                             : bruno_pool_rules::should_trim(held, busy, budget, w, est, solo != 0, running != 0);
    printf("%d\n", r ? 1 : 0);
  }
}
'''


@pytest.fixture(scope="module")
def pool_rules(tmp_path_factory):
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("rules")
    src, exe = d / "rules.cpp", d / "rules"
    src.write_text(RULES_HARNESS)
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", os.path.join(os.path.dirname(bg.__file__), "csrc"), str(src),
                    "-o", str(exe)], check=True)

    def run(lines):
        out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return [int(x) for x in out.stdout.split()]
    return run


def _q(op, budget, w, est, solo, held, busy, running=False):
    return " ".join(str(x) for x in [op, budget, w, est, int(solo), int(running), len(held), *held,
                                     *[int(b) for b in busy]])


def test_pool_estimate(pool_rules):
    assert pool_rules(["E 0", "E 1000"]) == [64 << 20, 20_000 + (64 << 20)]


def test_pool_admission_rules(pool_rules):
    cases = [
        # (expected, query)
        (1, _q("A", 1000, 0, 500, False, [0, 0], [False, False])),      # fits
        (1, _q("A", 1000, 0, 2000, False, [0, 0], [False, False])),     # too large, but nothing else runs
        (0, _q("A", 1000, 1, 500, False, [600, 0], [True, False])),     # 600 + 500 over budget beside a busy one
        (1, _q("A", 1000, 1, 300, False, [600, 0], [True, False])),     # 600 + 300 fits
        (1, _q("A", 1000, 1, 500, False, [600, 0], [False, False])),    # over budget, but the other is idle
        (1, _q("A", 1000, 0, 500, False, [800, 0], [False, False])),    # a worker counts at max(held, est)
        (0, _q("A", 1000, 0, 100, True, [0, 0], [False, True])),        # solo: waits for the busy one
        (1, _q("A", 1000, 0, 100, True, [0, 900], [False, False])),     # solo: nothing busy, budget ignored
        # trimming: only an idle worker holding buffers, only when no free worker can take the head
        (1, _q("T", 1000, 0, 600, False, [600, 500], [False, True])),
        (0, _q("T", 1000, 0, 300, False, [600, 0], [False, True])),     # worker 0 can take it
        (0, _q("T", 1000, 1, 600, False, [600, 500], [False, True])),   # worker 1 is busy
        (0, _q("T", 1000, 0, 600, False, [0, 500], [False, True])),     # holds nothing
        (1, _q("T", 1000, 0, 600, False, [400, 700, 0], [False, True, False])),
        # a retried (solo) request is running: nothing else starts beside it, however small,
        # and no idle worker trims for a head that cannot start anyway
        (0, _q("A", 1000, 0, 10, False, [0, 900], [False, True], running=True)),
        (0, _q("A", 1000, 0, 10, False, [0, 0, 0], [False, True, False], running=True)),
        (0, _q("T", 1000, 0, 600, False, [600, 500], [False, True], running=True)),
        (1, _q("A", 1000, 0, 10, False, [0, 900], [False, True], running=False)),
    ]
    assert pool_rules([q for _, q in cases]) == [e for e, _ in cases]


# ---------------------------------------------------- the C++ facade's -L/-U mapping
THRESH_HARNESS = r'''
#include "bruno_gb300.hpp"
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
/* each line: nlo lo... nhi hi...  ->  the six thresholds */
int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    std::istringstream in(line);
    size_t n;
    std::vector<uint64_t> lo, hi;
    in >> n; lo.resize(n); for (auto &x : lo) in >> x;
    in >> n; hi.resize(n); for (auto &x : hi) in >> x;
    for (uint64_t t : bruno_gb300::thresholds(lo, hi)) printf("%llu ", (unsigned long long)t);
    printf("\n");
  }
}
'''


def test_cpp_thresholds_match_python(tmp_path):
    """the driver's -L/-U handling in the C++ facade equals bruno_gb300.thresholds (and so the
    reference driver's, compact_dbg_freq_construct_clean.cpp:937-961)"""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    src, exe = tmp_path / "t.cpp", tmp_path / "t"
    src.write_text(THRESH_HARNESS)
    inc = os.path.join(os.path.dirname(os.path.dirname(bg.__file__)), "include")
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", inc, str(src), "-o", str(exe)], check=True)
    cases = [((), ()), ((2,), ()), ((3,), (50,)), ((1, 2, 3), ()), ((1, 2, 3), (10, 20, 30)), ((70000,), ()),
             ((), (5,)), ((0,), (65536,))]
    lines = [" ".join(str(x) for x in [len(lo), *lo, len(hi), *hi]) for lo, hi in cases]
    out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [[int(x) for x in l.split()] for l in out.stdout.splitlines()]
    assert got == [bg.thresholds(lo, hi) for lo, hi in cases]


# ----------------------------------------------------- table partitions and the scatter split
PLAN_HARNESS = r'''
#include "table_plan.h"
#include <cstdio>
#include <cstdlib>
using namespace bruno_table_plan;
int main(int argc, char **argv) {
  const char *what = argv[1];
  const unsigned long long a = strtoull(argv[2], 0, 10);
  if (what[0] == 'p') {
    const Plan p = partitions(a, strtoull(argv[3], 0, 10), atoi(argv[4]));
    printf("%d %llu %d\n", p.pbits, (unsigned long long)p.region, p.fits ? 1 : 0);
  } else if (what[0] == 'w') {
    printf("%d\n", scatter_lg_window((int)a));
  } else if (what[0] == 'r') {
    printf("%d\n", scatter_lg_runs(a));
  } else {
    printf("%d\n", region_class(a));
  }
}
'''


@pytest.fixture(scope="module")
def plan_cli(tmp_path_factory):
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("plan")
    src, exe = d / "plan.cpp", d / "plan"
    src.write_text(PLAN_HARNESS)
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(bg.__file__), "csrc"), str(src),
                    "-o", str(exe)], check=True)
    return lambda *args: [int(x) for x in subprocess.check_output([str(exe), *map(str, args)]).split()]


def test_partition_plans(plan_cli):
    # plain scale: 461M slots in 2^18 partitions of 1760 (k_split's 8 + 10 bits suffice)
    assert plan_cli("p", 461_373_440, 3072, 16) == [18, 1760, 1]
    # a forced 80M-slot table of regions of at most 256 slots: 2^19 partitions of 153
    assert plan_cli("p", 80_000_000, 256, 16) == [19, 153, 1]
    # large k: 1.70B 64-byte slots, regions of at most 1536: 2^21 partitions of 811
    assert plan_cli("p", 1_700_790_272, 1536, 16) == [21, 811, 1]
    # small tables keep the 256 buckets as partitions, at least 64 slots each
    assert plan_cli("p", 1000, 3072, 10) == [8, 64, 1]
    # too large for the split bits allowed: the caller falls back
    assert plan_cli("p", 1 << 32, 3072, 10)[2] == 0
    # every plan covers the slots asked for
    for slots in (1, 65_536, 3_000_001, 987_654_321):
        pb, region, fits = plan_cli("p", slots, 3072, 16)
        assert fits and region << pb >= slots and region <= 3072


def test_scatter_window_and_runs(plan_cli):
    # at least 8192 partition cursors in a window: one bucket once a bucket has 8192 partitions
    assert plan_cli("w", 21) == [0]
    assert plan_cli("w", 20) == [1]
    assert plan_cli("w", 15) == [6]
    assert plan_cli("w", 8) == [8]
    # a bucket's 32-record runs counted up to a power of two
    assert plan_cli("r", 1) == [0]
    assert plan_cli("r", 32) == [0]
    assert plan_cli("r", 33) == [1]
    assert plan_cli("r", 15_000_000) == [19]


def test_region_classes(plan_cli):
    bounds = [128, 192, 256, 384, 512, 768, 1024, 1536, 2048]
    for c, b in enumerate(bounds):
        assert plan_cli("c", b) == [c] and plan_cli("c", b + 1) == [c + 1]
    assert plan_cli("c", 64) == [0] and plan_cli("c", 3072) == [9]
