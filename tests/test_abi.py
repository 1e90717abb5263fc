"""The drop-in boundary: the C header, the shared library and the Python binding agree
(no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re
import subprocess

import pytest

import bruno_gb300 as bg
from bruno_gb300 import build
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bruno_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return bg.load_library()


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bruno_[a-z_0-9]+)\s*\(", text)))


def test_header_matches_binding():
    assert declared() == sorted(bg.EXPORTS)


def test_library_exports_every_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", bg.LIB_PATH], capture_output=True, text=True).stdout
    syms = {l.split()[-1] for l in out.splitlines() if l.strip()}
    missing = [s for s in declared() if s not in syms]
    assert not missing, missing


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(f'''
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu\\n", sizeof(bruno_cfg), offsetof(bruno_cfg, thresh), offsetof(bruno_cfg, table_slots),
         offsetof(bruno_cfg, keep_filtered), sizeof(bruno_sizes));
  return 0;
}}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    C = bg._Cfg
    want = [ctypes.sizeof(C), C.thresh.offset, C.table_slots.offset, C.keep_filtered.offset, ctypes.sizeof(bg._Sizes)]
    assert got == want


def test_pool_result_layout_matches_header(tmp_path):
    src = tmp_path / "layout2.c"
    src.write_text(f'''
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu\\n", sizeof(bruno_pool_result), offsetof(bruno_pool_result, sizes),
         offsetof(bruno_pool_result, n_chains), offsetof(bruno_pool_result, chars),
         offsetof(bruno_pool_result, run_ms));
  return 0;
}}''')
    exe = tmp_path / "layout2"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    R = bg._PoolResult
    assert got == [ctypes.sizeof(R), R.sizes.offset, R.n_chains.offset, R.chars.offset, R.run_ms.offset]


def test_pool_bad_arguments_rejected_without_gpu(lib):
    cfg = bg.GraphConfig().to_c()
    h = ctypes.c_void_p()
    assert lib.bruno_pool_create(ctypes.byref(cfg), 0, 0, ctypes.byref(h)) == 1
    assert lib.bruno_pool_create(None, 4, 0, ctypes.byref(h)) == 1


def test_bad_config_rejected_without_gpu(lib):
    """k outside 3..63 is refused before any CUDA call"""
    cfg = bg.GraphConfig(k=64).to_c()
    h = ctypes.c_void_p()
    assert lib.bruno_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert lib.bruno_ctx_create(None, ctypes.byref(h)) == 1
    # the (k+1)-mer edge filter runs on the partitioned count, not the whole-table one
    for bad in (bg.GraphConfig(k=45, edge_filter=True, direct_count=1),
                bg.GraphConfig(k=31, edge_filter=True, direct_count=1)):
        cfg = bad.to_c()
        assert lib.bruno_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == 1


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(bg.BrunoError):
        bg._lib_backup = bg._lib
        try:
            bg._lib = None
            bg.load_library(str(tmp_path / "absent.so"))
        finally:
            bg._lib = bg._lib_backup


def test_clean_stats_layout_matches_header(tmp_path):
    src = tmp_path / "layout3.c"
    src.write_text(f'''
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu\\n", sizeof(bruno_clean_stats), offsetof(bruno_clean_stats, edges),
         offsetof(bruno_clean_stats, status));
  printf("%zu %zu\\n", offsetof(bruno_cfg, h2d_chunk), offsetof(bruno_cfg, h2d_streams));
  return 0;
}}''')
    exe = tmp_path / "layout3"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    S, C = bg._CleanStats, bg._Cfg
    assert got == [ctypes.sizeof(S), S.edges.offset, S.status.offset, C.h2d_chunk.offset, C.h2d_streams.offset]


def test_device_view_layout_matches_header(tmp_path):
    src = tmp_path / "layout4.c"
    src.write_text(f'''
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu %zu\\n", sizeof(bruno_device_view), offsetof(bruno_device_view, chain_chars),
         offsetof(bruno_device_view, n_ranked), offsetof(bruno_device_view, words));
  printf("%zu\\n", offsetof(bruno_cfg, rank_fill));
  return 0;
}}''')
    exe = tmp_path / "layout4"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    V, C = bg._DeviceView, bg._Cfg
    assert got == [ctypes.sizeof(V), V.chain_chars.offset, V.n_ranked.offset, V.words.offset, C.rank_fill.offset]


def test_check_and_tunable_layouts_match_header(tmp_path):
    src = tmp_path / "layout5.c"
    src.write_text(f'''
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu\\n", sizeof(bruno_index_check), offsetof(bruno_index_check, n_unanswered),
         offsetof(bruno_index_check, edge_hist));
  printf("%zu %zu %zu\\n", offsetof(bruno_cfg, part_slots), offsetof(bruno_cfg, count_threads), sizeof(bruno_cfg));
  printf("%d %d %d\\n", (int)BRUNO_IS_CHAIN_NODE, (int)BRUNO_CHAIN_POINTS_TO_INTERNAL_NODE, (int)BRUNO_IS_BRANCH_POINT);
  return 0;
}}''')
    exe = tmp_path / "layout5"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    X, C = bg._IndexCheck, bg._Cfg
    assert got == [ctypes.sizeof(X), X.n_unanswered.offset, X.edge_hist.offset, C.part_slots.offset,
                   C.count_threads.offset, ctypes.sizeof(C), bg.NODE_FILTERS["IsChainNode"],
                   bg.CHAIN_FILTERS["PointsToInternalNode"], bg.NODE_FILTERS["IsBranchPoint"]]
