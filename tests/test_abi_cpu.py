"""CPU-side checks of the C ABI: the library builds, loads, exports every
symbol include/lelph_gpu.h declares, and the ctypes descriptor matches the C
struct layout.  No kernel runs."""
import os
import re
import subprocess
import tempfile

import ctypes

from letzelphc_gb300 import elph
from letzelphc_gb300.build import build_library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lelph_gpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(lelph_gpu_[a-z_]+)\s*\(", txt)))


def test_library_exports_header_symbols():
    lib = ctypes.CDLL(build_library())
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(elph.EXPORTS)


def test_ndb_writer_exports_header_symbols():
    from letzelphc_gb300 import ndb
    lib = ctypes.CDLL(build_library())
    names = sorted(set(re.findall(r"\b(lelph_ndb_[a-z_]+)\s*\(", open(os.path.join(ROOT, "include", "lelph_ndb.h")).read())))
    assert set(names) == set(ndb.EXPORTS)
    for n in names:
        assert hasattr(lib, n), n


def test_descriptor_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "lelph_gpu.h"
int main(void){
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(lelph_gpu_desc), offsetof(lelph_gpu_desc, alat_vec),
         offsetof(lelph_gpu_desc, npw), offsetof(lelph_gpu_desc, ntype), offsetof(lelph_gpu_desc, precision),
         sizeof(lelph_gpu_stats), offsetof(lelph_gpu_stats, product_grid), offsetof(lelph_gpu_desc, route),
         offsetof(lelph_gpu_stats, route), offsetof(lelph_gpu_stats, gs_plane_ms), offsetof(lelph_gpu_stats, gs_gemm_ms));
  return 0; }
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    D = elph.Desc
    S = elph.Stats
    assert out == [ctypes.sizeof(D), D.alat_vec.offset, D.npw.offset, D.ntype.offset, D.precision.offset,
                   ctypes.sizeof(S), S.product_grid.offset, D.route.offset, S.route.offset, S.gs_plane_ms.offset,
                   S.gs_gemm_ms.offset]


def test_route_constants_match_header():
    import re
    hdr = open(os.path.join(ROOT, "include", "lelph_gpu.h")).read()
    vals = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define LELPH_GPU_ROUTE_(\w+) (\d+)", hdr)}
    assert vals == {"AUTO": elph.ROUTE_AUTO, "REAL": elph.ROUTE_REAL, "GSPACE": elph.ROUTE_GSPACE}


def test_strerror_covers_status_codes():
    lib = elph.load_library(build_library())
    for code in range(0, -8, -1):
        assert lib.lelph_gpu_strerror(code).decode() not in ("", "unknown status")
