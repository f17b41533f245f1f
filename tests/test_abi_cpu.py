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


def test_partials_allocation_covers_kernel_indices():
    """The mixed real-space route's partial sums: for every band count the
    tensor-core tile takes and the mode counts of 1-16 atom cells, the bytes
    the library allocates cover the highest float the sandwich writes and the
    finish reads (host arithmetic of the library itself, no device work).  A
    tile holds whole modes, so 128 % nbnds != 0 needs more tiles than
    ceil(nmodes * nbnds / 128)."""
    lib = elph.load_library(build_library())
    out = (ctypes.c_ulonglong * 3)()
    short = 0
    for nb in range(1, 65):
        for nm in (3, 6, 9, 12, 24, 36, 48):
            for ns, nch, npairs in ((1, 1, 1), (2, 3, 5)):
                assert lib.lelph_gpu_debug_partials_extent(nm, nb, ns, nch, npairs, out) == 0
                alloc, wr, rd = out[0], out[1], out[2]
                assert wr <= alloc and rd <= alloc, (nb, nm, ns, nch, npairs, alloc, wr, rd)
                assert wr == alloc  # the last unit's block ends the buffer exactly
                nbp = (nb + 7) // 8 * 8
                short += alloc > ns * ((nm * nb + 127) // 128) * nch * 128 * 2 * nbp * npairs
    assert short > 0   # shapes where whole-mode tiles need more than ceil(nm nb / 128) tiles exist
    assert lib.lelph_gpu_debug_partials_extent(12, 65, 1, 1, 1, out) != 0


def test_reference_binding_compiles_into_the_reference():
    """The binding a LetzElPhC maintainer compiles in place of
    src/elph/compute_elph_matq.c builds against the reference's own headers in
    both of its precisions and defines the stage's symbol (build() makes these
    objects when the reference sources are at hand)."""
    import platform
    import shutil
    import pytest
    if not shutil.which("nm"):
        pytest.skip("nm is not installed")
    for sub in ("", "-f32"):
        d = os.path.join(ROOT, "oracle", "_ref", platform.machine() + sub)
        obj, exe = os.path.join(d, "binding.o"), os.path.join(d, "lelph_ref_gpu")
        if not os.path.exists(obj):
            pytest.skip("the reference sources were not available to build()")
        syms = subprocess.run(["nm", obj], capture_output=True, text=True, check=True).stdout
        assert re.search(r"\bT compute_and_write_elphq\b", syms)
        assert "lelph_gpu_compute_elphq_star" in syms and "nc_put_vara" in syms
        assert os.access(exe, os.X_OK)
