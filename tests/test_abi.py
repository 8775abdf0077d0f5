"""The C ABI: the library loads without a GPU and exports every function
include/cvl_gb300.h declares, which are exactly the prototypes of the
reference's cvl.h plus the gcvl_* extensions."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w ]*?[\s\*]+)(\w+)\s*\([^;{]*\)\s*;", txt, re.M):
            names.add(m.group(1))
    return names


def test_header_matches_reference_abi():
    from neslgpu_gb300 import abi
    declared = _declared()
    missing = set(abi.CVL) - declared
    assert not missing, f"cvl.h functions not declared: {sorted(missing)[:20]}"
    assert set(abi.EXTENSIONS) <= declared


def test_library_exports_every_declared_symbol():
    import ctypes
    from neslgpu_gb300.cvl import LIB_PATH
    assert LIB_PATH.exists(), "build the library first"
    lib = ctypes.CDLL(str(LIB_PATH))
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_host_side_functions_without_gpu():
    """Size, scratch, in-place and pointer arithmetic need no device."""
    from neslgpu_gb300.cvl import load
    c = load()
    # 8-byte units, rounded to even: vinterp's heap then keeps vectors 16-byte aligned
    assert c.siz_foz(3) == 2 and c.siz_fob(3) == 2 and c.siz_fod(3) == 4 and c.siz_fod(4) == 4
    assert c.siz_foz(1) == 2 and c.siz_fod(0) == 0
    assert all(c.siz_foz(k) % 2 == 0 and c.siz_fod(k) % 2 == 0 and c.siz_fos(k, k // 3) % 2 == 0
               for k in range(0, 200, 7))
    assert c.siz_fos(100, 10) >= c.siz_foz(10)
    assert c.add_fov(1000, 3) == 1024 and c.sub_fov(1024, 1000) == 3
    assert c.cmp_fov(1000, 1024) == -3 and c.eql_fov(8, 8) == 1
    assert c.add_sez_scratch(1 << 20, 100) > 0
    assert c.add_sez_inplace() == 1
    assert c.rku_luz_scratch(1 << 20) > 0 and c.rku_lez_scratch(1 << 20, 5) > c.rku_luz_scratch(1 << 20)
    assert c.mke_fov_inplace() == 0


def _lookback_bytes(tiles):
    # the look-back area a scan kernel carves from its scratch: 512 bytes of
    # counter and alignment slack, then 16 bytes per tile rounded to 256
    return 512 + -(-tiles * 16 // 256) * 256


def test_scratch_covers_the_kernels_tiles():
    """Every scan's scratch holds the look-back area of the persistent ring
    (tiles of 64 rows of 128 bytes: 1024 doubles or 2048 ints), and every
    segmented float64 +-reduction's holds the TMA kernel's area, its per-tile
    list of results to complete and the second pass's look-back (tiles of
    128 rows); the fused SpMV's the same for its 2048-element tiles."""
    from neslgpu_gb300.cvl import load
    c = load()
    for n in (1, 1000, 1 << 16, (1 << 20) + 7, 1 << 28):
        for m in (1, max(1, n // 64)):
            assert 8 * c.add_sed_scratch(n, m) >= _lookback_bytes(-(-n // 1024)), (n, m)
            assert 8 * c.add_sez_scratch(n, m) >= _lookback_bytes(-(-n // 2048)), (n, m)
            assert 8 * c.add_sud_scratch(n) >= _lookback_bytes(-(-n // 1024)), n
            t = -(-n // 2048)
            red = _lookback_bytes(t) + -(-t * 4 // 256) * 256 + _lookback_bytes(-(-t // 1024))
            assert 8 * c.add_red_scratch(n, m) >= red, (n, m)
            assert 8 * c.gcvl_spmv_csr_scratch(n, m) >= red, (n, m)
