"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/*.h declares (no compute calls: these run without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(spg_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    d = _declared()
    for must in ("spg_create", "spg_tile_from_csr", "spg_symbolic", "spg_numeric", "spg_spgemm"):
        assert must in d


@pytest.fixture(scope="module")
def lib():
    from gpu_spgemm_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from gpu_spgemm_gb300 import _lib
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)


def test_binding_struct_layout_matches_header():
    # field order/types of spg_tiles / spg_ctiles mirror the header
    from gpu_spgemm_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "spgemm_gb300.h")).read()
    body = src[src.index("typedef struct {\n    int m, n;\n    int64_t nnz;"):src.index("} spg_tiles;")]
    fields = re.findall(r"\*?\s*(\w+);", re.sub(r"/\*.*?\*/", "", body, flags=re.S))
    flat = []
    for line in re.sub(r"/\*.*?\*/", "", body, flags=re.S).splitlines()[1:]:
        line = line.strip().rstrip(";")
        if not line:
            continue
        decl = line.split(None, 1)[1] if " " in line else line
        flat += [x.strip().lstrip("*") for x in decl.split(",")]
    assert [f for f, _ in _lib.SpgTiles._fields_] == flat, (flat, fields)


def test_stats_layout_matches_header():
    from gpu_spgemm_gb300 import _lib
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "spgemm_gb300.h")).read(), flags=re.S)
    body = src[src.index("typedef struct {\n    float ms_step1;"):src.index("} spg_stats;")]
    names = re.findall(r"^\s*\w+\s+(\w+);", body, flags=re.M)
    assert [f for f, _ in _lib.SpgStats._fields_] == names, names


def test_missing_library_fails_loudly(tmp_path):
    from gpu_spgemm_gb300 import _lib
    with pytest.raises(RuntimeError):
        _lib.load.__wrapped__(str(tmp_path / "nope.so")) if hasattr(_lib.load, "__wrapped__") else \
            _lib_load_fresh(str(tmp_path / "nope.so"))


def _lib_load_fresh(path):
    from gpu_spgemm_gb300 import _lib
    saved = _lib._lib
    _lib._lib = None
    try:
        return _lib.load(path)
    finally:
        _lib._lib = saved


def test_enum_values_match_header():
    """Every SPG_* constant the header defines (enums and #defines) has the
    same value in the ctypes binding."""
    from gpu_spgemm_gb300 import _lib as L
    src = open(os.path.join(ROOT, "include", "spgemm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    num = r"(-?(?:0[xX][0-9a-fA-F]+|\d+))"
    found = {m.group(1): int(m.group(2), 0) for m in re.finditer(r"\b(SPG_[A-Z0-9_]+)\s*=\s*" + num, src)}
    found.update({m.group(1): int(m.group(2), 0)
                  for m in re.finditer(r"#define\s+(SPG_[A-Z0-9_]+)\s+\(?" + num, src)})
    assert len(found) >= 20, found
    for name, value in found.items():
        assert getattr(L, name) == value, name
