"""The C-ABI library loads and exports every symbol include/sparc_gpu.h declares (CPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sgpu_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_header_and_python_mirror_agree():
    import sparc_gb300
    assert declared_symbols() == sorted(sparc_gb300.EXPORTED)


def test_library_exports_every_declared_symbol():
    import sparc_gb300
    if not os.path.exists(sparc_gb300.LIB_PATH):
        from sparc_gb300 import build
        build.build()
    lib = sparc_gb300.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    import sparc_gb300
    monkeypatch.setattr(sparc_gb300, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(sparc_gb300, "_lib", None)
    with pytest.raises(sparc_gb300.SgpuError):
        sparc_gb300.lib()


def test_host_modules_import():
    """Every host-side module of the package and the bench import on a machine without a GPU."""
    import importlib
    for mod in ("sparc_gb300.setup", "sparc_gb300.psp8", "sparc_gb300.learned_density",
                "sparc_gb300.synthetic"):
        importlib.import_module(mod)
    import py_compile
    for fn in ("bench.py", "__graft_entry__.py"):
        py_compile.compile(os.path.join(ROOT, fn), doraise=True)


def test_python_mirror_constants_match_header():
    import sparc_gb300
    txt = open(os.path.join(ROOT, "include", "sparc_gpu.h")).read()
    n = int(re.search(r"#define SGPU_STENCIL_VARIANTS (\d+)", txt).group(1))
    assert sparc_gb300.STENCIL_VARIANTS == n
