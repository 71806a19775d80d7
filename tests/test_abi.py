"""The C-ABI library builds for sm_103a, loads, and exports every entry point of include/*.h.

No compute call is made here (this suite runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**\s*([a-z][a-z0-9_]*)\s*\(", text,
                             flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from rtc8_gb300 import build

    path = build.build()
    return ctypes.CDLL(str(path))


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "vpt_launch_plain" in names and "vpt_create" in names
    assert len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_covers_every_symbol():
    from rtc8_gb300 import _lib

    missing = [n for n in declared_functions() if n not in _lib.EXPORTS]
    assert not missing, f"no ctypes declaration for: {missing}"


def test_library_built_for_sm_103a():
    from rtc8_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in build.ARCH
