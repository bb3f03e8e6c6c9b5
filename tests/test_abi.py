"""The C-ABI library loads and exports every function include/openph.h
declares (no GPU needed: nothing is called)."""
import ctypes
import re
from pathlib import Path

HEADER = Path(__file__).resolve().parents[1] / "include" / "openph.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while")))


def test_header_declares_the_dropin():
    names = declared_functions()
    assert "openph" in names and "oph_openph" in names and "oph_reduce" in names


def test_library_exports_every_declared_symbol(cuda_lib):
    lib = ctypes.CDLL(str(Path(cuda_lib._name)))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_algorithm_strings(cuda_lib):
    for i, name in enumerate(["standard", "twist", "ph_row", "standard_parallel", "twist_parallel",
                              "ph_row_parallel", "pms"]):
        assert cuda_lib.oph_algo_from_string(name.encode()) == i
    assert cuda_lib.oph_algo_from_string(b"spectral") == -1
    assert cuda_lib.oph_status_string(3) == b"column store cannot grow any further"
