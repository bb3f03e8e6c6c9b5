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


def _header_constants():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {k: int(v) for k, v in re.findall(r"#define\s+(OPH_[A-Z0-9_]+)\s+(-?\d+)\b", text)}
    out.update({k: int(v) for k, v in re.findall(r"\b(OPH_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)})
    return out


def test_python_constants_match_the_header():
    from openph_gb300 import api
    c = _header_constants()
    for name in ("OPH_OK", "OPH_ERR_BAD_INPUT", "OPH_ERR_OOM", "OPH_ERR_OVERFLOW", "OPH_ERR_TIMEOUT", "OPH_ERR_CUDA",
                 "OPH_ERR_ALGO", "OPH_DUAL_AUTO", "OPH_DUAL_NEVER", "OPH_DUAL_ALWAYS"):
        assert getattr(api, name) == c[name], name


def test_python_structs_match_the_c_layout(tmp_path):
    """sizeof and field offsets of the structs the Python binding mirrors,
    from a C probe compiled against the header."""
    import shutil
    import subprocess
    import pytest
    from openph_gb300 import api
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    mirrors = {"oph_info": api.Info, "oph_profile": api.Profile, "oph_request_info": api.RequestInfo,
               "oph_server_counters": api.ServerCounters}
    text = HEADER.read_text()
    mirrors = {k: v for k, v in mirrors.items() if re.search(r"\}\s*%s\s*;" % k, text)}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "openph.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, val = ln.split()
        got[(cname, field)] = int(val)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
