"""C ABI checks that need no GPU: the library loads and exports every declared entry."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "psr" / "psr.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:psr_status|const char\*)\s+(psr_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import psr
    if not psr.LIB_PATH.exists():
        import build
        build.build()
    return ctypes.CDLL(str(psr.LIB_PATH))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n


def test_python_mirror_covers_header():
    import psr
    assert sorted(psr.EXPORTED) == declared_functions()


def test_config_defaults_without_gpu(lib):
    import psr
    cfg = psr.PsrConfig()
    lib.psr_config_default.argtypes = [ctypes.POINTER(psr.PsrConfig)]
    assert lib.psr_config_default(ctypes.byref(cfg)) == 0
    # reference compile-time caps (base/GlobalConfigs.h:7-8,34)
    assert cfg.max_depth == 7 and cfg.max_points == 300000 and cfg.max_triangles == 1000000
    assert abs(cfg.bbox_scale - 1.25) < 1e-7 and cfg.cg_max_iterations == 10000
    assert cfg.laplacian_epsilon == ctypes.c_float(1e-6).value and cfg.concurrent_stages == 1
    lib.psr_status_string.restype = ctypes.c_char_p
    assert lib.psr_status_string(1) == b"out of capacity"


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler gives the header."""
    import shutil
    import subprocess
    import psr
    assert ctypes.sizeof(psr.PsrConfig) == 21 * 4
    assert ctypes.sizeof(psr.PsrPoints) == 32
    assert ctypes.sizeof(psr.PsrOptions) == 8
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    mirrors = {"psr_config": psr.PsrConfig, "psr_points": psr.PsrPoints, "psr_options": psr.PsrOptions,
               "psr_mesh": psr.PsrMesh, "psr_stats": psr.PsrStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "psr/psr.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname}.{f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for cname, py in mirrors.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert int(got[f"{cname}.{f[0]}"]) == getattr(py, f[0]).offset, (cname, f[0])


def test_cpp_shim_compiles(tmp_path):
    """The header-only C++ shim (reference class and method names) compiles against psr.h."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "shim.cpp"
    src.write_text('#include "psr/PoissonReconstruction.hpp"\n#include "psr/Server.hpp"\n'
                   'int main() { psr_gb300::PoissonReconstruction* p = nullptr; (void)p; return 0; }\n')
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), "-I", cuda_inc, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
