"""The C++ boundary at run time: a C++ program compiled against include/psr/
PoissonReconstruction.hpp, include/psr/Server.hpp and libpsr.so reconstructs a coloured cloud
given as the reference's 64-byte DepthSurfel records on the device (the reference's
SolvePoissionReconstructionMesh(DeviceArrayView<DepthSurfel>) call,
mesh/PoissonReconstruction.h:124), then serves it twice through the header-only Server.
Its mesh, colours and normals must equal the Python path's bit for bit."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import synthetic as syn

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "poisson-surface-reconstruction-gpu_gb300"


def test_cpp_shim_and_server_match_python(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    import psr
    psr.load_library()   # built
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    libdirs = [d for d in (cuda / "lib64", cuda / "lib") if (d / "libcudart.so").exists()]
    exe = tmp_path / "shim_main"
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(ROOT / "tests" / "cpp" / "shim_main.cpp"), "-o", str(exe), "-L", str(PKG), "-lpsr",
           f"-Wl,-rpath,{PKG}"]
    for d in libdirs:
        cmd += ["-L", str(d), f"-Wl,-rpath,{d}"]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    p, nr, rgb, _ = syn.workload("mix", cloud=0, colour=True)
    n = p.shape[0]
    cloud = tmp_path / "cloud.bin"
    with open(cloud, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.ascontiguousarray(p, np.float32).tobytes())
        f.write(np.ascontiguousarray(nr, np.float32).tobytes())
        f.write(np.ascontiguousarray(rgb, np.uint8).tobytes())
    out = tmp_path / "mesh.bin"
    r = subprocess.run([str(exe), str(cloud), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
    b = out.read_bytes()
    nv, nt = np.frombuffer(b[:8], np.int32)
    off = 8
    V = np.frombuffer(b[off:off + 12 * nv], np.float32).reshape(-1, 3); off += 12 * nv
    T = np.frombuffer(b[off:off + 12 * nt], np.int32).reshape(-1, 3); off += 12 * nt
    C = np.frombuffer(b[off:off + 12 * nv], np.float32).reshape(-1, 3); off += 12 * nv
    N = np.frombuffer(b[off:off + 12 * nv], np.float32).reshape(-1, 3)
    with psr.PoissonReconstruction(max_depth=7, max_points=n, compute_colors=True, compute_normals=True) as rec:
        m = rec.SolvePoissionReconstructionMesh(p, nr, rgb, depth=7)
    np.testing.assert_array_equal(V, m.vertices)
    np.testing.assert_array_equal(T, m.triangles)
    np.testing.assert_array_equal(C, m.colors)
    np.testing.assert_array_equal(N, m.normals)
