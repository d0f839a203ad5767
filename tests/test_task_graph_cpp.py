"""Host invariants of the device task graph (no GPU): compiles
tests/cpp/task_graph_check.cpp against the package's C++ sources and the
built library and runs it. It checks dependency counts and successor lists,
the FP64 four-part items, the product+LU merging of the mixed path (same
outputs as the absorbed LU tasks), that ordering pairs by readiness only
permutes each product's pairs, and that the static claim order puts every
producer before its consumers."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG_DIR, ROOT, build_native


def test_task_graph_invariants(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    lib = build_native()
    exe = str(tmp_path / "task_graph_check")
    src = os.path.join(ROOT, "tests", "cpp", "task_graph_check.cpp")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", f"-I{os.path.join(PKG_DIR, 'csrc')}",
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(cuda, 'include')}", src,
           f"-L{os.path.dirname(lib)}", "-lsoglu_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-4000:] + r.stderr[-2000:]
