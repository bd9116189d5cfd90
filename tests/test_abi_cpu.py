"""The C-ABI library without a GPU: it loads, exports every entry point that
include/lpma.h declares, and the package refuses to run without it."""
import os
import re
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built_lib():
    import __graft_entry__
    __graft_entry__._load_builder().build()
    return os.path.join(ROOT, "lpma_gb300", "_lpma.so")


def declared_entry_points():
    src = open(os.path.join(ROOT, "include", "lpma.h")).read()
    return sorted(set(re.findall(r"LPMA_API\s+[\w\s\*]+?\b(lpma_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_entry_points()
    for must in ("lpma_create", "lpma_build", "lpma_update", "lpma_update_host", "lpma_csr_view", "lpma_to_csr",
                 "lpma_export_sorted", "lpma_export_layout", "lpma_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    lib = ctypes.CDLL(built_lib)
    for name in declared_entry_points():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lpma_\w+)", out))
    assert set(declared_entry_points()) <= exported
    # nothing but the C ABI is exported
    assert all(n.startswith("lpma_") for n in exported)


def test_python_binding_lists_the_same_entry_points(built_lib):
    from lpma_gb300 import _abi
    assert sorted(_abi.EXPORTS) == declared_entry_points()


def test_status_strings_and_config_without_gpu(built_lib):
    import ctypes
    from lpma_gb300 import _abi
    L = _abi.load()
    assert L.lpma_status_string(0) == b"ok"
    assert L.lpma_status_string(2) == b"invalid key in batch"
    cfg = _abi.LpmaConfig()
    assert L.lpma_config_default(ctypes.byref(cfg)) == 0
    assert cfg.segment_length == 32 and cfg.skip_rule == 1
    assert abs(cfg.density_lower_root - 0.42) < 1e-12 and cfg.density_upper_root == 1.0
    # null handles are rejected, not dereferenced
    assert L.lpma_destroy(None) == 1
    assert L.lpma_update(None, None, None, 0, None, 0, 0, None, None) == 1


def test_package_fails_loudly_without_the_library(tmp_path, built_lib):
    pkg = tmp_path / "lpma_gb300"
    shutil.copytree(os.path.join(ROOT, "lpma_gb300"), pkg,
                    ignore=shutil.ignore_patterns("_lpma.so", "_build", "__pycache__"))
    r = subprocess.run([sys.executable, "-c", "import lpma_gb300"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0
    assert "no CPU fallback" in r.stderr


def test_build_flags_target_sm103a():
    import __graft_entry__
    b = __graft_entry__._load_builder()
    assert "arch=compute_103a,code=sm_103a" in " ".join(b.ARCH)
    assert "-lineinfo" in b.FLAGS


def test_struct_layouts_match_the_header(tmp_path):
    """ctypes mirrors of LpmaConfig / LpmaStats / LpmaRequest have the C layout."""
    import ctypes
    import subprocess
    from lpma_gb300 import _abi
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lpma.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(LpmaConfig), sizeof(LpmaStats),'
                   ' sizeof(LpmaRequest), offsetof(LpmaRequest, stats), offsetof(LpmaRequest, done),'
                   ' offsetof(LpmaRequest, cap));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(_abi.LpmaConfig), ctypes.sizeof(_abi.LpmaStats), ctypes.sizeof(_abi.LpmaRequest),
            _abi.LpmaRequest.stats.offset, _abi.LpmaRequest.done.offset, _abi.LpmaRequest.cap.offset]
    assert got == want
