"""Per-device one-time set-up (lpma_gb300/csrc/per_device.h), without a GPU.

The sort kernels' shared-memory opt-ins, the cooperative sort's occupancy
and the fixed-scratch shuffle's device address are kept per device: a
process that makes a second device current must run the set-up again for
it.  The bookkeeping is host-only C++, compiled here with g++ against a
fake device id, so it is tested on the CPU.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "per_device.h"
using namespace lpma;
struct Occ { unsigned n[4]; };
static int calls[MAX_DEVICES];
static int fail_next[MAX_DEVICES];
static int setup(int dev, Occ &v) {
    calls[dev]++;
    if (fail_next[dev]) { fail_next[dev] = 0; return 77; }
    for (int i = 0; i < 4; i++) v.n[i] = 100u * (unsigned)dev + (unsigned)i;
    return 0;
}
#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s line %d\n", #c, __LINE__); return 1; } } while (0)
int main() {
    PerDevice<Occ> pd;
    const Occ *o = nullptr;
    CHECK(pd.peek(0) == nullptr);
    CHECK(pd.get(0, setup, &o, -5) == 0 && o && o->n[1] == 1 && calls[0] == 1);
    CHECK(pd.get(0, setup, &o, -5) == 0 && calls[0] == 1);          // once per device
    CHECK(pd.peek(1) == nullptr);                                      // a second device is not set up
    CHECK(pd.get(1, setup, &o, -5) == 0 && o->n[3] == 103 && calls[1] == 1);
    CHECK(pd.peek(0)->n[0] == 0 && pd.peek(1)->n[0] == 100);          // values kept apart
    fail_next[2] = 1;
    CHECK(pd.get(2, setup, &o, -5) == 77 && pd.peek(2) == nullptr);    // a failure is not recorded
    CHECK(pd.get(2, setup, &o, -5) == 0 && calls[2] == 2 && o->n[2] == 202);  // and is retried
    CHECK(pd.get(-1, setup, &o, -5) == -5 && pd.get(MAX_DEVICES, setup, &o, -5) == -5);
    CHECK(pd.peek(MAX_DEVICES) == nullptr);
    std::printf("ok\n");
    return 0;
}
"""


def test_per_device_setup_runs_once_per_device(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "pd.cpp"
    exe = tmp_path / "pd"
    src.write_text(PROGRAM)
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "lpma_gb300", "csrc"),
                           str(src), "-o", str(exe), "-lpthread"])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr


def test_library_keeps_sort_setup_per_device():
    """No process-wide 'done' flag is left in the sort set-up, and both
    users of device-specific state go through the per-device table."""
    prims = open(os.path.join(ROOT, "lpma_gb300", "csrc", "prims.cu")).read()
    noalloc = open(os.path.join(ROOT, "lpma_gb300", "csrc", "noalloc.cu")).read()
    assert "static bool done" not in prims
    assert "PerDevice<CoopCtas>" in prims and "PerDevice<unsigned char *>" in noalloc
