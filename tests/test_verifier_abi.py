"""The reference's C++ interface on libgbc.so (include/gb_verifier.hpp),
without a GPU: the structs have the reference's layout and the library
exports the reference's mangled entry points (tests/golden/verifier_abi.txt,
written from the reference's own headers by make_abi_golden.py), and a C++
caller compiled against the header links and runs (the CPU check)."""
import os
import subprocess

import pytest

import gbc
from conftest import ROOT, golden_path

PROBE = os.path.join(ROOT, "tests", "cpp", "abi_probe.cpp")
MAIN = os.path.join(ROOT, "tests", "cpp", "run_gpu_main.cpp")
INC = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "goldbach-l0_gb300")


def fixture():
    layout, syms = [], []
    with open(golden_path("verifier_abi.txt")) as f:
        for ln in f:
            (syms if ln.startswith("symbol ") else layout).append(ln.rstrip("\n"))
    return layout, [s.split()[1] for s in syms]


def build_main(tmp_path):
    """tests/cpp/run_gpu_main.cpp against include/gb_verifier.hpp, linked with libgbc.so."""
    gbc.load()
    exe = tmp_path / "run_gpu_main"
    subprocess.run(["g++", "-std=c++23", "-O2", "-I", INC, MAIN, "-o", str(exe), "-L", PKG, "-lgbc",
                    f"-Wl,-rpath,{PKG}"], check=True)
    return str(exe)


def test_struct_layouts_equal_the_references(tmp_path):
    want, _ = fixture()
    exe = tmp_path / "probe"
    subprocess.run(["g++", "-std=c++23", "-Wno-invalid-offsetof", "-I", INC, PROBE, "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    assert got == want


def test_library_exports_the_references_entry_points(tmp_path):
    _, want = fixture()
    obj = tmp_path / "probe.o"
    subprocess.run(["g++", "-std=c++23", "-Wno-invalid-offsetof", "-DNAME_CALLS", "-I", INC, "-c", PROBE, "-o",
                    str(obj)], check=True)
    nm = subprocess.run(["nm", "-u", str(obj)], check=True, capture_output=True, text=True).stdout
    assert sorted({ln.split()[-1] for ln in nm.splitlines() if "_ZN2gb" in ln}) == want
    gbc.load()
    exported = subprocess.run(["nm", "-D", "--defined-only", gbc.LIB_PATH], check=True, capture_output=True,
                              text=True).stdout
    for s in want:
        assert f" T {s}" in exported, s


def test_cpu_check_through_the_cpp_interface(tmp_path):
    exe = build_main(tmp_path)
    assert subprocess.run([exe, "--cpu-check", "20000"]).returncode == 0


def test_run_gpu_fails_closed_without_a_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = build_main(tmp_path)
    r = subprocess.run([exe, "1000000000", "0", "999000000", "0"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "FAIL" in r.stderr and "limit=" not in r.stdout
