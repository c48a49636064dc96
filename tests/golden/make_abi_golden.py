#!/usr/bin/env python3
"""Writes tests/golden/verifier_abi.txt from the reference's own headers:
the layout of gb::RunStats, gb::SegmentStats and gb::RidgeEntry (offset and
size of every member, tests/cpp/abi_probe.cpp compiled against the
reference's include/verifier.hpp and include/sparse_run.hpp) and the mangled
names of gb::run_gpu, gb::print_device_info, gb::verify_cpu and
gb::run_gpu_sparse (the undefined symbols of the probe's object file).

usage: make_abi_golden.py <goldbach-l0 tree>   (or GB_REFERENCE=<tree>)
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
PROBE = os.path.join(os.path.dirname(HERE), "cpp", "abi_probe.cpp")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GB_REFERENCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_abi_golden.py <goldbach-l0 tree> (or GB_REFERENCE=<tree>)")
    inc = os.path.join(ref, "include")
    flags = ["g++", "-std=c++23", "-O0", "-Wno-invalid-offsetof", "-DREF_HEADERS", "-I", inc]
    with tempfile.TemporaryDirectory() as d:
        exe, obj = os.path.join(d, "probe"), os.path.join(d, "probe.o")
        subprocess.run(flags + [PROBE, "-o", exe], check=True)
        layout = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
        subprocess.run(flags + ["-DNAME_CALLS", "-c", PROBE, "-o", obj], check=True)
        nm = subprocess.run(["nm", "-u", obj], check=True, capture_output=True, text=True).stdout
    syms = sorted({ln.split()[-1] for ln in nm.splitlines() if "_ZN2gb" in ln})
    with open(os.path.join(HERE, "verifier_abi.txt"), "w") as f:
        f.write(layout)
        for s in syms:
            f.write(f"symbol {s}\n")


if __name__ == "__main__":
    main()
