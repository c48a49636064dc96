"""The C ABI library without a GPU: it loads, exports every entry point
include/gbc.h declares, its structs have the layout the header gives, its
host-only functions work, and it fails loudly (an error code and text, no
fallback) when no GPU is there."""
import ctypes as C
import os
import re
import subprocess

import pytest

import gbc
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gbc.h")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(gbc.LIB_PATH):
        subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "goldbach-l0_gb300")], check=True)
    return gbc.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbc_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(gbc.SIGNATURES)


def test_struct_layout_matches_header(tmp_path):
    prog = tmp_path / "sz.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "gbc.h"\nint main(void){'
                    'printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gbc_config), sizeof(gbc_segment_result), '
                    'sizeof(gbc_batch_times), sizeof(gbc_run_result), offsetof(gbc_segment_result, first), '
                    'offsetof(gbc_segment_result, primes30), offsetof(gbc_segment_result, map_hash), '
                    'offsetof(gbc_segment_result, err));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    R = gbc.SegmentResult
    want = [C.sizeof(gbc.Config), C.sizeof(R), C.sizeof(gbc.BatchTimes), C.sizeof(gbc.RunResult),
            R.first.offset, R.primes30.offset, R.map_hash.offset, R.err.offset]
    assert got == want


def test_candidates(lib):
    c = gbc.candidates()
    assert len(c) == gbc.NCAND == 1205
    assert c[0] == 3 and c[-1] == 9781
    assert all(all(p % d for d in range(3, int(p ** 0.5) + 1, 2)) for p in c)


def test_segment_plan():
    s = gbc.segments_of(4, 200000, 100000)
    assert s[0] == (4, 65538) and s[-1][1] == 200000
    assert all(b[0] == a[1] + 2 for a, b in zip(s, s[1:]))
    s = gbc.segments_of(10**12, 10**12 + 10**6, 300000)
    assert s == [(10**12, 10**12 + 299998), (10**12 + 300000, 10**12 + 599998),
                 (10**12 + 600000, 10**12 + 899998), (10**12 + 900000, 10**12 + 10**6)]


def test_create_fails_loudly_without_a_gpu(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gbc.GbcError) as e:
        gbc.Context(limit=10**9, segment_even=10**6)
    assert e.value.code == -2


def test_bad_config_is_refused(lib):
    with pytest.raises(gbc.GbcError) as e:
        gbc.Context(limit=2**64 - 1)
    assert e.value.code == -1


def test_cli_usage_errors():
    exe = os.path.join(ROOT, "goldbach-l0_gb300", "bin", "goldbach_gb300")
    if not os.path.exists(exe):
        pytest.skip("CLI not built")
    assert subprocess.run([exe], capture_output=True).returncode == 2
    assert subprocess.run([exe, "--limit", "12x"], capture_output=True).returncode == 2
    assert subprocess.run([exe, "--start", "100", "--limit", "50"], capture_output=True).returncode == 2
    assert subprocess.run([exe, "--limit", "1.9e19"], capture_output=True).returncode == 2   # above 2^64
    assert subprocess.run([exe, "--limit", "18446743e12"], capture_output=True).returncode == 1  # > 2^64 - 2^40
    # the sparse path: the same limit check before any GPU work; no statistics
    r = subprocess.run([exe, "--start", "18446742974197000000", "--limit", "18446744073709551614", "--sparse"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "supported maximum" in r.stderr and "PASS" not in r.stdout
    assert subprocess.run([exe, "--limit", "1e12", "--sparse", "--stats"], capture_output=True).returncode == 2


def test_probe_library_is_separate_and_exports_its_header():
    """The measurement probe lives in libgbc_probe.so, not in the product
    library, and exports what include/gbc_probe.h declares."""
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "gbc_probe.h")).read(), flags=re.S)
    names = sorted(set(re.findall(r"\b(gbc_\w+)\s*\(", src)))
    assert names == ["gbc_smem_atomic_peak"]
    probe = gbc.load_probe()
    assert all(hasattr(probe, n) for n in names)
    out = subprocess.run(["nm", "-D", "--defined-only", gbc.LIB_PATH], capture_output=True, text=True).stdout
    assert "gbc_smem_atomic_peak" not in out


def test_smem_atomic_probe_fails_loudly_without_a_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gbc.GbcError):
        gbc.smem_atomic_peak()


def test_cli_crosscheck_status(tmp_path):
    # ci/sparse_crosscheck.sh status: both journals' PASS chains from start
    exe = os.path.join(ROOT, "goldbach-l0_gb300", "bin", "goldbach_gb300")
    if not os.path.exists(exe):
        pytest.skip("CLI not built")
    d, s = tmp_path / "dense.journal", tmp_path / "sparse.journal"
    d.write_text("PASS 1000 1998 t version=x\nPASS 2000 2998 t version=x\n")
    s.write_text("PASS 1000 1998 t version=x path=sparse\nRETRY 2000 2998 t reason=-3\n")
    r = subprocess.run([exe, "--start", "1000", "--limit", "9998", "--crosscheck-status", str(d), str(s)],
                       capture_output=True, text=True)
    assert r.returncode == 0
    lines = r.stdout.splitlines()
    assert lines[0].endswith("verified [1000, 2998]") and lines[1].endswith("verified [1000, 1998]")
    assert lines[2].startswith("both:   [1000, 1998] = 500 evens")


def test_binding_constants_equal_the_headers():
    """Every constant the ctypes binding mirrors has the value the header
    defines (GBC_X in include/gbc.h <-> gbc.X)."""
    src = open(HEADER).read()
    defs = {}
    for name, val in re.findall(r"^#define GBC_(\w+)\s+\(?(-?(?:0x[0-9A-Fa-f]+|\d+))[uUlL]*\)?", src, flags=re.M):
        defs[name] = int(val, 0)
    mirrored = ["NCAND", "NCLASS", "GBINS", "TAIL_CAP", "LEFT_CAP", "RIDGE_CAP", "TAIL_T", "DEFAULT_SEGMENT",
                "MAX_LIMIT", "SEG_NOHASH", "SEG_VERIFY", "SAMPLE_NONE", "TEST_STAGING_WAIT", "TEST_RETRY_LIMIT",
                "MAX_SLOTS"]
    for name in mirrored:
        assert name in defs, name
        assert getattr(gbc, name) == defs[name], name
