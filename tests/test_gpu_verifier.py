"""The reference's C++ interface on the GPU: a C++ caller compiled against
include/gb_verifier.hpp (tests/cpp/run_gpu_main.cpp) calls gb::run_gpu with
the reference's signature.

The runs of tests/golden/gstats/ (what the reference's own GoldbachStats
wrote for them, production sampling: merged, adjacent, refused, without
gaps, a gap backfill) and of tests/golden/gstats_gaps/ (statistics-only runs
around the record gaps 1476 and 1442, out of order) go through gb::run_gpu
with the reference's environment knobs; the state file, the gap state and
the log must equal the reference's byte for byte after every run. A window at 1e12 checks the RunStats counts against the
oracle and the per-segment records against the segment plan."""
import os
import subprocess

import pytest

import gbc
import oracle
from conftest import golden_path
from test_stats_campaign import SCENARIOS
from test_verifier_abi import build_main

pytestmark = pytest.mark.gpu

def read(p):
    with open(p, "rb") as f:
        return f.read()


def env_for(tmp_path, **kw):
    e = dict(os.environ, GB_STATS_STATE=str(tmp_path / "goldbach_stats.state"),
             GB_STATS_LOG=str(tmp_path / "goldbach_stats.log"), GB_RIDGE_FILE=str(tmp_path / "ridges.csv"),
             GB_RECORDS_FILE=str(tmp_path / "records.txt"), GB_STATS_LIVE=str(tmp_path / "live.json"),
             GB_RECORD_HOOK="")
    e.update(kw)
    return e


def kv(out):
    return dict(ln.split("=", 1) for ln in out.splitlines() if "=" in ln and not ln.startswith("ridge="))


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_run_gpu_statistics_files_equal_the_references(tmp_path, name):
    every, seg, runs, _ = SCENARIOS[name]
    exe = build_main(tmp_path)
    for i, (g, a, b) in enumerate(runs, 1):
        env = env_for(tmp_path, GB_STATS_SAMPLE=str(every), GB_GAPS="exact" if g else "0")
        r = subprocess.run([exe, str(b), str(seg), str(a), "0"], env=env, cwd=tmp_path, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert kv(r.stdout)["stats_on"] == "1"
        assert read(tmp_path / "goldbach_stats.state") == read(golden_path(f"{name}/after{i}.state")), i
        gp = golden_path(f"{name}/after{i}.gaps")
        if os.path.exists(gp):
            assert read(tmp_path / "goldbach_stats.state.gaps") == read(gp), i
    assert read(tmp_path / "goldbach_stats.log") == read(golden_path(f"{name}/goldbach_stats.log"))


def test_run_gpu_counts_and_per_segment_records(tmp_path):
    a, b, seg = 10**12, 10**12 + 20_000_000, 4_000_000
    exe = build_main(tmp_path)
    r = subprocess.run([exe, str(b), str(seg), str(a), "1"], env=env_for(tmp_path, GB_STATS_SAMPLE="1"), cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = kv(r.stdout)
    want = dict(t.split("=", 1) for t in oracle.stats_line(a, b, oracle.SIEVE).split())
    assert (got["stats_primes"], got["stats_twins"], got["stats_pmax"]) == (want["primes"], want["twins"], want["pmax"])
    segs = gbc.segments_of(a, b, seg)
    assert int(got["segments"]) == int(got["per_segment"]) == len(segs)
    assert int(got["per_segment_evens"]) == (b - a) // 2 + 1 == int(got["stats_sampled"])
    assert int(got["leftovers"]) == 0 and float(got["gpu_seconds"]) > 0


def test_print_device_info(tmp_path):
    exe = build_main(tmp_path)
    r = subprocess.run([exe, "--device-info"], capture_output=True, text=True)
    assert r.returncode == 0 and "device" in r.stdout and "multiprocessors" in r.stdout
