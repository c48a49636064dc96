"""Sparse class map, host side (no GPU): the residues reach every even class,
the checker plan holds exactly the candidates the geometry allows, each once,
and the device calls fail loudly without a device. Mirrors the reference's
host tests of its sparse path (tests/host_tests.cpp:473-530 residues and
first hits, 734-800 plan validation), against the oracle."""
import ctypes as C
import math
import os
import random
import subprocess

import pytest

import gbc
import sparse_oracle as so
from conftest import ROOT


@pytest.fixture(scope="module")
def plan_ctx():
    with gbc.Sparse(limit=5 * 10**18, host_only=True) as sp:
        yield sp


def test_struct_layout_matches_header(tmp_path):
    prog = tmp_path / "sz.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "gbc.h"\nint main(void){'
                    'printf("%zu %zu %zu %zu\\n", sizeof(gbc_sparse_config), sizeof(gbc_sparse_result), '
                    'offsetof(gbc_sparse_config, host_only), offsetof(gbc_sparse_result, ms_total));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [C.sizeof(gbc.SparseConfig), C.sizeof(gbc.SparseResult), gbc.SparseConfig.host_only.offset,
                   gbc.SparseResult.ms_total.offset]


def test_geometry_and_residues(plan_ctx):
    sp = plan_ctx
    assert (sp.M, sp.K, sp.pmax, sp.dlt) == (30030, 12, 40_000_000, 1 << 26)
    assert sp.tb == -(-sp.pmax // sp.M) + 2
    res = sp.residues
    assert res == sorted(res) and len(set(res)) == 12
    assert all(math.gcd(c, sp.M) == 1 and c % 2 == 1 for c in res)
    assert sorted(c % 3 for c in res) == [1] * 6 + [2] * 6
    assert so.cover_ok(res)
    # every even class reaches at least one class; count those with one only
    single = sum(1 for r in range(0, sp.M, 2) if len(so.usable(r, res)) == 1)
    assert single < sp.M // 2 // 20


def check_plan(sp, r, isp):
    got = sp.plan(r)
    want = so.candidates(r, sp.residues, sp.pmax, isp)
    ps = [p for p, _ in got]
    assert sorted(ps) == sorted(p for p, _ in want), r  # every candidate, each once
    entries = [g for _, g in got]
    assert entries == sorted(entries)
    ks = dict(want)

    def offset(p):
        c = sp.residues[ks[p]]
        return sp.tb - (p - (r - c) % sp.M) // sp.M - (1 if r < c else 0)

    # an entry: one class k and one window word, up to six offsets ascending;
    # consecutive entries of one (k, word) form a group: all but its last
    # entry full, groups fullest first, each (k, word) once
    groups = []
    for e in sorted(set(entries)):
        members = [p for p, g in got if g == e]
        offs = [offset(p) for p in members]
        assert 1 <= len(members) <= 6 and offs == sorted(offs)
        assert len({ks[p] for p in members}) == 1 and len({u // 32 for u in offs}) == 1
        assert all(0 <= u <= sp.tb for u in offs)
        key = (ks[members[0]], offs[0] // 32)
        if groups and groups[-1][0] == key:
            assert groups[-1][1][-1] == 6
            groups[-1][1].append(len(members))
        else:
            groups.append((key, [len(members)]))
    assert len({k for k, _ in groups}) == len(groups)
    sizes = [sum(n) for _, n in groups]
    assert sizes == sorted(sizes, reverse=True)


def test_plan_holds_every_candidate_once(plan_ctx):
    sp = plan_ctx
    isp = so.primes_upto(sp.pmax)
    flags = bytearray(sp.pmax + 1)
    for p in isp.tolist():
        flags[p] = 1
    rnd = random.Random(5)
    classes = [0, 2, sp.M - 2] + [2 * rnd.randrange(sp.M // 2) for _ in range(12)]
    for r in classes:
        check_plan(sp, r, flags)


def test_small_pmax_plan():
    with gbc.Sparse(limit=10**18, pmax=100_000, host_only=True) as sp:
        assert sp.tb == -(-100_000 // sp.M) + 2 == 6
        isp = bytearray(100_001)
        for p in so.primes_upto(100_000).tolist():
            isp[p] = 1
        for r in (0, 2, 4, 6, 1000, 30028):
            check_plan(sp, r, isp)


def test_config_limits():
    for kw in ({"dlt_log2": 11}, {"dlt_log2": 27}, {"pmax": 99_999}, {"pmax": 200_000_001}, {"limit": 10}):
        args = {"limit": 10**18, "host_only": True}
        args.update(kw)
        with pytest.raises(gbc.GbcError) as e:
            gbc.Sparse(**args)
        assert e.value.code == -1


def test_device_calls_fail_loudly_without_a_device(plan_ctx):
    sp = plan_ctx
    with pytest.raises(gbc.GbcError) as e:
        sp.verify(4 * 10**18, 4 * 10**18 + 1000)
    assert e.value.code == -5
    with pytest.raises(gbc.GbcError):
        sp.witness(4 * 10**18, 10)


def test_device_context_fails_loudly_without_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gbc.GbcError) as e:
        gbc.Sparse(limit=10**13)
    assert e.value.code == -2


def test_oracle_sieve_matches_miller_rabin(plan_ctx):
    # the oracle's progression sieve against primality by Miller-Rabin: every
    # bit at 1e12, a random sample at 1e15 (where both sieve stages' prime
    # ranges occur)
    sp = plan_ctx
    n0 = 10**12 - 10**12 % sp.M + 3 * sp.M
    a = so.class_map(n0, 2000, sp.tb, sp.residues)
    b = so.map_by_mr(n0, 2000, sp.tb, sp.residues)
    assert all((x == y).all() for x, y in zip(a, b))
    assert sum(int(x.sum()) for x in a) > 1000
    n0 = 10**15 - 10**15 % sp.M
    rows = so.class_map(n0, 50_000, sp.tb, sp.residues)
    rnd = random.Random(11)
    Q = n0 - sp.M * sp.tb
    import oracle
    for _ in range(4000):
        k = rnd.randrange(sp.K)
        t = rnd.randrange(len(rows[k]))
        assert bool(rows[k][t]) == oracle.is_prime(Q + sp.residues[k] + sp.M * t), (k, t)


def test_largest_pmax_plan():
    # pmax 2e8: window words up to 208 in the entries' 8-bit field; creation
    # validates every entry, and a few classes are checked here in full
    with gbc.Sparse(limit=5 * 10**18, pmax=200_000_000, host_only=True) as sp:
        assert sp.tb == -(-200_000_000 // sp.M) + 2 and sp.tb // 32 < 256
        isp = bytearray(sp.pmax + 1)
        for p in so.primes_upto(sp.pmax).tolist():
            isp[p] = 1
        for r in (0, 30028, 2 * 7001):
            check_plan(sp, r, isp)
