"""The shipped launch-shape table (chroma_gb300/tune/default.tunecache), checked on the CPU: every
entry is well formed, names a shape of the compiled candidate table (kHopShapes in
chroma_gb300/csrc/gbc_kernels.h) and carries that table's FNV-1a hash, so a change of the candidate
shapes cannot leave a stale table behind silently (its entries would stop matching and the solves
would fall back to timing); and it covers the stencil variants of the benchmark's propagator solve
(FP16 12-RHS operator, FP32 Schur prep and reliable updates, FP64 and double-float outer steps on
32^3 x 64)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE = os.path.join(ROOT, "chroma_gb300", "tune", "default.tunecache")


def compiled_shapes():
    src = open(os.path.join(ROOT, "chroma_gb300", "csrc", "gbc_kernels.h")).read()
    body = re.search(r"kHopShapes\[\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    return [tuple(int(x) for x in t) for t in re.findall(r"\{\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\s*\}", body)]


def fnv1a(shapes):
    h = 2166136261
    for s in shapes:
        for v in s:
            h ^= v
            h = (h * 16777619) & 0xFFFFFFFF
    return h


def entries():
    if not os.path.exists(TABLE):
        pytest.skip("no shipped tune table")
    out = {}
    for line in open(TABLE):
        key, *vals = line.split()
        out[key] = tuple(int(v) for v in vals)
    return out


def test_entries_match_the_compiled_shapes():
    shapes = compiled_shapes()
    assert len(shapes) == 16
    h = f"{fnv1a(shapes):08x}"
    table = entries()
    assert table
    pat = re.compile(r"^[^|]+\|cc\d+\|\d+x\d+x\d+x\d+\|prec=(2|4|8|16)\|recon=(12|18)\|mode=[012]\|dag=[01]\|"
                     r"reduce=[0123]\|nrhs=\d+\|shapes=([0-9a-f]{8})$")
    for key, shape in table.items():
        m = pat.match(key)
        assert m, key
        assert m.group(3) == h, (key, h)
        assert shape in shapes, (key, shape)


def test_table_covers_the_propagator_solve():
    table = entries()
    lat = [k for k in table if "|32x32x32x64|" in k]
    have = {tuple(re.search(p, k).group(1) for p in (r"prec=(\d+)", r"mode=(\d)", r"nrhs=(\d+)")) for k in lat}
    # FP16 operator; double-float intermediate residual (PLAIN, XPAY) and M~ (CLOV); FP64
    # reconstruction and final residual; FP32 Schur prep (PLAIN) and reliable updates (CLOV, XPAY)
    for want in [("2", "1", "12"), ("2", "2", "12"), ("16", "1", "12"), ("16", "2", "12"), ("16", "0", "12"),
                 ("8", "0", "12"), ("8", "2", "12"), ("4", "0", "12"), ("4", "1", "12"), ("4", "2", "12")]:
        assert want in have, want
    # the BiCGStab launches with fused reductions: (t, s), (t, t) and (r0, v)
    assert any("|32x32x32x64|prec=2|" in k and "|reduce=2|nrhs=12|" in k for k in lat)
    assert any("|32x32x32x64|prec=2|" in k and "|reduce=3|nrhs=12|" in k for k in lat)
