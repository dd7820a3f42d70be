"""The Naive Surface Nets mean divides each coordinate sum by the cell's
crossing count n (1..12).  The CUDA kernel replaces that Float64 / Float32
division by one product and two fused operations with a correctly rounded
1/n (div_count in meshing.jl_gb300/csrc/k_emit_halo.cu) and claims the result
equals the IEEE quotient bit for bit, the oracle's a / n.  count_division.c
restates those operations in the host's IEEE arithmetic (C99 fma) and
compares them with a / n over random values of every magnitude, quotients
next to rounding midpoints, powers of two, the fallback thresholds, zeros,
infinities and NaN; the GPU parity tests then compare the kernel's vertices
with the oracle's.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_count_division_equals_the_ieee_quotient(tmp_path):
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    exe = str(tmp_path / 'count_division')
    subprocess.run([cc, '-O2', '-std=c99', '-ffp-contract=off', '-o', exe, os.path.join(HERE, 'count_division.c'),
                    '-lm'], check=True)
    out = subprocess.run([exe, '200000'], check=True, capture_output=True, text=True)
    bad_d, bad_f, cases = (int(x) for x in out.stdout.split())
    assert cases > 20_000_000
    assert (bad_d, bad_f) == (0, 0), out.stderr
