"""Host-side helpers of bench.py that the reported numbers depend on."""
import pytest


def test_piece_count_follows_the_tiling_rule():
    import bench
    # 1024^3 on 152 SMs: 34 x 256 warp tiles per z segment, 2 segments of 512 cells
    assert bench.pieces(1024, 1024, 1024, 152) == 2 * 1023 * 1023
    # 64^3: 3 x 16 tiles, as many 8-cell segments as there are chunks
    assert bench.pieces(64, 64, 64, 152) == 8 * 63 * 63
    # one z segment when the x-y tiles alone fill the GPU
    assert bench.pieces(4096, 4096, 9, 152) == 4095 * 4095


def test_whole_job_rate_and_spread():
    import bench
    assert bench.whole_job_rate(10, 1, 2.0) == pytest.approx(5000.0)
    s = bench._spread([3.0, 1.0, 2.0, 10.0])
    assert (s['min'], s['median'], s['max']) == (1.0, 3.0, 10.0)
    assert s['mean'] == pytest.approx(4.0)
    assert bench._spread([]) is None


def test_reference_arm_prints_the_contract_line():
    # the reference arm runs on the host cores alone: a small field, one line
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, 'bench.py'), '--impl', 'reference', '--n', '96',
                          '--steps', '2', '--warmup', '1', '--cpu-planes', '8'],
                         check=True, capture_output=True, text=True, cwd=root, timeout=300)
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference' and d['unit'] == 'Gvoxels/s' and d['higher_is_better'] is True
    assert d['value'] > 0 and d['steps'] == 2 and d['warmup'] == 1 and d['n_gpus'] == 1
    assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['cores'] == 1
    assert d['cpu_baseline']['value'] == d['value']
    assert d['e2e'] == {'value': d['value'], 'unit': 'Gvoxels/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
    assert d['config']['sample_planes'] == 9
