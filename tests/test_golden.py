"""The committed golden fixtures (tests/golden/, written by make_golden.py):
their integrity, and the CPU oracle reproducing every one of them bit for bit.
The CUDA path is checked against the same fixtures in test_gpu_parity.py."""
import hashlib
import json
import os

import numpy as np
import pytest

import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _unscalar(d):
    return {'Float32': np.float32, 'Float64': float, 'Int64': int}[d['type']](d['value'])


def load_cases():
    """[(meta, vol, verts, faces, iso, eps, ranges)] of every golden case."""
    with open(os.path.join(GOLDEN, 'cases.json')) as fh:
        meta = json.load(fh)
    z = np.load(os.path.join(GOLDEN, 'golden.npz'))
    out = []
    for m in meta:
        n = m['name']
        ranges = tuple((_unscalar(a), _unscalar(b)) for a, b in m['ranges'])
        out.append((m, np.asfortranarray(z[n + '/vol']), z[n + '/verts'], z[n + '/faces'], _unscalar(m['iso']),
                    _unscalar(m['eps']), ranges))
    return out


CASES = load_cases()
IDS = [c[0]['name'] for c in CASES]


def test_fixture_integrity():
    assert len(CASES) >= 20
    algs = {c[0]['alg'] for c in CASES}
    assert algs == {'mc', 'mt', 'nsn', 'mcw'}
    for m, vol, v, f, *_ in CASES:
        assert vol.dtype.name == m['dtype'] and list(vol.shape) == m['shape']
        assert v.dtype.name == m['verts_dtype'] and v.shape == (m['nverts'], 3) and f.shape == (m['nfaces'], 3)
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == m['verts_sha256']
        assert hashlib.sha256(np.ascontiguousarray(f).tobytes()).hexdigest() == m['faces_sha256']
        if len(f):
            assert f.min() >= 1 and f.max() <= len(v)


@pytest.mark.parametrize('case', CASES, ids=IDS)
def test_oracle_reproduces_golden(oracle, case):
    m, vol, v, f, iso, eps, ranges = case
    gv, gf = oracle.isosurface(vol, m['alg'], iso, eps, ranges)
    assert gv.dtype == v.dtype
    assert np.array_equal(gf, f)
    assert np.array_equal(gv, v, equal_nan=True)


@pytest.mark.parametrize('name', ['single_cell_f32_mc', 'nonfinite_f64_mc', 'random_u16_mt_f64iso',
                                  'flat_f64_mc', 'constant_f64_mt', 'sphere_f64_mcw', 'random_i64_mcw',
                                  'sphere_f64_nsn', 'random_i8_nsn', 'gyroid_f32_nsn_f32range'])
def test_python_restatement_reproduces_golden(name):
    m, vol, v, f, iso, eps, ranges = CASES[IDS.index(name)]
    with np.errstate(all='ignore'):  # Inf - Inf in the non-finite case, as in the reference
        gv, gf = pyoracle.isosurface(vol, m['alg'], iso, eps, ranges)
    assert gv.dtype == v.dtype
    assert np.array_equal(gf, f)
    assert np.array_equal(gv, v, equal_nan=True)
