"""Writes the committed golden fixtures (tests/golden/golden.npz + cases.json).

Each case is a small seeded volume, the isosurface call's arguments and the
mesh that the CPU oracle (oracle/oracle.c, the loop-for-loop restatement of
src/marching_cubes.jl and src/marching_tetrahedra.jl) returns for it.  The
oracle is itself pinned to the reference's known-answer tests
(tests/test_oracle.py); these fixtures freeze its outputs, so that
tests/test_golden.py checks the oracle against them on the CPU and
tests/test_gpu_parity.py::test_golden_fixtures checks the CUDA path against
them byte for byte.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), 'oracle'))

import oracle  # noqa: E402


def _grid(shape, lo=-1.0, hi=1.0):
    g = [np.linspace(lo, hi, s) for s in shape]
    return np.meshgrid(*g, indexing='ij')


def sphere(shape, r=0.45, c=(0.05, -0.03, 0.02)):
    X, Y, Z = _grid(shape)
    return np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r


def torus(shape, R=0.55, r=0.2):
    X, Y, Z = _grid(shape)
    return np.sqrt((np.sqrt(X * X + Y * Y) - R) ** 2 + Z * Z) - r


def gyroid(shape):
    X, Y, Z = _grid(shape, 0.0, 2 * np.pi)
    return np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X)


def scalar(v):
    """JSON form of a scalar argument, keeping its Julia type."""
    if isinstance(v, np.float32):
        return {'type': 'Float32', 'value': float(v)}
    if isinstance(v, float):
        return {'type': 'Float64', 'value': v}
    return {'type': 'Int64', 'value': int(v)}


def unscalar(d):
    return {'Float32': np.float32, 'Float64': float, 'Int64': int}[d['type']](d['value'])


def cases():
    rng = np.random.default_rng(20240601)
    out = []

    def add(name, vol, alg, iso=0.0, eps=1e-3, ranges=((-1, 1),) * 3):
        out.append((name, np.asfortranarray(vol), alg, iso, eps, ranges))

    # closed surfaces, every algorithm
    for alg in ('mc', 'mt', 'nsn', 'mcw'):
        add('sphere_f64_%s' % alg, sphere((20, 17, 15)), alg)
    add('torus_f32_mc', torus((24, 24, 12)).astype(np.float32), 'mc', iso=np.float32(0.0))
    add('torus_f32_mt_f64iso', torus((24, 24, 12)).astype(np.float32), 'mt', iso=0.01, eps=1e-2)
    add('gyroid_f64_mc_floatrange', gyroid((16, 16, 16)), 'mc', iso=0.2, ranges=((0.0, 2.5),) * 3)
    add('gyroid_f32_nsn_f32range', gyroid((16, 16, 16)).astype(np.float32), 'nsn', iso=np.float32(0.1),
        ranges=((np.float32(-0.5), np.float32(1.5)),) * 3)
    # random fields: every cube case is met
    R = rng.standard_normal((11, 9, 7))
    for alg in ('mc', 'mt', 'nsn'):
        add('random_f64_%s' % alg, R, alg, iso=0.1)
    add('random_f32_mc_intrange', R.astype(np.float32), 'mc', iso=np.float32(-0.2), ranges=((0, 10), (0, 8), (0, 6)))
    # integer and half-precision volumes (Julia's wrapping differences)
    U = rng.integers(0, 65536, (10, 8, 6)).astype(np.uint16)
    add('random_u16_mc_intiso', U, 'mc', iso=30000)
    add('random_u16_mt_f64iso', U, 'mt', iso=20000.5)
    add('random_u8_mc', rng.integers(0, 256, (9, 9, 9)).astype(np.uint8), 'mc', iso=100)
    add('random_i16_mt', rng.integers(-2000, 2000, (9, 8, 7)).astype(np.int16), 'mt', iso=0.5)
    add('random_i8_nsn', rng.integers(-128, 128, (9, 8, 7)).astype(np.int8), 'nsn', iso=3)
    add('random_i32_mc', rng.integers(-10 ** 9, 10 ** 9, (8, 8, 8)).astype(np.int32), 'mc', iso=0)
    add('random_i64_mcw', rng.integers(-1000, 1000, (8, 9, 10)).astype(np.int64), 'mcw', iso=7)
    add('sphere_f16_mc_f32iso', sphere((14, 14, 14)).astype(np.float16), 'mc', iso=np.float32(0.0))
    # edge cases: non-finite values, ties, degenerate shapes
    S = sphere((9, 9, 9))
    S[4, 4, 4] = np.nan
    S[1, 2, 3] = np.inf
    S[7, 6, 5] = -np.inf
    S[2, 2, 2] = 0.0
    S[3, 3, 3] = -0.0
    add('nonfinite_f64_mc', S, 'mc')
    add('nonfinite_f64_mt', S, 'mt')
    add('single_cell_f32_mc', np.array([-1, 1, 1, 1, 1, 1, 1, -1], np.float32).reshape(2, 2, 2, order='F'), 'mc',
        iso=np.float32(0.0))
    add('flat_f64_mc', np.zeros((1, 5, 5)), 'mc')
    add('constant_f64_mt', np.ones((4, 4, 4)), 'mt', iso=1.0)
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    oracle.build()
    arrays, meta = {}, []
    for name, vol, alg, iso, eps, ranges in cases():
        v, f = oracle.isosurface(vol, alg, iso, eps, ranges)
        arrays[name + '/vol'] = vol
        arrays[name + '/verts'] = v
        arrays[name + '/faces'] = f
        meta.append({'name': name, 'alg': alg, 'dtype': vol.dtype.name, 'shape': list(vol.shape),
                     'iso': scalar(iso), 'eps': scalar(eps),
                     'ranges': [[scalar(a), scalar(b)] for a, b in ranges],
                     'nverts': len(v), 'nfaces': len(f), 'verts_dtype': v.dtype.name,
                     'verts_sha256': sha(v), 'faces_sha256': sha(f)})
    np.savez_compressed(os.path.join(HERE, 'golden.npz'), **arrays)
    with open(os.path.join(HERE, 'cases.json'), 'w') as fh:
        json.dump(meta, fh, indent=1)
        fh.write('\n')
    print('%d cases written' % len(meta))


if __name__ == '__main__':
    main()
