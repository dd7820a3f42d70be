"""Contexts driven from several host threads at once.

The reference is single-threaded; its drop-in must be safe when several
callers (Julia tasks, Python threads) each use their own context
concurrently.  Every thread below owns a Context and runs a mixed sequence of
extractions -- the three algorithms, welded Marching Cubes, Float32 / Float64
/ UInt16 volumes, host volumes on the context's own stream -- while the
others do the same; each result must be bit-identical to the one computed
alone, first, on a single context (which in turn equals the oracle).
ctypes drops the GIL around every C call, so the library's entry points run
concurrently.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields():
    rng = np.random.default_rng(5)
    g = [np.linspace(-1, 1, n) for n in (96, 88, 80)]
    X, Y, Z = np.meshgrid(*g, indexing='ij')
    waves = np.sin(5 * X) * np.cos(4 * Y) + np.sin(4 * Y) * np.cos(3 * Z) + 0.05 * rng.standard_normal(X.shape)
    s = [np.linspace(-1, 1, n) for n in (64, 60, 56)]
    X, Y, Z = np.meshgrid(*s, indexing='ij')
    sphere = np.sqrt(X * X + Y * Y + Z * Z) - 0.6
    ct = np.round((waves + 2) * 300).astype(np.uint16)
    return {'f32': np.asfortranarray(waves.astype(np.float32)), 'f64': np.asfortranarray(sphere),
            'u16': np.asfortranarray(ct)}


def _jobs(pkg):
    r = (-1, 1)
    return [
        ('f32', pkg.MarchingCubes(iso=np.float32(0.1)), (r, r, r)),
        ('f64', pkg.MarchingTetrahedra(iso=0.0, eps=1e-3), (r, r, r)),
        ('f32', pkg.NaiveSurfaceNets(iso=np.float32(-0.2)), ((0, 1), (0, 1), (0, 1))),
        ('u16', pkg.MarchingCubes(iso=600), (r, r, r)),
        ('f64', pkg.MarchingCubes(iso=0.0, weld=True), (r, r, r)),
        ('u16', pkg.MarchingTetrahedra(iso=np.float32(610.5), eps=1e-3), (r, r, r)),
        ('f32', pkg.MarchingCubes(iso=0.0), ((0, 2), (0, 2), (0, 2))),
    ]


def test_contexts_on_several_threads_give_the_single_thread_meshes(pkg, oracle, cuda):
    vols = _fields()
    jobs = _jobs(pkg)
    # alone, on one context, first
    ctx0 = pkg.Context(0)
    want = [pkg.isosurface(vols[k], m, *rg, ctx=ctx0) for k, m, rg in jobs]
    ctx0.close()
    assert all(len(f) > 0 for _, f in want)
    # and that equals the oracle (one case per algorithm)
    for i in (0, 1, 2):
        k, m, rg = jobs[i]
        alg = {'MarchingCubes': 'mc', 'MarchingTetrahedra': 'mt', 'NaiveSurfaceNets': 'nsn'}[type(m).__name__]
        wv, wf = oracle.isosurface(vols[k], alg, m.iso, getattr(m, 'eps', 1e-3), rg)
        assert np.array_equal(want[i][1], wf)
        assert np.array_equal(want[i][0].view(np.uint8), wv.view(np.uint8))

    nthreads, reps = 4, 3
    errors = []
    barrier = threading.Barrier(nthreads)

    def worker(w):
        try:
            ctx = pkg.Context(0)
            barrier.wait(timeout=120)
            order = list(range(len(jobs)))
            np.random.default_rng(w).shuffle(order)  # every thread its own interleaving
            for _ in range(reps):
                for i in order:
                    k, m, rg = jobs[i]
                    v, f = pkg.isosurface(vols[k], m, *rg, ctx=ctx)
                    if not (np.array_equal(f, want[i][1]) and v.dtype == want[i][0].dtype and
                            np.array_equal(v.view(np.uint8), want[i][0].view(np.uint8))):
                        errors.append((w, i, 'differs'))
            ctx.close()
        except Exception as e:  # reported on the main thread
            errors.append((w, -1, repr(e)))

    th = [threading.Thread(target=worker, args=(w,)) for w in range(nthreads)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in th)
    assert not errors, errors[:5]
