"""The pipelined host path: volume upload in groups of z segments, each group
classified as it arrives, and the Marching Cubes mesh emitted and downloaded in
x ranges (mesh_api.cu: upload_and_classify, emit_pipelined).  A context created
with MESHING_GB300_PIPELINE_BYTES=1 pipelines every host call, so small volumes
exercise it; results must equal the oracle's bit for bit, from pageable numpy
buffers and from pinned buffers through the C ABI."""
import ctypes
import os

import numpy as np
import pytest

from test_gpu_parity import assert_same, method, sphere

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def pctx(pkg, cuda):
    old = os.environ.get('MESHING_GB300_PIPELINE_BYTES')
    os.environ['MESHING_GB300_PIPELINE_BYTES'] = '1'
    try:
        c = pkg.Context(0)
    finally:
        if old is None:
            del os.environ['MESHING_GB300_PIPELINE_BYTES']
        else:
            os.environ['MESHING_GB300_PIPELINE_BYTES'] = old
    yield c
    c.close()


def meth(pkg, alg, iso):
    return pkg.MarchingCubes(iso=iso, weld=True) if alg == 'mcw' else method(pkg, alg, iso)


def field(shape, dt, seed):
    rng = np.random.default_rng(seed)
    A = sphere(0, 0.55, np.float64, c=(0.1, -0.05, 0.03), shape=shape)
    A = A + 0.05 * rng.standard_normal(shape)
    if dt == np.uint16:
        return np.asfortranarray((A * 1000 + 500).astype(np.uint16))
    if dt == np.int16:
        return np.asfortranarray((A * 1000).astype(np.int16))
    return np.asfortranarray(A.astype(dt))


ISO = {np.float64: 0.0, np.float32: np.float32(0.0), np.uint16: 500, np.int16: 3}


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn', 'mcw'])
@pytest.mark.parametrize('dt', [np.float32, np.float64, np.uint16, np.int16])
@pytest.mark.parametrize('shape', [(100, 40, 90), (70, 65, 20), (200, 9, 130)])
def test_pipelined_host_path_matches_oracle(pkg, oracle, pctx, alg, dt, shape):
    A = field(shape, dt, sum(shape) + ['mc', 'mt', 'nsn', 'mcw'].index(alg))
    iso = ISO[dt]
    want = oracle.isosurface(A, alg, iso)
    got = pkg.isosurface(A, meth(pkg, alg, iso), ctx=pctx)
    assert_same(got, want, 'pipelined %s %s %s' % (alg, dt.__name__, shape))


def test_empty_x_ranges(pkg, oracle, pctx):
    # a small sphere near x = 0 of a long volume: most x ranges hold no active cell
    A = sphere(0, 0.08, np.float32, c=(-0.85, 0.0, 0.0), shape=(400, 33, 70))
    for iso in (np.float32(0.0), np.float32(5.0)):  # the second one has no surface at all
        want = oracle.isosurface(A, 'mc', iso)
        assert_same(pkg.isosurface(A, pkg.MarchingCubes(iso=iso), ctx=pctx), want, 'sparse iso=%r' % iso)


def test_context_reuse_across_shapes(pkg, oracle, pctx):
    # buffers, events and the copy stream are reused: large, small, large again,
    # and a device-volume call in between
    import torch
    shapes = [(150, 60, 120), (20, 20, 20), (90, 120, 50), (150, 60, 120)]
    for k, sh in enumerate(shapes):
        A = field(sh, np.float32, 40 + k)
        want = oracle.isosurface(A, 'mc', np.float32(0.0))
        assert_same(pkg.isosurface(A, pkg.MarchingCubes(iso=np.float32(0.0)), ctx=pctx), want, 'reuse %s' % (sh,))
        if k == 1:
            t = torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
            v, f = pkg.isosurface(t, pkg.MarchingCubes(iso=np.float32(0.0)), ctx=pctx)
            torch.cuda.synchronize()
            assert_same((v.cpu().numpy(), f.cpu().numpy()), want, 'device volume between host calls')


def test_pinned_buffers_through_the_abi(pkg, oracle, pctx):
    # mesh_count / mesh_fill with pinned host volume and outputs, as the benchmark calls them
    import torch
    lib = pkg.load_library()
    A = field((180, 70, 110), np.float32, 7)
    want = oracle.isosurface(A, 'mc', np.float32(0.0))
    hvol = torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).pin_memory()
    p = pkg.make_params(pkg.MarchingCubes(iso=np.float32(0.0)))
    pctx.set_stream(None)
    for _ in range(2):
        nv, nf = ctypes.c_int64(), ctypes.c_int64()
        pkg._lib.check(lib.mesh_count(pctx.handle, ctypes.c_void_p(hvol.data_ptr()), 2, *A.shape, 0,
                                      ctypes.byref(p), ctypes.byref(nv), ctypes.byref(nf)), pctx.handle)
        hv = torch.empty((nv.value, 3), dtype=torch.float32, pin_memory=True)
        hf = torch.empty((nf.value, 3), dtype=torch.int64, pin_memory=True)
        pkg._lib.check(lib.mesh_fill(pctx.handle, ctypes.c_void_p(hv.data_ptr()), ctypes.c_void_p(hf.data_ptr()), 0),
                       pctx.handle)
        assert_same((hv.numpy(), hf.numpy()), want, 'pinned')
