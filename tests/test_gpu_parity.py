"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Contract (reference semantics): cube cases, face connectivity and vertex/face
counts bit-exact; positions within 1e-12 (Float64 output) or 2 ulp (Float32
output) of the oracle.  The kernels reproduce Julia's arithmetic operation by
operation, so every comparison below is also checked for bit equality.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = {'mc': 'MarchingCubes', 'mt': 'MarchingTetrahedra', 'nsn': 'NaiveSurfaceNets'}


def method(pkg, alg, iso=0.0, eps=1e-3):
    if alg == 'mt':
        return pkg.MarchingTetrahedra(iso=iso, eps=eps)
    return getattr(pkg, ALGS[alg])(iso=iso)


def assert_same(got, want, what=''):
    gv, gf = got
    wv, wf = want
    assert gv.dtype == wv.dtype, (what, gv.dtype, wv.dtype)
    assert gv.shape == wv.shape and gf.shape == wf.shape, (what, gv.shape, wv.shape, gf.shape, wf.shape)
    assert np.array_equal(gf, wf), what
    if len(gv):
        fin = np.isfinite(wv)
        assert np.array_equal(np.isnan(gv), np.isnan(wv)), what
        err = np.abs(gv[fin].astype(np.float64) - wv[fin].astype(np.float64))
        if gv.dtype == np.float64:
            assert err.max(initial=0) <= 1e-12, (what, err.max())
        else:
            ulp = np.spacing(np.abs(wv[fin]).astype(np.float32)).astype(np.float64)
            assert (err <= 2 * ulp).all(), (what, (err / ulp).max())
        assert np.array_equal(gv, wv, equal_nan=True), (what, 'not bit-exact', err.max())


def check(pkg, oracle, A, alg, iso=0.0, eps=1e-3, ranges=((-1, 1),) * 3, device=False):
    A = np.asfortranarray(A)
    m = method(pkg, alg, iso, eps)
    want = oracle.isosurface(A, alg, iso, eps, ranges)
    if device:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
        v, f = pkg.isosurface(t, m, *ranges)
        torch.cuda.synchronize()
        got = (v.cpu().numpy(), f.cpu().numpy())
    else:
        got = pkg.isosurface(A, m, *ranges)
    assert_same(got, want, '%s %s iso=%r eps=%r ranges=%r shape=%s' % (alg, A.dtype, iso, eps, ranges, A.shape))
    return got


def sphere(n, r=0.4, dtype=np.float64, c=(0, 0, 0), shape=None):
    shape = shape or (n, n, n)
    g = [np.linspace(-1, 1, s) for s in shape]
    X, Y, Z = np.meshgrid(*g, indexing='ij')
    return np.asfortranarray((np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r).astype(dtype))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_sphere64_f64(pkg, oracle, cuda, alg):
    # the 64^3 Float64 sphere fixture (signed distance, r = 0.4, iso 0)
    v, f = check(pkg, oracle, sphere(64), alg)
    if alg == 'mc':
        assert (len(v), len(f)) == (12000, 5996)
    if alg == 'mt':
        assert (len(v), len(f)) == (8978, 17952)


@pytest.mark.parametrize('device', [False, True])
def test_noisy_spheres_kat(pkg, oracle, cuda, device):
    # test/runtests.jl:152-172: MarchingTetrahedra(iso=8.0) on 21^3 noisy
    # distances (Julia 1.9's MersenneTwister(0) stream, restated in
    # oracle/julia_rand.py) gives 3466 vertices and 6928 faces; the CUDA path
    # gives the oracle's mesh bit for bit
    import julia_rand
    v, f = check(pkg, oracle, julia_rand.noisy_spheres(), 'mt', iso=8.0, device=device)
    assert (len(v), len(f)) == (3466, 6928)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_device_and_host_paths_agree(pkg, oracle, cuda, alg):
    A = sphere(40, 0.55, np.float32)
    check(pkg, oracle, A, alg, iso=np.float32(0.01), device=True)
    check(pkg, oracle, A, alg, iso=np.float32(0.01), device=False)


TYPE_CASES = [
    (np.float64, 0.0, 1e-3, (-1, 1)),
    (np.float64, np.float32(0.25), np.float32(1e-3), (0.0, 2.5)),
    (np.float32, 0.0, 1e-3, (-1, 1)),
    (np.float32, np.float32(0.1), np.float32(1e-3), (-1, 1)),
    (np.float32, np.float32(0.1), 1e-3, (np.float32(-2), np.float32(3))),
    (np.float32, 0, 1e-4, (0, 1)),
    (np.float32, np.float32(-0.3), np.float32(1e-2), (0.0, 1.0)),
    (np.uint16, 500, 1e-3, (-1, 1)),
    (np.uint16, 500, np.float32(1e-3), (np.float32(0), np.float32(7))),
    (np.uint16, np.float32(300.5), np.float32(1e-3), (-1, 1)),
    (np.uint16, 250.25, 1e-3, (0.0, 1.0)),
    (np.float16, 0.0, 1e-3, (-1, 1)),
    (np.float16, np.float32(0.1), np.float32(1e-3), (-1, 1)),
    (np.float16, np.float32(-0.3), 1e-3, (np.float32(-2), np.float32(3))),
    (np.float16, 0.25, np.float32(1e-2), (0.0, 1.0)),
]


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
@pytest.mark.parametrize('case', range(len(TYPE_CASES)))
def test_random_grids_all_types(pkg, oracle, cuda, alg, case):
    dt, iso, eps, r = TYPE_CASES[case]
    rng = np.random.default_rng(100 + case)
    for trial in range(4):
        shape = tuple(int(s) for s in rng.integers(2, 18, 3))
        if dt == np.uint16:
            A = rng.integers(0, 1000, shape).astype(np.uint16)
        else:
            A = rng.standard_normal(shape).astype(dt)
        check(pkg, oracle, A, alg, iso, eps, (r, r, r))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_ragged_multi_tile_shapes(pkg, oracle, cuda, alg):
    # shapes spanning several x tiles (31/30 cells), y tiles (4 rows), z segments and chunks
    rng = np.random.default_rng(7)
    for shape in [(67, 45, 133), (33, 9, 70), (95, 13, 17), (2, 70, 41), (70, 2, 9), (31, 5, 200)]:
        A = sphere(0, 0.7, np.float32, c=(0.1, -0.2, 0.05), shape=shape)
        A += np.float32(0.05) * rng.standard_normal(shape).astype(np.float32)
        check(pkg, oracle, A, alg, np.float32(0))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_sparse_surface_chunk_skipping(pkg, oracle, cuda, alg):
    # a small object: most z chunks and tiles are empty and skipped
    for c in [(0.8, 0.8, 0.8), (-0.85, 0.1, -0.9), (0.0, -0.9, 0.3)]:
        A = sphere(0, 0.12, np.float64, c=c, shape=(150, 90, 200))
        check(pkg, oracle, A, alg)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_all_256_cases(pkg, oracle, cuda, alg):
    # every cube case as a single cell, plus all of them planted in one grid
    for c in range(256):
        A = np.ones((2, 2, 2), np.float32)
        order = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        for k, (x, y, z) in enumerate(order):
            if (c >> k) & 1:
                A[x, y, z] = -1 - 0.37 * k
            else:
                A[x, y, z] = 0.5 + 0.21 * k
        check(pkg, oracle, A, alg, np.float32(0))
    A = np.ones((32, 32, 2), np.float32)
    rng = np.random.default_rng(3)
    for c in range(256):
        i, j = divmod(c, 16)
        for k, (x, y, z) in enumerate([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1),
                                       (0, 1, 1)]):
            A[2 * i + x, 2 * j + y, z] = -rng.random() if (c >> k) & 1 else rng.random()
    check(pkg, oracle, A, alg, np.float32(0))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_nan_inf_ties_and_signed_zero(pkg, oracle, cuda, alg):
    rng = np.random.default_rng(11)
    for dt in (np.float32, np.float64):
        A = rng.standard_normal((12, 11, 13)).astype(dt)
        A.flat[rng.choice(A.size, 40, replace=False)] = np.nan
        A.flat[rng.choice(A.size, 20, replace=False)] = np.inf
        A.flat[rng.choice(A.size, 20, replace=False)] = -np.inf
        A.flat[rng.choice(A.size, 60, replace=False)] = 0.0  # ties with iso
        A.flat[rng.choice(A.size, 30, replace=False)] = -0.0
        check(pkg, oracle, A, alg, dt(0) if dt == np.float32 else 0.0)
        # ranges through zero at a node (-0.0 handling of still coordinates)
        check(pkg, oracle, A, alg, 0.0, 1e-3, ((-1.0, 1.0), (0.0, 2.0), (-3.0, 0.0)))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_float32_subnormal_tiny_and_huge_samples_with_a_float64_iso(pkg, oracle, cuda, alg):
    # Float32 samples widened to the Float64 quotient type: normal values move
    # their bits, zeros keep their sign, subnormals / Inf / NaN take the
    # conversion instruction; every kind next to every other
    rng = np.random.default_rng(23)
    kinds = np.array([1e-45, -1e-45, 3e-42, -2.5e-40, 1.1754942e-38, -1.17549435e-38, 1.2e-38, 0.0, -0.0,
                      3.0e38, -3.4028235e38, 1.0, -1.0, 0.5, np.inf, -np.inf, np.nan], dtype=np.float32)
    A = kinds[rng.integers(0, len(kinds), (13, 12, 14))]
    for iso in (0.0, 1e-40, -2e-39, 1.0000000000000002):
        check(pkg, oracle, A, alg, iso)
    check(pkg, oracle, A, alg, 0.0, 1e-3, ((-1.0, 1.0), (0.0, 2.0), (-3.0, 0.0)), device=True)
    if alg == 'mc':
        A = np.asfortranarray(A)
        m = pkg.MarchingCubes(iso=1e-40, weld=True)
        assert_same(pkg.isosurface(A, m), oracle.isosurface(A, 'mcw', 1e-40), 'welded, special Float32 samples')


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_uint16_wraparound(pkg, oracle, cuda, alg):
    rng = np.random.default_rng(5)
    A = np.where(rng.random((20, 21, 22)) < 0.5, rng.integers(0, 400, (20, 21, 22)),
                 rng.integers(600, 65535, (20, 21, 22))).astype(np.uint16)
    check(pkg, oracle, A, alg, 500)
    check(pkg, oracle, A, alg, np.float32(500.5), np.float32(1e-3))


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_degenerate_volumes(pkg, oracle, cuda, alg):
    for shape in [(1, 5, 5), (5, 1, 5), (5, 5, 1), (0, 4, 4), (2, 2, 2)]:
        A = np.random.default_rng(1).standard_normal(shape)
        check(pkg, oracle, A, alg)
    check(pkg, oracle, np.ones((4, 4, 4)), alg)        # no crossings
    check(pkg, oracle, -np.ones((4, 4, 4)), alg)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_gyroid_256_f32(pkg, oracle, cuda, alg):
    # Float32 gyroid on [-3pi, 3pi]^3, iso 0 (Float64, the MarchingCubes() default)
    g = np.linspace(-3 * np.pi, 3 * np.pi, 256).astype(np.float32)
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    A = np.asfortranarray(np.sin(X) * np.cos(Y) + np.sin(Y) * np.cos(Z) + np.sin(Z) * np.cos(X))
    r = (-3 * np.pi, 3 * np.pi)
    check(pkg, oracle, A, alg, 0.0, 1e-3, (r, r, r))
    check(pkg, oracle, A, alg, np.float32(0), np.float32(1e-3), ((-3, 3),) * 3)


def test_extract_device_capacity(pkg, oracle, cuda):
    import torch
    A = sphere(48, 0.5, np.float32)
    t = torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    want = oracle.isosurface(A, 'mc', np.float32(0))
    m = pkg.MarchingCubes(iso=np.float32(0))
    verts = torch.empty((len(want[0]), 3), dtype=torch.float32, device='cuda')
    faces = torch.empty((len(want[1]), 3), dtype=torch.int64, device='cuda')
    counts = pkg.isosurface_device(t, m, verts=verts, faces=faces)
    pkg.api.sync()
    assert counts.tolist() == [len(want[0]), len(want[1])]
    assert_same((verts.cpu().numpy(), faces.cpu().numpy()), want)
    small = torch.empty((10, 3), dtype=torch.float32, device='cuda')
    counts = pkg.isosurface_device(t, m, verts=small, faces=faces)
    with pytest.raises(pkg.MeshError) as ei:
        pkg.api.sync()
    assert ei.value.status == 6  # MESH_ECAPACITY
    assert counts.tolist() == [len(want[0]), len(want[1])]


def test_fill_without_count_is_rejected(pkg, cuda):
    c = pkg.Context(0)
    rc = pkg.load_library().mesh_fill(c.handle, None, None, 0)
    assert rc == 5  # MESH_ESTATE


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
@pytest.mark.parametrize('dt', [np.int32, np.int64, np.int16, np.int8, np.uint8])
def test_integer_volumes(pkg, oracle, cuda, alg, dt):
    # test/runtests.jl:66-75 runs every algorithm on rand(Int, 10, 10, 10): exact
    # integer-vs-iso comparison, v2 - v1 wrapping in the data type, the quotient in
    # promote(typeof(iso), T) (Int / Int divides in Float64); output Float64 by default
    rng = np.random.default_rng(int(np.dtype(dt).itemsize) + len(alg))
    info = np.iinfo(dt)
    A = rng.integers(info.min, info.max, (10, 10, 10), dtype=dt, endpoint=True)
    v, f = check(pkg, oracle, A, alg)
    assert v.dtype == np.float64 and f.dtype == np.int64
    for trial in range(3):
        shape = tuple(int(s) for s in rng.integers(2, 20, 3))
        full = rng.integers(info.min, info.max, shape, dtype=dt, endpoint=True)
        small = rng.integers(-1000, 1000, shape).astype(dt)
        for B, isos in ((full, [0.0, np.float32(1e9), 0, -123456789]), (small, [0.5, np.float32(-3.25), 7])):
            for iso in isos:
                check(pkg, oracle, B, alg, iso, np.float32(1e-3) if isinstance(iso, np.float32) else 1e-3)
                check(pkg, oracle, B, alg, iso, 1e-3, ((np.float32(-2), np.float32(3)),) * 3, device=True)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_integer_field_many_tiles(pkg, oracle, cuda, alg):
    # a smooth Int32 field over several x tiles, y tiles and z segments
    A = (sphere(0, 0.6, np.float64, c=(0.1, 0.0, -0.05), shape=(97, 70, 133)) * 100000).astype(np.int32)
    check(pkg, oracle, A, alg, 0)
    check(pkg, oracle, A, alg, 2500.5, 1e-3, ((0, 1),) * 3, device=True)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_float16_volumes(pkg, oracle, cuda, alg):
    # test/runtests.jl:56-65 runs the algorithms on Float16 data.  Float32 / Float64 iso:
    # exact comparison, v2 - v1 a Float16 subtraction, quotient in promote(typeof(iso), Float16)
    rng = np.random.default_rng(61 + len(alg))
    A = sphere(0, 0.6, np.float16, c=(0.05, -0.1, 0.0), shape=(67, 45, 133))  # several x / y tiles, z segments
    check(pkg, oracle, A, alg, np.float32(0))
    check(pkg, oracle, A, alg, 0.0, 1e-3, ((0, 1),) * 3, device=True)
    big = np.clip(rng.standard_normal((23, 17, 29)) * 3e4, -65504, 65504).astype(np.float16)  # differences round / overflow
    big.ravel(order='K')[:4] = [np.inf, -np.inf, np.nan, np.float16(65504)]
    for iso in (np.float32(0), 1.0e4, np.float32(-2.5e4)):
        check(pkg, oracle, big, alg, iso, np.float32(1e-3) if isinstance(iso, np.float32) else 1e-3)
    check(pkg, oracle, big, alg, 0.0, 1e-3, ((np.float32(-2), np.float32(3)),) * 3, device=True)


@pytest.mark.parametrize('case', range(len(TYPE_CASES)))
def test_welded_marching_cubes(pkg, oracle, cuda, case):
    # MarchingCubes(weld=True): one vertex per crossed lattice edge in first-touch order,
    # against the oracle's welded restatement, on random grids of every type and on a
    # shape spanning several tiles / segments; host and device volumes
    dt, iso, eps, r = TYPE_CASES[case]
    rng = np.random.default_rng(300 + case)
    for trial in range(3):
        shape = tuple(int(s) for s in rng.integers(2, 18, 3))
        A = rng.integers(0, 1000, shape).astype(np.uint16) if dt == np.uint16 else rng.standard_normal(shape).astype(dt)
        A = np.asfortranarray(A)
        want = oracle.isosurface(A, 'mcw', iso, eps, (r, r, r))
        got = pkg.isosurface(A, pkg.MarchingCubes(iso=iso, weld=True), r, r, r)
        assert_same(got, want, 'welded %s %s' % (dt, shape))
    B = sphere(0, 0.6, np.float32, c=(0.05, -0.1, 0.02), shape=(67, 45, 133)).astype(dt) if dt != np.uint16 else \
        np.asfortranarray((sphere(0, 0.6, np.float64, shape=(67, 45, 133)) * 1000 + 500).astype(np.uint16))
    want = oracle.isosurface(B, 'mcw', iso, eps, (r, r, r))
    m = pkg.MarchingCubes(iso=iso, weld=True)
    assert_same(pkg.isosurface(B, m, r, r, r), want, 'welded sphere')
    import torch
    t = torch.from_numpy(np.ascontiguousarray(B.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    v, f = pkg.isosurface(t, m, r, r, r)
    torch.cuda.synchronize()
    assert_same((v.cpu().numpy(), f.cpu().numpy()), want, 'welded sphere, device volume')
    plain = oracle.isosurface(B, 'mc', iso, eps, (r, r, r))
    assert len(want[0]) < len(plain[0]) and len(want[1]) == len(plain[1])


def _golden_cases():
    from test_golden import CASES
    return CASES


@pytest.mark.parametrize('idx', range(25))
def test_golden_fixtures(pkg, cuda, idx):
    # the committed golden meshes (tests/golden, oracle outputs frozen by make_golden.py):
    # the CUDA path reproduces them byte for byte, from host and from device volumes
    import torch
    cases = _golden_cases()
    if idx >= len(cases):
        pytest.skip('fewer golden cases')
    m, vol, v, f, iso, eps, ranges = cases[idx]
    alg = m['alg']
    meth = pkg.MarchingCubes(iso=iso, weld=True) if alg == 'mcw' else method(pkg, alg, iso, eps)
    assert_same(pkg.isosurface(vol, meth, *ranges), (v, f), m['name'])
    t = torch.from_numpy(np.ascontiguousarray(vol.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    gv, gf = pkg.isosurface(t, meth, *ranges)
    torch.cuda.synchronize()
    assert_same((gv.cpu().numpy(), gf.cpu().numpy()), (v, f), m['name'] + ' (device volume)')


@pytest.mark.parametrize('axis', [0, 1, 2])
@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_maximum_axis_length(pkg, oracle, cuda, alg, axis):
    # the longest axis the engine takes: 2^21 samples on x and z (cell coordinates are
    # packed in 21 bits), 2^21 - 31 on y (65535 CTA rows of 32 cell rows in the launch
    # grid); one sample more is MESH_ETOOLARGE
    n = (1 << 21) - (31 if axis == 1 else 0)
    shape = [3, 3, 3]
    shape[axis] = n
    line = np.cos(2 * np.pi * np.arange(n) / 1000.0)
    a, b = np.meshgrid([0.0, 0.15, 0.3], [0.0, -0.1, -0.2], indexing='ij')
    along = np.moveaxis(line[:, None, None] + a[None] + b[None], 0, axis)
    A = np.asfortranarray(along.astype(np.float32))
    assert A.shape == tuple(shape)
    v, f = check(pkg, oracle, A, alg, iso=np.float32(0.1))
    assert len(f) > 4000
    shape[axis] += 1
    with pytest.raises(pkg.MeshError) as ei:
        pkg.isosurface(np.zeros(shape, np.float32, order='F'), method(pkg, alg, np.float32(0.1)))
    assert ei.value.status == 7  # MESH_ETOOLARGE


@pytest.mark.parametrize('dt,iso,rg', [(np.float32, np.float32(0.05), ((0, 1),) * 3), (np.float64, 0.0, ((-1, 1),) * 3),
                                       (np.uint16, 500, ((-1, 1),) * 3), (np.int8, 3, ((-1.0, 1.0),) * 3),
                                       (np.float16, np.float32(0.1), ((np.float32(-1), np.float32(1)),) * 3)])
def test_direct_and_list_emission_agree(pkg, oracle, cuda, dt, iso, rg, monkeypatch):
    # Marching Cubes is emitted straight from the volume by default; the list
    # form (compaction, then expansion) must give the same mesh, and both the
    # oracle's.  Shapes: several x tiles, z segments and partial chunks.
    torch = cuda
    rng = np.random.default_rng(11)
    shape = (77, 45, 83)
    if np.issubdtype(dt, np.integer):
        info = np.iinfo(dt)
        A = rng.integers(max(info.min, -200), min(info.max, 1000), shape).astype(dt)
    else:
        A = sphere(0, 0.5, dt, shape=shape) + (0.05 * rng.standard_normal(shape)).astype(dt)
    A = np.asfortranarray(A)
    got = check(pkg, oracle, A, 'mc', iso=iso, ranges=rg)
    monkeypatch.setenv('MESHING_GB300_LIST_EMIT', '1')
    ctx = pkg.Context(0)
    lst = pkg.isosurface(A, pkg.MarchingCubes(iso=iso), *rg, ctx=ctx)
    ctx.close()
    assert np.array_equal(got[1], lst[1]) and np.array_equal(got[0].view(np.uint8), lst[0].view(np.uint8))
