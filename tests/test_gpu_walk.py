"""Marching Cubes in one walk: the classify walk stages the active cells.

With MESHING_GB300_ONE_WALK=1 a context walks a Marching Cubes volume once;
the list of active cells is filled during mesh_count and expanded by
mesh_fill.  These tests check it against the oracle where the list has to
grow (volumes whose cells are nearly all active), against the default
two-pass form (classify, second walk, expansion) bit for bit, and with output
capacities that are exactly the mesh size.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same, sphere

pytestmark = pytest.mark.gpu


@pytest.fixture
def walk_ctx(pkg, cuda, monkeypatch):
    monkeypatch.setenv('MESHING_GB300_ONE_WALK', '1')
    ctx = pkg.Context(0)
    monkeypatch.delenv('MESHING_GB300_ONE_WALK')
    yield ctx
    ctx.close()


def to_device(torch, A):
    return torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).cuda().permute(2, 1, 0)


def noise(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    if dtype == np.uint16:
        return np.asfortranarray(rng.integers(0, 1000, shape).astype(np.uint16))
    return np.asfortranarray(rng.random(shape).astype(dtype))


def test_dense_volumes_grow_the_list(pkg, oracle, cuda, walk_ctx):
    # uniform noise around iso: ~99% of the cells are active, far above the
    # first guess of the list size; the walk reports the exact size and runs again
    torch = cuda
    ctx = walk_ctx
    for shape, dt, iso in [((40, 37, 33), np.float32, np.float32(0.5)), ((96, 96, 96), np.float32, np.float32(0.5)),
                           ((130, 70, 90), np.float64, 0.5), ((64, 80, 72), np.uint16, 500)]:
        A = noise(shape, dt, sum(shape))
        m = pkg.MarchingCubes(iso=iso)
        want = oracle.isosurface(A, 'mc', iso, 1e-3, ((-1, 1),) * 3)
        v, f = pkg.isosurface(to_device(torch, A), m, ctx=ctx)
        torch.cuda.synchronize()
        assert_same((v.cpu().numpy(), f.cpu().numpy()), want, str((shape, dt)))
        v, f = pkg.isosurface(A, m, ctx=ctx)  # host buffers, the context's grown list
        assert_same((v, f), want, str((shape, dt, 'host')))


@pytest.mark.parametrize('dt', ['f32', 'f64', 'u16'])
def test_one_walk_matches_two_pass(pkg, cuda, dt, walk_ctx):
    torch = cuda
    import meshing_gb300.fields as fields
    if dt == 'u16':
        t = fields.ct_like_u16(320, seed=4)
        m = pkg.MarchingCubes(iso=1000)
    else:
        t = fields.gyroid(300, dtype=torch.float32 if dt == 'f32' else torch.float64)
        m = pkg.MarchingCubes(iso=np.float32(0.1) if dt == 'f32' else 0.1)
    ranges = ((0.0, 1.0), (-1.0, 2.0), (0.0, 3.5))
    v1, f1 = pkg.isosurface(t, m, *ranges, ctx=walk_ctx)
    v2, f2 = pkg.isosurface(t, m, *ranges)
    torch.cuda.synchronize()
    assert f1.shape[0] > 100000
    assert torch.equal(f1, f2)
    assert torch.equal(v1, v2)


def test_extract_device_exact_capacity_dense(pkg, oracle, cuda, walk_ctx):
    # mesh_extract_device sizes its list from the vertex capacity; with exact
    # capacities on a dense volume every staged slot is needed
    torch = cuda
    A = noise((70, 66, 61), np.float32, 9)
    m = pkg.MarchingCubes(iso=np.float32(0.5))
    want = oracle.isosurface(A, 'mc', np.float32(0.5), 1e-3, ((-1, 1),) * 3)
    verts = torch.empty((len(want[0]), 3), dtype=torch.float32, device='cuda')
    faces = torch.empty((len(want[1]), 3), dtype=torch.int64, device='cuda')
    ctx = walk_ctx
    for _ in range(2):
        counts = pkg.isosurface_device(to_device(torch, A), m, verts=verts, faces=faces, ctx=ctx)
        ctx.sync()
        assert counts.tolist() == [len(want[0]), len(want[1])]
        assert_same((verts.cpu().numpy(), faces.cpu().numpy()), want)


def test_count_without_fill_then_new_count(pkg, oracle, cuda, walk_ctx):
    # a count whose fill never comes leaves the list to the next count
    ctx = walk_ctx
    lib = pkg.load_library()
    A = noise((50, 50, 50), np.float32, 3)
    p = pkg.make_params(pkg.MarchingCubes(iso=np.float32(0.5)), (-1, 1), (-1, 1), (-1, 1))
    import ctypes
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    assert lib.mesh_count(ctx.handle, A.ctypes.data_as(ctypes.c_void_p), 2, 50, 50, 50, 0, ctypes.byref(p),
                          ctypes.byref(nv), ctypes.byref(nf)) == 0
    B = sphere(57, 0.6, np.float32)
    want = oracle.isosurface(B, 'mc', np.float32(0), 1e-3, ((-1, 1),) * 3)
    got = pkg.isosurface(B, pkg.MarchingCubes(iso=np.float32(0)), ctx=ctx)
    assert_same(got, want)


@pytest.mark.parametrize('alg', ['mc', 'mt'])
def test_pinned_host_volume_read_in_place(pkg, cuda, alg, monkeypatch):
    # with MESHING_GB300_ZEROCOPY=1 a pinned (mapped) host volume is read in
    # place over the host link -- for Marching Cubes by the one walk -- and must
    # give the device path's mesh; without it, it is copied
    torch = cuda
    import meshing_gb300.fields as fields
    t = fields.gyroid(200, dtype=torch.float32)
    m = pkg.MarchingCubes(iso=np.float32(0.05)) if alg == 'mc' else pkg.MarchingTetrahedra(iso=np.float32(0.05))
    v1, f1 = pkg.isosurface(t, m)
    pinned = torch.empty((200, 200, 200), dtype=torch.float32, pin_memory=True)
    pinned.copy_(t.permute(2, 1, 0))  # Julia layout: x fastest
    A = pinned.permute(2, 1, 0)
    monkeypatch.setenv('MESHING_GB300_ZEROCOPY', '1')
    for ctx in (pkg.Context(0), pkg.Context(0)):  # fresh and reused context
        for _ in range(2):
            v2, f2 = pkg.isosurface(A, m, ctx=ctx)
            assert np.array_equal(f2, f1.cpu().numpy())
            assert np.array_equal(v2, v1.cpu().numpy())
        ctx.close()
    monkeypatch.delenv('MESHING_GB300_ZEROCOPY')
    ctx = pkg.Context(0)
    v3, f3 = pkg.isosurface(A, m, ctx=ctx)
    ctx.close()
    assert np.array_equal(f3, f1.cpu().numpy()) and np.array_equal(v3, v1.cpu().numpy())
