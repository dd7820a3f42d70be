"""Out-of-core isosurfaces over x slabs (isosurface_slabs, mesh_set_x_window).

x is the outermost axis of the reference's emission order
(src/marching_cubes.jl:40, src/marching_tetrahedra.jl:144): the slab meshes,
concatenated with face indices offset by the vertices before them, must equal
the whole volume's mesh bit for bit, with node coordinates taken from the whole
volume's LinRange.  Marching Tetrahedra and Naive Surface Nets slabs carry the
previous slab's last cell column as a halo, whose shared vertices they use."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _field(shape, dtype, seed=0):
    rng = np.random.default_rng(seed)
    g = [np.linspace(-1, 1, n) for n in shape]
    X, Y, Z = np.meshgrid(*g, indexing='ij')
    f = np.sin(3 * X + 1) * np.cos(2 * Y) + np.sin(2.5 * Z) * np.cos(3 * X) + 0.05 * rng.standard_normal(shape)
    if np.dtype(dtype).kind in 'iu':
        f = np.round((f + 2) * 1000)
    return np.asfortranarray(f.astype(dtype))


@pytest.mark.parametrize('dtype,iso,rng', [
    (np.float32, np.float32(0.1), (np.float32(-1.5), np.float32(2.0))),
    (np.float32, 0.0, (0, 1)),
    (np.float64, 0.0, (-3.0, 0.7)),
    (np.uint16, 2000, (-1, 1)),
    (np.int16, np.float32(1999.5), (np.float32(0), np.float32(5))),
    (np.float16, np.float32(0.05), (-1, 1)),
])
def test_slabs_equal_the_whole_volume(pkg, cuda, dtype, iso, rng):
    A = _field((67, 33, 45), dtype)
    m = pkg.MarchingCubes(iso=iso)
    want = pkg.isosurface(A, m, rng, rng, rng)
    assert len(want[1]) > 0
    for slab in (1, 2, 7, 31, 40, 66, 200):
        got = pkg.isosurface_slabs(A, m, rng, rng, rng, slab_cells=slab)
        assert got[0].dtype == want[0].dtype
        assert np.array_equal(got[1], want[1]), slab
        assert np.array_equal(got[0].view(np.uint8), want[0].view(np.uint8)), slab
    # the window is reset afterwards: a whole-volume call still matches
    again = pkg.isosurface(A, m, rng, rng, rng)
    assert np.array_equal(again[1], want[1]) and np.array_equal(again[0], want[0])


def test_slab_budget_and_rejections(pkg, cuda):
    A = _field((50, 20, 30), np.float32)
    m = pkg.MarchingCubes(iso=np.float32(0))
    want = pkg.isosurface(A, m)
    got = pkg.isosurface_slabs(A, m, slab_bytes=20 * 30 * 4 * 9)  # 8 cells per slab
    assert np.array_equal(got[1], want[1]) and np.array_equal(got[0], want[0])
    with pytest.raises(TypeError):
        pkg.isosurface_slabs(A, pkg.MarchingCubes(iso=np.float32(0), weld=True))
    lib, c = pkg.load_library(), pkg.default_context(0)
    assert lib.mesh_set_x_window(c.handle, -1, 10, 0) == 1
    assert lib.mesh_set_x_window(c.handle, 3, 0, 0) == 1
    assert lib.mesh_set_x_window(c.handle, 0, 0, 1) == 1
    assert lib.mesh_set_x_window(c.handle, 3, 10, 2) == 1
    # a volume reaching past its window is refused
    assert lib.mesh_set_x_window(c.handle, 45, 50, 0) == 0
    p = pkg.make_params(m)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    rc = lib.mesh_count(c.handle, ctypes.c_void_p(A.ctypes.data), 2, 50, 20, 30, 0, ctypes.byref(p),
                        ctypes.byref(nv), ctypes.byref(nf))
    assert rc == 1
    # a halo column is for MarchingTetrahedra / NaiveSurfaceNets slabs
    assert lib.mesh_set_x_window(c.handle, 0, 50, 1) == 0
    rc = lib.mesh_count(c.handle, ctypes.c_void_p(A.ctypes.data), 2, 50, 20, 30, 0, ctypes.byref(p),
                        ctypes.byref(nv), ctypes.byref(nf))
    assert rc == 1
    assert lib.mesh_set_x_window(c.handle, 0, 0, 0) == 0


@pytest.mark.parametrize('alg', ['mt', 'nsn'])
@pytest.mark.parametrize('dtype,iso,eps,rng', [
    (np.float32, np.float32(0.1), np.float32(1e-3), (np.float32(-1.5), np.float32(2.0))),
    (np.float32, 0.0, 1e-3, (0, 1)),
    (np.float64, 0.0, 1e-3, (-3.0, 0.7)),
    (np.uint16, 2000, 1e-3, (-1, 1)),
    (np.int8, 3, np.float32(1e-2), (-1, 1)),
])
def test_mt_and_nsn_slabs_equal_the_whole_volume(pkg, oracle, cuda, alg, dtype, iso, eps, rng):
    # the boundary vertices belong to the lower slab; each slab after the first
    # reads the previous slab's last cell column as a halo
    if dtype == np.int8:
        A = np.asfortranarray((_field((43, 29, 37), np.float64, seed=3) * 60).round().astype(np.int8))
    else:
        A = _field((43, 29, 37), dtype, seed=3)
    m = pkg.MarchingTetrahedra(iso=iso, eps=eps) if alg == 'mt' else pkg.NaiveSurfaceNets(iso=iso)
    want = pkg.isosurface(A, m, rng, rng, rng)
    wv, wf = oracle.isosurface(A, alg, iso, eps, (rng, rng, rng))
    assert np.array_equal(want[1], wf) and np.array_equal(want[0], wv) and len(wf) > 0
    for slab in (1, 2, 5, 13, 41, 42, 100):
        got = pkg.isosurface_slabs(A, m, rng, rng, rng, slab_cells=slab)
        assert got[0].dtype == want[0].dtype
        assert np.array_equal(got[1], want[1]), slab
        assert np.array_equal(got[0].view(np.uint8), want[0].view(np.uint8)), slab
    again = pkg.isosurface(A, m, rng, rng, rng)
    assert np.array_equal(again[1], want[1])


def test_halo_window_is_refused_by_the_device_entry_point(pkg, cuda):
    torch = cuda
    A = torch.rand((20, 20, 20), device='cuda')
    lib, c = pkg.load_library(), pkg.Context(0)
    assert lib.mesh_set_x_window(c.handle, 5, 40, 1) == 0
    with pytest.raises(pkg.MeshError) as ei:
        pkg.isosurface_device(A, pkg.MarchingTetrahedra(iso=np.float32(0.5)),
                              verts=torch.empty((100, 3), device='cuda'),
                              faces=torch.empty((100, 3), dtype=torch.int64, device='cuda'), ctx=c)
    assert ei.value.status == 1
    c.close()
