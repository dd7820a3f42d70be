"""Mesh export and post-processing (meshing.jl_gb300/export.py): PLY files (the
reference's etc/output_comparison.jl saves its meshes as PLY) and device vertex
normals (mesh_vertex_normals)."""
import numpy as np
import pytest


@pytest.fixture(scope='module')
def export(pkg):
    import meshing_gb300.export as ex
    return ex


def _mesh(dt=np.float32):
    rng = np.random.default_rng(5)
    v = rng.standard_normal((40, 3)).astype(dt)
    f = rng.integers(1, 41, (70, 3)).astype(np.int64)
    return v, f


@pytest.mark.parametrize('binary', [True, False])
@pytest.mark.parametrize('dt', [np.float32, np.float64])
def test_ply_round_trip(export, tmp_path, binary, dt):
    v, f = _mesh(dt)
    n = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(dt)
    for normals in (None, n):
        p = str(tmp_path / 'm.ply')
        export.write_ply(p, v, f, normals, binary=binary)
        head = open(p, 'rb').read(400).split(b'end_header')[0].decode()
        assert ('property %s x' % ('float' if dt == np.float32 else 'double')) in head
        assert 'element vertex 40' in head and 'element face 70' in head
        v2, f2, n2 = export.read_ply(p)
        assert v2.dtype == dt and np.array_equal(v2, v) and np.array_equal(f2, f)
        assert (n2 is None) == (normals is None)
        if normals is not None:
            assert np.array_equal(n2, n)
    if binary:  # 0-based int32 indices in the file
        export.write_ply(p, v, f)
        raw = open(p, 'rb').read()
        body = raw[raw.index(b'end_header\n') + 11:]
        first = np.frombuffer(body[40 * 3 * np.dtype(dt).itemsize:][:13],
                              dtype=np.dtype([('n', 'u1'), ('i', '<i4', (3,))]))
        assert first['n'][0] == 3 and list(first['i'][0]) == list(f[0] - 1)


def test_ply_rejects_bad_meshes(export, tmp_path):
    v, f = _mesh()
    with pytest.raises(ValueError):
        export.write_ply(str(tmp_path / 'x.ply'), v, f + 100)
    with pytest.raises(TypeError):
        export.write_ply(str(tmp_path / 'x.ply'), v.astype(np.int32), f)


def _reference_normals(v, f):
    v = v.astype(np.float64)
    a, b, c = v[f[:, 0] - 1], v[f[:, 1] - 1], v[f[:, 2] - 1]
    n = np.cross(b - a, c - a)
    acc = np.zeros_like(v)
    for k in range(3):
        np.add.at(acc, f[:, k] - 1, n)
    ln = np.linalg.norm(acc, axis=1, keepdims=True)
    return np.where(ln > 0, acc / np.where(ln > 0, ln, 1), 0)


@pytest.mark.gpu
@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_vertex_normals_on_the_device(pkg, cuda, export, tmp_path, alg):
    torch = cuda
    n = 48
    g = torch.linspace(-1, 1, n, dtype=torch.float64, device='cuda')
    x, y, z = g[:, None, None], g[None, :, None], g[None, None, :]
    A = (torch.sqrt(x * x + y * y + z * z) - 0.6)
    A = A.permute(2, 1, 0).contiguous().permute(2, 1, 0)
    for dt, iso in ((torch.float32, np.float32(0)), (torch.float64, 0.0)):
        m = {'mc': pkg.MarchingCubes, 'mt': pkg.MarchingTetrahedra, 'nsn': pkg.NaiveSurfaceNets}[alg](iso=iso)
        if alg == 'mt' and dt == torch.float32:
            m = pkg.MarchingTetrahedra(iso=iso, eps=np.float32(1e-3))
        rng = (np.float32(-1), np.float32(1)) if dt == torch.float32 else (-1.0, 1.0)
        v, f = pkg.isosurface(A.to(dt), m, rng, rng, rng)
        nrm = export.vertex_normals(v, f)
        assert nrm.dtype == v.dtype and nrm.shape == v.shape
        want = _reference_normals(v.cpu().numpy(), f.cpu().numpy())
        tol = 1e-6 if dt == torch.float32 else 1e-12
        assert np.abs(nrm.cpu().numpy() - want).max() <= tol
        # outward on a sphere (MC / MT / NSN wind faces so that cross products point outwards or inwards
        # consistently): |cos| with the radial direction close to 1 for almost every vertex
        vv = v.cpu().numpy().astype(np.float64)
        cosr = np.abs((nrm.cpu().numpy() * vv).sum(1) / np.linalg.norm(vv, axis=1))
        assert np.median(cosr) > 0.98
        p = str(tmp_path / ('s_%s.ply' % alg))
        export.write_ply(p, v, f, nrm)
        v2, f2, n2 = export.read_ply(p)
        assert np.array_equal(f2, f.cpu().numpy()) and np.array_equal(n2, nrm.cpu().numpy())
    bad = f.clone()
    bad[0, 0] = v.shape[0] + 5
    with pytest.raises(pkg.MeshError) as ei:
        export.vertex_normals(v, bad)
    assert ei.value.status == 4  # MESH_EDEVICE
