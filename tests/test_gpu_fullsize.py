"""Full-size checks on the benchmark volume (1024^3 Float32 sines) and the
512^3 UInt16 CT-like volume: properties that do not need the oracle to mesh
the whole volume.

* counts equal sum over cells of the per-case vertex / face counts, computed
  here independently with torch from the oracle's reference-layout tables;
* faces index existing vertices;
* an x slab of cells is a contiguous block of the full output (emission order
  is x-major), so it is compared with the oracle run on that slab:
  connectivity exactly, positions to 2 ulp (the slab's own LinRange nodes can
  differ from the full grid's by rounding);
* the exact float fast path for Float64 positions gives bit-identical output
  to the pure FP64 evaluation.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import pyoracle

MC_CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def case_tables():
    nv = np.zeros(256, np.int64)
    nf = np.zeros(256, np.int64)
    for c in range(1, 255):
        row = list(pyoracle._T['R_MC_VERTS'][c - 1])
        nv[c] = row.index(0) if 0 in row else 12
        o = pyoracle._T['R_MC_CONNECTIVITY'][pyoracle._T['R_MC_EQ_MAPPING'][c - 1] - 1]
        nf[c] = 1 + sum(1 for i in (0, 3, 6, 9) if o[i] != 0)
    return nv, nf


def torch_counts(torch, t, below):
    """sum of per-case counts over all cells; t indexed [x,y,z] (x fastest)."""
    nv_t, nf_t = (torch.from_numpy(a).to(t.device) for a in case_tables())
    nx, ny, nz = t.shape
    v = f = 0
    zs = 64
    for z0 in range(0, nz - 1, zs):
        z1 = min(z0 + zs, nz - 1)
        slab = t[:, :, z0:z1 + 1]
        b = below(slab).to(torch.int32)
        ci = torch.zeros((nx - 1, ny - 1, z1 - z0), dtype=torch.int32, device=t.device)
        for k, (dx, dy, dz) in enumerate(MC_CORNERS):
            ci |= b[dx:nx - 1 + dx, dy:ny - 1 + dy, dz:z1 - z0 + dz] << k
        v += int(nv_t[ci.long()].sum())
        f += int(nf_t[ci.long()].sum())
    return v, f


@pytest.fixture(scope='module')
def sines1024(cuda, pkg):
    import bench
    t = bench.sines_device(1024)
    cuda.cuda.synchronize()
    return t


def run_device(torch, pkg, t, method, ranges, ctx=None):
    v, f = pkg.isosurface(t, method, *ranges, ctx=ctx)
    torch.cuda.synchronize()
    return v, f


def test_sines1024_counts_faces_and_slab(pkg, oracle, cuda, sines1024):
    torch = cuda
    t = sines1024
    m = pkg.MarchingCubes(iso=np.float32(0))
    v, f = run_device(torch, pkg, t, m, ((0, 1),) * 3)
    assert v.dtype == torch.float32 and f.dtype == torch.int64
    cv, cf = torch_counts(torch, t, lambda s: s < 0)
    assert (v.shape[0], f.shape[0]) == (cv, cf)
    assert int(f.min()) >= 1 and int(f.max()) == v.shape[0]
    assert bool(torch.isfinite(v).all())
    # x slab [x0, x1): its vertices start after those of cells x < x0
    x0, x1 = 500, 524
    before_v, before_f = torch_counts(torch, t[:x0 + 1], lambda s: s < 0)
    slab_v, slab_f = torch_counts(torch, t[x0:x1 + 1], lambda s: s < 0)
    A = np.asfortranarray(t[x0:x1 + 1].cpu().numpy())
    nx = t.shape[0]
    ex = [(1 - i / (nx - 1)) * 0.0 + (i / (nx - 1)) * 1.0 for i in (x0, x1)]
    ov, of = oracle.isosurface(A, 'mc', np.float32(0), 1e-3, ((float(ex[0]), float(ex[1])), (0.0, 1.0), (0.0, 1.0)))
    assert (len(ov), len(of)) == (slab_v, slab_f)
    gv = v[before_v:before_v + slab_v].cpu().numpy()
    gf = f[before_f:before_f + slab_f].cpu().numpy()
    assert np.array_equal(gf - before_v, of)
    assert np.array_equal(gv[:, 1:], ov[:, 1:].astype(np.float32))  # y, z nodes are the same LinRange
    err = np.abs(gv[:, 0].astype(np.float64) - ov[:, 0])
    assert (err <= 2 * np.spacing(np.abs(ov[:, 0]).astype(np.float32))).all(), err.max()


def test_fast_path_is_bit_identical_to_fp64(pkg, cuda, sines1024, monkeypatch):
    torch = cuda
    t = sines1024
    m = pkg.MarchingCubes(iso=np.float32(0))
    v1, f1 = run_device(torch, pkg, t, m, ((0, 1),) * 3)
    monkeypatch.setenv('MESHING_GB300_FORCE_FP64', '1')
    ctx = pkg.Context(0)
    v2, f2 = run_device(torch, pkg, t, m, ((0, 1),) * 3, ctx=ctx)
    ctx.close()
    assert torch.equal(f1, f2)
    assert torch.equal(v1.view(torch.int32), v2.view(torch.int32))


def test_ct_u16_512(pkg, oracle, cuda):
    torch = cuda
    import meshing_gb300.fields as fields
    t = fields.ct_like_u16(512)
    m = pkg.MarchingCubes(iso=500)
    v, f = run_device(torch, pkg, t, m, ((-1, 1),) * 3)
    assert v.dtype == torch.float64
    cv, cf = torch_counts(torch, t, lambda s: s.to(torch.int32) < 500)
    assert (v.shape[0], f.shape[0]) == (cv, cf)
    x0, x1 = 200, 216
    before_v, before_f = torch_counts(torch, t[:x0 + 1], lambda s: s.to(torch.int32) < 500)
    slab_v, slab_f = torch_counts(torch, t[x0:x1 + 1], lambda s: s.to(torch.int32) < 500)
    A = np.asfortranarray(t[x0:x1 + 1].cpu().numpy())
    ex = [(1 - i / 511) * -1.0 + (i / 511) * 1.0 for i in (x0, x1)]
    ov, of = oracle.isosurface(A, 'mc', 500, 1e-3, ((float(ex[0]), float(ex[1])), (-1.0, 1.0), (-1.0, 1.0)))
    assert (len(ov), len(of)) == (slab_v, slab_f)
    gv = v[before_v:before_v + slab_v].cpu().numpy()
    gf = f[before_f:before_f + slab_f].cpu().numpy()
    assert np.array_equal(gf - before_v, of)
    assert np.array_equal(gv[:, 1:], ov[:, 1:])
    assert np.abs(gv[:, 0] - ov[:, 0]).max() <= 1e-12


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_tma_walk_matches_global_load_walk(pkg, cuda, alg, monkeypatch):
    # with MESHING_GB300_TMA=1 volumes with 16-byte aligned rows are classified
    # from TMA-staged bricks; the default plain global-load walk must give the
    # same mesh
    torch = cuda
    import meshing_gb300.fields as fields
    t = fields.gyroid(192, dtype=torch.float32)
    m = {'mc': pkg.MarchingCubes, 'nsn': pkg.NaiveSurfaceNets}.get(alg, pkg.MarchingTetrahedra)(iso=np.float32(0))
    v1, f1 = run_device(torch, pkg, t, m, ((0, 1),) * 3)
    monkeypatch.setenv('MESHING_GB300_TMA', '1')
    ctx = pkg.Context(0)
    v2, f2 = run_device(torch, pkg, t, m, ((0, 1),) * 3, ctx=ctx)
    ctx.close()
    assert f1.shape[0] > 0
    assert torch.equal(f1, f2) and torch.equal(v1, v2)
