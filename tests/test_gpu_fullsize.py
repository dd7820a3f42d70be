"""Full-size checks on the benchmark volume (1024^3 Float32 sines) and the
512^3 UInt16 CT-like volume.

* the whole mesh is compared with the oracle bit for bit: the oracle meshes
  consecutive x windows of cells with the whole volume's LinRange nodes on
  all host cores (the reference's loop is x-outermost, src/marching_cubes.jl:40,
  so each window's mesh is one contiguous block of the whole mesh), and every
  vertex (as bits) and every face of the GPU mesh is checked against it;
* counts also equal the sum over cells of the per-case vertex / face counts,
  computed here independently with torch from the oracle's reference-layout
  tables;
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


def assert_whole_mesh(v, f, windows):
    """GPU mesh (host numpy) == the oracle's x-window blocks, bit for bit."""
    ibits = np.uint32 if v.dtype == np.float32 else np.uint64
    vb = v.view(ibits)
    vo = fo = 0
    for x0, x1, ov, of in windows:
        nv, nf = len(ov), len(of)
        assert ov.dtype == v.dtype, (x0, x1)
        assert np.array_equal(vb[vo:vo + nv], ov.view(ibits)), ('vertices differ in cells x0..x1-1', x0, x1)
        assert np.array_equal(f[fo:fo + nf] - vo, of), ('faces differ in cells x0..x1-1', x0, x1)
        vo += nv
        fo += nf
    assert (vo, fo) == (len(v), len(f))


def test_sines1024_whole_mesh_bit_exact(pkg, oracle, cuda, sines1024):
    torch = cuda
    t = sines1024
    m = pkg.MarchingCubes(iso=np.float32(0))
    v, f = run_device(torch, pkg, t, m, ((0, 1),) * 3)
    assert v.dtype == torch.float32 and f.dtype == torch.int64
    cv, cf = torch_counts(torch, t, lambda s: s < 0)
    assert (v.shape[0], f.shape[0]) == (cv, cf)
    A = t.cpu().numpy()
    assert A.flags['F_CONTIGUOUS'] and A.shape == (1024, 1024, 1024)
    windows = oracle.mc_xwindows(A, np.float32(0), ((0, 1),) * 3, windows=128)
    assert_whole_mesh(v.cpu().numpy(), f.cpu().numpy(), windows)


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


def test_ct_u16_512_whole_mesh_bit_exact(pkg, oracle, cuda):
    torch = cuda
    import meshing_gb300.fields as fields
    t = fields.ct_like_u16(512)
    m = pkg.MarchingCubes(iso=500)
    v, f = run_device(torch, pkg, t, m, ((-1, 1),) * 3)
    assert v.dtype == torch.float64
    cv, cf = torch_counts(torch, t, lambda s: s.to(torch.int32) < 500)
    assert (v.shape[0], f.shape[0]) == (cv, cf)
    A = t.cpu().numpy()
    assert A.flags['F_CONTIGUOUS']
    windows = oracle.mc_xwindows(A, 500, ((-1, 1),) * 3, windows=64)
    assert_whole_mesh(v.cpu().numpy(), f.cpu().numpy(), windows)


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_tma_walk_matches_global_load_walk(pkg, cuda, alg, monkeypatch):
    # volumes with 16-byte aligned rows are classified from TMA-staged bricks
    # (by default for MarchingCubes; MESHING_GB300_TMA=1 for all, =0 for none);
    # the plain global-load walk must give the same mesh
    torch = cuda
    import meshing_gb300.fields as fields
    t = fields.gyroid(192, dtype=torch.float32)
    m = {'mc': pkg.MarchingCubes, 'nsn': pkg.NaiveSurfaceNets}.get(alg, pkg.MarchingTetrahedra)(iso=np.float32(0))
    got = {}
    for env in ('0', '1'):
        monkeypatch.setenv('MESHING_GB300_TMA', env)
        ctx = pkg.Context(0)
        got[env] = run_device(torch, pkg, t, m, ((0, 1),) * 3, ctx=ctx)
        ctx.close()
    assert got['0'][1].shape[0] > 0
    assert torch.equal(got['0'][1], got['1'][1]) and torch.equal(got['0'][0], got['1'][0])


@pytest.mark.parametrize('shape,dt,iso', [
    ((36, 33, 4), 'f32', np.float32(0.02)),       # one box, one stage
    ((100, 70, 45), 'f32', np.float32(-0.1)),     # ragged tiles, a short last stage
    ((128, 97, 203), 'f32', np.float32(0.3)),     # several segments, partial rows of CTAs
    ((64, 41, 61), 'f64', 0.0),
    ((96, 50, 77), 'u16', 500),
])
def test_tma_marching_cubes_walk_on_ragged_volumes(pkg, oracle, cuda, shape, dt, iso, monkeypatch):
    # the Marching Cubes TMA walk (default) against the load walk and the oracle,
    # bit for bit, on shapes that exercise edge tiles, short stages and chunks
    torch = cuda
    rng = np.random.default_rng(sum(shape))
    g = [np.linspace(-1, 1, n) for n in shape]
    X, Y, Z = np.meshgrid(*g, indexing='ij')
    f = np.sin(5 * X) * np.cos(4 * Y + 0.3) + np.sin(3 * Z) * np.cos(5 * X) + 0.05 * rng.standard_normal(shape)
    A = {'f32': f.astype(np.float32), 'f64': f, 'u16': np.round((f + 2) * 250).astype(np.uint16)}[dt]
    A = np.asfortranarray(A)
    vol = torch.from_numpy(np.ascontiguousarray(A.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    m = pkg.MarchingCubes(iso=iso)
    got = {}
    for env in ('1', '0'):
        monkeypatch.setenv('MESHING_GB300_TMA', env)
        ctx = pkg.Context(0)
        got[env] = run_device(torch, pkg, vol, m, ((-1, 1),) * 3, ctx=ctx)
        ctx.close()
    wv, wf = oracle.isosurface(A, 'mc', iso, 1e-3, ((-1, 1),) * 3)
    assert len(wf) > 0
    for env in ('1', '0'):
        assert np.array_equal(got[env][1].cpu().numpy(), wf), env
        assert np.array_equal(got[env][0].cpu().numpy().view(np.uint8), wv.view(np.uint8)), env


def test_u8_1700_past_2_32_samples_whole_mesh_bit_exact(pkg, oracle, cuda):
    # 1700^3 UInt8 = 4.91 G samples (more than 2^32): every 64-bit sample,
    # piece, list and output index path, and the walks' segment-relative
    # 32-bit offsets, against the oracle over the whole volume.  Three
    # low-frequency plane waves give surface through the whole volume; the
    # Float32 iso makes the quotient Float32 with UInt8 differences wrapping.
    torch = cuda
    import math
    n = 1700
    rng = np.random.default_rng(17)
    g = torch.linspace(0.0, 1.0, n, dtype=torch.float64, device='cuda').to(torch.float32)
    terms = []
    for _ in range(3):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        terms.append((rng.uniform(1, 2) * d, rng.uniform(0, 2 * math.pi)))
    vol = torch.empty((n, n, n), dtype=torch.uint8, device='cuda')   # [z, y, x]
    for k in range(n):
        acc = torch.zeros((n, n), dtype=torch.float32, device='cuda')
        for w, ph in terms:
            acc += torch.sin((2 * math.pi * w[0]) * g[None, :] + (2 * math.pi * w[1]) * g[:, None]
                             + float(2 * math.pi * w[2] * g[k].item() + ph))
        vol[k] = (acc * 40 + 128).round_().clamp_(0, 255).to(torch.uint8)
    t = vol.permute(2, 1, 0)
    iso = np.float32(127.5)
    m = pkg.MarchingCubes(iso=iso)
    v, f = run_device(torch, pkg, t, m, ((np.float32(0), np.float32(1)),) * 3)
    assert v.dtype == torch.float32 and v.shape[0] > 0
    A = t.cpu().numpy()
    assert A.flags['F_CONTIGUOUS'] and A.size > 2 ** 32
    windows = oracle.mc_xwindows(A, iso, ((np.float32(0), np.float32(1)),) * 3, windows=200)
    assert_whole_mesh(v.cpu().numpy(), f.cpu().numpy(), windows)
