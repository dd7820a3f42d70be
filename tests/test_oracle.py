"""Pins the CPU oracle to the reference's own known-answer tests (test/runtests.jl)
and cross-checks its two restatements (C and pure Python)."""
import numpy as np
import pytest

import pyoracle


def test_get_cubeindex_kats(oracle):
    # test/runtests.jl:15-27
    assert oracle.cubeindex([0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8], 0.35) == 0x07
    assert oracle.cubeindex([0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1, 1.2], 0.75) == 0x07
    assert oracle.cubeindex([0.9, 0.8, 0.7, 0.6, 0.5, 0.4, 0.3, 0.2], 0.5) == 0xe0


def test_vertex_interp_kats(oracle):
    # test/runtests.jl:29-33
    assert oracle.vertex_interp(0, (0, 0, 0), (0, 1, 0), -1, 1) == (0, 0.5, 0)
    assert oracle.vertex_interp(-1, (0, 0, 0), (0, 1, 0), -1, 1) == (0, 0, 0)
    assert oracle.vertex_interp(1, (0, 0, 0), (0, 1, 0), -1, 1) == (0, 1, 0)


def _norm_sdf(lo, hi, step):
    n = int(round((hi - lo) / step)) + 1
    g = lo + step * np.arange(n)
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    return np.asfortranarray(np.sqrt(X * X + Y * Y + Z * Z))


@pytest.mark.parametrize('alg', ['mc', 'mt'])
def test_respect_origin(oracle, alg):
    # test/runtests.jl:127-149: norm_sdf on -1:0.01:1, iso 0.5, default X/Y/Z
    A = _norm_sdf(-1.0, 1.0, 0.01)
    v, f = oracle.isosurface(A, alg, iso=0.5)
    assert np.allclose(v.mean(axis=0), 0, atol=0.015)
    for i in range(3):
        assert abs(v[:, i].max() - 0.5) <= 0.001
        assert abs(v[:, i].min() + 0.5) <= 0.001
    assert f.min() >= 1 and f.max() <= len(v)


@pytest.mark.parametrize('alg', ['mc', 'mt'])
def test_forward_diff_value(oracle, alg):
    # value part of test/runtests.jl:98-125: mean vertex radius equals iso
    rng = (-2.0, 2.0)
    A = _norm_sdf(-2.0, 2.0, 0.01)
    v, _ = oracle.isosurface(A, alg, iso=0.85, ranges=(rng, rng, rng))
    assert abs(np.linalg.norm(v, axis=1).mean() - 0.85) <= 1e-2


def test_defaults(oracle):
    # test/runtests.jl:76-79: isosurface(A) == isosurface(A, MarchingCubes())
    A = np.random.default_rng(1).random((10, 10, 10))
    a = oracle.isosurface(A)
    b = oracle.isosurface(A, 'mc', iso=0.0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_mixed_types(oracle):
    # test/runtests.jl:81-97: MT on Float64 vs Float32 copies of the same field
    s = np.random.default_rng(9).standard_normal((10, 10, 10))
    r = ((0, 1), (0, 1), (0, 1))
    v1, f1 = oracle.isosurface(s, 'mt', ranges=r)
    v2, f2 = oracle.isosurface(s.astype(np.float32), 'mt', ranges=r)
    assert len(v1) == len(v2) and np.array_equal(f1, f2)


@pytest.mark.parametrize('dtype,iso,eps,rt,alg,bits', [
    (np.float64, 0.2, 1e-4, 4, 'mt', 64),
    (np.float32, np.float32(0.2), np.float32(1e-4), 4, 'mt', 32),
    (np.float64, np.float32(0.2), np.float32(1e-4), 4, 'mt', 64),
    (np.float32, 0.0, 1e-3, 4, 'mc', 64),
    (np.float32, np.float32(0), 1e-3, 4, 'mc', 32),
    (np.float32, 0, 1e-3, 4, 'mc', 32),
    (np.float32, np.float32(0), 1e-3, 3, 'mc', 64),
    (np.uint16, 500, 1e-3, 4, 'mc', 64),
    (np.uint16, np.float32(500), 1e-3, 4, 'mc', 32),
    (np.uint16, 500, 1e-3, 2, 'mc', 32),
    (np.float32, np.float32(0), 1e-3, 4, 'mt', 64),
])
def test_output_eltype_rule(oracle, dtype, iso, eps, rt, alg, bits):
    # test/runtests.jl:35-75: float(promote_type(range, data, iso[, eps]))
    assert oracle.output_bits(dtype, alg, iso, eps, rt) == bits


def _sphere(n, r=0.4):
    g = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    return np.asfortranarray(np.sqrt(X * X + Y * Y + Z * Z) - r)


def test_sphere64_counts(oracle):
    # 64^3 Float64 sphere fixture: counts restated from the reference's counting rules
    A = _sphere(64)
    v, f = oracle.isosurface(A, 'mc')
    assert (len(v), len(f)) == (12000, 5996)
    v, f = oracle.isosurface(A, 'mt')
    assert (len(v), len(f)) == (8978, 17952)


def _edges(f):
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    return e


@pytest.mark.parametrize('alg', ['mt', 'nsn'])
def test_closed_manifold_sphere(oracle, alg):
    # MT (and our NSN) produce watertight, consistently oriented meshes:
    # every directed edge appears once and its reverse once; Euler characteristic 2.
    v, f = oracle.isosurface(_sphere(48, 0.55), alg)
    e = _edges(f)
    key = e[:, 0] * (len(v) + 1) + e[:, 1]
    rkey = e[:, 1] * (len(v) + 1) + e[:, 0]
    assert len(np.unique(key)) == len(key)
    assert np.array_equal(np.sort(key), np.sort(rkey))
    assert len(v) - len(key) // 2 + len(f) == 2
    # outward orientation (increasing values) for NSN: positive signed volume
    if alg == 'nsn':
        p = v[f - 1]
        vol = np.einsum('ij,ij->i', p[:, 0], np.cross(p[:, 1], p[:, 2])).sum() / 6
        assert vol > 0


def test_c_oracle_matches_python_restatement(oracle):
    rng = np.random.default_rng(0)
    cases = [(np.float64, 0.0), (np.float32, np.float32(0.1)), (np.float32, 0.0), (np.float32, 0),
             (np.uint16, 500), (np.uint16, np.float32(300.5)), (np.uint16, 250.25)]
    for trial in range(6):
        sh = tuple(int(s) for s in rng.integers(2, 7, 3))
        for dt, iso in cases:
            if dt == np.uint16:
                A = rng.integers(0, 1000, sh).astype(np.uint16)
            else:
                A = rng.standard_normal(sh).astype(dt)
            for alg in ('mc', 'mt'):
                for eps in ([1e-3, np.float32(1e-3)] if alg == 'mt' else [1e-3]):
                    for rg in (((-1, 1),) * 3, ((np.float32(-2), np.float32(3)),) * 3, ((0.0, 1.5),) * 3):
                        a = oracle.isosurface(A, alg, iso, eps, rg)
                        b = pyoracle.isosurface(A, alg, iso, eps, rg)
                        assert a[0].dtype == b[0].dtype
                        assert np.array_equal(a[1], b[1])
                        assert np.array_equal(a[0], b[0], equal_nan=True)


def test_uint16_wraparound_is_reproduced(oracle):
    # vertex_interp on UInt16 data: v2 - v1 wraps modulo 2^16 (src/marching_cubes.jl:101)
    A = np.zeros((2, 2, 2), np.uint16)
    A[0, 0, 0] = 900  # corner 1 above iso 500, the rest below: edge (1 -> 2) has v2 - v1 = 0 - 900 (wraps)
    v, f = oracle.isosurface(A, 'mc', iso=500)
    mu = (500 - 900) / float((0 - 900) % 65536)
    assert len(v) == 3 and len(f) == 1
    assert np.isclose(v[0, 0], -1 + mu * 2)  # edge 1 runs along +x from x=-1


@pytest.mark.parametrize('dt', [np.int32, np.int64, np.int16, np.int8, np.uint8])
def test_integer_volumes_c_matches_python(oracle, dt):
    # Int32 / Int64 volumes (test/runtests.jl:66-75 runs every algorithm on rand(Int, ...)):
    # exact integer-vs-iso comparison, v2 - v1 wrapping in the data type, and the
    # quotient in promote(typeof(iso), T) -- Int / Int divides in Float64
    rng = np.random.default_rng(int(np.dtype(dt).itemsize))
    info = np.iinfo(dt)
    for trial in range(5):
        sh = tuple(int(s) for s in rng.integers(2, 7, 3))
        full = rng.integers(info.min, info.max, sh, dtype=dt, endpoint=True)  # wrapping differences
        small = rng.integers(-1000, 1000, sh).astype(dt)
        for A, isos in ((full, [0.0, np.float32(1e9), 0, -123456789]), (small, [0.5, np.float32(-3.25), 7, 0.0])):
            A = np.asfortranarray(A)
            for iso in isos:
                for alg in ('mc', 'mt', 'nsn'):
                    for rg in (((-1, 1),) * 3, ((np.float32(-2), np.float32(3)),) * 3):
                        a = oracle.isosurface(A, alg, iso, 1e-3, rg)
                        b = pyoracle.isosurface(A, alg, iso, 1e-3, rg) if alg != 'nsn' else a
                        assert a[0].dtype == b[0].dtype
                        assert np.array_equal(a[1], b[1]), (dt, iso, alg)
                        assert np.array_equal(a[0], b[0], equal_nan=True), (dt, iso, alg)


@pytest.mark.parametrize('dtype,iso,rt,bits', [
    (np.int64, 0.0, 4, 64),            # test/runtests.jl:66-75: rand(Int) data, default iso -> Float64
    (np.int32, 0.0, 4, 64),
    (np.int64, np.float32(0), 4, 32),  # promote(Int64, Float32) == Float32
    (np.int64, 0, 4, 64),              # float(Int64) == Float64
    (np.int32, 0, 2, 32),
])
def test_integer_volume_eltype_rule(oracle, dtype, iso, rt, bits):
    for alg in ('mc', 'mt'):
        eps = np.float32(1e-3) if bits == 32 else 1e-3
        assert oracle.output_bits(dtype, alg, iso, eps, rt) == bits


def test_float16_volumes_c_matches_python(oracle):
    # Float16 volumes (test/runtests.jl:56-65 runs the algorithms on Float16 data): the
    # comparison with iso is exact, v2 - v1 is a Float16 subtraction (one rounding of
    # the exact difference), and the quotient runs in promote(typeof(iso), Float16)
    rng = np.random.default_rng(16)
    for trial in range(6):
        sh = tuple(int(s) for s in rng.integers(2, 7, 3))
        A = np.asfortranarray((rng.standard_normal(sh) * (1 if trial % 2 else 3e4)).astype(np.float16))
        if trial == 5:
            A.ravel(order='K')[:3] = [np.inf, -np.inf, np.nan]
        for iso in (0.0, np.float32(0.25), np.float32(-1e4), 1.5e4):
            for alg in ('mc', 'mt', 'nsn'):
                for rg in (((-1, 1),) * 3, ((np.float32(-2), np.float32(3)),) * 3, ((0.0, 1.0),) * 3):
                    for eps in (1e-3, np.float32(1e-3)):
                        a = oracle.isosurface(A, alg, iso, eps, rg)
                        b = pyoracle.isosurface(A, alg, iso, eps, rg) if alg != 'nsn' else a
                        assert a[0].dtype == b[0].dtype
                        assert np.array_equal(a[1], b[1]), (iso, alg, rg)
                        assert np.array_equal(a[0], b[0], equal_nan=True), (iso, alg, rg)


def test_float16_subtraction_rounds_once(oracle):
    # corner (x+1, y, z) at 1, the rest at -2048, iso 0f0: on the edge from that corner
    # along +y, v2 - v1 = -2048 - 1 = -2049 rounds to -2048 in Float16 (ties to even),
    # so mu = Float32(0 - 1) / Float32(-2048) = 2^-11 exactly and y = -1 + 2 mu
    A = np.full((2, 2, 2), np.float16(-2048), np.float16, order='F')
    A[1, 0, 0] = np.float16(1)
    v, f = oracle.isosurface(A, 'mc', iso=np.float32(0))
    assert len(f) == 1 and v.dtype == np.float32
    assert np.float32(-1 + 2 * 2.0 ** -11) in v[:, 1]
    assert np.float32(-1 + 2 / 2049) not in v[:, 1]


@pytest.mark.parametrize('iso,rt,bits', [
    (0.0, 4, 64),            # default iso: FT = Float64
    (np.float32(0), 4, 32),  # promote(Int range, Float16, Float32) == Float32
    (np.float32(0), 3, 64),  # a Float64 range
])
def test_float16_volume_eltype_rule(oracle, iso, rt, bits):
    for alg in ('mc', 'mt'):
        eps = np.float32(1e-3) if bits == 32 else 1e-3
        assert oracle.output_bits(np.float16, alg, iso, eps, rt) == bits


def test_mc_case_table_puts_a_vertex_on_every_crossed_edge():
    # the welded mode numbers vertices by lattice edge: it relies on every case's vertex
    # slots being exactly its crossed edges (src/lut/mc.jl tables, through ref_luts.h)
    T = pyoracle._T
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    edges = [tuple(int(t) - 1 for t in T['R_MC_EDGE_LIST'][k]) for k in range(12)]
    for ci in range(1, 255):
        slots = [int(s) for s in T['R_MC_VERTS'][ci - 1] if s]
        crossed = {k for k, (a, b) in enumerate(edges) if ((ci >> a) & 1) != ((ci >> b) & 1)}
        assert sorted(s - 1 for s in slots) == sorted(crossed), ci
        assert len(slots) == len(set(slots))
    assert all(sum(abs(corner[a][i] - corner[b][i]) for i in range(3)) == 1 for a, b in edges)


@pytest.mark.parametrize('dt,iso', [(np.float64, 0.0), (np.float32, np.float32(0.1)), (np.uint16, 500)])
def test_welded_mc_is_the_deduplicated_mesh(oracle, dt, iso):
    rng = np.random.default_rng(4)
    for trial in range(4):
        sh = tuple(int(s) for s in rng.integers(2, 12, 3))
        A = rng.integers(0, 1000, sh).astype(dt) if dt == np.uint16 else rng.standard_normal(sh).astype(dt)
        A = np.asfortranarray(A)
        uv, uf = oracle.isosurface(A, 'mc', iso)
        wv, wf = oracle.isosurface(A, 'mcw', iso)
        assert wf.shape == uf.shape and wv.dtype == uv.dtype
        # every welded vertex is the unwelded vertex where its edge first appears: the
        # welded list is an ordered subsequence of the unwelded one
        k = 0
        for j in range(len(uv)):
            if k < len(wv) and np.array_equal(uv[j], wv[k]):
                k += 1
        assert k == len(wv)
        # faces name the same corners: welded face vertices equal the unwelded ones, to
        # rounding where a later cell met the edge from its other end (UInt16 differences
        # wrap differently from the two ends, so there only the first cell's vertex counts)
        if dt != np.uint16:
            assert np.allclose(wv[wf - 1], uv[uf - 1], rtol=0, atol=1e-6)
        assert len(wv) <= len(uv) and (len(uv) == 0 or len(wv) < len(uv) or trial >= 0)
        # welded ids are numbered by first use in the face list's order of cells
        assert wf.min(initial=1) >= 1 and wf.max(initial=0) == len(wv)
        used = np.unique(wf)
        assert len(used) == len(wv)
        assert set(np.arange(1, len(wv) + 1)) == set(used.tolist())


def test_welded_mc_c_matches_python_restatement(oracle):
    # the welded mode restated twice: oracle.c (run_mc_welded) and pyoracle.py (a dict of
    # lattice edges over the plain Marching Cubes loop); positions from the first cell
    # that meets an edge, so UInt16 wraparound and Float16 rounding carry through unchanged
    rng = np.random.default_rng(5)
    cases = [(np.float64, 0.0), (np.float32, np.float32(0.1)), (np.float32, 0.0), (np.uint16, 500),
             (np.uint16, 250.25), (np.int16, 3), (np.float16, np.float32(0.0))]
    for trial in range(4):
        sh = tuple(int(x) for x in rng.integers(2, 8, 3))
        for dt, iso in cases:
            if dt in (np.uint16, np.int16):
                A = rng.integers(0, 1000, sh).astype(dt)
            else:
                A = rng.standard_normal(sh).astype(dt)
            A = np.asfortranarray(A)
            a = oracle.isosurface(A, 'mcw', iso)
            b = pyoracle.isosurface(A, 'mcw', iso)
            assert a[0].dtype == b[0].dtype
            assert np.array_equal(a[1], b[1]), (dt, sh)
            assert np.array_equal(a[0], b[0], equal_nan=True), (dt, sh)


def test_nsn_c_matches_python_restatement(oracle):
    # NaiveSurfaceNets (defined by this project; the reference has none) restated twice:
    # oracle.c (run_nsn) and pyoracle.py, over every scalar-type path and range type
    rng = np.random.default_rng(9)
    cases = [(np.float64, 0.0), (np.float32, np.float32(0.1)), (np.float32, 0.0), (np.uint16, 500),
             (np.uint16, 250.25), (np.int16, 3), (np.float16, np.float32(0.0)), (np.int32, 7)]
    for trial in range(3):
        sh = tuple(int(x) for x in rng.integers(2, 8, 3))
        for dt, iso in cases:
            if dt in (np.uint16, np.int16, np.int32):
                A = rng.integers(0, 1000, sh).astype(dt)
            else:
                A = rng.standard_normal(sh).astype(dt)
            A = np.asfortranarray(A)
            for rg in (((-1, 1),) * 3, ((np.float32(-2), np.float32(3)),) * 3, ((0.0, 1.5),) * 3):
                a = oracle.isosurface(A, 'nsn', iso, 1e-3, rg)
                b = pyoracle.isosurface(A, 'nsn', iso, 1e-3, rg)
                assert a[0].dtype == b[0].dtype
                assert np.array_equal(a[1], b[1]), (dt, sh, rg)
                assert np.array_equal(a[0], b[0], equal_nan=True), (dt, sh, rg)


@pytest.mark.parametrize('n,r', [(48, 0.55), (33, 0.7), (64, 0.4)])
def test_welded_mc_sphere_is_a_closed_sphere(oracle, n, r):
    # welding turns the per-cell Marching Cubes triangles of a sphere into one closed,
    # consistently oriented surface: every directed edge once with its reverse once,
    # Euler characteristic 2, and it encloses the sphere's volume (within 1%)
    v, f = oracle.isosurface(_sphere(n, r), 'mcw')
    e = _edges(f)
    key = e[:, 0] * (len(v) + 1) + e[:, 1]
    rkey = e[:, 1] * (len(v) + 1) + e[:, 0]
    assert len(np.unique(key)) == len(key)
    assert np.array_equal(np.sort(key), np.sort(rkey))
    assert len(v) - len(key) // 2 + len(f) == 2
    p = v[f - 1]
    vol = np.einsum('ij,ij->i', p[:, 0], np.cross(p[:, 1], p[:, 2])).sum() / 6
    assert abs(vol / (4 / 3 * np.pi * r ** 3) - 1) < 0.01


def test_julia_mersenne_twister_stream():
    # rand(MersenneTwister(0), 3) of Julia 1.9 (the values Julia's own
    # documentation examples print for this seed)
    import julia_rand
    assert julia_rand.rand_mersenne_twister(0, 3).tolist() == [0.8236475079774124, 0.9103565379264364,
                                                               0.16456579813368521]


@pytest.mark.parametrize('restatement', ['c', 'python'])
def test_noisy_spheres_kat(oracle, restatement):
    # test/runtests.jl:152-172: MarchingTetrahedra(iso=8.0) on the noisy distance
    # field gives 3466 vertices and 6928 faces
    import julia_rand
    vol = julia_rand.noisy_spheres()
    assert vol.dtype == np.float64 and vol.shape == (21, 21, 21)
    run = oracle.isosurface if restatement == 'c' else pyoracle.isosurface
    v, f = run(vol, 'mt', 8.0)
    assert (len(v), len(f)) == (3466, 6928)


@pytest.mark.parametrize('dt,iso,rg', [(np.float32, np.float32(0.1), ((0, 1),) * 3), (np.uint16, 500, ((-1, 1),) * 3),
                                       (np.float64, 0.0, ((-1.0, 2.5), (0.0, 1.0), (0.0, 1.0)))])
def test_mc_x_windows_concatenate_to_the_whole_mesh(oracle, dt, iso, rg):
    # the reference's MC loop is x-outermost (src/marching_cubes.jl:40): the
    # meshes of consecutive x windows of cells, with the whole volume's nodes,
    # are consecutive blocks of the whole mesh
    rng = np.random.default_rng(5)
    if dt == np.uint16:
        A = np.asfortranarray(rng.integers(0, 1000, (37, 20, 23)).astype(dt))
    else:
        A = np.asfortranarray(rng.standard_normal((37, 20, 23)).astype(dt))
    v, f = oracle.isosurface(A, 'mc', iso, 1e-3, rg)
    ws = oracle.mc_xwindows(A, iso, rg, windows=9, threads=3)
    assert [w[0] for w in ws] == [0] + [w[1] for w in ws[:-1]] and ws[-1][1] == 36
    off = np.cumsum([0] + [len(w[2]) for w in ws[:-1]])
    assert np.array_equal(np.concatenate([w[2] for w in ws]).view(np.uint8), v.view(np.uint8))
    assert np.array_equal(np.concatenate([w[3] + o for w, o in zip(ws, off)]), f)
