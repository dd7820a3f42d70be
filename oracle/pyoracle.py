"""Pure-Python restatement of Meshing.jl's MC / MT -- TEST INFRASTRUCTURE ONLY.

A second, independent restatement of src/marching_cubes.jl:27-120 and
src/marching_tetrahedra.jl:11-163, written with numpy scalar types so that
Julia's promotion is explicit (np.float32 ops are IEEE single, np.uint16
subtraction wraps).  It is slow and only used on small grids to cross-check
the C oracle (oracle.c).  Lookup tables are read from ref_luts.h.
"""
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


def _tables():
    src = open(os.path.join(_HERE, 'ref_luts.h')).read()
    out = {}
    for m in re.finditer(r'static const \w+ (\w+)((?:\[\d+\])+) = \{(.*?)\};', src, re.S):
        name, dims, body = m.group(1), m.group(2), m.group(3)
        nums = [int(x) for x in re.findall(r'-?\d+', body)]
        shape = [int(d) for d in re.findall(r'\d+', dims)]
        out[name] = np.array(nums, dtype=np.int64).reshape(shape)
    return out


_T = _tables()


def _jl_type(v):
    if isinstance(v, np.float32):
        return np.float32
    if isinstance(v, (float, np.float64)):
        return np.float64
    if isinstance(v, (int, np.integer)):
        return np.int64
    raise TypeError(v)


def _promote(*tys):
    tys = set(tys)
    if np.float64 in tys:
        return np.float64
    if np.float32 in tys:
        return np.float32
    if np.float16 in tys:  # promote(Float16, Int) is Float16
        return np.float16
    if np.int64 in tys:
        return np.int64
    if np.int32 in tys:
        return np.int32
    if np.int16 in tys:
        return np.int16
    if np.int8 in tys:
        return np.int8
    if np.uint16 in tys:
        return np.uint16
    return np.uint8


_INTS = (np.uint16, np.int32, np.int64, np.int16, np.int8, np.uint8)


def _float(t):
    return np.float32 if t is np.float32 else np.float64


def _linrange(a, b, n):
    L = _float(_jl_type(a))
    if _jl_type(a) is np.int64:
        L = np.float64
    aa, bb = np.float64(L(a)), np.float64(L(b))
    d = max(n - 1, 1)
    return [L(np.float64((1 - np.float64(i) / d) * aa + (np.float64(i) / d) * bb)) for i in range(n)], L


def _sub(T, a, b):
    """a - b in the promoted type of (T, T) -- machine integers wrap."""
    with np.errstate(over='ignore'):
        return T(a) - T(b)


def _quot(iso, v1, v2):
    """(iso - v1) / (v2 - v1) with Julia's promotion."""
    T = type(v1)
    I = _jl_type(iso)
    den = _sub(T, v2, v1)
    if T in _INTS and I is np.int64:
        # Int / Int: the integer difference (wrapping in Int64), then Float64 division
        return np.float64(_sub(np.int64, np.int64(iso), v1)) / np.float64(den)
    num_t = _promote(T, I)
    if num_t in _INTS:
        num_t = np.float64
    num = num_t(iso) - num_t(v1)
    q_t = _promote(type(num), type(den))
    if q_t in _INTS:
        q_t = np.float64
    return q_t(num) / q_t(den)


def _jl_max(x, y):
    t = _promote(type(x), type(y))
    x, y = t(x), t(y)
    if np.isnan(x) or np.isnan(y):
        return x - y
    return y if np.signbit(x - y) else x


def _jl_min(x, y):
    t = _promote(type(x), type(y))
    x, y = t(x), t(y)
    if np.isnan(x) or np.isnan(y):
        return x - y
    return x if np.signbit(x - y) else y


def _mul(a, b):
    t = _promote(type(a), type(b))
    return t(a) * t(b)


def _add(a, b):
    t = _promote(type(a), type(b))
    return t(a) + t(b)


def isosurface(vol, alg='mc', iso=0.0, eps=1e-3, ranges=((-1, 1), (-1, 1), (-1, 1))):
    vol = np.asfortranarray(vol)
    nx, ny, nz = vol.shape
    T = vol.dtype.type
    R = _jl_type(ranges[0][0])
    weld = alg == 'mcw'  # welded Marching Cubes: one vertex per crossed lattice edge, first touch wins
    if weld:
        alg = 'mc'
    tys = [R, T, _jl_type(iso)] + ([_jl_type(eps)] if alg == 'mt' else [])
    FT = _promote(*tys)
    O = _float(FT) if FT not in _INTS else np.float64
    xp, L = _linrange(ranges[0][0], ranges[0][1], nx)
    yp, _ = _linrange(ranges[1][0], ranges[1][1], ny)
    zp, _ = _linrange(ranges[2][0], ranges[2][1], nz)
    verts, faces = [], []

    def below(v):
        # exact mixed comparison, as Julia's `<` (Python compares int and float exactly)
        if T in _INTS:
            return int(v) < (iso if isinstance(iso, (int, np.integer)) else float(iso))
        return float(v) < float(iso)

    if alg == 'mc':
        corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        welded = {}  # (lower lattice node, axis) -> 1-based welded vertex
        for xi in range(nx - 1):
            for yi in range(ny - 1):
                for zi in range(nz - 1):
                    v = [vol[xi + a, yi + b, zi + c] for a, b, c in corner]
                    ci = sum(1 << k for k in range(8) if below(v[k]))
                    if ci in (0, 255):
                        continue
                    p = [(xp[xi + a], yp[yi + b], zp[zi + c]) for a, b, c in corner]
                    ids = []  # 1-based output index of the cell's k-th vertex
                    for vt in _T['R_MC_VERTS'][ci - 1]:
                        if vt == 0:
                            break
                        a, b = (int(e) - 1 for e in _T['R_MC_EDGE_LIST'][vt - 1])
                        if weld:
                            na = (xi + corner[a][0], yi + corner[a][1], zi + corner[a][2])
                            nb = (xi + corner[b][0], yi + corner[b][1], zi + corner[b][2])
                            key = (min(na, nb), [na[k] != nb[k] for k in range(3)].index(True))
                            if key in welded:
                                ids.append(welded[key])
                                continue
                        mu = _quot(iso, v[a], v[b])
                        verts.append(tuple(O(_add(p[a][k], _mul(mu, p[b][k] - p[a][k]))) for k in range(3)))
                        ids.append(len(verts))
                        if weld:
                            welded[key] = len(verts)
                    o = _T['R_MC_CONNECTIVITY'][_T['R_MC_EQ_MAPPING'][ci - 1] - 1]
                    faces.append((ids[2], ids[1], ids[0]))
                    for i in (0, 3, 6, 9):
                        if o[i] == 0:
                            break
                        faces.append((ids[int(o[i + 2]) - 1], ids[int(o[i + 1]) - 1], ids[int(o[i]) - 1]))
    elif alg == 'mt':
        corner = [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)]
        ids = {}
        pos = _T['R_voxCrnrPos']
        ecr = _T['R_voxEdgeCrnrs']
        for i in range(nx - 1):
            for j in range(ny - 1):
                for k in range(nz - 1):
                    vals = [vol[i + a, j + b, k + c] for a, b, c in corner]
                    ci = sum(1 << q for q in range(8) if below(vals[q]))
                    if ci in (0, 255):
                        continue

                    def vid(e):
                        dx, dy, dz = pos[ecr[e - 1][0] - 1]
                        key = int(_T['R_voxEdgeDir'][e - 1]) + 7 * (i + dx + nx * (j + dy + ny * (k + dz)))
                        if key in ids:
                            return ids[key]
                        i1, i2 = ecr[e - 1][0] - 1, ecr[e - 1][1] - 1
                        q = _quot(iso, vals[i1], vals[i2])
                        te = _promote(T if T is not np.uint16 else _jl_type(eps), _jl_type(eps))
                        hi = te(te(1) - te(eps))
                        a = _jl_min(_jl_max(q, _jl_type(eps)(eps)), hi)
                        at = type(a)
                        b = at(at(1) - a)
                        base = (xp[i], yp[j], zp[k])
                        d = (xp[i + 1] - xp[i], yp[j + 1] - yp[j], zp[k + 1] - zp[k])
                        out = []
                        for ax in range(3):
                            w = at(at(pos[i1][ax]) * b) + at(at(pos[i2][ax]) * a)
                            out.append(O(_add(base[ax], _mul(w, d[ax]))))
                        verts.append(tuple(out))
                        ids[key] = len(verts)
                        return len(verts)

                    for t in range(6):
                        m0, m1 = _T['R_subTetsMask'][t]
                        tix = (ci & 1) | ((ci & 0x40) >> 3) | (2 if m0 & ci else 0) | (4 if m1 & ci else 0)
                        if tix in (0, 15):
                            continue
                        e = _T['R_tetTri'][tix - 1]

                        def ve(te):
                            a = _T['R_subTets'][t][_T['R_tetEdgeCrnrs'][te - 1][0] - 1]
                            b = _T['R_subTets'][t][_T['R_tetEdgeCrnrs'][te - 1][1] - 1]
                            return int(_T['R_voxEdgeIx'][a - 1][b - 1])

                        f = [vid(ve(e[0])), vid(ve(e[1])), vid(ve(e[2]))]
                        faces.append(tuple(f))
                        if e[3] == 0:
                            continue
                        f = [vid(ve(e[3])), vid(ve(e[4])), vid(ve(e[5]))]
                        faces.append(tuple(f))
    elif alg == 'nsn':
        # NaiveSurfaceNets as this project defines it (the reference has none): one vertex
        # per active cell at the mean of its Marching Cubes edge crossings (summed from 0
        # in P, divided in Float64 and rounded to P, then to the output type); one quad per
        # crossed lattice edge with four cells around it, split into two triangles
        # oriented by which end of the edge lies below iso
        corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        cid = {}
        for xi in range(nx - 1):
            for yi in range(ny - 1):
                for zi in range(nz - 1):
                    v = [vol[xi + a, yi + b, zi + c] for a, b, c in corner]
                    ci = sum(1 << k for k in range(8) if below(v[k]))
                    if ci in (0, 255):
                        continue
                    p = [(xp[xi + a], yp[yi + b], zp[zi + c]) for a, b, c in corner]
                    acc, n = None, 0
                    for e in range(12):
                        a, b = (int(t) - 1 for t in _T['R_MC_EDGE_LIST'][e])
                        if ((ci >> a) & 1) == ((ci >> b) & 1):
                            continue
                        mu = _quot(iso, v[a], v[b])
                        x = [_add(p[a][k], _mul(mu, p[b][k] - p[a][k])) for k in range(3)]
                        if acc is None:
                            acc = [type(x[k])(0) for k in range(3)]
                        acc = [_add(acc[k], x[k]) for k in range(3)]
                        n += 1
                    Pt = type(acc[0])
                    verts.append(tuple(O(Pt(np.float64(acc[k]) / np.float64(n))) for k in range(3)))
                    cid[(xi, yi, zi)] = len(verts)
        for xi in range(nx - 1):
            for yi in range(ny - 1):
                for zi in range(nz - 1):
                    if (xi, yi, zi) not in cid:
                        continue
                    cc = (xi, yi, zi)
                    s0 = below(vol[xi, yi, zi])
                    for k in range(3):
                        u, w = (k + 1) % 3, (k + 2) % 3
                        if cc[u] == 0 or cc[w] == 0:
                            continue
                        n1 = list(cc)
                        n1[k] += 1
                        if below(vol[n1[0], n1[1], n1[2]]) == s0:
                            continue
                        a, b, d = list(cc), list(cc), list(cc)
                        a[u] -= 1
                        a[w] -= 1
                        b[w] -= 1
                        d[u] -= 1
                        A, B, C, D = cid[tuple(a)], cid[tuple(b)], cid[cc], cid[tuple(d)]
                        if s0:
                            faces += [(A, B, C), (A, C, D)]
                        else:
                            faces += [(A, C, B), (A, D, C)]
    else:
        raise ValueError(alg)
    V = np.array(verts, dtype=O).reshape(-1, 3)
    F = np.array(faces, dtype=np.int64).reshape(-1, 3)
    return V, F
