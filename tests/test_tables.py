"""The product's flattened per-case tables equal an independent walk of the
reference-layout tables the oracle uses (process_mc_voxel!, procVox)."""
import os
import re

import numpy as np

import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def product_tables():
    src = open(os.path.join(ROOT, 'meshing.jl_gb300', 'csrc', 'mesh_tables.h')).read()
    out = {}
    for m in re.finditer(r'MESH_TBL \w+ (\w+)((?:\[\d+\])+) = \{(.*?)\};', src, re.S):
        name, dims, body = m.group(1), m.group(2), m.group(3)
        nums = [int(x, 0) for x in re.findall(r'0x[0-9a-f]+|\d+', body.replace('ull', '').replace('u', ''))]
        shape = [int(d) for d in re.findall(r'\d+', dims)]
        out[name] = np.array(nums, dtype=object).reshape(shape)
    return out


T = product_tables()
R = pyoracle._T


def test_mc_tables_match_reference_walk():
    for c in range(256):
        tv, tf = int(T['MC_CASE_VERTS'][c]), int(T['MC_CASE_FACES'][c])
        nv, nf = (tv >> 48) & 15, (tv >> 52) & 7
        if c in (0, 255):
            assert nv == 0 and nf == 0
            continue
        # process_mc_voxel! stops at the first zero slot
        row = list(R['R_MC_VERTS'][c - 1])
        edges = [int(e) - 1 for e in row[:row.index(0)]] if 0 in row else [int(e) - 1 for e in row]
        assert [(tv >> (4 * k)) & 15 for k in range(nv)] == edges
        o = R['R_MC_CONNECTIVITY'][R['R_MC_EQ_MAPPING'][c - 1] - 1]
        faces = [(2, 1, 0)]
        for i in (0, 3, 6, 9):
            if o[i] == 0:
                break
            faces.append((int(o[i + 2]) - 1, int(o[i + 1]) - 1, int(o[i]) - 1))
        got = [((tf >> (12 * k)) & 15, (tf >> (12 * k + 4)) & 15, (tf >> (12 * k + 8)) & 15) for k in range(nf)]
        assert got == faces


def test_mt_tables_match_reference_walk():
    for c in range(256):
        faces = []
        if c not in (0, 255):
            for t in range(6):
                m0, m1 = R['R_subTetsMask'][t]
                tix = (c & 1) | ((c & 0x40) >> 3) | (2 if m0 & c else 0) | (4 if m1 & c else 0)
                if tix in (0, 15):
                    continue
                e = R['R_tetTri'][tix - 1]

                def ve(te):
                    a = R['R_subTets'][t][R['R_tetEdgeCrnrs'][te - 1][0] - 1]
                    b = R['R_subTets'][t][R['R_tetEdgeCrnrs'][te - 1][1] - 1]
                    return int(R['R_voxEdgeIx'][a - 1][b - 1]) - 1

                faces.append((ve(e[0]), ve(e[1]), ve(e[2])))
                if e[3] != 0:
                    faces.append((ve(e[3]), ve(e[4]), ve(e[5])))
        assert int(T['MT_CASE_NFACES'][c]) == len(faces)
        flat = [int(x) for x in T['MT_CASE_FACES'][c][:3 * len(faces)]]
        assert flat == [e for f in faces for e in f]
        order = []
        for e in flat:
            if e not in order:
                order.append(e)
        assert int(T['MT_TOUCHED'][c]) == sum(1 << e for e in order)
        assert [int(x) for x in T['MT_TOUCH_ORDER'][c][:len(order)]] == order
        for e in range(19):
            want = sum(1 << x for x in order[:order.index(e)]) if e in order else 0
            assert int(T['MT_BEFORE'][c][e]) == want


def test_mt_geometry_matches_reference():
    assert [list(map(int, r)) for r in T['MT_CORNER_POS']] == [list(map(int, r)) for r in R['R_voxCrnrPos']]
    assert [[int(a), int(b)] for a, b in T['MT_EDGE_CORNERS']] == [[int(a) - 1, int(b) - 1] for a, b in R['R_voxEdgeCrnrs']]
    assert [int(d) for d in T['MT_EDGE_DIR']] == [int(d) for d in R['R_voxEdgeDir']]
