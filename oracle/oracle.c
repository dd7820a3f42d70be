/*
 * CPU oracle for the isosurface hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A single-threaded restatement of Meshing.jl v0.7.0's `isosurface` for
 * MarchingCubes and MarchingTetrahedra, plus this project's own definition of
 * NaiveSurfaceNets (absent from the reference; parity for it is unpinned).
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * load this file; the product never does.
 *
 * It follows the reference loop for loop:
 *   - classification      src/common.jl:10-29          (strict `<`, NaN is "outside")
 *   - MC driver           src/marching_cubes.jl:27-64  (x outer, z inner; 1-based faces)
 *   - process_mc_voxel!   src/marching_cubes.jl:67-92
 *   - vertex_interp       src/marching_cubes.jl:100-104
 *   - mc_vert_points      src/marching_cubes.jl:111-120
 *   - MT driver           src/marching_tetrahedra.jl:129-163 (Dict-based dedup)
 *   - tetIx / vertId / vertPos / getVertId / voxEdgeId / procVox
 *                         src/marching_tetrahedra.jl:11-127
 * and reproduces Julia's arithmetic:
 *   - promotion: the output eltype is float(promote_type(range, data, iso[, eps]))
 *     (src/marching_cubes.jl:31, src/marching_tetrahedra.jl:131);
 *   - the interpolation quotient (iso - v1)/(v2 - v1) is evaluated in Julia's
 *     promoted types, including UInt16 wraparound of v2 - v1;
 *   - LinRange(a, b, n)[i] = T((1 - t)*a + t*b), t = (i-1)/(n-1) (Base.lerpi);
 *   - min/max propagate NaN and order -0.0 below +0.0 (Base.min/max on floats);
 *   - no fused multiply-add (build with -ffp-contract=off).
 * Float32 operations are done as double operations rounded to float, which is
 * exact for + - * / (double has more than 2*24+2 significand bits).
 * Int32 / Int64 samples travel as their exact int64 bit pattern inside the
 * sample slots (only `below` and `quotient` read sample values); their
 * differences wrap like Julia's machine integers.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ref_luts.h"

enum { ORC_U16 = 1, ORC_F32 = 2, ORC_F64 = 3, ORC_I64 = 4, ORC_I32 = 5, ORC_F16 = 6, ORC_I16 = 7, ORC_I8 = 8, ORC_U8 = 9 };
enum { ORC_MC = 0, ORC_MT = 1, ORC_NSN = 2, ORC_MCW = 3 };
enum { ORC_OK = 0, ORC_EINVAL = 1, ORC_ENOMEM = 2 };

typedef struct {
    void *verts;      /* 3 floats or 3 doubles per vertex (out_bits) */
    int64_t nverts;
    int64_t *faces;   /* 3 int64 per face, 1-based */
    int64_t nfaces;
    int out_bits;
    int64_t cap_v, cap_f;
} orc_mesh;

typedef struct {
    int T, I, E, R;   /* data, iso, eps, range-endpoint types */
    int Q;            /* type of (iso - v1)/(v2 - v1) */
    int A;            /* type of the clamped MT weight */
    int L;            /* LinRange eltype */
    int P;            /* type positions are computed in */
    int O;            /* output eltype float(FT) */
    double iso;       /* iso, exact */
    double isoq;      /* iso as it enters the quotient (Float32(iso) when Q is Float32) */
    double eps_a;     /* eps promoted to A */
    double hi_a;      /* one(T) - eps, in promote(T, E), promoted to A */
    const void *vol;
    int64_t nx, ny, nz;
    int64_t sx;       /* samples per row in memory (nx, or the whole volume's nx for an x window) */
    double *xp, *yp, *zp;
    double *xp_alloc; /* what linrange returned for x (xp is offset into it for an x window) */
} orc_ctx;

static double rnd(int ty, double x) { return ty == ORC_F32 ? (double)(float)x : x; }

static int is_float(int ty) { return ty == ORC_F32 || ty == ORC_F64; }

/* float(promote_type(types...)) for the supported set {UInt16, Int64, Float32, Float64}. */
static int out_type(const int *tys, int n) {
    int any64 = 0, any32 = 0;
    for (int i = 0; i < n; i++) {
        if (tys[i] == ORC_F64) any64 = 1;
        if (tys[i] == ORC_F32) any32 = 1;
    }
    if (any64) return ORC_F64;
    if (any32) return ORC_F32;
    return ORC_F64; /* float(Integer) == Float64 */
}

/* signed machine integers: values travel as Int64 bit patterns in the double slots */
static int is_wide_int(int ty) { return ty == ORC_I32 || ty == ORC_I64 || ty == ORC_I16 || ty == ORC_I8; }
static double pun(int64_t i) {
    double d;
    memcpy(&d, &i, sizeof d);
    return d;
}
static int64_t unpun(double d) {
    int64_t i;
    memcpy(&i, &d, sizeof i);
    return i;
}

/* IEEE binary16 bits -> the value (exact in double). */
static double half_value(uint16_t h) {
    const int s = h >> 15, e = (h >> 10) & 31, m = h & 1023;
    double v;
    if (e == 0) v = ldexp((double)m, -24);                 /* zero, subnormal */
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = ldexp((double)(m | 1024), e - 25);
    return s ? -v : v;
}
/* x rounded to the nearest binary16 (ties to even): Float16(x) in Julia. */
static double round_half(double x) { return (double)(_Float16)x; }

static double load(const orc_ctx *c, int64_t x, int64_t y, int64_t z) {
    int64_t i = x + c->sx * (y + c->ny * z);
    switch (c->T) {
    case ORC_U16: return (double)((const uint16_t *)c->vol)[i];
    case ORC_U8: return (double)((const uint8_t *)c->vol)[i];
    case ORC_I16: return pun((int64_t)((const int16_t *)c->vol)[i]);
    case ORC_I8: return pun((int64_t)((const int8_t *)c->vol)[i]);
    case ORC_F16: return half_value(((const uint16_t *)c->vol)[i]);
    case ORC_F32: return (double)((const float *)c->vol)[i];
    case ORC_I32: return pun((int64_t)((const int32_t *)c->vol)[i]);
    case ORC_I64: return pun(((const int64_t *)c->vol)[i]);
    default: return ((const double *)c->vol)[i];
    }
}

/* `iso_vals[k] < iso` (src/common.jl:11-18): Julia compares mixed types exactly.
 * UInt16 and float values are exact in double; an Int32 / Int64 value x is
 * compared with the (integral or float) iso as x < ceil(iso). */
static int below(const orc_ctx *c, double v) {
    if (!is_wide_int(c->T)) return v < c->iso;
    const int64_t x = unpun(v);
    if (isnan(c->iso)) return 0;
    const double t = ceil(c->iso);
    if (t >= 9223372036854775808.0) return 1;   /* beyond every Int64 */
    if (t < -9223372036854775808.0) return 0;
    return x < (int64_t)t;
}

/* (iso - v1) / (v2 - v1) in Julia's promoted arithmetic (src/marching_cubes.jl:101,
 * src/marching_tetrahedra.jl:48). */
static double quotient(const orc_ctx *c, double v1, double v2) {
    double den;
    if (is_wide_int(c->T)) {
        const int64_t a = unpun(v1), b = unpun(v2);
        /* v2 - v1 in the data type, wrapping */
        const int64_t d = c->T == ORC_I32   ? (int64_t)(int32_t)((uint32_t)b - (uint32_t)a)
                          : c->T == ORC_I16 ? (int64_t)(int16_t)(uint16_t)((uint16_t)b - (uint16_t)a)
                          : c->T == ORC_I8  ? (int64_t)(int8_t)(uint8_t)((uint8_t)b - (uint8_t)a)
                                            : (int64_t)((uint64_t)b - (uint64_t)a);
        if (c->Q == ORC_F32) {  /* Float32 iso: Float32(iso) - Float32(v1), Float32(v2 - v1) */
            const double num = rnd(ORC_F32, (double)(float)c->isoq - (double)(float)a);
            return rnd(ORC_F32, num / (double)(float)d);
        }
        if (c->I == ORC_I64) {  /* Int64 iso: (iso - v1) in Int64 (wrapping for Int64 data), then Int / Int */
            const int64_t n = c->T == ORC_I64 ? (int64_t)((uint64_t)(int64_t)c->iso - (uint64_t)a)
                                              : (int64_t)c->iso - a;
            return (double)n / (double)d;
        }
        return (c->isoq - (double)a) / (double)d;  /* Float64 iso */
    }
    if (c->T == ORC_U16)
        den = (double)(uint16_t)((uint16_t)v2 - (uint16_t)v1); /* UInt16 wraps */
    else if (c->T == ORC_U8)
        den = (double)(uint8_t)((uint8_t)v2 - (uint8_t)v1); /* UInt8 wraps */
    else if (c->T == ORC_F32)
        den = rnd(ORC_F32, v2 - v1);
    else if (c->T == ORC_F16)
        den = round_half(v2 - v1); /* Float16 - Float16: the exact difference, rounded once */
    else
        den = v2 - v1;
    if (c->Q == ORC_F32) {
        double num = rnd(ORC_F32, c->isoq - v1);
        return rnd(ORC_F32, num / den);
    }
    return (c->isoq - v1) / den;
}

/* Base.max / Base.min for IEEE floats: NaN propagates, -0.0 < +0.0. */
static double jl_max(int ty, double x, double y) {
    if (isnan(x) || isnan(y)) return rnd(ty, x - y);
    return signbit(rnd(ty, x - y)) ? y : x;
}
static double jl_min(int ty, double x, double y) {
    if (isnan(x) || isnan(y)) return rnd(ty, x - y);
    return signbit(rnd(ty, x - y)) ? x : y;
}

/* LinRange(a, b, n) node coordinates (Base.lerpi). */
static double *linrange(int L, double a, double b, int64_t n) {
    double *p = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!p) return NULL;
    double aa = rnd(L, a), bb = rnd(L, b);
    int64_t d = n > 1 ? n - 1 : 1;
    for (int64_t i = 0; i < n; i++) {
        double t = (double)i / (double)d;
        p[i] = rnd(L, (1.0 - t) * aa + t * bb);
    }
    return p;
}

/* p1 + mu*(p2 - p1) for one axis (src/marching_cubes.jl:102); p1, p2 are LinRange values. */
static double interp_axis(const orc_ctx *c, double mu, double p1, double p2) {
    double d = rnd(c->L, p2 - p1);
    return rnd(c->P, p1 + rnd(c->P, mu * d));
}

static int push_vert(orc_mesh *m, const double p[3]) {
    if (m->nverts == m->cap_v) {
        int64_t cap = m->cap_v ? m->cap_v * 2 : 1024;
        void *nv = realloc(m->verts, (size_t)cap * 3 * (m->out_bits / 8));
        if (!nv) return ORC_ENOMEM;
        m->verts = nv;
        m->cap_v = cap;
    }
    if (m->out_bits == 32) {
        float *v = (float *)m->verts + 3 * m->nverts;
        v[0] = (float)p[0]; v[1] = (float)p[1]; v[2] = (float)p[2];
    } else {
        double *v = (double *)m->verts + 3 * m->nverts;
        v[0] = p[0]; v[1] = p[1]; v[2] = p[2];
    }
    m->nverts++;
    return ORC_OK;
}

static int push_face(orc_mesh *m, int64_t a, int64_t b, int64_t cc) {
    if (m->nfaces == m->cap_f) {
        int64_t cap = m->cap_f ? m->cap_f * 2 : 1024;
        int64_t *nf = (int64_t *)realloc(m->faces, (size_t)cap * 3 * sizeof(int64_t));
        if (!nf) return ORC_ENOMEM;
        m->faces = nf;
        m->cap_f = cap;
    }
    int64_t *f = m->faces + 3 * m->nfaces;
    f[0] = a; f[1] = b; f[2] = cc;
    m->nfaces++;
    return ORC_OK;
}

/* ------------------------------------------------------------------ MC -- */

static const int MC_CORNER[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};

/* iso_vals and _get_cubeindex (src/marching_cubes.jl:42-53) */
static int mc_case(const orc_ctx *c, int64_t xi, int64_t yi, int64_t zi, double v[8]) {
    int ci = 0;
    for (int k = 0; k < 8; k++) {
        v[k] = load(c, xi + MC_CORNER[k][0], yi + MC_CORNER[k][1], zi + MC_CORNER[k][2]);
        if (below(c, v[k])) ci |= 1 << k;
    }
    return ci;
}

/* mc_vert_points (src/marching_cubes.jl:111-120), only for cells with triangles */
static void mc_points(const orc_ctx *c, int64_t xi, int64_t yi, int64_t zi, double p[8][3]) {
    for (int k = 0; k < 8; k++) {
        p[k][0] = c->xp[xi + MC_CORNER[k][0]];
        p[k][1] = c->yp[yi + MC_CORNER[k][1]];
        p[k][2] = c->zp[zi + MC_CORNER[k][2]];
    }
}

static void vertex_interp(const orc_ctx *c, const double p1[3], const double p2[3], double v1, double v2, double out[3]) {
    double mu = quotient(c, v1, v2);
    for (int k = 0; k < 3; k++) out[k] = rnd(c->O, interp_axis(c, mu, p1[k], p2[k]));
}

static int run_mc(const orc_ctx *c, orc_mesh *m) {
    double v[8], p[8][3], q[3];
    for (int64_t xi = 0; xi + 1 < c->nx; xi++)
        for (int64_t yi = 0; yi + 1 < c->ny; yi++)
            for (int64_t zi = 0; zi + 1 < c->nz; zi++) {
                int ci = mc_case(c, xi, yi, zi, v);
                if (ci == 0 || ci == 255) continue;
                mc_points(c, xi, yi, zi, p);
                int64_t fct = m->nverts;
                const uint8_t *row = R_MC_VERTS[ci - 1];
                for (int i = 0; i < 12; i++) {
                    int vt = row[i];
                    if (vt == 0) break;
                    int a = R_MC_EDGE_LIST[vt - 1][0] - 1, b = R_MC_EDGE_LIST[vt - 1][1] - 1;
                    vertex_interp(c, p[a], p[b], v[a], v[b], q);
                    if (push_vert(m, q)) return ORC_ENOMEM;
                }
                const uint8_t *o = R_MC_CONNECTIVITY[R_MC_EQ_MAPPING[ci - 1] - 1];
                if (push_face(m, fct + 3, fct + 2, fct + 1)) return ORC_ENOMEM;
                for (int i = 0; i < 12; i += 3) {
                    if (o[i] == 0) break;
                    if (push_face(m, fct + o[i + 2], fct + o[i + 1], fct + o[i])) return ORC_ENOMEM;
                }
            }
    return ORC_OK;
}

/* ------------------------------------------------------------------ MT -- */

typedef struct {
    int64_t *keys, *vals;
    int64_t cap, n;
} imap;

static uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

static int imap_grow(imap *h) {
    int64_t cap = h->cap ? h->cap * 2 : 1 << 12;
    int64_t *k = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    int64_t *v = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    if (!k || !v) { free(k); free(v); return ORC_ENOMEM; }
    for (int64_t i = 0; i < cap; i++) k[i] = -1;
    for (int64_t i = 0; i < h->cap; i++) {
        if (h->keys[i] < 0) continue;
        uint64_t s = mix64((uint64_t)h->keys[i]) & (uint64_t)(cap - 1);
        while (k[s] >= 0) s = (s + 1) & (uint64_t)(cap - 1);
        k[s] = h->keys[i];
        v[s] = h->vals[i];
    }
    free(h->keys); free(h->vals);
    h->keys = k; h->vals = v; h->cap = cap;
    return ORC_OK;
}

/* returns slot of key (existing or empty) */
static int64_t imap_slot(const imap *h, int64_t key) {
    uint64_t s = mix64((uint64_t)key) & (uint64_t)(h->cap - 1);
    while (h->keys[s] >= 0 && h->keys[s] != key) s = (s + 1) & (uint64_t)(h->cap - 1);
    return (int64_t)s;
}

/* tetIx (src/marching_tetrahedra.jl:11-18) */
static int tet_ix(int t, int ci) {
    int ix = (0x01 & ci) | ((0x40 & ci) >> 3);
    if (R_subTetsMask[t][0] & ci) ix |= 0x02;
    if (R_subTetsMask[t][1] & ci) ix |= 0x04;
    return ix;
}

/* voxEdgeId (src/marching_tetrahedra.jl:91-95), 1-based edge */
static int vox_edge_id(int t, int te) {
    int a = R_subTets[t][R_tetEdgeCrnrs[te - 1][0] - 1];
    int b = R_subTets[t][R_tetEdgeCrnrs[te - 1][1] - 1];
    return R_voxEdgeIx[a - 1][b - 1];
}

/* vertPos (src/marching_tetrahedra.jl:42-55); e 1-based, x/y/z 0-based voxel */
static void vert_pos(const orc_ctx *c, int e, int64_t x, int64_t y, int64_t z, const double vals[8], double out[3]) {
    int i1 = R_voxEdgeCrnrs[e - 1][0] - 1, i2 = R_voxEdgeCrnrs[e - 1][1] - 1;
    double q = quotient(c, vals[i1], vals[i2]);
    double a = jl_min(c->A, jl_max(c->A, q, c->eps_a), c->hi_a);
    double b = rnd(c->A, 1.0 - a);
    double base[3] = {c->xp[x], c->yp[y], c->zp[z]};
    double d[3] = {rnd(c->L, c->xp[x + 1] - c->xp[x]), rnd(c->L, c->yp[y + 1] - c->yp[y]),
                   rnd(c->L, c->zp[z + 1] - c->zp[z])};
    for (int k = 0; k < 3; k++) {
        double w = rnd(c->A, rnd(c->A, (double)R_voxCrnrPos[i1][k] * b) + rnd(c->A, (double)R_voxCrnrPos[i2][k] * a));
        out[k] = rnd(c->O, rnd(c->P, base[k] + rnd(c->P, w * d[k])));
    }
}

/* getVertId (src/marching_tetrahedra.jl:67-84) */
static int get_vert_id(const orc_ctx *c, imap *h, orc_mesh *m, int e, int64_t x, int64_t y, int64_t z,
                       const double vals[8], int64_t *id) {
    const int64_t *dd = R_voxCrnrPos[R_voxEdgeCrnrs[e - 1][0] - 1];
    int64_t key = R_voxEdgeDir[e - 1] + 7 * (x + dd[0] + c->nx * (y + dd[1] + c->ny * (z + dd[2])));
    if (2 * (h->n + 1) > h->cap && imap_grow(h)) return ORC_ENOMEM;
    int64_t s = imap_slot(h, key);
    if (h->keys[s] == key) { *id = h->vals[s]; return ORC_OK; }
    double pos[3];
    vert_pos(c, e, x, y, z, vals, pos);
    if (push_vert(m, pos)) return ORC_ENOMEM;
    h->keys[s] = key;
    h->vals[s] = m->nverts;
    h->n++;
    *id = m->nverts;
    return ORC_OK;
}

static const int MT_CORNER[8][3] = {{0,0,0},{0,1,0},{1,1,0},{1,0,0},{0,0,1},{0,1,1},{1,1,1},{1,0,1}};

/* Welded Marching Cubes (no counterpart in the reference, whose
 * process_mc_voxel! pushes a fresh vertex for every crossed edge of every cell,
 * src/marching_cubes.jl:72-79): one vertex per crossed lattice edge, numbered
 * when the edge is first met -- cells in the reference's emission order, a
 * cell's edges in its vertex-slot order -- and placed by that first cell's
 * vertex_interp; the faces are the reference's triangles on those ids. */

static int run_mc_welded(const orc_ctx *c, orc_mesh *m) {
    imap h = {0};
    int rc = imap_grow(&h);
    if (rc) return rc;
    double v[8], p[8][3], q[3];
    int64_t ids[12];
    for (int64_t xi = 0; xi + 1 < c->nx && !rc; xi++)
        for (int64_t yi = 0; yi + 1 < c->ny && !rc; yi++)
            for (int64_t zi = 0; zi + 1 < c->nz && !rc; zi++) {
                int ci = mc_case(c, xi, yi, zi, v);
                if (ci == 0 || ci == 255) continue;
                mc_points(c, xi, yi, zi, p);
                const uint8_t *row = R_MC_VERTS[ci - 1];
                for (int i = 0; i < 12; i++) {
                    int vt = row[i];
                    if (vt == 0) break;
                    int a = R_MC_EDGE_LIST[vt - 1][0] - 1, b = R_MC_EDGE_LIST[vt - 1][1] - 1;
                    int ax = MC_CORNER[a][0] != MC_CORNER[b][0] ? 0 : (MC_CORNER[a][1] != MC_CORNER[b][1] ? 1 : 2);
                    int64_t lx = xi + (MC_CORNER[a][0] < MC_CORNER[b][0] ? MC_CORNER[a][0] : MC_CORNER[b][0]);
                    int64_t ly = yi + (MC_CORNER[a][1] < MC_CORNER[b][1] ? MC_CORNER[a][1] : MC_CORNER[b][1]);
                    int64_t lz = zi + (MC_CORNER[a][2] < MC_CORNER[b][2] ? MC_CORNER[a][2] : MC_CORNER[b][2]);
                    int64_t key = ax + 3 * (lx + c->nx * (ly + c->ny * lz));
                    if (2 * (h.n + 1) > h.cap && (rc = imap_grow(&h))) break;
                    int64_t sl = imap_slot(&h, key);
                    if (h.keys[sl] == key) {
                        ids[i] = h.vals[sl];
                        continue;
                    }
                    vertex_interp(c, p[a], p[b], v[a], v[b], q);
                    if ((rc = push_vert(m, q))) break;
                    h.keys[sl] = key;
                    h.vals[sl] = m->nverts;  /* 1-based */
                    h.n++;
                    ids[i] = m->nverts;
                }
                if (rc) break;
                const uint8_t *o = R_MC_CONNECTIVITY[R_MC_EQ_MAPPING[ci - 1] - 1];
                if ((rc = push_face(m, ids[2], ids[1], ids[0]))) break;
                for (int i = 0; i < 12; i += 3) {
                    if (o[i] == 0) break;
                    if ((rc = push_face(m, ids[o[i + 2] - 1], ids[o[i + 1] - 1], ids[o[i] - 1]))) break;
                }
            }
    free(h.keys);
    free(h.vals);
    return rc;
}

static int run_mt(const orc_ctx *c, orc_mesh *m) {
    imap h = {0};
    int rc = imap_grow(&h);
    if (rc) return rc;
    double vals[8];
    for (int64_t i = 0; i + 1 < c->nx && !rc; i++)
        for (int64_t j = 0; j + 1 < c->ny && !rc; j++)
            for (int64_t k = 0; k + 1 < c->nz && !rc; k++) {
                int ci = 0;
                for (int q = 0; q < 8; q++) {
                    vals[q] = load(c, i + MT_CORNER[q][0], j + MT_CORNER[q][1], k + MT_CORNER[q][2]);
                    if (below(c, vals[q])) ci |= 1 << q;
                }
                if (ci == 0 || ci == 255) continue;
                for (int t = 0; t < 6 && !rc; t++) {
                    int tix = tet_ix(t, ci);
                    if (tix == 0 || tix == 15) continue;
                    const uint8_t *e = R_tetTri[tix - 1];
                    int64_t f[3];
                    for (int s = 0; s < 3 && !rc; s++)
                        rc = get_vert_id(c, &h, m, vox_edge_id(t, e[s]), i, j, k, vals, &f[s]);
                    if (rc || (rc = push_face(m, f[0], f[1], f[2]))) break;
                    if (e[3] == 0) continue;
                    for (int s = 0; s < 3 && !rc; s++)
                        rc = get_vert_id(c, &h, m, vox_edge_id(t, e[3 + s]), i, j, k, vals, &f[s]);
                    if (rc || (rc = push_face(m, f[0], f[1], f[2]))) break;
                }
            }
    free(h.keys); free(h.vals);
    return rc;
}

/* ----------------------------------------------------------------- NSN -- */
/* NaiveSurfaceNets as defined by this project (no reference implementation):
 *  - cells classified exactly like MC (MC corner order, strict `<`);
 *  - one vertex per active cell, numbered 1.. in MC traversal order;
 *  - vertex = mean of the crossing points on the cell's crossed edges, taken
 *    in _mc_edge_list order, each crossing point computed like MC's
 *    vertex_interp; sum and division in the position type P, then converted
 *    to the output type;
 *  - for every active cell (x,y,z) in traversal order and axis k = x,y,z: if the
 *    lattice edge from node (x,y,z) along +k is crossed and the cells
 *    A = cell-e_u-e_w, B = cell-e_w, C = cell, D = cell-e_u exist
 *    ((u,w) = (y,z), (z,x), (x,y) for k = x, y, z), emit (A,B,C),(A,C,D) when
 *    the edge's start node is below iso, else (A,C,B),(A,D,C).
 * Vertex ids of neighbouring cells come from a dense per-cell id array. */
static int run_nsn(const orc_ctx *c, orc_mesh *m) {
    int64_t cx = c->nx - 1, cy = c->ny - 1, cz = c->nz - 1;
    if (cx <= 0 || cy <= 0 || cz <= 0) return ORC_OK;
    int64_t *ids = (int64_t *)calloc((size_t)(cx * cy * cz), sizeof(int64_t));
    if (!ids) return ORC_ENOMEM;
    double v[8], p[8][3], q[3];
#define CID(x, y, z) ids[(z) + cz * ((y) + cy * (x))]
    for (int64_t xi = 0; xi < cx; xi++)
        for (int64_t yi = 0; yi < cy; yi++)
            for (int64_t zi = 0; zi < cz; zi++) {
                int ci = mc_case(c, xi, yi, zi, v);
                if (ci == 0 || ci == 255) continue;
                mc_points(c, xi, yi, zi, p);
                double s[3] = {0, 0, 0};
                int n = 0;
                for (int e = 0; e < 12; e++) {
                    int a = R_MC_EDGE_LIST[e][0] - 1, b = R_MC_EDGE_LIST[e][1] - 1;
                    if (((ci >> a) & 1) == ((ci >> b) & 1)) continue;
                    double mu = quotient(c, v[a], v[b]);
                    for (int k = 0; k < 3; k++) s[k] = rnd(c->P, s[k] + interp_axis(c, mu, p[a][k], p[b][k]));
                    n++;
                }
                for (int k = 0; k < 3; k++) q[k] = rnd(c->O, rnd(c->P, s[k] / (double)n));
                if (push_vert(m, q)) { free(ids); return ORC_ENOMEM; }
                CID(xi, yi, zi) = m->nverts;
            }
    for (int64_t xi = 0; xi < cx; xi++)
        for (int64_t yi = 0; yi < cy; yi++)
            for (int64_t zi = 0; zi < cz; zi++) {
                if (CID(xi, yi, zi) == 0) continue;
                int64_t cc[3] = {xi, yi, zi};
                double v0 = load(c, xi, yi, zi);
                for (int k = 0; k < 3; k++) {
                    int u = (k + 1) % 3, w = (k + 2) % 3;
                    if (cc[u] == 0 || cc[w] == 0) continue;
                    int64_t n1[3] = {xi, yi, zi};
                    n1[k] += 1;
                    double v1 = load(c, n1[0], n1[1], n1[2]);
                    int s0 = below(c, v0), s1 = below(c, v1);
                    if (s0 == s1) continue;
                    int64_t a[3] = {xi, yi, zi}, b[3] = {xi, yi, zi}, d[3] = {xi, yi, zi};
                    a[u]--; a[w]--; b[w]--; d[u]--;
                    int64_t A = CID(a[0], a[1], a[2]), B = CID(b[0], b[1], b[2]);
                    int64_t C = CID(xi, yi, zi), D = CID(d[0], d[1], d[2]);
                    int rc;
                    if (s0) rc = push_face(m, A, B, C) || push_face(m, A, C, D);
                    else rc = push_face(m, A, C, B) || push_face(m, A, D, C);
                    if (rc) { free(ids); return ORC_ENOMEM; }
                }
            }
#undef CID
    free(ids);
    return ORC_OK;
}

/* ------------------------------------------------------------- entry ---- */

static int setup(orc_ctx *c, const void *vol, int T, int64_t nx, int64_t ny, int64_t nz, int alg, int I, double iso,
                 int E, double eps, int R, const double *rg) {
    memset(c, 0, sizeof(*c));
    if (T != ORC_U16 && T != ORC_F32 && T != ORC_F64 && T != ORC_I32 && T != ORC_I64 && T != ORC_F16 && T != ORC_I16 &&
        T != ORC_I8 && T != ORC_U8)
        return ORC_EINVAL;
    if (T == ORC_F16 && I == ORC_I64) return ORC_EINVAL; /* promote(Int, Float16): Float16 arithmetic, not restated */
    if (I != ORC_F32 && I != ORC_F64 && I != ORC_I64) return ORC_EINVAL;
    if (R != ORC_F32 && R != ORC_F64 && R != ORC_I64) return ORC_EINVAL;
    if (alg == ORC_MT && E != ORC_F32 && E != ORC_F64) return ORC_EINVAL;
    if (nx < 0 || ny < 0 || nz < 0) return ORC_EINVAL;
    c->T = T; c->I = I; c->E = E; c->R = R;
    c->vol = vol; c->nx = nx; c->ny = ny; c->nz = nz; c->sx = nx;
    c->iso = iso;
    /* promote(typeof(iso), T) for the quotient; Int / Int divides in Float64 */
    int q64 = (T == ORC_F64) || (I == ORC_F64) || (T != ORC_F32 && I == ORC_I64);
    c->Q = q64 ? ORC_F64 : ORC_F32;
    c->isoq = rnd(c->Q, iso);
    c->L = (R == ORC_F32) ? ORC_F32 : ORC_F64;
    int tys[4] = {R, T, I, E};
    if (alg == ORC_MT) {
        c->A = (c->Q == ORC_F64 || E == ORC_F64) ? ORC_F64 : ORC_F32;
        int te = (T == ORC_F64 || E == ORC_F64) ? ORC_F64 : ORC_F32; /* promote(T, E) */
        c->eps_a = eps;
        c->hi_a = rnd(te, 1.0 - rnd(te, eps));
        c->P = (c->A == ORC_F32 && c->L == ORC_F32) ? ORC_F32 : ORC_F64;
        c->O = out_type(tys, 4);
    } else {
        c->P = (c->Q == ORC_F32 && c->L == ORC_F32) ? ORC_F32 : ORC_F64;
        c->O = out_type(tys, 3);
    }
    (void)is_float;
    c->xp = c->xp_alloc = linrange(c->L, rg[0], rg[1], nx);
    c->yp = linrange(c->L, rg[2], rg[3], ny);
    c->zp = linrange(c->L, rg[4], rg[5], nz);
    if (!c->xp || !c->yp || !c->zp) return ORC_ENOMEM;
    return ORC_OK;
}

int orc_output_bits(int T, int alg, int I, int E, int R) {
    int tys[4] = {R, T, I, E};
    return out_type(tys, alg == ORC_MT ? 4 : 3) == ORC_F32 ? 32 : 64;
}

int orc_isosurface(const void *vol, int T, int64_t nx, int64_t ny, int64_t nz, int alg, int I, double iso, int E,
                   double eps, int R, const double *range6, orc_mesh *out) {
    orc_ctx c;
    memset(out, 0, sizeof(*out));
    int rc = setup(&c, vol, T, nx, ny, nz, alg, I, iso, E, eps, R, range6);
    if (!rc) {
        out->out_bits = c.O == ORC_F32 ? 32 : 64;
        if (alg == ORC_MC) rc = run_mc(&c, out);
        else if (alg == ORC_MCW) rc = run_mc_welded(&c, out);
        else if (alg == ORC_MT) rc = run_mt(&c, out);
        else if (alg == ORC_NSN) rc = run_nsn(&c, out);
        else rc = ORC_EINVAL;
    }
    free(c.xp_alloc); free(c.yp); free(c.zp);
    return rc;
}

/* MarchingCubes over the x window of cells x0 .. x1 - 1 (samples x0 .. x1) of a
 * volume of nx samples per row, with the whole volume's LinRange node
 * coordinates.  The reference's loop is x-outermost (src/marching_cubes.jl:40),
 * so the window's mesh is the contiguous block of the whole mesh that follows
 * the vertices and faces of cells x < x0; its faces are numbered from 1 within
 * the window.  Windows of one volume can run on several threads at once. */
int orc_isosurface_mc_xwin(const void *vol, int T, int64_t nx, int64_t ny, int64_t nz, int64_t x0, int64_t x1, int I,
                           double iso, int R, const double *range6, orc_mesh *out) {
    orc_ctx c;
    memset(out, 0, sizeof(*out));
    if (x0 < 0 || x1 < x0 || x1 >= nx) return ORC_EINVAL;
    int rc = setup(&c, vol, T, nx, ny, nz, ORC_MC, I, iso, ORC_F64, 1e-3, R, range6);
    if (!rc) {
        static const int size_of[10] = {0, 2, 4, 8, 8, 4, 2, 2, 1, 1};
        c.vol = (const char *)vol + x0 * size_of[T];
        c.xp = c.xp_alloc + x0;
        c.nx = x1 - x0 + 1;
        out->out_bits = c.O == ORC_F32 ? 32 : 64;
        rc = run_mc(&c, out);
    }
    free(c.xp_alloc); free(c.yp); free(c.zp);
    return rc;
}

void orc_free(orc_mesh *m) {
    free(m->verts); free(m->faces);
    memset(m, 0, sizeof(*m));
}

/* _get_cubeindex (src/common.jl:10-20) on 8 doubles against a double iso. */
int orc_cubeindex(const double *vals, double iso) {
    int ci = 0;
    for (int k = 0; k < 8; k++)
        if (vals[k] < iso) ci |= 1 << k;
    return ci;
}

/* vertex_interp (src/marching_cubes.jl:100-104) with Float64 arithmetic throughout. */
void orc_vertex_interp_f64(double iso, const double *p1, const double *p2, double v1, double v2, double *out) {
    double mu = (iso - v1) / (v2 - v1);
    for (int k = 0; k < 3; k++) out[k] = p1[k] + mu * (p2[k] - p1[k]);
}

/* LinRange node coordinate (for tests of the lerp restatement). */
double orc_linrange_at(int L, double a, double b, int64_t n, int64_t i) {
    double *p = linrange(L, a, b, n);
    double v = p ? p[i] : NAN;
    free(p);
    return v;
}
