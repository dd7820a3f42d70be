// Marching Cubes vertex arithmetic and the expansion kernel, shared by the
// two ways the active-cell entries are produced (k_emit_mc.cu: a second walk
// after the scan, entries in emission order; k_walk_mc.cu: the classify walk
// itself stages the entries, each carrying its rank inside its piece).
//
// Replaces vertex_interp (src/marching_cubes.jl:100-104), mc_vert_points
// (:111-120) and the vertex / face pushes of process_mc_voxel! (:67-92).
//
// Arithmetic follows Julia's promotion exactly (no FMA contraction):
//   mu = (iso - v1) / (v2 - v1)         in Q (UInt16 differences wrap)
//   p  = p1 + mu * (p2 - p1)             in P = promote(Q, eltype(LinRange))
// then rounded to the output eltype.  On the two axes an edge does not move
// along, p2 - p1 == 0 and the result is p1 itself unless p1 == 0 or mu is not
// finite, in which case the literal expression is evaluated.  When P is
// Float64 but mu and the output are Float32, the moving coordinate is
// computed by the exact float path fast_f32_pos and only undecidable cases
// fall back to FP64.
//
// Include once per translation unit, after mesh_tables.h (MESH_TBL defined).
#pragma once
#include "mesh_internal.cuh"
#include "mesh_point.cuh"

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int XW = 256;  // expansion threads per CTA == entries per block
static_assert(XW == ENT_BLOCK, "one expansion CTA per block of entries");

// MC edges (src/lut/mc.jl:606-608) on the corner order of src/marching_cubes.jl:111-120,
// 9 bits per edge: a | b<<3 | moving axis<<6 | negative direction<<8; edges 0-5 in
// EDGE_LO, 6-11 in EDGE_HI, so the lookup needs no (lane-divergent) branch.
#define MC_EDGE(a, b, ax, neg) ((unsigned long long)((a) | (b) << 3 | (ax) << 6 | (neg) << 8))
constexpr unsigned long long EDGE_LO = MC_EDGE(0, 1, 0, 0) | MC_EDGE(1, 2, 1, 0) << 9 | MC_EDGE(2, 3, 0, 1) << 18 |
                                       MC_EDGE(3, 0, 1, 1) << 27 | MC_EDGE(4, 5, 0, 0) << 36 | MC_EDGE(5, 6, 1, 0) << 45;
constexpr unsigned long long EDGE_HI = MC_EDGE(6, 7, 0, 1) | MC_EDGE(7, 4, 1, 1) << 9 | MC_EDGE(0, 4, 2, 0) << 18 |
                                       MC_EDGE(1, 5, 2, 0) << 27 | MC_EDGE(2, 6, 2, 0) << 36 | MC_EDGE(3, 7, 2, 0) << 45;
#undef MC_EDGE
__device__ __forceinline__ int edge_info(int e) {
    const unsigned long long w = e < 6 ? EDGE_LO : EDGE_HI;
    return (int)((w >> (9 * (e < 6 ? e : e - 6))) & 0x1ffu);
}
// corner k of the MC order -> offsets: x 0 1 1 0 0 1 1 0, y 0 0 1 1 0 0 1 1, z 0 0 0 0 1 1 1 1
__device__ __forceinline__ int cdx(int k) { return ((k + 1) >> 1) & 1; }
__device__ __forceinline__ int cdy(int k) { return (k >> 1) & 1; }
__device__ __forceinline__ int cdz(int k) { return (k >> 2) & 1; }

// p1 + mu*d in P, rounded to float: the literal evaluation, kept out of line so
// that the rare cases that need it do not occupy the FP64 pipe for every vertex.
template <class P> __device__ __noinline__ float moving_fp64(double c1, double d, double m) {
    return (float)Ar<P>::add((P)c1, Ar<P>::mul((P)m, (P)d));
}
struct F3 {
    float v[3];
};
// (node pointers by value: a pointer to the table view would put it on the stack)
template <class P>
__device__ __noinline__ F3 still_fp64(const double *xp, const double *yp, const double *zp, const float *xpf,
                                      const float *ypf, const float *zpf, int xa, int ya, int za, double m) {
    F3 o;
    o.v[0] = (float)Ar<P>::add(tab<P>(xp, xpf, xa), Ar<P>::mul((P)m, P(0)));
    o.v[1] = (float)Ar<P>::add(tab<P>(yp, ypf, ya), Ar<P>::mul((P)m, P(0)));
    o.v[2] = (float)Ar<P>::add(tab<P>(zp, zpf, za), Ar<P>::mul((P)m, P(0)));
    return o;
}

// The vertex on MC edge e of cell (x, y, z) with corner values va (start) and
// vbv (end), written to vertex `out` of vout; node coordinates from the
// volume's tables tb.
template <class T, class Q, class P>
__device__ __forceinline__ void vertex_task(const Plan &p, const Tabs &tb, int e, int x, int y, int z, T va, T vbv,
                                            void *vout, int64_t out) {
    const int g = edge_info(e);
    const int a = g & 7, ax = (g >> 6) & 3, neg = (g >> 8) & 1;
    const int xa = x + cdx(a), ya = y + cdy(a), za = z + cdz(a);
    const Q mu = quotient<Q>(va, vbv, p);
    // moving axis: p1 + mu * (+-(p[i+1] - p[i]))
    const int ia = ax == 0 ? xa : (ax == 1 ? ya : za);
    const double *tp = ax == 0 ? tb.xp : (ax == 1 ? tb.yp : tb.zp);
    const double *td = ax == 0 ? tb.dx : (ax == 1 ? tb.dy : tb.dz);
    const float *tpf = ax == 0 ? tb.xpf : (ax == 1 ? tb.ypf : tb.zpf);
    const float *tdf = ax == 0 ? tb.dxf : (ax == 1 ? tb.dyf : tb.dzf);
    const int id = neg ? ia - 1 : ia;
    const bool fin = isfinite(mu);
    if (p.out64) {
        const P m = (P)mu;
        const P c1 = tab<P>(tp, tpf, ia);
        const P d = tab<P>(td, tdf, id);
        const P rm = Ar<P>::add(c1, Ar<P>::mul(m, neg ? -d : d));
        double o0 = __ldg(tb.xp + xa), o1 = __ldg(tb.yp + ya), o2 = __ldg(tb.zp + za);
        if (!fin || o0 == 0.0 || o1 == 0.0 || o2 == 0.0) {
            o0 = (double)Ar<P>::add((P)o0, Ar<P>::mul(m, P(0)));
            o1 = (double)Ar<P>::add((P)o1, Ar<P>::mul(m, P(0)));
            o2 = (double)Ar<P>::add((P)o2, Ar<P>::mul(m, P(0)));
        }
        double *o = (double *)vout + 3 * out;
        o[0] = ax == 0 ? (double)rm : o0;
        o[1] = ax == 1 ? (double)rm : o1;
        o[2] = ax == 2 ? (double)rm : o2;
    } else if (sizeof(P) == 4) {
        const P m = (P)mu;
        const P c1 = tab<P>(tp, tpf, ia);
        const P d = tab<P>(td, tdf, id);
        const float fr = (float)Ar<P>::add(c1, Ar<P>::mul(m, neg ? -d : d));
        float o0 = __ldg(tb.xpf + xa), o1 = __ldg(tb.ypf + ya), o2 = __ldg(tb.zpf + za);
        if (!fin || o0 == 0.0f || o1 == 0.0f || o2 == 0.0f) {
            o0 = (float)Ar<P>::add((P)o0, Ar<P>::mul(m, P(0)));
            o1 = (float)Ar<P>::add((P)o1, Ar<P>::mul(m, P(0)));
            o2 = (float)Ar<P>::add((P)o2, Ar<P>::mul(m, P(0)));
        }
        float *o = (float *)vout + 3 * out;
        o[0] = ax == 0 ? fr : o0;
        o[1] = ax == 1 ? fr : o1;
        o[2] = ax == 2 ? fr : o2;
    } else {
        // Float64 positions rounded to Float32 output
        float fr;
        bool done = false;
        if (sizeof(Q) == 4 && !p.force_fp64) {
            // Float32 mu: exact float fast path
            const int64_t off = (ax == 0 ? 0 : (ax == 1 ? tb.nx : tb.nx + tb.ny));
            const float *sp = tb.split;
            const float dh = __ldg(sp + 2 * tb.ntab + off + id), dl = __ldg(sp + 3 * tb.ntab + off + id);
            done = fin && fast_f32_pos((float)mu, __ldg(sp + off + ia), __ldg(sp + tb.ntab + off + ia),
                                       neg ? -dh : dh, neg ? -dl : dl, fr);
        }
        if (!done) {
            const double d = __ldg(td + id);
            fr = moving_fp64<P>(__ldg(tp + ia), neg ? -d : d, (double)mu);
        }
        F3 ov = {{__ldg(tb.xpf + xa), __ldg(tb.ypf + ya), __ldg(tb.zpf + za)}};
        if (!fin || ov.v[0] == 0.0f || ov.v[1] == 0.0f || ov.v[2] == 0.0f)
            ov = still_fp64<P>(tb.xp, tb.yp, tb.zp, tb.xpf, tb.ypf, tb.zpf, xa, ya, za, (double)mu);
        float *o = (float *)vout + 3 * out;
        o[0] = ax == 0 ? fr : ov.v[0];
        o[1] = ax == 1 ? fr : ov.v[1];
        o[2] = ax == 2 ? fr : ov.v[2];
    }
}

// 8 corner values of an entry, stored contiguously (16-byte aligned: the list's
// value array starts on a 256-byte boundary and an entry holds 8 values).
template <class T> __device__ __forceinline__ void store8(T *dst, const T (&v)[8]);
template <> __device__ __forceinline__ void store8<float>(float *dst, const float (&v)[8]) {
    float4 *d = reinterpret_cast<float4 *>(dst);
    d[0] = make_float4(v[0], v[1], v[2], v[3]);
    d[1] = make_float4(v[4], v[5], v[6], v[7]);
}
template <> __device__ __forceinline__ void store8<double>(double *dst, const double (&v)[8]) {
    double2 *d = reinterpret_cast<double2 *>(dst);
#pragma unroll
    for (int k = 0; k < 4; k++) d[k] = make_double2(v[2 * k], v[2 * k + 1]);
}
template <> __device__ __forceinline__ void store8<uint16_t>(uint16_t *dst, const uint16_t (&v)[8]) {
    uint4 q;
    q.x = v[0] | (uint32_t)v[1] << 16;
    q.y = v[2] | (uint32_t)v[3] << 16;
    q.z = v[4] | (uint32_t)v[5] << 16;
    q.w = v[6] | (uint32_t)v[7] << 16;
    *reinterpret_cast<uint4 *>(dst) = q;
}
template <> __device__ __forceinline__ void store8<int32_t>(int32_t *dst, const int32_t (&v)[8]) {
    int4 *d = reinterpret_cast<int4 *>(dst);
    d[0] = make_int4(v[0], v[1], v[2], v[3]);
    d[1] = make_int4(v[4], v[5], v[6], v[7]);
}
template <> __device__ __forceinline__ void store8<int64_t>(int64_t *dst, const int64_t (&v)[8]) {
    longlong2 *d = reinterpret_cast<longlong2 *>(dst);
#pragma unroll
    for (int k = 0; k < 4; k++) d[k] = make_longlong2(v[2 * k], v[2 * k + 1]);
}
template <> __device__ __forceinline__ void store8<int16_t>(int16_t *dst, const int16_t (&v)[8]) {
    uint4 q;
    q.x = (uint16_t)v[0] | (uint32_t)(uint16_t)v[1] << 16;
    q.y = (uint16_t)v[2] | (uint32_t)(uint16_t)v[3] << 16;
    q.z = (uint16_t)v[4] | (uint32_t)(uint16_t)v[5] << 16;
    q.w = (uint16_t)v[6] | (uint32_t)(uint16_t)v[7] << 16;
    *reinterpret_cast<uint4 *>(dst) = q;
}
template <class T> __device__ __forceinline__ void store8_bytes(T *dst, const T (&v)[8]) {
    uint2 q;
    q.x = (uint8_t)v[0] | (uint32_t)(uint8_t)v[1] << 8 | (uint32_t)(uint8_t)v[2] << 16 | (uint32_t)(uint8_t)v[3] << 24;
    q.y = (uint8_t)v[4] | (uint32_t)(uint8_t)v[5] << 8 | (uint32_t)(uint8_t)v[6] << 16 | (uint32_t)(uint8_t)v[7] << 24;
    *reinterpret_cast<uint2 *>(dst) = q;
}
template <> __device__ __forceinline__ void store8<int8_t>(int8_t *dst, const int8_t (&v)[8]) { store8_bytes(dst, v); }
template <> __device__ __forceinline__ void store8<uint8_t>(uint8_t *dst, const uint8_t (&v)[8]) { store8_bytes(dst, v); }
template <> __device__ __forceinline__ void store8<h16>(h16 *dst, const h16 (&v)[8]) {
    uint4 q;
    q.x = v[0].b | (uint32_t)v[1].b << 16;
    q.y = v[2].b | (uint32_t)v[3].b << 16;
    q.z = v[4].b | (uint32_t)v[5].b << 16;
    q.w = v[6].b | (uint32_t)v[7].b << 16;
    *reinterpret_cast<uint4 *>(dst) = q;
}
template <class T> __device__ __forceinline__ void load8(const T *src, T (&v)[8]);
template <> __device__ __forceinline__ void load8<int16_t>(const int16_t *src, int16_t (&v)[8]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(src);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[2 * k] = (int16_t)(uint16_t)(w[k] & 0xffffu);
        v[2 * k + 1] = (int16_t)(uint16_t)(w[k] >> 16);
    }
}
template <class T> __device__ __forceinline__ void load8_bytes(const T *src, T (&v)[8]) {
    const uint2 q = *reinterpret_cast<const uint2 *>(src);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = (T)(uint8_t)(q.x >> (8 * k));
        v[4 + k] = (T)(uint8_t)(q.y >> (8 * k));
    }
}
template <> __device__ __forceinline__ void load8<int8_t>(const int8_t *src, int8_t (&v)[8]) { load8_bytes(src, v); }
template <> __device__ __forceinline__ void load8<uint8_t>(const uint8_t *src, uint8_t (&v)[8]) { load8_bytes(src, v); }
template <> __device__ __forceinline__ void load8<h16>(const h16 *src, h16 (&v)[8]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(src);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[2 * k].b = (uint16_t)(w[k] & 0xffffu);
        v[2 * k + 1].b = (uint16_t)(w[k] >> 16);
    }
}
template <> __device__ __forceinline__ void load8<int32_t>(const int32_t *src, int32_t (&v)[8]) {
    const int4 a = reinterpret_cast<const int4 *>(src)[0], b = reinterpret_cast<const int4 *>(src)[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <> __device__ __forceinline__ void load8<int64_t>(const int64_t *src, int64_t (&v)[8]) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const longlong2 a = reinterpret_cast<const longlong2 *>(src)[k];
        v[2 * k] = a.x;
        v[2 * k + 1] = a.y;
    }
}
template <> __device__ __forceinline__ void load8<float>(const float *src, float (&v)[8]) {
    const float4 a = reinterpret_cast<const float4 *>(src)[0], b = reinterpret_cast<const float4 *>(src)[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <> __device__ __forceinline__ void load8<double>(const double *src, double (&v)[8]) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double2 a = reinterpret_cast<const double2 *>(src)[k];
        v[2 * k] = a.x;
        v[2 * k + 1] = a.y;
    }
}
template <> __device__ __forceinline__ void load8<uint16_t>(const uint16_t *src, uint16_t (&v)[8]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(src);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[2 * k] = (uint16_t)(w[k] & 0xffffu);
        v[2 * k + 1] = (uint16_t)(w[k] >> 16);
    }
}

// ------------------------------------------------------------ expansion ----
//
// Each CTA takes XW consecutive entries, scans their vertex and face counts,
// and turns them into one task per output vertex and one per face, so that
// consecutive threads write consecutive outputs of an entry and of
// neighbouring entries.
//
// EXP_ORDERED: entries are in emission order (k_compact_mc); every 256th
// entry carries the global vertex / face offsets of its cell (ent_side), the
// others follow by the block scan.  Entries: totals[2].
// EXP_STAGED: entries are in the order the walk found them (k_walk_mc); each
// carries its vertex / face rank inside its piece (ent_rank), and the scanned
// piece offsets give the global ones.  Entries: *stage_next slots, of which
// unused ones have case 0 and emit nothing.
// EXP_BATCH: as EXP_ORDERED over the volumes of a batch in order
// (k_compact_batch); each entry also names its volume (ent_vol), whose
// coordinate tables place its vertices and whose first vertex makes its faces
// 1-based within the volume.

constexpr int EXP_ORDERED = 0, EXP_STAGED = 1, EXP_BATCH = 2;

template <class T> struct ExpandSmem {
    T val[8][XW];
    unsigned long long pos[XW];
    uint32_t vol[XW];  // EXP_BATCH: the entry's volume
    long long vb[XW], fb[XW];  // global offsets of each entry's first vertex / face
    int32_t vs[XW], fs[XW];    // block-local offsets
    uint8_t cs[XW];
    uint8_t vmap[XW * MC_MAX_VERTS];
    uint8_t fmap[XW * MC_MAX_FACES];
    int32_t wsum[2][XW / 32];
};

// Coordinate tables of batch volume v.
__device__ __forceinline__ Tabs batch_tabs(const Plan &p, uint32_t v) {
    const BatchVol &b = p.bvols[v];
    return tabs_at(b.tabs, b.nx, b.ny, b.nz);
}

template <class T, class Q, class P, int MODE>
__global__ void __launch_bounds__(XW) k_expand_mc(const Plan p) {
    constexpr bool STAGED = MODE == EXP_STAGED;
    __shared__ uint64_t s_v[256], s_f[256];
    __shared__ ExpandSmem<T> sm;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_v[i] = MC_CASE_VERTS[i];
        s_f[i] = MC_CASE_FACES[i];
    }
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int64_t na = STAGED ? (int64_t)min(*p.stage_next, (unsigned long long)p.ent_cap) : min(p.totals[2], p.ent_cap);
    // ordered sub-range e_lo .. e_hi - 1: the blocks that hold it, with the
    // entries of those blocks before e_lo counted (offsets) but not emitted
    int64_t e_lo = 0;
    if (MODE == EXP_ORDERED) {
        if (p.e_hi > 0) na = min(na, p.e_hi);
        e_lo = p.e_lo;
    }
    const int64_t nblocks = (na + XW - 1) / XW;
    const int64_t np = p.pstride;
    const uint64_t pmask = (1ull << POS_BITS) - 1;
    const Tabs tb = tabs_of(p);
    __syncthreads();

    for (int64_t blk = e_lo / XW + blockIdx.x; blk < nblocks; blk += gridDim.x) {
        const int64_t e = blk * XW + tid;
        const int skip = (int)max((int64_t)0, e_lo - blk * XW);  // entries of this block before e_lo
        int nv = 0, nf = 0;
        if (e < na) {
            const int cs = p.ent_cs[e];
            const uint64_t t = s_v[cs];
            nv = (int)((t >> 48) & 15u);
            nf = (int)((t >> 52) & 7u);
            if (nv) {
                sm.cs[tid] = (uint8_t)cs;
                const unsigned long long pos = p.ent_pos[e];
                sm.pos[tid] = pos;
                T cv[8];
                load8<T>((const T *)p.ent_val + 8 * e, cv);
#pragma unroll
                for (int k = 0; k < 8; k++) sm.val[k][tid] = cv[k];
                if (MODE == EXP_BATCH) sm.vol[tid] = p.ent_vol[e];
                if (STAGED) {
                    const uint2 rk = p.ent_rank[e];
                    const int z = (int)(pos >> (2 * POS_BITS));
                    const int64_t i = piece(p, z / p.zs, (int)((pos >> POS_BITS) & pmask), (int)(pos & pmask));
                    const long long vb = p.base[i] + rk.x, fb = p.base[np + i] + rk.y;
                    if ((unsigned long long)(vb + nv) > (unsigned long long)p.verts_cap ||
                        (unsigned long long)(fb + nf) > (unsigned long long)p.faces_cap) {
                        atomicOr(p.err, ERR_CAPACITY);
                        nv = nf = 0;
                    }
                    sm.vb[tid] = vb;
                    sm.fb[tid] = fb;
                }
            }
        }
        // block exclusive scan of (nv, nf)
        int iv = nv, jf = nf;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int a = __shfl_up_sync(FULL, iv, o), b = __shfl_up_sync(FULL, jf, o);
            if (lane >= o) {
                iv += a;
                jf += b;
            }
        }
        if (lane == 31) {
            sm.wsum[0][w] = iv;
            sm.wsum[1][w] = jf;
        }
        __syncthreads();
        int wv = 0, wf = 0, V = 0, F = 0;
#pragma unroll
        for (int k = 0; k < XW / 32; k++) {
            const int a = sm.wsum[0][k], b = sm.wsum[1][k];
            if (k < w) {
                wv += a;
                wf += b;
            }
            V += a;
            F += b;
        }
        const int vs = wv + iv - nv, fs = wf + jf - nf;
        sm.vs[tid] = vs;
        sm.fs[tid] = fs;
        for (int k = 0; k < nv; k++) sm.vmap[vs + k] = (uint8_t)tid;
        for (int k = 0; k < nf; k++) sm.fmap[fs + k] = (uint8_t)tid;
        if (!STAGED) {
            const int64_t vb0 = p.ent_side[2 * blk], fb0 = p.ent_side[2 * blk + 1];
            if ((unsigned long long)(vb0 + V) > (unsigned long long)p.verts_cap ||
                (unsigned long long)(fb0 + F) > (unsigned long long)p.faces_cap) {
                if (tid == 0) atomicOr(p.err, ERR_CAPACITY);
                V = F = 0;
            }
            sm.vb[tid] = vb0 + vs;
            sm.fb[tid] = fb0 + fs;
        }
        __syncthreads();
        // the entries before e_lo come first in the block's numbering: start after them
        const int v0 = skip ? sm.vs[skip] : 0, f0 = skip ? sm.fs[skip] : 0;
        for (int t = v0 + tid; t < V; t += XW) {
            const int j = sm.vmap[t];
            const int k = t - sm.vs[j];
            const uint64_t pos = sm.pos[j];
            const int ed = (int)((s_v[sm.cs[j]] >> (4 * k)) & 15u);
            const int g = edge_info(ed);
            void *vout = p.verts;
            int64_t out = sm.vb[j] + k;
            if (MODE == EXP_BATCH && p.vol_outputs) {  // the volume's own outputs
                const BatchVol &b = p.bvols[sm.vol[j]];
                out -= p.vol_off[2 * sm.vol[j]];
                vout = b.verts;
                if (out < 0 || out >= b.vcap) {
                    atomicOr(p.err, ERR_CAPACITY);
                    continue;
                }
            }
            vertex_task<T, Q, P>(p, MODE == EXP_BATCH ? batch_tabs(p, sm.vol[j]) : tb, ed, (int)(pos & pmask),
                                 (int)((pos >> POS_BITS) & pmask), (int)(pos >> (2 * POS_BITS)), sm.val[g & 7][j],
                                 sm.val[(g >> 3) & 7][j], vout, out);
            if ((MODE == EXP_ORDERED || (MODE == EXP_BATCH && !p.vol_outputs)) && p.vkey) {
                // the edge's lower node; the cell owns the edge when, across each
                // other axis, the edge lies on the cell's upper side or the cell is first
                // (in a batch, each volume's keys start at its own base)
                const int x = (int)(pos & pmask), y = (int)((pos >> POS_BITS) & pmask), z = (int)(pos >> (2 * POS_BITS));
                const int a = g & 7, ax = (g >> 6) & 3;
                const int ox = ax == 0 ? 0 : cdx(a), oy = ax == 1 ? 0 : cdy(a), oz = ax == 2 ? 0 : cdz(a);
                const bool own = (ax == 0 || ox || x == 0) && (ax == 1 || oy || y == 0) && (ax == 2 || oz || z == 0);
                int64_t kx = p.nx, ky = p.ny, kb = 0;
                if (MODE == EXP_BATCH) {
                    const BatchVol &b = p.bvols[sm.vol[j]];
                    kx = b.nx;
                    ky = b.ny;
                    kb = b.kbase;
                }
                const long long key =
                    kb + ax + 3 * ((long long)(x + ox) + kx * ((long long)(y + oy) + ky * (long long)(z + oz)));
                p.vkey[out] = key | (own ? (long long)(1ull << 63) : 0ll);
            }
        }
        for (int t = f0 + tid; t < F; t += XW) {
            const int j = sm.fmap[t];
            const int k = t - sm.fs[j];
            const unsigned s = (unsigned)(s_f[sm.cs[j]] >> (12 * k));
            // 1-based within the volume
            const int64_t vb = sm.vb[j] + 1 - (MODE == EXP_BATCH ? p.vol_off[2 * sm.vol[j]] : 0);
            int64_t *o = p.faces + 3 * (sm.fb[j] + k);
            if (MODE == EXP_BATCH && p.vol_outputs) {
                const BatchVol &b = p.bvols[sm.vol[j]];
                const int64_t lf = sm.fb[j] + k - p.vol_off[2 * sm.vol[j] + 1];
                if (lf < 0 || lf >= b.fcap) {
                    atomicOr(p.err, ERR_CAPACITY);
                    continue;
                }
                o = b.faces + 3 * lf;
            }
            o[0] = vb + (s & 15u);
            o[1] = vb + ((s >> 4) & 15u);
            o[2] = vb + ((s >> 8) & 15u);
        }
        __syncthreads();
    }
}

// CTAs of `fn` resident on the whole device at `threads` threads per CTA.
inline int resident_ctas(const void *fn, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * sms;
}


// Shared memory the expansion keeps per SM (KB): its coordinate-table loads hit
// in L1, which gets the rest of the SM's 256 KB.  164 KB hold 6 CTAs (26 KB each
// for Float32 volumes) and leave 92 KB of L1.  1024^3 Float32 sines field:
// 164 KB 0.736 ms, 228 KB (8 CTAs) 0.760, 132 KB (4 CTAs) 0.822, 100 KB 0.951.
#ifndef EXPAND_SMEM_KB
#define EXPAND_SMEM_KB 164
#endif

// Resident CTAs of an expansion kernel with its shared-memory carveout set to
// EXPAND_SMEM_KB: the occupancy calculator's figure, clamped to what the carveout holds.
inline int expand_ctas(const void *fn) {
    int dev = 0, sms = 0, smem_sm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int want = EXPAND_SMEM_KB * 1024;
    if (smem_sm > 0 && want < smem_sm)  // percent of the maximum, rounded down to stay at or under it
        cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)((int64_t)want * 100 / smem_sm));
    cudaGetLastError();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, XW, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess && fa.sharedSizeBytes > 0)
        per_sm = std::max(1, std::min(per_sm, (int)(std::min(want, smem_sm) / (int)(fa.sharedSizeBytes + 1024))));
    cudaGetLastError();
    return per_sm * sms;
}

}  // namespace

}  // namespace mesh
