// K3 (Marching Cubes) -- emit vertices and faces at the scanned offsets.
//
// Replaces process_mc_voxel! (src/marching_cubes.jl:67-92), vertex_interp
// (:100-104) and mc_vert_points (:111-120).
//
// Walk.  The warp tiling is the classify kernel's (31 x-cells by WY y-cells,
// one z segment).  Every lane walks its column in z with a running (vertex,
// face) base per row, so each cell's output lands at the reference position
// base(x, y, seg) + running count.  Chunks whose activity bytes are all zero
// are skipped without touching the volume, and a z step whose corners all lie
// on one side of iso is dismissed with one warp-uniform test.
//
// Emission.  Only ~1-6 % of cells produce output, so emitting from the walking
// lanes would leave most of the warp idle.  Active cells are instead appended
// (ballot + popc) to a per-warp queue in shared memory; once 32 or more are
// queued the warp expands them into one task per output vertex and one per
// face and runs those with all lanes busy.  Consecutive lanes then handle
// consecutive vertices of a cell, so stores to the output are contiguous.
//
// Arithmetic follows Julia's promotion exactly (no FMA contraction):
//   mu = (iso - v1) / (v2 - v1)         in Q (UInt16 differences wrap)
//   p  = p1 + mu * (p2 - p1)             in P = promote(Q, eltype(LinRange))
// then rounded to the output eltype.  On the two axes an edge does not move
// along, p2 - p1 == 0 and the result is p1 itself unless p1 == 0 or mu is not
// finite, in which case the literal expression is evaluated.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_point.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int U = 2;  // z planes loaded ahead (only active chunks are walked)
constexpr int QFLUSH = 32;                  // expand once this many cells are queued
constexpr int QCAP = QFLUSH + TILE_X;        // a row appends at most 31 cells before the next check

// Per-warp queue of active cells of one tile (structure of arrays).
template <class T> struct McQueue {
    T val[8][QCAP];      // corner values, MC corner order
    int32_t z[QCAP];
    uint8_t lr[QCAP];    // lane | row << 5 (x = x0 + lane, y = y0 + row)
    uint8_t cs[QCAP];
    long long vb[QCAP], fb[QCAP];
    int16_t vstart[QCAP], fstart[QCAP];
    uint8_t vmap[QCAP * MC_MAX_VERTS];
    uint8_t fmap[QCAP * MC_MAX_FACES];
};
static_assert(QCAP <= 256, "queue slots are addressed with uint8_t");
constexpr size_t PLAN_BYTES = (sizeof(Plan) + 15) / 16 * 16;

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

// One output vertex: slot k of cell (x, y, z) with case cs, written to verts[out].
// Written without lane-divergent branches except the rare literal p1 + mu*0.
template <class T, class Q, class P>
__device__ __forceinline__ void vertex_task(const Plan &p, const uint64_t *s_v, const McQueue<T> &q, int j, int x,
                                            int y, int z, int64_t out, int k) {
    const int e = (int)((s_v[q.cs[j]] >> (4 * k)) & 15u);
    const int g = edge_info(e);
    const int a = g & 7, b = (g >> 3) & 7, ax = (g >> 6) & 3, neg = (g >> 8) & 1;
    const int xa = x + cdx(a), ya = y + cdy(a), za = z + cdz(a);
    const T va = q.val[a][j];
    const T vbv = q.val[b][j];
    const Q mu = quotient<Q>(va, vbv, p);
    const P m = (P)mu;
    // moving axis: p1 + mu * (+-(p[i+1] - p[i]))
    const int ia = ax == 0 ? xa : (ax == 1 ? ya : za);
    const double *tp = ax == 0 ? p.xp : (ax == 1 ? p.yp : p.zp);
    const double *td = ax == 0 ? p.dx : (ax == 1 ? p.dy : p.dz);
    const float *tpf = ax == 0 ? p.xpf : (ax == 1 ? p.ypf : p.zpf);
    const float *tdf = ax == 0 ? p.dxf : (ax == 1 ? p.dyf : p.dzf);
    const int id = neg ? ia - 1 : ia;
    // still axes: p1 itself unless p1 == 0 or mu is not finite
    const bool fin = isfinite(mu);
    if (p.out64) {
        const P c1 = tab<P>(tp, tpf, ia);
        const P d = tab<P>(td, tdf, id);
        const P rm = Ar<P>::add(c1, Ar<P>::mul(m, neg ? -d : d));
        double o0 = __ldg(p.xp + xa), o1 = __ldg(p.yp + ya), o2 = __ldg(p.zp + za);
        if (!fin || o0 == 0.0 || o1 == 0.0 || o2 == 0.0) {
            o0 = (double)Ar<P>::add((P)o0, Ar<P>::mul(m, P(0)));
            o1 = (double)Ar<P>::add((P)o1, Ar<P>::mul(m, P(0)));
            o2 = (double)Ar<P>::add((P)o2, Ar<P>::mul(m, P(0)));
        }
        double *o = (double *)p.verts + 3 * out;
        o[0] = ax == 0 ? (double)rm : o0;
        o[1] = ax == 1 ? (double)rm : o1;
        o[2] = ax == 2 ? (double)rm : o2;
    } else {
        float fr;
        bool done = false;
        if (sizeof(P) == 8 && sizeof(Q) == 4 && !p.force_fp64) {
            // Float32 mu, Float64 coordinates, Float32 output: exact float fast path
            const int64_t off = (ax == 0 ? 0 : (ax == 1 ? p.nx : p.nx + p.ny));
            const float *sp = p.split;
            const float dh = __ldg(sp + 2 * p.ntab + off + id), dl = __ldg(sp + 3 * p.ntab + off + id);
            done = fin && fast_f32_pos((float)mu, __ldg(sp + off + ia), __ldg(sp + p.ntab + off + ia),
                                       neg ? -dh : dh, neg ? -dl : dl, fr);
        }
        if (!done) {
            const P c1 = tab<P>(tp, tpf, ia);
            const P d = tab<P>(td, tdf, id);
            fr = (float)Ar<P>::add(c1, Ar<P>::mul(m, neg ? -d : d));
        }
        float o0 = __ldg(p.xpf + xa), o1 = __ldg(p.ypf + ya), o2 = __ldg(p.zpf + za);
        if (!fin || o0 == 0.0f || o1 == 0.0f || o2 == 0.0f) {
            o0 = (float)Ar<P>::add(tab<P>(p.xp, p.xpf, xa), Ar<P>::mul(m, P(0)));
            o1 = (float)Ar<P>::add(tab<P>(p.yp, p.ypf, ya), Ar<P>::mul(m, P(0)));
            o2 = (float)Ar<P>::add(tab<P>(p.zp, p.zpf, za), Ar<P>::mul(m, P(0)));
        }
        float *o = (float *)p.verts + 3 * out;
        o[0] = ax == 0 ? fr : o0;
        o[1] = ax == 1 ? fr : o1;
        o[2] = ax == 2 ? fr : o2;
    }
}

// Expand the n queued cells of the tile at (x0, y0) into vertex and face tasks
// and run them on all lanes.  Not inlined: the walk reaches it from several
// unrolled sites.
template <class T, class Q, class P>
__device__ __noinline__ void flush(const Plan *pp, McQueue<T> *qp, int n, const uint64_t *s_v, const uint64_t *s_f,
                                   int lane, int x0, int y0) {
    const Plan &p = *pp;
    McQueue<T> &q = *qp;
    __syncwarp();
    int nv = 0, nf = 0;
    if (lane < n) {
        const uint64_t t = s_v[q.cs[lane]];
        nv = (int)((t >> 48) & 15u);
        nf = (int)((t >> 52) & 7u);
        if (q.vb[lane] + nv > p.verts_cap || q.fb[lane] + nf > p.faces_cap) {
            atomicOr(p.err, ERR_CAPACITY);
            nv = nf = 0;
        }
    }
    int iv = nv, jf = nf;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(FULL, iv, o), b = __shfl_up_sync(FULL, jf, o);
        if (lane >= o) {
            iv += a;
            jf += b;
        }
    }
    // second batch of entries (n <= QCAP < 64)
    const int V0 = __shfl_sync(FULL, iv, 31), F0 = __shfl_sync(FULL, jf, 31);
    int nv2 = 0, nf2 = 0;
    const int j2 = lane + 32;
    if (j2 < n) {
        const uint64_t t = s_v[q.cs[j2]];
        nv2 = (int)((t >> 48) & 15u);
        nf2 = (int)((t >> 52) & 7u);
        if (q.vb[j2] + nv2 > p.verts_cap || q.fb[j2] + nf2 > p.faces_cap) {
            atomicOr(p.err, ERR_CAPACITY);
            nv2 = nf2 = 0;
        }
    }
    int iv2 = nv2, jf2 = nf2;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(FULL, iv2, o), b = __shfl_up_sync(FULL, jf2, o);
        if (lane >= o) {
            iv2 += a;
            jf2 += b;
        }
    }
    const int V = V0 + __shfl_sync(FULL, iv2, 31), F = F0 + __shfl_sync(FULL, jf2, 31);
    if (lane < n) {
        const int vs = iv - nv, fs = jf - nf;
        q.vstart[lane] = (int16_t)vs;
        q.fstart[lane] = (int16_t)fs;
        for (int k = 0; k < nv; k++) q.vmap[vs + k] = (uint8_t)lane;
        for (int k = 0; k < nf; k++) q.fmap[fs + k] = (uint8_t)lane;
    }
    if (j2 < n) {
        const int vs = V0 + iv2 - nv2, fs = F0 + jf2 - nf2;
        q.vstart[j2] = (int16_t)vs;
        q.fstart[j2] = (int16_t)fs;
        for (int k = 0; k < nv2; k++) q.vmap[vs + k] = (uint8_t)j2;
        for (int k = 0; k < nf2; k++) q.fmap[fs + k] = (uint8_t)j2;
    }
    __syncwarp();
    for (int t = lane; t < V; t += 32) {
        const int j = q.vmap[t];
        const int k = t - q.vstart[j];
        const int lr = q.lr[j];
        vertex_task<T, Q, P>(p, s_v, q, j, x0 + (lr & 31), y0 + (lr >> 5), q.z[j], q.vb[j] + k, k);
    }
    for (int t = lane; t < F; t += 32) {
        const int j = q.fmap[t];
        const int k = t - q.fstart[j];
        const unsigned s = (unsigned)(s_f[q.cs[j]] >> (12 * k));
        const int64_t vb = q.vb[j];
        int64_t *o = p.faces + 3 * (q.fb[j] + k);
        o[0] = vb + (s & 15u) + 1;
        o[1] = vb + ((s >> 4) & 15u) + 1;
        o[2] = vb + ((s >> 8) & 15u) + 1;
    }
    __syncwarp();
}

template <class T, class Q, class P>
__global__ void __launch_bounds__(256, 3) k_emit_mc(const Plan p, int nitems) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s_v = reinterpret_cast<uint64_t *>(smem);
    uint64_t *s_f = s_v + 256;
    Plan *s_plan = reinterpret_cast<Plan *>(s_f + 256);
    McQueue<T> *queues = reinterpret_cast<McQueue<T> *>(smem + 2 * 256 * sizeof(uint64_t) + PLAN_BYTES);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_v[i] = MC_CASE_VERTS[i];
        s_f[i] = MC_CASE_FACES[i];
    }
    if (threadIdx.x == 0) *s_plan = p;
    __syncthreads();

    const int lane = threadIdx.x & 31;
    McQueue<T> &q = queues[threadIdx.x >> 5];
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = npieces(p);
    const uint32_t lt = (1u << lane) - 1u;
    int qn = 0;

    // persistent warps: take (y tile, x tile, segment) items in order from a counter
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        const int ty = item % p.tiles_y;
        const int tx = (item / p.tiles_y) % p.tiles_x;
        const int seg = item / (p.tiles_y * p.tiles_x);
        const int xs = tx * TILE_X + lane;
        const int y0 = ty * WY;
        const int zbeg = seg * p.zs;
        const int zend = min(zbeg + p.zs, p.cz);
        const bool cellx = lane < TILE_X && xs < p.cx;

        bool rowok[WY + 1];
        const T *rowp[WY + 1];
#pragma unroll
        for (int r = 0; r <= WY; r++) {
            rowok[r] = xs < p.nx && y0 + r < p.ny;
            rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)(y0 + r) : vol;
        }
        const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
        const uint32_t cellm = __ballot_sync(FULL, cellx);
        int64_t bv[WY], bf[WY];
#pragma unroll
        for (int r = 0; r < WY; r++) {
            bv[r] = bf[r] = 0;
            if (cellx && y0 + r < p.cy) {
                const int64_t i = piece(p, seg, y0 + r, xs);
                bv[r] = p.base[i];
                bf[r] = p.base[np + i];
            }
        }

        uint32_t mlo[WY + 1];
        T lov[WY + 1];  // samples of plane z
        bool have_lo = false;
        const int x0 = tx * TILE_X;
        for (int zc0 = zbeg; zc0 < zend; zc0 += ZC) {
            const int zc1 = min(zc0 + ZC, zend);
            const int chunk = seg * p.chunks_per_seg + (zc0 - zbeg) / ZC;
            uint8_t f = 0;
            if (lane < WY && y0 + lane < p.cy) f = p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane];
            if (!__any_sync(FULL, f != 0)) {
                have_lo = false;
                continue;
            }
            if (!have_lo) {
#pragma unroll
                for (int r = 0; r <= WY; r++) {
                    lov[r] = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zc0) : T(0);
                    mlo[r] = __ballot_sync(FULL, rowok[r] && below(lov[r], p));
                }
                have_lo = true;
            }
            for (int z = zc0; z < zc1; z += U) {
                T v[U][WY + 1];
                const int64_t off = sxy * (int64_t)(z + 1);
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++)
                        v[u][r] = (rowok[r] && z + 1 + u <= zc1) ? ldv(rowp[r] + off + sxy * u) : T(0);
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int zc = z + u;
                    if (zc >= zc1) break;
                    uint32_t mhi[WY + 1];
                    uint32_t all1 = xval, any1 = 0;
#pragma unroll
                    for (int r = 0; r <= WY; r++) {
                        mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                        all1 &= mlo[r] & mhi[r];
                        any1 |= mlo[r] | mhi[r];
                    }
                    if (all1 != xval && any1 != 0) {
#pragma unroll
                        for (int r = 0; r < WY; r++) {
                            const uint32_t and4 = mlo[r] & mlo[r + 1] & mhi[r] & mhi[r + 1];
                            const uint32_t or4 = mlo[r] | mlo[r + 1] | mhi[r] | mhi[r + 1];
                            const uint32_t actm = (or4 | (or4 >> 1)) & ~(and4 & (and4 >> 1)) & cellm;
                            if (actm == 0u || y0 + r >= p.cy) continue;  // warp-uniform
                            // corner values; x+1 from the next lane
                            const T a0 = u == 0 ? lov[r] : v[u == 0 ? 0 : u - 1][r];
                            const T b0 = u == 0 ? lov[r + 1] : v[u == 0 ? 0 : u - 1][r + 1];
                            const T c0 = v[u][r], d0 = v[u][r + 1];
                            const T a1 = shfl_down1(a0), b1 = shfl_down1(b0), c1 = shfl_down1(c0), d1 = shfl_down1(d0);
                            if ((actm >> lane) & 1u) {
                                const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
                                const unsigned c = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
                                const unsigned cm = (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) |
                                                    ((c & 1u) << 4) | ((c >> 1) << 5) | ((d >> 1) << 6) |
                                                    ((d & 1u) << 7);
                                const int slot = qn + __popc(actm & lt);
                                const uint64_t t = s_v[cm];
                                q.val[0][slot] = a0;
                                q.val[1][slot] = a1;
                                q.val[2][slot] = b1;
                                q.val[3][slot] = b0;
                                q.val[4][slot] = c0;
                                q.val[5][slot] = c1;
                                q.val[6][slot] = d1;
                                q.val[7][slot] = d0;
                                q.z[slot] = zc;
                                q.lr[slot] = (uint8_t)(lane | (r << 5));
                                q.cs[slot] = (uint8_t)cm;
                                q.vb[slot] = bv[r];
                                q.fb[slot] = bf[r];
                                bv[r] += (int64_t)((t >> 48) & 15u);
                                bf[r] += (int64_t)((t >> 52) & 7u);
                            }
                            qn += __popc(actm);
                            if (qn >= QFLUSH) {
                                flush<T, Q, P>(s_plan, &q, qn, s_v, s_f, lane, x0, y0);
                                qn = 0;
                            }
                        }
                    }
#pragma unroll
                    for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
                }
#pragma unroll
                for (int r = 0; r <= WY; r++) lov[r] = v[U - 1][r];
            }
        }
        // the queue holds cells of this tile only
        if (qn) {
            flush<T, Q, P>(s_plan, &q, qn, s_v, s_f, lane, x0, y0);
            qn = 0;
        }
    }
}

int emit_grid(const void *fn, size_t smem, int sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * WARPS, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * sms;
}

template <class T, class Q, class P> cudaError_t go(const Plan &p, cudaStream_t s) {
    const size_t sm = 2 * 256 * sizeof(uint64_t) + PLAN_BYTES + WARPS * sizeof(McQueue<T>);
    static int grid = 0;  // per instantiation: resident CTAs on this device
    if (!grid) {
        cudaError_t e = cudaFuncSetAttribute(k_emit_mc<T, Q, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = emit_grid((const void *)k_emit_mc<T, Q, P>, sm, sms);
    }
    const int nitems = p.tiles_x * p.tiles_y * p.nseg;
    cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const int ctas = std::min(grid, (nitems + WARPS - 1) / WARPS);
    k_emit_mc<T, Q, P><<<ctas, 32 * WARPS, sm, s>>>(p, nitems);
    return cudaGetLastError();
}

template <class T> cudaError_t go_t(const Plan &p, int Q64, int P64, cudaStream_t s) {
    if (Q64) return go<T, double, double>(p, s);
    if (P64) return go<T, float, double>(p, s);
    return go<T, float, float>(p, s);
}

}  // namespace

cudaError_t launch_emit_mc(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return go_t<uint16_t>(p, Q64, P64, s);
    case MESH_DT_F32: return go_t<float>(p, Q64, P64, s);
    default: return go<double, double, double>(p, s);
    }
}

}  // namespace mesh
