// K3 (Marching Tetrahedra, Naive Surface Nets) -- emit with neighbour lookups.
//
// MT shares vertices between cells: the reference keys every lattice edge in
// a Dict and numbers a vertex when a cell first touches its edge in
// traversal order, computing its position from that first cell
// (getVertId/vertPos, src/marching_tetrahedra.jl:42-84; procVox :105-127).
// Here the same numbering is derived without a hash table:
//   * the first cell to touch a lattice edge is the owner: the cell reached by
//     stepping -1 along every axis on which both edge corners sit at 0, as far
//     as the grid allows (traversal order is lexicographic, x slowest);
//   * a cell's new vertices are its owned crossed edges, numbered in the
//     cell's first-use order (MT_BEFORE gives the rank), after all vertices
//     of earlier cells (the scanned per-piece base);
//   * a cell that uses an edge owned by a neighbour reads the neighbour's case
//     and base and recomputes the rank.
// NSN gives every active cell one vertex and connects the four cells around
// every crossed base edge, so it needs the same neighbour bases.
//
// Tiling: 30 x-cells (lanes 1..30) plus the -x neighbour (lane 0) by WY
// y-cells plus the -y neighbour row, one z segment; lane 31 only supplies
// samples.  Warps are persistent and take their tiles from a work counter.
// Per z step the warp classifies its cells lane by lane, then stages the step
// in its shared memory -- the sample values of both planes, the cases and
// vertex bases of the current and previous plane, each cell's first face --
// with the inclusive prefix of the cells' vertex and face counts in (lane,
// row) order.  All 32 lanes then work through the step's vertices and faces
// as dense task lists (task t -> its cell by binary search over the prefix;
// NSN vertices through a per-step table, one vertex per active cell), so a
// warp instruction serves up to 32 vertices or faces instead of the few
// active cells of one row.  NSN expands each round of cells into its (cell,
// crossed edge) pairs so that the Float64 crossing points run with full
// warps, and divides the means 32 at a time from a per-warp queue.
// Neighbour lookups are plain shared loads.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_point.cuh"

#include <algorithm>
#include <mutex>

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int R = WY + 1;  // cell rows per tile including the -y neighbour row
constexpr int NSN_VC = 10; // NSN: cells per vertex round (three lanes per cell add up its points)

struct MtTables {
    uint8_t faces[256][3 * MT_MAX_FACES];
    uint8_t nfaces[256];
    uint8_t za[19];          // axes on which both corners of the edge are 0
    uint8_t shifted[19][8];  // the same lattice edge seen from the cell shifted by -s
    uint8_t kth0[256][MT_MAX_TOUCH];  // interior cells: the k-th owned edge in first-use order
    uint8_t rank0[256][19];           // interior cells: rank of edge e among the owned edges
    uint32_t mtw[256];  // by MC case: MT case | interior vertex count << 8 | face count << 13
};

// One warp's state of a z step.
template <class T> struct HaloWarp {
    T samp[2][R + 1][32];        // samples of plane z (samp[cur ^ 1]) and z+1 (samp[cur])
    uint8_t cas[2][R][32];       // cases of the cells of planes z-1 (cur ^ 1) and z (cur)
    long long base[2][R][32];    // their first vertex
    long long fbase[R][32];      // first face of the cells of plane z
    uint16_t pv[R * 32], pf[R * 32];  // inclusive prefix of vertex / face tasks over (lane, row)
};

// NSN: a round of vertex tasks as (cell, crossed edge) pairs.
struct NsnPairs {
    double pt[32][3];    // crossing points of the round's (at most 32) pairs
    // vertices whose sums are complete, waiting for their mean: divided 32 at
    // a time, so that the Float64 divisions run with full warps across steps
    double qs[32][3];
    long long qv[32];
    uint8_t qn[32];
    uint8_t tcell[R * 32];  // the step's vertex task t (one per active cell) -> its cell lane * R + row
};

__device__ __forceinline__ uint32_t lanemask_le(int lane) { return (2u << lane) - 1u; }

// a / n for a vertex's crossing count n (1..12), rounded exactly as the IEEE
// division, from one product and two fused operations (division by a small
// constant after Markstein, IBM J. Res. Develop. 34(1), 1990).  With y = RN(1/n)
// (rcp[n]) and q = RN(a*y), within 1.5 ulps of a/n and |q| <= |a|, the
// remainder a - q*n is a multiple of ulp(q) below 18 ulps: the fma computes it
// exactly.  q + r*y = a/n + r*(y - 1/n) then lies within 36 * 2^-53 ulps of
// a/n, while a/n is at least ulp/24 away from every rounding midpoint: n is
// 2^j times an odd number o, a/2^j is exact, and a - n*M for a midpoint M is a
// nonzero multiple of ulp/2.  So the one rounding of q + r*y gives RN(a/n).
// Zeros, |a| below 2^-959 (where a/2^j could round) and Inf / NaN take the
// division.
__device__ __forceinline__ double div_count(double a, int n, const double *rcp) {
    const unsigned e = (unsigned)((unsigned long long)__double_as_longlong(a) >> 52) & 0x7ffu;
    if (e < 64u || e == 0x7ffu) return __ddiv_rn(a, (double)n);
    const double y = rcp[n], q = __dmul_rn(a, y);
    return __fma_rn(__fma_rn(-q, (double)n, a), y, q);
}
// The same in Float32 (24-bit significands; |a| below 2^-63 takes the division).
__device__ __forceinline__ float div_count(float a, int n, const float *rcp) {
    const unsigned e = (__float_as_uint(a) >> 23) & 0xffu;
    if (e < 64u || e == 0xffu) return __fdiv_rn(a, (float)n);
    const float y = rcp[n], q = __fmul_rn(a, y);
    return __fmaf_rn(__fmaf_rn(-q, (float)n, a), y, q);
}

// First entry of the inclusive prefix a[0..n) above t (a[n-1] > t).
__device__ __forceinline__ int task_cell(const uint16_t *a, int n, int t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int)a[mid] > t) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__device__ __forceinline__ unsigned mc_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) | ((c & 1u) << 4) | ((c >> 1) << 5) |
           ((d >> 1) << 6) | ((d & 1u) << 7);
}
__device__ __forceinline__ unsigned mt_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((b & 1u) << 1) | ((b >> 1) << 2) | ((a >> 1) << 3) | ((c & 1u) << 4) | ((d & 1u) << 5) |
           ((d >> 1) << 6) | ((c >> 1) << 7);
}


// c1*b + c2*a in A, with the corner coordinates c1, c2 in {0, 1} and a, b not
// NaN: the products are b or a (times 1) and zeros carrying the sign of b or a
// (times 0), so the sum is ab = b + a (both 1), or one term plus a zero -- the
// other term, or the IEEE sum of two zeros -- with no arithmetic.
template <class A> __device__ __forceinline__ A corner_mix(int c1, int c2, A b, A a, A ab) {
    if (c1 && c2) return ab;
    const A t1 = c1 ? b : copysign(A(0), b), t2 = c2 ? a : copysign(A(0), a);
    if (!bits_zero(t1)) return t1;  // t2 is a zero
    if (!bits_zero(t2)) return t2;
    return (signbit(t1) && signbit(t2)) ? -A(0) : A(0);
}

// vertPos (src/marching_tetrahedra.jl:42-55) for voxel edge e of cell (x,y,z)
// with the values sv, tv at the edge's corners (MT corner order).
template <class T, class Q, class A, class P>
__device__ __forceinline__ void mt_point(const Plan &p, int e, int x, int y, int z, T sv, T tv, P (&r)[3]) {
    const int i1 = MT_EDGE_CORNERS[e][0], i2 = MT_EDGE_CORNERS[e][1];
    const Q q = quotient<Q>(sv, tv, p);
    const A eps = sizeof(A) == 4 ? (A)p.eps_f : (A)p.eps_d;
    const A hi = sizeof(A) == 4 ? (A)p.hi_f : (A)p.hi_d;
    const A a = jl_min<A>(jl_max<A>((A)q, eps), hi);
    const A b = Ar<A>::sub(A(1), a);
    const bool nan = bits_nan(a);  // then b and every weight are NaN
    const A ab = Ar<A>::add(b, a);
    const int idx[3] = {x, y, z};
    const double *tp[3] = {p.xp, p.yp, p.zp};
    const double *td[3] = {p.dx, p.dy, p.dz};
    const float *tpf[3] = {p.xpf, p.ypf, p.zpf};
    const float *tdf[3] = {p.dxf, p.dyf, p.dzf};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const A w = nan ? a : corner_mix<A>(MT_CORNER_POS[i1][k], MT_CORNER_POS[i2][k], b, a, ab);
        const P base = tab<P>(tp[k], tpf[k], idx[k]);
        const P d = tab<P>(td[k], tdf[k], idx[k]);
        r[k] = Ar<P>::add(base, Ar<P>::mul((P)w, d));
    }
}

template <class T, class Q, class A, class P, int ALG>
__global__ void __launch_bounds__(256, 3) k_emit_halo(const Plan p, int tiles_xh) {
    extern __shared__ __align__(16) unsigned char smem[];
    HaloWarp<T> *ws_all = reinterpret_cast<HaloWarp<T> *>(smem);
    MtTables *tb = reinterpret_cast<MtTables *>(smem + sizeof(HaloWarp<T>) * WARPS);  // MT
    NsnPairs *prs = reinterpret_cast<NsnPairs *>(smem + sizeof(HaloWarp<T>) * WARPS);  // NSN
    __shared__ uint16_t s_cross[256];  // NSN: the crossed MC edges of each MC case
    __shared__ P s_rcp[13];            // NSN: RN(1/n) for the crossing counts n
    if (ALG == MESH_ALG_NSN) {
        if (threadIdx.x <= 12) s_rcp[threadIdx.x] = threadIdx.x ? Ar<P>::div(P(1), (P)threadIdx.x) : P(0);
        for (int c = threadIdx.x; c < 256; c += blockDim.x) {
            // edges 0-7 join corners e, e+1 of their face ring, 8-11 join e-8 and e-4
            unsigned m = 0;
            for (int e = 0; e < 12; e++) {
                const int ea = e < 8 ? (e & 3) + (e & 4) : e - 8;
                const int eb = e < 8 ? ((e + 1) & 3) + (e & 4) : e - 4;
                m |= (((c >> ea) ^ (c >> eb)) & 1u) << e;
            }
            s_cross[c] = (uint16_t)m;
        }
    }
    if (ALG == MESH_ALG_MT) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) {
            for (int k = 0; k < 3 * MT_MAX_FACES; k++) tb->faces[i][k] = MT_CASE_FACES[i][k];
            tb->nfaces[i] = MT_CASE_NFACES[i];
            const int nt = __popc(MT_TOUCHED[i]);
            for (int k = 0, seen = 0; k < nt; k++) {
                const int ee = MT_TOUCH_ORDER[i][k];
                if ((p.own[0] >> ee) & 1u) tb->kth0[i][seen++] = (uint8_t)ee;
            }
            for (int e = 0; e < 19; e++) tb->rank0[i][e] = (uint8_t)__popc(MT_BEFORE[i][e] & p.own[0]);
            // MC case i -> its corner fields a, b, c, d (the inverse of mc_case) -> the MT case
            const unsigned a = (i & 1u) | (((i >> 1) & 1u) << 1), b = ((i >> 3) & 1u) | (((i >> 2) & 1u) << 1);
            const unsigned c = ((i >> 4) & 1u) | (((i >> 5) & 1u) << 1), d = ((i >> 7) & 1u) | (((i >> 6) & 1u) << 1);
            const unsigned mt = mt_case(a, b, c, d);
            tb->mtw[i] = mt | ((unsigned)__popc(MT_TOUCHED[mt] & p.own[0] & 0x7ffffu) << 8) |
                         ((unsigned)MT_CASE_NFACES[mt] << 13);
        }
        if (threadIdx.x < 19) {
            const int e = threadIdx.x;
            const int i1 = MT_EDGE_CORNERS[e][0], i2 = MT_EDGE_CORNERS[e][1];
            int za = 0;
            for (int k = 0; k < 3; k++)
                if (MT_CORNER_POS[i1][k] == 0 && MT_CORNER_POS[i2][k] == 0) za |= 1 << k;
            tb->za[e] = (uint8_t)za;
            for (int s = 0; s < 8; s++) {
                int found = 0xff;
                if ((s & ~za) == 0) {
                    int a[3], b[3];
                    for (int k = 0; k < 3; k++) {
                        a[k] = MT_CORNER_POS[i1][k] + ((s >> k) & 1);
                        b[k] = MT_CORNER_POS[i2][k] + ((s >> k) & 1);
                    }
                    for (int f = 0; f < 19; f++) {
                        const int j1 = MT_EDGE_CORNERS[f][0], j2 = MT_EDGE_CORNERS[f][1];
                        if (MT_CORNER_POS[j1][0] == a[0] && MT_CORNER_POS[j1][1] == a[1] && MT_CORNER_POS[j1][2] == a[2] &&
                            MT_CORNER_POS[j2][0] == b[0] && MT_CORNER_POS[j2][1] == b[1] && MT_CORNER_POS[j2][2] == b[2])
                            found = f;
                    }
                }
                tb->shifted[e][s] = (uint8_t)found;
            }
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    HaloWarp<T> &ws = ws_all[wid];

    // one warp tile: x tile tx, y tile ty, z segment seg
    auto halo_tile = [&](int tx, int ty, int seg) {
    const int x0 = tx * TILE_XH - 1;         // x of lane 0 (the -x neighbour cell)
    const int xs = x0 + lane;                // sample / cell x of this lane
    const int y0 = ty * WY;                  // first real cell row; row 0 of the tile is y0-1
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < 31 && xs >= 0 && xs < p.cx;
    const bool realx = cellx && lane >= 1;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = p.pstride;
    // with an x halo, the totals of its cell column (every output is shifted by them)
    int64_t V0 = 0, F0 = 0;
    if (p.xhalo && p.cx > 1) {
        V0 = p.base[piece(p, 0, 0, 1)];
        F0 = p.base[np + piece(p, 0, 0, 1)];
    }

    bool rowok[R + 1];
    const T *rowp[R + 1];
#pragma unroll
    for (int r = 0; r <= R; r++) {
        const int ys = y0 - 1 + r;
        rowok[r] = xs >= 0 && xs < p.nx && ys >= 0 && ys < p.ny;
        rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)ys : vol;
    }
    bool cellok[R];
    int64_t bv[R], bf[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int yc = y0 - 1 + r;
        cellok[r] = cellx && yc >= 0 && yc < p.cy;
        bv[r] = bf[r] = 0;
        if (cellok[r]) {
            const int64_t i = piece(p, seg, yc, xs);
            bv[r] = p.base[i];
            bf[r] = p.base[np + i];
        }
    }

    // K1 x-tiles and rows that cover this tile, for the activity bytes
    const int cxa = max(tx * TILE_XH - 1, 0), cxb = min(tx * TILE_XH + TILE_XH - 1, p.cx - 1);
    const int kxa = cxa / TILE_X, kxb = cxb / TILE_X;
    const int frow = y0 - 1 + (lane % R);
    const int fkx = lane < R ? kxa : kxb;
    const bool fok = lane < 2 * R && frow >= 0 && frow < p.cy;

    auto chunk_active = [&](int chunk) -> bool {
        uint8_t f = 0;
        if (fok) f = p.flags[((int64_t)chunk * p.tiles_x + fkx) * p.cy + frow];
        return __any_sync(FULL, f != 0);
    };

    // per-cell case and vertex / face count for the cell of row r between planes (lo, hi)
    auto classify = [&](const uint32_t (&ml)[R + 1], const uint32_t (&mh)[R + 1], int r, int zc, unsigned &cs,
                        int &nv, int &nf) {
        const unsigned a = (ml[r] >> lane) & 3u, b = (ml[r + 1] >> lane) & 3u;
        const unsigned c = (mh[r] >> lane) & 3u, d = (mh[r + 1] >> lane) & 3u;
        const unsigned cm = mc_case(a, b, c, d);
        cs = 0;
        nv = nf = 0;
        if (!cellok[r] || cm == 0u || cm == 255u) return;
        const int yc = y0 - 1 + r;
        if (ALG == MESH_ALG_MT) {
            const unsigned w = tb->mtw[cm];
            cs = w & 255u;
            nf = (int)(w >> 13);
            const int bnd = (xs + p.xg0 == 0) | ((yc == 0) << 1) | ((zc == 0) << 2);
            nv = bnd == 0 ? (int)((w >> 8) & 31u) : __popc(__ldg(&MT_TOUCHED[cs]) & p.own[bnd] & 0x7ffffu);
        } else {
            cs = cm;
            nv = 1;
            const unsigned s0 = cm & 1u;
            const bool xk = xs + p.xg0 > 0, yk = yc > 0, zk = zc > 0;
            nf = 2 * (int)(((s0 != ((cm >> 1) & 1u)) && yk && zk) + ((s0 != ((cm >> 3) & 1u)) && zk && xk) +
                           ((s0 != ((cm >> 4) & 1u)) && xk && yk));
        }
    };

    // NSN: queued vertices (a warp-uniform count) and their means, lane i taking entry i
    int qcount = 0;
    auto nsn_means = [&](int m) {
        if (ALG != MESH_ALG_NSN) return;
        NsnPairs &pr = prs[wid];
        if (lane < m) {
            const int n = pr.qn[lane];
            store_vert(p, pr.qv[lane], div_count((P)pr.qs[lane][0], n, s_rcp), div_count((P)pr.qs[lane][1], n, s_rcp),
                       div_count((P)pr.qs[lane][2], n, s_rcp));
        }
        __syncwarp();
    };

    uint32_t mlo[R + 1];
    bool have_lo = false;
    int cur = 0;  // buffer of plane z+1 samples / plane z cells; cur ^ 1 holds plane z / plane z-1

    // samples of plane zz into ws.samp[buf] and their row masks
    auto load_plane = [&](int zz, int buf, uint32_t (&m)[R + 1]) {
#pragma unroll
        for (int r = 0; r <= R; r++) {
            const T v = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zz) : T(0);
            ws.samp[buf][r][lane] = v;
            m[r] = __ballot_sync(FULL, rowok[r] && below(v, p));
        }
    };

    for (int zc0 = zbeg; zc0 < zend; zc0 += ZC) {
        const int zc1 = min(zc0 + ZC, zend);
        const int chunk = seg * p.chunks_per_seg + (zc0 - zbeg) / ZC;
        if (!chunk_active(chunk)) {
            have_lo = false;
            continue;
        }
        if (!have_lo) {
            // the cells of plane zc0-1 are needed as -z neighbours: recompute them
            // when they lie in an active chunk of the previous segment, else they
            // are inactive (their chunk was skipped or does not exist)
            __syncwarp();
            if (zc0 == zbeg && zc0 > 0 && chunk_active(chunk - 1)) {
                uint32_t pm[R + 1];
                load_plane(zc0 - 1, cur, pm);
                load_plane(zc0, cur ^ 1, mlo);
#pragma unroll
                for (int r = 0; r < R; r++) {
                    unsigned cs;
                    int nv, nf;
                    classify(pm, mlo, r, zc0 - 1, cs, nv, nf);
                    ws.cas[cur ^ 1][r][lane] = (uint8_t)cs;
                    ws.base[cur ^ 1][r][lane] = bv[r] - nv;
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; r++) ws.cas[cur ^ 1][r][lane] = 0;
                load_plane(zc0, cur ^ 1, mlo);
            }
            have_lo = true;
        }
        for (int zc = zc0; zc < zc1; zc++) {
            uint32_t mhi[R + 1];
            load_plane(zc + 1, cur, mhi);
            unsigned cs[R];
            int nvs[R], nfs[R];
            bool any = false;
#pragma unroll
            for (int r = 0; r < R; r++) {
                classify(mlo, mhi, r, zc, cs[r], nvs[r], nfs[r]);
                ws.cas[cur][r][lane] = (uint8_t)cs[r];
                ws.base[cur][r][lane] = bv[r];
                ws.fbase[r][lane] = bf[r];
                any |= r >= 1 && realx && cs[r] != 0u;
            }
            if (__any_sync(FULL, any)) {
                // tasks of the real cells (rows 1.., lanes 1..30), in (lane, row) order
                // (each task writes to its cell's own outputs, so any order will do):
                // one scan of the lane's packed vertex | face << 16 totals, then the
                // inclusive prefix over the lane's rows
                int tv[R], tf[R], lt = 0;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    tv[r] = tf[r] = 0;
                    if (r >= 1 && realx && cs[r] != 0u && !(p.xhalo && xs == 0)) {
                        if (bv[r] - V0 + nvs[r] > p.verts_cap || bf[r] - F0 + nfs[r] > p.faces_cap) {
                            atomicOr(p.err, ERR_CAPACITY);
                        } else {
                            tv[r] = nvs[r];
                            tf[r] = nfs[r];
                        }
                    }
                    lt += tv[r] | (tf[r] << 16);
                }
                int inc = lt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int a = __shfl_up_sync(FULL, inc, o);
                    if (lane >= o) inc += a;
                }
                const int tot = __shfl_sync(FULL, inc, 31);
                const int accv = tot & 0xffff, accf = tot >> 16;
                int av = (inc - lt) & 0xffff, af = (inc - lt) >> 16;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    av += tv[r];
                    af += tf[r];
                    ws.pv[lane * R + r] = (uint16_t)av;
                    ws.pf[lane * R + r] = (uint16_t)af;
                    if (ALG == MESH_ALG_NSN && tv[r]) prs[wid].tcell[av - 1] = (uint8_t)(lane * R + r);
                }
                __syncwarp();
                const int lo_b = cur ^ 1, hi_b = cur;
                // vertices
                if (ALG == MESH_ALG_MT) {
                    for (int t = lane; t < accv; t += 32) {
                        const int sc = task_cell(ws.pv, R * 32, t);
                        const int l = sc / R, r = sc - l * R;
                        const int k = t - (sc ? (int)ws.pv[sc - 1] : 0);
                        const unsigned c = ws.cas[cur][r][l];
                        const int xc = x0 + l, yc = y0 - 1 + r;
                        const int64_t vb = ws.base[cur][r][l] - V0;  // this volume's first emitted vertex is 0
                        P q[3];
                        const int bnd = (xc + p.xg0 == 0) | ((yc == 0) << 1) | ((zc == 0) << 2);
                        const uint32_t own = p.own[bnd];
                        // the k-th owned edge in the cell's first-use order
                        int e = 0;
                        if (bnd == 0) {
                            e = tb->kth0[c][k];
                        } else {
                            const int nt = __popc(__ldg(&MT_TOUCHED[c]));
                            for (int i = 0, seen = 0; i < nt; i++) {
                                const int ee = __ldg(&MT_TOUCH_ORDER[c][i]);
                                if (!((own >> ee) & 1u)) continue;
                                if (seen == k) {
                                    e = ee;
                                    break;
                                }
                                seen++;
                            }
                        }
                        // MT corner order: (x,y,z) (x,y+1,z) (x+1,y+1,z) (x+1,y,z), then z+1
                        const int i1 = MT_EDGE_CORNERS[e][0], i2 = MT_EDGE_CORNERS[e][1];
                        auto corner = [&](int kk) -> T {
                            const int dy = (kk & 3) == 1 || (kk & 3) == 2, dx = (kk & 3) >= 2;
                            return ws.samp[kk >= 4 ? hi_b : lo_b][r + dy][l + dx];
                        };
                        mt_point<T, Q, A, P>(p, e, xc, yc, zc, corner(i1), corner(i2), q);
                        store_vert(p, vb + k, q[0], q[1], q[2]);
                    }
                } else {
                    // NSN: the mean of the crossing points on the cell's crossed MC edges,
                    // summed in edge order.  A round of 32 cells is expanded into its
                    // (cell, crossed edge) pairs, so that the Float64 quotient of every
                    // crossing runs with full warps; each lane then adds its cell's
                    // points in edge order from shared memory.
                    NsnPairs &pr = prs[wid];
                    for (int t0 = 0; t0 < accv;) {
                        // lanes 0 .. NSN_VC - 1 take the next cells; the round keeps those whose
                        // pairs fit one sub-round of 32 (at least one cell: a cell has <= 12)
                        const int t = t0 + lane;
                        int r = 0, l = 0, n = 0;
                        unsigned crossed = 0;
                        if (lane < NSN_VC && t < accv) {
                            const int sc = pr.tcell[t];
                            l = sc / R;
                            r = sc - l * R;
                            crossed = s_cross[ws.cas[cur][r][l]];
                            n = __popc(crossed);
                        }
                        int inc = n;
#pragma unroll
                        for (int o = 1; o < NSN_VC; o <<= 1) {
                            const int a = __shfl_up_sync(FULL, inc, o);
                            if (lane >= o) inc += a;
                        }
                        const int mr = max(1, __popc(__ballot_sync(FULL, lane < NSN_VC && t < accv && inc <= 32)));
                        const int S = __shfl_sync(FULL, inc, mr - 1);  // the round's pairs: at most 32
                        if (lane >= mr) n = 0;
                        const int beg = inc - n;  // the cell's first pair
                        const unsigned cw = crossed | ((unsigned)l << 12) | ((unsigned)r << 17);
                        const int64_t vq = n ? ws.base[cur][r][l] - V0 : 0;  // this volume's first vertex is 0
                        // pair j = lane: its cell is the last one that begins at or before j
                        const unsigned starts = __reduce_or_sync(FULL, n ? 1u << beg : 0u);
                        const int own = max(0, __popc(starts & lanemask_le(lane)) - 1);
                        const unsigned cwo = __shfl_sync(FULL, cw, own);
                        const int bego = __shfl_sync(FULL, beg, own);
                        if (lane < S) {
                            const int e = (int)__fns(cwo & 0xfffu, 0, lane - bego + 1);
                            const int r2 = (int)(cwo >> 17), l2 = (int)((cwo >> 12) & 31u);
                            const McEdge g = mc_edge(e);
                            const int ca = mc_corner_off(g.a), cb = mc_corner_off(g.b);
                            const T va = ws.samp[(ca & 4) ? hi_b : lo_b][r2 + ((ca >> 1) & 1)][l2 + (ca & 1)];
                            const T vbv = ws.samp[(cb & 4) ? hi_b : lo_b][r2 + ((cb >> 1) & 1)][l2 + (cb & 1)];
                            P q[3];
                            mc_edge_point<T, Q, P>(p, g, x0 + l2, y0 - 1 + r2, zc, va, vbv, q);
                            pr.pt[lane][0] = (double)q[0];
                            pr.pt[lane][1] = (double)q[1];
                            pr.pt[lane][2] = (double)q[2];
                        }
                        __syncwarp();
                        // the sums: lane 3c + k adds coordinate k of cell c's points in edge order
                        const int c3 = lane / 3, k3 = lane - 3 * c3;
                        const int src3 = c3 < mr ? c3 : 0;
                        const int qa3 = __shfl_sync(FULL, beg, src3), qb3 = __shfl_sync(FULL, inc, src3);
                        P acc = P(0);
                        if (c3 < mr)
                            for (int qq = qa3; qq < qb3; qq++) acc = Ar<P>::add(acc, (P)pr.pt[qq][k3]);
                        __syncwarp();
                        // queue the round's m finished cells (lanes 3c + k hold cell c's sums),
                        // dividing 32 at a time; cells past the queue's room wait for the flush
                        const int m = mr;
                        t0 += mr;
                        const long long vq3 = __shfl_sync(FULL, (long long)vq, c3 < NSN_VC ? c3 : 0);
                        const int n3 = __shfl_sync(FULL, n, c3 < NSN_VC ? c3 : 0);
                        auto push = [&](bool mine, int slot) {
                            if (mine) {
                                pr.qs[slot][k3] = (double)acc;
                                if (k3 == 0) {
                                    pr.qv[slot] = vq3;
                                    pr.qn[slot] = (uint8_t)n3;
                                }
                            }
                        };
                        push(c3 < m && qcount + c3 < 32, qcount + c3);
                        if (qcount + m >= 32) {
                            __syncwarp();
                            nsn_means(32);
                            push(c3 < m && qcount + c3 >= 32, qcount + c3 - 32);
                            qcount -= 32;
                        }
                        qcount += m;
                        __syncwarp();
                    }
                }
                // faces
                for (int t = lane; t < accf; t += 32) {
                    const int sc = task_cell(ws.pf, R * 32, t);
                    const int l = sc / R, r = sc - l * R;
                    const int f = t - (sc ? (int)ws.pf[sc - 1] : 0);
                    const unsigned c = ws.cas[cur][r][l];
                    const int xc = x0 + l, yc = y0 - 1 + r;
                    const int64_t vb = ws.base[cur][r][l] - V0;
                    int64_t *o = p.faces + 3 * (ws.fbase[r][l] - F0 + f);
                    if (ALG == MESH_ALG_MT) {
                        const int bnd = (xc + p.xg0 == 0) | ((yc == 0) << 1) | ((zc == 0) << 2);
                        const uint32_t own = p.own[bnd];
                        int64_t id[3];
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            const int e = tb->faces[c][3 * f + j];
                            const int sh = tb->za[e] & ~bnd;
                            if (sh == 0) {
                                id[j] = vb + (bnd == 0 ? (int)tb->rank0[c][e] : __popc(__ldg(&MT_BEFORE[c][e]) & own)) + 1;
                            } else {
                                // owned by the neighbour one step back along the axes of sh
                                const int e2 = tb->shifted[e][sh];
                                const int l2 = l - (sh & 1), r2 = r - ((sh >> 1) & 1);
                                const int b2 = (sh & 4) ? (cur ^ 1) : cur;
                                const unsigned c2 = ws.cas[b2][r2][l2];
                                const int64_t base2 = ws.base[b2][r2][l2] - V0;
                                const int bnd2 = ((xc - (sh & 1) + p.xg0) == 0) | (((yc - ((sh >> 1) & 1)) == 0) << 1) |
                                                 (((zc - ((sh >> 2) & 1)) == 0) << 2);
                                id[j] = base2 +
                                        (bnd2 == 0 ? (int)tb->rank0[c2][e2] : __popc(__ldg(&MT_BEFORE[c2][e2]) & p.own[bnd2])) + 1;
                            }
                        }
                        o[0] = id[0]; o[1] = id[1]; o[2] = id[2];
                    } else {
                        // NSN: the (f/2)-th crossed base edge of the cell, triangle f%2
                        const unsigned s0 = c & 1u;
                        const bool xk = xc + p.xg0 > 0, yk = yc > 0, zk = zc > 0;
                        const bool ex[3] = {s0 != ((c >> 1) & 1u) && yk && zk, s0 != ((c >> 3) & 1u) && zk && xk,
                                            s0 != ((c >> 4) & 1u) && xk && yk};
                        int kind = 0;
                        for (int j = f >> 1, q2 = 0; q2 < 3; q2++) {
                            if (!ex[q2]) continue;
                            if (j-- == 0) {
                                kind = q2;
                                break;
                            }
                        }
                        const int pv = cur ^ 1;
                        int64_t Aa, B, D;
                        if (kind == 0) {  // +x edge: u = y, w = z
                            Aa = ws.base[pv][r - 1][l]; B = ws.base[pv][r][l]; D = ws.base[cur][r - 1][l];
                        } else if (kind == 1) {  // +y edge: u = z, w = x
                            Aa = ws.base[pv][r][l - 1]; B = ws.base[cur][r][l - 1]; D = ws.base[pv][r][l];
                        } else {  // +z edge: u = x, w = y
                            Aa = ws.base[cur][r - 1][l - 1]; B = ws.base[cur][r - 1][l]; D = ws.base[cur][r][l - 1];
                        }
                        const int64_t C = vb + 1;
                        Aa += 1 - V0; B += 1 - V0; D += 1 - V0;
                        if (s0) {
                            if (f & 1) { o[0] = Aa; o[1] = C; o[2] = D; }
                            else { o[0] = Aa; o[1] = B; o[2] = C; }
                        } else {
                            if (f & 1) { o[0] = Aa; o[1] = D; o[2] = C; }
                            else { o[0] = Aa; o[1] = C; o[2] = B; }
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                bv[r] += nvs[r];
                bf[r] += nfs[r];
            }
#pragma unroll
            for (int r = 0; r <= R; r++) mlo[r] = mhi[r];
            __syncwarp();  // every lane is done with this step's shared state
            cur ^= 1;
        }
    }
    if (qcount > 0) nsn_means(qcount);
    };

    // persistent warps: tiles are taken from a work counter, x tile fastest
    const int nitems = tiles_xh * p.tiles_y * p.nseg;
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        __syncwarp();  // the previous tile is done with the warp's shared state
        halo_tile(item % tiles_xh, (item / tiles_xh) % p.tiles_y, item / (tiles_xh * p.tiles_y));
    }
}

template <class T, int ALG> constexpr size_t halo_smem() {
    return sizeof(HaloWarp<T>) * WARPS + (ALG == MESH_ALG_MT ? sizeof(MtTables) : WARPS * sizeof(NsnPairs));
}

// Resident CTAs of k_emit_halo<T, Q, A, P, ALG> on the current device, with its
// dynamic shared memory allowed (one-time per device and instantiation).
template <class T, class Q, class A, class P, int ALG> int halo_grid() {
    static std::mutex mu;
    static int grid[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!grid[dev]) {
        const void *fn = (const void *)k_emit_halo<T, Q, A, P, ALG>;
        const int smem = (int)halo_smem<T, ALG>();
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * WARPS, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        cudaGetLastError();
        grid[dev] = per_sm * sms;
    }
    return grid[dev];
}

template <class T, class Q, class A, class P, int ALG> cudaError_t go(const Plan &p, cudaStream_t s) {
    const int txh = (p.cx + TILE_XH - 1) / TILE_XH;
    const int64_t nitems = (int64_t)txh * p.tiles_y * p.nseg;
    const int grid = halo_grid<T, Q, A, P, ALG>();
    if (grid < 1) return cudaErrorInvalidDevice;
    cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
    if (e != cudaSuccess || nitems < 1) return e;
    const int ctas = (int)std::min<int64_t>(grid, (nitems + WARPS - 1) / WARPS);
    k_emit_halo<T, Q, A, P, ALG><<<ctas, 32 * WARPS, halo_smem<T, ALG>(), s>>>(p, txh);
    return cudaGetLastError();
}

template <class T> cudaError_t go_t(const Plan &p, int Q64, int A64, int P64, cudaStream_t s) {
    if (p.alg == MESH_ALG_MT) {
        if (Q64) return go<T, double, double, double, MESH_ALG_MT>(p, s);
        if (A64) return go<T, float, double, double, MESH_ALG_MT>(p, s);
        if (P64) return go<T, float, float, double, MESH_ALG_MT>(p, s);
        return go<T, float, float, float, MESH_ALG_MT>(p, s);
    }
    if (Q64) return go<T, double, double, double, MESH_ALG_NSN>(p, s);
    if (P64) return go<T, float, float, double, MESH_ALG_NSN>(p, s);
    return go<T, float, float, float, MESH_ALG_NSN>(p, s);
}

}  // namespace

cudaError_t launch_emit_halo(const Plan &p, int Q64, int A64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return go_t<uint16_t>(p, Q64, A64, P64, s);
    case MESH_DT_F16: return go_t<h16>(p, Q64, A64, P64, s);
    case MESH_DT_I16: return go_t<int16_t>(p, Q64, A64, P64, s);
    case MESH_DT_I8: return go_t<int8_t>(p, Q64, A64, P64, s);
    case MESH_DT_U8: return go_t<uint8_t>(p, Q64, A64, P64, s);
    case MESH_DT_F32: return go_t<float>(p, Q64, A64, P64, s);
    case MESH_DT_I32: return go_t<int32_t>(p, Q64, A64, P64, s);
    case MESH_DT_I64: return go_t<int64_t>(p, Q64, A64, P64, s);
    default:
        if (p.alg == MESH_ALG_MT) return go<double, double, double, double, MESH_ALG_MT>(p, s);
        return go<double, double, double, double, MESH_ALG_NSN>(p, s);
    }
}

}  // namespace mesh
