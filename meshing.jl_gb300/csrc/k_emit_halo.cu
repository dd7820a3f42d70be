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
// samples.  Cases and bases of the current and previous z plane live in
// per-warp shared memory, so neighbour lookups are plain shared loads.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_point.cuh"

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int R = WY + 1;  // cell rows per tile including the -y neighbour row

struct MtTables {
    uint8_t faces[256][3 * MT_MAX_FACES];
    uint8_t order[256][MT_MAX_TOUCH];
    uint32_t before[256][19];
    uint32_t touched[256];
    uint8_t nfaces[256];
    uint8_t za[19];          // axes on which both corners of the edge are 0
    uint8_t shifted[19][8];  // the same lattice edge seen from the cell shifted by -s
};

struct WarpState {
    uint32_t cas[2][R][32];
    long long base[2][R][32];
};

__device__ __forceinline__ unsigned mc_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) | ((c & 1u) << 4) | ((c >> 1) << 5) |
           ((d >> 1) << 6) | ((d & 1u) << 7);
}
__device__ __forceinline__ unsigned mt_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((b & 1u) << 1) | ((b >> 1) << 2) | ((a >> 1) << 3) | ((c & 1u) << 4) | ((d & 1u) << 5) |
           ((d >> 1) << 6) | ((c >> 1) << 7);
}


// vertPos (src/marching_tetrahedra.jl:42-55) for voxel edge e of cell (x,y,z);
// corner values in MT corner order.
template <class T, class Q, class A, class P>
__device__ __forceinline__ void mt_point(const Plan &p, int e, int x, int y, int z, const T (&c)[8], P (&r)[3]) {
    const int i1 = MT_EDGE_CORNERS[e][0], i2 = MT_EDGE_CORNERS[e][1];
    T s = c[0], t = c[0];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (k == i1) s = c[k];
        if (k == i2) t = c[k];
    }
    const Q q = quotient<Q>(s, t, p);
    const A eps = sizeof(A) == 4 ? (A)p.eps_f : (A)p.eps_d;
    const A hi = sizeof(A) == 4 ? (A)p.hi_f : (A)p.hi_d;
    const A a = jl_min<A>(jl_max<A>((A)q, eps), hi);
    const A b = Ar<A>::sub(A(1), a);
    const int idx[3] = {x, y, z};
    const double *tp[3] = {p.xp, p.yp, p.zp};
    const double *td[3] = {p.dx, p.dy, p.dz};
    const float *tpf[3] = {p.xpf, p.ypf, p.zpf};
    const float *tdf[3] = {p.dxf, p.dyf, p.dzf};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const A w = Ar<A>::add(Ar<A>::mul((A)MT_CORNER_POS[i1][k], b), Ar<A>::mul((A)MT_CORNER_POS[i2][k], a));
        const P base = tab<P>(tp[k], tpf[k], idx[k]);
        const P d = tab<P>(td[k], tdf[k], idx[k]);
        r[k] = Ar<P>::add(base, Ar<P>::mul((P)w, d));
    }
}

template <class T, class Q, class A, class P, int ALG>
__global__ void __launch_bounds__(256) k_emit_halo(const Plan p, int tiles_xh) {
    extern __shared__ __align__(16) unsigned char smem[];
    WarpState *ws_all = reinterpret_cast<WarpState *>(smem);
    MtTables *tb = reinterpret_cast<MtTables *>(smem + sizeof(WarpState) * WARPS);
    if (ALG == MESH_ALG_MT) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) {
            for (int k = 0; k < 3 * MT_MAX_FACES; k++) tb->faces[i][k] = MT_CASE_FACES[i][k];
            for (int k = 0; k < MT_MAX_TOUCH; k++) tb->order[i][k] = MT_TOUCH_ORDER[i][k];
            for (int k = 0; k < 19; k++) tb->before[i][k] = MT_BEFORE[i][k];
            tb->touched[i] = MT_TOUCHED[i];
            tb->nfaces[i] = MT_CASE_NFACES[i];
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
    const int ty = blockIdx.y * WARPS + wid;
    if (ty >= p.tiles_y) return;
    WarpState &ws = ws_all[wid];
    const int tx = blockIdx.x;
    const int seg = blockIdx.z;
    const int xs = tx * TILE_XH - 1 + lane;  // sample / cell x of this lane
    const int y0 = ty * WY;                  // first real cell row; row 0 of the tile is y0-1
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < 31 && xs >= 0 && xs < p.cx;
    const bool realx = cellx && lane >= 1;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = p.pstride;

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

    // per-cell case and vertex count for the cell of row r between planes (lo, hi)
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
            cs = mt_case(a, b, c, d);
            const int bnd = (xs == 0) | ((yc == 0) << 1) | ((zc == 0) << 2);
            nv = __popc(tb->touched[cs] & p.own[bnd] & 0x7ffffu);
            nf = tb->nfaces[cs];
        } else {
            cs = cm;
            nv = 1;
            const unsigned s0 = cm & 1u;
            const bool xk = xs > 0, yk = yc > 0, zk = zc > 0;
            nf = 2 * (int)(((s0 != ((cm >> 1) & 1u)) && yk && zk) + ((s0 != ((cm >> 3) & 1u)) && zk && xk) +
                           ((s0 != ((cm >> 4) & 1u)) && xk && yk));
        }
    };

    T lo[R + 1], lon[R + 1];
    uint32_t mlo[R + 1];
    bool have_lo = false;
    int cur = 0;  // buffer of the current z plane in ws; cur^1 holds z-1

    auto load_plane = [&](int zz, T (&v)[R + 1], T (&vn)[R + 1], uint32_t (&m)[R + 1]) {
#pragma unroll
        for (int r = 0; r <= R; r++) {
            v[r] = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zz) : T(0);
            vn[r] = shfl_down1(v[r]);
            m[r] = __ballot_sync(FULL, rowok[r] && below(v[r], p));
        }
    };

    auto clear_prev = [&]() {
#pragma unroll
        for (int r = 0; r < R; r++) ws.cas[cur ^ 1][r][lane] = 0;
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
            clear_prev();
            if (zc0 == zbeg && zc0 > 0 && chunk_active(chunk - 1)) {
                T pl[R + 1], pln[R + 1];
                uint32_t pm[R + 1];
                load_plane(zc0 - 1, pl, pln, pm);
                load_plane(zc0, lo, lon, mlo);
#pragma unroll
                for (int r = 0; r < R; r++) {
                    unsigned cs;
                    int nv, nf;
                    classify(pm, mlo, r, zc0 - 1, cs, nv, nf);
                    ws.cas[cur ^ 1][r][lane] = cs;
                    ws.base[cur ^ 1][r][lane] = bv[r] - nv;
                }
            } else {
                load_plane(zc0, lo, lon, mlo);
            }
            have_lo = true;
        }
        for (int zc = zc0; zc < zc1; zc++) {
            T hi[R + 1], hin[R + 1];
            uint32_t mhi[R + 1];
            load_plane(zc + 1, hi, hin, mhi);
            unsigned cs[R];
            int nvs[R], nfs[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                classify(mlo, mhi, r, zc, cs[r], nvs[r], nfs[r]);
                ws.cas[cur][r][lane] = cs[r];
                ws.base[cur][r][lane] = bv[r];
            }
            __syncwarp();
#pragma unroll
            for (int r = 1; r < R; r++) {
                if (!realx || !cellok[r] || cs[r] == 0u) continue;
                const int yc = y0 - 1 + r;
                const int64_t vb = bv[r], fb = bf[r];
                if (vb + nvs[r] > p.verts_cap || fb + nfs[r] > p.faces_cap) {
                    atomicOr(p.err, ERR_CAPACITY);
                    continue;
                }
                if (ALG == MESH_ALG_MT) {
                    // MT corner order: (x,y,z) (x,y+1,z) (x+1,y+1,z) (x+1,y,z), then z+1
                    const T cv[8] = {lo[r], lo[r + 1], lon[r + 1], lon[r], hi[r], hi[r + 1], hin[r + 1], hin[r]};
                    const unsigned c = cs[r];
                    const int bnd = (xs == 0) | ((yc == 0) << 1) | ((zc == 0) << 2);
                    const uint32_t own = p.own[bnd];
                    const int nt = __popc(tb->touched[c]);
                    int rank = 0;
                    for (int k = 0; k < nt; k++) {
                        const int e = tb->order[c][k];
                        if (!((own >> e) & 1u)) continue;
                        P q[3];
                        mt_point<T, Q, A, P>(p, e, xs, yc, zc, cv, q);
                        store_vert(p, vb + rank, q[0], q[1], q[2]);
                        rank++;
                    }
                    const int nf = tb->nfaces[c];
                    for (int f = 0; f < nf; f++) {
                        int64_t id[3];
                        for (int j = 0; j < 3; j++) {
                            const int e = tb->faces[c][3 * f + j];
                            const int s = tb->za[e] & ~bnd;
                            if (s == 0) {
                                id[j] = vb + __popc(tb->before[c][e] & own) + 1;
                            } else {
                                const int e2 = tb->shifted[e][s];
                                const int l2 = lane - (s & 1), r2 = r - ((s >> 1) & 1);
                                const int b2 = (s & 4) ? (cur ^ 1) : cur;
                                const unsigned c2 = ws.cas[b2][r2][l2];
                                const int64_t base2 = ws.base[b2][r2][l2];
                                const int bnd2 = ((xs - (s & 1)) == 0) | (((yc - ((s >> 1) & 1)) == 0) << 1) |
                                                 (((zc - ((s >> 2) & 1)) == 0) << 2);
                                id[j] = base2 + __popc(tb->before[c2][e2] & p.own[bnd2]) + 1;
                            }
                        }
                        int64_t *o = p.faces + 3 * (fb + f);
                        o[0] = id[0]; o[1] = id[1]; o[2] = id[2];
                    }
                } else {
                    // NSN: vertex = mean of the crossing points on the crossed MC edges
                    const T cv[8] = {lo[r], lon[r], lon[r + 1], lo[r + 1], hi[r], hin[r], hin[r + 1], hi[r + 1]};
                    const unsigned c = cs[r];
                    P sum[3] = {P(0), P(0), P(0)};
                    int n = 0;
                    for (int e = 0; e < 12; e++) {
                        const int ea = e < 8 ? (e & 3) + (e & 4) : e - 8;
                        const int eb = e < 8 ? ((e + 1) & 3) + (e & 4) : e - 4;
                        if (((c >> ea) & 1u) == ((c >> eb) & 1u)) continue;
                        P q[3];
                        mc_point<T, Q, P>(p, e, xs, yc, zc, cv, q);
#pragma unroll
                        for (int k = 0; k < 3; k++) sum[k] = Ar<P>::add(sum[k], q[k]);
                        n++;
                    }
                    store_vert(p, vb, Ar<P>::div(sum[0], (P)n), Ar<P>::div(sum[1], (P)n), Ar<P>::div(sum[2], (P)n));
                    const int64_t C = vb + 1;
                    const bool xk = xs > 0, yk = yc > 0, zk = zc > 0;
                    const unsigned s0 = c & 1u;
                    const int pv = cur ^ 1;
                    int f = 0;
                    // +x edge: u = y, w = z
                    if (s0 != ((c >> 1) & 1u) && yk && zk) {
                        const int64_t Aa = ws.base[pv][r - 1][lane] + 1, B = ws.base[pv][r][lane] + 1,
                                      D = ws.base[cur][r - 1][lane] + 1;
                        int64_t *o = p.faces + 3 * (fb + f);
                        if (s0) { o[0] = Aa; o[1] = B; o[2] = C; o[3] = Aa; o[4] = C; o[5] = D; }
                        else { o[0] = Aa; o[1] = C; o[2] = B; o[3] = Aa; o[4] = D; o[5] = C; }
                        f += 2;
                    }
                    // +y edge: u = z, w = x
                    if (s0 != ((c >> 3) & 1u) && zk && xk) {
                        const int64_t Aa = ws.base[pv][r][lane - 1] + 1, B = ws.base[cur][r][lane - 1] + 1,
                                      D = ws.base[pv][r][lane] + 1;
                        int64_t *o = p.faces + 3 * (fb + f);
                        if (s0) { o[0] = Aa; o[1] = B; o[2] = C; o[3] = Aa; o[4] = C; o[5] = D; }
                        else { o[0] = Aa; o[1] = C; o[2] = B; o[3] = Aa; o[4] = D; o[5] = C; }
                        f += 2;
                    }
                    // +z edge: u = x, w = y
                    if (s0 != ((c >> 4) & 1u) && xk && yk) {
                        const int64_t Aa = ws.base[cur][r - 1][lane - 1] + 1, B = ws.base[cur][r - 1][lane] + 1,
                                      D = ws.base[cur][r][lane - 1] + 1;
                        int64_t *o = p.faces + 3 * (fb + f);
                        if (s0) { o[0] = Aa; o[1] = B; o[2] = C; o[3] = Aa; o[4] = C; o[5] = D; }
                        else { o[0] = Aa; o[1] = C; o[2] = B; o[3] = Aa; o[4] = D; o[5] = C; }
                        f += 2;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                bv[r] += nvs[r];
                bf[r] += nfs[r];
            }
#pragma unroll
            for (int r = 0; r <= R; r++) {
                lo[r] = hi[r];
                lon[r] = hin[r];
                mlo[r] = mhi[r];
            }
            __syncwarp();
            cur ^= 1;
        }
    }
}

template <class T, class Q, class A, class P, int ALG> cudaError_t go(const Plan &p, cudaStream_t s) {
    const int txh = (p.cx + TILE_XH - 1) / TILE_XH;
    dim3 grid(txh, (p.tiles_y + WARPS - 1) / WARPS, p.nseg);
    const size_t sm = sizeof(WarpState) * WARPS + (ALG == MESH_ALG_MT ? sizeof(MtTables) : 0);
    cudaError_t e = cudaFuncSetAttribute(k_emit_halo<T, Q, A, P, ALG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sm);
    if (e != cudaSuccess) return e;
    k_emit_halo<T, Q, A, P, ALG><<<grid, 32 * WARPS, sm, s>>>(p, txh);
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
    case MESH_DT_F32: return go_t<float>(p, Q64, A64, P64, s);
    default:
        if (p.alg == MESH_ALG_MT) return go<double, double, double, double, MESH_ALG_MT>(p, s);
        return go<double, double, double, double, MESH_ALG_NSN>(p, s);
    }
}

}  // namespace mesh
