// K1 -- classify: per-cell cube case and per-piece vertex/face counts.
//
// Replaces the classification half of the reference's cell loops
// (src/marching_cubes.jl:40-56, src/marching_tetrahedra.jl:144-157,
// src/common.jl:10-29).  A warp owns a tile of 31 x-cells by WY y-cells and
// walks one z segment; lane l loads sample x0+l of WY+1 sample rows per z
// plane (coalesced rows along x, Julia layout), and one ballot per row turns
// the strict `v < iso` tests of a whole row into a bit mask, from which every
// lane assembles its 8-corner case without further memory traffic.
//
// Outputs: cnt[v|f|a][seg][y][x] (u32) -- vertices first-created, faces emitted
// and active cells of column x,y inside z segment seg -- and one activity byte per
// (z chunk, x tile, y row) that lets the emit kernels skip empty chunks.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_case.cuh"
#include "mesh_tma.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int U = 4;     // z planes loaded ahead
constexpr int CWY = WY;  // cell rows per warp tile of the load walk (the TMA walk keeps WY)

// MC corner order (src/marching_cubes.jl:42-49) from the 2-bit (x, x+1) fields
// of rows y/y+1 in planes z/z+1.
__device__ __forceinline__ unsigned mc_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) | ((c & 1u) << 4) | ((c >> 1) << 5) |
           ((d >> 1) << 6) | ((d & 1u) << 7);
}
// MT corner order (src/marching_tetrahedra.jl:146-153).
__device__ __forceinline__ unsigned mt_case(unsigned a, unsigned b, unsigned c, unsigned d) {
    return (a & 1u) | ((b & 1u) << 1) | ((b >> 1) << 2) | ((a >> 1) << 3) | ((c & 1u) << 4) | ((d & 1u) << 5) |
           ((d >> 1) << 6) | ((c >> 1) << 7);
}

template <int ALG> __device__ __forceinline__ void load_tables(uint32_t *s_tab) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        if (ALG == MESH_ALG_MC) {
            uint64_t t = MC_CASE_VERTS[i];
            s_tab[i] = (uint32_t)((t >> 48) & 15u) | ((uint32_t)((t >> 52) & 7u) << 8);
        } else if (ALG == MESH_ALG_MT) {
            s_tab[i] = MT_TOUCHED[i] | ((uint32_t)MT_CASE_NFACES[i] << 24);
        }
    }
}

// Per-lane running counts of the NR cells (rows) a lane owns, and per-row
// activity of the current z chunk (warp-uniform).
template <int NR> struct Counts {
    uint32_t v[NR], f[NR], a[NR], act[NR];
};

// One z step: the cells between the sample planes whose row masks are mlo
// (plane z) and mhi (plane z+1).
template <int ALG, int NR>
__device__ __forceinline__ void step(const Plan &p, const uint32_t *s_tab, const uint32_t (&mlo)[NR + 1],
                                     const uint32_t (&mhi)[NR + 1], uint32_t xval, uint32_t cellm, int lane, int xs,
                                     int y0, int zc, Counts<NR> &c) {
    uint32_t all1 = xval, any1 = 0;
#pragma unroll
    for (int r = 0; r <= NR; r++) {
        all1 &= mlo[r] & mhi[r];
        any1 |= mlo[r] | mhi[r];
    }
    // warp-uniform early out: every corner of every cell in this step on one side
    if (all1 == xval || any1 == 0) return;
#pragma unroll
    for (int r = 0; r < NR; r++) {
        // bit l: cell l has corners on both sides (bits l, l+1 of the four masks)
        const uint32_t and4 = mlo[r] & mlo[r + 1] & mhi[r] & mhi[r + 1];
        const uint32_t or4 = mlo[r] | mlo[r + 1] | mhi[r] | mhi[r + 1];
        const uint32_t actm = (or4 | (or4 >> 1)) & ~(and4 & (and4 >> 1)) & cellm;
        if (actm == 0u || y0 + r >= p.cy) continue;  // warp-uniform
        c.act[r] = 1;
        if (!((actm >> lane) & 1u)) continue;
        c.a[r] += 1;
        const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
        const unsigned cc = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
        const unsigned cm = mc_case(a, b, cc, d);
        if (ALG == MESH_ALG_MC) {
            const uint32_t t = s_tab[cm];
            c.v[r] += t & 15u;
            c.f[r] += t >> 8;
        } else if (ALG == MESH_ALG_MT) {
            const uint32_t t = s_tab[mt_case(a, b, cc, d)];
            const int bnd = (xs + p.xg0 == 0) | ((y0 + r == 0) << 1) | ((zc == 0) << 2);
            c.v[r] += __popc(t & p.own[bnd] & 0x7ffffu);
            c.f[r] += t >> 24;
        } else {  // NSN: one vertex per active cell, a quad per crossed base edge
            c.v[r] += 1;
            const unsigned s0 = cm & 1u;
            const bool yk = y0 + r > 0, zk = zc > 0, xk = xs + p.xg0 > 0;
            unsigned q = 0;
            q += (s0 != ((cm >> 1) & 1u)) && yk && zk;  // +x edge
            q += (s0 != ((cm >> 3) & 1u)) && zk && xk;  // +y edge
            q += (s0 != ((cm >> 4) & 1u)) && xk && yk;  // +z edge
            c.f[r] += 2 * q;
        }
    }
}

// At the end of an activity chunk: publish one byte per tile row.
template <int NR>
__device__ __forceinline__ void chunk_end(const Plan &p, int lane, int tx, int y0, int seg, int zbeg, int zc,
                                          int zend, Counts<NR> &c) {
    if (((zc + 1 - zbeg) % ZC) == 0 || zc + 1 == zend) {
        const int chunk = seg * p.chunks_per_seg + (zc - zbeg) / ZC;
        uint8_t mine = 0;
#pragma unroll
        for (int r = 0; r < NR; r++) {
            if (lane == r) mine = c.act[r] != 0;  // act[] is warp-uniform
            c.act[r] = 0;
        }
        if (lane < NR && y0 + lane < p.cy) p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine;
    }
}

template <int NR>
__device__ __forceinline__ void store_counts(const Plan &p, bool cellx, int xs, int y0, int seg, const Counts<NR> &c) {
    if (!cellx) return;
    const int64_t np = p.pstride;
#pragma unroll
    for (int r = 0; r < NR; r++) {
        if (y0 + r < p.cy) {
            const int64_t i = piece(p, seg, y0 + r, xs);
            p.cnt[i] = c.v[r];
            p.cnt[np + i] = c.f[r];
            p.cnt[2 * np + i] = c.a[r];
        }
    }
}

// The walk below for a warp tile inside the volume (all 32 lanes' samples and
// all WY + 1 rows exist) whose z segment spans fewer than 2^32 samples: no
// per-lane or per-row guards, 32-bit sample offsets from the segment's first
// plane, and each plane's row masks reduced once (AND / OR over the rows) for
// the one-side test of the two steps that use it.  Counts equal the walk
// below; lane 31 (no cell) is left out of the activity bytes and the counts.
template <class T>
__device__ __forceinline__ void classify_tile_mc_inner(const Plan &p, const uint32_t *s_tab, int lane, int tx,
                                                       int ty, int seg) {
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const uint32_t sxy = (uint32_t)(p.nx * p.ny), nx = (uint32_t)p.nx;
    const T *base = (const T *)p.vol + (int64_t)sxy * zbeg + xs + p.nx * (int64_t)y0;
    constexpr uint32_t CELLM = 0x7fffffffu;  // lanes 0..30 own cells

    uint32_t cv[WY], cf[WY], ca[WY];
#pragma unroll
    for (int r = 0; r < WY; r++) cv[r] = cf[r] = ca[r] = 0;
    uint32_t mlo[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) mlo[r] = __ballot_sync(FULL, below(ldv(base + r * nx), p));
    uint32_t alo = mlo[0] & mlo[1] & mlo[2] & mlo[3] & mlo[4], olo = mlo[0] | mlo[1] | mlo[2] | mlo[3] | mlo[4];
    static_assert(WY == 4, "the plane reductions below name rows 0..4");
    uint32_t zoff = 0;  // plane zc0 relative to zbeg

    for (int zc0 = zbeg; zc0 < zend; zc0 += ZC) {
        const int n = min(ZC, zend - zc0);
        uint32_t pk[WY];
#pragma unroll
        for (int r = 0; r < WY; r++) pk[r] = 0;
        for (int u0 = 0; u0 < n; u0 += U) {
            T v[U][WY + 1];
            if (u0 + U <= n) {
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++) v[u][r] = ldv(base + (zoff + (u + 1) * sxy + r * nx));
            } else {
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++)
                        v[u][r] = u0 + u < n ? ldv(base + (zoff + (u + 1) * sxy + r * nx)) : T(0);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (u0 + u >= n) break;  // warp-uniform
                uint32_t mhi[WY + 1];
#pragma unroll
                for (int r = 0; r <= WY; r++) mhi[r] = __ballot_sync(FULL, below(v[u][r], p));
                const uint32_t ahi = mhi[0] & mhi[1] & mhi[2] & mhi[3] & mhi[4];
                const uint32_t ohi = mhi[0] | mhi[1] | mhi[2] | mhi[3] | mhi[4];
                if ((alo & ahi) != FULL && (olo | ohi) != 0u) {
                    uint32_t nb[WY + 1];
#pragma unroll
                    for (int r = 0; r <= WY; r++) nb[r] = row_field(mlo[r], mhi[r], lane);
#pragma unroll
                    for (int r = 0; r < WY; r++) pk[r] += s_tab[nb[r] | (nb[r + 1] << 4)];
                }
#pragma unroll
                for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
                alo = ahi;
                olo = ohi;
            }
            zoff += U * sxy;
        }
        zoff += (uint32_t)(n - (n + U - 1) / U * U) * sxy;  // back to plane zc0 + n after a short chunk
        const int chunk = seg * p.chunks_per_seg + (zc0 - zbeg) / ZC;
        uint32_t mine = 0;  // lane r: the active columns of row y0 + r
#pragma unroll
        for (int r = 0; r < WY; r++) {
            const uint32_t am = __ballot_sync(FULL, pk[r] != 0u) & CELLM;
            if (lane == r) mine = am;
            cv[r] += pk[r] & ((1u << PK_F) - 1u);
            cf[r] += (pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u);
            ca[r] += pk[r] >> PK_A;
        }
        if (lane < WY) {
            p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine != 0u;
            if (p.cmask) p.cmask[((int64_t)tx * p.cy + y0 + lane) * p.nchunks + chunk] = mine;
        }
    }
    if (lane >= TILE_X) return;
    const int64_t np = p.pstride;
#pragma unroll
    for (int r = 0; r < WY; r++) {
        const int64_t i = piece(p, seg, y0 + r, xs);
        p.cnt[i] = cv[r];
        p.cnt[np + i] = cf[r];
        p.cnt[2 * np + i] = ca[r];
    }
}

// Marching Cubes walk of warp tile (tx, ty) through z segment seg.  Loads and
// ballots as in classify_tile; a step whose corners are not all on one side
// costs, per cell row, one lookup of the case's packed word (mesh_case.cuh)
// and one add (no branch per row or lane).  The words of an activity chunk
// (ZC planes: at most 12 * ZC vertices, 5 * ZC faces, ZC cells per field) are
// unpacked at the chunk's end, where a non-zero word marks the row active.
template <class T>
__device__ __forceinline__ void classify_tile_mc(const Plan &p, const uint32_t *s_tab, int lane, int tx, int ty,
                                                 int seg) {
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;

    bool rowok[WY + 1];
    const T *rowp[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        rowok[r] = xs < p.nx && y0 + r < p.ny;
        rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)(y0 + r) : vol;
    }
    uint32_t rmask[WY];  // the lane's cell of row r exists
    uint32_t cv[WY], cf[WY], ca[WY];
#pragma unroll
    for (int r = 0; r < WY; r++) {
        rmask[r] = (cellx && y0 + r < p.cy) ? 0xffffffffu : 0u;
        cv[r] = cf[r] = ca[r] = 0;
    }
    const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
    uint32_t mlo[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        T v = rowok[r] ? ldv(rowp[r] + sxy * zbeg) : T(0);
        mlo[r] = __ballot_sync(FULL, rowok[r] && below(v, p));
    }

    for (int zc0 = zbeg; zc0 < zend; zc0 += ZC) {
        const int zc1 = min(zc0 + ZC, zend);
        uint32_t pk[WY];
#pragma unroll
        for (int r = 0; r < WY; r++) pk[r] = 0;
        for (int z = zc0; z < zc1; z += U) {
            T v[U][WY + 1];
            const int64_t off = sxy * (int64_t)(z + 1);
            if (z + U <= zc1) {
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++) v[u][r] = rowok[r] ? ldv(rowp[r] + off + sxy * u) : T(0);
            } else {
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++)
                        v[u][r] = (rowok[r] && z + 1 + u <= zc1) ? ldv(rowp[r] + off + sxy * u) : T(0);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (z + u >= zc1) break;  // warp-uniform
                uint32_t mhi[WY + 1];
                uint32_t all1 = xval, any1 = 0;
#pragma unroll
                for (int r = 0; r <= WY; r++) {
                    mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                    all1 &= mlo[r] & mhi[r];
                    any1 |= mlo[r] | mhi[r];
                }
                // warp-uniform early out: every corner of every cell of this step on one side
                if (all1 != xval && any1 != 0u) {
                    uint32_t nb[WY + 1];
#pragma unroll
                    for (int r = 0; r <= WY; r++) nb[r] = row_field(mlo[r], mhi[r], lane);
#pragma unroll
                    for (int r = 0; r < WY; r++) pk[r] += s_tab[nb[r] | (nb[r + 1] << 4)] & rmask[r];
                }
#pragma unroll
                for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
            }
        }
        const int chunk = seg * p.chunks_per_seg + (zc0 - zbeg) / ZC;
        uint32_t mine = 0;  // lane r: the active columns of row y0 + r (pk holds existing cells only)
#pragma unroll
        for (int r = 0; r < WY; r++) {
            const uint32_t am = __ballot_sync(FULL, pk[r] != 0u);
            if (lane == r) mine = am;
            cv[r] += pk[r] & ((1u << PK_F) - 1u);
            cf[r] += (pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u);
            ca[r] += pk[r] >> PK_A;
        }
        if (lane < WY && y0 + lane < p.cy) {
            p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine != 0u;
            if (p.cmask) p.cmask[((int64_t)tx * p.cy + y0 + lane) * p.nchunks + chunk] = mine;
        }
    }
    if (!cellx) return;
    const int64_t np = p.pstride;
#pragma unroll
    for (int r = 0; r < WY; r++) {
        if (y0 + r < p.cy) {
            const int64_t i = piece(p, seg, y0 + r, xs);
            p.cnt[i] = cv[r];
            p.cnt[np + i] = cf[r];
            p.cnt[2 * np + i] = ca[r];
        }
    }
}

// Walk of warp tile (tx, ty) through z segment seg with one coalesced global
// load per lane, row and plane (any layout).
template <class T, int ALG>
__device__ __forceinline__ void classify_tile(const Plan &p, const uint32_t *s_tab, int lane, int tx, int ty, int seg) {
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * CWY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;

    bool rowok[CWY + 1];
    const T *rowp[CWY + 1];
#pragma unroll
    for (int r = 0; r <= CWY; r++) {
        rowok[r] = xs < p.nx && y0 + r < p.ny;
        rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)(y0 + r) : vol;
    }
    Counts<CWY> c;
#pragma unroll
    for (int r = 0; r < CWY; r++) c.v[r] = c.f[r] = c.a[r] = c.act[r] = 0;
    // lanes whose sample exists (x < nx): only their bits take part in the uniform test
    const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
    const uint32_t cellm = __ballot_sync(FULL, cellx);
    uint32_t mlo[CWY + 1];
#pragma unroll
    for (int r = 0; r <= CWY; r++) {
        T v = rowok[r] ? ldv(rowp[r] + sxy * zbeg) : T(0);
        mlo[r] = __ballot_sync(FULL, rowok[r] && below(v, p));
    }

    for (int z = zbeg; z < zend; z += U) {
        T v[U][CWY + 1];
        const int64_t off = sxy * (int64_t)(z + 1);
        if (z + U <= zend) {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= CWY; r++) v[u][r] = rowok[r] ? ldv(rowp[r] + off + sxy * u) : T(0);
        } else {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= CWY; r++)
                    v[u][r] = (rowok[r] && z + 1 + u <= zend) ? ldv(rowp[r] + off + sxy * u) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int zc = z + u;
            if (zc >= zend) break;  // warp-uniform
            uint32_t mhi[CWY + 1];
#pragma unroll
            for (int r = 0; r <= CWY; r++) mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
            step<ALG, CWY>(p, s_tab, mlo, mhi, xval, cellm, lane, xs, y0, zc, c);
#pragma unroll
            for (int r = 0; r <= CWY; r++) mlo[r] = mhi[r];
            chunk_end(p, lane, tx, y0, seg, zbeg, zc, zend, c);
        }
    }
    store_counts(p, cellx, xs, y0, seg, c);
}

template <class T, int ALG>
__global__ void __launch_bounds__(256, 3) k_classify(const Plan p) {
    __shared__ uint32_t s_tab[256];
    if (ALG == MESH_ALG_MC)
        load_tables_mc_packed(s_tab);
    else
        load_tables<ALG>(s_tab);
    __syncthreads();
    const int ty = blockIdx.y * WARPS + (threadIdx.x >> 5);
    if (ty * CWY >= p.cy) return;  // warp-uniform
    // a launch over segments seg0 .. seg1 - 1 (seg1 0: all) spans the whole grid and
    // its other blocks return at once: the segment stays the block index, which the
    // walks re-read instead of keeping it live
    if ((int)blockIdx.z < p.seg0 || (p.seg1 > 0 && (int)blockIdx.z >= p.seg1)) return;
    if (ALG == MESH_ALG_MC) {
        if (tile_inner(p, blockIdx.x, ty, blockIdx.z))
            classify_tile_mc_inner<T>(p, s_tab, threadIdx.x & 31, blockIdx.x, ty, blockIdx.z);
        else
            classify_tile_mc<T>(p, s_tab, threadIdx.x & 31, blockIdx.x, ty, blockIdx.z);
    } else
        classify_tile<T, ALG>(p, s_tab, threadIdx.x & 31, blockIdx.x, ty, blockIdx.z);
}

// Batch (Marching Cubes): persistent warps take work items -- a warp tile of
// one volume's z segment, volumes in order, y tiles fastest -- from a counter.
template <class T>
__global__ void __launch_bounds__(256) k_classify_batch(const Plan p) {
    __shared__ uint32_t s_tab[256];
    load_tables_mc_packed(s_tab);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if ((int64_t)item >= p.nitems) break;
        const BatchVol b = p.bvols[p.item_vol[item]];
        const Plan pv = vol_view(p, b);
        const int64_t local = (int64_t)item - b.item0;
        const int ty = (int)(local % b.tiles_y);
        const int tx = (int)((local / b.tiles_y) % b.tiles_x);
        const int seg = (int)(local / ((int64_t)b.tiles_y * b.tiles_x));
        classify_tile_mc<T>(pv, s_tab, lane, tx, ty, seg);
    }
}

// Walk over TMA-staged bricks.  The CTA's 31 x 32 cells of a z segment are
// streamed as boxes of TMA_BZ planes x 33 rows x BX samples through a ring of
// TMA_STAGES shared-memory stages.  Warp specialisation: warp WARPS (the
// producer) issues cp.async.bulk.tensor into a free stage and arms its `full`
// mbarrier with the byte count; the WARPS consumer warps wait on `full`,
// classify their 4 cell rows, and release the stage by arriving on its
// `empty` mbarrier.  The box starts on the 16-byte boundary at or below the
// tile's first sample; lanes index from the remainder.  Needs rows whose byte
// stride is a multiple of 16.  All waits are bounded; on expiry the CTA
// reports ERR_TMA_TIMEOUT, waits (bounded) for its copies in flight and exits.
template <class T, int ALG>
__global__ void __launch_bounds__(32 * (WARPS + 1)) k_classify_tma(const Plan p, const __grid_constant__ CUtensorMap tmap) {
    constexpr int BX = TmaBox<T>::BX, AL = TmaBox<T>::ALIGN;
    constexpr int PLANE = TMA_BY * BX;
    constexpr unsigned BYTES = TMA_BZ * PLANE * sizeof(T);         // one box
    constexpr int STAGE = (int)(tma_stage_bytes<T>() / sizeof(T));  // stage stride, 128-byte aligned
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *buf = reinterpret_cast<T *>(smem_raw);  // [TMA_STAGES][STAGE]
    __shared__ uint32_t s_tab[256];
    __shared__ __align__(8) uint64_t full[TMA_STAGES], empty[TMA_STAGES];
    __shared__ int s_fail;
    if (ALG == MESH_ALG_MC)
        load_tables_mc_packed(s_tab);
    else
        load_tables<ALG>(s_tab);

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int tx = blockIdx.x, seg = blockIdx.z;
    const int x0 = tx * TILE_X, xa = x0 & ~(AL - 1), xoff = x0 - xa;
    const int yc0 = blockIdx.y * WARPS * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const int nst = (zend - zbeg + 1 + TMA_BZ - 1) / TMA_BZ;  // planes zbeg..zend

    if (tid == 0) {
        for (int k = 0; k < TMA_STAGES; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], WARPS);
        }
        s_fail = 0;
        mbar_fence_init();
    }
    __syncthreads();

    if (w == WARPS) {  // producer
        int issued = 0;
        if (lane == 0) {
            for (int s = 0; s < nst; s++) {
                const int slot = s % TMA_STAGES;
                if (s >= TMA_STAGES && !mbar_wait(&empty[slot], (unsigned)(s / TMA_STAGES - 1) & 1u)) {
                    atomicOr(&s_fail, 1);
                    break;
                }
                if (*(volatile int *)&s_fail) break;
                fence_proxy_async();
                mbar_expect_tx(&full[slot], BYTES);
                tma_load_3d(buf + slot * STAGE, &tmap, xa, yc0, zbeg + s * TMA_BZ, &full[slot]);
                issued = s + 1;
            }
            // on failure, let the copies in flight land before the CTA exits
            if (*(volatile int *)&s_fail)
                for (int s = max(0, issued - TMA_STAGES); s < issued; s++)
                    mbar_wait(&full[s % TMA_STAGES], (unsigned)(s / TMA_STAGES) & 1u);
        }
        __syncwarp();
    } else {  // consumers
        const int ty = blockIdx.y * WARPS + w;
        const int y0 = ty * WY;
        const bool warp_on = ty < p.tiles_y;
        const int xs = x0 + lane;
        const bool cellx = lane < TILE_X && xs < p.cx;
        bool rowok[WY + 1];
#pragma unroll
        for (int r = 0; r <= WY; r++) rowok[r] = xs < p.nx && y0 + r < p.ny;
        Counts<WY> c;
        uint32_t pk[WY], rmask[WY];  // Marching Cubes: packed words of the current chunk
#pragma unroll
        for (int r = 0; r < WY; r++) {
            c.v[r] = c.f[r] = c.a[r] = c.act[r] = 0;
            pk[r] = 0;
            rmask[r] = (cellx && y0 + r < p.cy) ? 0xffffffffu : 0u;
        }
        const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
        const uint32_t cellm = __ballot_sync(FULL, cellx);
        uint32_t mlo[WY + 1];
#pragma unroll
        for (int r = 0; r <= WY; r++) mlo[r] = 0;
        bool ok = true;
        for (int s = 0; s < nst; s++) {
            const int slot = s % TMA_STAGES;
            ok = mbar_wait(&full[slot], (unsigned)(s / TMA_STAGES) & 1u);
            ok = __all_sync(FULL, ok) && !*(volatile int *)&s_fail;
            if (!ok) {
                if (lane == 0) atomicOr(&s_fail, 1);
                break;
            }
            const T *st = buf + slot * STAGE;
            if (warp_on) {
#pragma unroll
                for (int k = 0; k < TMA_BZ; k++) {
                    const int plane = zbeg + s * TMA_BZ + k;
                    if (plane > zend) break;  // warp-uniform
                    uint32_t m[WY + 1];
#pragma unroll
                    for (int r = 0; r <= WY; r++)
                        m[r] = __ballot_sync(FULL,
                                             rowok[r] && below(st[k * PLANE + (w * WY + r) * BX + xoff + lane], p));
                    if (plane > zbeg) {
                        const int zc = plane - 1;
                        if (ALG == MESH_ALG_MC) {  // packed words, as classify_tile_mc
                            uint32_t all1 = xval, any1 = 0;
#pragma unroll
                            for (int r = 0; r <= WY; r++) {
                                all1 &= mlo[r] & m[r];
                                any1 |= mlo[r] | m[r];
                            }
                            if (all1 != xval && any1 != 0u) {
                                uint32_t nb[WY + 1];
#pragma unroll
                                for (int r = 0; r <= WY; r++) nb[r] = row_field(mlo[r], m[r], lane);
#pragma unroll
                                for (int r = 0; r < WY; r++) pk[r] += s_tab[nb[r] | (nb[r + 1] << 4)] & rmask[r];
                            }
                            if (((zc + 1 - zbeg) % ZC) == 0 || zc + 1 == zend) {
                                const int chunk = seg * p.chunks_per_seg + (zc - zbeg) / ZC;
                                uint8_t mine = 0;
#pragma unroll
                                for (int r = 0; r < WY; r++) {
                                    const bool act = __any_sync(FULL, pk[r] != 0u);
                                    if (lane == r) mine = act;
                                    c.v[r] += pk[r] & ((1u << PK_F) - 1u);
                                    c.f[r] += (pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u);
                                    c.a[r] += pk[r] >> PK_A;
                                    pk[r] = 0;
                                }
                                if (lane < WY && y0 + lane < p.cy)
                                    p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine;
                            }
                        } else {
                            step<ALG, WY>(p, s_tab, mlo, m, xval, cellm, lane, xs, y0, zc, c);
                            chunk_end(p, lane, tx, y0, seg, zbeg, zc, zend, c);
                        }
                    }
#pragma unroll
                    for (int r = 0; r <= WY; r++) mlo[r] = m[r];
                }
            }
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&empty[slot])) : "memory");
        }
        if (ok && warp_on) store_counts(p, cellx, xs, y0, seg, c);
    }
    __syncthreads();
    if (tid == 0 && s_fail) atomicOr(p.err, ERR_TMA_TIMEOUT);
}

// Marching Cubes walk over TMA-staged bricks (the default for volumes a tensor
// map can describe).  The CTA's tile column -- 31 x-cells by WARPS * WY cell rows
// of one z segment -- is streamed through the same TMA_STAGES-deep ring of
// TMA_BZ-plane boxes as k_classify_tma, filled by one producer lane, so the
// consumers never wait on a global load.  The consumer is the load walk's
// guard-free form (classify_tile_mc_inner) reading shared memory: per stage
// five row addresses, per plane one ballot per sample row and the plane's
// AND / OR reduction (reused by the two steps that share the plane), per step
// one packed-word lookup per cell row; an activity chunk (ZC = 2 stages)
// closes at the first plane of every even stage.  Tiles at the volume's edge
// take the same loop with per-lane and per-row guards.  Outputs as the load
// walk: piece counts, activity bytes and the active-column masks (cmask).
template <class T, bool INNER>
__device__ __forceinline__ void tma_mc_consume(const Plan &p, const uint32_t *s_tab, const T *buf, uint64_t *full,
                                               uint64_t *empty, int *s_fail, int lane, int w, int tx, int seg,
                                               int xoff) {
    constexpr int BX = TmaBox<T>::BX;
    constexpr int PLANE = TMA_BY * BX;
    constexpr int STAGE = (int)(tma_stage_bytes<T>() / sizeof(T));
    const int ty = blockIdx.y * WARPS + w;
    const int y0 = ty * WY;
    const bool warp_on = ty < p.tiles_y;
    const int xs = tx * TILE_X + lane;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const int nst = (zend - zbeg + 1 + TMA_BZ - 1) / TMA_BZ;  // stages of planes zbeg..zend
    const bool cellx = lane < TILE_X && xs < p.cx;
    bool rowok[WY + 1];
    uint32_t rmask[WY];
#pragma unroll
    for (int r = 0; r <= WY; r++) rowok[r] = INNER || (xs < p.nx && y0 + r < p.ny);
#pragma unroll
    for (int r = 0; r < WY; r++) rmask[r] = (INNER ? lane < TILE_X : (cellx && y0 + r < p.cy)) ? 0xffffffffu : 0u;
    const uint32_t xval = INNER ? FULL : __ballot_sync(FULL, xs < p.nx);
    int off[WY + 1];  // the lane's sample of row r in a stage's first plane
#pragma unroll
    for (int r = 0; r <= WY; r++) off[r] = (w * WY + r) * BX + xoff + lane;
    uint32_t cv[WY], cf[WY], ca[WY], pk[WY];
#pragma unroll
    for (int r = 0; r < WY; r++) cv[r] = cf[r] = ca[r] = pk[r] = 0;
    // per sample row of a plane: the lane's 2-bit field (x, x+1), extracted once per
    // plane and shared by the two steps that use the plane
    uint32_t mlo[WY + 1], alo = 0, olo = 0;

    auto masks = [&](const T *st, int k, uint32_t (&m)[WY + 1], uint32_t &a, uint32_t &o) {
        a = xval;
        o = 0;
#pragma unroll
        for (int r = 0; r <= WY; r++) {
            const uint32_t b = __ballot_sync(FULL, rowok[r] && below(st[k * PLANE + off[r]], p));
            a &= b;
            o |= b;
            m[r] = (b >> lane) & 3u;
        }
    };
    auto step = [&](const uint32_t (&mhi)[WY + 1], uint32_t ahi, uint32_t ohi) {
        if ((alo & ahi) != xval && (olo | ohi) != 0u) {
            uint32_t nb[WY + 1];
#pragma unroll
            for (int r = 0; r <= WY; r++) nb[r] = mlo[r] | (mhi[r] << 2);
#pragma unroll
            for (int r = 0; r < WY; r++) pk[r] += s_tab[nb[r] | (nb[r + 1] << 4)] & rmask[r];
        }
#pragma unroll
        for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
        alo = ahi;
        olo = ohi;
    };
    auto flush = [&](int ci) {  // close activity chunk ci of the segment
        const int chunk = seg * p.chunks_per_seg + ci;
        uint32_t mine = 0;  // lane r: the active columns of row y0 + r
#pragma unroll
        for (int r = 0; r < WY; r++) {
            const uint32_t am = __ballot_sync(FULL, pk[r] != 0u);
            if (lane == r) mine = am;
            cv[r] += pk[r] & ((1u << PK_F) - 1u);
            cf[r] += (pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u);
            ca[r] += pk[r] >> PK_A;
            pk[r] = 0;
        }
        if (lane < WY && (INNER || y0 + lane < p.cy)) {
            p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine != 0u;
            if (p.cmask) p.cmask[((int64_t)tx * p.cy + y0 + lane) * p.nchunks + chunk] = mine;
        }
    };
    auto release = [&](int slot) {
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&empty[slot])) : "memory");
    };

    bool ok = true;
    for (int s = 0; s < nst; s++) {
        const int slot = s % TMA_STAGES;
        ok = mbar_wait(&full[slot], (unsigned)(s / TMA_STAGES) & 1u);
        ok = __all_sync(FULL, ok) && !*(volatile int *)s_fail;
        if (!ok) {
            if (lane == 0) atomicOr(s_fail, 1);
            break;
        }
        const T *st = buf + slot * STAGE;
        if (warp_on) {
            const int p0 = zbeg + s * TMA_BZ;  // the stage's first plane
            if (s == 0) {
                masks(st, 0, mlo, alo, olo);
#pragma unroll
                for (int k = 1; k < TMA_BZ; k++) {
                    if (p0 + k > zend) break;  // warp-uniform
                    uint32_t mhi[WY + 1], ahi, ohi;
                    masks(st, k, mhi, ahi, ohi);
                    step(mhi, ahi, ohi);
                }
            } else {
#pragma unroll
                for (int k = 0; k < TMA_BZ; k++) {
                    if (p0 + k > zend) break;  // warp-uniform
                    uint32_t mhi[WY + 1], ahi, ohi;
                    masks(st, k, mhi, ahi, ohi);
                    step(mhi, ahi, ohi);
                    // the step just taken ends an activity chunk (ZC == 2 * TMA_BZ)
                    if (k == 0 && !(s & 1)) flush(s / 2 - 1);
                }
            }
        }
        release(slot);
    }
    if (!ok || !warp_on) return;
    if ((zend - zbeg) % ZC) flush((zend - zbeg - 1) / ZC);  // the segment's last, shorter chunk
    if (!cellx) return;
    const int64_t np = p.pstride;
#pragma unroll
    for (int r = 0; r < WY; r++) {
        if (INNER || y0 + r < p.cy) {
            const int64_t i = piece(p, seg, y0 + r, xs);
            p.cnt[i] = cv[r];
            p.cnt[np + i] = cf[r];
            p.cnt[2 * np + i] = ca[r];
        }
    }
}
static_assert(ZC == 2 * TMA_BZ, "an activity chunk is two TMA stages");

template <class T>
__global__ void __launch_bounds__(32 * (WARPS + 1)) k_classify_tma_mc(const Plan p, const __grid_constant__ CUtensorMap tmap) {
    constexpr int AL = TmaBox<T>::ALIGN;
    constexpr unsigned BYTES = TMA_BZ * TMA_BY * TmaBox<T>::BX * sizeof(T);  // one box
    constexpr int STAGE = (int)(tma_stage_bytes<T>() / sizeof(T));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *buf = reinterpret_cast<T *>(smem_raw);  // [TMA_STAGES][STAGE]
    __shared__ uint32_t s_tab[256];
    __shared__ __align__(8) uint64_t full[TMA_STAGES], empty[TMA_STAGES];
    __shared__ int s_fail;
    load_tables_mc_packed(s_tab);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int tx = blockIdx.x, seg = blockIdx.z;
    const int x0 = tx * TILE_X, xa = x0 & ~(AL - 1);
    const int yc0 = blockIdx.y * WARPS * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const int nst = (zend - zbeg + 1 + TMA_BZ - 1) / TMA_BZ;
    if (tid == 0) {
        for (int k = 0; k < TMA_STAGES; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], WARPS);
        }
        s_fail = 0;
        mbar_fence_init();
    }
    __syncthreads();
    if (w == WARPS) {  // producer: one lane issues every stage's box
        if (lane == 0) {
            int issued = 0;
            for (int s = 0; s < nst; s++) {
                const int slot = s % TMA_STAGES;
                if (s >= TMA_STAGES && !mbar_wait(&empty[slot], (unsigned)(s / TMA_STAGES - 1) & 1u)) {
                    atomicOr(&s_fail, 1);
                    break;
                }
                if (*(volatile int *)&s_fail) break;
                fence_proxy_async();
                mbar_expect_tx(&full[slot], BYTES);
                tma_load_3d(buf + slot * STAGE, &tmap, xa, yc0, zbeg + s * TMA_BZ, &full[slot]);
                issued = s + 1;
            }
            // on failure, let the copies in flight land before the CTA exits
            if (*(volatile int *)&s_fail)
                for (int s = max(0, issued - TMA_STAGES); s < issued; s++)
                    mbar_wait(&full[s % TMA_STAGES], (unsigned)(s / TMA_STAGES) & 1u);
        }
        __syncwarp();
    } else {
        // inside the volume: all 32 lanes' samples and the WY + 1 sample rows exist
        const int ty = blockIdx.y * WARPS + w;
        const bool inner = x0 + 32 <= p.nx && ty * WY + WY <= p.cy;
        if (inner)
            tma_mc_consume<T, true>(p, s_tab, buf, full, empty, &s_fail, lane, w, tx, seg, x0 - xa);
        else
            tma_mc_consume<T, false>(p, s_tab, buf, full, empty, &s_fail, lane, w, tx, seg, x0 - xa);
    }
    __syncthreads();
    if (tid == 0 && s_fail) atomicOr(p.err, ERR_TMA_TIMEOUT);
}

template <class T> cudaError_t launch_t(const Plan &p, cudaStream_t s) {
    const int ty = (p.cy + CWY - 1) / CWY;  // warp tiles of the load walk along y
    dim3 grid(p.tiles_x, (ty + WARPS - 1) / WARPS, p.nseg);
    switch (p.alg) {
    case MESH_ALG_MC: k_classify<T, MESH_ALG_MC><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_ALG_MT: k_classify<T, MESH_ALG_MT><<<grid, 32 * WARPS, 0, s>>>(p); break;
    default: k_classify<T, MESH_ALG_NSN><<<grid, 32 * WARPS, 0, s>>>(p); break;
    }
    return cudaGetLastError();
}

template <class T> cudaError_t launch_tma_t(const Plan &p, const CUtensorMap &map, cudaStream_t s) {
    dim3 grid(p.tiles_x, (p.tiles_y + WARPS - 1) / WARPS, p.nseg);
    const size_t sm = (size_t)TMA_STAGES * tma_stage_bytes<T>();
    cudaError_t e = cudaSuccess;
    switch (p.alg) {
    case MESH_ALG_MC:
        e = cudaFuncSetAttribute(k_classify_tma_mc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess) k_classify_tma_mc<T><<<grid, 32 * (WARPS + 1), sm, s>>>(p, map);
        break;
    case MESH_ALG_MT:
        e = cudaFuncSetAttribute(k_classify_tma<T, MESH_ALG_MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess) k_classify_tma<T, MESH_ALG_MT><<<grid, 32 * (WARPS + 1), sm, s>>>(p, map);
        break;
    default:
        e = cudaFuncSetAttribute(k_classify_tma<T, MESH_ALG_NSN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e == cudaSuccess) k_classify_tma<T, MESH_ALG_NSN><<<grid, 32 * (WARPS + 1), sm, s>>>(p, map);
        break;
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace

cudaError_t launch_classify_tma(const Plan &p, const CUtensorMap &map, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return launch_tma_t<uint16_t>(p, map, s);
    case MESH_DT_F32: return launch_tma_t<float>(p, map, s);
    case MESH_DT_F64: return launch_tma_t<double>(p, map, s);
    default: return cudaErrorInvalidValue;  // integer volumes take the load walk
    }
}

int persistent_grid(const void *fn, int threads, int ctas_per_sm) {
    int dev = 0, sms = 0, fit = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, threads, 0) != cudaSuccess || fit < 1) {
        cudaGetLastError();
        fit = 1;
    }
    return sms * (ctas_per_sm > 0 ? std::min(ctas_per_sm, fit) : fit);
}

cudaError_t launch_classify_batch(const Plan &p, int ctas, cudaStream_t s) {
    const void *fn = nullptr;
    switch (p.T) {
    case MESH_DT_U16: fn = (const void *)k_classify_batch<uint16_t>; break;
    case MESH_DT_F16: fn = (const void *)k_classify_batch<h16>; break;
    case MESH_DT_I16: fn = (const void *)k_classify_batch<int16_t>; break;
    case MESH_DT_I8: fn = (const void *)k_classify_batch<int8_t>; break;
    case MESH_DT_U8: fn = (const void *)k_classify_batch<uint8_t>; break;
    case MESH_DT_F32: fn = (const void *)k_classify_batch<float>; break;
    case MESH_DT_I32: fn = (const void *)k_classify_batch<int32_t>; break;
    case MESH_DT_I64: fn = (const void *)k_classify_batch<int64_t>; break;
    default: fn = (const void *)k_classify_batch<double>; break;
    }
    const int grid = (int)std::min<int64_t>(persistent_grid(fn, 32 * WARPS, ctas), (p.nitems + WARPS - 1) / WARPS);
    if (grid < 1) return cudaSuccess;
    switch (p.T) {
    case MESH_DT_U16: k_classify_batch<uint16_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_F16: k_classify_batch<h16><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_I16: k_classify_batch<int16_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_I8: k_classify_batch<int8_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_U8: k_classify_batch<uint8_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_F32: k_classify_batch<float><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_I32: k_classify_batch<int32_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_DT_I64: k_classify_batch<int64_t><<<grid, 32 * WARPS, 0, s>>>(p); break;
    default: k_classify_batch<double><<<grid, 32 * WARPS, 0, s>>>(p); break;
    }
    return cudaGetLastError();
}

// Segments seg0 .. seg0 + nsegs - 1 (nsegs 0: every segment).
cudaError_t launch_classify(const Plan &p0, cudaStream_t s, int seg0, int nsegs) {
    Plan p = p0;
    if (nsegs <= 0) nsegs = p.nseg - seg0;
    if (seg0 < 0 || nsegs <= 0 || seg0 + nsegs > p.nseg) return cudaErrorInvalidValue;
    p.seg0 = seg0;
    p.seg1 = seg0 + nsegs;
    switch (p.T) {
    case MESH_DT_U16: return launch_t<uint16_t>(p, s);
    case MESH_DT_F16: return launch_t<h16>(p, s);
    case MESH_DT_I16: return launch_t<int16_t>(p, s);
    case MESH_DT_I8: return launch_t<int8_t>(p, s);
    case MESH_DT_U8: return launch_t<uint8_t>(p, s);
    case MESH_DT_F32: return launch_t<float>(p, s);
    case MESH_DT_I32: return launch_t<int32_t>(p, s);
    case MESH_DT_I64: return launch_t<int64_t>(p, s);
    default: return launch_t<double>(p, s);
    }
}

}  // namespace mesh
