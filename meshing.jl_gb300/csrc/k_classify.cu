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

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int U = 4;  // z planes loaded ahead

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

template <class T, int ALG>
__global__ void __launch_bounds__(256) k_classify(const Plan p) {
    __shared__ uint32_t s_tab[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        if (ALG == MESH_ALG_MC) {
            uint64_t t = MC_CASE_VERTS[i];
            s_tab[i] = (uint32_t)((t >> 48) & 15u) | ((uint32_t)((t >> 52) & 7u) << 8);
        } else if (ALG == MESH_ALG_MT) {
            s_tab[i] = MT_TOUCHED[i] | ((uint32_t)MT_CASE_NFACES[i] << 24);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int ty = blockIdx.y * WARPS + (threadIdx.x >> 5);
    if (ty >= p.tiles_y) return;  // warp-uniform
    const int tx = blockIdx.x;
    const int seg = blockIdx.z;
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

    uint32_t cntv[WY], cntf[WY], cnta[WY], act[WY];
#pragma unroll
    for (int r = 0; r < WY; r++) cntv[r] = cntf[r] = cnta[r] = act[r] = 0;

    // lanes whose sample exists (x < nx): only their bits take part in the uniform test
    const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
    const uint32_t cellm = __ballot_sync(FULL, cellx);
    uint32_t mlo[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        T v = rowok[r] ? ldv(rowp[r] + sxy * zbeg) : T(0);
        mlo[r] = __ballot_sync(FULL, rowok[r] && below(v, p));
    }

    for (int z = zbeg; z < zend; z += U) {
        T v[U][WY + 1];
        const int64_t off = sxy * (int64_t)(z + 1);
        if (z + U <= zend) {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= WY; r++) v[u][r] = rowok[r] ? ldv(rowp[r] + off + sxy * u) : T(0);
        } else {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= WY; r++)
                    v[u][r] = (rowok[r] && z + 1 + u <= zend) ? ldv(rowp[r] + off + sxy * u) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int zc = z + u;
            if (zc >= zend) break;  // warp-uniform
            uint32_t mhi[WY + 1];
            uint32_t all1 = xval, any1 = 0;
#pragma unroll
            for (int r = 0; r <= WY; r++) {
                mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                all1 &= mlo[r] & mhi[r];
                any1 |= mlo[r] | mhi[r];
            }
            // warp-uniform early out: every corner of every cell in this step on one side
            if (all1 != xval && any1 != 0) {
#pragma unroll
                for (int r = 0; r < WY; r++) {
                    // bit l: cell l has corners on both sides (bits l, l+1 of the four masks)
                    const uint32_t and4 = mlo[r] & mlo[r + 1] & mhi[r] & mhi[r + 1];
                    const uint32_t or4 = mlo[r] | mlo[r + 1] | mhi[r] | mhi[r + 1];
                    const uint32_t actm = (or4 | (or4 >> 1)) & ~(and4 & (and4 >> 1)) & cellm;
                    if (actm == 0u || y0 + r >= p.cy) continue;  // warp-uniform
                    act[r] = 1;
                    if (!((actm >> lane) & 1u)) continue;
                    cnta[r] += 1;
                    const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
                    const unsigned c = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
                    const unsigned cm = mc_case(a, b, c, d);
                    if (ALG == MESH_ALG_MC) {
                        const uint32_t t = s_tab[cm];
                        cntv[r] += t & 15u;
                        cntf[r] += t >> 8;
                    } else if (ALG == MESH_ALG_MT) {
                        const uint32_t t = s_tab[mt_case(a, b, c, d)];
                        const int bnd = (xs == 0) | ((y0 + r == 0) << 1) | ((zc == 0) << 2);
                        cntv[r] += __popc(t & p.own[bnd] & 0x7ffffu);
                        cntf[r] += t >> 24;
                    } else {  // NSN: one vertex per active cell, a quad per crossed base edge
                        cntv[r] += 1;
                        const unsigned s0 = cm & 1u;
                        const bool yk = y0 + r > 0, zk = zc > 0, xk = xs > 0;
                        unsigned q = 0;
                        q += (s0 != ((cm >> 1) & 1u)) && yk && zk;  // +x edge
                        q += (s0 != ((cm >> 3) & 1u)) && zk && xk;  // +y edge
                        q += (s0 != ((cm >> 4) & 1u)) && xk && yk;  // +z edge
                        cntf[r] += 2 * q;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
            // end of an activity chunk: publish one byte per tile row
            if (((zc + 1 - zbeg) % ZC) == 0 || zc + 1 == zend) {
                const int chunk = seg * p.chunks_per_seg + (zc - zbeg) / ZC;
                uint8_t mine = 0;
#pragma unroll
                for (int r = 0; r < WY; r++) {
                    if (lane == r) mine = act[r] != 0;  // act[] is warp-uniform
                    act[r] = 0;
                }
                if (lane < WY && y0 + lane < p.cy)
                    p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane] = mine;
            }
        }
    }

    if (cellx) {
        const int64_t np = npieces(p);
#pragma unroll
        for (int r = 0; r < WY; r++) {
            if (y0 + r < p.cy) {
                const int64_t i = piece(p, seg, y0 + r, xs);
                p.cnt[i] = cntv[r];
                p.cnt[np + i] = cntf[r];
                p.cnt[2 * np + i] = cnta[r];
            }
        }
    }
}

template <class T> cudaError_t launch_t(const Plan &p, cudaStream_t s) {
    dim3 grid(p.tiles_x, (p.tiles_y + WARPS - 1) / WARPS, p.nseg);
    switch (p.alg) {
    case MESH_ALG_MC: k_classify<T, MESH_ALG_MC><<<grid, 32 * WARPS, 0, s>>>(p); break;
    case MESH_ALG_MT: k_classify<T, MESH_ALG_MT><<<grid, 32 * WARPS, 0, s>>>(p); break;
    default: k_classify<T, MESH_ALG_NSN><<<grid, 32 * WARPS, 0, s>>>(p); break;
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_classify(const Plan &p, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return launch_t<uint16_t>(p, s);
    case MESH_DT_F32: return launch_t<float>(p, s);
    default: return launch_t<double>(p, s);
    }
}

}  // namespace mesh
