// K3 (Marching Cubes) -- emit vertices and faces at the scanned offsets.
//
// Replaces process_mc_voxel! (src/marching_cubes.jl:67-92), vertex_interp
// (:100-104) and mc_vert_points (:111-120).  The warp tiling is the classify
// kernel's (31 x-cells by WY y-cells, one z segment); every lane walks its
// column in z with a running (vertex, face) base per row, so each column's
// output is written in the reference's order at base(x, y, seg) from the scan.
// Chunks whose activity bytes are all zero are skipped without touching the
// volume.  Corner values of x+1 come from the neighbouring lane by shuffle.
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

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int U = 4;

template <class T, class Q, class P>
__global__ void __launch_bounds__(256) k_emit_mc(const Plan p) {
    __shared__ uint64_t s_v[256], s_f[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        s_v[i] = MC_CASE_VERTS[i];
        s_f[i] = MC_CASE_FACES[i];
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int ty = blockIdx.y * WARPS + (threadIdx.x >> 5);
    if (ty >= p.tiles_y) return;
    const int tx = blockIdx.x;
    const int seg = blockIdx.z;
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = npieces(p);

    bool rowok[WY + 1];
    const T *rowp[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        rowok[r] = xs < p.nx && y0 + r < p.ny;
        rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)(y0 + r) : vol;
    }
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

    T lo[WY + 1], lon[WY + 1];  // plane z: own sample, x+1 sample (from lane+1)
    uint32_t mlo[WY + 1];
    bool have_lo = false;

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
                lo[r] = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zc0) : T(0);
                lon[r] = __shfl_down_sync(FULL, lo[r], 1);
                mlo[r] = __ballot_sync(FULL, rowok[r] && below(lo[r], p));
            }
            have_lo = true;
        }
        for (int z = zc0; z < zc1; z += U) {
            T v[U][WY + 1];
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= WY; r++)
                    v[u][r] = (rowok[r] && z + 1 + u <= zc1) ? ldv(rowp[r] + sxy * (int64_t)(z + 1 + u)) : T(0);
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int zc = z + u;
                if (zc >= zc1) break;
                T hin[WY + 1];
                uint32_t mhi[WY + 1];
#pragma unroll
                for (int r = 0; r <= WY; r++) {
                    hin[r] = __shfl_down_sync(FULL, v[u][r], 1);
                    mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                }
#pragma unroll
                for (int r = 0; r < WY; r++) {
                    const bool ok = cellx && (y0 + r < p.cy);
                    const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
                    const unsigned c = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
                    const unsigned cm = (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) |
                                        ((c & 1u) << 4) | ((c >> 1) << 5) | ((d >> 1) << 6) | ((d & 1u) << 7);
                    if (ok && cm != 0u && cm != 255u) {
                        const uint64_t tv = s_v[cm], tf = s_f[cm];
                        const int nv = (int)((tv >> 48) & 15u), nf = (int)((tv >> 52) & 7u);
                        const int64_t vb = bv[r], fb = bf[r];
                        if (vb + nv <= p.verts_cap && fb + nf <= p.faces_cap) {
                            const T cv[8] = {lo[r], lon[r], lon[r + 1], lo[r + 1], v[u][r], hin[r], hin[r + 1],
                                             v[u][r + 1]};
                            for (int k = 0; k < nv; k++)
                                {
                                    P q[3];
                                    mc_point<T, Q, P>(p, (int)((tv >> (4 * k)) & 15u), xs, y0 + r, zc, cv, q);
                                    store_vert(p, vb + k, q[0], q[1], q[2]);
                                }
                            for (int k = 0; k < nf; k++) {
                                const unsigned s = (unsigned)(tf >> (12 * k));
                                int64_t *o = p.faces + 3 * (fb + k);
                                o[0] = vb + (s & 15u) + 1;
                                o[1] = vb + ((s >> 4) & 15u) + 1;
                                o[2] = vb + ((s >> 8) & 15u) + 1;
                            }
                        } else {
                            atomicOr(p.err, ERR_CAPACITY);
                        }
                        bv[r] = vb + nv;
                        bf[r] = fb + nf;
                    }
                }
#pragma unroll
                for (int r = 0; r <= WY; r++) {
                    lo[r] = v[u][r];
                    lon[r] = hin[r];
                    mlo[r] = mhi[r];
                }
            }
        }
    }
}

template <class T, class Q, class P> void go(const Plan &p, cudaStream_t s) {
    dim3 grid(p.tiles_x, (p.tiles_y + WARPS - 1) / WARPS, p.nseg);
    k_emit_mc<T, Q, P><<<grid, 32 * WARPS, 0, s>>>(p);
}

template <class T> void go_t(const Plan &p, int Q64, int P64, cudaStream_t s) {
    if (Q64) go<T, double, double>(p, s);
    else if (P64) go<T, float, double>(p, s);
    else go<T, float, float>(p, s);
}

}  // namespace

cudaError_t launch_emit_mc(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: go_t<uint16_t>(p, Q64, P64, s); break;
    case MESH_DT_F32: go_t<float>(p, Q64, P64, s); break;
    default: go<double, double, double>(p, s); break;
    }
    return cudaGetLastError();
}

}  // namespace mesh
