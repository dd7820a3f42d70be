// Device helpers shared by the emit kernels: LinRange table reads, the MC
// edge crossing point (vertex_interp, src/marching_cubes.jl:100-104, on the
// corners of mc_vert_points, :111-120) and vertex stores.
#pragma once
#include "mesh_internal.cuh"

namespace mesh {

template <class P> __device__ __forceinline__ P tab(const double *d, const float *f, int i);
template <> __device__ __forceinline__ double tab<double>(const double *d, const float *, int i) { return __ldg(d + i); }
template <> __device__ __forceinline__ float tab<float>(const double *, const float *f, int i) { return __ldg(f + i); }

// Coordinate on an axis the edge does not move along: p1 + mu*(p1 - p1).
template <class P> __device__ __forceinline__ P still(P c, P mu) {
    if (!bits_zero(c) && bits_finite(mu)) return c;
    return Ar<P>::add(c, Ar<P>::mul(mu, P(0)));
}

template <class P> __device__ __forceinline__ void store_vert(const Plan &p, int64_t i, P x, P y, P z) {
    if (p.out64) {
        double *o = (double *)p.verts + 3 * i;
        o[0] = (double)x; o[1] = (double)y; o[2] = (double)z;
    } else {
        float *o = (float *)p.verts + 3 * i;
        o[0] = (float)x; o[1] = (float)y; o[2] = (float)z;
    }
}

// MC cube edge e -> its start corner a, end corner b (MC corner order: c0
// (x,y,z) c1 (x+1,y,z) c2 (x+1,y+1,z) c3 (x,y+1,z), c4..c7 the same at z+1),
// moving axis, direction (1: the start corner is the +1 node of the moving
// axis) and the fixed offsets of the start corner's other axes.
struct McEdge {
    int a, b, ax, neg, ox, oy, oz;
};
__device__ __forceinline__ McEdge mc_edge(int e) {
    switch (e) {
    case 0: return {0, 1, 0, 0, 0, 0, 0};
    case 1: return {1, 2, 1, 0, 1, 0, 0};
    case 2: return {2, 3, 0, 1, 0, 1, 0};
    case 3: return {3, 0, 1, 1, 0, 0, 0};
    case 4: return {4, 5, 0, 0, 0, 0, 1};
    case 5: return {5, 6, 1, 0, 1, 0, 1};
    case 6: return {6, 7, 0, 1, 0, 1, 1};
    case 7: return {7, 4, 1, 1, 0, 0, 1};
    case 8: return {0, 4, 2, 0, 0, 0, 0};
    case 9: return {1, 5, 2, 0, 1, 0, 0};
    case 10: return {2, 6, 2, 0, 1, 1, 0};
    default: return {3, 7, 2, 0, 0, 1, 0};
    }
}
// corner k of the MC corner order as (dx, dy, dz) bits 0, 1, 2
__device__ __forceinline__ int mc_corner_off(int k) { return (((k + 1) >> 1) & 1) | (((k >> 1) & 1) << 1) | ((k >> 2) << 2); }

// Crossing point p1 + mu*(p2 - p1) on MC cube edge e of cell (x, y, z), with
// the values va, vb at the edge's start and end corners.
template <class T, class Q, class P>
__device__ __forceinline__ void mc_edge_point(const Plan &p, const McEdge &g, int x, int y, int z, T va, T vb,
                                              P (&r)[3]) {
    const Q mu = quotient<Q>(va, vb, p);
    const P m = (P)mu;
    // start point p1 = corner a; for a negative edge it sits at the +1 node of the moving axis
    const int ix = x + g.ox + (g.ax == 0 && g.neg), iy = y + g.oy + (g.ax == 1 && g.neg),
              iz = z + g.oz + (g.ax == 2 && g.neg);
    const int idx[3] = {ix, iy, iz};
    const double *tp[3] = {p.xp, p.yp, p.zp};
    const double *td[3] = {p.dx, p.dy, p.dz};
    const float *tpf[3] = {p.xpf, p.ypf, p.zpf};
    const float *tdf[3] = {p.dxf, p.dyf, p.dzf};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const P c1 = tab<P>(tp[k], tpf[k], idx[k]);
        if (k == g.ax) {
            // p2 - p1 = +-(p[i+1] - p[i]) exactly
            P d = tab<P>(td[k], tdf[k], g.neg ? idx[k] - 1 : idx[k]);
            if (g.neg) d = -d;
            r[k] = Ar<P>::add(c1, Ar<P>::mul(m, d));
        } else {
            r[k] = still<P>(c1, m);
        }
    }
}

// The same from the cell's eight corner values (MC corner order).
template <class T, class Q, class P>
__device__ __forceinline__ void mc_point(const Plan &p, int e, int x, int y, int z, const T (&c)[8], P (&r)[3]) {
    const McEdge g = mc_edge(e);
    T va = c[0], vb = c[0];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (k == g.a) va = c[k];
        if (k == g.b) vb = c[k];
    }
    mc_edge_point<T, Q, P>(p, g, x, y, z, va, vb, r);
}

}  // namespace mesh
