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
    if (c != P(0) && isfinite(mu)) return c;
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

// Crossing point p1 + mu*(p2 - p1) on MC cube edge e of cell (x, y, z).  Corner values follow the
// MC corner order: c0 (x,y,z) c1 (x+1,y,z) c2 (x+1,y+1,z) c3 (x,y+1,z), c4..c7
// the same at z+1.
template <class T, class Q, class P>
__device__ __forceinline__ void mc_point(const Plan &p, int e, int x, int y, int z, const T (&c)[8], P (&r)[3]) {
    // edge -> (corner a, corner b, moving axis, direction, fixed offsets)
    int a, b, ax, neg, ox, oy, oz;
    switch (e) {
    case 0: a = 0; b = 1; ax = 0; neg = 0; ox = 0; oy = 0; oz = 0; break;
    case 1: a = 1; b = 2; ax = 1; neg = 0; ox = 1; oy = 0; oz = 0; break;
    case 2: a = 2; b = 3; ax = 0; neg = 1; ox = 0; oy = 1; oz = 0; break;
    case 3: a = 3; b = 0; ax = 1; neg = 1; ox = 0; oy = 0; oz = 0; break;
    case 4: a = 4; b = 5; ax = 0; neg = 0; ox = 0; oy = 0; oz = 1; break;
    case 5: a = 5; b = 6; ax = 1; neg = 0; ox = 1; oy = 0; oz = 1; break;
    case 6: a = 6; b = 7; ax = 0; neg = 1; ox = 0; oy = 1; oz = 1; break;
    case 7: a = 7; b = 4; ax = 1; neg = 1; ox = 0; oy = 0; oz = 1; break;
    case 8: a = 0; b = 4; ax = 2; neg = 0; ox = 0; oy = 0; oz = 0; break;
    case 9: a = 1; b = 5; ax = 2; neg = 0; ox = 1; oy = 0; oz = 0; break;
    case 10: a = 2; b = 6; ax = 2; neg = 0; ox = 1; oy = 1; oz = 0; break;
    default: a = 3; b = 7; ax = 2; neg = 0; ox = 0; oy = 1; oz = 0; break;
    }
    T va = c[0], vb = c[0];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (k == a) va = c[k];
        if (k == b) vb = c[k];
    }
    const Q mu = quotient<Q>(va, vb, p);
    const P m = (P)mu;
    // start point p1 = corner a; for a negative edge it sits at the +1 node of the moving axis
    const int ix = x + ox + (ax == 0 && neg), iy = y + oy + (ax == 1 && neg), iz = z + oz + (ax == 2 && neg);
    const int idx[3] = {ix, iy, iz};
    const double *tp[3] = {p.xp, p.yp, p.zp};
    const double *td[3] = {p.dx, p.dy, p.dz};
    const float *tpf[3] = {p.xpf, p.ypf, p.zpf};
    const float *tdf[3] = {p.dxf, p.dyf, p.dzf};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const P c1 = tab<P>(tp[k], tpf[k], idx[k]);
        if (k == ax) {
            // p2 - p1 = +-(p[i+1] - p[i]) exactly
            P d = tab<P>(td[k], tdf[k], neg ? idx[k] - 1 : idx[k]);
            if (neg) d = -d;
            r[k] = Ar<P>::add(c1, Ar<P>::mul(m, d));
        } else {
            r[k] = still<P>(c1, m);
        }
    }
}

}  // namespace mesh
